#!/bin/sh
# Builds the reference's own engine (core/*.hpp of leodestiny/EndGraph) as a one-rank shared
# library for tests and the timed CPU baseline: oracle/_ref/libeg_ref.so.
#
# The reference headers are compiled as shipped.  Its compile errors and undefined values are
# fixed from the command line only:
#   -Ddense='(!sparse)'        undeclared `dense` (core/graph.hpp:733)
#   -Dout_degree=degree        undeclared `out_degree` (core/graph.hpp:1487)
#   -Dedges=edges_num          undeclared `edges` (core/graph.hpp:1491)
#   -Dhas_iterations=...       adds the members use_iteration / use_root that the toolkits set
#                              (toolkits/pagerank.cpp:148, bfs.cpp:127) and graph.hpp:1493 reads
#   mpi.h / numa.h             single-rank, single-node stand-ins (this folder)
#   -ffp-contract=off          IEEE double arithmetic identical on x86_64 and aarch64
# `sparse` and `max_iterations` are given defined values by ref_driver.cpp before assign_vertices.
#
# Sources: $EG_REFERENCE_DIR, else the checkout at /root/reference, when present (this recipe is
# the one place that names that location; oracle/_ref/REFERENCE_DIR records the directory it
# used, and the tests that read reference files find it there).  A copy of the reference headers
# is staged into oracle/_ref/src (git-ignored, never committed) so that the same build can be
# repeated on a machine without the reference checkout.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
REF="${EG_REFERENCE_DIR:-/root/reference}"
mkdir -p "$OUT/src/core"
if [ -f "$REF/core/graph.hpp" ]; then
    cp "$REF"/core/*.hpp "$OUT/src/core/"
    INC="$REF"
    (cd "$REF" && pwd) > "$OUT/REFERENCE_DIR"
elif [ -f "$OUT/src/core/graph.hpp" ]; then
    INC="$OUT/src"
else
    echo "build_ref.sh: reference sources not found" >&2
    exit 3
fi
${CXX:-g++} -O3 -std=c++14 -fopenmp -fno-strict-aliasing -ffp-contract=off -fPIC -shared -w \
    -I"$HERE/ref" -I"$INC" -I"$HERE/../include" \
    -D'dense=(!sparse)' -Dout_degree=degree -Dedges=edges_num \
    -D'has_iterations=has_iterations; bool use_iteration = false; bool use_root = false' \
    "$HERE/ref/ref_driver.cpp" -o "$OUT/libeg_ref.so.tmp"
mv "$OUT/libeg_ref.so.tmp" "$OUT/libeg_ref.so"
echo "$OUT/libeg_ref.so"
