"""CPU tests of the C-ABI library: it builds for sm_103a, loads, exports every entry point that
include/*.h declares, and rejects bad arguments before touching a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for path in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not path.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", path)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[\w\s\*]+?\b(eg_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    # static inline helpers of the generator header are not library symbols
    return {n for n in names if not n.startswith(("eg_rmat_", "eg_mix64", "eg_perm"))}


@pytest.fixture(scope="module")
def lib():
    from endgraph_gb300 import build
    build.build()
    import endgraph_gb300 as eg
    return eg.load_library()


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header(lib):
    import endgraph_gb300 as eg
    assert declared_functions() <= set(eg.SIGNATURES)


def test_python_constants_match_the_header():
    """Every EG_OPT_*, EG_ERR_* and location constant the header defines has the same value in the
    Python binding (a renumbered option would otherwise set another one silently)."""
    import endgraph_gb300 as eg
    text = open(os.path.join(ROOT, "include", "endgraph_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    consts = {m.group(1): int(m.group(2)) for m in re.finditer(r"\b(EG_(?:OPT|ERR)_\w+|EG_OK|EG_HOST|EG_DEVICE)\s*=\s*(-?\d+)", text)}
    assert "EG_OPT_BUILD_LAUNCH" in consts and len(consts) >= 15
    status = {k: v for k, v in consts.items() if k == "EG_OK" or k.startswith("EG_ERR_")}
    assert {v: k for k, v in status.items()} == eg.STATUS  # status names by value
    names = {k: v for k, v in consts.items() if k not in status}
    missing = [k for k in names if not hasattr(eg, k)]
    assert not missing, missing
    wrong = {k: (v, getattr(eg, k)) for k, v in names.items() if getattr(eg, k) != v}
    assert not wrong, wrong


def test_argument_errors_without_gpu(lib):
    import endgraph_gb300 as eg
    out = np.zeros(4, np.uint32)
    # k out of range is rejected before any device work
    st = lib.eg_optimal_offset(None, 0, 0, out.ctypes.data_as(ctypes.c_void_p))
    assert st == 1 and b"k" in lib.eg_last_error()
    st = lib.eg_generate_rmat(None, 8, 10, 16, 0.57, 0.19, 0.19, 1, 1, 0.0, 1.0, None)
    assert st == 1
    st = lib.eg_generate_rmat(ctypes.c_void_p(16), 7, 10, 16, 0.57, 0.19, 0.19, 1, 1, 0.0, 1.0, None)
    assert st == 1
    assert lib.eg_destroy(None) == 0
    with pytest.raises(eg.EndGraphError):
        eg.optimal_offset([1, 2, 3], 0)


def test_pack_edges_layout():
    import endgraph_gb300 as eg
    rec = eg.pack_edges(np.array([1, 2], np.uint32), np.array([3, 4], np.uint32), np.array([0.5, 1.5], np.float32))
    assert rec.dtype == np.uint32 and rec.shape == (2, 3)
    raw = rec.tobytes()
    assert np.frombuffer(raw[:8], np.uint32).tolist() == [1, 3]
    assert np.frombuffer(raw[8:12], np.float32)[0] == 0.5  # packed {u32 src, u32 dst, f32 w}


def test_nvcc_builds_for_sm103a():
    from endgraph_gb300 import build
    assert "arch=compute_103a,code=sm_103a" in " ".join(build.ARCH)
    assert os.path.exists(build.build())
