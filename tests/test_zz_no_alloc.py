"""eg_cpbt_partition_noalloc: the CPBT partitioner for callers that cannot allocate device memory
(a fixed pre-reserved budget, a host process whose allocator owns the GPU, or a pipeline that must
not take the device-wide synchronisation of cudaMalloc/cudaFree).  Its boundaries must equal the
allocating entry point's, call after call, through the C ABI.  This file sorts last on purpose."""
import ctypes

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_matches_allocating_entry_point(eg_lib):
    import torch

    import endgraph_gb300 as eg

    L = eg.load_library()
    V, E = 300_000, 2_000_000
    src, dst, _ = oracle.rmat(V, E, 41)
    outd, ind = oracle.degrees(src, dst, V)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for deg, dense in ((outd, True), (ind, False)):
        d_deg = torch.from_numpy(deg.view(np.int32)).cuda()
        for P, S, eta in ((1, 1, 1), (4, 2, 3), (64, 16, 1), (7, 3, 9)):
            want_po, want_lo = eg.cpbt_partition(deg, V, P, S, eta, 20, dense)
            ora_po, ora_lo = oracle.cpbt(deg, V, P, S, eta, 20, dense)
            assert np.array_equal(want_po, ora_po) and np.array_equal(want_lo, ora_lo)
            for _ in range(2):  # two calls in a row share the library's scratch array
                d_po = torch.full((P + 1,), -1, dtype=torch.int32, device="cuda")
                d_lo = torch.full((P * (S + 1),), -1, dtype=torch.int32, device="cuda")
                st = L.eg_cpbt_partition_noalloc(_ptr(d_deg), V, P, S, eta, 20, int(dense), _ptr(d_po), _ptr(d_lo),
                                                 stream)
                assert st == 0, L.eg_last_error()
                torch.cuda.synchronize()
                got_po = d_po.cpu().numpy().view(np.uint32)
                got_lo = d_lo.cpu().numpy().view(np.uint32).reshape(P, S + 1)
                assert np.array_equal(got_po, want_po), (P, S, eta, dense)
                assert np.array_equal(got_lo, want_lo), (P, S, eta, dense)


def test_noalloc_prefix_in_scratch_at_large_v(eg_lib):
    """Above about 84 M vertices the page-weight prefix no longer fits the search CTA's shared
    memory and lives in the scratch array instead: 2^27 random degrees (32,768 pages) against the
    oracle and the allocating entry point, dense and sparse weights, two calls in a row."""
    import torch

    import endgraph_gb300 as eg

    L = eg.load_library()
    V = 1 << 27
    rng = np.random.default_rng(43)
    deg = rng.integers(0, 48, V, dtype=np.uint32)
    deg[rng.integers(0, V, 64)] = rng.integers(1 << 16, 1 << 22, 64, dtype=np.uint32)  # a few hubs
    d_deg = torch.from_numpy(deg.view(np.int32)).cuda()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for P, S, eta, dense in ((64, 16, 1, True), (5, 3, 2, False)):
        ora_po, ora_lo = oracle.cpbt(deg, V, P, S, eta, 20, dense)
        want_po, want_lo = eg.cpbt_partition(deg, V, P, S, eta, 20, dense)
        assert np.array_equal(want_po, ora_po) and np.array_equal(want_lo, ora_lo)
        for _ in range(2):
            d_po = torch.full((P + 1,), -1, dtype=torch.int32, device="cuda")
            d_lo = torch.full((P * (S + 1),), -1, dtype=torch.int32, device="cuda")
            st = L.eg_cpbt_partition_noalloc(_ptr(d_deg), V, P, S, eta, 20, int(dense), _ptr(d_po), _ptr(d_lo),
                                             stream)
            assert st == 0, L.eg_last_error()
            torch.cuda.synchronize()
            assert np.array_equal(d_po.cpu().numpy().view(np.uint32), ora_po), (P, S, dense)
            assert np.array_equal(d_lo.cpu().numpy().view(np.uint32).reshape(P, S + 1), ora_lo), (P, S, dense)


def test_noalloc_rejects_sizes_beyond_its_scratch(eg_lib):
    import torch

    import endgraph_gb300 as eg

    L = eg.load_library()
    d_deg = torch.zeros(16, dtype=torch.int32, device="cuda")
    d_po = torch.zeros(128, dtype=torch.int32, device="cuda")
    st = L.eg_cpbt_partition_noalloc(_ptr(d_deg), (1 << 28) + 1, 2, 1, 1, 20, 1, _ptr(d_po), None, None)
    assert st == 1 and b"limits" in L.eg_last_error()
    st = L.eg_cpbt_partition_noalloc(_ptr(d_deg), 16, 65, 1, 1, 20, 1, _ptr(d_po), None, None)
    assert st == 1
