"""The allocation-free exclusive scan (PFCUDAExclusiveScanNoAlloc).

Callers that cannot call cudaMalloc while they work use this entry point: a
frame loop that must not stall on cudaMalloc's device synchronisation, a host
whose device memory belongs to its own pool allocator, or code running while
another module captures a CUDA graph.  It keeps its scratch in a fixed device
array (up to 16,777,216 values per call) instead of allocating.

The test calls it through the C ABI, twice in a row on the same inputs (the
fixed scratch keeps the previous call's contents), and checks the output
against the allocating entry point PFCUDAExclusiveScan: bit-exact, as for all
integer work here.  It builds its own renderer, so it passes alone in a fresh
process as well as after the other tests; pytest collects this file last.
"""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu

MAX_COUNT = 1 << 24


def _scan_pair(torch, L, handle, x, n):
    ref = torch.full((n + 1,), -1, dtype=torch.int32, device="cuda")
    got = torch.full((n + 1,), -7, dtype=torch.int32, device="cuda")
    assert L.PFCUDAExclusiveScan(handle, C.c_void_p(x.data_ptr()), C.c_void_p(ref.data_ptr()), n) == 0
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.PFCUDAExclusiveScanNoAlloc(C.c_void_p(x.data_ptr()), C.c_void_p(got.data_ptr()), n, C.c_void_p(stream))
    assert rc == 0
    torch.cuda.synchronize()
    return ref, got


def test_no_alloc_scan_matches_the_allocating_scan():
    torch = pytest.importorskip("torch")
    import __graft_entry__
    __graft_entry__.build()
    import pathfinder_gb300 as pf
    from pathfinder_gb300 import _abi
    L = _abi.lib()
    with pf.Renderer(0) as r:
        g = torch.Generator().manual_seed(11)
        for n in (1, 2049, 1_000_003, MAX_COUNT):
            x = torch.randint(0, 1 << 20, (n,), generator=g, dtype=torch.int32).cuda()
            for _ in range(2):  # two calls in a row share the fixed scratch
                ref, got = _scan_pair(torch, L, r.handle, x, n)
                assert torch.equal(ref, got), f"n={n}"
        # sizes beyond the fixed scratch are rejected before any launch
        x = torch.zeros((8,), dtype=torch.int32, device="cuda")
        out = torch.zeros((8,), dtype=torch.int32, device="cuda")
        rc = L.PFCUDAExclusiveScanNoAlloc(C.c_void_p(x.data_ptr()), C.c_void_p(out.data_ptr()), MAX_COUNT + 1,
                                          None)
        assert rc == _abi.PF_CUDA_ERR_CAPACITY
