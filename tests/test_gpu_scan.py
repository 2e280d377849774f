"""The device-wide exclusive scan behind fill offsets and alpha-tile ids,
through the C ABI, against numpy (exact: integer work)."""
import ctypes as C

import numpy as np
import pytest

from pathfinder_gb300 import _abi

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [0, 1, 5, 2047, 2048, 2049, 100_000, 3_000_001])
def test_exclusive_scan_matches_numpy(renderer, n):
    torch = pytest.importorskip("torch")
    g = torch.Generator().manual_seed(n)
    x = torch.randint(0, 5000, (max(n, 1),), generator=g, dtype=torch.int32)[:n].cuda()
    out = torch.full((n + 1,), -1, dtype=torch.int32, device="cuda")
    rc = _abi.lib().PFCUDAExclusiveScan(renderer.handle, C.c_void_p(x.data_ptr()), C.c_void_p(out.data_ptr()), n)
    assert rc == _abi.PF_CUDA_OK
    xs = x.cpu().numpy().astype(np.uint64)
    expect = np.concatenate([[0], np.cumsum(xs)]).astype(np.uint64) & 0xFFFFFFFF
    got = out.cpu().numpy().view(np.uint32).astype(np.uint64)
    assert np.array_equal(got, expect)


def test_exclusive_scan_rejects_bad_arguments(renderer):
    L = _abi.lib()
    assert L.PFCUDAExclusiveScan(renderer.handle, None, None, 4) == _abi.PF_CUDA_ERR_INVALID
    torch = pytest.importorskip("torch")
    out = torch.zeros((1,), dtype=torch.int32, device="cuda")
    assert L.PFCUDAExclusiveScan(renderer.handle, None, C.c_void_p(out.data_ptr()), 5) == _abi.PF_CUDA_ERR_INVALID
