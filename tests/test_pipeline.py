"""PFCUDAPipeline without a GPU: arguments are checked before any device work,
and creating a pipeline on a machine without a device reports it."""
import ctypes as C

import pytest

from pathfinder_gb300 import _abi


def test_pipeline_arguments_rejected_without_a_device(built):
    L = _abi.lib()
    h = C.c_void_p()
    assert L.PFCUDAPipelineCreate(0, 0, None, C.byref(h)) == _abi.PF_CUDA_ERR_INVALID
    assert L.PFCUDAPipelineCreate(0, 65, None, C.byref(h)) == _abi.PF_CUDA_ERR_INVALID
    assert L.PFCUDAPipelineCreate(0, 2, None, None) == _abi.PF_CUDA_ERR_INVALID
    t = C.c_uint64()
    assert L.PFCUDAPipelineSubmit(None, None, None, 16, 16, None, 0, C.byref(t)) == _abi.PF_CUDA_ERR_INVALID
    done = C.c_int32()
    assert L.PFCUDAPipelinePoll(None, 1, C.byref(done)) == _abi.PF_CUDA_ERR_INVALID
    assert L.PFCUDAPipelineWait(None, 1) == _abi.PF_CUDA_ERR_INVALID
    assert L.PFCUDAPipelineDestroy(None) == _abi.PF_CUDA_ERR_INVALID


def test_pipeline_without_a_device_raises(built):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import pathfinder_gb300 as pf
    with pytest.raises(_abi.PFCUDAError) as e:
        pf.RenderPipeline(0, depth=2)
    assert e.value.code == _abi.PF_CUDA_ERR_NO_DEVICE
