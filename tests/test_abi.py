"""The C ABI: the library loads without a GPU, exports every entry point that
include/*.h declares, and its structs have the same layout in C and ctypes."""
import ctypes as C
import os
import re
import subprocess

import pytest

from pathfinder_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")


def declared_functions(headers=None):
    names = []
    for h in sorted(os.listdir(INCLUDE)):
        if h.endswith(".h") and (headers is None or h in headers):
            src = open(os.path.join(INCLUDE, h)).read()
            names += re.findall(r"^\s*(?:int32_t|const char\s*\*|void|uint8_t)\s+(PF\w+)\s*\(", src, re.M)
    return names


def test_headers_declare_entry_points():
    names = declared_functions()
    assert "PFCUDARendererCreate" in names and "PFCUDARenderScene" in names and len(names) >= 19


def test_library_exports_every_declared_symbol(built):
    lib = C.CDLL(_abi.LIB_PATH)
    missing = [n for n in declared_functions(["pathfinder_cuda.h"]) if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"
    scenes = C.CDLL(_abi.SCENES_LIB_PATH)
    missing = [n for n in declared_functions(["pathfinder_cuda_scenes.h"]) if not hasattr(scenes, n)]
    assert not missing, f"scene generator library does not export: {missing}"
    # the renderer does not carry the generators
    assert not hasattr(lib, "PFCUDASceneGenerate")


STRUCTS = ["PFVector2F", "PFRectF", "PFRectI", "PFColorU", "PFColorF", "PFTransform2F", "PFCUDAPath",
           "PFCUDASceneDesc", "PFCUDABuildOptions", "PFCUDARendererOptions", "PFCUDARenderStats", "PFCUDAFill",
           "PFCUDATile", "PFCUDAClip", "PFCUDASceneParams", "PFCUDAColorStop", "PFCUDAGradient", "PFCUDAPattern", "PFCUDAStrokeStyle",
           "PFCUDAStrokeInput", "PFCUDAStrokeOutput", "PFCUDADashInput", "PFCUDAOutlineOutput"]


def test_struct_layouts_match_ctypes(tmp_path):
    src = tmp_path / "sizes.c"
    body = "\n".join(f'printf("{s} %zu\\n", sizeof({s}));' for s in STRUCTS)
    src.write_text('#include <stdio.h>\n#include "pathfinder_cuda.h"\n#include "pathfinder_cuda_scenes.h"\n'
                   f"int main(void) {{ {body} return 0; }}\n")
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-I", INCLUDE, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    sizes = dict(line.split() for line in out if line)
    for s in STRUCTS:
        assert int(sizes[s]) == C.sizeof(getattr(_abi, s)), s
    fill, tile, clip, path, rect = _abi.record_dtypes()
    assert fill.itemsize == int(sizes["PFCUDAFill"])
    assert tile.itemsize == int(sizes["PFCUDATile"])
    assert clip.itemsize == int(sizes["PFCUDAClip"])
    assert path.itemsize == int(sizes["PFCUDAPath"])


def test_status_strings(built):
    L = _abi.lib()
    assert L.PFCUDAStatusString(_abi.PF_CUDA_OK) == b"ok"
    assert b"capacity" in L.PFCUDAStatusString(_abi.PF_CUDA_ERR_CAPACITY)


def test_invalid_arguments_are_rejected_without_a_device(built):
    L = _abi.lib()
    assert L.PFCUDARendererCreate(0, None, None) == _abi.PF_CUDA_ERR_INVALID
    p = _abi.PFCUDASceneParams(99, 1, 1.0, 0.0, 0, 0, 0)
    h = C.c_void_p()
    assert _abi.scenes_lib().PFCUDASceneGenerate(C.byref(p), C.byref(h)) == _abi.PF_CUDA_ERR_INVALID
    assert L.PFCUDARenderScene(None, None, 16, 16, None, 0) == _abi.PF_CUDA_ERR_INVALID


def test_no_device_is_reported(built):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    L = _abi.lib()
    h = C.c_void_p()
    assert L.PFCUDARendererCreate(0, None, C.byref(h)) == _abi.PF_CUDA_ERR_NO_DEVICE
    assert not h.value
