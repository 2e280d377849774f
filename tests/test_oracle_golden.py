"""The oracle's arithmetic against the reference's own artefacts and tests.

* resources/textures/area-lut.png (the output of utils/area-lut/src/main.rs)
  pins the trapezoid-area formula: the oracle's single-precision evaluation
  reproduces every texel exactly; its FP64 evaluation (the coverage target)
  is within one 8-bit step.
* simd/src/test.rs:58 and :382 pin the float->int conversion
  (_mm_cvtps_epi32, round to nearest even).
"""
import os
import zlib

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def lut():
    with open(os.path.join(HERE, "golden", "area_lut_rgba8.bin.zz"), "rb") as f:
        return np.frombuffer(zlib.decompress(f.read()), np.uint8).reshape(256, 256, 4)


def test_area_lut_single_precision_exact(lut):
    bad = []
    for v in range(256):
        for u in range(256):
            for k in range(4):
                got = oracle.area_lut_value(u, v, k)
                if got != lut[v, u, k]:
                    bad.append((u, v, k, got, int(lut[v, u, k])))
    assert not bad, f"{len(bad)} LUT texels differ, e.g. {bad[:5]}"


def test_area_fp64_within_one_step(lut):
    worst = 0
    for v in range(0, 256, 3):
        for u in range(1, 255):
            y, d = (u - 128) / 16.0, -v / 16.0
            for k in range(4):
                a = oracle.area(y - k, d) * 255.0
                e = int(np.floor(a + 0.5))
                e = min(255, max(0, e))
                worst = max(worst, abs(e - int(lut[v, u, k])))
    assert worst <= 1


def test_area_limits():
    # line far above the pixel: full coverage; far below: none
    assert oracle.area(-10.0, 0.0) == 1.0
    assert oracle.area(10.0, 0.0) == 0.0
    # horizontal line through the centre: half
    assert abs(oracle.area(0.0, 0.0) - 0.5) < 1e-15
    # symmetric in slope sign for a centred line
    for y in np.linspace(-1.2, 1.2, 13):
        for s in (0.1, 0.7, 2.0, 9.0):
            assert abs(oracle.area(y, -s) - oracle.area(y, -s)) < 1e-15


def test_cvtps_pins():
    # simd/src/test.rs:58: <-1.0, 1.3, -20.0, 3.6>.to_i32x4() == <-1, 1, -20, 4>
    assert [oracle.sse_cvt(x) for x in (-1.0, 1.3, -20.0, 3.6)] == [-1, 1, -20, 4]
    # simd/src/test.rs:382: <48.0, -4.0, 200.0, 7.0> -> <48, -4, 200, 7>
    assert [oracle.sse_cvt(x) for x in (48.0, -4.0, 200.0, 7.0)] == [48, -4, 200, 7]
    # _mm_cvtps_epi32 under the default MXCSR: ties to even
    assert [oracle.sse_cvt(x) for x in (0.5, 1.5, 2.5, -2.5, 4095.5)] == [0, 2, 2, -2, 4096]
    # out of range and NaN give the "integer indefinite" value
    assert oracle.sse_cvt(3e9) == -2 ** 31
    assert oracle.sse_cvt(float("nan")) == -2 ** 31
