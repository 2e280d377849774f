"""Regenerates tests/golden/area_lut_rgba8.bin.zz from the reference's
resources/textures/area-lut.png (the output of utils/area-lut/src/main.rs).

Usage: python tests/golden/make_area_lut.py /path/to/pathfinder
Decodes the PNG with zlib (8-bit RGBA, non-interlaced; PNG filters undone
here) and stores the raw 256x256x4 bytes zlib-compressed.
"""
import os
import struct
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def decode_png_rgba8(data: bytes) -> np.ndarray:
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    i, idat, w, h = 8, b"", 0, 0
    while i < len(data):
        n, = struct.unpack(">I", data[i:i + 4])
        t = data[i + 4:i + 8]
        body = data[i + 8:i + 8 + n]
        if t == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
            assert depth == 8 and ctype == 6 and interlace == 0
        elif t == b"IDAT":
            idat += body
        i += 12 + n
    raw = zlib.decompress(idat)
    bpp, stride = 4, w * 4
    out = np.zeros((h, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    p = 0
    for y in range(h):
        ft = raw[p]; p += 1
        line = np.frombuffer(raw[p:p + stride], np.uint8).astype(np.int32); p += stride
        cur = np.zeros(stride, np.int32)
        for x in range(stride):
            a = cur[x - bpp] if x >= bpp else 0
            b = prev[x]
            c = prev[x - bpp] if x >= bpp else 0
            if ft == 0: v = line[x]
            elif ft == 1: v = line[x] + a
            elif ft == 2: v = line[x] + b
            elif ft == 3: v = line[x] + ((a + b) >> 1)
            elif ft == 4:
                pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                pr = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                v = line[x] + pr
            else:
                raise ValueError(f"bad filter {ft}")
            cur[x] = v & 0xff
        out[y] = cur
        prev = cur
    return out.reshape(h, w, 4)


def main():
    # the reference checkout: first argument, else $PATHFINDER_REFERENCE
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PATHFINDER_REFERENCE", "")
    if not ref:
        sys.exit("usage: make_area_lut.py <pathfinder checkout> (or set PATHFINDER_REFERENCE)")
    png = open(os.path.join(ref, "resources/textures/area-lut.png"), "rb").read()
    img = decode_png_rgba8(png)
    with open(os.path.join(HERE, "area_lut_rgba8.bin.zz"), "wb") as f:
        f.write(zlib.compress(img.tobytes(), 9))
    print(img.shape, img.dtype)


if __name__ == "__main__":
    main()
