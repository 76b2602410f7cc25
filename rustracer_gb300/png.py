"""Minimal PNG reader and writer (zlib only): the headless replacement of the
reference's swapchain present (crates/libs/app/src/lib.rs:585-590) writes
frames with write_png, and the glTF loader decodes embedded PNG textures
with read_png.

read_png handles 8-bit images of colour types 0 (grey), 2 (RGB), 3
(palette, with tRNS alpha), 4 (grey + alpha) and 6 (RGBA), non-interlaced,
with the five scanline filters; it returns an (H, W, 4) uint8 array.
"""
import struct
import zlib

import numpy as np


def write_png(path, rgba):
    """Writes an (H, W, 4) or (H, W, 3) uint8 image (filter 0 on every row)."""
    img = np.ascontiguousarray(rgba, np.uint8)
    h, w, c = img.shape
    ctype = {3: 2, 4: 6}[c]
    raw = b"".join(b"\x00" + img[y].tobytes() for y in range(h))

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n")
        f.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0)))
        f.write(chunk(b"IDAT", zlib.compress(raw, 6)))
        f.write(chunk(b"IEND", b""))


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def read_png(data):
    """Decodes PNG bytes to an (H, W, 4) uint8 array."""
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG")
    pos, idat, plte, trns = 8, [], None, None
    w = h = depth = ctype = interlace = None
    while pos < len(data):
        n, tag = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        pos += 12 + n
        if tag == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
        elif tag == b"IDAT":
            idat.append(body)
        elif tag == b"PLTE":
            plte = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif tag == b"tRNS":
            trns = np.frombuffer(body, np.uint8)
        elif tag == b"IEND":
            break
    if depth != 8 or interlace != 0:
        raise ValueError(f"unsupported PNG (bit depth {depth}, interlace {interlace})")
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    raw = zlib.decompress(b"".join(idat))
    stride = w * ch
    out = np.zeros((h, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    for y in range(h):
        f = raw[y * (stride + 1)]
        line = np.frombuffer(raw, np.uint8, stride, y * (stride + 1) + 1).astype(np.int32)
        if f == 0:
            cur = line
        elif f == 2:
            cur = (line + prev) & 0xFF
        elif f in (1, 3, 4):
            cur = np.zeros(stride, np.int32)
            for x in range(stride):
                a = cur[x - ch] if x >= ch else 0
                if f == 1:
                    cur[x] = (line[x] + a) & 0xFF
                elif f == 3:
                    cur[x] = (line[x] + ((a + prev[x]) >> 1)) & 0xFF
                else:
                    c = prev[x - ch] if x >= ch else 0
                    cur[x] = (line[x] + _paeth(a, prev[x], c)) & 0xFF
        else:
            raise ValueError(f"bad PNG filter {f}")
        out[y] = cur
        prev = cur
    px = out.reshape(h, w, ch)
    rgba = np.full((h, w, 4), 255, np.uint8)
    if ctype == 0:
        rgba[..., :3] = px
    elif ctype == 2:
        rgba[..., :3] = px
    elif ctype == 3:
        rgba[..., :3] = plte[px[..., 0]]
        if trns is not None:
            alpha = np.full(len(plte), 255, np.uint8)
            alpha[:len(trns)] = trns
            rgba[..., 3] = alpha[px[..., 0]]
    elif ctype == 4:
        rgba[..., :3] = px[..., :1]
        rgba[..., 3] = px[..., 1]
    else:
        rgba[:] = px
    return rgba
