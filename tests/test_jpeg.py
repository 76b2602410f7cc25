"""Baseline JPEG decoder (rustracer_gb300/jpeg.py), CPU.

* Round trips through a minimal baseline encoder written here (forward DCT,
  quantisation, canonical Huffman codes of fixed length, byte stuffing,
  restart markers): 4:4:4 and 4:2:0, grey and colour; the decoded image is
  within JPEG's quantisation error of the original.
* The reference's own Yokohama cube-map faces (when the reference checkout is
  on the machine) decode to six 2048^2 photographs.
"""
import os
import struct

import numpy as np
import pytest

from rustracer_gb300 import jpeg
from rustracer_gb300.jpeg import ZIGZAG, _C, read_jpeg

QY = np.array([16, 11, 10, 16, 24, 40, 51, 61, 12, 12, 14, 19, 26, 58, 60, 55, 14, 13, 16, 24, 40, 57, 69, 56, 14, 17,
               22, 29, 51, 87, 80, 62, 18, 22, 37, 56, 68, 109, 103, 77, 24, 35, 55, 64, 81, 104, 113, 92, 49, 64,
               78, 87, 103, 121, 120, 101, 72, 92, 95, 98, 112, 100, 103, 99])  # natural order


class _BitWriter:
    def __init__(self):
        self.out, self.acc, self.n = bytearray(), 0, 0

    def put(self, code, length):
        self.acc = (self.acc << length) | code
        self.n += length
        while self.n >= 8:
            b = (self.acc >> (self.n - 8)) & 0xFF
            self.out.append(b)
            if b == 0xFF:
                self.out.append(0)  # stuffing
            self.n -= 8

    def flush(self):
        if self.n:
            self.put((1 << (8 - self.n)) - 1, 8 - self.n)  # pad with ones
        self.acc = 0


def _category(v):
    return 0 if v == 0 else int(abs(v)).bit_length()


def _fixed_table(symbols, length):
    """Canonical table giving each symbol a code of `length` bits."""
    counts = [0] * 16
    counts[length - 1] = len(symbols)
    codes = {s: k for k, s in enumerate(symbols)}
    return counts, list(symbols), codes


def encode(rgb, sub420, quality=90, restart=0):
    h, w = rgb.shape[:2]
    grey = rgb.ndim == 2
    x = rgb.astype(np.float64)
    if grey:
        planes = [x]
    else:
        r, g, b = x[..., 0], x[..., 1], x[..., 2]
        planes = [0.299 * r + 0.587 * g + 0.114 * b, -0.168736 * r - 0.331264 * g + 0.5 * b + 128,
                  0.5 * r - 0.418688 * g - 0.081312 * b + 128]
    s = 200 - 2 * quality
    q = np.clip((QY * s + 50) // 100, 1, 255)
    hs = [2, 1, 1] if (sub420 and not grey) else [1, 1, 1]
    hs = hs[:len(planes)]
    hmax = max(hs)
    mcux, mcuy = -(-w // (8 * hmax)), -(-h // (8 * hmax))
    comps = []
    for ci, p in enumerate(planes):
        f = hmax // hs[ci]
        H, W = mcuy * 8 * hs[ci], mcux * 8 * hs[ci]
        pp = np.pad(p, ((0, H * f - h), (0, W * f - w)), mode="edge")
        if f > 1:
            pp = pp.reshape(H, f, W, f).mean((1, 3))
        blocks = pp.reshape(H // 8, 8, W // 8, 8).transpose(0, 2, 1, 3) - 128.0
        coef = np.einsum("ux,nmxy,vy->nmuv", _C, blocks, _C)
        qz = np.round(coef.reshape(H // 8, W // 8, 64) / q).astype(np.int64)
        zz = np.zeros_like(qz)
        zz[..., :] = qz[..., ZIGZAG]
        comps.append(zz)
    # symbols: DC categories 0..11, AC run/size pairs
    dc_syms = list(range(12))
    ac_syms = [0x00, 0xF0] + [(r << 4) | sz for r in range(16) for sz in range(1, 11)]
    dcc, dcv, dcmap = _fixed_table(dc_syms, 4)
    acc, acv, acmap = _fixed_table(ac_syms, 8)
    bw = _BitWriter()
    pred = [0] * len(comps)
    nmcu = mcux * mcuy
    for mcu in range(nmcu):
        if restart and mcu and mcu % restart == 0:
            bw.flush()
            bw.out += bytes([0xFF, 0xD0 + ((mcu // restart - 1) & 7)])
            pred = [0] * len(comps)
        my, mx = divmod(mcu, mcux)
        for ci, zz in enumerate(comps):
            for by in range(hs[ci]):
                for bx in range(hs[ci]):
                    blk = zz[my * hs[ci] + by, mx * hs[ci] + bx]
                    d = int(blk[0]) - pred[ci]
                    pred[ci] = int(blk[0])
                    t = _category(d)
                    bw.put(dcmap[t], 4)
                    if t:
                        bw.put(d if d > 0 else d + (1 << t) - 1, t)
                    run = 0
                    last = max([k for k in range(1, 64) if blk[k] != 0], default=0)
                    for k in range(1, last + 1):
                        v = int(blk[k])
                        if v == 0:
                            run += 1
                            continue
                        while run > 15:
                            bw.put(acmap[0xF0], 8)
                            run -= 16
                        t = _category(v)
                        bw.put(acmap[(run << 4) | t], 8)
                        bw.put(v if v > 0 else v + (1 << t) - 1, t)
                        run = 0
                    if last < 63:
                        bw.put(acmap[0x00], 8)
    bw.flush()
    seg = lambda m, body: bytes([0xFF, m]) + struct.pack(">H", len(body) + 2) + body
    out = b"\xff\xd8"
    out += seg(0xDB, bytes([0]) + bytes(int(v) for v in q[ZIGZAG]))
    nc = len(comps)
    sof = struct.pack(">BHHB", 8, h, w, nc) + b"".join(bytes([ci + 1, (hs[ci] << 4) | hs[ci], 0]) for ci in range(nc))
    out += seg(0xC0, sof)
    out += seg(0xC4, bytes([0x00]) + bytes(dcc) + bytes(dcv))
    out += seg(0xC4, bytes([0x10]) + bytes(acc) + bytes(acv))
    if restart:
        out += seg(0xDD, struct.pack(">H", restart))
    sos = bytes([nc]) + b"".join(bytes([ci + 1, 0x00]) for ci in range(nc)) + bytes([0, 63, 0])
    out += seg(0xDA, sos) + bytes(bw.out) + b"\xff\xd9"
    return out


def _image(h, w, seed):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w]
    img = np.stack([128 + 100 * np.sin(x / 9.0), 128 + 100 * np.cos(y / 13.0), (x + y) * 255.0 / (h + w)], -1)
    img[h // 3:h // 2, w // 4:w // 2] = (230, 40, 40)  # a hard-edged block
    img += rng.normal(0, 2, img.shape)
    return np.clip(img, 0, 255).astype(np.uint8)


def _psnr(a, b):
    mse = np.mean((a.astype(np.float64) - b.astype(np.float64)) ** 2)
    return 10 * np.log10(255.0 ** 2 / max(mse, 1e-12))


@pytest.mark.parametrize("sub420,restart", [(False, 0), (True, 0), (True, 5)])
def test_colour_round_trip(sub420, restart):
    img = _image(61, 77, 1)  # not a multiple of the MCU size
    dec = read_jpeg(encode(img, sub420, restart=restart))
    assert dec.shape == (61, 77, 4) and np.all(dec[..., 3] == 255)
    assert _psnr(dec[..., :3], img) > (30.0 if sub420 else 34.0)


def test_grey_round_trip():
    img = _image(40, 48, 2)[..., 0]
    dec = read_jpeg(encode(img, False))
    assert np.all(dec[..., 0] == dec[..., 1]) and np.all(dec[..., 1] == dec[..., 2])
    assert _psnr(dec[..., 0], img) > 34.0


def test_rejects_progressive():
    data = bytearray(encode(_image(16, 16, 3), False))
    i = data.index(b"\xff\xc0")
    data[i + 1] = 0xC2  # declare the frame progressive
    with pytest.raises(ValueError):
        read_jpeg(bytes(data))


def test_reference_skybox_faces():
    d = "/root/reference/assets/skyboxs/Yokohama"
    if not os.path.isdir(d):
        pytest.skip("the reference checkout is not on this machine")
    from rustracer_gb300.gltf import load_cubemap
    size, faces = load_cubemap(d)
    assert size == 2048 and faces.size == 6 * 2048 * 2048 * 4
    f = faces.reshape(6, 2048, 2048, 4)[..., :3].astype(np.int64)
    # photographs: smooth almost everywhere (a bad Huffman or zigzag decode gives noise)
    assert np.abs(np.diff(f, axis=2)).mean() < 6.0
    assert 5.0 < f.mean() < 200.0
