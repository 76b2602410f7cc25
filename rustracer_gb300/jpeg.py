"""Baseline JPEG decoder (numpy), for the glTF loader's JPEG textures and the
reference's JPEG cube-map faces (assets/skyboxs/*/pos[xyz].jpg, loaded by
crates/libs/asset_loader/src/globals.rs:175-199 through the `image` crate).

A restatement of ITU-T T.81 (JPEG) sequential DCT decoding with Huffman
coding: 8-bit samples, 1 or 3 components with any sampling factors, restart
intervals.  Progressive and arithmetic-coded files are rejected.  Chroma is
upsampled by replication and YCbCr is converted with the JFIF matrix, so
results can differ from libjpeg-based decoders by a few levels near chroma
edges.  read_jpeg returns an (H, W, 4) uint8 array (alpha 255).
"""
import struct

import numpy as np

ZIGZAG = np.array([
    0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5, 12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6, 7, 14, 21,
    28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51, 58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61,
    54, 47, 55, 62, 63], np.int64)  # zigzag position k -> natural (row-major) index


def _idct_matrix():
    c = np.zeros((8, 8))
    for u in range(8):
        a = np.sqrt(1 / 8) if u == 0 else np.sqrt(2 / 8)
        for x in range(8):
            c[u, x] = a * np.cos((2 * x + 1) * u * np.pi / 16)
    return c  # rows: frequency u; f(x) = sum_u c[u, x] F(u)


_C = _idct_matrix()


class _Huffman:
    """Canonical Huffman table (T.81 Annex C) as a 16-bit peek table."""

    def __init__(self, counts, symbols):
        self.sym = np.zeros(1 << 16, np.int32)
        self.len = np.zeros(1 << 16, np.int32)
        code, k = 0, 0
        for length in range(1, 17):
            for _ in range(counts[length - 1]):
                lo = code << (16 - length)
                hi = (code + 1) << (16 - length)
                self.sym[lo:hi] = symbols[k]
                self.len[lo:hi] = length
                code += 1
                k += 1
            code <<= 1
        self.sym = self.sym.tolist()
        self.len = self.len.tolist()


class _Bits:
    """Bit reader over one entropy-coded interval (stuffed zero bytes removed)."""

    def __init__(self, data):
        self.data = data + b"\x00\x00\x00\x00"
        self.pos = 0  # bit position

    def peek16(self):
        b = self.pos >> 3
        v = (self.data[b] << 16) | (self.data[b + 1] << 8) | self.data[b + 2]
        return (v >> (8 - (self.pos & 7))) & 0xFFFF

    def bits(self, n):
        if n == 0:
            return 0
        b = self.pos >> 3
        v = (self.data[b] << 24) | (self.data[b + 1] << 16) | (self.data[b + 2] << 8) | self.data[b + 3]
        r = (v >> (32 - (self.pos & 7) - n)) & ((1 << n) - 1)
        self.pos += n
        return r

    def decode(self, h):
        p = self.peek16()
        n = h.len[p]
        if n == 0:
            raise ValueError("bad Huffman code")
        self.pos += n
        return h.sym[p]


def _extend(v, t):  # T.81 F.2.2.1: the sign of a magnitude category
    return v - (1 << t) + 1 if t and v < (1 << (t - 1)) else v


def _split_scan(data, start):
    """Entropy-coded data from `start` to the next non-RST marker, split at
    restart markers, with 0xFF00 stuffing removed.  Returns (intervals, end)."""
    out, cur = [], bytearray()
    i, n = start, len(data)
    while i < n:
        b = data[i]
        if b != 0xFF:
            cur.append(b)
            i += 1
            continue
        m = data[i + 1]
        if m == 0x00:
            cur.append(0xFF)
            i += 2
        elif 0xD0 <= m <= 0xD7:
            out.append(bytes(cur))
            cur = bytearray()
            i += 2
        elif m == 0xFF:
            i += 1
        else:
            break
    out.append(bytes(cur))
    return out, i


def read_jpeg(data):
    """Decodes baseline JPEG bytes to an (H, W, 4) uint8 array."""
    if data[:2] != b"\xff\xd8":
        raise ValueError("not a JPEG")
    qt, hts = {}, {}
    frame, restart = None, 0
    i = 2
    while i < len(data):
        if data[i] != 0xFF:
            raise ValueError("marker expected")
        m = data[i + 1]
        if m == 0xD8 or m == 0x01 or 0xD0 <= m <= 0xD7:
            i += 2
            continue
        if m == 0xD9:
            break
        length = struct.unpack(">H", data[i + 2:i + 4])[0]
        seg = data[i + 4:i + 2 + length]
        if m == 0xDB:  # quantisation tables
            k = 0
            while k < len(seg):
                pq, tq = seg[k] >> 4, seg[k] & 15
                if pq:
                    q = np.frombuffer(seg[k + 1:k + 129], ">u2").astype(np.int32)
                    k += 129
                else:
                    q = np.frombuffer(seg[k + 1:k + 65], np.uint8).astype(np.int32)
                    k += 65
                qt[tq] = q  # in zigzag order
        elif m == 0xC4:  # Huffman tables
            k = 0
            while k < len(seg):
                tc, th = seg[k] >> 4, seg[k] & 15
                counts = list(seg[k + 1:k + 17])
                nsym = sum(counts)
                hts[(tc, th)] = _Huffman(counts, list(seg[k + 17:k + 17 + nsym]))
                k += 17 + nsym
        elif m in (0xC0, 0xC1):  # baseline / extended sequential, Huffman
            p, h, w, nc = struct.unpack(">BHHB", seg[:6])
            if p != 8:
                raise ValueError(f"{p}-bit JPEG samples are not supported")
            comps = [dict(id=seg[6 + 3 * k], hs=seg[7 + 3 * k] >> 4, vs=seg[7 + 3 * k] & 15, tq=seg[8 + 3 * k])
                     for k in range(nc)]
            frame = dict(h=h, w=w, comps=comps)
        elif m in (0xC2, 0xC3, 0xC5, 0xC6, 0xC7, 0xC9, 0xCA, 0xCB, 0xCD, 0xCE, 0xCF):
            raise ValueError("only baseline (sequential Huffman) JPEG is supported")
        elif m == 0xDD:
            restart = struct.unpack(">H", seg[:2])[0]
        elif m == 0xDA:
            if frame is None:
                raise ValueError("scan before frame header")
            ns = seg[0]
            sel = {seg[1 + 2 * k]: (seg[2 + 2 * k] >> 4, seg[2 + 2 * k] & 15) for k in range(ns)}
            if ns != len(frame["comps"]):
                raise ValueError("only single interleaved scans are supported")
            intervals, end = _split_scan(data, i + 2 + length)
            coefs = _decode_scan(frame, sel, hts, restart, intervals)
            return _reconstruct(frame, qt, coefs)
        i += 2 + length
    raise ValueError("no scan in JPEG")


def _decode_scan(frame, sel, hts, restart, intervals):
    comps = frame["comps"]
    hmax = max(c["hs"] for c in comps)
    vmax = max(c["vs"] for c in comps)
    mcux = -(-frame["w"] // (8 * hmax))
    mcuy = -(-frame["h"] // (8 * vmax))
    nmcu = mcux * mcuy
    coefs = []
    for c in comps:
        coefs.append(np.zeros((mcuy * c["vs"], mcux * c["hs"], 64), np.int32))
    plan = []  # per MCU: (component index, block row offset, block column offset)
    for ci, c in enumerate(comps):
        for by in range(c["vs"]):
            for bx in range(c["hs"]):
                plan.append((ci, by, bx))
    dc_tabs = [hts[(0, sel[c["id"]][0])] for c in comps]
    ac_tabs = [hts[(1, sel[c["id"]][1])] for c in comps]
    per = restart if restart else nmcu
    for iv, seg in enumerate(intervals):
        first = iv * per
        if first >= nmcu:
            break
        bits = _Bits(seg)
        pred = [0] * len(comps)
        for mcu in range(first, min(first + per, nmcu)):
            my, mx = divmod(mcu, mcux)
            for ci, by, bx in plan:
                c = comps[ci]
                blk = coefs[ci][my * c["vs"] + by, mx * c["hs"] + bx]
                t = bits.decode(dc_tabs[ci])
                pred[ci] += _extend(bits.bits(t), t)
                blk[0] = pred[ci]
                k = 1
                act = ac_tabs[ci]
                while k < 64:
                    rs = bits.decode(act)
                    r, s = rs >> 4, rs & 15
                    if s == 0:
                        if r != 15:
                            break  # end of block
                        k += 16
                        continue
                    k += r
                    blk[k] = _extend(bits.bits(s), s)
                    k += 1
    return coefs


def _reconstruct(frame, qt, coefs):
    comps = frame["comps"]
    hmax = max(c["hs"] for c in comps)
    vmax = max(c["vs"] for c in comps)
    H, W = frame["h"], frame["w"]
    planes = []
    for c, co in zip(comps, coefs):
        by, bx = co.shape[:2]
        zz = co.reshape(-1, 64) * qt[c["tq"]][None, :]
        nat = np.zeros_like(zz, dtype=np.float64)
        nat[:, ZIGZAG] = zz
        blocks = nat.reshape(-1, 8, 8)
        pix = np.einsum("ux,nuv,vy->nxy", _C, blocks, _C) + 128.0
        img = pix.reshape(by, bx, 8, 8).transpose(0, 2, 1, 3).reshape(by * 8, bx * 8)
        fy, fx = vmax // c["vs"], hmax // c["hs"]
        if fy > 1 or fx > 1:
            img = np.repeat(np.repeat(img, fy, axis=0), fx, axis=1)
        planes.append(img[:H, :W])
    if len(planes) == 1:
        g = np.clip(np.round(planes[0]), 0, 255).astype(np.uint8)
        rgb = np.stack([g, g, g], -1)
    else:
        y, cb, cr = planes[0], planes[1] - 128.0, planes[2] - 128.0
        r = y + 1.402 * cr
        g = y - 0.344136 * cb - 0.714136 * cr
        b = y + 1.772 * cb
        rgb = np.clip(np.round(np.stack([r, g, b], -1)), 0, 255).astype(np.uint8)
    out = np.full((H, W, 4), 255, np.uint8)
    out[..., :3] = rgb
    return out
