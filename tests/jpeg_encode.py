"""A small baseline (sequential DCT, Huffman) JPEG encoder for test fixtures,
and the image a conforming decoder reconstructs from its output.

Test infrastructure only: no JPEG encoder is available here, and the decoder
under test (the GPU colour path of the frame reader) needs JPEG files. The
encoder follows ITU-T T.81 (baseline process, interchange format): JFIF
YCbCr, 4:4:4 or 4:2:0 sampling, an 8x8 DCT, quantisation with tables of its
own (growing with spatial frequency, scaled by a quality), zig-zag order,
DC differences and AC run-lengths coded with canonical Huffman tables built
per image from the symbol counts (lengths limited to 16 bits by the
standard's length adjustment), byte stuffing, one scan. `reconstruct`
decodes the coefficients the encoder wrote in float64 (dequantisation,
inverse DCT, chroma upsampling by replication, JFIF YCbCr -> RGB): a
conforming decoder matches it to within its own IDCT and upsampling
arithmetic."""
from __future__ import annotations

import heapq
import struct

import numpy as np


def _zigzag() -> np.ndarray:
    """Zig-zag position -> row-major index (T.81 figure 5): anti-diagonals
    r + c = s in turn, rows rising on odd s and falling on even s."""
    order = []
    for s in range(15):
        cells = [(r, s - r) for r in range(8) if 0 <= s - r < 8]
        if s % 2 == 0:
            cells.reverse()
        order += [r * 8 + c for r, c in cells]
    return np.array(order)


ZIGZAG = _zigzag()


def quant_table(quality: int, chroma: bool) -> np.ndarray:
    """8x8 quantiser steps growing with u + v, scaled by quality (1..100)."""
    u, v = np.meshgrid(np.arange(8), np.arange(8), indexing="ij")
    base = (10.0 if not chroma else 14.0) + (u + v) * (5.0 if not chroma else 7.0)
    scale = (5000.0 / quality) if quality < 50 else (200.0 - 2.0 * quality)
    return np.clip(np.floor((base * scale + 50.0) / 100.0), 1, 255).astype(np.int32)


def _dct_matrix() -> np.ndarray:
    k = np.arange(8)
    C = np.cos((2 * k[None, :] + 1) * k[:, None] * np.pi / 16.0)
    C[0] *= np.sqrt(0.5)
    return C * 0.5  # F = C f C^T (T.81 A.3.3)


DCT = _dct_matrix()


def rgb_to_ycbcr(rgb: np.ndarray) -> np.ndarray:
    r, g, b = (rgb[..., c].astype(np.float64) for c in range(3))
    y = 0.299 * r + 0.587 * g + 0.114 * b
    cb = -0.168736 * r - 0.331264 * g + 0.5 * b + 128.0
    cr = 0.5 * r - 0.418688 * g - 0.081312 * b + 128.0
    return np.stack([y, cb, cr], -1)


def ycbcr_to_rgb(ycc: np.ndarray) -> np.ndarray:
    y, cb, cr = ycc[..., 0], ycc[..., 1] - 128.0, ycc[..., 2] - 128.0
    rgb = np.stack([y + 1.402 * cr, y - 0.344136 * cb - 0.714136 * cr, y + 1.772 * cb], -1)
    return np.clip(np.floor(rgb + 0.5), 0, 255).astype(np.uint8)


def _pad(a: np.ndarray, h: int, w: int) -> np.ndarray:
    return np.pad(a, ((0, h - a.shape[0]), (0, w - a.shape[1])), mode="edge")


def _blocks(plane: np.ndarray) -> np.ndarray:
    """[H, W] -> [H/8, W/8, 8, 8]"""
    h, w = plane.shape
    return plane.reshape(h // 8, 8, w // 8, 8).transpose(0, 2, 1, 3)


def _unblocks(b: np.ndarray) -> np.ndarray:
    n, m = b.shape[:2]
    return b.transpose(0, 2, 1, 3).reshape(n * 8, m * 8)


def _huffman_table(freq: dict) -> tuple[list, list, dict]:
    """(BITS[1..16], HUFFVAL, {symbol: (code, length)}) of a canonical Huffman
    code for the symbol counts: code sizes from a Huffman tree with one
    reserved symbol (so no code is all ones), lengths over 16 moved down by
    the adjustment of T.81 Annex K.2, the reserved code removed."""
    items = [(f, s, [s]) for s, f in freq.items() if f > 0] + [(1, 256, [256])]
    heapq.heapify(items)
    size = {s: 0 for _, s, _ in items}
    while len(items) > 1:
        f1, t1, s1 = heapq.heappop(items)
        f2, t2, s2 = heapq.heappop(items)
        for q in s1 + s2:
            size[q] += 1
        heapq.heappush(items, (f1 + f2, min(t1, t2), s1 + s2))
    bits = [0] * 33
    for q, n in size.items():
        bits[n] += 1
    for i in range(32, 16, -1):
        while bits[i] > 0:
            j = i - 2
            while bits[j] == 0:
                j -= 1
            bits[i] -= 2
            bits[i - 1] += 1
            bits[j + 1] += 2
            bits[j] -= 1
    i = 16
    while bits[i] == 0:
        i -= 1
    bits[i] -= 1  # the reserved symbol's code
    vals = sorted((q for q in size if q != 256), key=lambda q: (size[q], q))
    codes, code, k = {}, 0, 0
    for n in range(1, 17):
        for _ in range(bits[n]):
            codes[vals[k]] = (code, n)
            code += 1
            k += 1
        code <<= 1
    return bits[1:17], vals, codes


class _Bits:
    def __init__(self):
        self.out = bytearray()
        self.acc = 0
        self.n = 0

    def put(self, value: int, n: int):
        for b in range(n - 1, -1, -1):
            self.acc = (self.acc << 1) | ((value >> b) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                if self.acc == 0xFF:
                    self.out.append(0)  # byte stuffing
                self.acc = self.n = 0

    def flush(self) -> bytes:
        if self.n:
            self.put((1 << (8 - self.n)) - 1, 8 - self.n)  # pad with ones
        return bytes(self.out)


def _category(v: int) -> tuple[int, int]:
    """(size, extra bits) of a DC difference or AC coefficient (T.81 F.1.2)."""
    n = abs(v).bit_length()
    return n, (v if v >= 0 else v + (1 << n) - 1)


def encode(rgb: np.ndarray, quality: int = 90, subsample: bool = False) -> tuple[bytes, np.ndarray]:
    """Baseline JPEG of an [H, W, 3] uint8 RGB image; returns (file bytes,
    the RGB image a decoder reconstructs from them, by replicated chroma)."""
    h, w = rgb.shape[:2]
    mcu = 16 if subsample else 8
    H, W = -(-h // mcu) * mcu, -(-w // mcu) * mcu
    ycc = rgb_to_ycbcr(rgb)
    planes = [_pad(ycc[..., 0], H, W)]
    for c in (1, 2):
        p = _pad(ycc[..., c], H, W)
        planes.append(p.reshape(H // 2, 2, W // 2, 2).mean(axis=(1, 3)) if subsample else p)
    qts = [quant_table(quality, False), quant_table(quality, True)]
    coefs, recon = [], []
    for c, p in enumerate(planes):
        qt = qts[0 if c == 0 else 1]
        F = np.einsum("ij,abjk,lk->abil", DCT, _blocks(p - 128.0), DCT)
        Q = np.round(F / qt).astype(np.int64)
        coefs.append(Q)
        f = np.einsum("ji,abjk,kl->abil", DCT, (Q * qt).astype(np.float64), DCT) + 128.0
        recon.append(np.clip(np.floor(_unblocks(f) + 0.5), 0, 255))
    if subsample:
        recon[1:] = [np.repeat(np.repeat(r, 2, 0), 2, 1) for r in recon[1:]]
    rec = ycbcr_to_rgb(np.stack([r[:h, :w] for r in recon], -1))

    # symbols in scan order: (table class 0 DC / 1 AC, table id, symbol, extra, extra length)
    syms, pred = [], [0, 0, 0]
    ny, nx = H // mcu, W // mcu
    order = []
    for my in range(ny):
        for mx in range(nx):
            if subsample:
                order += [(0, 2 * my, 2 * mx), (0, 2 * my, 2 * mx + 1), (0, 2 * my + 1, 2 * mx),
                          (0, 2 * my + 1, 2 * mx + 1)]
            else:
                order.append((0, my, mx))
            order += [(1, my, mx), (2, my, mx)]
    for c, by, bx in order:
        z = coefs[c][by, bx].reshape(64)[ZIGZAG]
        t = 0 if c == 0 else 1
        n, e = _category(int(z[0]) - pred[c])
        pred[c] = int(z[0])
        syms.append((0, t, n, e, n))
        run = 0
        for k in range(1, 64):
            if z[k] == 0:
                run += 1
                continue
            while run > 15:
                syms.append((1, t, 0xF0, 0, 0))
                run -= 16
            n, e = _category(int(z[k]))
            syms.append((1, t, (run << 4) | n, e, n))
            run = 0
        if run:
            syms.append((1, t, 0x00, 0, 0))
    tables = {}
    for tc in (0, 1):
        for t in (0, 1):
            freq = {}
            for a, b, sym, _, _ in syms:
                if a == tc and b == t:
                    freq[sym] = freq.get(sym, 0) + 1
            tables[tc, t] = _huffman_table(freq)
    bw = _Bits()
    for tc, t, sym, e, n in syms:
        code, length = tables[tc, t][2][sym]
        bw.put(code, length)
        if n:
            bw.put(e, n)
    data = bw.flush()

    def seg(marker: int, body: bytes) -> bytes:
        return struct.pack(">HH", marker, len(body) + 2) + body

    dqt = b"".join(bytes([t]) + bytes(int(v) for v in qts[t].reshape(64)[ZIGZAG]) for t in (0, 1))
    samp = 0x22 if subsample else 0x11
    sof = struct.pack(">BHHB", 8, h, w, 3) + bytes([1, samp, 0, 2, 0x11, 1, 3, 0x11, 1])
    dht = b""
    for tc in (0, 1):
        for t in (0, 1):
            bits, vals, _ = tables[tc, t]
            dht += bytes([(tc << 4) | t]) + bytes(bits) + bytes(vals)
    sos = bytes([3, 1, 0x00, 2, 0x11, 3, 0x11, 0, 63, 0])
    out = (b"\xff\xd8" + seg(0xFFDB, dqt) + seg(0xFFC0, sof) + seg(0xFFC4, dht) + seg(0xFFDA, sos) + data +
           b"\xff\xd9")
    return out, rec
