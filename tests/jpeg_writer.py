"""A small sequential JPEG writer for the decoder's tests (ITU-T T.81,
baseline): YCbCr (or grey) from RGB, optional 2x1 / 2x2 chroma subsampling,
an 8x8 DCT in float64, quantisation by a given table, Huffman tables built
from the image's own symbol counts (limited to 16 bits by the adjustment of
T.81 Annex K.2), restart markers, and interleaved or one-component scans.

reconstruct() gives what a decoder following the standard returns for the
same quantised coefficients: exact inverse DCT rounded to 8 bits, chroma
upsampled by the triangle filter (3/4 nearer, 1/4 farther sample) for 2x1 and
2x2, JFIF YCbCr to RGB rounded."""
import heapq
import math
import struct

import numpy as np

ZZ = []  # natural index of zigzag position k
for s in range(15):
    rows = range(max(0, s - 7), min(s, 7) + 1)
    for r in (rows if s % 2 else reversed(rows)):
        ZZ.append(r * 8 + (s - r))
ZZ = np.array(ZZ)

_C = np.array([[(math.sqrt(0.5) if u == 0 else 1.0) * math.cos((2 * x + 1) * u * math.pi / 16) / 2
                for u in range(8)] for x in range(8)])  # [x][u]


def fdct(b):
    return _C.T @ b @ _C          # F[v][u] from f[y][x]


def idct(F):
    return _C @ F @ _C.T


def _category(v):
    return 0 if v == 0 else int(abs(v)).bit_length()


def _bits_of(v, s):
    return v if v >= 0 else v + (1 << s) - 1


class _BitWriter:
    def __init__(self):
        self.out = bytearray()
        self.acc = 0
        self.n = 0

    def put(self, code, length):
        for i in range(length - 1, -1, -1):
            self.acc = (self.acc << 1) | ((code >> i) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                if self.acc == 0xFF:
                    self.out.append(0)
                self.acc = self.n = 0

    def flush(self):
        while self.n:
            self.put(1, 1)  # pad with ones


def _huffman_table(freq):
    """(BITS[16], HUFFVAL) for symbol counts, lengths <= 16, no all-ones code."""
    freq = dict(freq)
    freq[256] = 1  # reserved code point (T.81 K.2)
    heap = [(f, i, [s]) for i, (s, f) in enumerate(sorted(freq.items()))]
    heapq.heapify(heap)
    length = {s: 0 for s in freq}
    if len(heap) == 1:
        length[heap[0][2][0]] = 1
    k = len(heap)
    while len(heap) > 1:
        f1, _, a = heapq.heappop(heap)
        f2, _, b = heapq.heappop(heap)
        for s in a + b:
            length[s] += 1
        heapq.heappush(heap, (f1 + f2, k, a + b))
        k += 1
    bits = [0] * 33
    for s, L in length.items():
        bits[L] += 1
    for i in range(32, 16, -1):   # Annex K.2: limit the code lengths to 16
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
    bits[i] -= 1                  # drop the reserved code point
    order = sorted((s for s in freq if s != 256), key=lambda s: (length[s], s))
    # the reserved symbol had the longest code: it was last; lengths after the
    # adjustment are assigned in this order
    return bits[1:17], order


def _codes(bits, vals):
    codes, code, k = {}, 0, 0
    for L in range(1, 17):
        for _ in range(bits[L - 1]):
            codes[vals[k]] = (code, L)
            code += 1
            k += 1
        code <<= 1
    return codes


def _segment(marker, body):
    return bytes([0xFF, marker]) + struct.pack(">H", len(body) + 2) + body


def encode(rgb, quality_table, subsampling=(2, 2), grey=False, restart=0, interleaved=True):
    """rgb: (H, W, 3) uint8. Returns (jpeg bytes, quantised blocks per
    component, component layout) for reconstruct()."""
    H, W = rgb.shape[:2]
    x = rgb.astype(np.float64)
    if grey:
        planes = [0.299 * x[..., 0] + 0.587 * x[..., 1] + 0.114 * x[..., 2]]
        factors = [(1, 1)]
    else:
        Y = 0.299 * x[..., 0] + 0.587 * x[..., 1] + 0.114 * x[..., 2]
        Cb = -0.168736 * x[..., 0] - 0.331264 * x[..., 1] + 0.5 * x[..., 2] + 128
        Cr = 0.5 * x[..., 0] - 0.418688 * x[..., 1] - 0.081312 * x[..., 2] + 128
        planes = [Y, Cb, Cr]
        factors = [subsampling, (1, 1), (1, 1)]
    hmax = max(f[0] for f in factors)
    vmax = max(f[1] for f in factors)
    mcux, mcuy = -(-W // (8 * hmax)), -(-H // (8 * vmax))
    q = np.asarray(quality_table, np.int64).reshape(64)  # zigzag order
    comps = []
    for ci, (pl, (h, v)) in enumerate(zip(planes, factors)):
        fx, fy = hmax // h, vmax // v
        cw, ch = -(-W * h // hmax), -(-H * v // vmax)
        # subsample by averaging, pad by edge replication to whole MCUs
        small = pl[: (H // fy) * fy or H, : (W // fx) * fx or W]
        if fx > 1 or fy > 1:
            padded = np.pad(pl, ((0, (-H) % fy), (0, (-W) % fx)), mode="edge")
            small = padded.reshape(padded.shape[0] // fy, fy, padded.shape[1] // fx, fx).mean((1, 3))
        small = small[:ch, :cw]
        bw, bh = mcux * h, mcuy * v
        full = np.pad(small, ((0, bh * 8 - small.shape[0]), (0, bw * 8 - small.shape[1])), mode="edge")
        blocks = np.zeros((bh, bw, 64), np.int64)
        for by in range(bh):
            for bx in range(bw):
                F = fdct(full[by * 8:by * 8 + 8, bx * 8:bx * 8 + 8] - 128).reshape(64)
                blocks[by, bx] = np.round(F[ZZ] / q).astype(np.int64)   # zigzag order
        comps.append(dict(id=ci + 1, h=h, v=v, bw=bw, bh=bh, cw=cw, ch=ch, blocks=blocks))

    def block_order(scan):
        if len(scan) > 1:
            for my in range(mcuy):
                for mx in range(mcux):
                    for c in scan:
                        for by in range(c["v"]):
                            for bx in range(c["h"]):
                                yield c, my * c["v"] + by, mx * c["h"] + bx
        else:
            c = scan[0]
            for by in range(-(-c["ch"] // 8)):
                for bx in range(-(-c["cw"] // 8)):
                    yield c, by, bx

    scans = [comps] if interleaved else [[c] for c in comps]
    # symbol statistics, then tables (one DC and one AC table per component)
    out = bytearray(b"\xFF\xD8")
    out += _segment(0xDB, bytes([0]) + bytes(int(v) for v in q))
    sof = struct.pack(">BHHB", 8, H, W, len(comps))
    for c in comps:
        sof += bytes([c["id"], c["h"] << 4 | c["v"], 0])
    out += _segment(0xC0, sof)
    if restart:
        out += _segment(0xDD, struct.pack(">H", restart))
    for scan in scans:
        units = list(block_order(scan))
        dcf, acf = [{} for _ in comps], [{} for _ in comps]
        pred = {c["id"]: 0 for c in comps}
        symbols = []
        mcu_len = sum(c["h"] * c["v"] for c in scan) if len(scan) > 1 else 1
        for n, (c, by, bx) in enumerate(units):
            if restart and n % (mcu_len * restart) == 0:
                pred = {k: 0 for k in pred}
            b = c["blocks"][by, bx]
            diff = int(b[0]) - pred[c["id"]]
            pred[c["id"]] = int(b[0])
            s = _category(diff)
            dcf[c["id"] - 1][s] = dcf[c["id"] - 1].get(s, 0) + 1
            seq = [("dc", c, s, diff)]
            run = 0
            last = max([k for k in range(1, 64) if b[k] != 0], default=0)
            for k in range(1, last + 1):
                if b[k] == 0:
                    run += 1
                    continue
                while run > 15:
                    seq.append(("ac", c, 0xF0, None))
                    run -= 16
                s = _category(int(b[k]))
                seq.append(("ac", c, run << 4 | s, int(b[k])))
                run = 0
            if last < 63:
                seq.append(("ac", c, 0x00, None))
            for kind, cc, sym, _ in seq:
                if kind == "ac":
                    acf[cc["id"] - 1][sym] = acf[cc["id"] - 1].get(sym, 0) + 1
            symbols.append(seq)
        tables = {}
        dht = bytearray()
        for c in scan:
            i = c["id"] - 1
            for cls, f in ((0, dcf[i]), (1, acf[i])):
                bits, vals = _huffman_table(f)
                tables[(cls, i)] = _codes(bits, vals)
                dht += bytes([cls << 4 | i]) + bytes(bits) + bytes(vals)
        out += _segment(0xC4, bytes(dht))
        sos = bytes([len(scan)])
        for c in scan:
            i = c["id"] - 1
            sos += bytes([c["id"], i << 4 | i])
        out += _segment(0xDA, sos + bytes([0, 63, 0]))
        w = _BitWriter()
        rst = 0
        for n, seq in enumerate(symbols):
            if restart and n and n % (mcu_len * restart) == 0:
                w.flush()
                out += bytes(w.out) + bytes([0xFF, 0xD0 + rst])
                w.out = bytearray()
                rst = (rst + 1) % 8
            for kind, c, sym, val in seq:
                i = c["id"] - 1
                if kind == "dc":
                    code, L = tables[(0, i)][sym]
                    w.put(code, L)
                    if sym:
                        w.put(_bits_of(val, sym), sym)
                else:
                    code, L = tables[(1, i)][sym]
                    w.put(code, L)
                    s = sym & 15
                    if s:
                        w.put(_bits_of(val, s), s)
        w.flush()
        out += bytes(w.out)
    out += b"\xFF\xD9"
    return bytes(out), comps, (W, H, hmax, vmax, q)


def reconstruct(comps, layout, grey=False):
    """(H, W, 3) BGR float64 as the standard decoder of the same file."""
    W, H, hmax, vmax, q = layout
    planes = []
    for c in comps:
        bh, bw = c["bh"], c["bw"]
        pl = np.zeros((bh * 8, bw * 8))
        for by in range(bh):
            for bx in range(bw):
                F = np.zeros(64)
                F[ZZ] = c["blocks"][by, bx] * q
                pl[by * 8:by * 8 + 8, bx * 8:bx * 8 + 8] = np.clip(np.floor(idct(F.reshape(8, 8)) + 128 + 0.5), 0, 255)
        pl = pl[:c["ch"], :c["cw"]]
        fx, fy = hmax // c["h"], vmax // c["v"]
        if fx == 2:
            xs = np.arange(W)
            near, far = xs >> 1, np.clip((xs >> 1) + np.where(xs & 1, 1, -1), 0, c["cw"] - 1)
            pl = 0.75 * pl[:, near] + 0.25 * pl[:, far]
        if fy == 2:
            ys = np.arange(H)
            near, far = ys >> 1, np.clip((ys >> 1) + np.where(ys & 1, 1, -1), 0, c["ch"] - 1)
            pl = 0.75 * pl[near, :] + 0.25 * pl[far, :]
        planes.append(pl[:H, :W])
    if grey:
        g = np.clip(np.floor(planes[0] + 0.5), 0, 255)
        return np.stack([g, g, g], -1)
    Y, cb, cr = planes[0], planes[1] - 128, planes[2] - 128
    r = Y + 1.402 * cr
    g = Y - 0.344136 * cb - 0.714136 * cr
    b = Y + 1.772 * cb
    return np.clip(np.floor(np.stack([b, g, r], -1) + 0.5), 0, 255)
