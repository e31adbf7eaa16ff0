"""A small baseline JPEG writer for the reader tests (test infrastructure).

Written from ITU-T T.81 and JFIF: RGB to YCbCr, chroma averaged over each
component's sampling cell, the 8x8 forward DCT, quantisation by a flat table,
and Huffman coding with simple valid tables (every DC category with a 4-bit
code, every AC run/size symbol with an 8-bit code -- never the all-ones code).
It makes the layouts the reference's own encoder (stb_image_write) never
writes: any sampling factors (4:2:2, 4:1:1, 4:4:0, ...), restart intervals,
and one scan per component. The files are decoded by the reader under test
and by the reference's reader and the bytes compared.
"""
from __future__ import annotations

import numpy as np

ZIGZAG = np.array([0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5, 12, 19, 26, 33, 40, 48, 41, 34, 27, 20,
                   13, 6, 7, 14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51, 58, 59, 52,
                   45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63])

_DCT = np.array([[(np.sqrt(0.5) if k == 0 else 1.0) * 0.5 * np.cos((2 * n + 1) * k * np.pi / 16) for n in range(8)]
                 for k in range(8)])
AC_SYMBOLS = [0x00, 0xF0] + [(r << 4) | s for r in range(16) for s in range(1, 11)]


class _Bits:
    def __init__(self):
        self.out = bytearray()
        self.acc = 0
        self.n = 0

    def put(self, code: int, length: int):
        for i in range(length - 1, -1, -1):
            self.acc = (self.acc << 1) | ((code >> i) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                if self.acc == 0xFF:
                    self.out.append(0)
                self.acc, self.n = 0, 0

    def flush(self):
        while self.n:
            self.put(1, 1)  # pad with ones


def _category(v: int) -> int:
    return 0 if v == 0 else int(abs(v)).bit_length()


def _magnitude(v: int, s: int) -> int:
    return v if v >= 0 else v + (1 << s) - 1


def _segment(marker: int, payload: bytes) -> bytes:
    return bytes([0xFF, marker]) + (len(payload) + 2).to_bytes(2, "big") + payload


def write_jpeg(img: np.ndarray, sampling=((2, 2), (1, 1), (1, 1)), quant: int = 4, restart: int = 0,
               interleaved: bool = True, ids=(1, 2, 3)) -> bytes:
    """img (h, w, 3) or (h, w) uint8. sampling: (h, v) per component.
    quant: every quantiser step. restart: MCUs between restart markers
    (0: none). interleaved: one scan for all components, else one per
    component. ids: component identifiers ('R', 'G', 'B' makes it RGB)."""
    img = np.asarray(img)
    grey = img.ndim == 2
    H, W = img.shape[:2]
    if grey:
        planes = [img.astype(np.float64)]
        sampling = sampling[:1]
    else:
        rgb = img.astype(np.float64)
        if ids == (ord("R"), ord("G"), ord("B")):
            planes = [rgb[..., 0], rgb[..., 1], rgb[..., 2]]
        else:
            r, g, b = rgb[..., 0], rgb[..., 1], rgb[..., 2]
            planes = [0.299 * r + 0.587 * g + 0.114 * b,
                      -0.168736 * r - 0.331264 * g + 0.5 * b + 128,
                      0.5 * r - 0.418688 * g - 0.081312 * b + 128]
    hmax = max(s[0] for s in sampling)
    vmax = max(s[1] for s in sampling)
    mcux, mcuy = -(-W // (8 * hmax)), -(-H // (8 * vmax))
    comps = []
    for p, (hs, vs) in zip(planes, sampling):
        fx, fy = hmax // hs, vmax // vs
        # pad to whole sampling cells, average each cell, pad to whole MCUs
        ph, pw = -(-H // fy) * fy, -(-W // fx) * fx
        p = np.pad(p, ((0, ph - H), (0, pw - W)), mode="edge")
        p = p.reshape(ph // fy, fy, pw // fx, fx).mean((1, 3))
        bh, bw = mcuy * vs * 8, mcux * hs * 8
        p = np.pad(p, ((0, bh - p.shape[0]), (0, bw - p.shape[1])), mode="edge")
        coef = np.zeros((bh // 8, bw // 8, 64), np.int32)
        for by in range(bh // 8):
            for bx in range(bw // 8):
                blk = p[by * 8:by * 8 + 8, bx * 8:bx * 8 + 8] - 128.0
                d = _DCT @ blk @ _DCT.T
                coef[by, bx] = np.round(d.reshape(64)[ZIGZAG] / quant).astype(np.int32)
        comps.append((hs, vs, coef))
    nc = len(comps)
    out = bytearray(b"\xFF\xD8")
    out += _segment(0xE0, b"JFIF\0\x01\x01\0\0\x01\0\x01\0\0")
    out += _segment(0xDB, bytes([0]) + bytes([quant] * 64))
    dc_bits = [0] * 16
    dc_bits[3] = 12  # 12 categories, 4-bit codes 0..11
    ac_bits = [0] * 16
    ac_bits[7] = len(AC_SYMBOLS)  # 8-bit codes 0..161
    out += _segment(0xC4, bytes([0x00]) + bytes(dc_bits) + bytes(range(12)))
    out += _segment(0xC4, bytes([0x10]) + bytes(ac_bits) + bytes(AC_SYMBOLS))
    sof = bytes([8]) + H.to_bytes(2, "big") + W.to_bytes(2, "big") + bytes([nc])
    for k, (hs, vs, _) in enumerate(comps):
        sof += bytes([ids[k], (hs << 4) | vs, 0])
    out += _segment(0xC0, sof)
    if restart:
        out += _segment(0xDD, restart.to_bytes(2, "big"))
    ac_code = {s: i for i, s in enumerate(AC_SYMBOLS)}

    def block(bits, coef, pred):
        dc = int(coef[0])
        diff = dc - pred
        s = _category(diff)
        bits.put(s, 4)
        if s:
            bits.put(_magnitude(diff, s), s)
        run = 0
        for k in range(1, 64):
            v = int(coef[k])
            if v == 0:
                run += 1
                continue
            while run > 15:
                bits.put(ac_code[0xF0], 8)
                run -= 16
            s = _category(v)
            bits.put(ac_code[(run << 4) | s], 8)
            bits.put(_magnitude(v, s), s)
            run = 0
        if run:
            bits.put(ac_code[0x00], 8)
        return dc

    def scan(members):
        sos = bytes([len(members)])
        for k in members:
            sos += bytes([ids[k], 0x00])
        sos += bytes([0, 63, 0])
        data = bytearray(_segment(0xDA, sos))
        bits = _Bits()
        preds = [0] * nc
        if len(members) == 1:
            hs, vs, coef = comps[members[0]]
            cw_px, ch_px = -(-W * hs // hmax), -(-H * vs // vmax)  # the component's samples covering the image
            cw, chh = -(-cw_px // 8), -(-ch_px // 8)
            units = [(members[0], bx, by) for by in range(chh) for bx in range(cw)]
            groups = [[u] for u in units]
        else:
            groups = []
            for my in range(mcuy):
                for mx in range(mcux):
                    g = []
                    for k in members:
                        hs, vs, _ = comps[k]
                        g += [(k, mx * hs + u, my * vs + v) for v in range(vs) for u in range(hs)]
                    groups.append(g)
        for i, g in enumerate(groups):
            if restart and i and i % restart == 0:
                bits.flush()
                data += bits.out
                bits.out = bytearray()
                data += bytes([0xFF, 0xD0 + ((i // restart - 1) & 7)])
                preds = [0] * nc
            for k, bx, by in g:
                preds[k] = block(bits, comps[k][2][by, bx], preds[k])
        bits.flush()
        data += bits.out
        return data

    if interleaved:
        out += scan(list(range(nc)))
    else:
        for k in range(nc):
            out += scan([k])
    out += b"\xFF\xD9"
    return bytes(out)
