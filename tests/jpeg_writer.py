"""A small DCT JPEG encoder for the loader tests (ITU-T T.81 baseline and progressive: 8-bit samples,
Huffman coding), and the image a decoder following the loader's rules must produce from it.

jpeg(img, sampling=(2, 2), restart=0, progressive=False) -> (file bytes, expected RGBA8): img is uint8
[h, w, 3] (JFIF YCbCr, the luma component sampled (h, v) times the chroma's) or [h, w] (grey);
progressive files carry the same quantised coefficients in the scans of PROGRESSIVE_SCANS, so they
decode to the same image. The expected image is computed from the quantised coefficients the file holds: dequantised, inverse DCT in float64, level
shift, rounding and clamping, chroma replicated, YCbCr -> RGB with the JFIF constants; a float32
decoder may differ from it by one level. Huffman tables are canonical codes over the symbols that
occur (lengths 2, 2, 3, 3, 4, 4, 5, 5, then 12), so codes of several lengths are exercised.
"""
import math

import numpy as np

ZIGZAG = np.array([0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5, 12, 19, 26, 33, 40, 48, 41, 34, 27, 20,
                   13, 6, 7, 14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51, 58, 59, 52,
                   45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63])
# T[x, u] = C(u) / 2 cos((2x + 1) u pi / 16)
_T = np.array([[(math.sqrt(0.5) if u == 0 else 1.0) * 0.5 * math.cos((2 * x + 1) * u * math.pi / 16) for u in range(8)]
               for x in range(8)])
# quantisation steps (natural order): coarser with frequency, luma and chroma
_QL = np.array([[4 + 2 * (x + y) for x in range(8)] for y in range(8)], np.int64)
_QC = np.array([[6 + 3 * (x + y) for x in range(8)] for y in range(8)], np.int64)


def _fdct(block):
    return _T.T @ block @ _T  # F[v, u]


def _idct(F):
    return _T @ F @ _T.T  # f[y, x]


def _category(v):
    return 0 if v == 0 else int(abs(int(v))).bit_length()


def _amp_bits(v, cat):
    return int(v) if v > 0 else int(v) + (1 << cat) - 1


def _table(symbols):
    syms = sorted(set(symbols))
    lens = [2, 2, 3, 3, 4, 4, 5, 5][:len(syms)] + [12] * max(0, len(syms) - 8)
    counts = [0] * 16
    for L in lens:
        counts[L - 1] += 1
    order = [s for _, s in sorted(zip(lens, syms))]
    codes, code, k = {}, 0, 0
    for L in range(1, 17):
        for _ in range(counts[L - 1]):
            codes[order[k]] = (code, L)
            code += 1
            k += 1
        code <<= 1
    return counts, order, codes


class _Bits:
    def __init__(self):
        self.out, self.acc, self.n = bytearray(), 0, 0

    def put(self, value, n):
        for i in range(n - 1, -1, -1):
            self.acc = (self.acc << 1) | ((value >> i) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                if self.acc == 0xFF:
                    self.out.append(0)
                self.acc, self.n = 0, 0

    def align(self):
        while self.n:
            self.put(1, 1)


def _seg(marker, payload):
    return bytes([0xFF, marker]) + (len(payload) + 2).to_bytes(2, "big") + bytes(payload)


# the progressive scan script (spectral selection, successive approximation) of a three-component
# image: (components, Ss, Se, Ah, Al); a grey image keeps the scans of component 0
PROGRESSIVE_SCANS = [((0, 1, 2), 0, 0, 0, 1), ((0,), 1, 5, 0, 2), ((2,), 1, 63, 0, 1), ((1,), 1, 63, 0, 1),
                     ((0,), 6, 63, 0, 2), ((0,), 1, 63, 2, 1), ((0, 1, 2), 0, 0, 1, 0), ((2,), 1, 63, 1, 0),
                     ((1,), 1, 63, 1, 0), ((0,), 1, 63, 1, 0)]


def _progressive_scans(coefs, factors, hmax, vmax, mcux, mcuy, w, h, restart=0):
    """the entropy-coded scans of a progressive file: per scan its component list, band, table
    definitions and data (T.81 G.1.2: DC first / refinement, AC first with end-of-band runs, AC
    refinement with correction bits buffered over the runs); restart: a marker every `restart` MCUs
    (a block in a one-component scan), the end-of-band run and the DC predictions ended there"""
    ncomp = len(coefs)
    out = []
    for comps, ss, se, ah, al in PROGRESSIVE_SCANS:
        comps = tuple(c for c in comps if c < ncomp)
        if not comps:
            continue
        if len(comps) > 1:
            mcus = [[(k, my * factors[k][1] + v, mx * factors[k][0] + u) for k in comps for v in range(factors[k][1])
                     for u in range(factors[k][0])] for my in range(mcuy) for mx in range(mcux)]
        else:
            k = comps[0]
            cw, ch = -(-w * factors[k][0] // hmax), -(-h * factors[k][1] // vmax)
            mcus = [[(k, by, bx)] for by in range(-(-ch // 8)) for bx in range(-(-cw // 8))]
        ev = []  # ("sym", class, symbol), ("bits", value, n) or ("rst", n)
        st = {"run": 0, "be": []}

        def flush():
            if st["run"]:
                nb = st["run"].bit_length() - 1
                ev.append(("sym", "ac", nb << 4))
                if nb:
                    ev.append(("bits", st["run"] - (1 << nb), nb))
                ev.extend(("bits", b, 1) for b in st["be"])
                st["run"], st["be"] = 0, []

        pred = [0] * ncomp

        def order():
            for m, mcu in enumerate(mcus):
                if restart and m and m % restart == 0:
                    flush()
                    pred[:] = [0] * ncomp
                    ev.append(("rst", (m // restart - 1) % 8))
                yield from mcu

        if ss == 0:
            for k, by, bx in order():
                c = int(coefs[k][by, bx, 0, 0])
                if ah == 0:
                    v = c >> al
                    d = v - pred[k]
                    pred[k] = v
                    cat = _category(d)
                    ev.append(("sym", "dc", cat))
                    if cat:
                        ev.append(("bits", _amp_bits(d, cat), cat))
                else:
                    ev.append(("bits", (c >> al) & 1, 1))
        else:
            for k, by, bx in order():
                zz = coefs[k][by, bx].reshape(-1)[ZIGZAG]
                if ah == 0:
                    r = 0
                    for i in range(ss, se + 1):
                        c = int(zz[i])
                        t = (abs(c) >> al) * (1 if c > 0 else -1)
                        if t == 0:
                            r += 1
                            continue
                        flush()
                        while r > 15:
                            ev.append(("sym", "ac", 0xF0))
                            r -= 16
                        cat = _category(t)
                        ev.append(("sym", "ac", (r << 4) | cat))
                        ev.append(("bits", _amp_bits(t, cat), cat))
                        r = 0
                    if r:
                        st["run"] += 1
                        if st["run"] == 0x7FFF:
                            flush()
                else:
                    absv = [abs(int(zz[i])) >> al for i in range(64)]
                    eob = max([i for i in range(ss, se + 1) if absv[i] == 1], default=-1)
                    r, br = 0, []
                    for i in range(ss, se + 1):
                        t = absv[i]
                        if t == 0:
                            r += 1
                            continue
                        while r > 15 and i <= eob:
                            flush()
                            ev.append(("sym", "ac", 0xF0))
                            r -= 16
                            ev.extend(("bits", b, 1) for b in br)
                            br = []
                        if t > 1:
                            br.append(t & 1)
                            continue
                        flush()
                        ev.append(("sym", "ac", (r << 4) | 1))
                        ev.append(("bits", 1 if zz[i] > 0 else 0, 1))
                        ev.extend(("bits", b, 1) for b in br)
                        br, r = [], 0
                    if r or br:
                        st["run"] += 1
                        st["be"].extend(br)
                        if st["run"] == 0x7FFF or len(st["be"]) > 900:
                            flush()
            flush()
        syms = {}
        for e in ev:
            if e[0] == "sym":
                syms.setdefault(e[1], []).append(e[2])
        tables = {cls: _table(v) for cls, v in syms.items()}
        bits = _Bits()
        for e in ev:
            if e[0] == "sym":
                code, L = tables[e[1]][2][e[2]]
                bits.put(code, L)
            elif e[0] == "rst":
                bits.align()
                bits.out += bytes([0xFF, 0xD0 + e[1]])
            else:
                bits.put(e[1], e[2])
        bits.align()
        dht = b"".join(_seg(0xC4, bytes([(0 if cls == "dc" else 1) << 4]) + bytes(t[0]) + bytes(t[1]))
                       for cls, t in sorted(tables.items()))
        sos = bytearray([len(comps)])
        for k in comps:
            sos += bytes([k + 1, 0x00])  # DC and AC tables 0, redefined before every scan
        sos += bytes([ss, se, (ah << 4) | al])
        out.append(dht + _seg(0xDA, sos) + bytes(bits.out))
    return out


def jpeg(img, sampling=(2, 2), restart=0, progressive=False, adobe_rgb=False):
    img = np.asarray(img, np.uint8)
    grey = img.ndim == 2
    h, w = img.shape[:2]
    if grey:
        planes_full = [img.astype(np.float64)]
        factors = [(1, 1)]
    elif adobe_rgb:
        # an Adobe APP14 marker with transform 0: the components are R, G, B, not subsampled
        planes_full = [img[..., i].astype(np.float64) for i in range(3)]
        factors = [(1, 1)] * 3
    else:
        r, g, b = (img[..., i].astype(np.float64) for i in range(3))
        y = 0.299 * r + 0.587 * g + 0.114 * b
        cb = -0.168736 * r - 0.331264 * g + 0.5 * b + 128
        cr = 0.5 * r - 0.418688 * g - 0.081312 * b + 128
        planes_full = [np.clip(np.rint(p), 0, 255) for p in (y, cb, cr)]
        factors = [tuple(sampling), (1, 1), (1, 1)]
    hmax, vmax = max(f[0] for f in factors), max(f[1] for f in factors)
    mcux, mcuy = -(-w // (8 * hmax)), -(-h // (8 * vmax))
    pw, ph = mcux * 8 * hmax, mcuy * 8 * vmax
    quant = [_QL] if grey else [_QL, _QC, _QC]
    coefs, recon = [], []
    for k, p in enumerate(planes_full):
        full = np.pad(p, ((0, ph - h), (0, pw - w)), mode="edge")
        fh, fv = factors[k]
        sx, sy = hmax // fh, vmax // fv
        plane = full.reshape(ph // sy, sy, pw // sx, sx).mean(axis=(1, 3))  # box-filtered to the component's size
        bh, bw = plane.shape[0] // 8, plane.shape[1] // 8
        q = quant[k]
        qc = np.zeros((bh, bw, 8, 8), np.int64)
        rec = np.zeros_like(plane)
        for by in range(bh):
            for bx in range(bw):
                F = _fdct(plane[8 * by:8 * by + 8, 8 * bx:8 * bx + 8] - 128.0)
                qv = np.rint(F / q).astype(np.int64)
                qc[by, bx] = qv
                f = _idct(qv * q)
                rec[8 * by:8 * by + 8, 8 * bx:8 * bx + 8] = np.clip(np.floor(f + 128.5), 0, 255)
        coefs.append(qc)
        recon.append(rec)
    # the expected image: chroma replicated, JFIF conversion
    yy, xx = np.mgrid[0:h, 0:w]
    samp = [recon[k][(yy * factors[k][1]) // vmax, (xx * factors[k][0]) // hmax] for k in range(len(recon))]
    exp = np.full((h, w, 4), 255, np.uint8)
    if grey:
        exp[..., 0] = exp[..., 1] = exp[..., 2] = samp[0].astype(np.uint8)
    elif adobe_rgb:
        for i in range(3):
            exp[..., i] = samp[i].astype(np.uint8)
    else:
        Y, Cb, Cr = samp[0], samp[1] - 128.0, samp[2] - 128.0
        rgb = [Y + 1.402 * Cr, Y - 0.344136 * Cb - 0.714136 * Cr, Y + 1.772 * Cb]
        for i in range(3):
            exp[..., i] = np.clip(np.floor(rgb[i] + 0.5), 0, 255).astype(np.uint8)

    app = _seg(0xEE, b"Adobe\x00\x64\x00\x00\x00\x00\x00") if adobe_rgb else \
        _seg(0xE0, b"JFIF\x00\x01\x01\x00\x00\x01\x00\x01\x00\x00")
    if progressive:
        data = bytearray(b"\xFF\xD8") + app
        for t, q in enumerate(quant[:1] if grey else quant[:2]):
            data += _seg(0xDB, bytes([t]) + bytes(int(v) for v in q.reshape(-1)[ZIGZAG]))
        comps = bytearray([8]) + h.to_bytes(2, "big") + w.to_bytes(2, "big") + bytes([len(coefs)])
        for k in range(len(coefs)):
            comps += bytes([k + 1, (factors[k][0] << 4) | factors[k][1], 0 if k == 0 else 1])
        data += _seg(0xC2, comps)
        if restart:
            data += _seg(0xDD, restart.to_bytes(2, "big"))
        for scan in _progressive_scans(coefs, factors, hmax, vmax, mcux, mcuy, w, h, restart):
            data += scan
        data += b"\xFF\xD9"
        return bytes(data), exp

    # the MCU sequence: (component, block row, block column) per block, MCUs in raster order
    def blocks():
        for my in range(mcuy):
            for mx in range(mcux):
                yield [(k, my * factors[k][1] + v, mx * factors[k][0] + u) for k in range(len(coefs))
                       for v in range(factors[k][1]) for u in range(factors[k][0])]

    def symbols():
        pred = [0] * len(coefs)
        for m, mcu in enumerate(blocks()):
            if restart and m and m % restart == 0:
                pred = [0] * len(coefs)
            for k, by, bx in mcu:
                zz = coefs[k][by, bx].reshape(-1)[ZIGZAG]
                d = int(zz[0]) - pred[k]
                pred[k] = int(zz[0])
                out = [("dc", k, _category(d), d)]
                run = 0
                last = max([i for i in range(1, 64) if zz[i] != 0], default=0)
                for i in range(1, last + 1):
                    if zz[i] == 0:
                        run += 1
                        continue
                    while run > 15:
                        out.append(("ac", k, 0xF0, 0))
                        run -= 16
                    c = _category(zz[i])
                    out.append(("ac", k, (run << 4) | c, int(zz[i])))
                    run = 0
                if last < 63:
                    out.append(("ac", k, 0x00, 0))
                yield m, out

    cls = (lambda k: 0 if k == 0 else 1)
    used = {}
    for _, out in symbols():
        for kind, k, s, _ in out:
            used.setdefault((kind, cls(k)), []).append(s)
    tables = {key: _table(v) for key, v in used.items()}
    bits = _Bits()
    prev_m = 0
    for m, out in symbols():
        if restart and m and m % restart == 0 and m != prev_m:
            bits.align()
            bits.out += bytes([0xFF, 0xD0 + ((m // restart - 1) % 8)])
        prev_m = m
        for kind, k, s, v in out:
            code, L = tables[(kind, cls(k))][2][s]
            bits.put(code, L)
            cat = s if kind == "dc" else s & 15
            if cat:
                bits.put(_amp_bits(v, cat), cat)
    bits.align()

    data = bytearray(b"\xFF\xD8") + app
    for t, q in enumerate(quant[:1] if grey else quant[:2]):
        data += _seg(0xDB, bytes([t]) + bytes(int(v) for v in q.reshape(-1)[ZIGZAG]))
    comps = bytearray([8]) + h.to_bytes(2, "big") + w.to_bytes(2, "big") + bytes([len(coefs)])
    for k in range(len(coefs)):
        comps += bytes([k + 1, (factors[k][0] << 4) | factors[k][1], cls(k)])
    data += _seg(0xC0, comps)
    for (kind, c), (counts, order, _) in sorted(tables.items()):
        data += _seg(0xC4, bytes([(0 if kind == "dc" else 1) << 4 | c]) + bytes(counts) + bytes(order))
    if restart:
        data += _seg(0xDD, restart.to_bytes(2, "big"))
    sos = bytearray([len(coefs)])
    for k in range(len(coefs)):
        sos += bytes([k + 1, (cls(k) << 4) | cls(k)])
    sos += bytes([0, 63, 0])
    data += _seg(0xDA, sos)
    data += bits.out
    data += b"\xFF\xD9"
    return bytes(data), exp
