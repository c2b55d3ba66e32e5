"""Writer of 16-bit mono FLAC (.ldf) RF captures.

The reference writes ``.ldf`` test captures through libsndfile
(Core/Decode/LdTestLdfWriter.cs, ``LdTestLdfWriter.Write``); this module
writes them without a codec library, following the published format (IETF
RFC 9639, "Free Lossless Audio Codec").  ``write`` makes a valid stream whose
frames use every subframe and residual form a decoder must read: CONSTANT,
VERBATIM, FIXED orders 0-4, LPC orders 1-32 with quantised Levinson-Durbin
coefficients, wasted bits, Rice and Rice2 partitions with partition orders
0-8, and escaped partitions, so a decoder that reads its streams back
losslessly reads every form.  A frame's CRC-8 and CRC-16 are those of the
format.
"""
import numpy as np

# ---------------------------------------------------------------- checksums


def _crc8_table():
    t = []
    for b in range(256):
        c = b
        for _ in range(8):
            c = ((c << 1) ^ 0x07) & 0xFF if c & 0x80 else (c << 1) & 0xFF
        t.append(c)
    return t


def _crc16_table():
    t = []
    for b in range(256):
        c = b << 8
        for _ in range(8):
            c = ((c << 1) ^ 0x8005) & 0xFFFF if c & 0x8000 else (c << 1) & 0xFFFF
        t.append(c)
    return t


CRC8 = _crc8_table()
CRC16 = _crc16_table()


def crc8(data):
    c = 0
    for b in data:
        c = CRC8[c ^ b]
    return c


def crc16(data):
    c = 0
    for b in data:
        c = ((c << 8) & 0xFFFF) ^ CRC16[(c >> 8) ^ b]
    return c


# ---------------------------------------------------------------- bit writer

class _Bits:
    """MSB-first bit writer built on a list of (value, width) pieces, packed at the end."""

    def __init__(self):
        self.parts = []   # numpy bool arrays
        self.n = 0

    def put(self, value, width):
        if width == 0:
            return
        v = int(value) & ((1 << width) - 1)
        bits = np.array([(v >> (width - 1 - i)) & 1 for i in range(width)], np.uint8)
        self.parts.append(bits)
        self.n += width

    def put_array(self, bits):
        self.parts.append(bits.astype(np.uint8))
        self.n += len(bits)

    def align(self):
        pad = (-self.n) % 8
        if pad:
            self.put(0, pad)

    def bytes(self):
        self.align()
        if not self.parts:
            return b""
        return np.packbits(np.concatenate(self.parts)).tobytes()


def _rice_bits(u, k):
    """Rice codes of unsigned values u (numpy int64) with parameter k, MSB first."""
    u = np.asarray(u, np.int64)
    q = u >> k
    lens = q + 1 + k
    total = int(lens.sum())
    bits = np.zeros(total, np.uint8)
    start = np.concatenate([[0], np.cumsum(lens)[:-1]])
    bits[start + q] = 1
    for j in range(k):
        bits[start + q + 1 + j] = (u >> (k - 1 - j)) & 1
    return bits


def _signed_bits(vals, width):
    vals = np.asarray(vals, np.int64) & ((1 << width) - 1)
    out = np.zeros((len(vals), width), np.uint8)
    for j in range(width):
        out[:, j] = (vals >> (width - 1 - j)) & 1
    return out.ravel()


def _zigzag(r):
    r = np.asarray(r, np.int64)
    return np.where(r >= 0, 2 * r, -2 * r - 1)


def _write_residual(w, res, order, block, method, porder, escape_every=0):
    """Residual section: partitioned Rice (method 0, 4-bit parameters) or Rice2 (1, 5-bit)."""
    w.put(method, 2)
    w.put(porder, 4)
    parts = 1 << porder
    pbits = 4 if method == 0 else 5
    esc = (1 << pbits) - 1
    pos = 0
    for p in range(parts):
        n = (block >> porder) - (order if p == 0 else 0)
        seg = res[pos:pos + n]
        pos += n
        u = _zigzag(seg)
        if escape_every and p % escape_every == escape_every - 1:
            # escaped partition: 5-bit raw width, then signed raw samples
            need = (int(np.max(np.abs(seg))).bit_length() + 1) if n else 0
            w.put(esc, pbits)
            w.put(need, 5)
            if n and need:
                w.put_array(_signed_bits(seg, need))
            continue
        mean = float(np.mean(u)) if n else 0.0
        k = max(0, int(np.floor(np.log2(mean))) if mean > 1 else 0)
        k = min(k, esc - 1)
        w.put(k, pbits)
        if n:
            w.put_array(_rice_bits(u, k))
    assert pos == block - order


FIXED_COEFS = {0: [], 1: [1], 2: [2, -1], 3: [3, -3, 1], 4: [4, -6, 4, -1]}


def _fixed_residual(x, order):
    x = np.asarray(x, np.int64)
    r = x[order:].copy()
    for j, c in enumerate(FIXED_COEFS[order]):
        r -= c * x[order - 1 - j:len(x) - 1 - j]
    return r


def _lpc_coefs(x, order, precision):
    """Levinson-Durbin on the autocorrelation, quantised to `precision` bits with a shift."""
    xf = np.asarray(x, np.float64)
    xf = xf * np.hanning(len(xf)) if len(xf) > 8 else xf
    ac = np.array([np.dot(xf[:len(xf) - i], xf[i:]) for i in range(order + 1)])
    if ac[0] <= 0:
        return None
    ac[0] *= 1.0 + 1e-9
    a = np.zeros(order)
    err = ac[0]
    for i in range(order):
        k = (ac[i + 1] - np.dot(a[:i], ac[i:0:-1])) / err
        a_new = a.copy()
        a_new[i] = k
        a_new[:i] = a[:i] - k * a[:i][::-1]
        a = a_new
        err *= (1.0 - k * k)
        if err <= 0:
            return None
    cmax = np.max(np.abs(a))
    if cmax == 0:
        return None
    lim = (1 << (precision - 1)) - 1
    shift = precision - 1 - int(np.floor(np.log2(cmax))) - 1
    shift = max(0, min(15, shift))
    q = np.round(a * (1 << shift)).astype(np.int64)
    q = np.clip(q, -lim - 1, lim)
    return q, shift


def _lpc_residual(x, coefs, shift):
    x = np.asarray(x, np.int64)
    order = len(coefs)
    pred = np.zeros(len(x) - order, np.int64)
    for j, c in enumerate(coefs):
        pred += int(c) * x[order - 1 - j:len(x) - 1 - j]
    return x[order:] - (pred >> shift)


def _utf8_number(n):
    if n < 0x80:
        return bytes([n])
    for nbytes, lead, top in ((2, 0xC0, 11), (3, 0xE0, 16), (4, 0xF0, 21), (5, 0xF8, 26),
                              (6, 0xFC, 31), (7, 0xFE, 36)):
        if n < (1 << top):
            out = []
            for _ in range(nbytes - 1):
                out.append(0x80 | (n & 0x3F))
                n >>= 6
            return bytes([lead | n] + out[::-1])
    raise ValueError(n)


BLOCK_CODES = {192: 1, 576: 2, 1152: 3, 2304: 4, 4608: 5, 256: 8, 512: 9, 1024: 10, 2048: 11,
               4096: 12, 8192: 13, 16384: 14, 32768: 15}


def _frame(x, frame_no, plan):
    block = len(x)
    hdr = bytearray(b"\xff\xf8")       # sync + fixed-blocksize strategy
    code = BLOCK_CODES.get(block)
    if code is None:
        code = 6 if block <= 256 else 7
    hdr.append((code << 4) | 0x0)      # sample rate from STREAMINFO
    hdr.append((0 << 4) | (4 << 1))    # mono, 16 bits per sample
    hdr += _utf8_number(frame_no)
    if code == 6:
        hdr.append(block - 1)
    elif code == 7:
        hdr += (block - 1).to_bytes(2, "big")
    hdr.append(crc8(hdr))
    w = _Bits()
    kind = plan["kind"]
    wasted = plan.get("wasted", 0)
    xs = np.asarray(x, np.int64) >> wasted
    bps = 16 - wasted
    w.put(0, 1)
    if kind == "constant":
        w.put(0, 6)
    elif kind == "verbatim":
        w.put(1, 6)
    elif kind == "fixed":
        w.put(8 | plan["order"], 6)
    else:
        w.put(32 | (plan["order"] - 1), 6)
    if wasted:
        w.put(1, 1)
        w.put(1, wasted)     # unary: wasted - 1 zeros, then a one
    else:
        w.put(0, 1)
    if kind == "constant":
        w.put(int(xs[0]), bps)
    elif kind == "verbatim":
        w.put_array(_signed_bits(xs, bps))
    elif kind == "fixed":
        o = plan["order"]
        w.put_array(_signed_bits(xs[:o], bps))
        _write_residual(w, _fixed_residual(xs, o), o, block, plan["method"], plan["porder"],
                        plan.get("escape", 0))
    else:
        o = plan["order"]
        coefs, shift, prec = plan["coefs"], plan["shift"], plan["precision"]
        w.put_array(_signed_bits(xs[:o], bps))
        w.put(prec - 1, 4)
        w.put(shift, 5)
        w.put_array(_signed_bits(coefs, prec))
        _write_residual(w, _lpc_residual(xs, coefs, shift), o, block, plan["method"],
                        plan["porder"], plan.get("escape", 0))
    body = bytes(hdr) + w.bytes()
    c = crc16(body)
    return body + bytes([c >> 8, c & 0xFF])


def _plan(x, rng, fi):
    """Subframe choice for frame fi: a rotation over the forms, LPC most of the time."""
    block = len(x)
    if np.all(x == x[0]):
        return {"kind": "constant"}
    if block < 40:
        return {"kind": "verbatim"}
    porders = [p for p in range(0, 9) if block % (1 << p) == 0 and (block >> p) > 32]
    method = int(rng.integers(0, 2))
    porder = int(rng.choice(porders)) if porders else 0
    esc = 3 if fi % 11 == 5 else 0
    sel = fi % 8
    if sel == 1:
        return {"kind": "verbatim"}
    if sel == 2:
        return {"kind": "fixed", "order": int(rng.integers(0, 5)), "method": method,
                "porder": porder, "escape": esc}
    order = int(rng.choice([1, 2, 4, 8, 12, 16, 24, 32]))
    prec = int(rng.integers(12, 16))
    q = _lpc_coefs(x, order, prec)
    if q is None or block <= order:
        return {"kind": "fixed", "order": 2, "method": method, "porder": porder, "escape": esc}
    coefs, shift = q
    return {"kind": "lpc", "order": order, "coefs": coefs, "shift": shift, "precision": prec,
            "method": method, "porder": porder, "escape": esc}


def write(samples, blocksize=4096, sample_rate=40000, seed=0, wasted_frames=()):
    """FLAC stream (bytes) of int16 mono `samples`: fixed block size (the last
    block short), the stream's sample rate field set to `sample_rate`, frames'
    subframe forms chosen by `seed`.  Frames listed in `wasted_frames` whose
    samples are all even are written with one wasted bit."""
    x = np.asarray(samples, np.int16).astype(np.int64)
    rng = np.random.default_rng(seed)
    n = len(x)
    out = bytearray(b"fLaC")
    si = bytearray()
    nfr = (n + blocksize - 1) // blocksize
    si += blocksize.to_bytes(2, "big") * 2
    si += (0).to_bytes(3, "big") * 2
    packed = (sample_rate << 44) | (0 << 41) | (15 << 36) | n
    si += packed.to_bytes(8, "big")
    si += bytes(16)                      # MD5 not computed
    out += bytes([0x80, 0, 0, 34]) + si
    for fi in range(nfr):
        xs = x[fi * blocksize:(fi + 1) * blocksize]
        plan = _plan(xs, rng, fi)
        if fi in wasted_frames and plan["kind"] not in ("constant",) and np.all(xs % 2 == 0):
            plan["wasted"] = 1
            if plan["kind"] == "lpc":
                q = _lpc_coefs(xs >> 1, plan["order"], plan["precision"])
                if q is None:
                    plan = {"kind": "verbatim", "wasted": 1}
                else:
                    plan["coefs"], plan["shift"] = q
        out += _frame(xs, fi, plan)
    return bytes(out)


