"""FLAC reader for 16-bit mono RF captures (test infrastructure: the checker).

Real captures (``.ldf``) are FLAC streams of 16-bit mono RF samples.  The
reference indexes their frames itself (Core/Rf/RawFlacFrameIndex.cs,
Core/Rf/RawFlacStreamInfo.cs) and decodes the samples through libsndfile or
ffmpeg (Core/Rf/LibsndfilePcm16SampleLoader.cs, Core/Rf/FfmpegPcm16SampleLoader.cs),
neither of which is present here.  This module restates the decoding rules of
the published format (IETF RFC 9639, "Free Lossless Audio Codec"):

* ``decode`` reads a stream bit by bit (constant, verbatim, fixed and LPC
  subframes, Rice and Rice2 residuals with escapes, wasted bits) and checks
  each frame's CRC-8 and CRC-16;
* ``stream_info`` parses and validates the STREAMINFO block the way the
  reference's tests expect (LibsndfilePcm16SampleLoaderTests.cs:1038-1110).

FLAC is lossless: the tests check that the device decoder returns the samples
a stream was written from, and that this reader agrees.
"""
import numpy as np

FIXED_COEFS = {0: [], 1: [1], 2: [2, -1], 3: [3, -3, 1], 4: [4, -6, 4, -1]}

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


# ---------------------------------------------------------------- reader

class FlacError(Exception):
    pass


def stream_info(data):
    """STREAMINFO fields of a stream, validated as the reference's loader tests require:
    the "fLaC" marker, a first metadata block of type 0 and length 34."""
    if len(data) < 8 + 34 or data[:4] != b"fLaC":
        raise FlacError("not a FLAC stream")
    if (data[4] & 0x7F) != 0 or int.from_bytes(data[5:8], "big") != 34:
        raise FlacError("first metadata block is not a 34-byte STREAMINFO")
    si = data[8:42]
    packed = int.from_bytes(si[10:18], "big")
    return {"min_block": int.from_bytes(si[0:2], "big"), "max_block": int.from_bytes(si[2:4], "big"),
            "sample_rate": packed >> 44, "channels": ((packed >> 41) & 7) + 1,
            "bits_per_sample": ((packed >> 36) & 31) + 1, "total_samples": packed & ((1 << 36) - 1)}


class _Reader:
    def __init__(self, data, pos):
        self.d = data
        self.bit = pos * 8

    def get(self, n):
        v = 0
        for _ in range(n):
            byte = self.d[self.bit >> 3]
            v = (v << 1) | ((byte >> (7 - (self.bit & 7))) & 1)
            self.bit += 1
        return v

    def sget(self, n):
        v = self.get(n)
        return v - (1 << n) if n and v >> (n - 1) else v

    def unary(self):
        q = 0
        while self.get(1) == 0:
            q += 1
        return q


def _residual(r, block, order):
    method = r.get(2)
    if method > 1:
        raise FlacError("reserved residual coding method")
    pbits = 4 if method == 0 else 5
    porder = r.get(4)
    out = []
    for p in range(1 << porder):
        n = (block >> porder) - (order if p == 0 else 0)
        k = r.get(pbits)
        if k == (1 << pbits) - 1:
            width = r.get(5)
            out += [r.sget(width) if width else 0 for _ in range(n)]
        else:
            for _ in range(n):
                u = (r.unary() << k) | r.get(k)
                out.append((u >> 1) ^ -(u & 1))
    return out


def decode(data):
    """int16 samples of a mono 16-bit stream (reference decoder, one bit at a time)."""
    info = stream_info(data)
    pos = 4
    while True:
        last = data[pos] & 0x80
        ln = int.from_bytes(data[pos + 1:pos + 4], "big")
        pos += 4 + ln
        if last:
            break
    samples = []
    while pos < len(data):
        r = _Reader(data, pos)
        if r.get(15) != 0x7FFC:
            raise FlacError("lost frame sync")
        r.get(1)
        bcode, _srate, _chan, _ssize, _ = r.get(4), r.get(4), r.get(4), r.get(3), r.get(1)
        b0 = r.get(8)
        extra = 0
        mask = 0x80
        while b0 & mask:
            extra += 1
            mask >>= 1
        extra = max(0, extra - 1)
        r.get(8 * extra)
        if bcode == 6:
            block = r.get(8) + 1
        elif bcode == 7:
            block = r.get(16) + 1
        elif bcode == 1:
            block = 192
        elif 2 <= bcode <= 5:
            block = 576 << (bcode - 2)
        else:
            block = 256 << (bcode - 8)
        hdr_end = r.bit >> 3
        if r.get(8) != crc8(data[pos:hdr_end]):
            raise FlacError("frame header CRC-8")
        bps = info["bits_per_sample"]
        r.get(1)
        t = r.get(6)
        wasted = 0
        if r.get(1):
            wasted = r.unary() + 1
        b = bps - wasted
        if t == 0:
            x = [r.sget(b)] * block
        elif t == 1:
            x = [r.sget(b) for _ in range(block)]
        elif 8 <= t <= 12:
            o = t - 8
            x = [r.sget(b) for _ in range(o)]
            res = _residual(r, block, o)
            c = FIXED_COEFS[o]
            for e in res:
                x.append(e + sum(c[j] * x[-1 - j] for j in range(o)))
        elif t >= 32:
            o = t - 31
            x = [r.sget(b) for _ in range(o)]
            prec = r.get(4) + 1
            shift = r.sget(5)
            coefs = [r.sget(prec) for _ in range(o)]
            res = _residual(r, block, o)
            for e in res:
                acc = sum(coefs[j] * x[-1 - j] for j in range(o))
                x.append(e + (acc >> shift))
        else:
            raise FlacError("reserved subframe type")
        x = [v << wasted for v in x]
        if r.bit & 7:
            r.get(8 - (r.bit & 7))
        end = r.bit >> 3
        c16 = int.from_bytes(data[end:end + 2], "big")
        if c16 != crc16(data[pos:end]):
            raise FlacError("frame CRC-16")
        pos = end + 2
        samples += x
    return np.array(samples, np.int64).astype(np.int16)
