"""Colour-under chroma decode of the VHS path (test infrastructure).

Restates the managed ``exact`` backend's chroma chain at its v0.4.0 defaults
(``--compat-version v0.4.0``; no AFC, comb on, colour killer off, track-phase
detection off, burst-hsync refinement on):

* per RF block: the float32 forward-backward chroma band-pass of the RF
  (``RfBlockDecodePipeline.DecodeChromaBurstFloat32``,
  Core/Decode/RfBlockDecodePipeline.cs:308-336, 540-577) and
  ``ShiftChromaAndRemoveDcFloat32InPlace`` (Core/Decode/VhsChromaDecoder.cs:2517-2533),
  stitched like the other channels;
* per field (``TbcFieldDecodePipeline.DecodeCore``,
  Core/Decode/TbcFieldDecodePipeline.cs:1366-1490): a TBC of the chroma
  channel from line 1, the burst phase sequence of that resample
  (``AnalyzeFieldPhaseWithWorkspace``, VhsChromaDecoder.cs:574-702, with
  ``GetPhaseRotationSequenceCore`` :1904-1965 and its helpers :3927-4290),
  the burst refinement of the line locations (``RefineLineLocationsFromBurst``
  :2342-2428), then the NTSC fsc shift and the final resample of luma and
  chroma from the output first line;
* the field decode (``CompleteFieldWithPhaseCore`` :947-1251): NTSC burst
  de-emphasis (:2649-2719) and phase-compensated up-conversion (:2167-2248),
  PAL heterodyne up-conversion with NumPy slice semantics (:2009-2165), the
  float32 forward-backward final band-pass, and the automatic chroma gain with
  the 1H/2H comb to uint16 (:3480-3659).

The filters are designed by ``butter_bandpass_sos``, which restates
``IirFilterDesign.ButterworthBandPassSos`` (Core/Dsp/IirFilterDesign.cs:594-606,
1143-1212, 1381-1437) with the .NET complex helpers it calls.
"""
import math
from fractions import Fraction

import numpy as np

from . import demod, native

STARTING_LINE = 16          # VhsChromaDecoder.StartingLine (:438)
BURST_CHECK_SKIP_LINES = 16  # VhsChromaDecoder.BurstCheckSkipLines (:440)
ANALYSIS_FIRST_LINE = 1     # TbcFieldDecodePipeline.VhsChromaPhaseAnalysisFirstLine (:227)


# ---------------------------------------------------------------- filter design

def _fma(a, b, c):
    """Exactly rounded a*b+c (Math.FusedMultiplyAdd)."""
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def _cmul_numpy(a, b):
    """IirFilterDesign.NumpyComplexMultiply (:670-677)."""
    return complex(a.real * b.real - a.imag * b.imag, a.real * b.imag + a.imag * b.real)


def _cmul_simd(a, b):
    """IirFilterDesign.NumpySimdComplexMultiply (:679-690)."""
    return complex(_fma(a.real, b.real, -(a.imag * b.imag)), _fma(a.imag, b.real, a.real * b.imag))


def _cmul_net(a, b):
    """System.Numerics.Complex multiplication."""
    return complex(a.real * b.real - a.imag * b.imag, a.imag * b.real + a.real * b.imag)


def _cdiv_numpy(l, r):
    """IirFilterDesign.NumpyComplexDivide (:692-715), Smith's algorithm."""
    if abs(r.real) >= abs(r.imag):
        ratio = r.imag / r.real
        sd = 1.0 / (r.real + (r.imag * ratio))
        return complex((l.real + (l.imag * ratio)) * sd, (l.imag - (l.real * ratio)) * sd)
    ratio = r.real / r.imag
    sd = 1.0 / (r.imag + (r.real * ratio))
    return complex(((l.real * ratio) + l.imag) * sd, ((l.imag * ratio) - l.real) * sd)


def _net_hypot(a, b):
    """System.Numerics.Complex's private hypotenuse (Complex.Abs)."""
    a, b = abs(a), abs(b)
    small, large = (a, b) if a < b else (b, a)
    if small == 0.0:
        return large
    ratio = small / large
    return large * math.sqrt(1.0 + ratio * ratio)


def _net_sqrt(z):
    """System.Numerics.Complex.Sqrt (no rescaling is needed at these magnitudes)."""
    re, im = z.real, z.imag
    if im == 0.0:
        return complex(0.0, math.sqrt(-re)) if re < 0.0 else complex(math.sqrt(re), 0.0)
    if re >= 0.0:
        x = math.sqrt((_net_hypot(re, im) + re) * 0.5)
        return complex(x, im / (2.0 * x))
    y = math.sqrt((_net_hypot(re, im) - re) * 0.5)
    if im < 0.0:
        y = -y
    return complex(im / (2.0 * y), y)


def _numpy_abs(z):
    """IirFilterDesign.NumpyComplexAbs (:1564-1580)."""
    larger, smaller = abs(z.real), abs(z.imag)
    if larger < smaller:
        larger, smaller = smaller, larger
    if larger == 0.0:
        return 0.0
    ratio = smaller / larger
    return larger * math.sqrt(_fma(ratio, ratio, 1.0))


def _bandpass_zpk(order, lo, hi):
    """``DesignButterworthBandPassZpk`` (:1143-1212)."""
    fs = 2.0
    wl = 2.0 * fs * math.tan(math.pi * lo / 2.0)
    wh = 2.0 * fs * math.tan(math.pi * hi / 2.0)
    bw = wh - wl
    c = math.sqrt(wl * wh)
    proto = []
    for i, m in enumerate(range(-order + 1, order, 2)):
        ang = (math.pi * m) / (2.0 * order)       # BuildButterworthPrototypePoles (:427-436)
        proto.append(complex(-math.cos(ang), -math.sin(ang)))
    pos, neg = [], []
    for p in proto:
        sp = complex(p.real * (bw / 2.0), p.imag * (bw / 2.0))
        sq = _cmul_numpy(sp, sp)
        root = _net_sqrt(complex(sq.real - c * c, sq.imag))
        pos.append(sp + root)
        neg.append(sp - root)
    bs = 2.0 * fs
    zeros = [complex(1.0, 0.0)] * order + [complex(-1.0, 0.0)] * order
    poles, dprod = [], complex(1.0, 0.0)
    for p in pos + neg:
        den = complex(bs - p.real, -p.imag)
        poles.append(_cdiv_numpy(complex(bs + p.real, p.imag), den))
        dprod = _cmul_simd(dprod, den)
    gain = math.pow(bw, order) * _cdiv_numpy(complex(math.pow(bs, order), 0.0), dprod).real
    return zeros, poles, gain


def _nearest(values, target):
    sel, best = 0, math.inf
    for i, v in enumerate(values):
        d = _numpy_abs(v - target)
        if d < best:
            best, sel = d, i
    return sel


def _zpk_to_nearest_sos(zeros, poles, gain):
    """``ZpkToNearestSos`` (:1381-1437)."""
    rem, pairs = list(poles), []
    while rem:
        fi = next((i for i, v in enumerate(rem) if v.imag > 1e-12), 0)
        first = rem.pop(fi)
        tgt = first.conjugate()
        si, best = 0, math.inf
        for i, v in enumerate(rem):
            d = _net_hypot((v - tgt).real, (v - tgt).imag)
            if d < best:
                best, si = d, i
        second = rem.pop(si)
        pairs.append((first, second, max(_net_hypot(first.real, first.imag),
                                         _net_hypot(second.real, second.imag))))
    remz, assigned = list(zeros), []
    for first, second, radius in sorted(pairs, key=lambda t: -t[2]):
        z1 = remz.pop(_nearest(remz, first))
        z2 = remz.pop(_nearest(remz, first))
        assigned.append((first, second, z1, z2, radius))
    sos = []
    for p1, p2, z1, z2, _ in sorted(assigned, key=lambda t: t[4]):
        sos.append([1.0, -(z1 + z2).real, _cmul_net(z1, z2).real,
                    1.0, -(p1 + p2).real, _cmul_net(p1, p2).real])
    sos[0][0] *= gain
    sos[0][1] *= gain
    sos[0][2] *= gain
    return np.array(sos, np.float64)


def butter_bandpass_sos(order, lo, hi):
    """``IirFilterDesign.ButterworthBandPassSos`` for order >= 2 (cutoffs / Nyquist)."""
    return _zpk_to_nearest_sos(*_bandpass_zpk(order, lo, hi))


def default_pad_length(sos):
    """``SosFilter.DefaultPadLength`` (Core/Dsp/SosFilter.cs:540-545)."""
    zb = int(np.sum(sos[:, 2] == 0.0))
    za = int(np.sum(sos[:, 5] == 0.0))
    return 3 * (2 * len(sos) + 1 - min(zb, za))


# ---------------------------------------------------------------- parameters

class ChromaParams:
    """``TbcFieldDecodePipeline.BuildChromaFieldOptions`` (:2626-2760, v0.4.0 branch)
    and the chroma filters of ``DecodeFilterSetBuilder.BuildBasic``
    (Core/Dsp/DecodeFilterSet.cs:173-238, 563-599, 663-752)."""

    def __init__(self, fmt, fs=40e6):
        sy, rf = fmt["sys"], fmt["rf"]
        self.system = fmt["system"]
        self.ntsc = self.system == "NTSC"
        self.fs = fs
        self.fsc_mhz = sy["fsc_mhz"]
        self.cu_hz = rf["color_under_carrier"]
        self.outlen = sy["outlinelen"]
        self.out_lines = sy["frame_lines"] // 2 + 1
        self.field_samples = self.outlen * self.out_lines
        self.output_rate_hz = sy["outfreq"] * 1_000_000.0
        outus = sy["outfreq"]
        b0 = int(math.floor(sy["colorBurstUS"][0] * outus)) - 5
        b1 = int(math.ceil(sy["colorBurstUS"][1] * outus)) + 10
        self.burst_start = min(max(b0, 0), self.outlen)
        self.burst_end = min(max(b1, self.burst_start), self.outlen)
        self.burst_abs_ref = float(sy["burst_abs_ref"])
        self.rotation = list(rf["chroma_rotation"]) if rf.get("chroma_rotation") else None
        nyq = fs / 2.0
        lo = rf.get("chroma_bpf_lower") or 60_000.0
        order = rf.get("chroma_bpf_order") or 4
        self.rf_sos = butter_bandpass_sos(order, lo / nyq, rf["chroma_bpf_upper"] / nyq)
        nyq_mhz = (self.fsc_mhz * 4.0) / 2.0
        cu_mhz = self.cu_hz / 1_000_000.0
        self.final_sos = butter_bandpass_sos(4, (self.fsc_mhz - cu_mhz * 0.9) / nyq_mhz,
                                             (self.fsc_mhz + cu_mhz * 0.75) / nyq_mhz)
        chroma_offset = rf.get("chroma_offset")
        self.offset = int((5.0 if chroma_offset is None else chroma_offset) * (fs / 40_000_000.0))
        self.fsc_ratio = (self.output_rate_hz / 1_000_000.0) / self.fsc_mhz
        self._tables = None

    def tables(self):
        """Heterodyne (4 phases) and carrier tables of one field."""
        if self._tables is None:
            rate = self.fsc_mhz * 4.0
            het = [heterodyne_table(self.field_samples, self.fsc_mhz, self.cu_hz / 1e6, rate, p)
                   for p in range(4)]
            self._tables = (het,) + carrier_tables(self.field_samples, self.fsc_mhz, rate)
        return self._tables


def heterodyne_table(n, fsc_mhz, cu_mhz, rate_mhz, phase, drift=0.0):
    """One phase of ``BuildHeterodyneTable`` (VhsChromaDecoder.cs:1967-2007)."""
    return native.chroma_heterodyne(n, (fsc_mhz + cu_mhz) / rate_mhz, (math.pi / 2.0 * phase) + drift)


def carrier_tables(n, carrier_mhz, rate_mhz):
    """``BuildCarrierTables`` (VhsChromaDecoder.cs:3793-3828): (sin, cos)."""
    return native.chroma_carrier(n, carrier_mhz / rate_mhz)


# ---------------------------------------------------------------- block stage

def shift_and_remove_dc_f32(y, move):
    """``ShiftChromaAndRemoveDcFloat32InPlace`` for float32 data (:2517-2533)."""
    y = np.roll(np.asarray(y, np.float32), move)
    mean = native.mean_f32_fast(y)
    return (y - np.float32(mean)).astype(np.float32)


def chroma_block(x, cp):
    """Chroma channel of one RF block (float32 values)."""
    y = native.sosfiltfilt_f32(np.asarray(x, np.float64), cp.rf_sos, default_pad_length(cp.rf_sos))
    return shift_and_remove_dc_f32(y, cp.offset)


def chroma_stream(rf, cp, first_block=0, nblocks=None):
    """Stitched chroma channel (stream sample d is RF sample d + CUT)."""
    total = demod.block_count(len(rf))
    if nblocks is None:
        nblocks = total - first_block
    out = np.empty(nblocks * demod.STRIDE)
    for j in range(nblocks):
        b = first_block + j
        x = rf[b * demod.STRIDE: b * demod.STRIDE + demod.BLOCK].astype(np.float64)
        c = chroma_block(x, cp)
        out[j * demod.STRIDE:(j + 1) * demod.STRIDE] = c[demod.CUT:demod.CUT + demod.STRIDE]
    return out


# ---------------------------------------------------------------- phase analysis

def positive_degrees(d):
    r = math.fmod(d, 360.0)
    return r + 360.0 if r < 0.0 else r


def demod_burst(burst, line_scale, line_start, burst_start, bsin, bcos, f32):
    """``DemodBurstValue`` / ``DemodBurstFloat32`` (:1438-1629) -> dict."""
    burst = np.ascontiguousarray(burst, np.float64)
    if burst_start < 0 or burst_start + len(burst) > len(bsin) or burst_start + len(burst) > len(bcos):
        raise ValueError("burst carrier tables must cover the requested burst range")
    v = native.chroma_burst_value(burst, np.ascontiguousarray(bsin[burst_start:], np.float64),
                                  np.ascontiguousarray(bcos[burst_start:], np.float64), f32,
                                  line_scale, burst_start - line_start)
    return {"phase": v[0], "offset": v[1], "mag": v[2], "i": v[3], "q": v[4]}


def probe_burst(chroma, het, rotation, burst_start, burst_end, bsin, bcos, line_scale, line,
                line_offset, line_length, burst_filter, f32):
    """``ProbeUpconvertedBurstValue`` (:1660-1713)."""
    idx = line - line_offset
    if idx < 0 or idx * line_length + line_length > len(chroma):
        raise ValueError("chroma phase line outside the field")
    line_start = idx * line_length
    pad = burst_end - burst_start
    p0 = max(0, line_start + burst_start - pad)
    p1 = min(len(chroma), p0 + burst_end + pad)
    h = het[rotation][p0:p1].astype(np.float32)
    c = np.asarray(chroma[p0:p1], np.float64)
    if f32:
        mixed = (h * c.astype(np.float32)).astype(np.float64)
    else:
        mixed = h.astype(np.float64) * c
    filt = burst_filter(mixed) if burst_filter is not None else mixed
    fs = min(pad, len(filt))
    fe = max(fs, len(filt) - pad)
    r = demod_burst(filt[fs:fe], line_scale, line_start, p0 + pad, bsin, bcos, f32)
    r["line"] = line
    r["rot"] = rotation
    return r


def _line_scale(locs, line, input_line_length, last_line):
    if line < last_line - 1:
        return (locs[line + 1] - locs[line]) / input_line_length
    return 1.0


def _build_sequence(rotation, start_index, locs, line_offset, input_line_length, end, probe):
    """``BuildPhaseSequence`` without track-phase detection (:3927-4033)."""
    if rotation:
        idx = start_index
        track = rotation[idx]
    else:
        idx, track = 0, start_index
    seq, phase = [], 0
    for line in range(line_offset, end):
        phase = (phase + track) % 4
        seq.append(probe(line, phase, _line_scale(locs, line, input_line_length, end)))
    if rotation:
        idx = (idx + 1) % 2
    return idx, seq


def should_flip(rotation, seq, end, ntsc):
    """``ShouldFlipTrackPhase`` (:4164-4217)."""
    if not rotation:
        return False
    d = [0, 0, 0, 0]
    check_end = end - BURST_CHECK_SKIP_LINES
    for prev, cur in zip(seq, seq[1:]):
        if cur["line"] <= BURST_CHECK_SKIP_LINES or cur["line"] >= check_end:
            continue
        delta = positive_degrees(cur["phase"] - prev["phase"])
        d[int(math.floor((delta + 45.0) / 90.0)) % 4] += 1
    if ntsc:
        return d[0] < d[2]
    return (d[1] + d[3]) < (d[0] + d[2])


def summarize(next_index, seq, end, color_killer=False, prev_burst_line=0, threshold=2.5e4):
    """``SummarizePhaseSequence`` (:4219-4290)."""
    check_end = end - BURST_CHECK_SKIP_LINES
    burst_line = 0
    ei = eq = oi = oq = 0.0
    count, mag_sum = 0, 0.0
    for p in seq:
        if p["line"] <= BURST_CHECK_SKIP_LINES or p["line"] >= check_end or p["mag"] == 0.0:
            continue
        ni, nq = p["i"] / p["mag"], p["q"] / p["mag"]
        count += 1
        mag_sum += p["mag"]
        if color_killer and prev_burst_line == -1 and burst_line == 0 and p["mag"] > threshold:
            burst_line = p["line"]
        if p["line"] & 1:
            oi += ni
            oq += nq
        else:
            ei += ni
            eq += nq
    if count == 0:
        raise ValueError("no valid chroma burst samples for phase averaging")
    mag_avg = mag_sum / count
    if color_killer and mag_avg < threshold:
        burst_line = -1
    return {"next_index": next_index, "seq": seq, "burst_line": burst_line, "mag_avg": mag_avg,
            "avg": positive_degrees(math.atan2(eq + oq, ei + oi) * 180.0 / math.pi),
            "even": positive_degrees(math.atan2(eq, ei) * 180.0 / math.pi),
            "odd": positive_degrees(math.atan2(oq, oi) * 180.0 / math.pi)}


def phase_rotation_sequence(rotation, rot_index, locs, line_offset, lines_out, input_line_length, probe,
                            ntsc, color_killer=False, prev_burst_line=0):
    """``GetPhaseRotationSequenceCore`` (:1904-1965) without track-phase detection;
    ``probe(line, rotation, line_scale)`` returns a burst dict."""
    end = lines_out + line_offset
    if len(locs) <= end:
        raise ValueError("line locations must include one entry past the last chroma line")
    nxt, seq = _build_sequence(rotation, rot_index, locs, line_offset, input_line_length, end, probe)
    if should_flip(rotation, seq, end, ntsc):
        nxt, seq = _build_sequence(rotation, nxt, locs, line_offset, input_line_length, end, probe)
    return summarize(nxt, seq, end, color_killer, prev_burst_line)


def analyze_field_phase(chroma, cp, locs, input_line_length, rot_index=0, line_offset=ANALYSIS_FIRST_LINE,
                        f32=True, burst_filter=None, prev_burst_line=0, sos=None):
    """``AnalyzeFieldPhaseWithWorkspace`` (:574-702) + ``GetPhaseRotationSequenceCore``."""
    het, bsin, bcos = cp.tables()
    sos = cp.final_sos if sos is None else sos
    if burst_filter is None:
        pad = default_pad_length(sos)
        if f32:
            def burst_filter(v):
                return native.sosfiltfilt_f32(v, sos, pad).astype(np.float64)
        else:
            def burst_filter(v):
                return native.sosfiltfilt_f64(v, sos, pad)

    def probe(line, rot, scale):
        return probe_burst(chroma, het, rot, cp.burst_start, cp.burst_end, bsin, bcos, scale, line,
                           line_offset, cp.outlen, burst_filter, f32)

    return phase_rotation_sequence(cp.rotation, rot_index, locs, line_offset, cp.out_lines, input_line_length,
                                   probe, cp.ntsc, prev_burst_line=prev_burst_line)


def refine_from_burst(locs, outlen, fsc_ratio, phase, ntsc):
    """``RefineLineLocationsFromBurst``, v0.4.0 form (:2342-2428)."""
    out = np.array(locs, np.float64)
    if phase["burst_line"] == -1:
        return out
    seq = phase["seq"]
    for p in seq[max(9, phase["burst_line"]):]:
        line = p["line"]
        if line < 0 or line + 1 >= len(out):
            continue
        target = phase["avg"] if ntsc else (phase["odd"] if line & 1 else phase["even"])
        delta = positive_degrees(target - p["phase"] + p["offset"] + 180.0) - 180.0
        scale = (out[line + 1] - out[line]) / outlen
        out[line] += (delta / 360.0) * fsc_ratio * scale
    return out


# ---------------------------------------------------------------- field decode

def _numpy_slice(n, line_offset, line_length, line):
    def norm(i):
        if i < 0:
            i += n
        return min(max(i, 0), n)
    s = (line - line_offset) * line_length
    a, b = norm(s), norm(s + line_length)
    return (a, b) if b > a else (a, a)


def upconvert_pal(chroma, line_offset, line_length, seq, het):
    """``UpconvertChroma`` (:2009-2045) with NumPy slice semantics."""
    out = np.zeros(len(chroma))
    for p in seq:
        a, b = _numpy_slice(len(chroma), line_offset, line_length, p["line"])
        h = het[p["rot"]]
        out[a:b] = (np.asarray(chroma[a:b], np.float64) * h[a:b]).astype(np.float32)
    return out


def burst_deemphasis(chroma, line_offset, lines, line_length, burst_end, after=5):
    """``ApplyBurstDeemphasisCore`` (:2696-2719)."""
    out = np.array(chroma, np.float64)
    first = burst_end + after
    if first >= line_length:
        return out
    for line in range(line_offset, lines + line_offset):
        s = (line - line_offset) * line_length
        out[s + first:s + line_length] *= 2.0
    return out


def ntsc_field_phase_target(first_field, field_number):
    """``NtscFieldPhaseTarget`` (:3915-3925) -> (phase id, degrees)."""
    second = ((field_number // 2) & 1) == 1
    return {(True, False): (1, -33.0), (False, True): (2, 147.0),
            (True, True): (3, 147.0), (False, False): (4, -33.0)}[(bool(first_field), second)]


def decode_field_chroma(chroma, cp, phase, first_field, field_number, line_offset):
    """``CompleteFieldWithPhaseCore`` (:947-1251), v0.4.0 path -> uint16 field."""
    chroma = np.asarray(chroma, np.float64)
    if phase["burst_line"] == -1:
        return np.full(len(chroma), 32767, np.uint16)
    seq = phase["seq"]
    if cp.ntsc:
        chroma = burst_deemphasis(chroma, line_offset, cp.out_lines, cp.outlen, cp.burst_end)
        _, target = ntsc_field_phase_target(first_field, field_number)
        up = native.chroma_upconvert_ntsc(chroma, line_offset, cp.outlen,
                                          [p["line"] for p in seq], [p["rot"] for p in seq],
                                          [p["phase"] for p in seq], cp.cu_hz, cp.fsc_mhz, target, target)
    else:
        het = cp.tables()[0]
        up = upconvert_pal(chroma, line_offset, cp.outlen, seq, het)
    up = native.sosfiltfilt_f32(up, cp.final_sos, default_pad_length(cp.final_sos)).astype(np.float64)
    return native.chroma_agc_comb_u16(up, cp.out_lines, cp.outlen, cp.burst_start, cp.burst_end,
                                      cp.burst_abs_ref, phase["burst_line"], 1 if cp.ntsc else 2,
                                      True, True)
