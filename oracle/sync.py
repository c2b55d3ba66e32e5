"""Field-level sync analysis for the VHS path (test infrastructure).

Restates, for the standard (non-fallback) VHS branch:

* ``PulseDetection.FindPulses`` state machine (Core/Dsp/PulseDetection.cs:45-222) -- via oracle_c.c
* ``TbcFieldDecodePipeline.FindRawPulses`` VHS limits (Core/Decode/TbcFieldDecodePipeline.cs:2375-2385)
* ``SyncAnalyzer.EstimateTiming / ClassifyPulses / RefinePulses / TryReadVBlank /
  ComputeMeanLineLength / BuildUpstreamLineLocations`` (Core/Dsp/SyncAnalysis.cs:84-640)
* ``VBlankSyncResolver.FindFirstGroup / EstimateLine0FromGroups / FirstHSyncLine /
  NextFieldLocation`` (Core/Dsp/VBlankSyncResolver.cs:49-115, 228-315, 447-497, 560-718)
* ``FieldParityDetector.ResolveCadence`` + boundary consensus (Core/Dsp/FieldParityDetector.cs:16-250)
* ``RefineLineLocationsFromHSync`` left/right edge refinement
  (Core/Decode/TbcFieldDecodePipeline.cs:4570-4679, 4807-5050)
* ``PulseDetection.CalculateZeroCrossing`` (Core/Dsp/PulseDetection.cs:17-40, 224-275)

The line-0 choice is the VBlank-group consensus (combined estimate when the
first and next VBlank agree, else the single-group estimate chosen as
``SelectSingleVBlankEstimate`` does).  The previous-field three-way consensus,
the transition-based fallback, fallback-VSync and serration level detection
of the reference are not part of this restatement.
"""
import math

import numpy as np

from . import native

HSYNC, EQ, VSYNC, EQ2 = 0, 1, 2, 3


def round_away(x):
    return math.floor(x + 0.5) if x >= 0 else -math.floor(-x + 0.5)


def np_median(values):
    return float(np.median(np.asarray(values, np.float64)))


class SyncParams:
    """``SyncAnalyzer.FromParameters`` (Core/Dsp/SyncAnalysis.cs:84-111) for VHS tolerances."""

    def __init__(self, fmt, fs, hsync_tol_us=0.7, eq_tol_us=0.9):
        s = fmt["sys"]
        self.system = fmt["system"]
        self.fs = fs
        self.mhz = fs / 1e6
        self.nominal = float(round(s["line_period"] * self.mhz))  # round-half-even == Python round
        self.line_period_us = self.nominal / self.mhz
        self.hsync_us = s["hsyncPulseUS"]
        self.eq_us = s["eqPulseUS"]
        self.vsync_us = s["vsyncPulseUS"]
        self.num_pulses = int(s["numPulses"])
        self.hsync_tol = hsync_tol_us
        self.eq_tol = eq_tol_us
        self.ire0 = s["ire0"]
        self.hz_ire = s["hz_ire"]
        self.vsync_ire = s["vsync_ire"]
        fl = s["frame_lines"]
        self.output_lines = fl // 2 + 1
        self.outlinelen = int(s["outlinelen"])
        self.fsc_mhz = s["fsc_mhz"]
        self.outfreq = s["outfreq"]

    def usec(self, us):
        return us * self.mhz

    def ire_to_hz(self, ire):
        return self.ire0 + self.hz_ire * ire

    def field_lines(self):
        """``FieldLinesForParityDetection`` (TbcFieldDecodePipeline.cs:728-733)."""
        n = self.output_lines
        return [n, n - 1] if self.system == "NTSC" else [n - 1, n]


def find_raw_pulses(sp, ref, threshold):
    lo = max(0, math.ceil(sp.usec(sp.eq_us) / 8.0))
    hi = max(1, int(sp.nominal * 5.0))
    return native.find_pulses(ref, threshold, lo, hi)


def in_range(v, lo, hi):
    return lo <= v <= hi


def estimate_timing(sp, raw, vhs_empty_median_units=True):
    """``SyncAnalyzer.EstimateTiming`` (SyncAnalysis.cs:131-167).

    The VHS field path passes ``preserveVhsEmptyHSyncMedianUnits``: with no
    hsync-length candidate the median falls back to the pulse width in
    microseconds, not samples.  ``vhs_empty_median_units=False`` is the
    analyser's default (samples)."""
    lo = sp.usec(sp.hsync_us - 1.75)
    hi = sp.usec(sp.hsync_us + 2.0)
    lens = [ln for (_, ln) in raw if in_range(ln, lo, hi)]
    if lens:
        med = np_median(lens)
    else:
        med = sp.hsync_us if vhs_empty_median_units else sp.usec(sp.hsync_us)
    off = med - sp.usec(sp.hsync_us)
    return {
        "hsync": (med - sp.usec(sp.hsync_tol), med + sp.usec(sp.hsync_tol)),
        "eq": (sp.usec(sp.eq_us - sp.eq_tol) + off, sp.usec(sp.eq_us + sp.eq_tol) + off),
        "vsync": (sp.usec(sp.vsync_us * 0.5) + off, sp.usec(sp.vsync_us + 1.0) + off),
    }


def _classify(ln, timing):
    if in_range(ln, *timing["hsync"]):
        return HSYNC
    if in_range(ln, *timing["eq"]):
        return EQ
    if in_range(ln, *timing["vsync"]):
        return VSYNC
    return None


def _quality(sp, prev, kind, start):
    pk = prev[0]
    if pk != HSYNC and kind != HSYNC:
        rng = (0.4, 0.6)
    elif pk == HSYNC and kind == HSYNC:
        rng = (0.9, 1.1)
    else:
        rng = (0.4, 1.1)
    return in_range((start - prev[1]) / sp.nominal, *rng)


def classify_pulses(sp, raw, timing):
    """``SyncAnalyzer.ClassifyPulses`` (SyncAnalysis.cs:175-197). Items: (kind, start, length, in_order)."""
    out = []
    for (s, ln) in raw:
        k = _classify(ln, timing)
        if k is None:
            continue
        ok = bool(out) and _quality(sp, out[-1], k, s)
        out.append((k, s, ln, ok))
    return out


def _rescue(sp, pulse, ref, step_hz):
    s, ln = pulse
    start = min(max(s, 0), len(ref))
    end = min(max(s + ln, start), len(ref))
    if start >= end:
        return None
    data = ref[start:end]
    thr = data[0] - step_hz
    cands = native.find_pulses(data, thr, max(0, math.ceil(sp.usec(sp.eq_us) / 8.0)),
                               max(1, int(sp.nominal * 5.0)))
    if cands:
        return (start + cands[0][0], cands[0][1])
    return None


def _read_vblank(sp, pulses, timing, start, end, dest):
    valid = []
    state = None
    state_end = 0.0
    state_len = None
    for idx in range(max(0, start), end):
        s, ln = pulses[idx]
        raw_kind = _classify(ln, timing)
        if raw_kind is None:
            continue
        acc = None
        done = False
        if state is None and raw_kind == HSYNC:
            acc = HSYNC
        elif state == HSYNC:
            if raw_kind == HSYNC:
                acc = HSYNC
            elif raw_kind == EQ:
                acc = EQ
                state_len = sp.num_pulses / 2.0
            elif raw_kind == VSYNC:
                acc = VSYNC
        elif state == EQ:
            if raw_kind == EQ:
                acc = EQ
            elif raw_kind == VSYNC:
                acc = VSYNC
                state_len = sp.num_pulses / 2.0
            elif raw_kind == HSYNC:
                acc = HSYNC
        elif state == VSYNC:
            if raw_kind == EQ:
                acc = EQ2
                state_len = sp.num_pulses / 2.0
            elif raw_kind == VSYNC:
                acc = VSYNC
            elif raw_kind == HSYNC and s > state_end:
                acc = HSYNC
        elif state == EQ2:
            if raw_kind == EQ:
                acc = EQ2
            elif raw_kind == HSYNC:
                acc = HSYNC
                done = True
        if acc is None:
            continue
        if acc != state:
            if s < state_end:
                acc = None
            elif state_len is not None:
                state_end = s + (state_len - 0.1) * sp.nominal
                state_len = None
        if acc is not None:
            ok = bool(valid) and _quality(sp, valid[-1], acc, s)
            valid.append((acc, s, ln, ok))
            state = acc
        if done:
            dest.extend(valid[2:])
            return len(valid)
    return 0


def refine_pulses(sp, raw, timing, ref, rescue_step_hz):
    """``SyncAnalyzer.RefinePulses`` with long-hsync rescue (SyncAnalysis.cs:259-438)."""
    work = list(raw)
    dest = []
    i = 0
    hmax = timing["hsync"][1]
    while i < len(work):
        s, ln = work[i]
        if in_range(ln, *timing["hsync"]):
            ok = bool(dest) and _quality(sp, dest[-1], HSYNC, s)
            dest.append((HSYNC, s, ln, ok))
            i += 1
            continue
        if ref is not None and rescue_step_hz > 0.0 and in_range(ln, hmax, hmax * 3.0):
            r = _rescue(sp, (s, ln), ref, rescue_step_hz)
            if r is not None and r != (s, ln):
                work[i] = r
                continue
            i += 1
            continue
        can = i > 2 and in_range(ln, *timing["eq"]) and bool(dest) and dest[-1][0] == HSYNC
        if not can:
            i += 1
            continue
        cnt = _read_vblank(sp, work, timing, i - 2, min(len(work), i + 24), dest)
        if cnt == 0:
            i += 1
            continue
        i += max(1, cnt - 2)
    return dest, work


def mean_line_length(sp, pulses):
    """``SyncAnalyzer.ComputeMeanLineLength`` (SyncAnalysis.cs:490-538)."""
    run_start, run_len, cur_start, cur_len = -1, -1, -1, 0
    for i, p in enumerate(pulses):
        if p[0] != HSYNC:
            if cur_start >= 0 and cur_len > run_len:
                run_start, run_len = cur_start, cur_len
            cur_start, cur_len = -1, 0
        elif cur_start < 0:
            cur_start, cur_len = i, 0
        else:
            cur_len += 1
    if cur_start >= 0 and cur_len > run_len:
        run_start, run_len = cur_start, cur_len
    lens = []
    for i in range(run_start + 1, run_start + run_len):
        ll = pulses[i][1] - pulses[i - 1][1]
        if in_range(ll / sp.nominal, 0.95, 1.05):
            lens.append(float(ll))
    if not lens:
        return sp.nominal
    tot = 0.0
    for v in lens:
        tot += v
    return tot / len(lens)


def find_first_group(pulses, min_eq1=None, blank_threshold=9):
    """``VBlankSyncResolver.FindFirstGroup`` (VBlankSyncResolver.cs:49-115)."""
    n = len(pulses)
    start = 1
    while start < n:
        prev, cur = pulses[start - 1], pulses[start]
        if prev[0] != HSYNC or cur[0] == HSYNC or not cur[3] or (min_eq1 is not None and cur[1] <= min_eq1):
            start += 1
            continue
        end = start
        while end < n and pulses[end][0] != HSYNC:
            end += 1
        if end >= n or not pulses[end][3]:
            start = max(start, end - 1) + 1
            continue
        if (end - 1 - start) <= blank_threshold:
            start = max(start, end - 1) + 1
            continue
        first_v = next((i for i in range(start, end) if pulses[i][0] == VSYNC), -1)
        first_eq_after = -1
        if first_v >= 0:
            first_eq_after = next((i for i in range(first_v + 1, min(end, n))
                                   if pulses[i][0] in (EQ, EQ2) and pulses[i][3]), -1)
        if first_v < 0 or first_eq_after < 0:
            start = max(start, end - 1) + 1
            continue
        vstart = pulses[first_v][1] if (first_v > start and pulses[first_v - 1][0] in (EQ, EQ2)
                                        and pulses[first_v][3]) else None
        return {"prev_hsync": prev[1], "eq1": cur[1], "vsync": vstart,
                "eq2": pulses[first_eq_after][1], "eq2_end": pulses[end - 1][1],
                "next_hsync": pulses[end][1]}
    return None


def _boundaries(system, first_field):
    return {("NTSC", True): (1.0, 0.5, 0.5, 1.0), ("NTSC", False): (0.5, 1.0, 1.0, 0.5),
            ("PAL", True): (0.5, 0.5, 1.0, 1.0), ("PAL", False): (1.0, 1.0, 0.5, 0.5)}[(system, first_field)]


def _markers(group, eq1_line, section):
    v_line = eq1_line + section
    eq2_line = v_line + section
    eq2_end_line = eq2_line + section - 0.5
    m = [(group["eq1"], eq1_line)]
    if group["vsync"] is not None:
        m.append((group["vsync"], v_line))
    m.append((group["eq2"], eq2_line))
    m.append((group["eq2_end"], eq2_end_line))
    return m


def _acc_pair(a, b, mll, fh_line):
    actual = (a[0] - b[0]) / mll
    expected = a[1] - b[1]
    if actual <= expected - 0.5 or actual >= expected + 0.5:
        return (0.0, 0.0, 0)
    return (b[0] + mll * (fh_line - b[1]), actual - expected, 1)


def _acc_add(x, y):
    return (x[0] + y[0], x[1] + y[1], x[2] + y[2])


def _acc_within(ms, mll, fh_line):
    acc = (0.0, 0.0, 0)
    for i in range(len(ms)):
        for j in range(i + 1, len(ms)):
            acc = _acc_add(acc, _acc_pair(ms[i], ms[j], mll, fh_line))
    return acc


def _finalize(pulses, acc, mll, fh_line, field_lines):
    if acc[2] == 0:
        return None
    fh = float(round_away((acc[0] + acc[1]) / acc[2]))
    unaligned = fh
    off, cnt = 0.0, 0
    for p in pulses:
        if p[0] != HSYNC or not p[3]:
            continue
        line = ((p[1] - fh) / mll) + fh_line
        rl = round_away(line)
        if rl > field_lines:
            break
        if rl >= fh_line:
            off += fh + mll * (rl - fh_line) - p[1]
            cnt += 1
    if cnt > 0:
        fh -= off / cnt
    return {"line0": fh - mll * fh_line, "first_hsync": fh, "first_hsync_line": fh_line,
            "count": acc[2], "unaligned": unaligned}


def estimate_line0_from_groups(sp, pulses, first, last, mll, first_field, field_lines):
    """``VBlankSyncResolver.EstimateLine0FromGroups`` (VBlankSyncResolver.cs:228-315)."""
    b = _boundaries(sp.system, first_field)
    section = sp.num_pulses / 2.0
    fm = _markers(first, b[0], section)
    fh_line = fm[-1][1] + b[1]
    facc = _acc_within(fm, mll, fh_line)
    fe = _finalize(pulses, facc, mll, fh_line, field_lines)
    if last is None:
        return fe, None, None
    lm = _markers(last, field_lines + b[2], section)
    lacc = _acc_within(lm, mll, fh_line)
    le = _finalize(pulses, lacc, mll, fh_line, field_lines)
    comb = None
    if facc[2] > 0 and lacc[2] > 0:
        f_raw = facc[0] / facc[2]
        l_raw = lacc[0] / lacc[2]
        if abs(f_raw - l_raw) < 0.5 * mll:
            cross = (0.0, 0.0, 0)
            for a in fm:
                for c in lm:
                    cross = _acc_add(cross, _acc_pair(a, c, mll, fh_line))
            comb = _finalize(pulses, _acc_add(_acc_add(facc, lacc), cross), mll, fh_line, field_lines)
    return fe, le, comb


def first_hsync_line(sp, first_field):
    b = _boundaries(sp.system, first_field)
    return b[0] + (sp.num_pulses / 2.0) * 3.0 - 0.5 + b[1]


def next_field_location(sp, first_field, field_lines, mll, first_hsync):
    b = _boundaries(sp.system, first_field)
    return first_hsync + mll * ((field_lines + b[2]) - first_hsync_line(sp, first_field))


def _round_half_line(v):
    hr = round_away(v / 0.5) * 0.5
    return round_away(hr * 10.0) / 10.0


def boundary_confidence(sp, pulses, mll):
    """``FieldParityDetector.MeasureVBlankBoundaryConsensus`` (FieldParityDetector.cs:147-250)."""
    fl = sp.field_lines()
    if len(fl) < 2 or not pulses:
        return (0, 0, 0, 0)
    lens = [-1.0] * 4
    group = 0
    last = -1
    second_boundary = pulses[0][1] + fl[0] * mll
    for i, cur in enumerate(pulses):
        if last >= 0 and cur[3]:
            prev = pulses[last]
            if group == 0 and cur[1] > second_boundary:
                group = 2
            if prev[0] == HSYNC and cur[0] != HSYNC:
                lens[group] = _round_half_line((cur[1] - prev[1]) / mll)
            elif prev[0] != HSYNC and cur[0] == HSYNC:
                lens[group + 1] = _round_half_line((cur[1] - prev[1]) / mll)
        last = i
    if sp.system == "NTSC":
        first_l, second_l = [1.0, 0.5, 0.5, 1.0], [0.5, 1.0, 1.0, 0.5]
    else:
        first_l, second_l = [0.5, 0.5, 1.0, 1.0], [1.0, 1.0, 0.5, 0.5]
    consensus = detected = 0
    for i, ln in enumerate(lens):
        if ln < 0.0:
            continue
        if abs(ln - first_l[i]) < 1e-9:
            consensus += 1
            detected += 1
        elif abs(ln - second_l[i]) < 1e-9:
            detected += 1
    if detected == 0:
        return (0, 0, 0, 0)
    w = detected / 4.0
    fc = int(round_away((consensus / detected) * w * 100.0))
    sc = int(round_away(((detected - consensus) / detected) * w * 100.0))
    return (consensus, detected, fc, sc)


def resolve_cadence(sp, pulses, mll, previous_first, min_conf, has_previous_hsync):
    """``FieldParityDetector.ResolveCadence`` without the fallback-VSync inputs (FieldParityDetector.cs:16-93)."""
    cons, det, fc, sc = boundary_confidence(sp, pulses, mll)
    if previous_first is not None:
        first = not previous_first
    else:
        first = det == 0 or round_away(cons / det) == 1.0
    eff = min_conf
    if det > 0 and not has_previous_hsync and eff > 50:
        eff = 50
    if fc >= eff and fc > sc:
        first = True
    elif sc >= eff and fc < sc:
        first = False
    return first


def build_upstream_line_locations(pulses, ref_pulse, ref_line, mll, processed, prefer_earlier=False):
    """``SyncAnalyzer.BuildUpstreamLineLocations`` (SyncAnalysis.cs:585-660).

    ``prefer_earlier`` is ``preferEarlierPulseOnEqualDistance``, which only the
    PAL CVBS line-0 anchor sets (TbcFieldDecodePipeline.cs:1286-1294); VHS
    leaves it off."""
    locs_p = sorted(float(p[1]) for p in pulses)
    out = [0.0] * processed
    cur = 0
    maxd = mll / 1.5
    for line in range(processed):
        expected = ref_pulse + mll * (line - ref_line)
        out[line] = expected
        if cur >= len(locs_p):
            continue
        cd = abs(locs_p[cur] - expected)
        smallest = maxd
        sel = -1.0
        si = cur
        while si < len(locs_p) - 1:
            if cd <= smallest:
                smallest = cd
                cur = si
                sel = locs_p[si]
            nd = abs(locs_p[si + 1] - expected)
            if nd > cd or (prefer_earlier and nd == cd):
                break
            cd = nd
            si += 1
        if sel >= 0.0:
            out[line] = sel
            cur += 1
    return np.array(out), np.zeros(processed, bool)


def zero_crossing(data, start, target, edge=0, count=16):
    """``PulseDetection.CalculateZeroCrossing`` forward form (PulseDetection.cs:17-40, 224-275)."""
    if edge == 0:
        edge = 1 if data[start] < target else -1
    end = min(len(data), start + count + 1)
    seg = data[start:end]
    loc = None
    if edge == 1:
        for i in range(1, len(seg)):
            if seg[i - 1] < target and seg[i] >= target:
                loc = i
                break
    else:
        for i in range(1, len(seg)):
            if seg[i - 1] > target and seg[i] <= target:
                loc = i
                break
    if loc is None:
        return None
    x = start + loc
    a = data[x - 1] - target
    b = data[x] - target
    y = -a / (-a + b) if (b - a) != 0.0 else 0.0
    return x - 1 + y


def _area_ok(ref, crossing, one_us, end_us, min_ire, max_ire, sp):
    s = min(max(int(round_away(crossing - 0.75 * one_us)), 0), len(ref))
    e = min(max(int(round_away(crossing + end_us * one_us)), s), len(ref))
    if e <= s:
        return False
    seg = ref[s:e]
    return seg.min() >= sp.ire_to_hz(min_ire) and seg.max() <= sp.ire_to_hz(max_ire)


def _mean_range(ref, start, end):
    s = min(max(int(round_away(start)), 0), len(ref))
    e = min(max(int(round_away(end)), s), len(ref))
    if e <= s:
        return None
    tot = 0.0
    for v in ref[s:e]:
        tot += float(v)
    return tot / (e - s)


def _is_vsync_line(sp, line):
    return (3 <= line <= 6) or (sp.system == "PAL" and 1 <= line <= 2)


def refine_hsync(sp, ref, locs, filled, threshold):
    """``RefineLineLocationsFromHSync`` VHS branch with right-edge refinement (TbcFieldDecodePipeline.cs:4570-4679)."""
    one_us = max(1, int(sp.mhz))
    normal = max(1, int(sp.usec(sp.hsync_us)))
    search = max(1, one_us * 2)
    refined = np.array(locs, np.float64)
    fill = np.array(filled, bool)
    orig_filled = np.array(filled, bool)
    prev_porch = -1.0
    n = len(ref)
    for line in range(len(refined)):
        if _is_vsync_line(sp, line):
            fill[line] = True
            continue
        if not math.isfinite(refined[line]):
            continue
        ss = int(round_away(refined[line] - one_us))
        if ss < 0 or ss >= n - 1:
            continue
        crossing = zero_crossing(ref, ss, threshold, 0, min(search, n - ss - 1))
        original = refined[line]
        right_ref = original
        if crossing is not None and not fill[line]:
            ok, loc, porch, preserve = _refine_left(sp, ref, ss, crossing, one_us, prev_porch)
            if ok:
                refined[line] = loc
                right_ref = loc
                fill[line] = orig_filled[line]
                if porch > 0.0:
                    prev_porch = porch
            else:
                fill[line] = True
                refined[line] = original
                if preserve:
                    right_ref = loc
        else:
            fill[line] = True
            refined[line] = original
        ok, loc, porch = _refine_right(sp, ref, ss, threshold, normal, one_us, right_ref)
        if ok:
            refined[line] = loc
            fill[line] = False
            if porch > 0.0:
                prev_porch = porch
    return refined, fill


def _refine_left(sp, ref, ss, crossing, one_us, prev_porch):
    if not _area_ok(ref, crossing, one_us, 3.5, -65.0, 110.0, sp):
        return False, crossing, 0.0, False
    sync = _mean_range(ref, crossing + one_us, crossing + 2.5 * one_us)
    if sync is None:
        return False, crossing, 0.0, False
    if prev_porch > 0.0:
        porch = prev_porch
    else:
        porch = _mean_range(ref, crossing - one_us, crossing - 0.5 * one_us)
        if porch is None:
            return False, crossing, 0.0, True
    n = len(ref)
    mid = (porch + sync) / 2.0
    rc = zero_crossing(ref, ss, mid, 0, min(400, n - ss - 1))
    if rc is None or abs(rc - crossing) >= one_us / 2.0:
        if prev_porch <= 0.0:
            return False, crossing, porch, True
        rc = zero_crossing(ref, ss, (prev_porch + sync) / 2.0, 0, min(400, n - ss - 1))
        if rc is None or abs(rc - crossing) >= one_us / 2.0:
            return False, crossing, porch, True
        porch = prev_porch
    return True, rc, porch, True


def _refine_right(sp, ref, left_ss, threshold, normal, one_us, reference):
    n = len(ref)
    rs = left_ss + normal - one_us
    if rs < 0 or rs >= n - 1:
        return False, 0.0, 0.0
    if ref[rs] > threshold:
        return False, 0.0, 0.0
    rc = zero_crossing(ref, rs, threshold, 1, min(max(1, normal * 2), n - rs - 1))
    if rc is None:
        return False, 0.0, 0.0
    derived = rc - normal
    if not _area_ok(ref, derived, one_us, 8.0, -65.0, 30.0, sp):
        return False, 0.0, 0.0
    sync = _mean_range(ref, derived + one_us, derived + 2.5 * one_us)
    porch = _mean_range(ref, derived + normal + one_us, derived + normal + 2.0 * one_us)
    if sync is None or porch is None:
        return False, 0.0, 0.0
    mid = (porch + sync) / 2.0
    rr = zero_crossing(ref, rs, mid, 0, min(400, n - rs - 1))
    if rr is None or abs(rr - rc) >= one_us / 2.0:
        return False, 0.0, 0.0
    mhz32 = float(np.float32(sp.mhz))
    cand = rc - normal + 2.25 * (mhz32 / 40.0)
    if abs(cand - reference) >= one_us * 2.0:
        return False, 0.0, 0.0
    return True, cand, porch
