"""Field decode and field sequencing for the VHS path (test infrastructure).

Per field (``TbcFieldDecodePipeline.DecodePrepared``,
Core/Decode/TbcFieldDecodePipeline.cs:1071-1440, standard VHS branch):
pulses on the sync reference at IreToHz(vsync_ire/2) -> timing -> classify ->
refine -> mean line length -> cadence -> VBlank line 0 -> upstream line
locations (output lines + 10) -> next-field offset -> hsync refinement ->
(chroma on: chroma TBC from line 1 -> burst phase sequence -> burst refinement
of the line locations) -> NTSC fsc phase shift -> sinc TBC of the output lines
-> uint16 -> dropouts (chroma on: chroma TBC -> uint16 chroma field).

Sequencing follows ``DecodeReadWindowPlanner`` (Core/Decode/DecodeReadWindowPlanner.cs:14-64)
and ``EstimateNextFieldStart`` (Core/Decode/TbcFieldSequenceDecodeEngine.cs:1934-1941).
"""
import math

import numpy as np

from . import chroma, demod, formats, sync, tbc, native
from .filters import FilterSet


class FieldError(Exception):
    """A field that could not be decoded, with the reference's recovery step
    (BuildRecoveryException / ThrowIfInsufficientFieldData,
    Core/Decode/TbcFieldDecodePipeline.cs:1150-1166, 5636-5650, 5936-6007; the engine
    loop Core/Decode/TbcFieldSequenceDecodeEngine.cs:804-847): the engine moves its
    read position on by ``offset`` samples and tries again."""

    def __init__(self, msg, offset):
        super().__init__(msg)
        self.offset = int(offset)   # C# (long) cast: truncation


def read_length(sp):
    line = int(round(sp.line_period_us * sp.mhz))
    if sp.system == "PAL":
        base = line * 400
    else:
        base = (line * 350 // 16384) * 16384
    return (base // demod.BLOCK + 2) * demod.BLOCK


def resolve_span(intended, read_len):
    read_loc = max(0, intended - demod.CUT)
    a0 = (read_loc // demod.BLOCK) * demod.BLOCK
    a1 = a0 + read_len
    first = a0 // demod.STRIDE
    last = a1 // demod.STRIDE
    return first * demod.STRIDE, (last - first + 1) * demod.STRIDE


class FieldState:
    def __init__(self):
        self.prev_first = None
        self.has_prev_hsync = False
        self.pulses_seen = False   # _vhsPulseSearchInitialized
        self.chroma_rot = 0        # _chromaRotationIndex (null -> 0)
        self.vhs_number = None     # _previousVhsFieldNumber
        self.vhs_loc = None        # _previousVhsFieldReadLocation


def vhs_field_number(state, read_location):
    """``ResolveVhsFieldNumber`` (Core/Decode/TbcFieldDecodePipeline.cs:860-874)."""
    if state.vhs_number is None or state.vhs_loc is None:
        return 0
    return state.vhs_number + 1 if read_location > state.vhs_loc else state.vhs_number


def _single_estimate(fe, le, has_prev):
    fc = fe["count"] if fe else 0
    lc = le["count"] if le else 0
    if fc == 6 or (not has_prev and fc > lc):
        return fe
    if le is not None:
        return le
    return fe


def output_first_line(sp, first_field):
    if sp.system == "NTSC":
        return 1
    return 3 if first_field else 4


def line_offset(sp, first_field):
    if sp.system != "PAL":
        return 0
    return 2 if first_field else 3


def decode_field(sp, fmt, video, vlp, env, state, want_tbc=True, chroma_span=None, cp=None, field_number=0):
    """Decode one field from span channels (arrays relative to the span start).

    With ``cp`` (chroma on, the reference's default for colour-under tapes) the
    burst phase of the chroma channel refines the line locations before the
    NTSC fsc shift (TbcFieldDecodePipeline.cs:1366-1399) and the field's
    chroma is decoded to uint16 (``res["chroma"]``)."""
    threshold = sp.ire_to_hz(sp.vsync_ire / 2.0)
    raw = sync.find_raw_pulses(sp, vlp, threshold)
    if not raw:
        # NoFirstHSync once pulses have been seen, else NoSyncPulses
        raise FieldError("no sync pulses", sp.nominal * 100.0 if state.pulses_seen else sp.fs / 10.0)
    state.pulses_seen = True
    timing = sync.estimate_timing(sp, raw)
    classified = sync.classify_pulses(sp, raw, timing)
    refined, _ = sync.refine_pulses(sp, raw, timing, vlp, 10.0 * sp.hz_ire)
    mll = sync.mean_line_length(sp, refined)
    first_field = sync.resolve_cadence(sp, refined, mll, state.prev_first, 100, state.has_prev_hsync)
    state.prev_first = first_field
    field_lines = sp.field_lines()[0 if first_field else 1]
    g1 = sync.find_first_group(refined, None, 9)
    if g1 is None:
        raise FieldError("no vblank", sp.nominal * 100.0)
    g2 = sync.find_first_group(refined, g1["eq1"] + (field_lines - 2.0) * mll, 9)
    fe, le, comb = sync.estimate_line0_from_groups(sp, classified, g1, g2, mll, first_field, field_lines)
    pick = comb if comb is not None else _single_estimate(fe, le, state.has_prev_hsync)
    if pick is None:
        raise FieldError("no line 0", sp.nominal * 100.0)
    line0 = pick["line0"]
    fh = pick["first_hsync"]
    state.has_prev_hsync = True
    processed = sp.output_lines + 10
    last_line = ((len(video) - line0) / mll) - 1.0
    if last_line < processed:
        raise FieldError("insufficient data", max(line0 - mll * 20.0, sp.nominal))
    fh_line = sync.first_hsync_line(sp, first_field)
    locs, filled = sync.build_upstream_line_locations(refined, float(math.trunc(fh)), int(fh_line),
                                                      mll, processed)
    next_loc = sync.next_field_location(sp, first_field, field_lines, mll, fh)
    next_off = next_loc - 8.0 * sp.nominal + demod.CUT
    locs, filled = sync.refine_hsync(sp, vlp, locs, filled, threshold)
    smoothing = fmt["sys"]["frame_lines"] / 2.0
    nominal_in = float(round(fmt["sys"]["line_period"] * sp.mhz))
    phase = None
    if cp is not None:
        ana = tbc.resample_field(chroma_span, locs, chroma.ANALYSIS_FIRST_LINE, sp.output_lines,
                                 sp.outlinelen, nominal_in, smoothing)
        input_line = max(1, int(round(sp.nominal)))
        phase = chroma.analyze_field_phase(ana, cp, locs, input_line, rot_index=state.chroma_rot)
        state.chroma_rot = phase["next_index"]
        locs = chroma.refine_from_burst(locs, sp.outlinelen, cp.fsc_ratio, phase, cp.ntsc)
    if sp.system == "NTSC":
        locs = locs - ((117.25 / 360.0) / sp.fsc_mhz) * sp.mhz
    res = {"first_field": first_field, "line0": line0, "first_hsync": fh, "mean_line": mll,
           "locs": locs, "next_offset": next_off, "pulses": raw, "refined": refined}
    if phase is not None:
        res["phase"] = phase
        res["field_number"] = field_number
    if want_tbc:
        ofl = output_first_line(sp, first_field)
        hz = tbc.resample_field(video, locs, ofl, sp.output_lines, sp.outlinelen, nominal_in, smoothing)
        res["tbc_hz"] = hz
        res["tbc"] = tbc.to_u16(hz, sp, formats.output_scale(fmt), fmt["sys"]["outputZero"])
        res["dropouts"] = dropouts(sp, env, locs, first_field)
        if phase is not None:
            c = tbc.resample_field(chroma_span, locs, ofl, sp.output_lines, sp.outlinelen, nominal_in, smoothing)
            res["chroma"] = chroma.decode_field_chroma(c, cp, phase, first_field, field_number, ofl)
    return res


def dropouts(sp, env, locs, first_field, frac=0.18, hyst=1.25):
    """``DetectTapeDropouts`` + ``RfDropoutDetector.FindDropouts`` + ``MapTapeRfToTbc``
    (TbcFieldDecodePipeline.cs:6593-6640; TbcDropoutMapping.cs:52-107, 288-370)."""
    off = line_offset(sp, first_field)
    start_line = off + 1
    field_lines = sp.field_lines()[0 if first_field else 1]
    end_line = min(len(locs) - 1, field_lines + start_line + 1)
    if start_line < 0 or end_line <= start_line or start_line >= len(locs):
        return []
    s0 = min(max(int(math.floor(locs[start_line])), 0), len(env))
    s1 = min(max(int(math.ceil(locs[end_line])), s0), len(env))
    if s1 <= s0:
        return []
    mean32 = np.mean(np.asarray(env, np.float32), dtype=np.float32)
    thr = float(np.float32(mean32 * np.float32(frac)))
    ranges = native.find_dropouts(env, s0, s1, thr, hyst)
    return map_rf_to_tbc(ranges, locs, sp.outlinelen, start_line, end_line, off)


def map_rf_to_tbc(ranges, locs, outlen, start_line, end_line, off):
    out = []
    li = start_line
    ls, le = locs[li], locs[li + 1]
    for (ds, de) in ranges:
        found = False
        while li < end_line:
            ll = le - ls
            if (ds >= ls or li == start_line) and ds < le and ll > 0.0:
                sx = int(math.floor(((ds - ls) / ll) * outlen))
                cur = [li - off, max(0, sx), None]
                found = True
                break
            li += 1
            if li < end_line:
                ls, le = locs[li], locs[li + 1]
        if not found:
            break
        while li < end_line:
            ll = le - ls
            if de < le and ll > 0.0:
                ex = int(math.ceil(((de - ls) / ll) * outlen))
                cur[2] = min(outlen, ex)
                out.append(tuple(cur))
                break
            cur[2] = outlen
            out.append(tuple(cur))
            li += 1
            if li < end_line:
                ls, le = locs[li], locs[li + 1]
                cur = [li - off, 0, None]
    return out


def decode_capture(rf, fmt, fs=40e6, max_fields=None, want_tbc=True, channels=None, with_chroma=False,
                   chroma_channel=None):
    """Decode a whole int16 capture; returns (fields, channels).

    ``with_chroma`` runs the reference's default colour-under chroma path
    (burst refinement of the lines and a uint16 chroma field); without it the
    decode is the reference's ``--skip_chroma`` one."""
    sp = sync.SyncParams(fmt, fs)
    filt = FilterSet(fmt, fs)
    diff_max = (sp.ire0 + sp.hz_ire * 100.0) * 2.0
    if channels is None:
        channels = demod.demod_stream(rf, filt, fs, diff_max)
    video, vlp, env, _ = channels
    cp = chroma.ChromaParams(fmt, fs) if with_chroma else None
    if cp is not None and chroma_channel is None:
        chroma_channel = chroma.chroma_stream(rf, cp)
    avail = len(video)
    rl = read_length(sp)
    state = FieldState()
    fields = []
    intended = 0
    while max_fields is None or len(fields) < max_fields:
        s0, slen = resolve_span(intended, rl)
        if s0 + slen > avail:
            break
        sl = slice(s0, s0 + slen)
        number = vhs_field_number(state, s0)
        try:
            f = decode_field(sp, fmt, video[sl], vlp[sl], env[sl], state, want_tbc,
                             chroma_channel[sl] if cp is not None else None, cp, number)
        except FieldError as exc:
            fields.append({"error": str(exc), "span_start": s0, "recovery": exc.offset})
            intended = max(0, intended + exc.offset)
            # v0.4.0 restarts the VHS field number after an invalid field
            state.vhs_number = state.vhs_loc = None
            continue
        state.vhs_number, state.vhs_loc = number, s0
        f["span_start"] = s0
        f["span_len"] = slen
        fields.append(f)
        intended = s0 + max(1, int(sync.round_away(f["next_offset"])))
    return fields, channels
