"""Seeded synthetic VHS RF generator.

Builds composite luma (IRE) with the PAL 625/50 or NTSC 525/60 sync structure
(equalising / broad pulses at half-line spacing, hsync, active video), applies
the VHS FM pre-emphasis (the high shelf whose inverse the decoder uses as its
de-emphasis), FM-modulates it with f = ire0 + hz_ire * IRE, adds the
line-locked colour-under chroma (burst and colour bars, heterodyned down with
the format's per-line phase rotation), optional carrier dropouts, timebase
wobble and head switching jumps, Gaussian noise at a stated SNR, and quantises to int16 with a
+/-12000 peak.  Everything is driven by one ``numpy.random.Generator`` seed.

The pulse geometry (half-line positions of the equalising and broad pulses
and the half/whole-line gaps either side of them) is the standard PAL / NTSC
field structure that the decoder's VBlank resolver expects.
"""
from dataclasses import dataclass, field
import math

import numpy as np
import scipy.signal as sps


@dataclass
class SynthConfig:
    system: str = "PAL"            # "PAL" or "NTSC"
    ire0: float = 4100000.0
    hz_ire: float = 7000.0
    vsync_ire: float = -42.857142857142854
    fs: float = 40e6
    fields: int = 4
    seed: int = 1
    snr_db: float = 40.0
    chroma_db: float = -10.0
    chroma_hz: float = 626953.0
    deemph_gain: float = 13.9794
    deemph_mid: float = 273755.82
    deemph_q: float = 0.462088186
    dropouts: int = 0
    dropout_us: tuple = (2.0, 40.0)
    dropout_level: float = 0.05
    wobble_frac: float = 0.0       # e.g. 0.005 for +/-0.5% timebase wobble
    wobble_hz: float = 15.0
    headswitch_samples: float = 0.0  # +/- jump applied once per field
    peak: float = 12000.0
    lead_lines: float = 12.0       # capture starts this many lines before a VBlank
    patterns: tuple = ("bars", "ramp", "noise", "noise")
    extra: dict = field(default_factory=dict)


def pal_vhs(**kw):
    return SynthConfig(**kw)


def ntsc_vhs(**kw):
    base = dict(system="NTSC", ire0=3685714.2857142854, hz_ire=7142.857142857143,
                vsync_ire=-40.0, chroma_hz=629370.6293706294)
    base.update(kw)
    return SynthConfig(**base)


def pal_svhs(**kw):
    """PAL S-VHS SP: sync tip 5.4 MHz, peak white 7.0 MHz.  The pre-emphasis is
    the linear shelf only (the decoder's sub-deemphasis is a nonlinear
    refinement on top of it)."""
    base = dict(ire0=5880000.0, hz_ire=11200.0)
    base.update(kw)
    return SynthConfig(**base)


def ntsc_svhs(**kw):
    base = dict(system="NTSC", ire0=5857142.857142857, hz_ire=11428.57142857143,
                vsync_ire=-40.0, chroma_hz=629370.6293706294)
    base.update(kw)
    return SynthConfig(**base)


def _geometry(system):
    if system == "PAL":
        return dict(lines=625, line_us=64.0, hsync_us=4.7, eq_us=2.35, vsync_us=27.3,
                    active=(10.5, 62.5))
    return dict(lines=525, line_us=1e6 / (4.5e6 / 286.0), hsync_us=4.7, eq_us=2.3,
                vsync_us=27.1, active=(9.45, 62.4))


def _halfline_kinds(system):
    """Pulse kind at the start of each half-line of one frame: 0 none, 1 hsync, 2 eq, 3 broad.

    Half-line h starts at h * line/2 from the start of frame line 1.
    """
    g = _geometry(system)
    n_half = 2 * g["lines"]
    kinds = np.zeros(n_half, np.int8)
    kinds[0::2] = 1
    if system == "PAL":
        broad = list(range(0, 5)) + list(range(625, 630))
        eq = list(range(5, 10)) + list(range(1245, 1250)) + list(range(620, 625)) + list(range(630, 635))
        no_hsync = [618 + 1 + 0]  # line 310.5 is a mid-line; keep standard: nothing extra
        del no_hsync
        # line 318 (h=634) carries an eq pulse; line 318.5 (h=635) none; 319 (h=636) hsync
    else:
        eq = list(range(0, 6)) + list(range(12, 18)) + list(range(525, 531)) + list(range(537, 543))
        broad = list(range(6, 12)) + list(range(531, 537))
    for h in range(n_half):
        if h in broad:
            kinds[h] = 3
        elif h in eq:
            kinds[h] = 2
    # mid-line positions that are not pulses must be none
    return kinds


def _active_line(system, frame_line):
    if system == "PAL":
        return (23 <= frame_line <= 310) or (336 <= frame_line <= 622)
    return (21 <= frame_line <= 262) or (284 <= frame_line <= 524)


def _field_of_line(system, frame_line):
    if system == "PAL":
        return 0 if frame_line <= 312 else 1
    return 0 if frame_line <= 263 else 1


def _smoothstep(t, width):
    """Raised-cosine step from 0 (t <= -w/2) to 1 (t >= w/2)."""
    x = np.clip(t / width + 0.5, 0.0, 1.0)
    return 0.5 - 0.5 * np.cos(np.pi * x)


def _content(pattern, rng, field_index):
    if pattern == "bars":
        levels = 75.0 * np.array([1.0, 0.886, 0.701, 0.587, 0.413, 0.299, 0.114, 0.0])
        return ("bars", levels)
    if pattern == "ramp":
        return ("ramp", None)
    blocks = rng.uniform(0.0, 100.0, size=(40, 32))
    return ("noise", blocks)


def _content_value(spec, field_line, x):
    kind, data = spec
    if kind == "bars":
        idx = np.clip((x * 8).astype(np.int64), 0, 7)
        return data[idx]
    if kind == "ramp":
        return 100.0 * x
    rows = np.clip(field_line // 8, 0, data.shape[0] - 1)
    cols = np.clip((x * data.shape[1]).astype(np.int64), 0, data.shape[1] - 1)
    return data[rows, cols]


def generate(cfg: SynthConfig):
    """Return (rf_int16, info) for ``cfg``."""
    rng = np.random.default_rng(cfg.seed)
    g = _geometry(cfg.system)
    fs = cfg.fs
    line_len = g["line_us"] * fs / 1e6
    half_len = line_len / 2.0
    frame_lines = g["lines"]
    field_samples = frame_lines * line_len / 2.0
    lead = cfg.lead_lines * line_len
    total = int(math.ceil((cfg.fields + 1.5) * field_samples + lead))
    # time base (with optional wobble and per-field head-switch jumps)
    n = np.arange(total, dtype=np.float64)
    t = n.copy()
    if cfg.wobble_frac:
        t = t + (cfg.wobble_frac * fs / (2 * np.pi * cfg.wobble_hz)) * np.sin(
            2 * np.pi * cfg.wobble_hz * n / fs + rng.uniform(0, 2 * np.pi))
    if cfg.headswitch_samples:
        jumps = rng.uniform(-cfg.headswitch_samples, cfg.headswitch_samples,
                            size=cfg.fields + 4)
        fidx = np.floor((n + (field_samples - lead)) / field_samples).astype(np.int64)
        t = t + np.cumsum(jumps)[np.clip(fidx, 0, len(jumps) - 1)]
    # frame position: start `lead` samples before the first field's VBlank (frame line 1 / h=0)
    frame_pos = t - lead + (frame_lines * line_len) - (frame_lines * line_len)  # h=0 at t=lead
    frame_len = frame_lines * line_len
    fp = np.mod(frame_pos, frame_len)
    frame_no = np.floor(frame_pos / frame_len).astype(np.int64)
    kinds = _halfline_kinds(cfg.system)
    h = np.floor(fp / half_len).astype(np.int64) % (2 * frame_lines)
    tau_h = fp - h * half_len                       # samples since half-line start
    frame_line = h // 2 + 1
    tau_l = fp - (frame_line - 1) * line_len        # samples since line start
    us = 1e6 / fs
    edge = 0.2 / us                                  # 200 ns transitions
    sync_level = cfg.vsync_ire
    kind = kinds[h]
    width = np.where(kind == 1, g["hsync_us"], np.where(kind == 2, g["eq_us"],
                     np.where(kind == 3, g["vsync_us"], 0.0))) / us
    pulse = _smoothstep(tau_h, edge) * (1.0 - _smoothstep(tau_h - width, edge))
    pulse = np.where(kind == 0, 0.0, pulse)
    # a pulse tail crossing into a 'none' half-line: handled because widths < half line
    ire = sync_level * pulse
    # active video
    a0, a1 = g["active"][0] / us, g["active"][1] / us
    act_win = _smoothstep(tau_l - a0, edge) * (1.0 - _smoothstep(tau_l - a1, edge))
    is_active = np.vectorize(lambda fl: _active_line(cfg.system, fl), otypes=[bool])(
        np.arange(frame_lines + 1))[np.clip(frame_line, 0, frame_lines)]
    fields_in_frame = np.vectorize(lambda fl: _field_of_line(cfg.system, fl), otypes=[np.int64])(
        np.arange(frame_lines + 1))[np.clip(frame_line, 0, frame_lines)]
    field_index = frame_no * 2 + fields_in_frame
    x = np.clip((tau_l - a0) / (a1 - a0), 0.0, 1.0)
    first_line_of_field = np.where(fields_in_frame == 0, 1, frame_lines // 2 + 2)
    field_line = frame_line - first_line_of_field
    video = np.zeros(total)
    uniq = np.unique(field_index)
    for fi in uniq:
        sel = (field_index == fi) & is_active
        if not np.any(sel):
            continue
        pattern = cfg.patterns[int(fi) % len(cfg.patterns)]
        spec = _content(pattern, np.random.default_rng((cfg.seed, int(fi) + 1000)), fi)
        video[sel] = _content_value(spec, field_line[sel], x[sel])
    ire = ire + video * act_win * is_active
    # band-limit the composite (about 4.5 MHz) before pre-emphasis
    ire = _gauss_smooth(ire, sigma_samples=fs / (2 * np.pi * 4.5e6))
    # VHS pre-emphasis: the high shelf whose inverse is the decoder's de-emphasis
    b, a = _high_shelf(cfg.deemph_mid, cfg.deemph_gain, fs, cfg.deemph_q)
    zi = sps.lfilter_zi(b, a) * ire[0]
    ire_pre, _ = sps.lfilter(b, a, ire, zi=zi)
    freq = cfg.ire0 + cfg.hz_ire * ire_pre
    phase = np.cumsum(2.0 * np.pi * freq / fs)
    carrier = np.cos(phase)
    if cfg.dropouts:
        amp = np.ones(total)
        lo, hi = cfg.dropout_us
        starts = rng.integers(int(lead), total - int(hi / us) - 1, size=cfg.dropouts)
        lens = rng.uniform(lo, hi, size=cfg.dropouts) / us
        for s, ln in zip(starts, lens):
            amp[s:s + int(ln)] = cfg.dropout_level
        carrier = carrier * amp
    chroma_amp = 10.0 ** (cfg.chroma_db / 20.0)
    chroma = _colour_under(cfg, g, fs, frame_no, frame_line, tau_l, field_index, x, act_win, is_active, edge)
    rf = carrier + chroma_amp * chroma
    sig_rms = math.sqrt(0.5 + 0.5 * chroma_amp ** 2)
    noise_std = sig_rms / (10.0 ** (cfg.snr_db / 20.0))
    rf = rf + rng.normal(0.0, noise_std, size=total)
    scale = cfg.peak / (1.0 + chroma_amp * 1.3 + 4.5 * noise_std)
    out = np.clip(np.rint(rf * scale), -32768, 32767).astype(np.int16)
    info = {"line_len": line_len, "field_samples": field_samples, "lead": lead,
            "total": total, "scale": scale}
    return out, info


# 75 % colour bars: (U, V) of white, yellow, cyan, green, magenta, red, blue, black
_BARS_UV = 0.75 * np.array([[0.0, 0.0], [-0.436, 0.100], [0.147, -0.615], [-0.289, -0.515],
                            [0.289, 0.515], [-0.147, 0.615], [0.436, -0.100], [0.0, 0.0]])


def _colour_under(cfg, g, fs, frame_no, frame_line, tau_l, field_index, x, act_win, is_active, edge):
    """Line-locked colour-under chroma, as a VCR records it: the composite
    chroma (burst, and the colour bars' U/V on 'bars' fields) is heterodyned
    down to the colour-under carrier with the format's per-line phase rotation
    (PAL: 0 or -90 degrees a line on alternate fields; NTSC: -90 or +90).  In
    the decoder's 4 fSC domain, up-converting with the same rotation gives the
    burst and the bars back at fSC.  Amplitude 1 is the peak chroma."""
    pal = cfg.system == "PAL"
    us = 1e6 / fs
    frame_lines = g["lines"]
    line_index = frame_no * frame_lines + (frame_line - 1)       # running line count
    rot = np.where(field_index % 2 == 0, 0, -1) if pal else np.where(field_index % 2 == 0, -1, 1)
    quarter = np.mod(rot * line_index, 4)
    # burst: PAL +-135 degrees (alternate lines), NTSC 180 degrees
    b0, b1 = (5.6, 7.85) if pal else (5.3, 7.8)
    bwin = _smoothstep(tau_l - b0 / us, edge) * (1.0 - _smoothstep(tau_l - b1 / us, edge))
    vsw = np.where(line_index % 2 == 0, 1.0, -1.0) if pal else np.ones_like(tau_l)
    burst_phase = np.where(vsw > 0, 0.75 * np.pi, 1.25 * np.pi) if pal else np.full_like(tau_l, np.pi)
    # active picture: the bars' chroma on 'bars' fields
    bars_field = np.zeros_like(tau_l, dtype=bool)
    for fi in np.unique(field_index):
        if cfg.patterns[int(fi) % len(cfg.patterns)] == "bars":
            bars_field |= field_index == fi
    idx = np.clip((x * 8).astype(np.int64), 0, 7)
    u = _BARS_UV[idx, 0]
    v = _BARS_UV[idx, 1] * vsw
    amp_act = np.hypot(u, v) * act_win * is_active * bars_field
    hue = np.arctan2(v, u)
    amp = 0.3 * bwin + amp_act
    theta = np.where(bwin > amp_act, burst_phase, hue)
    # colour-under phase of the line: rotation, the carrier's advance over one
    # output line of the 4 fSC time base (outlinelen samples; about 40.125
    # cycles PAL, 40 NTSC) and the composite phase, reversed by the down-conversion
    outlen, fsc = (1135, 4.43361875e6) if pal else (910, 315e6 / 88.0)
    per_line = 2.0 * np.pi * cfg.chroma_hz * outlen / (4.0 * fsc)
    psi = np.pi + quarter * (np.pi / 2.0) - theta + per_line * line_index
    return amp * np.cos(2.0 * np.pi * cfg.chroma_hz * tau_l / fs + psi)


def _gauss_smooth(x, sigma_samples):
    radius = int(4 * sigma_samples) + 1
    k = np.exp(-0.5 * (np.arange(-radius, radius + 1) / sigma_samples) ** 2)
    k /= k.sum()
    return sps.fftconvolve(np.pad(x, radius, mode="edge"), k, mode="valid")


def _high_shelf(center_hz, gain_db, fs, q):
    g = 10.0 ** (gain_db / 40.0)
    w = 2.0 * math.pi * center_hz / fs
    alpha = math.sin(w) / (2.0 * q)
    c = math.cos(w)
    rg = math.sqrt(g)
    b = [g * ((g + 1) + (g - 1) * c + 2 * rg * alpha), -2 * g * ((g - 1) + (g + 1) * c),
         g * ((g + 1) + (g - 1) * c - 2 * rg * alpha)]
    a = [(g + 1) - (g - 1) * c + 2 * rg * alpha, 2 * ((g - 1) - (g + 1) * c),
         (g + 1) - (g - 1) * c - 2 * rg * alpha]
    return np.array(b) / a[0], np.array(a) / a[0]


def config(name: str, **overrides):
    """Named workloads: 'pal4' (PAL VHS 4 fields), 'ntsc60' (NTSC VHS 60 fields, dropouts),
    'svhs100' (PAL S-VHS 100 fields, 42 dB SNR, +/-0.5 % timebase wobble at 15 Hz,
    +/-2-sample head-switch jumps every field) and small parity cases."""
    if name == "pal4":
        c = pal_vhs(fields=4, seed=11, snr_db=40.0)
    elif name == "ntsc60":
        c = ntsc_vhs(fields=60, seed=22, snr_db=38.0, dropouts=200,
                     patterns=("bars", "ramp", "noise"))
    elif name == "pal_small":
        c = pal_vhs(fields=3, seed=5, snr_db=40.0)
    elif name == "ntsc_small":
        c = ntsc_vhs(fields=3, seed=6, snr_db=38.0, dropouts=8)
    elif name == "svhs100":
        c = pal_svhs(fields=100, seed=33, snr_db=42.0, wobble_frac=0.005, wobble_hz=15.0,
                     headswitch_samples=2.0, patterns=("bars", "ramp", "noise", "noise"))
    elif name == "svhs_small":
        c = pal_svhs(fields=4, seed=7, snr_db=42.0, wobble_frac=0.005, wobble_hz=15.0,
                     headswitch_samples=2.0)
    elif name == "svhs_ntsc_small":
        c = ntsc_svhs(fields=3, seed=8, snr_db=42.0, dropouts=6, wobble_frac=0.005,
                      headswitch_samples=2.0)
    else:
        raise KeyError(name)
    for k, v in overrides.items():
        setattr(c, k, v)
    return c
