"""Filter spectra of the VHS RF path, restated with scipy (test infrastructure).

Follows ``DecodeFilterSetBuilder.BuildBasic`` (Core/Dsp/DecodeFilterSet.cs:140-256)
for colour-under tape formats.  Every response is a length-N "whole" frequency
response (``scipy.signal.freqz(..., worN=N, whole=True)`` semantics, as
``IirFilterDesign.FrequencyResponse`` Core/Dsp/IirFilterDesign.cs:962-1058);
the real-FFT path only reads bins 0..N/2.
"""
import math
import os

import numpy as np
import scipy.signal as sps

from . import formats

DATA = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                    "vhs-decode-dotnet_gb300", "data")


def _freqz_ba(b, a, n):
    _, h = sps.freqz(b, a, worN=n, whole=True)
    return h


def _freqz_sos(sos, n):
    _, h = sps.sosfreqz(sos, worN=n, whole=True)
    return h


def super_gaussian(x, freq, order=1, center=0.0):
    """``PortedMath.SuperGaussian`` (Core/Dsp/PortedMath.cs:476-480)."""
    scale = 2.0 * (x - center) * math.pow(math.log(2.0) / 2.0, 1.0 / (2.0 * order))
    return np.exp(-2.0 * np.power(scale / freq, 2.0 * order))


def lowpass_super_gaussian_half(corner, order, nyq, n):
    """``FrequencyDomainFilter.LowPassSuperGaussianHalf`` (Core/Dsp/FrequencyDomainFilter.cs:7-23)."""
    count = n // 2 + 1
    f = nyq * np.arange(count) / (count - 1)
    return super_gaussian(f, corner, order)


def mirror_half_to_full(half):
    """``FrequencyDomainFilter.MirrorHalfToFull`` (Core/Dsp/FrequencyDomainFilter.cs:46-62)."""
    n = (len(half) - 1) * 2
    out = np.zeros(n)
    out[: len(half)] = half
    out[n - np.arange(1, len(half) - 1)] = half[1:-1]
    return out


def ramp_filter(start_hz, boost_start, boost_max, nyq, n):
    """``FrequencyDomainFilter.RampFilter`` (Core/Dsp/FrequencyDomainFilter.cs:64-103).

    Note the mirror is ``out[N-1-i] = half[i]`` (one bin off a Hermitian mirror),
    so bin N/2 carries ``half[N/2-1]``.
    """
    max_f = 20e6
    half_n = n // 2
    zero = int((start_hz / nyq) * half_n)
    zero = min(max(zero, 0), half_n)
    half = np.zeros(half_n)
    ramp_count = half_n - zero
    if ramp_count == 1:
        half[zero] = boost_start
    elif ramp_count > 1:
        end = boost_max * (nyq / max_f)
        step = (end - boost_start) / (ramp_count - 1)
        half[zero:] = boost_start + np.arange(ramp_count) * step
        half[-1] = end
    out = np.zeros(n)
    out[:half_n] = half
    out[n - 1 - np.arange(half_n)] = half
    return out


def peaking_constant_q(norm_freq, gain_db, bw_oct):
    """``IirFilterDesign.PeakingConstantQ`` + ``BilinearSecondOrder`` (IirFilterDesign.cs:854-871,1614-1636)."""
    q = 1.0 / (2.0 * math.sinh((math.log(2.0) / 2.0) * bw_oct))
    gain = math.pow(10.0, gain_db / 20.0)
    zg = gain if gain_db > 0 else 1.0
    pg = 1.0 if gain_db > 0 else gain
    w = 4.0 * math.tan(math.pi * norm_freq / 2.0)
    an = [1.0, (zg / q) * w, w * w]
    ad = [1.0, (1.0 / (pg * q)) * w, w * w]
    c = 2.0 * 2.0
    c2 = c * c
    n0 = an[0] * c2 + an[1] * c + an[2]
    n1 = -2.0 * an[0] * c2 + 2.0 * an[2]
    n2 = an[0] * c2 - an[1] * c + an[2]
    d0 = ad[0] * c2 + ad[1] * c + ad[2]
    d1 = -2.0 * ad[0] * c2 + 2.0 * ad[2]
    d2 = ad[0] * c2 - ad[1] * c + ad[2]
    return [n0 / d0, n1 / d0, n2 / d0], [1.0, d1 / d0, d2 / d0]


def high_shelf(center_hz, gain_db, fs, q):
    """``IirFilterDesign.Shelf(kind=High)`` (Core/Dsp/IirFilterDesign.cs:873-921)."""
    g = math.pow(10.0, gain_db / 40.0)
    w = 2.0 * math.pi * (center_hz / fs)
    alpha = math.sin(w) / (2.0 * q)
    c = math.cos(w)
    rg = math.sqrt(g)
    b0 = g * ((g + 1.0) + ((g - 1.0) * c) + (2.0 * rg * alpha))
    b1 = -2.0 * g * ((g - 1.0) + ((g + 1.0) * c))
    b2 = g * ((g + 1.0) + ((g - 1.0) * c) - (2.0 * rg * alpha))
    a0 = (g + 1.0) - ((g - 1.0) * c) + (2.0 * rg * alpha)
    a1 = 2.0 * ((g - 1.0) - ((g + 1.0) * c))
    a2 = (g + 1.0) - ((g - 1.0) * c) - (2.0 * rg * alpha)
    return [b0, b1, b2], [a0, a1, a2]


def deemphasis_ba(fs, gain_db, mid_hz, q):
    """``VideoDeEmphasisShelf`` = inverse of the high shelf (IirFilterDesign.cs:924-934)."""
    b, a = high_shelf(mid_hz, gain_db, fs, q)
    return a, b


def custom_luma_table(filename, fs, n):
    """``DecodeFilterSetBuilder.TryLoadCustomFilter`` (Core/Dsp/DecodeFilterSet.cs:1658-1714):
    the resource ``<filename>-<(int)fs>.txt`` (bins 0..N/2, mirrored conjugate above),
    or None when the reference has no table for this rate.  The tables are the
    reference's resources converted to binary64 pairs (pinned by SHA-256 in
    tests/golden/format_params.json)."""
    path = os.path.join(DATA, "%s-%d.f64" % (filename, int(fs)))
    if not os.path.exists(path):
        return None
    half = np.fromfile(path, "<f8").reshape(-1, 2)
    half = half[:, 0] + 1j * half[:, 1]
    if len(half) != n // 2 + 1:
        return None
    out = np.zeros(n, complex)
    out[: len(half)] = half
    i = np.arange(1, len(half) - 1)
    out[n - i] = np.conj(half[i])
    return out


def apply_custom_video_filters(video, rf, fs, n):
    """``ApplyCustomVideoFilters`` (Core/Dsp/DecodeFilterSet.cs:1560-1609); shelves are
    designed with fs/2 as their rate argument, as the reference passes them."""
    for flt in rf.get("video_custom_luma_filters") or []:
        kind = flt["type"]
        resp = None
        if kind == "file":
            resp = custom_luma_table(flt["filename"], fs, n)
        elif kind == "highshelf":
            b, a = high_shelf(flt["midfreq"], flt["gain"], fs / 2.0, flt["q"])
            resp = _freqz_ba(b, a, n)
        elif kind == "lowshelf":
            raise NotImplementedError("low shelf custom luma filters")
        if resp is not None and len(resp) == len(video):
            video = video * resp
    return video


def firwin_lowpass_hamming(numtaps, cutoff):
    """``FirWinLowPass`` (Core/Dsp/DecodeFilterSet.cs:1346-1375) == scipy.signal.firwin."""
    return sps.firwin(numtaps, cutoff, window="hamming")


class FilterSet:
    """Bins 0..N/2 of the spectra the VHS block demodulator multiplies by."""

    def __init__(self, fmt: dict, fs: float, n: int = 32768):
        self.fmt = fmt
        self.fs = fs
        self.n = n
        nyq = fs / 2.0
        rf = fmt["rf"]
        # RfVideo (DecodeFilterSet.cs:307-406) -- tape formats use magnitudes.
        order = rf.get("video_bpf_order")
        if order:
            b, a = sps.butter(order, [rf["video_bpf_low"] / nyq, rf["video_bpf_high"] / nyq], "bandpass")
            out = np.abs(_freqz_ba(b, a, n))
        else:
            out = np.ones(n)
        if rf.get("video_lpf_extra") is not None:
            sos = sps.butter(rf["video_lpf_extra_order"], rf["video_lpf_extra"] / nyq, "low", output="sos")
            out = out * np.abs(_freqz_sos(sos, n))
        if rf.get("video_hpf_extra") is not None:
            sos = sps.butter(rf["video_hpf_extra_order"], rf["video_hpf_extra"] / nyq, "high", output="sos")
            out = out * np.abs(_freqz_sos(sos, n))
        if rf.get("video_rf_peak_freq"):
            b, a = peaking_constant_q(rf["video_rf_peak_freq"] / nyq, rf["video_rf_peak_gain"],
                                      rf["video_rf_peak_bandwidth"] / nyq)
            out = out * np.abs(_freqz_ba(b, a, n))
        if rf.get("boost_rf_linear_0") is not None:
            ramp = ramp_filter(rf.get("start_rf_linear", 0.0), rf["boost_rf_linear_0"],
                               rf.get("boost_rf_linear_20", 1.0), nyq, n)
            out = out * ramp
            if rf.get("boost_rf_linear_double"):
                out = out * ramp
        self.rf_video = np.abs(out)

        # VideoLowPass (DecodeFilterSet.cs:1019-1061), zero-phase magnitude for tape.
        corner = rf["video_lpf_freq"]
        lorder = rf["video_lpf_order"]
        if rf.get("video_lpf_supergauss"):
            vlp = mirror_half_to_full(lowpass_super_gaussian_half(corner, lorder, nyq, n)).astype(complex)
        else:
            if lorder % 2 == 0:
                sos = sps.butter(lorder, corner / nyq, "low", output="sos")
                vlp = _freqz_sos(sos, n)
            else:
                b, a = sps.butter(lorder, corner / nyq, "low")
                vlp = _freqz_ba(b, a, n)
            vlp = np.abs(vlp).astype(complex)
        self.video_lowpass = vlp
        # De-emphasis shelf (DecodeFilterSet.cs:1104-1152).
        db, da = deemphasis_ba(fs, rf["deemph_gain"], rf["deemph_mid"], rf["deemph_q"])
        deemp = _freqz_ba(db, da, n)
        # BuildVideo (DecodeFilterSet.cs:1063-1091): LPF x de-emphasis x custom luma filters
        self.video = apply_custom_video_filters(vlp * deemp, rf, fs, n)
        video_ref = vlp * deemp                        # BuildVideoReference
        if 500_000.0 >= nyq:
            self.video_lp05 = video_ref
        else:
            taps = firwin_lowpass_hamming(65, 0.5 / (nyq / 1e6))
            self.video_lp05 = video_ref * np.fft.fft(taps, n)
        self.video_lp05_offset = 32
        # Envelope low-pass: 1st-order Butterworth at 700 kHz (DecodeFilterSet.cs:602-620,
        # IirFilterDesign.cs:1078-1109).
        k = math.tan(math.pi * (700_000.0 / nyq) / 2.0)
        norm = 1.0 / (1.0 + k)
        self.env_b = (k * norm, k * norm)
        self.env_a1 = (k - 1.0) * norm
        # Sub-deemphasis (RfDemodulator.cs:2852-2990, 3101-3142): first-order Butterworth
        # high-pass (band-pass when nonlinear_bandpass_upper is set) and amplitude low-pass.
        self.sub = formats.sub_deemphasis(fmt)
        if self.sub is not None:
            o = self.sub
            if o["bandpass_upper"] is not None:
                raise NotImplementedError("sub-deemphasis band-pass")
            kh = math.tan(math.pi * (o["highpass"] / nyq) / 2.0)
            nh = 1.0 / (1.0 + kh)
            self.sub_highpass = _freqz_ba([nh, -nh, 0.0], [1.0, (kh - 1.0) * nh, 0.0], n)
            ka = math.tan(math.pi * (o["amp_lpf"] / nyq) / 2.0)
            na = 1.0 / (1.0 + ka)
            self.sub_amp_b = (ka * na, ka * na)
            self.sub_amp_a1 = (ka - 1.0) * na

    def half(self, name):
        return getattr(self, name)[: self.n // 2 + 1]
