"""Sinc TBC resampling to 4fSC and Hz -> uint16 conversion (test infrastructure).

Restates ``TbcLineResampler`` (Core/Tbc/TbcLineResampler.cs):
``LinearLineLocationInterpolator.FillOutputPositions`` (:1480-1532),
``BuildLinearLevelAdjusts`` median/MAD wow factors (:818-878) with
``SmoothLevelAdjusts`` (:997-1011), ``SampleSinc`` (:1167-1234) over the
Kaiser-sinc LUT (:1297-1330), and ``VideoOutputConverter.FastMathConversion``
(Core/Tbc/VideoOutputConverter.cs:9-40).
"""
import numpy as np

from . import native


def linear_positions(locs, first_line, line_count, outlen, nominal):
    """Bit-exact ``FillOutputPositions`` for lines [first_line, first_line+line_count)."""
    locs = np.asarray(locs, np.float64)
    out_scale = nominal / outlen
    idx = np.arange(first_line * outlen, (first_line + line_count) * outlen, dtype=np.int64)
    left = idx // outlen
    scaled = idx.astype(np.float64) * out_scale
    frac = np.clip((scaled - left.astype(np.float64) * nominal) / nominal, 0.0, 1.0)
    ll = locs[left]
    return ll + (locs[left + 1] - ll) * frac


def level_adjusts(locs, first_line, line_count, outlen, nominal, smoothing):
    """``BuildLinearLevelAdjusts`` + ``SmoothLevelAdjusts``; returns the [prefix+dest] array."""
    locs = np.asarray(locs, np.float64)
    total_lines = first_line + line_count
    inv = 1.0 / nominal
    lines = np.arange(total_lines)
    left = np.clip(lines, 0, len(locs) - 2)
    factors = (locs[left + 1] * inv) - (locs[left] * inv)
    med = float(np.median(factors))
    dev = np.abs(factors - med)
    mad = float(np.median(dev))
    thr = 15.0 * mad if mad > 0.0 else 0.001
    adj = np.where(np.abs(factors - med) > thr, med, factors)
    la = np.repeat(adj, outlen)
    if smoothing > 0.0:
        alpha = 1.0 / (smoothing * outlen)
        la = _smooth(la, alpha)
    return la


def _smooth(la, alpha):
    """levelAdjusts[i] = fma(levelAdjusts[i] - previous, alpha, previous), sequentially."""
    return native.smooth_levels(la, alpha)


def resample_field(video, locs, first_line, line_count, outlen, nominal, smoothing, lut=None):
    """Float output of ``ResamplePrepared`` (values are float32-rounded)."""
    if lut is None:
        lut = native.sinc_lut()
    pos = linear_positions(locs, first_line, line_count, outlen, nominal)
    la = level_adjusts(locs, first_line, line_count, outlen, nominal, smoothing)
    prefix = first_line * outlen
    return native.sinc_resample(video, pos, la[prefix:prefix + len(pos)], lut)


def to_u16(x, sp, output_scale, output_zero):
    return native.hz_to_u16(x, sp.ire0, output_scale, sp.hz_ire, output_zero, sp.vsync_ire)
