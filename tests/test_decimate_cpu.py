"""The 2:1 decimator's oracle (cuda-fast 20-MSPS reader mode) pinned without a GPU.

The reference has no golden vectors for its decimator
(src/VHSDecode.CudaFast.Native/src/cuda_fast_decimator.cu), so the oracle is
pinned to its defining arithmetic evaluated exactly: each output is the
centre product rounded to float32, then per tap pair one float32 add and one
fused multiply-add (exact product plus running value, rounded once).  The
exact values come from rational arithmetic and are rounded to nearest-even
float32 here, independently of the C oracle.
"""
from fractions import Fraction

import numpy as np
import pytest

from oracle import native as onative

COEFFS = np.array([0.5000046374907835, 0.3126333216205309, -0.09010692207961689,
                   0.040107417651266825, -0.017917030421899405, 0.007100857132041433,
                   -0.0022302855185240434, 0.00041032287080936366], np.float32)


def _rn32(q):
    """Fraction -> nearest float32, ties to even."""
    f = np.float32(float(q))
    best = None
    for c in (np.nextafter(f, np.float32(-np.inf)), f, np.nextafter(f, np.float32(np.inf))):
        d = abs(Fraction(float(c)) - q)
        key = (d, int(np.array(c).view(np.uint32)) & 1)
        if best is None or key < best[0]:
            best = (key, c)
    return best[1]


def _exact_decimate(x):
    n = len(x)
    c = [Fraction(float(v)) for v in COEFFS]

    def at(g):
        return x[g] if 0 <= g < n else x.dtype.type(0)

    out = np.zeros(n // 2, np.float32)
    for i in range(n // 2):
        v = _rn32(c[0] * Fraction(float(at(2 * i))))
        for t in range(1, 8):
            o = 2 * t - 1
            if x.dtype == np.int16:
                pair = Fraction(int(at(2 * i - o)) + int(at(2 * i + o)))
            else:
                pair = Fraction(float(np.float32(at(2 * i - o)) + np.float32(at(2 * i + o))))
            v = _rn32(c[t] * pair + Fraction(float(v)))
        out[i] = v
    return out


@pytest.mark.parametrize("n", [0, 1, 2, 3, 27, 28, 29, 200, 301])
def test_oracle_decimator_int16_exact(n):
    rng = np.random.default_rng(1000 + n)
    x = rng.integers(-32768, 32768, n).astype(np.int16)
    got = onative.decimate_half(x)
    want = _exact_decimate(x)
    assert got.shape == (n // 2,)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("n", [2, 31, 160])
def test_oracle_decimator_float32_exact(n):
    rng = np.random.default_rng(2000 + n)
    x = (rng.standard_normal(n) * 3000.0).astype(np.float32)
    x[::7] = np.float32(1e-3)   # mixed magnitudes: the pair sums round
    got = onative.decimate_half(x)
    want = _exact_decimate(x)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_oracle_decimator_is_a_unity_gain_half_band():
    # DC passes with the table's gain (1 + 4.6e-6); a tone at the source's
    # fs/4 (the decimated Nyquist) is halved; fs/8 passes
    dc = onative.decimate_half(np.full(400, 1000, np.int16))
    gain = float(COEFFS[0]) + 2 * float(np.sum(COEFFS[1:].astype(np.float64)))
    assert np.allclose(dc[10:-10], 1000 * gain, rtol=1e-6)
    k = np.arange(4000)
    quarter = onative.decimate_half((np.cos(np.pi / 2 * k) * 10000).astype(np.int16))
    assert np.allclose(quarter[10:-10], np.cos(np.pi * k[:2000][10:-10]) * 10000 * COEFFS[0], atol=0.5)
    eighth = (np.cos(np.pi / 4 * k) * 10000).astype(np.float32)
    y = onative.decimate_half(eighth)
    assert np.max(np.abs(y[10:-10] - eighth[::2][10:-10])) < 10000 * 2e-3
