"""Per-block VHS RF demodulation and block-stream stitching (test infrastructure).

Restates the managed ``exact`` VHS real-FFT path of
``RfDemodulator.DemodulateCore`` (Core/Dsp/RfDemodulator.cs:288-918) with
``useNumpyComplexVhsAnalytic`` set (Core/Decode/RfBlockDecodePipeline.cs:107):

* RF half-spectrum x RfVideo -> real inverse = band-passed RF (envelope source)
  (RfDemodulator.cs:396-478, 551);
* full complex FFT x RfVideo x Hilbert -> complex inverse = analytic signal
  (``BuildNumpyVhsComplexAnalyticSignal`` RfDemodulator.cs:1461-1536,
  ``PortedMath.BuildHilbertMultiplier`` PortedMath.cs:456-472);
* float32 polynomial-atan2 FM demod (PortedMath.cs:70-230, 519-551);
* diff-demod spike repair (RfDemodulator.cs:2527-2582, 966-1001);
* float32 envelope filtfilt (RfDemodulator.cs:1755-1839);
* demod real FFT x Video / x VideoLowPass05, real inverses, roll -32
  (RfDemodulator.cs:792-885);
* S-VHS sub-deemphasis of the video (``ApplySubDeemphasisRealCore``,
  RfDemodulator.cs:2852-2990, 3144-3220).

Stitching follows ``RfBlockStreamDecoder.ReadCore`` / ``CopyTrimmedWindow``
(Core/Decode/RfBlockStreamDecoder.cs:418-560, 1586-1610): block b reads RF
``[b*S, b*S+N)`` and contributes ``[cut, cut+S)`` to stream ``[b*S, b*S+S)``.
"""
import numpy as np

from . import native

BLOCK = 32768
CUT = 1024
CUT_END = 1024
STRIDE = BLOCK - CUT - CUT_END


def replace_spikes(demod, diffed, max_value, replace_start=8, replace_end=30):
    """``RfDemodulator.ReplaceSpikes`` (Core/Dsp/RfDemodulator.cs:966-1001)."""
    demod = np.asarray(demod, np.float64)
    to_fix = np.nonzero(demod > max_value)[0]
    n = len(demod)
    for i in to_fix:
        start = max(i - replace_start, 0)
        end = min(i + replace_end, n - 1)
        if start >= end:
            continue
        if np.max(diffed[start:end]) < np.max(demod[start:end]):
            demod[start:end] = diffed[start:end]
    return demod


def sub_deemphasis(video, video_spec, filters):
    """``ApplySubDeemphasisRealCore`` (Core/Dsp/RfDemodulator.cs:2852-2990)."""
    n = len(video)
    o = filters.sub
    high = np.fft.irfft(video_spec * filters.sub_highpass[: n // 2 + 1], n)
    # BuildAnalyticMagnitudeWithWorkspace (RfDemodulator.cs:3181-3220)
    spec = np.fft.fft(high)
    spec[1:n // 2] *= 2.0
    spec[n // 2 + 1:] = 0.0
    amp = np.abs(np.fft.ifft(spec))   # numpy's magnitude, as NumpyComplexMagnitude (:3222-3244)
    amp = amp / (o["deviation"] / 2.0)
    amp = native.filtfilt1_f64(amp, filters.sub_amp_b[0], filters.sub_amp_b[1], filters.sub_amp_a1)
    amp = np.maximum(0.0, amp)
    if o["scale1"] is not None:
        amp = amp * o["scale1"]
    amp = np.power(amp, o["exp"])
    if o["scale2"] is not None:
        amp = amp * o["scale2"]
    rate = o["logistic_rate"]
    if rate is not None and rate > 0.0:
        mid = o["logistic_mid"] if o["logistic_mid"] is not None else 0.0
        amp = amp * (1.0 / (1.0 + np.exp(-rate * (amp - mid))))
    static = o["static"] if o["static"] is not None else 0.0
    return video - ((high * (1.0 - amp)) + high * static)


def demod_block(x, filters, fs, diff_max, return_debug=False):
    """Demodulate one RF block; returns (video, video_lowpass, envelope, weak, debug)."""
    x = np.asarray(x, np.float64)
    n = len(x)
    h = n // 2 + 1
    rfv = filters.rf_video
    spec_half = np.fft.rfft(x)
    filtered_real = np.fft.irfft(spec_half * rfv[:h], n)
    hilbert = np.zeros(n)
    hilbert[0] = 1.0
    hilbert[n // 2] = 1.0
    hilbert[1:n // 2] = 2.0
    analytic = np.fft.ifft(np.fft.fft(x) * rfv * hilbert)
    demod = native.vhs_rust_demod(analytic.real, analytic.imag, fs)
    repaired = False
    if diff_max is not None and n > 40 and np.any(demod[20:n - 20] > diff_max):
        diffed = np.zeros(n, complex)
        diffed[1:] = analytic[1:] - analytic[:-1]
        demod_diffed = native.vhs_rust_demod(diffed.real, diffed.imag, fs)
        demod = replace_spikes(demod, demod_diffed, diff_max)
        repaired = True
    envelope = native.vhs_envelope(filtered_real, filters.env_b[0], filters.env_b[1], filters.env_a1)
    weak = bool(np.any(envelope == 0.0))
    dspec = np.fft.rfft(demod)
    vspec = dspec * filters.video[:h]
    video = np.fft.irfft(vspec, n)
    if getattr(filters, "sub", None) is not None:
        video = sub_deemphasis(video, vspec, filters)
    vlp = np.fft.irfft(dspec * filters.video_lp05[:h], n)
    vlp = np.roll(vlp, -filters.video_lp05_offset)
    dbg = None
    if return_debug:
        dbg = {"analytic": analytic, "demod": demod, "filtered_real": filtered_real,
               "repaired": repaired}
    return video, vlp, envelope, weak, dbg


def unwrap_conjugate_product(z, fs):
    """``PortedMath.UnwrapHilbertConjugateProduct`` (Core/Dsp/PortedMath.cs:38-68): binary64
    atan2 of z[i]·conj(z[i-1]), wrapped into [0, 2π), times fs/2π; output[0] = 0."""
    z = np.asarray(z, np.complex128)
    out = np.zeros(len(z))
    if len(z) < 2:
        return out
    cr, ci = z.real[1:], z.imag[1:]
    pr, pi = z.real[:-1], z.imag[:-1]
    re = (cr * pr) + (ci * pi)
    im = (ci * pr) - (cr * pi)
    d = np.arctan2(im, re)
    d = np.where(d < 0.0, d + 2.0 * np.pi, d)
    out[1:] = d * (fs / (2.0 * np.pi))
    return out


def clip_demod_for_video(demod, fs):
    """``RfDemodulator.ClipDemodForVideo`` (Core/Dsp/RfDemodulator.cs:1891-1901)."""
    return np.clip(np.asarray(demod, np.float64), 1_500_000.0, fs * 0.75)


def demod_block_complex(x, rf_video, video_filter, video_lp, fs, video_lp_offset=0,
                        rf_mtf=None, clip_for_video=False):
    """The full-spectrum (non-VHS, conjugate-product) branch of ``RfDemodulator.DemodulateCore``
    (Core/Dsp/RfDemodulator.cs:564-605, 756, 779-784, 814-833, 858-874): complex FFT of the
    block × RfVideo (× MTF) × Hilbert → inverse = analytic; FP64 conjugate-product FM demod;
    envelope |analytic|; video and sync reference as real parts of complex-spectrum inverses;
    the sync reference rolled by −offset.  Returns (video, demod_raw, analytic, envelope, vlp)."""
    x = np.asarray(x, np.float64)
    n = len(x)
    spec = np.fft.fft(x) * np.asarray(rf_video, np.complex128)
    if rf_mtf is not None:
        spec = spec * np.asarray(rf_mtf, np.complex128)
    hilbert = np.zeros(n)
    hilbert[0] = 1.0
    if n % 2 == 0:
        hilbert[n // 2] = 1.0
        hilbert[1:n // 2] = 2.0
    else:
        hilbert[1:(n + 1) // 2] = 2.0
    analytic = np.fft.ifft(spec * hilbert)
    demod_raw = unwrap_conjugate_product(analytic, fs)
    envelope = np.abs(analytic)
    source = clip_demod_for_video(demod_raw, fs) if clip_for_video else demod_raw
    dspec = np.fft.fft(source)
    video = np.fft.ifft(dspec * np.asarray(video_filter, np.complex128)).real
    vlp = np.fft.ifft(dspec * np.asarray(video_lp, np.complex128)).real
    if video_lp_offset:
        vlp = np.roll(vlp, -video_lp_offset)
    return video, demod_raw, analytic, envelope, vlp


def stitch_span(rf, block_fn, block_len, cut, cut_end, begin, length):
    """Overlap-save read of stream samples [begin, begin+length) (``RfBlockStreamDecoder.ReadCore`` /
    ``CopyTrimmedWindow``, Core/Decode/RfBlockStreamDecoder.cs:418-560, 1586-1610).

    Block b processes RF [b·S, b·S+N) with S = N − cut − cut_end and contributes its samples
    [cut, cut+S) to stream [b·S, b·S+S), so stream sample s is block-local sample
    s − b·S + cut and lines up with RF sample s + cut.  ``block_fn`` maps one RF block to a tuple
    of equal-length channels; returns the stitched channels."""
    stride = block_len - cut - cut_end
    first = begin // stride
    last = (begin + length - 1) // stride
    out = None
    for b in range(first, last + 1):
        chans = block_fn(np.asarray(rf[b * stride: b * stride + block_len], np.float64))
        if out is None:
            out = [np.empty(length) for _ in chans]
        lo = max(begin, b * stride)
        hi = min(begin + length, (b + 1) * stride)
        for o, c in zip(out, chans):
            o[lo - begin:hi - begin] = c[lo - b * stride + cut: hi - b * stride + cut]
    return out


def block_count(total_samples):
    """Number of whole 32768-sample blocks a capture of ``total_samples`` RF samples holds."""
    if total_samples < BLOCK:
        return 0
    return (total_samples - BLOCK) // STRIDE + 1


def demod_stream(rf, filters, fs, diff_max, first_block=0, nblocks=None):
    """Stitched stream channels for blocks ``first_block..first_block+nblocks``.

    Stream sample d corresponds to RF sample d + CUT.
    """
    total = block_count(len(rf))
    if nblocks is None:
        nblocks = total - first_block
    video = np.empty(nblocks * STRIDE)
    vlp = np.empty(nblocks * STRIDE)
    env = np.empty(nblocks * STRIDE)
    weak = False
    for j in range(nblocks):
        b = first_block + j
        x = rf[b * STRIDE: b * STRIDE + BLOCK].astype(np.float64)
        v, l, e, w, _ = demod_block(x, filters, fs, diff_max)
        sl = slice(j * STRIDE, (j + 1) * STRIDE)
        video[sl] = v[CUT:CUT + STRIDE]
        vlp[sl] = l[CUT:CUT + STRIDE]
        env[sl] = e[CUT:CUT + STRIDE]
        weak |= w
    return video, vlp, env, weak
