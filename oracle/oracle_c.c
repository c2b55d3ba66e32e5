/*
 * CPU oracle kernels for the VHS RF decode path -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain C restatements of the sequential, bit-sensitive loops of the
 * reference's managed `exact` backend (vhs-decode-dotnet, VHSDecode.Core).
 * They are called from oracle/*.py through ctypes; the product library never
 * links or calls this file.  Every float expression keeps the reference's
 * evaluation order and is compiled with -ffp-contract=off so no FMA is
 * introduced where the reference has none.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

/* PortedMath.VhsRustAtan2Approximation (Core/Dsp/PortedMath.cs:519-544). */
static float vhs_rust_atan2(float y, float x)
{
    const float min_normal = 1.17549435E-38f;
    x += copysignf(min_normal, x);
    int swap = fabsf(x) < fabsf(y);
    float in = swap ? x / y : y / x;
    float sq = in * in;
    float r = in * (0.99997726f + (sq * (-0.33262347f + (sq * (0.19354346f
              + (sq * (-0.11643287f + (sq * (0.05265332f + (sq * -0.01172120f))))))))));
    const float pi = 3.14159274f;
    float half_pi = in >= 0.0f ? pi / 2.0f : -pi / 2.0f;
    r = swap ? half_pi - r : r;
    int xp = x >= 0.0f, yp = y >= 0.0f;
    if (xp && yp) return r;
    if (!xp && yp) return pi + r;
    if (!xp && !yp) return -pi + r;
    return r;
}

/* PortedMath.VhsRustFrequencyDifference (Core/Dsp/PortedMath.cs:546-551). */
static float vhs_rust_freq_diff(float cur, float prev, float freq)
{
    const float tau = 6.28318548f;
    float d = cur - prev;
    d -= floorf(d / tau) * tau;
    return (d * freq) / tau;
}

/* UnwrapHilbertVhsRustApproximation scalar form (PortedMath.cs:114-230). */
void oracle_vhs_rust_demod(const double *re, const double *im, int64_t n,
                           double fs, double *out)
{
    if (n <= 0) return;
    float freq = (float)fs;
    float prev = vhs_rust_atan2((float)im[0], (float)re[0]);
    out[0] = 0.0;
    for (int64_t i = 1; i < n; i++) {
        float cur = vhs_rust_atan2((float)im[i], (float)re[i]);
        out[i] = (double)vhs_rust_freq_diff(cur, prev, freq);
        prev = cur;
    }
}

/* Angles only (used by the tests that check the device atan2 bit-exactly). */
void oracle_vhs_rust_angles(const float *re, const float *im, int64_t n, float *out)
{
    for (int64_t i = 0; i < n; i++) out[i] = vhs_rust_atan2(im[i], re[i]);
}

/*
 * RfDemodulator.BuildVhsEnvelope (Core/Dsp/RfDemodulator.cs:1755-1839):
 * raw[n] = |float(filtered[n-4])| (circular roll by +4), then
 * SosFilter.ApplyForwardBackwardFloat32 (Core/Dsp/SosFilter.cs:300-540, 924-950,
 * 1034-1064) with one first-order section: odd extension of 6 samples,
 * steady-state zi scaled by the first / last extended value, float32 DF2T.
 * `work` must hold n + 12 floats.
 */
/* RfDemodulator.BuildVhsRawEnvelope / FillVhsRawEnvelope (Core/Dsp/RfDemodulator.cs:1784-1839):
 * raw[(i + 4) mod n] = |float(filtered[i])|. */
void oracle_vhs_raw_envelope(const double *filtered, int64_t n, float *raw)
{
    if (n <= 0) return;
    int64_t shift = 4 % n;
    int64_t split = n - shift;
    for (int64_t i = 0; i < split; i++) raw[i + shift] = fabsf((float)filtered[i]);
    for (int64_t w = split; w < n; w++) raw[w - split] = fabsf((float)filtered[w]);
}

void oracle_vhs_envelope(const double *filtered, int64_t n, double b0d, double b1d,
                         double a1d, double *out, float *work)
{
    const int edge = 6;
    float *ext = work;
    float *raw = work + edge;  /* raw occupies ext[edge .. edge+n) */
    oracle_vhs_raw_envelope(filtered, n, raw);
    /* odd extension (float32 form reading the float raw values) */
    float first = raw[0];
    float tmp_left[6], tmp_right[6];
    for (int i = 0; i < edge; i++) tmp_left[i] = (2.0f * first) - raw[edge - i];
    float last = raw[n - 1];
    for (int i = 0; i < edge; i++) tmp_right[i] = (2.0f * last) - raw[n - 2 - i];
    for (int i = 0; i < edge; i++) ext[i] = tmp_left[i];
    for (int i = 0; i < edge; i++) ext[edge + n + i] = tmp_right[i];
    int64_t len = n + 2 * edge;
    float b0 = (float)b0d, b1 = (float)b1d, b2 = 0.0f, a1 = (float)a1d, a2 = 0.0f;
    /* SteadyStateInitialConditionsFloat32 for one section */
    float first_term = b1 - (a1 * b0);
    float second_term = b2 - (a2 * b0);
    float num = (0.0f + first_term) + second_term;
    float den = (1.0f + a1) + a2;
    float zi0 = num / den;
    float zi1 = ((1.0f + a1) * zi0) - first_term;
    float scale = 1.0f;
    zi0 = scale * zi0;
    zi1 = scale * zi1;
    /* forward */
    float z1 = zi0 * ext[0], z2 = zi1 * ext[0];
    for (int64_t s = 0; s < len; s++) {
        float v = ext[s];
        float f = (b0 * v) + z1;
        z1 = (b1 * v) - (a1 * f) + z2;
        z2 = (b2 * v) - (a2 * f);
        ext[s] = f;
    }
    /* backward */
    z1 = zi0 * ext[len - 1];
    z2 = zi1 * ext[len - 1];
    for (int64_t s = len - 1; s >= 0; s--) {
        float v = ext[s];
        float f = (b0 * v) + z1;
        z1 = (b1 * v) - (a1 * f) + z2;
        z2 = (b2 * v) - (a2 * f);
        ext[s] = f;
    }
    for (int64_t i = 0; i < n; i++) out[i] = (double)ext[edge + i];
}

/*
 * SosFilter.ApplyForwardBackward (Core/Dsp/SosFilter.cs:178-232, 281-298,
 * 540-570, 972-1001) for one first-order section (b0, b1, 0; 1, a1, 0), in
 * binary64: odd extension of 6 samples, steady-state zi scaled by the first /
 * last extended value, direct form II transposed forward then backward.
 * `work` must hold n + 12 doubles.  Used for the sub-deemphasis amplitude.
 */
void oracle_filtfilt1_f64(const double *x, int64_t n, double b0, double b1, double a1,
                          double *out, double *work)
{
    const int edge = 6;
    double *ext = work;
    double first = x[0], last = x[n - 1];
    for (int i = 0; i < edge; i++) ext[i] = (2.0 * first) - x[edge - i];
    for (int64_t i = 0; i < n; i++) ext[edge + i] = x[i];
    for (int i = 0; i < edge; i++) ext[edge + n + i] = (2.0 * last) - x[n - 2 - i];
    int64_t len = n + 2 * edge;
    double b2 = 0.0, a2 = 0.0;
    double first_term = b1 - (a1 * b0);
    double second_term = b2 - (a2 * b0);
    double num = (0.0 + first_term) + second_term;
    double den = (1.0 + a1) + a2;
    double zi0 = num / den;
    double zi1 = ((1.0 + a1) * zi0) - first_term;
    double z1 = zi0 * ext[0], z2 = zi1 * ext[0];
    for (int64_t s = 0; s < len; s++) {
        double v = ext[s];
        double f = (b0 * v) + z1;
        z1 = (b1 * v) - (a1 * f) + z2;
        z2 = (b2 * v) - (a2 * f);
        ext[s] = f;
    }
    z1 = zi0 * ext[len - 1];
    z2 = zi1 * ext[len - 1];
    for (int64_t s = len - 1; s >= 0; s--) {
        double v = ext[s];
        double f = (b0 * v) + z1;
        z1 = (b1 * v) - (a1 * f) + z2;
        z2 = (b2 * v) - (a2 * f);
        ext[s] = f;
    }
    for (int64_t i = 0; i < n; i++) out[i] = ext[edge + i];
}

/*
 * PulseDetection.FindPulsesScalar (Core/Dsp/PulseDetection.cs:186-222).
 * Returns the pulse count (capped at `cap`, the true count is still returned).
 */
int64_t oracle_find_pulses(const double *ref, int64_t n, double high, int64_t min_len,
                           int64_t max_len, int64_t *starts, int64_t *lens, int64_t cap)
{
    if (n <= 0) return 0;
    int in_pulse = ref[0] <= high;
    int64_t cur = 0, count = 0;
    for (int64_t p = 0; p < n; p++) {
        double v = ref[p];
        if (in_pulse) {
            if (v > high) {
                int64_t len = p - cur;
                if (len >= min_len && len <= max_len && cur != 0) {
                    if (count < cap) { starts[count] = cur; lens[count] = len; }
                    count++;
                }
                in_pulse = 0;
            }
        } else if (v <= high) {
            cur = p;
            in_pulse = 1;
        }
    }
    return count;
}

/*
 * TbcLineResampler.SampleSinc (Core/Tbc/TbcLineResampler.cs:1167-1234):
 * float32 coordinate, 65536-phase x 16-tap LUT rows blended with a float FMA,
 * float products accumulated in double, new tap as the left operand.
 */
static double sample_sinc(const double *src, int64_t n, double position, const float *lut)
{
    if (!isfinite(position)) return 0.0;
    const int taps = 16, phases = 65536;
    float coord = (float)position;
    int coord_int = (int)coord;
    float fraction = coord - (float)coord_int;
    float phase_pos = fraction * (float)phases;
    int ps = (int)phase_pos;
    int pe = ps + 1;
    float alpha = phase_pos - (float)ps;
    if (ps < 0) ps += phases + 1;
    if (ps < 0) ps = 0; if (ps > phases) ps = phases;
    if (pe < 0) pe += phases + 1;
    if (pe < 0) pe = 0; if (pe > phases) pe = phases;
    const float *ws = lut + (int64_t)ps * taps;
    const float *we = lut + (int64_t)pe * taps;
    int sample_start = coord_int - (taps / 2 - 1);
    double result = 0.0;
    int interior = n >= taps && (uint32_t)sample_start <= (uint32_t)(n - taps);
    for (int t = 0; t < taps; t++) {
        float sw = ws[t];
        float w = fmaf(alpha, we[t] - sw, sw);
        int64_t idx = (int64_t)sample_start + t;
        if (!interior) {
            if (idx < 0) idx += n;
            if (idx < 0) idx = 0;
            if (idx > n - 1) idx = n - 1;
        }
        float prod = (float)src[idx] * w;
        result = (double)prod + result;
    }
    return result;
}

void oracle_sinc_resample(const double *src, int64_t n, const double *positions,
                          const double *level, int64_t count, const float *lut, double *out)
{
    for (int64_t i = 0; i < count; i++)
        out[i] = (double)(float)(sample_sinc(src, n, positions[i], lut) * level[i]);
}

/* VideoOutputConverter.FastMathConversion.Convert (Core/Tbc/VideoOutputConverter.cs:9-40). */
void oracle_hz_to_u16(const double *in, int64_t count, double ire0, double output_scale,
                      double hz_ire, double output_zero, double vsync_ire, uint16_t *out)
{
    double inv = 1.0 / hz_ire;
    double offset = (output_zero + 0.5) - (vsync_ire * output_scale);
    for (int64_t i = 0; i < count; i++) {
        double scaled = output_scale * (in[i] - ire0);
        double v = fma(scaled, inv, offset);
        out[i] = v <= 0.0 ? 0 : (v >= 65535.0 ? 65535 : (uint16_t)v);
    }
}

/* Kaiser-windowed sinc LUT: TbcLineResampler.BuildKaiserSincLookup (TbcLineResampler.cs:1297-1330). */
static double bessel_i0(double x)
{
    double sum = 1.0, y = (x * x) / 4.0, term = 1.0;
    for (int k = 1; k < 100; k++) {
        term *= y / ((double)k * (double)k);
        double next = sum + term;
        if (next == sum) break;
        sum = next;
    }
    return sum;
}

void oracle_build_sinc_lut(float *lut)
{
    const int taps = 16, phases = 65536, half = 8;
    const double beta = 5.0;
    double i0b = bessel_i0(beta);
    const double pi = 3.14159265358979323846;
    double w[16];
    for (int p = 0; p < phases; p++) {
        double phase = (double)p / phases, sum = 0.0;
        for (int t = 0; t < taps; t++) {
            double x = (double)((half - 1) - t) + phase;
            double s = x == 0.0 ? 1.0 : sin(pi * x) / (pi * x);
            double r = x / half;
            double kw = (r < -1.0 || r > 1.0) ? 0.0 : bessel_i0(beta * sqrt(1.0 - (r * r))) / i0b;
            w[t] = s * kw;
            sum += w[t];
        }
        for (int t = 0; t < taps; t++) lut[(int64_t)p * taps + t] = (float)(w[t] / sum);
    }
    memcpy(lut + (int64_t)phases * taps, lut + (int64_t)(phases - 1) * taps, taps * sizeof(float));
}

/* TbcLineResampler.SmoothLevelAdjusts (Core/Tbc/TbcLineResampler.cs:997-1011). */
void oracle_smooth_levels(double *la, int64_t n, double alpha)
{
    for (int64_t i = 1; i < n; i++) {
        double prev = la[i - 1];
        la[i] = fma(la[i] - prev, alpha, prev);
    }
}

/*
 * RfDropoutDetector.FindDropouts (Core/Decode/TbcDropoutMapping.cs:52-107).
 * Writes raw [start,end) pairs before the minimum-length filter; returns the
 * count of ranges that pass `end - start > min_len`.
 */
int64_t oracle_find_dropouts(const double *env, int64_t start, int64_t end, double thr, double hyst,
                             int64_t merge, int64_t min_len, int64_t *out_start, int64_t *out_end,
                             int64_t cap)
{
    double down = thr, up = thr * hyst;
    int64_t n = 0;          /* raw ranges */
    int64_t idx = -1;
    int64_t rs_cap = cap;
    /* raw ranges are staged in the output arrays then compacted */
    for (int64_t i = start; i < end; i++) {
        double v = env[i];
        if (v <= down) {
            int ended = idx >= 0 && out_end[idx] != -1 && i - out_end[idx] > merge;
            if (idx == -1 || ended) {
                idx++;
                if (idx >= rs_cap) return -1;
                out_start[idx] = i;
                out_end[idx] = -1;
                n = idx + 1;
            }
        } else if (v >= up && idx != -1 && out_end[idx] == -1) {
            out_end[idx] = i;
        }
    }
    if (idx != -1 && out_end[idx] == -1) out_end[idx] = end;
    int64_t k = 0;
    for (int64_t j = 0; j < n; j++) {
        if (out_end[j] - out_start[j] > min_len) {
            out_start[k] = out_start[j];
            out_end[k] = out_end[j];
            k++;
        }
    }
    return k;
}

/* 2:1 decimation of the cuda-fast reader's 20-MSPS mode
 * (src/VHSDecode.CudaFast.Native/src/cuda_fast_decimator.cu:27-64, window
 * :67-100 over one window that covers the capture): y[i] is the half-band FIR
 * centred on source sample 2 i, sources outside [0, n) read as zero, n / 2
 * outputs.  The reference's `value += c * (a + b)` runs on the GPU, where
 * nvcc's default -fmad=true contracts it: the oracle writes that fused
 * multiply-add out with fmaf.  The filter table is the reference's. */
static const float half_band[8] = {
    0.5000046374907835f,    0.3126333216205309f,    -0.09010692207961689f,  0.040107417651266825f,
    -0.017917030421899405f, 0.007100857132041433f,  -0.0022302855185240434f, 0.00041032287080936366f};

static float dec_at_s16(const int16_t *x, int64_t n, int64_t g) { return (g >= 0 && g < n) ? (float)x[g] : 0.0f; }
static float dec_at_f32(const float *x, int64_t n, int64_t g) { return (g >= 0 && g < n) ? x[g] : 0.0f; }

void oracle_decimate_half_s16(const int16_t *x, int64_t n, float *out)
{
    for (int64_t i = 0; i < n / 2; i++) {
        int64_t c = 2 * i;
        float v = half_band[0] * dec_at_s16(x, n, c);
        for (int t = 1; t < 8; t++) {
            int64_t o = 2 * t - 1;
            float pair = dec_at_s16(x, n, c - o) + dec_at_s16(x, n, c + o);
            v = fmaf(half_band[t], pair, v);
        }
        out[i] = v;
    }
}

void oracle_decimate_half_f32(const float *x, int64_t n, float *out)
{
    for (int64_t i = 0; i < n / 2; i++) {
        int64_t c = 2 * i;
        float v = half_band[0] * dec_at_f32(x, n, c);
        for (int t = 1; t < 8; t++) {
            int64_t o = 2 * t - 1;
            float pair = dec_at_f32(x, n, c - o) + dec_at_f32(x, n, c + o);
            v = fmaf(half_band[t], pair, v);
        }
        out[i] = v;
    }
}

/*
 * SosFilter.ApplyForwardBackwardFloat32 (Core/Dsp/SosFilter.cs:369-398,
 * 502-538, 583-708, 710-833, 924-970, 1034-1060): float32 forward-backward
 * cascade of `nsec` second-order sections over an odd extension of `edge`
 * samples.  The coefficients are the binary64 sections cast to float; the
 * steady-state initial conditions are computed in float and scaled by the
 * first (forward) and last (backward) extended value; each section is the
 * transposed direct form II with one rounding per operation, in the
 * reference's operand order.  `work` holds n + 2*edge floats.
 */
void oracle_sosfiltfilt_f32(const double *x, int64_t n, const double *sos, int nsec, int64_t edge,
                            float *out, float *work)
{
    float b0[32], b1[32], b2[32], a0[32], a1[32], a2[32], zi[64], z[64];
    int64_t len = n + 2 * edge;
    float *ext = work;
    float first = (float)x[0], last = (float)x[n - 1];
    for (int64_t i = 0; i < edge; i++) ext[i] = (2.0f * first) - (float)x[edge - i];
    for (int64_t i = 0; i < n; i++) ext[edge + i] = (float)x[i];
    for (int64_t i = 0; i < edge; i++) ext[edge + n + i] = (2.0f * last) - (float)x[n - 2 - i];
    float scale = 1.0f;
    for (int s = 0; s < nsec; s++) {
        b0[s] = (float)sos[6 * s + 0]; b1[s] = (float)sos[6 * s + 1]; b2[s] = (float)sos[6 * s + 2];
        a0[s] = (float)sos[6 * s + 3]; a1[s] = (float)sos[6 * s + 4]; a2[s] = (float)sos[6 * s + 5];
        float ft = b1[s] - (a1[s] * b0[s]);
        float st = b2[s] - (a2[s] * b0[s]);
        float num = (0.0f + ft) + st;
        float den = (1.0f + a1[s]) + a2[s];
        float z0 = num / den;
        float z1 = ((1.0f + a1[s]) * z0) - ft;
        zi[2 * s] = scale * z0;
        zi[2 * s + 1] = scale * z1;
        float ndc = ((0.0f + b0[s]) + b1[s]) + b2[s];
        float ddc = ((0.0f + a0[s]) + a1[s]) + a2[s];
        scale *= ndc / ddc;
    }
    for (int pass = 0; pass < 2; pass++) {
        float x0 = pass == 0 ? ext[0] : ext[len - 1];
        for (int k = 0; k < 2 * nsec; k++) z[k] = zi[k] * x0;
        for (int64_t t = 0; t < len; t++) {
            int64_t i = pass == 0 ? t : len - 1 - t;
            float v = ext[i];
            for (int s = 0; s < nsec; s++) {
                float f = (b0[s] * v) + z[2 * s];
                z[2 * s] = ((b1[s] * v) - (a1[s] * f)) + z[2 * s + 1];
                z[2 * s + 1] = (b2[s] * v) - (a2[s] * f);
                v = f;
            }
            ext[i] = v;
        }
    }
    for (int64_t i = 0; i < n; i++) out[i] = ext[edge + i];
}

/*
 * SosFilter.ApplyForwardBackward (Core/Dsp/SosFilter.cs:178-298, 547-581,
 * 90-176, 972-1001) in binary64: odd extension, steady-state zi scaled by the
 * first sample, forward, reverse, forward again with zi scaled by the new
 * first sample, reverse.  `work` holds n + 2*edge doubles.
 */
void oracle_sosfiltfilt_f64(const double *x, int64_t n, const double *sos, int nsec, int64_t edge,
                            double *out, double *work)
{
    double zi[64], z[64];
    int64_t len = n + 2 * edge;
    double *ext = work;
    double first = x[0], last = x[n - 1];
    for (int64_t i = 0; i < edge; i++) ext[i] = (2.0 * first) - x[edge - i];
    for (int64_t i = 0; i < n; i++) ext[edge + i] = x[i];
    for (int64_t i = 0; i < edge; i++) ext[edge + n + i] = (2.0 * last) - x[n - 2 - i];
    double scale = 1.0;
    for (int s = 0; s < nsec; s++) {
        const double *c = sos + 6 * s;
        double ft = c[1] - (c[4] * c[0]);
        double st = c[2] - (c[5] * c[0]);
        double num = (0.0 + ft) + st;
        double den = (1.0 + c[4]) + c[5];
        double z0 = num / den;
        double z1 = ((1.0 + c[4]) * z0) - ft;
        zi[2 * s] = scale * z0;
        zi[2 * s + 1] = scale * z1;
        double ndc = ((0.0 + c[0]) + c[1]) + c[2];
        double ddc = ((0.0 + c[3]) + c[4]) + c[5];
        scale *= ndc / ddc;
    }
    for (int pass = 0; pass < 2; pass++) {
        double x0 = pass == 0 ? ext[0] : ext[len - 1];
        for (int k = 0; k < 2 * nsec; k++) z[k] = zi[k] * x0;
        for (int64_t t = 0; t < len; t++) {
            int64_t i = pass == 0 ? t : len - 1 - t;
            double v = ext[i];
            for (int s = 0; s < nsec; s++) {
                const double *c = sos + 6 * s;
                double f = (c[0] * v) + z[2 * s];
                z[2 * s] = ((c[1] * v) - (c[4] * f)) + z[2 * s + 1];
                z[2 * s + 1] = (c[2] * v) - (c[5] * f);
                v = f;
            }
            ext[i] = v;
        }
    }
    for (int64_t i = 0; i < n; i++) out[i] = ext[edge + i];
}

/*
 * VhsChromaDecoder.MeanFloat32FastMath (Core/Decode/VhsChromaDecoder.cs:3709-3791):
 * 32 float accumulators (8 lanes x 4 interleaved groups) each summing every
 * 32nd value in order, the groups folded pairwise, the 8 lanes folded as a
 * tree, divided by the count.
 */
float oracle_mean_f32_fast(const float *v, int64_t n)
{
    float acc[32] = {0};
    for (int64_t i = 0; i < n; i++) acc[i & 31] += v[i];
    float lanes[8];
    for (int l = 0; l < 8; l++) lanes[l] = (acc[l] + acc[8 + l]) + (acc[16 + l] + acc[24 + l]);
    for (int c = 8; c > 1; c /= 2)
        for (int l = 0; l < c / 2; l++) lanes[l] += lanes[l + c / 2];
    return lanes[0] / (float)n;
}

/*
 * VhsChromaDecoder.BuildHeterodyneTable (Core/Decode/VhsChromaDecoder.cs:1967-2007)
 * for one phase: (double)(float)-cos((tau * scale) * i + offset).
 */
void oracle_chroma_heterodyne(int64_t n, double het_scale, double phase_offset, double *out)
{
    const double tau = 6.283185307179586;
    double step = tau * het_scale;
    for (int64_t i = 0; i < n; i++) out[i] = (double)(float)(-cos((step * (double)i) + phase_offset));
}

/*
 * VhsChromaDecoder.NumpyTrigFloat32 (Core/Decode/VhsChromaDecoder.cs:3830-3893):
 * NumPy's float32 sin/cos (a three-part Cody-Waite reduction by pi/2 and
 * minimax polynomials evaluated with fused multiply-adds; libm beyond the
 * reduction's range), as the reference restates it.
 */
static float bits_f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

static float numpy_trig_f32(float x, int want_cos)
{
    if (isnan(x)) return NAN;
    float maxcw = want_cos ? 71476.0625f : 117435.992f;
    if (fabsf(x) > maxcw) return want_cos ? cosf(x) : sinf(x);
    float q = x * bits_f(0x3F22F983u);
    const float magic = 12582912.0f;
    q = (q + magic) - magic;
    float r = fmaf(q, bits_f(0xBFC90FD8u), x);
    r = fmaf(q, bits_f(0xB4A8885Au), r);
    r = fmaf(q, bits_f(0xA7C234C4u), r);
    float r2 = r * r;
    float c = fmaf(bits_f(0x37CC730Bu), r2, bits_f(0xBAB6036Eu));
    c = fmaf(c, r2, bits_f(0x3D2AAA9Eu));
    c = fmaf(c, r2, -0.5f);
    c = fmaf(c, r2, 1.0f);
    float s = fmaf(bits_f(0x363E9DDEu), r2, bits_f(0xB95035DDu));
    s = fmaf(s, r2, bits_f(0x3C0888CDu));
    s = fmaf(s, r2, -1.0f / 6.0f);
    s = fmaf(s, r2, 0.0f);
    s = fmaf(s, r, r);
    int iq = (int)rintf(q);
    if (want_cos) iq++;
    float res = (iq & 1) == 0 ? s : c;
    return (iq & 2) != 0 ? -res : res;
}

/* VhsChromaDecoder.BuildCarrierTables (Core/Decode/VhsChromaDecoder.cs:3793-3828). */
void oracle_chroma_carrier(int64_t n, double wave_scale, double *sin_out, double *cos_out)
{
    const double tau = 6.283185307179586;
    for (int64_t i = 0; i < n; i++) {
        float theta = (float)((tau * wave_scale) * (double)i);
        sin_out[i] = numpy_trig_f32(theta, 0);
        cos_out[i] = numpy_trig_f32(theta, 1);
    }
}

static double positive_degrees(double d)
{
    double r = fmod(d, 360.0);
    return r < 0.0 ? r + 360.0 : r;
}

/*
 * VhsChromaDecoder.DemodBurstValue / DemodBurstFloat32
 * (Core/Decode/VhsChromaDecoder.cs:1438-1629): I/Q of the burst against the
 * carrier tables (already offset to the burst start) in the reference's
 * lane and summation order, then the phase, the line-scale phase offset,
 * libm hypot, I and Q into out[0..4].
 */
void oracle_chroma_burst_value(const double *burst, int64_t n, const double *bsin, const double *bcos,
                               int f32, double line_scale, int64_t start_minus_line, double *out)
{
    double ic, qc;
    if (!f32) {
        double iF[4] = {0}, iS[4] = {0}, qF[4] = {0}, qS[4] = {0};
        int64_t vl = n & ~(int64_t)7;
        for (int64_t k = 0; k < vl; k += 8)
            for (int l = 0; l < 4; l++) {
                int64_t a = k + l, b = a + 4;
                iF[l] = fma(burst[a], (double)(float)bcos[a], iF[l]);
                iS[l] = fma(burst[b], (double)(float)bcos[b], iS[l]);
                qF[l] = fma(burst[a], (double)(float)bsin[a], qF[l]);
                qS[l] = fma(burst[b], (double)(float)bsin[b], qS[l]);
            }
        double i0 = iS[0] + iF[0], i1 = iS[1] + iF[1], i2 = iS[2] + iF[2], i3 = iS[3] + iF[3];
        double q0 = qS[0] + qF[0], q1 = qS[1] + qF[1], q2 = qS[2] + qF[2], q3 = qS[3] + qF[3];
        ic = (i0 + i2) + (i1 + i3);
        qc = (q0 + q2) + (q1 + q3);
        for (int64_t k = vl; k < n; k++) {
            ic = fma(burst[k], (double)(float)bcos[k], ic);
            qc = fma(burst[k], (double)(float)bsin[k], qc);
        }
    } else {
        double I[4][4] = {{0}}, Q[4][4] = {{0}};
        int64_t main_end = n & ~(int64_t)15;
        for (int64_t k = 0; k < main_end; k += 16)
            for (int l = 0; l < 4; l++)
                for (int g = 0; g < 4; g++) {
                    int64_t idx = k + l + 4 * g;
                    float s = (float)burst[idx];
                    float ip = s * (float)bcos[idx];
                    float qp = s * (float)bsin[idx];
                    I[g][l] += ip;
                    Q[g][l] += qp;
                }
        double li[4], lq[4];
        for (int l = 0; l < 4; l++) {
            li[l] = ((I[1][l] + I[0][l]) + I[2][l]) + I[3][l];
            lq[l] = ((Q[1][l] + Q[0][l]) + Q[2][l]) + Q[3][l];
        }
        ic = (li[0] + li[2]) + (li[1] + li[3]);
        qc = (lq[0] + lq[2]) + (lq[1] + lq[3]);
        int64_t epi_end = n & ~(int64_t)3;
        if (epi_end > main_end) {
            double ei[4] = {ic, 0, 0, 0}, eq[4] = {qc, 0, 0, 0};
            for (int64_t k = main_end; k < epi_end; k += 4)
                for (int l = 0; l < 4; l++) {
                    float s = (float)burst[k + l];
                    float ip = s * (float)bcos[k + l];
                    float qp = s * (float)bsin[k + l];
                    ei[l] += ip;
                    eq[l] += qp;
                }
            ic = (ei[0] + ei[2]) + (ei[1] + ei[3]);
            qc = (eq[0] + eq[2]) + (eq[1] + eq[3]);
        }
        for (int64_t k = epi_end; k < n; k++) {
            float s = (float)burst[k];
            float ip = s * (float)bcos[k];
            float qp = s * (float)bsin[k];
            ic += ip;
            qc += qp;
        }
    }
    out[0] = positive_degrees(atan2(qc, ic) * (180.0 / 3.141592653589793));
    out[1] = positive_degrees((double)start_minus_line * fma(-line_scale, 90.0, 90.0));
    out[2] = hypot(ic, qc);
    out[3] = ic;
    out[4] = qc;
}

/*
 * VhsChromaDecoder.UpconvertChromaPhaseCompensated
 * (Core/Decode/VhsChromaDecoder.cs:2167-2248): NTSC up-conversion, one line
 * per phase entry, theta advanced in four lanes as the reference does.
 */
void oracle_chroma_upconvert_ntsc(const double *chroma, int64_t n, int64_t line_offset, int64_t line_length,
                                  const int64_t *line_numbers, const int64_t *rotations,
                                  const double *burst_phases, int64_t count, double cu_hz, double fsc_mhz,
                                  double target_even, double target_odd, double *out)
{
    const double half_pi = 1.5707963267948966;
    const double deg = 0.017453292519943295;
    const double hpm = 1.5707963267948965e-6;
    double carrier_term = cu_hz * hpm;
    double ratio = carrier_term / fsc_mhz;
    double h = ratio + half_pi;
    double h2 = h * 2.0, h3 = h * 3.0, h4 = h * 4.0;
    for (int64_t i = 0; i < n; i++) out[i] = 0.0;
    for (int64_t e = 0; e < count; e++) {
        int64_t ls = (line_numbers[e] - line_offset) * line_length;
        int64_t le = ls + line_length;
        double target = line_numbers[e] % 2 == 0 ? target_even : target_odd;
        double theta = fma((double)ls, h, (double)rotations[e] * half_pi);
        theta = fma(target + burst_phases[e], deg, theta);
        if (ls < 0 || le > n) {
            for (int64_t k = ls; k < le; k++) {
                int64_t idx = k < 0 ? k + n : k;
                out[idx] = (double)(float)(chroma[idx] * -cos(theta));
                theta += h;
            }
            continue;
        }
        int64_t vc = (le - ls) & ~(int64_t)3;
        int64_t ve = ls + vc;
        double t0 = theta + (h * 0.0), t1 = theta + h, t2 = theta + h2, t3 = theta + h3;
        int64_t i = ls;
        for (; i < ve; i += 4) {
            out[i] = (double)(float)(chroma[i] * -cos(t0));
            out[i + 1] = (double)(float)(chroma[i + 1] * -cos(t1));
            out[i + 2] = (double)(float)(chroma[i + 2] * -cos(t2));
            out[i + 3] = (double)(float)(chroma[i + 3] * -cos(t3));
            t0 += h4; t1 += h4; t2 += h4; t3 += h4;
        }
        theta += h * (double)vc;
        for (; i < le; i++) {
            out[i] = (double)(float)(chroma[i] * -cos(theta));
            theta += h;
        }
    }
}

/* VhsChromaDecoder.RmsFloat32 / Rms (Core/Decode/VhsChromaDecoder.cs:4376-4423). */
static float rms_f32(const double *v, int64_t n)
{
    if (n <= 0) return 0.0f;
    float mean = 0.0f;
    for (int64_t i = 0; i < n; i++) mean += (float)v[i];
    mean /= (float)n;
    float ss = 0.0f;
    for (int64_t i = 0; i < n; i++) {
        float c = (float)v[i] - mean;
        float sq = c * c;
        ss += sq;
    }
    return sqrtf(ss / (float)n);
}

static double rms_f64(const double *v, int64_t n)
{
    if (n <= 0) return 0.0;
    double mean = 0.0;
    for (int64_t i = 0; i < n; i++) mean += v[i];
    mean /= (double)n;
    double ss = 0.0;
    for (int64_t i = 0; i < n; i++) {
        double c = v[i] - mean;
        ss += c * c;
    }
    return sqrt(ss / (double)n);
}

static void scaled_to_u16(const double *src, uint16_t *dst, int64_t out_start, int64_t len, double scale,
                          int64_t vec_len)
{
    int64_t sat = vec_len - out_start;
    if (sat < 0) sat = 0;
    if (sat > len) sat = len;
    for (int64_t i = 0; i < len; i++) {
        double shifted = (src[i] * scale) + 32767.0;
        if (i < sat) {
            dst[out_start + i] = !isfinite(shifted) || shifted <= 0.0 ? 0
                                 : shifted >= 65535.0 ? 65535 : (uint16_t)shifted;
        } else {
            dst[out_start + i] = (!isfinite(shifted) || shifted < -9223372036854775808.0 ||
                                  shifted > 9223372036854775807.0)
                                     ? 0 : (uint16_t)(uint64_t)(int64_t)shifted;
        }
    }
}

/*
 * VhsChromaDecoder.ApplyAutomaticChromaGainWithCombToU16
 * (Core/Decode/VhsChromaDecoder.cs:3480-3584, 3586-3659): lines before
 * max(16, burst line) stay at 32767; each later line is the 1H (NTSC) or
 * 2H (PAL) comb of the field (the last two lines uncombed), scaled so its
 * burst RMS equals burst_abs_ref, and written to uint16 (saturating; the
 * field's last n mod 4 samples wrap as the reference's scalar tail does).
 */
void oracle_chroma_agc_comb_u16(const double *chroma, int64_t n, int64_t lines, int64_t line_length,
                                int64_t burst_start, int64_t burst_end, double burst_abs_ref,
                                int64_t burst_line, int64_t dist, int retain_f32, int f32_rms,
                                uint16_t *out, double *work)
{
    int64_t first = burst_line > 16 ? burst_line : 16;
    if (first > lines) first = lines;
    int64_t configured = lines * line_length;
    for (int64_t i = 0; i < first * line_length; i++) out[i] = 32767;
    for (int64_t i = configured; i < n; i++) out[i] = 32767;
    int64_t vec_len = n & ~(int64_t)3;
    for (int64_t line = first; line < lines; line++) {
        int64_t ls = line * line_length;
        const double *src;
        if (line < lines - 2) {
            const double *cur = chroma + ls, *adv = chroma + (line + dist) * line_length,
                         *del = chroma + (line - dist) * line_length;
            for (int64_t i = 0; i < line_length; i++) {
                double c = (!retain_f32 && dist == 2) ? ((cur[i] * 2.0) - del[i] - adv[i]) / 4.0
                                                       : ((cur[i] * 2.0) - adv[i] - del[i]) / 4.0;
                work[i] = retain_f32 ? (double)(float)c : c;
            }
            src = work;
        } else {
            src = chroma + ls;
        }
        double rms = f32_rms ? (double)rms_f32(src + burst_start, burst_end - burst_start)
                             : rms_f64(src + burst_start, burst_end - burst_start);
        double scale = rms != 0.0 ? burst_abs_ref / rms : 1.0;
        scaled_to_u16(src, out, ls, line_length, scale, vec_len);
    }
}

double oracle_chroma_rms(const double *v, int64_t n, int f32)
{
    return f32 ? (double)rms_f32(v, n) : rms_f64(v, n);
}
