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
