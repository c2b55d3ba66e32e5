// Chroma filter design and tables (host).  See chroma.hpp.
//
// The band-pass design follows IirFilterDesign.ButterworthBandPassSos step by
// step with the complex helpers it calls (NumPy's complex multiply and
// Smith division, a fused-multiply-add product for the gain, and
// System.Numerics.Complex's square root, magnitude and product), so the
// sections match the reference's to the bit wherever the C library's tan,
// cos and sin do.
#include "chroma.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace vhsd {
namespace {

struct Cx {
    double re, im;
};

const double kPi = 3.141592653589793;
const double kTau = 6.283185307179586;

Cx add(Cx a, Cx b) { return {a.re + b.re, a.im + b.im}; }
Cx sub(Cx a, Cx b) { return {a.re - b.re, a.im - b.im}; }

// IirFilterDesign.NumpyComplexMultiply (:670-677)
Cx mul_numpy(Cx a, Cx b) {
    double rl = a.re * b.re, rr = a.im * b.im, il = a.re * b.im, ir = a.im * b.re;
    return {rl - rr, il + ir};
}
// IirFilterDesign.NumpySimdComplexMultiply (:679-690)
Cx mul_simd(Cx a, Cx b) { return {std::fma(a.re, b.re, -(a.im * b.im)), std::fma(a.im, b.re, a.re * b.im)}; }
// System.Numerics.Complex operator *
Cx mul_net(Cx a, Cx b) { return {a.re * b.re - a.im * b.im, a.im * b.re + a.re * b.im}; }

// IirFilterDesign.NumpyComplexDivide (:692-715)
Cx div_numpy(Cx l, Cx r) {
    if (std::fabs(r.re) >= std::fabs(r.im)) {
        double ratio = r.im / r.re;
        double sd = 1.0 / (r.re + (r.im * ratio));
        return {(l.re + (l.im * ratio)) * sd, (l.im - (l.re * ratio)) * sd};
    }
    double ratio = r.re / r.im;
    double sd = 1.0 / (r.im + (r.re * ratio));
    return {((l.re * ratio) + l.im) * sd, ((l.im * ratio) - l.re) * sd};
}

// System.Numerics.Complex's hypotenuse (Complex.Abs / Magnitude)
double hypot_net(double a, double b) {
    a = std::fabs(a);
    b = std::fabs(b);
    double small = a < b ? a : b, large = a < b ? b : a;
    if (small == 0.0) return large;
    double ratio = small / large;
    return large * std::sqrt(1.0 + ratio * ratio);
}

// System.Numerics.Complex.Sqrt (no rescaling at these magnitudes)
Cx sqrt_net(Cx z) {
    if (z.im == 0.0) return z.re < 0.0 ? Cx{0.0, std::sqrt(-z.re)} : Cx{std::sqrt(z.re), 0.0};
    if (z.re >= 0.0) {
        double x = std::sqrt((hypot_net(z.re, z.im) + z.re) * 0.5);
        return {x, z.im / (2.0 * x)};
    }
    double y = std::sqrt((hypot_net(z.re, z.im) - z.re) * 0.5);
    if (z.im < 0.0) y = -y;
    return {z.im / (2.0 * y), y};
}

// IirFilterDesign.NumpyComplexAbs (:1564-1580)
double abs_numpy(Cx z) {
    double larger = std::fabs(z.re), smaller = std::fabs(z.im);
    if (larger < smaller) std::swap(larger, smaller);
    if (larger == 0.0) return 0.0;
    double ratio = smaller / larger;
    return larger * std::sqrt(std::fma(ratio, ratio, 1.0));
}

size_t nearest(const std::vector<Cx>& v, Cx t) {
    size_t sel = 0;
    double best = INFINITY;
    for (size_t i = 0; i < v.size(); i++) {
        double d = abs_numpy(sub(v[i], t));
        if (d < best) {
            best = d;
            sel = i;
        }
    }
    return sel;
}

// NumPy's float32 sin/cos as the reference restates it
// (VhsChromaDecoder.NumpyTrigFloat32, :3830-3893)
float bits_f(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

float numpy_trig_f32(float x, bool want_cos) {
    if (std::isnan(x)) return NAN;
    float maxcw = want_cos ? 71476.0625f : 117435.992f;
    if (std::fabs(x) > maxcw) return want_cos ? std::cos(x) : std::sin(x);
    float q = x * bits_f(0x3F22F983u);
    const float magic = 12582912.0f;
    q = (q + magic) - magic;
    float r = std::fma(q, bits_f(0xBFC90FD8u), x);
    r = std::fma(q, bits_f(0xB4A8885Au), r);
    r = std::fma(q, bits_f(0xA7C234C4u), r);
    float r2 = r * r;
    float c = std::fma(bits_f(0x37CC730Bu), r2, bits_f(0xBAB6036Eu));
    c = std::fma(c, r2, bits_f(0x3D2AAA9Eu));
    c = std::fma(c, r2, -0.5f);
    c = std::fma(c, r2, 1.0f);
    float s = std::fma(bits_f(0x363E9DDEu), r2, bits_f(0xB95035DDu));
    s = std::fma(s, r2, bits_f(0x3C0888CDu));
    s = std::fma(s, r2, -1.0f / 6.0f);
    s = std::fma(s, r2, 0.0f);
    s = std::fma(s, r, r);
    int iq = (int)std::nearbyint(q);
    if (want_cos) iq++;
    float res = (iq & 1) == 0 ? s : c;
    return (iq & 2) != 0 ? -res : res;
}

}  // namespace

std::vector<double> butter_bandpass_sos(int order, double lo, double hi) {
    // DesignButterworthBandPassZpk (:1143-1212)
    const double fs = 2.0;
    double wl = 2.0 * fs * std::tan(kPi * lo / 2.0);
    double wh = 2.0 * fs * std::tan(kPi * hi / 2.0);
    double bw = wh - wl;
    double c = std::sqrt(wl * wh);
    std::vector<Cx> pos, neg;
    for (int m = -order + 1; m < order; m += 2) {
        double ang = (kPi * m) / (2.0 * order);   // BuildButterworthPrototypePoles (:427-436)
        Cx p{-std::cos(ang), -std::sin(ang)};
        Cx sp{p.re * (bw / 2.0), p.im * (bw / 2.0)};
        Cx sq = mul_numpy(sp, sp);
        Cx root = sqrt_net({sq.re - c * c, sq.im});
        pos.push_back(add(sp, root));
        neg.push_back(sub(sp, root));
    }
    const double bs = 2.0 * fs;
    std::vector<Cx> zeros, poles;
    for (int i = 0; i < order; i++) zeros.push_back({1.0, 0.0});
    for (int i = 0; i < order; i++) zeros.push_back({-1.0, 0.0});
    Cx dprod{1.0, 0.0};
    std::vector<Cx> analog = pos;
    analog.insert(analog.end(), neg.begin(), neg.end());
    for (const Cx& p : analog) {
        Cx den{bs - p.re, -p.im};
        poles.push_back(div_numpy({bs + p.re, p.im}, den));
        dprod = mul_simd(dprod, den);
    }
    double gain = std::pow(bw, order) * div_numpy({std::pow(bs, order), 0.0}, dprod).re;

    // ZpkToNearestSos (:1381-1437)
    struct Pair {
        Cx a, b;
        double radius;
    };
    std::vector<Cx> rem = poles;
    std::vector<Pair> pairs;
    while (!rem.empty()) {
        size_t fi = 0;
        for (size_t i = 0; i < rem.size(); i++)
            if (rem[i].im > 1e-12) { fi = i; break; }
        Cx first = rem[fi];
        rem.erase(rem.begin() + (long)fi);
        Cx tgt{first.re, -first.im};
        size_t si = 0;
        double best = INFINITY;
        for (size_t i = 0; i < rem.size(); i++) {
            Cx d = sub(rem[i], tgt);
            double dist = hypot_net(d.re, d.im);
            if (dist < best) {
                best = dist;
                si = i;
            }
        }
        Cx second = rem[si];
        rem.erase(rem.begin() + (long)si);
        pairs.push_back({first, second, std::max(hypot_net(first.re, first.im), hypot_net(second.re, second.im))});
    }
    std::stable_sort(pairs.begin(), pairs.end(), [](const Pair& x, const Pair& y) { return x.radius > y.radius; });
    struct Assigned {
        Cx p1, p2, z1, z2;
        double radius;
    };
    std::vector<Assigned> asg;
    std::vector<Cx> remz = zeros;
    for (const Pair& pr : pairs) {
        size_t i1 = nearest(remz, pr.a);
        Cx z1 = remz[i1];
        remz.erase(remz.begin() + (long)i1);
        size_t i2 = nearest(remz, pr.a);
        Cx z2 = remz[i2];
        remz.erase(remz.begin() + (long)i2);
        asg.push_back({pr.a, pr.b, z1, z2, pr.radius});
    }
    std::stable_sort(asg.begin(), asg.end(), [](const Assigned& x, const Assigned& y) { return x.radius < y.radius; });
    std::vector<double> sos;
    for (const Assigned& a : asg) {
        Cx zs = add(a.z1, a.z2), zp = mul_net(a.z1, a.z2);
        Cx ps = add(a.p1, a.p2), pp = mul_net(a.p1, a.p2);
        double row[6] = {1.0, -zs.re, zp.re, 1.0, -ps.re, pp.re};
        sos.insert(sos.end(), row, row + 6);
    }
    if (!sos.empty()) {
        sos[0] *= gain;
        sos[1] *= gain;
        sos[2] *= gain;
    }
    return sos;
}

FloatCascade float_cascade(const std::vector<double>& sos) {
    FloatCascade fc{};
    const int ns = (int)(sos.size() / 6);
    // SosFilter.DefaultPadLength (:540-545)
    int zb = 0, za = 0;
    for (int s = 0; s < ns; s++) {
        zb += sos[6 * s + 2] == 0.0;
        za += sos[6 * s + 5] == 0.0;
    }
    fc.edge = 3 * (2 * ns + 1 - std::min(zb, za));
    // SteadyStateInitialConditionsFloat32 (:924-951)
    float scale = 1.0f;
    for (int s = 0; s < ns && s < kChromaSections; s++) {
        for (int k = 0; k < 6; k++) fc.sec[s][k] = (float)sos[6 * s + k];
        const float* c = fc.sec[s];
        float ft = c[1] - (c[4] * c[0]);
        float st = c[2] - (c[5] * c[0]);
        float num = (0.0f + ft) + st;
        float den = (1.0f + c[4]) + c[5];
        float z0 = num / den;
        float z1 = ((1.0f + c[4]) * z0) - ft;
        fc.zi[s][0] = scale * z0;
        fc.zi[s][1] = scale * z1;
        float ndc = ((0.0f + c[0]) + c[1]) + c[2];
        float ddc = ((0.0f + c[3]) + c[4]) + c[5];
        scale *= ndc / ddc;
    }
    return fc;
}

ChromaDesign design_chroma(const FormatParams& f, double fs) {
    ChromaDesign d;
    d.ntsc = !f.pal;
    d.fsc_mhz = f.fsc_mhz;
    d.cu_hz = f.color_under;
    d.outlen = f.outlinelen;
    d.out_lines = f.frame_lines / 2 + 1;
    d.field_samples = (int64_t)d.outlen * d.out_lines;
    d.burst_abs_ref = f.burst_abs_ref;
    d.rot[0] = f.chroma_rot0;
    d.rot[1] = f.chroma_rot1;
    const double outus = f.outfreq_mhz;
    int b0 = (int)std::floor(f.burst_start_us * outus) - 5;
    int b1 = (int)std::ceil(f.burst_end_us * outus) + 10;
    d.burst_start = std::min(std::max(b0, 0), d.outlen);
    d.burst_end = std::min(std::max(b1, d.burst_start), d.outlen);
    const double nyq = fs / 2.0;
    d.rf_sos = butter_bandpass_sos(4, 60000.0 / nyq, f.chroma_bpf_upper / nyq);
    const double nyq_mhz = (f.fsc_mhz * 4.0) / 2.0;
    const double cu_mhz = f.color_under / 1000000.0;
    d.final_sos = butter_bandpass_sos(4, (f.fsc_mhz - cu_mhz * 0.9) / nyq_mhz, (f.fsc_mhz + cu_mhz * 0.75) / nyq_mhz);
    d.rf = float_cascade(d.rf_sos);
    d.fin = float_cascade(d.final_sos);
    d.move = (int)(5.0 * (fs / 40000000.0));
    d.fsc_ratio = ((f.outfreq_mhz * 1000000.0) / 1000000.0) / f.fsc_mhz;
    return d;
}

void chroma_tables(const ChromaDesign& d, std::vector<float>& het, std::vector<float>& bsin,
                   std::vector<float>& bcos) {
    const int64_t n = d.field_samples;
    const double rate = d.fsc_mhz * 4.0;
    const double scale = (d.fsc_mhz + d.cu_hz / 1000000.0) / rate;
    het.resize((size_t)(4 * n));
    for (int p = 0; p < 4; p++) {
        const double off = (kPi / 2.0 * p) + 0.0;
        const double step = kTau * scale;
        for (int64_t i = 0; i < n; i++) het[(size_t)(p * n + i)] = (float)(-std::cos((step * (double)i) + off));
    }
    const double wave = d.fsc_mhz / rate;
    bsin.resize((size_t)n);
    bcos.resize((size_t)n);
    for (int64_t i = 0; i < n; i++) {
        float theta = (float)((kTau * wave) * (double)i);
        bsin[(size_t)i] = numpy_trig_f32(theta, false);
        bcos[(size_t)i] = numpy_trig_f32(theta, true);
    }
}

}  // namespace vhsd
