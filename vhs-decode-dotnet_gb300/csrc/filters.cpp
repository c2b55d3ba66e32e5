// Filter spectra of the VHS RF path, designed on the host in binary64.
//
// Follows DecodeFilterSetBuilder.BuildBasic (Core/Dsp/DecodeFilterSet.cs:140-256)
// for colour-under tape formats; responses are the "whole" frequency response
// of IirFilterDesign.FrequencyResponse (Core/Dsp/IirFilterDesign.cs:962-1058)
// sampled at bins 0..N/2, which is all the real-FFT path reads.
//   RfVideo   (DecodeFilterSet.cs:307-406): |Butterworth band-pass| (when an
//             order is set) x |Butterworth low-pass extra| x |high-pass extra|
//             x |peaking| x linear ramp, magnitude only.
//   Video     (:1019-1091, :1104-1152): zero-phase video low-pass magnitude x
//             complex de-emphasis shelf.
//   VideoLowPass05 (:1093-1102, :1248-1263): Video reference x 65-tap Hamming
//             FIR at 0.5 MHz.
//   Custom luma filters (:1560-1609, S-VHS): Video x measured response table
//             x high shelf designed with sampleRate/2 as its rate argument.
//   Sub-deemphasis high-pass (RfDemodulator.cs:3101-3142): first-order
//             Butterworth SOS at nonlinear_highpass_freq; amplitude low-pass
//             first-order Butterworth at nonlinear_amp_lpf_freq
//             (IirFilterDesign.cs:1078-1114).
// Butterworth low/high-pass magnitudes use the bilinear closed form
// |H|^2 = 1 / (1 + (tan(w/2) / tan(wc/2))^(+-2N)); the band-pass keeps the
// transfer-function (polynomial) evaluation the reference uses.
#include "filters.hpp"

#include <dlfcn.h>

#include <cmath>
#include <complex>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

namespace vhsd {

using cd = std::complex<double>;
static const double kPi = 3.14159265358979323846;

static double butter_lp_mag(double w, double wc, int order) {
    // w, wc in radians/sample
    double r = std::tan(w / 2.0) / std::tan(wc / 2.0);
    if (w >= kPi) return 0.0;
    return 1.0 / std::sqrt(1.0 + std::pow(r, 2.0 * order));
}
static double butter_hp_mag(double w, double wc, int order) {
    if (w <= 0.0) return 0.0;
    if (w >= kPi) return 1.0;
    double r = std::tan(wc / 2.0) / std::tan(w / 2.0);
    return 1.0 / std::sqrt(1.0 + std::pow(r, 2.0 * order));
}

static std::vector<cd> poly_from_roots(const std::vector<cd>& roots) {
    std::vector<cd> a{cd(1.0, 0.0)};
    for (const cd& r : roots) {
        std::vector<cd> b(a.size() + 1, cd(0.0, 0.0));
        for (size_t i = 0; i < a.size(); i++) {
            b[i] += a[i];
            b[i + 1] -= a[i] * r;
        }
        a.swap(b);
    }
    return a;
}

// scipy.signal.butter(order, [lo, hi], 'bandpass') in transfer-function form
// (analog prototype, lp2bp, bilinear at fs = 2), as IirFilterDesign.ButterworthBandPass.
static void butter_bandpass_ba(int order, double lo, double hi, std::vector<double>& b,
                               std::vector<double>& a) {
    const double fs = 2.0;
    double wl = 2.0 * fs * std::tan(kPi * lo / fs);
    double wh = 2.0 * fs * std::tan(kPi * hi / fs);
    double bw = wh - wl;
    double wo = std::sqrt(wl * wh);
    std::vector<cd> p;
    for (int k = -order + 1; k < order; k += 2) p.push_back(-std::exp(cd(0.0, kPi * k / (2.0 * order))));
    double gain = 1.0;
    std::vector<cd> pb;
    for (const cd& pl : p) {
        cd ps = pl * (bw / 2.0);
        cd d = std::sqrt(ps * ps - wo * wo);
        pb.push_back(ps + d);
        pb.push_back(ps - d);
    }
    std::vector<cd> zb((size_t)order, cd(0.0, 0.0));
    gain *= std::pow(bw, (double)order);
    // bilinear
    const double fs2 = 2.0 * fs;
    std::vector<cd> zz, pz;
    cd num(1.0, 0.0), den(1.0, 0.0);
    for (const cd& z : zb) { zz.push_back((fs2 + z) / (fs2 - z)); num *= (fs2 - z); }
    for (const cd& q : pb) { pz.push_back((fs2 + q) / (fs2 - q)); den *= (fs2 - q); }
    for (size_t i = zb.size(); i < pb.size(); i++) zz.push_back(cd(-1.0, 0.0));
    double kz = gain * (num / den).real();
    std::vector<cd> bc = poly_from_roots(zz), ac = poly_from_roots(pz);
    b.resize(bc.size());
    a.resize(ac.size());
    for (size_t i = 0; i < bc.size(); i++) b[i] = kz * bc[i].real();
    for (size_t i = 0; i < ac.size(); i++) a[i] = ac[i].real();
}

// H(e^{jw}) = sum b[i] e^{-jwi} / sum a[i] e^{-jwi}, Horner from the top coefficient.
static cd freq_resp(const std::vector<double>& b, const std::vector<double>& a, double w) {
    cd z = std::polar(1.0, -w);
    cd nb(b.back(), 0.0), na(a.back(), 0.0);
    for (int i = (int)b.size() - 2; i >= 0; i--) nb = nb * z + b[i];
    for (int i = (int)a.size() - 2; i >= 0; i--) na = na * z + a[i];
    return nb / na;
}

static void high_shelf(double center, double gain_db, double fs, double q, std::vector<double>& b,
                       std::vector<double>& a) {
    double g = std::pow(10.0, gain_db / 40.0);
    double w = 2.0 * kPi * (center / fs);
    double alpha = std::sin(w) / (2.0 * q);
    double c = std::cos(w);
    double rg = std::sqrt(g);
    b = {g * ((g + 1.0) + ((g - 1.0) * c) + (2.0 * rg * alpha)),
         -2.0 * g * ((g - 1.0) + ((g + 1.0) * c)),
         g * ((g + 1.0) + ((g - 1.0) * c) - (2.0 * rg * alpha))};
    a = {(g + 1.0) - ((g - 1.0) * c) + (2.0 * rg * alpha),
         2.0 * ((g - 1.0) - ((g + 1.0) * c)),
         (g + 1.0) - ((g - 1.0) * c) - (2.0 * rg * alpha)};
}

static void peaking(double norm_freq, double gain_db, double bw_oct, std::vector<double>& b,
                    std::vector<double>& a) {
    double q = 1.0 / (2.0 * std::sinh((std::log(2.0) / 2.0) * bw_oct));
    double gain = std::pow(10.0, gain_db / 20.0);
    double zg = gain_db > 0 ? gain : 1.0;
    double pg = gain_db > 0 ? 1.0 : gain;
    double w = 4.0 * std::tan(kPi * norm_freq / 2.0);
    double an[3] = {1.0, (zg / q) * w, w * w};
    double ad[3] = {1.0, (1.0 / (pg * q)) * w, w * w};
    double c = 4.0, c2 = 16.0;
    double n0 = an[0] * c2 + an[1] * c + an[2], n1 = -2.0 * an[0] * c2 + 2.0 * an[2],
           n2 = an[0] * c2 - an[1] * c + an[2];
    double d0 = ad[0] * c2 + ad[1] * c + ad[2], d1 = -2.0 * ad[0] * c2 + 2.0 * ad[2],
           d2 = ad[0] * c2 - ad[1] * c + ad[2];
    b = {n0 / d0, n1 / d0, n2 / d0};
    a = {1.0, d1 / d0, d2 / d0};
}

// Folder of the data files: ../data relative to the folder of this library.
static std::string data_dir() {
    Dl_info info{};
    if (dladdr(reinterpret_cast<void*>(&data_dir), &info) && info.dli_fname) {
        std::string so(info.dli_fname);
        size_t slash = so.rfind('/');
        std::string dir = slash == std::string::npos ? std::string(".") : so.substr(0, slash);
        return dir + "/../data";
    }
    return "data";
}

bool load_custom_luma(double fs, std::vector<cd>& half) {
    const long rate = (long)fs;   // (int)sampleRateHz in the resource name
    if (rate != 40000000L && rate != 17734475L) return false;   // the reference ships these two
    std::string path = data_dir() + "/svhs-sp-linear-subdeemphasis-" + std::to_string(rate) + ".f64";
    FILE* fp = std::fopen(path.c_str(), "rb");
    if (!fp) throw std::runtime_error("custom luma filter table missing: " + path);
    const int H = 32768 / 2 + 1;
    std::vector<double> raw((size_t)2 * H);
    size_t got = std::fread(raw.data(), sizeof(double), raw.size(), fp);
    std::fclose(fp);
    if (got != raw.size()) throw std::runtime_error("custom luma filter table truncated: " + path);
    half.resize((size_t)H);
    for (int k = 0; k < H; k++) half[(size_t)k] = cd(raw[(size_t)2 * k], raw[(size_t)2 * k + 1]);
    return true;
}

static double sinc(double x) {
    if (std::fabs(x) < 1e-12) return 1.0;
    double s = kPi * x;
    return std::sin(s) / s;
}

static std::vector<double> firwin_lowpass_hamming(int ntaps, double cutoff) {
    std::vector<double> h((size_t)ntaps);
    double center = (ntaps - 1) / 2.0;
    double sum = 0.0;
    for (int n = 0; n < ntaps; n++) {
        double m = n - center;
        double win = 0.54 - 0.46 * std::cos(2.0 * kPi * n / (ntaps - 1));
        h[(size_t)n] = cutoff * sinc(cutoff * m) * win;
        sum += h[(size_t)n];
    }
    for (double& v : h) v /= sum;
    return h;
}

FilterSpectra design_filters(const FormatParams& f, double fs) {
    const int N = 32768, H = N / 2 + 1;
    const double nyq = fs / 2.0;
    FilterSpectra out;
    out.rf_video.assign(H, 0.0);
    out.video.assign(H, cd(0.0, 0.0));
    out.sync.assign(H, cd(0.0, 0.0));
    std::vector<double> bb, ba;
    if (f.bpf_order > 0) butter_bandpass_ba(f.bpf_order, f.bpf_low / nyq, f.bpf_high / nyq, bb, ba);
    std::vector<double> pb, pa;
    if (f.peak_freq > 0) peaking(f.peak_freq / nyq, f.peak_gain, f.peak_bandwidth / nyq, pb, pa);
    // ramp (FrequencyDomainFilter.RampFilter, Core/Dsp/FrequencyDomainFilter.cs:64-103)
    std::vector<double> ramp_half((size_t)(N / 2), 0.0);
    if (f.has_ramp) {
        int half = N / 2;
        int zero = (int)((f.ramp_start / nyq) * half);
        zero = zero < 0 ? 0 : (zero > half ? half : zero);
        int cnt = half - zero;
        if (cnt == 1) ramp_half[(size_t)zero] = f.ramp_boost0;
        else if (cnt > 1) {
            double end = f.ramp_boost20 * (nyq / 20e6);
            double step = (end - f.ramp_boost0) / (cnt - 1);
            for (int i = 0; i < cnt; i++) ramp_half[(size_t)(zero + i)] = f.ramp_boost0 + i * step;
            ramp_half[(size_t)(half - 1)] = end;
        }
    }
    std::vector<double> db, da;
    high_shelf(f.deemph_mid, f.deemph_gain, fs, f.deemph_q, db, da);  // inverse used below
    std::vector<double> fir = firwin_lowpass_hamming(65, 0.5 / (nyq / 1e6));
    std::vector<cd> custom;
    const bool has_custom = f.custom_luma_table && load_custom_luma(fs, custom);
    std::vector<double> shb, sha;
    if (f.shelf_mid > 0) high_shelf(f.shelf_mid, f.shelf_gain, fs / 2.0, f.shelf_q, shb, sha);
    std::vector<double> hpb, hpa;
    if (f.sub_deemph) {
        double k = std::tan(kPi * (f.sub_hp_freq / nyq) / 2.0);
        double norm = 1.0 / (1.0 + k);
        hpb = {norm, -norm, 0.0};
        hpa = {1.0, (k - 1.0) * norm, 0.0};
        out.sub_high.assign(H, cd(0.0, 0.0));
    }
    const double wc_lpx = kPi * f.lpf_extra / nyq, wc_hpx = kPi * f.hpf_extra / nyq;
    const double wc_v = kPi * f.video_lpf_freq / nyq;
    for (int k = 0; k < H; k++) {
        double w = 2.0 * kPi * k / N;
        double g = 1.0;
        if (f.bpf_order > 0) g = std::abs(freq_resp(bb, ba, w));
        if (f.lpf_extra > 0) g *= butter_lp_mag(w, wc_lpx, f.lpf_extra_order);
        if (f.hpf_extra > 0) g *= butter_hp_mag(w, wc_hpx, f.hpf_extra_order);
        if (f.peak_freq > 0) g *= std::abs(freq_resp(pb, pa, w));
        if (f.has_ramp) {
            int idx = k < N / 2 ? k : N / 2 - 1;  // bin N/2 mirrors half[N/2 - 1]
            double r = ramp_half[(size_t)idx];
            g *= r;
            if (f.ramp_double) g *= r;
        }
        out.rf_video[(size_t)k] = std::fabs(g);
        // video low-pass magnitude
        double vlp;
        if (f.video_lpf_supergauss) {
            double freq = nyq * k / (H - 1);
            double order = f.video_lpf_order;
            double scale = 2.0 * freq * std::pow(std::log(2.0) / 2.0, 1.0 / (2.0 * order));
            vlp = std::exp(-2.0 * std::pow(scale / f.video_lpf_freq, 2.0 * order));
        } else {
            vlp = butter_lp_mag(w, wc_v, f.video_lpf_order);
        }
        cd deemph = freq_resp(da, db, w);  // de-emphasis = 1 / high shelf
        cd v = vlp * deemph;
        cd vid = v;
        if (has_custom) vid *= custom[(size_t)k];
        if (f.shelf_mid > 0) vid *= freq_resp(shb, sha, w);
        out.video[(size_t)k] = vid;
        if (f.sub_deemph) out.sub_high[(size_t)k] = vid * freq_resp(hpb, hpa, w);
        cd firr(0.0, 0.0);
        for (int n = 0; n < 65; n++) firr += fir[(size_t)n] * std::polar(1.0, -w * n);
        out.sync[(size_t)k] = v * firr;
    }
    double kk = std::tan(kPi * (700000.0 / nyq) / 2.0);
    double norm = 1.0 / (1.0 + kk);
    out.env_b0 = kk * norm;
    out.env_b1 = kk * norm;
    out.env_a1 = (kk - 1.0) * norm;
    if (f.sub_deemph) {
        double ka = std::tan(kPi * (f.sub_amp_lpf / nyq) / 2.0);
        double na = 1.0 / (1.0 + ka);
        out.sub_b0 = ka * na;
        out.sub_b1 = ka * na;
        out.sub_a1 = (ka - 1.0) * na;
    }
    return out;
}

}  // namespace vhsd
