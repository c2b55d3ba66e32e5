// Field sync control plane (standard VHS branch of the reference):
//   SyncAnalyzer.FromParameters / EstimateTiming / ClassifyPulses /
//   RefinePulses (+ long-hsync rescue, TryReadVBlank) / ComputeMeanLineLength /
//   BuildUpstreamLineLocations        (Core/Dsp/SyncAnalysis.cs:84-640)
//   VBlankSyncResolver.FindFirstGroup / EstimateLine0FromGroups / FirstHSyncLine /
//   NextFieldLocation                 (Core/Dsp/VBlankSyncResolver.cs:49-315, 447-497, 560-746)
//   FieldParityDetector.ResolveCadence (Core/Dsp/FieldParityDetector.cs:16-250)
//   TbcFieldDecodePipeline.FindRawPulses / ComputeNextFieldOffsetSamples /
//   ThrowIfInsufficientFieldData      (Core/Decode/TbcFieldDecodePipeline.cs:2245-2325, 2375-2385, 5961-5990)
// The line-0 choice is the VBlank-group consensus (combined when the first
// and next VBlank agree, else the single-group estimate chosen as
// SelectSingleVBlankEstimate does).
#include "control.hpp"

#include <algorithm>
#include <cmath>
#include <optional>

namespace vhsd {

double round_away(double x) { return x >= 0 ? std::floor(x + 0.5) : -std::floor(-x + 0.5); }

// numpy median: the middle element, or the mean of the two middle ones
// (selection instead of a full sort; same values).
static double median(std::vector<double> v) {
    size_t n = v.size();
    if (n == 0) return NAN;
    auto mid = v.begin() + (ptrdiff_t)(n / 2);
    std::nth_element(v.begin(), mid, v.end());
    if (n & 1) return *mid;
    double lo = *std::max_element(v.begin(), mid);
    return (lo + *mid) / 2.0;
}

static RatioBounds ratio_bounds(double n, double lo, double hi) {
    RatioBounds b;
    b.lo = (int64_t)std::floor(lo * n) - 4;
    while ((double)b.lo / n < lo) b.lo++;
    b.hi = (int64_t)std::ceil(hi * n) + 4;
    while ((double)b.hi / n > hi) b.hi--;
    return b;
}

SyncParams SyncParams::make(const FormatParams& f, double fs) {
    SyncParams s{};
    s.pal = f.pal;
    s.fs = fs;
    s.mhz = fs / 1e6;
    s.nominal = std::nearbyint(f.line_period_us * s.mhz);  // round half to even
    s.line_period_us = s.nominal / s.mhz;
    s.hsync_us = f.hsync_us;
    s.eq_us = f.eq_us;
    s.vsync_us = f.vsync_us;
    s.num_pulses = f.num_pulses;
    s.ire0 = f.ire0;
    s.hz_ire = f.hz_ire;
    s.vsync_ire = f.vsync_ire;
    s.output_lines = f.frame_lines / 2 + 1;
    s.outlinelen = f.outlinelen;
    s.fsc_mhz = f.fsc_mhz;
    s.half_line = ratio_bounds(s.nominal, 0.4, 0.6);
    s.line = ratio_bounds(s.nominal, 0.9, 1.1);
    s.mixed = ratio_bounds(s.nominal, 0.4, 1.1);
    s.mean_line = ratio_bounds(s.nominal, 0.95, 1.05);
    return s;
}

std::vector<Pulse> span_pulses(const int64_t* ev, int64_t nev, int64_t s0, int64_t slen,
                               int64_t min_len, int64_t max_len) {
    std::vector<Pulse> out;
    out.reserve(512);
    int64_t s1 = s0 + slen;
    const int64_t* lo = std::lower_bound(ev, ev + nev, 2 * s0);
    int64_t cur = -1;
    for (const int64_t* e = lo; e < ev + nev; e++) {
        int64_t pos = *e >> 1;
        if (pos >= s1) break;
        if ((*e & 1) == 0) {
            cur = pos;
        } else {
            if (cur > s0) {
                int64_t len = pos - cur;
                if (len >= min_len && len <= max_len) out.push_back({cur - s0, len});
            }
            cur = -1;
        }
    }
    return out;
}

namespace {

bool in_range(double v, double lo, double hi) { return v >= lo && v <= hi; }

// The integer lengths L with lo <= L <= hi (empty for NaN bounds), so pulse
// length tests compare integers, with the same outcome as the double test.
struct LenRange {
    int64_t lo = 1, hi = 0;
    bool has(int64_t v) const { return v >= lo && v <= hi; }
};
LenRange len_range(double lo, double hi) {
    LenRange r;
    if (lo == lo && hi == hi) {
        r.lo = (int64_t)std::ceil(lo);
        r.hi = (int64_t)std::floor(hi);
    }
    return r;
}

struct Timing {
    double h0, h1, e0, e1, v0, v1;
    LenRange hs, eq, vs, long_hs;   // [h0,h1], [e0,e1], [v0,v1], [h1, 3 h1]
};

Timing estimate_timing(const SyncParams& sp, const std::vector<Pulse>& raw) {
    double lo = sp.usec(sp.hsync_us - 1.75), hi = sp.usec(sp.hsync_us + 2.0);
    std::vector<double> lens;
    lens.reserve(raw.size());
    for (const Pulse& p : raw) if (in_range((double)p.len, lo, hi)) lens.push_back((double)p.len);
    double med = lens.empty() ? sp.hsync_us : median(lens);
    double off = med - sp.usec(sp.hsync_us);
    Timing t;
    t.h0 = med - sp.usec(sp.hsync_tol);
    t.h1 = med + sp.usec(sp.hsync_tol);
    t.e0 = sp.usec(sp.eq_us - sp.eq_tol) + off;
    t.e1 = sp.usec(sp.eq_us + sp.eq_tol) + off;
    t.v0 = sp.usec(sp.vsync_us * 0.5) + off;
    t.v1 = sp.usec(sp.vsync_us + 1.0) + off;
    t.hs = len_range(t.h0, t.h1);
    t.eq = len_range(t.e0, t.e1);
    t.vs = len_range(t.v0, t.v1);
    t.long_hs = len_range(t.h1, t.h1 * 3.0);
    return t;
}

int classify(const Timing& t, int64_t len) {
    if (t.hs.has(len)) return kHSync;
    if (t.eq.has(len)) return kEq;
    if (t.vs.has(len)) return kVSync;
    return -1;
}

// (start - prev.start) / nominal within [0.4, 0.6] between two non-hsync
// pulses, [0.9, 1.1] between two hsyncs, else [0.4, 1.1]
bool quality(const SyncParams& sp, const CPulse& prev, int kind, int64_t start) {
    const int64_t d = start - prev.start;
    if (prev.kind != kHSync && kind != kHSync) return sp.half_line.contains(d);
    if (prev.kind == kHSync && kind == kHSync) return sp.line.contains(d);
    return sp.mixed.contains(d);
}

std::vector<CPulse> classify_pulses(const SyncParams& sp, const std::vector<Pulse>& raw, const Timing& t) {
    std::vector<CPulse> out;
    out.reserve(raw.size());
    for (const Pulse& p : raw) {
        int k = classify(t, p.len);
        if (k < 0) continue;
        bool ok = !out.empty() && quality(sp, out.back(), k, p.start);
        out.push_back({p.start, p.len, k, ok});
    }
    return out;
}

// PulseDetection.FindPulses on a small host buffer (rescue search)
std::vector<Pulse> find_pulses_host(const std::vector<double>& d, double high, int64_t mn, int64_t mx) {
    std::vector<Pulse> out;
    if (d.empty()) return out;
    bool in = d[0] <= high;
    int64_t cur = 0;
    for (int64_t p = 0; p < (int64_t)d.size(); p++) {
        double v = d[(size_t)p];
        if (in) {
            if (v > high) {
                int64_t len = p - cur;
                if (len >= mn && len <= mx && cur != 0) out.push_back({cur, len});
                in = false;
            }
        } else if (v <= high) {
            cur = p;
            in = true;
        }
    }
    return out;
}

int read_vblank(const SyncParams& sp, const std::vector<Pulse>& pulses, const Timing& t, int start,
                int end, std::vector<CPulse>& dest) {
    std::vector<CPulse> valid;
    valid.reserve((size_t)std::max(0, end - start));
    int state = -1;
    double state_end = 0.0;
    bool has_len = false;
    double state_len = 0.0;
    for (int idx = std::max(0, start); idx < end; idx++) {
        const Pulse& p = pulses[(size_t)idx];
        int rk = classify(t, p.len);
        if (rk < 0) continue;
        int acc = -1;
        bool done = false;
        if (state == -1 && rk == kHSync) acc = kHSync;
        else if (state == kHSync) {
            if (rk == kHSync) acc = kHSync;
            else if (rk == kEq) { acc = kEq; has_len = true; state_len = sp.num_pulses / 2.0; }
            else if (rk == kVSync) acc = kVSync;
        } else if (state == kEq) {
            if (rk == kEq) acc = kEq;
            else if (rk == kVSync) { acc = kVSync; has_len = true; state_len = sp.num_pulses / 2.0; }
            else if (rk == kHSync) acc = kHSync;
        } else if (state == kVSync) {
            if (rk == kEq) { acc = kEq2; has_len = true; state_len = sp.num_pulses / 2.0; }
            else if (rk == kVSync) acc = kVSync;
            else if (rk == kHSync && (double)p.start > state_end) acc = kHSync;
        } else if (state == kEq2) {
            if (rk == kEq) acc = kEq2;
            else if (rk == kHSync) { acc = kHSync; done = true; }
        }
        if (acc < 0) continue;
        if (acc != state) {
            if ((double)p.start < state_end) acc = -1;
            else if (has_len) {
                state_end = (double)p.start + (state_len - 0.1) * sp.nominal;
                has_len = false;
            }
        }
        if (acc >= 0) {
            bool ok = !valid.empty() && quality(sp, valid.back(), acc, p.start);
            valid.push_back({p.start, p.len, acc, ok});
            state = acc;
        }
        if (done) {
            for (size_t i = 2; i < valid.size(); i++) dest.push_back(valid[i]);
            return (int)valid.size();
        }
    }
    return 0;
}

std::vector<CPulse> refine_pulses(const SyncParams& sp, const std::vector<Pulse>& raw, const Timing& t,
                                  int64_t span_len, const RefFetch& fetch, double rescue_step) {
    std::vector<Pulse> work = raw;
    std::vector<CPulse> dest;
    dest.reserve(raw.size() + 32);
    size_t i = 0;
    int64_t mn = std::max<int64_t>(0, (int64_t)std::ceil(sp.usec(sp.eq_us) / 8.0));
    int64_t mx = std::max<int64_t>(1, (int64_t)(sp.nominal * 5.0));
    int rescues = 0;
    while (i < work.size()) {
        const Pulse p = work[i];
        if (t.hs.has(p.len)) {
            bool ok = !dest.empty() && quality(sp, dest.back(), kHSync, p.start);
            dest.push_back({p.start, p.len, kHSync, ok});
            i++;
            continue;
        }
        if (fetch && rescue_step > 0.0 && t.long_hs.has(p.len) && rescues < 100000) {
            int64_t st = std::min(std::max<int64_t>(p.start, 0), span_len);
            int64_t en = std::min(std::max<int64_t>(p.start + p.len, st), span_len);
            std::optional<Pulse> r;
            if (en > st) {
                std::vector<double> d;
                fetch(st, en - st, d);
                auto c = find_pulses_host(d, d[0] - rescue_step, mn, mx);
                if (!c.empty()) r = Pulse{st + c[0].start, c[0].len};
            }
            rescues++;
            if (r && (r->start != p.start || r->len != p.len)) {
                work[i] = *r;
                continue;
            }
            i++;
            continue;
        }
        bool can = i > 2 && t.eq.has(p.len) && !dest.empty() && dest.back().kind == kHSync;
        if (!can) { i++; continue; }
        int cnt = read_vblank(sp, work, t, (int)i - 2, (int)std::min(work.size(), i + 24), dest);
        if (cnt == 0) { i++; continue; }
        i += (size_t)std::max(1, cnt - 2);
    }
    return dest;
}

double mean_line_length(const SyncParams& sp, const std::vector<CPulse>& v) {
    int run_start = -1, run_len = -1, cur_start = -1, cur_len = 0;
    for (int i = 0; i < (int)v.size(); i++) {
        if (v[(size_t)i].kind != kHSync) {
            if (cur_start >= 0 && cur_len > run_len) { run_start = cur_start; run_len = cur_len; }
            cur_start = -1;
            cur_len = 0;
        } else if (cur_start < 0) {
            cur_start = i;
            cur_len = 0;
        } else {
            cur_len++;
        }
    }
    if (cur_start >= 0 && cur_len > run_len) { run_start = cur_start; run_len = cur_len; }
    double sum = 0.0;
    int cnt = 0;
    for (int i = run_start + 1; i < run_start + run_len; i++) {
        const int64_t d = v[(size_t)i].start - v[(size_t)i - 1].start;
        if (sp.mean_line.contains(d)) { sum += (double)d; cnt++; }
    }
    return cnt > 0 ? sum / cnt : sp.nominal;
}

struct Group { double prev_hsync, eq1; bool has_v; double vsync, eq2, eq2_end, next_hsync; };

std::optional<Group> find_first_group(const std::vector<CPulse>& p, std::optional<double> min_eq1,
                                      int blank_threshold) {
    int n = (int)p.size();
    for (int start = 1; start < n; start++) {
        const CPulse& prev = p[(size_t)start - 1];
        const CPulse& cur = p[(size_t)start];
        if (prev.kind != kHSync || cur.kind == kHSync || !cur.in_order ||
            (min_eq1 && (double)cur.start <= *min_eq1))
            continue;
        int end = start;
        while (end < n && p[(size_t)end].kind != kHSync) end++;
        if (end >= n || !p[(size_t)end].in_order) { start = std::max(start, end - 1); continue; }
        if ((end - 1 - start) <= blank_threshold) { start = std::max(start, end - 1); continue; }
        int fv = -1;
        for (int i = start; i < end; i++) if (p[(size_t)i].kind == kVSync) { fv = i; break; }
        int fe = -1;
        if (fv >= 0)
            for (int i = fv + 1; i < std::min(end, n); i++)
                if ((p[(size_t)i].kind == kEq || p[(size_t)i].kind == kEq2) && p[(size_t)i].in_order) { fe = i; break; }
        if (fv < 0 || fe < 0) { start = std::max(start, end - 1); continue; }
        Group g;
        g.prev_hsync = (double)prev.start;
        g.eq1 = (double)cur.start;
        g.has_v = fv > start && (p[(size_t)fv - 1].kind == kEq || p[(size_t)fv - 1].kind == kEq2) &&
                  p[(size_t)fv].in_order;
        g.vsync = g.has_v ? (double)p[(size_t)fv].start : 0.0;
        g.eq2 = (double)p[(size_t)fe].start;
        g.eq2_end = (double)p[(size_t)end - 1].start;
        g.next_hsync = (double)p[(size_t)end].start;
        return g;
    }
    return std::nullopt;
}

struct Bound { double first_hsync, first_eq2, last_hsync, last_eq2; };
Bound boundaries(bool pal, bool first) {
    if (!pal) return first ? Bound{1.0, 0.5, 0.5, 1.0} : Bound{0.5, 1.0, 1.0, 0.5};
    return first ? Bound{0.5, 0.5, 1.0, 1.0} : Bound{1.0, 1.0, 0.5, 0.5};
}

struct Marker { double sample, line; };
struct Acc { double loc_sum = 0, off_sum = 0; int count = 0; };
Acc add(Acc a, Acc b) { return {a.loc_sum + b.loc_sum, a.off_sum + b.off_sum, a.count + b.count}; }

std::vector<Marker> markers(const Group& g, double eq1_line, double section) {
    double vl = eq1_line + section, e2 = vl + section, e2e = e2 + section - 0.5;
    std::vector<Marker> m{{g.eq1, eq1_line}};
    if (g.has_v) m.push_back({g.vsync, vl});
    m.push_back({g.eq2, e2});
    m.push_back({g.eq2_end, e2e});
    return m;
}

Acc acc_pair(const Marker& a, const Marker& b, double mll, double fh_line) {
    double actual = (a.sample - b.sample) / mll;
    double expected = a.line - b.line;
    if (actual <= expected - 0.5 || actual >= expected + 0.5) return {};
    return {b.sample + mll * (fh_line - b.line), actual - expected, 1};
}

Acc acc_within(const std::vector<Marker>& m, double mll, double fh_line) {
    Acc a;
    for (size_t i = 0; i < m.size(); i++)
        for (size_t j = i + 1; j < m.size(); j++) a = add(a, acc_pair(m[i], m[j], mll, fh_line));
    return a;
}

struct Est { double line0, first_hsync, fh_line; int count; };

std::optional<Est> finalize(const std::vector<CPulse>& pulses, const Acc& acc, double mll, double fh_line,
                            int field_lines) {
    if (acc.count == 0) return std::nullopt;
    double fh = round_away((acc.loc_sum + acc.off_sum) / acc.count);
    double off = 0.0;
    int cnt = 0;
    const double inv = 1.0 / mll;
    for (const CPulse& p : pulses) {
        if (p.kind != kHSync || !p.in_order) continue;
        // round_away(((start - fh) / mll) + fh_line): a pulse sits near a
        // whole line, so the product with 1/mll (a few ulp off the quotient)
        // rounds the same unless it lands near a half-line, where the exact
        // division decides
        double approx = (((double)p.start - fh) * inv) + fh_line;
        double nearest = round_away(approx);
        int rl = (int)(std::fabs(approx - nearest) < 0.49
                           ? nearest
                           : round_away((((double)p.start - fh) / mll) + fh_line));
        if (rl > field_lines) break;
        if (rl >= fh_line) {
            off += fh + mll * (rl - fh_line) - (double)p.start;
            cnt++;
        }
    }
    if (cnt > 0) fh -= off / cnt;
    return Est{fh - mll * fh_line, fh, fh_line, acc.count};
}

double round_half_line(double v) {
    double hr = round_away(v / 0.5) * 0.5;
    return round_away(hr * 10.0) / 10.0;
}

bool resolve_cadence(const SyncParams& sp, const std::vector<CPulse>& p, double mll, const FieldState& st) {
    int fl0 = sp.field_lines(true);  // fieldLines[0]
    int cons = 0, det = 0, fc = 0, sc = 0;
    if (!p.empty()) {
        double lens[4] = {-1, -1, -1, -1};
        int group = 0, last = -1;
        double second = (double)p[0].start + fl0 * mll;
        for (int i = 0; i < (int)p.size(); i++) {
            const CPulse& cur = p[(size_t)i];
            if (last >= 0 && cur.in_order) {
                const CPulse& prev = p[(size_t)last];
                if (group == 0 && (double)cur.start > second) group = 2;
                if (prev.kind == kHSync && cur.kind != kHSync)
                    lens[group] = round_half_line((double)(cur.start - prev.start) / mll);
                else if (prev.kind != kHSync && cur.kind == kHSync)
                    lens[group + 1] = round_half_line((double)(cur.start - prev.start) / mll);
            }
            last = i;
        }
        const double* f1;
        const double* f2;
        static const double ntsc1[4] = {1.0, 0.5, 0.5, 1.0}, ntsc2[4] = {0.5, 1.0, 1.0, 0.5};
        static const double pal1[4] = {0.5, 0.5, 1.0, 1.0}, pal2[4] = {1.0, 1.0, 0.5, 0.5};
        f1 = sp.pal ? pal1 : ntsc1;
        f2 = sp.pal ? pal2 : ntsc2;
        for (int i = 0; i < 4; i++) {
            if (lens[i] < 0) continue;
            if (std::fabs(lens[i] - f1[i]) < 1e-9) { cons++; det++; }
            else if (std::fabs(lens[i] - f2[i]) < 1e-9) det++;
        }
        if (det > 0) {
            double w = det / 4.0;
            fc = (int)round_away(((double)cons / det) * w * 100.0);
            sc = (int)round_away(((double)(det - cons) / det) * w * 100.0);
        }
    }
    bool first;
    if (st.prev_first >= 0) first = st.prev_first == 0;
    else first = det == 0 || round_away((double)cons / det) == 1.0;
    int eff = 100;
    if (det > 0 && !st.has_prev_hsync && eff > 50) eff = 50;
    if (fc >= eff && fc > sc) first = true;
    else if (sc >= eff && fc < sc) first = false;
    return first;
}

}  // namespace

FieldSync analyse_field(const SyncParams& sp, const std::vector<Pulse>& raw, int64_t span_len,
                        FieldState& state, const RefFetch& fetch) {
    FieldSync out;
    // recovery steps of BuildRecoveryException / ThrowIfInsufficientFieldData
    // (Core/Decode/TbcFieldDecodePipeline.cs:1150-1166, 5636-5650, 5936-6007)
    auto fail = [&](const char* why, double offset) {
        out.error = why;
        out.recover_offset = (int64_t)offset;
        return out;
    };
    if (raw.empty())
        return fail("no sync pulses", state.pulses_seen ? sp.nominal * 100.0 : sp.fs / 10.0);
    state.pulses_seen = true;
    Timing t = estimate_timing(sp, raw);
    std::vector<CPulse> classified = classify_pulses(sp, raw, t);
    std::vector<CPulse> refined = refine_pulses(sp, raw, t, span_len, fetch, 10.0 * sp.hz_ire);
    double mll = mean_line_length(sp, refined);
    bool first = resolve_cadence(sp, refined, mll, state);
    state.prev_first = first ? 1 : 0;
    int field_lines = sp.field_lines(first);
    auto g1 = find_first_group(refined, std::nullopt, 9);
    if (!g1) return fail("no vblank", sp.nominal * 100.0);
    auto g2 = find_first_group(refined, g1->eq1 + (field_lines - 2.0) * mll, 9);
    Bound b = boundaries(sp.pal, first);
    double section = sp.num_pulses / 2.0;
    auto fm = markers(*g1, b.first_hsync, section);
    double fh_line = fm.back().line + b.first_eq2;
    Acc facc = acc_within(fm, mll, fh_line);
    auto fe = finalize(classified, facc, mll, fh_line, field_lines);
    std::optional<Est> le, comb;
    if (g2) {
        auto lm = markers(*g2, field_lines + b.last_hsync, section);
        Acc lacc = acc_within(lm, mll, fh_line);
        le = finalize(classified, lacc, mll, fh_line, field_lines);
        if (facc.count > 0 && lacc.count > 0) {
            double fr = facc.loc_sum / facc.count, lr = lacc.loc_sum / lacc.count;
            if (std::fabs(fr - lr) < 0.5 * mll) {
                Acc cross;
                for (const Marker& a : fm)
                    for (const Marker& c : lm) cross = add(cross, acc_pair(a, c, mll, fh_line));
                comb = finalize(classified, add(add(facc, lacc), cross), mll, fh_line, field_lines);
            }
        }
    }
    std::optional<Est> pick = comb;
    if (!pick) {
        int fc = fe ? fe->count : 0, lc = le ? le->count : 0;
        if (fc == 6 || (!state.has_prev_hsync && fc > lc)) pick = fe;
        else if (le) pick = le;
        else pick = fe;
    }
    if (!pick) return fail("no line 0", sp.nominal * 100.0);
    state.has_prev_hsync = true;
    int processed = sp.output_lines + 10;
    double last_line = (((double)span_len - pick->line0) / mll) - 1.0;
    if (last_line < processed)
        return fail("insufficient data", std::max(pick->line0 - mll * 20.0, sp.nominal));
    // BuildUpstreamLineLocations (SyncAnalysis.cs:551-614)
    std::vector<double> pl;
    pl.reserve(refined.size());
    for (const CPulse& p : refined) pl.push_back((double)p.start);
    if (!std::is_sorted(pl.begin(), pl.end())) std::sort(pl.begin(), pl.end());
    double ref_pulse = std::trunc(pick->first_hsync);
    int ref_line = (int)pick->fh_line;
    out.locs.assign((size_t)processed, 0.0);
    out.filled.assign((size_t)processed, 0);
    size_t cur = 0;
    double maxd = mll / 1.5;
    for (int line = 0; line < processed; line++) {
        double expected = ref_pulse + mll * (line - ref_line);
        out.locs[(size_t)line] = expected;
        if (cur >= pl.size()) continue;
        double cd = std::fabs(pl[cur] - expected);
        double smallest = maxd, sel = -1.0;
        size_t si = cur;
        while (si + 1 < pl.size()) {
            if (cd <= smallest) { smallest = cd; cur = si; sel = pl[si]; }
            double nd = std::fabs(pl[si + 1] - expected);
            if (nd > cd) break;
            cd = nd;
            si++;
        }
        if (sel >= 0.0) { out.locs[(size_t)line] = sel; cur++; }
    }
    // ComputeVhsNextFieldOffsetSamples (TbcFieldDecodePipeline.cs:2299-2325)
    double fhl = b.first_hsync + section * 3.0 - 0.5 + b.first_eq2;
    double next_loc = pick->first_hsync + mll * ((field_lines + b.last_hsync) - fhl);
    out.next_offset = next_loc - 8.0 * sp.nominal + 1024.0;
    out.first_field = first;
    out.line0 = pick->line0;
    out.first_hsync = pick->first_hsync;
    out.mean_line = mll;
    out.ok = true;
    return out;
}

}  // namespace vhsd
