// Host-side field sync control plane: pulse timing and classification, mean
// line length, field cadence, VBlank line-0 estimate, upstream line
// locations and next-field offset.  Inputs are the device-extracted sync
// pulses of one field span; everything here is scalar bookkeeping over a few
// hundred pulses.
#pragma once
#include <cstdint>
#include <functional>
#include <string>
#include <vector>

#include "formats.hpp"

namespace vhsd {

struct Pulse { int64_t start, len; };
enum PulseKind { kHSync = 0, kEq = 1, kVSync = 2, kEq2 = 3 };
struct CPulse { int64_t start, len; int kind; bool in_order; };

// The integers d with lo <= RN(d / n) <= hi, as [lo, hi] (RN(d / n) is
// monotone in d, so the set is an interval): ratio tests of sample distances
// without a division, bit-exact to the divided form.
struct RatioBounds {
    int64_t lo, hi;
    bool contains(int64_t d) const { return d >= lo && d <= hi; }
};

struct SyncParams {
    bool pal;
    double fs, mhz, nominal, line_period_us;
    double hsync_us, eq_us, vsync_us;
    int num_pulses;
    double hsync_tol = 0.7, eq_tol = 0.9;
    double ire0, hz_ire, vsync_ire;
    int output_lines, outlinelen;
    double fsc_mhz;
    // pulse spacing / nominal line in [0.4, 0.6], [0.9, 1.1], [0.4, 1.1], [0.95, 1.05]
    RatioBounds half_line, line, mixed, mean_line;
    static SyncParams make(const FormatParams& f, double fs);
    double usec(double us) const { return us * mhz; }
    double ire_to_hz(double ire) const { return ire0 + hz_ire * ire; }
    int field_lines(bool first) const {
        int n = output_lines;
        return pal ? (first ? n - 1 : n) : (first ? n : n - 1);
    }
};

struct FieldState {
    int prev_first = -1;   // -1 unknown, else 0/1
    bool has_prev_hsync = false;
    bool pulses_seen = false;   // a span with raw pulses was analysed (_vhsPulseSearchInitialized)
    // chroma: the rotation index carried from field to field (_chromaRotationIndex,
    // null = 0) and the VHS field number (ResolveVhsFieldNumber,
    // Core/Decode/TbcFieldDecodePipeline.cs:860-874; vhs_number -1 = none, after a
    // failed field; vhs_loc is the last field's read location in the current
    // stream, negative when a window join left it behind the window)
    int chroma_rot = 0;
    int vhs_number = -1;
    int64_t vhs_loc = -1;
};

struct FieldSync {
    bool ok = false;
    std::string error;
    // when !ok: samples the engine advances its read position before retrying
    // (TbcFieldDecodeRecoveryException.SuggestedOffsetSamples, C# long truncation)
    int64_t recover_offset = 0;
    bool first_field = false;
    double line0 = 0, first_hsync = 0, mean_line = 0, next_offset = 0;
    std::vector<double> locs;       // processed lines, span-relative
    std::vector<uint8_t> filled;
};

// Reads `len` samples of the sync reference at span-relative `start`.
using RefFetch = std::function<void(int64_t start, int64_t len, std::vector<double>& out)>;

// Raw pulses of a span from the global edge events (2*pos + type, stream
// coordinates): the state machine restarted at span_start as
// PulseDetection.FindPulses would see it.
std::vector<Pulse> span_pulses(const int64_t* events, int64_t nevents, int64_t span_start,
                               int64_t span_len, int64_t min_len, int64_t max_len);

FieldSync analyse_field(const SyncParams& sp, const std::vector<Pulse>& raw, int64_t span_len,
                        FieldState& state, const RefFetch& fetch);

double round_away(double x);

}  // namespace vhsd
