// Format parameters for the supported tape formats.
//
// Values restate the frozen upstream parameter snapshot the reference embeds
// (src/VHSDecode.Core/Formats/format-params.snapshot.json, cases PAL and NTSC
// VHS and SVHS at sp, lp and ep, read by
// Core/Formats/FormatCatalog.cs:46-112); only the keys the RF -> TBC luma and
// chroma paths read are kept.
#pragma once
#include <cmath>
#include <cstdint>

namespace vhsd {

struct FormatParams {
    // system
    bool pal;
    double fps, ire0, hz_ire, vsync_ire, line_period_us;
    double hsync_us, eq_us, vsync_us;
    int num_pulses, outlinelen, frame_lines, output_zero;
    double outfreq_mhz, fsc_mhz;
    double burst_start_us, burst_end_us;   // sysparams colorBurstUS (TBC metadata)
    // RF video band-pass
    double bpf_low, bpf_high;
    int bpf_order;                // 0 = none (magnitude path), >0 Butterworth band-pass
    double lpf_extra, hpf_extra;  // 0 = absent
    int lpf_extra_order, hpf_extra_order;
    double peak_freq, peak_gain, peak_bandwidth;
    bool has_ramp;
    double ramp_start, ramp_boost0, ramp_boost20;
    bool ramp_double;
    // video low-pass / de-emphasis
    double video_lpf_freq;
    int video_lpf_order;
    bool video_lpf_supergauss;
    double deemph_gain, deemph_mid, deemph_q;
    double color_under;
    // colour-under chroma (BuildChromaFieldOptions / BuildChromaBurstSos,
    // TbcFieldDecodePipeline.cs:2626-2760, DecodeFilterSet.cs:563-599)
    double burst_abs_ref;                    // sysparams burst_abs_ref
    double chroma_bpf_upper;                 // RF chroma band-pass top (Hz); bottom 60 kHz, order 4
    int chroma_rot0, chroma_rot1;            // rfparams chroma_rotation
    // video_custom_luma_filters (DecodeFilterSet.cs:1560-1609): the measured
    // "svhs-sp-linear-subdeemphasis" response (used where a table exists for
    // the sample rate) and a high shelf designed at half the sample rate
    bool custom_luma_table;
    double shelf_mid, shelf_gain, shelf_q;   // shelf_mid 0 = none
    // sub-deemphasis (DecodeSession.cs:1250-1278, RfDemodulator.cs:2852-2990)
    bool sub_deemph;
    double sub_hp_freq;                      // first-order Butterworth high-pass
    double sub_amp_lpf;                      // first-order Butterworth amplitude low-pass
    double sub_deviation;                    // hz_ire * (100 - vsync_ire)
    double sub_exp;                          // nonlinear_exp_scaling
    double sub_scale1, sub_scale2;           // NaN = absent
    double sub_logistic_mid, sub_logistic_rate;  // rate NaN or <= 0 = absent
    double sub_static;                       // nonlinear_static_factor (absent = 0)
};

inline FormatParams pal_vhs_sp() {
    FormatParams f{};
    f.pal = true;
    f.fps = 25.0; f.ire0 = 4100000.0; f.hz_ire = 7000.0; f.vsync_ire = -42.857142857142854;
    f.line_period_us = 64.0; f.hsync_us = 4.7; f.eq_us = 2.35; f.vsync_us = 27.3;
    f.num_pulses = 5; f.outlinelen = 1135; f.frame_lines = 625; f.output_zero = 256;
    f.outfreq_mhz = 17.734475; f.fsc_mhz = 4.43361875;
    f.burst_start_us = 5.6; f.burst_end_us = 7.85;
    f.bpf_low = 1300000.0; f.bpf_high = 5780000.0; f.bpf_order = 0;
    f.lpf_extra = 5910000.0; f.lpf_extra_order = 20;
    f.hpf_extra = 1320000.0; f.hpf_extra_order = 12;
    f.peak_freq = 4300000.0; f.peak_gain = 4.0; f.peak_bandwidth = 10000000.0;
    f.has_ramp = true; f.ramp_start = 626953.0; f.ramp_boost0 = 0.0; f.ramp_boost20 = 1.0;
    f.ramp_double = false;
    f.video_lpf_freq = 3400000.0; f.video_lpf_order = 6; f.video_lpf_supergauss = false;
    f.deemph_gain = 13.9794; f.deemph_mid = 273755.82; f.deemph_q = 0.462088186;
    f.color_under = 626953.0;
    f.burst_abs_ref = 5000.0; f.chroma_bpf_upper = 1300000.0; f.chroma_rot0 = 0; f.chroma_rot1 = -1;
    return f;
}

inline FormatParams ntsc_vhs_sp() {
    FormatParams f{};
    f.pal = false;
    f.fps = 29.970029970029973; f.ire0 = 3685714.2857142854; f.hz_ire = 7142.857142857143;
    f.vsync_ire = -40.0; f.line_period_us = 63.55555555555555; f.hsync_us = 4.7; f.eq_us = 2.3;
    f.vsync_us = 27.1; f.num_pulses = 6; f.outlinelen = 910; f.frame_lines = 525;
    f.output_zero = 1024; f.outfreq_mhz = 14.318181818181818; f.fsc_mhz = 3.5795454545454546;
    f.burst_start_us = 5.3; f.burst_end_us = 7.8;
    f.bpf_low = 500000.0; f.bpf_high = 6500000.0; f.bpf_order = 8;
    f.lpf_extra = 6000000.0; f.lpf_extra_order = 25;
    f.hpf_extra = 1200000.0; f.hpf_extra_order = 20;
    f.peak_freq = 3900000.0; f.peak_gain = 4.0; f.peak_bandwidth = 10000000.0;
    f.has_ramp = true; f.ramp_start = 629370.6293706294; f.ramp_boost0 = 0.0; f.ramp_boost20 = 1.0;
    f.ramp_double = false;
    f.video_lpf_freq = 6600000.0; f.video_lpf_order = 9; f.video_lpf_supergauss = true;
    f.deemph_gain = 13.9794; f.deemph_mid = 273755.82; f.deemph_q = 0.462088186;
    f.color_under = 629370.6293706294;
    f.burst_abs_ref = 4416.0; f.chroma_bpf_upper = 1200000.0; f.chroma_rot0 = -1; f.chroma_rot1 = 1;
    return f;
}

// S-VHS keeps its system's sync/TBC parameters and changes the FM levels,
// the RF and video filters and adds the custom luma filters and
// sub-deemphasis (snapshot cases PAL/SVHS/sp, NTSC/SVHS/sp).
inline void svhs_common(FormatParams& f) {
    f.lpf_extra = 9100000.0; f.lpf_extra_order = 25;
    f.hpf_extra = 1300000.0; f.hpf_extra_order = 20;
    f.bpf_low = 2000000.0; f.bpf_high = 8980000.0; f.bpf_order = 0;
    f.peak_freq = 6200000.0; f.peak_gain = 4.0; f.peak_bandwidth = 16000000.0;
    f.ramp_boost0 = 1.0; f.ramp_boost20 = 4.0;
    f.video_lpf_freq = 7500000.0; f.video_lpf_order = 6; f.video_lpf_supergauss = true;
    f.custom_luma_table = true;
    f.shelf_mid = 2000000.0; f.shelf_gain = 4.0; f.shelf_q = 0.4967045;
    f.sub_deemph = true;
    f.sub_hp_freq = 320000.0;
    f.sub_amp_lpf = 590000.0;
    f.sub_deviation = f.hz_ire * (100.0 + -f.vsync_ire);
    f.sub_exp = 0.23;
    f.sub_scale1 = NAN;
    f.sub_scale2 = 0.72;
    f.sub_logistic_mid = 0.2;
    f.sub_logistic_rate = 14.0;
    f.sub_static = 0.0;
}

inline FormatParams pal_svhs_sp() {
    FormatParams f = pal_vhs_sp();
    f.ire0 = 5880000.0; f.hz_ire = 11200.0;
    svhs_common(f);
    return f;
}

inline FormatParams ntsc_svhs_sp() {
    FormatParams f = ntsc_vhs_sp();
    f.ire0 = 5857142.857142857; f.hz_ire = 11428.57142857143;
    svhs_common(f);
    return f;
}

// VHS LP and EP (snapshot cases PAL/VHS/lp|ep and NTSC/VHS/lp|ep): the SP
// parameters with the format's sub-deemphasis switched on (use_sub_deemphasis:
// a first-order 820 kHz high-pass of the video, the amplitude low-pass at its
// 700 kHz default, nonlinear_exp_scaling 0.12, nonlinear_scaling_1 0.1, no
// second scale, logistic or static factor) and, for NTSC, a lower extra RF
// low-pass (LP 5.9 MHz, EP 5.8 MHz), an EP band-pass top of 6.4 MHz and an LP
// burst reference of 2208.
inline void vhs_long_play(FormatParams& f, bool ep) {
    f.sub_deemph = true;
    f.sub_hp_freq = 820000.0;
    f.sub_amp_lpf = 700000.0;
    f.sub_deviation = f.hz_ire * (100.0 + -f.vsync_ire);
    f.sub_exp = 0.12;
    f.sub_scale1 = 0.1;
    f.sub_scale2 = NAN;
    f.sub_logistic_mid = NAN;
    f.sub_logistic_rate = NAN;
    f.sub_static = 0.0;
    if (!f.pal) {
        f.lpf_extra = ep ? 5800000.0 : 5900000.0;
        if (ep) f.bpf_high = 6400000.0;
        else f.burst_abs_ref = 2208.0;   // NTSC VHS LP: half the SP burst reference
    }
}

// speed: 0 SP, 1 LP, 2 EP (the reference's tape_speed values).  S-VHS LP and EP
// carry the S-VHS SP parameters unchanged.
inline FormatParams vhs_format(bool pal, int speed) {
    FormatParams f = pal ? pal_vhs_sp() : ntsc_vhs_sp();
    if (speed != 0) vhs_long_play(f, speed == 2);
    return f;
}

// VideoOutputConverter.ComputeOutputScale (Core/Tbc/VideoOutputConverter.cs:129-138)
inline double output_scale(const FormatParams& f) {
    double dividend = f.pal ? (double)(0xD300 - 0x0100) : (double)(0xC800 - 0x0400);
    return dividend / (100.0 - f.vsync_ire);
}

}  // namespace vhsd
