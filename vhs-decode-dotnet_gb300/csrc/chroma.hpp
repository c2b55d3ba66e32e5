// Colour-under chroma: filter design, tables and the device stages.
//
// The chroma chain of the reference's exact backend at its v0.4.0 defaults:
// a float32 forward-backward band-pass of the RF per block with a roll and DC
// removal (RfBlockDecodePipeline.DecodeChromaBurstFloat32,
// Core/Decode/RfBlockDecodePipeline.cs:308-336, 540-577), and per field a TBC
// of that channel, the burst phase sequence, the burst refinement of the line
// locations and the field decode to uint16 (Core/Decode/VhsChromaDecoder.cs).
#pragma once
#include <cstdint>
#include <vector>

#include "formats.hpp"

namespace vhsd {

constexpr int kChromaSections = 4;   // order-4 Butterworth band-pass

// Second-order sections (b0 b1 b2 a0 a1 a2 per row) of
// IirFilterDesign.ButterworthBandPassSos (Core/Dsp/IirFilterDesign.cs:594-606,
// 1143-1212, 1381-1437) for order >= 2, cutoffs normalised to Nyquist.
std::vector<double> butter_bandpass_sos(int order, double lo, double hi);

// A section cascade as the float32 forward-backward filter runs it
// (SosFilter.ApplyForwardBackwardFloat32, Core/Dsp/SosFilter.cs:369-538, 924-970):
// float coefficients, float steady-state initial conditions (scaled by the
// first / last extended sample at run time) and the odd-extension length.
struct FloatCascade {
    float sec[kChromaSections][6];
    float zi[kChromaSections][2];
    int edge;
};
FloatCascade float_cascade(const std::vector<double>& sos);

struct ChromaDesign {
    std::vector<double> rf_sos, final_sos;  // binary64 designs
    FloatCascade rf, fin;
    int burst_start = 0, burst_end = 0;     // output samples of the line (v0.4.0 window)
    int move = 0;                           // chroma offset roll (decode samples)
    int out_lines = 0, outlen = 0;
    int64_t field_samples = 0;
    double fsc_mhz = 0, cu_hz = 0, burst_abs_ref = 0;
    double fsc_ratio = 0;                   // (output rate MHz) / fsc MHz
    int rot[2] = {0, 0};                    // chroma_rotation
    bool ntsc = false;
};

// TbcFieldDecodePipeline.BuildChromaFieldOptions (v0.4.0 branch,
// Core/Decode/TbcFieldDecodePipeline.cs:2626-2760) and the chroma filters of
// DecodeFilterSetBuilder.BuildBasic (Core/Dsp/DecodeFilterSet.cs:173-238,
// 563-599, 710-752) for a format decoded at fs Hz.
ChromaDesign design_chroma(const FormatParams& f, double fs);

// One field's heterodyne tables (4 phases x field_samples, BuildHeterodyneTable,
// VhsChromaDecoder.cs:1967-2007) and burst carrier tables (BuildCarrierTables
// with NumPy's float32 sin/cos, :3793-3893), as floats.
void chroma_tables(const ChromaDesign& d, std::vector<float>& het, std::vector<float>& bsin,
                   std::vector<float>& bcos);

}  // namespace vhsd
