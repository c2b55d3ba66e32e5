#pragma once
#include <complex>
#include <vector>

#include "formats.hpp"

namespace vhsd {

// Bins 0..N/2 (N = 32768) of the spectra the block demodulator multiplies by,
// plus the 700 kHz first-order envelope low-pass.
struct FilterSpectra {
    std::vector<double> rf_video;                 // real gain
    std::vector<std::complex<double>> video;      // video low-pass x de-emphasis
    std::vector<std::complex<double>> sync;       // video reference x 0.5 MHz FIR
    double env_b0 = 0, env_b1 = 0, env_a1 = 0;
    // sub-deemphasis (formats with sub_deemph): Video x first-order high-pass,
    // the amplitude low-pass and the nonlinear map's constants
    std::vector<std::complex<double>> sub_high;   // empty when the format has none
    double sub_b0 = 0, sub_b1 = 0, sub_a1 = 0;
};

// Throws std::runtime_error when a custom luma table the format needs at this
// sample rate is missing from the library's data folder.
FilterSpectra design_filters(const FormatParams& f, double fs);

// Bins 0..N/2 of the measured S-VHS luma response for sample rate fs, read from
// <library folder>/../data/svhs-sp-linear-subdeemphasis-<(int)fs>.f64; false
// when the reference has no table for this rate (the filter is then skipped,
// as DecodeFilterSetBuilder.TryLoadCustomFilter returns null).
bool load_custom_luma(double fs, std::vector<std::complex<double>>& half);

}  // namespace vhsd
