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
};

FilterSpectra design_filters(const FormatParams& f, double fs);

}  // namespace vhsd
