// Stage-level C entry points used by the parity tests: they run the same
// device code as the session pipeline on caller-provided host arrays.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#define VHSDECODE_GB300_EXPORTS 1
#include "../../include/vhsdecode_gb300.h"
#include "control.hpp"
#include "kernels.h"
#include "vhs_math.cuh"
#include "spikes.cuh"

namespace vhsd {
template <typename T>
cudaError_t launch_tbc_pw(const T*, int64_t, const TbcParams&, const double*, cudaStream_t);
// shared with abi.cpp
int32_t set_last_error(int32_t status, const char* msg);
std::vector<float> sinc_lut_host();
}  // namespace vhsd

using namespace vhsd;

namespace {

__global__ void k_demod(const float* re, const float* im, int64_t n, float freq, float* out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (i == 0) { out[0] = 0.0f; return; }
    out[i] = vhs_freq_diff(vhs_atan2(im[i], re[i]), vhs_atan2(im[i - 1], re[i - 1]), freq);
}

// ReplaceSpikes of a whole array on one CTA with the block demodulator's
// parallel form; n a multiple of 32.
__global__ void k_replace_spikes_test(float* demod, const float* diffed, unsigned* mask, int* cpos, int n,
                                      float max_value) {
    extern __shared__ unsigned repl[];
    const int lane = threadIdx.x & 31;
    for (int base = (threadIdx.x >> 5) * 32; base < n; base += blockDim.x) {
        unsigned m = __ballot_sync(0xffffffffu, demod[base + lane] > max_value);
        if (lane == 0) mask[base >> 5] = m;
    }
    __syncthreads();
    spike_thresholds(demod, diffed, mask, cpos, n, threadIdx.x, blockDim.x);
    __syncthreads();
    if (threadIdx.x < 32) spike_walk(mask, cpos, repl, n, lane);
    __syncthreads();
    spike_apply(demod, diffed, repl, n, threadIdx.x, blockDim.x);
}

__global__ void k_angles(const float* re, const float* im, int64_t n, float* out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = vhs_atan2(im[i], re[i]);
}

struct Scoped {
    std::vector<void*> ptrs;
    ~Scoped() { for (void* p : ptrs) cudaFree(p); }
    template <typename T>
    T* alloc(size_t n) {
        void* p = nullptr;
        if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return nullptr;
        ptrs.push_back(p);
        return (T*)p;
    }
};

int32_t cuda_status(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return VHSDECODE_GB300_STATUS_OK;
    int32_t st = (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
                     ? VHSDECODE_GB300_STATUS_CUDA_UNAVAILABLE
                     : VHSDECODE_GB300_STATUS_INTERNAL_ERROR;
    return set_last_error(st, (std::string(what) + ": " + cudaGetErrorString(e)).c_str());
}

bool have_device() {
    int n = 0;
    return cudaGetDeviceCount(&n) == cudaSuccess && n > 0;
}

}  // namespace

#define CUDA_OR_RETURN(call, what)                         \
    do {                                                   \
        int32_t _st = cuda_status((call), what);           \
        if (_st != VHSDECODE_GB300_STATUS_OK) return _st;  \
    } while (0)

extern "C" {

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_vhs_angles(
    const float* re, const float* im, uint64_t n, float* out) {
    if ((!re || !im || !out) && n) return set_last_error(VHSDECODE_GB300_STATUS_NULL_POINTER, "null argument");
    if (!have_device()) return set_last_error(VHSDECODE_GB300_STATUS_CUDA_UNAVAILABLE, "no CUDA device available");
    if (n == 0) return set_last_error(VHSDECODE_GB300_STATUS_OK, "");
    Scoped sc;
    float* dre = sc.alloc<float>(n);
    float* dim = sc.alloc<float>(n);
    float* dout = sc.alloc<float>(n);
    if (!dre || !dim || !dout) return set_last_error(VHSDECODE_GB300_STATUS_INTERNAL_ERROR, "cudaMalloc failed");
    CUDA_OR_RETURN(cudaMemcpy(dre, re, n * sizeof(float), cudaMemcpyHostToDevice), "h2d");
    CUDA_OR_RETURN(cudaMemcpy(dim, im, n * sizeof(float), cudaMemcpyHostToDevice), "h2d");
    k_angles<<<(unsigned)((n + 255) / 256), 256>>>(dre, dim, (int64_t)n, dout);
    CUDA_OR_RETURN(cudaGetLastError(), "launch");
    CUDA_OR_RETURN(cudaMemcpy(out, dout, n * sizeof(float), cudaMemcpyDeviceToHost), "d2h");
    return set_last_error(VHSDECODE_GB300_STATUS_OK, "");
}

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_decimate_half_rate(
    const void* source, uint32_t input_sample_format, uint64_t source_count, float* destination) {
    if ((!source || !destination) && source_count > 1)
        return set_last_error(VHSDECODE_GB300_STATUS_NULL_POINTER, "null argument");
    if (input_sample_format > VHSDECODE_GB300_INPUT_INT16)
        return set_last_error(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "unknown input_sample_format");
    if (!have_device()) return set_last_error(VHSDECODE_GB300_STATUS_CUDA_UNAVAILABLE, "no CUDA device available");
    const uint64_t nd = source_count / 2;
    if (nd == 0) return set_last_error(VHSDECODE_GB300_STATUS_OK, "");
    const bool s16 = input_sample_format == VHSDECODE_GB300_INPUT_INT16;
    const size_t esz = s16 ? sizeof(int16_t) : sizeof(float);
    Scoped sc;
    unsigned char* dsrc = sc.alloc<unsigned char>(source_count * esz);
    float* dout = sc.alloc<float>(nd);
    if (!dsrc || !dout) return set_last_error(VHSDECODE_GB300_STATUS_INTERNAL_ERROR, "cudaMalloc failed");
    CUDA_OR_RETURN(cudaMemcpy(dsrc, source, source_count * esz, cudaMemcpyHostToDevice), "h2d");
    CUDA_OR_RETURN(launch_decimate_half(s16 ? reinterpret_cast<const int16_t*>(dsrc) : nullptr,
                                        s16 ? nullptr : reinterpret_cast<const float*>(dsrc),
                                        (int64_t)source_count, dout, (int64_t)nd, 0),
                   "decimate launch");
    CUDA_OR_RETURN(cudaMemcpy(destination, dout, nd * sizeof(float), cudaMemcpyDeviceToHost), "d2h");
    return set_last_error(VHSDECODE_GB300_STATUS_OK, "");
}

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_vhs_demod(
    const float* re, const float* im, uint64_t n, double sample_rate_hz, float* out) {
    if ((!re || !im || !out) && n) return set_last_error(VHSDECODE_GB300_STATUS_NULL_POINTER, "null argument");
    if (!have_device()) return set_last_error(VHSDECODE_GB300_STATUS_CUDA_UNAVAILABLE, "no CUDA device available");
    if (n == 0) return set_last_error(VHSDECODE_GB300_STATUS_OK, "");
    Scoped sc;
    float* dre = sc.alloc<float>(n);
    float* dim = sc.alloc<float>(n);
    float* dout = sc.alloc<float>(n);
    if (!dre || !dim || !dout) return set_last_error(VHSDECODE_GB300_STATUS_INTERNAL_ERROR, "cudaMalloc failed");
    CUDA_OR_RETURN(cudaMemcpy(dre, re, n * sizeof(float), cudaMemcpyHostToDevice), "h2d");
    CUDA_OR_RETURN(cudaMemcpy(dim, im, n * sizeof(float), cudaMemcpyHostToDevice), "h2d");
    k_demod<<<(unsigned)((n + 255) / 256), 256>>>(dre, dim, (int64_t)n, (float)sample_rate_hz, dout);
    CUDA_OR_RETURN(cudaGetLastError(), "launch");
    CUDA_OR_RETURN(cudaMemcpy(out, dout, n * sizeof(float), cudaMemcpyDeviceToHost), "d2h");
    return set_last_error(VHSDECODE_GB300_STATUS_OK, "");
}

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_replace_spikes(
    float* demod, const float* diffed, uint64_t n, float max_value) {
    if ((!demod || !diffed) && n) return set_last_error(VHSDECODE_GB300_STATUS_NULL_POINTER, "null argument");
    if (n % 32 != 0 || n > (1u << 20))
        return set_last_error(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "n must be a multiple of 32, at most 2^20");
    if (!have_device()) return set_last_error(VHSDECODE_GB300_STATUS_CUDA_UNAVAILABLE, "no CUDA device available");
    if (n == 0) return set_last_error(VHSDECODE_GB300_STATUS_OK, "");
    Scoped sc;
    float* dd = sc.alloc<float>(n);
    float* df = sc.alloc<float>(n);
    unsigned* dm = sc.alloc<unsigned>(n / 32);
    int* dc = sc.alloc<int>(n);
    if (!dd || !df || !dm || !dc) return set_last_error(VHSDECODE_GB300_STATUS_INTERNAL_ERROR, "cudaMalloc failed");
    CUDA_OR_RETURN(cudaMemcpy(dd, demod, n * sizeof(float), cudaMemcpyHostToDevice), "h2d");
    CUDA_OR_RETURN(cudaMemcpy(df, diffed, n * sizeof(float), cudaMemcpyHostToDevice), "h2d");
    k_replace_spikes_test<<<1, 512, (n / 32) * sizeof(unsigned)>>>(dd, df, dm, dc, (int)n, max_value);
    CUDA_OR_RETURN(cudaGetLastError(), "launch");
    CUDA_OR_RETURN(cudaMemcpy(demod, dd, n * sizeof(float), cudaMemcpyDeviceToHost), "d2h");
    return set_last_error(VHSDECODE_GB300_STATUS_OK, "");
}

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_find_pulses(
    const double* ref, uint64_t n, double high, int64_t mn, int64_t mx, int64_t* starts,
    int64_t* lens, uint64_t cap, uint64_t* count) {
    if (!count || (!ref && n)) return set_last_error(VHSDECODE_GB300_STATUS_NULL_POINTER, "null argument");
    if (!have_device()) return set_last_error(VHSDECODE_GB300_STATUS_CUDA_UNAVAILABLE, "no CUDA device available");
    *count = 0;
    if (n == 0) return set_last_error(VHSDECODE_GB300_STATUS_OK, "");
    Scoped sc;
    int64_t pslots = pulse_count_slots((int64_t)n);
    int64_t capacity = (int64_t)n + 16;
    double* dref = sc.alloc<double>(n);
    int64_t* dcounts = sc.alloc<int64_t>(pslots);
    int64_t* doffs = sc.alloc<int64_t>(pslots);
    int64_t* dev = sc.alloc<int64_t>(capacity);
    int64_t* dtot = sc.alloc<int64_t>(1);
    if (!dref || !dcounts || !doffs || !dev || !dtot)
        return set_last_error(VHSDECODE_GB300_STATUS_INTERNAL_ERROR, "cudaMalloc failed");
    CUDA_OR_RETURN(cudaMemcpy(dref, ref, n * sizeof(double), cudaMemcpyHostToDevice), "h2d");
    CUDA_OR_RETURN(launch_pulse_events<double>(dref, (int64_t)n, high, dcounts, doffs, dev, capacity, dtot, 0),
                   "launch");
    int64_t total = 0;
    CUDA_OR_RETURN(cudaMemcpy(&total, dtot, sizeof(int64_t), cudaMemcpyDeviceToHost), "d2h");
    std::vector<int64_t> ev((size_t)total);
    if (total) CUDA_OR_RETURN(cudaMemcpy(ev.data(), dev, (size_t)total * sizeof(int64_t), cudaMemcpyDeviceToHost), "d2h");
    std::vector<Pulse> ps = span_pulses(ev.data(), total, 0, (int64_t)n, mn, mx);
    *count = ps.size();
    if (ps.size() > cap) return set_last_error(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "capacity too small");
    for (size_t i = 0; i < ps.size(); i++) { starts[i] = ps[i].start; lens[i] = ps[i].len; }
    return set_last_error(VHSDECODE_GB300_STATUS_OK, "");
}

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_tbc_resample_lines(
    const double* src, uint64_t n, const double* locs, uint32_t nlocs, uint32_t first_line,
    uint32_t line_count, uint32_t outlen, double nominal, double smoothing, double* dst) {
    if (!src || !locs || !dst) return set_last_error(VHSDECODE_GB300_STATUS_NULL_POINTER, "null argument");
    if (n == 0) return set_last_error(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "source must not be empty");
    if (nlocs < 2 || outlen == 0 || (uint64_t)first_line + line_count >= nlocs ||
        first_line + line_count > 500)
        return set_last_error(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "invalid line range");
    for (uint32_t i = 0; i < nlocs; i++)
        if (!std::isfinite(locs[i]))
            return set_last_error(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "line locations must be finite");
    if (!have_device()) return set_last_error(VHSDECODE_GB300_STATUS_CUDA_UNAVAILABLE, "no CUDA device available");
    if (!(nominal > 0.0)) {
        // TbcLineResampler.BuildInterpolator: max(1, median line length)
        std::vector<double> d(nlocs - 1);
        for (uint32_t i = 0; i + 1 < nlocs; i++) d[i] = locs[i + 1] - locs[i];
        std::sort(d.begin(), d.end());
        size_t m = d.size();
        double med = (m & 1) ? d[m / 2] : (d[m / 2 - 1] + d[m / 2]) / 2.0;
        nominal = std::max(1.0, med);
    }
    if (line_count == 0) return set_last_error(VHSDECODE_GB300_STATUS_OK, "");
    Scoped sc;
    std::vector<float> lut = sinc_lut_host();
    double* dsrc = sc.alloc<double>(n);
    double* dloc = sc.alloc<double>(nlocs);
    float* dlut = sc.alloc<float>(lut.size());
    double* dout = sc.alloc<double>((size_t)line_count * outlen);
    double* dlev = sc.alloc<double>(1024);
    double* dpw = sc.alloc<double>(outlen);
    int64_t* dspan = sc.alloc<int64_t>(1);
    int64_t* dslen = sc.alloc<int64_t>(1);
    int* dfl = sc.alloc<int>(1);
    if (!dsrc || !dloc || !dlut || !dout || !dlev || !dpw || !dspan || !dslen || !dfl)
        return set_last_error(VHSDECODE_GB300_STATUS_INTERNAL_ERROR, "cudaMalloc failed");
    std::vector<double> pw(outlen, 0.0);
    if (smoothing > 0.0) {
        double alpha = 1.0 / (smoothing * outlen);
        for (uint32_t k = 0; k < outlen; k++) pw[k] = std::pow(1.0 - alpha, (double)(k + 1));
    }
    int64_t zero = 0;
    int fl = (int)first_line;
    CUDA_OR_RETURN(cudaMemcpy(dsrc, src, n * sizeof(double), cudaMemcpyHostToDevice), "h2d");
    CUDA_OR_RETURN(cudaMemcpy(dloc, locs, nlocs * sizeof(double), cudaMemcpyHostToDevice), "h2d");
    CUDA_OR_RETURN(cudaMemcpy(dlut, lut.data(), lut.size() * sizeof(float), cudaMemcpyHostToDevice), "h2d");
    CUDA_OR_RETURN(cudaMemcpy(dpw, pw.data(), outlen * sizeof(double), cudaMemcpyHostToDevice), "h2d");
    CUDA_OR_RETURN(cudaMemcpy(dspan, &zero, sizeof(int64_t), cudaMemcpyHostToDevice), "h2d");
    CUDA_OR_RETURN(cudaMemcpy(dfl, &fl, sizeof(int), cudaMemcpyHostToDevice), "h2d");
    int64_t nn = (int64_t)n;
    CUDA_OR_RETURN(cudaMemcpy(dslen, &nn, sizeof(int64_t), cudaMemcpyHostToDevice), "h2d");
    TbcParams tp{};
    tp.nfields = 1;
    tp.lines = (int)nlocs;
    tp.locs = dloc;
    tp.span_start = dspan;
    tp.span_len = dslen;
    tp.first_line = dfl;
    tp.out_lines = (int)line_count;
    tp.outlen = (int)outlen;
    tp.nominal = nominal;
    tp.smoothing = smoothing;
    tp.lut = dlut;
    tp.out_hz = dout;
    tp.out_u16 = nullptr;
    tp.level_work = dlev;
    CUDA_OR_RETURN(launch_tbc_pw<double>(dsrc, (int64_t)n, tp, dpw, 0), "launch");
    CUDA_OR_RETURN(cudaMemcpy(dst, dout, (size_t)line_count * outlen * sizeof(double), cudaMemcpyDeviceToHost), "d2h");
    return set_last_error(VHSDECODE_GB300_STATUS_OK, "");
}

}  // extern "C"
