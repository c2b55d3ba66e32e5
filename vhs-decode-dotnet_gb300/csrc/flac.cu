// FLAC decoding of 16-bit mono RF captures (.ldf) on the GPU.
//
// The reference reads .ldf captures through libsndfile or ffmpeg
// (Core/Rf/LibsndfilePcm16SampleLoader.cs, Core/Rf/FfmpegPcm16SampleLoader.cs)
// and indexes their frames itself for seeking (Core/Rf/RawFlacFrameIndex.cs,
// Core/Rf/RawFlacStreamInfo.cs).  Here the decoding itself runs on the device,
// following the published format (IETF RFC 9639):
//
// * k_flac_sync scans every byte position of a chunk for a frame header
//   (the 14-bit sync code, valid field codes, a valid coded frame or sample
//   number and a matching CRC-8) and appends the candidates;
// * the host sorts the candidates and chains them: a frame is accepted where
//   its number continues the stream's sequence, so a sync pattern inside
//   compressed data (which also needs a matching CRC-8) is skipped;
// * k_flac_frames decodes each frame on its own thread (the residual is a
//   bit-serial Rice code and the prediction a recurrence, so a frame is
//   sequential work; captures have thousands of frames per second of RF):
//   each residual value is read and predicted at once, the predictor's
//   coefficients and history held in registers (one code path per predictor
//   order), frames handed to threads sorted by subframe type so a warp's lanes
//   run the same path; it checks that the subframe ends where the next frame
//   begins and that the frame's CRC-16 matches, and writes int16 samples.
//
// Only what RF captures use is accepted: one channel of 16 bits per sample.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/vhsdecode_gb300.h"
#include "flac.hpp"
#include "session.hpp"

using namespace vhsd::detail;

namespace vhsd {
namespace {

__device__ __forceinline__ uint32_t bswap32(uint32_t v) { return __byte_perm(v, 0, 0x0123); }

// MSB-first bit reader over 32-bit big-endian words; loads never pass `limit`
// (a word index): bits beyond it read as zero, and overrun() tells whether any
// were consumed (the refill looks up to 64 bits ahead, which alone is not an
// overrun).
struct BitReader {
    const uint32_t* w;
    int64_t next, limit;
    uint64_t cache;
    int avail;
    __device__ void init(const uint32_t* words, int64_t byte_off, int64_t byte_limit) {
        w = words;
        next = byte_off >> 2;
        limit = (byte_limit + 3) >> 2;
        cache = 0;
        avail = 0;
        refill();
        const int skip = (int)(byte_off & 3) * 8;
        cache <<= skip;
        avail -= skip;
    }
    __device__ __forceinline__ void refill() {
        while (avail <= 32) {
            uint32_t v = 0;
            if (next < limit) v = bswap32(__ldg(w + next));
            next++;
            cache |= (uint64_t)v << (32 - avail);
            avail += 32;
        }
    }
    __device__ __forceinline__ uint32_t get(int n) {   // 0 <= n <= 32
        if (n == 0) return 0;
        if (avail < n) refill();
        uint32_t v = (uint32_t)(cache >> (64 - n));
        cache <<= n;
        avail -= n;
        return v;
    }
    __device__ __forceinline__ int32_t sget(int n) {
        if (n == 0) return 0;
        uint32_t v = get(n);
        return (int32_t)(v << (32 - n)) >> (32 - n);
    }
    // zeros before the next one bit (the bit is consumed); -1 past `cap` zeros
    __device__ __forceinline__ int32_t unary(int32_t cap) {
        int32_t q = 0;
        for (;;) {
            if (avail < 32) refill();
            const uint32_t top = (uint32_t)(cache >> 32);
            if (top) {
                const int z = __clz(top);
                cache <<= (z + 1);
                avail -= z + 1;
                q += z;
                return q <= cap ? q : -1;
            }
            cache <<= 32;
            avail -= 32;
            q += 32;
            if (q > cap || overrun()) return -1;
        }
    }
    // bit position relative to the word array
    __device__ __forceinline__ int64_t bitpos() const { return next * 32 - avail; }
    __device__ __forceinline__ bool overrun() const { return bitpos() > limit * 32; }
};

__device__ __forceinline__ bool utf8_number(const uint8_t* p, int64_t n, int64_t at, int& len, uint64_t& val) {
    if (at >= n) return false;
    uint8_t b0 = p[at];
    int extra;
    uint64_t v;
    if (b0 < 0x80) { extra = 0; v = b0; }
    else if ((b0 & 0xE0) == 0xC0) { extra = 1; v = b0 & 0x1F; }
    else if ((b0 & 0xF0) == 0xE0) { extra = 2; v = b0 & 0x0F; }
    else if ((b0 & 0xF8) == 0xF0) { extra = 3; v = b0 & 0x07; }
    else if ((b0 & 0xFC) == 0xF8) { extra = 4; v = b0 & 0x03; }
    else if ((b0 & 0xFE) == 0xFC) { extra = 5; v = b0 & 0x01; }
    else if (b0 == 0xFE) { extra = 6; v = 0; }
    else return false;
    if (at + extra >= n) return false;
    for (int i = 1; i <= extra; i++) {
        uint8_t b = p[at + i];
        if ((b & 0xC0) != 0x80) return false;
        v = (v << 6) | (b & 0x3F);
    }
    len = 1 + extra;
    val = v;
    return true;
}

__constant__ uint8_t c_crc8[256];
__constant__ uint16_t c_crc16[256];

// Frame header at byte `at` (RFC 9639 section 9.1): returns its length (0 if
// not a valid header), the coded number and the block size.
__device__ int parse_header(const uint8_t* p, int64_t n, int64_t at, uint64_t& number, int& block,
                            bool& variable) {
    if (at + 6 > n || p[at] != 0xFF || (p[at + 1] & 0xFE) != 0xF8) return 0;
    variable = p[at + 1] & 1;
    const int bcode = p[at + 2] >> 4, rcode = p[at + 2] & 15;
    const int chan = p[at + 3] >> 4, scode = (p[at + 3] >> 1) & 7, res = p[at + 3] & 1;
    if (bcode == 0 || rcode == 15 || chan > 10 || scode == 3 || res) return 0;
    int len = 0;
    uint64_t num = 0;
    if (!utf8_number(p, n, at + 4, len, num)) return 0;
    int64_t q = at + 4 + len;
    if (bcode == 6) {
        if (q + 1 > n) return 0;
        block = p[q] + 1;
        q += 1;
    } else if (bcode == 7) {
        if (q + 2 > n) return 0;
        block = ((p[q] << 8) | p[q + 1]) + 1;
        q += 2;
    } else if (bcode == 1) {
        block = 192;
    } else if (bcode <= 5) {
        block = 576 << (bcode - 2);
    } else {
        block = 256 << (bcode - 8);
    }
    if (rcode == 12) q += 1;
    else if (rcode == 13 || rcode == 14) q += 2;
    if (q + 1 > n) return 0;
    uint8_t c = 0;
    for (int64_t i = at; i < q; i++) c = c_crc8[c ^ p[i]];
    if (c != p[q]) return 0;
    number = num;
    return (int)(q + 1 - at);
}

// Candidate frame headers: one thread per byte position.
__global__ void k_flac_sync(const uint8_t* __restrict__ p, int64_t n, int64_t* cand, int* count, int cap) {
    const int64_t at = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (at + 1 >= n || p[at] != 0xFF || (p[at + 1] & 0xFE) != 0xF8) return;
    uint64_t num;
    int block;
    bool var;
    if (!parse_header(p, n, at, num, block, var)) return;
    const int k = atomicAdd(count, 1);
    if (k < cap) cand[k] = at;
}

// Residual of a subframe (RFC 9639 section 9.2.7), read one value at a time:
// partitions of Rice (4-bit parameters) or Rice2 (5-bit) codes, or escaped
// partitions of raw signed values.
struct Residual {
    int pbits, esc, porder, part, parts, left, k, width, order, block;
    bool escaped;
    __device__ int init(BitReader& r, int block_, int order_) {
        block = block_;
        order = order_;
        const int method = (int)r.get(2);
        if (method > 1) return 1;
        pbits = method == 0 ? 4 : 5;
        esc = (1 << pbits) - 1;
        porder = (int)r.get(4);
        parts = 1 << porder;
        if ((block >> porder) < order || (block & (parts - 1))) return 2;
        part = -1;
        left = 0;
        return 0;
    }
    // next residual value; false on a malformed or overrunning stream
    __device__ __forceinline__ bool next(BitReader& r, int32_t& v) {
        while (left == 0) {
            if (++part >= parts) return false;
            left = (block >> porder) - (part == 0 ? order : 0);
            k = (int)r.get(pbits);
            escaped = k == esc;
            if (escaped) width = (int)r.get(5);
            if (r.overrun()) return false;
        }
        left--;
        if (escaped) {
            v = r.sget(width);
            return true;
        }
        const int32_t q = r.unary(1 << 20);
        if (q < 0) return false;
        const uint32_t u = ((uint32_t)q << k) | r.get(k);
        v = (int32_t)(u >> 1) ^ -(int32_t)(u & 1);
        return true;
    }
};

// Output of one frame's samples: four int16 packed per 8-byte store when the
// frame's first sample is 8-byte aligned (a thread's stores go to its own
// frame, so a warp's scalar stores would touch 32 lines each).
struct Out4 {
    int16_t* o;
    uint64_t a;
    int i, n;
    bool vec;
    __device__ void init(int16_t* o_) {
        o = o_;
        a = 0;
        i = n = 0;
        vec = ((uintptr_t)o_ & 7) == 0;
    }
    __device__ __forceinline__ void put(int32_t x) {
        if (!vec) {
            o[i++] = (int16_t)x;
            return;
        }
        a = (a >> 16) | ((uint64_t)(uint16_t)x << 48);
        i++;
        if (++n == 4) {
            *reinterpret_cast<uint64_t*>(o + i - 4) = a;
            n = 0;
        }
    }
    __device__ __forceinline__ void flush() {
        for (int k = 0; k < n; k++) o[i - n + k] = (int16_t)(a >> (16 * (4 - n + k)));
        n = 0;
    }
};

// Fixed predictor of order O (RFC 9639 section 9.2.5), history in registers.
template <int O>
__device__ int fixed_subframe(BitReader& r, int block, int bps, int wasted, Out4& o) {
    int32_t h[O > 0 ? O : 1];   // h[0]: the latest sample
#pragma unroll
    for (int j = O - 1; j >= 0; j--) {
        h[j] = r.sget(bps);
        o.put(h[j] << wasted);
    }
    Residual res;
    if (int e = res.init(r, block, O)) return e;
    for (int i = O; i < block; i++) {
        int32_t e;
        if (!res.next(r, e)) return 5;
        int32_t x = e;
        if (O == 1) x += h[0];
        if (O == 2) x += 2 * h[0] - h[1];
        if (O == 3) x += 3 * h[0] - 3 * h[1] + h[2];
        if (O == 4) x += 4 * h[0] - 6 * h[1] + 4 * h[2] - h[3];
#pragma unroll
        for (int j = O - 1; j > 0; j--) h[j] = h[j - 1];
        if (O > 0) h[0] = x;
        o.put(x << wasted);
    }
    return 0;
}

// Linear predictor of order P (RFC 9639 section 9.2.6): coefficients and
// history in registers, products accumulated in 64 bits.
template <int P>
__device__ int lpc_subframe(BitReader& r, int block, int bps, int wasted, Out4& o) {
    int32_t h[P];
#pragma unroll
    for (int j = P - 1; j >= 0; j--) {
        h[j] = r.sget(bps);
        o.put(h[j] << wasted);
    }
    const int prec = (int)r.get(4) + 1;
    if (prec == 16) return 6;
    const int shift = r.sget(5);
    if (shift < 0) return 7;
    int32_t c[P];
#pragma unroll
    for (int j = 0; j < P; j++) c[j] = r.sget(prec);
    Residual res;
    if (int e = res.init(r, block, P)) return e;
    for (int i = P; i < block; i++) {
        int32_t e;
        if (!res.next(r, e)) return 5;
        // four partial sums, so the products do not form one dependent chain
        int64_t acc[4] = {0, 0, 0, 0};
#pragma unroll
        for (int j = 0; j < P; j++) acc[j & 3] += (int64_t)c[j] * h[j];
        const int32_t x = e + (int32_t)(((acc[0] + acc[1]) + (acc[2] + acc[3])) >> shift);
#pragma unroll
        for (int j = P - 1; j > 0; j--) h[j] = h[j - 1];
        h[0] = x;
        o.put(x << wasted);
    }
    return 0;
}

template <int P = 1>
__device__ int lpc_dispatch(int order, BitReader& r, int block, int bps, int wasted, Out4& o) {
    if constexpr (P > 32) {
        return 8;
    } else {
        if (order == P) return lpc_subframe<P>(r, block, bps, wasted, o);
        return lpc_dispatch<P + 1>(order, r, block, bps, wasted, o);
    }
}

// One frame per thread, frames taken in the order `order_idx` gives (sorted
// by subframe type, so the lanes of a warp run the same predictor).
__global__ void __launch_bounds__(64, 1) k_flac_frames(const uint32_t* __restrict__ words, const FlacFrame* frames,
                                                     const int* order_idx, int nframes, int16_t* out, int* status) {
    __shared__ uint16_t t16[256];   // per-thread table indices: shared, not constant, memory
    for (int i = threadIdx.x; i < 256; i += blockDim.x) t16[i] = c_crc16[i];
    __syncthreads();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nframes) return;
    const int f = order_idx[t];
    const FlacFrame fr = frames[f];
    const uint8_t* bytes = reinterpret_cast<const uint8_t*>(words);
    Out4 o;
    o.init(out + fr.sample0);
    int err = 0;
    BitReader r;
    r.init(words, fr.off + fr.header_len, fr.end);
    const int block = fr.block;
    do {
        if (r.get(1) != 0) { err = 10; break; }
        const int type = (int)r.get(6);
        int wasted = 0;
        if (r.get(1)) {
            const int32_t z = r.unary(15);
            if (z < 0) { err = 11; break; }
            wasted = z + 1;
        }
        const int bps = 16 - wasted;
        if (bps <= 0) { err = 12; break; }
        if (type == 0) {
            const int32_t v = r.sget(bps);
            for (int i = 0; i < block; i++) o.put(v << wasted);
        } else if (type == 1) {
            for (int i = 0; i < block; i++) o.put(r.sget(bps) << wasted);
        } else if (type >= 8 && type <= 12) {
            const int ord = type - 8;
            if (ord > block) { err = 13; break; }
            int e = 0;
            switch (ord) {
            case 0: e = fixed_subframe<0>(r, block, bps, wasted, o); break;
            case 1: e = fixed_subframe<1>(r, block, bps, wasted, o); break;
            case 2: e = fixed_subframe<2>(r, block, bps, wasted, o); break;
            case 3: e = fixed_subframe<3>(r, block, bps, wasted, o); break;
            default: e = fixed_subframe<4>(r, block, bps, wasted, o); break;
            }
            if (e) { err = 20 + e; break; }
        } else if (type >= 32) {
            const int ord = type - 31;
            if (ord > block) { err = 14; break; }
            const int e = lpc_dispatch(ord, r, block, bps, wasted, o);
            if (e) { err = 30 + e; break; }
        } else {
            err = 17;
            break;
        }
        o.flush();
        if (r.overrun()) { err = 18; break; }
        // byte alignment, then the frame's CRC-16 must end the frame
        const int64_t bit = r.bitpos();
        const int64_t end_byte = (bit + 7) >> 3;
        if (end_byte + 2 != fr.end) { err = 19; break; }
        uint16_t crc = 0;
        for (int64_t i = fr.off; i < end_byte; i++)
            crc = (uint16_t)((crc << 8) ^ t16[(crc >> 8) ^ bytes[i]]);
        if (crc != (uint16_t)((bytes[end_byte] << 8) | bytes[end_byte + 1])) { err = 40; break; }
    } while (false);
    if (err) atomicCAS(status, 0, (f << 8) | err);
}

std::vector<uint8_t> make_crc8() {
    std::vector<uint8_t> t(256);
    for (int b = 0; b < 256; b++) {
        uint8_t c = (uint8_t)b;
        for (int i = 0; i < 8; i++) c = (c & 0x80) ? (uint8_t)((c << 1) ^ 0x07) : (uint8_t)(c << 1);
        t[b] = c;
    }
    return t;
}
std::vector<uint16_t> make_crc16() {
    std::vector<uint16_t> t(256);
    for (int b = 0; b < 256; b++) {
        uint16_t c = (uint16_t)(b << 8);
        for (int i = 0; i < 8; i++) c = (c & 0x8000) ? (uint16_t)((c << 1) ^ 0x8005) : (uint16_t)(c << 1);
        t[b] = c;
    }
    return t;
}

// host-side parse of one header (same rules as the device's), for chaining
int host_header(const uint8_t* p, int64_t n, int64_t at, uint64_t& number, int& block, bool& variable) {
    if (at + 6 > n || p[at] != 0xFF || (p[at + 1] & 0xFE) != 0xF8) return 0;
    variable = p[at + 1] & 1;
    const int bcode = p[at + 2] >> 4, rcode = p[at + 2] & 15;
    const int chan = p[at + 3] >> 4, scode = (p[at + 3] >> 1) & 7;
    if (bcode == 0 || rcode == 15 || chan > 10 || scode == 3 || (p[at + 3] & 1)) return 0;
    uint8_t b0 = p[at + 4];
    int extra;
    uint64_t v;
    if (b0 < 0x80) { extra = 0; v = b0; }
    else if ((b0 & 0xE0) == 0xC0) { extra = 1; v = b0 & 0x1F; }
    else if ((b0 & 0xF0) == 0xE0) { extra = 2; v = b0 & 0x0F; }
    else if ((b0 & 0xF8) == 0xF0) { extra = 3; v = b0 & 0x07; }
    else if ((b0 & 0xFC) == 0xF8) { extra = 4; v = b0 & 0x03; }
    else if ((b0 & 0xFE) == 0xFC) { extra = 5; v = b0 & 0x01; }
    else if (b0 == 0xFE) { extra = 6; v = 0; }
    else return 0;
    if (at + 4 + extra >= n) return 0;
    for (int i = 1; i <= extra; i++) {
        uint8_t b = p[at + 4 + i];
        if ((b & 0xC0) != 0x80) return 0;
        v = (v << 6) | (b & 0x3F);
    }
    int64_t q = at + 5 + extra;
    if (bcode == 6) { if (q + 1 > n) return 0; block = p[q] + 1; q += 1; }
    else if (bcode == 7) { if (q + 2 > n) return 0; block = ((p[q] << 8) | p[q + 1]) + 1; q += 2; }
    else if (bcode == 1) block = 192;
    else if (bcode <= 5) block = 576 << (bcode - 2);
    else block = 256 << (bcode - 8);
    if (rcode == 12) q += 1;
    else if (rcode == 13 || rcode == 14) q += 2;
    if (q + 1 > n) return 0;
    static const std::vector<uint8_t> t8 = make_crc8();
    uint8_t c = 0;
    for (int64_t i = at; i < q; i++) c = t8[c ^ p[i]];
    if (c != p[q]) return 0;
    number = v;
    if (chan != 0 || scode != 4) return -1;   // a valid header of a format RF captures do not use
    return (int)(q + 1 - at);
}

}  // namespace

int32_t flac_stream_info(const uint8_t* p, uint64_t n, FlacInfo& info) {
    // "fLaC", then a first metadata block that is a 34-byte STREAMINFO
    // (the reference's loader rejects anything else: LibsndfilePcm16SampleLoaderTests.cs:1038-1047)
    if (n < 42 || std::memcmp(p, "fLaC", 4) != 0) return fail(VHSDECODE_GB300_STATUS_INPUT_ERROR, "not a FLAC stream");
    if ((p[4] & 0x7F) != 0 || ((p[5] << 16) | (p[6] << 8) | p[7]) != 34)
        return fail(VHSDECODE_GB300_STATUS_INPUT_ERROR, "first FLAC metadata block is not a 34-byte STREAMINFO");
    const uint8_t* si = p + 8;
    info.min_block = (si[0] << 8) | si[1];
    info.max_block = (si[2] << 8) | si[3];
    uint64_t packed = 0;
    for (int i = 10; i < 18; i++) packed = (packed << 8) | si[i];
    info.sample_rate = (uint32_t)(packed >> 44);
    info.channels = (uint32_t)((packed >> 41) & 7) + 1;
    info.bits_per_sample = (uint32_t)((packed >> 36) & 31) + 1;
    info.total_samples = packed & ((uint64_t(1) << 36) - 1);
    // metadata blocks up to the first frame
    uint64_t pos = 4;
    for (;;) {
        if (pos + 4 > n) return fail(VHSDECODE_GB300_STATUS_INPUT_ERROR, "truncated FLAC metadata");
        const bool last = p[pos] & 0x80;
        const uint64_t len = ((uint64_t)p[pos + 1] << 16) | ((uint64_t)p[pos + 2] << 8) | p[pos + 3];
        pos += 4 + len;
        if (last) break;
    }
    if (pos > n) return fail(VHSDECODE_GB300_STATUS_INPUT_ERROR, "truncated FLAC metadata");
    info.first_frame = pos;
    return VHSDECODE_GB300_STATUS_OK;
}

FlacStreamDecoder::~FlacStreamDecoder() {
    if (d_bytes) cudaFree(d_bytes);
    if (d_cand) cudaFree(d_cand);
    if (d_frames) cudaFree(d_frames);
    if (d_work) cudaFree(d_work);
    if (d_out) cudaFree(d_out);
    if (d_misc) cudaFree(d_misc);
    if (stream) cudaStreamDestroy(stream);
}

void FlacStreamDecoder::init(int device) {
    ck(cudaSetDevice(device), "cudaSetDevice");
    ck(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
    // the CRC tables live in this device's copy of the module's constant memory
    const std::vector<uint8_t> t8 = make_crc8();
    const std::vector<uint16_t> t16 = make_crc16();
    ck(cudaMemcpyToSymbol(c_crc8, t8.data(), 256), "crc table");
    ck(cudaMemcpyToSymbol(c_crc16, t16.data(), 512), "crc table");
    ck(cudaMalloc(&d_misc, 2 * sizeof(int)), "cudaMalloc");
}

void FlacStreamDecoder::reserve(size_t bytes, size_t samples, size_t frames) {
    auto grow = [](void** p, size_t& have, size_t want) {
        if (want <= have) return;
        if (*p) cudaFree(*p);
        *p = nullptr;
        ck(cudaMalloc(p, want), "cudaMalloc");
        have = want;
    };
    grow((void**)&d_bytes, cap_bytes, (bytes + 96) & ~(size_t)15);
    grow((void**)&d_cand, cap_cand, std::max<size_t>(frames, 1024) * sizeof(int64_t));
    grow((void**)&d_frames, cap_frames, std::max<size_t>(frames + 16, 64) * sizeof(FlacFrame));
    grow((void**)&d_work, cap_work, std::max<size_t>(frames, 1) * sizeof(int32_t));   // frame order
    grow((void**)&d_out, cap_out, std::max<size_t>(samples, 1) * sizeof(int16_t));
}

size_t FlacStreamDecoder::decode(const uint8_t* p, size_t n, bool at_eof, std::vector<int16_t>& out) {
    return decode_to(p, n, at_eof, [&](size_t count) {
        const size_t old = out.size();
        out.resize(old + count);
        return out.data() + old;
    });
}

size_t FlacStreamDecoder::decode_to(const uint8_t* p, size_t n, bool at_eof,
                                    const std::function<int16_t*(size_t)>& dest) {
    if (n == 0) return 0;
    // header candidates: real frames of RF captures hold thousands of bytes; a
    // chunk may hold up to one candidate per 64 bytes (false sync patterns in
    // compressed data that also pass the CRC-8 are about 1 in 2^24 positions)
    const size_t max_frames = n / 64 + 1024;
    reserve(n, 0, max_frames);
    ck(cudaMemsetAsync(d_bytes + (n & ~(size_t)15), 0, 80, stream), "memset");   // zero pad after the data
    ck(cudaMemcpyAsync(d_bytes, p, n, cudaMemcpyHostToDevice, stream), "h2d flac");
    ck(cudaMemsetAsync(d_misc, 0, 2 * sizeof(int), stream), "memset");
    const bool timing = std::getenv("VHSD_STAGE_TIMING") != nullptr;
    cudaEvent_t ev[4] = {};
    if (timing)
        for (auto& e : ev) ck(cudaEventCreate(&e), "event");
    if (timing) ck(cudaEventRecord(ev[0], stream), "event");
    const int cap = (int)(cap_cand / sizeof(int64_t));
    k_flac_sync<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(d_bytes, (int64_t)n, d_cand, d_misc, cap);
    ck(cudaGetLastError(), "flac sync launch");
    if (timing) ck(cudaEventRecord(ev[1], stream), "event");
    int count = 0;
    ck(cudaMemcpyAsync(&count, d_misc, sizeof(int), cudaMemcpyDeviceToHost, stream), "d2h");
    ck(cudaStreamSynchronize(stream), "sync");
    if (count > cap) throw Failure(VHSDECODE_GB300_STATUS_INPUT_ERROR, "too many FLAC frame candidates");
    std::vector<int64_t> cand((size_t)count);
    if (count) ck(cudaMemcpy(cand.data(), d_cand, (size_t)count * sizeof(int64_t), cudaMemcpyDeviceToHost), "d2h");
    std::sort(cand.begin(), cand.end());
    // chain: the chunk starts on a frame; accept headers that continue the sequence
    std::vector<FlacFrame> frames;
    int64_t expect_at = 0;
    for (size_t i = 0; i < cand.size(); i++) {
        const int64_t at = cand[i];
        if (at < expect_at) continue;
        uint64_t num = 0;
        int block = 0;
        bool var = false;
        const int hl = host_header(p, (int64_t)n, at, num, block, var);
        if (hl == 0) continue;
        const uint64_t want = var ? next_sample : next_frame;
        if (hl < 0) {
            // a header of another sample format where this stream's next frame belongs
            if (num == want) throw Failure(VHSDECODE_GB300_STATUS_INPUT_ERROR, "FLAC stream is not 16-bit mono");
            continue;
        }
        if (num != want) {
            if (frames.empty() && at == 0)
                throw Failure(VHSDECODE_GB300_STATUS_INPUT_ERROR, "FLAC frame out of sequence");
            continue;
        }
        if (!frames.empty()) frames.back().end = at;
        else if (at != 0) throw Failure(VHSDECODE_GB300_STATUS_INPUT_ERROR, "FLAC data before the first frame");
        FlacFrame fr{};
        fr.off = at;
        fr.end = (int64_t)n;
        fr.header_len = hl;
        fr.block = block;
        fr.sample0 = (int64_t)(next_sample - sample_base);
        frames.push_back(fr);
        next_frame++;
        next_sample += (uint64_t)block;
        expect_at = at + hl;
    }
    // the last frame of a chunk is complete only at the end of the stream
    if (!at_eof && !frames.empty()) {
        next_frame--;
        next_sample -= (uint64_t)frames.back().block;
        frames.pop_back();
    }
    if (frames.empty()) {
        if (at_eof && n > 0) throw Failure(VHSDECODE_GB300_STATUS_INPUT_ERROR, "no FLAC frame in the final data");
        return 0;
    }
    const size_t nsamp = (size_t)(next_sample - sample_base);
    reserve(n, nsamp, frames.size());
    // frames sorted by subframe type (the byte after the frame header), so the
    // lanes of a warp decode with the same predictor
    std::vector<int> idx(frames.size());
    for (size_t i = 0; i < idx.size(); i++) idx[i] = (int)i;
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) {
        return (p[frames[(size_t)a].off + frames[(size_t)a].header_len] & 0x7E) <
               (p[frames[(size_t)b].off + frames[(size_t)b].header_len] & 0x7E);
    });
    ck(cudaMemcpyAsync(d_frames, frames.data(), frames.size() * sizeof(FlacFrame), cudaMemcpyHostToDevice, stream),
       "h2d frames");
    ck(cudaMemcpyAsync(d_work, idx.data(), idx.size() * sizeof(int), cudaMemcpyHostToDevice, stream), "h2d order");
    if (timing) ck(cudaEventRecord(ev[2], stream), "event");
    k_flac_frames<<<(unsigned)((frames.size() + 63) / 64), 64, 0, stream>>>(
        reinterpret_cast<const uint32_t*>(d_bytes), d_frames, d_work, (int)frames.size(), d_out, d_misc + 1);
    if (timing) ck(cudaEventRecord(ev[3], stream), "event");
    ck(cudaGetLastError(), "flac decode launch");
    int st = 0;
    int16_t* dst = dest(nsamp);
    if (dst) ck(cudaMemcpyAsync(dst, d_out, nsamp * sizeof(int16_t), cudaMemcpyDeviceToHost, stream), "d2h");
    ck(cudaMemcpyAsync(&st, d_misc + 1, sizeof(int), cudaMemcpyDeviceToHost, stream), "d2h");
    ck(cudaStreamSynchronize(stream), "sync");
    if (timing) {
        float t_sync = 0, t_frames = 0;
        cudaEventElapsedTime(&t_sync, ev[0], ev[1]);
        cudaEventElapsedTime(&t_frames, ev[2], ev[3]);
        std::fprintf(stderr, "vhsd flac: %zu bytes, %zu frames, header scan %.3f ms, frame decode %.3f ms\n", n,
                     frames.size(), t_sync, t_frames);
        for (auto& e : ev) cudaEventDestroy(e);
    }
    if (st) {
        char msg[128];
        std::snprintf(msg, sizeof msg, "corrupt FLAC frame %lld (code %d)",
                      (long long)(next_frame - frames.size() + (st >> 8)), st & 255);
        throw Failure(VHSDECODE_GB300_STATUS_INPUT_ERROR, msg);
    }
    sample_base = next_sample;
    decoded_frames += frames.size();
    return (size_t)frames.back().end;
}

}  // namespace vhsd

using namespace vhsd;

extern "C" {

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_flac_info(
    const uint8_t* data, uint64_t bytes, vhsdecode_gb300_flac_info_v1* info) {
    return guard([&]() -> int32_t {
        if (!data || !info) return fail(VHSDECODE_GB300_STATUS_NULL_POINTER, "null argument");
        if (info->struct_size != sizeof(vhsdecode_gb300_flac_info_v1))
            return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "flac_info struct_size mismatch");
        FlacInfo fi{};
        int32_t st = flac_stream_info(data, bytes, fi);
        if (st != VHSDECODE_GB300_STATUS_OK) return st;
        info->sample_rate = fi.sample_rate;
        info->channels = fi.channels;
        info->bits_per_sample = fi.bits_per_sample;
        info->min_block = fi.min_block;
        info->max_block = fi.max_block;
        info->total_samples = fi.total_samples;
        info->first_frame_offset = fi.first_frame;
        return VHSDECODE_GB300_STATUS_OK;
    });
}

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_flac_decode(
    const uint8_t* data, uint64_t bytes, int16_t* out, uint64_t capacity, uint64_t* samples, int32_t device_id) {
    return guard([&]() -> int32_t {
        if (!data || !samples || (capacity && !out)) return fail(VHSDECODE_GB300_STATUS_NULL_POINTER, "null argument");
        FlacInfo fi{};
        int32_t st = flac_stream_info(data, bytes, fi);
        if (st != VHSDECODE_GB300_STATUS_OK) return st;
        if (fi.channels != 1 || fi.bits_per_sample != 16)
            return fail(VHSDECODE_GB300_STATUS_INPUT_ERROR, "FLAC stream is not 16-bit mono");
        // one decoder (device buffers, stream) per device, reused across calls;
        // calls on one device are serialised
        static std::mutex m;
        static FlacStreamDecoder* decoders[64] = {};
        if (device_id < 0 || device_id >= 64) return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "device_id out of range");
        std::lock_guard<std::mutex> lk(m);
        if (!decoders[device_id]) {
            auto* d = new FlacStreamDecoder();
            try {
                d->init(device_id);
            } catch (...) {
                delete d;
                throw;
            }
            decoders[device_id] = d;
        }
        FlacStreamDecoder& dec = *decoders[device_id];
        ck(cudaSetDevice(device_id), "cudaSetDevice");
        dec.reset();
        // the samples go straight to the caller's buffer when they fit
        std::vector<int16_t> spill;
        uint64_t produced = 0;
        dec.decode_to(data + fi.first_frame, bytes - fi.first_frame, true, [&](size_t count) -> int16_t* {
            produced = count;
            if (count <= capacity) return out;
            if (!capacity) return nullptr;
            spill.resize(count);
            return spill.data();
        });
        *samples = produced;
        if (!spill.empty()) std::memcpy(out, spill.data(), capacity * sizeof(int16_t));
        return VHSDECODE_GB300_STATUS_OK;
    });
}

}  // extern "C"
