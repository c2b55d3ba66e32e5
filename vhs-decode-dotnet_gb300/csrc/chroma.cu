// Colour-under chroma on the device (the reference's exact backend, v0.4.0
// defaults; Core/Decode/VhsChromaDecoder.cs, Core/Decode/RfBlockDecodePipeline.cs).
//
// Block stage: the float32 forward-backward chroma band-pass of each RF block
// (SosFilter.ApplyForwardBackwardFloat32, Core/Dsp/SosFilter.cs:369-538) is a
// recurrence, so each block is a group of four lanes, lane s running section s
// a 32-sample batch behind lane s - 1 (four independent recurrences per step).
// The result is bit-identical to the reference's sample-by-sample loop (same
// operations, same order, one rounding each).
// The roll by the chroma offset and the removal of the float mean
// (ShiftChromaAndRemoveDcFloat32InPlace, VhsChromaDecoder.cs:2517-2533,
// MeanFloat32FastMath :3751-3791) then stitch the block into the stream.
//
// Field stage: burst probes of the line-1 chroma TBC for both rotation
// sequences of every field (ProbeUpconvertedBurstValue + DemodBurstFloat32,
// :1438-1713), the track-flip test (:4164-4217), the rotation index carried
// from field to field, the phase averages (:4219-4290) and the burst
// refinement of the line locations (:2342-2428, v0.4.0 form); after the TBC of
// the output lines, up-conversion (:2009-2248), the final float32
// band-pass and the automatic gain with the comb to uint16 (:3480-3659).
// The final band-pass runs on 1024-sample chunks, each started 448 samples
// early from zero state (its poles are inside radius 0.94: the dropped
// history weighs below 1e-12), so it equals the sequential filter to float
// rounding rather than bit for bit.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "kernels.h"

namespace vhsd {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kTile = 32;          // samples staged per group per tile
constexpr int kGroupsPerWarp = 8;  // 4-lane groups
constexpr int kIirWarps = 4;       // warps per CTA of the cascade kernels
constexpr int kChunk = 1024;       // final band-pass chunk
constexpr int kWarmup = 448;       // zero-state lead of a chunk

__device__ __forceinline__ float sos_step(const float* c, float v, float& z1, float& z2) {
    float f = __fadd_rn(__fmul_rn(c[0], v), z1);
    z1 = __fadd_rn(__fsub_rn(__fmul_rn(c[1], v), __fmul_rn(c[4], f)), z2);
    z2 = __fsub_rn(__fmul_rn(c[2], v), __fmul_rn(c[5], f));
    return f;
}

// One pass of the 4-section cascade over samples 0 .. len-1 of a sequence,
// run by a 4-lane group (lane s = section s).  Lane s filters sample t - 32 s
// at step t, so its input (the output of lane s - 1) was written a whole
// 32-step batch earlier and each lane runs only its own section's recurrence.
// Per batch a lane reads its 32 inputs (lane 0 from the staged input tile,
// the others from the ring of the lane before), filters them, and writes its
// outputs (lane 3: to the output tile, flushed by all four lanes).  Every
// group of the warp loops `steps` times (warp-uniform, >= len + 96).
// load(i) returns sample i of the pass; store(i, v) receives the cascade
// output of sample i.  The initial state is zi * x0.  `area` is the group's
// kCascadeArea floats of shared memory.
// Regions of kTile floats padded to kRegion, so the float4 accesses of the 32
// lanes of a warp (8 groups x 4 lanes, each lane its own region) spread over
// the shared-memory banks instead of all starting on bank 0.
constexpr int kRegion = kTile + 4;
constexpr int kCascadeArea = 9 * kRegion;   // input tiles [2], rings [3][2], output tile

// Staged input: fetch(i) loads the raw 32-bit word of sample i (an int16 read
// sign-extended by the load itself, or float bits) and cook(raw, i) turns it
// into the sample a batch later, so no instruction waits on the load while
// the recurrence runs.
template <typename Fetch, typename Cook, typename Store>
__device__ __forceinline__ void cascade_batch(const float* sec, float& z1, float& z2, int s, float* tin, float* ring,
                                              float* tout, int64_t base, int cur, int64_t len,
                                              uint32_t (&fetch_into)[kTile / 4], const uint32_t (&staged)[kTile / 4],
                                              Fetch fetch, Cook cook, Store store) {
    constexpr int per = kTile / 4;
    // loads for the tile two batches ahead (cooked at the end of the next batch)
#pragma unroll
    for (int k = 0; k < per; k++) {
        const int64_t i = base + 2 * kTile + s * per + k;
        fetch_into[k] = i < len ? fetch(i) : 0u;
    }
    const float* src = s == 0 ? tin + cur * kRegion : ring + ((s - 1) * 2 + (cur ^ 1)) * kRegion;
    float v[kTile];
#pragma unroll
    for (int j = 0; j < kTile; j += 4) {
        const float4 q = *reinterpret_cast<const float4*>(src + j);
        v[j] = q.x; v[j + 1] = q.y; v[j + 2] = q.z; v[j + 3] = q.w;
    }
    const int64_t i0 = base - (int64_t)s * kTile;
    if (i0 >= 0 && i0 + kTile <= len) {
#pragma unroll
        for (int j = 0; j < kTile; j++) v[j] = sos_step(sec, v[j], z1, z2);
    } else {
#pragma unroll
        for (int j = 0; j < kTile; j++) {
            const int64_t i = i0 + j;
            v[j] = (i >= 0 && i < len) ? sos_step(sec, v[j], z1, z2) : 0.0f;
        }
    }
    float* dst = s < 3 ? ring + (s * 2 + cur) * kRegion : tout;
#pragma unroll
    for (int j = 0; j < kTile; j += 4) *reinterpret_cast<float4*>(dst + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
    // the tile of the next batch, fetched one batch ago
#pragma unroll
    for (int k = 0; k < per; k++) {
        const int64_t i = base + kTile + s * per + k;
        tin[(cur ^ 1) * kRegion + s * per + k] = i < len ? cook(staged[k], i) : 0.0f;
    }
    __syncwarp();
#pragma unroll
    for (int k = 0; k < per; k++) {
        const int64_t i = base - 3 * kTile + s * per + k;
        if (i >= 0 && i < len) store(i, tout[s * per + k]);
    }
    __syncwarp();
}

template <typename Fetch, typename Cook, typename Store>
__device__ __forceinline__ void cascade(const ChromaCascade& c, int s, float* area, int64_t steps, int64_t len,
                                        float x0, Fetch fetch, Cook cook, Store store) {
    float* tin = area;                 // [2][kRegion]
    float* ring = area + 2 * kRegion;  // [3][2][kRegion]
    float* tout = ring + 6 * kRegion;  // [kRegion]
    float z1 = __fmul_rn(c.zi[s][0], x0), z2 = __fmul_rn(c.zi[s][1], x0);
    float sec[6];
#pragma unroll
    for (int k = 0; k < 6; k++) sec[k] = c.sec[s][k];
    constexpr int per = kTile / 4;
    uint32_t ra[per], rb[per];
#pragma unroll
    for (int k = 0; k < per; k++) {
        const int64_t i = s * per + k;
        tin[s * per + k] = i < len ? cook(fetch(i), i) : 0.0f;
        const int64_t i1 = kTile + s * per + k;
        ra[k] = i1 < len ? fetch(i1) : 0u;
    }
    __syncwarp();
    // two batches per trip so the staging registers alternate by name
    for (int64_t base = 0; base < steps; base += 2 * kTile) {
        cascade_batch(sec, z1, z2, s, tin, ring, tout, base, 0, len, rb, ra, fetch, cook, store);
        cascade_batch(sec, z1, z2, s, tin, ring, tout, base + kTile, 1, len, ra, rb, fetch, cook, store);
    }
}

// float sources: the raw word is the float's bits
__device__ __forceinline__ float as_f(uint32_t u) { return __uint_as_float(u); }
__device__ __forceinline__ uint32_t f_bits(float f) { return __float_as_uint(f); }

// ---------------------------------------------------------------- block stage

// The block stage runs the same section-per-lane cascade as cascade() above,
// with its input fed from a ring of 32-sample chunks that cp.async fills
// kRingDepth - 2 batches ahead (the latency of a global load is longer than
// a batch of the recurrence), the lane-to-lane hand-over in registers
// (shuffled as each output is made, consumed a batch later) and 16-byte stores
// of the last section's outputs.
constexpr int kExtBatches = kChromaExt / 32 + (kChromaExt % 32 != 0);
constexpr int kRingDepth = 8;                       // chunks in flight per block
constexpr int kRingSlot = 128;                      // bytes: 32 floats or 32 int16
constexpr int kRingBytes = kRingDepth * kRingSlot + 16;   // + 16: blocks start on different banks
constexpr int kBlockGroups = 32;                    // blocks per CTA (4 warps of 8 groups)
static_assert(kChromaRowStride == kExtBatches * 32, "scratch rows hold whole chunks");

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Forward input at extended position e near the ends of the block (odd
// extension: 2 x[0] - x[edge - e] before it, 2 x[last] - x[...] after it),
// read from the ring (chunk q holds source samples [32 (q - 1), 32 q)).
template <typename T>
__device__ __noinline__ float block_edge_input(const uint8_t* ring, int e, float first, float last) {
    if (e >= kChromaExt) return 0.0f;
    const bool lo = e < kChromaEdge, hi = e >= kChromaEdge + kBlock;
    const int i = lo ? kChromaEdge - e : hi ? kBlock - 2 - (e - kChromaEdge - kBlock) : e - kChromaEdge;
    const float x = (float)reinterpret_cast<const T*>(ring + (((i >> 5) + 1) % kRingDepth) * kRingSlot)[i & 31];
    return lo ? __fsub_rn(__fmul_rn(2.0f, first), x) : hi ? __fsub_rn(__fmul_rn(2.0f, last), x) : x;
}

// One pass of the block's 4-section cascade by its 4-lane group: lane s runs
// section s on batch k - s.  kMode 0: forward over the int16 block, 1: forward
// over the float block, 2: backward over the forward output in the row.
// The forward pass writes sample e at row[e]; the backward pass reads row[r]
// for sample kChromaExt - 1 - r and writes its output at row[r + kChromaRowShift]
// (every source position is in the ring long before a later sample's output
// lands on it).
template <int kMode>
__device__ __forceinline__ void block_pass(const float (&sec)[6], float zi0, float zi1, int s, bool active,
                                           const void* src, float* row, uint8_t* ring, float first, float last) {
    const uint32_t ring_s = (uint32_t)__cvta_generic_to_shared(ring);
    const float x0 = kMode == 2 ? row[kChromaExt - 1]
                                : __fsub_rn(__fmul_rn(2.0f, first),
                                            kMode == 0 ? (float)static_cast<const int16_t*>(src)[kChromaEdge]
                                                       : static_cast<const float*>(src)[kChromaEdge]);
    float z1 = __fmul_rn(zi0, x0), z2 = __fmul_rn(zi1, x0);
    // chunk q into slot q % depth: forward q = 1 .. kBlock/32 (source [32 (q-1), 32 q)),
    // backward q = 0 .. kExtBatches-1 (row floats [32 m, 32 m + 32), m = kExtBatches - 1 - q)
    auto issue = [&](int q) {
        if (active) {
            const uint32_t slot = ring_s + (q % kRingDepth) * kRingSlot;
            if (kMode == 0) {
                if (q >= 1 && q <= kBlock / 32)
                    cp_async16(slot + 16 * s, static_cast<const int16_t*>(src) + 32 * (q - 1) + 8 * s);
            } else if (kMode == 1) {
                if (q >= 1 && q <= kBlock / 32) {
                    const float* f = static_cast<const float*>(src) + 32 * (q - 1) + 4 * s;
                    cp_async16(slot + 16 * s, f);
                    cp_async16(slot + 64 + 16 * s, f + 16);
                }
            } else if (q >= 0 && q < kExtBatches) {
                const float* f = row + 32 * (kExtBatches - 1 - q) + 4 * s;
                cp_async16(slot + 16 * s, f);
                cp_async16(slot + 64 + 16 * s, f + 16);
            }
        }
        cp_async_commit();
    };
#pragma unroll
    for (int q = 0; q < kRingDepth - 1; q++) issue(q);
    float a[32], b[32];
#pragma unroll
    for (int q = 0; q < 32; q++) a[q] = b[q] = 0.0f;
    // batch k: chunks k and k + 1 are complete (the ones after them in flight)
    auto batch = [&](int k, float (&cur)[32], float (&nxt)[32]) {
        cp_async_wait<kRingDepth - 3>();
        __syncwarp();
        issue(k + kRingDepth - 1);   // into the slot of chunk k - 1, read last batch
        if (s == 0 && k < kExtBatches) {
            const uint8_t* r0 = ring + (k % kRingDepth) * kRingSlot;
            const uint8_t* r1 = ring + ((k + 1) % kRingDepth) * kRingSlot;
            if (kMode == 2) {
                constexpr int top = (kChromaExt - 1) % 32;
                const float* f0 = reinterpret_cast<const float*>(r0);
                const float* f1 = reinterpret_cast<const float*>(r1);
#pragma unroll
                for (int q = 0; q < 32; q++) cur[q] = q <= top ? f0[top - q] : f1[top + 32 - q];
            } else if (k >= 1 && k < kBlock / 32) {
                constexpr int lead = 32 - kChromaEdge;
                if (kMode == 0) {
                    const int16_t* h0 = reinterpret_cast<const int16_t*>(r0);
                    const int16_t* h1 = reinterpret_cast<const int16_t*>(r1);
#pragma unroll
                    for (int q = 0; q < 32; q++) cur[q] = (float)(q < kChromaEdge ? h0[q + lead] : h1[q - kChromaEdge]);
                } else {
                    const float* f0 = reinterpret_cast<const float*>(r0);
                    const float* f1 = reinterpret_cast<const float*>(r1);
#pragma unroll
                    for (int q = 0; q < 32; q++) cur[q] = q < kChromaEdge ? f0[q + lead] : f1[q - kChromaEdge];
                }
            } else {
#pragma unroll
                for (int q = 0; q < 32; q++)
                    cur[q] = kMode == 0 ? block_edge_input<int16_t>(ring, 32 * k + q, first, last)
                                        : block_edge_input<float>(ring, 32 * k + q, first, last);
            }
        }
        const int i0 = 32 * (k - s);
        if (i0 >= 0 && i0 + 32 <= kChromaExt) {
#pragma unroll
            for (int q = 0; q < 32; q++) {
                cur[q] = sos_step(sec, cur[q], z1, z2);
                nxt[q] = __shfl_up_sync(kFull, cur[q], 1, 4);
            }
        } else {
#pragma unroll
            for (int q = 0; q < 32; q++) {
                const int i = i0 + q;
                cur[q] = (i >= 0 && i < kChromaExt) ? sos_step(sec, cur[q], z1, z2) : 0.0f;
                nxt[q] = __shfl_up_sync(kFull, cur[q], 1, 4);
            }
        }
        const int kk = k - 3;   // the last section's batch
        if (s == 3 && active && kk >= 0 && kk < kExtBatches) {
            if (kMode != 2) {
#pragma unroll
                for (int u = 0; u < 8; u++)
                    *reinterpret_cast<float4*>(row + 32 * kk + 4 * u) =
                        make_float4(cur[4 * u], cur[4 * u + 1], cur[4 * u + 2], cur[4 * u + 3]);
            } else {
                const int base = kChromaExt + kChromaRowShift - 32 - 32 * kk;   // a multiple of 4
#pragma unroll
                for (int u = 0; u < 8; u++)
                    if (base + 4 * u >= 0)
                        *reinterpret_cast<float4*>(row + base + 4 * u) =
                            make_float4(cur[31 - 4 * u], cur[30 - 4 * u], cur[29 - 4 * u], cur[28 - 4 * u]);
            }
        }
    };
    constexpr int nb = kExtBatches + 3;
    for (int k = 0; k < nb; k += 2) {
        batch(k, a, b);
        batch(k + 1, b, a);
    }
    cp_async_wait_all();
}

// One 4-lane group per RF block: the forward pass over the odd extension of
// the block into its scratch row, then the backward pass in place.
__global__ void __launch_bounds__(4 * kBlockGroups) k_chroma_block_iir(ChromaBlockParams p) {
    __shared__ __align__(128) uint8_t rings[kBlockGroups * kRingBytes];
    const int s = threadIdx.x & 3, g = threadIdx.x >> 2;
    const int64_t j = (int64_t)blockIdx.x * kBlockGroups + g;
    const bool active = j < p.nblocks;
    const int64_t base = (p.first_block + (active ? j : 0)) * kStride;
    float* row = p.scratch + (active ? j : 0) * kChromaRowStride;
    uint8_t* ring = rings + g * kRingBytes;
    // section s of the cascade (selected with constant indices: a dynamic
    // index into the parameter block would copy it to local memory)
    float sec[6];
#pragma unroll
    for (int k = 0; k < 6; k++)
        sec[k] = s == 0 ? p.c.sec[0][k] : s == 1 ? p.c.sec[1][k] : s == 2 ? p.c.sec[2][k] : p.c.sec[3][k];
    const float zi0 = s == 0 ? p.c.zi[0][0] : s == 1 ? p.c.zi[1][0] : s == 2 ? p.c.zi[2][0] : p.c.zi[3][0];
    const float zi1 = s == 0 ? p.c.zi[0][1] : s == 1 ? p.c.zi[1][1] : s == 2 ? p.c.zi[2][1] : p.c.zi[3][1];
    if (p.rf32) {
        const float* x = p.rf32 + base;
        block_pass<1>(sec, zi0, zi1, s, active, x, row, ring, x[0], x[kBlock - 1]);
    } else {
        const int16_t* x = p.rf16 + base;
        block_pass<0>(sec, zi0, zi1, s, active, x, row, ring, (float)x[0], (float)x[kBlock - 1]);
    }
    // the forward outputs of lane 3 before the other lanes' copies of them
    __threadfence();
    __syncwarp();
    block_pass<2>(sec, zi0, zi1, s, active, nullptr, row, ring, 0.0f, 0.0f);
}

// One warp per block: the float mean of the rolled block in the reference's
// 32-accumulator order (lane a sums rolled samples a, a + 32, ... in order),
// then the stitched span minus the mean.
__global__ void __launch_bounds__(32) k_chroma_block_dc(ChromaBlockParams p) {
    const int64_t j = blockIdx.x;
    const int lane = threadIdx.x;
    const float* y = p.scratch + j * (int64_t)kChromaRowStride + kChromaEdge + kChromaRowShift;
    const int move = p.move;
    float acc = 0.0f;
    for (int i0 = 0; i0 < kBlock; i0 += 32 * 16) {
        float v[16];
#pragma unroll
        for (int q = 0; q < 16; q++) v[q] = y[(i0 + q * 32 + lane - move) & (kBlock - 1)];
#pragma unroll
        for (int q = 0; q < 16; q++) acc = __fadd_rn(acc, v[q]);
    }
    // lanes[l] = (acc[l] + acc[8 + l]) + (acc[16 + l] + acc[24 + l]), then a tree over 8 lanes
    float t = __fadd_rn(acc, __shfl_down_sync(kFull, acc, 8));
    float l8 = __fadd_rn(t, __shfl_down_sync(kFull, t, 16));
    for (int c = 8; c > 1; c /= 2) l8 = __fadd_rn(l8, __shfl_down_sync(kFull, l8, c / 2));
    const float mean = __fdiv_rn(__shfl_sync(kFull, l8, 0), (float)kBlock);
    float* out = p.out + (p.first_block + j) * kStride;
    for (int i0 = 0; i0 < kStride; i0 += 32 * 8) {
        float v[8];
#pragma unroll
        for (int q = 0; q < 8; q++) v[q] = y[(kCut + i0 + q * 32 + lane - move) & (kBlock - 1)];
#pragma unroll
        for (int q = 0; q < 8; q++) out[i0 + q * 32 + lane] = __fsub_rn(v[q], mean);
    }
}

// ---------------------------------------------------------------- burst probes

__device__ __forceinline__ double positive_degrees(double d) {
    double r = fmod(d, 360.0);
    return r < 0.0 ? r + 360.0 : r;
}

__device__ __forceinline__ int positive_mod4(int v) {
    int r = v % 4;
    return r < 0 ? r + 4 : r;
}

// One 4-lane group per (field, rotation sequence, line): the probe window of
// the line times the heterodyne of its phase rotation, the float32
// forward-backward final band-pass over it (odd extension, in shared memory),
// and the I/Q demodulation of the burst against the carrier tables.
__global__ void __launch_bounds__(128) k_chroma_probe(ChromaFieldParams p) {
    extern __shared__ float smem[];
    const int lane = threadIdx.x & 31, s = lane & 3;
    const int gi = threadIdx.x >> 2;   // group in the CTA
    const int64_t pid = (int64_t)blockIdx.x * (blockDim.x >> 2) + gi;
    const int64_t nprobe = (int64_t)p.nfields * 2 * p.out_lines;
    const bool active = pid < nprobe;
    const int64_t q = active ? pid : 0;
    const int f = (int)(q / (2 * p.out_lines));
    const int cnd = (int)((q / p.out_lines) % 2);
    const int pl = (int)(q % p.out_lines);   // sequence index; line = pl + 1
    const int edge = p.fin.edge;
    const int win = p.win;
    const int len = win + 2 * edge;
    const int lpad = (len + 3) & ~3;
    float* buf = smem + (size_t)gi * (lpad + kCascadeArea);
    float* tile = buf + lpad;
    const int64_t field = (int64_t)p.out_lines * p.outlen;
    const int rot = positive_mod4((cnd == 0 ? p.rot0 : p.rot1) * (pl + 1));
    const int64_t line_start = (int64_t)pl * p.outlen;
    const int64_t p0 = line_start + p.win0;
    const float* het = p.het + (int64_t)rot * field + p0;
    const float* ana = p.ana + ((int64_t)f * p.out_lines + pl) * win;
    // mixed samples into buf[edge .. edge + win), then the odd extension
    for (int i = s; i < win; i += 4) buf[edge + i] = __fmul_rn(het[i], ana[i]);
    __syncwarp();
    {
        const float first = buf[edge], last = buf[edge + win - 1];
        for (int e = s; e < edge; e += 4) {
            buf[e] = __fsub_rn(__fmul_rn(2.0f, first), buf[edge + edge - e]);
            buf[edge + win + e] = __fsub_rn(__fmul_rn(2.0f, last), buf[edge + win - 2 - e]);
        }
    }
    __syncwarp();
    const int64_t steps = len + 3 * kTile;
    cascade(p.fin, s, tile, steps, len, buf[0], [&](int64_t i) { return f_bits(buf[i]); },
            [](uint32_t raw, int64_t) { return as_f(raw); }, [&](int64_t i, float v) { buf[i] = v; });
    __syncwarp();
    const float xl = buf[len - 1];
    __syncwarp();
    cascade(p.fin, s, tile, steps, len, xl, [&](int64_t i) { return f_bits(buf[len - 1 - i]); },
            [](uint32_t raw, int64_t) { return as_f(raw); }, [&](int64_t i, float v) { buf[len - 1 - i] = v; });
    __syncwarp();
    // DemodBurstFloat32: burst = filtered[pad, win - pad), tables from line_start + bs
    const int pad = p.be - p.bs;
    const int n = win - 2 * pad;
    const float* burst = buf + edge + pad;
    const float* bc = p.bcos + line_start + p.bs;
    const float* bsn = p.bsin + line_start + p.bs;
    const int main_end = n & ~15, epi_end = n & ~3;
    double I[4] = {0, 0, 0, 0}, Q[4] = {0, 0, 0, 0};   // groups 0..3 of this lane
    for (int k = 0; k < main_end; k += 16) {
#pragma unroll
        for (int gr = 0; gr < 4; gr++) {
            const int idx = k + s + 4 * gr;
            const float sm = burst[idx];
            I[gr] = __dadd_rn(I[gr], (double)__fmul_rn(sm, bc[idx]));
            Q[gr] = __dadd_rn(Q[gr], (double)__fmul_rn(sm, bsn[idx]));
        }
    }
    const unsigned gmask = kFull;
    double li = __dadd_rn(__dadd_rn(__dadd_rn(I[1], I[0]), I[2]), I[3]);
    double lq = __dadd_rn(__dadd_rn(__dadd_rn(Q[1], Q[0]), Q[2]), Q[3]);
    auto fold4 = [&](double v) {
        // (l0 + l2) + (l1 + l3) within the group
        double v2 = __shfl_down_sync(gmask, v, 2, 4);
        double a = __dadd_rn(v, v2);   // lane 0: l0 + l2, lane 1: l1 + l3
        double b = __shfl_down_sync(gmask, a, 1, 4);
        return __shfl_sync(gmask, __dadd_rn(a, b), 0, 4);
    };
    double ic = fold4(li), qc = fold4(lq);
    if (epi_end > main_end) {
        double ei = s == 0 ? ic : 0.0, eq = s == 0 ? qc : 0.0;
        for (int k = main_end; k < epi_end; k += 4) {
            const float sm = burst[k + s];
            ei = __dadd_rn(ei, (double)__fmul_rn(sm, bc[k + s]));
            eq = __dadd_rn(eq, (double)__fmul_rn(sm, bsn[k + s]));
        }
        ic = fold4(ei);
        qc = fold4(eq);
    }
    if (s == 0 && active) {
        for (int k = epi_end; k < n; k++) {
            ic = __dadd_rn(ic, (double)__fmul_rn(burst[k], bc[k]));
            qc = __dadd_rn(qc, (double)__fmul_rn(burst[k], bsn[k]));
        }
        const int line = pl + 1;
        const double* loc = p.locs + (int64_t)f * p.lines;
        const double scale = pl < p.out_lines - 1 ? __ddiv_rn(__dsub_rn(loc[line + 1], loc[line]), (double)p.input_line)
                                                  : 1.0;
        double* o = p.probe + q * 5;
        o[0] = positive_degrees(atan2(qc, ic) * (180.0 / 3.141592653589793));
        o[1] = positive_degrees((double)p.bs * __fma_rn(-scale, 90.0, 90.0));
        o[2] = hypot(ic, qc);
        o[3] = ic;
        o[4] = qc;
    }
}

// ShouldFlipTrackPhase for each (field, rotation sequence): phase-step buckets
// between neighbouring lines away from the field edges.
__global__ void __launch_bounds__(128) k_chroma_flip(ChromaFieldParams p) {
    __shared__ int cnt[4];
    if (threadIdx.x < 4) cnt[threadIdx.x] = 0;
    __syncthreads();
    const int fc = blockIdx.x;   // field * 2 + sequence
    const double* pr = p.probe + (int64_t)fc * p.out_lines * 5;
    const int end = p.out_lines + 1;
    for (int k = 1 + threadIdx.x; k < p.out_lines; k += blockDim.x) {
        const int line = k + 1;
        if (line <= 16 || line >= end - 16) continue;
        double delta = positive_degrees(__dsub_rn(pr[k * 5], pr[(k - 1) * 5]));
        int bucket = ((int)floor(__dadd_rn(delta, 45.0) / 90.0)) % 4;
        atomicAdd(&cnt[bucket], 1);
    }
    __syncthreads();
    if (threadIdx.x == 0)
        p.flip[fc] = p.ntsc ? (cnt[0] < cnt[2]) : ((cnt[1] + cnt[3]) < (cnt[0] + cnt[2]));
}

// The rotation index runs from field to field: a field starts with index c
// and keeps sequence c, or the other one when that one flips; the next field
// starts with the other index unless the field flipped.
__global__ void k_chroma_chain(ChromaFieldParams p) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int c = *p.rot_in;
    for (int f = 0; f < p.nfields; f++) {
        const int fl = p.flip[f * 2 + c];
        p.chosen[f] = fl ? 1 - c : c;
        c = fl ? c : 1 - c;
    }
    *p.rot_out = c;
}

// SummarizePhaseSequence of each field's kept sequence: one warp per field,
// the normalised I/Q of every line in parallel, then the sums in line order.
__global__ void __launch_bounds__(128) k_chroma_summary(ChromaFieldParams p) {
    __shared__ double nrm[4][2][320];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int f = blockIdx.x * 4 + w;
    if (f >= p.nfields) return;
    const double* pr = p.probe + ((int64_t)f * 2 + p.chosen[f]) * p.out_lines * 5;
    const int end = p.out_lines + 1;
    const int nl = min(p.out_lines, 320);
    for (int k = lane; k < nl; k += 32) {
        const double mag = pr[k * 5 + 2];
        nrm[w][0][k] = mag != 0.0 ? __ddiv_rn(pr[k * 5 + 3], mag) : 0.0;
        nrm[w][1][k] = mag != 0.0 ? __ddiv_rn(pr[k * 5 + 4], mag) : 0.0;
    }
    __syncwarp();
    if (lane != 0) return;
    double ei = 0.0, eq = 0.0, oi = 0.0, oq = 0.0, msum = 0.0;
    int count = 0;
    for (int k = 0; k < nl; k++) {
        const int line = k + 1;
        const double mag = pr[k * 5 + 2];
        if (line <= 16 || line >= end - 16 || mag == 0.0) continue;
        count++;
        msum = __dadd_rn(msum, mag);
        if (line & 1) {
            oi = __dadd_rn(oi, nrm[w][0][k]);
            oq = __dadd_rn(oq, nrm[w][1][k]);
        } else {
            ei = __dadd_rn(ei, nrm[w][0][k]);
            eq = __dadd_rn(eq, nrm[w][1][k]);
        }
    }
    double* o = p.summary + (int64_t)f * 4;
    if (count == 0) {
        atomicExch(p.status, 1);
        o[0] = o[1] = o[2] = o[3] = 0.0;
        return;
    }
    const double k180 = 180.0, pi = 3.141592653589793;
    o[0] = positive_degrees(__ddiv_rn(__dmul_rn(atan2(__dadd_rn(eq, oq), __dadd_rn(ei, oi)), k180), pi));
    o[1] = positive_degrees(__ddiv_rn(__dmul_rn(atan2(eq, ei), k180), pi));
    o[2] = positive_degrees(__ddiv_rn(__dmul_rn(atan2(oq, oi), k180), pi));
    o[3] = __ddiv_rn(msum, (double)count);
}

// RefineLineLocationsFromBurst (v0.4.0) from sequence index 9 on, then the
// NTSC fsc shift of every location.
__global__ void k_chroma_refine(ChromaFieldParams p) {
    const int f = blockIdx.x;
    const double* loc = p.locs + (int64_t)f * p.lines;
    double* out = p.locs_out + (int64_t)f * p.lines;
    const double* pr = p.probe + ((int64_t)f * 2 + p.chosen[f]) * p.out_lines * 5;
    const double* sm = p.summary + (int64_t)f * 4;
    for (int L = threadIdx.x; L < p.lines; L += blockDim.x) {
        double v = loc[L];
        const int k = L - 1;
        if (k >= 9 && k < p.out_lines && L + 1 < p.lines) {
            const double target = p.ntsc ? sm[0] : ((L & 1) ? sm[2] : sm[1]);
            const double delta =
                __dsub_rn(positive_degrees(__dadd_rn(__dadd_rn(__dsub_rn(target, pr[k * 5]), pr[k * 5 + 1]), 180.0)),
                          180.0);
            const double scale = __ddiv_rn(__dsub_rn(loc[L + 1], loc[L]), (double)p.outlen);
            v = __dadd_rn(v, __dmul_rn(__dmul_rn(__ddiv_rn(delta, 360.0), p.fsc_ratio), scale));
        }
        out[L] = p.ntsc ? __dsub_rn(v, p.ntsc_shift) : v;
    }
}

// ---------------------------------------------------------------- field decode

// Up-conversion of one output line.  PAL: the line written by sequence entry
// L (NumPy slice of line L - first_line, negative indices from the end; the
// one that lands on -1 is empty) times the heterodyne of its rotation.  NTSC:
// the burst de-emphasis (x2 from burst end + 5) and the phase-compensated
// carrier -cos(theta), theta advanced per sample as the reference's four
// lanes do (closed form; cosine in float after an exact turn reduction).
__global__ void __launch_bounds__(256) k_chroma_upconvert(ChromaFieldParams p) {
    const int f = blockIdx.y;
    const int o = blockIdx.x;
    const int64_t field = (int64_t)p.out_lines * p.outlen;
    const int ofl = p.first_line[f];
    const float* src = p.cfield + (int64_t)f * field + (int64_t)o * p.outlen;
    float* dst = p.up + (int64_t)f * field + (int64_t)o * p.outlen;
    int L;
    if (o <= p.out_lines - ofl) L = o + ofl;
    else if (o >= p.out_lines + 1 - ofl && o < p.out_lines - 1) L = o + ofl - p.out_lines;
    else L = -1;
    if (L < 1 || L > p.out_lines) {
        for (int k = threadIdx.x; k < p.outlen; k += blockDim.x) dst[k] = 0.0f;
        return;
    }
    const int c = p.chosen[f];
    const int rot = positive_mod4((c == 0 ? p.rot0 : p.rot1) * L);
    if (!p.ntsc) {
        const float* het = p.het + (int64_t)rot * field + (int64_t)o * p.outlen;
        for (int k = threadIdx.x; k < p.outlen; k += blockDim.x) dst[k] = __fmul_rn(src[k], het[k]);
        return;
    }
    const double* pr = p.probe + ((int64_t)f * 2 + c) * p.out_lines * 5 + (int64_t)(L - 1) * 5;
    const double half_pi = 1.5707963267948966, deg = 0.017453292519943295;
    const double h = p.ntsc_h;
    (void)h;
    // NtscFieldPhaseTarget (:3915-3925): -33 degrees in the first colour frame
    // of the four-field sequence, 147 in the second, whatever the parity
    const bool second = ((p.field_number[f] / 2) & 1) == 1;
    const double target = second ? 147.0 : -33.0;
    const int64_t ls = (int64_t)(L - ofl) * p.outlen;
    double theta = __fma_rn((double)ls, h, (double)rot * half_pi);
    theta = __fma_rn(__dadd_rn(target, pr[0]), deg, theta);
    const int first_doubled = p.be + 5;
    const double two_pi = 6.283185307179586, inv_two_pi = 0.15915494309189535;
    // the line's start phase reduced by whole turns; each sample's advance
    // (the reference's four-lane theta steps, reduced the same way) is a table
    const double t0 = __fma_rn(-rint(__dmul_rn(theta, inv_two_pi)), two_pi, theta);
    for (int k = threadIdx.x; k < p.outlen; k += blockDim.x) {
        const float carrier = -cosf((float)__dadd_rn(t0, p.ntsc_advance[k]));
        float v = src[k];
        if (k >= first_doubled) v = __fmul_rn(v, 2.0f);   // burst de-emphasis, exact
        // the reference multiplies by the binary64 cosine and rounds to float;
        // with the float cosine the product agrees to float rounding
        dst[k] = __fmul_rn(v, carrier);
    }
}

// Final band-pass, forward: one 4-lane group per 1024-sample chunk of the odd
// extension of a field's up-converted chroma; chunks past the first
// kWarmup samples start kWarmup early from zero state.
__global__ void __launch_bounds__(32 * kIirWarps) k_chroma_final_fwd(ChromaFieldParams p, int64_t chunks_per_field) {
    __shared__ __align__(16) float tiles[kIirWarps * kGroupsPerWarp * kCascadeArea];
    const int lane = threadIdx.x & 31, s = lane & 3, g = lane >> 2;
    const int64_t gid = ((int64_t)blockIdx.x * kIirWarps + (threadIdx.x >> 5)) * kGroupsPerWarp + g;
    const bool active = gid < (int64_t)p.nfields * chunks_per_field;
    const int64_t q = active ? gid : 0;
    const int f = (int)(q / chunks_per_field);
    const int64_t ch = q % chunks_per_field;
    float* tile = tiles + ((threadIdx.x >> 5) * kGroupsPerWarp + g) * kCascadeArea;
    const int64_t field = (int64_t)p.out_lines * p.outlen;
    const int edge = p.fin.edge;
    const int64_t E = field + 2 * edge;
    const float* x = p.up + (int64_t)f * field;
    float* fwd = p.fwd + (int64_t)f * E;
    const float first = x[0], last = x[field - 1];
    auto fetch_e = [&](int64_t e) -> uint32_t {
        const int64_t i = e < edge ? edge - e : (e < edge + field ? e - edge : field - 2 - (e - edge - field));
        return f_bits(x[i]);
    };
    auto cook_e = [&](uint32_t raw, int64_t e) -> float {
        if (e < edge) return __fsub_rn(__fmul_rn(2.0f, first), as_f(raw));
        if (e < edge + field) return as_f(raw);
        return __fsub_rn(__fmul_rn(2.0f, last), as_f(raw));
    };
    const int64_t c0 = ch * kChunk, c1 = min(E, c0 + kChunk);
    const int64_t start = c0 <= kWarmup ? 0 : c0 - kWarmup;
    const int64_t len = active ? c1 - start : 0;
    const float x0 = start == 0 ? cook_e(fetch_e(0), 0) : 0.0f;
    cascade(p.fin, s, tile, (int64_t)kChunk + kWarmup + 3 * kTile, len, x0,
            [&](int64_t i) { return fetch_e(start + i); },
            [&](uint32_t raw, int64_t i) { return cook_e(raw, start + i); },
            [&](int64_t i, float v) {
                if (start + i >= c0) fwd[start + i] = v;
            });
}

// Final band-pass, backward over the forward output, chunks started kWarmup
// late from zero state except the last; the output samples land in `up`.
__global__ void __launch_bounds__(32 * kIirWarps) k_chroma_final_bwd(ChromaFieldParams p, int64_t chunks_per_field) {
    __shared__ __align__(16) float tiles[kIirWarps * kGroupsPerWarp * kCascadeArea];
    const int lane = threadIdx.x & 31, s = lane & 3, g = lane >> 2;
    const int64_t gid = ((int64_t)blockIdx.x * kIirWarps + (threadIdx.x >> 5)) * kGroupsPerWarp + g;
    const bool active = gid < (int64_t)p.nfields * chunks_per_field;
    const int64_t q = active ? gid : 0;
    const int f = (int)(q / chunks_per_field);
    const int64_t ch = q % chunks_per_field;
    float* tile = tiles + ((threadIdx.x >> 5) * kGroupsPerWarp + g) * kCascadeArea;
    const int64_t field = (int64_t)p.out_lines * p.outlen;
    const int edge = p.fin.edge;
    const int64_t E = field + 2 * edge;
    const float* fwd = p.fwd + (int64_t)f * E;
    float* y = p.up + (int64_t)f * field;
    const int64_t c0 = ch * kChunk, c1 = min(E, c0 + kChunk);
    const int64_t stop = c1 + kWarmup >= E ? E : c1 + kWarmup;   // exclusive upper end of the pass
    const int64_t len = active ? stop - c0 : 0;
    const float x0 = stop == E ? fwd[E - 1] : 0.0f;
    cascade(p.fin, s, tile, (int64_t)kChunk + kWarmup + 3 * kTile, len, x0,
            [&](int64_t i) { return f_bits(fwd[stop - 1 - i]); }, [](uint32_t raw, int64_t) { return as_f(raw); },
            [&](int64_t i, float v) {
                const int64_t e = stop - 1 - i;
                if (e < c1 && e >= edge && e < edge + field) y[e - edge] = v;
            });
}

__device__ __forceinline__ void two_sum_f(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ uint16_t u16_saturate(double shifted) {
    if (!isfinite(shifted) || shifted <= 0.0) return 0;
    if (shifted >= 65535.0) return 65535;
    return (uint16_t)shifted;
}

// The reference's scalar tail (the field's last n mod 4 samples): (ushort)(long)x.
__device__ __forceinline__ uint16_t u16_wrap(double shifted) {
    if (!isfinite(shifted) || shifted < -9223372036854775808.0 || shifted > 9223372036854775807.0) return 0;
    return (uint16_t)(uint64_t)(int64_t)shifted;
}

// ApplyAutomaticChromaGainWithCombToU16: lines below 16 neutral; from line 16
// the comb of the line with the lines `dist` before and after it (not for the
// last two lines), scaled so its burst RMS is burst_abs_ref.
__global__ void __launch_bounds__(256) k_chroma_gain(ChromaFieldParams p) {
    extern __shared__ float line[];
    __shared__ double scale_s;
    const int f = blockIdx.y, o = blockIdx.x;
    const int64_t field = (int64_t)p.out_lines * p.outlen;
    const float* x = p.up + (int64_t)f * field;
    uint16_t* out = p.out + (int64_t)f * field + (int64_t)o * p.outlen;
    if (o < 16) {
        for (int k = threadIdx.x; k < p.outlen; k += blockDim.x) out[k] = 32767;
        return;
    }
    const int dist = p.ntsc ? 1 : 2;
    const float* cur = x + (int64_t)o * p.outlen;
    if (o < p.out_lines - 2) {
        const float* adv = x + (int64_t)(o + dist) * p.outlen;
        const float* del = x + (int64_t)(o - dist) * p.outlen;
        for (int k = threadIdx.x; k < p.outlen; k += blockDim.x) {
            // ((2 cur - adv) - del) / 4 rounded to float: the binary64 sum of
            // these floats is exact, so take the exact sum as a float pair
            // (two TwoSums) and round it once; / 4 is exact
            float s1, e1, s2, e2;
            two_sum_f(__fmul_rn(cur[k], 2.0f), -adv[k], s1, e1);
            two_sum_f(s1, -del[k], s2, e2);
            line[k] = __fmul_rn(__fadd_rn(s2, __fadd_rn(e1, e2)), 0.25f);
        }
    } else {
        for (int k = threadIdx.x; k < p.outlen; k += blockDim.x) line[k] = cur[k];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        // RmsFloat32 (VhsChromaDecoder.cs:4400-4423)
        const int n = p.be - p.bs;
        float mean = 0.0f;
        for (int k = 0; k < n; k++) mean = __fadd_rn(mean, line[p.bs + k]);
        mean = __fdiv_rn(mean, (float)n);
        float ss = 0.0f;
        for (int k = 0; k < n; k++) {
            float c = __fsub_rn(line[p.bs + k], mean);
            ss = __fadd_rn(ss, __fmul_rn(c, c));
        }
        const float rms = n > 0 ? __fsqrt_rn(__fdiv_rn(ss, (float)n)) : 0.0f;
        scale_s = rms != 0.0f ? __ddiv_rn(p.burst_abs_ref, (double)rms) : 1.0;
    }
    __syncthreads();
    const double scale = scale_s;
    const int64_t vec_len = field & ~(int64_t)3;
    for (int k = threadIdx.x; k < p.outlen; k += blockDim.x) {
        const double shifted = __dadd_rn(__dmul_rn((double)line[k], scale), 32767.0);
        const int64_t gi = (int64_t)o * p.outlen + k;
        out[k] = gi < vec_len ? u16_saturate(shifted) : u16_wrap(shifted);
    }
}

}  // namespace

cudaError_t launch_chroma_blocks(const ChromaBlockParams& p, cudaStream_t s) {
    if (p.nblocks <= 0) return cudaSuccess;
    if (p.c.edge != kChromaEdge || (!p.rf32 && !p.rf16) ||
        (reinterpret_cast<uintptr_t>(p.rf32 ? (const void*)p.rf32 : (const void*)p.rf16) & 15u) != 0 ||
        (reinterpret_cast<uintptr_t>(p.scratch) & 15u) != 0)
        return cudaErrorInvalidValue;
    k_chroma_block_iir<<<(unsigned)((p.nblocks + kBlockGroups - 1) / kBlockGroups), 4 * kBlockGroups, 0, s>>>(p);
    k_chroma_block_dc<<<(unsigned)p.nblocks, 32, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_chroma_phase(const ChromaFieldParams& p, cudaStream_t s) {
    if (p.nfields <= 0) return cudaSuccess;
    const int64_t nprobe = (int64_t)p.nfields * 2 * p.out_lines;
    const int groups = 16;   // 64 threads
    const size_t smem = (size_t)groups * (((p.win + 2 * p.fin.edge + 3) & ~3) + kCascadeArea) * sizeof(float);
    k_chroma_probe<<<(unsigned)((nprobe + groups - 1) / groups), groups * 4, smem, s>>>(p);
    k_chroma_flip<<<(unsigned)(p.nfields * 2), 128, 0, s>>>(p);
    k_chroma_chain<<<1, 1, 0, s>>>(p);
    k_chroma_summary<<<(unsigned)((p.nfields + 3) / 4), 128, 0, s>>>(p);
    k_chroma_refine<<<(unsigned)p.nfields, 256, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_chroma_decode(const ChromaFieldParams& p, cudaStream_t s) {
    if (p.nfields <= 0) return cudaSuccess;
    dim3 lines(p.out_lines, p.nfields);
    k_chroma_upconvert<<<lines, 256, 0, s>>>(p);
    const int64_t field = (int64_t)p.out_lines * p.outlen;
    const int64_t chunks = (field + 2 * p.fin.edge + kChunk - 1) / kChunk;
    const int64_t groups = (int64_t)p.nfields * chunks;
    const int64_t per_cta = (int64_t)kIirWarps * kGroupsPerWarp;
    const unsigned grid = (unsigned)((groups + per_cta - 1) / per_cta);
    k_chroma_final_fwd<<<grid, 32 * kIirWarps, 0, s>>>(p, chunks);
    k_chroma_final_bwd<<<grid, 32 * kIirWarps, 0, s>>>(p, chunks);
    k_chroma_gain<<<lines, 256, (size_t)p.outlen * sizeof(float), s>>>(p);
    return cudaGetLastError();
}

}  // namespace vhsd
