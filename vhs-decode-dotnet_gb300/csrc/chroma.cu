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
// The final band-pass runs on 512-sample chunks, each started 384 samples
// early from zero state (the absolute sum of its impulse response beyond 384
// samples is below 1e-11 for PAL and NTSC, so the dropped history weighs
// under a thousandth of a float ulp), so it equals the sequential filter to
// float rounding rather than bit for bit.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "kernels.h"

namespace vhsd {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kChunk = 512;        // final band-pass chunk (a multiple of 32)
constexpr int kWarmup = 384;       // zero-state lead of a chunk (a multiple of 32)

__device__ __forceinline__ float sos_step(const float* c, float v, float& z1, float& z2) {
    float f = __fadd_rn(__fmul_rn(c[0], v), z1);
    z1 = __fadd_rn(__fsub_rn(__fmul_rn(c[1], v), __fmul_rn(c[4], f)), z2);
    z2 = __fsub_rn(__fmul_rn(c[2], v), __fmul_rn(c[5], f));
    return f;
}

// The 4-section cascade run by one lane: at step t section s filters sample
// t - s, so the four recurrences of a step are independent.  Each section
// sees its samples in order with its own state, so the outputs are those of
// the sample-by-sample loop.  The coefficients stay in the parameter bank
// (constant indices).
struct LaneCascade {
    float z[4][2];
    float v1, v2, v3;   // outputs of sections 0..2 waiting for the next section

    __device__ __forceinline__ void init(const ChromaCascade& c, float x0) {
#pragma unroll
        for (int q = 0; q < 4; q++) {
            z[q][0] = __fmul_rn(c.zi[q][0], x0);
            z[q][1] = __fmul_rn(c.zi[q][1], x0);
        }
        v1 = v2 = v3 = 0.0f;
    }
    // steps 0, 1, 2: only the sections that have a sample yet
    __device__ __forceinline__ void prime(const ChromaCascade& c, float x0, float x1, float x2) {
        v1 = sos_step(c.sec[0], x0, z[0][0], z[0][1]);
        v2 = sos_step(c.sec[1], v1, z[1][0], z[1][1]);
        v1 = sos_step(c.sec[0], x1, z[0][0], z[0][1]);
        v3 = sos_step(c.sec[2], v2, z[2][0], z[2][1]);
        v2 = sos_step(c.sec[1], v1, z[1][0], z[1][1]);
        v1 = sos_step(c.sec[0], x2, z[0][0], z[0][1]);
    }
    // step t >= 3: takes sample t, returns the cascade output of sample t - 3
    __device__ __forceinline__ float step(const ChromaCascade& c, float x) {
        const float y = sos_step(c.sec[3], v3, z[3][0], z[3][1]);
        v3 = sos_step(c.sec[2], v2, z[2][0], z[2][1]);
        v2 = sos_step(c.sec[1], v1, z[1][0], z[1][1]);
        v1 = sos_step(c.sec[0], x, z[0][0], z[0][1]);
        return y;
    }
};


// ---------------------------------------------------------------- block stage

// The block stage runs the 4-section cascade as a group of four lanes per
// block, lane s running section s one 32-sample batch behind lane s - 1,
// with its input fed from a ring of 32-sample chunks that cp.async fills
// kRingDepth - 2 batches ahead (the latency of a global load is longer than
// a batch of the recurrence), the lane-to-lane hand-over in registers
// (shuffled as each output is made, consumed a batch later) and 16-byte stores
// of the last section's outputs.
constexpr int kExtBatches = kChromaExt / 32 + (kChromaExt % 32 != 0);
constexpr int kRingDepth = 8;                       // chunks in flight per block
constexpr int kRingSlot = 128;                      // bytes: 32 floats or 32 int16
constexpr int kRingBytes = kRingDepth * kRingSlot + 16;   // + 16: blocks start on different banks
constexpr int kBlockGroups = 64;                    // blocks per CTA (8 warps of 8 groups): two warps per
                                                    // scheduler, so the stage holds few SMs beside the demod
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
    extern __shared__ __align__(128) uint8_t rings[];   // [kBlockGroups * kRingBytes]
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

constexpr int kProbeWinMax = 224;   // probe window samples (PAL 206, NTSC 174)

// One lane per (field, rotation sequence, line): the probe window of the
// line times the heterodyne of its phase rotation, the float32
// forward-backward final band-pass over it (odd extension, in place in the
// lane's shared-memory row; LaneCascade), and the I/Q demodulation of the
// burst against the carrier tables.  A warp fills its 32 rows together, each
// window read by the whole warp (coalesced); rows have an odd stride, so the
// lanes' own passes over their rows hit 32 different banks.
__global__ void __launch_bounds__(32) k_chroma_probe(ChromaFieldParams p) {
    extern __shared__ float smem[];
    const int lane = threadIdx.x;
    const int edge = p.fin.edge;
    const int win = p.win;
    const int len = win + 2 * edge;
    const int stride = len | 1;
    const int64_t nprobe = (int64_t)p.nfields * 2 * p.out_lines;
    const int64_t base = (int64_t)blockIdx.x * 32;
    const int64_t field = (int64_t)p.out_lines * p.outlen;
    // four probes' windows at a time, every load of them issued before the
    // products are stored (win <= kProbeWinMax)
    for (int j0 = 0; j0 < 32; j0 += 4) {
        const float* hp[4];
        const float* ap[4];
        bool ok[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int64_t qj = base + j0 + u;
            ok[u] = qj < nprobe;
            const int64_t qq = ok[u] ? qj : 0;
            const int fj = (int)(qq / (2 * p.out_lines));
            const int cj = (int)((qq / p.out_lines) % 2);
            const int lj = (int)(qq % p.out_lines);
            const int rot = positive_mod4((cj == 0 ? p.rot0 : p.rot1) * (lj + 1));
            hp[u] = p.het + (int64_t)rot * field + (int64_t)lj * p.outlen + p.win0;
            ap[u] = p.ana + ((int64_t)fj * p.out_lines + lj) * win;
        }
        float h[4][kProbeWinMax / 32], a[4][kProbeWinMax / 32];
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
            for (int m = 0; m < kProbeWinMax / 32; m++) {
                const int i = 32 * m + lane;
                const bool in = ok[u] && i < win;
                h[u][m] = in ? hp[u][i] : 0.0f;
                a[u][m] = in ? ap[u][i] : 0.0f;
            }
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
            for (int m = 0; m < kProbeWinMax / 32; m++) {
                const int i = 32 * m + lane;
                if (ok[u] && i < win) smem[(j0 + u) * stride + edge + i] = __fmul_rn(h[u][m], a[u][m]);
            }
    }
    __syncwarp();
    const bool active = base + lane < nprobe;
    const int64_t q = active ? base + lane : 0;
    const int f = (int)(q / (2 * p.out_lines));
    const int pl = (int)(q % p.out_lines);   // sequence index; line = pl + 1
    const int64_t line_start = (int64_t)pl * p.outlen;
    float* buf = smem + lane * stride;
    if (active) {
        const float first = buf[edge], last = buf[edge + win - 1];
        for (int e = 0; e < edge; e++) {
            buf[e] = __fsub_rn(__fmul_rn(2.0f, first), buf[2 * edge - e]);
            buf[edge + win + e] = __fsub_rn(__fmul_rn(2.0f, last), buf[edge + win - 2 - e]);
        }
        // in place over the row, forward then backward: sequence sample t at
        // row index pos(t); step t writes sample t - 3.  Tiles of 8 samples are
        // read a tile ahead (before the writes that reach them), so no step
        // waits on its shared-memory load.
        auto lane_pass = [&](auto pos) {
            LaneCascade lc;
            lc.init(p.fin, buf[pos(0)]);
            const int ntile = (len + 3 + 7) / 8;
            float x[8], nx[8];
#pragma unroll
            for (int j = 0; j < 8; j++) x[j] = buf[pos(j)];
            for (int k = 0; k < ntile; k++) {
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    const int t = 8 * (k + 1) + j;
                    nx[j] = t < len ? buf[pos(t)] : 0.0f;
                }
                int j0 = 0;
                if (k == 0) {
                    lc.prime(p.fin, x[0], x[1], x[2]);
                    j0 = 3;
                }
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    if (j < j0) continue;
                    const float y = lc.step(p.fin, x[j]);
                    const int u = 8 * k + j - 3;
                    if (u < len) buf[pos(u)] = y;
                }
#pragma unroll
                for (int j = 0; j < 8; j++) x[j] = nx[j];
            }
        };
        lane_pass([](int t) { return t; });
        lane_pass([len](int t) { return len - 1 - t; });
    }
    // DemodBurstFloat32: burst = filtered[pad, win - pad), tables from
    // line_start + bs; 16 accumulators (accumulator a takes samples
    // k + a), folded as the reference's lanes fold them, then the 4-wide
    // epilogue and the scalar tail
    if (!active) return;
    const int pad = p.be - p.bs;
    const int n = win - 2 * pad;
    const float* burst = buf + edge + pad;
    const float* bc = p.bcos + line_start + p.bs;
    const float* bsn = p.bsin + line_start + p.bs;
    const int main_end = n & ~15, epi_end = n & ~3;
    double I[16], Q[16];
#pragma unroll
    for (int a = 0; a < 16; a++) I[a] = Q[a] = 0.0;
    for (int k = 0; k < main_end; k += 16) {
#pragma unroll
        for (int a = 0; a < 16; a++) {
            const float sm = burst[k + a];
            I[a] = __dadd_rn(I[a], (double)__fmul_rn(sm, bc[k + a]));
            Q[a] = __dadd_rn(Q[a], (double)__fmul_rn(sm, bsn[k + a]));
        }
    }
    double li[4], lq[4];
#pragma unroll
    for (int g = 0; g < 4; g++) {
        li[g] = __dadd_rn(__dadd_rn(__dadd_rn(I[g + 4], I[g]), I[g + 8]), I[g + 12]);
        lq[g] = __dadd_rn(__dadd_rn(__dadd_rn(Q[g + 4], Q[g]), Q[g + 8]), Q[g + 12]);
    }
    double ic = __dadd_rn(__dadd_rn(li[0], li[2]), __dadd_rn(li[1], li[3]));
    double qc = __dadd_rn(__dadd_rn(lq[0], lq[2]), __dadd_rn(lq[1], lq[3]));
    if (epi_end > main_end) {
        double ei[4] = {ic, 0.0, 0.0, 0.0}, eq[4] = {qc, 0.0, 0.0, 0.0};
        for (int k = main_end; k < epi_end; k += 4) {
#pragma unroll
            for (int g = 0; g < 4; g++) {
                const float sm = burst[k + g];
                ei[g] = __dadd_rn(ei[g], (double)__fmul_rn(sm, bc[k + g]));
                eq[g] = __dadd_rn(eq[g], (double)__fmul_rn(sm, bsn[k + g]));
            }
        }
        ic = __dadd_rn(__dadd_rn(ei[0], ei[2]), __dadd_rn(ei[1], ei[3]));
        qc = __dadd_rn(__dadd_rn(eq[0], eq[2]), __dadd_rn(eq[1], eq[3]));
    }
    for (int k = epi_end; k < n; k++) {
        ic = __dadd_rn(ic, (double)__fmul_rn(burst[k], bc[k]));
        qc = __dadd_rn(qc, (double)__fmul_rn(burst[k], bsn[k]));
    }
    {
        const int line = pl + 1;
        const double* loc = p.locs + (int64_t)f * p.lines;
        const double scale = pl < p.out_lines - 1 ? __ddiv_rn(__dsub_rn(loc[line + 1], loc[line]), (double)p.input_line)
                                                  : 1.0;
        double* o = p.probe + q * 5;
        const double mag = hypot(ic, qc);
        o[0] = positive_degrees(atan2(qc, ic) * (180.0 / 3.141592653589793));
        o[1] = positive_degrees((double)p.bs * __fma_rn(-scale, 90.0, 90.0));
        o[2] = mag;
        o[3] = ic;
        o[4] = qc;
        // the normalised I/Q of the phase averages, divided here, a lane per
        // probe, instead of in the per-field summary
        p.probe_nrm[q * 2] = mag != 0.0 ? __ddiv_rn(ic, mag) : 0.0;
        p.probe_nrm[q * 2 + 1] = mag != 0.0 ? __ddiv_rn(qc, mag) : 0.0;
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
// the lines' normalised I/Q (divided by the probes) and magnitudes into shared
// memory, then the sums in line order.
__global__ void __launch_bounds__(32) k_chroma_summary(ChromaFieldParams p) {
    __shared__ double nrm[1][3][320];   // I / mag, Q / mag, mag
    const int w = 0, lane = threadIdx.x;
    const int f = blockIdx.x;
    if (f >= p.nfields) return;
    const int64_t row = ((int64_t)f * 2 + p.chosen[f]) * p.out_lines;
    const double* pr = p.probe + row * 5;
    const double* pn = p.probe_nrm + row * 2;
    const int end = p.out_lines + 1;
    const int nl = min(p.out_lines, 320);
    for (int k = lane; k < nl; k += 32) {
        nrm[w][0][k] = pn[k * 2];
        nrm[w][1][k] = pn[k * 2 + 1];
        nrm[w][2][k] = pr[k * 5 + 2];
    }
    __syncwarp();
    // Five ordered sums in line order, each in its own lane (lane 0: even-line
    // I, 1: even Q, 2: odd I, 3: odd Q, 4: magnitudes), so one binary64 add per
    // line serves all five chains.  The values come from shared memory only.
    const bool used = lane < 5;
    const int comp = lane == 4 ? 2 : (lane & 1);    // nrm row
    const int parity = lane < 2 ? 0 : 1;            // even lines: lanes 0, 1; odd: 2, 3
    double acc = 0.0;
    int count = 0;
    if (used) {
        for (int k = 0; k < nl; k++) {
            const int line = k + 1;
            const double mag = nrm[w][2][k];
            if (line <= 16 || line >= end - 16 || mag == 0.0) continue;
            count++;
            if (lane == 4 || (line & 1) == parity) acc = __dadd_rn(acc, nrm[w][comp][k]);
        }
    }
    const double ei = __shfl_sync(kFull, acc, 0), eq = __shfl_sync(kFull, acc, 1);
    const double oi = __shfl_sync(kFull, acc, 2), oq = __shfl_sync(kFull, acc, 3);
    const double msum = __shfl_sync(kFull, acc, 4);
    count = __shfl_sync(kFull, count, 4);
    double* o = p.summary + (int64_t)f * 4;
    if (count == 0) {
        if (lane == 0) {
            atomicExch(p.status, 1);
            o[0] = o[1] = o[2] = o[3] = 0.0;
        }
        return;
    }
    // the three phase averages in three lanes
    const double k180 = 180.0, pi = 3.141592653589793;
    if (lane < 3) {
        const double y = lane == 0 ? __dadd_rn(eq, oq) : lane == 1 ? eq : oq;
        const double x = lane == 0 ? __dadd_rn(ei, oi) : lane == 1 ? ei : oi;
        o[lane] = positive_degrees(__ddiv_rn(__dmul_rn(atan2(y, x), k180), pi));
    } else if (lane == 3) {
        o[3] = __ddiv_rn(msum, (double)count);
    }
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

// Knuth's TwoSum: s + e == a + b exactly.
__device__ __forceinline__ void two_sum_f(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}


// The sequence line L written to output line o (-1: none).  PAL follows the
// NumPy slice of line L - first_line with negative indices from the end; the
// one that lands on -1 is empty.
__device__ __forceinline__ int upconvert_source_line(const ChromaFieldParams& p, int o, int ofl) {
    int L;
    if (o <= p.out_lines - ofl) L = o + ofl;
    else if (o >= p.out_lines + 1 - ofl && o < p.out_lines - 1) L = o + ofl - p.out_lines;
    else L = -1;
    return (L < 1 || L > p.out_lines) ? -1 : L;
}

// NTSC, one lane per output line: the carrier phase theta at the line start
// (the reference's binary64 expression, reduced by whole turns) and its
// (cos, sin).  One lane per line keeps the binary64 work to one warp
// instruction per 32 lines.
__global__ void __launch_bounds__(128) k_chroma_up_lines(ChromaFieldParams p) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (!p.ntsc || id >= (int64_t)p.nfields * p.out_lines) return;
    const int f = (int)(id / p.out_lines), o = (int)(id % p.out_lines);
    const int ofl = p.first_line[f];
    const int L = upconvert_source_line(p, o, ofl);
    if (L < 0) {
        p.line_cs[id] = make_float2(1.0f, 0.0f);
        return;
    }
    const int c = p.chosen[f];
    const int rot = positive_mod4((c == 0 ? p.rot0 : p.rot1) * L);
    const double* pr = p.probe + ((int64_t)f * 2 + c) * p.out_lines * 5 + (int64_t)(L - 1) * 5;
    const double half_pi = 1.5707963267948966, deg = 0.017453292519943295;
    // NtscFieldPhaseTarget (:3915-3925): -33 degrees in the first colour frame
    // of the four-field sequence, 147 in the second, whatever the parity
    const bool second = ((p.field_number[f] / 2) & 1) == 1;
    const double target = second ? 147.0 : -33.0;
    const int64_t ls = (int64_t)(L - ofl) * p.outlen;
    double theta = __fma_rn((double)ls, p.ntsc_h, (double)rot * half_pi);
    theta = __fma_rn(__dadd_rn(target, pr[0]), deg, theta);
    const double two_pi = 6.283185307179586, inv_two_pi = 0.15915494309189535;
    const double t0 = __fma_rn(-rint(__dmul_rn(theta, inv_two_pi)), two_pi, theta);
    double sn, cs;
    sincos(t0, &sn, &cs);
    p.line_cs[id] = make_float2(__double2float_rn(cs), __double2float_rn(sn));
}

// Up-conversion of one output line.  PAL: the sequence line times the
// heterodyne of its rotation.  NTSC: the burst de-emphasis (x2 from burst end
// + 5) times the phase-compensated carrier -cos(theta_line + a_k), taken as
// -(cos theta_line cos a_k - sin theta_line sin a_k) from the line's and the
// per-sample (cos, sin); the reference multiplies by the binary64 cosine and
// rounds to float, which this agrees with to a few float ulps.
__global__ void __launch_bounds__(256) k_chroma_upconvert(ChromaFieldParams p) {
    const int f = blockIdx.y;
    const int o = blockIdx.x;
    const int64_t field = (int64_t)p.out_lines * p.outlen;
    const int ofl = p.first_line[f];
    const float* src = p.cfield + (int64_t)f * field + (int64_t)o * p.outlen;
    float* dst = p.up + (int64_t)f * p.crow + p.fin.edge + (int64_t)o * p.outlen;
    const int L = upconvert_source_line(p, o, ofl);
    if (L < 0) {
        for (int k = threadIdx.x; k < p.outlen; k += blockDim.x) dst[k] = 0.0f;
        return;
    }
    if (!p.ntsc) {
        const int c = p.chosen[f];
        const int rot = positive_mod4((c == 0 ? p.rot0 : p.rot1) * L);
        const float* het = p.het + (int64_t)rot * field + (int64_t)o * p.outlen;
        for (int k = threadIdx.x; k < p.outlen; k += blockDim.x) dst[k] = __fmul_rn(src[k], het[k]);
        return;
    }
    const float2 cs = p.line_cs[(int64_t)f * p.out_lines + o];
    const int first_doubled = p.be + 5;
    for (int k = threadIdx.x; k < p.outlen; k += blockDim.x) {
        const float2 a = p.ntsc_advance[k];
        const float carrier = __fsub_rn(__fmul_rn(cs.y, a.y), __fmul_rn(cs.x, a.x));
        float v = src[k];
        if (k >= first_doubled) v = __fmul_rn(v, 2.0f);   // burst de-emphasis, exact
        dst[k] = __fmul_rn(v, carrier);
    }
}

// The odd extension of each field's up-converted chroma in its row: edge
// samples before the field (2 x[0] - x[edge - e]) and after it, so the
// forward pass of the final band-pass reads one plain sequence.
__global__ void __launch_bounds__(64) k_chroma_extend(ChromaFieldParams p) {
    const int f = blockIdx.x;
    const int field = p.out_lines * p.outlen;
    const int edge = p.fin.edge;
    float* row = p.up + (int64_t)f * p.crow;
    const float first = row[edge], last = row[edge + field - 1];
    for (int e = threadIdx.x; e < edge; e += blockDim.x) {
        row[e] = __fsub_rn(__fmul_rn(2.0f, first), row[2 * edge - e]);
        row[edge + field + e] = __fsub_rn(__fmul_rn(2.0f, last), row[edge + field - 2 - e]);
    }
}

// The final band-pass over the odd-extended field, E = field + 2 edge
// samples, in chunks of kChunk samples each started kWarmup samples early
// from zero state (the first from the reference's initial state), one lane
// per chunk (LaneCascade).  kFwd: the forward pass over the extended row of
// up, written in reverse order into fwd; else the backward pass, i.e. the
// same recurrence over that reversed sequence, written back in reverse into
// up at the field's samples.  Sample t of a pass's sequence lands at row
// position E - 1 - t.  A lane's tiles of 32 samples are whole 128-byte lines
// (chunk starts are multiples of 32), read with 16-byte loads a tile ahead
// into registers; outputs leave in 16-byte stores, aligned for kM = E mod 4.
// One copy of the tile body keeps the loop in the instruction cache.
template <bool kFwd, int kM>
__global__ void __launch_bounds__(128) k_chroma_final(ChromaFieldParams p, int chunks_per_field) {
    const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = gid < (int64_t)p.nfields * chunks_per_field;
    const int64_t q = active ? gid : 0;
    const int f = (int)(q / chunks_per_field);
    const int ch = (int)(q % chunks_per_field);
    const int field = p.out_lines * p.outlen;
    const int edge = p.fin.edge;
    const int E = field + 2 * edge;
    const float* src = (kFwd ? p.up : p.fwd) + (int64_t)f * p.crow;
    float* dst = (kFwd ? p.fwd : p.up) + (int64_t)f * p.crow;
    const int c0 = ch * kChunk, c1 = min(E, c0 + kChunk);
    const int start = c0 <= kWarmup ? 0 : c0 - kWarmup;
    const int n = active ? c1 - start : 0;
    // outputs kept: sequence samples [lo, hi) of this lane's run
    int lo = c0 - start, hi = c1 - start;
    if (!kFwd) {
        lo = max(c0, edge) - start;
        hi = min(c1, E - edge) - start;
    }
    if (!active) hi = lo;
    const float* run = src + start;
    LaneCascade lc;
    lc.init(p.fin, start != 0 ? 0.0f : run[0]);
    const int ntile = __reduce_max_sync(kFull, (n + 3 + 31) / 32);
    constexpr int JH = (kM + 2) & 3;   // top sample of each aligned group of four outputs
    constexpr int NC = 3 - JH;         // outputs carried into the next tile's first group
    float cr[3] = {0.0f, 0.0f, 0.0f};
    // a lane touches no tile past its own run (steps up to n + 2), so every
    // access stays inside its row (crow >= E + 64)
    auto has = [&](int k) { return 32 * k <= n + 2; };
    auto load = [&](int k, float (&x)[32]) {
        if (has(k)) {
            const float4* in4 = reinterpret_cast<const float4*>(run + 32 * k);
#pragma unroll
            for (int g = 0; g < 8; g++) {
                const float4 v = in4[g];
                x[4 * g] = v.x; x[4 * g + 1] = v.y; x[4 * g + 2] = v.z; x[4 * g + 3] = v.w;
            }
        }
    };
    float x[32], nx[32];
#pragma unroll
    for (int j = 0; j < 32; j++) x[j] = nx[j] = 0.0f;
    load(0, x);
    for (int k = 0; k < ntile; k++) {
        load(k + 1, nx);   // a tile ahead: in flight while this tile runs
        int j0 = 0;
        if (k == 0) {
            lc.prime(p.fin, x[0], x[1], x[2]);
            x[0] = x[1] = x[2] = 0.0f;
            j0 = 3;
        }
        // x[j] becomes the output of sample 32 k + j - 3
#pragma unroll
        for (int j = 0; j < 32; j++)
            if (j >= j0) x[j] = lc.step(p.fin, x[j]);
#pragma unroll
        for (int g = 0; JH + 4 * g <= 31; g++) {
            const int jt = JH + 4 * g;
            float v[4];
#pragma unroll
            for (int m = 0; m < 4; m++) v[m] = jt - m >= 0 ? x[jt - m] : cr[NC + jt - m];
            const int ut = 32 * k + jt - 3;   // the group's samples ut - 3 .. ut
            float* d = dst + (E - 1 - start - ut);
            if (ut - 3 >= lo && ut < hi) {
                *reinterpret_cast<float4*>(d) = make_float4(v[0], v[1], v[2], v[3]);
            } else if (ut >= lo && ut - 3 < hi) {
#pragma unroll
                for (int m = 0; m < 4; m++)
                    if (ut - m >= lo && ut - m < hi) d[m] = v[m];
            }
        }
#pragma unroll
        for (int i = 0; i < NC; i++) cr[i] = x[32 - NC + i];
#pragma unroll
        for (int j = 0; j < 32; j++) x[j] = nx[j];
    }
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

// uint16 of (double)v * scale + 32767 as the reference converts it (saturated,
// truncated).  The value is formed as a float pair (Dekker's product of v and
// scale split into two floats, then TwoSum with 32767): it differs from the
// binary64 value by < 1e-9 for every in-range sample, so the floor is the
// same unless the value lies within 1e-6 of an integer; those samples and
// non-finite inputs take the binary64 path.
__device__ __forceinline__ uint16_t gain_u16(float v, float sh, float sl, double scale) {
    if (isfinite(v)) {
        const float ph = __fmul_rn(v, sh);
        const float pl = __fmaf_rn(v, sl, __fmaf_rn(v, sh, -ph));
        float s, e;
        two_sum_f(ph, 32767.0f, s, e);
        const float lo = __fadd_rn(e, pl);
        const float hi = __fadd_rn(s, lo);
        const float lo2 = __fsub_rn(lo, __fsub_rn(hi, s));
        const float r = rintf(hi);
        const float d = __fadd_rn(__fsub_rn(hi, r), lo2);   // value - r
        if (fabsf(d) > 1e-6f && fabsf(hi) < 1e9f) {
            const float fl = d > 0.0f ? r : __fsub_rn(r, 1.0f);
            return (uint16_t)fminf(fmaxf(fl, 0.0f), 65535.0f);
        }
    }
    return u16_saturate(__dadd_rn(__dmul_rn((double)v, scale), 32767.0));
}

// The comb of output line o at sample k: ((2 cur - adv) - del) / 4 with the
// lines `dist` after and before it (not for the last two lines).  The
// reference sums these floats in binary64, where the sum is exact, and rounds
// to float: the exact sum as a float pair (two TwoSums) rounded once; / 4 is
// exact.
__device__ __forceinline__ float comb_at(const float* x, int o, int k, const ChromaFieldParams& p) {
    const float* cur = x + (int64_t)o * p.outlen;
    if (o >= p.out_lines - 2) return cur[k];
    const int dist = p.ntsc ? 1 : 2;
    const float adv = x[(int64_t)(o + dist) * p.outlen + k], del = x[(int64_t)(o - dist) * p.outlen + k];
    float s1, e1, s2, e2;
    two_sum_f(__fmul_rn(cur[k], 2.0f), -adv, s1, e1);
    two_sum_f(s1, -del, s2, e2);
    return __fmul_rn(__fadd_rn(s2, __fadd_rn(e1, e2)), 0.25f);
}

// ApplyAutomaticChromaGainWithCombToU16, per line from 16: the RMS of the
// combed burst window (RmsFloat32, VhsChromaDecoder.cs:4400-4423, in its
// order) and the scale that brings it to burst_abs_ref, in binary64 and as a
// float pair.  A warp takes 32 lines: the combed windows of all of them
// together (independent loads), then each lane the ordered sums and the
// binary64 division of its own line.
constexpr int kBurstMax = 64;   // burst window samples (PAL 56, NTSC 52)
__global__ void __launch_bounds__(32) k_chroma_gain_lines(ChromaFieldParams p) {
    __shared__ float comb[32][kBurstMax + 1];
    const int lane = threadIdx.x;
    const int64_t total = (int64_t)p.nfields * p.out_lines;
    const int64_t id0 = (int64_t)blockIdx.x * 32;
    const int n = p.be - p.bs;
    {
        // eight lines at a time, every load of them issued before the sums
        // are stored (n <= kBurstMax = 64: two samples per lane per line)
        const int f0 = (int)(id0 / p.out_lines), o0 = (int)(id0 % p.out_lines);
        for (int j0 = 0; j0 < 32; j0 += 8) {
            float v[8][2];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                int f = f0, o = o0 + j0 + u;   // 32 lines cross at most one field end
                if (o >= p.out_lines) {
                    o -= p.out_lines;
                    f++;
                }
                const bool line_ok = id0 + j0 + u < total && o >= 16;
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int k = lane + 32 * h;
                    v[u][h] = line_ok && k < n ? comb_at(p.up + (int64_t)f * p.crow + p.fin.edge, o, p.bs + k, p)
                                               : 0.0f;
                }
            }
#pragma unroll
            for (int u = 0; u < 8; u++)
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int k = lane + 32 * h;
                    if (k < n) comb[j0 + u][k] = v[u][h];
                }
        }
    }
    __syncwarp();
    const int64_t id = id0 + lane;
    if (id >= total || (int)(id % p.out_lines) < 16) return;
    float mean = 0.0f;
    for (int k = 0; k < n; k++) mean = __fadd_rn(mean, comb[lane][k]);
    mean = __fdiv_rn(mean, (float)n);
    float ss = 0.0f;
    for (int k = 0; k < n; k++) {
        const float c = __fsub_rn(comb[lane][k], mean);
        ss = __fadd_rn(ss, __fmul_rn(c, c));
    }
    const float rms = n > 0 ? __fsqrt_rn(__fdiv_rn(ss, (float)n)) : 0.0f;
    const double scale = rms != 0.0f ? __ddiv_rn(p.burst_abs_ref, (double)rms) : 1.0;
    const float sh = __double2float_rn(scale);
    p.line_scale[id] = scale;
    p.line_scale_f[id] = make_float2(sh, __double2float_rn(__dsub_rn(scale, (double)sh)));
}

// The uint16 chroma: lines below 16 neutral (32767), the others combed and
// scaled by their line's gain.
__global__ void __launch_bounds__(320) k_chroma_gain(ChromaFieldParams p) {
    const int f = blockIdx.y, o = blockIdx.x;
    const int64_t field = (int64_t)p.out_lines * p.outlen;
    const float* x = p.up + (int64_t)f * p.crow + p.fin.edge;
    uint16_t* out = p.out + (int64_t)f * field + (int64_t)o * p.outlen;
    if (o < 16) {
        for (int k = threadIdx.x; k < p.outlen; k += blockDim.x) out[k] = 32767;
        return;
    }
    const int64_t id = (int64_t)f * p.out_lines + o;
    const double scale = p.line_scale[id];
    const float2 sp = p.line_scale_f[id];
    const int64_t vec_len = field & ~(int64_t)3;
    // four samples per thread (blockDim.x >= outlen / 4), their loads issued together
    float v[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
        const int k = threadIdx.x + u * blockDim.x;
        v[u] = k < p.outlen ? comb_at(x, o, k, p) : 0.0f;
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
        const int k = threadIdx.x + u * blockDim.x;
        if (k >= p.outlen) continue;
        const int64_t gi = (int64_t)o * p.outlen + k;
        out[k] = gi < vec_len ? gain_u16(v[u], sp.x, sp.y, scale)
                              : u16_wrap(__dadd_rn(__dmul_rn((double)v[u], scale), 32767.0));
    }
}

}  // namespace

int chroma_block_ctas(int64_t nblocks) { return (int)((nblocks + kBlockGroups - 1) / kBlockGroups); }

cudaError_t prepare_chroma_kernels() {
    // the block stage's rings above the default 48 KB of shared memory; all of
    // the SM's shared memory for the probe rows, so a decode's probe warps fit
    // in one wave
    cudaError_t e = cudaFuncSetAttribute(k_chroma_block_iir, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         kBlockGroups * kRingBytes);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_chroma_probe, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
}

cudaError_t launch_chroma_blocks(const ChromaBlockParams& p, cudaStream_t s) {
    if (p.nblocks <= 0) return cudaSuccess;
    if (p.c.edge != kChromaEdge || (!p.rf32 && !p.rf16) ||
        (reinterpret_cast<uintptr_t>(p.rf32 ? (const void*)p.rf32 : (const void*)p.rf16) & 15u) != 0 ||
        (reinterpret_cast<uintptr_t>(p.scratch) & 15u) != 0)
        return cudaErrorInvalidValue;
    constexpr int smem = kBlockGroups * kRingBytes;   // opted in by prepare_chroma_kernels
    k_chroma_block_iir<<<(unsigned)((p.nblocks + kBlockGroups - 1) / kBlockGroups), 4 * kBlockGroups, smem, s>>>(p);
    k_chroma_block_dc<<<(unsigned)p.nblocks, 32, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_chroma_phase(const ChromaFieldParams& p, cudaStream_t s) {
    if (p.nfields <= 0) return cudaSuccess;
    if (p.win > kProbeWinMax || p.win <= 32) return cudaErrorInvalidValue;
    const int64_t nprobe = (int64_t)p.nfields * 2 * p.out_lines;
    const size_t smem = (size_t)32 * ((p.win + 2 * p.fin.edge) | 1) * sizeof(float);
    k_chroma_probe<<<(unsigned)((nprobe + 31) / 32), 32, smem, s>>>(p);
    k_chroma_flip<<<(unsigned)(p.nfields * 2), 128, 0, s>>>(p);
    k_chroma_chain<<<1, 1, 0, s>>>(p);
    // one warp per field, each on its own SM: the binary64 divisions and
    // ordered sums share an SM's few FP64 units with nothing else
    k_chroma_summary<<<(unsigned)p.nfields, 32, 0, s>>>(p);
    k_chroma_refine<<<(unsigned)p.nfields, 256, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_chroma_decode(const ChromaFieldParams& p, cudaStream_t s) {
    if (p.nfields <= 0) return cudaSuccess;
    if (p.be - p.bs > kBurstMax || p.be <= p.bs || p.outlen > 4 * 320) return cudaErrorInvalidValue;
    dim3 lines(p.out_lines, p.nfields);
    const unsigned line_grid = (unsigned)(((int64_t)p.nfields * p.out_lines + 127) / 128);
    k_chroma_up_lines<<<line_grid, 128, 0, s>>>(p);   // NTSC only (returns at once for PAL)
    k_chroma_upconvert<<<lines, 256, 0, s>>>(p);
    const int64_t field = (int64_t)p.out_lines * p.outlen;
    const int64_t E = field + 2 * p.fin.edge;
    const int chunks = (int)((E + kChunk - 1) / kChunk);
    const unsigned grid = (unsigned)(((int64_t)p.nfields * chunks + 127) / 128);
    if (p.crow != chroma_final_row(field, p.fin.edge) || (reinterpret_cast<uintptr_t>(p.up) & 15u) != 0 ||
        (reinterpret_cast<uintptr_t>(p.fwd) & 15u) != 0 || E > (int64_t)1 << 30)
        return cudaErrorInvalidValue;
    k_chroma_extend<<<(unsigned)p.nfields, 64, 0, s>>>(p);
    switch ((int)(E & 3)) {
    case 0: k_chroma_final<true, 0><<<grid, 128, 0, s>>>(p, chunks); k_chroma_final<false, 0><<<grid, 128, 0, s>>>(p, chunks); break;
    case 1: k_chroma_final<true, 1><<<grid, 128, 0, s>>>(p, chunks); k_chroma_final<false, 1><<<grid, 128, 0, s>>>(p, chunks); break;
    case 2: k_chroma_final<true, 2><<<grid, 128, 0, s>>>(p, chunks); k_chroma_final<false, 2><<<grid, 128, 0, s>>>(p, chunks); break;
    default: k_chroma_final<true, 3><<<grid, 128, 0, s>>>(p, chunks); k_chroma_final<false, 3><<<grid, 128, 0, s>>>(p, chunks); break;
    }
    k_chroma_gain_lines<<<(unsigned)(((int64_t)p.nfields * p.out_lines + 31) / 32), 32, 0, s>>>(p);
    const int gain_threads = ((p.outlen + 3) / 4 + 31) / 32 * 32;   // four samples per thread
    k_chroma_gain<<<lines, gain_threads, 0, s>>>(p);
    return cudaGetLastError();
}

}  // namespace vhsd
