// Learned fixed-rate bound selection.
//
// The reference picks a fixed-rate bound by searching an analytic ratio
// model on every 10th block (szx/src/szx_float.cc:501-584, 684-832, 921-949)
// and never checks the ratio it gets.  Here the bound comes from the codec's
// exact byte count on every 10th block (a sampled ratio curve, resolved to
// 1/64 of a binade) corrected by a small MLP: from 32 features of the sampled
// blocks the network predicts by how much the whole field's ratio will miss
// the target at the sampled curve's crossing, log2(real / target), and the
// bound is the sampled crossing for the target divided by that miss.  A real
// compress pass (of the whole batch of fields at once) judges the bound, a
// field that misses by more than the tolerance gets one refined bound (the
// sampled crossing re-targeted by the miss it measured), and plain bisection
// over real compress passes is the fallback after that -- and, run alone, the
// baseline.
//
// Features of a (field, target) row (float data, blocks of 128 values, every
// 10th full block sampled; kF floats), with y = log2(bound / sampled range):
//   0       log2(target)
//   1       ys: where the sampled ratio curve crosses the target (finest level)
//   2       the curve's slope there, d log2(ratio) / d y
//   3       the second sample's curve at ys, relative to the target (see below)
//   4       yu: start of the 1/64-step window
//   5..12   quarter-step curve at y = yq - 1 .. yq + 0.75, relative to the target
//   13..28  1/64-step curve at y = yu + j/64, j = 0..15, relative to the target
//   29      fraction of coarse blocks (every 40th block) with radius 0
//   30      log2(values) / 26;  31  log2(sampled blocks + 1) / 20
// The sampled ratio at a bound is 4 * values / bytes with the codec's exact
// byte count on the sampled blocks (constant block: 4-byte median; otherwise
// a 5-byte header, 2-bit lead codes and the bytes left after the XOR leads,
// szx/src/szx_float.cc:49-252) plus one state bit per block.  The crossing is
// found in three passes, 16 probes each: y = -1.5j per field over every 4th
// sampled block (coarse), then per row a window of quarter steps around the
// coarse crossing, then 1/64 steps across the quarter step that brackets the
// target.  A second, disjoint sample -- every 10th full block from block 5
// on -- is evaluated at the same 1/64 probes; its curve at ys (interpolated)
// tells how far the first sample's crossing is off from what a twice larger
// sample sees: information the first sample's curve does not hold, which
// lets the network predict part of the sampling miss.
// Every probe bound is range * 2^(m/64) for an integer m, rounded
// the same way everywhere, and all sums are integers (deterministic atomics).
// A non-constant block's bytes change only where the bound crosses a power of
// two, so the curve is a staircase with smooth parts from the constant
// blocks; the 1/64 steps resolve both well inside the 5% tolerance.
//
// Network: 32 -> 64 -> 64 -> 64 -> 1, GELU, fp32, inputs standardised by the
// training set's mean / deviation; output: the predicted miss
// log2(real ratio / target) at the crossing ys (feature 1).
// Parameters (floats):
//   [0,32) mean, [32,64) deviation, then W1[64][32] b1[64] W2[64][64] b2[64]
//   W3[64][64] b3[64] W4[64] b4.
// Training: mean squared error, Adam; each CTA of the forward/backward kernel
// takes 32 samples, writes its gradient partials, and the update kernel sums
// them in a fixed order (runs are bit-reproducible).
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <random>
#include <vector>

#include "../../include/szx_gb300.h"
#include "batch.h"
#include "common.cuh"

using namespace szxg;

namespace {

constexpr int kF = 32;              // features
constexpr int kH = 64;              // hidden width
constexpr int kProbes = 16;         // coarse probes, y = -1.5 j (j = 1..16)
constexpr int kFine = 16;           // fine probes, y = yq + (k - 8) / 4
constexpr int kRate = 10;           // every 10th block sampled
constexpr int kTileBlocks = 32;     // sampled blocks per warp tile
constexpr int kCoarseStep = 4;      // the coarse curve uses every 4th sampled block (every 40th block)
constexpr int kAcc = 18;            // per field, over the coarse blocks: count, bytes[16], radius-0 blocks
constexpr int A_NS = 0, A_BYTES = 1, A_ZERO = 17;
constexpr int kRowAcc = 48;         // per row: quarter-step bytes[16], 1/64-step bytes[16], second sample's [16]
constexpr int kOff2 = 5;            // the second sample: blocks 5, 15, 25, ...
constexpr int kQMin = -100, kQMax = 4;   // quarter-step window centre, quarters of y
constexpr double kBracketStop = 1.0 / 1024;   // searches stop on a measured bracket this narrow

// parameter offsets
constexpr int P_MU = 0, P_SD = 32, P_W1 = 64, P_B1 = P_W1 + kH * kF, P_W2 = P_B1 + kH, P_B2 = P_W2 + kH * kH,
              P_W3 = P_B2 + kH, P_B3 = P_W3 + kH * kH, P_W4 = P_B3 + kH, P_B4 = P_W4 + kH, P_TOTAL = P_B4 + 1;
constexpr int P_TRAIN0 = P_W1, P_NTRAIN = P_TOTAL - P_W1;

__constant__ float c_probe[kProbes];   // 2^(-1.5 j), j = 1..16, rounded to float
__constant__ float c_frac64[64];       // 2^(i / 64), rounded to float

}  // namespace

// ------------------------------------------------------------------ features

struct LfxField {
    const float* x;
    unsigned long long n, ns, tile0;   // values, sampled blocks, first launch-wide tile
    unsigned long long ns2;            // blocks of the second sample (<= ns)
};

struct LfxWork {
    void* dev = nullptr;
    LfxField* d_f = nullptr;
    unsigned long long* acc = nullptr;   // [nf][kAcc]
    uint32_t* mm = nullptr;              // [nf][2] ordered-int min, max
    float* range = nullptr;              // [nf]
    int* rows = nullptr;                 // [cap_rows] field of each feature row
    float* tgt = nullptr;                // [cap_rows]
    int* mq = nullptr;                   // [cap_rows] quarter-step window start (1/64 units of y)
    int* mu = nullptr;                   // [cap_rows] 1/64-step window start
    unsigned long long* racc = nullptr;  // [cap_rows][kRowAcc]
    unsigned long long* rtile0 = nullptr;   // [cap_rows + 1] first (row, tile) item of each row
    float* X = nullptr;                  // [cap_rows][kF]
    float* pred = nullptr;               // [cap_rows]
    size_t cap_rows = 0;
    unsigned long long tiles = 0;
    std::vector<unsigned long long> ftiles;   // tiles of each field
};

void lfx_free(LfxWork* w) {
    if (!w) return;
    if (w->dev) cudaFree(w->dev);
    delete w;
}

namespace {

__device__ __forceinline__ uint32_t ord_f32(float v) {
    const uint32_t u = __float_as_uint(v);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float f32_ord(uint32_t o) {
    return __uint_as_float((o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o);
}

// 2^e for -126 <= e <= 127, exactly
__device__ __forceinline__ float pow2_int(int e) { return __int_as_float((127 + e) << 23); }

// range * 2^(m/64), rounded as range * 2^(frac/64) then scaled exactly
__device__ __forceinline__ float probe_bound(float range, int m) {
    const int fr = m & 63;
    return __fmul_rn(__fmul_rn(range, c_frac64[fr]), pow2_int((m - fr) / 64));
}

// last index i in [0, n) with key[i] <= g (key ascending, key[0] <= g)
template <typename K>
__device__ __forceinline__ int upper_index(const K* key, size_t stride_bytes, int n, unsigned long long g) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        const unsigned long long k = *(const unsigned long long*)((const uint8_t*)key + (size_t)mid * stride_bytes);
        if (k <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Sampled min / max of every field (one warp per tile of sampled blocks).
template <int BS>
__global__ void k_lfx_range(const LfxField* F, int nf, unsigned long long tiles, uint32_t* mm) {
    const int lane = threadIdx.x & 31;
    const unsigned long long w0 = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) >> 5;
    const unsigned long long nw = (gridDim.x * (unsigned long long)blockDim.x) >> 5;
    for (unsigned long long g = w0; g < tiles; g += nw) {
        const int f = upper_index(&F[0].tile0, sizeof(LfxField), nf, g);
        const LfxField D = F[f];
        const unsigned long long k0 = (g - D.tile0) * kTileBlocks;
        const unsigned long long k1 = min(k0 + kTileBlocks, D.ns);
        uint32_t lo = 0xFFFFFFFFu, hi = 0u;
        for (unsigned long long k = k0; k < k1; k++) {
            const float* p = D.x + k * kRate * BS;
            for (int i = lane; i < BS; i += 32) {
                const float v = p[i];
                if (v == v) {
                    lo = min(lo, ord_f32(v));
                    hi = max(hi, ord_f32(v));
                }
            }
        }
        lo = __reduce_min_sync(0xffffffffu, lo);
        hi = __reduce_max_sync(0xffffffffu, hi);
        if (lane == 0) {
            atomicMin(&mm[2 * f], lo);
            atomicMax(&mm[2 * f + 1], hi);
        }
    }
}

__device__ __forceinline__ float lfx_range_of(const uint32_t* mm, int f) {
    const uint32_t lo = mm[2 * f], hi = mm[2 * f + 1];
    if (lo > hi) return 0.f;   // no finite sample
    return __fsub_rn(f32_ord(hi), f32_ord(lo));
}

// Values 4*lane .. 4*lane+3 of sampled block k (128 values) and the block's
// radius and median as the codec computes them.
__device__ __forceinline__ void lfx_block(const float* x, unsigned long long k, int lane, float v[4], float* r,
                                          float* med, int off = 0) {
    const float* p = x + (k * kRate + off) * 128 + 4 * lane;
    if (((uintptr_t)x & 15) == 0) {
        const float4 q = *(const float4*)p;
        v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
    } else {
#pragma unroll
        for (int i = 0; i < 4; i++) v[i] = p[i];
    }
    float mn = fminf(fminf(v[0], v[1]), fminf(v[2], v[3]));
    float mx = fmaxf(fmaxf(v[0], v[1]), fmaxf(v[2], v[3]));
#pragma unroll
    for (int d = 16; d; d >>= 1) {
        mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, d));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, d));
    }
    *r = __fmul_rn(__fsub_rn(mx, mn), 0.5f);
    *med = __fadd_rn(mn, *r);
}

// reqLength of a non-constant block at bound eb, 33 standing for "above 32"
// (clamped to 32 with the median zeroed): the byte count's cache key.
__device__ __forceinline__ int lfx_req_key(float eb, float r) {
    const int q = 10 + exponent_f32(r) - exponent_f64_of_f32(eb);
    return q < 9 ? 9 : (q > 32 ? 33 : q);
}

// This lane's share of a non-constant block's stream bytes for reqLength key
// `key` (lane 0 carries the fixed part).  Called by the whole warp.
__device__ __forceinline__ uint32_t lfx_bytes_nc(const float v[4], float med, int key, int lane) {
    int R, s;
    split_reqlen(key > 32 ? 32 : key, &R, &s);
    const float m = key > 32 ? 0.f : med;
    uint32_t cur[4];
#pragma unroll
    for (int i = 0; i < 4; i++) cur[i] = __float_as_uint(__fsub_rn(v[i], m)) >> s;
    uint32_t prev = __shfl_up_sync(0xffffffffu, cur[3], 1);
    if (lane == 0) prev = 0;
    uint32_t st = 0;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int ld = Elem<float>::lead(cur[i] ^ (i ? cur[i - 1] : prev));
        st += ld < R ? (uint32_t)(R - ld) : 0u;
    }
    return st + (lane == 0 ? 5u + 128 / 4 : 0u);
}

// Add the block's bytes at every bound eb[0..N) to bytes[]: a
// constant block costs its 4-byte median; a non-constant block's count
// depends on the bound only through its reqLength, which changes only where
// the bound crosses a power of two, so it is computed once per distinct key.
// r is the same in every lane: all lanes take the same branches.
template <int N>
__device__ __forceinline__ void lfx_block_bytes(const float v[4], float r, float med, const float* eb,
                                                uint32_t* bytes, int lane) {
    int last = -1;
    uint32_t cached = 0;
#pragma unroll
    for (int j = 0; j < N; j++) {
        if (r <= eb[j]) {
            bytes[j] += lane == 0 ? 4u : 0u;
        } else {
            const int key = lfx_req_key(eb[j], r);
            if (key != last) {
                cached = lfx_bytes_nc(v, med, key, lane);
                last = key;
            }
            bytes[j] += cached;
        }
    }
}

__device__ __forceinline__ void lfx_flush(unsigned long long* dst, uint32_t v, int lane) {
    v = __reduce_add_sync(0xffffffffu, v);
    if (lane == 0 && v) atomicAdd(dst, (unsigned long long)v);
}

// Per-field sums (slots A_*) over every kCoarseStep-th sampled block: their
// count, bytes at the coarse probes, blocks of radius 0.  The coarse curve
// only places the quarter-step window.  A warp owns a tile of sampled blocks
// of one field (tiles start at multiples of kTileBlocks).
__global__ void __launch_bounds__(256) k_lfx_accumulate(const LfxField* F, int nf, unsigned long long tiles,
                                                        const uint32_t* mm, unsigned long long* acc) {
    const int lane = threadIdx.x & 31;
    const unsigned long long w0 = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) >> 5;
    const unsigned long long nw = (gridDim.x * (unsigned long long)blockDim.x) >> 5;
    for (unsigned long long g = w0; g < tiles; g += nw) {
        const int f = upper_index(&F[0].tile0, sizeof(LfxField), nf, g);
        const LfxField D = F[f];
        const float range = lfx_range_of(mm, f);
        float eb[kProbes];
#pragma unroll
        for (int j = 0; j < kProbes; j++) eb[j] = __fmul_rn(range, c_probe[j]);
        uint32_t bytes[kProbes], zero = 0, nsb = 0;
#pragma unroll
        for (int j = 0; j < kProbes; j++) bytes[j] = 0;
        const unsigned long long k0 = (g - D.tile0) * kTileBlocks;
        const unsigned long long k1 = min(k0 + kTileBlocks, D.ns);
        for (unsigned long long k = k0; k < k1; k += kCoarseStep) {
            float v[4], r, med;
            lfx_block(D.x, k, lane, v, &r, &med);
            if (lane == 0) {
                nsb++;
                zero += r == 0.f;
            }
            lfx_block_bytes<kProbes>(v, r, med, eb, bytes, lane);
        }
        unsigned long long* a = acc + (size_t)f * kAcc;
        lfx_flush(a + A_NS, nsb, lane);
#pragma unroll
        for (int j = 0; j < kProbes; j++) lfx_flush(a + A_BYTES + j, bytes[j], lane);
        lfx_flush(a + A_ZERO, zero, lane);
    }
}

__device__ __forceinline__ double lfx_log2_ratio(double bytes, double ns) {
    return log2(4.0 * 128.0 * ns / (bytes + ns / 8.0));
}

// Quarter-step window of every row: 16 probes at mq + 16k (1/64 units of y),
// centred on where the coarse curve crosses the target (clamped; above the
// largest or below the smallest coarse bound when the target is outside it).
__global__ void k_lfx_center(const unsigned long long* acc, int nrows, const int* rows, const float* tgt, int* mq) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrows) return;
    const unsigned long long* a = acc + (size_t)rows[r] * kAcc;
    const double ns = (double)a[A_NS];
    const double lt = log2((double)tgt[r]);
    double yc = -12.0;
    if (ns > 0) {
        double cprev = lfx_log2_ratio((double)a[A_BYTES], ns) - lt;   // j = 1, y = -1.5
        if (cprev < 0) {
            yc = -1.0;
        } else {
            yc = -24.0;
            for (int j = 1; j < kProbes; j++) {
                const double c = lfx_log2_ratio((double)a[A_BYTES + j], ns) - lt;
                if (c < 0) {   // crossed between y = -1.5 j and -1.5 (j + 1)
                    yc = -1.5 * j - 1.5 * cprev / (cprev - c);
                    break;
                }
                cprev = c;
            }
        }
    }
    int q = (int)floor(yc * 4.0 + 0.5);
    q = q < kQMin ? kQMin : (q > kQMax ? kQMax : q);
    mq[r] = 16 * q - 128;
}

// 1/64-step window of every row: the quarter step [k, k+1] of the quarter
// window where the curve crosses the target (the first or last step when it
// does not cross inside the window).
__global__ void k_lfx_center2(const LfxField* F, const unsigned long long* racc, int nrows, const int* rows,
                              const float* tgt, const int* mq, int* mu) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrows) return;
    const double ns = (double)F[rows[r]].ns;
    const unsigned long long* ra = racc + (size_t)r * kRowAcc;
    const double lt = log2((double)tgt[r]);
    int kx = 0;
    if (ns > 0) {
        if (lfx_log2_ratio((double)ra[kFine - 1], ns) - lt < 0) {
            kx = kFine - 1;
        } else {
            for (int k = 0; k + 1 < kFine; k++)
                if (lfx_log2_ratio((double)ra[k], ns) - lt < 0 && lfx_log2_ratio((double)ra[k + 1], ns) - lt >= 0) {
                    kx = k;
                    break;
                }
        }
    }
    mu[r] = mq[r] + 16 * kx;
}

// Per-row byte sums at 16 probes m = mstart[r] + stride * k into racc[r][slot..]:
// items (row, tile of the row's field).
__global__ void __launch_bounds__(256) k_lfx_probe(const LfxField* F, const uint32_t* mm, int nrows, const int* rows,
                                                   const int* mstart, int stride, const unsigned long long* rtile0,
                                                   unsigned long long items, unsigned long long* racc, int slot,
                                                   int off) {
    const int lane = threadIdx.x & 31;
    const unsigned long long w0 = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) >> 5;
    const unsigned long long nw = (gridDim.x * (unsigned long long)blockDim.x) >> 5;
    for (unsigned long long g = w0; g < items; g += nw) {
        const int r = upper_index(rtile0, sizeof(unsigned long long), nrows, g);
        const int f = rows[r];
        const LfxField D = F[f];
        const float range = lfx_range_of(mm, f);
        const int m0 = mstart[r];
        float eb[kFine];
#pragma unroll
        for (int k = 0; k < kFine; k++) eb[k] = probe_bound(range, m0 + stride * k);
        uint32_t bytes[kFine];
#pragma unroll
        for (int k = 0; k < kFine; k++) bytes[k] = 0;
        // the second sample's blocks are tiled like the first's (ns2 <= ns)
        const unsigned long long k0 = (g - rtile0[r]) * kTileBlocks;
        const unsigned long long k1 = min(k0 + kTileBlocks, off ? D.ns2 : D.ns);
        for (unsigned long long k = k0; k < k1; k++) {
            float v[4], rr, med;
            lfx_block(D.x, k, lane, v, &rr, &med, off);
            lfx_block_bytes<kFine>(v, rr, med, eb, bytes, lane);
        }
        unsigned long long* a = racc + (size_t)r * kRowAcc + slot;
#pragma unroll
        for (int j = 0; j < kFine; j++) lfx_flush(a + j, bytes[j], lane);
    }
}

// The feature row of every (field, target) row.
__global__ void k_lfx_rows(const LfxField* F, const unsigned long long* acc, const uint32_t* mm, int nrows,
                           const int* rows, const float* tgt, const int* mq, const int* mu,
                           const unsigned long long* racc, float* X, float* range_out, int nf) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < nf) range_out[r] = lfx_range_of(mm, r);
    if (r >= nrows) return;
    const int f = rows[r];
    const unsigned long long* a = acc + (size_t)f * kAcc;
    const unsigned long long* ra = racc + (size_t)r * kRowAcc;
    float* x = X + (size_t)r * kF;
    const double lt = log2((double)tgt[r]);
    const double ns = (double)F[f].ns, nc = (double)a[A_NS];
    const double yq = (mq[r] + 128) / 64.0, yu = mu[r] / 64.0;
    // 1/64-step curve, closed by the quarter-step probe at its end
    double u[kFine + 1];
    for (int j = 0; j < kFine; j++) u[j] = ns > 0 ? lfx_log2_ratio((double)ra[kFine + j], ns) - lt : 0.0;
    const int kx = (mu[r] - mq[r]) / 16;
    u[kFine] = (ns > 0 && kx + 1 < kFine) ? lfx_log2_ratio((double)ra[kx + 1], ns) - lt : u[kFine - 1];
    double ys = yu, slope = 0.0;
    if (ns > 0) {
        if (u[0] >= 0) {
            ys = yu;
        } else if (u[kFine] < 0) {
            ys = yu + kFine / 64.0;
        } else {
            for (int j = 0; j < kFine; j++)
                if (u[j] < 0 && u[j + 1] >= 0) {
                    ys = yu + (j + (-u[j]) / (u[j + 1] - u[j])) / 64.0;
                    slope = (u[j + 1] - u[j]) * 64.0;
                    break;
                }
        }
    }
    x[0] = (float)lt;
    x[1] = (float)ys;
    x[2] = (float)fmin(slope, 256.0);
    // the second sample's curve at ys: linear between its 1/64 probes (held
    // at the window's ends outside it)
    double ub = 0.0;
    const double ns2 = (double)F[f].ns2;
    if (ns2 > 0) {
        const double pos = (ys - yu) * 64.0;
        const int j0 = pos <= 0 ? 0 : (pos >= kFine - 1 ? kFine - 2 : (int)floor(pos));
        const double w = pos <= 0 ? 0.0 : (pos >= kFine - 1 ? 1.0 : pos - j0);
        const double b0 = lfx_log2_ratio((double)ra[2 * kFine + j0], ns2) - lt;
        const double b1 = lfx_log2_ratio((double)ra[2 * kFine + j0 + 1], ns2) - lt;
        ub = b0 + (b1 - b0) * w;
    }
    (void)yq;
    x[3] = (float)ub;
    x[4] = (float)yu;
    for (int k = 0; k < 8; k++) x[5 + k] = ns > 0 ? (float)(lfx_log2_ratio((double)ra[4 + k], ns) - lt) : 0.f;
    for (int j = 0; j < kFine; j++) x[13 + j] = (float)u[j];
    x[29] = nc > 0 ? (float)(a[A_ZERO] / nc) : 0.f;
    x[30] = (float)(log2((double)F[f].n) / 26.0);
    x[31] = (float)(log2(ns + 1.0) / 20.0);
}

}  // namespace

// ------------------------------------------------------------------ MLP kernels

namespace {

constexpr int kS = 32;            // samples per CTA
constexpr int kMlpThreads = 256;
constexpr int LD1 = kF + 1, LDH = kH + 1;   // padded row strides in shared memory

struct MlpSmem {
    float W1[kH * LD1], W2[kH * LDH], W3[kH * LDH];
    float b1[kH], b2[kH], b3[kH], W4[kH], mu[kF], sd[kF];
    float a0[kS * LD1];
    float z1[kS * LDH], a1[kS * LDH], z2[kS * LDH], a2[kS * LDH], z3[kS * LDH], a3[kS * LDH];
    float t[kS * LDH];            // backward scratch
    float out[kS], g4[kS], yv[kS];
    float b4;
    int valid;
};

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_d(float z) {
    return 0.5f * (1.f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

// out[s][j] = b[j] + sum_i W[j][i] in[s][i]  (64 outputs, K inputs), optional GELU copy
template <int K, int LDW, int LDI>
__device__ __forceinline__ void layer_fwd(const float* W, const float* b, const float* in, float* z, float* a) {
    const int j = threadIdx.x & 63, sg = threadIdx.x >> 6;
    float acc[8];
#pragma unroll
    for (int k = 0; k < 8; k++) acc[k] = b[j];
#pragma unroll 8
    for (int i = 0; i < K; i++) {
        const float w = W[j * LDW + i];
#pragma unroll
        for (int k = 0; k < 8; k++) acc[k] = fmaf(w, in[(sg * 8 + k) * LDI + i], acc[k]);
    }
#pragma unroll
    for (int k = 0; k < 8; k++) {
        z[(sg * 8 + k) * LDH + j] = acc[k];
        a[(sg * 8 + k) * LDH + j] = gelu(acc[k]);
    }
}

// grad partials of a 64 x K weight matrix and its bias: dW[j][i] = sum_s dz[s][j] in[s][i]
template <int K, int LDI>
__device__ __forceinline__ void layer_wgrad(const float* dz, const float* in, float* gW, float* gb) {
    constexpr int PER = K / 4;
    const int j = threadIdx.x >> 2, i0 = (threadIdx.x & 3) * PER;
    float acc[PER];
    float bs = 0.f;
#pragma unroll
    for (int m = 0; m < PER; m++) acc[m] = 0.f;
    for (int s = 0; s < kS; s++) {
        const float d = dz[s * LDH + j];
        bs += d;
#pragma unroll
        for (int m = 0; m < PER; m++) acc[m] = fmaf(d, in[s * LDI + i0 + m], acc[m]);
    }
#pragma unroll
    for (int m = 0; m < PER; m++) gW[j * K + i0 + m] = acc[m];
    if ((threadIdx.x & 3) == 0) gb[j] = bs;
}

// dprev[s][i] = (sum_j W[j][i] dz[s][j]) * gelu'(zprev[s][i])   (64 x 64 weights)
__device__ __forceinline__ void layer_bwd_input(const float* W, const float* dz, const float* zprev, float* dprev) {
    const int i = threadIdx.x & 63, sg = threadIdx.x >> 6;
    float acc[8];
#pragma unroll
    for (int k = 0; k < 8; k++) acc[k] = 0.f;
#pragma unroll 8
    for (int j = 0; j < kH; j++) {
        const float w = W[j * LDH + i];
#pragma unroll
        for (int k = 0; k < 8; k++) acc[k] = fmaf(w, dz[(sg * 8 + k) * LDH + j], acc[k]);
    }
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const int s = sg * 8 + k;
        dprev[s * LDH + i] = acc[k] * gelu_d(zprev[s * LDH + i]);
    }
}

// Forward (and with BWD the backward) of kS samples per CTA.  rows (optional)
// picks the samples; pred (optional) receives the outputs; with BWD, part
// receives this CTA's gradient of sum_s (out_s - y_s)^2 * scale (P_NTRAIN
// floats, training-parameter order) and part_loss its sum of squares.
template <bool BWD>
__global__ void __launch_bounds__(kMlpThreads) k_mlp(const float* P, const float* X, const float* y, const int* rows,
                                                     int n, float scale, float* pred, float* part, float* part_loss) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    MlpSmem& S = *(MlpSmem*)smem_raw;
    const int tid = threadIdx.x;
    for (int e = tid; e < kH * kF; e += kMlpThreads) S.W1[(e / kF) * LD1 + e % kF] = P[P_W1 + e];
    for (int e = tid; e < kH * kH; e += kMlpThreads) {
        S.W2[(e / kH) * LDH + e % kH] = P[P_W2 + e];
        S.W3[(e / kH) * LDH + e % kH] = P[P_W3 + e];
    }
    if (tid < kH) {
        S.b1[tid] = P[P_B1 + tid];
        S.b2[tid] = P[P_B2 + tid];
        S.b3[tid] = P[P_B3 + tid];
        S.W4[tid] = P[P_W4 + tid];
    }
    if (tid < kF) {
        S.mu[tid] = P[P_MU + tid];
        S.sd[tid] = P[P_SD + tid];
    }
    if (tid == 0) S.b4 = P[P_B4];
    const long long base = (long long)blockIdx.x * kS;
    __syncthreads();
    for (int e = tid; e < kS * kF; e += kMlpThreads) {
        const int s = e / kF, i = e % kF;
        const long long g = base + s;
        float v = 0.f;
        if (g < n) {
            const long long r = rows ? rows[g] : g;
            v = (X[r * kF + i] - S.mu[i]) / S.sd[i];
        }
        S.a0[s * LD1 + i] = v;
    }
    if (tid < kS) {
        const long long g = base + tid;
        S.yv[tid] = 0.f;
        if (BWD && g < n) S.yv[tid] = y[rows ? rows[g] : g];
    }
    __syncthreads();
    layer_fwd<kF, LD1, LD1>(S.W1, S.b1, S.a0, S.z1, S.a1);
    __syncthreads();
    layer_fwd<kH, LDH, LDH>(S.W2, S.b2, S.a1, S.z2, S.a2);
    __syncthreads();
    layer_fwd<kH, LDH, LDH>(S.W3, S.b3, S.a2, S.z3, S.a3);
    __syncthreads();
    // output: warp w sums samples w, w+8, w+16, w+24 (lanes over the 64 inputs)
    {
        const int w = tid >> 5, lane = tid & 31;
        for (int s = w; s < kS; s += kMlpThreads / 32) {
            float v = S.W4[lane] * S.a3[s * LDH + lane] + S.W4[lane + 32] * S.a3[s * LDH + lane + 32];
#pragma unroll
            for (int d = 16; d; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
            if (lane == 0) {
                const float o = v + S.b4;
                S.out[s] = o;
                const bool ok = base + s < n;
                if (pred && ok) pred[base + s] = o;
                S.g4[s] = ok ? 2.f * (o - S.yv[s]) * scale : 0.f;
            }
        }
    }
    if (!BWD) return;
    __syncthreads();
    float* g = part + (size_t)blockIdx.x * P_NTRAIN;
    auto at = [&](int p) { return g + (p - P_TRAIN0); };
    if (tid < kH) {
        float acc = 0.f;
        for (int s = 0; s < kS; s++) acc = fmaf(S.g4[s], S.a3[s * LDH + tid], acc);
        *at(P_W4 + tid) = acc;
    }
    if (tid == kH) {
        float acc = 0.f;
        for (int s = 0; s < kS; s++) acc += S.g4[s];
        *at(P_B4) = acc;
    }
    if (tid == kH + 32) {
        float l = 0.f;
        for (int s = 0; s < kS; s++)
            if (base + s < n) {
                const float d = S.out[s] - S.yv[s];
                l = fmaf(d, d, l);
            }
        part_loss[blockIdx.x] = l;
    }
    // dz3 = g4 * W4 * gelu'(z3)  -> t
    for (int e = tid; e < kS * kH; e += kMlpThreads) {
        const int s = e / kH, j = e % kH;
        S.t[s * LDH + j] = S.g4[s] * S.W4[j] * gelu_d(S.z3[s * LDH + j]);
    }
    __syncthreads();
    layer_wgrad<kH, LDH>(S.t, S.a2, at(P_W3), at(P_B3));
    layer_bwd_input(S.W3, S.t, S.z2, S.a3);   // dz2 -> a3 (a3 no longer needed)
    __syncthreads();
    layer_wgrad<kH, LDH>(S.a3, S.a1, at(P_W2), at(P_B2));
    layer_bwd_input(S.W2, S.a3, S.z1, S.t);   // dz1 -> t
    __syncthreads();
    layer_wgrad<kF, LD1>(S.t, S.a0, at(P_W1), at(P_B1));
}

// Sum the CTA partials in order; optionally an Adam step on the parameters.
__global__ void k_mlp_reduce(const float* part, int nparts, const float* part_loss, float* grad, float* P, float* m,
                             float* v, float lr, float b1t, float b2t, float* loss_acc, int adam) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0 && loss_acc) {
        double l = 0;
        for (int c = 0; c < nparts; c++) l += part_loss[c];
        *loss_acc += (float)l;
    }
    if (p >= P_NTRAIN) return;
    float gsum = 0.f;
    for (int c = 0; c < nparts; c++) gsum += part[(size_t)c * P_NTRAIN + p];
    if (grad) grad[p] = gsum;
    if (!adam) return;
    const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
    const float mm = beta1 * m[p] + (1.f - beta1) * gsum;
    const float vv = beta2 * v[p] + (1.f - beta2) * gsum * gsum;
    m[p] = mm;
    v[p] = vv;
    const float mh = mm / (1.f - b1t), vh = vv / (1.f - b2t);
    P[P_TRAIN0 + p] -= lr * mh / (sqrtf(vh) + eps);
}

// Column mean / deviation of X (one CTA per feature) and the mean label (the
// output bias).
__global__ void k_mlp_stats(const float* X, const float* y, long long n, float* P) {
    __shared__ double s1[256], s2[256];
    const int c = blockIdx.x;
    double a = 0, b = 0;
    for (long long r = threadIdx.x; r < n; r += blockDim.x) {
        const double v = c < kF ? (double)X[r * kF + c] : (double)y[r];
        a += v;
        b += v * v;
    }
    s1[threadIdx.x] = a;
    s2[threadIdx.x] = b;
    __syncthreads();
    for (int d = blockDim.x / 2; d; d >>= 1) {
        if (threadIdx.x < d) {
            s1[threadIdx.x] += s1[threadIdx.x + d];
            s2[threadIdx.x] += s2[threadIdx.x + d];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double mean = s1[0] / (double)n;
        const double var = s2[0] / (double)n - mean * mean;
        if (c < kF) {
            P[P_MU + c] = (float)mean;
            P[P_SD + c] = (float)fmax(sqrt(fmax(var, 0.0)), 1e-3);
        } else {
            P[P_B4] = (float)mean;
        }
    }
}

}  // namespace

// ------------------------------------------------------------------ host objects

struct SZxG_Mlp {
    float* P = nullptr;     // device parameters [P_TOTAL]
    float* scratch = nullptr;
    size_t scratch_floats = 0;
};

namespace {

size_t mlp_smem() { return sizeof(MlpSmem); }

cudaError_t mlp_attr() {
    static bool done[64] = {false};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && !done[dev]) {
        cudaError_t e = cudaFuncSetAttribute(k_mlp<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mlp_smem());
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_mlp<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mlp_smem());
        if (e != cudaSuccess) return e;
        done[dev] = true;
    }
    return cudaSuccess;
}

// scratch for nctas gradient partials + their losses + grads + Adam moments + loss
cudaError_t mlp_scratch(SZxG_Mlp* m, size_t nctas) {
    const size_t need = nctas * P_NTRAIN + nctas + 3 * (size_t)P_NTRAIN + 64;
    if (m->scratch_floats >= need) return cudaSuccess;
    if (m->scratch) cudaFree(m->scratch);
    m->scratch = nullptr;
    m->scratch_floats = 0;
    cudaError_t e = cudaMalloc(&m->scratch, need * sizeof(float));
    if (e != cudaSuccess) return e;
    m->scratch_floats = need;
    return cudaSuccess;
}

struct Scr {
    float *part, *ploss, *grad, *m, *v, *loss;
};
Scr scr_of(SZxG_Mlp* m, size_t nctas) {
    Scr s;
    s.part = m->scratch;
    s.ploss = s.part + nctas * P_NTRAIN;
    s.grad = s.ploss + nctas;
    s.m = s.grad + P_NTRAIN;
    s.v = s.m + P_NTRAIN;
    s.loss = s.v + P_NTRAIN;
    return s;
}

int fail_code(cudaError_t) {
    cudaGetLastError();
    set_last_error(SZXG_ERR_CUDA);
    return SZXG_ERR_CUDA;
}

}  // namespace

extern "C" {

size_t SZxG_mlp_param_count(void) { return (size_t)P_TOTAL; }

SZxG_Mlp* SZxG_mlp_create(unsigned long long seed) {
    std::vector<float> h(P_TOTAL, 0.f);
    for (int i = 0; i < kF; i++) h[P_SD + i] = 1.f;
    std::mt19937_64 rng(seed);
    auto init = [&](int off, int fo, int fi) {
        const double a = sqrt(6.0 / (double)(fi + fo));
        std::uniform_real_distribution<double> u(-a, a);
        for (int k = 0; k < fo * fi; k++) h[off + k] = (float)u(rng);
    };
    init(P_W1, kH, kF);
    init(P_W2, kH, kH);
    init(P_W3, kH, kH);
    init(P_W4, 1, kH);
    SZxG_Mlp* m = new SZxG_Mlp();
    if (cudaMalloc(&m->P, sizeof(float) * P_TOTAL) != cudaSuccess ||
        cudaMemcpy(m->P, h.data(), sizeof(float) * P_TOTAL, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        if (m->P) cudaFree(m->P);
        delete m;
        set_last_error(SZXG_ERR_CUDA);
        return nullptr;
    }
    set_last_error(SZXG_OK);
    return m;
}

void SZxG_mlp_destroy(SZxG_Mlp* m) {
    if (!m) return;
    if (m->P) cudaFree(m->P);
    if (m->scratch) cudaFree(m->scratch);
    delete m;
}

int SZxG_mlp_get_params(const SZxG_Mlp* m, float* h_params, size_t count) {
    if (!m || !h_params || count < (size_t)P_TOTAL) { set_last_error(SZXG_ERR_ARG); return SZXG_ERR_ARG; }
    if (cudaMemcpy(h_params, m->P, sizeof(float) * P_TOTAL, cudaMemcpyDeviceToHost) != cudaSuccess)
        return fail_code(cudaErrorUnknown);
    set_last_error(SZXG_OK);
    return SZXG_OK;
}

int SZxG_mlp_set_params(SZxG_Mlp* m, const float* h_params, size_t count) {
    if (!m || !h_params || count != (size_t)P_TOTAL) { set_last_error(SZXG_ERR_ARG); return SZXG_ERR_ARG; }
    if (cudaMemcpy(m->P, h_params, sizeof(float) * P_TOTAL, cudaMemcpyHostToDevice) != cudaSuccess)
        return fail_code(cudaErrorUnknown);
    set_last_error(SZXG_OK);
    return SZXG_OK;
}

int SZxG_mlp_forward(const SZxG_Mlp* m, const float* d_X, size_t n, float* d_out, void* stream) {
    if (!m || !d_X || !d_out || n == 0 || n > (size_t)1 << 30) { set_last_error(SZXG_ERR_ARG); return SZXG_ERR_ARG; }
    cudaError_t e = mlp_attr();
    if (e != cudaSuccess) return fail_code(e);
    const int grid = (int)((n + kS - 1) / kS);
    {
        TraceScope tr("mlp_forward", (cudaStream_t)stream);
        k_mlp<false><<<grid, kMlpThreads, mlp_smem(), (cudaStream_t)stream>>>(m->P, d_X, nullptr, nullptr, (int)n,
                                                                              1.f, d_out, nullptr, nullptr);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return fail_code(e);
    set_last_error(SZXG_OK);
    return SZXG_OK;
}

// Gradient of the mean squared error over all n samples (training-parameter
// order: W1 b1 W2 b2 W3 b3 W4 b4) into d_grad; *h_loss = the mean squared error.
int SZxG_mlp_gradient(SZxG_Mlp* m, const float* d_X, const float* d_y, size_t n, float* d_grad, float* h_loss,
                      void* stream) {
    if (!m || !d_X || !d_y || !d_grad || n == 0 || n > (size_t)1 << 24) { set_last_error(SZXG_ERR_ARG); return SZXG_ERR_ARG; }
    cudaStream_t s = (cudaStream_t)stream;
    const size_t nctas = (n + kS - 1) / kS;
    cudaError_t e = mlp_attr();
    if (e == cudaSuccess) e = mlp_scratch(m, nctas);
    if (e != cudaSuccess) return fail_code(e);
    Scr S = scr_of(m, nctas);
    cudaMemsetAsync(S.loss, 0, sizeof(float), s);
    k_mlp<true><<<(int)nctas, kMlpThreads, mlp_smem(), s>>>(m->P, d_X, d_y, nullptr, (int)n, 1.f / (float)n, nullptr,
                                                            S.part, S.ploss);
    k_mlp_reduce<<<(P_NTRAIN + 255) / 256, 256, 0, s>>>(S.part, (int)nctas, S.ploss, d_grad, m->P, S.m, S.v, 0.f, 0.f,
                                                        0.f, S.loss, 0);
    float l = 0.f;
    if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaMemcpyAsync(&l, S.loss, sizeof(float),
                                                                        cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return fail_code(e);
    if (h_loss) *h_loss = l / (float)n;
    set_last_error(SZXG_OK);
    return SZXG_OK;
}

// Train on n rows (X [n][32], y [n]): the input statistics and the output
// bias are set from the data, then `epochs` passes of Adam over minibatches
// of `batch` rows in an order shuffled by `seed`.  *h_loss = mean squared
// error over the last epoch.
int SZxG_mlp_train(SZxG_Mlp* m, const float* d_X, const float* d_y, size_t n, int epochs, int batch, float lr,
                   unsigned long long seed, float* h_loss, void* stream) {
    if (!m || !d_X || !d_y || n < 2 || n > (size_t)1 << 24 || epochs < 1 || batch < kS || lr <= 0.f) {
        set_last_error(SZXG_ERR_ARG);
        return SZXG_ERR_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const size_t B = std::min((size_t)batch, n);
    const size_t nctas = (B + kS - 1) / kS;
    cudaError_t e = mlp_attr();
    if (e == cudaSuccess) e = mlp_scratch(m, nctas);
    if (e != cudaSuccess) return fail_code(e);
    Scr S = scr_of(m, nctas);
    int* d_rows = nullptr;
    if ((e = cudaMalloc(&d_rows, sizeof(int) * n)) != cudaSuccess) return fail_code(e);
    cudaMemsetAsync(S.m, 0, sizeof(float) * 2 * P_NTRAIN, s);
    k_mlp_stats<<<kF + 1, 256, 0, s>>>(d_X, d_y, (long long)n, m->P);
    std::vector<int> order(n);
    for (size_t i = 0; i < n; i++) order[i] = (int)i;
    std::mt19937_64 rng(seed);
    double b1t = 1.0, b2t = 1.0;
    float last = 0.f;
    for (int ep = 0; ep < epochs && e == cudaSuccess; ep++) {
        std::shuffle(order.begin(), order.end(), rng);
        e = cudaMemcpyAsync(d_rows, order.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s);
        cudaMemsetAsync(S.loss, 0, sizeof(float), s);
        for (size_t off = 0; off < n && e == cudaSuccess; off += B) {
            const size_t bn = std::min(B, n - off);
            b1t *= 0.9;
            b2t *= 0.999;
            k_mlp<true><<<(int)((bn + kS - 1) / kS), kMlpThreads, mlp_smem(), s>>>(
                m->P, d_X, d_y, d_rows + off, (int)bn, 1.f / (float)bn, nullptr, S.part, S.ploss);
            k_mlp_reduce<<<(P_NTRAIN + 255) / 256, 256, 0, s>>>(S.part, (int)((bn + kS - 1) / kS), S.ploss, nullptr,
                                                                m->P, S.m, S.v, lr, (float)b1t, (float)b2t, S.loss, 1);
            e = cudaGetLastError();
        }
        // (a pageable source is staged before the copy call returns: the host order can be reshuffled)
        if (e == cudaSuccess && ep == epochs - 1) {
            e = cudaMemcpyAsync(&last, S.loss, sizeof(float), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        }
    }
    cudaFree(d_rows);
    if (e != cudaSuccess) return fail_code(e);
    if (h_loss) *h_loss = last / (float)n;
    set_last_error(SZXG_OK);
    return SZXG_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ features on a compress batch

namespace {

cudaError_t lfx_prepare(SZxG_Batch* b, size_t rows) {
    LfxWork* w = b->lfx;
    const size_t nf = (size_t)b->nf;
    if (w && w->cap_rows >= rows) return cudaSuccess;
    if (w) {
        lfx_free(w);
        b->lfx = nullptr;
    }
    static bool consts_set[64] = {false};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && !consts_set[dev]) {
        float c[kProbes], q[64];
        for (int j = 0; j < kProbes; j++) c[j] = (float)exp2(-1.5 * (j + 1));
        for (int i = 0; i < 64; i++) q[i] = (float)exp2(i / 64.0);
        cudaError_t e = cudaMemcpyToSymbol(c_probe, c, sizeof c);
        if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_frac64, q, sizeof q);
        if (e != cudaSuccess) return e;
        consts_set[dev] = true;
    }
    w = new LfxWork();
    w->cap_rows = std::max(rows, nf);
    w->ftiles.resize(nf);
    std::vector<LfxField> tab(nf);
    unsigned long long t = 0;
    for (size_t f = 0; f < nf; f++) {
        const BlkField& F = b->tab[f];
        LfxField& L = tab[f];
        L.x = (const float*)F.x;
        L.n = F.n;
        const unsigned long long full = F.n / 128;
        L.ns = (full + kRate - 1) / kRate;
        L.ns2 = (full + kRate - 1 - kOff2) / kRate;   // blocks kOff2, kOff2 + 10, ... below full
        if (full <= (unsigned long long)kOff2) L.ns2 = 0;
        L.tile0 = t;
        w->ftiles[f] = (L.ns + kTileBlocks - 1) / kTileBlocks;
        t += w->ftiles[f];
    }
    w->tiles = t;
    auto a256 = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t cr = w->cap_rows;
    size_t off = 0;
    const size_t o_f = off; off += a256(sizeof(LfxField) * nf);
    const size_t o_acc = off; off += a256(8 * kAcc * nf);
    const size_t o_mm = off; off += a256(8 * nf);
    const size_t o_rg = off; off += a256(4 * nf);
    const size_t o_rows = off; off += a256(4 * cr);
    const size_t o_tgt = off; off += a256(4 * cr);
    const size_t o_q = off; off += a256(4 * cr);
    const size_t o_u = off; off += a256(4 * cr);
    const size_t o_racc = off; off += a256(8 * kRowAcc * cr);
    const size_t o_rt = off; off += a256(8 * (cr + 1));
    const size_t o_X = off; off += a256(4 * kF * cr);
    const size_t o_pred = off; off += a256(4 * cr);
    cudaError_t e = cudaMalloc(&w->dev, off);
    if (e != cudaSuccess) {
        delete w;
        return e;
    }
    uint8_t* base = (uint8_t*)w->dev;
    w->d_f = (LfxField*)(base + o_f);
    w->acc = (unsigned long long*)(base + o_acc);
    w->mm = (uint32_t*)(base + o_mm);
    w->range = (float*)(base + o_rg);
    w->rows = (int*)(base + o_rows);
    w->tgt = (float*)(base + o_tgt);
    w->mq = (int*)(base + o_q);
    w->mu = (int*)(base + o_u);
    w->racc = (unsigned long long*)(base + o_racc);
    w->rtile0 = (unsigned long long*)(base + o_rt);
    w->X = (float*)(base + o_X);
    w->pred = (float*)(base + o_pred);
    e = cudaMemcpy(w->d_f, tab.data(), sizeof(LfxField) * nf, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        lfx_free(w);
        return e;
    }
    b->lfx = w;
    return cudaSuccess;
}

int lfx_grid(unsigned long long warps) {
    const unsigned long long cap = (unsigned long long)sm_count() * 8 * 8;
    return (int)((std::min(warps, cap) + 7) / 8);
}

// Sampled range (and, with coarse, the per-field coarse sums) of every field.
cudaError_t lfx_sample(SZxG_Batch* b, cudaStream_t s, bool coarse = true) {
    LfxWork* w = b->lfx;
    const size_t nf = (size_t)b->nf;
    cudaError_t e = cudaMemsetAsync(w->acc, 0, 8 * kAcc * nf, s);
    if (e != cudaSuccess) return e;
    std::vector<uint32_t> init(2 * nf);   // (min, max) slots start at (all ones, 0)
    for (size_t f = 0; f < nf; f++) { init[2 * f] = 0xFFFFFFFFu; init[2 * f + 1] = 0u; }
    if ((e = cudaMemcpyAsync(w->mm, init.data(), 8 * nf, cudaMemcpyHostToDevice, s)) != cudaSuccess) return e;
    if (!w->tiles) return cudaSuccess;
    {
        TraceScope tr("lfx_range", s);
        k_lfx_range<128><<<lfx_grid(w->tiles), 256, 0, s>>>(w->d_f, (int)nf, w->tiles, w->mm);
    }
    if (coarse) {
        TraceScope tr("lfx_accumulate", s);
        k_lfx_accumulate<<<lfx_grid(w->tiles), 256, 0, s>>>(w->d_f, (int)nf, w->tiles, w->mm, w->acc);
    }
    return cudaGetLastError();
}

__global__ void k_lfx_range_out(const uint32_t* mm, int nf, float* range) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f < nf) range[f] = lfx_range_of(mm, f);
}

// Feature rows (after lfx_sample): the two per-row probe windows, then the rows.
// second = false skips the second sample's probes (feature 3 is then not
// meaningful): for callers that only need the crossing (feature 1).
cudaError_t lfx_rows(SZxG_Batch* b, int nrows, const int* h_rows, const float* h_tgt, float* d_X, cudaStream_t s,
                     bool second = true) {
    LfxWork* w = b->lfx;
    std::vector<unsigned long long> rt(nrows + 1);
    unsigned long long items = 0;
    for (int r = 0; r < nrows; r++) {
        rt[r] = items;
        items += w->ftiles[h_rows[r]];
    }
    rt[nrows] = items;
    cudaError_t e = cudaMemcpyAsync(w->rows, h_rows, sizeof(int) * nrows, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(w->tgt, h_tgt, sizeof(float) * nrows, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(w->rtile0, rt.data(), 8 * (nrows + 1), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(w->racc, 0, 8 * kRowAcc * (size_t)nrows, s);
    if (e != cudaSuccess) return e;
    const int rg = (nrows + 127) / 128;
    k_lfx_center<<<rg, 128, 0, s>>>(w->acc, nrows, w->rows, w->tgt, w->mq);
    if (items) {
        TraceScope tr("lfx_probe", s);
        k_lfx_probe<<<lfx_grid(items), 256, 0, s>>>(w->d_f, w->mm, nrows, w->rows, w->mq, 16, w->rtile0, items,
                                                    w->racc, 0, 0);
    }
    k_lfx_center2<<<rg, 128, 0, s>>>(w->d_f, w->racc, nrows, w->rows, w->tgt, w->mq, w->mu);
    if (items) {
        TraceScope tr("lfx_probe", s);
        k_lfx_probe<<<lfx_grid(items), 256, 0, s>>>(w->d_f, w->mm, nrows, w->rows, w->mu, 1, w->rtile0, items,
                                                    w->racc, kFine, 0);
        if (second)
            k_lfx_probe<<<lfx_grid(items), 256, 0, s>>>(w->d_f, w->mm, nrows, w->rows, w->mu, 1, w->rtile0, items,
                                                        w->racc, 2 * kFine, kOff2);
    }
    const int n = std::max(nrows, b->nf);
    k_lfx_rows<<<(n + 127) / 128, 128, 0, s>>>(w->d_f, w->acc, w->mm, nrows, w->rows, w->tgt, w->mq, w->mu, w->racc,
                                               d_X, w->range, b->nf);
    return cudaGetLastError();
}

}  // namespace

extern "C" {

int SZxG_batch_features(SZxG_Batch* b, int nRows, const int* fieldOfRow, const float* targetRatio, float* d_X,
                        float* h_range, void* stream) {
    if (!b || b->direction != 0 || b->dtype != 0 || b->bs != 128 || nRows < 1 || !fieldOfRow || !targetRatio ||
        !d_X) {
        set_last_error(SZXG_ERR_ARG);
        return SZXG_ERR_ARG;
    }
    for (int r = 0; r < nRows; r++)
        if (fieldOfRow[r] < 0 || fieldOfRow[r] >= b->nf || !(targetRatio[r] > 0.f)) {
            set_last_error(SZXG_ERR_ARG);
            return SZXG_ERR_ARG;
        }
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = lfx_prepare(b, (size_t)nRows);
    if (e == cudaSuccess) e = lfx_sample(b, s);
    if (e == cudaSuccess) e = lfx_rows(b, nRows, fieldOfRow, targetRatio, d_X, s);
    if (e == cudaSuccess && h_range)
        e = cudaMemcpyAsync(h_range, b->lfx->range, sizeof(float) * b->nf, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail_code(e);
    set_last_error(SZXG_OK);
    return SZXG_OK;
}

// Pick every field's bound so that its stream reaches targetRatio[f] within
// `tolerance` (relative), judged by real compress passes of the batch; the
// streams of the chosen bounds are left in the fields' buffers and their
// results in d_info (when not NULL).  Bounds are searched as y =
// log2(bound / sampled range) in [-28, 1].
//   mlp == NULL: plain bisection.
//   otherwise: the sampled crossing for the target divided by the network's
//   predicted miss; for a field that misses, one re-aimed crossing (the aim
//   multiplied by target / measured); then the bracket is closed by steps
//   that double away from the measured side (as the reference's search
//   brackets before it bisects) and bisected.
// Both stop when a measured bracket is narrower than 2^-10 in y (the ratio
// jumps over the target band there).  With a network: the bound's exponent
// sets every block's reqLength, so the ratio steps at each power of two P of
// the bound; a bracket whose ends hold exactly one P between them probes P
// and the float just below it, and ends when both lie on opposite sides of
// the band.  Plain bisection stays plain.  At most maxPasses passes per field,
// plus one for a field that stopped unconverged after a pass that was not its
// best.
int SZxG_batch_fixed_rate(SZxG_Batch* b, const SZxG_Mlp* mlp, const float* targetRatio, float tolerance,
                          int maxPasses, float* h_eb, float* h_ratio, int* h_passes, SZxG_StreamInfo* d_info,
                          void* stream) {
    if (!b || b->direction != 0 || b->dtype != 0 || b->bs != 128 || !targetRatio || !(tolerance > 0.f) ||
        maxPasses < 1 || maxPasses > 64) {
        set_last_error(SZXG_ERR_ARG);
        return SZXG_ERR_ARG;
    }
    const int nf = b->nf;
    cudaStream_t s = (cudaStream_t)stream;
    for (int f = 0; f < nf; f++)
        if (!(targetRatio[f] > 0.f)) { set_last_error(SZXG_ERR_ARG); return SZXG_ERR_ARG; }
    cudaError_t e = lfx_prepare(b, (size_t)nf);
    if (e == cudaSuccess) e = lfx_sample(b, s, mlp != nullptr);   // bisection needs the range only
    if (e == cudaSuccess && mlp) e = mlp_attr();
    if (e != cudaSuccess) return fail_code(e);
    std::vector<int> all(nf);
    for (int f = 0; f < nf; f++) all[f] = f;
    std::vector<float> range(nf), pred(nf, 0.f), tgt(targetRatio, targetRatio + nf);
    // ys (feature 1) of the fields in fl for targets t[f]; their rows stay in lfx->X, in fl's order
    std::vector<float> col(nf), tsub(nf);
    // (second: with the second sample's probes, for rows the network reads)
    auto crossing = [&](const std::vector<int>& fl, const std::vector<float>& t, std::vector<double>& ys,
                        bool second) {
        const int nr = (int)fl.size();
        if (nr == 0) return cudaSuccess;
        for (int k = 0; k < nr; k++) tsub[k] = t[fl[k]];
        cudaError_t e2 = lfx_rows(b, nr, fl.data(), tsub.data(), b->lfx->X, s, second);
        if (e2 == cudaSuccess)
            e2 = cudaMemcpy2DAsync(col.data(), sizeof(float), b->lfx->X + 1, sizeof(float) * kF, sizeof(float), nr,
                                   cudaMemcpyDeviceToHost, s);
        if (e2 == cudaSuccess) e2 = cudaStreamSynchronize(s);
        for (int k = 0; k < nr && e2 == cudaSuccess; k++) ys[fl[k]] = col[k];
        return e2;
    };
    // the network's predicted miss for the nf rows in lfx->X
    auto predict_miss = [&](std::vector<float>& mu) -> cudaError_t {
        {
            TraceScope tr("mlp_forward", s);
            k_mlp<false><<<(nf + kS - 1) / kS, kMlpThreads, mlp_smem(), s>>>(mlp->P, b->lfx->X, nullptr, nullptr, nf,
                                                                              1.f, b->lfx->pred, nullptr, nullptr);
        }
        cudaError_t e2 = cudaGetLastError();
        if (e2 == cudaSuccess)
            e2 = cudaMemcpyAsync(mu.data(), b->lfx->pred, sizeof(float) * nf, cudaMemcpyDeviceToHost, s);
        return e2 == cudaSuccess ? cudaStreamSynchronize(s) : e2;
    };
    k_lfx_range_out<<<(nf + 127) / 128, 128, 0, s>>>(b->lfx->mm, nf, b->lfx->range);
    e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(range.data(), b->lfx->range, sizeof(float) * nf, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    // first bounds: the sampled crossing for the target, re-taken for the
    // fields whose predicted miss is more than a quarter of the tolerance
    // band (a smaller correction cannot change the outcome much)
    std::vector<double> ys(nf, 0.0);
    std::vector<float> aim = tgt;   // the target each field's sampled crossing was last taken for
    // the first crossing's feature rows (field order): a crossing for another
    // aim that falls inside a row's 1/64-step window is read off its curve
    // (the same probe bounds, the same linear step) instead of probed again
    std::vector<float> Xh;
    auto window_crossing = [&](int f, float a, double& yout) {
        const float* r = Xh.data() + (size_t)f * kF;
        const double v = log2((double)a) - (double)r[0];   // the aim relative to the row's target
        const float* u = r + 13;
        for (int j = 0; j + 1 < kFine; j++)
            if ((double)u[j] < v && v <= (double)u[j + 1]) {
                yout = (double)r[4] + (j + (v - u[j]) / ((double)u[j + 1] - u[j])) / 64.0;
                return true;
            }
        return false;
    };
    if (mlp && e == cudaSuccess) e = crossing(all, tgt, ys, true);
    if (mlp && e == cudaSuccess) {
        Xh.resize((size_t)nf * kF);
        e = cudaMemcpyAsync(Xh.data(), b->lfx->X, sizeof(float) * kF * nf, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
    if (mlp && e == cudaSuccess) e = predict_miss(pred);
    if (mlp && e == cudaSuccess) {
        std::vector<int> moved;
        const double quarter_band = 0.25 * log2(1.0 + (double)tolerance);
        for (int f = 0; f < nf; f++) {
            const double mu = std::min(std::max((double)pred[f], -1.0), 1.0);
            if (fabs(mu) >= quarter_band) {
                aim[f] = (float)((double)tgt[f] * exp2(-mu));
                double yw;
                if (window_crossing(f, aim[f], yw)) ys[f] = yw;
                else moved.push_back(f);
            }
        }
        e = crossing(moved, aim, ys, false);
    }
    if (e != cudaSuccess) return fail_code(e);

    const double lo0 = -28.0, hi0 = 1.0;
    std::vector<double> lo(nf, lo0), hi(nf, hi0), y(nf), yprev(nf, 0.0), step(nf, 0.0), best_y(nf, 0),
        best_err(nf, 1e300), best_cr(nf, 0);
    // done: 1 converged, 2 stopped on a jump over the target band
    std::vector<int> passes(nf, 0), done(nf, 0), stage(nf, 0), last_is_best(nf, 0), lo_m(nf, 0), hi_m(nf, 0);
    std::vector<float> ebk(nf);
    for (int f = 0; f < nf; f++) ebk[f] = b->tab[f].eb;
    // bounds of the bracket's measured ends, of the best pass, and a bound
    // to code exactly in the next pass (0: from y)
    std::vector<float> lo_eb(nf, 0.f), hi_eb(nf, 0.f), best_eb(nf, 0.f), ebx(nf, 0.f);
    // one power of two P between the bracket's ends: the side of P to code
    // next, -1 when both sides are measured (the ratio jumps over the band
    // at P), 0 when the ends hold none or several
    auto jump_probe = [](float le, float he) -> float {
        int xl, xh;
        frexpf(le, &xl);
        frexpf(he, &xh);
        if (xh != xl + 1) return 0.f;
        const float P = ldexpf(1.f, xh - 1), Pm = nextafterf(P, 0.f);
        if (le == Pm && he == P) return -1.f;
        return he > P ? P : Pm;
    };
    std::vector<StreamResult> res(nf);
    auto eb_of = [&](int f, double yy) {
        const float r = range[f] > 0.f ? range[f] : 1.f;
        return (float)((double)r * exp2(yy));
    };
    auto clampy = [&](double v) { return std::min(std::max(v, lo0), hi0); };
    // next bound of a field that missed, from its bracket
    auto next_y = [&](int f) {
        if (!mlp || (lo_m[f] && hi_m[f])) return 0.5 * (lo[f] + hi[f]);
        step[f] = step[f] > 0 ? 2.0 * step[f] : std::max(2.0 * fabs(y[f] - yprev[f]), 0.25);
        return lo_m[f] ? std::min(lo[f] + step[f], hi[f]) : std::max(hi[f] - step[f], lo[f]);
    };
    for (int f = 0; f < nf; f++) y[f] = mlp ? clampy(ys[f]) : 0.5 * (lo0 + hi0);
    int err_code = SZXG_OK;
    for (int pass = 0; pass < maxPasses; pass++) {
        std::vector<int> act;
        std::vector<float> ebs;
        for (int f = 0; f < nf; f++)
            if (!done[f]) {
                act.push_back(f);
                ebs.push_back(ebx[f] > 0.f ? ebx[f] : eb_of(f, y[f]));
                ebx[f] = 0.f;
            }
        if (act.empty()) break;
        e = batch_select(b, (int)act.size(), act.data(), ebs.data(), s);
        if (e == cudaSuccess) {
            const int rc = SZxG_batch_run(b, nullptr, stream);
            if (rc) { err_code = rc; break; }
            e = cudaMemcpyAsync(res.data(), b->results, sizeof(StreamResult) * nf, cudaMemcpyDeviceToHost, s);
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return fail_code(e);
        bool need_refine = false;
        std::vector<float> t2 = tgt;
        for (size_t k = 0; k < act.size(); k++) {
            const int f = act[k];
            passes[f]++;
            ebk[f] = ebs[k];
            const StreamResult& r = res[f];
            if (r.status) { err_code = r.status; done[f] = 1; continue; }
            const double cr = (double)b->tab[f].n * 4.0 / (double)r.size;
            const double rel = fabs(cr / tgt[f] - 1.0);
            last_is_best[f] = 0;
            if (rel < best_err[f]) {
                best_err[f] = rel;
                best_y[f] = y[f];
                best_eb[f] = ebs[k];
                best_cr[f] = cr;
                last_is_best[f] = 1;
            }
            if (rel <= tolerance) { done[f] = 1; continue; }
            if (cr < tgt[f]) {
                if (!lo_m[f] || ebs[k] > lo_eb[f]) lo_eb[f] = ebs[k];
                lo[f] = std::max(lo[f], y[f]);
                lo_m[f] = 1;
            } else {
                if (!hi_m[f] || ebs[k] < hi_eb[f]) hi_eb[f] = ebs[k];
                hi[f] = std::min(hi[f], y[f]);
                hi_m[f] = 1;
            }
            // the ratio jumps over the target band inside a bracket this narrow: nothing to find
            if (lo_m[f] && hi_m[f] && hi[f] - lo[f] < kBracketStop) { done[f] = 2; continue; }
            const double ycur = y[f];
            if (mlp && stage[f] == 0) {
                // re-aim the sampled crossing by the miss this pass measured
                stage[f] = 1;
                t2[f] = (float)((double)aim[f] * std::min(std::max((double)tgt[f] / cr, 0.25), 4.0));
                need_refine = true;
            } else {
                const float pr = mlp && lo_m[f] && hi_m[f] ? jump_probe(lo_eb[f], hi_eb[f]) : 0.f;
                if (pr < 0.f) { done[f] = 2; continue; }
                if (pr > 0.f) {
                    ebx[f] = pr;
                    y[f] = log2((double)pr / (double)(range[f] > 0.f ? range[f] : 1.f));
                } else {
                    y[f] = next_y(f);
                }
            }
            yprev[f] = ycur;
        }
        if (err_code) break;
        if (need_refine) {
            std::vector<int> fl, fw;
            for (int f = 0; f < nf; f++)
                if (!done[f] && stage[f] == 1) {
                    if (!(t2[f] > 0.f) || !std::isfinite(t2[f])) t2[f] = aim[f];
                    double yw;
                    if (window_crossing(f, t2[f], yw)) {
                        ys[f] = yw;
                        fw.push_back(f);
                    } else {
                        fl.push_back(f);
                    }
                }
            if ((e = crossing(fl, t2, ys, false)) != cudaSuccess) return fail_code(e);
            fl.insert(fl.end(), fw.begin(), fw.end());
            for (int f : fl) {
                stage[f] = 2;
                y[f] = (ys[f] > lo[f] && ys[f] < hi[f]) ? ys[f] : next_y(f);
            }
        }
    }
    // a field that stopped unconverged gets its best bound back
    if (!err_code) {
        std::vector<int> act;
        std::vector<float> ebs;
        for (int f = 0; f < nf; f++)
            if (done[f] != 1 && !last_is_best[f] && best_err[f] < 1e300) {
                act.push_back(f);
                ebs.push_back(best_eb[f]);
                passes[f]++;
                ebk[f] = ebs.back();
            }
        if (!act.empty()) {
            e = batch_select(b, (int)act.size(), act.data(), ebs.data(), s);
            if (e == cudaSuccess) {
                const int rc = SZxG_batch_run(b, nullptr, stream);
                if (rc) err_code = rc;
            }
            if (e != cudaSuccess) return fail_code(e);
        }
    }
    // leave the plan coding every field, at the chosen bounds
    e = batch_select(b, nf, nullptr, ebk.data(), s);
    if (e == cudaSuccess && d_info)
        e = cudaMemcpyAsync(d_info, b->results, sizeof(StreamResult) * nf, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail_code(e);
    for (int f = 0; f < nf; f++) {
        if (h_eb) h_eb[f] = ebk[f];
        if (h_ratio) h_ratio[f] = (float)best_cr[f];
        if (h_passes) h_passes[f] = passes[f];
    }
    set_last_error(err_code);
    return err_code;
}

}  // extern "C"
