// cuSZx ABI: the two host entry points of the reference's GPU codec
// (szx/include/cuszx_entry.h:10-11) with its own stream format and block
// semantics (szx/src/cuszx_entry.cu:20-209, szx/src/cuszx_float.cu,
// szx/src/cuszxd_float.cu), so that programs written against cuSZx get the
// same bytes and values:
//
//   [1,1,1,0] | blockSize u8 | nbConstant u64 BE | state bits of the
//   nbEle / blockSize full blocks (MSB first) | the nbEle % blockSize
//   remaining floats, raw | constant blocks' medians (native float) | per
//   non-constant block its mid-byte count (i16, native) | per non-constant
//   block: median (native float), reqLength u8, 2-bit lead codes
//   (blockSize / 4 bytes), mid bytes.
//
// Block rules that differ from the CPU codec (kept, because they define the
// stream): reqLength = 10 + exponent(radius) - exponent(bound) is not
// clamped; a value's lead is counted up to its required byte count, so a
// value identical to its predecessor at reqLength 25..32 gets a lead of 4 that
// its 2-bit code cannot hold (the OR of the shifted codes is truncated to a
// byte: the code reads 0 and the previous value's code gains a bit); with
// reqLength above 32 the required bytes are counted but none is stored or
// read.  Decoding takes each byte lane a value does not store from the latest
// earlier value that stored that lane (or value 0).
//
// GB300 layout: a warp per block (blockSize / 32 values per lane, value
// j * 32 + lane, the reference's thread order); compression is a sizes pass,
// one exclusive scan of (payload bytes, non-constant count) packed in 64 bits,
// and an emit pass that recomputes each block and writes it in place; the
// whole stream is built on the device and copied out once.  Differences from
// the reference's host code: the output buffer is sized exactly (the
// reference's is nbEle * 4 bytes and can overflow), a block size that is not
// a multiple of 32 in 32..224 is refused, and a stream with a block longer
// than blockSize * 4 bytes makes decompression fail (newData = NULL) where the
// reference prints a warning and exits the process.  No timing or debug lines
// are printed.
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "../../include/szx_gb300.h"
#include "common.cuh"
#include "kernels.h"

using namespace szxg;

namespace {

constexpr int kCzWarps = 8;
constexpr int kCzThreads = 32 * kCzWarps;
constexpr int kCzMaxBs = 224;
constexpr int kCzMaxJ = kCzMaxBs / 32;
constexpr int kCountBits = 26;   // packed scan: (payload bytes << 26) | non-constant count

__device__ __forceinline__ int cz_lead(uint32_t x, int R) {
    if (R == 2) return (x >> 16) == 0 ? 2 : ((x >> 24) == 0 ? 1 : 0);
    if (R == 3) return (x >> 8) == 0 ? 3 : ((x >> 16) == 0 ? 2 : ((x >> 24) == 0 ? 1 : 0));
    if (R == 1) return (x >> 24) == 0 ? 1 : 0;
    if (R == 4) return x == 0 ? 4 : ((x >> 8) == 0 ? 3 : ((x >> 16) == 0 ? 2 : ((x >> 24) == 0 ? 1 : 0)));
    return 0;
}

__device__ __forceinline__ void cz_split(int req, int* R, int* rsb) {
    if (req % 8 != 0) { *R = req / 8 + 1; *rsb = 8 - req % 8; }
    else { *R = req / 8; *rsb = 0; }
}

struct CzGeom {
    unsigned long long nb, nconst_off, off_off, pay_off;   // regions (filled after the scan)
};

// One block by one warp.  EMIT = false: per-block packed scan value and
// state / median; EMIT = true: the block's bytes at their place.
template <bool EMIT>
__global__ void __launch_bounds__(kCzThreads) k_cz_blocks(const float* __restrict__ x, unsigned long long nb, int bs,
                                                          float eb, unsigned long long* packed, uint8_t* state,
                                                          uint32_t* med_out, const unsigned long long* excl,
                                                          uint8_t* out, const unsigned long long* regions) {
    const int lane = threadIdx.x & 31;
    const unsigned long long w0 = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) >> 5;
    const unsigned long long nw = (gridDim.x * (unsigned long long)blockDim.x) >> 5;
    const int J = bs / 32, ncb = bs / 4, msize = 5 + ncb;
    // The reference combines its warps' minima with xor offsets J/2, J/4, ..
    // 1 (szx/src/cuszx_float.cu:248-256): the lane that keeps the result sees
    // the first 2^floor(log2 J) warps only (all of them when J is a power of
    // two), so only their values enter a block's range.
    const int Jc = 1 << (31 - __clz(J));
    for (unsigned long long b = w0; b < nb; b += nw) {
        const float* xb = x + b * (unsigned long long)bs;
        float v[kCzMaxJ];
        float mn = __int_as_float(0x7F800000), mx = -mn;
#pragma unroll
        for (int j = 0; j < kCzMaxJ; j++)
            if (j < J) {
                v[j] = xb[j * 32 + lane];
                if (j < Jc) {
                    mn = fminf(mn, v[j]);
                    mx = fmaxf(mx, v[j]);
                }
            }
#pragma unroll
        for (int d = 16; d; d >>= 1) {
            mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, d));
            mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, d));
        }
        const float radius = __fmul_rn(__fsub_rn(mx, mn), 0.5f);
        const float median = __fadd_rn(mn, radius);
        const bool coded = !(radius <= eb);
        if (!EMIT) {
            if (lane == 0) {
                state[b] = coded ? 1 : 0;
                med_out[b] = __float_as_uint(median);
            }
            if (!coded) {
                if (lane == 0) packed[b] = 0;
                continue;
            }
        } else if (!coded) {
            // constant block: its median in the median list
            const unsigned long long crank = b - (excl[b] & ((1ull << kCountBits) - 1));
            if (lane < 4) out[regions[0] + 4 * crank + lane] = (uint8_t)(__float_as_uint(median) >> (8 * lane));
            continue;
        }
        const int req = 10 + ((int)((__float_as_uint(radius) & 0x7F800000u) >> 23) - 127) -
                        ((int)((__float_as_uint(eb) & 0x7F800000u) >> 23) - 127);
        int R, rsb;
        cz_split(req, &R, &rsb);
        const uint32_t mask = rsb ? ((1u << (32 - rsb)) - 1u) : 0xFFFFFFFFu;
        uint32_t cur[kCzMaxJ];
        int lead[kCzMaxJ], incl[kCzMaxJ];
        int carry = 0;
        uint32_t last = 0;
#pragma unroll
        for (int j = 0; j < kCzMaxJ; j++)
            if (j < J) {
                cur[j] = (__float_as_uint(__fsub_rn(v[j], median)) >> rsb) & mask;
                uint32_t prev = __shfl_up_sync(0xffffffffu, cur[j], 1);
                if (lane == 0) prev = last;
                last = __shfl_sync(0xffffffffu, cur[j], 31);
                lead[j] = cz_lead(cur[j] ^ prev, R);
                int s = R - lead[j];
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const int o = __shfl_up_sync(0xffffffffu, s, d);
                    if (lane >= d) s += o;
                }
                incl[j] = carry + s;
                carry = __shfl_sync(0xffffffffu, incl[j], 31);
            }
        const int total = carry;   // mid bytes counted for the block
        if (!EMIT) {
            if (lane == 0) packed[b] = ((unsigned long long)(msize + total) << kCountBits) | 1ull;
            continue;
        }
        const unsigned long long e = excl[b];
        const unsigned long long nrank = e & ((1ull << kCountBits) - 1);
        uint8_t* ob = out + regions[2] + (e >> kCountBits);
        // the block's mid-byte count (i16, native) in the count list
        if (lane < 2) out[regions[1] + 2 * nrank + lane] = (uint8_t)((uint32_t)(short)total >> (8 * lane));
        if (lane < 4) ob[lane] = (uint8_t)(__float_as_uint(median) >> (8 * lane));
        if (lane == 0) ob[4] = (uint8_t)req;
        uint8_t* mid = ob + msize;
        if (R > 4)
            for (int k = lane; k < total; k += 32) mid[k] = 0;   // counted, never stored
#pragma unroll
        for (int j = 0; j < kCzMaxJ; j++)
            if (j < J) {
                // lead codes: OR of lead << 2(3 - v%4) over four values, truncated to a byte
                unsigned c = (unsigned)lead[j] << (2 * (3 - (lane & 3)));
                c |= __shfl_down_sync(0xffffffffu, c, 1);
                c |= __shfl_down_sync(0xffffffffu, c, 2);
                if ((lane & 3) == 0) ob[5 + ((j * 32 + lane) >> 2)] = (uint8_t)c;
                if (R <= 4) {
                    const int sz = R - lead[j], lo = 4 - R, at = incl[j] - sz;
                    for (int k = 0; k < sz; k++) mid[at + k] = (uint8_t)(cur[j] >> (8 * (lo + k)));
                }
            }
    }
}

// State bits, MSB first: one thread per byte.
__global__ void k_cz_state_bits(const uint8_t* state, unsigned long long nb, uint8_t* out) {
    const unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= (nb + 7) / 8) return;
    uint8_t v = 0;
    for (int k = 0; k < 8; k++) {
        const unsigned long long b = 8 * i + k;
        if (b < nb && state[b]) v |= (uint8_t)(0x80u >> k);
    }
    out[i] = v;
}

// Exclusive scan of n u64 values: tiles of 4096 scanned locally, the tile
// sums by one CTA, then the tile prefixes added.
constexpr int kScanItems = 16, kScanThreads = 256, kScanTile = kScanItems * kScanThreads;

__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const unsigned long long* in, unsigned long long* out,
                                                              unsigned long long* sums, unsigned long long n) {
    __shared__ unsigned long long ws[kScanThreads / 32];
    const unsigned long long base = (unsigned long long)blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    unsigned long long v[kScanItems], t = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        v[i] = base + i < n ? in[base + i] : 0ull;
        t += v[i];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long inc = t;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned long long o = __shfl_up_sync(0xffffffffu, inc, d);
        if (lane >= d) inc += o;
    }
    if (lane == 31) ws[warp] = inc;
    __syncthreads();
    unsigned long long wpre = 0, tot = 0;
    for (int w = 0; w < kScanThreads / 32; w++) {
        if (w < warp) wpre += ws[w];
        tot += ws[w];
    }
    unsigned long long run = wpre + inc - t;
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        if (base + i < n) out[base + i] = run;
        run += v[i];
    }
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

// One CTA: exclusive prefixes of the tile sums (in place); sums[ntiles] = total.
__global__ void k_scan_top(unsigned long long* sums, unsigned long long ntiles) {
    __shared__ unsigned long long ws[32];
    __shared__ unsigned long long s_carry;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (unsigned long long base = 0; base < ntiles; base += blockDim.x) {
        const unsigned long long i = base + threadIdx.x;
        const unsigned long long v = i < ntiles ? sums[i] : 0ull;
        unsigned long long inc = v;
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned long long o = __shfl_up_sync(0xffffffffu, inc, d);
            if (lane >= d) inc += o;
        }
        if (lane == 31) ws[warp] = inc;
        __syncthreads();
        unsigned long long wpre = 0, tot = 0;
        for (int w = 0; w < (int)(blockDim.x / 32); w++) {
            if (w < warp) wpre += ws[w];
            tot += ws[w];
        }
        const unsigned long long c = s_carry;
        if (i < ntiles) sums[i] = c + wpre + inc - v;
        __syncthreads();
        if (threadIdx.x == 0) s_carry = c + tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) sums[ntiles] = s_carry;
}

__global__ void k_scan_add(unsigned long long* out, const unsigned long long* sums, unsigned long long n) {
    const unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i < n) out[i] += sums[i / kScanTile];
}

cudaError_t scan_excl(const unsigned long long* in, unsigned long long* out, unsigned long long* sums,
                      unsigned long long n, cudaStream_t s) {
    const unsigned long long tiles = (n + kScanTile - 1) / kScanTile;
    if (n == 0) return cudaMemsetAsync(sums, 0, 8, s);
    k_scan_tiles<<<(unsigned)tiles, kScanThreads, 0, s>>>(in, out, sums, n);
    k_scan_top<<<1, 1024, 0, s>>>(sums, tiles);
    k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(out, sums, n);
    return cudaGetLastError();
}

int cz_grid(unsigned long long warps) {
    const unsigned long long cap = (unsigned long long)sm_count() * 16 * kCzWarps;
    const unsigned long long w = warps < cap ? warps : cap;
    return (int)((w + kCzWarps - 1) / kCzWarps);
}

// ---------------------------------------------------------------- decode

// One block by one warp.  Constant blocks fill their median; a non-constant
// block's bytes (the first msize + count bytes of a blockSize * 4 buffer, the
// rest zero) are decoded as the reference's decompress_float does.
__global__ void __launch_bounds__(kCzThreads) k_cz_decode(const uint8_t* s, unsigned long long nb, int bs,
                                                          const uint8_t* sbits, const unsigned long long* nrank_excl,
                                                          const unsigned long long* pay_excl, const uint8_t* meds,
                                                          const uint8_t* counts, const uint8_t* pay,
                                                          unsigned long long pay_len, float* y, int* err) {
    __shared__ __align__(16) uint8_t s_blk[kCzWarps][kCzMaxBs * 4];
    __shared__ uint32_t s_tmp[kCzWarps][kCzMaxBs];
    const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
    const unsigned long long w0 = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) >> 5;
    const unsigned long long nw = (gridDim.x * (unsigned long long)blockDim.x) >> 5;
    const int J = bs / 32, msize = 5 + bs / 4;
    uint8_t* blk = s_blk[wi];
    uint32_t* tmp = s_tmp[wi];
    for (unsigned long long b = w0; b < nb; b += nw) {
        float* yb = y + b * (unsigned long long)bs;
        const bool coded = (sbits[b >> 3] >> (7 - (b & 7))) & 1;
        const unsigned long long nr = nrank_excl[b];
        if (!coded) {
            const uint8_t* m = meds + 4 * (b - nr);
            const float med = __uint_as_float((uint32_t)m[0] | ((uint32_t)m[1] << 8) | ((uint32_t)m[2] << 16) |
                                              ((uint32_t)m[3] << 24));
            for (int j = 0; j < J; j++) yb[j * 32 + lane] = med;
            continue;
        }
        const short cnt = (short)((uint16_t)counts[2 * nr] | ((uint16_t)counts[2 * nr + 1] << 8));
        const int leng = (int)cnt + msize;
        const unsigned long long at = pay_excl[b];
        if (leng < 0 || leng > bs * 4 || at + (unsigned long long)leng > pay_len) {
            if (lane == 0) atomicExch(err, 1);
            continue;
        }
        for (int k = lane; k < bs * 4; k += 32) blk[k] = k < leng ? pay[at + k] : 0;
        __syncwarp();
        const float med = __uint_as_float((uint32_t)blk[0] | ((uint32_t)blk[1] << 8) | ((uint32_t)blk[2] << 16) |
                                          ((uint32_t)blk[3] << 24));
        const int req = blk[4];
        int R, rsb;
        cz_split(req, &R, &rsb);
        int carry = 0, pcarry = 0;
        uint32_t t[kCzMaxJ];
        int lead[kCzMaxJ], pos[kCzMaxJ];
#pragma unroll
        for (int j = 0; j < kCzMaxJ; j++)
            if (j < J) {
                const int v = j * 32 + lane;
                lead[j] = (blk[5 + (v >> 2)] >> (6 - ((v & 3) << 1))) & 3;
                const int sz = R - lead[j];
                int sc = sz;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const int o = __shfl_up_sync(0xffffffffu, sc, d);
                    if (lane >= d) sc += o;
                }
                const int incl = carry + sc;
                carry = __shfl_sync(0xffffffffu, incl, 31);
                const int base = msize + incl;
                auto mb = [&](int k) -> uint32_t {
                    const int i = base - k;
                    return (i >= 0 && i < bs * 4) ? blk[i] : 0u;
                };
                uint32_t w = 0;
                int p = 0;
                if (R == 2) {
                    if (sz == 1) { w = mb(1) << 16; p = v << 8; }
                    else if (sz == 2) { w = (mb(1) << 24) | (mb(2) << 16); p = v | (v << 8); }
                } else if (R == 3) {
                    if (sz == 1) { w = mb(1) << 8; p = v << 16; }
                    else if (sz == 2) { w = (mb(1) << 16) | (mb(2) << 8); p = (v << 8) | (v << 16); }
                    else if (sz == 3) { w = (mb(1) << 24) | (mb(2) << 16) | (mb(3) << 8); p = v | (v << 8) | (v << 16); }
                } else if (R == 1) {
                    if (sz == 1) w = mb(1) << 24;
                    p = v;
                } else if (R == 4) {
                    if (sz == 1) { w = mb(1); p = v << 24; }
                    else if (sz == 2) { w = (mb(1) << 8) | mb(2); p = (v << 16) | (v << 24); }
                    else if (sz == 3) { w = (mb(1) << 16) | (mb(2) << 8) | mb(3); p = (v << 8) | (v << 16) | (v << 24); }
                    else if (sz == 4) {
                        w = (mb(1) << 24) | (mb(2) << 16) | (mb(3) << 8) | mb(4);
                        p = v | (v << 8) | (v << 16) | (v << 24);
                    }
                }
                t[j] = w;
                // latest value <= v that stored each byte lane: prefix max per lane
                auto comb = [&](int pre, int c) -> int {
                    if (R == 1) return pre > c ? pre : c;
                    if (R < 2 || R > 4) return c;
                    for (int k = 0; k < R; k++) {
                        const int sh = 8 * k;
                        const int pl = (pre >> sh) & 0xFF, cl = (c >> sh) & 0xFF;
                        if (pl > cl) c = (c & ~(0xFF << sh)) | (pl << sh);
                    }
                    return c;
                };
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const int o = __shfl_up_sync(0xffffffffu, p, d);
                    if (lane >= d) p = comb(o, p);
                }
                p = comb(pcarry, p);
                pcarry = __shfl_sync(0xffffffffu, p, 31);
                pos[j] = p;
            }
#pragma unroll
        for (int j = 0; j < kCzMaxJ; j++)
            if (j < J) tmp[j * 32 + lane] = t[j];
        __syncwarp();
#pragma unroll
        for (int j = 0; j < kCzMaxJ; j++)
            if (j < J) {
                uint32_t w = t[j];
                const int p = pos[j];
                if (lead[j] >= 1) w = (w & 0x00FFFFFFu) | (tmp[p & 0xFF] & 0xFF000000u);
                if (lead[j] >= 2) w = (w & 0xFF00FFFFu) | (tmp[(p >> 8) & 0xFF] & 0x00FF0000u);
                if (lead[j] >= 3) w = (w & 0xFFFF00FFu) | (tmp[(p >> 16) & 0xFF] & 0x0000FF00u);
                yb[j * 32 + lane] = __fadd_rn(__int_as_float((int)w << rsb), med);
            }
        __syncwarp();
    }
}

__global__ void k_cz_nc_flags(const uint8_t* sbits, unsigned long long nb, unsigned long long* flag) {
    const unsigned long long b = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (b < nb) flag[b] = (sbits[b >> 3] >> (7 - (b & 7))) & 1;
}

__global__ void k_cz_pay_sizes(const uint8_t* sbits, unsigned long long nb, int msize, const unsigned long long* nr,
                               const uint8_t* counts, unsigned long long* sz) {
    const unsigned long long b = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const bool coded = (sbits[b >> 3] >> (7 - (b & 7))) & 1;
    long long v = 0;
    if (coded) {
        const unsigned long long k = nr[b];
        const short c = (short)((uint16_t)counts[2 * k] | ((uint16_t)counts[2 * k + 1] << 8));
        v = (long long)c + msize;
        if (v < 0) v = 0;   // rejected by the decoder
    }
    sz[b] = (unsigned long long)v;
}

bool cz_bs_ok(int bs) { return bs >= 32 && bs <= kCzMaxBs && bs % 32 == 0; }

}  // namespace

extern "C" {

unsigned char* cuSZx_fast_compress_args_unpredictable_blocked_float(float* oriData, size_t* outSize,
                                                                    float absErrBound, size_t nbEle, int blockSize) {
    if (!oriData || !outSize || !cz_bs_ok(blockSize) || nbEle >= ((size_t)1 << 31)) {
        set_last_error(SZXG_ERR_ARG);
        return nullptr;
    }
    const unsigned long long nb = nbEle / (size_t)blockSize, tail = nbEle % (size_t)blockSize;
    const unsigned long long sb = (nb + 7) / 8;
    cudaStream_t s = nullptr;
    float* d_x = nullptr;
    unsigned long long *d_packed = nullptr, *d_excl = nullptr, *d_sums = nullptr, *d_reg = nullptr;
    uint8_t *d_state = nullptr, *d_out = nullptr;
    uint32_t* d_med = nullptr;
    unsigned char* host = nullptr;
    const unsigned long long tiles = (nb + kScanTile - 1) / kScanTile;
    cudaError_t e = cudaMalloc(&d_x, nbEle * 4 + 16);
    if (e == cudaSuccess) e = cudaMalloc(&d_packed, 8 * (nb + 1));
    if (e == cudaSuccess) e = cudaMalloc(&d_excl, 8 * (nb + 1));
    if (e == cudaSuccess) e = cudaMalloc(&d_sums, 8 * (tiles + 2));
    if (e == cudaSuccess) e = cudaMalloc(&d_reg, 8 * 4);
    if (e == cudaSuccess) e = cudaMalloc(&d_state, nb + 1);
    if (e == cudaSuccess) e = cudaMalloc(&d_med, 4 * (nb + 1));
    if (e == cudaSuccess && nbEle) e = cudaMemcpyAsync(d_x, oriData, nbEle * 4, cudaMemcpyHostToDevice, s);
    const int grid = cz_grid(nb ? nb : 1);
    unsigned long long total_packed = 0;
    if (e == cudaSuccess && nb) {
        k_cz_blocks<false><<<grid, kCzThreads, 0, s>>>(d_x, nb, blockSize, absErrBound, d_packed, d_state, d_med,
                                                      nullptr, nullptr, nullptr);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = scan_excl(d_packed, d_excl, d_sums, nb, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(&total_packed, d_sums + tiles, 8, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
    const unsigned long long nnc = total_packed & ((1ull << kCountBits) - 1), pay = total_packed >> kCountBits;
    const unsigned long long nconst = nb - nnc;
    const unsigned long long c0 = 13 + sb + 4 * tail, o0 = c0 + 4 * nconst, p0 = o0 + 2 * nnc;
    const unsigned long long total = p0 + pay;
    if (e == cudaSuccess) e = cudaMalloc(&d_out, total + 16);
    if (e == cudaSuccess && nb) {
        const unsigned long long reg[3] = {c0, o0, p0};
        e = cudaMemcpyAsync(d_reg, reg, sizeof reg, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) {
            k_cz_state_bits<<<(unsigned)((sb + 255) / 256), 256, 0, s>>>(d_state, nb, d_out + 13);
            k_cz_blocks<true><<<grid, kCzThreads, 0, s>>>(d_x, nb, blockSize, absErrBound, nullptr, nullptr, nullptr,
                                                         d_excl, d_out, d_reg);
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess && tail)
        e = cudaMemcpyAsync(d_out + 13 + sb, d_x + nb * blockSize, 4 * tail, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) {
        host = (unsigned char*)malloc(total ? total : 1);
        if (!host) e = cudaErrorMemoryAllocation;
    }
    if (e == cudaSuccess && total > 13) e = cudaMemcpyAsync(host + 13, d_out + 13, total - 13, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(d_x); cudaFree(d_packed); cudaFree(d_excl); cudaFree(d_sums); cudaFree(d_reg);
    cudaFree(d_state); cudaFree(d_med); cudaFree(d_out);
    if (e != cudaSuccess) {
        cudaGetLastError();
        free(host);
        set_last_error(SZXG_ERR_CUDA);
        return nullptr;
    }
    host[0] = 1; host[1] = 1; host[2] = 1; host[3] = 0; host[4] = (unsigned char)blockSize;
    for (int k = 0; k < 8; k++) host[5 + k] = (unsigned char)(nconst >> (56 - 8 * k));
    *outSize = (size_t)total;
    set_last_error(SZXG_OK);
    return host;
}

void cuSZx_fast_decompress_args_unpredictable_blocked_float(float** newData, size_t nbEle, unsigned char* cmpBytes) {
    if (!newData) return;
    *newData = nullptr;
    if (!cmpBytes) { set_last_error(SZXG_ERR_ARG); return; }
    const int bs = cmpBytes[4];
    if (!cz_bs_ok(bs)) { set_last_error(SZXG_ERR_STREAM); return; }
    unsigned long long nconst = 0;
    for (int k = 0; k < 8; k++) nconst = (nconst << 8) | cmpBytes[5 + k];
    const unsigned long long nb = nbEle / (size_t)bs, tail = nbEle % (size_t)bs, sb = (nb + 7) / 8;
    if (nconst > nb) { set_last_error(SZXG_ERR_STREAM); return; }
    const unsigned long long nnc = nb - nconst;
    const unsigned long long c0 = 13 + sb + 4 * tail, o0 = c0 + 4 * nconst, p0 = o0 + 2 * nnc;
    const int msize = 5 + bs / 4;
    // the stream's length follows from its counts (read on the host, like the reference's copy loop)
    unsigned long long pay = 0;
    for (unsigned long long k = 0; k < nnc; k++) {
        const short c = (short)((uint16_t)cmpBytes[o0 + 2 * k] | ((uint16_t)cmpBytes[o0 + 2 * k + 1] << 8));
        const long long l = (long long)c + msize;
        if (l < 0 || l > 4 * bs) { set_last_error(SZXG_ERR_STREAM); return; }
        pay += (unsigned long long)l;
    }
    const unsigned long long len = p0 + pay;
    float* host = (float*)malloc(nbEle ? nbEle * 4 : 4);
    if (!host) { set_last_error(SZXG_ERR_CUDA); return; }
    cudaStream_t s = nullptr;
    uint8_t* d_s = nullptr;
    float* d_y = nullptr;
    unsigned long long *d_f = nullptr, *d_nr = nullptr, *d_sz = nullptr, *d_pe = nullptr, *d_sums = nullptr;
    int* d_err = nullptr;
    const unsigned long long tiles = (nb + kScanTile - 1) / kScanTile;
    cudaError_t e = cudaMalloc(&d_s, len + 16);
    if (e == cudaSuccess) e = cudaMalloc(&d_y, nbEle * 4 + 16);
    if (e == cudaSuccess) e = cudaMalloc(&d_f, 8 * (nb + 1));
    if (e == cudaSuccess) e = cudaMalloc(&d_nr, 8 * (nb + 1));
    if (e == cudaSuccess) e = cudaMalloc(&d_sz, 8 * (nb + 1));
    if (e == cudaSuccess) e = cudaMalloc(&d_pe, 8 * (nb + 1));
    if (e == cudaSuccess) e = cudaMalloc(&d_sums, 8 * (tiles + 2));
    if (e == cudaSuccess) e = cudaMalloc(&d_err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemsetAsync(d_err, 0, sizeof(int), s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_s, cmpBytes, len, cudaMemcpyHostToDevice, s);
    int herr = 0;
    if (e == cudaSuccess && nb) {
        const unsigned g = (unsigned)((nb + 255) / 256);
        k_cz_nc_flags<<<g, 256, 0, s>>>(d_s + 13, nb, d_f);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = scan_excl(d_f, d_nr, d_sums, nb, s);
        if (e == cudaSuccess) {
            k_cz_pay_sizes<<<g, 256, 0, s>>>(d_s + 13, nb, msize, d_nr, d_s + o0, d_sz);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = scan_excl(d_sz, d_pe, d_sums, nb, s);
        if (e == cudaSuccess) {
            k_cz_decode<<<cz_grid(nb), kCzThreads, 0, s>>>(d_s, nb, bs, d_s + 13, d_nr, d_pe, d_s + c0, d_s + o0,
                                                           d_s + p0, pay, d_y, d_err);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, s);
    }
    if (e == cudaSuccess && nb) e = cudaMemcpyAsync(host, d_y, 4 * nb * bs, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (tail) memcpy(host + nb * bs, cmpBytes + 13 + sb, 4 * tail);
    cudaFree(d_s); cudaFree(d_y); cudaFree(d_f); cudaFree(d_nr); cudaFree(d_sz); cudaFree(d_pe); cudaFree(d_sums);
    cudaFree(d_err);
    if (e != cudaSuccess || herr) {
        cudaGetLastError();
        free(host);
        set_last_error(e != cudaSuccess ? SZXG_ERR_CUDA : SZXG_ERR_STREAM);
        return;
    }
    *newData = host;
    set_last_error(SZXG_OK);
}

}  // extern "C"
