// Blocked layouts of the SZx stream (fastMode 2, 3, 4): encode and decode.
//
// Stream (mode 3, szx/src/szx_float.cc:1407-1489):
//   [1,1,1,1] | blockSize u64 BE | nbConstant u64 BE | O u16[nnc] | state bits
//   | constant medians f32 BE [nc] | payloads of the non-constant blocks
// mode 2 (szx/src/szx_float.cc:1059-1139): [1,1,1,0] | blockSize u8 | nbConstant
//   u64 BE | state bits | medians | payloads  (no size index)
// mode 4 (szx/src/szx_float.cc:1218-1405): mode-3 layout, medians native endian.
// Block payload (szx/src/szx_float.cc:49-252): reqLength u8 | median f32 BE |
//   2-bit lead codes MSB-first | mid bytes.
//
// GB300 design
// * Encode is ONE pass over the input: a CTA takes a tile of blocks from an
//   atomic tile counter, a warp per block computes min/max (warp shuffles),
//   state, reqLength and the shifted words in registers, the tile's payload
//   bytes and non-constant count are placed by a decoupled look-back, and the
//   payload bytes are emitted from registers into a per-warp shared staging
//   buffer and stored with aligned 16-byte writes.
// * The payload region is written at a fixed position (as if no block were
//   non-constant); the stream is then shifted to start 2*nnc (mode 3/4) or
//   4*nnc (mode 2) bytes into the buffer so that header, index, state bits and
//   medians (assembled by a small second kernel from per-block scratch) end
//   exactly where the payload region begins.  Nothing is ever moved.
// * Decode scans the size index and the state bits (single-pass look-back),
//   then a warp per block reconstructs its values: mid-byte offsets come from
//   a warp prefix sum, and the bytes carried over from previous values (the
//   top three byte lanes, the only ones a lead code can inherit) from one
//   packed "last writer" warp scan.
#include "common.cuh"
#include "kernels.h"

namespace szxg {

constexpr int kEncWarps = 8;
constexpr int kEncThreads = kEncWarps * 32;
constexpr int kDecThreads = 256;
constexpr int kIdxThreads = 256;
constexpr int kIdxItems = 8;   // items per thread in the index scans

// ------------------------------------------------------------------ lane loads / stores

template <int B> struct RawVec;
template <> struct RawVec<4> { static __device__ __forceinline__ void ld(const void* p, uint32_t* d) { d[0] = *(const uint32_t*)p; } };
template <> struct RawVec<8> { static __device__ __forceinline__ void ld(const void* p, uint32_t* d) { uint2 v = *(const uint2*)p; d[0] = v.x; d[1] = v.y; } };
template <> struct RawVec<16> { static __device__ __forceinline__ void ld(const void* p, uint32_t* d) { uint4 v = *(const uint4*)p; d[0] = v.x; d[1] = v.y; d[2] = v.z; d[3] = v.w; } };

// Load E consecutive elements of one lane; vector loads when the caller knows
// the lane's first element is aligned to min(E*sizeof(T), 16) bytes.
template <typename T, int E>
__device__ __forceinline__ void load_lane(const T* p, int nv, bool vec_ok, T (&v)[E]) {
    constexpr int B = E * (int)sizeof(T);
    if (vec_ok && nv == E) {
        uint32_t w[B / 4];
        if constexpr (B >= 16) {
#pragma unroll
            for (int i = 0; i < B / 16; i++) RawVec<16>::ld((const uint8_t*)p + 16 * i, w + 4 * i);
        } else {
            RawVec<B>::ld(p, w);
        }
#pragma unroll
        for (int e = 0; e < E; e++) {
            if constexpr (sizeof(T) == 4) v[e] = __uint_as_float(w[e]);
            else v[e] = __longlong_as_double((long long)(((unsigned long long)w[2 * e + 1] << 32) | w[2 * e]));
        }
    } else {
#pragma unroll
        for (int e = 0; e < E; e++) v[e] = e < nv ? p[e] : (T)0;
    }
}

template <typename T, int E>
__device__ __forceinline__ void store_lane(T* p, int nv, bool vec_ok, const T (&v)[E]) {
    constexpr int B = E * (int)sizeof(T);
    if (vec_ok && nv == E) {
        uint32_t w[B / 4];
#pragma unroll
        for (int e = 0; e < E; e++) {
            if constexpr (sizeof(T) == 4) w[e] = __float_as_uint(v[e]);
            else {
                unsigned long long u = (unsigned long long)__double_as_longlong(v[e]);
                w[2 * e] = (uint32_t)u;
                w[2 * e + 1] = (uint32_t)(u >> 32);
            }
        }
        if constexpr (B >= 16) {
#pragma unroll
            for (int i = 0; i < B / 16; i++)
                *(uint4*)((uint8_t*)p + 16 * i) = make_uint4(w[4 * i], w[4 * i + 1], w[4 * i + 2], w[4 * i + 3]);
        } else if constexpr (B == 8) {
            *(uint2*)p = make_uint2(w[0], w[1]);
        } else {
            *(uint32_t*)p = w[0];
        }
    } else {
#pragma unroll
        for (int e = 0; e < E; e++)
            if (e < nv) p[e] = v[e];
    }
}

template <typename T, int E>
__device__ __forceinline__ bool lane_vec_ok(const void* block_base) {
    constexpr int B = E * (int)sizeof(T);
    constexpr int A = B < 16 ? B : 16;
    return ((uintptr_t)block_base % A) == 0;
}

// ------------------------------------------------------------------ block statistics

// Warp-wide min/max of one block with the reference's sequential semantics
// (szx/src/szx_float.cc:322-345): the first element reaching an extreme wins,
// NaNs are skipped unless the block's first element is NaN.
template <typename T, int E>
__device__ __forceinline__ void block_minmax(const T (&v)[E], int nv, T& mn, T& mx);

template <typename T, int E>
__device__ __forceinline__ void block_minmax(const T (&v)[E], int nv, T& mn, T& mx) {
    if constexpr (sizeof(T) == 4) {
        float a = __int_as_float(0x7f800000), b = __int_as_float(0xff800000);
#pragma unroll
        for (int e = 0; e < E; e++)
            if (e < nv) { a = fminf(a, v[e]); b = fmaxf(b, v[e]); }
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) {
            a = fminf(a, __shfl_xor_sync(0xffffffffu, a, d));
            b = fmaxf(b, __shfl_xor_sync(0xffffffffu, b, d));
        }
        mn = a;
        mx = b;
    } else {
        // order-preserving integer keys keep the FP64 pipe out of the reduction
        long long a = 0x7FFFFFFFFFFFFFFFll, b = (long long)0x8000000000000000ull;
#pragma unroll
        for (int e = 0; e < E; e++) {
            unsigned long long u = (unsigned long long)__double_as_longlong(v[e]);
            bool ok = e < nv && (u & 0x7FFFFFFFFFFFFFFFull) <= 0x7FF0000000000000ull;
            long long k = (long long)(u ^ ((unsigned long long)((long long)u >> 63) & 0x7FFFFFFFFFFFFFFFull));
            if (ok) { a = k < a ? k : a; b = k > b ? k : b; }
        }
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) {
            long long oa = __shfl_xor_sync(0xffffffffu, a, d), ob = __shfl_xor_sync(0xffffffffu, b, d);
            a = oa < a ? oa : a;
            b = ob > b ? ob : b;
        }
        auto inv = [](long long k) {
            unsigned long long u = (unsigned long long)k;
            return __longlong_as_double((long long)(u ^ ((unsigned long long)(k >> 63) & 0x7FFFFFFFFFFFFFFFull)));
        };
        mn = inv(a);
        mx = inv(b);
    }
    T x0 = __shfl_sync(0xffffffffu, v[0], 0);
    if (isnan(x0)) { mn = x0; mx = x0; return; }
    if (mn == (T)0 || mx == (T)0) {
        // a zero extreme keeps the sign of the first zero in the block
        int ze = E;
        T zv = 0;
#pragma unroll
        for (int e = E - 1; e >= 0; e--)
            if (e < nv && v[e] == (T)0) { ze = e; zv = v[e]; }
        unsigned m = __ballot_sync(0xffffffffu, ze < E);
        T first = __shfl_sync(0xffffffffu, zv, __ffs(m) - 1);
        if (mn == (T)0) mn = first;
        if (mx == (T)0) mx = first;
    }
}

// ------------------------------------------------------------------ encode

struct EncArgs {
    const void* x;
    unsigned long long n, nb, ntiles;
    int bs;
    int omp_stats;               // mode-4 double statistics
    float eb;
    const CodecParams* params;   // when set, params->eb overrides eb
    uint8_t* payload;            // fixed position of the payload region
    unsigned long long payload_cap;
    uint16_t* o_scr;
    uint32_t* m_scr;
    uint8_t* s_scr;
    TileStatus st;
    unsigned long long* tile_ctr;
    int* err;
    Totals* tot;
};

template <typename T, int E>
struct LaneEnc {
    typename Elem<T>::U cur[E];
    uint32_t codes;       // 2 bits per element, MSB-first
    uint32_t lane_bytes;  // mid bytes this lane emits
};

struct BlockEnc {
    int state;            // 0 constant, 1 non-constant, 2 absent
    int reqLength;
    uint32_t med_bits;    // median as stored
    uint32_t size;        // payload bytes (non-constant)
};

// Stats + shifted words + lead codes of one block (pass A).
template <typename T, int E>
__device__ __forceinline__ BlockEnc enc_block_a(const T* __restrict__ xb, int len, float eb, bool omp_stats,
                                                LaneEnc<T, E>& L) {
    using EL = Elem<T>;
    using U = typename EL::U;
    constexpr int W = EL::W;
    const int lane = (int)lane_id();
    int nv = len - lane * E;
    nv = nv < 0 ? 0 : (nv > E ? E : nv);
    T v[E];
    load_lane<T, E>(xb + lane * E, nv, lane_vec_ok<T, E>(xb) , v);
    T mn, mx;
    block_minmax<T, E>(v, nv, mn, mx);
    BlockEnc B;
    float radius_f, median_f;
    if constexpr (sizeof(T) == 4) {
        float range = xsub(mx, mn);
        radius_f = xdiv(range, 2.0f);
        median_f = xadd(mn, radius_f);
        B.state = (radius_f <= eb) ? 0 : 1;
    } else if (!omp_stats) {
        // szx/src/szx_double.cc:991-1003: double statistics, float median/radius
        double range = xsub(mx, mn);
        double radius = xdiv(range, 2.0);
        double median = xadd(mn, radius);
        B.state = (radius <= (double)eb) ? 0 : 1;
        radius_f = xd2f(radius);
        median_f = xd2f(median);
    } else {
        // OpenMP layout, computeStateMedianRadius_double2 (szx/src/szx_double.cc:1120-1135):
        // the median is formed from the float-rounded radius, compared in float
        double range = xsub(mx, mn);
        radius_f = xd2f(xdiv(range, 2.0));
        median_f = xd2f(xadd(mn, xf2d(radius_f)));
        B.state = (radius_f <= eb) ? 0 : 1;
    }
    B.med_bits = __float_as_uint(median_f);
    B.size = 0;
    B.reqLength = 0;
    L.codes = 0;
    L.lane_bytes = 0;
    if (B.state == 0) return B;
    bool zm;
    B.reqLength = req_length<T>(eb, radius_f, &zm);
    int R, s;
    split_reqlen(B.reqLength, &R, &s);
    if (zm) B.med_bits = 0;
    // float data subtracts the (possibly zeroed) median; double data subtracts
    // the float median widened, even when the stored one is zeroed (szx_double.cc:38)
    T med;
    if constexpr (sizeof(T) == 4) med = zm ? 0.0f : median_f;
    else med = xf2d(median_f);
    T d[E];
    bool bad = false;
#pragma unroll
    for (int e = 0; e < E; e++) {
        d[e] = EL::sub(v[e], med);
        bad |= d[e] != d[e];
    }
    if (__any_sync(0xffffffffu, bad)) {
#pragma unroll
        for (int e = 0; e < E; e++) d[e] = xsub(v[e], med);
    }
#pragma unroll
    for (int e = 0; e < E; e++) L.cur[e] = EL::bits(d[e]) >> s;
    U prev = __shfl_up_sync(0xffffffffu, L.cur[E - 1], 1);
    if (lane == 0) prev = 0;
#pragma unroll
    for (int e = 0; e < E; e++) {
        U xr = L.cur[e] ^ (e ? L.cur[e - 1] : prev);
        int lz;
        if constexpr (sizeof(T) == 4) lz = __clz(xr) >> 3;
        else lz = __clzll((long long)xr) >> 3;
        int ld = lz < 3 ? lz : 3;
        int cnt = R - ld;
        cnt = cnt > 0 ? cnt : 0;
        if (e < nv) {
            L.codes |= (uint32_t)ld << (2 * (E - 1 - e));
            L.lane_bytes += cnt;
        }
    }
    uint32_t total = warp_sum(L.lane_bytes);
    B.size = 5 + (uint32_t)((len + 3) / 4) + total;
    (void)W;
    return B;
}

// OR `cnt` bytes of `ev` into 32-bit words of a zeroed shared buffer at byte q.
__device__ __forceinline__ void or_bytes(uint32_t* buf, uint32_t q, uint32_t ev, int cnt) {
    if (cnt <= 0) return;
    uint32_t sh = (q & 3) * 8;
    uint32_t* w = buf + (q >> 2);
    atomicOr(w, ev << sh);
    if ((int)(q & 3) + cnt > 4) atomicOr(w + 1, ev >> (32 - sh));
}
__device__ __forceinline__ void or_bytes(uint32_t* buf, uint32_t q, unsigned long long ev, int cnt) {
    if (cnt <= 0) return;
    uint32_t sh = (q & 3) * 8;
    uint32_t* w = buf + (q >> 2);
    unsigned long long lo = ev << sh;
    atomicOr(w, (uint32_t)lo);
    int span = (int)(q & 3) + cnt;
    if (span > 4) atomicOr(w + 1, (uint32_t)(lo >> 32));
    if (span > 8) atomicOr(w + 2, (uint32_t)(ev >> (64 - sh)));
}

// Copy n bytes from a 16-aligned shared buffer (payload at offset sh) to global
// dst (with dst % 16 == sh) using aligned 16-byte stores for whole chunks.
__device__ __forceinline__ void warp_copy_out(const uint8_t* stage, uint32_t sh, uint32_t n, uint8_t* dst) {
    uint8_t* gbase = dst - sh;
    uint32_t end = sh + n;
    uint32_t nch = (end + 15) >> 4;
    for (uint32_t c = lane_id(); c < nch; c += 32) {
        uint32_t lo = c << 4, hi = lo + 16;
        if (lo >= sh && hi <= end) {
            *(uint4*)(gbase + lo) = *(const uint4*)(stage + lo);
        } else {
            uint32_t a = lo > sh ? lo : sh, b = hi < end ? hi : end;
            for (uint32_t j = a; j < b; j++) gbase[j] = stage[j];
        }
    }
}

// Emit one non-constant block's payload (pass B).
template <typename T, int E>
__device__ __forceinline__ void enc_block_b(uint8_t* stage, uint8_t* dst, int len, const BlockEnc& B,
                                            const LaneEnc<T, E>& L) {
    using EL = Elem<T>;
    using U = typename EL::U;
    constexpr int W = EL::W;
    const int lane = (int)lane_id();
    const uint32_t sh = (uint32_t)((uintptr_t)dst & 15);
    const uint32_t span = sh + B.size;
    const uint32_t nz = (span + 16 + 15) >> 4;
    for (uint32_t i = lane; i < nz; i += 32) ((uint4*)stage)[i] = make_uint4(0, 0, 0, 0);
    __syncwarp();
    uint8_t* p = stage + sh;
    int R, s;
    split_reqlen(B.reqLength, &R, &s);
    const int Lb = (len + 3) / 4;
    if (lane == 0) {
        p[0] = (uint8_t)B.reqLength;
        p[1] = (uint8_t)(B.med_bits >> 24);
        p[2] = (uint8_t)(B.med_bits >> 16);
        p[3] = (uint8_t)(B.med_bits >> 8);
        p[4] = (uint8_t)B.med_bits;
    }
    // lead codes: 4 per byte, MSB first (szx/src/szx_TypeManager.cc:198-273)
    if constexpr (E == 4) {
        if (lane < Lb) p[5 + lane] = (uint8_t)L.codes;
    } else if constexpr (E == 8) {
        if (2 * lane < Lb) p[5 + 2 * lane] = (uint8_t)(L.codes >> 8);
        if (2 * lane + 1 < Lb) p[6 + 2 * lane] = (uint8_t)L.codes;
    } else if constexpr (E == 2) {
        uint32_t nb = __shfl_down_sync(0xffffffffu, L.codes, 1);
        if ((lane & 1) == 0 && lane / 2 < Lb) p[5 + lane / 2] = (uint8_t)((L.codes << 4) | nb);
    } else {
        uint32_t c1 = __shfl_down_sync(0xffffffffu, L.codes, 1);
        uint32_t c2 = __shfl_down_sync(0xffffffffu, L.codes, 2);
        uint32_t c3 = __shfl_down_sync(0xffffffffu, L.codes, 3);
        if ((lane & 3) == 0 && lane / 4 < Lb) p[5 + lane / 4] = (uint8_t)((L.codes << 6) | (c1 << 4) | (c2 << 2) | c3);
    }
    // mid bytes: bytes [W-R .. W-1-lead] of each shifted word, ascending
    uint32_t incl = warp_inclusive_sum(L.lane_bytes);
    uint32_t q = sh + 5 + Lb + (incl - L.lane_bytes);
    uint32_t* buf = (uint32_t*)stage;
#pragma unroll
    for (int e = 0; e < E; e++) {
        int ld = (L.codes >> (2 * (E - 1 - e))) & 3;
        int cnt = R - ld;
        if (lane * E + e < len && cnt > 0) {
            U ev = L.cur[e] >> (8 * (W - R));
            if constexpr (sizeof(T) == 4) {
                ev &= cnt >= 4 ? 0xFFFFFFFFu : ((1u << (8 * cnt)) - 1);
                or_bytes(buf, q, (uint32_t)ev, cnt);
            } else {
                ev &= cnt >= 8 ? ~0ull : ((1ull << (8 * cnt)) - 1);
                or_bytes(buf, q, (unsigned long long)ev, cnt);
            }
            q += cnt;
        }
    }
    __syncwarp();
    warp_copy_out(stage, sh, B.size, dst);
    __syncwarp();
}

template <typename T, int E>
constexpr int enc_stage_bytes() {
    return ((16 + 5 + (32 * E + 3) / 4 + (int)sizeof(T) * 32 * E + 32 + 15) / 16) * 16;
}

template <typename T, int E, int BPW>
__global__ void __launch_bounds__(kEncThreads) k_blocked_encode(EncArgs a) {
    constexpr int TB = kEncWarps * BPW;
    static_assert(TB == 8 || TB == 16 || TB == 32, "tile of 8, 16 or 32 blocks");
    constexpr int STAGE = enc_stage_bytes<T, E>();
    __shared__ __align__(16) uint8_t s_stage[kEncWarps][STAGE];
    __shared__ uint32_t s_size[TB], s_med[TB];
    __shared__ int s_state[TB];
    __shared__ unsigned long long s_off[TB];
    __shared__ long long s_tile;
    __shared__ int s_skip;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const T* x = (const T*)a.x;
    const float eb = a.params ? a.params->eb : a.eb;
    for (;;) {
        if (threadIdx.x == 0) s_tile = (long long)atomicAdd(a.tile_ctr, 1ull);
        __syncthreads();
        const long long tile = s_tile;
        if (tile >= (long long)a.ntiles) break;
        LaneEnc<T, E> L[BPW];
        BlockEnc B[BPW];
#pragma unroll
        for (int k = 0; k < BPW; k++) {
            const int lb = warp * BPW + k;
            const unsigned long long b = (unsigned long long)tile * TB + lb;
            int len = 0;
            if (b < a.nb) {
                unsigned long long off = b * (unsigned long long)a.bs;
                unsigned long long rem = a.n - off;
                len = rem < (unsigned long long)a.bs ? (int)rem : a.bs;
                B[k] = enc_block_a<T, E>(x + off, len, eb, a.omp_stats, L[k]);
            } else {
                B[k].state = 2;
                B[k].size = 0;
                B[k].med_bits = 0;
            }
            if (lane == 0) {
                s_size[lb] = B[k].state == 1 ? B[k].size : 0;
                s_med[lb] = B[k].med_bits;
                s_state[lb] = B[k].state;
            }
        }
        __syncthreads();
        if (warp == 0) {
            const bool in = lane < TB;
            const int stt = in ? s_state[lane] : 2;
            const uint32_t sz = in ? s_size[lane] : 0;
            const uint32_t nn = stt == 1;
            const uint32_t isz = warp_inclusive_sum(sz);
            const uint32_t inn = warp_inclusive_sum(nn);
            const uint32_t agg_sz = __shfl_sync(0xffffffffu, isz, 31);
            const uint32_t agg_nn = __shfl_sync(0xffffffffu, inn, 31);
            unsigned long long base_sz, base_nn;
            lookback(a.st, tile, agg_sz, agg_nn, &base_sz, &base_nn, a.err);
            const bool cap_ok = base_sz + agg_sz <= a.payload_cap;
            if (in) s_off[lane] = base_sz + (isz - sz);
            if (in && stt != 2) {
                const unsigned long long b = (unsigned long long)tile * TB + lane;
                const unsigned long long rank = base_nn + (inn - nn);
                if (stt == 1) a.o_scr[rank] = (uint16_t)sz;
                else a.m_scr[b - rank] = s_med[lane];
            }
            const uint32_t mask = __ballot_sync(0xffffffffu, in && stt == 1);
            if (lane == 0) {
                const uint32_t rev = __brev(mask);
                if constexpr (TB == 32) *(uint32_t*)(a.s_scr + (unsigned long long)tile * 4) = bswap32(rev);
                else {
#pragma unroll
                    for (int k = 0; k < TB / 8; k++)
                        a.s_scr[(unsigned long long)tile * (TB / 8) + k] = (uint8_t)(rev >> (24 - 8 * k));
                }
                if (!cap_ok) atomicExch(a.err, kErrCapacity);
                if (tile == (long long)a.ntiles - 1) {
                    a.tot->payload_bytes = base_sz + agg_sz;
                    a.tot->nnc = base_nn + agg_nn;
                }
                s_skip = !cap_ok;
            }
        }
        __syncthreads();
        if (!s_skip) {
#pragma unroll
            for (int k = 0; k < BPW; k++) {
                const int lb = warp * BPW + k;
                if (B[k].state == 1) {
                    const unsigned long long b = (unsigned long long)tile * TB + lb;
                    const unsigned long long off = b * (unsigned long long)a.bs;
                    const unsigned long long rem = a.n - off;
                    const int len = rem < (unsigned long long)a.bs ? (int)rem : a.bs;
                    enc_block_b<T, E>(s_stage[warp], a.payload + s_off[lb], len, B[k], L[k]);
                }
            }
        }
        __syncthreads();
    }
}

// Header, size index, state bits and constant medians (szx/src/szx_float.cc:1437-1483).
__global__ void k_blocked_assemble(int layout, unsigned long long bs, unsigned long long nb, uint8_t* out,
                                   const Totals* tot, const uint16_t* o_scr, const uint32_t* m_scr,
                                   const uint8_t* s_scr, StreamResult* res, const CodecParams* params, float eb_abs,
                                   const int* err) {
    const unsigned long long nnc = tot->nnc, nc = nb - nnc, sb = (nb + 7) / 8;
    const bool ra = layout != kBlocked;
    const unsigned long long hdr = ra ? 20 : 13;
    const unsigned long long shift = ra ? 2 * nnc : 4 * nnc;
    uint8_t* s = out + shift;
    uint8_t* O = s + hdr;
    uint8_t* R = O + (ra ? 2 * nnc : 0);
    uint8_t* P = R + sb;
    const unsigned long long tid = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned long long nthr = (unsigned long long)gridDim.x * blockDim.x;
    unsigned long long m = nnc > nc ? nnc : nc;
    m = m > sb ? m : sb;
    for (unsigned long long i = tid; i < m; i += nthr) {
        if (ra && i < nnc) {
            uint16_t v = o_scr[i];
            O[2 * i] = (uint8_t)v;
            O[2 * i + 1] = (uint8_t)(v >> 8);
        }
        if (i < sb) R[i] = s_scr[i];
        if (i < nc) {
            uint32_t v = m_scr[i];
            if (layout == kRandomAccessNative) {
                P[4 * i] = (uint8_t)v; P[4 * i + 1] = (uint8_t)(v >> 8);
                P[4 * i + 2] = (uint8_t)(v >> 16); P[4 * i + 3] = (uint8_t)(v >> 24);
            } else {
                P[4 * i] = (uint8_t)(v >> 24); P[4 * i + 1] = (uint8_t)(v >> 16);
                P[4 * i + 2] = (uint8_t)(v >> 8); P[4 * i + 3] = (uint8_t)v;
            }
        }
    }
    if (tid == 0) {
        s[0] = 1; s[1] = 1; s[2] = 1; s[3] = ra ? 1 : 0;
        if (ra) {
            for (int k = 0; k < 8; k++) s[4 + k] = (uint8_t)(bs >> (56 - 8 * k));
            for (int k = 0; k < 8; k++) s[12 + k] = (uint8_t)(nc >> (56 - 8 * k));
        } else {
            s[4] = (uint8_t)bs;
            for (int k = 0; k < 8; k++) s[5 + k] = (uint8_t)(nc >> (56 - 8 * k));
        }
        StreamResult r;
        r.offset = shift;
        r.size = hdr + (ra ? 2 * nnc : 0) + sb + 4 * nc + tot->payload_bytes;
        r.nb_const = nc;
        r.eb = params ? params->eb : eb_abs;
        r.status = *err;
        *res = r;
    }
}

size_t blocked_bound(int layout, int dtype, size_t n, int bs) {
    size_t es = dtype == 0 ? 4 : 8;
    size_t nb = (n + bs - 1) / bs, sb = (nb + 7) / 8;
    size_t hdr = layout == kBlocked ? 13 : 20;
    return hdr + sb + 4 * nb + nb * (5 + ((size_t)bs + 3) / 4) + es * n + 64;
}

template <typename T, int E, int BPW>
static cudaError_t run_encode(const EncArgs& a, int grid, cudaStream_t s) {
    TraceScope tr("blocked_encode", s);
    k_blocked_encode<T, E, BPW><<<grid, kEncThreads, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_blocked_encode(int layout, int dtype, const void* x, size_t n, int bs, bool use_params,
                                  float abs_eb, uint8_t* d_out, size_t cap, const Workspace& ws, cudaStream_t s) {
    if (n == 0 || bs < 1 || bs > 256) return cudaErrorInvalidValue;
    if (layout == kBlocked && bs > 255) return cudaErrorInvalidValue;
    const int E = bs <= 32 ? 1 : bs <= 64 ? 2 : bs <= 128 ? 4 : 8;
    const int TB = E == 8 ? 16 : 32;
    const size_t nb = (n + bs - 1) / bs, sb = (nb + 7) / 8;
    const size_t ntiles = (nb + TB - 1) / TB;
    const size_t hdr = layout == kBlocked ? 13 : 20;
    const size_t qfix = hdr + sb + 4 * nb;
    if (cap < qfix) return cudaErrorInvalidValue;
    cudaError_t e;
    if ((e = cudaMemsetAsync(ws.st_word, 0, sizeof(unsigned long long) * ntiles, s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(ws.counters, 0, sizeof(unsigned long long), s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(ws.err, 0, sizeof(int), s)) != cudaSuccess) return e;
    EncArgs a;
    a.x = x; a.n = n; a.nb = nb; a.ntiles = ntiles; a.bs = bs; a.eb = abs_eb;
    a.omp_stats = layout == kRandomAccessNative;
    a.params = use_params ? ws.params : nullptr;
    a.payload = d_out + qfix;
    a.payload_cap = cap - qfix;
    a.o_scr = ws.o_scr; a.m_scr = ws.m_scr; a.s_scr = ws.s_scr;
    a.st = TileStatus{ws.st_word, ws.st_agg2, ws.st_inc2};
    a.tile_ctr = &ws.counters[0];
    a.err = ws.err;
    a.tot = ws.totals;
    const int per_sm = 4;
    size_t g = (size_t)sm_count() * per_sm;
    int grid = (int)(ntiles < g ? ntiles : g);
    if (dtype == 0) {
        if (E == 1) e = run_encode<float, 1, 4>(a, grid, s);
        else if (E == 2) e = run_encode<float, 2, 4>(a, grid, s);
        else if (E == 4) e = run_encode<float, 4, 4>(a, grid, s);
        else e = run_encode<float, 8, 2>(a, grid, s);
    } else {
        if (E == 1) e = run_encode<double, 1, 4>(a, grid, s);
        else if (E == 2) e = run_encode<double, 2, 4>(a, grid, s);
        else if (E == 4) e = run_encode<double, 4, 4>(a, grid, s);
        else e = run_encode<double, 8, 2>(a, grid, s);
    }
    if (e != cudaSuccess) return e;
    int ag = (int)((nb + 255) / 256);
    if (ag < 1) ag = 1;
    if (ag > sm_count() * 4) ag = sm_count() * 4;
    TraceScope tr("blocked_assemble", s);
    k_blocked_assemble<<<ag, 256, 0, s>>>(layout, (unsigned long long)bs, nb, d_out, ws.totals, ws.o_scr, ws.m_scr,
                                          ws.s_scr, ws.result, use_params ? ws.params : nullptr, abs_eb, ws.err);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ decode

__device__ __forceinline__ unsigned long long be64(const uint8_t* p) {
    unsigned long long v = 0;
    for (int i = 0; i < 8; i++) v = (v << 8) | p[i];
    return v;
}

// Parse and validate the mode-3/4 header (szx/src/szxd_float.cc:402-434).
__global__ void k_blocked_parse(const uint8_t* s, unsigned long long len, unsigned long long n,
                                unsigned long long bs_expect, BlockedHdr* h, int* err) {
    BlockedHdr r = {};
    r.n = n;
    r.ok = 0;
    if (len >= 20 && s[3] == 1) {
        r.bs = be64(s + 4);
        r.nc = be64(s + 12);
        if (r.bs >= 1 && r.bs <= 256 && (bs_expect == 0 || r.bs == bs_expect)) {
            r.nb = (n + r.bs - 1) / r.bs;
            r.sb = (r.nb + 7) / 8;
            if (r.nc <= r.nb) {
                r.nnc = r.nb - r.nc;
                r.o_off = 20;
                r.s_off = 20 + 2 * r.nnc;
                r.m_off = r.s_off + r.sb;
                r.q_off = r.m_off + 4 * r.nc;
                r.ok = r.q_off <= len;
            }
        }
    }
    *h = r;
    *err = r.ok ? kErrNone : kErrStream;
}

// CTA-wide exclusive sum over kIdxThreads threads.
__device__ __forceinline__ unsigned long long cta_exclusive_sum(unsigned long long v, unsigned long long* total,
                                                                unsigned long long* smem /*[8]*/) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned long long incl = warp_inclusive_sum(v);
    if (lane == 31) smem[warp] = incl;
    __syncthreads();
    unsigned long long wpre = 0, tot = 0;
#pragma unroll
    for (int w = 0; w < kIdxThreads / 32; w++) {
        unsigned long long x = smem[w];
        if (w < warp) wpre += x;
        tot += x;
    }
    __syncthreads();
    *total = tot;
    return wpre + incl - v;
}

// Two independent exclusive scans in one persistent launch:
//   family A: payload offsets  P[k] = sum O[0..k)          (k < nnc)
//   family B: rank words       RW[w] = popcount(state < 32w) (w < ceil(nb/32))
__global__ void __launch_bounds__(kIdxThreads) k_blocked_index(const uint8_t* s, const BlockedHdr* hp,
                                                               unsigned long long* P, uint32_t* RW,
                                                               TileStatus stA, TileStatus stB,
                                                               unsigned long long* ctr, int* err,
                                                               unsigned long long len) {
    __shared__ unsigned long long sm[8];
    __shared__ long long s_tile;
    __shared__ unsigned long long s_base;
    const BlockedHdr h = *hp;
    if (!h.ok) return;
    constexpr unsigned long long per = (unsigned long long)kIdxThreads * kIdxItems;
    const unsigned long long nw = (h.nb + 31) / 32;
    const long long TA = (long long)((h.nnc + per - 1) / per);
    const long long TBt = (long long)((nw + per - 1) / per);
    for (;;) {
        if (threadIdx.x == 0) s_tile = (long long)atomicAdd(ctr, 1ull);
        __syncthreads();
        long long t = s_tile;
        if (t >= TA + TBt) break;
        const bool famA = t < TA;
        const long long lt = famA ? t : t - TA;
        const unsigned long long first = (unsigned long long)lt * per + threadIdx.x * kIdxItems;
        unsigned long long vals[kIdxItems];
        unsigned long long mine = 0;
#pragma unroll
        for (int i = 0; i < kIdxItems; i++) {
            unsigned long long k = first + i;
            unsigned long long v = 0;
            if (famA) {
                if (k < h.nnc) v = (unsigned long long)s[h.o_off + 2 * k] | ((unsigned long long)s[h.o_off + 2 * k + 1] << 8);
            } else if (k < nw) {
                uint32_t w = 0;
                for (int j = 0; j < 4; j++) {
                    unsigned long long bi = 4 * k + j;
                    w = (w << 8) | (bi < h.sb ? s[h.s_off + bi] : 0u);
                }
                v = __popc(w);
            }
            vals[i] = v;
            mine += v;
        }
        unsigned long long tot;
        unsigned long long ex = cta_exclusive_sum(mine, &tot, sm);
        if (threadIdx.x < 32) {
            unsigned long long ba, bb;
            lookback(famA ? stA : stB, lt, tot, 0, &ba, &bb, err);
            if (threadIdx.x == 0) s_base = ba;
        }
        __syncthreads();
        unsigned long long run = s_base + ex;
#pragma unroll
        for (int i = 0; i < kIdxItems; i++) {
            unsigned long long k = first + i;
            if (famA) {
                if (k < h.nnc) P[k] = run;
                if (k == h.nnc - 1 && h.q_off + run + vals[i] > len) atomicExch(err, kErrStream);
            } else if (k < nw) {
                RW[k] = (uint32_t)run;
            }
            run += vals[i];
        }
        __syncthreads();
    }
}

// Stage `n` stream bytes starting at src into shared memory at offset src % 16.
__device__ __forceinline__ void warp_copy_in(uint8_t* stage, const uint8_t* src, uint32_t n, const uint8_t* s0,
                                             const uint8_t* s1) {
    const uint32_t sh = (uint32_t)((uintptr_t)src & 15);
    const uint8_t* gbase = src - sh;
    const uint32_t end = sh + n;
    const uint32_t nch = (end + 15) >> 4;
    for (uint32_t c = lane_id(); c < nch; c += 32) {
        const uint8_t* lo = gbase + (c << 4);
        if (lo >= s0 && lo + 16 <= s1) {
            *(uint4*)(stage + (c << 4)) = __ldg((const uint4*)lo);
        } else {
            for (int j = 0; j < 16; j++) {
                const uint8_t* q = lo + j;
                stage[(c << 4) + j] = (q >= s0 && q < s1) ? q[0] : 0;
            }
        }
    }
}

// Decode one non-constant block held in shared memory at p.
template <typename T, int E>
__device__ __forceinline__ void dec_block(const uint8_t* p, int len, T* outb) {
    using EL = Elem<T>;
    using U = typename EL::U;
    constexpr int W = EL::W;
    const int lane = (int)lane_id();
    const int reqLength = p[0];
    const uint32_t mb = ((uint32_t)p[1] << 24) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 8) | p[4];
    const float med_f = __uint_as_float(mb);
    int R, s;
    split_reqlen(reqLength, &R, &s);
    const int Lb = (len + 3) / 4;
    int nv = len - lane * E;
    nv = nv < 0 ? 0 : (nv > E ? E : nv);
    uint32_t codes;
    if constexpr (E == 4) codes = lane < Lb ? p[5 + lane] : 0;
    else if constexpr (E == 8) codes = ((2 * lane < Lb ? (uint32_t)p[5 + 2 * lane] : 0u) << 8) |
                                      (2 * lane + 1 < Lb ? (uint32_t)p[6 + 2 * lane] : 0u);
    else if constexpr (E == 2) codes = lane / 2 < Lb ? ((uint32_t)p[5 + lane / 2] >> ((lane & 1) ? 0 : 4)) & 0xF : 0;
    else codes = lane / 4 < Lb ? ((uint32_t)p[5 + lane / 4] >> (6 - 2 * (lane & 3))) & 3 : 0;
    int cnt[E];
    uint32_t lane_bytes = 0;
#pragma unroll
    for (int e = 0; e < E; e++) {
        int ld = (codes >> (2 * (E - 1 - e))) & 3;
        int c = R - ld;
        cnt[e] = (e < nv && c > 0) ? c : 0;
        lane_bytes += cnt[e];
    }
    const uint32_t incl = warp_inclusive_sum(lane_bytes);
    uint32_t q = (uint32_t)((uintptr_t)p & 15) + 5 + Lb + (incl - lane_bytes);
    const uint32_t* buf = (const uint32_t*)((uintptr_t)p & ~(uintptr_t)15);
    // stored parts, placed at their byte lanes
    U sp[E];
#pragma unroll
    for (int e = 0; e < E; e++) {
        uint32_t w0 = buf[q >> 2], w1 = buf[(q >> 2) + 1];
        uint32_t lo = __funnelshift_r(w0, w1, (q & 3) * 8);
        if constexpr (sizeof(T) == 4) {
            uint32_t m = cnt[e] >= 4 ? 0xFFFFFFFFu : ((1u << (8 * cnt[e])) - 1);
            sp[e] = (lo & m) << (8 * (W - R));
        } else {
            uint32_t w2 = buf[(q >> 2) + 2];
            uint32_t hi = __funnelshift_r(w1, w2, (q & 3) * 8);
            unsigned long long v = ((unsigned long long)hi << 32) | lo;
            unsigned long long m = cnt[e] >= 8 ? ~0ull : ((1ull << (8 * cnt[e])) - 1);
            sp[e] = (v & m) << (8 * (W - R));
        }
        q += cnt[e];
    }
    // top three byte lanes: the only ones a value can inherit from its
    // predecessor.  Packed summary: bits 0..23 bytes W-3..W-1, bits 24..26 written.
    constexpr int TOPSH = 8 * (W - 3);
    uint32_t sv = 0, sm = 0;
#pragma unroll
    for (int e = 0; e < E; e++) {
        if (e < nv) {
            int ld = (codes >> (2 * (E - 1 - e))) & 3;
            uint32_t wm = (1u << (3 - ld)) - 1;                       // lanes written: W-3 .. W-1-ld
            uint32_t wb = (wm & 1) * 0xFFu | (wm & 2) * 0x7F80u | (wm & 4) * 0x3FC000u;
            uint32_t top = (uint32_t)(sp[e] >> TOPSH) & 0xFFFFFFu;
            sv = (sv & ~wb) | (top & wb);
            sm |= wm;
        }
    }
    uint32_t sum = (sm << 24) | sv;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t o = __shfl_up_sync(0xffffffffu, sum, d);
        if (lane >= d) {
            uint32_t bm = sum >> 24;
            uint32_t wb = (bm & 1) * 0xFFu | (bm & 2) * 0x7F80u | (bm & 4) * 0x3FC000u;
            sum = (((o >> 24) | bm) << 24) | ((o & 0xFFFFFFu & ~wb) | (sum & 0xFFFFFFu & wb));
        }
    }
    uint32_t ex = __shfl_up_sync(0xffffffffu, sum, 1);
    if (lane == 0) ex = 0;   // previous value at block start is zero
    U prev = (U)(ex & 0xFFFFFFu) << TOPSH;
    const T med = widen_median<T>(med_f);
    T v[E];
    bool bad = false;
#pragma unroll
    for (int e = 0; e < E; e++) {
        int ld = (codes >> (2 * (E - 1 - e))) & 3;
        U inh = ld ? ~(((U)1 << (8 * (W - ld))) - 1) : (U)0;       // top `ld` bytes come from prev
        U cur = sp[e] | (prev & inh);
        sp[e] = cur << s;
        v[e] = EL::add(EL::of(sp[e]), med);
        bad |= v[e] != v[e];
        prev = cur;
    }
    if (__any_sync(0xffffffffu, bad)) {
#pragma unroll
        for (int e = 0; e < E; e++) v[e] = xadd(EL::of(sp[e]), med);
    }
    store_lane<T, E>(outb + lane * E, nv, lane_vec_ok<T, E>(outb), v);
}

template <typename T, int E>
constexpr int dec_stage_bytes() {
    return ((16 + 5 + (32 * E + 3) / 4 + (int)sizeof(T) * 32 * E + 32 + 15) / 16) * 16;
}

template <typename T, int E>
__global__ void __launch_bounds__(kDecThreads) k_blocked_decode(const uint8_t* __restrict__ s, unsigned long long len,
                                                                const BlockedHdr* hp,
                                                                const unsigned long long* __restrict__ P,
                                                                const uint32_t* __restrict__ RW, T* out,
                                                                int native_medians, int* err) {
    constexpr int STAGE = dec_stage_bytes<T, E>();
    __shared__ __align__(16) uint8_t s_stage[kDecThreads / 32][STAGE];
    const BlockedHdr h = *hp;
    if (!h.ok) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned long long gw = (unsigned long long)blockIdx.x * (kDecThreads / 32) + warp;
    const unsigned long long nwarps = (unsigned long long)gridDim.x * (kDecThreads / 32);
    const uint8_t* send = s + len;
    for (unsigned long long b = gw; b < h.nb; b += nwarps) {
        const unsigned long long off = b * h.bs;
        const unsigned long long rem = h.n - off;
        const int blen = rem < h.bs ? (int)rem : (int)h.bs;
        // state bit and non-constant rank
        const unsigned long long w = b >> 5;
        uint32_t word = 0;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            unsigned long long bi = 4 * w + j;
            word = (word << 8) | (bi < h.sb ? (uint32_t)s[h.s_off + bi] : 0u);
        }
        const int bit = (int)(b & 31);
        const bool nonconst = (word >> (31 - bit)) & 1;
        const unsigned long long rank = RW[w] + (bit ? __popc(word >> (32 - bit)) : 0);
        T* ob = out + off;
        if (!nonconst) {
            const uint8_t* mp = s + h.m_off + 4 * (b - rank);
            uint32_t mbits = native_medians
                                 ? ((uint32_t)mp[0] | ((uint32_t)mp[1] << 8) | ((uint32_t)mp[2] << 16) | ((uint32_t)mp[3] << 24))
                                 : (((uint32_t)mp[0] << 24) | ((uint32_t)mp[1] << 16) | ((uint32_t)mp[2] << 8) | mp[3]);
            T m = widen_median<T>(__uint_as_float(mbits));
            int nv = blen - lane * E;
            nv = nv < 0 ? 0 : (nv > E ? E : nv);
            T v[E];
#pragma unroll
            for (int e = 0; e < E; e++) v[e] = m;
            store_lane<T, E>(ob + lane * E, nv, lane_vec_ok<T, E>(ob), v);
            continue;
        }
        const unsigned long long po = h.q_off + P[rank];
        const uint32_t size = (uint32_t)s[h.o_off + 2 * rank] | ((uint32_t)s[h.o_off + 2 * rank + 1] << 8);
        const uint32_t minsz = 5 + (uint32_t)((blen + 3) / 4);
        if (po + size > len || size < minsz || size + 32 > (uint32_t)STAGE) {
            if (lane == 0) atomicExch(err, kErrStream);
            continue;
        }
        uint8_t* st = s_stage[warp];
        warp_copy_in(st, s + po, size, s, send);
        __syncwarp();
        dec_block<T, E>(st + ((uintptr_t)(s + po) & 15), blen, ob);
        __syncwarp();
    }
}

template <typename T, int E>
static void run_decode(const uint8_t* s, size_t len, size_t nb, const Workspace& ws, void* out, int native,
                       cudaStream_t st) {
    size_t want = (nb + (kDecThreads / 32) - 1) / (kDecThreads / 32);
    size_t cap = (size_t)sm_count() * 8;
    int grid = (int)(want < cap ? (want ? want : 1) : cap);
    TraceScope tr("blocked_decode", st);
    k_blocked_decode<T, E><<<grid, kDecThreads, 0, st>>>(s, len, ws.bhdr, ws.p_off, ws.rank_w, (T*)out, native,
                                                         ws.err);
}

cudaError_t launch_blocked_decode(int layout, int dtype, const uint8_t* d_stream, size_t len, size_t n, int bs,
                                  void* d_out, const Workspace& ws, cudaStream_t s) {
    if (layout != kRandomAccess && layout != kRandomAccessNative) return cudaErrorInvalidValue;
    if (bs < 1 || bs > 256 || n == 0) return cudaErrorInvalidValue;
    cudaError_t e;
    if ((e = cudaMemsetAsync(ws.counters, 0, sizeof(unsigned long long), s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(ws.st_word, 0, sizeof(unsigned long long) * ws.status_tiles, s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(ws.st2_word, 0, sizeof(unsigned long long) * ws.status2_tiles, s)) != cudaSuccess) return e;
    {
        TraceScope tr("blocked_parse", s);
        k_blocked_parse<<<1, 1, 0, s>>>(d_stream, len, n, (unsigned long long)bs, ws.bhdr, ws.err);
    }
    {
        int ig = sm_count() * 4;
        TraceScope tr("blocked_index", s);
        k_blocked_index<<<ig, kIdxThreads, 0, s>>>(d_stream, ws.bhdr, ws.p_off, ws.rank_w,
                                                    TileStatus{ws.st_word, ws.st_agg2, ws.st_inc2},
                                                    TileStatus{ws.st2_word, ws.st2_agg2, ws.st2_inc2},
                                                    &ws.counters[0], ws.err, len);
    }
    // bs comes from the stream header (read by the caller); the device header
    // is validated again by every kernel and a mismatch is reported, not used.
    const int native = layout == kRandomAccessNative;
    const int E = bs <= 32 ? 1 : bs <= 64 ? 2 : bs <= 128 ? 4 : 8;
    const size_t nb = (n + bs - 1) / bs;
    if (dtype == 0) {
        if (E == 1) run_decode<float, 1>(d_stream, len, nb, ws, d_out, native, s);
        else if (E == 2) run_decode<float, 2>(d_stream, len, nb, ws, d_out, native, s);
        else if (E == 4) run_decode<float, 4>(d_stream, len, nb, ws, d_out, native, s);
        else run_decode<float, 8>(d_stream, len, nb, ws, d_out, native, s);
    } else {
        if (E == 1) run_decode<double, 1>(d_stream, len, nb, ws, d_out, native, s);
        else if (E == 2) run_decode<double, 2>(d_stream, len, nb, ws, d_out, native, s);
        else if (E == 4) run_decode<double, 4>(d_stream, len, nb, ws, d_out, native, s);
        else run_decode<double, 8>(d_stream, len, nb, ws, d_out, native, s);
    }
    return cudaGetLastError();
}

}  // namespace szxg
