// Segment helpers shared by the blocked codec kernels: a block of up to G*E
// values is handled by a segment of G lanes of a warp (G a power of two),
// E = 16 float / 8 double values per lane, in chunks of 4 values.
#pragma once
#include "common.cuh"

namespace szxg {

// Reductions and scans run inside segments with shuffle widths of G, so
// several blocks share one warp instruction and the per-block work is
// replicated G times, not 32.

template <typename T> struct EncCfg;
template <> struct EncCfg<float> { static constexpr int E = 16; };    // values per lane
template <> struct EncCfg<double> { static constexpr int E = 8; };

template <int G, typename V>
__device__ __forceinline__ V seg_sum(V v) {
#pragma unroll
    for (int d = G / 2; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d, G);
    return v;
}
template <int G, typename V>
__device__ __forceinline__ V seg_inclusive_sum(V v) {
    const int sl = (int)(lane_id() & (G - 1));
#pragma unroll
    for (int d = 1; d < G; d <<= 1) {
        V o = __shfl_up_sync(0xffffffffu, v, d, G);
        if (sl >= d) v += o;
    }
    return v;
}

// Chunked lane layout.  A block is split into chunks of 4 values (one lead
// byte each); lane sl of a G-lane segment owns chunks sl, sl+G, sl+2G, ...
// so consecutive lanes touch consecutive chunks (no shared-memory bank
// conflicts) while each chunk stays contiguous for the XOR chain.
template <typename T, int G>
struct Chunks {
    static constexpr int E = EncCfg<T>::E;
    static constexpr int NC = E / 4;                  // chunks per lane
    static constexpr int CB = 4 * (int)sizeof(T);     // bytes per chunk
    // first value of the lane's k-th chunk
    static __device__ __forceinline__ int first(int sl, int k) { return 4 * (sl + k * G); }
};

template <typename T, int G>
__device__ __forceinline__ void load_chunks(const T* xs, int len, bool vec, T (&v)[EncCfg<T>::E]) {
    using C = Chunks<T, G>;
    const int sl = (int)(lane_id() & (G - 1));
#pragma unroll
    for (int k = 0; k < C::NC; k++) {
        const int f = C::first(sl, k);
        if (vec && f + 4 <= len) {
            if constexpr (sizeof(T) == 4) {
                const float4 q = *(const float4*)(xs + f);
                v[4 * k] = q.x; v[4 * k + 1] = q.y; v[4 * k + 2] = q.z; v[4 * k + 3] = q.w;
            } else {
                const double2 a = *(const double2*)(xs + f), b = *(const double2*)(xs + f + 2);
                v[4 * k] = a.x; v[4 * k + 1] = a.y; v[4 * k + 2] = b.x; v[4 * k + 3] = b.y;
            }
        } else {
#pragma unroll
            for (int i = 0; i < 4; i++) v[4 * k + i] = f + i < len ? xs[f + i] : (T)0;
        }
    }
}


template <typename T, int G>
__device__ __forceinline__ void store_chunks(T* ob, int len, bool vec, const T (&v)[EncCfg<T>::E]) {
    using C = Chunks<T, G>;
    const int sl = (int)(lane_id() & (G - 1));
#pragma unroll
    for (int k = 0; k < C::NC; k++) {
        const int f = C::first(sl, k);
        if (vec && f + 4 <= len) {
            if constexpr (sizeof(T) == 4) {
                *(float4*)(ob + f) = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
            } else {
                *(double2*)(ob + f) = make_double2(v[4 * k], v[4 * k + 1]);
                *(double2*)(ob + f + 2) = make_double2(v[4 * k + 2], v[4 * k + 3]);
            }
        } else {
#pragma unroll
            for (int i = 0; i < 4; i++)
                if (f + i < len) ob[f + i] = v[4 * k + i];
        }
    }
}

// Three-input forms (sm_100 and later): NaN inputs are ignored like fminf /
// fmaxf (fmax_nan / fmax3_nan, which propagate them, are in common.cuh).
__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
__device__ __forceinline__ float fmax3(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
// bytes [0, n) of a word set (n <= 0: none, n >= 4: all)
__device__ __forceinline__ uint32_t low_bytes_mask(int n) {
    return n >= 4 ? 0xFFFFFFFFu : (n <= 0 ? 0u : 0xFFFFFFFFu >> (32 - 8 * n));
}

// Segment-wide min/max with the reference's sequential semantics
// (szx/src/szx_float.cc:322-345): the first value reaching an extreme wins,
// NaNs are skipped unless the block's first value is NaN.  `special` is set
// (segment-uniform) when the block holds a NaN or an infinity, where the
// x86 NaN rules of the subtraction matter.
template <typename T, int G, bool FULL>
__device__ __forceinline__ void seg_minmax(const T (&v)[EncCfg<T>::E], int len, T& mn, T& mx, bool& special) {
    using C = Chunks<T, G>;
    constexpr int E = C::E;
    const int sl = (int)(lane_id() & (G - 1));
    if constexpr (sizeof(T) == 4) {
        float lo = __builtin_huge_valf(), hi = -__builtin_huge_valf(), hn = -__builtin_huge_valf();
        if constexpr (FULL) {
#pragma unroll
            for (int e = 0; e < E; e += 2) {
                lo = fmin3(lo, v[e], v[e + 1]);
                hi = fmax3(hi, v[e], v[e + 1]);
                hn = fmax3_nan(hn, v[e], v[e + 1]);
            }
        } else {
#pragma unroll
            for (int e = 0; e < E; e++) {
                if (C::first(sl, e / 4) + (e & 3) < len) {
                    lo = fminf(lo, v[e]);
                    hi = fmaxf(hi, v[e]);
                    hn = fmax_nan(hn, v[e]);
                }
            }
        }
#pragma unroll
        for (int d = G / 2; d > 0; d >>= 1) {
            lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, d, G));
            hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, d, G));
        }
        mn = lo;
        mx = hi;
        // a NaN anywhere in the segment: one vote instead of a reduction
        const unsigned seg0 = lane_id() & ~(unsigned)(G - 1);
        const unsigned segmask = G == 32 ? 0xffffffffu : (((1u << G) - 1) << seg0);
        special = (__ballot_sync(0xffffffffu, isnan(hn)) & segmask) != 0 || isinf(lo) || isinf(hi);
    } else {
        long long lo = 0x7FFFFFFFFFFFFFFFll, hi = (long long)0x8000000000000000ull;
        bool nan = false;
#pragma unroll
        for (int e = 0; e < E; e++) {
            const unsigned long long u = (unsigned long long)__double_as_longlong(v[e]);
            const bool in = FULL || C::first(sl, e / 4) + (e & 3) < len;
            const bool fin = (u & 0x7FFFFFFFFFFFFFFFull) <= 0x7FF0000000000000ull;
            const long long k = (long long)(u ^ ((unsigned long long)((long long)u >> 63) & 0x7FFFFFFFFFFFFFFFull));
            if (in && fin) {
                lo = k < lo ? k : lo;
                hi = k > hi ? k : hi;
            }
            nan |= in && !fin;
        }
#pragma unroll
        for (int d = G / 2; d > 0; d >>= 1) {
            const long long a = __shfl_xor_sync(0xffffffffu, lo, d, G), b = __shfl_xor_sync(0xffffffffu, hi, d, G);
            lo = a < lo ? a : lo;
            hi = b > hi ? b : hi;
        }
        auto inv = [](long long k) {
            const unsigned long long u = (unsigned long long)k;
            return __longlong_as_double((long long)(u ^ ((unsigned long long)(k >> 63) & 0x7FFFFFFFFFFFFFFFull)));
        };
        mn = inv(lo);
        mx = inv(hi);
        const unsigned nm = __ballot_sync(0xffffffffu, nan);
        const unsigned seg0 = lane_id() & ~(unsigned)(G - 1);
        const unsigned segmask = G == 32 ? 0xffffffffu : (((1u << G) - 1) << seg0);
        special = (nm & segmask) != 0 || isinf(mn) || isinf(mx);
    }
    // a zero extreme takes the sign of the block's first zero; only warps
    // that met one pay for the search
    if (__any_sync(0xffffffffu, mn == (T)0 || mx == (T)0)) {
        int zi = 1 << 30;
        T zv = 0;
#pragma unroll
        for (int e = E - 1; e >= 0; e--) {
            const int idx = C::first(sl, e / 4) + (e & 3);
            if ((FULL || idx < len) && v[e] == (T)0 && idx < zi) { zi = idx; zv = v[e]; }
        }
        int best = zi;
#pragma unroll
        for (int d = G / 2; d > 0; d >>= 1) best = min(best, __shfl_xor_sync(0xffffffffu, best, d, G));
        const unsigned m = __ballot_sync(0xffffffffu, zi == best && zi < (1 << 30));
        const unsigned seg0 = lane_id() & ~(unsigned)(G - 1);
        const unsigned segmask = G == 32 ? 0xffffffffu : (((1u << G) - 1) << seg0);
        const unsigned mm = m & segmask;
        const T first = __shfl_sync(0xffffffffu, zv, mm ? __ffs(mm) - 1 : (int)seg0);
        if (mm) {
            if (mn == (T)0) mn = first;
            if (mx == (T)0) mx = first;
        }
    }
    // a NaN first value pins both extremes; only a block holding a NaN can have one
    if (__any_sync(0xffffffffu, special)) {
        const T x0 = __shfl_sync(0xffffffffu, v[0], 0, G);
        if (isnan(x0)) { mn = x0; mx = x0; }
    }
}


// Lead codes of a block's shifted words (szx/src/szx_float.cc:94-113,
// szx/src/szx_double.cc:78-97): per chunk of the lane, the leading identical
// bytes (capped at 3) of each value with its predecessor in block order
// (zero before the block), value i of the chunk in byte i.
template <typename T, int G>
__device__ __forceinline__ void seg_lead_bytes(const typename Elem<T>::U (&cur)[EncCfg<T>::E],
                                               uint32_t (&ldb)[EncCfg<T>::E / 4]) {
    using U = typename Elem<T>::U;
    constexpr int NC = EncCfg<T>::E / 4;
    const int sl = (int)(lane_id() & (G - 1));
    U wrap = 0;   // lane 0: the last lane's value of the previous round (zero before the block)
#pragma unroll
    for (int k = 0; k < NC; k++) {
        // value before this chunk: the previous lane's chunk k, or for lane 0
        // the last lane's chunk k-1 -- one rotation per round serves both
        const U rot = __shfl_sync(0xffffffffu, cur[4 * k + 3], (sl + G - 1) & (G - 1), G);
        const U prev = sl ? rot : wrap;
        wrap = rot;
        uint32_t b = 0;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const U xr = cur[4 * k + i] ^ (i ? cur[4 * k + i - 1] : prev);
            uint32_t lz;
            if constexpr (sizeof(T) == 4) lz = (uint32_t)__clz(xr | 0xFFu) >> 3;
            else lz = (uint32_t)__clzll((long long)(xr | 0xFFFFFFFFFFull)) >> 3;
            b |= lz << (8 * i);
        }
        ldb[k] = b;
    }
}

}  // namespace szxg
