// Device-side building blocks shared by the SZx codec kernels.
//
// Everything here is bit-level arithmetic of the SZx stream format
// (szcompressor/SZx) restated for the GPU: IEEE patterns, the logical shifts of
// the reference's unsigned unions (szx/include/szx.h:56-68), big-endian header
// fields (szx/src/szx_BytesToolkit.cc:266-317,460-476) and the scans that place
// variable-length payloads.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace szxg {

constexpr int kWarp = 32;

// ------------------------------------------------------------------ element traits

template <typename T> struct Elem;
template <> struct Elem<float> {
    using U = uint32_t;
    static constexpr int W = 4;          // bytes per word
    static __device__ __forceinline__ U bits(float v) { return __float_as_uint(v); }
    static __device__ __forceinline__ float of(U u) { return __uint_as_float(u); }
    // leading identical bytes of the XOR, szx/src/szx_float.cc:96-101
    static __device__ __forceinline__ int lead(U x) {
        return x < (1u << 8) ? 3 : x < (1u << 16) ? 2 : x < (1u << 24) ? 1 : 0;
    }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
};
template <> struct Elem<double> {
    using U = unsigned long long;
    static constexpr int W = 8;
    static __device__ __forceinline__ U bits(double v) { return (U)__double_as_longlong(v); }
    static __device__ __forceinline__ double of(U u) { return __longlong_as_double((long long)u); }
    // szx/src/szx_double.cc:80-85
    static __device__ __forceinline__ int lead(U x) {
        return x < (1ull << 40) ? 3 : x < (1ull << 48) ? 2 : x < (1ull << 56) ? 1 : 0;
    }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
};

// ------------------------------------------------------------------ x86 NaN rules
//
// The reference runs on x86-64 SSE, where an arithmetic NaN result is the
// first NaN operand, quieted (the second when only it is NaN), an invalid
// operation (inf - inf, 0/0) gives the negative "indefinite" NaN, and
// float<->double conversions keep the payload.  CUDA returns one canonical
// NaN instead.  These helpers restore the x86 result; the hot loops call the
// plain operation and take the fix-up path only when a warp saw a NaN.
__device__ __forceinline__ float nan_rule(float a, float b) {
    uint32_t ua = __float_as_uint(a), ub = __float_as_uint(b);
    if ((ua & 0x7FFFFFFFu) > 0x7F800000u) return __uint_as_float(ua | 0x00400000u);
    if ((ub & 0x7FFFFFFFu) > 0x7F800000u) return __uint_as_float(ub | 0x00400000u);
    return __uint_as_float(0xFFC00000u);
}
__device__ __forceinline__ double nan_rule(double a, double b) {
    unsigned long long ua = (unsigned long long)__double_as_longlong(a);
    unsigned long long ub = (unsigned long long)__double_as_longlong(b);
    if ((ua & 0x7FFFFFFFFFFFFFFFull) > 0x7FF0000000000000ull) return __longlong_as_double((long long)(ua | 0x0008000000000000ull));
    if ((ub & 0x7FFFFFFFFFFFFFFFull) > 0x7FF0000000000000ull) return __longlong_as_double((long long)(ub | 0x0008000000000000ull));
    return __longlong_as_double((long long)0xFFF8000000000000ull);
}
__device__ __forceinline__ float xsub(float a, float b) { float r = __fsub_rn(a, b); return r == r ? r : nan_rule(a, b); }
__device__ __forceinline__ float xadd(float a, float b) { float r = __fadd_rn(a, b); return r == r ? r : nan_rule(a, b); }
__device__ __forceinline__ float xmul(float a, float b) { float r = __fmul_rn(a, b); return r == r ? r : nan_rule(a, b); }
__device__ __forceinline__ float xdiv(float a, float b) { float r = __fdiv_rn(a, b); return r == r ? r : nan_rule(a, b); }
__device__ __forceinline__ double xsub(double a, double b) { double r = __dsub_rn(a, b); return r == r ? r : nan_rule(a, b); }
__device__ __forceinline__ double xadd(double a, double b) { double r = __dadd_rn(a, b); return r == r ? r : nan_rule(a, b); }
__device__ __forceinline__ double xmul(double a, double b) { double r = __dmul_rn(a, b); return r == r ? r : nan_rule(a, b); }
__device__ __forceinline__ double xdiv(double a, double b) { double r = __ddiv_rn(a, b); return r == r ? r : nan_rule(a, b); }
// cvtsd2ss / cvtss2sd
__device__ __forceinline__ float xd2f(double d) {
    if (d == d) return __double2float_rn(d);
    unsigned long long b = (unsigned long long)__double_as_longlong(d);
    return __uint_as_float((uint32_t)(b >> 32 & 0x80000000u) | 0x7FC00000u | (uint32_t)(b >> 29 & 0x7FFFFFu));
}
__device__ __forceinline__ double xf2d(float f) {
    if (f == f) return (double)f;
    uint32_t b = __float_as_uint(f);
    return __longlong_as_double((long long)(((unsigned long long)(b & 0x80000000u) << 32) | 0x7FF8000000000000ull |
                                            ((unsigned long long)(b & 0x7FFFFFu) << 29)));
}
template <typename T> __device__ __forceinline__ T widen_median(float m);
template <> __device__ __forceinline__ float widen_median<float>(float m) { return m; }
template <> __device__ __forceinline__ double widen_median<double>(float m) { return xf2d(m); }

// getExponent_float / getPrecisionReqLength_double, szx/src/szx_BytesToolkit.cc:335-387
__device__ __forceinline__ int exponent_f32(float v) { return (int)((__float_as_uint(v) & 0x7F800000u) >> 23) - 127; }
__device__ __forceinline__ int exponent_f64_of_f32(float v) {
    unsigned long long b = (unsigned long long)__double_as_longlong((double)v);
    return (int)((b & 0x7FF0000000000000ull) >> 52) - 1023;
}
// computeReqLength_float (szx/src/szx_float.cc:1708-1717) / _double
// (szx/src/szx_double.cc:2020-2031).  Returns reqLength; *zero_median set when
// the clamp at the word width zeroes the stored median.
template <typename T> __device__ __forceinline__ int req_length(float eb, float radius, bool* zero_median);
template <> __device__ __forceinline__ int req_length<float>(float eb, float radius, bool* zm) {
    int r = 10 + exponent_f32(radius) - exponent_f64_of_f32(eb);
    *zm = false;
    if (r < 9) r = 9;
    if (r > 32) { r = 32; *zm = true; }
    return r;
}
template <> __device__ __forceinline__ int req_length<double>(float eb, float radius, bool* zm) {
    int r = 12 + exponent_f32(radius) - exponent_f64_of_f32(eb);
    *zm = false;
    if (r < 12) r = 12;
    if (r > 64) { r = 64; *zm = true; }
    return r;
}
__device__ __forceinline__ void split_reqlen(int reqLength, int* R, int* s) {
    int rb = reqLength & 7;
    *R = (reqLength >> 3) + (rb != 0);
    *s = rb ? 8 - rb : 0;
}

__device__ __forceinline__ uint32_t bswap32(uint32_t v) { return __byte_perm(v, 0, 0x0123); }

// ------------------------------------------------------------------ warp scans

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31; }

template <typename V>
__device__ __forceinline__ V warp_inclusive_sum(V v) {
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        V o = __shfl_up_sync(0xffffffffu, v, d);
        if ((int)lane_id() >= d) v += o;
    }
    return v;
}
template <typename V>
__device__ __forceinline__ V warp_sum(V v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
    return v;
}

// ------------------------------------------------------------------ acquire/release

__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned long long* p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_acquire32(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// ------------------------------------------------------------------ decoupled look-back
//
// Single-pass exclusive prefix over tiles (Merrill & Garland, "Single-pass
// Parallel Prefix Scan with Decoupled Look-back", NVR-2016-002).  The status
// word of a tile packs a 2-bit flag over a 62-bit byte count; a second 64-bit
// count (e.g. non-constant blocks) travels in side arrays written before the
// flag is released.  Tiles are taken in order from an atomic counter, so every
// predecessor is running or done and the look-back always ends; the spin is
// still capped and reports through *err instead of hanging.

constexpr unsigned long long kFlagAgg = 1ull << 62;
constexpr unsigned long long kFlagInc = 2ull << 62;
constexpr unsigned long long kValMask = (1ull << 62) - 1;
constexpr unsigned kSpinLimit = 1u << 22;   // polls before giving up (~seconds with backoff)

enum : int { kErrNone = 0, kErrLookback = 1, kErrCapacity = 2, kErrStream = 3 };

struct TileStatus {
    unsigned long long* word;     // [ntiles] flag|bytes
    unsigned long long* agg2;     // [ntiles] second count, aggregate
    unsigned long long* inc2;     // [ntiles] second count, inclusive
};

// Combine rules for the second value.
struct SumOp {
    static __device__ __forceinline__ unsigned long long id() { return 0; }
    static __device__ __forceinline__ unsigned long long op(unsigned long long x, unsigned long long y) { return x + y; }
    static __device__ __forceinline__ unsigned long long warp_reduce(unsigned long long v) { return warp_sum(v); }
};
// Three 21-bit fields combined by max each (latest tile index + 1, 0 = none).
struct Max3x21Op {
    static __device__ __forceinline__ unsigned long long id() { return 0; }
    static __device__ __forceinline__ unsigned long long op(unsigned long long x, unsigned long long y) {
        unsigned long long r = 0;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            unsigned long long a = (x >> (21 * k)) & 0x1FFFFF, b = (y >> (21 * k)) & 0x1FFFFF;
            r |= (a > b ? a : b) << (21 * k);
        }
        return r;
    }
    static __device__ __forceinline__ unsigned long long warp_reduce(unsigned long long v) {
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, d));
        return v;
    }
};

// Called by one whole warp.  Publishes the tile's aggregate (a, b), walks back
// over predecessors and returns the exclusive prefix.  Lane 0 of the warp
// publishes; all lanes get the result.  `a` is always a sum; `b` combines by Op.
template <typename Op = SumOp>
__device__ __forceinline__ void lookback(TileStatus st, long long tile, unsigned long long a,
                                         unsigned long long b, unsigned long long* ex_a,
                                         unsigned long long* ex_b, int* err) {
    const unsigned lane = lane_id();
    if (tile == 0) {
        if (lane == 0) {
            st.inc2[0] = b;
            __threadfence();
            st_release(&st.word[0], kFlagInc | (a & kValMask));
        }
        *ex_a = 0;
        *ex_b = Op::id();
        return;
    }
    if (lane == 0) {
        st.agg2[tile] = b;
        __threadfence();
        st_release(&st.word[tile], kFlagAgg | (a & kValMask));
    }
    unsigned long long pa = 0, pb = Op::id();
    long long base = tile - 1;
    unsigned spins = 0;
    bool failed = false;
    while (true) {
        // lane l inspects predecessor base - l; tiles below 0 read as an
        // inclusive prefix of zero, so the walk always stops.
        long long t = base - (long long)lane;
        unsigned long long w = kFlagInc;
        if (t >= 0) w = ld_acquire(&st.word[t]);
        unsigned long long flag = w & ~kValMask;
        unsigned inc_mask = __ballot_sync(0xffffffffu, flag == kFlagInc);
        unsigned stop = inc_mask ? (unsigned)__ffs(inc_mask) - 1 : 31u;
        unsigned window = stop == 31u ? 0xffffffffu : ((1u << (stop + 1)) - 1);
        unsigned not_ready = __ballot_sync(0xffffffffu, flag == 0) & window;
        if (not_ready) {
            if (++spins > kSpinLimit) { failed = true; break; }
            __nanosleep(spins < 64 ? 32 : 256);
            continue;
        }
        unsigned long long va = 0, vb = Op::id();
        if (t >= 0 && lane <= stop) {
            va = w & kValMask;
            vb = (flag == kFlagInc) ? __ldcg(&st.inc2[t]) : __ldcg(&st.agg2[t]);
        }
        pa += warp_sum(va);
        pb = Op::op(Op::warp_reduce(vb), pb);
        if (inc_mask) break;
        base -= 32;
    }
    if (failed && lane == 0) atomicExch(err, kErrLookback);
    if (lane == 0) {
        st.inc2[tile] = Op::op(pb, b);
        __threadfence();
        st_release(&st.word[tile], kFlagInc | ((pa + a) & kValMask));
    }
    *ex_a = pa;
    *ex_b = pb;
}

}  // namespace szxg
