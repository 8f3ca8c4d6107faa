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
// max with NaN propagation (a NaN input gives a NaN), two and three inputs
// (the three-input form is sm_100 and later)
__device__ __forceinline__ float fmax_nan(float a, float b) {
    float r;
    asm("max.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float fmax3_nan(float a, float b, float c) {
    float r;
    asm("max.NaN.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
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
// x / 2 as a multiplication: both are the correctly rounded value of the same
// real number (subnormal results included), and a NaN x propagates the same
// way, so the result is bit-identical to the division at a fraction of its
// cost.
__device__ __forceinline__ float xhalf(float x) { return xmul(x, 0.5f); }
__device__ __forceinline__ double xhalf(double x) { return xmul(x, 0.5); }
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
// The bound's exponent (exponent_f64_of_f32(eb)) is a per-field constant:
// callers that place many blocks under one bound compute it once and use the
// eb_exp overloads.
template <typename T> __device__ __forceinline__ int req_length_e(int eb_exp, float radius, bool* zero_median);
template <> __device__ __forceinline__ int req_length_e<float>(int eb_exp, float radius, bool* zm) {
    int r = 10 + exponent_f32(radius) - eb_exp;
    *zm = false;
    if (r < 9) r = 9;
    if (r > 32) { r = 32; *zm = true; }
    return r;
}
template <> __device__ __forceinline__ int req_length_e<double>(int eb_exp, float radius, bool* zm) {
    int r = 12 + exponent_f32(radius) - eb_exp;
    *zm = false;
    if (r < 12) r = 12;
    if (r > 64) { r = 64; *zm = true; }
    return r;
}
template <typename T> __device__ __forceinline__ int req_length(float eb, float radius, bool* zero_median) {
    return req_length_e<T>(exponent_f64_of_f32(eb), radius, zero_median);
}
// Stored-byte counts of four values, max(R - lead, 0) per byte, for leads in
// 0..3 and R in 1..8 (what __vsubus4(R * 0x01010101, leads) returns) without
// the emulated SIMD instruction: R is raised by the bytes whose lead exceeds
// it (lead 3 when R <= 2, lead >= 2 when R == 1) so the subtraction never
// borrows across bytes.
__device__ __forceinline__ uint32_t stored_counts(int R, uint32_t ldb) {
    const uint32_t hi = (ldb >> 1) & 0x01010101u;   // lead >= 2
    const uint32_t l3 = ldb & hi;                   // lead == 3
    uint32_t up = R <= 2 ? l3 : 0u;
    if (R <= 1) up += hi;
    return (uint32_t)R * 0x01010101u + up - ldb;
}
__device__ __forceinline__ void split_reqlen(int reqLength, int* R, int* s) {
    int rb = reqLength & 7;
    *R = (reqLength >> 3) + (rb != 0);
    *s = rb ? 8 - rb : 0;
}

__device__ __forceinline__ uint32_t bswap32(uint32_t v) { return __byte_perm(v, 0, 0x0123); }
// byte i of x, zero-extended
__device__ __forceinline__ uint32_t byte_of(uint32_t x, int i) { return __byte_perm(x, 0, 0x4440 | i); }
// top `n8 / 8` bytes of a 32-bit word set (n8 = 8 * bytes, 0..24)
__device__ __forceinline__ uint32_t top_bytes_mask(uint32_t n8) { return __funnelshift_r(0u, 0xFFFFFFFFu, n8); }

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
constexpr unsigned kSpinLimit = 1u << 22;   // polls before giving up (~1 s with backoff)
// Every look-back below takes its poll limit as a last argument (default
// kSpinLimit); the failure-detection self-test (selftest.cu) passes a small
// one and withholds a tile, so the give-up path runs for real.

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
                                         unsigned long long* ex_b, int* err, unsigned limit = kSpinLimit) {
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
            if (++spins > limit) { failed = true; break; }
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

// ------------------------------------------------------------------ TMA bulk copies + mbarriers
//
// One thread arms an mbarrier with the byte count and issues a 1-D bulk copy
// (cp.async.bulk) global -> shared; consumers wait on the barrier's phase.
// Source, destination and size must be multiples of 16 bytes.

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// Raise the transaction count the current phase waits for, without arriving.
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, uint32_t bytes) {
    asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void tma_load_1d(void* dst, const void* src, uint32_t bytes, unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: gives up (returns false) after kSpinLimit polls.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, uint32_t parity) {
    for (unsigned i = 0; i < (1u << 22); i++) {
        if (mbar_try_wait(bar, parity)) return true;
        if (i > 16) __nanosleep(64);
    }
    return false;
}

// ------------------------------------------------------------------ wide look-back
//
// Tile status as one 32-bit word: [31:30] flag (0 empty, 1 aggregate,
// 2 inclusive), [29:23] the tile's second count (<= 127), [22:0] the tile's
// byte count (< 8 MiB).  Inclusive prefixes (64-bit) live in side arrays
// written before the inclusive flag is released.  A walking warp reads 8
// consecutive status words per lane (two 16-byte loads), i.e. 256
// predecessors per memory round trip: the rate at which tiles can be placed
// is then (256 / round-trip latency) instead of 32 / latency, which is what
// lets a look-back over 16-32 KiB tiles keep up with HBM3e.
struct TileStatus32 {
    uint32_t* st;                  // [ntiles + 8], zeroed before the launch
    unsigned long long* inc_a;     // [ntiles]
    unsigned long long* inc_b;     // [ntiles]
};
constexpr uint32_t kSt32Agg = 1u << 30, kSt32Inc = 2u << 30;

__device__ __forceinline__ void st_volatile32(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint4 ld_volatile_v4(const uint32_t* p) {
    uint4 v;
    asm volatile("ld.relaxed.gpu.global.v4.u32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p)
                 : "memory");
    return v;
}

// Second-value policies of the wide look-back.
// SumPolicy: the 7-bit field is a count, prefixes add.
struct SumPolicy {
    static __device__ __forceinline__ unsigned long long contrib(uint32_t f, long long) { return f; }
    static __device__ __forceinline__ unsigned long long op(unsigned long long x, unsigned long long y) { return x + y; }
    static __device__ __forceinline__ unsigned long long reduce(unsigned long long v) { return warp_sum(v); }
};

// Whole warp.  agg_a < 2^23 (a sum), agg_b < 128 (combined by Policy).
// Returns the exclusive prefixes.
template <typename Policy = SumPolicy>
__device__ __forceinline__ void lookback_wide(TileStatus32 s, long long tile, uint32_t agg_a, uint32_t agg_b,
                                              unsigned long long* ex_a, unsigned long long* ex_b, int* err,
                                              unsigned limit = kSpinLimit) {
    const unsigned lane = lane_id();
    const uint32_t packed = (agg_b << 23) | (agg_a & 0x7FFFFFu);
    const unsigned long long self_b = Policy::contrib(agg_b, tile);
    if (tile == 0) {
        if (lane == 0) {
            __stcg(&s.inc_a[0], (unsigned long long)agg_a);
            __stcg(&s.inc_b[0], self_b);
            __threadfence();
            st_volatile32(&s.st[0], kSt32Inc | packed);
        }
        *ex_a = 0;
        *ex_b = 0;
        return;
    }
    if (lane == 0) st_volatile32(&s.st[tile], kSt32Agg | packed);
    unsigned long long pa = 0, pb = 0;
    long long g0 = ((tile - 1) >> 3) << 3;   // group of 8 holding the nearest predecessor
    unsigned spins = 0;
    bool failed = false;
    while (true) {
        const long long g = g0 - 8 * (long long)lane;
        uint32_t w[8];
        if (g >= 0) {
            uint4 a = ld_volatile_v4(s.st + g), b = ld_volatile_v4(s.st + g + 4);
            w[0] = a.x; w[1] = a.y; w[2] = a.z; w[3] = a.w; w[4] = b.x; w[5] = b.y; w[6] = b.z; w[7] = b.w;
        } else {
#pragma unroll
            for (int j = 0; j < 8; j++) w[j] = kSt32Inc;   // before tile 0: an inclusive zero
        }
        // nearest inclusive predecessor in this lane (highest index), and the
        // readiness / combination of the aggregates above it
        int inc_j = -1;
        bool ready = true;
        uint32_t sa = 0;
        unsigned long long sb = 0;
#pragma unroll
        for (int j = 7; j >= 0; j--) {
            const long long u = g + j;
            const bool pred = u < tile;
            const uint32_t f = w[j] & 0xC0000000u;
            if (pred && inc_j < 0) {
                if (f == kSt32Inc) inc_j = j;
                else {
                    ready = ready && f != 0;
                    sa += w[j] & 0x7FFFFFu;
                    sb = Policy::op(sb, Policy::contrib((w[j] >> 23) & 0x7Fu, u));
                }
            }
        }
        const unsigned inc_mask = __ballot_sync(0xffffffffu, inc_j >= 0);
        const unsigned stop = inc_mask ? (unsigned)__ffs(inc_mask) - 1 : 31u;
        const unsigned window = stop == 31u ? 0xffffffffu : ((1u << (stop + 1)) - 1);
        if (__ballot_sync(0xffffffffu, !ready) & window) {
            if (++spins > limit) { failed = true; break; }
            __nanosleep(spins < 64 ? 32 : 256);
            continue;
        }
        unsigned long long va = 0, vb = 0;
        if (lane <= stop) { va = sa; vb = sb; }
        if (lane == stop && inc_j >= 0 && g + inc_j >= 0) {
            __threadfence();
            va += __ldcg(&s.inc_a[g + inc_j]);
            vb = Policy::op(vb, __ldcg(&s.inc_b[g + inc_j]));
        }
        pa += warp_sum(va);
        pb = Policy::op(pb, Policy::reduce(vb));
        if (inc_mask) break;
        g0 -= 256;
    }
    if (failed && lane == 0) atomicExch(err, kErrLookback);
    if (lane == 0) {
        __stcg(&s.inc_a[tile], pa + agg_a);
        __stcg(&s.inc_b[tile], Policy::op(pb, self_b));
        __threadfence();
        st_volatile32(&s.st[tile], kSt32Inc | packed);
    }
    *ex_a = pa;
    *ex_b = pb;
}

// The wide look-back in two halves, so a tile's aggregate can be published
// well before its prefix is needed (software-pipelined placement).
template <typename Policy = SumPolicy>
__device__ __forceinline__ void lookback_publish(TileStatus32 s, long long tile, uint32_t agg_a, uint32_t agg_b) {
    if (lane_id() != 0) return;
    const uint32_t packed = (agg_b << 23) | (agg_a & 0x7FFFFFu);
    if (tile == 0) {
        __stcg(&s.inc_a[0], (unsigned long long)agg_a);
        __stcg(&s.inc_b[0], Policy::contrib(agg_b, 0));
        __threadfence();
        st_volatile32(&s.st[0], kSt32Inc | packed);
    } else {
        st_volatile32(&s.st[tile], kSt32Agg | packed);
    }
}

// Whole warp; the tile's aggregate must already be published.
template <typename Policy = SumPolicy>
__device__ __forceinline__ void lookback_resolve(TileStatus32 s, long long tile, uint32_t agg_a, uint32_t agg_b,
                                                 unsigned long long* ex_a, unsigned long long* ex_b, int* err,
                                                 unsigned limit = kSpinLimit) {
    const unsigned lane = lane_id();
    if (tile == 0) {
        *ex_a = 0;
        *ex_b = 0;
        return;
    }
    const uint32_t packed = (agg_b << 23) | (agg_a & 0x7FFFFFu);
    const unsigned long long self_b = Policy::contrib(agg_b, tile);
    unsigned long long pa = 0, pb = 0;
    long long g0 = ((tile - 1) >> 3) << 3;
    unsigned spins = 0;
    bool failed = false;
    while (true) {
        const long long g = g0 - 8 * (long long)lane;
        uint32_t w[8];
        if (g >= 0) {
            uint4 a = ld_volatile_v4(s.st + g), b = ld_volatile_v4(s.st + g + 4);
            w[0] = a.x; w[1] = a.y; w[2] = a.z; w[3] = a.w; w[4] = b.x; w[5] = b.y; w[6] = b.z; w[7] = b.w;
        } else {
#pragma unroll
            for (int j = 0; j < 8; j++) w[j] = kSt32Inc;
        }
        int inc_j = -1;
        bool ready = true;
        uint32_t sa = 0;
        unsigned long long sb = 0;
#pragma unroll
        for (int j = 7; j >= 0; j--) {
            const long long u = g + j;
            const bool pred = u < tile;
            const uint32_t f = w[j] & 0xC0000000u;
            if (pred && inc_j < 0) {
                if (f == kSt32Inc) inc_j = j;
                else {
                    ready = ready && f != 0;
                    sa += w[j] & 0x7FFFFFu;
                    sb = Policy::op(sb, Policy::contrib((w[j] >> 23) & 0x7Fu, u));
                }
            }
        }
        const unsigned inc_mask = __ballot_sync(0xffffffffu, inc_j >= 0);
        const unsigned stop = inc_mask ? (unsigned)__ffs(inc_mask) - 1 : 31u;
        const unsigned window = stop == 31u ? 0xffffffffu : ((1u << (stop + 1)) - 1);
        if (__ballot_sync(0xffffffffu, !ready) & window) {
            if (++spins > limit) { failed = true; break; }
            __nanosleep(spins < 64 ? 32 : 256);
            continue;
        }
        unsigned long long va = 0, vb = 0;
        if (lane <= stop) { va = sa; vb = sb; }
        if (lane == stop && inc_j >= 0 && g + inc_j >= 0) {
            __threadfence();
            va += __ldcg(&s.inc_a[g + inc_j]);
            vb = Policy::op(vb, __ldcg(&s.inc_b[g + inc_j]));
        }
        pa += warp_sum(va);
        pb = Policy::op(pb, Policy::reduce(vb));
        if (inc_mask) break;
        g0 -= 256;
    }
    if (failed && lane == 0) atomicExch(err, kErrLookback);
    if (lane == 0) {
        __stcg(&s.inc_a[tile], pa + agg_a);
        __stcg(&s.inc_b[tile], Policy::op(pb, self_b));
        __threadfence();
        st_volatile32(&s.st[tile], kSt32Inc | packed);
    }
    *ex_a = pa;
    *ex_b = pb;
}

// ------------------------------------------------------------------ inline-prefix look-back
//
// One 64-bit status word per tile: [63:62] flag (0 empty, 1 aggregate,
// 2 inclusive), [61:0] the tile's byte count (aggregate) or the inclusive
// prefix itself.  Resolving a tile is then one memory round trip per window
// of 128 predecessors (4 words per lane), with no second load for the prefix.
constexpr unsigned long long kS64Agg = 1ull << 62, kS64Inc = 2ull << 62, kS64Val = (1ull << 62) - 1;

// Status words are read and written with relaxed GPU-scope accesses: every
// party is on this GPU, and system scope (what `volatile` means) costs far
// more on a coherent CPU-GPU node.
__device__ __forceinline__ void st_volatile64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void ld_volatile_v2x2(const unsigned long long* p, unsigned long long (&w)[4]) {
    unsigned long long a, b, c, d;
    asm volatile("ld.relaxed.gpu.global.v2.u64 {%0,%1}, [%2];" : "=l"(a), "=l"(b) : "l"(p) : "memory");
    asm volatile("ld.relaxed.gpu.global.v2.u64 {%0,%1}, [%2];" : "=l"(c), "=l"(d) : "l"(p + 2) : "memory");
    w[0] = a; w[1] = b; w[2] = c; w[3] = d;
}

// Lane 0 publishes the tile's aggregate (tile 0 publishes its inclusive value).
__device__ __forceinline__ void prefix_publish(unsigned long long* st, long long tile, unsigned long long agg) {
    if (lane_id() != 0) return;
    st_volatile64(&st[tile], (tile == 0 ? kS64Inc : kS64Agg) | (agg & kS64Val));
}

// Whole warp: exclusive prefix of `tile` (aggregate already published), then
// publish its inclusive value.  `st` holds ntiles + 4 zeroed words.
__device__ __forceinline__ unsigned long long prefix_resolve(unsigned long long* st, long long tile,
                                                            unsigned long long agg, int* err,
                                                            unsigned limit = kSpinLimit) {
    if (tile == 0) return 0;
    const unsigned lane = lane_id();
    unsigned long long pa = 0;
    long long g0 = ((tile - 1) >> 2) << 2;
    unsigned spins = 0;
    bool failed = false;
    while (true) {
        const long long g = g0 - 4 * (long long)lane;
        unsigned long long w[4];
        if (g >= 0) ld_volatile_v2x2(st + g, w);
        else { w[0] = w[1] = w[2] = w[3] = kS64Inc; }
        int inc_j = -1;
        bool ready = true;
        unsigned long long sa = 0;
#pragma unroll
        for (int j = 3; j >= 0; j--) {
            const unsigned long long f = w[j] & ~kS64Val;
            if (g + j < tile && inc_j < 0) {
                if (f == kS64Inc) { inc_j = j; sa += w[j] & kS64Val; }
                else { ready = ready && f != 0; sa += w[j] & kS64Val; }
            }
        }
        const unsigned inc_mask = __ballot_sync(0xffffffffu, inc_j >= 0);
        const unsigned stop = inc_mask ? (unsigned)__ffs(inc_mask) - 1 : 31u;
        const unsigned window = stop == 31u ? 0xffffffffu : ((1u << (stop + 1)) - 1);
        if (__ballot_sync(0xffffffffu, !ready) & window) {
            if (++spins > limit) { failed = true; break; }
            __nanosleep(spins < 64 ? 32 : 256);
            continue;
        }
        pa += warp_sum(lane <= stop ? sa : 0ull);
        if (inc_mask) break;
        g0 -= 128;
    }
    if (failed && lane == 0) atomicExch(err, kErrLookback);
    if (lane == 0) st_volatile64(&st[tile], kS64Inc | ((pa + agg) & kS64Val));
    return pa;
}

// The look-back from a window of status words that a TMA bulk copy has put
// in shared memory: win[i] holds the word of tile lo + i, for every tile in
// [lo, tile).  Lane l reads the words of tiles tile-1-l-32k (k = 0..15, rows
// of 32 consecutive tiles, conflict-free) all at once; the nearest inclusive
// prefix is the lowest (row, lane) holding one, found with two warp
// reductions, so the walk is a handful of independent instructions rather
// than a chain of dependent rows.  A window that holds no inclusive prefix,
// or an empty word before it, falls back to the global look-back (which then
// waits); either way the tile's inclusive value is published and its
// exclusive prefix returned.
constexpr int kLbWin = 512;   // status words per window (4 KiB)
__device__ __forceinline__ unsigned long long prefix_resolve_win(unsigned long long* st, long long tile,
                                                                unsigned long long agg, int* err,
                                                                const unsigned long long* win, long long lo) {
    if (tile == 0) return 0;
    constexpr int R = kLbWin / 32;
    const unsigned lane = lane_id();
    unsigned long long w[R];
    unsigned first = R;   // this lane's first row holding an inclusive word
#pragma unroll
    for (int k = 0; k < R; k++) {
        const long long j = tile - 1 - 32 * (long long)k - (long long)lane;
        w[k] = j >= lo ? win[j - lo] : 0ull;   // outside the window reads as empty
        if (first == R && (w[k] & ~kS64Val) == kS64Inc) first = k;
    }
    const unsigned K = __reduce_min_sync(0xffffffffu, first);
    bool ok = K < R;
    unsigned long long sa = 0;
    if (ok) {
        const unsigned stop = __ffs(__ballot_sync(0xffffffffu, first == K)) - 1;
        bool ready = true;
#pragma unroll
        for (int k = 0; k < R; k++) {
            const bool take = (unsigned)k < K || ((unsigned)k == K && lane <= stop);
            if (take) {
                ready = ready && (w[k] & ~kS64Val) != 0;
                sa += w[k] & kS64Val;
            }
        }
        ok = __all_sync(0xffffffffu, ready);
    }
    if (!ok) return prefix_resolve(st, tile, agg, err);
    const unsigned long long pa = warp_sum(sa);
    if (lane == 0) st_volatile64(&st[tile], kS64Inc | ((pa + agg) & kS64Val));
    return pa;
}

// Copy n bytes from a 16-aligned staging buffer (data at offset 0) to global
// dst of any alignment with the whole CTA: 16-byte aligned stores, the
// staging words realigned with funnel shifts; byte copies at the ragged ends.
__device__ __forceinline__ void cta_copy_realign(const uint8_t* stg, uint32_t n, uint8_t* dst) {
    if (n == 0) return;
    const uint32_t sh = (uint32_t)((uintptr_t)dst & 15);
    uint8_t* gbase = dst - sh;
    const uint32_t end = sh + n, nch = (end + 15) >> 4;
    const uint32_t* sw = (const uint32_t*)stg;
    const uint32_t rs = ((16u - sh) & 3u) * 8u;   // byte phase of staging vs. destination words
    for (uint32_t c = threadIdx.x; c < nch; c += blockDim.x) {
        const uint32_t lo = c << 4;
        if (lo >= sh && lo + 16 <= end) {
            const uint32_t so = lo - sh, w = so >> 2;
            const uint32_t a0 = sw[w], a1 = sw[w + 1], a2 = sw[w + 2], a3 = sw[w + 3], a4 = sw[w + 4];
            *(uint4*)(gbase + lo) = make_uint4(__funnelshift_r(a0, a1, rs), __funnelshift_r(a1, a2, rs),
                                               __funnelshift_r(a2, a3, rs), __funnelshift_r(a3, a4, rs));
        }
    }
    if (threadIdx.x < 32) {
        const uint32_t last = nch - 1;
        const uint32_t c = threadIdx.x < 16 ? 0 : last;
        const bool part = threadIdx.x < 16 ? (sh > 0 || end < 16) : (last > 0 && (end & 15) != 0);
        const uint32_t gb = (c << 4) + (threadIdx.x & 15);
        if (part && gb >= sh && gb < end) gbase[gb] = stg[gb - sh];
    }
}

// 16-byte asynchronous global -> shared copies (cp.async, the LSU path: they
// do not queue behind the TMA unit's bulk copies), L2 only.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// wait until at most N of this thread's committed groups are still in flight
template <int N>
__device__ __forceinline__ void cp_async_wait_group() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }
__device__ __forceinline__ void st_relaxed16(uint16_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u16 [%0], %1;" ::"l"(p), "h"((unsigned short)v) : "memory");
}
}  // namespace szxg
