// Global value range pass: computeValueRange_float / _double
// (szx/src/szx_float.cc:478-499, szx/src/szx_double.cc:1137-1158) and the
// bound conversion of SZx_fast_compress_args (szx/src/szx.cc:249-253,
// :277-287, :304-308, :332-340), done in one launch: grid-stride partials,
// then the last CTA to finish reduces them and derives the codec parameters.
//
// The reference's sequential scan (`if (min > v) min = v; else if (max < v)
// max = v;` starting from x[0]) keeps the FIRST element that reaches the
// extreme and ignores NaNs unless x[0] itself is NaN.  A parallel min/max
// reproduces that exactly once two cases are patched: a NaN x[0] pins both
// extremes to it, and a zero extreme takes the sign of the first zero.
#include "common.cuh"
#include "kernels.h"

namespace szxg {

struct RangePartial {
    unsigned long long lo, hi;   // float: value bits; double: order keys
    unsigned long long zidx;     // first zero element
};

constexpr unsigned long long kNoIdx = ~0ull;
constexpr int kRangeThreads = 256;

__device__ __forceinline__ long long dkey(unsigned long long b) {
    // monotone signed key of a non-NaN double pattern
    return (long long)(b ^ ((unsigned long long)((long long)b >> 63) & 0x7FFFFFFFFFFFFFFFull));
}
__device__ __forceinline__ unsigned long long dkey_inv(long long k) {
    unsigned long long u = (unsigned long long)k;
    return u ^ ((unsigned long long)(k >> 63) & 0x7FFFFFFFFFFFFFFFull);
}

template <typename T> struct RangeOps;

template <> struct RangeOps<float> {
    float mn = __builtin_huge_valf(), mx = -__builtin_huge_valf();
    unsigned long long z = kNoIdx;
    __device__ __forceinline__ void add(float v, unsigned long long i) {
        mn = fminf(mn, v);
        mx = fmaxf(mx, v);
        if (v == 0.0f && i < z) z = i;
    }
    __device__ __forceinline__ void merge(const RangeOps& o) {
        mn = fminf(mn, o.mn);
        mx = fmaxf(mx, o.mx);
        z = o.z < z ? o.z : z;
    }
    __device__ __forceinline__ RangePartial pack() const {
        return {(unsigned long long)__float_as_uint(mn), (unsigned long long)__float_as_uint(mx), z};
    }
    __device__ __forceinline__ void unpack(const RangePartial& p) {
        mn = __uint_as_float((uint32_t)p.lo);
        mx = __uint_as_float((uint32_t)p.hi);
        z = p.zidx;
    }
    __device__ __forceinline__ void shfl_merge(int d) {
        RangeOps o;
        o.mn = __shfl_xor_sync(0xffffffffu, mn, d);
        o.mx = __shfl_xor_sync(0xffffffffu, mx, d);
        o.z = __shfl_xor_sync(0xffffffffu, z, d);
        merge(o);
    }
};

template <> struct RangeOps<double> {
    long long kmn = 0x7FFFFFFFFFFFFFFFll, kmx = (long long)0x8000000000000000ull;
    unsigned long long z = kNoIdx;
    __device__ __forceinline__ void add(double v, unsigned long long i) {
        unsigned long long b = (unsigned long long)__double_as_longlong(v);
        unsigned long long mag = b & 0x7FFFFFFFFFFFFFFFull;
        if (mag <= 0x7FF0000000000000ull) {          // not NaN
            long long k = dkey(b);
            kmn = k < kmn ? k : kmn;
            kmx = k > kmx ? k : kmx;
            if (mag == 0 && i < z) z = i;
        }
    }
    __device__ __forceinline__ void merge(const RangeOps& o) {
        kmn = o.kmn < kmn ? o.kmn : kmn;
        kmx = o.kmx > kmx ? o.kmx : kmx;
        z = o.z < z ? o.z : z;
    }
    __device__ __forceinline__ RangePartial pack() const {
        return {(unsigned long long)kmn, (unsigned long long)kmx, z};
    }
    __device__ __forceinline__ void unpack(const RangePartial& p) {
        kmn = (long long)p.lo;
        kmx = (long long)p.hi;
        z = p.zidx;
    }
    __device__ __forceinline__ void shfl_merge(int d) {
        RangeOps o;
        o.kmn = __shfl_xor_sync(0xffffffffu, kmn, d);
        o.kmx = __shfl_xor_sync(0xffffffffu, kmx, d);
        o.z = __shfl_xor_sync(0xffffffffu, z, d);
        merge(o);
    }
};

template <typename T> struct Vec;
template <> struct Vec<float> { using V = float4; static constexpr int N = 4; };
template <> struct Vec<double> { using V = double2; static constexpr int N = 2; };

template <typename T>
__device__ __forceinline__ void add_vec(RangeOps<T>& acc, const typename Vec<T>::V& v, unsigned long long i);
template <> __device__ __forceinline__ void add_vec<float>(RangeOps<float>& a, const float4& v, unsigned long long i) {
    a.add(v.x, i); a.add(v.y, i + 1); a.add(v.z, i + 2); a.add(v.w, i + 3);
}
template <> __device__ __forceinline__ void add_vec<double>(RangeOps<double>& a, const double2& v, unsigned long long i) {
    a.add(v.x, i); a.add(v.y, i + 1);
}

// STREAM: the field is larger than L2, so its lines are loaded evict-first
// (the encoder re-reads it from HBM either way); smaller fields keep the
// default policy and stay in L2 for the encoder that follows.
template <typename T, bool STREAM>
__global__ void __launch_bounds__(kRangeThreads) k_range(const T* __restrict__ x, unsigned long long n, int err_mode,
                                                          float abs_eb, float rel, RangePartial* partials,
                                                          unsigned long long* counter, CodecParams* out) {
    using V = typename Vec<T>::V;
    constexpr int VN = Vec<T>::N;
    RangeOps<T> acc;
    const unsigned long long tid = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned long long nthr = (unsigned long long)gridDim.x * blockDim.x;
    const bool aligned = ((uintptr_t)x % 16) == 0;
    if (aligned) {
        const unsigned long long nv = n / VN;
        const V* xv = reinterpret_cast<const V*>(x);
        unsigned long long i = tid;
        for (; i + 7 * nthr < nv; i += 8 * nthr) {   // 8 independent 16-byte loads in flight
            V a[8];
#pragma unroll
            for (int u = 0; u < 8; u++) a[u] = STREAM ? __ldcs(xv + i + u * nthr) : xv[i + u * nthr];
#pragma unroll
            for (int u = 0; u < 8; u++) add_vec<T>(acc, a[u], (i + u * nthr) * VN);
        }
        if (i < nv) {   // the last partial round: its loads in flight together too
            V a[8];
#pragma unroll
            for (int u = 0; u < 8; u++)
                if (i + u * nthr < nv) a[u] = STREAM ? __ldcs(xv + i + u * nthr) : xv[i + u * nthr];
#pragma unroll
            for (int u = 0; u < 8; u++)
                if (i + u * nthr < nv) add_vec<T>(acc, a[u], (i + u * nthr) * VN);
        }
        for (unsigned long long j = nv * VN + tid; j < n; j += nthr) acc.add(x[j], j);
    } else {
        for (unsigned long long j = tid; j < n; j += nthr) acc.add(x[j], j);
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) acc.shfl_merge(d);
    __shared__ RangePartial sp[kRangeThreads / 32];
    __shared__ bool last;
    if ((threadIdx.x & 31) == 0) sp[threadIdx.x >> 5] = acc.pack();
    __syncthreads();
    if (threadIdx.x == 0) {
        RangeOps<T> r;
        for (int w = 0; w < kRangeThreads / 32; w++) {
            RangeOps<T> o;
            o.unpack(sp[w]);
            r.merge(o);
        }
        partials[blockIdx.x] = r.pack();
        __threadfence();
        unsigned long long ticket = atomicAdd(counter, 1ull);
        last = (ticket == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    // ---- last CTA: reduce all partials and derive parameters
    __threadfence();
    RangeOps<T> r;
    for (unsigned i = threadIdx.x; i < gridDim.x; i += blockDim.x) {
        RangeOps<T> o;
        RangePartial p;
        p.lo = __ldcg(&partials[i].lo);
        p.hi = __ldcg(&partials[i].hi);
        p.zidx = __ldcg(&partials[i].zidx);
        o.unpack(p);
        r.merge(o);
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) r.shfl_merge(d);
    if ((threadIdx.x & 31) == 0) sp[threadIdx.x >> 5] = r.pack();
    __syncthreads();
    if (threadIdx.x != 0) return;
    RangeOps<T> f;
    for (int w = 0; w < kRangeThreads / 32; w++) {
        RangeOps<T> o;
        o.unpack(sp[w]);
        f.merge(o);
    }
    *counter = 0;   // ready for the next launch
    CodecParams p;
    p.has_range = 1;
    p.pad = 0;
    if constexpr (sizeof(T) == 4) {
        float mn = f.mn, mx = f.mx;
        float x0 = x[0];
        if (isnan(x0)) { mn = x0; mx = x0; }
        else if (f.z != kNoIdx) {
            if (mn == 0.0f) mn = x[f.z];
            if (mx == 0.0f) mx = x[f.z];
        }
        float range = xsub(mx, mn);
        p.range_f = range;
        p.range_d = xf2d(range);
        p.radius = xdiv(range, 2.0f);
        p.median = xadd(mn, p.radius);
        p.eb = err_mode == 1 ? xmul(range, rel) : abs_eb;
    } else {
        double x0 = x[0];
        double mn, mx;
        if (isnan(x0)) { mn = x0; mx = x0; }
        else {
            mn = __longlong_as_double((long long)dkey_inv(f.kmn));
            mx = __longlong_as_double((long long)dkey_inv(f.kmx));
            if (f.z != kNoIdx) {
                if (mn == 0.0) mn = x[f.z];
                if (mx == 0.0) mx = x[f.z];
            }
        }
        double range = xsub(mx, mn);
        p.range_d = range;
        p.range_f = xd2f(range);
        p.radius = xd2f(xdiv(range, 2.0));
        p.median = xd2f(xadd(mn, xf2d(p.radius)));
        p.eb = err_mode == 1 ? xd2f(xmul(range, xf2d(rel))) : abs_eb;
    }
    *out = p;
}

// Fields above this size do not fit beside the encoder's working set in L2.
constexpr size_t kStreamBytes = size_t(96) << 20;

cudaError_t launch_range(int dtype, const void* x, size_t n, int err_mode, float abs_eb, float rel,
                         const Workspace& ws, cudaStream_t s, bool cleared) {
    if (n == 0) return cudaErrorInvalidValue;
    size_t es = dtype == 0 ? 4 : 8;
    size_t per_cta = (size_t)kRangeThreads * (64 / es) * 4;  // ~64 B per thread per round, 4 rounds
    size_t want = (n + per_cta - 1) / per_cta;
    // one wave of resident CTAs: a second, partial wave would leave most SMs idle at the end
    static int per_sm[2][2][64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    const bool stream = n * es > kStreamBytes;
    int& occ = per_sm[dtype == 0 ? 0 : 1][stream ? 1 : 0][dev];
    if (!occ) {
        cudaError_t eo;
        if (dtype == 0)
            eo = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &occ, stream ? k_range<float, true> : k_range<float, false>, kRangeThreads, 0);
        else
            eo = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &occ, stream ? k_range<double, true> : k_range<double, false>, kRangeThreads, 0);
        if (eo != cudaSuccess) return eo;
        if (occ < 1) occ = 1;
    }
    size_t cap = (size_t)sm_count() * occ;
    int grid = (int)(want < cap ? (want ? want : 1) : cap);
    if (grid > 4096) grid = 4096;
    RangePartial* parts = reinterpret_cast<RangePartial*>(ws.partials);
    cudaError_t e = cleared ? cudaSuccess : cudaMemsetAsync(&ws.counters[3], 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    TraceScope tr("range", s);
    if (dtype == 0)
        (stream ? k_range<float, true> : k_range<float, false>)<<<grid, kRangeThreads, 0, s>>>(
            (const float*)x, n, err_mode, abs_eb, rel, parts, &ws.counters[3], ws.params);
    else
        (stream ? k_range<double, true> : k_range<double, false>)<<<grid, kRangeThreads, 0, s>>>(
            (const double*)x, n, err_mode, abs_eb, rel, parts, &ws.counters[3], ws.params);
    return cudaGetLastError();
}

}  // namespace szxg
