// Fixed-rate (FXR) error-bound search of the reference, with every pass over
// the data on the GPU.
//
// The reference picks the absolute bound for a target compression ratio from
// a sample of the field: every 10th block of 128 values, its min/max, radius
// and median (computeRadiusBuffer_float, szx/src/szx_float.cc:254-312), a
// ratio model evaluated on that sample for a candidate bound
// (estimateCRbasedonErrorBound_buffered_float, :501-584: constant blocks,
// required bytes and leading bytes per value), and a bracket-then-bisect
// search over candidate bounds (estimateErrorBoundbasedonCR_buffered_float,
// :684-832).  The chosen bound then drives an ordinary fastMode-2 compress
// (:921-949).  Double data follows szx/src/szx_double.cc:437-940.
//
// Here the sample statistics and each evaluation are kernels (one segment of
// G lanes per sampled block, the codec's own block machinery); the search
// itself is the reference's sequential decision procedure, run on the host
// with the integer sums each evaluation returns and the reference's exact
// float/double expression for the ratio.
#include <math.h>
#include <string.h>

#include "../../include/szx_gb300.h"
#include "kernels.h"
#include "segment.cuh"

namespace szxg {

namespace {

constexpr int kFxThreads = 256;

// Workspace carve for ns sampled blocks.
struct FxWs {
    float* rads;             // radius (float) per sampled block
    float* meds;             // median (float) per sampled block
    double* rads_d;          // radius in double (double data)
    void* bmin;              // block min / max (data type)
    void* bmax;
    unsigned long long* acc; // [0] constant blocks, [1] required bytes, [2] leading bytes
    float* range;
};

size_t fx_a256(size_t x) { return (x + 255) & ~(size_t)255; }

size_t fx_bytes(size_t ns) {
    return fx_a256(4 * ns) * 2 + fx_a256(8 * ns) * 3 + 256;
}

FxWs fx_carve(void* base, size_t ns) {
    uint8_t* b = (uint8_t*)base;
    FxWs w;
    w.rads = (float*)b; b += fx_a256(4 * ns);
    w.meds = (float*)b; b += fx_a256(4 * ns);
    w.rads_d = (double*)b; b += fx_a256(8 * ns);
    w.bmin = b; b += fx_a256(8 * ns);
    w.bmax = b; b += fx_a256(8 * ns);
    w.acc = (unsigned long long*)b;
    w.range = (float*)(b + 64);
    return w;
}

int lanes_for(int dtype, int bs) {
    const int per = dtype == 0 ? 16 : 8;
    const int need = (bs + per - 1) / per;
    return need <= 1 ? 1 : need <= 2 ? 2 : need <= 4 ? 4 : need <= 8 ? 8 : need <= 16 ? 16 : 32;
}

}  // namespace

// Sampled-block statistics: block i of the sample holds bs values starting
// at x + i*stride.  min/max keep the reference's sequential semantics
// (first value reaching an extreme; NaN skipped unless first); radius and
// median as computeRadiusBuffer_float / _double compute them.
template <typename T, int G>
__global__ void __launch_bounds__(kFxThreads) k_fxr_sample(const T* x, unsigned long long ns,
                                                           unsigned long long stride, int bs, float* rads,
                                                           float* meds, double* rads_d, T* bmin, T* bmax) {
    constexpr int E = EncCfg<T>::E;
    const int lane = threadIdx.x & 31, seg = lane / G, sl = lane & (G - 1);
    const unsigned long long gw = ((unsigned long long)blockIdx.x * kFxThreads + threadIdx.x) >> 5;
    const unsigned long long i = gw * (32 / G) + seg;
    const bool in = i < ns;
    const int len = in ? bs : 0;
    const T* xs = x + (in ? i * stride : 0);
    const bool vec = ((uintptr_t)x & 15) == 0 && ((stride * sizeof(T)) & 15) == 0;
    T v[E];
    load_chunks<T, G>(xs, len, vec, v);
    T mn, mx;
    bool special;
    if (__all_sync(0xffffffffu, len == G * E)) seg_minmax<T, G, true>(v, len, mn, mx, special);
    else seg_minmax<T, G, false>(v, len, mn, mx, special);
    (void)special;
    if (in && sl == 0) {
        if constexpr (sizeof(T) == 4) {
            const float r = xhalf(xsub(mx, mn));
            rads[i] = r;
            meds[i] = xadd(mn, r);
        } else {
            const double r = xhalf(xsub(mx, mn));
            rads[i] = xd2f(r);
            meds[i] = xd2f(xadd(mn, r));
            rads_d[i] = r;
        }
        bmin[i] = mn;
        bmax[i] = mx;
    }
}

// Sampled value range: the reference folds the block extremes in block order
// starting from data[0] with `if (g < mx) g = mx` (and the mirror for min):
// the result is the first block extreme of the largest value, unless data[0]
// is NaN.  One CTA; ties go to the smaller index.
template <typename T>
__global__ void __launch_bounds__(1024) k_fxr_range(const T* x, const T* bmin, const T* bmax,
                                                    unsigned long long ns, float* range) {
    __shared__ T s_v[2][32];
    __shared__ long long s_i[2][32];
    T best[2];
    long long bi[2] = {-1, -1};
    best[0] = 0;
    best[1] = 0;
    for (unsigned long long i = threadIdx.x; i < ns; i += blockDim.x) {
        const T hi = bmax[i], lo = bmin[i];
        if (hi == hi && (bi[0] < 0 || hi > best[0])) { best[0] = hi; bi[0] = (long long)i; }
        if (lo == lo && (bi[1] < 0 || lo < best[1])) { best[1] = lo; bi[1] = (long long)i; }
    }
    auto better = [](int which, T a, long long ai, T b, long long bidx) {
        // is (b, bidx) the earlier extreme of (a, ai) and (b, bidx)?
        if (bidx < 0) return false;
        if (ai < 0) return true;
        if (which == 0 ? b > a : b < a) return true;
        return b == a && bidx < ai;
    };
    for (int w = 0; w < 2; w++) {
        for (int d = 16; d > 0; d >>= 1) {
            const T ov = __shfl_down_sync(0xffffffffu, best[w], d);
            const long long oi = __shfl_down_sync(0xffffffffu, bi[w], d);
            if (better(w, best[w], bi[w], ov, oi)) { best[w] = ov; bi[w] = oi; }
        }
        if ((threadIdx.x & 31) == 0) { s_v[w][threadIdx.x >> 5] = best[w]; s_i[w][threadIdx.x >> 5] = bi[w]; }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        T g[2];
        for (int w = 0; w < 2; w++) {
            T b = s_v[w][0];
            long long ib = s_i[w][0];
            for (int k = 1; k < nw; k++)
                if (better(w, b, ib, s_v[w][k], s_i[w][k])) { b = s_v[w][k]; ib = s_i[w][k]; }
            const T x0 = x[0];
            g[w] = x0;
            if (ib >= 0 && (w == 0 ? x0 < b : x0 > b)) g[w] = b;
        }
        if constexpr (sizeof(T) == 4) *range = xsub(g[0], g[1]);
        else *range = xd2f(xsub(g[0], g[1]));
    }
}

// One evaluation of the ratio model at bound eb over the sampled blocks
// (estimateCRbasedonErrorBound_buffered_float / _double): constant blocks,
// required bytes per coded block, and min(lead, required bytes) summed over
// the coded blocks' values.  The subtraction uses the median the reference
// hands to the value loop: zeroed when the required length is clamped.
template <typename T, int G>
__global__ void __launch_bounds__(kFxThreads) k_fxr_eval(const T* x, unsigned long long ns, unsigned long long stride,
                                                         int bs, const float* rads, const float* meds,
                                                         const double* rads_d, float eb, unsigned long long* acc) {
    using EL = Elem<T>;
    using U = typename EL::U;
    constexpr int E = EncCfg<T>::E;
    constexpr int NC = E / 4;
    const int lane = threadIdx.x & 31, seg = lane / G, sl = lane & (G - 1);
    const unsigned long long gw = ((unsigned long long)blockIdx.x * kFxThreads + threadIdx.x) >> 5;
    const unsigned long long i = gw * (32 / G) + seg;
    const bool in = i < ns;
    const float radius = in ? rads[i] : 0.0f;
    const float median = in ? meds[i] : 0.0f;
    const bool cst = in && (rads_d ? rads_d[i] <= (double)eb : radius <= eb);
    const bool coded = in && !cst;
    const int len = coded ? bs : 0;
    bool zm;
    const int reqLength = req_length<T>(eb, radius, &zm);
    int R, s;
    split_reqlen(reqLength, &R, &s);
    T med;
    if constexpr (sizeof(T) == 4) med = zm ? 0.0f : median;
    else med = zm ? 0.0 : xf2d(median);
    const T* xs = x + (coded ? i * stride : 0);
    const bool vec = ((uintptr_t)x & 15) == 0 && ((stride * sizeof(T)) & 15) == 0;
    T v[E];
    load_chunks<T, G>(xs, len, vec, v);
    U cur[E];
#pragma unroll
    for (int e = 0; e < E; e++) cur[e] = EL::bits(xsub(v[e], med)) >> s;
    uint32_t ldb[NC];
    seg_lead_bytes<T, G>(cur, ldb);
    const uint32_t R4 = (uint32_t)R * 0x01010101u;
    uint32_t lead = 0;
#pragma unroll
    for (int k = 0; k < NC; k++) {
        // min(lead, R) per value = R - max(R - lead, 0), bytewise
        const uint32_t m = R4 - stored_counts(R, ldb[k]);
        const uint32_t keep = low_bytes_mask(len - 4 * (sl + k * G));
        lead += ((m & keep) * 0x01010101u) >> 24;
    }
    lead = seg_sum<G>(lead);
    unsigned long long c0 = (sl == 0 && cst) ? 1ull : 0ull;
    unsigned long long c1 = (sl == 0 && coded) ? (unsigned long long)R : 0ull;
    unsigned long long c2 = (sl == 0 && coded) ? (unsigned long long)lead : 0ull;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        c0 += __shfl_xor_sync(0xffffffffu, c0, d);
        c1 += __shfl_xor_sync(0xffffffffu, c1, d);
        c2 += __shfl_xor_sync(0xffffffffu, c2, d);
    }
    if (lane == 0 && (c0 | c1 | c2)) {
        atomicAdd(&acc[0], c0);
        atomicAdd(&acc[1], c1);
        atomicAdd(&acc[2], c2);
    }
}

// Copies of the sampled blocks, contiguous (the `buffer` computeRadiusBuffer hands back).
template <typename T>
__global__ void k_fxr_gather(const T* x, unsigned long long ns, unsigned long long stride, int bs, T* out) {
    const unsigned long long total = ns * (unsigned long long)bs;
    for (unsigned long long j = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; j < total;
         j += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long b = j / (unsigned long long)bs, e = j - b * bs;
        out[j] = x[b * stride + e];
    }
}

// ------------------------------------------------------------------ host side

namespace {

// The reference's ratio model from the sample sums, with its exact mix of
// float and double arithmetic (szx/src/szx_float.cc:575-581,
// szx/src/szx_double.cc:571-577).  nden: the sampled-block count the model
// divides by.
// A division as x86-64 SSE performs it: an invalid one (0/0) gives the
// negative "indefinite" NaN, where other hosts give a positive default NaN.
double x86_div(double a, double b) {
    const double r = a / b;
    if (r != r && a == a && b == b) {
        const unsigned long long indefinite = 0xFFF8000000000000ull;
        double v;
        memcpy(&v, &indefinite, sizeof v);
        return v;
    }
    return r;
}

float fx_model(int dtype, int bs, size_t n, size_t nden, size_t ncst, size_t sumReq, size_t sumLead) {
    float metadata = 13.0 * bs / n;
    float block_cost = dtype == 0 ? 33.0 / 8 : 65.0 / 8;
    // all sampled blocks constant: 0/0 in the reference
    float avgReqNbBytes = x86_div(1.0 * sumReq, (double)(nden - ncst));
    float avg_actual_lead = x86_div(1.0 * sumLead, (double)(nden - ncst));
    float p_lambda = x86_div(1.0 * ncst, (double)nden);
    float cr;
    if (dtype == 0)
        cr = 4 * bs / (metadata + block_cost + (1 + (0.25 + avgReqNbBytes) * bs - avg_actual_lead) * (1 - p_lambda));
    else
        cr = 8 * bs / (metadata + block_cost + (1 + (0.25 + avgReqNbBytes) * bs - avg_actual_lead) * (1 - p_lambda));
    return cr;
}

// One sampled view of a device array: ns blocks of bs values, block i at x + i*stride.
struct FxSample {
    int dtype, bs, G;
    size_t n;          // element count the model's metadata term uses
    size_t ns;         // sampled blocks evaluated
    size_t nden;       // sampled-block count in the model's averages
    size_t stride;     // elements between sampled blocks
    const void* x;
    FxWs w;
    bool double_radius;   // constant test on the double radius (unbuffered double model)
    cudaStream_t s;

    cudaError_t stats(float* range_out) {
        if (ns) {
            const size_t warps = (ns + (32 / G) - 1) / (32 / G);
            const unsigned grid = (unsigned)((warps * 32 + kFxThreads - 1) / kFxThreads);
            TraceScope tr("fxr_sample", s);
#define FX_SAMPLE(TT, GG)                                                                                         \
    k_fxr_sample<TT, GG><<<grid, kFxThreads, 0, s>>>((const TT*)x, ns, stride, bs, w.rads, w.meds, w.rads_d,     \
                                                     (TT*)w.bmin, (TT*)w.bmax)
            if (dtype == 0) {
                switch (G) {
                    case 1: FX_SAMPLE(float, 1); break;
                    case 2: FX_SAMPLE(float, 2); break;
                    case 4: FX_SAMPLE(float, 4); break;
                    case 8: FX_SAMPLE(float, 8); break;
                    default: FX_SAMPLE(float, 16); break;
                }
            } else {
                switch (G) {
                    case 1: FX_SAMPLE(double, 1); break;
                    case 2: FX_SAMPLE(double, 2); break;
                    case 4: FX_SAMPLE(double, 4); break;
                    case 8: FX_SAMPLE(double, 8); break;
                    case 16: FX_SAMPLE(double, 16); break;
                    default: FX_SAMPLE(double, 32); break;
                }
            }
#undef FX_SAMPLE
        }
        if (dtype == 0) k_fxr_range<float><<<1, 1024, 0, s>>>((const float*)x, (const float*)w.bmin, (const float*)w.bmax, ns, w.range);
        else k_fxr_range<double><<<1, 1024, 0, s>>>((const double*)x, (const double*)w.bmin, (const double*)w.bmax, ns, w.range);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess && range_out) e = cudaMemcpyAsync(range_out, w.range, sizeof(float), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        return e;
    }

    // ratio estimate at eb; the integer sums in *sr, *sl, *sc
    cudaError_t eval(float eb, float* cr, size_t* sr, size_t* sl, size_t* sc) {
        cudaError_t e = cudaMemsetAsync(w.acc, 0, 3 * sizeof(unsigned long long), s);
        if (e != cudaSuccess) return e;
        if (ns) {
            const size_t warps = (ns + (32 / G) - 1) / (32 / G);
            const unsigned grid = (unsigned)((warps * 32 + kFxThreads - 1) / kFxThreads);
            const double* rd = double_radius ? w.rads_d : nullptr;
            TraceScope tr("fxr_eval", s);
#define FX_EVAL(TT, GG) \
    k_fxr_eval<TT, GG><<<grid, kFxThreads, 0, s>>>((const TT*)x, ns, stride, bs, w.rads, w.meds, rd, eb, w.acc)
            if (dtype == 0) {
                switch (G) {
                    case 1: FX_EVAL(float, 1); break;
                    case 2: FX_EVAL(float, 2); break;
                    case 4: FX_EVAL(float, 4); break;
                    case 8: FX_EVAL(float, 8); break;
                    default: FX_EVAL(float, 16); break;
                }
            } else {
                switch (G) {
                    case 1: FX_EVAL(double, 1); break;
                    case 2: FX_EVAL(double, 2); break;
                    case 4: FX_EVAL(double, 4); break;
                    case 8: FX_EVAL(double, 8); break;
                    case 16: FX_EVAL(double, 16); break;
                    default: FX_EVAL(double, 32); break;
                }
            }
#undef FX_EVAL
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
        }
        unsigned long long h[3] = {0, 0, 0};
        if ((e = cudaMemcpyAsync(h, w.acc, sizeof h, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
        *sc = (size_t)h[0];
        *sr = (size_t)h[1];
        *sl = (size_t)h[2];
        *cr = fx_model(dtype, bs, n, nden, *sc, *sr, *sl);
        return cudaSuccess;
    }
};

}  // namespace

size_t fxr_ws_bytes(int dtype, size_t n, int bs, int rate) {
    (void)dtype;
    if (bs < 1 || rate < 1) return 256;
    const size_t nb = n / (size_t)bs;
    return fx_bytes(nb / (size_t)rate + 4);
}

// estimateErrorBoundbasedonCR_buffered_float / _double, started from 1% of
// the sampled range (szx/src/szx_float.cc:684-832, :921-949).
cudaError_t fxr_bound(int dtype, const void* d_x, size_t n, int bs, float targetCompressionRatio, float tolerance,
                      void* d_ws, size_t wsb, cudaStream_t s, float* eb_out) {
    const int samplingRate = 10;
    if (bs < 1 || n == 0 || wsb < fxr_ws_bytes(dtype, n, bs, samplingRate)) return cudaErrorInvalidValue;
    FxSample S;
    S.dtype = dtype; S.bs = bs; S.G = lanes_for(dtype, bs); S.n = n;
    S.ns = n / ((size_t)bs * samplingRate); S.nden = S.ns; S.stride = (size_t)bs * samplingRate;
    S.x = d_x; S.w = fx_carve(d_ws, S.ns + 2); S.double_radius = false; S.s = s;
    float range = 0;
    cudaError_t e = S.stats(&range);
    if (e != cudaSuccess) return e;
    const int stride = 8, nbIterations = 10;
    float errorBound = range * 1E-2;
    size_t sumReqNbBytes[20] = {0}, sum_actual_leadNumbers[20] = {0};
    float errorBounds[20], ratios[20];
    int k = 0;
    size_t sr = 0, sl = 0, sc = 0;
    float CR = 0;
    if ((e = S.eval(errorBound, &CR, &sr, &sl, &sc)) != cudaSuccess) return e;
    sumReqNbBytes[k] = sr; sum_actual_leadNumbers[k] = sl; errorBounds[k] = errorBound; ratios[k] = CR; k++;
    if (fabs(targetCompressionRatio - CR) < tolerance) { *eb_out = errorBound; return cudaSuccess; }
    float left_error = 0, right_error = 0, result_error = 0;
    int foundFlag = 0;
    float targetTolerance = targetCompressionRatio * tolerance;
    if (targetCompressionRatio < CR) {
        left_error = errorBound / stride;
        right_error = errorBound;
        for (int i = 0; i < nbIterations; i++) {
            if ((e = S.eval(left_error, &CR, &sr, &sl, &sc)) != cudaSuccess) return e;
            sumReqNbBytes[k] = sr; sum_actual_leadNumbers[k] = sl; errorBounds[k] = left_error; ratios[k] = CR; k++;
            if (fabs(CR - targetCompressionRatio) < targetTolerance) { foundFlag = 1; result_error = left_error; break; }
            if (targetCompressionRatio > CR) break;
            right_error = left_error;
            left_error = left_error / stride;
        }
    } else if (targetCompressionRatio > CR) {
        left_error = errorBound;
        right_error = errorBound * stride;
        for (int i = 0; i < nbIterations; i++) {
            if ((e = S.eval(right_error, &CR, &sr, &sl, &sc)) != cudaSuccess) return e;
            sumReqNbBytes[k] = sr; sum_actual_leadNumbers[k] = sl; errorBounds[k] = right_error; ratios[k] = CR; k++;
            if (fabs(targetCompressionRatio - CR) < targetTolerance) { foundFlag = 1; result_error = right_error; break; }
            if (targetCompressionRatio < CR) break;
            left_error = right_error;
            right_error = right_error * stride;
        }
    }
    if (foundFlag == 0) {
        for (int i = 0; i < nbIterations; i++) {
            errorBound = (left_error + right_error) / 2;
            if ((e = S.eval(errorBound, &CR, &sr, &sl, &sc)) != cudaSuccess) return e;
            int appeared = 0;
            for (int j = 0; j < k; j++)
                if (sumReqNbBytes[j] == sr && sum_actual_leadNumbers[j] == sl) { appeared = 1; break; }
            float min_ratio_error = 10000000;
            int index = 0;
            for (int j = 0; j < k; j++) {
                float r = ratios[j];
                float er = fabs(r - targetCompressionRatio);
                if (er < min_ratio_error) { min_ratio_error = er; index = j; }
            }
            if (appeared) { result_error = errorBounds[index]; break; }
            sumReqNbBytes[k] = sr; sum_actual_leadNumbers[k] = sl; errorBounds[k] = errorBound; ratios[k] = CR; k++;
            if (fabs(CR - targetCompressionRatio) < targetTolerance) { foundFlag = 1; result_error = errorBound; break; }
            if (targetCompressionRatio > CR) left_error = errorBound;
            else right_error = errorBound;
        }
    }
    *eb_out = result_error;
    return cudaSuccess;
}

// estimateErrorBoundbasedonCR_float / _double (szx/src/szx_float.cc:834-920,
// szx/src/szx_double.cc:831-917): the unbuffered model samples blocks 0, 10,
// 20, ... below nbEle/bs but averages over (nbEle/bs)/10 of them; the double
// model tests constancy on the double radius.  (The reference's model ends in
// exit(0), szx/src/szx_float.cc:681; this returns the search's result.)
cudaError_t fxr_bound_unbuffered(int dtype, const void* d_x, size_t n, int bs, float targetCompressionRatio,
                                 float tolerance, float initErrorBound, void* d_ws, size_t wsb, cudaStream_t s,
                                 float* eb_out) {
    const int samplingRate = 10;
    if (bs < 1 || n == 0 || wsb < fxr_ws_bytes(dtype, n, bs, samplingRate)) return cudaErrorInvalidValue;
    const size_t nbBlocks = n / (size_t)bs;
    FxSample S;
    S.dtype = dtype; S.bs = bs; S.G = lanes_for(dtype, bs); S.n = n;
    S.ns = (nbBlocks + samplingRate - 1) / samplingRate; S.nden = nbBlocks / samplingRate;
    S.stride = (size_t)bs * samplingRate;
    S.x = d_x; S.w = fx_carve(d_ws, S.ns + 2); S.double_radius = dtype != 0; S.s = s;
    cudaError_t e = S.stats(nullptr);
    if (e != cudaSuccess) return e;
    float errorBound = initErrorBound;
    size_t sr, sl, sc;
    float CR = 0;
    if ((e = S.eval(errorBound, &CR, &sr, &sl, &sc)) != cudaSuccess) return e;
    const int nbIterations = 15;
    if (fabs(targetCompressionRatio - CR) < tolerance) { *eb_out = errorBound; return cudaSuccess; }
    float left_error = 0, right_error = 0, result_error = 0;
    int foundFlag = 0;
    float targetTolerance = targetCompressionRatio * tolerance;
    float preCR = CR;
    if (targetCompressionRatio < CR) {
        left_error = errorBound / 8;
        right_error = errorBound;
        for (int i = 0; i < nbIterations; i++) {
            if ((e = S.eval(left_error, &CR, &sr, &sl, &sc)) != cudaSuccess) return e;
            if (fabs(CR - targetCompressionRatio) < targetTolerance || fabs(CR - preCR) < targetTolerance / 2) {
                foundFlag = 1;
                result_error = left_error;
                break;
            }
            if (targetCompressionRatio > CR) break;
            right_error = left_error;
            left_error = left_error / 8;
            preCR = CR;
        }
    } else if (targetCompressionRatio > CR) {
        left_error = errorBound;
        right_error = errorBound * 8;
        for (int i = 0; i < nbIterations; i++) {
            if ((e = S.eval(right_error, &CR, &sr, &sl, &sc)) != cudaSuccess) return e;
            if (fabs(targetCompressionRatio - CR) < targetTolerance || fabs(CR - preCR) < targetTolerance / 2) {
                foundFlag = 1;
                result_error = right_error;
                break;
            }
            if (targetCompressionRatio < CR) break;
            left_error = right_error;
            right_error = right_error * 8;
        }
        preCR = CR;
    }
    if (foundFlag == 0) {
        for (int i = 0; i < nbIterations; i++) {
            errorBound = (left_error + right_error) / 2;
            if ((e = S.eval(errorBound, &CR, &sr, &sl, &sc)) != cudaSuccess) return e;
            if (fabs(CR - targetCompressionRatio) < targetTolerance || fabs(CR - preCR) < targetTolerance / 2) {
                foundFlag = 1;
                result_error = errorBound;
                break;
            }
            if (targetCompressionRatio > CR) left_error = errorBound;
            else right_error = errorBound;
            preCR = CR;
        }
    }
    *eb_out = result_error;
    return cudaSuccess;
}

// computeRadiusBuffer (szx/src/szx.cc:475-485): radius and median of the
// sampled blocks and their copies, into host arrays; returns the sampled range.
cudaError_t fxr_radius_buffer(int dtype, const void* d_x, size_t n, int rate, int bs, void* d_ws, size_t wsb,
                              void* d_copy, cudaStream_t s, float* h_rads, float* h_meds, void* h_copy,
                              float* range_out) {
    if (bs < 1 || rate < 1 || n == 0 || wsb < fxr_ws_bytes(dtype, n, bs, rate)) return cudaErrorInvalidValue;
    FxSample S;
    S.dtype = dtype; S.bs = bs; S.G = lanes_for(dtype, bs); S.n = n;
    S.ns = n / ((size_t)bs * rate); S.nden = S.ns; S.stride = (size_t)bs * rate;
    S.x = d_x; S.w = fx_carve(d_ws, S.ns + 2); S.double_radius = false; S.s = s;
    cudaError_t e = S.stats(range_out);
    if (e != cudaSuccess || S.ns == 0) return e;
    const size_t es = dtype == 0 ? 4 : 8;
    const unsigned grid = (unsigned)((S.ns * bs + 255) / 256 < 4096 ? (S.ns * bs + 255) / 256 : 4096);
    if (dtype == 0) k_fxr_gather<float><<<grid, 256, 0, s>>>((const float*)d_x, S.ns, S.stride, bs, (float*)d_copy);
    else k_fxr_gather<double><<<grid, 256, 0, s>>>((const double*)d_x, S.ns, S.stride, bs, (double*)d_copy);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(h_rads, S.w.rads, 4 * S.ns, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(h_meds, S.w.meds, 4 * S.ns, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(h_copy, d_copy, es * S.ns * bs, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
    return cudaStreamSynchronize(s);
}

// estimateCRbasedonErrorBound_buffered (szx/src/szx.cc:487-498) over sampled
// blocks already copied contiguously to the device, with their radius and
// median arrays.
cudaError_t fxr_estimate_buffered(int dtype, const void* d_copy, size_t n, int rate, int bs, const float* h_rads,
                                  const float* h_meds, float eb, void* d_ws, size_t wsb, cudaStream_t s, float* cr,
                                  size_t* sumReq, size_t* sumLead) {
    if (bs < 1 || rate < 1 || n == 0 || wsb < fxr_ws_bytes(dtype, n, bs, rate)) return cudaErrorInvalidValue;
    FxSample S;
    S.dtype = dtype; S.bs = bs; S.G = lanes_for(dtype, bs); S.n = n;
    S.ns = n / ((size_t)bs * rate); S.nden = S.ns; S.stride = (size_t)bs;
    S.x = d_copy; S.w = fx_carve(d_ws, S.ns + 2); S.double_radius = false; S.s = s;
    cudaError_t e;
    if (S.ns) {
        if ((e = cudaMemcpyAsync(S.w.rads, h_rads, 4 * S.ns, cudaMemcpyHostToDevice, s)) != cudaSuccess) return e;
        if ((e = cudaMemcpyAsync(S.w.meds, h_meds, 4 * S.ns, cudaMemcpyHostToDevice, s)) != cudaSuccess) return e;
    }
    size_t sc = 0;
    return S.eval(eb, cr, sumReq, sumLead, &sc);
}

}  // namespace szxg
