// Failure-detection self-test of the device-wide look-back scans.
//
// Every variable-length placement in this library (payload offsets of the
// encoders, the decoders' offset and rank scans) goes through a decoupled
// look-back: a tile waits for its predecessors' status words.  Tiles are
// taken in order, so in the codecs every predecessor is running and the wait
// ends; the waits are still bounded, and a tile that gives up records
// SZXG_ERR_LOOKBACK in the call's error word instead of hanging the GPU.
//
// SZxG_selftest_lookback runs the same look-back functions the codecs use over
// ntiles one-warp tiles (tile t contributes t + 1 bytes), with one tile
// `withheld` that never publishes, and a small poll limit.  The tile after the
// withheld one waits, gives up after `spinLimit` polls, and the call reports
// SZXG_ERR_LOOKBACK; with nothing withheld it returns every tile's exclusive
// prefix, t(t+1)/2.  Nothing faults, traps or waits without a limit.
#include <vector>

#include "../../include/szx_gb300.h"
#include "common.cuh"
#include "kernels.h"

namespace szxg {
namespace {

// scan 0: the 64-bit status words of the encoders' placement (prefix_resolve);
// scan 1: the 32-bit words with an inclusive side array (lookback_wide) of the
//         decoders and the non-blocked layout.
__global__ void k_selftest_lookback(int scan, unsigned long long* st64, TileStatus32 st32, int ntiles, int withheld,
                                    unsigned limit, unsigned long long* prefix, int* err) {
    const long long tile = blockIdx.x;
    if (tile >= ntiles || tile == withheld) return;   // the withheld tile never publishes
    const unsigned long long agg = (unsigned long long)tile + 1;
    unsigned long long p = 0;
    if (scan == 0) {
        prefix_publish(st64, tile, agg);
        p = prefix_resolve(st64, tile, agg, err, limit);
    } else {
        unsigned long long dummy = 0;
        lookback_wide(st32, tile, (uint32_t)agg, 0u, &p, &dummy, err, limit);
    }
    if (lane_id() == 0) prefix[tile] = p;
}

}  // namespace
}  // namespace szxg

using namespace szxg;

extern "C" int SZxG_selftest_lookback(int scan, int ntiles, int withheld, unsigned spinLimit,
                                      unsigned long long* prefix, void* stream) {
    if ((scan != 0 && scan != 1) || ntiles < 1 || ntiles > 4096 || withheld >= ntiles || spinLimit < 1) {
        set_last_error(SZXG_ERR_ARG);
        return SZXG_ERR_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const size_t n = (size_t)ntiles;
    auto a256 = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t o32 = a256(8 * (n + 8)), oinc = o32 + a256(4 * (n + 8)), opre = oinc + a256(16 * n),
                 oerr = opre + a256(8 * n), bytes = oerr + 256;
    unsigned char* b = nullptr;
    if (cudaMalloc(&b, bytes) != cudaSuccess) {
        cudaGetLastError();
        set_last_error(SZXG_ERR_CUDA);
        return SZXG_ERR_CUDA;
    }
    unsigned long long* st64 = (unsigned long long*)b;          // [n + 8]
    TileStatus32 st32;
    st32.st = (uint32_t*)(b + o32);                             // [n + 8]
    st32.inc_a = (unsigned long long*)(b + oinc);               // [n]
    st32.inc_b = st32.inc_a + n;                                // [n]
    unsigned long long* d_prefix = (unsigned long long*)(b + opre);
    int* d_err = (int*)(b + oerr);
    int rc = SZXG_OK;
    cudaError_t e = cudaMemsetAsync(b, 0, bytes, s);
    if (e == cudaSuccess) {
        k_selftest_lookback<<<ntiles, kWarp, 0, s>>>(scan, st64, st32, ntiles, withheld, spinLimit, d_prefix, d_err);
        e = cudaGetLastError();
    }
    int h_err = 0;
    std::vector<unsigned long long> h(n);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), d_prefix, 8 * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(b);
    if (e != cudaSuccess) {
        cudaGetLastError();
        rc = SZXG_ERR_CUDA;
    } else {
        rc = h_err == kErrLookback ? SZXG_ERR_LOOKBACK : h_err ? SZXG_ERR_ARG : SZXG_OK;
        if (prefix)
            for (size_t i = 0; i < n; i++) prefix[i] = h[i];
    }
    set_last_error(rc);
    return rc;
}
