// SZxG_compress_noalloc: the blocked compress (fastMode 2, 3, 4) with its
// scratch in a fixed, file-scope device array instead of a caller-provided or
// library-allocated workspace.
//
// Who needs it: host applications that hand all device memory to their own
// pool allocator and do not let libraries call cudaMalloc, and loops that
// cannot afford cudaMalloc/cudaFree, which synchronise the whole device.
// They pass the input and output buffers; everything else lives in
// g_noalloc_scratch below.
//
// Cost and limits:
// * every GPU that loads this library holds kNoAllocBytes (about 7.2 MiB) of
//   device memory for the array until the process exits;
// * one call handles at most kNoAllocMaxBlocks = 1,048,576 blocks
//   (ceil(nbEle / blockSize)), i.e. 134,217,728 values at blockSize 128;
//   larger inputs are rejected with SZXG_ERR_TOO_LARGE before any GPU work;
// * all calls on a device share the array: two calls that overlap on the GPU
//   (different streams, or different host threads) race and corrupt each
//   other's result.  Calls must be ordered (same stream, or synchronised).
//   Each call re-clears the parts that must start at zero (tile status
//   words, tile counter, error word), so a call never sees the previous
//   call's contents.
// * the first call on a device resolves the array's device address with
//   cudaGetSymbolAddress (host code cannot use the symbol itself: in host
//   code it names a host-side stand-in); that first call should therefore
//   come before any stream capture.
#include <mutex>

#include "../../include/szx_gb300.h"
#include "kernels.h"

namespace szxg {

constexpr size_t kNoAllocMaxBlocks = size_t(1) << 20;
constexpr size_t kNoAllocHeader = 4096;
constexpr size_t na_a256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kNaSt = kNoAllocHeader;                                           // look-back status
constexpr size_t kNaPartials = kNaSt + na_a256(8 * blocked_status_words(kNoAllocMaxBlocks));
constexpr size_t kNaO = kNaPartials + na_a256(4096 * 24);                         // range-pass partials
constexpr size_t kNaM = kNaO + na_a256(2 * kNoAllocMaxBlocks);                    // sizes by block
constexpr size_t kNaS = kNaM + na_a256(4 * kNoAllocMaxBlocks);                    // medians by block
constexpr size_t kNoAllocBytes = kNaS + na_a256(kNoAllocMaxBlocks / 8 + 64);      // state bits

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {
std::mutex g_na_mu;
void* g_na_ptr[64] = {nullptr};

// Device address of g_noalloc_scratch on the current device (resolved once
// per device, with that device current).
int scratch_address(void** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return SZXG_ERR_CUDA;
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_na_ptr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return SZXG_ERR_CUDA;
        }
        g_na_ptr[dev] = p;
    }
    *out = g_na_ptr[dev];
    return SZXG_OK;
}

// The compress-only parts of a Workspace, carved out of the fixed array with
// the same header offsets as the allocating entry points use.
Workspace carve(unsigned char* b) {
    Workspace w = {};
    unsigned char* h = b;
    w.params = (CodecParams*)(h + 0);
    w.totals = (Totals*)(h + 64);
    w.result = (StreamResult*)(h + 128);
    w.err = (int*)(h + 448);
    w.counters = (unsigned long long*)(h + 512);
    w.st_word = (unsigned long long*)(b + kNaSt);
    w.partials = b + kNaPartials;
    w.o_scr = (uint16_t*)(b + kNaO);
    w.m_scr = (uint32_t*)(b + kNaM);
    w.s_scr = b + kNaS;
    w.status_tiles = blocked_status_words(kNoAllocMaxBlocks);
    w.blocks = kNoAllocMaxBlocks;
    return w;
}
}  // namespace

}  // namespace szxg

using namespace szxg;

namespace {
int na_ret(int rc) {
    set_last_error(rc);
    return rc;
}
}  // namespace

extern "C" int SZxG_compress_noalloc(int fastMode, int dataType, const void* d_data, size_t nbEle, int blockSize,
                                     int errBoundMode, float absErrBound, float relBoundRatio, void* d_out,
                                     size_t outCapacity, SZxG_StreamInfo* d_info, void* stream) {
    // Same codes as SZxG_compress, plus SZXG_ERR_UNSUPPORTED for fastMode 1
    // (no blocks: this entry point has no non-blocked variant) and
    // SZXG_ERR_TOO_LARGE beyond the fixed scratch.  Every return sets the
    // thread's last error.
    if (fastMode != kBlocked && fastMode != kRandomAccess && fastMode != kRandomAccessNative)
        return na_ret(fastMode == kNonBlocked ? SZXG_ERR_UNSUPPORTED : SZXG_ERR_ARG);
    if (!d_data || !d_out || !d_info || nbEle == 0 || (dataType != 0 && dataType != 1) || blockSize < 1 ||
        blockSize > 256 || (fastMode == kBlocked && blockSize > 255) || (errBoundMode != ABS && errBoundMode != REL))
        return na_ret(SZXG_ERR_ARG);
    const size_t nb = (nbEle + (size_t)blockSize - 1) / (size_t)blockSize;
    if (nb > kNoAllocMaxBlocks) return na_ret(SZXG_ERR_TOO_LARGE);
    if (outCapacity < blocked_bound(fastMode, dataType, nbEle, blockSize)) return na_ret(SZXG_ERR_ARG);
    void* base = nullptr;
    int rc = scratch_address(&base);
    if (rc) return na_ret(rc);
    Workspace ws = carve((unsigned char*)base);
    cudaStream_t s = (cudaStream_t)stream;
    const bool rel = errBoundMode == REL;
    cudaError_t e = cudaSuccess;
    if (rel) e = launch_range(dataType, d_data, nbEle, errBoundMode, absErrBound, relBoundRatio, ws, s);
    if (e == cudaSuccess)
        e = launch_blocked_encode(fastMode, dataType, d_data, nbEle, blockSize, rel, absErrBound, (uint8_t*)d_out,
                                  outCapacity, ws, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_info, ws.result, sizeof(StreamResult), cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return na_ret(SZXG_ERR_CUDA);
    }
    return na_ret(SZXG_OK);
}
