// C-ABI layer: the reference's C entry points (szx/include/szx.h) and this
// library's device-pointer extensions, on top of the codec kernels.
//
// Host-buffer calls stage through a per-device context (stream + device
// buffers that grow on demand and are reused), so repeated calls cost no
// allocation.  Every failure returns NULL / 0 and records a code for
// SZxG_get_last_error(); no path falls back to the CPU.
#include <stdlib.h>
#include <string.h>

#include <mutex>

#include "../../include/szx_gb300.h"
#include "kernels.h"

namespace szxg {

// ------------------------------------------------------------------ device facts

int sm_count() {
    static int cache[64] = {0};
    int d = 0;
    cudaGetDevice(&d);
    if (d < 0 || d >= 64) d = 0;
    if (!cache[d]) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, d);
        cache[d] = v > 0 ? v : 1;
    }
    return cache[d];
}

// ------------------------------------------------------------------ workspace layout

static size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

struct WsLayout {
    size_t hdr, st32, st, st2, partials, o, m, s, p, rw, aux, m2, m2_bytes, total;
    size_t status_tiles, status2_tiles, blocks, words, aux_tiles;
};

static WsLayout ws_layout(int layout, int dtype, size_t n, int bs) {
    (void)dtype;
    WsLayout L = {};
    size_t nb = (layout == kNonBlocked || bs <= 0) ? 0 : (n + bs - 1) / bs;
    size_t tiles_elem = (n + 4095) / 4096 + 1;          // non-blocked tiles
    size_t tiles_blk = nb / 8 + 2;                        // blocked encode tiles (>= 8 blocks)
    L.status_tiles = tiles_elem > tiles_blk ? tiles_elem : tiles_blk;
    L.words = nb / 32 + 2;
    L.status2_tiles = L.words / 2048 + 2;
    L.blocks = nb + 1;
    L.aux_tiles = tiles_elem;
    size_t off = 0;
    L.hdr = off; off += 4096;
    L.st32 = off; off += a256(4 * (L.status_tiles + 16));
    L.st = off; off += a256(8 * (3 * L.status_tiles > blocked_status_words(nb) ? 3 * L.status_tiles : blocked_status_words(nb)));
    L.st2 = off; off += a256(3 * 8 * L.status2_tiles);
    L.partials = off; off += a256(4096 * 24);
    L.o = off; off += a256(2 * L.blocks);
    L.m = off; off += a256(4 * L.blocks);
    L.s = off; off += a256(L.blocks / 8 + 64);
    L.p = off; off += a256(8 * L.blocks);
    L.rw = off; off += a256(4 * L.words);
    L.aux = off; off += a256(3 * 8 * L.aux_tiles);
    // fastMode 2 decode: boundary-search tables for the largest valid stream
    L.m2_bytes = layout == kBlocked && bs > 0 ? m2_ws_bytes(dtype, n, bs, blocked_bound(kBlocked, dtype, n, bs)) : 0;
    L.m2 = off; off += a256(L.m2_bytes);
    L.total = off;
    return L;
}

size_t ws_bytes(int layout, int dtype, size_t n, int bs) { return ws_layout(layout, dtype, n, bs).total; }

Workspace ws_carve(void* base, int layout, int dtype, size_t n, int bs) {
    WsLayout L = ws_layout(layout, dtype, n, bs);
    uint8_t* b = (uint8_t*)base;
    Workspace w;
    uint8_t* h = b + L.hdr;
    w.params = (CodecParams*)(h + 0);
    w.totals = (Totals*)(h + 64);
    w.result = (StreamResult*)(h + 128);
    w.bhdr = (BlockedHdr*)(h + 192);
    w.nhdr = (NonBlockedHdr*)(h + 320);
    w.err = (int*)(h + 448);
    w.counters = (unsigned long long*)(h + 512);
    w.st32 = (uint32_t*)(b + L.st32);
    w.st_word = (unsigned long long*)(b + L.st);
    w.st_agg2 = w.st_word + L.status_tiles;
    w.st_inc2 = w.st_agg2 + L.status_tiles;
    w.st2_word = (unsigned long long*)(b + L.st2);
    w.st2_agg2 = w.st2_word + L.status2_tiles;
    w.st2_inc2 = w.st2_agg2 + L.status2_tiles;
    w.partials = b + L.partials;
    w.o_scr = (uint16_t*)(b + L.o);
    w.m_scr = (uint32_t*)(b + L.m);
    w.s_scr = b + L.s;
    w.p_off = (unsigned long long*)(b + L.p);
    w.rank_w = (uint32_t*)(b + L.rw);
    w.tile_aux = (unsigned long long*)(b + L.aux);
    w.m2 = b + L.m2;
    w.m2_bytes = L.m2_bytes;
    w.status_tiles = L.status_tiles;
    w.status2_tiles = L.status2_tiles;
    w.blocks = L.blocks;
    w.words = L.words;
    w.aux_tiles = L.aux_tiles;
    return w;
}

// Offset of the header region's error word / result inside a workspace.
static const size_t kWsErrOff = 448, kWsResultOff = 128;

// ------------------------------------------------------------------ errors

static thread_local int g_last_error = SZXG_OK;
static void set_err(int e) { g_last_error = e; }
void set_last_error(int e) { g_last_error = e; }

// ------------------------------------------------------------------ per-device context

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    bool ensure(size_t want, bool zero_header = false) {
        if (want <= cap) return true;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        size_t c = want + want / 8 + 4096;
        if (cudaMalloc(&p, c) != cudaSuccess) { p = nullptr; return false; }
        if (zero_header && cudaMemset(p, 0, c < (1u << 20) ? c : (1u << 20)) != cudaSuccess) return false;
        cap = c;
        return true;
    }
};

struct Ctx {
    std::mutex mu;
    cudaStream_t stream = nullptr;
    DevBuf in, out, ws, fx, fx2;   // fx / fx2: fixed-rate search scratch and sample copies
    bool init() {
        if (stream) return true;
        return cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) == cudaSuccess;
    }
};

static Ctx* ctx_for_device() {
    static Ctx ctxs[64];
    int d = 0;
    if (cudaGetDevice(&d) != cudaSuccess || d < 0 || d >= 64) return nullptr;
    return &ctxs[d];
}

static int cuda_fail(cudaError_t e) {
    (void)e;
    cudaGetLastError();
    set_err(SZXG_ERR_CUDA);
    return SZXG_ERR_CUDA;
}

// ------------------------------------------------------------------ core enqueue

static bool layout_ok(int mode) { return mode >= 1 && mode <= 4; }

size_t bound_for(int mode, int dtype, size_t n, int bs) {
    return mode == kNonBlocked ? nonblocked_bound(dtype, n) : blocked_bound(mode, dtype, n, bs);
}

__global__ void k_ws_clear(ClearList c) {
    const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t nthr = (size_t)gridDim.x * blockDim.x;
    for (int r = 0; r < c.n; r++) {
        uint32_t* p = (uint32_t*)c.p[r];
        const size_t words = c.bytes[r] / 4;
        for (size_t i = tid; i < words; i += nthr) p[i] = 0u;
    }
}

cudaError_t launch_ws_clear(const ClearList& c, cudaStream_t s) {
    size_t words = 0;
    for (int r = 0; r < c.n; r++) {
        if (((uintptr_t)c.p[r] & 3) || (c.bytes[r] & 3)) return cudaErrorInvalidValue;
        words = words > c.bytes[r] / 4 ? words : c.bytes[r] / 4;
    }
    const size_t want = (words + 255) / 256, cap = (size_t)sm_count() * 4;
    const int grid = (int)(want < 1 ? 1 : (want < cap ? want : cap));
    k_ws_clear<<<grid, 256, 0, s>>>(c);
    return cudaGetLastError();
}

// Enqueue compress; the result record lands in res_out (device; default
// ws.result).  One launch clears what the passes expect zeroed (the
// value-range pass's ticket and the result record among it), so the
// value-range pass and the encoder skip their own clears.
static int enqueue_compress(int mode, int dtype, const void* d_x, size_t n, int bs, int err_mode, float abs_eb,
                            float rel, uint8_t* d_out, size_t cap, const Workspace& ws, cudaStream_t s,
                            StreamResult* res_out = nullptr) {
    cudaError_t e;
    if (n == 0 || (mode != kNonBlocked && bs < 1)) return cuda_fail(cudaErrorInvalidValue);
    ClearList c = mode == kNonBlocked ? nonblocked_enc_clear(ws, n) : blocked_enc_clear(ws, (n + bs - 1) / bs);
    if (res_out) {
        c.p[c.n] = res_out;
        c.bytes[c.n] = sizeof(StreamResult);
        c.n++;
    }
    if ((e = launch_ws_clear(c, s)) != cudaSuccess) return cuda_fail(e);
    if (mode == kNonBlocked) {
        if ((e = launch_range(dtype, d_x, n, err_mode, abs_eb, rel, ws, s, true)) != cudaSuccess) return cuda_fail(e);
        if ((e = launch_nonblocked_encode(dtype, d_x, n, d_out, cap, ws, s, true, res_out)) != cudaSuccess)
            return cuda_fail(e);
        return SZXG_OK;
    }
    bool use_params = err_mode == REL;
    if (use_params && (e = launch_range(dtype, d_x, n, err_mode, abs_eb, rel, ws, s, true)) != cudaSuccess)
        return cuda_fail(e);
    if ((e = launch_blocked_encode(mode, dtype, d_x, n, bs, use_params, abs_eb, d_out, cap, ws, s, true, res_out)) !=
        cudaSuccess)
        return cuda_fail(e);
    return SZXG_OK;
}

static int enqueue_decompress(int mode, int dtype, const uint8_t* d_s, size_t len, size_t n, int bs, void* d_out,
                              const Workspace& ws, cudaStream_t s) {
    cudaError_t e;
    if (mode == kNonBlocked) e = launch_nonblocked_decode(dtype, d_s, len, n, d_out, ws, s);
    else e = launch_blocked_decode(mode, dtype, d_s, len, n, bs, d_out, ws, s);
    if (e != cudaSuccess) return cuda_fail(e);
    return SZXG_OK;
}

static bool check_compress_args(int mode, int dtype, size_t n, int bs, int err_mode) {
    if (!layout_ok(mode) || (dtype != 0 && dtype != 1) || n == 0) return false;
    if (err_mode != ABS && err_mode != REL) return false;
    if (mode != kNonBlocked && (bs < 1 || bs > 256)) return false;
    if (mode == kBlocked && bs > 255) return false;
    return true;
}

// Device -> library-allocated host copy in pieces, each enqueued once the
// prefault workers have made its pages resident.
static cudaError_t copy_out_pieces(void* dst, const uint8_t* src, size_t len, cudaStream_t s) {
    for (size_t lo = 0; lo < len; lo += kHostCopyPiece) {
        const size_t m = std::min(kHostCopyPiece, len - lo);
        host_prefault_wait(lo + m);
        cudaError_t e = cudaMemcpyAsync((uint8_t*)dst + lo, src + lo, m, cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// Host round trip: compress host values, stream back into a host buffer.
// `out` == nullptr allocates with malloc.  Returns stream size, 0 on failure.
static size_t host_compress(int mode, int dtype, const void* data, size_t n, int bs, int err_mode, float abs_eb,
                            float rel, unsigned char** out, size_t out_cap, float fxr_ratio = 0.f,
                            float fxr_tolerance = 0.f) {
    // fixed rate: the bound comes from the reference's search on the device,
    // then the field is compressed into the fastMode-2 layout
    // (szx/src/szx_float.cc:921-949, szx/src/szx.cc:240-243)
    const bool fxr = err_mode == FXR;
    if (fxr) {
        mode = kBlocked;
        err_mode = ABS;
    }
    if (!data || !check_compress_args(mode, dtype, n, bs, err_mode)) { set_err(SZXG_ERR_ARG); return 0; }
    Ctx* c = ctx_for_device();
    if (!c) { set_err(SZXG_ERR_CUDA); return 0; }
    std::lock_guard<std::mutex> lk(c->mu);
    if (!c->init()) { set_err(SZXG_ERR_CUDA); return 0; }
    const size_t es = dtype == 0 ? 4 : 8;
    const size_t cap = bound_for(mode, dtype, n, bs);
    const size_t wsb = ws_bytes(mode, dtype, n, bs);
    if (!c->in.ensure(n * es) || !c->out.ensure(cap) || !c->ws.ensure(wsb, true)) { set_err(SZXG_ERR_CUDA); return 0; }
    Workspace ws = ws_carve(c->ws.p, mode, dtype, n, bs);
    cudaStream_t s = c->stream;
    // a library-allocated output is faulted in by host threads while the GPU works
    unsigned char* dst = *out;
    const bool own = dst == nullptr;
    if (own) {
        dst = (unsigned char*)malloc(cap ? cap : 1);
        if (!dst) { set_err(SZXG_ERR_ARG); return 0; }
        host_prefault_start(dst, cap);
    }
    auto drop = [&]() {
        if (own) {
            host_prefault_finish(0);
            free(dst);
        }
    };
    cudaError_t e = cudaMemcpyAsync(c->in.p, data, n * es, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) { drop(); cuda_fail(e); return 0; }
    if (fxr) {
        const size_t fb = fxr_ws_bytes(dtype, n, bs, 10);
        if (!c->fx.ensure(fb)) { drop(); set_err(SZXG_ERR_CUDA); return 0; }
        if ((e = fxr_bound(dtype, c->in.p, n, bs, fxr_ratio, fxr_tolerance, c->fx.p, c->fx.cap, s, &abs_eb)) !=
            cudaSuccess) {
            drop();
            cuda_fail(e);
            return 0;
        }
    }
    if (enqueue_compress(mode, dtype, c->in.p, n, bs, err_mode, abs_eb, rel, (uint8_t*)c->out.p, c->out.cap, ws, s)) {
        drop();
        return 0;
    }
    StreamResult r;
    int err = 0;
    if ((e = cudaMemcpyAsync(&r, ws.result, sizeof(r), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(&err, ws.err, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess) {
        drop();
        cuda_fail(e);
        return 0;
    }
    if (err) { drop(); set_err(err); return 0; }
    if (own) {
        host_prefault_limit(r.size);
        e = copy_out_pieces(dst, (const uint8_t*)c->out.p + r.offset, r.size, s);
        host_prefault_finish(r.size);
    } else if (out_cap < r.size) {
        set_err(SZXG_ERR_CAPACITY);
        return 0;
    } else {
        e = cudaMemcpyAsync(dst, (uint8_t*)c->out.p + r.offset, r.size, cudaMemcpyDeviceToHost, s);
    }
    const cudaError_t es2 = cudaStreamSynchronize(s);   // no copy may still target dst when it is freed
    if (e == cudaSuccess) e = es2;
    if (e != cudaSuccess) {
        if (own) free(dst);
        cuda_fail(e);
        return 0;
    }
    if (own) {
        // give back the tail of the bound-sized allocation
        unsigned char* shrunk = (unsigned char*)realloc(dst, r.size ? r.size : 1);
        if (shrunk) dst = shrunk;
    }
    *out = dst;
    set_err(SZXG_OK);
    return r.size;
}

static uint64_t be64h(const unsigned char* p) {
    uint64_t v = 0;
    for (int i = 0; i < 8; i++) v = (v << 8) | p[i];
    return v;
}

// Decode a host stream into host memory (`out` == nullptr: malloc).
static void* host_decompress(int mode, int dtype, const unsigned char* bytes, size_t len, size_t n, void* out) {
    if (!bytes || n == 0 || (dtype != 0 && dtype != 1)) { set_err(SZXG_ERR_ARG); return nullptr; }
    if (!layout_ok(mode)) {
        set_err(SZXG_ERR_UNSUPPORTED);
        return nullptr;
    }
    int bs = 0;
    if (mode == kBlocked) {
        if (len < 13) { set_err(SZXG_ERR_STREAM); return nullptr; }
        bs = bytes[4];
        if (bs < 1) { set_err(SZXG_ERR_STREAM); return nullptr; }
    } else if (mode != kNonBlocked) {
        if (len < 20) { set_err(SZXG_ERR_STREAM); return nullptr; }
        uint64_t b = be64h(bytes + 4);
        if (b < 1 || b > 256) { set_err(b > 256 ? SZXG_ERR_UNSUPPORTED : SZXG_ERR_STREAM); return nullptr; }
        bs = (int)b;
    }
    Ctx* c = ctx_for_device();
    if (!c) { set_err(SZXG_ERR_CUDA); return nullptr; }
    std::lock_guard<std::mutex> lk(c->mu);
    if (!c->init()) { set_err(SZXG_ERR_CUDA); return nullptr; }
    const size_t es = dtype == 0 ? 4 : 8;
    const size_t wsb = ws_bytes(mode, dtype, n, bs);
    // stream staged 15 bytes past an aligned address: the non-blocked lead
    // codes (stream offset 17) then start 16-byte aligned
    const size_t pad = mode == kNonBlocked ? 15 : 0;
    if (!c->in.ensure(len + pad + 16) || !c->out.ensure(n * es) || !c->ws.ensure(wsb, true)) {
        set_err(SZXG_ERR_CUDA);
        return nullptr;
    }
    Workspace ws = ws_carve(c->ws.p, mode, dtype, n, bs);
    cudaStream_t s = c->stream;
    // a library-allocated output is faulted in by host threads while the GPU works
    const bool own = out == nullptr;
    void* dst = own ? malloc(n * es) : out;
    if (!dst) { set_err(SZXG_ERR_ARG); return nullptr; }
    if (own) host_prefault_start(dst, n * es);
    auto drop = [&]() {
        if (own) {
            host_prefault_finish(0);
            free(dst);
        }
    };
    uint8_t* d_s = (uint8_t*)c->in.p + pad;
    cudaError_t e = cudaMemcpyAsync(d_s, bytes, len, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) { drop(); cuda_fail(e); return nullptr; }
    if (enqueue_decompress(mode, dtype, d_s, len, n, bs, c->out.p, ws, s)) { drop(); return nullptr; }
    int err = 0;
    if (own) {
        // the values follow the decode on the stream piece by piece, each as
        // soon as its pages are in; a failed decode's copy is discarded
        e = cudaMemcpyAsync(&err, ws.err, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = copy_out_pieces(dst, (const uint8_t*)c->out.p, n * es, s);
        host_prefault_finish(n * es);
        const cudaError_t es2 = cudaStreamSynchronize(s);   // no copy may still target dst when it is freed
        if (e == cudaSuccess) e = es2;
        if (e != cudaSuccess) { free(dst); cuda_fail(e); return nullptr; }
        if (err) { free(dst); set_err(err); return nullptr; }
        set_err(SZXG_OK);
        return dst;
    }
    // a caller's buffer is written only once the decode has succeeded
    if ((e = cudaMemcpyAsync(&err, ws.err, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess) {
        cuda_fail(e);
        return nullptr;
    }
    if (err) { set_err(err); return nullptr; }
    e = cudaMemcpyAsync(dst, c->out.p, n * es, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        cuda_fail(e);
        return nullptr;
    }
    set_err(SZXG_OK);
    return dst;
}

}  // namespace szxg

using namespace szxg;

// ===================================================================== C ABI

extern "C" {

int SZxG_get_last_error(void) { return g_last_error; }

const char* SZxG_error_string(int code) {
    switch (code) {
        case SZXG_OK: return "ok";
        case SZXG_ERR_LOOKBACK: return "device-wide scan timed out waiting for a predecessor tile";
        case SZXG_ERR_CAPACITY: return "output buffer too small";
        case SZXG_ERR_STREAM: return "malformed or truncated compressed stream";
        case SZXG_ERR_ARG: return "invalid argument";
        case SZXG_ERR_CUDA: return "CUDA runtime error";
        case SZXG_ERR_UNSUPPORTED: return "unsupported layout, type or block size";
        case SZXG_ERR_TOO_LARGE: return "input larger than the fixed scratch of SZxG_compress_noalloc (1,048,576 blocks)";
        default: return "unknown error";
    }
}

// szx/src/szx.cc:41-71
int SZx_computeDimension(size_t r5, size_t r4, size_t r3, size_t r2, size_t r1) {
    if (r1 == 0) return 0;
    if (r2 == 0) return 1;
    if (r3 == 0) return 2;
    if (r4 == 0) return 3;
    if (r5 == 0) return 4;
    return 5;
}

// szx/src/szx.cc:73-101
size_t SZx_computeDataLength(size_t r5, size_t r4, size_t r3, size_t r2, size_t r1) {
    if (r1 == 0) return 0;
    if (r2 == 0) return r1;
    if (r3 == 0) return r1 * r2;
    if (r4 == 0) return r1 * r2 * r3;
    if (r5 == 0) return r1 * r2 * r3 * r4;
    return r1 * r2 * r3 * r4 * r5;
}

// szx/src/szx.cc:109-229: drop size-1 dimensions; 0 unchanged, 1 corrected, 2 invalid.
int SZx_filterDimension(size_t r5, size_t r4, size_t r3, size_t r2, size_t r1, size_t* c) {
    int dim = SZx_computeDimension(r5, r4, r3, r2, r1);
    int changed = 0;
    c[0] = r1; c[1] = r2; c[2] = r3; c[3] = r4; c[4] = r5;
    if (dim == 1) {
        if (r1 < 1) return 2;
    } else if (dim == 2) {
        if (r2 == 1) { c[1] = 0; changed = 1; }
        if (r1 == 1) { c[0] = c[1]; c[1] = c[2]; changed = 1; }
    } else if (dim == 3) {
        if (r3 == 1) { c[2] = 0; changed = 1; }
        if (r2 == 1) { c[1] = c[2]; c[2] = c[3]; changed = 1; }
        if (r1 == 1) { c[0] = c[1]; c[1] = c[2]; c[2] = c[3]; changed = 1; }
    } else if (dim == 4) {
        if (r4 == 1) { c[3] = 0; changed = 1; }
        if (r3 == 1) { c[2] = c[3]; c[3] = c[4]; changed = 1; }
        if (r2 == 1) { c[1] = c[2]; c[2] = c[3]; c[3] = c[4]; changed = 1; }
        if (r1 == 1) { c[0] = c[1]; c[1] = c[2]; c[2] = c[3]; c[3] = c[4]; changed = 1; }
    } else if (dim == 5) {
        if (r5 == 1) { c[4] = 0; changed = 1; }
        if (r4 == 1) { c[3] = c[4]; c[4] = 0; changed = 1; }
        if (r3 == 1) { c[2] = c[3]; c[3] = c[4]; c[4] = 0; changed = 1; }
        if (r2 == 1) { c[1] = c[2]; c[2] = c[3]; c[3] = c[4]; c[4] = 0; changed = 1; }
        if (r1 == 1) { c[0] = c[1]; c[1] = c[2]; c[2] = c[3]; c[3] = c[4]; c[4] = 0; changed = 1; }
    }
    return changed;
}

unsigned char* SZx_fast_compress_args(int fastMode, int dataType, void* data, size_t* outSize, int errBoundMode,
                                      float absErrBound, float relBoundRatio, float compressionRatio, float tolerance,
                                      size_t r5, size_t r4, size_t r3, size_t r2, size_t r1) {
    if (outSize) *outSize = 0;
    const size_t n = SZx_computeDataLength(r5, r4, r3, r2, r1);
    unsigned char* out = nullptr;
    size_t sz = host_compress(fastMode, dataType, data, n, 128, errBoundMode, absErrBound, relBoundRatio, &out, 0,
                              compressionRatio, tolerance);
    if (!sz) return nullptr;
    if (outSize) *outSize = sz;
    return out;
}

void* SZx_fast_decompress(int fastMode, int dataType, unsigned char* bytes, size_t byteLength, size_t r5, size_t r4,
                          size_t r3, size_t r2, size_t r1) {
    const size_t n = SZx_computeDataLength(r5, r4, r3, r2, r1);
    return host_decompress(fastMode, dataType, bytes, byteLength, n, nullptr);
}

double SZx_computeValueRange(void* oriData, int dataType, size_t length, float* radius, float* medianValue) {
    if (!oriData || length == 0 || (dataType != 0 && dataType != 1)) { set_err(SZXG_ERR_ARG); return 0; }
    Ctx* c = ctx_for_device();
    if (!c) { set_err(SZXG_ERR_CUDA); return 0; }
    std::lock_guard<std::mutex> lk(c->mu);
    if (!c->init()) { set_err(SZXG_ERR_CUDA); return 0; }
    const size_t es = dataType == 0 ? 4 : 8;
    if (!c->in.ensure(length * es) || !c->ws.ensure(ws_bytes(1, dataType, length, 128), true)) {
        set_err(SZXG_ERR_CUDA);
        return 0;
    }
    Workspace ws = ws_carve(c->ws.p, 1, dataType, length, 128);
    cudaStream_t s = c->stream;
    CodecParams p;
    cudaError_t e = cudaMemcpyAsync(c->in.p, oriData, length * es, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = launch_range(dataType, c->in.p, length, ABS, 0.f, 0.f, ws, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&p, ws.params, sizeof(p), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { cuda_fail(e); return 0; }
    if (radius) { *radius = p.radius; if (medianValue) *medianValue = p.median; }
    set_err(SZXG_OK);
    return dataType == 0 ? (double)p.range_f : p.range_d;
}

unsigned char* SZx_fast_compress_args_unpredictable_blocked_randomaccess_openmp(void* oriData, int dataType,
                                                                                size_t* outSize, float absErrBound,
                                                                                size_t nbEle, int blockSize) {
    unsigned char* out = nullptr;
    size_t sz = host_compress(kRandomAccessNative, dataType, oriData, nbEle, blockSize, ABS, absErrBound, 0.f, &out, 0);
    if (outSize) *outSize = sz;
    return sz ? out : nullptr;
}

void* SZx_fast_decompress_args_unpredictable_blocked_randomaccess_openmp(int dataType, size_t nbEle,
                                                                         unsigned char* cmpBytes) {
    // the reference passes no stream length; bound it by the largest stream
    // nbEle values can produce
    if (!cmpBytes || nbEle == 0) { set_err(SZXG_ERR_ARG); return nullptr; }
    uint64_t bs = be64h(cmpBytes + 4);
    if (bs < 1 || bs > 256) { set_err(SZXG_ERR_STREAM); return nullptr; }
    size_t len = blocked_bound(kRandomAccessNative, dataType, nbEle, (int)bs) - 64;
    return host_decompress(kRandomAccessNative, dataType, cmpBytes, len, nbEle, nullptr);
}

unsigned char* SZx_fast_compress_args_unpredictable_blocked(void* oriData, int dataType, size_t* outSize,
                                                            float absErrBound, size_t nbEle, int blockSize) {
    unsigned char* out = nullptr;
    size_t sz = host_compress(kBlocked, dataType, oriData, nbEle, blockSize, ABS, absErrBound, 0.f, &out, 0);
    if (outSize) *outSize = sz;
    return sz ? out : nullptr;
}

size_t SZx_fast_compress_args_unpredictable_blocked_args(void* oriData, int dataType, unsigned char* outputBytes,
                                                         float absErrBound, size_t nbEle, int blockSize) {
    if (dataType != SZx_FLOAT) return 0;   // szx/src/szx.cc:507-510
    unsigned char* out = outputBytes;
    return host_compress(kBlocked, dataType, oriData, nbEle, blockSize, ABS, absErrBound, 0.f, &out,
                         blocked_bound(kBlocked, dataType, nbEle, blockSize));
}

// Length of a fastMode-2 stream of nbEle values, read from its block headers
// (this entry point gets no length; the payload has no size index).  Only the
// 1 + ceil(bs/4) header bytes of each non-constant block are read.  0 when
// the bytes cannot be a stream.
static size_t m2_stream_length(const unsigned char* b, size_t nbEle, int dataType) {
    const size_t bs = b[4];
    if (bs < 1 || b[3] != 0) return 0;
    const size_t nb = (nbEle + bs - 1) / bs, sb = (nb + 7) / 8;
    const size_t nc = (size_t)be64h(b + 5);
    if (nc > nb) return 0;
    size_t nnc = 0;
    for (size_t i = 0; i < sb; i++) nnc += (size_t)__builtin_popcount(b[13 + i]);
    if (nnc + nc != nb) return 0;   // also rejects set padding bits
    const int lo = dataType == 0 ? 9 : 12, hi = dataType == 0 ? 32 : 64;
    size_t p = 13 + sb + 4 * nc;
    const bool last_coded = (b[13 + (nb - 1) / 8] >> (7 - (nb - 1) % 8)) & 1;
    for (size_t r = 0; r < nnc; r++) {
        const size_t blen = (r + 1 == nnc && last_coded) ? nbEle - (nb - 1) * bs : bs;
        const int rl = b[p];
        if (rl < lo || rl > hi) return 0;
        const int R = (rl >> 3) + ((rl & 7) != 0);
        const size_t Lb = (blen + 3) / 4;
        size_t mid = 0;
        for (size_t v = 0; v < blen; v++) {
            const int ld = (b[p + 5 + v / 4] >> (6 - 2 * (v % 4))) & 3;
            mid += R > ld ? (size_t)(R - ld) : 0;
        }
        p += 5 + Lb + mid;
    }
    return p;
}

// szx/src/szx.cc:513-520: fastMode-2 stream -> *newData (a float** or
// double** by type, malloc'd here as the reference does).
void SZx_fast_decompress_args_unpredictable_blocked(void* newData, int dataType, size_t nbEle,
                                                   unsigned char* cmpBytes) {
    if (!newData || !cmpBytes || nbEle == 0 || (dataType != 0 && dataType != 1)) { set_err(SZXG_ERR_ARG); return; }
    const size_t len = m2_stream_length(cmpBytes, nbEle, dataType);
    if (!len) { set_err(SZXG_ERR_STREAM); return; }
    void* out = host_decompress(kBlocked, dataType, cmpBytes, len, nbEle, nullptr);
    if (out) *(void**)newData = out;
}

// Stage n values of a host array on the device (Ctx input buffer).
static bool stage_input(Ctx* c, const void* data, size_t bytes) {
    if (!c->in.ensure(bytes)) return false;
    return cudaMemcpyAsync(c->in.p, data, bytes, cudaMemcpyHostToDevice, c->stream) == cudaSuccess;
}

// szx/src/szx.cc:458-464.  The reference's model behind this entry point ends
// the process (exit(0), szx/src/szx_float.cc:681, szx/src/szx_double.cc:678);
// this one returns the bound its search settles on (0 on failure, with
// SZxG_get_last_error() set).
float SZx_estimateErrorBoundbasedonCR(int dataType, float targetCompressionRatio, float tolerance, void* data,
                                      float initErrorBound, int blockSize, size_t nbEle) {
    if (!data || nbEle == 0 || blockSize < 1 || (dataType != 0 && dataType != 1)) { set_err(SZXG_ERR_ARG); return 0.f; }
    Ctx* c = ctx_for_device();
    if (!c) { set_err(SZXG_ERR_CUDA); return 0.f; }
    std::lock_guard<std::mutex> lk(c->mu);
    if (!c->init()) { set_err(SZXG_ERR_CUDA); return 0.f; }
    const size_t es = dataType == 0 ? 4 : 8;
    if (!stage_input(c, data, nbEle * es) || !c->fx.ensure(fxr_ws_bytes(dataType, nbEle, blockSize, 10))) {
        set_err(SZXG_ERR_CUDA);
        return 0.f;
    }
    float eb = 0.f;
    cudaError_t e = fxr_bound_unbuffered(dataType, c->in.p, nbEle, blockSize, targetCompressionRatio, tolerance,
                                         initErrorBound, c->fx.p, c->fx.cap, c->stream, &eb);
    if (e != cudaSuccess) { cuda_fail(e); return 0.f; }
    set_err(SZXG_OK);
    return eb;
}

// szx/src/szx.cc:475-485: radius, median and a copy of every samplingRate-th
// block (arrays malloc'd here, nbEle/(samplingRate*blockSize)+1 entries as
// the reference allocates; the caller frees them).  `buffer` is a float** or
// double** by data type.  Returns the sampled value range.
float computeRadiusBuffer(void* oriData, int dataType, size_t nbEle, int samplingRate, int blockSize,
                          float** radiusArray, float** mediusArray, void* buffer) {
    if (!oriData || !radiusArray || !mediusArray || !buffer || nbEle == 0 || blockSize < 1 || samplingRate < 1 ||
        (dataType != 0 && dataType != 1)) {
        set_err(SZXG_ERR_ARG);
        return 0.f;
    }
    Ctx* c = ctx_for_device();
    if (!c) { set_err(SZXG_ERR_CUDA); return 0.f; }
    std::lock_guard<std::mutex> lk(c->mu);
    if (!c->init()) { set_err(SZXG_ERR_CUDA); return 0.f; }
    const size_t es = dataType == 0 ? 4 : 8;
    const size_t ns = nbEle / ((size_t)samplingRate * blockSize);
    float* rads = (float*)malloc(sizeof(float) * (ns + 1));
    float* meds = (float*)malloc(sizeof(float) * (ns + 1));
    void* copy = malloc(es * (ns + 1) * blockSize);
    if (!rads || !meds || !copy) {
        free(rads); free(meds); free(copy);
        set_err(SZXG_ERR_ARG);
        return 0.f;
    }
    float range = 0.f;
    cudaError_t e = cudaSuccess;
    if (!stage_input(c, oriData, nbEle * es) || !c->fx.ensure(fxr_ws_bytes(dataType, nbEle, blockSize, samplingRate)) ||
        !c->fx2.ensure(es * (ns + 1) * blockSize))
        e = cudaErrorMemoryAllocation;
    if (e == cudaSuccess)
        e = fxr_radius_buffer(dataType, c->in.p, nbEle, samplingRate, blockSize, c->fx.p, c->fx.cap, c->fx2.p,
                              c->stream, rads, meds, copy, &range);
    if (e != cudaSuccess) {
        free(rads); free(meds); free(copy);
        cuda_fail(e);
        return 0.f;
    }
    *radiusArray = rads;
    *mediusArray = meds;
    *(void**)buffer = copy;
    set_err(SZXG_OK);
    return range;
}

// szx/src/szx.cc:487-498: the ratio model at errorBound over the sampled
// blocks computeRadiusBuffer returned.
float estimateCRbasedonErrorBound_buffered(int dataType, float errorBound, void* buffer, float* medianArray,
                                          float* radiusArray, int samplingRate, int blockSize, size_t nbEle,
                                          size_t* sumReqNbBytes, size_t* sum_actual_leadNumbers) {
    if (!buffer || !medianArray || !radiusArray || !sumReqNbBytes || !sum_actual_leadNumbers || nbEle == 0 ||
        blockSize < 1 || samplingRate < 1 || (dataType != 0 && dataType != 1)) {
        set_err(SZXG_ERR_ARG);
        return 0.f;
    }
    Ctx* c = ctx_for_device();
    if (!c) { set_err(SZXG_ERR_CUDA); return 0.f; }
    std::lock_guard<std::mutex> lk(c->mu);
    if (!c->init()) { set_err(SZXG_ERR_CUDA); return 0.f; }
    const size_t es = dataType == 0 ? 4 : 8;
    const size_t ns = nbEle / ((size_t)samplingRate * blockSize);
    float cr = 0.f;
    cudaError_t e = cudaSuccess;
    if ((ns && !stage_input(c, buffer, es * ns * blockSize)) ||
        !c->fx.ensure(fxr_ws_bytes(dataType, nbEle, blockSize, samplingRate)))
        e = cudaErrorMemoryAllocation;
    if (e == cudaSuccess && !c->in.p && !c->in.ensure(16)) e = cudaErrorMemoryAllocation;
    if (e == cudaSuccess)
        e = fxr_estimate_buffered(dataType, c->in.p, nbEle, samplingRate, blockSize, radiusArray, medianArray,
                                  errorBound, c->fx.p, c->fx.cap, c->stream, &cr, sumReqNbBytes,
                                  sum_actual_leadNumbers);
    if (e != cudaSuccess) { cuda_fail(e); return 0.f; }
    set_err(SZXG_OK);
    return cr;
}

// ------------------------------------------------------------------ SZxG device-pointer interface

size_t SZxG_compress_bound(int fastMode, int dataType, size_t nbEle, int blockSize) {
    if (!layout_ok(fastMode)) return 0;
    return bound_for(fastMode, dataType, nbEle, blockSize);
}

size_t SZxG_workspace_size(int fastMode, int dataType, size_t nbEle, int blockSize) {
    if (!layout_ok(fastMode)) return 0;
    return ws_bytes(fastMode, dataType, nbEle, blockSize);
}

int SZxG_compress(int fastMode, int dataType, const void* d_data, size_t nbEle, int blockSize, int errBoundMode,
                  float absErrBound, float relBoundRatio, void* d_out, size_t outCapacity, void* d_workspace,
                  size_t workspaceBytes, SZxG_StreamInfo* d_info, void* stream) {
    if (!d_data || !d_out || !d_workspace || !check_compress_args(fastMode, dataType, nbEle, blockSize, errBoundMode) ||
        workspaceBytes < ws_bytes(fastMode, dataType, nbEle, blockSize) ||
        outCapacity < bound_for(fastMode, dataType, nbEle, blockSize)) {
        set_err(SZXG_ERR_ARG);
        return SZXG_ERR_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    Workspace ws = ws_carve(d_workspace, fastMode, dataType, nbEle, blockSize);
    static_assert(sizeof(SZxG_StreamInfo) == sizeof(StreamResult), "info layout");
    // the kernels write the result record straight into an 8-byte aligned
    // d_info; any other d_info gets a copy of it
    const bool direct = d_info && ((uintptr_t)d_info & 7) == 0;
    int rc = enqueue_compress(fastMode, dataType, d_data, nbEle, blockSize, errBoundMode, absErrBound, relBoundRatio,
                              (uint8_t*)d_out, outCapacity, ws, s, direct ? (StreamResult*)d_info : nullptr);
    if (rc) return rc;
    if (d_info && !direct) {
        cudaError_t e = cudaMemcpyAsync(d_info, ws.result, sizeof(StreamResult), cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) return cuda_fail(e);
    }
    set_err(SZXG_OK);
    return SZXG_OK;
}

int SZxG_decompress(int fastMode, int dataType, const void* d_stream, size_t streamBytes, size_t nbEle,
                    int blockSize, void* d_out, void* d_workspace, size_t workspaceBytes, void* stream) {
    if (!d_stream || !d_out || !d_workspace || nbEle == 0 || (dataType != 0 && dataType != 1)) {
        set_err(SZXG_ERR_ARG);
        return SZXG_ERR_ARG;
    }
    if (!layout_ok(fastMode)) {
        set_err(SZXG_ERR_UNSUPPORTED);
        return SZXG_ERR_UNSUPPORTED;
    }
    cudaStream_t s = (cudaStream_t)stream;
    if (fastMode == kBlocked && blockSize == 0) {
        unsigned char h[5];
        if (streamBytes < 13 || cudaMemcpyAsync(h, d_stream, 5, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess || h[4] < 1) {
            set_err(SZXG_ERR_STREAM);
            return SZXG_ERR_STREAM;
        }
        blockSize = h[4];
    } else if (fastMode != kNonBlocked && blockSize == 0) {
        unsigned char h[12];
        if (streamBytes < 20 || cudaMemcpyAsync(h, d_stream, 12, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) {
            set_err(SZXG_ERR_STREAM);
            return SZXG_ERR_STREAM;
        }
        uint64_t b = be64h(h + 4);
        if (b < 1 || b > 256) { set_err(SZXG_ERR_UNSUPPORTED); return SZXG_ERR_UNSUPPORTED; }
        blockSize = (int)b;
    }
    if (workspaceBytes < ws_bytes(fastMode, dataType, nbEle, blockSize)) { set_err(SZXG_ERR_ARG); return SZXG_ERR_ARG; }
    Workspace ws = ws_carve(d_workspace, fastMode, dataType, nbEle, blockSize);
    // (the first kernel of every decode, the header parse, sets ws.err)
    int rc = enqueue_decompress(fastMode, dataType, (const uint8_t*)d_stream, streamBytes, nbEle, blockSize, d_out, ws,
                                s);
    if (rc == SZXG_OK) set_err(SZXG_OK);
    return rc;
}

int SZxG_workspace_status(const void* d_workspace, void* stream) {
    int err = 0;
    cudaStream_t s = (cudaStream_t)stream;
    if (cudaMemcpyAsync(&err, (const uint8_t*)d_workspace + kWsErrOff, sizeof(int), cudaMemcpyDeviceToHost, s) !=
            cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return cuda_fail(cudaErrorUnknown);
    (void)kWsResultOff;
    return err;
}

unsigned char* SZxG_compress_host(int fastMode, int dataType, const void* data, size_t nbEle, int blockSize,
                                  int errBoundMode, float absErrBound, float relBoundRatio, size_t* outSize) {
    unsigned char* out = nullptr;
    size_t sz = host_compress(fastMode, dataType, data, nbEle, blockSize, errBoundMode, absErrBound, relBoundRatio,
                              &out, 0);
    if (outSize) *outSize = sz;
    return sz ? out : nullptr;
}

void* SZxG_decompress_host(int fastMode, int dataType, const unsigned char* bytes, size_t byteLength, size_t nbEle) {
    return host_decompress(fastMode, dataType, bytes, byteLength, nbEle, nullptr);
}

size_t SZxG_compress_host_into(int fastMode, int dataType, const void* data, size_t nbEle, int blockSize,
                               int errBoundMode, float absErrBound, float relBoundRatio, unsigned char* out,
                               size_t outCapacity) {
    if (!out) { set_err(SZXG_ERR_ARG); return 0; }
    unsigned char* o = out;
    return host_compress(fastMode, dataType, data, nbEle, blockSize, errBoundMode, absErrBound, relBoundRatio, &o,
                         outCapacity);
}

int SZxG_decompress_host_into(int fastMode, int dataType, const unsigned char* bytes, size_t byteLength, size_t nbEle,
                              void* out) {
    if (!out) { set_err(SZXG_ERR_ARG); return SZXG_ERR_ARG; }
    return host_decompress(fastMode, dataType, bytes, byteLength, nbEle, out) ? SZXG_OK : g_last_error;
}

}  // extern "C"
