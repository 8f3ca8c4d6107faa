// Non-blocked layout of the SZx stream (fastMode 1):
//   SZx_fast_compress_args_unpredictable_float, szx/src/szx_float.cc:1492-1699
//   (double: szx/src/szx_double.cc:1593-2011), decoded by
//   szx/src/szxd_float.cc:478-662 (double: szx/src/szxd_double.cc:683-1114).
//
//   [1,1,1,0] | reqLength u8 | median f32 BE | leadBytes u64 BE | 2-bit lead
//   codes for all N values | mid bytes
//
// One global median/radius (from the value-range pass) and ONE XOR chain over
// the whole array: each value's lead code depends only on its predecessor, so
// codes are data-parallel; mid-byte positions need a device-wide prefix sum
// (encoder: decoupled look-back over 4096-value tiles, placed from the CTA's
// own previous tile and a window of status words).  Decoding must also find,
// for every value, the last earlier value that stored each of the top three
// byte lanes -- possibly many tiles back.  The lead codes alone give every
// tile's byte count and its last writers, so the decoder needs no look-back:
// per-tile counts (k_nb_count), one scan of group totals (k_nb_scan), the
// carried bytes per tile (k_nb_carry), then the tiles decode independently.
//
// The stream is placed 15 bytes into the output buffer so the lead-code array
// (stream offset 17) starts 16-byte aligned.
#include "common.cuh"
#include "kernels.h"

namespace szxg {

constexpr int kNbThreads = 256;
constexpr int kNbPer = 16;                        // values per thread
constexpr int kNbTile = kNbThreads * kNbPer;      // 4096 values per tile
constexpr unsigned long long kNbShift = 15;

// CTA-wide exclusive sum (256 threads), returns the total through *tot.  One
// barrier: the caller places another barrier between this call and the next
// one that writes `sm`.
__device__ __forceinline__ uint32_t cta_excl_sum32(uint32_t v, uint32_t* tot, uint32_t* sm /*[8]*/) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t incl = warp_inclusive_sum(v);
    if (lane == 31) sm[warp] = incl;
    __syncthreads();
    uint32_t pre = 0, t = 0;
#pragma unroll
    for (int w = 0; w < kNbThreads / 32; w++) {
        uint32_t x = sm[w];
        pre += w < warp ? x : 0;
        t += x;
    }
    *tot = t;
    return pre + incl - v;
}

// Copy [sh, sh+n) of a 16-aligned shared buffer to global dst (dst % 16 == sh).
__device__ __forceinline__ void cta_copy_out(const uint8_t* stage, uint32_t sh, uint32_t n, uint8_t* dst) {
    uint8_t* gbase = dst - sh;
    const uint32_t end = sh + n, nch = (end + 15) >> 4;
    for (uint32_t c = threadIdx.x; c < nch; c += blockDim.x) {
        uint32_t lo = c << 4;
        if (lo >= sh && lo + 16 <= end) *(uint4*)(gbase + lo) = *(const uint4*)(stage + lo);
    }
    // partial head chunk: threads 0-15, partial tail chunk: threads 16-31
    if (threadIdx.x < 32) {
        const uint32_t last = nch - 1;
        const uint32_t c = threadIdx.x < 16 ? 0 : last;
        const bool part = threadIdx.x < 16 ? (sh > 0 || end < 16) : (last > 0 && (end & 15) != 0);
        const uint32_t b = (c << 4) + (threadIdx.x & 15);
        if (part && b >= sh && b < end) gbase[b] = stage[b];
    }
}

// Stage [src, src+n) into a 16-aligned shared buffer at offset src % 16; bytes
// outside [s0, s1) are never read.
__device__ __forceinline__ void cta_copy_in(uint8_t* stage, const uint8_t* src, uint32_t n, const uint8_t* s0,
                                            const uint8_t* s1) {
    const uint32_t sh = (uint32_t)((uintptr_t)src & 15);
    const uint8_t* gbase = src - sh;
    const uint32_t nch = (sh + n + 15) >> 4;
    for (uint32_t c = threadIdx.x; c < nch; c += blockDim.x) {
        const uint8_t* lo = gbase + (c << 4);
        if (lo >= s0 && lo + 16 <= s1) *(uint4*)(stage + (c << 4)) = __ldg((const uint4*)lo);
        else
            for (int j = 0; j < 16; j++) stage[(c << 4) + j] = (lo + j >= s0 && lo + j < s1) ? lo[j] : 0;
    }
}

template <typename T>
__device__ __forceinline__ void load16(const T* p, unsigned long long first, unsigned long long n, T (&v)[kNbPer]) {
    const bool full = first + kNbPer <= n;
    if (full && ((uintptr_t)(p + first) % 16) == 0) {
        const uint4* q = (const uint4*)(p + first);
#pragma unroll
        for (int i = 0; i < kNbPer * (int)sizeof(T) / 16; i++) {
            uint4 w = q[i];
            if constexpr (sizeof(T) == 4) {
                v[4 * i] = __uint_as_float(w.x); v[4 * i + 1] = __uint_as_float(w.y);
                v[4 * i + 2] = __uint_as_float(w.z); v[4 * i + 3] = __uint_as_float(w.w);
            } else {
                v[2 * i] = __longlong_as_double((long long)(((unsigned long long)w.y << 32) | w.x));
                v[2 * i + 1] = __longlong_as_double((long long)(((unsigned long long)w.w << 32) | w.z));
            }
        }
    } else {
#pragma unroll
        for (int e = 0; e < kNbPer; e++) v[e] = first + e < n ? p[first + e] : (T)0;
    }
}

template <typename T>
__device__ __forceinline__ void store16(T* p, unsigned long long first, unsigned long long n, const T (&v)[kNbPer]) {
    const bool full = first + kNbPer <= n;
    if (full && ((uintptr_t)(p + first) % 16) == 0) {
        uint4* q = (uint4*)(p + first);
#pragma unroll
        for (int i = 0; i < kNbPer * (int)sizeof(T) / 16; i++) {
            uint4 w;
            if constexpr (sizeof(T) == 4) {
                w = make_uint4(__float_as_uint(v[4 * i]), __float_as_uint(v[4 * i + 1]), __float_as_uint(v[4 * i + 2]),
                               __float_as_uint(v[4 * i + 3]));
            } else {
                unsigned long long a = (unsigned long long)__double_as_longlong(v[2 * i]);
                unsigned long long b = (unsigned long long)__double_as_longlong(v[2 * i + 1]);
                w = make_uint4((uint32_t)a, (uint32_t)(a >> 32), (uint32_t)b, (uint32_t)(b >> 32));
            }
            q[i] = w;
        }
    } else {
#pragma unroll
        for (int e = 0; e < kNbPer; e++)
            if (first + e < n) p[first + e] = v[e];
    }
}

// ------------------------------------------------------------------ encode

struct NbEncArgs {
    const void* x;
    unsigned long long n, ntiles, cap;
    const CodecParams* params;
    uint8_t* out;
    TileStatus32 st;
    unsigned long long* tile_ctr;
    int* err;
    StreamResult* res;
};

// One pass over the input in tiles of kNbTile values taken from an atomic
// counter, one tile ahead.  Per tile T_j: the values (loaded during the
// previous iteration), shifted words and lead codes (one XOR chain over the
// whole array: a thread's first value's predecessor is the previous
// thread's last, or the value before the tile), a CTA scan of the
// stored-byte counts, the tile's byte count published to the look-back, the
// lead codes written to their fixed place, the mid bytes emitted into one of
// three shared staging buffers with byte stores at tile-local offsets.
// T_{j-2} is placed two iterations late, so that the other CTAs' tiles
// claimed before it have normally published their counts: its offset is the
// inclusive prefix of this CTA's previous tile (known here) plus the counts
// of the tiles claimed in between, read from a window of status words copied
// in with cp.async during the emission (a window with unpublished words is
// copied again a few times, then the global look-back takes over); then the
// CTA copies T_{j-2}'s bytes out, realigned.  Two barriers per tile: the
// scan's and the one that hands the placement to the copy-out.
constexpr int kNbWin = 1024;   // status words per placement window (4 KiB)
constexpr int kNbRepolls = 32;

template <typename T>
constexpr int nb_stage_bytes() { return ((kNbTile * (int)sizeof(T) + 48) + 15) / 16 * 16; }

template <typename T>
__global__ void __launch_bounds__(kNbThreads, sizeof(T) == 4 ? 4 : 2) k_nb_encode(NbEncArgs a) {
    using EL = Elem<T>;
    using U = typename EL::U;
    constexpr int W = EL::W;
    extern __shared__ __align__(16) uint8_t nb_dyn[];   // three staging buffers of nb_stage_bytes<T>()
    auto stage = [&](int k) { return nb_dyn + ((unsigned)k % 3u) * nb_stage_bytes<T>(); };
    __shared__ __align__(16) uint32_t s_win[kNbWin + 8];
    __shared__ uint32_t s_sum[8];
    __shared__ long long s_tile[2];
    __shared__ uint32_t s_total[3];
    __shared__ unsigned long long s_base;
    __shared__ int s_skip;
    const T* x = (const T*)a.x;
    const CodecParams P = *a.params;
    // szx/src/szx_float.cc:1514-1535 / szx_double.cc:1615-1636
    bool zm;
    const int reqLength = req_length<T>(P.eb, P.radius, &zm);
    int R, s;
    split_reqlen(reqLength, &R, &s);
    T med;
    if constexpr (sizeof(T) == 4) med = zm ? 0.0f : P.median;
    else med = xf2d(P.median);
    const uint32_t med_stored = zm ? 0u : __float_as_uint(P.median);
    const unsigned long long L = (a.n + 3) / 4;
    uint8_t* lead = a.out + kNbShift + 17;
    uint8_t* mid = lead + L;
    const unsigned long long mid_cap = a.cap - (kNbShift + 17 + L);
    const int lane = threadIdx.x & 31;
    const int low = 8 * (W - R);
    const long long nt = (long long)a.ntiles;
    // warp 0's placement state: anchor tile and its inclusive prefix; window
    long long an_t = -1;
    unsigned long long an_incl = 0;
    long long w_lo = 0;
    int w_ok = 0;
    long long pend_t = -1;   // a tile placed from the window, its inclusive prefix not yet published
    uint32_t pend_agg = 0;
    auto publish = [&]() {
        if (pend_t > 0 && lane == 0) {
            __stcg(&a.st.inc_a[pend_t], an_incl);
            __stcg(&a.st.inc_b[pend_t], 0ull);
            __threadfence();
            st_volatile32(&a.st.st[pend_t], kSt32Inc | (pend_agg & 0x7FFFFFu));
        }
        pend_t = -1;
    };
    // warp 0: copy the status words of the tiles between the anchor and t
    auto win_issue = [&](long long t) {
        w_ok = 0;
        if (an_t >= 0 && an_t < t && t - an_t - 1 <= kNbWin) {
            if (t - an_t == 1) {
                w_ok = 2;
            } else {
                w_lo = (an_t + 1) & ~3ll;
                const int units = (int)((t - w_lo + 3) >> 2);
                for (int u = lane; u < units; u += 32) cp_async16(&s_win[4 * u], a.st.st + w_lo + 4 * u);
                w_ok = 1;
            }
        }
    };
    // warp 0: offset of tile t (count agg), its inclusive prefix published
    auto place = [&](long long t, uint32_t agg) {
        unsigned long long base = 0;
        bool placed = t == 0;
        if (!placed && w_ok == 2) {
            base = an_incl;
            placed = true;
        } else if (!placed && w_ok == 1) {
            const int units = (int)((t - w_lo + 3) >> 2);
            for (int attempt = 0;; attempt++) {
                cp_async_wait_all();
                __syncwarp();
                unsigned long long sum = 0;
                bool ready = true;
                for (long long i = an_t + 1 + lane; i < t; i += 32) {
                    const uint32_t w = s_win[i - w_lo];
                    ready = ready && (w & 0xC0000000u) != 0;
                    sum += w & 0x7FFFFFu;
                }
                if (__all_sync(0xffffffffu, ready)) {
                    base = an_incl + warp_sum(sum);
                    placed = true;
                    break;
                }
                if (attempt == kNbRepolls) break;
                __nanosleep(128);
                for (int u = lane; u < units; u += 32) cp_async16(&s_win[4 * u], a.st.st + w_lo + 4 * u);
            }
        }
        if (!placed) {
            unsigned long long dummy;
            lookback_resolve(a.st, t, agg, 0, &base, &dummy, a.err);   // publishes t's inclusive prefix
        } else if (t > 0) {
            pend_t = t;   // published after the barrier, off the CTA's critical path
            pend_agg = agg;
        }
        an_t = t;
        an_incl = base + agg;
        if (lane == 0) {
            s_base = base;
            const bool ok = base + agg <= mid_cap;
            s_skip = !ok;
            if (!ok) atomicExch(a.err, kErrCapacity);
            if (t == nt - 1) {
                uint8_t* h = a.out + kNbShift;
                h[0] = 1; h[1] = 1; h[2] = 1; h[3] = 0;
                h[4] = (uint8_t)reqLength;
                h[5] = (uint8_t)(med_stored >> 24); h[6] = (uint8_t)(med_stored >> 16);
                h[7] = (uint8_t)(med_stored >> 8); h[8] = (uint8_t)med_stored;
                for (int k = 0; k < 8; k++) h[9 + k] = (uint8_t)(L >> (56 - 8 * k));
                StreamResult r;
                r.offset = kNbShift;
                r.size = 17 + L + base + agg;
                r.nb_const = 0;
                r.eb = P.eb;
                r.status = 0;
                *a.res = r;
            }
        }
    };
    if (threadIdx.x == 0) s_tile[0] = (long long)atomicAdd(a.tile_ctr, 1ull);
    __syncthreads();
    long long tile = s_tile[0];
    long long t1 = -1, t2 = -1;   // T_{j-1}, T_{j-2}: staged, T_{j-2} placed in this iteration
    T v[kNbPer];
    T before = (T)0;     // lane 0: the value before its first one
    auto fetch = [&](long long t) {
        const unsigned long long first = (unsigned long long)t * kNbTile + threadIdx.x * kNbPer;
        load16<T>(x, first, a.n, v);
        before = (lane == 0 && first > 0 && first - 1 < a.n) ? x[first - 1] : (T)0;
    };
    if (tile < nt) fetch(tile);
    int it = 0;
    for (; tile < nt; it++) {
        // the next tile, claimed now and read after the scan's barriers
        if (threadIdx.x == 0) s_tile[(it + 1) & 1] = (long long)atomicAdd(a.tile_ctr, 1ull);
        const unsigned long long first = (unsigned long long)tile * kNbTile + threadIdx.x * kNbPer;
        U cur[kNbPer];
        bool bad = false;
#pragma unroll
        for (int e = 0; e < kNbPer; e++) {
            T d = EL::sub(v[e], med);
            bad |= d != d;
            cur[e] = EL::bits(d) >> s;
        }
        const T dprev = EL::sub(before, med);
        U prev_l0 = first > 0 ? (EL::bits(dprev) >> s) : (U)0;
        if (__any_sync(0xffffffffu, bad || (lane == 0 && first > 0 && dprev != dprev))) {
#pragma unroll
            for (int e = 0; e < kNbPer; e++) cur[e] = EL::bits(xsub(v[e], med)) >> s;
            if (lane == 0 && first > 0) prev_l0 = EL::bits(xsub(before, med)) >> s;
        }
        U prev = __shfl_up_sync(0xffffffffu, cur[kNbPer - 1], 1);
        if (lane == 0) prev = prev_l0;
        uint32_t codes = 0, mine = 0, cnt4[kNbPer / 4];
#pragma unroll
        for (int k = 0; k < kNbPer / 4; k++) {
            uint32_t c4 = 0;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int e = 4 * k + i;
                const U xr = cur[e] ^ (e ? cur[e - 1] : prev);
                int lz;
                if constexpr (sizeof(T) == 4) lz = __clz(xr) >> 3;
                else lz = __clzll((long long)xr) >> 3;
                const int ld = lz < 3 ? lz : 3;
                if (first + e < a.n) {
                    codes |= (uint32_t)ld << (8 * k + 6 - 2 * i);
                    const int c = R - ld;
                    c4 |= (uint32_t)(c > 0 ? c : 0) << (8 * i);
                }
            }
            cnt4[k] = c4;
            mine += (c4 * 0x01010101u) >> 24;
        }
        uint32_t total;
        const uint32_t ex = cta_excl_sum32(mine, &total, s_sum);   // one barrier
        if (threadIdx.x < 32) lookback_publish(a.st, tile, total, 0);
        if (threadIdx.x == 0) s_total[it % 3] = total;
        // T_{j-2}'s window, in flight during the emission
        if (threadIdx.x < 32 && t2 >= 0) win_issue(t2);
        // lead codes: 4 bytes per thread, at their fixed place
        const unsigned long long lb = first >> 2;
        if (lb + 4 <= L && ((uintptr_t)(lead + lb) & 3) == 0) *(uint32_t*)(lead + lb) = codes;
        else
            for (int j = 0; j < 4; j++)
                if (lb + j < L) lead[lb + j] = (uint8_t)(codes >> (8 * j));
        // mid bytes: each value's low (R - lead) bytes of its word shifted down
        // to the stored range, at tile-local offsets (every byte written once)
        uint8_t* stg = stage(it);
        uint32_t q = ex;
#pragma unroll
        for (int k = 0; k < kNbPer / 4; k++) {
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const uint32_t c = byte_of(cnt4[k], i);
                const U ev = cur[4 * k + i] >> low;
#pragma unroll
                for (int j = 0; j < W; j++)
                    if ((uint32_t)j < c) stg[q + j] = (uint8_t)(ev >> (8 * j));
                q += c;
            }
        }
        // the next tile's values are in flight during the placement
        const long long next = s_tile[(it + 1) & 1];
        if (next < nt) fetch(next);
        if (threadIdx.x < 32 && t2 >= 0) place(t2, s_total[(it - 2) % 3]);
        __syncthreads();   // T_j staged; T_{j-2}'s offset known
        if (threadIdx.x < 32) publish();
        if (t2 >= 0 && !s_skip) cta_copy_realign(stage(it - 2), s_total[(it - 2) % 3], mid + s_base);
        // no barrier here: the next writes of T_{j-2}'s buffer (T_{j+1}'s
        // emission), of s_base / s_skip (the next placement) and of s_sum /
        // s_total all come after the next iteration's scan barrier
        t2 = t1;
        t1 = tile;
        tile = next;
    }
    // the CTA's last two tiles, oldest first
    for (int back = 2; back >= 1; back--) {
        const long long t = back == 2 ? t2 : t1;
        if (t < 0) continue;
        __syncthreads();   // the last copy-out has read s_base / s_skip
        if (threadIdx.x < 32) {
            win_issue(t);
            place(t, s_total[(it - back) % 3]);
        }
        __syncthreads();
        if (threadIdx.x < 32) publish();
        if (!s_skip) cta_copy_realign(stage(it - back), s_total[(it - back) % 3], mid + s_base);
    }
}

size_t nonblocked_bound(int dtype, size_t n) {
    size_t es = dtype == 0 ? 4 : 8;
    return kNbShift + 17 + (n + 3) / 4 + es * n + 64;
}

ClearList nonblocked_enc_clear(const Workspace& ws, size_t n) {
    const size_t ntiles = (n + kNbTile - 1) / kNbTile;
    ClearList c{};
    c.p[0] = ws.st32;
    c.bytes[0] = sizeof(uint32_t) * (ntiles + 8);
    c.p[1] = ws.totals;
    c.bytes[1] = kWsHeaderClear;
    c.n = 2;
    return c;
}

cudaError_t launch_nonblocked_encode(int dtype, const void* x, size_t n, uint8_t* d_out, size_t cap,
                                     const Workspace& ws, cudaStream_t s, bool cleared, StreamResult* res_out) {
    if (n == 0 || cap < nonblocked_bound(dtype, n) - 64) return cudaErrorInvalidValue;
    const size_t ntiles = (n + kNbTile - 1) / kNbTile;
    cudaError_t e;
    if (!cleared && (e = launch_ws_clear(nonblocked_enc_clear(ws, n), s)) != cudaSuccess) return e;
    NbEncArgs a;
    a.x = x; a.n = n; a.ntiles = ntiles; a.cap = cap; a.params = ws.params; a.out = d_out;
    a.st = TileStatus32{ws.st32, ws.st_agg2, ws.st_inc2};
    a.tile_ctr = &ws.counters[0];
    a.err = ws.err;
    a.res = res_out ? res_out : ws.result;
    static int per_sm[2][64] = {{0}};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    int& occ = per_sm[dtype == 0 ? 0 : 1][dev];
    const size_t dyn = 3 * (size_t)(dtype == 0 ? nb_stage_bytes<float>() : nb_stage_bytes<double>());
    if (!occ) {
        if (dtype == 0) {
            e = cudaFuncSetAttribute(k_nb_encode<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
            if (e == cudaSuccess)
                e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_nb_encode<float>, kNbThreads, dyn);
        } else {
            e = cudaFuncSetAttribute(k_nb_encode<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
            if (e == cudaSuccess)
                e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_nb_encode<double>, kNbThreads, dyn);
        }
        if (e != cudaSuccess) return e;
        if (occ < 1) occ = 1;
    }
    size_t g = (size_t)sm_count() * occ;
    int grid = (int)(ntiles < g ? ntiles : g);
    {
        TraceScope tr("nonblocked_encode", s);
        if (dtype == 0) k_nb_encode<float><<<grid, kNbThreads, dyn, s>>>(a);
        else k_nb_encode<double><<<grid, kNbThreads, dyn, s>>>(a);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // fold the error word into the result
    return cudaSuccess;
}

// ------------------------------------------------------------------ decode

__global__ void k_nb_parse(const uint8_t* s, unsigned long long len, unsigned long long n, NonBlockedHdr* h,
                           int* err) {
    NonBlockedHdr r = {};
    r.n = n;
    r.ok = 0;
    if (len >= 17 && s[3] == 0) {
        unsigned long long L = 0;
        for (int k = 0; k < 8; k++) L = (L << 8) | s[9 + k];
        r.L = L;
        r.reqLength = s[4];
        r.median = __uint_as_float(((uint32_t)s[5] << 24) | ((uint32_t)s[6] << 16) | ((uint32_t)s[7] << 8) | s[8]);
        r.mid_off = 17 + L;
        r.ok = L == (n + 3) / 4 && r.mid_off <= len && r.reqLength >= 1 && r.reqLength <= 64;
        r.mid_len = r.ok ? len - r.mid_off : 0;
    }
    *h = r;
    *err = r.ok ? kErrNone : kErrStream;
}

__device__ __forceinline__ uint32_t lead_word(const uint8_t* lead, unsigned long long lb, unsigned long long L) {
    uint32_t w = 0;
#pragma unroll
    for (int j = 0; j < 4; j++) w |= (lb + j < L ? (uint32_t)lead[lb + j] : 0u) << (8 * j);
    return w;
}

// Lead codes of 16 values in one 32-bit word (value e at bits 8*(e/4) + 6 -
// 2*(e%4)), as masks with one bit per value: m_k has the low bit of value
// e's pair set when its lead code is <= k, i.e. when its byte lane W-1-k is
// stored.  vorder() moves value e's bit to position 2e+1 (value order).
__device__ __forceinline__ uint32_t vorder(uint32_t m) { return __byte_perm(__brev(m), 0, 0x0123); }

// Valid-value mask (pair low bits) of a word whose first value is `first`.
__device__ __forceinline__ uint32_t valid_pairs(unsigned long long first, unsigned long long n) {
    if (first + 16 <= n) return 0x55555555u;
    uint32_t v = 0;
    for (int e = 0; e < 16; e++)
        if (first + e < n) v |= 1u << (8 * (e >> 2) + 6 - 2 * (e & 3));
    return v;
}

// Lead word of values [first, first + 16): one 4-byte load when aligned.
__device__ __forceinline__ uint32_t lead_word16(const uint8_t* lead, unsigned long long first,
                                                unsigned long long L) {
    const unsigned long long lb = first >> 2;
    if (lb + 4 <= L && ((uintptr_t)(lead + lb) & 3) == 0) return __ldg((const uint32_t*)(lead + lb));
    return lead_word(lead, lb, L);
}

// Per tile (one warp): its mid-byte count (tcnt[t]) and, for each of the top
// three byte lanes, where in the tile's mid bytes the last value storing that
// lane put it (aux[3t+2], 3x21 bits, position+1, 0 = none).  A lane takes the
// tile's 16-code words lane, lane+32, ... so that every load of the warp reads
// 128 consecutive lead bytes; a warp scan per round orders the words.  Counts
// and positions come from population counts of the per-lane masks:
// a value stores max(R - lead, 0) bytes = the number of k < R with lead <= k.
// The CTA's eight tiles form a group: aux[3t] / aux[3t+1] get the tile's
// exclusive prefix within its group (bytes; latest writer tiles, 3x21 bits,
// tile+1), gsum[g] / gwr[g] the group's totals.  Independent per group: no
// look-back.
template <typename T>
__global__ void __launch_bounds__(kNbThreads) k_nb_count(const uint8_t* __restrict__ s, const NonBlockedHdr* hp,
                                                         uint32_t* __restrict__ tcnt,
                                                         unsigned long long* __restrict__ aux,
                                                         unsigned long long* __restrict__ gsum,
                                                         unsigned long long* __restrict__ gwr) {
    constexpr int W = Elem<T>::W;
    constexpr int kTpg = kNbThreads / 32;   // tiles per group
    __shared__ uint32_t s_cnt[kTpg];
    __shared__ unsigned long long s_own[kTpg];
    const NonBlockedHdr h = *hp;
    if (!h.ok) return;
    int R, sft;
    split_reqlen(h.reqLength, &R, &sft);
    if (R > W) return;
    const unsigned long long ntiles = (h.n + kNbTile - 1) / kNbTile;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long tile = (long long)blockIdx.x * kTpg + warp;
    const uint8_t* lead = s + 17;
    const uint32_t full = R > 3 ? (uint32_t)(R - 3) : 0u;   // bytes every value stores below the top three lanes
    uint32_t run = 0;
    int gpos[3] = {-1, -1, -1};
    if (tile < (long long)ntiles) {
#pragma unroll 2
        for (int j = 0; j < kNbTile / (32 * kNbPer); j++) {
            const unsigned long long first =
                (unsigned long long)tile * kNbTile + (unsigned long long)kNbPer * (32 * j + lane);
            const uint32_t codes = lead_word16(lead, first, h.L);
            const uint32_t valid = valid_pairs(first, h.n);
            const uint32_t lo = codes & 0x55555555u, hi = (codes >> 1) & 0x55555555u;
            const uint32_t m0 = ~(lo | hi) & valid, m1 = ~hi & valid, m2 = ~(lo & hi) & valid;
            const uint32_t nv = __popc(valid);
            const uint32_t mine = __popc(m0) + (R >= 2 ? __popc(m1) : 0u) + (R >= 3 ? __popc(m2) : 0u) + full * nv;
            const uint32_t incl = warp_inclusive_sum(mine);
            const uint32_t ex = run + incl - mine;
            const uint32_t v0 = vorder(m0), v1 = vorder(m1), v2 = vorder(m2);
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const uint32_t vk = k == 0 ? v0 : k == 1 ? v1 : v2;
                if (k <= R - 1 && vk) {   // later words hold later positions
                    const int e = (31 - __clz(vk)) >> 1;
                    const uint32_t below = (1u << (2 * e)) - 1;
                    const uint32_t before = __popc(v0 & below) + (R >= 2 ? __popc(v1 & below) : 0u) +
                                            (R >= 3 ? __popc(v2 & below) : 0u) + full * (uint32_t)e;
                    gpos[k] = (int)(ex + before) + (R - 1 - k);
                }
            }
            run += __shfl_sync(0xffffffffu, incl, 31);
        }
    }
    unsigned long long own = 0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        int p = gpos[k];
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) p = max(p, __shfl_xor_sync(0xffffffffu, p, d));
        own |= (unsigned long long)(p + 1) << (21 * k);
    }
    if (lane == 0) {
        s_cnt[warp] = run;
        s_own[warp] = own;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long pa = 0, pb = 0;
        for (int w = 0; w < kTpg; w++) {
            const long long t = (long long)blockIdx.x * kTpg + w;
            if (t >= (long long)ntiles) break;
            const unsigned long long o = s_own[w];
            aux[3 * t] = pa;
            aux[3 * t + 1] = pb;
            aux[3 * t + 2] = o;
            tcnt[t] = s_cnt[w];
            pa += s_cnt[w];
            unsigned long long wr = 0;
#pragma unroll
            for (int k = 0; k < 3; k++)
                if ((o >> (21 * k)) & 0x1FFFFF) wr |= (unsigned long long)(t + 1) << (21 * k);
            pb = Max3x21Op::op(pb, wr);
        }
        gsum[blockIdx.x] = pa;
        gwr[blockIdx.x] = pb;
    }
}

// One CTA: exclusive scan, in place, of the group totals (gsum: bytes, a
// sum; gwr: latest writer tiles, combined by max), over chunks of
// kScanThreads * kScanPer groups carried from chunk to chunk.  A stream
// whose mid bytes run past its end is reported.
constexpr int kScanThreads = 512, kScanPer = 8;

__global__ void __launch_bounds__(kScanThreads) k_nb_scan(const NonBlockedHdr* hp, unsigned long long* gsum,
                                                          unsigned long long* gwr, int* err) {
    __shared__ unsigned long long s_a[kScanThreads / 32], s_b[kScanThreads / 32];
    const NonBlockedHdr h = *hp;
    if (!h.ok) return;
    const unsigned long long ntiles = (h.n + kNbTile - 1) / kNbTile;
    const unsigned long long ng = (ntiles + kNbThreads / 32 - 1) / (kNbThreads / 32);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned long long ca = 0, cb = 0;   // totals of the earlier chunks
    for (unsigned long long c0 = 0; c0 < ng; c0 += (unsigned long long)kScanThreads * kScanPer) {
        const unsigned long long g0 = c0 + (unsigned long long)threadIdx.x * kScanPer;
        unsigned long long va[kScanPer], vb[kScanPer];
        unsigned long long la = 0, lb = 0;
#pragma unroll
        for (int i = 0; i < kScanPer; i++) {
            va[i] = g0 + i < ng ? gsum[g0 + i] : 0ull;
            vb[i] = g0 + i < ng ? gwr[g0 + i] : 0ull;
            la += va[i];
            lb = Max3x21Op::op(lb, vb[i]);
        }
        unsigned long long ia = la, ib = lb;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned long long oa = __shfl_up_sync(0xffffffffu, ia, d);
            const unsigned long long ob = __shfl_up_sync(0xffffffffu, ib, d);
            if (lane >= d) {
                ia += oa;
                ib = Max3x21Op::op(ob, ib);
            }
        }
        if (lane == 31) {
            s_a[warp] = ia;
            s_b[warp] = ib;
        }
        __syncthreads();
        unsigned long long pa = ca, pb = cb, ta = ca, tb = cb;
        for (int w = 0; w < kScanThreads / 32; w++) {
            if (w < warp) {
                pa += s_a[w];
                pb = Max3x21Op::op(pb, s_b[w]);
            }
            ta += s_a[w];
            tb = Max3x21Op::op(tb, s_b[w]);
        }
        unsigned long long ea = __shfl_up_sync(0xffffffffu, ia, 1), eb = __shfl_up_sync(0xffffffffu, ib, 1);
        if (lane == 0) {
            ea = 0;
            eb = 0;
        }
        pa += ea;
        pb = Max3x21Op::op(pb, eb);
#pragma unroll
        for (int i = 0; i < kScanPer; i++) {
            if (g0 + i < ng) {
                gsum[g0 + i] = pa;
                gwr[g0 + i] = pb;
            }
            pa += va[i];
            pb = Max3x21Op::op(pb, vb[i]);
        }
        ca = ta;
        cb = tb;
        __syncthreads();   // s_a / s_b are read before the next chunk writes them
    }
    if (threadIdx.x == 0 && ca > h.mid_len) atomicExch(err, kErrStream);
}

// One thread per tile: the bytes that the top three byte lanes carry into the
// tile (the last earlier value that stored each lane), read from the stream
// and packed into aux[3t+1] (lane W-1-k at bits 8*(2-k)).  A tile's offset is
// its group's prefix (gsum) plus its offset in the group (aux[3t]); each
// thread rewrites only its own tile's aux[3t+1] and reads only the other two
// words of other tiles.
__global__ void k_nb_carry(const uint8_t* __restrict__ s, unsigned long long len, const NonBlockedHdr* hp,
                           unsigned long long* aux, const unsigned long long* __restrict__ gsum,
                           const unsigned long long* __restrict__ gwr) {
    constexpr int kTpg = kNbThreads / 32;
    const NonBlockedHdr h = *hp;
    if (!h.ok) return;
    const unsigned long long ntiles = (h.n + kNbTile - 1) / kNbTile;
    const unsigned long long t = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntiles) return;
    const unsigned long long lw = Max3x21Op::op(gwr[t / kTpg], aux[3 * t + 1]);
    uint32_t carry = 0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const unsigned long long t1 = (lw >> (21 * k)) & 0x1FFFFF;
        if (t1) {
            const unsigned long long u = t1 - 1;
            const unsigned long long p1 = (aux[3 * u + 2] >> (21 * k)) & 0x1FFFFF;
            const unsigned long long pos = h.mid_off + gsum[u / kTpg] + aux[3 * u] + (p1 - 1);
            const uint32_t byte = pos < len ? s[pos] : 0u;
            carry |= byte << (8 * (2 - k));
        }
    }
    aux[3 * t + 1] = carry;
}

// Decode, tiles taken in a fixed order (blockIdx.x, + gridDim.x, ...): a
// tile's offset, carried bytes and byte count are known before it starts, so
// the next tile's lead codes and per-tile words are loaded at the start of an
// iteration and its mid bytes copied with cp.async into the second staging
// buffer while the current tile decodes.
template <typename T>
constexpr int nb_dec_stage_bytes() { return ((kNbTile * (int)sizeof(T) + 48) + 15) / 16 * 16; }

template <typename T>
__global__ void __launch_bounds__(kNbThreads, sizeof(T) == 4 ? 3 : 2)
    k_nb_decode(const uint8_t* __restrict__ s, unsigned long long len, const NonBlockedHdr* hp,
                const uint32_t* __restrict__ tcnt, const unsigned long long* __restrict__ aux,
                const unsigned long long* __restrict__ gsum, T* out) {
    constexpr int kTpg = kNbThreads / 32;
    using EL = Elem<T>;
    using U = typename EL::U;
    constexpr int W = EL::W;
    constexpr int TOPSH = 8 * (W - 3);
    extern __shared__ __align__(16) uint8_t nb_dyn[];   // two staging buffers of nb_dec_stage_bytes<T>()
    __shared__ uint32_t s_sum[8];
    __shared__ uint32_t s_wv[8], s_wm[8];   // per warp: last written top bytes, their byte mask
    const NonBlockedHdr h = *hp;
    if (!h.ok) return;
    int R, sft;
    split_reqlen(h.reqLength, &R, &sft);
    if (R > W) return;
    const long long ntiles = (long long)((h.n + kNbTile - 1) / kNbTile);
    long long tile = blockIdx.x;
    if (tile >= ntiles) return;
    const uint8_t* lead = s + 17;
    const uint8_t* mid = s + h.mid_off;
    const uint8_t* send = s + len;
    const T med = widen_median<T>(h.median);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    auto stage = [&](int k) { return nb_dyn + (k & 1) * nb_dec_stage_bytes<T>(); };
    // the tile's mid bytes [base, base + tot) into staging buffer k, 16-byte
    // chunks by cp.async, a chunk at either end of the stream byte by byte
    auto copy_in = [&](int k, unsigned long long base, uint32_t tot) {
        const uint8_t* src = mid + base;
        const uint32_t sh = (uint32_t)((uintptr_t)src & 15);
        const uint8_t* gbase = src - sh;
        const uint32_t nch = (sh + tot + 15) >> 4;
        uint8_t* stg = stage(k);
        for (uint32_t c = threadIdx.x; c < nch; c += kNbThreads) {
            const uint8_t* lo = gbase + (c << 4);
            if (lo >= s && lo + 16 <= send) cp_async16(stg + (c << 4), lo);
            else
                for (int j = 0; j < 16; j++) stg[(c << 4) + j] = (lo + j >= s && lo + j < send) ? lo[j] : 0;
        }
        cp_async_commit();
    };
    // a tile's words: lead codes (per thread), group prefix + offset in the
    // group, carried bytes, byte count
    auto words = [&](long long t, uint32_t& cd, unsigned long long& ga, unsigned long long& la, uint32_t& cy,
                     uint32_t& tot) {
        cd = lead_word16(lead, (unsigned long long)t * kNbTile + threadIdx.x * kNbPer, h.L);
        ga = gsum[t / kTpg];
        la = aux[3 * t];
        cy = (uint32_t)aux[3 * t + 1];
        tot = tcnt[t];
    };
    const long long G = gridDim.x;
    uint32_t cd0, cy0, tot0, cd1 = 0, cy1 = 0, tot1 = 0;
    unsigned long long ga0, la0, ga1 = 0, la1 = 0;
    words(tile, cd0, ga0, la0, cy0, tot0);
    if (tile + G < ntiles) words(tile + G, cd1, ga1, la1, cy1, tot1);
    copy_in(0, ga0 + la0, tot0);
    const uint32_t full = R > 3 ? (uint32_t)(R - 3) : 0u;
    for (int it = 0;; it++) {
        const bool more = tile + G < ntiles;
        // the words of the tile after next, in flight during this tile
        uint32_t cd2 = 0, cy2 = 0, tot2 = 0;
        unsigned long long ga2 = 0, la2 = 0;
        if (tile + 2 * G < ntiles) words(tile + 2 * G, cd2, ga2, la2, cy2, tot2);
        const uint32_t codes = cd0, carry = cy0;
        const unsigned long long base = ga0 + la0;
        const unsigned long long first = (unsigned long long)tile * kNbTile + threadIdx.x * kNbPer;
        // lanes written by this thread's values: lane W-1-k by a value with lead <= k
        uint32_t mine, sm;
        {
            const uint32_t valid = valid_pairs(first, h.n);
            const uint32_t lo = codes & 0x55555555u, hi = (codes >> 1) & 0x55555555u;
            const uint32_t m0 = ~(lo | hi) & valid, m1 = ~hi & valid, m2 = ~(lo & hi) & valid;
            mine = __popc(m0) + (R >= 2 ? __popc(m1) : 0u) + (R >= 3 ? __popc(m2) : 0u) + full * __popc(valid);
            sm = (m2 ? 0xFFu : 0u) | (m1 ? 0xFF00u : 0u) | (m0 ? 0xFF0000u : 0u);
        }
        uint32_t total;
        const uint32_t ex = cta_excl_sum32(mine, &total, s_sum);   // one barrier
        if (more) copy_in(it + 1, ga1 + la1, tot1);
        else cp_async_commit();   // an empty group: the wait below still means "this tile's copy"
        cp_async_wait_group<1>();
        __syncthreads();   // this tile's bytes are staged
        const uint32_t* buf = (const uint32_t*)stage(it);
        uint32_t q = (uint32_t)((uintptr_t)(mid + base) & 15) + ex;
        // Values past the end of the field (codes 0) are decoded like the
        // others and never stored: they follow every real value, so nothing
        // they change reaches one.
        U sp[kNbPer];
        U prev0 = 0;   // the thread's chain from an all-zero start: its top bytes summarise the thread
#pragma unroll
        for (int e = 0; e < kNbPer; e++) {
            const uint32_t ld = (codes >> (8 * (e >> 2) + 6 - 2 * (e & 3))) & 3;
            const int c0 = R - (int)ld;
            const uint32_t c = c0 > 0 ? (uint32_t)c0 : 0u;
            const uint32_t w0 = buf[q >> 2], w1 = buf[(q >> 2) + 1];
            const uint32_t lo = __funnelshift_r(w0, w1, q << 3);   // the shift wraps: (q & 3) * 8
            // the value's c bytes moved to the top of its R-byte window; the
            // bytes that follow them (the next values') land in the top `ld`
            // bytes, which the chain below takes from the previous value
            if constexpr (sizeof(T) == 4) {
                sp[e] = lo << (8 * (W - R));
            } else {
                const uint32_t w2 = buf[(q >> 2) + 2];
                const uint32_t hi = __funnelshift_r(w1, w2, q << 3);
                sp[e] = (((unsigned long long)hi << 32) | lo) << (8 * (W - R));
            }
            q += c;
            const U inh = ~((~(U)0) >> (8 * ld));   // the top `ld` bytes come from the previous value
            prev0 = (sp[e] & ~inh) | (prev0 & inh);
        }
        // (top bytes, byte mask) pairs: a later pair's masked bytes win,
        // masks accumulate -- one three-input logic op each
        uint32_t sv = (uint32_t)(prev0 >> TOPSH) & 0xFFFFFFu, sw = sm;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t ov = __shfl_up_sync(0xffffffffu, sv, d), ow = __shfl_up_sync(0xffffffffu, sw, d);
            if (lane >= d) {
                sv = (ov & ~sw) | (sv & sw);
                sw |= ow;
            }
        }
        if (lane == 31) {
            s_wv[warp] = sv;
            s_wm[warp] = sw;
        }
        __syncthreads();
        uint32_t pv = carry;   // the carried bytes: all three lanes written before the tile
        for (int w = 0; w < warp; w++) {
            const uint32_t m = s_wm[w];
            pv = (pv & ~m) | (s_wv[w] & m);
        }
        const uint32_t ev = __shfl_up_sync(0xffffffffu, sv, 1), ew = __shfl_up_sync(0xffffffffu, sw, 1);
        if (lane) pv = (pv & ~ew) | (ev & ew);
        U prev = (U)pv << TOPSH;
        T v[kNbPer];
        bool bad = false;
#pragma unroll
        for (int e = 0; e < kNbPer; e++) {
            const uint32_t ld = (codes >> (8 * (e >> 2) + 6 - 2 * (e & 3))) & 3;
            const U inh = ~((~(U)0) >> (8 * ld));
            const U cur = (sp[e] & ~inh) | (prev & inh);
            sp[e] = cur << sft;
            v[e] = EL::add(EL::of(sp[e]), med);
            if constexpr (sizeof(T) != 4) bad |= v[e] != v[e];
            prev = cur;
        }
        if constexpr (sizeof(T) == 4) {   // a NaN anywhere: three-input max with NaN propagation
            float hn = v[0];
#pragma unroll
            for (int e = 1; e + 1 < kNbPer; e += 2) hn = fmax3_nan(hn, v[e], v[e + 1]);
            hn = fmax_nan(hn, v[kNbPer - 1]);
            bad = hn != hn;
        }
        if (__any_sync(0xffffffffu, bad)) {
#pragma unroll
            for (int e = 0; e < kNbPer; e++) v[e] = xadd(EL::of(sp[e]), med);
        }
        store16<T>(out, first, h.n, v);
        if (!more) break;
        // no barrier here: this tile's buffer is next written by the copy
        // issued after the next iteration's scan barrier, s_wsum after the
        // barrier that follows that copy
        tile += G;
        cd0 = cd1; ga0 = ga1; la0 = la1; cy0 = cy1; tot0 = tot1;
        cd1 = cd2; ga1 = ga2; la1 = la2; cy1 = cy2; tot1 = tot2;
    }
    cp_async_wait_all();
}

cudaError_t launch_nonblocked_decode(int dtype, const uint8_t* d_stream, size_t len, size_t n, void* d_out,
                                     const Workspace& ws, cudaStream_t s) {
    if (n == 0) return cudaErrorInvalidValue;
    const size_t ntiles = (n + kNbTile - 1) / kNbTile;
    if (ntiles >= (1u << 21) - 1) return cudaErrorInvalidValue;
    cudaError_t e;
    uint32_t* tcnt = ws.st32;   // [ntiles] tile byte counts
    const size_t ng = (ntiles + kNbThreads / 32 - 1) / (kNbThreads / 32);
    unsigned long long* gsum = ws.st_word;                     // [ng] group byte totals, then prefixes
    unsigned long long* gwr = ws.st_word + ws.status_tiles;    // [ng] group latest writers, then prefixes
    {
        TraceScope tr("nonblocked_parse", s);
        k_nb_parse<<<1, 1, 0, s>>>(d_stream, len, n, ws.nhdr, ws.err);
    }
    {
        TraceScope tr("nonblocked_count", s);
        if (dtype == 0) k_nb_count<float><<<(int)ng, kNbThreads, 0, s>>>(d_stream, ws.nhdr, tcnt, ws.tile_aux, gsum, gwr);
        else k_nb_count<double><<<(int)ng, kNbThreads, 0, s>>>(d_stream, ws.nhdr, tcnt, ws.tile_aux, gsum, gwr);
    }
    {
        TraceScope tr("nonblocked_scan", s);
        k_nb_scan<<<1, kScanThreads, 0, s>>>(ws.nhdr, gsum, gwr, ws.err);
    }
    {
        TraceScope tr("nonblocked_carry", s);
        k_nb_carry<<<(int)((ntiles + 255) / 256), 256, 0, s>>>(d_stream, len, ws.nhdr, ws.tile_aux, gsum, gwr);
    }
    static int per_sm[2][64] = {{0}};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    int& occ = per_sm[dtype == 0 ? 0 : 1][dev];
    const size_t dyn = 2 * (size_t)(dtype == 0 ? nb_dec_stage_bytes<float>() : nb_dec_stage_bytes<double>());
    if (!occ) {
        if (dtype == 0) {
            e = cudaFuncSetAttribute(k_nb_decode<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
            if (e == cudaSuccess)
                e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_nb_decode<float>, kNbThreads, dyn);
        } else {
            e = cudaFuncSetAttribute(k_nb_decode<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
            if (e == cudaSuccess)
                e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_nb_decode<double>, kNbThreads, dyn);
        }
        if (e != cudaSuccess) return e;
        if (occ < 1) occ = 1;
    }
    const size_t g = (size_t)sm_count() * occ;
    const int grid = (int)(ntiles < g ? ntiles : g);
    {
        TraceScope tr("nonblocked_decode", s);
        if (dtype == 0)
            k_nb_decode<float><<<grid, kNbThreads, dyn, s>>>(d_stream, len, ws.nhdr, tcnt, ws.tile_aux, gsum,
                                                             (float*)d_out);
        else
            k_nb_decode<double><<<grid, kNbThreads, dyn, s>>>(d_stream, len, ws.nhdr, tcnt, ws.tile_aux, gsum,
                                                              (double*)d_out);
    }
    return cudaGetLastError();
}

}  // namespace szxg
