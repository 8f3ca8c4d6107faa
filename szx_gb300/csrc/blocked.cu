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
// * Encode is ONE pass over the input.  Persistent CTAs take tiles of blocks
//   from an atomic counter and pipeline them over three shared-memory buffers
//   filled by TMA bulk copies.  A block is handled by a segment of G lanes
//   (16 float / 8 double values per lane) in a chunk-interleaved layout; the
//   tile's payload bytes are placed by a decoupled look-back whose 64-bit
//   status words carry the inclusive prefix inline, and each tile's payloads
//   are emitted into shared memory and written with aligned 16-byte stores.
// * The payload region is written at a fixed position (as if no block were
//   non-constant); the stream then starts 2*nnc (mode 3/4) or 4*nnc (mode 2)
//   bytes into the buffer, so that header, size index, state bits and
//   medians (compacted from per-block scratch by a small look-back kernel) end
//   exactly where the payload region begins.  Nothing is ever moved.
// * Decode scans the size index and the state bits once (payload offsets by
//   non-constant rank, rank at each 32-block state word); then a producer
//   warp per CTA stages each tile's payload range by TMA into a ring of
//   buffers while eight consumer warps decode G lanes per block, with the
//   bytes carried from earlier values resolved by a packed "last writer"
//   scan over 4-value chunks.
#include "common.cuh"
#include "kernels.h"
#include "segment.cuh"

namespace szxg {

// Encoder tiles: ~16 KiB of input per tile, as many warps as the tile has
// block groups (at least 4), 24 warps per SM.  Measured on 512^3 fp32: 8 KiB
// tiles in 4-warp CTAs (6 per SM) encode in 0.396 ms against 0.380 ms -- the
// extra look-backs and tile claims cost more than the extra barrier domains
// save.
constexpr int kEncTileBytes = 16384;
constexpr int kEncWarpsPerSm = 24;
constexpr int kWinRepolls = 32;   // window re-reads before the global look-back walk
constexpr int kIdxThreads = 256;
constexpr int kIdxItems = 8;   // items per thread in the index scans

// ------------------------------------------------------------------ encode
//
// Per-block state a segment keeps in registers from its statistics pass to
// its emission (szx/src/szx_float.cc:49-252 for one block).
// Chunk-round byte totals of a segment are scanned packed, one field per
// round: 8-bit fields for float up to 8 lanes (a round holds at most 8 x 16
// bytes), 16-bit otherwise; in 32 bits whenever they fit.
template <typename T, int G>
struct RoundPack {
    static constexpr int NC = EncCfg<T>::E / 4;
    static constexpr int FB = (sizeof(T) == 4 && G <= 8) ? 8 : 16;
    static constexpr uint32_t MASK = (1u << FB) - 1;
    using P = typename std::conditional<NC * FB <= 32, uint32_t, unsigned long long>::type;
};

template <typename T, int G>
struct BlockEnc {
    using U = typename Elem<T>::U;
    using P = typename RoundPack<T, G>::P;
    static constexpr int E = EncCfg<T>::E;
    static constexpr int NC = E / 4;
    U cur[E];                        // shifted words
    uint32_t cnt4[NC];               // stored bytes of the chunk's 4 values (byte i: value i)
    uint32_t pre4[NC];               // exclusive offsets of those bytes within the chunk
    uint32_t codes;                  // lead byte of chunk round k in byte k
    P excl, tot;                     // per round (packed fields): bytes of earlier lanes, round total
    int state;                       // 0 constant, 1 coded, 2 no block
    int reqLength;
    uint32_t med_bits;               // median as stored (payload or constant list)
    uint32_t size;                   // payload bytes of a coded block
};

struct EncArgs {
    BlkField one;                // the field when nf == 1
    const BlkField* fields;      // nf > 1: device table in ascending enc_tile0
    int nf;
    int bs;
    int omp_stats;               // mode-4 double statistics
    unsigned long long total_tiles;
    unsigned long long* tile_ctr;
    const uint32_t* tile_field;  // nf > 1: field of every launch-wide tile
    int* err;
};

// Statistics pass of one block by a G-lane segment: state, reqLength and
// median (szx/src/szx_float.cc:314-371), the shifted words, lead codes
// (szx/src/szx_float.cc:94-113) and stored-byte counts, all kept in registers.
template <typename T, int G, bool FULL>
__device__ __forceinline__ void enc_block_stats(const T* xs, int len, bool vec, float eb, int eb_exp, int omp_stats,
                                                BlockEnc<T, G>& b) {
    using C = Chunks<T, G>;
    using RP = RoundPack<T, G>;
    using P = typename RP::P;
    using EL = Elem<T>;
    using U = typename EL::U;
    constexpr int E = C::E;
    constexpr int NC = C::NC;
    const int sl = (int)(lane_id() & (G - 1));
    T v[E];
    load_chunks<T, G>(xs, FULL ? G * E : len, vec, v);
    T mn, mx;
    bool special;
    seg_minmax<T, G, FULL>(v, len, mn, mx, special);
    int state;
    float radius_f, median_f;
    if constexpr (sizeof(T) == 4) {
        const float range = xsub(mx, mn);
        radius_f = xhalf(range);
        median_f = xadd(mn, radius_f);
        state = (radius_f <= eb) ? 0 : 1;
    } else if (!omp_stats) {
        // szx/src/szx_double.cc:991-1003: double statistics, float median/radius
        const double range = xsub(mx, mn);
        const double radius = xhalf(range);
        const double median = xadd(mn, radius);
        state = (radius <= (double)eb) ? 0 : 1;
        radius_f = xd2f(radius);
        median_f = xd2f(median);
    } else {
        // computeStateMedianRadius_double2 (szx/src/szx_double.cc:1120-1135)
        const double range = xsub(mx, mn);
        radius_f = xd2f(xhalf(range));
        median_f = xd2f(xadd(mn, xf2d(radius_f)));
        state = (radius_f <= eb) ? 0 : 1;
    }
    bool zm;
    const int reqLength = req_length_e<T>(eb_exp, radius_f, &zm);
    int R, s;
    split_reqlen(reqLength, &R, &s);
    const uint32_t payload_med = zm ? 0u : __float_as_uint(median_f);
    T med;
    if constexpr (sizeof(T) == 4) med = __uint_as_float(payload_med);
    else med = xf2d(median_f);
    // shifted words (szx/src/szx_float.cc:88-92); x86 NaN rules only where a NaN can arise
    if (__any_sync(0xffffffffu, special)) {
#pragma unroll
        for (int e = 0; e < E; e++) b.cur[e] = EL::bits(xsub(v[e], med)) >> s;
    } else {
#pragma unroll
        for (int e = 0; e < E; e++) b.cur[e] = EL::bits(EL::sub(v[e], med)) >> s;
    }
    // lead codes: leading identical bytes with the previous value, capped at 3
    uint32_t ldbs[NC];
    seg_lead_bytes<T, G>(b.cur, ldbs);
    P pk = 0;
    uint32_t codes = 0;
#pragma unroll
    for (int k = 0; k < NC; k++) {
        uint32_t ldb = ldbs[k];
        uint32_t cnt4 = stored_counts(R, ldb);   // max(R - lead, 0) per value
        if constexpr (!FULL) {
            const uint32_t m = low_bytes_mask(len - 4 * (sl + k * G));
            ldb &= m;
            cnt4 &= m;
        }
        b.cnt4[k] = cnt4;
        b.pre4[k] = cnt4 * 0x01010100u;
        pk |= (P)((cnt4 * 0x01010101u) >> 24) << (RP::FB * k);
        codes |= ((ldb * 0x40100401u) >> 24) << (8 * k);   // 4 leads -> one byte, MSB first
    }
    const P incl = seg_inclusive_sum<G>(pk);
    b.tot = __shfl_sync(0xffffffffu, incl, G - 1, G);
    b.excl = incl - pk;
    b.codes = codes;
    uint32_t mid = 0;
#pragma unroll
    for (int k = 0; k < NC; k++) mid += (uint32_t)((b.tot >> (RP::FB * k)) & RP::MASK);
    const int Lb = FULL ? G * NC : (len + 3) / 4;
    b.size = 5 + (uint32_t)Lb + mid;
    b.state = len ? state : 2;
    b.reqLength = reqLength;
    b.med_bits = state == 1 ? payload_med : __float_as_uint(median_f);
}

// Emission of one coded block into the tile's staging buffer: header and lead
// bytes, then each value's stored bytes with predicated byte stores.  Every
// byte of [loc, loc + size) is written exactly once, so the staging buffer
// needs no clearing and no atomics (a value's bytes are contiguous, values
// follow each other without gaps).
template <typename T, int G, bool FULL>
__device__ __forceinline__ void enc_block_emit(uint8_t* stg, uint32_t loc, int len, const BlockEnc<T, G>& b) {
    using RP = RoundPack<T, G>;
    using C = Chunks<T, G>;
    using EL = Elem<T>;
    using U = typename EL::U;
    constexpr int W = EL::W;
    constexpr int NC = C::NC;
    const int sl = (int)(lane_id() & (G - 1));
    uint8_t* p = stg + loc;
    if (sl == 0) {
        p[0] = (uint8_t)b.reqLength;
        p[1] = (uint8_t)(b.med_bits >> 24);
        p[2] = (uint8_t)(b.med_bits >> 16);
        p[3] = (uint8_t)(b.med_bits >> 8);
        p[4] = (uint8_t)b.med_bits;
    }
    const int Lb = FULL ? G * NC : (len + 3) / 4;
    int R, s;
    split_reqlen(b.reqLength, &R, &s);
    (void)s;
    const int low = 8 * (W - R);
    uint32_t before = loc + 5 + (uint32_t)Lb;
#pragma unroll
    for (int k = 0; k < NC; k++) {
        const int c = sl + k * G;
        // lead codes: 4 per byte, MSB first (szx/src/szx_TypeManager.cc:198-273)
        if (FULL || c < Lb) p[5 + c] = (uint8_t)(b.codes >> (8 * k));
        const uint32_t qb = before + (uint32_t)((b.excl >> (RP::FB * k)) & RP::MASK);
        before += (uint32_t)((b.tot >> (RP::FB * k)) & RP::MASK);
        // mid bytes: bytes [W-R .. W-1-lead] of each shifted word, ascending
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const uint32_t n = byte_of(b.cnt4[k], i);
            uint8_t* d = stg + qb + byte_of(b.pre4[k], i);
            const U ev = b.cur[4 * k + i] >> low;
#pragma unroll
            for (int j = 0; j < W; j++)
                if ((uint32_t)j < n) d[j] = (uint8_t)(ev >> (8 * j));
        }
    }
}

template <typename T, int G, int TBYTES = kEncTileBytes>
struct EncTile {
    static constexpr int E = EncCfg<T>::E;
    static constexpr int kBsMax = G * E;                               // largest block of this variant
    static constexpr int kBpw = 32 / G;                                // blocks per warp
    static constexpr int kRaw = TBYTES / (kBsMax * (int)sizeof(T));
    static constexpr int kBlocks = kRaw >= 64 ? 64 : (kRaw < 8 ? 8 : kRaw);   // blocks per tile
    static constexpr int kGroups = kBlocks / kBpw;                     // warps with blocks
    static constexpr int kWarps = kGroups > 4 ? kGroups : 4;
    static constexpr int kThreads = kWarps * 32;
    static constexpr int kMinCtas = kEncWarpsPerSm / kWarps;
    static constexpr int kIn = kBlocks * kBsMax * (int)sizeof(T);      // input bytes per buffer
    static constexpr int kMaxPay = 5 + (kBsMax + 3) / 4 + (int)sizeof(T) * kBsMax;
    // payloads of a tile + slack for the word-wise reads of the realigning copy
    static constexpr int kStage = ((kBlocks * kMaxPay + 32 + 15) / 16) * 16;
    // a ring buffer holds a tile's input, then (in place) its payloads
    static constexpr int kBuf = kIn > kStage ? kIn : kStage;
    static constexpr int kDynSmem = 4 * kBuf;
    static_assert(kGroups <= 8 && kBlocks % kBpw == 0, "one block group per warp");
    static_assert(kBlocks <= 64, "a tile's sizes are scanned as two warp-wide halves");
    static_assert(kBlocks * kMaxPay < 65535, "a tile's byte count + 1 fits the 16-bit aggregate words");
    static_assert(kIn % 16 == 0 && kBuf % 16 == 0, "TMA destinations stay 16-byte aligned");
};

// One pass over the input.  A CTA works through its tiles T_j in a ring of
// four shared-memory buffers; iteration j, between two CTA barriers:
//   TMA load of T_{j+1} (into the buffer T_{j-3} left); warp 0 places T_{j-2}
//   from the look-back window copied in during iteration j-1; statistics of
//   T_j's blocks (registers)  |  barrier  |  window copy for T_{j-1}; every
//   warp scans T_j's block sizes for its own blocks' offsets (warp 0
//   publishes T_j's byte count) and emits them into T_j's buffer in place
//   (its input is dead); copy-out of T_{j-2} to its place in the payload
//   region  |  barrier.
// Every global round trip of a tile -- input load, tile claim, look-back --
// thus has a whole iteration to complete.  Tile ids come from an atomic
// counter, taken in increasing order two tiles ahead (the look-back stays
// deadlock-free with any number of resident CTAs).  The look-back window
// holds the 512 nearest predecessors, which normally reach back to this
// CTA's own previous tile (already placed); otherwise it falls back to the
// global walk.  A segment of G lanes owns one block from its statistics to
// its emission.
template <typename T, int G, bool MULTI, int TBYTES = kEncTileBytes>
__global__ void __launch_bounds__(EncTile<T, G, TBYTES>::kThreads, EncTile<T, G, TBYTES>::kMinCtas)
    k_blocked_encode(EncArgs a) {
    using TL = EncTile<T, G, TBYTES>;
    constexpr int TB = TL::kBlocks;
    constexpr int BPW = TL::kBpw;
    constexpr int NGRP = TB / BPW;
    extern __shared__ __align__(128) uint8_t dsm[];
    __shared__ unsigned long long bar[4];
    __shared__ __align__(16) uint16_t s_w16[2][kLbWin + 8];   // look-back windows (16-bit aggregates)
    __shared__ long long s_an_t, s_wlo[2];                     // placement anchor tile; window first tiles
    __shared__ unsigned long long s_an_incl;                   // the anchor's inclusive prefix
    __shared__ int s_an_f, s_wok[2];                           // its field; window states
    __shared__ uint32_t s_size[4][TB], s_med[4][TB];
    __shared__ uint8_t s_state[4][TB];
    __shared__ uint32_t s_agg[4];
    __shared__ long long s_tile[4];     // launch-wide tile index of each ring position
    __shared__ int s_fld[4];            // its field
    __shared__ unsigned long long s_base;
    __shared__ int s_skip;
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int seg = lane / G, sl = lane & (G - 1);
    const long long nt = (long long)a.total_tiles;
    const unsigned long long tile_elems = (unsigned long long)TB * a.bs;
    const bool vec = ((a.bs * (int)sizeof(T)) & 15) == 0;   // every block starts 16-byte aligned
    // field of a launch-wide tile: one load from the plan's tile map
    auto field_of = [&](long long g) { return (int)a.tile_field[g]; };
    auto buf_ptr = [&](int r) { return dsm + r * TL::kBuf; };
    if (threadIdx.x == 0) {
        for (int r = 0; r < 4; r++) mbar_init(&bar[r], 1);
        mbar_fence_init();
        for (int r = 0; r < 2; r++) {
            s_tile[r] = (long long)atomicAdd(a.tile_ctr, 1ull);
            s_fld[r] = (MULTI && s_tile[r] < nt) ? field_of(s_tile[r]) : 0;
        }
    }
    __syncthreads();
    // a field's members: from the kernel parameters for one field, from the table for a batch
    auto fld = [&](int f) -> const BlkField* { return MULTI ? a.fields + f : nullptr; };
#define FV(F_, m) (MULTI ? (F_)->m : a.one.m)
    uint32_t phase = 0;   // bit r: parity to wait for on ring buffer r

    auto tile_count = [&](const BlkField* F, long long t) {
        const unsigned long long start = (unsigned long long)t * tile_elems;
        const unsigned long long rem = FV(F, n) - start;
        return rem < tile_elems ? rem : tile_elems;
    };
    // all threads: TMA of the 16-byte part by thread 0, the rest by plain copies
    auto issue = [&](long long g, int f, int r) {
        const BlkField* F = fld(f);
        const long long t = g - (long long)FV(F, enc_tile0);
        const T* x = (const T*)FV(F, x);
        const bool tma_ok = ((uintptr_t)x & 15) == 0;
        const unsigned long long cnt = tile_count(F, t);
        const uint32_t bytes = (uint32_t)(cnt * sizeof(T));
        const uint32_t tbytes = tma_ok ? (bytes & ~15u) : 0u;
        T* dst = (T*)buf_ptr(r);
        const T* src = x + (unsigned long long)t * tile_elems;
        if (threadIdx.x == 0 && tbytes) {
            fence_proxy_async();   // the buffer's last generic accesses come before the async write
            mbar_arrive_expect_tx(&bar[r], tbytes);
            tma_load_1d(dst, src, tbytes, &bar[r]);
        }
        for (unsigned long long i = tbytes / sizeof(T) + threadIdx.x; i < cnt; i += TL::kThreads) dst[i] = src[i];
    };
    auto wait_buf = [&](const BlkField* F, long long t, int r) {
        if (((uintptr_t)FV(F, x) & 15) == 0 && ((tile_count(F, t) * sizeof(T)) & ~15ull)) {
            if (!mbar_wait(&bar[r], (phase >> r) & 1u) && threadIdx.x == 0) atomicExch(a.err, kErrLookback);
            phase ^= 1u << r;
        }
    };
    auto block_len = [&](const BlkField* F, long long t, int lb) {
        const unsigned long long b = (unsigned long long)t * TB + lb;
        if (b >= FV(F, nb)) return 0;
        const unsigned long long rem = FV(F, n) - b * (unsigned long long)a.bs;
        return rem < (unsigned long long)a.bs ? (int)rem : a.bs;
    };

    unsigned long long nnc_cta = 0;   // warp 0 lane 0, single field: non-constant blocks of this CTA's tiles
    // Placement (warp 0).  A tile's offset is the inclusive prefix of this
    // CTA's previous tile (the anchor, known here) plus the aggregates of the
    // tiles claimed between the two, read from the field's 16-bit aggregate
    // words: a window of at most kLbWin of them is copied into shared memory
    // an iteration before it is needed.  No anchor in the same field within
    // kLbWin tiles, or an aggregate not yet published, falls back to the
    // global look-back over the 64-bit status words.
    // (the anchor and window state live in shared memory: warp 0 alone uses
    // them, lane 0 writes, and registers stay free for the statistics)
    if (threadIdx.x == 0) {
        s_an_t = -1;
        s_an_f = -1;
        s_an_incl = 0;
    }
    auto agg16_of = [&](const BlkField* F) {
        return (uint16_t*)(FV(F, st_enc) + enc_tile_words(FV(F, nb)));
    };
    auto win_issue = [&](const BlkField* F, int f, long long t, int buf) {
        int ok = 0;
        long long lo = 0;
        const long long an_t = s_an_t;
        if (t > 0 && an_t >= 0 && s_an_f == f && an_t < t && t - an_t - 1 <= kLbWin) {
            if (t - an_t == 1) {
                ok = 2;
            } else {
                lo = (an_t + 1) & ~7ll;
                const int units = (int)((t - lo + 7) >> 3);
                const uint16_t* src = agg16_of(F) + lo;
                for (int u = lane; u < units; u += 32) cp_async16(&s_w16[buf][8 * u], src + 8 * u);
                ok = 1;
            }
        }
        if (lane == 0) {
            s_wlo[buf] = lo;
            s_wok[buf] = ok;
        }
        __syncwarp();
    };
    // warp 0: tile t of field F (metadata set r) placed at `base`: its sizes /
    // medians / state bits by block, the capacity check, the field's totals
    auto meta = [&](const BlkField* F, long long t, int r, unsigned long long base) {
        const uint32_t agg = s_agg[r];
        const bool cap_ok = base + agg <= FV(F, payload_cap);
        const unsigned long long tb0 = (unsigned long long)t * TB;
        uint32_t m01[2];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int lb = lane + 32 * h;
            const bool in = lb < TB;
            const int st = in ? s_state[r][lb] : 2;
            if (in && st != 2) {
                FV(F, size_blk)[tb0 + lb] = (uint16_t)s_size[r][lb];
                FV(F, med_blk)[tb0 + lb] = s_med[r][lb];
            }
            m01[h] = __ballot_sync(0xffffffffu, in && st == 1);
        }
        if (lane == 0) {
            // state bits, MSB first (szx/src/szx_TypeManager.cc:16-40)
            uint8_t* sbp = FV(F, s_scr) + (unsigned long long)t * (TB / 8);
            const uint32_t r0 = __brev(m01[0]), r1 = __brev(m01[1]);
#pragma unroll
            for (int k = 0; k < TB / 8; k++) sbp[k] = (uint8_t)((k < 4 ? r0 : r1) >> (24 - 8 * (k & 3)));
            if (!cap_ok) atomicExch(a.err, kErrCapacity);
            const unsigned long long k = (unsigned long long)(__popc(m01[0]) + __popc(m01[1]));
            if (!MULTI) nnc_cta += k;
            else if (k) atomicAdd(&FV(F, tot)->nnc, k);
            if (t == (long long)FV(F, enc_tiles) - 1) FV(F, tot)->payload_bytes = base + agg;
            s_base = base;
            s_skip = !cap_ok;
        }
    };
    // warp 0: place tile t of field f (metadata set r; its window in buffer buf)
    auto place = [&](const BlkField* F, int f, long long t, int r, int buf) {
        const uint32_t agg = s_agg[r];
        unsigned long long base = 0;
        if (t > 0) {
            const int ok = s_wok[buf];
            const long long lo = s_wlo[buf];
            const long long an_t = s_an_t;
            const unsigned long long an_incl = s_an_incl;
            bool placed = false;
            if (ok == 2) {
                base = an_incl;
                placed = true;
            } else if (ok == 1) {
                // a window with aggregates not yet published is copied again
                // (one round trip each) a few times before the global walk
                const int units = (int)((t - lo + 7) >> 3);
                for (int attempt = 0;; attempt++) {
                    cp_async_wait_all();
                    __syncwarp();
                    unsigned long long sum = 0;
                    bool ready = true;
                    for (long long i = an_t + 1 + lane; i < t; i += 32) {
                        const uint32_t v = s_w16[buf][i - lo];
                        ready = ready && v != 0;
                        sum += v - 1;
                    }
                    if (__all_sync(0xffffffffu, ready)) {
                        base = an_incl + warp_sum(sum);
                        placed = true;
                        break;
                    }
                    if (attempt == kWinRepolls) break;
                    __nanosleep(128);
                    const uint16_t* src = agg16_of(F) + lo;
                    for (int u = lane; u < units; u += 32) cp_async16(&s_w16[buf][8 * u], src + 8 * u);
                }
            }
            if (!placed) base = prefix_resolve(FV(F, st_enc), t, agg, a.err);   // publishes t's inclusive prefix
            else if (lane == 0) st_volatile64(&FV(F, st_enc)[t], kS64Inc | ((base + agg) & kS64Val));
        }
        meta(F, t, r, base);
        if (lane == 0) {
            s_an_t = t;
            s_an_f = f;
            s_an_incl = base + agg;
        }
        __syncwarp();
    };
    auto copy_out = [&](const BlkField* F, int r) {
        if (!s_skip) cta_copy_realign(buf_ptr(r), s_agg[r], FV(F, payload) + s_base);
    };

    if (s_tile[0] < nt) issue(s_tile[0], s_fld[0], 0);
    const bool taker = warp == TL::kWarps - 1 && lane == 0;
    long long t1 = -1, t2 = -1;   // T_{j-1}, T_{j-2} (field-local), -1: none
    int eb_f = -1, eb_exp = 0;    // field whose bound is loaded, the bound's exponent
    float eb = 0.f;
    int f1 = 0, f2 = 0;
    int j = 0;
    for (;; j++) {
        const int r = j & 3;
        __syncthreads();   // ring position j+1 claimed, copy-out of T_{j-3} done
        {
            const int rn = (j + 1) & 3;
            const long long gn = s_tile[rn];
            if (gn < nt) issue(gn, s_fld[rn], rn);
        }
        if (warp == 0 && t2 >= 0) place(fld(f2), f2, t2, (j - 2) & 3, (j - 1) & 1);
        const long long g = s_tile[r];
        if (g >= nt) break;
        const int f = s_fld[r];
        const BlkField* F = fld(f);
        const long long t = g - (long long)FV(F, enc_tile0);
        // the last warp takes the tile of ring position j+2; the reply is used after the statistics
        unsigned long long gc = 0;
        if (taker) gc = atomicAdd(a.tile_ctr, 1ull);
        wait_buf(F, t, r);
        // ---- statistics of the tile's blocks, one block per segment
        const int lb = warp * BPW + seg;
        const bool mine = warp < NGRP;
        // every tile but a field's last holds whole blocks only
        const bool whole = (unsigned long long)(t + 1) * tile_elems <= FV(F, n);
        const int len = !mine ? 0 : (whole ? a.bs : block_len(F, t, lb));
        const bool full = __all_sync(0xffffffffu, len == TL::kBsMax);
        if (f != eb_f) {   // the field's bound and its exponent, once per field
            eb = FV(F, params) ? FV(F, params)->eb : FV(F, eb);
            eb_exp = exponent_f64_of_f32(eb);
            eb_f = f;
        }
        BlockEnc<T, G> b;
        if (mine) {
            const T* xs = (const T*)buf_ptr(r) + (size_t)lb * a.bs;
            if (full) enc_block_stats<T, G, true>(xs, len, vec, eb, eb_exp, a.omp_stats, b);
            else enc_block_stats<T, G, false>(xs, len, vec, eb, eb_exp, a.omp_stats, b);
            if (sl == 0) {
                s_state[r][lb] = (uint8_t)b.state;
                s_size[r][lb] = b.state == 1 ? b.size : 0;
                s_med[r][lb] = b.med_bits;
            }
        }
        if (taker) {
            const int rc = (j + 2) & 3;   // T_{j-2}'s position: its id was read two barriers ago
            s_tile[rc] = (long long)gc;
            s_fld[rc] = (MULTI && (long long)gc < nt) ? field_of((long long)gc) : 0;
        }
        __syncthreads();   // statistics in (T_j's input is dead), T_{j-2} placed
        // warp 0: T_{j-1}'s look-back window, in flight until the next iteration
        if (warp == 0 && t1 >= 0) win_issue(fld(f1), f1, t1, j & 1);
        // every warp: the tile's block offsets (two warp-wide halves)
        const bool in0 = lane < TB;
        const uint32_t sz0 = in0 ? s_size[r][lane] : 0;
        const uint32_t i0 = warp_inclusive_sum(sz0);
        const uint32_t loc_lo = __shfl_sync(0xffffffffu, i0 - sz0, lb & 31);
        uint32_t i1 = i0, loc_hi = 0;   // tiles of up to 32 blocks have no second half
        if constexpr (TB > 32) {
            const bool in1 = lane + 32 < TB;
            const uint32_t sz1 = in1 ? s_size[r][lane + 32] : 0;
            i1 = warp_inclusive_sum(sz1) + __shfl_sync(0xffffffffu, i0, 31);
            loc_hi = __shfl_sync(0xffffffffu, i1 - sz1, lb & 31);
        }
        if (warp == 0) {
            const uint32_t agg = __shfl_sync(0xffffffffu, i1, 31);
            if (lane == 0) {
                s_agg[r] = agg;
                st_relaxed16(agg16_of(F) + t, agg + 1);
            }
            prefix_publish(FV(F, st_enc), t, agg);
        }
        if (mine && b.state == 1) {
            const uint32_t loc = lb < 32 ? loc_lo : loc_hi;
            if (full) enc_block_emit<T, G, true>(buf_ptr(r), loc, len, b);
            else enc_block_emit<T, G, false>(buf_ptr(r), loc, len, b);
        }
        if (t2 >= 0) copy_out(fld(f2), (j - 2) & 3);
        t2 = t1;
        f2 = f1;
        t1 = t;
        f1 = f;
    }
    // this CTA's last two tiles: T_{j-2} was placed at the top of the final
    // iteration, T_{j-1} still needs its window and placement
    if (t2 >= 0) {
        __syncthreads();
        copy_out(fld(f2), (j - 2) & 3);
    }
    if (t1 >= 0) {
        __syncthreads();   // s_base is free again
        if (warp == 0) {
            win_issue(fld(f1), f1, t1, j & 1);
            place(fld(f1), f1, t1, (j - 1) & 3, j & 1);
        }
        __syncthreads();
        copy_out(fld(f1), (j - 1) & 3);
    }
    if (threadIdx.x == 0 && nnc_cta) atomicAdd(&a.one.tot->nnc, nnc_cta);
#undef FV
}

// Header, size index, state bits and medians (szx/src/szx_float.cc:1437-1483).
// The encoder leaves payload sizes and medians by block index; this kernel
// compacts them: an assemble tile covers kAsmWords state words (32 blocks
// each), the non-constant rank of its first block comes from an inline-prefix
// look-back over the tiles' popcounts, and each block then writes its size
// (non-constant, by rank) or its median (constant, by constant rank).
constexpr int kAsmThreads = 256;
constexpr int kAsmWords = (int)(kAsmBlocksPerTile / 32);

struct AsmArgs {
    BlkField one;                // the field when nf == 1
    const BlkField* fields;      // nf > 1: device table in ascending asm_tile0
    int nf;
    int layout;
    unsigned long long bs;
    unsigned long long total_tiles;
    unsigned long long* ctr;     // [0] tile counter, [1] finished CTAs
    int* err;
};

// Header of field F (szx/src/szx_float.cc:1437-1447) and its result record.
__device__ __forceinline__ void asm_header(const BlkField* F, int layout, unsigned long long bs, int status) {
    const unsigned long long nb = F->nb, nnc = F->tot->nnc, nc = nb - nnc, sb = (nb + 7) / 8;
    const bool ra = layout != kBlocked;
    const unsigned long long hdr = ra ? 20 : 13;
    const unsigned long long shift = ra ? 2 * nnc : 4 * nnc;
    uint8_t* s = F->out + shift;
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
    r.size = hdr + (ra ? 2 * nnc : 0) + sb + 4 * nc + F->tot->payload_bytes;
    r.nb_const = nc;
    r.eb = F->params ? F->params->eb : F->eb;
    r.status = status;
    *F->res = r;
}

__global__ void __launch_bounds__(kAsmThreads) k_blocked_assemble(AsmArgs a) {
    __shared__ uint32_t s_word[kAsmWords], s_pre[kAsmWords];
    __shared__ uint32_t s_wsum[kAsmThreads / 32];
    __shared__ long long s_t;
    __shared__ int s_f;
    __shared__ unsigned long long s_base;
    __shared__ int s_last;
    __shared__ BlkField s_one;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const bool ra = a.layout != kBlocked;
    if (tid == 0 && a.nf == 1) s_one = a.one;
    for (;;) {
        if (tid == 0) {
            const long long g = (long long)atomicAdd(a.ctr, 1ull);
            int f = 0;
            if (a.nf > 1 && g < (long long)a.total_tiles) {
                int lo = 0, hi = a.nf - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if ((long long)a.fields[mid].asm_tile0 <= g) lo = mid;
                    else hi = mid - 1;
                }
                f = lo;
            }
            s_t = g;
            s_f = f;
        }
        __syncthreads();
        if (s_t >= (long long)a.total_tiles) break;
        const BlkField* F = a.nf == 1 ? &s_one : a.fields + s_f;
        const long long t = s_t - (long long)F->asm_tile0;
        const unsigned long long nb = F->nb, nnc = F->tot->nnc, sb = (nb + 7) / 8;
        const unsigned long long hdr = ra ? 20 : 13;
        uint8_t* O = F->out + (ra ? 2 * nnc : 4 * nnc) + hdr;
        uint8_t* R = O + (ra ? 2 * nnc : 0);
        uint8_t* M = R + sb;
        const bool o_aligned = ((uintptr_t)O & 1) == 0;
        const unsigned long long nw = (nb + 31) / 32;
        const unsigned long long w = (unsigned long long)t * kAsmWords + tid;
        uint32_t word = 0;
        if (tid < kAsmWords && w < nw) {
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const unsigned long long bi = 4 * w + j;
                const uint32_t byte = bi < sb ? (uint32_t)F->s_scr[bi] : 0u;
                word = (word << 8) | byte;
                if (bi < sb) R[bi] = (uint8_t)byte;
            }
        }
        const uint32_t pc = __popc(word);
        const uint32_t incl = warp_inclusive_sum(pc);
        if (lane == 31) s_wsum[warp] = incl;
        __syncthreads();
        uint32_t wpre = 0, agg = 0;
#pragma unroll
        for (int k = 0; k < kAsmThreads / 32; k++) {
            const uint32_t v = s_wsum[k];
            wpre += k < warp ? v : 0u;
            agg += v;
        }
        if (tid < kAsmWords) {
            s_word[tid] = word;
            s_pre[tid] = wpre + incl - pc;
        }
        if (warp == 0) {
            prefix_publish(F->st_asm, t, agg);
            const unsigned long long base = prefix_resolve(F->st_asm, t, agg, a.err);
            if (lane == 0) s_base = base;
        }
        __syncthreads();
        const unsigned long long base = s_base;
        const unsigned long long b0 = (unsigned long long)t * kAsmWords * 32;
#pragma unroll 4
        for (int k = 0; k < kAsmWords * 32 / kAsmThreads; k++) {
            const int lb = k * kAsmThreads + tid;
            const unsigned long long b = b0 + lb;
            if (b >= nb) break;
            const uint32_t wd = s_word[lb >> 5];
            const int bit = lb & 31;
            const unsigned long long rank = base + s_pre[lb >> 5] + (bit ? __popc(wd >> (32 - bit)) : 0);
            if ((wd >> (31 - bit)) & 1u) {
                if (ra) {
                    const uint16_t v = F->size_blk[b];
                    if (o_aligned) {
                        *(uint16_t*)(O + 2 * rank) = v;   // little-endian u16
                    } else {
                        O[2 * rank] = (uint8_t)v;
                        O[2 * rank + 1] = (uint8_t)(v >> 8);
                    }
                }
            } else {
                const uint32_t v = F->med_blk[b];
                uint8_t* q = M + 4 * (b - rank);
                if (a.layout == kRandomAccessNative) {
                    q[0] = (uint8_t)v; q[1] = (uint8_t)(v >> 8); q[2] = (uint8_t)(v >> 16); q[3] = (uint8_t)(v >> 24);
                } else {
                    q[0] = (uint8_t)(v >> 24); q[1] = (uint8_t)(v >> 16); q[2] = (uint8_t)(v >> 8); q[3] = (uint8_t)v;
                }
            }
        }
        __syncthreads();
    }
    // the last CTA to finish writes every field's header and result record
    if (tid == 0) {
        __threadfence();
        s_last = atomicAdd(&a.ctr[1], 1ull) == (unsigned long long)gridDim.x - 1;
    }
    __syncthreads();
    if (s_last) {
        __threadfence();
        const int status = *(volatile int*)a.err;
        for (int f = tid; f < a.nf; f += kAsmThreads) asm_header(a.nf == 1 ? &s_one : a.fields + f, a.layout, a.bs, status);
    }
}

size_t blocked_bound(int layout, int dtype, size_t n, int bs) {
    size_t es = dtype == 0 ? 4 : 8;
    size_t nb = (n + bs - 1) / bs, sb = (nb + 7) / 8;
    size_t hdr = layout == kBlocked ? 13 : 20;
    return hdr + sb + 4 * nb + nb * (5 + ((size_t)bs + 3) / 4) + es * n + 64;
}

// ctas_per_sm: 0 as many as fit, else at most that many.
template <typename T, int G, int TBYTES = kEncTileBytes>
static cudaError_t run_encode(EncArgs a, int ctas_per_sm, cudaStream_t s) {
    using TL = EncTile<T, G, TBYTES>;
    static bool attr_set[64] = {false};
    static int per_sm[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (!attr_set[dev]) {
        // the ring needs the largest shared-memory carveout for 3 CTAs per SM
        cudaError_t e = cudaSuccess;
        for (auto k : {k_blocked_encode<T, G, false, TBYTES>, k_blocked_encode<T, G, true, TBYTES>}) {
            if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, TL::kDynSmem);
            if (e == cudaSuccess)
                e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
        }
        int occ = 0;
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_blocked_encode<T, G, false, TBYTES>,
                                                              TL::kThreads, TL::kDynSmem);
        if (e != cudaSuccess) return e;
        per_sm[dev] = occ < 1 ? 1 : occ;
        attr_set[dev] = true;
    }
    const int cps = ctas_per_sm > 0 && ctas_per_sm < per_sm[dev] ? ctas_per_sm : per_sm[dev];
    const size_t g = (size_t)sm_count() * cps;
    const int grid = (int)(a.total_tiles < g ? a.total_tiles : g);
    TraceScope tr("blocked_encode", s);
    if (a.nf > 1) k_blocked_encode<T, G, true, TBYTES><<<grid, TL::kThreads, TL::kDynSmem, s>>>(a);
    else k_blocked_encode<T, G, false, TBYTES><<<grid, TL::kThreads, TL::kDynSmem, s>>>(a);
    return cudaGetLastError();
}
// The one encoder tile variant a launch shape can pick besides the default:
// 8 KiB tiles (16 blocks, 4 warps, 6 CTAs per SM) for float blocks of 65..128
// values.
constexpr int kEncTileBytesSmall = 8192;

static int lanes_for_bs(int dtype, int bs) {
    const int per = dtype == 0 ? 16 : 8;   // values per lane
    const int need = (bs + per - 1) / per;
    return need <= 1 ? 1 : need <= 2 ? 2 : need <= 4 ? 4 : need <= 8 ? 8 : need <= 16 ? 16 : 32;
}

int blocked_tile_blocks(int dtype, int bs, int tile_variant) {
    const int G = lanes_for_bs(dtype, bs);
    if (tile_variant == 1 && dtype == 0 && G == 8) return EncTile<float, 8, kEncTileBytesSmall>::kBlocks;
    if (dtype == 0) {
        switch (G) {
            case 1: return EncTile<float, 1>::kBlocks;
            case 2: return EncTile<float, 2>::kBlocks;
            case 4: return EncTile<float, 4>::kBlocks;
            case 8: return EncTile<float, 8>::kBlocks;
            default: return EncTile<float, 16>::kBlocks;
        }
    }
    switch (G) {
        case 1: return EncTile<double, 1>::kBlocks;
        case 2: return EncTile<double, 2>::kBlocks;
        case 4: return EncTile<double, 4>::kBlocks;
        case 8: return EncTile<double, 8>::kBlocks;
        case 16: return EncTile<double, 16>::kBlocks;
        default: return EncTile<double, 32>::kBlocks;
    }
}

cudaError_t launch_blocked_encode_fields(int layout, int dtype, int bs, int nf, const BlkField& one,
                                         const BlkField* d_fields, const uint32_t* d_tile_field,
                                         unsigned long long enc_total, unsigned long long asm_total,
                                         unsigned long long* counters, int* err, cudaStream_t s,
                                         const LaunchShape& shape) {
    if (nf < 1 || enc_total == 0 || (nf > 1 && !d_tile_field)) return cudaErrorInvalidValue;
    EncArgs a;
    a.one = one;
    a.fields = d_fields;
    a.nf = nf;
    a.bs = bs;
    a.omp_stats = layout == kRandomAccessNative;
    a.total_tiles = enc_total;
    a.tile_ctr = &counters[0];
    a.tile_field = d_tile_field;
    a.err = err;
    cudaError_t e;
    const int G = lanes_for_bs(dtype, bs);
    if (dtype == 0) {
        switch (G) {
            case 1: e = run_encode<float, 1>(a, shape.enc_ctas_per_sm, s); break;
            case 2: e = run_encode<float, 2>(a, shape.enc_ctas_per_sm, s); break;
            case 4: e = run_encode<float, 4>(a, shape.enc_ctas_per_sm, s); break;
            case 8:
                e = shape.enc_tile_variant == 1
                        ? run_encode<float, 8, kEncTileBytesSmall>(a, shape.enc_ctas_per_sm, s)
                        : run_encode<float, 8>(a, shape.enc_ctas_per_sm, s);
                break;
            default: e = run_encode<float, 16>(a, shape.enc_ctas_per_sm, s); break;
        }
    } else {
        switch (G) {
            case 1: e = run_encode<double, 1>(a, shape.enc_ctas_per_sm, s); break;
            case 2: e = run_encode<double, 2>(a, shape.enc_ctas_per_sm, s); break;
            case 4: e = run_encode<double, 4>(a, shape.enc_ctas_per_sm, s); break;
            case 8: e = run_encode<double, 8>(a, shape.enc_ctas_per_sm, s); break;
            case 16: e = run_encode<double, 16>(a, shape.enc_ctas_per_sm, s); break;
            default: e = run_encode<double, 32>(a, shape.enc_ctas_per_sm, s); break;
        }
    }
    if (e != cudaSuccess) return e;
    AsmArgs m;
    m.one = one;
    m.fields = d_fields;
    m.nf = nf;
    m.layout = layout;
    m.bs = (unsigned long long)bs;
    m.total_tiles = asm_total;
    m.ctr = &counters[1];
    m.err = err;
    const size_t gmax = (size_t)sm_count() * 4;
    const int ag = (int)(asm_total < gmax ? (asm_total ? asm_total : 1) : gmax);
    TraceScope tr("blocked_assemble", s);
    k_blocked_assemble<<<ag, kAsmThreads, 0, s>>>(m);
    return cudaGetLastError();
}

ClearList blocked_enc_clear(const Workspace& ws, size_t nb) {
    ClearList c{};
    c.p[0] = ws.st_word;
    c.bytes[0] = 8 * blocked_status_words(nb);
    c.p[1] = ws.totals;
    c.bytes[1] = kWsHeaderClear;
    c.n = 2;
    return c;
}

cudaError_t launch_blocked_encode(int layout, int dtype, const void* x, size_t n, int bs, bool use_params,
                                  float abs_eb, uint8_t* d_out, size_t cap, const Workspace& ws, cudaStream_t s,
                                  bool cleared, StreamResult* res_out) {
    if (n == 0 || bs < 1 || bs > 256) return cudaErrorInvalidValue;
    if (layout == kBlocked && bs > 255) return cudaErrorInvalidValue;
    const size_t nb = (n + bs - 1) / bs, sb = (nb + 7) / 8;
    const size_t hdr = layout == kBlocked ? 13 : 20;
    const size_t qfix = hdr + sb + 4 * nb;
    if (cap < qfix) return cudaErrorInvalidValue;
    cudaError_t e;
    // status words of both look-backs, then totals / result / error / counters
    if (!cleared && (e = launch_ws_clear(blocked_enc_clear(ws, nb), s)) != cudaSuccess) return e;
    const size_t tb = (size_t)blocked_tile_blocks(dtype, bs, 0);
    BlkField F;
    F.x = x; F.n = n; F.nb = nb;
    F.enc_tiles = (nb + tb - 1) / tb; F.enc_tile0 = 0;
    F.asm_tiles = (nb + kAsmBlocksPerTile - 1) / kAsmBlocksPerTile; F.asm_tile0 = 0;
    F.eb = abs_eb; F.pad = 0;
    F.params = use_params ? ws.params : nullptr;
    F.out = d_out;
    F.payload = d_out + qfix;
    F.payload_cap = cap - qfix;
    F.st_enc = ws.st_word;
    F.st_asm = ws.st_word + enc_status_words(nb);   // encoder's words first
    F.size_blk = ws.o_scr; F.med_blk = ws.m_scr; F.s_scr = ws.s_scr;
    F.tot = ws.totals;
    F.res = res_out ? res_out : ws.result;
    return launch_blocked_encode_fields(layout, dtype, bs, 1, F, nullptr, nullptr, F.enc_tiles, F.asm_tiles,
                                        ws.counters, ws.err, s, LaunchShape{});
}

// ------------------------------------------------------------------ decode

__device__ __forceinline__ unsigned long long be64(const uint8_t* p) {
    unsigned long long v = 0;
    for (int i = 0; i < 8; i++) v = (v << 8) | p[i];
    return v;
}

// Parse and validate the mode-3/4 header (szx/src/szxd_float.cc:402-434).
__device__ BlockedHdr parse_blocked(const uint8_t* s, unsigned long long len, unsigned long long n,
                                    unsigned long long bs_expect) {
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
    return r;
}

__global__ void k_blocked_parse(const uint8_t* s, unsigned long long len, unsigned long long n,
                                unsigned long long bs_expect, BlockedHdr* h, int* err) {
    const BlockedHdr r = parse_blocked(s, len, n, bs_expect);
    *h = r;
    *err = r.ok ? kErrNone : kErrStream;
}

// Every stream of a batch: one thread per field.
__global__ void k_blocked_parse_fields(const DecField* F, int nf, unsigned long long bs) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const DecField& D = F[f];
    const BlockedHdr r = parse_blocked(D.s, D.len, D.n, bs);
    *D.hdr = r;
    if (!r.ok) *D.err = kErrStream;
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

// Two independent exclusive scans:
//   family A: payload offsets  P[k] = sum O[0..k)          (k < nnc)
//   family B: rank words       RW[w] = popcount(state < 32w) (w < ceil(nb/32))
// One tile (kIdxPerTile items) of either, by the whole CTA.
__device__ __forceinline__ void index_tile(const uint8_t* s, const BlockedHdr& h, unsigned long long* P, uint32_t* RW,
                                           TileStatus st, bool famA, long long lt, unsigned long long len, int* err,
                                           unsigned long long* sm, unsigned long long* s_base) {
    static_assert((unsigned long long)kIdxThreads * kIdxItems == kIdxPerTile, "index tile size");
    const unsigned long long nw = (h.nb + 31) / 32;
    const unsigned long long first = (unsigned long long)lt * kIdxPerTile + threadIdx.x * kIdxItems;
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
        lookback(st, lt, tot, 0, &ba, &bb, err);
        if (threadIdx.x == 0) *s_base = ba;
    }
    __syncthreads();
    unsigned long long run = *s_base + ex;
#pragma unroll
    for (int i = 0; i < kIdxItems; i++) {
        unsigned long long k = first + i;
        if (famA) {
            if (k < h.nnc) P[k] = run;
            if (k == h.nnc - 1) {
                P[h.nnc] = run + vals[i];
                if (h.q_off + run + vals[i] > len) atomicExch(err, kErrStream);
            }
        } else if (k < nw) {
            RW[k] = (uint32_t)run;
        }
        run += vals[i];
    }
    __syncthreads();
}

// The scans of one stream in one persistent launch (family A first).
__global__ void __launch_bounds__(kIdxThreads) k_blocked_index(const uint8_t* s, const BlockedHdr* hp,
                                                               unsigned long long* P, uint32_t* RW,
                                                               TileStatus stA, TileStatus stB,
                                                               unsigned long long* ctr, int* err,
                                                               unsigned long long len, int famA) {
    __shared__ unsigned long long sm[8];
    __shared__ long long s_tile;
    __shared__ unsigned long long s_base;
    const BlockedHdr h = *hp;
    if (!h.ok) return;
    const unsigned long long nw = (h.nb + 31) / 32;
    const long long TA = famA ? (long long)((h.nnc + kIdxPerTile - 1) / kIdxPerTile) : 0;   // no size index in fastMode 2
    const long long TBt = (long long)((nw + kIdxPerTile - 1) / kIdxPerTile);
    for (;;) {
        if (threadIdx.x == 0) s_tile = (long long)atomicAdd(ctr, 1ull);
        __syncthreads();
        long long t = s_tile;
        if (t >= TA + TBt) break;
        const bool fa = t < TA;
        index_tile(s, h, P, RW, fa ? stA : stB, fa, fa ? t : t - TA, len, err, sm, &s_base);
    }
}

// The scans of every stream of a batch: tiles in field order (each field's
// offset tiles, then its rank tiles) from one counter; a field whose header
// failed, and offset tiles past a field's real nnc, do nothing.
__global__ void __launch_bounds__(kIdxThreads) k_blocked_index_fields(const DecField* F, int nf,
                                                                      unsigned long long total,
                                                                      unsigned long long* ctr) {
    __shared__ unsigned long long sm[8];
    __shared__ long long s_tile;
    __shared__ int s_f;
    __shared__ unsigned long long s_base;
    for (;;) {
        if (threadIdx.x == 0) {
            const long long g = (long long)atomicAdd(ctr, 1ull);
            int lo = 0, hi = nf - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if ((long long)F[mid].idx_tile0 <= g) lo = mid;
                else hi = mid - 1;
            }
            s_tile = g;
            s_f = lo;
        }
        __syncthreads();
        const long long g = s_tile;
        if (g >= (long long)total) break;
        const DecField& D = F[s_f];
        const BlockedHdr h = *D.hdr;
        const long long local = g - (long long)D.idx_tile0;
        const bool fa = local < (long long)D.idxA_tiles;
        const long long lt = fa ? local : local - (long long)D.idxA_tiles;
        const long long TA = (long long)((h.nnc + kIdxPerTile - 1) / kIdxPerTile);
        if (h.ok && (!fa || lt < TA)) {
            const TileStatus st = fa ? TileStatus{D.stA[0], D.stA[1], D.stA[2]} : TileStatus{D.stB[0], D.stB[1], D.stB[2]};
            index_tile(D.s, h, D.P, D.RW, st, fa, lt, D.len, D.err, sm, &s_base);
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ decode, per block
//
// A segment of G lanes decodes one non-constant block with the encoder's
// chunk layout: lane sl owns the 4-value chunks sl, sl+G, sl+2G, ... (chunk c
// = lead byte c of the payload).  Stored bytes are read from the staged
// payload in shared memory; every value is first rebuilt with a zero carry
// (its top `lead` bytes come from its predecessor, szx/src/szxd_float.cc:
// 431-470), then the bytes still inherited from before the chunk are filled in
// from a "last writer" scan over chunk summaries in block order.

// Chunk summary: [25:24] the smallest lead in the chunk (it wrote the top-3
// bytes at indices >= that lead), [23:0] the top three bytes of its last value.
__device__ __forceinline__ uint32_t lw_op(uint32_t a, uint32_t b) {
    const uint32_t ma = a >> 24, mb = b >> 24;
    const uint32_t mask = 0xFFFFFFu >> (8 * mb);
    return ((ma < mb ? ma : mb) << 24) | (a & 0xFFFFFFu & ~mask) | (b & mask);
}
constexpr uint32_t kLwNone = 3u << 24;   // writes nothing; the value before a block is zero

// Lead-byte tables (a lead byte holds 4 codes, MSB first): the four leads as
// bytes (value 0 in byte 0), and their running minimum from a start of 3
// (the byte lanes a value still inherits from before its chunk).
__device__ __forceinline__ void lead_tables_init(uint32_t* lut_ld, uint32_t* lut_cm) {
    for (int c = threadIdx.x; c < 256; c += blockDim.x) {
        uint32_t ldb = 0, cmb = 0, m = 3;
        for (int i = 0; i < 4; i++) {
            const uint32_t ld = (c >> (6 - 2 * i)) & 3;
            m = ld < m ? ld : m;
            ldb |= ld << (8 * i);
            cmb |= m << (8 * i);
        }
        lut_ld[c] = ldb;
        lut_cm[c] = cmb;
    }
}

// FULL: every segment of the warp decodes a whole block of G*E values (no
// range checks); otherwise values at or past len are ignored.
template <typename T, int G, bool FULL>
__device__ __forceinline__ void dec_segment(const uint8_t* p, int len, T* ob, bool vec, const uint32_t* lut_ld,
                                            const uint32_t* lut_cm) {
    using C = Chunks<T, G>;
    using EL = Elem<T>;
    using U = typename EL::U;
    constexpr int W = EL::W;
    constexpr int E = C::E;
    constexpr int NC = C::NC;
    constexpr int TOPSH = 8 * (W - 3);
    const int sl = (int)(lane_id() & (G - 1));
    const int reqLength = p[0];
    const uint32_t mb = ((uint32_t)p[1] << 24) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 8) | p[4];
    int R, s;
    split_reqlen(reqLength, &R, &s);
    R = R < 1 ? 1 : (R > W ? W : R);   // a no-op for valid streams; keeps the shifts defined otherwise
    const int low = 8 * (W - R);
    const int Lb = FULL ? G * NC : (len + 3) / 4;
    // per chunk: leads, running minima, stored-byte counts and their offsets (bytes of a word)
    uint32_t ldb[NC], cmb[NC], pre[NC];
    unsigned long long pk = 0;
#pragma unroll
    for (int k = 0; k < NC; k++) {
        const int c = sl + k * G;
        const uint32_t code = (FULL || c < Lb) ? (uint32_t)p[5 + c] : 0u;
        ldb[k] = lut_ld[code];
        cmb[k] = lut_cm[code];
        uint32_t cnt4 = stored_counts(R, ldb[k]);   // max(R - lead, 0) per value
        if constexpr (!FULL) {
            const int nin = len - 4 * c;
            cnt4 &= nin >= 4 ? 0xFFFFFFFFu : (nin <= 0 ? 0u : 0xFFFFFFFFu >> (32 - 8 * nin));
        }
        pre[k] = cnt4 * 0x01010100u;   // byte i: bytes of values 0..i-1
        pk |= (unsigned long long)((cnt4 * 0x01010101u) >> 24) << (16 * k);
    }
    const unsigned long long incl = seg_inclusive_sum<G>(pk);
    const unsigned long long tot = __shfl_sync(0xffffffffu, incl, G - 1, G);
    const unsigned long long excl = incl - pk;
    const uint32_t ph = (uint32_t)((uintptr_t)p & 15);
    const uint32_t* buf = (const uint32_t*)(p - ph);
    U cur[E];
    uint32_t sum[NC];
    uint32_t before = ph + 5 + (uint32_t)Lb;
#pragma unroll
    for (int k = 0; k < NC; k++) {
        const uint32_t qb = before + (uint32_t)((excl >> (16 * k)) & 0xFFFF);
        before += (uint32_t)((tot >> (16 * k)) & 0xFFFF);
        const uint32_t ld8 = ldb[k] << 3;
        U run = 0;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const uint32_t q = qb + byte_of(pre[k], i);
            const uint32_t* wp = buf + (q >> 2);
            const uint32_t w0 = wp[0], w1 = wp[1];
            const uint32_t inh = top_bytes_mask(byte_of(ld8, i));   // top lead bytes: from the predecessor
            // stored bytes land at [W-R, W-lead); the bytes above them are inherited
            if constexpr (sizeof(T) == 4) {
                const uint32_t sp = __funnelshift_r(w0, w1, q << 3) << low;
                run = (run & inh) | (sp & ~inh);
            } else {
                const uint32_t w2 = wp[2];
                const uint32_t lo = __funnelshift_r(w0, w1, q << 3), hi = __funnelshift_r(w1, w2, q << 3);
                const unsigned long long sp = (((unsigned long long)hi << 32) | lo) << low;
                const unsigned long long ih = (unsigned long long)inh << 32;
                run = (run & ih) | (sp & ~ih);
            }
            cur[4 * k + i] = run;
        }
        sum[k] = (byte_of(cmb[k], 3) << 24) | ((uint32_t)(run >> TOPSH) & 0xFFFFFFu);
    }
    // last-writer scans: one per chunk round (independent), then the round carries
    uint32_t inc[NC];
#pragma unroll
    for (int k = 0; k < NC; k++) inc[k] = sum[k];
#pragma unroll
    for (int d = 1; d < G; d <<= 1) {
#pragma unroll
        for (int k = 0; k < NC; k++) {
            const uint32_t o = __shfl_up_sync(0xffffffffu, inc[k], d, G);
            if (sl >= d) inc[k] = lw_op(o, inc[k]);
        }
    }
    uint32_t carry_in = kLwNone;
    const T med = widen_median<T>(__uint_as_float(mb));
    T v[E];
    bool bad = false;
#pragma unroll
    for (int k = 0; k < NC; k++) {
        uint32_t ex = __shfl_up_sync(0xffffffffu, inc[k], 1, G);
        if (sl == 0) ex = kLwNone;
        const uint32_t fin = lw_op(carry_in, ex);
        carry_in = lw_op(carry_in, __shfl_sync(0xffffffffu, inc[k], G - 1, G));
        const uint32_t carry = (fin & 0xFFFFFFu) << 8;   // top three bytes of a 32-bit word
        const uint32_t cm8 = cmb[k] << 3;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const uint32_t keep = top_bytes_mask(byte_of(cm8, i));   // byte lanes inherited from before the chunk
            U u = cur[4 * k + i];
            if constexpr (sizeof(T) == 4) u |= carry & keep;
            else u |= (unsigned long long)(carry & keep) << 32;
            u <<= s;
            cur[4 * k + i] = u;
            v[4 * k + i] = EL::add(EL::of(u), med);
            bad |= v[4 * k + i] != v[4 * k + i];
        }
    }
    if (__any_sync(0xffffffffu, bad)) {
#pragma unroll
        for (int e = 0; e < E; e++) v[e] = xadd(EL::of(cur[e]), med);
    }
    store_chunks<T, G>(ob, len, vec, v);
}

// Consecutive layout: lane sl of the segment decodes the E consecutive values
// [E*sl, E*sl + E) of the block (chunks NC*sl .. NC*sl + NC-1).  Each value is
// rebuilt in order with one running word per lane, so inheritance from
// earlier values of the same lane (szx/src/szxd_float.cc:431-470: the top
// `lead` bytes come from the predecessor) is resolved as it goes; only the
// bytes inherited from before the lane's first value are unknown, and one
// "last writer" scan over the G lane summaries per block supplies them.
// 32-byte stores (sm_100 and later): a lane's 8 floats / 4 doubles at a
// 32-byte aligned address, so that lanes writing consecutive 64-byte runs fill
// whole 32-byte sectors.
__device__ __forceinline__ void st_v8(float* p, const float* v) {
    asm volatile("st.global.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(p), "f"(v[0]), "f"(v[1]), "f"(v[2]),
                 "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7])
                 : "memory");
}
__device__ __forceinline__ void st_v8(double* p, const double* v) {
    asm volatile("st.global.v4.f64 [%0], {%1,%2,%3,%4};" ::"l"(p), "d"(v[0]), "d"(v[1]), "d"(v[2]), "d"(v[3])
                 : "memory");
}

// vec: 0 scalar stores, 1 16-byte stores, 2 32-byte stores (the output's
// alignment and the block's byte size allow them).
template <typename T, int G, bool FULL>
__device__ __forceinline__ void dec_segment_seq(const uint8_t* p, int len, T* ob, int vec, const uint32_t* lut_ld,
                                                const uint32_t* lut_cm) {
    using EL = Elem<T>;
    using U = typename EL::U;
    constexpr int W = EL::W;
    constexpr int E = EncCfg<T>::E;
    constexpr int NC = E / 4;
    constexpr int TOPSH = 8 * (W - 3);
    const int sl = (int)(lane_id() & (G - 1));
    const int reqLength = p[0];
    const uint32_t mb = ((uint32_t)p[1] << 24) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 8) | p[4];
    int R, s;
    split_reqlen(reqLength, &R, &s);
    R = R < 1 ? 1 : (R > W ? W : R);   // a no-op for valid streams; keeps the shifts defined otherwise
    const int low = 8 * (W - R);
    const int Lb = FULL ? G * NC : (len + 3) / 4;
    const int c0 = sl * NC;            // the lane's first chunk
    uint32_t ldb[NC], cmb[NC], cnt[NC];
    uint32_t mine = 0;
#pragma unroll
    for (int k = 0; k < NC; k++) {
        const int c = c0 + k;
        const uint32_t code = (FULL || c < Lb) ? (uint32_t)p[5 + c] : 0u;
        ldb[k] = lut_ld[code];
        cmb[k] = lut_cm[code];
        uint32_t cnt4 = stored_counts(R, ldb[k]);   // max(R - lead, 0) per value
        if constexpr (!FULL) {
            const int nin = len - 4 * c;
            cnt4 &= nin >= 4 ? 0xFFFFFFFFu : (nin <= 0 ? 0u : 0xFFFFFFFFu >> (32 - 8 * nin));
        }
        cnt[k] = cnt4;
        mine += (cnt4 * 0x01010101u) >> 24;
    }
    const uint32_t incl = seg_inclusive_sum<G>(mine);
    const uint32_t ph = (uint32_t)((uintptr_t)p & 15);
    const uint32_t* buf = (const uint32_t*)(p - ph);
    uint32_t q = ph + 5 + (uint32_t)Lb + incl - mine;
    U cur[E];
    U run = 0;
    uint32_t mlead = 3;   // smallest lead so far in the lane: its top bytes still come from before the lane
    uint32_t keep8[NC];   // per value (byte i of chunk k): 8 * bytes inherited from before the lane
#pragma unroll
    for (int k = 0; k < NC; k++) {
        // byte-wise min(running minimum within the chunk, minimum before it):
        // all values are <= 3, so bit 7 of a byte of (c | 0x80..) - m says c >= m
        const uint32_t M = mlead * 0x01010101u;
        const uint32_t ge = (((cmb[k] | 0x80808080u) - M) & 0x80808080u) >> 7;
        const uint32_t kb = (M & (ge * 0xFFu)) | (cmb[k] & ~(ge * 0xFFu));
        keep8[k] = kb << 3;
        mlead = kb >> 24;
        const uint32_t ld8 = ldb[k] << 3;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const uint32_t* wp = buf + (q >> 2);
            const uint32_t w0 = wp[0], w1 = wp[1];
            const uint32_t inh = top_bytes_mask(byte_of(ld8, i));   // top lead bytes: from the predecessor
            if constexpr (sizeof(T) == 4) {
                const uint32_t sp = __funnelshift_r(w0, w1, q << 3) << low;
                run = (run & inh) | (sp & ~inh);
            } else {
                const uint32_t w2 = wp[2];
                const uint32_t lo = __funnelshift_r(w0, w1, q << 3), hi = __funnelshift_r(w1, w2, q << 3);
                const unsigned long long sp = (((unsigned long long)hi << 32) | lo) << low;
                const unsigned long long ih = (unsigned long long)inh << 32;
                run = (run & ih) | (sp & ~ih);
            }
            cur[4 * k + i] = run;
            q += byte_of(cnt[k], i);
        }
    }
    // lane summary: the top three bytes of its last value, scanned over the
    // segment as (top three bytes, byte mask of the ones the lane wrote): a later
    // lane's written bytes win; bytes no lane wrote stay zero (the chain of
    // every lane starts at zero)
    uint32_t sv = (uint32_t)(run >> TOPSH) & 0xFFFFFFu, sw = 0xFFFFFFu >> (8 * mlead);
#pragma unroll
    for (int d = 1; d < G; d <<= 1) {
        const uint32_t ov = __shfl_up_sync(0xffffffffu, sv, d, G), ow = __shfl_up_sync(0xffffffffu, sw, d, G);
        if (sl >= d) {
            sv = (ov & ~sw) | (sv & sw);
            sw |= ow;
        }
    }
    const uint32_t ex = __shfl_up_sync(0xffffffffu, sv, 1, G);
    const uint32_t carry = sl ? ex << 8 : 0u;   // top three bytes of a 32-bit word
    const T med = widen_median<T>(__uint_as_float(mb));
    T v[E];
#pragma unroll
    for (int k = 0; k < NC; k++) {
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const uint32_t keep = top_bytes_mask(byte_of(keep8[k], i));
            U u = cur[4 * k + i];
            if constexpr (sizeof(T) == 4) u |= carry & keep;
            else u |= (unsigned long long)(carry & keep) << 32;
            u <<= s;
            cur[4 * k + i] = u;
            v[4 * k + i] = EL::add(EL::of(u), med);
        }
    }
    // a NaN result anywhere (three-input max with NaN propagation, float)
    bool bad;
    if constexpr (sizeof(T) == 4) {
        float hn = v[0];
#pragma unroll
        for (int e = 1; e + 1 < E; e += 2) hn = fmax3_nan(hn, v[e], v[e + 1]);
        hn = fmax_nan(hn, v[E - 1]);
        bad = hn != hn;
    } else {
        bad = false;
#pragma unroll
        for (int e = 0; e < E; e++) bad |= v[e] != v[e];
    }
    if (__any_sync(0xffffffffu, bad)) {
#pragma unroll
        for (int e = 0; e < E; e++) v[e] = xadd(EL::of(cur[e]), med);
    }
    // store the lane's E consecutive values (a segment called with len 0 --
    // a constant block, whose median is already stored -- stores nothing)
    const int f0 = E * sl;
    constexpr int V8 = 32 / (int)sizeof(T);   // values per 32-byte store
    if (vec == 2 && f0 + E <= len) {
#pragma unroll
        for (int k = 0; k < E / V8; k++) st_v8(ob + f0 + V8 * k, v + V8 * k);
    } else if (vec && f0 + E <= len) {
#pragma unroll
        for (int k = 0; k < NC; k++) {
            if constexpr (sizeof(T) == 4) {
                *(float4*)(ob + f0 + 4 * k) = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
            } else {
                *(double2*)(ob + f0 + 4 * k) = make_double2(v[4 * k], v[4 * k + 1]);
                *(double2*)(ob + f0 + 4 * k + 2) = make_double2(v[4 * k + 2], v[4 * k + 3]);
            }
        }
    } else {
#pragma unroll
        for (int e = 0; e < E; e++)
            if (f0 + e < len) ob[f0 + e] = v[e];
    }
}

// ------------------------------------------------------------------ decode, pipelined tiles
//
// One producer warp per CTA walks the CTA's tiles ahead of the decoders: it
// reads the tile's state bits and first rank, the payload offsets of its
// non-constant blocks and the medians of its constant blocks, checks them,
// and stages the tile's payload bytes (one contiguous range) into a ring of
// kDecStages shared-memory buffers with a TMA bulk copy.  Eight consumer
// warps decode a tile per step, G lanes per block, and write the values with
// 16-byte stores.  Full/empty mbarriers hand the buffers back and forth; every
// wait is bounded and reports kErrLookback instead of hanging.
constexpr int kDecWarps = 8;
constexpr int kDecThreadsP = (kDecWarps + 1) * 32;
constexpr int kDecStages = 3;
// 4 CTAs of 9 warps per SM (56 registers, three ring stages of shared memory)
constexpr int kDecCtasPerSm = 4;

template <typename T, int G>
struct DecTileV {
    static constexpr int E = EncCfg<T>::E;
    static constexpr int kBsMax = G * E;
    static constexpr int kBpw = 32 / G;
    static constexpr int kBlocks = kDecWarps * kBpw;     // one segment per consumer warp and tile
    static constexpr int kMaxPay = 5 + (kBsMax + 3) / 4 + (int)sizeof(T) * kBsMax;
    // a valid tile's payloads fit kBlocks * kMaxPay; one more kMaxPay + 32
    // keeps the reads of a corrupt block inside the buffer
    static constexpr int kStage = (((kBlocks + 1) * kMaxPay + 32) + 15) / 16 * 16;
    static constexpr int kDynSmem = kDecStages * kStage;
};

struct DecArgs {
    const uint8_t* s;
    unsigned long long len;
    const BlockedHdr* hdr;
    const unsigned long long* P;   // payload offsets by non-constant rank, [nnc + 1]
    const uint32_t* RW;            // non-constant rank at each 32-block state word
    void* out;
    int native_medians;
    int* err;                      // one stream: its error word; a batch: the launch's (bounded waits)
    const DecField* fields;        // a batch: the field table (ascending dec_tile0), else unused
    const uint32_t* tile_field;    // a batch: field of every launch-wide decode tile
    int nf, bs;
    unsigned long long total_tiles;
};

enum : uint8_t { kBlkConst = 0, kBlkCoded = 1, kBlkNone = 2 };

template <typename T, int G, bool MULTI>
__global__ void __launch_bounds__(kDecThreadsP, kDecCtasPerSm) k_blocked_decode(DecArgs a) {
    using TL = DecTileV<T, G>;
    constexpr int TB = TL::kBlocks;
    constexpr int NS = kDecStages;
    extern __shared__ __align__(128) uint8_t dsm[];
    __shared__ unsigned long long full[NS], empty[NS];
    __shared__ uint32_t s_info[NS][TB];    // coded: payload position in the stage; constant: median bits
    __shared__ uint8_t s_kind[NS][TB];
    __shared__ uint8_t s_ok[NS];
    __shared__ int s_fld[NS];              // a batch: the tile's field
    __shared__ uint16_t s_rank[TB];        // producer scratch: rank within the tile
    __shared__ uint32_t lut_ld[256], lut_cm[256];
    BlockedHdr h = {};
    if constexpr (!MULTI) {
        h = *a.hdr;
        if (!h.ok) return;
        if (h.bs > (unsigned long long)TL::kBsMax) {
            if (threadIdx.x == 0 && blockIdx.x == 0) atomicExch(a.err, kErrStream);
            return;
        }
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int i = 0; i < NS; i++) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], kDecWarps);
        }
        mbar_fence_init();
    }
    lead_tables_init(lut_ld, lut_cm);
    __syncthreads();
    const long long ntiles = MULTI ? (long long)a.total_tiles : (long long)((h.nb + TB - 1) / TB);
    const int bs = MULTI ? a.bs : (int)h.bs;
    // field of a launch-wide tile (batch): one load from the plan's tile map
    auto field_of = [&](long long g) { return (int)a.tile_field[g]; };

    if (warp == kDecWarps) {
        // ---------------------------------------------------------- producer
        long long i = 0;
        for (long long t = blockIdx.x; t < ntiles; t += gridDim.x, i++) {
            const int slot = (int)(i % NS);
            if (i >= NS && !mbar_wait(&empty[slot], (uint32_t)((i / NS - 1) & 1))) {
                if (lane == 0) atomicExch(a.err, kErrLookback);
                break;
            }
            uint8_t* stage = dsm + slot * TL::kStage;
            // the tile's stream: the launch's, or its field's
            const uint8_t* S = a.s;
            unsigned long long L = a.len;
            const unsigned long long* P = a.P;
            const uint32_t* RW = a.RW;
            int* ferr = a.err;
            BlockedHdr hh = h;
            long long lt = t;
            if constexpr (MULTI) {
                const int f = field_of(t);
                const DecField* D = a.fields + f;
                S = D->s; L = D->len; P = D->P; RW = D->RW; ferr = D->err;
                hh = *D->hdr;
                lt = t - (long long)D->dec_tile0;
                if (lane == 0) s_fld[slot] = f;
            }
            const unsigned long long b0 = (unsigned long long)lt * TB;
            const unsigned long long rest = hh.ok ? hh.nb - b0 : 0;   // a batch's failed header: no blocks
            const int nblk = rest < (unsigned long long)TB ? (int)rest : TB;
            // rank of the tile's first block
            const unsigned long long w = b0 >> 5;
            const int bit0 = (int)(b0 & 31);
            uint32_t word = 0;
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const unsigned long long bi = 4 * w + j;
                word = (word << 8) | (bi < hh.sb ? (uint32_t)S[hh.s_off + bi] : 0u);
            }
            const unsigned long long rank0 = hh.ok ? RW[w] + (bit0 ? __popc(word >> (32 - bit0)) : 0) : 0;
            // state of every block (loads independent of the rank above)
            uint32_t ok = 1, running = 0;
            for (int j = 0; j < TB; j += 32) {
                const int lb = j + lane;
                const unsigned long long b = b0 + lb;
                const bool in = lb < nblk;
                const uint32_t coded = in ? (S[hh.s_off + (b >> 3)] >> (7 - (b & 7))) & 1u : 0u;
                const unsigned m = __ballot_sync(0xffffffffu, coded);
                const uint32_t r = running + __popc(m & ((1u << lane) - 1));
                running += __popc(m);
                if (lb < TB) {
                    s_kind[slot][lb] = !in ? kBlkNone : (coded ? kBlkCoded : kBlkConst);
                    s_rank[lb] = (uint16_t)r;   // coded: rank among the tile's coded blocks; else among them before
                }
            }
            const uint32_t nnc_t = running;
            // the tile's payload range, then its copy at once: the rest of the
            // metadata is gathered while the copy is in flight
            unsigned long long pa = 0, pb = 0;
            if (rank0 + nnc_t > hh.nnc) ok = 0;
            if (ok && nnc_t) {
                pa = P[rank0];
                pb = P[rank0 + nnc_t];
                if (pb < pa || pb - pa > (unsigned long long)TB * TL::kMaxPay || hh.q_off + pb > L) ok = 0;
            }
            const uint8_t* src = S + hh.q_off + pa;
            const uint32_t ph = (uint32_t)((uintptr_t)src & 15);
            const unsigned long long nbytes = ok ? pb - pa : 0;
            const uintptr_t sa = (uintptr_t)src;
            const uintptr_t a0 = (sa + 15) & ~(uintptr_t)15, a1 = (sa + nbytes) & ~(uintptr_t)15;
            uint32_t tx = 0;
            uintptr_t head_end = sa + nbytes, tail_beg = sa + nbytes;
            if (a1 > a0) {
                tx = (uint32_t)(a1 - a0);
                head_end = a0;
                tail_beg = a1;
            }
            __syncwarp();
            if (lane == 0 && tx) {
                fence_proxy_async();
                mbar_expect_tx(&full[slot], tx);
                tma_load_1d(stage + ph + (a0 - sa), (const void*)a0, tx, &full[slot]);
            }
            // medians of the constant blocks, payload offsets of the coded ones
            for (int j = 0; j < TB; j += 32) {
                const int lb = j + lane;
                if (lb >= nblk) continue;
                const unsigned long long b = b0 + lb;
                const uint32_t r = s_rank[lb];
                if (s_kind[slot][lb] == kBlkConst) {
                    const unsigned long long mo = hh.m_off + 4 * (b - (rank0 + r));
                    uint32_t mbits = 0;
                    if (b >= rank0 + r && mo + 4 <= hh.q_off) {
                        const uint8_t* mp = S + mo;
                        mbits = a.native_medians
                                    ? ((uint32_t)mp[0] | ((uint32_t)mp[1] << 8) | ((uint32_t)mp[2] << 16) |
                                       ((uint32_t)mp[3] << 24))
                                    : (((uint32_t)mp[0] << 24) | ((uint32_t)mp[1] << 16) | ((uint32_t)mp[2] << 8) |
                                       mp[3]);
                    } else {
                        ok = 0;
                    }
                    s_info[slot][lb] = mbits;
                } else if (nbytes) {
                    const unsigned long long k = rank0 + r;
                    const unsigned long long p0 = P[k], p1 = P[k + 1];
                    const unsigned long long rem = hh.n - b * hh.bs;
                    const int blen = rem < hh.bs ? (int)rem : bs;
                    const unsigned long long minsz = 5 + (unsigned long long)((blen + 3) / 4);
                    if (p0 < pa || p1 > pb || p1 < p0 + minsz || p1 - p0 > (unsigned long long)TL::kMaxPay) ok = 0;
                    s_info[slot][lb] = ph + (uint32_t)(p0 - pa);
                } else {
                    ok = 0;   // a coded block without a valid payload range
                }
            }
            ok = __all_sync(0xffffffffu, ok);
            // ragged ends of the payload range by the lanes
            for (uintptr_t x = sa + lane; x < head_end; x += 32) stage[ph + (x - sa)] = *(const uint8_t*)x;
            for (uintptr_t x = tail_beg + lane; x < sa + nbytes; x += 32) stage[ph + (x - sa)] = *(const uint8_t*)x;
            __threadfence_block();
            __syncwarp();
            if (lane == 0) {
                s_ok[slot] = (uint8_t)ok;
                if (!ok) atomicExch(ferr, kErrStream);
                mbar_arrive(&full[slot]);
            }
        }
        // copies still in flight finish before the CTA exits
        for (long long j = i > NS ? i - NS : 0; j < i; j++) mbar_wait(&full[j % NS], (uint32_t)((j / NS) & 1));
        return;
    }

    // -------------------------------------------------------------- consumers
    T* out = (T*)a.out;
    auto vec_of = [&](const T* o) {
        const uintptr_t al = (uintptr_t)o | (uintptr_t)(bs * (int)sizeof(T));
        return (al & 31) == 0 ? 2 : ((al & 15) == 0 ? 1 : 0);
    };
    int vec = vec_of(out);
    unsigned long long n = h.n;
    const int seg = lane / G;
    const int lb = warp * TL::kBpw + seg;
    long long i = 0;
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x, i++) {
        const int slot = (int)(i % NS);
        if (!mbar_wait(&full[slot], (uint32_t)((i / NS) & 1))) {
            if (lane == 0) atomicExch(a.err, kErrLookback);
            break;
        }
        long long lt = t;
        if constexpr (MULTI) {
            const DecField* D = a.fields + s_fld[slot];
            out = (T*)D->out;
            n = D->n;
            lt = t - (long long)D->dec_tile0;
            vec = vec_of(out);
        }
        const unsigned long long b = (unsigned long long)lt * TB + lb;
        const int kind = s_kind[slot][lb];
        const uint32_t info = s_info[slot][lb];
        int blen = 0;
        T* ob = out;
        if (kind != kBlkNone) {
            const unsigned long long off = b * (unsigned long long)bs, rem = n - off;
            blen = rem < (unsigned long long)bs ? (int)rem : bs;
            ob = out + off;
        }
        if (kind == kBlkConst) {
            const T m = widen_median<T>(__uint_as_float(info));
            T v[EncCfg<T>::E];
#pragma unroll
            for (int e = 0; e < EncCfg<T>::E; e++) v[e] = m;
            store_chunks<T, G>(ob, blen, vec, v);
        }
        const bool coded = kind == kBlkCoded && s_ok[slot];
        const uint8_t* stage = dsm + slot * TL::kStage;
        // the whole warp takes one path: segments that decode nothing store nothing either way
        if (__all_sync(0xffffffffu, !coded || blen == TL::kBsMax))
            dec_segment_seq<T, G, true>(stage + (coded ? info : 0u), coded ? blen : 0, ob, vec, lut_ld, lut_cm);
        else
            dec_segment_seq<T, G, false>(stage + (coded ? info : 0u), coded ? blen : 0, ob, vec, lut_ld, lut_cm);
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[slot]);
    }
}

template <typename T, int G, bool MULTI>
static cudaError_t dec_attr() {
    static bool attr_set[64] = {false};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && !attr_set[dev]) {
        cudaError_t e = cudaFuncSetAttribute(k_blocked_decode<T, G, MULTI>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, DecTileV<T, G>::kDynSmem);
        if (e != cudaSuccess) return e;
        attr_set[dev] = true;
    }
    return cudaSuccess;
}

template <typename T, int G>
static cudaError_t run_decode(const uint8_t* s, size_t len, size_t nb, const Workspace& ws, void* out, int native,
                              cudaStream_t st) {
    using TL = DecTileV<T, G>;
    cudaError_t e = dec_attr<T, G, false>();
    if (e != cudaSuccess) return e;
    const size_t tiles = (nb + TL::kBlocks - 1) / TL::kBlocks;
    const size_t cap = (size_t)sm_count() * kDecCtasPerSm;
    const int grid = (int)(tiles < cap ? (tiles ? tiles : 1) : cap);
    DecArgs a = {};
    a.s = s; a.len = len; a.hdr = ws.bhdr; a.P = ws.p_off; a.RW = ws.rank_w; a.out = out;
    a.native_medians = native; a.err = ws.err;
    TraceScope tr("blocked_decode", st);
    k_blocked_decode<T, G, false><<<grid, kDecThreadsP, TL::kDynSmem, st>>>(a);
    return cudaGetLastError();
}

template <typename T, int G>
static cudaError_t run_decode_fields(const DecField* F, const uint32_t* tf, int nf, int bs, unsigned long long total,
                                     int native, int* lerr, int ctas_per_sm, cudaStream_t st) {
    using TL = DecTileV<T, G>;
    cudaError_t e = dec_attr<T, G, true>();
    if (e != cudaSuccess) return e;
    const int cps = ctas_per_sm > 0 && ctas_per_sm < kDecCtasPerSm ? ctas_per_sm : kDecCtasPerSm;
    const size_t cap = (size_t)sm_count() * cps;
    const int grid = (int)(total < cap ? (total ? total : 1) : cap);
    DecArgs a = {};
    a.native_medians = native; a.err = lerr;
    a.fields = F; a.tile_field = tf; a.nf = nf; a.bs = bs; a.total_tiles = total;
    TraceScope tr("blocked_decode_fields", st);
    k_blocked_decode<T, G, true><<<grid, kDecThreadsP, TL::kDynSmem, st>>>(a);
    return cudaGetLastError();
}

// Lanes per block as in the encoder: 16 (float) / 8 (double) values per lane.
static int dec_lanes(int dtype, int bs) {
    const int per = dtype == 0 ? 16 : 8;
    const int need = (bs + per - 1) / per;
    return need <= 1 ? 1 : need <= 2 ? 2 : need <= 4 ? 4 : need <= 8 ? 8 : need <= 16 ? 16 : 32;
}

int blocked_dec_tile_blocks(int dtype, int bs) { return kDecWarps * (32 / dec_lanes(dtype, bs)); }

// Per-field outcome of a batched decode; *err gets the first failing status.
__global__ void k_blocked_decode_finish(const DecField* F, int nf, int esize, StreamResult* res, const int* lerr,
                                        int* err) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const DecField& D = F[f];
    int st = *D.err;
    if (!st) st = *lerr;
    StreamResult r;
    r.offset = 0;
    r.size = D.n * (unsigned long long)esize;
    r.nb_const = D.hdr->ok ? D.hdr->nc : 0;
    r.eb = 0.f;
    r.status = st;
    *(D.res ? D.res : res + f) = r;
    if (st) atomicCAS(err, 0, st);
}

cudaError_t launch_blocked_decode_fields(int layout, int dtype, int bs, int nf, const DecField* d_fields,
                                         const uint32_t* d_tile_field, unsigned long long idx_total,
                                         unsigned long long dec_total,
                                         unsigned long long* counters, StreamResult* res, int* err,
                                         cudaStream_t s, const LaunchShape& shape) {
    if (layout != kRandomAccess && layout != kRandomAccessNative) return cudaErrorInvalidValue;
    if (bs < 1 || bs > 256 || nf < 1) return cudaErrorInvalidValue;
    int* lerr = (int*)(counters + 3);
    {
        TraceScope tr("blocked_parse_fields", s);
        k_blocked_parse_fields<<<(nf + 127) / 128, 128, 0, s>>>(d_fields, nf, (unsigned long long)bs);
    }
    {
        const unsigned long long cap = (unsigned long long)sm_count() * 4;
        const int ig = (int)(idx_total < cap ? (idx_total ? idx_total : 1) : cap);
        TraceScope tr("blocked_index_fields", s);
        k_blocked_index_fields<<<ig, kIdxThreads, 0, s>>>(d_fields, nf, idx_total, &counters[0]);
    }
    const int native = layout == kRandomAccessNative;
    cudaError_t e;
    if (dtype == 0) {
        switch (dec_lanes(dtype, bs)) {
            case 1: e = run_decode_fields<float, 1>(d_fields, d_tile_field, nf, bs, dec_total, native, lerr, shape.dec_ctas_per_sm, s); break;
            case 2: e = run_decode_fields<float, 2>(d_fields, d_tile_field, nf, bs, dec_total, native, lerr, shape.dec_ctas_per_sm, s); break;
            case 4: e = run_decode_fields<float, 4>(d_fields, d_tile_field, nf, bs, dec_total, native, lerr, shape.dec_ctas_per_sm, s); break;
            case 8: e = run_decode_fields<float, 8>(d_fields, d_tile_field, nf, bs, dec_total, native, lerr, shape.dec_ctas_per_sm, s); break;
            default: e = run_decode_fields<float, 16>(d_fields, d_tile_field, nf, bs, dec_total, native, lerr, shape.dec_ctas_per_sm, s); break;
        }
    } else {
        switch (dec_lanes(dtype, bs)) {
            case 1: e = run_decode_fields<double, 1>(d_fields, d_tile_field, nf, bs, dec_total, native, lerr, shape.dec_ctas_per_sm, s); break;
            case 2: e = run_decode_fields<double, 2>(d_fields, d_tile_field, nf, bs, dec_total, native, lerr, shape.dec_ctas_per_sm, s); break;
            case 4: e = run_decode_fields<double, 4>(d_fields, d_tile_field, nf, bs, dec_total, native, lerr, shape.dec_ctas_per_sm, s); break;
            case 8: e = run_decode_fields<double, 8>(d_fields, d_tile_field, nf, bs, dec_total, native, lerr, shape.dec_ctas_per_sm, s); break;
            case 16: e = run_decode_fields<double, 16>(d_fields, d_tile_field, nf, bs, dec_total, native, lerr, shape.dec_ctas_per_sm, s); break;
            default: e = run_decode_fields<double, 32>(d_fields, d_tile_field, nf, bs, dec_total, native, lerr, shape.dec_ctas_per_sm, s); break;
        }
    }
    if (e != cudaSuccess) return e;
    k_blocked_decode_finish<<<(nf + 127) / 128, 128, 0, s>>>(d_fields, nf, dtype == 0 ? 4 : 8, res, lerr, err);
    return cudaGetLastError();
}

cudaError_t launch_blocked_decode(int layout, int dtype, const uint8_t* d_stream, size_t len, size_t n, int bs,
                                  void* d_out, const Workspace& ws, cudaStream_t s) {
    if (layout != kBlocked && layout != kRandomAccess && layout != kRandomAccessNative) return cudaErrorInvalidValue;
    if (bs < 1 || bs > 256 || n == 0) return cudaErrorInvalidValue;
    const bool m2 = layout == kBlocked;
    cudaError_t e;
    {
        ClearList c{};   // the index kernel's tile counter and both look-backs' status words
        c.p[0] = ws.counters;
        c.bytes[0] = sizeof(unsigned long long);
        c.p[1] = ws.st_word;
        c.bytes[1] = sizeof(unsigned long long) * ws.status_tiles;
        c.p[2] = ws.st2_word;
        c.bytes[2] = sizeof(unsigned long long) * ws.status2_tiles;
        c.n = 3;
        if ((e = launch_ws_clear(c, s)) != cudaSuccess) return e;
    }
    {
        TraceScope tr("blocked_parse", s);
        if (m2) k_m2_parse<<<1, 1, 0, s>>>(d_stream, len, n, (unsigned long long)bs, ws.bhdr, ws.err);
        else k_blocked_parse<<<1, 1, 0, s>>>(d_stream, len, n, (unsigned long long)bs, ws.bhdr, ws.err);
    }
    {
        int ig = sm_count() * 4;
        TraceScope tr("blocked_index", s);
        k_blocked_index<<<ig, kIdxThreads, 0, s>>>(d_stream, ws.bhdr, ws.p_off, ws.rank_w,
                                                    TileStatus{ws.st_word, ws.st_agg2, ws.st_inc2},
                                                    TileStatus{ws.st2_word, ws.st2_agg2, ws.st2_inc2},
                                                    &ws.counters[0], ws.err, len, m2 ? 0 : 1);
    }
    if (m2 && (e = launch_m2_offsets(dtype, d_stream, len, n, bs, ws.m2, ws.m2_bytes, ws, s)) != cudaSuccess)
        return e;
    // bs comes from the stream header (read by the caller); the device header
    // is validated again by every kernel and a mismatch is reported, not used.
    const int native = layout == kRandomAccessNative;
    const size_t nb = (n + bs - 1) / bs;
    const int G = dec_lanes(dtype, bs);
    if (dtype == 0) {
        switch (G) {
            case 1: e = run_decode<float, 1>(d_stream, len, nb, ws, d_out, native, s); break;
            case 2: e = run_decode<float, 2>(d_stream, len, nb, ws, d_out, native, s); break;
            case 4: e = run_decode<float, 4>(d_stream, len, nb, ws, d_out, native, s); break;
            case 8: e = run_decode<float, 8>(d_stream, len, nb, ws, d_out, native, s); break;
            default: e = run_decode<float, 16>(d_stream, len, nb, ws, d_out, native, s); break;
        }
    } else {
        switch (G) {
            case 1: e = run_decode<double, 1>(d_stream, len, nb, ws, d_out, native, s); break;
            case 2: e = run_decode<double, 2>(d_stream, len, nb, ws, d_out, native, s); break;
            case 4: e = run_decode<double, 4>(d_stream, len, nb, ws, d_out, native, s); break;
            case 8: e = run_decode<double, 8>(d_stream, len, nb, ws, d_out, native, s); break;
            case 16: e = run_decode<double, 16>(d_stream, len, nb, ws, d_out, native, s); break;
            default: e = run_decode<double, 32>(d_stream, len, nb, ws, d_out, native, s); break;
        }
    }
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

}  // namespace szxg
