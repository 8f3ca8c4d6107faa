// Block boundaries of the fastMode-2 stream, found in parallel.
//
// Layout (szx/src/szx_float.cc:1059-1139, the FXR output as well):
//   [1,1,1,0] | blockSize u8 | nbConstant u64 BE | state bits | medians f32 BE
//   | payloads of the non-constant blocks, back to back, with no size index.
// A payload's length follows from its own first bytes: reqLength (-> R
// stored bytes per value), then ceil(n/4) lead bytes, then sum over values of
// max(R - lead, 0) mid bytes.  The reference decoder walks the chain serially
// (szx/src/szxd_float.cc:247-311).
//
// Here the payload region is cut into segments.  Pass 1 starts a walk at
// every position of each segment's first `maxsize` bytes (a block that began
// in the previous segment ends there); walks from positions that are not
// block starts read a reqLength outside the valid range within a step or two
// and stop, and the few that land on a true boundary follow the true chain
// from then on, so the walks that reach the end of a segment all leave it at
// the same offset: the next segment's entry.  Each walk also records how many
// blocks it passed, so the true chain's count per segment is read off at the
// entry, ranks are an exclusive scan of those counts, and pass 2 replays the
// true chain in every segment in parallel, writing each block's payload
// offset by rank.  The replay checks itself (segment exits must meet the next
// entries, the last block must end the stream); if anything disagrees, a
// one-thread serial walk rebuilds the offsets.  The offsets then feed the same
// tile decoder as the random-access layout.
#include "common.cuh"
#include "kernels.h"

namespace szxg {

namespace {

constexpr int kM2Threads = 256;
constexpr unsigned short kM2Dead = 0xFFFF;

struct M2Geom {
    unsigned long long len;    // stream bytes; the payload region is [q_off, len)
    unsigned long long seg;    // segment bytes
    unsigned long long nseg;   // segments covering the largest possible payload region
    int maxsize;               // largest payload of a full block
};

__device__ __forceinline__ unsigned long long be64d(const uint8_t* p) {
    unsigned long long v = 0;
    for (int i = 0; i < 8; i++) v = (v << 8) | p[i];
    return v;
}

// Payload bytes of the block whose payload starts at p (blen values);
// -1 when the bytes there cannot start a block, -2 when they could but the
// block would run past the end L.  W = bytes per value.
__device__ __forceinline__ long long m2_size(const uint8_t* P, unsigned long long L, unsigned long long p, int blen,
                                             int W, const uint8_t* lut /*[9][256]*/) {
    if (p + 5 > L) return -1;
    const int rl = P[p];
    // reqLength: float 9..32 (szx/src/szx_float.cc:1708-1717), double 12..64 (szx/src/szx_double.cc:2020-2031)
    if (W == 4 ? (rl < 9 || rl > 32) : (rl < 12 || rl > 64)) return -1;
    const int R = (rl >> 3) + ((rl & 7) != 0);
    const int Lb = (blen + 3) >> 2;
    if (p + 5 + (unsigned long long)Lb > L) return -2;
    const uint8_t* q = P + p + 5;
    const uint8_t* t = lut + 256 * R;
    long long mid = 0;
    const int full = blen >> 2;
    for (int b = 0; b < full; b++) mid += t[q[b]];
    if (blen & 3) {
        const int code = q[full];
        for (int i = 0; i < (blen & 3); i++) {
            const int ld = (code >> (6 - 2 * i)) & 3;
            mid += R > ld ? R - ld : 0;
        }
    }
    const long long size = 5 + Lb + mid;
    return p + (unsigned long long)size > L ? -2 : size;
}

// lut[R][byte] = sum over the byte's 4 lead codes of max(R - lead, 0)
__device__ __forceinline__ void m2_lut_init(uint8_t* lut) {
    for (int i = threadIdx.x; i < 9 * 256; i += blockDim.x) {
        const int R = i >> 8, b = i & 255;
        int c = 0;
        for (int k = 0; k < 4; k++) {
            const int ld = (b >> (6 - 2 * k)) & 3;
            c += R > ld ? R - ld : 0;
        }
        lut[i] = (uint8_t)c;
    }
}

}  // namespace

// Parse and validate the mode-2 header (szx/src/szxd_float.cc:247-270).
__global__ void k_m2_parse(const uint8_t* s, unsigned long long len, unsigned long long n,
                           unsigned long long bs_expect, BlockedHdr* h, int* err) {
    BlockedHdr r = {};
    r.n = n;
    r.ok = 0;
    if (len >= 13 && s[3] == 0) {
        r.bs = s[4];
        r.nc = be64d(s + 5);
        if (r.bs >= 1 && (bs_expect == 0 || r.bs == bs_expect)) {
            r.nb = (n + r.bs - 1) / r.bs;
            r.sb = (r.nb + 7) / 8;
            if (r.nc <= r.nb) {
                r.nnc = r.nb - r.nc;
                r.o_off = 13;
                r.s_off = 13;
                r.m_off = r.s_off + r.sb;
                r.q_off = r.m_off + 4 * r.nc;
                r.ok = r.q_off <= len;
            }
        }
    }
    *h = r;
    *err = r.ok ? kErrNone : kErrStream;
}

// Pass 1: one thread per candidate start (segment j, offset c < maxsize).
__global__ void __launch_bounds__(kM2Threads) k_m2_walk(const uint8_t* s, const BlockedHdr* hp, M2Geom g, int W,
                                                        unsigned short* cnt_tab, unsigned long long* exit_lo,
                                                        unsigned long long* exit_hi) {
    __shared__ uint8_t lut[9 * 256];
    m2_lut_init(lut);
    __syncthreads();
    const BlockedHdr h = *hp;
    if (!h.ok) return;
    const unsigned long long t = (unsigned long long)blockIdx.x * kM2Threads + threadIdx.x;
    const unsigned long long j = t / (unsigned long long)g.maxsize, c = t % (unsigned long long)g.maxsize;
    if (j >= g.nseg) return;
    const uint8_t* P = s + h.q_off;
    const unsigned long long L = g.len - h.q_off;
    const unsigned long long end = (j + 1) * g.seg;
    unsigned long long p = j * g.seg + c;
    unsigned short count = kM2Dead;
    if (p < L) {
        unsigned int k = 0;
        bool alive = true;
        while (p < end && p < L) {
            const long long sz = m2_size(P, L, p, (int)h.bs, W, lut);
            if (sz == -2) {   // runs past the end: the stream's last block when it is short
                p = L;
                k++;
                break;
            }
            if (sz < 0) { alive = false; break; }
            p += (unsigned long long)sz;
            k++;
        }
        if (alive && k > 0) {
            count = (unsigned short)k;
            atomicMin(&exit_lo[j], p);
            atomicMax(&exit_hi[j], p);
        }
    }
    cnt_tab[j * (unsigned long long)g.maxsize + c] = count;
}

// Entries and counts of the true chain per segment (one thread per segment).
__global__ void k_m2_link(const BlockedHdr* hp, M2Geom g, const unsigned short* cnt_tab,
                          const unsigned long long* exit_lo, const unsigned long long* exit_hi,
                          unsigned long long* entry, unsigned int* cnt, unsigned int* ambiguous) {
    const unsigned long long j = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    const BlockedHdr h = *hp;
    if (!h.ok || j >= g.nseg) return;
    const unsigned long long L = g.len - h.q_off;
    unsigned long long e = 0;
    bool ok = true;
    if (j > 0) {
        e = exit_lo[j - 1];
        ok = e != ~0ull;
        if (ok && exit_hi[j - 1] != e) ambiguous[j] = 1;
    }
    unsigned int k = 0;
    if (ok && e >= j * g.seg && e - j * g.seg < (unsigned long long)g.maxsize && e < L) {
        const unsigned short v = cnt_tab[j * (unsigned long long)g.maxsize + (e - j * g.seg)];
        k = v == kM2Dead ? 0 : v;
    } else {
        e = ~0ull;
    }
    entry[j] = e;
    cnt[j] = k;
}

// Exclusive scan of the per-segment counts (one CTA).
__global__ void __launch_bounds__(1024) k_m2_scan(unsigned long long nseg, const unsigned int* cnt,
                                                  unsigned long long* base) {
    __shared__ unsigned long long s_w[32];
    __shared__ unsigned long long s_carry;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    for (unsigned long long j0 = 0; j0 < nseg; j0 += 1024) {
        const unsigned long long j = j0 + threadIdx.x;
        const unsigned long long v = j < nseg ? cnt[j] : 0;
        const unsigned long long incl = warp_inclusive_sum(v);
        if ((threadIdx.x & 31) == 31) s_w[threadIdx.x >> 5] = incl;
        __syncthreads();
        if (threadIdx.x < 32) s_w[threadIdx.x] = warp_inclusive_sum(s_w[threadIdx.x]);
        __syncthreads();
        const unsigned long long pre = (threadIdx.x >= 32 ? s_w[(threadIdx.x >> 5) - 1] : 0) + s_carry;
        if (j < nseg) base[j] = pre + incl - v;
        __syncthreads();
        if (threadIdx.x == 0) s_carry += s_w[31];
        __syncthreads();
    }
}

// Pass 2: replay the true chain of each segment, writing payload offsets by
// rank (P[nnc] = end of the last block); disagreements raise `redo`.
__global__ void __launch_bounds__(kM2Threads) k_m2_replay(const uint8_t* s, const BlockedHdr* hp, M2Geom g, int W,
                                                          const unsigned long long* entry,
                                                          const unsigned long long* base,
                                                          const unsigned int* ambiguous, unsigned long long* Poff,
                                                          unsigned int* redo) {
    __shared__ uint8_t lut[9 * 256];
    m2_lut_init(lut);
    __syncthreads();
    const BlockedHdr h = *hp;
    if (!h.ok) return;
    const unsigned long long j = (unsigned long long)blockIdx.x * kM2Threads + threadIdx.x;
    if (j >= g.nseg) return;
    unsigned long long rank = base[j];
    if (rank >= h.nnc) return;   // the chain ended in an earlier segment
    if (ambiguous[j] || entry[j] == ~0ull) { atomicExch(redo, 1u); return; }
    const uint8_t* P = s + h.q_off;
    const unsigned long long L = g.len - h.q_off;
    const unsigned long long end = (j + 1) * g.seg;
    // the last block is short when n is not a multiple of bs and block nb-1 is non-constant
    const unsigned long long last_len = h.n - (h.nb - 1) * h.bs;
    const bool last_coded = (s[h.s_off + ((h.nb - 1) >> 3)] >> (7 - ((h.nb - 1) & 7))) & 1;
    unsigned long long p = entry[j];
    while (p < end && rank < h.nnc) {
        const int blen = (rank == h.nnc - 1 && last_coded) ? (int)last_len : (int)h.bs;
        const long long sz = m2_size(P, L, p, blen, W, lut);
        if (sz < 0) { atomicExch(redo, 1u); return; }
        Poff[rank] = p;
        p += (unsigned long long)sz;
        rank++;
    }
    if (rank == h.nnc) {
        Poff[h.nnc] = p;
        if (p != L) atomicExch(redo, 1u);
    } else if (j + 1 < g.nseg && entry[j + 1] != p) {
        atomicExch(redo, 1u);
    }
}

// Fallback when the parallel passes disagree: the serial walk (one thread).
__global__ void k_m2_serial(const uint8_t* s, const BlockedHdr* hp, M2Geom g, int W, const unsigned int* redo,
                            unsigned long long* Poff, int* err) {
    __shared__ uint8_t lut[9 * 256];
    m2_lut_init(lut);
    __syncthreads();
    if (threadIdx.x != 0 || !*redo) return;
    const BlockedHdr h = *hp;
    if (!h.ok) return;
    const uint8_t* P = s + h.q_off;
    const unsigned long long L = g.len - h.q_off;
    const unsigned long long last_len = h.n - (h.nb - 1) * h.bs;
    const bool last_coded = (s[h.s_off + ((h.nb - 1) >> 3)] >> (7 - ((h.nb - 1) & 7))) & 1;
    unsigned long long p = 0;
    for (unsigned long long r = 0; r < h.nnc; r++) {
        const int blen = (r == h.nnc - 1 && last_coded) ? (int)last_len : (int)h.bs;
        const long long sz = m2_size(P, L, p, blen, W, lut);
        if (sz < 0) { atomicExch(err, kErrStream); return; }
        Poff[r] = p;
        p += (unsigned long long)sz;
    }
    Poff[h.nnc] = p;
    if (p != L) atomicExch(err, kErrStream);
}

namespace {

int m2_maxsize(int dtype, int bs) { return 5 + (bs + 3) / 4 + (dtype == 0 ? 4 : 8) * bs; }

}  // namespace

// Segments for a stream of len bytes of n values in blocks of bs: the payload
// region is at most len - 13 - state bytes.
size_t m2_segments(int dtype, size_t n, int bs, size_t len) {
    const size_t nb = (n + bs - 1) / bs, sb = (nb + 7) / 8;
    const size_t pmax = len > 13 + sb ? len - 13 - sb : 0;
    return pmax / (32 * (size_t)m2_maxsize(dtype, bs)) + 1;
}

size_t m2_ws_bytes(int dtype, size_t n, int bs, size_t len) {
    if (bs < 1 || n == 0) return 256;
    const size_t ms = (size_t)m2_maxsize(dtype, bs);
    const size_t nseg = m2_segments(dtype, n, bs, len);
    auto a = [](size_t x) { return (x + 255) & ~(size_t)255; };
    return a(2 * nseg * ms) + 3 * a(8 * nseg) + 2 * a(4 * nseg) + 256;
}

// Payload offsets by non-constant rank for a fastMode-2 stream of len bytes
// (ws.p_off; P[nnc] = payload end), after the header is parsed into ws.bhdr.
cudaError_t launch_m2_offsets(int dtype, const uint8_t* d_stream, size_t len, size_t n, int bs, void* m2ws,
                              size_t m2wsb, const Workspace& ws, cudaStream_t s) {
    const int ms = m2_maxsize(dtype, bs);
    M2Geom g;
    g.len = len;
    g.maxsize = ms;
    g.seg = 32ull * ms;
    g.nseg = m2_segments(dtype, n, bs, len);
    if (m2wsb < m2_ws_bytes(dtype, n, bs, len)) return cudaErrorInvalidValue;
    auto a = [](size_t x) { return (x + 255) & ~(size_t)255; };
    uint8_t* b = (uint8_t*)m2ws;
    unsigned short* cnt_tab = (unsigned short*)b; b += a(2 * g.nseg * ms);
    unsigned long long* exit_lo = (unsigned long long*)b; b += a(8 * g.nseg);
    unsigned long long* exit_hi = (unsigned long long*)b; b += a(8 * g.nseg);
    unsigned long long* entry = (unsigned long long*)b; b += a(8 * g.nseg);
    unsigned int* cnt = (unsigned int*)b; b += a(4 * g.nseg);
    unsigned int* amb = (unsigned int*)b; b += a(4 * g.nseg);
    unsigned long long* base = exit_hi;   // reused after the link pass
    unsigned int* redo = (unsigned int*)b;
    const int W = dtype == 0 ? 4 : 8;
    cudaError_t e;
    if ((e = cudaMemsetAsync(exit_lo, 0xFF, 8 * g.nseg, s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(exit_hi, 0, 8 * g.nseg, s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(amb, 0, 4 * g.nseg, s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(redo, 0, 4, s)) != cudaSuccess) return e;
    {
        TraceScope tr("m2_walk", s);
        const unsigned long long threads = g.nseg * (unsigned long long)ms;
        k_m2_walk<<<(unsigned)((threads + kM2Threads - 1) / kM2Threads), kM2Threads, 0, s>>>(d_stream, ws.bhdr, g, W,
                                                                                          cnt_tab, exit_lo, exit_hi);
    }
    k_m2_link<<<(unsigned)((g.nseg + 255) / 256), 256, 0, s>>>(ws.bhdr, g, cnt_tab, exit_lo, exit_hi, entry, cnt, amb);
    k_m2_scan<<<1, 1024, 0, s>>>(g.nseg, cnt, base);
    {
        TraceScope tr("m2_replay", s);
        k_m2_replay<<<(unsigned)((g.nseg + kM2Threads - 1) / kM2Threads), kM2Threads, 0, s>>>(
            d_stream, ws.bhdr, g, W, entry, base, amb, ws.p_off, redo);
    }
    k_m2_serial<<<1, 256, 0, s>>>(d_stream, ws.bhdr, g, W, redo, ws.p_off, ws.err);
    return cudaGetLastError();
}

}  // namespace szxg
