/* CPU restatement of the reference's cuSZx float codec -- test infrastructure
 * only.  Its stream differs from the CPU codec's (szx/src/cuszx_entry.cu:20-60):
 *
 *   [1,1,1,0] | blockSize u8 | nbConstant u64 BE | state bits (full blocks,
 *   MSB first) | nbEle % blockSize raw floats | constant medians (native
 *   float) | per non-constant block: mid-byte count i16 (native) | per
 *   non-constant block: median (native float), reqLength u8, 2-bit lead
 *   codes (blockSize / 4 bytes), mid bytes.
 *
 * Per block (szx/src/cuszx_float.cu:221-300, 118-219): min / max (over the
 * first 32 * 2^floor(log2(bs/32)) values: the reference's cross-warp
 * reduction misses the rest when bs/32 is not a power of two), radius =
 * (max - min) / 2, median = min + radius, constant when radius <= bound;
 * otherwise reqLength = 10 + exponent(radius) - exponent(bound) with no
 * clamping, words = bits(x - median) shifted right logically, leading
 * identical bytes with the previous value counted up to the required byte
 * count (so a value may get a lead of 4, whose 2-bit code then spills into
 * its neighbour's, cuszx_float.cu:54-65), stored bytes = required - lead.
 * Decoding (szx/src/cuszxd_float.cu:146-296) takes each byte lane a value
 * does not store from the latest earlier value that stored that lane, or
 * from the block's first value when none did; with reqLength above 32 no
 * byte is stored or read and the block decodes to its median.
 *
 * NaN inputs are outside what this restatement pins (the GPU's min/max and
 * NaN rules are not modelled).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static int expo(uint32_t bits) { return (int)((bits & 0x7F800000u) >> 23) - 127; }

/* the GPU's float min / max (finite values): -0 orders below +0 */
static float fmin_gpu(float a, float b) {
    if (a == b) return (f2u(a) & 0x80000000u) ? a : b;
    return a < b ? a : b;
}
static float fmax_gpu(float a, float b) {
    if (a == b) return (f2u(a) & 0x80000000u) ? b : a;
    return a > b ? a : b;
}
static void block_range(const float* v, int bs, float* mn, float* mx) {
    float lo = v[0], hi = v[0];
    for (int i = 1; i < bs; i++) { lo = fmin_gpu(lo, v[i]); hi = fmax_gpu(hi, v[i]); }
    *mn = lo;
    *mx = hi;
}

static void req_split(int reqLength, int* R, int* rsb) {
    if (reqLength % 8 != 0) { *R = reqLength / 8 + 1; *rsb = 8 - reqLength % 8; }
    else { *R = reqLength / 8; *rsb = 0; }
}

/* lead of one value for R required bytes (cuszx_float.cu:147-170) */
static int cusz_lead(uint32_t x, int R) {
    if (R == 2) return (x >> 16) == 0 ? 2 : ((x >> 24) == 0 ? 1 : 0);
    if (R == 3) return (x >> 8) == 0 ? 3 : ((x >> 16) == 0 ? 2 : ((x >> 24) == 0 ? 1 : 0));
    if (R == 1) return (x >> 24) == 0 ? 1 : 0;
    if (R == 4) return x == 0 ? 4 : ((x >> 8) == 0 ? 3 : ((x >> 16) == 0 ? 2 : ((x >> 24) == 0 ? 1 : 0)));
    return 0;
}

/* stored bytes of value word w (as uchar4 x,y,z,w = bytes 0..3), in stream order */
static int cusz_stored(uint32_t w, int R, int n, uint8_t* out) {
    uint8_t b[4] = {(uint8_t)w, (uint8_t)(w >> 8), (uint8_t)(w >> 16), (uint8_t)(w >> 24)};
    /* first stored byte index for R: R=1 -> 3, R=2 -> 2, R=3 -> 1, R=4 -> 0 */
    if (R < 1 || R > 4 || n <= 0 || n > R) return 0;
    int lo = 4 - R;
    for (int k = 0; k < n; k++) out[k] = b[lo + k];
    return n;
}

/* Compressed size bound for n floats, blocks of bs. */
size_t orc_cusz_bound(size_t n, int bs) {
    size_t nb = n / (size_t)bs;
    size_t m = 4 + 1 + (size_t)bs / 4;
    /* a block's required bytes reach 33 per value when the bound is tiny next to its radius */
    return 13 + (nb + 7) / 8 + (n % (size_t)bs) * 4 + nb * (2 + m + 34 * (size_t)bs) + 16;
}

/* Stream of x[0..n) at bound eb, blocks of bs (a multiple of 32, <= 224); returns its length. */
size_t orc_cusz_compress(const float* x, size_t n, float eb, int bs, uint8_t* out) {
    const size_t nb = n / (size_t)bs, ncb = (size_t)bs / 4, msize = 4 + 1 + ncb;
    uint8_t* st = (uint8_t*)calloc(nb ? nb : 1, 1);
    float* med = (float*)malloc((nb ? nb : 1) * sizeof(float));
    size_t nconst = 0;
    for (size_t b = 0; b < nb; b++) {
        const float* v = x + b * (size_t)bs;
        float mn, mx;
        /* the reference's cross-warp reduction (xor offsets w/2, w/4, .. 1
         * over w = bs/32 warps, szx/src/cuszx_float.cu:248-256) reaches the
         * first 2^floor(log2 w) warps only */
        int wc = 1;
        while (2 * wc <= bs / 32) wc *= 2;
        block_range(v, 32 * wc, &mn, &mx);
        const float radius = (mx - mn) / 2;
        med[b] = mn + radius;
        st[b] = radius <= eb ? 0 : 1;
        nconst += st[b] == 0;
    }
    uint8_t* r = out;
    r[0] = 1; r[1] = 1; r[2] = 1; r[3] = 0; r[4] = (uint8_t)bs;
    r += 5;
    for (int k = 0; k < 8; k++) r[k] = (uint8_t)((uint64_t)nconst >> (56 - 8 * k));
    r += 8;
    const size_t sbytes = (nb + 7) / 8;
    memset(r, 0, sbytes);
    for (size_t b = 0; b < nb; b++) if (st[b]) r[b >> 3] |= (uint8_t)(0x80u >> (b & 7));
    r += sbytes;
    memcpy(r, x + nb * (size_t)bs, (n % (size_t)bs) * 4);
    r += (n % (size_t)bs) * 4;
    uint8_t* c = r;
    for (size_t b = 0; b < nb; b++) if (!st[b]) { memcpy(c, &med[b], 4); c += 4; }
    uint8_t* o = c;
    uint8_t* p = o + (nb - nconst) * 2;
    uint32_t* w = (uint32_t*)malloc((size_t)bs * 4);
    for (size_t b = 0; b < nb; b++) {
        if (!st[b]) continue;
        const float* v = x + b * (size_t)bs;
        float mn, mx;
        /* the reference's cross-warp reduction (xor offsets w/2, w/4, .. 1
         * over w = bs/32 warps, szx/src/cuszx_float.cu:248-256) reaches the
         * first 2^floor(log2 w) warps only */
        int wc = 1;
        while (2 * wc <= bs / 32) wc *= 2;
        block_range(v, 32 * wc, &mn, &mx);
        const float rad = (mx - mn) / 2;
        const int reqLength = 9 + expo(f2u(rad)) - expo(f2u(eb)) + 1;
        int R, rsb;
        req_split(reqLength, &R, &rsb);
        const uint32_t mask = rsb ? ((1u << (32 - rsb)) - 1u) : 0xFFFFFFFFu;
        for (int i = 0; i < bs; i++) w[i] = (f2u(v[i] - med[b]) >> rsb) & mask;
        uint8_t* meta = p;
        memcpy(meta, &med[b], 4);
        meta[4] = (uint8_t)reqLength;
        uint8_t* codes = meta + 5;
        memset(codes, 0, ncb);
        uint8_t* mid = meta + msize;
        int total = 0;
        for (int i = 0; i < bs; i++) total += R - cusz_lead(w[i] ^ (i ? w[i - 1] : 0u), R);
        memset(mid, 0, (size_t)total);   /* required bytes above four are counted but never written */
        total = 0;
        for (int i = 0; i < bs; i++) {
            const int lead = cusz_lead(w[i] ^ (i ? w[i - 1] : 0u), R);
            /* each code byte is the OR of lead << 2(3 - i%4) over its four
             * values, truncated to 8 bits: a lead of 4 sets the low bit of the
             * previous value's code and leaves its own code 0 */
            codes[i >> 2] = (uint8_t)(codes[i >> 2] | (uint8_t)((unsigned)lead << (2 * (3 - (i & 3)))));
            const int sz = R - lead;
            if (R >= 1 && R <= 4) cusz_stored(w[i], R, sz, mid + total);
            total += sz;
        }
        const short off = (short)total;
        memcpy(o, &off, 2);
        o += 2;
        p = mid + total;
    }
    free(w);
    free(st);
    free(med);
    return (size_t)(p - out);
}

/* Decode a stream of n floats into y. Returns 0, or -1 for a malformed stream. */
int orc_cusz_decompress(const uint8_t* s, size_t len, size_t n, float* y) {
    if (len < 13) return -1;
    const int bs = s[4];
    if (bs < 32 || bs % 32) return -1;
    uint64_t nconst = 0;
    for (int k = 0; k < 8; k++) nconst = (nconst << 8) | s[5 + k];
    const size_t nb = n / (size_t)bs, ncb = (size_t)bs / 4, msize = 4 + 1 + ncb;
    if (nconst > nb) return -1;
    const size_t nnc = nb - nconst, sbytes = (nb + 7) / 8, tail = n % (size_t)bs;
    const uint8_t* r = s + 13;
    const uint8_t* sbits = r;
    r += sbytes;
    if ((size_t)(r - s) + tail * 4 + nconst * 4 + nnc * 2 > len) return -1;
    memcpy(y + nb * (size_t)bs, r, tail * 4);
    r += tail * 4;
    const uint8_t* meds = r;
    r += nconst * 4;
    const uint8_t* offs = r;
    const uint8_t* p = r + nnc * 2;
    uint32_t* tmp = (uint32_t*)malloc((size_t)bs * 4);
    int* pos = (int*)malloc((size_t)bs * sizeof(int));
    size_t kc = 0, kn = 0;
    for (size_t b = 0; b < nb; b++) {
        float* out = y + b * (size_t)bs;
        if (!((sbits[b >> 3] >> (7 - (b & 7))) & 1)) {
            float m;
            memcpy(&m, meds + 4 * kc++, 4);
            for (int i = 0; i < bs; i++) out[i] = m;
            continue;
        }
        short off;
        memcpy(&off, offs + 2 * kn++, 2);
        const int leng = (int)off + (int)msize;
        if (leng > bs * 4 || (size_t)(p - s) + (size_t)(leng < 0 ? 0 : leng) > len) { free(tmp); free(pos); return -1; }
        /* the block's bytes as the reference places them: the first leng bytes of a bs*4 buffer */
        uint8_t* blk = (uint8_t*)calloc((size_t)bs * 4, 1);
        memcpy(blk, p, leng < 0 ? 0 : (size_t)leng);
        p += leng < 0 ? 0 : leng;
        float med;
        memcpy(&med, blk, 4);
        const int reqLength = blk[4];
        int R, rsb;
        req_split(reqLength, &R, &rsb);
        int sum = 0;
        for (int i = 0; i < bs; i++) {
            const int lead = (blk[5 + (i >> 2)] >> (6 - ((i & 3) << 1))) & 3;
            const int sz = R - lead;
            sum += sz;   /* inclusive prefix of the mid-byte sizes */
            uint8_t t[4] = {0, 0, 0, 0};
            int ps = 0;
            const int base = (int)msize + sum;
#define MB(k) (base - (k) >= 0 && base - (k) < bs * 4 ? blk[base - (k)] : 0)
            if (R == 2) {
                if (sz == 1) { t[2] = MB(1); ps |= i << 8; }
                else if (sz == 2) { t[3] = MB(1); t[2] = MB(2); ps |= i; ps |= i << 8; }
            } else if (R == 3) {
                if (sz == 1) { t[1] = MB(1); ps |= i << 16; }
                else if (sz == 2) { t[2] = MB(1); t[1] = MB(2); ps |= i << 8; ps |= i << 16; }
                else if (sz == 3) { t[3] = MB(1); t[2] = MB(2); t[1] = MB(3); ps |= i; ps |= i << 8; ps |= i << 16; }
            } else if (R == 1) {
                if (sz == 1) t[3] = MB(1);
                ps |= i;
            } else if (R == 4) {
                if (sz == 1) { t[0] = MB(1); ps |= i << 24; }
                else if (sz == 2) { t[1] = MB(1); t[0] = MB(2); ps |= i << 16; ps |= i << 24; }
                else if (sz == 3) { t[2] = MB(1); t[1] = MB(2); t[0] = MB(3); ps |= i << 8; ps |= i << 16; ps |= i << 24; }
                else if (sz == 4) {
                    t[3] = MB(1); t[2] = MB(2); t[1] = MB(3); t[0] = MB(4);
                    ps |= i; ps |= i << 8; ps |= i << 16; ps |= i << 24;
                }
            }
#undef MB
            tmp[i] = (uint32_t)t[0] | ((uint32_t)t[1] << 8) | ((uint32_t)t[2] << 16) | ((uint32_t)t[3] << 24);
            pos[i] = ps;
        }
        /* latest earlier (or same) value that stored each byte lane: a running
         * per-lane max of the owner indices (lane k of pos <-> byte 3-k) */
        int run = 0;
        for (int i = 0; i < bs; i++) {
            int cur = pos[i];
            for (int k = 0; k < 4; k++) {
                const int sh = 8 * k;
                if (R == 1 && k > 0) break;
                if (R >= 2 && R <= 4 && k >= R) break;
                const int pl = (run >> sh) & 0xFF, cl = (cur >> sh) & 0xFF;
                if (pl > cl) cur = (cur & ~(0xFF << sh)) | (pl << sh);
            }
            if (R == 1) { if (run > cur) cur = run; }
            run = cur;
            pos[i] = cur;
        }
        for (int i = 0; i < bs; i++) {
            const int lead = (blk[5 + (i >> 2)] >> (6 - ((i & 3) << 1))) & 3;
            uint32_t v = tmp[i];
            const int ps = pos[i];
            if (lead >= 1) v = (v & 0x00FFFFFFu) | (tmp[ps & 0xFF] & 0xFF000000u);
            if (lead >= 2) v = (v & 0xFF00FFFFu) | (tmp[(ps >> 8) & 0xFF] & 0x00FF0000u);
            if (lead >= 3) v = (v & 0xFFFF00FFu) | (tmp[(ps >> 16) & 0xFF] & 0x0000FF00u);
            tmp[i] = v;   /* written back before the next value reads owners (owners are earlier values' stored bytes) */
            out[i] = u2f((uint32_t)((int32_t)v << rsb)) + med;
        }
        free(blk);
    }
    free(tmp);
    free(pos);
    return 0;
}
