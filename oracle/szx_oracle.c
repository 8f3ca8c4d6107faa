/*
 * CPU oracle for the SZx blocked codec -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C restatement of the reference algorithm, written from its observable
 * behaviour (byte layout, arithmetic, rounding) with each function citing the
 * reference code it follows.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py use it; the product never does.
 *
 * Compile with -ffp-contract=off: the reference does plain IEEE float/double
 * adds, subtracts and one multiply, never fused.
 */
#include "szx_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---------------------------------------------------------------- bits */

static inline uint32_t f32_bits(float v) { uint32_t u; memcpy(&u, &v, 4); return u; }
static inline float f32_of(uint32_t u) { float v; memcpy(&v, &u, 4); return v; }
static inline uint64_t f64_bits(double v) { uint64_t u; memcpy(&u, &v, 8); return u; }
static inline double f64_of(uint64_t u) { double v; memcpy(&v, &u, 8); return v; }

/* The reference shifts the IEEE pattern through `lfloat.ivalue` (unsigned int)
 * and `ldouble.lvalue` (unsigned long), szx/include/szx.h:56-68, so every shift
 * in the codec is a LOGICAL shift of the unsigned pattern
 * (szx/src/szx_float.cc:92, szx/src/szx_double.cc:76, szx/src/szxd_float.cc:117-119). */

/* IEEE arithmetic with the NaN results of x86-64 SSE, the reference's native
 * platform: a NaN operand is returned quieted (the first operand when both
 * are NaN), an invalid operation (inf - inf, 0/0, ...) returns the negative
 * "indefinite" quiet NaN, and float<->double conversions carry the payload.
 * Written out explicitly so that the oracle gives the x86 answer on any host
 * (AArch64 prefers signalling NaNs and returns a positive default NaN). */
static inline float nan_rule32(float a, float b) {
    if (a != a) return f32_of(f32_bits(a) | 0x00400000u);
    if (b != b) return f32_of(f32_bits(b) | 0x00400000u);
    return f32_of(0xFFC00000u);
}
static inline double nan_rule64(double a, double b) {
    if (a != a) return f64_of(f64_bits(a) | 0x0008000000000000ull);
    if (b != b) return f64_of(f64_bits(b) | 0x0008000000000000ull);
    return f64_of(0xFFF8000000000000ull);
}
static inline float fsub32(float a, float b) { float r = a - b; return r == r ? r : nan_rule32(a, b); }
static inline float fadd32(float a, float b) { float r = a + b; return r == r ? r : nan_rule32(a, b); }
static inline float fmul32(float a, float b) { float r = a * b; return r == r ? r : nan_rule32(a, b); }
static inline float fdiv32(float a, float b) { float r = a / b; return r == r ? r : nan_rule32(a, b); }
static inline double fsub64(double a, double b) { double r = a - b; return r == r ? r : nan_rule64(a, b); }
static inline double fadd64(double a, double b) { double r = a + b; return r == r ? r : nan_rule64(a, b); }
static inline double fmul64(double a, double b) { double r = a * b; return r == r ? r : nan_rule64(a, b); }
static inline double fdiv64(double a, double b) { double r = a / b; return r == r ? r : nan_rule64(a, b); }
/* cvtsd2ss / cvtss2sd on NaN: top mantissa bits kept, quiet bit set. */
static inline float d2f(double d) {
    if (d == d) return (float)d;
    uint64_t b = f64_bits(d);
    return f32_of((uint32_t)(b >> 32 & 0x80000000u) | 0x7FC00000u | (uint32_t)(b >> 29 & 0x7FFFFFu));
}
static inline double f2d(float f) {
    if (f == f) return (double)f;
    uint32_t b = f32_bits(f);
    return f64_of(((uint64_t)(b & 0x80000000u) << 32) | 0x7FF8000000000000ull | ((uint64_t)(b & 0x7FFFFFu) << 29));
}

/* Big-endian field helpers: floatToBytes / bytesToFloat and sizeToBytes /
 * bytesToLong_bigEndian, szx/src/szx_BytesToolkit.cc:266-317,460-476,805-814. */
static void put_be32(uint8_t* p, uint32_t v) {
    p[0] = (uint8_t)(v >> 24); p[1] = (uint8_t)(v >> 16); p[2] = (uint8_t)(v >> 8); p[3] = (uint8_t)v;
}
static uint32_t get_be32(const uint8_t* p) {
    return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3];
}
static void put_be64(uint8_t* p, uint64_t v) {
    for (int i = 0; i < 8; i++) p[i] = (uint8_t)(v >> (56 - 8 * i));
}
static uint64_t get_be64(const uint8_t* p) {
    uint64_t v = 0;
    for (int i = 0; i < 8; i++) v = (v << 8) | p[i];
    return v;
}
static void put_le32(uint8_t* p, uint32_t v) {
    p[0] = (uint8_t)v; p[1] = (uint8_t)(v >> 8); p[2] = (uint8_t)(v >> 16); p[3] = (uint8_t)(v >> 24);
}
static uint32_t get_le32(const uint8_t* p) {
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

/* getExponent_float: biased exponent field minus 127 (szx_BytesToolkit.cc:335-346). */
static int exponent_f32(float v) { return (int)((f32_bits(v) & 0x7F800000u) >> 23) - 127; }
/* getPrecisionReqLength_double: exponent field of the double minus 1023 (:375-387). */
static int exponent_f64(double v) { return (int)((f64_bits(v) & 0x7FF0000000000000ull) >> 52) - 1023; }

/* computeReqLength_float, szx/src/szx_float.cc:1708-1717. */
static int reqlen_f32(float eb, float radius, float* median) {
    int r = 9 + exponent_f32(radius) - exponent_f64((double)eb) + 1;
    if (r < 9) r = 9;
    if (r > 32) { r = 32; *median = 0; }
    return r;
}
/* computeReqLength_double, szx/src/szx_double.cc:2020-2031 (radius exponent
 * taken from the float radius, szx_double.cc:45). */
static int reqlen_f64(float eb, float radius, float* median) {
    int r = 12 + exponent_f32(radius) - exponent_f64((double)eb);
    if (r < 12) r = 12;
    if (r > 64) { r = 64; *median = 0; }
    return r;
}
/* reqBytesLength / rightShiftBits, szx/src/szx_float.cc:62-79. */
static void split_reqlen(int reqLength, int* R, int* s) {
    *R = reqLength / 8;
    *s = 0;
    if (reqLength % 8) { *s = 8 - reqLength % 8; (*R)++; }
}

/* Leading identical bytes of the XOR (0..3): szx/src/szx_float.cc:96-101 and
 * szx/src/szx_double.cc:80-85 (`x >> k == 0` on the unsigned word is x < 2^k). */
static inline int lead_code32(uint32_t x) {
    return x < (1u << 8) ? 3 : x < (1u << 16) ? 2 : x < (1u << 24) ? 1 : 0;
}
static inline int lead_code64(uint64_t x) {
    return x < (1ull << 40) ? 3 : x < (1ull << 48) ? 2 : x < (1ull << 56) ? 1 : 0;
}

static size_t ceil_div(size_t a, size_t b) { return (a + b - 1) / b; }

/* ---------------------------------------------------------------- range */

/* computeValueRange_float, szx/src/szx_float.cc:478-499. */
float orc_value_range_f32(const float* x, size_t n, float* radius, float* median) {
    float mn = x[0], mx = x[0];
    for (size_t i = 0; i < n; i++) {
        float v = x[i];
        if (mn > v) mn = v;
        else if (mx < v) mx = v;
    }
    float range = fsub32(mx, mn);
    if (radius) { *radius = fdiv32(range, 2); *median = fadd32(mn, *radius); }
    return range;
}

/* computeValueRange_double, szx/src/szx_double.cc:1137-1158: the radius is
 * stored as float and the median is formed from that float radius. */
double orc_value_range_f64(const double* x, size_t n, float* radius, float* median) {
    double mn = x[0], mx = x[0];
    for (size_t i = 0; i < n; i++) {
        double v = x[i];
        if (mn > v) mn = v;
        else if (mx < v) mx = v;
    }
    double range = fsub64(mx, mn);
    if (radius) { *radius = d2f(fdiv64(range, 2)); *median = d2f(fadd64(mn, f2d(*radius))); }
    return range;
}

/* ---------------------------------------------------------------- block stats */

/* computeStateMedianRadius_float, szx/src/szx_float.cc:314-371. */
static int stats_block_f32(const float* x, size_t n, float eb, float* median, float* radius) {
    float mn = x[0], mx = x[0];
    for (size_t j = 1; j < n; j++) {
        float v = x[j];
        if (mn > v) mn = v;
        else if (mx < v) mx = v;
    }
    float range = fsub32(mx, mn);
    float r = fdiv32(range, 2);
    *radius = r;
    *median = fadd32(mn, r);
    return r <= eb ? 0 : 1;
}

/* computeStateMedianRadius_double, szx/src/szx_double.cc:973-1030: statistics
 * in double, median and radius then narrowed to float. */
static int stats_block_f64(const double* x, size_t n, float eb, float* median, float* radius) {
    double mn = x[0], mx = x[0];
    for (size_t j = 1; j < n; j++) {
        double v = x[j];
        if (mn > v) mn = v;
        else if (mx < v) mx = v;
    }
    double range = fsub64(mx, mn);
    double r = fdiv64(range, 2);
    double m = fadd64(mn, r);
    *radius = d2f(r);
    *median = d2f(m);
    return r <= (double)eb ? 0 : 1;
}

/* computeStateMedianRadius_double2 (OpenMP variant), szx/src/szx_double.cc:1120-1135:
 * the median is formed from the float-rounded radius. */
static int stats_block_f64_omp(const double* x, size_t n, float eb, float* median, float* radius) {
    double mn = x[0], mx = x[0];
    for (size_t j = 0; j < n; j++) {
        if (x[j] > mx) mx = x[j];
        if (x[j] < mn) mn = x[j];
    }
    double range = fsub64(mx, mn);
    *radius = d2f(fdiv64(range, 2));
    *median = d2f(fadd64(mn, f2d(*radius)));
    return *radius <= eb ? 0 : 1;
}

size_t orc_block_stats(int dataType, const void* data, size_t n, float eb, int bs,
                       uint8_t* state, float* median, float* radius) {
    size_t nb = ceil_div(n, (size_t)bs), nc = 0;
    for (size_t b = 0; b < nb; b++) {
        size_t off = b * (size_t)bs, len = (n - off < (size_t)bs) ? n - off : (size_t)bs;
        int st = dataType == ORC_FLOAT
                     ? stats_block_f32((const float*)data + off, len, eb, &median[b], &radius[b])
                     : stats_block_f64((const double*)data + off, len, eb, &median[b], &radius[b]);
        state[b] = (uint8_t)st;
        nc += (size_t)(st == 0);
    }
    return nc;
}

/* ---------------------------------------------------------------- block encoders */

/* SZx_fast_compress_args_unpredictable_one_block_float, szx/src/szx_float.cc:49-252.
 * Payload: reqLength u8 | median f32 BE | 2-bit lead codes MSB-first | mid bytes. */
static size_t enc_block_f32(const float* x, size_t n, float eb, float median, float radius, uint8_t* out) {
    int reqLength = reqlen_f32(eb, radius, &median);
    int R, s;
    split_reqlen(reqLength, &R, &s);
    size_t L = ceil_div(n, 4);
    uint8_t* lead = out + 5;
    uint8_t* mid = lead + L;
    memset(lead, 0, L);
    uint32_t prev = 0;
    size_t m = 0;
    for (size_t i = 0; i < n; i++) {
        float d = fsub32(x[i], median);
        uint32_t cur = f32_bits(d) >> s;
        int ld = lead_code32(cur ^ prev);
        lead[i >> 2] |= (uint8_t)(ld << (6 - 2 * (i & 3)));
        for (int b = 4 - R; b <= 3 - ld; b++) mid[m++] = (uint8_t)(cur >> (8 * b));
        prev = cur;
    }
    out[0] = (uint8_t)reqLength;
    put_be32(out + 1, f32_bits(median));
    return 5 + L + m;
}

/* SZx_fast_compress_args_unpredictable_one_block_double, szx/src/szx_double.cc:34-433.
 * The subtraction uses the float median widened to double (:38) even when the
 * stored median is zeroed by the reqLength clamp (:46, :421). */
static size_t enc_block_f64(const double* x, size_t n, float eb, float mValue, float radius, uint8_t* out) {
    double median = f2d(mValue);
    int reqLength = reqlen_f64(eb, radius, &mValue);
    int R, s;
    split_reqlen(reqLength, &R, &s);
    size_t L = ceil_div(n, 4);
    uint8_t* lead = out + 5;
    uint8_t* mid = lead + L;
    memset(lead, 0, L);
    uint64_t prev = 0;
    size_t m = 0;
    for (size_t i = 0; i < n; i++) {
        double d = fsub64(x[i], median);
        uint64_t cur = f64_bits(d) >> s;
        int ld = lead_code64(cur ^ prev);
        lead[i >> 2] |= (uint8_t)(ld << (6 - 2 * (i & 3)));
        for (int b = 8 - R; b <= 7 - ld; b++) mid[m++] = (uint8_t)(cur >> (8 * b));
        prev = cur;
    }
    out[0] = (uint8_t)reqLength;
    put_be32(out + 1, f32_bits(mValue));
    return 5 + L + m;
}

/* ---------------------------------------------------------------- block decoders */

/* SZx_fast_decompress_args_unpredictable_one_block_float, szx/src/szxd_float.cc:34-244.
 * Bytes [4-R .. 3-lead] come from the stream, higher required bytes from the
 * previous value, lower bytes are zero.  Returns the payload size consumed. */
static size_t dec_block_f32(const uint8_t* p, size_t n, float* out) {
    int reqLength = p[0];
    float median = f32_of(get_be32(p + 1));
    int R, s;
    split_reqlen(reqLength, &R, &s);
    size_t L = ceil_div(n, 4);
    const uint8_t* lead = p + 5;
    const uint8_t* q = lead + L;
    uint32_t prev = 0;
    size_t m = 0;
    for (size_t i = 0; i < n; i++) {
        int ld = (lead[i >> 2] >> (6 - 2 * (i & 3))) & 3;
        uint32_t cur = 0;
        for (int b = 4 - R; b <= 3; b++) {
            if (b > 3 - ld) cur |= prev & (0xFFu << (8 * b));
            else cur |= (uint32_t)q[m++] << (8 * b);
        }
        uint32_t sh = cur << s;
        out[i] = fadd32(f32_of(sh), median);
        prev = sh >> s;
    }
    return 5 + L + m;
}

/* SZx_fast_decompress_args_unpredictable_one_block_double, szx/src/szxd_double.cc:25-449.
 * With ref_compat, byte 7 of a reqBytes==5, lead==0 value is taken from the
 * fourth stored byte instead of the fifth, as szxd_double.cc:244 does. */
static size_t dec_block_f64(const uint8_t* p, size_t n, double* out, int ref_compat) {
    int reqLength = p[0];
    double median = f2d(f32_of(get_be32(p + 1)));
    int R, s;
    split_reqlen(reqLength, &R, &s);
    size_t L = ceil_div(n, 4);
    const uint8_t* lead = p + 5;
    const uint8_t* q = lead + L;
    uint64_t prev = 0;
    size_t m = 0;
    for (size_t i = 0; i < n; i++) {
        int ld = (lead[i >> 2] >> (6 - 2 * (i & 3))) & 3;
        uint64_t cur = 0;
        size_t m0 = m;
        for (int b = 8 - R; b <= 7; b++) {
            if (b > 7 - ld) cur |= prev & (0xFFull << (8 * b));
            else cur |= (uint64_t)q[m++] << (8 * b);
        }
        if (ref_compat && R == 5 && ld == 0)
            cur = (cur & 0x00FFFFFFFFFFFFFFull) | ((uint64_t)q[m0 + 3] << 56);
        uint64_t sh = cur << s;
        out[i] = fadd64(f64_of(sh), median);
        prev = sh >> s;
    }
    return 5 + L + m;
}

/* ---------------------------------------------------------------- layouts */

size_t orc_capacity(int fastMode, int dataType, size_t n, int bs) {
    size_t es = dataType == ORC_FLOAT ? 4 : 8;
    if (fastMode == 1) return 17 + ceil_div(n, 4) + es * n;
    size_t nb = ceil_div(n, (size_t)bs);
    size_t per_block = 2 + 4 + 5 + ceil_div((size_t)bs, 4) + es * (size_t)bs;
    return 21 + ceil_div(nb, 8) + nb * per_block;
}

static size_t enc_block(int dt, const void* data, size_t off, size_t len, float eb, float med, float rad, uint8_t* out) {
    return dt == ORC_FLOAT ? enc_block_f32((const float*)data + off, len, eb, med, rad, out)
                           : enc_block_f64((const double*)data + off, len, eb, med, rad, out);
}

/* convertIntArray2ByteArray_fast_1b_args, szx/src/szx_TypeManager.cc:16-40:
 * 1 bit per block, MSB first, 1 = non-constant. */
static void pack_state(const uint8_t* st, size_t nb, uint8_t* out) {
    memset(out, 0, ceil_div(nb, 8));
    for (size_t b = 0; b < nb; b++)
        if (st[b]) out[b >> 3] |= (uint8_t)(0x80u >> (b & 7));
}

/* Blocked layouts.
 *  mode 2  szx/src/szx_float.cc:1059-1139: [1,1,1,0] bs:u8 nbConst:u64BE state medians(BE) payloads
 *  mode 3  szx/src/szx_float.cc:1407-1489: [1,1,1,1] bs:u64BE nbConst:u64BE O:u16[nnc] state medians(BE) payloads
 *  mode 4  szx/src/szx_float.cc:1218-1405: mode-3 layout, medians native (little) endian */
static size_t compress_blocked(int mode, int dt, const void* data, size_t n, float eb, int bs, uint8_t* out, size_t cap) {
    size_t nb = ceil_div(n, (size_t)bs);
    if (cap < orc_capacity(mode, dt, n, bs)) return 0;
    uint8_t* st = (uint8_t*)malloc(nb ? nb : 1);
    float* med = (float*)malloc(sizeof(float) * (nb ? nb : 1));
    float* rad = (float*)malloc(sizeof(float) * (nb ? nb : 1));
    size_t nc = 0;
    for (size_t b = 0; b < nb; b++) {
        size_t off = b * (size_t)bs, len = (n - off < (size_t)bs) ? n - off : (size_t)bs;
        int s;
        if (dt == ORC_FLOAT) s = stats_block_f32((const float*)data + off, len, eb, &med[b], &rad[b]);
        else if (mode == 4) s = stats_block_f64_omp((const double*)data + off, len, eb, &med[b], &rad[b]);
        else s = stats_block_f64((const double*)data + off, len, eb, &med[b], &rad[b]);
        st[b] = (uint8_t)s;
        nc += (size_t)(s == 0);
    }
    size_t nnc = nb - nc, SB = ceil_div(nb, 8);
    uint8_t *r, *O = NULL;
    out[0] = 1; out[1] = 1; out[2] = 1; out[3] = mode == 2 ? 0 : 1;
    if (mode == 2) {
        out[4] = (uint8_t)bs;
        put_be64(out + 5, nc);
        r = out + 13;
    } else {
        put_be64(out + 4, (uint64_t)bs);
        put_be64(out + 12, nc);
        O = out + 20;
        r = O + 2 * nnc;
    }
    pack_state(st, nb, r);
    uint8_t* p = r + SB;
    uint8_t* q = p + 4 * nc;
    size_t k = 0;
    for (size_t b = 0; b < nb; b++) {
        size_t off = b * (size_t)bs, len = (n - off < (size_t)bs) ? n - off : (size_t)bs;
        if (st[b]) {
            size_t sz = enc_block(dt, data, off, len, eb, med[b], rad[b], q);
            q += sz;
            if (O) { O[2 * k] = (uint8_t)sz; O[2 * k + 1] = (uint8_t)(sz >> 8); }
            k++;
        } else {
            if (mode == 4) put_le32(p, f32_bits(med[b]));
            else put_be32(p, f32_bits(med[b]));
            p += 4;
        }
    }
    free(st); free(med); free(rad);
    return (size_t)(q - out);
}

/* Non-blocked layout, SZx_fast_compress_args_unpredictable_float,
 * szx/src/szx_float.cc:1492-1699 (double: szx_double.cc:1593-2011):
 * [1,1,1,0] reqLength:u8 median:f32BE leadBytes:u64BE leads mid. */
static size_t compress_nonblocked(int dt, const void* data, size_t n, float eb, float mValue, float radius,
                                  uint8_t* out, size_t cap) {
    if (cap < orc_capacity(1, dt, n, 1)) return 0;
    out[0] = 1; out[1] = 1; out[2] = 1; out[3] = 0;
    size_t L = ceil_div(n, 4);
    /* the one-block encoders write reqLength | median | leads | mid; the
     * non-blocked stream has an extra u64 lead-array size between median and
     * leads, so encode into place and then open the gap. */
    uint8_t* body = out + 4;
    size_t sz = dt == ORC_FLOAT ? enc_block_f32((const float*)data, n, eb, mValue, radius, body)
                                : enc_block_f64((const double*)data, n, eb, mValue, radius, body);
    memmove(body + 13, body + 5, sz - 5);
    put_be64(body + 5, L);
    return 4 + sz + 8;
}

size_t orc_compress(int fastMode, int dt, const void* data, size_t n, float eb, int bs, uint8_t* out, size_t cap) {
    if (n == 0 || (dt != ORC_FLOAT && dt != ORC_DOUBLE)) return 0;
    if (fastMode == 1) {
        float radius = 0, median = 0;
        if (dt == ORC_FLOAT) orc_value_range_f32((const float*)data, n, &radius, &median);
        else orc_value_range_f64((const double*)data, n, &radius, &median);
        return compress_nonblocked(dt, data, n, eb, median, radius, out, cap);
    }
    if (fastMode < 2 || fastMode > 4 || bs <= 0) return 0;
    if (fastMode == 2 && bs > 255) return 0;
    return compress_blocked(fastMode, dt, data, n, eb, bs, out, cap);
}

size_t orc_fast_compress_args(int fastMode, int dt, const void* data, size_t n, int errBoundMode,
                              float absErrBound, float rel, int bs, uint8_t* out, size_t cap) {
    float eb = absErrBound;
    if (n == 0) return 0;
    if (errBoundMode == 1) {
        /* szx/src/szx.cc:249-253 (float product) and :304-308 (double product
         * narrowed to float); the non-blocked branch :279-285 does the same. */
        if (dt == ORC_FLOAT) {
            float range = orc_value_range_f32((const float*)data, n, NULL, NULL);
            eb = fmul32(range, rel);
        } else {
            double range = orc_value_range_f64((const double*)data, n, NULL, NULL);
            eb = d2f(fmul64(range, f2d(rel)));
        }
    }
    return orc_compress(fastMode, dt, data, n, eb, bs, out, cap);
}

/* convertByteArray2IntArray_fast_1b_args, szx/src/szx_TypeManager.cc:98-140. */
static int state_bit(const uint8_t* r, size_t b) { return (r[b >> 3] >> (7 - (b & 7))) & 1; }

/* SZx_fast_decompress_args_unpredictable_blocked_{randomaccess_,}float,
 * szx/src/szxd_float.cc:247-311 (mode 2), :402-476 (mode 3), :313-399 (mode 4);
 * double szx/src/szxd_double.cc:452-516, :607-681, :518-604. */
static int decompress_blocked(int mode, int dt, const uint8_t* s, size_t len, size_t n, void* outv, int rc) {
    size_t bs, nc;
    const uint8_t* r;
    if (mode == 2) {
        if (len < 13) return -1;
        bs = s[4];
        nc = get_be64(s + 5);
        r = s + 13;
    } else {
        if (len < 20) return -1;
        bs = get_be64(s + 4);
        nc = get_be64(s + 12);
        r = s + 20;
    }
    if (bs == 0) return -2;
    size_t nb = ceil_div(n, bs);
    if (nc > nb) return -3;
    size_t nnc = nb - nc, SB = ceil_div(nb, 8);
    const uint8_t* O = mode == 2 ? NULL : r;
    if (O) r += 2 * nnc;
    const uint8_t* p = r + SB;
    const uint8_t* q = p + 4 * nc;
    if ((size_t)(q - s) > len) return -4;
    size_t k = 0, j = 0;
    for (size_t b = 0; b < nb; b++) {
        size_t off = b * bs, blen = (n - off < bs) ? n - off : bs;
        if (state_bit(r, b)) {
            size_t used = dt == ORC_FLOAT ? dec_block_f32(q, blen, (float*)outv + off)
                                          : dec_block_f64(q, blen, (double*)outv + off, rc);
            if (O) used = (size_t)O[2 * k] | ((size_t)O[2 * k + 1] << 8);
            q += used;
            k++;
        } else {
            float m = mode == 4 ? f32_of(get_le32(p + 4 * j)) : f32_of(get_be32(p + 4 * j));
            j++;
            if (dt == ORC_FLOAT) for (size_t e = 0; e < blen; e++) ((float*)outv)[off + e] = m;
            else for (size_t e = 0; e < blen; e++) ((double*)outv)[off + e] = f2d(m);
        }
    }
    return 0;
}

/* SZx_fast_decompress_args_unpredictable_float, szx/src/szxd_float.cc:478-662;
 * double szx/src/szxd_double.cc:683-1114. */
static int decompress_nonblocked(int dt, const uint8_t* s, size_t len, size_t n, void* outv, int rc) {
    if (len < 17) return -1;
    size_t L = get_be64(s + 9);
    if (L != ceil_div(n, 4)) return -2;
    /* Re-assemble a one-block payload view: reqLength | median | leads | mid. */
    uint8_t* tmp = (uint8_t*)malloc(len);
    memcpy(tmp, s + 4, 5);
    memcpy(tmp + 5, s + 17, len - 17);
    if (dt == ORC_FLOAT) dec_block_f32(tmp, n, (float*)outv);
    else dec_block_f64(tmp, n, (double*)outv, rc);
    free(tmp);
    return 0;
}

int orc_decompress(int fastMode, int dt, const uint8_t* s, size_t len, size_t n, void* out, int rc) {
    if (n == 0) return 0;
    if (fastMode == 1) return decompress_nonblocked(dt, s, len, n, out, rc);
    if (fastMode >= 2 && fastMode <= 4) return decompress_blocked(fastMode, dt, s, len, n, out, rc);
    return -10;
}

/* ---------------------------------------------------------------- OpenMP baseline */

size_t orc_compress_m3_omp(int dt, const void* data, size_t n, float eb, int bs, uint8_t* out, size_t cap,
                           int nthreads) {
    if (n == 0 || bs <= 0 || cap < orc_capacity(3, dt, n, bs)) return 0;
    size_t nb = ceil_div(n, (size_t)bs), es = dt == ORC_FLOAT ? 4 : 8;
    size_t slot = 5 + ceil_div((size_t)bs, 4) + es * (size_t)bs;
    uint8_t* st = (uint8_t*)malloc(nb);
    float* med = (float*)malloc(4 * nb);
    uint32_t* sz = (uint32_t*)malloc(4 * nb);
    size_t* pos = (size_t*)malloc(sizeof(size_t) * (nb + 1));
    size_t* rank = (size_t*)malloc(sizeof(size_t) * (nb + 1));
    uint8_t* tmp = (uint8_t*)malloc(slot * nb);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    long long B = (long long)nb;
#pragma omp parallel for schedule(static)
    for (long long b = 0; b < B; b++) {
        size_t off = (size_t)b * bs, len = (n - off < (size_t)bs) ? n - off : (size_t)bs;
        float rad;
        int s = dt == ORC_FLOAT ? stats_block_f32((const float*)data + off, len, eb, &med[b], &rad)
                                : stats_block_f64((const double*)data + off, len, eb, &med[b], &rad);
        st[b] = (uint8_t)s;
        sz[b] = s ? (uint32_t)enc_block(dt, data, off, len, eb, med[b], rad, tmp + (size_t)b * slot) : 0;
    }
    pos[0] = 0; rank[0] = 0;
    for (size_t b = 0; b < nb; b++) { pos[b + 1] = pos[b] + sz[b]; rank[b + 1] = rank[b] + st[b]; }
    size_t nnc = rank[nb], nc = nb - nnc, SB = ceil_div(nb, 8);
    out[0] = 1; out[1] = 1; out[2] = 1; out[3] = 1;
    put_be64(out + 4, (uint64_t)bs);
    put_be64(out + 12, nc);
    uint8_t* O = out + 20;
    uint8_t* R = O + 2 * nnc;
    pack_state(st, nb, R);
    uint8_t* P = R + SB;
    uint8_t* Q = P + 4 * nc;
#pragma omp parallel for schedule(static)
    for (long long b = 0; b < B; b++) {
        if (st[b]) {
            memcpy(Q + pos[b], tmp + (size_t)b * slot, sz[b]);
            O[2 * rank[b]] = (uint8_t)sz[b];
            O[2 * rank[b] + 1] = (uint8_t)(sz[b] >> 8);
        } else {
            put_be32(P + 4 * ((size_t)b - rank[b]), f32_bits(med[b]));
        }
    }
    size_t total = (size_t)(Q - out) + pos[nb];
    free(st); free(med); free(sz); free(pos); free(rank); free(tmp);
    return total;
}

int orc_decompress_m3_omp(int dt, const uint8_t* s, size_t len, size_t n, void* out, int nthreads) {
    if (n == 0) return 0;
    if (len < 20) return -1;
    size_t bs = get_be64(s + 4), nc = get_be64(s + 12);
    if (bs == 0) return -2;
    size_t nb = ceil_div(n, bs);
    if (nc > nb) return -3;
    size_t nnc = nb - nc, SB = ceil_div(nb, 8);
    const uint8_t* O = s + 20;
    const uint8_t* R = O + 2 * nnc;
    const uint8_t* P = R + SB;
    const uint8_t* Q = P + 4 * nc;
    size_t* pos = (size_t*)malloc(sizeof(size_t) * (nb + 1));
    size_t* rank = (size_t*)malloc(sizeof(size_t) * (nb + 1));
    size_t acc = 0, k = 0;
    for (size_t b = 0; b < nb; b++) {
        rank[b] = k;
        pos[b] = acc;
        if (state_bit(R, b)) { acc += (size_t)O[2 * k] | ((size_t)O[2 * k + 1] << 8); k++; }
    }
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    long long B = (long long)nb;
#pragma omp parallel for schedule(static)
    for (long long b = 0; b < B; b++) {
        size_t off = (size_t)b * bs, blen = (n - off < bs) ? n - off : bs;
        if (state_bit(R, (size_t)b)) {
            if (dt == ORC_FLOAT) dec_block_f32(Q + pos[b], blen, (float*)out + off);
            else dec_block_f64(Q + pos[b], blen, (double*)out + off, 0);
        } else {
            float m = f32_of(get_be32(P + 4 * ((size_t)b - rank[b])));
            if (dt == ORC_FLOAT) for (size_t e = 0; e < blen; e++) ((float*)out)[off + e] = m;
            else for (size_t e = 0; e < blen; e++) ((double*)out)[off + e] = f2d(m);
        }
    }
    free(pos); free(rank);
    return 0;
}

/* ---------------------------------------------------------------- fixed rate */

/* Sampled-block statistics of computeRadiusBuffer_float / _double
 * (szx/src/szx_float.cc:254-312, szx/src/szx_double.cc:437-495): every
 * rate-th block of bs values (nbEle / (rate*bs) of them), its float radius and
 * median (double data: computed in double, stored as float), and the sampled
 * value range (the global extremes start at data[0]). */
static void fxr_sample_t(int dt, const void* x, size_t n, int bs, int rate, float** rads, float** meds,
                         float* range) {
    size_t stride = (size_t)rate * bs, nsamp = n / stride;
    *rads = (float*)malloc(sizeof(float) * (nsamp + 1));
    *meds = (float*)malloc(sizeof(float) * (nsamp + 1));
    if (dt == ORC_FLOAT) {
        const float* xf = (const float*)x;
        float gmin = xf[0], gmax = xf[0];
        for (size_t i = 0; i < nsamp; i++) {
            const float* d = xf + i * stride;
            float mn = d[0], mx = d[0];
            for (int j = 1; j < bs; j++) {
                float v = d[j];
                if (mn > v) mn = v;
                else if (mx < v) mx = v;
            }
            if (gmax < mx) gmax = mx;
            if (gmin > mn) gmin = mn;
            float r = fdiv32(fsub32(mx, mn), 2);
            (*rads)[i] = r;
            (*meds)[i] = fadd32(mn, r);
        }
        *range = fsub32(gmax, gmin);
    } else {
        const double* xd = (const double*)x;
        double gmin = xd[0], gmax = xd[0];
        for (size_t i = 0; i < nsamp; i++) {
            const double* d = xd + i * stride;
            double mn = d[0], mx = d[0];
            for (int j = 1; j < bs; j++) {
                double v = d[j];
                if (mn > v) mn = v;
                else if (mx < v) mx = v;
            }
            if (gmax < mx) gmax = mx;
            if (gmin > mn) gmin = mn;
            double r = fdiv64(fsub64(mx, mn), 2);
            (*rads)[i] = d2f(r);
            (*meds)[i] = d2f(fadd64(mn, r));
        }
        *range = d2f(fsub64(gmax, gmin));
    }
}

/* One call of estimateCRbasedonErrorBound_buffered_float / _double
 * (szx/src/szx_float.cc:501-584, szx/src/szx_double.cc:497-580) over the
 * sampled blocks.  The expression types follow the reference exactly; the
 * double variant subtracts the (possibly zeroed) float median widened to
 * double, and its sizes use 65/8 and 8*bs. */
static float fxr_cr_t(int dt, const void* x, size_t n, int bs, int rate, const float* rads, const float* meds,
                      float eb, size_t* sumReq, size_t* sumLead, size_t* nconst) {
    size_t nsamp = n / ((size_t)bs * rate);
    size_t ncst = 0;
    *sumLead = 0;
    *sumReq = 0;
    float metadata = 13.0 * bs / n;
    float block_cost = dt == ORC_FLOAT ? 33.0 / 8 : 65.0 / 8;
    for (size_t i = 0; i < nsamp; i++) {
        float median = meds[i], radius = rads[i];
        if (radius <= eb) { ncst++; continue; }
        int reqLength = dt == ORC_FLOAT ? reqlen_f32(eb, radius, &median) : reqlen_f64(eb, radius, &median);
        int R, s;
        split_reqlen(reqLength, &R, &s);
        *sumReq += (size_t)R;
        int acc = 0;
        if (dt == ORC_FLOAT) {
            const float* d = (const float*)x + i * (size_t)bs * rate;
            uint32_t prev = 0;
            for (int j = 0; j < bs; j++) {
                uint32_t cur = f32_bits(fsub32(d[j], median)) >> s;
                int ld = lead_code32(cur ^ prev);
                acc += ld >= R ? R : ld;
                prev = cur;
            }
        } else {
            const double* d = (const double*)x + i * (size_t)bs * rate;
            uint64_t prev = 0;
            for (int j = 0; j < bs; j++) {
                uint64_t cur = f64_bits(fsub64(d[j], f2d(median))) >> s;
                int ld = lead_code64(cur ^ prev);
                acc += ld >= R ? R : ld;
                prev = cur;
            }
        }
        *sumLead += (size_t)acc;
    }
    if (nconst) *nconst = ncst;
    /* 0/0 (every sampled block constant) as x86 computes it, on any host */
    float avgReq = fdiv64(1.0 * (*sumReq), (double)(nsamp - ncst));
    float avgLead = fdiv64(1.0 * (*sumLead), (double)(nsamp - ncst));
    float p_lambda = fdiv64(1.0 * ncst, (double)nsamp);
    float cr;
    if (dt == ORC_FLOAT)
        cr = 4 * bs / (metadata + block_cost + (1 + (0.25 + avgReq) * bs - avgLead) * (1 - p_lambda));
    else
        cr = 8 * bs / (metadata + block_cost + (1 + (0.25 + avgReq) * bs - avgLead) * (1 - p_lambda));
    return cr;
}

float orc_fxr_range(int dataType, const void* x, size_t n, int bs) {
    float *rads, *meds, range;
    fxr_sample_t(dataType, x, n, bs, 10, &rads, &meds, &range);
    free(rads); free(meds);
    return range;
}

float orc_fxr_estimate_cr(int dataType, const void* x, size_t n, int bs, float eb, size_t* sumReq, size_t* sumLead,
                          size_t* nconst) {
    float *rads, *meds, range;
    fxr_sample_t(dataType, x, n, bs, 10, &rads, &meds, &range);
    float cr = fxr_cr_t(dataType, x, n, bs, 10, rads, meds, eb, sumReq, sumLead, nconst);
    free(rads); free(meds);
    return cr;
}

float orc_fxr_estimate_cr_f32(const float* x, size_t n, int bs, float eb, size_t* sumReq, size_t* sumLead) {
    return orc_fxr_estimate_cr(ORC_FLOAT, x, n, bs, eb, sumReq, sumLead, NULL);
}

/* estimateErrorBoundbasedonCR_buffered_float / _double
 * (szx/src/szx_float.cc:684-832, szx/src/szx_double.cc:682-830), started from
 * 1% of the sampled range as szx/src/szx_float.cc:941 does. */
float orc_fxr_bound(int dataType, const void* x, size_t n, float target, float tolerance, int bs) {
    float *rads, *meds, range;
    const int rate = 10, stride = 8, iters = 10;
    fxr_sample_t(dataType, x, n, bs, rate, &rads, &meds, &range);
    float errorBound = range * 1E-2;
    size_t sumReq[20] = {0}, sumLead[20] = {0};
    float bounds[20], ratios[20];
    int k = 0, i, j;
    size_t sr = 0, sl = 0;
    float CR = fxr_cr_t(dataType, x, n, bs, rate, rads, meds, errorBound, &sr, &sl, NULL);
    sumReq[k] = sr; sumLead[k] = sl; bounds[k] = errorBound; ratios[k] = CR; k++;
    float result = 0;
    if (fabs(target - CR) < tolerance) { result = errorBound; goto done; }
    float left = 0, right = 0;
    int found = 0;
    float targetTol = target * tolerance;
    if (target < CR) {
        left = errorBound / stride;
        right = errorBound;
        for (i = 0; i < iters; i++) {
            CR = fxr_cr_t(dataType, x, n, bs, rate, rads, meds, left, &sr, &sl, NULL);
            sumReq[k] = sr; sumLead[k] = sl; bounds[k] = left; ratios[k] = CR; k++;
            if (fabs(CR - target) < targetTol) { found = 1; result = left; break; }
            if (target > CR) break;
            right = left;
            left = left / stride;
        }
    } else if (target > CR) {
        left = errorBound;
        right = errorBound * stride;
        for (i = 0; i < iters; i++) {
            CR = fxr_cr_t(dataType, x, n, bs, rate, rads, meds, right, &sr, &sl, NULL);
            sumReq[k] = sr; sumLead[k] = sl; bounds[k] = right; ratios[k] = CR; k++;
            if (fabs(target - CR) < targetTol) { found = 1; result = right; break; }
            if (target < CR) break;
            left = right;
            right = right * stride;
        }
    }
    if (!found) {
        for (i = 0; i < iters; i++) {
            errorBound = (left + right) / 2;
            CR = fxr_cr_t(dataType, x, n, bs, rate, rads, meds, errorBound, &sr, &sl, NULL);
            int appeared = 0;
            for (j = 0; j < k; j++)
                if (sumReq[j] == sr && sumLead[j] == sl) { appeared = 1; break; }
            float min_err = 10000000;
            int index = 0;
            for (j = 0; j < k; j++) {
                float e = fabs(ratios[j] - target);
                if (e < min_err) { min_err = e; index = j; }
            }
            if (appeared) { result = bounds[index]; break; }
            sumReq[k] = sr; sumLead[k] = sl; bounds[k] = errorBound; ratios[k] = CR; k++;
            if (fabs(CR - target) < targetTol) { result = errorBound; break; }
            if (target > CR) left = errorBound;
            else right = errorBound;
        }
    }
done:
    free(rads); free(meds);
    return result;
}

float orc_fxr_bound_f32(const float* x, size_t n, float target, float tolerance, int bs) {
    return orc_fxr_bound(ORC_FLOAT, x, n, target, tolerance, bs);
}
