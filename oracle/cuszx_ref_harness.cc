// Test infrastructure only: C entry points around the reference's own cuSZx
// codec (szx/src/cuszx_entry.cu:72-209), compiled from the reference sources
// by `make -C oracle cuszx_ref REF=<tree>` on a machine with a GPU, to make
// golden vectors for the cuSZx format (tests/golden/make_cuszx_golden.py).
#include <stdlib.h>
#include <string.h>

#include "cuszx_entry.h"

extern "C" {

// Stream of x (n floats, bound eb, block size bs) into out[cap]; its size, 0
// when it does not fit.
size_t refcusz_compress(const float* x, size_t n, float eb, int bs, unsigned char* out, size_t cap) {
    float* copy = (float*)malloc(n * sizeof(float));
    memcpy(copy, x, n * sizeof(float));
    size_t sz = 0;
    unsigned char* s = cuSZx_fast_compress_args_unpredictable_blocked_float(copy, &sz, eb, n, bs);
    free(copy);
    if (!s) return 0;
    const size_t got = sz <= cap ? sz : 0;
    if (got) memcpy(out, s, sz);
    free(s);
    return got;
}

// n decoded floats of stream s into y.
int refcusz_decompress(const unsigned char* s, size_t len, size_t n, float* y) {
    unsigned char* copy = (unsigned char*)malloc(len);
    memcpy(copy, s, len);
    float* out = nullptr;
    cuSZx_fast_decompress_args_unpredictable_blocked_float(&out, n, copy);
    free(copy);
    if (!out) return -1;
    memcpy(y, out, n * sizeof(float));
    free(out);
    return 0;
}

}  // extern "C"
