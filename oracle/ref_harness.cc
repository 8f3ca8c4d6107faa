// Test-only harness around the reference SZx library, compiled from the
// reference's own sources by oracle/Makefile into oracle/_ref/.
//
// It exposes the blocked assemblers with an explicit block size (the public
// C entry point fixes blockSize = 128, szx/src/szx.cc:234) under a distinct
// `ref_` prefix, so that the golden-vector generator and the tests can call
// them through ctypes.  Nothing in the product links or loads this file.
#include <stdlib.h>
#include <stddef.h>
#include "szx.h"
#include "szx_float.h"
#include "szx_double.h"
#include "szxd_float.h"
#include "szxd_double.h"

extern "C" {

// fastMode 2 / 3 / 4 stream with an explicit block size and ABS bound.
// szx/src/szx_float.cc:1059 (mode 2), :1407 (mode 3), :1218 (mode 4);
// szx/src/szx_double.cc:1160, :1509, :1320.
unsigned char* ref_compress_blocked(int fastMode, int dataType, void* data, size_t nbEle,
                                    float absErrBound, int blockSize, size_t* outSize) {
    if (dataType == SZx_FLOAT) {
        float* d = (float*)data;
        if (fastMode == 2) return szx::SZx_fast_compress_args_unpredictable_blocked_float(d, outSize, absErrBound, nbEle, blockSize);
        if (fastMode == 3) return szx::SZx_fast_compress_args_unpredictable_blocked_randomaccess_float(d, outSize, absErrBound, nbEle, blockSize);
        if (fastMode == 4) return szx::SZx_fast_compress_args_unpredictable_blocked_randomaccess_float_openmp(d, outSize, absErrBound, nbEle, blockSize);
    } else {
        double* d = (double*)data;
        if (fastMode == 2) return szx::SZx_fast_compress_args_unpredictable_blocked_double(d, outSize, absErrBound, nbEle, blockSize);
        if (fastMode == 3) return szx::SZx_fast_compress_args_unpredictable_blocked_randomaccess_double(d, outSize, absErrBound, nbEle, blockSize);
        if (fastMode == 4) return szx::SZx_fast_compress_args_unpredictable_blocked_randomaccess_double_openmp(d, outSize, absErrBound, nbEle, blockSize);
    }
    return NULL;
}

// Fixed-rate search of the reference (szx/src/szx_float.cc:921-949) with the
// error bound it settled on reported back, so that the oracle's restatement of
// the estimator can be compared number for number.
float ref_fxr_bound_float(float* data, size_t nbEle, float ratio, float tolerance, int blockSize) {
    float* radius = NULL; float* median = NULL; float* buffer = NULL;
    float range = szx::computeRadiusBuffer_float(data, nbEle, 10, blockSize, &radius, &median, &buffer);
    float eb = szx::estimateErrorBoundbasedonCR_buffered_float(ratio, tolerance, 10, range * 1E-2, blockSize, nbEle,
                                                               buffer, median, radius);
    free(radius); free(median); free(buffer);
    return eb;
}

// The same search for double data (szx/src/szx_double.cc:918-940).
float ref_fxr_bound_double(double* data, size_t nbEle, float ratio, float tolerance, int blockSize) {
    float* radius = NULL; float* median = NULL; double* buffer = NULL;
    float range = szx::computeRadiusBuffer_double(data, nbEle, 10, blockSize, &radius, &median, &buffer);
    float eb = szx::estimateErrorBoundbasedonCR_buffered_double(ratio, tolerance, 10, range * 1E-2, blockSize, nbEle,
                                                                buffer, median, radius);
    free(radius); free(median); free(buffer);
    return eb;
}

// Sampled range and one ratio estimate (szx/src/szx.cc:475-498 C entry points).
float ref_fxr_estimate(int dataType, void* data, size_t nbEle, int blockSize, float eb, size_t* sumReq,
                       size_t* sumLead, float* range) {
    float* radius = NULL; float* median = NULL; void* buffer = NULL;
    *range = computeRadiusBuffer(data, dataType, nbEle, 10, blockSize, &radius, &median, &buffer);
    float cr = estimateCRbasedonErrorBound_buffered(dataType, eb, buffer, median, radius, 10, blockSize, nbEle,
                                                    sumReq, sumLead);
    free(radius); free(median); free(buffer);
    return cr;
}

void ref_free(void* p) { free(p); }

}
