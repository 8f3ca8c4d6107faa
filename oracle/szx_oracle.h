/*
 * CPU oracle for the SZx blocked codec -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference algorithm (szcompressor/SZx), used by
 * tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg: the
 * oracle GPU results are compared with, and the timed CPU stand-in.  The
 * product library never links,
 * loads or calls it.  Every function cites the reference file:line it follows.
 *
 * Parity of this restatement is pinned against the reference library itself,
 * compiled from the reference sources (oracle/Makefile target `ref`), through
 * the golden vectors under tests/golden/.
 */
#ifndef SZX_ORACLE_H
#define SZX_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_FLOAT 0
#define ORC_DOUBLE 1

/* computeValueRange_float / _double: szx/src/szx_float.cc:478-499,
 * szx/src/szx_double.cc:1137-1158.  radius/median may be NULL. */
float  orc_value_range_f32(const float* x, size_t n, float* radius, float* median);
double orc_value_range_f64(const double* x, size_t n, float* radius, float* median);

/* Worst-case stream size of a layout (the reference's own output buffer is
 * only sizeof(T)*n, szx/src/szx_float.cc:1413-1416, which overflows when the
 * ratio drops below 1). */
size_t orc_capacity(int fastMode, int dataType, size_t n, int blockSize);

/* Encode with an absolute bound into out[0..cap).  fastMode 1: non-blocked
 * (global median/radius computed here, as szx/src/szx.cc:277-287 does);
 * 2: blocked; 3: blocked + size index; 4: mode-3 layout with native-endian
 * constant medians (the OpenMP variant).  Returns the stream size, 0 on error. */
size_t orc_compress(int fastMode, int dataType, const void* data, size_t n, float absErrBound,
                    int blockSize, uint8_t* out, size_t cap);

/* Mirror of SZx_fast_compress_args' bound handling (szx/src/szx.cc:231-348):
 * errBoundMode 0 = ABS, 1 = REL (bound = range * ratio, float product for
 * float data, double product narrowed to float for double data). */
size_t orc_fast_compress_args(int fastMode, int dataType, const void* data, size_t n, int errBoundMode,
                              float absErrBound, float relBoundRatio, int blockSize, uint8_t* out, size_t cap);

/* Decode.  ref_compat != 0 reproduces the reference double decoder's byte
 * slip for reqBytes == 5 with no leading zero bytes (szx/src/szxd_double.cc:244,
 * :906), so the oracle can be checked against the reference decoder itself;
 * ref_compat == 0 decodes the stream as the encoder wrote it.  Returns 0 on
 * success, negative on a malformed stream. */
int orc_decompress(int fastMode, int dataType, const uint8_t* stream, size_t len, size_t n, void* out,
                   int ref_compat);

/* Per-block statistics, szx/src/szx_float.cc:314-371 / szx/src/szx_double.cc:973-1030.
 * Returns the number of constant blocks. */
size_t orc_block_stats(int dataType, const void* data, size_t n, float absErrBound, int blockSize,
                       uint8_t* state, float* median, float* radius);

/* Block-parallel (OpenMP) mode-3 codec producing exactly the serial mode-3
 * stream; the parallel structure follows the reference OpenMP variant
 * (szx/src/szx_float.cc:1271-1400, szx/src/szxd_float.cc:358-378).  Used as
 * the timed CPU baseline. */
size_t orc_compress_m3_omp(int dataType, const void* data, size_t n, float absErrBound, int blockSize,
                           uint8_t* out, size_t cap, int nthreads);
int    orc_decompress_m3_omp(int dataType, const uint8_t* stream, size_t len, size_t n, void* out,
                             int nthreads);

/* Fixed-rate bound search of the reference: computeRadiusBuffer_float
 * (szx/src/szx_float.cc:254-312), estimateCRbasedonErrorBound_buffered_float
 * (:501-584), estimateErrorBoundbasedonCR_buffered_float (:684-832). */
float orc_fxr_estimate_cr_f32(const float* x, size_t n, int blockSize, float errorBound,
                              size_t* sumReqNbBytes, size_t* sumActualLead);
float orc_fxr_bound_f32(const float* x, size_t n, float ratio, float tolerance, int blockSize);
/* The same for either type (szx/src/szx_double.cc:437-495, :497-580, :682-830). */
float orc_fxr_range(int dataType, const void* x, size_t n, int blockSize);
float orc_fxr_estimate_cr(int dataType, const void* x, size_t n, int blockSize, float errorBound,
                          size_t* sumReqNbBytes, size_t* sumActualLead, size_t* nbConstant);
float orc_fxr_bound(int dataType, const void* x, size_t n, float ratio, float tolerance, int blockSize);

#ifdef __cplusplus
}
#endif
#endif
