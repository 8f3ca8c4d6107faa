/*
 * szx_gb300 -- SZx's blocked error-bounded codec on one NVIDIA GB300 (sm_103a).
 *
 * Part 1 is a drop-in for the reference's C API (szcompressor/SZx,
 * szx/include/szx.h): same symbol names, argument meaning, stream format and
 * ownership rules.  Outputs are malloc'd host buffers the caller free()s;
 * failures return NULL (or 0) and leave a code readable with
 * SZxG_get_last_error().  All compute runs on the current CUDA device; there
 * is no CPU fallback.
 *
 * Part 2 (SZxG_*) is this library's own device-pointer interface: explicit
 * block size, caller-provided device buffers and workspace, a CUDA stream,
 * and no host synchronisation on the compress path.
 *
 * Plain pointers and sizes only; a CUDA stream is passed as void*.
 */
#ifndef SZX_GB300_H
#define SZX_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Constants of the reference, szx/include/szx_defines.h:19-21,36-37,54-57. */
#define SZx_FLOAT 0
#define SZx_DOUBLE 1
#define ABS 0
#define REL 1
#define FXR 2
#define SZx_NO_BLOCK_FAST_CMPR 1
#define SZx_WITH_BLOCK_FAST_CMPR 2
#define SZx_RANDOMACCESS_FAST_CMPR 3
#define SZx_OPENMP_FAST_CMPR 4

/* =====================================================================
 * Part 1: reference C API (szx/include/szx.h:28-102)
 * ===================================================================== */

/* szx/include/szx.h:72, szx/src/szx.cc:41-71 */
int SZx_computeDimension(size_t r5, size_t r4, size_t r3, size_t r2, size_t r1);
/* szx/include/szx.h:73, szx/src/szx.cc:73-101 */
size_t SZx_computeDataLength(size_t r5, size_t r4, size_t r3, size_t r2, size_t r1);
/* szx/include/szx.h:74, szx/src/szx.cc:109-229 */
int SZx_filterDimension(size_t r5, size_t r4, size_t r3, size_t r2, size_t r1, size_t* correctedDimension);

/* szx/include/szx.h:75-76, szx/src/szx.cc:231-348.  Block size 128 as in the
 * reference.  fastMode 1, 2, 3, 4; ABS / REL / FXR.  Returns a malloc'd stream. */
unsigned char* SZx_fast_compress_args(int fastMode, int dataType, void* data, size_t* outSize, int errBoundMode,
                                      float absErrBound, float relBoundRatio, float compressionRatio, float tolerance,
                                      size_t r5, size_t r4, size_t r3, size_t r2, size_t r1);

/* szx/include/szx.h:78, szx/src/szx.cc:378-430.  fastMode 1, 2, 3, 4 (the
 * reference's dispatcher decodes 1, 3, 4; fastMode 2 streams, which FXR
 * produces, are decoded here too).  Returns a malloc'd array of
 * SZx_computeDataLength(r5..r1) values. */
void* SZx_fast_decompress(int fastMode, int dataType, unsigned char* bytes, size_t byteLength, size_t r5, size_t r4,
                          size_t r3, size_t r2, size_t r1);

/* szx/include/szx.h:79, szx/src/szx.cc:432-438 */
double SZx_computeValueRange(void* oriData, int dataType, size_t length, float* radius, float* medianValue);

/* szx/include/szx.h:80-82, szx/src/szx.cc:441-448: mode-4 layout (native-endian
 * constant medians) with an explicit block size. */
unsigned char* SZx_fast_compress_args_unpredictable_blocked_randomaccess_openmp(void* oriData, int dataType,
                                                                                size_t* outSize, float absErrBound,
                                                                                size_t nbEle, int blockSize);
/* szx/include/szx.h:83, szx/src/szx.cc:450-456 */
void* SZx_fast_decompress_args_unpredictable_blocked_randomaccess_openmp(int dataType, size_t nbEle,
                                                                         unsigned char* cmpBytes);

/* szx/include/szx.h:85, szx/src/szx.cc:458-464.  Fixed-rate bound search of
 * the reference (sampled-block ratio estimator + bracketing + bisection). */
float SZx_estimateErrorBoundbasedonCR(int dataType, float targetCompressionRatio, float tolerance, void* data,
                                      float initErrorBound, int blockSize, size_t nbEle);

/* szx/include/szx.h:87, szx/src/szx.cc:466-473: mode-2 layout, explicit block size. */
unsigned char* SZx_fast_compress_args_unpredictable_blocked(void* oriData, int dataType, size_t* outSize,
                                                            float absErrBound, size_t nbEle, int blockSize);

/* szx/include/szx.h:89, szx/src/szx.cc:475-485: copies every samplingRate-th
 * block into *buffer and returns the sampled value range. */
float computeRadiusBuffer(void* oriData, int dataType, size_t nbEle, int samplingRate, int blockSize,
                          float** radiusArray, float** mediusArray, void* buffer);

/* szx/include/szx.h:91-92, szx/src/szx.cc:487-498 */
float estimateCRbasedonErrorBound_buffered(int dataType, float errorBound, void* buffer, float* medianArray,
                                          float* radiusArray, int samplingRate, int blockSize, size_t nbEle,
                                          size_t* sumReqNbBytes, size_t* sum_actual_leadNumbers);

/* szx/include/szx.h:95, szx/src/szx.cc:501-512: mode-2 stream into a caller
 * buffer; returns its size (0 for double data, as the reference does). */
size_t SZx_fast_compress_args_unpredictable_blocked_args(void* oriData, int dataType, unsigned char* outputBytes,
                                                         float absErrBound, size_t nbEle, int blockSize);

/* szx/include/szx.h:96, szx/src/szx.cc:514-524: *(float**)newData receives a
 * malloc'd array (float data only, as in the reference). */
void SZx_fast_decompress_args_unpredictable_blocked(void* newData, int dataType, size_t nbEle,
                                                   unsigned char* cmpBytes);

/* =====================================================================
 * Part 2: device-pointer interface (no counterpart in the reference)
 * ===================================================================== */

/* Error codes. */
#define SZXG_OK 0
#define SZXG_ERR_LOOKBACK 1   /* a device-wide scan gave up waiting (bounded spin) */
#define SZXG_ERR_CAPACITY 2   /* output buffer too small */
#define SZXG_ERR_STREAM 3     /* malformed or truncated stream */
#define SZXG_ERR_ARG 4        /* invalid argument */
#define SZXG_ERR_CUDA 5       /* CUDA runtime error */
#define SZXG_ERR_UNSUPPORTED 6
#define SZXG_ERR_TOO_LARGE 7      /* input beyond the fixed scratch of SZxG_compress_noalloc */

int SZxG_get_last_error(void);
const char* SZxG_error_string(int code);

/* Where a compressed stream sits in a device output buffer. */
typedef struct {
    unsigned long long offset;   /* stream start, relative to the output buffer */
    unsigned long long size;     /* stream length in bytes */
    unsigned long long nb_const; /* constant blocks (blocked layouts) */
    float eb;                    /* absolute bound used */
    int status;                  /* SZXG_* code */
} SZxG_StreamInfo;

/* Worst-case output bytes for one compress call (stream + alignment slack). */
size_t SZxG_compress_bound(int fastMode, int dataType, size_t nbEle, int blockSize);
/* Device scratch bytes one compress or decompress call needs. */
size_t SZxG_workspace_size(int fastMode, int dataType, size_t nbEle, int blockSize);

/* Enqueue a compress of nbEle device values on `stream`.  The stream lands at
 * d_out + info.offset; *d_info (device memory) receives the info.  Nothing is
 * synchronised.  blockSize 1..256 (2..255 for fastMode 2). */
int SZxG_compress(int fastMode, int dataType, const void* d_data, size_t nbEle, int blockSize, int errBoundMode,
                  float absErrBound, float relBoundRatio, void* d_out, size_t outCapacity, void* d_workspace,
                  size_t workspaceBytes, SZxG_StreamInfo* d_info, void* stream);

/* Enqueue a decompress of a device-resident stream into nbEle device values.
 * blockSize must be the stream's (blocked layouts); 0 reads it from the
 * stream with a synchronous 20-byte copy. */
int SZxG_decompress(int fastMode, int dataType, const void* d_stream, size_t streamBytes, size_t nbEle,
                    int blockSize, void* d_out, void* d_workspace, size_t workspaceBytes, void* stream);

/* Read back the status a previous SZxG_* call left in its workspace (waits
 * for `stream`). */
int SZxG_workspace_status(const void* d_workspace, void* stream);

/* No counterpart in the reference.  SZxG_compress for the blocked layouts
 * (fastMode 2, 3, 4) that allocates nothing: its scratch is a fixed array in
 * device memory that every GPU loading this library holds until exit (about
 * 7.2 MiB).  For callers that may not call cudaMalloc -- applications whose
 * own pool allocator owns all device memory, or loops that cannot pay for
 * cudaMalloc's device-wide synchronisation.  At most 1,048,576 blocks per
 * call (ceil(nbEle/blockSize); 134,217,728 values at blockSize 128), else
 * SZXG_ERR_TOO_LARGE before any GPU work.  All calls on a device share the
 * array: calls that overlap on the GPU race, so order them on one stream.
 * The first call on a device resolves the array's address; make it before
 * any stream capture.  Output and info as SZxG_compress; the same error codes,
 * plus SZXG_ERR_UNSUPPORTED for fastMode 1 and SZXG_ERR_TOO_LARGE beyond the
 * limit; every return sets SZxG_get_last_error(). */
int SZxG_compress_noalloc(int fastMode, int dataType, const void* d_data, size_t nbEle, int blockSize,
                          int errBoundMode, float absErrBound, float relBoundRatio, void* d_out, size_t outCapacity,
                          SZxG_StreamInfo* d_info, void* stream);

/* Host-buffer codec with an explicit block size (same stream as Part 1). */
unsigned char* SZxG_compress_host(int fastMode, int dataType, const void* data, size_t nbEle, int blockSize,
                                  int errBoundMode, float absErrBound, float relBoundRatio, size_t* outSize);
void* SZxG_decompress_host(int fastMode, int dataType, const unsigned char* bytes, size_t byteLength, size_t nbEle);

/* Host-buffer codec into caller-provided host memory (pinned memory gives
 * full-speed copies).  Returns the stream size, 0 on failure. */
size_t SZxG_compress_host_into(int fastMode, int dataType, const void* data, size_t nbEle, int blockSize,
                               int errBoundMode, float absErrBound, float relBoundRatio, unsigned char* out,
                               size_t outCapacity);
int SZxG_decompress_host_into(int fastMode, int dataType, const unsigned char* bytes, size_t byteLength, size_t nbEle,
                              void* out);

/* ---------------------------------------------------------------- batches
 * Many fields of one type and block size coded by ONE persistent launch per
 * kernel over a device work queue of (field, block-range) tiles, instead of
 * a launch sequence per field (no counterpart in the reference, which codes
 * one array per call; each field's stream is exactly what
 * SZx_fast_compress_args / SZxG_compress would produce for it).
 *
 * SZxG_batch_create plans the batch once: it checks the fields, lays out
 * every field's scratch, allocates it (one cudaMalloc) and uploads the field
 * table.  SZxG_batch_run then only enqueues memsets, kernels and (optionally)
 * a device-to-device copy of the per-field results on `stream`, so it can be
 * captured into a CUDA graph and replayed; the fields' buffers must stay
 * valid while the plan is used.  Runs of one plan must not overlap. */
typedef struct {
    const void* in;          /* compress: nbEle values (device); decompress: the stream (device) */
    size_t nbEle;            /* values */
    size_t inBytes;          /* decompress: stream bytes; compress: ignored */
    float absErrBound;       /* compress: absolute bound */
    int reserved;
    void* out;               /* compress: stream buffer, >= SZxG_compress_bound bytes; decompress: nbEle values */
    size_t outCapacity;      /* bytes at out */
} SZxG_Field;

typedef struct SZxG_Batch SZxG_Batch;

/* direction 0: compress (fastMode 2, 3, 4); 1: decompress (fastMode 3, 4).
 * Returns NULL on failure (SZxG_get_last_error). */
SZxG_Batch* SZxG_batch_create(int direction, int fastMode, int dataType, int blockSize, int nFields,
                              const SZxG_Field* fields);
/* Enqueue the batch; per-field results go to d_info[nFields] when d_info is
 * not NULL: compress, where the stream sits (out + offset, size bytes);
 * decompress, the field's status (a malformed stream fails only its own
 * field, whose values are then unspecified) and size = nbEle * element size.
 * Each decompress stream's blockSize must equal the batch's. */
int SZxG_batch_run(SZxG_Batch* batch, SZxG_StreamInfo* d_info, void* stream);
/* Wait for `stream` and report the batch's error word (0: all fields fine). */
int SZxG_batch_status(SZxG_Batch* batch, void* stream);
void SZxG_batch_destroy(SZxG_Batch* batch);

/* Launch shapes by field-size class (no counterpart in the reference).  A
 * batch groups its fields by size class -- the first entry whose maxValues is
 * >= the field's value count, the last entry for larger fields -- and codes
 * each class with one persistent launch per kernel of that class's shape:
 * encoder tile variant (0: 16 KiB of input per tile, 8 warps per CTA; 1:
 * 8 KiB, 4 warps -- float blocks of 65..128 values only, else as 0) and CTAs
 * per SM of the encoder and the decoder (0: as many as fit).  Shapes change
 * how the work is cut, never a stream.  The table in effect is read from the
 * autotuner's file (tuning/batch_shapes.txt beside the library, or the file
 * the SZXG_TUNING_FILE environment variable names); without one, a single
 * class with the default shape.  At most 8 entries, maxValues ascending;
 * n == 0 reloads the file.  Applies to batches created afterwards. */
typedef struct {
    unsigned long long maxValues;
    int encTileVariant;
    int encCtasPerSm;
    int decCtasPerSm;
    int reserved;
} SZxG_LaunchShape;
int SZxG_set_launch_shapes(const SZxG_LaunchShape* table, int n);
/* The table in effect (up to cap entries into table); returns its length. */
int SZxG_get_launch_shapes(SZxG_LaunchShape* table, int cap);

/* Change the bounds of a compress plan's fields and which fields a run codes:
 * fieldIndex[k] (k < nActive) in that order, all fields when fieldIndex is
 * NULL (nActive == nFields); absErrBound[k] is field fieldIndex[k]'s new bound
 * (NULL keeps the bounds).  Ordered on `stream`.  A graph captured before a
 * call that changes the set of fields must be captured again; one that only
 * changes bounds stays valid (the bounds are read from device memory). */
int SZxG_batch_set_bounds(SZxG_Batch* batch, int nActive, const int* fieldIndex, const float* absErrBound,
                          void* stream);

/* ---------------------------------------------------------------- fixed rate, learned
 * A small network predicts the bound that gives a target compression ratio
 * from 32 features of every 10th block; real compress passes of the whole
 * batch judge it (float fields, blockSize 128).  Features of a field, row
 * layout of X (SZXG_FXR_FEATURES floats): see szx_gb300/csrc/learned.cu. */
#define SZXG_FXR_FEATURES 32
typedef struct SZxG_Mlp SZxG_Mlp;
size_t SZxG_mlp_param_count(void);
SZxG_Mlp* SZxG_mlp_create(unsigned long long seed);          /* Xavier-uniform initial weights */
void SZxG_mlp_destroy(SZxG_Mlp* mlp);
int SZxG_mlp_get_params(const SZxG_Mlp* mlp, float* params, size_t count);
int SZxG_mlp_set_params(SZxG_Mlp* mlp, const float* params, size_t count);
/* d_out[i] = the network's output for feature row i: the predicted miss
 * log2(real ratio / target) at the sampled curve's crossing (feature 1). */
int SZxG_mlp_forward(const SZxG_Mlp* mlp, const float* d_X, size_t n, float* d_out, void* stream);
/* Gradient of the mean squared error over n rows (trainable parameters, in
 * order W1 b1 W2 b2 W3 b3 W4 b4) and the error itself (synchronous). */
int SZxG_mlp_gradient(SZxG_Mlp* mlp, const float* d_X, const float* d_y, size_t n, float* d_grad, float* loss,
                      void* stream);
/* Adam on minibatches; input statistics and output bias set from the data. */
int SZxG_mlp_train(SZxG_Mlp* mlp, const float* d_X, const float* d_y, size_t n, int epochs, int batch, float lr,
                   unsigned long long seed, float* loss, void* stream);
/* Feature rows of a compress plan's fields: row r describes field
 * fieldOfRow[r] for targetRatio[r]; h_range[nFields] receives each field's
 * sampled range (synchronous). */
int SZxG_batch_features(SZxG_Batch* batch, int nRows, const int* fieldOfRow, const float* targetRatio, float* d_X,
                        float* h_range, void* stream);
/* Choose every field's bound for targetRatio[f] within `tolerance` by real
 * compress passes of the plan (mlp NULL: plain bisection; else prediction,
 * one re-targeted prediction, then bisection), leaving the chosen streams in
 * the fields' buffers.  Outputs per field: bound, achieved ratio, passes. */
int SZxG_batch_fixed_rate(SZxG_Batch* batch, const SZxG_Mlp* mlp, const float* targetRatio, float tolerance,
                          int maxPasses, float* eb, float* ratio, int* passes, SZxG_StreamInfo* d_info,
                          void* stream);

/* Launch tracing: CUDA events around every kernel this library enqueues.
 * enable(1) starts (and clears) a trace, enable(0) stops and clears it.
 * collect() waits for the recorded events and writes, per kernel name, the
 * summed milliseconds and launch count; names are '\n'-separated in `names`.
 * Returns the number of kernels reported. */
/* Failure detection (no counterpart in the reference): runs the device-wide
 * look-back the codecs use to place variable-length payloads (scan 0: the
 * encoders' 64-bit status words; scan 1: the decoders' 32-bit words) over
 * ntiles (<= 4096) one-warp tiles, tile t contributing t + 1, with tile
 * `withheld` (-1: none) never publishing, and waits bounded by spinLimit
 * polls.  Returns SZXG_ERR_LOOKBACK when a wait gave up, else SZXG_OK with
 * prefix[t] = t(t+1)/2 (host array of ntiles, may be NULL).  Synchronous. */
int SZxG_selftest_lookback(int scan, int ntiles, int withheld, unsigned spinLimit, unsigned long long* prefix,
                           void* stream);

void SZxG_trace_enable(int on);
int SZxG_trace_collect(char* names, size_t names_len, double* ms, unsigned long long* counts, int max_kernels);

#ifdef __cplusplus
}
#endif
#endif /* SZX_GB300_H */
