/* cuSZx entry points (the reference's szx/include/cuszx_entry.h:10-11),
 * provided by libszx_gb300.so: float data, blocks of blockSize values (a
 * multiple of 32 in 32..224), the cuSZx stream format.  The compressed buffer
 * and the decompressed array are malloc'd; the caller frees them.  On
 * failure compress returns NULL and decompress sets *newData = NULL
 * (SZxG_get_last_error tells why). */
#ifndef SZX_GB300_CUSZX_ENTRY_H
#define SZX_GB300_CUSZX_ENTRY_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

unsigned char* cuSZx_fast_compress_args_unpredictable_blocked_float(float* oriData, size_t* outSize,
                                                                    float absErrBound, size_t nbEle, int blockSize);
void cuSZx_fast_decompress_args_unpredictable_blocked_float(float** newData, size_t nbEle, unsigned char* cmpBytes);

#ifdef __cplusplus
}
#endif

#endif
