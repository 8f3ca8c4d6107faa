/* File I/O of the SZx library (the reference's szx/include/szx_rw.h:26-43),
 * provided by libszx_gb300.so with the same names, arguments and status
 * codes.  Raw files hold native-endian values unless dataEndianType says
 * otherwise (the reference's global, szx/src/szx.cc:36); text output writes
 * one value per line (%.30G float, %.20G double).  Buffers returned are
 * malloc'd; the caller frees them. */
#ifndef SZX_GB300_RW_H
#define SZX_GB300_RW_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SZx_SCES 0   /* successful */
#define SZx_NSCS -1  /* not successful */
#define SZx_FERR -2  /* failed to open a file */
#define SZx_TERR -3  /* wrong data type */

#define LITTLE_ENDIAN_DATA 0
#define BIG_ENDIAN_DATA 1

/* Byte order of the raw files read by SZx_readFloatData / SZx_readDoubleData
 * (LITTLE_ENDIAN_DATA by default). */
extern int dataEndianType;

int SZx_checkFileExistance(char* filePath);
size_t SZx_checkFileSize(char* srcFilePath, int* status);
unsigned char* SZx_readByteData(char* srcFilePath, size_t* byteLength, int* status);
double* SZx_readDoubleData(char* srcFilePath, size_t* nbEle, int* status);
float* SZx_readFloatData(char* srcFilePath, size_t* nbEle, int* status);
double* SZx_readDoubleData_systemEndian(char* srcFilePath, size_t* nbEle, int* status);
float* SZx_readFloatData_systemEndian(char* srcFilePath, size_t* nbEle, int* status);
void SZx_writeByteData(unsigned char* bytes, size_t byteLength, char* tgtFilePath, int* status);
void SZx_writeDoubleData(double* data, size_t nbEle, char* tgtFilePath, int* status);
void SZx_writeFloatData(float* data, size_t nbEle, char* tgtFilePath, int* status);
void SZx_writeIntData(int* data, size_t nbEle, char* tgtFilePath, int* status);
void SZx_writeData(void* data, int dataType, size_t nbEle, char* tgtFilePath, int* status);
void SZx_writeFloatData_inBytes(float* data, size_t nbEle, char* tgtFilePath, int* status);
void SZx_writeDoubleData_inBytes(double* data, size_t nbEle, char* tgtFilePath, int* status);

#ifdef __cplusplus
}
#endif

#endif
