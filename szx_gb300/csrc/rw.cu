// File I/O of the SZx API (szx/src/szx_rw.cc:25-372): raw byte / float /
// double files in and out, text output, byte-order swapping for files of the
// other endianness.  Host code only; the codec never depends on it.
//
// Reads and writes go through one open file each in large chunks (the
// reference opens a file twice and makes one fread/fwrite call per file);
// results, status codes and messages follow the reference.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <unistd.h>

#include "../../include/szx_rw.h"

extern "C" int dataEndianType = LITTLE_ENDIAN_DATA;

namespace {

constexpr size_t kChunk = size_t(64) << 20;   // bytes per read / write call

int sys_little() {
    const unsigned one = 1;
    unsigned char b;
    memcpy(&b, &one, 1);
    return b == 1;
}

// Whole file into a malloc'd buffer (n bytes); NULL (and *status = SZx_FERR) on failure.
unsigned char* read_all(const char* path, size_t* n, int* status) {
    FILE* f = path ? fopen(path, "rb") : nullptr;
    if (!f) {
        printf("Failed to open input file. 1\n");
        *status = SZx_FERR;
        return nullptr;
    }
    struct stat st;
    if (fstat(fileno(f), &st) != 0) {
        fclose(f);
        printf("Failed to open input file. 1\n");
        *status = SZx_FERR;
        return nullptr;
    }
    const size_t len = (size_t)st.st_size;
    unsigned char* buf = (unsigned char*)malloc(len ? len : 1);
    size_t got = 0;
    while (buf && got < len) {
        const size_t want = len - got < kChunk ? len - got : kChunk;
        const size_t r = fread(buf + got, 1, want, f);
        if (r == 0) break;
        got += r;
    }
    fclose(f);
    if (!buf || got != len) {
        free(buf);
        printf("Failed to open input file. 2\n");
        *status = SZx_FERR;
        return nullptr;
    }
    *n = len;
    *status = SZx_SCES;
    return buf;
}

void write_all(const void* p, size_t n, const char* path, int* status) {
    FILE* f = path ? fopen(path, "wb") : nullptr;
    if (!f) {
        printf("Failed to open input file. 3\n");
        *status = SZx_FERR;
        return;
    }
    size_t put = 0;
    while (put < n) {
        const size_t want = n - put < kChunk ? n - put : kChunk;
        const size_t w = fwrite((const unsigned char*)p + put, 1, want, f);
        if (w == 0) break;
        put += w;
    }
    const bool ok = put == n && fclose(f) == 0;
    *status = ok ? SZx_SCES : SZx_FERR;
}

template <int W>
void swap_words(unsigned char* p, size_t n) {
    for (size_t i = 0; i + W <= n; i += W)
        for (int k = 0; k < W / 2; k++) {
            const unsigned char t = p[i + k];
            p[i + k] = p[i + W - 1 - k];
            p[i + W - 1 - k] = t;
        }
}

template <typename T>
T* read_values(char* path, size_t* nbEle, int* status, bool system_endian) {
    size_t len = 0;
    unsigned char* b = read_all(path, &len, status);
    if (!b) return nullptr;
    *nbEle = len / sizeof(T);
    if (len == 0 && sizeof(T) == 4) {   // szx/src/szx_rw.cc:186-190: an empty float file is an error
        printf("Error: input file is wrong!\n");
        *status = SZx_FERR;
    }
    if (!system_endian && (dataEndianType == BIG_ENDIAN_DATA) == (bool)sys_little()) swap_words<sizeof(T)>(b, len);
    return (T*)b;
}

template <typename T>
void write_text(const T* data, size_t n, char* path, int* status, const char* fmt) {
    FILE* f = path ? fopen(path, "wb") : nullptr;
    if (!f) {
        printf("Failed to open input file. 3\n");
        *status = SZx_FERR;
        return;
    }
    char s[64];
    for (size_t i = 0; i < n; i++) {
        snprintf(s, sizeof s, fmt, data[i]);
        fputs(s, f);
    }
    fclose(f);
    *status = SZx_SCES;
}

}  // namespace

extern "C" {

int SZx_checkFileExistance(char* filePath) { return filePath && access(filePath, F_OK) != -1 ? 1 : 0; }

size_t SZx_checkFileSize(char* srcFilePath, int* status) {
    struct stat st;
    if (!srcFilePath || stat(srcFilePath, &st) != 0) {
        printf("Failed to open input file. 1\n");
        *status = SZx_FERR;
        return (size_t)-1;
    }
    *status = SZx_SCES;
    return (size_t)st.st_size;
}

unsigned char* SZx_readByteData(char* srcFilePath, size_t* byteLength, int* status) {
    return read_all(srcFilePath, byteLength, status);
}

double* SZx_readDoubleData(char* srcFilePath, size_t* nbEle, int* status) {
    return read_values<double>(srcFilePath, nbEle, status, false);
}

float* SZx_readFloatData(char* srcFilePath, size_t* nbEle, int* status) {
    return read_values<float>(srcFilePath, nbEle, status, false);
}

double* SZx_readDoubleData_systemEndian(char* srcFilePath, size_t* nbEle, int* status) {
    return read_values<double>(srcFilePath, nbEle, status, true);
}

float* SZx_readFloatData_systemEndian(char* srcFilePath, size_t* nbEle, int* status) {
    return read_values<float>(srcFilePath, nbEle, status, true);
}

void SZx_writeByteData(unsigned char* bytes, size_t byteLength, char* tgtFilePath, int* status) {
    write_all(bytes, byteLength, tgtFilePath, status);
}

void SZx_writeDoubleData(double* data, size_t nbEle, char* tgtFilePath, int* status) {
    write_text(data, nbEle, tgtFilePath, status, "%.20G\n");
}

void SZx_writeFloatData(float* data, size_t nbEle, char* tgtFilePath, int* status) {
    // the float is promoted to double for printf, as in the reference
    write_text(data, nbEle, tgtFilePath, status, "%.30G\n");
}

void SZx_writeIntData(int* data, size_t nbEle, char* tgtFilePath, int* status) {
    write_text(data, nbEle, tgtFilePath, status, "%d\n");
}

void SZx_writeData(void* data, int dataType, size_t nbEle, char* tgtFilePath, int* status) {
    if (dataType == 0) {
        SZx_writeFloatData((float*)data, nbEle, tgtFilePath, status);
    } else if (dataType == 1) {
        SZx_writeDoubleData((double*)data, nbEle, tgtFilePath, status);
    } else {
        printf("Error: data type cannot be the types other than SZx_FLOAT or SZx_DOUBLE\n");
        *status = SZx_TERR;
    }
}

void SZx_writeFloatData_inBytes(float* data, size_t nbEle, char* tgtFilePath, int* status) {
    write_all(data, nbEle * sizeof(float), tgtFilePath, status);
}

void SZx_writeDoubleData_inBytes(double* data, size_t nbEle, char* tgtFilePath, int* status) {
    write_all(data, nbEle * sizeof(double), tgtFilePath, status);
}

}  // extern "C"
