// szx: command-line compressor / decompressor on the GB300 library, with the
// options, file naming, messages and analysis output of the reference's `szx`
// tool (example/szx.cc:82-618), so that scripts written for it keep working.
//
//   szx -z [out] -f|-d -i <raw file> [-m mode] -M ABS|REL|VR_REL|FXR -A|-R|-C|-T <value>
//   szx -x [out] -f|-d -s <compressed file> -1|-2|-3|-4 <dims> [-i <raw file> -a] [-b|-t]
//
// Compression reads native-endian raw values, converts a REL bound to an
// absolute one outside the timed region (value range times the ratio, as the
// reference tool does), and writes the stream to <raw file>.szx unless a name
// follows -z.  Decompression writes <compressed file>.out (binary, or text
// with -t) unless a name follows -x; -a prints the distortion statistics
// against the original file.  The codec runs on the GPU through
// SZx_fast_compress_args / SZx_fast_decompress.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>

#include <string>

#include "../../include/szx_gb300.h"
#include "../../include/szx_rw.h"

namespace {

double now_s() {
    struct timeval tv;
    gettimeofday(&tv, nullptr);
    return tv.tv_sec + tv.tv_usec * 1e-6;
}

[[noreturn]] void usage() {
    printf("Usage: szx <options>\n");
    printf("Operation:\n");
    printf("  -z [file]   compress (output: <input>.szx unless a file name follows)\n");
    printf("  -x [file]   decompress (output: <compressed>.out unless a file name follows)\n");
    printf("  -h          this help;  -v  version\n");
    printf("Data type:\n");
    printf("  -f          float (single precision);  -d  double\n");
    printf("Layout (fastMode):\n");
    printf("  -m <mode>   1 non-blocked, 2 blocked, 3 blocked with size index (random access),\n");
    printf("              4 blocked, native-endian medians\n");
    printf("Error bound:\n");
    printf("  -M <mode>   ABS | REL (alias VR_REL) | FXR\n");
    printf("  -A <eb>     absolute bound;  -R <ratio>  bound relative to the value range\n");
    printf("  -C <cr>     target compression ratio (FXR);  -T <tol>  its relative tolerance\n");
    printf("Files:\n");
    printf("  -i <file>   raw input (compression; original data for -a)\n");
    printf("  -s <file>   compressed input (decompression)\n");
    printf("  -b          binary output (default);  -t  text output, one value per line\n");
    printf("Dimensions (fastest first):\n");
    printf("  -1 <nx> | -2 <nx> <ny> | -3 <nx> <ny> <nz> | -4 <nx> <ny> <nz> <np>\n");
    printf("Analysis:\n");
    printf("  -a          print distortion statistics after decompression (needs -i)\n");
    printf("Examples:\n");
    printf("  szx -z -f -i data.f32 -3 512 512 512 -M REL -R 1E-3\n");
    printf("  szx -x -f -s data.f32.szx -i data.f32 -3 512 512 512 -a\n");
    exit(0);
}

// Statistics of the reference tool's -a option (example/szx.cc:440-495),
// sequential double sums so the printed digits match.
template <typename T>
void analyse(const T* ori, const T* dec, size_t n, size_t byteLength) {
    T Max = ori[0], Min = ori[0];
    T diffMax = dec[0] > ori[0] ? dec[0] - ori[0] : ori[0] - dec[0];
    double sum1 = 0, sum2 = 0, sum22 = 0;
    for (size_t i = 0; i < n; i++) {
        sum1 += ori[i];
        sum2 += dec[i];
        sum22 += dec[i] * dec[i];
    }
    const double mean1 = sum1 / n, mean2 = sum2 / n;
    double sum3 = 0, sum4 = 0, sum = 0, prodSum = 0, maxpw = 0;
    for (size_t i = 0; i < n; i++) {
        if (Max < ori[i]) Max = ori[i];
        if (Min > ori[i]) Min = ori[i];
        const float err = fabs(dec[i] - ori[i]);
        if (ori[i] != 0) {
            const double rel = err / fabs(ori[i]);
            if (maxpw < rel) maxpw = rel;
        }
        if (diffMax < err) diffMax = err;
        prodSum += (ori[i] - mean1) * (dec[i] - mean2);
        sum3 += (ori[i] - mean1) * (ori[i] - mean1);
        sum4 += (dec[i] - mean2) * (dec[i] - mean2);
        sum += err * err;
    }
    const double std1 = sqrt(sum3 / n), std2 = sqrt(sum4 / n);
    const double ee = prodSum / n, acEff = ee / std1 / std2;
    const double mse = sum / n, range = Max - Min;
    const double psnr = 20 * log10(range) - 10 * log10(mse);
    const double nrmse = sqrt(mse) / range;
    const double cr = 1.0 * n * sizeof(T) / byteLength;
    const double normErr = sqrt(sum), normErr_norm = normErr / sqrt(sum22);
    printf("Min=%.20G, Max=%.20G, range=%.20G\n", (double)Min, (double)Max, range);
    printf("Max absolute error = %.10f\n", (double)diffMax);
    printf("Max relative error = %f\n", diffMax / (Max - Min));
    printf("Max pw relative error = %f\n", maxpw);
    printf("PSNR = %f, NRMSE= %.20G\n", psnr, nrmse);
    printf("normError = %f, normErr_norm = %f\n", normErr, normErr_norm);
    printf("acEff=%f\n", acEff);
    printf("compressionRatio=%f\n", cr);
}

template <typename T>
int compress(int dataType, int fastMode, char* inPath, char* cmpPath, int errMode, float absEb, float rel, float cr,
             float tol, size_t r[5]) {
    size_t n = 0;
    int status = SZx_SCES;
    T* data = dataType == SZx_FLOAT ? (T*)SZx_readFloatData(inPath, &n, &status)
                                    : (T*)SZx_readDoubleData(inPath, &n, &status);
    if (status != SZx_SCES || !data) {
        printf("Error: cannot read the input file: %s\n", inPath);
        return 1;
    }
    if (errMode == REL) {
        // value range -> absolute bound before timing, as the reference tool
        float radius, median;
        const double range = SZx_computeValueRange(data, dataType, n, &radius, &median);
        if (dataType == SZx_FLOAT) absEb = (float)range * rel;
        else absEb = (float)(range * (double)rel);
        errMode = ABS;
    }
    size_t outSize = 0;
    const double t0 = now_s();
    unsigned char* bytes = SZx_fast_compress_args(fastMode, dataType, data, &outSize, errMode, absEb, rel, cr, tol,
                                                  r[4], r[3], r[2], r[1], r[0]);
    const double t = now_s() - t0;
    free(data);
    if (!bytes) {
        printf("Error: compression failed (%s)\n", SZxG_error_string(SZxG_get_last_error()));
        return 1;
    }
    std::string out = cmpPath ? std::string(cmpPath) : std::string(inPath) + ".szx";
    SZx_writeByteData(bytes, outSize, (char*)out.c_str(), &status);
    free(bytes);
    if (status != SZx_SCES) {
        printf("Error: data file %s cannot be written!\n", out.c_str());
        return 1;
    }
    printf("compression time = %f\n", t);
    printf("compressed data file: %s\n", out.c_str());
    return 0;
}

template <typename T>
int decompress(int dataType, int fastMode, char* cmpPath, char* decPath, char* inPath, int binary, int analysis,
               size_t r[5]) {
    size_t n = r[0];
    for (int k = 1; k < 5 && r[k]; k++) n *= r[k];
    if (!SZx_checkFileExistance(cmpPath)) {
        printf("Error: compression file (%s) is not readable.\n", cmpPath);
        return 1;
    }
    int status = SZx_SCES;
    size_t byteLength = 0;
    unsigned char* bytes = SZx_readByteData(cmpPath, &byteLength, &status);
    if (status != SZx_SCES || !bytes) {
        printf("Error: %s cannot be read!\n", cmpPath);
        return 1;
    }
    const double t0 = now_s();
    T* data = (T*)SZx_fast_decompress(fastMode, dataType, bytes, byteLength, r[4], r[3], r[2], r[1], r[0]);
    const double t = now_s() - t0;
    free(bytes);
    if (!data) {
        printf("Error: decompression failed (%s)\n", SZxG_error_string(SZxG_get_last_error()));
        return 1;
    }
    std::string out = decPath ? std::string(decPath) : std::string(cmpPath) + ".out";
    if (binary) {
        if (dataType == SZx_FLOAT) SZx_writeFloatData_inBytes((float*)data, n, (char*)out.c_str(), &status);
        else SZx_writeDoubleData_inBytes((double*)data, n, (char*)out.c_str(), &status);
    } else {
        SZx_writeData(data, dataType, n, (char*)out.c_str(), &status);
    }
    if (status != SZx_SCES) {
        printf("Error: %s cannot be written!\n", out.c_str());
        free(data);
        return 1;
    }
    int rc = 0;
    if (analysis) {
        size_t m = 0;
        T* ori = dataType == SZx_FLOAT ? (T*)SZx_readFloatData(inPath, &m, &status)
                                       : (T*)SZx_readDoubleData(inPath, &m, &status);
        if (status != SZx_SCES || !ori || m < n) {
            printf("Error: %s cannot be read!\n", inPath);
            rc = 1;
        } else {
            analyse<T>(ori, data, n, byteLength);
        }
        free(ori);
    }
    free(data);
    printf("decompression time = %f seconds.\n", t);
    printf("decompressed data file: %s\n", out.c_str());
    return rc;
}

}  // namespace

int main(int argc, char* argv[]) {
    int binary = 1, analysis = 0, isCompression = -1, dataType = SZx_FLOAT;
    int fastMode = SZx_WITH_BLOCK_FAST_CMPR;
    char *inPath = nullptr, *cmpPath = nullptr, *decPath = nullptr;
    const char *ebMode = nullptr, *absS = nullptr, *relS = nullptr, *crS = nullptr;
    float tol = 0;
    size_t r[5] = {0, 0, 0, 0, 0};   // r[0] fastest
    if (argc == 1) usage();
    auto dim = [&](int& i, int k) {
        if (++i == argc || sscanf(argv[i], "%zu", &r[k]) != 1) usage();
    };
    for (int i = 1; i < argc; i++) {
        if (argv[i][0] != '-' || argv[i][1] == 0 || argv[i][2]) usage();
        switch (argv[i][1]) {
            case 'h': usage();
            case 'v': printf("version: %d.%d.%d\n", 1, 1, 0); return 0;
            case 'b': binary = 1; break;
            case 't': binary = 0; break;
            case 'a': analysis = 1; break;
            case 'z':
                isCompression = 1;
                if (i + 1 < argc && argv[i + 1][0] != '-') cmpPath = argv[++i];
                break;
            case 'x':
                isCompression = 0;
                if (i + 1 < argc && argv[i + 1][0] != '-') decPath = argv[++i];
                break;
            case 'f': dataType = SZx_FLOAT; break;
            case 'd': dataType = SZx_DOUBLE; break;
            case 'i': if (++i == argc) usage(); inPath = argv[i]; break;
            case 's': if (++i == argc) usage(); cmpPath = argv[i]; break;
            case '1': dim(i, 0); break;
            case '2': dim(i, 0); dim(i, 1); break;
            case '3': dim(i, 0); dim(i, 1); dim(i, 2); break;
            case '4': dim(i, 0); dim(i, 1); dim(i, 2); dim(i, 3); break;
            case 'm': if (++i == argc) usage(); fastMode = atoi(argv[i]); break;
            case 'M': if (++i == argc) usage(); ebMode = argv[i]; break;
            case 'A': if (++i == argc) usage(); absS = argv[i]; break;
            case 'R': if (++i == argc) usage(); relS = argv[i]; break;
            case 'C': if (++i == argc) usage(); crS = argv[i]; break;
            case 'T': if (++i == argc) usage(); tol = (float)atof(argv[i]); break;
            default: usage();
        }
    }
    if (!inPath && !cmpPath) {
        printf("Error: you need to specify either a raw binary data file or a compressed data file as input\n");
        usage();
    }
    if (isCompression == 1) {
        int errMode = ABS;
        if (ebMode) {
            if (!strcmp(ebMode, "ABS")) errMode = ABS;
            else if (!strcmp(ebMode, "REL") || !strcmp(ebMode, "VR_REL")) errMode = REL;
            else if (!strcmp(ebMode, "FXR")) errMode = FXR;
            else {
                printf("Error: wrong error bound mode setting by using the option '-M'\n");
                usage();
            }
        }
        const float absEb = absS ? (float)atof(absS) : 0.f, rel = relS ? (float)atof(relS) : 0.f;
        const float cr = crS ? (float)atof(crS) : 0.f;
        if (analysis) printf("Error: -a can be only used in decompression.\n");
        return dataType == SZx_FLOAT ? compress<float>(dataType, fastMode, inPath, cmpPath, errMode, absEb, rel, cr,
                                                       tol, r)
                                     : compress<double>(dataType, fastMode, inPath, cmpPath, errMode, absEb, rel, cr,
                                                        tol, r);
    }
    if (isCompression == 0) {
        if (analysis && !inPath) {
            printf("Error: Since you add -a option (analysis), please specify the original data path by -i <path>.\n");
            return 1;
        }
        return dataType == SZx_FLOAT ? decompress<float>(dataType, fastMode, cmpPath, decPath, inPath, binary,
                                                         analysis, r)
                                     : decompress<double>(dataType, fastMode, cmpPath, decPath, inPath, binary,
                                                          analysis, r);
    }
    usage();
}
