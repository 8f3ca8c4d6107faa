// The plan behind SZxG_Batch (batch.cu), shared with the fixed-rate driver
// (learned.cu), which re-targets a compress plan's bounds between runs.
#pragma once
#include <vector>

#include "kernels.h"

using szxg::BlkField;
using szxg::DecField;
using szxg::StreamResult;

struct LfxWork;   // fixed-rate feature scratch (learned.cu)

// Fields of one size class, coded by one persistent launch per kernel with
// the class's launch shape: entries [i0, i1) of the device table, tile map
// entries from map0 on (field indices relative to i0), tile counts.
struct BatchPart {
    int i0 = 0, i1 = 0;
    szxg::LaunchShape shape;
    unsigned long long map0 = 0;
    unsigned long long enc_total = 0, asm_total = 0;   // compress
    unsigned long long idx_total = 0, dec_total = 0;   // decompress
};
constexpr int kMaxBatchParts = 8;

struct SZxG_Batch {
    int direction, mode, dtype, bs, nf;
    void* dev = nullptr;
    BlkField* d_fields = nullptr;     // device table of the fields a run codes (compress), by class
    StreamResult* results = nullptr;  // by field index
    unsigned long long* counters = nullptr;   // [4 * part + 0..3] tile counters of each part's launches
    int* err = nullptr;
    uint8_t* zero = nullptr;          // status words and totals of every field
    size_t zero_bytes = 0;
    DecField* d_dec = nullptr;        // decode: device table, by class
    // compress: every field's table entry (host copy), its size class and
    // the launch shape of every class; the parts of the current run
    std::vector<BlkField> tab;
    std::vector<int> cls;
    std::vector<szxg::LaunchShape> class_shape;
    std::vector<BlkField> run;        // host copy of the run's device table
    std::vector<BatchPart> parts;
    uint32_t* d_tile_field = nullptr;   // per part: field (relative to the part) of every encode / decode tile
    std::vector<uint32_t> h_tile_field;
    LfxWork* lfx = nullptr;
};

// The launch-shape table in effect (per size class, ascending bounds):
// class of a field with n values, and the shape of class k.
int batch_class_of(unsigned long long n, int* nclasses);
szxg::LaunchShape batch_class_shape(int k);

// Upload the table of the fields a compress run codes (h_idx[k] < nf, in
// that order; all fields when h_idx is NULL) with their bounds; ordered on
// stream s.  Returns a cudaError_t.
cudaError_t batch_select(SZxG_Batch* b, int nActive, const int* h_idx, const float* h_eb, cudaStream_t s);
void lfx_free(LfxWork* w);
