// The plan behind SZxG_Batch (batch.cu), shared with the fixed-rate driver
// (learned.cu), which re-targets a compress plan's bounds between runs.
#pragma once
#include <vector>

#include "kernels.h"

using szxg::BlkField;
using szxg::DecField;
using szxg::StreamResult;

struct LfxWork;   // fixed-rate feature scratch (learned.cu)

struct SZxG_Batch {
    int direction, mode, dtype, bs, nf;
    void* dev = nullptr;
    BlkField* d_fields = nullptr;     // device table of the fields a run codes (compress)
    BlkField one;                     // the field when a run codes one field
    StreamResult* results = nullptr;  // by field index
    unsigned long long* counters = nullptr;   // [0..3] tile counters, then the error word
    int* err = nullptr;
    uint8_t* zero = nullptr;          // status words and totals of every field
    size_t zero_bytes = 0;
    unsigned long long enc_total = 0, asm_total = 0;
    DecField* d_dec = nullptr;        // decode: device table
    unsigned long long idx_total = 0, dec_total = 0;
    // compress: every field's table entry (host copy) and how many a run codes
    std::vector<BlkField> tab;
    int nrun = 0;
    uint32_t* d_tile_field = nullptr;   // field (index into the run's table) of every encode tile
    std::vector<uint32_t> h_tile_field;
    LfxWork* lfx = nullptr;
};

// Upload the table of the fields a compress run codes (h_idx[k] < nf, in
// that order; all fields when h_idx is NULL) with their bounds; ordered on
// stream s.  Returns a cudaError_t.
cudaError_t batch_select(SZxG_Batch* b, int nActive, const int* h_idx, const float* h_eb, cudaStream_t s);
void lfx_free(LfxWork* w);
