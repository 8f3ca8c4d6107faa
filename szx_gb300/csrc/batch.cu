// Batches: many fields of one type and block size coded by one persistent
// launch per kernel over a device work queue of (field, block-range) tiles.
// Compress (direction 0): fastMode 2, 3, 4.  Decompress (direction 1):
// fastMode 3 and 4, whose size index makes every stream's payload offsets a
// scan; a fastMode-2 stream needs the single-stream boundary search.
//
// The blocked kernels take a table of fields (a single-field call is a table
// of one): a launch-wide tile index maps to (field, local tile) by a binary
// search over the fields' first tiles, and every field keeps its own
// look-back status words, totals, scratch and stream.  Tiles are handed out
// in field order from one atomic counter, so a field's tiles are always
// acquired before any later field's, which is all the per-field look-back
// needs to make progress.  This file plans a batch (layout of the per-field
// scratch in one allocation, the field table on the device) and runs it as a
// handful of memsets and launches that a CUDA graph can capture.
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "../../include/szx_gb300.h"
#include "batch.h"

using namespace szxg;

namespace {

size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

SZxG_Batch* fail(int code) {
    set_last_error(code);
    return nullptr;
}

}  // namespace

cudaError_t batch_select(SZxG_Batch* b, int nActive, const int* h_idx, const float* h_eb, cudaStream_t s) {
    if (b->direction != 0 || nActive < 1 || nActive > b->nf) return cudaErrorInvalidValue;
    if (!h_idx && nActive != b->nf) return cudaErrorInvalidValue;
    const size_t tb = (size_t)blocked_tile_blocks(b->dtype, b->bs);
    std::vector<BlkField> run((size_t)nActive);
    unsigned long long et = 0, at = 0;
    for (int k = 0; k < nActive; k++) {
        const int f = h_idx ? h_idx[k] : k;
        if (f < 0 || f >= b->nf) return cudaErrorInvalidValue;
        if (h_eb) b->tab[f].eb = h_eb[k];
        BlkField F = b->tab[f];
        F.enc_tiles = (F.nb + tb - 1) / tb; F.enc_tile0 = et; et += F.enc_tiles;
        F.asm_tiles = (F.nb + kAsmBlocksPerTile - 1) / kAsmBlocksPerTile; F.asm_tile0 = at; at += F.asm_tiles;
        run[(size_t)k] = F;
    }
    b->enc_total = et;
    b->asm_total = at;
    b->one = run[0];
    b->nrun = nActive;
    // pageable sources: each copy is staged before the call returns, ordered after earlier runs on s
    cudaError_t e = cudaMemcpyAsync(b->d_fields, run.data(), sizeof(BlkField) * (size_t)nActive,
                                    cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess || nActive == 1) return e;
    b->h_tile_field.resize(et);
    for (int k = 0; k < nActive; k++)
        for (unsigned long long t = 0; t < run[(size_t)k].enc_tiles; t++) b->h_tile_field[run[(size_t)k].enc_tile0 + t] = (uint32_t)k;
    return cudaMemcpyAsync(b->d_tile_field, b->h_tile_field.data(), 4 * et, cudaMemcpyHostToDevice, s);
}

extern "C" {

int SZxG_batch_set_bounds(SZxG_Batch* b, int nActive, const int* fieldIndex, const float* absErrBound, void* stream) {
    if (!b || b->direction != 0) { set_last_error(SZXG_ERR_ARG); return SZXG_ERR_ARG; }
    cudaError_t e = batch_select(b, nActive, fieldIndex, absErrBound, (cudaStream_t)stream);
    if (e == cudaErrorInvalidValue) { set_last_error(SZXG_ERR_ARG); return SZXG_ERR_ARG; }
    if (e != cudaSuccess) { cudaGetLastError(); set_last_error(SZXG_ERR_CUDA); return SZXG_ERR_CUDA; }
    set_last_error(SZXG_OK);
    return SZXG_OK;
}

static SZxG_Batch* create_decode(int fastMode, int dataType, int blockSize, int nFields, const SZxG_Field* fields) {
    if (fastMode != kRandomAccess && fastMode != kRandomAccessNative) return fail(SZXG_ERR_UNSUPPORTED);
    if (blockSize < 1 || blockSize > 256) return fail(SZXG_ERR_ARG);
    const size_t nf = (size_t)nFields, es = dataType == 0 ? 4 : 8;
    const size_t tb = (size_t)blocked_dec_tile_blocks(dataType, blockSize);
    // layout: table | results | counters+err | headers | zeroed (errors, look-back words) | offsets, ranks
    size_t off = 0;
    const size_t o_tab = off; off += a256(sizeof(DecField) * nf);
    const size_t o_res = off; off += a256(sizeof(StreamResult) * nf);
    const size_t o_ctr = off; off += 256;
    const size_t o_hdr = off; off += a256(sizeof(BlockedHdr) * nf);
    unsigned long long dec_tiles_all = 0;
    for (size_t f = 0; f < nf; f++) dec_tiles_all += ((fields[f].nbEle + blockSize - 1) / blockSize + tb - 1) / tb;
    const size_t o_map = off; off += a256(4 * dec_tiles_all);
    const size_t o_zero = off;
    const size_t o_err = off; off += a256(sizeof(int) * nf);
    std::vector<size_t> o_st(nf), o_p(nf), o_rw(nf), ta(nf), tbw(nf);
    for (size_t f = 0; f < nf; f++) {
        const SZxG_Field& F = fields[f];
        if (!F.in || !F.out || F.nbEle == 0) return fail(SZXG_ERR_ARG);
        if (F.outCapacity < F.nbEle * es) return fail(SZXG_ERR_CAPACITY);
        const size_t nb = (F.nbEle + blockSize - 1) / blockSize, nw = (nb + 31) / 32;
        ta[f] = (nb + kIdxPerTile - 1) / kIdxPerTile;
        tbw[f] = (nw + kIdxPerTile - 1) / kIdxPerTile;
        o_st[f] = off; off += a256(3 * 8 * (ta[f] + tbw[f]));
    }
    const size_t zero_bytes = off - o_zero;
    for (size_t f = 0; f < nf; f++) {
        const size_t nb = (fields[f].nbEle + blockSize - 1) / blockSize;
        o_p[f] = off; off += a256(8 * (nb + 1));
        o_rw[f] = off; off += a256(4 * (nb / 32 + 2));
    }
    SZxG_Batch* b = new SZxG_Batch();
    b->direction = 1; b->mode = fastMode; b->dtype = dataType; b->bs = blockSize; b->nf = nFields;
    if (cudaMalloc(&b->dev, off) != cudaSuccess) {
        cudaGetLastError();
        delete b;
        return fail(SZXG_ERR_CUDA);
    }
    uint8_t* base = (uint8_t*)b->dev;
    b->results = (StreamResult*)(base + o_res);
    b->counters = (unsigned long long*)(base + o_ctr);
    b->err = (int*)(base + o_ctr + 64);
    b->zero = base + o_zero;
    b->zero_bytes = zero_bytes;
    std::vector<DecField> tab(nf);
    unsigned long long it = 0, dt = 0;
    for (size_t f = 0; f < nf; f++) {
        const SZxG_Field& S = fields[f];
        DecField& D = tab[f];
        memset(&D, 0, sizeof D);
        D.s = (const uint8_t*)S.in; D.len = S.inBytes; D.n = S.nbEle;
        D.nb = (S.nbEle + blockSize - 1) / blockSize;
        D.out = S.out;
        D.hdr = (BlockedHdr*)(base + o_hdr) + f;
        D.P = (unsigned long long*)(base + o_p[f]);
        D.RW = (uint32_t*)(base + o_rw[f]);
        unsigned long long* st = (unsigned long long*)(base + o_st[f]);
        for (int k = 0; k < 3; k++) D.stA[k] = st + k * ta[f];
        st += 3 * ta[f];
        for (int k = 0; k < 3; k++) D.stB[k] = st + k * tbw[f];
        D.idxA_tiles = ta[f]; D.idxB_tiles = tbw[f];
        D.idx_tile0 = it; it += ta[f] + tbw[f];
        D.dec_tiles = (D.nb + tb - 1) / tb;
        D.dec_tile0 = dt; dt += D.dec_tiles;
        D.err = (int*)(base + o_err) + f;
    }
    b->idx_total = it;
    b->dec_total = dt;
    b->d_dec = (DecField*)(base + o_tab);
    b->d_tile_field = (uint32_t*)(base + o_map);
    b->h_tile_field.resize(dt);
    for (size_t f = 0; f < nf; f++)
        for (unsigned long long t = 0; t < tab[f].dec_tiles; t++) b->h_tile_field[tab[f].dec_tile0 + t] = (uint32_t)f;
    if (cudaMemcpy(b->d_tile_field, b->h_tile_field.data(), 4 * dt, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(b->d_dec, tab.data(), sizeof(DecField) * nf, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(b->dev);
        delete b;
        return fail(SZXG_ERR_CUDA);
    }
    set_last_error(SZXG_OK);
    return b;
}

SZxG_Batch* SZxG_batch_create(int direction, int fastMode, int dataType, int blockSize, int nFields,
                              const SZxG_Field* fields) {
    if (direction == 1 && nFields >= 1 && fields && (dataType == 0 || dataType == 1))
        return create_decode(fastMode, dataType, blockSize, nFields, fields);
    if (direction != 0 || nFields < 1 || !fields || (dataType != 0 && dataType != 1)) return fail(SZXG_ERR_ARG);
    if (fastMode != kBlocked && fastMode != kRandomAccess && fastMode != kRandomAccessNative)
        return fail(SZXG_ERR_UNSUPPORTED);
    if (blockSize < 1 || blockSize > 256 || (fastMode == kBlocked && blockSize > 255)) return fail(SZXG_ERR_ARG);
    const size_t nf = (size_t)nFields;
    const size_t tb = (size_t)blocked_tile_blocks(dataType, blockSize);
    const size_t hdr = fastMode == kBlocked ? 13 : 20;
    // layout: table | results | counters+err | zeroed status words and totals | scratch
    size_t off = 0;
    const size_t o_tab = off; off += a256(sizeof(BlkField) * nf);
    const size_t o_res = off; off += a256(sizeof(StreamResult) * nf);
    const size_t o_ctr = off; off += 256;
    unsigned long long tiles_all = 0;
    for (size_t f = 0; f < nf; f++)
        tiles_all += ((fields[f].nbEle + blockSize - 1) / blockSize + tb - 1) / tb;
    const size_t o_map = off; off += a256(4 * tiles_all);
    const size_t o_zero = off;
    std::vector<size_t> o_st(nf), o_tot(nf), o_sz(nf), o_md(nf), o_ss(nf);
    for (size_t f = 0; f < nf; f++) {
        const SZxG_Field& F = fields[f];
        if (!F.in || !F.out || F.nbEle == 0) return fail(SZXG_ERR_ARG);
        const size_t nb = (F.nbEle + blockSize - 1) / blockSize;
        if (F.outCapacity < blocked_bound(fastMode, dataType, F.nbEle, blockSize)) return fail(SZXG_ERR_CAPACITY);
        o_st[f] = off; off += a256(8 * blocked_status_words(nb));
    }
    for (size_t f = 0; f < nf; f++) { o_tot[f] = off; off += 64; }
    off = a256(off);
    const size_t zero_bytes = off - o_zero;
    for (size_t f = 0; f < nf; f++) {
        const size_t nb = (fields[f].nbEle + blockSize - 1) / blockSize;
        o_sz[f] = off; off += a256(2 * nb);
        o_md[f] = off; off += a256(4 * nb);
        o_ss[f] = off; off += a256(nb / 8 + 64);
    }
    SZxG_Batch* b = new SZxG_Batch();
    b->direction = direction; b->mode = fastMode; b->dtype = dataType; b->bs = blockSize; b->nf = nFields;
    if (cudaMalloc(&b->dev, off) != cudaSuccess) {
        cudaGetLastError();
        delete b;
        return fail(SZXG_ERR_CUDA);
    }
    uint8_t* base = (uint8_t*)b->dev;
    b->results = (StreamResult*)(base + o_res);
    b->counters = (unsigned long long*)(base + o_ctr);
    b->err = (int*)(base + o_ctr + 64);
    b->zero = base + o_zero;
    b->zero_bytes = zero_bytes;
    std::vector<BlkField> tab(nf);
    unsigned long long et = 0, at = 0;
    for (size_t f = 0; f < nf; f++) {
        const SZxG_Field& S = fields[f];
        const size_t nb = (S.nbEle + blockSize - 1) / blockSize, sb = (nb + 7) / 8;
        const size_t qfix = hdr + sb + 4 * nb;
        BlkField& F = tab[f];
        memset(&F, 0, sizeof F);
        F.x = S.in; F.n = S.nbEle; F.nb = nb;
        F.enc_tiles = (nb + tb - 1) / tb; F.enc_tile0 = et; et += F.enc_tiles;
        F.asm_tiles = (nb + kAsmBlocksPerTile - 1) / kAsmBlocksPerTile; F.asm_tile0 = at; at += F.asm_tiles;
        F.eb = S.absErrBound;
        F.params = nullptr;
        F.out = (uint8_t*)S.out;
        F.payload = F.out + qfix;
        F.payload_cap = S.outCapacity - qfix;
        F.st_enc = (unsigned long long*)(base + o_st[f]);
        F.st_asm = F.st_enc + enc_status_words(nb);
        F.size_blk = (uint16_t*)(base + o_sz[f]);
        F.med_blk = (uint32_t*)(base + o_md[f]);
        F.s_scr = base + o_ss[f];
        F.tot = (Totals*)(base + o_tot[f]);
        F.res = b->results + f;
    }
    b->enc_total = et;
    b->asm_total = at;
    b->one = tab[0];
    b->tab = tab;
    b->nrun = nFields;
    b->d_fields = (BlkField*)(base + o_tab);
    b->d_tile_field = (uint32_t*)(base + o_map);
    b->h_tile_field.resize(et);
    for (size_t f = 0; f < nf; f++)
        for (unsigned long long t = 0; t < tab[f].enc_tiles; t++) b->h_tile_field[tab[f].enc_tile0 + t] = (uint32_t)f;
    if (cudaMemcpy(b->d_tile_field, b->h_tile_field.data(), 4 * et, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(b->d_fields, tab.data(), sizeof(BlkField) * nf, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(b->dev);
        delete b;
        return fail(SZXG_ERR_CUDA);
    }
    set_last_error(SZXG_OK);
    return b;
}

int SZxG_batch_run(SZxG_Batch* b, SZxG_StreamInfo* d_info, void* stream) {
    if (!b) { set_last_error(SZXG_ERR_ARG); return SZXG_ERR_ARG; }
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(b->zero, 0, b->zero_bytes, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->counters, 0, 128, s);
    if (e == cudaSuccess && b->direction == 1)
        e = launch_blocked_decode_fields(b->mode, b->dtype, b->bs, b->nf, b->d_dec, b->d_tile_field, b->idx_total,
                                         b->dec_total,
                                         b->counters, b->results, b->err, s);
    else if (e == cudaSuccess)
        e = launch_blocked_encode_fields(b->mode, b->dtype, b->bs, b->nrun, b->one, b->nrun > 1 ? b->d_fields : nullptr,
                                         b->d_tile_field, b->enc_total, b->asm_total, b->counters, b->err, s);
    if (e == cudaSuccess && d_info)
        e = cudaMemcpyAsync(d_info, b->results, sizeof(StreamResult) * b->nf, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_last_error(SZXG_ERR_CUDA);
        return SZXG_ERR_CUDA;
    }
    set_last_error(SZXG_OK);
    return SZXG_OK;
}

int SZxG_batch_status(SZxG_Batch* b, void* stream) {
    if (!b) return SZXG_ERR_ARG;
    int h = 0;
    cudaStream_t s = (cudaStream_t)stream;
    if (cudaMemcpyAsync(&h, b->err, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        cudaGetLastError();
        return SZXG_ERR_CUDA;
    }
    return h;
}

void SZxG_batch_destroy(SZxG_Batch* b) {
    if (!b) return;
    lfx_free(b->lfx);
    if (b->dev) cudaFree(b->dev);
    delete b;
}

}  // extern "C"
