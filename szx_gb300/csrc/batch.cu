// Batches: many fields of one type and block size coded by persistent
// launches over a device work queue of (field, block-range) tiles.
// Compress (direction 0): fastMode 2, 3, 4.  Decompress (direction 1):
// fastMode 3 and 4, whose size index makes every stream's payload offsets a
// scan; a fastMode-2 stream needs the single-stream boundary search.
//
// The blocked kernels take a table of fields (a single-field call is a table
// of one): a launch-wide tile index maps to (field, local tile) through a
// tile map, and every field keeps its own look-back status words, totals,
// scratch and stream.  Tiles are handed out in field order from one atomic
// counter, so a field's tiles are always acquired before any later field's,
// which is all the per-field look-back needs to make progress.
//
// Fields are grouped by size class (a table of value-count bounds, each with
// its launch shape: encoder tile size and CTAs per SM of the encoder and the
// decoder), and each class is one persistent launch per kernel with its own
// shape.  The table comes from the tuning file written by the project's
// autotuner (szx_gb300/tune.py: tuning/batch_shapes.txt next to the
// library, or the file SZXG_TUNING_FILE names), or from
// SZxG_set_launch_shapes; with neither, one class with the default shape.
// The shape never changes a stream: only how the work is cut and spread.
//
// This file plans a batch (layout of the per-field scratch in one
// allocation, the field table and tile map on the device) and runs it as a
// handful of memsets and launches that a CUDA graph can capture.
#include <dlfcn.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <mutex>
#include <string>
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

// ------------------------------------------------------------------ launch shapes by size class

struct ShapeEntry {
    unsigned long long max_values;
    LaunchShape shape;
};
std::mutex g_shape_mu;
std::vector<ShapeEntry> g_shapes;   // ascending max_values; the last one takes every larger field
bool g_shapes_loaded = false;

std::string tuning_path() {
    if (const char* e = getenv("SZXG_TUNING_FILE")) return e;
    Dl_info info;
    if (dladdr((void*)&tuning_path, &info) && info.dli_fname) {
        std::string so = info.dli_fname;
        const size_t k = so.find_last_of('/');
        return (k == std::string::npos ? std::string(".") : so.substr(0, k)) + "/tuning/batch_shapes.txt";
    }
    return "";
}

// "max_values enc_tile_variant enc_ctas_per_sm dec_ctas_per_sm" per line, '#' comments
std::vector<ShapeEntry> read_tuning(const std::string& path) {
    std::vector<ShapeEntry> v;
    FILE* f = path.empty() ? nullptr : fopen(path.c_str(), "r");
    if (!f) return v;
    char line[256];
    while (fgets(line, sizeof line, f)) {
        if (line[0] == '#') continue;
        unsigned long long m = 0;
        int tv = 0, ec = 0, dc = 0;
        if (sscanf(line, "%llu %d %d %d", &m, &tv, &ec, &dc) != 4) continue;
        if ((int)v.size() == kMaxBatchParts || (!v.empty() && m <= v.back().max_values)) break;
        LaunchShape s;
        s.enc_tile_variant = tv == 1 ? 1 : 0;
        s.enc_ctas_per_sm = ec < 0 ? 0 : ec;
        s.dec_ctas_per_sm = dc < 0 ? 0 : dc;
        v.push_back({m, s});
    }
    fclose(f);
    return v;
}

void ensure_shapes_locked() {
    if (g_shapes_loaded) return;
    g_shapes = read_tuning(tuning_path());
    if (g_shapes.empty()) g_shapes.push_back({~0ull, LaunchShape{}});
    g_shapes_loaded = true;
}

}  // namespace

int batch_class_of(unsigned long long n, int* nclasses) {
    std::lock_guard<std::mutex> lk(g_shape_mu);
    ensure_shapes_locked();
    if (nclasses) *nclasses = (int)g_shapes.size();
    for (size_t k = 0; k < g_shapes.size(); k++)
        if (n <= g_shapes[k].max_values) return (int)k;
    return (int)g_shapes.size() - 1;
}

LaunchShape batch_class_shape(int k) {
    std::lock_guard<std::mutex> lk(g_shape_mu);
    ensure_shapes_locked();
    return g_shapes[(size_t)k < g_shapes.size() ? (size_t)k : g_shapes.size() - 1].shape;
}

// The fields a compress run codes, grouped by class in a stable order, their
// device table and tile map (per class: tiles numbered from 0, field
// indices relative to the class's first table entry).
cudaError_t batch_select(SZxG_Batch* b, int nActive, const int* h_idx, const float* h_eb, cudaStream_t s) {
    if (b->direction != 0 || nActive < 1 || nActive > b->nf) return cudaErrorInvalidValue;
    if (!h_idx && nActive != b->nf) return cudaErrorInvalidValue;
    const int ncls = (int)b->class_shape.size();
    std::vector<std::vector<int>> by(ncls);
    for (int k = 0; k < nActive; k++) {
        const int f = h_idx ? h_idx[k] : k;
        if (f < 0 || f >= b->nf) return cudaErrorInvalidValue;
        if (h_eb) b->tab[f].eb = h_eb[k];
        by[b->cls[f]].push_back(f);
    }
    b->run.clear();
    b->parts.clear();
    b->h_tile_field.clear();
    for (int c = 0; c < ncls; c++) {
        if (by[c].empty()) continue;
        BatchPart P;
        P.shape = b->class_shape[c];
        P.i0 = (int)b->run.size();
        P.map0 = b->h_tile_field.size();
        unsigned long long et = 0, at = 0;
        for (int f : by[c]) {
            BlkField F = b->tab[f];   // enc_tiles already for this class's tile size
            F.enc_tile0 = et; et += F.enc_tiles;
            F.asm_tile0 = at; at += F.asm_tiles;
            for (unsigned long long t = 0; t < F.enc_tiles; t++)
                b->h_tile_field.push_back((uint32_t)(b->run.size() - P.i0));
            b->run.push_back(F);
        }
        P.i1 = (int)b->run.size();
        P.enc_total = et;
        P.asm_total = at;
        b->parts.push_back(P);
    }
    // pageable sources: each copy is staged before the call returns, ordered after earlier runs on s
    cudaError_t e = cudaMemcpyAsync(b->d_fields, b->run.data(), sizeof(BlkField) * b->run.size(),
                                    cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->d_tile_field, b->h_tile_field.data(), 4 * b->h_tile_field.size(),
                            cudaMemcpyHostToDevice, s);
    return e;
}

extern "C" {

int SZxG_set_launch_shapes(const SZxG_LaunchShape* table, int n) {
    if (n < 0 || n > kMaxBatchParts || (n > 0 && !table)) {
        set_last_error(SZXG_ERR_ARG);
        return SZXG_ERR_ARG;
    }
    std::vector<ShapeEntry> v;
    for (int k = 0; k < n; k++) {
        const SZxG_LaunchShape& t = table[k];
        if ((k > 0 && t.maxValues <= table[k - 1].maxValues) || (t.encTileVariant != 0 && t.encTileVariant != 1) ||
            t.encCtasPerSm < 0 || t.decCtasPerSm < 0) {
            set_last_error(SZXG_ERR_ARG);
            return SZXG_ERR_ARG;
        }
        LaunchShape s;
        s.enc_tile_variant = t.encTileVariant;
        s.enc_ctas_per_sm = t.encCtasPerSm;
        s.dec_ctas_per_sm = t.decCtasPerSm;
        v.push_back({t.maxValues, s});
    }
    std::lock_guard<std::mutex> lk(g_shape_mu);
    if (n == 0) {
        g_shapes_loaded = false;
        ensure_shapes_locked();
    } else {
        g_shapes = v;
        g_shapes_loaded = true;
    }
    set_last_error(SZXG_OK);
    return SZXG_OK;
}

int SZxG_get_launch_shapes(SZxG_LaunchShape* table, int cap) {
    std::lock_guard<std::mutex> lk(g_shape_mu);
    ensure_shapes_locked();
    const int n = (int)g_shapes.size();
    for (int k = 0; k < n && k < cap && table; k++) {
        table[k].maxValues = g_shapes[k].max_values;
        table[k].encTileVariant = g_shapes[k].shape.enc_tile_variant;
        table[k].encCtasPerSm = g_shapes[k].shape.enc_ctas_per_sm;
        table[k].decCtasPerSm = g_shapes[k].shape.dec_ctas_per_sm;
        table[k].reserved = 0;
    }
    return n;
}

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
    // fields by class, in a stable order: the device table's order
    int ncls = 1;
    std::vector<std::vector<size_t>> by;
    for (size_t f = 0; f < nf; f++) {
        const int c = batch_class_of(fields[f].nbEle, &ncls);
        if (by.size() < (size_t)ncls) by.resize((size_t)ncls);
        by[(size_t)c].push_back(f);
    }
    std::vector<size_t> order;
    for (auto& v : by) order.insert(order.end(), v.begin(), v.end());
    // layout: table | results | counters+err | headers | tile map | zeroed (errors, look-back words) | offsets, ranks
    size_t off = 0;
    const size_t o_tab = off; off += a256(sizeof(DecField) * nf);
    const size_t o_res = off; off += a256(sizeof(StreamResult) * nf);
    const size_t o_ctr = off; off += 512;
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
    b->err = (int*)(base + o_ctr + 384);
    b->zero = base + o_zero;
    b->zero_bytes = zero_bytes;
    std::vector<DecField> tab(nf);
    for (size_t c = 0, k = 0; c < by.size(); c++) {
        if (by[c].empty()) continue;
        BatchPart P;
        P.shape = batch_class_shape((int)c);
        P.i0 = (int)k;
        P.map0 = b->h_tile_field.size();
        unsigned long long it = 0, dt = 0;
        for (size_t f : by[c]) {
            const SZxG_Field& S = fields[f];
            DecField& D = tab[k];
            memset(&D, 0, sizeof D);
            D.s = (const uint8_t*)S.in; D.len = S.inBytes; D.n = S.nbEle;
            D.nb = (S.nbEle + blockSize - 1) / blockSize;
            D.out = S.out;
            D.hdr = (BlockedHdr*)(base + o_hdr) + f;
            D.P = (unsigned long long*)(base + o_p[f]);
            D.RW = (uint32_t*)(base + o_rw[f]);
            unsigned long long* st = (unsigned long long*)(base + o_st[f]);
            for (int q = 0; q < 3; q++) D.stA[q] = st + q * ta[f];
            st += 3 * ta[f];
            for (int q = 0; q < 3; q++) D.stB[q] = st + q * tbw[f];
            D.idxA_tiles = ta[f]; D.idxB_tiles = tbw[f];
            D.idx_tile0 = it; it += ta[f] + tbw[f];
            D.dec_tiles = (D.nb + tb - 1) / tb;
            D.dec_tile0 = dt; dt += D.dec_tiles;
            D.err = (int*)(base + o_err) + f;
            D.res = b->results + f;
            for (unsigned long long t = 0; t < D.dec_tiles; t++) b->h_tile_field.push_back((uint32_t)(k - P.i0));
            k++;
        }
        P.i1 = (int)k;
        P.idx_total = it;
        P.dec_total = dt;
        b->parts.push_back(P);
    }
    b->d_dec = (DecField*)(base + o_tab);
    b->d_tile_field = (uint32_t*)(base + o_map);
    if (cudaMemcpy(b->d_tile_field, b->h_tile_field.data(), 4 * b->h_tile_field.size(), cudaMemcpyHostToDevice) !=
            cudaSuccess ||
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
    const size_t hdr = fastMode == kBlocked ? 13 : 20;
    // every field's class; the class's tile size sets the field's tile count
    std::vector<int> cls(nf);
    int ncls = 1;
    for (size_t f = 0; f < nf; f++) cls[f] = batch_class_of(fields[f].nbEle, &ncls);
    std::vector<LaunchShape> cshape((size_t)ncls);
    std::vector<size_t> ctb((size_t)ncls);
    for (int c = 0; c < ncls; c++) {
        cshape[(size_t)c] = batch_class_shape(c);
        ctb[(size_t)c] = (size_t)blocked_tile_blocks(dataType, blockSize, cshape[(size_t)c].enc_tile_variant);
    }
    // layout: table | results | counters+err | tile map | zeroed status words and totals | scratch
    size_t off = 0;
    const size_t o_tab = off; off += a256(sizeof(BlkField) * nf);
    const size_t o_res = off; off += a256(sizeof(StreamResult) * nf);
    const size_t o_ctr = off; off += 512;
    unsigned long long tiles_all = 0;
    for (size_t f = 0; f < nf; f++)
        tiles_all += ((fields[f].nbEle + blockSize - 1) / blockSize + ctb[(size_t)cls[f]] - 1) / ctb[(size_t)cls[f]];
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
    b->err = (int*)(base + o_ctr + 384);
    b->zero = base + o_zero;
    b->zero_bytes = zero_bytes;
    b->tab.resize(nf);
    for (size_t f = 0; f < nf; f++) {
        const SZxG_Field& S = fields[f];
        const size_t nb = (S.nbEle + blockSize - 1) / blockSize, sb = (nb + 7) / 8;
        const size_t qfix = hdr + sb + 4 * nb;
        const size_t tb = ctb[(size_t)cls[f]];
        BlkField& F = b->tab[f];
        memset(&F, 0, sizeof F);
        F.x = S.in; F.n = S.nbEle; F.nb = nb;
        F.enc_tiles = (nb + tb - 1) / tb;
        F.asm_tiles = (nb + kAsmBlocksPerTile - 1) / kAsmBlocksPerTile;
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
    b->cls = cls;
    b->class_shape = cshape;
    b->d_fields = (BlkField*)(base + o_tab);
    b->d_tile_field = (uint32_t*)(base + o_map);
    if (batch_select(b, nFields, nullptr, nullptr, 0) != cudaSuccess || cudaStreamSynchronize(0) != cudaSuccess) {
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
    if (e == cudaSuccess) e = cudaMemsetAsync(b->counters, 0, 32 * kMaxBatchParts, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->err, 0, sizeof(int), s);
    for (size_t k = 0; k < b->parts.size() && e == cudaSuccess; k++) {
        const BatchPart& P = b->parts[k];
        const int n = P.i1 - P.i0;
        unsigned long long* ctr = b->counters + 4 * k;
        if (b->direction == 1)
            e = launch_blocked_decode_fields(b->mode, b->dtype, b->bs, n, b->d_dec + P.i0, b->d_tile_field + P.map0,
                                             P.idx_total, P.dec_total, ctr, b->results, b->err, s, P.shape);
        else
            e = launch_blocked_encode_fields(b->mode, b->dtype, b->bs, n, b->run[(size_t)P.i0],
                                             n > 1 ? b->d_fields + P.i0 : nullptr, b->d_tile_field + P.map0,
                                             P.enc_total, P.asm_total, ctr, b->err, s, P.shape);
    }
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
