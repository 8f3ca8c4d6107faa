// Host-visible launchers and device-resident structures of the SZx codec.
// Shared by the kernels (*.cu) and the C-ABI layer (api.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace szxg {

// Parameters derived on the device from the data (value range pass) so that a
// relative bound never needs a host round trip.
struct CodecParams {
    float eb;          // absolute bound the codec uses (ABS passthrough or range * ratio)
    float radius;      // global radius (non-blocked layout), szx/src/szx_float.cc:494
    float median;      // global median (non-blocked layout), szx/src/szx_float.cc:495
    float range_f;     // value range as float (float data)
    double range_d;    // value range as double (double data)
    int has_range;
    int pad;
};

// Totals written by the last tile of an encode and read by the assembler.
struct Totals {
    unsigned long long payload_bytes;  // bytes of non-constant payloads / mid bytes
    unsigned long long nnc;            // non-constant blocks
};

// Where the finished stream sits inside the caller's output buffer.
struct StreamResult {
    unsigned long long offset;   // stream start relative to the output buffer
    unsigned long long size;     // stream length in bytes
    unsigned long long nb_const; // constant blocks (blocked layouts)
    float eb;                    // bound used
    int status;                  // 0 ok, otherwise an SZxG error code
};

// Header of a blocked stream parsed on the device (decode).
struct BlockedHdr {
    unsigned long long bs, nb, nc, nnc, sb;
    unsigned long long o_off, s_off, m_off, q_off;  // byte offsets in the stream
    unsigned long long n;
    int ok;
    int pad;
};

// Header of a non-blocked stream parsed on the device (decode).
struct NonBlockedHdr {
    unsigned long long n, L, mid_off, mid_len;
    float median;
    int reqLength;
    int ok;
};

enum Layout : int { kNonBlocked = 1, kBlocked = 2, kRandomAccess = 3, kRandomAccessNative = 4 };

// Sets what SZxG_get_last_error() reports on this host thread (api.cu).
void set_last_error(int e);

// One field of a blocked-layout encode launch (a single-field call is a
// table of one): where its values, stream and scratch live.
struct BlkField {
    const void* x;                               // values (device)
    unsigned long long n, nb;                    // values, blocks
    unsigned long long enc_tiles, enc_tile0;     // encode tiles, first launch-wide encode tile
    unsigned long long asm_tiles, asm_tile0;     // assemble tiles, first launch-wide assemble tile
    float eb;                                    // absolute bound (params->eb when params is set)
    int pad;
    const CodecParams* params;
    uint8_t* out;                                // stream buffer; the stream lands at out + res->offset
    uint8_t* payload;                            // fixed payload position (out + header, index, medians)
    unsigned long long payload_cap;
    unsigned long long* st_enc;                  // encode look-back status [enc_tiles + 4], zeroed
    unsigned long long* st_asm;                  // assemble look-back status [asm_tiles + 4], zeroed
    uint16_t* size_blk;                          // [nb] payload bytes by block
    uint32_t* med_blk;                           // [nb] stored medians by block
    uint8_t* s_scr;                              // state bits [nb / 8 + 64]
    Totals* tot;                                 // zeroed
    StreamResult* res;
};

// One stream of a batched blocked decode (fastMode 3/4).  Tile counts are
// known from n alone: the payload-offset scan is given ceil(nb / 2048) tiles
// (nnc <= nb) and skips those past the stream's real nnc.
struct DecField {
    const uint8_t* s;                            // stream (device)
    unsigned long long len, n, nb;               // stream bytes, values, blocks
    void* out;                                   // values (device)
    BlockedHdr* hdr;                             // parsed header
    unsigned long long* P;                       // [nb + 1] payload offsets by non-constant rank
    uint32_t* RW;                                // [nb / 32 + 2] rank at each 32-block state word
    unsigned long long* stA[3];                  // offset-scan look-back: word, agg2, inc2 [idxA_tiles], zeroed
    unsigned long long* stB[3];                  // rank-scan look-back [idxB_tiles], zeroed
    unsigned long long idx_tile0, idxA_tiles, idxB_tiles;   // launch-wide first index tile, tiles per scan
    unsigned long long dec_tile0, dec_tiles;     // launch-wide first decode tile, decode tiles
    int* err;                                    // this stream's error word, zeroed
    int pad;
    StreamResult* res;                           // where its outcome goes (NULL: res[f] of the launch)
};

// ------------------------------------------------------------------ workspace

// Device scratch needed by one compress or decompress call; carved by
// ws_carve() out of one caller-provided allocation.
struct Workspace {
    CodecParams* params;
    Totals* totals;
    StreamResult* result;
    BlockedHdr* bhdr;
    NonBlockedHdr* nhdr;
    int* err;
    unsigned long long* counters;   // 4 tile counters
    uint32_t* st32;                 // 32-bit tile status words ([status_tiles + 16])
    unsigned long long* st_word;    // tile status words (family A)
    unsigned long long* st_agg2;
    unsigned long long* st_inc2;
    unsigned long long* st2_word;   // tile status (family B)
    unsigned long long* st2_agg2;
    unsigned long long* st2_inc2;
    void* partials;                 // range-pass partials
    uint16_t* o_scr;                // payload sizes by non-constant rank
    uint32_t* m_scr;                // median bits by constant rank
    uint8_t* s_scr;                 // state bits
    unsigned long long* p_off;      // decode: payload offsets by non-constant rank
    uint32_t* rank_w;               // decode: non-constant rank at each 32-block word
    unsigned long long* tile_aux;   // non-blocked decode: per-tile summaries
    void* m2;                       // fastMode-2 decode: block-boundary search tables
    size_t m2_bytes;
    size_t status_tiles, status2_tiles, blocks, words, aux_tiles;
};

// Bytes cleared at the start of every encode, from Workspace::totals up to
// and including the tile counters (totals, result, headers, error word).
constexpr size_t kWsHeaderClear = 512;
// 64-bit look-back status words a blocked encode of nb blocks needs (the
// encoder's tiles hold >= 8 blocks, the assembler's 2048).  Both arrays start
// on 32-byte boundaries: the look-back reads them with 16-byte vector loads.
constexpr size_t kAsmBlocksPerTile = 2048;
constexpr size_t round4(size_t w) { return (w + 3) & ~size_t(3); }
// The encoder's region: its 64-bit words, then (at enc_tile_words) one 16-bit
// word per tile, aggregate + 1 (0: not published), with room for the
// 16-byte reads past the last tile.
constexpr size_t enc_tile_words(size_t nb) { return round4(nb / 8 + 9); }
constexpr size_t enc_agg16_words(size_t nb) { return round4((nb / 8 + 40) / 4); }
constexpr size_t enc_status_words(size_t nb) { return enc_tile_words(nb) + enc_agg16_words(nb); }
constexpr size_t blocked_status_words(size_t nb) { return enc_status_words(nb) + round4(nb / kAsmBlocksPerTile + 9); }

// Host: fault in the pages of a fresh malloc'd output buffer [p, p+n) on a
// few worker threads, asynchronously.  host_prefault_limit(m) lowers the
// job's extent to m bytes (the rest is skipped); host_prefault_wait(h) returns
// once [p, p+h) is resident; host_prefault_finish(m) lowers the extent, waits
// for the workers and ends the job.  One job at a time per process; every
// start must be paired with a finish, and the buffer must outlive it.
void host_prefault_start(void* p, size_t n);
void host_prefault_limit(size_t m);
void host_prefault_wait(size_t h);
void host_prefault_finish(size_t m);

// Bytes a library-allocated host output is copied in: each piece leaves as
// soon as its pages are resident.
constexpr size_t kHostCopyPiece = size_t(32) << 20;

// ------------------------------------------------------------------ fixed-rate search (fxr.cu)

// Device scratch of the searches below for n values, blocks of bs, every
// rate-th block sampled.
size_t fxr_ws_bytes(int dtype, size_t n, int bs, int rate);
// Bound the reference's fixed-rate mode picks for the target ratio (buffered
// model, started from 1% of the sampled range).  Synchronous on stream s.
cudaError_t fxr_bound(int dtype, const void* d_x, size_t n, int bs, float ratio, float tolerance, void* d_ws,
                      size_t wsb, cudaStream_t s, float* eb_out);
// Search of SZx_estimateErrorBoundbasedonCR (unbuffered model) from initErrorBound.
cudaError_t fxr_bound_unbuffered(int dtype, const void* d_x, size_t n, int bs, float ratio, float tolerance,
                                 float initErrorBound, void* d_ws, size_t wsb, cudaStream_t s, float* eb_out);
// computeRadiusBuffer: sampled radius / median / block copies into host arrays
// (d_copy: device room for the copies); the sampled range in *range_out.
cudaError_t fxr_radius_buffer(int dtype, const void* d_x, size_t n, int rate, int bs, void* d_ws, size_t wsb,
                              void* d_copy, cudaStream_t s, float* h_rads, float* h_meds, void* h_copy,
                              float* range_out);
// estimateCRbasedonErrorBound_buffered over contiguous sampled blocks on the device.
cudaError_t fxr_estimate_buffered(int dtype, const void* d_copy, size_t n, int rate, int bs, const float* h_rads,
                                  const float* h_meds, float eb, void* d_ws, size_t wsb, cudaStream_t s, float* cr,
                                  size_t* sumReq, size_t* sumLead);

// Scratch of the fastMode-2 boundary search for a stream of len bytes (mode2.cu).
size_t m2_ws_bytes(int dtype, size_t n, int bs, size_t len);
// Payload offsets of a fastMode-2 stream by non-constant rank into ws.p_off
// (header already parsed into ws.bhdr).
cudaError_t launch_m2_offsets(int dtype, const uint8_t* d_stream, size_t len, size_t n, int bs, void* m2ws,
                              size_t m2wsb, const Workspace& ws, cudaStream_t s);
__global__ void k_m2_parse(const uint8_t* s, unsigned long long len, unsigned long long n,
                           unsigned long long bs_expect, BlockedHdr* h, int* err);

size_t ws_bytes(int layout, int dtype, size_t n, int bs);
Workspace ws_carve(void* base, int layout, int dtype, size_t n, int bs);

// ------------------------------------------------------------------ launchers (return cudaError_t)

// Zeroes up to four workspace regions (4-byte aligned, sizes multiples of 4
// bytes) in one launch: the status words, totals and counters a codec pass
// expects clear, instead of one memset per region.
struct ClearList {
    void* p[4];
    size_t bytes[4];
    int n;
};
cudaError_t launch_ws_clear(const ClearList& c, cudaStream_t s);

// Global value range + derived bound; writes *params.  err_mode 0 = ABS, 1 = REL.
// cleared: the caller has zeroed counters[3] (the CTA ticket) already.
cudaError_t launch_range(int dtype, const void* x, size_t n, int err_mode, float abs_eb, float rel,
                         const Workspace& ws, cudaStream_t s, bool cleared = false);

// Blocked encode (layouts 2, 3, 4): stats + encode + placement + header assembly.
// d_out must hold blocked_bound() bytes; the stream lands at d_out + result.offset.
size_t blocked_bound(int layout, int dtype, size_t n, int bs);
// cleared: the caller has zeroed blocked_enc_clear()'s regions already;
// res_out: where the stream's result record goes (default ws.result).
cudaError_t launch_blocked_encode(int layout, int dtype, const void* x, size_t n, int bs, bool use_params,
                                  float abs_eb, uint8_t* d_out, size_t cap, const Workspace& ws, cudaStream_t s,
                                  bool cleared = false, StreamResult* res_out = nullptr);
// The regions a blocked encode of nb blocks expects zeroed: both look-backs'
// status words, then totals / result / error / counters (counters[3], the
// value-range pass's ticket, among them).
ClearList blocked_enc_clear(const Workspace& ws, size_t nb);
// Blocks per encode tile for this type and block size (tile counts of a
// field table), and the encode + assemble of nf fields in one launch each:
// `one` when nf == 1, else the device table d_fields (ascending tile starts)
// with d_tile_field[g] = the field of launch-wide encode tile g;
// counters[0..2] and err zeroed by the caller, like every field's status
// words and totals.
// Launch shape of the blocked kernels (chosen per field-size class for
// batches): the encoder's tile variant (0: 16 KiB of input, 1: 8 KiB -- float
// blocks of 65..128 values only, else the default) and CTAs per SM of the
// encoder and the decoder (0: as many as fit).
struct LaunchShape {
    int enc_tile_variant = 0;
    int enc_ctas_per_sm = 0;
    int dec_ctas_per_sm = 0;
};
int blocked_tile_blocks(int dtype, int bs, int tile_variant = 0);
cudaError_t launch_blocked_encode_fields(int layout, int dtype, int bs, int nf, const BlkField& one,
                                         const BlkField* d_fields, const uint32_t* d_tile_field,
                                         unsigned long long enc_total, unsigned long long asm_total,
                                         unsigned long long* counters, int* err, cudaStream_t s,
                                         const LaunchShape& shape = LaunchShape{});
// Blocked decode of nf streams (layouts 3, 4) in one launch per kernel: the
// headers are parsed into the fields' hdr, counters[0] and every field's
// look-back words and error word zeroed by the caller; res[f] receives field
// f's outcome and *err the first failing status.  idx_total / dec_total: the
// launch-wide index and decode tiles (sums over the table); d_tile_field[g]:
// the field of launch-wide decode tile g.
int blocked_dec_tile_blocks(int dtype, int bs);
constexpr unsigned long long kIdxPerTile = 2048;   // items per tile of the index scans
cudaError_t launch_blocked_decode_fields(int layout, int dtype, int bs, int nf, const DecField* d_fields,
                                         const uint32_t* d_tile_field, unsigned long long idx_total,
                                         unsigned long long dec_total,
                                         unsigned long long* counters, StreamResult* res, int* err,
                                         cudaStream_t s, const LaunchShape& shape = LaunchShape{});
// Blocked decode (layouts 3, 4).
cudaError_t launch_blocked_decode(int layout, int dtype, const uint8_t* d_stream, size_t len, size_t n, int bs,
                                  void* d_out, const Workspace& ws, cudaStream_t s);

// Non-blocked (layout 1) encode / decode.
size_t nonblocked_bound(int dtype, size_t n);
// cleared: the caller has zeroed nonblocked_enc_clear()'s regions already;
// res_out: where the stream's result record goes (default ws.result).
cudaError_t launch_nonblocked_encode(int dtype, const void* x, size_t n, uint8_t* d_out, size_t cap,
                                     const Workspace& ws, cudaStream_t s, bool cleared = false,
                                     StreamResult* res_out = nullptr);
// The regions a non-blocked encode of n values expects zeroed: its tile
// status words, then totals / result / error / counters.
ClearList nonblocked_enc_clear(const Workspace& ws, size_t n);
cudaError_t launch_nonblocked_decode(int dtype, const uint8_t* d_stream, size_t len, size_t n, void* d_out,
                                     const Workspace& ws, cudaStream_t s);

int sm_count();

// Records CUDA events around one kernel launch when tracing is enabled
// (SZxG_trace_enable); a no-op otherwise.
class TraceScope {
  public:
    TraceScope(const char* name, cudaStream_t s);
    ~TraceScope();
  private:
    const char* name_;
    cudaStream_t s_;
    void* a_;
};

}  // namespace szxg
