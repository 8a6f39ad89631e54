// Host-side launchers of the CUDA kernels (declarations).
#pragma once
#include <functional>

#include "common.cuh"

namespace prodm {

// mgard.cu
template <class T>
int launch_decompose_level_packed(const T* in, uint64_t s0, uint64_t s1, const Box& F, const Box& C, T* coef, T* coarse,
                                  T* fnat, void* maxkey_level, void* maxkey_coarse, cudaStream_t st);
template <class T>
int launch_decompose_level_inplace(const T* in, const Box& F, const Box& C, T* out, uint64_t o0, uint64_t o1, T* fnat,
                                   cudaStream_t st);
template <class T>
int launch_recompose_level_packed(const T* coarse, const T* coef, const Box& F, const Box& C, T* out, uint64_t s0,
                                  uint64_t s1, cudaStream_t st, bool pdl = false);
template <class T>
int launch_recompose_level_inplace(const T* rin, const Box& F, const Box& C, T* out, uint64_t s0, uint64_t s1,
                                   cudaStream_t st);
template <class T>
int launch_copy_box(const T* src, uint64_t a0, uint64_t a1, const Box& B, T* dst, uint64_t b0, uint64_t b1,
                    cudaStream_t st);
template <class T>
int launch_coef_to_natural(const T* coef, const Box& F, const Box& C, T* fnat, cudaStream_t st);
template <class T>
int launch_reordered_to_natural(const T* rin, const Box& F, const Box& C, T* fnat, cudaStream_t st);
template <class W>
void mass_factors(uint32_t n, W* tab);
// coef != nullptr: read the level's packed coefficients (coarse box *C) instead of fnat
template <class T>
int launch_l2_correction(const T* fnat, const Box& F, T* t1, T* t2, T* z, const T* const tabs[3], cudaStream_t st,
                         const T* coef = nullptr, const Box* C = nullptr);
template <class T>
int launch_add_box(T* dst, uint64_t b0, uint64_t b1, const T* z, const Box& B, T sign, cudaStream_t st);
template <class T>
int launch_interleave(T* data, uint64_t s0, uint64_t s1, const Box& F, const Box& C, T* buf, bool gather,
                      cudaStream_t st);

// adjoint.cu: transpose of one hierarchical recomposition level (field
// gradient of box F -> gradient of the level's packed coefficients and of the
// coarse box C, natural order)
template <class T>
int launch_recompose_adjoint_level(const T* g, const Box& F, const Box& C, T* gcoef, T* gcoarse, cudaStream_t st);
// the same for the orthogonal basis (tabs: Thomas factors per dim; scratch
// boxes (n0, c1, c2), (n0, n1, c2), F, and one C box)
template <class T>
int launch_recompose_adjoint_level_orth(const T* g, const Box& F, const Box& C, T* gcoef, T* gcoarse,
                                        const T* const tabs[3], T* s_a, T* s_b, T* s_w, T* s_u, cudaStream_t st);

// bitplane.cu
template <class T>
int launch_nb_encode(const T* x, uint64_t n, const void* maxkey, int exp, int B, void* out, uint64_t stride,
                     double* partial, double* errs_out, cudaStream_t st);
template <class T>
int launch_nb_decode(const void* base, uint64_t stride, uint64_t n, const void* maxkey, int exp, int s, int num,
                     const uint8_t* dnum, T* out, cudaStream_t st);
uint64_t gr_nchunks(uint64_t nblocks);
template <class T>
int launch_gr_encode(const T* x, uint64_t n, const void* maxkey, int exp, int B, uint8_t* rbs, uint32_t* chunk_words,
                     uint32_t* chunk_off, uint32_t* sizes, void* out, uint64_t cap, double* partial, double* errs_out,
                     cudaStream_t st);
template <class T>
int launch_gr_decode(const void* const* planes, uint64_t n, const void* maxkey, int exp, int B, int s, int e,
                     const uint8_t* dnum, const uint8_t* rbs, const uint32_t* chunk_off, void* signs, T* out,
                     cudaStream_t st);
template <class T>
int launch_sq_collect(const T* x, uint64_t n, int B, T maxv, double* partial, double* out, cudaStream_t st);
template <class T>
int launch_max_collect(const T* bounds, int nl, int B, double* out, cudaStream_t st);
constexpr int kPartialSlots = kSMs * 4;   // per-CTA partial error tables of the fused collectors
// bytes of `parts` per-CTA partials: B + 1 doubles (fp64 tables, squared-error
// collector) or one record of the exact fp32 tables (errtab.cuh)
constexpr int kErrRecWords = 200;   // errtab::kSlotsPad
inline uint64_t partial_bytes(uint64_t parts, int B) {
    return parts * (uint64_t)(kErrRecWords > B + 1 ? kErrRecWords : B + 1) * 8;
}

// interpret.cu
template <class T>
int launch_interpret(int nfields, int kind, int est_kind, const int* d_ndims, const int* d_levels, double s, int B,
                     const uint32_t* d_sizes, uint64_t sz_stride, const double* d_errs, uint64_t err_stride,
                     const double* d_tols, double tol0, uint8_t* d_index, uint64_t idx_stride, uint32_t* d_rsz,
                     cudaStream_t st, bool pdl = false, bool early = false);

// one segment per (field, level) of the multi-level fp32 negabinary encode /
// decode launches; chunk_begin is the segment's first global chunk
struct ChunkSeg {
    const float* x;         // encode input
    float* y;               // decode output
    uint32_t* words;        // plane 0 of the level's streams
    uint64_t n, nblocks, stride;
    const uint32_t* key;
    const uint8_t* dnum;    // decode: retrieved plane count
    uint64_t chunk_begin;
};
// bitplane.cu: every level of one fp32 field decoded in one launch; segments
// chunked by kDecodeChunkBlocks blocks
constexpr int kDecodeChunkBlocks = 128;
int launch_nb_decode_levels(const ChunkSeg* segs, int nseg, uint64_t total_chunks, cudaStream_t st, bool pdl = false);
// bitplane.cu: every level of one fp32 field in one encode launch; with
// errs_out, per-level squared-error tables (partial: nseg * nb_encode_levels_grid(1)
// records of kErrRecWords words)
int nb_encode_levels_grid(int with_errors);
int launch_nb_encode_levels(const ChunkSeg* segs, int nseg, uint64_t total_chunks, int B, double* partial,
                            const uint32_t* keys, double* errs_out, cudaStream_t st);

// fused.cu
bool decode_recompose_nb32_ok(const Box& F);
int launch_decode_recompose_nb32(const void* base, uint64_t stride, int planes, uint64_t nblocks, const void* maxkey,
                                 const uint8_t* dnum, const float* coarse, const Box& F, const Box& C, float* out,
                                 uint64_t s0, uint64_t s1, int* status, cudaStream_t st, bool pdl = false);
void fused_tma_test_hook(int tx_extra, long long wait_cycles);
// one segment per field of the batched fused launch: the finest level of an
// fp32 negabinary field (odd row length) decoded and recomposed from its
// coarse box; unit_begin is the field's first global 8-row unit
struct FusedSeg {
    const uint32_t* base;   // plane 0 of the level's streams
    uint64_t stride;        // words per plane row
    const uint32_t* key;    // level |max| key
    const uint8_t* dnum;    // retrieved plane count
    const float* coarse;
    float* out;
    Box F, C;
    uint64_t s0, s1;
    uint64_t unit_begin;
    const void* map;        // TMA form: the planes' tensor map (a CUtensorMap in device memory)
    uint32_t bw;            // TMA form: the unit's block range plus alignment, in words
    uint32_t rpu;           // TMA form: rows per unit (a multiple of 8, at most kMaxUnitRows)
    uint32_t tall;          // TMA form: 1 = the map's box is the tile's row stride x 32 plane rows
                            // (one copy per unit), 0 = bw words x 1 plane (one copy per plane)
};
constexpr uint32_t kMaxUnitRows = 64;
// blocks of the plane tile of an 8-row unit of box F, and the launch's dynamic
// shared memory for units of at most that many blocks
uint32_t fused_unit_blocks(const Box& F);
size_t fused_multi_smem(uint32_t tld);
int launch_decode_recompose_nb32_multi(const FusedSeg* segs, int nseg, uint64_t total_units, uint32_t tld,
                                       unsigned ctas_per_sm, cudaStream_t st);
// TMA form: box width of a level's tensor map for units of nr rows (0: rows
// too long or even), the
// map of one level's planes (CUtensorMap, 128 bytes, into `map`), the launch
// over segments whose maps live in device memory (64-byte aligned)
// rows per unit of the TMA form: a multiple of 8, about `values` values
uint32_t fused_unit_rows(const Box& F, uint32_t values);
uint32_t fused_unit_blocks_rows(const Box& F, uint32_t nr);      // tile blocks of nr rows
uint32_t fused_tma_box(const Box& F, uint32_t nr);
int encode_plane_map(void* map, const void* base, uint64_t nblocks, int planes, uint64_t stride, uint32_t bw,
                     uint32_t box_planes = 1);
bool fused_tma_tall();                                            // PRODM_TMA_TALL (default 1)
// the warp-specialised batched kernel: units of fused_ws_unit_rows() rows,
// tall maps with boxes of kWsMultiStride words x 32 plane rows
constexpr uint32_t kWsMultiStride = 96;
uint32_t fused_ws_unit_rows();
int launch_decode_recompose_nb32_ws_multi(const FusedSeg* segs, int nseg, uint64_t total_units, uint32_t tld,
                                          int* status, cudaStream_t st);
uint32_t fused_tma_stride(uint32_t bw);                           // tile row stride of the TMA kernels for box bw
int launch_decode_recompose_nb32_tma_multi(const FusedSeg* segs, int nseg, uint64_t total_units, uint32_t tld,
                                           uint32_t max_bw, unsigned ctas_per_sm, int* status, cudaStream_t st);

// perbit.cu: per-bit format; rows of 32-element group words (magnitude
// planes 0..B-1, sign row B, unseen row B+1), each row `stride` words
uint64_t pb_groups(uint64_t n);
uint64_t pb_row_words(uint64_t n);
template <class T>
int launch_pb_encode(const T* x, uint64_t n, const void* maxkey, int exp, int B, uint32_t* rows, uint64_t stride,
                     uint32_t* counts, uint32_t* sizes, cudaStream_t st);
template <class T>
int launch_pb_decode(const uint32_t* rows, uint64_t stride, uint64_t n, const void* maxkey, int exp, int B, int s, int e,
                     const uint8_t* dnum, const uint32_t* srow, const uint32_t* unseen, T* out, cudaStream_t st);
size_t pb_pack_scratch_bytes(uint64_t n, int B);
int launch_pb_pack(const uint32_t* rows, uint64_t stride, uint64_t n, int B, const uint32_t* sizes, uint64_t total,
                   uint8_t* dst, void* scratch, cudaStream_t st);
int launch_pb_init_unseen(uint32_t* unseen, uint32_t* signs, uint64_t n, cudaStream_t st);
size_t pb_parse_scratch_bytes(int np);
int launch_pb_parse(const uint64_t* const* planes, const uint64_t* nwords, int a, int np, uint64_t n, uint32_t* rows,
                    uint64_t stride, uint32_t* unseen, uint32_t* signs, void* scratch, int* status, cudaStream_t st);

// lossless.cu: ZCB codec, one descriptor per stream; chunk0 = the stream's
// first chunk in the flattened chunk index (sorted), clen = compressed length
struct ZStream {
    const uint8_t* src;
    uint8_t* dst;
    uint64_t len;
    uint64_t clen;
    uint64_t chunk0;
};
uint64_t zcb_bound(uint64_t len);
int launch_zcb_count(const ZStream* d_ss, int ns, uint64_t total_chunks, uint32_t* csize, uint32_t* coff,
                     uint32_t* out_sizes, cudaStream_t st);
int launch_zcb_write(const ZStream* d_ss, int ns, uint64_t total_chunks, const uint32_t* csize, const uint32_t* coff,
                     cudaStream_t st);
int launch_zcb_read(const ZStream* d_ss, int ns, uint64_t total_chunks, int* status, cudaStream_t st);
int adaptive_stopping(const uint32_t* raw, const uint32_t* comp, int B, int latter, uint8_t* compressed);
// one level's streams (device, concatenated, raw sizes h_sizes) -> stored
// streams (compressed where flags say, else raw) concatenated into d_out
int ll_compress_level(const uint8_t* d_raw, const uint32_t* h_sizes, int B, int latter, uint8_t* d_out,
                      uint64_t cap, uint32_t* h_out_sizes, int* h_stop, const uint8_t* h_flags, cudaStream_t st);
// compressed sizes of every stream (the ZCB size; no output written)
int ll_stream_sizes(const uint8_t* d_raw, const uint32_t* h_sizes, int B, uint32_t* h_comp, cudaStream_t st);
// stored streams of `num` planes (sizes h_sizes, flags) -> raw streams
// concatenated into d_out (capacity cap); h_raw_sizes: their raw sizes
int ll_decompress_planes(const uint8_t* d_in, const uint32_t* h_sizes, const uint8_t* h_flags, int num, uint8_t* d_out,
                         uint64_t cap, uint32_t* h_raw_sizes, cudaStream_t st);

// fileio.cu: byte ranges of a file into the handle's loader (sink(src,
// offset within the range, bytes, src_is_host)); *mode: 1 cuFile, 0 pinned
struct FileStaging;
void file_staging_free(FileStaging* s);
int file_staging_mode(const FileStaging* s);
int read_file_range(FileStaging*& fs, const char* path, uint64_t file_off, uint64_t bytes,
                    const std::function<int(const void*, uint64_t, uint64_t, int)>& sink, cudaStream_t st,
                    int* mode);

// pack.cu
int launch_gr_pack(const void* const* planes, const uint32_t* sizes, int B, uint64_t nblocks, const uint8_t* rbs,
                   int word_bytes, uint8_t* dst, cudaStream_t st);
int launch_unpack_planes(const uint8_t* src, const uint64_t* src_off, const uint64_t* nwords, int nplanes,
                         int word_bytes, void* const* dst, uint64_t max_words, cudaStream_t st);
int launch_chunk_words_from_rb(const uint8_t* rbs, uint64_t nblocks, int B, uint32_t* chunk_words, cudaStream_t st);
int launch_gr_scan_only(const uint32_t* chunk_words, uint64_t nchunks, int B, uint64_t nblocks, int word_bytes,
                        uint32_t* chunk_off, uint32_t* sizes, cudaStream_t st);
template <class T>
int launch_maxabs(const T* x, uint64_t n, void* maxkey, cudaStream_t st);
template <class T>
int launch_bounds_from_keys(const void* keys, int nl, int negabinary, T* bounds, cudaStream_t st);
int launch_fill_u32(uint32_t* dst, uint64_t n, uint32_t v, cudaStream_t st);

}  // namespace prodm
