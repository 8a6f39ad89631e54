/*
 * prodm_gb300 -- C ABI of the GB300 (sm_103a) implementation of ProDM's MDR
 * refactor / retrieve path (lxAltria/ProDM, the headers under include/MDR).
 *
 * Plain C types only: device buffers are raw pointers, CUDA streams are passed
 * as void* (cudaStream_t), sizes are 64-bit. Every function returns a status
 * code; prodm_last_error_string() describes the last failure on the calling
 * thread. Nothing here exits the process (the reference calls exit() on
 * unsupported input, e.g. DirectInterleaver.hpp:33-36).
 *
 * Enumerations
 *   dtype      PRODM_F32 (float data, u32 stream words, 32-value blocks)
 *              PRODM_F64 (double data, u64 stream words, 64-value blocks)
 *   encoder    PRODM_ENC_NEGABINARY  NegaBinaryBPEncoder<T, S>
 *              PRODM_ENC_GROUPED     GroupedBPEncoder<T, S>
 *              PRODM_ENC_PERBIT      PerBitBPEncoder<T, S> (the stream word type
 *                                    does not enter its format; fp64 up to 63 planes)
 *   basis      PRODM_BASIS_HIERARCHICAL  MGARDHierarchicalDecomposer (MGARD.hpp:42-70)
 *              PRODM_BASIS_ORTHOGONAL    MGARDOrthoganalDecomposer   (MGARD.hpp:11-39)
 *   interpreter PRODM_INTERP_GREEDY / _SIGN_EXCLUDE / _NEGABINARY
 *              (GreedyBasedSizeInterpreter.hpp:28-64 / :78-140 / :166-248)
 *   estimator  PRODM_EST_MAX_HB / _MAX_OB / _L2_HB / _SNORM
 *              (MaxErrorEstimator.hpp:53-68 / :13-49; SquaredErrorEstimator.hpp:12-38 / :42-68)
 *   collector  PRODM_COLLECT_MAX / _SQUARED (MaxErrorCollector.hpp / SquaredErrorCollector.hpp)
 */
#ifndef PRODM_GB300_H
#define PRODM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define PRODM_OK 0
#define PRODM_EINVAL 1        /* invalid argument (sizes, levels, enums)      */
#define PRODM_ENOMEM 2        /* device allocation failed                     */
#define PRODM_ECUDA 3         /* CUDA runtime error                           */
#define PRODM_ETIMEOUT 4      /* a bounded device wait gave up                */
#define PRODM_ECORRUPT 5      /* malformed stream / metadata                  */
#define PRODM_EUNSUPPORTED 6  /* valid but not supported combination          */

#define PRODM_F32 0
#define PRODM_F64 1
#define PRODM_ENC_NEGABINARY 0
#define PRODM_ENC_GROUPED 1
#define PRODM_ENC_PERBIT 2
#define PRODM_BASIS_HIERARCHICAL 0
#define PRODM_BASIS_ORTHOGONAL 1
#define PRODM_INTERP_GREEDY 0
#define PRODM_INTERP_SIGN_EXCLUDE 1
#define PRODM_INTERP_NEGABINARY 2
#define PRODM_EST_MAX_HB 0
#define PRODM_EST_MAX_OB 1
#define PRODM_EST_L2_HB 2
#define PRODM_EST_SNORM 3
#define PRODM_COLLECT_MAX 0
#define PRODM_COLLECT_SQUARED 1

const char* prodm_last_error_string(void);
int prodm_version(void);

/* ---------------------------------------------------------------------------
 * Level geometry
 * ------------------------------------------------------------------------- */
/* ComposedRefactor.hpp:79 -- largest target level accepted for dims. */
int prodm_max_level(int ndims, const uint32_t* dims, int* out_level);
/* RefactorUtils.hpp:21-34 (compute_level_dims) and :41-59
 * (compute_level_elements): out_dims[(L+1)*ndims], out_elems[L+1]. */
int prodm_level_dims(int ndims, const uint32_t* dims, int target_level, uint32_t* out_dims, uint64_t* out_elems);

/* ---------------------------------------------------------------------------
 * Decomposer -- DecomposerInterface<T>::decompose / recompose
 * (DecomposerInterface.hpp:14-16; MGARD.hpp:14-35, :45-66).
 * In place on device data of shape dims (1-3 dims) with the reference's
 * per-level reordered layout. strides: NULL for row-major, else ndims element
 * strides with the last equal to 1. workspace: NULL to let the call allocate
 * (stream ordered), else at least prodm_decompose_workspace() bytes.
 * ------------------------------------------------------------------------- */
int prodm_decompose_workspace(int dtype, int ndims, const uint32_t* dims, uint32_t target_level, int basis,
                              size_t* bytes);
int prodm_decompose(int dtype, void* d_data, int ndims, const uint32_t* dims, uint32_t target_level,
                    const uint32_t* strides, int basis, void* d_workspace, size_t workspace_bytes, void* stream);
int prodm_recompose(int dtype, void* d_data, int ndims, const uint32_t* dims, uint32_t target_level,
                    const uint32_t* strides, int basis, void* d_workspace, size_t workspace_bytes, void* stream);

/* ---------------------------------------------------------------------------
 * Interleaver -- DirectInterleaver<T>::interleave / reposition
 * (InterleaverInterface.hpp:14-16; DirectInterleaver.hpp:12-37, :38-63).
 * d_buf holds prod(fine) - prod(coarse) values in the reference's order.
 * 1-D, 2-D and 3-D (the reference supports 1-D and 3-D).
 * ------------------------------------------------------------------------- */
int prodm_interleave(int dtype, const void* d_data, int ndims, const uint32_t* dims, const uint32_t* dims_fine,
                     const uint32_t* dims_coarse, void* d_buf, const uint32_t* strides, void* stream);
int prodm_reposition(int dtype, const void* d_buf, int ndims, const uint32_t* dims, const uint32_t* dims_fine,
                     const uint32_t* dims_coarse, void* d_data, const uint32_t* strides, void* stream);

/* ---------------------------------------------------------------------------
 * Bitplane encoder -- BitplaneEncoderInterface<T>::encode
 * (BitplaneEncoderInterface.hpp:16; NegaBinaryBPEncoder.hpp:18-125;
 * GroupedBPEncoder.hpp:18-145; PerBitBPEncoder.hpp:81-146, whose d_errors is
 * not computed: the reference pipeline calls its plain overload,
 * ComposedRefactor.hpp:124). PRODM_ENC_PERBIT needs d_blob 8-byte aligned.
 * Writes the level's streams concatenated in plane order into d_blob (the
 * byte layout of the reference level file with NullLevelCompressor) and the
 * per-plane byte sizes into d_sizes[B]. d_errors (nullable): the
 * error-collecting overload's B+1 squared-error table. n >= 1; a level with
 * fewer values than one block is one short block (the reference's loops wrap
 * there). workspace as for prodm_decompose.
 * ------------------------------------------------------------------------- */
int prodm_encode_bound(int encoder, int dtype, uint64_t n, int num_bitplanes, uint64_t* max_blob_bytes);
int prodm_encode_workspace(int encoder, int dtype, uint64_t n, int num_bitplanes, size_t* bytes);
int prodm_encode(int encoder, int dtype, const void* d_data, uint64_t n, int exp, int num_bitplanes, void* d_blob,
                 uint64_t blob_capacity, uint32_t* d_sizes, double* d_errors, void* d_workspace,
                 size_t workspace_bytes, void* stream);

/* Progressive decoder -- BitplaneEncoderInterface<T>::decode / progressive_decode
 * (BitplaneEncoderInterface.hpp:18-20; NegaBinaryBPEncoder.hpp:127-192;
 * GroupedBPEncoder.hpp:147-297; PerBitBPEncoder.hpp:290-383). The handle keeps
 * the per-level state of the grouped decoder (recording bitplanes and signs,
 * GroupedBPEncoder.hpp:379-380) and of the per-bit decoder (which elements'
 * signs are known, and the signs, PerBitBPEncoder.hpp:399-400), indexed by
 * level. A per-bit level is decoded plane after plane (each call starts where
 * the previous one stopped): a plane's bit positions depend on the planes
 * before it. d_blob holds planes [start, start+num) concatenated as the
 * reference retriever hands them over (FileRetriever.hpp:69-81); h_sizes are
 * their byte sizes (host). The first call for a level must start at plane 0.
 * Output: the contribution of these planes, n values, into d_out. */
typedef struct prodm_decoder prodm_decoder;
int prodm_decoder_create(prodm_decoder** out, int encoder, int dtype);
int prodm_progressive_decode(prodm_decoder* h, const void* d_blob, const uint32_t* h_sizes, uint64_t n, int exp,
                             int start_bitplane, int num_bitplanes, int level, int total_bitplanes, void* d_out,
                             void* stream);
int prodm_decoder_destroy(prodm_decoder* h);

/* ---------------------------------------------------------------------------
 * Lossless stage -- LevelCompressorInterface::compress_level / decompress_level
 * (LevelCompressorInterface.hpp:14-18) with AdaptiveLevelCompressor's rule
 * (AdaptiveLevelCompressor.hpp:13-53: planes 0..stopping and those from
 * max(latter, stopping + 1) on are compressed; the run stops at the first
 * plane after plane 0 whose ratio raw/compressed is below 1.05). The codec is
 * this library's GPU codec "ZCB" (zero-compacted bytes: u64 raw length, u32
 * chunk count, chunk end offsets, then per 4096-byte chunk 32 word masks, a
 * nibble of nonzero bytes per nonzero word and the nonzero bytes), not zstd:
 * files compressed by the reference's zstd stage are not readable with it.
 * d_blob: the level's streams concatenated (raw for compress, stored for
 * decompress); h_sizes: their byte sizes (host; for decompress the sizes of
 * planes [starting_bitplane, +num)). Outputs are concatenated into d_out;
 * h_out_sizes / h_raw_sizes receive the per-stream sizes (host).
 * ------------------------------------------------------------------------- */
int prodm_lossless_compress_bound(const uint32_t* h_sizes, int num_bitplanes, uint64_t* max_bytes);
int prodm_lossless_compress_level(const void* d_blob, const uint32_t* h_sizes, int num_bitplanes, int latter_index,
                                  void* d_out, uint64_t capacity, uint32_t* h_out_sizes, int* h_stopping_index,
                                  void* stream);
int prodm_lossless_decompress_level(const void* d_blob, const uint32_t* h_sizes, int starting_bitplane,
                                    int num_bitplanes, int stopping_index, int latter_index, void* d_out,
                                    uint64_t capacity, uint32_t* h_raw_sizes, void* stream);

/* ---------------------------------------------------------------------------
 * Error collectors -- ErrorCollectorInterface<T>::collect_level_error
 * (ErrorCollectorInterface.hpp:14). Max: MaxErrorCollector.hpp:14-25 (needs
 * no data; host output). Squared: SquaredErrorCollector.hpp:54-96 (device
 * data, device output of B+1 doubles).
 * ------------------------------------------------------------------------- */
int prodm_collect_max(int dtype, double max_level_error, int num_bitplanes, double* h_out);
int prodm_collect_squared_workspace(int dtype, int num_bitplanes, size_t* bytes);
int prodm_collect_squared(int dtype, const void* d_data, uint64_t n, int num_bitplanes, double max_level_error,
                          double* d_out, void* d_workspace, size_t workspace_bytes, void* stream);
/* Same table as prodm_collect_squared, allocating nothing. No counterpart in
 * the reference: it is for callers that cannot allocate device memory (hosts
 * whose own pool owns the HBM, or that forbid the device-synchronising
 * cudaMalloc/cudaFree inside their callbacks) and have no workspace to pass.
 * Its scratch is a fixed 316,160-byte device array, enough for
 * num_bitplanes <= 64 (fp64) / 32 (fp32); larger values return PRODM_EINVAL.
 * Every call on a stream that is not capturing looks up that array's address
 * on the current device (so it stays right after cudaDeviceReset); a call
 * during a stream capture uses the address of the device's last uncaptured
 * call, so make the first call before any capture. All calls on a device
 * share the array: calls that overlap on the GPU race; calls on one stream
 * are ordered. */
int prodm_collect_squared_noalloc(int dtype, const void* d_data, uint64_t n, int num_bitplanes,
                                  double max_level_error, double* d_out, void* stream);

/* ---------------------------------------------------------------------------
 * Packed level coefficients <-> natural field (hierarchical basis; the
 * _basis forms below take either basis).
 * prodm_recompose_packed: d_coef holds every level's coefficients packed as
 * the retrieval decodes them (level 0 box, then box(l) minus box(l-1) per
 * level in interleaved order, the layout of prodm_mdr_coefficients); output
 * is the natural-order field -- the reconstructor's reposition + recompose
 * (ComposedReconstructor.hpp:124-131; MGARD.hpp:25-35).
 * prodm_recompose_adjoint: its transpose. d_grad is the gradient of a scalar
 * quantity of interest with respect to the natural-order field; d_grad_coef
 * receives the gradient with respect to the packed level coefficients. No
 * counterpart in the reference (the reference has no derivatives); it gives
 * the per-level sensitivities used for QoI-bounded retrieval.
 * Workspace (both): prodm_recompose_packed_workspace bytes, or NULL to let
 * the call allocate it stream-ordered.
 * ------------------------------------------------------------------------- */
int prodm_recompose_packed_workspace(int dtype, int ndims, const uint32_t* dims, uint32_t target_level,
                                     size_t* bytes);
int prodm_recompose_packed(int dtype, const void* d_coef, int ndims, const uint32_t* dims, uint32_t target_level,
                           void* d_out, void* d_workspace, size_t workspace_bytes, void* stream);
int prodm_recompose_adjoint(int dtype, const void* d_grad, int ndims, const uint32_t* dims, uint32_t target_level,
                            void* d_grad_coef, void* d_workspace, size_t workspace_bytes, void* stream);
/* The same three for either basis (PRODM_BASIS_HIERARCHICAL as above, or
 * PRODM_BASIS_ORTHOGONAL: MGARDOrthoganalDecomposer's recomposition,
 * MGARD.hpp:11-39, which removes each level's L2 correction from its coarse
 * box before interpolating; its adjoint runs the correction's transpose --
 * per dim a coarse mass-matrix solve, the interpolation and the fine mass
 * matrix). The orthogonal workspace adds the correction's scratch boxes and
 * the adjoint's, the largest the level-L box. */
int prodm_recompose_packed_basis_workspace(int dtype, int basis, int ndims, const uint32_t* dims,
                                           uint32_t target_level, size_t* bytes);
int prodm_recompose_packed_basis(int dtype, int basis, const void* d_coef, int ndims, const uint32_t* dims,
                                 uint32_t target_level, void* d_out, void* d_workspace, size_t workspace_bytes,
                                 void* stream);
int prodm_recompose_adjoint_basis(int dtype, int basis, const void* d_grad, int ndims, const uint32_t* dims,
                                  uint32_t target_level, void* d_grad_coef, void* d_workspace, size_t workspace_bytes,
                                  void* stream);

/* ---------------------------------------------------------------------------
 * GE quantities of interest (fp64 fields), for QoI-bounded retrieval.
 * prodm_qoi_ge_values -- QoI::compute_QoIs (qoi_utils.hpp:135-165): V_TOT, T,
 * C, Mach, PT and mu of every point of (Vx, Vy, Vz, P, D), n values each
 * (products, quotients and square roots as the reference rounds them; its
 * pow(x, 7) and pow(x, 3) as multiplication chains, within a few ulp).
 * prodm_qoi_ge_bounds -- the pointwise error estimates the GE drivers form
 * from the propagation rules (qoi_utils.hpp:18-98): V_TOT from the square
 * and square-root rules given |error| <= eb_v* of each velocity component
 * (halving_Vtot.cpp:38-45), T from the division rule given eb_p, eb_d (0 where
 * the rule cannot bound it, as the reference). Pass NULL velocities or NULL
 * P/D to skip one QoI; bound arrays may be NULL; max_bounds (nullable, device,
 * 2 doubles) receives the maxima over the field.
 * ------------------------------------------------------------------------- */
int prodm_qoi_ge_values(int dtype, const void* d_vx, const void* d_vy, const void* d_vz, const void* d_p,
                        const void* d_d, uint64_t n, void* d_vtot, void* d_temp, void* d_c, void* d_mach,
                        void* d_pt, void* d_mu, void* stream);
int prodm_qoi_ge_bounds(int dtype, const void* d_vx, const void* d_vy, const void* d_vz, const void* d_p,
                        const void* d_d, uint64_t n, double eb_vx, double eb_vy, double eb_vz, double eb_p,
                        double eb_d, double* d_bound_vtot, double* d_bound_t, double* d_max_bounds, void* stream);

/* ---------------------------------------------------------------------------
 * Size interpreter -- SizeInterpreterInterface::interpret_retrieve_size
 * (SizeInterpreterInterface.hpp:13). Runs on the device. d_sizes[nl*B] plane
 * byte sizes, d_errors[nl*(B+1)] level error tables, d_index[nl] in/out
 * bitplanes already retrieved, d_retrieve_sizes[nl] out. target_level and
 * ndims parameterise the estimator tables; s is the S-norm exponent.
 * ------------------------------------------------------------------------- */
int prodm_interpret(int interpreter, int estimator, int dtype, int ndims, int target_level, double s, int nlevels,
                    int num_bitplanes, const uint32_t* d_sizes, const double* d_errors, double tolerance,
                    uint8_t* d_index, uint32_t* d_retrieve_sizes, void* stream);

/* ---------------------------------------------------------------------------
 * Device-resident composed refactor / reconstructor
 * (ComposedRefactor.hpp:21-141; ComposedReconstructor.hpp:27-258).
 * One handle per field configuration; all buffers are allocated at create.
 * Refactor: decompose -> per level interleave + max -> encode (+ squared error
 * tables when collector == PRODM_COLLECT_SQUARED), all on `stream`.
 * Retrieve: error tables -> interpreter -> decode every retrieved plane ->
 * recompose to full resolution into d_out; the per-level plane counts persist
 * between calls (progressive retrieval), prodm_mdr_reset_retrieval() clears them.
 * ------------------------------------------------------------------------- */
typedef struct prodm_config {
    int dtype;
    int ndims;
    uint32_t dims[3];
    int target_level;
    int num_bitplanes;
    int encoder;
    int basis;
    int collector;
} prodm_config;

typedef struct prodm_mdr prodm_mdr;
int prodm_mdr_create(prodm_mdr** out, const prodm_config* cfg);
int prodm_mdr_refactor(prodm_mdr* h, const void* d_field, void* stream);
/* host copies (synchronise the stream): sizes[(L+1)*B], bounds[L+1] as
 * double, errors[(L+1)*(B+1)] (squared tables; zeros when not collected) */
int prodm_mdr_level_info(prodm_mdr* h, uint32_t* h_sizes, double* h_bounds, double* h_errors, void* stream);
/* reference metadata bytes (ComposedRefactor.hpp:48-67) followed by an
 * extension carrying the squared-error tables; *len receives the size. */
int prodm_mdr_metadata(prodm_mdr* h, uint8_t* h_buf, size_t capacity, size_t* len, void* stream);
/* reference level-file bytes of one level into dst: dst_is_host 0 device
 * memory, 1 host memory (returns when the bytes are there), 2 pinned host
 * memory filled asynchronously in stream order (synchronise the stream, or
 * wait on an event recorded after the call, before reading it). */
int prodm_mdr_export_level(prodm_mdr* h, int level, void* dst, uint64_t capacity, int dst_is_host, uint64_t* len,
                           void* stream);
/* bytes [offset, offset + bytes) of the same level file into dst (dst_is_host
 * as above): a reader can start on the first planes of a level before the
 * rest of the file is out (ConcatLevelFileRetriever reads level files in
 * such consecutive pieces, FileRetriever.hpp:15-35) */
int prodm_mdr_export_level_range(prodm_mdr* h, int level, uint64_t offset, uint64_t bytes, void* dst,
                                 int dst_is_host, void* stream);

/* Lossless stage of the handle (AdaptiveLevelCompressor's rule with the ZCB
 * codec, see prodm_lossless_compress_level): latter_index >= 0 switches it on
 * (the reference's default is 26), < 0 off. While on, the plane sizes the
 * interpreter uses, prodm_mdr_level_info reports and the metadata carries are
 * the stored (compressed where the rule says) sizes, exactly as the
 * reference's ComposedRefactor records them after compress_level
 * (ComposedRefactor.hpp:131-135); the planes stay uncompressed in HBM;
 * prodm_mdr_export_level writes the stored streams and the metadata the
 * stopping indices plus a "ZCB1" marker with the latter index. A handle fed by
 * prodm_mdr_load_metadata takes the stage from the metadata; levels whose
 * metadata has stopping indices but no marker were written by the reference's
 * zstd stage (see prodm_mdr_set_zstd_latter). */
int prodm_mdr_set_lossless(prodm_mdr* h, int latter_index, void* stream);

/* Reading level files that the reference's lossless stage wrote: metadata
 * with stopping indices and no "ZCB1" marker came from
 * AdaptiveLevelCompressor (AdaptiveLevelCompressor.hpp:13-60), whose planes
 * at or below a level's stopping index and from its latter index on are zstd
 * frames (ZSTD.hpp:11-28: an 8-byte raw length, then the frame). The latter
 * index is the compressor's constructor argument and is not in the metadata:
 * this call gives it (26, the reference's default, when never called) and
 * must come before prodm_mdr_load_metadata. Such planes are expanded on the
 * host with libzstd.so.1, opened at run time, as their bytes complete (the
 * level bytes are kept on the host until then), and go to the device raw;
 * the stored sizes stay the interpreter's cost model, as in the reference's
 * reconstructor. Without libzstd, loading such metadata returns
 * PRODM_EUNSUPPORTED; a frame that does not expand to its recorded length
 * (for example with the wrong latter index) PRODM_ECORRUPT at the next
 * reconstruction. Replaces the reference's AdaptiveLevelCompressor::
 * decompress_level in ComposedReconstructor::progressive_reconstruct
 * (ComposedReconstructor.hpp:199-206) for the device-resident handle. */
int prodm_mdr_set_zstd_latter(prodm_mdr* h, int latter_index);
/* Level files (ConcatLevelFileWriter / ConcatLevelFileRetriever,
 * FileWriter.hpp:13-39, FileRetriever.hpp:15-35). load_level_file reads bytes
 * [file_offset, file_offset + bytes) of a level file straight into device
 * memory as the level's data at level_offset, like prodm_mdr_load_level: via
 * cuFile (GPUDirect Storage) where its driver opens and the file registers,
 * else via pread into pinned buffers whose asynchronous copies overlap the
 * next read. read_mode: 1 cuFile, 0 pinned, -1 no read yet. write_level_file
 * writes the level file (the bytes of prodm_mdr_export_level). */
int prodm_mdr_load_level_file(prodm_mdr* h, int level, const char* path, uint64_t file_offset, uint64_t level_offset,
                              uint64_t bytes, void* stream);
int prodm_mdr_write_level_file(prodm_mdr* h, int level, const char* path, void* stream);
int prodm_mdr_file_read_mode(prodm_mdr* h, int* read_mode);
int prodm_mdr_retrieve(prodm_mdr* h, double tolerance, int interpreter, int estimator, double s, void* d_out,
                       void* stream);
/* the two halves of prodm_mdr_retrieve: the interpreter alone (updates the
 * per-level plane counts on the device), then decode + recompose */
int prodm_mdr_interpret(prodm_mdr* h, double tolerance, int interpreter, int estimator, double s, void* stream);
int prodm_mdr_reconstruct(prodm_mdr* h, void* d_out, void* stream);
/* Reconstructor fed from the reference's on-disk format instead of a device
 * refactor (ComposedReconstructor::load_metadata, ComposedReconstructor.hpp:
 * 133-154, and ConcatLevelFileRetriever::retrieve_level_components,
 * FileRetriever.hpp:15-35): metadata bytes as written by
 * ComposedRefactor::write_metadata (the squared-error extension is optional),
 * then byte ranges [offset, offset+bytes) of level files as they are fetched.
 * A level's planes must be loaded before a reconstruct uses them. */
int prodm_mdr_load_metadata(prodm_mdr* h, const uint8_t* h_buf, size_t len, void* stream);
int prodm_mdr_load_level(prodm_mdr* h, int level, const void* src, uint64_t offset, uint64_t bytes, int src_is_host,
                         void* stream);
/* retrieve with explicit per-level plane counts (h_index[L+1]) */
int prodm_mdr_retrieve_planes(prodm_mdr* h, const uint8_t* h_index, void* d_out, void* stream);
/* h_index[L+1] <- the per-level plane counts; also reports (and clears) a
 * bounded wait of an earlier retrieval kernel that gave up (PRODM_ETIMEOUT) */
int prodm_mdr_get_index(prodm_mdr* h, uint8_t* h_index, void* stream);
/* synchronises the stream and reports (and clears) the status of the handle's
 * retrieval kernels: PRODM_OK, or PRODM_ETIMEOUT when a bounded wait for the
 * plane tiles of the fused finest-level kernel gave up (the output of that
 * retrieval is then incomplete) */
int prodm_mdr_status(prodm_mdr* h, void* stream);
/* test hook for the timeout path: later fused finest-level launches expect
 * extra_tx_bytes more bytes per plane tile than their copies deliver, so each
 * wait runs out after wait_cycles SM clock cycles (0, 0 restores the
 * defaults: exact byte counts, about two seconds) */
int prodm_debug_tile_wait(int extra_tx_bytes, long long wait_cycles);
int prodm_mdr_reset_retrieval(prodm_mdr* h, void* stream);
/* copies the packed level coefficients of the last refactor (level l at the
 * offset given by the sum of the earlier level sizes) into d_dst */
int prodm_mdr_coefficients(prodm_mdr* h, void* d_dst, void* stream);
int prodm_mdr_destroy(prodm_mdr* h);

/* ---------------------------------------------------------------------------
 * Batched refactor / retrieve of many fields (no counterpart in the
 * reference, which refactors one field per ComposedRefactor call,
 * ComposedRefactor.hpp:21-46). All fields share fp32, the negabinary encoder,
 * the hierarchical basis and the bitplane count; shapes and target levels are
 * per field. Each stage is one launch over all fields, so a whole batched
 * refactor or retrieve is a short fixed launch sequence that can be captured
 * in a CUDA graph (buffers are bound once with prodm_batch_bind).
 * Retrieval uses the max-error estimators with per-field tolerances
 * (prodm_batch_set_tolerances, L-inf absolute values).
 * ------------------------------------------------------------------------- */
typedef struct prodm_batch prodm_batch;
int prodm_batch_create(prodm_batch** out, int nfields, const prodm_config* cfgs);
int prodm_batch_bind(prodm_batch* h, const void* const* d_fields, void* const* d_outs);
/* launch shape of the row stages (decompose, recompose: 64, 128 or 256
 * threads per CTA, 1..32 CTAs per SM) and the encode grid (min(ctas, 8) CTAs
 * of 256 threads per SM) */
int prodm_batch_set_launch(prodm_batch* h, int threads_per_cta, int ctas_per_sm);
/* one stage's launch shape, as the autotuner sets them one stage at a time:
 * PRODM_BATCH_DECOMPOSE / PRODM_BATCH_RECOMPOSE (one warp per fine row;
 * threads 64, 128 or 256, CTAs per SM 1..32), PRODM_BATCH_ENCODE (256
 * threads, 1..8 CTAs per SM) or PRODM_BATCH_FUSED (the finest levels, decoded
 * inside their recomposition: 256 threads, 1..8 CTAs per SM, capped by what
 * fits on an SM) */
#define PRODM_BATCH_DECOMPOSE 0
#define PRODM_BATCH_ENCODE 1
#define PRODM_BATCH_RECOMPOSE 2
#define PRODM_BATCH_FUSED 3
int prodm_batch_set_stage_launch(prodm_batch* h, int stage, int threads_per_cta, int ctas_per_sm);
/* tile shape of the fused finest levels: about this many values per unit of
 * consecutive fine rows (256..8192; default 2112 = 8 rows of 264); rows per
 * unit are a multiple of 8, at most 64, and a unit whose planes no longer fit
 * a TMA box takes the cp.async kernel */
int prodm_batch_set_fused_unit(prodm_batch* h, int values_per_unit);
int prodm_batch_refactor(prodm_batch* h, void* stream);
int prodm_batch_set_tolerances(prodm_batch* h, const double* h_tolerances, void* stream);
int prodm_batch_retrieve(prodm_batch* h, int interpreter, int estimator, double s, void* stream);
int prodm_batch_reset(prodm_batch* h, void* stream);
int prodm_batch_field_info(prodm_batch* h, int field, uint8_t* h_index, uint32_t* h_sizes, double* h_bounds,
                           void* stream);
int prodm_batch_export_level(prodm_batch* h, int field, int level, void* dst, uint64_t capacity, int dst_is_host,
                             uint64_t* len, void* stream);
/* status of the batched fused kernels since the last call (PRODM_ETIMEOUT when
 * a wait for plane tiles gave up), reported once */
int prodm_batch_status(prodm_batch* h, void* stream);
int prodm_batch_destroy(prodm_batch* h);

/* ---------------------------------------------------------------------------
 * Diagnostics (no counterpart in the reference, whose only instrument is a
 * wall-clock Timer, RefactorUtils.hpp:145-170).
 * Stage timing records CUDA events on the launching stream around each stage;
 * prodm_mdr_stage_times returns accumulated milliseconds and counts for stage
 * id = kind * 17 + level, kinds 0 decompose, 1 encode, 2 interpret,
 * 3 decode, 4 recompose (arrays of 85 entries).
 * prodm_kernel_launch_count: kernels launched by this library so far.
 * ------------------------------------------------------------------------- */
int prodm_mdr_set_timing(prodm_mdr* h, int enable);
int prodm_mdr_stage_times(prodm_mdr* h, double* h_ms, uint32_t* h_counts);
int prodm_kernel_launch_count(uint64_t* out);

#ifdef __cplusplus
}
#endif
#endif /* PRODM_GB300_H */
