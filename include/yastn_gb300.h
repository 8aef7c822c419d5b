/*
 * yastn_gb300 — C ABI of the GB300 (sm_103a) block-sparse backend for YASTN.
 *
 * Every entry point takes device pointers, a device-resident plan (packed int64
 * records built by the host from YASTN's metadata tuples), element/dtype codes and
 * a cudaStream_t passed as void*. Entry points only enqueue work on that stream;
 * they allocate nothing (outputs and workspaces are owned by the caller) and return
 * a status code (YB_OK on success). Plans and record layouts are documented next to
 * each entry point; the record field indices are the YB_* constants below.
 *
 * Reference interfaces replaced (paths within the YASTN source tree):
 *   transpose_and_merge  yastn/backend/backend_torch.py:588-589 (-> _backend_torch_backwards.py:338-392)
 *   unmerge              yastn/backend/backend_torch.py:592-593 (-> _backend_torch_backwards.py:395-426)
 *   dot                  yastn/backend/backend_torch.py:549-550 (-> _backend_torch_backwards.py:98-138)
 *   transpose_dot_sum    yastn/backend/backend_torch.py:553-554 (-> _backend_torch_backwards.py:141-226)
 *   svd                  yastn/backend/backend_torch.py:318-319 (-> _backend_torch_backwards.py:26-66,
 *                        yastn/backend/linalg/torch_svd_gesdd.py:15-21, 296-428)
 *   eigh                 yastn/backend/backend_torch.py:369-384
 *   fix_svd_signs        yastn/backend/backend_torch.py:353-366
 *   apply_mask           yastn/backend/backend_torch.py:576-577 (-> _backend_torch_backwards.py:251-279)
 *   truncation_mask      yastn/tensor/linalg.py:637-735 (caller-side rule, fused here into one launch)
 *   append_vec_tl/br/tr/bl  yastn/tn/fpeps/envs/_env_contractions.py:211-365 (their copy chains, composed
 *                        into one yb_map_gather each)
 */
#ifndef YASTN_GB300_H
#define YASTN_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------- */
#define YB_OK 0
#define YB_ERR_INVALID 1      /* bad argument (sizes, null pointers, unsupported dtype) */
#define YB_ERR_CUDA 2         /* a CUDA launch/runtime call failed; see yb_last_cuda_error */
#define YB_ERR_NOT_CONVERGED 3 /* an iterative solver hit its sweep cap */
#define YB_ERR_TOO_LARGE 4    /* problem exceeds a documented size limit of the kernel */

/* ---- dtype codes ------------------------------------------------------------------- */
#define YB_F64 0
#define YB_C128 1

/* Version of this ABI (major*100 + minor). */
int yb_abi_version(void);
/* Last CUDA error code seen by the library on this thread (0 if none). */
int yb_last_cuda_error(void);

/* ==== family (a): strided block copies ================================================
 * One launch moves every block of a merge, unmerge or their adjoints.
 *
 * tasks: n_tasks records of YB_COPY_REC int64 each:
 *   [YB_CP_SRC] src offset (units)  [YB_CP_DST] dst offset (units)
 *   [YB_CP_NDIM] number of dims (1..YB_CP_MAXD), outermost first
 *   [YB_CP_COUNT] number of units in the task (< 2^31)
 *   [YB_CP_VEC] 1 if an FP64 task moves pairs of elements as 16-byte units (offsets,
 *   strides and extents of the record are then in pairs)
 *   [YB_CP_SIZE+i] extent, [YB_CP_SSTR+i] src stride, [YB_CP_DSTR+i] dst stride (units),
 *   [YB_CP_MAGIC+i], [YB_CP_SHIFT+i] fast-division constants of extent i
 *   [YB_CP_KIND] 0: a plain task (above); 1: a tiled transpose, for a task whose source is
 *   contiguous along a dim other than the destination-contiguous innermost one. Its dims
 *   are then the outer dims followed by two tile dims, y (the source-contiguous dim) and
 *   x (the destination-contiguous dim), whose extents count YB_COPY_TILE-wide tiles and
 *   whose strides are per tile (YB_COPY_TILE x the element stride; the source stride of y
 *   and the destination stride of x are YB_COPY_TILE); [YB_CP_NX], [YB_CP_NY] hold the
 *   element extents of x and y, [YB_CP_COUNT] the number of tiles. A CTA moves a tile
 *   through shared memory, reading along y and writing along x, both coalesced.
 * items: n_items pairs (task index, first unit or tile); each item covers up to
 *   YB_COPY_ITEM_UNITS units (YB_COPY_ITEM_TILES tiles for kind 1) of its task.
 * unit_bytes: element size, 8 (FP64) or 16 (complex128); src/dst must be 16-byte aligned
 *   when any task has YB_CP_VEC set.
 * Replaces the per-block copy loops of transpose_and_merge / unmerge and their adjoints.
 */
#define YB_COPY_REC 48
#define YB_CP_SRC 0
#define YB_CP_DST 1
#define YB_CP_NDIM 2
#define YB_CP_COUNT 3
#define YB_CP_VEC 4
#define YB_CP_KIND 5
#define YB_CP_NX 6
#define YB_CP_NY 7
#define YB_CP_MAXD 8
#define YB_CP_SIZE 8
#define YB_CP_SSTR 16
#define YB_CP_DSTR 24
#define YB_CP_MAGIC 32
#define YB_CP_SHIFT 40
#define YB_COPY_ITEM_UNITS 2048
#define YB_COPY_TILE 32
#define YB_COPY_ITEM_TILES 2
int yb_block_copy(const void* src, void* dst, int unit_bytes,
                  const int64_t* tasks, int n_tasks,
                  const int64_t* items, int n_items, void* stream);

/* Composed copy: one pass for a chain of block copies (merges, unmerges, transposes, block
 * negations, conjugation) between two GEMMs of a double-layer PEPS contraction.
 *   dst[i] = conj?(sign * src[|map[i]| - 1]) for map[i] != 0, sign = -1 where map[i] < 0;
 *   dst[i] = 0 for map[i] == 0.
 * map: n int32 entries (source indices + 1, so sources hold fewer than 2^31 - 1 elements);
 * dtype YB_F64 or YB_C128 (conj conjugates complex elements; ignored for YB_F64). Negation
 * and conjugation flip IEEE sign bits (as -x and conj(x) do), so the result is bit-exact.
 * src and dst must not overlap. The adjoint of an injective map is the same call with the
 * inverse map (inv[|map[i]| - 1] = sign * (i + 1)).
 * Replaces the chain fuse_legs / unfuse_legs / swap_gate / conj / the merges of tensordot in
 * append_vec_tl, append_vec_br, append_vec_tr, append_vec_bl
 * (yastn/tn/fpeps/envs/_env_contractions.py:211-365), each of whose steps is one
 * transpose_and_merge / unmerge / negate_blocks / conj call of the backend
 * (backend_torch.py:588-593). */
int yb_map_gather(const void* src, void* dst, int dtype, const int32_t* map, int64_t n, int conj,
                  void* stream);

/* ==== family (b): grouped sum-of-products GEMM ========================================
 * For every output block o:  C_o = alpha * sum_{t in terms(o)} op(A_t) op(B_t) + beta * C_o
 * outs: n_out records of YB_GEMM_OUT_REC int64:
 *   [0] c offset (elements) [1] m [2] n [3] ldc [4] first term [5] end term
 * terms: records of YB_GEMM_TERM_REC int64:
 *   [0] a offset [1] b offset [2] k [3] a row stride [4] a col stride
 *   [5] b row stride [6] b col stride [7] flags (bit0: conj A, bit1: conj B)
 *   A_t[i,l] = a[a_off + i*a_rs + l*a_cs], B_t[l,j] = b[b_off + l*b_rs + j*b_cs].
 * tiles: n_tiles records of 4 int32: (output, tile row, tile col, kind), ordered by the
 *   host (largest work first). kind 0: a 64x64 tile; kind 1: a skinny tile covering all
 *   m <= 16 rows and columns [w*col, w*col + w) with w = 1024 for m <= 8, 256 above (tile
 *   row 0; the host's plans use skinny tiles for m <= 8); kind 2: a short skinny tile, for an
 *   output of one term with m <= 8 rows and K <= 8 (any n), covering all rows and the 512
 *   columns [512*col, 512*col + 512); its "tile row" field holds the index of that term (the
 *   output's first term), so that the output and term records are read at once.
 * dtype: YB_F64 or YB_C128 (alpha, beta are real).
 * Replaces dot (one term per output), transpose_dot_sum after the merge of its operands,
 * and the adjoint products A_b += C_b B^H, B_b += A^H C_b (terms grouped by operand block).
 */
#define YB_GEMM_OUT_REC 8
#define YB_GEMM_TERM_REC 8
#define YB_GEMM_TILE 64
#define YB_GEMM_SKINNY_COLS 1024
#define YB_GEMM_SHORT_COLS 512
int yb_grouped_gemm(const void* a, const void* b, void* c, int dtype,
                    const int64_t* outs, const int64_t* terms, const int32_t* tiles, int n_tiles,
                    double alpha, double beta, void* stream);
/* yb_grouped_gemm_short: yb_grouped_gemm for plans whose tiles are all of kind 2 (the
 * contractions of a tensor with a small MPO block): a kernel of its own with few registers,
 * eight warps per SM scheduler, all loads of a thread's columns issued before its FMAs. */
int yb_grouped_gemm_short(const void* a, const void* b, void* c, int dtype,
                          const int64_t* outs, const int64_t* terms, const int32_t* tiles, int n_tiles,
                          double alpha, double beta, void* stream);
/* yb_gemm_reduce: the second pass of a split-K product. The host splits the K range of
 * outputs whose few tiles would leave most SMs idle into chunks, computes each chunk's
 * product into its own slot of a workspace P (yb_grouped_gemm with alpha 1, beta 0), then
 *   C_o = alpha * sum_{c < chunks} P[p_off + c*m*n + i*n + j] + beta * C_o
 * summed in chunk order. recs: YB_GEMM_RED_REC int64 per output: [0] c offset [1] m [2] n
 * [3] ldc [4] p offset [5] chunks. tasks: int32 pairs (record, item) covering each
 * output's m*n elements in items of YB_GEMM_RED_ITEM. */
#define YB_GEMM_RED_REC 8
#define YB_GEMM_RED_ITEM 1024
int yb_gemm_reduce(void* c, const void* p, int dtype, const int64_t* recs, const int32_t* tasks,
                   int n_tasks, double alpha, double beta, void* stream);

/* ==== family (b'): FP64 sector GEMMs emulated on BF16 tensor cores (split operands) ====
 * yb_ozaki_split: every row of each record is scaled by 2^-e (|entries| < 1, e stored as
 * int32) and written as slices_count (6, 7 or 8) balanced base-128 digits (|d_0| <= 128,
 * d_t in [-64, 63]) with weights 2^{-7(t+1)}, stored exactly as BF16. A rows are A's block
 * rows; B rows are B's block columns, read in place (no transposed copy). One launch splits
 * both operands of a dot.
 * recs: YB_OZ_SPLIT_REC int64 per record: [0] source offset [1] rows [2] K (real row length;
 *   2x the complex length for modes 1-3) [3] row stride [4] mode (0 real; 1, 2, 3: complex
 *   rows read as [re | im], [re | -im], [im | re]) [5] destination offset (BF16 elements,
 *   multiple of 16) [6] exponent offset [7] Kp = K rounded up to 16 (padding zeroed)
 *   [8] stride between consecutive k [9] operand (bit 0: 0 reads a_src and writes
 *   a_slices / a_exps, 1 the b_ ones) | tile rows << 8 (0: planes [slice][row][Kp] for
 *   yb_ozaki_gemm; 32, 64 or 128: the tile layout of yb_ozaki_gemm_tc, rows padded with zeros
 *   to a multiple of the tile rows, per slice blocks of tile rows x 16 ordered (row tile,
 *   K step), each in the canonical K-major core-matrix order: byte offset of (row r, k) in a
 *   block (r/8)*256 + (k/8)*128 + (r%8)*16 + (k%8)*2).
 *   Element k of row i is at source offset [0] + i*[3] + k*[8] (FP64 or complex elements).
 * groups: int32 pairs (record, first row) of 8-row groups covering each record's rows
 *   (padded rows included for the tile layout), one CTA each.
 * yb_ozaki_gemm: C = A B for every output record (16 int64): [0] c offset [1] m [2] n
 *   [3] ldc [4] A slices offset [5] A exponents offset [6] B slices offset
 *   [7] B exponents offset [8] K [9] Kp; tiles as for yb_grouped_gemm (64 x 64).
 *   Slice pairs with digit-weight sum below slices_count (6, 7 or 8) are multiplied with
 *   mma.sync BF16 -> FP32 (exact integer sums per 400-wide K-chunk) and combined in FP64.
 *   slices_count = 8 represents 57 bits of each operand (FP64-grade products).
 * Replaces dot (backend_torch.py:549-550) for real FP64 operands when the emulated path
 * is selected; the native yb_grouped_gemm stays the default.
 */
#define YB_OZ_SPLIT_REC 10
int yb_ozaki_split(const double* a_src, const double* b_src, void* a_slices, void* b_slices,
                   int* a_exps, int* b_exps, const int64_t* recs, const int32_t* groups, int n_groups,
                   int slices_count, void* stream);
int yb_ozaki_gemm(const void* a_slices, const int* a_exps, const void* b_slices, const int* b_exps,
                  double* c, const int64_t* outs, const int32_t* tiles, int n_tiles, int slices_count,
                  void* stream);
/* yb_ozaki_gemm_tc: yb_ozaki_gemm on the tcgen05 tensor cores, operands from
 * yb_ozaki_split in the tile layout (128 rows for A, tile_n for B; output records [4], [6] =
 * the A / B slice-0 offsets in that layout); tiles are (output, tile row, tile col, 0) of 128
 * rows x tile_n columns, tile_n = 64 or 32 (else YB_ERR_INVALID). With tile_n = 32 a chunk's
 * digit-diagonal accumulators take slices_count x 32 of the 512 tensor-memory columns and
 * consecutive chunks alternate between two such buffers, so the fold of one tile overlaps the
 * MMAs of the next. A persistent kernel, one CTA per SM, each walking its share of the tiles:
 * with cta_tiles = NULL CTA b takes tiles b, b + G, ... (G = min(n_tiles, SMs)); otherwise
 * the tiles are grouped by CTA and CTA b takes [cta_tiles[b], cta_tiles[b+1]) of n_ctas CTAs
 * (n_ctas <= the SM count, else YB_ERR_INVALID).
 * one warp streams the digit tiles (cp.async.bulk into a 4-stage ring), one issues the
 * tcgen05.mma into the digit-diagonal accumulators in tensor memory, sixteen fold the
 * accumulators exactly and write the tile (the same bits as yb_ozaki_gemm) while the next
 * tile's MMAs run. A CTA that gives up on a bounded wait stops writing and sets the status
 * word read by yb_ozaki_device_error. */
int yb_ozaki_gemm_tc(const void* a_slices, const int* a_exps, const void* b_slices, const int* b_exps,
                     double* c, const int64_t* outs, const int32_t* tiles, int n_tiles,
                     const int32_t* cta_tiles, int n_ctas, int tile_n, int slices_count, void* stream);
/* yb_ozaki_device_error: copies the tcgen05 kernel's status word to *out (0: no failure),
 * synchronising the stream, and clears it when reset != 0. */
int yb_ozaki_device_error(int* out, int reset, void* stream);

/* yb_ozaki_dot_static: a whole emulated dot in one call -- the native FP64 sectors
 * (yb_grouped_gemm), yb_ozaki_split (A and B) and yb_ozaki_gemm -- with all scratch
 * (digit planes and exponents) placed in a device array built into the library instead of
 * caller-provided memory.
 * No counterpart in the reference: it exists for callers that cannot allocate device
 * memory at call time (a host framework that owns the whole device memory budget and
 * forbids allocations after start-up, or a caller for which an allocation would
 * synchronise the device in the middle of its stream work). The caller still provides
 * A, B, C and the plan records, laid out as for the separate calls (split records in the
 * planes layout, tile rows 0). The sectors the emulation does not take (K < 16, or at most
 * 8 rows and more than 64 columns) come as yb_grouped_gemm records (nat_outs, nat_terms,
 * nat_tiles; alpha 1, beta 0) and must be a direct plan without split-K, whose chunk
 * workspace this call does not hold.
 * Limits and behaviour:
 *   - real FP64 only: dtype must be YB_F64 (YB_C128 returns YB_ERR_INVALID);
 *   - the scratch holds YB_STATIC_SCRATCH_BYTES; the call returns YB_ERR_TOO_LARGE when
 *     2*(a_slice_elems + b_slice_elems) + 4*(a_exp_count + b_exp_count) bytes (each
 *     region rounded up to 256 bytes) exceed it;
 *   - it allocates nothing; the first call on a device resolves the array's device
 *     address (cudaGetSymbolAddress, with that device current) and caches it, so that
 *     first call should come before any stream capture;
 *   - every call shares the array, which keeps the last call's contents; each region is
 *     rewritten before it is read, and calls that overlap on the GPU race on it;
 *   - C positions not covered by an output record are left untouched (zero them first). */
#define YB_STATIC_SCRATCH_BYTES (16u << 20)
int yb_ozaki_dot_static(const double* A, const double* B, double* C, int dtype,
                        const int64_t* split_recs, const int32_t* split_groups, int n_groups,
                        const int64_t* outs, const int32_t* tiles, int n_tiles,
                        const int64_t* nat_outs, const int64_t* nat_terms, const int32_t* nat_tiles,
                        int n_nat_tiles, int slices_count,
                        int64_t a_slice_elems, int64_t b_slice_elems, int64_t a_exp_count,
                        int64_t b_exp_count, void* stream);

/* ==== device-resident Lanczos (yastn/tensor/_krylov.py:17-46, yastn/krylov/_krylov.py:177-238;
 * the backend's vdot / add / norm, backend_np.py:553-577) ======================================
 * Vector operations of a Krylov expansion whose coefficients stay on the device (no host
 * synchronisation per step; capturable in a CUDA graph). YB_F64 or YB_C128 vectors of n
 * elements; parts: a workspace of yb_krylov_parts() values of the vector type (FP64 for the
 * norms); reductions are deterministic (fixed grid, partial sums added in order).
 *   yb_krylov_dot:     *out = sum_i conj(x_i) y_i
 *   yb_krylov_update:  w <- w - (*alpha) v1 - (*beta) v0 (v0 may be NULL), *norm_out = |w|
 *   yb_krylov_norm:    *out = |x|
 *   yb_krylov_scale:   out <- w / (*beta)
 *   yb_krylov_combine: y <- sum_{r < m} coeffs_r V[r] (V row-major, row stride ldv) */
int yb_krylov_parts(void);
int yb_krylov_dot(const void* x, const void* y, int64_t n, int dtype, void* parts, void* out, void* stream);
int yb_krylov_update(void* w, const void* v1, const void* v0, const void* alpha, const double* beta, int64_t n,
                     int dtype, double* parts, double* norm_out, void* stream);
int yb_krylov_norm(const void* x, int64_t n, int dtype, double* parts, double* out, void* stream);
int yb_krylov_scale(const void* w, const double* beta, int64_t n, int dtype, void* out, void* stream);
int yb_krylov_combine(const void* V, int64_t ldv, const void* coeffs, int m, int64_t n, int dtype, void* y,
                      void* stream);

/* ==== family (c): batched one-sided Jacobi SVD / symmetric eigendecomposition ==========
 * blocks: n_blocks records of YB_SVD_REC int64:
 *   [0] a offset [1] m [2] n [3] U offset [4] S offset [5] Vh offset
 *   [6] X offset (FP64 workspace) [7] W offset (FP64 workspace) [8] first pair item
 *   [9] k=min(m,n) [10] L=max(m,n) [11] N = k rounded up to even [12] 1 if m > n
 *   [13] X offset (FP32 workspace) [14] W offset (FP32 workspace)
 *   [15] number of super-vectors for yb_svd_block_sweeps (ceil(k / rows_per_super), even)
 *   [16] 1: QR-preconditioned (see yb_svd_qr; then [10] = k, the rows of R being k long)
 *   [17] L = max(m,n) of the QR workspaces [18] Z offset (k x L: X_0, then Q^T)
 *   [19] offset of the Householder vectors (k x L) [20] offset of tau (k)
 *   [21] offset of R's rows (k x k) [22] offset of the sorted W written by yb_svd_finalize
 *   (all FP64 workspace offsets) [23] number of super-vectors of the blocked FP64 phase
 * X holds the k vectors (rows of A, or of A^T when m > n) of length L, W the k x k
 * accumulated rotations (X = W X_0 throughout).
 * pair_items: int32 pairs (block, pair index 0..N/2-1) over all blocks.
 * state: int64[6*n_blocks + 4]: per block (max |cos| of the sweep in progress as double
 *   bits, converged flag, sweeps run in the current phase, largest |cos| of the last
 *   completed sweep, and the squared noise row norms of the FP32 and FP64 phases as double
 *   bits: (1e-5 scale_b ||A_b||_F)^2 and (1e-14 ||A_b||_F)^2, written by yb_svd_init), then
 *   the control words of the grid barrier (count, generation, error flag, all-converged
 *   flag). A pair with a row at or below its phase's noise norm is not rotated and does not
 *   count for convergence (rank-deficient blocks would otherwise keep O(1) cosines among
 *   their rounding-noise rows).
 * dtype: YB_F64 (workspaces float / double) or YB_C128 (complex64 / complex128, element
 *   offsets as above); tall complex blocks start from X_0 = A^H.
 * Sequence (mixed precision): yb_svd_init (X32 = scale_b (A or A^H), W32 = I, with
 * scale[b] a power of two that brings the block below 1 in magnitude; scale: double
 * [n_blocks] scratch); yb_svd_sweeps with precision 32 (or yb_svd_block_sweeps);
 * yb_svd_widen (W = widen(W32)); the host orthonormalises W (Newton-Schulz with the
 * grouped GEMM, T = W^H W) and forms X = W X_0 (for eigh: yb_svd_shift_prefill, then
 * X += W A); yb_svd_sweeps with precision 64; yb_svd_finalize. yb_svd_sweeps runs every
 * sweep of a phase in one cooperative launch (rounds separated by a grid barrier with a
 * bounded spin; on timeout the error control word is set and the kernel exits) and stops
 * after the first sweep in which each block's largest rotation |cos| was <= tol_stop, or
 * after max_sweeps (the host reads the state and maps non-convergence to an error).
 * shift != NULL (eigh): per-block shifts c_b = ||A_b||_F + 1 are computed and A_b + c_b I
 * is decomposed (Hermitian positive definite, so its SVD is its eigendecomposition);
 * finalize mode 1 writes eigenvalues ascending, mode 2 by descending magnitude, with
 * eigenvectors as columns of U (= W^H); mode 0 is the SVD (S descending; the vectors of
 * singular values at or below the FP64 noise norm completed to orthonormal vectors; state
 * as left by the sweeps, or NULL for a zero noise norm).
 * Replaces svd (backend_torch.py:318-319, torch_svd_gesdd.py:15-21) and eigh
 * (backend_torch.py:369-384, torch_eig_sym.py:14-32) for FP64 and complex128 blocks.
 */
#define YB_SVD_REC 24
int yb_svd_init(const void* a, void* work32, const int64_t* blocks, int n_blocks, int dtype,
                int64_t* state, double* shift, double* scale, void* stream);
int yb_svd_sweeps(void* work, const int64_t* blocks, int n_blocks, const int32_t* pair_items,
                  int n_pair_items, int max_rounds, int precision, int dtype, int max_sweeps,
                  double tol_stop, int64_t* state, void* stream);
/* yb_svd_block_sweeps: the FP32 phase with rows grouped into super-vectors of
 * rows_per_super (16, 8 or 4) rows: one CTA per pair of super-vectors holds their rows in
 * shared memory (2 * rows_per_super * lmax FP32 elements, lmax >= every L), runs up to
 * inner_sweeps Jacobi sweeps among them and applies the accumulated rotation to the W rows.
 * super_items: int32 pairs (block, super pair index 0..[15]/2-1); max_rounds = max([15]) - 1.
 * precision 32: the FP32 phase (rows_per_super 16, 8 or 4; super-vector count [15]);
 * precision 64: the FP64 phase on the FP64 workspace (rows_per_super 4 or 8; count [23]).
 * Returns YB_ERR_TOO_LARGE if the rows do not fit in shared memory. */
int yb_svd_block_sweeps(void* work32, const int64_t* blocks, int n_blocks, const int32_t* super_items,
                        int n_items, int max_rounds, int rows_per_super, int precision, int dtype, int max_sweeps,
                        int inner_sweeps, double tol_stop, int lmax, int64_t* state, void* stream);
int yb_svd_widen(const void* work32, void* work64, const int64_t* blocks, int n_blocks, int dtype,
                 int64_t* state, void* stream);
int yb_svd_shift_prefill(void* work64, const int64_t* blocks, int n_blocks, int dtype,
                         const double* shift, void* stream);
/* yb_svd_qr: the QR-preconditioned start (every block of the records has [16] = 1), in
 * place of yb_svd_init. Per block: scale and noise norms as yb_svd_init (the FP32 noise
 * norm is FP64's, 1e-14 scale_b ||A_b||_F), Z = X_0 in FP64, the Householder QR of M = Z^T
 * (M's columns are Z's rows: A^T for wide/square blocks, conj(A) for tall ones) in one
 * cooperative launch (groups of CTAs per block, group barriers with a bounded spin; on
 * timeout qctrl's error word is set), R's rows to [21], the FP32 start X32 = scale_b R and
 * W32 = I, the Householder vectors and tau kept, and Q^T formed in Z. The sweeps then run
 * on R's rows (row length k); yb_svd_finalize writes U's columns (wide) or Vh's rows (tall)
 * from X and the sorted W to [22]; the host completes Vh = conj(W_sorted) Q^T (wide) or
 * U = conj(Q) W_sorted^T (tall) with grouped GEMMs. qctrl: int64[qctrl_words] scratch,
 * at least n_blocks + 4 words: per block a counter of published reflectors (warps wait on
 * it with a bounded spin instead of a barrier per Householder step), then 4 words per CTA
 * group (barrier count, generation, error flag, unused); on a timeout a group's error word
 * (qctrl[n_blocks + 4 g + 2]) is set. On a graded spectrum Jacobi from R's rows needs a few
 * FP64 sweeps where Jacobi from A's rows needs tens. */
int yb_svd_qr(const void* a, void* work64, void* work32, const int64_t* blocks, int n_blocks, int dtype,
              int64_t* state, double* scale, int64_t* qctrl, int qctrl_words, void* stream);
int yb_svd_finalize(void* work, void* U, double* S, void* Vh, const int64_t* blocks,
                    int n_blocks, int dtype, int max_k, int mode, const double* shift,
                    const int64_t* state, int64_t* n_small, void* stream);
/* n_small (nullable, int64[n_blocks], zeroed by the caller): blocks whose completion would
 * cost more than 2^22 element operations in one CTA (n_zero k L) are not completed by
 * yb_svd_finalize; their count of small values is written there, and the caller completes
 * them: candidates from yb_fill_candidates (G, L x n_zero per block, uniform in [-1, 1)),
 * projected twice against the earlier vectors with grouped GEMMs, orthonormalised by yb_qr,
 * copied into the factor. recs of yb_fill_candidates: int64 pairs (offset, count). */
int yb_fill_candidates(void* G, const int64_t* recs, int n_recs, int dtype, void* stream);

/* SVD adjoint core (torch_svd_gesdd.py:296-428): per block record YB_ADJ_REC int64:
 *   [0] dA offset [1] m [2] n [3] U/gU offset [4] S/gS offset [5] Vh/gVh offset
 *   [6] offset of the k x k matrices P, Q, K [7] offset of TR [8] k
 *   [9] kind: 0 square, 1 wide (n > m), 2 tall (m > n)
 * With P = U^H gU and Q = Vh gVh^H given, writes K and initialises TR; the host
 * completes dA with grouped GEMMs (see yb_adjoint.cu). gS may be NULL. */
#define YB_ADJ_REC 16
int yb_svd_adjoint_core(const void* P, const void* Q, const double* S, const double* gS, void* K,
                        const void* gU, const void* gVh, void* TR, const int64_t* blocks,
                        int n_blocks, int dtype, void* stream);
/* ==== QR (backend qr, backend_np.py:511-520, backend_torch.py:475-484) ===============
 * yb_qr: reduced QR of every block, A = Q R with R's diagonal made positive (real), Q
 * m x k and R k x n row-major (k = min(m, n)). Records YB_SVD_REC int64 with [16] = 2:
 * [0] a offset [1] m [2] n [3] Q offset [5] R offset [9] k [17] m [18] Z offset (k x m)
 * [19] reflector offset (k x m) [20] tau offset (k) [21] R rows offset (k x k), workspace
 * offsets in FP64 (complex128) elements. The Householder factorisation is the one of
 * yb_svd_qr applied to M = A (wide blocks: to A's first m columns; the host forms
 * R[:, m:] = Q^H A[:, m:] with the grouped GEMM); R's part below the diagonal is zeroed.
 * yb_qr_adjoint_sym / yb_trsm_rt: the two elementwise steps of the QR adjoint (YB_F64 or
 * YB_C128; the rule torch's autograd applies to the reference's qr, backend_torch.py:475-484),
 *   dA = (gQ' + Q copyltu(M)) R^{-H},  M = R gR^H - gQ'^H Q
 * (gQ' = gQ, or gQ + A[:, m:] gR[:, m:]^H for wide blocks, whose dA[:, m:] = Q gR[:, m:]);
 * the products are grouped GEMMs. Records YB_QRADJ_REC int64: [0] M offset [1] k
 * [2] B offset [3] rows [4] ldb [5] R offset [6] ldr. copyltu: M <- tril(M, -1) +
 * tril(M, -1)^H + Re diag(M). trsm_rt: B <- B R^{-H} (R upper triangular with a real
 * diagonal, back substitution per row). */
#define YB_QRADJ_REC 8
int yb_qr(const void* a, void* Q, void* R, void* work64, const int64_t* blocks, int n_blocks, int dtype,
          int64_t* qctrl, int qctrl_words, void* stream);
int yb_qr_adjoint_sym(void* M, const int64_t* recs, int n_blocks, int dtype, void* stream);
int yb_trsm_rt(void* B, const void* R, const int64_t* recs, int n_blocks, int dtype, void* stream);

/* yb_eigh_adjoint_core: the inner matrix K of the eigh adjoint dA = U K op(U)^T per block,
 * from X = op(U)^T gU (k x k, grouped GEMM): symeig != 0 (order_by_magnitude, SYMEIG of
 * yastn/backend/linalg/torch_eig_sym.py:43-54, op(U) = U): K_ij = X_ij (d_j - d_i) /
 * ((d_j - d_i)^2 + eps); symeig == 0 (torch.linalg.eigh's adjoint, op(U) = conj(U)):
 * K_ij = (X_ij - conj X_ji) / (2 (d_j - d_i)); K_ii = gD_i (gD may be NULL: 0, or
 * i Im X_ii for symeig == 0). blocks: records of 4 int64 (X/K offset, k, d offset, 0).
 * Replaces SYMEIG.backward and torch.linalg.eigh's backward (backend_torch.py:369-384). */
int yb_eigh_adjoint_core(const void* X, const double* D, const double* gD, void* K,
                         const int64_t* blocks, int n_blocks, int dtype, int symeig, double eps,
                         void* stream);

/* ==== masks / gauge ================================================================== */
/* Gather along one axis: out[sln].reshape(pre, Dn_ax, post)[:, i, :] =
 *   A[sla].reshape(pre, Da_ax, post)[:, idx[idx_off + i], :]
 * recs: records of YB_MASK_REC int64: [0] sln start [1] sla start [2] pre [3] Da_ax
 *   [4] Dn_ax [5] post [6] idx offset [7] unused (offsets in units).
 * items: n_items pairs (record, first output unit), each covering up to
 *   YB_COPY_ITEM_UNITS units. scatter != 0 runs the adjoint: A positions are written
 *   from out (the caller zero-fills the destination first).
 * Replaces apply_mask (backend_torch.py:576-577) and kernel_apply_mask.backward. */
#define YB_MASK_REC 8
int yb_mask_gather(const void* A, void* out, int unit_bytes, const int64_t* recs, const int64_t* items,
                   int n_items, const int64_t* idx, int scatter, void* stream);

/* fix_svd_signs (backend_np.py:447-458): per block record YB_SVD_REC (uses [1] m, [2] n,
 * [3] U offset, [4] S offset, [5] Vh offset, [9] k). U[:, c] *= conj(phase_c),
 * Vh[c, :] *= phase_c, where phase_c = U[r, c]/|U[r, c]| at the first row r maximising
 * int64(|U[r, c]| * 2^40). Writes Uout/Vout (may alias the inputs).
 * apply_given = 0: phases are computed and stored in `phases` (dtype, indexed like S;
 * may be NULL). apply_given = 1: the phases are read from `phases` instead (used by
 * the real adjoint, where the phases are the constants +-1). max_k: largest k. */
int yb_fix_signs(const void* Uin, const void* Vin, void* Uout, void* Vout, void* phases,
                 const int64_t* blocks, int n_blocks, int max_k, int dtype, int apply_given,
                 void* stream);
/* yb_fix_signs_adjoint: the adjoint of fix_svd_signs as torch's autograd differentiates the
 * reference's backend_torch.py:353-366 (YB_F64 or YB_C128; complex gradients in torch's
 * convention). Uin/Vin: the forward's inputs; gU/gV: cotangents of its outputs; per column c
 * with p the forward's phase (recomputed from Uin by the same row rule):
 * dU[:, c] = gU[:, c] p, dVh[c, :] = gVh[c, :] conj(p), and for complex data
 * dU[r, c] += -i (p / |U[r, c]|) Im(conj(G) p) at the selected row r, with
 * G = sum_i U[i, c] conj(gU[i, c]) + sum_j conj(Vh[c, j]) gVh[c, j]. Records as yb_fix_signs. */
int yb_fix_signs_adjoint(const void* Uin, const void* Vin, const void* gU, const void* gV, void* dU, void* dV,
                         const int64_t* blocks, int n_blocks, int max_k, int dtype, void* stream);

/* Fused truncation rule of yastn/tensor/linalg.py:637-735 over a flat spectrum.
 * S: n values; blk: n_blk records of 4 int64 (start, stop, D_block (or -1 = inf), unused);
 * tol_block: n_blk doubles; D_total < 0 means inf. Outputs mask (uint8[n]) and
 * kept (int64[n_blk]). Single-CTA kernel: n <= YB_TRUNC_MAX. */
#define YB_TRUNC_MAX 16384
int yb_truncation_mask(const double* S, int64_t n, const int64_t* blk, const double* tol_block,
                       int n_blk, double tol, int64_t D_total, int truncate_multiplets,
                       uint8_t* mask, int64_t* kept, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* YASTN_GB300_H */
