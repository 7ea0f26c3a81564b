/* fhgb300.h - C ABI of the GB300-native Fast-Higashi fit hot path (libfhgb300.so).
 *
 * Every entry point takes device pointers, plain sizes and a cudaStream_t passed as
 * void*, launches on that stream and returns an fh_status (0 = ok).  Nothing here
 * allocates device memory unless its comment says so; temporary storage is a caller
 * workspace whose size the matching *_workspace function reports.  The library has no
 * CPU fallback: without a usable GPU every entry point returns FH_ERR_LAUNCH.
 *
 * Reference citations are paths within ma-compbio/Fast-Higashi.
 */
#ifndef FHGB300_H
#define FHGB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum fh_status {
  FH_OK = 0,
  FH_ERR_ARG = 1,          /* bad pointer, shape or count                                   */
  FH_ERR_UNSUPPORTED = 2,  /* a size or option outside what the kernels handle              */
  FH_ERR_NONFINITE = 3,    /* NaN/Inf met in an input or produced by a factorisation        */
  FH_ERR_ILLCOND = 4,      /* a factorisation met a zero or non-positive pivot              */
  FH_ERR_LAUNCH = 5,       /* a CUDA launch or runtime call failed                          */
  FH_ERR_INDEX = 6,        /* a contact index lies outside its tile                         */
  FH_ERR_TIMEOUT = 7       /* a bounded device-side wait ran out                            */
} fh_status;

/* A packed contact of one (tile, cell) segment: local row in the low 16 bits of rc, local
 * compact column in the high 16 bits, and its value. */
typedef struct fh_entry {
  uint32_t rc;
  float v;
} fh_entry;

/* One bin batch of one chromosome in the compact band layout (Chrom_Dataset with
 * compact=True, fasthigashi/sparse_for_schic.py:401-492). */
typedef struct fh_tile {
  int32_t chrom;   /* dataset (chromosome) index                                        */
  int32_t row0;    /* first row bin of the bin batch within its chromosome              */
  int32_t rows;    /* b: row bins of the batch                                          */
  int32_t width;   /* n: compact columns (local_bin_slice / col_bin_slice widths)       */
  int32_t shift;   /* local column = chromosome column - shift                          */
  int32_t s0;      /* first compact column holding the batch's own bins (s1 = s0+rows)  */
  int32_t rank;    /* r of the chromosome (chrom2size)                                  */
  int32_t n_rwr;   /* RWR epochs (force_rwr_epochs)                                     */
  int64_t xoff;    /* first band row of the tile: band row = xoff + i*width + j         */
  int64_t brow0;   /* first bin row of the tile in the all-chromosome bin-row numbering */
  int64_t uoff;    /* first element of the tile's projection U (rows x width x rank)    */
} fh_tile;

const char* fh_status_string(int status);
int fh_version(void);

/* ---- sparse per-cell contact build (sparse_for_schic.py:401-503 tiling + 279-353 densify) */

/* Counts the contacts of one chromosome per (tile, cell).  row/col/cell: int32[nnz] COO of
 * the chromosome (Sparse.indices); tiles[tile_base .. tile_base+n_tiles) are its bin
 * batches of bs_bin rows; counts: int32[n_tiles_total * n_cells], accumulated.  Entries
 * whose compact column falls one step outside the tile are dropped, as the reference's
 * padded densify crops them; anything farther sets FH_ERR_INDEX in *status. */
int fh_contacts_count(const int32_t* row, const int32_t* col, const int32_t* cell, int64_t nnz,
                      int32_t bs_bin, const fh_tile* tiles, int32_t tile_base, int32_t n_tiles,
                      int32_t n_cells, int32_t* counts, int* status, void* stream);

/* Exclusive prefix sum of int32 counts into int64 offsets[n+1].  workspace: see below. */
size_t fh_scan_workspace(int64_t n);
int fh_exclusive_scan(const int32_t* counts, int64_t n, int64_t* offsets, void* workspace,
                      size_t workspace_bytes, void* stream);

/* x[i] += *base for i < n (base: one device int64).  Chains the scan of one dataset's counts
 * onto the total of the datasets before it, so a contact build can proceed dataset by dataset
 * without a host round trip. */
int fh_scan_add_base(int64_t* x, int64_t n, const int64_t* base, void* stream);

/* fh_exclusive_scan without a workspace argument, for callers that cannot allocate device
 * memory (a foreign-language binding that holds only its own buffers, or code that must not
 * call cudaMalloc because it synchronizes the device).  No counterpart in the reference.
 * The scratch is a 64 KiB array in the library's device memory, held by every GPU that
 * loads the library until exit; n may be at most 16,775,168 (FH_ERR_UNSUPPORTED beyond).
 * The first call on a device looks up the array's address once; make that first call
 * before any stream capture.  All calls share the array: calls that overlap on the GPU
 * (on different streams, or from several threads at once) race and must be serialized by
 * the caller.  Allocates nothing. */
int fh_exclusive_scan_noalloc(const int32_t* counts, int64_t n, int64_t* offsets, void* stream);

/* Writes each contact as a packed entry (uint32 local_row | local_col << 16, float value)
 * into its (tile, cell) segment [offsets[t*n_cells+c], offsets[t*n_cells+c+1]).  cursor:
 * int32[n_tiles_total * n_cells], zeroed by the caller before the first chromosome. */
int fh_contacts_scatter(const int32_t* row, const int32_t* col, const int32_t* cell,
                        const float* val, int64_t nnz, int32_t bs_bin, const fh_tile* tiles,
                        int32_t tile_base, int32_t n_tiles, int32_t n_cells,
                        const int64_t* offsets, int32_t* cursor, fh_entry* entries,
                        void* stream);

/* Densifies cells [c0, c0+ncell) of tile t from its packed segments into
 * out[ncell][rows][width] with the 1e-8 floor (Fake_Sparse.densify / densify_jit with
 * transpose=True, sparse_for_schic.py:279-320, 352-353). */
int fh_densify_tile(const fh_tile* tiles, int32_t t, int32_t n_cells, int32_t c0, int32_t ncell,
                    const int64_t* offsets, const fh_entry* entries, float* out, void* stream);

/* ---- partial random walk with restart (partial_rwr.py:47-175, do_conv=False, do_col=False)
 *
 * fh_rwr_tiles_f32: densifies every (tile, cell) segment (floor 1e-8,
 * sparse_for_schic.py:320), builds the column-stochastic P (partial_rwr.py:84-111) and
 * writes out[c * cell_stride + xoff + i*width + j] = (Q_{n_rwr} A)[i][j] with
 * Q_{t+1} = 0.5 Q_t P + 0.5 I (partial_rwr.py:112-138), all in fp32.  sumsq (optional,
 * double[n_tiles * n_cells]) receives each (tile, cell)'s squared Frobenius norm of the
 * output (parafac2_intergrative.py:369).  max_rows / max_width bound every tile's rows and
 * width (b <= 128, n <= 320); a tile outside them sets FH_ERR_ARG in *status. */
int fh_rwr_tiles_f32(const fh_tile* tiles, int32_t n_tiles, int32_t n_cells,
                     int32_t max_rows, int32_t max_width, const fh_entry* entries,
                     const int64_t* offsets, float* out, int64_t cell_stride, double* sumsq,
                     int* status, void* stream);

/* fh_rwr_tiles_f32 with the output stored as bf16 planes (out16: bf16 bits, same indexing):
 * plane 0 = bf16(x); with plane_stride > 0 a second plane at out16 + plane_stride holds
 * bf16(x - plane 0), which carries x to 16 significant bits.  The sumsq entries are taken
 * over the stored value.  Feeds fh_xe_bf16 / fh_xg_bf16. */
int fh_rwr_tiles_bf16(const fh_tile* tiles, int32_t n_tiles, int32_t n_cells,
                      int32_t max_rows, int32_t max_width, const fh_entry* entries,
                      const int64_t* offsets, uint16_t* out16, int64_t cell_stride,
                      int64_t plane_stride, double* sumsq, int* status, void* stream);

/* The same partial RWR on the tcgen05 tensor cores (no reference counterpart: the reference
 * runs torch.bmm in fp32, partial_rwr.py:85-138): S2 = A A^T and every P Z_t product with
 * bf16 operands split hi|lo (three products, fp32 accumulators in TMEM), the recurrence
 * Z_{t+1} = 0.5 P Z_t + 0.5 A of fh_rwr_tiles_f32, and the same output planes as
 * fh_rwr_tiles_bf16.  max_rows <= 128 and max_width <= 256 (FH_ERR_UNSUPPORTED otherwise).
 * form: 0 the library default (1); 1 P in shared memory, one product group per epoch over the
 * tile's width; 2 P in tensor memory as the MMAs' A operand, epochs pipelined by 64-column
 * blocks of Z (each block's epilogue behind the other blocks' products) and the output moved
 * by bulk copies that run on into the next item (max_width <= 192, FH_ERR_UNSUPPORTED
 * otherwise).  Both forms give the same values; which is faster depends on the shape (the
 * engine's autotuner times both). */
int fh_rwr_tiles_tc(const fh_tile* tiles, int32_t n_tiles, int32_t n_cells, int32_t max_rows,
                    int32_t max_width, const fh_entry* entries, const int64_t* offsets,
                    uint16_t* out16, int64_t cell_stride, int64_t plane_stride, double* sumsq,
                    int32_t form, int* status, void* stream);

/* fh_rwr_tiles_f32 with the walk weight free: Q_{t+1} = rp Q_t P + (1 - rp) I, the form of
 * partial_rwr.py:109,116-118 where rp is fixed at 0.5 (0 <= rp < 1).  The forward of the
 * differentiable reconstruction loss. */
int fh_rwr_tiles_rp_f32(const fh_tile* tiles, int32_t n_tiles, int32_t n_cells,
                        int32_t max_rows, int32_t max_width, const fh_entry* entries,
                        const int64_t* offsets, float rp, float* out, int64_t cell_stride,
                        double* sumsq, int* status, void* stream);

/* Derivative of the RWR output with respect to rp, recomputing each tile (no reference
 * counterpart: the reference has no backward pass).  With Z_0 = A, Z_{t+1} = rp P Z_t +
 * (1 - rp) A and Z'_{t+1} = rp P Z'_t + P Z_t - A, writes dx = Z'_{n_rwr} and, when x is not
 * null, x = Z_{n_rwr} (bit-identical to fh_rwr_tiles_rp_f32), in the layout of
 * fh_rwr_tiles_f32.  max_rows <= 128, and 4 * (b*((b+3)&~3) + b*(n|1) + 130 b + 384) bytes
 * of shared memory must fit in 227 KB (n <= 203 at b = 125). */
int fh_rwr_grad_f32(const fh_tile* tiles, int32_t n_tiles, int32_t n_cells, int32_t max_rows,
                    int32_t max_width, const fh_entry* entries, const int64_t* offsets,
                    float rp, float* x, float* dx, int64_t cell_stride, int* status,
                    void* stream);

/* ---- do_conv: the 3 x 3 mean before the walk (partial_rwr.py:79-83) ----------------------
 * fh_conv_tiles_f32: for every (tile, cell), the floored densified tile (segments as in
 * fh_rwr_tiles_f32) smoothed by F.avg_pool2d(x, 3, 1, padding=1) (zero padding counted: the
 * window sum over 9) and floored at 1e-8 again, written to out in the X layout
 * (out[c * cell_stride + xoff + i*width + j]); tiles of one row are copied unsmoothed.
 * fh_conv_dense_f32: the same on a dense x[n_cells][rows][width] -> out (same shape).
 * fh_rwr_tiles_dense_f32 / _bf16 / _deltas: fh_rwr_tiles_f32 / _bf16 / _deltas with the tiles
 * read from a dense fp32 array in the X layout (src; out may be src: each tile is read by the
 * CTA that writes it, before it writes). */
int fh_conv_tiles_f32(const fh_tile* tiles, int32_t n_tiles, int32_t n_cells, int32_t max_rows,
                      int32_t max_width, const fh_entry* entries, const int64_t* offsets,
                      float* out, int64_t cell_stride, int* status, void* stream);
int fh_conv_dense_f32(const float* x, int32_t n_cells, int32_t rows, int32_t width, float* out,
                      void* stream);
int fh_rwr_tiles_dense_f32(const fh_tile* tiles, int32_t n_tiles, int32_t n_cells,
                           int32_t max_rows, int32_t max_width, const float* src, float* out,
                           int64_t cell_stride, double* sumsq, int* status, void* stream);
int fh_rwr_tiles_dense_bf16(const fh_tile* tiles, int32_t n_tiles, int32_t n_cells,
                            int32_t max_rows, int32_t max_width, const float* src,
                            uint16_t* out16, int64_t cell_stride, int64_t plane_stride,
                            double* sumsq, int* status, void* stream);
int fh_rwr_tiles_dense_deltas(const fh_tile* tiles, int32_t n_tiles, int32_t n_cells,
                              int32_t max_rows, int32_t max_width, const float* src,
                              int64_t cell_stride, int32_t cap, float* deltas, int* status,
                              void* stream);

/* ---- do_col: the column-normalised walk (partial_rwr.py:112-138, parafac2_intergrative.py
 * :96-276) -------------------------------------------------------------------------------
 * fh_rwr_col_tiles: for every (tile, cell), Q_T (Q_0 = I, Q_{t+1} = 0.5 Q_t P + 0.5 I), then
 *   with cov: X = Q' (A / cov_row), Q' = rownorm(max((Q + Q^T) / 2, 0)) (row sums + 1e-15),
 *             cov_row[j] = cov[c * cov_ld + (brow0 - row0) + shift + j] (the cell's coverage
 *             of the tile's global column j, bins numbered across chromosomes);
 *   cov null: X = Q A (the plain walk in the reference's association).
 * A is the floored tile of the (tile, cell) segment (entries/offsets as fh_rwr_tiles_f32), or
 * the dense fp32 tile in the X layout when dense is given (the 3 x 3 mean of do_conv; out may
 * be dense).  cell_epochs[t * n_cells + c] overrides the tile's n_rwr when given.  X goes to
 * out (fp32, X layout), else to out16 (bf16 planes as fh_rwr_tiles_bf16), else nowhere;
 * sumsq[t * n_cells + c] = ||X||^2 when sumsq is given (and X is written); colsum, when given,
 * receives the column sums of X at colsum[(t * n_cells + c) * max_width + j].  Shared memory
 * 4 * (2 b ((b+3)&~3) + b (((n+31)/32)*32 + 1) + 384) bytes must fit in 227 KB.
 * fh_rwr_col_dense: the with-cov form on a dense x[n_cells][rows][width] with cov[n_cells]
 *   [width] (partial_rwr's bin_cov argument) -> out[n_cells][rows][width].
 * fh_col_coverage: cov[c][g] = 1e-4 + the colsum entries of every tile holding global column
 *   g, added in tile order (bin_cov of init_params, :96-99, 141-142, 199-200), for g < n_cols.
 * fh_col_coverage_finalize: cov[i] <= 1e-4 -> +inf for i < n (:266-270). */
int fh_rwr_col_tiles(const fh_tile* tiles, int32_t n_tiles, int32_t n_cells, int32_t max_rows,
                     int32_t max_width, const fh_entry* entries, const int64_t* offsets,
                     const float* dense, const float* cov, int64_t cov_ld,
                     const int32_t* cell_epochs, float* out, uint16_t* out16,
                     int64_t cell_stride, int64_t plane_stride, double* sumsq, float* colsum,
                     int* status, void* stream);
int fh_rwr_col_dense(const float* x, int32_t n_cells, int32_t rows, int32_t width, int32_t s0,
                     int32_t n_epochs, const float* cov, float* out, int* status, void* stream);
int fh_col_coverage(const fh_tile* tiles, int32_t n_tiles, int32_t n_cells, const float* colsum,
                    int32_t max_width, float* cov, int64_t cov_ld, int64_t n_cols, int* status,
                    void* stream);
int fh_col_coverage_finalize(float* cov, int64_t n, void* stream);

/* Same arithmetic on a dense tile x[n_cells][rows][width] (the partial_rwr drop-in: no
 * floor is applied to x); out[n_cells][rows][width]. */
int fh_rwr_dense_f32(const float* x, int32_t n_cells, int32_t rows, int32_t width, int32_t s0,
                     int32_t n_epochs, float* out, int* status, void* stream);

/* Auto-stop rule of partial_rwr.py:99-126: deltas[c * cap + e] = ||Q_e - Q_{e+1}||_F for
 * e < cap, per cell of a dense tile x[n_cells][rows][width]. */
int fh_rwr_dense_deltas(const float* x, int32_t n_cells, int32_t rows, int32_t width,
                        int32_t s0, int32_t cap, float* deltas, int* status, void* stream);

/* Same on the packed segments of every tile (init_params, parafac2_intergrative.py:124-140):
 * deltas[(t * n_cells + c) * cap + e]. */
int fh_rwr_tiles_deltas(const fh_tile* tiles, int32_t n_tiles, int32_t n_cells,
                        int32_t max_rows, int32_t max_width, const fh_entry* entries,
                        const int64_t* offsets, int32_t cap, float* deltas, int* status,
                        void* stream);


/* ---- ALS streaming contractions over the cached RWR output (parafac2_intergrative.py:304-540)
 *
 * X: float[n_cells][ldx], band rows [0, rows), ldx a multiple of 128, padding zero.
 * E: float[n_cells][rp] (meta_embedding, columns >= R zero).  rp in {16, 32, 64, 128}.
 *
 * fh_xe_f32:  W[row][m] = sum_c X[c][row] E[c][m]  (W: float[rows][rp]).  W_i = X_i E gives
 *             temp_i = W_i D diag(A_i) B^T (:336,374-383) and Y_i = U_i^T W_i (:522-529).
 * fh_xg_f32:  out[c][m] = sum_row X[c][row] Gt[row][m]  (SVD_term^T, :422-477) with
 *             Gt_i = U_i lhs2_i^T; partial: float[splits][n_cells][rp] workspace, splits from
 *             fh_xg_splits (the reduction over splits runs in a fixed order).  accumulate != 0
 *             adds the sum into out instead (X held in several row ranges, one call each). */
int fh_xe_f32(const float* X, int64_t ldx, int32_t n_cells, int64_t rows, const float* E,
              int32_t rp, float* W, void* stream);
int fh_xg_splits(int32_t n_cells, int64_t rows);
int fh_xg_f32(const float* X, int64_t ldx, int32_t n_cells, int64_t rows, const float* Gt,
              int32_t rp, int32_t splits, float* partial, float* out, int32_t accumulate,
              void* stream);

/* ---- the same two passes over X held in bf16, on the tcgen05 tensor cores (no reference
 * counterpart: the reference's passes are fp32 torch.bmm / opt_einsum calls at
 * parafac2_intergrative.py:374-383, 422-430 and 522-529).
 * X16: bf16[planes][n_cells_total][ldx] (ldx % 128 == 0, columns >= rows zero), written by
 * fh_rwr_tiles_bf16; planes = 1 (bf16(X)) or 2 (X to 16 significant bits).  The small
 * operand is passed split, hi | lo = fh_split_bf16(x), so the products carry it to 16
 * significant bits; the error is that of X's planes.
 * fh_split_bf16: dst[row][0, rp) = bf16(x), dst[row][rp, 2 rp) = bf16(x - bf16(x)) for
 *                x = src[row * ld_src + m].
 * fh_xe_bf16:    W[row][m] = sum_{c < n_cells} X16[c][row] E[c][m];  E2 = split of E
 *                (bf16[n_cells][2 rp]).  rp in {32, 64, 128}.
 * fh_xg_bf16:    out[c][m] = sum_row X16[c][row] Gt[row][m] for c < n_cells;  G2 = split of
 *                Gt (bf16[rows][2 rp]); partial: float[splits][n_cells][rp] with splits from
 *                fh_xg_bf16_splits (fixed-order reduction in fp64); accumulate != 0 adds
 *                the sum into out.
 * fold: K chunks of 64 (cells for fh_xe_bf16, band rows for fh_xg_bf16) summed in one tensor
 *       memory accumulator before the epilogue folds them into Kahan-compensated fp32 running
 *       sums; 0 selects the library default (8).  Short runs keep the fp32 rounding of long K
 *       ranges out of the result.
 * status: int32 device word; a device-side wait that runs out sets FH_ERR_TIMEOUT. */
int fh_split_bf16(const float* src, int64_t n_rows, int32_t rp, int64_t ld_src, uint16_t* dst,
                  void* stream);
int fh_xe_bf16(const uint16_t* X16, int64_t ldx, int32_t n_cells_total, int32_t planes,
               int32_t n_cells, int64_t rows, const uint16_t* E2, int32_t rp, int32_t fold,
               float* W, int* status, void* stream);
int fh_xg_bf16_splits(int32_t n_cells, int64_t rows);
int fh_xg_bf16(const uint16_t* X16, int64_t ldx, int32_t n_cells_total, int32_t planes,
               int32_t n_cells, int64_t rows, const uint16_t* G2, int32_t rp, int32_t splits,
               int32_t fold, float* partial, float* out, int32_t accumulate, int* status,
               void* stream);

/* Y[g][l][m] = sum_j U_g[j][l] W[xoff + i*width + j][m] for every bin row g (K16 tail,
 * parafac2_intergrative.py:522-529); Y: float[n_rows][ldy_l][rp]; row_tile: int32[n_rows];
 * every tile rank r <= rp (a bin row with r > rp is left untouched). */
int fh_project_y_f32(const fh_tile* tiles, const int32_t* row_tile, int64_t n_rows,
                     const float* U, const float* W, int32_t rp, float* Y, int32_t ldy_l,
                     void* stream);

/* ---- Procrustes step per bin row (parafac2_intergrative.py:336,374-417,422-423;
 * project2orthogonal.py:6-34), fp32.  For bin row g of tile t (local row i):
 *   M = D_c diag(A_g) B_c^T (R x r); temp = W_g M (n x r);
 *   U_g = polar(temp) by Householder QR + scaled Newton / Newton-Schulz on R,
 *   ssum[g] = sum of the singular values of temp,
 *   Gt[xoff + i*n + j][m] = sum_l U_g[j][l] M[m][l]  (the rows of lhs2 U^T).
 * A: float[n_rows][lda]; B: float[nchrom][ldb][ldb]; D: float[nchrom][rp][ldb] (rows >= R
 * zero); U: tile-major (rows x width x rank at tile.uoff).  r <= rp, width <= 320, width >= r.
 * rp <= 64: two CTAs per SM.  rp = 128 (r <= 128): one CTA per SM with two regions of
 * max(width, 128) rows of r + 1 floats (2 x max(width, 128) x (r + 1) x 4 + 12 KB <= 227 KB,
 * so width <= 217 at r = 128); the CTA parks M in the bin row's own Gt rows and the factored
 * temp in its own U rows while it iterates, then overwrites both (FH_ERR_UNSUPPORTED beyond). */
int fh_procrustes_f32(const fh_tile* tiles, const int32_t* row_tile, int64_t n_rows,
                      int32_t max_width, int32_t max_rank, const float* W, const float* A,
                      int32_t lda, const float* B, const float* D, int32_t ldb, int32_t R,
                      int32_t rp, float* U, float* Gt, double* ssum, int* status, void* stream);

/* Gt rows from stored projections, no polar step: Gt[xoff + i*n + j][m] = sum_l U_g[j][l]
 * M[m][l] with M = D_c diag(A_g) B_c^T (transform, parafac2_intergrative.py:772-801). */
int fh_projection_g_f32(const fh_tile* tiles, const int32_t* row_tile, int64_t n_rows,
                        int32_t max_width, int32_t max_rank, const float* A, int32_t lda,
                        const float* B, const float* D, int32_t ldb, int32_t R, int32_t rp,
                        const float* U, float* Gt, void* stream);

/* ---- Fused per-cell reconstruction loss and its backward pass (no reference counterpart;
 * the loss is the reference's reconstruction error, parafac2_intergrative.py:336-383,
 * 667-713, split by cell).  With Gt from fh_projection_g_f32 (Gt_g = U_g B diag(A_g) D^T),
 *   L_c = sum_rows (X[c][row] - sum_m E[c][m] Gt[row][m])^2,   rows < `rows`, c < n_cells,
 * the residual formed in shared memory and never stored.  X: float[n_cells][ldx] (ldx a
 * multiple of 64; entries past `rows` are ignored), Gt: float[rows][rp], E: float[n_cells]
 * [rp], rp in {16, 32, 64}.  ws: fh_recon_workspace bytes of device memory.
 * fh_recon_loss_f32: loss = double[n_cells].
 * fh_recon_loss_bwd_f32, for w = dOut/dL (double[n_cells]) and Xp = dX/drp
 * (fh_rwr_grad_f32; same layout as X):
 *   dE[c] = -2 w_c sum_rows Res[c] Gt,   dGt[row] = -2 sum_c w_c Res[c][row] E[c],
 *   *drp = 2 sum_c w_c <Res[c], Xp[c]>,  and loss (optional) as above. */
size_t fh_recon_workspace(int32_t n_cells, int64_t rows, int32_t rp);
int fh_recon_loss_f32(const float* X, int64_t ldx, int32_t n_cells, int64_t rows,
                      const float* Gt, const float* E, int32_t rp, double* loss, void* ws,
                      size_t ws_bytes, void* stream);
int fh_recon_loss_bwd_f32(const float* X, const float* Xp, int64_t ldx, int32_t n_cells,
                          int64_t rows, const float* Gt, const float* E, int32_t rp,
                          const double* w, double* loss, float* dE, float* dGt, double* drp,
                          void* ws, size_t ws_bytes, void* stream);

/* Factor gradients from H_g = U_g^T dGt_g (fh_project_y_f32 applied to dGt; H: float[n_rows]
 * [ldh][rp]), for Gt_g = U_g B_c diag(A_g) D_c^T:
 *   dA[g][p] = sum_l B_c[l][p] (H_g D_c)[l][p],   dB_c = sum_g (H_g D_c) diag(A_g),
 *   dD_c = sum_g H_g^T B_c diag(A_g).
 * meta: the chunk table of fh_cp_als; A, dA: float[n_rows][ld]; B, dB: float[nchrom][ld][ld];
 * D, dD: float[nchrom][rp][ld]; ld, rp <= 64.  ws: fh_factor_grad_workspace bytes. */
size_t fh_factor_grad_workspace(int32_t nchunks, int32_t ld, int32_t rp);
int fh_factor_grad_f32(int32_t nchrom, int32_t nchunks, const int32_t* meta, const float* H,
                       int32_t ldh, const float* A, const float* B, const float* D, int32_t ld,
                       int32_t rp, int32_t R, float* dA, float* dB, float* dD, void* ws,
                       size_t ws_bytes, void* stream);

/* project2orthogonal drop-in (project2orthogonal.py:6-34) for a batch of tall matrices:
 * M: float[batch][n][r] (n >= r, r <= 128, fh_polar_smem(n, r) <= 227 KB) -> U: float[batch]
 * [n][r] polar factor (Householder QR + Newton), ssum (optional): double[batch] the sums of
 * the singular values. */
size_t fh_polar_smem(int32_t n, int32_t r);
int fh_polar_f32(const float* M, int64_t batch, int32_t n, int32_t r, float* U, double* ssum,
                 int* status, void* stream);

/* Singular values (descending) of tall matrices M (any n) given their polar factors U: the
 * one-sided Jacobi of the symmetric U^T M (accumulated in fp64). */
int fh_polar_svals_f32(const float* M, const float* U, int64_t batch, int32_t n, int32_t r,
                       float* S, void* stream);

/* ---- meta polar (parafac2_intergrative.py:483-486): E = polar(S), S = SVD_term^T
 * (float[n_cells][rp], R columns used, R <= 128); *ssum = sum of singular values = <E, S>.
 * fp64 Gram, fp64 Cholesky, Newton polar of the factor, fp64 apply. */
size_t fh_meta_polar_workspace(int32_t n_cells, int32_t R);
int fh_meta_polar(const float* S, int32_t n_cells, int32_t R, int32_t rp, float* E,
                  double* ssum, void* workspace, size_t workspace_bytes, int* status,
                  void* stream);

/* ---- CP-ALS on every chromosome's projected tensor (parafac_integrative.py:28-112 with
 * n_iter_max = n_iter; parafac2_intergrative.py:674-706).  A: float[bin rows][ld],
 * B: float[nchrom][ld][ld], D: float[nchrom][rp][ld], Y: float[bin rows][ldy][rp]; the
 * factors are updated in place.  meta (device int32): c_row0, c_nbin, c_rank, c_chunk0,
 * c_nchunk (nchrom each) then k_chrom, k_row0, k_nrow (nchunks each): bin-row chunks of at
 * most 8 rows, each inside one chromosome.  core: double[nchrom] = ||[[A,B,D]]||^2 after
 * the sweeps; cross (optional): double[nchrom] = <[[A,B,D]], Y> of the last sweep
 * (parafac's loss_norm and loss_x).  Requires r <= ld <= 128, R <= rp <= ld (ld > 64 runs
 * the 512-thread instantiation). */
size_t fh_cp_workspace(int32_t nchrom, int32_t nchunks, int32_t ld, int32_t rp);
int fh_cp_als(int32_t nchrom, int32_t nchunks, const int32_t* meta, float* A, float* B,
              float* D, const float* Y, int32_t ld, int32_t rp, int32_t R, int32_t ldy,
              int32_t n_iter, double* core, double* cross, void* workspace,
              size_t workspace_bytes, int* status, void* stream);
/* core[chrom] = ||[[A,B,D]]||^2 of the current factors, which stay unchanged
 * (parafac2_intergrative.py:621-632). */
int fh_core_norm(int32_t nchrom, int32_t nchunks, const int32_t* meta, float* A, float* B,
                 float* D, const float* Y, int32_t ld, int32_t rp, int32_t R, int32_t ldy,
                 double* core, void* workspace, size_t workspace_bytes, int* status,
                 void* stream);

/* ---- input packing of one chromosome (FastHigashi.pack_training_data_one_process,
 * fasthigashi/FastHigashi_Wrapper.py:221-366 with preprocessing.py:114-193, 474-489; no
 * blacklist, no batch ids).  Raw cell c's contacts are row/col/val[cell_off[c] ..
 * cell_off[c + 1]) (device; coordinates in [0, nbin), values non-negative), n_raw cells;
 * output cell k takes raw cell reorder[k] (n_cells entries).  Coordinates are divided by merge,
 * contacts with |col - row| > off_diag dropped, merged bin rows with no positive kept contact
 * removed and the rest renumbered, each cell scaled so that its kept contacts sum to
 * ceil(nbin / merge), then log1p and a clip at mean + 15 std of all values.  Output, in the
 * reference's order (cell by cell, each cell's entries in input order): out_idx int32[3][cap]
 * (row, col, cell), out_val float32[cap], cap >= the input's contacts (the work is cut into
 * segments of at most 4,096 contacts sized by cap); out_counts int64[2] (device) = { entries
 * written, kept bins }.  Workspace size from fh_pack_workspace (the same cap).  status:
 * FH_ERR_INDEX for a coordinate or reorder entry out of range, or more contacts than cap. */
size_t fh_pack_workspace(int32_t n_cells, int32_t nbin, int32_t merge, int64_t cap);
int fh_pack_chromosome(const int32_t* row, const int32_t* col, const float* val,
                       const int64_t* cell_off, int32_t n_raw, const int32_t* reorder,
                       int32_t n_cells, int32_t nbin, int32_t merge, int32_t off_diag,
                       int32_t* out_idx, float* out_val, int64_t cap, int64_t* out_counts,
                       void* workspace, size_t workspace_bytes, int* status, void* stream);

/* ---- embedding post-processing (FastHigashi.fetch_cell_embedding / correct_batch_linear,
 * fasthigashi/FastHigashi_Wrapper.py:750-878).  All buffers are device memory.
 * fh_embed_assemble:  Y[c][j] = sum_l E[c][l] D[l][j] / ||D[:, j]|| (:753-758): D is every
 *                     chromosome's D (R x r_i) side by side (R x m, row stride ldd);
 *                     inv_norm: float[m] scratch (receives 1 / ||D[:, j]||).
 * fh_gemm_scale_f32:  out[i][j] = scale[j] * sum_l A[i][l] B[l][j] (scale optional).
 * fh_quantile_uniform: the quantile transform of one column (:763, n_quantiles = 100 there)
 *                     to [0, 1], fp64 in and out.
 * fh_lstsq_residual:  out = Y minus its least-squares fit on V (double[n_cells][p]) with an
 *                     intercept, the minimum-norm coefficients (:861-866); the intercept is
 *                     added back when add_intercept_back != 0.  p <= 256.
 * fh_range_svd:       out[c][j] = U[c][j] s_j for the top k singular triplets of Y (n_cells x
 *                     m) whose columns lie in the column space of F (n_cells x r, r <= 256):
 *                     the truncated SVD of :767-768 and :870-871 (TruncatedSVD.fit_transform,
 *                     component signs by its rule: each component's largest-magnitude entry
 *                     positive); sigma (optional): double[k].
 * fh_l2_rows:         rows scaled to unit Euclidean norm, zero rows unchanged (:778, :873).
 * fh_cross_f32:       out[i][j] = sum_c A[c][i] B[c][j] in fp64 (A: n_rows x na, B: n_rows x
 *                     nb), fixed order; init_params' sketch products use it too.
 * status (fh_lstsq_residual, fh_range_svd): FH_ERR_ILLCOND if an fp64 Jacobi eigen-solve did
 * not converge. */
int fh_embed_assemble(const float* E, int32_t n_cells, int32_t R, int64_t lde, const float* D,
                      int32_t m, int64_t ldd, float* inv_norm, float* Y, int64_t ldy,
                      void* stream);
int fh_gemm_scale_f32(const float* A, int64_t lda, const float* B, int64_t ldb,
                      const float* scale, int32_t n, int32_t m, int32_t K, float* out,
                      int64_t ldo, void* stream);
size_t fh_quantile_workspace(int32_t n, int32_t n_quantiles);
int fh_quantile_uniform(const double* x, int32_t n, int32_t n_quantiles, double* out,
                        void* workspace, size_t workspace_bytes, void* stream);
size_t fh_lstsq_workspace(int32_t p, int32_t m);
int fh_lstsq_residual(const double* V, int32_t n_cells, int32_t p, const float* Y, int64_t ldy,
                      int32_t m, int32_t add_intercept_back, float* out, int64_t ldo,
                      void* workspace, size_t workspace_bytes, int* status, void* stream);
size_t fh_range_svd_workspace(int32_t r, int32_t m, int32_t k);
int fh_range_svd(const float* F, int64_t ldf, int32_t n_cells, int32_t r, const float* Y,
                 int64_t ldy, int32_t m, int32_t k, float* out, int64_t ldo, double* sigma,
                 void* workspace, size_t workspace_bytes, int* status, void* stream);
int fh_l2_rows(const float* X, int64_t ldx, int32_t n, int32_t m, float* out, int64_t ldo,
               void* stream);
int fh_cross_f32(const float* A, int64_t lda, int32_t na, const float* B, int64_t ldb,
                 int32_t nb, int32_t n_rows, double* out, int64_t ldo, void* stream);

/* ---- imputed contact maps (FastHigashi.only_partial_rwr, FastHigashi_Wrapper.py:569-655):
 * out[c][i][j] (float[ncell][nbin][nbin]) = M[i][j] + M[j][i] for i != j and M[i][i] on the
 * diagonal, M[i][j] = the walk output X[cell0 + c] of the tile holding row i at compact
 * column j - shift (0 outside its columns).  row_tile[row_base + i]: the tile of the
 * chromosome's row i (tiles as the fit's table); X: float[cells][ldx] in the compact band
 * layout.  status: FH_ERR_INDEX when row_tile names a tile without row i. */
int fh_impute_maps(const fh_tile* tiles, const int32_t* row_tile, int64_t row_base,
                   int32_t nbin, const float* X, int64_t ldx, int32_t cell0, int32_t ncell,
                   float* out, int* status, void* stream);

/* ---- the 1 Mb pooling of init_params' features (parafac2_intergrative.py:102-151): for the
 * n_tiles consecutive tiles at tiles (one chromosome's datasets), block (py, px) of tile t is
 * pooled row prow0[t] + py * (width_t / ll_t) + px (prow0: int64[n_tiles + 1]), the mean of
 * band rows xoff_t + (py ll + dy) width_t + px ll + dx (dy, dx < ll_t); rows are counted from
 * band row x0.  fh_pool_rows: out (pooled rows x m) = Pm^T in (band rows x m);
 * fh_unpool_rows: out (rows x m) = Pm in (pooled rows x m), zero on the cropped remainders. */
int fh_pool_rows(const fh_tile* tiles, int32_t n_tiles, const int64_t* prow0,
                 const int32_t* ll, int64_t x0, const float* in, int64_t ldi, int32_t m,
                 float* out, int64_t ldo, void* stream);
int fh_unpool_rows(const fh_tile* tiles, int32_t n_tiles, const int64_t* prow0,
                   const int32_t* ll, int64_t x0, int64_t rows, const float* in, int64_t ldi,
                   int32_t m, float* out, int64_t ldo, void* stream);

/* ---- host memory for X held partly outside HBM (no reference counterpart: the reference
 * tiles its work by free GPU memory instead, FastHigashi_Wrapper.py:497-517, and copies each
 * tile's COO slice to the device, sparse_for_schic.py:588-613).
 * fh_host_alloc: page-locked host memory, mapped into the device address space (cudaHostAlloc,
 *   portable | mapped); fh_host_free releases it.
 * fh_memcpy_async: one asynchronous copy of bytes between any two of host and device memory on
 *   stream (a memcpy node when the stream is being captured into a CUDA graph); the streamed
 *   windows of X and the chunks of a chromosome's COO for the contact build move by it. */
int fh_host_alloc(int64_t bytes, void** out);
int fh_host_free(void* p);
int fh_memcpy_async(void* dst, const void* src, int64_t bytes, void* stream);

/* ---- self-test of the bounded device-side waits (no reference counterpart: the reference
 * has no device code).  One warp allocates tensor memory, waits on an mbarrier that nothing
 * arrives on until limit_ns of device time pass, sets *status = FH_ERR_TIMEOUT, frees the
 * tensor memory and returns: the path every tcgen05 kernel here takes when a wait runs out.
 * limit_ns in (0, 1e9]; status: int32 device word (cleared by the caller). */
int fh_selftest_wait(int* status, int64_t limit_ns, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* FHGB300_H */
