// Partial RWR with column normalisation (do_col=True, fasthigashi/partial_rwr.py:112-138):
//   Q_0 = I,  Q_{t+1} = rp Q_t P + (1 - rp) I            (t < n_rwr; :112-126)
//   Q' = (Q + Q^T) / 2, clipped at 0, each row divided by (its sum + 1e-15)      (:131-134)
//   X  = Q' (A / bin_cov)                                                           (:135-138)
// with bin_cov[c][g] the cell's coverage of global column g (init_params, parafac2_
// intergrative.py:96-276).  The other walks never form Q (Z_t = Q_t A is iterated instead);
// this one must, for the symmetrisation: P^T, Q and the tile A stay in shared memory (for
// b = 125 rows and n <= 185 columns that is 226 KB).  A is the floored densified tile from
// the (tile, cell) segment, or a dense tile (the 3 x 3 mean of do_conv) in the X layout.
// One CTA of 256 threads per (tile, cell), or per cell of one dense tile shape (drop-in).
//
// Without coverage rows the same kernel runs the plain walk X = Q A in the reference's own
// association (Q first, then one product), which init_params uses for the coverage itself:
// per (tile, cell) epoch counts (the auto-stop rule is decided per cell batch, :99-126) and
// per (tile, cell) column sums of X (b_c = X.sum(1), parafac2_intergrative.py:141), which
// col_coverage_kernel then adds into the coverage rows in bin-batch order (:142, :200).
#include <cuda_bf16.h>
#include "rwr_common.cuh"

namespace fh {

struct ColArgs {
  const fh_tile* tiles;      // null: one dense tile shape (the partial_rwr drop-in)
  int n_cells;
  const uint2* entries;
  const int64_t* offsets;
  const float* dense;        // dense A: X layout (tiles) or [cell][rows][width]
  int d_rows, d_width, d_s0, d_epochs;
  const float* cov;          // coverage rows: cov[c * cov_ld + global column]; null: plain walk
  int64_t cov_ld;
  const int32_t* cell_epochs;  // [tile][cell] epoch counts overriding the tile's, or null
  float* colsum;             // [tile][cell][max_width] column sums of X, or null
  int max_rows, max_width;
  float rp;
  float* out;                // fp32 output (X layout or [cell][rows][width]), or null
  __nv_bfloat16* out16;      // bf16 planes (X layout), or null
  int64_t cell_stride, plane_stride;
  double* sumsq;
  int* status;
};

__host__ __device__ inline size_t col_smem_bytes(int b, int n) {
  return (size_t)(2 * b * rwr_ldp(b) + b * lds_stride_odd(n) + 3 * kMaxBinRows) * sizeof(float);
}

template <int MAXU>
__global__ void __launch_bounds__(kRwrThreads, 1) rwr_col_kernel(ColArgs a) {
  extern __shared__ __align__(16) float smem[];
  __shared__ double dred[32];
  const int c = blockIdx.x, t = blockIdx.y;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  int b, n, s0, epochs;
  int64_t xoff = 0, gcol0 = 0;
  if (a.tiles) {
    const fh_tile T = a.tiles[t];
    b = T.rows; n = T.width; s0 = T.s0; xoff = T.xoff;
    epochs = a.cell_epochs ? a.cell_epochs[(int64_t)t * a.n_cells + c] : T.n_rwr;
    gcol0 = (T.brow0 - T.row0) + T.shift;   // global column of tile column 0
    if (b <= 0 || b > a.max_rows || n < b || n > a.max_width || s0 < 0 || s0 + b > n ||
        epochs < 0) {
      if (tid == 0) set_status(a.status, FH_ERR_ARG);
      return;
    }
  } else {
    b = a.d_rows; n = a.d_width; s0 = a.d_s0; epochs = a.d_epochs;
  }
  const int ldp = rwr_ldp(b), lda = lds_stride_odd(n);
  float* Pt = smem;               // b x ldp: P^T, then Q'^T
  float* Qm = Pt + b * ldp;       // b x ldp: Q_t
  float* Am = Qm + b * ldp;       // b x lda: A, A / bin_cov, then X
  float* cs1 = Am + b * lda;
  float* cs2 = cs1 + kMaxBinRows;
  float* csl = cs2 + kMaxBinRows;

  // ---- A
  if (a.dense) {
    const float* x = a.tiles ? a.dense + (int64_t)c * a.cell_stride + xoff
                             : a.dense + (int64_t)c * b * n;
    for (int i = tid; i < b * n; i += kRwrThreads) Am[(i / n) * lda + i % n] = x[i];
  } else {
    const int64_t e0 = a.offsets[(int64_t)t * a.n_cells + c];
    const int64_t e1 = a.offsets[(int64_t)t * a.n_cells + c + 1];
    for (int i = tid; i < b * lda; i += kRwrThreads) Am[i] = 0.f;
    __syncthreads();
    for (int64_t e = e0 + tid; e < e1; e += kRwrThreads) {
      const uint2 en = a.entries[e];
      const int r = (int)(en.x & 0xffffu), j = (int)(en.x >> 16);
      if (r < b && j < n) Am[r * lda + j] = __uint_as_float(en.y);
      else set_status(a.status, FH_ERR_INDEX);
    }
    __syncthreads();
    for (int i = tid; i < b * n; i += kRwrThreads) {
      float* z = Am + (i / n) * lda + (i % n);
      *z = fmaxf(*z, kFloor);
    }
  }
  __syncthreads();
  rwr_transition(Am, lda, Pt, ldp, b, n, s0, cs1, cs2, csl);

  // ---- Q_T from Q_0 = I (P Q_t = Q_t P: Q_t is a polynomial in P)
  for (int i = tid; i < b * ldp; i += kRwrThreads) Qm[i] = (i / ldp == i % ldp) ? 1.f : 0.f;
  __syncthreads();
  const float om = a.rp, al = 1.f - a.rp;
  for (int ep = 0; ep < epochs; ++ep) {
    float acc[8][8];
    pz_product<8>(Qm, ldp, Pt, ldp, b, ty, tx, acc);   // (P Q)[tx + 16v][ty + 16u]
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
      for (int v = 0; v < 8; ++v) {
        const int i = ty + 16 * u, j = tx + 16 * v;     // column i, row j of Q
        if (i < b && j < b) Qm[j * ldp + i] = fmaf(om, acc[u][v], i == j ? al : 0.f);
      }
    __syncthreads();
  }
  if (a.cov) {
    // ---- Q' = rownorm(max((Q + Q^T) / 2, 0)) stored transposed in Pt (P is no longer needed)
    if (tid < b) {
      float s = 0.f;
      for (int k = 0; k < b; ++k) s += fmaxf((Qm[tid * ldp + k] + Qm[k * ldp + tid]) * 0.5f, 0.f);
      cs1[tid] = s;
    }
    __syncthreads();
    for (int idx = tid; idx < b * b; idx += kRwrThreads) {
      const int i = idx / b, k = idx % b;
      const float v = fmaxf((Qm[i * ldp + k] + Qm[k * ldp + i]) * 0.5f, 0.f);
      Pt[k * ldp + i] = v / (cs1[i] + kEps);
    }
    // ---- A / bin_cov (the cell's coverage of each column)
    const float* cv = a.cov + (int64_t)c * a.cov_ld + gcol0;
    for (int i = tid; i < b * n; i += kRwrThreads) Am[(i / n) * lda + i % n] /= cv[i % n];
  } else {
    for (int idx = tid; idx < b * b; idx += kRwrThreads) {
      const int i = idx / b, k = idx % b;
      Pt[k * ldp + i] = Qm[i * ldp + k];
    }
  }
  __syncthreads();
  // ---- X = Q' (A / bin_cov) (or Q A), staged back into Am
  {
    float acc[MAXU][8];
    pz_product<MAXU>(Am, lda, Pt, ldp, b, ty, tx, acc);   // (Q' A)[tx + 16v][ty + 16u]
    __syncthreads();
#pragma unroll
    for (int u = 0; u < MAXU; ++u)
#pragma unroll
      for (int v = 0; v < 8; ++v) {
        const int i = ty + 16 * u, j = tx + 16 * v;     // column i, row j
        if (i < n && j < b) Am[j * lda + i] = acc[u][v];
      }
    __syncthreads();
  }
  // ---- output
  if (a.colsum) {
    float* cs = a.colsum + ((int64_t)t * a.n_cells + c) * a.max_width;
    for (int j = tid; j < n; j += kRwrThreads) {
      float s = 0.f;
      for (int i = 0; i < b; ++i) s += Am[i * lda + j];
      cs[j] = s;
    }
  }
  if (!a.out && !a.out16) return;
  double ss = 0.0;
  for (int i = tid; i < b * n; i += kRwrThreads) {
    float v = Am[(i / n) * lda + (i % n)];
    if (a.out) {
      const int64_t o = a.tiles ? (int64_t)c * a.cell_stride + xoff + i : (int64_t)c * b * n + i;
      a.out[o] = v;
    } else {
      const int64_t o = (int64_t)c * a.cell_stride + xoff + i;
      const __nv_bfloat16 h = __float2bfloat16_rn(v);
      a.out16[o] = h;
      if (a.plane_stride > 0) {
        const __nv_bfloat16 l = __float2bfloat16_rn(v - __bfloat162float(h));
        a.out16[a.plane_stride + o] = l;
        v = __bfloat162float(h) + __bfloat162float(l);
      } else {
        v = __bfloat162float(h);
      }
    }
    ss += (double)v * v;
  }
  if (a.sumsq) {
    ss = block_sum<double>(ss, dred);
    if (tid == 0) a.sumsq[(int64_t)t * a.n_cells + c] = ss;
  }
}

// The coverage rows of init_params (parafac2_intergrative.py:96-99, 141-142, 199-200):
// cov[c][g] = 1e-4 + the column sums of every tile holding column g, added in tile order
// (the bin-batch order of the reference's loop).  One CTA per cell.
__global__ void col_coverage_kernel(const fh_tile* __restrict__ tiles, int n_tiles, int n_cells,
                                    const float* __restrict__ colsum, int max_width,
                                    float* __restrict__ cov, int64_t cov_ld, int64_t n_cols,
                                    int* status) {
  const int c = blockIdx.x;
  float* row = cov + (int64_t)c * cov_ld;
  for (int64_t g = threadIdx.x; g < n_cols; g += blockDim.x) row[g] = 1e-4f;
  __syncthreads();
  for (int t = 0; t < n_tiles; ++t) {
    const fh_tile T = tiles[t];
    const int64_t g0 = (T.brow0 - T.row0) + T.shift;
    if (T.width > max_width || g0 < 0 || g0 + T.width > n_cols) {
      if (threadIdx.x == 0) set_status(status, FH_ERR_ARG);
      return;
    }
    const float* cs = colsum + ((int64_t)t * n_cells + c) * max_width;
    for (int j = threadIdx.x; j < T.width; j += blockDim.x) row[g0 + j] += cs[j];
    __syncthreads();   // the next tile's overlapping columns may belong to other threads
  }
}

// bin_cov[bin_cov <= 1e-4] = inf (parafac2_intergrative.py:266-270).
__global__ void col_coverage_finalize_kernel(float* __restrict__ cov, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    if (cov[i] <= 1e-4f) cov[i] = __int_as_float(0x7f800000);
}

static int launch_col(const ColArgs& a, int n_tiles, int mr, int mw, cudaStream_t s) {
  if (mr <= 0 || mr > kMaxBinRows || mw < mr || mw > kMaxWidth) return FH_ERR_UNSUPPORTED;
  const size_t smem = col_smem_bytes(mr, mw);
  if (smem > 227 * 1024) return FH_ERR_UNSUPPORTED;
  dim3 grid((unsigned)a.n_cells, (unsigned)n_tiles);
#define FH_COL(U)                                                              \
  {                                                                            \
    if (ensure_smem((const void*)rwr_col_kernel<U>, smem)) return FH_ERR_LAUNCH; \
    rwr_col_kernel<U><<<grid, kRwrThreads, smem, s>>>(a);                      \
  }
  if (mw <= 128) FH_COL(8)
  else if (mw <= 192) FH_COL(12)
  else if (mw <= 256) FH_COL(16)
  else FH_COL(20)
#undef FH_COL
  FH_CHECK_LAUNCH();
  return FH_OK;
}

}  // namespace fh

using namespace fh;

extern "C" int fh_rwr_col_tiles(const fh_tile* tiles, int32_t n_tiles, int32_t n_cells,
                                int32_t mr, int32_t mw, const fh_entry* entries,
                                const int64_t* offsets, const float* dense, const float* cov,
                                int64_t cov_ld, const int32_t* cell_epochs, float* out,
                                uint16_t* out16, int64_t cell_stride, int64_t plane_stride,
                                double* sumsq, float* colsum, int* status, void* stream) {
  if (!tiles || n_tiles <= 0 || n_cells <= 0 || (cov && cov_ld <= 0) ||
      (!out && !out16 && !colsum) || (!dense && (!entries || !offsets)) || plane_stride < 0)
    return FH_ERR_ARG;
  ColArgs a{};
  a.tiles = tiles; a.n_cells = n_cells; a.entries = reinterpret_cast<const uint2*>(entries);
  a.offsets = offsets; a.dense = dense; a.cov = cov; a.cov_ld = cov_ld;
  a.cell_epochs = cell_epochs; a.colsum = colsum;
  a.max_rows = mr; a.max_width = mw; a.rp = 0.5f;   // partial_rwr.py:109
  a.out = out; a.out16 = out ? nullptr : reinterpret_cast<__nv_bfloat16*>(out16);
  a.cell_stride = cell_stride; a.plane_stride = plane_stride; a.sumsq = sumsq;
  a.status = status;
  return launch_col(a, n_tiles, mr, mw, (cudaStream_t)stream);
}

extern "C" int fh_rwr_col_dense(const float* x, int32_t n_cells, int32_t rows, int32_t width,
                                int32_t s0, int32_t n_epochs, const float* cov, float* out,
                                int* status, void* stream) {
  if (!x || !cov || !out || n_cells <= 0 || rows <= 0 || width < rows || s0 < 0 ||
      s0 + rows > width || n_epochs < 0)
    return FH_ERR_ARG;
  ColArgs a{};
  a.n_cells = n_cells; a.dense = x; a.d_rows = rows; a.d_width = width; a.d_s0 = s0;
  a.d_epochs = n_epochs; a.cov = cov; a.cov_ld = width;
  a.max_rows = rows; a.max_width = width; a.rp = 0.5f;   // partial_rwr.py:109
  a.out = out; a.status = status;
  return launch_col(a, 1, rows, width, (cudaStream_t)stream);
}

extern "C" int fh_col_coverage(const fh_tile* tiles, int32_t n_tiles, int32_t n_cells,
                               const float* colsum, int32_t mw, float* cov, int64_t cov_ld,
                               int64_t n_cols, int* status, void* stream) {
  if (!tiles || n_tiles <= 0 || n_cells <= 0 || !colsum || mw <= 0 || !cov || n_cols <= 0 ||
      cov_ld < n_cols)
    return FH_ERR_ARG;
  col_coverage_kernel<<<n_cells, 256, 0, (cudaStream_t)stream>>>(tiles, n_tiles, n_cells, colsum,
                                                                  mw, cov, cov_ld, n_cols, status);
  FH_CHECK_LAUNCH();
  return FH_OK;
}

extern "C" int fh_col_coverage_finalize(float* cov, int64_t n, void* stream) {
  if (!cov || n <= 0) return FH_ERR_ARG;
  const int64_t blocks = (n + 255) / 256;
  col_coverage_finalize_kernel<<<(unsigned)(blocks < 4 * 152 ? blocks : 4 * 152), 256, 0,
                                 (cudaStream_t)stream>>>(cov, n);
  FH_CHECK_LAUNCH();
  return FH_OK;
}
