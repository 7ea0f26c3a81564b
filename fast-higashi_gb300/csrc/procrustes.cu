// Per-bin-row Procrustes step (fp32): polar factor of temp_i by Householder QR + Newton.
//
// Reference: project2orthogonal.py:6-34 (U Vh of the thin SVD and S) applied per bin row to
// temp_i = X_i lhs_i (parafac2_intergrative.py:374-417), with lhs2 of :422-423.
//
// temp = W_g M, M = D_c diag(A_g) B_c^T (n x r), W_g = X_g E the bin row's band rows of the
// X^T E pass.  temp = Q R (Householder), polar(temp) = Q polar(R), polar(R) by scaled
// Newton finished by Newton-Schulz (polar_common.cuh), sum(S) = trace(polar(R)^T R).
// Against an fp64 SVD of the reference's own temp matrices (condition numbers up to 5e6)
// this fp32 route errs by a median 5.1e-6 (max 4.7e-4), the same class as the reference's
// fp32 SVD (median 4.4e-6, max 1.2e-3); a Gram-matrix route squares the condition number
// and fails in fp32, and one-sided Jacobi needs 12+ sweeps on these matrices.
//
// The same CTA then writes U_g and the rows Gt[j][m] = sum_l U_g[j][l] M[m][l] (lhs2 U^T)
// that the X G^T pass consumes.
#include "polar_common.cuh"

namespace fh {

constexpr int kProcThreads = 512;

struct ProcArgs {
  const fh_tile* tiles;
  const int32_t* row_tile;
  const float* W;    // [band rows][RP]
  const float* A;    // [bin rows][lda]
  int lda;
  const float* B;    // [chrom][ldb][ldb]
  int ldb;
  const float* D;    // [chrom][RP][ldb]
  int R;
  float* U;          // tile-major projections
  float* Gt;         // [band rows][RP]
  double* ssum;      // [bin rows]
  int* status;
  int mode;          // 0 fit step, 1 Gt from the stored U (transform)
};

__host__ __device__ inline size_t proc_region_floats(int n, int r, int rp) {
  const int ldt = r + 1;
  size_t region = (size_t)n * ldt;                                  // U
  const size_t newton = (size_t)r * ldt + newton_scratch_floats(r); // X + scratch
  if (newton > region) region = newton;
  const size_t stage = (size_t)rp * ldt + (size_t)r * ldt;          // D diag(A), B
  if (stage > region) region = stage;
  return region;
}

__host__ __device__ inline size_t proc_smem_floats(int n, int r, int rp) {
  const int ldt = r + 1;
  return (size_t)rp * ldt + (size_t)n * ldt + proc_region_floats(n, r, rp) + kPolarMiscFloats;
}

template <int RP>
__global__ void __launch_bounds__(kProcThreads) procrustes_qr_kernel(ProcArgs a) {
  extern __shared__ __align__(16) float sm[];
  __shared__ float red[32];
  __shared__ double dred[32];
  __shared__ int ival[4];
  const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5, nw = kProcThreads / 32;
  const int64_t g = blockIdx.x;
  const fh_tile T = a.tiles[a.row_tile[g]];
  const int i0 = (int)(g - T.brow0);
  const int n = T.width, r = T.rank, ci = T.chrom, R = a.R;
  const int ldt = r + 1;
  float* Ms = sm;                        // RP x ldt: M[m][l]
  float* Tm = Ms + (size_t)RP * ldt;     // n x ldt: temp, then R and the reflectors
  float* reg = Tm + (size_t)n * ldt;     // reused region
  float* misc = reg + proc_region_floats(n, r, RP);
  PolarScratch s{misc, misc + kMaxRank, misc + 2 * kMaxRank, misc + 4 * kMaxRank, red, dred,
                 ival};
  if (tid == 0) ival[0] = 0;
  // ---- M[m][l] = sum_rho D[m][rho] A_g[rho] B[l][rho]
  {
    float* DA = reg;
    float* Bs = reg + (size_t)RP * ldt;
    const float* Ag = a.A + g * a.lda;
    const float* Dc = a.D + (size_t)ci * RP * a.ldb;
    const float* Bc = a.B + (size_t)ci * a.ldb * a.ldb;
    for (int m = ty; m < RP; m += nw)
      for (int rho = tx; rho < r; rho += 32)
        DA[m * ldt + rho] = m < R ? Dc[m * a.ldb + rho] * Ag[rho] : 0.f;
    for (int l = ty; l < r; l += nw)
      for (int rho = tx; rho < r; rho += 32) Bs[l * ldt + rho] = Bc[l * a.ldb + rho];
    __syncthreads();
    for (int m = ty; m < RP; m += nw)
      for (int l = tx; l < r; l += 32) {
        float acc = 0.f;
        for (int rho = 0; rho < r; ++rho) acc = fmaf(DA[m * ldt + rho], Bs[l * ldt + rho], acc);
        Ms[m * ldt + l] = acc;
      }
    __syncthreads();
  }
  const int64_t brow = T.xoff + (int64_t)i0 * n;
  float* Gg = a.Gt + brow * RP;
  if (a.mode == 1) {
    // transform: Gt_g = U_g M^T with the stored projection (parafac2_intergrative.py:772-801)
    const float* Ug = a.U + T.uoff + (int64_t)i0 * n * r;
    for (int i = ty; i < n; i += nw)
      for (int m = tx; m < RP; m += 32) {
        float acc = 0.f;
        for (int l = 0; l < r; ++l) acc = fmaf(__ldg(Ug + (int64_t)i * r + l), Ms[m * ldt + l], acc);
        Gg[(int64_t)i * RP + m] = acc;
      }
    return;
  }
  // ---- temp[i][l] = sum_m W_g[i][m] M[m][l]
  {
    const float* Wg = a.W + brow * RP;
    for (int i = ty; i < n; i += nw) {
      const float* wr = Wg + (int64_t)i * RP;
      for (int l = tx; l < r; l += 32) {
        float acc = 0.f;
#pragma unroll 8
        for (int m = 0; m < RP; ++m) acc = fmaf(__ldg(wr + m), Ms[m * ldt + l], acc);
        Tm[i * ldt + l] = acc;
      }
    }
    __syncthreads();
  }
  // ---- QR, polar factor of R, sum(S)
  householder_qr(Tm, n, r, ldt, s);
  float* X = reg;
  for (int p = ty; p < r; p += nw)
    for (int q = tx; q < r; q += 32) X[p * ldt + q] = q >= p ? Tm[p * ldt + q] : 0.f;
  __syncthreads();
  newton_polar(X, ldt, reg + (size_t)r * ldt, r, true, s);
  {
    double acc = 0.0;
    for (int p = ty; p < r; p += nw)
      for (int q = p + tx; q < r; q += 32) acc += (double)X[p * ldt + q] * (double)Tm[p * ldt + q];
    acc = block_sum<double>(acc, dred);
    if (tid == 0) a.ssum[g] = acc;
  }
  // ---- U = Q [P; 0]: U's first r rows are X (same storage and stride)
  float* Uu = reg;
  for (int j = r + ty; j < n; j += nw)
    for (int l = tx; l < r; l += 32) Uu[j * ldt + l] = 0.f;
  __syncthreads();
  apply_q(Tm, ldt, Uu, ldt, n, r, s);
  float* Ug = a.U + T.uoff + (int64_t)i0 * n * r;
  for (int j = ty; j < n; j += nw) {
    for (int l = tx; l < r; l += 32) Ug[(int64_t)j * r + l] = Uu[j * ldt + l];
    for (int m = tx; m < RP; m += 32) {
      float acc = 0.f;
      for (int l = 0; l < r; ++l) acc = fmaf(Uu[j * ldt + l], Ms[m * ldt + l], acc);
      Gg[(int64_t)j * RP + m] = acc;
    }
  }
  if (tid == 0 && ival[0]) set_status(a.status, FH_ERR_ILLCOND);
}

// project2orthogonal drop-in: polar factor of each M[b] (n x r, n >= r).
__global__ void __launch_bounds__(kProcThreads) polar_qr_kernel(const float* __restrict__ M, int n,
                                                                int r, float* __restrict__ U,
                                                                double* __restrict__ ssum,
                                                                int* status) {
  extern __shared__ __align__(16) float sm[];
  __shared__ float red[32];
  __shared__ double dred[32];
  __shared__ int ival[4];
  const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5, nw = kProcThreads / 32;
  const int64_t b = blockIdx.x;
  const int ldt = r + 1;
  float* Tm = sm;
  float* reg = Tm + (size_t)n * ldt;
  size_t regsz = (size_t)n * ldt;
  const size_t newton = (size_t)r * ldt + newton_scratch_floats(r);
  if (newton > regsz) regsz = newton;
  float* misc = reg + regsz;
  PolarScratch s{misc, misc + kMaxRank, misc + 2 * kMaxRank, misc + 4 * kMaxRank, red, dred,
                 ival};
  if (tid == 0) ival[0] = 0;
  const float* Mb = M + b * (int64_t)n * r;
  for (int i = ty; i < n; i += nw)
    for (int l = tx; l < r; l += 32) Tm[i * ldt + l] = Mb[(int64_t)i * r + l];
  __syncthreads();
  householder_qr(Tm, n, r, ldt, s);
  float* X = reg;
  for (int p = ty; p < r; p += nw)
    for (int q = tx; q < r; q += 32) X[p * ldt + q] = q >= p ? Tm[p * ldt + q] : 0.f;
  __syncthreads();
  newton_polar(X, ldt, reg + (size_t)r * ldt, r, true, s);
  double acc = 0.0;
  for (int p = ty; p < r; p += nw)
    for (int q = p + tx; q < r; q += 32) acc += (double)X[p * ldt + q] * (double)Tm[p * ldt + q];
  acc = block_sum<double>(acc, dred);
  if (tid == 0 && ssum) ssum[b] = acc;
  for (int j = r + ty; j < n; j += nw)
    for (int l = tx; l < r; l += 32) reg[j * ldt + l] = 0.f;
  __syncthreads();
  apply_q(Tm, ldt, reg, ldt, n, r, s);
  float* Ub = U + b * (int64_t)n * r;
  for (int j = ty; j < n; j += nw)
    for (int l = tx; l < r; l += 32) Ub[(int64_t)j * r + l] = reg[j * ldt + l];
  if (tid == 0 && ival[0]) set_status(status, FH_ERR_ILLCOND);
}

}  // namespace fh

using namespace fh;

static int proc_launch(const ProcArgs& a, int64_t n_rows, int max_width, int max_rank, int rp,
                       cudaStream_t s) {
  if (max_rank > 64 || max_width > kMaxWidth) return FH_ERR_UNSUPPORTED;
  const size_t smem = proc_smem_floats(max_width, max_rank, rp) * sizeof(float);
  if (smem > 227 * 1024) return FH_ERR_UNSUPPORTED;
#define FH_PROC(RPV)                                                                        \
  case RPV: {                                                                               \
    if (ensure_smem((const void*)procrustes_qr_kernel<RPV>, smem)) return FH_ERR_LAUNCH;    \
    procrustes_qr_kernel<RPV><<<(unsigned)n_rows, kProcThreads, smem, s>>>(a);              \
    break;                                                                                  \
  }
  switch (rp) {
    FH_PROC(16)
    FH_PROC(32)
    FH_PROC(64)
    default: return FH_ERR_UNSUPPORTED;
  }
#undef FH_PROC
  FH_CHECK_LAUNCH();
  return FH_OK;
}

extern "C" int fh_procrustes_f32(const fh_tile* tiles, const int32_t* row_tile, int64_t n_rows,
                                 int32_t max_width, int32_t max_rank, const float* W,
                                 const float* A, int32_t lda, const float* B, const float* D,
                                 int32_t ldb, int32_t R, int32_t rp, float* U, float* Gt,
                                 double* ssum, int* status, void* stream) {
  if (!tiles || !row_tile || !W || !A || !B || !D || !U || !Gt || !ssum || n_rows <= 0 ||
      R > rp || max_rank > ldb || max_rank > lda)
    return FH_ERR_ARG;
  ProcArgs a{tiles, row_tile, W, A, lda, B, ldb, D, R, U, Gt, ssum, status, 0};
  return proc_launch(a, n_rows, max_width, max_rank, rp, (cudaStream_t)stream);
}

extern "C" int fh_projection_g_f32(const fh_tile* tiles, const int32_t* row_tile, int64_t n_rows,
                                   int32_t max_width, int32_t max_rank, const float* A,
                                   int32_t lda, const float* B, const float* D, int32_t ldb,
                                   int32_t R, int32_t rp, const float* U, float* Gt,
                                   void* stream) {
  if (!tiles || !row_tile || !A || !B || !D || !U || !Gt || n_rows <= 0 || R > rp)
    return FH_ERR_ARG;
  ProcArgs a{tiles, row_tile, nullptr, A, lda, B, ldb, D, R, const_cast<float*>(U), Gt,
             nullptr, nullptr, 1};
  return proc_launch(a, n_rows, max_width, max_rank, rp, (cudaStream_t)stream);
}

extern "C" size_t fh_polar_smem(int32_t n, int32_t r) {
  const size_t ldt = (size_t)r + 1;
  size_t regsz = (size_t)n * ldt;
  const size_t newton = (size_t)r * ldt + newton_scratch_floats(r);
  if (newton > regsz) regsz = newton;
  return ((size_t)n * ldt + regsz + kPolarMiscFloats) * sizeof(float);
}

extern "C" int fh_polar_f32(const float* M, int64_t batch, int32_t n, int32_t r, float* U,
                            double* ssum, int* status, void* stream) {
  if (!M || !U || batch <= 0 || n < r || r <= 0) return FH_ERR_ARG;
  if (r > kMaxRank) return FH_ERR_UNSUPPORTED;
  const size_t smem = fh_polar_smem(n, r);
  if (smem > 227 * 1024) return FH_ERR_UNSUPPORTED;
  if (ensure_smem((const void*)polar_qr_kernel, smem)) return FH_ERR_LAUNCH;
  polar_qr_kernel<<<(unsigned)batch, kProcThreads, smem, (cudaStream_t)stream>>>(M, n, r, U, ssum,
                                                                                status);
  FH_CHECK_LAUNCH();
  return FH_OK;
}
