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

// Shared memory: two regions of row stride ldt = r + 1 and the polar scratch.
//   region 0 (max(n, RP + r) rows): D diag(A_g) and B staging, then temp -> R and the
//            Householder vectors, then the staging and M again for the Gt product
//   region 1 (max(n, 2 r, RP) rows): M, then the Newton iterate X (rows < r) with its
//            scratch (rows r .. 2r), then U = Q [polar(R); 0]
__host__ __device__ inline int proc_r0_rows(int n, int r, int rp) { return n > rp + r ? n : rp + r; }
__host__ __device__ inline int proc_r1_rows(int n, int r, int rp) {
  // also >= 2 r ldv / ldt + 4 floats: the polar iterate and its scratch at row stride
  // ldv = ((r + 3) & ~3) + 4 <= r + 7, 16-byte aligned
  int m = n > 2 * r + 12 ? n : 2 * r + 12;
  return m > rp ? m : rp;
}
__host__ __device__ inline size_t proc_smem_floats(int n, int r, int rp) {
  return (size_t)(proc_r0_rows(n, r, rp) + proc_r1_rows(n, r, rp)) * (r + 1) + kPolarMiscFloats;
}

// M[m][l] = sum_rho D[m][rho] A_g[rho] B[l][rho] (m < RP, rows m >= R zero) into dst (stride
// ldt); stage: (RP + r) x ldt floats, may overlap dst (the product is held in registers).
// Called by the whole CTA.
template <int RP>
__device__ inline void form_m(const ProcArgs& a, int64_t g, int ci, int r, int ldt, float* stage,
                              float* dst) {
  const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
  float* DA = stage;
  float* Bs = stage + (size_t)RP * ldt;
  const float* Ag = a.A + g * a.lda;
  const float* Dc = a.D + (size_t)ci * RP * a.ldb;
  const float* Bc = a.B + (size_t)ci * a.ldb * a.ldb;
  for (int m = ty; m < RP; m += 16)
    for (int rho = tx; rho < r; rho += 32)
      DA[m * ldt + rho] = m < a.R ? Dc[m * a.ldb + rho] * Ag[rho] : 0.f;
  for (int l = ty; l < r; l += 16)
    for (int rho = tx; rho < r; rho += 32) Bs[l * ldt + rho] = Bc[l * a.ldb + rho];
  __syncthreads();
  constexpr int TM = RP > 64 ? 8 : 4, TN = RP > 64 ? 4 : 2;   // the whole RP x r in registers
  float acc[TM][TN];
  cta_mm<TM, TN>(RP, r, r, 0, [&](int m, int rho) { return DA[m * ldt + rho]; },
                 [&](int rho, int l) { return Bs[l * ldt + rho]; }, acc);
  __syncthreads();
#pragma unroll
  for (int u = 0; u < TM; ++u)
#pragma unroll
    for (int v = 0; v < TN; ++v) {
      const int m = ty + 16 * u, l = tx + 32 * v;
      if (m < RP && l < r) dst[m * ldt + l] = acc[u][v];
    }
  __syncthreads();
}

// Gg[i][m] = sum_l U[i][l] M[m][l] for i < n, m < RP (U read through fu(i, l)).
template <int RP, class FU>
__device__ inline void gt_rows(int n, int r, int ldt, FU fu, const float* M, float* Gg) {
  constexpr int TN = RP >= 128 ? 4 : (RP >= 64 ? 2 : 1);
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int row0 = 0; row0 < n; row0 += 96) {
    float acc[6][TN];
    cta_mm<6, TN>(n, RP, r, row0, fu, [&](int l, int m) { return M[m * ldt + l]; }, acc);
#pragma unroll
    for (int u = 0; u < 6; ++u)
#pragma unroll
      for (int v = 0; v < TN; ++v) {
        const int i = row0 + ty + 16 * u, m = tx + 32 * v;
        if (i < n && m < RP) Gg[(int64_t)i * RP + m] = acc[u][v];
      }
  }
}

template <int RP>
__global__ void __launch_bounds__(kProcThreads, 2) procrustes_qr_kernel(ProcArgs a) {
  extern __shared__ __align__(16) float sm[];
  __shared__ float red[32];
  __shared__ double dred[32];
  __shared__ int ival[4];
  const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5, nw = kProcThreads / 32;
  const int64_t g = blockIdx.x;
  const fh_tile T = a.tiles[a.row_tile[g]];
  const int i0 = (int)(g - T.brow0);
  const int n = T.width, r = T.rank, ci = T.chrom;
  const int ldt = r + 1;
  float* R0 = sm;
  float* R1 = R0 + (size_t)proc_r0_rows(n, r, RP) * ldt;
  float* misc = R1 + (size_t)proc_r1_rows(n, r, RP) * ldt;
  PolarScratch s = polar_scratch(misc, red, dred, ival);
  if (tid == 0) ival[0] = 0;
  const int64_t brow = T.xoff + (int64_t)i0 * n;
  float* Gg = a.Gt + brow * RP;
  form_m<RP>(a, g, ci, r, ldt, R0, R1);   // M in region 1
  if (a.mode == 1) {
    // transform: Gt_g = U_g M^T with the stored projection (parafac2_intergrative.py:772-801)
    const float* Ug = a.U + T.uoff + (int64_t)i0 * n * r;
    gt_rows<RP>(n, r, ldt, [&](int i, int l) { return __ldg(Ug + (int64_t)i * r + l); }, R1, Gg);
    return;
  }
  // ---- temp[i][l] = sum_m W_g[i][m] M[m][l] into region 0
  {
    const float* Wg = a.W + brow * RP;
    for (int row0 = 0; row0 < n; row0 += 96) {
      float acc[6][2];
      cta_mm<6, 2>(n, r, RP, row0, [&](int i, int m) { return __ldg(Wg + (int64_t)i * RP + m); },
                   [&](int m, int l) { return R1[m * ldt + l]; }, acc);
#pragma unroll
      for (int u = 0; u < 6; ++u)
#pragma unroll
        for (int v = 0; v < 2; ++v) {
          const int i = row0 + ty + 16 * u, l = tx + 32 * v;
          if (i < n && l < r) R0[i * ldt + l] = acc[u][v];
        }
    }
    __syncthreads();
  }
  // ---- QR, polar factor of R, sum(S)
  householder_qr_fast<(RP + 15) / 16>(R0, n, r, ldt, s);
  // polar(R) on 16-byte aligned rows of stride ldv (4 x 4 register-tiled products), then
  // back to stride ldt in region 1 for the Q apply
  const int ldv = ((r + 3) & ~3) + 4;
  float* Xv = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(R1) + 15) & ~uintptr_t(15));
  for (int p = ty; p < r; p += nw)
    for (int q = tx; q < r; q += 32) Xv[p * ldv + q] = q >= p ? R0[p * ldt + q] : 0.f;
  __syncthreads();
  newton_polar_r64v(Xv, ldv, Xv + (size_t)r * ldv, r, s);
  float* X = R1;
  {
    float v[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int idx = tid + kProcThreads * e;
      v[e] = idx < r * r ? Xv[(idx / r) * ldv + idx % r] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int idx = tid + kProcThreads * e;
      if (idx < r * r) X[(idx / r) * ldt + idx % r] = v[e];
    }
    __syncthreads();
  }
  {
    double acc = 0.0;
    for (int p = ty; p < r; p += nw)
      for (int q = p + tx; q < r; q += 32) acc += (double)X[p * ldt + q] * (double)R0[p * ldt + q];
    acc = block_sum<double>(acc, dred);
    if (tid == 0) a.ssum[g] = acc;
  }
  // ---- U = Q [P; 0]: U's first r rows are X (same storage and stride)
  apply_q_fast<(RP + 15) / 16>(R0, ldt, R1, ldt, n, r, s);
  float* Ug = a.U + T.uoff + (int64_t)i0 * n * r;
  for (int j = ty; j < n; j += nw)
    for (int l = tx; l < r; l += 32) Ug[(int64_t)j * r + l] = R1[j * ldt + l];
  // ---- Gt = U M^T (M formed again in region 0)
  form_m<RP>(a, g, ci, r, ldt, R0, R0);
  gt_rows<RP>(n, r, ldt, [&](int i, int l) { return R1[i * ldt + l]; }, R0, Gg);
  if (tid == 0 && ival[0]) set_status(a.status, FH_ERR_ILLCOND);
}

// ---- ranks up to 128 (RP = 128) ------------------------------------------------------------
// The same step with two regions of max(n, RP) rows at stride ldt = r + 1 (219.5 KB at
// n = 205, r = 128; one CTA per SM).  The regions cannot hold the reflectors, the Newton
// iterate and its scratch at once, so the CTA parks what it needs later in the bin row's own
// output slots, which it overwrites at the end: M (RP x r) in its G^T rows (n x RP floats) and
// the factored temp (R and the reflectors, n x r) in its U rows.  Reads of those parked values
// come after a barrier and use ordinary loads (the CTA's own global writes are visible to it).
//   RA: stage of M / temp -> QR / Newton scratch / reflectors again / M again
//   RB: M / the Newton iterate (stride ldv) / U = Q [polar(R); 0]
__host__ __device__ inline size_t procb_region_floats(int n, int r, int rp) {
  const int ldt = r + 1, ldv = ((r + 3) & ~3) + 4;
  size_t a = (size_t)(n > rp ? n : rp) * ldt;
  const size_t v = (size_t)(r + 4) * ldv + 4;   // aligned iterate / scratch plus the rows mm4t
  if (v > a) a = v;                             // reads past r
  return (a + 3) & ~(size_t)3;
}
__host__ __device__ inline size_t procb_smem_floats(int n, int r, int rp) {
  return 2 * procb_region_floats(n, r, rp) + kPolarMiscFloats;
}

__global__ void __launch_bounds__(kProcThreads, 1) procrustes_qr_big_kernel(ProcArgs a,
                                                                           int region) {
  constexpr int RP = 128;
  extern __shared__ __align__(16) float sm[];
  __shared__ float red[32];
  __shared__ double dred[32];
  __shared__ int ival[4];
  const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5, nw = kProcThreads / 32;
  const int64_t g = blockIdx.x;
  const fh_tile T = a.tiles[a.row_tile[g]];
  const int i0 = (int)(g - T.brow0);
  const int n = T.width, r = T.rank, ci = T.chrom;
  const int ldt = r + 1, ldv = ((r + 3) & ~3) + 4;
  float* RA = sm;
  float* RB = sm + region;
  PolarScratch s = polar_scratch(RB + region, red, dred, ival);
  if (tid == 0) ival[0] = 0;
  const int64_t brow = T.xoff + (int64_t)i0 * n;
  float* Gg = a.Gt + brow * RP;
  float* Ug = a.U + T.uoff + (int64_t)i0 * n * r;
  form_m<RP>(a, g, ci, r, ldt, RA, RB);   // M in RB (the stage spans RA and RB)
  if (a.mode == 1) {
    // transform: Gt_g = U_g M^T with the stored projection (parafac2_intergrative.py:772-801)
    const float* Us = Ug;
    gt_rows<RP>(n, r, ldt, [&](int i, int l) { return __ldg(Us + (int64_t)i * r + l); }, RB, Gg);
    return;
  }
  for (int m = ty; m < RP; m += nw)
    for (int l = tx; l < r; l += 32) Gg[m * r + l] = RB[m * ldt + l];   // park M
  // ---- temp[i][l] = sum_m W_g[i][m] M[m][l] into RA
  {
    const float* Wg = a.W + brow * RP;
    for (int row0 = 0; row0 < n; row0 += 96) {
      float acc[6][4];
      cta_mm<6, 4>(n, r, RP, row0, [&](int i, int m) { return __ldg(Wg + (int64_t)i * RP + m); },
                   [&](int m, int l) { return RB[m * ldt + l]; }, acc);
#pragma unroll
      for (int u = 0; u < 6; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          const int i = row0 + ty + 16 * u, l = tx + 32 * v;
          if (i < n && l < r) RA[i * ldt + l] = acc[u][v];
        }
    }
    __syncthreads();
  }
  householder_qr_fast<8>(RA, n, r, ldt, s);
  // park R and the reflectors; the iterate X = R (upper) at stride ldv in RB, scratch in RA
  for (int i = ty; i < n; i += nw)
    for (int l = tx; l < r; l += 32) Ug[(int64_t)i * r + l] = RA[i * ldt + l];
  for (int p = ty; p < r; p += nw)
    for (int q = tx; q < r; q += 32) RB[p * ldv + q] = q >= p ? RA[p * ldt + q] : 0.f;
  __syncthreads();
  newton_polar_tiled<8>(RB, ldv, RA, r, s);
  // X to stride ldt in place (through registers), the parked factorization back into RA
  {
    float v[32];
#pragma unroll
    for (int e = 0; e < 32; ++e) {
      const int idx = tid + kProcThreads * e;
      v[e] = idx < r * r ? RB[(idx / r) * ldv + idx % r] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int e = 0; e < 32; ++e) {
      const int idx = tid + kProcThreads * e;
      if (idx < r * r) RB[(idx / r) * ldt + idx % r] = v[e];
    }
    for (int i = ty; i < n; i += nw)
      for (int l = tx; l < r; l += 32) RA[i * ldt + l] = Ug[(int64_t)i * r + l];
    __syncthreads();
  }
  {
    double acc = 0.0;
    for (int p = ty; p < r; p += nw)
      for (int q = p + tx; q < r; q += 32) acc += (double)RB[p * ldt + q] * (double)RA[p * ldt + q];
    acc = block_sum<double>(acc, dred);
    if (tid == 0) a.ssum[g] = acc;
  }
  // ---- U = Q [P; 0]
  __syncthreads();
  apply_q_fast<8>(RA, ldt, RB, ldt, n, r, s);
  for (int j = ty; j < n; j += nw)
    for (int l = tx; l < r; l += 32) Ug[(int64_t)j * r + l] = RB[j * ldt + l];
  // ---- Gt = U M^T with the parked M
  for (int m = ty; m < RP; m += nw)
    for (int l = tx; l < r; l += 32) RA[m * ldt + l] = Gg[m * r + l];
  __syncthreads();
  gt_rows<RP>(n, r, ldt, [&](int i, int l) { return RB[i * ldt + l]; }, RA, Gg);
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
  PolarScratch s = polar_scratch(misc, red, dred, ival);
  if (tid == 0) ival[0] = 0;
  const float* Mb = M + b * (int64_t)n * r;
  for (int i = ty; i < n; i += nw)
    for (int l = tx; l < r; l += 32) Tm[i * ldt + l] = Mb[(int64_t)i * r + l];
  __syncthreads();
  householder_qr_fast<8>(Tm, n, r, ldt, s);
  float* X = reg;
  for (int p = ty; p < r; p += nw)
    for (int q = tx; q < r; q += 32) X[p * ldt + q] = q >= p ? Tm[p * ldt + q] : 0.f;
  __syncthreads();
  if (r <= 64) newton_polar_r64(X, ldt, reg + (size_t)r * ldt, r, true, s);
  else newton_polar(X, ldt, reg + (size_t)r * ldt, r, true, s);
  double acc = 0.0;
  for (int p = ty; p < r; p += nw)
    for (int q = p + tx; q < r; q += 32) acc += (double)X[p * ldt + q] * (double)Tm[p * ldt + q];
  acc = block_sum<double>(acc, dred);
  if (tid == 0 && ssum) ssum[b] = acc;
  __syncthreads();
  apply_q_fast<8>(Tm, ldt, reg, ldt, n, r, s);
  float* Ub = U + b * (int64_t)n * r;
  for (int j = ty; j < n; j += nw)
    for (int l = tx; l < r; l += 32) Ub[(int64_t)j * r + l] = reg[j * ldt + l];
  if (tid == 0 && ival[0]) set_status(status, FH_ERR_ILLCOND);
}

}  // namespace fh

using namespace fh;

static int proc_launch(const ProcArgs& a, int64_t n_rows, int max_width, int max_rank, int rp,
                       cudaStream_t s) {
  if (max_width > kMaxWidth || max_rank > rp) return FH_ERR_UNSUPPORTED;
  if (rp == 128) {
    const size_t region = procb_region_floats(max_width, max_rank, rp);
    const size_t smem = procb_smem_floats(max_width, max_rank, rp) * sizeof(float);
    if (smem > 227 * 1024) return FH_ERR_UNSUPPORTED;
    if (ensure_smem((const void*)procrustes_qr_big_kernel, smem)) return FH_ERR_LAUNCH;
    procrustes_qr_big_kernel<<<(unsigned)n_rows, kProcThreads, smem, s>>>(a, (int)region);
    FH_CHECK_LAUNCH();
    return FH_OK;
  }
  if (max_rank > 64) return FH_ERR_UNSUPPORTED;
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
