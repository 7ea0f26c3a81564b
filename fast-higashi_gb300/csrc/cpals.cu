// CP-ALS inner solver on the projected tensors Y_chrom (nbin x r x R), all chromosomes at once.
//
// Reference: fasthigashi/parafac_integrative.py:12-112 (update_factor, balance_norm, parafac)
// called per chromosome from parafac2_intergrative.py:674-695, and the core norm
// ||[[A, B, D]]||^2 of :621-632 / :697-706.
//
// One sweep updates A, B, D in turn from normal equations
//     A <- MTTKRP_A (B^T B * D^T D + 1e-10 I)^{-1}   (and likewise for B, D)
// The Hadamard Gram matrices are r x r; they are assembled in fp64, factored by fp64
// Cholesky and the factor rows solved in fp64.  The MTTKRP products run in fp32:
//     MTTKRP_A[i] = sum_j B[j] * (Y_i D)[j],   MTTKRP_B = sum_i A_i (x) (Y_i D),
//     MTTKRP_D   = sum_i A_i (x) (Y_i^T B)      ((x): column-wise product).
// The reconstruction loss needs no Xhat:  ||Xhat||^2 = sum(A^TA * B^TB * D^TD) and
// <Xhat, Y> = sum(D * MTTKRP_D) with the final A, B.  balance_norm (unit columns, the
// product of the column norms folded into D) follows each sweep unless the relative loss
// change fell below 1e-5, exactly as the reference breaks before balancing.
//
// Bin rows are processed in chunks of <= 8 rows of one chromosome; per-chunk fp64 partial
// sums are reduced in a fixed order by the per-chromosome kernel (deterministic).
#include "fh_common.cuh"

namespace fh {

constexpr int kCpThreads = 256;
constexpr int kCpMaxR = 64;  // r and R handled by these kernels

struct CpArgs {
  int nchrom;
  const int32_t* c_row0;   // first global bin row of the chromosome
  const int32_t* c_nbin;
  const int32_t* c_rank;
  const int32_t* c_chunk0; // first chunk of the chromosome
  const int32_t* c_nchunk;
  const int32_t* k_chrom;  // chunk -> chromosome
  const int32_t* k_row0;   // chunk -> first global bin row
  const int32_t* k_nrow;
  float* A;        // [bin rows][ld]
  float* B;        // [chrom][ld][ld]
  float* D;        // [chrom][RP][ld]
  const float* Y;  // [bin rows][ldy][RP]
  int ld, RP, R, ldy;
  double* L;       // [chrom][ld][ld]    Cholesky factor of the current mode
  double* part;    // [chunk][2][ld*ld] or [chunk][RP*ld]
  double* gAA;     // [chrom][ld*ld]
  double* gBB;
  double* gDD;
  double* rhs;     // [chrom][RP*ld]
  float* scaleA;   // [chrom][ld]
  double* ynorm;   // [chrom]
  double* loss;    // [chrom][2]: previous, current
  int* state;      // [chrom]: 0 = running, 1 = converged (stop), bit 2: first sweep done
  double* core;    // [chrom] ||[[A,B,D]]||^2
  double* cross;   // [chrom] <[[A,B,D]], Y> of the last sweep (optional)
  int* status;
};

enum CpRowMode { kRowsNorm = 0, kRowsAB = 1, kRowsD = 2, kRowsScale = 3, kRowsGram = 4 };
enum CpSmallMode { kSmallInit = 0, kSmallB = 1, kSmallD = 2, kSmallCore = 3 };

// Z = Y_g D (r x r) or Z = Y_g^T B (R x r) into shared memory.
__device__ void cp_load_y(const CpArgs& a, int64_t g, int r, float* Ys) {
  const float* Yg = a.Y + g * (int64_t)a.ldy * a.RP;
  for (int idx = threadIdx.x; idx < r * a.R; idx += blockDim.x) {
    const int j = idx / a.R, m = idx % a.R;
    Ys[j * (kCpMaxR + 1) + m] = Yg[(int64_t)j * a.RP + m];
  }
}

__host__ __device__ inline size_t cp_pstride(int ld) { return (size_t)2 * ld * ld + 1; }
constexpr int kCpLz = kCpMaxR + 1;
constexpr size_t kCpRowsSmem = 4 * (size_t)kCpMaxR * kCpLz * sizeof(float);

__global__ void __launch_bounds__(kCpThreads) cp_rows_kernel(CpArgs a, int mode) {
  extern __shared__ __align__(16) float cps[];
  float* Ys = cps;                        // Y_g (r x R)
  float* Fs = Ys + kCpMaxR * kCpLz;       // D (R x r) or B (r x r)
  float* Bs = Fs + kCpMaxR * kCpLz;       // B (mode AB)
  float* Zs = Bs + kCpMaxR * kCpLz;
  __shared__ float rhs[kCpMaxR];
  __shared__ double dred[32];
  const int k = blockIdx.x;
  const int ci = a.k_chrom[k];
  if (mode != kRowsNorm && mode != kRowsGram && (a.state[ci] & 1)) return;
  const int r = a.c_rank[ci], R = a.R, ld = a.ld, lz = kCpMaxR + 1;
  const int64_t row0 = a.k_row0[k];
  const int nrow = a.k_nrow[k];
  const int tid = threadIdx.x;

  if (mode == kRowsScale) {
    const float* sc = a.scaleA + (size_t)ci * ld;
    for (int idx = tid; idx < nrow * r; idx += blockDim.x) {
      const int64_t g = row0 + idx / r;
      a.A[g * ld + idx % r] *= sc[idx % r];
    }
    return;
  }
  if (mode == kRowsNorm || mode == kRowsGram) {
    // partial column sums of squares of A (or the full A^T A) and of Y
    double* out = a.part + (size_t)k * cp_pstride(ld);
    for (int idx = tid; idx < r * r; idx += blockDim.x) {
      const int p = idx / r, q = idx % r;
      double s = 0.0;
      if (mode == kRowsGram || p == q)
        for (int i = 0; i < nrow; ++i)
          s = fma((double)a.A[(row0 + i) * ld + p], (double)a.A[(row0 + i) * ld + q], s);
      out[p * ld + q] = s;
    }
    double ys = 0.0;
    for (int i = 0; i < nrow; ++i) {
      const float* Yg = a.Y + (row0 + i) * (int64_t)a.ldy * a.RP;
      for (int idx = tid; idx < r * R; idx += blockDim.x) {
        const double v = Yg[(int64_t)(idx / R) * a.RP + idx % R];
        ys = fma(v, v, ys);
      }
    }
    ys = block_sum<double>(ys, dred);
    if (tid == 0) out[ld * ld] = ys;
    return;
  }
  // mode AB or D: stage the fixed factors
  const float* Dc = a.D + (size_t)ci * a.RP * ld;
  const float* Bc = a.B + (size_t)ci * ld * ld;
  if (mode == kRowsAB) {
    for (int idx = tid; idx < R * r; idx += blockDim.x) Fs[(idx / r) * lz + idx % r] = Dc[(idx / r) * ld + idx % r];
    for (int idx = tid; idx < r * r; idx += blockDim.x) Bs[(idx / r) * lz + idx % r] = Bc[(idx / r) * ld + idx % r];
  } else {
    for (int idx = tid; idx < r * r; idx += blockDim.x) Fs[(idx / r) * lz + idx % r] = Bc[(idx / r) * ld + idx % r];
  }
  // chunk partial accumulators (registers -> fp64)
  const int npart = mode == kRowsAB ? r * r : R * r;
  double pA[(kCpMaxR * kCpMaxR + kCpThreads - 1) / kCpThreads];   // A^T A or rhs_D partial
  double pB[(kCpMaxR * kCpMaxR + kCpThreads - 1) / kCpThreads];   // rhs_B partial
#pragma unroll
  for (int q = 0; q < (kCpMaxR * kCpMaxR + kCpThreads - 1) / kCpThreads; ++q) pA[q] = pB[q] = 0.0;
  const double* Lc = a.L + (size_t)ci * ld * ld;
  __syncthreads();
  for (int i = 0; i < nrow; ++i) {
    const int64_t g = row0 + i;
    cp_load_y(a, g, r, Ys);
    __syncthreads();
    if (mode == kRowsAB) {
      // Z[j][rho] = sum_m Y[j][m] D[m][rho]
      for (int idx = tid; idx < r * r; idx += blockDim.x) {
        const int j = idx / r, rho = idx % r;
        float s = 0.f;
        for (int m = 0; m < R; ++m) s = fmaf(Ys[j * lz + m], Fs[m * lz + rho], s);
        Zs[j * lz + rho] = s;
      }
      __syncthreads();
      if (tid < r) {
        float s = 0.f;
        for (int j = 0; j < r; ++j) s = fmaf(Bs[j * lz + tid], Zs[j * lz + tid], s);
        rhs[tid] = s;
      }
      __syncthreads();
      // solve L L^T a = rhs (fp64), one warp
      if (tid < 32) {
        // forward: y = L^{-1} rhs, L lower stored in Lc[p*ld+q] (q <= p)
        __shared__ double ys[kCpMaxR];
        for (int p = 0; p < r; ++p) {
          double s = 0.0;
          for (int q = tid; q < p; q += 32) s = fma(Lc[p * ld + q], ys[q], s);
          s = warp_sum(s);
          if (tid == 0) ys[p] = ((double)rhs[p] - s) / Lc[p * ld + p];
          __syncwarp();
        }
        // backward: x = L^{-T} y
        for (int p = r - 1; p >= 0; --p) {
          double s = 0.0;
          for (int q = p + 1 + tid; q < r; q += 32) s = fma(Lc[q * ld + p], ys[q], s);
          s = warp_sum(s);
          if (tid == 0) ys[p] = (ys[p] - s) / Lc[p * ld + p];
          __syncwarp();
        }
        for (int p = tid; p < r; p += 32) {
          const float v = (float)ys[p];
          a.A[g * ld + p] = v;
          rhs[p] = v;  // the new A row for the partials below
        }
      }
      __syncthreads();
      // partials: A^T A and rhs_B[j][rho] += A[rho] Z[j][rho]
      int q = 0;
      for (int idx = tid; idx < r * r; idx += blockDim.x, ++q) {
        const int p = idx / r, s2 = idx % r;
        pA[q] = fma((double)rhs[p], (double)rhs[s2], pA[q]);
        pB[q] = fma((double)rhs[s2], (double)Zs[p * lz + s2], pB[q]);
      }
      __syncthreads();
    } else {
      // Z'[m][rho] = sum_j Y[j][m] B[j][rho];  rhs_D[m][rho] += A[rho] Z'[m][rho]
      const float* Ag = a.A + g * ld;
      int q = 0;
      for (int idx = tid; idx < R * r; idx += blockDim.x, ++q) {
        const int m = idx / r, rho = idx % r;
        float s = 0.f;
        for (int j = 0; j < r; ++j) s = fmaf(Ys[j * lz + m], Fs[j * lz + rho], s);
        pA[q] = fma((double)Ag[rho], (double)s, pA[q]);
      }
      __syncthreads();
    }
  }
  double* out = a.part + (size_t)k * cp_pstride(ld);
  int q = 0;
  for (int idx = tid; idx < npart; idx += blockDim.x, ++q) {
    if (mode == kRowsAB) {
      out[(idx / r) * ld + idx % r] = pA[q];
      out[ld * ld + (idx / r) * ld + idx % r] = pB[q];
    } else {
      out[(idx / r) * ld + idx % r] = pA[q];  // R x r with stride ld (R <= ld)
    }
  }
}

// fp64 Cholesky of G (r x r, stride ld) in place into its lower triangle.
__device__ bool cp_cholesky(double* G, int r, int ld) {
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  for (int k = 0; k < r; ++k) {
    if (threadIdx.x == 0) {
      double d = G[k * ld + k];
      if (!(d > 0.0)) { bad = 1; d = 1e-300; }
      G[k * ld + k] = sqrt(d);
    }
    __syncthreads();
    const double dk = G[k * ld + k];
    for (int p = k + 1 + threadIdx.x; p < r; p += blockDim.x) G[p * ld + k] /= dk;
    __syncthreads();
    const int nc = r - k - 1;
    for (int idx = threadIdx.x; idx < nc * nc; idx += blockDim.x) {
      const int p = k + 1 + idx / nc, q = k + 1 + idx % nc;
      if (q <= p) G[p * ld + q] -= G[p * ld + k] * G[q * ld + k];
    }
    __syncthreads();
  }
  return bad == 0;
}

// x = (L L^T)^{-1} b for rows of RHS (nrhs x r, stride ld), one thread per row, fp64.
__device__ void cp_solve_rows(const double* L, int r, int ld, const double* RHS, int nrhs,
                              float* out, int ldo, double* work /* nrhs x ld */) {
  for (int row = threadIdx.x; row < nrhs; row += blockDim.x) {
    double* y = work + (size_t)row * ld;
    for (int p = 0; p < r; ++p) {
      double s = RHS[(size_t)row * ld + p];
      for (int q = 0; q < p; ++q) s -= L[p * ld + q] * y[q];
      y[p] = s / L[p * ld + p];
    }
    for (int p = r - 1; p >= 0; --p) {
      double s = y[p];
      for (int q = p + 1; q < r; ++q) s -= L[q * ld + p] * y[q];
      y[p] = s / L[p * ld + p];
    }
    for (int p = 0; p < r; ++p) out[(size_t)row * ldo + p] = (float)y[p];
  }
}

// Gram F^T F (fp64) of an (nrows x r, stride ld) fp32 factor into G (stride ld).
__device__ void cp_gram(const float* F, int nrows, int r, int ld, double* G) {
  for (int idx = threadIdx.x; idx < r * r; idx += blockDim.x) {
    const int p = idx / r, q = idx % r;
    double s = 0.0;
    for (int i = 0; i < nrows; ++i) s = fma((double)F[i * ld + p], (double)F[i * ld + q], s);
    G[p * ld + q] = s;
  }
}

__global__ void __launch_bounds__(kCpThreads) cp_small_kernel(CpArgs a, int mode) {
  extern __shared__ __align__(16) double sd[];
  const int ci = blockIdx.x;
  const int r = a.c_rank[ci], R = a.R, ld = a.ld;
  const int tid = threadIdx.x;
  double* G = sd;                         // ld*ld
  double* work = G + ld * ld;             // RP*ld
  __shared__ double dred[32];
  __shared__ double nA[kCpMaxR], nB[kCpMaxR], nD[kCpMaxR];
  double* gAA = a.gAA + (size_t)ci * ld * ld;
  double* gBB = a.gBB + (size_t)ci * ld * ld;
  double* gDD = a.gDD + (size_t)ci * ld * ld;
  float* Bc = a.B + (size_t)ci * ld * ld;
  float* Dc = a.D + (size_t)ci * a.RP * ld;
  double* Lc = a.L + (size_t)ci * ld * ld;
  const int k0 = a.c_chunk0[ci], nk = a.c_nchunk[ci];
  const size_t pstride = cp_pstride(ld);

  if (mode == kSmallCore) {
    // core norm from full partial A^T A (kRowsGram) and fresh B^T B, D^T D
    for (int idx = tid; idx < r * r; idx += blockDim.x) {
      const int p = idx / r, q = idx % r;
      double s = 0.0;
      for (int k = 0; k < nk; ++k) s += a.part[(k0 + k) * pstride + p * ld + q];
      gAA[p * ld + q] = s;
    }
    cp_gram(Bc, r, r, ld, gBB);
    cp_gram(Dc, R, r, ld, gDD);
    __syncthreads();
    double c = 0.0;
    for (int idx = tid; idx < r * r; idx += blockDim.x) {
      const int p = idx / r, q = idx % r;
      c += gAA[p * ld + q] * gBB[p * ld + q] * gDD[p * ld + q];
    }
    c = block_sum<double>(c, dred);
    if (tid == 0) a.core[ci] = c;
    return;
  }
  if (mode == kSmallInit) {
    // reduce the column norms of A and ||Y||^2, balance (parafac_integrative.py:19-27, :65)
    if (tid < r) {
      double s = 0.0;
      for (int k = 0; k < nk; ++k) s += a.part[(k0 + k) * pstride + tid * ld + tid];
      nA[tid] = sqrt(s);
    }
    if (tid == 0) {
      double s = 0.0;
      for (int k = 0; k < nk; ++k) s += a.part[(k0 + k) * pstride + ld * ld];
      a.ynorm[ci] = s;
      a.state[ci] = 0;
      a.loss[2 * ci] = 0.0;
      a.loss[2 * ci + 1] = 0.0;
    }
    cp_gram(Bc, r, r, ld, gBB);
    cp_gram(Dc, R, r, ld, gDD);
    __syncthreads();
  } else {
    if (a.state[ci] & 1) return;
  }

  if (mode == kSmallB) {
    // reduce A^T A and rhs_B; G_B = A^T A * D^T D + 1e-10 I; B <- rhs_B G_B^{-1}
    for (int idx = tid; idx < r * r; idx += blockDim.x) {
      const int p = idx / r, q = idx % r;
      double s = 0.0, t = 0.0;
      for (int k = 0; k < nk; ++k) {
        s += a.part[(k0 + k) * pstride + p * ld + q];
        t += a.part[(k0 + k) * pstride + ld * ld + p * ld + q];
      }
      gAA[p * ld + q] = s;
      work[p * ld + q] = t;
    }
    __syncthreads();
    for (int idx = tid; idx < r * r; idx += blockDim.x) {
      const int p = idx / r, q = idx % r;
      G[p * ld + q] = gAA[p * ld + q] * gDD[p * ld + q] + (p == q ? 1e-10 : 0.0);
    }
    __syncthreads();
    if (!cp_cholesky(G, r, ld) && tid == 0) set_status(a.status, FH_ERR_ILLCOND);
    __syncthreads();
    // solve rows in place: work rows are the rhs; the solution overwrites B
    double* w2 = a.rhs + (size_t)ci * a.RP * ld;
    cp_solve_rows(G, r, ld, work, r, Bc, ld, w2);
    __syncthreads();
    cp_gram(Bc, r, r, ld, gBB);
    return;
  }
  if (mode == kSmallD) {
    // reduce rhs_D; G_D = A^T A * B^T B + 1e-10 I; D <- rhs_D G_D^{-1}; loss; balance
    for (int idx = tid; idx < R * r; idx += blockDim.x) {
      const int m = idx / r, q = idx % r;
      double s = 0.0;
      for (int k = 0; k < nk; ++k) s += a.part[(k0 + k) * pstride + m * ld + q];
      work[m * ld + q] = s;
    }
    for (int idx = tid; idx < r * r; idx += blockDim.x) {
      const int p = idx / r, q = idx % r;
      G[p * ld + q] = gAA[p * ld + q] * gBB[p * ld + q] + (p == q ? 1e-10 : 0.0);
    }
    __syncthreads();
    if (!cp_cholesky(G, r, ld) && tid == 0) set_status(a.status, FH_ERR_ILLCOND);
    __syncthreads();
    double* w2 = a.rhs + (size_t)ci * a.RP * ld;
    cp_solve_rows(G, r, ld, work, R, Dc, ld, w2);
    __syncthreads();
    cp_gram(Dc, R, r, ld, gDD);
    __syncthreads();
    // loss = ||Y||^2 + ||Xhat||^2 - 2 <Xhat, Y>
    double xh = 0.0, xy = 0.0;
    for (int idx = tid; idx < r * r; idx += blockDim.x) {
      const int p = idx / r, q = idx % r;
      xh += gAA[p * ld + q] * gBB[p * ld + q] * gDD[p * ld + q];
    }
    for (int idx = tid; idx < R * r; idx += blockDim.x) {
      const int m = idx / r, q = idx % r;
      xy += (double)Dc[m * ld + q] * work[m * ld + q];
    }
    xh = block_sum<double>(xh, dred);
    __syncthreads();
    xy = block_sum<double>(xy, dred);
    __shared__ int stop;
    if (tid == 0) {
      const double loss = a.ynorm[ci] + xh - 2.0 * xy;
      const double prev = a.loss[2 * ci + 1];
      const bool first = (a.state[ci] & 2) == 0;
      const double wdiff = first ? NAN : (prev - loss) / prev;
      a.loss[2 * ci] = prev;
      a.loss[2 * ci + 1] = loss;
      a.core[ci] = xh;
      if (a.cross) a.cross[ci] = xy;
      stop = (!first && wdiff < 1e-5) ? 1 : 0;
      a.state[ci] = (a.state[ci] | 2) | stop;
    }
    __syncthreads();
    if (stop) {
      // no balance: A needs no scaling
      if (tid < r) a.scaleA[(size_t)ci * ld + tid] = 1.f;
      return;
    }
    if (tid < r) nA[tid] = sqrt(gAA[tid * ld + tid]);
    __syncthreads();
  }
  // ---- balance_norm: A /= |A|, B /= |B|, D = D / |D| * (|A||B||D| + 1e-15)
  if (tid < r) {
    nB[tid] = sqrt(gBB[tid * ld + tid]);
    nD[tid] = sqrt(gDD[tid * ld + tid]);
  }
  __syncthreads();
  if (tid < r) a.scaleA[(size_t)ci * ld + tid] = (float)(1.0 / (nA[tid] + 1e-15));
  for (int idx = tid; idx < r * r; idx += blockDim.x) {
    const int j = idx / r, q = idx % r;
    Bc[j * ld + q] = (float)((double)Bc[j * ld + q] / (nB[q] + 1e-15));
  }
  for (int idx = tid; idx < R * r; idx += blockDim.x) {
    const int m = idx / r, q = idx % r;
    const double even = nA[q] * nB[q] * nD[q] + 1e-15;
    Dc[m * ld + q] = (float)((double)Dc[m * ld + q] / (nD[q] + 1e-15) * even);
  }
  __syncthreads();
  // Grams of the balanced factors and the next mode-A factor L_A = chol(B^T B * D^T D + eps I)
  cp_gram(Bc, r, r, ld, gBB);
  cp_gram(Dc, R, r, ld, gDD);
  __syncthreads();
  for (int idx = tid; idx < r * r; idx += blockDim.x) {
    const int p = idx / r, q = idx % r;
    G[p * ld + q] = gBB[p * ld + q] * gDD[p * ld + q] + (p == q ? 1e-10 : 0.0);
  }
  __syncthreads();
  if (!cp_cholesky(G, r, ld) && tid == 0) set_status(a.status, FH_ERR_ILLCOND);
  __syncthreads();
  for (int idx = tid; idx < r * r; idx += blockDim.x) Lc[idx / r * ld + idx % r] = G[idx / r * ld + idx % r];
}

}  // namespace fh

using namespace fh;

extern "C" size_t fh_cp_workspace(int32_t nchrom, int32_t nchunks, int32_t ld, int32_t rp) {
  const size_t l = (size_t)ld * ld;
  return sizeof(double) * ((size_t)nchrom * (4 * l + (size_t)rp * ld + 4) +
                           (size_t)nchunks * cp_pstride(ld)) +
         sizeof(float) * (size_t)nchrom * ld + sizeof(int) * (size_t)nchrom + 64;
}

// Runs n_iter CP-ALS sweeps on every chromosome (parafac with n_iter_max = n_iter) and leaves
// core[chrom] = ||[[A,B,D]]||^2 of the result.  meta: int32 tables
//   [c_row0, c_nbin, c_rank, c_chunk0, c_nchunk] (nchrom each) then
//   [k_chrom, k_row0, k_nrow] (nchunks each).
extern "C" int fh_cp_als(int32_t nchrom, int32_t nchunks, const int32_t* meta, float* A,
                         float* B, float* D, const float* Y, int32_t ld, int32_t rp, int32_t R,
                         int32_t ldy, int32_t n_iter, double* core, double* cross,
                         void* workspace, size_t workspace_bytes, int* status, void* stream) {
  if (nchrom <= 0 || nchunks <= 0 || !meta || !A || !B || !D || !Y || !core || !workspace ||
      n_iter < 0 || R > rp || ld < R || rp > ld)
    return FH_ERR_ARG;
  if (ld > kCpMaxR || R > kCpMaxR) return FH_ERR_UNSUPPORTED;
  if (workspace_bytes < fh_cp_workspace(nchrom, nchunks, ld, rp)) return FH_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t l = (size_t)ld * ld;
  CpArgs a{};
  a.nchrom = nchrom;
  a.c_row0 = meta; a.c_nbin = meta + nchrom; a.c_rank = meta + 2 * nchrom;
  a.c_chunk0 = meta + 3 * nchrom; a.c_nchunk = meta + 4 * nchrom;
  a.k_chrom = meta + 5 * nchrom; a.k_row0 = a.k_chrom + nchunks; a.k_nrow = a.k_row0 + nchunks;
  a.A = A; a.B = B; a.D = D; a.Y = Y; a.ld = ld; a.RP = rp; a.R = R; a.ldy = ldy;
  double* w = (double*)workspace;
  a.L = w; w += nchrom * l;
  a.gAA = w; w += nchrom * l;
  a.gBB = w; w += nchrom * l;
  a.gDD = w; w += nchrom * l;
  a.rhs = w; w += (size_t)nchrom * rp * ld;
  a.ynorm = w; w += nchrom;
  a.loss = w; w += 2 * (size_t)nchrom;
  w += nchrom;  // spare
  a.part = w; w += (size_t)nchunks * cp_pstride(ld);
  a.scaleA = (float*)w;
  a.state = (int*)(a.scaleA + (size_t)nchrom * ld);
  a.core = core;
  a.cross = cross;
  a.status = status;
  const size_t small_smem = (l + (size_t)rp * ld) * sizeof(double);
  if (ensure_smem((const void*)cp_small_kernel, small_smem) ||
      ensure_smem((const void*)cp_rows_kernel, kCpRowsSmem))
    return FH_ERR_LAUNCH;
  const size_t rs = kCpRowsSmem;
  if (n_iter == 0) {  // core norm only, factors untouched
    cp_rows_kernel<<<nchunks, kCpThreads, rs, s>>>(a, kRowsGram);
    cp_small_kernel<<<nchrom, kCpThreads, small_smem, s>>>(a, kSmallCore);
    FH_CHECK_LAUNCH();
    return FH_OK;
  }
  cp_rows_kernel<<<nchunks, kCpThreads, rs, s>>>(a, kRowsNorm);
  cp_small_kernel<<<nchrom, kCpThreads, small_smem, s>>>(a, kSmallInit);
  cp_rows_kernel<<<nchunks, kCpThreads, rs, s>>>(a, kRowsScale);
  for (int it = 0; it < n_iter; ++it) {
    cp_rows_kernel<<<nchunks, kCpThreads, rs, s>>>(a, kRowsAB);
    cp_small_kernel<<<nchrom, kCpThreads, small_smem, s>>>(a, kSmallB);
    cp_rows_kernel<<<nchunks, kCpThreads, rs, s>>>(a, kRowsD);
    cp_small_kernel<<<nchrom, kCpThreads, small_smem, s>>>(a, kSmallD);
    cp_rows_kernel<<<nchunks, kCpThreads, rs, s>>>(a, kRowsScale);
  }
  FH_CHECK_LAUNCH();
  return FH_OK;
}

// core[chrom] = ||[[A, B, D]]||^2 without changing the factors (parafac2_intergrative.py:621-632).
extern "C" int fh_core_norm(int32_t nchrom, int32_t nchunks, const int32_t* meta, float* A,
                            float* B, float* D, const float* Y, int32_t ld, int32_t rp,
                            int32_t R, int32_t ldy, double* core, void* workspace,
                            size_t workspace_bytes, int* status, void* stream) {
  return fh_cp_als(nchrom, nchunks, meta, A, B, D, Y, ld, rp, R, ldy, 0, core, nullptr,
                   workspace, workspace_bytes, status, stream);
}
