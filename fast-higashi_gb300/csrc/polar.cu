// Polar factors of the Procrustes steps.
//
// Reference: fasthigashi/project2orthogonal.py:6-34 returns U[:, :r] Vh of a thin SVD, the
// orthonormal polar factor of a tall matrix, and S; the driver uses it per bin row on
// temp_i = X_i lhs_i (n x r, parafac2_intergrative.py:396-417) and once per iteration on
// SVD_term^T (cells x R, :483-486).
//
// Per bin row (fp32, one CTA): the temp_i matrices of real fits are ill-conditioned
// (condition numbers 1e4 .. 5e6 on the reference's own inputs), so a Gram-matrix route in
// fp32 fails and an fp64 Gram with an fp32 apply is no better than the reference's fp32
// SVD.  The kernel factors temp_i = Q R by Householder QR and takes the polar factor of the
// small r x r triangle by the scaled Newton iteration X <- (z X + X^{-T} / z) / 2 (Higham;
// Frobenius-norm scaling z), then U = Q P.  On the reference's matrices this measured
// 1.5e-7 worst relative error against an fp64 SVD, against 1.2e-3 for the reference's own
// fp32 SVD.  sum(S) = trace(P^T R).
//
// Meta polar (fp64 where it is cheap): G = S^T S (R x R) accumulated in fp64 across the
// whole GPU, G = Rc^T Rc by fp64 Cholesky, P = polar(Rc) by the same Newton iteration,
// K = Rc^{-1} P in fp64, E = SVD_term^T K in fp64.  sum(S) = trace(P^T Rc).
#include "fh_common.cuh"

namespace fh {

constexpr int kPolThreads = 256;
constexpr int kNewtonMaxIt = 30;

struct PolarScratch {
  float* vh;     // [kMaxRank] Householder head v_k[k]
  float* beta;   // [kMaxRank]
  float* wv;     // [2 * kMaxRank] per-column dot products / pivot row
  float* fcol;   // [kMaxRank] pivot column
  float* red;    // [32]
  double* dred;  // [32]
  int* ival;     // [4]
};

// ---- Householder QR of T (n x r, row stride ldt, n >= r), in place ---------------------
// On return the upper triangle of T[0:r][0:r] is R, T[i][k] (i > k) holds v_k below the
// diagonal, vh[k] the head of v_k and beta[k] = 2 / v_k^T v_k (0 for a zero column).
__device__ void householder_qr(float* T, int n, int r, int ldt, PolarScratch& s) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nwarp = blockDim.x >> 5;
  for (int k = 0; k < r; ++k) {
    if (warp == 0) {
      float ss = 0.f;
      for (int i = k + 1 + lane; i < n; i += 32) ss = fmaf(T[i * ldt + k], T[i * ldt + k], ss);
      ss = warp_sum(ss);
      if (lane == 0) {
        const float x0 = T[k * ldt + k];
        const float s2 = fmaf(x0, x0, ss);
        if (s2 == 0.f) {
          s.beta[k] = 0.f; s.vh[k] = 0.f; s.wv[2 * kMaxRank - 1] = 0.f;
        } else {
          const float nrm = sqrtf(s2);
          const float alpha = x0 >= 0.f ? -nrm : nrm;
          s.vh[k] = x0 - alpha;
          s.beta[k] = 1.f / (s2 - x0 * alpha);
          s.wv[2 * kMaxRank - 1] = alpha;
        }
      }
    }
    __syncthreads();
    const float beta = s.beta[k], vh = s.vh[k];
    // w_j = v^T T[k:, j] for j > k
    for (int j = k + 1 + warp; j < r; j += nwarp) {
      float d = 0.f;
      for (int i = k + 1 + lane; i < n; i += 32) d = fmaf(T[i * ldt + k], T[i * ldt + j], d);
      d = warp_sum(d);
      if (lane == 0) s.wv[j] = fmaf(vh, T[k * ldt + j], d);
    }
    __syncthreads();
    const int nc = r - k - 1;
    if (beta != 0.f && nc > 0) {
      for (int idx = tid; idx < (n - k) * nc; idx += blockDim.x) {
        const int i = k + idx / nc, j = k + 1 + idx % nc;
        const float vi = (i == k) ? vh : T[i * ldt + k];
        T[i * ldt + j] = fmaf(-beta * vi, s.wv[j], T[i * ldt + j]);
      }
    }
    if (tid == 0) T[k * ldt + k] = s.wv[2 * kMaxRank - 1];
    __syncthreads();
  }
}

// ---- inverse of X (r x r, stride ldx) by Gauss-Jordan with partial pivoting ------------
// Aug: r x 2r scratch (stride 2r+1).  Result written to Xi (stride ldx).  Returns through
// s.ival[0] a nonzero flag if a zero pivot was met (the pivot is then nudged).
__device__ void gj_inverse(const float* X, int ldx, float* Xi, float* Aug, int r,
                           PolarScratch& s) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int la = 2 * r + 1, w2 = 2 * r;
  for (int idx = tid; idx < r * w2; idx += blockDim.x) {
    const int i = idx / w2, j = idx % w2;
    Aug[i * la + j] = j < r ? X[i * ldx + j] : (j - r == i ? 1.f : 0.f);
  }
  __syncthreads();
  for (int k = 0; k < r; ++k) {
    if (warp == 0) {
      // pivot search over rows k..r-1
      float best = -1.f;
      int bi = k;
      for (int i = k + lane; i < r; i += 32) {
        const float a = fabsf(Aug[i * la + k]);
        if (a > best) { best = a; bi = i; }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      // swap rows k and bi (columns k..2r-1)
      if (bi != k)
        for (int j = k + lane; j < w2; j += 32) {
          const float a = Aug[k * la + j];
          Aug[k * la + j] = Aug[bi * la + j];
          Aug[bi * la + j] = a;
        }
      __syncwarp();
      float piv = Aug[k * la + k];
      if (piv == 0.f) {
        piv = 1e-30f;
        if (lane == 0) s.ival[0] = 1;
      }
      for (int i = lane; i < r; i += 32) s.fcol[i] = Aug[i * la + k];
      __syncwarp();
      const float rp = 1.f / piv;
      for (int j = k + 1 + lane; j < w2; j += 32) {
        const float v = Aug[k * la + j] * rp;
        s.wv[j] = v;
        Aug[k * la + j] = v;
      }
    }
    __syncthreads();
    const int nc = w2 - k - 1;
    for (int idx = tid; idx < r * nc; idx += blockDim.x) {
      const int i = idx / nc, j = k + 1 + idx % nc;
      if (i != k) Aug[i * la + j] = fmaf(-s.fcol[i], s.wv[j], Aug[i * la + j]);
    }
    __syncthreads();
  }
  for (int idx = tid; idx < r * r; idx += blockDim.x) {
    const int i = idx / r, j = idx % r;
    Xi[i * ldx + j] = Aug[i * la + r + j];
  }
  __syncthreads();
}

// ---- polar factor of a square X (r x r, stride ldx) in place by scaled Newton ----------
// Xi: r x ldx scratch, Aug: r x (2r+1) scratch.
__device__ void newton_polar(float* X, int ldx, float* Xi, float* Aug, int r, PolarScratch& s) {
  const int tid = threadIdx.x;
  bool last = false;
  for (int it = 0; it < kNewtonMaxIt; ++it) {
    gj_inverse(X, ldx, Xi, Aug, r, s);
    float zeta = 1.f;
    if (!last) {
      float a = 0.f, b = 0.f;
      for (int idx = tid; idx < r * r; idx += blockDim.x) {
        const int i = idx / r, j = idx % r;
        a = fmaf(X[i * ldx + j], X[i * ldx + j], a);
        b = fmaf(Xi[i * ldx + j], Xi[i * ldx + j], b);
      }
      a = block_sum<float>(a, s.red);
      __syncthreads();
      b = block_sum<float>(b, s.red);
      zeta = sqrtf(sqrtf(b) / sqrtf(a));
      if (it >= 1 && fabsf(zeta - 1.f) < 1e-2f) zeta = 1.f;
    }
    // X_new = 0.5 (zeta X + Xi^T / zeta); measure the step
    float dn = 0.f, nn = 0.f;
    const float iz = 1.f / zeta;
    for (int idx = tid; idx < r * r; idx += blockDim.x) {
      const int i = idx / r, j = idx % r;
      const float xn = 0.5f * (zeta * X[i * ldx + j] + iz * Xi[j * ldx + i]);
      const float d = xn - X[i * ldx + j];
      dn = fmaf(d, d, dn);
      nn = fmaf(xn, xn, nn);
      Aug[idx] = xn;  // staged: X is still read through Xi^T by other threads
    }
    __syncthreads();
    for (int idx = tid; idx < r * r; idx += blockDim.x) X[(idx / r) * ldx + idx % r] = Aug[idx];
    dn = block_sum<float>(dn, s.red);
    __syncthreads();
    nn = block_sum<float>(nn, s.red);
    __syncthreads();
    if (last) break;
    if (sqrtf(dn) <= 1e-4f * sqrtf(nn)) last = true;
  }
}

// ---- U = Q [P; 0]: apply the stored reflectors in reverse to U (n x r, stride ldu) -----
__device__ void apply_q(const float* T, int ldt, float* U, int ldu, int n, int r,
                        PolarScratch& s) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nwarp = blockDim.x >> 5;
  for (int k = r - 1; k >= 0; --k) {
    const float beta = s.beta[k], vh = s.vh[k];
    if (beta == 0.f) continue;  // uniform across the block
    for (int j = warp; j < r; j += nwarp) {
      float d = 0.f;
      for (int i = k + 1 + lane; i < n; i += 32) d = fmaf(T[i * ldt + k], U[i * ldu + j], d);
      d = warp_sum(d);
      if (lane == 0) s.wv[j] = fmaf(vh, U[k * ldu + j], d);
    }
    __syncthreads();
    for (int idx = tid; idx < (n - k) * r; idx += blockDim.x) {
      const int i = k + idx / r, j = idx % r;
      const float vi = (i == k) ? vh : T[i * ldt + k];
      U[i * ldu + j] = fmaf(-beta * vi, s.wv[j], U[i * ldu + j]);
    }
    __syncthreads();
  }
}

// =========================================================================================
// Per bin row: M = D diag(A_g) B^T; temp = W_g M; U, sum(S) = polar(temp); Gt_g = U M^T.
// =========================================================================================
struct ProcArgs {
  const fh_tile* tiles;
  const int32_t* row_tile;
  const float* W;    // [band rows][RP]
  const float* A;    // [bin rows][lda]
  int lda;
  const float* B;    // [chrom][ldb][ldb]   (r x r used)
  int ldb;
  const float* D;    // [chrom][RP][ldb]    (R x r used, rows >= R zero)
  int R;
  float* U;          // tile-major (rows, width, rank)
  float* Gt;         // [band rows][RP]
  double* ssum;      // [bin rows]
  int* status;
  int from_u;        // 1: skip the polar step and take U_g from U (transform)
};

__host__ __device__ inline int proc_ldt(int r) { return r + 1; }

__host__ __device__ inline size_t proc_smem_floats(int n, int r, int rp) {
  const int ldt = proc_ldt(r);
  const size_t tm = (size_t)n * ldt;
  const size_t ms = (size_t)rp * ldt;
  size_t region = (size_t)n * ldt;                                  // U
  const size_t newton = (size_t)r * (2 * r + 1) + 2 * (size_t)r * ldt;  // Aug + X + Xi
  if (newton > region) region = newton;
  const size_t stage = 64 * (size_t)rp + (size_t)rp * ldt + (size_t)r * ldt;  // W chunk / DA + B
  if (stage > region) region = stage;
  return tm + ms + region + 5 * kMaxRank + 64;
}

template <int RP>
__global__ void __launch_bounds__(kPolThreads) procrustes_f32_kernel(ProcArgs a) {
  extern __shared__ __align__(16) float sm[];
  __shared__ float red[32];
  __shared__ double dred[32];
  __shared__ int ival[4];
  const int tid = threadIdx.x;
  const int64_t g = blockIdx.x;
  const fh_tile T = a.tiles[a.row_tile[g]];
  const int i = (int)(g - T.brow0);
  const int n = T.width, r = T.rank, ci = T.chrom, R = a.R;
  const int ldt = proc_ldt(r);
  float* Tm = sm;                        // n x ldt
  float* Ms = Tm + (size_t)n * ldt;      // RP x ldt
  float* reg = Ms + (size_t)RP * ldt;    // reused region
  float* misc = reg + (proc_smem_floats(n, r, RP) - (size_t)n * ldt - (size_t)RP * ldt -
                       5 * kMaxRank - 64);
  PolarScratch s{misc, misc + kMaxRank, misc + 2 * kMaxRank, misc + 4 * kMaxRank, red, dred,
                 ival};
  if (tid == 0) ival[0] = 0;

  // ---- M[m][l] = sum_rho D[m][rho] A_g[rho] B[l][rho]
  {
    float* DA = reg;                       // RP x ldt
    float* Bs = reg + (size_t)RP * ldt;    // r x ldt
    const float* Ag = a.A + g * a.lda;
    const float* Dc = a.D + (size_t)ci * RP * a.ldb;
    const float* Bc = a.B + (size_t)ci * a.ldb * a.ldb;
    for (int idx = tid; idx < RP * r; idx += kPolThreads) {
      const int m = idx / r, rho = idx % r;
      DA[m * ldt + rho] = m < R ? Dc[m * a.ldb + rho] * Ag[rho] : 0.f;
    }
    for (int idx = tid; idx < r * r; idx += kPolThreads) {
      const int l = idx / r, rho = idx % r;
      Bs[l * ldt + rho] = Bc[l * a.ldb + rho];
    }
    __syncthreads();
    for (int idx = tid; idx < RP * r; idx += kPolThreads) {
      const int m = idx / r, l = idx % r;
      float acc = 0.f;
      for (int rho = 0; rho < r; ++rho) acc = fmaf(DA[m * ldt + rho], Bs[l * ldt + rho], acc);
      Ms[m * ldt + l] = acc;
    }
    __syncthreads();
  }
  if (a.from_u) {
    // Gt_g = U_g M^T with the stored projection (parafac2_intergrative.py:772-801)
    const float* Ug = a.U + T.uoff + (int64_t)i * n * r;
    float* Uu = reg;
    for (int idx = tid; idx < n * r; idx += kPolThreads) Uu[(idx / r) * ldt + idx % r] = Ug[idx];
    __syncthreads();
    float* Gg = a.Gt + (T.xoff + (int64_t)i * n) * RP;
    for (int idx = tid; idx < n * RP; idx += kPolThreads) {
      const int j = idx / RP, m = idx % RP;
      float acc = 0.f;
      for (int l = 0; l < r; ++l) acc = fmaf(Uu[j * ldt + l], Ms[m * ldt + l], acc);
      Gg[idx] = acc;
    }
    return;
  }
  // ---- temp = W_g M  (n x r), W staged 64 rows at a time
  {
    const float* Wg = a.W + (T.xoff + (int64_t)i * n) * RP;
    float* Ws = reg;  // 64 x RP
    for (int j0 = 0; j0 < n; j0 += 64) {
      const int jn = min(64, n - j0);
      for (int idx = tid; idx < jn * RP; idx += kPolThreads) Ws[idx] = Wg[(int64_t)j0 * RP + idx];
      __syncthreads();
      for (int idx = tid; idx < jn * r; idx += kPolThreads) {
        const int jj = idx / r, l = idx % r;
        float acc = 0.f;
#pragma unroll 8
        for (int m = 0; m < RP; ++m) acc = fmaf(Ws[jj * RP + m], Ms[m * ldt + l], acc);
        Tm[(j0 + jj) * ldt + l] = acc;
      }
      __syncthreads();
    }
  }
  // ---- QR, then polar factor of R by Newton
  householder_qr(Tm, n, r, ldt, s);
  float* X = reg;                         // r x ldt
  float* Xi = reg + (size_t)r * ldt;      // r x ldt
  float* Aug = reg + 2 * (size_t)r * ldt; // r x (2r+1)
  for (int idx = tid; idx < r * r; idx += kPolThreads) {
    const int p = idx / r, q = idx % r;
    X[p * ldt + q] = q >= p ? Tm[p * ldt + q] : 0.f;
  }
  __syncthreads();
  newton_polar(X, ldt, Xi, Aug, r, s);
  // ---- sum(S) = trace(P^T R) (fp64)
  {
    double acc = 0.0;
    for (int idx = tid; idx < r * r; idx += kPolThreads) {
      const int p = idx / r, q = idx % r;
      if (q >= p) acc += (double)X[p * ldt + q] * (double)Tm[p * ldt + q];
    }
    acc = block_sum<double>(acc, dred);
    if (tid == 0) a.ssum[g] = acc;
  }
  // ---- U = Q [P; 0]  (U occupies the region from its start; X sits behind it)
  float* Uu = reg;  // n x ldt
  {
    // move P to the top of U: U rows [0, r) overlap X rows only when ldt*r > 0 => copy via
    // registers in two passes (X lives at reg, so U's first r rows ARE X's storage).
    for (int idx = tid; idx < (n - r) * ldt; idx += kPolThreads) Uu[(size_t)r * ldt + idx] = 0.f;
    __syncthreads();
    // U[0:r] already equals X (same storage and stride); clear the padding column
  }
  apply_q(Tm, ldt, Uu, ldt, n, r, s);
  // ---- write U_g (n x r) and Gt_g[j][m] = sum_l U[j][l] M[m][l]
  float* Ug = a.U + T.uoff + (int64_t)i * n * r;
  for (int idx = tid; idx < n * r; idx += kPolThreads) Ug[idx] = Uu[(idx / r) * ldt + idx % r];
  float* Gg = a.Gt + (T.xoff + (int64_t)i * n) * RP;
  for (int idx = tid; idx < n * RP; idx += kPolThreads) {
    const int j = idx / RP, m = idx % RP;
    float acc = 0.f;
    for (int l = 0; l < r; ++l) acc = fmaf(Uu[j * ldt + l], Ms[m * ldt + l], acc);
    Gg[idx] = acc;
  }
  if (tid == 0 && ival[0]) set_status(a.status, FH_ERR_ILLCOND);
}

// =========================================================================================
// Drop-in batched polar factor (project2orthogonal on a (batch, n, r) tensor, n >= r).
// =========================================================================================
__global__ void __launch_bounds__(kPolThreads) polar_batched_kernel(const float* __restrict__ M,
                                                                    int n, int r,
                                                                    float* __restrict__ U,
                                                                    double* __restrict__ ssum,
                                                                    int* status) {
  extern __shared__ __align__(16) float sm[];
  __shared__ float red[32];
  __shared__ double dred[32];
  __shared__ int ival[4];
  const int tid = threadIdx.x;
  const int64_t b = blockIdx.x;
  const int ldt = proc_ldt(r);
  float* Tm = sm;
  float* reg = Tm + (size_t)n * ldt;
  size_t regsz = (size_t)n * ldt;
  const size_t newton = (size_t)r * (2 * r + 1) + 2 * (size_t)r * ldt;
  if (newton > regsz) regsz = newton;
  float* misc = reg + regsz;
  PolarScratch s{misc, misc + kMaxRank, misc + 2 * kMaxRank, misc + 4 * kMaxRank, red, dred,
                 ival};
  if (tid == 0) ival[0] = 0;
  const float* Mb = M + b * (int64_t)n * r;
  for (int idx = tid; idx < n * r; idx += kPolThreads) Tm[(idx / r) * ldt + idx % r] = Mb[idx];
  __syncthreads();
  householder_qr(Tm, n, r, ldt, s);
  float* X = reg;
  float* Xi = reg + (size_t)r * ldt;
  float* Aug = reg + 2 * (size_t)r * ldt;
  for (int idx = tid; idx < r * r; idx += kPolThreads) {
    const int p = idx / r, q = idx % r;
    X[p * ldt + q] = q >= p ? Tm[p * ldt + q] : 0.f;
  }
  __syncthreads();
  newton_polar(X, ldt, Xi, Aug, r, s);
  double acc = 0.0;
  for (int idx = tid; idx < r * r; idx += kPolThreads) {
    const int p = idx / r, q = idx % r;
    if (q >= p) acc += (double)X[p * ldt + q] * (double)Tm[p * ldt + q];
  }
  acc = block_sum<double>(acc, dred);
  if (tid == 0 && ssum) ssum[b] = acc;
  for (int idx = tid; idx < (n - r) * ldt; idx += kPolThreads) reg[(size_t)r * ldt + idx] = 0.f;
  __syncthreads();
  apply_q(Tm, ldt, reg, ldt, n, r, s);
  float* Ub = U + b * (int64_t)n * r;
  for (int idx = tid; idx < n * r; idx += kPolThreads) Ub[idx] = reg[(idx / r) * ldt + idx % r];
  if (tid == 0 && ival[0]) set_status(status, FH_ERR_ILLCOND);
}

// =========================================================================================
// Meta polar: E = polar(S), S = SVD_term^T (cells x R, stride RP).
// =========================================================================================
constexpr int kGramCells = 16;

// partial[blk][a][b] = sum_{c in blk} S[c][a] S[c][b]  (fp64, upper triangle a <= b)
__global__ void __launch_bounds__(256) meta_gram_kernel(const float* __restrict__ S, int C, int R,
                                                        int RP, double* __restrict__ partial) {
  __shared__ double Ss[kGramCells][kMaxRank];
  const int c0 = blockIdx.x * kGramCells;
  const int nc = min(kGramCells, C - c0);
  for (int idx = threadIdx.x; idx < kGramCells * R; idx += blockDim.x) {
    const int cc = idx / R, m = idx % R;
    Ss[cc][m] = cc < nc ? (double)S[(int64_t)(c0 + cc) * RP + m] : 0.0;
  }
  __syncthreads();
  double* out = partial + (int64_t)blockIdx.x * R * R;
  for (int idx = threadIdx.x; idx < R * R; idx += blockDim.x) {
    const int p = idx / R, q = idx % R;
    if (q < p) continue;
    double acc = 0.0;
    for (int cc = 0; cc < nc; ++cc) acc = fma(Ss[cc][p], Ss[cc][q], acc);
    out[idx] = acc;
  }
}

__global__ void meta_gram_reduce_kernel(const double* __restrict__ partial, int blocks, int R,
                                        double* __restrict__ G) {
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < R * R;
       idx += gridDim.x * blockDim.x) {
    const int p = idx / R, q = idx % R;
    if (q < p) continue;
    double s = 0.0;
    for (int k = 0; k < blocks; ++k) s += partial[(int64_t)k * R * R + idx];
    G[p * R + q] = s;
    G[q * R + p] = s;
  }
}

// One CTA: Cholesky (fp64), Newton polar of Rc (fp32), sum(S), K = Rc^{-1} P (fp64).
__global__ void __launch_bounds__(kPolThreads) meta_small_kernel(const double* __restrict__ Gg,
                                                                 int R, double* __restrict__ K,
                                                                 double* __restrict__ ssum_out,
                                                                 int* status) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ float red[32];
  __shared__ double dred[32];
  __shared__ int ival[4];
  const int tid = threadIdx.x;
  double* G = reinterpret_cast<double*>(smraw);     // R x R (becomes Rc, upper)
  float* fbase = reinterpret_cast<float*>(G + (size_t)R * R);
  const int ldt = R + 1;
  float* X = fbase;
  float* Xi = X + (size_t)R * ldt;
  float* Aug = Xi + (size_t)R * ldt;
  float* misc = Aug + (size_t)R * (2 * R + 1);
  PolarScratch s{misc, misc + kMaxRank, misc + 2 * kMaxRank, misc + 4 * kMaxRank, red, dred,
                 ival};
  if (tid == 0) ival[0] = 0;
  for (int idx = tid; idx < R * R; idx += kPolThreads) G[idx] = Gg[idx];
  __syncthreads();
  // right-looking Cholesky: G = Rc^T Rc, Rc upper, stored in G's upper triangle
  for (int k = 0; k < R; ++k) {
    if (tid == 0) {
      double d = G[k * R + k];
      if (!(d > 0.0)) {
        ival[0] = 1;
        d = 1e-300;
      }
      G[k * R + k] = sqrt(d);
    }
    __syncthreads();
    const double dk = G[k * R + k];
    for (int j = k + 1 + tid; j < R; j += kPolThreads) G[k * R + j] /= dk;
    __syncthreads();
    const int nc = R - k - 1;
    for (int idx = tid; idx < nc * nc; idx += kPolThreads) {
      const int p = k + 1 + idx / nc, q = k + 1 + idx % nc;
      if (q >= p) G[p * R + q] -= G[k * R + p] * G[k * R + q];
    }
    __syncthreads();
  }
  for (int idx = tid; idx < R * R; idx += kPolThreads) {
    const int p = idx / R, q = idx % R;
    X[p * ldt + q] = q >= p ? (float)G[p * R + q] : 0.f;
  }
  __syncthreads();
  newton_polar(X, ldt, Xi, Aug, R, s);
  double acc = 0.0;
  for (int idx = tid; idx < R * R; idx += kPolThreads) {
    const int p = idx / R, q = idx % R;
    if (q >= p) acc += (double)X[p * ldt + q] * G[p * R + q];
  }
  acc = block_sum<double>(acc, dred);
  if (tid == 0) *ssum_out = acc;
  // K = Rc^{-1} P by back substitution, one column per thread
  for (int j = tid; j < R; j += kPolThreads) {
    for (int p = R - 1; p >= 0; --p) {
      double v = (double)X[p * ldt + j];
      for (int l = p + 1; l < R; ++l) v -= G[p * R + l] * K[l * R + j];
      K[p * R + j] = v / G[p * R + p];
    }
  }
  if (tid == 0 && ival[0]) set_status(status, FH_ERR_ILLCOND);
}

// E[c][m] = sum_l S[c][l] K[l][m] (fp64 accumulate), m >= R written as zero.
__global__ void __launch_bounds__(256) meta_apply_kernel(const float* __restrict__ S, int C, int R,
                                                         int RP, const double* __restrict__ K,
                                                         float* __restrict__ E) {
  __shared__ double Ks[64 * 64];  // R <= 64 here
  for (int idx = threadIdx.x; idx < R * R; idx += blockDim.x) Ks[idx] = K[idx];
  __syncthreads();
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < (int64_t)C * RP;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = idx / RP;
    const int m = (int)(idx % RP);
    double acc = 0.0;
    if (m < R) {
      const float* sr = S + c * RP;
      for (int l = 0; l < R; ++l) acc = fma((double)sr[l], Ks[l * R + m], acc);
    }
    E[idx] = (float)acc;
  }
}

// Singular values of M (n x r) given its polar factor U: the eigenvalues of the symmetric
// H = U^T M, by cyclic Jacobi with a round-robin pair schedule (one CTA per matrix), sorted
// in descending order.  Serves the S output of the project2orthogonal drop-in.
__global__ void __launch_bounds__(kPolThreads) polar_svals_kernel(const float* __restrict__ M,
                                                                  const float* __restrict__ U,
                                                                  int n, int r,
                                                                  float* __restrict__ S) {
  extern __shared__ __align__(16) float hs[];
  __shared__ float red[32];
  __shared__ float cs[kMaxRank / 2 + 1], sn[kMaxRank / 2 + 1];
  __shared__ int pp[kMaxRank / 2 + 1], qq[kMaxRank / 2 + 1];
  __shared__ int stop;
  const int tid = threadIdx.x;
  const int64_t b = blockIdx.x;
  const int m = r + (r & 1);     // even size for the schedule (a zero row/column if odd)
  const int ld = m + 1;
  float* H = hs;
  const float* Mb = M + b * (int64_t)n * r;
  const float* Ub = U + b * (int64_t)n * r;
  for (int idx = tid; idx < m * m; idx += kPolThreads) {
    const int i = idx / m, j = idx % m;
    float acc = 0.f;
    if (i < r && j < r)
      for (int k = 0; k < n; ++k) acc = fmaf(Ub[(int64_t)k * r + i], Mb[(int64_t)k * r + j], acc);
    H[i * ld + j] = acc;
  }
  __syncthreads();
  for (int idx = tid; idx < m * m; idx += kPolThreads) {   // symmetrize
    const int i = idx / m, j = idx % m;
    if (i < j) {
      const float v = 0.5f * (H[i * ld + j] + H[j * ld + i]);
      H[i * ld + j] = v;
      H[j * ld + i] = v;
    }
  }
  __syncthreads();
  for (int sweep = 0; sweep < 30; ++sweep) {
    float off = 0.f, tot = 0.f;
    for (int idx = tid; idx < m * m; idx += kPolThreads) {
      const float v = H[(idx / m) * ld + idx % m];
      tot = fmaf(v, v, tot);
      if (idx / m != idx % m) off = fmaf(v, v, off);
    }
    off = block_sum<float>(off, red);
    __syncthreads();
    tot = block_sum<float>(tot, red);
    if (tid == 0) stop = !(off > 1e-14f * tot);
    __syncthreads();
    if (stop) break;
    for (int round = 0; round < m - 1; ++round) {
      if (tid < m / 2) {
        // round-robin: position 0 fixed, the rest rotate
        const int a = tid == 0 ? 0 : 1 + (tid - 1 + round) % (m - 1);
        const int bb = 1 + (m - 2 - tid + round) % (m - 1);
        const int p = min(a, bb), q = max(a, bb);
        pp[tid] = p; qq[tid] = q;
        const float apq = H[p * ld + q];
        float c = 1.f, s2 = 0.f;
        if (apq != 0.f) {
          const float theta = 0.5f * (H[q * ld + q] - H[p * ld + p]) / apq;
          const float t = (theta >= 0.f ? 1.f : -1.f) / (fabsf(theta) + sqrtf(1.f + theta * theta));
          c = rsqrtf(1.f + t * t);
          s2 = t * c;
        }
        cs[tid] = c; sn[tid] = s2;
      }
      __syncthreads();
      for (int idx = tid; idx < (m / 2) * m; idx += kPolThreads) {   // rows p, q
        const int k = idx / m, j = idx % m;
        const int p = pp[k], q = qq[k];
        const float hp = H[p * ld + j], hq = H[q * ld + j];
        H[p * ld + j] = cs[k] * hp - sn[k] * hq;
        H[q * ld + j] = sn[k] * hp + cs[k] * hq;
      }
      __syncthreads();
      for (int idx = tid; idx < (m / 2) * m; idx += kPolThreads) {   // columns p, q
        const int k = idx / m, i = idx % m;
        const int p = pp[k], q = qq[k];
        const float hp = H[i * ld + p], hq = H[i * ld + q];
        H[i * ld + p] = cs[k] * hp - sn[k] * hq;
        H[i * ld + q] = sn[k] * hp + cs[k] * hq;
      }
      __syncthreads();
    }
  }
  if (tid == 0) {
    // insertion sort of the diagonal, descending (r <= 128)
    float* out = S + b * r;
    int cnt = 0;
    for (int i = 0; i < r; ++i) {
      const float v = H[i * ld + i];
      int j = cnt++;
      while (j > 0 && out[j - 1] < v) { out[j] = out[j - 1]; --j; }
      out[j] = v;
    }
  }
}

}  // namespace fh

using namespace fh;

extern "C" int fh_polar_svals_f32(const float* M, const float* U, int64_t batch, int32_t n,
                                  int32_t r, float* S, void* stream) {
  if (!M || !U || !S || batch <= 0 || n < r || r <= 0) return FH_ERR_ARG;
  if (r > kMaxRank) return FH_ERR_UNSUPPORTED;
  const int m = r + (r & 1);
  const size_t smem = (size_t)m * (m + 1) * sizeof(float);
  if (ensure_smem((const void*)polar_svals_kernel, smem)) return FH_ERR_LAUNCH;
  polar_svals_kernel<<<(unsigned)batch, kPolThreads, smem, (cudaStream_t)stream>>>(M, U, n, r, S);
  FH_CHECK_LAUNCH();
  return FH_OK;
}

extern "C" size_t fh_procrustes_smem(int32_t n, int32_t r, int32_t rp) {
  return proc_smem_floats(n, r, rp) * sizeof(float);
}

static int procrustes_launch(const fh_tile* tiles, const int32_t* row_tile, int64_t n_rows,
                             int32_t max_width, int32_t max_rank, const float* W,
                             const float* A, int32_t lda, const float* B, const float* D,
                             int32_t ldb, int32_t R, int32_t rp, float* U, float* Gt,
                             double* ssum, int* status, void* stream, int from_u) {
  if (!tiles || !row_tile || !A || !B || !D || !U || !Gt || n_rows <= 0) return FH_ERR_ARG;
  if (!from_u && (!W || !ssum)) return FH_ERR_ARG;
  if (max_rank > 64 || rp > 64 || R > rp || max_width > kMaxWidth || max_rank > ldb ||
      max_rank > lda)
    return FH_ERR_UNSUPPORTED;
  const size_t smem = proc_smem_floats(max_width, max_rank, rp) * sizeof(float);
  if (smem > 227 * 1024) return FH_ERR_UNSUPPORTED;
  ProcArgs a{tiles, row_tile, W, A, lda, B, ldb, D, R, U, Gt, ssum, status, from_u};
  cudaStream_t s = (cudaStream_t)stream;
#define FH_PROC(RPV)                                                                        \
  case RPV: {                                                                               \
    auto k = procrustes_f32_kernel<RPV>;                                                    \
    if (ensure_smem((const void*)k, smem))    \
      return FH_ERR_LAUNCH;                                                                 \
    k<<<(unsigned)n_rows, kPolThreads, smem, s>>>(a);                                       \
    break;                                                                                  \
  }
  switch (rp) {
    FH_PROC(16)
    FH_PROC(32)
    FH_PROC(64)
    default: return FH_ERR_ARG;
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
  return procrustes_launch(tiles, row_tile, n_rows, max_width, max_rank, W, A, lda, B, D, ldb,
                           R, rp, U, Gt, ssum, status, stream, 0);
}

extern "C" int fh_projection_g_f32(const fh_tile* tiles, const int32_t* row_tile, int64_t n_rows,
                                   int32_t max_width, int32_t max_rank, const float* A,
                                   int32_t lda, const float* B, const float* D, int32_t ldb,
                                   int32_t R, int32_t rp, const float* U, float* Gt,
                                   void* stream) {
  return procrustes_launch(tiles, row_tile, n_rows, max_width, max_rank, nullptr, A, lda, B, D,
                           ldb, R, rp, const_cast<float*>(U), Gt, nullptr, nullptr, stream, 1);
}

extern "C" int fh_polar_f32(const float* M, int64_t batch, int32_t n, int32_t r, float* U,
                            double* ssum, int* status, void* stream) {
  if (!M || !U || batch <= 0 || n < r || r <= 0) return FH_ERR_ARG;
  if (r > 64 || n > kMaxWidth) return FH_ERR_UNSUPPORTED;
  const int ldt = proc_ldt(r);
  size_t regsz = (size_t)n * ldt;
  const size_t newton = (size_t)r * (2 * r + 1) + 2 * (size_t)r * ldt;
  if (newton > regsz) regsz = newton;
  const size_t smem = ((size_t)n * ldt + regsz + 5 * kMaxRank + 64) * sizeof(float);
  if (smem > 227 * 1024) return FH_ERR_UNSUPPORTED;
  if (ensure_smem((const void*)polar_batched_kernel, smem))
    return FH_ERR_LAUNCH;
  polar_batched_kernel<<<(unsigned)batch, kPolThreads, smem, (cudaStream_t)stream>>>(
      M, n, r, U, ssum, status);
  FH_CHECK_LAUNCH();
  return FH_OK;
}

extern "C" size_t fh_meta_polar_workspace(int32_t n_cells, int32_t R) {
  const int64_t blocks = ceil_div(n_cells, kGramCells);
  return (size_t)(blocks + 2) * R * R * sizeof(double);
}

extern "C" int fh_meta_polar(const float* S, int32_t n_cells, int32_t R, int32_t rp, float* E,
                             double* ssum, void* workspace, size_t workspace_bytes, int* status,
                             void* stream) {
  if (!S || !E || !ssum || !workspace || n_cells <= 0 || R <= 0 || R > rp) return FH_ERR_ARG;
  if (R > 64) return FH_ERR_UNSUPPORTED;
  if (workspace_bytes < fh_meta_polar_workspace(n_cells, R)) return FH_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int blocks = (int)ceil_div(n_cells, kGramCells);
  double* partial = (double*)workspace;
  double* G = partial + (size_t)blocks * R * R;
  double* K = G + (size_t)R * R;
  meta_gram_kernel<<<blocks, 256, 0, s>>>(S, n_cells, R, rp, partial);
  meta_gram_reduce_kernel<<<(R * R + 255) / 256, 256, 0, s>>>(partial, blocks, R, G);
  const int ldt = R + 1;
  const size_t smem = (size_t)R * R * sizeof(double) +
                      ((size_t)2 * R * ldt + (size_t)R * (2 * R + 1) + 5 * kMaxRank + 64) *
                          sizeof(float);
  if (ensure_smem((const void*)meta_small_kernel, smem))
    return FH_ERR_LAUNCH;
  meta_small_kernel<<<1, kPolThreads, smem, s>>>(G, R, K, ssum, status);
  const int64_t total = (int64_t)n_cells * rp;
  int grid = (int)ceil_div(total, 256);
  if (grid > 152 * 8) grid = 152 * 8;
  meta_apply_kernel<<<grid, 256, 0, s>>>(S, n_cells, R, rp, K, E);
  FH_CHECK_LAUNCH();
  return FH_OK;
}
