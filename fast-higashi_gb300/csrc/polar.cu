// Meta-embedding polar factor (once per ALS iteration).
//
// Reference: fasthigashi/project2orthogonal.py:6-34 returns U[:, :r] Vh of a thin SVD, the
// orthonormal polar factor, and S; the driver applies it to SVD_term^T (cells x R,
// parafac2_intergrative.py:483-486).  The per-bin-row polar factors are in jacobi.cu.
//
// The matrix is tall (cells x R) and its condition number reaches ~5e3, so the route keeps
// the squared-conditioned steps in fp64 and works in fp64 where the work is O(R^2) per
// cell or O(R^3) once: G = S^T S (R x R) accumulated in fp64 across the whole GPU,
// G = Rc^T Rc by fp64 Cholesky, P = polar(Rc) (R x R, well inside fp32's reach) by the
// scaled Newton iteration X <- (z X + X^{-T} / z) / 2 (Higham; Frobenius-norm scaling z),
// K = Rc^{-1} P in fp64, E = SVD_term^T K in fp64.  sum(S) = trace(P^T Rc).
#include "polar_common.cuh"

namespace fh {

constexpr int kPolThreads = 512;

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

// Bytes before the misc floats of meta_small_kernel for R > 64: G (fp64), later reused by the
// iterate and its scratch ((R + 4) rows each at stride ldv).
__host__ __device__ inline size_t meta_big_body_bytes(int R) {
  const int ldv = ((R + 3) & ~3) + 4;
  const size_t g = (size_t)R * R * sizeof(double);
  const size_t it = 2 * (size_t)(R + 4) * ldv * sizeof(float);
  return g > it ? g : it;
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
  float* Aug = X + (size_t)R * ldt;
  float* misc = Aug + newton_scratch_floats(R);
  if (R > 64) misc = reinterpret_cast<float*>(smraw + meta_big_body_bytes(R));
  PolarScratch s = polar_scratch(misc, red, dred, ival);
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
  if (R > 64) {
    // R <= 128: Rc goes out to K first, then the iterate and its scratch (stride ldv) take
    // the shared memory G used; P = polar(Rc) by the 4 x 8-tiled iteration
    for (int idx = tid; idx < R * R; idx += kPolThreads) {
      const int p = idx / R, q = idx % R;
      K[R * R + idx] = q >= p ? G[idx] : 0.0;
    }
    __syncthreads();
    const int ldv = ((R + 3) & ~3) + 4;
    float* Xv = reinterpret_cast<float*>(smraw);
    float* Sv = Xv + (size_t)(R + 4) * ldv;
    const double* Rg = K + (size_t)R * R;
    for (int idx = tid; idx < R * R; idx += kPolThreads) {
      const int p = idx / R, q = idx % R;
      Xv[p * ldv + q] = (float)Rg[idx];
    }
    __syncthreads();
    newton_polar_tiled<8>(Xv, ldv, Sv, R, s);
    double acc = 0.0;
    for (int idx = tid; idx < R * R; idx += kPolThreads) {
      const int p = idx / R, q = idx % R;
      if (q >= p) acc += (double)Xv[p * ldv + q] * Rg[idx];
    }
    acc = block_sum<double>(acc, dred);
    if (tid == 0) *ssum_out = acc;
    for (int idx = tid; idx < R * R; idx += kPolThreads)
      K[idx] = (double)Xv[(idx / R) * ldv + idx % R];   // P, overwritten by K column by column
    if (tid == 0 && ival[0]) set_status(status, FH_ERR_ILLCOND);
    return;
  }
  for (int idx = tid; idx < R * R; idx += kPolThreads) {
    const int p = idx / R, q = idx % R;
    X[p * ldt + q] = q >= p ? (float)G[p * R + q] : 0.f;
  }
  __syncthreads();
  newton_polar_r64(X, ldt, Aug, R, true, s);
  double acc = 0.0;
  for (int idx = tid; idx < R * R; idx += kPolThreads) {
    const int p = idx / R, q = idx % R;
    if (q >= p) acc += (double)X[p * ldt + q] * G[p * R + q];
  }
  acc = block_sum<double>(acc, dred);
  if (tid == 0) *ssum_out = acc;
  // export Rc (upper, fp64) and P (fp32) for the column solves
  for (int idx = tid; idx < R * R; idx += kPolThreads) {
    const int p = idx / R, q = idx % R;
    K[R * R + idx] = q >= p ? G[idx] : 0.0;     // Rc
    K[idx] = (double)X[p * ldt + q];            // P, overwritten by K column by column
  }
  if (tid == 0 && ival[0]) set_status(status, FH_ERR_ILLCOND);
}

// K[:, j] = Rc^{-1} P[:, j] by back substitution, one warp (CTA) per column, fp64.
// KR: [0, R*R) holds P on entry and K on exit; [R*R, 2R*R) holds Rc.
__global__ void __launch_bounds__(32) meta_ksolve_kernel(double* __restrict__ KR, int R) {
  const int j = blockIdx.x, lane = threadIdx.x;
  const double* Rc = KR + (size_t)R * R;
  double* K = KR;
  for (int p = R - 1; p >= 0; --p) {
    double s = 0.0;
    for (int l = p + 1 + lane; l < R; l += 32) s = fma(Rc[p * R + l], K[l * R + j], s);
    s = warp_sum(s);
    if (lane == 0) K[p * R + j] = (K[p * R + j] - s) / Rc[p * R + p];
    __syncwarp();
  }
}

// E[c][m] = sum_l S[c][l] K[l][m] (fp64 accumulate), m >= R written as zero.
__global__ void __launch_bounds__(256) meta_apply_kernel(const float* __restrict__ S, int C, int R,
                                                         int RP, const double* __restrict__ K,
                                                         float* __restrict__ E) {
  extern __shared__ double Ks[];  // R x R
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

}  // namespace fh

using namespace fh;

extern "C" size_t fh_meta_polar_workspace(int32_t n_cells, int32_t R) {
  const int64_t blocks = ceil_div(n_cells, kGramCells);
  return (size_t)(blocks + 3) * R * R * sizeof(double);
}

extern "C" int fh_meta_polar(const float* S, int32_t n_cells, int32_t R, int32_t rp, float* E,
                             double* ssum, void* workspace, size_t workspace_bytes, int* status,
                             void* stream) {
  if (!S || !E || !ssum || !workspace || n_cells <= 0 || R <= 0 || R > rp) return FH_ERR_ARG;
  if (R > kMaxRank) return FH_ERR_UNSUPPORTED;
  if (workspace_bytes < fh_meta_polar_workspace(n_cells, R)) return FH_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int blocks = (int)ceil_div(n_cells, kGramCells);
  double* partial = (double*)workspace;
  double* G = partial + (size_t)blocks * R * R;
  double* K = G + (size_t)R * R;
  meta_gram_kernel<<<blocks, 256, 0, s>>>(S, n_cells, R, rp, partial);
  meta_gram_reduce_kernel<<<(R * R + 255) / 256, 256, 0, s>>>(partial, blocks, R, G);
  const int ldt = R + 1;
  size_t smem = (size_t)R * R * sizeof(double) +
                ((size_t)R * ldt + newton_scratch_floats(R) + kPolarMiscFloats) * sizeof(float);
  if (R > 64)   // G, then the iterate and scratch in the same bytes, then the misc floats
    smem = meta_big_body_bytes(R) + (size_t)kPolarMiscFloats * sizeof(float);
  if (smem > 227 * 1024) return FH_ERR_UNSUPPORTED;
  if (ensure_smem((const void*)meta_small_kernel, smem))
    return FH_ERR_LAUNCH;
  meta_small_kernel<<<1, kPolThreads, smem, s>>>(G, R, K, ssum, status);
  meta_ksolve_kernel<<<R, 32, 0, s>>>(K, R);
  const int64_t total = (int64_t)n_cells * rp;
  int grid = (int)ceil_div(total, 256);
  if (grid > 152 * 8) grid = 152 * 8;
  const size_t ksmem = (size_t)R * R * sizeof(double);
  if (ensure_smem((const void*)meta_apply_kernel, ksmem)) return FH_ERR_LAUNCH;
  meta_apply_kernel<<<grid, 256, ksmem, s>>>(S, n_cells, R, rp, K, E);
  FH_CHECK_LAUNCH();
  return FH_OK;
}
