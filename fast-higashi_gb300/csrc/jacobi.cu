// Singular values of small matrices by one-sided Jacobi (fp32), for the S output of the
// project2orthogonal drop-in (project2orthogonal.py:6-34 returns S with the polar factor).
//
// With U the polar factor of M (n x r), H = U^T M is symmetric positive semidefinite and
// its singular values are those of M.  One-sided Jacobi rotates pairs of columns of H (a
// round-robin schedule, one warp per pair, one barrier per round) until they are
// orthogonal; the column norms are then the singular values.
#include "fh_common.cuh"

namespace fh {

constexpr int kJacThreads = 512;
constexpr int kJacWarps = kJacThreads / 32;
constexpr int kJacMaxSweeps = 24;
constexpr float kJacTol = 1e-6f;   // rotate a pair while |<t_p, t_q>| > tol ||t_p|| ||t_q||

__host__ __device__ inline int jac_ldn(int n) { return n | 1; }   // odd column stride
__host__ __device__ inline int jac_m(int r) { return r + (r & 1); }

__device__ __forceinline__ void rr_pair(int k, int rnd, int m, int& p, int& q) {
  const int a = k == 0 ? 0 : 1 + (k - 1 + rnd) % (m - 1);
  const int b = 1 + (m - 2 - k + rnd) % (m - 1);
  p = min(a, b);
  q = max(a, b);
}

// One-sided Jacobi on the columns of Tt (m columns of length n, stride ldn) accumulating the
// rotations into the columns of Vt (length r, stride ldv).  Returns the sweeps run.
__device__ int jacobi_columns(float* Tt, int ldn, int n, float* Vt, int ldv, int r, float* red) {
  const int m = jac_m(r);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int sweep = 0;
  for (; sweep < kJacMaxSweeps; ++sweep) {
    float mx = 0.f;
    for (int rnd = 0; rnd < m - 1; ++rnd) {
      for (int k = warp; k < m / 2; k += kJacWarps) {
        int p, q;
        rr_pair(k, rnd, m, p, q);
        float* tp = Tt + p * ldn;
        float* tq = Tt + q * ldn;
        float a = 0.f, b = 0.f, g = 0.f;
        for (int i = lane; i < n; i += 32) {
          const float x = tp[i], y = tq[i];
          a = fmaf(x, x, a);
          b = fmaf(y, y, b);
          g = fmaf(x, y, g);
        }
        a = warp_sum(a);
        b = warp_sum(b);
        g = warp_sum(g);
        if (a > 0.f && b > 0.f) {
          const float rel = fabsf(g) / sqrtf(a * b);
          mx = fmaxf(mx, rel);
          if (rel > kJacTol) {
            const float zeta = (b - a) / (2.f * g);
            const float t = (zeta >= 0.f ? 1.f : -1.f) / (fabsf(zeta) + sqrtf(1.f + zeta * zeta));
            const float c = 1.f / sqrtf(1.f + t * t);
            const float s = c * t;
            for (int i = lane; i < n; i += 32) {
              const float x = tp[i], y = tq[i];
              tp[i] = c * x - s * y;
              tq[i] = s * x + c * y;
            }
            float* vp = Vt + p * ldv;
            float* vq = Vt + q * ldv;
            for (int i = lane; i < r; i += 32) {
              const float x = vp[i], y = vq[i];
              vp[i] = c * x - s * y;
              vq[i] = s * x + c * y;
            }
          }
        }
      }
      __syncthreads();
    }
    // block max of the largest relative off-orthogonality seen in this sweep
    if (lane == 0) red[warp] = mx;
    __syncthreads();
    float bm = 0.f;
    for (int w = 0; w < kJacWarps; ++w) bm = fmaxf(bm, red[w]);
    __syncthreads();
    if (bm <= kJacTol) { ++sweep; break; }
  }
  return sweep;
}

// Singular values (descending) of a tall M (n x r, any n) given its polar factor U: one-sided
// Jacobi on the columns of the symmetric H = U^T M (accumulated in fp64), whose singular
// values are those of M.  Serves S of the project2orthogonal drop-in for matrices too tall
// for polar_jacobi_kernel.
__global__ void __launch_bounds__(kJacThreads) svals_from_polar_kernel(const float* __restrict__ M,
                                                                       const float* __restrict__ U,
                                                                       int n, int r,
                                                                       float* __restrict__ S) {
  extern __shared__ __align__(16) float sm[];
  __shared__ float red[kJacWarps];
  const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
  const int64_t b = blockIdx.x;
  const int ldr = r + 1, m = jac_m(r), ldn = jac_ldn(r);
  float* Vt = sm;                        // m x ldr (rotations, unused afterwards)
  float* Ht = Vt + (size_t)m * ldr;      // m x ldn: columns of H
  const float* Mb = M + b * (int64_t)n * r;
  const float* Ub = U + b * (int64_t)n * r;
  for (int j = ty; j < m; j += kJacWarps)
    for (int i = tx; i < r; i += 32) {
      double acc = 0.0;
      if (j < r)
        for (int k = 0; k < n; ++k) acc = fma((double)Ub[(int64_t)k * r + i], (double)Mb[(int64_t)k * r + j], acc);
      Ht[j * ldn + i] = (float)acc;
      Vt[j * ldr + i] = (i == j) ? 1.f : 0.f;
    }
  __syncthreads();
  jacobi_columns(Ht, ldn, r, Vt, ldr, r, red);
  __shared__ float sv[kMaxRank];
  for (int j = ty; j < r; j += kJacWarps) {
    float s = 0.f;
    for (int i = tx; i < r; i += 32) s = fmaf(Ht[j * ldn + i], Ht[j * ldn + i], s);
    s = warp_sum(s);
    if (tx == 0) sv[j] = sqrtf(s);
  }
  __syncthreads();
  if (tid == 0) {
    float* out = S + b * r;
    for (int j = 0; j < r; ++j) {
      const float v = sv[j];
      int k = j;
      while (k > 0 && out[k - 1] < v) { out[k] = out[k - 1]; --k; }
      out[k] = v;
    }
  }
}

}  // namespace fh

using namespace fh;

extern "C" int fh_polar_svals_f32(const float* M, const float* U, int64_t batch, int32_t n,
                                  int32_t r, float* S, void* stream) {
  if (!M || !U || !S || batch <= 0 || n < r || r <= 0) return FH_ERR_ARG;
  if (r > kMaxRank) return FH_ERR_UNSUPPORTED;
  const size_t smem = ((size_t)jac_m(r) * (r + 1) + (size_t)jac_m(r) * jac_ldn(r)) * sizeof(float);
  if (ensure_smem((const void*)svals_from_polar_kernel, smem)) return FH_ERR_LAUNCH;
  svals_from_polar_kernel<<<(unsigned)batch, kJacThreads, smem, (cudaStream_t)stream>>>(M, U, n, r, S);
  FH_CHECK_LAUNCH();
  return FH_OK;
}

