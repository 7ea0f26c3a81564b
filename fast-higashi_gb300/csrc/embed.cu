// Embedding post-processing on the GPU: FastHigashi.fetch_cell_embedding and
// correct_batch_linear (fasthigashi/FastHigashi_Wrapper.py:750-878).
//
// The reference assembles the cell embedding Y = [E D_1 / ||D_1||_col | E D_2 / .. | ..]
// (C x m, :753-758), takes its truncated SVD with scikit-learn's randomized TruncatedSVD
// (:767-768, again at :870-871 after the regression), quantile-transforms the read counts
// (:763), regresses a covariate out of Y by least squares with an intercept (:861-866) and
// row-normalises (:778, :873).  Here:
//
//   fh_embed_assemble    Y = E (D / ||D||_col): column norms in fp64, the product in fp32 as
//                        the reference's float32 matmul
//   fh_quantile_uniform  the quantile transform of one column to [0, 1]: a stable rank sort
//                        (each value's count of smaller values and of equal earlier ones), the
//                        percentile table at evenly spaced probabilities, and each value
//                        mapped by the mean of the forward and the reversed interpolation, all
//                        in fp64 with the operation order that gives the reference's values
//   fh_lstsq_residual    Y minus its least-squares fit on V with an intercept: centred fp64
//                        cross products, the minimum-norm coefficients from the eigenvectors
//                        of the centred Gram (fp64 Jacobi), the residual in fp64
//   fh_range_svd         the top-k singular triplets of Y whose columns lie in the column
//                        space of a narrow F (C x r, r <= 256): Y = E M lies in span(E), and
//                        the regressed Y in span([E, V, 1]).  With F^T F = Q L Q^T (fp64
//                        Jacobi; directions with l <= 1e-12 l_max dropped), U_F = F Q L^-1/2
//                        is an orthonormal basis, B = U_F^T Y (r x m), B B^T = U_B S^2 U_B^T,
//                        and Y = (U_F U_B) S V_B^T exactly: the SVD the reference's randomized
//                        sketch approximates, with no random start.  The component signs follow
//                        the reference's rule (each row of V_B^T has its largest-magnitude
//                        entry positive), and the output is U S (TruncatedSVD.fit_transform)
//   fh_l2_rows           rows scaled to unit norm, zero rows unchanged (sklearn normalize)
#include "fh_common.cuh"

namespace fh {

constexpr int kEmThreads = 256;

// ---- fp32 product with a column scale: out[i][j] = s[j] * sum_l A[i][l] B[l][j] --------------
constexpr int kGmTile = 64, kGmK = 16;

__global__ void __launch_bounds__(256) gemm_scale_kernel(const float* __restrict__ A, int64_t lda,
                                                         const float* __restrict__ B, int64_t ldb,
                                                         const float* __restrict__ scale, int n,
                                                         int m, int K, float* __restrict__ out,
                                                         int64_t ldo) {
  __shared__ float As[kGmK][kGmTile + 4];
  __shared__ float Bs[kGmK][kGmTile + 4];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t i0 = (int64_t)blockIdx.y * kGmTile;
  const int j0 = blockIdx.x * kGmTile;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += kGmK) {
    for (int e = threadIdx.x; e < kGmTile * kGmK; e += 256) {
      const int r = e / kGmK, kk = e % kGmK;           // A tile: row r, column k0 + kk
      const int64_t gi = i0 + r;
      As[kk][r] = (gi < n && k0 + kk < K) ? A[gi * lda + k0 + kk] : 0.f;
      const int kb = e / kGmTile, c = e % kGmTile;     // B tile: row k0 + kb, column c
      Bs[kb][c] = (k0 + kb < K && j0 + c < m) ? B[(int64_t)(k0 + kb) * ldb + j0 + c] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kGmK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        a[u] = As[kk][ty + 16 * u];
        b[u] = Bs[kk][tx + 16 * u];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(a[u], b[v], acc[u][v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int64_t gi = i0 + ty + 16 * u;
    if (gi >= n) continue;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int gj = j0 + tx + 16 * v;
      if (gj < m) out[gi * ldo + gj] = scale ? acc[u][v] * scale[gj] : acc[u][v];
    }
  }
}

// 1 / ||D[:, j]|| (norm summed in fp64, rounded to fp32 before the division as the
// reference's float32 norm)
__global__ void colnorm_inv_kernel(const float* __restrict__ D, int K, int m, int64_t ldd,
                                   float* __restrict__ inv) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  double s = 0.0;
  for (int l = 0; l < K; ++l) {
    const double v = D[(int64_t)l * ldd + j];
    s += v * v;
  }
  inv[j] = 1.f / (float)sqrt(s);
}

// ---- quantile transform -------------------------------------------------------------------
constexpr int kQtStage = 2048;

// sorted[pos(i)] = x[i], pos(i) = #{j: x[j] < x[i]} + #{j < i: x[j] == x[i]} (a stable sort)
__global__ void __launch_bounds__(kEmThreads) qt_rank_kernel(const double* __restrict__ x, int n,
                                                            double* __restrict__ sorted) {
  __shared__ double xs[kQtStage];
  const int i = blockIdx.x * kEmThreads + threadIdx.x;
  const double v = i < n ? x[i] : 0.0;
  int pos = 0;
  for (int b = 0; b < n; b += kQtStage) {
    const int nb = min(kQtStage, n - b);
    __syncthreads();
    for (int t = threadIdx.x; t < nb; t += kEmThreads) xs[t] = x[b + t];
    __syncthreads();
    if (i < n)
      for (int t = 0; t < nb; ++t) {
        const double u = xs[t];
        pos += (u < v) || (u == v && b + t < i);
      }
  }
  if (i < n) sorted[pos] = v;
}

// Evenly spaced probabilities refs[t] = t * (1 / (nq - 1)) (the last exactly 1) and the
// percentiles of the sorted values there, given as percentages: virtual index
// (n - 1) * ((refs * 100) / 100), interpolated from the nearer order statistic; then made
// non-decreasing.  One thread (nq is small).
__global__ void qt_table_kernel(const double* __restrict__ s, int n, int nq,
                                double* __restrict__ refs, double* __restrict__ q) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const double step = nq > 1 ? 1.0 / (double)(nq - 1) : 0.0;
  double run = 0.0;
  for (int t = 0; t < nq; ++t) {
    const double r = (t == nq - 1 && nq > 1) ? 1.0 : __dmul_rn((double)t, step);
    refs[t] = r;
    const double pr = __ddiv_rn(__dmul_rn(r, 100.0), 100.0);
    double v = __dmul_rn((double)(n - 1), pr);
    v = v < 0.0 ? 0.0 : (v > (double)(n - 1) ? (double)(n - 1) : v);
    const int lo = (int)floor(v);
    const int hi = lo + 1 < n ? lo + 1 : n - 1;
    const double g = __dsub_rn(v, (double)lo);
    const double a = s[lo], b = s[hi];
    const double d = __dsub_rn(b, a);
    const double val = g >= 0.5 ? __dsub_rn(b, __dmul_rn(d, __dsub_rn(1.0, g)))
                                : __dadd_rn(a, __dmul_rn(d, g));
    run = (t == 0 || val > run) ? val : run;
    q[t] = run;
  }
}

// Interpolation on increasing xp[i] = sgn * tab[idx(i)], fp[i] = sgn * ref[idx(i)] with
// idx(i) = i (sgn = 1) or nq - 1 - i (sgn = -1): the segment from the last xp[j] <= x; the end
// values outside.
__device__ double qt_interp(double x, const double* tab, const double* ref, int nq, double sgn) {
  auto xp = [&](int i) { return sgn > 0 ? tab[i] : -tab[nq - 1 - i]; };
  auto fp = [&](int i) { return sgn > 0 ? ref[i] : -ref[nq - 1 - i]; };
  if (x < xp(0)) return fp(0);
  if (x >= xp(nq - 1)) return fp(nq - 1);
  int lo = 0, hi = nq - 1;                // xp(lo) <= x < xp(hi)
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (xp(mid) <= x) lo = mid; else hi = mid;
  }
  if (xp(lo) == x) return fp(lo);
  const double slope = __ddiv_rn(__dsub_rn(fp(lo + 1), fp(lo)), __dsub_rn(xp(lo + 1), xp(lo)));
  return __dadd_rn(__dmul_rn(slope, __dsub_rn(x, xp(lo))), fp(lo));
}

__global__ void qt_apply_kernel(const double* __restrict__ x, int n, const double* __restrict__ q,
                                const double* __restrict__ refs, int nq, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = x[i];
  const double f = qt_interp(v, q, refs, nq, 1.0);
  const double b = qt_interp(-v, q, refs, nq, -1.0);
  double o = __dmul_rn(0.5, __dsub_rn(f, b));
  if (__dadd_rn(v, 1e-7) > q[nq - 1]) o = 1.0;
  if (__dsub_rn(v, 1e-7) < q[0]) o = 0.0;
  out[i] = o;
}

// ---- tall fp64 reductions ---------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ double ld_d(const T* p) { return (double)*p; }

// mean[j] = (1 / n) sum_c A[c][j], one block per column, fixed order
template <typename T>
__global__ void __launch_bounds__(kEmThreads) colmean_kernel(const T* __restrict__ A, int64_t lda,
                                                             int n, double* __restrict__ mean) {
  __shared__ double red[32];
  const int j = blockIdx.x;
  double s = 0.0;
  for (int c = threadIdx.x; c < n; c += kEmThreads) s += ld_d(A + (int64_t)c * lda + j);
  s = block_sum<double>(s, red);
  if (threadIdx.x == 0) mean[j] = s / (double)n;
}

// out[i][j] = sum_c (A[c][i] - ma[i]) (B[c][j] - mb[j])  (ma, mb optional), 32 x 32 outputs per
// block, rows staged 32 at a time; fixed order.
constexpr int kCrT = 32;
template <typename TA, typename TB>
__global__ void __launch_bounds__(kEmThreads) cross_kernel(const TA* __restrict__ A, int64_t lda,
                                                           int na, const double* __restrict__ ma,
                                                           const TB* __restrict__ B, int64_t ldb,
                                                           int nb, const double* __restrict__ mb,
                                                           int n, double* __restrict__ out,
                                                           int64_t ldo) {
  __shared__ double As[kCrT][kCrT + 1];
  __shared__ double Bs[kCrT][kCrT + 1];
  const int i0 = blockIdx.y * kCrT, j0 = blockIdx.x * kCrT;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 8 rows of 4 outputs each
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int c0 = 0; c0 < n; c0 += kCrT) {
    for (int e = threadIdx.x; e < kCrT * kCrT; e += kEmThreads) {
      const int r = e / kCrT, k = e % kCrT;
      const int c = c0 + r;
      double a = 0.0, b = 0.0;
      if (c < n && i0 + k < na) a = ld_d(A + (int64_t)c * lda + i0 + k) - (ma ? ma[i0 + k] : 0.0);
      if (c < n && j0 + k < nb) b = ld_d(B + (int64_t)c * ldb + j0 + k) - (mb ? mb[j0 + k] : 0.0);
      As[r][k] = a;
      Bs[r][k] = b;
    }
    __syncthreads();
    for (int r = 0; r < kCrT; ++r) {
      const double b = Bs[r][tx];
#pragma unroll
      for (int u = 0; u < 4; ++u) acc[u] = fma(As[r][ty + 8 * u], b, acc[u]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int i = i0 + ty + 8 * u, j = j0 + tx;
    if (i < na && j < nb) out[(int64_t)i * ldo + j] = acc[u];
  }
}

// ---- small dense fp64 products: C[i][j] = cs[j] * sum_l op(A)[i][l] op(B)[l][j] ----------------
// op(A)[i][l] = A[i * sa0 + l * sa1], op(B)[l][j] = B[l * sb0 + j * sb1]
__global__ void dsmall_kernel(const double* __restrict__ A, int64_t sa0, int64_t sa1,
                              const double* __restrict__ B, int64_t sb0, int64_t sb1,
                              const double* __restrict__ cs, int M, int N, int K,
                              double* __restrict__ Cm, int64_t ldc) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= (int64_t)M * N) return;
  const int i = (int)(e / N), j = (int)(e % N);
  double s = 0.0;
  for (int l = 0; l < K; ++l) s = fma(A[i * sa0 + l * sa1], B[l * sb0 + j * sb1], s);
  Cm[(int64_t)i * ldc + j] = cs ? s * cs[j] : s;
}

// ---- symmetric eigen-decomposition in fp64 (one CTA, parallel cyclic Jacobi) -----------------
// G (n x n, in place, ld n) -> eigenvalues w (descending) and eigenvectors Q (columns, ld n;
// Q is written in the order of w).  Round-robin pairs: each round rotates n/2 disjoint pairs
// (a warp per pair), first the columns of G and Q, then the rows of G.  Sweeps until every
// off-diagonal entry is below 1e-15 sqrt(g_pp g_qq) (or 1e-18 of the largest diagonal entry),
// at most 40 (FH_ERR_ILLCOND when they run out).
constexpr int kEigThreads = 512, kEigWarps = kEigThreads / 32, kEigMax = 256;

__device__ __forceinline__ void eig_pair(int k, int rnd, int m, int& p, int& q) {
  const int a = k == 0 ? 0 : 1 + (k - 1 + rnd) % (m - 1);
  const int b = 1 + (m - 2 - k + rnd) % (m - 1);
  p = min(a, b);
  q = max(a, b);
}

// G and Q move to shared memory when 2 n^2 doubles fit (n <= kEigSmemMax): the rotations are
// then latency-bound on shared memory instead of L2.
constexpr int kEigSmemMax = 100;

__global__ void __launch_bounds__(kEigThreads) sym_eig_kernel(double* __restrict__ Gg, int n,
                                                               double* __restrict__ w,
                                                               double* __restrict__ Qg,
                                                               double* __restrict__ Qs,
                                                               int* status) {
  extern __shared__ double eig_sm[];
  __shared__ double cs_c[kEigMax / 2], cs_s[kEigMax / 2];
  __shared__ int pr_p[kEigMax / 2], pr_q[kEigMax / 2];
  __shared__ int any;
  __shared__ double gmax;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int m = n + (n & 1);            // even count: the extra index is a dummy
  const bool on_chip = n <= kEigSmemMax;
  double* G = on_chip ? eig_sm : Gg;
  double* Q = on_chip ? eig_sm + n * n : Qg;
  if (on_chip)
    for (int e = threadIdx.x; e < n * n; e += kEigThreads) G[e] = Gg[e];
  for (int e = threadIdx.x; e < n * n; e += kEigThreads) Q[e] = (e / n == e % n) ? 1.0 : 0.0;
  __syncthreads();
  if (threadIdx.x == 0) {
    double g = 0.0;
    for (int i = 0; i < n; ++i) g = fmax(g, fabs(G[i * n + i]));
    gmax = g;
  }
  __syncthreads();
  // off-diagonal entries below this are left alone: rounding noise of a (near) null space
  const double floor_abs = 1e-18 * gmax;
  int sweep = 0;
  for (; sweep < 40; ++sweep) {
    if (threadIdx.x == 0) any = 0;
    __syncthreads();
    for (int rnd = 0; rnd < m - 1; ++rnd) {
      // angles of this step's pairs from the current G
      for (int k = threadIdx.x; k < m / 2; k += kEigThreads) {
        int p, q;
        eig_pair(k, rnd, m, p, q);
        double c = 1.0, s = 0.0;
        if (q < n) {
          const double gpp = G[p * n + p], gqq = G[q * n + q], gpq = G[p * n + q];
          if (fabs(gpq) > 1e-15 * sqrt(fabs(gpp * gqq)) && fabs(gpq) > floor_abs) {
            any = 1;
            const double zeta = (gqq - gpp) / (2.0 * gpq);
            const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
            c = 1.0 / sqrt(1.0 + t * t);
            s = c * t;
          }
        }
        cs_c[k] = c; cs_s[k] = s; pr_p[k] = p; pr_q[k] = q;
      }
      __syncthreads();
      // columns p, q of G and Q
      for (int k = warp; k < m / 2; k += kEigWarps) {
        const int p = pr_p[k], q = pr_q[k];
        const double c = cs_c[k], s = cs_s[k];
        if (q >= n || s == 0.0) continue;
        for (int i = lane; i < n; i += 32) {
          const double gp = G[i * n + p], gq = G[i * n + q];
          G[i * n + p] = c * gp - s * gq;
          G[i * n + q] = s * gp + c * gq;
          const double qp = Q[i * n + p], qq = Q[i * n + q];
          Q[i * n + p] = c * qp - s * qq;
          Q[i * n + q] = s * qp + c * qq;
        }
      }
      __syncthreads();
      // rows p, q of G
      for (int k = warp; k < m / 2; k += kEigWarps) {
        const int p = pr_p[k], q = pr_q[k];
        const double c = cs_c[k], s = cs_s[k];
        if (q >= n || s == 0.0) continue;
        for (int j = lane; j < n; j += 32) {
          const double gp = G[p * n + j], gq = G[q * n + j];
          G[p * n + j] = c * gp - s * gq;
          G[q * n + j] = s * gp + c * gq;
        }
      }
      __syncthreads();
    }
    const int done = !any;
    __syncthreads();
    if (done) break;
  }
  if (threadIdx.x == 0 && sweep == 40) set_status(status, FH_ERR_ILLCOND);
  // order by descending eigenvalue (selection by rank; ties by index)
  for (int j = threadIdx.x; j < n; j += kEigThreads) {
    const double v = G[j * n + j];
    int r = 0;
    for (int i = 0; i < n; ++i) {
      const double u = G[i * n + i];
      r += (u > v) || (u == v && i < j);
    }
    w[r] = v;
    for (int i = 0; i < n; ++i) Qs[i * n + r] = Q[i * n + j];
  }
}

// ---- least-squares residual ---------------------------------------------------------------
// coef[i][j] (p x m): pinv(Gvv) Hvy from the eigenpairs (w, Q) of Gvv; directions with
// w <= 1e-12 w_max dropped.  One thread per coefficient.
__global__ void lstsq_coef_kernel(const double* __restrict__ w, const double* __restrict__ Q,
                                  const double* __restrict__ H, int p, int m,
                                  double* __restrict__ coef) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= (int64_t)p * m) return;
  const int i = (int)(e / m), j = (int)(e % m);
  const double cut = 1e-12 * (w[0] > 0.0 ? w[0] : 0.0);
  double s = 0.0;
  for (int k = 0; k < p; ++k) {
    if (!(w[k] > cut)) continue;
    double t = 0.0;
    for (int l = 0; l < p; ++l) t = fma(Q[l * p + k], H[(int64_t)l * m + j], t);
    s = fma(Q[i * p + k] / w[k], t, s);
  }
  coef[(int64_t)i * m + j] = s;
}

// out[c][j] = (Y[c][j] - my[j]) - sum_i (V[c][i] - mv[i]) coef[i][j]  (+ my[j] - mv . coef[:, j]
// when the intercept goes back)
__global__ void __launch_bounds__(kEmThreads) lstsq_apply_kernel(
    const double* __restrict__ V, int p, const float* __restrict__ Y, int64_t ldy, int n, int m,
    const double* __restrict__ mv, const double* __restrict__ my, const double* __restrict__ coef,
    int add_back, float* __restrict__ out, int64_t ldo) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= (int64_t)n * m) return;
  const int64_t c = e / m;
  const int j = (int)(e % m);
  double r = (double)Y[c * ldy + j] - my[j];
  double icpt = my[j];
  for (int i = 0; i < p; ++i) {
    const double b = coef[(int64_t)i * m + j];
    r -= (V[c * p + i] - mv[i]) * b;
    icpt -= mv[i] * b;
  }
  out[c * ldo + j] = (float)(add_back ? r + icpt : r);
}

// ---- range SVD helpers ------------------------------------------------------------------------
// basis coefficients: T[i][k] = Q[i][k] / sqrt(w[k]) for kept k (w[k] > 1e-12 w[0]), else 0
__global__ void range_basis_kernel(const double* __restrict__ w, const double* __restrict__ Q,
                                   int r, double* __restrict__ T) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= r * r) return;
  const int k = e % r;
  const double cut = 1e-12 * (w[0] > 0.0 ? w[0] : 0.0);
  T[e] = w[k] > cut ? Q[e] / sqrt(w[k]) : 0.0;
}

// sign[j] = sign of column j's entry of largest magnitude (the first such) of Vb (m x k, ld k);
// the scale of U_B's column j in the output: sigma_j * sign_j.  One block per column.
__global__ void __launch_bounds__(kEmThreads) svd_sign_kernel(const double* __restrict__ Vb, int m,
                                                              int k, const double* __restrict__ w2,
                                                              double* __restrict__ scale) {
  __shared__ double bv[kEmThreads];
  __shared__ int bi[kEmThreads];
  const int j = blockIdx.x;
  double best = -1.0;
  int arg = 0x7fffffff;
  for (int i = threadIdx.x; i < m; i += kEmThreads) {
    const double a = fabs(Vb[(int64_t)i * k + j]);
    if (a > best) { best = a; arg = i; }
  }
  bv[threadIdx.x] = best;
  bi[threadIdx.x] = arg;
  __syncthreads();
  for (int o = kEmThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      const double a = bv[threadIdx.x + o];
      const int ia = bi[threadIdx.x + o];
      if (a > bv[threadIdx.x] || (a == bv[threadIdx.x] && ia < bi[threadIdx.x])) {
        bv[threadIdx.x] = a;
        bi[threadIdx.x] = ia;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double v = bi[0] < m ? Vb[(int64_t)bi[0] * k + j] : 1.0;
    const double sg = v < 0.0 ? -1.0 : 1.0;
    const double sig = w2[j] > 0.0 ? sqrt(w2[j]) : 0.0;
    scale[j] = sig * sg;
  }
}

// 1 / sigma_j for the components (0 when sigma_j is 0)
__global__ void inv_sigma_kernel(const double* __restrict__ w2, int k, double* __restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < k) out[j] = w2[j] > 0.0 ? 1.0 / sqrt(w2[j]) : 0.0;
}

__global__ void d2f_kernel(const double* __restrict__ a, int64_t n, float* __restrict__ b) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e < n) b[e] = (float)a[e];
}

// sigma values out (fp64, descending)
__global__ void sigma_kernel(const double* __restrict__ w2, int k, double* __restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < k) out[j] = w2[j] > 0.0 ? sqrt(w2[j]) : 0.0;
}

__global__ void __launch_bounds__(kEmThreads) l2_rows_kernel(const float* __restrict__ X,
                                                             int64_t ldx, int n, int m,
                                                             float* __restrict__ out,
                                                             int64_t ldo) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t r = (int64_t)blockIdx.x * (kEmThreads / 32) + warp;
  if (r >= n) return;
  double s = 0.0;
  for (int j = lane; j < m; j += 32) {
    const double v = X[r * ldx + j];
    s += v * v;
  }
  s = warp_sum(s);
  const double nr = sqrt(s);
  const double d = nr == 0.0 ? 1.0 : nr;
  for (int j = lane; j < m; j += 32) out[r * ldo + j] = (float)((double)X[r * ldx + j] / d);
}

__host__ __device__ inline size_t em_align(size_t x) { return (x + 255) & ~(size_t)255; }

inline size_t eig_smem(int n) {
  return n <= kEigSmemMax ? 2 * (size_t)n * n * sizeof(double) : 0;
}

// The on-chip eigen-solve's shared memory (up to 160 KB) needs the opt-in once.
inline int eig_prepare() {
  return ensure_smem((const void*)sym_eig_kernel, eig_smem(kEigSmemMax)) ? FH_ERR_LAUNCH : FH_OK;
}

inline unsigned em_grid(int64_t n, int t = kEmThreads) { return (unsigned)ceil_div(n, t); }

}  // namespace fh

using namespace fh;

extern "C" int fh_embed_assemble(const float* E, int32_t n_cells, int32_t R, int64_t lde,
                                 const float* D, int32_t m, int64_t ldd, float* inv_norm,
                                 float* Y, int64_t ldy, void* stream) {
  if (!E || !D || !inv_norm || !Y || n_cells <= 0 || R <= 0 || m <= 0 || lde < R || ldd < m ||
      ldy < m)
    return FH_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  colnorm_inv_kernel<<<em_grid(m), kEmThreads, 0, s>>>(D, R, m, ldd, inv_norm);
  const dim3 grid((unsigned)ceil_div(m, kGmTile), (unsigned)ceil_div(n_cells, kGmTile));
  gemm_scale_kernel<<<grid, 256, 0, s>>>(E, lde, D, ldd, inv_norm, n_cells, m, R, Y, ldy);
  FH_CHECK_LAUNCH();
  return FH_OK;
}

extern "C" int fh_gemm_scale_f32(const float* A, int64_t lda, const float* B, int64_t ldb,
                                 const float* scale, int32_t n, int32_t m, int32_t K, float* out,
                                 int64_t ldo, void* stream) {
  if (!A || !B || !out || n <= 0 || m <= 0 || K <= 0 || lda < K || ldb < m || ldo < m)
    return FH_ERR_ARG;
  const dim3 grid((unsigned)ceil_div(m, kGmTile), (unsigned)ceil_div(n, kGmTile));
  gemm_scale_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(A, lda, B, ldb, scale, n, m, K, out,
                                                            ldo);
  FH_CHECK_LAUNCH();
  return FH_OK;
}

extern "C" size_t fh_quantile_workspace(int32_t n, int32_t n_quantiles) {
  if (n <= 0 || n_quantiles <= 0) return 0;
  return em_align(sizeof(double) * n) + 2 * em_align(sizeof(double) * n_quantiles);
}

extern "C" int fh_quantile_uniform(const double* x, int32_t n, int32_t n_quantiles, double* out,
                                   void* workspace, size_t workspace_bytes, void* stream) {
  if (!x || !out || !workspace || n <= 0 || n_quantiles <= 0) return FH_ERR_ARG;
  if (workspace_bytes < fh_quantile_workspace(n, n_quantiles)) return FH_ERR_ARG;
  const int nq = n_quantiles < n ? n_quantiles : n;
  cudaStream_t s = (cudaStream_t)stream;
  uint8_t* w = (uint8_t*)workspace;
  double* sorted = (double*)w;  w += em_align(sizeof(double) * n);
  double* refs = (double*)w;    w += em_align(sizeof(double) * n_quantiles);
  double* q = (double*)w;
  qt_rank_kernel<<<em_grid(n), kEmThreads, 0, s>>>(x, n, sorted);
  qt_table_kernel<<<1, 32, 0, s>>>(sorted, n, nq, refs, q);
  qt_apply_kernel<<<em_grid(n), kEmThreads, 0, s>>>(x, n, q, refs, nq, out);
  FH_CHECK_LAUNCH();
  return FH_OK;
}

extern "C" size_t fh_lstsq_workspace(int32_t p, int32_t m) {
  if (p <= 0 || m <= 0) return 0;
  return em_align(sizeof(double) * p) + em_align(sizeof(double) * m) +
         3 * em_align(sizeof(double) * p * p) + em_align(sizeof(double) * p) +
         2 * em_align(sizeof(double) * (size_t)p * m);
}

extern "C" int fh_lstsq_residual(const double* V, int32_t n_cells, int32_t p, const float* Y,
                                 int64_t ldy, int32_t m, int32_t add_intercept_back, float* out,
                                 int64_t ldo, void* workspace, size_t workspace_bytes,
                                 int* status, void* stream) {
  if (!V || !Y || !out || !workspace || !status || n_cells <= 0 || p <= 0 || m <= 0 ||
      ldy < m || ldo < m)
    return FH_ERR_ARG;
  if (p > kEigMax) return FH_ERR_UNSUPPORTED;
  if (workspace_bytes < fh_lstsq_workspace(p, m)) return FH_ERR_ARG;
  if (eig_prepare()) return FH_ERR_LAUNCH;
  cudaStream_t s = (cudaStream_t)stream;
  uint8_t* w = (uint8_t*)workspace;
  double* mv = (double*)w;    w += em_align(sizeof(double) * p);
  double* my = (double*)w;    w += em_align(sizeof(double) * m);
  double* G = (double*)w;     w += em_align(sizeof(double) * p * p);
  double* Q = (double*)w;     w += em_align(sizeof(double) * p * p);
  double* Qs = (double*)w;    w += em_align(sizeof(double) * p * p);
  double* ev = (double*)w;    w += em_align(sizeof(double) * p);
  double* H = (double*)w;     w += em_align(sizeof(double) * (size_t)p * m);
  double* coef = (double*)w;
  colmean_kernel<double><<<p, kEmThreads, 0, s>>>(V, p, n_cells, mv);
  colmean_kernel<float><<<m, kEmThreads, 0, s>>>(Y, ldy, n_cells, my);
  cross_kernel<double, double><<<dim3((unsigned)ceil_div(p, kCrT), (unsigned)ceil_div(p, kCrT)),
                                 kEmThreads, 0, s>>>(V, p, p, mv, V, p, p, mv, n_cells, G, p);
  cross_kernel<double, float><<<dim3((unsigned)ceil_div(m, kCrT), (unsigned)ceil_div(p, kCrT)),
                                kEmThreads, 0, s>>>(V, p, p, mv, Y, ldy, m, my, n_cells, H, m);
  sym_eig_kernel<<<1, kEigThreads, eig_smem(p), s>>>(G, p, ev, Q, Qs, status);
  lstsq_coef_kernel<<<em_grid((int64_t)p * m), kEmThreads, 0, s>>>(ev, Qs, H, p, m, coef);
  lstsq_apply_kernel<<<em_grid((int64_t)n_cells * m), kEmThreads, 0, s>>>(
      V, p, Y, ldy, n_cells, m, mv, my, coef, add_intercept_back, out, ldo);
  FH_CHECK_LAUNCH();
  return FH_OK;
}

extern "C" size_t fh_range_svd_workspace(int32_t r, int32_t m, int32_t k) {
  if (r <= 0 || m <= 0 || k <= 0) return 0;
  const size_t rr = sizeof(double) * (size_t)r * r;
  return 5 * em_align(rr) + 2 * em_align(sizeof(double) * r) +
         2 * em_align(sizeof(double) * (size_t)r * m) + em_align(sizeof(double) * (size_t)m * k) +
         2 * em_align(sizeof(double) * k) + em_align(sizeof(double) * (size_t)r * k) +
         em_align(sizeof(float) * (size_t)r * k);
}

extern "C" int fh_range_svd(const float* F, int64_t ldf, int32_t n_cells, int32_t r,
                            const float* Y, int64_t ldy, int32_t m, int32_t k, float* out,
                            int64_t ldo, double* sigma, void* workspace, size_t workspace_bytes,
                            int* status, void* stream) {
  if (!F || !Y || !out || !workspace || !status || n_cells <= 0 || r <= 0 || m <= 0 || k <= 0 ||
      ldf < r || ldy < m || ldo < k || k > r || k > m)
    return FH_ERR_ARG;
  if (r > kEigMax) return FH_ERR_UNSUPPORTED;
  if (workspace_bytes < fh_range_svd_workspace(r, m, k)) return FH_ERR_ARG;
  if (eig_prepare()) return FH_ERR_LAUNCH;
  cudaStream_t s = (cudaStream_t)stream;
  uint8_t* w = (uint8_t*)workspace;
  const size_t rr = sizeof(double) * (size_t)r * r;
  double* G = (double*)w;     w += em_align(rr);        // F^T F, then B B^T
  double* Q = (double*)w;     w += em_align(rr);
  double* Qs = (double*)w;    w += em_align(rr);
  double* T = (double*)w;     w += em_align(rr);        // F -> orthonormal basis coefficients
  double* Ub = (double*)w;    w += em_align(rr);        // eigenvectors of B B^T
  double* ev = (double*)w;    w += em_align(sizeof(double) * r);
  double* ev2 = (double*)w;   w += em_align(sizeof(double) * r);
  double* FY = (double*)w;    w += em_align(sizeof(double) * (size_t)r * m);
  double* Bm = (double*)w;    w += em_align(sizeof(double) * (size_t)r * m);
  double* Vb = (double*)w;    w += em_align(sizeof(double) * (size_t)m * k);
  double* isg = (double*)w;   w += em_align(sizeof(double) * k);
  double* sc = (double*)w;    w += em_align(sizeof(double) * k);
  double* Wc = (double*)w;    w += em_align(sizeof(double) * (size_t)r * k);
  float* Wf = (float*)w;
  // F^T F and F^T Y in fp64
  cross_kernel<float, float><<<dim3((unsigned)ceil_div(r, kCrT), (unsigned)ceil_div(r, kCrT)),
                               kEmThreads, 0, s>>>(F, ldf, r, nullptr, F, ldf, r, nullptr,
                                                   n_cells, G, r);
  cross_kernel<float, float><<<dim3((unsigned)ceil_div(m, kCrT), (unsigned)ceil_div(r, kCrT)),
                               kEmThreads, 0, s>>>(F, ldf, r, nullptr, Y, ldy, m, nullptr,
                                                   n_cells, FY, m);
  // U_F = F T with T = Q L^-1/2 (kept directions)
  sym_eig_kernel<<<1, kEigThreads, eig_smem(r), s>>>(G, r, ev, Q, Qs, status);
  range_basis_kernel<<<em_grid((int64_t)r * r), kEmThreads, 0, s>>>(ev, Qs, r, T);
  // B = T^T (F^T Y)  (r x m)
  dsmall_kernel<<<em_grid((int64_t)r * m), kEmThreads, 0, s>>>(T, 1, r, FY, m, 1, nullptr, r, m,
                                                                r, Bm, m);
  // B B^T = U_B S^2 U_B^T
  dsmall_kernel<<<em_grid((int64_t)r * r), kEmThreads, 0, s>>>(Bm, m, 1, Bm, 1, m, nullptr, r, r,
                                                                m, G, r);
  sym_eig_kernel<<<1, kEigThreads, eig_smem(r), s>>>(G, r, ev2, Q, Ub, status);
  // components V_B = B^T U_B / S (m x k) and their signs
  inv_sigma_kernel<<<em_grid(k), kEmThreads, 0, s>>>(ev2, k, isg);
  dsmall_kernel<<<em_grid((int64_t)m * k), kEmThreads, 0, s>>>(Bm, 1, m, Ub, r, 1, isg, m, k, r,
                                                                Vb, k);
  svd_sign_kernel<<<k, kEmThreads, 0, s>>>(Vb, m, k, ev2, sc);
  if (sigma) sigma_kernel<<<em_grid(k), kEmThreads, 0, s>>>(ev2, k, sigma);
  // out = F (T U_B[:, :k] diag(sigma sign))
  dsmall_kernel<<<em_grid((int64_t)r * k), kEmThreads, 0, s>>>(T, r, 1, Ub, r, 1, sc, r, k, r,
                                                                Wc, k);
  d2f_kernel<<<em_grid((int64_t)r * k), kEmThreads, 0, s>>>(Wc, (int64_t)r * k, Wf);
  const dim3 grid((unsigned)ceil_div(k, kGmTile), (unsigned)ceil_div(n_cells, kGmTile));
  gemm_scale_kernel<<<grid, 256, 0, s>>>(F, ldf, Wf, k, nullptr, n_cells, k, r, out, ldo);
  FH_CHECK_LAUNCH();
  return FH_OK;
}

extern "C" int fh_cross_f32(const float* A, int64_t lda, int32_t na, const float* B,
                            int64_t ldb, int32_t nb, int32_t n_rows, double* out, int64_t ldo,
                            void* stream) {
  if (!A || !B || !out || na <= 0 || nb <= 0 || n_rows <= 0 || lda < na || ldb < nb || ldo < nb)
    return FH_ERR_ARG;
  cross_kernel<float, float><<<dim3((unsigned)ceil_div(nb, kCrT), (unsigned)ceil_div(na, kCrT)),
                               kEmThreads, 0, (cudaStream_t)stream>>>(A, lda, na, nullptr, B, ldb,
                                                                      nb, nullptr, n_rows, out,
                                                                      ldo);
  FH_CHECK_LAUNCH();
  return FH_OK;
}

extern "C" int fh_l2_rows(const float* X, int64_t ldx, int32_t n, int32_t m, float* out,
                          int64_t ldo, void* stream) {
  if (!X || !out || n <= 0 || m <= 0 || ldx < m || ldo < m) return FH_ERR_ARG;
  l2_rows_kernel<<<(unsigned)ceil_div(n, kEmThreads / 32), kEmThreads, 0, (cudaStream_t)stream>>>(
      X, ldx, n, m, out, ldo);
  FH_CHECK_LAUNCH();
  return FH_OK;
}
