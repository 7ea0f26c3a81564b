// CTA-wide building blocks of the polar-factor kernels (fp32, shared memory).
//
// All routines are called by every thread of the block (blockDim.x a multiple of 32) with
// uniform arguments.  Loops map lanes to columns and warps to rows, so no loop divides by a
// runtime extent.
#pragma once
#include "fh_common.cuh"

namespace fh {

constexpr int kNewtonMaxIt = 30;

struct PolarScratch {
  float* vh;     // [kMaxRank] head of each Householder vector
  float* beta;   // [kMaxRank] 2 / v^T v
  float* wv;     // [2 * kMaxRank] per-column dot products / pivot row
  float* fcol;   // [kMaxRank] pivot column
  float* red;    // [32]
  double* dred;  // [32]
  int* ival;     // [4]: [0] a zero pivot was met
  float* gcol;   // [2][64]  register Gauss-Jordan: pivot column (double-buffered)
  float* grow;   // [2][128] scaled pivot row
  float* grp;    // [2]      1 / pivot
  int* gi;       // [0, 64) row used as a pivot, [64, 128) step that pivoted the row, [128, 130) pivot
  float* tri;    // [7][16][16] off-diagonal block products of the blocked triangular inverse
};
constexpr int kPolarMiscFloats = 5 * kMaxRank + 64 + 128 + 256 + 4 + 132 + 7 * 256;

// Carves the scratch out of kPolarMiscFloats floats of shared memory.
__device__ inline PolarScratch polar_scratch(float* misc, float* red, double* dred, int* ival) {
  PolarScratch s;
  s.vh = misc;
  s.beta = misc + kMaxRank;
  s.wv = misc + 2 * kMaxRank;
  s.fcol = misc + 4 * kMaxRank;
  s.red = red;
  s.dred = dred;
  s.ival = ival;
  float* g = misc + 5 * kMaxRank + 64;
  s.gcol = g;
  s.grow = g + 128;
  s.grp = g + 384;
  s.gi = reinterpret_cast<int*>(g + 388);
  s.tri = g + 388 + 132;
  return s;
}

// ---- register-tiled CTA matrix product (512 threads) -----------------------------------
// acc[u][v] = sum_k fa(i_u, k) fb(k, j_v) for the thread's outputs i_u = warp + 16 u,
// j_v = lane + 32 v (u < TM, v < TN), k in increasing order.  Rows / columns past M / N are
// clamped to the last one (their results are to be discarded).  fa is read with one address
// per warp (a broadcast), fb with consecutive or odd-strided addresses across the lanes.
template <int TM, int TN, class FA, class FB>
__device__ __forceinline__ void cta_mm(int M, int N, int K, int row0, FA fa, FB fb,
                                       float (&acc)[TM][TN]) {
  const int rt = threadIdx.x >> 5, ct = threadIdx.x & 31;
  int ri[TM], cj[TN];
#pragma unroll
  for (int u = 0; u < TM; ++u) ri[u] = min(row0 + rt + 16 * u, M - 1);
#pragma unroll
  for (int v = 0; v < TN; ++v) cj[v] = min(ct + 32 * v, N - 1);
#pragma unroll
  for (int u = 0; u < TM; ++u)
#pragma unroll
    for (int v = 0; v < TN; ++v) acc[u][v] = 0.f;
#pragma unroll 2
  for (int k = 0; k < K; ++k) {
    float av[TM], bv[TN];
#pragma unroll
    for (int u = 0; u < TM; ++u) av[u] = fa(ri[u], k);
#pragma unroll
    for (int v = 0; v < TN; ++v) bv[v] = fb(k, cj[v]);
#pragma unroll
    for (int u = 0; u < TM; ++u)
#pragma unroll
      for (int v = 0; v < TN; ++v) acc[u][v] = fmaf(av[u], bv[v], acc[u][v]);
  }
}

__device__ __forceinline__ int pc_lane() { return threadIdx.x & 31; }
__device__ __forceinline__ int pc_warp() { return threadIdx.x >> 5; }
__device__ __forceinline__ int pc_nwarps() { return blockDim.x >> 5; }

// ---- Householder QR of T (n x r, row stride ldt, n >= r), in place ---------------------
// On return the upper triangle of T[0:r][0:r] is R, T[i][k] (i > k) holds v_k below the
// diagonal, vh[k] the head of v_k and beta[k] = 2 / v_k^T v_k (0 for a zero column).
// householder_panel factors columns [k0, k1) and applies each reflector to the columns
// below k1 only; householder_qr is the whole matrix as one panel.  (A blocked variant with
// UT-form trailing updates measured 9 % slower here: the panel steps keep their barriers.)
__device__ inline void householder_panel(float* T, int n, int k0, int k1, int ldt,
                                         PolarScratch& s) {
  const int tx = pc_lane(), ty = pc_warp(), nw = pc_nwarps();
  for (int k = k0; k < k1; ++k) {
    if (ty == 0) {
      float ss = 0.f;
      for (int i = k + 1 + tx; i < n; i += 32) ss = fmaf(T[i * ldt + k], T[i * ldt + k], ss);
      ss = warp_sum(ss);
      if (tx == 0) {
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
    // w_j = v^T T[k:, j]: four columns per warp (independent chains, one pass over v)
    for (int jb = k + 1 + 4 * ty; jb < k1; jb += 4 * nw) {
      float d[4] = {0.f, 0.f, 0.f, 0.f};
      for (int i = k + 1 + tx; i < n; i += 32) {
        const float vi = T[i * ldt + k];
#pragma unroll
        for (int c = 0; c < 4; ++c)
          if (jb + c < k1) d[c] = fmaf(vi, T[i * ldt + jb + c], d[c]);
      }
#pragma unroll
      for (int c = 0; c < 4; ++c) d[c] = warp_sum(d[c]);
      if (tx == 0) {
#pragma unroll
        for (int c = 0; c < 4; ++c)
          if (jb + c < k1) s.wv[jb + c] = fmaf(vh, T[k * ldt + jb + c], d[c]);
      }
    }
    __syncthreads();
    if (beta != 0.f) {
      for (int i = k + ty; i < n; i += nw) {
        const float bv = -beta * ((i == k) ? vh : T[i * ldt + k]);
        for (int j = k + 1 + tx; j < k1; j += 32) T[i * ldt + j] = fmaf(bv, s.wv[j], T[i * ldt + j]);
      }
    }
    if (threadIdx.x == 0) T[k * ldt + k] = s.wv[2 * kMaxRank - 1];
    __syncthreads();
  }
}

__device__ inline void householder_qr(float* T, int n, int r, int ldt, PolarScratch& s) {
  householder_panel(T, n, 0, r, ldt, s);
}

// ---- Householder QR with warp-owned columns held in registers --------------------------
// The same factorization and output layout as householder_qr, organised so that each step
// costs one hardware barrier instead of three CTA-wide ones: warp w owns columns
// j = w + NW c (c < NC) and keeps them in registers, lane l holding rows l + 32 t (t < NT).
// Step k: the owner of column k (whose column has had reflectors 0..k-1 applied) forms
// reflector k from its registers (norm by a warp reduction), writes v_k below the diagonal of
// T, vh[k], beta[k] and R[k][k] = alpha, and signals with bar.arrive on named barrier
// 1 + (k & 1); every other warp waits there with bar.sync.  Then each warp applies reflector
// k to its own columns j > k (warp-reduced dot products, no further synchronisation).  A warp
// reaches step k + 2's barrier (the same id) only after every warp passed step k + 1's, so two
// ids suffice.  At the end the warps store R's strict upper triangle.  Every warp executes
// exactly one barrier operation per step, for every step, whatever the data (a zero column
// gives beta = 0 and the step still synchronises).  (A look-ahead variant, the owner of column
// k + 1 forming its reflector before updating its other columns, measured 1 % slower: the
// kernel is issue-bound with two CTAs per SM, and the extra selects cost more than the
// shortened chain gains.)
template <int ID>
__device__ __forceinline__ void named_bar_sync(int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"n"(ID), "r"(nthreads) : "memory");
}
template <int ID>
__device__ __forceinline__ void named_bar_arrive(int nthreads) {
  asm volatile("bar.arrive %0, %1;" ::"n"(ID), "r"(nthreads) : "memory");
}

template <int NC, int NT>
__device__ inline void householder_qr_cols(float* T, int n, int r, int ldt, PolarScratch& s) {
  const int tx = pc_lane(), w = pc_warp(), nw = pc_nwarps();
  const int nthreads = (int)blockDim.x;
  float a[NC][NT];
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    const int j = w + nw * c;
#pragma unroll
    for (int t = 0; t < NT; ++t) {
      const int i = tx + 32 * t;
      a[c][t] = (j < r && i < n) ? T[i * ldt + j] : 0.f;
    }
  }
  __syncthreads();   // every warp has its columns before any column of T is overwritten
  // The owner of column k forms reflector k from its registers and arrives on k's barrier.
  auto form = [&](int k) {
    const int kc = k / nw;
    float ss = 0.f, x0 = 0.f;
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      if (c == kc) {
#pragma unroll
        for (int t = 0; t < NT; ++t) {
          const int i = tx + 32 * t;
          if (i > k && i < n) {
            ss = fmaf(a[c][t], a[c][t], ss);
            T[i * ldt + k] = a[c][t];              // v_k below the diagonal
          }
          if (i == k) x0 = a[c][t];
        }
      }
    }
    ss = warp_sum(ss);
    x0 = __shfl_sync(0xffffffffu, x0, k & 31);
    if (tx == 0) {
      const float s2 = fmaf(x0, x0, ss);
      if (s2 == 0.f) {
        s.beta[k] = 0.f;
        s.vh[k] = 0.f;
        T[k * ldt + k] = 0.f;
      } else {
        const float nrm = sqrtf(s2);
        const float alpha = x0 >= 0.f ? -nrm : nrm;
        s.vh[k] = x0 - alpha;
        s.beta[k] = 1.f / (s2 - x0 * alpha);
        T[k * ldt + k] = alpha;
      }
    }
    __threadfence_block();
    if (k & 1) named_bar_arrive<2>(nthreads);
    else named_bar_arrive<1>(nthreads);
    __syncwarp();                   // lane 0's vh / beta visible to the owner's other lanes
  };
  // Applies reflector k (v, -beta) to local column c.
  auto update = [&](int c, float nbeta, const float (&v)[NT]) {
#pragma unroll
    for (int cc = 0; cc < NC; ++cc) {
      if (cc == c) {
        float d = 0.f;
#pragma unroll
        for (int t = 0; t < NT; ++t) d = fmaf(v[t], a[cc][t], d);
        d = nbeta * warp_sum(d);
#pragma unroll
        for (int t = 0; t < NT; ++t) a[cc][t] = fmaf(d, v[t], a[cc][t]);
      }
    }
  };
  for (int k = 0; k < r; ++k) {
    if (k % nw == w) {
      form(k);
    } else {
      if (k & 1) named_bar_sync<2>(nthreads);
      else named_bar_sync<1>(nthreads);
    }
    const float beta = s.beta[k];
    if (beta == 0.f) continue;      // uniform: every warp read the same value
    float v[NT];
    const float vh = s.vh[k];
#pragma unroll
    for (int t = 0; t < NT; ++t) {
      const int i = tx + 32 * t;
      v[t] = (i > k && i < n) ? T[i * ldt + k] : (i == k ? vh : 0.f);
    }
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      const int j = w + nw * c;
      if (j > k && j < r) update(c, -beta, v);
    }
  }
  // R's strict upper triangle (rows i < j of column j); the diagonal and the reflectors are
  // in T already
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    const int j = w + nw * c;
#pragma unroll
    for (int t = 0; t < NT; ++t) {
      const int i = tx + 32 * t;
      if (j < r && i < j) T[i * ldt + j] = a[c][t];
    }
  }
  __syncthreads();
}

// Dispatch on the row count: NT = 4, 6 or 8 rows per lane (n <= 256); wider tiles take the
// CTA-wide householder_qr.
template <int NC>
__device__ inline void householder_qr_fast(float* T, int n, int r, int ldt, PolarScratch& s) {
  if (n <= 128) householder_qr_cols<NC, 4>(T, n, r, ldt, s);
  else if (n <= 192) householder_qr_cols<NC, 6>(T, n, r, ldt, s);
  else if (n <= 256) householder_qr_cols<NC, 8>(T, n, r, ldt, s);
  else householder_qr(T, n, r, ldt, s);
}

// ---- U = Q U: apply the stored reflectors in reverse to U (n x r, stride ldu) ----------
// The dot products v^T U[:, j] go four columns per warp (independent chains, one pass over v);
// each column's sum runs in the same order as one column at a time.
__device__ inline void apply_q(const float* T, int ldt, float* U, int ldu, int n, int r,
                               PolarScratch& s) {
  const int tx = pc_lane(), ty = pc_warp(), nw = pc_nwarps();
  for (int k = r - 1; k >= 0; --k) {
    const float beta = s.beta[k], vh = s.vh[k];
    if (beta == 0.f) continue;  // uniform across the block
    for (int jb = 4 * ty; jb < r; jb += 4 * nw) {
      float d[4] = {0.f, 0.f, 0.f, 0.f};
      for (int i = k + 1 + tx; i < n; i += 32) {
        const float vi = T[i * ldt + k];
#pragma unroll
        for (int c = 0; c < 4; ++c)
          if (jb + c < r) d[c] = fmaf(vi, U[i * ldu + jb + c], d[c]);
      }
#pragma unroll
      for (int c = 0; c < 4; ++c) d[c] = warp_sum(d[c]);
      if (tx == 0) {
#pragma unroll
        for (int c = 0; c < 4; ++c)
          if (jb + c < r) s.wv[jb + c] = fmaf(vh, U[k * ldu + jb + c], d[c]);
      }
    }
    __syncthreads();
    for (int i = k + ty; i < n; i += nw) {
      const float bv = -beta * ((i == k) ? vh : T[i * ldt + k]);
      for (int j = tx; j < r; j += 32) U[i * ldu + j] = fmaf(bv, s.wv[j], U[i * ldu + j]);
    }
    __syncthreads();
  }
}

// ---- U = Q U with warp-owned columns in registers (no barriers) ------------------------
// The product of the reflectors stored by householder_qr / householder_qr_cols (v_k below the
// diagonal of T, vh[k], beta[k]) applied in reverse to U (n x r, stride ldu; rows < r hold X on
// entry, the rows below are taken as zero; all n rows of U on return).  Each warp owns columns
// j = w + NW c and applies every reflector to them in registers, lane l holding rows l + 32 t:
// a column's dot product with v_k is a warp reduction, so the warps never wait on one another.
// The caller synchronises before (X and the reflectors complete) and this routine once after.
template <int NC, int NT>
__device__ inline void apply_q_cols(const float* T, int ldt, float* U, int ldu, int n, int r,
                                    PolarScratch& s) {
  const int tx = pc_lane(), w = pc_warp(), nw = pc_nwarps();
  float u[NC][NT];
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    const int j = w + nw * c;
#pragma unroll
    for (int t = 0; t < NT; ++t) {
      const int i = tx + 32 * t;
      u[c][t] = (j < r && i < r) ? U[i * ldu + j] : 0.f;
    }
  }
  for (int k = r - 1; k >= 0; --k) {
    const float beta = s.beta[k];
    if (beta == 0.f) continue;      // uniform across the warp
    const float vh = s.vh[k];
    float v[NT];
#pragma unroll
    for (int t = 0; t < NT; ++t) {
      const int i = tx + 32 * t;
      v[t] = (i > k && i < n) ? T[i * ldt + k] : (i == k ? vh : 0.f);
    }
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      float d = 0.f;
#pragma unroll
      for (int t = 0; t < NT; ++t) d = fmaf(v[t], u[c][t], d);
      d = -beta * warp_sum(d);
#pragma unroll
      for (int t = 0; t < NT; ++t) u[c][t] = fmaf(d, v[t], u[c][t]);
    }
  }
  __syncthreads();   // every warp has read its columns of X before any row of U is written
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    const int j = w + nw * c;
#pragma unroll
    for (int t = 0; t < NT; ++t) {
      const int i = tx + 32 * t;
      if (j < r && i < n) U[i * ldu + j] = u[c][t];
    }
  }
  __syncthreads();
}

// Dispatch on the row count: NT = 4, 6 or 8 rows per lane (n <= 256); wider tiles zero U's
// rows past r and take the CTA-wide apply_q.
template <int NC>
__device__ inline void apply_q_fast(const float* T, int ldt, float* U, int ldu, int n, int r,
                                    PolarScratch& s) {
  if (n <= 128) {
    apply_q_cols<NC, 4>(T, ldt, U, ldu, n, r, s);
  } else if (n <= 192) {
    apply_q_cols<NC, 6>(T, ldt, U, ldu, n, r, s);
  } else if (n <= 256) {
    apply_q_cols<NC, 8>(T, ldt, U, ldu, n, r, s);
  } else {
    for (int j = r + pc_warp(); j < n; j += pc_nwarps())
      for (int l = pc_lane(); l < r; l += 32) U[j * ldu + l] = 0.f;
    __syncthreads();
    apply_q(T, ldt, U, ldu, n, r, s);
  }
}

// ---- inverse of an upper-triangular R (r x r, stride ldr) into Xi (stride ldo) ---------
// Column j of R^{-1} by back substitution; one warp per column, lanes share each dot product.
__device__ inline void tri_inverse(const float* R, int ldr, float* Xi, int ldo, int r,
                                   PolarScratch& s) {
  const int tx = pc_lane(), ty = pc_warp(), nw = pc_nwarps();
  for (int j = ty; j < r; j += nw) {
    for (int i = tx; i < r; i += 32) Xi[i * ldo + j] = 0.f;
    __syncwarp();
    for (int i = j; i >= 0; --i) {
      float d = 0.f;
      for (int l = i + 1 + tx; l <= j; l += 32) d = fmaf(R[i * ldr + l], Xi[l * ldo + j], d);
      d = warp_sum(d);
      if (tx == 0) {
        float rii = R[i * ldr + i];
        if (rii == 0.f) { rii = 1e-30f; s.ival[0] = 1; }
        Xi[i * ldo + j] = ((i == j ? 1.f : 0.f) - d) / rii;
      }
      __syncwarp();
    }
  }
  __syncthreads();
}

// ---- inverse of an upper-triangular R (r <= 128, stride ldr) into Xi (stride ldo), 512 threads
// Blocked: the 16 x 16 diagonal blocks are inverted by one warp each (a lane per column, the
// column in registers, no synchronisation), then the off-diagonal blocks by block diagonals,
// X_ij = -X_ii sum_{k=i+1..j} R_ik X_kj, as small products over all threads: 2 (r/16 - 1) + 1
// barriers in all instead of a serial chain of r dependent steps.  Writes the upper triangle of Xi (and
// zeroes the strictly lower part when zero_lower is set).
__device__ inline void tri_inverse_blocked(const float* R, int ldr, float* Xi, int ldo, int r,
                                           bool zero_lower, PolarScratch& s) {
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  const int nb = (r + 15) >> 4;
  if (w < nb && l < 16) {
    const int b0 = 16 * w;
    const int c = b0 + l;              // this lane's column
    float x[16];
#pragma unroll
    for (int ii = 15; ii >= 0; --ii) {
      const int i = b0 + ii;
      float v = 0.f;
      if (ii <= l && c < r) {
        float d = (ii == l) ? 1.f : 0.f;
#pragma unroll
        for (int ll = ii + 1; ll < 16; ++ll)
          if (ll <= l) d = fmaf(-R[i * ldr + b0 + ll], x[ll], d);
        float rii = R[i * ldr + i];
        if (rii == 0.f) { rii = 1e-30f; s.ival[0] = 1; }
        v = d / rii;
      }
      x[ii] = v;
    }
    if (c < r) {
#pragma unroll
      for (int ii = 0; ii < 16; ++ii)
        if (b0 + ii < r && ii <= l) Xi[(b0 + ii) * ldo + c] = x[ii];
    }
  }
  if (zero_lower)
    for (int idx = threadIdx.x; idx < r * r; idx += blockDim.x) {
      const int i = idx / r, j = idx - i * r;
      if (i > j) Xi[i * ldo + j] = 0.f;
    }
  __syncthreads();
  for (int d = 1; d < nb; ++d) {
    const int nblk = nb - d;
    // T_i = sum_{k=i+1..i+d} R_ik X_k,i+d  (16 x 16 each), into the scratch
    for (int idx = threadIdx.x; idx < nblk * 256; idx += blockDim.x) {
      const int bi = idx >> 8, p = (idx >> 4) & 15, q = idx & 15;
      const int row = 16 * bi + p, col = 16 * (bi + d) + q;
      float acc = 0.f;
      if (row < r && col < r)
        for (int k = 16 * (bi + 1); k <= col; ++k) acc = fmaf(R[row * ldr + k], Xi[k * ldo + col], acc);
      s.tri[idx] = acc;
    }
    __syncthreads();
    // X_i,i+d = -X_ii T_i
    for (int idx = threadIdx.x; idx < nblk * 256; idx += blockDim.x) {
      const int bi = idx >> 8, p = (idx >> 4) & 15, q = idx & 15;
      const int row = 16 * bi + p, col = 16 * (bi + d) + q;
      if (row < r && col < r) {
        float acc = 0.f;
        for (int m = p; m < 16; ++m) acc = fmaf(Xi[row * ldo + 16 * bi + m], s.tri[(bi << 8) + (m << 4) + q], acc);
        Xi[row * ldo + col] = -acc;
      }
    }
    __syncthreads();
  }
}

// ---- inverse of X (r x r, stride ldx) by Gauss-Jordan with partial pivoting ------------
// Aug: r x (2r+1) scratch; on return its columns [r, 2r) hold X^{-1}.
__device__ inline void gj_inverse(const float* X, int ldx, float* Aug, int r, PolarScratch& s) {
  const int tx = pc_lane(), ty = pc_warp(), nw = pc_nwarps();
  const int la = 2 * r + 1, w2 = 2 * r;
  for (int i = ty; i < r; i += nw)
    for (int j = tx; j < w2; j += 32)
      Aug[i * la + j] = j < r ? X[i * ldx + j] : (j - r == i ? 1.f : 0.f);
  __syncthreads();
  for (int k = 0; k < r; ++k) {
    if (ty == 0) {
      float best = -1.f;
      int bi = k;
      for (int i = k + tx; i < r; i += 32) {
        const float a = fabsf(Aug[i * la + k]);
        if (a > best) { best = a; bi = i; }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (bi != k)
        for (int j = k + tx; j < w2; j += 32) {
          const float a = Aug[k * la + j];
          Aug[k * la + j] = Aug[bi * la + j];
          Aug[bi * la + j] = a;
        }
      __syncwarp();
      float piv = Aug[k * la + k];
      if (piv == 0.f) {
        piv = 1e-30f;
        if (tx == 0) s.ival[0] = 1;
      }
      for (int i = tx; i < r; i += 32) s.fcol[i] = Aug[i * la + k];
      const float rp = 1.f / piv;
      for (int j = k + 1 + tx; j < w2; j += 32) {
        const float v = Aug[k * la + j] * rp;
        s.wv[j] = v;
        Aug[k * la + j] = v;
      }
    }
    __syncthreads();
    for (int i = ty; i < r; i += nw) {
      if (i == k) continue;
      const float f = -s.fcol[i];
      for (int j = k + 1 + tx; j < w2; j += 32) Aug[i * la + j] = fmaf(f, s.wv[j], Aug[i * la + j]);
    }
    __syncthreads();
  }
}

// ---- U = Q [X; 0] from the compact UT form of the reflectors (512 threads) ------------
// Q = H_0 ... H_{r-1} = I - V T V^T with T^{-1} = diag(1/beta) + striu(V^T V) (the UT
// transform of the Householder product), so U = [X; 0] - V (T (V_top^T X)), V_top = V's first
// r rows: three register-tiled products, one triangular inverse, no per-reflector steps.
// T: n x ldt reflector storage of householder_qr (its upper triangle, no longer needed after
// the Newton iteration, receives T); U: rows < r hold X on entry, n rows of U on return;
// Sc: r x ldt scratch.  n <= 192, r <= 64.
__device__ inline void apply_q_ut(float* T, int ldt, float* U, int ldu, float* Sc, int n, int r,
                                  PolarScratch& s) {
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  const float* vh = s.vh;
  const float* beta = s.beta;
  auto V = [&](int k, int c) -> float {
    return k > c ? T[k * ldt + c] : (k == c ? vh[c] : 0.f);
  };
  float acc[4][2];
  // Sc = diag(1/beta) + striu(V^T V)
  cta_mm<4, 2>(r, r, n, 0, [&](int i, int k) { return V(k, i); },
               [&](int k, int j) { return V(k, j); }, acc);
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 2; ++v) {
      const int i = w + 16 * u, j = l + 32 * v;
      if (i < r && j < r)
        Sc[i * ldt + j] = i < j ? acc[u][v] : (i == j ? (beta[i] != 0.f ? 1.f / beta[i] : 1.f) : 0.f);
    }
  __syncthreads();
  // T = Sc^{-1} into the upper triangle of the reflector storage (its lower part holds V)
  tri_inverse_blocked(Sc, ldt, T, ldt, r, false, s);
  // Sc = V_top^T X
  cta_mm<4, 2>(r, r, r, 0, [&](int c, int k) { return V(k, c); },
               [&](int k, int j) { return U[k * ldu + j]; }, acc);
  __syncthreads();
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 2; ++v) {
      const int i = w + 16 * u, j = l + 32 * v;
      if (i < r && j < r) Sc[i * ldt + j] = acc[u][v];
    }
  __syncthreads();
  // Sc = T Sc
  cta_mm<4, 2>(r, r, r, 0, [&](int i, int k) { return k >= i ? T[i * ldt + k] : 0.f; },
               [&](int k, int j) { return Sc[k * ldt + j]; }, acc);
  __syncthreads();
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 2; ++v) {
      const int i = w + 16 * u, j = l + 32 * v;
      if (i < r && j < r) Sc[i * ldt + j] = acc[u][v];
    }
  __syncthreads();
  // U = [X; 0] - V Sc, both 96-row tiles held in registers until every thread has read X
  float a0[6][2], a1[6][2];
  cta_mm<6, 2>(n, r, r, 0, [&](int i, int c) { return V(i, c); },
               [&](int c, int j) { return Sc[c * ldt + j]; }, a0);
  cta_mm<6, 2>(n, r, r, 96, [&](int i, int c) { return V(i, c); },
               [&](int c, int j) { return Sc[c * ldt + j]; }, a1);
  float x0[6][2];
#pragma unroll
  for (int u = 0; u < 6; ++u)
#pragma unroll
    for (int v = 0; v < 2; ++v) {
      const int i = w + 16 * u, j = l + 32 * v;
      x0[u][v] = (i < r && j < r) ? U[i * ldu + j] : 0.f;
    }
  __syncthreads();
#pragma unroll
  for (int u = 0; u < 6; ++u)
#pragma unroll
    for (int v = 0; v < 2; ++v) {
      const int j = l + 32 * v;
      const int i0 = w + 16 * u, i1 = 96 + w + 16 * u;
      if (j < r) {
        if (i0 < n) U[i0 * ldu + j] = x0[u][v] - a0[u][v];
        if (i1 < n) U[i1 * ldu + j] = -a1[u][v];
      }
    }
  __syncthreads();
}

// ---- inverse of X (r x r, r <= 64, stride ldx) into Xi (stride ldo), 512 threads -------
// Gauss-Jordan with partial pivoting on [X | I] held in registers: thread (warp w, lane l)
// owns rows w + 16 u (u < 4) and columns l + 32 v (v < 4).  Rows are not swapped: each step
// picks the largest |entry| of the column among the rows not yet used as pivots (every warp
// finds it from the published column, so no thread waits for a pivot broadcast), so every
// element sees the same operations as in gj_inverse; row p_k of the right block is row k of
// X^{-1}.  Two barriers per column: the eliminating step also publishes the next column.
__device__ inline void gj_inverse_reg(const float* X, int ldx, float* Xi, int ldo, int r,
                                      PolarScratch& s) {
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  float a[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int i = w + 16 * u;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int j = l + 32 * v;
      float x = 0.f;
      if (i < r) {
        if (j < r) x = X[i * ldx + j];
        else if (j - r == i) x = 1.f;
      }
      a[u][v] = x;
    }
  }
  uint64_t used = r >= 64 ? 0ull : (~0ull << r);   // rows taken as pivots (and rows >= r)
  int kof[4] = {0, 0, 0, 0};                       // step that pivoted each owned row
  if (l == 0) {                                    // publish column 0
#pragma unroll
    for (int u = 0; u < 4; ++u) s.gcol[w + 16 * u] = a[u][0];
  }
  for (int k = 0; k < r; ++k) {
    const int b = k & 1;
    const float* colk = s.gcol + 64 * b;
    float* prow = s.grow + 128 * b;
    __syncthreads();
    // every warp: argmax |colk[i]| over the unused rows (ties to the lower row)
    float best = -1.f;
    int bi = 64;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int i = l + 32 * h;
      if (!((used >> i) & 1ull)) {
        const float v = fabsf(colk[i]);
        if (v > best) { best = v; bi = i; }
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    const int p = bi;
    used |= 1ull << p;
    float pv = colk[p];
    if (pv == 0.f) {
      pv = 1e-30f;
      if (threadIdx.x == 0) s.ival[0] = 1;
    }
    const float rp = 1.f / pv;
    if (w == (p & 15)) {
      const int pu = p >> 4;
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (u == pu) {
          kof[u] = k;
#pragma unroll
          for (int v = 0; v < 4; ++v) {
            a[u][v] *= rp;
            prow[l + 32 * v] = a[u][v];
          }
        }
    }
    __syncthreads();
    const int kn = k + 1;
    float* coln = s.gcol + 64 * (b ^ 1);
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = w + 16 * u;
      if (i != p) {
        const float f = -colk[i];
#pragma unroll
        for (int v = 0; v < 4; ++v) a[u][v] = fmaf(f, prow[l + 32 * v], a[u][v]);
      }
      if (l == (kn & 31) && kn < r) coln[i] = (kn >> 5) ? a[u][1] : a[u][0];
    }
  }
  __syncthreads();
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int i = w + 16 * u;
    if (i < r) {
      const int kk = kof[u];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int j = l + 32 * v;
        if (j >= r && j < 2 * r) Xi[kk * ldo + (j - r)] = a[u][v];
      }
    }
  }
  __syncthreads();
}

// Scratch floats newton_polar needs after X: [X | I] (r x (2r+1)) or two r x (r+1) buffers.
__host__ __device__ inline size_t newton_scratch_floats(int r) { return 2 * (size_t)r * (r + 1) + 8; }

// ---- polar factor of a square X (r x r, stride ldx) in place ---------------------------
// Scaled Newton X <- (z X + X^{-T} / z) / 2 (Higham, Frobenius scaling z) while the step is
// large; once a step moves X by less than 10 % it is close to orthogonal and the pivot-free
// Newton-Schulz step X <- X (3 I - X^T X) / 2 finishes the convergence.  When X enters
// upper triangular (the R of a QR), the first inverse is a triangular solve.
// Aug: newton_scratch_floats(r) floats; ldx must be r + 1.
__device__ inline void newton_polar(float* X, int ldx, float* Aug, int r, bool upper,
                                    PolarScratch& s) {
  const int tx = pc_lane(), ty = pc_warp(), nw = pc_nwarps();
  const int la = 2 * r + 1;
  bool schulz = false, last = false;
  for (int it = 0; it < kNewtonMaxIt; ++it) {
    float dn = 0.f, nn = 0.f;
    if (!schulz) {
      // ---- X^{-1}: Xinv[i][j] at Aug[i * la + r + j]
      if (it == 0 && upper) tri_inverse(X, ldx, Aug + r, la, r, s);
      else gj_inverse(X, ldx, Aug, r, s);
      float a = 0.f, b = 0.f;
      for (int i = ty; i < r; i += nw)
        for (int j = tx; j < r; j += 32) {
          a = fmaf(X[i * ldx + j], X[i * ldx + j], a);
          b = fmaf(Aug[i * la + r + j], Aug[i * la + r + j], b);
        }
      a = block_sum<float>(a, s.red);
      b = block_sum<float>(b, s.red);
      float zeta = sqrtf(sqrtf(b) / sqrtf(a));
      if (it >= 1 && fabsf(zeta - 1.f) < 1e-2f) zeta = 1.f;
      const float iz = 1.f / zeta;
      for (int i = ty; i < r; i += nw)
        for (int j = tx; j < r; j += 32) {
          const float x = X[i * ldx + j];
          const float xn = 0.5f * (zeta * x + iz * Aug[j * la + r + i]);
          const float d = xn - x;
          dn = fmaf(d, d, dn);
          nn = fmaf(xn, xn, nn);
          X[i * ldx + j] = xn;
        }
    } else {
      // ---- Newton-Schulz: G = 1.5 I - 0.5 X^T X;  X <- X G
      float* G = Aug;              // r x ldx
      float* Xn = Aug + r * ldx;   // r x ldx
      for (int i = ty; i < r; i += nw)
        for (int j = tx; j < r; j += 32) {
          float acc = 0.f;
          for (int k = 0; k < r; ++k) acc = fmaf(X[k * ldx + i], X[k * ldx + j], acc);
          G[i * ldx + j] = (i == j ? 1.5f : 0.f) - 0.5f * acc;
        }
      __syncthreads();
      for (int i = ty; i < r; i += nw)
        for (int j = tx; j < r; j += 32) {
          float acc = 0.f;
          for (int k = 0; k < r; ++k) acc = fmaf(X[i * ldx + k], G[k * ldx + j], acc);
          Xn[i * ldx + j] = acc;
          const float d = acc - X[i * ldx + j];
          dn = fmaf(d, d, dn);
          nn = fmaf(acc, acc, nn);
        }
      __syncthreads();
      for (int i = ty; i < r; i += nw)
        for (int j = tx; j < r; j += 32) X[i * ldx + j] = Xn[i * ldx + j];
    }
    dn = block_sum<float>(dn, s.red);
    nn = block_sum<float>(nn, s.red);
    __syncthreads();
    const float rel = sqrtf(dn / nn);
    if (last) break;
    if (schulz && rel < 3e-5f) last = true;     // quadratic: one more step reaches ~1e-9
    if (!schulz && rel < 0.1f) schulz = true;
  }
}

// ---- polar factor of X (r <= 64, stride ldx odd) in place, 512 threads -----------------
// One scaled Newton step X <- (zeta X + X^{-T} / zeta) / 2 (the triangular inverse when X is
// the R of a QR) maps every singular value into [1, m]; dividing by
// U = sqrt(||X^T X||_inf) >= sigma_max puts them into [1/U, 1].  Then k quintic steps
// X <- X (a I + b A + c A^2), A = X^T X, with (a, b, c) = (3.4445, -4.7750, 2.0315) raise
// small singular values about 3.2-fold per step (k = ceil(log(0.6 U) / log 3.2)) into
// [0.6, 1.2], and cubic Newton-Schulz steps X <- X (3 I - A) / 2 finish the convergence
// (until a step moves X by less than 3e-5, then one more).  Every step after the first is
// three or two register-tiled r x r products: on the per-bin matrices of a 2,000-cell fit
// (condition numbers 2e7 to 3e12) this replaces 4 Gauss-Jordan inverses per matrix and errs
// against an fp64 polar factor of the same fp32 R by a median 6e-7 (max 3e-6).
// Sc: r x ldx scratch.
__device__ inline void newton_polar_r64(float* X, int ldx, float* Sc, int r, bool upper,
                                        PolarScratch& s) {
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  // ---- 1. scaled Newton step
  if (upper) tri_inverse_blocked(X, ldx, Sc, ldx, r, true, s);
  else gj_inverse_reg(X, ldx, Sc, ldx, r, s);
  {
    float a = 0.f, b = 0.f;
    for (int i = w; i < r; i += 16)
      for (int j = l; j < r; j += 32) {
        a = fmaf(X[i * ldx + j], X[i * ldx + j], a);
        b = fmaf(Sc[i * ldx + j], Sc[i * ldx + j], b);
      }
    a = block_sum<float>(a, s.red);
    b = block_sum<float>(b, s.red);
    const float zeta = sqrtf(sqrtf(b) / sqrtf(a));
    const float iz = 1.f / zeta;
    for (int i = w; i < r; i += 16)
      for (int j = l; j < r; j += 32)
        X[i * ldx + j] = 0.5f * (zeta * X[i * ldx + j] + iz * Sc[j * ldx + i]);
    __syncthreads();
  }
  // ---- 2. scale into [1/U, 1]
  float acc[4][2];
  cta_mm<4, 2>(r, r, r, 0, [&](int i, int k) { return X[k * ldx + i]; },
               [&](int k, int j) { return X[k * ldx + j]; }, acc);
  float rmax = 0.f;
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    float rs = 0.f;
#pragma unroll
    for (int v = 0; v < 2; ++v)
      if (l + 32 * v < r) rs += fabsf(acc[u][v]);
    rs = warp_sum(rs);
    if (w + 16 * u < r) rmax = fmaxf(rmax, rs);
  }
  if (l == 0) s.red[w] = rmax;
  __syncthreads();
  float Ub = 0.f;
  for (int q = 0; q < 16; ++q) Ub = fmaxf(Ub, s.red[q]);
  Ub = sqrtf(Ub);
  __syncthreads();
  {
    const float iu = Ub > 0.f ? 1.f / Ub : 1.f;
    for (int i = w; i < r; i += 16)
      for (int j = l; j < r; j += 32) X[i * ldx + j] *= iu;
    __syncthreads();
  }
  // ---- 3. quintic boost of the small singular values
  int kq = (Ub > 0.f) ? (int)ceilf(logf(0.6f * Ub) / logf(3.2f)) : 0;
  kq = kq < 0 ? 0 : (kq > 16 ? 16 : kq);
  for (int q = 0; q < kq; ++q) {
    cta_mm<4, 2>(r, r, r, 0, [&](int i, int k) { return X[k * ldx + i]; },
                 [&](int k, int j) { return X[k * ldx + j]; }, acc);     // A = X^T X
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 2; ++v) {
        const int i = w + 16 * u, j = l + 32 * v;
        if (i < r && j < r) Sc[i * ldx + j] = acc[u][v];
      }
    __syncthreads();
    float a2[4][2];
    cta_mm<4, 2>(r, r, r, 0, [&](int i, int k) { return Sc[i * ldx + k]; },
                 [&](int k, int j) { return Sc[k * ldx + j]; }, a2);      // A^2
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 2; ++v) {
        const int i = w + 16 * u, j = l + 32 * v;
        if (i < r && j < r)
          Sc[i * ldx + j] = (i == j ? 3.4445f : 0.f) - 4.7750f * acc[u][v] + 2.0315f * a2[u][v];
      }
    __syncthreads();
    cta_mm<4, 2>(r, r, r, 0, [&](int i, int k) { return X[i * ldx + k]; },
                 [&](int k, int j) { return Sc[k * ldx + j]; }, acc);     // X P
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 2; ++v) {
        const int i = w + 16 * u, j = l + 32 * v;
        if (i < r && j < r) X[i * ldx + j] = acc[u][v];
      }
    __syncthreads();
  }
  // ---- 4. cubic Newton-Schulz to convergence
  bool last = false;
  for (int it = 0; it < 16; ++it) {
    float dn = 0.f, nn = 0.f;
    cta_mm<4, 2>(r, r, r, 0, [&](int i, int k) { return X[k * ldx + i]; },
                 [&](int k, int j) { return X[k * ldx + j]; }, acc);
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 2; ++v) {
        const int i = w + 16 * u, j = l + 32 * v;
        if (i < r && j < r) Sc[i * ldx + j] = (i == j ? 1.5f : 0.f) - 0.5f * acc[u][v];
      }
    __syncthreads();
    cta_mm<4, 2>(r, r, r, 0, [&](int i, int k) { return X[i * ldx + k]; },
                 [&](int k, int j) { return Sc[k * ldx + j]; }, acc);
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 2; ++v) {
        const int i = w + 16 * u, j = l + 32 * v;
        if (i < r && j < r) {
          const float d = acc[u][v] - X[i * ldx + j];
          dn = fmaf(d, d, dn);
          nn = fmaf(acc[u][v], acc[u][v], nn);
          X[i * ldx + j] = acc[u][v];
        }
      }
    dn = block_sum<float>(dn, s.red);
    nn = block_sum<float>(nn, s.red);
    __syncthreads();
    if (last) break;
    if (sqrtf(dn / nn) < 3e-5f) last = true;
  }
}


// ---- r x r products on 4 x TJ register tiles (r <= 16 TJ; threads 0 .. 64 TJ - 1) -------
// Thread t owns rows i0 .. i0+3, i0 = 4 (t >> 4), and TJ / 4 column chunks of four: chunk h
// starts at 4 (t & 15) + 64 h, so each float4 access of a half-warp covers 64 consecutive
// floats (conflict-free).  TJ = 4 covers r <= 64 on 256 threads, TJ = 8 covers r <= 128 on
// 512.  acc[u][4 h + e] = sum_{k < r} A[i0 + u][k] B[k][chunk h + e]; fa4(k, i0) returns
// A[i0 .. i0+3][k], B is read as float4 rows (ldb a multiple of 4, the base 16-byte aligned,
// ldb >= 4 ceil(r / 4) + 4 so a chunk starting below r stays inside its row).  Threads past
// 64 TJ, rows past r and chunks starting at or past r leave acc zero.
__device__ __forceinline__ int tile_chunk(int h) { return 4 * (threadIdx.x & 15) + 64 * h; }

template <int TJ, class FA>
__device__ __forceinline__ void mm4t(int r, FA fa4, const float* B, int ldb, float (&acc)[4][TJ]) {
  const int t = threadIdx.x, i0 = 4 * (t >> 4);
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < TJ; ++v) acc[u][v] = 0.f;
  if (t >= 64 * TJ || i0 >= r || tile_chunk(0) >= r) return;
  const bool hi = TJ > 4 && tile_chunk(1) < r;
#pragma unroll 4
  for (int k = 0; k < r; ++k) {
    const float4 a = fa4(k, i0);
    const float av[4] = {a.x, a.y, a.z, a.w};
    float bv[TJ];
#pragma unroll
    for (int h = 0; h < TJ / 4; ++h) {
      float4 b = make_float4(0.f, 0.f, 0.f, 0.f);
      if (h == 0 || hi) b = *reinterpret_cast<const float4*>(B + k * ldb + tile_chunk(h));
      bv[4 * h] = b.x; bv[4 * h + 1] = b.y; bv[4 * h + 2] = b.z; bv[4 * h + 3] = b.w;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < TJ; ++v) acc[u][v] = fmaf(av[u], bv[v], acc[u][v]);
  }
}

// Writes mm4t's tile of C (ldc a multiple of 4): rows i0.. below r, the chunks starting below
// r (their last columns stay inside the row padding).
template <int TJ>
__device__ __forceinline__ void st4t(float* C, int ldc, int r, const float (&v)[4][TJ]) {
  const int t = threadIdx.x, i0 = 4 * (t >> 4);
  if (t >= 64 * TJ || i0 >= r) return;
#pragma unroll
  for (int u = 0; u < 4; ++u)
    if (i0 + u < r)   // rows past r belong to the next buffer
#pragma unroll
      for (int h = 0; h < TJ / 4; ++h)
        if (tile_chunk(h) < r)
          *reinterpret_cast<float4*>(C + (i0 + u) * ldc + tile_chunk(h)) =
              make_float4(v[u][4 * h], v[u][4 * h + 1], v[u][4 * h + 2], v[u][4 * h + 3]);
}

// newton_polar_r64 for an upper-triangular R with its products on 4 x TJ register tiles:
// X and Sc use the row stride ldv (a multiple of 4, 16-byte aligned rows, >= 4 ceil(r/4) + 4),
// the steps and their arithmetic are those of newton_polar_r64 (scaled Newton step with the
// triangular inverse, scaling by sqrt of the largest row sum of X^T X, quintic boosts, cubic
// Newton-Schulz to 3e-5 plus one step).  512 threads; TJ = 4 for r <= 64 (products on threads
// 0..255), TJ = 8 for r <= 128 (products on all 512 threads).
template <int TJ>
__device__ inline void newton_polar_tiled(float* X, int ldv, float* Sc, int r, PolarScratch& s) {
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, t = threadIdx.x;
  const int i0 = 4 * (t >> 4);
  const bool mine = t < 64 * TJ && i0 < r && tile_chunk(0) < r;
  auto jcol = [&](int v) { return tile_chunk(v >> 2) + (v & 3); };   // column of acc[.][v]
  auto at = [&](const float* M, int k, int i) {            // M[i..i+3][k] (rows)
    return make_float4(M[i * ldv + k], M[(i + 1) * ldv + k], M[(i + 2) * ldv + k],
                       M[(i + 3) * ldv + k]);
  };
  auto col = [&](const float* M, int k, int i) {           // M[k][i..i+3] (M symmetric or M^T)
    return *reinterpret_cast<const float4*>(M + k * ldv + i);
  };
  // ---- 1. scaled Newton step
  tri_inverse_blocked(X, ldv, Sc, ldv, r, true, s);
  {
    float a = 0.f, b = 0.f;
    for (int i = w; i < r; i += 16)
      for (int j = l; j < r; j += 32) {
        a = fmaf(X[i * ldv + j], X[i * ldv + j], a);
        b = fmaf(Sc[i * ldv + j], Sc[i * ldv + j], b);
      }
    a = block_sum<float>(a, s.red);
    b = block_sum<float>(b, s.red);
    const float zeta = sqrtf(sqrtf(b) / sqrtf(a));
    const float iz = 1.f / zeta;
    for (int i = w; i < r; i += 16)
      for (int j = l; j < r; j += 32)
        X[i * ldv + j] = 0.5f * (zeta * X[i * ldv + j] + iz * Sc[j * ldv + i]);
    __syncthreads();
  }
  // ---- 2. scale into [1/U, 1]: U = sqrt of the largest row sum of |X^T X|
  float acc[4][TJ];
  mm4t<TJ>(r, [&](int k, int i) { return col(X, k, i); }, X, ldv, acc);
  {
    float rmax = 0.f;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      float rs = 0.f;
#pragma unroll
      for (int v = 0; v < TJ; ++v)
        if (jcol(v) < r) rs += fabsf(acc[u][v]);
      for (int o = 8; o > 0; o >>= 1) rs += __shfl_xor_sync(0xffffffffu, rs, o);  // 16 lanes
      if (mine && i0 + u < r) rmax = fmaxf(rmax, rs);
    }
    for (int o = 16; o > 0; o >>= 1) rmax = fmaxf(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
    if (l == 0) s.red[w] = rmax;
  }
  __syncthreads();
  float Ub = 0.f;
  for (int q = 0; q < 16; ++q) Ub = fmaxf(Ub, s.red[q]);
  Ub = sqrtf(Ub);
  __syncthreads();
  {
    const float iu = Ub > 0.f ? 1.f / Ub : 1.f;
    for (int i = w; i < r; i += 16)
      for (int j = l; j < r; j += 32) X[i * ldv + j] *= iu;
    __syncthreads();
  }
  // ---- 3. quintic boost of the small singular values
  int kq = (Ub > 0.f) ? (int)ceilf(logf(0.6f * Ub) / logf(3.2f)) : 0;
  kq = kq < 0 ? 0 : (kq > 16 ? 16 : kq);
  for (int q = 0; q < kq; ++q) {
    mm4t<TJ>(r, [&](int k, int i) { return col(X, k, i); }, X, ldv, acc);     // A = X^T X
    st4t<TJ>(Sc, ldv, r, acc);
    __syncthreads();
    float a2[4][TJ];
    mm4t<TJ>(r, [&](int k, int i) { return col(Sc, k, i); }, Sc, ldv, a2);   // A^2 (A symmetric)
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < TJ; ++v)
        a2[u][v] = (i0 + u == jcol(v) ? 3.4445f : 0.f) - 4.7750f * acc[u][v] + 2.0315f * a2[u][v];
    st4t<TJ>(Sc, ldv, r, a2);
    __syncthreads();
    mm4t<TJ>(r, [&](int k, int i) { return at(X, k, i); }, Sc, ldv, acc);     // X P
    __syncthreads();
    st4t<TJ>(X, ldv, r, acc);
    __syncthreads();
  }
  // ---- 4. cubic Newton-Schulz to convergence
  bool last = false;
  for (int it = 0; it < 16; ++it) {
    float dn = 0.f, nn = 0.f;
    mm4t<TJ>(r, [&](int k, int i) { return col(X, k, i); }, X, ldv, acc);
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < TJ; ++v) acc[u][v] = (i0 + u == jcol(v) ? 1.5f : 0.f) - 0.5f * acc[u][v];
    st4t<TJ>(Sc, ldv, r, acc);
    __syncthreads();
    mm4t<TJ>(r, [&](int k, int i) { return at(X, k, i); }, Sc, ldv, acc);
    float old[4][TJ] = {};
    if (mine) {
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (i0 + u < r) {
#pragma unroll
          for (int h = 0; h < TJ / 4; ++h)
            if (tile_chunk(h) < r) {
              const float4 o = *reinterpret_cast<const float4*>(X + (i0 + u) * ldv + tile_chunk(h));
              old[u][4 * h] = o.x; old[u][4 * h + 1] = o.y;
              old[u][4 * h + 2] = o.z; old[u][4 * h + 3] = o.w;
            }
        }
    }
    __syncthreads();
    if (mine) {
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < TJ; ++v)
          if (i0 + u < r && jcol(v) < r) {
            const float d = acc[u][v] - old[u][v];
            dn = fmaf(d, d, dn);
            nn = fmaf(acc[u][v], acc[u][v], nn);
          }
    }
    st4t<TJ>(X, ldv, r, acc);
    dn = block_sum<float>(dn, s.red);
    nn = block_sum<float>(nn, s.red);
    __syncthreads();
    if (last) break;
    if (sqrtf(dn / nn) < 3e-5f) last = true;
  }
}

__device__ inline void newton_polar_r64v(float* X, int ldv, float* Sc, int r, PolarScratch& s) {
  newton_polar_tiled<4>(X, ldv, Sc, r, s);
}

}  // namespace fh
