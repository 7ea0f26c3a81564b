// CP-ALS inner solver on the projected tensors Y_chrom (nbin x r x R), all chromosomes at once.
//
// Reference: fasthigashi/parafac_integrative.py:12-112 (update_factor, balance_norm, parafac)
// called per chromosome from parafac2_intergrative.py:674-695, and the core norm
// ||[[A, B, D]]||^2 of :621-632 / :697-706.
//
// One sweep updates A, B, D in turn from the normal equations
//     A <- MTTKRP_A (B^T B * D^T D + 1e-10 I)^{-1}   (and likewise for B, D)
//     MTTKRP_A[i] = sum_j B[j] * (Y_i D)[j],   MTTKRP_B = sum_i A_i (x) (Y_i D),
//     MTTKRP_D   = sum_i A_i (x) (Y_i^T B)      ((x): column-wise product).
// The r x r systems (symmetric positive definite) are formed and inverted in fp64 by
// Gauss-Jordan without pivoting (the sweep operator) once per chromosome, and the B and D
// right-hand sides are multiplied by the fp64 inverse with fp64 sums, so every solve is a
// register-tiled product instead of a serial substitution; the A rows (many small solves in
// cp_rows_kernel) use the fp64 inverse rounded to fp32.  The reference solves in fp32
// (parafac_integrative.py:12-15).  Scalar sums (loss, core norm) are fp64 too.  The reconstruction loss needs no Xhat:
// ||Xhat||^2 = sum(A^TA * B^TB * D^TD) and <Xhat, Y> = sum(D * MTTKRP_D) with the final
// A, B.  balance_norm (unit columns, the product of the column norms folded into D) follows
// each sweep unless the relative loss change fell below 1e-5, as the reference breaks before
// balancing.
//
// Bin rows are processed in chunks of <= 8 rows of one chromosome; per-chunk partial sums
// are reduced in a fixed order by the per-chromosome kernel (deterministic).
//
// The kernels are instantiated for ranks up to MR = 64 (256 threads) and up to MR = 128
// (512 threads): 4 MR threads, outputs on 8 x (MR / 32) register tiles.  At MR = 128 the
// row kernel keeps two Y tiles and one factor in shared memory and holds Y_g D in registers;
// B and the A-row inverse are read from global memory (L2).
#include "fh_common.cuh"

namespace fh {

constexpr int kCpMaxR = 128;  // r and R handled by these kernels

// Launch shape of the MR instantiation: 4 MR threads, NW warps, output tiles 8 x TN.
template <int MR>
struct CpShape {
  static constexpr int NT = 4 * MR, NW = NT / 32, TN = MR / 32;
  static constexpr int LY = MR + 4;   // row stride of the Y tiles (16-byte rows for cp.async)
  static constexpr int LZ = MR + 1;   // odd stride of the staged factors
};

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
  float* L;        // [chrom][ld][ld]    inverse of the A-row system (B^T B * D^T D + 1e-10 I)
  float* part;     // [chunk][pstride]
  float* gAA;      // [chrom][ld*ld]
  float* gBB;
  float* gDD;
  float* scaleA;   // [chrom][ld]
  double* ynorm;   // [chrom]
  double* loss;    // [chrom][2]: previous, current
  int* state;      // [chrom]: bit 0 converged (stop), bit 1 first sweep done
  double* core;    // [chrom] ||[[A,B,D]]||^2
  double* cross;   // [chrom] <[[A,B,D]], Y> of the last sweep (optional)
  int* status;
};

enum CpRowMode { kRowsNorm = 0, kRowsAB = 1, kRowsD = 2, kRowsScale = 3, kRowsGram = 4 };
// kSmallDLast: the D update of a call's last sweep, whose balanced Grams and A-row inverse
// nobody reads (the next call starts from kSmallInit).
enum CpSmallMode { kSmallInit = 0, kSmallB = 1, kSmallD = 2, kSmallCore = 3, kSmallDLast = 4 };

__host__ __device__ inline size_t cp_pstride(int ld) { return (size_t)2 * ld * ld + 2; }
// Dynamic shared memory of cp_rows_kernel<MR>: two Y tiles and four factor tiles (MR = 64),
// or two Y tiles, one factor tile and the warps' column partials (MR = 128).
template <int MR>
constexpr size_t cp_rows_smem() {
  using S = CpShape<MR>;
  return MR <= 64 ? (2 * (size_t)MR * S::LY + 4 * (size_t)MR * S::LZ) * sizeof(float)
                  : (2 * (size_t)MR * S::LY + (size_t)MR * S::LZ + (size_t)S::NW * MR) *
                        sizeof(float);
}

// sum over k < nk of p[k * stride], in increasing k (the loads go out eight at a time)
__device__ __forceinline__ float chunk_sum(const float* p, size_t stride, int nk) {
  float s = 0.f;
  int k = 0;
  for (; k + 8 <= nk; k += 8) {
    float v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = p[(size_t)(k + u) * stride];
#pragma unroll
    for (int u = 0; u < 8; ++u) s += v[u];
  }
  for (; k < nk; ++k) s += p[(size_t)k * stride];
  return s;
}

// acc[u][v] = sum_k fa(w + NW u, k) fb(k, lane + 32v) over k < K for the 4 MR threads (rows
// w + NW u, u < 8; columns lane + 32 v, v < TN), rows / columns clamped to M-1 / N-1.
template <int MR, class FA, class FB>
__device__ __forceinline__ void cp_mm(int M, int N, int K, FA fa, FB fb,
                                      float (&acc)[8][CpShape<MR>::TN]) {
  constexpr int NW = CpShape<MR>::NW, TN = CpShape<MR>::TN;
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  int ri[8], cj[TN];
#pragma unroll
  for (int u = 0; u < 8; ++u) ri[u] = min(w + NW * u, M - 1);
#pragma unroll
  for (int v = 0; v < TN; ++v) cj[v] = min(l + 32 * v, N - 1);
#pragma unroll
  for (int u = 0; u < 8; ++u)
#pragma unroll
    for (int v = 0; v < TN; ++v) acc[u][v] = 0.f;
  for (int k = 0; k < K; ++k) {
    float av[8], bv[TN];
#pragma unroll
    for (int u = 0; u < 8; ++u) av[u] = fa(ri[u], k);
#pragma unroll
    for (int v = 0; v < TN; ++v) bv[v] = fb(k, cj[v]);
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
      for (int v = 0; v < TN; ++v) acc[u][v] = fmaf(av[u], bv[v], acc[u][v]);
  }
}

template <int MR>
__global__ void __launch_bounds__(4 * MR) cp_rows_kernel(CpArgs a, int mode) {
  using S = CpShape<MR>;
  constexpr int NT = S::NT, NW = S::NW, TN = S::TN, LY = S::LY, LZ = S::LZ;
  extern __shared__ __align__(16) float cps[];
  float* Yb = cps;                        // two Y_g tiles (r x RP, stride LY): row i, row i+1
  float* Fs = Yb + 2 * MR * LY;           // D (R x r) or B (r x r)
  // MR <= 64: B, Y_g D and the A-row inverse staged too; MR = 128: the warps' partials
  float* Bs = Fs + MR * LZ;               // B (mode AB)
  float* Zs = Bs + MR * LZ;               // Y_g D (r x r)
  float* Ls = Zs + MR * LZ;               // the A-row system's inverse (mode AB)
  float* red = Fs + MR * LZ;              // [NW][MR] (MR = 128)
  __shared__ float rhs[MR];
  __shared__ float ysol[MR];
  __shared__ float red4[4][MR];
  __shared__ double dred[32];
  const int k = blockIdx.x;
  const int ci = a.k_chrom[k];
  if (mode != kRowsNorm && mode != kRowsGram && (a.state[ci] & 1)) return;
  const int r = a.c_rank[ci], R = a.R, ld = a.ld, lz = LZ;
  const int64_t row0 = a.k_row0[k];
  const int nrow = a.k_nrow[k];
  const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;

  if (mode == kRowsScale) {
    const float* sc = a.scaleA + (size_t)ci * ld;
    for (int i = ty; i < nrow; i += NW)
      for (int p = tx; p < r; p += 32) a.A[(row0 + i) * ld + p] *= sc[p];
    return;
  }
  float* out = a.part + (size_t)k * cp_pstride(ld);
  if (mode == kRowsNorm || mode == kRowsGram) {
    // partial A^T A (diagonal only for kRowsNorm) and ||Y||^2 of the chunk
    for (int p = ty; p < r; p += NW)
      for (int q = tx; q < r; q += 32) {
        float s = 0.f;
        if (mode == kRowsGram || p == q)
          for (int i = 0; i < nrow; ++i) s = fmaf(a.A[(row0 + i) * ld + p], a.A[(row0 + i) * ld + q], s);
        out[p * ld + q] = s;
      }
    // ||Y||^2 of the chunk's rows as one contiguous run, four floats per load
    float ys[4] = {0.f, 0.f, 0.f, 0.f};
    const int64_t per = (int64_t)a.ldy * a.RP;
    const float* Y0 = a.Y + row0 * per;
#pragma unroll 4
    for (int64_t e = (int64_t)tid * 4; e < nrow * per; e += NT * 4) {
      const float4 v = *reinterpret_cast<const float4*>(Y0 + e);
      const int64_t wv = e % per;
      const int j = (int)(wv / a.RP), m = (int)(wv % a.RP);
      if (j < r) {
        const float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (m + u < R) ys[u] = fmaf(vv[u], vv[u], ys[u]);
      }
    }
    const double ysd = block_sum<double>((double)((ys[0] + ys[1]) + (ys[2] + ys[3])), dred);
    if (tid == 0) reinterpret_cast<double*>(out + 2 * ld * ld)[0] = ysd;
    return;
  }
  // ---- mode AB (solve the A rows, then the partials of A^T A and MTTKRP_B) or D
  const float* Dc = a.D + (size_t)ci * a.RP * ld;
  const float* Bc = a.B + (size_t)ci * ld * ld;
  const float* Lc = a.L + (size_t)ci * ld * ld;
  if (mode == kRowsAB) {
    for (int m = ty; m < R; m += NW)
      for (int q = tx; q < r; q += 32) Fs[m * lz + q] = Dc[m * ld + q];
    if constexpr (MR <= 64) {
      for (int j = ty; j < r; j += NW)
        for (int q = tx; q < r; q += 32) {
          Bs[j * lz + q] = Bc[j * ld + q];
          Ls[j * lz + q] = Lc[j * ld + q];
        }
    }
  } else {
    for (int j = ty; j < r; j += NW)
      for (int q = tx; q < r; q += 32) Fs[j * lz + q] = Bc[j * ld + q];
  }
  float pA[TN][8], pB[TN][8];   // partials at (row p = ty + NW u, column q = tx + 32v)
#pragma unroll
  for (int v = 0; v < TN; ++v)
#pragma unroll
    for (int u = 0; u < 8; ++u) pA[v][u] = pB[v][u] = 0.f;
  // Y_g tiles through a two-deep cp.async ring: row i + 1 loads while row i is used
  const int q4 = a.RP / 4;
  auto load_y = [&](int i) {
    const float* Yg = a.Y + (row0 + i) * (int64_t)a.ldy * a.RP;
    float* dst = Yb + (i & 1) * MR * LY;
    for (int idx = tid; idx < r * q4; idx += NT) {
      const int j = idx / q4, c = idx - j * q4;
      cp_async16(dst + j * LY + 4 * c, Yg + (int64_t)j * a.RP + 4 * c, true);
    }
    cp_async_commit();
  };
  if (nrow > 0) load_y(0);
  for (int i = 0; i < nrow; ++i) {
    const int64_t g = row0 + i;
    if (i + 1 < nrow) { load_y(i + 1); cp_async_wait<1>(); }
    else cp_async_wait<0>();
    __syncthreads();
    const float* Ys = Yb + (i & 1) * MR * LY;
    const int ly = LY;
    if (mode == kRowsAB) {
      // Z[j][q] = sum_m Y[j][m] D[m][q]
      float zc[8][TN];
      cp_mm<MR>(r, r, R, [&](int j, int m) { return Ys[j * ly + m]; },
                [&](int m, int q) { return Fs[m * lz + q]; }, zc);
      if constexpr (MR <= 64) {
#pragma unroll
        for (int u = 0; u < 8; ++u)
#pragma unroll
          for (int v = 0; v < TN; ++v) {
            const int j = ty + NW * u, q = tx + 32 * v;
            if (j < r && q < r) Zs[j * lz + q] = zc[u][v];
          }
        __syncthreads();
        // rhs[q] = sum_j B[j][q] Z[j][q]: four partial sums per column, then their sum
        {
          const int q = tid & (MR - 1), part = tid / MR;
          float s = 0.f;
          if (q < r)
            for (int j = part; j < r; j += 4) s = fmaf(Bs[j * lz + q], Zs[j * lz + q], s);
          red4[part][q] = s;
        }
        __syncthreads();
        if (tid < r) rhs[tid] = (red4[0][tid] + red4[1][tid]) + (red4[2][tid] + red4[3][tid]);
        __syncthreads();
        // A_g = G_A^{-1} rhs with the inverse the per-chromosome kernel left in L
        {
          const int p = tid & (MR - 1), part = tid / MR;
          float s = 0.f;
          if (p < r)
            for (int q = part; q < r; q += 4) s = fmaf(Ls[p * lz + q], rhs[q], s);
          red4[part][p] = s;
        }
        __syncthreads();
        if (tid < r) {
          const float s = (red4[0][tid] + red4[1][tid]) + (red4[2][tid] + red4[3][tid]);
          ysol[tid] = s;
          a.A[g * ld + tid] = s;
        }
        __syncthreads();
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int p = ty + NW * u;
          if (p < r) {
#pragma unroll
            for (int v = 0; v < TN; ++v) {
              const int q = tx + 32 * v;
              if (q < r) {
                pA[v][u] = fmaf(ysol[p], ysol[q], pA[v][u]);           // A^T A
                pB[v][u] = fmaf(ysol[q], Zs[p * lz + q], pB[v][u]);    // MTTKRP_B[p][q]
              }
            }
          }
        }
      } else {
        // Z stays in registers: rhs[q] = sum_j B[j][q] Z[j][q] as per-warp partials, summed
        // over the warps in order
#pragma unroll
        for (int v = 0; v < TN; ++v) {
          const int q = tx + 32 * v;
          float s = 0.f;
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const int j = ty + NW * u;
            if (j < r && q < r) s = fmaf(__ldg(Bc + j * ld + q), zc[u][v], s);
          }
          red[ty * MR + q] = s;
        }
        __syncthreads();
        if (tid < r) {
          float s = 0.f;
          for (int w = 0; w < NW; ++w) s += red[w * MR + tid];
          rhs[tid] = s;
        }
        __syncthreads();
        // A_g = G_A^{-1} rhs: one warp per row of the inverse, lanes along its columns
        for (int p = ty; p < r; p += NW) {
          float s = 0.f;
          for (int q = tx; q < r; q += 32) s = fmaf(__ldg(Lc + p * ld + q), rhs[q], s);
          s = warp_sum(s);
          if (tx == 0) {
            ysol[p] = s;
            a.A[g * ld + p] = s;
          }
        }
        __syncthreads();
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int p = ty + NW * u;
          if (p < r) {
#pragma unroll
            for (int v = 0; v < TN; ++v) {
              const int q = tx + 32 * v;
              if (q < r) {
                pA[v][u] = fmaf(ysol[p], ysol[q], pA[v][u]);           // A^T A
                pB[v][u] = fmaf(ysol[q], zc[u][v], pB[v][u]);          // MTTKRP_B[p][q]
              }
            }
          }
        }
      }
      __syncthreads();
    } else {
      // MTTKRP_D[m][q] += A[q] * sum_j Y[j][m] B[j][q]
      const float* Ag = a.A + g * ld;
      float ag[TN];
#pragma unroll
      for (int v = 0; v < TN; ++v) ag[v] = tx + 32 * v < r ? Ag[tx + 32 * v] : 0.f;
      float yb[8][TN];
      cp_mm<MR>(R, r, r, [&](int m, int j) { return Ys[j * ly + m]; },
                [&](int j, int q) { return Fs[j * lz + q]; }, yb);
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int m = ty + NW * u;
        if (m < R) {
#pragma unroll
          for (int v = 0; v < TN; ++v) {
            const int q = tx + 32 * v;
            if (q < r) pA[v][u] = fmaf(ag[v], yb[u][v], pA[v][u]);
          }
        }
      }
      __syncthreads();
    }
  }
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    const int p = ty + NW * u;
#pragma unroll
    for (int v = 0; v < TN; ++v) {
      const int q = tx + 32 * v;
      if (mode == kRowsAB) {
        if (p < r && q < r) {
          out[p * ld + q] = pA[v][u];
          out[ld * ld + p * ld + q] = pB[v][u];
        }
      } else if (p < R && q < r) {
        out[p * ld + q] = pA[v][u];
      }
    }
  }
}

// Gram F^T F of an (nrows x r, stride ld) factor into G (stride ld), fp32.
template <int MR>
__device__ void cp_gram(const float* F, int nrows, int r, int ld, float* G) {
  constexpr int NW = CpShape<MR>::NW, TN = CpShape<MR>::TN;
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  float acc[8][TN];
  cp_mm<MR>(r, r, nrows, [&](int p, int i) { return F[i * ld + p]; },
            [&](int i, int q) { return F[i * ld + q]; }, acc);
#pragma unroll
  for (int u = 0; u < 8; ++u)
#pragma unroll
    for (int v = 0; v < TN; ++v) {
      const int p = w + NW * u, q = l + 32 * v;
      if (p < r && q < r) G[p * ld + q] = acc[u][v];
    }
}

// Dynamic shared memory of cp_small_kernel: the fp64 system, inverted in place (ld x (ld + 1)
// doubles), the inverse's two fp64 scratch rows and an RP x ld fp32 work tile.
__host__ __device__ inline size_t cp_small_smem(int ld, int rp, int mr) {
  return ((size_t)ld * (ld + 1) + 2 * (size_t)mr) * sizeof(double) + (size_t)rp * ld * sizeof(float);
}

// In place: Gd (r x r, stride lg, SPD) <- Gd^{-1} in fp64 by Gauss-Jordan without pivoting
// (the sweep operator; an SPD matrix's pivots are positive), two barriers per pivot.
// scratch: 2 MR doubles.  Returns false on a pivot that is not positive (in every thread).
template <int MR>
__device__ bool cp_spd_inverse_d(double* Gd, int r, int lg, double* scratch) {
  constexpr int NW = CpShape<MR>::NW;
  __shared__ int bad;
  const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
  double* prow = scratch;
  double* pcol = scratch + MR;
  if (tid == 0) bad = 0;
  __syncthreads();
  for (int k = 0; k < r; ++k) {
    if (tid < r) {
      prow[tid] = Gd[k * lg + tid];
      pcol[tid] = Gd[tid * lg + k];
    }
    __syncthreads();
    double d = prow[k];
    if (!(d > 0.0)) {
      d = 1e-300;
      if (tid == 0) bad = 1;
    }
    const double inv = 1.0 / d;
    for (int p = ty; p < r; p += NW) {
      const double cp = pcol[p] * inv;
      for (int q = tx; q < r; q += 32) {
        double v;
        if (p == k) v = (q == k) ? inv : prow[q] * inv;
        else if (q == k) v = -cp;
        else v = fma(-cp, prow[q], Gd[p * lg + q]);
        Gd[p * lg + q] = v;
      }
    }
    __syncthreads();
  }
  return bad == 0;
}

// out rows = RHS rows Gd^{-1} (RHS fp32 nrhs x r, stride ldr; Gd the fp64 inverse, stride lg),
// summed in fp64 and rounded once.
template <int MR>
__device__ void cp_apply_inverse_d(const float* RHS, int ldr, int nrhs, const double* Gd, int r,
                                   int lg, float* out, int ldo) {
  constexpr int NW = CpShape<MR>::NW, TN = CpShape<MR>::TN;
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  int ri[8], cj[TN];
#pragma unroll
  for (int u = 0; u < 8; ++u) ri[u] = min(w + NW * u, nrhs - 1);
#pragma unroll
  for (int v = 0; v < TN; ++v) cj[v] = min(l + 32 * v, r - 1);
  double acc[8][TN];
#pragma unroll
  for (int u = 0; u < 8; ++u)
#pragma unroll
    for (int v = 0; v < TN; ++v) acc[u][v] = 0.0;
  for (int p = 0; p < r; ++p) {
    double av[8], bv[TN];
#pragma unroll
    for (int u = 0; u < 8; ++u) av[u] = (double)RHS[(size_t)ri[u] * ldr + p];
#pragma unroll
    for (int v = 0; v < TN; ++v) bv[v] = Gd[p * lg + cj[v]];
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
      for (int v = 0; v < TN; ++v) acc[u][v] = fma(av[u], bv[v], acc[u][v]);
  }
#pragma unroll
  for (int u = 0; u < 8; ++u)
#pragma unroll
    for (int v = 0; v < TN; ++v) {
      const int row = w + NW * u, q = l + 32 * v;
      if (row < nrhs && q < r) out[(size_t)row * ldo + q] = (float)acc[u][v];
    }
}

template <int MR>
__global__ void __launch_bounds__(4 * MR) cp_small_kernel(CpArgs a, int mode) {
  constexpr int NW = CpShape<MR>::NW;
  extern __shared__ __align__(16) float sf[];
  const int ci = blockIdx.x;
  const int r = a.c_rank[ci], R = a.R, ld = a.ld;
  const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
  const int lg = ld + 1;                  // odd stride: column walks hit distinct banks
  double* Gd = reinterpret_cast<double*>(sf);   // ld x lg: the system, inverted in place (fp64)
  double* Li = Gd + ld * lg;              // 2 MR: scratch rows of the inverse
  float* work = reinterpret_cast<float*>(Li + 2 * MR);   // RP*ld
  __shared__ double dred[32];
  __shared__ float nA[MR], nB[MR], nD[MR];
  __shared__ int stop;
  float* gAA = a.gAA + (size_t)ci * ld * ld;
  float* gBB = a.gBB + (size_t)ci * ld * ld;
  float* gDD = a.gDD + (size_t)ci * ld * ld;
  float* Bc = a.B + (size_t)ci * ld * ld;
  float* Dc = a.D + (size_t)ci * a.RP * ld;
  float* Lc = a.L + (size_t)ci * ld * ld;
  const int k0 = a.c_chunk0[ci], nk = a.c_nchunk[ci];
  const size_t ps = cp_pstride(ld);

  if (mode == kSmallCore) {
    for (int p = ty; p < r; p += NW)
      for (int q = tx; q < r; q += 32) {
        gAA[p * ld + q] = chunk_sum(a.part + k0 * ps + p * ld + q, ps, nk);
      }
    cp_gram<MR>(Bc, r, r, ld, gBB);
    cp_gram<MR>(Dc, R, r, ld, gDD);
    __syncthreads();
    double c = 0.0;
    for (int p = ty; p < r; p += NW)
      for (int q = tx; q < r; q += 32)
        c += (double)gAA[p * ld + q] * (double)gBB[p * ld + q] * (double)gDD[p * ld + q];
    c = block_sum<double>(c, dred);
    if (tid == 0) a.core[ci] = c;
    return;
  }
  if (mode == kSmallInit) {
    // column norms of A, ||Y||^2, then balance (parafac_integrative.py:19-27, :65)
    if (tid < r) nA[tid] = sqrtf(chunk_sum(a.part + k0 * ps + tid * ld + tid, ps, nk));
    if (tid == 0) {
      double s = 0.0;
      for (int k = 0; k < nk; ++k)
        s += reinterpret_cast<const double*>(a.part + (k0 + k) * ps + 2 * ld * ld)[0];
      a.ynorm[ci] = s;
      a.state[ci] = 0;
      a.loss[2 * ci] = 0.0;
      a.loss[2 * ci + 1] = 0.0;
    }
    cp_gram<MR>(Bc, r, r, ld, gBB);
    cp_gram<MR>(Dc, R, r, ld, gDD);
    __syncthreads();
  } else if (a.state[ci] & 1) {
    return;
  }

  if (mode == kSmallB) {
    // A^T A, MTTKRP_B; G_B = A^T A * D^T D + 1e-10 I; B <- MTTKRP_B G_B^{-1}
    for (int p = ty; p < r; p += NW)
      for (int q = tx; q < r; q += 32) {
        const float s = chunk_sum(a.part + k0 * ps + p * ld + q, ps, nk);
        const float t = chunk_sum(a.part + k0 * ps + ld * ld + p * ld + q, ps, nk);
        gAA[p * ld + q] = s;
        work[p * ld + q] = t;
        Gd[p * lg + q] = (double)s * (double)gDD[p * ld + q] + (p == q ? 1e-10 : 0.0);
      }
    __syncthreads();
    if (!cp_spd_inverse_d<MR>(Gd, r, lg, Li) && tid == 0) set_status(a.status, FH_ERR_ILLCOND);
    cp_apply_inverse_d<MR>(work, ld, r, Gd, r, lg, Bc, ld);
    __syncthreads();
    cp_gram<MR>(Bc, r, r, ld, gBB);
    return;
  }
  if (mode == kSmallD || mode == kSmallDLast) {
    // MTTKRP_D; G_D = A^T A * B^T B + 1e-10 I; D <- MTTKRP_D G_D^{-1}; loss; balance
    for (int m = ty; m < R; m += NW)
      for (int q = tx; q < r; q += 32) {
        work[m * ld + q] = chunk_sum(a.part + k0 * ps + m * ld + q, ps, nk);
      }
    for (int p = ty; p < r; p += NW)
      for (int q = tx; q < r; q += 32)
        Gd[p * lg + q] = (double)gAA[p * ld + q] * (double)gBB[p * ld + q] + (p == q ? 1e-10 : 0.0);
    __syncthreads();
    if (!cp_spd_inverse_d<MR>(Gd, r, lg, Li) && tid == 0) set_status(a.status, FH_ERR_ILLCOND);
    cp_apply_inverse_d<MR>(work, ld, R, Gd, r, lg, Dc, ld);
    __syncthreads();
    cp_gram<MR>(Dc, R, r, ld, gDD);
    __syncthreads();
    double xh = 0.0, xy = 0.0;
    for (int p = ty; p < r; p += NW)
      for (int q = tx; q < r; q += 32)
        xh += (double)gAA[p * ld + q] * (double)gBB[p * ld + q] * (double)gDD[p * ld + q];
    for (int m = ty; m < R; m += NW)
      for (int q = tx; q < r; q += 32) xy += (double)Dc[m * ld + q] * (double)work[m * ld + q];
    xh = block_sum<double>(xh, dred);
    xy = block_sum<double>(xy, dred);
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
      if (tid < r) a.scaleA[(size_t)ci * ld + tid] = 1.f;
      return;
    }
    if (tid < r) nA[tid] = sqrtf(gAA[tid * ld + tid]);
    __syncthreads();
  }
  // ---- balance_norm: A /= |A|, B /= |B|, D = D / |D| * (|A||B||D| + 1e-15)
  if (tid < r) {
    nB[tid] = sqrtf(gBB[tid * ld + tid]);
    nD[tid] = sqrtf(gDD[tid * ld + tid]);
  }
  __syncthreads();
  if (tid < r) a.scaleA[(size_t)ci * ld + tid] = 1.f / (nA[tid] + 1e-15f);
  for (int j = ty; j < r; j += NW)
    for (int q = tx; q < r; q += 32) Bc[j * ld + q] = Bc[j * ld + q] / (nB[q] + 1e-15f);
  for (int m = ty; m < R; m += NW)
    for (int q = tx; q < r; q += 32)
      Dc[m * ld + q] = Dc[m * ld + q] / (nD[q] + 1e-15f) * (nA[q] * nB[q] * nD[q] + 1e-15f);
  __syncthreads();
  if (mode == kSmallDLast) return;
  // Grams of the balanced factors; the inverse of B^T B * D^T D + 1e-10 I for the next A rows
  cp_gram<MR>(Bc, r, r, ld, gBB);
  cp_gram<MR>(Dc, R, r, ld, gDD);
  __syncthreads();
  for (int p = ty; p < r; p += NW)
    for (int q = tx; q < r; q += 32)
      Gd[p * lg + q] = (double)gBB[p * ld + q] * (double)gDD[p * ld + q] + (p == q ? 1e-10 : 0.0);
  __syncthreads();
  if (!cp_spd_inverse_d<MR>(Gd, r, lg, Li) && tid == 0) set_status(a.status, FH_ERR_ILLCOND);
  for (int p = ty; p < r; p += NW)
    for (int q = tx; q < r; q += 32) Lc[p * ld + q] = (float)Gd[p * lg + q];
}

}  // namespace fh

using namespace fh;

extern "C" size_t fh_cp_workspace(int32_t nchrom, int32_t nchunks, int32_t ld, int32_t rp) {
  const size_t l = (size_t)ld * ld;
  (void)rp;
  return sizeof(double) * (size_t)nchrom * 4 +
         sizeof(float) * ((size_t)nchrom * (4 * l + ld) + (size_t)nchunks * cp_pstride(ld)) +
         sizeof(int) * (size_t)nchrom + 256;
}

template <int MR>
static int cp_launch(int32_t nchrom, int32_t nchunks, const int32_t* meta, float* A, float* B,
                     float* D, const float* Y, int32_t ld, int32_t rp, int32_t R, int32_t ldy,
                     int32_t n_iter, double* core, double* cross, void* workspace, int* status,
                     void* stream) {
  constexpr int NT = CpShape<MR>::NT;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t l = (size_t)ld * ld;
  CpArgs a{};
  a.nchrom = nchrom;
  a.c_row0 = meta; a.c_nbin = meta + nchrom; a.c_rank = meta + 2 * nchrom;
  a.c_chunk0 = meta + 3 * nchrom; a.c_nchunk = meta + 4 * nchrom;
  a.k_chrom = meta + 5 * nchrom; a.k_row0 = a.k_chrom + nchunks; a.k_nrow = a.k_row0 + nchunks;
  a.A = A; a.B = B; a.D = D; a.Y = Y; a.ld = ld; a.RP = rp; a.R = R; a.ldy = ldy;
  double* w = (double*)workspace;
  a.ynorm = w; w += nchrom;
  a.loss = w; w += 2 * (size_t)nchrom;
  w += nchrom;  // spare
  float* f = (float*)w;
  a.L = f; f += nchrom * l;
  a.gAA = f; f += nchrom * l;
  a.gBB = f; f += nchrom * l;
  a.gDD = f; f += nchrom * l;
  a.scaleA = f; f += (size_t)nchrom * ld;
  f = (float*)(((uintptr_t)f + 15) & ~(uintptr_t)15);
  a.part = f; f += (size_t)nchunks * cp_pstride(ld);
  a.state = (int*)f;
  a.core = core;
  a.cross = cross;
  a.status = status;
  const size_t small_smem = cp_small_smem(ld, rp, MR);
  const size_t rs = cp_rows_smem<MR>();
  if (small_smem > 227 * 1024) return FH_ERR_UNSUPPORTED;
  if (ensure_smem((const void*)cp_small_kernel<MR>, small_smem) ||
      ensure_smem((const void*)cp_rows_kernel<MR>, rs))
    return FH_ERR_LAUNCH;
  if (n_iter == 0) {  // core norm only, factors untouched
    cp_rows_kernel<MR><<<nchunks, NT, rs, s>>>(a, kRowsGram);
    cp_small_kernel<MR><<<nchrom, NT, small_smem, s>>>(a, kSmallCore);
    FH_CHECK_LAUNCH();
    return FH_OK;
  }
  // Each sweep recomputes every A row from Y, B and D, so the A scaling of a balance only
  // matters after the last sweep: the initial balance and the intermediate ones rescale B
  // and D (in place) and leave A to the next sweep.
  cp_rows_kernel<MR><<<nchunks, NT, rs, s>>>(a, kRowsNorm);
  cp_small_kernel<MR><<<nchrom, NT, small_smem, s>>>(a, kSmallInit);
  for (int it = 0; it < n_iter; ++it) {
    cp_rows_kernel<MR><<<nchunks, NT, rs, s>>>(a, kRowsAB);
    cp_small_kernel<MR><<<nchrom, NT, small_smem, s>>>(a, kSmallB);
    cp_rows_kernel<MR><<<nchunks, NT, rs, s>>>(a, kRowsD);
    cp_small_kernel<MR><<<nchrom, NT, small_smem, s>>>(a, it + 1 < n_iter ? kSmallD : kSmallDLast);
  }
  cp_rows_kernel<MR><<<nchunks, NT, rs, s>>>(a, kRowsScale);
  FH_CHECK_LAUNCH();
  return FH_OK;
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
  if (ld > 64) return cp_launch<128>(nchrom, nchunks, meta, A, B, D, Y, ld, rp, R, ldy, n_iter,
                                     core, cross, workspace, status, stream);
  return cp_launch<64>(nchrom, nchunks, meta, A, B, D, Y, ld, rp, R, ldy, n_iter, core, cross,
                       workspace, status, stream);
}

// core[chrom] = ||[[A, B, D]]||^2 without changing the factors (parafac2_intergrative.py:621-632).
extern "C" int fh_core_norm(int32_t nchrom, int32_t nchunks, const int32_t* meta, float* A,
                            float* B, float* D, const float* Y, int32_t ld, int32_t rp,
                            int32_t R, int32_t ldy, double* core, void* workspace,
                            size_t workspace_bytes, int* status, void* stream) {
  return fh_cp_als(nchrom, nchunks, meta, A, B, D, Y, ld, rp, R, ldy, 0, core, nullptr,
                   workspace, workspace_bytes, status, stream);
}
