// ALS streaming contractions over the cached RWR output X, fp32 CUDA-core path.
//
// X holds every cell's RWR tiles as X[c][band row], band row = tile.xoff + i*width + j
// (row i, compact column j of a bin batch).  The reference's three passes over X per
// iteration (fasthigashi/parafac2_intergrative.py:374-383, 422-477, 522-529) re-associate
// into two dense products that each read X once:
//
//   W       = X^T E       (band rows x R)   W_i = X_i E feeds both
//             temp_i = X_i (E D) diag(A_i) B^T = W_i M_i  (:336,374-383, K8/K9) and
//             Y_i = U_i^T X_i E = U_i^T W_i               (:522-529, K16)
//   SVD^T   = X G^T       (cells x R)       with G_i = lhs2_i U_i^T, since
//             SVD_term[:, c] = sum_i lhs2_i (U_i^T X_i[:, :, c])   (:422-430, K12-K14)
//
// W computed after the meta-embedding update serves this iteration's Y and the next
// iteration's temp, so an iteration costs two passes over X instead of three passes plus
// three RWR recomputations.
//
// Summation order.  Both passes sum long runs (10,000 cells in W, ~35,000 band rows per split
// in SVD^T at 10,000 cells x 500 kb).  A single fp32 chain over such a run loses about
// sqrt(n) ulps where the terms cancel, and the fitted embedding inherits it (the meta polar
// amplifies the error of SVD^T by its condition number).  Each thread therefore sums one
// staged tile of K (16 or 32 terms) in a fresh fp32 chain and folds that partial into a
// running sum with Kahan compensation: the register that holds the tile's chain starts at
// minus the running compensation, so the fold is three adds and no extra registers.  Split
// partials are added in fp64.
#include "fh_common.cuh"

namespace fh {

// Folds a tile's chain into the running sum (Kahan).  On entry acc = tile sum - c, where c is
// the running compensation; on exit sum holds the new running sum and acc = -c' (the start of
// the next tile's chain).  sum + acc is the compensated total.
__device__ __forceinline__ void kahan_fold(float& sum, float& acc) {
  const float t = sum + acc;
  acc = acc - (t - sum);
  sum = t;
}

// ---------------------------------------------------------------------------------------
// W[row][m] = sum_c X[c][row] * E[c][m]; CTA = 128 band rows x RP, K = cells in steps of 32
// (16 at RP = 128, which keeps the two staged tiles within 48 KB).
// ---------------------------------------------------------------------------------------
constexpr int kXeRows = 128;

template <int RP>
__global__ void __launch_bounds__(256) xe_f32_kernel(const float* __restrict__ X, int64_t ldx,
                                                     int C, const float* __restrict__ E,
                                                     float* __restrict__ W, int64_t rows) {
  constexpr int kXeK = RP >= 128 ? 16 : 32;
  constexpr int MG = RP / 4;          // m-groups of 4
  constexpr int RG = 256 / MG;        // row groups
  constexpr int RPT = kXeRows / RG;   // rows per thread
  __shared__ __align__(16) float Xs[2][kXeK][kXeRows];
  __shared__ __align__(16) float Es[2][kXeK][RP];
  const int tid = threadIdx.x;
  const int mg = tid % MG, rg = tid / MG;
  const int64_t r0 = (int64_t)blockIdx.x * kXeRows;
  const int ntiles = (C + kXeK - 1) / kXeK;

  auto load = [&](int kt, int buf) {
    const int k0 = kt * kXeK;
#pragma unroll
    for (int q = 0; q < (kXeK * kXeRows / 4) / 256; ++q) {
      const int idx = tid + 256 * q;
      const int kk = idx / (kXeRows / 4), c4 = idx % (kXeRows / 4);
      const bool ok = k0 + kk < C;
      cp_async16(&Xs[buf][kk][c4 * 4], X + (ok ? (int64_t)(k0 + kk) * ldx + r0 + c4 * 4 : 0), ok);
    }
    for (int idx = tid; idx < kXeK * RP / 4; idx += 256) {
      const int kk = idx / (RP / 4), m4 = idx % (RP / 4);
      const bool ok = k0 + kk < C;
      cp_async16(&Es[buf][kk][m4 * 4], E + (ok ? (int64_t)(k0 + kk) * RP + m4 * 4 : 0), ok);
    }
    cp_async_commit();
  };

  float acc[RPT][4], sum[RPT][4];   // tile chains (from -compensation) and running sums
#pragma unroll
  for (int i = 0; i < RPT; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = sum[i][j] = 0.f;

  load(0, 0);
  for (int kt = 0; kt < ntiles; ++kt) {
    const int buf = kt & 1;
    if (kt + 1 < ntiles) { load(kt + 1, buf ^ 1); cp_async_wait<1>(); }
    else cp_async_wait<0>();
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < kXeK; ++kk) {
      float xv[RPT];
      const float* xs = &Xs[buf][kk][rg * RPT];
      if constexpr (RPT % 4 == 0) {
#pragma unroll
        for (int i = 0; i < RPT; i += 4) {
          const float4 v = *reinterpret_cast<const float4*>(xs + i);
          xv[i] = v.x; xv[i + 1] = v.y; xv[i + 2] = v.z; xv[i + 3] = v.w;
        }
      } else {
#pragma unroll
        for (int i = 0; i < RPT; ++i) xv[i] = xs[i];
      }
      const float4 ev = *reinterpret_cast<const float4*>(&Es[buf][kk][mg * 4]);
#pragma unroll
      for (int i = 0; i < RPT; ++i) {
        acc[i][0] = fmaf(xv[i], ev.x, acc[i][0]);
        acc[i][1] = fmaf(xv[i], ev.y, acc[i][1]);
        acc[i][2] = fmaf(xv[i], ev.z, acc[i][2]);
        acc[i][3] = fmaf(xv[i], ev.w, acc[i][3]);
      }
    }
#pragma unroll
    for (int i = 0; i < RPT; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) kahan_fold(sum[i][j], acc[i][j]);
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < RPT; ++i) {
    const int64_t r = r0 + rg * RPT + i;
    if (r < rows)
      *reinterpret_cast<float4*>(W + r * RP + mg * 4) =
          make_float4(sum[i][0] + acc[i][0], sum[i][1] + acc[i][1], sum[i][2] + acc[i][2],
                      sum[i][3] + acc[i][3]);
  }
}

// ---------------------------------------------------------------------------------------
// Partial[s][c][m] = sum_{row in split s} X[c][row] * Gt[row][m]; CTA = 128 cells x RP.
// Thread (cg, mg) owns cells cg + 16*i (i < 8) and m = mg*MPT + j.  Band rows are staged 32
// at a time (16 at RP = 128); splits span multiples of 32 rows.
// ---------------------------------------------------------------------------------------
constexpr int kXgCells = 128;
constexpr int kXgSplitK = 32;

template <int RP>
__global__ void __launch_bounds__(256) xg_f32_kernel(const float* __restrict__ X, int64_t ldx,
                                                     int C, const float* __restrict__ Gt,
                                                     int64_t rows, int64_t rows_per_split,
                                                     float* __restrict__ partial) {
  constexpr int kXgK = RP >= 128 ? 16 : 32;
  constexpr int kXgLd = kXgK + 4;
  constexpr int MPT = RP / 16;
  __shared__ __align__(16) float Xs[2][kXgCells][kXgLd];
  __shared__ __align__(16) float Gs[2][kXgK][RP];
  const int tid = threadIdx.x;
  const int mg = tid & 15, cg = tid >> 4;
  const int c0 = blockIdx.x * kXgCells;
  const int s = blockIdx.y;
  const int64_t k_begin = (int64_t)s * rows_per_split;
  int64_t k_end = k_begin + rows_per_split;
  if (k_end > rows) k_end = rows;
  const int ntiles = k_end > k_begin ? (int)((k_end - k_begin + kXgK - 1) / kXgK) : 0;

  auto load = [&](int kt, int buf) {
    const int64_t k0 = k_begin + (int64_t)kt * kXgK;
#pragma unroll
    for (int q = 0; q < (kXgCells * kXgK / 4) / 256; ++q) {
      const int idx = tid + 256 * q;
      const int cc = idx / (kXgK / 4), k4 = idx % (kXgK / 4);
      const bool ok = c0 + cc < C;  // rows past k_end read zero padding of X / Gt
      cp_async16(&Xs[buf][cc][k4 * 4], X + (ok ? (int64_t)(c0 + cc) * ldx + k0 + k4 * 4 : 0), ok);
    }
    for (int idx = tid; idx < kXgK * RP / 4; idx += 256) {
      const int kk = idx / (RP / 4), m4 = idx % (RP / 4);
      const bool ok = k0 + kk < k_end;
      cp_async16(&Gs[buf][kk][m4 * 4], Gt + (ok ? (k0 + kk) * RP + m4 * 4 : 0), ok);
    }
    cp_async_commit();
  };

  float acc[8][MPT], sum[8][MPT];   // tile chains (from -compensation) and running sums
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < MPT; ++j) acc[i][j] = sum[i][j] = 0.f;

  if (ntiles > 0) load(0, 0);
  for (int kt = 0; kt < ntiles; ++kt) {
    const int buf = kt & 1;
    if (kt + 1 < ntiles) { load(kt + 1, buf ^ 1); cp_async_wait<1>(); }
    else cp_async_wait<0>();
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < kXgK; ++kk) {
      float xv[8], gv[MPT];
#pragma unroll
      for (int i = 0; i < 8; ++i) xv[i] = Xs[buf][cg + 16 * i][kk];
#pragma unroll
      for (int j = 0; j < MPT; ++j) gv[j] = Gs[buf][kk][mg * MPT + j];
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < MPT; ++j) acc[i][j] = fmaf(xv[i], gv[j], acc[i][j]);
    }
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < MPT; ++j) kahan_fold(sum[i][j], acc[i][j]);
    __syncthreads();
  }
  float* out = partial + (int64_t)s * C * RP;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int c = c0 + cg + 16 * i;
    if (c < C) {
#pragma unroll
      for (int j = 0; j < MPT; ++j) out[(int64_t)c * RP + mg * MPT + j] = sum[i][j] + acc[i][j];
    }
  }
}

// ---------------------------------------------------------------------------------------
// Y[g][l][m] = sum_j U_g[j][l] W[xoff + i*n + j][m]   (K16 tail), one CTA per bin row g.
// ---------------------------------------------------------------------------------------
template <int RP>
__global__ void __launch_bounds__(256) project_y_kernel(const fh_tile* __restrict__ tiles,
                                                        const int32_t* __restrict__ row_tile,
                                                        const float* __restrict__ U,
                                                        const float* __restrict__ W,
                                                        float* __restrict__ Y, int ldy_l) {
  constexpr int JC = RP >= 128 ? 32 : 64;   // band columns per staged chunk
  __shared__ __align__(16) float Uf[JC * RP];  // U_g rows j0.. (r <= RP floats each, packed)
  __shared__ __align__(16) float Ws[JC * RP];
  const int g = blockIdx.x;
  const fh_tile T = tiles[row_tile[g]];
  const int i = (int)(g - T.brow0);
  const int n = T.width, r = T.rank;
  if (r > RP) return;                        // the staged U rows hold at most RP values
  const float* Ug = U + T.uoff + (int64_t)i * n * r;
  const float* Wg = W + (T.xoff + (int64_t)i * n) * RP;
  const int tid = threadIdx.x;
  // thread tile: l = lg + 16*a (a < LA), m = mg*MPT + b
  constexpr int MPT = RP / 16;
  const int mg = tid & 15, lg = tid >> 4;
  const int LA = (r + 15) / 16;
  float acc[8][MPT];
#pragma unroll
  for (int a = 0; a < 8; ++a)
#pragma unroll
    for (int b = 0; b < MPT; ++b) acc[a][b] = 0.f;
  for (int j0 = 0; j0 < n; j0 += JC) {
    const int jn = min(JC, n - j0);
    // both chunks are contiguous runs in global memory: U_g rows of r floats, W rows of RP
    const float* us = Ug + (int64_t)j0 * r;
#pragma unroll 4
    for (int idx = tid; idx < jn * r; idx += 256) Uf[idx] = us[idx];
    const float4* ws = reinterpret_cast<const float4*>(Wg + (int64_t)j0 * RP);
#pragma unroll 4
    for (int idx = tid; idx < jn * (RP / 4); idx += 256)
      reinterpret_cast<float4*>(Ws)[idx] = ws[idx];
    __syncthreads();
    for (int jj = 0; jj < jn; ++jj) {
      float wv[MPT];
#pragma unroll
      for (int b = 0; b < MPT; ++b) wv[b] = Ws[jj * RP + mg * MPT + b];
#pragma unroll
      for (int a = 0; a < 8; ++a) {
        if (a < LA) {
          const int l = lg + 16 * a;
          const float uv = l < r ? Uf[jj * r + l] : 0.f;
#pragma unroll
          for (int b = 0; b < MPT; ++b) acc[a][b] = fmaf(uv, wv[b], acc[a][b]);
        }
      }
    }
    __syncthreads();
  }
  float* Yg = Y + (int64_t)g * ldy_l * RP;
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const int l = lg + 16 * a;
    if (a < LA && l < r) {
#pragma unroll
      for (int b = 0; b < MPT; ++b) Yg[(int64_t)l * RP + mg * MPT + b] = acc[a][b];
    }
  }
}

}  // namespace fh

using namespace fh;

static bool rp_ok(int rp) { return rp == 16 || rp == 32 || rp == 64 || rp == 128; }

extern "C" int fh_xe_f32(const float* X, int64_t ldx, int32_t n_cells, int64_t rows,
                         const float* E, int32_t rp, float* W, void* stream) {
  if (!X || !E || !W || n_cells <= 0 || rows <= 0 || ldx < rows || ldx % 128 || !rp_ok(rp))
    return FH_ERR_ARG;
  const unsigned grid = (unsigned)ceil_div(rows, kXeRows);
  cudaStream_t s = (cudaStream_t)stream;
  switch (rp) {
    case 16: xe_f32_kernel<16><<<grid, 256, 0, s>>>(X, ldx, n_cells, E, W, rows); break;
    case 32: xe_f32_kernel<32><<<grid, 256, 0, s>>>(X, ldx, n_cells, E, W, rows); break;
    case 64: xe_f32_kernel<64><<<grid, 256, 0, s>>>(X, ldx, n_cells, E, W, rows); break;
    default: xe_f32_kernel<128><<<grid, 256, 0, s>>>(X, ldx, n_cells, E, W, rows); break;
  }
  FH_CHECK_LAUNCH();
  return FH_OK;
}

extern "C" int fh_xg_splits(int32_t n_cells, int64_t rows) {
  const int64_t ct = ceil_div(n_cells, kXgCells);
  int64_t s = ceil_div(3 * 152, ct);
  const int64_t max_s = ceil_div(rows, 4 * kXgSplitK);
  if (s > max_s) s = max_s;
  if (s < 1) s = 1;
  return (int)s;
}

extern "C" int fh_xg_f32(const float* X, int64_t ldx, int32_t n_cells, int64_t rows,
                         const float* Gt, int32_t rp, int32_t splits, float* partial,
                         float* out, int32_t accumulate, void* stream) {
  if (!X || !Gt || !partial || !out || n_cells <= 0 || rows <= 0 || ldx < rows || ldx % 128 ||
      !rp_ok(rp) || splits <= 0)
    return FH_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  int64_t per = ceil_div(ceil_div(rows, splits), kXgSplitK) * kXgSplitK;
  dim3 grid((unsigned)ceil_div(n_cells, kXgCells), (unsigned)splits);
  switch (rp) {
    case 16: xg_f32_kernel<16><<<grid, 256, 0, s>>>(X, ldx, n_cells, Gt, rows, per, partial); break;
    case 32: xg_f32_kernel<32><<<grid, 256, 0, s>>>(X, ldx, n_cells, Gt, rows, per, partial); break;
    case 64: xg_f32_kernel<64><<<grid, 256, 0, s>>>(X, ldx, n_cells, Gt, rows, per, partial); break;
    default: xg_f32_kernel<128><<<grid, 256, 0, s>>>(X, ldx, n_cells, Gt, rows, per, partial); break;
  }
  const int64_t n = (int64_t)n_cells * rp;
  reduce_splits_kernel<float><<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(partial, splits, n, out,
                                                                      accumulate != 0);
  FH_CHECK_LAUNCH();
  return FH_OK;
}

extern "C" int fh_project_y_f32(const fh_tile* tiles, const int32_t* row_tile, int64_t n_rows,
                                const float* U, const float* W, int32_t rp, float* Y,
                                int32_t ldy_l, void* stream) {
  if (!tiles || !row_tile || !U || !W || !Y || n_rows <= 0 || !rp_ok(rp) || ldy_l <= 0 ||
      ldy_l > kMaxRank)
    return FH_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  switch (rp) {
    case 16: project_y_kernel<16><<<(unsigned)n_rows, 256, 0, s>>>(tiles, row_tile, U, W, Y, ldy_l); break;
    case 32: project_y_kernel<32><<<(unsigned)n_rows, 256, 0, s>>>(tiles, row_tile, U, W, Y, ldy_l); break;
    case 64: project_y_kernel<64><<<(unsigned)n_rows, 256, 0, s>>>(tiles, row_tile, U, W, Y, ldy_l); break;
    default: project_y_kernel<128><<<(unsigned)n_rows, 256, 0, s>>>(tiles, row_tile, U, W, Y, ldy_l); break;
  }
  FH_CHECK_LAUNCH();
  return FH_OK;
}
