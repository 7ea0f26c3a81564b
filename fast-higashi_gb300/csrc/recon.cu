// Fused per-cell reconstruction loss of the fit and its backward pass (fp32 CUDA cores).
//
// The model reconstructs bin batch i of a chromosome as X_i[:, :, c] ~ U_i lhs_i[c]^T with
// lhs_i[c][l] = sum_rho A[i][rho] B[l][rho] (E D)[c][rho]  (parafac2_intergrative.py:336-383,
// the KR product of A, B and E D).  In the band-row layout of the cached RWR output
// (X[c][band row], band row = tile.xoff + i*width + j) that is X ~ E Gt^T with
// Gt_i = U_i B diag(A_i) D^T, the rows fh_projection_g_f32 writes.  The per-cell loss is
//   L_c = sum_rows (X[c][row] - sum_m E[c][m] Gt[row][m])^2
// and, for weights w_c = dOut/dL_c,
//   dE[c]    = -2 w_c sum_rows Res[c][row] Gt[row]
//   dGt[row] = -2 sum_c w_c Res[c][row] E[c]
//   drp      =  2 sum_c w_c sum_rows Res[c][row] X'[c][row]     (X' = dX/drp, rwr_grad.cu)
// with Res = X - E Gt^T formed tile by tile in shared memory and never stored: the loss
// has no ||X||^2 - 2<X, E Gt^T> + ||E Gt^T||^2 cancellation.  Two streaming kernels:
//   recon_cells_kernel  CTA = 64 cells x a split of the band rows: loss, dE and drp partials
//   recon_rows_kernel   CTA = 64 band rows x all cells: dGt
// Both form a 64 x 64 residual tile per step (a K = RP product), then fold it into their
// accumulator with a second K = 64 product.  Reductions run in a fixed order.
#include "fh_common.cuh"

namespace fh {

constexpr int kRcT = 64;         // cells and band rows of a residual tile
constexpr int kRcLd = kRcT + 4;  // row stride of the X, X' and residual tiles

struct RcArgs {
  const float* X;
  const float* Xp;      // X' (backward of recon_cells only)
  int64_t ldx;
  int C;
  int64_t rows;
  const float* Gt;      // [row][RP]
  const float* E;       // [cell][RP]
  const double* w;      // [cell] (backward)
  double* ploss;        // [split][cell]
  double* pdrp;         // [split][cell]
  float* pE;            // [split][cell][RP]
  float* dGt;           // [row][RP]
};

// res[i][j] = X[tc + 16 i][tr + 16 j] - sum_m Es[tc + 16 i][m] Gs[tr + 16 j][m] for cells
// below cmax and rows below rmax, 0 elsewhere (the select keeps padding garbage out).
template <int RP>
__device__ __forceinline__ void residual_tile(const float* __restrict__ Xs,
                                              const float* __restrict__ Es,
                                              const float* __restrict__ Gs, int tc, int tr,
                                              int cmax, int rmax, float (&res)[4][4]) {
  constexpr int LG = RP + 4;
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
#pragma unroll 2
  for (int m = 0; m < RP; m += 4) {
    float4 e[4], g[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) e[i] = *reinterpret_cast<const float4*>(Es + (tc + 16 * i) * LG + m);
#pragma unroll
    for (int j = 0; j < 4; ++j) g[j] = *reinterpret_cast<const float4*>(Gs + (tr + 16 * j) * LG + m);
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        acc[i][j] = fmaf(e[i].x, g[j].x, acc[i][j]);
        acc[i][j] = fmaf(e[i].y, g[j].y, acc[i][j]);
        acc[i][j] = fmaf(e[i].z, g[j].z, acc[i][j]);
        acc[i][j] = fmaf(e[i].w, g[j].w, acc[i][j]);
      }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = tc + 16 * i, r = tr + 16 * j;
      res[i][j] = (c < cmax && r < rmax) ? Xs[c * kRcLd + r] - acc[i][j] : 0.f;
    }
}

// Kahan's compensated summation: s - c carries the running sum to about twice fp32
// precision.  The per-tile partials added here are sums of 64 products.
__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
  const float y = x - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

// 64 rows of RP floats (row stride RP in global, LG in shared); rows >= valid read zeros.
template <int RP>
__device__ __forceinline__ void load_rows_rp(float* dst, const float* src, int valid, int tid) {
  constexpr int LG = RP + 4, Q = RP / 4;
  for (int idx = tid; idx < kRcT * Q; idx += 256) {
    const int rr = idx / Q, q = idx % Q;
    const bool ok = rr < valid;
    cp_async16(dst + rr * LG + 4 * q, src + (ok ? (int64_t)rr * RP + 4 * q : 0), ok);
  }
}

// 64 cells x 64 band rows of X starting at (c0, r0); cells >= valid read zeros.
__device__ __forceinline__ void load_x_tile(float* dst, const float* X, int64_t ldx, int c0,
                                            int64_t r0, int valid, int tid) {
#pragma unroll
  for (int q = 0; q < kRcT * kRcT / 4 / 256; ++q) {
    const int idx = tid + 256 * q;
    const int cc = idx >> 4, r4 = idx & 15;
    const bool ok = cc < valid;
    cp_async16(dst + cc * kRcLd + 4 * r4,
               X + (ok ? (int64_t)(c0 + cc) * ldx + r0 + 4 * r4 : 0), ok);
  }
}

__host__ __device__ inline size_t rc_cells_smem(int rp, bool bwd) {
  const int lg = rp + 4;
  return (size_t)(3 * kRcT * lg + (bwd ? 5 : 2) * kRcT * kRcLd) * sizeof(float);
}
__host__ __device__ inline size_t rc_rows_smem(int rp) {
  const int lg = rp + 4;
  return (size_t)(3 * kRcT * lg + 3 * kRcT * kRcLd) * sizeof(float);
}

template <int RP, bool BWD>
__global__ void __launch_bounds__(256) recon_cells_kernel(RcArgs a, int64_t rows_per_split) {
  constexpr int LG = RP + 4;
  constexpr int MG = RP / 4, CG = 256 / MG, CPT = kRcT / CG;
  extern __shared__ __align__(16) float sm[];
  float* Es = sm;                                   // 64 x LG
  float* Gs = Es + kRcT * LG;                       // 2 x 64 x LG
  float* Xs = Gs + 2 * kRcT * LG;                   // 2 x 64 x kRcLd
  float* Ps = Xs + 2 * kRcT * kRcLd;                // 2 x 64 x kRcLd (X', backward)
  float* Rs = Ps + 2 * kRcT * kRcLd;                // 64 x kRcLd     (residual, backward)
  const int tid = threadIdx.x, tc = tid & 15, tr = tid >> 4;
  const int mg = tid % MG, cg = tid / MG;
  const int c0 = blockIdx.x * kRcT, s = blockIdx.y;
  const int cvalid = min(kRcT, a.C - c0);
  const int64_t k_begin = (int64_t)s * rows_per_split;
  const int64_t k_end = a.rows < k_begin + rows_per_split ? a.rows : k_begin + rows_per_split;
  const int nt = k_end > k_begin ? (int)ceil_div(k_end - k_begin, kRcT) : 0;

  auto load = [&](int kt, int buf) {
    const int64_t r0 = k_begin + (int64_t)kt * kRcT;
    load_rows_rp<RP>(Gs + buf * kRcT * LG, a.Gt + r0 * RP, (int)(a.rows - r0 < kRcT ? a.rows - r0 : kRcT), tid);
    load_x_tile(Xs + buf * kRcT * kRcLd, a.X, a.ldx, c0, r0, cvalid, tid);
    if (BWD) load_x_tile(Ps + buf * kRcT * kRcLd, a.Xp, a.ldx, c0, r0, cvalid, tid);
    cp_async_commit();
  };

  load_rows_rp<RP>(Es, a.E + (int64_t)c0 * RP, cvalid, tid);
  double lacc[4] = {0, 0, 0, 0}, dacc[4] = {0, 0, 0, 0};
  float eacc[CPT][4], ecmp[CPT][4];
#pragma unroll
  for (int i = 0; i < CPT; ++i)
#pragma unroll
    for (int q = 0; q < 4; ++q) eacc[i][q] = ecmp[i][q] = 0.f;

  if (nt > 0) load(0, 0);
  for (int kt = 0; kt < nt; ++kt) {
    const int buf = kt & 1;
    if (kt + 1 < nt) { load(kt + 1, buf ^ 1); cp_async_wait<1>(); }
    else cp_async_wait<0>();
    __syncthreads();
    const int64_t left = k_end - (k_begin + (int64_t)kt * kRcT);
    const int rmax = (int)(left < kRcT ? left : kRcT);
    const float* xs = Xs + buf * kRcT * kRcLd;
    const float* gs = Gs + buf * kRcT * LG;
    float res[4][4];
    residual_tile<RP>(xs, Es, gs, tc, tr, cvalid, rmax, res);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      float l = 0.f;
#pragma unroll
      for (int j = 0; j < 4; ++j) l = fmaf(res[i][j], res[i][j], l);
      lacc[i] += (double)l;
    }
    if (BWD) {
      const float* ps = Ps + buf * kRcT * kRcLd;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        float d = 0.f;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int c = tc + 16 * i, r = tr + 16 * j;
          const float p = (c < cvalid && r < rmax) ? ps[c * kRcLd + r] : 0.f;
          d = fmaf(res[i][j], p, d);
          Rs[c * kRcLd + r] = res[i][j];
        }
        dacc[i] += (double)d;
      }
      __syncthreads();
      // eacc[i][q] += sum_r Rs[cg*CPT + i][r] * Gs[r][mg*4 + q]
      float et[CPT][4];
#pragma unroll
      for (int i = 0; i < CPT; ++i)
#pragma unroll
        for (int q = 0; q < 4; ++q) et[i][q] = 0.f;
#pragma unroll 2
      for (int r = 0; r < kRcT; r += 4) {
        float4 g[4], rv[CPT];
#pragma unroll
        for (int u = 0; u < 4; ++u) g[u] = *reinterpret_cast<const float4*>(gs + (r + u) * LG + mg * 4);
#pragma unroll
        for (int i = 0; i < CPT; ++i)
          rv[i] = *reinterpret_cast<const float4*>(Rs + (cg * CPT + i) * kRcLd + r);
#pragma unroll
        for (int i = 0; i < CPT; ++i) {
          const float rr[4] = {rv[i].x, rv[i].y, rv[i].z, rv[i].w};
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            et[i][0] = fmaf(rr[u], g[u].x, et[i][0]);
            et[i][1] = fmaf(rr[u], g[u].y, et[i][1]);
            et[i][2] = fmaf(rr[u], g[u].z, et[i][2]);
            et[i][3] = fmaf(rr[u], g[u].w, et[i][3]);
          }
        }
      }
#pragma unroll
      for (int i = 0; i < CPT; ++i)
#pragma unroll
        for (int q = 0; q < 4; ++q) kahan_add(eacc[i][q], ecmp[i][q], et[i][q]);
    }
    __syncthreads();
  }

  cp_async_wait<0>();   // the E tile when this split has no rows
  __syncthreads();
  // per-cell sums over the 16 row groups, in a fixed order
  double* red = reinterpret_cast<double*>(Xs);      // 2 x 16 x 64 doubles (16 KB)
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    red[tr * kRcT + tc + 16 * i] = lacc[i];
    red[16 * kRcT + tr * kRcT + tc + 16 * i] = dacc[i];
  }
  __syncthreads();
  if (tid < kRcT && tid < cvalid) {
    double l = 0, d = 0;
    for (int g = 0; g < 16; ++g) {
      l += red[g * kRcT + tid];
      d += red[16 * kRcT + g * kRcT + tid];
    }
    a.ploss[(int64_t)s * a.C + c0 + tid] = l;
    if (BWD) a.pdrp[(int64_t)s * a.C + c0 + tid] = d;
  }
  if (BWD) {
#pragma unroll
    for (int i = 0; i < CPT; ++i) {
      const int c = cg * CPT + i;
      if (c < cvalid)
        *reinterpret_cast<float4*>(a.pE + ((int64_t)s * a.C + c0 + c) * RP + mg * 4) =
            make_float4(eacc[i][0] - ecmp[i][0], eacc[i][1] - ecmp[i][1],
                        eacc[i][2] - ecmp[i][2], eacc[i][3] - ecmp[i][3]);
    }
  }
}

template <int RP>
__global__ void __launch_bounds__(256) recon_rows_kernel(RcArgs a) {
  constexpr int LG = RP + 4;
  constexpr int MG = RP / 4, RG = 256 / MG, RPT = kRcT / RG;
  extern __shared__ __align__(16) float sm[];
  float* Gs = sm;                                   // 64 x LG
  float* Es = Gs + kRcT * LG;                       // 2 x 64 x LG
  float* Xs = Es + 2 * kRcT * LG;                   // 2 x 64 x kRcLd
  float* Rs = Xs + 2 * kRcT * kRcLd;                // 64 x kRcLd: w_c Res[c][r]
  const int tid = threadIdx.x, tc = tid & 15, tr = tid >> 4;
  const int mg = tid % MG, rg = tid / MG;
  const int64_t r0 = (int64_t)blockIdx.x * kRcT;
  const int rmax = (int)(a.rows - r0 < kRcT ? a.rows - r0 : kRcT);
  const int nt = (int)ceil_div(a.C, kRcT);

  auto load = [&](int kt, int buf) {
    const int c0 = kt * kRcT;
    const int cv = min(kRcT, a.C - c0);
    load_rows_rp<RP>(Es + buf * kRcT * LG, a.E + (int64_t)c0 * RP, cv, tid);
    load_x_tile(Xs + buf * kRcT * kRcLd, a.X, a.ldx, c0, r0, cv, tid);
    cp_async_commit();
  };

  load_rows_rp<RP>(Gs, a.Gt + r0 * RP, rmax, tid);
  float acc[RPT][4], cmp[RPT][4];
#pragma unroll
  for (int i = 0; i < RPT; ++i)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[i][q] = cmp[i][q] = 0.f;

  load(0, 0);
  for (int kt = 0; kt < nt; ++kt) {
    const int buf = kt & 1;
    if (kt + 1 < nt) { load(kt + 1, buf ^ 1); cp_async_wait<1>(); }
    else cp_async_wait<0>();
    __syncthreads();
    const int c0 = kt * kRcT;
    const int cv = min(kRcT, a.C - c0);
    const float* es = Es + buf * kRcT * LG;
    float res[4][4];
    residual_tile<RP>(Xs + buf * kRcT * kRcLd, es, Gs, tc, tr, cv, rmax, res);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int c = tc + 16 * i;
      const float wc = c < cv ? (float)a.w[c0 + c] : 0.f;
#pragma unroll
      for (int j = 0; j < 4; ++j) Rs[c * kRcLd + tr + 16 * j] = wc * res[i][j];
    }
    __syncthreads();
    // acc[i][q] += sum_c Rs[c][rg*RPT + i] * Es[c][mg*4 + q]
    float at[RPT][4];
#pragma unroll
    for (int i = 0; i < RPT; ++i)
#pragma unroll
      for (int q = 0; q < 4; ++q) at[i][q] = 0.f;
#pragma unroll 4
    for (int c = 0; c < kRcT; ++c) {
      const float4 e = *reinterpret_cast<const float4*>(es + c * LG + mg * 4);
      float rv[RPT];
      if constexpr (RPT % 4 == 0) {
#pragma unroll
        for (int i = 0; i < RPT; i += 4) {
          const float4 v = *reinterpret_cast<const float4*>(Rs + c * kRcLd + rg * RPT + i);
          rv[i] = v.x; rv[i + 1] = v.y; rv[i + 2] = v.z; rv[i + 3] = v.w;
        }
      } else if constexpr (RPT == 2) {
        const float2 v = *reinterpret_cast<const float2*>(Rs + c * kRcLd + rg * RPT);
        rv[0] = v.x; rv[1] = v.y;
      } else {
#pragma unroll
        for (int i = 0; i < RPT; ++i) rv[i] = Rs[c * kRcLd + rg * RPT + i];
      }
#pragma unroll
      for (int i = 0; i < RPT; ++i) {
        at[i][0] = fmaf(rv[i], e.x, at[i][0]);
        at[i][1] = fmaf(rv[i], e.y, at[i][1]);
        at[i][2] = fmaf(rv[i], e.z, at[i][2]);
        at[i][3] = fmaf(rv[i], e.w, at[i][3]);
      }
    }
#pragma unroll
    for (int i = 0; i < RPT; ++i)
#pragma unroll
      for (int q = 0; q < 4; ++q) kahan_add(acc[i][q], cmp[i][q], at[i][q]);
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < RPT; ++i) {
    const int r = rg * RPT + i;
    if (r < rmax)
      *reinterpret_cast<float4*>(a.dGt + (r0 + r) * RP + mg * 4) =
          make_float4(-2.f * (acc[i][0] - cmp[i][0]), -2.f * (acc[i][1] - cmp[i][1]),
                      -2.f * (acc[i][2] - cmp[i][2]), -2.f * (acc[i][3] - cmp[i][3]));
  }
}

// loss[c] = sum_s ploss[s][c]; backward: dE[c][m] = -2 w_c sum_s pE[s][c][m] and
// cdrp[c] = sum_s pdrp[s][c]
template <bool BWD>
__global__ void recon_finish_kernel(RcArgs a, int splits, int rp, double* loss, float* dE,
                                    double* cdrp) {
  const int64_t n = (int64_t)a.C * rp;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i / rp), m = (int)(i % rp);
    if (m == 0) {
      double l = 0, d = 0;
      for (int s = 0; s < splits; ++s) {
        l += a.ploss[(int64_t)s * a.C + c];
        if (BWD) d += a.pdrp[(int64_t)s * a.C + c];
      }
      if (loss) loss[c] = l;
      if (BWD) cdrp[c] = d;
    }
    if (BWD) {
      float e = 0.f;
      for (int s = 0; s < splits; ++s) e += a.pE[(int64_t)s * n + i];
      dE[i] = (float)(-2.0 * a.w[c]) * e;
    }
  }
}

// drp = 2 sum_c w_c cdrp[c] (one CTA, fixed order)
__global__ void recon_drp_kernel(const double* w, const double* cdrp, int C, double* drp) {
  __shared__ double red[32];
  double s = 0;
  for (int c = threadIdx.x; c < C; c += blockDim.x) s += w[c] * cdrp[c];
  s = block_sum<double>(s, red);
  if (threadIdx.x == 0) *drp = 2.0 * s;
}

static int rc_splits(int C, int64_t rows) {
  const int64_t ct = ceil_div(C, kRcT);
  int64_t s = ceil_div(4 * 152, ct);
  const int64_t max_s = ceil_div(rows, 4 * kRcT);   // at least 4 tiles per split
  if (s > max_s) s = max_s;
  if (s < 1) s = 1;
  return (int)s;
}

struct RcWorkspace {
  double* ploss;
  double* pdrp;
  double* cdrp;
  float* pE;
};

static size_t rc_layout(int C, int64_t rows, int rp, char* base, RcWorkspace* w) {
  const int s = rc_splits(C, rows);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off += (bytes + 255) & ~(size_t)255;
    return base ? base + o : nullptr;
  };
  RcWorkspace t;
  t.ploss = reinterpret_cast<double*>(take((size_t)s * C * sizeof(double)));
  t.pdrp = reinterpret_cast<double*>(take((size_t)s * C * sizeof(double)));
  t.cdrp = reinterpret_cast<double*>(take((size_t)C * sizeof(double)));
  t.pE = reinterpret_cast<float*>(take((size_t)s * C * rp * sizeof(float)));
  if (w) *w = t;
  return off;
}

template <int RP, bool BWD>
static int launch_cells(const RcArgs& a, int splits, int64_t per, cudaStream_t st) {
  const size_t smem = rc_cells_smem(RP, BWD);
  auto k = recon_cells_kernel<RP, BWD>;
  if (ensure_smem((const void*)k, smem)) return FH_ERR_LAUNCH;
  dim3 grid((unsigned)ceil_div(a.C, kRcT), (unsigned)splits);
  k<<<grid, 256, smem, st>>>(a, per);
  FH_CHECK_LAUNCH();
  return FH_OK;
}

template <int RP>
static int launch_rows(const RcArgs& a, cudaStream_t st) {
  const size_t smem = rc_rows_smem(RP);
  auto k = recon_rows_kernel<RP>;
  if (ensure_smem((const void*)k, smem)) return FH_ERR_LAUNCH;
  k<<<(unsigned)ceil_div(a.rows, kRcT), 256, smem, st>>>(a);
  FH_CHECK_LAUNCH();
  return FH_OK;
}

template <bool BWD>
static int run_cells(const RcArgs& a, int rp, int splits, int64_t per, cudaStream_t st) {
  switch (rp) {
    case 16: return launch_cells<16, BWD>(a, splits, per, st);
    case 32: return launch_cells<32, BWD>(a, splits, per, st);
    case 64: return launch_cells<64, BWD>(a, splits, per, st);
    default: return FH_ERR_UNSUPPORTED;
  }
}

// ---------------------------------------------------------------------------------------
// Factor gradients from H_g = U_g^T dGt_g (bin row g; H[g][l][m], l < ldh, m < RP), which
// fh_project_y_f32 forms from dGt exactly as it forms Y from W.  With Gt_g = U_g B diag(A_g)
// D^T (chromosome c of bin row g):
//   T_g[l][rho]  = sum_m H_g[l][m] D_c[m][rho]
//   dA[g][rho]   = sum_l B_c[l][rho] T_g[l][rho]
//   dB_c[l][rho] = sum_g A[g][rho] T_g[l][rho]
//   dD_c[m][rho] = sum_g A[g][rho] sum_l H_g[l][m] B_c[l][rho]
// One CTA per chunk of <= 8 bin rows of one chromosome (the CP-ALS chunk table) writes its
// dB and dD partials; factor_grad_reduce_kernel adds a chromosome's chunks in order.
// ---------------------------------------------------------------------------------------
constexpr int kFgMax = 64;         // r and RP handled here
constexpr int kFgLd = kFgMax + 1;

struct FgArgs {
  const int32_t* c_rank;
  const int32_t* c_chunk0;
  const int32_t* c_nchunk;
  const int32_t* k_chrom;
  const int32_t* k_row0;
  const int32_t* k_nrow;
  const float* H;   // [bin rows][ldh][RP]
  const float* A;   // [bin rows][ld]
  const float* B;   // [chrom][ld][ld]
  const float* D;   // [chrom][RP][ld]
  int ld, RP, R, ldh;
  float* dA;        // [bin rows][ld]
  float* pB;        // [chunk][ld][ld]
  float* pD;        // [chunk][RP][ld]
  float* dB;        // [chrom][ld][ld]
  float* dD;        // [chrom][RP][ld]
};

__global__ void __launch_bounds__(256) factor_grad_chunk_kernel(FgArgs a) {
  extern __shared__ float fsm[];
  float(*Bs)[kFgLd] = reinterpret_cast<float(*)[kFgLd]>(fsm);   // B_c[l][rho]
  float(*Ds)[kFgLd] = Bs + kFgMax;                               // D_c[m][rho]
  float(*Hs)[kFgLd] = Ds + kFgMax;                               // H_g[l][m]
  float(*Ts)[kFgLd] = Hs + kFgMax;                               // T_g[l][rho]
  const int k = blockIdx.x, tid = threadIdx.x;
  const int ci = a.k_chrom[k], g0 = a.k_row0[k], ng = a.k_nrow[k];
  const int r = a.c_rank[ci], R = a.R, ld = a.ld;
  const float* Bc = a.B + (size_t)ci * ld * ld;
  const float* Dc = a.D + (size_t)ci * a.RP * ld;
  for (int i = tid; i < kFgMax * kFgMax; i += 256) {
    const int p = i / kFgMax, q = i % kFgMax;
    Bs[p][q] = (p < r && q < r) ? Bc[p * ld + q] : 0.f;
    Ds[p][q] = (p < R && q < r) ? Dc[p * ld + q] : 0.f;
  }
  // this thread's entries (p, q) = (e / 64, e % 64), e = tid + 256 u: rows p of dB (l) and
  // of dD (m), column q = rho
  float accB[16], accD[16];
#pragma unroll
  for (int u = 0; u < 16; ++u) accB[u] = accD[u] = 0.f;
  for (int gi = 0; gi < ng; ++gi) {
    const int g = g0 + gi;
    __syncthreads();
    for (int i = tid; i < kFgMax * kFgMax; i += 256) {
      const int p = i / kFgMax, q = i % kFgMax;
      Hs[p][q] = (p < r && q < R) ? a.H[((int64_t)g * a.ldh + p) * a.RP + q] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int e = tid + 256 * u, p = e >> 6, q = e & 63;
      float t = 0.f, v = 0.f;
      for (int x = 0; x < kFgMax; ++x) {
        t = fmaf(Hs[p][x], Ds[x][q], t);   // T[l = p][rho = q]
        v = fmaf(Hs[x][p], Bs[x][q], v);   // (H^T B)[m = p][rho = q]
      }
      const float aq = q < r ? a.A[(int64_t)g * ld + q] : 0.f;
      Ts[p][q] = t;
      accB[u] = fmaf(aq, t, accB[u]);
      accD[u] = fmaf(aq, v, accD[u]);
    }
    __syncthreads();
    if (tid < ld) {
      float s = 0.f;
      if (tid < r)
        for (int l = 0; l < r; ++l) s = fmaf(Bs[l][tid], Ts[l][tid], s);
      a.dA[(int64_t)g * ld + tid] = s;
    }
  }
  float* pB = a.pB + (size_t)k * ld * ld;
  float* pD = a.pD + (size_t)k * a.RP * ld;
#pragma unroll
  for (int u = 0; u < 16; ++u) {
    const int e = tid + 256 * u, p = e >> 6, q = e & 63;
    if (p < ld && q < ld) pB[p * ld + q] = accB[u];
    if (p < a.RP && q < ld) pD[p * ld + q] = accD[u];
  }
}

__global__ void factor_grad_reduce_kernel(FgArgs a) {
  const int ci = blockIdx.x;
  const int k0 = a.c_chunk0[ci], nk = a.c_nchunk[ci];
  const int ld = a.ld, nb = ld * ld, nd = a.RP * ld;
  for (int i = threadIdx.x; i < nb + nd; i += blockDim.x) {
    float s = 0.f;
    if (i < nb) {
      for (int k = 0; k < nk; ++k) s += a.pB[(size_t)(k0 + k) * nb + i];
      a.dB[(size_t)ci * nb + i] = s;
    } else {
      const int j = i - nb;
      for (int k = 0; k < nk; ++k) s += a.pD[(size_t)(k0 + k) * nd + j];
      a.dD[(size_t)ci * nd + j] = s;
    }
  }
}

}  // namespace fh

using namespace fh;

extern "C" size_t fh_recon_workspace(int32_t n_cells, int64_t rows, int32_t rp) {
  if (n_cells <= 0 || rows <= 0 || rp <= 0) return 0;
  return rc_layout(n_cells, rows, rp, nullptr, nullptr);
}

static int rc_check(const float* X, int64_t ldx, int32_t n_cells, int64_t rows, const float* Gt,
                    const float* E, int32_t rp, void* ws, size_t ws_bytes) {
  if (!X || !Gt || !E || !ws || n_cells <= 0 || rows <= 0 || ldx < rows || ldx % 64)
    return FH_ERR_ARG;
  if (rp != 16 && rp != 32 && rp != 64) return FH_ERR_UNSUPPORTED;
  if (ws_bytes < rc_layout(n_cells, rows, rp, nullptr, nullptr)) return FH_ERR_ARG;
  return FH_OK;
}

extern "C" int fh_recon_loss_f32(const float* X, int64_t ldx, int32_t n_cells, int64_t rows,
                                 const float* Gt, const float* E, int32_t rp, double* loss,
                                 void* ws, size_t ws_bytes, void* stream) {
  int st = rc_check(X, ldx, n_cells, rows, Gt, E, rp, ws, ws_bytes);
  if (st) return st;
  if (!loss) return FH_ERR_ARG;
  RcWorkspace w;
  rc_layout(n_cells, rows, rp, static_cast<char*>(ws), &w);
  RcArgs a{};
  a.X = X; a.ldx = ldx; a.C = n_cells; a.rows = rows; a.Gt = Gt; a.E = E;
  a.ploss = w.ploss; a.pdrp = w.pdrp; a.pE = w.pE;
  const int splits = rc_splits(n_cells, rows);
  const int64_t per = ceil_div(ceil_div(rows, splits), kRcT) * kRcT;
  cudaStream_t s = (cudaStream_t)stream;
  if ((st = run_cells<false>(a, rp, splits, per, s))) return st;
  recon_finish_kernel<false><<<(unsigned)ceil_div((int64_t)n_cells * rp, 256), 256, 0, s>>>(
      a, splits, rp, loss, nullptr, nullptr);
  FH_CHECK_LAUNCH();
  return FH_OK;
}

extern "C" int fh_recon_loss_bwd_f32(const float* X, const float* Xp, int64_t ldx,
                                     int32_t n_cells, int64_t rows, const float* Gt,
                                     const float* E, int32_t rp, const double* w, double* loss,
                                     float* dE, float* dGt, double* drp, void* ws,
                                     size_t ws_bytes, void* stream) {
  int st = rc_check(X, ldx, n_cells, rows, Gt, E, rp, ws, ws_bytes);
  if (st) return st;
  if (!Xp || !w || !dE || !dGt || !drp) return FH_ERR_ARG;
  RcWorkspace wk;
  rc_layout(n_cells, rows, rp, static_cast<char*>(ws), &wk);
  RcArgs a{};
  a.X = X; a.Xp = Xp; a.ldx = ldx; a.C = n_cells; a.rows = rows; a.Gt = Gt; a.E = E; a.w = w;
  a.ploss = wk.ploss; a.pdrp = wk.pdrp; a.pE = wk.pE; a.dGt = dGt;
  const int splits = rc_splits(n_cells, rows);
  const int64_t per = ceil_div(ceil_div(rows, splits), kRcT) * kRcT;
  cudaStream_t s = (cudaStream_t)stream;
  if ((st = run_cells<true>(a, rp, splits, per, s))) return st;
  recon_finish_kernel<true><<<(unsigned)ceil_div((int64_t)n_cells * rp, 256), 256, 0, s>>>(
      a, splits, rp, loss, dE, wk.cdrp);
  recon_drp_kernel<<<1, 256, 0, s>>>(w, wk.cdrp, n_cells, drp);
  FH_CHECK_LAUNCH();
  switch (rp) {
    case 16: return launch_rows<16>(a, s);
    case 32: return launch_rows<32>(a, s);
    default: return launch_rows<64>(a, s);
  }
}

extern "C" size_t fh_factor_grad_workspace(int32_t nchunks, int32_t ld, int32_t rp) {
  if (nchunks <= 0 || ld <= 0 || rp <= 0) return 0;
  return (size_t)nchunks * ((size_t)ld * ld + (size_t)rp * ld) * sizeof(float);
}

extern "C" int fh_factor_grad_f32(int32_t nchrom, int32_t nchunks, const int32_t* meta,
                                  const float* H, int32_t ldh, const float* A, const float* B,
                                  const float* D, int32_t ld, int32_t rp, int32_t R, float* dA,
                                  float* dB, float* dD, void* ws, size_t ws_bytes,
                                  void* stream) {
  if (nchrom <= 0 || nchunks <= 0 || !meta || !H || !A || !B || !D || !dA || !dB || !dD ||
      !ws || R > rp || ld < R || ldh <= 0)
    return FH_ERR_ARG;
  if (ld > kFgMax || rp > kFgMax) return FH_ERR_UNSUPPORTED;
  if (ws_bytes < fh_factor_grad_workspace(nchunks, ld, rp)) return FH_ERR_ARG;
  FgArgs a{};
  a.c_rank = meta + 2 * nchrom; a.c_chunk0 = meta + 3 * nchrom; a.c_nchunk = meta + 4 * nchrom;
  a.k_chrom = meta + 5 * nchrom; a.k_row0 = a.k_chrom + nchunks; a.k_nrow = a.k_row0 + nchunks;
  a.H = H; a.A = A; a.B = B; a.D = D; a.ld = ld; a.RP = rp; a.R = R; a.ldh = ldh;
  a.dA = dA; a.dB = dB; a.dD = dD;
  a.pB = static_cast<float*>(ws);
  a.pD = a.pB + (size_t)nchunks * ld * ld;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t smem = 4 * kFgMax * kFgLd * sizeof(float);
  if (ensure_smem((const void*)factor_grad_chunk_kernel, smem)) return FH_ERR_LAUNCH;
  factor_grad_chunk_kernel<<<(unsigned)nchunks, 256, smem, s>>>(a);
  factor_grad_reduce_kernel<<<(unsigned)nchrom, 256, 0, s>>>(a);
  FH_CHECK_LAUNCH();
  return FH_OK;
}
