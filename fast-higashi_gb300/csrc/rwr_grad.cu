// Derivative of the partial RWR output with respect to the walk weight rp, recomputing the
// band tiles instead of storing the recurrence.
//
// Forward (rwr_f32.cu; partial_rwr.py:109-118 with rp free instead of fixed at 0.5):
//   Z_0 = A,  Z_{t+1} = rp P Z_t + (1 - rp) A,  X = Z_T
// (Q_{t+1} = rp Q_t P + (1 - rp) I and X = Q_T A; Q_t commutes with P).  P depends on the
// contacts only, so differentiating the recurrence gives
//   Z'_0 = 0,  Z'_{t+1} = rp P Z'_t + P Z_t - A,  X' = dX/drp = Z'_T.
// One CTA per (bin batch, cell) rebuilds A and P exactly as the forward kernel does and runs
// both recurrences side by side over 64-column blocks of the tile (the columns evolve
// independently): the block's Z and Z' and the whole floored A stay in shared memory, and
// the products P Z and P Z' share their loads of P.  The Z arithmetic is the forward
// kernel's, operation for operation, so the X written here equals fh_rwr_tiles_rp_f32's
// output bit for bit.
#include "rwr_common.cuh"

namespace fh {

constexpr int kGradCols = 64;   // columns of Z and Z' per block

struct GradArgs {
  const fh_tile* tiles;
  int n_cells;
  const uint2* entries;
  const int64_t* offsets;
  int max_rows, max_width;
  float rp;
  float* x;             // X  [cell][band row] (may be null)
  float* dx;            // X' [cell][band row]
  int64_t cell_stride;
  int* status;
};

__host__ __device__ inline int grad_lda(int n) { return n | 1; }
__host__ __device__ inline size_t grad_smem_bytes(int b, int n) {
  return (size_t)(b * rwr_ldp(b) + b * grad_lda(n) + 2 * b * (kGradCols + 1) +
                  3 * kMaxBinRows) * sizeof(float);
}

__global__ void __launch_bounds__(kRwrThreads, 1) rwr_grad_kernel(GradArgs a) {
  extern __shared__ __align__(16) float smem[];
  const int c = blockIdx.x, t = blockIdx.y;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const fh_tile T = a.tiles[t];
  const int b = T.rows, n = T.width, s0 = T.s0, epochs = T.n_rwr;
  if (b <= 0 || b > a.max_rows || n < b || n > a.max_width || s0 < 0 || s0 + b > n ||
      epochs < 0) {
    if (tid == 0) set_status(a.status, FH_ERR_ARG);
    return;
  }
  const int ldp = rwr_ldp(b), lda = grad_lda(n), ldc = kGradCols + 1;
  float* Pt = smem;                  // b x ldp: P^T
  float* Af = Pt + b * ldp;          // b x lda: the floored tile A
  float* Zc = Af + b * lda;          // b x ldc: a column block of Z
  float* Zd = Zc + b * ldc;          // b x ldc: the same block of Z'
  float* cs1 = Zd + b * ldc;
  float* cs2 = cs1 + kMaxBinRows;
  float* csl = cs2 + kMaxBinRows;
  const int64_t e0 = a.offsets[(int64_t)t * a.n_cells + c];
  const int64_t e1 = a.offsets[(int64_t)t * a.n_cells + c + 1];
  for (int i = tid; i < b * lda; i += kRwrThreads) Af[i] = 0.f;
  __syncthreads();
  for (int64_t e = e0 + tid; e < e1; e += kRwrThreads) {
    const uint2 en = a.entries[e];
    const int r = (int)(en.x & 0xffffu), j = (int)(en.x >> 16);
    if (r < b && j < n) Af[r * lda + j] = __uint_as_float(en.y);
    else set_status(a.status, FH_ERR_INDEX);
  }
  __syncthreads();
  for (int i = tid; i < b * n; i += kRwrThreads) {
    float* z = Af + (i / n) * lda + (i % n);
    *z = fmaxf(*z, kFloor);
  }
  __syncthreads();
  rwr_transition(Af, lda, Pt, ldp, b, n, s0, cs1, cs2, csl);

  const float om = a.rp, al = 1.f - a.rp;   // walk and restart weights
  const float base = al * kFloor;
  for (int j0 = 0; j0 < n; j0 += kGradCols) {
    const int cw = min(kGradCols, n - j0);
    for (int i = tid; i < b * kGradCols; i += kRwrThreads) {
      const int p = i / kGradCols, q = i % kGradCols;
      Zc[p * ldc + q] = q < cw ? Af[p * lda + j0 + q] : 0.f;
      Zd[p * ldc + q] = 0.f;
    }
    __syncthreads();
    for (int ep = 0; ep < epochs; ++ep) {
      // thread (ty, tx): rows ty + 16 u (u < 8), columns tx + 16 v (v < 4) of the block
      float az[8][4], ad[8][4];
#pragma unroll
      for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) az[u][v] = ad[u][v] = 0.f;
      for (int k = 0; k < b; ++k) {
        float pk[8], zk[4], dk[4];
        const float* pr = Pt + k * ldp + ty;
#pragma unroll
        for (int u = 0; u < 8; ++u) pk[u] = ty + 16 * u < b ? pr[16 * u] : 0.f;
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          zk[v] = Zc[k * ldc + tx + 16 * v];
          dk[v] = Zd[k * ldc + tx + 16 * v];
        }
        // same operand order as the forward kernel's fmaf(z, p, acc)
#pragma unroll
        for (int u = 0; u < 8; ++u)
#pragma unroll
          for (int v = 0; v < 4; ++v) {
            az[u][v] = fmaf(zk[v], pk[u], az[u][v]);
            ad[u][v] = fmaf(dk[v], pk[u], ad[u][v]);
          }
      }
      __syncthreads();
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int i = ty + 16 * u;
        if (i < b) {
#pragma unroll
          for (int v = 0; v < 4; ++v) {
            const int j = tx + 16 * v;
            const float av = j < cw ? Af[i * lda + j0 + j] : kFloor;
            // forward: the floor term, then the contact above the floor (rwr_f32.cu)
            float z = fmaf(om, az[u][v], base);
            if (av > kFloor) z += al * (av - kFloor);
            Zc[i * ldc + j] = z;
            Zd[i * ldc + j] = fmaf(om, ad[u][v], az[u][v] - av);
          }
        }
      }
      __syncthreads();
    }
    const int64_t o = (int64_t)c * a.cell_stride + T.xoff + j0;
    for (int i = tid; i < b * cw; i += kRwrThreads) {
      const int p = i / cw, q = i % cw;
      if (a.x) a.x[o + (int64_t)p * n + q] = Zc[p * ldc + q];
      a.dx[o + (int64_t)p * n + q] = Zd[p * ldc + q];
    }
    __syncthreads();
  }
}

}  // namespace fh

using namespace fh;

extern "C" int fh_rwr_grad_f32(const fh_tile* tiles, int32_t n_tiles, int32_t n_cells,
                               int32_t mr, int32_t mw, const fh_entry* entries,
                               const int64_t* offsets, float rp, float* x, float* dx,
                               int64_t cell_stride, int* status, void* stream) {
  if (!tiles || n_tiles <= 0 || n_cells <= 0 || !offsets || !dx || mr <= 0 || mw < mr ||
      !(rp >= 0.f && rp < 1.f))
    return FH_ERR_ARG;
  if (mr > kMaxBinRows || mw > kMaxWidth) return FH_ERR_UNSUPPORTED;
  const size_t smem = grad_smem_bytes(mr, mw);
  if (smem > 227 * 1024) return FH_ERR_UNSUPPORTED;
  if (ensure_smem((const void*)rwr_grad_kernel, smem)) return FH_ERR_LAUNCH;
  GradArgs a{};
  a.tiles = tiles; a.n_cells = n_cells; a.entries = reinterpret_cast<const uint2*>(entries);
  a.offsets = offsets; a.max_rows = mr; a.max_width = mw; a.rp = rp; a.x = x; a.dx = dx;
  a.cell_stride = cell_stride; a.status = status;
  dim3 grid((unsigned)n_cells, (unsigned)n_tiles);
  rwr_grad_kernel<<<grid, kRwrThreads, smem, (cudaStream_t)stream>>>(a);
  FH_CHECK_LAUNCH();
  return FH_OK;
}
