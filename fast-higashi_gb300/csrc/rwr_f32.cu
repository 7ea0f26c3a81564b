// Partial random walk with restart, fp32 CUDA-core path (one CTA per (bin batch, cell)).
//
// Reference: fasthigashi/partial_rwr.py:75-138 (do_conv=False, do_col=False) fed by
// densify_jit (fasthigashi/sparse_for_schic.py:279-320).
//
// The tile A (b x n, the cell's rows of one bin batch over its compact columns) is densified
// straight into shared memory from the cell's packed segment and floored at 1e-8.  Then:
//   S2 = A A^T with a zero diagonal; S1 = A[:, s0:s0+b]
//   L  = 0.75 * S1 / colsum(S1) + 0.25 * S2 / colsum(S2);  zero columns get a unit diagonal
//   P  = L / colsum(L)
// The reference iterates Q_{t+1} = 0.5 Q_t P + 0.5 I from Q_0 = I and returns Q_n A.  Every
// Q_t is a polynomial in P, so Q_t P = P Q_t, and Z_t = Q_t A obeys Z_{t+1} = 0.5 P Z_t +
// 0.5 A.  The kernel runs that recurrence in place (P^T and Z resident in shared memory,
// the product accumulated in registers), which needs no b x b Q buffer and no final Q A
// product.  The +0.5 A term is the constant 0.5e-8 floor plus the segment's entries.
//
// The auto-stop variant (partial_rwr.py:99-123) runs the same recurrence with A = I, which
// is Q_t itself, and records ||Q_t - Q_{t+1}||_F per epoch.
#include <cuda_bf16.h>
#include "rwr_common.cuh"

namespace fh {


// kSparse: densified from the (tile, cell) segments; kDense: one dense tile shape for every
// cell (the partial_rwr drop-in); kDenseTiles: dense tiles in the X layout (row stride of a
// cell cell_stride, a tile at tile.xoff), e.g. the 3 x 3 mean of conv_tiles_kernel.
enum RwrSource { kSparse = 0, kDense = 1, kDenseTiles = 2 };
enum RwrMode { kOutput = 0, kDeltas = 1, kOutput16 = 2 };

struct RwrArgs {
  const fh_tile* tiles;
  int n_cells;
  const uint2* entries;
  const int64_t* offsets;
  const float* dense;  // dense source: [n_cells][rows][width]
  int d_rows, d_width, d_s0, d_epochs;
  int max_rows, max_width;  // extents the shared-memory carve-out was sized for
  float* out;
  __nv_bfloat16* out16;
  int64_t plane_stride;  // > 0: a second bf16 plane with the rounding residual
  int64_t cell_stride;
  double* sumsq;
  float* deltas;
  int cap;
  float rp;  // walk weight: Q_{t+1} = rp Q_t P + (1 - rp) I (partial_rwr.py:109,116-118)
  int* status;
};

__host__ __device__ inline size_t rwr_smem_bytes(int b, int n) {
  const int ldp = rwr_ldp(b), ldz = lds_stride_odd(n > b ? n : b);
  return (size_t)(b * ldp + b * ldz + 4 * kMaxBinRows) * sizeof(float);
}

template <int MAXU, int SRC, int MODE>
__global__ void __launch_bounds__(kRwrThreads, 1) rwr_f32_kernel(RwrArgs a) {
  extern __shared__ __align__(16) float smem[];
  __shared__ double dred[32];
  __shared__ float fred[32];
  const int c = blockIdx.x;
  const int t = blockIdx.y;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;

  int b, n, s0, epochs;
  int64_t xoff = 0;
  if (SRC == kSparse || SRC == kDenseTiles) {
    const fh_tile T = a.tiles[t];
    b = T.rows; n = T.width; s0 = T.s0; epochs = T.n_rwr; xoff = T.xoff;
    if (b <= 0 || b > a.max_rows || n < b || n > a.max_width || s0 < 0 || s0 + b > n ||
        epochs < 0) {
      if (tid == 0) set_status(a.status, FH_ERR_ARG);
      return;
    }
  } else {
    b = a.d_rows; n = a.d_width; s0 = a.d_s0; epochs = a.d_epochs;
  }
  if (MODE == kDeltas) epochs = a.cap;
  const int ldp = rwr_ldp(b);
  const int ldz = lds_stride_odd(n > b ? n : b);
  float* Pt = smem;               // b x ldp : S2, then L, then P^T
  float* Z = smem + b * ldp;      // b x ldz : A, then Z_t (or Q_t in delta mode)
  float* cs1 = Z + b * ldz;       // column sums
  float* cs2 = cs1 + kMaxBinRows;
  float* csl = cs2 + kMaxBinRows;

  int64_t e0 = 0, e1 = 0;
  const float* xin = nullptr;
  if (SRC == kSparse) {
    e0 = a.offsets[(int64_t)t * a.n_cells + c];
    e1 = a.offsets[(int64_t)t * a.n_cells + c + 1];
    for (int i = tid; i < b * ldz; i += kRwrThreads) Z[i] = 0.f;
    __syncthreads();
    for (int64_t e = e0 + tid; e < e1; e += kRwrThreads) {
      const uint2 en = a.entries[e];
      Z[(en.x & 0xffff) * ldz + (en.x >> 16)] = __uint_as_float(en.y);
    }
    __syncthreads();
    for (int i = tid; i < b * n; i += kRwrThreads) {
      float* z = Z + (i / n) * ldz + (i % n);
      *z = fmaxf(*z, kFloor);
    }
  } else {
    xin = SRC == kDense ? a.dense + (int64_t)c * b * n : a.dense + (int64_t)c * a.cell_stride + xoff;
    for (int i = tid; i < b * n; i += kRwrThreads) Z[(i / n) * ldz + (i % n)] = xin[i];
  }
  __syncthreads();

  rwr_transition(Z, ldz, Pt, ldp, b, n, s0, cs1, cs2, csl);

  const float om = a.rp, al = 1.f - a.rp;   // walk and restart weights
  int zw = n;  // columns of the recurrence state
  if (MODE == kDeltas) {
    zw = b;    // Q_0 = I
    for (int i = tid; i < b * b; i += kRwrThreads) Z[(i / b) * ldz + (i % b)] = (i / b == i % b);
    __syncthreads();
  }

  // ---- Z_{t+1} = 0.5 P Z_t + 0.5 A   (Q_{t+1} = 0.5 P Q_t + 0.5 I in delta mode)
  for (int ep = 0; ep < epochs; ++ep) {
    float acc[MAXU][8];
    pz_product<MAXU>(Z, ldz, Pt, ldp, b, ty, tx, acc);
    float d2 = 0.f;
    if (MODE == kDeltas) {
#pragma unroll
      for (int u = 0; u < MAXU; ++u)
#pragma unroll
        for (int v = 0; v < 8; ++v) {
          const int i = ty + 16 * u, j = tx + 16 * v;
          if (i < zw && j < b) {
            const float nv = om * acc[u][v] + (i == j ? al : 0.f);
            const float dd = Z[j * ldz + i] - nv;
            d2 = fmaf(dd, dd, d2);
          }
        }
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < MAXU; ++u)
#pragma unroll
      for (int v = 0; v < 8; ++v) {
        const int i = ty + 16 * u, j = tx + 16 * v;
        if (i < zw && j < b) {
          float base;
          if (MODE == kDeltas) base = (i == j) ? al : 0.f;
          else if (SRC == kSparse) base = al * kFloor;
          else base = al * xin[j * n + i];
          Z[j * ldz + i] = fmaf(om, acc[u][v], base);
        }
      }
    if (MODE == kDeltas) {
      const float s = block_sum<float>(d2, fred);
      if (tid == 0) a.deltas[((int64_t)t * a.n_cells + c) * a.cap + ep] = sqrtf(s);
    }
    __syncthreads();
    if (MODE != kDeltas && SRC == kSparse) {
      for (int64_t e = e0 + tid; e < e1; e += kRwrThreads) {
        const uint2 en = a.entries[e];
        const float v = __uint_as_float(en.y);
        if (v > kFloor) Z[(en.x & 0xffff) * ldz + (en.x >> 16)] += al * (v - kFloor);
      }
      __syncthreads();
    }
  }

  if (MODE == kOutput || MODE == kOutput16) {
    double ss = 0.0;
    for (int i = tid; i < b * n; i += kRwrThreads) {
      float v = Z[(i / n) * ldz + (i % n)];
      if (MODE == kOutput) {
        a.out[(int64_t)c * a.cell_stride + xoff + i] = v;
      } else {
        const int64_t o = (int64_t)c * a.cell_stride + xoff + i;
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        a.out16[o] = h;
        if (a.plane_stride > 0) {
          const __nv_bfloat16 l = __float2bfloat16_rn(v - __bfloat162float(h));
          a.out16[a.plane_stride + o] = l;
          v = __bfloat162float(h) + __bfloat162float(l);
        } else {
          v = __bfloat162float(h);
        }
      }
      ss += (double)v * v;
    }
    if (a.sumsq) {
      ss = block_sum<double>(ss, dred);
      if (tid == 0) a.sumsq[(int64_t)t * a.n_cells + c] = ss;
    }
  }
}

template <int U, int SRC, int MODE>
static int launch_rwr_u(const RwrArgs& a, dim3 grid, size_t smem, cudaStream_t s) {
  if constexpr (MODE == kDeltas && U != 8) {
    return FH_ERR_UNSUPPORTED;  // the delta recurrence is b x b, b <= 128
  } else {
    auto k = rwr_f32_kernel<U, SRC, MODE>;
    if (ensure_smem((const void*)k, smem))
      return FH_ERR_LAUNCH;
    k<<<grid, kRwrThreads, smem, s>>>(a);
    FH_CHECK_LAUNCH();
    return FH_OK;
  }
}

template <int SRC, int MODE>
static int launch_rwr(const RwrArgs& a, int n_tiles, int max_rows, int max_width,
                      cudaStream_t s) {
  if (max_rows > kMaxBinRows || max_rows <= 0) return FH_ERR_UNSUPPORTED;
  const int w = MODE == kDeltas ? (max_width > max_rows ? max_width : max_rows) : max_width;
  if (w > kMaxWidth) return FH_ERR_UNSUPPORTED;
  const size_t smem = rwr_smem_bytes(max_rows, w);
  if (smem > 227 * 1024) return FH_ERR_UNSUPPORTED;
  dim3 grid(a.n_cells, n_tiles);
  const int zw = MODE == kDeltas ? max_rows : max_width;
  if (zw <= 128) return launch_rwr_u<8, SRC, MODE>(a, grid, smem, s);
  if (zw <= 192) return launch_rwr_u<12, SRC, MODE>(a, grid, smem, s);
  if (zw <= 256) return launch_rwr_u<16, SRC, MODE>(a, grid, smem, s);
  return launch_rwr_u<20, SRC, MODE>(a, grid, smem, s);
}

// ---------------------------------------------------------------------------------------
// 3 x 3 mean of each tile before the walk (partial_rwr.py:79-83, do_conv=True):
// F.avg_pool2d(x, 3, stride 1, padding 1) counts the zero padding, so every output is the sum
// of its 3 x 3 window (zeros outside the tile) over 9, then floored at 1e-8; a tile of one row
// is left as it is (:80).  The input is the floored densified tile (sparse_for_schic.py:320):
// from the (tile, cell) segment (sparse) or a dense [cell][rows][width] array.  One CTA per
// (tile, cell); the output goes to the X layout (or the dense layout).
// ---------------------------------------------------------------------------------------
struct ConvArgs {
  const fh_tile* tiles;
  int n_cells;
  const uint2* entries;
  const int64_t* offsets;
  const float* dense;      // dense source [cell][rows][width] (tiles == nullptr)
  int d_rows, d_width;
  int max_rows, max_width;
  float* out;
  int64_t cell_stride;
  int* status;
};

__host__ __device__ inline size_t conv_smem_bytes(int b, int n) {
  return (size_t)(b + 2) * (n + 2) * sizeof(float);
}

__global__ void __launch_bounds__(kRwrThreads) conv_tiles_kernel(ConvArgs a) {
  extern __shared__ float cz[];
  const int c = blockIdx.x, t = blockIdx.y, tid = threadIdx.x;
  int b, n;
  int64_t xoff = 0;
  if (a.tiles) {
    const fh_tile T = a.tiles[t];
    b = T.rows; n = T.width; xoff = T.xoff;
    if (b <= 0 || b > a.max_rows || n <= 0 || n > a.max_width) {
      if (tid == 0) set_status(a.status, FH_ERR_ARG);
      return;
    }
  } else {
    b = a.d_rows; n = a.d_width;
  }
  const int ld = n + 2;
  for (int i = tid; i < (b + 2) * ld; i += kRwrThreads) {
    const int p = i / ld, q = i % ld;
    cz[i] = (p >= 1 && p <= b && q >= 1 && q <= n && a.tiles) ? kFloor : 0.f;
  }
  __syncthreads();
  if (a.tiles) {
    const int64_t e0 = a.offsets[(int64_t)t * a.n_cells + c];
    const int64_t e1 = a.offsets[(int64_t)t * a.n_cells + c + 1];
    for (int64_t e = e0 + tid; e < e1; e += kRwrThreads) {
      const uint2 en = a.entries[e];
      const int r = (int)(en.x & 0xffffu), j = (int)(en.x >> 16);
      if (r < b && j < n) cz[(r + 1) * ld + j + 1] = fmaxf(__uint_as_float(en.y), kFloor);
      else set_status(a.status, FH_ERR_INDEX);
    }
  } else {
    const float* x = a.dense + (int64_t)c * b * n;
    for (int i = tid; i < b * n; i += kRwrThreads) cz[(i / n + 1) * ld + i % n + 1] = x[i];
  }
  __syncthreads();
  float* o = a.tiles ? a.out + (int64_t)c * a.cell_stride + xoff : a.out + (int64_t)c * b * n;
  for (int i = tid; i < b * n; i += kRwrThreads) {
    const int p = i / n, q = i % n;
    float v;
    if (b > 1) {
      float s = 0.f;
#pragma unroll
      for (int di = 0; di < 3; ++di)
#pragma unroll
        for (int dj = 0; dj < 3; ++dj) s += cz[(p + di) * ld + q + dj];
      v = fmaxf(s / 9.f, kFloor);
    } else {
      v = cz[(p + 1) * ld + q + 1];
    }
    o[i] = v;
  }
}

}  // namespace fh

using namespace fh;

extern "C" int fh_rwr_tiles_f32(const fh_tile* tiles, int32_t n_tiles, int32_t n_cells,
                                int32_t mr, int32_t mw, const fh_entry* entries,
                                const int64_t* offsets, float* out, int64_t cell_stride,
                                double* sumsq, int* status, void* stream) {
  if (!tiles || n_tiles <= 0 || n_cells <= 0 || !offsets || !out || mr <= 0 || mw < mr)
    return FH_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  RwrArgs a{};
  a.rp = 0.5f;   // partial_rwr.py:109
  a.max_rows = mr; a.max_width = mw;
  a.tiles = tiles; a.n_cells = n_cells; a.entries = reinterpret_cast<const uint2*>(entries);
  a.offsets = offsets; a.out = out; a.cell_stride = cell_stride; a.sumsq = sumsq;
  a.status = status;
  return launch_rwr<kSparse, kOutput>(a, n_tiles, mr, mw, s);
}

extern "C" int fh_rwr_tiles_bf16(const fh_tile* tiles, int32_t n_tiles, int32_t n_cells,
                                 int32_t mr, int32_t mw, const fh_entry* entries,
                                 const int64_t* offsets, uint16_t* out16, int64_t cell_stride,
                                 int64_t plane_stride, double* sumsq, int* status, void* stream) {
  if (!tiles || n_tiles <= 0 || n_cells <= 0 || !offsets || !out16 || mr <= 0 || mw < mr ||
      plane_stride < 0)
    return FH_ERR_ARG;
  RwrArgs a{};
  a.rp = 0.5f;   // partial_rwr.py:109
  a.max_rows = mr; a.max_width = mw;
  a.tiles = tiles; a.n_cells = n_cells; a.entries = reinterpret_cast<const uint2*>(entries);
  a.offsets = offsets; a.out16 = reinterpret_cast<__nv_bfloat16*>(out16);
  a.cell_stride = cell_stride; a.plane_stride = plane_stride; a.sumsq = sumsq;
  a.status = status;
  return launch_rwr<kSparse, kOutput16>(a, n_tiles, mr, mw, (cudaStream_t)stream);
}

extern "C" int fh_rwr_tiles_rp_f32(const fh_tile* tiles, int32_t n_tiles, int32_t n_cells,
                                   int32_t mr, int32_t mw, const fh_entry* entries,
                                   const int64_t* offsets, float rp, float* out,
                                   int64_t cell_stride, double* sumsq, int* status,
                                   void* stream) {
  if (!tiles || n_tiles <= 0 || n_cells <= 0 || !offsets || !out || mr <= 0 || mw < mr ||
      !(rp >= 0.f && rp < 1.f))
    return FH_ERR_ARG;
  RwrArgs a{};
  a.rp = rp;
  a.max_rows = mr; a.max_width = mw;
  a.tiles = tiles; a.n_cells = n_cells; a.entries = reinterpret_cast<const uint2*>(entries);
  a.offsets = offsets; a.out = out; a.cell_stride = cell_stride; a.sumsq = sumsq;
  a.status = status;
  return launch_rwr<kSparse, kOutput>(a, n_tiles, mr, mw, (cudaStream_t)stream);
}

extern "C" int fh_rwr_dense_f32(const float* x, int32_t n_cells, int32_t rows, int32_t width,
                                int32_t s0, int32_t n_epochs, float* out, int* status,
                                void* stream) {
  if (!x || !out || n_cells <= 0 || rows <= 0 || width < rows || s0 < 0 ||
      s0 + rows > width || n_epochs < 0)
    return FH_ERR_ARG;
  RwrArgs a{};
  a.rp = 0.5f;   // partial_rwr.py:109
  a.n_cells = n_cells; a.dense = x; a.d_rows = rows; a.d_width = width; a.d_s0 = s0;
  a.max_rows = rows; a.max_width = width;
  a.d_epochs = n_epochs; a.out = out; a.cell_stride = (int64_t)rows * width; a.status = status;
  return launch_rwr<kDense, kOutput>(a, 1, rows, width, (cudaStream_t)stream);
}

extern "C" int fh_rwr_dense_deltas(const float* x, int32_t n_cells, int32_t rows, int32_t width,
                                   int32_t s0, int32_t cap, float* deltas, int* status,
                                   void* stream) {
  if (!x || !deltas || n_cells <= 0 || rows <= 0 || width < rows || s0 < 0 ||
      s0 + rows > width || cap <= 0)
    return FH_ERR_ARG;
  RwrArgs a{};
  a.rp = 0.5f;   // partial_rwr.py:109
  a.n_cells = n_cells; a.dense = x; a.d_rows = rows; a.d_width = width; a.d_s0 = s0;
  a.max_rows = rows; a.max_width = width;
  a.deltas = deltas; a.cap = cap; a.status = status;
  return launch_rwr<kDense, kDeltas>(a, 1, rows, width, (cudaStream_t)stream);
}

extern "C" int fh_rwr_tiles_deltas(const fh_tile* tiles, int32_t n_tiles, int32_t n_cells,
                                   int32_t mr, int32_t mw, const fh_entry* entries,
                                   const int64_t* offsets, int32_t cap, float* deltas,
                                   int* status, void* stream) {
  if (!tiles || n_tiles <= 0 || n_cells <= 0 || !offsets || !deltas || cap <= 0 || mr <= 0 ||
      mw < mr)
    return FH_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  RwrArgs a{};
  a.rp = 0.5f;   // partial_rwr.py:109
  a.max_rows = mr; a.max_width = mw;
  a.tiles = tiles; a.n_cells = n_cells; a.entries = reinterpret_cast<const uint2*>(entries);
  a.offsets = offsets; a.deltas = deltas; a.cap = cap; a.status = status;
  return launch_rwr<kSparse, kDeltas>(a, n_tiles, mr, mw, s);
}

// ---- 3 x 3 mean (do_conv) and the walk from dense tiles -----------------------------------
extern "C" int fh_conv_tiles_f32(const fh_tile* tiles, int32_t n_tiles, int32_t n_cells,
                                 int32_t mr, int32_t mw, const fh_entry* entries,
                                 const int64_t* offsets, float* out, int64_t cell_stride,
                                 int* status, void* stream) {
  if (!tiles || n_tiles <= 0 || n_cells <= 0 || !offsets || !out || mr <= 0 || mw <= 0)
    return FH_ERR_ARG;
  if (mr > kMaxBinRows || mw > kMaxWidth) return FH_ERR_UNSUPPORTED;
  const size_t smem = conv_smem_bytes(mr, mw);
  if (ensure_smem((const void*)conv_tiles_kernel, smem)) return FH_ERR_LAUNCH;
  ConvArgs a{};
  a.tiles = tiles; a.n_cells = n_cells; a.entries = reinterpret_cast<const uint2*>(entries);
  a.offsets = offsets; a.max_rows = mr; a.max_width = mw; a.out = out;
  a.cell_stride = cell_stride; a.status = status;
  conv_tiles_kernel<<<dim3((unsigned)n_cells, (unsigned)n_tiles), kRwrThreads, smem,
                      (cudaStream_t)stream>>>(a);
  FH_CHECK_LAUNCH();
  return FH_OK;
}

extern "C" int fh_conv_dense_f32(const float* x, int32_t n_cells, int32_t rows, int32_t width,
                                 float* out, void* stream) {
  if (!x || !out || n_cells <= 0 || rows <= 0 || width <= 0) return FH_ERR_ARG;
  if (rows > kMaxBinRows || width > kMaxWidth) return FH_ERR_UNSUPPORTED;
  const size_t smem = conv_smem_bytes(rows, width);
  if (ensure_smem((const void*)conv_tiles_kernel, smem)) return FH_ERR_LAUNCH;
  ConvArgs a{};
  a.dense = x; a.d_rows = rows; a.d_width = width; a.n_cells = n_cells; a.out = out;
  conv_tiles_kernel<<<dim3((unsigned)n_cells, 1u), kRwrThreads, smem, (cudaStream_t)stream>>>(a);
  FH_CHECK_LAUNCH();
  return FH_OK;
}

extern "C" int fh_rwr_tiles_dense_f32(const fh_tile* tiles, int32_t n_tiles, int32_t n_cells,
                                      int32_t mr, int32_t mw, const float* src, float* out,
                                      int64_t cell_stride, double* sumsq, int* status,
                                      void* stream) {
  if (!tiles || n_tiles <= 0 || n_cells <= 0 || !src || !out || mr <= 0 || mw < mr)
    return FH_ERR_ARG;
  RwrArgs a{};
  a.rp = 0.5f;   // partial_rwr.py:109
  a.max_rows = mr; a.max_width = mw;
  a.tiles = tiles; a.n_cells = n_cells; a.dense = src; a.out = out;
  a.cell_stride = cell_stride; a.sumsq = sumsq; a.status = status;
  return launch_rwr<kDenseTiles, kOutput>(a, n_tiles, mr, mw, (cudaStream_t)stream);
}

extern "C" int fh_rwr_tiles_dense_bf16(const fh_tile* tiles, int32_t n_tiles, int32_t n_cells,
                                       int32_t mr, int32_t mw, const float* src, uint16_t* out16,
                                       int64_t cell_stride, int64_t plane_stride, double* sumsq,
                                       int* status, void* stream) {
  if (!tiles || n_tiles <= 0 || n_cells <= 0 || !src || !out16 || mr <= 0 || mw < mr ||
      plane_stride < 0)
    return FH_ERR_ARG;
  RwrArgs a{};
  a.rp = 0.5f;   // partial_rwr.py:109
  a.max_rows = mr; a.max_width = mw;
  a.tiles = tiles; a.n_cells = n_cells; a.dense = src;
  a.out16 = reinterpret_cast<__nv_bfloat16*>(out16);
  a.cell_stride = cell_stride; a.plane_stride = plane_stride; a.sumsq = sumsq; a.status = status;
  return launch_rwr<kDenseTiles, kOutput16>(a, n_tiles, mr, mw, (cudaStream_t)stream);
}

extern "C" int fh_rwr_tiles_dense_deltas(const fh_tile* tiles, int32_t n_tiles, int32_t n_cells,
                                         int32_t mr, int32_t mw, const float* src,
                                         int64_t cell_stride, int32_t cap, float* deltas,
                                         int* status, void* stream) {
  if (!tiles || n_tiles <= 0 || n_cells <= 0 || !src || !deltas || cap <= 0 || mr <= 0 ||
      mw < mr)
    return FH_ERR_ARG;
  RwrArgs a{};
  a.rp = 0.5f;   // partial_rwr.py:109
  a.max_rows = mr; a.max_width = mw;
  a.tiles = tiles; a.n_cells = n_cells; a.dense = src; a.cell_stride = cell_stride;
  a.deltas = deltas; a.cap = cap; a.status = status;
  return launch_rwr<kDenseTiles, kDeltas>(a, n_tiles, mr, mw, (cudaStream_t)stream);
}
