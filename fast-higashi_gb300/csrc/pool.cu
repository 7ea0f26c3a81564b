// The 1 Mb pooling of init_params' features (fasthigashi/parafac2_intergrative.py:102-151):
// at a resolution finer than 1 Mb the reference averages every bin batch's walk output over
// ll x ll blocks (ll = ceil(1 Mb / resolution), F.avg_pool2d with stride ll, no padding, the
// floor of each side) before the features' truncated SVD.  The sketch of that SVD only needs
// products with the pooled features Fp = F Pm (F: cells x band rows, Pm: band rows x pooled
// rows, 1 / ll^2 on each block's entries), so two maps along the band-row axis suffice:
//   fh_pool_rows    out = Pm^T in   (band rows x m -> pooled rows x m; after F^T E)
//   fh_unpool_rows  out = Pm in     (pooled rows x m -> band rows x m; before F Q)
// Tile t's block (py, px) is pooled row prow0[t] + py * (n_t / ll) + px, its band rows
// xoff_t + (py ll + dy) n_t + px ll + dx for dy, dx < ll; band rows outside every block (the
// cropped remainders) map to nothing.  Rows are relative to band row x0 (the chromosome's
// first).  One thread per (output row, column).
#include "fh_common.cuh"

namespace fh {

// Tile of pooled row g (prow0 ascending, prow0[n_tiles] = total): binary search.
__device__ __forceinline__ int pool_tile(const int64_t* prow0, int n_tiles, int64_t g) {
  int lo = 0, hi = n_tiles;           // prow0[lo] <= g < prow0[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (prow0[mid] <= g) lo = mid; else hi = mid;
  }
  return lo;
}

__global__ void pool_rows_kernel(const fh_tile* __restrict__ tiles, int n_tiles,
                                 const int64_t* __restrict__ prow0,
                                 const int32_t* __restrict__ ll_of, int64_t x0,
                                 const float* __restrict__ in, int64_t ldi, int m,
                                 float* __restrict__ out, int64_t ldo) {
  const int64_t total = prow0[n_tiles] * m;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t g = e / m;
    const int j = (int)(e - g * m);
    const int t = pool_tile(prow0, n_tiles, g);
    const fh_tile T = tiles[t];
    const int ll = ll_of[t], pn = T.width / ll;
    const int64_t q = g - prow0[t];
    const int py = (int)(q / pn), px = (int)(q - (int64_t)py * pn);
    float s = 0.f;
    for (int dy = 0; dy < ll; ++dy)
      for (int dx = 0; dx < ll; ++dx) {
        const int64_t row = T.xoff + (int64_t)(py * ll + dy) * T.width + px * ll + dx - x0;
        s += in[row * ldi + j];
      }
    out[g * ldo + j] = s / (float)(ll * ll);
  }
}

__global__ void unpool_rows_kernel(const fh_tile* __restrict__ tiles, int t0, int n_tiles,
                                   const int64_t* __restrict__ prow0,
                                   const int32_t* __restrict__ ll_of, int64_t x0, int64_t rows,
                                   const float* __restrict__ in, int64_t ldi, int m,
                                   float* __restrict__ out, int64_t ldo) {
  const int64_t total = rows * m;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / m;
    const int j = (int)(e - r * m);
    // the tile holding band row x0 + r (tiles t0.. are consecutive in band rows)
    int lo = 0, hi = n_tiles;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (tiles[t0 + mid].xoff - x0 <= r) lo = mid; else hi = mid;
    }
    const fh_tile T = tiles[t0 + lo];
    const int ll = ll_of[lo];
    const int64_t local = r - (T.xoff - x0);
    const int i = (int)(local / T.width), c = (int)(local - (int64_t)i * T.width);
    const int pb = T.rows / ll, pn = T.width / ll;
    float v = 0.f;
    if (i < pb * ll && c < pn * ll && i < T.rows)
      v = in[(prow0[lo] + (int64_t)(i / ll) * pn + c / ll) * ldi + j] / (float)(ll * ll);
    out[r * ldo + j] = v;
  }
}

}  // namespace fh

using namespace fh;

extern "C" int fh_pool_rows(const fh_tile* tiles, int32_t n_tiles, const int64_t* prow0,
                            const int32_t* ll_of, int64_t x0, const float* in, int64_t ldi,
                            int32_t m, float* out, int64_t ldo, void* stream) {
  if (!tiles || !prow0 || !ll_of || !in || !out || n_tiles <= 0 || m <= 0 || ldi < m ||
      ldo < m || x0 < 0)
    return FH_ERR_ARG;
  pool_rows_kernel<<<152 * 8, 256, 0, (cudaStream_t)stream>>>(tiles, n_tiles, prow0, ll_of, x0,
                                                              in, ldi, m, out, ldo);
  FH_CHECK_LAUNCH();
  return FH_OK;
}

extern "C" int fh_unpool_rows(const fh_tile* tiles, int32_t n_tiles, const int64_t* prow0,
                              const int32_t* ll_of, int64_t x0, int64_t rows, const float* in,
                              int64_t ldi, int32_t m, float* out, int64_t ldo, void* stream) {
  if (!tiles || !prow0 || !ll_of || !in || !out || n_tiles <= 0 || m <= 0 || rows <= 0 ||
      ldi < m || ldo < m || x0 < 0)
    return FH_ERR_ARG;
  unpool_rows_kernel<<<152 * 8, 256, 0, (cudaStream_t)stream>>>(tiles, 0, n_tiles, prow0, ll_of,
                                                                x0, rows, in, ldi, m, out, ldo);
  FH_CHECK_LAUNCH();
  return FH_OK;
}
