// Imputed contact maps of FastHigashi.only_partial_rwr (fasthigashi/FastHigashi_Wrapper.py:
// 569-655): every cell's walk output placed into a dense chromosome map and symmetrised.
//
// The reference writes each (bin batch, cell batch) walk into imputed_map[:, slice_row,
// slice_col] (:588-600), then stores m = M + M^T with the diagonal halved (:601-605), i.e.
//   out[i][j] = M[i][j] + M[j][i]  (i != j),   out[i][i] = M[i][i].
// M[i][j] is the walk output of the bin batch holding row i at its compact column j - shift
// when that column lies in the batch's columns, else 0.  One thread per output entry reads
// both M[i][j] and M[j][i] straight from X (the compact band layout), so no dense M is
// formed; each tile's X run is read in rows, the map written in rows.
#include "fh_common.cuh"

namespace fh {

__device__ __forceinline__ float impute_m(const fh_tile* __restrict__ tiles,
                                          const int32_t* __restrict__ row_tile, int64_t row_base,
                                          const float* __restrict__ Xc, int i, int j,
                                          int* status) {
  const int t = row_tile[row_base + i];
  const fh_tile T = tiles[t];
  const int li = i - T.row0, lj = j - T.shift;
  if (li < 0 || li >= T.rows) {
    set_status(status, FH_ERR_INDEX);
    return 0.f;
  }
  if (lj < 0 || lj >= T.width) return 0.f;
  return Xc[T.xoff + (int64_t)li * T.width + lj];
}

__global__ void __launch_bounds__(256) impute_maps_kernel(const fh_tile* __restrict__ tiles,
                                                          const int32_t* __restrict__ row_tile,
                                                          int64_t row_base, int nbin,
                                                          const float* __restrict__ X,
                                                          int64_t ldx, int cell0, int ncell,
                                                          float* __restrict__ out, int* status) {
  const int64_t per = (int64_t)nbin * nbin;
  const int64_t total = per * ncell;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(e / per);
    const int64_t ij = e - c * per;
    const int i = (int)(ij / nbin), j = (int)(ij - (int64_t)i * nbin);
    const float* Xc = X + (int64_t)(cell0 + c) * ldx;
    const float a = impute_m(tiles, row_tile, row_base, Xc, i, j, status);
    out[e] = i == j ? a : a + impute_m(tiles, row_tile, row_base, Xc, j, i, status);
  }
}

}  // namespace fh

using namespace fh;

extern "C" int fh_impute_maps(const fh_tile* tiles, const int32_t* row_tile, int64_t row_base,
                              int32_t nbin, const float* X, int64_t ldx, int32_t cell0,
                              int32_t ncell, float* out, int* status, void* stream) {
  if (!tiles || !row_tile || !X || !out || !status || row_base < 0 || nbin <= 0 || cell0 < 0 ||
      ncell <= 0 || ldx <= 0)
    return FH_ERR_ARG;
  const int64_t total = (int64_t)nbin * nbin * ncell;
  int64_t grid = ceil_div(total, 256);
  if (grid > 152 * 16) grid = 152 * 16;
  impute_maps_kernel<<<(unsigned)grid, 256, 0, (cudaStream_t)stream>>>(
      tiles, row_tile, row_base, nbin, X, ldx, cell0, ncell, out, status);
  FH_CHECK_LAUNCH();
  return FH_OK;
}
