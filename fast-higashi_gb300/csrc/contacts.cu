// Sparse per-cell contact build: COO of one chromosome -> packed (tile, cell) segments.
//
// Replaces the host-side tiling of Chrom_Dataset.__init__ (fasthigashi/sparse_for_schic.py:
// 401-503, the per-bin-batch slice and per-cell-batch boolean mask) and the pinned int16/int32
// Fake_Sparse copies (sparse_for_schic.py:322-340).  The COO is uploaded once; a counting
// sort keyed by (tile, cell) groups each cell's contacts of a bin batch into one contiguous
// segment of 8-byte entries that the fused densify+RWR kernel reads with coalesced loads.
#include "fh_common.cuh"

namespace fh {

// Tile and local coordinates of one contact.  Returns 1 if it lands in the tile, 0 if it is
// to be dropped (one step outside, where the reference's padded densify crops it,
// sparse_for_schic.py:316-319), -1 if it is farther out (an index error).
__device__ __forceinline__ int locate(const fh_tile* __restrict__ tiles, int tile_base,
                                      int n_tiles, int bs_bin, int n_cells, int r, int col,
                                      int cell, int& t, uint32_t& rc) {
  if (r < 0 || cell < 0 || cell >= n_cells) return -1;
  const int bi = r / bs_bin;
  if (bi >= n_tiles) return -1;
  t = tile_base + bi;
  const int row0 = __ldg(&tiles[t].row0);
  const int width = __ldg(&tiles[t].width);
  const int shift = __ldg(&tiles[t].shift);
  const int lr = r - row0;
  const int lc = col - shift;
  if (lr >= __ldg(&tiles[t].rows)) return -1;
  if (lc < 0 || lc >= width) return (lc == -1 || lc == width) ? 0 : -1;
  rc = (uint32_t)lr | ((uint32_t)lc << 16);
  return 1;
}

__global__ void contacts_count_kernel(const int32_t* __restrict__ row,
                                      const int32_t* __restrict__ col,
                                      const int32_t* __restrict__ cell, int64_t nnz, int bs_bin,
                                      const fh_tile* __restrict__ tiles, int tile_base,
                                      int n_tiles, int n_cells, int32_t* __restrict__ counts,
                                      int* status) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nnz;
       e += (int64_t)gridDim.x * blockDim.x) {
    int t;
    uint32_t rc;
    const int k = __ldg(&cell[e]);
    const int s = locate(tiles, tile_base, n_tiles, bs_bin, n_cells, __ldg(&row[e]),
                         __ldg(&col[e]), k, t, rc);
    if (s > 0) atomicAdd(&counts[(int64_t)t * n_cells + k], 1);
    else if (s < 0) set_status(status, FH_ERR_INDEX);
  }
}

__global__ void contacts_scatter_kernel(const int32_t* __restrict__ row,
                                        const int32_t* __restrict__ col,
                                        const int32_t* __restrict__ cell,
                                        const float* __restrict__ val, int64_t nnz, int bs_bin,
                                        const fh_tile* __restrict__ tiles, int tile_base,
                                        int n_tiles, int n_cells,
                                        const int64_t* __restrict__ offsets,
                                        int32_t* __restrict__ cursor, uint2* __restrict__ out) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nnz;
       e += (int64_t)gridDim.x * blockDim.x) {
    int t;
    uint32_t rc;
    const int k = __ldg(&cell[e]);
    if (locate(tiles, tile_base, n_tiles, bs_bin, n_cells, __ldg(&row[e]), __ldg(&col[e]), k,
               t, rc) <= 0)
      continue;
    const int64_t key = (int64_t)t * n_cells + k;
    const int64_t pos = offsets[key] + atomicAdd(&cursor[key], 1);
    out[pos] = make_uint2(rc, __float_as_uint(__ldg(&val[e])));
  }
}

// Three-phase exclusive scan: per-block totals, a scan of the totals, then per-block scans.
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void scan_block_totals(const int32_t* __restrict__ in, int64_t n,
                                  int64_t* __restrict__ totals) {
  __shared__ int64_t red[32];
  const int64_t base = blockIdx.x * (int64_t)kScanTile;
  int64_t s = 0;
  for (int i = threadIdx.x; i < kScanTile; i += kScanThreads) {
    const int64_t g = base + i;
    if (g < n) s += in[g];
  }
  s = block_sum<int64_t>(s, red);
  if (threadIdx.x == 0) totals[blockIdx.x] = s;
}

__global__ void scan_totals(int64_t* __restrict__ totals, int64_t nblocks) {
  // single block: running exclusive scan of the block totals in chunks of blockDim
  __shared__ int64_t buf[1024];
  __shared__ int64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t base = 0; base < nblocks; base += blockDim.x) {
    const int64_t g = base + threadIdx.x;
    const int64_t v = g < nblocks ? totals[g] : 0;
    buf[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < (int)blockDim.x; o <<= 1) {
      const int64_t a = threadIdx.x >= o ? buf[threadIdx.x - o] : 0;
      __syncthreads();
      buf[threadIdx.x] += a;
      __syncthreads();
    }
    if (g < nblocks) totals[g] = carry + buf[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry += buf[threadIdx.x];
    __syncthreads();
  }
  if (threadIdx.x == 0) totals[nblocks] = carry;
}

__global__ void scan_blocks(const int32_t* __restrict__ in, int64_t n,
                            const int64_t* __restrict__ block_off, int64_t* __restrict__ out) {
  __shared__ int64_t buf[kScanThreads];
  const int64_t base = blockIdx.x * (int64_t)kScanTile + threadIdx.x * (int64_t)kScanItems;
  int64_t loc[kScanItems];
  int64_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    const int64_t g = base + i;
    loc[i] = s;
    s += g < n ? in[g] : 0;
  }
  buf[threadIdx.x] = s;
  __syncthreads();
  for (int o = 1; o < kScanThreads; o <<= 1) {
    const int64_t a = threadIdx.x >= o ? buf[threadIdx.x - o] : 0;
    __syncthreads();
    buf[threadIdx.x] += a;
    __syncthreads();
  }
  const int64_t pre = block_off[blockIdx.x] + buf[threadIdx.x] - s;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    const int64_t g = base + i;
    if (g < n) out[g] = pre + loc[i];
  }
}

// Dense tile of cells [c0, c0 + ncell) of tile t: out[c][i][j] (transpose=True layout of
// densify_jit, sparse_for_schic.py:286-320), floor 1e-8 everywhere.
__global__ void densify_tile_kernel(const fh_tile* __restrict__ tiles, int t, int n_cells, int c0,
                                    const int64_t* __restrict__ offsets,
                                    const uint2* __restrict__ entries, float* __restrict__ out) {
  const int c = c0 + blockIdx.x;
  const int b = tiles[t].rows, n = tiles[t].width;
  float* o = out + (int64_t)blockIdx.x * b * n;
  for (int i = threadIdx.x; i < b * n; i += blockDim.x) o[i] = 1e-8f;
  __syncthreads();
  const int64_t e0 = offsets[(int64_t)t * n_cells + c], e1 = offsets[(int64_t)t * n_cells + c + 1];
  for (int64_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
    const uint2 en = entries[e];
    o[(en.x & 0xffff) * n + (en.x >> 16)] = fmaxf(__uint_as_float(en.y), 1e-8f);
  }
}

// x[i] += *base for i < n: chains a scan of one dataset's counts onto the previous dataset's
// total, read on the device (no host round trip).
__global__ void scan_add_base_kernel(int64_t* __restrict__ x, int64_t n,
                                     const int64_t* __restrict__ base) {
  const int64_t b = *base;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] += b;
}

}  // namespace fh

using namespace fh;

extern "C" int fh_scan_add_base(int64_t* x, int64_t n, const int64_t* base, void* stream) {
  if (!x || !base || n <= 0) return FH_ERR_ARG;
  int64_t grid = ceil_div(n, 256);
  if (grid > 152 * 8) grid = 152 * 8;
  scan_add_base_kernel<<<(unsigned)grid, 256, 0, (cudaStream_t)stream>>>(x, n, base);
  FH_CHECK_LAUNCH();
  return FH_OK;
}

extern "C" int fh_densify_tile(const fh_tile* tiles, int32_t t, int32_t n_cells, int32_t c0,
                               int32_t ncell, const int64_t* offsets, const fh_entry* entries,
                               float* out, void* stream) {
  if (!tiles || !offsets || !entries || !out || t < 0 || c0 < 0 || ncell <= 0 ||
      c0 + ncell > n_cells)
    return FH_ERR_ARG;
  densify_tile_kernel<<<ncell, 256, 0, (cudaStream_t)stream>>>(
      tiles, t, n_cells, c0, offsets, reinterpret_cast<const uint2*>(entries), out);
  FH_CHECK_LAUNCH();
  return FH_OK;
}

static inline int grid_for(int64_t n, int threads) {
  int64_t g = ceil_div(n, threads);
  if (g > 152 * 64) g = 152 * 64;
  return (int)(g < 1 ? 1 : g);
}

extern "C" int fh_contacts_count(const int32_t* row, const int32_t* col, const int32_t* cell,
                                 int64_t nnz, int32_t bs_bin, const fh_tile* tiles,
                                 int32_t tile_base, int32_t n_tiles, int32_t n_cells,
                                 int32_t* counts, int* status, void* stream) {
  if (nnz < 0 || bs_bin <= 0 || n_tiles <= 0 || n_cells <= 0 || !tiles || !counts)
    return FH_ERR_ARG;
  if (nnz == 0) return FH_OK;
  if (!row || !col || !cell) return FH_ERR_ARG;
  contacts_count_kernel<<<grid_for(nnz, 256), 256, 0, (cudaStream_t)stream>>>(
      row, col, cell, nnz, bs_bin, tiles, tile_base, n_tiles, n_cells, counts, status);
  FH_CHECK_LAUNCH();
  return FH_OK;
}

extern "C" size_t fh_scan_workspace(int64_t n) {
  return (size_t)(ceil_div(n < 1 ? 1 : n, kScanTile) + 1) * sizeof(int64_t);
}

extern "C" int fh_exclusive_scan(const int32_t* counts, int64_t n, int64_t* offsets,
                                 void* workspace, size_t workspace_bytes, void* stream) {
  if (n <= 0 || !counts || !offsets || !workspace) return FH_ERR_ARG;
  if (workspace_bytes < fh_scan_workspace(n)) return FH_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t nb = ceil_div(n, kScanTile);
  int64_t* totals = (int64_t*)workspace;
  scan_block_totals<<<(unsigned)nb, kScanThreads, 0, s>>>(counts, n, totals);
  scan_totals<<<1, 1024, 0, s>>>(totals, nb);
  scan_blocks<<<(unsigned)nb, kScanThreads, 0, s>>>(counts, n, totals, offsets);
  // offsets[n] = total
  cudaMemcpyAsync(offsets + n, totals + nb, sizeof(int64_t), cudaMemcpyDeviceToDevice, s);
  FH_CHECK_LAUNCH();
  return FH_OK;
}

// ---------------------------------------------------------------------------------------
// fh_exclusive_scan_noalloc: the same scan with its scratch in a fixed device array.
//
// Some callers cannot hand the library a workspace: host code that owns no CUDA allocator
// (a binding from another language that only passes the buffers it already has), or code
// that must not call cudaMalloc because it synchronizes the device and would stall work
// other streams have in flight.  This variant takes only the input and the output.  Its
// scratch, the per-block totals of the three-phase scan, lives in the array below, which
// every GPU that loads the library holds until the process exits.
// ---------------------------------------------------------------------------------------
constexpr int64_t kNoAllocScanBlocks = 8191;   // 64 KiB of int64 block totals
constexpr int64_t kNoAllocScanMax = kNoAllocScanBlocks * kScanTile;   // 16,775,168 counts
static __device__ __align__(256) int64_t g_scan_scratch[kNoAllocScanBlocks + 1];

// Device address of g_scan_scratch on the current device, looked up once per device.
static int scan_scratch_address(int64_t** out) {
  static std::mutex mu;
  static std::unordered_map<int, int64_t*> addr;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return FH_ERR_LAUNCH;
  std::lock_guard<std::mutex> g(mu);
  auto it = addr.find(dev);
  if (it == addr.end()) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_scan_scratch) != cudaSuccess || !p) return FH_ERR_LAUNCH;
    it = addr.emplace(dev, (int64_t*)p).first;
  }
  *out = it->second;
  return FH_OK;
}

extern "C" int fh_exclusive_scan_noalloc(const int32_t* counts, int64_t n, int64_t* offsets,
                                         void* stream) {
  if (n <= 0 || !counts || !offsets) return FH_ERR_ARG;
  if (n > kNoAllocScanMax) return FH_ERR_UNSUPPORTED;   // the block totals would not fit
  int64_t* totals = nullptr;
  const int st = scan_scratch_address(&totals);
  if (st) return st;
  // Every entry the scan reads is written first in the same call (block totals, then their
  // prefix sums), so the array needs no clearing between calls.
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t nb = ceil_div(n, kScanTile);
  scan_block_totals<<<(unsigned)nb, kScanThreads, 0, s>>>(counts, n, totals);
  scan_totals<<<1, 1024, 0, s>>>(totals, nb);
  scan_blocks<<<(unsigned)nb, kScanThreads, 0, s>>>(counts, n, totals, offsets);
  cudaMemcpyAsync(offsets + n, totals + nb, sizeof(int64_t), cudaMemcpyDeviceToDevice, s);
  FH_CHECK_LAUNCH();
  return FH_OK;
}

extern "C" int fh_contacts_scatter(const int32_t* row, const int32_t* col, const int32_t* cell,
                                   const float* val, int64_t nnz, int32_t bs_bin,
                                   const fh_tile* tiles, int32_t tile_base, int32_t n_tiles,
                                   int32_t n_cells, const int64_t* offsets, int32_t* cursor,
                                   fh_entry* entries, void* stream) {
  if (nnz < 0 || bs_bin <= 0 || n_tiles <= 0 || n_cells <= 0 || !tiles || !offsets || !cursor)
    return FH_ERR_ARG;
  if (nnz == 0) return FH_OK;
  if (!row || !col || !cell || !val || !entries) return FH_ERR_ARG;
  contacts_scatter_kernel<<<grid_for(nnz, 256), 256, 0, (cudaStream_t)stream>>>(
      row, col, cell, val, nnz, bs_bin, tiles, tile_base, n_tiles, n_cells, offsets, cursor,
      reinterpret_cast<uint2*>(entries));
  FH_CHECK_LAUNCH();
  return FH_OK;
}
