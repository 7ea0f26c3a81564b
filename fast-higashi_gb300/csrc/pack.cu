// Input packing of raw per-cell contact matrices on the GPU, one chromosome at a time.
//
// Reference: FastHigashi.pack_training_data_one_process (fasthigashi/FastHigashi_Wrapper.py:
// 221-366) with preprocessing.py:114-193 and 474-489, for a chromosome without a blacklist or
// batch ids: every cell's raw COO (row, col, value) in the cell order `reorder`, bins merged by
// `merge` (coordinates divided, :255-261; duplicates of a merged coordinate stay separate
// entries), contacts with |col - row| > off_diag dropped (:264-268), bins whose row has no
// positive contact in any cell removed and the rest renumbered (filter_bin, :474-489), each
// cell scaled so that its kept contacts sum to the number of merged bins (normalize_by_coverage,
// preprocessing.py:137-142), then log1p and a clip at mean + 15 std over the chromosome's
// values (:358-364).  Output: the packed (row, col, cell) indices and values in the reference's
// order (cell by cell, each cell's entries in input order) and the number of kept bins.
//
// Kernels (one warp per output cell; entries are visited in input order and compacted with a
// ballot, so the order is the reference's):
//   pack_mark    band filter, positive-row marks for the bin filter, fp64 coverage per cell
//   (scan)       kept bins -> new ids; per-cell kept counts -> output offsets (fh_exclusive_scan)
//   pack_count   entries of each cell that survive the band and the bin filter
//   pack_write   the output entries and values log1p(value * scale), per-cell fp64 moments
//   pack_stats   the mean + 15 std threshold (fp64 sums in a fixed order)
//   pack_clip    values above the threshold set to it
// The coverage sum and the moments are accumulated in fp64 where the reference sums fp32 in
// numpy's order, so values agree with the reference's to an ulp or two, indices exactly.
// Contact values are taken as non-negative (counts): a bin row is kept when one of its kept
// contacts is positive, as its row sum is then positive.
#include "fh_common.cuh"

namespace fh {

constexpr int kPackThreads = 256;   // 8 warps, one output cell each

struct PackArgs {
  const int32_t* row;
  const int32_t* col;
  const float* val;
  const int64_t* cell_off;   // raw cell c: entries [cell_off[c], cell_off[c + 1])
  const int32_t* reorder;    // output cell k takes raw cell reorder[k]
  int n_cells, n_raw, nbin, nb, merge, off_diag;
  int32_t* mark;             // [nb] 1: the bin row has a positive kept contact
  int64_t* bin_off;          // [nb + 1] exclusive scan of mark
  double* cov;               // [n_cells] sum of each cell's kept values
  int32_t* cnt;              // [n_cells] entries of each cell in the output
  int64_t* cell_out;         // [n_cells + 1] exclusive scan of cnt
  double* mom;               // [n_cells][2] sum and sum of squares of each cell's values
  float* thr;                // clip threshold
  int32_t* out_idx;          // [3][cap]
  float* out_val;            // [cap]
  int64_t cap;
  int* status;
};

// Warp w of the CTA handles output cell k = blockIdx.x * 8 + w; returns false past the end.  A
// bad reorder entry sets FH_ERR_INDEX and gives the cell no entries.
__device__ __forceinline__ bool pack_cell(const PackArgs& a, int& k, int64_t& e0, int64_t& e1) {
  k = blockIdx.x * (kPackThreads / 32) + (threadIdx.x >> 5);
  if (k >= a.n_cells) return false;
  const int raw = a.reorder[k];
  if (raw < 0 || raw >= a.n_raw) {
    if ((threadIdx.x & 31) == 0) set_status(a.status, FH_ERR_INDEX);
    e0 = e1 = 0;
    return true;
  }
  e0 = a.cell_off[raw];
  e1 = a.cell_off[raw + 1];
  return true;
}

// Merged coordinates of entry e and whether it survives the band filter (bad raw coordinates
// set FH_ERR_INDEX and drop the entry).
__device__ __forceinline__ bool pack_entry(const PackArgs& a, int64_t e, int& r, int& c, float& v) {
  const int r0 = a.row[e], c0 = a.col[e];
  v = a.val[e];
  if (r0 < 0 || r0 >= a.nbin || c0 < 0 || c0 >= a.nbin) {
    set_status(a.status, FH_ERR_INDEX);
    return false;
  }
  r = r0 / a.merge;
  c = c0 / a.merge;
  const int d = c - r;
  return (d < 0 ? -d : d) <= a.off_diag;
}

__global__ void __launch_bounds__(kPackThreads) pack_mark_kernel(PackArgs a) {
  int k;
  int64_t e0, e1;
  if (!pack_cell(a, k, e0, e1)) return;
  const int lane = threadIdx.x & 31;
  double s = 0.0;
  for (int64_t e = e0 + lane; e < e1; e += 32) {
    int r, c;
    float v;
    if (pack_entry(a, e, r, c, v)) {
      s += (double)v;
      if (v > 0.f) a.mark[r] = 1;     // every writer stores the same value
    }
  }
  s = warp_sum(s);
  if (lane == 0) a.cov[k] = s;
}

__global__ void __launch_bounds__(kPackThreads) pack_count_kernel(PackArgs a) {
  int k;
  int64_t e0, e1;
  if (!pack_cell(a, k, e0, e1)) return;
  const int lane = threadIdx.x & 31;
  int n = 0;
  for (int64_t e = e0 + lane; e < e1; e += 32) {
    int r, c;
    float v;
    if (pack_entry(a, e, r, c, v) && a.mark[r] && a.mark[c]) ++n;
  }
  n = warp_sum(n);
  if (lane == 0) a.cnt[k] = n;
}

__global__ void __launch_bounds__(kPackThreads) pack_write_kernel(PackArgs a) {
  int k;
  int64_t e0, e1;
  if (!pack_cell(a, k, e0, e1)) return;
  const int lane = threadIdx.x & 31;
  // normalize_by_coverage: scale = bins / total, in fp32 as the reference's float32 arrays
  const float scale = (float)a.nb / ((float)a.cov[k] + 1e-15f);
  int64_t pos = a.cell_out[k];
  double s1 = 0.0, s2 = 0.0;
  for (int64_t base = e0; base < e1; base += 32) {
    const int64_t e = base + lane;
    int r = 0, c = 0;
    float v = 0.f;
    bool keep = false;
    if (e < e1) keep = pack_entry(a, e, r, c, v) && a.mark[r] && a.mark[c];
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (keep) {
      const int64_t o = pos + __popc(m & ((1u << lane) - 1u));
      const float x = log1pf(v * scale);
      if (o < a.cap) {
        a.out_idx[o] = (int32_t)a.bin_off[r];
        a.out_idx[a.cap + o] = (int32_t)a.bin_off[c];
        a.out_idx[2 * a.cap + o] = k;
        a.out_val[o] = x;
      } else {
        set_status(a.status, FH_ERR_INDEX);
      }
      s1 += (double)x;
      s2 += (double)x * (double)x;
    }
    pos += __popc(m);
  }
  s1 = warp_sum(s1);
  s2 = warp_sum(s2);
  if (lane == 0) {
    a.mom[2 * k] = s1;
    a.mom[2 * k + 1] = s2;
  }
}

// mean + 15 std (population std, numpy's default) of all values, from the per-cell moments
// summed in a fixed order; the threshold is formed in fp32 as the reference forms it from its
// fp32 mean and std.
__global__ void __launch_bounds__(256) pack_stats_kernel(PackArgs a) {
  __shared__ double red[32];
  double s1 = 0.0, s2 = 0.0;
  for (int k = threadIdx.x; k < a.n_cells; k += blockDim.x) {
    s1 += a.mom[2 * k];
    s2 += a.mom[2 * k + 1];
  }
  s1 = block_sum<double>(s1, red);
  s2 = block_sum<double>(s2, red);
  if (threadIdx.x == 0) {
    const double n = (double)a.cell_out[a.n_cells];
    float t = __int_as_float(0x7f800000);   // no values: nothing to clip
    if (n > 0) {
      const double mean = s1 / n;
      double var = s2 / n - mean * mean;
      if (var < 0.0) var = 0.0;
      t = (float)mean + 15.f * (float)sqrt(var);
    }
    *a.thr = t;
  }
}

__global__ void pack_clip_kernel(PackArgs a) {
  const int64_t n = a.cell_out[a.n_cells] < a.cap ? a.cell_out[a.n_cells] : a.cap;
  const float t = *a.thr;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    a.out_val[i] = fminf(a.out_val[i], t);
}

__global__ void pack_counts_kernel(PackArgs a, int64_t* out_counts) {
  out_counts[0] = a.cell_out[a.n_cells];
  out_counts[1] = a.bin_off[a.nb];
}

__host__ __device__ inline size_t pack_align(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace fh

using namespace fh;

extern "C" size_t fh_pack_workspace(int32_t n_cells, int32_t nbin, int32_t merge) {
  if (n_cells <= 0 || nbin <= 0 || merge <= 0) return 0;
  const int64_t nb = ceil_div(nbin, merge);
  size_t scan = fh_scan_workspace(nb);
  if (fh_scan_workspace(n_cells) > scan) scan = fh_scan_workspace(n_cells);
  return pack_align(sizeof(int32_t) * nb) + pack_align(sizeof(int64_t) * (nb + 1)) +
         pack_align(sizeof(double) * n_cells) + pack_align(sizeof(int32_t) * n_cells) +
         pack_align(sizeof(int64_t) * (n_cells + 1)) + pack_align(sizeof(double) * 2 * n_cells) +
         pack_align(sizeof(float)) + pack_align(scan);
}

extern "C" int fh_pack_chromosome(const int32_t* row, const int32_t* col, const float* val,
                                  const int64_t* cell_off, int32_t n_raw, const int32_t* reorder,
                                  int32_t n_cells, int32_t nbin, int32_t merge, int32_t off_diag,
                                  int32_t* out_idx, float* out_val, int64_t cap,
                                  int64_t* out_counts, void* workspace, size_t workspace_bytes,
                                  int* status, void* stream) {
  if (!row || !col || !val || !cell_off || !reorder || !out_idx || !out_val || !out_counts ||
      !workspace || !status ||
      n_cells <= 0 || n_raw <= 0 || nbin <= 0 || merge <= 0 || off_diag < 0 || cap <= 0)
    return FH_ERR_ARG;
  if (workspace_bytes < fh_pack_workspace(n_cells, nbin, merge)) return FH_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int nb = (int)ceil_div(nbin, merge);
  uint8_t* w = (uint8_t*)workspace;
  PackArgs a{};
  a.row = row; a.col = col; a.val = val; a.cell_off = cell_off; a.reorder = reorder;
  a.n_cells = n_cells; a.n_raw = n_raw; a.nbin = nbin; a.nb = nb; a.merge = merge;
  a.off_diag = off_diag;
  a.mark = (int32_t*)w;              w += pack_align(sizeof(int32_t) * nb);
  a.bin_off = (int64_t*)w;           w += pack_align(sizeof(int64_t) * (nb + 1));
  a.cov = (double*)w;                w += pack_align(sizeof(double) * n_cells);
  a.cnt = (int32_t*)w;               w += pack_align(sizeof(int32_t) * n_cells);
  a.cell_out = (int64_t*)w;          w += pack_align(sizeof(int64_t) * (n_cells + 1));
  a.mom = (double*)w;                w += pack_align(sizeof(double) * 2 * n_cells);
  a.thr = (float*)w;                 w += pack_align(sizeof(float));
  void* scan_ws = w;
  size_t scan_bytes = fh_scan_workspace(nb);
  if (fh_scan_workspace(n_cells) > scan_bytes) scan_bytes = fh_scan_workspace(n_cells);
  a.out_idx = out_idx; a.out_val = out_val; a.cap = cap; a.status = status;
  if (cudaMemsetAsync(a.mark, 0, sizeof(int32_t) * nb, s) != cudaSuccess) return FH_ERR_LAUNCH;
  const unsigned grid = (unsigned)ceil_div(n_cells, kPackThreads / 32);
  pack_mark_kernel<<<grid, kPackThreads, 0, s>>>(a);
  FH_CHECK_LAUNCH();
  int rc = fh_exclusive_scan(a.mark, nb, a.bin_off, scan_ws, scan_bytes, stream);
  if (rc) return rc;
  pack_count_kernel<<<grid, kPackThreads, 0, s>>>(a);
  FH_CHECK_LAUNCH();
  rc = fh_exclusive_scan(a.cnt, n_cells, a.cell_out, scan_ws, scan_bytes, stream);
  if (rc) return rc;
  pack_write_kernel<<<grid, kPackThreads, 0, s>>>(a);
  pack_stats_kernel<<<1, 256, 0, s>>>(a);
  int64_t blocks = ceil_div(cap, 256);
  if (blocks > 4096) blocks = 4096;
  pack_clip_kernel<<<(unsigned)blocks, 256, 0, s>>>(a);
  pack_counts_kernel<<<1, 1, 0, s>>>(a, out_counts);
  FH_CHECK_LAUNCH();
  return FH_OK;
}
