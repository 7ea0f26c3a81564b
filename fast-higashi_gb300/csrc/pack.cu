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
// The entries are cut into segments of at most kPackSeg entries, cell by cell in output order
// (segment b of cell k: entries [e0 + j kPackSeg, ..) of its raw cell), and one CTA takes a
// segment, so a few large cells do not set the time.  Loads are lane-consecutive (entry
// base + 256 u + t for u < 4); the compaction keeps input order with one ballot per warp and
// row u and one exchange of the 32 warp counts per 1,024 entries; the scan of the segments'
// kept counts gives each segment's output offset, so the output is in input order, cell by
// cell (the reference's order).  Kernels:
//   pack_segs    segments per output cell (a bad reorder entry: FH_ERR_INDEX, no entries)
//   (scan)       -> first segment of each cell; pack_segcell: the cell of every segment
//   pack_mark    band filter, positive-row marks for the bin filter, fp64 coverage partials
//   pack_cov     per-cell coverage: the cell's partials summed in segment order
//   (scan)       kept bins -> new ids, then pack_ids: int32 new id or -1
//   pack_count   entries of each segment that survive the band and the bin filter, and the
//                fp64 moment partials of their values log1p(value * scale)
//   (scan)       -> each segment's output offset
//   pack_stats   the mean + 15 std threshold (fp64 sums in segment order)
//   pack_write   the output entries and values min(log1p(value * scale), threshold)
// The coverage sum and the moments are summed per thread in fp32 (at most 16 contacts of a
// segment) and across threads and segments in fp64, where the reference sums fp32 in numpy's
// order, so values agree with the reference's to an ulp or two, indices exactly.
// Contact values are taken as non-negative (counts): a bin row is kept when one of its kept
// contacts is positive, as its row sum is then positive.
#include "fh_common.cuh"

namespace fh {

constexpr int kPackThreads = 256;
constexpr int kPackPer = 4;                        // consecutive entries per thread
constexpr int kPackChunk = kPackThreads * kPackPer;
constexpr int kPackSeg = 4 * kPackChunk;           // entries per segment

struct PackArgs {
  const int32_t* row;
  const int32_t* col;
  const float* val;
  const int64_t* cell_off;   // raw cell c: entries [cell_off[c], cell_off[c + 1])
  const int32_t* reorder;    // output cell k takes raw cell reorder[k]
  int n_cells, n_raw, nbin, nb, merge, off_diag;
  int64_t max_seg;           // segments the launches cover (>= the segments of the input)
  int32_t* nseg;             // [n_cells] segments of each output cell
  int64_t* seg0;             // [n_cells + 1] exclusive scan of nseg
  int32_t* seg_cell;         // [max_seg] output cell of each segment
  int32_t* mark;             // [nb] 1: the bin row has a positive kept contact
  int64_t* bin_off;          // [nb + 1] exclusive scan of mark
  int32_t* new_id;           // [nb] renumbered bin, -1 when the bin is removed
  double* seg_cov;           // [max_seg] sum of the segment's band-kept values
  double* cov;               // [n_cells] sum of each cell's band-kept values
  int32_t* seg_cnt;          // [max_seg] entries of each segment in the output
  int64_t* seg_out;          // [max_seg + 1] exclusive scan of seg_cnt
  double* seg_mom;           // [max_seg][2] sum and sum of squares of the segment's values
  float* thr;                // clip threshold
  int32_t* out_idx;          // [3][cap]
  float* out_val;            // [cap]
  int64_t cap;
  int* status;
};

// Raw cell of output cell k, or -1 (with FH_ERR_INDEX) for a bad reorder entry.
__device__ __forceinline__ int pack_raw(const PackArgs& a, int k) {
  const int raw = a.reorder[k];
  if (raw < 0 || raw >= a.n_raw) return -1;
  return raw;
}

__global__ void pack_segs_kernel(PackArgs a) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < a.n_cells;
       k += gridDim.x * blockDim.x) {
    const int raw = pack_raw(a, k);
    int64_t n = 0;
    if (raw < 0) set_status(a.status, FH_ERR_INDEX);
    else n = a.cell_off[raw + 1] - a.cell_off[raw];
    a.nseg[k] = n > 0 ? (int32_t)ceil_div(n, (int64_t)kPackSeg) : 0;
  }
}

// The cell of every segment: cell k writes its own segments' entries.
__global__ void pack_segcell_kernel(PackArgs a) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < a.n_cells;
       k += gridDim.x * blockDim.x) {
    const int64_t b1 = a.seg0[k + 1] < a.max_seg ? a.seg0[k + 1] : a.max_seg;
    for (int64_t b = a.seg0[k]; b < b1; ++b) a.seg_cell[b] = k;
  }
}

// Segment blockIdx.x: its output cell k and entries [e0, e1); false past the last segment.
__device__ __forceinline__ bool pack_segment(const PackArgs& a, int& k, int64_t& e0, int64_t& e1) {
  const int64_t b = blockIdx.x;
  if (b >= a.seg0[a.n_cells]) return false;
  k = a.seg_cell[b];
  const int raw = pack_raw(a, k);
  const int64_t c0 = a.cell_off[raw], c1 = a.cell_off[raw + 1];
  e0 = c0 + (b - a.seg0[k]) * kPackSeg;
  e1 = e0 + kPackSeg < c1 ? e0 + kPackSeg : c1;
  return true;
}

// Merged coordinates of an entry and whether it survives the band filter (bad raw
// coordinates set FH_ERR_INDEX and drop the entry).
__device__ __forceinline__ bool pack_band(const PackArgs& a, int r0, int c0, int& r, int& c) {
  if (r0 < 0 || r0 >= a.nbin || c0 < 0 || c0 >= a.nbin) {
    set_status(a.status, FH_ERR_INDEX);
    return false;
  }
  if (a.merge == 1) {            // the common case: no division
    r = r0;
    c = c0;
  } else {
    r = r0 / a.merge;
    c = c0 / a.merge;
  }
  const int d = c - r;
  return (d < 0 ? -d : d) <= a.off_diag;
}

// Output offsets of one chunk of kPackChunk entries in input order: entry base + 256 u + t is
// kept when keep[u]; its offset within the chunk is the kept entries of rows u' < u plus
// those of row u before it.  The 32 counts (row u, warp w) sit at cnt[8 u + w] in input order;
// every warp scans them with shuffles (lane i holds count i), so a thread needs one shared
// load and no loop.  cnt: >= 32 ints of shared memory.  Returns the chunk's kept total.
__device__ __forceinline__ int pack_chunk_offsets(const bool (&keep)[kPackPer], int* cnt,
                                                  int (&off)[kPackPer]) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  constexpr int kW = kPackThreads / 32;
  static_assert(kPackPer * kW == 32, "one count per lane");
  unsigned m[kPackPer];
#pragma unroll
  for (int u = 0; u < kPackPer; ++u) m[u] = __ballot_sync(0xffffffffu, keep[u]);
  __syncthreads();                           // the previous chunk's readers are done
  if (lane < kPackPer) {
    unsigned mm = 0;
#pragma unroll
    for (int u = 0; u < kPackPer; ++u) mm = lane == u ? m[u] : mm;
    cnt[lane * kW + w] = __popc(mm);
  }
  __syncthreads();
  const int c = cnt[lane];
  int x = c;                                 // inclusive scan of the 32 counts
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  const int ex = x - c;                      // exclusive
#pragma unroll
  for (int u = 0; u < kPackPer; ++u)
    off[u] = __shfl_sync(0xffffffffu, ex, u * kW + w) + __popc(m[u] & ((1u << lane) - 1u));
  return __shfl_sync(0xffffffffu, x, 31);
}

__global__ void __launch_bounds__(kPackThreads) pack_mark_kernel(PackArgs a) {
  __shared__ double red[32];
  if (blockIdx.x == 0 && threadIdx.x == 0 && a.seg0[a.n_cells] > a.max_seg)
    set_status(a.status, FH_ERR_INDEX);      // more entries than the output capacity
  int k;
  int64_t e0, e1;
  if (!pack_segment(a, k, e0, e1)) return;
  // a thread sums its (at most 16) contacts of the segment in fp32 (integer counts: exact),
  // then the block adds the partials in fp64: fp64 adds per contact are slow on this GPU
  float sf = 0.f;
  for (int64_t base = e0 + threadIdx.x; base < e1; base += kPackChunk) {
    int r0[kPackPer], c0[kPackPer];
    float v[kPackPer];
#pragma unroll
    for (int u = 0; u < kPackPer; ++u) {
      const int64_t e = base + (int64_t)u * kPackThreads;
      const bool in = e < e1;
      r0[u] = in ? a.row[e] : 0;
      c0[u] = in ? a.col[e] : 0;
      v[u] = in ? a.val[e] : 0.f;
    }
#pragma unroll
    for (int u = 0; u < kPackPer; ++u) {
      int r, c;
      if (base + (int64_t)u * kPackThreads < e1 && pack_band(a, r0[u], c0[u], r, c)) {
        sf += v[u];
        // read before writing: after the first few segments every row is marked, and the
        // stores of all CTAs to the same few words would serialise in L2
        if (v[u] > 0.f && a.mark[r] == 0) a.mark[r] = 1;
      }
    }
  }
  const double s = block_sum<double>((double)sf, red);
  if (threadIdx.x == 0) a.seg_cov[blockIdx.x] = s;
}

__global__ void pack_cov_kernel(PackArgs a) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < a.n_cells;
       k += gridDim.x * blockDim.x) {
    double s = 0.0;
    const int64_t b1 = a.seg0[k + 1] < a.max_seg ? a.seg0[k + 1] : a.max_seg;
    for (int64_t b = a.seg0[k]; b < b1; ++b) s += a.seg_cov[b];
    a.cov[k] = s;
  }
}

__global__ void pack_ids_kernel(PackArgs a) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.nb; i += gridDim.x * blockDim.x)
    a.new_id[i] = a.mark[i] ? (int32_t)a.bin_off[i] : -1;
}

__global__ void __launch_bounds__(kPackThreads) pack_count_kernel(PackArgs a) {
  __shared__ int red[32];
  __shared__ double dred[32];
  int k;
  int64_t e0, e1;
  if (!pack_segment(a, k, e0, e1)) {
    if (threadIdx.x == 0) a.seg_cnt[blockIdx.x] = 0;
    return;
  }
  // normalize_by_coverage: scale = bins / total, in fp32 as the reference's float32 arrays
  const float scale = (float)a.nb / ((float)a.cov[k] + 1e-15f);
  int n = 0;
  // moments of the kept values (the clip threshold's): fp32 over a thread's (at most 16)
  // contacts of the segment, then fp64 across the block
  float s1f = 0.f, s2f = 0.f;
  for (int64_t base = e0 + threadIdx.x; base < e1; base += kPackChunk) {
    int r0[kPackPer], c0[kPackPer];
    float v[kPackPer];
#pragma unroll
    for (int u = 0; u < kPackPer; ++u) {
      const int64_t e = base + (int64_t)u * kPackThreads;
      const bool in = e < e1;
      r0[u] = in ? a.row[e] : 0;
      c0[u] = in ? a.col[e] : 0;
      v[u] = in ? a.val[e] : 0.f;
    }
#pragma unroll
    for (int u = 0; u < kPackPer; ++u) {
      int r, c;
      if (base + (int64_t)u * kPackThreads < e1 && pack_band(a, r0[u], c0[u], r, c) &&
          a.new_id[r] >= 0 && a.new_id[c] >= 0) {
        ++n;
        const float x = log1pf(v[u] * scale);
        s1f += x;
        s2f = fmaf(x, x, s2f);
      }
    }
  }
  n = block_sum<int>(n, red);
  const double s1 = block_sum<double>((double)s1f, dred);
  const double s2 = block_sum<double>((double)s2f, dred);
  if (threadIdx.x == 0) {
    a.seg_cnt[blockIdx.x] = n;
    a.seg_mom[2 * blockIdx.x] = s1;
    a.seg_mom[2 * blockIdx.x + 1] = s2;
  }
}

__global__ void __launch_bounds__(kPackThreads) pack_write_kernel(PackArgs a) {
  __shared__ int cnt[kPackPer * (kPackThreads / 32)];
  int k;
  int64_t e0, e1;
  if (!pack_segment(a, k, e0, e1)) return;
  // normalize_by_coverage: scale = bins / total, in fp32 as the reference's float32 arrays
  const float scale = (float)a.nb / ((float)a.cov[k] + 1e-15f);
  const float thr = *a.thr;      // the mean + 15 std clip, from pack_count's moments
  int64_t pos = a.seg_out[blockIdx.x];
  // every thread runs the same number of chunks (the offsets' barriers)
  for (int64_t chunk = e0; chunk < e1; chunk += kPackChunk) {
    int nr[kPackPer], nc[kPackPer];
    float v[kPackPer];
    bool keep[kPackPer];
#pragma unroll
    for (int u = 0; u < kPackPer; ++u) {
      const int64_t e = chunk + (int64_t)u * kPackThreads + threadIdx.x;
      const bool in = e < e1;
      const int r0 = in ? a.row[e] : 0, c0 = in ? a.col[e] : 0;
      v[u] = in ? a.val[e] : 0.f;
      int r, c;
      nr[u] = nc[u] = -1;
      if (in && pack_band(a, r0, c0, r, c)) {
        nr[u] = a.new_id[r];
        nc[u] = a.new_id[c];
      }
      keep[u] = nr[u] >= 0 && nc[u] >= 0;
    }
    int off[kPackPer];
    const int total = pack_chunk_offsets(keep, cnt, off);
#pragma unroll
    for (int u = 0; u < kPackPer; ++u) {
      if (!keep[u]) continue;
      const int64_t o = pos + off[u];
      const float x = fminf(log1pf(v[u] * scale), thr);
      if (o < a.cap) {
        a.out_idx[o] = nr[u];
        a.out_idx[a.cap + o] = nc[u];
        a.out_idx[2 * a.cap + o] = k;
        a.out_val[o] = x;
      } else {
        set_status(a.status, FH_ERR_INDEX);
      }
    }
    pos += total;
  }
}

// mean + 15 std (population std, numpy's default) of all values, from the segments' moments
// summed in a fixed order; the threshold is formed in fp32 as the reference forms it from its
// fp32 mean and std.
__global__ void __launch_bounds__(256) pack_stats_kernel(PackArgs a) {
  __shared__ double red[32];
  double s1 = 0.0, s2 = 0.0;
  const int64_t nseg = a.seg0[a.n_cells] < a.max_seg ? a.seg0[a.n_cells] : a.max_seg;
  for (int64_t b = threadIdx.x; b < nseg; b += blockDim.x) {
    s1 += a.seg_mom[2 * b];
    s2 += a.seg_mom[2 * b + 1];
  }
  s1 = block_sum<double>(s1, red);
  s2 = block_sum<double>(s2, red);
  if (threadIdx.x == 0) {
    const double n = (double)a.seg_out[a.max_seg];
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

__global__ void pack_counts_kernel(PackArgs a, int64_t* out_counts) {
  out_counts[0] = a.seg_out[a.max_seg];
  out_counts[1] = a.bin_off[a.nb];
}

__host__ __device__ inline size_t pack_align(size_t x) { return (x + 255) & ~(size_t)255; }

// Segments the launches cover: every cell's segments fit when the input has at most cap
// entries (sum of ceil(len / S) <= cap / S + cells).
inline int64_t pack_max_seg(int32_t n_cells, int64_t cap) {
  return cap / kPackSeg + n_cells;
}

}  // namespace fh

using namespace fh;

extern "C" size_t fh_pack_workspace(int32_t n_cells, int32_t nbin, int32_t merge, int64_t cap) {
  if (n_cells <= 0 || nbin <= 0 || merge <= 0 || cap <= 0) return 0;
  const int64_t nb = ceil_div(nbin, merge);
  const int64_t ms = pack_max_seg(n_cells, cap);
  size_t scan = fh_scan_workspace(nb);
  if (fh_scan_workspace(n_cells) > scan) scan = fh_scan_workspace(n_cells);
  if (fh_scan_workspace(ms) > scan) scan = fh_scan_workspace(ms);
  return pack_align(sizeof(int32_t) * n_cells) + pack_align(sizeof(int64_t) * (n_cells + 1)) +
         pack_align(sizeof(int32_t) * nb) + pack_align(sizeof(int64_t) * (nb + 1)) +
         pack_align(sizeof(int32_t) * nb) + pack_align(sizeof(double) * ms) +
         pack_align(sizeof(int32_t) * ms) +
         pack_align(sizeof(double) * n_cells) + pack_align(sizeof(int32_t) * ms) +
         pack_align(sizeof(int64_t) * (ms + 1)) + pack_align(sizeof(double) * 2 * ms) +
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
  if (workspace_bytes < fh_pack_workspace(n_cells, nbin, merge, cap)) return FH_ERR_ARG;
  const int64_t ms = pack_max_seg(n_cells, cap);
  if (ms > 0x7fffffff) return FH_ERR_UNSUPPORTED;
  cudaStream_t s = (cudaStream_t)stream;
  const int nb = (int)ceil_div(nbin, merge);
  uint8_t* w = (uint8_t*)workspace;
  PackArgs a{};
  a.row = row; a.col = col; a.val = val; a.cell_off = cell_off; a.reorder = reorder;
  a.n_cells = n_cells; a.n_raw = n_raw; a.nbin = nbin; a.nb = nb; a.merge = merge;
  a.off_diag = off_diag;
  a.max_seg = ms;
  a.nseg = (int32_t*)w;              w += pack_align(sizeof(int32_t) * n_cells);
  a.seg0 = (int64_t*)w;              w += pack_align(sizeof(int64_t) * (n_cells + 1));
  a.mark = (int32_t*)w;              w += pack_align(sizeof(int32_t) * nb);
  a.bin_off = (int64_t*)w;           w += pack_align(sizeof(int64_t) * (nb + 1));
  a.new_id = (int32_t*)w;            w += pack_align(sizeof(int32_t) * nb);
  a.seg_cov = (double*)w;            w += pack_align(sizeof(double) * ms);
  a.seg_cell = (int32_t*)w;          w += pack_align(sizeof(int32_t) * ms);
  a.cov = (double*)w;                w += pack_align(sizeof(double) * n_cells);
  a.seg_cnt = (int32_t*)w;           w += pack_align(sizeof(int32_t) * ms);
  a.seg_out = (int64_t*)w;           w += pack_align(sizeof(int64_t) * (ms + 1));
  a.seg_mom = (double*)w;            w += pack_align(sizeof(double) * 2 * ms);
  a.thr = (float*)w;                 w += pack_align(sizeof(float));
  void* scan_ws = w;
  size_t scan_bytes = fh_scan_workspace(nb);
  if (fh_scan_workspace(n_cells) > scan_bytes) scan_bytes = fh_scan_workspace(n_cells);
  if (fh_scan_workspace(ms) > scan_bytes) scan_bytes = fh_scan_workspace(ms);
  a.out_idx = out_idx; a.out_val = out_val; a.cap = cap; a.status = status;
  if (cudaMemsetAsync(a.mark, 0, sizeof(int32_t) * nb, s) != cudaSuccess) return FH_ERR_LAUNCH;
  const unsigned cgrid = (unsigned)ceil_div(n_cells, 256);
  pack_segs_kernel<<<cgrid, 256, 0, s>>>(a);
  FH_CHECK_LAUNCH();
  int rc = fh_exclusive_scan(a.nseg, n_cells, a.seg0, scan_ws, scan_bytes, stream);
  if (rc) return rc;
  pack_segcell_kernel<<<cgrid, 256, 0, s>>>(a);
  pack_mark_kernel<<<(unsigned)ms, kPackThreads, 0, s>>>(a);
  pack_cov_kernel<<<cgrid, 256, 0, s>>>(a);
  FH_CHECK_LAUNCH();
  rc = fh_exclusive_scan(a.mark, nb, a.bin_off, scan_ws, scan_bytes, stream);
  if (rc) return rc;
  pack_ids_kernel<<<(unsigned)ceil_div(nb, 256), 256, 0, s>>>(a);
  pack_count_kernel<<<(unsigned)ms, kPackThreads, 0, s>>>(a);
  FH_CHECK_LAUNCH();
  rc = fh_exclusive_scan(a.seg_cnt, ms, a.seg_out, scan_ws, scan_bytes, stream);
  if (rc) return rc;
  pack_stats_kernel<<<1, 256, 0, s>>>(a);
  pack_write_kernel<<<(unsigned)ms, kPackThreads, 0, s>>>(a);
  pack_counts_kernel<<<1, 1, 0, s>>>(a, out_counts);
  FH_CHECK_LAUNCH();
  return FH_OK;
}
