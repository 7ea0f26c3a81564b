// ALS streaming contractions over X in bf16 on the 5th-generation tensor cores.
//
// The two passes over the RWR output X of every ALS iteration (the re-associated form of
// fasthigashi/parafac2_intergrative.py:374-383, 422-477, 522-529; the fp32 kernels in
// als_f32.cu state the algebra) as persistent TMA -> tcgen05 -> TMEM GEMMs:
//
//   W   = X^T [E_hi | E_lo]   M = 128 band rows, N = 2 rp, K = cells      (X read MN-major)
//   S^T = X   [G_hi | G_lo]   M = 128 cells,     N = 2 rp, K = band rows  (X read K-major),
//                             split over K with a deterministic reduction
//
// X is stored in bf16 planes X16[plane][cell][band row] (row pitch ldx, the padding zero):
// one plane (bf16(X)) or two (hi = bf16(X), lo = bf16(X - hi), X to 16 significant bits).
// The small operands E (cells x rp) and G^T (band rows x rp) are split the same way and
// stacked along N, so one MMA per plane and K step produces X*hi and X*lo side by side in
// TMEM; the epilogue adds them.  The products are exact in the fp32 accumulator, so the
// representation error is that of the operands: X's planes (2^-9 relative with one plane,
// 2^-17 with two) and the 16-significant-bit split of the small operand.
//
// Summation order.  A run of K chunks (fold, 8 by default: 512 cells or band rows) goes into
// one TMEM accumulator, which the epilogue then folds into fp32 running sums with Kahan
// compensation (plain running sums at rank 128) while the MMAs of the next run fill the other
// accumulator.  Each output is
// therefore a short tensor-core chain per run plus a compensated sum over runs, instead of
// one chain over the whole K range (10,000 cells in W, ~35,000 band rows per split of S^T at
// 10,000 cells x 500 kb), whose rounding the fitted embedding inherits.
//
// CTA (64 + 32 EW threads, one per SM, persistent over work items):
//   warp 0  TMA producer: per K step one 128 x 64 tile of X (two 64 x 64 boxes) and the
//           N x 64 slab of the hi|lo operand (N/64 boxes) into an NST-deep smem ring
//   warp 1  TMEM owner and MMA issuer: 4 x tcgen05.mma (K = 16 each) per K step and plane,
//           commit to free the stage; a commit to the accumulator's barrier after each run
//   warps 2..  EW epilogue warps (4 per 64 output columns): tcgen05.ld of their 32-lane
//           quarter and column group, hi + lo, the compensated fold, fp32 stores at the end
//           of an item
#include "tc_common.cuh"

namespace fh {

enum XPassKind { kPassXE = 0, kPassXG = 1 };

struct XPassArgs {
  int64_t rows;         // band rows
  int n_cells;          // xe: cells contracted; xg: output cells
  int rp;               // output columns (N = 2 rp)
  int64_t n_items;
  int64_t k_chunks;     // xe: chunks of 64 cells; xg: chunks of 64 band rows in total
  int64_t chunks_per_split;  // xg
  int cell_tiles;       // xg
  int plane_rows;       // rows of the X map between planes (the cells of a plane)
  int fold;             // K chunks per accumulator run (>= 1)
  float* out;           // xe: W[rows][rp]; xg: partial[splits][n_cells][rp]
  int* status;
};

constexpr int kXpFold = 8;     // default run length in K chunks of 64

template <int N, int PLANES>
struct XpCfg {
  static constexpr int kRP = N / 2;                     // output columns
  static constexpr int kCW = kRP < 64 ? kRP : 64;       // output columns per epilogue warp
  static constexpr int kEW = 4 * (kRP / kCW);           // epilogue warps
  static constexpr int kThreads = 64 + 32 * kEW;
  static constexpr bool kKahan = kEW == 4;              // compensated folds (ranks <= 64)
  static constexpr uint32_t kA = PLANES * 128 * 64 * 2; // 16 KB per plane: two 64 x 64 boxes
  static constexpr uint32_t kB = (uint32_t)N * 64 * 2;  // N/64 boxes of the hi|lo operand
  static constexpr uint32_t kStage = kA + kB;
  static constexpr int kStages = (int)((192u * 1024u) / kStage);
  static constexpr uint32_t kCols = 2 * N;              // two accumulators
  static constexpr size_t kSmem = (size_t)kStages * kStage + 1024 + 256;
};

struct XpItem {
  int x0;        // xe: first band row of the tile; xg: first cell of the tile
  int split;     // xg
  int64_t k0, k1;
  int64_t runs;  // accumulator runs of the item (one, empty, when k1 == k0)
};

template <int PASS>
__device__ __forceinline__ XpItem xp_item(const XPassArgs& p, int64_t item) {
  XpItem it;
  if (PASS == kPassXE) {
    it.x0 = (int)(item * 128);
    it.split = 0;
    it.k0 = 0;
    it.k1 = p.k_chunks;
  } else {
    const int ct = (int)(item % p.cell_tiles);
    it.split = (int)(item / p.cell_tiles);
    it.x0 = ct * 128;
    it.k0 = (int64_t)it.split * p.chunks_per_split;
    it.k1 = it.k0 + p.chunks_per_split;
    if (it.k1 > p.k_chunks) it.k1 = p.k_chunks;
    if (it.k0 > it.k1) it.k0 = it.k1;
  }
  it.runs = it.k1 > it.k0 ? (it.k1 - it.k0 + p.fold - 1) / p.fold : 1;
  return it;
}

template <int PASS, int N, int PLANES>
__global__ void __launch_bounds__(XpCfg<N, PLANES>::kThreads, 1)
    xpass_bf16_kernel(const __grid_constant__ CUtensorMap amap,
                      const __grid_constant__ CUtensorMap bmap, XPassArgs p) {
  using Cfg = XpCfg<N, PLANES>;
  constexpr int NST = Cfg::kStages;
  constexpr int CW = Cfg::kCW;
  constexpr uint32_t kIdesc = idesc_bf16(128, N, PASS == kPassXE, true);
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + (base - raw) + NST * Cfg::kStage);
  // bars: [0, NST) full, [NST, 2 NST) empty, 2 NST + {0,1} acc full, 2 NST + {2,3} acc empty,
  //       2 NST + 4 drain
  uint32_t* misc = reinterpret_cast<uint32_t*>(bars + 2 * NST + 5);
  // misc: [0] TMEM base, [1] abort flag, [2] stages issued, [3] stages consumed
  volatile int* abort = reinterpret_cast<volatile int*>(misc + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t bar0 = smem_u32(bars);
  auto full = [&](uint32_t s) { return bar0 + 8u * s; };
  auto empty = [&](uint32_t s) { return bar0 + 8u * (NST + s); };
  auto accf = [&](uint32_t a) { return bar0 + 8u * (2 * NST + a); };
  auto acce = [&](uint32_t a) { return bar0 + 8u * (2 * NST + 2 + a); };
  const uint32_t drain = bar0 + 8u * (2 * NST + 4);

  if (threadIdx.x == 0) {
    for (int i = 0; i < NST; ++i) {
      mbar_init(full(i), 1);
      mbar_init(empty(i), 1);
    }
    for (int a = 0; a < 2; ++a) {
      mbar_init(accf(a), 1);
      mbar_init(acce(a), Cfg::kEW);
    }
    mbar_init(drain, 1);
    misc[1] = 0;
    misc[2] = 0;
    misc[3] = 0;
    mbar_fence_init();
    tma_prefetch_map(&amap);
    tma_prefetch_map(&bmap);
  }
  if (warp == 1) {
    tmem_alloc(smem_u32(misc), Cfg::kCols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = misc[0];

  if (warp == 0) {
    // ------------------------------------------------------------- TMA producer
    if (lane == 0) {
      uint32_t it = 0;
      bool ok = true;
      for (int64_t item = blockIdx.x; ok && item < p.n_items; item += gridDim.x) {
        const XpItem w = xp_item<PASS>(p, item);
        for (int64_t kc = w.k0; kc < w.k1; ++kc, ++it) {
          const uint32_t s = it % NST, ph = (it / NST) & 1u;
          if (!mbar_wait(empty(s), ph ^ 1u, abort)) { ok = false; break; }
          const uint32_t sa = base + s * Cfg::kStage, sb = sa + Cfg::kA;
          const int k = (int)(kc * 64);
          mbar_expect_tx(full(s), Cfg::kStage);
#pragma unroll
          for (int pl = 0; pl < PLANES; ++pl) {
            const uint32_t d = sa + 16384u * pl;
            const int y = pl * p.plane_rows;
            if (PASS == kPassXE) {
              tma_load_2d(d, &amap, w.x0, y + k, full(s));
              tma_load_2d(d + 8192, &amap, w.x0 + 64, y + k, full(s));
            } else {
              tma_load_2d(d, &amap, k, y + w.x0, full(s));
              tma_load_2d(d + 8192, &amap, k, y + w.x0 + 64, full(s));
            }
          }
#pragma unroll
          for (int b = 0; b < N / 64; ++b) tma_load_2d(sb + 8192u * b, &bmap, 64 * b, k, full(s));
          misc[2] = it + 1;
        }
      }
      if (!ok) {
        *abort = 1;
        set_status(p.status, FH_ERR_TIMEOUT);
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    // ------------------------------------------------------------- MMA issuer
    if (lane == 0) {
      uint32_t it = 0, tc = 0;   // stages consumed, accumulator runs issued
      bool ok = true;
      for (int64_t item = blockIdx.x; ok && item < p.n_items; item += gridDim.x) {
        const XpItem w = xp_item<PASS>(p, item);
        for (int64_t run = 0; ok && run < w.runs; ++run, ++tc) {
          const uint32_t a = tc & 1u, aph = (tc >> 1) & 1u;
          if (!mbar_wait(acce(a), aph ^ 1u, abort)) { ok = false; break; }
          tc_fence_after();
          const uint32_t d = tmem + a * (uint32_t)N;
          const int64_t ks = w.k0 + run * p.fold;
          const int64_t ke = ks + p.fold < w.k1 ? ks + p.fold : w.k1;
          for (int64_t kc = ks; kc < ke; ++kc, ++it) {
            const uint32_t s = it % NST, ph = (it / NST) & 1u;
            if (!mbar_wait(full(s), ph, abort)) { ok = false; break; }
            tc_fence_after();
            misc[3] = it + 1;
            const uint32_t sa = base + s * Cfg::kStage, sb = sa + Cfg::kA;
#pragma unroll
            for (int pl = 0; pl < PLANES; ++pl)
#pragma unroll
              for (int kk = 0; kk < 4; ++kk) {
                const uint32_t ap = sa + 16384u * pl;
                const uint64_t ad = PASS == kPassXE ? sdesc_sw128(ap + 2048u * kk, 8192, 1024)
                                                    : sdesc_sw128(ap + 32u * kk, 16, 1024);
                const uint64_t bd = sdesc_sw128(sb + 2048u * kk, 8192, 1024);
                mma_bf16(d, ad, bd, kIdesc, (kc > ks || kk > 0 || pl > 0) ? 1u : 0u);
              }
            mma_commit(empty(s));
          }
          if (!ok) break;
          mma_commit(accf(a));
        }
      }
      if (!ok) {
        *abort = 1;
        set_status(p.status, FH_ERR_TIMEOUT);
      }
    }
    __syncwarp();
  } else {
    // ------------------------------------------------------------- epilogue
    const int q = warp & 3;                 // TMEM lane quarter this warp may access
    const int cb = ((warp - 2) >> 2) * CW;  // first output column of this warp
    uint32_t tc = 0;
    bool ok = true;
    for (int64_t item = blockIdx.x; ok && item < p.n_items; item += gridDim.x) {
      const XpItem w = xp_item<PASS>(p, item);
      // running sums; acc = minus the Kahan compensation (ranks <= 64; at rank 128 the ten
      // warps leave no registers for it, and the runs add into plain fp32 running sums)
      float sum[CW], acc[Cfg::kKahan ? CW : 1];
#pragma unroll
      for (int c = 0; c < CW; ++c) sum[c] = 0.f;
#pragma unroll
      for (int c = 0; c < (Cfg::kKahan ? CW : 1); ++c) acc[c] = 0.f;
      for (int64_t run = 0; run < w.runs; ++run, ++tc) {
        const uint32_t a = tc & 1u, aph = (tc >> 1) & 1u;
        const bool got = __all_sync(0xffffffffu, mbar_wait(accf(a), aph, abort));
        if (!got) {
          if (lane == 0) {
            *abort = 1;
            set_status(p.status, FH_ERR_TIMEOUT);
          }
          ok = false;
          break;
        }
        tc_fence_after();
        if (w.k1 > w.k0) {
          const uint32_t ta = tmem + ((uint32_t)(32 * q) << 16) + a * (uint32_t)N + cb;
          // 8 columns per load at rank 128, where 320 threads leave fewer registers each
          constexpr int STEP = Cfg::kEW > 4 ? 8 : 16;
#pragma unroll
          for (int c = 0; c < CW; c += STEP) {
            float hi[STEP], lo[STEP];
            if constexpr (STEP == 16) tmem_ld16x2(ta + c, ta + N / 2 + c, hi, lo);
            else tmem_ld8x2(ta + c, ta + N / 2 + c, hi, lo);
#pragma unroll
            for (int v = 0; v < STEP; ++v) {
              if constexpr (Cfg::kKahan) {
                const float y = acc[c + v] + (hi[v] + lo[v]);
                const float t = sum[c + v] + y;
                acc[c + v] = y - (t - sum[c + v]);
                sum[c + v] = t;
              } else {
                sum[c + v] += hi[v] + lo[v];
              }
            }
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(acce(a));
      }
      if (!ok) break;
      const int64_t r = (int64_t)w.x0 + 32 * q + lane;
      float* o;
      bool valid;
      if (PASS == kPassXE) {
        valid = r < p.rows;
        o = p.out + r * p.rp + cb;
      } else {
        valid = r < p.n_cells;
        o = p.out + ((int64_t)w.split * p.n_cells + r) * p.rp + cb;
      }
      if (valid) {
        float4* o4 = reinterpret_cast<float4*>(o);
#pragma unroll
        for (int v = 0; v < CW / 4; ++v) {
          if constexpr (Cfg::kKahan)
            o4[v] = make_float4(sum[4 * v] + acc[4 * v], sum[4 * v + 1] + acc[4 * v + 1],
                                sum[4 * v + 2] + acc[4 * v + 2], sum[4 * v + 3] + acc[4 * v + 3]);
          else
            o4[v] = make_float4(sum[4 * v], sum[4 * v + 1], sum[4 * v + 2], sum[4 * v + 3]);
        }
      }
    }
  }

  // ------------------------------------------------------------- teardown
  tc_fence_before();
  __syncthreads();
  if (*abort) {
    // An aborted CTA still lets its copies and MMAs in flight land before it releases TMEM
    // and exits; these waits are time-bounded and ignore the abort flag.
    if (threadIdx.x == 0)
      for (uint32_t it = misc[3]; it < misc[2]; ++it) mbar_wait(full(it % NST), (it / NST) & 1u, nullptr);
    if (threadIdx.x == 32) {
      mma_commit(drain);
      mbar_wait(drain, 0, nullptr);
    }
  }
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, Cfg::kCols);
  }
}

// x = hi + lo with hi = bf16(x), lo = bf16(x - hi): dst[row][0, rp) = hi, [rp, 2 rp) = lo.
__global__ void split_bf16_kernel(const float* __restrict__ src, int64_t n_rows, int rp,
                                  int64_t ld_src, __nv_bfloat16* __restrict__ dst) {
  const int64_t n = n_rows * rp;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = i / rp;
    const int m = (int)(i - row * rp);
    const float x = src[row * ld_src + m];
    const __nv_bfloat16 hi = __float2bfloat16_rn(x);
    const __nv_bfloat16 lo = __float2bfloat16_rn(x - __bfloat162float(hi));
    dst[row * 2 * rp + m] = hi;
    dst[row * 2 * rp + rp + m] = lo;
  }
}

template <int PASS, int N, int PLANES>
static int launch_xpass(const CUtensorMap& am, const CUtensorMap& bm, const XPassArgs& p,
                        cudaStream_t s) {
  auto k = xpass_bf16_kernel<PASS, N, PLANES>;
  using Cfg = XpCfg<N, PLANES>;
  if (ensure_smem((const void*)k, Cfg::kSmem)) return FH_ERR_LAUNCH;
  const int sms = sm_count();
  if (sms <= 0) return FH_ERR_LAUNCH;
  const int64_t grid = p.n_items < sms ? p.n_items : sms;
  k<<<(unsigned)grid, Cfg::kThreads, Cfg::kSmem, s>>>(am, bm, p);
  FH_CHECK_LAUNCH();
  return FH_OK;
}

template <int PASS, int PLANES>
static int dispatch_xpass_p(const CUtensorMap& am, const CUtensorMap& bm, const XPassArgs& p,
                            cudaStream_t s) {
  switch (p.rp) {
    case 32: return launch_xpass<PASS, 64, PLANES>(am, bm, p, s);
    case 64: return launch_xpass<PASS, 128, PLANES>(am, bm, p, s);
    case 128: return launch_xpass<PASS, 256, PLANES>(am, bm, p, s);
    default: return FH_ERR_UNSUPPORTED;
  }
}

template <int PASS>
static int dispatch_xpass(const CUtensorMap& am, const CUtensorMap& bm, const XPassArgs& p,
                          int planes, cudaStream_t s) {
  return planes == 2 ? dispatch_xpass_p<PASS, 2>(am, bm, p, s)
                     : dispatch_xpass_p<PASS, 1>(am, bm, p, s);
}

}  // namespace fh

using namespace fh;

extern "C" int fh_split_bf16(const float* src, int64_t n_rows, int32_t rp, int64_t ld_src,
                             uint16_t* dst, void* stream) {
  if (!src || !dst || n_rows <= 0 || rp <= 0 || ld_src < rp) return FH_ERR_ARG;
  const int64_t n = n_rows * rp;
  int64_t blocks = ceil_div(n, 256);
  if (blocks > 4096) blocks = 4096;
  split_bf16_kernel<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(
      src, n_rows, rp, ld_src, reinterpret_cast<__nv_bfloat16*>(dst));
  FH_CHECK_LAUNCH();
  return FH_OK;
}

extern "C" int fh_xe_bf16(const uint16_t* X16, int64_t ldx, int32_t n_cells_total,
                          int32_t planes, int32_t n_cells, int64_t rows, const uint16_t* E2,
                          int32_t rp, int32_t fold, float* W, int* status, void* stream) {
  if (!X16 || !E2 || !W || n_cells <= 0 || n_cells > n_cells_total || rows <= 0 || ldx < rows ||
      ldx % 128 || (planes != 1 && planes != 2) || fold < 0)
    return FH_ERR_ARG;
  if (rp != 32 && rp != 64 && rp != 128) return FH_ERR_UNSUPPORTED;
  // the map ends at the last 128-row tile, so no box reads past the band rows asked for
  const uint64_t inner = (uint64_t)ceil_div(rows, 128) * 128;
  CUtensorMap am, bm;
  if (!make_map_bf16(&am, X16, inner, (uint64_t)n_cells_total * planes, (uint64_t)ldx, 64) ||
      !make_map_bf16(&bm, E2, (uint64_t)(2 * rp), (uint64_t)n_cells, (uint64_t)(2 * rp), 64))
    return FH_ERR_LAUNCH;
  XPassArgs p{};
  p.plane_rows = n_cells_total;
  p.rows = rows;
  p.n_cells = n_cells;
  p.rp = rp;
  p.n_items = ceil_div(rows, 128);
  p.k_chunks = ceil_div(n_cells, 64);
  p.fold = fold > 0 ? fold : kXpFold;
  p.out = W;
  p.status = status;
  return dispatch_xpass<kPassXE>(am, bm, p, planes, (cudaStream_t)stream);
}

// Splits of the band-row dimension for fh_xg_bf16: about whole waves of items over the SMs,
// each split at least 16 chunks of 64 band rows.
extern "C" int fh_xg_bf16_splits(int32_t n_cells, int64_t rows) {
  if (n_cells <= 0 || rows <= 0) return 1;
  const int sms = sm_count() > 0 ? sm_count() : 152;
  const int64_t ct = ceil_div(n_cells, 128), chunks = ceil_div(rows, 64);
  int best = 1;
  double best_cost = 1e300;
  for (int s = 1; s <= 256; ++s) {
    if (s > 1 && ceil_div(chunks, s) < 16) break;
    const int64_t items = ct * s;
    const double cost = (double)ceil_div(items, sms) / s * (1.0 + 0.002 * s);
    if (cost < best_cost) { best_cost = cost; best = s; }
  }
  return best;
}

extern "C" int fh_xg_bf16(const uint16_t* X16, int64_t ldx, int32_t n_cells_total,
                          int32_t planes, int32_t n_cells, int64_t rows, const uint16_t* G2,
                          int32_t rp, int32_t splits, int32_t fold, float* partial, float* out,
                          int32_t accumulate, int* status, void* stream) {
  if (!X16 || !G2 || !partial || !out || n_cells <= 0 || n_cells > n_cells_total || rows <= 0 ||
      ldx < rows || ldx % 128 || splits <= 0 || (planes != 1 && planes != 2) || fold < 0)
    return FH_ERR_ARG;
  if (rp != 32 && rp != 64 && rp != 128) return FH_ERR_UNSUPPORTED;
  const uint64_t inner = (uint64_t)ceil_div(rows, 128) * 128;
  CUtensorMap am, bm;
  if (!make_map_bf16(&am, X16, inner, (uint64_t)n_cells_total * planes, (uint64_t)ldx, 64) ||
      !make_map_bf16(&bm, G2, (uint64_t)(2 * rp), (uint64_t)rows, (uint64_t)(2 * rp), 64))
    return FH_ERR_LAUNCH;
  const int64_t chunks = ceil_div(rows, 64);
  const int64_t per = ceil_div(chunks, splits);
  const int used = (int)ceil_div(chunks, per);   // every split non-empty
  XPassArgs p{};
  p.rows = rows;
  p.n_cells = n_cells;
  p.rp = rp;
  p.cell_tiles = (int)ceil_div(n_cells, 128);
  p.plane_rows = n_cells_total;
  p.n_items = (int64_t)p.cell_tiles * used;
  p.k_chunks = chunks;
  p.chunks_per_split = per;
  p.fold = fold > 0 ? fold : kXpFold;
  p.out = partial;
  p.status = status;
  cudaStream_t s = (cudaStream_t)stream;
  int rc = dispatch_xpass<kPassXG>(am, bm, p, planes, s);
  if (rc) return rc;
  const int64_t n = (int64_t)n_cells * rp;
  int64_t blocks = ceil_div(n, 256);
  if (blocks > 4096) blocks = 4096;
  reduce_splits_kernel<float><<<(unsigned)blocks, 256, 0, s>>>(partial, used, n, out,
                                                                accumulate != 0);
  FH_CHECK_LAUNCH();
  return FH_OK;
}
