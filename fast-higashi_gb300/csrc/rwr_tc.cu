// Partial random walk with restart on the 5th-generation tensor cores (tcgen05), writing the
// bf16 planes of X that the tensor-core X passes read.
//
// Reference: fasthigashi/partial_rwr.py:75-138 (do_conv=False, do_col=False) fed by
// densify_jit (fasthigashi/sparse_for_schic.py:279-320); rwr_f32.cu states the algebra:
//   S2 = A A^T (diagonal zeroed), S1 = A[:, s0:s0+b]
//   L  = 0.75 S1 / colsum(S1) + 0.25 S2 / colsum(S2),  P = L / colsum(L)
//   Z_0 = A,  Z_{t+1} = 0.5 P Z_t + 0.5 A,  X = Z_epochs  (= Q_epochs A of the reference)
//
// One CTA (8 warps, one per SM, persistent over (tile, cell) items) per item at a time:
//   smem   Z as bf16 hi and lo planes (128 rows x npad columns, 128-byte swizzled, the
//          layout tcgen05 reads), P as hi and lo planes (128 x 128)
//   TMEM   D (the fp32 accumulator, npad columns) and A in fp32 (npad columns)
//   S2     = A_hi A_hi^T + A_hi A_lo^T + A_lo A_hi^T   (K = npad)        -> D
//   P      from D row by row: colsum(S2) is a row sum (S2 is symmetric), colsum(S1) a
//          column sum of the smem tile, colsum(L) = 0.75 c1/(c1+eps) + 0.25 c2/(c2+eps)
//          in closed form (the reference sums L's columns numerically; they agree to
//          rounding).  With the 1e-8 floor every column sum is positive, so the reference's
//          zero-column rule (partial_rwr.py:96-97) never applies; it is kept for c1 = c2 = 0.
//   epoch  D = P_hi Z_hi + P_hi Z_lo + P_lo Z_hi  (K = 128, N = npad), then each thread
//          turns its row of D and A into Z_{t+1} = 0.5 D + 0.5 A and writes the hi/lo planes
//          back in place (the MMA that read them has completed)
//   out    the last epoch's fp32 Z is rounded to the output planes (one: bf16(Z); two: hi and
//          the residual lo) through a staging copy in smem, then stored contiguously.
// The split products carry every operand to 16 significant bits, so the result is fp32-class.
// Thread (warp w, lane l) serves row p = 32 (w % 4) + l (the TMEM lane quarter its warp may
// read) and the column quarter w / 4 (16 warps).  Tiles wider than 256 columns use rwr_f32.cu.
// The contacts of an item are loaded into registers before its Z init, so their latency
// overlaps the init (per item, measured with clock stamps at c3 shapes: 3.2k -> 1.1k cycles),
// and the Z init writes whole 16-byte chunks of the thread's row and column quarter without a
// division (3.2k -> 2.0k cycles).  Loading two 16-column chunks per tensor-memory wait in the
// epochs and in the P build measured slower (127 registers; 107 against 105 ms per c3 fit).
//
// Form 2 (kPipe, tiles up to 192 columns): P goes to tensor memory (columns 384-511) as the
// A operand of the epoch products, the epochs are issued per 64-column block of Z with an
// mbarrier each (block j's epilogue overlaps blocks j+1..'s products; the columns of Z are
// independent recurrences sharing P), and the output leaves through a dedicated staging
// buffer by bulk copies that run on into the next item.  Measured at c3 shapes it is the
// slower form (epochs 39k against 30k cycles per item: each block's epilogue pays a full
// tensor-memory round trip and two barriers, more than the products it hides behind, while
// the bulk output saves 2k cycles), so form 1 is the default and the engine's autotuner
// times both.
#include "tc_common.cuh"

namespace fh {

constexpr int kRtThreads = 512;   // 16 warps: four per TMEM lane quarter
constexpr float kRtFloor = 1e-8f;  // densify floor, sparse_for_schic.py:320
constexpr float kRtEps = 1e-15f;   // column-sum guard, partial_rwr.py:90,91,111
constexpr int kRtMaxPad = 256;     // npad: columns rounded up to 64, at most one MMA's N
constexpr int kRtPre = 8;          // contacts per thread loaded ahead of the Z init

struct RtArgs {
  const fh_tile* tiles;
  int n_tiles;
  int n_cells;
  int max_rows, max_width, npad_max;
  const uint2* entries;
  const int64_t* offsets;
  __nv_bfloat16* out16;
  int64_t cell_stride;
  int64_t plane_stride;  // > 0: write the lo plane too
  double* sumsq;
  int* status;
};

// Byte offset of element (row p, column j) in a 128-row operand of 64-column blocks with the
// 128-byte swizzle (16-byte chunk index XOR row mod 8), the layout TMA's SWIZZLE_128B writes.
__device__ __forceinline__ uint32_t sw_off(int p, int j) {
  return (uint32_t)((j >> 6) * 16384 + p * 128 + ((((j & 63) >> 3) ^ (p & 7)) << 4) + (j & 7) * 2);
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void tmem_st16(uint32_t ta, const float (&v)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(ta),
      "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
      "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
      "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])), "r"(__float_as_uint(v[8])),
      "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
      "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])),
      "r"(__float_as_uint(v[15]))
      : "memory");
}
__device__ __forceinline__ void tmem_wait_st() {
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 a, __nv_bfloat16 b) {
  return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}

// Rounds a pair to bf16 (one packed conversion) and returns the residuals' pair too.
__device__ __forceinline__ void split2(float a, float b, uint32_t& hi, uint32_t& lo) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  hi = *reinterpret_cast<const uint32_t*>(&h);
  const float ra = a - __uint_as_float(hi << 16), rb = b - __uint_as_float(hi & 0xffff0000u);
  const __nv_bfloat162 l = __floats2bfloat162_rn(ra, rb);
  lo = *reinterpret_cast<const uint32_t*>(&l);
}

// Splits 8 values into bf16 hi and lo and stores both 16-byte chunks.
__device__ __forceinline__ void store_split8(uint8_t* hi, uint8_t* lo, uint32_t off,
                                             const float* v) {
  uint32_t h[4], l[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) split2(v[2 * e], v[2 * e + 1], h[e], l[e]);
  *reinterpret_cast<uint4*>(hi + off) = make_uint4(h[0], h[1], h[2], h[3]);
  *reinterpret_cast<uint4*>(lo + off) = make_uint4(l[0], l[1], l[2], l[3]);
}

__device__ __forceinline__ float ld_split(const uint8_t* hi, const uint8_t* lo, uint32_t off) {
  return __bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(hi + off)) +
         __bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(lo + off));
}

// Output staging of the pipelined form: both planes of a 128 x 192 tile with their 16-byte
// phase offsets.
constexpr uint32_t kRpStageBytes = 2u * 128u * 192u * 2u + 256u;
constexpr int kRpMaxPad = 192;
// tensor memory columns of the pipelined form: D [0, 192), A [192, 384), P hi / lo [384, 512)
constexpr uint32_t kRpColA = 192, kRpColPh = 384, kRpColPl = 448;

// Shared memory of the kernel: Z planes, then P planes (plain form) or the output staging
// (pipelined form), then the per-column sums, factors, reductions and barriers.
__host__ __device__ inline size_t rt_smem_bytes(int npad_max, bool pipe) {
  return (size_t)npad_max / 64 * 16384 * 2 + (pipe ? kRpStageBytes : 65536u) +
         11 * 128 * sizeof(float) + 64 * sizeof(double) + 64 + 1024;
}

// D[tmem] (+)= A[tmem] * B[smem] (A: 128 lanes, K along the columns as bf16 pairs).
__device__ __forceinline__ void mma_bf16_ta(uint32_t d_tmem, uint32_t a_tmem, uint64_t bdesc,
                                            uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "r"(a_tmem), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void tmem_st8(uint32_t ta, const uint32_t (&v)[8]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(ta),
      "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7])
      : "memory");
}
// Shared -> global bulk copy (both addresses 16-byte aligned, bytes a multiple of 16).
__device__ __forceinline__ void bulk_store(void* gdst, uint32_t ssrc, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst),
               "r"(ssrc), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
// Waits until the committed bulk copies have read their shared memory / have completed.
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_all() {
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

template <bool kPipe>
__global__ void __launch_bounds__(kRtThreads, 1) rwr_tc_kernel(RtArgs a) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  uint8_t* g = smem_raw + (base - raw);
  const uint32_t zbytes = (uint32_t)(a.npad_max / 64) * 16384u;
  uint8_t* Zhi = g;
  uint8_t* Zlo = g + zbytes;
  uint8_t* Phi = g + 2 * zbytes;        // plain form: P planes; pipelined form: the staging
  uint8_t* Plo = Phi + 32768;
  uint8_t* Stg = g + 2 * zbytes;
  float* cs1p = reinterpret_cast<float*>(g + 2 * zbytes + (kPipe ? kRpStageBytes : 65536u));
  float* cs2p = cs1p + 512;                              // [4][128] partial row sums of S2
  float* fac = cs2p + 512;                               // [3][128] per-column P factors
  double* dred = reinterpret_cast<double*>(fac + 384);   // [64]
  uint64_t* mbar = reinterpret_cast<uint64_t*>(dred + 64);  // [0] A A^T, [1 + j] block j
  uint32_t* misc = reinterpret_cast<uint32_t*>(mbar + 4);  // [0] TMEM base
  const uint32_t sZhi = base, sZlo = base + zbytes, sPhi = base + 2 * zbytes,
                 sPlo = sPhi + 32768, sStg = base + 2 * zbytes;

  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  const int q4 = w & 3, h = w >> 2;
  const int p = 32 * q4 + lane;
  const uint32_t bar = smem_u32(mbar);
  if (tid == 0) {
    for (int i = 0; i < (kPipe ? 4 : 1); ++i) mbar_init(bar + 8u * i, 1);
    mbar_fence_init();
  }
  if (w == 0) {
    tmem_alloc(smem_u32(misc), 512);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = misc[0];
  const uint32_t lane_off = (uint32_t)(32 * q4) << 16;
  const uint32_t tD = tmem + lane_off, tA = tmem + (kPipe ? kRpColA : 256u) + lane_off;
  const __nv_bfloat16 fl_hi = __float2bfloat16_rn(kRtFloor);
  const __nv_bfloat16 fl_lo = __float2bfloat16_rn(kRtFloor - __bfloat162float(fl_hi));
  uint32_t phase = 0;
  uint32_t bphase = 0;   // pipelined form, bit j: parity of block j's next mbarrier phase
  bool ok = true;

  // Issues the MMAs of one product group (thread 0) and waits for them (all threads).
  auto mma_wait = [&]() -> bool {
    if (tid == 0) mma_commit(bar);
    const bool got = mbar_wait(bar, phase, nullptr);
    phase ^= 1u;
    const bool any_fail = __syncthreads_or(!got);
    tc_fence_after();
    return !any_fail;
  };

  const int64_t items = (int64_t)a.n_tiles * a.n_cells;
  for (int64_t item = blockIdx.x; ok && item < items; item += gridDim.x) {
    const int t = (int)(item / a.n_cells), c = (int)(item - (int64_t)t * a.n_cells);
    const fh_tile T = a.tiles[t];
    const int b = T.rows, n = T.width, s0 = T.s0, epochs = T.n_rwr;
    if (b <= 0 || b > a.max_rows || b > 128 || n < b || n > a.max_width || n > a.npad_max ||
        s0 < 0 || s0 + b > n || epochs < 0 || (kPipe && n > kRpMaxPad)) {
      if (tid == 0) set_status(a.status, FH_ERR_ARG);
      continue;
    }
    const int npad = (n + 63) & ~63;
    const int hw = npad / 4;  // columns per quarter (a multiple of 16)
    // the first kRtPre entries of every thread go to registers now: their loads overlap the
    // Z init below
    const int64_t e0 = a.offsets[(int64_t)t * a.n_cells + c];
    const int64_t e1 = a.offsets[(int64_t)t * a.n_cells + c + 1];
    uint2 pre[kRtPre];
#pragma unroll
    for (int u = 0; u < kRtPre; ++u) {
      const int64_t e = e0 + tid + (int64_t)u * kRtThreads;
      pre[u] = e < e1 ? a.entries[e] : make_uint2(0u, 0u);
    }
    // ---- 1. Z = floor on the tile, zero on the padding (both planes): row p, the thread's
    // column quarter, 16-byte chunks; only the chunk holding column n is mixed
    {
      const uint32_t fh2 = pack2(fl_hi, fl_hi), fl2 = pack2(fl_lo, fl_lo);
      const __nv_bfloat16 zb = __float2bfloat16_rn(0.f);
      for (int j0 = h * hw; j0 < (h + 1) * hw; j0 += 8) {
        uint4 hv = make_uint4(0u, 0u, 0u, 0u), lv = hv;
        if (p < b && j0 + 8 <= n) {
          hv = make_uint4(fh2, fh2, fh2, fh2);
          lv = make_uint4(fl2, fl2, fl2, fl2);
        } else if (p < b && j0 < n) {
          uint32_t h4[4], l4[4];
#pragma unroll
          for (int e = 0; e < 8; e += 2) {
            const bool in0 = j0 + e < n, in1 = j0 + e + 1 < n;
            h4[e / 2] = pack2(in0 ? fl_hi : zb, in1 ? fl_hi : zb);
            l4[e / 2] = pack2(in0 ? fl_lo : zb, in1 ? fl_lo : zb);
          }
          hv = make_uint4(h4[0], h4[1], h4[2], h4[3]);
          lv = make_uint4(l4[0], l4[1], l4[2], l4[3]);
        }
        const uint32_t off = sw_off(p, j0);
        *reinterpret_cast<uint4*>(Zhi + off) = hv;
        *reinterpret_cast<uint4*>(Zlo + off) = lv;
      }
    }
    __syncthreads();
    // ---- 2. the cell's contacts (floored at 1e-8)
    {
      auto put = [&](const uint2 en) {
        const int r = (int)(en.x & 0xffffu), j = (int)(en.x >> 16);
        if (r >= b || j >= n) {
          set_status(a.status, FH_ERR_INDEX);
          return;
        }
        const float v = fmaxf(__uint_as_float(en.y), kRtFloor);
        uint32_t hv, lv;
        split2(v, 0.f, hv, lv);                 // packed conversions (low halves used)
        const uint32_t off = sw_off(r, j);
        *reinterpret_cast<uint16_t*>(Zhi + off) = (uint16_t)(hv & 0xffffu);
        *reinterpret_cast<uint16_t*>(Zlo + off) = (uint16_t)(lv & 0xffffu);
      };
#pragma unroll
      for (int u = 0; u < kRtPre; ++u)
        if (e0 + tid + (int64_t)u * kRtThreads < e1) put(pre[u]);
      for (int64_t e = e0 + tid + (int64_t)kRtPre * kRtThreads; e < e1; e += kRtThreads)
        put(a.entries[e]);
    }
    __syncthreads();
    // ---- 3. row p of A into TMEM (this thread's column quarter); column sums of S1
    for (int j0 = h * hw; j0 < (h + 1) * hw; j0 += 16) {
      float v[16];
#pragma unroll
      for (int e = 0; e < 16; e += 8) {
        const uint32_t off = sw_off(p, j0 + e);
        const uint4 hv = *reinterpret_cast<const uint4*>(Zhi + off);
        const uint4 lv = *reinterpret_cast<const uint4*>(Zlo + off);
        const uint32_t hw4[4] = {hv.x, hv.y, hv.z, hv.w}, lw4[4] = {lv.x, lv.y, lv.z, lv.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          v[e + 2 * k] = __uint_as_float(hw4[k] << 16) + __uint_as_float(lw4[k] << 16);
          v[e + 2 * k + 1] = __uint_as_float(hw4[k] & 0xffff0000u) +
                             __uint_as_float(lw4[k] & 0xffff0000u);
        }
      }
      tmem_st16(tA + j0, v);
    }
    {
      const int q = tid & 127, part = tid >> 7;
      float s = 0.f;
      if (q < b) {
        const int pe = min(b, 32 * part + 32);
#pragma unroll 8
        for (int pp = 32 * part; pp < pe; ++pp) s += ld_split(Zhi, Zlo, sw_off(pp, s0 + q));
      }
      cs1p[part * 128 + q] = s;
    }
    tmem_wait_st();
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    // ---- 4. S2 = A A^T (split products) into D
    if (tid == 0) {
      tc_fence_after();
      const uint32_t idesc = idesc_bf16(128, 128, false, false);
      for (int ks = 0; ks < npad / 16; ++ks) {
        const uint32_t ko = (uint32_t)(ks >> 2) * 16384u + (uint32_t)(ks & 3) * 32u;
        const uint64_t ah = sdesc_sw128(sZhi + ko, 16, 1024), al = sdesc_sw128(sZlo + ko, 16, 1024);
        mma_bf16(tmem, ah, ah, idesc, ks > 0 ? 1u : 0u);
        mma_bf16(tmem, ah, al, idesc, 1u);
        mma_bf16(tmem, al, ah, idesc, 1u);
      }
    }
    if (!mma_wait()) { ok = false; break; }
    // ---- 5. P: row sums of S2 (diagonal excluded) = its column sums, then P row by row
    {
      float s = 0.f;
      for (int q0 = 32 * h; q0 < 32 * h + 32; q0 += 16) {
        float d[16], unused[16];
        tmem_ld16x2(tD + q0, tD + q0, d, unused);
#pragma unroll
        for (int e = 0; e < 16; ++e) {
          const int q = q0 + e;
          if (q != p && q < b) s += d[e];
        }
      }
      cs2p[h * 128 + p] = s;
    }
    __syncthreads();
    // per column q: f1 = 0.75 / (c1 + eps), f2 = 0.25 / (c2 + eps), fl = 1 / (colsum(L) + eps)
    if (tid < 128) {
      const int q = tid;
      const float c1 = (cs1p[q] + cs1p[128 + q]) + (cs1p[256 + q] + cs1p[384 + q]);
      const float c2 = (cs2p[q] + cs2p[128 + q]) + (cs2p[256 + q] + cs2p[384 + q]);
      const float f1 = 0.75f / (c1 + kRtEps), f2 = 0.25f / (c2 + kRtEps);
      fac[q] = f1;
      fac[128 + q] = f2;
      fac[256 + q] = (c1 == 0.f && c2 == 0.f) ? -1.f : 1.f / (fmaf(c1, f1, c2 * f2) + kRtEps);
    }
    __syncthreads();
    for (int q0 = 32 * h; q0 < 32 * h + 32; q0 += 16) {
      // S2 from D; S1 = A[p][s0 + q] from A's fp32 copy in TMEM when the 16-column window
      // lies inside A's columns (else from the smem planes, same values)
      const bool in_tm = s0 + q0 + 16 <= (kPipe ? npad : kRtMaxPad);
      float d[16], a1v[16], pv[16];
      tmem_ld16x2(tD + q0, in_tm ? tA + s0 + q0 : tA, d, a1v);
#pragma unroll
      for (int e = 0; e < 16; ++e) {
        const int q = q0 + e;
        float v = 0.f;
        if (p < b && q < b) {
          const float fl = fac[256 + q];
          if (fl < 0.f) {
            v = (p == q) ? 1.f / (1.f + kRtEps) : 0.f;   // zero column: unit diagonal
          } else {
            const float s2 = (p == q) ? 0.f : d[e];
            const float a1 = in_tm ? a1v[e] : ld_split(Zhi, Zlo, sw_off(p, s0 + q));
            v = fmaf(a1, fac[q], s2 * fac[128 + q]) * fl;
          }
        }
        pv[e] = v;
      }
      if constexpr (kPipe) {
        // row p of P as bf16 pairs (K along the columns) for the A operand of the epochs
        uint32_t hv[8], lv[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) split2(pv[2 * e], pv[2 * e + 1], hv[e], lv[e]);
        tmem_st8(tmem + lane_off + kRpColPh + (uint32_t)(q0 >> 1), hv);
        tmem_st8(tmem + lane_off + kRpColPl + (uint32_t)(q0 >> 1), lv);
      } else {
        store_split8(Phi, Plo, sw_off(p, q0), pv);
        store_split8(Phi, Plo, sw_off(p, q0 + 8), pv + 8);
      }
    }
    if constexpr (kPipe) tmem_wait_st();
    else fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    // ---- 6. Z_{t+1} = 0.5 P Z_t + 0.5 A; the last epoch writes the output staging
    // plain form: the staging overlaps Zhi, free once the last MMA has completed
    uint8_t* stage = kPipe ? Stg : Zhi;
    const int64_t g0 = (int64_t)c * a.cell_stride + T.xoff;
    const int mis = (int)(g0 & 7);           // staging shares the global 16-byte phase
    float ss = 0.f;
    const bool two = a.plane_stride > 0;
    const int64_t tot = (int64_t)b * n;
    const int64_t lo_base = (tot + 15) & ~(int64_t)7;   // lo plane staging, 16-byte aligned
    auto emit = [&](int j0, const float (&z)[16]) {
      if (p >= b) return;
      uint16_t* st16 = reinterpret_cast<uint16_t*>(stage);
#pragma unroll
      for (int e = 0; e < 16; e += 2) {
        uint32_t hv, lv;
        split2(z[e], z[e + 1], hv, lv);        // packed conversions of the pair
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const int j = j0 + e + u;
          if (j < n) {
            const uint32_t hb = u ? (hv >> 16) : (hv & 0xffffu);
            const uint32_t lb = u ? (lv >> 16) : (lv & 0xffffu);
            const int64_t k = (int64_t)p * n + j + mis;
            st16[k] = (uint16_t)hb;
            float sv = __uint_as_float(hb << 16);
            if (two) {
              st16[lo_base + k] = (uint16_t)lb;
              sv += __uint_as_float(lb << 16);
            }
            ss = fmaf(sv, sv, ss);
          }
        }
      }
    };
    if constexpr (kPipe) {
      const int nblk = npad / 64;
      // block j's products of one epoch: D[:, 64 j ..] = P Z[:, 64 j ..] split three ways,
      // P (the A operand) from tensor memory, Z from shared memory
      auto issue_block = [&](int jb) {
        tc_fence_after();
        const uint32_t idesc = idesc_bf16(128, 64, false, true);
        const uint32_t d = tmem + 64u * (uint32_t)jb;
        for (int ks = 0; ks < 8; ++ks) {
          const uint32_t zk = (uint32_t)jb * 16384u + (uint32_t)ks * 2048u;
          const uint64_t zh = sdesc_sw128(sZhi + zk, 16384, 1024),
                         zl = sdesc_sw128(sZlo + zk, 16384, 1024);
          const uint32_t ph = tmem + kRpColPh + 8u * (uint32_t)ks;
          const uint32_t pl = tmem + kRpColPl + 8u * (uint32_t)ks;
          mma_bf16_ta(d, ph, zh, idesc, ks > 0 ? 1u : 0u);
          mma_bf16_ta(d, ph, zl, idesc, 1u);
          mma_bf16_ta(d, pl, zh, idesc, 1u);
        }
        mma_commit(bar + 8u * (uint32_t)(1 + jb));
      };
      if (epochs > 0) {
        if (tid == 0)
          for (int jb = 0; jb < nblk; ++jb) issue_block(jb);
        // the next item's contact segment into L2 while this item's epochs run
        const int64_t nitem = item + gridDim.x;
        if (nitem < items) {
          const int tn = (int)(nitem / a.n_cells), cn = (int)(nitem - (int64_t)tn * a.n_cells);
          const int64_t f0 = a.offsets[(int64_t)tn * a.n_cells + cn];
          const int64_t f1 = a.offsets[(int64_t)tn * a.n_cells + cn + 1];
          const char* seg = reinterpret_cast<const char*>(a.entries + f0);
          for (int64_t off = (int64_t)tid * 128; off < (f1 - f0) * 8; off += kRtThreads * 128)
            asm volatile("prefetch.global.L2 [%0];" ::"l"(seg + off));
        }
      }
      for (int ep = 0; ep < epochs && ok; ++ep) {
        if (ep == epochs - 1) {
          // every block's products; the previous item's bulk copy has read the staging
          bool got = true;
          for (int jb = 0; jb < nblk; ++jb) {
            got = mbar_wait(bar + 8u * (uint32_t)(1 + jb), (bphase >> jb) & 1u, nullptr) && got;
            bphase ^= 1u << jb;
          }
          if (tid == 0) bulk_wait_read();
          if (__syncthreads_or(!got)) { ok = false; break; }
          tc_fence_after();
          for (int jb = 0; jb < nblk; ++jb) {
            const int j0 = 64 * jb + 16 * h;
            float d[16], av[16], z[16];
            tmem_ld16x2(tD + j0, tA + j0, d, av);
#pragma unroll
            for (int e = 0; e < 16; ++e) z[e] = fmaf(0.5f, d[e], 0.5f * av[e]);
            emit(j0, z);
          }
          tc_fence_before();
          break;
        }
        for (int jb = 0; jb < nblk; ++jb) {
          const bool got = mbar_wait(bar + 8u * (uint32_t)(1 + jb), (bphase >> jb) & 1u, nullptr);
          bphase ^= 1u << jb;
          tc_fence_after();
          if (got) {
            const int j0 = 64 * jb + 16 * h;
            float d[16], av[16], z[16];
            tmem_ld16x2(tD + j0, tA + j0, d, av);
#pragma unroll
            for (int e = 0; e < 16; ++e) z[e] = fmaf(0.5f, d[e], 0.5f * av[e]);
            store_split8(Zhi, Zlo, sw_off(p, j0), z);
            store_split8(Zhi, Zlo, sw_off(p, j0 + 8), z + 8);
          }
          fence_proxy_async();
          tc_fence_before();
          if (__syncthreads_or(!got)) { ok = false; break; }
          if (tid == 0) issue_block(jb);
        }
      }
    } else {
      for (int ep = 0; ep < epochs; ++ep) {
        if (tid == 0) {
          tc_fence_after();
          const uint32_t idesc = idesc_bf16(128, npad, false, true);
          for (int ks = 0; ks < 8; ++ks) {
            const uint32_t pk = (uint32_t)(ks >> 2) * 16384u + (uint32_t)(ks & 3) * 32u;
            const uint32_t zk = (uint32_t)ks * 2048u;
            const uint64_t ph = sdesc_sw128(sPhi + pk, 16, 1024), pl = sdesc_sw128(sPlo + pk, 16, 1024);
            const uint64_t zh = sdesc_sw128(sZhi + zk, 16384, 1024),
                           zl = sdesc_sw128(sZlo + zk, 16384, 1024);
            mma_bf16(tmem, ph, zh, idesc, ks > 0 ? 1u : 0u);
            mma_bf16(tmem, ph, zl, idesc, 1u);
            mma_bf16(tmem, pl, zh, idesc, 1u);
          }
        }
        if (ep == 0) {
          // the next item's contact segment into L2 while this item's first
          // epoch runs on the tensor cores (issued above)
          const int64_t nitem = item + gridDim.x;
          if (nitem < items) {
            const int tn = (int)(nitem / a.n_cells), cn = (int)(nitem - (int64_t)tn * a.n_cells);
            const int64_t f0 = a.offsets[(int64_t)tn * a.n_cells + cn];
            const int64_t f1 = a.offsets[(int64_t)tn * a.n_cells + cn + 1];
            const char* seg = reinterpret_cast<const char*>(a.entries + f0);
            for (int64_t off = (int64_t)tid * 128; off < (f1 - f0) * 8; off += kRtThreads * 128)
              asm volatile("prefetch.global.L2 [%0];" ::"l"(seg + off));
          }
        }
        if (!mma_wait()) { ok = false; break; }
        const bool last = ep == epochs - 1;
        if (last) __syncthreads();   // nobody reads Z any more: the staging may overwrite it
        for (int j0 = h * hw; j0 < (h + 1) * hw; j0 += 16) {
          float d[16], av[16], z[16];
          tmem_ld16x2(tD + j0, tA + j0, d, av);
#pragma unroll
          for (int e = 0; e < 16; ++e) z[e] = fmaf(0.5f, d[e], 0.5f * av[e]);
          if (last) {
            emit(j0, z);
          } else {
            store_split8(Zhi, Zlo, sw_off(p, j0), z);
            store_split8(Zhi, Zlo, sw_off(p, j0 + 8), z + 8);
          }
        }
        if (!last) fence_proxy_async();
        tc_fence_before();
        __syncthreads();
      }
    }
    if (!ok) break;
    if (epochs == 0) {
      if constexpr (kPipe) {
        if (tid == 0) bulk_wait_read();
        __syncthreads();
      }
      for (int j0 = h * hw; j0 < (h + 1) * hw; j0 += 16) {
        float av[16], unused[16];
        tmem_ld16x2(tA + j0, tA + j0, av, unused);
        emit(j0, av);
      }
      tc_fence_before();
      __syncthreads();
    }
    // ---- 7. staging -> X16 (contiguous b x n run of the cell's row), squared norm
    if constexpr (kPipe) {
      fence_proxy_async();
      __syncthreads();
    }
    {
      // the staging holds element k at index k + mis, and X16's planes start 16-byte aligned
      // with every plane a multiple of 8 elements long, so element k and its staging copy
      // share the 16-byte phase: the middle of the run moves as 16-byte vectors
      for (int pl = 0; pl < (two ? 2 : 1); ++pl) {
        const __nv_bfloat16* st = reinterpret_cast<const __nv_bfloat16*>(stage) + pl * lo_base;
        __nv_bfloat16* o = a.out16 + g0 + pl * a.plane_stride;
        const int64_t head = (8 - mis) & 7;                  // elements before the first vector
        const int64_t nvec = tot > head ? (tot - head) >> 3 : 0;
        const int64_t tail0 = head + (nvec << 3);
        for (int64_t k = tid; k < head && k < tot; k += kRtThreads) o[k] = st[k + mis];
        if constexpr (kPipe) {
          // the middle as one bulk copy that runs on while the next item starts (its
          // last epoch waits for the copy to have read the staging)
          if (tid == 0 && nvec > 0)
            bulk_store(o + head, sStg + (uint32_t)(pl * lo_base + head + mis) * 2u,
                       (uint32_t)(nvec * 16));
        } else {
          const uint4* sv = reinterpret_cast<const uint4*>(st + head + mis);
          uint4* ov = reinterpret_cast<uint4*>(o + head);
          for (int64_t k = tid; k < nvec; k += kRtThreads) ov[k] = sv[k];
        }
        for (int64_t k = tail0 + tid; k < tot; k += kRtThreads) o[k] = st[k + mis];
      }
      if constexpr (kPipe) {
        if (tid == 0) bulk_commit();
      }
      const double sst = block_sum<double>((double)ss, dred);
      if (tid == 0 && a.sumsq) a.sumsq[(int64_t)t * a.n_cells + c] = sst;
      __syncthreads();
    }
  }

  if constexpr (kPipe) {
    if (tid == 0) bulk_wait_all();
  }
  tc_fence_before();
  __syncthreads();
  if (!ok) {
    if (tid == 0) set_status(a.status, FH_ERR_TIMEOUT);
    if (tid == 0) {
      mma_commit(bar);
      mbar_wait(bar, phase, nullptr);
    }
    __syncthreads();
  }
  if (w == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
}

}  // namespace fh

using namespace fh;

extern "C" int fh_rwr_tiles_tc(const fh_tile* tiles, int32_t n_tiles, int32_t n_cells,
                               int32_t mr, int32_t mw, const fh_entry* entries,
                               const int64_t* offsets, uint16_t* out16, int64_t cell_stride,
                               int64_t plane_stride, double* sumsq, int32_t form, int* status,
                               void* stream) {
  if (!tiles || n_tiles <= 0 || n_cells <= 0 || !offsets || !out16 || mr <= 0 || mw < mr ||
      plane_stride < 0 || form < 0 || form > 2)
    return FH_ERR_ARG;
  if (mr > 128 || mw > kRtMaxPad) return FH_ERR_UNSUPPORTED;
  RtArgs a{};
  a.tiles = tiles;
  a.n_tiles = n_tiles;
  a.n_cells = n_cells;
  a.max_rows = mr;
  a.max_width = mw;
  a.npad_max = (mw + 63) & ~63;
  a.entries = reinterpret_cast<const uint2*>(entries);
  a.offsets = offsets;
  a.out16 = reinterpret_cast<__nv_bfloat16*>(out16);
  a.cell_stride = cell_stride;
  a.plane_stride = plane_stride;
  a.sumsq = sumsq;
  a.status = status;
  // form 2: P in tensor memory, epochs pipelined by 64-column blocks, bulk output copies
  const bool pipe = form == 2;
  if (pipe && a.npad_max > kRpMaxPad) return FH_ERR_UNSUPPORTED;
  const void* kern = pipe ? (const void*)rwr_tc_kernel<true> : (const void*)rwr_tc_kernel<false>;
  // at least 120 KB so that one CTA (and one 512-column TMEM allocation) sits on an SM
  size_t smem = rt_smem_bytes(a.npad_max, pipe);
  if (smem < 120 * 1024) smem = 120 * 1024;
  if (smem > 227 * 1024) return FH_ERR_UNSUPPORTED;
  if (ensure_smem(kern, smem)) return FH_ERR_LAUNCH;
  const int sms = sm_count();
  if (sms <= 0) return FH_ERR_LAUNCH;
  const int64_t items = (int64_t)n_tiles * n_cells;
  const int64_t grid = items < sms ? items : sms;
  if (pipe)
    rwr_tc_kernel<true><<<(unsigned)grid, kRtThreads, smem, (cudaStream_t)stream>>>(a);
  else
    rwr_tc_kernel<false><<<(unsigned)grid, kRtThreads, smem, (cudaStream_t)stream>>>(a);
  FH_CHECK_LAUNCH();
  return FH_OK;
}
