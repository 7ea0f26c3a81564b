// The column-stochastic transition matrix of the partial RWR (partial_rwr.py:84-111), shared
// by the RWR kernels that run on 256 threads (a 16 x 16 thread grid).
#pragma once
#include "fh_common.cuh"

namespace fh {

constexpr int kRwrThreads = 256;
constexpr float kFloor = 1e-8f;  // densify floor, sparse_for_schic.py:320
constexpr float kEps = 1e-15f;   // column-sum guard, partial_rwr.py:90,91,111

// Row stride of the b x b transition matrix in shared memory.
__host__ __device__ inline int rwr_ldp(int b) { return (b + 3) & ~3; }

// From the densified tile Z (b x n, stride ldz) builds P^T (b x b, stride ldp) in Pt:
//   S2 = Z Z^T with a zero diagonal; S1 = Z[:, s0:s0+b]
//   L  = 0.75 * S1 / colsum(S1) + 0.25 * S2 / colsum(S2);  zero columns get a unit diagonal
//   P  = L / colsum(L)
// cs1, cs2, csl: kMaxBinRows floats each.  Ends with a barrier.
__device__ inline void rwr_transition(const float* Z, int ldz, float* Pt, int ldp, int b, int n,
                                      int s0, float* cs1, float* cs2, float* csl) {
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  // ---- S2 = Z Z^T (b x b), diagonal zeroed (partial_rwr.py:85-87)
  {
    float acc[8][8];
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
      for (int v = 0; v < 8; ++v) acc[u][v] = 0.f;
    const float* zp[8];
    const float* zq[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      zp[u] = Z + min(ty + 16 * u, b - 1) * ldz;
      zq[u] = Z + min(tx + 16 * u, b - 1) * ldz;
    }
    for (int k = 0; k < n; ++k) {
      float ap[8], aq[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) { ap[u] = zp[u][k]; aq[u] = zq[u][k]; }
#pragma unroll
      for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int v = 0; v < 8; ++v) acc[u][v] = fmaf(ap[u], aq[v], acc[u][v]);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
      for (int v = 0; v < 8; ++v) {
        const int p = ty + 16 * u, q = tx + 16 * v;
        if (p < b && q < b) Pt[p * ldp + q] = (p == q) ? 0.f : acc[u][v];
      }
  }
  __syncthreads();

  // ---- column sums of S2 and of the first-order block S1 = Z[:, s0:s0+b]
  if (tid < b) {
    float s = 0.f;
    for (int p = 0; p < b; ++p) s += Pt[p * ldp + tid];
    cs2[tid] = s;
  } else if (tid >= 128 && tid - 128 < b) {
    const int q = tid - 128;
    float s = 0.f;
    for (int p = 0; p < b; ++p) s += Z[p * ldz + s0 + q];
    cs1[q] = s;
  }
  __syncthreads();
  // ---- L = (S1 / (cs1 + eps)) * 0.75 + (S2 / (cs2 + eps)) * 0.25   (partial_rwr.py:90-93)
  for (int i = tid; i < b * b; i += kRwrThreads) {
    const int p = i / b, q = i % b;
    const float l1 = (Z[p * ldz + s0 + q] / (cs1[q] + kEps)) * 0.75f;
    const float l2 = (Pt[p * ldp + q] / (cs2[q] + kEps)) * 0.25f;
    Pt[p * ldp + q] = l1 + l2;
  }
  __syncthreads();
  // ---- zero columns get a unit diagonal (:96-97); P = L / (colsum(L) + eps) (:111)
  if (tid < b) {
    float s = 0.f;
    for (int p = 0; p < b; ++p) s += Pt[p * ldp + tid];
    if (s == 0.f) {
      Pt[tid * ldp + tid] += 1.f;
      s = 0.f;
      for (int p = 0; p < b; ++p) s += Pt[p * ldp + tid];
    }
    csl[tid] = s;
  }
  __syncthreads();
  // P stored transposed in place: Pt[q][p] = P[p][q] = L[p][q] / (csl[q] + eps)
  for (int i = tid; i < b * b; i += kRwrThreads) {
    const int p = i / b, q = i % b;
    if (p < q) {
      const float lpq = Pt[p * ldp + q], lqp = Pt[q * ldp + p];
      Pt[q * ldp + p] = lpq / (csl[q] + kEps);
      Pt[p * ldp + q] = lqp / (csl[p] + kEps);
    } else if (p == q) {
      Pt[p * ldp + p] = Pt[p * ldp + p] / (csl[p] + kEps);
    }
  }
  __syncthreads();
}

// acc[u][v] += sum_k Z[k][ty + 16u] * Pt[k][tx + 16v]  ==  (P Z)[tx+16v][ty+16u]
template <int MAXU>
__device__ __forceinline__ void pz_product(const float* __restrict__ Z, int ldz,
                                           const float* __restrict__ Pt, int ldp, int b,
                                           int ty, int tx, float (&acc)[MAXU][8]) {
#pragma unroll
  for (int u = 0; u < MAXU; ++u)
#pragma unroll
    for (int v = 0; v < 8; ++v) acc[u][v] = 0.f;
  for (int k = 0; k < b; ++k) {
    float zk[MAXU], pk[8];
    const float* zr = Z + k * ldz + ty;
    const float* pr = Pt + k * ldp + tx;
#pragma unroll
    for (int u = 0; u < MAXU; ++u) zk[u] = zr[16 * u];
#pragma unroll
    for (int v = 0; v < 8; ++v) pk[v] = pr[16 * v];
#pragma unroll
    for (int u = 0; u < MAXU; ++u)
#pragma unroll
      for (int v = 0; v < 8; ++v) acc[u][v] = fmaf(zk[u], pk[v], acc[u][v]);
  }
}

}  // namespace fh
