// Device-side helpers shared by the kernels of libhdg.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "hdg_internal.h"

template <int P> struct Dims {
  static constexpr int NW = (P + 1) * (P + 2) / 2;  // scalar Dubiner functions (u)
  static constexpr int NT = P + 1;                  // Legendre functions per edge (trace)
  static constexpr int NV = 2 * NW;                 // vector functions (q)
  static constexpr int N = NV + NW;                 // local (q,u) system size
  static constexpr int M = 3 * NT;                  // trace dofs of a cell
  static constexpr int NC = N + M + 1;              // augmented columns [Me | EF | Bte]
  static constexpr int LD = NC | 1;                 // odd row stride: conflict-free FP64 column reads
};

// Field evaluation: the kinds of hdg.h (HDG_FIELD_*), parameters in device memory.
__device__ __forceinline__ double eval_field_kind(int kind, const double* __restrict__ p, double x, double y) {
  switch (kind) {
    case HDG_FIELD_CONST: return p[0];
    case HDG_FIELD_SINSIN: return p[0] * sinpi(p[1] * x) * sinpi(p[2] * y);
    case HDG_FIELD_BUMPS: {
      int K = (int)p[0];
      double s = 0.0;
      for (int k = 0; k < K; ++k) {
        const double* b = p + 1 + 4 * k;
        double dx = x - b[0], dy = y - b[1];
        s += b[3] * exp(-(dx * dx + dy * dy) / (2.0 * b[2] * b[2]));
      }
      return s;
    }
    case HDG_FIELD_FOURIER:
    case HDG_FIELD_EXP_FOURIER: {
      int K = (int)p[0];
      double g = p[1];
      for (int k = 0; k < K; ++k) {
        const double* b = p + 2 + 4 * k;
        g += b[3] * cos(6.283185307179586 * (b[0] * x + b[1] * y) + b[2]);
      }
      return kind == HDG_FIELD_EXP_FOURIER ? exp(g) : g;
    }
  }
  return 0.0;
}
__device__ __forceinline__ double eval_field_dev(const FieldDev& f, double x, double y) {
  return eval_field_kind(f.kind, f.prm, x, y);
}



__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Deterministic block reduction of one double (all threads get the result).
template <int BLOCK> __device__ __forceinline__ double block_sum(double v, double* sh) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  if (w == 0) {
    t = (l < BLOCK / 32) ? sh[l] : 0.0;
    t = warp_sum(t);
    if (l == 0) sh[0] = t;
  }
  __syncthreads();
  t = sh[0];
  __syncthreads();
  return t;
}

// Segments: every CUDA block of a row-parallel kernel covers rows [row0, row1) of one problem.
// A per-problem sum is formed deterministically: each block writes its partial, and the last
// block of the problem to finish (atomic ticket, no waiting) adds the problem's partials in
// block order.  part holds 2 doubles per block; cnt holds one ticket per (problem, slot).
struct SegArgs {
  const int32_t* seg_prob;
  const int32_t* seg_row0;
  const int32_t* seg_row1;
  const int32_t* prob_blk0;
  const int32_t* prob_nblk;
  double* part;
  unsigned* cnt;  // [nprob][4]
};

template <int BLOCK>
__device__ __forceinline__ bool seg_finish(const SegArgs& g, int P, int slot, double v0, double v1, double* sh,
                                           double* sum0, double* sum1) {
  __shared__ bool last;
  v0 = block_sum<BLOCK>(v0, sh);
  v1 = block_sum<BLOCK>(v1, sh);
  if (threadIdx.x == 0) {
    g.part[2 * blockIdx.x] = v0;
    g.part[2 * blockIdx.x + 1] = v1;
    __threadfence();
    const unsigned t = atomicAdd(&g.cnt[4 * P + slot], 1u);
    last = (t == (unsigned)g.prob_nblk[P] - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  const int b0 = g.prob_blk0[P], nb = g.prob_nblk[P];
  double s0 = 0.0, s1 = 0.0;
  for (int k = threadIdx.x; k < nb; k += BLOCK) {
    s0 += ((volatile double*)g.part)[2 * (b0 + k)];
    s1 += ((volatile double*)g.part)[2 * (b0 + k) + 1];
  }
  *sum0 = block_sum<BLOCK>(s0, sh);
  *sum1 = block_sum<BLOCK>(s1, sh);
  if (threadIdx.x == 0) g.cnt[4 * P + slot] = 0;
  return true;
}
