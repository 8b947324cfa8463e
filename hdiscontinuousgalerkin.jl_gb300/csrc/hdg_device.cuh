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
// The source as the element kernels read it (CoefDev::fprep): Gaussian bumps carry -1/(2 s^2) in
// place of s, every other kind its plain parameters.
__device__ __forceinline__ double eval_source_prepared(int kind, const double* __restrict__ p, double x, double y) {
  if (kind != HDG_FIELD_BUMPS) return eval_field_kind(kind, p, x, y);
  const int K = (int)p[0];
  double s = 0.0;
  for (int k = 0; k < K; ++k) {
    const double* b = p + 1 + 4 * k;
    const double dx = x - b[0], dy = y - b[1];
    s += b[3] * exp((dx * dx + dy * dy) * b[2]);
  }
  return s;
}

// 1/d by Newton-Raphson iteration from the FP32 approximate reciprocal: each step r <- r + r (1 - d r)
// squares the relative error (about 2^-22 -> 2^-44 -> below 2^-53), so two steps give the FP64
// reciprocal to within an ulp at a fraction of the cost of a correctly rounded FP64 division.
// Outside the FP32 range the FP64 division is used.
__device__ __forceinline__ double recip_newton(double d) {
  const float df = (float)d;
  if (!(fabsf(df) > 1e-30f && fabsf(df) < 1e30f)) return 1.0 / d;
  double r = (double)__fdividef(1.0f, df);
  r = fma(r, fma(-d, r, 1.0), r);
  r = fma(r, fma(-d, r, 1.0), r);
  return r;
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

// ---- reductions with few FP64 instructions ---------------------------------------------------
// GB300 issues FP64 at about 2 lanes per clock per SM, 1/64 of its FP32 rate, so a shuffle tree
// over every warp of a block (5 FP64 adds per warp per value) costs more than the rows it sums.
// The block sums below stage the per-thread values in shared memory and add them with 1 or 2
// warps (8 values per lane in sequence, then one shuffle tree).  Dot products of the FP32
// iteration are accumulated in float-float arithmetic on the FP32 pipe instead (FF).  All sums
// run in a fixed order, so the results are deterministic.  Results are valid in thread 0.

// Float-float accumulator: the pair (hi, lo) holds the sum to about 2^-44 relative.  a*b is split
// exactly with an FMA (Dekker's product, via fmaf) and added with Knuth's TwoSum followed by a
// renormalisation; the _rn intrinsics keep the compiler from contracting or reordering the steps.
struct FF {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add2(float h, float l) {
    const float s = __fadd_rn(hi, h);
    const float bv = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bv)), __fsub_rn(h, bv));
    const float t = __fadd_rn(__fadd_rn(lo, l), err);
    hi = __fadd_rn(s, t);
    lo = __fsub_rn(t, __fsub_rn(hi, s));
  }
  __device__ __forceinline__ void add_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    add2(p, __fmaf_rn(a, b, -p));
  }
  __device__ __forceinline__ double to_double() const { return (double)hi + (double)lo; }
};

// FP64 accumulator with the FF interface.
struct D64 {
  double v = 0.0;
  __device__ __forceinline__ void add_prod(double a, double b) { v = fma(a, b, v); }
  __device__ __forceinline__ double to_double() const { return v; }
};

template <typename T> struct DotAcc;
template <> struct DotAcc<double> { using type = D64; };
template <> struct DotAcc<float> { using type = FF; };

__device__ __forceinline__ FF warp_sum(FF v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float h = __shfl_xor_sync(0xffffffffu, v.hi, o);
    const float l = __shfl_xor_sync(0xffffffffu, v.lo, o);
    v.add2(h, l);
  }
  return v;
}

// Block sums of NV (1 or 2) doubles.
template <int BLOCK, int NV>
__device__ __forceinline__ void block_sum_lean(const double (&v)[NV], double (&out)[NV]) {
  static_assert(BLOCK % 32 == 0 && BLOCK <= 1024 && (NV == 1 || NV == 2), "block shape");
  constexpr int PER = BLOCK / 32;
  __shared__ double red[NV * BLOCK];
#pragma unroll
  for (int i = 0; i < NV; ++i) red[i * BLOCK + threadIdx.x] = v[i];
  __syncthreads();
  if (threadIdx.x < 32 * NV) {
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    const double* src = red + w * BLOCK + l * PER;
    double t = src[0];
#pragma unroll
    for (int k = 1; k < PER; ++k) t += src[k];
    t = warp_sum(t);
    if (l == 0) red[w * BLOCK] = t;  // this warp alone read red[w*BLOCK, (w+1)*BLOCK)
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < NV; ++i) out[i] = red[i * BLOCK];
  __syncthreads();
}

// Block sums of NV float-float values, returned as doubles.
template <int BLOCK, int NV>
__device__ __forceinline__ void block_sum_lean(const FF (&v)[NV], double (&out)[NV]) {
  static_assert(BLOCK % 32 == 0 && BLOCK <= 1024 && (NV == 1 || NV == 2), "block shape");
  __shared__ float2 red[NV][BLOCK / 32];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    const FF t = warp_sum(v[i]);
    if (l == 0) red[i][w] = make_float2(t.hi, t.lo);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      FF s;
      for (int k = 0; k < BLOCK / 32; ++k) s.add2(red[i][k].x, red[i][k].y);
      out[i] = s.to_double();
    }
  }
  __syncthreads();
}

// Cross-block stage: the block's partials (valid in thread 0) go to part[], and the last block of
// the problem adds the problem's partials (each thread its strided share, then a block sum, in a
// fixed order).  Returns true in every thread of that last block; the sums are valid in its
// thread 0.
template <int BLOCK, int NV>
__device__ __forceinline__ bool seg_combine(const SegArgs& g, int P, int slot, const double (&bp)[NV],
                                            double (&sum)[NV]) {
  __shared__ bool last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int i = 0; i < NV; ++i) g.part[2 * blockIdx.x + i] = bp[i];
    __threadfence();
    const unsigned t = atomicAdd(&g.cnt[4 * P + slot], 1u);
    last = (t == (unsigned)g.prob_nblk[P] - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  const int b0 = g.prob_blk0[P], nb = g.prob_nblk[P];
  double s[NV];
#pragma unroll
  for (int i = 0; i < NV; ++i) s[i] = 0.0;
  for (int k = threadIdx.x; k < nb; k += BLOCK)  // every thread loads its strided partials
#pragma unroll
    for (int i = 0; i < NV; ++i) s[i] += ((volatile double*)g.part)[2 * (b0 + k) + i];
  double tot[NV];
  block_sum_lean<BLOCK, NV>(s, tot);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int i = 0; i < NV; ++i) sum[i] = tot[i];
    g.cnt[4 * P + slot] = 0;
  }
  return true;
}

// Per-problem sums of two (seg_finish) or one (seg_finish1) values: block sums, then the
// cross-block stage.  V is double or FF (a D64 accumulator is passed as its double).
template <int BLOCK, typename V>
__device__ __forceinline__ bool seg_finish(const SegArgs& g, int P, int slot, V v0, V v1, double* sum0,
                                           double* sum1) {
  const V v[2] = {v0, v1};
  double bp[2], s[2];
  block_sum_lean<BLOCK, 2>(v, bp);
  if (!seg_combine<BLOCK, 2>(g, P, slot, bp, s)) return false;
  *sum0 = s[0];
  *sum1 = s[1];
  return true;
}
template <int BLOCK>
__device__ __forceinline__ bool seg_finish(const SegArgs& g, int P, int slot, D64 v0, D64 v1, double* sum0,
                                           double* sum1) {
  return seg_finish<BLOCK, double>(g, P, slot, v0.v, v1.v, sum0, sum1);
}
template <int BLOCK, typename V>
__device__ __forceinline__ bool seg_finish1(const SegArgs& g, int P, int slot, V v0, double* sum0) {
  const V v[1] = {v0};
  double bp[1], s[1];
  block_sum_lean<BLOCK, 1>(v, bp);
  if (!seg_combine<BLOCK, 1>(g, P, slot, bp, s)) return false;
  *sum0 = s[0];
  return true;
}
