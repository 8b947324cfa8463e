// Jacobi-preconditioned conjugate gradients on the trace system (stands in for the sparse
// direct `K \ b` of examples/poisson2D_HDG.jl:195), for one or many independent problems.
//
// The matrix is the block-ELL solver form of K (free rows negated, so SPD).  One iteration is
// two kernels:
//   A: q = A p_new, p_new = z + beta p, pq = p_new.q
//   B: alpha = rz/pq;  x += alpha p_new;  r -= alpha q;  z = D^-1 r;  rz, rr
// In FP64, A uses q_{k+1} = A z_{k+1} + beta q_k so that p and q update in place in the same pass.
// Reductions are deterministic per problem (seg_finish in hdg_device.cuh).  Every CUDA block
// belongs to one problem, so many problems share one launch and a converged problem's blocks
// return at once.  CHUNK iterations are captured in a CUDA graph and replayed; the host reads the
// per-problem status between replays, and drives several systems (degree bins of a batch) in one
// loop.
//
// Precision.  FP64: matrix, vectors and scalars in FP64.  Mixed: the Krylov iteration runs on an
// FP32 copy of the matrix with FP32 r, z, p, q, while x, every dot product and every scalar stay
// FP64.  Accuracy is won back by an FP64 refinement that keeps the Krylov space ("reliable
// updates": Sleijpen & van der Vorst 1996; Clark et al. 2010): once a problem's recursive
// residual has dropped by DELTA since its last refinement, its true residual r = b - K x is
// formed in FP64 with the FP64 matrix and replaces the recursive one, and the iteration goes on
// with the same search direction.  Convergence is declared on the true FP64 residual only.  In
// FP32 the product is recomputed every iteration (no q recurrence, whose rounding would
// accumulate), with p alternating between two buffers.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>

#include "hdg_device.cuh"

namespace {
constexpr int CG_BLOCK = 256;
// resident blocks per SM the iteration kernels are compiled for (at least the 4 segments of 1024
// rows per SM that a large problem gets): 6 in FP32 (40 registers), 4 in FP64 (64 registers)
template <typename T> constexpr int cg_min_blocks() { return sizeof(T) == sizeof(float) ? 6 : 4; }
constexpr int SAMPLE_EVERY = 8;  // with profiling on, every 8th chunk runs un-graphed and timed
constexpr int SC = 10;           // per problem: rz, rz_old, pq, rr, bb, tol2, alpha, beta, rr_true, -
constexpr int ST = HDG_CG_ST;    // per problem: status, iterations, maxit, refine flag
constexpr double DELTA = 0.1;    // refine once the recursive residual fell by this factor
// status: 0 running, 1 converged (recursive, FP64), 2 iteration cap, 3 breakdown (p'Ap <= 0),
//         4 converged (true residual, mixed), 5 stopped (mixed: cap or stagnation)
}  // namespace

struct CgState {
  int nprob = 0, nrow = 0;
  DevBuf<double> sc;
  DevBuf<int32_t> st;
  DevBuf<double> r, z, p, q, dinv;
  DevBuf<float> rf, zf, pf, pf2, qf, dinvf, xh, xl;
  DevBuf<float> r32, z32;  // multigrid preconditioner input / output
  cudaGraphExec_t graph64 = nullptr, graph32 = nullptr;
  int chunk64 = 0, chunk32 = 0;
  bool graph_mg = false;  // graph64 holds the multigrid iteration
  int graph_amg_gen = -1; // ... of this multigrid setup (hdg_system::amg_gen)
  int32_t* h_st = nullptr;  // pinned mirrors
  double* h_sc = nullptr;
  std::vector<double> rr_best;
  std::vector<int> stagnant, outer;
  ~CgState() {
    if (graph64) cudaGraphExecDestroy(graph64);
    if (graph32) cudaGraphExecDestroy(graph32);
    if (h_st) cudaFreeHost(h_st);
    if (h_sc) cudaFreeHost(h_sc);
  }
};

void destroy_cg(CgState* c) { delete c; }

namespace {

template <typename T> struct CgArgs {
  SegArgs g;
  const int32_t* bcol5;
  int nf;
  const T* val;
  const double* b;
  const T* dinv;
  double* x;
  T* r;
  T* z;
  T* p;
  T* q;
  T* p2;
  double* sc;
  int32_t* st;
  float* xh;  // FP32 iteration: steps since the last refinement as a float-float pair (hi, lo)
  float* xl;
};

// (A v)_row over the block-ELL layout: 5 block slots, values slot-major and row-contiguous.
template <int NT, typename T, typename V>
__device__ __forceinline__ double row_dot(const int32_t* __restrict__ bcol5, int nf, const T* __restrict__ val, int row,
                                          const V* __restrict__ v) {
  const int f = row / NT;
  const int64_t ndofs = (int64_t)nf * NT;
  int g[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) g[k] = __ldg(bcol5 + k * nf + f);
  T acc = T(0);
#pragma unroll
  for (int k = 0; k < 5; ++k) {
#pragma unroll
    for (int j = 0; j < NT; ++j) acc += __ldg(val + (k * NT + j) * ndofs + row) * (T)__ldg(v + g[k] * NT + j);
  }
  return (double)acc;
}

template <int NT, typename T> __global__ void __launch_bounds__(CG_BLOCK) k_cg_init(CgArgs<T> a) {
  const int P = a.g.seg_prob[blockIdx.x];
  double rz = 0.0, bb = 0.0;
  for (int row = a.g.seg_row0[blockIdx.x] + threadIdx.x; row < a.g.seg_row1[blockIdx.x]; row += CG_BLOCK) {
    const double bv = a.b[row];
    const T rv = (T)bv;
    const T zv = a.dinv[row] * rv;
    a.x[row] = 0.0;
    if (a.xh) {
      a.xh[row] = 0.f;
      a.xl[row] = 0.f;
    }
    a.r[row] = rv;
    a.z[row] = zv;
    a.p[row] = T(0);
    a.p2[row] = T(0);
    a.q[row] = T(0);
    rz += (double)rv * (double)zv;
    bb += bv * bv;
  }
  double s0, s1;
  if (seg_finish<CG_BLOCK>(a.g, P, 0, rz, bb, &s0, &s1) && threadIdx.x == 0) {
    double* sc = a.sc + SC * P;
    sc[0] = s0;
    sc[1] = s0;
    sc[3] = s1;
    sc[4] = s1;
    sc[6] = 0.0;
    sc[7] = 0.0;
    sc[8] = s1;
    a.st[ST * P] = (s1 == 0.0) ? 1 : 0;
    a.st[ST * P + 1] = 0;
  }
}

// FP64 product kernel with the q recurrence (p, q in place)
template <int NT, typename T> __global__ void __launch_bounds__(CG_BLOCK, cg_min_blocks<T>()) k_cg_a(CgArgs<T> a) {
  const int P = a.g.seg_prob[blockIdx.x];
  // status and beta are loaded together (one round trip); beta is formed once by the reducing
  // block of the update kernel
  const int status = a.st[ST * P];
  const double beta = a.sc[SC * P + 7];
  if (status != 0) return;
  const T bt = (T)beta;
  double pq = 0.0;
  const int r0 = a.g.seg_row0[blockIdx.x], r1 = a.g.seg_row1[blockIdx.x];
  // four rows per thread in flight together (independent gathers and accumulation chains)
  constexpr int ROWS = 4;
  for (int base = r0 + threadIdx.x; base < r1; base += ROWS * CG_BLOCK) {
    double w[ROWS];
#pragma unroll
    for (int u = 0; u < ROWS; ++u) {
      const int row = min(base + u * CG_BLOCK, r1 - 1);
      w[u] = row_dot<NT>(a.bcol5, a.nf, a.val, row, a.z);
    }
    T qo[ROWS], po[ROWS], zo[ROWS];
#pragma unroll
    for (int u = 0; u < ROWS; ++u) {
      const int row = min(base + u * CG_BLOCK, r1 - 1);
      qo[u] = a.q[row];
      po[u] = a.p[row];
      zo[u] = a.z[row];
    }
#pragma unroll
    for (int u = 0; u < ROWS; ++u) {
      const int row = base + u * CG_BLOCK;
      if (row < r1) {
        const T qn = (T)(w[u] + beta * (double)qo[u]);
        const T pn = zo[u] + bt * po[u];
        a.q[row] = qn;
        a.p[row] = pn;
        pq += (double)pn * (double)qn;
      }
    }
  }
  double s0;
  if (seg_finish1<CG_BLOCK>(a.g, P, 0, pq, &s0) && threadIdx.x == 0) {
    // alpha = rz / p.q; no step along a direction with p.q <= 0 (the update kernel then stops the
    // problem, and the host restarts it or reports the breakdown)
    a.sc[SC * P + 2] = s0;
    a.sc[SC * P + 6] = (s0 > 0.0) ? a.sc[SC * P] / s0 : 0.0;
  }
}

// Low-precision product kernel: p_new = z + beta p_old formed on the fly for every column the row
// touches, q = A p_new a fresh product; p_old / p_new alternate buffers (flip).  p.q is summed
// in float-float arithmetic (FP32 pipe); only each thread's total is converted to FP64.
template <int NT, typename T> __global__ void __launch_bounds__(CG_BLOCK, cg_min_blocks<T>()) k_cg_a_fresh(CgArgs<T> a, int flip) {
  const int P = a.g.seg_prob[blockIdx.x];
  const int status = a.st[ST * P];
  const T bt = (T)a.sc[SC * P + 7];
  if (status != 0) return;
  const T* __restrict__ pin = flip ? a.p2 : a.p;
  T* __restrict__ pout = flip ? a.p : a.p2;
  const int64_t ndofs = (int64_t)a.nf * NT;
  FF pq;
  for (int row = a.g.seg_row0[blockIdx.x] + threadIdx.x; row < a.g.seg_row1[blockIdx.x]; row += CG_BLOCK) {
    const int f = row / NT;
    T acc = T(0);
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      const int g = __ldg(a.bcol5 + k * a.nf + f);
#pragma unroll
      for (int j = 0; j < NT; ++j) {
        const int c = g * NT + j;
        acc += __ldg(a.val + (k * NT + j) * ndofs + row) * (__ldg(a.z + c) + bt * __ldg(pin + c));
      }
    }
    const T pn = a.z[row] + bt * pin[row];
    pout[row] = pn;
    a.q[row] = acc;
    pq.add_prod((float)pn, (float)acc);
  }
  double s0;
  if (seg_finish1<CG_BLOCK>(a.g, P, 0, pq, &s0) && threadIdx.x == 0) {
    a.sc[SC * P + 2] = s0;
    a.sc[SC * P + 6] = (s0 > 0.0) ? a.sc[SC * P] / s0 : 0.0;
  }
}

// Update kernel.  In FP64 the dot products are FP64 FMAs; in the FP32 iteration they are summed
// in float-float arithmetic (FP32 pipe) and only each thread's totals are converted to FP64.
template <int NT, typename T> __global__ void __launch_bounds__(CG_BLOCK, cg_min_blocks<T>()) k_cg_b(CgArgs<T> a, int flip) {
  const int P = a.g.seg_prob[blockIdx.x];
  const int status = a.st[ST * P];
  const double alpha = a.sc[SC * P + 6];
  if (status != 0) return;
  const T at = (T)alpha;
  const T* __restrict__ pcur = flip ? a.p2 : a.p;  // the direction the product kernel just wrote
  // alpha as a float-float pair for the x update of the FP32 iteration
  const float ah = (float)alpha, al = (float)(alpha - (double)ah);
  typename DotAcc<T>::type rz, rr;
  const int r0 = a.g.seg_row0[blockIdx.x], r1 = a.g.seg_row1[blockIdx.x];
  // the loads of ROWS rows are issued before any store (stores may alias the loads, so the
  // compiler would not hoist the next row's loads above them by itself)
  constexpr int ROWS = 4;
  for (int base = r0 + threadIdx.x; base < r1; base += ROWS * CG_BLOCK) {
    T pv[ROWS], rv[ROWS], qv[ROWS], dv[ROWS];
    double xv[ROWS];
    float xhv[ROWS], xlv[ROWS];
#pragma unroll
    for (int u = 0; u < ROWS; ++u) {
      const int row = min(base + u * CG_BLOCK, r1 - 1);
      pv[u] = pcur[row];
      rv[u] = a.r[row];
      qv[u] = a.q[row];
      dv[u] = a.dinv[row];
      if constexpr (sizeof(T) == sizeof(double)) {
        xv[u] = a.x[row];
      } else {
        xhv[u] = a.xh[row];
        xlv[u] = a.xl[row];
      }
    }
#pragma unroll
    for (int u = 0; u < ROWS; ++u) {
      const int row = base + u * CG_BLOCK;
      if (row < r1) {
        if constexpr (sizeof(T) == sizeof(double)) {
          a.x[row] = xv[u] + alpha * (double)pv[u];
        } else {  // x += alpha p in float-float: exact ah*p, plus al*p, added with TwoSum
          const float ph = __fmul_rn(ah, (float)pv[u]);
          const float pe = __fmaf_rn(al, (float)pv[u], __fmaf_rn(ah, (float)pv[u], -ph));
          FF xx;
          xx.hi = xhv[u];
          xx.lo = xlv[u];
          xx.add2(ph, pe);
          a.xh[row] = xx.hi;
          a.xl[row] = xx.lo;
        }
        const T rn = rv[u] - at * qv[u];
        const T zn = dv[u] * rn;
        a.r[row] = rn;
        a.z[row] = zn;
        rz.add_prod(rn, zn);
        rr.add_prod(rn, rn);
      }
    }
  }
  double s0, s1;
  if (seg_finish<CG_BLOCK>(a.g, P, 1, rz, rr, &s0, &s1) && threadIdx.x == 0) {
    double* sc = a.sc + SC * P;
    const double pq = sc[2], rr_prev = sc[3];
    sc[1] = sc[0];
    sc[0] = s0;
    sc[3] = s1;
    sc[7] = s0 / sc[1];  // beta for the next product kernel
    sc[9] = (double)flip;  // 1: the latest direction is in p2 (FP32 iteration stopped mid-chunk)
    const int it = a.st[ST * P + 1] + 1;
    a.st[ST * P + 1] = it;
    int next = 0;
    if (!(pq > 0.0) || !isfinite(s1)) {
      // p'Ap <= 0 once the residual is at rounding level (tiny problems solved exactly in a few
      // steps) is convergence, not breakdown
      next = (isfinite(s1) && rr_prev <= fmax(1e-24, 100.0 * sc[5]) * sc[4]) ? 1 : 3;
    } else if (s1 <= sc[5] * sc[4]) {
      next = 1;
    } else if (it >= a.st[ST * P + 2]) {
      next = 2;
    }
    a.st[ST * P] = next;
  }
}

// ---- multigrid-preconditioned iteration (FP64 CG, FP32 V-cycle) ---------------------------
// One iteration: k_cg_a (q = A z + beta q, p, alpha) -> k_cg_b_mg (x, r, r32 = r, r.r, status)
// -> V-cycle z32 = M^-1 r32 -> k_cg_c (z = z32, r.z, beta).

// r = b, x = 0, r32 = b, b.b; z follows from the V-cycle and k_cg_c (mode 1).
template <int NT> __global__ void __launch_bounds__(CG_BLOCK) k_cg_init_mg(CgArgs<double> a, float* r32) {
  const int P = a.g.seg_prob[blockIdx.x];
  double bb = 0.0;
  for (int row = a.g.seg_row0[blockIdx.x] + threadIdx.x; row < a.g.seg_row1[blockIdx.x]; row += CG_BLOCK) {
    const double bv = a.b[row];
    a.x[row] = 0.0;
    a.r[row] = bv;
    r32[row] = (float)bv;
    a.p[row] = 0.0;
    a.q[row] = 0.0;
    bb += bv * bv;
  }
  double s0;
  if (seg_finish1<CG_BLOCK>(a.g, P, 0, bb, &s0) && threadIdx.x == 0) {
    double* sc = a.sc + SC * P;
    sc[3] = s0;
    sc[4] = s0;
    sc[6] = 0.0;
    sc[7] = 0.0;
    sc[8] = s0;
    a.st[ST * P] = (s0 == 0.0) ? 1 : 0;
    a.st[ST * P + 1] = 0;
  }
}

// x += alpha p, r -= alpha q, r32 = r, r.r; convergence and breakdown decisions.
template <int NT> __global__ void __launch_bounds__(CG_BLOCK, 4) k_cg_b_mg(CgArgs<double> a, float* r32) {
  const int P = a.g.seg_prob[blockIdx.x];
  const int status = a.st[ST * P];
  const double alpha = a.sc[SC * P + 6];
  if (status != 0) return;
  double rr = 0.0;
  const int r0 = a.g.seg_row0[blockIdx.x], r1 = a.g.seg_row1[blockIdx.x];
  constexpr int ROWS = 4;
  for (int base = r0 + threadIdx.x; base < r1; base += ROWS * CG_BLOCK) {
    double xv[ROWS], pv[ROWS], rv[ROWS], qv[ROWS];
#pragma unroll
    for (int u = 0; u < ROWS; ++u) {
      const int row = min(base + u * CG_BLOCK, r1 - 1);
      xv[u] = a.x[row];
      pv[u] = a.p[row];
      rv[u] = a.r[row];
      qv[u] = a.q[row];
    }
#pragma unroll
    for (int u = 0; u < ROWS; ++u) {
      const int row = base + u * CG_BLOCK;
      if (row < r1) {
        a.x[row] = xv[u] + alpha * pv[u];
        const double rn = rv[u] - alpha * qv[u];
        a.r[row] = rn;
        r32[row] = (float)rn;
        rr = fma(rn, rn, rr);
      }
    }
  }
  double s0;
  if (seg_finish1<CG_BLOCK>(a.g, P, 1, rr, &s0) && threadIdx.x == 0) {
    double* sc = a.sc + SC * P;
    const double pq = sc[2], rr_prev = sc[3];
    sc[3] = s0;
    const int it = a.st[ST * P + 1] + 1;
    a.st[ST * P + 1] = it;
    int next = 0;
    if (!(pq > 0.0) || !isfinite(s0)) {
      next = (isfinite(s0) && rr_prev <= fmax(1e-24, 100.0 * sc[5]) * sc[4]) ? 1 : 3;
    } else if (s0 <= sc[5] * sc[4]) {
      next = 1;
    } else if (it >= a.st[ST * P + 2]) {
      next = 2;
    }
    a.st[ST * P] = next;
  }
}

// z = z32 (FP64), r.z and beta.  mode 0: a regular iteration of the running problems (beta =
// rz / rz_old); mode 1: a (re)start of the running problems (init) or of the problems whose
// refine flag is set (restart), beta = 0.
template <int NT> __global__ void __launch_bounds__(CG_BLOCK) k_cg_c(CgArgs<double> a, const float* z32, int mode,
                                                                      int restart) {
  const int P = a.g.seg_prob[blockIdx.x];
  const int status = a.st[ST * P];
  const int flag = a.st[ST * P + 3];
  if (restart ? (flag == 0) : (status != 0)) return;
  double rz = 0.0;
  for (int row = a.g.seg_row0[blockIdx.x] + threadIdx.x; row < a.g.seg_row1[blockIdx.x]; row += CG_BLOCK) {
    const double zv = (double)z32[row];
    a.z[row] = zv;
    rz = fma(a.r[row], zv, rz);
  }
  double s0;
  if (seg_finish1<CG_BLOCK>(a.g, P, 2, rz, &s0) && threadIdx.x == 0) {
    double* sc = a.sc + SC * P;
    if (mode == 0) {
      sc[1] = sc[0];
      sc[0] = s0;
      sc[7] = s0 / sc[1];
    } else {
      sc[0] = s0;
      sc[1] = s0;
      sc[7] = 0.0;
    }
  }
}

// True residual r = b - K x in FP64 (FP64 matrix) for the problems whose refine flag is set;
// with `replace` it also replaces the Krylov residual: r = r_true, z = D^-1 r, rz and beta.
// The search direction is kept (beta = rz_true / rz_old) unless the refine flag is 2 or the
// true residual norm exceeds twice the recursive one, which then restarts the iteration (beta
// 0, p = z).  In the FP32 iteration the latest direction is moved into p if it sits in p2, and
// the next refinement is set to trigger once the recursive residual fell by DELTA.
// With the multigrid preconditioner (r32 != NULL) the replacement writes r and its FP32 copy
// only; the V-cycle and k_cg_c (restart) then form z, r.z and beta = 0.
template <int NT, typename T>
__global__ void __launch_bounds__(CG_BLOCK) k_cg_residual(CgArgs<T> a, const double* __restrict__ val64, int replace,
                                                          float* r32) {
  const int P = a.g.seg_prob[blockIdx.x];
  if (a.st[ST * P + 3] == 0) return;
  const bool move_p = replace && a.p2 != a.p && a.sc[SC * P + 9] != 0.0;
  double rz = 0.0, rr = 0.0;
  for (int row = a.g.seg_row0[blockIdx.x] + threadIdx.x; row < a.g.seg_row1[blockIdx.x]; row += CG_BLOCK) {
    const double rv = a.b[row] - row_dot<NT>(a.bcol5, a.nf, val64, row, a.x);
    rr += rv * rv;
    if (replace && r32) {
      a.r[row] = (T)rv;
      r32[row] = (float)rv;
    } else if (replace) {
      const T rt = (T)rv;
      const T zt = a.dinv[row] * rt;
      a.r[row] = rt;
      a.z[row] = zt;
      rz += (double)rt * (double)zt;
      if (move_p) a.p[row] = a.p2[row];
    }
  }
  double s0, s1;
  if (seg_finish<CG_BLOCK>(a.g, P, 2, rz, rr, &s0, &s1) && threadIdx.x == 0) {
    double* sc = a.sc + SC * P;
    sc[8] = s1;
    if (replace && r32) {
      sc[3] = s1;
    } else if (replace) {
      const bool restart = a.st[ST * P + 1] == 0 || a.st[ST * P + 3] == 2 || s1 > 4.0 * sc[3];
      sc[0] = s0;
      sc[3] = s1;
      sc[7] = restart ? 0.0 : s0 / sc[1];
      sc[9] = 0.0;
      if (a.p2 != a.p) sc[5] = DELTA * DELTA * s1 / sc[4];
    }
  }
}

// FP32 iteration: x = x64 + (xh + xl), where the float-float pair holds the steps taken since the
// last refinement.  Folding adds the pair to the FP64 x and clears it, so the pair only ever holds
// a correction; its 2^-44 relative precision then limits the correction, not x itself.
__global__ void k_x_fold(int64_t n, float* __restrict__ xh, float* __restrict__ xl, double* __restrict__ x) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    x[t] += (double)xh[t] + (double)xl[t];
    xh[t] = 0.f;
    xl[t] = 0.f;
  }
}

template <int NT, typename T>
__global__ void k_dinv(int nrow, const int8_t* kdiag, const double* val, T* dinv) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nrow) return;
  const int f = t / NT, i = t - f * NT;
  const double d = val[(int64_t)(kdiag[f] * NT + i) * nrow + t];
  dinv[t] = (T)(1.0 / d);
}

__global__ void k_to_float(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    b[t] = (float)a[t];
}

// ------------------------------------------------------------------ per-system solver (CgSolver)
template <int NT> struct SolverNT : CgSolver {
  CgState* c;
  cudaStream_t st;
  int nrow, nprob, chunk = 32;
  bool mixed = false;
  bool mg = false;  // multigrid preconditioner (FP64 iteration)
  CgArgs<double> a64;
  CgArgs<float> a32;
  // Segment compaction: once most problems have finished, the launch grid is rebuilt from the
  // segments of the problems still running, so the tail of a batch does not pay for blocks that
  // would only return.  The full tables are restored when the solve ends.
  std::vector<int32_t> full_prob, full_r0, full_r1, full_b0, full_nb;
  int nseg_full = 0;
  // Byte accounting of sampled chunks: iteration counts at the launch of the sampled chunk; and of
  // every chunk: iteration counts at the previous read-back.
  std::vector<int32_t> sample_it0, it_prev;
  bool sample_pending = false;

  explicit SolverNT(hdg_system* s_) {
    s = s_;
    if (!s->cg) s->cg = new CgState();
    c = s->cg;
    st = s->ctx->stream;
    nrow = s->ndofs;
    nprob = s->nprob;
  }

  void set_stream(cudaStream_t stream) override { st = stream; }

  SegArgs seg() const {
    return SegArgs{s->d_seg_prob.p, s->d_seg_row0.p, s->d_seg_row1.p, s->d_prob_blk0.p, s->d_prob_nblk.p,
                   s->d_part.p, s->d_cnt.p};
  }

  template <typename T> void launch_pair(const CgArgs<T>& a, cudaStream_t stream, int it) {
    if constexpr (sizeof(T) == sizeof(double)) {
      k_cg_a<NT, T><<<s->nseg, CG_BLOCK, 0, stream>>>(a);
      if (mg) {
        k_cg_b_mg<NT><<<s->nseg, CG_BLOCK, 0, stream>>>(a, c->r32.p);
        amg_apply(s, c->r32.p, c->z32.p, c->st.p, stream);
        k_cg_c<NT><<<s->nseg, CG_BLOCK, 0, stream>>>(a, c->z32.p, 0, 0);
      } else {
        k_cg_b<NT, T><<<s->nseg, CG_BLOCK, 0, stream>>>(a, 0);
      }
    } else {
      k_cg_a_fresh<NT, T><<<s->nseg, CG_BLOCK, 0, stream>>>(a, it & 1);
      k_cg_b<NT, T><<<s->nseg, CG_BLOCK, 0, stream>>>(a, (it & 1) ^ 1);
    }
  }

  template <typename T> void build_graph(const CgArgs<T>& a, cudaGraphExec_t* graph, int* graph_chunk) {
    if (*graph && *graph_chunk == chunk) return;
    if (*graph) cudaGraphExecDestroy(*graph);
    cudaStream_t cap;
    HDG_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaGraph_t g;
    HDG_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
    for (int it = 0; it < chunk; ++it) launch_pair<T>(a, cap, it);
    HDG_CUDA(cudaStreamEndCapture(cap, &g));
    HDG_CUDA(cudaGraphInstantiate(graph, g, 0));
    cudaGraphDestroy(g);
    cudaStreamDestroy(cap);
    *graph_chunk = chunk;
  }

  void prepare(const hdg_solver& o) override {
    mg = (o.preconditioner == HDG_PRECOND_AMG);
    // The multigrid iteration runs in FP64.  An FP32 multigrid iteration with FP64 reliable
    // updates was built and measured: on the high-contrast batch it needed up to 1.5x the
    // iterations (474 -> 726) and lost 25 % overall, and it did not reach 1e-12 on a
    // 131072-cell p=2 problem.
    mixed = (o.precision == HDG_PREC_MIXED) && !mg;
    chunk = o.chunk > 1 ? (o.chunk + 1) / 2 * 2 : 2;  // even: the FP32 iteration alternates p buffers
    if (mg) chunk = std::min(chunk, 8);  // a multigrid iteration is ~25 launches
    if (c->nprob != nprob || c->nrow != nrow) {
      c->sc.alloc((size_t)SC * nprob);
      c->st.alloc((size_t)ST * nprob);
      if (c->h_st) cudaFreeHost(c->h_st);
      if (c->h_sc) cudaFreeHost(c->h_sc);
      HDG_CUDA(cudaMallocHost(&c->h_st, sizeof(int32_t) * ST * nprob));
      HDG_CUDA(cudaMallocHost(&c->h_sc, sizeof(double) * SC * nprob));
      c->nprob = nprob;
      c->nrow = nrow;
      if (c->graph64) { cudaGraphExecDestroy(c->graph64); c->graph64 = nullptr; }
      if (c->graph32) { cudaGraphExecDestroy(c->graph32); c->graph32 = nullptr; }
    }
    s->ensure_reduction_buffers();
    s->d_x.alloc(nrow);
    nseg_full = s->nseg;  // full tables (a solve restores them when it ends)
    full_prob = s->h_seg_prob;
    full_r0 = s->h_seg_row0;
    full_r1 = s->h_seg_row1;
    full_b0 = s->h_prob_blk0;
    full_nb = s->h_prob_nblk;
    for (auto* e : s->ev_cg_a) delete e;
    for (auto* e : s->ev_cg_b) delete e;
    s->ev_cg_a.clear();
    s->ev_cg_b.clear();
    s->prof_a_bytes = s->prof_b_bytes = s->prof_all_bytes = 0.0;
    for (auto* e : s->ev_cheb0) delete e;
    s->ev_cheb0.clear();
    s->prof_cheb0_bytes = 0.0;
    for (auto* e : s->ev_l1) delete e;
    s->ev_l1.clear();
    s->prof_l1_bytes = 0.0;
    sample_pending = false;
    it_prev.assign(nprob, 0);
    if (s->ctx->profiling) s->ev_cg.start(st);
    // per-problem tolerance (mixed: the recursive residual only triggers a refinement) and cap
    for (int P = 0; P < nprob; ++P) {
      std::memset(c->h_sc + SC * P, 0, sizeof(double) * SC);
      c->h_sc[SC * P + 5] = mixed ? DELTA * DELTA : o.tol * o.tol;  // mixed: first refinement trigger
      c->h_st[ST * P + 0] = 0;
      c->h_st[ST * P + 1] = 0;
      c->h_st[ST * P + 2] = o.maxit;
      c->h_st[ST * P + 3] = 0;
    }
    HDG_CUDA(cudaMemcpyAsync(c->sc.p, c->h_sc, sizeof(double) * SC * nprob, cudaMemcpyHostToDevice, st));
    HDG_CUDA(cudaMemcpyAsync(c->st.p, c->h_st, sizeof(int32_t) * ST * nprob, cudaMemcpyHostToDevice, st));
    if (mg) {
      c->r.alloc(nrow); c->z.alloc(nrow); c->p.alloc(nrow); c->q.alloc(nrow); c->dinv.alloc(nrow);
      c->r32.alloc(nrow); c->z32.alloc(nrow);
      if (!s->amg) amg_setup_symbolic(s, s->h_dir_face);
      amg_setup_numeric(s, st);
      a64 = CgArgs<double>{seg(), s->d_bcol5.p, s->nf, s->d_val.p, s->d_b.p, c->dinv.p, s->d_x.p, c->r.p, c->z.p,
                           c->p.p, c->q.p, c->p.p, c->sc.p, c->st.p, nullptr, nullptr};
      k_cg_init_mg<NT><<<s->nseg, CG_BLOCK, 0, st>>>(a64, c->r32.p);
      amg_apply(s, c->r32.p, c->z32.p, c->st.p, st);
      k_cg_c<NT><<<s->nseg, CG_BLOCK, 0, st>>>(a64, c->z32.p, 1, 0);
      // the graph holds the hierarchy's buffers: rebuilt after a Jacobi solve or a new setup
      if (c->graph64 && (!c->graph_mg || c->graph_amg_gen != s->amg_gen)) {
        cudaGraphExecDestroy(c->graph64);
        c->graph64 = nullptr;
      }
      build_graph<double>(a64, &c->graph64, &c->chunk64);
      c->graph_mg = true;
      c->graph_amg_gen = s->amg_gen;
    } else if (!mixed) {
      c->r.alloc(nrow); c->z.alloc(nrow); c->p.alloc(nrow); c->q.alloc(nrow); c->dinv.alloc(nrow);
      k_dinv<NT, double><<<(nrow + 255) / 256, 256, 0, st>>>(nrow, s->d_kdiag.p, s->d_val.p, c->dinv.p);
      a64 = CgArgs<double>{seg(), s->d_bcol5.p, s->nf, s->d_val.p, s->d_b.p, c->dinv.p, s->d_x.p, c->r.p, c->z.p,
                           c->p.p, c->q.p, c->p.p, c->sc.p, c->st.p, nullptr, nullptr};
      k_cg_init<NT, double><<<s->nseg, CG_BLOCK, 0, st>>>(a64);
      if (c->graph_mg && c->graph64) { cudaGraphExecDestroy(c->graph64); c->graph64 = nullptr; }
      c->graph_mg = false;
      build_graph<double>(a64, &c->graph64, &c->chunk64);
    } else {
      const int64_t nval = (int64_t)hdg_system::SLOTS * NT * nrow;
      s->d_valf.alloc((size_t)nval);
      k_to_float<<<(unsigned)std::min<int64_t>((nval + 255) / 256, 152 * 32), 256, 0, st>>>(nval, s->d_val.p,
                                                                                           s->d_valf.p);
      c->rf.alloc(nrow); c->zf.alloc(nrow); c->pf.alloc(nrow); c->pf2.alloc(nrow); c->qf.alloc(nrow);
      c->dinvf.alloc(nrow); c->xh.alloc(nrow); c->xl.alloc(nrow);
      k_dinv<NT, float><<<(nrow + 255) / 256, 256, 0, st>>>(nrow, s->d_kdiag.p, s->d_val.p, c->dinvf.p);
      a32 = CgArgs<float>{seg(), s->d_bcol5.p, s->nf, s->d_valf.p, s->d_b.p, c->dinvf.p, s->d_x.p, c->rf.p, c->zf.p,
                          c->pf.p, c->qf.p, c->pf2.p, c->sc.p, c->st.p, c->xh.p, c->xl.p};
      k_cg_init<NT, float><<<s->nseg, CG_BLOCK, 0, st>>>(a32);
      build_graph<float>(a32, &c->graph32, &c->chunk32);
      s->ctx->launches++;
    }
    HDG_CUDA(cudaGetLastError());
    s->ctx->launches += 2;
    c->rr_best.assign(nprob, 0.0);
    c->stagnant.assign(nprob, 0);
    c->outer.assign(nprob, 0);
  }

  template <typename T> void chunk_t(const CgArgs<T>& a, cudaGraphExec_t graph, int rep) {
    if (s->ctx->profiling && rep % SAMPLE_EVERY == SAMPLE_EVERY - 1) {
      sample_it0.resize(nprob);
      for (int P = 0; P < nprob; ++P) sample_it0[P] = c->h_st[ST * P + 1];
      sample_pending = true;
      for (int it = 0; it < chunk; ++it) {
        EventPair* ea = new EventPair();
        EventPair* eb = new EventPair();
        ea->start(st);
        if constexpr (sizeof(T) == sizeof(double)) k_cg_a<NT, T><<<s->nseg, CG_BLOCK, 0, st>>>(a);
        else k_cg_a_fresh<NT, T><<<s->nseg, CG_BLOCK, 0, st>>>(a, it & 1);
        ea->stop(st);
        eb->start(st);
        if constexpr (sizeof(T) == sizeof(double)) {
          if (mg) {  // the update, the V-cycle and the r.z kernel are timed together
            k_cg_b_mg<NT><<<s->nseg, CG_BLOCK, 0, st>>>(a, c->r32.p);
            s->prof_cheb0 = true;  // and each level-0 smoother sweep on its own
            amg_apply(s, c->r32.p, c->z32.p, c->st.p, st);
            s->prof_cheb0 = false;
            k_cg_c<NT><<<s->nseg, CG_BLOCK, 0, st>>>(a, c->z32.p, 0, 0);
          } else {
            k_cg_b<NT, T><<<s->nseg, CG_BLOCK, 0, st>>>(a, 0);
          }
        } else {
          k_cg_b<NT, T><<<s->nseg, CG_BLOCK, 0, st>>>(a, (it & 1) ^ 1);
        }
        eb->stop(st);
        s->ev_cg_a.push_back(ea);
        s->ev_cg_b.push_back(eb);
      }
      HDG_CUDA(cudaGetLastError());
    } else {
      HDG_CUDA(cudaGraphLaunch(graph, st));
    }
    s->ctx->launches += (int64_t)chunk * (mg ? 3 + amg_cycle_launches(s) : 2);
  }

  void launch_chunk(int rep) override {
    if (mixed) chunk_t<float>(a32, c->graph32, rep);
    else chunk_t<double>(a64, c->graph64, rep);
  }

  void enqueue_status_copy() override {
    HDG_CUDA(cudaMemcpyAsync(c->h_st, c->st.p, sizeof(int32_t) * ST * nprob, cudaMemcpyDeviceToHost, st));
    HDG_CUDA(cudaMemcpyAsync(c->h_sc, c->sc.p, sizeof(double) * SC * nprob, cudaMemcpyDeviceToHost, st));
  }

  // true residuals of the flagged problems (and replacement of their Krylov residual)
  // FP64 x: fold the float-float steps of the FP32 iteration into it
  void x_to_double() {
    k_x_fold<<<(unsigned)std::min<int64_t>((nrow + 255) / 256, 152 * 16), 256, 0, st>>>(nrow, c->xh.p, c->xl.p,
                                                                                        s->d_x.p);
    HDG_CUDA(cudaGetLastError());
    s->ctx->launches++;
  }

  void residual(bool replace, bool sync = true) {
    HDG_CUDA(cudaMemcpyAsync(c->st.p, c->h_st, sizeof(int32_t) * ST * nprob, cudaMemcpyHostToDevice, st));
    if (mixed) x_to_double();
    if (mixed) k_cg_residual<NT, float><<<s->nseg, CG_BLOCK, 0, st>>>(a32, s->d_val.p, replace ? 1 : 0, nullptr);
    else k_cg_residual<NT, double><<<s->nseg, CG_BLOCK, 0, st>>>(a64, s->d_val.p, replace ? 1 : 0,
                                                                 mg ? c->r32.p : nullptr);
    HDG_CUDA(cudaGetLastError());
    s->ctx->launches++;
    if (mg && replace) {  // z for the replaced residuals, and a restart (beta = 0) of those problems
      amg_apply(s, c->r32.p, c->z32.p, c->st.p, st);
      k_cg_c<NT><<<s->nseg, CG_BLOCK, 0, st>>>(a64, c->z32.p, 1, 1);
      HDG_CUDA(cudaGetLastError());
      s->ctx->launches++;
    }
    HDG_CUDA(cudaMemcpyAsync(c->h_sc, c->sc.p, sizeof(double) * SC * nprob, cudaMemcpyDeviceToHost, st));
    if (sync) HDG_CUDA(cudaStreamSynchronize(st));
  }

  // Rebuilds the segment tables from the running problems (all = restore the full tables).
  void set_segments(bool all) {
    std::vector<int32_t> sp, r0, r1, b0(full_b0), nb(full_nb);
    for (int P = 0; P < nprob; ++P) {
      if (!all && c->h_st[ST * P] != 0) continue;
      b0[P] = (int32_t)sp.size();
      for (int k = full_b0[P]; k < full_b0[P] + full_nb[P]; ++k) {
        sp.push_back(full_prob[k]);
        r0.push_back(full_r0[k]);
        r1.push_back(full_r1[k]);
      }
    }
    if (sp.empty()) return;
    const int n = (int)sp.size();
    HDG_CUDA(cudaMemcpyAsync(s->d_seg_prob.p, sp.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    HDG_CUDA(cudaMemcpyAsync(s->d_seg_row0.p, r0.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    HDG_CUDA(cudaMemcpyAsync(s->d_seg_row1.p, r1.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    HDG_CUDA(cudaMemcpyAsync(s->d_prob_blk0.p, b0.data(), nprob * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    HDG_CUDA(cudaStreamSynchronize(st));  // host staging vectors go out of scope
    if (n != s->nseg) {
      s->nseg = n;
      if (mixed) { c->chunk32 = 0; build_graph<float>(a32, &c->graph32, &c->chunk32); }
      else { c->chunk64 = 0; build_graph<double>(a64, &c->graph64, &c->chunk64); }
    }
  }

  void maybe_compact() {
    int active = 0;
    for (int P = 0; P < nprob; ++P)
      if (c->h_st[ST * P] == 0) active += full_nb[P];
    if (active > 0 && s->nseg >= 16 && 2 * active <= s->nseg) set_segments(false);
  }

  // Algorithmic bytes per row of the two iteration kernels: the matrix row (5 blocks of NT values),
  // the block columns (5 per face), and each vector element read or written once; gathered
  // neighbour values are counted once, at their own row.
  double bytes_per_row_a() const { return mixed ? 20.0 * NT + 20.0 / NT + 16.0 : 40.0 * NT + 20.0 / NT + 40.0; }
  // the multigrid "update" is k_cg_b_mg (x, p, r r/w, q, r32) + the V-cycle + k_cg_c (z32, z, r)
  double bytes_per_row_b() const {
    if (mg) return 52.0 + 20.0 + amg_cycle_bytes(s) / (double)nrow;
    return mixed ? 40.0 : 64.0;
  }

  void account_sample() {
    // all launches: rows x iterations since the previous read-back
    if ((int)it_prev.size() != nprob) it_prev.assign(nprob, 0);
    double rows_all = 0.0;
    for (int P = 0; P < nprob; ++P) {
      const int32_t now = c->h_st[ST * P + 1];
      rows_all += (double)(now - it_prev[P]) * (double)(s->h_prob_row0[P + 1] - s->h_prob_row0[P]);
      it_prev[P] = now;
    }
    s->prof_all_bytes += rows_all * (bytes_per_row_a() + bytes_per_row_b());
    if (!sample_pending) return;
    sample_pending = false;
    double rows_it = 0.0;
    for (int P = 0; P < nprob; ++P) {
      const double d = (double)(c->h_st[ST * P + 1] - sample_it0[P]);
      rows_it += d * (double)(s->h_prob_row0[P + 1] - s->h_prob_row0[P]);
    }
    s->prof_a_bytes += rows_it * bytes_per_row_a();
    s->prof_b_bytes += rows_it * bytes_per_row_b();
    if (mg) {
      s->prof_cheb0_bytes += rows_it * amg_cheb0_bytes_per_row(s);
      s->prof_l1_bytes += rows_it * amg_l1sweep_bytes_per_row(s);
    }
  }

  bool process(const hdg_solver& o) override {
    account_sample();
    bool done = process_impl(o);
    if (!done) maybe_compact();
    return done;
  }

  // Host step between chunks.  A problem stopped by p.q <= 0 (status 3) with a finite residual is
  // restarted from its true FP64 residual with p = z (refine flag 2), in both precisions.  In the
  // mixed precision the update kernel also stops a problem once its recursive residual fell by
  // DELTA since the last refinement (status 1); it is then refined here (flag 1).  Refining that
  // early keeps the recursive and true residuals close, so the search direction stays valid.
  // Convergence is declared on the true residual; five refinements in a row that do not reduce
  // it 4x stop the problem.
  bool process_impl(const hdg_solver& o) {
    bool any = false, running = false;
    for (int P = 0; P < nprob; ++P) {
      int32_t* stp = c->h_st + ST * P;
      const double* scp = c->h_sc + SC * P;
      if (c->rr_best[P] == 0.0) c->rr_best[P] = scp[4];
      stp[3] = 0;
      if (stp[0] == 3) {
        if (std::isfinite(scp[3])) {
          stp[3] = 2;
          any = true;
        }
        continue;
      }
      if (!mixed) {
        if (stp[0] == 0) running = true;
        continue;
      }
      if (stp[0] >= 4) continue;  // final
      if (stp[0] != 0) {
        stp[3] = 1;
        any = true;
      } else {
        running = true;
      }
    }
    if (!any) return !running;
    residual(true);
    const double tol2 = o.tol * o.tol;
    for (int P = 0; P < nprob; ++P) {
      int32_t* stp = c->h_st + ST * P;
      if (!stp[3]) continue;
      const double* scp = c->h_sc + SC * P;
      const double rr = scp[8], bb = scp[4];
      c->outer[P]++;
      if (rr <= tol2 * bb) { stp[0] = mixed ? 4 : 1; continue; }  // converged on the true residual
      if (stp[0] == 2) { stp[0] = mixed ? 5 : 2; continue; }      // iteration cap reached
      c->stagnant[P] = (rr > 0.25 * c->rr_best[P]) ? c->stagnant[P] + 1 : 0;
      c->rr_best[P] = std::min(c->rr_best[P], rr);
      if (c->stagnant[P] >= 5 || !std::isfinite(rr)) {
        stp[0] = mixed ? 5 : 3;  // the FP32 operator limits the residual / repeated breakdown
        continue;
      }
      stp[0] = 0;
      running = true;
    }
    for (int P = 0; P < nprob; ++P) c->h_st[ST * P + 3] = 0;
    HDG_CUDA(cudaMemcpyAsync(c->st.p, c->h_st, sizeof(int32_t) * ST * nprob, cudaMemcpyHostToDevice, st));
    return !running;
  }

  void finish(const hdg_solver& o, std::vector<hdg_stats>* out) override {
    (void)o;
    finish_enqueue();
    HDG_CUDA(cudaStreamSynchronize(st));
    finish_collect(out);
  }

  void finish_enqueue() override {
    if (s->nseg != nseg_full) set_segments(true);  // restore the full tables (other kernels use them)
    if (mixed) x_to_double();
    if (!mixed) {  // report the true FP64 residual of every problem
      for (int P = 0; P < nprob; ++P) c->h_st[ST * P + 3] = 1;
      residual(false, false);
    }
    if (s->ctx->profiling) s->ev_cg.stop(st);
  }

  // After the work finish_enqueue queued has landed.  The refine flags it raised on the host are
  // cleared here; the device copy is rewritten by the next prepare().
  void finish_collect(std::vector<hdg_stats>* out) override {
    if (!mixed)
      for (int P = 0; P < nprob; ++P) c->h_st[ST * P + 3] = 0;
    out->assign(nprob, hdg_stats{});
    int itmax = 0;
    for (int P = 0; P < nprob; ++P) {
      const int status = c->h_st[ST * P];
      hdg_stats& r = (*out)[P];
      r.iterations = c->h_st[ST * P + 1];
      r.outer = mixed ? c->outer[P] : 1 + c->outer[P];  // FP64: 1 + restarts
      const double bb = c->h_sc[SC * P + 4];
      r.rel_residual = bb > 0 ? std::sqrt(c->h_sc[SC * P + 8] / bb) : 0.0;
      r.converged = mixed ? (status == 4) : (status == 1);
      if (status == 3) r.converged = -1;  // breakdown marker, mapped to an error by the caller
      itmax = std::max(itmax, r.iterations);
    }
    s->cg_iterations = itmax;
  }
};

}  // namespace

CgSolver* make_cg_solver(hdg_system* s) {
  switch (s->nt) {
    case 2: return new SolverNT<2>(s);
    case 3: return new SolverNT<3>(s);
    case 4: return new SolverNT<4>(s);
    case 5: return new SolverNT<5>(s);
  }
  throw HdgError{HDG_ERR_ARG, "degree not supported"};
}

int run_batch_step(const std::vector<hdg_system*>& sys, const hdg_solver& o, int flags,
                   std::vector<std::vector<hdg_stats>>* stats) {
  std::vector<CgSolver*> sv;
  struct Guard {
    std::vector<CgSolver*>& v;
    ~Guard() {
      for (auto* p : v) delete p;
    }
  } guard{sv};
  for (auto* s : sys) sv.push_back(make_cg_solver(s));
  // The multigrid's symbolic setup is host work (and synchronises): done for every system before
  // any of them is queued, so that it never stalls the pipeline.  It runs once per system.
  if (o.preconditioner == HDG_PRECOND_AMG)
    for (auto* s : sys)
      if (!s->amg) amg_setup_symbolic(s, s->h_dir_face);
  // Several systems (degree bins) run on streams of their own, forked from and joined back to
  // the context's stream: one system's assembly, reduction tails, chunk boundaries and recovery
  // overlap the other systems' iterations.
  struct Fork {
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> events;
    cudaStream_t home = nullptr;
    ~Fork() {
      for (size_t i = 0; i < streams.size(); ++i) {
        cudaEventRecord(events[i], streams[i]);
        cudaStreamWaitEvent(home, events[i], 0);
      }
      for (auto e : events) cudaEventDestroy(e);
      for (auto q : streams) cudaStreamDestroy(q);
    }
  } fork;
  const size_t ns = sv.size();
  std::vector<cudaStream_t> q(ns, sys[0]->ctx->stream);
  if (ns > 1) {
    fork.home = sys[0]->ctx->stream;
    cudaEvent_t start;
    HDG_CUDA(cudaEventCreateWithFlags(&start, cudaEventDisableTiming));
    for (auto* s : sys)
      if (s->ctx->stream != fork.home) {
        HDG_CUDA(cudaEventRecord(start, s->ctx->stream));
        HDG_CUDA(cudaStreamWaitEvent(fork.home, start, 0));
      }
    HDG_CUDA(cudaEventRecord(start, fork.home));
    // One system gets the greatest stream priority: the one on the longest chain of dependent
    // launches.  When the systems have been solved before (a batch stepped again with new data),
    // that is the one whose hardest problem took the most CG iterations; otherwise the one with
    // the most element work (the FP64-bound condensation of the highest degree), whose element
    // kernel would otherwise be starved of SM slots by the other systems' iteration kernels.
    // Measured on the 256-problem batch: 490 solves/s with the element-work rule alone, 504 with
    // the bin of the most iterations raised, 503 with all bins ranked by their iterations.
    int prio_lo = 0, prio_hi = 0;
    HDG_CUDA(cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi));
    bool seen_all = true;
    for (auto* s : sys) seen_all = seen_all && s->last_max_iters > 0;
    auto elem_work = [&](size_t i) { return (double)sys[i]->nc * sys[i]->n * sys[i]->n * (sys[i]->m + 1); };
    size_t crit = 0;
    for (size_t i = 1; i < ns; ++i)
      if (seen_all ? sys[i]->last_max_iters > sys[crit]->last_max_iters : elem_work(i) > elem_work(crit)) crit = i;
    std::vector<int> prio(ns, prio_lo);
    prio[crit] = prio_hi;
    for (size_t i = 0; i < ns; ++i) {
      cudaStream_t qs;
      cudaEvent_t e;
      HDG_CUDA(cudaStreamCreateWithPriority(&qs, cudaStreamNonBlocking, prio[i]));
      fork.streams.push_back(qs);
      HDG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      fork.events.push_back(e);
      HDG_CUDA(cudaStreamWaitEvent(qs, start, 0));
      q[i] = qs;
    }
    HDG_CUDA(cudaEventDestroy(start));
  } else {
    q[0] = sys[0]->ctx->stream;
  }
  // per system: [assembly] -> [apply!] -> initialisation -> first chunk, queued system by system
  std::vector<cudaEvent_t> ready(ns);
  struct EvGuard {
    std::vector<cudaEvent_t>& v;
    ~EvGuard() {
      for (auto e : v)
        if (e) cudaEventDestroy(e);
    }
  } evguard{ready};
  struct UseStream {  // buffers allocated while a system is queued are ordered before its stream
    ~UseStream() { g_use_stream = nullptr; }
  } use_stream;
  for (size_t i = 0; i < ns; ++i) {
    hdg_system* s = sys[i];
    const bool prof = s->ctx->profiling;
    g_use_stream = q[i];
    HDG_CUDA(cudaEventCreateWithFlags(&ready[i], cudaEventDisableTiming));
    if (flags & HDG_STEP_ASSEMBLE) assemble_async(s, q[i]);
    if (flags & HDG_STEP_APPLY) {
      if (prof) s->ev_apply.start(q[i]);
      launch_dirichlet_apply(s, q[i]);
      if (prof) s->ev_apply.stop(q[i]);
      s->applied = true;
    }
    sv[i]->set_stream(q[i]);
    sv[i]->prepare(o);
    sv[i]->launch_chunk(0);
    sv[i]->enqueue_status_copy();
    HDG_CUDA(cudaEventRecord(ready[i], q[i]));
  }
  // Event-driven host loop: a system whose status read-back has landed is processed and given its
  // next chunk at once, without waiting for the others.
  stats->assign(ns, {});
  std::vector<char> done(ns, 0);
  std::vector<int> rep(ns, 0);
  size_t left = ns;
  while (left > 0) {
    bool progressed = false;
    for (size_t i = 0; i < ns; ++i) {
      if (done[i]) continue;
      const cudaError_t qe = cudaEventQuery(ready[i]);
      if (qe == cudaErrorNotReady) continue;
      HDG_CUDA(qe);
      progressed = true;
      g_use_stream = q[i];
      if (sv[i]->process(o)) {
        sv[i]->finish(o, &(*stats)[i]);
        hdg_system* s = sys[i];
        s->last_max_iters = 0;
        for (auto& r : (*stats)[i]) s->last_max_iters = std::max(s->last_max_iters, r.iterations);
        if (flags & HDG_STEP_RECOVER) {
          if (s->ctx->profiling) s->ev_recover.start(q[i]);
          launch_recover(s, q[i]);
          if (s->ctx->profiling) s->ev_recover.stop(q[i]);
        }
        if (flags & HDG_STEP_DOWNLOAD) {  // on the system's stream: overlaps the others' iterations
          if (s->h_dl_uhat) s->d_x.download(s->h_dl_uhat, (size_t)s->ndofs, q[i]);
          if (s->h_dl_qu) s->d_qu.download(s->h_dl_qu, (size_t)s->nc * s->n, q[i]);
        }
        done[i] = 1;
        --left;
        continue;
      }
      sv[i]->launch_chunk(++rep[i]);
      sv[i]->enqueue_status_copy();
      HDG_CUDA(cudaEventRecord(ready[i], q[i]));
    }
    if (!progressed) std::this_thread::yield();
  }
  g_use_stream = nullptr;
  if (flags & HDG_STEP_ASSEMBLE)  // element error flags (the step went on regardless)
    for (size_t i = 0; i < ns; ++i) assembly_check(sys[i], q[i]);
  if (flags & HDG_STEP_DOWNLOAD)  // the host arrays are complete on return
    for (size_t i = 0; i < ns; ++i) HDG_CUDA(cudaStreamSynchronize(q[i]));
  int rc = HDG_OK;
  for (size_t i = 0; i < ns; ++i) {
    for (auto& r : (*stats)[i]) {
      if (r.converged < 0) {
        r.converged = 0;
        rc = HDG_ERR_BREAKDOWN;
      } else if (!r.converged && rc == HDG_OK) {
        rc = HDG_ERR_NO_CONVERGENCE;
      }
    }
  }
  return rc;
}

// Solves every problem of every system; the systems' chunks are interleaved so that one host
// loop drives a whole degree-binned batch.  stats[i] receives the per-problem results of sys[i].
int run_solve_many(const std::vector<hdg_system*>& sys, const hdg_solver& o,
                   std::vector<std::vector<hdg_stats>>* stats) {
  return run_batch_step(sys, o, 0, stats);
}

int run_solve(hdg_system* s, const hdg_solver& o, hdg_stats* stats) {
  std::vector<std::vector<hdg_stats>> st;
  int rc = run_solve_many({s}, o, &st);
  if (stats) {  // aggregate over the system's problems
    hdg_stats agg{0, 0, 0.0, 1};
    for (auto& r : st[0]) {
      agg.iterations = std::max(agg.iterations, r.iterations);
      agg.outer = std::max(agg.outer, r.outer);
      agg.rel_residual = std::max(agg.rel_residual, r.rel_residual);
      agg.converged = agg.converged && r.converged;
    }
    *stats = agg;
  }
  return rc;
}
