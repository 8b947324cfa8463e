// Jacobi-preconditioned conjugate gradients on the trace system (stands in for the sparse
// direct `K \ b` of examples/poisson2D_HDG.jl:195).
//
// The matrix is the block-sparse solver form of K (free rows negated, so SPD).  One iteration
// is two kernels, using q_{k+1} = A z_{k+1} + beta q_k so that p and q are updated in the same
// pass as the product:
//   A: beta = rz/rz_old;  q = A z + beta q;  p = z + beta p;  pq = p.q
//   B: alpha = rz/pq;     x += alpha p;  r -= alpha q;  z = D^-1 r;  rz, rr
// Reductions are deterministic: each CUDA block writes a partial and the last block of a problem
// to finish (atomic ticket) sums that problem's partials in a fixed order.  Every CUDA block
// belongs to exactly one problem ("segment"), so independent problems can share one launch; a
// converged problem's blocks return at once.  CHUNK iterations are captured in a CUDA graph and
// replayed; the host reads the per-problem status between replays.
//
// Precision.  FP64: matrix, vectors and scalars in FP64.  Mixed: the inner CG runs on an FP32
// copy of the matrix with FP32 r, z, p, q, while the correction x, every dot product and every
// scalar stay FP64; an outer loop in FP64 forms r = b - K x with the FP64 matrix and solves for
// the next correction until |r| <= tol |b|.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "hdg_device.cuh"

namespace {
constexpr int CG_BLOCK = 256;
constexpr int SAMPLE_EVERY = 8;  // with profiling on, every 8th chunk runs un-graphed and timed
}  // namespace

struct CgState {
  int nseg = 0, nrow = 0;
  DevBuf<int32_t> seg_prob, seg_row0, seg_row1, prob_blk0, prob_nblk;
  DevBuf<double> part;   // [nseg][2]
  DevBuf<double> sc;     // per problem: rz, rzold, pq, rr, bb, tol2
  DevBuf<int32_t> st;    // per problem: status, iters, maxit
  DevBuf<unsigned> cnt;  // per problem tickets (2 per problem)
  DevBuf<double> r, z, p, q, dinv;      // FP64 inner vectors
  DevBuf<float> rf, zf, pf, qf, dinvf;  // FP32 inner vectors
  DevBuf<double> r64, d;                // mixed: outer residual and inner correction
  DevBuf<double> rpart, rsc;            // residual-norm reduction
  DevBuf<unsigned> rcnt;
  cudaGraphExec_t graph64 = nullptr, graph32 = nullptr;
  int chunk64 = 0, chunk32 = 0;
  int32_t* h_st = nullptr;  // pinned
  double* h_sc = nullptr;   // pinned
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
  const int32_t* seg_prob;
  const int32_t* seg_row0;
  const int32_t* seg_row1;
  const int32_t* prob_blk0;
  const int32_t* prob_nblk;
  const int32_t* browptr;
  const int32_t* bcol;
  const T* val;
  const double* b;
  const T* dinv;
  double* x;
  T* r;
  T* z;
  T* p;
  T* q;
  double* part;
  double* sc;
  int32_t* st;
  unsigned* cnt;
};

template <typename T>
__device__ __forceinline__ bool finish_reduce(const CgArgs<T>& a, int P, int slot, double v0, double v1, double* sh,
                                              double* sum0, double* sum1) {
  __shared__ bool last;
  v0 = block_sum<CG_BLOCK>(v0, sh);
  v1 = block_sum<CG_BLOCK>(v1, sh);
  if (threadIdx.x == 0) {
    a.part[2 * blockIdx.x] = v0;
    a.part[2 * blockIdx.x + 1] = v1;
    __threadfence();
    unsigned t = atomicAdd(&a.cnt[2 * P + slot], 1u);
    last = (t == (unsigned)a.prob_nblk[P] - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  const int b0 = a.prob_blk0[P], nb = a.prob_nblk[P];
  double s0 = 0.0, s1 = 0.0;
  for (int k = threadIdx.x; k < nb; k += CG_BLOCK) {
    s0 += ((volatile double*)a.part)[2 * (b0 + k)];
    s1 += ((volatile double*)a.part)[2 * (b0 + k) + 1];
  }
  *sum0 = block_sum<CG_BLOCK>(s0, sh);
  *sum1 = block_sum<CG_BLOCK>(s1, sh);
  if (threadIdx.x == 0) a.cnt[2 * P + slot] = 0;
  return true;
}

template <int NT, typename T, typename V>
__device__ __forceinline__ double row_dot(const int32_t* __restrict__ browptr, const int32_t* __restrict__ bcol,
                                          const T* __restrict__ val, int row, const V* __restrict__ v) {
  const int f = row / NT, i = row - f * NT;
  double s = 0.0;
  const int k1 = browptr[f + 1];
  for (int k = browptr[f]; k < k1; ++k) {
    const int g = bcol[k];
    const T* blk = val + (int64_t)k * NT * NT + i * NT;
    T acc = T(0);
#pragma unroll
    for (int j = 0; j < NT; ++j) acc += blk[j] * (T)v[g * NT + j];
    s += (double)acc;
  }
  return s;
}

template <int NT, typename T> __global__ void __launch_bounds__(CG_BLOCK) k_cg_init(CgArgs<T> a) {
  __shared__ double sh[32];
  const int P = a.seg_prob[blockIdx.x];
  double rz = 0.0, bb = 0.0;
  for (int row = a.seg_row0[blockIdx.x] + threadIdx.x; row < a.seg_row1[blockIdx.x]; row += CG_BLOCK) {
    const double bv = a.b[row];
    const T rv = (T)bv;
    const T zv = a.dinv[row] * rv;
    a.x[row] = 0.0;
    a.r[row] = rv;
    a.z[row] = zv;
    a.p[row] = T(0);
    a.q[row] = T(0);
    rz += (double)rv * (double)zv;
    bb += bv * bv;
  }
  double s0, s1;
  if (finish_reduce(a, P, 0, rz, bb, sh, &s0, &s1) && threadIdx.x == 0) {
    double* sc = a.sc + 6 * P;
    sc[0] = s0;
    sc[1] = s0;
    sc[3] = s1;
    sc[4] = s1;
    a.st[3 * P] = (s1 == 0.0) ? 1 : 0;
    a.st[3 * P + 1] = 0;
  }
}

template <int NT, typename T> __global__ void __launch_bounds__(CG_BLOCK) k_cg_a(CgArgs<T> a) {
  __shared__ double sh[32];
  const int P = a.seg_prob[blockIdx.x];
  if (a.st[3 * P] != 0) return;
  const double* sc = a.sc + 6 * P;
  const double beta = (a.st[3 * P + 1] == 0) ? 0.0 : sc[0] / sc[1];
  const T bt = (T)beta;
  double pq = 0.0;
  for (int row = a.seg_row0[blockIdx.x] + threadIdx.x; row < a.seg_row1[blockIdx.x]; row += CG_BLOCK) {
    const double w = row_dot<NT>(a.browptr, a.bcol, a.val, row, a.z);
    const T qn = (T)(w + beta * (double)a.q[row]);
    const T pn = a.z[row] + bt * a.p[row];
    a.q[row] = qn;
    a.p[row] = pn;
    pq += (double)pn * (double)qn;
  }
  double s0, s1;
  if (finish_reduce(a, P, 0, pq, 0.0, sh, &s0, &s1) && threadIdx.x == 0) a.sc[6 * P + 2] = s0;
}

template <int NT, typename T> __global__ void __launch_bounds__(CG_BLOCK) k_cg_b(CgArgs<T> a) {
  __shared__ double sh[32];
  const int P = a.seg_prob[blockIdx.x];
  if (a.st[3 * P] != 0) return;
  const double* sc = a.sc + 6 * P;
  const double alpha = sc[0] / sc[2];
  const T at = (T)alpha;
  double rz = 0.0, rr = 0.0;
  for (int row = a.seg_row0[blockIdx.x] + threadIdx.x; row < a.seg_row1[blockIdx.x]; row += CG_BLOCK) {
    a.x[row] += alpha * (double)a.p[row];
    const T rn = a.r[row] - at * a.q[row];
    const T zn = a.dinv[row] * rn;
    a.r[row] = rn;
    a.z[row] = zn;
    rz += (double)rn * (double)zn;
    rr += (double)rn * (double)rn;
  }
  double s0, s1;
  if (finish_reduce(a, P, 1, rz, rr, sh, &s0, &s1) && threadIdx.x == 0) {
    double* scw = a.sc + 6 * P;
    const double pq = scw[2];
    scw[1] = scw[0];
    scw[0] = s0;
    scw[3] = s1;
    const int it = a.st[3 * P + 1] + 1;
    a.st[3 * P + 1] = it;
    int status = 0;
    if (!(pq > 0.0) || !isfinite(s1)) status = 3;
    else if (s1 <= scw[5] * scw[4]) status = 1;
    else if (it >= a.st[3 * P + 2]) status = 2;
    a.st[3 * P] = status;
  }
}

template <int NT, typename T>
__global__ void k_dinv(int nrow, const int32_t* browptr, const int32_t* bcol, const double* val, T* dinv) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nrow) return;
  const int f = t / NT, i = t - f * NT;
  double d = 1.0;
  for (int k = browptr[f]; k < browptr[f + 1]; ++k)
    if (bcol[k] == f) d = val[(int64_t)k * NT * NT + i * NT + i];
  dinv[t] = (T)(1.0 / d);
}

__global__ void k_to_float(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    b[t] = (float)a[t];
}

// r = b - A x in FP64, with |r|^2 and |b|^2 reduced by the last block into out[0], out[1]
template <int NT>
__global__ void k_residual(int nrow, const int32_t* browptr, const int32_t* bcol, const double* val,
                           const double* __restrict__ b, const double* __restrict__ x, double* __restrict__ r,
                           double* part, unsigned* cnt, double* out) {
  __shared__ double sh[32];
  __shared__ bool last;
  double rr = 0.0, bb = 0.0;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nrow; t += gridDim.x * blockDim.x) {
    double bv = b[t];
    double rv = bv - row_dot<NT>(browptr, bcol, val, t, x);
    if (r) r[t] = rv;
    rr += rv * rv;
    bb += bv * bv;
  }
  rr = block_sum<256>(rr, sh);
  bb = block_sum<256>(bb, sh);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = rr;
    part[2 * blockIdx.x + 1] = bb;
    __threadfence();
    last = (atomicAdd(cnt, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (last) {
    __threadfence();
    double s0 = 0.0, s1 = 0.0;
    for (int k = threadIdx.x; k < gridDim.x; k += blockDim.x) {
      s0 += ((volatile double*)part)[2 * k];
      s1 += ((volatile double*)part)[2 * k + 1];
    }
    s0 = block_sum<256>(s0, sh);
    s1 = block_sum<256>(s1, sh);
    if (threadIdx.x == 0) {
      out[0] = s0;
      out[1] = s1;
      *cnt = 0;
    }
  }
}

__global__ void k_axpy_inplace(int n, double* __restrict__ x, const double* __restrict__ d) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) x[t] += d[t];
}

template <int NT> struct Runner {
  hdg_system* s;
  CgState& c;
  cudaStream_t st;
  int nrow;

  Runner(hdg_system* s_) : s(s_), c(*s_->cg), st(s_->ctx->stream), nrow(s_->ndofs) {}

  void setup() {
    if (c.nseg && c.nrow == nrow) return;
    const int nseg = std::max(1, std::min((nrow + 1023) / 1024, 152 * 4));
    std::vector<int32_t> sp(nseg, 0), r0(nseg), r1(nseg);
    const int per = (nrow + nseg - 1) / nseg;
    for (int k = 0; k < nseg; ++k) {
      r0[k] = std::min(nrow, k * per);
      r1[k] = std::min(nrow, (k + 1) * per);
    }
    int32_t b0 = 0, nb = nseg;
    c.seg_prob.upload(sp.data(), nseg, st);
    c.seg_row0.upload(r0.data(), nseg, st);
    c.seg_row1.upload(r1.data(), nseg, st);
    c.prob_blk0.upload(&b0, 1, st);
    c.prob_nblk.upload(&nb, 1, st);
    c.part.alloc(2 * (size_t)nseg);
    c.sc.alloc(6);
    c.st.alloc(3);
    c.cnt.alloc(2);
    HDG_CUDA(cudaMemsetAsync(c.cnt.p, 0, 2 * sizeof(unsigned), st));
    c.rpart.alloc(2 * 1024);
    c.rsc.alloc(2);
    c.rcnt.alloc(1);
    HDG_CUDA(cudaMemsetAsync(c.rcnt.p, 0, sizeof(unsigned), st));
    if (!c.h_st) HDG_CUDA(cudaMallocHost(&c.h_st, 3 * sizeof(int32_t)));
    if (!c.h_sc) HDG_CUDA(cudaMallocHost(&c.h_sc, 2 * sizeof(double)));
    c.nseg = nseg;
    c.nrow = nrow;
  }

  template <typename T> CgArgs<T> args(const T* val, const double* b, const T* dinv, double* x, T* r, T* z, T* p, T* q) {
    return CgArgs<T>{c.seg_prob.p, c.seg_row0.p, c.seg_row1.p, c.prob_blk0.p, c.prob_nblk.p, s->d_browptr.p,
                     s->d_bcol.p, val, b, dinv, x, r, z, p, q, c.part.p, c.sc.p, c.st.p, c.cnt.p};
  }

  template <typename T> void launch_pair(const CgArgs<T>& a, cudaStream_t stream) {
    k_cg_a<NT, T><<<c.nseg, CG_BLOCK, 0, stream>>>(a);
    k_cg_b<NT, T><<<c.nseg, CG_BLOCK, 0, stream>>>(a);
  }

  // Runs the inner CG (x = A^-1 b approximately) to |r| <= tol |b|; returns status, adds iterations.
  template <typename T> int cg(const CgArgs<T>& a, double tol, int maxit, int chunk, cudaGraphExec_t* graph,
                               int* graph_chunk, int* iters_out) {
    double tol2 = tol * tol;
    HDG_CUDA(cudaMemcpyAsync(c.sc.p + 5, &tol2, sizeof(double), cudaMemcpyHostToDevice, st));
    int32_t mx = maxit;
    HDG_CUDA(cudaMemcpyAsync(c.st.p + 2, &mx, sizeof(int32_t), cudaMemcpyHostToDevice, st));
    k_cg_init<NT, T><<<c.nseg, CG_BLOCK, 0, st>>>(a);
    HDG_CUDA(cudaGetLastError());
    s->ctx->launches++;
    if (!*graph || *graph_chunk != chunk) {
      if (*graph) cudaGraphExecDestroy(*graph);
      cudaStream_t cap;
      HDG_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
      cudaGraph_t g;
      HDG_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
      for (int it = 0; it < chunk; ++it) launch_pair<T>(a, cap);
      HDG_CUDA(cudaStreamEndCapture(cap, &g));
      HDG_CUDA(cudaGraphInstantiate(graph, g, 0));
      cudaGraphDestroy(g);
      cudaStreamDestroy(cap);
      *graph_chunk = chunk;
    }
    const bool prof = s->ctx->profiling;
    int status = 0;
    for (int rep = 0;; ++rep) {
      if (prof && rep % SAMPLE_EVERY == SAMPLE_EVERY - 1) {
        // a timed, un-graphed chunk: events around each kernel
        for (int it = 0; it < chunk; ++it) {
          EventPair* ea = new EventPair();
          EventPair* eb = new EventPair();
          ea->start(st);
          k_cg_a<NT, T><<<c.nseg, CG_BLOCK, 0, st>>>(a);
          ea->stop(st);
          eb->start(st);
          k_cg_b<NT, T><<<c.nseg, CG_BLOCK, 0, st>>>(a);
          eb->stop(st);
          s->ev_cg_a.push_back(ea);
          s->ev_cg_b.push_back(eb);
        }
        HDG_CUDA(cudaGetLastError());
      } else {
        HDG_CUDA(cudaGraphLaunch(*graph, st));
      }
      s->ctx->launches += 2 * chunk;
      HDG_CUDA(cudaMemcpyAsync(c.h_st, c.st.p, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
      HDG_CUDA(cudaStreamSynchronize(st));
      status = c.h_st[0];
      if (status != 0) break;
    }
    *iters_out += c.h_st[1];
    return status;
  }

  // |b - K x| / |b| in FP64 (optionally storing r)
  double residual(double* r) {
    const int blocks = std::min(1024, (nrow + 255) / 256);
    k_residual<NT><<<blocks, 256, 0, st>>>(nrow, s->d_browptr.p, s->d_bcol.p, s->d_val.p, s->d_b.p, s->d_x.p, r,
                                           c.rpart.p, c.rcnt.p, c.rsc.p);
    HDG_CUDA(cudaGetLastError());
    s->ctx->launches++;
    HDG_CUDA(cudaMemcpyAsync(c.h_sc, c.rsc.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
    HDG_CUDA(cudaStreamSynchronize(st));
    return c.h_sc[1] > 0 ? std::sqrt(c.h_sc[0] / c.h_sc[1]) : 0.0;
  }

  int run(const hdg_solver& o, hdg_stats* stats) {
    setup();
    s->d_x.alloc(nrow);
    for (auto* e : s->ev_cg_a) delete e;
    for (auto* e : s->ev_cg_b) delete e;
    s->ev_cg_a.clear();
    s->ev_cg_b.clear();
    if (s->ctx->profiling) s->ev_cg.start(st);
    const int chunk = o.chunk > 0 ? o.chunk : 32;
    int iters = 0, outer = 0, status = 0;
    double relres = 0.0;
    if (o.precision == HDG_PREC_FP64) {
      c.r.alloc(nrow); c.z.alloc(nrow); c.p.alloc(nrow); c.q.alloc(nrow); c.dinv.alloc(nrow);
      k_dinv<NT, double><<<(nrow + 255) / 256, 256, 0, st>>>(nrow, s->d_browptr.p, s->d_bcol.p, s->d_val.p, c.dinv.p);
      s->ctx->launches++;
      auto a = args<double>(s->d_val.p, s->d_b.p, c.dinv.p, s->d_x.p, c.r.p, c.z.p, c.p.p, c.q.p);
      status = cg<double>(a, o.tol, o.maxit, chunk, &c.graph64, &c.chunk64, &iters);
      outer = 1;
      relres = residual(nullptr);
    } else {
      // FP32 copy of the solver-form matrix and FP32 inner vectors
      s->d_valf.alloc((size_t)s->nnz);
      k_to_float<<<(unsigned)std::min<int64_t>((s->nnz + 255) / 256, 152 * 32), 256, 0, st>>>(s->nnz, s->d_val.p,
                                                                                             s->d_valf.p);
      c.rf.alloc(nrow); c.zf.alloc(nrow); c.pf.alloc(nrow); c.qf.alloc(nrow); c.dinvf.alloc(nrow);
      c.r64.alloc(nrow); c.d.alloc(nrow);
      k_dinv<NT, float><<<(nrow + 255) / 256, 256, 0, st>>>(nrow, s->d_browptr.p, s->d_bcol.p, s->d_val.p, c.dinvf.p);
      s->ctx->launches += 2;
      HDG_CUDA(cudaMemsetAsync(s->d_x.p, 0, nrow * sizeof(double), st));
      auto a = args<float>(s->d_valf.p, c.r64.p, c.dinvf.p, c.d.p, c.rf.p, c.zf.p, c.pf.p, c.qf.p);
      relres = residual(c.r64.p);  // r = b (x = 0)
      const int max_outer = 60;
      while (relres > o.tol && outer < max_outer && iters < o.maxit) {
        // inner tolerance relative to the current residual; never ask for less than the target
        const double itol = std::max(o.inner_tol, 0.5 * o.tol / std::max(relres, 1e-300));
        status = cg<float>(a, std::min(itol, 0.5), o.maxit - iters, chunk, &c.graph32, &c.chunk32, &iters);
        ++outer;
        if (status == 3) break;
        k_axpy_inplace<<<(nrow + 255) / 256, 256, 0, st>>>(nrow, s->d_x.p, c.d.p);
        s->ctx->launches++;
        relres = residual(c.r64.p);
      }
      if (status != 3) status = (relres <= o.tol) ? 1 : 2;
    }
    if (s->ctx->profiling) s->ev_cg.stop(st);
    s->cg_iterations = iters;
    if (stats) {
      stats->iterations = iters;
      stats->outer = outer;
      stats->rel_residual = relres;
      stats->converged = (status == 1);
    }
    if (status == 3) return HDG_ERR_BREAKDOWN;
    if (status == 2) return HDG_ERR_NO_CONVERGENCE;
    return HDG_OK;
  }
};

}  // namespace

int run_solve(hdg_system* s, const hdg_solver& o, hdg_stats* stats) {
  if (!s->cg) s->cg = new CgState();
  switch (s->nt) {
    case 2: return Runner<2>(s).run(o, stats);
    case 3: return Runner<3>(s).run(o, stats);
    case 4: return Runner<4>(s).run(o, stats);
    case 5: return Runner<5>(s).run(o, stats);
  }
  return HDG_ERR_ARG;
}
