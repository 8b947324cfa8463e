// FP64 iterative refinement of the trace solution with a double-double residual.
//
// The reference solves the trace system directly (`K \ b`, examples/poisson2D_HDG.jl:195), so its
// answer carries the direct solver's forward error, of order cond(K) 2^-53.  The CG of cg.cu
// stops on a relative residual, and an FP64 residual cannot certify more: for a solution x that is
// already correct to the last bit, b - K x formed in FP64 is of the size of its own rounding error
// (2^-53 |K||x|), about 1e-12 of |b| on a 2*256^2-cell system.  A refinement step
//   r = b - K x  (double-double: exact products by FMA, TwoSum accumulation, one final rounding)
//   K d = r      (the CG of cg.cu, to a loose relative tolerance)
//   x = x + d
// shrinks the error by the correction solve's relative accuracy each time (Wilkinson 1963;
// Moler 1967), down to the rounding of x itself.  Two steps bring a 1e-12-tolerance CG solution to
// within a few units in the last place of the FP64 system's exact solution, which is what a
// 1e-12 comparison against an independently computed direct solution needs.
//
// The correction solve reuses the system's CG (and its preconditioner) unchanged: the right-hand
// side buffer temporarily holds r and the solution buffer d, so every captured graph stays valid.
#include <cmath>
#include <vector>

#include "hdg_device.cuh"

namespace {

// r = b - K x over the block-ELL solver form (5 block slots per face row, slot-major values).
// Every product a x is split exactly as p + e with one FMA; the row sum is an unevaluated pair
// (hi, lo) updated by TwoSum.  __dmul_rn / __dadd_rn keep the compiler from contracting the
// error-free transformations into FMAs of its own.
template <int NT>
__global__ void __launch_bounds__(256) k_residual_dd(const int32_t* __restrict__ bcol5, int nf,
                                                     const double* __restrict__ val, const double* __restrict__ b,
                                                     const double* __restrict__ x, double* __restrict__ r) {
  const int64_t ndofs = (int64_t)nf * NT;
  for (int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; row < ndofs;
       row += (int64_t)gridDim.x * blockDim.x) {
    const int f = (int)(row / NT);
    double hi = b[row], lo = 0.0;
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      const int g = __ldg(bcol5 + (int64_t)k * nf + f);
#pragma unroll
      for (int j = 0; j < NT; ++j) {
        const double a = -__ldg(val + (int64_t)(k * NT + j) * ndofs + row);
        const double xv = __ldg(x + (int64_t)g * NT + j);
        const double p = __dmul_rn(a, xv);
        const double e = fma(a, xv, -p);
        const double s = __dadd_rn(hi, p);
        const double bv = __dsub_rn(s, hi);
        const double err = __dadd_rn(__dsub_rn(hi, __dsub_rn(s, bv)), __dsub_rn(p, bv));
        hi = s;
        lo = __dadd_rn(lo, __dadd_rn(err, e));
      }
    }
    r[row] = __dadd_rn(hi, lo);
  }
}

__global__ void k_add_into(int64_t n, const double* __restrict__ a, double* __restrict__ x) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    x[t] = a[t] + x[t];
}

void launch_residual_dd(hdg_system* s, const double* b, const double* x, double* r, cudaStream_t st) {
  const unsigned grid = (unsigned)std::min<int64_t>(((int64_t)s->ndofs + 255) / 256, 152 * 16);
  switch (s->nt) {
    case 2: k_residual_dd<2><<<grid, 256, 0, st>>>(s->d_bcol5.p, s->nf, s->d_val.p, b, x, r); break;
    case 3: k_residual_dd<3><<<grid, 256, 0, st>>>(s->d_bcol5.p, s->nf, s->d_val.p, b, x, r); break;
    case 4: k_residual_dd<4><<<grid, 256, 0, st>>>(s->d_bcol5.p, s->nf, s->d_val.p, b, x, r); break;
    case 5: k_residual_dd<5><<<grid, 256, 0, st>>>(s->d_bcol5.p, s->nf, s->d_val.p, b, x, r); break;
    default: throw HdgError{HDG_ERR_ARG, "degree not supported"};
  }
  HDG_CUDA(cudaGetLastError());
  s->ctx->launches++;
}

}  // namespace

int run_refine(hdg_system* s, const hdg_solver& o, int steps, double ctol, std::vector<hdg_stats>* out) {
  cudaStream_t st = s->ctx->stream;
  const int64_t n = s->ndofs;
  DevBuf<double> b0, x0, r;
  b0.alloc(n);
  x0.alloc(n);
  r.alloc(n);
  HDG_CUDA(cudaMemcpyAsync(b0.p, s->d_b.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
  hdg_solver oc = o;
  oc.tol = ctol;
  std::vector<int> iters(s->nprob, 0);
  int rc = HDG_OK;
  const unsigned grid = (unsigned)std::min<int64_t>((n + 255) / 256, 152 * 16);
  for (int k = 0; k < steps && rc == HDG_OK; ++k) {
    launch_residual_dd(s, b0.p, s->d_x.p, r.p, st);
    HDG_CUDA(cudaMemcpyAsync(x0.p, s->d_x.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    HDG_CUDA(cudaMemcpyAsync(s->d_b.p, r.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    std::vector<std::vector<hdg_stats>> sk;
    rc = run_solve_many({s}, oc, &sk);
    for (int P = 0; P < s->nprob; ++P) iters[P] += sk[0][P].iterations;
    k_add_into<<<grid, 256, 0, st>>>(n, x0.p, s->d_x.p);  // x = x0 + d
    HDG_CUDA(cudaGetLastError());
    s->ctx->launches++;
  }
  HDG_CUDA(cudaMemcpyAsync(s->d_b.p, b0.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
  // relative double-double residual of the refined solution, per problem
  launch_residual_dd(s, b0.p, s->d_x.p, r.p, st);
  std::vector<double> hr(n), hb(n);
  r.download(hr.data(), n, st);
  b0.download(hb.data(), n, st);
  HDG_CUDA(cudaStreamSynchronize(st));
  out->assign(s->nprob, hdg_stats{});
  for (int P = 0; P < s->nprob; ++P) {
    double rr = 0.0, bb = 0.0;
    for (int i = s->h_prob_row0[P]; i < s->h_prob_row0[P + 1]; ++i) {
      rr += hr[i] * hr[i];
      bb += hb[i] * hb[i];
    }
    hdg_stats& t = (*out)[P];
    t.iterations = iters[P];
    t.outer = steps;
    t.rel_residual = bb > 0 ? std::sqrt(rr / bb) : std::sqrt(rr);
    t.converged = (rc == HDG_OK) ? 1 : 0;
  }
  return rc;
}
