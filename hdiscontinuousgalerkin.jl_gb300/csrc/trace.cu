// Global trace system: deterministic gather of the condensed cell blocks into a block-sparse
// matrix, and the Dirichlet treatment of apply!.
//
// The reference appends every cell's Ate as COO triplets and lets `sparse(I,J,V)` sort them
// and sum duplicates (src/assembler.jl:31-49).  Here the pattern is known from the topology:
// block row f (a face) holds nt x nt blocks for f itself and for the other faces of its one or
// two cells, sorted by face id.  Each block has at most two sources (cell, local face pair): the
// diagonal block sums the blocks of the face's two cells, an off-diagonal block has exactly one.
// The source map is built once per mesh, so assembly is an atomic-free gather, and because a
// sum of two terms does not depend on their order it reproduces the reference values exactly.
#include <algorithm>

#include "hdg_device.cuh"

void build_block_structure(hdg_system* s) {
  const hdg_mesh* m = s->space->mesh;
  const int nf = m->nf;
  s->h_browptr.assign(nf + 1, 0);
  s->h_bcol.clear();
  s->h_bsrc.clear();
  s->h_bcol.reserve((size_t)nf * 5);
  s->h_bsrc.reserve((size_t)nf * 10);
  int nb[8];
  for (int f = 0; f < nf; ++f) {
    const int c1 = m->faces[4 * f + 2], c2 = m->faces[4 * f + 3];
    int cnt = 0;
    nb[cnt++] = f;
    for (int c : {c1, c2}) {
      if (c < 0) continue;
      for (int l = 0; l < 3; ++l) {
        int g = m->cfaces[3 * c + l];
        if (g != f) nb[cnt++] = g;
      }
    }
    std::sort(nb, nb + cnt);
    cnt = (int)(std::unique(nb, nb + cnt) - nb);
    for (int k = 0; k < cnt; ++k) {
      const int g = nb[k];
      int src[2] = {-1, -1}, ns = 0;
      for (int c : {c1, c2}) {
        if (c < 0) continue;
        int lf = -1, lg = -1;
        for (int l = 0; l < 3; ++l) {
          if (m->cfaces[3 * c + l] == f) lf = l;
          if (m->cfaces[3 * c + l] == g) lg = l;
        }
        if (lf >= 0 && lg >= 0 && ns < 2) src[ns++] = c * 9 + lf * 3 + lg;
      }
      s->h_bcol.push_back(g);
      s->h_bsrc.push_back(src[0]);
      s->h_bsrc.push_back(src[1]);
    }
    s->h_browptr[f + 1] = (int32_t)s->h_bcol.size();
  }
  s->nblocks = (int64_t)s->h_bcol.size();
  s->nnz = s->nblocks * s->nt * s->nt;
  cudaStream_t st = s->ctx->stream;
  s->d_browptr.upload(s->h_browptr.data(), s->h_browptr.size(), st);
  s->d_bcol.upload(s->h_bcol.data(), s->h_bcol.size(), st);
  s->d_bsrc.upload(s->h_bsrc.data(), s->h_bsrc.size(), st);
}

namespace {

// value entry t of block b: K[f nt + i, g nt + j] = sum over sources of Ate_c[lf nt + i, lg nt + j]
template <int NT>
__global__ void k_gather(const int64_t nval, const int32_t* __restrict__ bsrc, const double* __restrict__ AB,
                         double* __restrict__ val) {
  constexpr int M = 3 * NT, MS = M + 1, BB = NT * NT;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nval; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = t / BB;
    const int ij = (int)(t - b * BB), i = ij / NT, j = ij - (ij / NT) * NT;
    double v = 0.0;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const int s = bsrc[2 * b + k];
      if (s >= 0) {
        const int c = s / 9, lf = (s / 3) % 3, lg = s % 3;
        v += AB[(int64_t)c * M * MS + (lf * NT + i) * MS + lg * NT + j];
      }
    }
    val[t] = v;
  }
}

// b[f nt + i] = sum over the face's cells of bte_c[lf nt + i] (assemble!(rhs, gdof, bte))
template <int NT>
__global__ void k_gather_rhs(const int nf, const int32_t* __restrict__ fcell, const int8_t* __restrict__ flf,
                             const double* __restrict__ AB, double* __restrict__ b) {
  constexpr int M = 3 * NT, MS = M + 1;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nf * NT) return;
  const int f = t / NT, i = t - f * NT;
  double v = 0.0;
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int c = fcell[2 * f + k];
    if (c >= 0) v += AB[(int64_t)c * M * MS + (flf[2 * f + k] * NT + i) * MS + M];
  }
  b[t] = v;
}

// meandiag(K) = mean |K_ii| (src/boundary.jl:374-380): fixed-order per-block partial sums,
// reduced by the last block to finish (deterministic, no floating-point atomics).
template <int NT>
__global__ void k_meandiag(const int nf, const int32_t* __restrict__ browptr, const int32_t* __restrict__ bcol,
                           const double* __restrict__ val, double* __restrict__ partial, unsigned* counter,
                           double* out) {
  __shared__ double sh[32];
  __shared__ bool last;
  double acc = 0.0;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nf * NT; t += gridDim.x * blockDim.x) {
    const int f = t / NT, i = t - f * NT;
    for (int b = browptr[f]; b < browptr[f + 1]; ++b)
      if (bcol[b] == f) acc += fabs(val[(int64_t)b * NT * NT + i * NT + i]);
  }
  acc = block_sum<256>(acc, sh);
  if (threadIdx.x == 0) {
    partial[blockIdx.x] = acc;
    __threadfence();
    unsigned v = atomicAdd(counter, 1u);
    last = (v == gridDim.x - 1);
  }
  __syncthreads();
  if (last) {
    __threadfence();
    double s = 0.0;
    for (int k = threadIdx.x; k < gridDim.x; k += blockDim.x) s += ((volatile double*)partial)[k];
    s = block_sum<256>(s, sh);
    if (threadIdx.x == 0) {
      out[0] = s / (double)(nf * NT);
      *counter = 0;
    }
  }
}

// b -= sum_d v_d K[:, d] over prescribed dofs with v_d != 0 (src/boundary.jl:334-343); gv holds
// v at prescribed dofs and 0 elsewhere, so this is one block-sparse product with gv.
template <int NT>
__global__ void k_lift(const int nf, const int32_t* __restrict__ browptr, const int32_t* __restrict__ bcol,
                       const double* __restrict__ val, const double* __restrict__ gv, double* __restrict__ b) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nf * NT) return;
  const int f = t / NT, i = t - f * NT;
  double s = 0.0;
  for (int k = browptr[f]; k < browptr[f + 1]; ++k) {
    const int g = bcol[k];
#pragma unroll
    for (int j = 0; j < NT; ++j) s += val[(int64_t)k * NT * NT + i * NT + j] * gv[g * NT + j];
  }
  b[t] -= s;
}

// Rows and columns of prescribed dofs zeroed, K[d,d] = m, b[d] = v m (src/boundary.jl:344-362).
// The result is stored in "solver form": free rows negated, so that the matrix the CG sees is
// symmetric positive definite (the condensed HDG trace operator is negative definite on the free
// dofs).  hdg_system_get_csc undoes the sign when exporting.
template <int NT>
__global__ void k_apply(const int nf, const int32_t* __restrict__ browptr, const int32_t* __restrict__ bcol,
                        const uint8_t* __restrict__ pres, const double* __restrict__ gv, const double* __restrict__ md,
                        double* __restrict__ val, double* __restrict__ b) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nf * NT) return;
  const int f = t / NT, i = t - f * NT;
  const double m = md[0];
  const bool pr = pres[t];
  for (int k = browptr[f]; k < browptr[f + 1]; ++k) {
    const int g = bcol[k];
#pragma unroll
    for (int j = 0; j < NT; ++j) {
      const int c = g * NT + j;
      double& v = val[(int64_t)k * NT * NT + i * NT + j];
      if (pr || pres[c]) v = (c == t) ? m : 0.0;
      else v = -v;
    }
  }
  b[t] = pr ? gv[t] * m : -b[t];
}

template <int NT> void gather_t(hdg_system* s, cudaStream_t st) {
  hdg_mesh* m = s->space->mesh;
  const int64_t nval = s->nblocks * NT * NT;
  int blocks = (int)std::min<int64_t>((nval + 255) / 256, 152 * 32);
  k_gather<NT><<<blocks, 256, 0, st>>>(nval, s->d_bsrc.p, s->d_AB.p, s->d_val.p);
  HDG_CUDA(cudaGetLastError());
  const int nrow = m->nf * NT;
  k_gather_rhs<NT><<<(nrow + 255) / 256, 256, 0, st>>>(m->nf, m->d_fcell.p, m->d_flf.p, s->d_AB.p, s->d_b.p);
  HDG_CUDA(cudaGetLastError());
  s->ctx->launches += 2;
}

// prescribed dofs -> per-dof flag and value
__global__ void k_scatter_dirichlet(const int n, const int32_t* __restrict__ dofs, const double* __restrict__ vals,
                                    uint8_t* __restrict__ pres, double* __restrict__ gv) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  pres[dofs[k]] = 1;
  gv[dofs[k]] = vals[k];
}

template <int NT>
void apply_t(hdg_system* s, const std::vector<int32_t>& dofs0, const std::vector<double>& vals, cudaStream_t st) {
  hdg_mesh* m = s->space->mesh;
  const int nrow = m->nf * NT;
  bool lift = false;
  for (size_t k = 0; k < dofs0.size(); ++k)
    if (vals[k] != 0.0) lift = true;
  s->ensure_reduction_buffers();
  s->d_pres.alloc(nrow);
  s->d_gv.alloc(nrow);
  HDG_CUDA(cudaMemsetAsync(s->d_pres.p, 0, nrow, st));
  HDG_CUDA(cudaMemsetAsync(s->d_gv.p, 0, nrow * sizeof(double), st));
  const int nd = (int)dofs0.size();
  if (nd > 0) {
    s->d_dofs.upload(dofs0.data(), nd, st);
    s->d_dvals.upload(vals.data(), nd, st);
    k_scatter_dirichlet<<<(nd + 255) / 256, 256, 0, st>>>(nd, s->d_dofs.p, s->d_dvals.p, s->d_pres.p, s->d_gv.p);
    HDG_CUDA(cudaGetLastError());
    s->ctx->launches++;
  }
  const int rb = std::min(1024, (nrow + 255) / 256);
  k_meandiag<NT><<<rb, 256, 0, st>>>(m->nf, s->d_browptr.p, s->d_bcol.p, s->d_val.p, s->d_part.p, s->d_cnt.p,
                                     s->d_scal.p);
  HDG_CUDA(cudaGetLastError());
  if (lift) {
    k_lift<NT><<<(nrow + 255) / 256, 256, 0, st>>>(m->nf, s->d_browptr.p, s->d_bcol.p, s->d_val.p, s->d_gv.p, s->d_b.p);
    HDG_CUDA(cudaGetLastError());
    s->ctx->launches++;
  }
  k_apply<NT><<<(nrow + 255) / 256, 256, 0, st>>>(m->nf, s->d_browptr.p, s->d_bcol.p, s->d_pres.p, s->d_gv.p,
                                                  s->d_scal.p, s->d_val.p, s->d_b.p);
  HDG_CUDA(cudaGetLastError());
  s->ctx->launches += 2;
}

}  // namespace

void launch_gather(hdg_system* s, cudaStream_t st) {
  switch (s->nt) {
    case 2: gather_t<2>(s, st); break;
    case 3: gather_t<3>(s, st); break;
    case 4: gather_t<4>(s, st); break;
    case 5: gather_t<5>(s, st); break;
    default: throw HdgError{HDG_ERR_ARG, "degree not supported"};
  }
}

void launch_apply_dirichlet(hdg_system* s, const std::vector<int32_t>& dofs0, const std::vector<double>& vals,
                            cudaStream_t st) {
  switch (s->nt) {
    case 2: apply_t<2>(s, dofs0, vals, st); break;
    case 3: apply_t<3>(s, dofs0, vals, st); break;
    case 4: apply_t<4>(s, dofs0, vals, st); break;
    case 5: apply_t<5>(s, dofs0, vals, st); break;
    default: throw HdgError{HDG_ERR_ARG, "degree not supported"};
  }
}
