// Global trace system: deterministic gather of the condensed cell blocks into the trace matrix,
// and the Dirichlet treatment of apply!.
//
// The reference appends every cell's Ate as COO triplets and lets `sparse(I,J,V)` sort them and
// sum duplicates (src/assembler.jl:31-49).  Here the pattern is known from the topology: block
// row f (a face) holds nt x nt blocks for f itself and for the other faces of its one or two
// cells.  Each block has at most two sources (cell, local face pair): the diagonal block sums the
// blocks of the face's two cells, an off-diagonal block has exactly one.  The source map is built
// once per mesh, so assembly is an atomic-free gather; a sum of two terms does not depend on
// their order, so it reproduces the reference values exactly.
//
// Device layout (block-ELL, see hdg_internal.h): 5 slots per face, slot-major and
// row-contiguous, so every warp-wide load of the matrix in the CG is one contiguous segment.
#include <algorithm>

#include <numeric>

#include "hdg_device.cuh"

void build_block_structure(hdg_system* s) {
  const hdg_mesh* m = s->space->mesh;
  const int nf = m->nf;
  constexpr int S = hdg_system::SLOTS;
  s->h_browptr.assign(nf + 1, 0);
  s->h_bcol.clear();
  s->h_bsrc.clear();
  s->h_bcol.reserve((size_t)nf * S);
  s->h_bsrc.reserve((size_t)nf * S * 2);
  std::vector<int32_t> bcol5((size_t)S * nf), src5((size_t)S * nf * 2, -1);
  std::vector<int8_t> kdiag(nf, 0);
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
    if (cnt > S) throw HdgError{HDG_ERR_ARG, "a face couples to more than 4 other faces (invalid triangle mesh)"};
    for (int k = 0; k < S; ++k) bcol5[(size_t)k * nf + f] = f;
    for (int k = 0; k < cnt; ++k) {
      const int g = nb[k];
      if (g == f) kdiag[f] = (int8_t)k;
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
      bcol5[(size_t)k * nf + f] = g;
      src5[((size_t)k * nf + f) * 2] = src[0];
      src5[((size_t)k * nf + f) * 2 + 1] = src[1];
    }
    s->h_browptr[f + 1] = (int32_t)s->h_bcol.size();
  }
  s->nblocks = (int64_t)s->h_bcol.size();
  s->nnz = s->nblocks * s->nt * s->nt;
  cudaStream_t st = s->ctx->stream;
  s->d_bcol5.upload(bcol5.data(), bcol5.size(), st);
  s->d_src5.upload(src5.data(), src5.size(), st);
  s->d_kdiag.upload(kdiag.data(), kdiag.size(), st);
  HDG_CUDA(cudaStreamSynchronize(st));
}

// Segments of the row-parallel kernels: every problem's trace rows are cut into ranges of at most
// SEG_ROWS rows, one CUDA block each, so a block never spans two problems.
void build_segments(hdg_system* s) {
  // About 1024 rows per segment (four per thread in the CG kernels).  Once the segments can fill
  // the GPU, their number is rounded up to a multiple of the SM count (the extra segments go to
  // the largest problems), so that every SM gets the same number of equal blocks.
  constexpr int SEG_ROWS = 1024, NUM_SM = 152;
  const hdg_mesh* m = s->space->mesh;
  s->nprob = m->nprob;
  s->h_prob_row0.assign(s->nprob + 1, 0);
  std::vector<int32_t> sp, r0, r1, b0(s->nprob), nb(s->nprob), rowp((size_t)s->ndofs);
  std::vector<int> nseg(s->nprob);
  int64_t total = 0;
  for (int P = 0; P < s->nprob; ++P) {
    s->h_prob_row0[P] = m->prob_face0[P] * s->nt;
    s->h_prob_row0[P + 1] = m->prob_face0[P + 1] * s->nt;
    const int rows = std::max(s->h_prob_row0[P + 1] - s->h_prob_row0[P], 1);
    nseg[P] = (rows + SEG_ROWS - 1) / SEG_ROWS;
    total += nseg[P];
  }
  if (total >= NUM_SM) {
    int64_t extra = (NUM_SM - total % NUM_SM) % NUM_SM;
    std::vector<int> order(s->nprob);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
      return s->h_prob_row0[x + 1] - s->h_prob_row0[x] > s->h_prob_row0[y + 1] - s->h_prob_row0[y];
    });
    for (size_t k = 0; extra > 0; k = (k + 1) % order.size(), --extra) ++nseg[order[k]];
  }
  for (int P = 0; P < s->nprob; ++P) {
    const int a = s->h_prob_row0[P], e = s->h_prob_row0[P + 1];
    const int rows = std::max(e - a, 1);
    const int n = std::min(nseg[P], rows);
    const int per = (rows + n - 1) / n;
    b0[P] = (int32_t)sp.size();
    nb[P] = n;
    for (int k = 0; k < n; ++k) {
      sp.push_back(P);
      r0.push_back(std::min(e, a + k * per));
      r1.push_back(std::min(e, a + (k + 1) * per));
    }
    for (int r = a; r < e; ++r) rowp[r] = P;
  }
  s->nseg = (int)sp.size();
  s->h_seg_prob = sp;
  s->h_seg_row0 = r0;
  s->h_seg_row1 = r1;
  s->h_prob_blk0 = b0;
  s->h_prob_nblk = nb;
  cudaStream_t st = s->ctx->stream;
  s->d_seg_prob.upload(sp.data(), sp.size(), st);
  s->d_seg_row0.upload(r0.data(), r0.size(), st);
  s->d_seg_row1.upload(r1.data(), r1.size(), st);
  s->d_prob_blk0.upload(b0.data(), b0.size(), st);
  s->d_prob_nblk.upload(nb.data(), nb.size(), st);
  s->d_row_prob.upload(rowp.data(), rowp.size(), st);
  s->ensure_reduction_buffers();
  HDG_CUDA(cudaStreamSynchronize(st));
}

namespace {
constexpr int S5 = hdg_system::SLOTS;

// Assembly of the trace system from the condensed blocks, GF faces per CTA:
//   val[(k nt + j) ndofs + r] = sum over sources of Ate_c[lf nt + i, lg nt + j],  r = f nt + i
//   b[r] = sum over the face's cells of bte_c[lf nt + i]        (assemble!(K, gdof, Ate) and (b, gdof, bte))
// The CTA first copies, for each of its faces and each of the face's two cells, the cell's nt rows of
// [Ate | bte] that belong to the face (one contiguous run of nt (m+1) doubles) into shared memory,
// then writes the faces' 5 nt x nt slot blocks slot-major, so that both the reads and the writes
// are contiguous.  The sources of a slot are added in the order src5 lists them (first the face's
// first cell), the right-hand side's in the face's cell order.  Shared rows are padded to an odd
// number of doubles so that the threads of a half-warp (consecutive rows of consecutive faces)
// fall on different banks.
template <int NT> struct GatherTile {
  static constexpr int M = 3 * NT, MS = M + 1;
  static constexpr int MSP = MS | 1;                             // padded row
  static constexpr int RBP = (NT * MSP) | 1;                     // padded row block (one face, one cell)
  static constexpr int GF = 32;                                  // faces per CTA
  static constexpr size_t SMEM = sizeof(double) * (size_t)GF * 2 * RBP;
};

template <int NT>
__global__ void __launch_bounds__(256) k_gather_faces(const int nf, const int32_t* __restrict__ fcell,
                                                      const int8_t* __restrict__ flf,
                                                      const int32_t* __restrict__ src5,
                                                      const double* __restrict__ AB, double* __restrict__ val,
                                                      double* __restrict__ b) {
  using T = GatherTile<NT>;
  constexpr int M = T::M, MS = T::MS, MSP = T::MSP, RBP = T::RBP, GF = T::GF, RB = NT * MS;
  extern __shared__ double sm[];
  const int f0 = blockIdx.x * GF;
  const int nfb = min(GF, nf - f0);
  for (int t = threadIdx.x; t < nfb * 2 * RB; t += blockDim.x) {
    const int fq = t / RB, e = t - fq * RB;                  // fq = 2 (face in tile) + side
    const int c = fcell[2 * f0 + fq];
    const int i = e / MS, col = e - i * MS;
    sm[fq * RBP + i * MSP + col] = c >= 0 ? AB[(int64_t)c * M * MS + (int64_t)flf[2 * f0 + fq] * RB + e] : 0.0;
  }
  __syncthreads();
  const int64_t ndofs = (int64_t)nf * NT;
  const int nr = nfb * NT;                                       // rows of the tile
  for (int t = threadIdx.x; t < S5 * NT * nr; t += blockDim.x) {
    const int sl = t / nr, r = t - sl * nr;
    const int fl = r / NT, i = r - fl * NT, k = sl / NT, j = sl - k * NT;
    const int f = f0 + fl;
    const int2 sp = *reinterpret_cast<const int2*>(src5 + ((int64_t)k * nf + f) * 2);
    const int c1 = fcell[2 * f];
    double v = 0.0;
    if (sp.x >= 0) v += sm[(2 * fl + (sp.x / 9 == c1 ? 0 : 1)) * RBP + i * MSP + (sp.x % 3) * NT + j];
    if (sp.y >= 0) v += sm[(2 * fl + (sp.y / 9 == c1 ? 0 : 1)) * RBP + i * MSP + (sp.y % 3) * NT + j];
    val[(int64_t)sl * ndofs + (int64_t)f0 * NT + r] = v;
  }
  for (int r = threadIdx.x; r < nr; r += blockDim.x) {
    const int fl = r / NT, i = r - fl * NT;
    double v = 0.0;
    v += sm[(2 * fl) * RBP + i * MSP + M];
    if (fcell[2 * (f0 + fl) + 1] >= 0) v += sm[(2 * fl + 1) * RBP + i * MSP + M];
    b[(int64_t)f0 * NT + r] = v;
  }
}

// meandiag(K) = mean |K_ii| of each problem (src/boundary.jl:169-175), a deterministic
// per-problem reduction over the segments.
template <int NT>
__global__ void k_meandiag(SegArgs g, const int32_t* __restrict__ prob_row0, const int nf,
                           const int8_t* __restrict__ kdiag, const double* __restrict__ val, double* __restrict__ mdiag) {
  const int P = g.seg_prob[blockIdx.x];
  const int ndofs = nf * NT;
  double acc = 0.0;
  for (int r = g.seg_row0[blockIdx.x] + threadIdx.x; r < g.seg_row1[blockIdx.x]; r += blockDim.x) {
    const int f = r / NT, i = r - f * NT;
    acc += fabs(val[(int64_t)(kdiag[f] * NT + i) * ndofs + r]);
  }
  double s0;
  if (seg_finish1<256>(g, P, 3, acc, &s0) && threadIdx.x == 0)
    mdiag[P] = s0 / (double)(prob_row0[P + 1] - prob_row0[P]);
}

// b -= sum_d v_d K[:, d] over prescribed dofs with v_d != 0 (src/boundary.jl:128-137); gv holds
// v at prescribed dofs and 0 elsewhere, so this is one sparse product with gv.
template <int NT>
__global__ void k_lift(const int nf, const int32_t* __restrict__ bcol5, const double* __restrict__ val,
                       const double* __restrict__ gv, double* __restrict__ b) {
  const int ndofs = nf * NT;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= ndofs) return;
  const int f = r / NT;
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < S5; ++k) {
    const int g = bcol5[k * nf + f];
#pragma unroll
    for (int j = 0; j < NT; ++j) s += val[(int64_t)(k * NT + j) * ndofs + r] * gv[g * NT + j];
  }
  b[r] -= s;
}

// Rows and columns of prescribed dofs zeroed, K[d,d] = m, b[d] = v m (src/boundary.jl:138-157).
// The result is stored in "solver form": free rows negated, so that the matrix the CG sees is
// symmetric positive definite (the condensed HDG trace operator is negative definite on the free
// dofs).  hdg_system_get_csc undoes the sign when exporting.
template <int NT>
__global__ void k_apply(const int nf, const int32_t* __restrict__ bcol5, const int8_t* __restrict__ kdiag,
                        const uint8_t* __restrict__ pres, const double* __restrict__ gv, const double* __restrict__ md,
                        const int32_t* __restrict__ row_prob, double* __restrict__ val, double* __restrict__ b) {
  const int ndofs = nf * NT;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= ndofs) return;
  const int f = r / NT, i = r - f * NT, kd = kdiag[f];
  const double m = md[row_prob[r]];
  const bool pr = pres[r];
#pragma unroll
  for (int k = 0; k < S5; ++k) {
    const int g = bcol5[k * nf + f];
#pragma unroll
    for (int j = 0; j < NT; ++j) {
      double& v = val[(int64_t)(k * NT + j) * ndofs + r];
      if (pr || pres[g * NT + j]) v = (k == kd && j == i) ? m : 0.0;
      else v = -v;
    }
  }
  b[r] = pr ? gv[r] * m : -b[r];
}

// prescribed dofs -> per-dof flag and value
__global__ void k_scatter_dirichlet(const int n, const int32_t* __restrict__ dofs, const double* __restrict__ vals,
                                    uint8_t* __restrict__ pres, double* __restrict__ gv) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  pres[dofs[k]] = 1;
  gv[dofs[k]] = vals[k];
}

template <int NT> void gather_t(hdg_system* s, cudaStream_t st) {
  using T = GatherTile<NT>;
  hdg_mesh* m = s->space->mesh;
  if (m->nf <= 0) return;
  const unsigned blocks = (unsigned)((m->nf + T::GF - 1) / T::GF);
  k_gather_faces<NT><<<blocks, 256, T::SMEM, st>>>(m->nf, m->d_fcell.p, m->d_flf.p, s->d_src5.p, s->d_AB.p,
                                                    s->d_val.p, s->d_b.p);
  HDG_CUDA(cudaGetLastError());
  s->ctx->launches += 1;
}

// Scatter of the prescribed dofs and values into per-row flags and values (d_pres, d_gv): the
// part of apply! that depends only on the Dirichlet data, so it survives reassembly.
void dirichlet_scatter(hdg_system* s, const std::vector<int32_t>& dofs0, const std::vector<double>& vals,
                       cudaStream_t st) {
  const int nrow = s->ndofs;
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
  s->d_mdiag.alloc(s->nprob);
  s->d_prob_row0_dev();
  s->dir_lift = lift;
  s->dir_ready = true;
}

// apply! on the assembled system from the scattered Dirichlet data: per-problem mean |diag|,
// lifting of the prescribed values into b, and the symmetric row/column elimination.
template <int NT> void apply_t(hdg_system* s, cudaStream_t st) {
  hdg_mesh* m = s->space->mesh;
  const int nrow = m->nf * NT;
  const SegArgs g{s->d_seg_prob.p, s->d_seg_row0.p, s->d_seg_row1.p, s->d_prob_blk0.p, s->d_prob_nblk.p, s->d_part.p,
                  s->d_cnt.p};
  k_meandiag<NT><<<s->nseg, 256, 0, st>>>(g, s->d_prob_row0.p, m->nf, s->d_kdiag.p, s->d_val.p, s->d_mdiag.p);
  HDG_CUDA(cudaGetLastError());
  if (s->dir_lift) {
    k_lift<NT><<<(nrow + 255) / 256, 256, 0, st>>>(m->nf, s->d_bcol5.p, s->d_val.p, s->d_gv.p, s->d_b.p);
    HDG_CUDA(cudaGetLastError());
    s->ctx->launches++;
  }
  k_apply<NT><<<(nrow + 255) / 256, 256, 0, st>>>(m->nf, s->d_bcol5.p, s->d_kdiag.p, s->d_pres.p, s->d_gv.p,
                                                  s->d_mdiag.p, s->d_row_prob.p, s->d_val.p, s->d_b.p);
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

void launch_dirichlet_scatter(hdg_system* s, const std::vector<int32_t>& dofs0, const std::vector<double>& vals,
                              cudaStream_t st) {
  dirichlet_scatter(s, dofs0, vals, st);
}

void launch_dirichlet_apply(hdg_system* s, cudaStream_t st) {
  if (!s->dir_ready) throw HdgError{HDG_ERR_ARG, "no Dirichlet set was given to this system"};
  switch (s->nt) {
    case 2: apply_t<2>(s, st); break;
    case 3: apply_t<3>(s, st); break;
    case 4: apply_t<4>(s, st); break;
    case 5: apply_t<5>(s, st); break;
    default: throw HdgError{HDG_ERR_ARG, "degree not supported"};
  }
}

void launch_apply_dirichlet(hdg_system* s, const std::vector<int32_t>& dofs0, const std::vector<double>& vals,
                            cudaStream_t st) {
  launch_dirichlet_scatter(s, dofs0, vals, st);
  launch_dirichlet_apply(s, st);
}
