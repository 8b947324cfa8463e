// Local recovery of (q, u) from the trace solution (get_uσ!, examples/poisson2D_HDG.jl:197-212)
// and the squared L2 error (errornorm, src/DiscreteFunctions.jl:97-120).
#include <vector>

#include "hdg_device.cuh"

namespace {

// [q; u]_c = K_e u_hat_e + b_e, with u_hat_e gathered face by face, slice (f-1)nt+1 : f nt.
template <int P>
__global__ void k_recover(const int nc, const int32_t* __restrict__ cfaces, const double* __restrict__ KB,
                          const double* __restrict__ x, double* __restrict__ qu) {
  using D = Dims<P>;
  constexpr int N = D::N, M = D::M, NT = D::NT;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)nc * N) return;
  const int c = (int)(t / N), i = (int)(t - (int64_t)c * N);
  const double* row = KB + ((int64_t)c * N + i) * (M + 1);
  double s = row[M];
#pragma unroll
  for (int f = 0; f < 3; ++f) {
    const int g = cfaces[3 * c + f];
#pragma unroll
    for (int j = 0; j < NT; ++j) s += row[f * NT + j] * x[g * NT + j];
  }
  qu[t] = s;
}

// Recovery for the Cholesky-Schur element path, which stores only the u rows [X_u | b_u] of
// [K_e | b_e]: u = X_u u_hat_e + b_u, then q from u, q_c = kf (adl0_c M^-1 D0 u + adl1_c M^-1 D1 u
// - sum_f wn_f,c M^-1 F_{f,o} u_hat_f) (the q rows of K_e applied to the same u_hat_e, in closed form:
// Ae = (det J / kappa) diag(M, M) on this path).  One thread per cell; tables read through L1.
template <int P>
__global__ void k_recover_u(const int nc, const int32_t* __restrict__ cells, const int32_t* __restrict__ cfaces,
                            const uint8_t* __restrict__ orient, const double* __restrict__ xy,
                            const double* __restrict__ kcell, const double* __restrict__ SMD0,
                            const double* __restrict__ SMD1, const double* __restrict__ SMF,
                            const double* __restrict__ KBu, const double* __restrict__ x, double* __restrict__ qu) {
  using D = Dims<P>;
  constexpr int NW = D::NW, NT = D::NT, NV = D::NV, N = D::N, M = D::M;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nc) return;
  double uh[M];
#pragma unroll
  for (int f = 0; f < 3; ++f) {
    const int g = cfaces[3 * e + f];
#pragma unroll
    for (int j = 0; j < NT; ++j) uh[f * NT + j] = x[g * NT + j];
  }
  const double* Xu = KBu + (size_t)e * NW * (M + 1);
  double u[NW];
#pragma unroll
  for (int ia = 0; ia < NW; ++ia) {
    double t = Xu[ia * (M + 1) + M];
#pragma unroll
    for (int j = 0; j < M; ++j) t += Xu[ia * (M + 1) + j] * uh[j];
    u[ia] = t;
    qu[(size_t)e * N + NV + ia] = t;
  }
  const int n0 = cells[3 * e], n1 = cells[3 * e + 1], n2 = cells[3 * e + 2];
  const double J00 = xy[2 * n1] - xy[2 * n0], J01 = xy[2 * n2] - xy[2 * n0];
  const double J10 = xy[2 * n1 + 1] - xy[2 * n0 + 1], J11 = xy[2 * n2 + 1] - xy[2 * n0 + 1];
  const double detJ = J00 * J11 - J01 * J10;
  const double ad00 = J11, ad01 = -J01, ad10 = -J10, ad11 = J00;
  const double wn[3][2] = {{-(J10 - J11), J00 - J01}, {-J11, J01}, {J10, -J00}};
  const double kinv = kcell ? 1.0 / kcell[e] : 1.0;
  const double kf = 1.0 / (kinv * detJ);
  const unsigned ob = orient[e];
#pragma unroll 1
  for (int ia = 0; ia < NW; ++ia) {
    double g0 = 0.0, g1 = 0.0;
#pragma unroll
    for (int ib = 0; ib < NW; ++ib) {
      g0 += __ldg(SMD0 + ia * NW + ib) * u[ib];
      g1 += __ldg(SMD1 + ia * NW + ib) * u[ib];
    }
    double q0 = ad00 * g0 + ad10 * g1, q1 = ad01 * g0 + ad11 * g1;
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      const int fo = f * 2 + ((ob >> f) & 1);
      double mf = 0.0;
#pragma unroll
      for (int j = 0; j < NT; ++j) mf += __ldg(SMF + (fo * NW + ia) * NT + j) * uh[f * NT + j];
      q0 -= wn[f][0] * mf;
      q1 -= wn[f][1] * mf;
    }
    qu[(size_t)e * N + ia] = kf * q0;
    qu[(size_t)e * N + NW + ia] = kf * q1;
  }
}

template <int P>
__global__ void k_errornorm(const int nc, const int32_t* __restrict__ cells, const double* __restrict__ xy,
                            const double* __restrict__ ref, int nq, int offN, int offQ, const double* __restrict__ qw,
                            const double* __restrict__ qu, FieldDev uex, double* partial, unsigned* counter,
                            double* out) {
  using D = Dims<P>;
  constexpr int NW = D::NW, N = D::N, NV = D::NV;
  __shared__ double sh[32];
  __shared__ bool last;
  double acc = 0.0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
    const int n0 = cells[3 * c], n1 = cells[3 * c + 1], n2 = cells[3 * c + 2];
    const double x1 = xy[2 * n0], y1 = xy[2 * n0 + 1], x2 = xy[2 * n1], y2 = xy[2 * n1 + 1];
    const double x3 = xy[2 * n2], y3 = xy[2 * n2 + 1];
    const double detJ = (x2 - x1) * (y3 - y1) - (x3 - x1) * (y2 - y1);
    double el = 0.0;
    for (int q = 0; q < nq; ++q) {
      double uh = 0.0;
#pragma unroll
      for (int a = 0; a < NW; ++a) uh += qu[(int64_t)c * N + NV + a] * ref[offN + a * nq + q];
      const double xi = ref[offQ + 2 * q], eta = ref[offQ + 2 * q + 1];
      const double xq = (1.0 - xi - eta) * x1 + xi * x2 + eta * x3;
      const double yq = (1.0 - xi - eta) * y1 + xi * y2 + eta * y3;
      const double d = uh - eval_field_dev(uex, xq, yq);
      el += d * d * detJ * qw[q];
    }
    acc += el;
  }
  acc = block_sum<256>(acc, sh);
  if (threadIdx.x == 0) {
    partial[blockIdx.x] = acc;
    __threadfence();
    last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (last) {
    __threadfence();
    double s = 0.0;
    for (int k = threadIdx.x; k < gridDim.x; k += blockDim.x) s += ((volatile double*)partial)[k];
    s = block_sum<256>(s, sh);
    if (threadIdx.x == 0) {
      out[0] = s;
      *counter = 0;
    }
  }
}

template <int P> void recover_p(hdg_system* s, cudaStream_t st) {
  using D = Dims<P>;
  hdg_mesh* m = s->space->mesh;
  const int64_t tot = (int64_t)m->nc * D::N;
  s->d_qu.alloc((size_t)tot);
  if constexpr (P != 2) {
    if (s->kb_u_only) {
      const RefLayout L = ref_layout(s->space->t.nw, s->space->t.nt, s->space->t.nq);
      const double* ref = s->space->d_ref.p;
      k_recover_u<P><<<(unsigned)((m->nc + 127) / 128), 128, 0, st>>>(
          m->nc, m->d_cells.p, m->d_cfaces.p, m->d_orient.p, m->d_xy.p, s->kappa_cells ? s->d_kappa.p : nullptr,
          ref + L.SMD0, ref + L.SMD1, ref + L.SMF, s->d_KB.p, s->d_x.p, s->d_qu.p);
      HDG_CUDA(cudaGetLastError());
      s->ctx->launches++;
      return;
    }
  }
  k_recover<P><<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(m->nc, m->d_cfaces.p, s->d_KB.p, s->d_x.p, s->d_qu.p);
  HDG_CUDA(cudaGetLastError());
  s->ctx->launches++;
}

template <int P> double errornorm_p(hdg_system* s, const FieldSpec& uex, cudaStream_t st) {
  hdg_space* sp = s->space;
  hdg_mesh* m = sp->mesh;
  const RefTables& t = sp->t;
  RefLayout L = ref_layout(t.nw, t.nt, t.nq);
  DevBuf<double> prm, qw, partial, out;
  prm.upload(uex.prm.data(), uex.prm.size(), st);
  qw.upload(t.qw.data(), t.qw.size(), st);
  const int blocks = std::min(1024, (m->nc + 255) / 256);
  partial.alloc(blocks);
  out.alloc(1);
  DevBuf<unsigned> counter;
  counter.alloc(1);
  HDG_CUDA(cudaMemsetAsync(counter.p, 0, sizeof(unsigned), st));
  FieldDev fd{uex.kind, (int)uex.prm.size(), prm.p};
  k_errornorm<P><<<blocks, 256, 0, st>>>(m->nc, m->d_cells.p, m->d_xy.p, sp->d_ref.p, t.nq, L.N, L.Q, qw.p, s->d_qu.p,
                                         fd, partial.p, counter.p, out.p);
  HDG_CUDA(cudaGetLastError());
  s->ctx->launches++;
  double h = 0;
  out.download(&h, 1, st);
  HDG_CUDA(cudaStreamSynchronize(st));
  return h;
}

// u_h at the three vertices of every cell: uv[c][k] = sum_a u[c,a] N_a(vertex k)
template <int P>
__global__ void k_vertex_values(const int nc, const double* __restrict__ qu, const double* __restrict__ nv,
                                double* __restrict__ uv) {
  using D = Dims<P>;
  constexpr int NW = D::NW, N = D::N, NV = D::NV;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)nc * 3) return;
  const int c = (int)(t / 3), k = (int)(t - (int64_t)c * 3);
  double s = 0.0;
#pragma unroll
  for (int a = 0; a < NW; ++a) s += qu[(int64_t)c * N + NV + a] * nv[a * 3 + k];
  uv[t] = s;
}

// nodal_avg: every node averages the vertex values of its cells, summed in cell order
__global__ void k_node_average(const int nn, const int32_t* __restrict__ ptr, const int32_t* __restrict__ ent,
                               const double* __restrict__ uv, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn) return;
  double s = 0.0;
  for (int e = ptr[i]; e < ptr[i + 1]; ++e) s += uv[ent[e]];
  out[i] = (ptr[i + 1] > ptr[i]) ? s / (double)(ptr[i + 1] - ptr[i]) : 0.0;
}

template <int P> void nodal_avg_p(hdg_system* s, double* host_out, cudaStream_t st) {
  hdg_space* sp = s->space;
  hdg_mesh* m = sp->mesh;
  // node -> (cell, vertex) entries in cell order
  std::vector<int32_t> ptr(m->nn + 1, 0), ent((size_t)m->nc * 3);
  for (int c = 0; c < m->nc; ++c)
    for (int k = 0; k < 3; ++k) ++ptr[m->cells[3 * c + k] + 1];
  for (int i = 0; i < m->nn; ++i) ptr[i + 1] += ptr[i];
  std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
  for (int c = 0; c < m->nc; ++c)
    for (int k = 0; k < 3; ++k) ent[fill[m->cells[3 * c + k]]++] = 3 * c + k;
  DevBuf<int32_t> dptr, dent;
  DevBuf<double> nv, uv, out;
  dptr.upload(ptr.data(), ptr.size(), st);
  dent.upload(ent.data(), ent.size(), st);
  nv.upload(sp->t.Nv.data(), sp->t.Nv.size(), st);
  uv.alloc((size_t)m->nc * 3);
  out.alloc(m->nn);
  const int64_t tot = (int64_t)m->nc * 3;
  k_vertex_values<P><<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(m->nc, s->d_qu.p, nv.p, uv.p);
  k_node_average<<<(m->nn + 255) / 256, 256, 0, st>>>(m->nn, dptr.p, dent.p, uv.p, out.p);
  HDG_CUDA(cudaGetLastError());
  s->ctx->launches += 2;
  out.download(host_out, m->nn, st);
  HDG_CUDA(cudaStreamSynchronize(st));
}

}  // namespace

void run_nodal_avg(hdg_system* s, double* host_out, cudaStream_t st) {
  switch (s->space->t.p) {
    case 1: nodal_avg_p<1>(s, host_out, st); break;
    case 2: nodal_avg_p<2>(s, host_out, st); break;
    case 3: nodal_avg_p<3>(s, host_out, st); break;
    case 4: nodal_avg_p<4>(s, host_out, st); break;
  }
}

void launch_recover(hdg_system* s, cudaStream_t st) {
  switch (s->space->t.p) {
    case 1: recover_p<1>(s, st); break;
    case 2: recover_p<2>(s, st); break;
    case 3: recover_p<3>(s, st); break;
    case 4: recover_p<4>(s, st); break;
  }
}

double run_errornorm(hdg_system* s, const FieldSpec& uex, cudaStream_t st) {
  switch (s->space->t.p) {
    case 1: return errornorm_p<1>(s, uex, st);
    case 2: return errornorm_p<2>(s, uex, st);
    case 3: return errornorm_p<3>(s, uex, st);
    case 4: return errornorm_p<4>(s, uex, st);
  }
  return -1.0;
}
