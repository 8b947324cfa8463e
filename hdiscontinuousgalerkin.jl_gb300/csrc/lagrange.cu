// Continuous-Galerkin Poisson path (examples/poisson2D_CG.jl, test/test_CGExample.jl): the
// nodal Lagrange element of a DofHandler, stiffness and load assembled on the device straight
// into the DofHandler's CSC pattern, apply!, preconditioned CG and errornorm.
//
//  * Element kernel: one thread per (cell, local row i) forms row i of
//    Ke = sum_q kappa (grad phi_i . grad phi_j) detJ w_q and fe_i = sum_q f(x_q) phi_i detJ w_q
//    (the element loop of doassemble, poisson2D_CG.jl:76-113), with grad phi = J^-T grad_ref phi
//    (reinit!, src/ScalarFunctionSpaces.jl:101-132).
//  * assemble! (src/assembler.jl:97-137) as a gather: every stored entry of K, and every entry of
//    b, sums its contributions (cell, i, j) in cell order from a list built once on the host, so
//    the assembly is deterministic and needs no atomics.
//  * apply! (src/boundary.jl:121-158, APPLY_TRANSPOSE): b -= v K[:, d] for the prescribed dofs
//    in increasing order, prescribed rows and columns zeroed, K[d, d] = mean |diag K|,
//    b[d] = v mean |diag K|.
//  * K \ b (poisson2D_CG.jl:126) by Jacobi-preconditioned CG in FP64.  Two kernels per
//    iteration; the dot products are per-block partial sums that every block of the next kernel
//    adds in the same fixed order, so all blocks take the same decisions and the result is
//    reproducible.
//  * errornorm (src/DiscreteFunctions.jl:97-120): sum over cells and points of
//    (u_h(x_q) - u(x_q))^2 detJ w_q.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "hdg_device.cuh"

struct hdg_lagrange {
  hdg_ctx* ctx = nullptr;
  const hdg_mesh* mesh = nullptr;
  int order = 1, qd = 2, nl = 3, nq = 0, nc = 0, ndofs = 0;
  int64_t nnz = 0;
  LagrangeTables t;
  DevBuf<double> d_tab;        // N [nl][nq], dN [nl][nq][2], qx, qy, qw
  DevBuf<int32_t> d_cdofs;     // [nc][nl] 0-based
  DevBuf<int32_t> d_colptr, d_rowval;
  DevBuf<int32_t> d_gptr, d_gsrc, d_bptr, d_bsrc;  // contributions per stored entry / per dof
  DevBuf<double> d_ke, d_fe;   // [nc][nl][nl], [nc][nl]
  DevBuf<double> d_val, d_b;   // K (CSC values), b
  DevBuf<double> d_fprm, d_kappa;
  DevBuf<uint8_t> d_pres;
  DevBuf<double> d_gv;
  DevBuf<double> d_x, d_r, d_z, d_p, d_p2, d_q, d_dinv, d_part, d_sc;
  DevBuf<int32_t> d_err;
  bool assembled = false, applied = false, solved = false;
  std::vector<int32_t> h_colptr, h_rowval;
};

namespace {

constexpr int LB = 256;       // threads per block of the row kernels
constexpr int LMAX_BLOCKS = 592;  // 4 x 148: enough blocks to fill the GPU, few partials to add

// ---- element kernel: row i of Ke and fe_i of one cell per thread -------------------------------
__global__ void k_lag_element(int nc, int nl, int nq, const double* __restrict__ xy, const int32_t* __restrict__ cells,
                              const double* __restrict__ tab, int fkind, const double* __restrict__ fprm,
                              const double* __restrict__ kappa, double* __restrict__ ke, double* __restrict__ fe,
                              int* __restrict__ err) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)nc * nl) return;
  const int c = (int)(t / nl), i = (int)(t - (int64_t)c * nl);
  const double* N = tab;
  const double* dN = tab + (size_t)nl * nq;
  const double* qx = dN + (size_t)nl * nq * 2;
  const double* qy = qx + nq;
  const double* qw = qy + nq;
  const int n0 = cells[3 * c], n1 = cells[3 * c + 1], n2 = cells[3 * c + 2];
  const double x1 = xy[2 * n0], y1 = xy[2 * n0 + 1];
  const double J00 = xy[2 * n1] - x1, J01 = xy[2 * n2] - x1;
  const double J10 = xy[2 * n1 + 1] - y1, J11 = xy[2 * n2 + 1] - y1;
  const double detJ = J00 * J11 - J01 * J10;
  if (!(detJ > 0.0)) {
    if (i == 0) atomicOr(err, 1);
    return;
  }
  // Jinv[a][b] = d xi_a / d x_b
  const double i00 = J11 / detJ, i01 = -J01 / detJ, i10 = -J10 / detJ, i11 = J00 / detJ;
  const double kc = kappa ? kappa[c] : 1.0;
  double row[HDG_LAGRANGE_MAX_NL];
  for (int j = 0; j < nl; ++j) row[j] = 0.0;
  double f_i = 0.0;
  for (int q = 0; q < nq; ++q) {
    const double dV = detJ * qw[q];
    const double gxi = dN[((size_t)i * nq + q) * 2], gei = dN[((size_t)i * nq + q) * 2 + 1];
    const double gix = gxi * i00 + gei * i10, giy = gxi * i01 + gei * i11;
    for (int j = 0; j < nl; ++j) {
      const double gxj = dN[((size_t)j * nq + q) * 2], gej = dN[((size_t)j * nq + q) * 2 + 1];
      const double gjx = gxj * i00 + gej * i10, gjy = gxj * i01 + gej * i11;
      row[j] += kc * (gix * gjx + giy * gjy) * dV;
    }
    const double xi = qx[q], eta = qy[q];
    const double xq = (1.0 - xi - eta) * x1 + xi * xy[2 * n1] + eta * xy[2 * n2];
    const double yq = (1.0 - xi - eta) * y1 + xi * xy[2 * n1 + 1] + eta * xy[2 * n2 + 1];
    f_i += eval_field_kind(fkind, fprm, xq, yq) * N[(size_t)i * nq + q] * dV;
  }
  for (int j = 0; j < nl; ++j) ke[((size_t)c * nl + i) * nl + j] = row[j];
  fe[(size_t)c * nl + i] = f_i;
}

// ---- assemble! as a gather ----------------------------------------------------------------------
__global__ void k_lag_gather(int64_t n, const int32_t* __restrict__ ptr, const int32_t* __restrict__ src,
                             const double* __restrict__ from, double* __restrict__ to) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int k = ptr[e]; k < ptr[e + 1]; ++k) s += from[src[k]];
    to[e] = s;
  }
}

// ---- apply! -------------------------------------------------------------------------------------
// mean |diag K| in two deterministic levels: every block sums a grid-strided share of the
// columns with a fixed tree (part[block]), then one block sums the partials in block order
constexpr int MD_BLOCK = 256, MD_MAX_BLOCKS = 1024;
__global__ void __launch_bounds__(MD_BLOCK) k_lag_meandiag_part(int n, const int32_t* __restrict__ colptr,
                                                                const int32_t* __restrict__ rowval,
                                                                const double* __restrict__ val,
                                                                double* __restrict__ part) {
  __shared__ double sh[32];
  double s = 0.0;
  for (int j = blockIdx.x * MD_BLOCK + threadIdx.x; j < n; j += gridDim.x * MD_BLOCK)
    for (int e = colptr[j]; e < colptr[j + 1]; ++e)
      if (rowval[e] == j) s += fabs(val[e]);
  s = block_sum<MD_BLOCK>(s, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}
__global__ void __launch_bounds__(MD_MAX_BLOCKS) k_lag_meandiag_final(int n, int nparts, const double* __restrict__ part,
                                                                      double* __restrict__ sc) {
  __shared__ double sh[32];
  double s = (int)threadIdx.x < nparts ? part[threadIdx.x] : 0.0;
  s = block_sum<MD_MAX_BLOCKS>(s, sh);
  if (threadIdx.x == 0) sc[0] = s / n;
}

// b[r] -= sum over prescribed d (increasing) of v_d K[r, d]; K is symmetric, so row r's entries
// are read down column r
__global__ void k_lag_lift(int n, const int32_t* __restrict__ colptr, const int32_t* __restrict__ rowval,
                           const double* __restrict__ val, const uint8_t* __restrict__ pres,
                           const double* __restrict__ gv, double* __restrict__ b) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  double br = b[r];
  for (int e = colptr[r]; e < colptr[r + 1]; ++e) {
    const int d = rowval[e];
    if (pres[d] && gv[d] != 0.0) br -= gv[d] * val[e];
  }
  b[r] = br;
}

__global__ void k_lag_zero(int n, const int32_t* __restrict__ colptr, const int32_t* __restrict__ rowval,
                           double* __restrict__ val, const uint8_t* __restrict__ pres, const double* __restrict__ gv,
                           const double* __restrict__ sc, double* __restrict__ b) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const double m = sc[0];
  for (int e = colptr[j]; e < colptr[j + 1]; ++e) {
    const int r = rowval[e];
    if (pres[r] || pres[j]) val[e] = (r == j) ? m : 0.0;
  }
  if (pres[j]) b[j] = gv[j] * m;
}

__global__ void k_lag_scatter(int nd, const int32_t* __restrict__ dofs, const double* __restrict__ vals,
                              uint8_t* __restrict__ pres, double* __restrict__ gv) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nd) return;
  pres[dofs[k]] = 1;
  gv[dofs[k]] = vals[k];
}

// ---- Jacobi-PCG ---------------------------------------------------------------------------------
// sc: [0] mean diag, [1] b.b, [2] rz of even iterations, [3] rz of odd ones, [4] status
// (0 running, 1 converged, 2 iteration cap, 3 non-finite), [5] iterations, [6] final r.r
// part: [3][nblocks] partial p.q, r.z, r.r
// The per-block partials of the previous kernel, added by warp 0 (lane-strided, then a fixed
// shuffle tree) and handed to the block through shared memory: every block gets the same sums.
// Also reads the status once per block, so that a whole block leaves together.  Contains a
// barrier: call it from every thread of the block.
__device__ __forceinline__ void block_inputs(const double* __restrict__ a, const double* __restrict__ b, int nb,
                                             const double* __restrict__ sc, double* ra, double* rb, double* status) {
  __shared__ double sh[3];
  if (threadIdx.x < 32) {
    double sa = 0.0, sb = 0.0;
    for (int k = threadIdx.x; k < nb; k += 32) {
      sa += a[k];
      if (b) sb += b[k];
    }
    sa = warp_sum(sa);
    sb = warp_sum(sb);
    if (threadIdx.x == 0) {
      sh[0] = sa;
      sh[1] = sb;
      sh[2] = sc[4];
    }
  }
  __syncthreads();
  *ra = sh[0];
  *rb = sh[1];
  *status = sh[2];
}

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double sh[LB / 32];
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int k = 0; k < LB / 32; ++k) t += sh[k];
  return t;  // valid in thread 0
}

__global__ void __launch_bounds__(LB) k_lag_cg_init(int n, const int32_t* __restrict__ colptr,
                                                    const int32_t* __restrict__ rowval, const double* __restrict__ val,
                                                    const double* __restrict__ b, double* __restrict__ x,
                                                    double* __restrict__ r, double* __restrict__ z,
                                                    double* __restrict__ p, double* __restrict__ dinv,
                                                    double* __restrict__ part, int nb) {
  double rz = 0.0, rr = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double d = 0.0;
    for (int e = colptr[i]; e < colptr[i + 1]; ++e)
      if (rowval[e] == i) d = val[e];
    const double di = (d != 0.0) ? 1.0 / d : 1.0;
    dinv[i] = di;
    x[i] = 0.0;
    r[i] = b[i];
    z[i] = di * b[i];
    p[i] = 0.0;
    rz += b[i] * z[i];
    rr += b[i] * b[i];
  }
  rz = block_sum(rz);
  __syncthreads();
  rr = block_sum(rr);
  if (threadIdx.x == 0) {
    part[nb + blockIdx.x] = rz;
    part[2 * nb + blockIdx.x] = rr;
  }
}

// p_new = z + beta p_old, q = K p_new (gathered column by column: K is symmetric), partial p.q.
// Every block adds the previous kernel's partials in the same order, so all blocks agree on
// convergence; block 0 records it.
__global__ void __launch_bounds__(LB) k_lag_cg_a(int n, const int32_t* __restrict__ colptr,
                                                 const int32_t* __restrict__ rowval, const double* __restrict__ val,
                                                 const double* __restrict__ z, const double* __restrict__ pold,
                                                 double* __restrict__ pnew, double* __restrict__ q,
                                                 double* __restrict__ part, double* __restrict__ sc, int nb, int it,
                                                 int maxit, double tol2) {
  double rz, rr, status;
  block_inputs(part + nb, part + 2 * nb, nb, sc, &rz, &rr, &status);
  if (status != 0.0) return;  // uniform in the block
  // the scalar decisions once per block (thread 0), handed out through shared memory: on this
  // part a division per thread costs more FP64 issue than the whole row loop
  __shared__ double sh_beta;
  __shared__ int sh_go;
  if (threadIdx.x == 0) {
    if (it == 0 && blockIdx.x == 0) sc[1] = rr;
    const double bb = (it == 0) ? rr : sc[1];
    int go = 1;
    if (rr <= tol2 * bb || !(rr == rr) || it >= maxit) {
      go = 0;
      if (blockIdx.x == 0) {
        sc[4] = (it >= maxit && rr == rr && !(rr <= tol2 * bb)) ? 2.0 : ((rr == rr) ? 1.0 : 3.0);
        sc[5] = it;
        sc[6] = rr;
      }
    }
    sh_go = go;
    sh_beta = (it == 0) ? 0.0 : rz / sc[2 + ((it - 1) & 1)];
    if (go && blockIdx.x == 0) sc[2 + (it & 1)] = rz;
  }
  __syncthreads();
  if (!sh_go) return;  // uniform in the block
  const double beta = sh_beta;
  double pq = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int e = colptr[i]; e < colptr[i + 1]; ++e) {
      const int k = rowval[e];
      s += val[e] * (z[k] + beta * pold[k]);
    }
    const double pn = z[i] + beta * pold[i];
    pnew[i] = pn;
    q[i] = s;
    pq += pn * s;
  }
  pq = block_sum(pq);
  if (threadIdx.x == 0) part[blockIdx.x] = pq;
}

// alpha = r.z / p.q; x += alpha p, r -= alpha q, z = D^-1 r; partial r.z, r.r
__global__ void __launch_bounds__(LB) k_lag_cg_b(int n, const double* __restrict__ p, const double* __restrict__ q,
                                                 const double* __restrict__ dinv, double* __restrict__ x,
                                                 double* __restrict__ r, double* __restrict__ z,
                                                 double* __restrict__ part, double* __restrict__ sc, int nb, int it) {
  double pq, unused, status;
  block_inputs(part, nullptr, nb, sc, &pq, &unused, &status);
  if (status != 0.0) return;  // uniform in the block
  __shared__ double sh_alpha;
  if (threadIdx.x == 0) sh_alpha = (pq > 0.0) ? sc[2 + (it & 1)] / pq : 0.0;
  __syncthreads();
  const double alpha = sh_alpha;
  double rz = 0.0, rr = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    x[i] += alpha * p[i];
    const double rn = r[i] - alpha * q[i];
    const double zn = dinv[i] * rn;
    r[i] = rn;
    z[i] = zn;
    rz += rn * zn;
    rr += rn * rn;
  }
  rz = block_sum(rz);
  __syncthreads();
  rr = block_sum(rr);
  if (threadIdx.x == 0) {
    part[nb + blockIdx.x] = rz;
    part[2 * nb + blockIdx.x] = rr;
  }
}

// ---- errornorm: per-cell sums, added on the host in cell order ------------------------------------
__global__ void k_lag_errornorm(int nc, int nl, int nq, const double* __restrict__ xy, const int32_t* __restrict__ cells,
                                const int32_t* __restrict__ cdofs, const double* __restrict__ tab,
                                const double* __restrict__ u, int ukind, const double* __restrict__ uprm,
                                double* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const double* N = tab;
  const double* qx = tab + (size_t)nl * nq * 3;
  const double* qy = qx + nq;
  const double* qw = qy + nq;
  const int n0 = cells[3 * c], n1 = cells[3 * c + 1], n2 = cells[3 * c + 2];
  const double x1 = xy[2 * n0], y1 = xy[2 * n0 + 1];
  const double J00 = xy[2 * n1] - x1, J01 = xy[2 * n2] - x1;
  const double J10 = xy[2 * n1 + 1] - y1, J11 = xy[2 * n2 + 1] - y1;
  const double detJ = J00 * J11 - J01 * J10;
  double s = 0.0;
  for (int q = 0; q < nq; ++q) {
    double uh = 0.0;
    for (int i = 0; i < nl; ++i) uh += u[cdofs[(size_t)c * nl + i]] * N[(size_t)i * nq + q];
    const double xi = qx[q], eta = qy[q];
    const double xq = (1.0 - xi - eta) * x1 + xi * xy[2 * n1] + eta * xy[2 * n2];
    const double yq = (1.0 - xi - eta) * y1 + xi * xy[2 * n1 + 1] + eta * xy[2 * n2 + 1];
    const double d = uh - eval_field_kind(ukind, uprm, xq, yq);
    s += d * d * detJ * qw[q];
  }
  out[c] = s;
}

unsigned nblk(int64_t n, int t = 256) { return (unsigned)std::max<int64_t>(1, (n + t - 1) / t); }

// contributions of (cell, i[, j]) to the stored entries / dofs, in cell order
void build_contributions(hdg_lagrange* L, const std::vector<int32_t>& cd) {
  const int nc = L->nc, nl = L->nl;
  const int64_t nnz = L->nnz;
  std::vector<int32_t> cnt(nnz + 1, 0), pos((size_t)nc * nl * nl);
  for (int c = 0; c < nc; ++c)
    for (int i = 0; i < nl; ++i)
      for (int j = 0; j < nl; ++j) {
        const int gi = cd[(size_t)c * nl + i], gj = cd[(size_t)c * nl + j];
        const int32_t* b = L->h_rowval.data() + L->h_colptr[gj];
        const int32_t* e = L->h_rowval.data() + L->h_colptr[gj + 1];
        const int32_t* it = std::lower_bound(b, e, gi);
        if (it == e || *it != gi) throw HdgError{HDG_ERR_ARG, "the sparsity pattern lacks an entry of an element"};
        const int p = (int)(it - L->h_rowval.data());
        pos[((size_t)c * nl + i) * nl + j] = p;
        ++cnt[p + 1];
      }
  for (int64_t p = 0; p < nnz; ++p) cnt[p + 1] += cnt[p];
  std::vector<int32_t> src(cnt[nnz]), fill(cnt.begin(), cnt.end() - 1);
  for (size_t k = 0; k < pos.size(); ++k) src[fill[pos[k]]++] = (int32_t)k;  // k = (c nl + i) nl + j
  cudaStream_t st = L->ctx->stream;
  L->d_gptr.upload(cnt.data(), cnt.size(), st);
  L->d_gsrc.upload(src.data(), src.size(), st);
  const int n = L->ndofs;
  std::vector<int32_t> bc(n + 1, 0);
  for (size_t k = 0; k < cd.size(); ++k) ++bc[cd[k] + 1];
  for (int d = 0; d < n; ++d) bc[d + 1] += bc[d];
  std::vector<int32_t> bsrc(bc[n]), bfill(bc.begin(), bc.end() - 1);
  for (size_t k = 0; k < cd.size(); ++k) bsrc[bfill[cd[k]]++] = (int32_t)k;  // k = c nl + i
  L->d_bptr.upload(bc.data(), bc.size(), st);
  L->d_bsrc.upload(bsrc.data(), bsrc.size(), st);
  HDG_CUDA(cudaStreamSynchronize(st));
}

int lag_fail(hdg_lagrange* L, int code, const char* msg) {
  if (L && L->ctx) L->ctx->err = msg;
  return code;
}

template <class F> int lag_guard(hdg_lagrange* L, F&& fn) {
  try {
    HDG_CUDA(cudaSetDevice(L->ctx->device));
    g_alloc_stream = L->ctx->stream;
    return fn();
  } catch (const HdgError& e) {
    L->ctx->err = e.msg;
    return e.code;
  } catch (const std::bad_alloc&) {
    L->ctx->err = "out of host memory";
    return HDG_ERR_OOM;
  }
}

}  // namespace

extern "C" {

int hdg_lagrange_create(hdg_ctx* ctx, const hdg_mesh* mesh, int order, int quad_degree, int ndofs,
                        const int32_t* cell_dofs, int64_t nnz, const int64_t* colptr, const int64_t* rowval,
                        hdg_lagrange** out) {
  if (!ctx || !mesh || !cell_dofs || !colptr || !rowval || !out || ndofs < 1 || nnz < 1) return HDG_ERR_ARG;
  if (mesh->ctx != ctx) return HDG_ERR_ARG;
  hdg_lagrange* L = new hdg_lagrange();
  L->ctx = ctx;
  const int rc = lag_guard(L, [&]() -> int {
    L->mesh = mesh;
    L->order = order;
    L->qd = quad_degree > 0 ? quad_degree : order + 1;
    if (!build_lagrange_tables(order, L->qd, &L->t))
      throw HdgError{HDG_ERR_BAD_ORDER, "no nodal basis or quadrature rule for this order / degree"};
    L->nl = L->t.nl;
    L->nq = L->t.nq;
    if (L->nl > HDG_LAGRANGE_MAX_NL) throw HdgError{HDG_ERR_ARG, "order too high"};
    L->nc = mesh->nc;
    L->ndofs = ndofs;
    L->nnz = nnz;
    const int nl = L->nl, nc = L->nc;
    std::vector<int32_t> cd((size_t)nc * nl);
    for (size_t k = 0; k < cd.size(); ++k) {
      if (cell_dofs[k] < 1 || cell_dofs[k] > ndofs) throw HdgError{HDG_ERR_ARG, "cell dof out of range"};
      cd[k] = cell_dofs[k] - 1;
    }
    L->h_colptr.resize(ndofs + 1);
    L->h_rowval.resize(nnz);
    for (int j = 0; j <= ndofs; ++j) L->h_colptr[j] = (int32_t)colptr[j];
    for (int64_t e = 0; e < nnz; ++e) L->h_rowval[e] = (int32_t)rowval[e];
    if (L->h_colptr[0] != 0 || L->h_colptr[ndofs] != nnz) throw HdgError{HDG_ERR_ARG, "bad CSC pattern"};
    cudaStream_t st = ctx->stream;
    std::vector<double> tab;
    tab.insert(tab.end(), L->t.N.begin(), L->t.N.end());
    tab.insert(tab.end(), L->t.dN.begin(), L->t.dN.end());
    tab.insert(tab.end(), L->t.qx.begin(), L->t.qx.end());
    tab.insert(tab.end(), L->t.qy.begin(), L->t.qy.end());
    tab.insert(tab.end(), L->t.qw.begin(), L->t.qw.end());
    L->d_tab.upload(tab.data(), tab.size(), st);
    L->d_cdofs.upload(cd.data(), cd.size(), st);
    L->d_colptr.upload(L->h_colptr.data(), L->h_colptr.size(), st);
    L->d_rowval.upload(L->h_rowval.data(), L->h_rowval.size(), st);
    build_contributions(L, cd);
    L->d_ke.alloc((size_t)nc * nl * nl);
    L->d_fe.alloc((size_t)nc * nl);
    L->d_val.alloc(nnz);
    L->d_b.alloc(ndofs);
    L->d_err.alloc(1);
    L->d_sc.alloc(8);
    return HDG_OK;
  });
  if (rc != HDG_OK) {
    delete L;
    return rc;
  }
  *out = L;
  return HDG_OK;
}

int hdg_lagrange_assemble(hdg_lagrange* L, const hdg_field* f, const double* kappa_cell) {
  if (!L) return HDG_ERR_ARG;
  return lag_guard(L, [&]() -> int {
    cudaStream_t st = L->ctx->stream;
    const FieldSpec fs = field_from(f, 0.0);
    L->d_fprm.upload(fs.prm.data(), fs.prm.size(), st);
    if (kappa_cell) L->d_kappa.upload(kappa_cell, (size_t)L->nc, st);
    HDG_CUDA(cudaMemsetAsync(L->d_err.p, 0, sizeof(int), st));
    k_lag_element<<<nblk((int64_t)L->nc * L->nl), 256, 0, st>>>(
        L->nc, L->nl, L->nq, L->mesh->d_xy.p, L->mesh->d_cells.p, L->d_tab.p, fs.kind, L->d_fprm.p,
        kappa_cell ? L->d_kappa.p : nullptr, L->d_ke.p, L->d_fe.p, L->d_err.p);
    k_lag_gather<<<std::min<unsigned>(nblk(L->nnz), 152 * 16), 256, 0, st>>>(L->nnz, L->d_gptr.p, L->d_gsrc.p,
                                                                            L->d_ke.p, L->d_val.p);
    k_lag_gather<<<std::min<unsigned>(nblk(L->ndofs), 152 * 16), 256, 0, st>>>(L->ndofs, L->d_bptr.p, L->d_bsrc.p,
                                                                              L->d_fe.p, L->d_b.p);
    HDG_CUDA(cudaGetLastError());
    L->ctx->launches += 3;
    int err = 0;
    HDG_CUDA(cudaMemcpyAsync(&err, L->d_err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    HDG_CUDA(cudaStreamSynchronize(st));
    if (err & 1) return lag_fail(L, HDG_ERR_NEG_DETJ, "det(J) is not positive on some cell");
    L->assembled = true;
    L->applied = false;
    L->solved = false;
    return HDG_OK;
  });
}

int hdg_lagrange_get_csc(hdg_lagrange* L, double* nzval, double* rhs) {
  if (!L || !L->assembled) return HDG_ERR_ARG;
  return lag_guard(L, [&]() -> int {
    cudaStream_t st = L->ctx->stream;
    if (nzval) L->d_val.download(nzval, (size_t)L->nnz, st);
    if (rhs) L->d_b.download(rhs, (size_t)L->ndofs, st);
    HDG_CUDA(cudaStreamSynchronize(st));
    return HDG_OK;
  });
}

int hdg_lagrange_apply_dirichlet(hdg_lagrange* L, const int32_t* dofs, const double* vals, int n) {
  if (!L || n < 0 || (n > 0 && (!dofs || !vals))) return HDG_ERR_ARG;
  if (!L->assembled) return lag_fail(L, HDG_ERR_ARG, "assemble first");
  if (L->applied) return lag_fail(L, HDG_ERR_ARG, "apply! was already called on this system");
  return lag_guard(L, [&]() -> int {
    cudaStream_t st = L->ctx->stream;
    const int nd = L->ndofs;
    std::vector<int32_t> d0(n);
    for (int k = 0; k < n; ++k) {
      if (dofs[k] < 1 || dofs[k] > nd) throw HdgError{HDG_ERR_ARG, "prescribed dof out of range"};
      d0[k] = dofs[k] - 1;
    }
    L->d_pres.alloc(nd);
    L->d_gv.alloc(nd);
    HDG_CUDA(cudaMemsetAsync(L->d_pres.p, 0, nd, st));
    HDG_CUDA(cudaMemsetAsync(L->d_gv.p, 0, sizeof(double) * nd, st));
    DevBuf<int32_t> dd;
    DevBuf<double> dv;
    if (n > 0) {
      dd.upload(d0.data(), n, st);
      dv.upload(vals, n, st);
      k_lag_scatter<<<nblk(n), 256, 0, st>>>(n, dd.p, dv.p, L->d_pres.p, L->d_gv.p);
    }
    {
      const int nparts = (int)std::min<int64_t>(std::max<int64_t>(((int64_t)nd + MD_BLOCK - 1) / MD_BLOCK, 1),
                                                 MD_MAX_BLOCKS);
      DevBuf<double> part;
      part.alloc((size_t)nparts);
      k_lag_meandiag_part<<<nparts, MD_BLOCK, 0, st>>>(nd, L->d_colptr.p, L->d_rowval.p, L->d_val.p, part.p);
      k_lag_meandiag_final<<<1, MD_MAX_BLOCKS, 0, st>>>(nd, nparts, part.p, L->d_sc.p);
      L->ctx->launches++;
    }
    k_lag_lift<<<nblk(nd), 256, 0, st>>>(nd, L->d_colptr.p, L->d_rowval.p, L->d_val.p, L->d_pres.p, L->d_gv.p,
                                         L->d_b.p);
    k_lag_zero<<<nblk(nd), 256, 0, st>>>(nd, L->d_colptr.p, L->d_rowval.p, L->d_val.p, L->d_pres.p, L->d_gv.p,
                                         L->d_sc.p, L->d_b.p);
    HDG_CUDA(cudaGetLastError());
    L->ctx->launches += n > 0 ? 4 : 3;
    HDG_CUDA(cudaStreamSynchronize(st));
    L->applied = true;
    return HDG_OK;
  });
}

int hdg_lagrange_solve(hdg_lagrange* L, const hdg_solver* opts, double* u, hdg_stats* stats) {
  if (!L || !L->assembled) return HDG_ERR_ARG;
  return lag_guard(L, [&]() -> int {
    const double tol = (opts && opts->tol > 0) ? opts->tol : 1e-12;
    const int maxit = (opts && opts->maxit > 0) ? opts->maxit : 100000;
    cudaStream_t st = L->ctx->stream;
    const int n = L->ndofs;
    const int nb = (int)std::min<int64_t>(nblk(n, LB), LMAX_BLOCKS);
    L->d_x.alloc(n); L->d_r.alloc(n); L->d_z.alloc(n); L->d_p.alloc(n); L->d_p2.alloc(n); L->d_q.alloc(n);
    L->d_dinv.alloc(n);
    L->d_part.alloc((size_t)3 * nb);
    HDG_CUDA(cudaMemsetAsync(L->d_sc.p + 1, 0, sizeof(double) * 7, st));
    k_lag_cg_init<<<nb, LB, 0, st>>>(n, L->d_colptr.p, L->d_rowval.p, L->d_val.p, L->d_b.p, L->d_x.p, L->d_r.p,
                                     L->d_z.p, L->d_p.p, L->d_dinv.p, L->d_part.p, nb);
    L->ctx->launches++;
    constexpr int CHUNK = 32;
    double sc[8];
    int it = 0;
    for (;;) {
      for (int k = 0; k < CHUNK; ++k, ++it) {
        double* pold = (it & 1) ? L->d_p2.p : L->d_p.p;
        double* pnew = (it & 1) ? L->d_p.p : L->d_p2.p;
        k_lag_cg_a<<<nb, LB, 0, st>>>(n, L->d_colptr.p, L->d_rowval.p, L->d_val.p, L->d_z.p, pold, pnew, L->d_q.p,
                                      L->d_part.p, L->d_sc.p, nb, it, maxit, tol * tol);
        k_lag_cg_b<<<nb, LB, 0, st>>>(n, pnew, L->d_q.p, L->d_dinv.p, L->d_x.p, L->d_r.p, L->d_z.p, L->d_part.p,
                                      L->d_sc.p, nb, it);
      }
      HDG_CUDA(cudaGetLastError());
      L->ctx->launches += 2 * CHUNK;
      HDG_CUDA(cudaMemcpyAsync(sc, L->d_sc.p, sizeof(sc), cudaMemcpyDeviceToHost, st));
      HDG_CUDA(cudaStreamSynchronize(st));
      if (sc[4] != 0.0) break;
    }
    const int status = (int)sc[4];
    if (stats) {
      stats->iterations = (int)sc[5];
      stats->outer = 1;
      stats->converged = (status == 1) ? 1 : 0;
      stats->rel_residual = sc[1] > 0.0 ? std::sqrt(sc[6] / sc[1]) : 0.0;
    }
    if (u) {
      L->d_x.download(u, (size_t)n, st);
      HDG_CUDA(cudaStreamSynchronize(st));
    }
    L->solved = true;
    if (status == 2) return lag_fail(L, HDG_ERR_NO_CONVERGENCE, "CG did not reach the tolerance within maxit");
    if (status == 3) return lag_fail(L, HDG_ERR_BREAKDOWN, "CG breakdown (non-finite residual)");
    return HDG_OK;
  });
}

int hdg_lagrange_errornorm_l2sq(hdg_lagrange* L, const double* u, const hdg_field* u_exact, double* out) {
  if (!L || !u_exact || !out) return HDG_ERR_ARG;
  if (!u && !L->solved) return lag_fail(L, HDG_ERR_ARG, "solve first or pass the dof values");
  return lag_guard(L, [&]() -> int {
    cudaStream_t st = L->ctx->stream;
    DevBuf<double> du, prm, cellv;
    if (u) du.upload(u, (size_t)L->ndofs, st);
    const FieldSpec fs = field_from(u_exact, 0.0);
    prm.upload(fs.prm.data(), fs.prm.size(), st);
    cellv.alloc(L->nc);
    k_lag_errornorm<<<nblk(L->nc), 256, 0, st>>>(L->nc, L->nl, L->nq, L->mesh->d_xy.p, L->mesh->d_cells.p,
                                                 L->d_cdofs.p, L->d_tab.p, u ? du.p : L->d_x.p, fs.kind, prm.p,
                                                 cellv.p);
    HDG_CUDA(cudaGetLastError());
    L->ctx->launches++;
    std::vector<double> h(L->nc);
    cellv.download(h.data(), h.size(), st);
    HDG_CUDA(cudaStreamSynchronize(st));
    double s = 0.0;
    for (double v : h) s += v;
    *out = s;
    return HDG_OK;
  });
}

int hdg_lagrange_destroy(hdg_lagrange* L) {
  if (!L) return HDG_OK;
  cudaSetDevice(L->ctx->device);
  delete L;
  return HDG_OK;
}

}  // extern "C"
