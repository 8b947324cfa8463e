// Element assembly + static condensation (the body of doassemble,
// examples/poisson2D_HDG.jl:77-174), one warp per cell.
//
// Per cell the warp
//   1. gathers the three vertices and forms J, det J, adj(J) = det J * J^-1, the weighted
//      outward normals wn_f (|wn_f| = |e_f|) and the orientation bits (src/mesh.jl:51-54);
//   2. writes the augmented local system [Me | EF | Bte] of size n x (n+m+1) into shared memory,
//      Me = [Ae -Be; Be' Ce], EF = [-Ee; Fe], Bte = [0; be], every block being a combination
//      of the packed reference matrices of tables.cpp (no per-point basis loops);
//   3. eliminates with partial pivoting (the LU of `factorize`, :160) and back-substitutes all
//      m+1 right-hand sides: X = [K_e | b_e] (:171,:173);
//   4. forms [Ate | bte] = [Ee;Fe]' X - [He | 0] through the factorised form of Ee and Fe
//      (Ee = wn_f (x) F_{f,o}, Fe = tau |e_f| F_{f,o}), with bte = -[Ee;Fe]' b_e (:172,:174).
// Outputs per cell: AB = [Ate | bte] (m x (m+1)) and KB = [K_e | b_e] (n x (m+1)), row-major.
#include <map>
#include <mutex>
#include <tuple>
#include <cstdlib>
#include "hdg_device.cuh"

namespace {

struct ElemArgs {
  const double* xy;
  const int32_t* cells;
  const uint8_t* orient;
  const double* ref;
  int ref_len, nq;
  int nc;
  CoefDev co;      // per-problem source, coefficient and tau (one problem unless batched)
  int kappa_mode;  // 0: kappa = 1, 1: per-cell array, 2: per-problem field
  const double* kcell;
  double* AB;
  double* KB;
  int* err;
  int schur;  // 1: the Schur-complement path (invertible reference mass, kappa constant per cell)
  int he_tau; // 1: He carries tau
  RefLayout L;  // offsets of the packed reference tables (tables.cpp: ref_layout)
};

// One warp per cell; EWARPS warps (cells) per CTA, picked per degree, quadrature size and mesh
// size by the launch-time autotuner below.  This is the general path (any quadrature, kappa as a
// field): the full augmented system, eliminated with partial pivoting.
template <int P, int EWARPS>
__global__ void __launch_bounds__(EWARPS * 32) k_element_condense(ElemArgs a) {
  using D = Dims<P>;
  constexpr int NW = D::NW, NT = D::NT, NV = D::NV, N = D::N, M = D::M, NC = D::NC;
  // Per-warp scratch: the augmented system [Me | EF | Bte] (row stride D::LD, solution X in
  // columns N..N+M).
  constexpr int LDW = D::LD;
  constexpr int XO = N;  // first column of X
  extern __shared__ double smem[];
  double* ref = smem;
  const int nq = a.nq;
  const RefLayout L = a.L;
  // the tables this path reads, [M .. Q], sit at the start of the packed table
  const int ref_len = a.ref_len;
  for (int i = threadIdx.x; i < ref_len; i += blockDim.x) ref[i] = a.ref[i];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wstride = N * LDW + 2 * nq + NW + N + 2;
  double* W = smem + ((ref_len + 1) & ~1) + warp * wstride;
  double* sq = W + N * LDW;  // per-warp scratch: f (or kappa^-1) at the quadrature points, be
  __syncthreads();

  for (int e = blockIdx.x * EWARPS + warp; e < a.nc; e += gridDim.x * EWARPS) {
    // ---- geometry (reinit!, src/ScalarFunctionSpaces.jl:101-132) -------------------------
    int nid = (lane < 3) ? a.cells[3 * e + lane] : 0;
    double px = 0.0, py = 0.0;
    if (lane < 3) {
      px = a.xy[2 * nid];
      py = a.xy[2 * nid + 1];
    }
    const double x1 = __shfl_sync(0xffffffffu, px, 0), y1 = __shfl_sync(0xffffffffu, py, 0);
    const double x2 = __shfl_sync(0xffffffffu, px, 1), y2 = __shfl_sync(0xffffffffu, py, 1);
    const double x3 = __shfl_sync(0xffffffffu, px, 2), y3 = __shfl_sync(0xffffffffu, py, 2);
    const double J00 = x2 - x1, J01 = x3 - x1, J10 = y2 - y1, J11 = y3 - y1;
    const double detJ = J00 * J11 - J01 * J10;
    if (!(detJ > 0.0) && lane == 0) atomicOr(a.err, 1);
    // adj(J) = detJ * J^-1 ; Be[(c,a),j] = sum_l adj[l][c] D_l[a][j]
    const double ad00 = J11, ad01 = -J01, ad10 = -J10, ad11 = J00;
    // weighted normals (src/shapes.jl:80-87)
    double wn[3][2] = {{-(J10 - J11), J00 - J01}, {-J11, J01}, {J10, -J00}};
    double el[3];
#pragma unroll
    for (int f = 0; f < 3; ++f) el[f] = sqrt(wn[f][0] * wn[f][0] + wn[f][1] * wn[f][1]);
    const unsigned ob = a.orient[e];
    const int prob = a.co.cell_prob[e];
    const double tau = a.co.tau[prob];
    const int fkind = a.co.fkind[prob];
    const double* fprm = a.co.fprep + a.co.foff[prob];
    double kinv = 1.0;
    if (a.kappa_mode == 1) kinv = 1.0 / a.kcell[e];
    const double smass = kinv * detJ;
    // ---- source (and kappa field) at the volume points -----------------------------------
    for (int q = lane; q < nq; q += 32) {
      double xi = ref[L.Q + 2 * q], eta = ref[L.Q + 2 * q + 1];
      double xq = (1.0 - xi - eta) * x1 + xi * x2 + eta * x3;
      double yq = (1.0 - xi - eta) * y1 + xi * y2 + eta * y3;
      sq[q] = eval_source_prepared(fkind, fprm, xq, yq);
      if (a.kappa_mode == 2) sq[nq + q] = 1.0 / eval_field_kind(a.co.kkind[prob], a.co.kprm + a.co.koff[prob], xq, yq);
    }
    __syncwarp();
    double* be = sq + 2 * nq;
    for (int i = lane; i < NW; i += 32) {
      double s = 0.0;
      for (int q = 0; q < nq; ++q) s += ref[L.NW + i * nq + q] * sq[q];
      be[i] = s * detJ;
    }
    __syncwarp();
    // ---- augmented local system ----------------------------------------------------------
    for (int idx = lane; idx < N * NC; idx += 32) {
      const int r = idx / NC, col = idx - (idx / NC) * NC;
      double v;
      if (r < NV) {
        const int c = r / NW, ia = r - c * NW;
        const double adl0 = c ? ad01 : ad00, adl1 = c ? ad11 : ad10;
        if (col < NV) {
          const int c2 = col / NW, ib = col - c2 * NW;
          if (c2 != c) {
            v = 0.0;
          } else if (a.kappa_mode == 2) {
            double s = 0.0;
            for (int q = 0; q < nq; ++q) s += ref[L.NW + ia * nq + q] * sq[nq + q] * ref[L.N + ib * nq + q];
            v = s * detJ;
          } else {
            v = smass * ref[L.M + ia * NW + ib];
          }
        } else if (col < N) {
          const int j = col - NV;
          v = -(adl0 * ref[L.D0 + ia * NW + j] + adl1 * ref[L.D1 + ia * NW + j]);
        } else if (col < N + M) {
          const int f = (col - N) / NT, j = (col - N) - f * NT;
          const int o = (ob >> f) & 1;
          v = -wn[f][c] * ref[L.F + ((f * 2 + o) * NW + ia) * NT + j];
        } else {
          v = 0.0;
        }
      } else {
        const int ia = r - NV;
        if (col < NV) {
          const int c2 = col / NW, ib = col - c2 * NW;
          const double adl0 = c2 ? ad01 : ad00, adl1 = c2 ? ad11 : ad10;
          v = adl0 * ref[L.D0 + ib * NW + ia] + adl1 * ref[L.D1 + ib * NW + ia];
        } else if (col < N) {
          const int ib = col - NV;
          v = tau * (el[0] * ref[L.C + (0 * NW + ia) * NW + ib] + el[1] * ref[L.C + (1 * NW + ia) * NW + ib] +
                     el[2] * ref[L.C + (2 * NW + ia) * NW + ib]);
        } else if (col < N + M) {
          const int f = (col - N) / NT, j = (col - N) - f * NT;
          const int o = (ob >> f) & 1;
          v = tau * el[f] * ref[L.F + ((f * 2 + o) * NW + ia) * NT + j];
        } else {
          v = be[ia];
        }
      }
      W[r * LDW + col] = v;
    }
    __syncwarp();
    // ---- Gaussian elimination with partial pivoting --------------------------------------
    // The pivot search compares |a_ik| through its bit pattern: for non-negative IEEE doubles
    // the unsigned-integer order of the bits is the numeric order, so the search runs on the
    // integer pipe instead of the (narrow) FP64 pipe.  Ties keep the smallest row, as idamax.
    double* rinv = be + NW;  // reciprocals of the pivots, reused by the back substitution
    for (int k = 0; k < N; ++k) {
      unsigned long long best = 0ull;
      int bi = N;
      for (int i = k + lane; i < N; i += 32) {
        const unsigned long long v = (unsigned long long)__double_as_longlong(W[i * LDW + k]) & 0x7fffffffffffffffull;
        if (v > best || (v == best && i < bi)) { best = v; bi = i; }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long ov = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
      }
      if (best == 0ull && lane == 0) atomicOr(a.err, 2);
      if (bi != k) {
        for (int j = k + lane; j < NC; j += 32) {
          double t = W[k * LDW + j];
          W[k * LDW + j] = W[bi * LDW + j];
          W[bi * LDW + j] = t;
        }
        __syncwarp();
      }
      const double pinv = 1.0 / W[k * LDW + k];
      if (lane == 0) rinv[k] = pinv;
      for (int i = k + 1 + lane; i < N; i += 32) W[i * LDW + k] *= pinv;
      __syncwarp();
      const int cols = NC - k - 1, rows = N - k - 1;
      for (int t = lane; t < rows * cols; t += 32) {
        const int i = k + 1 + t / cols, j = k + 1 + (t - (t / cols) * cols);
        W[i * LDW + j] -= W[i * LDW + k] * W[k * LDW + j];
      }
      __syncwarp();
    }
    // ---- back substitution on the m+1 right-hand sides -----------------------------------
    for (int k = N - 1; k >= 0; --k) {
      const double dinv = rinv[k];
      for (int j = lane; j <= M; j += 32) W[k * LDW + N + j] *= dinv;
      __syncwarp();
      for (int t = lane; t < k * (M + 1); t += 32) {
        const int i = t / (M + 1), j = t - (t / (M + 1)) * (M + 1);
        W[i * LDW + N + j] -= W[i * LDW + k] * W[k * LDW + N + j];
      }
      __syncwarp();
    }
    // ---- K_e, b_e out; Y_f = wn_f,x X_qx + wn_f,y X_qy + tau |e_f| X_u into the free columns --
    double* KB = a.KB + (size_t)e * N * (M + 1);
    for (int t = lane; t < N * (M + 1); t += 32) {
      const int r = t / (M + 1), j = t - (t / (M + 1)) * (M + 1);
      KB[t] = W[r * LDW + XO + j];
    }
    for (int t = lane; t < 3 * NW * (M + 1); t += 32) {
      const int fa = t / (M + 1), j = t - (t / (M + 1)) * (M + 1);
      const int f = fa / NW, ia = fa - f * NW;
      W[fa * LDW + j] = wn[f][0] * W[ia * LDW + XO + j] + wn[f][1] * W[(NW + ia) * LDW + XO + j] +
                       tau * el[f] * W[(NV + ia) * LDW + XO + j];
    }
    __syncwarp();
    // ---- [Ate | bte] ----------------------------------------------------------------------
    double* AB = a.AB + (size_t)e * M * (M + 1);
    for (int t = lane; t < M * (M + 1); t += 32) {
      const int row = t / (M + 1), col = t - (t / (M + 1)) * (M + 1);
      const int f = row / NT, i = row - f * NT;
      const int o = (ob >> f) & 1;
      const double* F = ref + L.F + (f * 2 + o) * NW * NT;
      double s = 0.0;
#pragma unroll
      for (int ia = 0; ia < NW; ++ia) s += F[ia * NT + i] * W[(f * NW + ia) * LDW + col];
      double v;
      if (col < M) {
        const int g = col / NT, j = col - g * NT;
        v = (g == f) ? s - (a.he_tau ? tau : 1.0) * el[f] * ref[L.H + i * NT + j] : s;
      } else {
        v = -s;
      }
      AB[t] = v;
    }
    __syncwarp();
  }
}

// Schur path with an LDL' factorisation: invertible reference mass and kappa constant on each
// cell (p = 1, and p = 3, 4 with exact-enough rules).  Then Ae = (det J / kappa) diag(M, M) is
// inverted in closed form, and with kf = kappa / det J the condensation needs only the nw x nw
// Schur complement
//   S  = C + kf sum_c B_c' M^-1 B_c = C + kf (a00 Q00 + a01 (Q01 + Q01') + a11 Q11)    (SPD)
//   R' = [R'_f] with R'_f = tau |e_f| F_{f,o} + kf (b0_f DMF0_{f,o} + b1_f DMF1_{f,o}), and be,
// where B_c = adl0_c D0 + adl1_c D1, b_l f = adj(J) row l . wn_f.  Writing S = U' D U (U unit
// upper triangular) and R~ = U'^-1 [R' | be], the condensed blocks are
//   Ate_{fi,gj} = (R~' D^-1 R~)_{fi,gj} - kf (wn_f . wn_g) (F_{f,o}' M^-1 F_{g,o'})_{ij} - [f = g] |e_f| He_ij
//   bte_{fi}    = -(R~' D^-1 R~)_{fi,be}
// (the same Ate = [Ee;Fe]' Me^-1 [-Ee;Fe] - He and bte = -[Ee;Fe]' Me^-1 [0;be] that the full
// elimination of examples/poisson2D_HDG.jl:155-174 forms, reordered), symmetric by construction, so
// only the upper triangle is computed.  The u rows of [K_e | b_e], X_u = U^-1 D^-1 R~, are stored;
// the q rows follow linearly from them, q = kf (adl0 M^-1 D0 u + adl1 M^-1 D1 u - sum_f wn_f M^-1
// F_f u_hat_f), and are formed at recovery (k_recover_u) or when the blocks are exported
// (k_expand_ke).  Per cell at p = 4 this is about 8k FP64 FMAs instead of the 20k of the pivoted
// elimination of S with the q rows, and 3.8 KB written instead of 7.7 KB.  The kernel is bound by
// the FP64 pipe, which counts warp instructions: the pivots need no square root, their
// reciprocals come from recip_newton, and the bump source's -1/(2 s^2) is formed on the host.
// v[f] for a face index f known only at run time, without indexing a local array (which would
// place the array in local memory)
__device__ __forceinline__ double sel3(int f, double v0, double v1, double v2) {
  return f == 0 ? v0 : (f == 1 ? v1 : v2);
}

template <int P, int EWARPS>
__global__ void __launch_bounds__(EWARPS * 32) k_element_chol(ElemArgs a) {
  using D = Dims<P>;
  constexpr int NW = D::NW, NT = D::NT, M = D::M;
  constexpr int RC = NW + M + 1;  // columns of [S | R' | be]
  constexpr int LDW = RC | 1;     // odd row stride: conflict-free FP64 column reads
  extern __shared__ double smem[];
  const int nq = a.nq;
  const RefLayout G = a.L;
  // staged tables: [C .. Q] (C, F, H, N w, points), [Q00 Q01 Q11], [DMF .. PFF]
  const int n1 = G.Q + 2 * nq - G.C, n2 = 3 * NW * NW, n3 = G.PFF + 36 * NT * NT - G.SDMF;
  for (int i = threadIdx.x; i < n1; i += blockDim.x) smem[i] = a.ref[G.C + i];
  for (int i = threadIdx.x; i < n2; i += blockDim.x) smem[n1 + i] = a.ref[G.SQ00 + i];
  for (int i = threadIdx.x; i < n3; i += blockDim.x) smem[n1 + n2 + i] = a.ref[G.SDMF + i];
  const double* Cf = smem;                       // [3][NW][NW]
  const double* Ff = smem + (G.F - G.C);         // [6][NW][NT]   (f, o)
  const double* Hh = smem + (G.H - G.C);         // [NT][NT]
  const double* Nw = smem + (G.NW - G.C);        // [NW][nq]      N times the weights
  const double* Qp = smem + (G.Q - G.C);         // [nq][2]
  const double* SQ = smem + n1;                  // [3][NW][NW]   Q00, Q01, Q11
  const double* DMF = smem + n1 + n2;            // [2][6][NW][NT]
  const double* PFF = DMF + 12 * NW * NT;        // [6][6][NT][NT]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wstride = ((NW * LDW + NW * (M + 1) + nq + 2 * NW) + 1) & ~1;
  double* W = smem + ((n1 + n2 + n3 + 1) & ~1) + warp * wstride;
  double* Y = W + NW * LDW;   // D^-1 R~ (NW x (M+1))
  double* sq = Y + NW * (M + 1);  // f at the quadrature points
  double* be = sq + nq;
  double* rinv = be + NW;     // 1 / d_k
  __syncthreads();

  for (int e = blockIdx.x * EWARPS + warp; e < a.nc; e += gridDim.x * EWARPS) {
    // ---- geometry (reinit!, src/ScalarFunctionSpaces.jl:101-132) -------------------------
    int nid = (lane < 3) ? a.cells[3 * e + lane] : 0;
    double px = 0.0, py = 0.0;
    if (lane < 3) {
      px = a.xy[2 * nid];
      py = a.xy[2 * nid + 1];
    }
    const double x1 = __shfl_sync(0xffffffffu, px, 0), y1 = __shfl_sync(0xffffffffu, py, 0);
    const double x2 = __shfl_sync(0xffffffffu, px, 1), y2 = __shfl_sync(0xffffffffu, py, 1);
    const double x3 = __shfl_sync(0xffffffffu, px, 2), y3 = __shfl_sync(0xffffffffu, py, 2);
    const double J00 = x2 - x1, J01 = x3 - x1, J10 = y2 - y1, J11 = y3 - y1;
    const double detJ = J00 * J11 - J01 * J10;
    if (!(detJ > 0.0) && lane == 0) atomicOr(a.err, 1);
    const double ad00 = J11, ad01 = -J01, ad10 = -J10, ad11 = J00;  // adj(J) = det J J^-1
    const double wn[3][2] = {{-(J10 - J11), J00 - J01}, {-J11, J01}, {J10, -J00}};  // src/shapes.jl:80-87
    double el[3];
#pragma unroll
    for (int f = 0; f < 3; ++f) el[f] = sqrt(wn[f][0] * wn[f][0] + wn[f][1] * wn[f][1]);
    const unsigned ob = a.orient[e];
    const int prob = a.co.cell_prob[e];
    const double tau = a.co.tau[prob];
    const double hs = a.he_tau ? tau : 1.0;
    const int fkind = a.co.fkind[prob];
    const double* fprm = a.co.fprep + a.co.foff[prob];
    const double kinv = (a.kappa_mode == 1) ? 1.0 / a.kcell[e] : 1.0;
    const double kf = 1.0 / (kinv * detJ);
    // ---- source at the volume points, be ----------------------------------------------------
    for (int q = lane; q < nq; q += 32) {
      const double xi = Qp[2 * q], eta = Qp[2 * q + 1];
      const double xq = (1.0 - xi - eta) * x1 + xi * x2 + eta * x3;
      const double yq = (1.0 - xi - eta) * y1 + xi * y2 + eta * y3;
      sq[q] = eval_source_prepared(fkind, fprm, xq, yq);
    }
    __syncwarp();
    for (int i = lane; i < NW; i += 32) {
      double t = 0.0;
      for (int q = 0; q < nq; ++q) t += Nw[i * nq + q] * sq[q];
      be[i] = t * detJ;
    }
    __syncwarp();
    // ---- [S (upper triangle) | R' | be] ------------------------------------------------------
    const double a00 = ad00 * ad00 + ad01 * ad01, a11 = ad10 * ad10 + ad11 * ad11, a01 = ad00 * ad10 + ad01 * ad11;
    double b0f[3], b1f[3];
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      b0f[f] = ad00 * wn[f][0] + ad01 * wn[f][1];
      b1f[f] = ad10 * wn[f][0] + ad11 * wn[f][1];
    }
    for (int idx = lane; idx < NW * RC; idx += 32) {
      const int ia = idx / RC, col = idx - ia * RC;
      double v;
      if (col < NW) {
        if (col < ia) continue;  // lower triangle of S: never read
        const int ib = col;
        v = tau * (el[0] * Cf[(0 * NW + ia) * NW + ib] + el[1] * Cf[(1 * NW + ia) * NW + ib] +
                   el[2] * Cf[(2 * NW + ia) * NW + ib]) +
            kf * (a00 * SQ[ia * NW + ib] + a01 * (SQ[NW * NW + ia * NW + ib] + SQ[NW * NW + ib * NW + ia]) +
                  a11 * SQ[2 * NW * NW + ia * NW + ib]);
      } else if (col < NW + M) {
        const int f = (col - NW) / NT, j = (col - NW) - f * NT;
        const int fo = f * 2 + ((ob >> f) & 1);
        v = tau * sel3(f, el[0], el[1], el[2]) * Ff[(fo * NW + ia) * NT + j] +
            kf * (sel3(f, b0f[0], b0f[1], b0f[2]) * DMF[((0 * 6 + fo) * NW + ia) * NT + j] +
                  sel3(f, b1f[0], b1f[1], b1f[2]) * DMF[((1 * 6 + fo) * NW + ia) * NT + j]);
      } else {
        v = be[ia];
      }
      W[ia * LDW + col] = v;
    }
    __syncwarp();
    // ---- S = U' D U (LDL', no square roots), carrying the right-hand sides ---------------------
    // Elimination without pivoting (S is SPD): after step k, row k holds d_k and d_k U_k., and the
    // right-hand sides R~ = (D U)'^-1 ... = L^-1 [R' | be]; Y = D^-1 R~ (row k scaled when it is
    // final).  Lane l owns column j = k+1+l (RC - k - 1 <= 31 columns: one pass).
    static_assert(RC <= 32, "one lane per column of [S | R' | be]");
    for (int k = 0; k < NW; ++k) {
      const double d = W[k * LDW + k];
      if (!(d > 0.0) && lane == 0) atomicOr(a.err, 2);  // not positive definite (LAPACK PosDefException)
      const double r = recip_newton(d);
      const int j = k + 1 + lane;
      if (lane == 0) rinv[k] = r;
      if (j < RC) {
        const double t = W[k * LDW + j] * r;
        if (j >= NW) Y[k * (M + 1) + (j - NW)] = t;
#pragma unroll 4
        for (int i = k + 1; i < NW; ++i)
          if (j >= i) W[i * LDW + j] -= W[k * LDW + i] * t;
      }
      __syncwarp();
    }
    // ---- [Ate | bte] from Z'Z (upper triangle and the be column), then the face-face term and He
    double* AB = a.AB + (size_t)e * M * (M + 1);
    constexpr int NPAIR = M * (M + 1) / 2 + M;
    for (int t = lane; t < NPAIR; t += 32) {
      int r = 0, rem = t;
      while (rem >= M - r + 1) {  // row r holds columns r..M-1 and the be column
        rem -= M - r + 1;
        ++r;
      }
      const int c = (rem == M - r) ? M : r + rem;
      double dot = 0.0;  // (R~' D^-1 R~)_rc = (R' S^-1 R')_rc
#pragma unroll
      for (int ia = 0; ia < NW; ++ia) dot += Y[ia * (M + 1) + r] * W[ia * LDW + NW + c];
      if (c == M) {
        AB[r * (M + 1) + M] = -dot;
      } else {
        const int f = r / NT, i = r - f * NT, g = c / NT, j = c - g * NT;
        const int fo = f * 2 + ((ob >> f) & 1), go = g * 2 + ((ob >> g) & 1);
        const double wfx = sel3(f, wn[0][0], wn[1][0], wn[2][0]), wfy = sel3(f, wn[0][1], wn[1][1], wn[2][1]);
        const double wgx = sel3(g, wn[0][0], wn[1][0], wn[2][0]), wgy = sel3(g, wn[0][1], wn[1][1], wn[2][1]);
        double v = dot - kf * (wfx * wgx + wfy * wgy) * PFF[((fo * 6 + go) * NT + i) * NT + j];
        if (f == g) v -= hs * sel3(f, el[0], el[1], el[2]) * Hh[i * NT + j];
        AB[r * (M + 1) + c] = v;
        if (c != r) AB[c * (M + 1) + r] = v;
      }
    }
    __syncwarp();
    // ---- X_u = U^-1 Y: lane j <= m owns column j; the back substitution runs in its registers,
    // and each row of X_u goes out as one coalesced store of m+1 values --------------------------
    if (lane <= M) {
      double x[NW];
#pragma unroll
      for (int k = NW - 1; k >= 0; --k) {
        double t = 0.0;
#pragma unroll
        for (int i = k + 1; i < NW; ++i) t += W[k * LDW + i] * x[i];
        x[k] = Y[k * (M + 1) + lane] - rinv[k] * t;
      }
      double* KB = a.KB + (size_t)e * NW * (M + 1);
#pragma unroll
      for (int ia = 0; ia < NW; ++ia) KB[ia * (M + 1) + lane] = x[ia];
    }
    __syncwarp();
  }
}

// The q rows of [K_e | b_e] from the stored u rows (the Cholesky-Schur path stores X_u only):
// X_q,c = kf (adl0_c M^-1 D0 X_u + adl1_c M^-1 D1 X_u - [j < m] wn_f,c M^-1 F_{f,o}), one thread per
// entry of the full n x (m+1) block.  Used when the blocks are exported, not on the solve path.
template <int P>
__global__ void k_expand_ke(ElemArgs a, const double* __restrict__ KBu, double* __restrict__ KB) {
  using D = Dims<P>;
  constexpr int NW = D::NW, NT = D::NT, NV = D::NV, N = D::N, M = D::M;
  const RefLayout G = a.L;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)a.nc * N * (M + 1)) return;
  const int e = (int)(t / (N * (M + 1)));
  const int rj = (int)(t - (int64_t)e * N * (M + 1));
  const int r = rj / (M + 1), j = rj - r * (M + 1);
  const double* Xu = KBu + (size_t)e * NW * (M + 1);
  if (r >= NV) {
    KB[t] = Xu[(r - NV) * (M + 1) + j];
    return;
  }
  const int n0 = a.cells[3 * e], n1 = a.cells[3 * e + 1], n2 = a.cells[3 * e + 2];
  const double J00 = a.xy[2 * n1] - a.xy[2 * n0], J01 = a.xy[2 * n2] - a.xy[2 * n0];
  const double J10 = a.xy[2 * n1 + 1] - a.xy[2 * n0 + 1], J11 = a.xy[2 * n2 + 1] - a.xy[2 * n0 + 1];
  const double detJ = J00 * J11 - J01 * J10;
  const double ad00 = J11, ad01 = -J01, ad10 = -J10, ad11 = J00;
  const double wn[3][2] = {{-(J10 - J11), J00 - J01}, {-J11, J01}, {J10, -J00}};
  const double kinv = (a.kappa_mode == 1) ? 1.0 / a.kcell[e] : 1.0;
  const double kf = 1.0 / (kinv * detJ);
  const int c = r / NW, ia = r - c * NW;
  double g0 = 0.0, g1 = 0.0;
  for (int ib = 0; ib < NW; ++ib) {
    const double x = Xu[ib * (M + 1) + j];
    g0 += a.ref[G.SMD0 + ia * NW + ib] * x;
    g1 += a.ref[G.SMD1 + ia * NW + ib] * x;
  }
  double v = c ? (ad01 * g0 + ad11 * g1) : (ad00 * g0 + ad10 * g1);
  if (j < M) {
    const int f = j / NT, jj = j - f * NT;
    const int fo = f * 2 + ((a.orient[e] >> f) & 1);
    v -= wn[f][c] * a.ref[G.SMF + (fo * NW + ia) * NT + jj];
  }
  KB[t] = kf * v;
}

template <int P, int EWARPS> size_t smem_bytes_chol(const ElemArgs& a) {
  using D = Dims<P>;
  constexpr int LDW = (D::NW + D::M + 1) | 1;
  const RefLayout& G = a.L;
  const int tab = (G.Q + 2 * a.nq - G.C) + 3 * D::NW * D::NW + (G.PFF + 36 * D::NT * D::NT - G.SDMF);
  const int wstride = ((D::NW * LDW + D::NW * (D::M + 1) + a.nq + 2 * D::NW) + 1) & ~1;
  return (size_t)(((tab + 1) & ~1) + EWARPS * wstride) * sizeof(double);
}

template <int P, int EWARPS> size_t smem_bytes_lu(const ElemArgs& a) {
  using D = Dims<P>;
  const int wstride = D::N * D::LD + 2 * a.nq + D::NW + D::N + 2;
  return (size_t)(((a.ref_len + 1) & ~1) + EWARPS * wstride) * sizeof(double);
}

constexpr size_t ELEM_SMEM_MAX = 200 * 1024;

// Launches one path's kernel with EWARPS warps per CTA and a grid of `oversub` x the resident CTAs
// (a grid-stride loop covers the rest).  Returns false when the configuration does not fit.
template <int P, int EWARPS, bool CHOL>
bool launch_pw(hdg_system* s, cudaStream_t st, const ElemArgs& a, int oversub) {
  void (*kern)(ElemArgs);
  size_t smem;
  if constexpr (CHOL) {
    kern = k_element_chol<P, EWARPS>;
    smem = smem_bytes_chol<P, EWARPS>(a);
  } else {
    kern = k_element_condense<P, EWARPS>;
    smem = smem_bytes_lu<P, EWARPS>(a);
  }
  if (smem > ELEM_SMEM_MAX) return false;
  static bool attr_set = false;
  if (!attr_set) {
    HDG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ELEM_SMEM_MAX));
    attr_set = true;
  }
  int dev_sms = 152;
  cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, s->ctx->device);
  int blocks_per_sm = 0;
  HDG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, kern, EWARPS * 32, smem));
  if (blocks_per_sm < 1) return false;
  const long need = (a.nc + EWARPS - 1) / EWARPS;
  long grid = std::min<long>(need, (long)dev_sms * blocks_per_sm * oversub);
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, EWARPS * 32, smem, st>>>(a);
  HDG_CUDA(cudaGetLastError());
  s->ctx->launches++;
  return true;
}

template <int P, bool CHOL>
bool launch_cfg_path(hdg_system* s, cudaStream_t st, const ElemArgs& a, int warps, int oversub) {
  switch (warps) {
    case 1: return launch_pw<P, 1, CHOL>(s, st, a, oversub);
    case 2: return launch_pw<P, 2, CHOL>(s, st, a, oversub);
    case 4: return launch_pw<P, 4, CHOL>(s, st, a, oversub);
    case 8: return launch_pw<P, 8, CHOL>(s, st, a, oversub);
    case 16: return launch_pw<P, 16, CHOL>(s, st, a, oversub);
  }
  return false;
}

// P = 2 never takes the Schur path with the default rule (Strang(3) leaves M^ of rank 5), so its
// Cholesky-Schur kernels are not built; launch_element_condense keeps it on the full LU.
template <int P> bool launch_cfg(hdg_system* s, cudaStream_t st, const ElemArgs& a, int warps, int oversub) {
  if constexpr (P != 2) {
    if (a.schur) return launch_cfg_path<P, true>(s, st, a, warps, oversub);
  }
  return launch_cfg_path<P, false>(s, st, a, warps, oversub);
}

// Autotuner: the first launch for a (device, degree, quadrature size, log2 of the cell count, path)
// times every (warps per CTA, grid oversubscription) pair on the real inputs, on at most the first
// 65536 cells (the kernel only writes its outputs from its inputs, and every configuration
// computes each cell with the same instruction sequence, so the results are bit-identical; the
// real launch that follows writes every cell), and keeps the fastest.  The choice is cached for
// the process.  On a thread that builds one-shot systems (g_tuning_allowed false) a key without a
// cached choice takes the cached choice of the nearest cell count for the same degree, quadrature
// and path, and is timed only when there is none.  HDG_ELEMENT_WARPS=<1|2|4|8|16> fixes the warps
// per CTA instead.
template <int P> void launch_p(hdg_system* s, cudaStream_t st, const ElemArgs& a) {
  static std::mutex mu;
  static std::map<std::tuple<int, int, int, int>, std::pair<int, int>> best;
  if (const char* env = std::getenv("HDG_ELEMENT_WARPS")) {
    if (!launch_cfg<P>(s, st, a, std::atoi(env), 4)) throw HdgError{HDG_ERR_ARG, "HDG_ELEMENT_WARPS does not fit"};
    return;
  }
  int lg = 0;
  while ((1L << (lg + 1)) <= (long)a.nc) ++lg;
  const auto key = std::make_tuple(s->ctx->device, a.nq, lg, a.schur);
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = best.find(key);
    if (it == best.end() && !g_tuning_allowed) {  // nearest cached cell count, same degree and path
      int dist = 1 << 30;
      for (auto jt = best.begin(); jt != best.end(); ++jt) {
        const auto& k = jt->first;
        if (std::get<0>(k) != std::get<0>(key) || std::get<1>(k) != a.nq || std::get<3>(k) != a.schur) continue;
        const int d = std::abs(std::get<2>(k) - lg);
        if (d < dist) {
          dist = d;
          it = jt;
        }
      }
    }
    if (it != best.end()) {
      launch_cfg<P>(s, st, a, it->second.first, it->second.second);
      return;
    }
  }
  float best_ms = 1e30f;
  std::pair<int, int> pick{4, 4};
  cudaEvent_t e0, e1;
  HDG_CUDA(cudaEventCreate(&e0));
  HDG_CUDA(cudaEventCreate(&e1));
  ElemArgs t = a;  // the trials run on a prefix of the cells
  t.nc = std::min(a.nc, 65536);
  for (int w : {1, 2, 4, 8, 16})
    for (int g : {1, 4}) {
      if (!launch_cfg<P>(s, st, t, w, g)) continue;  // warm-up launch of this configuration
      HDG_CUDA(cudaEventRecord(e0, st));
      launch_cfg<P>(s, st, t, w, g);
      HDG_CUDA(cudaEventRecord(e1, st));
      HDG_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      HDG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      if (ms < best_ms) {
        best_ms = ms;
        pick = {w, g};
      }
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (best_ms == 1e30f) throw HdgError{HDG_ERR_ARG, "no element-kernel configuration fits in shared memory"};
  {
    std::lock_guard<std::mutex> lk(mu);
    best[key] = pick;
  }
  launch_cfg<P>(s, st, a, pick.first, pick.second);
}

}  // namespace

namespace {
ElemArgs element_args(hdg_system* s) {
  hdg_space* sp = s->space;
  hdg_mesh* m = sp->mesh;
  ElemArgs a;
  a.xy = m->d_xy.p;
  a.cells = m->d_cells.p;
  a.orient = m->d_orient.p;
  a.ref = sp->d_ref.p;
  a.nq = sp->t.nq;
  a.nc = m->nc;
  a.co = s->coef_dev();
  a.kappa_mode = s->kappa_cells ? 1 : (s->kappa_field ? 2 : 0);
  a.he_tau = s->he_tau ? 1 : 0;
  a.kcell = s->d_kappa.p;
  a.AB = s->d_AB.p;
  a.KB = s->d_KB.p;
  a.err = reinterpret_cast<int*>(s->d_scal.p + 1);
  // Cholesky-Schur path: invertible reference mass and kappa constant on each cell (a kappa field
  // makes Ae a weighted mass matrix that is no multiple of the reference one)
  a.schur = (sp->t.schur && a.kappa_mode != 2 && sp->t.p != 2 && std::getenv("HDG_ELEMENT_FULL_LU") == nullptr) ? 1
                                                                                                                 : 0;
  a.L = ref_layout(sp->t.nw, sp->t.nt, sp->t.nq);
  a.ref_len = a.L.SMD0;  // the full path stages [M .. Q]; the Cholesky path stages its own ranges
  return a;
}
}  // namespace

void launch_element_condense(hdg_system* s, cudaStream_t st) {
  const ElemArgs a = element_args(s);
  s->kb_u_only = a.schur != 0;
  switch (s->space->t.p) {
    case 1: launch_p<1>(s, st, a); break;
    case 2: launch_p<2>(s, st, a); break;
    case 3: launch_p<3>(s, st, a); break;
    case 4: launch_p<4>(s, st, a); break;
    default: throw HdgError{HDG_ERR_ARG, "degree not supported"};
  }
}

void launch_expand_ke(hdg_system* s, double* out, cudaStream_t st) {
  const ElemArgs a = element_args(s);
  const int64_t tot = (int64_t)a.nc * s->n * (s->m + 1);
  const unsigned grid = (unsigned)((tot + 255) / 256);
  switch (s->space->t.p) {
    case 1: k_expand_ke<1><<<grid, 256, 0, st>>>(a, s->d_KB.p, out); break;
    case 3: k_expand_ke<3><<<grid, 256, 0, st>>>(a, s->d_KB.p, out); break;
    case 4: k_expand_ke<4><<<grid, 256, 0, st>>>(a, s->d_KB.p, out); break;
    default: throw HdgError{HDG_ERR_ARG, "the stored element blocks are complete for this degree"};
  }
  HDG_CUDA(cudaGetLastError());
  s->ctx->launches++;
}
