// Reference-element tables of the HDG spaces, built once per (p, quad_degree) on the host in FP64.
//
// The function spaces of the reference (src/ScalarFunctionSpaces.jl:31-99,
// src/VectorFunctionSpaces.jl:10-18, src/TraceFunctionSpaces.jl:11-28) cache basis values at
// the quadrature points and re-multiply them per cell.  On an affine triangle every element
// integral of examples/poisson2D_HDG.jl:88-153 is a small combination of a few fixed
// reference matrices, so this file also packs those matrices for the device:
//   M  [a][b]      = sum_q w_q N_a N_b                      (mass; Ae = kappa^-1 detJ (M (+) M))
//   D_l[a][j]      = sum_q w_q dN_a/dxi_l N_j               (Be[(c,a),j] = sum_l adj(J)[l][c] D_l[a][j])
//   C_f[a][b]      = sum_k fw_k E_a(k,f) E_b(k,f)           (Ce = tau sum_f |e_f| C_f)
//   F_{f,o}[a][j]  = sum_k fw_k T_j(k) E_a(o ? k : nfq-1-k, f)  (Fe = tau |e_f| F, Ee = wn_f (x) F)
//   H[i][j]        = sum_k fw_k T_i(k) T_j(k)               (He = |e_f| H per face block)
//   NW[a][q]       = N_a(q) w_q                             (be = detJ sum_q f(x_q) NW[a][q])
#include <string>
#include <algorithm>
#include <cmath>
#include <cstring>

#include "hdg_internal.h"

namespace {

// Forward-mode dual number in two variables, for exact basis gradients.
struct Dd {
  double v, gx, gy;
};
inline Dd dconst(double c) { return {c, 0, 0}; }
inline Dd operator+(Dd a, Dd b) { return {a.v + b.v, a.gx + b.gx, a.gy + b.gy}; }
inline Dd operator-(Dd a, Dd b) { return {a.v - b.v, a.gx - b.gx, a.gy - b.gy}; }
inline Dd operator*(Dd a, Dd b) { return {a.v * b.v, a.gx * b.v + a.v * b.gx, a.gy * b.v + a.v * b.gy}; }
inline Dd operator*(double s, Dd a) { return {s * a.v, s * a.gx, s * a.gy}; }
inline Dd operator/(Dd a, Dd b) {
  double q = a.v / b.v;
  return {q, (a.gx - q * b.gx) / b.v, (a.gy - q * b.gy) / b.v};
}

// Jacobi polynomial P_n^{(al,be)}(x) by the standard three-term recurrence.
Dd jacobi_p(Dd x, int n, double al, double be) {
  Dd p0 = dconst(1.0);
  if (n == 0) return p0;
  Dd p1 = 0.5 * ((2.0 + al + be) * x + dconst(al - be));
  for (int k = 2; k <= n; ++k) {
    double c1 = 2.0 * k * (k + al + be) * (2.0 * k - 2.0 + al + be);
    double c2 = (2.0 * k - 1.0 + al + be) * (al * al - be * be);
    double c3 = (2.0 * k - 2.0 + al + be) * (2.0 * k - 1.0 + al + be) * (2.0 * k + al + be);
    double c4 = 2.0 * (k - 1.0 + al) * (k - 1.0 + be) * (2.0 * k + al + be);
    Dd p2 = (1.0 / c1) * ((dconst(c2) + c3 * x) * p1 - c4 * p0);
    p0 = p1;
    p1 = p2;
  }
  return p1;
}

// Orthonormal Dubiner (Koornwinder) basis function of bidegree (n, m) on the triangle
// (0,0),(1,0),(0,1), normalised so that the L2 norm over the triangle is 1 (phi_1 = sqrt 2).
// Collapsed coordinates a = 2x/(1-y) - 1, b = 2y - 1; the x = 0 corner uses a = -1, as the
// reference does (src/basis.jl:173).
Dd dubiner_nm(Dd x, Dd y, int n, int m) {
  Dd a = (std::fabs(x.v) < 2.220446049250313e-16) ? dconst(-1.0) : (2.0 * x) / (dconst(1.0) - y) - dconst(1.0);
  Dd b = 2.0 * y - dconst(1.0);
  Dd h = 0.5 * (dconst(1.0) - b);  // (1-b)/2 = 1 - y
  Dd hn = dconst(1.0);
  for (int i = 0; i < n; ++i) hn = hn * h;
  Dd P = jacobi_p(a, n, 0, 0) * jacobi_p(b, m, 2.0 * n + 1.0, 0) * hn;
  double norm = std::sqrt(2.0 * (2.0 * n + 1.0) * (n + m + 1.0));
  return norm * P;
}

// Basis index j (1-based) -> bidegree: degree d = n + m, within a degree n runs d, d-1, ..., 0
// (the ordering of the reference's closed forms, src/basis.jl:65-86 and :211-218).
void dubiner_index(int j, int* n, int* m) {
  int d = 0;
  while ((d + 1) * (d + 2) / 2 < j) ++d;
  int first = d * (d + 1) / 2 + 1;
  *n = d - (j - first);
  *m = d - *n;
}

// Orthonormal Legendre on (0,1): sqrt(2k+1) P_k(2s-1), k = 0..  (src/basis.jl:351-354).
double legendre01(int k, double s) {
  double x = 2.0 * s - 1.0, p0 = 1.0, p1 = x;
  if (k == 0) return 1.0;
  for (int i = 2; i <= k; ++i) {
    double p2 = ((2.0 * i - 1.0) * x * p1 - (i - 1.0) * p0) / i;
    p0 = p1;
    p1 = p2;
  }
  return std::sqrt(2.0 * k + 1.0) * p1;
}

// Strang–Fix triangle rules of orders 1..6 (the constants of src/StrangQuad.jl; the rule must
// be the same one for parity).  Points given by orbit generators.
bool strang_rule(int order, std::vector<double>& x, std::vector<double>& y, std::vector<double>& w) {
  x.clear(); y.clear(); w.clear();
  auto pt = [&](double a, double b, double wt) { x.push_back(a); y.push_back(b); w.push_back(wt); };
  switch (order) {
    case 0:
    case 1: pt(1.0 / 3.0, 1.0 / 3.0, 0.5); return true;
    case 2:
      pt(1.0 / 6.0, 1.0 / 6.0, 1.0 / 6); pt(1.0 / 6.0, 2.0 / 3.0, 1.0 / 6); pt(2.0 / 3.0, 1.0 / 6.0, 1.0 / 6);
      return true;
    case 3: {
      const double a = 0.659027622374092, b = 0.231933368553031, c = 0.109039009072877, wt = 1.0 / 12.0;
      pt(a, b, wt); pt(a, c, wt); pt(b, a, wt); pt(b, c, wt); pt(c, a, wt); pt(c, b, wt);
      return true;
    }
    case 4: {
      const double a = 0.816847572980459, b = 0.091576213509771, c = 0.108103018168070, d = 0.445948490915965;
      const double w1 = 0.109951743655322 * 0.5, w2 = 0.223381589678011 * 0.5;
      pt(a, b, w1); pt(b, a, w1); pt(b, b, w1); pt(c, d, w2); pt(d, c, w2); pt(d, d, w2);
      return true;
    }
    case 5: {
      const double a = 0.79742698535308720, b = 0.10128650732345633, c = 0.05971587178976981,
                   d = 0.47014206410511505;
      const double w0 = 0.22500000000000000 * 0.5, w1 = 0.12593918054482717 * 0.5, w2 = 0.13239415278850616 * 0.5;
      pt(0.33333333333333333, 0.33333333333333333, w0);
      pt(a, b, w1); pt(b, a, w1); pt(b, b, w1); pt(c, d, w2); pt(d, c, w2); pt(d, d, w2);
      return true;
    }
    case 6: {
      const double a = 0.873821971016996, b = 0.063089014491502, c = 0.501426509658179, d = 0.249286745170910;
      const double e = 0.636502499121399, f = 0.310352451033785, g = 0.053145049844816;
      const double w1 = 0.050844906370207 * 0.5, w2 = 0.116786275726379 * 0.5, w3 = 0.082851075618374 * 0.5;
      pt(a, b, w1); pt(b, a, w1); pt(b, b, w1); pt(c, d, w2); pt(d, c, w2); pt(d, d, w2);
      pt(e, f, w3); pt(e, g, w3); pt(f, e, w3); pt(f, g, w3); pt(g, e, w3); pt(g, f, w3);
      return true;
    }
  }
  return false;
}

// Grundmann–Möller rule of index s on the triangle (exact to degree 2s+1; weights may be
// negative), Grundmann & Möller, SIAM J. Numer. Anal. 15 (1978) 282-290.
void gm_rule(int s, std::vector<double>& x, std::vector<double>& y, std::vector<double>& w) {
  x.clear(); y.clear(); w.clear();
  const int d = 2 * s + 1;
  double sum = 0;
  for (int i = 0; i <= s; ++i) {
    double lg = -2.0 * s * std::log(2.0) + d * std::log((double)(d + 2 - 2 * i)) - std::lgamma(i + 1.0) -
                std::lgamma(d + 3.0 - i);
    double wi = ((i & 1) ? -1.0 : 1.0) * std::exp(lg);
    const int t = s - i, den = d + 2 - 2 * i;
    for (int b1 = 0; b1 <= t; ++b1)
      for (int b2 = 0; b1 + b2 <= t; ++b2) {
        x.push_back((2.0 * b1 + 1.0) / den);
        y.push_back((2.0 * b2 + 1.0) / den);
        w.push_back(wi);
        sum += wi;
      }
  }
  for (double& v : w) v *= 0.5 / sum;
}

// n-point Gauss–Legendre nodes/weights on (0,1), ascending, by Newton on P_n in long double.
void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n, 0);
  w.assign(n, 0);
  for (int i = 0; i < n; ++i) {
    long double t = std::cos(3.141592653589793238462643383279502884L * (n - i - 0.25L) / (n + 0.5L));
    long double dp = 1;
    for (int it = 0; it < 60; ++it) {
      long double p0 = 1, p1 = t;
      for (int k = 2; k <= n; ++k) {
        long double p2 = ((2 * k - 1) * t * p1 - (k - 1) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      if (n == 1) p0 = 1, p1 = t;
      dp = n * (t * p1 - p0) / (t * t - 1);
      long double step = p1 / dp;
      t -= step;
      if (std::fabs((double)step) < 1e-22) break;
    }
    long double p0 = 1, p1 = t;
    for (int k = 2; k <= n; ++k) {
      long double p2 = ((2 * k - 1) * t * p1 - (k - 1) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    if (n == 1) p0 = 1, p1 = t;
    dp = n * (t * p1 - p0) / (t * t - 1);
    x[i] = (double)((t + 1) / 2);
    w[i] = (double)(1 / ((1 - t * t) * dp * dp));  // 2/((1-t^2)P'^2) scaled by 1/2
  }
}

// reference edges of the triangle (src/shapes.jl:19-23): 1: (1,0)->(0,1), 2: (0,1)->(0,0), 3: (0,0)->(1,0)
const double EDGE[3][4] = {{1, 0, 0, 1}, {0, 1, 0, 0}, {0, 0, 1, 0}};

}  // namespace

RefLayout ref_layout(int nw, int nt, int nq) {
  RefLayout L;
  int o = 0;
  // the full-LU path reads [M .. Q], the Schur path [C .. SDMF]: each range is contiguous
  L.M = o; o += nw * nw;
  L.D0 = o; o += nw * nw;
  L.D1 = o; o += nw * nw;
  L.N = o; o += nw * nq;
  L.C = o; o += 3 * nw * nw;
  L.F = o; o += 6 * nw * nt;
  L.H = o; o += nt * nt;
  L.NW = o; o += nw * nq;
  L.Q = o; o += 2 * nq;
  L.SMD0 = o; o += nw * nw;
  L.SMD1 = o; o += nw * nw;
  L.SQ00 = o; o += nw * nw;
  L.SQ01 = o; o += nw * nw;
  L.SQ11 = o; o += nw * nw;
  L.SMF = o; o += 6 * nw * nt;
  L.SDMF = o; o += 12 * nw * nt;
  L.PFF = o; o += 36 * nt * nt;
  L.total = o;
  return L;
}

// QuadratureRule{2}(DefaultQuad(), qd) dispatch of src/quadrature.jl:17-26: Strang for qd <= 6,
// Grundmann–Möller of index (qd-1)/2 for odd qd > 6, otherwise not available.
bool build_ref_tables(int p, int qd, RefTables* t) {
  if (p < 1 || p > HDG_MAX_P) return false;
  t->p = p;
  t->qd = qd;
  t->nw = (p + 1) * (p + 2) / 2;
  t->nt = p + 1;
  if (qd <= 6) {
    if (!strang_rule(qd, t->qx, t->qy, t->qw)) return false;
  } else if (qd % 2 == 1) {
    gm_rule((qd - 1) / 2, t->qx, t->qy, t->qw);
  } else {
    return false;
  }
  if (qd < 1) return false;
  gauss_legendre(qd, t->fx, t->fw);
  const int nw = t->nw, nt = t->nt;
  t->nq = (int)t->qw.size();
  t->nfq = (int)t->fw.size();
  const int nq = t->nq, nfq = t->nfq;
  t->N.assign(nw * nq, 0);
  t->dN.assign(nw * nq * 2, 0);
  for (int a = 0; a < nw; ++a) {
    int n, m;
    dubiner_index(a + 1, &n, &m);
    for (int q = 0; q < nq; ++q) {
      Dd v = dubiner_nm(Dd{t->qx[q], 1, 0}, Dd{t->qy[q], 0, 1}, n, m);
      t->N[a * nq + q] = v.v;
      t->dN[(a * nq + q) * 2] = v.gx;
      t->dN[(a * nq + q) * 2 + 1] = v.gy;
    }
  }
  t->Nv.assign(nw * 3, 0);
  static const double VX[3] = {0.0, 1.0, 0.0}, VY[3] = {0.0, 0.0, 1.0};
  for (int a = 0; a < nw; ++a) {
    int n, m;
    dubiner_index(a + 1, &n, &m);
    for (int k = 0; k < 3; ++k) t->Nv[a * 3 + k] = dubiner_nm(Dd{VX[k], 0, 0}, Dd{VY[k], 0, 0}, n, m).v;
  }
  t->E.assign(nw * nfq * 3, 0);
  for (int f = 0; f < 3; ++f)
    for (int k = 0; k < nfq; ++k) {
      double s = t->fx[k];
      double ex = (1.0 - s) * EDGE[f][0] + s * EDGE[f][2];
      double ey = (1.0 - s) * EDGE[f][1] + s * EDGE[f][3];
      for (int a = 0; a < nw; ++a) {
        int n, m;
        dubiner_index(a + 1, &n, &m);
        t->E[(a * nfq + k) * 3 + f] = dubiner_nm(Dd{ex, 0, 0}, Dd{ey, 0, 0}, n, m).v;
      }
    }
  t->T.assign(nt * nfq, 0);
  for (int j = 0; j < nt; ++j)
    for (int k = 0; k < nfq; ++k) t->T[j * nfq + k] = legendre01(j, t->fx[k]);

  // packed reference matrices
  RefLayout L = ref_layout(nw, nt, nq);
  std::vector<double>& P = t->packed;
  P.assign(L.total, 0.0);
  for (int a = 0; a < nw; ++a)
    for (int b = 0; b < nw; ++b) {
      double s = 0, s0 = 0, s1 = 0;
      for (int q = 0; q < nq; ++q) {
        double w = t->qw[q];
        s += w * t->N[a * nq + q] * t->N[b * nq + q];
        s0 += w * t->dN[(a * nq + q) * 2] * t->N[b * nq + q];
        s1 += w * t->dN[(a * nq + q) * 2 + 1] * t->N[b * nq + q];
      }
      P[L.M + a * nw + b] = s;
      P[L.D0 + a * nw + b] = s0;
      P[L.D1 + a * nw + b] = s1;
      for (int f = 0; f < 3; ++f) {
        double c = 0;
        for (int k = 0; k < nfq; ++k) c += t->fw[k] * t->E[(a * nfq + k) * 3 + f] * t->E[(b * nfq + k) * 3 + f];
        P[L.C + (f * nw + a) * nw + b] = c;
      }
    }
  for (int f = 0; f < 3; ++f)
    for (int o = 0; o < 2; ++o)
      for (int a = 0; a < nw; ++a)
        for (int j = 0; j < nt; ++j) {
          double s = 0;
          for (int k = 0; k < nfq; ++k) {
            int kk = o ? k : nfq - 1 - k;
            s += t->fw[k] * t->T[j * nfq + k] * t->E[(a * nfq + kk) * 3 + f];
          }
          P[L.F + ((f * 2 + o) * nw + a) * nt + j] = s;
        }
  for (int i = 0; i < nt; ++i)
    for (int j = 0; j < nt; ++j) {
      double s = 0;
      for (int k = 0; k < nfq; ++k) s += t->fw[k] * t->T[i * nfq + k] * t->T[j * nfq + k];
      P[L.H + i * nt + j] = s;
    }
  for (int a = 0; a < nw; ++a)
    for (int q = 0; q < nq; ++q) {
      P[L.NW + a * nq + q] = t->N[a * nq + q] * t->qw[q];
      P[L.N + a * nq + q] = t->N[a * nq + q];
    }
  for (int q = 0; q < nq; ++q) {
    P[L.Q + 2 * q] = t->qx[q];
    P[L.Q + 2 * q + 1] = t->qy[q];
  }
  // Schur-complement tables.  With the mass block Ae = (det J / kappa) diag(M, M) of an affine
  // cell and constant kappa, Me^-1 follows from M^-1 and the Schur complement
  // S = Ce + Be' Ae^-1 Be (nw x nw); every product of reference matrices it needs is tabulated
  // here once.  They are used only when the volume rule makes M invertible (for p = 2 the
  // default Strang(3) rule leaves M of rank 5, and the element kernel keeps its full LU).
  {
    std::vector<long double> a((size_t)nw * 2 * nw, 0.0L);
    for (int i = 0; i < nw; ++i) {
      for (int j = 0; j < nw; ++j) a[(size_t)i * 2 * nw + j] = P[L.M + i * nw + j];
      a[(size_t)i * 2 * nw + nw + i] = 1.0L;
    }
    long double maxpiv = 0.0L, minpiv = 1e300L;
    bool ok = true;
    for (int c = 0; c < nw && ok; ++c) {
      int piv = c;
      for (int i = c + 1; i < nw; ++i)
        if (std::fabs(a[(size_t)i * 2 * nw + c]) > std::fabs(a[(size_t)piv * 2 * nw + c])) piv = i;
      if (piv != c)
        for (int j = 0; j < 2 * nw; ++j) std::swap(a[(size_t)c * 2 * nw + j], a[(size_t)piv * 2 * nw + j]);
      const long double d = a[(size_t)c * 2 * nw + c];
      maxpiv = std::max(maxpiv, std::fabs(d));
      minpiv = std::min(minpiv, std::fabs(d));
      if (d == 0.0L) { ok = false; break; }
      for (int j = 0; j < 2 * nw; ++j) a[(size_t)c * 2 * nw + j] /= d;
      for (int i = 0; i < nw; ++i) {
        if (i == c) continue;
        const long double m = a[(size_t)i * 2 * nw + c];
        for (int j = 0; j < 2 * nw; ++j) a[(size_t)i * 2 * nw + j] -= m * a[(size_t)c * 2 * nw + j];
      }
    }
    t->schur = ok && minpiv > 1e-10L * maxpiv;
    if (t->schur) {
      auto Mi = [&](int i, int j) { return a[(size_t)i * 2 * nw + nw + j]; };
      const double* D[2] = {&P[L.D0], &P[L.D1]};
      std::vector<long double> MD[2];
      for (int l = 0; l < 2; ++l) {
        MD[l].assign((size_t)nw * nw, 0.0L);
        for (int i = 0; i < nw; ++i)
          for (int j = 0; j < nw; ++j) {
            long double s = 0;
            for (int k = 0; k < nw; ++k) s += Mi(i, k) * D[l][k * nw + j];
            MD[l][(size_t)i * nw + j] = s;
            P[(l ? L.SMD1 : L.SMD0) + i * nw + j] = (double)s;
          }
      }
      const int QO[3] = {L.SQ00, L.SQ01, L.SQ11};
      const int QL[3][2] = {{0, 0}, {0, 1}, {1, 1}};
      for (int q = 0; q < 3; ++q)
        for (int i = 0; i < nw; ++i)
          for (int j = 0; j < nw; ++j) {
            long double s = 0;  // (D_l' M^-1 D_m)[i][j] = sum_k D_l[k][i] (M^-1 D_m)[k][j]
            for (int k = 0; k < nw; ++k) s += (long double)D[QL[q][0]][k * nw + i] * MD[QL[q][1]][(size_t)k * nw + j];
            P[QO[q] + i * nw + j] = (double)s;
          }
      for (int fo = 0; fo < 6; ++fo) {
        std::vector<long double> MF((size_t)nw * nt, 0.0L);
        for (int i = 0; i < nw; ++i)
          for (int j = 0; j < nt; ++j) {
            long double s = 0;
            for (int k = 0; k < nw; ++k) s += Mi(i, k) * P[L.F + (fo * nw + k) * nt + j];
            MF[(size_t)i * nt + j] = s;
            P[L.SMF + (fo * nw + i) * nt + j] = (double)s;
          }
        for (int l = 0; l < 2; ++l)
          for (int i = 0; i < nw; ++i)
            for (int j = 0; j < nt; ++j) {
              long double s = 0;
              for (int k = 0; k < nw; ++k) s += (long double)D[l][k * nw + i] * MF[(size_t)k * nt + j];
              P[L.SDMF + ((l * 6 + fo) * nw + i) * nt + j] = (double)s;
            }
        // PFF_{go,fo} = F_{go}' M^-1 F_{fo} (nt x nt), the face-face term of the condensed operator
        for (int go = 0; go < 6; ++go)
          for (int i = 0; i < nt; ++i)
            for (int j = 0; j < nt; ++j) {
              long double s = 0;
              for (int k = 0; k < nw; ++k) s += (long double)P[L.F + (go * nw + k) * nt + i] * MF[(size_t)k * nt + j];
              P[L.PFF + ((go * 6 + fo) * nt + i) * nt + j] = (double)s;
            }
      }
    }
  }
  return true;
}

// ------------------------------------------------------------------ continuous Lagrange
// ContinuousLagrange{2,RefTetrahedron,k} (src/LagrangeFE.jl:17-39): the nodal basis is the dual
// of the Dubiner basis at the nodal points, phi_k = sum_j C[j][k] D_j with C = V^-1 and
// V[i][j] = D_j(node_i).  Nodal points as get_nodal_points (src/shapes.jl:46-77): the vertices
// (0,0), (1,0), (0,1); the k-1 interior points of the edges (1,0)->(0,1), (0,1)->(0,0),
// (0,0)->(1,0); then the interior grid (j/k, i/k).
bool build_lagrange_tables(int order, int qd, LagrangeTables* t) {
  if (order < 1 || order > HDG_MAX_P) return false;
  RefTables r;
  if (!build_ref_tables(order, qd, &r)) return false;  // the rule and the Dubiner tables
  const int k = order, nl = (k + 1) * (k + 2) / 2, nq = r.nq;
  std::vector<double> px, py;
  const double V0[3][2] = {{0, 0}, {1, 0}, {0, 1}};
  const double ED[3][4] = {{1, 0, 0, 1}, {0, 1, 0, 0}, {0, 0, 1, 0}};
  for (int v = 0; v < 3; ++v) { px.push_back(V0[v][0]); py.push_back(V0[v][1]); }
  for (int e = 0; e < 3; ++e)
    for (int i = 1; i < k; ++i) {
      px.push_back(ED[e][0] + i * (ED[e][2] - ED[e][0]) / k);
      py.push_back(ED[e][1] + i * (ED[e][3] - ED[e][1]) / k);
    }
  for (int i = 1; i < k; ++i)
    for (int j = 1; j < k - i; ++j) { px.push_back((double)j / k); py.push_back((double)i / k); }
  if ((int)px.size() != nl) return false;
  // [V | I] -> [I | V^-1] by Gauss-Jordan with partial pivoting in long double
  std::vector<long double> a((size_t)nl * 2 * nl, 0.0L);
  for (int i = 0; i < nl; ++i) {
    for (int j = 0; j < nl; ++j) {
      int n, m;
      dubiner_index(j + 1, &n, &m);
      a[(size_t)i * 2 * nl + j] = dubiner_nm(Dd{px[i], 0, 0}, Dd{py[i], 0, 0}, n, m).v;
    }
    a[(size_t)i * 2 * nl + nl + i] = 1.0L;
  }
  for (int c = 0; c < nl; ++c) {
    int piv = c;
    for (int i = c + 1; i < nl; ++i)
      if (std::fabs(a[(size_t)i * 2 * nl + c]) > std::fabs(a[(size_t)piv * 2 * nl + c])) piv = i;
    if (a[(size_t)piv * 2 * nl + c] == 0.0L) return false;
    if (piv != c)
      for (int j = 0; j < 2 * nl; ++j) std::swap(a[(size_t)c * 2 * nl + j], a[(size_t)piv * 2 * nl + j]);
    const long double d = a[(size_t)c * 2 * nl + c];
    for (int j = 0; j < 2 * nl; ++j) a[(size_t)c * 2 * nl + j] /= d;
    for (int i = 0; i < nl; ++i) {
      if (i == c) continue;
      const long double f = a[(size_t)i * 2 * nl + c];
      if (f != 0.0L)
        for (int j = 0; j < 2 * nl; ++j) a[(size_t)i * 2 * nl + j] -= f * a[(size_t)c * 2 * nl + j];
    }
  }
  t->order = k;
  t->nl = nl;
  t->nq = nq;
  t->qx = r.qx;
  t->qy = r.qy;
  t->qw = r.qw;
  t->N.assign((size_t)nl * nq, 0.0);
  t->dN.assign((size_t)nl * nq * 2, 0.0);
  for (int kk = 0; kk < nl; ++kk)
    for (int q = 0; q < nq; ++q) {
      long double v = 0, gx = 0, gy = 0;
      for (int j = 0; j < nl; ++j) {
        const long double cjk = a[(size_t)j * 2 * nl + nl + kk];  // (V^-1)[j][kk]
        v += cjk * r.N[(size_t)j * nq + q];
        gx += cjk * r.dN[((size_t)j * nq + q) * 2];
        gy += cjk * r.dN[((size_t)j * nq + q) * 2 + 1];
      }
      t->N[(size_t)kk * nq + q] = (double)v;
      t->dN[((size_t)kk * nq + q) * 2] = (double)gx;
      t->dN[((size_t)kk * nq + q) * 2 + 1] = (double)gy;
    }
  return true;
}

// ------------------------------------------------------------------ fields (host side)
// A field's parameter count must cover what its kind reads (the device evaluator indexes them
// without bounds): CONST c; SINSIN a, kx, ky; BUMPS K then 4 per bump; FOURIER / EXP_FOURIER K,
// g0 then 4 per mode, with K a finite non-negative integer.
int field_check(const hdg_field* f, std::string* why) {
  if (!f) return HDG_OK;
  auto bad = [&](const std::string& m) {
    if (why) *why = m;
    return HDG_ERR_ARG;
  };
  if (f->nparams < 0) return bad("field: negative parameter count");
  if (f->nparams > 0 && !f->params) return bad("field: parameter count without parameters");
  const int np = f->nparams;
  const double* p = f->params;
  auto count_of = [&](int first) -> long {  // K in p[0], items of 4 after `first` leading values
    if (np < 1 || !std::isfinite(p[0]) || p[0] < 0.0 || p[0] != std::floor(p[0]) || p[0] > 1e6) return -1;
    return first + 4L * (long)p[0];
  };
  switch (f->kind) {
    case HDG_FIELD_CONST:
      if (np < 1) return bad("field CONST needs 1 parameter (c)");
      return HDG_OK;
    case HDG_FIELD_SINSIN:
      if (np < 3) return bad("field SINSIN needs 3 parameters (a, kx, ky)");
      return HDG_OK;
    case HDG_FIELD_BUMPS: {
      const long need = count_of(1);
      if (need < 0) return bad("field BUMPS: the first parameter must be the bump count K >= 0");
      if (np < need) return bad("field BUMPS with K = " + std::to_string((long)p[0]) + " needs " + std::to_string(need) +
                                " parameters, got " + std::to_string(np));
      return HDG_OK;
    }
    case HDG_FIELD_FOURIER:
    case HDG_FIELD_EXP_FOURIER: {
      const long need = count_of(2);
      if (need < 0) return bad("field FOURIER: the first parameter must be the mode count K >= 0");
      if (np < need) return bad("field FOURIER with K = " + std::to_string((long)p[0]) + " needs " +
                                std::to_string(need) + " parameters, got " + std::to_string(np));
      return HDG_OK;
    }
  }
  return bad("field: unknown kind " + std::to_string(f->kind));
}

FieldSpec field_from(const hdg_field* f, double default_const) {
  FieldSpec s;
  if (!f) {
    s.kind = HDG_FIELD_CONST;
    s.prm = {default_const};
    return s;
  }
  std::string why;
  if (field_check(f, &why) != HDG_OK) throw HdgError{HDG_ERR_ARG, why};
  s.kind = f->kind;
  s.prm.assign(f->params, f->params + f->nparams);
  return s;
}

double eval_field_host(const FieldSpec& f, double x, double y) {
  const double* p = f.prm.data();
  switch (f.kind) {
    case HDG_FIELD_CONST: return p[0];
    case HDG_FIELD_SINSIN: return p[0] * std::sin(p[1] * M_PI * x) * std::sin(p[2] * M_PI * y);
    case HDG_FIELD_BUMPS: {
      int K = (int)p[0];
      double s = 0;
      for (int k = 0; k < K; ++k) {
        const double* b = p + 1 + 4 * k;
        double dx = x - b[0], dy = y - b[1];
        s += b[3] * std::exp(-(dx * dx + dy * dy) / (2.0 * b[2] * b[2]));
      }
      return s;
    }
    case HDG_FIELD_FOURIER:
    case HDG_FIELD_EXP_FOURIER: {
      int K = (int)p[0];
      double g = p[1];
      for (int k = 0; k < K; ++k) {
        const double* b = p + 2 + 4 * k;
        g += b[3] * std::cos(2.0 * M_PI * (b[0] * x + b[1] * y) + b[2]);
      }
      return f.kind == HDG_FIELD_EXP_FOURIER ? std::exp(g) : g;
    }
  }
  return 0.0;
}
