// hdgref — CPU restatement of the HDiscontinuousGalerkin.jl 2D HDG Poisson flow.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle that the GPU library is checked
// against.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it,
// and only as the test oracle or the timed CPU baseline; the product (libhdg) never links it.
//
// Every routine restates one piece of the reference (Julia) and cites the file:line it
// follows.  The reference's quirks are kept on purpose (quadrature degree p+1, face
// orientation flips, He without tau, the trace-Dirichlet projection), because parity is
// defined by the reference's behaviour, not against textbook HDG.  The one deliberate
// generalisation is the recovery slice (examples/poisson2D_HDG.jl:205-206 hard-codes two
// trace functions per edge); here it is (f-1)*nt+1 : f*nt for any nt.
//
// Third-party arithmetic restated here (absent from the reference tree):
//   * FastGaussQuadrature.jl (REQUIRE: >= 0.3.0) `gausslegendre(n)`: Newton iteration on the
//     Legendre three-term recurrence in long double (ascending nodes), call site
//     src/quadrature.jl:30.
//   * Tensors.jl (REQUIRE: >= 0.8.0) forward-mode `gradient`: a dual-number type, call sites
//     src/ScalarFunctionSpaces.jl:65,82,85.
//   * LinearAlgebra `factorize` on a general square matrix = LU with partial pivoting
//     (examples/poisson2D_HDG.jl:160); restated as a textbook right-looking getrf.
//   * SparseArrays `sparse(I,J,V)` = COO -> CSC with duplicates summed (src/assembler.jl:48).
// The sparse direct solve (`K \ b`, examples/poisson2D_HDG.jl:195) is done by the Python side
// of the oracle with scipy's SuperLU.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <utility>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------- dual numbers (AD)
struct Dual {
  double v, dx, dy;
  Dual(double a = 0.0) : v(a), dx(0.0), dy(0.0) {}
  Dual(double a, double b, double c) : v(a), dx(b), dy(c) {}
};
inline Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.dx + b.dx, a.dy + b.dy}; }
inline Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.dx - b.dx, a.dy - b.dy}; }
inline Dual operator-(Dual a) { return {-a.v, -a.dx, -a.dy}; }
inline Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.dx * b.v + a.v * b.dx, a.dy * b.v + a.v * b.dy}; }
inline Dual operator/(Dual a, Dual b) {
  double iv = 1.0 / b.v;
  return {a.v / b.v, (a.dx * b.v - a.v * b.dx) * iv * iv, (a.dy * b.v - a.v * b.dy) * iv * iv};
}
inline Dual operator+(Dual a, double b) { return {a.v + b, a.dx, a.dy}; }
inline Dual operator+(double b, Dual a) { return {a.v + b, a.dx, a.dy}; }
inline Dual operator-(Dual a, double b) { return {a.v - b, a.dx, a.dy}; }
inline Dual operator-(double b, Dual a) { return {b - a.v, -a.dx, -a.dy}; }
inline Dual operator*(Dual a, double b) { return {a.v * b, a.dx * b, a.dy * b}; }
inline Dual operator*(double b, Dual a) { return {a.v * b, a.dx * b, a.dy * b}; }
inline Dual operator/(Dual a, double b) { return {a.v / b, a.dx / b, a.dy / b}; }
inline double val(double a) { return a; }
inline double val(const Dual& a) { return a.v; }
template <class T> inline T ipow(T x, int k) {
  T r(1.0);
  for (int i = 0; i < k; ++i) r = r * x;
  return r;
}

// ---------------------------------------------------------------- bases
// jacobi(x, p, a, b): three-term recursion, src/basis.jl:132-150
template <class T> T jacobi(T x, int p, double al, double be) {
  T a(1.0);
  T b = ((2 + al + be) * x + (al - be)) / 2.0;
  if (p <= 0) return a;
  if (p == 1) return b;
  for (int n = 2; n <= p; ++n) {
    double a1 = 2.0 * n * (n + al + be) * (2.0 * n - 2 + al + be);
    double a2 = (2.0 * n - 1 + al + be) * (al + be) * (al - be);
    double a3 = (2.0 * n - 2 + al + be) * (2.0 * n - 1 + al + be) * (2.0 * n + al + be);
    double a4 = 2.0 * (n - 1 + al) * (n - 1 + be) * (2.0 * n + al + be);
    T nb = ((a2 + a3 * x) * b - a4 * a) / a1;
    a = b;
    b = nb;
  }
  return b;
}

// dubiner(x,y,n,m), src/basis.jl:169-181
template <class T> T dubiner_nm(T x, T y, int n, int m) {
  T xi = (std::fabs(val(x)) < 2.220446049250313e-16) ? T(-1.0) : 2.0 * x / (1.0 - y) - 1.0;
  T eta = 2.0 * y - 1.0;
  int k = 2 * n + 1;
  T P = jacobi(xi, n, 0.0, 0.0) * jacobi(eta, m, (double)k, 0.0) * ipow((1.0 - eta) / 2.0, n);
  double N = std::sqrt(2.0 / ((2.0 * n + 1) * (m + n + 1)));
  return (2.0 * P) / N;
}

// dubiner_basis(x,y,j) index map, src/basis.jl:211-218
inline void dubiner_degrees(int j, int* n, int* m) {
  double t = -1.5 + 0.5 * std::sqrt(1.0 + 8.0 * j);
  double c = std::ceil(t);
  *n = (int)((c + 1) * (c + 2) / 2 - j);
  *m = (int)(c - *n);
}

// value(::Dubiner{2}, j, ξ): closed forms for j<=15, src/basis.jl:65-86
template <class T> T dubiner_value(int j, T r, T s) {
  const double s2 = std::sqrt(2.0), s3 = std::sqrt(3.0), s6 = std::sqrt(6.0), s10 = std::sqrt(10.0);
  const double s14 = std::sqrt(14.0), s30 = std::sqrt(30.0), s70 = std::sqrt(70.0);
  T q4 = 6.0 * r * r + 6.0 * r * (s - 1.0) + s * s - 2.0 * s + 1.0;
  T l2 = 2.0 * r + s - 1.0;
  T c10 = 10.0 * r * r + 10.0 * r * (s - 1.0) + s * s - 2.0 * s + 1.0;
  switch (j) {
    case 0: return T(0.0);
    case 1: return T(s2);
    case 2: return 2.0 * s3 * l2;
    case 3: return 2.0 * (3.0 * s - 1.0);
    case 4: return s30 * q4;
    case 5: return 3.0 * s2 * (5.0 * s - 1.0) * l2;
    case 6: return s6 * (10.0 * s * s - 8.0 * s + 1.0);
    case 7: return 2.0 * s14 * l2 * c10;
    case 8: return 2.0 * s10 * (7.0 * s - 1.0) * q4;
    case 9: return 2.0 * s6 * (21.0 * s * s - 12.0 * s + 1.0) * l2;
    case 10: return 2.0 * s2 * (35.0 * s * s * s - 45.0 * s * s + 15.0 * s - 1.0);
    case 11:
      return 3.0 * s10 *
             (70.0 * ipow(r, 4) + 140.0 * ipow(r, 3) * (s - 1.0) + 90.0 * r * r * (s * s - 2.0 * s + 1.0) +
              20.0 * r * (ipow(s, 3) - 3.0 * s * s + 3.0 * s - 1.0) + ipow(s, 4) - 4.0 * ipow(s, 3) + 6.0 * s * s -
              4.0 * s + 1.0);
    case 12: return s70 * (9.0 * s - 1.0) * l2 * c10;
    case 13: return 5.0 * s2 * (36.0 * s * s - 16.0 * s + 1.0) * q4;
    case 14: return s30 * (84.0 * ipow(s, 3) - 84.0 * s * s + 21.0 * s - 1.0) * l2;
    case 15: return s10 * (126.0 * ipow(s, 4) - 224.0 * ipow(s, 3) + 126.0 * s * s - 24.0 * s + 1.0);
    default: {
      int n, m;
      dubiner_degrees(j, &n, &m);
      return dubiner_nm(r, s, n, m);
    }
  }
}
template <class T> T dubiner_generic(int j, T r, T s) {
  int n, m;
  dubiner_degrees(j, &n, &m);
  return dubiner_nm(r, s, n, m);
}

// value(::Legendre{1}, k, ξ) = sqrt(2(k-1)+1) * jacobi(2ξ-1, k-1, 0, 0), src/basis.jl:351-354
inline double legendre_value(int k, double x) {
  return std::sqrt((double)(2 * (k - 1) + 1)) * jacobi(2.0 * x - 1.0, k - 1, 0.0, 0.0);
}

// ---------------------------------------------------------------- quadrature
struct Rule2 {
  std::vector<double> w, x, y;
};
struct Rule1 {
  std::vector<double> w, x;
};

// Strang rules, src/StrangQuad.jl:1-61
bool strang(int order, Rule2* r) {
  auto add = [&](double a, double b) {
    r->x.push_back(a);
    r->y.push_back(b);
  };
  r->w.clear(); r->x.clear(); r->y.clear();
  if (order == 0 || order == 1) {
    add(1.0 / 3.0, 1.0 / 3.0);
    r->w = {0.5};
  } else if (order == 2) {
    add(1.0 / 6.0, 1.0 / 6.0); add(1.0 / 6.0, 2.0 / 3.0); add(2.0 / 3.0, 1.0 / 6.0);
    r->w = {1.0 / 6, 1.0 / 6, 1.0 / 6};
  } else if (order == 3) {
    const double a = 0.659027622374092, b = 0.231933368553031, c = 0.109039009072877;
    add(a, b); add(a, c); add(b, a); add(b, c); add(c, a); add(c, b);
    r->w.assign(6, 1.0 / 12.0);
  } else if (order == 4) {
    add(0.816847572980459, 0.091576213509771); add(0.091576213509771, 0.816847572980459);
    add(0.091576213509771, 0.091576213509771); add(0.108103018168070, 0.445948490915965);
    add(0.445948490915965, 0.108103018168070); add(0.445948490915965, 0.445948490915965);
    r->w.assign(6, 0.5);
    for (int i = 0; i < 3; ++i) r->w[i] = 0.109951743655322 * r->w[i];
    for (int i = 3; i < 6; ++i) r->w[i] = 0.223381589678011 * r->w[i];
  } else if (order == 5) {
    add(0.33333333333333333, 0.33333333333333333); add(0.79742698535308720, 0.10128650732345633);
    add(0.10128650732345633, 0.79742698535308720); add(0.10128650732345633, 0.10128650732345633);
    add(0.05971587178976981, 0.47014206410511505); add(0.47014206410511505, 0.05971587178976981);
    add(0.47014206410511505, 0.47014206410511505);
    r->w.assign(7, 0.5);
    r->w[0] = 0.22500000000000000 * r->w[0];
    for (int i = 1; i < 4; ++i) r->w[i] = 0.12593918054482717 * r->w[i];
    for (int i = 4; i < 7; ++i) r->w[i] = 0.13239415278850616 * r->w[i];
  } else if (order == 6) {
    const double a = 0.873821971016996, b = 0.063089014491502, c = 0.501426509658179, d = 0.249286745170910;
    const double e = 0.636502499121399, f = 0.310352451033785, g = 0.053145049844816;
    add(a, b); add(b, a); add(b, b); add(c, d); add(d, c); add(d, d);
    add(e, f); add(e, g); add(f, e); add(f, g); add(g, e); add(g, f);
    r->w.assign(12, 0.5);
    for (int i = 0; i < 3; ++i) r->w[i] = 0.050844906370207 * r->w[i];
    for (int i = 3; i < 6; ++i) r->w[i] = 0.116786275726379 * r->w[i];
    for (int i = 6; i < 12; ++i) r->w[i] = 0.082851075618374 * r->w[i];
  } else {
    return false;
  }
  return true;
}

// Grundmann–Möller simplex rule of index s in 2D, src/GrundmannMoellerQuad.jl:11-26
// (Grundmann & Möller, SIAM J. Numer. Anal. 15 (1978)): nodes are the barycentric
// compositions of s-i into 3 parts, weights (-1)^i 2^(-2s) (d+n-2i)^d / (i! (d+n-i)!),
// normalised so that they sum to 1/2.
void grundmann_moeller(int s, Rule2* r) {
  r->w.clear(); r->x.clear(); r->y.clear();
  const int n = 2, d = 2 * s + 1;
  auto fact = [](int k) { double f = 1; for (int i = 2; i <= k; ++i) f *= i; return f; };
  for (int i = 0; i <= s; ++i) {
    double w = ((i % 2) ? -1.0 : 1.0) * std::pow(2.0, -2.0 * s) * std::pow((double)(d + n - 2 * i), d) /
               (fact(i) * fact(d + n - i));
    int t = s - i;
    // compositions (p0,p1,p2) of t, the point uses p1, p2
    for (int p2 = 0; p2 <= t; ++p2)
      for (int p1 = 0; p1 <= t - p2; ++p1) {
        r->x.push_back((2.0 * p1 + 1) / (d + n - 2 * i));
        r->y.push_back((2.0 * p2 + 1) / (d + n - 2 * i));
        r->w.push_back(w);
      }
  }
  double sum = 0;
  for (double w : r->w) sum += 2 * w;
  for (double& w : r->w) w = w / sum;
}

// QuadratureRule{2}(DefaultQuad(), order), src/quadrature.jl:17-26
bool default_quad2(int order, Rule2* r) {
  if (order <= 6) return strang(order, r);
  if (order % 2 == 1) {
    grundmann_moeller((order - 1) / 2, r);
    return true;
  }
  return false;
}

// gausslegendre(n) mapped to (0,1), src/quadrature.jl:29-35 (weights *= 0.5; (x+1)/2)
void gauss_legendre01(int n, Rule1* r) {
  r->w.assign(n, 0.0);
  r->x.assign(n, 0.0);
  std::vector<long double> xs(n), ws(n);
  for (int i = 0; i < n; ++i) {
    long double x = std::cos(3.14159265358979323846264338327950288L * (i + 0.75L) / (n + 0.5L));
    for (int it = 0; it < 100; ++it) {
      long double p0 = 1, p1 = x;
      for (int k = 2; k <= n; ++k) {
        long double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      if (n == 1) { p1 = x; p0 = 1; }
      long double dp = n * (x * p1 - p0) / (x * x - 1);
      long double dx = p1 / dp;
      x -= dx;
      if (std::fabs((double)dx) < 1e-30) break;
    }
    long double p0 = 1, p1 = x;
    for (int k = 2; k <= n; ++k) {
      long double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    if (n == 1) { p1 = x; p0 = 1; }
    long double dp = n * (x * p1 - p0) / (x * x - 1);
    xs[i] = x;
    ws[i] = 2 / ((1 - x * x) * dp * dp);
  }
  // ascending order, as FastGaussQuadrature returns
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  std::sort(idx.begin(), idx.end(), [&](int a, int b) { return xs[a] < xs[b]; });
  for (int i = 0; i < n; ++i) {
    double x = (double)xs[idx[i]], w = (double)ws[idx[i]];
    w *= 0.5;
    x = x + 1.0;
    x /= 2.0;
    r->w[i] = w;
    r->x[i] = x;
  }
}

// reference edges of the triangle, src/shapes.jl:19-23
const double REF_EDGE[3][2][2] = {{{1, 0}, {0, 1}}, {{0, 1}, {0, 0}}, {{0, 0}, {1, 0}}};
// local edge -> local nodes (1-based in Julia: (2,3),(3,1),(1,2)), src/shapes.jl:24
const int EDGE_NODES[3][2] = {{1, 2}, {2, 0}, {0, 1}};

// ---------------------------------------------------------------- tables
struct Tables {
  int p, qd, nw, nt, nq, nfq;
  Rule2 vol;
  Rule1 face;
  std::vector<double> N;    // [nw][nq]
  std::vector<double> dN;   // [nw][nq][2]
  std::vector<double> M;    // [3][nq] (P1 geometry)
  std::vector<double> E;    // [nw][nfq][3]
  std::vector<double> T;    // [nt][nfq]
};

// _scalar_fs tables (src/ScalarFunctionSpaces.jl:31-99) + trace tables
// (src/TraceFunctionSpaces.jl:11-28); face points via src/quadrature.jl:60-75.
bool build_tables(int p, int qd, Tables* t) {
  t->p = p;
  t->qd = qd;
  t->nw = (p + 1) * (p + 2) / 2;
  t->nt = p + 1;
  if (!default_quad2(qd, &t->vol)) return false;
  gauss_legendre01(qd, &t->face);  // QuadratureRule{1}(DefaultQuad(), qd) -> gausslegendre(qd)
  t->nq = (int)t->vol.w.size();
  t->nfq = (int)t->face.w.size();
  t->N.assign(t->nw * t->nq, 0);
  t->dN.assign(t->nw * t->nq * 2, 0);
  t->M.assign(3 * t->nq, 0);
  for (int q = 0; q < t->nq; ++q) {
    double x = t->vol.x[q], y = t->vol.y[q];
    for (int i = 0; i < t->nw; ++i) {
      Dual v = dubiner_value(i + 1, Dual(x, 1, 0), Dual(y, 0, 1));
      t->N[i * t->nq + q] = v.v;
      t->dN[(i * t->nq + q) * 2 + 0] = v.dx;
      t->dN[(i * t->nq + q) * 2 + 1] = v.dy;
    }
    t->M[0 * t->nq + q] = 1.0 - x - y;
    t->M[1 * t->nq + q] = x;
    t->M[2 * t->nq + q] = y;
  }
  t->E.assign(t->nw * t->nfq * 3, 0);
  for (int f = 0; f < 3; ++f)
    for (int q = 0; q < t->nfq; ++q) {
      double s = t->face.x[q];
      double ex = (1.0 - s) * REF_EDGE[f][0][0] + s * REF_EDGE[f][1][0];
      double ey = (1.0 - s) * REF_EDGE[f][0][1] + s * REF_EDGE[f][1][1];
      for (int i = 0; i < t->nw; ++i) t->E[(i * t->nfq + q) * 3 + f] = dubiner_value(i + 1, ex, ey);
    }
  t->T.assign(t->nt * t->nfq, 0);
  for (int k = 0; k < t->nt; ++k)
    for (int q = 0; q < t->nfq; ++q) t->T[k * t->nfq + q] = legendre_value(k + 1, t->face.x[q]);
  return true;
}

// ---------------------------------------------------------------- fields
// A field is (kind, params).  Kinds are shared with the GPU library's own evaluator.
enum { F_CONST = 0, F_SINSIN = 1, F_BUMPS = 2, F_FOURIER = 3, F_EXP_FOURIER = 4 };
struct Field {
  int kind = F_CONST;
  std::vector<double> prm{0.0};
};
double eval_field(const Field& f, double x, double y) {
  const double* p = f.prm.data();
  switch (f.kind) {
    case F_CONST: return p[0];
    case F_SINSIN: return p[0] * std::sin(p[1] * M_PI * x) * std::sin(p[2] * M_PI * y);
    case F_BUMPS: {
      int K = (int)p[0];
      double s = 0;
      for (int k = 0; k < K; ++k) {
        const double* b = p + 1 + 4 * k;
        double dx = x - b[0], dy = y - b[1];
        s += b[3] * std::exp(-(dx * dx + dy * dy) / (2.0 * b[2] * b[2]));
      }
      return s;
    }
    case F_FOURIER:
    case F_EXP_FOURIER: {
      int K = (int)p[0];
      double g = p[1];
      for (int k = 0; k < K; ++k) {
        const double* b = p + 2 + 4 * k;
        g += b[3] * std::cos(2.0 * M_PI * (b[0] * x + b[1] * y) + b[2]);
      }
      return f.kind == F_EXP_FOURIER ? std::exp(g) : g;
    }
  }
  return 0.0;
}

// ---------------------------------------------------------------- mesh
struct Mesh {
  std::vector<double> xy;            // [nn][2]
  std::vector<int> cells;            // [nc][3] 1-based node ids
  std::vector<int> cfaces;           // [nc][3] 1-based face ids
  std::vector<int> faces;            // [nf][4] v1 v2 c1 c2 (1-based, c2 = 0 on boundary)
  std::map<std::string, std::vector<int>> facesets;  // sorted
  int nn() const { return (int)xy.size() / 2; }
  int nc() const { return (int)cells.size() / 3; }
  int nf() const { return (int)faces.size() / 4; }
};

// _check_node_data: swap vertices 2,3 if clockwise, src/generate_mesh.jl:49-57
void check_node_data(const Mesh& m, int n1, int n2, int n3, int out[3]) {
  const double* a1 = &m.xy[2 * (n1 - 1)];
  const double* a2 = &m.xy[2 * (n2 - 1)];
  const double* a3 = &m.xy[2 * (n3 - 1)];
  double ax = a2[0] - a1[0], ay = a2[1] - a1[1], bx = a3[0] - a1[0], by = a3[1] - a1[1];
  if ((ax * by - ay * bx) < 0) {
    out[0] = n1; out[1] = n3; out[2] = n2;
  } else {
    out[0] = n1; out[1] = n2; out[2] = n3;
  }
}

// _build_cells: first-visit face numbering, src/generate_mesh.jl:20-46
void build_cell(Mesh& m, std::map<std::pair<int, int>, int>& dict, const int el[3], int n_el,
                std::vector<int>* boundary_new, const std::map<std::pair<int, int>, int>* markers) {
  int ef[3];
  for (int i = 0; i < 3; ++i) {
    int v1 = el[EDGE_NODES[i][0]], v2 = el[EDGE_NODES[i][1]];
    auto key = std::make_pair(std::min(v1, v2), std::max(v1, v2));
    auto it = dict.find(key);
    if (it != dict.end()) {
      ef[i] = it->second;
      if (m.faces[4 * (it->second - 1) + 3] != n_el) m.faces[4 * (it->second - 1) + 3] = n_el;
    } else {
      int fid = m.nf() + 1;
      m.faces.push_back(v1);
      m.faces.push_back(v2);
      m.faces.push_back(n_el);
      m.faces.push_back(0);
      dict[key] = fid;
      ef[i] = fid;
      if (markers && boundary_new) {  // src/triangle_mesh.jl:81-96
        auto mk = markers->find(key);
        if (mk != markers->end() && mk->second > 0) boundary_new->push_back(fid);
      }
    }
  }
  for (int i = 0; i < 3; ++i) {
    m.cells.push_back(el[i]);
    m.cfaces.push_back(ef[i]);
  }
}

}  // namespace

extern "C" {

typedef struct hr_mesh hr_mesh;

// rectangle_mesh(TriangleCell, (nx,ny), LL, UR), src/generate_mesh.jl:110-143
void* hr_rect_mesh(int nx, int ny, double llx, double lly, double urx, double ury) {
  Mesh* m = new Mesh();
  const double LL[2] = {llx, lly}, UR[2] = {urx, ury}, LR[2] = {urx, lly}, UL[2] = {llx, ury};
  const int NX = nx + 1, NY = ny + 1;
  // _generate_2d_nodes!, src/generate_mesh.jl:1-18
  for (int i = 0; i < NY; ++i) {
    double rb = (double)i / (double)(NY - 1);
    double x0 = LL[0] * (1 - rb) + rb * UL[0];
    double x1 = LR[0] * (1 - rb) + rb * UR[0];
    double y0 = LL[1] * (1 - rb) + rb * UL[1];
    double y1 = LR[1] * (1 - rb) + rb * UR[1];
    for (int j = 0; j < NX; ++j) {
      double r = (double)j / (double)(NX - 1);
      m->xy.push_back(x0 * (1 - r) + r * x1);
      m->xy.push_back(y0 * (1 - r) + r * y1);
    }
  }
  std::map<std::pair<int, int>, int> dict;
  auto nid = [&](int i, int j) { return i + (j - 1) * NX; };
  int n_el = 0;
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      int el[3];
      check_node_data(*m, nid(i, j), nid(i + 1, j), nid(i, j + 1), el);
      build_cell(*m, dict, el, ++n_el, nullptr, nullptr);
      check_node_data(*m, nid(i + 1, j), nid(i + 1, j + 1), nid(i, j + 1), el);
      build_cell(*m, dict, el, ++n_el, nullptr, nullptr);
    }
  // _get_rectangular_boundary_sets, src/generate_mesh.jl:60-89
  std::vector<int> bottom, right, top, left, all;
  for (int k = 1; k <= m->nf(); ++k) {
    const int* f = &m->faces[4 * (k - 1)];
    if (f[3] != 0) continue;
    const double* a = &m->xy[2 * (f[0] - 1)];
    const double* b = &m->xy[2 * (f[1] - 1)];
    if (a[1] == LL[1] && b[1] == LL[1]) bottom.push_back(k);
    else if (a[0] == UR[0] && b[0] == UR[0]) right.push_back(k);
    else if (a[1] == UR[1] && b[1] == UR[1]) top.push_back(k);
    else if (a[0] == LL[0] && b[0] == LL[0]) left.push_back(k);
    else { delete m; return nullptr; }  // "Face k belongs to one cell but is not in boundary"
    all.push_back(k);
  }
  m->facesets["bottom"] = bottom;
  m->facesets["right"] = right;
  m->facesets["top"] = top;
  m->facesets["left"] = left;
  m->facesets["boundary"] = all;
  return m;
}

// parse_cells! face construction for a Triangle-format mesh, src/triangle_mesh.jl:48-108.
// The text parsing itself is done by the Python side of the oracle.
void* hr_mesh_from_triangle(int nn, const double* xy, int nc, const int* ele, int ne, const int* edges) {
  Mesh* m = new Mesh();
  m->xy.assign(xy, xy + 2 * nn);
  std::map<std::pair<int, int>, int> markers;  // parse_faces!, src/triangle_mesh.jl:72-92
  for (int e = 0; e < ne; ++e) {
    auto key = std::make_pair(std::min(edges[3 * e], edges[3 * e + 1]), std::max(edges[3 * e], edges[3 * e + 1]));
    if (!markers.count(key)) markers[key] = edges[3 * e + 2];
  }
  std::map<std::pair<int, int>, int> dict;
  std::vector<int> bnd;
  for (int c = 0; c < nc; ++c) {
    int el[3];
    check_node_data(*m, ele[3 * c], ele[3 * c + 1], ele[3 * c + 2], el);
    build_cell(*m, dict, el, c + 1, &bnd, &markers);
  }
  std::sort(bnd.begin(), bnd.end());
  m->facesets["boundary"] = bnd;
  return m;
}

void hr_mesh_free(void* m) { delete (Mesh*)m; }
void hr_mesh_sizes(const void* mv, int* nn, int* nc, int* nf) {
  const Mesh* m = (const Mesh*)mv;
  *nn = m->nn(); *nc = m->nc(); *nf = m->nf();
}
void hr_mesh_arrays(const void* mv, double* xy, int* cells, int* cfaces, int* faces) {
  const Mesh* m = (const Mesh*)mv;
  if (xy) std::memcpy(xy, m->xy.data(), m->xy.size() * sizeof(double));
  if (cells) std::memcpy(cells, m->cells.data(), m->cells.size() * sizeof(int));
  if (cfaces) std::memcpy(cfaces, m->cfaces.data(), m->cfaces.size() * sizeof(int));
  if (faces) std::memcpy(faces, m->faces.data(), m->faces.size() * sizeof(int));
}
void hr_mesh_set_xy(void* mv, const double* xy) {
  Mesh* m = (Mesh*)mv;
  std::memcpy(m->xy.data(), xy, m->xy.size() * sizeof(double));
}
// getfaceset(mesh, name) as a sorted list; returns the count (or -1 if unknown)
int hr_mesh_faceset(const void* mv, const char* name, int* out) {
  const Mesh* m = (const Mesh*)mv;
  auto it = m->facesets.find(name);
  if (it == m->facesets.end()) return -1;
  std::vector<int> v = it->second;
  std::sort(v.begin(), v.end());
  if (out) std::memcpy(out, v.data(), v.size() * sizeof(int));
  return (int)v.size();
}

// Reference tables of the scalar/trace spaces.
int hr_table_sizes(int p, int qd, int* nq, int* nfq) {
  Tables t;
  if (!build_tables(p, qd, &t)) return -1;
  *nq = t.nq;
  *nfq = t.nfq;
  return 0;
}
int hr_tables(int p, int qd, double* vx, double* vy, double* vw, double* N, double* dN, double* fx, double* fw,
              double* E, double* T) {
  Tables t;
  if (!build_tables(p, qd, &t)) return -1;
  std::memcpy(vx, t.vol.x.data(), t.nq * 8);
  std::memcpy(vy, t.vol.y.data(), t.nq * 8);
  std::memcpy(vw, t.vol.w.data(), t.nq * 8);
  std::memcpy(N, t.N.data(), t.N.size() * 8);
  std::memcpy(dN, t.dN.data(), t.dN.size() * 8);
  std::memcpy(fx, t.face.x.data(), t.nfq * 8);
  std::memcpy(fw, t.face.w.data(), t.nfq * 8);
  std::memcpy(E, t.E.data(), t.E.size() * 8);
  std::memcpy(T, t.T.data(), t.T.size() * 8);
  return 0;
}
// Dubiner closed form versus generic Jacobi form (src/basis.jl:65-86 vs :169-218), for the
// reference's own basis KAT (test/test_basis.jl:34-39).
void hr_dubiner(int j, double x, double y, int generic, double* v, double* gx, double* gy) {
  Dual d = generic ? dubiner_generic(j, Dual(x, 1, 0), Dual(y, 0, 1)) : dubiner_value(j, Dual(x, 1, 0), Dual(y, 0, 1));
  *v = d.v; *gx = d.dx; *gy = d.dy;
}
double hr_legendre(int k, double x) { return legendre_value(k, x); }
// Raw quadrature rules (Strang kind=0, Grundmann–Möller kind=1, Gauss–Legendre kind=2).
int hr_rule(int kind, int order, double* x, double* y, double* w) {
  if (kind == 2) {
    Rule1 r;
    gauss_legendre01(order, &r);
    if (x) std::memcpy(x, r.x.data(), r.x.size() * 8);
    if (w) std::memcpy(w, r.w.data(), r.w.size() * 8);
    return (int)r.w.size();
  }
  Rule2 r;
  if (kind == 0) {
    if (!strang(order, &r)) return -1;
  } else {
    grundmann_moeller(order, &r);
  }
  if (x) std::memcpy(x, r.x.data(), r.x.size() * 8);
  if (y) std::memcpy(y, r.y.data(), r.y.size() * 8);
  if (w) std::memcpy(w, r.w.data(), r.w.size() * 8);
  return (int)r.w.size();
}

}  // extern "C"

namespace {

// reinit!(::ScalarFunctionSpace, x), src/ScalarFunctionSpaces.jl:101-132 (+ weighted_normal
// src/shapes.jl:80-87).  P1 geometry: dMdξ = (-1,-1),(1,0),(0,1).
struct Geo {
  double detJ, J[2][2], Jinv[2][2], detJf[3], nrm[3][2];
};
bool reinit_geo(const Mesh& m, int c, Geo* g) {
  const int* nd = &m.cells[3 * c];
  const double* x1 = &m.xy[2 * (nd[0] - 1)];
  const double* x2 = &m.xy[2 * (nd[1] - 1)];
  const double* x3 = &m.xy[2 * (nd[2] - 1)];
  // J = Σ x_j ⊗ dMdξ_j
  const double dM[3][2] = {{-1, -1}, {1, 0}, {0, 1}};
  const double* X[3] = {x1, x2, x3};
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b) {
      double s = 0;
      for (int j = 0; j < 3; ++j) s += X[j][a] * dM[j][b];
      g->J[a][b] = s;
    }
  g->detJ = g->J[0][0] * g->J[1][1] - g->J[0][1] * g->J[1][0];
  if (!(g->detJ > 0.0)) return false;  // ArgumentError("det(J) is not positive")
  double id = 1.0 / g->detJ;
  g->Jinv[0][0] = g->J[1][1] * id;
  g->Jinv[0][1] = -g->J[0][1] * id;
  g->Jinv[1][0] = -g->J[1][0] * id;
  g->Jinv[1][1] = g->J[0][0] * id;
  const double (*J)[2] = g->J;
  double wn[3][2] = {{-(J[1][0] - J[1][1]), J[0][0] - J[0][1]}, {-J[1][1], J[0][1]}, {J[1][0], -J[0][0]}};
  for (int l = 0; l < 3; ++l) {
    double nn = std::sqrt(wn[l][0] * wn[l][0] + wn[l][1] * wn[l][1]);
    g->nrm[l][0] = wn[l][0] / nn;
    g->nrm[l][1] = wn[l][1] / nn;
    g->detJf[l] = nn;
    if (!(nn > 0.0)) return false;
  }
  return true;
}

// face_orientation(mesh, cell, face), src/mesh.jl:51-54
inline bool orientation(const Mesh& m, int c, int f) {
  const int* nd = &m.cells[3 * c];
  return nd[EDGE_NODES[f][1]] > nd[EDGE_NODES[f][0]];
}

struct Blocks {
  int nw, nv, nt, m, n;
  std::vector<double> A, B, C, E, F, H, be;  // row-major
};

// Element integrals of doassemble, examples/poisson2D_HDG.jl:88-153.  kappa_inv scales the
// (σ,v) mass term (κ ≡ 1 in the reference); fx/kx select the source and coefficient.
void element_blocks(const Mesh& m, const Tables& t, int c, double tau, const Field& fsrc, const Field* kfield,
                    double kappa_cell, const Geo& g, Blocks* b) {
  const int nw = t.nw, nv = 2 * nw, nt = t.nt, mm = 3 * nt;
  b->nw = nw; b->nv = nv; b->nt = nt; b->m = mm; b->n = nv + nw;
  b->A.assign(nv * nv, 0); b->B.assign(nv * nw, 0); b->C.assign(nw * nw, 0);
  b->E.assign(nv * mm, 0); b->F.assign(nw * mm, 0); b->H.assign(mm * mm, 0); b->be.assign(nw, 0);
  // shape_gradient / dNdx = dNdξ ⋅ Jinv, src/ScalarFunctionSpaces.jl:114-116
  std::vector<double> dNdx(nw * t.nq * 2);
  for (int i = 0; i < nw; ++i)
    for (int q = 0; q < t.nq; ++q)
      for (int k = 0; k < 2; ++k) {
        const double* d = &t.dN[(i * t.nq + q) * 2];
        dNdx[(i * t.nq + q) * 2 + k] = d[0] * g.Jinv[0][k] + d[1] * g.Jinv[1][k];
      }
  const int* nd = &m.cells[3 * c];
  const double* X[3] = {&m.xy[2 * (nd[0] - 1)], &m.xy[2 * (nd[1] - 1)], &m.xy[2 * (nd[2] - 1)]};
  // Cell integrals, examples/poisson2D_HDG.jl:88-104
  for (int q = 0; q < t.nq; ++q) {
    double dO = g.detJ * t.vol.w[q];  // getdetJdV, src/ScalarFunctionSpaces.jl:138
    double xq = 0, yq = 0;            // spatial_coordinate, src/DiscreteFunctions.jl:16-24
    for (int i = 0; i < 3; ++i) {
      xq += t.M[i * t.nq + q] * X[i][0];
      yq += t.M[i * t.nq + q] * X[i][1];
    }
    double kinv = 1.0 / (kfield ? eval_field(*kfield, xq, yq) : kappa_cell);
    for (int i = 0; i < nv; ++i) {
      int ci = i / nw, ai = i % nw;  // VectorFunctionSpace component-major, src/VectorFunctionSpaces.jl:28-34
      double vi = t.N[ai * t.nq + q];
      double divv = dNdx[(ai * t.nq + q) * 2 + ci];  // tr(shape_gradient), :36-47
      for (int j = 0; j < nv; ++j) {
        int cj = j / nw, aj = j % nw;
        double dot = (ci == cj) ? t.N[aj * t.nq + q] * vi : 0.0;
        b->A[i * nv + j] += dot * kinv * dO;
      }
      for (int j = 0; j < nw; ++j) b->B[i * nw + j] += (t.N[j * t.nq + q] * divv) * dO;
    }
  }
  // RHS, examples/poisson2D_HDG.jl:106-114 (function_value, src/DiscreteFunctions.jl:6-9)
  for (int q = 0; q < t.nq; ++q) {
    double dO = g.detJ * t.vol.w[q];
    double xq = 0, yq = 0;
    for (int i = 0; i < 3; ++i) {
      xq += t.M[i * t.nq + q] * X[i][0];
      yq += t.M[i * t.nq + q] * X[i][1];
    }
    double fh = eval_field(fsrc, xq, yq);
    for (int i = 0; i < nw; ++i) b->be[i] += fh * t.N[i * t.nq + q] * dO;
  }
  // Face integrals, examples/poisson2D_HDG.jl:116-153
  const int nfq = t.nfq;
  for (int f = 0; f < 3; ++f) {
    bool o = orientation(m, c, f);
    for (int q = 0; q < nfq; ++q) {
      double dS = g.detJf[f] * t.face.w[q];  // getfacedetJdS, src/ScalarFunctionSpaces.jl:152
      int qf = o ? q : nfq - 1 - q;          // shape_value(..., orientation), :303
      for (int i = 0; i < nw; ++i) {
        double w = t.E[(i * nfq + q) * 3 + f];
        for (int j = 0; j < nw; ++j) b->C[i * nw + j] += tau * (t.E[(j * nfq + q) * 3 + f] * w) * dS;
        double wf = t.E[(i * nfq + qf) * 3 + f];
        for (int j = 0; j < nt; ++j) b->F[i * mm + nt * f + j] += (tau * (t.T[j * nfq + q] * wf)) * dS;
      }
      // trace space shares the parent's detJf (src/TraceFunctionSpaces.jl:34)
      for (int i = 0; i < nv; ++i) {
        int ci = i / nw, ai = i % nw;
        double vn = t.E[(ai * nfq + qf) * 3 + f] * g.nrm[f][ci];  // v ⋅ n, src/VectorFunctionSpaces.jl:50-57
        for (int j = 0; j < nt; ++j) b->E[i * mm + nt * f + j] += (t.T[j * nfq + q] * vn) * dS;
      }
      for (int i = 0; i < nt; ++i)
        for (int j = 0; j < nt; ++j)
          b->H[(nt * f + i) * mm + nt * f + j] += (t.T[j * nfq + q] * t.T[i * nfq + q]) * dS;  // no τ (:149)
    }
  }
}

// Dense LU with partial pivoting (getrf) and solve (getrs) on a row-major n×n matrix.
bool lu_factor(int n, double* a, int* piv) {
  for (int k = 0; k < n; ++k) {
    int p = k;
    double mx = std::fabs(a[k * n + k]);
    for (int i = k + 1; i < n; ++i)
      if (std::fabs(a[i * n + k]) > mx) { mx = std::fabs(a[i * n + k]); p = i; }
    piv[k] = p;
    if (mx == 0.0) return false;
    if (p != k)
      for (int j = 0; j < n; ++j) std::swap(a[k * n + j], a[p * n + j]);
    double inv = 1.0 / a[k * n + k];
    for (int i = k + 1; i < n; ++i) {
      double l = a[i * n + k] * inv;
      a[i * n + k] = l;
      for (int j = k + 1; j < n; ++j) a[i * n + j] -= l * a[k * n + j];
    }
  }
  return true;
}
// solve for nrhs columns of a row-major n×nrhs matrix b (in place)
void lu_solve(int n, const double* a, const int* piv, int nrhs, double* b) {
  for (int k = 0; k < n; ++k)
    if (piv[k] != k)
      for (int j = 0; j < nrhs; ++j) std::swap(b[k * nrhs + j], b[piv[k] * nrhs + j]);
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < i; ++k) {
      double l = a[i * n + k];
      for (int j = 0; j < nrhs; ++j) b[i * nrhs + j] -= l * b[k * nrhs + j];
    }
  for (int i = n - 1; i >= 0; --i) {
    for (int k = i + 1; k < n; ++k) {
      double u = a[i * n + k];
      for (int j = 0; j < nrhs; ++j) b[i * nrhs + j] -= u * b[k * nrhs + j];
    }
    double d = a[i * n + i];
    for (int j = 0; j < nrhs; ++j) b[i * nrhs + j] /= d;
  }
}

struct System {
  int p, qd, nt, nw, n, m, ncells, ndofs;
  std::vector<int64_t> colptr, rowval;  // 0-based CSC
  std::vector<double> nzval, rhs;
  std::vector<double> Ke;  // [ncells][n][m]
  std::vector<double> be;  // [ncells][n]
  std::vector<int> cfaces; // [ncells][3] 1-based
};

}  // namespace

extern "C" {

// reinit! geometry for one cell (0-based cell index).  Returns 0, or -1 if det(J) <= 0.
int hr_cell_geometry(const void* mv, int c, double* detJ, double* Jinv4, double* detJf3, double* normals6) {
  Geo g;
  if (!reinit_geo(*(const Mesh*)mv, c, &g)) return -1;
  *detJ = g.detJ;
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b) Jinv4[2 * a + b] = g.Jinv[a][b];
  for (int l = 0; l < 3; ++l) {
    detJf3[l] = g.detJf[l];
    normals6[2 * l] = g.nrm[l][0];
    normals6[2 * l + 1] = g.nrm[l][1];
  }
  return 0;
}

static Field make_field(int kind, int np, const double* prm) {
  Field f;
  f.kind = kind;
  f.prm.assign(prm, prm + np);
  if (f.prm.empty()) f.prm.push_back(0.0);
  return f;
}

// Element blocks Ae (nv×nv), Be (nv×nw), Ce, Ee (nv×3nt), Fe (nw×3nt), He, be for one cell,
// all row-major; the golden-matrix KAT of test/test_FunctionSpace.jl:49-72,125,176-178.
int hr_element_blocks(const void* mv, int c, int p, int qd, double tau, int fkind, int fnp, const double* fprm,
                      double* A, double* B, double* C, double* E, double* F, double* H, double* be) {
  const Mesh& m = *(const Mesh*)mv;
  Tables t;
  if (!build_tables(p, qd, &t)) return -2;
  Geo g;
  if (!reinit_geo(m, c, &g)) return -1;
  Blocks b;
  Field fs = make_field(fkind, fnp, fprm);
  element_blocks(m, t, c, tau, fs, nullptr, 1.0, g, &b);
  std::memcpy(A, b.A.data(), b.A.size() * 8);
  std::memcpy(B, b.B.data(), b.B.size() * 8);
  std::memcpy(C, b.C.data(), b.C.size() * 8);
  std::memcpy(E, b.E.data(), b.E.size() * 8);
  std::memcpy(F, b.F.data(), b.F.size() * 8);
  std::memcpy(H, b.H.data(), b.H.size() * 8);
  std::memcpy(be, b.be.data(), b.be.size() * 8);
  return 0;
}

// doassemble, examples/poisson2D_HDG.jl:58-186: element loop, dense-LU condensation
// (:155-174), trace dof map (:176-181), triplet assembly (src/assembler.jl:31-40) and
// end_assemble's COO->CSC with duplicates summed (src/assembler.jl:47-49); rhs scatter-add
// (src/assembler.jl:55-60).  kappa: per-cell array (or null) or a field (kkind >= 0).
// Returns an opaque system, or null with *status set (-1 det(J)<=0, -2 bad rule, -3 singular).
// he_tau != 0 subtracts τ·He instead of He: the hybridised flux is q̂·n = q·n + τ(u - û), so the
// trace equation's He term carries τ; the reference leaves it out (:149), which agrees for τ = 1.
void* hr_assemble_ex(const void* mv, int p, int qd, double tau, int fkind, int fnp, const double* fprm, int kkind,
                     int knp, const double* kprm, const double* kappa_cell, int nthreads, int he_tau, int* status) {
  const double hs = he_tau ? tau : 1.0;
  const Mesh& m = *(const Mesh*)mv;
  Tables t;
  *status = 0;
  if (!build_tables(p, qd, &t)) { *status = -2; return nullptr; }
  Field fs = make_field(fkind, fnp, fprm);
  Field kf = make_field(kkind, knp, kprm);
  const int nw = t.nw, nv = 2 * nw, nt = t.nt, mm = 3 * nt, n = nv + nw, nc = m.nc();
  System* S = new System();
  S->p = p; S->qd = qd; S->nt = nt; S->nw = nw; S->n = n; S->m = mm; S->ncells = nc;
  S->ndofs = m.nf() * nt;
  S->Ke.assign((size_t)nc * n * mm, 0);
  S->be.assign((size_t)nc * n, 0);
  S->cfaces = m.cfaces;
  std::vector<double> Ate((size_t)nc * mm * mm), bte((size_t)nc * mm);
  int bad = 0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static) reduction(min : bad)
#endif
  for (int c = 0; c < nc; ++c) {
    Geo g;
    if (!reinit_geo(m, c, &g)) { bad = std::min(bad, -1); continue; }
    Blocks b;
    element_blocks(m, t, c, tau, fs, kkind >= 0 ? &kf : nullptr, kappa_cell ? kappa_cell[c] : 1.0, g, &b);
    // Me = [Ae -Be; Beᵀ Ce]
    std::vector<double> Me(n * n), rhs(n * (mm + 1), 0.0);
    std::vector<int> piv(n);
    for (int i = 0; i < nv; ++i) {
      for (int j = 0; j < nv; ++j) Me[i * n + j] = b.A[i * nv + j];
      for (int j = 0; j < nw; ++j) Me[i * n + nv + j] = -b.B[i * nw + j];
    }
    for (int i = 0; i < nw; ++i) {
      for (int j = 0; j < nv; ++j) Me[(nv + i) * n + j] = b.B[j * nw + i];
      for (int j = 0; j < nw; ++j) Me[(nv + i) * n + nv + j] = b.C[i * nw + j];
    }
    // [EFe | Bte] = [[-Ee; Fe] | [0; be]]
    for (int i = 0; i < nv; ++i)
      for (int j = 0; j < mm; ++j) rhs[i * (mm + 1) + j] = -b.E[i * mm + j];
    for (int i = 0; i < nw; ++i) {
      for (int j = 0; j < mm; ++j) rhs[(nv + i) * (mm + 1) + j] = b.F[i * mm + j];
      rhs[(nv + i) * (mm + 1) + mm] = b.be[i];
    }
    if (!lu_factor(n, Me.data(), piv.data())) { bad = std::min(bad, -3); continue; }
    lu_solve(n, Me.data(), piv.data(), mm + 1, rhs.data());
    double* K = &S->Ke[(size_t)c * n * mm];
    double* bl = &S->be[(size_t)c * n];
    for (int i = 0; i < n; ++i) {
      for (int j = 0; j < mm; ++j) K[i * mm + j] = rhs[i * (mm + 1) + j];
      bl[i] = rhs[i * (mm + 1) + mm];
    }
    // Ate = Geᵀ K_e - He with Ge = [Ee; Fe]ᵀ ; bte = -Ge b_e
    double* At = &Ate[(size_t)c * mm * mm];
    double* bt = &bte[(size_t)c * mm];
    for (int i = 0; i < mm; ++i) {
      for (int j = 0; j < mm; ++j) {
        double s = 0;
        for (int k = 0; k < nv; ++k) s += b.E[k * mm + i] * K[k * mm + j];
        for (int k = 0; k < nw; ++k) s += b.F[k * mm + i] * K[(nv + k) * mm + j];
        At[i * mm + j] = s - hs * b.H[i * mm + j];
      }
      double s = 0;
      for (int k = 0; k < nv; ++k) s += b.E[k * mm + i] * bl[k];
      for (int k = 0; k < nw; ++k) s += b.F[k * mm + i] * bl[nv + k];
      bt[i] = -s;
    }
  }
  if (bad < 0) { *status = bad; delete S; return nullptr; }
  // gdof, triplets, CSC
  const int N = S->ndofs;
  std::vector<int64_t> cnt(N + 1, 0);
  std::vector<int> gd(mm);
  S->rhs.assign(N, 0.0);
  for (int c = 0; c < nc; ++c) {
    for (int f = 0; f < 3; ++f)
      for (int j = 0; j < nt; ++j) gd[f * nt + j] = (m.cfaces[3 * c + f] - 1) * nt + j;  // 0-based
    for (int j = 0; j < mm; ++j) cnt[gd[j] + 1] += mm;
    for (int i = 0; i < mm; ++i) S->rhs[gd[i]] += bte[(size_t)c * mm + i];
  }
  for (int j = 0; j < N; ++j) cnt[j + 1] += cnt[j];
  std::vector<int64_t> row(cnt[N]);
  std::vector<double> v(cnt[N]);
  std::vector<int64_t> pos(cnt.begin(), cnt.end() - 1);
  for (int c = 0; c < nc; ++c) {
    for (int f = 0; f < 3; ++f)
      for (int j = 0; j < nt; ++j) gd[f * nt + j] = (m.cfaces[3 * c + f] - 1) * nt + j;
    const double* At = &Ate[(size_t)c * mm * mm];
    for (int j = 0; j < mm; ++j)
      for (int i = 0; i < mm; ++i) {
        int64_t q = pos[gd[j]]++;
        row[q] = gd[i];
        v[q] = At[i * mm + j];
      }
  }
  S->colptr.assign(N + 1, 0);
  for (int j = 0; j < N; ++j) {
    std::vector<std::pair<int64_t, int64_t>> e;  // (row, original position) -> stable order
    for (int64_t q = cnt[j]; q < cnt[j + 1]; ++q) e.push_back({row[q], q});
    std::stable_sort(e.begin(), e.end(), [](auto& a, auto& b) { return a.first < b.first; });
    for (size_t k = 0; k < e.size(); ++k) {
      if (k > 0 && e[k].first == e[k - 1].first) {
        S->nzval.back() += v[e[k].second];
      } else {
        S->rowval.push_back(e[k].first);
        S->nzval.push_back(v[e[k].second]);
      }
    }
    S->colptr[j + 1] = (int64_t)S->rowval.size();
  }
  return S;
}

void* hr_assemble(const void* mv, int p, int qd, double tau, int fkind, int fnp, const double* fprm, int kkind,
                  int knp, const double* kprm, const double* kappa_cell, int nthreads, int* status) {
  return hr_assemble_ex(mv, p, qd, tau, fkind, fnp, fprm, kkind, knp, kprm, kappa_cell, nthreads, 0, status);
}

void hr_system_free(void* s) { delete (System*)s; }
void hr_system_sizes(const void* sv, int* ndofs, int64_t* nnz, int* n, int* m) {
  const System* S = (const System*)sv;
  *ndofs = S->ndofs;
  *nnz = (int64_t)S->nzval.size();
  *n = S->n;
  *m = S->m;
}
void hr_system_csc(const void* sv, int64_t* colptr, int64_t* rowval, double* nzval, double* rhs) {
  const System* S = (const System*)sv;
  if (colptr) std::memcpy(colptr, S->colptr.data(), S->colptr.size() * 8);
  if (rowval) std::memcpy(rowval, S->rowval.data(), S->rowval.size() * 8);
  if (nzval) std::memcpy(nzval, S->nzval.data(), S->nzval.size() * 8);
  if (rhs) std::memcpy(rhs, S->rhs.data(), S->rhs.size() * 8);
}
void hr_system_set_csc_values(void* sv, const double* nzval, const double* rhs) {
  System* S = (System*)sv;
  if (nzval) std::memcpy(S->nzval.data(), nzval, S->nzval.size() * 8);
  if (rhs) std::memcpy(S->rhs.data(), rhs, S->rhs.size() * 8);
}
void hr_system_local(const void* sv, double* Ke, double* be) {
  const System* S = (const System*)sv;
  if (Ke) std::memcpy(Ke, S->Ke.data(), S->Ke.size() * 8);
  if (be) std::memcpy(be, S->be.data(), S->be.size() * 8);
}

// Dirichlet(::ScalarTraceFunctionSpace, mesh, faceset, g), src/boundary.jl:11-42, kept
// with its projection as written (accumulator not reset per basis function, parent volume
// weights, no detJf).  Fills dofs (1-based) and values; returns the count.
int hr_dirichlet(const void* mv, int p, int qd, const char* faceset, int gkind, int gnp, const double* gprm, int* dofs,
                 double* vals) {
  const Mesh& m = *(const Mesh*)mv;
  Tables t;
  if (!build_tables(p, qd, &t)) return -2;
  auto it = m.facesets.find(faceset);
  if (it == m.facesets.end()) return -1;
  std::vector<char> in(m.nf() + 1, 0);
  for (int f : it->second) in[f] = 1;
  Field g = make_field(gkind, gnp, gprm);
  const int nt = t.nt, nfq = t.nfq;
  int k = 0;
  for (int fidx = 1; fidx <= m.nf(); ++fidx) {
    if (!in[fidx]) continue;
    if (m.faces[4 * (fidx - 1) + 3] != 0) return -3;  // "Face is not in boundary"
    int c = m.faces[4 * (fidx - 1) + 2] - 1;
    int fl = 0;
    while (m.cfaces[3 * c + fl] != fidx) ++fl;
    bool o = orientation(m, c, fl);
    const int* nd = &m.cells[3 * c];
    double N = 0.0;
    for (int i = 0; i < nt; ++i) {
      for (int q = 0; q < nfq; ++q) {
        int oq = o ? q : nfq - 1 - q;  // spatial_coordinate(fs, face, q, x, orientation), src/TraceFunctionSpaces.jl:43-57
        double s = t.face.x[oq];
        // L = P1 geometry at the face point of local edge fl
        double ex = (1.0 - s) * REF_EDGE[fl][0][0] + s * REF_EDGE[fl][1][0];
        double ey = (1.0 - s) * REF_EDGE[fl][0][1] + s * REF_EDGE[fl][1][1];
        double L[3] = {1.0 - ex - ey, ex, ey};
        double xq = 0, yq = 0;
        for (int a = 0; a < 3; ++a) {
          xq += L[a] * m.xy[2 * (nd[a] - 1)];
          yq += L[a] * m.xy[2 * (nd[a] - 1) + 1];
        }
        N += t.vol.w[q] * eval_field(g, xq, yq) * t.T[i * nfq + q];
      }
      vals[k] = N;
      dofs[k] = fidx * nt - nt + (i + 1);
      ++k;
    }
  }
  return k;
}

// The L2 projection of g onto the trace basis of each boundary face: û_i = ∫₀¹ g μ_i ds with the
// face rule's weights (the trace basis is orthonormal on [0, 1], and |e| cancels against the
// trace mass matrix |e|·I).  Same dofs and order as hr_dirichlet; returns the count.
int hr_dirichlet_l2(const void* mv, int p, int qd, const char* faceset, int gkind, int gnp, const double* gprm,
                    int* dofs, double* vals) {
  const Mesh& m = *(const Mesh*)mv;
  Tables t;
  if (!build_tables(p, qd, &t)) return -2;
  auto it = m.facesets.find(faceset);
  if (it == m.facesets.end()) return -1;
  std::vector<char> in(m.nf() + 1, 0);
  for (int f : it->second) in[f] = 1;
  Field g = make_field(gkind, gnp, gprm);
  const int nt = t.nt, nfq = t.nfq;
  int k = 0;
  for (int fidx = 1; fidx <= m.nf(); ++fidx) {
    if (!in[fidx]) continue;
    if (m.faces[4 * (fidx - 1) + 3] != 0) return -3;
    int c = m.faces[4 * (fidx - 1) + 2] - 1;
    int fl = 0;
    while (m.cfaces[3 * c + fl] != fidx) ++fl;
    bool o = orientation(m, c, fl);
    const int* nd = &m.cells[3 * c];
    for (int i = 0; i < nt; ++i) {
      double u = 0.0;
      for (int q = 0; q < nfq; ++q) {
        int oq = o ? q : nfq - 1 - q;
        double s = t.face.x[oq];
        double ex = (1.0 - s) * REF_EDGE[fl][0][0] + s * REF_EDGE[fl][1][0];
        double ey = (1.0 - s) * REF_EDGE[fl][0][1] + s * REF_EDGE[fl][1][1];
        double L[3] = {1.0 - ex - ey, ex, ey};
        double xq = 0, yq = 0;
        for (int a = 0; a < 3; ++a) {
          xq += L[a] * m.xy[2 * (nd[a] - 1)];
          yq += L[a] * m.xy[2 * (nd[a] - 1) + 1];
        }
        u += t.face.w[q] * eval_field(g, xq, yq) * t.T[i * nfq + q];
      }
      vals[k] = u;
      dofs[k] = fidx * nt - nt + (i + 1);
      ++k;
    }
  }
  return k;
}

// apply!(K, f, dbc) with APPLY_TRANSPOSE, src/boundary.jl:121-175.
void hr_apply(void* sv, int nd, const int* dofs1, const double* vals) {
  System* S = (System*)sv;
  const int N = S->ndofs;
  auto diag = [&](int j) -> double* {
    for (int64_t q = S->colptr[j]; q < S->colptr[j + 1]; ++q)
      if (S->rowval[q] == j) return &S->nzval[q];
    return nullptr;
  };
  double z = 0;  // meandiag, :374-380
  for (int i = 0; i < N; ++i) {
    double* d = diag(i);
    z += std::fabs(d ? *d : 0.0);
  }
  double mdiag = z / N;
  for (int k = 0; k < nd; ++k) {
    int d = dofs1[k] - 1;
    double v = vals[k];
    if (v != 0)
      for (int64_t q = S->colptr[d]; q < S->colptr[d + 1]; ++q) S->rhs[S->rowval[q]] -= v * S->nzval[q];
  }
  std::vector<char> pres(N, 0);
  for (int k = 0; k < nd; ++k) pres[dofs1[k] - 1] = 1;
  for (int j = 0; j < N; ++j)
    for (int64_t q = S->colptr[j]; q < S->colptr[j + 1]; ++q)
      if (pres[j] || pres[S->rowval[q]]) S->nzval[q] = 0.0;
  for (int k = 0; k < nd; ++k) {
    int d = dofs1[k] - 1;
    *diag(d) = mdiag;
    S->rhs[d] = vals[k] * mdiag;
  }
}

// get_uσ!, examples/poisson2D_HDG.jl:197-212, with the trace slice generalised to
// (f-1)nt+1 : f nt.  q: [ncells][nv], u: [ncells][nw], uhat_cell: [ncells][3][nt].
void hr_recover(const void* sv, const double* uhat, double* q, double* u, double* uhat_cell) {
  const System* S = (const System*)sv;
  const int n = S->n, mm = S->m, nt = S->nt, nw = S->nw, nv = 2 * nw;
  for (int c = 0; c < S->ncells; ++c) {
    double ue[64];
    for (int f = 0; f < 3; ++f)
      for (int j = 0; j < nt; ++j) {
        ue[f * nt + j] = uhat[(S->cfaces[3 * c + f] - 1) * nt + j];
        if (uhat_cell) uhat_cell[((size_t)c * 3 + f) * nt + j] = ue[f * nt + j];
      }
    const double* K = &S->Ke[(size_t)c * n * mm];
    const double* bl = &S->be[(size_t)c * n];
    for (int i = 0; i < n; ++i) {
      double s = 0;
      for (int j = 0; j < mm; ++j) s += K[i * mm + j] * ue[j];
      s += bl[i];
      if (i < nv) q[(size_t)c * nv + i] = s;
      else u[(size_t)c * nw + (i - nv)] = s;
    }
  }
}

// errornorm(u_h, u_ex), src/DiscreteFunctions.jl:97-120: the SQUARED L2 error.
double hr_errornorm(const void* mv, int p, int qd, const double* u, int ukind, int unp, const double* uprm) {
  const Mesh& m = *(const Mesh*)mv;
  Tables t;
  if (!build_tables(p, qd, &t)) return -1.0;
  Field ue = make_field(ukind, unp, uprm);
  double Et = 0;
  for (int c = 0; c < m.nc(); ++c) {
    Geo g;
    if (!reinit_geo(m, c, &g)) return -1.0;
    const int* nd = &m.cells[3 * c];
    double El = 0;
    for (int q = 0; q < t.nq; ++q) {
      double dO = g.detJ * t.vol.w[q];
      double uh = 0;
      for (int i = 0; i < t.nw; ++i) uh += u[(size_t)c * t.nw + i] * t.N[i * t.nq + q];
      double xq = 0, yq = 0;
      for (int a = 0; a < 3; ++a) {
        xq += t.M[a * t.nq + q] * m.xy[2 * (nd[a] - 1)];
        yq += t.M[a * t.nq + q] * m.xy[2 * (nd[a] - 1) + 1];
      }
      double d = uh - eval_field(ue, xq, yq);
      El += d * d * dO;
    }
    Et += El;
  }
  return Et;
}

// Field evaluation, so that tests can check the GPU evaluator against the same definition.
double hr_eval_field(int kind, int np, const double* prm, double x, double y) {
  Field f = make_field(kind, np, prm);
  return eval_field(f, x, y);
}

// r = b - K x for a CSC matrix, accumulated in double-double arithmetic and rounded once: each
// product is split exactly with an FMA (Dekker/Kahan TwoProduct) and each row sum is carried as
// an unevaluated pair with Knuth's TwoSum.  The residual of an FP64 solution of K x = b is as
// small as the rounding of x itself, so a plain FP64 residual is mostly rounding noise; this one
// is accurate to about 2^-100 of the summed magnitudes, which lets the Python side refine the
// sparse direct solve of examples/poisson2D_HDG.jl:195 to the correctly rounded solution of the
// assembled FP64 system (iterative refinement with an extra-precise residual, Wilkinson 1963).
void hr_csc_residual_dd(int n, const int64_t* colptr, const int64_t* rowval, const double* nzval, const double* x,
                        const double* b, double* r) {
  std::vector<double> hi(b, b + n), lo(n, 0.0);
  for (int j = 0; j < n; ++j) {
    const double xj = x[j];
    for (int64_t k = colptr[j]; k < colptr[j + 1]; ++k) {
      const int64_t i = rowval[k];
      const double p = -nzval[k] * xj;
      const double e = std::fma(-nzval[k], xj, -p);  // -nzval*xj = p + e exactly
      const double s = hi[i] + p;
      const double bv = s - hi[i];
      const double err = (hi[i] - (s - bv)) + (p - bv);  // hi + p = s + err exactly
      hi[i] = s;
      lo[i] += err + e;
    }
  }
  for (int i = 0; i < n; ++i) r[i] = hi[i] + lo[i];
}

}  // extern "C"
