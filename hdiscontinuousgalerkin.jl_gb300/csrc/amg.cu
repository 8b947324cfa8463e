// Smoothed-aggregation algebraic multigrid (SA-AMG) V-cycle used as the preconditioner of the
// trace CG (an alternative to Jacobi).  It has no reference counterpart: the reference solves
// K \ b with a sparse direct solver (examples/poisson2D_HDG.jl:195).
//
// Method (Vanek, Mandel & Brezina 1996; Vanek, Brezina & Mandel 2001).
//  * Level 0 is the trace matrix itself: faces with nt dofs each, in the block-ELL layout.  The
//    near-null space is the constant trace (Legendre mode 0 = 1 on every face).  Faces are
//    aggregated greedily on the graph of their strong couplings (faces of a common cell whose
//    mode-0 coupling is at least theta times the geometric mean of their diagonals); Dirichlet
//    faces (decoupled after apply!) belong to no aggregate.  The tentative prolongator puts
//    1/sqrt(|J|) on the mode-0 row of every face of aggregate J.
//  * Level l >= 1 is a scalar CSR matrix.  Its nodes are aggregated on the quotient of the level
//    below's graph; the tentative prolongator normalises the near-null vector carried down
//    (B_{l+1}[J] = |B_l restricted to J|).
//  * Smoothed prolongator P = (I - w D^-1 A) P_tent: D is the face-block diagonal (nt x nt) on
//    level 0 with w = 4/(3 lambda), lambda a Gershgorin bound of D^-1 A per problem, and the
//    l1 row sums on the coarse levels with w = 4/3 (their spectrum lies in (0, 1]).
//  * Coarse operator A_{l+1} = P' A P.  Coarsening stops once every problem has at most 96
//    coarse rows; the coarsest systems are inverted densely, one per problem.
//  * V(2,2) cycle: degree-2 Chebyshev smoothing with the face-block diagonal on level 0 (the
//    interval [lambda/30, lambda] of D^-1 A), two l1-Jacobi sweeps on the coarse levels, exact
//    coarsest solve.  Pre- and post-smoothing apply the same polynomial, so the cycle is a
//    symmetric positive definite preconditioner.
//
// Level-0 aggregates follow the strong couplings of the matrix assembled when the symbolic setup
// runs (strength of connection on the constant trace mode, theta = 0.2); coarser aggregates depend
// only on the graph.  The symbolic setup (aggregates, every sparsity pattern, the P' lists) runs
// once per system on the host, at its first multigrid solve, and is kept when the system is
// reassembled: with new coefficients the preconditioner stays symmetric positive definite and
// valid, fitted to the first ones.  The numeric setup (block inverses, bounds, P, A P, P' A P,
// coarsest inverses) runs on the device after every assembly.  Batched systems are block diagonal: aggregates never cross problems,
// so each problem gets its own hierarchy inside the shared arrays.
//
// Everything in the hierarchy and the cycle is FP32: the preconditioner only has to be a fixed
// SPD approximation.  All sums run in a fixed order, so the cycle is deterministic.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <numeric>
#include <thread>

#include <cuda_fp16.h>

#include "hdg_device.cuh"

namespace {

constexpr int AMG_MAX_COARSE = 96;  // per problem, dense inverse on the coarsest level
constexpr int AMG_MAX_LEVELS = 12;
constexpr int AMG_CINV_MAX = 150;   // largest dense coarsest block: (2 m^2 + m) floats of shared memory
constexpr int PW = 5;               // level-0 prolongator row width (a face and its 4 neighbours)
constexpr int AMG_TAIL_THREADS = 512;  // threads of a k_amg_tail CTA (one CTA per problem)

// Lanes per row of a coarse level with n rows (see the coarse-level kernels).
inline int amg_group(int n) { return n >= 16384 ? 4 : (n >= 2048 ? 8 : 32); }

constexpr int AMG_TAIL_MAXROWS = 4096;  // largest problem level the tail kernel may take
constexpr int AMG_ROW_SWEEP_FACES = 100000;  // untuned default: a thread per row below this many faces

// The coarse levels below some level T can be cycled by one k_amg_tail launch (one CTA per
// problem) instead of a launch per kernel per level; both give the same bits, and the V-cycle
// autotuner (amg_tune) picks T by timing.  HDG_AMG_TAIL_ROWS=k forces T = the first level whose
// largest problem has at most k rows (0: no tail) and leaves T out of the tuning; -1 (unset):
// tuned.
int amg_tail_rows() {
  static const int v = [] {
    const char* e = std::getenv("HDG_AMG_TAIL_ROWS");
    const int k = e ? std::atoi(e) : -1;
    return (k >= -1 && k <= 65536) ? k : -1;
  }();
  return v;
}

// Level-0 smoother variant: -1 tuned (default), 0 a thread per face, 1 a thread per row
// (HDG_AMG_SWEEP=face|row).  Both give the same bits.
int amg_sweep_forced() {
  static const int v = [] {
    const char* e = std::getenv("HDG_AMG_SWEEP");
    if (!e) return -1;
    if (std::strcmp(e, "face") == 0) return 0;
    if (std::strcmp(e, "row") == 0) return 1;
    return -1;
  }();
  return v;
}

// ---- host parallelism of the symbolic set-up ------------------------------------------------
// Rows of the set-up's per-row loops are independent; they run on up to 4 threads in contiguous
// ranges (the calling thread takes the first), and every range's output is concatenated in row
// order, so the hierarchy is the same as one built on one thread.
int set_up_ranges(int64_t n, int64_t grain = 16384) {
  static const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
  return (int)std::max<int64_t>(1, std::min<int64_t>(std::min(hw, 4), n / grain));
}
template <class F> void run_ranges(int64_t n, int k, F fn) {  // fn(range, begin, end)
  if (k <= 1) {
    fn(0, (int64_t)0, n);
    return;
  }
  std::vector<std::thread> ts;
  for (int t = 1; t < k; ++t) ts.emplace_back(fn, t, n * t / k, n * (t + 1) / k);
  fn(0, (int64_t)0, n / k);
  for (auto& t : ts) t.join();
}
// CSR rows [0, nr): rowfn(r, mark, out) appends the candidate columns of row r, using mark (one
// int per column, private to the range) to skip repeats within the row; each row's columns are
// then sorted.
template <class RowFn>
void build_csr(int nr, int ncol, RowFn rowfn, std::vector<int32_t>* ptr, std::vector<int32_t>* col) {
  const int k = set_up_ranges(nr);
  std::vector<std::vector<int32_t>> lc(k), lp(k);
  run_ranges(nr, k, [&](int t, int64_t a, int64_t b) {
    std::vector<int32_t> mark((size_t)std::max(ncol, 1), -1);
    std::vector<int32_t>& c = lc[t];
    std::vector<int32_t>& p = lp[t];
    p.reserve((size_t)(b - a));
    for (int64_t r = a; r < b; ++r) {
      const size_t start = c.size();
      rowfn((int)r, mark, c);
      std::sort(c.begin() + start, c.end());
      p.push_back((int32_t)c.size());
    }
  });
  ptr->assign((size_t)nr + 1, 0);
  size_t tot = 0;
  for (int t = 0; t < k; ++t) tot += lc[t].size();
  col->clear();
  col->reserve(tot);
  int64_t r = 0;
  for (int t = 0; t < k; ++t) {
    const int32_t off = (int32_t)col->size();
    for (int32_t e : lp[t]) (*ptr)[(size_t)++r] = off + e;
    col->insert(col->end(), lc[t].begin(), lc[t].end());
  }
}

// Greedy aggregation on an adjacency graph (CSR, symmetric, no self loops needed):
// 1. a node whose active neighbours are all free becomes a root with all of them;
// 2. a free node joins the aggregate of its first aggregated neighbour;
// 3. the rest become roots with their free neighbours.
// Aggregates are renumbered by their smallest member, so aggregates of one problem (whose nodes
// are contiguous) are contiguous too.
int aggregate(int n, const std::vector<int32_t>& ptr, const std::vector<int32_t>& adj, const std::vector<char>& active,
              std::vector<int32_t>* agg_out) {
  std::vector<int32_t>& agg = *agg_out;
  agg.assign(n, -1);
  int na = 0;
  for (int i = 0; i < n; ++i) {
    if (!active[i] || agg[i] >= 0) continue;
    bool free_all = true;
    for (int e = ptr[i]; e < ptr[i + 1]; ++e) {
      const int j = adj[e];
      if (j != i && active[j] && agg[j] >= 0) {
        free_all = false;
        break;
      }
    }
    if (!free_all) continue;
    agg[i] = na;
    for (int e = ptr[i]; e < ptr[i + 1]; ++e)
      if (active[adj[e]]) agg[adj[e]] = na;
    ++na;
  }
  for (int i = 0; i < n; ++i) {
    if (!active[i] || agg[i] >= 0) continue;
    for (int e = ptr[i]; e < ptr[i + 1]; ++e) {
      const int j = adj[e];
      if (j != i && active[j] && agg[j] >= 0) {
        agg[i] = agg[j];
        break;
      }
    }
  }
  for (int i = 0; i < n; ++i) {
    if (!active[i] || agg[i] >= 0) continue;
    agg[i] = na;
    for (int e = ptr[i]; e < ptr[i + 1]; ++e)
      if (active[adj[e]] && agg[adj[e]] < 0) agg[adj[e]] = na;
    ++na;
  }
  // renumber by smallest member
  std::vector<int32_t> first(na, INT32_MAX);
  for (int i = 0; i < n; ++i)
    if (agg[i] >= 0) first[agg[i]] = std::min(first[agg[i]], (int32_t)i);
  std::vector<int32_t> order(na);
  std::iota(order.begin(), order.end(), 0);
  std::sort(order.begin(), order.end(), [&](int a, int b) { return first[a] < first[b]; });
  std::vector<int32_t> rank(na);
  for (int k = 0; k < na; ++k) rank[order[k]] = k;
  for (int i = 0; i < n; ++i)
    if (agg[i] >= 0) agg[i] = rank[agg[i]];
  return na;
}

// Quotient graph of (ptr, adj) by agg: J ~ K when some member of J neighbours some member of K.
void quotient(int n, const std::vector<int32_t>& ptr, const std::vector<int32_t>& adj, const std::vector<int32_t>& agg,
              int na, std::vector<int32_t>* qptr, std::vector<int32_t>* qadj) {
  // members of each aggregate (counting sort keeps them in node order)
  std::vector<int32_t> mptr(na + 1, 0), mem;
  for (int i = 0; i < n; ++i)
    if (agg[i] >= 0) ++mptr[agg[i] + 1];
  for (int J = 0; J < na; ++J) mptr[J + 1] += mptr[J];
  mem.resize(mptr[na]);
  {
    std::vector<int32_t> fill(mptr.begin(), mptr.end() - 1);
    for (int i = 0; i < n; ++i)
      if (agg[i] >= 0) mem[fill[agg[i]]++] = i;
  }
  qptr->assign(na + 1, 0);
  qadj->clear();
  std::vector<int32_t> v;
  for (int J = 0; J < na; ++J) {
    v.clear();
    for (int t = mptr[J]; t < mptr[J + 1]; ++t) {
      const int i = mem[t];
      for (int e = ptr[i]; e < ptr[i + 1]; ++e) {
        const int j = adj[e];
        if (agg[j] >= 0 && agg[j] != J) v.push_back(agg[j]);
      }
    }
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
    qadj->insert(qadj->end(), v.begin(), v.end());
    (*qptr)[J + 1] = (int32_t)qadj->size();
  }
}

// Lists of entries per key, in entry order (counting sort): key[e] in [0, nk) or < 0 (skipped).
void bucket(int nk, const std::vector<int32_t>& key, std::vector<int32_t>* bptr, std::vector<int32_t>* bent) {
  bptr->assign(nk + 1, 0);
  for (size_t e = 0; e < key.size(); ++e)
    if (key[e] >= 0) ++(*bptr)[key[e] + 1];
  for (int k = 0; k < nk; ++k) (*bptr)[k + 1] += (*bptr)[k];
  bent->resize((*bptr)[nk]);
  std::vector<int32_t> fill(bptr->begin(), bptr->end() - 1);
  for (size_t e = 0; e < key.size(); ++e)
    if (key[e] >= 0) (*bent)[fill[key[e]]++] = (int32_t)e;
}

// Device copy of a host array that may be empty (a one-element buffer is kept so that kernels get
// a valid pointer; nothing reads it when the array is empty).
template <class T> void upload_min1(DevBuf<T>& d, const std::vector<T>& v, cudaStream_t st) {
  if (v.empty()) d.alloc(1);
  else d.upload(v.data(), v.size(), st);
}

}  // namespace

// ------------------------------------------------------------------------------------------
// Host-side structure
struct AmgLevel {  // a scalar level l >= 1 (rows = aggregates of level l-1)
  int n = 0;
  std::vector<int32_t> h_ptr, h_col;  // pattern of A_l (sorted columns, diagonal included)
  std::vector<int32_t> h_prob;        // problem of each row
  std::vector<double> h_B;            // near-null vector on this level
  DevBuf<int32_t> ptr, col;
  DevBuf<float> val, dl1inv;
  DevBuf<float> b, x, t, r;           // cycle vectors: rhs, iterate, sweep target, residual
  // transfer to the next level (all empty on the coarsest)
  int nc = 0;
  DevBuf<int32_t> prob;               // problem of each row (device copy of h_prob)
  DevBuf<int32_t> agg;                // aggregate of each row
  DevBuf<float> tent;                 // tentative weight of each row
  DevBuf<int32_t> pptr, pcol;         // P (CSR, sorted columns)
  DevBuf<float> pval;
  DevBuf<int32_t> apptr, apcol;       // A P pattern
  DevBuf<float> apval;
  DevBuf<int32_t> rptr, rent, rrow;   // P': per coarse row the P entries (index, fine row)
  DevBuf<int32_t> prow0;              // [nprob+1] first row of each problem (rows are grouped by problem)
  int maxrows = 0;                    // rows of the largest problem
};

// One level as the tail kernel (k_amg_tail) reads it.
struct TailLevel {
  int g;                                      // lanes per row (amg_group of the level's rows)
  const int32_t *ptr, *col, *prow0;
  const float *val, *dl1inv;
  float *b, *x, *t, *r;
  const int32_t *pptr, *pcol, *rptr, *rent, *rrow;  // transfer to the next level
  const float* pval;
};

struct AmgHierarchy {
  int nf = 0, nt = 0, nprob = 0;
  // level 0 (faces)
  DevBuf<int32_t> agg0;      // [nf] aggregate (-1: Dirichlet face)
  DevBuf<float> tent0;       // [nf]
  DevBuf<int32_t> pcol0;     // [nf][PW] prolongator columns (-1 pad), shared by the face's nt rows
  DevBuf<float> pval0;       // [nf*nt][PW]
  int wap = 0;               // width of an A0 P0 row
  DevBuf<int32_t> apcol0;    // [nf][wap]
  DevBuf<int8_t> apmap0;     // [nf][5 slots][PW]: position of pcol0[g_k][c] in apcol0[f]
  DevBuf<float> apval0;      // [nf*nt][wap]
  DevBuf<int32_t> rptr0, rent0;  // P0': per coarse row J the (face*PW + c) entries with pcol0 == J
  DevBuf<float> dinv0;       // [nf][nt][nt]
  DevBuf<float> lam0;        // [nprob] Gershgorin bound of D^-1 A0
  DevBuf<int32_t> face_prob; // [nf]
  DevBuf<float> val0f;       // FP32 trace matrix (set-up products); with FP32 cycle storage, D^-1 A0 afterwards
  DevBuf<__half> val0h;      // D^-1 A0 in FP16, read by the cycle's level-0 sweeps (default storage)
  DevBuf<float> x0, r0, d0;  // level-0 cycle vectors (iterate, scaled residual, Chebyshev correction)
  DevBuf<float> bt0;         // D^-1 b of the current cycle
  DevBuf<float> dpval0;      // [nf*nt][PW] D P0 (restriction of the scaled residual)
  std::vector<AmgLevel> lev; // lev[0] is level 1
  // coarsest (last level): per-problem dense inverses
  std::vector<int32_t> h_crow0;  // [nprob+1] first coarsest row of each problem
  DevBuf<int32_t> crow0, coff;   // coff: offset of each problem's dense block
  DevBuf<float> cinv;
  int cmax = 0;
  int tail_from = -1;        // first level (index into lev) cycled by k_amg_tail; -1: none
  std::vector<int> tail_cands; // levels the tail may start at (problems' rows <= AMG_TAIL_MAXROWS)
  DevBuf<TailLevel> tail_tab;  // every level's arrays for k_amg_tail
  bool row_sweep = false;    // level-0 smoother, residual and prolongation: a thread per row (else per face)
  bool tuned = false;        // the V-cycle autotuner has run (or its choice was taken from its cache)
  bool built = false;
};

void destroy_amg(AmgHierarchy* h) { delete h; }

namespace {
// The (0,0) entry (constant trace mode) of each of the 5 block slots of every face row.
__global__ void k_amg_mode0(int nf, int nt, const double* __restrict__ val, double* __restrict__ out) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= 5 * (int64_t)nf) return;
  const int k = (int)(t / nf), f = (int)(t - (int64_t)k * nf);
  const int64_t ndofs = (int64_t)nf * nt;
  out[t] = val[(int64_t)(k * nt) * ndofs + (int64_t)f * nt];
}

// Strength threshold of the level-0 aggregation (HDG_AMG_THETA; 0 = aggregate on every coupling).
// Measured on the 256-problem batch (kappa per cell over four decades, degree-4 Chebyshev):
// theta = 0 / 0.02 / 0.05 / 0.1 / 0.15 / 0.2 / 0.25 / 0.35 gave 541 / 716 / 834 / 912 / 921 / 930 /
// 893 / 873 solves/s (mean CG iterations 162 / 106 / 86 / 74 / 70 / 69 / 70 / 71); with kappa = 1
// (2*256^2 cells, p = 2) 0.2 changes nothing (95 iterations), and on 2*128^2 cells at p = 4 it
// takes 52 iterations instead of 68.
double amg_theta() {
  static const double th = [] {
    const char* e = std::getenv("HDG_AMG_THETA");
    const double v = e ? std::atof(e) : 0.2;
    return (v >= 0.0 && v < 1.0) ? v : 0.2;
  }();
  return th;
}
}  // namespace

// ------------------------------------------------------------------------------------------
// Symbolic setup
void amg_setup_symbolic(hdg_system* s, const std::vector<char>& dirichlet_face) {
  const bool verbose = std::getenv("HDG_AMG_VERBOSE") != nullptr;
  auto clk = [] { return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count(); };
  double tph[8] = {clk(), 0, 0, 0, 0, 0, 0, 0};
  if (s->amg) destroy_amg(s->amg);
  s->amg = new AmgHierarchy();
  ++s->amg_gen;
  AmgHierarchy* H = s->amg;
  const int nf = s->nf, nt = s->nt;
  H->nf = nf;
  H->nt = nt;
  H->nprob = s->nprob;
  const hdg_mesh* m = s->space->mesh;
  cudaStream_t st = s->ctx->stream;
  // face graph and problem of each face
  std::vector<int32_t> fptr(nf + 1, 0), fadj;
  std::vector<int32_t> fprob(nf, 0);
  for (int P = 0; P < s->nprob; ++P)
    for (int f = m->prob_face0[P]; f < m->prob_face0[P + 1]; ++f) fprob[f] = P;
  for (int f = 0; f < nf; ++f) {
    for (int e = s->h_browptr[f]; e < s->h_browptr[f + 1]; ++e)
      if (s->h_bcol[e] != f) fadj.push_back(s->h_bcol[e]);
    fptr[f + 1] = (int32_t)fadj.size();
  }
  std::vector<char> active(nf);
  for (int f = 0; f < nf; ++f) active[f] = !dirichlet_face[f];
  std::vector<int32_t> bcol5((size_t)5 * nf);
  s->d_bcol5.download(bcol5.data(), bcol5.size(), st);
  HDG_CUDA(cudaStreamSynchronize(st));
  // Level-0 aggregation graph: all face couplings, or (theta > 0) only the strong ones,
  // |a_fg| >= theta sqrt(a_ff a_gg) on the constant trace mode (the near-null space), from the
  // matrix assembled when the setup runs.  With kappa jumping between cells, a face's couplings
  // through a low-kappa cell are weak next to its diagonal, and aggregates that span such a jump
  // interpolate the smooth error badly (Vanek, Mandel & Brezina 1996, strength of connection).
  const double theta = amg_theta();
  std::vector<int32_t> sptr(fptr), sadj(fadj);
  if (theta > 0.0) {
    DevBuf<double> d_m0;
    d_m0.alloc((size_t)5 * nf);
    k_amg_mode0<<<(unsigned)((5 * (int64_t)nf + 255) / 256), 256, 0, st>>>(nf, nt, s->d_val.p, d_m0.p);
    HDG_CUDA(cudaGetLastError());
    s->ctx->launches++;
    std::vector<double> m0((size_t)5 * nf);
    d_m0.download(m0.data(), m0.size(), st);
    HDG_CUDA(cudaStreamSynchronize(st));
    std::vector<double> dg(nf, 0.0);
    run_ranges(nf, set_up_ranges(nf), [&](int, int64_t a, int64_t b) {
      for (int64_t f = a; f < b; ++f)
        for (int k = 0; k < 5; ++k)
          if (bcol5[(size_t)k * nf + f] == f) dg[f] = std::max(dg[f], std::fabs(m0[(size_t)k * nf + f]));
    });
    // g is a strong neighbour of f when the coupling is strong in f's row or in g's (symmetric
    // closure); each face's row is formed from the two rows alone
    auto strong = [&](int f, int k) {
      const int g = bcol5[(size_t)k * nf + f];
      return std::fabs(m0[(size_t)k * nf + f]) >= theta * std::sqrt(dg[f] * dg[g]);
    };
    build_csr(
        nf, nf,
        [&](int f, std::vector<int32_t>& mark, std::vector<int32_t>& out) {
          for (int k = 0; k < 5; ++k) {
            const int g = bcol5[(size_t)k * nf + f];
            if (g == f || mark[g] == f) continue;
            bool st_ = strong(f, k);
            for (int kk = 0; kk < 5 && !st_; ++kk)
              if (bcol5[(size_t)kk * nf + g] == f) st_ = strong(g, kk);
            if (st_) {
              mark[g] = f;
              out.push_back(g);
            }
          }
        },
        &sptr, &sadj);
  }
  tph[1] = clk();
  std::vector<int32_t> agg0;
  const int na0 = aggregate(nf, sptr, sadj, active, &agg0);
  tph[2] = clk();
  std::vector<int> size0(na0, 0);
  for (int f = 0; f < nf; ++f)
    if (agg0[f] >= 0) ++size0[agg0[f]];
  std::vector<float> tent0(nf, 0.f);
  for (int f = 0; f < nf; ++f)
    if (agg0[f] >= 0) tent0[f] = (float)(1.0 / std::sqrt((double)size0[agg0[f]]));
  // P0 pattern per face: aggregates of the face and its neighbours (active only)
  std::vector<int32_t> pcol0((size_t)nf * PW, -1);
  const int kf = set_up_ranges(nf);
  run_ranges(nf, kf, [&](int, int64_t a, int64_t b) {
    for (int64_t f = a; f < b; ++f) {
      if (!active[f]) continue;
      int cols[8], nc = 0;
      cols[nc++] = agg0[f];
      for (int e = fptr[f]; e < fptr[f + 1]; ++e)
        if (agg0[fadj[e]] >= 0) cols[nc++] = agg0[fadj[e]];
      std::sort(cols, cols + nc);
      nc = (int)(std::unique(cols, cols + nc) - cols);
      for (int c = 0; c < nc && c < PW; ++c) pcol0[(size_t)f * PW + c] = cols[c];
    }
  });
  // A0 P0 pattern per face: union over the 5 slot faces of their P0 columns
  // (at most 5 slots x PW columns = 25 entries per face, kept in a fixed-width table)
  constexpr int APW = 5 * PW;
  std::vector<int32_t> apc((size_t)nf * APW);
  std::vector<uint8_t> apn(nf);
  std::vector<int> wapr(kf, 1);
  run_ranges(nf, kf, [&](int t, int64_t a, int64_t b) {
    for (int64_t f = a; f < b; ++f) {
      int32_t* v = &apc[(size_t)f * APW];
      int n = 0;
      for (int k = 0; k < 5; ++k) {
        const int g = bcol5[(size_t)k * nf + f];
        for (int c = 0; c < PW; ++c)
          if (pcol0[(size_t)g * PW + c] >= 0) v[n++] = pcol0[(size_t)g * PW + c];
      }
      std::sort(v, v + n);
      n = (int)(std::unique(v, v + n) - v);
      apn[f] = (uint8_t)n;
      wapr[t] = std::max(wapr[t], n);
    }
  });
  const int wap = *std::max_element(wapr.begin(), wapr.end());
  if (wap > 32) throw HdgError{HDG_ERR_ARG, "AMG: prolongator pattern wider than 32 (invalid trace mesh)"};
  std::vector<int32_t> apcol0((size_t)nf * wap, -1);
  std::vector<int8_t> apmap0((size_t)nf * 5 * PW, -1);
  run_ranges(nf, kf, [&](int, int64_t a, int64_t b) {
    for (int64_t f = a; f < b; ++f) {
      const int32_t* v = &apc[(size_t)f * APW];
      const int n = apn[f];
      std::copy(v, v + n, apcol0.begin() + (size_t)f * wap);
      for (int k = 0; k < 5; ++k) {
        const int g = bcol5[(size_t)k * nf + f];
        for (int c = 0; c < PW; ++c) {
          const int J = pcol0[(size_t)g * PW + c];
          if (J < 0) continue;
          apmap0[((size_t)f * 5 + k) * PW + c] = (int8_t)(std::lower_bound(v, v + n, J) - v);
        }
      }
    }
  });
  tph[3] = clk();
  // P0' lists and the level-1 pattern (rows = aggregates)
  std::vector<int32_t> rptr0, rent0;  // entries f * PW + c of P0 per column, in entry order
  bucket(na0, pcol0, &rptr0, &rent0);
  AmgLevel L1;
  L1.n = na0;
  L1.h_ptr.assign(na0 + 1, 0);
  L1.h_prob.assign(na0, 0);
  L1.h_B.assign(na0, 0.0);
  // column unions below use a stamp per column (the row that last added it): each candidate is
  // looked at once, and only the distinct columns of a row are sorted
  build_csr(
      na0, na0,
      [&](int J, std::vector<int32_t>& mark, std::vector<int32_t>& out) {
        for (int t = rptr0[J]; t < rptr0[J + 1]; ++t) {
          const int f = rent0[t] / PW;
          for (int q = 0; q < apn[f]; ++q) {
            const int32_t c = apc[(size_t)f * APW + q];
            if (mark[c] != J) {
              mark[c] = J;
              out.push_back(c);
            }
          }
        }
      },
      &L1.h_ptr, &L1.h_col);
  for (int J = 0; J < na0; ++J) L1.h_B[J] = std::sqrt((double)size0[J]);
  for (int f = 0; f < nf; ++f)
    if (agg0[f] >= 0) L1.h_prob[agg0[f]] = fprob[f];
  tph[4] = clk();
  // quotient graph of the face graph for level 1's aggregation
  std::vector<int32_t> gptr, gadj;
  quotient(nf, fptr, fadj, agg0, na0, &gptr, &gadj);
  // upload level 0
  H->agg0.upload(agg0.data(), agg0.size(), st);
  H->tent0.upload(tent0.data(), tent0.size(), st);
  H->pcol0.upload(pcol0.data(), pcol0.size(), st);
  H->pval0.alloc((size_t)nf * nt * PW);
  H->wap = wap;
  H->apcol0.upload(apcol0.data(), apcol0.size(), st);
  H->apmap0.upload(apmap0.data(), apmap0.size(), st);
  H->apval0.alloc((size_t)nf * nt * wap);
  H->rptr0.upload(rptr0.data(), rptr0.size(), st);
  upload_min1(H->rent0, rent0, st);
  H->dinv0.alloc((size_t)nf * nt * nt);
  H->lam0.alloc(std::max(s->nprob, 1));
  H->face_prob.upload(fprob.data(), fprob.size(), st);
  H->x0.alloc((size_t)nf * nt);
  H->r0.alloc((size_t)nf * nt);
  H->d0.alloc((size_t)nf * nt);
  H->bt0.alloc((size_t)nf * nt);
  H->dpval0.alloc((size_t)nf * nt * PW);
  H->lev.clear();
  H->lev.push_back(std::move(L1));
  tph[5] = clk();
  // coarser levels
  auto max_per_problem = [&](const AmgLevel& L) {
    std::vector<int> cnt(s->nprob, 0);
    for (int i = 0; i < L.n; ++i) ++cnt[L.h_prob[i]];
    return cnt.empty() ? 0 : *std::max_element(cnt.begin(), cnt.end());
  };
  while ((int)H->lev.size() < AMG_MAX_LEVELS && max_per_problem(H->lev.back()) > AMG_MAX_COARSE) {
    AmgLevel& F = H->lev.back();
    const int n = F.n;
    std::vector<char> act(n, 1);
    std::vector<int32_t> agg;
    const int na = aggregate(n, gptr, gadj, act, &agg);
    if (na > (int)(0.85 * n)) break;  // no longer coarsening
    std::vector<double> nrm(na, 0.0);
    for (int i = 0; i < n; ++i) nrm[agg[i]] += F.h_B[i] * F.h_B[i];
    for (int J = 0; J < na; ++J) nrm[J] = std::sqrt(nrm[J]);
    std::vector<float> tent(n);
    for (int i = 0; i < n; ++i) tent[i] = nrm[agg[i]] > 0 ? (float)(F.h_B[i] / nrm[agg[i]]) : 0.f;
    auto add = [](std::vector<int32_t>& mark, std::vector<int32_t>& out, int32_t c, int32_t row) {
      if (mark[c] != row) {
        mark[c] = row;
        out.push_back(c);
      }
    };
    // P pattern row i: aggregates of the columns of A row i
    std::vector<int32_t> pptr, pcol;
    build_csr(
        n, na,
        [&](int i, std::vector<int32_t>& mark, std::vector<int32_t>& out) {
          for (int e = F.h_ptr[i]; e < F.h_ptr[i + 1]; ++e) add(mark, out, agg[F.h_col[e]], i);
        },
        &pptr, &pcol);
    // A P pattern row i: union of the P rows of A row i's columns
    std::vector<int32_t> apptr, apcol;
    build_csr(
        n, na,
        [&](int i, std::vector<int32_t>& mark, std::vector<int32_t>& out) {
          for (int e = F.h_ptr[i]; e < F.h_ptr[i + 1]; ++e) {
            const int k = F.h_col[e];
            for (int q = pptr[k]; q < pptr[k + 1]; ++q) add(mark, out, pcol[q], i);
          }
        },
        &apptr, &apcol);
    // P' lists and the next level's pattern
    std::vector<int32_t> prow_of(pcol.size());
    for (int i = 0; i < n; ++i)
      for (int e = pptr[i]; e < pptr[i + 1]; ++e) prow_of[e] = i;
    std::vector<int32_t> rptr, rent, rrow;  // entries of P per column, in entry order
    bucket(na, pcol, &rptr, &rent);
    rrow.resize(rent.size());
    for (size_t t = 0; t < rent.size(); ++t) rrow[t] = prow_of[rent[t]];
    AmgLevel C;
    C.n = na;
    C.h_prob.assign(na, 0);
    C.h_B = nrm;
    build_csr(
        na, na,
        [&](int J, std::vector<int32_t>& mark, std::vector<int32_t>& out) {
          for (int t = rptr[J]; t < rptr[J + 1]; ++t) {
            const int i = rrow[t];
            for (int q = apptr[i]; q < apptr[i + 1]; ++q) add(mark, out, apcol[q], J);
          }
        },
        &C.h_ptr, &C.h_col);
    for (int i = 0; i < n; ++i) C.h_prob[agg[i]] = F.h_prob[i];
    F.nc = na;
    F.agg.upload(agg.data(), agg.size(), st);
    F.tent.upload(tent.data(), tent.size(), st);
    F.pptr.upload(pptr.data(), pptr.size(), st);
    F.pcol.upload(pcol.data(), pcol.size(), st);
    F.pval.alloc(pcol.size());
    F.apptr.upload(apptr.data(), apptr.size(), st);
    F.apcol.upload(apcol.data(), apcol.size(), st);
    F.apval.alloc(apcol.size());
    F.rptr.upload(rptr.data(), rptr.size(), st);
    upload_min1(F.rent, rent, st);
    upload_min1(F.rrow, rrow, st);
    std::vector<int32_t> qptr, qadj;
    quotient(n, gptr, gadj, agg, na, &qptr, &qadj);
    gptr.swap(qptr);
    gadj.swap(qadj);
    H->lev.push_back(std::move(C));
  }
  tph[6] = clk();
  // device copies of every level's matrix pattern and vectors
  for (auto& L : H->lev) {
    L.ptr.upload(L.h_ptr.data(), L.h_ptr.size(), st);
    upload_min1(L.col, L.h_col, st);
    upload_min1(L.prob, L.h_prob, st);
    L.val.alloc(std::max<size_t>(L.h_col.size(), 1));
    L.dl1inv.alloc(std::max(L.n, 1));
    L.b.alloc(std::max(L.n, 1));
    L.x.alloc(std::max(L.n, 1));
    L.t.alloc(std::max(L.n, 1));
    L.r.alloc(std::max(L.n, 1));
  }
  // per-problem row ranges of every level (aggregates are numbered by their smallest member, so a
  // problem's rows are contiguous on every level) and the first level the tail kernel takes
  bool grouped = true;
  for (auto& L : H->lev) {
    std::vector<int32_t> r0(s->nprob + 1, 0);
    for (int i = 0; i < L.n; ++i) {
      if (i > 0 && L.h_prob[i] < L.h_prob[i - 1]) grouped = false;
      ++r0[L.h_prob[i] + 1];
    }
    L.maxrows = 0;
    for (int P = 0; P < s->nprob; ++P) {
      L.maxrows = std::max(L.maxrows, r0[P + 1]);
      r0[P + 1] += r0[P];
    }
    L.prow0.upload(r0.data(), r0.size(), st);
  }
  H->tail_from = -1;
  H->tail_cands.clear();
  H->tuned = false;
  H->row_sweep = nf < AMG_ROW_SWEEP_FACES;
  const int tail_rows = amg_tail_rows();
  if (grouped)
    for (int l = 1; l + 1 < (int)H->lev.size(); ++l) {
      if (tail_rows < 0 && H->lev[l].maxrows <= AMG_TAIL_MAXROWS) H->tail_cands.push_back(l);
      if (tail_rows > 0 && H->tail_from < 0 && H->lev[l].maxrows <= tail_rows) H->tail_from = l;
    }
  if (H->tail_from >= 0) H->tail_cands.assign(1, H->tail_from);
  // coarsest: per-problem dense blocks
  const AmgLevel& C = H->lev.back();
  H->h_crow0.assign(s->nprob + 1, 0);
  for (int i = 0; i < C.n; ++i) ++H->h_crow0[C.h_prob[i] + 1];
  for (int P = 0; P < s->nprob; ++P) H->h_crow0[P + 1] += H->h_crow0[P];
  std::vector<int32_t> coff(s->nprob + 1, 0);
  H->cmax = 0;
  for (int P = 0; P < s->nprob; ++P) {
    const int mP = H->h_crow0[P + 1] - H->h_crow0[P];
    H->cmax = std::max(H->cmax, mP);
    coff[P + 1] = coff[P] + mP * mP;
  }
  if (H->cmax > AMG_CINV_MAX)
    throw HdgError{HDG_ERR_ARG, "AMG: coarsening stalled above the dense coarsest size"};
  H->crow0.upload(H->h_crow0.data(), H->h_crow0.size(), st);
  H->coff.upload(coff.data(), coff.size(), st);
  H->cinv.alloc(std::max(coff[s->nprob], 1));
  if (!H->tail_cands.empty()) {
    std::vector<TailLevel> tab(H->lev.size());
    for (size_t l = 0; l < H->lev.size(); ++l) {
      const AmgLevel& L = H->lev[l];
      tab[l] = TailLevel{amg_group(L.n), L.ptr.p, L.col.p, L.prow0.p, L.val.p, L.dl1inv.p, L.b.p, L.x.p, L.t.p,
                         L.r.p, L.pptr.p, L.pcol.p, L.rptr.p, L.rent.p, L.rrow.p, L.pval.p};
    }
    H->tail_tab.upload(tab.data(), tab.size(), st);
  }
  H->built = true;
  if (verbose) {  // level sizes: rows (largest problem's rows; nonzeros); host time of the set-up phases (ms)
    tph[7] = clk();
    std::fprintf(stderr, "amg setup ms: strength %.1f agg0 %.1f p0 %.1f level1 %.1f upload0 %.1f coarse %.1f upload %.1f\n",
                 1e3 * (tph[1] - tph[0]), 1e3 * (tph[2] - tph[1]), 1e3 * (tph[3] - tph[2]), 1e3 * (tph[4] - tph[3]),
                 1e3 * (tph[5] - tph[4]), 1e3 * (tph[6] - tph[5]), 1e3 * (tph[7] - tph[6]));
    std::fprintf(stderr, "amg: %d problems, level 0: %d faces x %d", s->nprob, nf, nt);
    for (const AmgLevel& L : H->lev) {
      std::vector<int> cnt(s->nprob, 0);
      for (int i = 0; i < L.n; ++i) ++cnt[L.h_prob[i]];
      std::fprintf(stderr, ", %d (%d; %zu nnz)", L.n, *std::max_element(cnt.begin(), cnt.end()), L.h_col.size());
    }
    std::fprintf(stderr, "; tail from level %d\n", H->tail_from + 1);
  }
  HDG_CUDA(cudaStreamSynchronize(st));
}

// ------------------------------------------------------------------------------------------
// Numeric setup kernels
namespace {

// Inverse of each face's diagonal block (Gauss-Jordan, partial pivoting) and the per-problem
// Gershgorin bound of D^-1 A0: max over rows of sum_j |(D^-1 A0)_ij|.
template <int NT>
__global__ void k_amg_block_inv(int nf, const int32_t* __restrict__ bcol5, const int8_t* __restrict__ kdiag,
                                const float* __restrict__ val, const int32_t* __restrict__ face_prob,
                                float* __restrict__ dinv, float* __restrict__ lam) {
  // Threads past the end repeat the last face (whole warps stay for the reduction at the end) and
  // write nothing.
  const int fg = blockIdx.x * blockDim.x + threadIdx.x;
  if (fg - (int)(threadIdx.x & 31) >= nf) return;  // whole warps past the end
  const bool own = fg < nf;
  const int f = own ? fg : nf - 1;
  const int64_t nd = (int64_t)nf * NT;
  float a[NT][2 * NT];
  const int kd = kdiag[f];
  for (int i = 0; i < NT; ++i)
    for (int j = 0; j < NT; ++j) {
      a[i][j] = val[(kd * NT + j) * nd + (int64_t)f * NT + i];
      a[i][NT + j] = (i == j) ? 1.f : 0.f;
    }
  for (int c = 0; c < NT; ++c) {
    int piv = c;
    for (int i = c + 1; i < NT; ++i)
      if (fabsf(a[i][c]) > fabsf(a[piv][c])) piv = i;
    if (piv != c)
      for (int j = 0; j < 2 * NT; ++j) {
        const float t = a[c][j];
        a[c][j] = a[piv][j];
        a[piv][j] = t;
      }
    const float inv = (a[c][c] != 0.f) ? 1.f / a[c][c] : 0.f;
    for (int j = 0; j < 2 * NT; ++j) a[c][j] *= inv;
    for (int i = 0; i < NT; ++i) {
      if (i == c) continue;
      const float m = a[i][c];
      for (int j = 0; j < 2 * NT; ++j) a[i][j] -= m * a[c][j];
    }
  }
  if (own)
    for (int i = 0; i < NT; ++i)
      for (int j = 0; j < NT; ++j) dinv[((int64_t)f * NT + i) * NT + j] = a[i][NT + j];
  // row sums of |D^-1 A0| over the face's rows
  float rs[NT];
  for (int i = 0; i < NT; ++i) rs[i] = 0.f;
  for (int k = 0; k < 5; ++k) {
    const int g = bcol5[k * nf + f];
    if (k > 0 && g == f && k != kd) continue;  // padding slot (zero block)
    for (int j = 0; j < NT; ++j) {
      float col[NT];
      for (int i = 0; i < NT; ++i) col[i] = val[(k * NT + j) * nd + (int64_t)f * NT + i];
      for (int i = 0; i < NT; ++i) {
        float t = 0.f;
        for (int l = 0; l < NT; ++l) t += a[i][NT + l] * col[l];
        rs[i] += fabsf(t);
      }
    }
  }
  float mx = 0.f;
  for (int i = 0; i < NT; ++i) mx = fmaxf(mx, rs[i]);
  // one atomic per problem present in the warp (consecutive faces mostly share one): the lanes of
  // a problem take their maximum first (non-negative floats order like their bit patterns)
  const int P = own ? face_prob[f] : -1;
  const unsigned grp = __match_any_sync(0xffffffffu, P);
  const int mxi = __reduce_max_sync(grp, __float_as_int(mx));
  if (own && (int)(threadIdx.x & 31) == __ffs(grp) - 1) atomicMax(reinterpret_cast<int*>(lam + P), mxi);
}

// P0 = (I - w D^-1 A0) P_tent, w = 4/(3 lambda); one thread per face (all its nt rows).
template <int NT>
__global__ void k_amg_p0(int nf, const int32_t* __restrict__ bcol5, const float* __restrict__ val,
                         const float* __restrict__ dinv, const float* __restrict__ lam,
                         const int32_t* __restrict__ face_prob, const int32_t* __restrict__ agg0,
                         const float* __restrict__ tent0, const int32_t* __restrict__ pcol0,
                         float* __restrict__ pval0) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const int64_t nd = (int64_t)nf * NT;
  float out[NT][PW];
  for (int i = 0; i < NT; ++i)
    for (int c = 0; c < PW; ++c) out[i][c] = 0.f;
  if (pcol0[f * PW] < 0) {  // Dirichlet face: no prolongator rows
    for (int i = 0; i < NT; ++i)
      for (int c = 0; c < PW; ++c) pval0[((int64_t)f * NT + i) * PW + c] = 0.f;
    return;
  }
  const float w = (4.f / 3.f) / fmaxf(lam[face_prob[f]], 1e-30f);
  int done[5];
  int nd_ = 0;
  for (int k = 0; k < 5; ++k) {
    const int g = bcol5[k * nf + f];
    bool dup = false;
    for (int t = 0; t < nd_; ++t) dup |= (done[t] == g);
    if (dup) continue;  // padding slots repeat the face itself; its block is counted once (real slot)
    done[nd_++] = g;
    const int J = agg0[g];
    if (J < 0) continue;
    int c = 0;
    while (c < PW && pcol0[f * PW + c] != J) ++c;
    if (c == PW) continue;  // not in the pattern (cannot happen for a valid setup)
    // column (g, mode 0) of A0's block row f, for the real slot holding g
    int ks = k;
    for (int kk = 0; kk < 5; ++kk)
      if (bcol5[kk * nf + f] == g) { ks = kk; break; }
    float col[NT];
    for (int i = 0; i < NT; ++i) col[i] = val[(ks * NT + 0) * nd + (int64_t)f * NT + i];
    for (int i = 0; i < NT; ++i) {
      float t = 0.f;
      for (int l = 0; l < NT; ++l) t += dinv[((int64_t)f * NT + i) * NT + l] * col[l];
      out[i][c] -= w * t * tent0[g];
    }
  }
  {
    const int J = agg0[f];
    int c = 0;
    while (c < PW && pcol0[f * PW + c] != J) ++c;
    if (c < PW) out[0][c] += tent0[f];
  }
  for (int i = 0; i < NT; ++i)
    for (int c = 0; c < PW; ++c) pval0[((int64_t)f * NT + i) * PW + c] = out[i][c];
}

// A0 P0, one thread per fine row.
template <int NT>
__global__ void k_amg_ap0(int nf, int wap, const int32_t* __restrict__ bcol5, const float* __restrict__ val,
                          const int32_t* __restrict__ pcol0, const float* __restrict__ pval0,
                          const int8_t* __restrict__ apmap0, float* __restrict__ apval0) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nd = (int64_t)nf * NT;
  if (r >= nd) return;
  const int f = (int)(r / NT);
  float acc[32];
  for (int q = 0; q < wap && q < 32; ++q) acc[q] = 0.f;
  int seen[5];
  int ns = 0;
  for (int k = 0; k < 5; ++k) {
    const int g = bcol5[k * nf + f];
    bool dup = false;
    for (int t = 0; t < ns; ++t) dup |= (seen[t] == g);
    if (dup) continue;
    seen[ns++] = g;
    for (int j = 0; j < NT; ++j) {
      const float a = val[(k * NT + j) * nd + r];
      if (a == 0.f) continue;
      for (int c = 0; c < PW; ++c) {
        if (pcol0[g * PW + c] < 0) break;
        const int q = apmap0[((int64_t)f * 5 + k) * PW + c];
        if (q >= 0 && q < wap) acc[q] += a * pval0[((int64_t)g * NT + j) * PW + c];
      }
    }
  }
  for (int q = 0; q < wap; ++q) apval0[r * wap + q] = acc[q];
}

__device__ __forceinline__ int find_col(const int32_t* __restrict__ col, int a, int b, int key) {
  while (a < b) {  // lower bound in the sorted columns [a, b)
    const int m = (a + b) >> 1;
    if (col[m] < key) a = m + 1;
    else b = m;
  }
  return a;
}

// val[position of key in the sorted columns [a, b)] += v; a key outside the pattern is ignored
// (the symbolic setup puts every product's column in the pattern, so this never drops anything)
__device__ __forceinline__ void add_at(const int32_t* __restrict__ col, float* __restrict__ val, int a, int b, int key,
                                       float v) {
  const int e = find_col(col, a, b, key);
  if (e < b && col[e] == key) val[e] += v;
}

// A1 = P0' (A0 P0), one warp per coarse row.  For each of the row's P0' entries (face f, mode c)
// and each of the face's rows i in turn, the lanes take the entries of the A0 P0 row: their
// columns are distinct, so no two lanes add to the same coarse entry at once, and every entry
// receives its terms in the order (t, i) whatever the launch.
template <int NT>
__global__ void k_amg_rap0(int na, int wap, const int32_t* __restrict__ rptr0, const int32_t* __restrict__ rent0,
                           const float* __restrict__ pval0, const int32_t* __restrict__ apcol0,
                           const float* __restrict__ apval0, const int32_t* __restrict__ ptr1,
                           const int32_t* __restrict__ col1, float* __restrict__ val1) {
  const int64_t gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int J = (int)(gt >> 5), lane = threadIdx.x & 31;
  if (J >= na) return;  // whole warps
  const int a0 = ptr1[J], a1 = ptr1[J + 1];
  for (int e = a0 + lane; e < a1; e += 32) val1[e] = 0.f;
  __syncwarp();
  for (int t = rptr0[J]; t < rptr0[J + 1]; ++t) {
    const int f = rent0[t] / PW, c = rent0[t] - f * PW;
    for (int i = 0; i < NT; ++i) {
      const float p = pval0[((int64_t)f * NT + i) * PW + c];
      if (p == 0.f) continue;
      const float* apr = apval0 + ((int64_t)f * NT + i) * wap;
      for (int q = lane; q < wap; q += 32) {
        const int K = apcol0[(int64_t)f * wap + q];
        if (K >= 0) add_at(col1, val1, a0, a1, K, p * apr[q]);
      }
      __syncwarp();
    }
  }
}

// 1 / l1 row sums of a CSR level
__global__ void k_amg_dl1(int n, const int32_t* __restrict__ ptr, const float* __restrict__ val,
                          float* __restrict__ dl1inv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float s = 0.f;
  for (int e = ptr[i]; e < ptr[i + 1]; ++e) s += fabsf(val[e]);
  dl1inv[i] = s > 0.f ? 1.f / s : 0.f;
}

// P = (I - 4/3 D_l1^-1 A) P_tent on a CSR level, one thread per row
__global__ void k_amg_p(int n, const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                        const float* __restrict__ val, const float* __restrict__ dl1inv, const int32_t* __restrict__ agg,
                        const float* __restrict__ tent, const int32_t* __restrict__ pptr,
                        const int32_t* __restrict__ pcol, float* __restrict__ pval) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int p0 = pptr[i], p1 = pptr[i + 1];
  for (int e = p0; e < p1; ++e) pval[e] = 0.f;
  const float w = (4.f / 3.f) * dl1inv[i];
  for (int e = ptr[i]; e < ptr[i + 1]; ++e) {
    const int k = col[e];
    add_at(pcol, pval, p0, p1, agg[k], -w * val[e] * tent[k]);
  }
  add_at(pcol, pval, p0, p1, agg[i], tent[i]);
}

// A P on a CSR level, one warp per row: for each entry (i, k) of A's row in turn, the lanes take
// the entries of P's row k, whose columns are distinct (so no two lanes add to the same entry at
// once, and each entry receives its terms in the order of A's row).
__global__ void k_amg_ap(int n, const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                         const float* __restrict__ val, const int32_t* __restrict__ pptr,
                         const int32_t* __restrict__ pcol, const float* __restrict__ pval,
                         const int32_t* __restrict__ apptr, const int32_t* __restrict__ apcol,
                         float* __restrict__ apval) {
  const int64_t gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int i = (int)(gt >> 5), lane = threadIdx.x & 31;
  if (i >= n) return;  // whole warps
  const int a0 = apptr[i], a1 = apptr[i + 1];
  for (int e = a0 + lane; e < a1; e += 32) apval[e] = 0.f;
  __syncwarp();
  for (int e = ptr[i]; e < ptr[i + 1]; ++e) {
    const int k = col[e];
    const float a = val[e];
    for (int t = pptr[k] + lane; t < pptr[k + 1]; t += 32) add_at(apcol, apval, a0, a1, pcol[t], a * pval[t]);
    __syncwarp();
  }
}

// A_{l+1} = P' (A P), one warp per coarse row: for each of the row's P' entries (fine row i) in
// turn, the lanes take the entries of the A P row i (distinct columns), as in k_amg_rap0.
__global__ void k_amg_rap(int nc, const int32_t* __restrict__ rptr, const int32_t* __restrict__ rent,
                          const int32_t* __restrict__ rrow, const float* __restrict__ pval,
                          const int32_t* __restrict__ apptr, const int32_t* __restrict__ apcol,
                          const float* __restrict__ apval, const int32_t* __restrict__ cptr,
                          const int32_t* __restrict__ ccol, float* __restrict__ cval) {
  const int64_t gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int J = (int)(gt >> 5), lane = threadIdx.x & 31;
  if (J >= nc) return;  // whole warps
  const int a0 = cptr[J], a1 = cptr[J + 1];
  for (int e = a0 + lane; e < a1; e += 32) cval[e] = 0.f;
  __syncwarp();
  for (int t = rptr[J]; t < rptr[J + 1]; ++t) {
    const float p = pval[rent[t]];
    const int i = rrow[t];
    for (int q = apptr[i] + lane; q < apptr[i + 1]; q += 32) add_at(ccol, cval, a0, a1, apcol[q], p * apval[q]);
    __syncwarp();
  }
}

// Dense inverse of each problem's coarsest matrix (Gauss-Jordan with partial pivoting in shared
// memory, one CTA per problem).  Sizes are at most AMG_CINV_MAX (the symbolic setup checks).
__global__ void k_amg_coarse_inv(const int32_t* __restrict__ crow0, const int32_t* __restrict__ coff,
                                 const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                                 const float* __restrict__ val, float* __restrict__ cinv) {
  extern __shared__ float sm[];
  const int P = blockIdx.x;
  const int r0 = crow0[P], m = crow0[P + 1] - r0;
  if (m == 0) return;
  const int w = 2 * m;
  float* a = sm;          // m x 2m augmented matrix
  float* mult = sm + m * w;  // m multipliers of the current column
  __shared__ int piv;
  for (int t = threadIdx.x; t < m * w; t += blockDim.x) a[t] = 0.f;
  __syncthreads();
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    for (int e = ptr[r0 + i]; e < ptr[r0 + i + 1]; ++e) {
      const int c = col[e] - r0;
      if (c >= 0 && c < m) a[i * w + c] = val[e];
    }
    a[i * w + m + i] = 1.f;
  }
  __syncthreads();
  for (int c = 0; c < m; ++c) {
    if (threadIdx.x == 0) {
      int p = c;
      for (int i = c + 1; i < m; ++i)
        if (fabsf(a[i * w + c]) > fabsf(a[p * w + c])) p = i;
      piv = p;
    }
    __syncthreads();
    const int pr = piv;
    if (pr != c)
      for (int j = threadIdx.x; j < w; j += blockDim.x) {
        const float t = a[c * w + j];
        a[c * w + j] = a[pr * w + j];
        a[pr * w + j] = t;
      }
    __syncthreads();
    const float d = a[c * w + c];
    const float inv = d != 0.f ? 1.f / d : 0.f;
    __syncthreads();
    for (int j = threadIdx.x; j < w; j += blockDim.x) a[c * w + j] *= inv;
    for (int i = threadIdx.x; i < m; i += blockDim.x) mult[i] = (i == c) ? 0.f : a[i * w + c];
    __syncthreads();
    for (int t = threadIdx.x; t < m * w; t += blockDim.x) {
      const int i = t / w, j = t - i * w;
      if (i != c) a[t] -= mult[i] * a[c * w + j];
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < m * m; t += blockDim.x) {
    const int i = t / m, j = t - i * m;
    cinv[coff[P] + t] = a[i * w + m + j];
  }
}

// D P0 (D the face-block diagonal of A0), for the restriction of the scaled residual.
template <int NT>
__global__ void k_amg_dp0(int nf, const int8_t* __restrict__ kdiag, const float* __restrict__ val,
                          const float* __restrict__ pval0, float* __restrict__ dpval0) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const int64_t nd = (int64_t)nf * NT;
  const int kd = kdiag[f];
  for (int i = 0; i < NT; ++i)
    for (int c = 0; c < PW; ++c) {
      float s = 0.f;
      for (int l = 0; l < NT; ++l)
        s += val[(kd * NT + l) * nd + (int64_t)f * NT + i] * pval0[((int64_t)f * NT + l) * PW + c];
      dpval0[((int64_t)f * NT + i) * PW + c] = s;
    }
}

// Level-0 value storage of the cycle: FP32 or FP16, read as FP32.
template <typename VT> __device__ __forceinline__ VT to_vt(float v);
template <> __device__ __forceinline__ float to_vt<float>(float v) { return v; }
template <> __device__ __forceinline__ __half to_vt<__half>(float v) { return __float2half_rn(v); }
__device__ __forceinline__ float ldv(const float* p) { return *p; }
__device__ __forceinline__ float ldv(const __half* p) { return __half2float(*p); }

// A0 -> D^-1 A0, block row by block row, into `out` (FP32, which may be `val` itself: each face
// reads and rewrites only its own rows, or FP16).  Runs after every set-up product that needs A0
// itself; the cycle then needs no D^-1 per sweep.  The scaled diagonal block is I and the
// off-diagonal entries are of order one, well inside FP16's range; the rounding (2^-11 relative)
// changes the preconditioner, not the FP64 Krylov iteration around it.
template <int NT, typename VT>
__global__ void k_amg_scale0(int nf, const float* __restrict__ dinv, const float* val, VT* out) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const int64_t nd = (int64_t)nf * NT;
  float di[NT][NT];
  for (int i = 0; i < NT; ++i)
    for (int l = 0; l < NT; ++l) di[i][l] = dinv[((int64_t)f * NT + i) * NT + l];
  for (int k = 0; k < 5; ++k)
    for (int j = 0; j < NT; ++j) {
      float col[NT];
      for (int l = 0; l < NT; ++l) col[l] = val[(k * NT + j) * nd + (int64_t)f * NT + l];
      for (int i = 0; i < NT; ++i) {
        float s = 0.f;
        for (int l = 0; l < NT; ++l) s += di[i][l] * col[l];
        out[(k * NT + j) * nd + (int64_t)f * NT + i] = to_vt<VT>(s);
      }
    }
}

// ------------------------------------------------------------------------------------------
// Cycle kernels.  `st` is the CG's per-problem state (HDG_CG_ST ints per problem: status, ...,
// refine flag): rows of a problem that has stopped iterating and waits for no refinement are
// skipped, so the tail of a batch, where a few problems still iterate, does not pay for a
// V-cycle over every problem.  Their outputs keep stale values, which the CG never reads.
// st == NULL runs every row.
__device__ __forceinline__ bool amg_live(const int32_t* __restrict__ st, int P) {
  return !st || st[HDG_CG_ST * P] == 0 || st[HDG_CG_ST * P + 3] != 0;
}


// Level-0 smoother: step `step` of the Chebyshev iteration (Saad, Iterative Methods, 12.3) for
// D^-1 A0 on [lambda / ratio, lambda], D the face-block diagonal and lambda the problem's
// Gershgorin bound.  xin == NULL stands for x = 0 (no product); d holds the previous step's
// correction and is updated in place (each face reads and writes only its own rows of d).
template <int NT, typename VT>
__global__ void k_amg_face_cheb(int nf, const int32_t* __restrict__ bcol5, const VT* __restrict__ val,
                                const float* __restrict__ dinv, const float* __restrict__ lam,
                                const int32_t* __restrict__ face_prob, const float* __restrict__ b,
                                float* __restrict__ bt, const float* __restrict__ xin, float* __restrict__ xout,
                                float* __restrict__ d, int step, float ratio, const int32_t* __restrict__ st) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf || !amg_live(st, face_prob[f])) return;
  const int64_t nd = (int64_t)nf * NT;
  // t = D^-1 (b - A x) = bt - (D^-1 A) x: val holds the block rows of A scaled by D^-1, and
  // the first step (x = 0) forms bt = D^-1 b for the rest of the cycle
  float t[NT];
  if (!xin) {
    float bv[NT];
    for (int l = 0; l < NT; ++l) bv[l] = b[(int64_t)f * NT + l];
    for (int i = 0; i < NT; ++i) {
      float s = 0.f;
      for (int l = 0; l < NT; ++l) s += dinv[((int64_t)f * NT + i) * NT + l] * bv[l];
      t[i] = s;
      bt[(int64_t)f * NT + i] = s;
    }
  } else {
    for (int i = 0; i < NT; ++i) t[i] = bt[(int64_t)f * NT + i];
    // padding slots (faces with fewer than four neighbours) repeat the face with zero values,
    // so every slot is summed without a test and all loads can be issued up front
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      const int g = bcol5[k * nf + f];
#pragma unroll
      for (int j = 0; j < NT; ++j) {
        const float xv = xin[(int64_t)g * NT + j];
        for (int i = 0; i < NT; ++i) t[i] -= ldv(&val[(k * NT + j) * nd + (int64_t)f * NT + i]) * xv;
      }
    }
  }
  const float hi = fmaxf(lam[face_prob[f]], 1e-30f), lo = hi / ratio;
  const float theta = 0.5f * (hi + lo), delta = 0.5f * (hi - lo), sigma = theta / delta;
  float rp = 1.f / sigma, rc = rp;  // rho_{step-1}, rho_step
  for (int u = 1; u <= step; ++u) {
    rc = 1.f / (2.f * sigma - rp);
    if (u < step) rp = rc;
  }
  const float cd = (step == 0) ? 0.f : rc * rp, cr = (step == 0) ? 1.f / theta : 2.f * rc / delta;
  for (int i = 0; i < NT; ++i) {
    const int64_t row = (int64_t)f * NT + i;
    const float dn = cr * t[i] + (step == 0 ? 0.f : cd * d[row]);
    d[row] = dn;
    xout[row] = (xin ? xin[row] : 0.f) + dn;
  }
}

template <int NT, typename VT>
__global__ void k_amg_row_cheb(int nf, const int32_t* __restrict__ bcol5, const VT* __restrict__ val,
                                const float* __restrict__ dinv, const float* __restrict__ lam,
                                const int32_t* __restrict__ face_prob, const float* __restrict__ b,
                                float* __restrict__ bt, const float* __restrict__ xin, float* __restrict__ xout,
                                float* __restrict__ d, int step, float ratio, const int32_t* __restrict__ st) {
  // one thread per row (f, i): with the block rows scaled by D^-1 the rows of a face are
  // independent.  For small systems (too few faces to fill the GPU) this runs nt times more
  // threads than the face kernel; on large ones it re-reads each face's columns and neighbour
  // values nt times and loses (amg_row_sweeps)
  const int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nd = (int64_t)nf * NT;
  if (row >= nd) return;
  const int f = (int)(row / NT), i = (int)(row - (int64_t)f * NT);
  if (!amg_live(st, face_prob[f])) return;
  // t = D^-1 (b - A x) = bt - (D^-1 A) x: the first step (x = 0) forms bt = D^-1 b for the rest
  // of the cycle
  float t;
  if (!xin) {
    t = 0.f;
    for (int l = 0; l < NT; ++l) t += dinv[((int64_t)f * NT + i) * NT + l] * b[(int64_t)f * NT + l];
    bt[row] = t;
  } else {
    t = bt[row];
    // padding slots repeat the face with zero values: no test needed
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      const int g = bcol5[k * nf + f];
#pragma unroll
      for (int j = 0; j < NT; ++j) t -= ldv(&val[(k * NT + j) * nd + row]) * xin[(int64_t)g * NT + j];
    }
  }
  const float hi = fmaxf(lam[face_prob[f]], 1e-30f), lo = hi / ratio;
  const float theta = 0.5f * (hi + lo), delta = 0.5f * (hi - lo), sigma = theta / delta;
  float rp = 1.f / sigma, rc = rp;  // rho_{step-1}, rho_step
  for (int u = 1; u <= step; ++u) {
    rc = 1.f / (2.f * sigma - rp);
    if (u < step) rp = rc;
  }
  const float cd = (step == 0) ? 0.f : rc * rp, cr = (step == 0) ? 1.f / theta : 2.f * rc / delta;
  const float dn = cr * t + (step == 0 ? 0.f : cd * d[row]);
  d[row] = dn;
  xout[row] = (xin ? xin[row] : 0.f) + dn;
}

// scaled residual r~ = D^-1 (b - A0 x) = bt - (D^-1 A0) x (level 0); the restriction uses D P0
template <int NT, typename VT>
__global__ void k_amg_face_residual(int nf, const int32_t* __restrict__ bcol5, const VT* __restrict__ val,
                                    const float* __restrict__ b, const float* __restrict__ x, float* __restrict__ r,
                                    const int32_t* __restrict__ face_prob, const int32_t* __restrict__ st) {
  const int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nd = (int64_t)nf * NT;
  if (row >= nd) return;
  const int f = (int)(row / NT);
  if (!amg_live(st, face_prob[f])) return;
  float s = b[row];
  // padding slots repeat the face with zero values: no test needed
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const int g = bcol5[k * nf + f];
#pragma unroll
    for (int j = 0; j < NT; ++j) s -= ldv(&val[(k * NT + j) * nd + row]) * x[(int64_t)g * NT + j];
  }
  r[row] = s;
}

// The same residual with a thread per face (its nt rows): the face's block columns and neighbour
// values are read once instead of nt times; each row's operations are those of the row kernel.
template <int NT, typename VT>
__global__ void k_amg_face_residual_f(int nf, const int32_t* __restrict__ bcol5, const VT* __restrict__ val,
                                      const float* __restrict__ b, const float* __restrict__ x,
                                      float* __restrict__ r, const int32_t* __restrict__ face_prob,
                                      const int32_t* __restrict__ st) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf || !amg_live(st, face_prob[f])) return;
  const int64_t nd = (int64_t)nf * NT;
  float s[NT];
#pragma unroll
  for (int i = 0; i < NT; ++i) s[i] = b[(int64_t)f * NT + i];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const int g = bcol5[k * nf + f];
#pragma unroll
    for (int j = 0; j < NT; ++j) {
      const float xv = x[(int64_t)g * NT + j];
#pragma unroll
      for (int i = 0; i < NT; ++i) s[i] -= ldv(&val[(k * NT + j) * nd + (int64_t)f * NT + i]) * xv;
    }
  }
#pragma unroll
  for (int i = 0; i < NT; ++i) r[(int64_t)f * NT + i] = s[i];
}

// b1 = P0' r0 = (D P0)' r~0 and the first l1-Jacobi sweep of level 1: x1 = b1 / dl1
template <int NT>
__global__ void k_amg_restrict0(int na, const int32_t* __restrict__ rptr0, const int32_t* __restrict__ rent0,
                                const float* __restrict__ pval0, const float* __restrict__ r0,
                                const float* __restrict__ dl1inv, float* __restrict__ b1, float* __restrict__ x1,
                                const int32_t* __restrict__ prob1, const int32_t* __restrict__ st) {
  const int J = blockIdx.x * blockDim.x + threadIdx.x;
  if (J >= na || !amg_live(st, prob1[J])) return;
  float s = 0.f;
  for (int t = rptr0[J]; t < rptr0[J + 1]; ++t) {
    const int f = rent0[t] / PW, c = rent0[t] - f * PW;
    for (int i = 0; i < NT; ++i) s += pval0[((int64_t)f * NT + i) * PW + c] * r0[(int64_t)f * NT + i];
  }
  b1[J] = s;
  x1[J] = s * dl1inv[J];
}

// x0 += P0 x1
template <int NT>
__global__ void k_amg_prolong0(int nf, const int32_t* __restrict__ pcol0, const float* __restrict__ pval0,
                               const float* __restrict__ x1, float* __restrict__ x0,
                               const int32_t* __restrict__ face_prob, const int32_t* __restrict__ st) {
  const int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (row >= (int64_t)nf * NT) return;
  const int f = (int)(row / NT);
  if (!amg_live(st, face_prob[f])) return;
  float s = 0.f;
  for (int c = 0; c < PW; ++c) {
    const int J = pcol0[f * PW + c];
    if (J < 0) break;
    s += pval0[row * PW + c] * x1[J];
  }
  x0[row] += s;
}

// The same prolongation with a thread per face: the face's prolongator columns and coarse values
// are read once for its nt rows; each row's operations are those of the row kernel.
template <int NT>
__global__ void k_amg_prolong0_f(int nf, const int32_t* __restrict__ pcol0, const float* __restrict__ pval0,
                                 const float* __restrict__ x1, float* __restrict__ x0,
                                 const int32_t* __restrict__ face_prob, const int32_t* __restrict__ st) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf || !amg_live(st, face_prob[f])) return;
  float xv[PW];
  int nc = 0;
#pragma unroll
  for (int c = 0; c < PW; ++c) {
    const int J = pcol0[f * PW + c];
    if (J < 0) break;
    xv[c] = x1[J];
    nc = c + 1;
  }
#pragma unroll
  for (int i = 0; i < NT; ++i) {
    const int64_t row = (int64_t)f * NT + i;
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < PW; ++c)
      if (c < nc) s += pval0[row * PW + c] * xv[c];
    x0[row] += s;
  }
}

// Coarse-level kernels: G lanes per row (G a power of two <= 32).  The lanes of a group take a
// row's entries in turn and add their partial sums with a shuffle tree (FP32, fixed order), so
// the result does not depend on the launch.  Small levels (a few thousand rows) are latency-bound
// and use whole warps, which shortens each row's chain of dependent loads; large levels (the
// first coarse levels of a batch hold 10^5 rows and more) are bandwidth-bound and use 4 lanes,
// which keeps most lanes busy on rows of 10-20 entries.
// Row and lane of a thread.  Warps whose first row is past the end leave at once (uniformly);
// in the last warp every lane stays until the shuffle, which names all 32 lanes.
#define AMG_GROUP_ROW(ROW, LANE, N)                                                   \
  const int64_t t_ = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;                 \
  if ((t_ - (threadIdx.x & 31)) / G >= (N)) return;                                   \
  const int ROW = (int)(t_ / G), LANE = (int)(t_ % G)

template <int G> __device__ __forceinline__ float group_sum_f(float v) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// x_out = x_in + (b - A x_in) / dl1
template <int G>
__global__ void k_amg_l1_sweep(int n, const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                               const float* __restrict__ val, const float* __restrict__ dl1inv,
                               const float* __restrict__ b, const float* __restrict__ xin, float* __restrict__ xout,
                               const int32_t* __restrict__ prob, const int32_t* __restrict__ st) {
  AMG_GROUP_ROW(i, lane, n);
  const bool on = i < n && amg_live(st, prob[i]);
  float s = 0.f;
  if (on)
    for (int e = ptr[i] + lane; e < ptr[i + 1]; e += G) s += val[e] * xin[col[e]];
  s = group_sum_f<G>(s);
  if (lane == 0 && on) xout[i] = xin[i] + (b[i] - s) * dl1inv[i];
}

// r = b - A x
template <int G>
__global__ void k_amg_residual(int n, const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                               const float* __restrict__ val, const float* __restrict__ b, const float* __restrict__ x,
                               float* __restrict__ r, const int32_t* __restrict__ prob,
                               const int32_t* __restrict__ st) {
  AMG_GROUP_ROW(i, lane, n);
  const bool on = i < n && amg_live(st, prob[i]);
  float s = 0.f;
  if (on)
    for (int e = ptr[i] + lane; e < ptr[i + 1]; e += G) s += val[e] * x[col[e]];
  s = group_sum_f<G>(s);
  if (lane == 0 && on) r[i] = b[i] - s;
}

// b_c = P' r and x_c = b_c / dl1_c (first sweep of the coarse level; dl1 NULL on the coarsest)
template <int G>
__global__ void k_amg_restrict(int nc, const int32_t* __restrict__ rptr, const int32_t* __restrict__ rent,
                               const int32_t* __restrict__ rrow, const float* __restrict__ pval,
                               const float* __restrict__ r, const float* __restrict__ dl1inv, float* __restrict__ bc,
                               float* __restrict__ xc, const int32_t* __restrict__ probc,
                               const int32_t* __restrict__ st) {
  AMG_GROUP_ROW(J, lane, nc);
  const bool on = J < nc && amg_live(st, probc[J]);
  float s = 0.f;
  if (on)
    for (int k = rptr[J] + lane; k < rptr[J + 1]; k += G) s += pval[rent[k]] * r[rrow[k]];
  s = group_sum_f<G>(s);
  if (lane == 0 && on) {
    bc[J] = s;
    if (dl1inv) xc[J] = s * dl1inv[J];
  }
}

// x += P x_c
template <int G>
__global__ void k_amg_prolong(int n, const int32_t* __restrict__ pptr, const int32_t* __restrict__ pcol,
                              const float* __restrict__ pval, const float* __restrict__ xc, float* __restrict__ x,
                              const int32_t* __restrict__ prob, const int32_t* __restrict__ st) {
  AMG_GROUP_ROW(i, lane, n);
  const bool on = i < n && amg_live(st, prob[i]);
  float s = 0.f;
  if (on)
    for (int e = pptr[i] + lane; e < pptr[i + 1]; e += G) s += pval[e] * xc[pcol[e]];
  s = group_sum_f<G>(s);
  if (lane == 0 && on) x[i] += s;
}

// coarsest: x = A^-1 b per problem (one CTA per problem)
__global__ void k_amg_coarse_solve(const int32_t* __restrict__ crow0, const int32_t* __restrict__ coff,
                                   const float* __restrict__ cinv, const float* __restrict__ b, float* __restrict__ x,
                                   const int32_t* __restrict__ st) {
  const int P = blockIdx.x;
  if (!amg_live(st, P)) return;
  const int r0 = crow0[P], m = crow0[P + 1] - r0;
  const float* A = cinv + coff[P];
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    float s = 0.f;
    for (int j = 0; j < m; ++j) s += A[i * m + j] * b[r0 + j];
    x[r0 + i] = s;
  }
}

// ---- the coarse levels below a row limit, one CTA per problem ----------------------------
// k_amg_tail runs the part of the V-cycle from level T down to the coarsest and back up to level
// T for one problem per CTA, with a CTA barrier between the phases instead of a kernel boundary:
// (nu - 1) sweeps, residual and restriction (with the next level's first sweep) on each level
// going down, the dense coarsest solve, then prolongation and nu sweeps on each level going up.
// Each row is computed exactly as the per-level kernels compute it (the same G lanes per row,
// taken from the level's size, the same per-lane order and shuffle tree), and the iterates move
// through the same buffers, so the cycle's result is bit-identical to theirs.
struct TailArgs {
  int T, nl, nu;
  const TailLevel* L;  // device copy of the level table (nl entries), built with the hierarchy
  const int32_t *crow0, *coff;
  const float* cinv;
  const int32_t* st;
};

__device__ __forceinline__ float group_sum_rt(float v, int G) {
  for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Rows [r0, r1) in groups of G lanes: FN(row, lane, active) returns the lane's partial sum (0 when
// inactive); every lane of a warp runs the same number of rounds, so the shuffles name all lanes.
template <typename FN, typename OUT>
__device__ __forceinline__ void tail_rows(int r0, int r1, int G, FN part, OUT out) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, rpw = 32 / G;
  const int nw = AMG_TAIL_THREADS / 32;
  for (int base = r0 + warp * rpw; base < r1; base += nw * rpw) {
    const int i = base + lane / G, gl = lane % G;
    const bool on = i < r1;
    float v = on ? part(i, gl) : 0.f;
    v = group_sum_rt(v, G);
    if (on && gl == 0) out(i, v);
  }
}

__global__ void __launch_bounds__(AMG_TAIL_THREADS) k_amg_tail(TailArgs a) {
  const int P = blockIdx.x;
  if (!amg_live(a.st, P)) return;
  float* iter[AMG_MAX_LEVELS];
  const int nu = a.nu, last = a.nl - 1;
  // down
  for (int l = a.T; l < last; ++l) {
    const TailLevel L = a.L[l];
    const TailLevel C = a.L[l + 1];
    const int r0 = L.prow0[P], r1 = L.prow0[P + 1];
    float* cur = L.x;
    float* oth = L.t;
    for (int sw = 1; sw < nu; ++sw) {
      const float* xin = cur;
      float* xout = oth;
      tail_rows(r0, r1, L.g,
                [&](int i, int gl) {
                  float s = 0.f;
                  for (int e = L.ptr[i] + gl; e < L.ptr[i + 1]; e += L.g) s += L.val[e] * xin[L.col[e]];
                  return s;
                },
                [&](int i, float s) { xout[i] = xin[i] + (L.b[i] - s) * L.dl1inv[i]; });
      __syncthreads();
      float* tmp = cur;
      cur = oth;
      oth = tmp;
    }
    iter[l] = cur;
    {
      const float* x = cur;
      tail_rows(r0, r1, L.g,
                [&](int i, int gl) {
                  float s = 0.f;
                  for (int e = L.ptr[i] + gl; e < L.ptr[i + 1]; e += L.g) s += L.val[e] * x[L.col[e]];
                  return s;
                },
                [&](int i, float s) { L.r[i] = L.b[i] - s; });
    }
    __syncthreads();
    const bool coarsest = (l + 1 == last);
    tail_rows(C.prow0[P], C.prow0[P + 1], C.g,
              [&](int J, int gl) {
                float s = 0.f;
                for (int k = L.rptr[J] + gl; k < L.rptr[J + 1]; k += C.g) s += L.pval[L.rent[k]] * L.r[L.rrow[k]];
                return s;
              },
              [&](int J, float s) {
                C.b[J] = s;
                if (!coarsest) C.x[J] = s * C.dl1inv[J];
              });
    __syncthreads();
  }
  // coarsest: x = A^-1 b
  {
    const TailLevel C = a.L[last];
    const int r0 = a.crow0[P], m = a.crow0[P + 1] - r0;
    const float* A = a.cinv + a.coff[P];
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
      float s = 0.f;
      for (int j = 0; j < m; ++j) s += A[i * m + j] * C.b[r0 + j];
      C.x[r0 + i] = s;
    }
  }
  __syncthreads();
  // up
  const float* fin = a.L[last].x;
  for (int l = last - 1; l >= a.T; --l) {
    const TailLevel L = a.L[l];
    const int r0 = L.prow0[P], r1 = L.prow0[P + 1];
    float* x = iter[l];
    float* y = L.r;
    {
      const float* xc = fin;
      tail_rows(r0, r1, L.g,
                [&](int i, int gl) {
                  float s = 0.f;
                  for (int e = L.pptr[i] + gl; e < L.pptr[i + 1]; e += L.g) s += L.pval[e] * xc[L.pcol[e]];
                  return s;
                },
                [&](int i, float s) { x[i] += s; });
    }
    __syncthreads();
    for (int sw = 0; sw < nu; ++sw) {
      const float* xin = x;
      float* xout = y;
      tail_rows(r0, r1, L.g,
                [&](int i, int gl) {
                  float s = 0.f;
                  for (int e = L.ptr[i] + gl; e < L.ptr[i + 1]; e += L.g) s += L.val[e] * xin[L.col[e]];
                  return s;
                },
                [&](int i, float s) { xout[i] = xin[i] + (L.b[i] - s) * L.dl1inv[i]; });
      __syncthreads();
      float* tmp = x;
      x = y;
      y = tmp;
    }
    fin = x;
  }
}

inline unsigned nblk(int64_t n, int t = 256) { return (unsigned)std::max<int64_t>(1, (n + t - 1) / t); }

// Degree of the level-0 Chebyshev smoother (HDG_AMG_CHEB_DEGREE, 1..4, default 4): each degree
// beyond 1 adds a matrix sweep before and after the coarse correction.  Measured on the
// 256-problem batch (kappa contrast 1e4, tol 1e-9) with the FP32 level-0 copy: degree 1/2/3
// took 754/474/359 iterations at most and gave 302/367/398 solves/s; with the FP16 copy, which
// makes a sweep cheaper, degree 2/3/4 took 474/359/313 iterations and gave 410/447/461 solves/s.
// On the 131072-cell p=2 problem with kappa = 1, degree 2 was 5 % faster than 3 (103 vs 99
// iterations).
// l1-Jacobi sweeps before and after the coarse correction on each coarse level
// (HDG_AMG_COARSE_SWEEPS=1..8 sets one value for all).  With the strength-of-connection
// aggregates, on the 256-problem batch (kappa per cell over four decades) 1/2/3/4 sweeps gave
// 972/1068/1112-1121/1137 solves/s (mean CG iterations 98/80/72/67); on 2*256^2 cells, p = 2,
// kappa = 1, 2/3/4 gave 43.6/43.0/41.6 solves/s (103/95/89 iterations); the request stream was
// within 1.5 % for 2-4.  So 4 for systems with a variable kappa (per cell or a field), 2 for a
// constant one.
int amg_coarse_sweeps(const hdg_system* s) {
  static const int env = [] {
    const char* e = std::getenv("HDG_AMG_COARSE_SWEEPS");
    const int v = e ? std::atoi(e) : 0;
    return (v >= 1 && v <= 8) ? v : 0;
  }();
  if (env > 0) return env;
  return (s->kappa_cells || s->kappa_field) ? 4 : 2;
}

// Storage of the scaled level-0 matrix that the cycle reads: FP16 (default; half the bytes of
// the dominant sweeps) or FP32 (HDG_AMG_LEVEL0_FP32=1).
bool amg_level0_fp32() {
  static const bool v = [] {
    const char* e = std::getenv("HDG_AMG_LEVEL0_FP32");
    return e && std::atoi(e) != 0;
  }();
  return v;
}

// The Chebyshev interval is [lambda / ratio, lambda].  A wider interval damps more of the smooth
// error that coarse aggregates leave behind where kappa jumps; with a constant kappa it smooths
// the high end less well.  (With the strength-of-connection aggregates the ratio hardly matters:
// 30 and 120 are within 1 % on the batch.)  Measured before them (degree 4): on the 256-problem
// batch (kappa per cell over four decades) ratios 12/20/30/60/120/250/500 gave
// 462/490/507/528/538/538/533 solves/s; on the 131072-cell p=2 problem with kappa = 1, 30 gave
// 38.0 solves/s (95 iterations) and 120 gave 33.3 (113).  So 120 for systems with a variable
// kappa, 30 otherwise; HDG_AMG_CHEB_RATIO (2..1000) sets one value for all.
float amg_cheb_ratio(const hdg_system* s) {
  static const float env = [] {
    const char* e = std::getenv("HDG_AMG_CHEB_RATIO");
    const float r = e ? (float)std::atof(e) : 0.f;
    return (r >= 2.f && r <= 1000.f) ? r : 0.f;
  }();
  if (env > 0.f) return env;
  return (s->kappa_cells || s->kappa_field) ? 120.f : 30.f;
}

// Degree of the level-0 Chebyshev smoother (HDG_AMG_CHEB_DEGREE, 1..4).  With the
// strength-of-connection aggregates the cheaper polynomial wins: on the 256-problem batch degree
// 2 / 3 / 4 gave 1015 / 961 / 931 solves/s (mean CG iterations 78 / 73 / 68); with kappa = 1 on
// 2*256^2 cells (p = 2) degree 2 was already the fastest.
int amg_cheb_degree() {
  static const int k = [] {
    const char* e = std::getenv("HDG_AMG_CHEB_DEGREE");
    const int v = e ? std::atoi(e) : 2;
    return (v >= 1 && v <= 4) ? v : 2;
  }();
  return k;
}

#define AMG_LAUNCH_G(KERNEL, ROWS, ST, ...)                                                        \
  do {                                                                                             \
    const int rows_ = (ROWS);                                                                      \
    switch (amg_group(rows_)) {                                                                    \
      case 4: KERNEL<4><<<nblk((int64_t)rows_ * 4), 256, 0, ST>>>(__VA_ARGS__); break;             \
      case 8: KERNEL<8><<<nblk((int64_t)rows_ * 8), 256, 0, ST>>>(__VA_ARGS__); break;             \
      default: KERNEL<32><<<nblk((int64_t)rows_ * 32), 256, 0, ST>>>(__VA_ARGS__); break;          \
    }                                                                                              \
  } while (0)

template <int NT> void numeric_nt(hdg_system* s, const float* val0, cudaStream_t st) {
  AmgHierarchy* H = s->amg;
  const int nf = H->nf;
  HDG_CUDA(cudaMemsetAsync(H->lam0.p, 0, sizeof(float) * std::max(s->nprob, 1), st));
  k_amg_block_inv<NT><<<nblk(nf), 256, 0, st>>>(nf, s->d_bcol5.p, s->d_kdiag.p, val0, H->face_prob.p, H->dinv0.p,
                                                H->lam0.p);
  k_amg_p0<NT><<<nblk(nf), 256, 0, st>>>(nf, s->d_bcol5.p, val0, H->dinv0.p, H->lam0.p, H->face_prob.p, H->agg0.p,
                                         H->tent0.p, H->pcol0.p, H->pval0.p);
  k_amg_ap0<NT><<<nblk((int64_t)nf * NT), 256, 0, st>>>(nf, H->wap, s->d_bcol5.p, val0, H->pcol0.p, H->pval0.p,
                                                        H->apmap0.p, H->apval0.p);
  AmgLevel& L1 = H->lev[0];
  k_amg_rap0<NT><<<nblk((int64_t)L1.n * 32), 256, 0, st>>>(L1.n, H->wap, H->rptr0.p, H->rent0.p, H->pval0.p, H->apcol0.p,
                                             H->apval0.p, L1.ptr.p, L1.col.p, L1.val.p);
  k_amg_dp0<NT><<<nblk(nf), 256, 0, st>>>(nf, s->d_kdiag.p, val0, H->pval0.p, H->dpval0.p);
  if (amg_level0_fp32()) {
    k_amg_scale0<NT, float><<<nblk(nf), 256, 0, st>>>(nf, H->dinv0.p, val0, const_cast<float*>(val0));
  } else {
    H->val0h.alloc((size_t)hdg_system::SLOTS * NT * NT * nf);
    k_amg_scale0<NT, __half><<<nblk(nf), 256, 0, st>>>(nf, H->dinv0.p, val0, H->val0h.p);
  }
  s->ctx->launches += 6;
  for (size_t l = 0; l < H->lev.size(); ++l) {
    AmgLevel& L = H->lev[l];
    k_amg_dl1<<<nblk(L.n), 256, 0, st>>>(L.n, L.ptr.p, L.val.p, L.dl1inv.p);
    s->ctx->launches++;
    if (l + 1 == H->lev.size()) break;
    AmgLevel& C = H->lev[l + 1];
    k_amg_p<<<nblk(L.n), 256, 0, st>>>(L.n, L.ptr.p, L.col.p, L.val.p, L.dl1inv.p, L.agg.p, L.tent.p, L.pptr.p,
                                       L.pcol.p, L.pval.p);
    k_amg_ap<<<nblk((int64_t)L.n * 32), 256, 0, st>>>(L.n, L.ptr.p, L.col.p, L.val.p, L.pptr.p, L.pcol.p, L.pval.p, L.apptr.p,
                                        L.apcol.p, L.apval.p);
    k_amg_rap<<<nblk((int64_t)C.n * 32), 256, 0, st>>>(C.n, L.rptr.p, L.rent.p, L.rrow.p, L.pval.p, L.apptr.p, L.apcol.p,
                                         L.apval.p, C.ptr.p, C.col.p, C.val.p);
    s->ctx->launches += 3;
  }
  const AmgLevel& C = H->lev.back();
  const size_t smem = sizeof(float) * ((size_t)H->cmax * 2 * H->cmax + H->cmax);
  static bool attr = false;
  if (!attr) {
    HDG_CUDA(cudaFuncSetAttribute(k_amg_coarse_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    attr = true;
  }
  if (H->cmax > 0)
    k_amg_coarse_inv<<<s->nprob, 256, smem, st>>>(H->crow0.p, H->coff.p, C.ptr.p, C.col.p, C.val.p, H->cinv.p);
  s->ctx->launches++;
  HDG_CUDA(cudaGetLastError());
}

// One level-0 Chebyshev step, a thread per row or a thread per face (H->row_sweep, tuned; both
// give the same bits).  Measured before the tuner: 49 k faces (p = 4): rows 15 -> 10 us per
// sweep; 197 k faces (p = 2) and the batch's bins (0.4-0.7 M faces): faces faster.
template <int NT, typename VT>
void cheb_sweep(hdg_system* s, const VT* val0, const float* b0, const float* in, float* out, int step,
                const int32_t* cst, cudaStream_t st) {
  AmgHierarchy* H = s->amg;
  const int nf = H->nf;
  EventPair* ep = nullptr;
  if (s->prof_cheb0) {  // a sampled chunk: each sweep timed on its own
    ep = new EventPair();
    ep->start(st);
  }
  if (H->row_sweep)
    k_amg_row_cheb<NT, VT><<<nblk((int64_t)nf * NT), 256, 0, st>>>(nf, s->d_bcol5.p, val0, H->dinv0.p, H->lam0.p,
                                                              H->face_prob.p, b0, H->bt0.p, in, out, H->d0.p, step,
                                                              amg_cheb_ratio(s), cst);
  else
    k_amg_face_cheb<NT, VT><<<nblk(nf), 256, 0, st>>>(nf, s->d_bcol5.p, val0, H->dinv0.p, H->lam0.p, H->face_prob.p, b0,
                                                  H->bt0.p, in, out, H->d0.p, step, amg_cheb_ratio(s), cst);
  if (ep) {
    ep->stop(st);
    s->ev_cheb0.push_back(ep);
  }
}

template <int NT, typename VT>
void apply_nt(hdg_system* s, const VT* val0, const float* b0, float* z0, const int32_t* cst, cudaStream_t st) {
  AmgHierarchy* H = s->amg;
  const int nf = H->nf;
  const int64_t n0 = (int64_t)nf * NT;
  const int nl = (int)H->lev.size();
  // level 0 pre-smoothing: Chebyshev of degree k from x = 0; the steps alternate between x0
  // and z0 so that the last one writes z0 (a step never reads the vector it writes)
  const int k = amg_cheb_degree();
  for (int t = 0; t < k; ++t) {
    float* out = ((k - 1 - t) % 2 == 0) ? z0 : H->x0.p;
    const float* in = (t == 0) ? nullptr : (out == z0 ? H->x0.p : z0);
    cheb_sweep<NT, VT>(s, val0, b0, in, out, t, cst, st);
  }
  if (H->row_sweep)
    k_amg_face_residual<NT, VT><<<nblk(n0), 256, 0, st>>>(nf, s->d_bcol5.p, val0, H->bt0.p, z0, H->r0.p,
                                                          H->face_prob.p, cst);
  else
    k_amg_face_residual_f<NT, VT><<<nblk(nf), 256, 0, st>>>(nf, s->d_bcol5.p, val0, H->bt0.p, z0, H->r0.p,
                                                            H->face_prob.p, cst);
  AmgLevel& L1 = H->lev[0];
  k_amg_restrict0<NT><<<nblk(L1.n), 256, 0, st>>>(L1.n, H->rptr0.p, H->rent0.p, H->dpval0.p, H->r0.p, L1.dl1inv.p,
                                                  L1.b.p, L1.x.p, L1.prob.p, cst);
  // coarse levels down: x holds the first l1-Jacobi sweep (done by the restriction); the other
  // nu - 1 sweeps alternate between x and t; the iterate then stays where it is until the way up
  const int nu = amg_coarse_sweeps(s);
  float* iter[AMG_MAX_LEVELS];
  float* fin[AMG_MAX_LEVELS];
  // levels from T on (the coarsest included) are cycled by one k_amg_tail launch
  const int T = H->tail_from >= 0 ? H->tail_from : nl;
  for (int l = 0; l + 1 < std::min(T + 1, nl); ++l) {
    AmgLevel& L = H->lev[l];
    AmgLevel& C = H->lev[l + 1];
    float* cur = L.x.p;
    float* oth = L.t.p;
    for (int sw = 1; sw < nu; ++sw) {
      EventPair* ep = (s->prof_cheb0 && l == 0) ? new EventPair() : nullptr;  // sampled chunk: time level 1
      if (ep) ep->start(st);
      AMG_LAUNCH_G(k_amg_l1_sweep, L.n, st, L.n, L.ptr.p, L.col.p, L.val.p, L.dl1inv.p, L.b.p, cur, oth, L.prob.p,
                   cst);
      if (ep) {
        ep->stop(st);
        s->ev_l1.push_back(ep);
      }
      std::swap(cur, oth);
    }
    iter[l] = cur;
    AMG_LAUNCH_G(k_amg_residual, L.n, st, L.n, L.ptr.p, L.col.p, L.val.p, L.b.p, cur, L.r.p, L.prob.p, cst);
    const bool coarsest = (l + 2 == nl);
    AMG_LAUNCH_G(k_amg_restrict, C.n, st, C.n, L.rptr.p, L.rent.p, L.rrow.p, L.pval.p, L.r.p,
                 coarsest ? nullptr : C.dl1inv.p, C.b.p, C.x.p, C.prob.p, cst);
  }
  int up_from = nl - 2;
  if (T < nl) {
    const TailArgs ta{T, nl, nu, H->tail_tab.p, H->crow0.p, H->coff.p, H->cinv.p, cst};
    k_amg_tail<<<s->nprob, AMG_TAIL_THREADS, 0, st>>>(ta);
    // where the tail leaves level T's result: the iterate after nu - 1 sweeps from x (alternating
    // with t), then nu sweeps from it alternating with r
    AmgLevel& L = H->lev[T];
    float* it = ((nu - 1) % 2 == 0) ? L.x.p : L.t.p;
    fin[T] = (nu % 2 == 0) ? it : L.r.p;
    up_from = T - 1;
  } else {
    AmgLevel& C = H->lev.back();
    if (H->cmax > 0) k_amg_coarse_solve<<<s->nprob, 128, 0, st>>>(H->crow0.p, H->coff.p, H->cinv.p, C.b.p, C.x.p, cst);
    fin[nl - 1] = C.x.p;
  }
  // coarse levels up: prolongate the coarser level's result into this level's iterate, then nu
  // sweeps alternating with r (free again); the last one holds the level's result
  for (int l = up_from; l >= 0; --l) {
    AmgLevel& L = H->lev[l];
    float* a = iter[l];
    float* b = L.r.p;
    AMG_LAUNCH_G(k_amg_prolong, L.n, st, L.n, L.pptr.p, L.pcol.p, L.pval.p, fin[l + 1], a, L.prob.p, cst);
    for (int sw = 0; sw < nu; ++sw) {
      EventPair* ep = (s->prof_cheb0 && l == 0) ? new EventPair() : nullptr;
      if (ep) ep->start(st);
      AMG_LAUNCH_G(k_amg_l1_sweep, L.n, st, L.n, L.ptr.p, L.col.p, L.val.p, L.dl1inv.p, L.b.p, a, b, L.prob.p, cst);
      if (ep) {
        ep->stop(st);
        s->ev_l1.push_back(ep);
      }
      std::swap(a, b);
    }
    fin[l] = a;
  }
  // level 0 up: prolongate, then the same Chebyshev polynomial from the corrected iterate (z0,
  // x0, z0, ...); for odd k the result lands in x0 and is copied to z0
  if (H->row_sweep)
    k_amg_prolong0<NT><<<nblk(n0), 256, 0, st>>>(nf, H->pcol0.p, H->pval0.p, fin[0], z0, H->face_prob.p, cst);
  else
    k_amg_prolong0_f<NT><<<nblk(nf), 256, 0, st>>>(nf, H->pcol0.p, H->pval0.p, fin[0], z0, H->face_prob.p, cst);
  for (int t = 0; t < k; ++t) {
    const float* in = (t % 2 == 0) ? z0 : H->x0.p;
    float* out = (t % 2 == 0) ? H->x0.p : z0;
    cheb_sweep<NT, VT>(s, val0, b0, in, out, t, cst, st);
  }
  if (k % 2 == 1) HDG_CUDA(cudaMemcpyAsync(z0, H->x0.p, sizeof(float) * n0, cudaMemcpyDeviceToDevice, st));
}

}  // namespace

// The FP32 level-0 matrix: the system's FP32 copy when it has one, else a copy made here.
const float* amg_level0_values(hdg_system* s, cudaStream_t st);

void amg_tune(hdg_system* s, cudaStream_t st);

void amg_setup_numeric(hdg_system* s, cudaStream_t st) {
  const float* v0 = amg_level0_values(s, st);
  switch (s->nt) {
    case 2: numeric_nt<2>(s, v0, st); break;
    case 3: numeric_nt<3>(s, v0, st); break;
    case 4: numeric_nt<4>(s, v0, st); break;
    case 5: numeric_nt<5>(s, v0, st); break;
  }
  if (!s->amg->tuned) amg_tune(s, st);
}

// Algorithmic bytes of one V-cycle: every array a cycle kernel reads or writes, once (gathered
// neighbour values are counted at their own row).  Level 0: the block-ELL values (FP16 or FP32), block
// columns, block inverses and vectors of the four matrix-touching sweeps (second pre-sweep,
// residual, two post-sweeps), the first sweep, restriction and prolongation; coarse levels: their
// CSR matrices and vectors in the same sweeps.
double amg_cycle_bytes(const hdg_system* s) {
  const AmgHierarchy* H = s->amg;
  const double nf = H->nf, nt = H->nt, n0 = nf * nt, n1 = H->lev.empty() ? 0.0 : H->lev[0].n;
  const double vb = H->val0h.p ? 2.0 : 4.0;             // FP16 or FP32 level-0 values
  const double mat0 = 5.0 * vb * nt * nt * nf + 20.0 * nf;  // values + block columns
  const double dinv = 4.0 * nt * nt * nf;
  const int k = amg_cheb_degree();
  double b = 16.0 * n0 + dinv;                             // first sweep: b, D^-1 -> bt, x, d
  b += (2 * k - 1) * (mat0 + 20.0 * n0);                   // k-1 pre-sweeps, k post-sweeps (D^-1 A0, bt, x, d)
  if (k % 2 == 1) b += 8.0 * n0;                           // copy of the result
  b += mat0 + 12.0 * n0;                                   // residual (D^-1 A0, bt, x -> r~)
  b += 24.0 * n0 + 20.0 * nf + 8.0 * n1;                   // restriction (P0 values, r) + first coarse sweep
  b += 28.0 * n0 + 20.0 * nf + 4.0 * n1;                   // prolongation
  const int nl = (int)H->lev.size();
  for (int l = 0; l < nl; ++l) {
    const double n = H->lev[l].n, nnz = (double)H->lev[l].h_col.size();
    const double spmv = 8.0 * nnz + 4.0 * n;               // values + columns + row pointers
    if (l + 1 == nl) {
      b += 8.0 * n + 4.0 * H->cinv.n;                      // coarsest dense solve
      break;
    }
    const double npc = (double)H->lev[l].h_col.size();      // P and P' sizes are comparable to A's
    b += (2 * amg_coarse_sweeps(s) - 1) * (spmv + 20.0 * n) + (spmv + 16.0 * n);  // sweeps, one residual
    b += 2.0 * (8.0 * npc + 12.0 * n);                      // restriction and prolongation
  }
  return b;
}

// Algorithmic bytes per trace row of the 2k level-0 Chebyshev sweeps of one V-cycle: the first
// forms D^-1 b (b and the row's D^-1 row read, bt, x, d written); each of the other 2k - 1 reads
// the row of D^-1 A0 (5 nt values of 2 or 4 bytes), the block columns (20 bytes per face), bt, x
// (neighbour values counted once, at their own row), d read and written, x out.
double amg_cheb0_bytes_per_row(const hdg_system* s) {
  const AmgHierarchy* H = s->amg;
  const double nt = H->nt, vb = H->val0h.p ? 2.0 : 4.0;
  const int k = amg_cheb_degree();
  return (16.0 + 4.0 * nt) + (2 * k - 1) * (5.0 * vb * nt + 20.0 / nt + 20.0);
}

// Algorithmic bytes per trace row of the first coarse level's l1-Jacobi sweeps in one V-cycle
// (2 nu - 1 of them): each reads the level's CSR values and columns (8 per entry), row pointers,
// b, dl1, the iterate (neighbour values counted once, at their own row) and writes the new
// iterate: 8 nnz + 20 n bytes per sweep, spread over the trace rows.
double amg_l1sweep_bytes_per_row(const hdg_system* s) {
  const AmgHierarchy* H = s->amg;
  if (!H || H->lev.size() < 2) return 0.0;
  const AmgLevel& L = H->lev[0];
  const double per_sweep = 8.0 * (double)L.h_col.size() + 20.0 * L.n;
  return (2 * amg_coarse_sweeps(s) - 1) * per_sweep / ((double)H->nf * H->nt);
}

int amg_cycle_launches(const hdg_system* s) {
  const int nl = (int)s->amg->lev.size(), k = amg_cheb_degree(), nu = amg_coarse_sweeps(s);
  // level 0 down, coarse levels down, coarsest, coarse levels up, level 0 up (the D2D copy of an
  // odd degree is no kernel); levels from the tail's first on are one launch
  const int T = s->amg->tail_from >= 0 ? s->amg->tail_from : nl - 1;
  return (k + 2) + (nu + 1) * T + 1 + (nu + 1) * T + (1 + k);
}

template <typename VT> void apply_dispatch(hdg_system* s, const VT* v0, const float* r, float* z,
                                           const int32_t* cg_state, cudaStream_t st) {
  switch (s->nt) {
    case 2: apply_nt<2, VT>(s, v0, r, z, cg_state, st); break;
    case 3: apply_nt<3, VT>(s, v0, r, z, cg_state, st); break;
    case 4: apply_nt<4, VT>(s, v0, r, z, cg_state, st); break;
    case 5: apply_nt<5, VT>(s, v0, r, z, cg_state, st); break;
  }
}

void amg_apply(hdg_system* s, const float* r, float* z, const int32_t* cg_state, cudaStream_t st) {
  if (s->amg->val0h.p)
    apply_dispatch<__half>(s, s->amg->val0h.p, r, z, cg_state, st);
  else
    apply_dispatch<float>(s, s->amg->val0f.p, r, z, cg_state, st);
  HDG_CUDA(cudaGetLastError());
}

// ---- V-cycle autotuner ---------------------------------------------------------------------
// The launch shapes of the cycle that do not change its result are picked by timing, once per
// hierarchy: the level-0 smoother with a thread per face or per row, and the level T from which
// one k_amg_tail launch (a CTA per problem) replaces the per-level launches (or none).  Every
// candidate computes the same bits, so the choice changes only the time.  Each candidate's cycle
// is captured twice into a CUDA graph, as the CG chunks run it (timing un-graphed launches would
// charge the host's launch overhead to the many-launch candidates), and the graph runs once
// untimed and three times timed (CUDA events on the system's stream, on a zero right-hand side:
// the cycle's work does not depend on the values); the fastest minimum wins.
// Choices are cached by (nt, log2 faces, log2 problems, levels), so systems of similar shape
// reuse them; a system marked one-shot (amg_tune_time false: the serving engine's flights) takes
// a cached choice when there is one and the defaults otherwise, without timing.
namespace {
struct TuneKey {
  int nt, lnf, lnp, nl;
  bool operator<(const TuneKey& o) const { return std::tie(nt, lnf, lnp, nl) < std::tie(o.nt, o.lnf, o.lnp, o.nl); }
};
struct TuneVal {
  bool row;
  int tail;
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneVal> g_tune;
int ilog2(int64_t v) {
  int k = 0;
  while (v > 1) {
    v >>= 1;
    ++k;
  }
  return k;
}
}  // namespace

void amg_tune(hdg_system* s, cudaStream_t st) {
  AmgHierarchy* H = s->amg;
  H->tuned = true;
  const int fs = amg_sweep_forced();
  if (fs >= 0) H->row_sweep = (fs == 1);
  const bool tune_sweep = fs < 0;
  const bool tune_tail = amg_tail_rows() < 0 && !H->tail_cands.empty();
  if (!tune_sweep && !tune_tail) return;
  const bool verbose = std::getenv("HDG_AMG_VERBOSE") != nullptr;
  const TuneKey key{s->nt, ilog2(H->nf), ilog2(std::max(s->nprob, 1)), (int)H->lev.size()};
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
      if (tune_sweep) H->row_sweep = it->second.row;
      if (tune_tail) {
        const int t = it->second.tail;
        const bool ok = t < 0 || std::find(H->tail_cands.begin(), H->tail_cands.end(), t) != H->tail_cands.end();
        H->tail_from = ok ? t : -1;
      }
      return;
    }
  }
  if (!s->amg_tune_time) return;  // the defaults: sweep by face count, no tail
  const int64_t n0 = (int64_t)H->nf * s->nt;
  DevBuf<float> rin, zout;
  rin.alloc((size_t)n0);
  zout.alloc((size_t)n0);
  HDG_CUDA(cudaMemsetAsync(rin.p, 0, sizeof(float) * n0, st));
  std::vector<int> rows = tune_sweep ? std::vector<int>{0, 1} : std::vector<int>{(int)H->row_sweep};
  std::vector<int> tails{H->tail_from};
  if (tune_tail) {
    tails.assign(1, -1);
    tails.insert(tails.end(), H->tail_cands.begin(), H->tail_cands.end());
  }
  const bool prof = s->prof_cheb0;
  s->prof_cheb0 = false;
  cudaEvent_t e0, e1;
  HDG_CUDA(cudaEventCreate(&e0));
  HDG_CUDA(cudaEventCreate(&e1));
  cudaStream_t cap;
  HDG_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
  float best = 3.4e38f;
  bool brow = H->row_sweep;
  int btail = H->tail_from;
  for (int rw : rows)
    for (int tl : tails) {
      H->row_sweep = (rw == 1);
      H->tail_from = tl;
      cudaGraph_t g;
      cudaGraphExec_t ge;
      HDG_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
      amg_apply(s, rin.p, zout.p, nullptr, cap);
      amg_apply(s, rin.p, zout.p, nullptr, cap);
      HDG_CUDA(cudaStreamEndCapture(cap, &g));
      HDG_CUDA(cudaGraphInstantiate(&ge, g, 0));
      cudaGraphDestroy(g);
      HDG_CUDA(cudaGraphLaunch(ge, st));
      float tmin = 3.4e38f;
      for (int rep = 0; rep < 3; ++rep) {
        HDG_CUDA(cudaEventRecord(e0, st));
        HDG_CUDA(cudaGraphLaunch(ge, st));
        HDG_CUDA(cudaEventRecord(e1, st));
        HDG_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        HDG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        tmin = std::min(tmin, 0.5f * ms);
      }
      cudaGraphExecDestroy(ge);
      s->ctx->launches += 8 * amg_cycle_launches(s);
      if (verbose)
        std::fprintf(stderr, "amg tune: nt %d, %d faces, %d problems: %s sweep, tail from level %d: %.1f us\n", s->nt,
                     H->nf, s->nprob, rw ? "row" : "face", tl + 1, 1e3 * tmin);
      if (tmin < best) {
        best = tmin;
        brow = (rw == 1);
        btail = tl;
      }
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(cap);
  H->row_sweep = brow;
  H->tail_from = btail;
  s->prof_cheb0 = prof;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[key] = TuneVal{brow, btail};
}

namespace {
__global__ void k_amg_to_float(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    b[t] = (float)a[t];
}
}  // namespace

const float* amg_level0_values(hdg_system* s, cudaStream_t st) {
  AmgHierarchy* H = s->amg;
  const int64_t nval = (int64_t)hdg_system::SLOTS * s->nt * s->nt * s->nf;
  H->val0f.alloc((size_t)nval);
  k_amg_to_float<<<(unsigned)std::min<int64_t>((nval + 255) / 256, 152 * 32), 256, 0, st>>>(nval, s->d_val.p,
                                                                                            H->val0f.p);
  HDG_CUDA(cudaGetLastError());
  s->ctx->launches++;
  return H->val0f.p;
}
