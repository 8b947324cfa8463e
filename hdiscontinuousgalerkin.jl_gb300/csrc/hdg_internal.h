// Internal declarations of libhdg (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <map>
#include <string>
#include <vector>

#include "../../include/hdg.h"

#define HDG_MAX_P 4
#define HDG_LAGRANGE_MAX_NL 15  // nodal basis functions of the highest Lagrange order (4)

// ------------------------------------------------------------------ errors
struct HdgError {
  int code;
  std::string msg;
};
#define HDG_CUDA(call)                                                                          \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess)                                                                      \
      throw HdgError{e_ == cudaErrorMemoryAllocation ? HDG_ERR_OOM : HDG_ERR_CUDA,              \
                     std::string(#call) + ": " + cudaGetErrorString(e_)};                       \
  } while (0)

// ------------------------------------------------------------------ device buffers
// Device memory comes from the stream-ordered pool allocator on the stream of the context that
// owns the object (set by every C-ABI entry point): a batch or a served request allocates and
// frees its buffers without synchronising the device, and freed memory stays in the pool.
extern thread_local cudaStream_t g_alloc_stream;
// Stream that will use buffers allocated now, when it is not the allocation stream (a forked
// stream of a pipelined batch step): a new allocation is ordered before that stream's later work.
extern thread_local cudaStream_t g_use_stream;
// The launch autotuners (element kernel, V-cycle) may time candidate configurations on this
// thread.  Threads that build one-shot systems (the serving engine's flight builders) clear it:
// they then take the nearest cached choice, and time candidates only when nothing is cached.
extern thread_local bool g_tuning_allowed;
void order_streams(cudaStream_t before, cudaStream_t after);  // `after` waits for `before`'s work so far
template <class T> struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaStream_t s = nullptr;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n), s(o.s) {
    o.p = nullptr;
    o.n = 0;
  }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p;
      n = o.n;
      s = o.s;
      o.p = nullptr;
      o.n = 0;
    }
    return *this;
  }
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
    n = 0;
  }
  void alloc(size_t count) {
    if (count == n && p) return;
    release();
    if (count == 0) return;
    s = g_alloc_stream;
    HDG_CUDA(cudaMallocAsync((void**)&p, count * sizeof(T), s));
    n = count;
    if (g_use_stream && g_use_stream != s) order_streams(s, g_use_stream);
  }
  void upload(const T* h, size_t count, cudaStream_t s) {
    alloc(count);
    if (count) HDG_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
  }
  void download(T* h, size_t count, cudaStream_t s) const {
    if (count) HDG_CUDA(cudaMemcpyAsync(h, p, count * sizeof(T), cudaMemcpyDeviceToHost, s));
  }
};

// ------------------------------------------------------------------ fields
struct FieldSpec {
  int kind = HDG_FIELD_CONST;
  std::vector<double> prm{0.0};
};
// HDG_OK, or HDG_ERR_ARG with the reason when f's parameters do not cover what its kind reads.
int field_check(const hdg_field* f, std::string* why);
// FieldSpec of f (NULL: the constant default_const); throws HdgError{HDG_ERR_ARG} on a bad field.
FieldSpec field_from(const hdg_field* f, double default_const);
double eval_field_host(const FieldSpec& f, double x, double y);

// POD view passed to kernels: parameters live in device memory
struct FieldDev {
  int kind;
  int np;
  const double* prm;
};

// Per-problem coefficients of a system holding several independent problems (a batch): the
// problem of a cell indexes the source/coefficient field kinds, parameter offsets and tau.
struct CoefDev {
  const int32_t* cell_prob;  // [ncells]
  const int32_t* fkind;      // [nprob]
  const int32_t* foff;       // [nprob] offset into fprm
  const double* fprm;
  const int32_t* kkind;      // [nprob] kappa field kind (kappa_mode 2)
  const int32_t* koff;
  const double* kprm;
  const double* tau;         // [nprob]
  // fprm with each Gaussian bump's width s replaced by -1/(2 s^2) (element kernels' source)
  const double* fprep;
};

// ------------------------------------------------------------------ objects
struct hdg_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string err;
  int64_t launches = 0;
  bool profiling = false;
};

// A pair of CUDA events bracketing work on one stream (used only while profiling).
struct EventPair {
  cudaEvent_t a = nullptr, b = nullptr;
  bool armed = false;
  void start(cudaStream_t s) {
    if (!a) {
      cudaEventCreate(&a);
      cudaEventCreate(&b);
    }
    cudaEventRecord(a, s);
    armed = false;
  }
  void stop(cudaStream_t s) {
    cudaEventRecord(b, s);
    armed = true;
  }
  double ms() {
    if (!armed) return 0.0;
    float t = 0.f;
    cudaEventSynchronize(b);
    cudaEventElapsedTime(&t, a, b);
    return t;
  }
  ~EventPair() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
  }
};

struct hdg_mesh {
  hdg_ctx* ctx = nullptr;
  int nn = 0, nc = 0, nf = 0;
  // A mesh may be the disjoint union of several problems' meshes (a batch): problem P owns
  // nodes [prob_node0[P], prob_node0[P+1]) and likewise cells and faces.
  int nprob = 1;
  std::vector<int32_t> prob_node0, prob_cell0, prob_face0;
  void single_problem() {
    nprob = 1;
    prob_node0 = {0, nn};
    prob_cell0 = {0, nc};
    prob_face0 = {0, nf};
  }
  std::vector<double> xy;       // [nn][2]
  std::vector<int32_t> cells;   // [nc][3] 0-based
  std::vector<int32_t> cfaces;  // [nc][3] 0-based
  std::vector<int32_t> faces;   // [nf][4] v1 v2 c1 c2, 0-based, c2 = -1 on the boundary
  std::map<std::string, std::vector<int32_t>> facesets;  // 0-based, sorted
  bool structured = false;
  int nx = 0, ny = 0;
  double LL[2] = {0, 0}, UR[2] = {1, 1};
  // device copies
  DevBuf<double> d_xy;
  DevBuf<int32_t> d_cells, d_cfaces;
  DevBuf<uint8_t> d_orient;   // bit f = face_orientation(cell, f)
  DevBuf<int32_t> d_fcell;    // [nf][2] cells of a face (second -1 on the boundary)
  DevBuf<int8_t> d_flf;       // [nf][2] local face index in those cells
  DevBuf<int32_t> d_cell_prob;  // [nc] problem of each cell
  void upload();
  void upload_coordinates();
};

// Reference-element tables of one (p, quad_degree) pair.
struct RefTables {
  int p, qd, nw, nt, nq, nfq;
  std::vector<double> qx, qy, qw;  // volume rule
  std::vector<double> fx, fw;      // face rule on (0,1)
  std::vector<double> N, dN;       // [nw][nq], [nw][nq][2]
  std::vector<double> E;           // [nw][nfq][3]
  std::vector<double> T;           // [nt][nfq]
  std::vector<double> Nv;          // [nw][3] basis at the reference vertices (0,0), (1,0), (0,1)
  bool schur = false;              // the reference mass matrix is invertible (see tables.cpp)
  // packed device tables (see tables.cpp: ref_layout)
  std::vector<double> packed;
};
bool build_ref_tables(int p, int qd, RefTables* t);

// Nodal (continuous Lagrange) basis of order k on the reference triangle, at the volume points of
// QuadratureRule{2}(qd): nodes in the order of get_nodal_points (vertices, edge points, interior
// points); values N [nl][nq] and reference gradients dN [nl][nq][2].
struct LagrangeTables {
  int order = 0, nl = 0, nq = 0;
  std::vector<double> qx, qy, qw, N, dN;
};
bool build_lagrange_tables(int order, int qd, LagrangeTables* t);

// Offsets of the packed table, in doubles.
struct RefLayout {
  int M, D0, D1, C, F, H, NW, N, Q;
  // Schur-complement tables (valid when RefTables::schur): M^-1 D_l, Q_lm = D_l' M^-1 D_m,
  // MF_{f,o} = M^-1 F_{f,o}, DMF_{l,f,o} = D_l' M^-1 F_{f,o}, PFF_{g,o';f,o} = F_{g,o'}' M^-1 F_{f,o}
  int SMD0, SMD1, SQ00, SQ01, SQ11, SMF, SDMF, PFF, total;
};
RefLayout ref_layout(int nw, int nt, int nq);

struct hdg_space {
  hdg_mesh* mesh = nullptr;
  RefTables t;
  DevBuf<double> d_ref;
  bool he_tau = false;  // He = tau int mu mu dS (off: the reference's He without tau)
};

struct CgState;       // cg.cu
struct AmgHierarchy;  // amg.cu

struct hdg_system {
  hdg_space* space = nullptr;
  hdg_ctx* ctx = nullptr;
  int precision = HDG_PREC_FP64;
  int nw, nt, n, m, nc, nf, ndofs;
  int64_t nblocks, nnz;
  double tau = 1.0;
  bool he_tau = false;  // He carries tau (copied from the space at creation)
  // Problems held by this system (several when batched; all share the degree).  Problem P owns
  // trace rows [h_prob_row0[P], h_prob_row0[P+1]).
  int nprob = 1;
  std::vector<int32_t> h_prob_row0;
  std::vector<FieldSpec> fsp, ksp;  // per-problem source and coefficient fields
  std::vector<double> taus;
  DevBuf<int32_t> d_fkind, d_foff, d_kkind, d_koff, d_row_prob;
  DevBuf<double> d_tau;
  DevBuf<double> d_mdiag;           // [nprob] mean |diag K| per problem
  DevBuf<int32_t> d_prob_row0;      // [nprob+1]
  DevBuf<int32_t>& d_prob_row0_dev() {
    if (!d_prob_row0.p)
      d_prob_row0.upload(h_prob_row0.data(), h_prob_row0.size(), g_use_stream ? g_use_stream : ctx->stream);
    return d_prob_row0;
  }
  // Segments: the CUDA blocks of the row-parallel kernels (CG, meandiag, residual); each block
  // covers a row range inside one problem, so per-problem reductions need no cross-problem sums.
  int nseg = 0;
  DevBuf<int32_t> d_seg_prob, d_seg_row0, d_seg_row1, d_prob_blk0, d_prob_nblk;
  std::vector<int32_t> h_seg_prob, h_seg_row0, h_seg_row1, h_prob_blk0, h_prob_nblk;  // host copies
  CoefDev coef_dev() const {
    return CoefDev{space->mesh->d_cell_prob.p, d_fkind.p, d_foff.p, d_fprm.p, d_kkind.p, d_koff.p, d_kprm.p,
                   d_tau.p, d_fprep.p};
  }
  // per-cell condensed blocks: AB = [Ate | bte] (m x (m+1)), KB = [K_e | b_e] (n x (m+1)), or,
  // after the Cholesky-Schur element path (kb_u_only), only its u rows [X_u | b_u] (nw x (m+1))
  DevBuf<double> d_AB, d_KB;
  bool kb_u_only = false;
  DevBuf<float> d_ABf, d_KBf;
  DevBuf<double> d_kappa;  // per-cell kappa (optional)
  DevBuf<double> d_fprm, d_kprm;
  DevBuf<double> d_fprep;  // d_fprm prepared for the element kernels (CoefDev::fprep)
  FieldSpec f, kappa;
  bool kappa_field = false, kappa_cells = false;
  // Trace matrix.  Host: block rows sorted by face id (h_browptr/h_bcol, the export pattern).
  // Device: block-ELL with SLOTS block slots per face (an interior face couples to itself and
  // the 4 other faces of its two cells, a boundary face to 3); missing slots are zero blocks
  // that point at the face itself.  Values are slot-major, row-contiguous:
  // val[(k*nt + j)*ndofs + f*nt + i] = K[f*nt + i, bcol5[k*nf + f]*nt + j], so that consecutive
  // rows read consecutive addresses.
  static constexpr int SLOTS = 5;
  std::vector<int32_t> h_browptr, h_bcol;
  std::vector<int32_t> h_bsrc;  // [nblocks][2] source (cell*9 + lf*3 + lg) or -1
  DevBuf<int32_t> d_bcol5;      // [SLOTS][nf]
  DevBuf<int32_t> d_src5;       // [SLOTS][nf][2]
  DevBuf<int8_t> d_kdiag;       // [nf] slot of the diagonal block
  DevBuf<double> d_val;         // [SLOTS*nt*nt][ndofs] (as above)
  DevBuf<float> d_valf;         // FP32 copy for the mixed solve
  DevBuf<double> d_b;     // rhs
  // Dirichlet state
  bool applied = false;   // apply! done: d_val/d_b are in solver form (free rows negated)
  bool dir_ready = false; // d_pres/d_gv hold a Dirichlet set (scattered; survives reassembly)
  bool dir_lift = false;  // some prescribed value is nonzero
  double* h_dl_uhat = nullptr;  // host destinations of HDG_STEP_DOWNLOAD (hdg_system_set_download)
  double* h_dl_qu = nullptr;
  DevBuf<uint8_t> d_pres;
  DevBuf<double> d_gv;    // prescribed values scattered to dofs
  DevBuf<int32_t> d_dofs; // prescribed dofs (0-based)
  DevBuf<double> d_dvals;
  DevBuf<double> d_part;  // reduction partials
  DevBuf<unsigned> d_cnt; // reduction tickets
  DevBuf<double> d_scal;  // device scalars: [0] = meandiag, [1] = error flags, [2],[3] = residual norms
  // profiling
  EventPair ev_element, ev_gather, ev_apply, ev_cg, ev_recover;
  std::vector<EventPair*> ev_cg_a, ev_cg_b;
  // level-0 multigrid smoother sweeps of the sampled chunks, each timed on its own
  bool prof_cheb0 = false;
  // The multigrid V-cycle autotuner may time candidates when it has no cached choice for this
  // system's shape; one-shot systems (the serving engine's flights) take a cached choice or the
  // defaults instead.
  bool amg_tune_time = true;
  std::vector<EventPair*> ev_cheb0;
  std::vector<EventPair*> ev_l1;  // sampled chunks: each l1-Jacobi sweep of the first coarse level
  double prof_l1_bytes = 0.0;     // their algorithmic bytes (rows of the problems that iterated)
  double prof_cheb0_bytes = 0.0;  // their algorithmic bytes (rows of the problems that iterated)
  // algorithmic bytes moved by the sampled CG launches (rows of the problems that iterated)
  double prof_a_bytes = 0.0, prof_b_bytes = 0.0;
  double prof_all_bytes = 0.0;  // algorithmic bytes of every iteration launch of the last solve
  int cg_iterations = 0;
  double mdiag = 0.0;
  // solution and recovery
  DevBuf<double> d_x;
  DevBuf<double> d_qu;  // [nc][n] recovered (q; u)
  bool have_solution = false, have_recovery = false;
  CgState* cg = nullptr;
  AmgHierarchy* amg = nullptr;      // multigrid preconditioner (symbolic part kept across reassembly)
  int amg_gen = 0;                  // count of symbolic setups (captured CG graphs hold their buffers)
  int last_max_iters = 0;           // most CG iterations of any problem in the last solve (scheduling hint)
  std::vector<char> h_dir_face;     // faces whose dofs apply! prescribed (set by hdg_apply_dirichlet)
  ~hdg_system();
  // partials: 2 per segment; tickets: 4 per problem (CG product, CG update, residual, meandiag)
  void ensure_reduction_buffers() {
    const size_t np = 2 * (size_t)std::max(nseg, 1024), nc = 4 * (size_t)nprob;
    if (d_part.n < np) d_part.alloc(np);
    if (d_cnt.n < nc) {
      d_cnt.alloc(nc);
      HDG_CUDA(cudaMemsetAsync(d_cnt.p, 0, nc * sizeof(unsigned), g_use_stream ? g_use_stream : ctx->stream));
    }
  }
};

// Per-problem CG state: HDG_CG_ST ints (status, iterations, iteration cap, refine flag).
constexpr int HDG_CG_ST = 4;

// ------------------------------------------------------------------ kernel launchers
void launch_element_condense(hdg_system* s, cudaStream_t st);
void launch_gather(hdg_system* s, cudaStream_t st);
void launch_apply_dirichlet(hdg_system* s, const std::vector<int32_t>& dofs0, const std::vector<double>& vals,
                            cudaStream_t st);  // scatter + apply
void launch_dirichlet_scatter(hdg_system* s, const std::vector<int32_t>& dofs0, const std::vector<double>& vals,
                              cudaStream_t st);
void launch_dirichlet_apply(hdg_system* s, cudaStream_t st);  // apply! from the scattered set
void assemble_async(hdg_system* s, cudaStream_t st);          // element + gather, errors left on the device
void assembly_check(hdg_system* s, cudaStream_t st);          // read the element error flags (synchronises)
// One pipelined step over several systems: each system's (assembly, apply!, CG, recovery) runs on a
// stream of its own, so that one system's assembly overlaps the others' iterations.
int run_batch_step(const std::vector<hdg_system*>& sys, const hdg_solver& o, int flags,
                   std::vector<std::vector<hdg_stats>>* stats);
int run_solve(hdg_system* s, const hdg_solver& o, hdg_stats* st);
// FP64 iterative refinement of d_x with a double-double residual (refine.cu): `steps` corrections
// solved by the system's CG to relative tolerance ctol; out: per problem, the total correction
// iterations and the final double-double relative residual.
int run_refine(hdg_system* s, const hdg_solver& o, int steps, double ctol, std::vector<hdg_stats>* out);
int run_solve_many(const std::vector<hdg_system*>& sys, const hdg_solver& o,
                   std::vector<std::vector<hdg_stats>>* stats);
void build_segments(hdg_system* s);

// The CG of one system, driven chunk by chunk by a host loop (run_solve_many, the serving engine).
struct CgSolver {
  virtual ~CgSolver() {}
  virtual void prepare(const hdg_solver& o) = 0;      // allocate, initialise, capture the chunk graph
  virtual void launch_chunk(int rep) = 0;             // enqueue one chunk of iterations
  virtual void enqueue_status_copy() = 0;             // enqueue the per-problem status read-back
  virtual bool process(const hdg_solver& o) = 0;      // after the read-back: true when all problems are done
  virtual void finish(const hdg_solver& o, std::vector<hdg_stats>* out) = 0;
  // finish() in two halves, for callers that do not wait: finish_enqueue queues the final true
  // residual on the stream; finish_collect forms the statistics once that work has landed.
  virtual void finish_enqueue() = 0;
  virtual void finish_collect(std::vector<hdg_stats>* out) = 0;
  virtual void set_stream(cudaStream_t stream) = 0;   // stream of the iteration (after prepare)
  hdg_system* s = nullptr;
};
CgSolver* make_cg_solver(hdg_system* s);
void mesh_concat(hdg_mesh* out, const std::vector<const hdg_mesh*>& parts);
void launch_recover(hdg_system* s, cudaStream_t st);
// The full [K_e | b_e] (ncells x n x (m+1), device) from the stored u rows (kb_u_only systems).
void launch_expand_ke(hdg_system* s, double* out, cudaStream_t st);
double run_errornorm(hdg_system* s, const FieldSpec& uex, cudaStream_t st);
void run_nodal_avg(hdg_system* s, double* host_out, cudaStream_t st);
void destroy_cg(CgState* c);
void destroy_amg(AmgHierarchy* h);
void amg_setup_symbolic(hdg_system* s, const std::vector<char>& dirichlet_face);
void amg_setup_numeric(hdg_system* s, cudaStream_t st);
// z = M^-1 r (FP32).  cg_state: the CG's per-problem state (HDG_CG_ST ints per problem; NULL: all
// problems); problems that neither iterate nor wait for a refinement are skipped.
void amg_apply(hdg_system* s, const float* r, float* z, const int32_t* cg_state, cudaStream_t st);
int amg_cycle_launches(const hdg_system* s);                             // kernels per V-cycle
double amg_cycle_bytes(const hdg_system* s);                             // algorithmic bytes per V-cycle
double amg_l1sweep_bytes_per_row(const hdg_system* s);  // first-coarse-level sweeps per cycle, per trace row
double amg_cheb0_bytes_per_row(const hdg_system* s);  // level-0 sweeps of one V-cycle, per trace row

void mesh_build_rectangle(hdg_mesh* m, int nx, int ny, const double LL[2], const double UR[2]);
int mesh_build_from_cells(hdg_mesh* m, int nnodes, const double* xy, int ncells, const int32_t* cells1, int nedges,
                          const int32_t* edges1);
void build_block_structure(hdg_system* s);
