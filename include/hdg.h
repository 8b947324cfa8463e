/*
 * hdg.h — C ABI of libhdg, the GB300 (sm_103a) implementation of the 2D HDG Poisson path of
 * HDiscontinuousGalerkin.jl: per-element assembly over the Dubiner scalar/vector and Legendre
 * trace spaces, static condensation onto the edge traces, assembly of the global trace system,
 * its solve, and local recovery of u and q.
 *
 * Conventions
 *   - Every function returns an int status: HDG_OK (0) or a negative HDG_ERR_* code; the
 *     message of the last failure on a context is hdg_last_error().
 *   - Ids crossing this boundary are 1-based, as in the reference's Julia data structures
 *     (cells, faces, nodes, dofs); arrays are caller-owned host memory that the library copies.
 *   - Matrices are row-major unless stated.  The library owns all device memory behind opaque
 *     handles.  A context is bound to one device and one CUDA stream and is not thread-safe.
 *   - The reference has no FFI; each entry point names the Julia function it stands in for.
 */
#ifndef HDG_H
#define HDG_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  HDG_OK = 0,
  HDG_ERR_ARG = -1,            /* invalid argument / size */
  HDG_ERR_NEG_DETJ = -2,       /* ArgumentError("det(J) is not positive"), src/ScalarFunctionSpaces.jl:110 */
  HDG_ERR_BAD_ORDER = -3,      /* ArgumentError("Quadrature rule of order … not available"), src/quadrature.jl:24 */
  HDG_ERR_NOT_BOUNDARY = -4,   /* "Face … is not in boundary", src/boundary.jl:22 / generate_mesh.jl:80 */
  HDG_ERR_NO_CONVERGENCE = -5, /* CG reached maxit (no reference counterpart: the reference solves directly) */
  HDG_ERR_OOM = -6,            /* device allocation failed */
  HDG_ERR_CUDA = -7,           /* CUDA runtime error */
  HDG_ERR_SINGULAR = -8,       /* a local system had a zero pivot (LAPACK SingularException) */
  HDG_ERR_BREAKDOWN = -9,      /* CG breakdown: p'Ap <= 0 (trace system not definite) */
  HDG_ERR_UNKNOWN_SET = -10,   /* KeyError on a face set name, src/mesh.jl:75 */
  HDG_ERR_TIMEOUT = -11,       /* a bounded device wait gave up */
  HDG_ERR_CAPACITY = -12       /* a request exceeds a fixed capacity (admission budget, scratch size) */
};

/* Scalar fields for the source f, the coefficient kappa, the boundary data g and the exact
 * solution u_ex.  The reference passes Julia closures; across a C ABI a field is a kind plus
 * parameters, evaluated on the device.
 *   HDG_FIELD_CONST       c                                   params = {c}
 *   HDG_FIELD_SINSIN      a sin(kx pi x) sin(ky pi y)         params = {a, kx, ky}
 *   HDG_FIELD_BUMPS       sum_k a_k exp(-|x-c_k|^2/(2 s_k^2)) params = {K, (cx, cy, s, a) x K}
 *   HDG_FIELD_FOURIER     g = g0 + sum_k a_k cos(2 pi (kx x + ky y) + phi_k)
 *                                                             params = {K, g0, (kx, ky, phi, a) x K}
 *   HDG_FIELD_EXP_FOURIER exp(g) with g as above                                              */
enum { HDG_FIELD_CONST = 0, HDG_FIELD_SINSIN = 1, HDG_FIELD_BUMPS = 2, HDG_FIELD_FOURIER = 3, HDG_FIELD_EXP_FOURIER = 4 };
typedef struct {
  int kind;
  int nparams;
  const double* params;
} hdg_field;

/* Arithmetic of the element kernels and of the trace solve. */
enum {
  HDG_PREC_FP64 = 0,  /* FP64 throughout (the plain path) */
  HDG_PREC_MIXED = 1  /* trace solve: FP32 matrix and Krylov vectors with FP64 x, dot products and
                         scalars; FP64 true-residual refinement ("reliable updates") decides
                         convergence.  Element condensation stays FP64 (local condition numbers
                         reach 3e5, beyond what FP32 plus one refinement step recovers). */
};

typedef struct hdg_ctx hdg_ctx;
typedef struct hdg_mesh hdg_mesh;
typedef struct hdg_space hdg_space;
typedef struct hdg_system hdg_system;
typedef struct hdg_assembler hdg_assembler;

/* ---- context ------------------------------------------------------------------------- */
int hdg_ctx_create(int device, hdg_ctx** out);
int hdg_ctx_destroy(hdg_ctx* ctx);
const char* hdg_last_error(const hdg_ctx* ctx);
/* Use a caller-owned cudaStream_t for all work of this context (NULL = the library's own). */
int hdg_ctx_set_stream(hdg_ctx* ctx, void* cuda_stream);
/* Number of kernels this context has launched so far (for launch accounting). */
int64_t hdg_ctx_launch_count(const hdg_ctx* ctx);
/* Profiling: when on, the library times its own launches with CUDA events on its stream
 * (element, gather, apply, recover, the CG loop, and a sample of un-graphed CG iterations);
 * read them with hdg_system_timings.  No reference counterpart (the reference only has @time). */
int hdg_ctx_set_profiling(hdg_ctx* ctx, int on);

/* ---- mesh ---------------------------------------------------------------------------- */
/* rectangle_mesh(TriangleCell, (nx,ny), LL, UR): src/generate_mesh.jl:101-143.
 * With ctx == NULL (here and in hdg_mesh_from_cells) the mesh is host-only: its topology can be
 * queried, but no space can be built on it. */
int hdg_mesh_rectangle(hdg_ctx* ctx, int nx, int ny, const double LL[2], const double UR[2], hdg_mesh** out);
/* Triangle-format mesh from already-parsed arrays: parse_cells! face construction,
 * src/triangle_mesh.jl:48-108.  cell_nodes: ncells x 3 (1-based); edges: nedges x 3
 * (v1, v2, boundary marker) as in the .edge file. */
int hdg_mesh_from_cells(hdg_ctx* ctx, int nnodes, const double* xy, int ncells, const int32_t* cell_nodes,
                        int nedges, const int32_t* edges, hdg_mesh** out);
/* Replace all node coordinates (nnodes x 2).  Topology and face sets are kept. */
int hdg_mesh_set_coordinates(hdg_mesh* mesh, const double* xy);
/* Move interior nodes of a rectangle mesh by U(-a,a)*h per coordinate (seeded; h = cell size). */
int hdg_mesh_jitter(hdg_mesh* mesh, double a, uint64_t seed);
int hdg_mesh_sizes(const hdg_mesh* mesh, int* nnodes, int* ncells, int* nfaces);
/* Node coordinates (nnodes x 2), cell nodes and faces (ncells x 3, 1-based), and the face
 * table rows [v1 v2 cell1 cell2] (nfaces x 4, cell2 = 0 on the boundary), src/mesh.jl:43-49.
 * Any pointer may be NULL. */
int hdg_mesh_get_topology(const hdg_mesh* mesh, double* xy, int32_t* cell_nodes, int32_t* cell_faces,
                          int32_t* faces);
/* getfaceset(mesh, name), sorted ascending, 1-based: src/mesh.jl:75.  out may be NULL. */
int hdg_mesh_faceset(const hdg_mesh* mesh, const char* name, int32_t* out, int* count);
int hdg_mesh_destroy(hdg_mesh* mesh);

/* ---- function spaces ----------------------------------------------------------------- */
/* The triple (ScalarFunctionSpace, VectorFunctionSpace, ScalarTraceFunctionSpace) of
 * examples/poisson2D_HDG.jl:41-44 over one mesh: Dubiner degree p for u and q (component-major
 * vector dofs), Legendre degree p on the edges.  quad_degree <= 0 selects the reference default
 * p+1 (src/ScalarFunctionSpaces.jl:24-29). */
int hdg_space_create(hdg_mesh* mesh, int p, int quad_degree, hdg_space** out);
/* getnbasefunctions of W, V and M; getnquadpoints; getnfacequadpoints. */
int hdg_space_info(const hdg_space* space, int* nw, int* nv, int* nt, int* nq, int* nfq);
/* Reference tables: volume points (nq x 2), weights (nq), N (nw x nq), dN/dxi (nw x nq x 2),
 * face points (nfq), face weights (nfq), E (nw x nfq x 3), trace T (nt x nfq).  NULL skips. */
int hdg_space_tables(const hdg_space* space, double* pts, double* w, double* N, double* dN, double* fpts,
                     double* fw, double* E, double* T);
/* reinit!(fs, cell) geometry on the host: detJ, Jinv (2x2), detJf (3), unit normals (3x2).
 * src/ScalarFunctionSpaces.jl:101-132.  cell is 1-based. */
int hdg_space_cell_geometry(const hdg_space* space, int cell, double* detJ, double* Jinv, double* detJf,
                            double* normals);
int hdg_space_destroy(hdg_space* space);

/* ---- assembly and condensation ------------------------------------------------------- */
/* doassemble(Vh, Wh, Mh, tau), examples/poisson2D_HDG.jl:58-186, on the device: element
 * integrals, dense LU condensation, and the deterministic gather into the global trace system
 * (end_assemble's CSC with duplicates summed, src/assembler.jl:47-49; rhs scatter-add :55-60).
 * kappa (NULL = 1) scales the (q,v) term as (kappa^-1 q, v); kappa_cell (host, ncells, NULL =
 * unused) is a piecewise-constant alternative.  precision: HDG_PREC_*. */
int hdg_assemble_condense(hdg_space* space, double tau, const hdg_field* f, const hdg_field* kappa,
                          const double* kappa_cell, int precision, hdg_system** out);
/* Recompute with a new source and/or coefficient on the same mesh and space, reusing every
 * topology buffer (no reallocation). */
int hdg_system_reassemble(hdg_system* sys, double tau, const hdg_field* f, const hdg_field* kappa,
                          const double* kappa_cell);
/* Recompute the element blocks and the trace system with the coefficients already on the device
 * (those of the last assemble or reassemble call): no host transfer.  No reference counterpart. */
int hdg_system_reassemble_resident(hdg_system* sys);
/* Trace dofs, stored entries of K, local system size n = 3 nw, trace dofs per cell m = 3 nt. */
int hdg_system_sizes(const hdg_system* sys, int* ndofs, int64_t* nnz, int* n, int* m);
/* K and b as the reference holds them (sign included) in CSC; base 0 or 1 (Julia). */
int hdg_system_get_csc(const hdg_system* sys, int base, int64_t* colptr, int64_t* rowval, double* nzval,
                       double* rhs);
/* Per-cell condensed blocks: Ate (ncells x m x m), bte (ncells x m), K_e (ncells x n x m),
 * b_e (ncells x n); K_element / b_element of examples/poisson2D_HDG.jl:171-174.  NULL skips. */
int hdg_system_get_element_blocks(const hdg_system* sys, double* Ate, double* bte, double* Ke, double* be);

/* ---- boundary conditions ------------------------------------------------------------- */
/* Dirichlet(u_hat, mesh, faceset, g), src/boundary.jl:11-42: prescribed trace dofs (1-based)
 * and values.  The values follow the reference's projection exactly (its accumulator is not
 * reset between basis functions); they are all 0 for g = 0, the case every example uses.
 * dofs/vals may be NULL to query count. */
int hdg_dirichlet(const hdg_space* space, const char* faceset, const hdg_field* g, int32_t* dofs, double* vals,
                  int* count);
/* The corrected trace projection: u_i = int_0^1 g mu_i ds on every face of the set, the L2
 * projection onto the orthonormal Legendre basis (same arguments and dof order as hdg_dirichlet,
 * which keeps the reference's projection, src/boundary.jl:27-37, for parity). */
int hdg_dirichlet_l2(const hdg_space* space, const char* faceset, const hdg_field* g, int32_t* dofs, double* vals,
                     int* count);
/* on != 0: systems assembled from this space from now on use He = tau int mu mu dS in the
 * condensation (each system keeps the choice it was created with, also when reassembled).  The
 * reference's He carries no tau (examples/poisson2D_HDG.jl:149), consistent only for tau = 1. */
int hdg_space_set_he_tau(hdg_space* space, int on);
/* apply!(K, b, dbc), src/boundary.jl:121-158 (APPLY_TRANSPOSE): b -= v K[:,d]; zero rows and
 * columns of the prescribed dofs; K[d,d] = mean|diag K|; b[d] = v * mean|diag K|. */
int hdg_apply_dirichlet(hdg_system* sys, const int32_t* dofs, const double* vals, int n);

/* ---- solve --------------------------------------------------------------------------- */
/* Preconditioner of the trace CG. */
enum {
  HDG_PRECOND_JACOBI = 0, /* diagonal (the default) */
  HDG_PRECOND_AMG = 1     /* smoothed-aggregation multigrid V-cycle in FP32 (CG itself in FP64): Chebyshev
                             smoothing on the trace level, l1-Jacobi on the coarse levels */
};
typedef struct {
  double tol;         /* relative residual |r|/|b| to reach (default 1e-12) */
  int maxit;          /* iteration cap (default 100000) */
  int precision;      /* HDG_PREC_FP64: Jacobi-PCG in FP64; HDG_PREC_MIXED: FP32 iteration + FP64 refinement */
  int chunk;          /* CG iterations per CUDA-graph launch between convergence checks (default 32) */
  double inner_tol;   /* unused (kept for the layout of earlier callers) */
  int preconditioner; /* HDG_PRECOND_*; with AMG the CG runs in FP64 whatever `precision` says */
} hdg_solver;
typedef struct {
  int iterations;     /* inner CG iterations in total */
  int outer;          /* outer refinement steps (1 for FP64) */
  double rel_residual;/* final |b - K u|/|b| measured in FP64 */
  int converged;
} hdg_stats;
/* u_hat = K \ b (examples/poisson2D_HDG.jl:195) by Jacobi-preconditioned CG on the free
 * trace dofs.  uhat (host, ndofs) may be NULL to keep the result on the device only. */
int hdg_solve(hdg_system* sys, const hdg_solver* opts, double* uhat, hdg_stats* stats);
/* No reference counterpart (the reference's `K \ b`, examples/poisson2D_HDG.jl:195, is a direct
 * solve with a forward error of order cond(K) 2^-53).  FP64 iterative refinement of the current
 * device solution: `steps` times r = b - K u_hat in double-double arithmetic (exact products,
 * TwoSum accumulation), K d = r by the CG of hdg_solve (same preconditioner and precision) to the
 * relative residual correction_tol, u_hat += d.  Each step shrinks the error by about
 * correction_tol times the condition-dependent CG error factor, down to the rounding of u_hat,
 * so two steps after a 1e-12 CG give the assembled FP64 system's solution to a few ulps.  stats:
 * iterations = correction iterations (max over problems), outer = steps, rel_residual = the
 * double-double |b - K u_hat| / |b| after the last step.  uhat (host) may be NULL. */
int hdg_refine(hdg_system* sys, const hdg_solver* opts, int steps, double correction_tol, double* uhat,
               hdg_stats* stats);

/* ---- recovery and errors ------------------------------------------------------------- */
/* get_uσ!, examples/poisson2D_HDG.jl:197-212 (trace slice for any nt): q (ncells x nv),
 * u (ncells x nw), uhat per cell (ncells x 3 x nt).  Host outputs; NULL skips a copy. */
int hdg_recover(hdg_system* sys, double* q, double* u, double* uhat_cell);
/* errornorm(u_h, u_ex), src/DiscreteFunctions.jl:97-120: the SQUARED L2 error of the last
 * recovery. */
int hdg_errornorm_l2sq(hdg_system* sys, const hdg_field* u_exact, double* out);
/* nodal_avg(u_h), src/DiscreteFunctions.jl:81-95: at every mesh node, the mean over the node's
 * cells of the last recovered u evaluated at that node (host output, nnodes values).  The
 * reference feeds it to its plotting; here it is a plain buffer. */
int hdg_nodal_avg(hdg_system* sys, double* out);
int hdg_system_destroy(hdg_system* sys);

/* No counterpart in the reference.  The squared L2 error of hdg_errornorm_l2sq for callers that
 * cannot allocate device memory: a runtime that owns the whole device heap, or code inside a
 * region where allocation is forbidden.  All inputs are caller-owned DEVICE arrays: xy
 * (nnodes x 2), cells (ncells x 3, 0-based), u (ncells x nw, the recovered Dubiner coefficients).
 * The result goes to the host double *out.  The scratch is one fixed 32.8 KB device array per
 * device (at most 2048 doubles of tables, enough for p <= 4, and 1024 field parameters; larger
 * requests return HDG_ERR_CAPACITY; a field whose parameters do not cover its kind returns
 * HDG_ERR_ARG).  The call allocates nothing.  Calls that overlap on one device race on that
 * array, so the caller serialises them.  The first call on a device looks up the array's address
 * and must come before any stream capture; the address is kept for the process, and dropped after
 * a call that fails with a CUDA error (a device reset moves it).  Errors go to
 * hdg_noalloc_last_error(). */
int hdg_errornorm_l2sq_noalloc(int device, void* stream, int p, int quad_degree, int ncells, const double* xy,
                               const int32_t* cells, const double* u, const hdg_field* u_exact, double* out);
const char* hdg_noalloc_last_error(void);

typedef struct {
  double element_ms;   /* element assemble+condense kernel of the last (re)assembly */
  double gather_ms;    /* matrix + rhs gather of the last (re)assembly */
  double apply_ms;     /* apply! (meandiag, lift, zeroing) */
  double cg_ms;        /* whole CG loop of the last solve */
  double cg_a_ms;      /* mean duration of the CG product kernel (q = A z + beta q), sampled */
  double cg_b_ms;      /* mean duration of the CG update kernel (x, r, z), sampled */
  int cg_samples;      /* number of sampled iterations */
  int cg_iterations;   /* iterations of the last solve */
  double recover_ms;   /* last recovery */
  double cg_a_bytes;   /* mean algorithmic bytes of a sampled product-kernel launch (rows that iterated) */
  double cg_b_bytes;   /* mean algorithmic bytes of a sampled update-kernel launch */
  double cg_bytes;     /* algorithmic bytes of all iteration launches of the last solve */
} hdg_timings;
/* Per-phase device times recorded while profiling was on (0 where nothing was recorded). */
int hdg_system_timings(hdg_system* sys, hdg_timings* out);
/* No reference counterpart.  One kernel family timed launch by launch in the sampled chunks of
 * the last solve (profiling on): the summed CUDA-event durations, the summed algorithmic bytes
 * (rows of the problems that iterated times the bytes per row) and the number of launches.
 * HDG_SAMPLE_CHEB0: the level-0 Chebyshev smoother sweeps of the multigrid cycle;
 * HDG_SAMPLE_L1SWEEP: the l1-Jacobi sweeps of the first coarse level. */
#define HDG_SAMPLE_CHEB0 1
#define HDG_SAMPLE_L1SWEEP 2
int hdg_system_kernel_sample(hdg_system* sys, int which, double* total_ms, double* total_bytes, int* launches);

/* ---- batches of independent problems ------------------------------------------------ */
/* No reference counterpart: the reference solves one problem per script run.  A batch is a
 * disjoint union of problem meshes of one degree: one space, one system, one set of launches. */
/* Disjoint union of meshes (host-only parts, built with ctx == NULL, are fine): ids of part P are
 * shifted by the sizes of the parts before it; face sets are merged. */
int hdg_mesh_concat(hdg_ctx* ctx, int nparts, const hdg_mesh* const* parts, hdg_mesh** out);
/* Problems of a (union) mesh and their first node/cell/face (arrays of nprob+1, 0-based; NULL skips). */
int hdg_mesh_problems(const hdg_mesh* mesh, int* nprob, int32_t* node0, int32_t* cell0, int32_t* face0);
/* As hdg_assemble_condense, with one tau / source / kappa field per problem (arrays of nprob;
 * tau and kappa may be NULL). */
int hdg_assemble_condense_batch(hdg_space* space, const double* tau, const hdg_field* f, const hdg_field* kappa,
                                const double* kappa_cell, int precision, hdg_system** out);
int hdg_system_reassemble_batch(hdg_system* sys, const double* tau, const hdg_field* f, const hdg_field* kappa,
                                const double* kappa_cell);
/* Solves every problem of several systems (for example one per degree) in one interleaved loop;
 * each problem stops independently.  stats: one entry per problem, systems in order. */
int hdg_solve_batch(int nsys, hdg_system* const* systems, const hdg_solver* opts, hdg_stats* stats);
/* Uploads new per-problem coefficients (as hdg_system_reassemble_batch) without assembling:
 * the next hdg_batch_step with HDG_STEP_ASSEMBLE assembles from them. */
int hdg_system_set_coefficients_batch(hdg_system* sys, const double* tau, const hdg_field* f,
                                      const hdg_field* kappa, const double* kappa_cell);
/* Records a Dirichlet set (the arguments of hdg_apply_dirichlet) without applying it: the next
 * hdg_batch_step with HDG_STEP_APPLY applies it.  The set is kept across reassembly.  On a
 * system that is already applied, the new set takes effect after the next reassembly. */
int hdg_system_set_dirichlet(hdg_system* sys, const int32_t* dofs, const double* vals, int n);
#define HDG_STEP_ASSEMBLE 1 /* assemble + condense from the coefficients on the device */
#define HDG_STEP_APPLY 2    /* apply! the recorded Dirichlet set */
#define HDG_STEP_RECOVER 4  /* local recovery of (q, u) after the solve */
#define HDG_STEP_DOWNLOAD 8 /* copy each system's solution to its registered host arrays */
/* Page-locked host memory (cudaMallocHost), for download destinations that the device writes
 * directly and asynchronously. */
int hdg_host_alloc(size_t bytes, void** out);
int hdg_host_free(void* p);
/* Registers host destinations for HDG_STEP_DOWNLOAD: uhat (ndofs) and, after recovery, qu
 * (ncells x n, as hdg_system_get_solution); either may be NULL.  Page-locked memory
 * (hdg_host_alloc) lets the copies overlap the other systems' work; pageable memory works but
 * the copies then hold the host. */
int hdg_system_set_download(hdg_system* sys, double* uhat, double* qu);
/* One pipelined step over several systems: per system, on a CUDA stream of its own,
 * [assemble + condense] -> [apply!] -> CG -> [recovery], so that one system's assembly and
 * recovery overlap the other systems' iterations.  The results equal those of
 * hdg_system_reassemble_resident, hdg_apply_dirichlet, hdg_solve_batch and hdg_recover called
 * in turn.  Without HDG_STEP_APPLY the systems must be applied already (and HDG_STEP_ASSEMBLE,
 * which undoes apply!, is then refused).  With HDG_STEP_DOWNLOAD each system's solution is
 * copied to its registered host arrays on its own stream as soon as it is recovered; the call
 * returns once every copy has landed.  stats: one entry per problem, systems in order. */
int hdg_batch_step(int nsys, hdg_system* const* systems, const hdg_solver* opts, int flags, hdg_stats* stats);
/* Device solution of a system: trace values (ndofs) and, after recovery, [q; u] per cell (ncells x n). */
int hdg_system_get_solution(const hdg_system* sys, double* uhat, double* qu);

/* ---- continuous Galerkin (nodal Lagrange) Poisson path --------------------------------- */
/* examples/poisson2D_CG.jl / test/test_CGExample.jl on the device: -div(kappa grad u) = f with a
 * nodal ContinuousLagrange{2,RefTetrahedron,order} element (order 1..4, P1 geometry) whose dofs a
 * DofHandler numbered.  The system is assembled straight into the caller's CSC pattern (the one
 * create_sparsity_pattern returns), so K and b are those of start_assemble(K, f) + assemble! in
 * the reference's element loop (src/assembler.jl:62-137). */
typedef struct hdg_lagrange hdg_lagrange;
/* mesh on the device (ctx); cell_dofs: ncells x nbasefuncs, 1-based, as DofHandler.cell_dofs of a
 * one-field handler; colptr (ndofs+1) / rowval (nnz): 0-based CSC pattern with every element
 * coupling stored (else HDG_ERR_ARG).  quad_degree <= 0: order + 1 (the reference default). */
int hdg_lagrange_create(hdg_ctx* ctx, const hdg_mesh* mesh, int order, int quad_degree, int ndofs,
                        const int32_t* cell_dofs, int64_t nnz, const int64_t* colptr, const int64_t* rowval,
                        hdg_lagrange** out);
/* doassemble: K = sum_cells int kappa grad v . grad u, b = sum_cells int f v (kappa_cell may be
 * NULL: kappa = 1); HDG_ERR_NEG_DETJ for an inverted cell. */
int hdg_lagrange_assemble(hdg_lagrange* sys, const hdg_field* f, const double* kappa_cell);
/* K's stored values (nnz, in the pattern's order) and b (ndofs); either may be NULL. */
int hdg_lagrange_get_csc(hdg_lagrange* sys, double* nzval, double* rhs);
/* apply!(K, b, dbc), src/boundary.jl:121-158: dofs 1-based (sorted, as Dirichlet returns them). */
int hdg_lagrange_apply_dirichlet(hdg_lagrange* sys, const int32_t* dofs, const double* vals, int n);
/* u = K \ b by Jacobi-preconditioned CG in FP64 to opts->tol (relative residual); u (ndofs) may
 * be NULL (the solution stays on the device for hdg_lagrange_errornorm_l2sq). */
int hdg_lagrange_solve(hdg_lagrange* sys, const hdg_solver* opts, double* u, hdg_stats* stats);
/* errornorm(u_h, u_exact) (squared L2, src/DiscreteFunctions.jl:97-120) of the dof values u
 * (ndofs; NULL: the last solution). */
int hdg_lagrange_errornorm_l2sq(hdg_lagrange* sys, const double* u, const hdg_field* u_exact, double* out);
int hdg_lagrange_destroy(hdg_lagrange* sys);

/* ---- serving: continuous batching of solve requests ----------------------------------- */
/* No reference counterpart.  Requests queue on the host; every hdg_engine_step admits pending
 * requests into "flights" (one disjoint union system per degree, at most max_batch requests)
 * while the HBM budget and the flight slots allow, advances every flight by one chunk of CG
 * iterations on its own CUDA stream, and completes the flights whose problems are all done.
 * Requests arriving while others run join at the next step; flights overlap on the device.
 * Flights are built on HDG_ENGINE_BUILDERS worker threads (default 8); their launch autotuners
 * take cached choices instead of timing.  Measured on a 2000 req/s stream of problems of 130 to
 * 33000 cells: 16 flights of at most 32 requests served the most (965 requests/s), against 831
 * for 8 flights of 64. */
typedef struct hdg_engine hdg_engine;
int hdg_engine_create(hdg_ctx* ctx, double hbm_budget_gb, int max_batch, int max_flights, const hdg_solver* opts,
                      hdg_engine** out);
/* Registers a host mesh (built with ctx == NULL) of degree p as resident: requests on it need no
 * mesh construction.  With HDG_ENGINE_RESIDENT_COPIES=k (default 0) the engine also keeps up to k
 * device-resident single-problem systems per resident mesh (device mesh, space, trace system, CG
 * state, multigrid hierarchy fitted to the first request's matrix); a request on an idle one only
 * uploads its coefficients, reassembles and solves. */
int hdg_engine_add_resident_mesh(hdg_engine* e, const hdg_mesh* host_mesh, int p, int* mesh_id);
/* Queues a request on resident mesh `mesh_id`, or (mesh_id < 0) on its own host mesh `mesh`. */
int hdg_engine_submit(hdg_engine* e, int mesh_id, const hdg_mesh* mesh, int p, int quad_degree, const hdg_field* f,
                      const double* kappa_cell, double tau, int64_t* request_id);
int hdg_engine_step(hdg_engine* e, int* n_inflight, int* n_pending);
/* Completed requests since the last poll (at most max): id, latency in seconds, iterations,
 * true relative residual, converged flag.  NULL arrays are skipped. */
int hdg_engine_poll(hdg_engine* e, int max, int64_t* ids, double* latency, int* iterations, double* residual,
                    int* converged, int* n);
/* Solution of a completed request: û (its trace dofs), q (ncells x nv), u (ncells x nw); with all
 * three NULL only the sizes are returned.  Released after the copy. */
int hdg_engine_result(hdg_engine* e, int64_t id, double* uhat, double* q, double* u, int* nuhat, int* nq, int* nu);
int hdg_engine_set_keep_results(hdg_engine* e, int keep);
int hdg_engine_destroy(hdg_engine* e);

/* ---- whole flow ---------------------------------------------------------------------- */
/* The poisson2D_HDG flow in one call: assemble+condense, Dirichlet on `faceset` with g,
 * apply!, solve, recover.  Outputs are host arrays (any may be NULL). */
int hdg_solve_poisson(hdg_space* space, double tau, const hdg_field* f, const hdg_field* kappa,
                      const double* kappa_cell, const char* faceset, const hdg_field* g, const hdg_solver* opts,
                      double* uhat, double* q, double* u, hdg_stats* stats);

/* ---- triplet assembler (host) -------------------------------------------------------- */
/* start_assemble(N) / assemble!(a, edof, Ke) / end_assemble(a), src/assembler.jl:1-60.
 * Ke is ndofs x ndofs column-major (Julia order); edof is 1-based. */
int hdg_assembler_create(int64_t sizehint, hdg_assembler** out);
int hdg_assembler_add(hdg_assembler* a, int ndofs, const int64_t* edof, const double* Ke);
/* end_assemble -> CSC with duplicates summed; sizes first (colptr may be NULL), then values. */
int hdg_assembler_finish(hdg_assembler* a, int64_t* nrows, int64_t* ncols, int64_t* nnz);
int hdg_assembler_get_csc(const hdg_assembler* a, int base, int64_t* colptr, int64_t* rowval, double* nzval);
int hdg_assembler_destroy(hdg_assembler* a);

/* ---- DofHandler and the sparsity-pattern assembler (host) ------------------------------ */
/* DofHandler(fields, mesh), src/dofhandler.jl:13-16 and _distribute_dofs :91-151, for nodal
 * fields.  Field i carries vdofs[i] (0 or 1) dofs per vertex, fdofs[i] per face and cdofs[i] per
 * cell, each times ncomp[i] components (gettopology of its element, src/LagrangeFE.jl:60).
 * mesh must outlive the handler. */
typedef struct hdg_dofhandler hdg_dofhandler;
int hdg_dofhandler_create(const hdg_mesh* mesh, int nfields, const int* vdofs, const int* fdofs, const int* cdofs,
                          const int* ncomp, hdg_dofhandler** out);
/* ndofs(dh) and the length of cell_dofs. */
int hdg_dofhandler_sizes(const hdg_dofhandler* dh, int* ndofs, int64_t* ncelldofs);
/* dh.cell_dofs (1-based, concatenated per cell) and dh.cell_dofs_offset (ncells + 1, 1-based). */
int hdg_dofhandler_cell_dofs(const hdg_dofhandler* dh, int32_t* cell_dofs, int32_t* offsets);
/* dof_range(dh, field): first..last local dof of a field in a cell (1-based), src/dofhandler.jl:77-82. */
int hdg_dofhandler_field_range(const hdg_dofhandler* dh, int field, int* first, int* last);
/* create_sparsity_pattern / create_symmetric_sparsity_pattern (upper triangle),
 * src/dofhandler.jl:171-229: CSC pattern with the diagonal; sizes first (colptr/rowval NULL). */
int hdg_dofhandler_sparsity(const hdg_dofhandler* dh, int symmetric, int base, int64_t* colptr, int64_t* rowval,
                            int64_t* nnz);
/* Dirichlet(u, dh, faceset, f) dof selection, src/boundary.jl:44-95: sorted 1-based dofs of
 * field `field` (0-based) on the face set, with the cell (1-based) and local node (1-based) that
 * gives each one's nodal point for evaluating f.  Outputs may be NULL (count only). */
int hdg_dofhandler_dirichlet(const hdg_dofhandler* dh, const char* faceset, int field, int32_t* dofs, int32_t* cells,
                             int32_t* local, int* count);
int hdg_dofhandler_destroy(hdg_dofhandler* dh);
const char* hdg_dofhandler_last_error(void);
/* assemble!(A::AssemblerSparsityPattern, dofs, Ke, fe), src/assembler.jl:97-137, for nel
 * elements at once: K.nzval += Ke at the stored positions of a CSC pattern (colptr/rowval with
 * base 0 or 1, rows sorted per column), f += fe.  dofs (nel x ndofs_e) are 1-based; Ke is
 * column-major per element.  upper_only assembles the upper triangle (Symmetric pattern).  A
 * pair that is not stored is an error ("some row indices were not found"). */
int hdg_csc_assemble(int64_t n, const int64_t* colptr, const int64_t* rowval, int base, double* nzval, double* f,
                     int upper_only, int nel, int ndofs_e, const int64_t* dofs, const double* Ke, const double* fe);

#ifdef __cplusplus
}
#endif
#endif /* HDG_H */
