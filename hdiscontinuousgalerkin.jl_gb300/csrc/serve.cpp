// Serving engine: continuous batching of HDG solve requests on one GPU.
//
// Requests (a mesh, a degree, a source, a per-cell coefficient) queue on the host.  Each engine
// step
//   1. admits pending requests into new "flights" while the HBM budget allows: the requests of one
//      degree form a disjoint union mesh with one space and one trace system, assembled,
//      condensed and gathered by the same launches as a batch;
//   2. processes every flight whose last chunk of CG iterations has finished (its per-problem
//      status read back): a flight whose problems are all done is completed (recovery, result
//      copy, latency stamp) and its memory freed for the next admissions; any other is given its
//      next chunk at once.  Each flight runs on its own CUDA stream, so flights overlap on the
//      device and none waits for another.
// So requests that arrive while others are on the GPU join at the next chunk boundary: admission
// is by memory and slots, not by waiting for the device to drain.  Meshes registered as
// resident keep their host topology in the engine, so a request on a resident mesh costs no mesh
// construction.  No reference counterpart: the reference is a single-problem script.
#include <cstdio>
#include <cstdlib>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <condition_variable>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>

#include "hdg_internal.h"

namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Request {
  int64_t id;
  int mesh_id;                       // resident mesh, or -1
  std::shared_ptr<hdg_mesh> mesh;    // the host mesh (shared with the engine's list when resident)
  int p, qd;
  FieldSpec f;
  std::vector<double> kappa;         // per cell (empty = 1)
  double tau;
  double t_submit;
};

struct Result {
  int64_t id;
  double t_submit, t_done;
  hdg_stats stats;
  std::vector<double> uhat, q, u;
};

// Bytes a flight holds on the device, per cell of degree p (condensed blocks, FP64 and FP32
// matrix, CG vectors); a conservative estimate used for admission.
size_t bytes_per_cell(int p) {
  const size_t nt = p + 1, nw = (p + 1) * (p + 2) / 2, m = 3 * nt, n = 3 * nw;
  const double faces_per_cell = 1.6;
  return (size_t)(8 * (m * (m + 1) + n * (m + 1)) + faces_per_cell * (5 * nt * nt * 12 + 16 * nt * 8) + 64);
}

}  // namespace

struct Flight {
  hdg_ctx ctx;  // own stream
  std::vector<Request> reqs;
  hdg_mesh* mesh = nullptr;
  hdg_space* space = nullptr;
  hdg_system* sys = nullptr;
  CgSolver* cg = nullptr;
  int rep = 0;
  size_t bytes = 0;
  cudaEvent_t ready = nullptr;  // recorded after each chunk's status read-back
  double t[5] = {0, 0, 0, 0, 0};  // build time: concat, space, assemble, apply, prepare
  ~Flight() {
    if (ready) cudaEventDestroy(ready);
    delete cg;
    if (sys) hdg_system_destroy(sys);
    if (space) hdg_space_destroy(space);
    if (mesh) hdg_mesh_destroy(mesh);
  }
};

// A resident mesh's device-resident single-problem system: device mesh, space, trace system
// (with its Dirichlet set recorded), CG state and multigrid hierarchy stay allocated between
// requests.  A request on it uploads its source and coefficients, reassembles, applies the
// recorded Dirichlet set, runs the multigrid numeric set-up and the CG, and recovers: no mesh,
// space or system is built and no symbolic set-up runs.  The multigrid aggregates are the ones
// fitted to the first request's matrix; later coefficients keep a valid preconditioner.
struct ResidentSys {
  hdg_ctx ctx;  // own stream
  int mesh_id = -1, p = 0, qd = 0;
  hdg_mesh* mesh = nullptr;
  hdg_space* space = nullptr;
  hdg_system* sys = nullptr;
  CgSolver* cg = nullptr;
  cudaEvent_t ready = nullptr;
  bool busy = false;        // serving a request or being built
  bool completing = false;  // CG done; the final residual, recovery and downloads are queued
  int rep = 0;
  size_t bytes = 0;
  std::vector<Request> reqs;  // the request being served (one)
  double* h_x = nullptr;      // page-locked destinations of the solution downloads
  double* h_qu = nullptr;
  explicit ResidentSys(int device) {
    ctx.device = device;
    ctx.own_stream = false;
    ctx.profiling = false;
    HDG_CUDA(cudaStreamCreateWithFlags(&ctx.stream, cudaStreamNonBlocking));
    HDG_CUDA(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
  }
  ~ResidentSys() {
    cudaStreamSynchronize(ctx.stream);
    if (ready) cudaEventDestroy(ready);
    delete cg;
    if (sys) hdg_system_destroy(sys);
    if (space) hdg_space_destroy(space);
    if (mesh) hdg_mesh_destroy(mesh);
    if (h_x) cudaFreeHost(h_x);
    if (h_qu) cudaFreeHost(h_qu);
    cudaStreamDestroy(ctx.stream);
  }
};

struct hdg_engine {
  hdg_ctx* ctx = nullptr;
  double budget = 0;
  int max_batch = 256;
  int max_flights = 8;
  hdg_solver solver{};
  std::vector<std::shared_ptr<hdg_mesh>> resident;
  std::vector<int> resident_p;
  // device-resident systems per resident mesh (HDG_ENGINE_RESIDENT_COPIES of them at most; 0 turns
  // the resident path off and sends resident requests to union flights like the others)
  std::vector<std::vector<std::unique_ptr<ResidentSys>>> rpool;
  std::vector<ResidentSys*> ractive;  // serving a request
  // Off by default: on the 2000 req/s stream 2 / 4 copies per mesh served 311 / 373 requests/s
  // against 458 for union flights alone.  A resident request costs about 1 ms of host work, but a
  // single small problem is launch-bound (some 29 kernels per multigrid CG iteration), and the
  // aggregates fitted to the first request's kappa take about twice the iterations (157 against
  // 77 on average) for the next requests' random kappa.
  int resident_copies = 0;
  int64_t n_resident_solves = 0;
  double t_resident_start = 0;
  std::deque<Request> pending;
  std::vector<std::unique_ptr<Flight>> flights;
  std::deque<Result> done;
  std::vector<cudaStream_t> streams;  // pool, one per flight slot
  std::vector<char> stream_busy;
  size_t in_use = 0;
  int64_t next_id = 1;
  bool keep_results = true;
  // Flight builders: admission (union mesh, space, system, assembly, apply!, CG set-up) is host
  // work of 0.1 s and more per flight, so it runs on worker threads while step() keeps feeding
  // the flights in progress.  jobs / built / building / the t_* counters are guarded by mu.
  struct Job {
    std::vector<Request> reqs;
    int slot;
    size_t bytes;
    ResidentSys* rs;  // a resident system to build (slot unused), or null for a flight
  };
  std::vector<std::thread> builders;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Job> jobs;
  struct Done {  // a finished build: the flight (or resident system), or the failure of its admission
    Flight* fl;
    int slot;
    size_t bytes;
    int rc;
    std::string msg;
    int nreq;
    ResidentSys* rs;
  };
  std::vector<Done> built;
  int building = 0;       // jobs queued or being built
  int building_reqs = 0;  // their requests
  bool stop = false;
  // host time spent per phase (s), reported on destroy when HDG_ENGINE_VERBOSE is set
  double t_concat = 0, t_space = 0, t_assemble = 0, t_apply = 0, t_prepare = 0, t_complete = 0, t_wait = 0;
  double t_steps = 0;
  int64_t n_flights = 0, n_steps = 0;
};

namespace {

std::shared_ptr<hdg_mesh> copy_host_mesh(const hdg_mesh* m) {
  auto c = std::make_shared<hdg_mesh>();
  c->ctx = nullptr;
  c->nn = m->nn; c->nc = m->nc; c->nf = m->nf;
  c->xy = m->xy; c->cells = m->cells; c->cfaces = m->cfaces; c->faces = m->faces; c->facesets = m->facesets;
  c->structured = m->structured; c->nx = m->nx; c->ny = m->ny;
  c->LL[0] = m->LL[0]; c->LL[1] = m->LL[1]; c->UR[0] = m->UR[0]; c->UR[1] = m->UR[1];
  c->nprob = m->nprob; c->prob_node0 = m->prob_node0; c->prob_cell0 = m->prob_cell0; c->prob_face0 = m->prob_face0;
  return c;
}

const hdg_mesh* request_mesh(const hdg_engine*, const Request& r) { return r.mesh.get(); }

// Builds and starts a flight from `reqs` (same degree and quadrature) on stream slot `slot`.
Flight* launch_flight(hdg_engine* e, std::vector<Request>&& reqs, int slot) {
  std::unique_ptr<Flight> fl(new Flight());
  fl->ctx.device = e->ctx->device;
  fl->ctx.stream = e->streams[slot];
  fl->ctx.own_stream = false;
  fl->ctx.profiling = false;
  fl->reqs = std::move(reqs);
  std::vector<const hdg_mesh*> parts;
  for (auto& r : fl->reqs) parts.push_back(request_mesh(e, r));
  hdg_ctx* c = &fl->ctx;
  double t0 = now_s();
  int rc = hdg_mesh_concat(c, (int)parts.size(), parts.data(), &fl->mesh);
  if (rc != HDG_OK) throw HdgError{rc, c->err};
  double t1 = now_s();
  fl->t[0] += t1 - t0;
  const int p = fl->reqs[0].p, qd = fl->reqs[0].qd;
  rc = hdg_space_create(fl->mesh, p, qd, &fl->space);
  if (rc != HDG_OK) throw HdgError{rc, c->err};
  t0 = now_s();
  fl->t[1] += t0 - t1;
  const int np = (int)fl->reqs.size();
  std::vector<hdg_field> fs(np);
  std::vector<double> taus(np), kappa;
  bool any_kappa = false;
  for (auto& r : fl->reqs) any_kappa |= !r.kappa.empty();
  for (int P = 0; P < np; ++P) {
    const Request& r = fl->reqs[P];
    fs[P] = hdg_field{r.f.kind, (int)r.f.prm.size(), r.f.prm.data()};
    taus[P] = r.tau;
    if (any_kappa) {
      const int nc = request_mesh(e, r)->nc;
      if (r.kappa.empty()) kappa.insert(kappa.end(), nc, 1.0);
      else kappa.insert(kappa.end(), r.kappa.begin(), r.kappa.end());
    }
  }
  rc = hdg_assemble_condense_batch(fl->space, taus.data(), fs.data(), nullptr, any_kappa ? kappa.data() : nullptr,
                                   e->solver.precision, &fl->sys);
  if (rc != HDG_OK) throw HdgError{rc, c->err};
  t1 = now_s();
  fl->t[2] += t1 - t0;
  int cnt = 0;
  static const double kZero = 0.0;
  hdg_field zero{HDG_FIELD_CONST, 1, &kZero};
  rc = hdg_dirichlet(fl->space, "boundary", &zero, nullptr, nullptr, &cnt);
  if (rc != HDG_OK) throw HdgError{rc, c->err};
  std::vector<int32_t> dofs(cnt);
  std::vector<double> vals(cnt);
  rc = hdg_dirichlet(fl->space, "boundary", &zero, dofs.data(), vals.data(), &cnt);
  if (rc == HDG_OK) rc = hdg_apply_dirichlet(fl->sys, dofs.data(), vals.data(), cnt);
  if (rc != HDG_OK) throw HdgError{rc, c->err};
  t0 = now_s();
  fl->t[3] += t0 - t1;
  g_alloc_stream = c->stream;
  fl->cg = make_cg_solver(fl->sys);
  fl->cg->prepare(e->solver);
  HDG_CUDA(cudaEventCreateWithFlags(&fl->ready, cudaEventDisableTiming));
  fl->t[4] += now_s() - t0;
  return fl.release();
}

// Builds a resident system from its first request and queues that request's solve (set-up and
// first CG preparation, as a flight of one problem; the engine step gives it its chunks).
void build_resident(hdg_engine* e, ResidentSys* rs, std::vector<Request>&& reqs) {
  hdg_ctx* c = &rs->ctx;
  const Request& r = reqs[0];
  const hdg_mesh* part = request_mesh(e, r);
  int rc = hdg_mesh_concat(c, 1, &part, &rs->mesh);
  if (rc != HDG_OK) throw HdgError{rc, c->err};
  rc = hdg_space_create(rs->mesh, r.p, r.qd, &rs->space);
  if (rc != HDG_OK) throw HdgError{rc, c->err};
  hdg_field f{r.f.kind, (int)r.f.prm.size(), r.f.prm.data()};
  double tau = r.tau;
  rc = hdg_assemble_condense_batch(rs->space, &tau, &f, nullptr, r.kappa.empty() ? nullptr : r.kappa.data(),
                                   e->solver.precision, &rs->sys);
  if (rc != HDG_OK) throw HdgError{rc, c->err};
  int cnt = 0;
  static const double kZero = 0.0;
  hdg_field zero{HDG_FIELD_CONST, 1, &kZero};
  rc = hdg_dirichlet(rs->space, "boundary", &zero, nullptr, nullptr, &cnt);
  if (rc != HDG_OK) throw HdgError{rc, c->err};
  std::vector<int32_t> dofs(cnt);
  std::vector<double> vals(cnt);
  rc = hdg_dirichlet(rs->space, "boundary", &zero, dofs.data(), vals.data(), &cnt);
  if (rc == HDG_OK) rc = hdg_apply_dirichlet(rs->sys, dofs.data(), vals.data(), cnt);
  if (rc != HDG_OK) throw HdgError{rc, c->err};
  g_alloc_stream = c->stream;
  HDG_CUDA(cudaMallocHost(&rs->h_x, sizeof(double) * rs->sys->ndofs));
  HDG_CUDA(cudaMallocHost(&rs->h_qu, sizeof(double) * (size_t)rs->sys->nc * rs->sys->n));
  rs->cg = make_cg_solver(rs->sys);
  rs->cg->prepare(e->solver);
  rs->reqs = std::move(reqs);
  rs->rep = 0;
}

// Starts a request on an idle, built resident system (engine thread): new coefficients,
// reassembly, apply! of the recorded Dirichlet set and the CG preparation (the multigrid's numeric
// set-up) are queued on the system's stream; the engine step gives it its chunks.
void start_resident(hdg_engine* e, ResidentSys* rs, Request&& r) {
  hdg_system* s = rs->sys;
  const cudaStream_t st = rs->ctx.stream;
  hdg_field f{r.f.kind, (int)r.f.prm.size(), r.f.prm.data()};
  double tau = r.tau;
  int rc = hdg_system_set_coefficients_batch(s, &tau, &f, nullptr, r.kappa.empty() ? nullptr : r.kappa.data());
  if (rc != HDG_OK) throw HdgError{rc, rs->ctx.err};
  g_alloc_stream = st;
  assemble_async(s, st);
  launch_dirichlet_apply(s, st);
  s->applied = true;
  rs->cg->prepare(e->solver);
  rs->reqs.clear();
  rs->reqs.push_back(std::move(r));
  rs->rep = 0;
}

// Worker thread: builds flights from the job queue until the engine stops.
void builder_main(hdg_engine* e) {
  cudaSetDevice(e->ctx->device);
  g_tuning_allowed = false;  // flights are solved once: autotuners take cached choices here
  for (;;) {
    hdg_engine::Job job;
    {
      std::unique_lock<std::mutex> lk(e->mu);
      e->cv.wait(lk, [&] { return e->stop || !e->jobs.empty(); });
      if (e->stop) return;
      job = std::move(e->jobs.front());
      e->jobs.pop_front();
    }
    hdg_engine::Done d{nullptr, job.slot, job.bytes, HDG_OK, std::string(), (int)job.reqs.size(), job.rs};
    try {
      if (job.rs) {
        build_resident(e, job.rs, std::move(job.reqs));
      } else {
        d.fl = launch_flight(e, std::move(job.reqs), job.slot);
        d.fl->bytes = job.bytes;
      }
    } catch (const HdgError& err) {
      d.rc = err.code;
      d.msg = err.msg;
    } catch (const std::exception& ex) {
      d.rc = HDG_ERR_CUDA;
      d.msg = ex.what();
    }
    std::lock_guard<std::mutex> lk(e->mu);
    if (d.fl) {
      e->t_concat += d.fl->t[0];
      e->t_space += d.fl->t[1];
      e->t_assemble += d.fl->t[2];
      e->t_apply += d.fl->t[3];
      e->t_prepare += d.fl->t[4];
      ++e->n_flights;
    }
    e->built.push_back(std::move(d));
  }
}

void file_results(hdg_engine* e, const hdg_system* s, const hdg_mesh* m, const std::vector<Request>& reqs,
                  const std::vector<hdg_stats>& st, const double* x, const double* qu);

// Finishes the CG of a flight or resident system, recovers q and u, and files one result per request.
void complete_solves(hdg_engine* e, hdg_ctx* ctx, CgSolver* cg, hdg_system* s, const hdg_mesh* m,
                     const std::vector<Request>& reqs) {
  std::vector<hdg_stats> st;
  g_alloc_stream = ctx->stream;
  cg->finish(e->solver, &st);
  s->have_solution = true;
  launch_recover(s, ctx->stream);
  s->have_recovery = true;
  std::vector<double> x, qu;
  if (e->keep_results) {
    x.resize(s->ndofs);
    qu.resize((size_t)s->nc * s->n);
    s->d_x.download(x.data(), x.size(), ctx->stream);
    s->d_qu.download(qu.data(), qu.size(), ctx->stream);
  }
  HDG_CUDA(cudaStreamSynchronize(ctx->stream));
  file_results(e, s, m, reqs, st, x.data(), qu.data());
}

// One result per request of a finished system (x, qu: its downloaded solution, if kept).
void file_results(hdg_engine* e, const hdg_system* s, const hdg_mesh* m, const std::vector<Request>& reqs,
                  const std::vector<hdg_stats>& st, const double* x, const double* qu) {
  const double t = now_s();
  const int nv = 2 * s->nw;
  for (size_t P = 0; P < reqs.size(); ++P) {
    Result r;
    r.id = reqs[P].id;
    r.t_submit = reqs[P].t_submit;
    r.t_done = t;
    r.stats = st[P];
    if (e->keep_results) {
      r.uhat.assign(x + (size_t)m->prob_face0[P] * s->nt, x + (size_t)m->prob_face0[P + 1] * s->nt);
      for (int c = m->prob_cell0[P]; c < m->prob_cell0[P + 1]; ++c) {
        r.q.insert(r.q.end(), qu + (size_t)c * s->n, qu + (size_t)c * s->n + nv);
        r.u.insert(r.u.end(), qu + (size_t)c * s->n + nv, qu + (size_t)(c + 1) * s->n);
      }
    }
    e->done.push_back(std::move(r));
  }
}

void complete_flight(hdg_engine* e, Flight* fl) {
  complete_solves(e, &fl->ctx, fl->cg, fl->sys, fl->mesh, fl->reqs);
}

}  // namespace

extern "C" {

int hdg_engine_create(hdg_ctx* ctx, double hbm_budget_gb, int max_batch, int max_flights, const hdg_solver* opts,
                      hdg_engine** out) {
  if (!ctx || !out || !(hbm_budget_gb > 0) || max_batch < 1 || max_flights < 1) return HDG_ERR_ARG;
  try {
    HDG_CUDA(cudaSetDevice(ctx->device));
    hdg_engine* e = new hdg_engine();
    e->ctx = ctx;
    e->budget = hbm_budget_gb * 1e9;
    e->max_batch = max_batch;
    e->max_flights = max_flights;
    hdg_solver d{1e-10, 100000, HDG_PREC_MIXED, 32, 1e-5, HDG_PRECOND_JACOBI};
    e->solver = opts ? *opts : d;
    if (!(e->solver.tol > 0)) e->solver.tol = d.tol;
    if (e->solver.maxit <= 0) e->solver.maxit = d.maxit;
    if (e->solver.chunk <= 0) e->solver.chunk = d.chunk;
    if (e->solver.preconditioner != HDG_PRECOND_AMG) e->solver.preconditioner = HDG_PRECOND_JACOBI;
    e->streams.resize(max_flights);
    e->stream_busy.assign(max_flights, 0);
    for (auto& s : e->streams) HDG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    // HDG_ENGINE_BUILDERS worker threads build flights (default 8, at most the flight slots;
    // on the 2000 req/s stream 4 / 8 / 12 builders served 392 / 458 / 429 requests/s)
    int nb = 8;
    if (const char* env = std::getenv("HDG_ENGINE_BUILDERS")) nb = std::atoi(env);
    nb = std::max(1, std::min(nb, std::max(1, max_flights)));
    for (int i = 0; i < nb; ++i) e->builders.emplace_back(builder_main, e);
    if (const char* env = std::getenv("HDG_ENGINE_RESIDENT_COPIES")) e->resident_copies = std::max(0, std::atoi(env));
    *out = e;
    return HDG_OK;
  } catch (const HdgError& err) {
    ctx->err = err.msg;
    return err.code;
  }
}

int hdg_engine_add_resident_mesh(hdg_engine* e, const hdg_mesh* host_mesh, int p, int* mesh_id) {
  if (!e || !host_mesh || !mesh_id) return HDG_ERR_ARG;
  e->resident.push_back(copy_host_mesh(host_mesh));
  e->resident_p.push_back(p);
  e->rpool.emplace_back();
  *mesh_id = (int)e->resident.size() - 1;
  return HDG_OK;
}

int hdg_engine_submit(hdg_engine* e, int mesh_id, const hdg_mesh* mesh, int p, int quad_degree, const hdg_field* f,
                      const double* kappa_cell, double tau, int64_t* request_id) {
  if (!e || !f || (mesh_id < 0 && !mesh) || mesh_id >= (int)e->resident.size() || p < 1 || p > HDG_MAX_P)
    return HDG_ERR_ARG;
  if (field_check(f, nullptr) != HDG_OK) return HDG_ERR_ARG;
  Request r;
  r.id = e->next_id++;
  r.mesh_id = mesh_id;
  r.mesh = mesh_id >= 0 ? e->resident[mesh_id] : copy_host_mesh(mesh);
  r.p = p;
  r.qd = quad_degree > 0 ? quad_degree : p + 1;
  r.f = field_from(f, 0.0);
  const int nc = mesh_id >= 0 ? e->resident[mesh_id]->nc : mesh->nc;
  if (kappa_cell) r.kappa.assign(kappa_cell, kappa_cell + nc);
  r.tau = tau > 0 ? tau : 1.0;
  r.t_submit = now_s();
  e->pending.push_back(std::move(r));
  if (request_id) *request_id = e->pending.back().id;
  return HDG_OK;
}

// One engine step: admit, advance every flight by one chunk, complete finished flights.
int hdg_engine_step(hdg_engine* e, int* n_inflight, int* n_pending) {
  if (!e) return HDG_ERR_ARG;
  const double ts = now_s();
  struct StepClock {
    hdg_engine* e;
    double t0;
    ~StepClock() {
      e->t_steps += now_s() - t0;
      ++e->n_steps;
    }
  } clock{e, ts};
  try {
    HDG_CUDA(cudaSetDevice(e->ctx->device));
    // 0. flights the builders finished join the ones in progress (their first chunk goes below)
    std::vector<hdg_engine::Done> done;
    int building = 0;
    {
      std::lock_guard<std::mutex> lk(e->mu);
      done.swap(e->built);
      for (auto& d : done) {
        --e->building;
        e->building_reqs -= d.nreq;
      }
      building = e->building;
    }
    int fail_rc = HDG_OK;
    for (auto& d : done) {
      if (d.rs) {
        if (d.rc == HDG_OK) {
          e->ractive.push_back(d.rs);
        } else {  // the resident system could not be built: drop it, report after the step
          auto& pool = e->rpool[d.rs->mesh_id];
          for (size_t k = 0; k < pool.size(); ++k)
            if (pool[k].get() == d.rs) {
              pool.erase(pool.begin() + k);
              break;
            }
          e->in_use -= d.bytes;
          fail_rc = d.rc;
          e->ctx->err = d.msg;
        }
      } else if (d.fl) {
        e->flights.emplace_back(d.fl);
      } else {  // the admission failed: free its slot and memory, report after the step
        e->stream_busy[d.slot] = 0;
        e->in_use -= d.bytes;
        fail_rc = d.rc;
        e->ctx->err = d.msg;
      }
    }
    // 1a. requests on resident meshes of their registered degree go to an idle resident system of
    //     that mesh (started here, nothing built), or to a new one while the mesh has fewer than
    //     resident_copies (built by a builder), or wait for one to become idle
    auto resident_eligible = [&](const Request& r) {
      return e->resident_copies > 0 && r.mesh_id >= 0 && r.p == e->resident_p[r.mesh_id];
    };
    for (auto it = e->pending.begin(); it != e->pending.end();) {
      if (!resident_eligible(*it)) {
        ++it;
        continue;
      }
      auto& pool = e->rpool[it->mesh_id];
      ResidentSys* idle = nullptr;
      for (auto& r : pool)
        if (!r->busy && r->qd == it->qd) {
          idle = r.get();
          break;
        }
      if (idle) {
        idle->busy = true;
        const double t0 = now_s();
        start_resident(e, idle, std::move(*it));
        e->t_resident_start += now_s() - t0;
        e->ractive.push_back(idle);
        it = e->pending.erase(it);
        continue;
      }
      const size_t b = bytes_per_cell(it->p) * (size_t)e->resident[it->mesh_id]->nc;
      if ((int)pool.size() < e->resident_copies && e->in_use + b <= e->budget) {
        pool.emplace_back(new ResidentSys(e->ctx->device));
        ResidentSys* rs = pool.back().get();
        rs->mesh_id = it->mesh_id;
        rs->p = it->p;
        rs->qd = it->qd;
        rs->busy = true;
        rs->bytes = b;
        e->in_use += b;
        std::vector<Request> one;
        one.push_back(std::move(*it));
        it = e->pending.erase(it);
        {
          std::lock_guard<std::mutex> lk(e->mu);
          e->building_reqs += 1;
          ++e->building;
          e->jobs.push_back(hdg_engine::Job{std::move(one), -1, b, rs});
        }
        e->cv.notify_one();
        continue;
      }
      ++it;
    }
    {
      std::lock_guard<std::mutex> lk(e->mu);
      building = e->building;
    }
    // 1. admission: one flight per (degree, quadrature) group of the pending queue, FIFO order,
    //    handed to the builders
    while ((int)e->flights.size() + building < e->max_flights) {
      auto first = e->pending.begin();
      while (first != e->pending.end() && resident_eligible(*first)) ++first;
      if (first == e->pending.end()) break;
      const int p = first->p, qd = first->qd;
      std::vector<Request> take;
      size_t bytes = 0;
      for (auto it = first; it != e->pending.end() && (int)take.size() < e->max_batch;) {
        if (it->p != p || it->qd != qd || resident_eligible(*it)) { ++it; continue; }
        const size_t b = bytes_per_cell(p) * (size_t)request_mesh(e, *it)->nc;
        if (e->in_use + bytes + b > e->budget && !take.empty()) break;
        if (e->in_use + bytes + b > e->budget && !e->flights.empty()) break;  // wait for memory
        bytes += b;
        take.push_back(std::move(*it));
        it = e->pending.erase(it);
      }
      if (take.empty()) break;
      int slot = 0;
      while (e->stream_busy[slot]) ++slot;
      e->stream_busy[slot] = 1;
      e->in_use += bytes;
      {
        std::lock_guard<std::mutex> lk(e->mu);
        e->building_reqs += (int)take.size();
        ++e->building;
        e->jobs.push_back(hdg_engine::Job{std::move(take), slot, bytes, nullptr});
      }
      ++building;
      e->cv.notify_one();
    }
    // 2. every flight whose last status read-back has landed is processed at once: completed, or
    //    given its next chunk.  Flights still iterating are left alone, so no flight waits for
    //    another.  When none is ready the step polls for up to 0.2 ms before returning, so that
    //    the caller can admit new arrivals.
    const double tw = now_s();
    bool progressed = false;
    for (int spin = 0;; ++spin) {
      for (size_t i = 0; i < e->flights.size();) {
        Flight* fl = e->flights[i].get();
        g_alloc_stream = fl->ctx.stream;
        if (fl->rep > 0) {  // a chunk is queued: has its read-back landed?
          const cudaError_t q = cudaEventQuery(fl->ready);
          if (q == cudaErrorNotReady) {
            ++i;
            continue;
          }
          HDG_CUDA(q);
          progressed = true;
          if (fl->cg->process(e->solver)) {
            const double tc = now_s();
            complete_flight(e, fl);
            e->t_complete += now_s() - tc;
            e->ctx->launches += fl->ctx.launches;
            for (size_t k = 0; k < e->streams.size(); ++k)
              if (e->streams[k] == fl->ctx.stream) e->stream_busy[k] = 0;
            e->in_use -= fl->bytes;
            e->flights.erase(e->flights.begin() + i);
            continue;
          }
        }
        progressed = true;
        fl->cg->launch_chunk(fl->rep++);
        fl->cg->enqueue_status_copy();
        HDG_CUDA(cudaEventRecord(fl->ready, fl->ctx.stream));
        ++i;
      }
      for (size_t i = 0; i < e->ractive.size();) {
        ResidentSys* rs = e->ractive[i];
        g_alloc_stream = rs->ctx.stream;
        if (rs->rep > 0 || rs->completing) {
          const cudaError_t q = cudaEventQuery(rs->ready);
          if (q == cudaErrorNotReady) {
            ++i;
            continue;
          }
          HDG_CUDA(q);
          progressed = true;
          const double tc = now_s();
          if (rs->completing) {  // the final residual, recovery and downloads have landed
            std::vector<hdg_stats> st;
            rs->cg->finish_collect(&st);
            file_results(e, rs->sys, rs->mesh, rs->reqs, st, rs->h_x, rs->h_qu);
            e->t_complete += now_s() - tc;
            e->ctx->launches += rs->ctx.launches;
            rs->ctx.launches = 0;
            ++e->n_resident_solves;
            rs->completing = false;
            rs->busy = false;
            e->ractive.erase(e->ractive.begin() + i);
            continue;
          }
          if (rs->cg->process(e->solver)) {  // converged: queue the completion, poll it later
            hdg_system* s = rs->sys;
            rs->cg->finish_enqueue();
            s->have_solution = true;
            launch_recover(s, rs->ctx.stream);
            s->have_recovery = true;
            if (e->keep_results) {
              s->d_x.download(rs->h_x, (size_t)s->ndofs, rs->ctx.stream);
              s->d_qu.download(rs->h_qu, (size_t)s->nc * s->n, rs->ctx.stream);
            }
            HDG_CUDA(cudaEventRecord(rs->ready, rs->ctx.stream));
            rs->completing = true;
            e->t_complete += now_s() - tc;
            ++i;
            continue;
          }
        }
        progressed = true;
        rs->cg->launch_chunk(rs->rep++);
        rs->cg->enqueue_status_copy();
        HDG_CUDA(cudaEventRecord(rs->ready, rs->ctx.stream));
        ++i;
      }
      if (progressed || now_s() - tw > 2e-4) break;
      std::this_thread::yield();
    }
    if (!progressed) e->t_wait += now_s() - tw;
    if (n_inflight) {  // requests being built count as in flight
      int n = (int)e->ractive.size();
      for (auto& fl : e->flights) n += (int)fl->reqs.size();
      std::lock_guard<std::mutex> lk(e->mu);
      *n_inflight = n + e->building_reqs;
    }
    if (n_pending) *n_pending = (int)e->pending.size();
    return fail_rc;
  } catch (const HdgError& err) {
    e->ctx->err = err.msg;
    return err.code;
  }
}

// Completed requests since the last poll: ids, latency (s), CG iterations, final relative
// residual, converged flag.  Results stay available to hdg_engine_result until taken.
int hdg_engine_poll(hdg_engine* e, int max, int64_t* ids, double* latency, int* iterations, double* residual,
                    int* converged, int* n) {
  if (!e || !n) return HDG_ERR_ARG;
  int k = 0;
  for (auto& r : e->done) {
    if (k >= max) break;
    if (r.t_done < 0) continue;  // already polled
    if (ids) ids[k] = r.id;
    if (latency) latency[k] = r.t_done - r.t_submit;
    if (iterations) iterations[k] = r.stats.iterations;
    if (residual) residual[k] = r.stats.rel_residual;
    if (converged) converged[k] = r.stats.converged;
    r.t_done = -1.0;
    ++k;
  }
  *n = k;
  while (!e->done.empty() && e->done.front().t_done < 0 && e->done.front().uhat.empty()) e->done.pop_front();
  return HDG_OK;
}

// Solution of a completed request (trace values, q per cell, u per cell; any may be NULL to query
// sizes); the result is released after this call.
int hdg_engine_result(hdg_engine* e, int64_t id, double* uhat, double* q, double* u, int* nuhat, int* nq, int* nu) {
  if (!e) return HDG_ERR_ARG;
  for (auto it = e->done.begin(); it != e->done.end(); ++it) {
    if (it->id != id) continue;
    if (nuhat) *nuhat = (int)it->uhat.size();
    if (nq) *nq = (int)it->q.size();
    if (nu) *nu = (int)it->u.size();
    if (!uhat && !q && !u) return HDG_OK;
    if (uhat) std::memcpy(uhat, it->uhat.data(), it->uhat.size() * sizeof(double));
    if (q) std::memcpy(q, it->q.data(), it->q.size() * sizeof(double));
    if (u) std::memcpy(u, it->u.data(), it->u.size() * sizeof(double));
    it->uhat.clear(); it->uhat.shrink_to_fit();
    it->q.clear(); it->q.shrink_to_fit();
    it->u.clear(); it->u.shrink_to_fit();
    return HDG_OK;
  }
  return HDG_ERR_ARG;
}

int hdg_engine_set_keep_results(hdg_engine* e, int keep) {
  if (!e) return HDG_ERR_ARG;
  e->keep_results = keep != 0;
  return HDG_OK;
}

int hdg_engine_destroy(hdg_engine* e) {
  if (!e) return HDG_OK;
  {
    std::lock_guard<std::mutex> lk(e->mu);
    e->stop = true;
    e->jobs.clear();
  }
  e->cv.notify_all();
  for (auto& t : e->builders) t.join();
  for (auto& d : e->built) delete d.fl;
  e->built.clear();
  if (std::getenv("HDG_ENGINE_VERBOSE"))
    std::fprintf(stderr,
                 "engine: %lld steps %.3f s, %lld flights; host s: concat %.3f space %.3f assemble %.3f apply %.3f "
                 "prepare %.3f complete %.3f wait %.3f; resident solves %lld, start %.3f\n",
                 (long long)e->n_steps, e->t_steps, (long long)e->n_flights, e->t_concat, e->t_space, e->t_assemble,
                 e->t_apply, e->t_prepare, e->t_complete, e->t_wait, (long long)e->n_resident_solves,
                 e->t_resident_start);
  cudaSetDevice(e->ctx->device);
  for (auto& fl : e->flights) cudaStreamSynchronize(fl->ctx.stream);
  e->flights.clear();
  e->ractive.clear();
  e->rpool.clear();
  for (auto s : e->streams) {
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
  }
  delete e;
  return HDG_OK;
}

}  // extern "C"
