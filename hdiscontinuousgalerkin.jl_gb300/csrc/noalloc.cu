// errornorm without device allocation.
//
// Some callers of this library cannot allocate device memory: an embedding runtime that owns the
// whole device heap (a Julia GC-managed pool, a serving process with a fixed arena), or code that
// runs inside a region where allocation is forbidden.  They can still evaluate the squared L2 error
// of a recovered solution on arrays they already hold: this entry point computes what
// hdg_errornorm_l2sq computes, but its scratch (per-block partial sums, the reduction ticket, the
// quadrature tables and the field parameters) lives in one file-scope device array of fixed size,
// so it calls no cudaMalloc/cudaFree and no allocating library routine.
//
// Limits and rules, stated for the user:
//  * the scratch holds at most NA_TABLE doubles of basis/quadrature tables (p <= 4 with any rule
//    the spaces accept fits) and NA_PARAMS field parameters; larger requests fail with
//    HDG_ERR_CAPACITY and touch nothing;
//  * every call on a device shares the one array, which keeps the last call's contents: calls that
//    overlap on the GPU (different streams, or threads) race and must be serialised by the caller;
//  * the first call on each device looks up the array's device address (set-up, once per device,
//    with that device current); make that first call before any stream capture.  The address is
//    cached for the process; a call that fails with a CUDA error drops it, so that after a device
//    reset (which reloads the module) the next call looks it up again.
#include <mutex>

#include "hdg_device.cuh"

namespace {

constexpr int NA_BLOCKS = 1024;  // partial sums (grid-stride kernel with at most this many blocks)
constexpr int NA_TABLE = 2048;   // N (nw x nq), weights (nq), points (2 nq)
constexpr int NA_PARAMS = 1024;  // exact-solution field parameters
constexpr int NA_OFF_TABLE = NA_BLOCKS;
constexpr int NA_OFF_PARAMS = NA_OFF_TABLE + NA_TABLE;
constexpr int NA_OFF_TICKET = NA_OFF_PARAMS + NA_PARAMS;  // one unsigned in a double slot
constexpr int NA_OFF_RESULT = NA_OFF_TICKET + 1;
constexpr int NA_TOTAL = NA_OFF_RESULT + 7;  // 4104 doubles = 32.8 KB per device

static __device__ __align__(256) double hdg_noalloc_scratch[NA_TOTAL];

// Device address of the scratch array, per device (host code may not use the symbol directly:
// on the host it is only a stand-in, not a device address).
std::mutex g_na_lock;
double* g_na_ptr[64] = {nullptr};

int na_setup(int device, double** out) {
  if (device < 0 || device >= 64) return HDG_ERR_ARG;
  std::lock_guard<std::mutex> lk(g_na_lock);
  if (!g_na_ptr[device]) {
    int cur = 0;
    if (cudaGetDevice(&cur) != cudaSuccess) return HDG_ERR_CUDA;
    if (cudaSetDevice(device) != cudaSuccess) return HDG_ERR_CUDA;
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, hdg_noalloc_scratch);
    cudaSetDevice(cur);
    if (e != cudaSuccess || !p) return HDG_ERR_CUDA;
    g_na_ptr[device] = (double*)p;
  }
  *out = g_na_ptr[device];
  return HDG_OK;
}

template <int P>
__global__ void k_errornorm_na(const int nc, const int32_t* __restrict__ cells, const double* __restrict__ xy,
                               const double* __restrict__ u, int nq, int ukind, double* scratch) {
  constexpr int NW = Dims<P>::NW;
  __shared__ double sh[32];
  __shared__ bool last;
  const double* N = scratch + NA_OFF_TABLE;       // [NW][nq]
  const double* w = N + NW * nq;                  // [nq]
  const double* pts = w + nq;                     // [nq][2]
  const double* prm = scratch + NA_OFF_PARAMS;
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
      for (int a = 0; a < NW; ++a) uh += u[(int64_t)c * NW + a] * N[a * nq + q];
      const double xi = pts[2 * q], eta = pts[2 * q + 1];
      const double xq = (1.0 - xi - eta) * x1 + xi * x2 + eta * x3;
      const double yq = (1.0 - xi - eta) * y1 + xi * y2 + eta * y3;
      const double d = uh - eval_field_kind(ukind, prm, xq, yq);
      el += d * d * detJ * w[q];
    }
    acc += el;
  }
  acc = block_sum<256>(acc, sh);
  if (threadIdx.x == 0) {
    scratch[blockIdx.x] = acc;
    __threadfence();
    unsigned* ticket = reinterpret_cast<unsigned*>(scratch + NA_OFF_TICKET);
    last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (last) {
    __threadfence();
    double s = 0.0;
    for (int k = threadIdx.x; k < gridDim.x; k += blockDim.x) s += ((volatile double*)scratch)[k];
    s = block_sum<256>(s, sh);
    if (threadIdx.x == 0) scratch[NA_OFF_RESULT] = s;
  }
}

thread_local std::string g_na_err;

}  // namespace

extern "C" {

const char* hdg_noalloc_last_error(void) { return g_na_err.c_str(); }

int hdg_errornorm_l2sq_noalloc(int device, void* stream, int p, int quad_degree, int ncells, const double* xy,
                               const int32_t* cells, const double* u, const hdg_field* u_exact, double* out) {
  if (p < 1 || p > HDG_MAX_P || ncells < 1 || !xy || !cells || !u || !u_exact || !out) {
    g_na_err = "hdg_errornorm_l2sq_noalloc: bad arguments";
    return HDG_ERR_ARG;
  }
  const int qd = quad_degree > 0 ? quad_degree : p + 1;
  // host-side reference tables, built once per (p, quadrature) and kept
  static std::mutex tl;
  static std::map<std::pair<int, int>, RefTables> cache;
  const RefTables* t = nullptr;
  {
    std::lock_guard<std::mutex> lk(tl);
    auto key = std::make_pair(p, qd);
    auto it = cache.find(key);
    if (it == cache.end()) {
      RefTables nt;
      if (!build_ref_tables(p, qd, &nt)) {
        g_na_err = "Quadrature rule of order " + std::to_string(qd) + " not available";
        return HDG_ERR_BAD_ORDER;
      }
      it = cache.emplace(key, std::move(nt)).first;
    }
    t = &it->second;
  }
  const int nq = t->nq, nw = t->nw;
  const int need = nw * nq + 3 * nq;
  if (need > NA_TABLE) {
    g_na_err = "hdg_errornorm_l2sq_noalloc: tables of " + std::to_string(need) + " doubles exceed the " +
               std::to_string(NA_TABLE) + "-double scratch";
    return HDG_ERR_CAPACITY;
  }
  if (u_exact->nparams < 0 || (u_exact->nparams > 0 && !u_exact->params)) {
    g_na_err = "hdg_errornorm_l2sq_noalloc: negative parameter count or missing parameters";
    return HDG_ERR_ARG;
  }
  if (u_exact->nparams > NA_PARAMS) {
    g_na_err = "hdg_errornorm_l2sq_noalloc: more than " + std::to_string(NA_PARAMS) + " field parameters";
    return HDG_ERR_CAPACITY;
  }
  {
    std::string why;
    if (field_check(u_exact, &why) != HDG_OK) {
      g_na_err = "hdg_errornorm_l2sq_noalloc: " + why;
      return HDG_ERR_ARG;
    }
  }
  double* scratch = nullptr;
  int rc = na_setup(device, &scratch);
  if (rc != HDG_OK) {
    g_na_err = "hdg_errornorm_l2sq_noalloc: scratch set-up failed on this device";
    return rc;
  }
  // host staging in a static buffer: no allocation per call
  static thread_local double stage[NA_TABLE + NA_PARAMS];
  for (int a = 0; a < nw; ++a)
    for (int q = 0; q < nq; ++q) stage[a * nq + q] = t->N[a * nq + q];
  for (int q = 0; q < nq; ++q) {
    stage[nw * nq + q] = t->qw[q];
    stage[nw * nq + nq + 2 * q] = t->qx[q];
    stage[nw * nq + nq + 2 * q + 1] = t->qy[q];
  }
  const int np = u_exact->nparams;  // >= 1: field_check requires what the kind reads
  for (int k = 0; k < np; ++k) stage[NA_TABLE + k] = u_exact->params[k];
  cudaStream_t st = (cudaStream_t)stream;
  int cur = 0;
  cudaGetDevice(&cur);
  if (cudaSetDevice(device) != cudaSuccess) {
    g_na_err = "hdg_errornorm_l2sq_noalloc: cudaSetDevice(" + std::to_string(device) + ") failed";
    return HDG_ERR_CUDA;
  }
  cudaError_t e = cudaMemcpyAsync(scratch + NA_OFF_TABLE, stage, sizeof(double) * need, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(scratch + NA_OFF_PARAMS, stage + NA_TABLE, sizeof(double) * np, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(scratch + NA_OFF_TICKET, 0, sizeof(double), st);  // ticket starts at 0
  const int blocks = std::min(NA_BLOCKS, (ncells + 255) / 256);
  if (e == cudaSuccess) {
    switch (p) {
      case 1: k_errornorm_na<1><<<blocks, 256, 0, st>>>(ncells, cells, xy, u, nq, u_exact->kind, scratch); break;
      case 2: k_errornorm_na<2><<<blocks, 256, 0, st>>>(ncells, cells, xy, u, nq, u_exact->kind, scratch); break;
      case 3: k_errornorm_na<3><<<blocks, 256, 0, st>>>(ncells, cells, xy, u, nq, u_exact->kind, scratch); break;
      case 4: k_errornorm_na<4><<<blocks, 256, 0, st>>>(ncells, cells, xy, u, nq, u_exact->kind, scratch); break;
    }
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, scratch + NA_OFF_RESULT, sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaSetDevice(cur);
  if (e != cudaSuccess) {
    // forget the cached address: after a device reset the module reloads at another address,
    // and the next call looks it up again
    {
      std::lock_guard<std::mutex> lk(g_na_lock);
      g_na_ptr[device] = nullptr;
    }
    g_na_err = std::string("hdg_errornorm_l2sq_noalloc: ") + cudaGetErrorString(e);
    return HDG_ERR_CUDA;
  }
  g_na_err.clear();
  return HDG_OK;
}

}  // extern "C"
