// The reference's triplet assembler (src/assembler.jl:1-60) for user-written element loops:
// assemble!(a, edof, Ke) appends Ke column by column, end_assemble builds a CSC matrix with
// duplicates summed in the order they were appended.  Host-side API object; the HDG path itself
// uses the device gather of trace.cu instead.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "hdg_internal.h"

struct hdg_assembler {
  std::vector<int64_t> I, J;
  std::vector<double> V;
  int64_t nrows = 0, ncols = 0;
  std::vector<int64_t> colptr, rowval;
  std::vector<double> nzval;
  bool finished = false;
};

extern "C" {

int hdg_assembler_create(int64_t sizehint, hdg_assembler** out) {
  if (!out) return HDG_ERR_ARG;
  hdg_assembler* a = new hdg_assembler();
  if (sizehint > 0) {
    a->I.reserve(sizehint);
    a->J.reserve(sizehint);
    a->V.reserve(sizehint);
  }
  *out = a;
  return HDG_OK;
}

int hdg_assembler_add(hdg_assembler* a, int n, const int64_t* edof, const double* Ke) {
  if (!a || n < 0 || (n > 0 && (!edof || !Ke))) return HDG_ERR_ARG;
  for (int k = 0; k < n; ++k)
    if (edof[k] < 1) return HDG_ERR_ARG;
  a->finished = false;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      a->I.push_back(edof[i]);
      a->J.push_back(edof[j]);
      a->V.push_back(Ke[(size_t)j * n + i]);
    }
  return HDG_OK;
}

int hdg_assembler_finish(hdg_assembler* a, int64_t* nrows, int64_t* ncols, int64_t* nnz) {
  if (!a) return HDG_ERR_ARG;
  const size_t T = a->V.size();
  a->nrows = T ? *std::max_element(a->I.begin(), a->I.end()) : 0;
  a->ncols = T ? *std::max_element(a->J.begin(), a->J.end()) : 0;
  std::vector<int64_t> cnt(a->ncols + 1, 0);
  for (size_t t = 0; t < T; ++t) cnt[a->J[t]]++;
  std::vector<int64_t> start(a->ncols + 1, 0);
  for (int64_t c = 0; c < a->ncols; ++c) start[c + 1] = start[c] + cnt[c + 1];
  std::vector<int64_t> order(T);
  std::vector<int64_t> pos(start.begin(), start.end() - 1);
  for (size_t t = 0; t < T; ++t) order[pos[a->J[t] - 1]++] = (int64_t)t;
  a->colptr.assign(a->ncols + 1, 0);
  a->rowval.clear();
  a->nzval.clear();
  for (int64_t c = 0; c < a->ncols; ++c) {
    std::stable_sort(order.begin() + start[c], order.begin() + start[c + 1],
                     [&](int64_t x, int64_t y) { return a->I[x] < a->I[y]; });
    int64_t last = -1;
    for (int64_t k = start[c]; k < start[c + 1]; ++k) {
      const int64_t t = order[k];
      if (a->I[t] == last) {
        a->nzval.back() += a->V[t];
      } else {
        a->rowval.push_back(a->I[t] - 1);
        a->nzval.push_back(a->V[t]);
        last = a->I[t];
      }
    }
    a->colptr[c + 1] = (int64_t)a->rowval.size();
  }
  a->finished = true;
  if (nrows) *nrows = a->nrows;
  if (ncols) *ncols = a->ncols;
  if (nnz) *nnz = (int64_t)a->nzval.size();
  return HDG_OK;
}

int hdg_assembler_get_csc(const hdg_assembler* a, int base, int64_t* colptr, int64_t* rowval, double* nzval) {
  if (!a || !a->finished || (base != 0 && base != 1)) return HDG_ERR_ARG;
  if (colptr)
    for (size_t k = 0; k < a->colptr.size(); ++k) colptr[k] = a->colptr[k] + base;
  if (rowval)
    for (size_t k = 0; k < a->rowval.size(); ++k) rowval[k] = a->rowval[k] + base;
  if (nzval) std::memcpy(nzval, a->nzval.data(), a->nzval.size() * sizeof(double));
  return HDG_OK;
}

int hdg_assembler_destroy(hdg_assembler* a) {
  delete a;
  return HDG_OK;
}

}  // extern "C"
