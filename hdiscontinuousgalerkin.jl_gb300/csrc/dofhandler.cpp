// DofHandler, sparsity pattern and the in-place sparsity-pattern assembler (host code).
//
//  * hdg_dofhandler_create: DofHandler(fields, mesh) and _distribute_dofs of
//    src/dofhandler.jl:13-16,91-151.  Cells are visited in order; for each field, vertex dofs then
//    face dofs are taken from the first cell that reaches the entity (first-visit numbering, keyed
//    by node id and face id), cell dofs are always new.  On a revisit the reference reuses one dof
//    per component of the entity (src/dofhandler.jl:118-122, the dof stored for the entity is the
//    last one distributed to it); that behaviour is kept, so entities carrying more than one dof
//    per component (Lagrange order >= 3 faces) reproduce the reference's numbering as it is.
//  * hdg_dofhandler_sparsity: _create_sparsity_pattern of src/dofhandler.jl:189-229: all (i, j)
//    pairs of every cell's dofs (upper triangle only when symmetric) plus the diagonal, as CSC
//    with duplicates merged (stored values are zero).
//  * hdg_dofhandler_dirichlet: Dirichlet(u, dh, faceset, f) of src/boundary.jl:44-95 for nodal
//    fields: per boundary face of the set, its two vertex dofs then its face dofs, first visit
//    only, sorted at the end.  The local index of each dof in its cell is returned so that the
//    caller evaluates f at the nodal point.
//  * hdg_csc_assemble: assemble!(A::AssemblerSparsityPattern, dofs, Ke, fe) of
//    src/assembler.jl:97-137: K.nzval[r] += Ke[i, j] for every stored (dofs[i], dofs[j]) found
//    in column dofs[j], rows located by a walk of the sorted element dofs against the sorted
//    column; a missing row is an error.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <unordered_map>

#include "hdg_internal.h"

struct hdg_dofhandler {
  const hdg_mesh* mesh = nullptr;
  int nfields = 0;
  std::vector<int> vdofs, fdofs, cdofs, ncomp;  // per field: per vertex, per face, per cell, components
  std::vector<int32_t> cell_dofs;               // 1-based, concatenated
  std::vector<int32_t> offset;                  // 1-based, ncells + 1
  int ndofs = 0;
};

namespace {

int field_local_size(const hdg_dofhandler* d, int f) {
  return (3 * d->vdofs[f] + 3 * d->fdofs[f] + d->cdofs[f]) * d->ncomp[f];
}

int field_offset(const hdg_dofhandler* d, int f) {
  int o = 0;
  for (int i = 0; i < f; ++i) o += field_local_size(d, i);
  return o;
}

void distribute(hdg_dofhandler* d) {
  const hdg_mesh* m = d->mesh;
  std::vector<std::unordered_map<int32_t, int32_t>> vdict(d->nfields), fdict(d->nfields);
  int32_t next = 1;
  d->offset.assign(1, 1);
  d->cell_dofs.clear();
  for (int c = 0; c < m->nc; ++c) {
    for (int fi = 0; fi < d->nfields; ++fi) {
      const int nc_ = d->ncomp[fi];
      for (int kind = 0; kind < 2; ++kind) {  // 0 vertices, 1 faces
        const int per = kind == 0 ? d->vdofs[fi] : d->fdofs[fi];
        if (per <= 0) continue;
        auto& dict = kind == 0 ? vdict[fi] : fdict[fi];
        for (int k = 0; k < 3; ++k) {
          const int32_t ent = kind == 0 ? m->cells[3 * c + k] : m->cfaces[3 * c + k];
          auto it = dict.find(ent);
          if (it != dict.end()) {
            for (int comp = 0; comp < nc_; ++comp) d->cell_dofs.push_back(it->second + comp);
          } else {
            for (int e = 0; e < per; ++e) {
              dict[ent] = next;
              for (int comp = 0; comp < nc_; ++comp) d->cell_dofs.push_back(next++);
            }
          }
        }
      }
      for (int e = 0; e < d->cdofs[fi]; ++e)
        for (int comp = 0; comp < nc_; ++comp) d->cell_dofs.push_back(next++);
    }
    d->offset.push_back((int32_t)d->cell_dofs.size() + 1);
  }
  d->ndofs = d->cell_dofs.empty() ? 0 : *std::max_element(d->cell_dofs.begin(), d->cell_dofs.end());
}

thread_local std::string g_dh_err;

}  // namespace

extern "C" {

const char* hdg_dofhandler_last_error(void) { return g_dh_err.c_str(); }

int hdg_dofhandler_create(const hdg_mesh* mesh, int nfields, const int* vdofs, const int* fdofs, const int* cdofs,
                          const int* ncomp, hdg_dofhandler** out) {
  if (!mesh || nfields < 1 || !vdofs || !fdofs || !cdofs || !ncomp || !out) return HDG_ERR_ARG;
  try {
    auto* d = new hdg_dofhandler();
    d->mesh = mesh;
    d->nfields = nfields;
    d->vdofs.assign(vdofs, vdofs + nfields);
    d->fdofs.assign(fdofs, fdofs + nfields);
    d->cdofs.assign(cdofs, cdofs + nfields);
    d->ncomp.assign(ncomp, ncomp + nfields);
    for (int i = 0; i < nfields; ++i)
      if (vdofs[i] < 0 || fdofs[i] < 0 || cdofs[i] < 0 || ncomp[i] < 1 || vdofs[i] > 1) {
        delete d;
        g_dh_err = "hdg_dofhandler_create: bad field topology (at most one dof per vertex)";
        return HDG_ERR_ARG;
      }
    distribute(d);
    *out = d;
    return HDG_OK;
  } catch (const std::bad_alloc&) {
    g_dh_err = "hdg_dofhandler_create: out of host memory";
    return HDG_ERR_OOM;
  }
}

int hdg_dofhandler_sizes(const hdg_dofhandler* d, int* ndofs, int64_t* ncelldofs) {
  if (!d) return HDG_ERR_ARG;
  if (ndofs) *ndofs = d->ndofs;
  if (ncelldofs) *ncelldofs = (int64_t)d->cell_dofs.size();
  return HDG_OK;
}

int hdg_dofhandler_cell_dofs(const hdg_dofhandler* d, int32_t* cell_dofs, int32_t* offsets) {
  if (!d) return HDG_ERR_ARG;
  if (cell_dofs) std::memcpy(cell_dofs, d->cell_dofs.data(), d->cell_dofs.size() * sizeof(int32_t));
  if (offsets) std::memcpy(offsets, d->offset.data(), d->offset.size() * sizeof(int32_t));
  return HDG_OK;
}

int hdg_dofhandler_field_range(const hdg_dofhandler* d, int field, int* first, int* last) {
  if (!d || field < 0 || field >= d->nfields || !first || !last) return HDG_ERR_ARG;
  const int o = field_offset(d, field);
  *first = o + 1;
  *last = o + field_local_size(d, field);
  return HDG_OK;
}

int hdg_dofhandler_sparsity(const hdg_dofhandler* d, int symmetric, int base, int64_t* colptr, int64_t* rowval,
                            int64_t* nnz) {
  if (!d || !nnz || (base != 0 && base != 1)) return HDG_ERR_ARG;
  try {
    const int n = d->ndofs;
    // per column: the rows that appear with it in some cell (and the diagonal)
    std::vector<std::vector<int32_t>> cols((size_t)n);
    for (int c = 0; c + 1 < (int)d->offset.size(); ++c) {
      const int32_t* g = d->cell_dofs.data() + (d->offset[c] - 1);
      const int k = d->offset[c + 1] - d->offset[c];
      for (int j = 0; j < k; ++j)
        for (int i = 0; i < k; ++i) {
          if (symmetric && g[i] > g[j]) continue;
          cols[g[j] - 1].push_back(g[i]);
        }
    }
    int64_t total = 0;
    for (int j = 0; j < n; ++j) {
      auto& v = cols[j];
      v.push_back(j + 1);
      std::sort(v.begin(), v.end());
      v.erase(std::unique(v.begin(), v.end()), v.end());
      total += (int64_t)v.size();
    }
    *nnz = total;
    if (!colptr || !rowval) return HDG_OK;
    int64_t k = 0;
    for (int j = 0; j < n; ++j) {
      colptr[j] = k + base;
      for (int32_t r : cols[j]) rowval[k++] = r - 1 + base;
    }
    colptr[n] = k + base;
    return HDG_OK;
  } catch (const std::bad_alloc&) {
    g_dh_err = "hdg_dofhandler_sparsity: out of host memory";
    return HDG_ERR_OOM;
  }
}

int hdg_dofhandler_dirichlet(const hdg_dofhandler* d, const char* faceset, int field, int32_t* dofs, int32_t* cells,
                             int32_t* local, int* count) {
  if (!d || !faceset || !count || field < 0 || field >= d->nfields) return HDG_ERR_ARG;
  const hdg_mesh* m = d->mesh;
  auto it = m->facesets.find(faceset);
  if (it == m->facesets.end()) {
    g_dh_err = std::string("no face set ") + faceset;
    return HDG_ERR_UNKNOWN_SET;
  }
  std::vector<char> is_set((size_t)m->nf, 0);
  for (int32_t f : it->second) is_set[f] = 1;
  static const int EDGE_NODES[3][2] = {{1, 2}, {2, 0}, {0, 1}};  // (2,3),(3,1),(1,2), 0-based
  const int nvd = 3 * d->vdofs[field];  // vertex dofs of the field in a cell (one component)
  std::vector<int32_t> pd, pc, pl;
  std::vector<char> seen((size_t)d->ndofs + 1, 0);
  for (int f = 0; f < m->nf; ++f) {
    if (!is_set[f]) continue;
    if (m->faces[4 * f + 3] >= 0) {
      g_dh_err = "Face " + std::to_string(f + 1) + " is not in boundary";
      return HDG_ERR_NOT_BOUNDARY;
    }
    const int c = m->faces[4 * f + 2];
    int lf = 0;
    while (lf < 3 && m->cfaces[3 * c + lf] != f) ++lf;
    const int off = d->offset[c] - 1 + field_offset(d, field);
    auto add = [&](int loc) {  // loc: 0-based local dof index within the field
      const int32_t g = d->cell_dofs[off + loc];
      if (seen[g]) return;
      seen[g] = 1;
      pd.push_back(g);
      pc.push_back(c + 1);
      pl.push_back(loc + 1);
    };
    if (d->vdofs[field] > 0)
      for (int j = 0; j < 2; ++j) add(EDGE_NODES[lf][j]);
    for (int j = 0; j < d->fdofs[field]; ++j) add(nvd + d->fdofs[field] * lf + j);
  }
  std::vector<int> perm(pd.size());
  std::iota(perm.begin(), perm.end(), 0);
  std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return pd[a] < pd[b]; });
  *count = (int)pd.size();
  for (size_t k = 0; k < perm.size(); ++k) {
    if (dofs) dofs[k] = pd[perm[k]];
    if (cells) cells[k] = pc[perm[k]];
    if (local) local[k] = pl[perm[k]];
  }
  return HDG_OK;
}

int hdg_dofhandler_destroy(hdg_dofhandler* d) {
  delete d;
  return HDG_OK;
}

int hdg_csc_assemble(int64_t n, const int64_t* colptr, const int64_t* rowval, int base, double* nzval, double* f,
                     int upper_only, int nel, int ndofs_e, const int64_t* dofs, const double* Ke, const double* fe) {
  if (n < 0 || !colptr || !rowval || !nzval || nel < 0 || ndofs_e < 1 || !dofs || !Ke || (base != 0 && base != 1))
    return HDG_ERR_ARG;
  std::vector<int> perm((size_t)ndofs_e);
  std::vector<int64_t> sorted((size_t)ndofs_e);
  for (int e = 0; e < nel; ++e) {
    const int64_t* dof = dofs + (size_t)e * ndofs_e;
    const double* K = Ke + (size_t)e * ndofs_e * ndofs_e;  // column-major (Julia order)
    for (int i = 0; i < ndofs_e; ++i)
      if (dof[i] < 1 || dof[i] > n) {
        g_dh_err = "hdg_csc_assemble: dof out of range";
        return HDG_ERR_ARG;
      }
    if (f && fe)
      for (int i = 0; i < ndofs_e; ++i) f[dof[i] - 1] += fe[(size_t)e * ndofs_e + i];
    std::iota(perm.begin(), perm.end(), 0);
    std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return dof[a] < dof[b]; });
    for (int i = 0; i < ndofs_e; ++i) sorted[i] = dof[perm[i]];
    for (int cc = 0; cc < ndofs_e; ++cc) {
      const int64_t col = sorted[cc];
      const int maxlook = upper_only ? cc + 1 : ndofs_e;
      int cur = 0;
      for (int64_t r = colptr[col - 1] - base; r < colptr[col] - base && cur < maxlook; ++r) {
        const int krow = perm[cur];
        if (rowval[r] - base + 1 == dof[krow]) {
          nzval[r] += K[(size_t)perm[cc] * ndofs_e + krow];
          ++cur;
        }
      }
      if (cur < maxlook) {
        g_dh_err = "some row indices were not found";
        return HDG_ERR_ARG;
      }
    }
  }
  return HDG_OK;
}

}  // extern "C"
