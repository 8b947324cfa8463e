// Mesh construction on the host and its device mirror.
//
// rectangle_mesh (src/generate_mesh.jl:101-143) numbers faces "at first visit" through a
// Dict while it walks the quads row by row.  For the structured right-diagonal mesh that
// numbering has a closed form, used here instead of a hash table:
//   quad (i,j), 1-based, i fastest; faces created before it
//     base(i,j) = (j-1)(3nx+1) + [j>1] nx + 3(i-1) + [i>1] + [j=1](i-1)
//   lower cell (nodes a=n(i,j), b=n(i+1,j), c=n(i,j+1)) local faces (b,c),(c,a),(a,b):
//     diagonal D = base+1, left V = base+2 if i=1 (else the right face of quad i-1),
//     bottom H = base+2+[i=1] if j=1 (else the top face of quad (i,j-1))
//   upper cell (nodes b, d=n(i+1,j+1), c) local faces (d,c),(c,b),(b,d):
//     top = k+1, D, right = k+2 with k = base+1+[i=1]+[j=1].
// The face table rows [v1 v2 c1 c2] keep the vertex order of the creating cell, as the
// reference does.  Triangle-format meshes use the generic first-visit hash construction
// (src/triangle_mesh.jl:48-108).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <unordered_map>

#include "hdg_internal.h"

static const int EDGE_NODES[3][2] = {{1, 2}, {2, 0}, {0, 1}};  // src/shapes.jl:24 (0-based)

void mesh_build_rectangle(hdg_mesh* m, int nx, int ny, const double LL[2], const double UR[2]) {
  m->structured = true;
  m->nx = nx;
  m->ny = ny;
  m->LL[0] = LL[0]; m->LL[1] = LL[1]; m->UR[0] = UR[0]; m->UR[1] = UR[1];
  const int NX = nx + 1, NY = ny + 1;
  m->nn = NX * NY;
  m->nc = 2 * nx * ny;
  m->nf = nx + ny + 3 * nx * ny;
  // node grid, x fastest: the interpolation of _generate_2d_nodes! (src/generate_mesh.jl:1-18),
  // evaluated with the same operation order (this file is built without FMA contraction)
  const double LR[2] = {UR[0], LL[1]}, UL[2] = {LL[0], UR[1]};
  m->xy.resize(2 * (size_t)m->nn);
  for (int i = 0; i < NY; ++i) {
    double rb = (double)i / (double)(NY - 1);
    double x0 = LL[0] * (1 - rb) + rb * UL[0];
    double x1 = LR[0] * (1 - rb) + rb * UR[0];
    double y0 = LL[1] * (1 - rb) + rb * UL[1];
    double y1 = LR[1] * (1 - rb) + rb * UR[1];
    for (int j = 0; j < NX; ++j) {
      double r = (double)j / (double)(NX - 1);
      m->xy[2 * ((size_t)i * NX + j)] = x0 * (1 - r) + r * x1;
      m->xy[2 * ((size_t)i * NX + j) + 1] = y0 * (1 - r) + r * y1;
    }
  }
  m->cells.resize(3 * (size_t)m->nc);
  m->cfaces.resize(3 * (size_t)m->nc);
  m->faces.assign(4 * (size_t)m->nf, -1);
  auto node = [&](int i, int j) { return (i - 1) + (j - 1) * NX; };  // 0-based id of grid (i,j)
  auto base = [&](int i, int j) {
    return (int64_t)(j - 1) * (3 * nx + 1) + (j > 1 ? nx : 0) + 3 * (i - 1) + (i > 1 ? 1 : 0) + (j == 1 ? (i - 1) : 0);
  };
  auto kk = [&](int i, int j) { return base(i, j) + 1 + (i == 1) + (j == 1); };
  auto set_face = [&](int64_t f1, int v1, int v2, int c1) {  // f1 1-based
    int32_t* r = &m->faces[4 * (f1 - 1)];
    r[0] = v1; r[1] = v2; r[2] = c1;
  };
  auto set_c2 = [&](int64_t f1, int c2) { m->faces[4 * (f1 - 1) + 3] = c2; };
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      const int lo = 2 * ((j - 1) * nx + (i - 1)), up = lo + 1;  // 0-based cell ids
      const int a = node(i, j), b = node(i + 1, j), c = node(i, j + 1), d = node(i + 1, j + 1);
      const int64_t B = base(i, j), K = kk(i, j);
      const int64_t D = B + 1;
      const int64_t V = (i == 1) ? B + 2 : kk(i - 1, j) + 2;
      const int64_t H = (j == 1) ? B + 2 + (i == 1) : kk(i, j - 1) + 1;
      const int64_t T = K + 1, R = K + 2;
      // lower cell: nodes (a,b,c), faces (D, V, H)
      m->cells[3 * lo] = a; m->cells[3 * lo + 1] = b; m->cells[3 * lo + 2] = c;
      m->cfaces[3 * lo] = (int32_t)(D - 1); m->cfaces[3 * lo + 1] = (int32_t)(V - 1); m->cfaces[3 * lo + 2] = (int32_t)(H - 1);
      set_face(D, b, c, lo);
      if (i == 1) set_face(V, c, a, lo); else set_c2(V, lo);
      if (j == 1) set_face(H, a, b, lo); else set_c2(H, lo);
      // upper cell: nodes (b,d,c), faces (T, D, R)
      m->cells[3 * up] = b; m->cells[3 * up + 1] = d; m->cells[3 * up + 2] = c;
      m->cfaces[3 * up] = (int32_t)(T - 1); m->cfaces[3 * up + 1] = (int32_t)(D - 1); m->cfaces[3 * up + 2] = (int32_t)(R - 1);
      set_face(T, d, c, up);
      set_c2(D, up);
      set_face(R, b, d, up);
    }
  for (int f = 0; f < m->nf; ++f) {
    int32_t* r = &m->faces[4 * f];
    if (r[3] < 0) r[3] = -1;
  }
  // boundary sets by exact coordinate equality, src/generate_mesh.jl:60-89
  std::vector<int32_t> bottom, right, top, left, all;
  for (int f = 0; f < m->nf; ++f) {
    const int32_t* r = &m->faces[4 * f];
    if (r[3] >= 0) continue;
    const double* p = &m->xy[2 * r[0]];
    const double* q = &m->xy[2 * r[1]];
    if (p[1] == LL[1] && q[1] == LL[1]) bottom.push_back(f);
    else if (p[0] == UR[0] && q[0] == UR[0]) right.push_back(f);
    else if (p[1] == UR[1] && q[1] == UR[1]) top.push_back(f);
    else if (p[0] == LL[0] && q[0] == LL[0]) left.push_back(f);
    else throw HdgError{HDG_ERR_NOT_BOUNDARY, "Face " + std::to_string(f + 1) + " belongs to one cell but is not in boundary"};
    all.push_back(f);
  }
  m->facesets["bottom"] = bottom;
  m->facesets["right"] = right;
  m->facesets["top"] = top;
  m->facesets["left"] = left;
  m->facesets["boundary"] = all;
  m->single_problem();
}

namespace {
struct PairHash {
  size_t operator()(uint64_t k) const { return std::hash<uint64_t>()(k * 0x9E3779B97F4A7C15ull); }
};
}  // namespace

int mesh_build_from_cells(hdg_mesh* m, int nnodes, const double* xy, int ncells, const int32_t* cells1, int nedges,
                          const int32_t* edges1) {
  m->structured = false;
  m->nn = nnodes;
  m->nc = ncells;
  m->xy.assign(xy, xy + 2 * (size_t)nnodes);
  std::unordered_map<uint64_t, int32_t, PairHash> marker, dict;
  auto key = [](int a, int b) { return ((uint64_t)std::min(a, b) << 32) | (uint32_t)std::max(a, b); };
  for (int e = 0; e < nedges; ++e) {
    int a = edges1[3 * e] - 1, b = edges1[3 * e + 1] - 1;
    if (a < 0 || b < 0 || a >= nnodes || b >= nnodes) return HDG_ERR_ARG;
    marker.emplace(key(a, b), edges1[3 * e + 2]);  // first occurrence wins (parse_faces!)
  }
  m->cells.resize(3 * (size_t)ncells);
  m->cfaces.resize(3 * (size_t)ncells);
  m->faces.clear();
  std::vector<int32_t> bnd;
  for (int c = 0; c < ncells; ++c) {
    int n[3];
    for (int k = 0; k < 3; ++k) {
      n[k] = cells1[3 * c + k] - 1;
      if (n[k] < 0 || n[k] >= nnodes) return HDG_ERR_ARG;
    }
    // _check_node_data: swap nodes 2,3 of a clockwise cell (src/generate_mesh.jl:49-57)
    const double* p1 = &m->xy[2 * n[0]];
    const double* p2 = &m->xy[2 * n[1]];
    const double* p3 = &m->xy[2 * n[2]];
    double ax = p2[0] - p1[0], ay = p2[1] - p1[1], bx = p3[0] - p1[0], by = p3[1] - p1[1];
    if ((ax * by - ay * bx) < 0) std::swap(n[1], n[2]);
    for (int k = 0; k < 3; ++k) m->cells[3 * c + k] = n[k];
    for (int f = 0; f < 3; ++f) {
      int v1 = n[EDGE_NODES[f][0]], v2 = n[EDGE_NODES[f][1]];
      uint64_t kkey = key(v1, v2);
      auto it = dict.find(kkey);
      if (it != dict.end()) {
        m->cfaces[3 * c + f] = it->second;
        m->faces[4 * (size_t)it->second + 3] = c;
      } else {
        int32_t fid = (int32_t)(m->faces.size() / 4);
        m->faces.push_back(v1);
        m->faces.push_back(v2);
        m->faces.push_back(c);
        m->faces.push_back(-1);
        dict.emplace(kkey, fid);
        m->cfaces[3 * c + f] = fid;
        auto mk = marker.find(kkey);
        if (mk != marker.end() && mk->second > 0) bnd.push_back(fid);
      }
    }
  }
  m->nf = (int)(m->faces.size() / 4);
  std::sort(bnd.begin(), bnd.end());
  m->facesets["boundary"] = bnd;
  m->single_problem();
  return HDG_OK;
}

// Disjoint union of meshes (a batch of independent problems): node, cell and face ids of part P
// are shifted by the totals of parts 0..P-1, so each part keeps its own numbering order (and its
// face orientations, which depend only on the order of node ids); face sets are merged.
void mesh_concat(hdg_mesh* out, const std::vector<const hdg_mesh*>& parts) {
  out->structured = false;
  out->nn = out->nc = out->nf = 0;
  out->xy.clear(); out->cells.clear(); out->cfaces.clear(); out->faces.clear(); out->facesets.clear();
  out->nprob = 0;
  out->prob_node0 = {0};
  out->prob_cell0 = {0};
  out->prob_face0 = {0};
  for (const hdg_mesh* m : parts) {
    for (int P = 0; P < m->nprob; ++P) {  // a part may itself be a union
      out->prob_node0.push_back(out->nn + m->prob_node0[P + 1]);
      out->prob_cell0.push_back(out->nc + m->prob_cell0[P + 1]);
      out->prob_face0.push_back(out->nf + m->prob_face0[P + 1]);
    }
    out->nprob += m->nprob;
    out->xy.insert(out->xy.end(), m->xy.begin(), m->xy.end());
    for (int32_t v : m->cells) out->cells.push_back(v + out->nn);
    for (int32_t v : m->cfaces) out->cfaces.push_back(v + out->nf);
    for (int f = 0; f < m->nf; ++f) {
      const int32_t* r = &m->faces[4 * f];
      out->faces.push_back(r[0] + out->nn);
      out->faces.push_back(r[1] + out->nn);
      out->faces.push_back(r[2] + out->nc);
      out->faces.push_back(r[3] < 0 ? -1 : r[3] + out->nc);
    }
    for (const auto& kv : m->facesets) {
      auto& dst = out->facesets[kv.first];
      for (int32_t f : kv.second) dst.push_back(f + out->nf);
    }
    out->nn += m->nn;
    out->nc += m->nc;
    out->nf += m->nf;
  }
  for (auto& kv : out->facesets) std::sort(kv.second.begin(), kv.second.end());
}

void hdg_mesh::upload() {
  cudaStream_t s = ctx->stream;
  HDG_CUDA(cudaSetDevice(ctx->device));
  upload_coordinates();
  d_cells.upload(cells.data(), cells.size(), s);
  d_cfaces.upload(cfaces.data(), cfaces.size(), s);
  std::vector<uint8_t> orient(nc);
  for (int c = 0; c < nc; ++c) {
    uint8_t o = 0;
    for (int f = 0; f < 3; ++f)
      if (cells[3 * c + EDGE_NODES[f][1]] > cells[3 * c + EDGE_NODES[f][0]]) o |= (uint8_t)(1u << f);
    orient[c] = o;
  }
  d_orient.upload(orient.data(), orient.size(), s);
  std::vector<int32_t> fcell(2 * (size_t)nf);
  std::vector<int8_t> flf(2 * (size_t)nf, -1);
  for (int f = 0; f < nf; ++f) {
    for (int k = 0; k < 2; ++k) {
      int c = faces[4 * f + 2 + k];
      fcell[2 * f + k] = c;
      if (c >= 0)
        for (int l = 0; l < 3; ++l)
          if (cfaces[3 * c + l] == f) flf[2 * f + k] = (int8_t)l;
    }
  }
  d_fcell.upload(fcell.data(), fcell.size(), s);
  d_flf.upload(flf.data(), flf.size(), s);
  std::vector<int32_t> cp(nc);
  for (int P = 0; P < nprob; ++P)
    for (int c = prob_cell0[P]; c < prob_cell0[P + 1]; ++c) cp[c] = P;
  d_cell_prob.upload(cp.data(), cp.size(), s);
  HDG_CUDA(cudaStreamSynchronize(s));
}

void hdg_mesh::upload_coordinates() { d_xy.upload(xy.data(), xy.size(), ctx->stream); }
