// Coarse-graining of a fine-mesh state onto a coarser mesh (training data
// and the truth of the learned closure's held-out comparison).
//
// Cells: area-weighted aggregation over kites.  Each fine cell is cut into
// its kites (cell centre, one vertex and the two half-edges between them;
// kiteAreasOnVertex), and each kite goes to the coarse cell whose generator
// is nearest the kite's centre point (the midpoint of the fine cell centre
// and the vertex).  A kite within a small tie band of two coarse generators
// (refined icosahedral meshes put many on coarse Voronoi boundaries) is split
// equally between them.  The coarse value is the kite-area-weighted mean.
//
// Edges: strip averaging of the fine velocity's component along the coarse
// normal.  For a coarse edge, the fine edges whose midpoints lie within
// 0.75 fine dcEdge of the coarse Voronoi edge's great circle, between its two
// vertices, each give the full velocity u n + v t (v the TRiSK tangential
// velocity, sum of weightsOnEdge u over edgesOnEdge) dotted with the coarse
// normal; the coarse u is their mean.  Edge scalars (pv on edges) are means
// over the same fine edges.  Both maps are linear and stored as CSR rows over
// the fine arrays; gather kernels apply them.
//
// The fine edges that can lie in a coarse edge's strip are found through the
// cell map (each fine cell's nearest coarse generator, by a greedy walk over
// the coarse cellsOnCell graph, which ends at the nearest generator on a
// Voronoi mesh): the fine edges touching either coarse cell's fine cells.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <utility>
#include <vector>

#include "tmcore_gpu.h"

namespace {

__global__ void k_gather_csr(int n, const int32_t* start, const int32_t* idx, const double* w, const double* src,
                             double* dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int k = start[i]; k < start[i + 1]; ++k) s += w[k] * src[idx[k]];
  dst[i] = s;
}

struct Csr {
  std::vector<int32_t> start, idx;
  std::vector<double> w;
  // append one row from (column, weight) pairs, merging repeated columns
  void add_row(std::vector<std::pair<int, double>>& row) {
    if (start.empty()) start.push_back(0);
    std::sort(row.begin(), row.end(), [](const std::pair<int, double>& a, const std::pair<int, double>& b) {
      return a.first < b.first;
    });
    for (size_t i = 0; i < row.size();) {
      double s = 0.0;
      size_t j = i;
      for (; j < row.size() && row[j].first == row[i].first; ++j) s += row[j].second;
      idx.push_back(row[i].first);
      w.push_back(s);
      i = j;
    }
    start.push_back((int32_t)idx.size());
  }
};

struct V3 {
  double x, y, z;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline V3 unit(V3 a) { return (1.0 / std::sqrt(dot(a, a))) * a; }

inline V3 cell_pt(const tmc_mesh_desc& m, int i) { return unit({m.xCell[i], m.yCell[i], m.zCell[i]}); }
inline V3 edge_pt(const tmc_mesh_desc& m, int e) { return unit({m.xEdge[e], m.yEdge[e], m.zEdge[e]}); }
inline V3 vert_pt(const tmc_mesh_desc& m, int v) { return unit({m.xVertex[v], m.yVertex[v], m.zVertex[v]}); }

// unit normal of edge e (from cellsOnEdge 1 to 2) in the tangent plane at the edge
V3 edge_normal(const tmc_mesh_desc& m, int e) {
  const V3 r = edge_pt(m, e);
  V3 d = cell_pt(m, m.cellsOnEdge[(size_t)e * 2 + 1] - 1) - cell_pt(m, m.cellsOnEdge[(size_t)e * 2] - 1);
  d = d - dot(d, r) * r;
  return unit(d);
}

// nearest coarse generator of the unit vector p, by a greedy walk from g
int walk_nearest(const tmc_mesh_desc& c, const V3& p, int g) {
  double best = dot(p, cell_pt(c, g));
  for (int it = 0; it < 4 * c.nCells; ++it) {
    int nb = -1;
    double nbv = best;
    for (int j = 0; j < c.nEdgesOnCell[g]; ++j) {
      const int k = c.cellsOnCell[(size_t)g * c.maxEdges + j] - 1;
      if (k < 0) continue;
      const double v = dot(p, cell_pt(c, k));
      if (v > nbv) {
        nbv = v;
        nb = k;
      }
    }
    if (nb < 0) break;
    g = nb;
    best = nbv;
  }
  return g;
}

constexpr double kTieBand = 0.1;     // kites within 0.1 fine dcEdge of two generators are split
constexpr double kStripHalf = 0.75;  // strip half-width in fine dcEdge

}  // namespace

struct tmc_coarsen {
  int ncf = 0, nef = 0, ncc = 0, nec = 0;
  long long unmatched = 0;
  std::vector<int> cell_map;  // fine cell -> coarse cell (0-based)
  cudaStream_t st = nullptr;
  int32_t *c_start = nullptr, *c_idx = nullptr, *e_start = nullptr, *e_idx = nullptr, *p_start = nullptr,
          *p_idx = nullptr;
  double *c_w = nullptr, *e_w = nullptr, *p_w = nullptr;
  double *fin = nullptr, *fout = nullptr;
  Csr host[3];  // cells, u, edge scalars
  std::string err;
};

namespace {

template <class X>
X* upload(const std::vector<X>& v) {
  X* d = nullptr;
  if (cudaMalloc(&d, sizeof(X) * (v.empty() ? 1 : v.size())) != cudaSuccess) return nullptr;
  if (!v.empty()) cudaMemcpy(d, v.data(), sizeof(X) * v.size(), cudaMemcpyHostToDevice);
  return d;
}

// kite-area-weighted cell aggregation
Csr cell_rows(const tmc_mesh_desc& f, const tmc_mesh_desc& c, const std::vector<int>& map, double R) {
  std::vector<std::vector<std::pair<int, double>>> rows(c.nCells);
  const int deg = f.vertexDegree;
  for (int v = 0; v < f.nVertices; ++v) {
    const V3 pv = vert_pt(f, v);
    for (int j = 0; j < deg; ++j) {
      const int i = f.cellsOnVertex[(size_t)v * deg + j] - 1;
      if (i < 0) continue;
      const double a = f.kiteAreasOnVertex[(size_t)v * deg + j];
      const V3 p = unit(cell_pt(f, i) + pv);
      const int g = walk_nearest(c, p, map[i]);
      // the nearest neighbouring generator, for the tie band
      const double ag = std::acos(std::min(1.0, dot(p, cell_pt(c, g))));
      int g2 = -1;
      double a2 = 1e300;
      for (int q = 0; q < c.nEdgesOnCell[g]; ++q) {
        const int k = c.cellsOnCell[(size_t)g * c.maxEdges + q] - 1;
        if (k < 0) continue;
        const double ak = std::acos(std::min(1.0, dot(p, cell_pt(c, k))));
        if (ak < a2) {
          a2 = ak;
          g2 = k;
        }
      }
      int ce = -1;  // the fine edge between this kite's cell and the next, for its dcEdge
      for (int q = 0; q < f.nEdgesOnCell[i] && ce < 0; ++q) {
        const int e = f.edgesOnCell[(size_t)i * f.maxEdges + q] - 1;
        if (e >= 0 && (f.verticesOnEdge[(size_t)e * 2] - 1 == v || f.verticesOnEdge[(size_t)e * 2 + 1] - 1 == v))
          ce = e;
      }
      const double band = kTieBand * (ce >= 0 ? f.dcEdge[ce] / R : 0.0);
      if (g2 >= 0 && a2 - ag <= band) {
        rows[g].push_back({i, 0.5 * a});
        rows[g2].push_back({i, 0.5 * a});
      } else {
        rows[g].push_back({i, a});
      }
    }
  }
  Csr out;
  for (auto& r : rows) {
    double s = 0.0;
    for (auto& pr : r) s += pr.second;
    for (auto& pr : r) pr.second /= s;
    out.add_row(r);
  }
  return out;
}

// strip averaging of the velocity's component along each coarse normal (ce),
// and the plain mean over the same fine edges (cp)
long long edge_rows(const tmc_mesh_desc& f, const tmc_mesh_desc& c, const std::vector<int>& map, double R, Csr& ce,
                    Csr& cp) {
  std::vector<std::vector<int>> by_cell(c.nCells);  // fine edges touching each aggregate
  for (int e = 0; e < f.nEdges; ++e) {
    const int a = map[f.cellsOnEdge[(size_t)e * 2] - 1];
    const int b = f.cellsOnEdge[(size_t)e * 2 + 1] > 0 ? map[f.cellsOnEdge[(size_t)e * 2 + 1] - 1] : a;
    by_cell[a].push_back(e);
    if (b != a) by_cell[b].push_back(e);
  }
  std::vector<V3> nf(f.nEdges), tf(f.nEdges), xf(f.nEdges);
  for (int e = 0; e < f.nEdges; ++e) {
    xf[e] = edge_pt(f, e);
    nf[e] = edge_normal(f, e);
    tf[e] = cross(xf[e], nf[e]);
  }
  std::vector<int> stamp(f.nEdges, -1);
  long long unmatched = 0;
  std::vector<std::pair<int, double>> ru, rp;
  std::vector<int> sel;
  for (int k = 0; k < c.nEdges; ++k) {
    const int A = c.cellsOnEdge[(size_t)k * 2] - 1, B = c.cellsOnEdge[(size_t)k * 2 + 1] - 1;
    const V3 P = vert_pt(c, c.verticesOnEdge[(size_t)k * 2] - 1), Q = vert_pt(c, c.verticesOnEdge[(size_t)k * 2 + 1] - 1);
    const V3 gc = unit(cross(P, Q));
    const double arc = std::atan2(std::sqrt(dot(cross(P, Q), cross(P, Q))), dot(P, Q));
    const V3 nk = edge_normal(c, k);
    sel.clear();
    for (double widen = 1.0; sel.empty() && widen <= 4.0; widen *= 2.0) {
      for (int side = 0; side < 2; ++side) {
        const int agg = side == 0 ? A : B;
        if (agg < 0) continue;
        for (int e : by_cell[agg]) {
          if (stamp[e] == k * 4 + (int)widen) continue;
          stamp[e] = k * 4 + (int)widen;
          const V3& X = xf[e];
          if (std::fabs(dot(X, gc)) >= kStripHalf * widen * f.dcEdge[e] / R) continue;
          const double s = std::atan2(dot(cross(P, X), gc), dot(P, X)) / arc;
          if (s < 0.0 || s > 1.0) continue;
          sel.push_back(e);
        }
      }
    }
    ru.clear();
    rp.clear();
    if (sel.empty()) {
      ++unmatched;
    } else {
      const double inv = 1.0 / (double)sel.size();
      for (int e : sel) {
        ru.push_back({e, inv * dot(nf[e], nk)});
        const double wt = inv * dot(tf[e], nk);
        for (int j = 0; j < f.nEdgesOnEdge[e]; ++j) {
          const int e2 = f.edgesOnEdge[(size_t)e * f.maxEdges2 + j] - 1;
          if (e2 >= 0) ru.push_back({e2, wt * f.weightsOnEdge[(size_t)e * f.maxEdges2 + j]});
        }
        rp.push_back({e, inv});
      }
    }
    ce.add_row(ru);
    cp.add_row(rp);
  }
  return unmatched;
}

}  // namespace

extern "C" {

int tmc_coarsen_create(const tmc_mesh_desc* fine, const tmc_mesh_desc* coarse, int32_t device, tmc_coarsen** out) {
  if (!out || !fine || !coarse) return TMC_E_ARG;
  *out = nullptr;
  auto* C = new tmc_coarsen();
  *out = C;
  const tmc_mesh_desc &f = *fine, &c = *coarse;
  if (!f.xCell || !f.yCell || !f.zCell || !f.cellsOnEdge || !f.dcEdge || !f.xEdge || !f.yEdge || !f.zEdge ||
      !f.xVertex || !f.yVertex || !f.zVertex || !f.cellsOnVertex || !f.kiteAreasOnVertex || !f.nEdgesOnCell ||
      !f.edgesOnCell || !f.verticesOnEdge || !f.nEdgesOnEdge || !f.edgesOnEdge || !f.weightsOnEdge || !c.xCell ||
      !c.yCell || !c.zCell || !c.xVertex || !c.yVertex || !c.zVertex || !c.xEdge || !c.yEdge || !c.zEdge ||
      !c.nEdgesOnCell || !c.cellsOnCell || !c.cellsOnEdge || !c.verticesOnEdge) {
    C->err = "tmc_coarsen_create: missing mesh arrays";
    return TMC_E_ARG;
  }
  C->ncf = f.nCells;
  C->nef = f.nEdges;
  C->ncc = c.nCells;
  C->nec = c.nEdges;
  const double R = std::sqrt(f.xCell[0] * f.xCell[0] + f.yCell[0] * f.yCell[0] + f.zCell[0] * f.zCell[0]);
  std::vector<int>& map = C->cell_map;
  map.assign(f.nCells, 0);
  for (int i = 0, g = 0; i < f.nCells; ++i) g = map[i] = walk_nearest(c, cell_pt(f, i), g);
  const Csr cc = cell_rows(f, c, map, R);
  Csr ce, cp;
  C->unmatched = edge_rows(f, c, map, R, ce, cp);
  C->host[0] = cc;
  C->host[1] = ce;
  C->host[2] = cp;
  if (device < 0) return TMC_OK;  // maps only
  if (cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    C->err = "cudaSetDevice failed (no CUDA device?)";
    return TMC_E_CUDA;
  }
  cudaStreamCreateWithFlags(&C->st, cudaStreamNonBlocking);
  C->c_start = upload(cc.start);
  C->c_idx = upload(cc.idx);
  C->c_w = upload(cc.w);
  C->e_start = upload(ce.start);
  C->e_idx = upload(ce.idx);
  C->e_w = upload(ce.w);
  C->p_start = upload(cp.start);
  C->p_idx = upload(cp.idx);
  C->p_w = upload(cp.w);
  const size_t nmax = std::max(std::max(f.nCells, f.nEdges), std::max(c.nCells, c.nEdges));
  if (cudaMalloc(&C->fin, sizeof(double) * nmax) != cudaSuccess ||
      cudaMalloc(&C->fout, sizeof(double) * nmax) != cudaSuccess || !C->p_w) {
    C->err = std::string("tmc_coarsen_create: ") + cudaGetErrorString(cudaGetLastError());
    return TMC_E_CUDA;
  }
  return TMC_OK;
}

static int coarsen_one(tmc_coarsen* C, const double* src, int nsrc, double* dst, int ndst, const int32_t* start,
                       const int32_t* idx, const double* w) {
  cudaMemcpyAsync(C->fin, src, sizeof(double) * nsrc, cudaMemcpyHostToDevice, C->st);
  k_gather_csr<<<(ndst + 255) / 256, 256, 0, C->st>>>(ndst, start, idx, w, C->fin, C->fout);
  cudaMemcpyAsync(dst, C->fout, sizeof(double) * ndst, cudaMemcpyDeviceToHost, C->st);
  if (cudaStreamSynchronize(C->st) != cudaSuccess) {
    C->err = std::string("tmc_coarsen_apply: ") + cudaGetErrorString(cudaGetLastError());
    return TMC_E_CUDA;
  }
  return TMC_OK;
}

int tmc_coarsen_apply(tmc_coarsen* C, const double* fine_gd, const double* fine_u, const double* fine_pv_edge,
                      double* coarse_gd, double* coarse_u, double* coarse_pv_edge) {
  if (!C) return TMC_E_ARG;
  if (!C->c_w) {
    C->err = "tmc_coarsen_apply: a coarsener created with device < 0 holds the maps only";
    return TMC_E_UNSUP;
  }
  int rc;
  if (fine_gd && coarse_gd &&
      (rc = coarsen_one(C, fine_gd, C->ncf, coarse_gd, C->ncc, C->c_start, C->c_idx, C->c_w)))
    return rc;
  if (fine_u && coarse_u && (rc = coarsen_one(C, fine_u, C->nef, coarse_u, C->nec, C->e_start, C->e_idx, C->e_w)))
    return rc;
  if (fine_pv_edge && coarse_pv_edge &&
      (rc = coarsen_one(C, fine_pv_edge, C->nef, coarse_pv_edge, C->nec, C->p_start, C->p_idx, C->p_w)))
    return rc;
  return TMC_OK;
}

int tmc_coarsen_rows(const tmc_coarsen* C, int32_t which, int64_t* nnz, int32_t* start, int32_t* idx, double* w) {
  if (!C || !nnz || which < 0 || which > 2) return TMC_E_ARG;
  const Csr& r = C->host[which];
  *nnz = (int64_t)r.idx.size();
  if (start) std::copy(r.start.begin(), r.start.end(), start);
  if (idx) std::copy(r.idx.begin(), r.idx.end(), idx);
  if (w) std::copy(r.w.begin(), r.w.end(), w);
  return TMC_OK;
}

int tmc_coarsen_unmatched(const tmc_coarsen* C, int64_t* edges) {
  if (!C || !edges) return TMC_E_ARG;
  *edges = C->unmatched;
  return TMC_OK;
}

int tmc_coarsen_cell_map(const tmc_coarsen* C, int32_t* coarse_cell_of_fine) {
  if (!C || !coarse_cell_of_fine) return TMC_E_ARG;
  for (int i = 0; i < C->ncf; ++i) coarse_cell_of_fine[i] = C->cell_map[i] + 1;
  return TMC_OK;
}

const char* tmc_coarsen_last_error(const tmc_coarsen* C) { return C ? C->err.c_str() : "null coarsener"; }

int tmc_coarsen_destroy(tmc_coarsen* C) {
  if (!C) return TMC_OK;
  if (C->st) cudaStreamSynchronize(C->st);
  void* p[] = {C->c_start, C->c_idx, C->c_w, C->e_start, C->e_idx, C->e_w, C->p_start, C->p_idx, C->p_w, C->fin, C->fout};
  for (void* q : p)
    if (q) cudaFree(q);
  if (C->st) cudaStreamDestroy(C->st);
  delete C;
  return TMC_OK;
}

}  // extern "C"
