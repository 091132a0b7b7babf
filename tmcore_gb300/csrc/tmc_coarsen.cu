// Coarse-graining of a fine-mesh state onto a coarser mesh (training data
// of the learned closure): area-weighted aggregation of cell values over the
// fine cells whose centres lie in each coarse Voronoi cell, and edge-flux
// averaging of the normal velocity (the fine normal fluxes u dvEdge across
// the boundary between two aggregates, divided by the coarse dvEdge); edge
// scalars (pv on edges) are dvEdge-weighted means over the same fine edges.
//
// The maps are built on the host (nearest coarse generator by a greedy walk
// over the coarse cellsOnCell graph, which ends at the nearest generator on a
// Voronoi mesh) and applied by gather kernels in CSR form.
#include <cuda_runtime.h>

#include <cmath>
#include <string>
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
};

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

// nearest coarse generator of each fine cell
std::vector<int> nearest_cells(const tmc_mesh_desc& f, const tmc_mesh_desc& c) {
  std::vector<int> map(f.nCells, 0);
  int g = 0;
  for (int i = 0; i < f.nCells; ++i) {
    const double px = f.xCell[i], py = f.yCell[i], pz = f.zCell[i];
    auto dot = [&](int k) { return px * c.xCell[k] + py * c.yCell[k] + pz * c.zCell[k]; };
    double best = dot(g);
    for (int it = 0; it < 4 * c.nCells; ++it) {
      int nb = -1;
      double nbv = best;
      const int n = c.nEdgesOnCell[g];
      for (int j = 0; j < n; ++j) {
        const int k = c.cellsOnCell[(size_t)g * c.maxEdges + j] - 1;
        if (k < 0) continue;
        const double v = dot(k);
        if (v > nbv) {
          nbv = v;
          nb = k;
        }
      }
      if (nb < 0) break;
      g = nb;
      best = nbv;
    }
    map[i] = g;
  }
  return map;
}

}  // namespace

extern "C" {

int tmc_coarsen_create(const tmc_mesh_desc* fine, const tmc_mesh_desc* coarse, int32_t device, tmc_coarsen** out) {
  if (!out || !fine || !coarse) return TMC_E_ARG;
  *out = nullptr;
  auto* C = new tmc_coarsen();
  *out = C;
  const tmc_mesh_desc &f = *fine, &c = *coarse;
  if (!f.xCell || !f.yCell || !f.zCell || !f.areaCell || !f.cellsOnEdge || !f.dvEdge || !c.xCell || !c.yCell ||
      !c.zCell || !c.nEdgesOnCell || !c.cellsOnCell || !c.edgesOnCell || !c.cellsOnEdge || !c.dvEdge) {
    C->err = "tmc_coarsen_create: missing mesh arrays";
    return TMC_E_ARG;
  }
  if (cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    C->err = "cudaSetDevice failed (no CUDA device?)";
    return TMC_E_CUDA;
  }
  C->ncf = f.nCells;
  C->nef = f.nEdges;
  C->ncc = c.nCells;
  C->nec = c.nEdges;
  C->cell_map = nearest_cells(f, c);
  const std::vector<int>& map = C->cell_map;
  // cells: area-weighted mean over the fine cells of each coarse cell
  Csr cc;
  {
    std::vector<double> asum(c.nCells, 0.0);
    std::vector<int> cnt(c.nCells, 0);
    for (int i = 0; i < f.nCells; ++i) {
      asum[map[i]] += f.areaCell[i];
      cnt[map[i]]++;
    }
    cc.start.assign(c.nCells + 1, 0);
    for (int k = 0; k < c.nCells; ++k) cc.start[k + 1] = cc.start[k] + cnt[k];
    cc.idx.resize(f.nCells);
    cc.w.resize(f.nCells);
    std::vector<int> fill(c.nCells, 0);
    for (int i = 0; i < f.nCells; ++i) {
      const int k = map[i], pos = cc.start[k] + fill[k]++;
      cc.idx[pos] = i;
      cc.w[pos] = f.areaCell[i] / asum[k];
    }
  }
  // edges: fine edges whose two cells fall in two neighbouring coarse cells
  Csr ce, cp;
  {
    std::vector<std::vector<std::pair<int, double>>> lu(c.nEdges), lp(c.nEdges);
    for (int e = 0; e < f.nEdges; ++e) {
      const int a = map[f.cellsOnEdge[(size_t)e * 2] - 1], b = map[f.cellsOnEdge[(size_t)e * 2 + 1] - 1];
      if (a == b) continue;
      int hit = -1;
      for (int j = 0; j < c.nEdgesOnCell[a]; ++j) {
        const int k = c.edgesOnCell[(size_t)a * c.maxEdges + j] - 1;
        const int k1 = c.cellsOnEdge[(size_t)k * 2] - 1, k2 = c.cellsOnEdge[(size_t)k * 2 + 1] - 1;
        if ((k1 == a && k2 == b) || (k1 == b && k2 == a)) {
          hit = k;
          break;
        }
      }
      if (hit < 0) continue;
      const double s = (c.cellsOnEdge[(size_t)hit * 2] - 1 == a) ? 1.0 : -1.0;
      lu[hit].push_back({e, s * f.dvEdge[e] / c.dvEdge[hit]});
      lp[hit].push_back({e, f.dvEdge[e]});
    }
    ce.start.assign(c.nEdges + 1, 0);
    cp.start.assign(c.nEdges + 1, 0);
    for (int k = 0; k < c.nEdges; ++k) {
      if (lu[k].empty()) C->unmatched++;
      ce.start[k + 1] = ce.start[k] + (int)lu[k].size();
      cp.start[k + 1] = cp.start[k] + (int)lp[k].size();
      double wsum = 0.0;
      for (auto& pr : lp[k]) wsum += pr.second;
      for (auto& pr : lu[k]) {
        ce.idx.push_back(pr.first);
        ce.w.push_back(pr.second);
      }
      for (auto& pr : lp[k]) {
        cp.idx.push_back(pr.first);
        cp.w.push_back(pr.second / wsum);
      }
    }
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
  if (!C || !C->c_w) return TMC_E_ARG;
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
  for (void* q : p) cudaFree(q);
  if (C->st) cudaStreamDestroy(C->st);
  delete C;
  return TMC_OK;
}

}  // extern "C"
