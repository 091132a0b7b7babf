// Host-side mesh preparation for the device: the derivations of TMCORE's
// mesh_init (src/core/mesh_mod.F90:169-224), the least-squares stencil tables
// of poly_fit_run (src/utils/poly_fit_mod.F90:119-609), space-filling-curve
// renumbering and the structure-of-arrays device layout.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "tmcore_gpu.h"

namespace tmc {

constexpr int kMaxFit = 30;         // poly_fit_mod.F90:33 maxFitCells
constexpr int kFitLd = kMaxFit + 1;  // fit arrays are (0:30, n)

// One upwind stencil family compacted for the device: for edge e and side s
// (s = 0 for cellsOnEdge/verticesOnEdge(1,e), 1 for (2,e)) the centre is the
// side's cell/vertex, and the stencil is fit(1:n-1, centre) with weights
// deriv(1:n-1, s+1, e).  Slot-major: idx[(j*2+s)*ne + e].
struct Stencil {
  int width = 0;
  std::vector<uint8_t> count;  // [2][ne]
  std::vector<int32_t> idx;    // [width][2][ne], new numbering
  std::vector<double> w;       // [width][2][ne]
};

struct HostMesh {
  int nc = 0, ne = 0, nv = 0, me = 0, me2 = 0, vd = 0;
  double radius = 0, totalArea = 0, sumAreaTriangle = 0;
  // permutations: new index -> original (file) index, 0-based, and inverse
  std::vector<int32_t> cell_n2o, edge_n2o, vert_n2o, cell_o2n, edge_o2n, vert_o2n;

  // cells (new numbering, slot-major [slot][nc])
  std::vector<uint8_t> nEdgesOnCell;
  std::vector<int32_t> edgesOnCell;
  std::vector<int32_t> cellsOnCell;  // the other cell of edgesOnCell(i), derived from cellsOnEdge
  std::vector<int8_t> nSignEdge;
  std::vector<double> areaCell;
  // edges
  std::vector<int32_t> cellsOnEdge, verticesOnEdge;  // [2][ne]
  std::vector<uint8_t> nEdgesOnEdge;
  std::vector<int32_t> edgesOnEdge;   // [me2][ne]
  std::vector<double> weightsOnEdge;  // [me2][ne]
  std::vector<double> dcEdge, dvEdge, areaEdge;
  // vertices
  std::vector<int32_t> cellsOnVertex, edgesOnVertex;  // [vd][nv]
  std::vector<int8_t> tSignEdge;
  std::vector<double> kite;  // [vd][nv]
  std::vector<double> areaTriangle, fVertex;
  std::vector<double> latVertex, lonVertex;  // radians (lonVertex empty when not given)
  // vector reconstruction to cell centres (mpas_init_reconstruct): coefficients
  // [3][me][nc] (x, y, z per edge slot) and cos/sin of lat and lon [4][nc]
  // (empty when lonCell is not given)
  std::vector<double> recon, cell_trig;
  // v2c gather table (scalar_v2c_interp_operator, operators_mod.F90:125-141):
  // per cell, contributions in ascending ORIGINAL vertex order.
  std::vector<int32_t> v2c_start, v2c_vertex;
  std::vector<double> v2c_kite;
  // upwind stencils
  Stencil cell2, cell3, cell4, vert2, vert4;

  std::string err;
};

struct PrepOptions {
  int renumber = 1;  // element order: 0 as given, 1 Hilbert curve, 2 Morton curve
  bool cell_fit = false;    // deriv2/3/4OnCell tables
  int min_me = 0;           // pad the per-cell slot arrays to at least this many slots
  int min_me2 = 0;          // pad the per-edge edgesOnEdge/weightsOnEdge slots
  bool vertex_fit = false;  // deriv2/4OnVertex tables
};

// Returns false and sets hm.err on invalid input.
bool prepare_mesh(const tmc_mesh_desc& d, const tmc_params& p, const PrepOptions& opt, HostMesh& hm);

// 3-D Hilbert index of a point of the unit cube [-1,1]^3 (Skilling 2004).
uint64_t hilbert_key(double x, double y, double z);
// 3-D Morton (bit-interleaved) index of a point of [-1,1]^3.
uint64_t morton_key(double x, double y, double z);

}  // namespace tmc
