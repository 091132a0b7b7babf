// Icosahedral spherical centroidal Voronoi (SCVT) mesh generator that emits the
// MPAS grid layout read by TMCORE's mesh_init (src/core/mesh_mod.F90:130-167).
//
// TMCORE ships no mesh file and no generator, so this is the project's own:
//   1. bisect the 20 faces of an icosahedron `level` times (generators = cell
//      centres, triangles = Delaunay triangles = Voronoi vertices);
//   2. run Lloyd iterations with the topology held fixed (each generator moves to
//      the area centroid of its Voronoi polygon, projected back to the sphere);
//   3. derive the MPAS connectivity, lengths, areas, kite areas and the TRiSK
//      tangential-reconstruction weights (Thuburn et al. 2009, Ringler et al.
//      2010) on the unit sphere.  mesh_init scales lengths by the radius itself
//      (mesh_mod.F90:205-222), so everything here is dimensionless.
//
// Conventions (the ones the reference operators rely on):
//   * the normal of edge e points from cellsOnEdge(1,e) to cellsOnEdge(2,e);
//   * the tangent k x n points from verticesOnEdge(1,e) to verticesOnEdge(2,e)
//     (the streamfunction initial conditions, e.g.
//     src/test_cases/swm/mountain_zonal_flow_test_mod.F90:50-52, and
//     curl_operator, src/core/operators_mod.F90:76-91, assume this);
//   * edgesOnCell(i,c) is the edge shared with cellsOnCell(i,c), counter-
//     clockwise (poly_fit_mod.F90:156-160 and :233-245 pair them by index); it
//     runs from verticesOnCell(i,c) to verticesOnCell(i+1,c);
//   * edgesOnVertex(i,v) joins cellsOnVertex(i,v) and cellsOnVertex(i+1,v),
//     and kiteAreasOnVertex(i,v) is the part of triangle v inside
//     cellsOnVertex(i,v);
//   * edgesOnEdge(:,e) lists the other edges of cellsOnEdge(1,e) counter-
//     clockwise starting after e, then those of cellsOnEdge(2,e).
//
// All indices stored here are 0-based; the Python side adds 1 when it writes
// an MPAS file.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct V3 {
  double x, y, z;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double norm(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 unit(V3 a) { return (1.0 / norm(a)) * a; }

// Great-circle distance between unit vectors (atan2 form: accurate for short arcs).
inline double arc(V3 a, V3 b) { return std::atan2(norm(cross(a, b)), dot(a, b)); }

// Signed area of the spherical triangle (a, b, c) on the unit sphere,
// positive when a, b, c are counter-clockwise seen from outside
// (Eriksson 1990: tan(E/2) = a.(b x c) / (1 + a.b + b.c + c.a)).
inline double tri_area(V3 a, V3 b, V3 c) {
  double num = dot(a, cross(b, c));
  double den = 1.0 + dot(a, b) + dot(b, c) + dot(c, a);
  return 2.0 * std::atan2(num, den);
}

inline void latlon(V3 p, double* lat, double* lon) {
  *lat = std::asin(std::max(-1.0, std::min(1.0, p.z)));
  double l = std::atan2(p.y, p.x);
  if (l < 0.0) l += 2.0 * M_PI;
  *lon = l;
}

}  // namespace

struct tmc_meshgen {
  int nCells = 0, nEdges = 0, nVertices = 0;
  int maxEdges = 6, maxEdges2 = 10, vertexDegree = 3;
  // int32 fields, element-major (k fastest), 0-based indices
  std::vector<int32_t> nEdgesOnCell, nEdgesOnEdge;
  std::vector<int32_t> cellsOnCell, edgesOnCell, verticesOnCell;  // [nCells][maxEdges]
  std::vector<int32_t> cellsOnEdge, verticesOnEdge;                // [nEdges][2]
  std::vector<int32_t> edgesOnEdge;                                // [nEdges][maxEdges2]
  std::vector<int32_t> cellsOnVertex, edgesOnVertex;               // [nVertices][3]
  // float64 fields (unit sphere)
  std::vector<double> xCell, yCell, zCell, latCell, lonCell;
  std::vector<double> xEdge, yEdge, zEdge, latEdge, lonEdge;
  std::vector<double> xVertex, yVertex, zVertex, latVertex, lonVertex;
  std::vector<double> dcEdge, dvEdge, dv1Edge, dv2Edge, angleEdge;
  std::vector<double> areaCell, areaTriangle, kiteAreasOnVertex;  // kite: [nVertices][3]
  std::vector<double> weightsOnEdge;                              // [nEdges][maxEdges2]
  std::vector<double> meshDensity;
  std::string err;
};

namespace {

// Recursive bisection of the icosahedron.  Returns generators and ccw triangles.
void build_icosahedral(int level, std::vector<V3>& pts, std::vector<int32_t>& tris) {
  const double p = (1.0 + std::sqrt(5.0)) / 2.0;
  const double base[12][3] = {{-1, p, 0}, {1, p, 0}, {-1, -p, 0}, {1, -p, 0},
                              {0, -1, p}, {0, 1, p}, {0, -1, -p}, {0, 1, -p},
                              {p, 0, -1}, {p, 0, 1}, {-p, 0, -1}, {-p, 0, 1}};
  const int faces[20][3] = {{0, 11, 5}, {0, 5, 1},  {0, 1, 7},   {0, 7, 10}, {0, 10, 11},
                            {1, 5, 9},  {5, 11, 4}, {11, 10, 2}, {10, 7, 6}, {7, 1, 8},
                            {3, 9, 4},  {3, 4, 2},  {3, 2, 6},   {3, 6, 8},  {3, 8, 9},
                            {4, 9, 5},  {2, 4, 11}, {6, 2, 10},  {8, 6, 7},  {9, 8, 1}};
  pts.clear();
  for (auto& b : base) pts.push_back(unit(V3{b[0], b[1], b[2]}));
  tris.clear();
  for (auto& f : faces) {
    int a = f[0], b = f[1], c = f[2];
    V3 n = cross(pts[b] - pts[a], pts[c] - pts[a]);
    if (dot(n, pts[a] + pts[b] + pts[c]) < 0) std::swap(b, c);
    tris.push_back(a);
    tris.push_back(b);
    tris.push_back(c);
  }
  for (int lev = 0; lev < level; ++lev) {
    std::unordered_map<uint64_t, int32_t> mid;
    mid.reserve(tris.size());
    auto midpoint = [&](int32_t a, int32_t b) -> int32_t {
      uint64_t lo = (uint64_t)std::min(a, b), hi = (uint64_t)std::max(a, b);
      uint64_t key = (lo << 32) | hi;
      auto it = mid.find(key);
      if (it != mid.end()) return it->second;
      int32_t id = (int32_t)pts.size();
      pts.push_back(unit(pts[a] + pts[b]));
      mid.emplace(key, id);
      return id;
    };
    std::vector<int32_t> nt;
    nt.reserve(tris.size() * 4);
    for (size_t t = 0; t < tris.size(); t += 3) {
      int32_t a = tris[t], b = tris[t + 1], c = tris[t + 2];
      int32_t ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
      const int32_t sub[4][3] = {{a, ab, ca}, {ab, b, bc}, {ca, bc, c}, {ab, bc, ca}};
      for (auto& s : sub) nt.insert(nt.end(), s, s + 3);
    }
    tris.swap(nt);
  }
}

inline V3 circumcentre(const std::vector<V3>& P, const int32_t* t) {
  return unit(cross(P[t[1]] - P[t[0]], P[t[2]] - P[t[0]]));
}

}  // namespace

extern "C" {

// Generate a level-`level` icosahedral SCVT (nCells = 10*4^level + 2) with
// `lloyd_iters` Lloyd iterations.  Returns 0 on success.
int tmc_meshgen_create(int level, int lloyd_iters, tmc_meshgen** out) {
  if (!out) return -1;
  *out = nullptr;
  if (level < 0 || level > 11 || lloyd_iters < 0) return -1;
  auto* m = new tmc_meshgen();
  std::vector<V3> P;
  std::vector<int32_t> T;
  build_icosahedral(level, P, T);
  const int nc = (int)P.size();
  const int nv = (int)(T.size() / 3);
  m->nCells = nc;
  m->nVertices = nv;

  // ---- ccw fan of triangles around each generator --------------------------
  // For triangle (a,b,c) ccw, around corner a it spans the wedge from ray a->b
  // to ray a->c; the next triangle counter-clockwise around a starts at ray a->c.
  std::vector<int32_t> deg(nc, 0);
  for (int t = 0; t < nv; ++t)
    for (int j = 0; j < 3; ++j) deg[T[3 * t + j]]++;
  for (int c = 0; c < nc; ++c) {
    if (deg[c] < 3 || deg[c] > 6) {
      m->err = "unexpected vertex degree";
      *out = m;
      return -2;
    }
  }
  std::vector<int32_t> fanStart(nc + 1, 0);
  for (int c = 0; c < nc; ++c) fanStart[c + 1] = fanStart[c] + deg[c];
  std::vector<int32_t> fanTri(fanStart[nc]), fanB(fanStart[nc]), fanC(fanStart[nc]);
  {
    std::vector<int32_t> fill(nc, 0);
    for (int t = 0; t < nv; ++t)
      for (int j = 0; j < 3; ++j) {
        int a = T[3 * t + j], b = T[3 * t + (j + 1) % 3], c = T[3 * t + (j + 2) % 3];
        int k = fanStart[a] + fill[a]++;
        fanTri[k] = t;
        fanB[k] = b;
        fanC[k] = c;
      }
  }
  // Order each fan counter-clockwise by chaining c -> b.
  for (int a = 0; a < nc; ++a) {
    int s = fanStart[a], n = deg[a];
    for (int k = 0; k + 1 < n; ++k) {
      int want = fanC[s + k];
      for (int q = k + 1; q < n; ++q)
        if (fanB[s + q] == want) {
          std::swap(fanTri[s + k + 1], fanTri[s + q]);
          std::swap(fanB[s + k + 1], fanB[s + q]);
          std::swap(fanC[s + k + 1], fanC[s + q]);
          break;
        }
    }
  }

  // ---- Lloyd iterations (topology fixed) -----------------------------------
  std::vector<V3> CC(nv);
  for (int it = 0; it < lloyd_iters; ++it) {
#pragma omp parallel for schedule(static)
    for (int t = 0; t < nv; ++t) CC[t] = circumcentre(P, &T[3 * t]);
    std::vector<V3> NP(nc);
#pragma omp parallel for schedule(static)
    for (int a = 0; a < nc; ++a) {
      int s = fanStart[a], n = deg[a];
      V3 acc{0, 0, 0};
      for (int k = 0; k < n; ++k) {
        V3 p1 = CC[fanTri[s + k]], p2 = CC[fanTri[s + (k + 1) % n]];
        double w = 0.5 * norm(cross(p1 - P[a], p2 - P[a]));
        acc = acc + (w / 3.0) * (P[a] + p1 + p2);
      }
      NP[a] = unit(acc);
    }
    P.swap(NP);
  }
#pragma omp parallel for schedule(static)
  for (int t = 0; t < nv; ++t) CC[t] = circumcentre(P, &T[3 * t]);

  // ---- edges -----------------------------------------------------------------
  const int ME = m->maxEdges, ME2 = m->maxEdges2;
  m->nEdgesOnCell.assign(nc, 0);
  m->cellsOnCell.assign((size_t)nc * ME, -1);
  m->edgesOnCell.assign((size_t)nc * ME, -1);
  m->verticesOnCell.assign((size_t)nc * ME, -1);
  int ne = 0;
  for (int a = 0; a < nc; ++a) {
    int s = fanStart[a], n = deg[a];
    m->nEdgesOnCell[a] = n;
    for (int k = 0; k < n; ++k) {
      // edge k joins a and b_k = fanB[s+k]; it lies between triangles
      // fanTri[s+k-1] (clockwise side) and fanTri[s+k] (ccw side).
      m->cellsOnCell[(size_t)a * ME + k] = fanB[s + k];
      m->verticesOnCell[(size_t)a * ME + k] = fanTri[s + (k + n - 1) % n];
      if (a < fanB[s + k]) m->edgesOnCell[(size_t)a * ME + k] = ne++;
    }
  }
  m->nEdges = ne;
  m->cellsOnEdge.assign((size_t)ne * 2, -1);
  m->verticesOnEdge.assign((size_t)ne * 2, -1);
  for (int a = 0; a < nc; ++a) {
    int s = fanStart[a], n = deg[a];
    for (int k = 0; k < n; ++k) {
      int b = fanB[s + k];
      if (a < b) {
        int e = m->edgesOnCell[(size_t)a * ME + k];
        m->cellsOnEdge[2 * e] = a;
        m->cellsOnEdge[2 * e + 1] = b;
        m->verticesOnEdge[2 * e] = fanTri[s + (k + n - 1) % n];
        m->verticesOnEdge[2 * e + 1] = fanTri[s + k];
      } else {
        // find the edge id created from b's side
        int sb = fanStart[b], nb = deg[b], e = -1;
        for (int q = 0; q < nb; ++q)
          if (fanB[sb + q] == a) e = m->edgesOnCell[(size_t)b * ME + q];
        m->edgesOnCell[(size_t)a * ME + k] = e;
      }
    }
  }

  // ---- vertices: corners ccw, edges between consecutive corners --------------
  m->cellsOnVertex.assign((size_t)nv * 3, -1);
  m->edgesOnVertex.assign((size_t)nv * 3, -1);
  auto edge_between = [&](int a, int b) -> int {
    int s = fanStart[a], n = deg[a];
    for (int q = 0; q < n; ++q)
      if (fanB[s + q] == b) return m->edgesOnCell[(size_t)a * ME + q];
    return -1;
  };
  for (int t = 0; t < nv; ++t)
    for (int j = 0; j < 3; ++j) {
      m->cellsOnVertex[3 * t + j] = T[3 * t + j];
      m->edgesOnVertex[3 * t + j] = edge_between(T[3 * t + j], T[3 * t + (j + 1) % 3]);
    }

  // ---- coordinates -----------------------------------------------------------
  auto fill_xyz = [](const std::vector<V3>& Q, std::vector<double>& x, std::vector<double>& y,
                     std::vector<double>& z, std::vector<double>& lat, std::vector<double>& lon) {
    size_t n = Q.size();
    x.resize(n);
    y.resize(n);
    z.resize(n);
    lat.resize(n);
    lon.resize(n);
    for (size_t i = 0; i < n; ++i) {
      x[i] = Q[i].x;
      y[i] = Q[i].y;
      z[i] = Q[i].z;
      latlon(Q[i], &lat[i], &lon[i]);
    }
  };
  std::vector<V3> EP(ne);
  for (int e = 0; e < ne; ++e)
    EP[e] = unit(P[m->cellsOnEdge[2 * e]] + P[m->cellsOnEdge[2 * e + 1]]);
  fill_xyz(P, m->xCell, m->yCell, m->zCell, m->latCell, m->lonCell);
  fill_xyz(EP, m->xEdge, m->yEdge, m->zEdge, m->latEdge, m->lonEdge);
  fill_xyz(CC, m->xVertex, m->yVertex, m->zVertex, m->latVertex, m->lonVertex);

  // ---- lengths and normal angle ------------------------------------------------
  m->dcEdge.resize(ne);
  m->dvEdge.resize(ne);
  m->dv1Edge.resize(ne);
  m->dv2Edge.resize(ne);
  m->angleEdge.resize(ne);
  for (int e = 0; e < ne; ++e) {
    V3 c1 = P[m->cellsOnEdge[2 * e]], c2 = P[m->cellsOnEdge[2 * e + 1]];
    V3 v1 = CC[m->verticesOnEdge[2 * e]], v2 = CC[m->verticesOnEdge[2 * e + 1]];
    V3 p = EP[e];
    m->dcEdge[e] = arc(c1, c2);
    m->dvEdge[e] = arc(v1, v2);
    m->dv1Edge[e] = arc(v1, p);
    m->dv2Edge[e] = arc(v2, p);
    V3 d = c2 - c1;
    V3 nrm = unit(d - dot(d, p) * p);
    V3 east{-p.y, p.x, 0.0};
    double ne_ = norm(east);
    if (ne_ < 1e-300) {
      m->angleEdge[e] = 0.0;
    } else {
      east = (1.0 / ne_) * east;
      V3 north = cross(p, east);
      m->angleEdge[e] = std::atan2(dot(nrm, north), dot(nrm, east));
    }
  }

  // ---- kite areas, triangle and cell areas -------------------------------------
  m->kiteAreasOnVertex.assign((size_t)nv * 3, 0.0);
  m->areaTriangle.assign(nv, 0.0);
  m->areaCell.assign(nc, 0.0);
  for (int t = 0; t < nv; ++t) {
    V3 v = CC[t];
    double tot = 0.0;
    for (int j = 0; j < 3; ++j) {
      int eNext = m->edgesOnVertex[3 * t + j];             // corner j -> corner j+1
      int ePrev = m->edgesOnVertex[3 * t + (j + 2) % 3];   // corner j-1 -> corner j
      V3 c = P[m->cellsOnVertex[3 * t + j]];
      double k = tri_area(c, EP[eNext], v) + tri_area(c, v, EP[ePrev]);
      m->kiteAreasOnVertex[3 * t + j] = k;
      tot += k;
    }
    m->areaTriangle[t] = tot;
  }
  for (int t = 0; t < nv; ++t)
    for (int j = 0; j < 3; ++j) m->areaCell[m->cellsOnVertex[3 * t + j]] += m->kiteAreasOnVertex[3 * t + j];

  // ---- TRiSK weights -------------------------------------------------------------
  // Kite fraction R(c, v) = kite area of cell c at vertex v / areaCell(c).
  // For cell i of edge e, going ccw from e over the other edges e_k of i, with S_k
  // the sum of R(i, v) over the vertices passed from e to e_k:
  //   w(e, e_k) = n(e,i) n(e_k,i) (1/2 - S_k) dvEdge(e_k) / dcEdge(e),
  // n(e,i) = +1 when i = cellsOnEdge(1,e).  This makes the tangential flux the
  // sum of the two cells' half-dual-edge fluxes that spread each cell's
  // divergence over its kites in proportion to area, and it is antisymmetric:
  // areaEdge(e) w(e,e') = -areaEdge(e') w(e',e).
  auto kite_of = [&](int c, int v) -> double {
    for (int j = 0; j < 3; ++j)
      if (m->cellsOnVertex[3 * v + j] == c) return m->kiteAreasOnVertex[3 * v + j];
    return 0.0;
  };
  m->nEdgesOnEdge.assign(ne, 0);
  m->edgesOnEdge.assign((size_t)ne * ME2, -1);
  m->weightsOnEdge.assign((size_t)ne * ME2, 0.0);
  for (int e = 0; e < ne; ++e) {
    int cnt = 0;
    for (int side = 0; side < 2; ++side) {
      int i = m->cellsOnEdge[2 * e + side];
      double ne_i = (side == 0) ? 1.0 : -1.0;
      int n = m->nEdgesOnCell[i];
      int pos = -1;
      for (int q = 0; q < n; ++q)
        if (m->edgesOnCell[(size_t)i * ME + q] == e) pos = q;
      double S = 0.0;
      for (int k = 1; k < n; ++k) {
        int q = (pos + k) % n;
        int ek = m->edgesOnCell[(size_t)i * ME + q];
        int vpass = m->verticesOnCell[(size_t)i * ME + q];  // vertex between edge q-1 and edge q
        S += kite_of(i, vpass) / m->areaCell[i];
        double nk = (m->cellsOnEdge[2 * ek] == i) ? 1.0 : -1.0;
        m->edgesOnEdge[(size_t)e * ME2 + cnt] = ek;
        m->weightsOnEdge[(size_t)e * ME2 + cnt] = ne_i * nk * (0.5 - S) * m->dvEdge[ek] / m->dcEdge[e];
        ++cnt;
      }
    }
    m->nEdgesOnEdge[e] = cnt;
  }
  m->meshDensity.assign(nc, 1.0);
  *out = m;
  return 0;
}

void tmc_meshgen_destroy(tmc_meshgen* m) { delete m; }

// dims = {nCells, nEdges, nVertices, maxEdges, maxEdges2, vertexDegree}
int tmc_meshgen_dims(const tmc_meshgen* m, int32_t* dims) {
  if (!m || !dims) return -1;
  dims[0] = m->nCells;
  dims[1] = m->nEdges;
  dims[2] = m->nVertices;
  dims[3] = m->maxEdges;
  dims[4] = m->maxEdges2;
  dims[5] = m->vertexDegree;
  return 0;
}

const char* tmc_meshgen_error(const tmc_meshgen* m) { return m ? m->err.c_str() : "null"; }

// Copy a named int32 field (MPAS variable name, 0-based indices) into dst.
// Returns the number of elements copied, or -1 if the name is unknown.
int64_t tmc_meshgen_get_i32(const tmc_meshgen* m, const char* name, int32_t* dst) {
  if (!m || !name) return -1;
  const std::vector<int32_t>* v = nullptr;
  std::string n(name);
  if (n == "nEdgesOnCell") v = &m->nEdgesOnCell;
  else if (n == "nEdgesOnEdge") v = &m->nEdgesOnEdge;
  else if (n == "cellsOnCell") v = &m->cellsOnCell;
  else if (n == "edgesOnCell") v = &m->edgesOnCell;
  else if (n == "verticesOnCell") v = &m->verticesOnCell;
  else if (n == "cellsOnEdge") v = &m->cellsOnEdge;
  else if (n == "verticesOnEdge") v = &m->verticesOnEdge;
  else if (n == "edgesOnEdge") v = &m->edgesOnEdge;
  else if (n == "cellsOnVertex") v = &m->cellsOnVertex;
  else if (n == "edgesOnVertex") v = &m->edgesOnVertex;
  if (!v) return -1;
  if (dst) std::memcpy(dst, v->data(), v->size() * sizeof(int32_t));
  return (int64_t)v->size();
}

int64_t tmc_meshgen_get_f64(const tmc_meshgen* m, const char* name, double* dst) {
  if (!m || !name) return -1;
  const std::vector<double>* v = nullptr;
  std::string n(name);
#define F(x) else if (n == #x) v = &m->x;
  if (false) {
  }
  F(xCell) F(yCell) F(zCell) F(latCell) F(lonCell)
  F(xEdge) F(yEdge) F(zEdge) F(latEdge) F(lonEdge)
  F(xVertex) F(yVertex) F(zVertex) F(latVertex) F(lonVertex)
  F(dcEdge) F(dvEdge) F(dv1Edge) F(dv2Edge) F(angleEdge)
  F(areaCell) F(areaTriangle) F(kiteAreasOnVertex) F(weightsOnEdge) F(meshDensity)
#undef F
  if (!v) return -1;
  if (dst) std::memcpy(dst, v->data(), v->size() * sizeof(double));
  return (int64_t)v->size();
}

}  // extern "C"
