/* TEST INFRASTRUCTURE ONLY - the CPU FP64 oracle of TMCORE's hot path.
 *
 * A plain-C restatement of the reference Fortran (TMCORE-Project/TMCORE):
 *   src/core/mesh_mod.F90:169-224        derived mesh quantities and scaling
 *   src/utils/poly_fit_mod.F90:119-609   least-squares stencil tables
 *   src/utils/math_mod.F90:52-133        scaled partial-pivot Gauss inverse
 *   src/utils/sphere_geometry_mod.F90    calc_sphere_angle, calc_arc_length
 *   src/core/operators_mod.F90           every operator on the path
 *   src/core/tmcore_swm_mod.F90:60-255   run loop, spatial_operators, tendencies,
 *                                        update_state, invariants
 *   src/core/time_scheme_mod.F90:47-184  CRK3 / CRK4 / PC2
 *   src/core/adv_schemes/adv_scheme_sg11_mod.F90:33-48 and
 *   src/core/tmcore_adv_mod.F90:78-97    tracer advection model
 * Each function cites the lines it follows.  Element loops keep the
 * reference's per-element summation order; global sums are serial, as in the
 * reference.  Build with -O2 -ffp-contract=off (no FMA contraction).
 *
 * PARITY UNPINNED: the reference is Fortran, no Fortran compiler exists in
 * the build image, and it ships no golden vectors, meshes or expected
 * outputs.  The restatement is cross-checked by physics-level known answers
 * (steady geostrophic flow, conservation of mass / absolute vorticity,
 * energy conservation with the CRK4 beta, tracer return after one period).
 *
 * Only tests, the smoke check and the CPU baseline of bench.py may use this.
 */
#ifndef TMC_ORACLE_H
#define TMC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* The MPAS grid exactly as mesh_init reads it: unit sphere, int32 1-based
 * connectivity, Fortran (k, n) column-major 2-D arrays. */
typedef struct orc_mesh_in {
  int32_t nCells, nEdges, nVertices, maxEdges, maxEdges2, vertexDegree;
  const int32_t *nEdgesOnCell, *nEdgesOnEdge;
  const int32_t *cellsOnCell, *edgesOnCell, *verticesOnCell; /* (maxEdges, nCells) */
  const int32_t *cellsOnEdge, *verticesOnEdge;               /* (2, nEdges) */
  const int32_t *edgesOnEdge;                                /* (maxEdges2, nEdges) */
  const int32_t *cellsOnVertex, *edgesOnVertex;              /* (vertexDegree, nVertices) */
  const double *xCell, *yCell, *zCell, *latCell, *lonCell;
  const double *xEdge, *yEdge, *zEdge, *latEdge, *lonEdge;
  const double *xVertex, *yVertex, *zVertex, *latVertex, *lonVertex;
  const double *dvEdge, *dcEdge, *areaCell, *areaTriangle;
  const double *kiteAreasOnVertex; /* (vertexDegree, nVertices) */
  const double *weightsOnEdge;     /* (maxEdges2, nEdges) */
} orc_mesh_in;

/* namelist &tmcore (src/core/params_mod.F90:35-55) and const_mod constants */
typedef struct orc_params {
  double dt;
  int32_t time_scheme;     /* 1 CRK3, 2 CRK4, 3 PC2 */
  int32_t pv_scheme;       /* 1 APVM, 2 conservative APVM, 3 high-order upwind */
  int32_t conserve_energy;
  int32_t flux_4th_order_correct;
  double apvm_weight;
  int32_t adv_order;
  int32_t adv_mono;
  int32_t interp_pv_order;
  double radius, g, omega;
  int32_t n_tracers;        /* coupled mass-weighted tracers (no reference counterpart) */
  int32_t tracer_adv_order; /* 0: same as adv_order */
  int32_t tracer_adv_mono;
  int32_t nthreads;         /* OpenMP threads for element loops (0: runtime default) */
} orc_params;

typedef struct orc_model orc_model;

void orc_default_params(orc_params* p);
orc_model* orc_create(const orc_mesh_in* mesh, const orc_params* p);
void orc_destroy(orc_model* m);
const char* orc_error(const orc_model* m);

/* Derived mesh quantities after mesh_init (radius-scaled), element order as read. */
const double* orc_areaEdge(const orc_model* m);
const double* orc_fVertex(const orc_model* m);
double orc_totalArea(const orc_model* m);
const int32_t* orc_nSignEdge(const orc_model* m); /* (maxEdges, nCells) */
const int32_t* orc_tSignEdge(const orc_model* m); /* (vertexDegree, nVertices) */
/* poly_fit tables, fit arrays (0:30, n) 1-based entries, deriv (0:30, 2, nEdges) */
int orc_poly_fit_table(const orc_model* m, const char* name, const void** data, int64_t* count);

/* ---- single operators on caller arrays (1:1 with operators_mod publics) ---- */
void orc_op_div(orc_model* m, const double* f_edge, double* div);
void orc_op_curl(orc_model* m, const double* f_edge, double* curl);
void orc_op_c2e(orc_model* m, const double* f_cell, double* f_edge);
void orc_op_c2v(orc_model* m, const double* f_cell, double* f_vertex);
void orc_op_v2c(orc_model* m, const double* f_vertex, double* f_cell);
void orc_op_v2e(orc_model* m, const double* f_vertex, double* f_edge);
void orc_op_kinetic_energy(orc_model* m, const double* u, double* ke);
void orc_op_tangent_wind(orc_model* m, const double* u, double* v);
void orc_op_tangent_vor_flux(orc_model* m, const double* u, const double* gd_e, const double* pv_e, double* out);
void orc_op_upwind_correction(orc_model* m, const double* f_cell, const double* u_edge, double* f_edge,
                              int order, int mono);

/* ---- shallow-water model (tmcore_swm_mod) ---- */
/* state(old): gd (cells), u (edges) from an initial condition; ghs (cells).
 * Runs the pre-loop of tmcore_swm_run (tmcore_swm_mod.F90:62-71). */
void orc_swm_set_initial(orc_model* m, const double* gd, const double* u, const double* ghs);
/* Set prognostics of state(old) directly (gd, iap_u) and recompute diagnostics. */
void orc_swm_set_state(orc_model* m, const double* gd, const double* iap_u);
/* One call of spatial_operators (tmcore_swm_mod.F90:92-125) on (gd, iap_u). */
void orc_swm_spatial_operators(orc_model* m, const double* gd, const double* iap_u, double* tend_gd,
                               double* tend_iap_u);
/* nsteps iterations of the tmcore_swm_run loop body (tmcore_swm_mod.F90:75-88). */
void orc_swm_step(orc_model* m, int nsteps);
/* state(old) prognostics and diagnostics */
void orc_swm_get_state(const orc_model* m, double* gd, double* iap_u, double* u);
void orc_swm_get_vertex(const orc_model* m, double* pv, double* vor);
/* {total_mass, total_energy, total_potential_enstrophy, total_absolute_vorticity, beta} */
void orc_swm_get_diag(const orc_model* m, double out[5]);
/* coupled tracers, mass weighted (gd*q), [n_tracers][nCells] */
void orc_set_tracers(orc_model* m, const double* q);
void orc_get_tracers(const orc_model* m, double* q);

/* ---- tracer advection model (tmcore_adv_mod, sg11) ---- */
enum { ORC_WIND_COSINE_BELL = 1, ORC_WIND_DEFORMATION_CASE4 = 2 };
void orc_adv_set_initial(orc_model* m, const double* q, int wind_case);
void orc_adv_step(orc_model* m, int nsteps);
void orc_adv_get(const orc_model* m, double* q, double* u);
double orc_adv_elapsed(const orc_model* m);

/* cell-centre wind from edge normal velocity (mpas_reconstruct_1d):
 * Cartesian components and the zonal / meridional winds */
void orc_reconstruct(orc_model* m, const double* u, double* uX, double* uY, double* uZ, double* uzon,
                     double* umer);

#ifdef __cplusplus
}
#endif
#endif
