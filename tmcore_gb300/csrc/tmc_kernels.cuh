// Device kernels of one TRiSK shallow-water stage and of the CRK4 step.
//
// Included by tmc_kernels_f64.cu (T = double, compiled with -fmad=false so
// every element is computed in the reference's expression order and matches
// the FP64 oracle bit for bit) and tmc_kernels_f32.cu (T = float: FP32 edge
// and vertex state and stencil arithmetic from FP32-rounded copies of the
// metrics; FP64 gd and tracer mass with the mass-flux divergence accumulated
// in FP64; FP64 compensated sums).
//
// One stage (spatial_operators, src/core/tmcore_swm_mod.F90:92-125) is five
// passes over structure-of-arrays data in space-filling-curve order:
//   edge_prep : gd_edge = c2e(gd) [+upwind], u = iap_u / sqrt(gd_edge),
//               F = u gd_edge, tracer fluxes       (operators_mod.F90:93-104,
//                                                   :168-176, :423-472)
//   cell      : tend_gd = div_operator(F), ke, E = ke+gd+ghs, the RK stage
//               update of gd and tracers            (:40-55, :206-221,
//                                                   tmcore_swm_mod.F90:127-139)
//   vertex    : gd_vertex = c2v(gd), vor = curl(u), pv = (f+vor)/gd_vertex
//                                                   (:76-91, :106-123, :262-270)
//   edge_pv   : pv on edges (APVM or high-order upwind) (:273-412)
//   edge_flux : q.F_perp (calc_tangent_vor_flux :239-260), kinetic-energy and
//               geopotential gradient, iap_u tendency (tmcore_swm_mod.F90:155-201),
//               the RK stage update of iap_u and the CRK4 inner products
//               (time_scheme_mod.F90:109-154)
// Each thread handles kEPT elements (block-strided, so loads stay coalesced).
// Global sums (beta, invariants) are per-thread sums, a warp shuffle tree and
// a double-double combination of the warp sums per block; k_finalize reduces
// the per-block partials in a fixed order: deterministic and compensated.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace tmc {

constexpr int kEPT = 4;  // elements per thread
constexpr int kUpW32 = 16;  // widest vertex fit stencil of the packed FP32 upwind pv kernel

struct DStencil {
  int width;
  const uint8_t* count;  // [2][ne]
  const int32_t* idx;    // [width][2][ne]
  const double* w;       // [width][2][ne]
};

struct DevMesh {
  int nc, ne, nv, me, me2;
  const uint8_t* nEdgesOnCell;
  const int32_t* edgesOnCell;  // [me][nc]
  const int32_t* cellsOnCell;  // [me][nc], the cell across edgesOnCell (derived)
  const int8_t* nSign;         // [me][nc]
  const double* areaCell;
  const int32_t* cellsOnEdge;     // [2][ne]
  const int32_t* verticesOnEdge;  // [2][ne]
  const uint8_t* nEdgesOnEdge;
  const int32_t* edgesOnEdge;    // [me2][ne]
  const double* weightsOnEdge;   // [me2][ne]
  const double* dcEdge;
  const double* dvEdge;
  const double* areaEdge;
  const int32_t* cellsOnVertex;  // [3][nv]
  const int32_t* edgesOnVertex;  // [3][nv]
  const int8_t* tSign;           // [3][nv]
  const double* kite;            // [3][nv]
  const double* areaTriangle;
  const double* fVertex;
  const int32_t* v2c_start;
  const int32_t* v2c_vertex;
  const double* v2c_kite;
  DStencil cell2, cell3, cell4, vert2, vert4;  // cell3: deriv3OnCell on the fit3 (= fit4) stencils
  // FP32 path with upwind pv of order 3 or 4 (pv_scheme 3): vert2 packed as
  // (stencil vertex, FP32 weight bits) entries [width][2][ne], width at most
  // kUpW32 (null otherwise: the generic stencil loop runs)
  const int2* vert2_iw;
  // FP32 path: FP32-rounded copies of the metrics used in FP32 arithmetic
  // and FP64 reciprocals of the areas used in FP64 arithmetic (null in FP64 mode)
  const float* weightsOnEdge_f;
  const float* dcEdge_f;
  const float* dvEdge_f;
  const float* areaEdge_f;
  const float* kite_f;
  const float* invAreaTriangle_f;
  const float* fVertex_f;
  const float* invAreaCell_f;
  const float* areaCell_f;
  const float* areaTriangle_f;
  const double* invAreaCell;
  // vector reconstruction (history): coefficients [3][me][nc], cos/sin lat, lon [4][nc]
  const double* recon;
  const double* cell_trig;
};

struct ModelOpt {
  double dt;
  int adv_order;       // gd upwind correction (operators_mod.F90:423-472)
  double cell_coef2, cell_coef4;
  int pv_scheme;       // 1 APVM, 3 high-order upwind
  double apvm_weight;
  int interp_pv_order;
  double vert_coef2, vert_coef4;
  int n_tracers;
  int tr_order;
  double tr_coef2, tr_coef4;
  int flux4;  // flux_4th_order_correct (tmcore_swm_mod.F90:183-195)
  int need_pv_c;  // pv on cells every stage (the learned closure reads it)
};

// CRK4 stage program (time_scheme_mod.F90:109-154):
//   mode 0: tendency only (spatial_operators)
//   mode 1: acc = t, next = old + a_dt t
//   mode 2/3: R(k-1,k) += t_prev t area, acc = acc + 2 t, next = old + a_dt t
//   mode 4: R34 += t_prev t area, t_new = (acc + t)/6, R44 += t_new t_new area
struct RKStage {
  int mode;
  double a_dt;
};

// Partial-sum regions (one double-double per block each).
enum Region {
  R_IP_C = 0,  // inner product <t_prev, t> cells   (region + 2*(stage-2))
  R_IP_E = 1,  // inner product edges
  R_44_C = 6,
  R_44_E = 7,
  R_MASS = 8,
  R_EN_E = 9,
  R_EN_C = 10,
  R_PE = 11,
  R_AV = 12,
  R_C1 = 13,  // conservative APVM sums (operators_mod.F90:349-353)
  R_C2 = 14,
  R_C3 = 15,
  R_COUNT = 16
};
constexpr int kFinalizeRegions = R_C1;  // regions k_finalize reduces
constexpr int kFinSplit = 16;            // blocks of k_finalize per region

struct Partials {
  double* base;  // [member][R_COUNT][cap][2]
  int cap;
  double* fin;   // [member][kFinalizeRegions][kFinSplit][2]: k_finalize's sums of one block's slots
  __host__ __device__ double* region(int r) const { return base + (size_t)r * cap * 2; }
  __host__ __device__ size_t member_stride() const { return (size_t)R_COUNT * cap * 2; }
  __host__ __device__ Partials at(int m) const {
    return Partials{base + (size_t)m * member_stride(), cap,
                    fin ? fin + (size_t)m * kFinalizeRegions * kFinSplit * 2 : nullptr};
  }
};

// device results: [0] mass [1] energy [2] enstrophy [3] abs vort [4] beta
//                 [5] R12 [6] R23 [7] R34 [8] R44 [9] beta*dt
//                 [10] epsilon of the conservative APVM [11] elapsed seconds (adv model)
constexpr int kDiagLen = 12;
// per-member block of the device diag array: outputs, region sums, counters
constexpr int kDiagStride = 32;
static_assert(kDiagLen + R_COUNT + 2 <= kDiagStride, "diag block too small");

template <class T>
struct StageIO {
  // stage input state and RK buffers
  const double* gd_in;
  const double* gd_old;
  double* gd_next;
  double* gd_acc;
  double* gd_tend;  // current tendency (read as t_prev before overwrite)
  const T* iap_in;
  const T* iap_old;
  T* iap_next;
  T* iap_acc;
  T* iap_tend;
  const T* q_in;  // tracer mass gd*q [ntr][nc] (FP32 in the FP32 path)
  const T* q_old;
  T* q_next;
  T* q_acc;
  // FP32 shadows (FP32 path only): gd and tracer mixing ratio of the stage,
  // the current gd tendency, topography
  const float* gdf_in;
  float* gdf_next;
  const float* qr_in;  // [ntr][nc]
  float* qr_next;
  float* tendf;        // gd tendency of the stage (read as t_prev before overwrite)
  const float* ghsf;
  // intermediates
  T* gd_e;
  T* u;
  T* F;   // u * gd_e
  T* Fq;  // [ntr][ne]
  // the next stage's gd_e, u, F, Fq, written by k_edge_flux (stages 1-3) and
  // k_final_edges (next step): the edge preparation of the next stage fused
  // into the pass that produces its iap_u (null: not fused)
  T* gd_e_nx;
  T* u_nx;
  T* F_nx;
  T* Fq_nx;
  T* E;
  T* pv_v;
  T* vor;
  T* gd_v;
  T* pv_c;
  T* v_e;
  T* pv_e;
  const double* ghs;
  // conservative APVM (pv_scheme 2): correction direction and the two
  // tangent fluxes of pv_edge and of the correction
  T* dpv;
  T* pvf;
  T* dpvf;
  // Ensemble members of one mesh, member-outermost: the kernels run member
  // blockIdx.y, whose arrays start `members strides` further on.
  int members;
  long long msc, mse, msv, msq, msqe;  // cells, edges, vertices, [ntr][nc], [ntr][ne]
  template <class P>
  __host__ __device__ static P* off(P* p, long long o) {
    return p ? p + o : p;
  }
  __host__ __device__ StageIO at(int m) const {
    if (m == 0) return *this;
    StageIO s = *this;
    const long long c = m * msc, e = m * mse, v = m * msv, q = m * msq, qe = m * msqe;
    s.gd_in = off(gd_in, c);
    s.gd_old = off(gd_old, c);
    s.gd_next = off(gd_next, c);
    s.gd_acc = off(gd_acc, c);
    s.gd_tend = off(gd_tend, c);
    s.iap_in = off(iap_in, e);
    s.iap_old = off(iap_old, e);
    s.iap_next = off(iap_next, e);
    s.iap_acc = off(iap_acc, e);
    s.iap_tend = off(iap_tend, e);
    s.q_in = off(q_in, q);
    s.q_old = off(q_old, q);
    s.q_next = off(q_next, q);
    s.q_acc = off(q_acc, q);
    s.gdf_in = off(gdf_in, c);
    s.gdf_next = off(gdf_next, c);
    s.qr_in = off(qr_in, q);
    s.qr_next = off(qr_next, q);
    s.tendf = off(tendf, c);
    s.ghsf = off(ghsf, c);
    s.gd_e = off(gd_e, e);
    s.u = off(u, e);
    s.F = off(F, e);
    s.Fq = off(Fq, qe);
    s.gd_e_nx = off(gd_e_nx, e);
    s.u_nx = off(u_nx, e);
    s.F_nx = off(F_nx, e);
    s.Fq_nx = off(Fq_nx, qe);
    s.E = off(E, c);
    s.pv_v = off(pv_v, v);
    s.vor = off(vor, v);
    s.gd_v = off(gd_v, v);
    s.pv_c = off(pv_c, c);
    s.v_e = off(v_e, e);
    s.pv_e = off(pv_e, e);
    s.ghs = off(ghs, c);
    s.dpv = off(dpv, e);
    s.pvf = off(pvf, e);
    s.dpvf = off(dpvf, e);
    return s;
  }
};

// ensemble members a launch covers (gridDim.y)
template <class T>
inline unsigned nmem(const StageIO<T>& S) {
  return S.members > 1 ? (unsigned)S.members : 1u;
}

// ---- launchers (instantiated in tmc_kernels_f64.cu / _f32.cu) ----
template <class T>
void launch_edge_prep(const DevMesh& M, const ModelOpt& O, const StageIO<T>& S, Partials P, bool diag, int bs,
                      cudaStream_t st);
template <class T>
void launch_cell(const DevMesh& M, const ModelOpt& O, const StageIO<T>& S, RKStage rk, Partials P, bool diag,
                 int bs, cudaStream_t st);
// FP32, single member, 1, 2 or 4 second-order tracers: the tracer terms of
// the cell pass of stage rk, after a tracer-free cell pass of that stage
// (launch_cell with n_tracers 0); a no-op otherwise
template <class T>
void launch_tracers_fast(const DevMesh& M, const ModelOpt& O, const StageIO<T>& S, RKStage rk, int bs,
                         cudaStream_t st);
template <class T>
void launch_vertex(const DevMesh& M, const ModelOpt& O, const StageIO<T>& S, Partials P, bool diag, int bs,
                   cudaStream_t st);
template <class T>
void launch_edge_pv(const DevMesh& M, const ModelOpt& O, const StageIO<T>& S, int bs, cudaStream_t st);
template <class T>
void launch_edge_flux(const DevMesh& M, const ModelOpt& O, const StageIO<T>& S, RKStage rk, Partials P, int bs,
                      cudaStream_t st);
// final update (beta-scaled) of cells, then of edges together with the edge
// preparation of the next step's first stage and its energy partials
template <class T>
void launch_final_update(const DevMesh& M, const ModelOpt& O, const StageIO<T>& S, const double* diag, Partials P,
                         int bs, cudaStream_t st);
// number of blocks a launcher uses for n elements
__host__ __device__ inline int grid_for(int n, int bs) { return (n + bs * kEPT - 1) / (bs * kEPT); }

// reduction of partial regions into diag[]; counts per region.  scheme: the
// beta formula (1 CRK3, 2 CRK4, 3 PC2; time_scheme_mod.F90:94-100,144-150,174-180)
void launch_finalize(Partials P, const int* counts_host, double totalArea, double sumAreaTriangle, double dt,
                     bool step, bool diag, bool conserve, double* diag_out, cudaStream_t st, int scheme = 2,
                     int members = 1);

// conservative APVM (pv_scheme 2) after k_edge_pv: both tangent fluxes, their
// curls and the three global sums, epsilon, and the correction of pv_edge
template <class T>
void launch_cons_apvm(const DevMesh& M, const ModelOpt& O, const StageIO<T>& S, Partials P, double* diag_out, int bs,
                      cudaStream_t st);
void launch_cons_eps(Partials P, int count, double dt, double* diag_out, cudaStream_t st, int members = 1);

// Generic integrators (CRK3, PC2, and CRK4 of the adv model): state update
// new = old + coef t (update_state, tmcore_swm_mod.F90:203-213), coef from the
// host or from device memory (beta*dt); FP32 shadows of the new state.
template <class T>
struct UpdateArgs {
  const double* gd_o;
  double* gd_n;
  const double* tgd;
  const T* iap_o;
  T* iap_n;
  const T* tiap;  // null: no edge update (adv model)
  const T* q_o;
  T* q_n;
  const T* tq;
  float* gdf_n;
  float* qr_n;
  double a_dt;
  const double* coef_dev;  // non-null: coef = *coef_dev
};
template <class T>
void launch_update(const DevMesh& M, int ntr, const UpdateArgs<T>& a, int bs, cudaStream_t st);

// Combination of the stage tendencies into t_new (written over t[0]) and the
// inner products of the beta formula (operators_mod.F90:187-194), into the
// partial regions R_IP_*(k) and R_44_*:  CRK4 (scheme 2): t_new = (t1 + 2 t2 +
// 2 t3 + t4)/6, <t1,t2>, <t2,t3>, <t3,t4>, <tn,tn>; CRK3 (1): (t1 + 4 t2 +
// t3)/6, <t1,t2>, <t1,t3>, <t2,t3>, <tn,tn>; PC2 (3): no combination, <t0,t1>
// and <t1,t1>.  Partial counts: grid_for(nc) for cells, grid_for(ne) for edges.
template <class T>
struct CombineArgs {
  double* tgd[4];
  T* tiap[4];  // null: no edge tendency (adv model; the edge products are zero)
  T* tq[4];
};
template <class T>
void launch_combine(const DevMesh& M, int ntr, int scheme, const CombineArgs<T>& a, Partials P, int bs,
                    cudaStream_t st);

// adv model (tmcore_adv_mod.F90:78-97): gd_edge = c2e(gd) + upwind correction
// with the sign of u, tend = div_operator(u gd_edge) (adv_scheme_sg11_mod.F90:33-48)
void launch_adv_spatial(const DevMesh& M, const ModelOpt& O, const double* gd, const double* u, double* gd_e,
                        double* F, double* tend, int bs, cudaStream_t st);
// prescribed wind at t0 + offset seconds (offset from the host, or *offset_dev
// when non-null), u = -(psi(v2) - psi(v1))/dvEdge (cosine_bell_rotation_test_mod.F90:45-68,
// deformation_flow_test_mod.F90:74-105)
void launch_adv_wind(const DevMesh& M, int wind_case, double radius, const double* latV, const double* lonV,
                     const double* t0_dev, double offset, const double* offset_dev, double* psi, double* u,
                     cudaStream_t st);
void launch_adv_advance(double* elapsed_dev, double dt, cudaStream_t st);
// mass of gd into R_MASS and zero partials for the other invariant regions;
// returns the partial count used
int launch_mass_only(const DevMesh& M, const double* gd, Partials P, int bs, cudaStream_t st);

// state transfer in the caller's element order: dst[i] = src[n2o[i]] / dst[n2o[i]] = src[i]
template <class T>
void launch_gather(int n, const double* src, const int32_t* n2o, T* dst, cudaStream_t st);
template <class T>
void launch_scatter(int n, const T* src, const int32_t* n2o, double* dst, cudaStream_t st);
// iap_u = sqrt(gd_edge) * u (iap_swm_operator, operators_mod.F90:158-166)
template <class T>
void launch_iap_from_u(int ne, const double* gd_e, const double* u, T* iap, cudaStream_t st);
// FP32 shadows of gd and tracer mixing ratios of a state slot (FP32 path)
void launch_shadows(int nc, int ntr, const double* gd, const float* q, float* gdf, float* qr, cudaStream_t st);
void launch_to_f32(size_t n, const double* src, float* dst, cudaStream_t st);

// Learned PV-on-edge closure (FP32 path, after k_edge_pv): 24 features per
// edge from the stage state, the MLP on the tensor cores, pv_edge += the
// output for every member whose flag is set.  `net` is a tmc::mlp::Net.
// Needs pv_c (k_v2c) of the stage.  *err is set when a completion wait ran out.
struct ClosureArgs {
  const void* net;         // const tmc::mlp::Net*
  const int* member_on;    // [members] 1: apply
  int* err;
  int sms;
  float* dq;               // held correction [members][edge stride] (modes 1 and 2)
  int mode;                // 0: run the network; 1: run it and hold its output in dq; 2: add dq only
};
void launch_closure(const DevMesh& M, const StageIO<float>& S, const ClosureArgs& a, cudaStream_t st);
// the features (and pv_edge) of every edge of member m, into feat[ne][24] / pv[ne]
void launch_closure_features(const DevMesh& M, const StageIO<float>& S, int member, float* feat, float* pv,
                             cudaStream_t st);

// History diagnostics (history_mod.F90:124-174): the cell-centre wind of
// mpas_reconstruct_1d (mpas_vector_reconstruction.F90:207-261), h = (gd + ghs)/g,
// and a copy of an edge field in FP64.  Outputs may be null.
template <class T>
void launch_reconstruct(const DevMesh& M, const T* u, double* uX, double* uY, double* uZ, double* zonal,
                        double* meridional, cudaStream_t st);
void launch_h_field(int nc, const double* gd, const double* ghs, double g, double* h, cudaStream_t st);
template <class T>
void launch_to_f64(size_t n, const T* src, double* dst, cudaStream_t st);

// single operators for parity (FP64 only)
void launch_op(int op, const DevMesh& M, const ModelOpt& O, const double* a, const double* b, const double* c,
               double* out, int order, int mono, double coef2, double coef4, int bs, cudaStream_t st);

// operator ids for launch_op
enum OpId { OP_DIV = 0, OP_CURL, OP_C2E, OP_C2V, OP_V2C, OP_V2E, OP_KE, OP_TWIND, OP_TVF, OP_UPWIND };

}  // namespace tmc
