// C ABI of the library (include/tmcore_gpu.h): handle life cycle, device
// buffers, the CRK4 step program and its CUDA graph, state transfer in the
// caller's element order, timing.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <type_traits>
#include <string>
#include <vector>

#include "tmc_ensemble.cuh"
#include "tmc_kernels.cuh"
#include "tmc_mlp.cuh"
#include "tmc_prep.h"
#include "tmcore_gpu.h"

using namespace tmc;

namespace {

// coef2 / coef4 of the upwind corrections (operators_mod.F90:437-441, :377-380)
double coef2_cell(int order, int mono) {
  double c = 0.0;
  if (order == 3) c = 1.0;
  if (order == 3 && mono) c = 0.25;
  return c;
}
double coef2_vertex(int order) { return order == 3 ? 1.0 : 0.0; }

struct EngineBase {
  virtual ~EngineBase() {}
  virtual int alloc() = 0;
  virtual void launch_step(bool diag, std::vector<cudaEvent_t>* flux_ev, size_t* ev_pos) = 0;
  // The fused step split for tmc_time_integrate, whose tracers arrive after
  // gd and iap_u: stage 1 with a tracer-free cell pass (launch_stage1_early),
  // the stage's tracer terms once the tracers are in (launch_late_tracers),
  // then stages 2-4 and the final update (launch_step with first_stage 2).
  // can_split: the FP32 fused program with 1, 2 or 4 second-order tracers.
  virtual bool can_split() const { return false; }
  // the tracers gathered from raw (original order) into state slot 0 and
  // their FP32 ratios, on stream s; gd's FP32 shadow is left as it is
  virtual void gather_tracers_on(const double*, cudaStream_t) {}
  virtual void launch_stage1_early(bool) {}
  virtual void launch_late_tracers() {}
  int first_stage = 1;
  virtual void launch_diag_pass(bool finalize) = 0;
  virtual void launch_prep() = 0;
  virtual void launch_spatial_only() = 0;
  virtual void set_state_dev(const double* raw_gd, const double* raw_iap) = 0;  // from raw (original order)
  virtual void gather_field(int which, const double* raw) = 0;                  // F_GD, F_IAP or tracers (-1), no shadows
  virtual void get_field(int which, double* raw_out) = 0;                       // scatter to raw
  virtual void set_iap_from_u(const double* ge_new, const double* u_new) = 0;
  virtual void set_tracers_dev(const double* raw_q) = 0;
  // FP32 shadows of state slot `slot` (gd, and the tracer ratios unless !tracers)
  virtual void refresh_shadows(int slot, bool tracers = true) = 0;
  virtual void get_tracers_dev(double* raw_q) = 0;
  virtual void set_ghs_dev(const double* raw) = 0;
  virtual int launches_per_step() const = 0;
  virtual void adv_set_initial_dev(const double* raw_q) = 0;  // adv model: gd <- q, wind at t = 0
  virtual void adv_get_dev(double* raw_q, double* raw_u) = 0;
  virtual void state_slot0(void** gd, void** iap, void** q, void** ghs) = 0;  // all members
  virtual void refresh_all_shadows() = 0;
  virtual void closure_features(float* feat, float* pv) = 0;
  // history fields of the selected member into device arrays (null: skip):
  // u [ne], zonal, meridional, h, div [nc], pv, vor [nv]
  virtual void history_dev(double* u, double* zon, double* mer, double* hc, double* div, double* pv, double* vor,
                           double* scratch_e) = 0;
};

enum Field { F_GD = 0, F_IAP, F_U, F_PV_V, F_VOR, F_TEND_GD, F_TEND_IAP, F_GD_STAGE };
// passes of the fused step (block sizes, timing)
enum Pass { P_CELL = 0, P_VERTEX, P_PV, P_FLUX, P_FINAL, P_COUNT };

}  // namespace

struct tmc_handle {
  tmc_params p{};
  HostMesh hm;
  DevMesh M{};
  ModelOpt O{};
  cudaStream_t st = nullptr;
  std::vector<void*> dptrs;
  size_t dbytes = 0;
  std::string err;
  int32_t *d_cell_n2o = nullptr, *d_edge_n2o = nullptr, *d_vert_n2o = nullptr;
  double *raw_c = nullptr, *raw_e = nullptr, *raw_v = nullptr, *raw_q = nullptr;
  double *op_a = nullptr, *op_b = nullptr, *op_c = nullptr, *op_out = nullptr;
  Partials P{};
  int counts[R_COUNT] = {};
  double* d_diag = nullptr;
  double* h_diag = nullptr;
  int bs = 256;
  bool have_state = false;
  bool prep_valid = false;  // edge set 0 holds the preparation of state(old)
  std::unique_ptr<EngineBase> eng;
  cudaGraphExec_t g_step = nullptr, g_step_diag = nullptr;
  // stages 2-4 and the final update, after a stage 1 launched outside the
  // graph (tmc_time_integrate with late tracers); [diag]
  cudaGraphExec_t g_tail[2] = {nullptr, nullptr};
  void drop_graphs() {
    for (cudaGraphExec_t* g : {&g_step, &g_step_diag, &g_tail[0], &g_tail[1]}) {
      if (*g) cudaGraphExecDestroy(*g);
      *g = nullptr;
    }
  }
  long step_count = 0;
  double cell_coef4 = 0.25, vert_coef4 = 0.25;  // SAVE'd coef4 of the upwind routines
  // ensemble members of this mesh (member-outermost arrays) and the member the
  // state-transfer calls address (tmc_select_member)
  int members = 1;
  int cur = 0;
  // generic integrator program: CRK3, PC2, or the adv model (any scheme)
  bool generic = false;
  bool adv = false;
  int gen_counts[R_COUNT] = {};  // partial counts of the generic step's finaliser
  const double* d_latV = nullptr;
  const double* d_lonV = nullptr;
  std::vector<cudaEvent_t> ev_pool;
  // block size per pass of the fused step (cell, vertex, edge_pv, edge_flux,
  // final), chosen by tmc_autotune; the partial-sum counts follow them
  int bsp[5] = {256, 256, 256, 256, 256};
  // learned PV-on-edge closure (FP32 path): network, per-member switch, wait status
  const tmc_mlp* closure = nullptr;
  tmc::mlp::Net closure_net{};
  int* d_member_on = nullptr;
  int* d_closure_err = nullptr;
  bool closure_every_stage = true;
  float* d_closure_dq = nullptr;  // the held correction (closure in stage 1 only)
  int sms = 148;
  double* d_hist = nullptr;    // history outputs on cells (5 x nCells)
  cudaStream_t cst = nullptr;  // host-copy stream of tmc_time_integrate
  // second stream of the step program: the vertex and pv-on-edge passes of a
  // stage run on it, concurrent with the cell pass (fork/join events)
  cudaStream_t st2 = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  cudaEvent_t cev[8] = {};
  double* d_hist_e = nullptr;  // history outputs on edges and vertices
  int timed_pass = 3;  // the pass tmc_time_steps brackets with events

  template <class X>
  X* dalloc(size_t n) {
    void* ptr = nullptr;
    if (n == 0) n = 1;
    if (cudaMalloc(&ptr, n * sizeof(X)) != cudaSuccess) return nullptr;
    dptrs.push_back(ptr);
    dbytes += n * sizeof(X);
    return (X*)ptr;
  }
  template <class X>
  X* upload(const std::vector<X>& v) {
    X* d = dalloc<X>(v.size());
    if (d && !v.empty()) cudaMemcpy(d, v.data(), v.size() * sizeof(X), cudaMemcpyHostToDevice);
    return d;
  }
  int fail(int code, const std::string& msg) {
    err = msg;
    return code;
  }
  int cuda_check(const char* where) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(TMC_E_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
    return TMC_OK;
  }
  // The vertex pass and the pv-on-edge pass of a CRK4 stage read only the
  // stage's input state (gd and the edge set the previous pass prepared),
  // nothing the stage's cell pass writes, and the cell pass reads nothing
  // they write: between fork_side() and join_side() they run on st2 while
  // the cell pass runs on st.  The two branches fill each other's tails and
  // memory-latency gaps; the flux pass (and the closure, which reads E) come
  // after the join.  In a captured step this is a fork and a join in the
  // graph.
  cudaStream_t fork_side() {
    cudaEventRecord(fork_ev, st);
    cudaStreamWaitEvent(st2, fork_ev, 0);
    return st2;
  }
  void join_side() {
    cudaEventRecord(join_ev, st2);
    cudaStreamWaitEvent(st, join_ev, 0);
  }
};

namespace {

template <class T>
struct Engine : EngineBase {
  tmc_handle* h;
  double* gd[3] = {};
  T* iap[3] = {};
  T* q[3] = {};
  float* tendf = nullptr;  // FP32 path: gd tendency and topography shadows
  float* ghsf = nullptr;
  float* gdf[3] = {};  // FP32 path: shadows of gd and tracer mixing ratios per slot
  float* qr[3] = {};
  // edge quantities of a stage, double-buffered by stage parity: stage k reads
  // set (k-1)%2 while its flux pass prepares the next stage's set
  T* F[2] = {};
  T* gd_e[2] = {};
  T* u[2] = {};
  T* Fq[2] = {};
  double *gd_acc = nullptr, *gd_tend = nullptr, *ghs = nullptr;
  T* q_acc = nullptr;
  T *iap_acc = nullptr, *iap_tend = nullptr, *E = nullptr;
  T *pv_v = nullptr, *vor = nullptr, *gd_v = nullptr, *pv_c = nullptr, *v_e = nullptr, *pv_e = nullptr;
  T *dpv = nullptr, *pvf = nullptr, *dpvf = nullptr;  // conservative APVM
  // generic integrators: tendency slots (gd FP64; iap_u and tracer mass in T)
  double* tgd[4] = {};
  T* tiap[4] = {};
  T* tq[4] = {};
  double* psi = nullptr;  // adv model: stream function on vertices
  // adv model, CRK3: the wind of state(one), which time_integrate_CRK3 never
  // sets (it copies gd and iap_u only, time_scheme_mod.F90:78-79): zero
  T* u_one = nullptr;
  explicit Engine(tmc_handle* hh) : h(hh) {}

  // per-member sizes (members are stored one after another)
  size_t qsz() const { return (size_t)h->M.nc * (h->O.n_tracers > 0 ? h->O.n_tracers : 1); }
  size_t fqsz() const {
    return (h->O.n_tracers > 0 && h->O.tr_order >= 3) ? (size_t)h->M.ne * h->O.n_tracers : 1;
  }

  int alloc() override {
    const size_t M_ = (size_t)h->members;
    const size_t nc = h->M.nc * M_, ne = h->M.ne * M_, nv = h->M.nv * M_;
    const int nt = h->O.n_tracers;
    const size_t nq = qsz() * M_, nfq = fqsz() * M_;
    for (int i = 0; i < 3; ++i) {
      gd[i] = h->dalloc<double>(nc);
      iap[i] = h->dalloc<T>(ne);
      q[i] = h->dalloc<T>(nq);
    }
    gd_acc = h->dalloc<double>(nc);
    gd_tend = h->dalloc<double>(nc);
    q_acc = h->dalloc<T>(nq);
    ghs = h->dalloc<double>(nc);
    iap_acc = h->dalloc<T>(ne);
    iap_tend = h->dalloc<T>(ne);
    for (int i = 0; i < 2; ++i) {
      gd_e[i] = h->dalloc<T>(ne);
      u[i] = h->dalloc<T>(ne);
      F[i] = h->dalloc<T>(ne);
      Fq[i] = h->dalloc<T>(nfq);
    }
    E = h->dalloc<T>(nc);
    pv_v = h->dalloc<T>(nv);
    vor = h->dalloc<T>(nv);
    gd_v = h->dalloc<T>(nv);
    pv_c = h->dalloc<T>(nc);
    v_e = h->dalloc<T>(ne);
    pv_e = h->dalloc<T>(ne);
    if (!std::is_same<T, double>::value) {
      for (int i = 0; i < 3; ++i) {
        gdf[i] = h->dalloc<float>(nc);
        qr[i] = h->dalloc<float>(nq);
      }
    }
    if (!pv_e || !F[1] || !Fq[1]) return TMC_E_CUDA;
    if (h->O.pv_scheme == 2) {
      dpv = h->dalloc<T>(ne);
      pvf = h->dalloc<T>(ne);
      dpvf = h->dalloc<T>(ne);
      if (!dpvf) return TMC_E_CUDA;
    }
    if (h->generic) {
      const int ns = h->p.time_scheme == 1 ? 3 : (h->p.time_scheme == 3 ? 2 : 4);
      for (int i = 0; i < ns; ++i) {
        tgd[i] = h->dalloc<double>(nc);
        tiap[i] = h->adv ? nullptr : h->dalloc<T>(ne);
        tq[i] = h->dalloc<T>(nq);
        if (!tgd[i] || !tq[i] || (!h->adv && !tiap[i])) return TMC_E_CUDA;
      }
    }
    if (h->adv) {
      psi = h->dalloc<double>(nv);
      u_one = h->dalloc<T>(ne);
      if (!psi || !u_one) return TMC_E_CUDA;
      cudaMemset(u_one, 0, sizeof(T) * ne);
    }
    cudaMemset(ghs, 0, sizeof(double) * nc);
    if (!std::is_same<T, double>::value) {
      tendf = h->dalloc<float>(nc);
      ghsf = h->dalloc<float>(nc);
      if (!tendf || !ghsf) return TMC_E_CUDA;
      cudaMemset(ghsf, 0, sizeof(float) * nc);
    }
    cudaMemset(q[0], 0, sizeof(T) * nq);
    (void)nt;
    return TMC_OK;
  }

  // Buffers of CRK4 stage k (1..4; 0 for the stand-alone passes on slot 0).
  // State slots: stage inputs old, A, B, A; stage k writes the next stage's gd
  // (and tracers) into next_slot.  Edge quantities: set (k-1)%2, and stages
  // 1-3 prepare the next stage's set in their flux pass.
  StageIO<T> io(int k) const {
    StageIO<T> s{};
    static const int in_slot[5] = {0, 0, 1, 2, 1}, next_slot[5] = {-1, 1, 2, 1, -1};
    const int set = (k >= 1) ? (k - 1) % 2 : 0;
    const bool fuse = (k >= 1 && k <= 3);
    s.gd_in = gd[in_slot[k]];
    s.gd_old = gd[0];
    s.gd_next = next_slot[k] >= 0 ? gd[next_slot[k]] : nullptr;
    s.gd_acc = gd_acc;
    s.gd_tend = gd_tend;
    s.iap_in = iap[in_slot[k]];
    s.iap_old = iap[0];
    s.iap_next = next_slot[k] >= 0 ? iap[next_slot[k]] : nullptr;
    s.iap_acc = iap_acc;
    s.iap_tend = iap_tend;
    s.q_in = q[in_slot[k]];
    s.q_old = q[0];
    s.q_next = next_slot[k] >= 0 ? q[next_slot[k]] : nullptr;
    s.q_acc = q_acc;
    s.gd_e = gd_e[set];
    s.u = u[set];
    s.F = F[set];
    s.Fq = Fq[set];
    s.gd_e_nx = fuse ? gd_e[1 - set] : nullptr;
    s.u_nx = fuse ? u[1 - set] : nullptr;
    s.F_nx = fuse ? F[1 - set] : nullptr;
    s.Fq_nx = fuse ? Fq[1 - set] : nullptr;
    s.E = E;
    s.pv_v = pv_v;
    s.vor = vor;
    s.gd_v = gd_v;
    s.pv_c = pv_c;
    s.v_e = v_e;
    s.pv_e = pv_e;
    s.ghs = ghs;
    s.dpv = dpv;
    s.pvf = pvf;
    s.dpvf = dpvf;
    s.gdf_in = gdf[in_slot[k]];
    s.gdf_next = next_slot[k] >= 0 ? gdf[next_slot[k]] : nullptr;
    s.qr_in = qr[in_slot[k]];
    s.qr_next = next_slot[k] >= 0 ? qr[next_slot[k]] : nullptr;
    s.tendf = tendf;
    s.ghsf = ghsf;
    s.members = h->members;
    s.msc = h->M.nc;
    s.mse = h->M.ne;
    s.msv = h->M.nv;
    s.msq = (long long)qsz();
    s.msqe = (long long)fqsz();
    return s;
  }

  int launches_per_stage_passes() const {
    const bool v2c = (h->O.pv_scheme == 1 && h->O.apvm_weight != 0.0) || h->O.pv_scheme == 2;
    return 4 + (v2c ? 1 : 0) + (h->O.pv_scheme == 2 ? 4 : 0);
  }
  int launches_per_step() const override {
    if (!h->generic) return 4 * launches_per_stage_passes() + 3;
    // generic: spatial passes per evaluation (+ the edge preparation), state
    // updates (adv: + 2 wind kernels each), combination, finaliser, final update
    const int ts = h->p.time_scheme;
    const int evals = ts == 1 ? 3 : (ts == 3 ? 3 : 4);
    const int updates = ts == 1 ? 4 : (ts == 3 ? 3 : 4);
    const int per_eval = h->adv ? 2 : 1 + launches_per_stage_passes();
    const int per_update = h->adv ? 3 : 1;
    return evals * per_eval + updates * per_update + 2 + (h->adv ? 1 : 0);
  }

  // Edge preparation of state(old) into set 0 (+ the energy partials); needed
  // once after the state was set from outside, afterwards each step's final
  // pass keeps it current.
  void launch_prep() override {
    StageIO<T> s = io(0);
    launch_edge_prep<T>(h->M, h->O, s, h->P, true, h->bsp[P_FINAL], h->st);
  }

  // one CRK4 step (time_scheme_mod.F90:109-154); state(old) updated in place.
  // Requires set 0 prepared from state(old) (launch_prep or the previous step).
  void launch_step(bool diag, std::vector<cudaEvent_t>* flux_ev, size_t* ev_pos) override {
    if (h->generic) {
      launch_generic_step(diag);
      return;
    }
    const DevMesh& M = h->M;
    const ModelOpt& O = h->O;
    const double dt = O.dt;
    for (int k = first_stage; k <= 4; ++k) launch_stage(k, diag && k == 1, false, flux_ev, ev_pos);
    launch_finalize(h->P, h->counts, h->hm.totalArea, h->hm.sumAreaTriangle, dt, true, diag,
                    h->p.conserve_energy != 0, h->d_diag, h->st, 2, h->members);
    if (flux_ev && h->timed_pass == P_FINAL) cudaEventRecord((*flux_ev)[(*ev_pos)++], h->st);
    launch_final_update<T>(M, O, io(0), h->d_diag, h->P, h->bsp[P_FINAL], h->st);
    if (flux_ev && h->timed_pass == P_FINAL) cudaEventRecord((*flux_ev)[(*ev_pos)++], h->st);
  }

  // stage k of the fused CRK4 program; with no_tracers its cell pass leaves
  // the tracer terms out (launch_late_tracers adds them)
  void launch_stage(int k, bool dg, bool no_tracers, std::vector<cudaEvent_t>* flux_ev, size_t* ev_pos) {
    const DevMesh& M = h->M;
    const ModelOpt& O = h->O;
    const double dt = O.dt;
    const double adt[5] = {0.0, 0.5 * dt, 0.5 * dt, dt, 0.0};
    StageIO<T> s = io(k);
    s.vor = nullptr;  // vorticity and gd on vertices are kept only by the diagnostic pass
    s.gd_v = nullptr;
    RKStage rk{k, adt[k]};
    const int* b = h->bsp;
    auto mark = [&](int pass) {
      if (flux_ev && h->timed_pass == pass) cudaEventRecord((*flux_ev)[(*ev_pos)++], h->st);
    };
    // concurrent cell and vertex / pv-on-edge branches, except while passes
    // are timed one by one and for the conservative APVM (its global sums)
    const bool branch = !flux_ev && O.pv_scheme != 2;
    const cudaStream_t side = branch ? h->fork_side() : h->st;
    mark(P_CELL);
    if (no_tracers) {
      ModelOpt O0 = O;
      O0.n_tracers = 0;
      launch_cell<T>(M, O0, s, rk, h->P, dg, b[P_CELL], h->st);
    } else {
      launch_cell<T>(M, O, s, rk, h->P, dg, b[P_CELL], h->st);
    }
    mark(P_CELL);
    mark(P_VERTEX);
    launch_vertex<T>(M, O, s, h->P, dg, b[P_VERTEX], side);
    mark(P_VERTEX);
    mark(P_PV);
    launch_edge_pv<T>(M, O, s, b[P_PV], side);
    if (branch) h->join_side();
    if (O.pv_scheme == 2) launch_cons_apvm<T>(M, O, s, h->P, h->d_diag, b[P_VERTEX], h->st);
    launch_closure_pass(s, k);
    mark(P_PV);
    mark(P_FLUX);
    launch_edge_flux<T>(M, O, s, rk, h->P, b[P_FLUX], h->st);
    mark(P_FLUX);
  }

  bool can_split() const override {
    const int n = h->O.n_tracers;
    return std::is_same<T, float>::value && !h->generic && h->members <= 1 && h->O.tr_order == 2 &&
           (n == 1 || n == 2 || n == 4);
  }
  void launch_stage1_early(bool diag) override { launch_stage(1, diag, true, nullptr, nullptr); }
  void gather_tracers_on(const double* raw_q, cudaStream_t s) override {
    if constexpr (std::is_same<T, float>::value) {
      for (int k = 0; k < h->O.n_tracers; ++k)
        launch_gather<T>(h->M.nc, raw_q + (size_t)k * h->M.nc, h->d_cell_n2o, q[0] + oq() + (size_t)k * h->M.nc,
                         s);
      launch_shadows(h->M.nc, h->O.n_tracers, gd[0] + oc(), q[0] + oq(), nullptr, qr[0] + oq(), s);
    }
  }
  // stage 1's tracer terms: its F (edge set 0) and next gd (slot 1) stay as
  // the stage left them until stage 2
  void launch_late_tracers() override {
    launch_tracers_fast<T>(h->M, h->O, io(1), RKStage{1, 0.5 * h->O.dt}, h->bsp[P_CELL], h->st);
  }

  // the learned closure on this stage's pv_edge (FP32 path)
  // (in every stage, or in stage 1 with its output held for stages 2-4)
  void launch_closure_pass(const StageIO<T>& s, int stage) {
    if constexpr (std::is_same<T, float>::value) {
      if (h->closure) {
        const int mode = h->closure_every_stage ? 0 : (stage == 1 ? 1 : 2);
        ClosureArgs a{&h->closure_net, h->d_member_on, h->d_closure_err, h->sms, h->d_closure_dq, mode};
        launch_closure(h->M, s, a, h->st);
      }
    }
  }

  // features of state(old) of the selected member (after a diagnostic pass and
  // the pv-on-edge pass), internal edge order
  void closure_features(float* feat, float* pv) {
    if constexpr (std::is_same<T, float>::value) {
      launch_diag_pass(false);
      StageIO<T> s = io(0);
      launch_edge_pv<T>(h->M, h->O, s, h->bsp[P_PV], h->st);
      if (h->O.pv_scheme == 2) launch_cons_apvm<T>(h->M, h->O, s, h->P, h->d_diag, h->bsp[P_VERTEX], h->st);
      launch_closure_features(h->M, s, h->cur, feat, pv, h->st);
    }
  }

  void history_dev(double* uo, double* zon, double* mer, double* hc, double* div, double* pv, double* vor,
                   double* scratch_e) override {
    launch_diag_pass(false);  // gd_edge, u, pv and vorticity of state(old)
    const T* ue = u[0] + oe();
    if (uo) launch_to_f64<T>((size_t)h->M.ne, ue, uo, h->st);
    if (zon || mer) launch_reconstruct<T>(h->M, ue, nullptr, nullptr, nullptr, zon, mer, h->st);
    if (hc) launch_h_field(h->M.nc, gd[0] + oc(), ghs + oc(), h->p.g, hc, h->st);
    if (div) {
      launch_to_f64<T>((size_t)h->M.ne, ue, scratch_e, h->st);
      launch_op(OP_DIV, h->M, h->O, scratch_e, nullptr, nullptr, div, 0, 0, 0.0, 0.0, h->bs, h->st);
    }
    if (pv) launch_to_f64<T>((size_t)h->M.nv, pv_v + ov(), pv, h->st);
    if (vor) launch_to_f64<T>((size_t)h->M.nv, this->vor + ov(), vor, h->st);
  }

  // ---- generic integrator program (time_scheme_mod.F90:65-107 CRK3,
  // :109-154 CRK4, :156-184 PC2; the adv model's spatial_operators and
  // update_state, tmcore_adv_mod.F90:78-97).  State slots: old = 0 (also the
  // stage state "one", which the schemes only read), scratch 1 and 2.

  // spatial_operators of state slot xs into tendency slot ts (unfused passes,
  // edge set 0); the adv model takes the wind of slot xs unless `wind` is given
  void gen_spatial(int xs, int ts, const T* wind = nullptr) {
    const DevMesh& M = h->M;
    const ModelOpt& O = h->O;
    if constexpr (std::is_same<T, double>::value) {
      if (h->adv) {
        launch_adv_spatial(M, O, gd[xs], wind ? wind : iap[xs], gd_e[0], F[0], tgd[ts], h->bs, h->st);
        return;
      }
    }
    StageIO<T> s = io(0);
    s.gd_in = gd[xs];
    s.iap_in = iap[xs];
    s.q_in = q[xs];
    s.gdf_in = gdf[xs];
    s.qr_in = qr[xs];
    s.gd_tend = tgd[ts];
    s.iap_tend = tiap[ts];
    s.q_acc = tq[ts];  // mode 0 writes the tracer tendency here
    s.vor = nullptr;
    s.gd_v = nullptr;
    RKStage rk{0, 0.0};
    launch_edge_prep<T>(M, O, s, h->P, false, h->bs, h->st);
    launch_cell<T>(M, O, s, rk, h->P, false, h->bs, h->st);
    launch_vertex<T>(M, O, s, h->P, false, h->bs, h->st);
    launch_edge_pv<T>(M, O, s, h->bs, h->st);
    if (O.pv_scheme == 2) launch_cons_apvm<T>(M, O, s, h->P, h->d_diag, h->bs, h->st);
    launch_edge_flux<T>(M, O, s, rk, h->P, h->bs, h->st);
  }

  // update_state: slot `to` = slot `from` + coef * tendency slot ts, coef the
  // host value a_dt or *coef_dev; the adv model then re-sets the wind of the
  // new state at elapsed + coef (tmcore_adv_mod.F90:87-97)
  void gen_update(int ts, int from, int to, double a_dt, const double* coef_dev) {
    UpdateArgs<T> a{};
    a.gd_o = gd[from];
    a.gd_n = gd[to];
    a.tgd = tgd[ts];
    if (!h->adv) {
      a.iap_o = iap[from];
      a.iap_n = iap[to];
      a.tiap = tiap[ts];
    }
    a.q_o = q[from];
    a.q_n = q[to];
    a.tq = tq[ts];
    a.gdf_n = gdf[to];
    a.qr_n = qr[to];
    a.a_dt = a_dt;
    a.coef_dev = coef_dev;
    launch_update<T>(h->M, h->O.n_tracers, a, h->bs, h->st);
    if constexpr (std::is_same<T, double>::value) {
      if (h->adv)
        launch_adv_wind(h->M, h->p.adv_wind, h->p.radius, h->d_latV, h->d_lonV, h->d_diag + 11, a_dt, coef_dev, psi,
                        iap[to], h->st);
    }
  }

  void launch_generic_step(bool diag) {
    const double dt = h->O.dt;
    const int ts = h->p.time_scheme;
    if (diag) {
      // invariants of state(old), reduced together with beta below
      if (h->adv)
        launch_mass_only(h->M, gd[0], h->P, h->bs, h->st);
      else
        launch_diag_pass(false);
    }
    CombineArgs<T> c{};
    if (ts == 2) {  // CRK4: two -> 1, three -> 2, four -> 1
      gen_spatial(0, 0);
      gen_update(0, 0, 1, 0.5 * dt, nullptr);
      gen_spatial(1, 1);
      gen_update(1, 0, 2, 0.5 * dt, nullptr);
      gen_spatial(2, 2);
      gen_update(2, 0, 1, dt, nullptr);
      gen_spatial(1, 3);
    } else if (ts == 1) {  // CRK3: two -> 1, three -> 2
      gen_spatial(0, 0, u_one);
      gen_update(0, 0, 1, 0.5 * dt, nullptr);
      gen_spatial(1, 1);
      gen_update(0, 0, 2, -dt, nullptr);
      gen_update(1, 2, 2, 2.0 * dt, nullptr);
      gen_spatial(2, 2);
    } else {  // PC2: new -> 1; tend(old) -> 0, tend(new) -> 1
      gen_spatial(0, 0);
      gen_update(0, 0, 1, 0.5 * dt, nullptr);
      gen_spatial(1, 0);
      gen_update(0, 0, 1, 0.5 * dt, nullptr);
      gen_spatial(1, 1);
    }
    for (int k = 0; k < 4; ++k) {
      c.tgd[k] = tgd[k];
      c.tiap[k] = tiap[k];
      c.tq[k] = tq[k];
    }
    launch_combine<T>(h->M, h->O.n_tracers, ts, c, h->P, h->bs, h->st);
    launch_finalize(h->P, h->gen_counts, h->hm.totalArea, h->hm.sumAreaTriangle, dt, true, diag,
                    h->p.conserve_energy != 0, h->d_diag, h->st, ts);
    // new = old + beta dt t_new, in place (t_new: slot 0, PC2 slot 1)
    gen_update(ts == 3 ? 1 : 0, 0, 0, 0.0, h->d_diag + 9);
    if (h->adv) launch_adv_advance(h->d_diag + 11, dt, h->st);
  }

  void adv_set_initial_dev(const double* raw_q) override {
    if constexpr (std::is_same<T, double>::value) {
      launch_gather<double>(h->M.nc, raw_q, h->d_cell_n2o, gd[0], h->st);
      cudaMemsetAsync(h->d_diag + 11, 0, sizeof(double), h->st);
      launch_adv_wind(h->M, h->p.adv_wind, h->p.radius, h->d_latV, h->d_lonV, h->d_diag + 11, 0.0, nullptr, psi,
                      iap[0], h->st);
    }
  }
  void adv_get_dev(double* raw_q, double* raw_u) override {
    if (raw_q) launch_scatter<double>(h->M.nc, gd[0], h->d_cell_n2o, raw_q, h->st);
    if (raw_u) launch_scatter<T>(h->M.ne, iap[0], h->d_edge_n2o, raw_u, h->st);
  }

  // diagnostics of state(old): gd_edge, u, gd/pv/vor on vertices, invariants
  void launch_diag_pass(bool finalize) override {
    if (h->adv) {
      launch_mass_only(h->M, gd[0], h->P, h->bs, h->st);
      if (finalize)
        launch_finalize(h->P, h->gen_counts, h->hm.totalArea, h->hm.sumAreaTriangle, h->O.dt, false, true, false,
                        h->d_diag, h->st);
      return;
    }
    StageIO<T> s = io(0);
    RKStage rk{0, 0.0};
    launch_edge_prep<T>(h->M, h->O, s, h->P, true, h->bsp[P_FINAL], h->st);
    launch_cell<T>(h->M, h->O, s, rk, h->P, true, h->bsp[P_CELL], h->st);
    launch_vertex<T>(h->M, h->O, s, h->P, true, h->bsp[P_VERTEX], h->st);
    if (finalize)
      launch_finalize(h->P, h->counts, h->hm.totalArea, h->hm.sumAreaTriangle, h->O.dt, false, true,
                      h->p.conserve_energy != 0, h->d_diag, h->st, 2, h->members);
  }

  // spatial_operators on the state in slot 1 -> gd_tend, iap_tend (uses edge set 0)
  void launch_spatial_only() override {
    StageIO<T> s = io(0);
    s.gd_in = gd[1];
    s.iap_in = iap[1];
    s.q_in = q[1];
    s.gdf_in = gdf[1];
    s.qr_in = qr[1];
    RKStage rk{0, 0.0};
    launch_edge_prep<T>(h->M, h->O, s, h->P, false, h->bs, h->st);
    launch_cell<T>(h->M, h->O, s, rk, h->P, false, h->bs, h->st);
    launch_vertex<T>(h->M, h->O, s, h->P, false, h->bs, h->st);
    launch_edge_pv<T>(h->M, h->O, s, h->bs, h->st);
    if (h->O.pv_scheme == 2) launch_cons_apvm<T>(h->M, h->O, s, h->P, h->d_diag, h->bs, h->st);
    launch_edge_flux<T>(h->M, h->O, s, rk, h->P, h->bs, h->st);
  }

  void state_slot0(void** g, void** i, void** qq, void** gh) override {
    *g = gd[0];
    *i = iap[0];
    *qq = q[0];
    *gh = ghs;
  }
  void refresh_all_shadows() override {
    if constexpr (!std::is_same<T, double>::value) {
      const int save = h->cur;
      for (int m = 0; m < h->members; ++m) {
        h->cur = m;
        refresh_shadows(0);
      }
      h->cur = save;
    }
  }

  // offsets of the selected member's arrays
  size_t oc() const { return (size_t)h->cur * h->M.nc; }
  size_t oe() const { return (size_t)h->cur * h->M.ne; }
  size_t ov() const { return (size_t)h->cur * h->M.nv; }
  size_t oq() const { return (size_t)h->cur * qsz(); }

  void gather_field(int which, const double* raw) override {
    if (which == F_GD)
      launch_gather<double>(h->M.nc, raw, h->d_cell_n2o, gd[0] + oc(), h->st);
    else if (which == F_IAP)
      launch_gather<T>(h->M.ne, raw, h->d_edge_n2o, iap[0] + oe(), h->st);
    else
      for (int k = 0; k < h->O.n_tracers; ++k)
        launch_gather<T>(h->M.nc, raw + (size_t)k * h->M.nc, h->d_cell_n2o, q[0] + oq() + (size_t)k * h->M.nc,
                         h->st);
  }
  void set_state_dev(const double* raw_gd, const double* raw_iap) override {
    launch_gather<double>(h->M.nc, raw_gd, h->d_cell_n2o, gd[0] + oc(), h->st);
    launch_gather<T>(h->M.ne, raw_iap, h->d_edge_n2o, iap[0] + oe(), h->st);
    refresh_shadows(0);
  }
  void refresh_shadows(int slot, bool tracers = true) override {
    if constexpr (!std::is_same<T, double>::value)
      launch_shadows(h->M.nc, tracers ? h->O.n_tracers : 0, gd[slot] + oc(), q[slot] + oq(), gdf[slot] + oc(),
                     qr[slot] + oq(), h->st);
  }
  void get_field(int which, double* raw) override {
    switch (which) {
      case F_GD: launch_scatter<double>(h->M.nc, gd[0] + oc(), h->d_cell_n2o, raw, h->st); break;
      case F_IAP: launch_scatter<T>(h->M.ne, iap[0] + oe(), h->d_edge_n2o, raw, h->st); break;
      case F_U: launch_scatter<T>(h->M.ne, u[0] + oe(), h->d_edge_n2o, raw, h->st); break;
      case F_PV_V: launch_scatter<T>(h->M.nv, pv_v + ov(), h->d_vert_n2o, raw, h->st); break;
      case F_VOR: launch_scatter<T>(h->M.nv, vor + ov(), h->d_vert_n2o, raw, h->st); break;
      case F_TEND_GD: launch_scatter<double>(h->M.nc, gd_tend + oc(), h->d_cell_n2o, raw, h->st); break;
      case F_TEND_IAP: launch_scatter<T>(h->M.ne, iap_tend + oe(), h->d_edge_n2o, raw, h->st); break;
    }
  }
  void set_iap_from_u(const double* ge_new, const double* u_new) override {
    launch_iap_from_u<T>(h->M.ne, ge_new, u_new, iap[0] + oe(), h->st);
  }
  void set_tracers_dev(const double* raw_q) override {
    for (int k = 0; k < h->O.n_tracers; ++k)
      launch_gather<T>(h->M.nc, raw_q + (size_t)k * h->M.nc, h->d_cell_n2o, q[0] + oq() + (size_t)k * h->M.nc,
                       h->st);
    refresh_shadows(0);
  }
  void get_tracers_dev(double* raw_q) override {
    for (int k = 0; k < h->O.n_tracers; ++k)
      launch_scatter<T>(h->M.nc, q[0] + oq() + (size_t)k * h->M.nc, h->d_cell_n2o, raw_q + (size_t)k * h->M.nc,
                        h->st);
  }
  void set_ghs_dev(const double* raw) override {
    launch_gather<double>(h->M.nc, raw, h->d_cell_n2o, ghs + oc(), h->st);
    if (ghsf) launch_to_f32((size_t)h->M.nc, ghs + oc(), ghsf + oc(), h->st);
  }
  void copy_tracers_to_slot1() {
    cudaMemcpyAsync(q[1], q[0], sizeof(T) * h->M.nc * (h->O.n_tracers > 0 ? h->O.n_tracers : 1),
                    cudaMemcpyDeviceToDevice, h->st);
  }
};

// Member-innermost ensemble engine (tmc_params.member_layout = 1): the
// same CRK4 stage program as Engine<float> on arrays [element][member]
// (tmc_ensemble.cuh).  State slots old, A, B for gd (double-float: the FP32
// h halves are what the stencils read); iap_u lives in slot old only (the
// fused stages keep the next stage's iap_u in registers and store its edge
// preparation instead).
struct EnsEngine : EngineBase {
  tmc_handle* h;
  ens::Dims D{};
  ens::Partials EP{};
  float* gd[3] = {};  // FF: [2][nCells * M]
  float* iap0 = nullptr;
  float* gd_acc = nullptr;  // FF
  double* ghs = nullptr;
  float *iap_acc = nullptr, *iap_tend = nullptr, *tendf = nullptr, *ghsf = nullptr;
  float* gd_e[2] = {};
  float* u[2] = {};
  float* F[2] = {};
  float *E = nullptr, *pv_v = nullptr, *vor = nullptr, *gd_v = nullptr, *pv_e = nullptr;
  float* pv_c = nullptr;  // pv on cells (the learned closure's features)
  float *invA_hl = nullptr, *A_hl = nullptr;
  float *cdv = nullptr, *cae = nullptr, *vdc = nullptr;
  ens::Upwind up{};  // pv_scheme 3: the vertex fit stencils (width 0 otherwise)
  explicit EnsEngine(tmc_handle* hh) : h(hh) {}
  const ens::Upwind* upwind() const { return up.width ? &up : nullptr; }

  int alloc() override {
    const size_t M_ = (size_t)h->members;
    const size_t nc = h->M.nc * M_, ne = h->M.ne * M_, nv = h->M.nv * M_;
    D.M = h->members;
    D.G = (h->members + 31) / 32;
    if (!ens::lanes_for(h->members, h->p.member_lanes, &D.V, &D.LPE)) return TMC_E_ARG;
    D.slots_c = ens::slots_for(h->M.nc);
    D.slots_e = ens::slots_for(h->M.ne);
    D.slots_v = ens::slots_for(h->M.nv);
    EP.cap = std::max(D.slots_c, std::max(D.slots_e, D.slots_v));
    EP.M = D.M;
    EP.sf = h->dalloc<float>((size_t)(R_44_E + 1) * EP.cap * M_);
    EP.sd = h->dalloc<double>((size_t)(R_AV - R_MASS + 1) * EP.cap * M_);
    for (int i = 0; i < 3; ++i) gd[i] = h->dalloc<float>(2 * nc);
    iap0 = h->dalloc<float>(ne);
    gd_acc = h->dalloc<float>(2 * nc);
    ghs = h->dalloc<double>(nc);
    ghsf = h->dalloc<float>(nc);
    tendf = h->dalloc<float>(nc);
    iap_acc = h->dalloc<float>(ne);
    iap_tend = h->dalloc<float>(ne);
    for (int i = 0; i < 2; ++i) {
      gd_e[i] = h->dalloc<float>(ne);
      u[i] = h->dalloc<float>(ne);
      F[i] = h->dalloc<float>(ne);
    }
    E = h->dalloc<float>(nc);
    pv_v = h->dalloc<float>(nv);
    vor = h->dalloc<float>(nv);
    gd_v = h->dalloc<float>(nv);
    pv_e = h->dalloc<float>(ne);
    pv_c = h->dalloc<float>(nc);
    // 1 / areaCell and areaCell as double-float pairs [2][nCells]
    const int ncell = h->M.nc;
    std::vector<float> ia(2 * (size_t)ncell), a(2 * (size_t)ncell);
    for (int c = 0; c < ncell; ++c) {
      const double A = h->hm.areaCell[c], iA = 1.0 / A;
      ia[c] = (float)iA;
      ia[ncell + c] = (float)(iA - (double)ia[c]);
      a[c] = (float)A;
      a[ncell + c] = (float)(A - (double)a[c]);
    }
    invA_hl = h->upload(ia);
    A_hl = h->upload(a);
    // the edge metrics the cell and vertex passes read per slot, gathered once
    // here (FP32, as Engine<float> reads them), so staging them is one
    // coalesced load instead of an index load and a dependent gather
    const HostMesh& hm = h->hm;
    const int nvert = h->M.nv, me = hm.me;
    std::vector<float> v_cdv((size_t)me * ncell), v_cae((size_t)me * ncell), v_vdc(3 * (size_t)nvert);
    for (size_t k = 0; k < v_cdv.size(); ++k) {
      const int e = hm.edgesOnCell[k];
      v_cdv[k] = (float)hm.dvEdge[e];
      v_cae[k] = (float)hm.areaEdge[e];
    }
    for (size_t k = 0; k < v_vdc.size(); ++k) v_vdc[k] = (float)hm.dcEdge[hm.edgesOnVertex[k]];
    cdv = h->upload(v_cdv);
    cae = h->upload(v_cae);
    vdc = h->upload(v_vdc);
    if (h->O.pv_scheme == 3) {
      // the weights in FP32, as the FP32 single-model kernel converts them
      std::vector<float> wf(hm.vert2.w.begin(), hm.vert2.w.end());
      up.count = h->M.vert2.count;
      up.idx = h->M.vert2.idx;
      up.w = h->upload(wf);
      up.width = hm.vert2.width;
      up.coef2 = (float)h->O.vert_coef2;
      if (!up.w || !up.count || !up.idx) return TMC_E_CUDA;
    }
    if (!EP.sf || !EP.sd || !pv_e || !pv_c || !F[1] || !gd_v || !invA_hl || !A_hl || !cdv || !cae || !vdc)
      return TMC_E_CUDA;
    cudaMemset(ghs, 0, sizeof(double) * nc);
    cudaMemset(ghsf, 0, sizeof(float) * nc);
    return TMC_OK;
  }

  // buffers of CRK4 stage k (1..4; 0: the stand-alone passes on state(old)),
  // the slot program of Engine::io
  ens::IO io(int k) const {
    static const int in_slot[5] = {0, 0, 1, 2, 1}, next_slot[5] = {-1, 1, 2, 1, -1};
    const int set = (k >= 1) ? (k - 1) % 2 : 0;
    const bool fuse = (k >= 1 && k <= 3);
    ens::IO s{};
    s.gd_in = gd[in_slot[k]];
    s.gd_old = gd[0];
    s.gd_next = next_slot[k] >= 0 ? gd[next_slot[k]] : nullptr;
    s.gd_acc = gd_acc;
    s.iap_in = iap0;
    s.iap_old = iap0;
    s.iap_next = nullptr;
    s.iap_acc = iap_acc;
    s.iap_tend = iap_tend;
    s.tendf = tendf;
    s.ghsf = ghsf;
    s.gd_e = gd_e[set];
    s.u = u[set];
    s.F = F[set];
    s.gd_e_nx = fuse ? gd_e[1 - set] : nullptr;
    s.u_nx = fuse ? u[1 - set] : nullptr;
    s.F_nx = fuse ? F[1 - set] : nullptr;
    s.E = E;
    s.pv_v = pv_v;
    s.vor = vor;
    s.gd_v = gd_v;
    s.pv_e = pv_e;
    s.invA_hl = invA_hl;
    s.A_hl = A_hl;
    s.cdv = cdv;
    s.cae = cae;
    s.vdc = vdc;
    s.ffs = (size_t)h->M.nc * D.M;
    return s;
  }

  int launches_per_step() const override {
    const int closure = !h->closure ? 0 : (h->closure_every_stage ? 4 * 2 : 2 + 3);
    return 4 * 4 + 2 + 2 + closure;
  }

  void launch_prep() override { ens::launch_edge_prep(h->M, D, io(0), EP, true, h->bsp[P_FINAL], h->st); }

  void launch_step(bool diag, std::vector<cudaEvent_t>* ev, size_t* pos) override {
    const DevMesh& M = h->M;
    const double dt = h->O.dt;
    const double adt[5] = {0.0, 0.5 * dt, 0.5 * dt, dt, 0.0};
    const int* b = h->bsp;
    auto mark = [&](int pass) {
      if (ev && h->timed_pass == pass) cudaEventRecord((*ev)[(*pos)++], h->st);
    };
    for (int k = 1; k <= 4; ++k) {
      ens::IO s = io(k);
      s.vor = nullptr;  // kept only by the diagnostic pass
      s.gd_v = nullptr;
      const bool dg = diag && k == 1;
      const RKStage rk{k, adt[k]};
      // concurrent cell and vertex / pv-on-edge branches (tmc_handle::fork_side),
      // except while passes are timed one by one
      const cudaStream_t side = ev ? h->st : h->fork_side();
      mark(P_CELL);
      ens::launch_cell(M, D, s, rk, EP, dg, b[P_CELL], h->st);
      mark(P_CELL);
      mark(P_VERTEX);
      ens::launch_vertex(M, D, s, EP, dg, b[P_VERTEX], side);
      mark(P_VERTEX);
      mark(P_PV);
      ens::launch_edge_pv(M, D, s, upwind(), b[P_PV], side);
      if (!ev) h->join_side();
      if (h->closure) {
        // the learned closure on this stage's pv_edge: in every stage, or in
        // stage 1 with its output held for stages 2-4
        const int mode = h->closure_every_stage ? 0 : (k == 1 ? 1 : 2);
        if (mode != 2) ens::launch_v2c(M, D, s, pv_c, h->st);
        const ClosureArgs a{&h->closure_net, h->d_member_on, h->d_closure_err, h->sms, h->d_closure_dq, mode};
        ens::launch_closure(M, D, s, pv_c, a, h->st);
      }
      mark(P_PV);
      mark(P_FLUX);
      ens::launch_edge_flux(M, D, s, rk, EP, b[P_FLUX], h->st);
      mark(P_FLUX);
    }
    ens::launch_finalize(D, EP, true, diag, h->p.conserve_energy != 0, h->hm.totalArea, h->hm.sumAreaTriangle, dt,
                         h->d_diag, h->st);
    mark(P_FINAL);
    ens::launch_final(M, D, io(0), h->d_diag, EP, b[P_FINAL], h->st);
    mark(P_FINAL);
  }

  // gd_edge, u, pv, vorticity and invariants of state(old)
  void launch_diag_pass(bool finalize) override {
    const ens::IO s = io(0);
    ens::launch_edge_prep(h->M, D, s, EP, true, h->bsp[P_FINAL], h->st);
    ens::launch_cell_diag(h->M, D, s, EP, h->bsp[P_CELL], h->st);
    ens::launch_vertex(h->M, D, s, EP, true, h->bsp[P_VERTEX], h->st);
    if (finalize)
      ens::launch_finalize(D, EP, false, true, false, h->hm.totalArea, h->hm.sumAreaTriangle, h->O.dt, h->d_diag,
                           h->st);
  }
  void launch_spatial_only() override {}  // tmc_spatial_operators needs members <= 1

  void set_state_dev(const double* raw_gd, const double* raw_iap) override {
    ens::launch_gather_ff(h->M.nc, D.M, h->cur, raw_gd, h->d_cell_n2o, gd[0], h->st);
    ens::launch_gather_f32(h->M.ne, D.M, h->cur, raw_iap, h->d_edge_n2o, iap0, h->st);
  }
  void gather_field(int which, const double* raw) override {
    if (which == F_GD)
      ens::launch_gather_ff(h->M.nc, D.M, h->cur, raw, h->d_cell_n2o, gd[0], h->st);
    else if (which == F_IAP)
      ens::launch_gather_f32(h->M.ne, D.M, h->cur, raw, h->d_edge_n2o, iap0, h->st);
  }
  void get_field(int which, double* raw) override {
    const int m = h->cur, Mm = D.M;
    switch (which) {
      case F_GD: ens::launch_scatter_ff(h->M.nc, Mm, m, gd[0], h->d_cell_n2o, raw, h->st); break;
      case F_IAP: ens::launch_scatter_f32(h->M.ne, Mm, m, iap0, h->d_edge_n2o, raw, h->st); break;
      case F_U: ens::launch_scatter_f32(h->M.ne, Mm, m, u[0], h->d_edge_n2o, raw, h->st); break;
      case F_PV_V: ens::launch_scatter_f32(h->M.nv, Mm, m, pv_v, h->d_vert_n2o, raw, h->st); break;
      case F_VOR: ens::launch_scatter_f32(h->M.nv, Mm, m, vor, h->d_vert_n2o, raw, h->st); break;
      default: break;  // tendencies: tmc_spatial_operators needs members <= 1
    }
  }
  void set_iap_from_u(const double* ge_new, const double* u_new) override {
    ens::launch_iap_from_u(h->M.ne, D.M, h->cur, ge_new, u_new, iap0, h->st);
  }
  void set_tracers_dev(const double*) override {}  // member_layout 1 has no tracers
  void get_tracers_dev(double*) override {}
  void refresh_shadows(int, bool) override {}  // the h halves of gd are its FP32 values
  void set_ghs_dev(const double* raw) override {
    ens::launch_gather_f64(h->M.nc, D.M, h->cur, raw, h->d_cell_n2o, ghs, h->st);
    ens::launch_to_f32(h->M.nc, D.M, h->cur, ghs, ghsf, h->st);
  }
  void adv_set_initial_dev(const double*) override {}
  void adv_get_dev(double*, double*) override {}
  void state_slot0(void** g, void** i, void** q, void** gh) override {
    *g = gd[0];
    *i = iap0;
    *q = nullptr;  // no tracers
    *gh = ghs;
  }
  void refresh_all_shadows() override {}
  // the closure's features of state(old) of the selected member: its edge
  // preparation, E (a cell pass without update), pv on vertices, edges and cells
  void closure_features(float* feat, float* pv) override {
    launch_diag_pass(false);
    const ens::IO s = io(0);
    ens::launch_cell(h->M, D, s, RKStage{0, 0.0}, EP, false, h->bsp[P_CELL], h->st);
    ens::launch_edge_pv(h->M, D, s, upwind(), h->bsp[P_PV], h->st);
    ens::launch_v2c(h->M, D, s, pv_c, h->st);
    ens::launch_closure_features(h->M, D, s, pv_c, h->cur, feat, pv, h->st);
  }

  // history fields of the selected member: its u, gd and ghs copied out of
  // the member-innermost arrays, then the single-model kernels
  void history_dev(double* uo, double* zon, double* mer, double* hc, double* div, double* pv, double* vo,
                   double* scratch_e) override {
    launch_diag_pass(false);
    const int m = h->cur, Mm = D.M, nc = h->M.nc, ne = h->M.ne, nv = h->M.nv;
    ens::launch_extract_f32(ne, Mm, m, u[0], scratch_e, h->st);
    if (uo) cudaMemcpyAsync(uo, scratch_e, sizeof(double) * ne, cudaMemcpyDeviceToDevice, h->st);
    if (zon || mer) launch_reconstruct<double>(h->M, scratch_e, nullptr, nullptr, nullptr, zon, mer, h->st);
    if (hc) {
      ens::launch_extract_ff(nc, Mm, m, gd[0], h->op_a, h->st);
      ens::launch_extract_f64(nc, Mm, m, ghs, h->op_b, h->st);
      launch_h_field(nc, h->op_a, h->op_b, h->p.g, hc, h->st);
    }
    if (div) launch_op(OP_DIV, h->M, h->O, scratch_e, nullptr, nullptr, div, 0, 0, 0.0, 0.0, h->bs, h->st);
    if (pv) ens::launch_extract_f32(nv, Mm, m, pv_v, pv, h->st);
    if (vo) ens::launch_extract_f32(nv, Mm, m, vor, vo, h->st);
  }
};

DStencil upload_stencil(tmc_handle* h, const Stencil& S) {
  DStencil d{};
  d.width = S.width;
  if (S.width > 0) {
    d.count = h->upload(S.count);
    d.idx = h->upload(S.idx);
    d.w = h->upload(S.w);
  }
  return d;
}

// the step program from stage first_stage on, captured as one graph
int build_graph(tmc_handle* h, bool diag, cudaGraphExec_t* out, int first_stage = 1) {
  cudaGraph_t g = nullptr;
  if (cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return h->cuda_check("cudaStreamBeginCapture");
  h->eng->first_stage = first_stage;
  h->eng->launch_step(diag, nullptr, nullptr);
  h->eng->first_stage = 1;
  if (cudaStreamEndCapture(h->st, &g) != cudaSuccess) return h->cuda_check("cudaStreamEndCapture");
  cudaError_t e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return h->fail(TMC_E_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
  return TMC_OK;
}

// partial counts per region: the grid of the passes that write it
void set_counts(tmc_handle* h) {
  const int bc = grid_for(h->M.nc, h->bsp[P_CELL]), bf = grid_for(h->M.ne, h->bsp[P_FLUX]),
            bfin = grid_for(h->M.ne, h->bsp[P_FINAL]), bv = grid_for(h->M.nv, h->bsp[P_VERTEX]);
  static const int cells[6] = {R_IP_C, R_IP_C + 2, R_IP_C + 4, R_44_C, R_MASS, R_EN_C};
  static const int edges[4] = {R_IP_E, R_IP_E + 2, R_IP_E + 4, R_44_E};
  static const int verts[5] = {R_PE, R_AV, R_C1, R_C2, R_C3};
  for (int r : cells) h->counts[r] = bc;
  for (int r : edges) h->counts[r] = bf;
  h->counts[R_EN_E] = bfin;
  for (int r : verts) h->counts[r] = bv;
}

void ensure_prep(tmc_handle* h) {
  if (h->generic) return;  // the generic program prepares every evaluation itself
  if (!h->prep_valid) {
    h->eng->launch_prep();
    h->prep_valid = true;
  }
}

int launch_one_step(tmc_handle* h) {
  ensure_prep(h);
  const bool diag = h->p.diag_every > 0 && (h->step_count % h->p.diag_every) == 0;
  if (h->p.use_graph) {
    cudaGraphExec_t* g = diag ? &h->g_step_diag : &h->g_step;
    if (!*g) {
      int rc = build_graph(h, diag, g);
      if (rc) return rc;
    }
    if (cudaGraphLaunch(*g, h->st) != cudaSuccess) return h->cuda_check("cudaGraphLaunch");
  } else {
    h->eng->launch_step(diag, nullptr, nullptr);
  }
  h->step_count++;
  return h->cuda_check("step");
}

// One step split around the late arrival of the tracers (tmc_time_integrate):
// stage 1 without its tracer terms, then tracers_in() (which makes the stream
// wait for the tracers and their FP32 ratios), the stage's tracer terms, and
// stages 2-4 with the final update as one graph.  Same results as
// launch_one_step.
template <class F>
int launch_one_step_split(tmc_handle* h, F&& tracers_in) {
  ensure_prep(h);
  const bool diag = h->p.diag_every > 0 && (h->step_count % h->p.diag_every) == 0;
  h->eng->launch_stage1_early(diag);
  tracers_in();
  h->eng->launch_late_tracers();
  if (h->p.use_graph) {
    cudaGraphExec_t* g = &h->g_tail[diag ? 1 : 0];
    if (!*g) {
      int rc = build_graph(h, diag, g, 2);
      if (rc) return rc;
    }
    if (cudaGraphLaunch(*g, h->st) != cudaSuccess) return h->cuda_check("cudaGraphLaunch");
  } else {
    h->eng->first_stage = 2;
    h->eng->launch_step(diag, nullptr, nullptr);
    h->eng->first_stage = 1;
  }
  h->step_count++;
  return h->cuda_check("step");
}

int sync(tmc_handle* h, const char* where) {
  cudaError_t e = cudaStreamSynchronize(h->st);
  if (e != cudaSuccess) return h->fail(TMC_E_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
  return TMC_OK;
}

// The closure network's timeout flag (set by k_closure / k_closure_inner when
// a tensor-core completion wait ran out, after which that tile group skipped
// its remaining rows): queue its read into *flag and its reset on the
// handle's stream; the value is valid after the next sync.
void closure_flag_fetch(tmc_handle* h, int* flag) {
  *flag = 0;
  if (!h->d_closure_err) return;
  cudaMemcpyAsync(flag, h->d_closure_err, sizeof(int), cudaMemcpyDeviceToHost, h->st);
  cudaMemsetAsync(h->d_closure_err, 0, sizeof(int), h->st);
}
constexpr const char* kClosureTimeout =
    ": a tensor-core completion wait of the closure network timed out; edges after it got no correction";

int h2d(tmc_handle* h, double* dst, const double* src, size_t n) {
  // cudaMemcpyDefault: the caller's array may be host or device memory
  // (unified addressing tells the direction)
  if (cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDefault, h->st) != cudaSuccess)
    return h->cuda_check("H2D");
  return TMC_OK;
}
int d2h(tmc_handle* h, double* dst, const double* src, size_t n) {
  if (cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDefault, h->st) != cudaSuccess)
    return h->cuda_check("D2H");
  return TMC_OK;
}

}  // namespace

extern "C" {

int tmc_default_params(tmc_params* p) {
  if (!p) return TMC_E_ARG;
  std::memset(p, 0, sizeof(*p));
  p->dt = 240.0; /* run/namelist.tmcore_swm */
  p->time_scheme = 2;
  p->pv_scheme = 3;
  p->conserve_energy = 1;
  p->flux_4th_order_correct = 0;
  p->apvm_weight = 0.5;
  p->adv_order = 2;
  p->adv_mono = 1;
  p->interp_pv_order = 3;
  p->radius = 6371220.0;
  p->g = 9.80616;
  p->omega = 7.292e-5;
  p->precision = TMC_FP64;
  p->renumber = 1;
  p->use_graph = 1;
  p->diag_every = 1;
  return TMC_OK;
}

int tmc_create(const tmc_mesh_desc* mesh, const tmc_params* params, tmc_handle** out) {
  if (!out) return TMC_E_ARG;
  *out = nullptr;
  auto h = std::make_unique<tmc_handle>();
  if (!mesh || !params) return TMC_E_ARG;
  h->p = *params;
  const tmc_params& p = h->p;
  auto bad = [&](const char* m) {
    h->err = m;
    *out = h.release();
    return TMC_E_ARG;
  };
  if (p.time_scheme < 1 || p.time_scheme > 3) return bad("time_scheme must be 1 (CRK3), 2 (CRK4) or 3 (PC2)");
  if (p.pv_scheme < 1 || p.pv_scheme > 3) return bad("pv_scheme must be 1 (APVM), 2 (conservative APVM) or 3 (upwind)");
  if (p.adv_wind < 0 || p.adv_wind > 2) return bad("adv_wind must be 0 (shallow water), 1 or 2 (adv model)");
  if (p.adv_wind != 0) {
    if (p.precision != TMC_FP64) {
      h->err = "the adv model runs in FP64 only";
      *out = h.release();
      return TMC_E_UNSUP;
    }
    if (!mesh || !mesh->lonVertex) return bad("the adv model needs lonVertex in tmc_mesh_desc");
    if (p.n_tracers != 0) return bad("the adv model advects gd only (n_tracers must be 0)");
  }
  h->adv = p.adv_wind != 0;
  h->generic = h->adv || p.time_scheme != 2;
  h->members = p.members > 0 ? p.members : 1;
  if (h->members > 1) {
    if (p.precision != TMC_FP32 || h->generic) {
      h->err = "ensembles (members > 1) run the FP32 shallow-water model with CRK4";
      *out = h.release();
      return TMC_E_UNSUP;
    }
    if (h->members > 65535) return bad("members must be at most 65535");
  }
  if (p.member_layout != 0) {
    if (p.member_layout != 1) return bad("member_layout must be 0 (member-outermost) or 1 (member-innermost)");
    if (h->members < 16 || h->members % 16 != 0) return bad("member_layout 1 needs members a multiple of 16");
    int V_, L_;
    if (!ens::lanes_for(h->members, p.member_lanes, &V_, &L_))
      return bad("member_lanes must be 0, or 8, 16 or 32 dividing the member count");
    const bool centred = p.pv_scheme == 1 && p.apvm_weight == 0.0;
    const bool upwind = p.pv_scheme == 3 && (p.interp_pv_order == 3 || p.interp_pv_order == 4);
    if (!(centred || upwind) || p.adv_order != 2 || p.n_tracers != 0 || p.flux_4th_order_correct) {
      h->err = "member_layout 1 runs centred pv (pv_scheme 1, apvm_weight 0) or upwind pv (pv_scheme 3, "
               "interp_pv_order 3 or 4), adv_order 2, no tracers";
      *out = h.release();
      return TMC_E_UNSUP;
    }
  }
  if (!(p.dt > 0.0) || !(p.radius > 0.0)) return bad("dt and radius must be positive");
  if (p.adv_order < 2 || p.adv_order > 6) return bad("adv_order must be 2..6");
  if (p.pv_scheme == 3 && (p.interp_pv_order < 3 || p.interp_pv_order > 6)) return bad("interp_pv_order must be 3..6");
  if (p.n_tracers < 0 || p.n_tracers > 64) return bad("n_tracers must be 0..64");
  const int tro = p.tracer_adv_order ? p.tracer_adv_order : p.adv_order;
  if (tro < 2 || tro > 6) return bad("tracer_adv_order must be 2..6");
  if (p.precision != TMC_FP64 && p.precision != TMC_FP32) return bad("precision must be TMC_FP64 or TMC_FP32");
  h->bs = p.block_size > 0 ? p.block_size : 256;
  if (h->bs % 32 != 0 || h->bs > 512) return bad("block_size must be a multiple of 32 up to 512");
  if (p.members > 1 && h->bs > 256) return bad("block_size must be at most 256 for ensembles");

  if (cudaSetDevice(p.device) != cudaSuccess) {
    h->err = "cudaSetDevice failed (no CUDA device?)";
    cudaGetLastError();
    *out = h.release();
    return TMC_E_CUDA;
  }
  PrepOptions opt;
  if (p.renumber < 0 || p.renumber > 2) return bad("renumber must be 0 (as given), 1 (Hilbert) or 2 (Morton)");
  opt.renumber = p.renumber;
  if (p.precision == TMC_FP32) {
    // the FP32 kernels unroll over 6 edges per cell and 10 edges per edge
    if (mesh->maxEdges > 6 || mesh->maxEdges2 > 10) {
      h->err = "the FP32 path supports maxEdges <= 6 and maxEdges2 <= 10";
      *out = h.release();
      return TMC_E_UNSUP;
    }
    opt.min_me = 6;
    opt.min_me2 = 10;
  }
  opt.cell_fit = p.stencils || p.adv_order >= 3 || (p.n_tracers > 0 && tro >= 3) || p.flux_4th_order_correct;
  opt.vertex_fit = p.stencils || p.pv_scheme == 3;
  if (!prepare_mesh(*mesh, p, opt, h->hm)) {
    h->err = h->hm.err;
    *out = h.release();
    return TMC_E_ARG;
  }
  HostMesh& hm = h->hm;
  if (cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&h->st2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->fork_ev, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->join_ev, cudaEventDisableTiming) != cudaSuccess) {
    h->err = "cudaStreamCreate / cudaEventCreate failed";
    *out = h.release();
    return TMC_E_CUDA;
  }
  DevMesh& M = h->M;
  M.nc = hm.nc;
  M.ne = hm.ne;
  M.nv = hm.nv;
  M.me = hm.me;
  M.me2 = hm.me2;
  M.nEdgesOnCell = h->upload(hm.nEdgesOnCell);
  M.edgesOnCell = h->upload(hm.edgesOnCell);
  M.cellsOnCell = h->upload(hm.cellsOnCell);
  M.nSign = h->upload(hm.nSignEdge);
  M.areaCell = h->upload(hm.areaCell);
  M.cellsOnEdge = h->upload(hm.cellsOnEdge);
  M.verticesOnEdge = h->upload(hm.verticesOnEdge);
  M.nEdgesOnEdge = h->upload(hm.nEdgesOnEdge);
  M.edgesOnEdge = h->upload(hm.edgesOnEdge);
  M.weightsOnEdge = h->upload(hm.weightsOnEdge);
  M.dcEdge = h->upload(hm.dcEdge);
  M.dvEdge = h->upload(hm.dvEdge);
  M.areaEdge = h->upload(hm.areaEdge);
  M.cellsOnVertex = h->upload(hm.cellsOnVertex);
  M.edgesOnVertex = h->upload(hm.edgesOnVertex);
  M.tSign = h->upload(hm.tSignEdge);
  M.kite = h->upload(hm.kite);
  M.areaTriangle = h->upload(hm.areaTriangle);
  M.fVertex = h->upload(hm.fVertex);
  M.v2c_start = h->upload(hm.v2c_start);
  M.v2c_vertex = h->upload(hm.v2c_vertex);
  M.v2c_kite = h->upload(hm.v2c_kite);
  if (!hm.recon.empty()) {
    M.recon = h->upload(hm.recon);
    M.cell_trig = h->upload(hm.cell_trig);
  }
  if (h->adv) {
    h->d_latV = h->upload(hm.latVertex);
    h->d_lonV = h->upload(hm.lonVertex);
  }
  if (p.precision == TMC_FP32) {
    auto f32 = [](const std::vector<double>& v) { return std::vector<float>(v.begin(), v.end()); };
    auto inv32 = [](const std::vector<double>& v) {
      std::vector<float> o(v.size());
      for (size_t i = 0; i < v.size(); ++i) o[i] = (float)(1.0 / v[i]);
      return o;
    };
    std::vector<double> invA(hm.areaCell.size());
    for (size_t i = 0; i < invA.size(); ++i) invA[i] = 1.0 / hm.areaCell[i];
    M.weightsOnEdge_f = h->upload(f32(hm.weightsOnEdge));
    M.dcEdge_f = h->upload(f32(hm.dcEdge));
    M.dvEdge_f = h->upload(f32(hm.dvEdge));
    M.areaEdge_f = h->upload(f32(hm.areaEdge));
    M.kite_f = h->upload(f32(hm.kite));
    M.invAreaTriangle_f = h->upload(inv32(hm.areaTriangle));
    M.fVertex_f = h->upload(f32(hm.fVertex));
    M.invAreaCell_f = h->upload(inv32(hm.areaCell));
    M.areaCell_f = h->upload(f32(hm.areaCell));
    M.areaTriangle_f = h->upload(f32(hm.areaTriangle));
    M.invAreaCell = h->upload(invA);
  }
  M.cell2 = upload_stencil(h.get(), hm.cell2);
  M.cell3 = upload_stencil(h.get(), hm.cell3);
  M.cell4 = upload_stencil(h.get(), hm.cell4);
  M.vert2 = upload_stencil(h.get(), hm.vert2);
  M.vert4 = upload_stencil(h.get(), hm.vert4);
  if (p.precision == TMC_FP32 && p.pv_scheme == 3 && (p.interp_pv_order == 3 || p.interp_pv_order == 4) &&
      hm.vert2.width > 0 && hm.vert2.width <= kUpW32) {
    // the packed FP32 form of the vertex fit stencils (k_edge_pv_up32)
    std::vector<int2> iw(hm.vert2.idx.size());
    for (size_t k = 0; k < iw.size(); ++k) {
      const float wf = (float)hm.vert2.w[k];
      int wb;
      std::memcpy(&wb, &wf, sizeof(wb));
      iw[k] = make_int2(hm.vert2.idx[k], wb);
    }
    M.vert2_iw = h->upload(iw);
    if (!M.vert2_iw) {
      h->err = "device allocation failed";
      cudaGetLastError();
      *out = h.release();
      return TMC_E_CUDA;
    }
  }
  h->d_cell_n2o = h->upload(hm.cell_n2o);
  h->d_edge_n2o = h->upload(hm.edge_n2o);
  h->d_vert_n2o = h->upload(hm.vert_n2o);

  ModelOpt& O = h->O;
  O.dt = p.dt;
  O.adv_order = p.adv_order;
  O.cell_coef2 = coef2_cell(p.adv_order, p.adv_mono);
  if (p.adv_order == 6 || tro == 6) h->cell_coef4 = 0.0;
  O.cell_coef4 = h->cell_coef4;
  O.pv_scheme = p.pv_scheme;
  O.apvm_weight = p.apvm_weight;
  O.interp_pv_order = p.interp_pv_order;
  O.vert_coef2 = coef2_vertex(p.interp_pv_order);
  if (p.pv_scheme == 3 && p.interp_pv_order == 6) h->vert_coef4 = 0.0;
  O.vert_coef4 = h->vert_coef4;
  O.n_tracers = p.n_tracers;
  O.tr_order = tro;
  O.tr_coef2 = coef2_cell(tro, p.tracer_adv_order ? p.tracer_adv_mono : p.adv_mono);
  O.tr_coef4 = h->cell_coef4;
  O.flux4 = p.flux_4th_order_correct ? 1 : 0;

  const int nmax = std::max(hm.nc, std::max(hm.ne, hm.nv));
  h->raw_c = h->dalloc<double>(hm.nc);
  h->raw_e = h->dalloc<double>(hm.ne);
  h->raw_v = h->dalloc<double>(hm.nv);
  h->raw_q = h->dalloc<double>((size_t)hm.nc * (p.n_tracers > 0 ? p.n_tracers : 1));
  h->op_a = h->dalloc<double>(nmax);
  h->op_b = h->dalloc<double>(nmax);
  h->op_c = h->dalloc<double>(nmax);
  h->op_out = h->dalloc<double>(nmax);
  const int minbs = 32;
  h->P.cap = (nmax + minbs - 1) / minbs;
  h->P.base = h->dalloc<double>(h->P.member_stride() * h->members);
  h->P.fin = h->dalloc<double>((size_t)kFinalizeRegions * kFinSplit * 2 * h->members);
  for (int k = 0; k < P_COUNT; ++k) h->bsp[k] = h->bs;
  // the FP32 cell pass is compiled for at most 256 threads per block (its
  // register budget leaves room for 3 blocks per SM)
  if (p.precision == TMC_FP32) h->bsp[P_CELL] = std::min(h->bsp[P_CELL], 256);
  set_counts(h.get());
  const int bc = grid_for(hm.nc, h->bs);
  for (int r = 0; r < R_COUNT; ++r) h->gen_counts[r] = h->counts[r];
  if (h->adv)  // the invariant pass of the adv model is the mass alone, over cells
    for (int r = R_MASS; r <= R_AV; ++r) h->gen_counts[r] = bc;
  h->d_diag = h->dalloc<double>((size_t)kDiagStride * h->members);  // per member: outputs, region sums, counters
  if (cudaMallocHost(&h->h_diag, sizeof(double) * kDiagLen) != cudaSuccess) h->h_diag = nullptr;
  if (!h->d_diag || !h->h_diag || !h->P.base || !h->P.fin) {
    h->err = "device allocation failed";
    cudaGetLastError();
    *out = h.release();
    return TMC_E_CUDA;
  }
  cudaMemset(h->d_diag, 0, sizeof(double) * kDiagStride * h->members);
  cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, p.device);
  h->d_member_on = h->dalloc<int>(h->members);
  h->d_closure_err = h->dalloc<int>(1);
  if (!h->d_member_on || !h->d_closure_err) {
    h->err = "device allocation failed";
    cudaGetLastError();
    *out = h.release();
    return TMC_E_CUDA;
  }
  {
    std::vector<int> on(h->members, 1);
    cudaMemcpy(h->d_member_on, on.data(), sizeof(int) * h->members, cudaMemcpyHostToDevice);
  }
  cudaMemset(h->d_closure_err, 0, sizeof(int));
  cudaMemset(h->P.base, 0, sizeof(double) * h->P.member_stride() * h->members);
  if (p.member_layout == 1 && p.pv_scheme == 3 && h->hm.vert2.width > ens::kUpW) {
    h->err = "member_layout 1: vertex fit stencils wider than " + std::to_string(ens::kUpW);
    *out = h.release();
    return TMC_E_UNSUP;
  }
  if (p.member_layout == 1)
    h->eng = std::make_unique<EnsEngine>(h.get());
  else if (p.precision == TMC_FP32)
    h->eng = std::make_unique<Engine<float>>(h.get());
  else
    h->eng = std::make_unique<Engine<double>>(h.get());
  if (h->eng->alloc() != TMC_OK) {
    h->err = "device allocation failed";
    cudaGetLastError();
    *out = h.release();
    return TMC_E_CUDA;
  }
  int rc = sync(h.get(), "tmc_create");
  if (rc == TMC_OK) rc = h->cuda_check("tmc_create");
  *out = h.release();
  return rc;
}

int tmc_destroy(tmc_handle* h) {
  if (!h) return TMC_OK;
  if (h->st) cudaStreamSynchronize(h->st);
  if (h->cst) {
    cudaStreamSynchronize(h->cst);
    for (cudaEvent_t e : h->cev)
      if (e) cudaEventDestroy(e);
    cudaStreamDestroy(h->cst);
  }
  h->drop_graphs();
  for (cudaEvent_t e : h->ev_pool) cudaEventDestroy(e);
  h->eng.reset();
  for (void* q : h->dptrs) cudaFree(q);
  if (h->h_diag) cudaFreeHost(h->h_diag);
  if (h->st2) {
    cudaStreamSynchronize(h->st2);
    cudaStreamDestroy(h->st2);
  }
  if (h->fork_ev) cudaEventDestroy(h->fork_ev);
  if (h->join_ev) cudaEventDestroy(h->join_ev);
  if (h->st) cudaStreamDestroy(h->st);
  delete h;
  return TMC_OK;
}

const char* tmc_last_error(const tmc_handle* h) { return h ? h->err.c_str() : "null handle"; }

#define TMC_REQUIRE_HANDLE(h) \
  if (!(h) || !(h)->eng) return TMC_E_ARG;
// entry points of the shallow-water model only
#define TMC_REQUIRE_SWM(h)   \
  TMC_REQUIRE_HANDLE(h);     \
  if ((h)->adv) return (h)->fail(TMC_E_UNSUP, "not available in the adv model (adv_wind != 0)");

int tmc_set_initial(tmc_handle* h, const double* gd, const double* u, const double* ghs) {
  TMC_REQUIRE_SWM(h);
  if (!gd || !u || !ghs) return h->fail(TMC_E_ARG, "tmc_set_initial: NULL array");
  const int nc = h->M.nc, ne = h->M.ne;
  int rc;
  if ((rc = h2d(h, h->raw_c, gd, nc))) return rc;
  launch_gather<double>(nc, h->raw_c, h->d_cell_n2o, h->op_a, h->st);  // gd (new order, double)
  if ((rc = h2d(h, h->raw_e, u, ne))) return rc;
  launch_gather<double>(ne, h->raw_e, h->d_edge_n2o, h->op_b, h->st);  // u
  // tmcore_swm_mod.F90:62-64: gd_edge = c2e(gd) [+ upwind, sign of u], iap_u = sqrt(gd_edge) u
  launch_op(OP_C2E, h->M, h->O, h->op_a, nullptr, nullptr, h->op_out, 0, 0, 0.0, 0.0, h->bs, h->st);
  if (h->p.adv_order >= 3)
    launch_op(OP_UPWIND, h->M, h->O, h->op_a, h->op_b, nullptr, h->op_out, h->p.adv_order, h->p.adv_mono,
              h->O.cell_coef2, h->O.cell_coef4, h->bs, h->st);
  h->eng->set_state_dev(h->raw_c, h->raw_e);  // gd (iap overwritten below)
  h->eng->set_iap_from_u(h->op_out, h->op_b);
  if ((rc = h2d(h, h->raw_c, ghs, nc))) return rc;
  h->eng->set_ghs_dev(h->raw_c);
  h->have_state = true;
  h->prep_valid = false;
  h->step_count = 0;
  if ((rc = sync(h, "tmc_set_initial"))) return rc;
  return h->cuda_check("tmc_set_initial");
}

int tmc_set_state(tmc_handle* h, const double* gd, const double* iap_u) {
  TMC_REQUIRE_SWM(h);
  if (!gd || !iap_u) return h->fail(TMC_E_ARG, "tmc_set_state: NULL array");
  int rc;
  if ((rc = h2d(h, h->raw_c, gd, h->M.nc))) return rc;
  if ((rc = h2d(h, h->raw_e, iap_u, h->M.ne))) return rc;
  h->eng->set_state_dev(h->raw_c, h->raw_e);
  h->have_state = true;
  h->prep_valid = false;
  if ((rc = sync(h, "tmc_set_state"))) return rc;
  return h->cuda_check("tmc_set_state");
}

int tmc_get_state(tmc_handle* h, double* gd, double* iap_u, double* u) {
  TMC_REQUIRE_SWM(h);
  if (!h->have_state) return h->fail(TMC_E_STATE, "no state set");
  int rc;
  if (u) h->eng->launch_diag_pass(false);
  if (gd) {
    h->eng->get_field(F_GD, h->raw_c);
    if ((rc = d2h(h, gd, h->raw_c, h->M.nc))) return rc;
    if ((rc = sync(h, "tmc_get_state"))) return rc;
  }
  if (iap_u) {
    h->eng->get_field(F_IAP, h->raw_e);
    if ((rc = d2h(h, iap_u, h->raw_e, h->M.ne))) return rc;
    if ((rc = sync(h, "tmc_get_state"))) return rc;
  }
  if (u) {
    h->eng->get_field(F_U, h->raw_e);
    if ((rc = d2h(h, u, h->raw_e, h->M.ne))) return rc;
  }
  if ((rc = sync(h, "tmc_get_state"))) return rc;
  return h->cuda_check("tmc_get_state");
}

int tmc_get_vertex(tmc_handle* h, double* pv, double* vor) {
  TMC_REQUIRE_SWM(h);
  if (!h->have_state) return h->fail(TMC_E_STATE, "no state set");
  int rc;
  h->eng->launch_diag_pass(false);
  if (pv) {
    h->eng->get_field(F_PV_V, h->raw_v);
    if ((rc = d2h(h, pv, h->raw_v, h->M.nv))) return rc;
    if ((rc = sync(h, "tmc_get_vertex"))) return rc;
  }
  if (vor) {
    h->eng->get_field(F_VOR, h->raw_v);
    if ((rc = d2h(h, vor, h->raw_v, h->M.nv))) return rc;
  }
  if ((rc = sync(h, "tmc_get_vertex"))) return rc;
  return h->cuda_check("tmc_get_vertex");
}

int tmc_set_tracers(tmc_handle* h, const double* qgd) {
  TMC_REQUIRE_SWM(h);
  if (h->O.n_tracers == 0) return TMC_OK;
  if (!qgd) return h->fail(TMC_E_ARG, "tmc_set_tracers: NULL array");
  int rc;
  if ((rc = h2d(h, h->raw_q, qgd, (size_t)h->M.nc * h->O.n_tracers))) return rc;
  h->eng->set_tracers_dev(h->raw_q);
  h->prep_valid = false;
  if ((rc = sync(h, "tmc_set_tracers"))) return rc;
  return h->cuda_check("tmc_set_tracers");
}

int tmc_get_tracers(tmc_handle* h, double* qgd) {
  TMC_REQUIRE_SWM(h);
  if (h->O.n_tracers == 0) return TMC_OK;
  if (!qgd) return h->fail(TMC_E_ARG, "tmc_get_tracers: NULL array");
  h->eng->get_tracers_dev(h->raw_q);
  int rc;
  if ((rc = d2h(h, qgd, h->raw_q, (size_t)h->M.nc * h->O.n_tracers))) return rc;
  if ((rc = sync(h, "tmc_get_tracers"))) return rc;
  return h->cuda_check("tmc_get_tracers");
}

int tmc_step(tmc_handle* h, int32_t nsteps) {
  TMC_REQUIRE_HANDLE(h);
  if (!h->have_state) return h->fail(TMC_E_STATE, "tmc_step before tmc_set_state/tmc_set_initial");
  if (nsteps < 0) return h->fail(TMC_E_ARG, "nsteps < 0");
  for (int i = 0; i < nsteps; ++i) {
    int rc = launch_one_step(h);
    if (rc) return rc;
  }
  return TMC_OK;
}

int tmc_synchronize(tmc_handle* h) {
  TMC_REQUIRE_HANDLE(h);
  int rc = sync(h, "tmc_synchronize");
  if (rc) return rc;
  return h->cuda_check("tmc_synchronize");
}

int tmc_get_diag(tmc_handle* h, double out[5]) {
  TMC_REQUIRE_HANDLE(h);
  if (!out) return TMC_E_ARG;
  if (!h->have_state) return h->fail(TMC_E_STATE, "no state set");
  h->eng->launch_diag_pass(true);
  cudaMemcpyAsync(h->h_diag, h->d_diag + (size_t)h->cur * kDiagStride, sizeof(double) * kDiagLen,
                  cudaMemcpyDeviceToHost, h->st);
  int timed_out = 0;
  closure_flag_fetch(h, &timed_out);
  int rc = sync(h, "tmc_get_diag");
  if (rc) return rc;
  for (int i = 0; i < 4; ++i) out[i] = h->h_diag[i];
  out[4] = h->step_count > 0 ? h->h_diag[4] : 1.0;
  if ((rc = h->cuda_check("tmc_get_diag"))) return rc;
  if (timed_out) return h->fail(TMC_E_HEALTH, std::string("tmc_get_diag") + kClosureTimeout);
  // device health: a non-finite invariant means the state has left the
  // physical range (a negative depth makes sqrt(gd_edge) and everything
  // after it NaN); the outputs are filled all the same
  for (int i = 0; i < 5; ++i)
    if (!std::isfinite(out[i])) return h->fail(TMC_E_HEALTH, "tmc_get_diag: non-finite invariants (the state blew up)");
  return TMC_OK;
}

int tmc_get_diag_all(tmc_handle* h, double* out) {
  TMC_REQUIRE_HANDLE(h);
  if (!out) return TMC_E_ARG;
  if (!h->have_state) return h->fail(TMC_E_STATE, "no state set");
  h->eng->launch_diag_pass(true);
  std::vector<double> all((size_t)kDiagStride * h->members);
  cudaMemcpyAsync(all.data(), h->d_diag, sizeof(double) * all.size(), cudaMemcpyDeviceToHost, h->st);
  int timed_out = 0;
  closure_flag_fetch(h, &timed_out);
  int rc = sync(h, "tmc_get_diag_all");
  if (rc) return rc;
  for (int m = 0; m < h->members; ++m) {
    const double* d = all.data() + (size_t)m * kDiagStride;
    for (int i = 0; i < 4; ++i) out[(size_t)m * 5 + i] = d[i];
    out[(size_t)m * 5 + 4] = h->step_count > 0 ? d[4] : 1.0;
  }
  if ((rc = h->cuda_check("tmc_get_diag_all"))) return rc;
  if (timed_out) return h->fail(TMC_E_HEALTH, std::string("tmc_get_diag_all") + kClosureTimeout);
  return TMC_OK;
}

int tmc_time_integrate(tmc_handle* h, const double* gd_old, const double* iap_u_old, const double* qgd_old,
                       double* gd_new, double* iap_u_new, double* qgd_new) {
  TMC_REQUIRE_SWM(h);
  if (h->members > 1) return h->fail(TMC_E_UNSUP, "tmc_time_integrate needs members <= 1");
  if (!gd_old || !iap_u_old || !gd_new || !iap_u_new) return h->fail(TMC_E_ARG, "tmc_time_integrate: NULL array");
  const bool trc = h->O.n_tracers > 0;
  if (trc && (!qgd_old || !qgd_new)) return h->fail(TMC_E_ARG, "tmc_time_integrate: tracers need qgd arrays");
  const size_t nq = (size_t)h->M.nc * h->O.n_tracers;
  // The host copies run on a second stream, overlapped with the permutation
  // gathers and scatters on the compute stream: each field's gather waits for
  // its own copy only, each field's copy back waits for its own scatter only.
  if (!h->cst) {
    if (cudaStreamCreateWithFlags(&h->cst, cudaStreamNonBlocking) != cudaSuccess)
      return h->cuda_check("tmc_time_integrate: copy stream");
    for (auto& e : h->cev)
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
        return h->cuda_check("tmc_time_integrate: events");
  }
  cudaStream_t cs = h->cst;
  cudaEventRecord(h->cev[0], h->st);  // earlier work on the raw buffers is done
  cudaStreamWaitEvent(cs, h->cev[0], 0);
  struct Io {
    const double* in;
    double* out;
    double* raw;
    size_t n;
    int field;
  } io[3] = {{gd_old, gd_new, h->raw_c, (size_t)h->M.nc, F_GD},
             {iap_u_old, iap_u_new, h->raw_e, (size_t)h->M.ne, F_IAP},
             {qgd_old, qgd_new, h->raw_q, nq, -1}};
  const int nio = trc ? 3 : 2;
  for (int i = 0; i < nio; ++i) {
    if (cudaMemcpyAsync(io[i].raw, io[i].in, io[i].n * sizeof(double), cudaMemcpyDefault, cs) != cudaSuccess)
      return h->cuda_check("H2D");
    cudaEventRecord(h->cev[1 + i], cs);
  }
  // The step's edge preparation reads gd and iap_u only (second-order tracers
  // are fluxed in the cell pass): with such tracers it runs before their
  // copy has arrived, beside it.  Where the fused program allows (FP32, 1, 2
  // or 4 tracers), so does all of stage 1 but its tracer terms, which follow
  // the tracers' arrival.
  const bool prep_early = trc && h->O.tr_order < 3 && !h->generic;
  const bool split = trc && h->eng->can_split();
  h->have_state = true;
  h->prep_valid = false;
  for (int i = 0; i < nio; ++i) {
    if (split && io[i].field == -1) break;  // the tracers: beside stage 1
    cudaStreamWaitEvent(h->st, h->cev[1 + i], 0);
    h->eng->gather_field(io[i].field, io[i].raw);
    if (split && io[i].field == F_GD) {
      // the tracers' gather and ratios (which read gd) on the copy stream,
      // behind their copy; stage 1 without its tracer terms reads neither
      cudaEventRecord(h->cev[7], h->st);
      cudaStreamWaitEvent(cs, h->cev[7], 0);
      h->eng->gather_tracers_on(h->raw_q, cs);
      cudaEventRecord(h->cev[3], cs);
    }
    if (prep_early && io[i].field == F_IAP) {
      h->eng->refresh_shadows(0, false);
      ensure_prep(h);
    }
  }
  int rc;
  if (split) {
    rc = launch_one_step_split(h, [&] { cudaStreamWaitEvent(h->st, h->cev[3], 0); });
    if (rc) return rc;
  } else {
    h->eng->refresh_shadows(0);
    if ((rc = launch_one_step(h))) return rc;
  }
  for (int i = 0; i < nio; ++i) {
    if (io[i].field == F_GD || io[i].field == F_IAP)
      h->eng->get_field(io[i].field, io[i].raw);
    else
      h->eng->get_tracers_dev(io[i].raw);
    cudaEventRecord(h->cev[4 + i], h->st);
    cudaStreamWaitEvent(cs, h->cev[4 + i], 0);
    if (cudaMemcpyAsync(io[i].out, io[i].raw, io[i].n * sizeof(double), cudaMemcpyDefault, cs) != cudaSuccess)
      return h->cuda_check("D2H");
  }
  int timed_out = 0;
  if (h->closure) closure_flag_fetch(h, &timed_out);
  if (cudaStreamSynchronize(cs) != cudaSuccess) return h->cuda_check("tmc_time_integrate");
  if ((rc = sync(h, "tmc_time_integrate"))) return rc;
  if ((rc = h->cuda_check("tmc_time_integrate"))) return rc;
  if (timed_out) return h->fail(TMC_E_HEALTH, std::string("tmc_time_integrate") + kClosureTimeout);
  return TMC_OK;
}

int tmc_spatial_operators(tmc_handle* h, const double* gd, const double* iap_u, double* tend_gd,
                          double* tend_iap_u) {
  TMC_REQUIRE_SWM(h);
  if (h->members > 1) return h->fail(TMC_E_UNSUP, "tmc_spatial_operators needs members <= 1");
  if (!gd || !iap_u || !tend_gd || !tend_iap_u) return h->fail(TMC_E_ARG, "tmc_spatial_operators: NULL array");
  // uses state slot 1 as scratch; state(old) is untouched
  int rc;
  if ((rc = h2d(h, h->raw_c, gd, h->M.nc))) return rc;
  if ((rc = h2d(h, h->raw_e, iap_u, h->M.ne))) return rc;
  // gather into slot 1 via a temporary engine state swap: slot 0 is saved in op buffers
  auto* e64 = dynamic_cast<Engine<double>*>(h->eng.get());
  auto* e32 = dynamic_cast<Engine<float>*>(h->eng.get());
  if (e64) {
    launch_gather<double>(h->M.nc, h->raw_c, h->d_cell_n2o, e64->gd[1], h->st);
    launch_gather<double>(h->M.ne, h->raw_e, h->d_edge_n2o, e64->iap[1], h->st);
    e64->copy_tracers_to_slot1();
  } else {
    launch_gather<double>(h->M.nc, h->raw_c, h->d_cell_n2o, e32->gd[1], h->st);
    launch_gather<float>(h->M.ne, h->raw_e, h->d_edge_n2o, e32->iap[1], h->st);
    e32->copy_tracers_to_slot1();
    e32->refresh_shadows(1);
  }
  h->eng->launch_spatial_only();
  h->prep_valid = false;
  h->eng->get_field(F_TEND_GD, h->raw_c);
  if ((rc = d2h(h, tend_gd, h->raw_c, h->M.nc))) return rc;
  h->eng->get_field(F_TEND_IAP, h->raw_e);
  if ((rc = d2h(h, tend_iap_u, h->raw_e, h->M.ne))) return rc;
  if ((rc = sync(h, "tmc_spatial_operators"))) return rc;
  return h->cuda_check("tmc_spatial_operators");
}

static int run_op(tmc_handle* h, int op, const double* a, int na, const double* b, int nb, const double* c, int nc_,
                  const double* inout, double* out, int nout, int order, int mono) {
  TMC_REQUIRE_HANDLE(h);
  if (!a || !out) return h->fail(TMC_E_ARG, "NULL array");
  const int32_t* n2o_for[4] = {nullptr, h->d_cell_n2o, h->d_edge_n2o, h->d_vert_n2o};
  auto n_of = [&](int kind) { return kind == 1 ? h->M.nc : (kind == 2 ? h->M.ne : h->M.nv); };
  auto raw_of = [&](int kind) { return kind == 1 ? h->raw_c : (kind == 2 ? h->raw_e : h->raw_v); };
  int rc;
  struct In {
    const double* host;
    int kind;
    double* dev;
  } ins[4] = {{a, na, h->op_a}, {b, nb, h->op_b}, {c, nc_, h->op_c}, {inout, nout, h->op_out}};
  for (auto& in : ins) {
    if (!in.host || !in.kind) continue;
    if ((rc = h2d(h, raw_of(in.kind), in.host, n_of(in.kind)))) return rc;
    launch_gather<double>(n_of(in.kind), raw_of(in.kind), n2o_for[in.kind], in.dev, h->st);
  }
  double coef2 = coef2_cell(order, mono), coef4 = 0.25;
  if (op == OP_UPWIND) {
    if (order >= 3 && h->M.cell2.width == 0)
      return h->fail(TMC_E_STATE, "upwind stencil tables were not built (set tmc_params.stencils = 1)");
    if (order == 6) h->cell_coef4 = 0.0;
    coef4 = h->cell_coef4;
  }
  launch_op(op, h->M, h->O, h->op_a, h->op_b, h->op_c, h->op_out, order, mono, coef2, coef4, h->bs, h->st);
  launch_scatter<double>(n_of(nout), h->op_out, n2o_for[nout], raw_of(nout), h->st);
  if ((rc = d2h(h, out, raw_of(nout), n_of(nout)))) return rc;
  if ((rc = sync(h, "tmc_op"))) return rc;
  return h->cuda_check("tmc_op");
}

enum { K_NONE = 0, K_CELL = 1, K_EDGE = 2, K_VERT = 3 };

int tmc_op_div(tmc_handle* h, const double* f, double* o) {
  return run_op(h, OP_DIV, f, K_EDGE, nullptr, 0, nullptr, 0, nullptr, o, K_CELL, 0, 0);
}
int tmc_op_curl(tmc_handle* h, const double* f, double* o) {
  return run_op(h, OP_CURL, f, K_EDGE, nullptr, 0, nullptr, 0, nullptr, o, K_VERT, 0, 0);
}
int tmc_op_c2e(tmc_handle* h, const double* f, double* o) {
  return run_op(h, OP_C2E, f, K_CELL, nullptr, 0, nullptr, 0, nullptr, o, K_EDGE, 0, 0);
}
int tmc_op_c2v(tmc_handle* h, const double* f, double* o) {
  return run_op(h, OP_C2V, f, K_CELL, nullptr, 0, nullptr, 0, nullptr, o, K_VERT, 0, 0);
}
int tmc_op_v2c(tmc_handle* h, const double* f, double* o) {
  return run_op(h, OP_V2C, f, K_VERT, nullptr, 0, nullptr, 0, nullptr, o, K_CELL, 0, 0);
}
int tmc_op_v2e(tmc_handle* h, const double* f, double* o) {
  return run_op(h, OP_V2E, f, K_VERT, nullptr, 0, nullptr, 0, nullptr, o, K_EDGE, 0, 0);
}
int tmc_op_kinetic_energy(tmc_handle* h, const double* u, double* o) {
  return run_op(h, OP_KE, u, K_EDGE, nullptr, 0, nullptr, 0, nullptr, o, K_CELL, 0, 0);
}
int tmc_op_tangent_wind(tmc_handle* h, const double* u, double* o) {
  return run_op(h, OP_TWIND, u, K_EDGE, nullptr, 0, nullptr, 0, nullptr, o, K_EDGE, 0, 0);
}
int tmc_op_tangent_vor_flux(tmc_handle* h, const double* u, const double* g, const double* pv, double* o) {
  if (!g || !pv) return h ? h->fail(TMC_E_ARG, "NULL array") : TMC_E_ARG;
  return run_op(h, OP_TVF, u, K_EDGE, g, K_EDGE, pv, K_EDGE, nullptr, o, K_EDGE, 0, 0);
}
int tmc_op_upwind_correction(tmc_handle* h, const double* f_cell, const double* u_edge, double* f_edge, int32_t order,
                             int32_t mono) {
  if (!u_edge || !f_edge) return h ? h->fail(TMC_E_ARG, "NULL array") : TMC_E_ARG;
  if (order < 2 || order > 6) return h ? h->fail(TMC_E_ARG, "order must be 2..6") : TMC_E_ARG;
  return run_op(h, OP_UPWIND, f_cell, K_CELL, u_edge, K_EDGE, nullptr, 0, f_edge, f_edge, K_EDGE, order, mono);
}

int tmc_time_steps(tmc_handle* h, int32_t nsteps, double* ms_total, double* ms_flux, int32_t* flux_launches,
                   int32_t* total_launches) {
  TMC_REQUIRE_HANDLE(h);
  if (!h->have_state) return h->fail(TMC_E_STATE, "no state set");
  if (nsteps <= 0) return h->fail(TMC_E_ARG, "nsteps must be positive");
  const size_t nev = (size_t)nsteps * 8 + 2;
  while (h->ev_pool.size() < nev) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return h->cuda_check("cudaEventCreate");
    h->ev_pool.push_back(e);
  }
  int rc;
  if ((rc = sync(h, "tmc_time_steps"))) return rc;
  // region 1: the production path (CUDA graph per step when enabled)
  if (ms_total) {
    cudaEventRecord(h->ev_pool[0], h->st);
    for (int i = 0; i < nsteps; ++i)
      if ((rc = launch_one_step(h))) return rc;
    cudaEventRecord(h->ev_pool[1], h->st);
    if ((rc = sync(h, "tmc_time_steps"))) return rc;
    float t = 0.f;
    cudaEventElapsedTime(&t, h->ev_pool[0], h->ev_pool[1]);
    *ms_total = t;
  }
  // region 2: the same steps launched directly, with events around the edge flux pass
  if (ms_flux) {
    std::vector<cudaEvent_t> evs(h->ev_pool.begin() + 2, h->ev_pool.begin() + nev);
    size_t pos = 0;
    for (int i = 0; i < nsteps; ++i) {
      const bool diag = h->p.diag_every > 0 && (h->step_count % h->p.diag_every) == 0;
      ensure_prep(h);
      h->eng->launch_step(diag, &evs, &pos);
      h->step_count++;
    }
    if ((rc = sync(h, "tmc_time_steps"))) return rc;
    double sum = 0.0;
    for (size_t k = 0; k + 1 < pos; k += 2) {
      float dt = 0.f;
      cudaEventElapsedTime(&dt, evs[k], evs[k + 1]);
      sum += dt;
    }
    *ms_flux = sum;
    if (flux_launches) *flux_launches = (int32_t)(pos / 2);
  }
  if (total_launches) *total_launches = nsteps * h->eng->launches_per_step();
  return h->cuda_check("tmc_time_steps");
}

int tmc_select_member(tmc_handle* h, int32_t member) {
  TMC_REQUIRE_HANDLE(h);
  if (member < 0 || member >= h->members) return h->fail(TMC_E_ARG, "member out of range");
  h->cur = member;
  return TMC_OK;
}

int tmc_set_closure(tmc_handle* h, const tmc_mlp* net) {
  TMC_REQUIRE_SWM(h);
  if (net && (h->p.precision != TMC_FP32 || h->generic))
    return h->fail(TMC_E_UNSUP, "the learned closure runs in the FP32 CRK4 shallow-water step");
  if (sync(h, "tmc_set_closure")) return TMC_E_CUDA;
  h->closure = net;
  if (net) h->closure_net = tmc_mlp_net(net);
  h->O.need_pv_c = net ? 1 : 0;
  h->drop_graphs();
  return TMC_OK;
}

int tmc_set_closure_stages(tmc_handle* h, int32_t every_stage) {
  TMC_REQUIRE_SWM(h);
  if (h->p.precision != TMC_FP32 || h->generic)
    return h->fail(TMC_E_UNSUP, "the learned closure runs in the FP32 CRK4 shallow-water step");
  if (sync(h, "tmc_set_closure_stages")) return TMC_E_CUDA;
  h->closure_every_stage = every_stage != 0;
  if (!h->closure_every_stage && !h->d_closure_dq) {
    h->d_closure_dq = h->dalloc<float>((size_t)h->members * h->M.ne);
    if (!h->d_closure_dq) return h->cuda_check("tmc_set_closure_stages: allocation");
  }
  h->drop_graphs();
  return TMC_OK;
}

int tmc_set_member_closure(tmc_handle* h, int32_t member, int32_t on) {
  TMC_REQUIRE_SWM(h);
  if (member < 0 || member >= h->members) return h->fail(TMC_E_ARG, "member out of range");
  const int v = on ? 1 : 0;
  if (cudaMemcpyAsync(h->d_member_on + member, &v, sizeof(int), cudaMemcpyHostToDevice, h->st) != cudaSuccess)
    return h->cuda_check("tmc_set_member_closure");
  return sync(h, "tmc_set_member_closure");
}

int tmc_closure_status(tmc_handle* h, int32_t* timed_out) {
  TMC_REQUIRE_SWM(h);
  int v = 0;
  closure_flag_fetch(h, &v);
  int rc = sync(h, "tmc_closure_status");
  if (rc) return rc;
  if (timed_out) *timed_out = v;
  return TMC_OK;
}

int tmc_closure_correction(tmc_handle* h, float* dq) {
  TMC_REQUIRE_SWM(h);
  if (!dq) return h->fail(TMC_E_ARG, "NULL array");
  if (!h->closure || h->closure_every_stage || !h->d_closure_dq)
    return h->fail(TMC_E_STATE, "tmc_closure_correction needs a closure held from stage 1 (tmc_set_closure_stages 0)");
  if (h->step_count <= 0) return h->fail(TMC_E_STATE, "tmc_closure_correction: no step taken with the closure");
  const int ne = h->M.ne, mem = h->members;
  std::vector<float> all((size_t)ne * mem);
  cudaMemcpyAsync(all.data(), h->d_closure_dq, sizeof(float) * all.size(), cudaMemcpyDeviceToHost, h->st);
  int rc = sync(h, "tmc_closure_correction");
  if (rc) return rc;
  // member-outermost [member][edge] or member-innermost [edge][member]; caller's edge order
  const bool inner = h->p.member_layout == 1;
  for (int i = 0; i < ne; ++i)
    dq[h->hm.edge_n2o[i]] = inner ? all[(size_t)i * mem + h->cur] : all[(size_t)h->cur * ne + i];
  return h->cuda_check("tmc_closure_correction");
}

int tmc_closure_features(tmc_handle* h, float* features, double* pv_edge) {
  TMC_REQUIRE_SWM(h);
  if (!features) return h->fail(TMC_E_ARG, "NULL array");
  if (h->p.precision != TMC_FP32 || h->generic)
    return h->fail(TMC_E_UNSUP, "closure features come from the FP32 CRK4 shallow-water step");
  if (!h->have_state) return h->fail(TMC_E_STATE, "no state set");
  const int ne = h->M.ne;
  float *d_feat = nullptr, *d_pv = nullptr;
  if (cudaMalloc(&d_feat, sizeof(float) * (size_t)ne * mlp::kIn) != cudaSuccess ||
      cudaMalloc(&d_pv, sizeof(float) * ne) != cudaSuccess) {
    cudaFree(d_feat);
    return h->cuda_check("tmc_closure_features: allocation");
  }
  const int saved = h->O.need_pv_c;
  h->O.need_pv_c = 1;
  h->eng->closure_features(d_feat, d_pv);
  h->O.need_pv_c = saved;
  h->prep_valid = false;
  std::vector<float> f((size_t)ne * mlp::kIn), pv(ne);
  cudaMemcpyAsync(f.data(), d_feat, sizeof(float) * f.size(), cudaMemcpyDeviceToHost, h->st);
  cudaMemcpyAsync(pv.data(), d_pv, sizeof(float) * ne, cudaMemcpyDeviceToHost, h->st);
  int rc = sync(h, "tmc_closure_features");
  cudaFree(d_feat);
  cudaFree(d_pv);
  if (rc) return rc;
  // caller's edge order
  for (int i = 0; i < ne; ++i) {
    const int o = h->hm.edge_n2o[i];
    std::memcpy(features + (size_t)o * mlp::kIn, f.data() + (size_t)i * mlp::kIn, sizeof(float) * mlp::kIn);
    if (pv_edge) pv_edge[o] = pv[i];
  }
  return h->cuda_check("tmc_closure_features");
}

int tmc_reconstruct(tmc_handle* h, const double* u, double* uX, double* uY, double* uZ, double* zonal,
                    double* meridional) {
  TMC_REQUIRE_HANDLE(h);
  if (!u) return h->fail(TMC_E_ARG, "NULL array");
  if (!h->M.recon) return h->fail(TMC_E_STATE, "tmc_reconstruct needs lonCell, latCell and x/y/zEdge in the mesh");
  const int nc = h->M.nc;
  if (!h->d_hist && !(h->d_hist = h->dalloc<double>((size_t)5 * nc))) return h->cuda_check("tmc_reconstruct");
  int rc;
  if ((rc = h2d(h, h->raw_e, u, h->M.ne))) return rc;
  launch_gather<double>(h->M.ne, h->raw_e, h->d_edge_n2o, h->op_b, h->st);
  double* d[5] = {h->d_hist, h->d_hist + nc, h->d_hist + 2 * (size_t)nc, h->d_hist + 3 * (size_t)nc,
                  h->d_hist + 4 * (size_t)nc};
  launch_reconstruct<double>(h->M, h->op_b, d[0], d[1], d[2], d[3], d[4], h->st);
  double* outs[5] = {uX, uY, uZ, zonal, meridional};
  for (int k = 0; k < 5; ++k) {
    if (!outs[k]) continue;
    launch_scatter<double>(nc, d[k], h->d_cell_n2o, h->raw_c, h->st);
    if ((rc = d2h(h, outs[k], h->raw_c, nc))) return rc;
    if ((rc = sync(h, "tmc_reconstruct"))) return rc;
  }
  return h->cuda_check("tmc_reconstruct");
}

int tmc_history_fields(tmc_handle* h, double* u, double* zonal, double* meridional, double* h_cell, double* div,
                       double* pv, double* vor) {
  TMC_REQUIRE_SWM(h);
  if (!h->have_state) return h->fail(TMC_E_STATE, "no state set");
  if ((zonal || meridional) && !h->M.recon)
    return h->fail(TMC_E_STATE, "the zonal/meridional wind needs lonCell, latCell and x/y/zEdge in the mesh");
  const int nc = h->M.nc, ne = h->M.ne, nv = h->M.nv;
  if (!h->d_hist && !(h->d_hist = h->dalloc<double>((size_t)5 * nc))) return h->cuda_check("tmc_history_fields");
  if (!h->d_hist_e && !(h->d_hist_e = h->dalloc<double>((size_t)2 * ne + 2 * (size_t)nv)))
    return h->cuda_check("tmc_history_fields");
  double *c0 = h->d_hist, *c1 = c0 + nc, *c2 = c1 + nc, *c3 = c2 + nc;
  double *e0 = h->d_hist_e, *e1 = e0 + ne, *v0 = e1 + ne, *v1 = v0 + nv;
  h->eng->history_dev(u ? e0 : nullptr, zonal ? c0 : nullptr, meridional ? c1 : nullptr, h_cell ? c2 : nullptr,
                      div ? c3 : nullptr, pv ? v0 : nullptr, vor ? v1 : nullptr, e1);
  h->prep_valid = false;
  struct Out {
    double* host;
    double* dev;
    int n;
    const int32_t* n2o;
    double* raw;
  } outs[7] = {{u, e0, ne, h->d_edge_n2o, h->raw_e},       {zonal, c0, nc, h->d_cell_n2o, h->raw_c},
               {meridional, c1, nc, h->d_cell_n2o, h->raw_c}, {h_cell, c2, nc, h->d_cell_n2o, h->raw_c},
               {div, c3, nc, h->d_cell_n2o, h->raw_c},       {pv, v0, nv, h->d_vert_n2o, h->raw_v},
               {vor, v1, nv, h->d_vert_n2o, h->raw_v}};
  int rc;
  for (auto& o : outs) {
    if (!o.host) continue;
    launch_scatter<double>(o.n, o.dev, o.n2o, o.raw, h->st);
    if ((rc = d2h(h, o.host, o.raw, o.n))) return rc;
    if ((rc = sync(h, "tmc_history_fields"))) return rc;
  }
  return h->cuda_check("tmc_history_fields");
}

int tmc_adv_set_initial(tmc_handle* h, const double* q) {
  TMC_REQUIRE_HANDLE(h);
  if (!h->adv) return h->fail(TMC_E_UNSUP, "tmc_adv_set_initial needs adv_wind = 1 or 2");
  if (!q) return h->fail(TMC_E_ARG, "tmc_adv_set_initial: NULL array");
  int rc;
  if ((rc = h2d(h, h->raw_c, q, h->M.nc))) return rc;
  h->eng->adv_set_initial_dev(h->raw_c);
  h->have_state = true;
  h->step_count = 0;
  if ((rc = sync(h, "tmc_adv_set_initial"))) return rc;
  return h->cuda_check("tmc_adv_set_initial");
}

int tmc_adv_get(tmc_handle* h, double* q, double* u) {
  TMC_REQUIRE_HANDLE(h);
  if (!h->adv) return h->fail(TMC_E_UNSUP, "tmc_adv_get needs adv_wind = 1 or 2");
  if (!h->have_state) return h->fail(TMC_E_STATE, "no state set");
  h->eng->adv_get_dev(q ? h->raw_c : nullptr, u ? h->raw_e : nullptr);
  int rc;
  if (q && (rc = d2h(h, q, h->raw_c, h->M.nc))) return rc;
  if (u && (rc = d2h(h, u, h->raw_e, h->M.ne))) return rc;
  if ((rc = sync(h, "tmc_adv_get"))) return rc;
  return h->cuda_check("tmc_adv_get");
}

int tmc_adv_elapsed(tmc_handle* h, double* seconds) {
  TMC_REQUIRE_HANDLE(h);
  if (!seconds) return h->fail(TMC_E_ARG, "NULL pointer");
  int rc;
  if ((rc = d2h(h, h->h_diag, h->d_diag, kDiagLen))) return rc;
  if ((rc = sync(h, "tmc_adv_elapsed"))) return rc;
  *seconds = h->h_diag[11];
  return TMC_OK;
}

int tmc_pass_times(tmc_handle* h, int32_t steps, double ms[5]) {
  TMC_REQUIRE_HANDLE(h);
  if (!ms) return TMC_E_ARG;
  if (!h->have_state) return h->fail(TMC_E_STATE, "no state set");
  if (h->generic) return h->fail(TMC_E_UNSUP, "tmc_pass_times times the fused CRK4 shallow-water step");
  if (steps <= 0) steps = 3;
  const size_t nev = (size_t)steps * 8 + 2;
  while (h->ev_pool.size() < nev) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return h->cuda_check("cudaEventCreate");
    h->ev_pool.push_back(e);
  }
  int rc;
  const int saved = h->timed_pass;
  for (int pass = 0; pass < P_COUNT; ++pass) {
    h->timed_pass = pass;
    std::vector<cudaEvent_t> evs(h->ev_pool.begin(), h->ev_pool.begin() + nev);
    size_t pos = 0;
    for (int i = 0; i < steps; ++i) {
      const bool diag = h->p.diag_every > 0 && (h->step_count % h->p.diag_every) == 0;
      ensure_prep(h);
      h->eng->launch_step(diag, &evs, &pos);
      h->step_count++;
    }
    if ((rc = sync(h, "tmc_pass_times"))) {
      h->timed_pass = saved;
      return rc;
    }
    double sum = 0.0;
    for (size_t k = 0; k + 1 < pos; k += 2) {
      float dt = 0.f;
      cudaEventElapsedTime(&dt, evs[k], evs[k + 1]);
      sum += dt;
    }
    ms[pass] = pos ? sum / (double)(pos / 2) : 0.0;
  }
  h->timed_pass = saved;
  return h->cuda_check("tmc_pass_times");
}

int tmc_autotune(tmc_handle* h, int32_t steps, int32_t block_sizes[5]) {
  TMC_REQUIRE_HANDLE(h);
  if (!h->have_state) return h->fail(TMC_E_STATE, "tmc_autotune needs a state (tmc_set_initial)");
  if (h->generic) return h->fail(TMC_E_UNSUP, "tmc_autotune tunes the fused CRK4 shallow-water step");
  if (steps <= 0) steps = 3;
  int rc;
  if ((rc = sync(h, "tmc_autotune"))) return rc;
  // events first: a failure here leaves nothing allocated and the state as it was
  const size_t nev = (size_t)steps * 8 + 2;
  while (h->ev_pool.size() < nev) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return h->cuda_check("cudaEventCreate");
    h->ev_pool.push_back(e);
  }
  // save state(old) of every member; the timing steps advance it
  const size_t M_ = (size_t)h->members;
  const bool f32 = h->p.precision == TMC_FP32;
  const size_t es = f32 ? sizeof(float) : sizeof(double);
  const size_t nq = (size_t)h->M.nc * (h->O.n_tracers > 0 ? h->O.n_tracers : 1);
  void *sv_gd = nullptr, *sv_iap = nullptr, *sv_q = nullptr;
  void *gd0, *iap0, *q0, *ghs0;
  h->eng->state_slot0(&gd0, &iap0, &q0, &ghs0);
  const size_t b_gd = 8 * h->M.nc * M_, b_iap = es * h->M.ne * M_, b_q = es * nq * M_;
  if (cudaMalloc(&sv_gd, b_gd) != cudaSuccess || cudaMalloc(&sv_iap, b_iap) != cudaSuccess ||
      (q0 && cudaMalloc(&sv_q, b_q) != cudaSuccess)) {
    cudaFree(sv_gd);
    cudaFree(sv_iap);
    cudaFree(sv_q);
    return h->cuda_check("tmc_autotune: scratch allocation");
  }
  cudaMemcpyAsync(sv_gd, gd0, b_gd, cudaMemcpyDeviceToDevice, h->st);
  cudaMemcpyAsync(sv_iap, iap0, b_iap, cudaMemcpyDeviceToDevice, h->st);
  if (q0) cudaMemcpyAsync(sv_q, q0, b_q, cudaMemcpyDeviceToDevice, h->st);
  const int cand_all[6] = {64, 128, 192, 256, 384, 512};
  const int limit = h->members > 1 ? 256 : 512;
  const int order[P_COUNT] = {P_FLUX, P_CELL, P_VERTEX, P_PV, P_FINAL};
  const int saved_timed = h->timed_pass;
  for (int pi = 0; pi < P_COUNT; ++pi) {
    const int pass = order[pi];
    h->timed_pass = pass;
    double best = 1e300;
    int best_bs = h->bsp[pass];
    for (int c : cand_all) {
      if (c > limit || (pass == P_CELL && f32 && c > 256)) continue;
      h->bsp[pass] = c;
      set_counts(h);
      // one untimed step with this block size, then `steps` timed ones
      h->prep_valid = false;
      ensure_prep(h);
      h->eng->launch_step(false, nullptr, nullptr);
      std::vector<cudaEvent_t> evs(h->ev_pool.begin(), h->ev_pool.begin() + nev);
      size_t pos = 0;
      for (int i = 0; i < steps; ++i) h->eng->launch_step(false, &evs, &pos);
      if ((rc = sync(h, "tmc_autotune"))) break;
      // a block size whose launches were refused (its events would time
      // nothing) is not a candidate
      if (cudaGetLastError() != cudaSuccess) continue;
      double sum = 0.0;
      for (size_t k = 0; k + 1 < pos; k += 2) {
        float dt = 0.f;
        cudaEventElapsedTime(&dt, evs[k], evs[k + 1]);
        sum += dt;
      }
      if (sum < best) {
        best = sum;
        best_bs = c;
      }
    }
    if (rc) break;
    h->bsp[pass] = best_bs;
  }
  h->timed_pass = saved_timed;
  set_counts(h);
  // restore the state and drop the graphs captured with the old block sizes
  cudaMemcpyAsync(gd0, sv_gd, b_gd, cudaMemcpyDeviceToDevice, h->st);
  cudaMemcpyAsync(iap0, sv_iap, b_iap, cudaMemcpyDeviceToDevice, h->st);
  if (q0) cudaMemcpyAsync(q0, sv_q, b_q, cudaMemcpyDeviceToDevice, h->st);
  h->eng->refresh_all_shadows();
  h->prep_valid = false;
  int rc2 = sync(h, "tmc_autotune");
  cudaFree(sv_gd);
  cudaFree(sv_iap);
  cudaFree(sv_q);
  h->drop_graphs();
  if (rc) return rc;
  if (rc2) return rc2;
  if (block_sizes)
    for (int k = 0; k < P_COUNT; ++k) block_sizes[k] = h->bsp[k];
  return h->cuda_check("tmc_autotune");
}

}  // extern "C"

// A group of handles (different meshes, each possibly an ensemble) advanced
// together: one CUDA graph per cycle of `cycle_seconds`.
//   mode 0: one branch per handle that runs cycle_seconds / dt steps of that
//           handle; the branches are independent, so the levels' kernels
//           overlap on the GPU.
//   mode 1: one launch per pass over every handle (member-innermost
//           ensembles of one member count and pv scheme).  The handles are
//           ordered by steps per cycle, most first; sub-step s of a cycle
//           advances the handles with more than s steps per cycle, each pass
//           one launch over all their element blocks (ens::launch_jobs_step).
struct tmc_group {
  std::vector<tmc_handle*> hs;
  std::vector<int> steps;  // per handle and cycle
  int mode = 0;
  std::unique_ptr<tmc::ens::JobTable> jobs;  // mode 1: the job table (the kernels' parameter)
  std::vector<int> order;                    // mode 1: handles by steps per cycle, most first
  int big = 0;                               // mode 1: the job whose block sizes the launches use
  cudaStream_t st = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_done = nullptr;
  std::vector<cudaEvent_t> ev_join;
  // mode 1: the stages' vertex and pv-on-edge passes beside the cell pass
  cudaStream_t side = nullptr;
  cudaEvent_t side_fork = nullptr, side_join = nullptr;
  cudaGraphExec_t graph = nullptr;
  std::string err;
};

namespace {

// mode 1: checks, and the job table (g->jobs); returns TMC_OK or an error
// with g->err set
int prepare_batched(tmc_group* g) {
  using namespace tmc::ens;
  const int n = (int)g->hs.size();
  if (n > kMaxJobs) {
    g->err = "tmc_group_create_ex: mode 1 takes at most " + std::to_string(kMaxJobs) + " handles";
    return TMC_E_UNSUP;
  }
  const tmc_handle* h0 = g->hs[0];
  for (const tmc_handle* h : g->hs) {
    if (h->p.member_layout != 1) {
      g->err = "tmc_group_create_ex: mode 1 runs member-innermost ensembles (member_layout 1)";
      return TMC_E_UNSUP;
    }
    const EnsEngine* e = static_cast<const EnsEngine*>(h->eng.get());
    const EnsEngine* e0 = static_cast<const EnsEngine*>(h0->eng.get());
    if (h->members != h0->members || h->p.pv_scheme != h0->p.pv_scheme || e->D.V != e0->D.V ||
        e->D.LPE != e0->D.LPE) {
      g->err = "tmc_group_create_ex: mode 1 needs one member count, lane layout and pv scheme for all handles";
      return TMC_E_UNSUP;
    }
    if (h->closure) {
      g->err = "tmc_group_create_ex: mode 1 runs without the learned closure";
      return TMC_E_UNSUP;
    }
  }
  std::vector<int>& order = g->order;
  order.resize(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return g->steps[a] > g->steps[b]; });
  auto T = std::make_unique<JobTable>();
  std::memset(T.get(), 0, sizeof(JobTable));
  T->n = n;
  int big = 0;  // the handle with the most edges lends its block sizes
  for (int j = 0; j < n; ++j) {
    tmc_handle* h = g->hs[order[j]];
    const EnsEngine* e = static_cast<const EnsEngine*>(h->eng.get());
    Job& J = T->job[j];
    J.Mh = h->M;
    J.D = e->D;
    for (int k = 0; k <= 4; ++k) {
      J.io[k] = e->io(k);
      if (k >= 1) J.io[k].vor = J.io[k].gd_v = nullptr;  // kept only by the diagnostic pass
    }
    J.P = e->EP;
    if (e->upwind()) J.up = *e->upwind();
    J.diag = h->d_diag;
    J.dt = h->O.dt;
    J.totalArea = h->hm.totalArea;
    J.sumAreaTriangle = h->hm.sumAreaTriangle;
    J.conserve = h->p.conserve_energy != 0;
    T->off[J_CELLS][j + 1] = T->off[J_CELLS][j] + e->D.slots_c;
    T->off[J_EDGES][j + 1] = T->off[J_EDGES][j] + e->D.slots_e;
    T->off[J_VERTS][j + 1] = T->off[J_VERTS][j] + e->D.slots_v;
    T->off[J_EDGES_UP][j + 1] = T->off[J_EDGES_UP][j] + ens::slots_up(h->M.ne);
    if (h->M.ne > g->hs[order[big]]->M.ne) big = j;
  }
  g->jobs = std::move(T);
  g->big = big;
  return TMC_OK;
}

// mode 1: one cycle into the group's stream (capturing)
void capture_batched(tmc_group* g) {
  const int n = (int)g->hs.size();
  const int* bsp = g->hs[g->order[g->big]]->bsp;
  const bool upwind = g->hs[0]->p.pv_scheme == 3;
  const int nsub = g->steps[g->order[0]];
  for (int s = 0; s < nsub; ++s) {
    int nj = 0;
    while (nj < n && g->steps[g->order[nj]] > s) ++nj;
    tmc::ens::launch_jobs_step(*g->jobs, nj, bsp, upwind, g->st, g->side, g->side_fork, g->side_join);
  }
}

}  // namespace

extern "C" {

int tmc_group_create(tmc_handle* const* handles, int32_t n, double cycle_seconds, tmc_group** out) {
  return tmc_group_create_ex(handles, n, cycle_seconds, 0, out);
}

int tmc_group_create_ex(tmc_handle* const* handles, int32_t n, double cycle_seconds, int32_t mode, tmc_group** out) {
  if (!out || !handles || n <= 0 || !(cycle_seconds > 0.0) || mode < 0 || mode > 1) return TMC_E_ARG;
  *out = nullptr;
  auto g = std::make_unique<tmc_group>();
  g->mode = mode;
  for (int i = 0; i < n; ++i) {
    tmc_handle* h = handles[i];
    if (!h || !h->eng) return TMC_E_ARG;
    if (h->generic) {
      h->err = "tmc_group_create: groups run the fused CRK4 shallow-water step";
      return TMC_E_UNSUP;
    }
    if (!h->have_state) {
      h->err = "tmc_group_create: set the state first";
      return TMC_E_STATE;
    }
    const double k = cycle_seconds / h->O.dt;
    const int ki = (int)(k + 0.5);
    if (ki < 1 || std::fabs(k - ki) > 1e-9 * k) {
      h->err = "tmc_group_create: cycle_seconds must be a whole number of this handle's dt";
      return TMC_E_ARG;
    }
    for (tmc_handle* o : g->hs)
      if (o == h) return TMC_E_ARG;
    g->hs.push_back(h);
    g->steps.push_back(ki);
  }
  auto cerr = [&](const char* where) {
    cudaError_t e = cudaGetLastError();
    g->err = std::string(where) + ": " + cudaGetErrorString(e);
    *out = g.release();
    return TMC_E_CUDA;
  };
  if (cudaStreamCreateWithFlags(&g->st, cudaStreamNonBlocking) != cudaSuccess) return cerr("cudaStreamCreate");
  if (cudaEventCreateWithFlags(&g->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&g->ev_done, cudaEventDisableTiming) != cudaSuccess)
    return cerr("cudaEventCreate");
  g->ev_join.resize(n);
  for (auto& e : g->ev_join)
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return cerr("cudaEventCreate");
  // every handle's edge preparation is current before capture
  for (tmc_handle* h : g->hs) {
    ensure_prep(h);
    if (cudaStreamSynchronize(h->st) != cudaSuccess) return cerr("cudaStreamSynchronize");
  }
  if (mode == 1) {
    const int rc = prepare_batched(g.get());
    if (rc != TMC_OK) {
      *out = g.release();
      return rc;
    }
    if (cudaStreamCreateWithFlags(&g->side, cudaStreamNonBlocking) != cudaSuccess) return cerr("cudaStreamCreate");
    if (cudaEventCreateWithFlags(&g->side_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&g->side_join, cudaEventDisableTiming) != cudaSuccess)
      return cerr("cudaEventCreate");
  }
  cudaGraph_t graph = nullptr;
  if (cudaStreamBeginCapture(g->st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return cerr("BeginCapture");
  if (mode == 1) {
    capture_batched(g.get());
  } else {
    cudaEventRecord(g->ev_fork, g->st);
    for (int i = 0; i < n; ++i) {
      tmc_handle* h = g->hs[i];
      cudaStreamWaitEvent(h->st, g->ev_fork, 0);
      for (int k = 0; k < g->steps[i]; ++k) h->eng->launch_step(false, nullptr, nullptr);
      cudaEventRecord(g->ev_join[i], h->st);
      cudaStreamWaitEvent(g->st, g->ev_join[i], 0);
    }
  }
  if (cudaStreamEndCapture(g->st, &graph) != cudaSuccess) return cerr("EndCapture");
  cudaError_t e = cudaGraphInstantiate(&g->graph, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cerr("cudaGraphInstantiate");
  *out = g.release();
  return TMC_OK;
}

int tmc_group_run(tmc_group* g, int32_t cycles) {
  if (!g || !g->graph || cycles < 0) return TMC_E_ARG;
  // the group's stream starts after all work already queued on the handles
  for (size_t i = 0; i < g->hs.size(); ++i) {
    cudaEventRecord(g->ev_join[i], g->hs[i]->st);
    cudaStreamWaitEvent(g->st, g->ev_join[i], 0);
  }
  for (int c = 0; c < cycles; ++c)
    if (cudaGraphLaunch(g->graph, g->st) != cudaSuccess) {
      g->err = std::string("cudaGraphLaunch: ") + cudaGetErrorString(cudaGetLastError());
      return TMC_E_CUDA;
    }
  // later calls on each handle are ordered after the group's work
  cudaEventRecord(g->ev_done, g->st);
  for (size_t i = 0; i < g->hs.size(); ++i) {
    cudaStreamWaitEvent(g->hs[i]->st, g->ev_done, 0);
    g->hs[i]->step_count += (long)g->steps[i] * cycles;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    g->err = cudaGetErrorString(e);
    return TMC_E_CUDA;
  }
  return TMC_OK;
}

int tmc_group_synchronize(tmc_group* g) {
  if (!g) return TMC_E_ARG;
  cudaError_t e = cudaStreamSynchronize(g->st);
  if (e != cudaSuccess) {
    g->err = cudaGetErrorString(e);
    return TMC_E_CUDA;
  }
  return TMC_OK;
}

const char* tmc_group_last_error(const tmc_group* g) { return g ? g->err.c_str() : "null group"; }

int tmc_group_destroy(tmc_group* g) {
  if (!g) return TMC_OK;
  if (g->st) cudaStreamSynchronize(g->st);
  if (g->graph) cudaGraphExecDestroy(g->graph);
  for (cudaEvent_t e : g->ev_join) cudaEventDestroy(e);
  if (g->ev_fork) cudaEventDestroy(g->ev_fork);
  if (g->ev_done) cudaEventDestroy(g->ev_done);
  if (g->side_fork) cudaEventDestroy(g->side_fork);
  if (g->side_join) cudaEventDestroy(g->side_join);
  if (g->side) cudaStreamDestroy(g->side);
  if (g->st) cudaStreamDestroy(g->st);
  delete g;
  return TMC_OK;
}

int tmc_sizes(const tmc_handle* h, int64_t* nc, int64_t* ne, int64_t* nv, int64_t* bytes) {
  if (!h) return TMC_E_ARG;
  if (nc) *nc = h->M.nc;
  if (ne) *ne = h->M.ne;
  if (nv) *nv = h->M.nv;
  if (bytes) *bytes = (int64_t)h->dbytes;
  return TMC_OK;
}

}  // extern "C"
