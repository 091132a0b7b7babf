// Member-innermost ensembles (tmc_params.member_layout = 1).
//
// M members of one mesh (M a multiple of 16) are stored member-innermost:
// element i of member m sits at [i * M + m].  A warp owns 32 consecutive
// members of one element at a time, so every neighbour gather of a warp is
// one 128-byte line (FP32) and every mesh index or metric it needs is the
// same for all its lanes.  A block covers one member group and kEnsEPB
// consecutive elements; it first stages those elements' stencils (indices,
// signs, weights, metrics) in shared memory, then its W warps take elements
// w, w + W, ..., so that they work on neighbouring elements together and
// share the neighbours' lines in L1.  The arithmetic is that of the FP32
// single-model kernels (tmc_kernels_impl.cuh) in the same expression order
// (FP32 edge and vertex state, the gd tendency from an FP32 two-sum flux
// divergence), except that gd and its RK accumulation are double-float
// (see IO) instead of FP64.
//
// Global sums: the warps of a block combine their lanes' sums in shared
// memory, and lane m of warp 0 stores member m's partial sum of the block,
// [region][slot][M] (coalesced across the warp).  The CRK4 inner products are FP32 partials
// combined with FP32 two-sum arithmetic; the invariants are FP64 partials.
// k_ens_reduce sums the slots of one region for 32 members per block and
// k_ens_beta forms beta and the invariants per member into the per-member
// diag block that the member-outermost path also uses.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "tmc_kernels.cuh"

namespace tmc {
namespace ens {

// elements per block: on 512 level-6 members 64 -> 4.92 ms per step, 128 -> 4.91, 32 -> 5.12;
// on the 16-member level-7 ensemble of the mixed batch 64 -> 7.55-7.71 ms per
// 1200-s cycle, 128 -> 7.17
#ifndef TMC_ENS_EPB
#define TMC_ENS_EPB 128
#endif
constexpr int kEnsEPB = TMC_ENS_EPB;  // elements per block (and per partial-sum slot)

struct Dims {
  int M;    // members (a multiple of 16)
  int G;    // groups of 32 members for the reductions (the last may be partial)
  int V;    // members per lane (lanes_for)
  int LPE;  // lanes per element (lanes_for)
  int slots_c, slots_e, slots_v;  // partial slots: blocks along cells, edges, vertices
};

// Members per lane and lanes per element for M members (M a multiple of 16).
// lanes 0 (automatic): 2 and 32 when M is a multiple of 64, else 1 and 32 (M
// a multiple of 32) or 16.  lanes 8, 16 or 32: that many lanes per element,
// two members per lane when M is a multiple of 2 x lanes, else one.  Returns
// false when M is not a multiple of lanes.  Four members per lane (16-byte
// loads, 4 or 8 lanes per element) made a 16-member level-7 step 2.4x slower
// (2.87 against 1.20 ms): a warp then gathers from 8 elements at once.
inline bool lanes_for(int M, int lanes, int* V, int* LPE) {
  if (lanes == 0) {
    *V = M % 64 == 0 ? 2 : 1;
    *LPE = M % 32 == 0 ? 32 : 16;
    return true;
  }
  if ((lanes != 8 && lanes != 16 && lanes != 32) || M % lanes != 0) return false;
  *LPE = lanes;
  *V = M % (2 * lanes) == 0 ? 2 : 1;
  return true;
}

__host__ __device__ inline int slots_for(int n) { return (n + kEnsEPB - 1) / kEnsEPB; }

// Per-thread partial sums: step regions R_IP_C..R_44_E (FP32) and invariant
// regions R_MASS..R_AV (FP64), each [slots][M].
struct Partials {
  float* sf;   // [R_44_E + 1][cap][M]
  double* sd;  // [R_AV - R_MASS + 1][cap][M]
  int cap;     // slots per region
  int M;
  __host__ __device__ float* f(int r, int slot) const { return sf + ((size_t)r * cap + slot) * M; }
  __host__ __device__ double* d(int r, int slot) const { return sd + ((size_t)(r - R_MASS) * cap + slot) * M; }
};

// Buffers of one CRK4 stage, all member-innermost.  gd and its RK
// accumulator are double-float (FF) values h + l in two FP32 halves of one
// array, h for every element first, then l at offset `ffs` (nCells * M): the
// h half is the FP32 value of gd the stencils read, the pair keeps about 48
// significant bits, and all gd arithmetic runs on the FP32 pipes (GB300
// issues FP64 at 1/64 of the FP32 rate).
struct IO {
  const float* gd_in;
  const float* gd_old;
  float* gd_next;
  float* gd_acc;
  const float* iap_in;
  const float* iap_old;
  float* iap_next;
  float* iap_acc;
  float* iap_tend;
  float* tendf;
  const float* ghsf;
  const float* gd_e;
  const float* u;
  const float* F;
  float* gd_e_nx;  // the next stage's edge set (stages 1-3), null: not fused
  float* u_nx;
  float* F_nx;
  float* E;
  float* pv_v;
  float* vor;   // null: not kept
  float* gd_v;  // null: not kept
  float* pv_e;
  const float* cdv;      // dvEdge of edgesOnCell: [6][nCells] (FP32)
  const float* cae;      // areaEdge of edgesOnCell: [6][nCells] (FP32)
  const float* vdc;      // dcEdge of edgesOnVertex: [3][nVertices] (FP32)
  const float* invA_hl;  // 1 / areaCell as FF: [2][nCells]
  const float* A_hl;     // areaCell as FF: [2][nCells]
  size_t ffs;            // offset of the l halves (nCells * M)
};

// passes of the fused CRK4 step (bs: threads per block, a multiple of 32);
// launch_cell with rk.mode 0 computes E only (no RK update)
void launch_cell(const DevMesh& Mh, const Dims& D, const IO& S, RKStage rk, const Partials& P, bool diag, int bs,
                 cudaStream_t st);
void launch_vertex(const DevMesh& Mh, const Dims& D, const IO& S, const Partials& P, bool diag, int bs,
                   cudaStream_t st);
// Upwind pv on edges (pv_scheme 3, interp_pv_order 3 or 4): the two-sided
// vertex fit stencils of the edges, [width][2][nEdges] as DStencil, with FP32
// weights; width at most kUpW.
constexpr int kUpW = 16;
// edges per block of the upwind pv pass: its stencils take kUpW x 2 entries
// per edge, and blocks of kEnsEPB edges would cost it a resident block per SM
// (512 level-6 members: 0.43-0.46 ms per pass with 64, 0.55 with 128)
constexpr int kUpEPB = 64;
__host__ __device__ inline int slots_up(int n) { return (n + kUpEPB - 1) / kUpEPB; }
struct Upwind {
  const uint8_t* count;  // [2][nEdges]
  const int32_t* idx;    // [width][2][nEdges]
  const float* w;        // [width][2][nEdges]
  int width;
  float coef2;           // 1 for order 3, 0 for order 4
};
// centred pv (up null) or upwind pv on edges
void launch_edge_pv(const DevMesh& Mh, const Dims& D, const IO& S, const Upwind* up, int bs, cudaStream_t st);
void launch_edge_flux(const DevMesh& Mh, const Dims& D, const IO& S, RKStage rk, const Partials& P, int bs,
                      cudaStream_t st);
// new = old + beta dt t_new for cells, then edges with the edge preparation
// of the next step's first stage and the edge energy of the new state
void launch_final(const DevMesh& Mh, const Dims& D, const IO& S, const double* diag, const Partials& P, int bs,
                  cudaStream_t st);
// edge preparation of slot S.gd_in / S.iap_in into S.gd_e/u/F (+ edge energy)
void launch_edge_prep(const DevMesh& Mh, const Dims& D, const IO& S, const Partials& P, bool diag, int bs,
                      cudaStream_t st);
// mass and the cell part of the energy of S.gd_in (the diagnostic pass)
void launch_cell_diag(const DevMesh& Mh, const Dims& D, const IO& S, const Partials& P, int bs, cudaStream_t st);
// region sums, beta (CRK4) and invariants into diag[m * kDiagStride + ...]
void launch_finalize(const Dims& D, const Partials& P, bool step, bool diag, bool conserve, double totalArea,
                     double sumAreaTriangle, double dt, double* diag_out, cudaStream_t st);

// ---------------------------------------------------------------------------
// Batches: the member-innermost ensembles of several meshes (different
// resolutions and time steps, the same member count and pv scheme) advanced
// by one launch per pass.  A batch kernel's blocks are the concatenation of
// every active mesh's element blocks along one element kind; block b finds
// its mesh j from the block offsets (off[kind][j] <= b < off[kind][j + 1])
// and runs the same per-block body as the single-mesh kernel on mesh j's
// tables and buffers.  The table (14 KB) is the kernels' __grid_constant__
// parameter: a block reads its mesh's pointers from the constant bank as it
// needs them instead of holding them in registers.  The first nj jobs
// are active in a launch (the host orders the meshes by steps per cycle,
// most first, so every sub-step's active set is a prefix).
// ---------------------------------------------------------------------------
constexpr int kMaxJobs = 8;
// J_EDGES_UP: the edges in the upwind pv pass's blocks of kUpEPB
enum JobKind { J_CELLS = 0, J_EDGES = 1, J_VERTS = 2, J_EDGES_UP = 3 };
struct Job {
  DevMesh Mh;
  Dims D;
  IO io[5];  // the buffers of CRK4 stage k (1-4) and of the final update (0)
  Partials P;
  Upwind up;     // upwind pv tables (width 0: centred pv)
  double* diag;  // per-member diag blocks (beta dt of the step at [m * kDiagStride + 9])
  double dt, totalArea, sumAreaTriangle;
  int conserve;
};
struct JobTable {
  int n;
  int off[4][kMaxJobs + 1];  // first block of each job along each JobKind
  Job job[kMaxJobs];
};
// What the pass kernels of one CRK4 stage (or of the final update, k = 0)
// read of each job: that stage's buffers only, so that every pointer sits at
// a fixed offset of the kernel parameter
struct JobStage {
  DevMesh Mh;
  Dims D;
  IO io;
  Partials P;
  Upwind up;
  double* diag;
  double dt;
};
struct StageTable {
  int off[4][kMaxJobs + 1];
  JobStage job[kMaxJobs];
};
// both are kernel parameters (__grid_constant__), whose size CUDA caps
static_assert(sizeof(JobTable) <= 32764 && sizeof(StageTable) <= 32764, "job tables exceed the kernel parameter limit");
// one CRK4 step of the first nj jobs of T; bsp: block sizes of the cell,
// vertex, edge_pv, edge_flux and final passes; upwind: the jobs run upwind pv.
// With a side stream (and two events for the fork and the join) each stage's
// vertex and pv-on-edge passes run on it beside the cell pass: they read only
// the stage's input gd and edge set, and the cell pass reads nothing they write.
void launch_jobs_step(const JobTable& T, int nj, const int* bsp, bool upwind, cudaStream_t st,
                      cudaStream_t side = nullptr, cudaEvent_t fork = nullptr, cudaEvent_t join = nullptr);

// The learned PV-on-edge closure (after the pv-on-edge pass): pv on cells
// (the network reads it), then the network on rows [edge][member] with its
// output added to pv_edge of members whose switch is on (a.mode 0 every stage;
// 1 stage 1, output also held in a.dq; 2 add the held a.dq only)
void launch_v2c(const DevMesh& Mh, const Dims& D, const IO& S, float* pv_c, cudaStream_t st);
void launch_closure_hold(const DevMesh& Mh, const Dims& D, const IO& S, const float* dq, cudaStream_t st);
void launch_closure(const DevMesh& Mh, const Dims& D, const IO& S, const float* pv_c, const ClosureArgs& a,
                    cudaStream_t st);
// the closure's features and pv_edge of member m (internal edge order) into feat[ne][24], pv[ne]
void launch_closure_features(const DevMesh& Mh, const Dims& D, const IO& S, const float* pv_c, int m, float* feat,
                             float* pv, cudaStream_t st);

// state transfer of member m (caller's element order <-> member-innermost);
// _ff: an FF array (h, then l at offset n * M)
void launch_gather_f64(int n, int M, int m, const double* raw, const int32_t* n2o, double* dst, cudaStream_t st);
void launch_gather_f32(int n, int M, int m, const double* raw, const int32_t* n2o, float* dst, cudaStream_t st);
void launch_gather_ff(int n, int M, int m, const double* raw, const int32_t* n2o, float* dst, cudaStream_t st);
void launch_scatter_f32(int n, int M, int m, const float* src, const int32_t* n2o, double* raw, cudaStream_t st);
void launch_scatter_ff(int n, int M, int m, const float* src, const int32_t* n2o, double* raw, cudaStream_t st);
// member m of a member-innermost array into a contiguous FP64 array (internal order)
void launch_extract_f64(int n, int M, int m, const double* src, double* dst, cudaStream_t st);
void launch_extract_f32(int n, int M, int m, const float* src, double* dst, cudaStream_t st);
void launch_extract_ff(int n, int M, int m, const float* src, double* dst, cudaStream_t st);
// iap_u of member m = sqrt(gd_edge) u (internal order inputs)
void launch_iap_from_u(int ne, int M, int m, const double* gd_e, const double* u, float* iap, cudaStream_t st);
// FP32 copy of member m's FP64 array of n elements (m < 0: every member)
void launch_to_f32(int n, int M, int m, const double* src, float* dst, cudaStream_t st);

}  // namespace ens
}  // namespace tmc
