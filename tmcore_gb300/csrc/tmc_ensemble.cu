// Member-innermost ensemble kernels (see tmc_ensemble.cuh).  FP32 path,
// CRK4 (time_scheme_mod.F90:109-154), centred pv on edges (APVM weight 0,
// operators_mod.F90:296-316), second-order gd on edges, no tracers.
//
// Thread layout of every pass: blockIdx.x = kEnsEPB consecutive elements (kUpEPB
// edges in the upwind pv pass)
// (space-filling-curve order), blockIdx.y = a group of 32 V members, lane l
// = members (32 blockIdx.y + l) V ... + V - 1 (V = 2 when the member count
// is a multiple of 64: a lane's two members are one 8-byte load, and the
// index, shared-memory and address work of an element is shared by both).
// The block stages the stencils of its elements in shared memory; its W
// warps then take elements w, w + W, ..., neighbouring elements at the same
// time, and every neighbour gather of a warp reads whole 128-byte lines.
#include <cuda_runtime.h>

#include <cstring>

#include "tmc_ensemble.cuh"

// Minimum resident blocks per SM the heavy passes are compiled for (0: none
// given).  Any minimum changes the compiler's register heuristics: on 512
// level-6 members, 1 (flux 96, cell 110 registers with two members per
// lane) measured 4.87 ms per step, none 5.07, 3 4.94, flux 4 (64 registers,
// spilled) 5.50; vertex 4 (64 registers against 71, 44 bytes of spill
// loads) 125.7 against 122.7 us per launch.
#ifndef TMC_ENS_FLUX_MINB
#define TMC_ENS_FLUX_MINB 1
#endif
#ifndef TMC_ENS_CELL_MINB
#define TMC_ENS_CELL_MINB 1
#endif
#ifndef TMC_ENS_VERT_MINB
#define TMC_ENS_VERT_MINB 1
#endif
// with one member per lane the flux pass needs 69 registers; a minimum of 4
// resident blocks of 256 threads caps it at 64 without spills: 16 level-7
// members 121.1 against 125.6 us per launch (the cell pass, capped the same
// way from 66 registers, went from 52.5 to 54.6 us and is not capped)
#ifndef TMC_ENS_MINB_V1
#define TMC_ENS_MINB_V1 4
#endif
// vertices per warp iteration of the vertex pass (512 level-6 members:
// 2 -> 4.85 ms per step, 1 -> 4.86, 4 -> 4.89)
#ifndef TMC_ENS_VU
#define TMC_ENS_VU 2
#endif
// members per lane of the upwind pv kernel: 4 (when M is a multiple of 128),
// else the ensemble's V.  It issues more instructions per member than it
// moves bytes: on 512 level-6 members its pass takes 0.45 ms with 4, 0.64 ms
// with 2 and 0.61 ms with 8 (two float4 loads per gather)
#ifndef TMC_ENS_UP_V
#define TMC_ENS_UP_V 4
#endif
#define TMC_ENS_LB_0 __launch_bounds__(256)
#define TMC_ENS_LB_1 __launch_bounds__(256, 1)
#define TMC_ENS_LB_2 __launch_bounds__(256, 2)
#define TMC_ENS_LB_3 __launch_bounds__(256, 3)
#define TMC_ENS_LB_4 __launch_bounds__(256, 4)
#define TMC_ENS_LB_(n) TMC_ENS_LB_##n
#define TMC_ENS_LB(n) TMC_ENS_LB_(n)

namespace tmc {
namespace ens {

namespace {

constexpr int kME = 6;    // edges per cell (padded slots: sign 0)
constexpr int kME2 = 10;  // edges per edge (padded slots: weight 0)
constexpr int kMaxBS = 256;

// FP32 error-free addition (Knuth TwoSum): hi + lo accumulates p exactly
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float p) {
  const float t = __fadd_rn(hi, p);
  const float bp = __fsub_rn(t, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, bp)), __fsub_rn(p, bp));
  hi = t;
  lo = __fadd_rn(lo, err);
}

struct DD {
  double hi, lo;
};
__device__ __forceinline__ DD dd_add(DD a, DD b) {
  const double s = __dadd_rn(a.hi, b.hi);
  const double bb = __dsub_rn(s, a.hi);
  double e = __dadd_rn(__dsub_rn(a.hi, __dsub_rn(s, bb)), __dsub_rn(b.hi, bb));
  e = __dadd_rn(e, __dadd_rn(a.lo, b.lo));
  const double hi = __dadd_rn(s, e);
  return {hi, __dsub_rn(e, __dsub_rn(hi, s))};
}

// Double-float (FF) arithmetic for gd: a value h + l with |l| <= ulp(h) / 2.
// Error-free transforms (Knuth TwoSum; the FMA product error) with explicit
// rounding, so the compiler cannot contract them.
struct FF {
  float h, l;
};
__device__ __forceinline__ FF ff_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
  const FF s = ff_two_sum(a.h, b.h);
  return ff_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ FF ff_mul(FF a, FF b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return ff_two_sum(p, e);
}
__host__ __device__ __forceinline__ FF ff_from(double x) {
  const float h = (float)x;
  return {h, (float)(x - (double)h)};
}
__device__ __forceinline__ double ff_to_double(FF a) { return (double)a.h + (double)a.l; }

// V consecutive members of one element: one load / store of V * 4 (or 8) bytes
template <int V>
__device__ __forceinline__ void ldv(const float* p, size_t i, float (&o)[V]) {
  if constexpr (V == 4) {
    const float4 t = *reinterpret_cast<const float4*>(p + i);
    o[0] = t.x;
    o[1] = t.y;
    o[2] = t.z;
    o[3] = t.w;
  } else if constexpr (V == 2) {
    const float2 t = *reinterpret_cast<const float2*>(p + i);
    o[0] = t.x;
    o[1] = t.y;
  } else {
    o[0] = p[i];
  }
}
template <int V>
__device__ __forceinline__ void ldv(const double* p, size_t i, double (&o)[V]) {
  if constexpr (V == 4) {
    const double2 a = *reinterpret_cast<const double2*>(p + i), b = *reinterpret_cast<const double2*>(p + i + 2);
    o[0] = a.x;
    o[1] = a.y;
    o[2] = b.x;
    o[3] = b.y;
  } else if constexpr (V == 2) {
    const double2 t = *reinterpret_cast<const double2*>(p + i);
    o[0] = t.x;
    o[1] = t.y;
  } else {
    o[0] = p[i];
  }
}
template <int V>
__device__ __forceinline__ void stv(float* p, size_t i, const float (&v)[V]) {
  if constexpr (V == 4)
    *reinterpret_cast<float4*>(p + i) = make_float4(v[0], v[1], v[2], v[3]);
  else if constexpr (V == 2)
    *reinterpret_cast<float2*>(p + i) = make_float2(v[0], v[1]);
  else
    p[i] = v[0];
}
template <int V>
__device__ __forceinline__ void stv(double* p, size_t i, const double (&v)[V]) {
  if constexpr (V == 4) {
    *reinterpret_cast<double2*>(p + i) = make_double2(v[0], v[1]);
    *reinterpret_cast<double2*>(p + i + 2) = make_double2(v[2], v[3]);
  } else if constexpr (V == 2)
    *reinterpret_cast<double2*>(p + i) = make_double2(v[0], v[1]);
  else
    p[i] = v[0];
}

template <int V>
__device__ __forceinline__ void ldff(const float* p, size_t i, size_t ffs, FF (&o)[V]) {
  float h[V], l[V];
  ldv<V>(p, i, h);
  ldv<V>(p + ffs, i, l);
#pragma unroll
  for (int c = 0; c < V; ++c) o[c] = FF{h[c], l[c]};
}
template <int V>
__device__ __forceinline__ void stff(float* p, size_t i, size_t ffs, const FF (&v)[V]) {
  float h[V], l[V];
#pragma unroll
  for (int c = 0; c < V; ++c) h[c] = v[c].h, l[c] = v[c].l;
  stv<V>(p, i, h);
  stv<V>(p + ffs, i, l);
}

// This thread's members and elements.  One block = one member group
// (blockIdx.y) and kEnsEPB consecutive elements (blockIdx.x).  A warp covers
// 32 / LPE elements at a time, LPE lanes each (LPE = 32, 16, 8 or 4; see
// Dims): its warps take elements j0, j0 + js, ...
struct Lane {
  int m0;      // first member of the lane
  size_t M;    // member stride
  int j0, js;  // first element and element stride of the thread
  int slot, nslot;  // this thread's row of a block reduction, and the rows
  int ml;      // member lane (0 .. LPE-1)
  int lpe;     // lanes per element
};
template <int V>
__device__ __forceinline__ Lane lane_of(const Dims& D) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, W = blockDim.x >> 5;
  const int epw = 32 / D.LPE, sub = lane / D.LPE, ml = lane % D.LPE;
  return Lane{(int)((blockIdx.y * D.LPE + ml) * V), (size_t)D.M, w * epw + sub, W * epw, w * epw + sub, W * epw, ml,
              D.LPE};
}

inline dim3 grid_of(int n, const Dims& D, int bs, int* threads) {
  int W = bs / 32;
  if (W < 1) W = 1;
  if (W > kMaxBS / 32) W = kMaxBS / 32;
  *threads = W * 32;
  return dim3((unsigned)slots_for(n), (unsigned)(D.M / (D.LPE * D.V)));
}

// Per-member partial sums of one block: the rows (warps and the element
// groups of a warp) of each member are combined in a fixed order (FP32
// TwoSum here, double-float in block_partials_ff) and row 0 stores them.  Entry (row, member lane) sits at
// row * LPE + lane: rows x LPE = the block's threads.  Every thread of the
// block calls these (they synchronise).
template <int N, int V>
__device__ __forceinline__ void block_partials_f(const Lane& L, const float (&v)[N][V], float* const (&dst)[N]) {
  __shared__ float sh[N][V][kMaxBS];
  const int at = L.slot * L.lpe + L.ml;
#pragma unroll
  for (int k = 0; k < N; ++k)
#pragma unroll
    for (int c = 0; c < V; ++c) sh[k][c][at] = v[k][c];
  __syncthreads();
  if (L.slot == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) {
      if (!dst[k]) continue;
      float o[V];
#pragma unroll
      for (int c = 0; c < V; ++c) {
        float hi = 0.f, lo = 0.f;
        for (int q = 0; q < L.nslot; ++q) two_sum_acc(hi, lo, sh[k][c][q * L.lpe + L.ml]);
        o[c] = hi + lo;
      }
      stv<V>(dst[k], (size_t)L.m0, o);
    }
  }
  __syncthreads();
}
// The same for sums held as double-float pairs (compensated FP32 sums, or
// FF values): the rows are combined in FF arithmetic on the FP32 pipes and
// row 0 converts each member's pair to FP64 once.  Converting every thread's
// pair and adding the rows in FP64 cost about 130 FP64 instructions per block
// (each one warp-wide on GB300's 2-lane FP64 pipe, 16 cycles): on the
// invariant stage that made the vertex pass of 256 level-6 members 115 us
// against 78 us on the other stages.
template <int N, int V>
__device__ __forceinline__ void block_partials_ff(const Lane& L, const FF (&v)[N][V], double* const (&dst)[N]) {
  __shared__ float shh[N][V][kMaxBS], shl[N][V][kMaxBS];
  const int at = L.slot * L.lpe + L.ml;
#pragma unroll
  for (int k = 0; k < N; ++k)
#pragma unroll
    for (int c = 0; c < V; ++c) shh[k][c][at] = v[k][c].h, shl[k][c][at] = v[k][c].l;
  __syncthreads();
  if (L.slot == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) {
      double o[V];
#pragma unroll
      for (int c = 0; c < V; ++c) {
        FF a{0.f, 0.f};
        for (int q = 0; q < L.nslot; ++q) a = ff_add(a, FF{shh[k][c][q * L.lpe + L.ml], shl[k][c][q * L.lpe + L.ml]});
        o[c] = ff_to_double(a);
      }
      stv<V>(dst[k], (size_t)L.m0, o);
    }
  }
  __syncthreads();
}

// Edge preparation of one edge (operators_mod.F90:93-104 c2e, :168-176
// inverse IAP; mass flux u gd_edge, tmcore_swm_mod.F90:135), the FP32
// single-model arithmetic.
__device__ __forceinline__ void prep1(float ia, float g1, float g2, float& ge, float& uu, float& Fv) {
  ge = 0.5f * (g1 + g2);
  const float sq = sqrtf(ge);
  uu = ia / sq;
  Fv = uu * ge;
}
template <int V>
__device__ __forceinline__ void prep(const float (&ia)[V], const float (&g1)[V], const float (&g2)[V], float* gd_e,
                                     float* u, float* F, size_t em) {
  float ge[V], uu[V], Fv[V];
#pragma unroll
  for (int c = 0; c < V; ++c) prep1(ia[c], g1[c], g2[c], ge[c], uu[c], Fv[c]);
  stv<V>(gd_e, em, ge);
  stv<V>(u, em, uu);
  stv<V>(F, em, Fv);
}

// ---------------------------------------------------------------------------
// cell: div of the mass flux (FP32 two-sum -> FP64 tendency), kinetic energy,
// E = ke + gd + ghs, RK update of gd (div_operator operators_mod.F90:40-55,
// calc_kinetic_energy :206-221, calc_gd_tend_on_cell tmcore_swm_mod.F90:127-139)
// ---------------------------------------------------------------------------
template <int V>
__device__ __forceinline__ void ens_cell(const DevMesh& Mh, const Dims& D, const IO& S, const RKStage& rk,
                                         const Partials& P, int diag, int bx) {
  __shared__ int s_e[kME][kEnsEPB];
  __shared__ float s_ns[kME][kEnsEPB];
  __shared__ float s_dv[kME][kEnsEPB];
  __shared__ float s_ae[kME][kEnsEPB];
  __shared__ FF s_invA[kEnsEPB];
  __shared__ FF s_A[kEnsEPB];
  __shared__ float s_invAf[kEnsEPB];
  __shared__ float s_Af[kEnsEPB];
  const int nc = Mh.nc, c0 = bx * kEnsEPB, nel = min(kEnsEPB, nc - c0);
  for (int t = threadIdx.x; t < kME * kEnsEPB; t += blockDim.x) {
    const int i = t / kEnsEPB, j = t - i * kEnsEPB;
    if (j < nel) {
      const size_t k = (size_t)i * nc + c0 + j;
      s_e[i][j] = Mh.edgesOnCell[k];
      s_ns[i][j] = (float)Mh.nSign[k];
      s_dv[i][j] = S.cdv[k];  // dvEdge and areaEdge of the cell's edges, gathered at set-up
      s_ae[i][j] = S.cae[k];
    }
  }
  for (int j = threadIdx.x; j < nel; j += blockDim.x) {
    s_invA[j] = FF{S.invA_hl[c0 + j], S.invA_hl[nc + c0 + j]};
    s_A[j] = FF{S.A_hl[c0 + j], S.A_hl[nc + c0 + j]};
    s_invAf[j] = Mh.invAreaCell_f[c0 + j];
    s_Af[j] = Mh.areaCell_f[c0 + j];
  }
  __syncthreads();
  const Lane L = lane_of<V>(D);
  const size_t Mm = L.M, ffs = S.ffs;
  const int mode = rk.mode;
  const FF adt = ff_from(rk.a_dt), sixth = ff_from(1.0 / 6.0);
  float rip[V], r44[V], eh[V], el[V];
  FF mass[V];
#pragma unroll
  for (int c = 0; c < V; ++c) rip[c] = r44[c] = eh[c] = el[c] = 0.f, mass[c] = FF{0.f, 0.f};
  for (int j = L.j0; j < nel; j += L.js) {
    const size_t cm = (size_t)(c0 + j) * Mm + L.m0;
    FF gold[V], gacc[V];
    float tprev[V], gdf[V], ghf[V], gdl[V];
    if (mode >= 1 && mode <= 3) ldff<V>(S.gd_old, cm, ffs, gold);
    if (mode >= 2) {
      ldff<V>(S.gd_acc, cm, ffs, gacc);
      ldv<V>(S.tendf, cm, tprev);
    }
    ldv<V>(S.gd_in, cm, gdf);
    ldv<V>(S.ghsf, cm, ghf);
    if (diag) ldv<V>(S.gd_in + ffs, cm, gdl);
    float uu[kME][V], Fv[kME][V];
#pragma unroll
    for (int i = 0; i < kME; ++i) {
      const size_t k = (size_t)s_e[i][j] * Mm + L.m0;
      ldv<V>(S.u, k, uu[i]);
      ldv<V>(S.F, k, Fv[i]);
    }
    FF acc_o[V], gnext[V];
    float Eo[V], tT[V];
#pragma unroll
    for (int c = 0; c < V; ++c) {
      float hi = 0.f, lo = 0.f, k = 0.f;
#pragma unroll
      for (int i = 0; i < kME; ++i) {
        const float ns = s_ns[i][j];
        two_sum_acc(hi, lo, __fmul_rn(__fmul_rn(ns, Fv[i][c]), s_dv[i][j]));
        k += fabsf(ns) * uu[i][c] * uu[i][c] * s_ae[i][j];
      }
      // gd tendency t = -(flux divergence) / areaCell
      FF t = ff_mul(ff_two_sum(hi, lo), s_invA[j]);
      t = FF{-t.h, -t.l};
      tT[c] = t.h;
      Eo[c] = k * 0.25f * s_invAf[j] + gdf[c] + ghf[c];
      const float Af = s_Af[j];
      gnext[c] = FF{0.f, 0.f};
      switch (mode) {
        case 0:  // E only (the closure's features of a state)
          acc_o[c] = t;
          break;
        case 1:
          acc_o[c] = t;
          gnext[c] = ff_add(gold[c], ff_mul(adt, t));
          break;
        case 2:
        case 3:
          rip[c] += tprev[c] * tT[c] * Af;
          acc_o[c] = ff_add(gacc[c], FF{2.f * t.h, 2.f * t.l});
          gnext[c] = ff_add(gold[c], ff_mul(adt, t));
          break;
        default: {
          rip[c] += tprev[c] * tT[c] * Af;
          const FF tn = ff_mul(ff_add(gacc[c], t), sixth);
          acc_o[c] = tn;
          r44[c] += tn.h * tn.h * Af;
        }
      }
      if (diag) {
        // total mass from the FF gd (FF products, FF sum), and the cell part
        // of the total energy (gd^2 + 2 gd ghs) areaCell from FP32 terms,
        // compensated (tmcore_swm_mod.F90:215-231)
        mass[c] = ff_add(mass[c], ff_mul(FF{gdf[c], gdl[c]}, s_A[j]));
        two_sum_acc(eh[c], el[c], gdf[c] * (gdf[c] + 2.f * ghf[c]) * Af);
      }
    }
    stv<V>(S.E, cm, Eo);
    if (mode >= 1) {
      stff<V>(S.gd_acc, cm, ffs, acc_o);
      stv<V>(S.tendf, cm, tT);
    }
    if (mode >= 1 && mode <= 3) stff<V>(S.gd_next, cm, ffs, gnext);
  }
  const int slot = bx;
  if (mode >= 2) {
    float v[2][V];
#pragma unroll
    for (int c = 0; c < V; ++c) v[0][c] = rip[c], v[1][c] = r44[c];
    float* const dst[2] = {P.f(R_IP_C + 2 * (mode - 2), slot), mode == 4 ? P.f(R_44_C, slot) : nullptr};
    block_partials_f<2, V>(L, v, dst);
  }
  if (diag) {
    FF v[2][V];
#pragma unroll
    for (int c = 0; c < V; ++c) v[0][c] = mass[c], v[1][c] = FF{eh[c], el[c]};
    double* const dst[2] = {P.d(R_MASS, slot), P.d(R_EN_C, slot)};
    block_partials_ff<2, V>(L, v, dst);
  }
}
template <int V>
__global__ void TMC_ENS_LB(TMC_ENS_CELL_MINB) k_ens_cell(DevMesh Mh, Dims D, IO S, RKStage rk, Partials P, int diag) {
  ens_cell<V>(Mh, D, S, rk, P, diag, blockIdx.x);
}

// invariants of a state only (the diagnostic pass): mass and cell energy
template <int V>
__global__ void __launch_bounds__(kMaxBS) k_ens_cell_diag(DevMesh Mh, Dims D, IO S, Partials P) {
  __shared__ FF s_A[kEnsEPB];
  __shared__ float s_Af[kEnsEPB];
  const int nc = Mh.nc, c0 = blockIdx.x * kEnsEPB, nel = min(kEnsEPB, nc - c0);
  for (int j = threadIdx.x; j < nel; j += blockDim.x) {
    s_A[j] = FF{S.A_hl[c0 + j], S.A_hl[nc + c0 + j]};
    s_Af[j] = Mh.areaCell_f[c0 + j];
  }
  __syncthreads();
  const Lane L = lane_of<V>(D);
  float eh[V], el[V];
  FF mass[V];
#pragma unroll
  for (int c = 0; c < V; ++c) eh[c] = el[c] = 0.f, mass[c] = FF{0.f, 0.f};
  for (int j = L.j0; j < nel; j += L.js) {
    const size_t cm = (size_t)(c0 + j) * L.M + L.m0;
    FF g[V];
    float ghf[V];
    ldff<V>(S.gd_in, cm, S.ffs, g);
    ldv<V>(S.ghsf, cm, ghf);
#pragma unroll
    for (int c = 0; c < V; ++c) {
      mass[c] = ff_add(mass[c], ff_mul(g[c], s_A[j]));
      two_sum_acc(eh[c], el[c], g[c].h * (g[c].h + 2.f * ghf[c]) * s_Af[j]);
    }
  }
  FF v[2][V];
#pragma unroll
  for (int c = 0; c < V; ++c) v[0][c] = mass[c], v[1][c] = FF{eh[c], el[c]};
  double* const dst[2] = {P.d(R_MASS, blockIdx.x), P.d(R_EN_C, blockIdx.x)};
  block_partials_ff<2, V>(L, v, dst);
}

// ---------------------------------------------------------------------------
// vertex: gd on vertices, vorticity, pv (operators_mod.F90:106-123, :76-91,
// :262-270); potential enstrophy and absolute vorticity on diag stages
// ---------------------------------------------------------------------------
template <int V>
__device__ __forceinline__ void ens_vertex(const DevMesh& Mh, const Dims& D, const IO& S, const Partials& P, int diag,
                                           int bx) {
  constexpr int kVU = TMC_ENS_VU;  // vertices per warp iteration (their loads first)
  // A vertex's staged stencil as five 16-byte records, so a lane reads it with
  // five shared-memory loads instead of eighteen scalar ones:
  //   s_ix[j] = {cell 0, cell 1, cell 2, edge 0}, {edge 1, edge 2, -, -}
  //   s_w[j]  = {kite 0, kite 1, kite 2, tSign 0}, {tSign 1, tSign 2, dcEdge 0, dcEdge 1},
  //             {dcEdge 2, 1 / areaTriangle, fVertex, areaTriangle}
  __shared__ int4 s_ix[kEnsEPB][2];
  __shared__ float4 s_w[kEnsEPB][3];
  const int nv = Mh.nv, v0 = bx * kEnsEPB, nel = min(kEnsEPB, nv - v0);
  for (int t = threadIdx.x; t < 3 * kEnsEPB; t += blockDim.x) {
    const int i = t / kEnsEPB, j = t - i * kEnsEPB;
    if (j < nel) {
      const size_t k = (size_t)i * nv + v0 + j;
      int* const ix = reinterpret_cast<int*>(&s_ix[j][0]);
      float* const w = reinterpret_cast<float*>(&s_w[j][0]);
      ix[i] = Mh.cellsOnVertex[k];
      ix[3 + i] = Mh.edgesOnVertex[k];
      w[i] = Mh.kite_f[k];
      w[3 + i] = (float)Mh.tSign[k];
      w[6 + i] = S.vdc[k];  // dcEdge of the vertex's edges, gathered at set-up
    }
  }
  for (int j = threadIdx.x; j < nel; j += blockDim.x) {
    float* const w = reinterpret_cast<float*>(&s_w[j][0]);
    w[9] = Mh.invAreaTriangle_f[v0 + j];
    w[10] = Mh.fVertex_f[v0 + j];
    w[11] = (float)Mh.areaTriangle[v0 + j];
  }
  __syncthreads();
  const Lane L = lane_of<V>(D);
  const size_t Mm = L.M;
  float ph[V], pl[V], ah[V], al[V];
#pragma unroll
  for (int c = 0; c < V; ++c) ph[c] = pl[c] = ah[c] = al[c] = 0.f;
  for (int base = L.j0; base < nel; base += L.js * kVU) {
    float g[kVU][3][V], uu[kVU][3][V];
#pragma unroll
    for (int q = 0; q < kVU; ++q) {
      const int j = min(base + q * L.js, nel - 1);
      const int4 a = s_ix[j][0], b = s_ix[j][1];
      const int cv[3] = {a.x, a.y, a.z}, ev[3] = {a.w, b.x, b.y};
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        ldv<V>(S.gd_in, (size_t)cv[i] * Mm + L.m0, g[q][i]);
        ldv<V>(S.u, (size_t)ev[i] * Mm + L.m0, uu[q][i]);
      }
    }
#pragma unroll
    for (int q = 0; q < kVU; ++q) {
      const int j = base + q * L.js;
      if (j >= nel) break;
      const float4 w0 = s_w[j][0], w1 = s_w[j][1], w2 = s_w[j][2];
      const float kt[3] = {w0.x, w0.y, w0.z}, ts[3] = {w0.w, w1.x, w1.y}, dc[3] = {w1.z, w1.w, w2.x};
      const float iA = w2.y, fv = w2.z, At = w2.w;
      float pv[V], vo[V], gv[V];
#pragma unroll
      for (int c = 0; c < V; ++c) {
        gv[c] = (g[q][0][c] * kt[0] + g[q][1][c] * kt[1] + g[q][2][c] * kt[2]) * iA;
        const float sv = ts[0] * uu[q][0][c] * dc[0] + ts[1] * uu[q][1][c] * dc[1] + ts[2] * uu[q][2][c] * dc[2];
        vo[c] = -sv * iA;
        pv[c] = (fv + vo[c]) / gv[c];
        if (diag) {
          // potential enstrophy and absolute vorticity (tmcore_swm_mod.F90:233-255),
          // FP32 terms, compensated; vorticity and f as separate terms
          two_sum_acc(ph[c], pl[c], gv[c] * (pv[c] * pv[c]) * At);
          two_sum_acc(ah[c], al[c], vo[c] * At);
          two_sum_acc(ah[c], al[c], fv * At);
        }
      }
      const size_t vm = (size_t)(v0 + j) * Mm + L.m0;
      stv<V>(S.pv_v, vm, pv);
      if (S.vor) stv<V>(S.vor, vm, vo);
      if (S.gd_v) stv<V>(S.gd_v, vm, gv);
    }
  }
  if (diag) {
    FF v[2][V];
#pragma unroll
    for (int c = 0; c < V; ++c) v[0][c] = FF{ph[c], pl[c]}, v[1][c] = FF{ah[c], al[c]};
    double* const dst[2] = {P.d(R_PE, bx), P.d(R_AV, bx)};
    block_partials_ff<2, V>(L, v, dst);
  }
}
template <int V>
__global__ void TMC_ENS_LB(TMC_ENS_VERT_MINB) k_ens_vertex(DevMesh Mh, Dims D, IO S, Partials P, int diag) {
  ens_vertex<V>(Mh, D, S, P, diag, blockIdx.x);
}

// ---------------------------------------------------------------------------
// edge_pv: centred pv on edges (APVM weight 0, operators_mod.F90:296-316)
// ---------------------------------------------------------------------------
template <int V>
__device__ __forceinline__ void ens_edge_pv(const DevMesh& Mh, const Dims& D, const IO& S, int bx) {
  constexpr int kPU = 4;
  __shared__ int s_v[2][kEnsEPB];
  const int ne = Mh.ne, e0 = bx * kEnsEPB, nel = min(kEnsEPB, ne - e0);
  for (int t = threadIdx.x; t < 2 * kEnsEPB; t += blockDim.x) {
    const int i = t / kEnsEPB, j = t - i * kEnsEPB;
    if (j < nel) s_v[i][j] = Mh.verticesOnEdge[(size_t)i * ne + e0 + j];
  }
  __syncthreads();
  const Lane L = lane_of<V>(D);
  const size_t Mm = L.M;
  for (int base = L.j0; base < nel; base += L.js * kPU) {
    float p1[kPU][V], p2[kPU][V];
#pragma unroll
    for (int q = 0; q < kPU; ++q) {
      const int j = min(base + q * L.js, nel - 1);
      ldv<V>(S.pv_v, (size_t)s_v[0][j] * Mm + L.m0, p1[q]);
      ldv<V>(S.pv_v, (size_t)s_v[1][j] * Mm + L.m0, p2[q]);
    }
#pragma unroll
    for (int q = 0; q < kPU; ++q) {
      const int j = base + q * L.js;
      if (j >= nel) break;
      float pe[V];
#pragma unroll
      for (int c = 0; c < V; ++c) pe[c] = 0.5f * (p1[q][c] + p2[q][c]);
      stv<V>(S.pv_e, (size_t)(e0 + j) * Mm + L.m0, pe);
    }
  }
}
template <int V>
__global__ void __launch_bounds__(kMaxBS) k_ens_edge_pv(DevMesh Mh, Dims D, IO S) {
  ens_edge_pv<V>(Mh, D, S, blockIdx.x);
}

// ---------------------------------------------------------------------------
// edge_pv, upwind (pv_scheme 3, orders 3 and 4; operators_mod.F90:359-412):
// the centred value corrected by the two-sided fit-stencil second
// derivatives, upwinded by the sign of the tangential velocity
// (operators_mod.F90:296-316 for the tangential velocity)
// ---------------------------------------------------------------------------
template <int V>
__device__ __forceinline__ void ens_edge_pv_up(const DevMesh& Mh, const Dims& D, const IO& S, const Upwind& U,
                                               int bx) {
  // blocks of kUpEPB edges: the stencils take kUpW x 2 entries per edge
  __shared__ int s_v[2][kUpEPB];
  __shared__ int2 s_ew[kME2][kUpEPB];      // edgesOnEdge, weightsOnEdge (FP32 bits)
  __shared__ int s_n[2][kUpEPB];
  __shared__ int2 s_iw[kUpW][2][kUpEPB];   // stencil point, weight (FP32 bits)
  __shared__ float s_dv[kUpEPB];
  const int ne = Mh.ne, e0 = bx * kUpEPB, nel = min(kUpEPB, ne - e0);
  for (int t = threadIdx.x; t < 2 * kUpEPB; t += blockDim.x) {
    const int i = t / kUpEPB, j = t - i * kUpEPB;
    if (j < nel) {
      s_v[i][j] = Mh.verticesOnEdge[(size_t)i * ne + e0 + j];
      s_n[i][j] = U.count[(size_t)i * ne + e0 + j];
    }
  }
  for (int t = threadIdx.x; t < kME2 * kUpEPB; t += blockDim.x) {
    const int i = t / kUpEPB, j = t - i * kUpEPB;
    if (j < nel) {
      const size_t k = (size_t)i * ne + e0 + j;
      // padded entries: the edge itself, weight 0
      s_ew[i][j] = make_int2(Mh.edgesOnEdge[k], __float_as_int(Mh.weightsOnEdge_f[k]));
    }
  }
  for (int t = threadIdx.x; t < U.width * 2 * kUpEPB; t += blockDim.x) {
    const int q = t / kUpEPB, j = t - q * kUpEPB;  // q = stencil point * 2 + side
    if (j < nel) {
      const size_t k = (size_t)q * ne + e0 + j;
      s_iw[q >> 1][q & 1][j] = make_int2(U.idx[k], __float_as_int(U.w[k]));
    }
  }
  for (int j = threadIdx.x; j < nel; j += blockDim.x) s_dv[j] = Mh.dvEdge_f[e0 + j];
  __syncthreads();
  const Lane L = lane_of<V>(D);
  const size_t Mm = L.M;
  const float coef2 = U.coef2;
  for (int j = L.j0; j < nel; j += L.js) {
    float p[2][V], ve[V], d[2][V];
    ldv<V>(S.pv_v, (size_t)s_v[0][j] * Mm + L.m0, p[0]);
    ldv<V>(S.pv_v, (size_t)s_v[1][j] * Mm + L.m0, p[1]);
#pragma unroll
    for (int c = 0; c < V; ++c) ve[c] = 0.f;
#pragma unroll
    for (int i = 0; i < kME2; ++i) {
      float uu[V];
      const int2 ew = s_ew[i][j];
      ldv<V>(S.u, (size_t)ew.x * Mm + L.m0, uu);
      const float w = __int_as_float(ew.y);
#pragma unroll
      for (int c = 0; c < V; ++c) ve[c] = ve[c] + uu[c] * w;
    }
#pragma unroll
    for (int sd = 0; sd < 2; ++sd) {
#pragma unroll
      for (int c = 0; c < V; ++c) d[sd][c] = 0.f;
      const int n = s_n[sd][j];
      for (int q = 0; q < n; ++q) {
        float f[V];
        const int2 iw = s_iw[q][sd][j];
        ldv<V>(S.pv_v, (size_t)iw.x * Mm + L.m0, f);
        const float w = __int_as_float(iw.y);
#pragma unroll
        for (int c = 0; c < V; ++c) d[sd][c] = d[sd][c] + w * (f[c] - p[sd][c]);
      }
    }
    const float dist = s_dv[j];
    float pe[V];
#pragma unroll
    for (int c = 0; c < V; ++c) {
      const float fe = 0.5f * (p[0][c] + p[1][c]);
      pe[c] = fe - dist * dist * ((d[0][c] + d[1][c]) - copysignf(1.f, ve[c]) * coef2 * (d[1][c] - d[0][c])) / 12.f;
    }
    stv<V>(S.pv_e, (size_t)(e0 + j) * Mm + L.m0, pe);
  }
}
template <int V>
__global__ void __launch_bounds__(kMaxBS) k_ens_edge_pv_up(DevMesh Mh, Dims D, IO S, Upwind U) {
  ens_edge_pv_up<V>(Mh, D, S, U, blockIdx.x);
}

// ---------------------------------------------------------------------------
// edge_flux: q.F_perp over the 10 neighbours (calc_tangent_vor_flux,
// operators_mod.F90:239-260), the gradient of E and the iap_u tendency
// (calc_u_tend_on_edge, tmcore_swm_mod.F90:155-201), the RK update of iap_u
// and the CRK4 inner products (time_scheme_mod.F90:109-154); stages 1-3 also
// prepare the next stage's gd_edge, u and F from its gd and iap_u.
// ---------------------------------------------------------------------------
template <int V>
__device__ __forceinline__ void ens_edge_flux(const DevMesh& Mh, const Dims& D, const IO& S, const RKStage& rk,
                                              const Partials& P, int bx) {
  __shared__ int s_ep[kME2][kEnsEPB];
  __shared__ float s_w[kME2][kEnsEPB];
  __shared__ int s_c[2][kEnsEPB];
  __shared__ float s_dc[kEnsEPB];
  __shared__ float s_ae[kEnsEPB];
  const int ne = Mh.ne, e0 = bx * kEnsEPB, nel = min(kEnsEPB, ne - e0);
  for (int t = threadIdx.x; t < kME2 * kEnsEPB; t += blockDim.x) {
    const int i = t / kEnsEPB, j = t - i * kEnsEPB;
    if (j < nel) {
      const size_t k = (size_t)i * ne + e0 + j;
      s_ep[i][j] = Mh.edgesOnEdge[k];  // padded entries: the edge itself, weight 0
      s_w[i][j] = Mh.weightsOnEdge_f[k];
    }
  }
  for (int t = threadIdx.x; t < 2 * kEnsEPB; t += blockDim.x) {
    const int i = t / kEnsEPB, j = t - i * kEnsEPB;
    if (j < nel) s_c[i][j] = Mh.cellsOnEdge[(size_t)i * ne + e0 + j];
  }
  for (int j = threadIdx.x; j < nel; j += blockDim.x) {
    s_dc[j] = Mh.dcEdge_f[e0 + j];
    s_ae[j] = Mh.areaEdge_f[e0 + j];
  }
  __syncthreads();
  const Lane L = lane_of<V>(D);
  const size_t Mm = L.M;
  const int mode = rk.mode;
  const bool fuse = S.u_nx != nullptr;
  const float adt = (float)rk.a_dt;
  float rip[V], r44[V];
#pragma unroll
  for (int c = 0; c < V; ++c) rip[c] = r44[c] = 0.f;
  for (int j = L.j0; j < nel; j += L.js) {
    const size_t em = (size_t)(e0 + j) * Mm + L.m0;
    const size_t c1m = (size_t)s_c[0][j] * Mm + L.m0, c2m = (size_t)s_c[1][j] * Mm + L.m0;
    float pe[V], uu[V], ge[V], tp[V], accv[V], oldv[V], gn1[V], gn2[V], E1[V], E2[V], t1[V], t2[V];
    ldv<V>(S.pv_e, em, pe);
    ldv<V>(S.u, em, uu);
    ldv<V>(S.gd_e, em, ge);
    if (mode >= 2) {
      ldv<V>(S.iap_tend, em, tp);
      ldv<V>(S.iap_acc, em, accv);
    }
    if (mode >= 1 && mode <= 3) ldv<V>(S.iap_old, em, oldv);
    if (fuse) {
      ldv<V>(S.gd_next, c1m, gn1);  // h halves: the FP32 gd of the next stage
      ldv<V>(S.gd_next, c2m, gn2);
    }
    ldv<V>(S.E, c1m, E1);
    ldv<V>(S.E, c2m, E2);
    ldv<V>(S.tendf, c1m, t1);
    ldv<V>(S.tendf, c2m, t2);
    float Fv[kME2][V], pp[kME2][V];
#pragma unroll
    for (int i = 0; i < kME2; ++i) {
      const size_t k = (size_t)s_ep[i][j] * Mm + L.m0;
      ldv<V>(S.F, k, Fv[i]);
      ldv<V>(S.pv_e, k, pp[i]);
    }
    const float dc = s_dc[j], ae = s_ae[j];
    float acc_o[V], it_o[V], inext[V];
#pragma unroll
    for (int c = 0; c < V; ++c) {
      float s = 0.f;
#pragma unroll
      for (int i = 0; i < kME2; ++i) s += s_w[i][j] * Fv[i][c] * (0.5f * (pe[c] + pp[i][c]));
      const float dEdx = (E2[c] - E1[c]) / dc;
      const float tge = 0.5f * (t1[c] + t2[c]);
      const float ut = s - dEdx;
      const float sq = sqrtf(ge[c]);
      const float it = sq * ut + 0.5f * uu[c] / sq * tge;
      it_o[c] = it;
      inext[c] = 0.f;
      switch (mode) {
        case 1:
          acc_o[c] = it;
          inext[c] = oldv[c] + adt * it;
          break;
        case 2:
        case 3:
          rip[c] = rip[c] + tp[c] * it * ae;
          acc_o[c] = accv[c] + 2.f * it;
          inext[c] = oldv[c] + adt * it;
          break;
        default: {
          rip[c] = rip[c] + tp[c] * it * ae;
          const float tn = (accv[c] + it) * (1.0f / 6.0f);
          acc_o[c] = tn;
          r44[c] = r44[c] + tn * tn * ae;
        }
      }
    }
    stv<V>(S.iap_acc, em, acc_o);
    stv<V>(S.iap_tend, em, it_o);
    if (fuse)
      prep<V>(inext, gn1, gn2, S.gd_e_nx, S.u_nx, S.F_nx, em);
    else if (mode <= 3)
      stv<V>(S.iap_next, em, inext);
  }
  if (mode >= 2) {
    float v[2][V];
#pragma unroll
    for (int c = 0; c < V; ++c) v[0][c] = rip[c], v[1][c] = r44[c];
    float* const dst[2] = {P.f(R_IP_E + 2 * (mode - 2), bx), mode == 4 ? P.f(R_44_E, bx) : nullptr};
    block_partials_f<2, V>(L, v, dst);
  }
}
template <int V>
__global__ void __launch_bounds__(256, V == 1 ? TMC_ENS_MINB_V1 : TMC_ENS_FLUX_MINB)
    k_ens_edge_flux(DevMesh Mh, Dims D, IO S, RKStage rk, Partials P) {
  ens_edge_flux<V>(Mh, D, S, rk, P, blockIdx.x);
}

// ---------------------------------------------------------------------------
// final update new = old + (beta dt) t_new (update_state, tmcore_swm_mod.F90:203-213),
// in place in state(old), with beta per member
// ---------------------------------------------------------------------------
constexpr int kFU = 4;

template <int V>
__device__ __forceinline__ void ens_final_cells(const DevMesh& Mh, const Dims& D, const IO& S, const double* diag,
                                                int bx) {
  const Lane L = lane_of<V>(D);
  const size_t Mm = L.M, ffs = S.ffs;
  FF bdt[V];
#pragma unroll
  for (int c = 0; c < V; ++c) bdt[c] = ff_from(diag[(size_t)(L.m0 + c) * kDiagStride + 9]);
  const int nc = Mh.nc, c0 = bx * kEnsEPB, nel = min(kEnsEPB, nc - c0);
  float* gd = const_cast<float*>(S.gd_old);
  for (int base = L.j0; base < nel; base += L.js * kFU) {
    FF g[kFU][V], a[kFU][V];
#pragma unroll
    for (int q = 0; q < kFU; ++q) {
      const size_t cm = (size_t)(c0 + min(base + q * L.js, nel - 1)) * Mm + L.m0;
      ldff<V>(gd, cm, ffs, g[q]);
      ldff<V>(S.gd_acc, cm, ffs, a[q]);
    }
#pragma unroll
    for (int q = 0; q < kFU; ++q) {
      const int j = base + q * L.js;
      if (j >= nel) break;
      FF gn[V];
#pragma unroll
      for (int c = 0; c < V; ++c) gn[c] = ff_add(g[q][c], ff_mul(bdt[c], a[q][c]));
      stff<V>(gd, (size_t)(c0 + j) * Mm + L.m0, ffs, gn);
    }
  }
}
template <int V>
__global__ void __launch_bounds__(kMaxBS) k_ens_final_cells(DevMesh Mh, Dims D, IO S, const double* diag) {
  ens_final_cells<V>(Mh, D, S, diag, blockIdx.x);
}

// Edges: iap_u of state(old) in place, then the edge preparation of the next
// step's first stage and the edge energy iap_u^2 areaEdge of the new state
// (tmcore_swm_mod.F90:229), FP32 terms, compensated.  kUpdate false: the
// stand-alone edge preparation of S.iap_in (energy only when want_energy).
template <int V, bool kUpdate>
__device__ __forceinline__ void ens_edges(const DevMesh& Mh, const Dims& D, const IO& S, const double* diag,
                                          const Partials& P, int want_energy, int bx) {
  __shared__ int s_c[2][kEnsEPB];
  __shared__ float s_ae[kEnsEPB];
  const int ne = Mh.ne, e0 = bx * kEnsEPB, nel = min(kEnsEPB, ne - e0);
  for (int t = threadIdx.x; t < 2 * kEnsEPB; t += blockDim.x) {
    const int i = t / kEnsEPB, j = t - i * kEnsEPB;
    if (j < nel) s_c[i][j] = Mh.cellsOnEdge[(size_t)i * ne + e0 + j];
  }
  for (int j = threadIdx.x; j < nel; j += blockDim.x) s_ae[j] = Mh.areaEdge_f[e0 + j];
  __syncthreads();
  const Lane L = lane_of<V>(D);
  const size_t Mm = L.M;
  float bdt[V];
#pragma unroll
  for (int c = 0; c < V; ++c) bdt[c] = kUpdate ? (float)diag[(size_t)(L.m0 + c) * kDiagStride + 9] : 0.f;
  float* iap = const_cast<float*>(kUpdate ? S.iap_old : S.iap_in);
  float eh[V], el[V];
#pragma unroll
  for (int c = 0; c < V; ++c) eh[c] = el[c] = 0.f;
  for (int base = L.j0; base < nel; base += L.js * kFU) {
    float ia[kFU][V], ac[kFU][V], g1[kFU][V], g2[kFU][V];
#pragma unroll
    for (int q = 0; q < kFU; ++q) {
      const int j = min(base + q * L.js, nel - 1);
      const size_t em = (size_t)(e0 + j) * Mm + L.m0;
      ldv<V>(iap, em, ia[q]);
      if (kUpdate) ldv<V>(S.iap_acc, em, ac[q]);
      ldv<V>(S.gd_in, (size_t)s_c[0][j] * Mm + L.m0, g1[q]);
      ldv<V>(S.gd_in, (size_t)s_c[1][j] * Mm + L.m0, g2[q]);
    }
#pragma unroll
    for (int q = 0; q < kFU; ++q) {
      const int j = base + q * L.js;
      if (j >= nel) break;
      const size_t em = (size_t)(e0 + j) * Mm + L.m0;
      if (kUpdate) {
#pragma unroll
        for (int c = 0; c < V; ++c) ia[q][c] = ia[q][c] + bdt[c] * ac[q][c];
        stv<V>(iap, em, ia[q]);
      }
      prep<V>(ia[q], g1[q], g2[q], const_cast<float*>(S.gd_e), const_cast<float*>(S.u), const_cast<float*>(S.F),
              em);
      if (want_energy)
#pragma unroll
        for (int c = 0; c < V; ++c) two_sum_acc(eh[c], el[c], ia[q][c] * ia[q][c] * s_ae[j]);
    }
  }
  if (want_energy) {
    FF v[1][V];
#pragma unroll
    for (int c = 0; c < V; ++c) v[0][c] = FF{eh[c], el[c]};
    double* const dst[1] = {P.d(R_EN_E, bx)};
    block_partials_ff<1, V>(L, v, dst);
  }
}
template <int V, bool kUpdate>
__global__ void __launch_bounds__(kMaxBS) k_ens_edges(DevMesh Mh, Dims D, IO S, const double* diag, Partials P,
                                                      int want_energy) {
  ens_edges<V, kUpdate>(Mh, D, S, diag, P, want_energy, blockIdx.x);
}

// ---------------------------------------------------------------------------
// reduction of the per-thread partials: block = (region, group of 32
// members), warp w sums slots w, w + W, ... for its 32 members (FP32 TwoSum
// for the step products, FP64 for the invariants), warp 0 combines the warps
// in double-double and stores the region sum after the member's kDiagLen
// outputs.
// ---------------------------------------------------------------------------
struct RegionList {
  int n;
  int r[R_COUNT];
  int count[R_COUNT];
};

// One block per (region, group of 32 members), 32 warps: warp w takes slots
// w, w + 32, ... in rounds of four with four independent accumulators (all
// four loads in flight), which it combines in a fixed order; the warps'
// sums are then combined in warp order.  Deterministic for a given slot
// count.  (With 8 warps and one accumulator the 7,680 slots of a level-7
// edge region took about 0.3 ms, a quarter of a 16-member step.)
constexpr int kRedThreads = 1024;
__device__ __forceinline__ void ens_reduce(const Partials& P, int r, int count, double* diag_out) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int m = blockIdx.y * 32 + lane;
  const bool in = m < P.M;
  DD acc{0.0, 0.0};
  if (in) {
    if (r <= R_44_E) {
      float fh[4] = {0.f, 0.f, 0.f, 0.f}, fl[4] = {0.f, 0.f, 0.f, 0.f};
      int s = w;
      for (; s + 3 * nw < count; s += 4 * nw) {
        float v[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) v[q] = P.f(r, s + q * nw)[m];
#pragma unroll
        for (int q = 0; q < 4; ++q) two_sum_acc(fh[q], fl[q], v[q]);
      }
#pragma unroll
      for (int q = 0; q < 3; ++q)  // the last at most 3 slots of this warp
        if (s + q * nw < count) two_sum_acc(fh[q], fl[q], P.f(r, s + q * nw)[m]);
#pragma unroll
      for (int q = 0; q < 4; ++q) acc = dd_add(acc, DD{(double)fh[q], (double)fl[q]});
    } else {
      double dh[4] = {0.0, 0.0, 0.0, 0.0};
      int s = w;
      for (; s + 3 * nw < count; s += 4 * nw) {
        double v[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) v[q] = P.d(r, s + q * nw)[m];
#pragma unroll
        for (int q = 0; q < 4; ++q) dh[q] += v[q];
      }
#pragma unroll
      for (int q = 0; q < 3; ++q)
        if (s + q * nw < count) dh[q] += P.d(r, s + q * nw)[m];
#pragma unroll
      for (int q = 0; q < 4; ++q) acc = dd_add(acc, DD{dh[q], 0.0});
    }
  }
  __shared__ double sh[kRedThreads / 32][32], sl[kRedThreads / 32][32];
  sh[w][lane] = acc.hi;
  sl[w][lane] = acc.lo;
  __syncthreads();
  if (w != 0 || !in) return;
  DD tot{0.0, 0.0};
  for (int k = 0; k < nw; ++k) tot = dd_add(tot, DD{sh[k][lane], sl[k][lane]});
  diag_out[(size_t)m * kDiagStride + kDiagLen + r] = tot.hi + tot.lo;
}
__global__ void __launch_bounds__(kRedThreads) k_ens_reduce(Partials P, RegionList RL, double* diag_out) {
  ens_reduce(P, RL.r[blockIdx.x], RL.count[blockIdx.x], diag_out);
}

// beta (time_scheme_mod.F90:144-150) and the invariants (tmcore_swm_mod.F90:215-255)
// of every member from its region sums
__device__ __forceinline__ void ens_beta(int M, int step, int diag, int conserve, double totalArea,
                                         double sumAreaTriangle, double dt, double* diag_out, int m) {
  if (m >= M) return;
  double* out = diag_out + (size_t)m * kDiagStride;
  const double* rv = out + kDiagLen;
  if (step) {
    double R[4];
    for (int k = 0; k < 3; ++k) R[k] = (rv[R_IP_E + 2 * k] + rv[R_IP_C + 2 * k]) / totalArea;
    R[3] = (rv[R_44_E] + rv[R_44_C]) / totalArea;
    // beta = 1 for a member whose tendency is zero everywhere (k_finalize)
    const double beta = conserve && R[3] != 0.0 ? (R[0] + R[1] + R[2]) / (3.0 * R[3]) : 1.0;
    out[4] = beta;
    out[5] = R[0];
    out[6] = R[1];
    out[7] = R[2];
    out[8] = R[3];
    out[9] = beta * dt;
  }
  if (diag) {
    out[0] = rv[R_MASS];
    out[1] = rv[R_EN_E] + rv[R_EN_C];
    out[2] = rv[R_PE];
    out[3] = rv[R_AV] / sumAreaTriangle;
  }
}
__global__ void k_ens_beta(int M, int step, int diag, int conserve, double totalArea, double sumAreaTriangle,
                           double dt, double* diag_out) {
  ens_beta(M, step, diag, conserve, totalArea, sumAreaTriangle, dt, diag_out, blockIdx.x * blockDim.x + threadIdx.x);
}

// pv on cells for the learned closure: scalar_v2c_interp_operator as a
// gather over the cell's vertices (operators_mod.F90:125-141), the FP32
// arithmetic of k_v2c; block = one cell, threads = members
__global__ void k_ens_v2c(DevMesh Mh, int M, const float* pv_v, float* pv_c) {
  const int c = blockIdx.x, m = blockIdx.y * blockDim.x + threadIdx.x;
  if (m >= M) return;
  const float A = (float)Mh.areaCell[c];
  float s = 0.f;
  for (int k = Mh.v2c_start[c]; k < Mh.v2c_start[c + 1]; ++k)
    s = s + pv_v[(size_t)Mh.v2c_vertex[k] * M + m] * (float)Mh.v2c_kite[k] / A;
  pv_c[(size_t)c * M + m] = s;
}

// the held closure correction of stage 1 added to pv_edge in stages 2-4
__global__ void k_ens_closure_hold(size_t n, float* pv_e, const float* dq) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) pv_e[i] += dq[i];
}

// ---- state transfer ----
__global__ void k_ens_gather_f64(int n, int M, int m, const double* raw, const int32_t* n2o, double* dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[(size_t)i * M + m] = raw[n2o[i]];
}
__global__ void k_ens_gather_f32(int n, int M, int m, const double* raw, const int32_t* n2o, float* dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[(size_t)i * M + m] = (float)raw[n2o[i]];
}
__global__ void k_ens_gather_ff(int n, int M, int m, const double* raw, const int32_t* n2o, float* dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const FF v = ff_from(raw[n2o[i]]);
  dst[(size_t)i * M + m] = v.h;
  dst[(size_t)n * M + (size_t)i * M + m] = v.l;
}
__global__ void k_ens_scatter_f32(int n, int M, int m, const float* src, const int32_t* n2o, double* raw) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) raw[n2o[i]] = (double)src[(size_t)i * M + m];
}
__global__ void k_ens_scatter_ff(int n, int M, int m, const float* src, const int32_t* n2o, double* raw) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) raw[n2o[i]] = ff_to_double(FF{src[(size_t)i * M + m], src[(size_t)n * M + (size_t)i * M + m]});
}
template <class T>
__global__ void k_ens_extract(int n, int M, int m, const T* src, double* dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (double)src[(size_t)i * M + m];
}
__global__ void k_ens_extract_ff(int n, int M, int m, const float* src, double* dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = ff_to_double(FF{src[(size_t)i * M + m], src[(size_t)n * M + (size_t)i * M + m]});
}
__global__ void k_ens_iap_from_u(int ne, int M, int m, const double* gd_e, const double* u, float* iap) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < ne) iap[(size_t)i * M + m] = (float)(sqrt(gd_e[i]) * u[i]);
}
__global__ void k_ens_to_f32(size_t n, int M, int m, const double* src, float* dst) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const size_t k = m < 0 ? i : i * M + m;
  dst[k] = (float)src[k];
}

inline unsigned nb(size_t n) { return (unsigned)((n + 255) / 256); }

// ---------------------------------------------------------------------------
// batch kernels: block b of kind K belongs to the job j with
// off[K][j] <= b < off[K][j + 1] (j < nj), as block b - off[K][j] of that
// job's mesh; the bodies are those of the single-mesh kernels
// ---------------------------------------------------------------------------
__device__ __forceinline__ int job_of(const int (&off)[4][kMaxJobs + 1], int kind, int nj, int* j) {
  const int b = blockIdx.x;
  int k = 0;
  while (k + 1 < nj && b >= off[kind][k + 1]) ++k;
  *j = k;
  return b - off[kind][k];
}
__device__ __forceinline__ double stage_adt(int stage, double dt) {
  return (stage == 1 || stage == 2) ? 0.5 * dt : (stage == 3 ? dt : 0.0);
}

// f(job j of T) with j a constant in each branch: the body then reads the
// job's pointers at fixed offsets of the parameter (constant-bank operands,
// as in the single-mesh kernels) rather than into registers
template <class F>
__device__ __forceinline__ void on_job(const StageTable& T, int j, F&& f) {
  static_assert(kMaxJobs == 8, "one branch per job slot");
  switch (j) {
    case 0: f(T.job[0]); break;
    case 1: f(T.job[1]); break;
    case 2: f(T.job[2]); break;
    case 3: f(T.job[3]); break;
    case 4: f(T.job[4]); break;
    case 5: f(T.job[5]); break;
    case 6: f(T.job[6]); break;
    default: f(T.job[7]); break;
  }
}

template <int V>
__global__ void TMC_ENS_LB(TMC_ENS_CELL_MINB) k_jobs_cell(const __grid_constant__ StageTable T, int nj, int stage) {
  int j;
  const int bx = job_of(T.off, J_CELLS, nj, &j);
  on_job(T, j, [&](const JobStage& J) {
    ens_cell<V>(J.Mh, J.D, J.io, RKStage{stage, stage_adt(stage, J.dt)}, J.P, 0, bx);
  });
}
template <int V>
__global__ void TMC_ENS_LB(TMC_ENS_VERT_MINB) k_jobs_vertex(const __grid_constant__ StageTable T, int nj) {
  int j;
  const int bx = job_of(T.off, J_VERTS, nj, &j);
  on_job(T, j, [&](const JobStage& J) { ens_vertex<V>(J.Mh, J.D, J.io, J.P, 0, bx); });
}
template <int V>
__global__ void __launch_bounds__(kMaxBS) k_jobs_edge_pv(const __grid_constant__ StageTable T, int nj) {
  int j;
  const int bx = job_of(T.off, J_EDGES, nj, &j);
  on_job(T, j, [&](const JobStage& J) { ens_edge_pv<V>(J.Mh, J.D, J.io, bx); });
}
template <int V>
__global__ void __launch_bounds__(kMaxBS) k_jobs_edge_pv_up(const __grid_constant__ StageTable T, int nj) {
  int j;
  const int bx = job_of(T.off, J_EDGES_UP, nj, &j);
  on_job(T, j, [&](const JobStage& J) { ens_edge_pv_up<V>(J.Mh, J.D, J.io, J.up, bx); });
}
template <int V>
__global__ void TMC_ENS_LB(TMC_ENS_FLUX_MINB) k_jobs_edge_flux(const __grid_constant__ StageTable T, int nj,
                                                               int stage) {
  int j;
  const int bx = job_of(T.off, J_EDGES, nj, &j);
  on_job(T, j, [&](const JobStage& J) {
    ens_edge_flux<V>(J.Mh, J.D, J.io, RKStage{stage, stage_adt(stage, J.dt)}, J.P, bx);
  });
}
template <int V>
__global__ void __launch_bounds__(kMaxBS) k_jobs_final_cells(const __grid_constant__ StageTable T, int nj) {
  int j;
  const int bx = job_of(T.off, J_CELLS, nj, &j);
  on_job(T, j, [&](const JobStage& J) { ens_final_cells<V>(J.Mh, J.D, J.io, J.diag, bx); });
}
template <int V>
__global__ void __launch_bounds__(kMaxBS) k_jobs_final_edges(const __grid_constant__ StageTable T, int nj) {
  int j;
  const int bx = job_of(T.off, J_EDGES, nj, &j);
  on_job(T, j, [&](const JobStage& J) { ens_edges<V, true>(J.Mh, J.D, J.io, J.diag, J.P, 1, bx); });
}
// the step's region sums: block (job * nr + i, group of 32 members) sums
// region r[i] of its job, over the job's blocks of the region's element kind
struct StepRegions {
  int n;
  int r[8];
  int kind[8];
};
__global__ void __launch_bounds__(kRedThreads) k_jobs_reduce(const __grid_constant__ JobTable T, StepRegions R) {
  const int j = blockIdx.x / R.n, i = blockIdx.x - j * R.n;
  const Job& J = T.job[j];
  const int count = R.kind[i] == J_CELLS ? J.D.slots_c : J.D.slots_e;
  ens_reduce(J.P, R.r[i], count, J.diag);
}
// beta of every member of every job (blockIdx.y = job)
__global__ void k_jobs_beta(const __grid_constant__ JobTable T) {
  const Job& J = T.job[blockIdx.y];
  ens_beta(J.D.M, 1, 0, J.conserve, J.totalArea, J.sumAreaTriangle, J.dt, J.diag,
           blockIdx.x * blockDim.x + threadIdx.x);
}

}  // namespace

// ---- launchers ----
void launch_cell(const DevMesh& Mh, const Dims& D, const IO& S, RKStage rk, const Partials& P, bool diag, int bs,
                 cudaStream_t st) {
  int th;
  const dim3 g = grid_of(Mh.nc, D, bs, &th);
  if (D.V == 2)
    k_ens_cell<2><<<g, th, 0, st>>>(Mh, D, S, rk, P, diag ? 1 : 0);
  else
    k_ens_cell<1><<<g, th, 0, st>>>(Mh, D, S, rk, P, diag ? 1 : 0);
}
void launch_cell_diag(const DevMesh& Mh, const Dims& D, const IO& S, const Partials& P, int bs, cudaStream_t st) {
  int th;
  const dim3 g = grid_of(Mh.nc, D, bs, &th);
  if (D.V == 2)
    k_ens_cell_diag<2><<<g, th, 0, st>>>(Mh, D, S, P);
  else
    k_ens_cell_diag<1><<<g, th, 0, st>>>(Mh, D, S, P);
}
void launch_vertex(const DevMesh& Mh, const Dims& D, const IO& S, const Partials& P, bool diag, int bs,
                   cudaStream_t st) {
  int th;
  const dim3 g = grid_of(Mh.nv, D, bs, &th);
  if (D.V == 2)
    k_ens_vertex<2><<<g, th, 0, st>>>(Mh, D, S, P, diag ? 1 : 0);
  else
    k_ens_vertex<1><<<g, th, 0, st>>>(Mh, D, S, P, diag ? 1 : 0);
}
void launch_edge_pv(const DevMesh& Mh, const Dims& D, const IO& S, const Upwind* up, int bs, cudaStream_t st) {
  int th;
  const dim3 g = grid_of(Mh.ne, D, bs, &th);
  if (up) {
    // four members per lane when the member groups allow (the kernel issues
    // more instructions per member than it moves bytes); blocks of kUpEPB edges
    const dim3 gu((unsigned)slots_up(Mh.ne), g.y);
    if (D.LPE == 32 && D.M % 128 == 0 && TMC_ENS_UP_V == 4)
      k_ens_edge_pv_up<4><<<dim3(gu.x, (unsigned)(D.M / 128)), th, 0, st>>>(Mh, D, S, *up);
    else if (D.V == 2)
      k_ens_edge_pv_up<2><<<gu, th, 0, st>>>(Mh, D, S, *up);
    else
      k_ens_edge_pv_up<1><<<gu, th, 0, st>>>(Mh, D, S, *up);
    return;
  }
  if (D.V == 2)
    k_ens_edge_pv<2><<<g, th, 0, st>>>(Mh, D, S);
  else
    k_ens_edge_pv<1><<<g, th, 0, st>>>(Mh, D, S);
}
void launch_edge_flux(const DevMesh& Mh, const Dims& D, const IO& S, RKStage rk, const Partials& P, int bs,
                      cudaStream_t st) {
  int th;
  const dim3 g = grid_of(Mh.ne, D, bs, &th);
  if (D.V == 2)
    k_ens_edge_flux<2><<<g, th, 0, st>>>(Mh, D, S, rk, P);
  else
    k_ens_edge_flux<1><<<g, th, 0, st>>>(Mh, D, S, rk, P);
}
void launch_final(const DevMesh& Mh, const Dims& D, const IO& S, const double* diag, const Partials& P, int bs,
                  cudaStream_t st) {
  int th;
  const dim3 gc = grid_of(Mh.nc, D, bs, &th);
  if (D.V == 2)
    k_ens_final_cells<2><<<gc, th, 0, st>>>(Mh, D, S, diag);
  else
    k_ens_final_cells<1><<<gc, th, 0, st>>>(Mh, D, S, diag);
  const dim3 ge = grid_of(Mh.ne, D, bs, &th);
  if (D.V == 2)
    k_ens_edges<2, true><<<ge, th, 0, st>>>(Mh, D, S, diag, P, 1);
  else
    k_ens_edges<1, true><<<ge, th, 0, st>>>(Mh, D, S, diag, P, 1);
}
void launch_edge_prep(const DevMesh& Mh, const Dims& D, const IO& S, const Partials& P, bool diag, int bs,
                      cudaStream_t st) {
  int th;
  const dim3 g = grid_of(Mh.ne, D, bs, &th);
  if (D.V == 2)
    k_ens_edges<2, false><<<g, th, 0, st>>>(Mh, D, S, nullptr, P, diag ? 1 : 0);
  else
    k_ens_edges<1, false><<<g, th, 0, st>>>(Mh, D, S, nullptr, P, diag ? 1 : 0);
}
void launch_finalize(const Dims& D, const Partials& P, bool step, bool diag, bool conserve, double totalArea,
                     double sumAreaTriangle, double dt, double* diag_out, cudaStream_t st) {
  RegionList RL{};
  auto add = [&](int r, int count) {
    RL.r[RL.n] = r;
    RL.count[RL.n] = count;
    RL.n++;
  };
  if (step) {
    for (int k = 0; k < 3; ++k) {
      add(R_IP_C + 2 * k, D.slots_c);
      add(R_IP_E + 2 * k, D.slots_e);
    }
    add(R_44_C, D.slots_c);
    add(R_44_E, D.slots_e);
  }
  if (diag) {
    add(R_MASS, D.slots_c);
    add(R_EN_C, D.slots_c);
    add(R_EN_E, D.slots_e);
    add(R_PE, D.slots_v);
    add(R_AV, D.slots_v);
  }
  if (RL.n == 0) return;
  k_ens_reduce<<<dim3(RL.n, D.G), kRedThreads, 0, st>>>(P, RL, diag_out);
  k_ens_beta<<<nb(D.M), 256, 0, st>>>(D.M, step ? 1 : 0, diag ? 1 : 0, conserve ? 1 : 0, totalArea,
                                      sumAreaTriangle, dt, diag_out);
}

void launch_v2c(const DevMesh& Mh, const Dims& D, const IO& S, float* pv_c, cudaStream_t st) {
  k_ens_v2c<<<dim3(Mh.nc, (D.M + 127) / 128), 128, 0, st>>>(Mh, D.M, S.pv_v, pv_c);
}
void launch_closure_hold(const DevMesh& Mh, const Dims& D, const IO& S, const float* dq, cudaStream_t st) {
  const size_t n = (size_t)Mh.ne * D.M;
  k_ens_closure_hold<<<nb(n), 256, 0, st>>>(n, S.pv_e, dq);
}

void launch_gather_f64(int n, int M, int m, const double* raw, const int32_t* n2o, double* dst, cudaStream_t st) {
  k_ens_gather_f64<<<nb(n), 256, 0, st>>>(n, M, m, raw, n2o, dst);
}
void launch_gather_f32(int n, int M, int m, const double* raw, const int32_t* n2o, float* dst, cudaStream_t st) {
  k_ens_gather_f32<<<nb(n), 256, 0, st>>>(n, M, m, raw, n2o, dst);
}
void launch_gather_ff(int n, int M, int m, const double* raw, const int32_t* n2o, float* dst, cudaStream_t st) {
  k_ens_gather_ff<<<nb(n), 256, 0, st>>>(n, M, m, raw, n2o, dst);
}
void launch_scatter_f32(int n, int M, int m, const float* src, const int32_t* n2o, double* raw, cudaStream_t st) {
  k_ens_scatter_f32<<<nb(n), 256, 0, st>>>(n, M, m, src, n2o, raw);
}
void launch_scatter_ff(int n, int M, int m, const float* src, const int32_t* n2o, double* raw, cudaStream_t st) {
  k_ens_scatter_ff<<<nb(n), 256, 0, st>>>(n, M, m, src, n2o, raw);
}
void launch_extract_f64(int n, int M, int m, const double* src, double* dst, cudaStream_t st) {
  k_ens_extract<double><<<nb(n), 256, 0, st>>>(n, M, m, src, dst);
}
void launch_extract_f32(int n, int M, int m, const float* src, double* dst, cudaStream_t st) {
  k_ens_extract<float><<<nb(n), 256, 0, st>>>(n, M, m, src, dst);
}
void launch_extract_ff(int n, int M, int m, const float* src, double* dst, cudaStream_t st) {
  k_ens_extract_ff<<<nb(n), 256, 0, st>>>(n, M, m, src, dst);
}
void launch_iap_from_u(int ne, int M, int m, const double* gd_e, const double* u, float* iap, cudaStream_t st) {
  k_ens_iap_from_u<<<nb(ne), 256, 0, st>>>(ne, M, m, gd_e, u, iap);
}
void launch_to_f32(int n, int M, int m, const double* src, float* dst, cudaStream_t st) {
  const size_t k = m < 0 ? (size_t)n * M : (size_t)n;
  k_ens_to_f32<<<nb(k), 256, 0, st>>>(k, M, m, src, dst);
}


// One CRK4 step of the first nj jobs of T, one launch per pass (the program
// of EnsEngine::launch_step without the closure and the diagnostics).
// the table of stage k (0: the final update) of the first nj jobs of T
static StageTable stage_table(const JobTable& T, int nj, int k) {
  StageTable S;
  std::memset(&S, 0, sizeof(S));
  std::memcpy(S.off, T.off, sizeof(S.off));
  for (int j = 0; j < nj; ++j) {
    const Job& J = T.job[j];
    S.job[j] = JobStage{J.Mh, J.D, J.io[k], J.P, J.up, J.diag, J.dt};
  }
  return S;
}

void launch_jobs_step(const JobTable& T, int nj, const int* bsp, bool upwind, cudaStream_t st, cudaStream_t side,
                      cudaEvent_t fork, cudaEvent_t join) {
  const Dims& D = T.job[0].D;  // every job has the same members, hence V and lanes
  int th[5];
  const unsigned gy = (unsigned)(D.M / (D.LPE * D.V));
  for (int p = 0; p < 5; ++p) grid_of(1, D, bsp[p], &th[p]);
  const dim3 gc((unsigned)T.off[J_CELLS][nj], gy), ge((unsigned)T.off[J_EDGES][nj], gy),
      gv((unsigned)T.off[J_VERTS][nj], gy), gu((unsigned)T.off[J_EDGES_UP][nj], gy);
  const bool up4 = upwind && D.LPE == 32 && D.M % 128 == 0 && TMC_ENS_UP_V == 4;
  const bool branch = side && fork && join;
  const cudaStream_t sv = branch ? side : st;
  for (int k = 1; k <= 4; ++k) {
    const StageTable S = stage_table(T, nj, k);
    if (branch) {
      cudaEventRecord(fork, st);
      cudaStreamWaitEvent(side, fork, 0);
    }
    if (D.V == 2) {
      k_jobs_cell<2><<<gc, th[0], 0, st>>>(S, nj, k);
      k_jobs_vertex<2><<<gv, th[1], 0, sv>>>(S, nj);
    } else {
      k_jobs_cell<1><<<gc, th[0], 0, st>>>(S, nj, k);
      k_jobs_vertex<1><<<gv, th[1], 0, sv>>>(S, nj);
    }
    if (up4)
      k_jobs_edge_pv_up<4><<<dim3(gu.x, (unsigned)(D.M / 128)), th[2], 0, sv>>>(S, nj);
    else if (upwind && D.V == 2)
      k_jobs_edge_pv_up<2><<<gu, th[2], 0, sv>>>(S, nj);
    else if (upwind)
      k_jobs_edge_pv_up<1><<<gu, th[2], 0, sv>>>(S, nj);
    else if (D.V == 2)
      k_jobs_edge_pv<2><<<ge, th[2], 0, sv>>>(S, nj);
    else
      k_jobs_edge_pv<1><<<ge, th[2], 0, sv>>>(S, nj);
    if (branch) {
      cudaEventRecord(join, side);
      cudaStreamWaitEvent(st, join, 0);
    }
    if (D.V == 2)
      k_jobs_edge_flux<2><<<ge, th[3], 0, st>>>(S, nj, k);
    else
      k_jobs_edge_flux<1><<<ge, th[3], 0, st>>>(S, nj, k);
  }
  StepRegions R{};
  for (int k = 0; k < 3; ++k) {
    R.r[R.n] = R_IP_C + 2 * k, R.kind[R.n++] = J_CELLS;
    R.r[R.n] = R_IP_E + 2 * k, R.kind[R.n++] = J_EDGES;
  }
  R.r[R.n] = R_44_C, R.kind[R.n++] = J_CELLS;
  R.r[R.n] = R_44_E, R.kind[R.n++] = J_EDGES;
  k_jobs_reduce<<<dim3((unsigned)(nj * R.n), (unsigned)D.G), kRedThreads, 0, st>>>(T, R);
  k_jobs_beta<<<dim3(nb(D.M), (unsigned)nj), 256, 0, st>>>(T);
  const StageTable S0 = stage_table(T, nj, 0);
  if (D.V == 2) {
    k_jobs_final_cells<2><<<gc, th[4], 0, st>>>(S0, nj);
    k_jobs_final_edges<2><<<ge, th[4], 0, st>>>(S0, nj);
  } else {
    k_jobs_final_cells<1><<<gc, th[4], 0, st>>>(S0, nj);
    k_jobs_final_edges<1><<<ge, th[4], 0, st>>>(S0, nj);
  }
}

}  // namespace ens
}  // namespace tmc
