// Kernel bodies for tmc_kernels.cuh (included once per precision TU).
//
// Every kernel has two branches selected at compile time:
//  * T = double: the reference's arithmetic, element by element, in its
//    expression order (no FMA: the TU is compiled with -fmad=false);
//  * T = float: the fast path.  Neighbour indices and weights are loaded
//    first (fixed unrolled widths: maxEdges 6, maxEdges2 10, padded entries
//    carry zero weights or zero signs), then the neighbour gathers, then the
//    arithmetic, so each thread keeps tens of independent loads in flight.
//    GB300 executes FP64 at a small fraction of its FP32 rate, so the FP32
//    path keeps FP64 only for the gd tendency (from an FP32 two-sum
//    compensated flux divergence), the gd RK accumulation and the per-thread
//    invariant sums.
#pragma once

// Resident 256-thread blocks per SM the heavy ensemble kernels are built for
// (their register budget: 4 -> 64 registers, 3 -> 80).  On 512 level-6
// members, 4 for the flux, the cell pass without tracers and the final edge
// update takes the step from 9.85 to about 9.3 ms: the occupancy gain
// outweighs the few spilled bytes.
#ifndef TMC_FLUX_MIN_BLOCKS
#define TMC_FLUX_MIN_BLOCKS 4
#endif
#ifndef TMC_CELL_MIN_BLOCKS
#define TMC_CELL_MIN_BLOCKS 4
#endif
#ifndef TMC_FINAL_MIN_BLOCKS
#define TMC_FINAL_MIN_BLOCKS 4
#endif
// The same for the single-model cell pass (blocks of kCellBlock) and final
// edge update (blocks of up to kMaxBlock).  Level 9: the cell pass takes 139 us
// at 3 (80 registers) and 165 us at 4; the final pass 122 us at 2 (64
// registers, no spill), 129 us with no minimum (64 registers, 4 bytes
// spilled) and 176 us at 1 (120 registers).
#ifndef TMC_CELL_SINGLE_MIN_BLOCKS
#define TMC_CELL_SINGLE_MIN_BLOCKS 3
#endif
#ifndef TMC_FINAL_SINGLE_MIN_BLOCKS
#define TMC_FINAL_SINGLE_MIN_BLOCKS 2
#endif

#include <type_traits>

#include "tmc_kernels.cuh"

namespace tmc {

constexpr int kMaxBlock = 512;
constexpr int kMemberBlock = 256;  // block size limit of the ensemble (member-batched) kernels
constexpr int kCellBlock = 256;    // block size limit of the FP32 cell pass (register budget for 3 blocks/SM)
constexpr int kME = 6;    // unrolled maxEdges of the FP32 path
constexpr int kME2 = 10;  // unrolled maxEdges2 of the FP32 path

// ---------------------------------------------------------------------------
// double-double accumulation (Knuth TwoSum), never contracted into FMA
// ---------------------------------------------------------------------------
struct DD {
  double hi, lo;
};
__device__ __forceinline__ DD dd_add(DD a, DD b) {
  double s = __dadd_rn(a.hi, b.hi);
  double bb = __dsub_rn(s, a.hi);
  double e = __dadd_rn(__dsub_rn(a.hi, __dsub_rn(s, bb)), __dsub_rn(b.hi, bb));
  e = __dadd_rn(e, __dadd_rn(a.lo, b.lo));
  double hi = __dadd_rn(s, e);
  double lo = __dsub_rn(e, __dsub_rn(hi, s));
  return {hi, lo};
}
__device__ __forceinline__ DD warp_reduce_dd(DD v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    DD o;
    o.hi = __shfl_down_sync(0xffffffffu, v.hi, off);
    o.lo = __shfl_down_sync(0xffffffffu, v.lo, off);
    v = dd_add(v, o);
  }
  return v;
}

// Reduce N per-thread partial sums over the block and store region[r[k]][block]
// as (sum, 0).  Warps sum their lanes with a shuffle tree in A (double or
// float), warp 0 sums the warp sums the same way; the compensated
// (double-double) combination happens across blocks in k_finalize.  No
// double-double arithmetic here: warp 0 of every block sits on the same SM
// sub-partition, and GB300 issues FP64 at 1/64 of the FP32 rate, so a
// double-double tail per block serialises behind the whole kernel.  Every
// thread of the block must call this (it synchronises).
template <class A, int N>
__device__ __forceinline__ void block_store(const A (&v)[N], const Partials& P, const int (&r)[N], int slot = -1) {
  if (slot < 0) slot = blockIdx.x;
  __shared__ A sm[N][kMaxBlock / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < N; ++k) {
    A w = v[k];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) w += __shfl_down_sync(0xffffffffu, w, off);
    if (lane == 0) sm[k][warp] = w;
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) {
      A w = (lane < nw) ? sm[k][lane] : A(0);
#pragma unroll
      for (int off = kMaxBlock / 64; off > 0; off >>= 1) w += __shfl_down_sync(0xffffffffu, w, off);
      if (lane == 0) {
        double* reg = P.region(r[k]);
        reg[2 * slot] = (double)w;
        reg[2 * slot + 1] = 0.0;
      }
    }
  }
  __syncthreads();
}

template <class T>
constexpr bool kF64 = std::is_same<T, double>::value;

// metric in the arithmetic type: FP64 array in FP64 mode, FP32 copy otherwise
template <class T>
__device__ __forceinline__ T met(const double* d, const float* f, size_t i) {
  if constexpr (kF64<T>)
    return d[i];
  else
    return f[i];
}

template <class T>
__device__ __forceinline__ T sgn1(T x) {
  return copysign(T(1), x);
}

// FP32 error-free addition (TwoSum): hi + lo accumulates p exactly
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float p) {
  const float t = __fadd_rn(hi, p);
  const float bp = __fsub_rn(t, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, bp)), __fsub_rn(p, bp));
  hi = t;
  lo = __fadd_rn(lo, err);
}

// block_store for compensated FP32 sums: the threads' (hi, lo) pairs are
// combined over each warp and then over the block with FP32 TwoSum
// arithmetic, and the block's pair is stored as (hi, lo) in FP64 (two
// conversions per block).  An FP64 shuffle tree costs ten FP64 instructions
// per warp, and GB300 runs each warp-wide FP64 instruction on a 2-lane pipe
// (16 cycles), which in the final edge update was most of the FP64 pipe's
// busy time.  Every thread of the block must call this (it synchronises).
template <int N>
__device__ __forceinline__ void block_store_ff(const float (&hi)[N], const float (&lo)[N], const Partials& P,
                                               const int (&r)[N]) {
  const int slot = blockIdx.x;
  __shared__ float sh[N][kMaxBlock / 32], sl[N][kMaxBlock / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < N; ++k) {
    float h = hi[k], l = lo[k];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const float oh = __shfl_down_sync(0xffffffffu, h, off), ol = __shfl_down_sync(0xffffffffu, l, off);
      two_sum_acc(h, l, oh);
      l = __fadd_rn(l, ol);
    }
    if (lane == 0) {
      sh[k][warp] = h;
      sl[k][warp] = l;
    }
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) {
      float h = (lane < nw) ? sh[k][lane] : 0.f, l = (lane < nw) ? sl[k][lane] : 0.f;
#pragma unroll
      for (int off = kMaxBlock / 64; off > 0; off >>= 1) {
        const float oh = __shfl_down_sync(0xffffffffu, h, off), ol = __shfl_down_sync(0xffffffffu, l, off);
        two_sum_acc(h, l, oh);
        l = __fadd_rn(l, ol);
      }
      if (lane == 0) {
        double* reg = P.region(r[k]);
        reg[2 * slot] = (double)h;
        reg[2 * slot + 1] = (double)l;
      }
    }
  }
  __syncthreads();
}

// block-strided loop: thread handles i = base + k*blockDim.x, k < kEPT
#define TMC_FOR_EPT(i, n)                                                              \
  for (int _k = 0, i = blockIdx.x * (kEPT * blockDim.x) + threadIdx.x; _k < kEPT; \
       ++_k, i += blockDim.x)                                                          \
    if (i < (n))

// Upwind correction of an edge value from two-sided polynomial-fit stencils
// (operators_mod.F90:423-472 for cells, :359-412 for vertices).  `f(i)`
// returns the field at stencil point i as T; ctr0/ctr1 are the two centres.
template <class T, class F>
__device__ __forceinline__ T upwind_edge(const DStencil& S2, const DStencil& S4, int order, T coef2, T coef4, int ne,
                                         int e, int ctr0, int ctr1, T fe, T sgn_of, T dist, F f) {
  if (order == 3 || order == 4) {
    T d0, d1;
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const T fc = f(s == 0 ? ctr0 : ctr1);
      T acc = T(0);
      const int n = S2.count[(size_t)s * ne + e];
      for (int j = 0; j < n; ++j) {
        const size_t k = ((size_t)j * 2 + s) * ne + e;
        acc = acc + T(S2.w[k]) * (f(S2.idx[k]) - fc);
      }
      if (s == 0)
        d0 = acc;
      else
        d1 = acc;
    }
    fe = fe - dist * dist * ((d0 + d1) - sgn1(sgn_of) * coef2 * (d1 - d0)) / T(12);
  } else if (order == 5 || order == 6) {
    T a0, a1, b0, b1;
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const T fc = f(s == 0 ? ctr0 : ctr1);
      T acc = T(0);
      int n = S2.count[(size_t)s * ne + e];
      for (int j = 0; j < n; ++j) {
        const size_t k = ((size_t)j * 2 + s) * ne + e;
        acc = acc + T(S2.w[k]) * (f(S2.idx[k]) - fc);
      }
      T acc4 = T(0);
      n = S4.count[(size_t)s * ne + e];
      for (int j = 0; j < n; ++j) {
        const size_t k = ((size_t)j * 2 + s) * ne + e;
        acc4 = acc4 + T(S4.w[k]) * (f(S4.idx[k]) - fc);
      }
      if (s == 0) {
        a0 = acc;
        b0 = acc4;
      } else {
        a1 = acc;
        b1 = acc4;
      }
    }
    fe = fe - dist * dist * (a0 + a1) / T(12) +
         (dist * dist) * (dist * dist) * ((b0 + b1) - sgn1(sgn_of) * coef4 * (b1 - b0)) / T(60);
  }
  return fe;
}

// sum_j deriv(j, side, e) (f(fit_j) - f(centre)) of one stencil side, in stencil order
template <class T, class F>
__device__ __forceinline__ T stencil_side(const DStencil& S, int ne, int e, int side, T fc, F f) {
  T acc = T(0);
  const int n = S.count[(size_t)side * ne + e];
  for (int j = 0; j < n; ++j) {
    const size_t k = ((size_t)j * 2 + side) * ne + e;
    acc = acc + T(S.w[k]) * (f(S.idx[k]) - fc);
  }
  return acc;
}

// ---------------------------------------------------------------------------
// edge_prep: gd_edge, u, mass flux F, tracer fluxes
// ---------------------------------------------------------------------------
// The cell-side values an edge preparation reads: gd (FP64, or the FP32
// shadow) and the tracer mass (FP64) or mixing-ratio shadow (FP32) of one
// state slot.
template <class T>
struct CellSrc {
  const double* gd;
  const float* gdf;
  const T* q;
  const float* qr;
};

// Edge preparation of one edge (operators_mod.F90:93-104 c2e, :423-472 upwind
// correction with the sign of iap_u, :168-176 inverse IAP; the mass flux
// u*gd_edge of tmcore_swm_mod.F90:135; for tracers of order >= 3 the sg11
// edge value of adv_scheme_sg11_mod.F90:42-45 times the mass flux).
// g1, g2 are the two cells' gd in T, already loaded by the caller.
template <class T>
__device__ __forceinline__ void prep_edge(const DevMesh& M, const ModelOpt& O, int e, int c1, int c2, T ia, T g1,
                                          T g2, const CellSrc<T>& C, T* gd_e, T* u, T* F, T* Fq) {
  T ge = T(0.5) * (g1 + g2);
  if (O.adv_order >= 3) {
    if constexpr (kF64<T>) {
      const double* gd = C.gd;
      ge = upwind_edge<T>(M.cell2, M.cell4, O.adv_order, T(O.cell_coef2), T(O.cell_coef4), M.ne, e, c1, c2, ge, ia,
                          M.dcEdge[e], [gd](int i) { return gd[i]; });
    } else {
      const float* gd = C.gdf;
      ge = upwind_edge<T>(M.cell2, M.cell4, O.adv_order, T(O.cell_coef2), T(O.cell_coef4), M.ne, e, c1, c2, ge, ia,
                          M.dcEdge_f[e], [gd](int i) { return gd[i]; });
    }
  }
  const T sq = sqrt(ge);
  const T uu = ia / sq;
  const T Fv = uu * ge;
  gd_e[e] = ge;
  u[e] = uu;
  F[e] = Fv;
  // second-order tracers are fluxed by k_cell directly (no per-edge flux stored)
  for (int k = 0; k < (O.tr_order >= 3 ? O.n_tracers : 0); ++k) {
    T qe;
    if constexpr (kF64<T>) {
      const double* q = C.q + (size_t)k * M.nc;
      const double* gd = C.gd;
      qe = 0.5 * (q[c1] / g1 + q[c2] / g2);
      qe = upwind_edge<T>(M.cell2, M.cell4, O.tr_order, T(O.tr_coef2), T(O.tr_coef4), M.ne, e, c1, c2, qe, ia,
                          M.dcEdge[e], [q, gd](int i) { return q[i] / gd[i]; });
    } else {
      const float* qr = C.qr + (size_t)k * M.nc;
      qe = 0.5f * (qr[c1] + qr[c2]);
      qe = upwind_edge<T>(M.cell2, M.cell4, O.tr_order, T(O.tr_coef2), T(O.tr_coef4), M.ne, e, c1, c2, qe, ia,
                          M.dcEdge_f[e], [qr](int i) { return qr[i]; });
    }
    Fq[(size_t)k * M.ne + e] = Fv * qe;
  }
}

template <class T>
__device__ __forceinline__ T energy_term(const DevMesh& M, int e, T ia) {
  if constexpr (kF64<T>)
    return ia * ia * M.areaEdge[e];  // tmcore_swm_mod.F90:229
  else
    return ia * ia * M.areaEdge_f[e];
}

// Stand-alone edge preparation of a state slot (the first stage after the
// state was set, the diagnostic pass, spatial_operators).
template <class T, bool kB>
__global__ void __launch_bounds__(kMaxBlock) k_edge_prep(DevMesh M, ModelOpt O, StageIO<T> S0, Partials P0, int diag) {
  const StageIO<T> S = kB ? S0.at(blockIdx.y) : S0;
  const Partials P = kB ? P0.at(blockIdx.y) : P0;
  double en = 0.0;
  const CellSrc<T> C{S.gd_in, S.gdf_in, S.q_in, S.qr_in};
  TMC_FOR_EPT(e, M.ne) {
    const int c1 = M.cellsOnEdge[e], c2 = M.cellsOnEdge[M.ne + e];
    const T ia = S.iap_in[e];
    T g1, g2;
    if constexpr (kF64<T>) {
      g1 = S.gd_in[c1];
      g2 = S.gd_in[c2];
    } else {
      g1 = S.gdf_in[c1];
      g2 = S.gdf_in[c2];
    }
    prep_edge<T>(M, O, e, c1, c2, ia, g1, g2, C, S.gd_e, S.u, S.F, S.Fq);
    if (diag) {
      if constexpr (kF64<T>)
        en = en + energy_term<T>(M, e, ia);
      else
        en += (double)energy_term<T>(M, e, ia);
    }
  }
  if (diag) {
    const double v[1] = {en};
    const int r[1] = {R_EN_E};
    block_store<double, 1>(v, P, r);
  }
}

// ---------------------------------------------------------------------------
// cell: div of mass flux, kinetic energy, E, RK update of gd and tracers
// ---------------------------------------------------------------------------
template <class T, bool kB>
__global__ void __launch_bounds__(kMaxBlock) k_cell(DevMesh M, ModelOpt O, StageIO<T> S0, RKStage rk, Partials P0,
                                                    int diag) {
  const StageIO<T> S = kB ? S0.at(blockIdx.y) : S0;
  const Partials P = kB ? P0.at(blockIdx.y) : P0;
  T rip = T(0), r44 = T(0);
  double mass = 0.0, enc = 0.0;
  TMC_FOR_EPT(c, M.nc) {
    double t;  // gd tendency, FP64 in both modes
    T tT, ke;
    int eidx[kME], cidx[kME];
    float nsg[kME];
    const int n = M.nEdgesOnCell[c];
    const int mode = rk.mode;
    // RK inputs before any store (see k_edge_flux)
    const double gold = (mode >= 1 && mode <= 3) ? S.gd_old[c] : 0.0;
    const double gacc = (mode >= 2) ? S.gd_acc[c] : 0.0;
    T tprev = T(0);
    if constexpr (kF64<T>)
      tprev = (mode >= 2) ? S.gd_tend[c] : 0.0;
    else
      tprev = (mode >= 2) ? S.tendf[c] : 0.f;
    const double gdin = diag ? S.gd_in[c] : 0.0, ghsd = diag ? S.ghs[c] : 0.0;
    if constexpr (kF64<T>) {
      // operators_mod.F90:40-55 (div_operator of u*gd_edge) and :206-221, in order
      double s = 0.0, k = 0.0;
      for (int i = 0; i < n; ++i) {
        const int e = M.edgesOnCell[(size_t)i * M.nc + c];
        const double uu = S.u[e];
        s = s + (double)M.nSign[(size_t)i * M.nc + c] * S.F[e] * M.dvEdge[e];
        k = k + uu * uu * M.areaEdge[e];
      }
      const double A = M.areaCell[c];
      t = (-s) / A;
      tT = t;
      ke = (k * 0.25) / A;
      S.E[c] = ke + S.gd_in[c] + S.ghs[c];
      (void)eidx;
      (void)cidx;
      (void)nsg;
    } else {
      float uu[kME], Fv[kME], dv[kME], ae[kME];
      const bool tr_direct = O.n_tracers > 0 && O.tr_order == 2;
#pragma unroll
      for (int i = 0; i < kME; ++i) {
        eidx[i] = M.edgesOnCell[(size_t)i * M.nc + c];  // padded slots: index 0, sign 0
        nsg[i] = (float)M.nSign[(size_t)i * M.nc + c];
        cidx[i] = tr_direct ? M.cellsOnCell[(size_t)i * M.nc + c] : 0;
      }
#pragma unroll
      for (int i = 0; i < kME; ++i) {
        uu[i] = S.u[eidx[i]];
        Fv[i] = S.F[eidx[i]];
        dv[i] = M.dvEdge_f[eidx[i]];
        ae[i] = M.areaEdge_f[eidx[i]];
      }
      float hi = 0.f, lo = 0.f, k = 0.f;
#pragma unroll
      for (int i = 0; i < kME; ++i) {
        // the FP32 flux of an edge is bit-identical in its two cells; the two-sum
        // keeps their sum exact enough for mass conservation to FP64 round-off
        two_sum_acc(hi, lo, __fmul_rn(__fmul_rn(nsg[i], Fv[i]), dv[i]));
        k += fabsf(nsg[i]) * uu[i] * uu[i] * ae[i];
      }
      t = -((double)hi + (double)lo) * M.invAreaCell[c];
      tT = (float)t;
      ke = k * 0.25f * M.invAreaCell_f[c];
      S.E[c] = ke + S.gdf_in[c] + S.ghsf[c];
    }
    (void)n;
    const double Ad = M.areaCell[c];
    double gnext = 0.0;
    if constexpr (kF64<T>) {
      double* tb = S.gd_tend;
      switch (mode) {
        case 0:
          tb[c] = t;
          break;
        case 1:
          S.gd_acc[c] = t;
          tb[c] = t;
          gnext = gold + rk.a_dt * t;
          S.gd_next[c] = gnext;
          break;
        case 2:
        case 3: {
          rip = rip + tprev * t * Ad;
          S.gd_acc[c] = gacc + 2.0 * t;
          tb[c] = t;
          gnext = gold + rk.a_dt * t;
          S.gd_next[c] = gnext;
          break;
        }
        case 4: {
          rip = rip + tprev * t * Ad;
          const double tn = (gacc + t) / 6.0;
          S.gd_acc[c] = tn;
          r44 = r44 + tn * tn * Ad;
          tb[c] = t;
          break;
        }
      }
    } else {
      float* tb = S.tendf;
      const float Af = M.areaCell_f[c];
      switch (mode) {
        case 0:
          S.gd_tend[c] = t;
          tb[c] = tT;
          break;
        case 1:
          S.gd_acc[c] = t;
          tb[c] = tT;
          gnext = gold + rk.a_dt * t;
          S.gd_next[c] = gnext;
          S.gdf_next[c] = (float)gnext;
          break;
        case 2:
        case 3: {
          rip += tprev * tT * Af;
          S.gd_acc[c] = gacc + 2.0 * t;
          tb[c] = tT;
          gnext = gold + rk.a_dt * t;
          S.gd_next[c] = gnext;
          S.gdf_next[c] = (float)gnext;
          break;
        }
        case 4: {
          rip += tprev * tT * Af;
          const double tn = (gacc + t) * (1.0 / 6.0);
          S.gd_acc[c] = tn;
          const float tnf = (float)tn;
          r44 += tnf * tnf * Af;
          tb[c] = tT;
          break;
        }
      }
    }
    // tracers, kTr at a time: loads and divergences first, then the stores
    constexpr int kTr = 4;
    for (int q0 = 0; q0 < O.n_tracers; q0 += kTr) {
      T tq[kTr], qo[kTr], qa[kTr];
#pragma unroll
      for (int j = 0; j < kTr; ++j) {
        const int q = q0 + j;
        tq[j] = qo[j] = qa[j] = T(0);
        if (q >= O.n_tracers) continue;
        const size_t qi = (size_t)q * M.nc + c;
        qo[j] = (mode >= 1 && mode <= 3) ? S.q_old[qi] : T(0);
        qa[j] = (mode >= 2) ? S.q_acc[qi] : T(0);
        // Second-order tracers take the edge value from the two cells directly,
        // q_edge = (q(c1) + q(c2))/2, so no per-edge tracer flux is stored;
        // higher orders read the fluxes k_edge_prep wrote with the upwind
        // correction.
        const bool direct = (O.tr_order == 2);
        if constexpr (kF64<T>) {
          double sq = 0.0;
          const double qs = direct ? S.q_in[qi] / S.gd_in[c] : 0.0;
          for (int i = 0; i < n; ++i) {
            const int e = M.edgesOnCell[(size_t)i * M.nc + c];
            double flux;
            if (direct) {
              const int nb = M.cellsOnCell[(size_t)i * M.nc + c];
              const double qn = S.q_in[(size_t)q * M.nc + nb] / S.gd_in[nb];
              flux = S.F[e] * (0.5 * (qs + qn));
            } else {
              flux = S.Fq[(size_t)q * M.ne + e];
            }
            sq = sq + (double)M.nSign[(size_t)i * M.nc + c] * flux * M.dvEdge[e];
          }
          tq[j] = (-sq) / M.areaCell[c];
        } else {
          float sq = 0.f;
          if (direct) {
            const float qs = S.qr_in[qi];
#pragma unroll
            for (int i = 0; i < kME; ++i) {
              const float qn = S.qr_in[(size_t)q * M.nc + cidx[i]];
              sq += nsg[i] * S.F[eidx[i]] * (0.5f * (qs + qn)) * M.dvEdge_f[eidx[i]];
            }
          } else {
#pragma unroll
            for (int i = 0; i < kME; ++i)
              sq += nsg[i] * S.Fq[(size_t)q * M.ne + eidx[i]] * M.dvEdge_f[eidx[i]];
          }
          tq[j] = -sq * M.invAreaCell_f[c];
        }
      }
#pragma unroll
      for (int j = 0; j < kTr; ++j) {
        const int q = q0 + j;
        if (q >= O.n_tracers) continue;
        const size_t qi = (size_t)q * M.nc + c;
        T qnext = T(0);
        const T adt = T(rk.a_dt);
        switch (mode) {
          case 1:
            S.q_acc[qi] = tq[j];
            qnext = qo[j] + adt * tq[j];
            if constexpr (kF64<T>) S.q_next[qi] = qnext;  // FP32: the next stage reads the ratio only
            break;
          case 2:
          case 3:
            S.q_acc[qi] = qa[j] + T(2) * tq[j];
            qnext = qo[j] + adt * tq[j];
            if constexpr (kF64<T>) S.q_next[qi] = qnext;
            break;
          case 4:
            if constexpr (kF64<T>)
              S.q_acc[qi] = (qa[j] + tq[j]) / 6.0;
            else
              S.q_acc[qi] = (qa[j] + tq[j]) * (1.0f / 6.0f);
            break;
          default:
            S.q_acc[qi] = tq[j];
        }
        if constexpr (!kF64<T>) {
          if (mode >= 1 && mode <= 3) S.qr_next[qi] = qnext / (float)gnext;
        }
      }
    }
    if (diag) {
      mass = mass + gdin * Ad;
      enc = enc + (gdin * gdin + 2.0 * gdin * ghsd) * Ad;
    }
  }
  if (rk.mode >= 2) {
    const T v[2] = {rip, r44};
    const int r[2] = {R_IP_C + 2 * (rk.mode - 2), R_44_C};
    block_store<T, 2>(v, P, r);
  }
  if (diag) {
    const double v[2] = {mass, enc};
    const int r[2] = {R_MASS, R_EN_C};
    block_store<double, 2>(v, P, r);
  }
}

// ---------------------------------------------------------------------------
// vertex: gd on vertices, vorticity, potential vorticity
// ---------------------------------------------------------------------------
template <class T, bool kB>
__global__ void __launch_bounds__(kMaxBlock) k_vertex(DevMesh M, ModelOpt O, StageIO<T> S0, Partials P0, int diag) {
  const StageIO<T> S = kB ? S0.at(blockIdx.y) : S0;
  const Partials P = kB ? P0.at(blockIdx.y) : P0;
  double pe = 0.0, av = 0.0;      // FP64 path
  float ph = 0.f, pl = 0.f, ah = 0.f, al = 0.f;  // FP32 path: compensated sums
  if constexpr (kF64<T>) {
    TMC_FOR_EPT(v, M.nv) {
      // operators_mod.F90:106-123 (c2v), :76-91 (curl), :262-270 (pv)
      double s = 0.0, gv = 0.0;
#pragma unroll
      for (int i = 0; i < 3; ++i)
        gv = gv + S.gd_in[M.cellsOnVertex[(size_t)i * M.nv + v]] * M.kite[(size_t)i * M.nv + v];
      const double At = M.areaTriangle[v];
      gv = gv / At;
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const int e = M.edgesOnVertex[(size_t)i * M.nv + v];
        s = s + (double)M.tSign[(size_t)i * M.nv + v] * S.u[e] * M.dcEdge[e];
      }
      const double vo = (-s) / At;
      const double pv = (M.fVertex[v] + vo) / gv;
      S.pv_v[v] = pv;
      if (S.vor) S.vor[v] = vo;
      if (S.gd_v) S.gd_v[v] = gv;
      if (diag) {
        pe = pe + gv * (pv * pv) * At;
        av = av + (vo + M.fVertex[v]) * At;
      }
    }
  } else {
    // one vertex at a time: measured faster than batching the loads of the
    // thread's vertices (which costs occupancy for a pass with three gathers)
    // Every load is a read-only (non-coherent) load: nothing this kernel
    // stores aliases them, which lets the compiler issue a vertex's loads
    // ahead of the previous vertex's stores.
    TMC_FOR_EPT(v, M.nv) {
      int ci[3], ei[3];
      float kt[3], ts[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        ci[i] = __ldg(M.cellsOnVertex + (size_t)i * M.nv + v);
        ei[i] = __ldg(M.edgesOnVertex + (size_t)i * M.nv + v);
        kt[i] = __ldg(M.kite_f + (size_t)i * M.nv + v);
        ts[i] = (float)__ldg(M.tSign + (size_t)i * M.nv + v);
      }
      float g[3], uu[3], dc[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        g[i] = __ldg(S.gdf_in + ci[i]);
        uu[i] = __ldg(S.u + ei[i]);
        dc[i] = __ldg(M.dcEdge_f + ei[i]);
      }
      const float iA = __ldg(M.invAreaTriangle_f + v);
      const float At = diag ? __ldg(M.areaTriangle_f + v) : 0.f;
      const float fv = __ldg(M.fVertex_f + v);
      const float gv = (g[0] * kt[0] + g[1] * kt[1] + g[2] * kt[2]) * iA;
      const float sv = ts[0] * uu[0] * dc[0] + ts[1] * uu[1] * dc[1] + ts[2] * uu[2] * dc[2];
      const float vo = -sv * iA;
      const float pv = (fv + vo) / gv;
      S.pv_v[v] = pv;
      if (S.vor) S.vor[v] = vo;
      if (S.gd_v) S.gd_v[v] = gv;
      if (diag) {
        // potential enstrophy and absolute vorticity (tmcore_swm_mod.F90:233-255)
        // from FP32 terms with compensated sums: FP64 terms made this launch
        // FP64-pipe bound
        two_sum_acc(ph, pl, gv * (pv * pv) * At);
        two_sum_acc(ah, al, vo * At);
        two_sum_acc(ah, al, fv * At);
      }
    }
  }
  (void)O;
  if (diag) {
    const int r[2] = {R_PE, R_AV};
    if constexpr (kF64<T>) {
      const double vv[2] = {pe, av};
      block_store<double, 2>(vv, P, r);
    } else {
      const float h[2] = {ph, ah}, l[2] = {pl, al};
      block_store_ff<2>(h, l, P, r);
    }
  }
}

// pv on cells: scalar_v2c_interp_operator as a gather (operators_mod.F90:125-141)
template <class T>
__global__ void __launch_bounds__(kMaxBlock) k_v2c(DevMesh M, const T* pv_v0, T* pv_c0, long long msv, long long msc) {
  const T* pv_v = pv_v0 + blockIdx.y * msv;
  T* pv_c = pv_c0 + blockIdx.y * msc;
  TMC_FOR_EPT(c, M.nc) {
    const T A = T(M.areaCell[c]);
    T s = T(0);
    for (int k = M.v2c_start[c]; k < M.v2c_start[c + 1]; ++k) s = s + pv_v[M.v2c_vertex[k]] * T(M.v2c_kite[k]) / A;
    pv_c[c] = s;
  }
}

// ---------------------------------------------------------------------------
// edge_pv: PV on edges (calc_pv_on_edge, operators_mod.F90:273-412)
// ---------------------------------------------------------------------------
template <class T, bool kB>
__global__ void __launch_bounds__(kMaxBlock) k_edge_pv(DevMesh M, ModelOpt O, StageIO<T> S0) {
  const StageIO<T> S = kB ? S0.at(blockIdx.y) : S0;
  const bool need_v = (O.pv_scheme >= 2) || (O.pv_scheme == 1 && O.apvm_weight != 0.0);
  if (!need_v) {
    // centred pv (APVM weight 0): all loads of the thread's kEPT edges first
    const int e0 = blockIdx.x * (kEPT * blockDim.x) + threadIdx.x;
    int v1[kEPT], v2[kEPT];
    T pe[kEPT];
#pragma unroll
    for (int j = 0; j < kEPT; ++j) {
      const int e = e0 + j * blockDim.x;
      v1[j] = e < M.ne ? M.verticesOnEdge[e] : 0;
      v2[j] = e < M.ne ? M.verticesOnEdge[M.ne + e] : 0;
    }
#pragma unroll
    for (int j = 0; j < kEPT; ++j) pe[j] = T(0.5) * (S.pv_v[v1[j]] + S.pv_v[v2[j]]);
#pragma unroll
    for (int j = 0; j < kEPT; ++j) {
      const int e = e0 + j * blockDim.x;
      if (e < M.ne) S.pv_e[e] = pe[j];
    }
    return;
  }
  TMC_FOR_EPT(e, M.ne) {
    const int v1 = M.verticesOnEdge[e], v2 = M.verticesOnEdge[M.ne + e];
    const T p1 = S.pv_v[v1], p2 = S.pv_v[v2];
    T pe = T(0.5) * (p1 + p2);
    T ve = T(0);
    if (need_v) {
      const int n = M.nEdgesOnEdge[e];
      for (int i = 0; i < n; ++i) {
        const size_t k = (size_t)i * M.ne + e;
        ve = ve + S.u[M.edgesOnEdge[k]] * met<T>(M.weightsOnEdge, M.weightsOnEdge_f, k);
      }
      if (S.v_e) S.v_e[e] = ve;
    }
    if (O.pv_scheme == 1) {
      if (O.apvm_weight != 0.0) {
        const int c1 = M.cellsOnEdge[e], c2 = M.cellsOnEdge[M.ne + e];
        const T a = ve * (p2 - p1) / met<T>(M.dvEdge, M.dvEdge_f, e);
        const T b = S.u[e] * (S.pv_c[c2] - S.pv_c[c1]) / met<T>(M.dcEdge, M.dcEdge_f, e);
        pe = pe - T(O.apvm_weight * O.dt) * (a + b);
      }
    } else if (O.pv_scheme == 2) {
      // correction direction of the conservative APVM (operators_mod.F90:336-341);
      // pv_edge stays the centred average until k_cons_apply
      const int c1 = M.cellsOnEdge[e], c2 = M.cellsOnEdge[M.ne + e];
      const T a = ve * (p2 - p1) / met<T>(M.dvEdge, M.dvEdge_f, e);
      const T b = S.u[e] * (S.pv_c[c2] - S.pv_c[c1]) / met<T>(M.dcEdge, M.dcEdge_f, e);
      S.dpv[e] = a + b;
    } else if (O.pv_scheme == 3) {
      const T* pv = S.pv_v;
      pe = upwind_edge<T>(M.vert2, M.vert4, O.interp_pv_order, T(O.vert_coef2), T(O.vert_coef4), M.ne, e, v1, v2,
                          pe, ve, met<T>(M.dvEdge, M.dvEdge_f, e), [pv](int i) { return pv[i]; });
    }
    S.pv_e[e] = pe;
  }
}

// FP32 upwind pv on edges (pv_scheme 3, interp_pv_order 3 or 4;
// operators_mod.F90:359-412, the tangential velocity :223-237): one edge per
// thread.  The two-sided vertex fit stencils come as packed (index, FP32
// weight) entries, one 8-byte load each, and every load of the edge is issued
// up front: the tangential-velocity gathers over a fixed 10 slots (padded
// slots are the edge itself with weight 0) and the stencil points up to the
// width with the side's count as a predicate, so an edge's ~35 gathers are in
// flight together instead of a count-dependent chain.  Sums in stencil order.
// Resident 256-thread blocks per SM the kernel is compiled for.  It is
// latency bound (two dependent loads per stencil point): at level 8 the pass
// takes 0.295 ms with 2 (128 registers), 0.183 ms with 3 (80) and 0.171 ms
// with 4 (64 registers, about 100 bytes spilled to L1).
#ifndef TMC_UP32_MINB
#define TMC_UP32_MINB 4
#endif
template <bool kB>
__global__ void __launch_bounds__(256, TMC_UP32_MINB) k_edge_pv_up32(DevMesh M, ModelOpt O, StageIO<float> S0) {
  const StageIO<float> S = kB ? S0.at(blockIdx.y) : S0;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= M.ne) return;
  const int ne = M.ne, W = M.vert2.width;
  const int v1 = __ldg(M.verticesOnEdge + e), v2 = __ldg(M.verticesOnEdge + ne + e);
  const int n0 = __ldg(M.vert2.count + e), n1 = __ldg(M.vert2.count + ne + e);
  int eo[kME2];
  float wo[kME2];
#pragma unroll
  for (int i = 0; i < kME2; ++i) {
    eo[i] = __ldg(M.edgesOnEdge + (size_t)i * ne + e);
    wo[i] = __ldg(M.weightsOnEdge_f + (size_t)i * ne + e);
  }
  const int m0 = min(n0, W), m1 = min(n1, W);
  int2 iw[2][kUpW32];
#pragma unroll
  for (int j = 0; j < kUpW32; ++j) {
    iw[0][j] = j < m0 ? __ldg(M.vert2_iw + ((size_t)j * 2 + 0) * ne + e) : make_int2(0, 0);
    iw[1][j] = j < m1 ? __ldg(M.vert2_iw + ((size_t)j * 2 + 1) * ne + e) : make_int2(0, 0);
  }
  const float p1 = __ldg(S.pv_v + v1), p2 = __ldg(S.pv_v + v2);
  float uo[kME2];
#pragma unroll
  for (int i = 0; i < kME2; ++i) uo[i] = __ldg(S.u + eo[i]);
  float f[2][kUpW32];
#pragma unroll
  for (int j = 0; j < kUpW32; ++j) {
    f[0][j] = j < m0 ? __ldg(S.pv_v + iw[0][j].x) : 0.f;
    f[1][j] = j < m1 ? __ldg(S.pv_v + iw[1][j].x) : 0.f;
  }
  float ve = 0.f;
#pragma unroll
  for (int i = 0; i < kME2; ++i) ve = ve + uo[i] * wo[i];
  float d[2];
#pragma unroll
  for (int sd = 0; sd < 2; ++sd) {
    const float fc = sd == 0 ? p1 : p2;
    const int n = sd == 0 ? m0 : m1;
    float acc = 0.f;
#pragma unroll
    for (int j = 0; j < kUpW32; ++j)
      if (j < n) acc = acc + __int_as_float(iw[sd][j].y) * (f[sd][j] - fc);
    d[sd] = acc;
  }
  const float dist = __ldg(M.dvEdge_f + e);
  const float pe = 0.5f * (p1 + p2) -
                   dist * dist * ((d[0] + d[1]) - sgn1(ve) * (float)O.vert_coef2 * (d[1] - d[0])) / 12.f;
  if (S.v_e) S.v_e[e] = ve;
  S.pv_e[e] = pe;
}

// ---------------------------------------------------------------------------
// conservative APVM (calc_pv_on_edge, pv_scheme 2, operators_mod.F90:318-357)
// ---------------------------------------------------------------------------
// calc_tangent_vor_flux (:239-260) of pv_edge and of the correction dpv; the
// factor w u gd_edge / 2 of a neighbour is shared by both sums
template <class T, bool kB>
__global__ void __launch_bounds__(kMaxBlock) k_cons_tvf(DevMesh M, StageIO<T> S0) {
  const StageIO<T> S = kB ? S0.at(blockIdx.y) : S0;
  TMC_FOR_EPT(e, M.ne) {
    const int n = M.nEdgesOnEdge[e];
    const T pe = S.pv_e[e], dp = S.dpv[e];
    T a = T(0), b = T(0);
    for (int i = 0; i < n; ++i) {
      const size_t k = (size_t)i * M.ne + e;
      const int ep = M.edgesOnEdge[k];
      const T f = met<T>(M.weightsOnEdge, M.weightsOnEdge_f, k) * S.u[ep] * S.gd_e[ep] * T(0.5);
      a = a + f * (pe + S.pv_e[ep]);
      b = b + f * (dp + S.dpv[ep]);
    }
    S.pvf[e] = a;
    S.dpvf[e] = b;
  }
}

// per vertex: c2v of the gd tendency (:106-123), the curls of both tangent
// fluxes (calc_vor_tend_on_vertex :414-421), and the partial sums
// s1 = sum pv^2 tend_gd_v A, s2 = sum pv curl(pvf) A, s3 = sum pv curl(dpvf) A
template <class T, bool kB>
__global__ void __launch_bounds__(kMaxBlock) k_cons_vertex(DevMesh M, StageIO<T> S0, Partials P0) {
  const StageIO<T> S = kB ? S0.at(blockIdx.y) : S0;
  const Partials P = kB ? P0.at(blockIdx.y) : P0;
  double s1 = 0.0, s2 = 0.0, s3 = 0.0;
  TMC_FOR_EPT(v, M.nv) {
    if constexpr (kF64<T>) {
      const double At = M.areaTriangle[v];
      double g = 0.0, a = 0.0, b = 0.0;
#pragma unroll
      for (int i = 0; i < 3; ++i)
        g = g + S.gd_tend[M.cellsOnVertex[(size_t)i * M.nv + v]] * M.kite[(size_t)i * M.nv + v];
      g = g / At;
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const int e = M.edgesOnVertex[(size_t)i * M.nv + v];
        const double ts = (double)M.tSign[(size_t)i * M.nv + v];
        a = a + ts * S.pvf[e] * M.dcEdge[e];
        b = b + ts * S.dpvf[e] * M.dcEdge[e];
      }
      const double vt = (-a) / At, dvt = (-b) / At, pv = S.pv_v[v];
      s1 = s1 + pv * pv * g * At;
      s2 = s2 + pv * vt * At;
      s3 = s3 + pv * dvt * At;
    } else {
      const float iA = M.invAreaTriangle_f[v];
      float g = 0.f, a = 0.f, b = 0.f;
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        g += S.tendf[M.cellsOnVertex[(size_t)i * M.nv + v]] * M.kite_f[(size_t)i * M.nv + v];
        const int e = M.edgesOnVertex[(size_t)i * M.nv + v];
        const float ts = (float)M.tSign[(size_t)i * M.nv + v];
        a += ts * S.pvf[e] * M.dcEdge_f[e];
        b += ts * S.dpvf[e] * M.dcEdge_f[e];
      }
      const double At = M.areaTriangle[v];
      const float pv = S.pv_v[v];
      s1 += (double)(pv * pv * (g * iA)) * At;
      s2 += (double)(pv * (-a * iA)) * At;
      s3 += (double)(pv * (-b * iA)) * At;
    }
  }
  const double vals[3] = {s1, s2, s3};
  const int r[3] = {R_C1, R_C2, R_C3};
  block_store<double, 3>(vals, P, r);
}

// pv_edge = pv_edge - eps dt dpv (:355)
template <class T, bool kB>
__global__ void __launch_bounds__(kMaxBlock) k_cons_apply(DevMesh M, ModelOpt O, StageIO<T> S0, const double* eps0) {
  const StageIO<T> S = kB ? S0.at(blockIdx.y) : S0;
  const double* eps = kB ? eps0 + (size_t)blockIdx.y * kDiagStride : eps0;
  const double ed = *eps * O.dt;
  TMC_FOR_EPT(e, M.ne) S.pv_e[e] = S.pv_e[e] - T(ed) * S.dpv[e];
}

// ---------------------------------------------------------------------------
// generic integrators: state update, combination of tendencies, inner products
// ---------------------------------------------------------------------------
// cells [0, nc) then edges [nc, nc + ne) in one index space
template <class T>
__global__ void __launch_bounds__(kMaxBlock) k_update(DevMesh M, int ntr, UpdateArgs<T> a) {
  const double coef = a.coef_dev ? *a.coef_dev : a.a_dt;
  const int n = M.nc + (a.tiap ? M.ne : 0);
  TMC_FOR_EPT(i, n) {
    if (i < M.nc) {
      const int c = i;
      const double g = a.gd_o[c] + coef * a.tgd[c];  // tmcore_swm_mod.F90:211
      a.gd_n[c] = g;
      if constexpr (!kF64<T>) a.gdf_n[c] = (float)g;
      for (int k = 0; k < ntr; ++k) {
        const size_t qi = (size_t)k * M.nc + c;
        const T q = a.q_o[qi] + T(coef) * a.tq[qi];
        a.q_n[qi] = q;
        if constexpr (!kF64<T>) a.qr_n[qi] = q / (float)g;
      }
    } else {
      const int e = i - M.nc;
      a.iap_n[e] = a.iap_o[e] + T(coef) * a.tiap[e];  // :210
    }
  }
}

template <class T>
__global__ void __launch_bounds__(kMaxBlock) k_combine(DevMesh M, int ntr, int scheme, CombineArgs<T> a,
                                                       Partials P) {
  // inner products of operators_mod.F90:187-194 per region, FP64 accumulation
  double ip[4] = {0.0, 0.0, 0.0, 0.0};
  const int ncb = grid_for(M.nc, blockDim.x);  // blocks [0, ncb) do cells, the rest edges
  const bool cells = (int)blockIdx.x < ncb;
  const int n = cells ? M.nc : M.ne;
  const int b0 = cells ? 0 : ncb;
  for (int j = 0; j < kEPT; ++j) {
    const int i = ((int)blockIdx.x - b0) * blockDim.x * kEPT + j * blockDim.x + threadIdx.x;
    if (i >= n) break;
    double t[4], w;
    if (cells) {
      for (int k = 0; k < 4; ++k) t[k] = a.tgd[k] ? a.tgd[k][i] : 0.0;
      w = M.areaCell[i];
    } else {
      for (int k = 0; k < 4; ++k) t[k] = a.tiap[k] ? (double)a.tiap[k][i] : 0.0;
      w = M.areaEdge[i];
    }
    if (scheme == 3) {  // PC2: <t0,t1>, <t1,t1>
      ip[0] = ip[0] + t[0] * t[1] * w;
      ip[3] = ip[3] + t[1] * t[1] * w;
      continue;
    }
    double tn;
    if (scheme == 1) {  // CRK3 (time_scheme_mod.F90:90-100)
      tn = (t[0] + 4.0 * t[1] + t[2]) / 6.0;
      ip[0] = ip[0] + t[0] * t[1] * w;
      ip[1] = ip[1] + t[0] * t[2] * w;
      ip[2] = ip[2] + t[1] * t[2] * w;
    } else {  // CRK4 (:140-150)
      tn = (t[0] + 2.0 * t[1] + 2.0 * t[2] + t[3]) / 6.0;
      ip[0] = ip[0] + t[0] * t[1] * w;
      ip[1] = ip[1] + t[1] * t[2] * w;
      ip[2] = ip[2] + t[2] * t[3] * w;
    }
    if (cells) {
      a.tgd[0][i] = tn;
      for (int q = 0; q < ntr; ++q) {
        const size_t qi = (size_t)q * M.nc + i;
        const T q0 = a.tq[0][qi], q1 = a.tq[1][qi], q2 = a.tq[2][qi];
        if (scheme == 1) {
          a.tq[0][qi] = (q0 + T(4) * q1 + q2) / T(6);
        } else {
          const T q3 = a.tq[3][qi];
          a.tq[0][qi] = (q0 + T(2) * q1 + T(2) * q2 + q3) / T(6);
        }
      }
    } else if (a.tiap[0]) {
      if constexpr (kF64<T>) {
        a.tiap[0][i] = tn;
      } else {
        tn = (double)(T)tn;
        a.tiap[0][i] = (T)tn;
      }
    }
    if (cells || a.tiap[0]) ip[3] = ip[3] + tn * tn * w;
  }
  const int base = cells ? R_IP_C : R_IP_E;
  const int r4 = cells ? R_44_C : R_44_E;
  const int r[4] = {base, base + 2, base + 4, r4};
  // partial slot: the block index within its half, cells [0, ncb), edges [0, neb)
  block_store<double, 4>(ip, P, r, (int)blockIdx.x - b0);
}

// Launch KERNEL<T, kB> over (GRIDX, members): the member-batched variant
// (kB = true, FP32 only) when the stage has several ensemble members, else the
// single-member code, which addresses its arrays straight from the kernel
// parameters.
#define TMC_LAUNCH(KERNEL, GRIDX, ...)                                     \
  do {                                                                     \
    if constexpr (!kF64<T>) {                                              \
      if (S.members > 1) {                                                 \
        KERNEL<T, true><<<dim3(GRIDX, nmem(S)), bs, 0, st>>>(__VA_ARGS__); \
        break;                                                             \
      }                                                                    \
    }                                                                      \
    KERNEL<T, false><<<dim3(GRIDX, 1), bs, 0, st>>>(__VA_ARGS__);          \
  } while (0)

template <class T>
void launch_cons_apvm(const DevMesh& M, const ModelOpt& O, const StageIO<T>& S, Partials P, double* diag_out, int bs,
                      cudaStream_t st) {
  TMC_LAUNCH(k_cons_tvf, grid_for(M.ne, bs), M, S);
  TMC_LAUNCH(k_cons_vertex, grid_for(M.nv, bs), M, S, P);
  launch_cons_eps(P, grid_for(M.nv, bs), O.dt, diag_out, st, (int)nmem(S));
  TMC_LAUNCH(k_cons_apply, grid_for(M.ne, bs), M, O, S, diag_out + 10);
}

template <class T>
void launch_update(const DevMesh& M, int ntr, const UpdateArgs<T>& a, int bs, cudaStream_t st) {
  const int n = M.nc + (a.tiap ? M.ne : 0);
  k_update<T><<<grid_for(n, bs), bs, 0, st>>>(M, ntr, a);
}

template <class T>
void launch_combine(const DevMesh& M, int ntr, int scheme, const CombineArgs<T>& a, Partials P, int bs,
                    cudaStream_t st) {
  const int g = grid_for(M.nc, bs) + grid_for(M.ne, bs);
  k_combine<T><<<g, bs, 0, st>>>(M, ntr, scheme, a, P);
}

// ---------------------------------------------------------------------------
// edge_flux: q.F_perp, gradient of E, iap_u tendency, RK update, inner products
// ---------------------------------------------------------------------------
template <class T, bool kB>
__device__ __forceinline__ void edge_flux_body(const DevMesh& M, const ModelOpt& O, const StageIO<T>& S0, RKStage rk,
                                               const Partials& P0) {
  const StageIO<T> S = kB ? S0.at(blockIdx.y) : S0;
  const Partials P = kB ? P0.at(blockIdx.y) : P0;
  T rip = T(0), r44 = T(0);  // FP32 path: FP32 products and per-thread sums, FP64 across warps
  const int mode = rk.mode;
  TMC_FOR_EPT(e, M.ne) {
    // Loads that depend on no other load come first, before any store: a load
    // issued after a store through a pointer the compiler must assume aliases
    // would wait a full memory round trip.
    const int c1 = M.cellsOnEdge[e], c2 = M.cellsOnEdge[M.ne + e];
    const T pe = S.pv_e[e];
    const T uu = S.u[e];
    const T ge = S.gd_e[e];
    const T tp = (mode >= 2) ? S.iap_tend[e] : T(0);
    const T accv = (mode >= 2) ? S.iap_acc[e] : T(0);
    const T oldv = (mode >= 1 && mode <= 3) ? S.iap_old[e] : T(0);
    const T ae = (mode >= 2) ? met<T>(M.areaEdge, M.areaEdge_f, e) : T(0);
    // the next stage's gd on the two cells (written by this stage's k_cell)
    const bool fuse = (S.u_nx != nullptr);
    T gn1 = T(0), gn2 = T(0);
    if (fuse) {
      if constexpr (kF64<T>) {
        gn1 = S.gd_next[c1];
        gn2 = S.gd_next[c2];
      } else {
        gn1 = S.gdf_next[c1];
        gn2 = S.gdf_next[c2];
      }
    }
    T s = T(0), tge, dEdx, dc;
    if constexpr (kF64<T>) {
      // calc_tangent_vor_flux (operators_mod.F90:239-260), in order
      const int n = M.nEdgesOnEdge[e];
      for (int i = 0; i < n; ++i) {
        const size_t k = (size_t)i * M.ne + e;
        const int ep = M.edgesOnEdge[k];
        s = s + M.weightsOnEdge[k] * S.u[ep] * S.gd_e[ep] * 0.5 * (pe + S.pv_e[ep]);
      }
      dc = M.dcEdge[e];
      dEdx = (S.E[c2] - S.E[c1]) / dc;
      tge = 0.5 * (S.gd_tend[c1] + S.gd_tend[c2]);
    } else {
      int ep[kME2];
      float w[kME2];
#pragma unroll
      for (int i = 0; i < kME2; ++i) {
        const size_t k = (size_t)i * M.ne + e;
        ep[i] = M.edgesOnEdge[k];  // padded entries: own edge with weight 0
        w[i] = M.weightsOnEdge_f[k];
      }
      const float E1 = S.E[c1], E2 = S.E[c2], t1 = S.tendf[c1], t2 = S.tendf[c2];
      dc = M.dcEdge_f[e];
      float Fv[kME2], pp[kME2];
#pragma unroll
      for (int i = 0; i < kME2; ++i) {
        Fv[i] = S.F[ep[i]];
        pp[i] = S.pv_e[ep[i]];
      }
#pragma unroll
      for (int i = 0; i < kME2; ++i) s += w[i] * Fv[i] * (0.5f * (pe + pp[i]));
      dEdx = (E2 - E1) / dc;
      tge = 0.5f * (t1 + t2);
    }
    if (O.flux4) {
      // flux_4th_order_correct (tmcore_swm_mod.F90:183-195): third derivatives
      // of E on the two cells' fit3 stencils
      const T* Ev = S.E;
      auto fE = [Ev](int i) { return Ev[i]; };
      const T d1 = stencil_side<T>(M.cell3, M.ne, e, 0, Ev[c1], fE);
      const T d2 = stencil_side<T>(M.cell3, M.ne, e, 1, Ev[c2], fE);
      dEdx = dEdx - (d2 - d1) * dc / T(24);
    }
    const T ut = s - dEdx;
    if (O.adv_order >= 3) {
      // the upwind side is the sign of the stage's iap_u (tmcore_swm_mod.F90:107-108);
      // u = iap_u / sqrt(gd_edge) carries the same sign bit, and unlike iap_u it
      // is always stored (the fused stages keep the next iap_u in registers)
      if constexpr (kF64<T>) {
        const double* gt = S.gd_tend;
        tge = upwind_edge<T>(M.cell2, M.cell4, O.adv_order, T(O.cell_coef2), T(O.cell_coef4), M.ne, e, c1, c2, tge,
                             uu, dc, [gt](int i) { return gt[i]; });
      } else {
        const float* gt = S.tendf;
        tge = upwind_edge<T>(M.cell2, M.cell4, O.adv_order, T(O.cell_coef2), T(O.cell_coef4), M.ne, e, c1, c2, tge,
                             uu, dc, [gt](int i) { return gt[i]; });
      }
    }
    // calc_u_tend_on_edge (tmcore_swm_mod.F90:155-201)
    const T sq = sqrt(ge);
    const T it = sq * ut + T(0.5) * uu / sq * tge;
    T* tb = S.iap_tend;
    T inext = T(0);  // iap_u of the next stage (update_state, tmcore_swm_mod.F90:210)
    switch (mode) {
      case 0:
        tb[e] = it;
        break;
      case 1:
        S.iap_acc[e] = it;
        tb[e] = it;
        inext = oldv + T(rk.a_dt) * it;
        break;
      case 2:
      case 3: {
        rip = rip + tp * it * ae;
        S.iap_acc[e] = accv + T(2) * it;
        tb[e] = it;
        inext = oldv + T(rk.a_dt) * it;
        break;
      }
      case 4: {
        rip = rip + tp * it * ae;
        T tn;
        if constexpr (kF64<T>)
          tn = (accv + it) / 6.0;
        else
          tn = (accv + it) * (1.0f / 6.0f);
        S.iap_acc[e] = tn;
        r44 = r44 + tn * tn * ae;
        tb[e] = it;
        break;
      }
    }
    if (fuse) {
      // edge preparation of the next stage from its gd and iap_u
      const CellSrc<T> C{S.gd_next, S.gdf_next, S.q_next, S.qr_next};
      prep_edge<T>(M, O, e, c1, c2, inext, gn1, gn2, C, S.gd_e_nx, S.u_nx, S.F_nx, S.Fq_nx);
    } else if (mode >= 1 && mode <= 3) {
      S.iap_next[e] = inext;
    }
  }
  if (rk.mode >= 2) {
    const T v[2] = {rip, r44};
    const int r[2] = {R_IP_E + 2 * (rk.mode - 2), R_44_E};
    block_store<T, 2>(v, P, r);
  }
}

// the single-model kernel, and the ensemble kernel (member = blockIdx.y) with
// its register budget capped so that member pointers do not halve occupancy
template <class T>
__global__ void __launch_bounds__(kMaxBlock) k_edge_flux(DevMesh M, ModelOpt O, StageIO<T> S0, RKStage rk, Partials P0) {
  edge_flux_body<T, false>(M, O, S0, rk, P0);
}
template <class T>
__global__ void __launch_bounds__(kMemberBlock, TMC_FLUX_MIN_BLOCKS) k_edge_flux_members(DevMesh M, ModelOpt O, StageIO<T> S0, RKStage rk,
                                                                    Partials P0) {
  edge_flux_body<T, true>(M, O, S0, rk, P0);
}

// new = old + (beta dt) t_new (update_state, tmcore_swm_mod.F90:203-213)
// Cells: gd and tracer mass of state(old) in place, and their FP32 shadows.
template <class T, bool kB>
__global__ void __launch_bounds__(kMaxBlock) k_final_cells(DevMesh M, ModelOpt O, StageIO<T> S0, const double* diag0) {
  const StageIO<T> S = kB ? S0.at(blockIdx.y) : S0;
  const double* diag = kB ? diag0 + (size_t)blockIdx.y * kDiagStride : diag0;
  const double bdt = diag[9];
  // all loads of the thread's kEPT cells before any store (a load after a
  // store through a possibly aliasing pointer waits a full round trip)
  const int i0 = blockIdx.x * (kEPT * blockDim.x) + threadIdx.x;
  double* gd = const_cast<double*>(S.gd_old);
  double g[kEPT];
#pragma unroll
  for (int j = 0; j < kEPT; ++j) {
    const int i = i0 + j * blockDim.x;
    g[j] = i < M.nc ? gd[i] + bdt * S.gd_acc[i] : 0.0;
  }
#pragma unroll
  for (int j = 0; j < kEPT; ++j) {
    const int i = i0 + j * blockDim.x;
    if (i >= M.nc) continue;
    gd[i] = g[j];
    if constexpr (!kF64<T>) const_cast<float*>(S.gdf_in)[i] = (float)g[j];
  }
  T* qq = const_cast<T*>(S.q_old);
  for (int q = 0; q < O.n_tracers; ++q) {
    T qn[kEPT];
#pragma unroll
    for (int j = 0; j < kEPT; ++j) {
      const int i = i0 + j * blockDim.x;
      const size_t qi = (size_t)q * M.nc + i;
      qn[j] = i < M.nc ? qq[qi] + T(bdt) * S.q_acc[qi] : T(0);
    }
#pragma unroll
    for (int j = 0; j < kEPT; ++j) {
      const int i = i0 + j * blockDim.x;
      if (i >= M.nc) continue;
      const size_t qi = (size_t)q * M.nc + i;
      qq[qi] = qn[j];
      if constexpr (!kF64<T>) const_cast<float*>(S.qr_in)[qi] = qn[j] / (float)g[j];
    }
  }
}

// Edges: iap_u of state(old) in place, then the edge preparation of the next
// step's first stage (into S.gd_e/u/F/Fq) and the edge part of the total
// energy of the new state (tmcore_swm_mod.F90:229) for the next step's
// invariants.
template <class T, bool kB>
__global__ void __launch_bounds__(kB ? kMemberBlock : kMaxBlock, kB ? TMC_FINAL_MIN_BLOCKS : TMC_FINAL_SINGLE_MIN_BLOCKS)
    k_final_edges(DevMesh M, ModelOpt O, StageIO<T> S0, const double* diag0, Partials P0) {
  const StageIO<T> S = kB ? S0.at(blockIdx.y) : S0;
  const Partials P = kB ? P0.at(blockIdx.y) : P0;
  const double* diag = kB ? diag0 + (size_t)blockIdx.y * kDiagStride : diag0;
  const double bdt = diag[9];
  double en = 0.0;
  const CellSrc<T> C{S.gd_old, S.gdf_in, S.q_old, S.qr_in};
  // loads of all kEPT edges first (see k_final_cells)
  const int e0 = blockIdx.x * (kEPT * blockDim.x) + threadIdx.x;
  T* iap = const_cast<T*>(S.iap_old);
  int c1[kEPT], c2[kEPT];
  T ia[kEPT], g1[kEPT], g2[kEPT], ae[kEPT];
#pragma unroll
  for (int j = 0; j < kEPT; ++j) {
    const int e = e0 + j * blockDim.x;
    const bool in = e < M.ne;
    c1[j] = in ? M.cellsOnEdge[e] : 0;
    c2[j] = in ? M.cellsOnEdge[M.ne + e] : 0;
    ia[j] = in ? iap[e] + T(bdt) * S.iap_acc[e] : T(0);
    ae[j] = in ? met<T>(M.areaEdge, M.areaEdge_f, e) : T(0);  // for the energy, loaded before any store
  }
#pragma unroll
  for (int j = 0; j < kEPT; ++j) {
    if constexpr (kF64<T>) {
      g1[j] = S.gd_old[c1[j]];
      g2[j] = S.gd_old[c2[j]];
    } else {
      g1[j] = S.gdf_in[c1[j]];
      g2[j] = S.gdf_in[c2[j]];
    }
  }
  float eh = 0.f, el = 0.f;  // FP32 path: the thread's few terms, compensated
#pragma unroll
  for (int j = 0; j < kEPT; ++j) {
    const int e = e0 + j * blockDim.x;
    if (e >= M.ne) continue;
    iap[e] = ia[j];
    prep_edge<T>(M, O, e, c1[j], c2[j], ia[j], g1[j], g2[j], C, S.gd_e, S.u, S.F, S.Fq);
    // energy_term (tmcore_swm_mod.F90:229) with areaEdge already loaded
    if constexpr (kF64<T>)
      en = en + ia[j] * ia[j] * ae[j];
    else
      two_sum_acc(eh, el, ia[j] * ia[j] * ae[j]);
  }
  const int r[1] = {R_EN_E};
  if constexpr (kF64<T>) {
    const double v[1] = {en};
    block_store<double, 1>(v, P, r);
  } else {
    const float h[1] = {eh}, l[1] = {el};
    block_store_ff<1>(h, l, P, r);
  }
}

template <class T>
__global__ void k_gather(int n, const double* src, const int32_t* n2o, T* dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = T(src[n2o[i]]);
}
template <class T>
__global__ void k_scatter(int n, const T* src, const int32_t* n2o, double* dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[n2o[i]] = (double)src[i];
}
template <class T>
__global__ void k_iap_from_u(int ne, const double* gd_e, const double* u, T* iap) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < ne) iap[i] = T(sqrt(gd_e[i]) * u[i]);
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
inline int nblk(int n, int bs) { return (n + bs - 1) / bs; }


template <class T>
void launch_edge_prep(const DevMesh& M, const ModelOpt& O, const StageIO<T>& S, Partials P, bool diag, int bs,
                      cudaStream_t st) {
  TMC_LAUNCH(k_edge_prep, grid_for(M.ne, bs), M, O, S, P, diag ? 1 : 0);
}
// The second-order tracer terms of the FP32 cell pass (the mass-weighted
// form d(gd q)/dt = div_operator(F q_edge), q_edge the mean of the two
// cells' mixing ratios): the tendency of each tracer of one cell ...
template <int NTR, int NQ>
__device__ __forceinline__ void tracer_tend_f(const float (&ns)[kME], const float (&Fv)[kME], const float (&dv)[kME],
                                              const float (&qs)[NQ], const float (&qn)[NQ][kME], float invAf,
                                              float (&tq)[NQ]) {
#pragma unroll
  for (int j = 0; j < NTR; ++j) {
    float sq = 0.f;
#pragma unroll
    for (int i = 0; i < kME; ++i) sq += ns[i] * Fv[i] * (0.5f * (qs[j] + qn[j][i])) * dv[i];
    tq[j] = -sq * invAf;
  }
}
// ... and its RK update (mode as RKStage; gnf the stage's next gd in FP32).
// The next stage reads the mixing ratio only (and q_old, q_acc), so the
// stage's tracer mass itself is not stored.
template <int NTR, int NQ>
__device__ __forceinline__ void tracer_update_f(const StageIO<float>& S, size_t nc, int c, int mode, float adt,
                                                const float (&tq)[NQ], const float (&qo)[NQ], const float (&qa)[NQ],
                                                float gnf) {
#pragma unroll
  for (int j = 0; j < NTR; ++j) {
    const size_t qi = (size_t)j * nc + c;
    if (mode == 1) {
      S.q_acc[qi] = tq[j];
    } else if (mode <= 3) {
      S.q_acc[qi] = qa[j] + 2.f * tq[j];
    } else {
      S.q_acc[qi] = (qa[j] + tq[j]) * (1.0f / 6.0f);
    }
    if (mode <= 3) {
      const float qnext = qo[j] + adt * tq[j];
      S.qr_next[qi] = qnext / gnf;
    }
  }
}

// FP32 cell pass of the CRK4 stages (modes 1-4) with NTR second-order
// tracers: every load is issued before the first store, in two waves
// (indices and the cell's own values, then the gathers of the edges' u, F,
// dvEdge, areaEdge and of the neighbours' tracer mixing ratios), so one cell
// costs two memory round trips.  Same arithmetic as the FP32 branch of k_cell.
template <int NTR, bool kB>
__device__ __forceinline__ void cell_fast_body(const DevMesh& M, const StageIO<float>& S0, RKStage rk,
                                               const Partials& P0, int diag) {
  const StageIO<float> S = kB ? S0.at(blockIdx.y) : S0;
  const Partials P = kB ? P0.at(blockIdx.y) : P0;
  constexpr int NQ = NTR > 0 ? NTR : 1;
  float rip = 0.f, r44 = 0.f;
  double mass = 0.0;
  float eh = 0.f, el = 0.f;
  const int mode = rk.mode;
  TMC_FOR_EPT(c, M.nc) {
    int ei[kME], ci[kME];
    float ns[kME];
#pragma unroll
    for (int i = 0; i < kME; ++i) {
      ei[i] = M.edgesOnCell[(size_t)i * M.nc + c];
      ns[i] = (float)M.nSign[(size_t)i * M.nc + c];
      ci[i] = NTR > 0 ? M.cellsOnCell[(size_t)i * M.nc + c] : 0;
    }
    const double gold = (mode <= 3) ? S.gd_old[c] : 0.0;
    const double gacc = (mode >= 2) ? S.gd_acc[c] : 0.0;
    const float tprev = (mode >= 2) ? S.tendf[c] : 0.f;
    const float gdf = S.gdf_in[c], ghf = S.ghsf[c];
    const double invA = M.invAreaCell[c];
    const float invAf = M.invAreaCell_f[c];
    const float Af = (mode >= 2) ? M.areaCell_f[c] : 0.f;
    float qs[NQ], qo[NQ], qa[NQ];
#pragma unroll
    for (int j = 0; j < NTR; ++j) {
      const size_t qi = (size_t)j * M.nc + c;
      qs[j] = S.qr_in[qi];
      qo[j] = (mode <= 3) ? S.q_old[qi] : 0.f;
      qa[j] = (mode >= 2) ? S.q_acc[qi] : 0.f;
    }
    double gdin = 0.0, Ad = 0.0;
    float Afd = 0.f;
    if (diag) {
      gdin = S.gd_in[c];
      Ad = M.areaCell[c];
      Afd = M.areaCell_f[c];
    }
    float uu[kME], Fv[kME], dv[kME], ae[kME], qn[NQ][kME];
#pragma unroll
    for (int i = 0; i < kME; ++i) {
      uu[i] = S.u[ei[i]];
      Fv[i] = S.F[ei[i]];
      dv[i] = M.dvEdge_f[ei[i]];
      ae[i] = M.areaEdge_f[ei[i]];
    }
#pragma unroll
    for (int j = 0; j < NTR; ++j)
#pragma unroll
      for (int i = 0; i < kME; ++i) qn[j][i] = S.qr_in[(size_t)j * M.nc + ci[i]];
    // divergence of the mass flux (two-sum), kinetic energy, E
    float hi = 0.f, lo = 0.f, k = 0.f;
#pragma unroll
    for (int i = 0; i < kME; ++i) {
      two_sum_acc(hi, lo, __fmul_rn(__fmul_rn(ns[i], Fv[i]), dv[i]));
      k += fabsf(ns[i]) * uu[i] * uu[i] * ae[i];
    }
    const double t = -((double)hi + (double)lo) * invA;
    const float tT = (float)t;
    S.E[c] = k * 0.25f * invAf + gdf + ghf;
    float tq[NQ];
    tracer_tend_f<NTR, NQ>(ns, Fv, dv, qs, qn, invAf, tq);
    double gnext = 0.0;
    switch (mode) {
      case 1:
        S.gd_acc[c] = t;
        S.tendf[c] = tT;
        gnext = gold + rk.a_dt * t;
        break;
      case 2:
      case 3:
        rip += tprev * tT * Af;
        S.gd_acc[c] = gacc + 2.0 * t;
        S.tendf[c] = tT;
        gnext = gold + rk.a_dt * t;
        break;
      default: {
        rip += tprev * tT * Af;
        const double tn = (gacc + t) * (1.0 / 6.0);
        S.gd_acc[c] = tn;
        const float tnf = (float)tn;
        r44 += tnf * tnf * Af;
        S.tendf[c] = tT;
      }
    }
    const float gnf = (float)gnext;
    if (mode <= 3) {
      S.gd_next[c] = gnext;
      S.gdf_next[c] = gnf;
    }
    tracer_update_f<NTR, NQ>(S, M.nc, c, mode, (float)rk.a_dt, tq, qo, qa, gnf);
    if (diag) {
      // total mass from the FP64 gd; the cell part of the total energy
      // (gd^2 + 2 gd ghs) areaCell (tmcore_swm_mod.F90:215-231) from FP32
      // terms with a compensated sum (an FP64 term would cost four FP64
      // operations per cell at 1/64 of the FP32 rate)
      mass = mass + gdin * Ad;
      two_sum_acc(eh, el, gdf * (gdf + 2.f * ghf) * Afd);
    }
  }
  if (mode >= 2) {
    const float v[2] = {rip, r44};
    const int r[2] = {R_IP_C + 2 * (mode - 2), R_44_C};
    block_store<float, 2>(v, P, r);
  }
  if (diag) {
    const double v[2] = {mass, (double)eh + (double)el};
    const int r[2] = {R_MASS, R_EN_C};
    block_store<double, 2>(v, P, r);
  }
}

template <int NTR>
__global__ void __launch_bounds__(kCellBlock, TMC_CELL_SINGLE_MIN_BLOCKS) k_cell_fast(DevMesh M, StageIO<float> S0, RKStage rk, Partials P0,
                                                         int diag) {
  cell_fast_body<NTR, false>(M, S0, rk, P0, diag);
}
// The tracer terms of the FP32 cell pass alone, for a stage whose cell pass
// ran tracer-free (k_cell_fast<0>): the same loads and the same arithmetic
// (tracer_tend_f, tracer_update_f) as k_cell_fast<NTR>, with the stage's next
// gd in FP32 read back from S.gdf_next.  Single member.
template <int NTR>
__global__ void __launch_bounds__(kCellBlock) k_tracers_fast(DevMesh M, StageIO<float> S, RKStage rk) {
  const int mode = rk.mode;
  TMC_FOR_EPT(c, M.nc) {
    int ei[kME], ci[kME];
    float ns[kME];
#pragma unroll
    for (int i = 0; i < kME; ++i) {
      ei[i] = M.edgesOnCell[(size_t)i * M.nc + c];
      ns[i] = (float)M.nSign[(size_t)i * M.nc + c];
      ci[i] = M.cellsOnCell[(size_t)i * M.nc + c];
    }
    const float invAf = M.invAreaCell_f[c];
    const float gnf = (mode <= 3) ? S.gdf_next[c] : 0.f;
    float qs[NTR], qo[NTR], qa[NTR];
#pragma unroll
    for (int j = 0; j < NTR; ++j) {
      const size_t qi = (size_t)j * M.nc + c;
      qs[j] = S.qr_in[qi];
      qo[j] = (mode <= 3) ? S.q_old[qi] : 0.f;
      qa[j] = (mode >= 2) ? S.q_acc[qi] : 0.f;
    }
    float Fv[kME], dv[kME], qn[NTR][kME];
#pragma unroll
    for (int i = 0; i < kME; ++i) {
      Fv[i] = S.F[ei[i]];
      dv[i] = M.dvEdge_f[ei[i]];
    }
#pragma unroll
    for (int j = 0; j < NTR; ++j)
#pragma unroll
      for (int i = 0; i < kME; ++i) qn[j][i] = S.qr_in[(size_t)j * M.nc + ci[i]];
    float tq[NTR];
    tracer_tend_f<NTR, NTR>(ns, Fv, dv, qs, qn, invAf, tq);
    tracer_update_f<NTR, NTR>(S, M.nc, c, mode, (float)rk.a_dt, tq, qo, qa, gnf);
  }
}

template <int NTR>
__global__ void __launch_bounds__(kMemberBlock, NTR == 0 ? TMC_CELL_MIN_BLOCKS : 3) k_cell_fast_members(DevMesh M, StageIO<float> S0, RKStage rk,
                                                                    Partials P0, int diag) {
  cell_fast_body<NTR, true>(M, S0, rk, P0, diag);
}

template <class T>
void launch_cell(const DevMesh& M, const ModelOpt& O, const StageIO<T>& S, RKStage rk, Partials P, bool diag, int bs,
                 cudaStream_t st) {
  if constexpr (!kF64<T>) {
    const bool fast = rk.mode >= 1 && rk.mode <= 4 && (O.n_tracers == 0 || O.tr_order == 2);
    if (fast) {
      const int g = grid_for(M.nc, bs), dg = diag ? 1 : 0;
      switch (O.n_tracers) {
        case 0:
          if (S.members > 1)
            k_cell_fast_members<0><<<dim3(g, nmem(S)), bs, 0, st>>>(M, S, rk, P, dg);
          else
            k_cell_fast<0><<<g, bs, 0, st>>>(M, S, rk, P, dg);
          return;
        case 1:
          if (S.members > 1)
            k_cell_fast_members<1><<<dim3(g, nmem(S)), bs, 0, st>>>(M, S, rk, P, dg);
          else
            k_cell_fast<1><<<g, bs, 0, st>>>(M, S, rk, P, dg);
          return;
        case 2:
          if (S.members > 1)
            k_cell_fast_members<2><<<dim3(g, nmem(S)), bs, 0, st>>>(M, S, rk, P, dg);
          else
            k_cell_fast<2><<<g, bs, 0, st>>>(M, S, rk, P, dg);
          return;
        case 4:
          if (S.members > 1)
            k_cell_fast_members<4><<<dim3(g, nmem(S)), bs, 0, st>>>(M, S, rk, P, dg);
          else
            k_cell_fast<4><<<g, bs, 0, st>>>(M, S, rk, P, dg);
          return;
        default: break;
      }
    }
  }
  TMC_LAUNCH(k_cell, grid_for(M.nc, bs), M, O, S, rk, P, diag ? 1 : 0);
}
template <class T>
void launch_tracers_fast(const DevMesh& M, const ModelOpt& O, const StageIO<T>& S, RKStage rk, int bs,
                         cudaStream_t st) {
  if constexpr (!kF64<T>) {
    const int g = grid_for(M.nc, bs);
    switch (O.n_tracers) {
      case 1: k_tracers_fast<1><<<g, bs, 0, st>>>(M, S, rk); return;
      case 2: k_tracers_fast<2><<<g, bs, 0, st>>>(M, S, rk); return;
      case 4: k_tracers_fast<4><<<g, bs, 0, st>>>(M, S, rk); return;
      default: return;
    }
  }
}
template <class T>
void launch_vertex(const DevMesh& M, const ModelOpt& O, const StageIO<T>& S, Partials P, bool diag, int bs,
                   cudaStream_t st) {
  TMC_LAUNCH(k_vertex, grid_for(M.nv, bs), M, O, S, P, diag ? 1 : 0);
}
template <class T>
void launch_edge_pv(const DevMesh& M, const ModelOpt& O, const StageIO<T>& S, int bs, cudaStream_t st) {
  if ((O.pv_scheme == 1 && O.apvm_weight != 0.0) || O.pv_scheme == 2 || O.need_pv_c)
    k_v2c<T><<<dim3(grid_for(M.nc, bs), nmem(S)), bs, 0, st>>>(M, S.pv_v, S.pv_c, S.msv, S.msc);
  if constexpr (!kF64<T>) {
    if (O.pv_scheme == 3 && (O.interp_pv_order == 3 || O.interp_pv_order == 4) && M.vert2_iw) {
      const int b = bs < 256 ? bs : 256;  // compiled for at most 256 threads per block
      const dim3 g(nblk(M.ne, b), nmem(S));
      if (S.members > 1)
        k_edge_pv_up32<true><<<g, b, 0, st>>>(M, O, S);
      else
        k_edge_pv_up32<false><<<g, b, 0, st>>>(M, O, S);
      return;
    }
  }
  TMC_LAUNCH(k_edge_pv, grid_for(M.ne, bs), M, O, S);
}
template <class T>
void launch_edge_flux(const DevMesh& M, const ModelOpt& O, const StageIO<T>& S, RKStage rk, Partials P, int bs,
                      cudaStream_t st) {
  if constexpr (!kF64<T>) {
    if (S.members > 1) {
      k_edge_flux_members<T><<<dim3(grid_for(M.ne, bs), nmem(S)), bs, 0, st>>>(M, O, S, rk, P);
      return;
    }
  }
  k_edge_flux<T><<<grid_for(M.ne, bs), bs, 0, st>>>(M, O, S, rk, P);
}
template <class T>
void launch_final_update(const DevMesh& M, const ModelOpt& O, const StageIO<T>& S, const double* diag, Partials P,
                         int bs, cudaStream_t st) {
  TMC_LAUNCH(k_final_cells, grid_for(M.nc, bs), M, O, S, diag);
  TMC_LAUNCH(k_final_edges, grid_for(M.ne, bs), M, O, S, diag, P);
}
template <class T>
void launch_gather(int n, const double* src, const int32_t* n2o, T* dst, cudaStream_t st) {
  k_gather<T><<<nblk(n, 256), 256, 0, st>>>(n, src, n2o, dst);
}
template <class T>
void launch_scatter(int n, const T* src, const int32_t* n2o, double* dst, cudaStream_t st) {
  k_scatter<T><<<nblk(n, 256), 256, 0, st>>>(n, src, n2o, dst);
}
template <class T>
void launch_iap_from_u(int ne, const double* gd_e, const double* u, T* iap, cudaStream_t st) {
  k_iap_from_u<T><<<nblk(ne, 256), 256, 0, st>>>(ne, gd_e, u, iap);
}

// mpas_reconstruct_1d (mpas_vector_reconstruction.F90:207-261), reference order
template <class T>
__global__ void k_reconstruct(DevMesh M, const T* u, double* uX, double* uY, double* uZ, double* zon, double* mer) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= M.nc) return;
  double x = 0.0, y = 0.0, z = 0.0;
  for (int i = 0; i < M.nEdgesOnCell[c]; ++i) {
    const double ue = (double)u[M.edgesOnCell[(size_t)i * M.nc + c]];
    x = x + M.recon[((size_t)0 * M.me + i) * M.nc + c] * ue;
    y = y + M.recon[((size_t)1 * M.me + i) * M.nc + c] * ue;
    z = z + M.recon[((size_t)2 * M.me + i) * M.nc + c] * ue;
  }
  if (uX) uX[c] = x;
  if (uY) uY[c] = y;
  if (uZ) uZ[c] = z;
  const double clat = M.cell_trig[c], slat = M.cell_trig[(size_t)M.nc + c];
  const double clon = M.cell_trig[(size_t)2 * M.nc + c], slon = M.cell_trig[(size_t)3 * M.nc + c];
  if (zon) zon[c] = -x * slon + y * clon;
  if (mer) mer[c] = -(x * clon + y * slon) * slat + z * clat;
}

template <class T>
__global__ void k_to_f64(size_t n, const T* src, double* dst) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (double)src[i];
}

template <class T>
void launch_reconstruct(const DevMesh& M, const T* u, double* uX, double* uY, double* uZ, double* zonal,
                        double* meridional, cudaStream_t st) {
  k_reconstruct<T><<<nblk(M.nc, 256), 256, 0, st>>>(M, u, uX, uY, uZ, zonal, meridional);
}
template <class T>
void launch_to_f64(size_t n, const T* src, double* dst, cudaStream_t st) {
  k_to_f64<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, src, dst);
}

#define TMC_INSTANTIATE(T)                                                                                        \
  template void launch_gather<T>(int, const double*, const int32_t*, T*, cudaStream_t);                          \
  template void launch_scatter<T>(int, const T*, const int32_t*, double*, cudaStream_t);                         \
  template void launch_iap_from_u<T>(int, const double*, const double*, T*, cudaStream_t);                       \
  template void launch_edge_prep<T>(const DevMesh&, const ModelOpt&, const StageIO<T>&, Partials, bool, int,     \
                                    cudaStream_t);                                                                \
  template void launch_cell<T>(const DevMesh&, const ModelOpt&, const StageIO<T>&, RKStage, Partials, bool, int, \
                               cudaStream_t);                                                                     \
  template void launch_tracers_fast<T>(const DevMesh&, const ModelOpt&, const StageIO<T>&, RKStage, int,           \
                                       cudaStream_t);                                                             \
  template void launch_vertex<T>(const DevMesh&, const ModelOpt&, const StageIO<T>&, Partials, bool, int,        \
                                 cudaStream_t);                                                                   \
  template void launch_edge_pv<T>(const DevMesh&, const ModelOpt&, const StageIO<T>&, int, cudaStream_t);        \
  template void launch_edge_flux<T>(const DevMesh&, const ModelOpt&, const StageIO<T>&, RKStage, Partials, int,  \
                                    cudaStream_t);                                                                \
  template void launch_final_update<T>(const DevMesh&, const ModelOpt&, const StageIO<T>&, const double*,         \
                                       Partials, int, cudaStream_t);                                             \
  template void launch_cons_apvm<T>(const DevMesh&, const ModelOpt&, const StageIO<T>&, Partials, double*, int,   \
                                    cudaStream_t);                                                                \
  template void launch_update<T>(const DevMesh&, int, const UpdateArgs<T>&, int, cudaStream_t);                 \
  template void launch_reconstruct<T>(const DevMesh&, const T*, double*, double*, double*, double*, double*,   \
                                      cudaStream_t);                                                            \
  template void launch_to_f64<T>(size_t, const T*, double*, cudaStream_t);                                       \
  template void launch_combine<T>(const DevMesh&, int, int, const CombineArgs<T>&, Partials, int, cudaStream_t);

}  // namespace tmc
