// Kernel bodies for tmc_kernels.cuh (included once per precision TU).
#pragma once

#include "tmc_kernels.cuh"

namespace tmc {

constexpr int kMaxBlock = 512;

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
__device__ __forceinline__ DD warp_reduce(DD v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    DD o;
    o.hi = __shfl_down_sync(0xffffffffu, v.hi, off);
    o.lo = __shfl_down_sync(0xffffffffu, v.lo, off);
    v = dd_add(v, o);
  }
  return v;
}
// Reduce N values over the block; thread 0 writes region[r[k]][block] for each k.
template <int N>
__device__ __forceinline__ void block_reduce_store(DD (&v)[N], const Partials& P, const int (&r)[N]) {
  __shared__ DD sm[N][kMaxBlock / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < N; ++k) {
    DD w = warp_reduce(v[k]);
    if (lane == 0) sm[k][warp] = w;
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) {
      DD w = (lane < nw) ? sm[k][lane] : DD{0.0, 0.0};
      w = warp_reduce(w);
      if (lane == 0) {
        double* reg = P.region(r[k]);
        reg[2 * blockIdx.x] = w.hi;
        reg[2 * blockIdx.x + 1] = w.lo;
      }
    }
  }
}

template <class T>
__device__ __forceinline__ T sgn1(T x) {
  return copysign(T(1), x);
}

// Upwind correction of an edge value from two-sided polynomial-fit stencils
// (operators_mod.F90:423-472 for cells, :359-412 for vertices).  `f(i)`
// returns the field at stencil point i as T; ctr0/ctr1 are the two centres.
template <class T, class F>
__device__ __forceinline__ T upwind_edge(const DStencil& S2, const DStencil& S4, int order, T coef2, T coef4, int ne,
                                         int e, int ctr0, int ctr1, T fe, T sgn_of, T dist, F f) {
  if (order == 3 || order == 4) {
    T d[2];
    const int ctr[2] = {ctr0, ctr1};
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      T fc = f(ctr[s]);
      T acc = T(0);
      int n = S2.count[(size_t)s * ne + e];
      for (int j = 0; j < n; ++j) {
        size_t k = ((size_t)j * 2 + s) * ne + e;
        acc = acc + T(S2.w[k]) * (f(S2.idx[k]) - fc);
      }
      d[s] = acc;
    }
    fe = fe - dist * dist * ((d[0] + d[1]) - sgn1(sgn_of) * coef2 * (d[1] - d[0])) / T(12);
  } else if (order == 5 || order == 6) {
    T d2[2], d4[2];
    const int ctr[2] = {ctr0, ctr1};
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      T fc = f(ctr[s]);
      T acc = T(0);
      int n = S2.count[(size_t)s * ne + e];
      for (int j = 0; j < n; ++j) {
        size_t k = ((size_t)j * 2 + s) * ne + e;
        acc = acc + T(S2.w[k]) * (f(S2.idx[k]) - fc);
      }
      d2[s] = acc;
      acc = T(0);
      n = S4.count[(size_t)s * ne + e];
      for (int j = 0; j < n; ++j) {
        size_t k = ((size_t)j * 2 + s) * ne + e;
        acc = acc + T(S4.w[k]) * (f(S4.idx[k]) - fc);
      }
      d4[s] = acc;
    }
    fe = fe - dist * dist * (d2[0] + d2[1]) / T(12) +
         (dist * dist) * (dist * dist) * ((d4[0] + d4[1]) - sgn1(sgn_of) * coef4 * (d4[1] - d4[0])) / T(60);
  }
  return fe;
}

// ---------------------------------------------------------------------------
// edge_prep
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(kMaxBlock) k_edge_prep(DevMesh M, ModelOpt O, StageIO<T> S, Partials P, int diag) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  DD en{0.0, 0.0};
  if (e < M.ne) {
    const int c1 = M.cellsOnEdge[e], c2 = M.cellsOnEdge[M.ne + e];
    const T g1 = T(S.gd_in[c1]), g2 = T(S.gd_in[c2]);
    T ge = T(0.5) * (g1 + g2);
    const T ia = S.iap_in[e];
    if (O.adv_order >= 3) {
      const double* gd = S.gd_in;
      ge = upwind_edge<T>(M.cell2, M.cell4, O.adv_order, T(O.cell_coef2), T(O.cell_coef4), M.ne, e, c1, c2, ge, ia,
                          T(M.dcEdge[e]), [gd](int i) { return T(gd[i]); });
    }
    const T sq = sqrt(ge);
    const T uu = ia / sq;
    S.gd_e[e] = ge;
    S.u[e] = uu;
    if (O.n_tracers > 0) {
      const T F = uu * ge;
      for (int k = 0; k < O.n_tracers; ++k) {
        const double* q = S.q_in + (size_t)k * M.nc;
        const double* gd = S.gd_in;
        T qe = T(0.5) * (T(q[c1]) / g1 + T(q[c2]) / g2);
        if (O.tr_order >= 3)
          qe = upwind_edge<T>(M.cell2, M.cell4, O.tr_order, T(O.tr_coef2), T(O.tr_coef4), M.ne, e, c1, c2, qe, ia,
                              T(M.dcEdge[e]), [q, gd](int i) { return T(q[i]) / T(gd[i]); });
        S.Fq[(size_t)k * M.ne + e] = F * qe;
      }
    }
    if (diag) {
      const double a = (double)ia;
      en.hi = __dmul_rn(__dmul_rn(a, a), M.areaEdge[e]);
    }
  }
  if (diag) {
    DD v[1] = {en};
    const int r[1] = {R_EN_E};
    block_reduce_store<1>(v, P, r);
  }
}

// ---------------------------------------------------------------------------
// cell: div of mass flux, kinetic energy, E, RK update of gd and tracers
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(kMaxBlock) k_cell(DevMesh M, ModelOpt O, StageIO<T> S, RKStage rk, Partials P,
                                                    int diag) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  DD rip{0.0, 0.0}, r44{0.0, 0.0}, mass{0.0, 0.0}, enc{0.0, 0.0};
  if (c < M.nc) {
    const int n = M.nEdgesOnCell[c];
    T s = T(0), k = T(0);
    for (int i = 0; i < n; ++i) {
      const int e = M.edgesOnCell[(size_t)i * M.nc + c];
      const T uu = S.u[e], ge = S.gd_e[e];
      const T F = uu * ge;
      s = s + T(M.nSign[(size_t)i * M.nc + c]) * F * T(M.dvEdge[e]);
      k = k + uu * uu * T(M.areaEdge[e]);
    }
    const double Ad = M.areaCell[c];
    const T A = T(Ad);
    const T tend = (-s) / A;
    const T ke = (k * T(0.25)) / A;
    const double gd = S.gd_in[c];
    S.E[c] = ke + T(gd) + T(S.ghs[c]);
    const double t = (double)tend;
    double* tb = S.gd_tend;
    switch (rk.mode) {
      case 0:
        tb[c] = t;
        break;
      case 1:
        S.gd_acc[c] = t;
        tb[c] = t;
        S.gd_next[c] = S.gd_old[c] + rk.a_dt * t;
        break;
      case 2:
      case 3: {
        const double tp = tb[c];
        rip.hi = __dmul_rn(__dmul_rn(tp, t), Ad);
        S.gd_acc[c] = S.gd_acc[c] + 2.0 * t;
        tb[c] = t;
        S.gd_next[c] = S.gd_old[c] + rk.a_dt * t;
        break;
      }
      case 4: {
        const double tp = tb[c];
        rip.hi = __dmul_rn(__dmul_rn(tp, t), Ad);
        const double tn = (S.gd_acc[c] + t) / 6.0;
        S.gd_acc[c] = tn;
        r44.hi = __dmul_rn(__dmul_rn(tn, tn), Ad);
        tb[c] = t;
        break;
      }
    }
    for (int q = 0; q < O.n_tracers; ++q) {
      T sq = T(0);
      for (int i = 0; i < n; ++i) {
        const int e = M.edgesOnCell[(size_t)i * M.nc + c];
        sq = sq + T(M.nSign[(size_t)i * M.nc + c]) * S.Fq[(size_t)q * M.ne + e] * T(M.dvEdge[e]);
      }
      const double tq = (double)((-sq) / A);
      const size_t qi = (size_t)q * M.nc + c;
      switch (rk.mode) {
        case 1:
          S.q_acc[qi] = tq;
          S.q_next[qi] = S.q_old[qi] + rk.a_dt * tq;
          break;
        case 2:
        case 3:
          S.q_acc[qi] = S.q_acc[qi] + 2.0 * tq;
          S.q_next[qi] = S.q_old[qi] + rk.a_dt * tq;
          break;
        case 4:
          S.q_acc[qi] = (S.q_acc[qi] + tq) / 6.0;
          break;
        default:
          S.q_acc[qi] = tq;
      }
    }
    if (diag) {
      mass.hi = __dmul_rn(gd, Ad);
      const double gh = S.ghs[c];
      enc.hi = __dmul_rn(__dadd_rn(__dmul_rn(gd, gd), __dmul_rn(__dmul_rn(2.0, gd), gh)), Ad);
    }
  }
  if (rk.mode >= 2) {
    DD v[2] = {rip, r44};
    const int r[2] = {R_IP_C + 2 * (rk.mode - 2), R_44_C};
    block_reduce_store<2>(v, P, r);
  }
  if (diag) {
    __syncthreads();
    DD v[2] = {mass, enc};
    const int r[2] = {R_MASS, R_EN_C};
    block_reduce_store<2>(v, P, r);
  }
}

// ---------------------------------------------------------------------------
// vertex: gd on vertices, vorticity, potential vorticity
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(kMaxBlock) k_vertex(DevMesh M, ModelOpt O, StageIO<T> S, Partials P, int diag) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  DD pe{0.0, 0.0}, av{0.0, 0.0};
  if (v < M.nv) {
    T gv = T(0), s = T(0);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const int c = M.cellsOnVertex[(size_t)i * M.nv + v];
      gv = gv + T(S.gd_in[c]) * T(M.kite[(size_t)i * M.nv + v]);
    }
    const double Atd = M.areaTriangle[v];
    const T At = T(Atd);
    gv = gv / At;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const int e = M.edgesOnVertex[(size_t)i * M.nv + v];
      s = s + T(M.tSign[(size_t)i * M.nv + v]) * S.u[e] * T(M.dcEdge[e]);
    }
    const T vo = (-s) / At;
    const T pv = (T(M.fVertex[v]) + vo) / gv;
    S.pv_v[v] = pv;
    if (S.vor) S.vor[v] = vo;
    if (S.gd_v) S.gd_v[v] = gv;
    if (diag) {
      const double p = (double)pv;
      pe.hi = __dmul_rn(__dmul_rn((double)gv, __dmul_rn(p, p)), Atd);
      av.hi = __dmul_rn(__dadd_rn((double)vo, M.fVertex[v]), Atd);
    }
  }
  (void)O;
  if (diag) {
    DD vv[2] = {pe, av};
    const int r[2] = {R_PE, R_AV};
    block_reduce_store<2>(vv, P, r);
  }
}

// pv on cells: scalar_v2c_interp_operator as a gather (operators_mod.F90:125-141)
template <class T>
__global__ void __launch_bounds__(kMaxBlock) k_v2c(DevMesh M, const T* pv_v, T* pv_c) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= M.nc) return;
  const T A = T(M.areaCell[c]);
  T s = T(0);
  for (int k = M.v2c_start[c]; k < M.v2c_start[c + 1]; ++k) s = s + pv_v[M.v2c_vertex[k]] * T(M.v2c_kite[k]) / A;
  pv_c[c] = s;
}

// ---------------------------------------------------------------------------
// edge_pv: PV on edges (calc_pv_on_edge, operators_mod.F90:273-412)
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(kMaxBlock) k_edge_pv(DevMesh M, ModelOpt O, StageIO<T> S) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= M.ne) return;
  const int v1 = M.verticesOnEdge[e], v2 = M.verticesOnEdge[M.ne + e];
  const T p1 = S.pv_v[v1], p2 = S.pv_v[v2];
  T pe = T(0.5) * (p1 + p2);
  const bool need_v = (O.pv_scheme == 3) || (O.pv_scheme == 1 && O.apvm_weight != 0.0);
  T ve = T(0);
  if (need_v) {
    const int n = M.nEdgesOnEdge[e];
    for (int i = 0; i < n; ++i)
      ve = ve + S.u[M.edgesOnEdge[(size_t)i * M.ne + e]] * T(M.weightsOnEdge[(size_t)i * M.ne + e]);
    if (S.v_e) S.v_e[e] = ve;
  }
  if (O.pv_scheme == 1) {
    if (O.apvm_weight != 0.0) {
      const int c1 = M.cellsOnEdge[e], c2 = M.cellsOnEdge[M.ne + e];
      const T a = ve * (p2 - p1) / T(M.dvEdge[e]);
      const T b = S.u[e] * (S.pv_c[c2] - S.pv_c[c1]) / T(M.dcEdge[e]);
      pe = pe - T(O.apvm_weight * O.dt) * (a + b);
    }
  } else if (O.pv_scheme == 3) {
    const T* pv = S.pv_v;
    pe = upwind_edge<T>(M.vert2, M.vert4, O.interp_pv_order, T(O.vert_coef2), T(O.vert_coef4), M.ne, e, v1, v2, pe,
                        ve, T(M.dvEdge[e]), [pv](int i) { return pv[i]; });
  }
  S.pv_e[e] = pe;
}

// ---------------------------------------------------------------------------
// edge_flux: q.F_perp, gradient of E, iap_u tendency, RK update, inner products
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(kMaxBlock) k_edge_flux(DevMesh M, ModelOpt O, StageIO<T> S, RKStage rk, Partials P) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  DD rip{0.0, 0.0}, r44{0.0, 0.0};
  if (e < M.ne) {
    const T pe = S.pv_e[e];
    T s = T(0);
    const int n = M.nEdgesOnEdge[e];
    for (int i = 0; i < n; ++i) {
      const size_t k = (size_t)i * M.ne + e;
      const int ep = M.edgesOnEdge[k];
      s = s + T(M.weightsOnEdge[k]) * S.u[ep] * S.gd_e[ep] * T(0.5) * (pe + S.pv_e[ep]);
    }
    const int c1 = M.cellsOnEdge[e], c2 = M.cellsOnEdge[M.ne + e];
    const T dc = T(M.dcEdge[e]);
    const T dEdx = (S.E[c2] - S.E[c1]) / dc;
    const T ut = s - dEdx;
    T tge = T(0.5) * (T(S.gd_tend[c1]) + T(S.gd_tend[c2]));
    const T ia = S.iap_in[e];
    if (O.adv_order >= 3) {
      const double* gt = S.gd_tend;
      tge = upwind_edge<T>(M.cell2, M.cell4, O.adv_order, T(O.cell_coef2), T(O.cell_coef4), M.ne, e, c1, c2, tge, ia,
                           dc, [gt](int i) { return T(gt[i]); });
    }
    const T sq = sqrt(S.gd_e[e]);
    const T it = sq * ut + T(0.5) * S.u[e] / sq * tge;
    const double ae = M.areaEdge[e];
    T* tb = S.iap_tend;
    switch (rk.mode) {
      case 0:
        tb[e] = it;
        break;
      case 1:
        S.iap_acc[e] = it;
        tb[e] = it;
        S.iap_next[e] = S.iap_old[e] + T(rk.a_dt) * it;
        break;
      case 2:
      case 3: {
        const T tp = tb[e];
        rip.hi = __dmul_rn(__dmul_rn((double)tp, (double)it), ae);
        S.iap_acc[e] = S.iap_acc[e] + T(2) * it;
        tb[e] = it;
        S.iap_next[e] = S.iap_old[e] + T(rk.a_dt) * it;
        break;
      }
      case 4: {
        const T tp = tb[e];
        rip.hi = __dmul_rn(__dmul_rn((double)tp, (double)it), ae);
        const T tn = (S.iap_acc[e] + it) / T(6);
        S.iap_acc[e] = tn;
        r44.hi = __dmul_rn(__dmul_rn((double)tn, (double)tn), ae);
        tb[e] = it;
        break;
      }
    }
  }
  if (rk.mode >= 2) {
    DD v[2] = {rip, r44};
    const int r[2] = {R_IP_E + 2 * (rk.mode - 2), R_44_E};
    block_reduce_store<2>(v, P, r);
  }
}

// new = old + (beta dt) t_new (update_state, tmcore_swm_mod.F90:203-213)
template <class T>
__global__ void __launch_bounds__(kMaxBlock) k_final_update(DevMesh M, ModelOpt O, StageIO<T> S, const double* diag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const double bdt = diag[9];
  if (i < M.ne) {
    T* iap = const_cast<T*>(S.iap_old);
    iap[i] = iap[i] + T(bdt) * S.iap_acc[i];
  }
  if (i < M.nc) {
    double* gd = const_cast<double*>(S.gd_old);
    gd[i] = gd[i] + bdt * S.gd_acc[i];
    for (int q = 0; q < O.n_tracers; ++q) {
      double* qq = const_cast<double*>(S.q_old) + (size_t)q * M.nc;
      qq[i] = qq[i] + bdt * S.q_acc[(size_t)q * M.nc + i];
    }
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
  k_edge_prep<T><<<nblk(M.ne, bs), bs, 0, st>>>(M, O, S, P, diag ? 1 : 0);
}
template <class T>
void launch_cell(const DevMesh& M, const ModelOpt& O, const StageIO<T>& S, RKStage rk, Partials P, bool diag, int bs,
                 cudaStream_t st) {
  k_cell<T><<<nblk(M.nc, bs), bs, 0, st>>>(M, O, S, rk, P, diag ? 1 : 0);
}
template <class T>
void launch_vertex(const DevMesh& M, const ModelOpt& O, const StageIO<T>& S, Partials P, bool diag, int bs,
                   cudaStream_t st) {
  k_vertex<T><<<nblk(M.nv, bs), bs, 0, st>>>(M, O, S, P, diag ? 1 : 0);
}
template <class T>
void launch_edge_pv(const DevMesh& M, const ModelOpt& O, const StageIO<T>& S, int bs, cudaStream_t st) {
  if (O.pv_scheme == 1 && O.apvm_weight != 0.0) k_v2c<T><<<nblk(M.nc, bs), bs, 0, st>>>(M, S.pv_v, S.pv_c);
  k_edge_pv<T><<<nblk(M.ne, bs), bs, 0, st>>>(M, O, S);
}
template <class T>
void launch_edge_flux(const DevMesh& M, const ModelOpt& O, const StageIO<T>& S, RKStage rk, Partials P, int bs,
                      cudaStream_t st) {
  k_edge_flux<T><<<nblk(M.ne, bs), bs, 0, st>>>(M, O, S, rk, P);
}
template <class T>
void launch_final_update(const DevMesh& M, const ModelOpt& O, const StageIO<T>& S, const double* diag, int bs,
                         cudaStream_t st) {
  k_final_update<T><<<nblk(M.ne > M.nc ? M.ne : M.nc, bs), bs, 0, st>>>(M, O, S, diag);
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

#define TMC_INSTANTIATE(T)                                                                                        \
  template void launch_gather<T>(int, const double*, const int32_t*, T*, cudaStream_t);                          \
  template void launch_scatter<T>(int, const T*, const int32_t*, double*, cudaStream_t);                         \
  template void launch_iap_from_u<T>(int, const double*, const double*, T*, cudaStream_t);                       \
  template void launch_edge_prep<T>(const DevMesh&, const ModelOpt&, const StageIO<T>&, Partials, bool, int,     \
                                    cudaStream_t);                                                                \
  template void launch_cell<T>(const DevMesh&, const ModelOpt&, const StageIO<T>&, RKStage, Partials, bool, int, \
                               cudaStream_t);                                                                     \
  template void launch_vertex<T>(const DevMesh&, const ModelOpt&, const StageIO<T>&, Partials, bool, int,        \
                                 cudaStream_t);                                                                   \
  template void launch_edge_pv<T>(const DevMesh&, const ModelOpt&, const StageIO<T>&, int, cudaStream_t);        \
  template void launch_edge_flux<T>(const DevMesh&, const ModelOpt&, const StageIO<T>&, RKStage, Partials, int,  \
                                    cudaStream_t);                                                                \
  template void launch_final_update<T>(const DevMesh&, const ModelOpt&, const StageIO<T>&, const double*, int,   \
                                       cudaStream_t);

}  // namespace tmc
