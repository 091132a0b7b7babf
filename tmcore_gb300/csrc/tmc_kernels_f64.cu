// FP64 instantiation (compiled with -fmad=false: no FMA contraction, so each
// element follows the reference's IEEE operation order), the reduction
// finaliser, the FP32 shadow helpers and the single-operator kernels used for
// parity.
#include "tmc_kernels_impl.cuh"

namespace tmc {

TMC_INSTANTIATE(double)

struct FinalizeArgs {
  int counts[R_COUNT];
  double totalArea, sumAreaTriangle, dt;
  int step, diag, conserve, scheme;
  int split;  // blocks per region (1..kFinSplit)
};

// Fixed-order double-double sum of `count` per-block partials (hi, lo pairs),
// by one block; lane 0 of warp 0 returns it.
__device__ DD region_sum_pair(const double* reg, int count) {
  double hi = 0.0, lo = 0.0;
  for (int i = threadIdx.x; i < count; i += blockDim.x) {
    hi = __dadd_rn(hi, reg[2 * i]);
    lo = __dadd_rn(lo, reg[2 * i + 1]);
  }
  __shared__ DD sm[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  DD w = warp_reduce_dd(DD{hi, lo});
  if (lane == 0) sm[warp] = w;
  __syncthreads();
  if (warp == 0) {
    w = (lane < nw) ? sm[lane] : DD{0.0, 0.0};
    w = warp_reduce_dd(w);
  }
  return w;
}
__device__ double region_sum_dd(const double* reg, int count) {
  const DD w = region_sum_pair(reg, count);
  return w.hi + w.lo;
}

// a.split blocks per partial region (kFinSplit for one model, fewer for a
// batch of members), each a fixed-order double-double reduction of a contiguous
// 1/a.split of the region's per-block partials into P.fin; the last block to
// finish (atomic counter, no waiting) combines each region's a.split sums in
// order (one thread per region), then the
// region sums into beta and the invariants (time_scheme_mod.F90:144-150;
// tmcore_swm_mod.F90:215-255), and re-arms the counter.  With one block per
// region the widest region (15,360 partials at level 9) cost ~15,000 cycles
// of one SM's 2-lane FP64 pipe, and the launch 28 us.
__global__ void __launch_bounds__(256) k_finalize(Partials P0, FinalizeArgs a, double* out0, double* res0,
                                                  unsigned int* counter0) {
  // one member per blockIdx.y: its partials, outputs, region sums and counter
  const Partials P = P0.at(blockIdx.y);
  double* out = out0 + (size_t)blockIdx.y * kDiagStride;
  double* res = res0 + (size_t)blockIdx.y * kDiagStride;
  unsigned int* counter = reinterpret_cast<unsigned int*>(reinterpret_cast<double*>(counter0) +
                                                          (size_t)blockIdx.y * kDiagStride);
  const int r = blockIdx.x / a.split, part = blockIdx.x - r * a.split;
  const bool want = (r <= R_44_E) ? a.step : a.diag;
  if (want) {
    const int count = a.counts[r], chunk = (count + a.split - 1) / a.split;
    const int i0 = min(count, part * chunk), i1 = min(count, i0 + chunk);
    const DD v = region_sum_pair(P.region(r) + 2 * (size_t)i0, i1 - i0);
    if (threadIdx.x == 0) {
      P.fin[2 * (r * kFinSplit + part)] = v.hi;
      P.fin[2 * (r * kFinSplit + part) + 1] = v.lo;
    }
  }
  __shared__ bool last;
  if (threadIdx.x == 0) {
    __threadfence();
    last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  __shared__ double rs[kFinalizeRegions];
  if (threadIdx.x < kFinalizeRegions) {
    const int q = threadIdx.x;
    DD acc{0.0, 0.0};
    if ((q <= R_44_E) ? a.step : a.diag)
      for (int k = 0; k < a.split; ++k)  // L2 loads: the other blocks wrote them
        acc = dd_add(acc, DD{__ldcg(P.fin + 2 * (q * kFinSplit + k)), __ldcg(P.fin + 2 * (q * kFinSplit + k) + 1)});
    rs[q] = acc.hi + acc.lo;
    res[q] = rs[q];
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  const double* rv = rs;
  if (a.step) {
    double R[4];
    for (int k = 0; k < 3; ++k) R[k] = (rv[R_IP_E + 2 * k] + rv[R_IP_C + 2 * k]) / a.totalArea;
    R[3] = (rv[R_44_E] + rv[R_44_C]) / a.totalArea;
    double beta = 1.0;
    if (a.conserve) {
      if (a.scheme == 1)  // CRK3: R[0] = <t1,t2>, R[1] = <t1,t3>, R[2] = <t2,t3>
        beta = R[3] != 0.0 ? (2.0 * R[0] - R[1] + 2.0 * R[2]) / (3.0 * R[3]) : 1.0;
      else if (a.scheme == 3)  // PC2: R[0] = <t_old,t_new>, R[3] = <t_new,t_new>
        beta = (R[0] != 0.0 && R[3] != 0.0) ? R[0] / R[3] : 1.0;
      else  // CRK4
        beta = R[3] != 0.0 ? (R[0] + R[1] + R[2]) / (3.0 * R[3]) : 1.0;
      // time_scheme_mod.F90:145 (CRK4) and :94-100 (CRK3) divide 0 / 0 when the
      // tendency is zero everywhere (a state at rest); beta = 1 there, as the
      // reference's PC2 has it (:178)
    }
    out[4] = beta;
    out[5] = R[0];
    out[6] = R[1];
    out[7] = R[2];
    out[8] = R[3];
    out[9] = beta * a.dt;
  }
  if (a.diag) {
    out[0] = rv[R_MASS];
    out[1] = rv[R_EN_E] + rv[R_EN_C];
    out[2] = rv[R_PE];
    out[3] = rv[R_AV] / a.sumAreaTriangle;
  }
  *counter = 0u;
}

void launch_finalize(Partials P, const int* counts_host, double totalArea, double sumAreaTriangle, double dt,
                     bool step, bool diag, bool conserve, double* diag_out, cudaStream_t st, int scheme,
                     int members) {
  FinalizeArgs a;
  for (int r = 0; r < R_COUNT; ++r) a.counts[r] = counts_host[r];
  a.totalArea = totalArea;
  a.sumAreaTriangle = sumAreaTriangle;
  a.dt = dt;
  a.step = step ? 1 : 0;
  a.diag = diag ? 1 : 0;
  a.conserve = conserve ? 1 : 0;
  a.scheme = scheme;
  // A single model's widest region (the edge partials of level 9: 15,360)
  // would leave one block's FP64 additions on one SM's 2-lane FP64 pipe, so
  // each region is split over kFinSplit blocks.  A batch of members already
  // has a block per region and member; splitting it as much multiplies the
  // blocks' fixed cost of a double-double block reduction (512 level-6
  // members: 0.2 -> 4 ms per step), so the split shrinks with the members
  // (about kFinSplit x the regions' blocks in all).
  const int nm = members > 1 ? members : 1;
  a.split = kFinSplit / nm > 1 ? kFinSplit / nm : 1;
  // scratch after the kDiagLen outputs: R_COUNT region sums, then the counter
  double* res = diag_out + kDiagLen;
  unsigned int* counter = reinterpret_cast<unsigned int*>(diag_out + kDiagLen + R_COUNT);
  k_finalize<<<dim3(kFinalizeRegions * a.split, members > 1 ? members : 1), 256, 0, st>>>(P, a, diag_out, res,
                                                                                         counter);
}

// Conservative APVM epsilon (operators_mod.F90:349-354): one block per sum
// region R_C1..R_C3, the last block to finish computes
// eps = -(s1 - 2 s2) / (2 dt s3) into out[10] and re-arms its counter.
__global__ void __launch_bounds__(256) k_cons_eps(Partials P0, int count, double dt, double* out0, double* res0,
                                                  unsigned int* counter0) {
  const Partials P = P0.at(blockIdx.y);
  double* out = out0 + (size_t)blockIdx.y * kDiagStride;
  double* res = res0 + (size_t)blockIdx.y * kDiagStride;
  unsigned int* counter = reinterpret_cast<unsigned int*>(reinterpret_cast<double*>(counter0) +
                                                          (size_t)blockIdx.y * kDiagStride);
  const int r = R_C1 + blockIdx.x;
  const double v = region_sum_dd(P.region(r), count);
  if (threadIdx.x == 0) res[r] = v;
  __shared__ bool last;
  if (threadIdx.x == 0) {
    __threadfence();
    last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  volatile const double* rv = res;
  const double s1 = rv[R_C1], s2 = rv[R_C2], s3 = rv[R_C3];
  // eps = 0 when s3 = 0: with no wind the correction dpv is zero on every
  // edge and the reference's quotient is 0 / 0 (operators_mod.F90:349-351)
  out[10] = s3 != 0.0 ? -(s1 - s2 * 2.0) / (2.0 * dt * s3) : 0.0;
  *counter = 0u;
}

void launch_cons_eps(Partials P, int count, double dt, double* diag_out, cudaStream_t st, int members) {
  double* res = diag_out + kDiagLen;
  unsigned int* counter = reinterpret_cast<unsigned int*>(diag_out + kDiagLen + R_COUNT + 1);
  k_cons_eps<<<dim3(3, members > 1 ? members : 1), 256, 0, st>>>(P, count, dt, diag_out, res, counter);
}

// adv model spatial operator, edges: c2e + upwind correction with the sign of
// u (operators_mod.F90:93-104, :423-472), mass flux u*gd_edge
// (adv_scheme_sg11_mod.F90:42-46)
__global__ void __launch_bounds__(kMaxBlock) k_adv_edge(DevMesh M, ModelOpt O, const double* gd, const double* u,
                                                        double* gd_e, double* F) {
  TMC_FOR_EPT(e, M.ne) {
    const int c1 = M.cellsOnEdge[e], c2 = M.cellsOnEdge[M.ne + e];
    const double ue = u[e];
    double ge = 0.5 * (gd[c1] + gd[c2]);
    if (O.adv_order >= 3)
      ge = upwind_edge<double>(M.cell2, M.cell4, O.adv_order, O.cell_coef2, O.cell_coef4, M.ne, e, c1, c2, ge, ue,
                               M.dcEdge[e], [gd](int i) { return gd[i]; });
    gd_e[e] = ge;
    F[e] = ue * ge;
  }
}

// div_operator (operators_mod.F90:40-55) of the mass flux
__global__ void __launch_bounds__(kMaxBlock) k_adv_div(DevMesh M, const double* F, double* tend) {
  TMC_FOR_EPT(c, M.nc) {
    double s = 0.0;
    for (int i = 0; i < M.nEdgesOnCell[c]; ++i) {
      const int e = M.edgesOnCell[(size_t)i * M.nc + c];
      s = s + (double)M.nSign[(size_t)i * M.nc + c] * F[e] * M.dvEdge[e];
    }
    tend[c] = (-s) / M.areaCell[c];
  }
}

void launch_adv_spatial(const DevMesh& M, const ModelOpt& O, const double* gd, const double* u, double* gd_e,
                        double* F, double* tend, int bs, cudaStream_t st) {
  k_adv_edge<<<grid_for(M.ne, bs), bs, 0, st>>>(M, O, gd, u, gd_e, F);
  k_adv_div<<<grid_for(M.nc, bs), bs, 0, st>>>(M, F, tend);
}

// stream function of the prescribed wind on vertices
__global__ void k_adv_psi(int nv, int wind_case, double radius, const double* latV, const double* lonV,
                          const double* t0, double offset, const double* offset_dev, double* psi) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const double pi = 4.0 * atan(1.0);
  const double lat = latV[v], lon = lonV[v];
  if (wind_case == 1) {
    // cosine_bell_rotation_test_mod.F90:45-68 (alpha = pi/2, one revolution in 12 days)
    const double u0 = 2.0 * pi * radius / 12.0 / 86400.0, alpha = 0.5 * pi;
    const double ca = cos(alpha), sa = sin(alpha);
    psi[v] = -radius * u0 * (sin(lat) * ca - cos(lon) * cos(lat) * sa);
  } else {
    // deformation_flow_test_mod.F90:74-105 (case 4: deformation plus solid-body rotation)
    const double seconds = *t0 + (offset_dev ? *offset_dev : offset);
    const double T0 = 12.0 * 86400.0, u0 = 2.0 * pi * radius / T0;
    const double c = pi * 2.0 * seconds / T0, k = 10.0 * radius / T0, cosT = cos(pi * seconds / T0);
    const double sn = sin(lon - c), cl = cos(lat);
    const double p = k * (sn * sn) * (cl * cl) * cosT - u0 * sin(lat);
    psi[v] = p * radius;
  }
}

__global__ void k_adv_u(int ne, const int32_t* verticesOnEdge, const double* dvEdge, const double* psi, double* u) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  u[e] = -(psi[verticesOnEdge[ne + e]] - psi[verticesOnEdge[e]]) / dvEdge[e];
}

void launch_adv_wind(const DevMesh& M, int wind_case, double radius, const double* latV, const double* lonV,
                     const double* t0_dev, double offset, const double* offset_dev, double* psi, double* u,
                     cudaStream_t st) {
  k_adv_psi<<<nblk(M.nv, 256), 256, 0, st>>>(M.nv, wind_case, radius, latV, lonV, t0_dev, offset, offset_dev, psi);
  k_adv_u<<<nblk(M.ne, 256), 256, 0, st>>>(M.ne, M.verticesOnEdge, M.dvEdge, psi, u);
}

__global__ void k_adv_advance(double* elapsed, double dt) { *elapsed = *elapsed + dt; }

void launch_adv_advance(double* elapsed_dev, double dt, cudaStream_t st) {
  k_adv_advance<<<1, 1, 0, st>>>(elapsed_dev, dt);
}

// total mass (tmcore_swm_mod.F90:215-220) alone; the other invariant regions
// get zero partials so that the finaliser reports 0 for them
__global__ void __launch_bounds__(kMaxBlock) k_mass_only(DevMesh M, const double* gd, Partials P) {
  double mass = 0.0;
  TMC_FOR_EPT(c, M.nc) mass = mass + gd[c] * M.areaCell[c];
  const double v[5] = {mass, 0.0, 0.0, 0.0, 0.0};
  const int r[5] = {R_MASS, R_EN_E, R_EN_C, R_PE, R_AV};
  block_store<double, 5>(v, P, r);
}

int launch_mass_only(const DevMesh& M, const double* gd, Partials P, int bs, cudaStream_t st) {
  const int g = grid_for(M.nc, bs);
  k_mass_only<<<g, bs, 0, st>>>(M, gd, P);
  return g;
}

// h = (gd + ghs) / g (history_mod.F90:166)
__global__ void k_h_field(int nc, const double* gd, const double* ghs, double g, double* h) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < nc) h[c] = (gd[c] + ghs[c]) / g;
}

void launch_h_field(int nc, const double* gd, const double* ghs, double g, double* h, cudaStream_t st) {
  k_h_field<<<nblk(nc, 256), 256, 0, st>>>(nc, gd, ghs, g, h);
}

// gdf = FP32 gd (skipped when null), qr = q / FP32 gd
__global__ void k_shadows(int nc, int ntr, const double* gd, const float* q, float* gdf, float* qr) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const float g = (float)gd[c];
  if (gdf) gdf[c] = g;
  for (int k = 0; k < ntr; ++k) qr[(size_t)k * nc + c] = q[(size_t)k * nc + c] / g;
}

void launch_shadows(int nc, int ntr, const double* gd, const float* q, float* gdf, float* qr, cudaStream_t st) {
  k_shadows<<<nblk(nc, 256), 256, 0, st>>>(nc, ntr, gd, q, gdf, qr);
}

__global__ void k_to_f32(size_t n, const double* src, float* dst) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (float)src[i];
}

void launch_to_f32(size_t n, const double* src, float* dst, cudaStream_t st) {
  k_to_f32<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, src, dst);
}

// ---------------------------------------------------------------------------
// single operators (operators_mod.F90), FP64, reference expression order
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kMaxBlock) k_op(int op, DevMesh M, const double* a, const double* b,
                                                  const double* c, double* out, int order, double coef2,
                                                  double coef4) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  switch (op) {
    case OP_DIV:  // :40-55
      if (i < M.nc) {
        double s = 0.0;
        for (int k = 0; k < M.nEdgesOnCell[i]; ++k) {
          int e = M.edgesOnCell[(size_t)k * M.nc + i];
          s = s + (double)M.nSign[(size_t)k * M.nc + i] * a[e] * M.dvEdge[e];
        }
        out[i] = (-s) / M.areaCell[i];
      }
      break;
    case OP_CURL:  // :76-91
      if (i < M.nv) {
        double s = 0.0;
        for (int k = 0; k < 3; ++k) {
          int e = M.edgesOnVertex[(size_t)k * M.nv + i];
          s = s + (double)M.tSign[(size_t)k * M.nv + i] * a[e] * M.dcEdge[e];
        }
        out[i] = (-s) / M.areaTriangle[i];
      }
      break;
    case OP_C2E:  // :93-104
      if (i < M.ne) out[i] = 0.5 * (a[M.cellsOnEdge[i]] + a[M.cellsOnEdge[M.ne + i]]);
      break;
    case OP_C2V:  // :106-123
      if (i < M.nv) {
        double s = 0.0;
        for (int k = 0; k < 3; ++k) s = s + a[M.cellsOnVertex[(size_t)k * M.nv + i]] * M.kite[(size_t)k * M.nv + i];
        out[i] = s / M.areaTriangle[i];
      }
      break;
    case OP_V2C:  // :125-141
      if (i < M.nc) {
        double s = 0.0;
        for (int k = M.v2c_start[i]; k < M.v2c_start[i + 1]; ++k)
          s = s + a[M.v2c_vertex[k]] * M.v2c_kite[k] / M.areaCell[i];
        out[i] = s;
      }
      break;
    case OP_V2E:  // :143-156
      if (i < M.ne) out[i] = 0.5 * (a[M.verticesOnEdge[i]] + a[M.verticesOnEdge[M.ne + i]]);
      break;
    case OP_KE:  // :206-221
      if (i < M.nc) {
        double s = 0.0;
        for (int k = 0; k < M.nEdgesOnCell[i]; ++k) {
          int e = M.edgesOnCell[(size_t)k * M.nc + i];
          s = s + a[e] * a[e] * M.areaEdge[e];
        }
        out[i] = (s * 0.25) / M.areaCell[i];
      }
      break;
    case OP_TWIND:  // :223-237
      if (i < M.ne) {
        double s = 0.0;
        for (int k = 0; k < M.nEdgesOnEdge[i]; ++k)
          s = s + a[M.edgesOnEdge[(size_t)k * M.ne + i]] * M.weightsOnEdge[(size_t)k * M.ne + i];
        out[i] = s;
      }
      break;
    case OP_TVF:  // :239-260
      if (i < M.ne) {
        double s = 0.0;
        for (int k = 0; k < M.nEdgesOnEdge[i]; ++k) {
          int ep = M.edgesOnEdge[(size_t)k * M.ne + i];
          s = s + M.weightsOnEdge[(size_t)k * M.ne + i] * a[ep] * b[ep] * 0.5 * (c[i] + c[ep]);
        }
        out[i] = s;
      }
      break;
    case OP_UPWIND:  // :423-472
      if (i < M.ne) {
        const int c1 = M.cellsOnEdge[i], c2 = M.cellsOnEdge[M.ne + i];
        out[i] = upwind_edge<double>(M.cell2, M.cell4, order, coef2, coef4, M.ne, i, c1, c2, out[i], b[i],
                                     M.dcEdge[i], [a](int j) { return a[j]; });
      }
      break;
  }
}

void launch_op(int op, const DevMesh& M, const ModelOpt& O, const double* a, const double* b, const double* c,
               double* out, int order, int mono, double coef2, double coef4, int bs, cudaStream_t st) {
  (void)O;
  (void)mono;
  int n = M.ne;
  if (op == OP_DIV || op == OP_V2C || op == OP_KE) n = M.nc;
  if (op == OP_CURL || op == OP_C2V) n = M.nv;
  k_op<<<nblk(n, bs), bs, 0, st>>>(op, M, a, b, c, out, order, coef2, coef4);
}

}  // namespace tmc
