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
  int step, diag, conserve;
};

// One block per partial region: a fixed-order double-double reduction of the
// region's per-block partials; the last block to finish (atomic counter, no
// waiting) combines the region sums into beta and the invariants
// (time_scheme_mod.F90:144-150; tmcore_swm_mod.F90:215-255) and re-arms the
// counter.
__global__ void __launch_bounds__(256) k_finalize(Partials P, FinalizeArgs a, double* out, double* res,
                                                  unsigned int* counter) {
  const int r = blockIdx.x;
  const bool want = (r <= R_44_E) ? a.step : a.diag;
  if (want) {
    // per-thread FP64 sums over a strided subset of the block partials, then
    // double-double across lanes and warps
    double hi = 0.0, lo = 0.0;
    const double* reg = P.region(r);
    for (int i = threadIdx.x; i < a.counts[r]; i += blockDim.x) {
      hi = __dadd_rn(hi, reg[2 * i]);
      lo = __dadd_rn(lo, reg[2 * i + 1]);
    }
    __shared__ DD sm[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    DD w = warp_reduce_dd(DD{hi, lo});
    if (lane == 0) sm[warp] = w;
    __syncthreads();
    if (warp == 0) {
      w = (lane < nw) ? sm[lane] : DD{0.0, 0.0};
      w = warp_reduce_dd(w);
      if (lane == 0) res[r] = w.hi + w.lo;
    }
  }
  __shared__ bool last;
  if (threadIdx.x == 0) {
    __threadfence();
    last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  volatile const double* rv = res;
  if (a.step) {
    double R[4];
    for (int k = 0; k < 3; ++k) R[k] = (rv[R_IP_E + 2 * k] + rv[R_IP_C + 2 * k]) / a.totalArea;
    R[3] = (rv[R_44_E] + rv[R_44_C]) / a.totalArea;
    double beta = 1.0;
    if (a.conserve) beta = (R[0] + R[1] + R[2]) / (3.0 * R[3]);
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
                     bool step, bool diag, bool conserve, double* diag_out, cudaStream_t st) {
  FinalizeArgs a;
  for (int r = 0; r < R_COUNT; ++r) a.counts[r] = counts_host[r];
  a.totalArea = totalArea;
  a.sumAreaTriangle = sumAreaTriangle;
  a.dt = dt;
  a.step = step ? 1 : 0;
  a.diag = diag ? 1 : 0;
  a.conserve = conserve ? 1 : 0;
  // scratch after the kDiagLen outputs: R_COUNT region sums, then the counter
  double* res = diag_out + kDiagLen;
  unsigned int* counter = reinterpret_cast<unsigned int*>(diag_out + kDiagLen + R_COUNT);
  k_finalize<<<R_COUNT, 256, 0, st>>>(P, a, diag_out, res, counter);
}

__global__ void k_shadows(int nc, int ntr, const double* gd, const float* q, float* gdf, float* qr) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const float g = (float)gd[c];
  gdf[c] = g;
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
