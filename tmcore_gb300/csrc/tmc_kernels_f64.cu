// FP64 instantiation (compiled with -fmad=false: no FMA contraction, so each
// element follows the reference's IEEE operation order), the reduction
// finaliser and the single-operator kernels used for parity.
#include "tmc_kernels_impl.cuh"

namespace tmc {

TMC_INSTANTIATE(double)

struct FinalizeArgs {
  int counts[R_COUNT];
  double totalArea, sumAreaTriangle, dt;
  int step, diag, conserve;
};

// Fixed-order reduction of the per-block partials into diag_out
// (time_scheme_mod.F90:144-150 beta; tmcore_swm_mod.F90:215-255 invariants).
__global__ void __launch_bounds__(256) k_finalize(Partials P, FinalizeArgs a, double* out) {
  __shared__ double res[R_COUNT];
  for (int r = 0; r < R_COUNT; ++r) {
    const bool want = (r <= R_44_E) ? a.step : a.diag;
    if (!want) continue;  // uniform across the block
    DD acc{0.0, 0.0};
    const double* reg = P.region(r);
    for (int i = threadIdx.x; i < a.counts[r]; i += blockDim.x) acc = dd_add(acc, DD{reg[2 * i], reg[2 * i + 1]});
    DD v[1] = {acc};
    const int rr[1] = {r};
    // reduce into a scratch slot: reuse region r's first entry after the loop
    __syncthreads();
    {
      __shared__ DD sm[8];
      const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
      DD w = warp_reduce(v[0]);
      if (lane == 0) sm[warp] = w;
      __syncthreads();
      if (warp == 0) {
        w = (lane < nw) ? sm[lane] : DD{0.0, 0.0};
        w = warp_reduce(w);
        if (lane == 0) res[r] = w.hi;
      }
      __syncthreads();
    }
    (void)rr;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (a.step) {
      double R[4];
      for (int k = 0; k < 3; ++k) R[k] = (res[R_IP_E + 2 * k] + res[R_IP_C + 2 * k]) / a.totalArea;
      R[3] = (res[R_44_E] + res[R_44_C]) / a.totalArea;
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
      out[0] = res[R_MASS];
      out[1] = res[R_EN_E] + res[R_EN_C];
      out[2] = res[R_PE];
      out[3] = res[R_AV] / a.sumAreaTriangle;
    }
  }
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
  k_finalize<<<1, 256, 0, st>>>(P, a, diag_out);
}

// ---------------------------------------------------------------------------
// single operators (operators_mod.F90), FP64, reference expression order
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kMaxBlock) k_op(int op, DevMesh M, const double* a, const double* b,
                                                  const double* c, double* out, int order, double coef2,
                                                  double coef4) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  switch (op) {
    case OP_DIV:
      if (i < M.nc) {
        double s = 0.0;
        for (int k = 0; k < M.nEdgesOnCell[i]; ++k) {
          int e = M.edgesOnCell[(size_t)k * M.nc + i];
          s = s + (double)M.nSign[(size_t)k * M.nc + i] * a[e] * M.dvEdge[e];
        }
        out[i] = (-s) / M.areaCell[i];
      }
      break;
    case OP_CURL:
      if (i < M.nv) {
        double s = 0.0;
        for (int k = 0; k < 3; ++k) {
          int e = M.edgesOnVertex[(size_t)k * M.nv + i];
          s = s + (double)M.tSign[(size_t)k * M.nv + i] * a[e] * M.dcEdge[e];
        }
        out[i] = (-s) / M.areaTriangle[i];
      }
      break;
    case OP_C2E:
      if (i < M.ne) out[i] = 0.5 * (a[M.cellsOnEdge[i]] + a[M.cellsOnEdge[M.ne + i]]);
      break;
    case OP_C2V:
      if (i < M.nv) {
        double s = 0.0;
        for (int k = 0; k < 3; ++k) s = s + a[M.cellsOnVertex[(size_t)k * M.nv + i]] * M.kite[(size_t)k * M.nv + i];
        out[i] = s / M.areaTriangle[i];
      }
      break;
    case OP_V2C:
      if (i < M.nc) {
        double s = 0.0;
        for (int k = M.v2c_start[i]; k < M.v2c_start[i + 1]; ++k)
          s = s + a[M.v2c_vertex[k]] * M.v2c_kite[k] / M.areaCell[i];
        out[i] = s;
      }
      break;
    case OP_V2E:
      if (i < M.ne) out[i] = 0.5 * (a[M.verticesOnEdge[i]] + a[M.verticesOnEdge[M.ne + i]]);
      break;
    case OP_KE:
      if (i < M.nc) {
        double s = 0.0;
        for (int k = 0; k < M.nEdgesOnCell[i]; ++k) {
          int e = M.edgesOnCell[(size_t)k * M.nc + i];
          s = s + a[e] * a[e] * M.areaEdge[e];
        }
        out[i] = (s * 0.25) / M.areaCell[i];
      }
      break;
    case OP_TWIND:
      if (i < M.ne) {
        double s = 0.0;
        for (int k = 0; k < M.nEdgesOnEdge[i]; ++k)
          s = s + a[M.edgesOnEdge[(size_t)k * M.ne + i]] * M.weightsOnEdge[(size_t)k * M.ne + i];
        out[i] = s;
      }
      break;
    case OP_TVF:
      if (i < M.ne) {
        double s = 0.0;
        for (int k = 0; k < M.nEdgesOnEdge[i]; ++k) {
          int ep = M.edgesOnEdge[(size_t)k * M.ne + i];
          s = s + M.weightsOnEdge[(size_t)k * M.ne + i] * a[ep] * b[ep] * 0.5 * (c[i] + c[ep]);
        }
        out[i] = s;
      }
      break;
    case OP_UPWIND:
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
