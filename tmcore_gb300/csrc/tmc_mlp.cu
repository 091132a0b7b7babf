// The learned PV-on-edge closure network: tensor-core forward (tcgen05),
// training (forward and backward) on the tensor cores or on the CUDA cores
// in FP32, Adam, and its C ABI (include/tmcore_gpu.h, tmc_mlp_*).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "tmc_ensemble.cuh"
#include "tmc_kernels.cuh"
#include "tmc_mlp_tc.cuh"
#include "tmc_mlp_train_tc.cuh"
#include "tmcore_gpu.h"

using namespace tmc::mlp;
using tmc::DevMesh;
using tmc::StageIO;

namespace {

// ---------------------------------------------------------------------------
// forward on the tensor cores, features from a [rows][24] FP32 buffer
// ---------------------------------------------------------------------------
struct BufSrc {
  const float* x;
  float* y;
  long long rows;
  __device__ bool features(long long i, float (&f)[kIn]) const {
    if (i >= rows) return false;
#pragma unroll
    for (int k = 0; k < kIn; ++k) f[k] = x[i * kIn + k];
    return true;
  }
  __device__ void output(long long i, float v) const { y[i] = v; }
};

__global__ void __launch_bounds__(kTcThreads, kTcMinBlocks) k_mlp_fwd_tc(Net net, BufSrc src, long long ntiles, int* err) {
  extern __shared__ __align__(128) uint8_t smem[];
  if (!forward_tiles(net, src, ntiles, smem) && threadIdx.x % kTile == 0) atomicExch(err, 1);
}

// ---------------------------------------------------------------------------
// the closure: features of an edge of one member from the stage state
// ---------------------------------------------------------------------------
// 0 u, 1 tangential velocity, 2 gd_edge, 3 pv_edge, 4-5 pv on the two
// vertices, 6-7 pv on the two cells, 8-9 gd, 10-11 E = ke + gd + ghs,
// 12-13 ghs on the two cells, 14-15 Coriolis on the two vertices, 16 dvEdge,
// 17 dcEdge, 18-21 u on the first four edgesOnEdge, 22 pv gradient along the
// edge, 23 pv gradient across it
__device__ __forceinline__ void closure_features(const DevMesh& M, const StageIO<float>& S, int m, int e,
                                                 float (&x)[kIn]) {
  const long long oc = (long long)m * S.msc, oe = (long long)m * S.mse, ov = (long long)m * S.msv;
  const float* u = S.u + oe;
  const int c1 = M.cellsOnEdge[e], c2 = M.cellsOnEdge[M.ne + e];
  const int v1 = M.verticesOnEdge[e], v2 = M.verticesOnEdge[M.ne + e];
  float ve = 0.f;
#pragma unroll
  for (int i = 0; i < 10; ++i) {
    const size_t k = (size_t)i * M.ne + e;
    ve += u[M.edgesOnEdge[k]] * M.weightsOnEdge_f[k];  // padded entries carry weight 0
  }
  const float dv = M.dvEdge_f[e], dc = M.dcEdge_f[e];
  const float pv1 = S.pv_v[ov + v1], pv2 = S.pv_v[ov + v2];
  const float pc1 = S.pv_c[oc + c1], pc2 = S.pv_c[oc + c2];
  x[0] = u[e];
  x[1] = ve;
  x[2] = S.gd_e[oe + e];
  x[3] = S.pv_e[oe + e];
  x[4] = pv1;
  x[5] = pv2;
  x[6] = pc1;
  x[7] = pc2;
  x[8] = S.gdf_in[oc + c1];
  x[9] = S.gdf_in[oc + c2];
  x[10] = S.E[oc + c1];
  x[11] = S.E[oc + c2];
  x[12] = S.ghsf[oc + c1];
  x[13] = S.ghsf[oc + c2];
  x[14] = M.fVertex_f[v1];
  x[15] = M.fVertex_f[v2];
  x[16] = dv;
  x[17] = dc;
#pragma unroll
  for (int i = 0; i < 4; ++i) x[18 + i] = u[M.edgesOnEdge[(size_t)i * M.ne + e]];
  x[22] = (pv2 - pv1) / dv;
  x[23] = (pc2 - pc1) / dc;
}

// rows: tile-major per member (tiles_per_member tiles of 128 edges each), so
// the member and the edge of a row come from the tile index without a 64-bit
// division; rows past a member's last edge are empty
struct ClosureSrc {
  DevMesh M;
  StageIO<float> S;
  const int* on;
  float* dq;  // non-null: the correction is also held here (0 for members switched off)
  int members, tpm;
  __device__ bool where(long long i, int& m, int& e) const {
    const int tile = (int)(i >> 7), t = (int)(i & (kTile - 1));
    m = tile / tpm;
    e = (tile - m * tpm) * kTile + t;
    return m < members && e < M.ne;
  }
  __device__ bool features(long long i, float (&x)[kIn]) const {
    int m, e;
    if (!where(i, m, e)) return false;
    closure_features(M, S, m, e, x);
    return true;
  }
  __device__ void output(long long i, float r) const {
    int m, e;
    if (!where(i, m, e)) return;
    const long long k = (long long)m * S.mse + e;
    const float v = on[m] ? r : 0.f;
    if (dq) dq[k] = v;
    if (on[m]) S.pv_e[k] = S.pv_e[k] + v;
  }
};

// Rows of the member-innermost layout: row i = element i / M, member i % M,
// the order of the arrays, so the 128 rows of a tile read whole lines.  The
// features are those of closure_features, from [element][member] arrays.
// log2(n) for a power of two n, else -1
inline int pow2_shift(int n) {
  if (n <= 0 || (n & (n - 1))) return -1;
  int k = 0;
  while ((1 << k) < n) ++k;
  return k;
}
struct EnsClosureSrc {
  DevMesh M;
  tmc::ens::IO S;
  const float* pv_c;
  const int* on;
  float* dq;  // non-null: the correction is also held here (0 for members switched off)
  int mem;
  long long rows;
  int mshift;  // log2(mem) when mem is a power of two (shift and mask), else -1 (division)
  __device__ __forceinline__ void split(long long i, int& e, int& m) const {
    if (mshift >= 0) {
      e = (int)(i >> mshift);
      m = (int)i & (mem - 1);
    } else {
      e = (int)(i / mem);
      m = (int)(i - (long long)e * mem);
    }
  }
  __device__ bool features(long long i, float (&x)[kIn]) const {
    if (i >= rows) return false;
    int e, m;
    split(i, e, m);
    const size_t W = (size_t)mem;
    const int c1 = M.cellsOnEdge[e], c2 = M.cellsOnEdge[M.ne + e];
    const int v1 = M.verticesOnEdge[e], v2 = M.verticesOnEdge[M.ne + e];
    float ve = 0.f;
#pragma unroll
    for (int k = 0; k < 10; ++k) {
      const size_t s = (size_t)k * M.ne + e;
      ve += S.u[M.edgesOnEdge[s] * W + m] * M.weightsOnEdge_f[s];  // padded entries carry weight 0
    }
    const float dv = M.dvEdge_f[e], dc = M.dcEdge_f[e];
    const float pv1 = S.pv_v[v1 * W + m], pv2 = S.pv_v[v2 * W + m];
    const float pc1 = pv_c[c1 * W + m], pc2 = pv_c[c2 * W + m];
    x[0] = S.u[i];
    x[1] = ve;
    x[2] = S.gd_e[i];
    x[3] = S.pv_e[i];
    x[4] = pv1;
    x[5] = pv2;
    x[6] = pc1;
    x[7] = pc2;
    x[8] = S.gd_in[c1 * W + m];  // h halves: the FP32 gd
    x[9] = S.gd_in[c2 * W + m];
    x[10] = S.E[c1 * W + m];
    x[11] = S.E[c2 * W + m];
    x[12] = S.ghsf[c1 * W + m];
    x[13] = S.ghsf[c2 * W + m];
    x[14] = M.fVertex_f[v1];
    x[15] = M.fVertex_f[v2];
    x[16] = dv;
    x[17] = dc;
#pragma unroll
    for (int k = 0; k < 4; ++k) x[18 + k] = S.u[M.edgesOnEdge[(size_t)k * M.ne + e] * W + m];
    x[22] = (pv2 - pv1) / dv;
    x[23] = (pc2 - pc1) / dc;
    return true;
  }
  __device__ void output(long long i, float r) const {
    if (i >= rows) return;
    int e, m;
    split(i, e, m);
    const float v = on[m] ? r : 0.f;
    if (dq) dq[i] = v;
    if (on[m]) S.pv_e[i] = S.pv_e[i] + v;
  }
};

__global__ void __launch_bounds__(kTcThreads, kTcMinBlocks) k_closure_inner(Net net, EnsClosureSrc src, long long ntiles,
                                                               int* err) {
  extern __shared__ __align__(128) uint8_t smem[];
  if (!forward_tiles(net, src, ntiles, smem) && threadIdx.x % kTile == 0) atomicExch(err, 1);
}

__global__ void k_closure_features_inner(EnsClosureSrc src, int m, float* feat, float* pv) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= src.M.ne) return;
  float x[kIn];
  src.features((long long)e * src.mem + m, x);
  for (int k = 0; k < kIn; ++k) feat[(size_t)e * kIn + k] = x[k];
  pv[e] = x[3];
}

// the held correction of stage 1 added to pv_edge in the later stages
__global__ void k_closure_hold(float* pv_e, const float* dq, int ne, long long mse) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const long long k = (long long)blockIdx.y * mse + e;  // member blockIdx.y
  pv_e[k] += dq[k];
}

__global__ void __launch_bounds__(kTcThreads, kTcMinBlocks) k_closure(Net net, ClosureSrc src, long long ntiles, int* err) {
  extern __shared__ __align__(128) uint8_t smem[];
  if (!forward_tiles(net, src, ntiles, smem) && threadIdx.x % kTile == 0) atomicExch(err, 1);
}

__global__ void k_closure_features(DevMesh M, StageIO<float> S, int m, float* feat, float* pv) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= M.ne) return;
  float x[kIn];
  closure_features(M, S, m, e, x);
  for (int k = 0; k < kIn; ++k) feat[(size_t)e * kIn + k] = x[k];
  pv[e] = x[3];
}

// ---------------------------------------------------------------------------
// CUDA-core forward (FP32 activations, BF16-rounded weights): the reference
// the tensor-core path is checked against
// ---------------------------------------------------------------------------
__device__ __forceinline__ float gelu_ref(float z) { return gelu_tanh(z, tanhf(gelu_arg(z))); }
__device__ __forceinline__ float gelu_grad(float z) {
  const float c = 0.7978845608028654f;
  const float th = tanhf(gelu_arg(z));
  return 0.5f * (1.f + th) + 0.5f * z * (1.f - th * th) * c * (1.f + 3.f * 0.044715f * z * z);
}

struct SimtW {
  float W1[kH][kIn], W2[kH][kH], W3[kH][kH], b[3][kH], w4[kH], b4;
  float xm[kIn], xi[kIn];
};

__device__ void load_simt_weights(const Net& net, SimtW& w) {
  for (int i = threadIdx.x; i < kH * kIn; i += blockDim.x) w.W1[i / kIn][i % kIn] = __bfloat162float(net.pb[kOffW1 + i]);
  for (int i = threadIdx.x; i < kH * kH; i += blockDim.x) {
    w.W2[i / kH][i % kH] = __bfloat162float(net.pb[kOffW2 + i]);
    w.W3[i / kH][i % kH] = __bfloat162float(net.pb[kOffW3 + i]);
  }
  for (int i = threadIdx.x; i < kH; i += blockDim.x) {
    w.b[0][i] = net.p[kOffB1 + i];
    w.b[1][i] = net.p[kOffB2 + i];
    w.b[2][i] = net.p[kOffB3 + i];
    w.w4[i] = __bfloat162float(net.pb[kOffW4 + i]);
  }
  for (int i = threadIdx.x; i < kIn; i += blockDim.x) {
    w.xm[i] = net.xmean[i];
    w.xi[i] = net.xinv[i];
  }
  if (threadIdx.x == 0) w.b4 = net.p[kOffB4];
  __syncthreads();
}

__global__ void __launch_bounds__(128) k_mlp_fwd_simt(Net net, const float* x, float* y, long long rows) {
  extern __shared__ __align__(128) uint8_t smem[];
  SimtW& w = *reinterpret_cast<SimtW*>(smem);
  load_simt_weights(net, w);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (long long)gridDim.x * blockDim.x) {
    float a[kH], b[kH];
    float xr[kIn], xs[kIn];
    for (int k = 0; k < kIn; ++k) {
      xr[k] = x[i * kIn + k];
      xs[k] = (xr[k] - w.xm[k]) * w.xi[k];
    }
    for (int j = 0; j < kH; ++j) {
      float z = w.b[0][j];
      for (int k = 0; k < kIn; ++k) z += w.W1[j][k] * xs[k];
      a[j] = gelu_ref(z);
    }
    for (int j = 0; j < kH; ++j) {
      float z = w.b[1][j];
      for (int k = 0; k < kH; ++k) z += w.W2[j][k] * a[k];
      b[j] = gelu_ref(z);
    }
    float out = w.b4;
    for (int j = 0; j < kH; ++j) {
      float z = w.b[2][j];
      for (int k = 0; k < kH; ++k) z += w.W3[j][k] * b[k];
      out += w.w4[j] * gelu_ref(z);
    }
    y[i] = head_out(net, out, head_dir(net, xr));
  }
}

// ---------------------------------------------------------------------------
// training: one block = 128 samples of the batch; forward keeping the
// pre-activations, MSE loss, backward, block-level weight-gradient GEMMs
// accumulated into the global FP32 gradient with atomics
// ---------------------------------------------------------------------------
constexpr int kLd = kH + 1;  // padded row length (bank conflicts)
struct TrainSmem {
  SimtW w;
  float x[kTile][kIn + 1];
  float z[3][kTile][kLd];  // pre-activations, overwritten by their gradients
  float h[kTile][kLd];     // the activations of one layer at a time
  float dy[kTile];
};

__device__ void block_dw(const float (*dz)[kLd], const float (*hin)[kLd], int kin, float* gW, float* gb) {
  // gW[j][k] += sum_s dz[s][j] hin[s][k]; gb[j] += sum_s dz[s][j]
  const int t = threadIdx.x, j = t >> 1, k0 = (t & 1) * 32;
  float acc[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) acc[i] = 0.f;
  float accb = 0.f;
  for (int s = 0; s < kTile; ++s) {
    const float d = dz[s][j];
    accb += d;
#pragma unroll
    for (int i = 0; i < 32; ++i) acc[i] += d * hin[s][k0 + i];
  }
#pragma unroll
  for (int i = 0; i < 32; ++i)
    if (k0 + i < kin) atomicAdd(&gW[j * kin + k0 + i], acc[i]);
  if ((t & 1) == 0) atomicAdd(&gb[j], accb);
}

__global__ void __launch_bounds__(kTile) k_mlp_train(Net net, const float* X, const float* Y, long long rows,
                                                     long long offset, float inv_batch, float* grad, double* loss) {
  extern __shared__ __align__(128) uint8_t smem[];
  TrainSmem& S = *reinterpret_cast<TrainSmem*>(smem);
  load_simt_weights(net, S.w);
  const int t = threadIdx.x;
  const long long i = (offset + (long long)blockIdx.x * kTile + t) % rows;
  // forward
  float xr[kIn];
  for (int k = 0; k < kIn; ++k) {
    xr[k] = X[i * kIn + k];
    S.x[t][k] = (xr[k] - S.w.xm[k]) * S.w.xi[k];
  }
  const float dir = head_dir(net, xr);
  float a[kH];
  for (int j = 0; j < kH; ++j) {
    float z = S.w.b[0][j];
    for (int k = 0; k < kIn; ++k) z += S.w.W1[j][k] * S.x[t][k];
    S.z[0][t][j] = z;
    a[j] = gelu_ref(z);
  }
  float b[kH];
  for (int j = 0; j < kH; ++j) {
    float z = S.w.b[1][j];
    for (int k = 0; k < kH; ++k) z += S.w.W2[j][k] * a[k];
    S.z[1][t][j] = z;
    b[j] = gelu_ref(z);
  }
  float out = S.w.b4;
  for (int j = 0; j < kH; ++j) {
    float z = S.w.b[2][j];
    for (int k = 0; k < kH; ++k) z += S.w.W3[j][k] * b[k];
    S.z[2][t][j] = z;
    const float h3 = gelu_ref(z);
    S.h[t][j] = h3;
    out += S.w.w4[j] * h3;
  }
  float dpred;
  const float e = head_pred(net, out, dir, dpred) - Y[i] / net.yscale;
  const float dy = 2.f * e * inv_batch * dpred;
  S.dy[t] = dy;
  // loss: block sum of e^2
  {
    float l = e * e;
    for (int off = 16; off > 0; off >>= 1) l += __shfl_down_sync(0xffffffffu, l, off);
    if ((t & 31) == 0) atomicAdd(loss, (double)l * inv_batch);
  }
  __syncthreads();
  // output layer
  if (t < kH) {
    float acc = 0.f;
    for (int s = 0; s < kTile; ++s) acc += S.dy[s] * S.h[s][t];
    atomicAdd(&grad[kOffW4 + t], acc);
  }
  if (t == kH) {
    float acc = 0.f;
    for (int s = 0; s < kTile; ++s) acc += S.dy[s];
    atomicAdd(&grad[kOffB4], acc);
  }
  // dz3 = dy w4 gelu'(z3), in place of z3
  for (int j = 0; j < kH; ++j) S.z[2][t][j] = dy * S.w.w4[j] * gelu_grad(S.z[2][t][j]);
  __syncthreads();
  // layer 3: h = h2
  for (int j = 0; j < kH; ++j) S.h[t][j] = gelu_ref(S.z[1][t][j]);
  __syncthreads();
  block_dw(S.z[2], S.h, kH, grad + kOffW3, grad + kOffB3);
  // dz2 = (dz3 W3) gelu'(z2)
  {
    float d[kH];
    for (int k = 0; k < kH; ++k) d[k] = 0.f;
    for (int j = 0; j < kH; ++j) {
      const float g = S.z[2][t][j];
      for (int k = 0; k < kH; ++k) d[k] += g * S.w.W3[j][k];
    }
    for (int k = 0; k < kH; ++k) S.z[1][t][k] = d[k] * gelu_grad(S.z[1][t][k]);
  }
  __syncthreads();
  // layer 2: h = h1
  for (int j = 0; j < kH; ++j) S.h[t][j] = gelu_ref(S.z[0][t][j]);
  __syncthreads();
  block_dw(S.z[1], S.h, kH, grad + kOffW2, grad + kOffB2);
  // dz1 = (dz2 W2) gelu'(z1)
  {
    float d[kH];
    for (int k = 0; k < kH; ++k) d[k] = 0.f;
    for (int j = 0; j < kH; ++j) {
      const float g = S.z[1][t][j];
      for (int k = 0; k < kH; ++k) d[k] += g * S.w.W2[j][k];
    }
    for (int k = 0; k < kH; ++k) S.z[0][t][k] = d[k] * gelu_grad(S.z[0][t][k]);
  }
  __syncthreads();
  // layer 1: h = normalised input
  for (int k = 0; k < kIn; ++k) S.h[t][k] = S.x[t][k];
  __syncthreads();
  block_dw(S.z[0], S.h, kIn, grad + kOffW1, grad + kOffB1);
}

// Adam (Kingma & Ba 2015) on the FP32 master parameters; BF16 copy refreshed,
// gradient cleared.  A batch whose tensor-core gradient is incomplete (*err
// set: a completion wait ran out) is not applied; its gradient is dropped.
__global__ void k_adam(float* p, __nv_bfloat16* pb, float* g, float* m, float* v, int n, float lr, float b1c,
                       float b2c, const int* err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (*err) {
    g[i] = 0.f;
    return;
  }
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float mh = mi / b1c, vh = vi / b2c;
  const float pi = p[i] - lr * mh / (sqrtf(vh) + eps);
  p[i] = pi;
  pb[i] = __float2bfloat16_rn(pi);
  g[i] = 0.f;
}

__global__ void k_to_bf16(const float* p, __nv_bfloat16* pb, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) pb[i] = __float2bfloat16_rn(p[i]);
}

// ---------------------------------------------------------------------------
// training on the tensor cores (tmc_mlp_train_tc.cuh): rows of the batch
// from the dataset, wrapping at its end
// ---------------------------------------------------------------------------
struct TrainSrc {
  const float* X;
  const float* Y;
  long long rows, offset;
  float yscale;
  // row i of the batch as the trainer's column group cg (0..3) needs it: the
  // eight features 8 cg .. 8 cg + 7 (none for cg 3, whose columns are the
  // constants), the four the output heads use (x0, x1, x22, x23) and the
  // target.  A row is 96 bytes, 16-byte aligned.
  __device__ bool sample(long long i, int cg, float (&x)[8], float (&xd)[4], float& t) const {
    const long long j = (offset + i) % rows;
    const float* xr = X + j * kIn;
    if (cg < 3) {
      const float4 a = *reinterpret_cast<const float4*>(xr + 8 * cg);
      const float4 b = *reinterpret_cast<const float4*>(xr + 8 * cg + 4);
      x[0] = a.x, x[1] = a.y, x[2] = a.z, x[3] = a.w, x[4] = b.x, x[5] = b.y, x[6] = b.z, x[7] = b.w;
    } else {
#pragma unroll
      for (int k = 0; k < 8; ++k) x[k] = 0.f;
    }
    const float2 d0 = *reinterpret_cast<const float2*>(xr);
    const float2 d1 = *reinterpret_cast<const float2*>(xr + 22);
    xd[0] = d0.x, xd[1] = d0.y, xd[2] = d1.x, xd[3] = d1.y;
    t = Y[j] / yscale;
    return true;
  }
};

__global__ void __launch_bounds__(kTrThreads, 1) k_mlp_train_tc(Net net, TrainSrc src, long long ntiles, float inv_batch,
                                                             float* part, double* ploss, int* err) {
  extern __shared__ __align__(128) uint8_t smem[];
  if (!train_tiles(net, src, ntiles, inv_batch, part, ploss, smem) && threadIdx.x == 0) atomicExch(err, 1);
}

// The tensor-core trainer's per-block partial gradients and losses, summed
// in a fixed order (the result does not depend on scheduling).  A block of
// 256 threads takes 32 parameters: warp q adds the partials of blocks q,
// q + 8, q + 16, ... (independent loads), and warp 0 adds the eight chains
// in order.  Warp 0 of block 0 sums the losses (lane chains, then a fixed
// shuffle tree).
constexpr int kRedChains = 8;
__device__ __forceinline__ float grad_sum(const float* part, int nblk, int i) {
  __shared__ float red[kRedChains][32];
  const int c = threadIdx.x & 31, q = threadIdx.x >> 5;
  float s = 0.f;
  if (i < kParams) {
#pragma unroll 4
    for (int b = q; b < nblk; b += kRedChains) s += part[(size_t)b * kParams + i];
  }
  red[q][c] = s;
  __syncthreads();
  float g = 0.f;
  if (q == 0)
#pragma unroll
    for (int k = 0; k < kRedChains; ++k) g += red[k][c];
  return g;
}
__device__ __forceinline__ double loss_sum(const double* ploss, int nblk) {
  double l = 0.0;
  for (int b = threadIdx.x; b < nblk; b += 32) l += ploss[b];
  for (int off = 16; off > 0; off >>= 1) l += __shfl_down_sync(0xffffffffu, l, off);
  return l;
}
// grad += the summed partial gradient; loss += the summed loss
__global__ void __launch_bounds__(32 * kRedChains) k_grad_reduce(const float* part, const double* ploss, int nblk,
                                                                 float* grad, double* loss) {
  const int i = blockIdx.x * 32 + (threadIdx.x & 31);
  const float g = grad_sum(part, nblk, i);
  if (threadIdx.x < 32 && i < kParams) grad[i] += g;
  if (blockIdx.x == 0 && threadIdx.x < 32) {
    const double l = loss_sum(ploss, nblk);
    if (threadIdx.x == 0) *loss += l;
  }
}
// the summed partial gradient applied by Adam (as k_adam), the summed loss
// stored in *loss; nothing is applied when *err is set (a completion wait of
// the batch ran out)
__global__ void __launch_bounds__(32 * kRedChains) k_grad_adam(const float* part, const double* ploss, int nblk,
                                                               float* p, __nv_bfloat16* pb, float* m, float* v,
                                                               float lr, float b1c, float b2c, const int* err,
                                                               double* loss) {
  const int i = blockIdx.x * 32 + (threadIdx.x & 31);
  const float gi = grad_sum(part, nblk, i);
  if (blockIdx.x == 0 && threadIdx.x < 32) {
    const double l = loss_sum(ploss, nblk);
    if (threadIdx.x == 0) *loss = l;
  }
  if (threadIdx.x >= 32 || i >= kParams || *err) return;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float mh = mi / b1c, vh = vi / b2c;
  const float pi = p[i] - lr * mh / (sqrtf(vh) + eps);
  p[i] = pi;
  pb[i] = __float2bfloat16_rn(pi);
}

}  // namespace

namespace tmc {
void launch_closure(const DevMesh& M, const StageIO<float>& S, const ClosureArgs& a, cudaStream_t st) {
  const int members = S.members > 1 ? S.members : 1;
  const int tpm = (M.ne + kTile - 1) / kTile;
  if (a.mode == 2) {
    k_closure_hold<<<dim3((M.ne + 255) / 256, members), 256, 0, st>>>(S.pv_e, a.dq, M.ne, S.mse);
    return;
  }
  ClosureSrc src{M, S, a.member_on, a.mode == 1 ? a.dq : nullptr, members, tpm};
  const long long ntiles = (long long)tpm * members;
  const int grid = (int)std::min<long long>((ntiles + kGroups - 1) / kGroups, (long long)a.sms * 4);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_closure, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemTc);
    attr = true;
  }
  k_closure<<<grid, kTcThreads, kSmemTc, st>>>(*static_cast<const Net*>(a.net), src, ntiles, a.err);
}
namespace ens {
void launch_closure(const DevMesh& Mh, const Dims& D, const IO& S, const float* pv_c, const ClosureArgs& a,
                    cudaStream_t st) {
  if (a.mode == 2) {
    launch_closure_hold(Mh, D, S, a.dq, st);
    return;
  }
  const long long rows = (long long)Mh.ne * D.M;
  EnsClosureSrc src{Mh, S, pv_c, a.member_on, a.mode == 1 ? a.dq : nullptr, D.M, rows, pow2_shift(D.M)};
  const long long ntiles = (rows + kTile - 1) / kTile;
  const int grid = (int)std::min<long long>((ntiles + kGroups - 1) / kGroups, (long long)a.sms * 4);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_closure_inner, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemTc);
    attr = true;
  }
  k_closure_inner<<<grid, kTcThreads, kSmemTc, st>>>(*static_cast<const Net*>(a.net), src, ntiles, a.err);
}
void launch_closure_features(const DevMesh& Mh, const Dims& D, const IO& S, const float* pv_c, int m, float* feat,
                             float* pv, cudaStream_t st) {
  const EnsClosureSrc src{Mh, S, pv_c, nullptr, nullptr, D.M, (long long)Mh.ne * D.M, pow2_shift(D.M)};
  k_closure_features_inner<<<(Mh.ne + 255) / 256, 256, 0, st>>>(src, m, feat, pv);
}
}  // namespace ens
void launch_closure_features(const DevMesh& M, const StageIO<float>& S, int member, float* feat, float* pv,
                             cudaStream_t st) {
  k_closure_features<<<(M.ne + 255) / 256, 256, 0, st>>>(M, S, member, feat, pv);
}
}  // namespace tmc

struct tmc_mlp {
  int device = 0;
  cudaStream_t st = nullptr;
  float* p = nullptr;  // master FP32
  __nv_bfloat16* pb = nullptr;
  float *g = nullptr, *m = nullptr, *v = nullptr;
  float *xmean = nullptr, *xinv = nullptr;
  float yscale = 1.f;
  float *dx = nullptr, *dy = nullptr;  // dataset
  long long rows = 0;
  long long cursor = 0;
  int adam_t = 0;
  float *io_x = nullptr, *io_y = nullptr;
  long long io_cap = 0;
  int* d_err = nullptr;
  double* d_loss = nullptr;
  double* d_losses = nullptr;  // tmc_mlp_train: one loss per step, read back once at the end
  int losses_cap = 0;
  int train_tc = 1;          // tmc_mlp_train / tmc_mlp_gradient on the tensor cores (0: CUDA cores)
  float* part = nullptr;     // [sms][kParams] per-block partial gradients (tensor-core trainer)
  double* ploss = nullptr;   // [sms]
  int sms = 148;
  int wait_polls = tmc::mlp::kWaitPolls;  // tmc_mlp_set_wait_limit
  int head = tmc::mlp::kHeadPlain;        // tmc_mlp_set_head
  float head_dt = 0.f;
  std::string err;
  int fail(int code, const std::string& s) {
    err = s;
    return code;
  }
  int check(const char* where) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(TMC_E_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
    return TMC_OK;
  }
  Net net() const { return Net{p, pb, xmean, xinv, yscale, wait_polls, head, head_dt}; }
};

tmc::mlp::Net tmc_mlp_net(const tmc_mlp* n) { return n->net(); }

extern "C" {

int tmc_mlp_create(int32_t device, uint64_t seed, tmc_mlp** out) {
  if (!out) return TMC_E_ARG;
  *out = nullptr;
  auto n = new tmc_mlp();
  n->device = device;
  if (cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    n->err = "cudaSetDevice failed (no CUDA device?)";
    *out = n;
    return TMC_E_CUDA;
  }
  cudaDeviceGetAttribute(&n->sms, cudaDevAttrMultiProcessorCount, device);
  bool okc = cudaStreamCreateWithFlags(&n->st, cudaStreamNonBlocking) == cudaSuccess;
  okc = okc && cudaMalloc(&n->p, sizeof(float) * kParams) == cudaSuccess;
  okc = okc && cudaMalloc(&n->pb, sizeof(__nv_bfloat16) * kParams) == cudaSuccess;
  okc = okc && cudaMalloc(&n->g, sizeof(float) * kParams) == cudaSuccess;
  okc = okc && cudaMalloc(&n->m, sizeof(float) * kParams) == cudaSuccess;
  okc = okc && cudaMalloc(&n->v, sizeof(float) * kParams) == cudaSuccess;
  okc = okc && cudaMalloc(&n->xmean, sizeof(float) * kIn) == cudaSuccess;
  okc = okc && cudaMalloc(&n->xinv, sizeof(float) * kIn) == cudaSuccess;
  okc = okc && cudaMalloc(&n->d_err, sizeof(int)) == cudaSuccess;
  okc = okc && cudaMalloc(&n->d_loss, sizeof(double)) == cudaSuccess;
  okc = okc && cudaMalloc(&n->part, sizeof(float) * kParams * n->sms) == cudaSuccess;
  okc = okc && cudaMalloc(&n->ploss, sizeof(double) * n->sms) == cudaSuccess;
  *out = n;
  if (!okc) return n->check("tmc_mlp_create");
  // PyTorch-style Linear initialisation: U(-1/sqrt(fan_in), 1/sqrt(fan_in))
  std::vector<float> h(kParams);
  std::mt19937_64 rng(seed);
  auto fill = [&](int off, int count, int fan_in) {
    std::uniform_real_distribution<float> d(-1.f / std::sqrt((float)fan_in), 1.f / std::sqrt((float)fan_in));
    for (int i = 0; i < count; ++i) h[off + i] = d(rng);
  };
  fill(kOffW1, kH * kIn, kIn);
  fill(kOffB1, kH, kIn);
  fill(kOffW2, kH * kH, kH);
  fill(kOffB2, kH, kH);
  fill(kOffW3, kH * kH, kH);
  fill(kOffB3, kH, kH);
  fill(kOffW4, kH, kH);
  fill(kOffB4, 1, kH);
  std::vector<float> zero(kIn, 0.f), one(kIn, 1.f);
  cudaMemcpy(n->xmean, zero.data(), sizeof(float) * kIn, cudaMemcpyHostToDevice);
  cudaMemcpy(n->xinv, one.data(), sizeof(float) * kIn, cudaMemcpyHostToDevice);
  cudaMemset(n->g, 0, sizeof(float) * kParams);
  cudaMemset(n->m, 0, sizeof(float) * kParams);
  cudaMemset(n->v, 0, sizeof(float) * kParams);
  cudaMemset(n->d_err, 0, sizeof(int));
  int rc = tmc_mlp_set_params(n, h.data());
  if (rc) return rc;
  cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TrainSmem));
  cudaFuncSetAttribute(k_mlp_fwd_simt, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SimtW));
  cudaFuncSetAttribute(k_mlp_fwd_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemTc);
  cudaFuncSetAttribute(k_mlp_train_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemTrain);
  return n->check("tmc_mlp_create");
}

int tmc_mlp_destroy(tmc_mlp* n) {
  if (!n) return TMC_OK;
  if (n->st) cudaStreamSynchronize(n->st);
  void* ptrs[] = {n->p, n->pb, n->g, n->m, n->v, n->xmean, n->xinv, n->dx, n->dy, n->io_x, n->io_y, n->d_err, n->d_loss,
                   n->d_losses, n->part,  n->ploss};
  for (void* q : ptrs) cudaFree(q);
  if (n->st) cudaStreamDestroy(n->st);
  delete n;
  return TMC_OK;
}

const char* tmc_mlp_last_error(const tmc_mlp* n) { return n ? n->err.c_str() : "null network"; }

int tmc_mlp_get_params(tmc_mlp* n, float* params) {
  if (!n || !params) return TMC_E_ARG;
  if (cudaMemcpyAsync(params, n->p, sizeof(float) * kParams, cudaMemcpyDeviceToHost, n->st) != cudaSuccess)
    return n->check("tmc_mlp_get_params");
  cudaStreamSynchronize(n->st);
  return n->check("tmc_mlp_get_params");
}

int tmc_mlp_set_params(tmc_mlp* n, const float* params) {
  if (!n || !params) return TMC_E_ARG;
  cudaMemcpyAsync(n->p, params, sizeof(float) * kParams, cudaMemcpyHostToDevice, n->st);
  k_to_bf16<<<(kParams + 255) / 256, 256, 0, n->st>>>(n->p, n->pb, kParams);
  cudaMemsetAsync(n->m, 0, sizeof(float) * kParams, n->st);
  cudaMemsetAsync(n->v, 0, sizeof(float) * kParams, n->st);
  n->adam_t = 0;
  cudaStreamSynchronize(n->st);
  return n->check("tmc_mlp_set_params");
}

int tmc_mlp_set_scaling(tmc_mlp* n, const float* x_mean, const float* x_inv_std, float y_scale) {
  if (!n || !x_mean || !x_inv_std) return TMC_E_ARG;
  if (!(y_scale > 0.f) || !std::isfinite(y_scale)) return n->fail(TMC_E_ARG, "tmc_mlp_set_scaling: y_scale must be finite and > 0");
  for (int k = 0; k < kIn; ++k)
    if (!std::isfinite(x_mean[k]) || !std::isfinite(x_inv_std[k]))
      return n->fail(TMC_E_ARG, "tmc_mlp_set_scaling: non-finite feature scaling");
  cudaMemcpyAsync(n->xmean, x_mean, sizeof(float) * kIn, cudaMemcpyHostToDevice, n->st);
  cudaMemcpyAsync(n->xinv, x_inv_std, sizeof(float) * kIn, cudaMemcpyHostToDevice, n->st);
  n->yscale = y_scale;
  cudaStreamSynchronize(n->st);
  return n->check("tmc_mlp_set_scaling");
}

static int ensure_io(tmc_mlp* n, long long rows) {
  if (rows <= n->io_cap) return TMC_OK;
  cudaFree(n->io_x);
  cudaFree(n->io_y);
  n->io_x = n->io_y = nullptr;
  n->io_cap = 0;
  if (cudaMalloc(&n->io_x, sizeof(float) * kIn * rows) != cudaSuccess ||
      cudaMalloc(&n->io_y, sizeof(float) * rows) != cudaSuccess)
    return n->check("tmc_mlp io buffers");
  n->io_cap = rows;
  return TMC_OK;
}

int tmc_mlp_forward(tmc_mlp* n, const float* x, int64_t rows, float* y, int32_t tensor_cores) {
  if (!n || !x || !y || rows < 0) return TMC_E_ARG;
  if (rows == 0) return TMC_OK;
  int rc = ensure_io(n, rows);
  if (rc) return rc;
  cudaMemcpyAsync(n->io_x, x, sizeof(float) * kIn * rows, cudaMemcpyHostToDevice, n->st);
  if (tensor_cores) {
    const long long ntiles = (rows + kTile - 1) / kTile;
    const int grid = (int)std::min<long long>((ntiles + kGroups - 1) / kGroups, (long long)n->sms * 4);
    cudaMemsetAsync(n->d_err, 0, sizeof(int), n->st);
    k_mlp_fwd_tc<<<grid, kTcThreads, kSmemTc, n->st>>>(n->net(), BufSrc{n->io_x, n->io_y, rows}, ntiles, n->d_err);
  } else {
    const int grid = (int)std::min<long long>((rows + 127) / 128, (long long)n->sms * 8);
    k_mlp_fwd_simt<<<grid, 128, sizeof(SimtW), n->st>>>(n->net(), n->io_x, n->io_y, rows);
  }
  cudaMemcpyAsync(y, n->io_y, sizeof(float) * rows, cudaMemcpyDeviceToHost, n->st);
  int herr = 0;
  if (tensor_cores) cudaMemcpyAsync(&herr, n->d_err, sizeof(int), cudaMemcpyDeviceToHost, n->st);
  if (cudaStreamSynchronize(n->st) != cudaSuccess) return n->check("tmc_mlp_forward");
  if (herr) return n->fail(TMC_E_HEALTH, "tmc_mlp_forward: a tensor-core completion wait timed out");
  return n->check("tmc_mlp_forward");
}

int tmc_mlp_set_dataset(tmc_mlp* n, const float* x, const float* y, int64_t rows) {
  if (!n || !x || !y || rows <= 0) return TMC_E_ARG;
  cudaFree(n->dx);
  cudaFree(n->dy);
  n->dx = n->dy = nullptr;
  n->rows = 0;
  if (cudaMalloc(&n->dx, sizeof(float) * kIn * rows) != cudaSuccess ||
      cudaMalloc(&n->dy, sizeof(float) * rows) != cudaSuccess)
    return n->check("tmc_mlp_set_dataset");
  cudaMemcpyAsync(n->dx, x, sizeof(float) * kIn * rows, cudaMemcpyHostToDevice, n->st);
  cudaMemcpyAsync(n->dy, y, sizeof(float) * rows, cudaMemcpyHostToDevice, n->st);
  n->rows = rows;
  n->cursor = 0;
  cudaStreamSynchronize(n->st);
  return n->check("tmc_mlp_set_dataset");
}

// one gradient pass over `batch` rows of X/Y from row `offset` (wrapping at
// `rows`), added into n->g and its loss into *loss (device)
// the tensor-core gradient tiles of one batch into n->part / n->ploss; returns
// the number of blocks (partials)
static int launch_train_tc(tmc_mlp* n, const float* X, const float* Y, long long rows, long long offset,
                           long long batch) {
  const long long ntiles = batch / kTile;
  const int grid = (int)std::min<long long>(ntiles, (long long)n->sms);
  k_mlp_train_tc<<<grid, kTrThreads, kSmemTrain, n->st>>>(n->net(), TrainSrc{X, Y, rows, offset, n->yscale}, ntiles,
                                                        1.f / (float)batch, n->part, n->ploss, n->d_err);
  return grid;
}

static void launch_gradient(tmc_mlp* n, const float* X, const float* Y, long long rows, long long offset, long long batch,
                            double* loss) {
  const float inv_batch = 1.f / (float)batch;
  if (n->train_tc) {
    const int grid = launch_train_tc(n, X, Y, rows, offset, batch);
    k_grad_reduce<<<(kParams + 31) / 32, 32 * kRedChains, 0, n->st>>>(n->part, n->ploss, grid, n->g, loss);
  } else {
    k_mlp_train<<<(unsigned)(batch / kTile), kTile, sizeof(TrainSmem), n->st>>>(n->net(), X, Y, rows, offset,
                                                                                inv_batch, n->g, loss);
  }
}

// the completion-wait flag of the tensor-core trainer, read and cleared
static int train_status(tmc_mlp* n, const char* where) {
  int herr = 0;
  cudaMemcpyAsync(&herr, n->d_err, sizeof(int), cudaMemcpyDeviceToHost, n->st);
  cudaMemsetAsync(n->d_err, 0, sizeof(int), n->st);
  if (cudaStreamSynchronize(n->st) != cudaSuccess) return n->check(where);
  if (herr) return n->fail(TMC_E_HEALTH, std::string(where) + ": a tensor-core completion wait timed out");
  return n->check(where);
}

int tmc_mlp_set_head(tmc_mlp* n, int32_t head, double dt) {
  if (!n) return TMC_E_ARG;
  if (head != kHeadPlain && head != kHeadApvm && head != kHeadSign)
    return n->fail(TMC_E_ARG, "tmc_mlp_set_head: head must be 0, 1 or 2");
  if (head == kHeadApvm && !(dt > 0.0)) return n->fail(TMC_E_ARG, "tmc_mlp_set_head: the APVM head needs dt > 0");
  n->head = head;
  n->head_dt = head == kHeadApvm ? (float)dt : 0.f;
  return TMC_OK;
}

int tmc_mlp_set_wait_limit(tmc_mlp* n, int32_t polls) {
  if (!n) return TMC_E_ARG;
  n->wait_polls = polls < 0 ? tmc::mlp::kWaitPolls : std::min<int32_t>(polls, tmc::mlp::kWaitPolls);
  return TMC_OK;
}

int tmc_mlp_set_train_mode(tmc_mlp* n, int32_t tensor_cores) {
  if (!n || (tensor_cores != 0 && tensor_cores != 1)) return n ? n->fail(TMC_E_ARG, "tensor_cores must be 0 or 1") : TMC_E_ARG;
  n->train_tc = tensor_cores;
  return TMC_OK;
}

int tmc_mlp_train(tmc_mlp* n, int32_t batch, int32_t steps, float lr, float* losses) {
  if (!n || batch <= 0 || batch % kTile != 0 || steps < 0) return n ? n->fail(TMC_E_ARG, "batch must be a positive multiple of 128") : TMC_E_ARG;
  if (!n->dx) return n->fail(TMC_E_STATE, "tmc_mlp_train: no dataset");
  // the steps' losses stay on the device until the last step: no host round
  // trip between steps
  if (losses && steps > n->losses_cap) {
    cudaFree(n->d_losses);
    n->d_losses = nullptr;
    n->losses_cap = 0;
    if (cudaMalloc(&n->d_losses, sizeof(double) * steps) != cudaSuccess) return n->check("tmc_mlp_train");
    n->losses_cap = steps;
  }
  cudaMemsetAsync(n->d_err, 0, sizeof(int), n->st);
  for (int s = 0; s < steps; ++s) {
    double* dl = losses ? n->d_losses + s : n->d_loss;
    n->adam_t += 1;
    const float b1c = 1.f - std::pow(0.9f, (float)n->adam_t), b2c = 1.f - std::pow(0.999f, (float)n->adam_t);
    if (n->train_tc) {
      // two launches per step: the gradient tiles, then the fixed-order sum
      // of their partials with Adam
      const int grid = launch_train_tc(n, n->dx, n->dy, n->rows, n->cursor, batch);
      k_grad_adam<<<(kParams + 31) / 32, 32 * kRedChains, 0, n->st>>>(n->part, n->ploss, grid, n->p, n->pb, n->m,
                                                                      n->v, lr, b1c, b2c, n->d_err, dl);
    } else {
      cudaMemsetAsync(dl, 0, sizeof(double), n->st);
      launch_gradient(n, n->dx, n->dy, n->rows, n->cursor, batch, dl);
      k_adam<<<(kParams + 255) / 256, 256, 0, n->st>>>(n->p, n->pb, n->g, n->m, n->v, kParams, lr, b1c, b2c,
                                                       n->d_err);
    }
    n->cursor = (n->cursor + batch) % n->rows;
  }
  if (losses && steps > 0) {
    std::vector<double> h(steps);
    cudaMemcpyAsync(h.data(), n->d_losses, sizeof(double) * steps, cudaMemcpyDeviceToHost, n->st);
    if (cudaStreamSynchronize(n->st) != cudaSuccess) return n->check("tmc_mlp_train");
    for (int s = 0; s < steps; ++s) losses[s] = (float)h[s];
  }
  return train_status(n, "tmc_mlp_train");
}

int tmc_mlp_gradient(tmc_mlp* n, const float* x, const float* y, int64_t rows, float* grad, double* loss) {
  if (!n || !x || !y || !grad || rows <= 0 || rows % kTile != 0)
    return n ? n->fail(TMC_E_ARG, "rows must be a positive multiple of 128") : TMC_E_ARG;
  int rc = ensure_io(n, rows);
  if (rc) return rc;
  cudaMemcpyAsync(n->io_x, x, sizeof(float) * kIn * rows, cudaMemcpyHostToDevice, n->st);
  cudaMemcpyAsync(n->io_y, y, sizeof(float) * rows, cudaMemcpyHostToDevice, n->st);
  cudaMemsetAsync(n->g, 0, sizeof(float) * kParams, n->st);
  cudaMemsetAsync(n->d_loss, 0, sizeof(double), n->st);
  cudaMemsetAsync(n->d_err, 0, sizeof(int), n->st);
  launch_gradient(n, n->io_x, n->io_y, rows, 0, rows, n->d_loss);
  cudaMemcpyAsync(grad, n->g, sizeof(float) * kParams, cudaMemcpyDeviceToHost, n->st);
  double l = 0.0;
  cudaMemcpyAsync(&l, n->d_loss, sizeof(double), cudaMemcpyDeviceToHost, n->st);
  cudaMemsetAsync(n->g, 0, sizeof(float) * kParams, n->st);
  rc = train_status(n, "tmc_mlp_gradient");
  if (rc == TMC_OK && loss) *loss = l;
  return rc;
}

}  // extern "C"
