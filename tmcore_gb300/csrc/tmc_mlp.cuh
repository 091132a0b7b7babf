// The learned PV-on-edge closure: a 24 -> 64 -> 64 -> 64 -> 1 MLP with GELU
// (tanh form, Hendrycks & Gimpel 2016) between the hidden layers, BF16
// weights and FP32 accumulation.
//
// Inference runs on the 5th-generation tensor cores: tiles of 128 edges, one
// tcgen05.mma (M = 128, N = 64, K = 16, BF16 x BF16 -> FP32 in tensor memory)
// per 16 inputs of a layer, issued by one thread; the weights and the
// activations sit in shared memory in the canonical no-swizzle K-major
// layout (8-row x 16-byte core matrices); the epilogue (bias, GELU, BF16
// rounding) reads the accumulator back with tcgen05.ld and writes the next
// layer's operand.  Training (forward with stored pre-activations, backward,
// Adam) runs on the CUDA cores in FP32 from the BF16 weights.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace tmc {
namespace mlp {

constexpr int kIn = 24;     // features per edge
constexpr int kInPad = 32;  // first-layer K padded to two MMA K-steps
constexpr int kH = 64;      // hidden width
constexpr int kTile = 128;  // edges per tensor-core tile (MMA M)
constexpr int kGroups = 2;       // tiles in flight per block of the tensor-core forward
constexpr int kTcThreads = kTile * kGroups;  // one thread per row of each tile
// blocks per SM the tensor-core forward is compiled for: its shared memory
// (53 KB) allows 4, whose 4 x 128 accumulator columns fill the 512 of TMEM,
// so an allocation never waits.  4 (64 registers, ~100 bytes spilled) beats
// 3 and 2: 256 level-6 members with the closure in every stage take 13.4 ms
// per step against 14.9 and 14.8 (one tile group per block: 14.2)
#ifndef TMC_TC_MIN_BLOCKS
#define TMC_TC_MIN_BLOCKS 4
#endif
constexpr int kTcMinBlocks = TMC_TC_MIN_BLOCKS;

// parameter vector layout (FP32 master copy; the BF16 copy has the same layout)
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kH * kIn;
constexpr int kOffW2 = kOffB1 + kH;
constexpr int kOffB2 = kOffW2 + kH * kH;
constexpr int kOffW3 = kOffB2 + kH;
constexpr int kOffB3 = kOffW3 + kH * kH;
constexpr int kOffW4 = kOffB3 + kH;
constexpr int kOffB4 = kOffW4 + kH;
constexpr int kParams = kOffB4 + 1;  // 9985
static_assert(kParams == 9985, "24-64-64-64-1 MLP has 9985 parameters");

// device view of the network for the forward kernels
struct Net {
  const float* p;             // FP32 master parameters (biases are read from here)
  const __nv_bfloat16* pb;    // BF16 parameters (weights are read from here)
  const float* xmean;         // [kIn] feature normalisation
  const float* xinv;          // [kIn]
  float yscale;               // output scale
  int wait_polls;             // poll limit of each tensor-core completion wait (kWaitPolls)
  int head;                   // kHeadPlain, kHeadApvm or kHeadSign
  float head_dt;              // kHeadApvm: the model time step (s)
};

// Poll limit of a tensor-core completion wait (mbarrier try_wait loop).  A
// wait that runs out flags an error; the wait that then drains the
// outstanding MMAs before the tensor memory is freed always uses this limit.
constexpr int kWaitPolls = 1 << 20;

// Output heads: how the network's raw output y of an edge becomes the
// correction added to pv_edge (and the prediction the training loss fits).
//   kHeadPlain  y * yscale, unconstrained.
//   kHeadApvm   -softplus(y) dt (v (q_v2 - q_v1)/dvEdge + u (q_c2 - q_c1)/dcEdge):
//               the anticipated-potential-vorticity correction of
//               operators_mod.F90:296-316 with a learned non-negative
//               per-edge weight softplus(y) in place of apvm_weight.  The
//               correction lies along APVM's upwinding direction with APVM's
//               sign, so like APVM it can only remove potential enstrophy.
//   kHeadSign   y * yscale where it has APVM's sign along the edge, i.e.
//               where y v (q_v2 - q_v1) <= 0, else 0: the unconstrained
//               correction restricted to the edges where it removes potential
//               enstrophy through q.F_perp (the correction times the edge's
//               tangential PV flux difference is never positive).
// Inside the energy-conserving q.F_perp form no head changes mass or energy.
constexpr int kHeadPlain = 0, kHeadApvm = 1, kHeadSign = 2;

// The head's auxiliary value of an edge from its raw closure features (1: v,
// 22: pv gradient along the edge, 0: u, 23: across it): kHeadApvm the APVM
// direction dt (v dq/dt + u dq/dn); kHeadSign v dq/dt.
// from the four features the heads use: x0, x1, x22, x23
__device__ __forceinline__ float head_dir4(const Net& net, float x0, float x1, float x22, float x23) {
  if (net.head == kHeadApvm) return net.head_dt * (x1 * x22 + x0 * x23);
  if (net.head == kHeadSign) return x1 * x22;
  return 0.f;
}
__device__ __forceinline__ float head_dir(const Net& net, const float (&x)[kIn]) {
  return head_dir4(net, x[0], x[1], x[22], x[23]);
}
__device__ __forceinline__ float softplus_f(float y) { return y > 20.f ? y : log1pf(__expf(y)); }
// the correction from the raw output y (units of pv_edge)
__device__ __forceinline__ float head_out(const Net& net, float y, float dir) {
  if (net.head == kHeadApvm) return -softplus_f(y) * dir;
  if (net.head == kHeadSign) return y * dir <= 0.f ? y * net.yscale : 0.f;
  return y * net.yscale;
}
// the prediction in units of yscale and its derivative with respect to y
// (the training loss is the mean of (prediction - target / yscale)^2)
__device__ __forceinline__ float head_pred(const Net& net, float y, float dir, float& dpred) {
  if (net.head == kHeadApvm) {
    const float inv = 1.f / net.yscale;
    dpred = -dir * inv / (1.f + __expf(-y));
    return -softplus_f(y) * dir * inv;
  }
  if (net.head == kHeadSign && y * dir > 0.f) {
    dpred = 0.f;
    return 0.f;
  }
  dpred = 1.f;
  return y;
}

__device__ __forceinline__ float gelu_tanh(float x, float t) { return 0.5f * x * (1.f + t); }
__device__ __forceinline__ float gelu_arg(float x) { return 0.7978845608028654f * (x + 0.044715f * x * x * x); }

// shared-memory size of the tensor-core forward kernel
constexpr int kSmemW1 = kH * kInPad * 2;  // 4 KB
constexpr int kSmemW = kH * kH * 2;       // 8 KB
constexpr int kSmemA = kTile * kH * 2;    // 16 KB
constexpr int kSmemTc = kSmemW1 + 2 * kSmemW + kGroups * kSmemA + 64;

}  // namespace mlp
}  // namespace tmc

struct tmc_mlp;
// the device view of a network handle (tmc_mlp.cu)
tmc::mlp::Net tmc_mlp_net(const tmc_mlp* n);
