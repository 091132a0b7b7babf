// tcgen05 building blocks of the MLP forward (inline PTX, sm_100a / sm_103a):
// shared-memory matrix descriptors, the BF16 MMA with its accumulator in
// tensor memory, commit to an mbarrier, bounded mbarrier waits, tensor-memory
// allocation and loads, and the tile loop of the forward pass.
#pragma once

#include "tmc_mlp.cuh"

namespace tmc {
namespace mlp {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Byte offset of element (row, k) of a K-major operand with K columns in the
// no-swizzle canonical layout: 8x8 core matrices of 16-byte rows, stored
// 128 bytes each, K-chunks of one 8-row group adjacent (stride 128 B), 8-row
// groups (K/8)*128 B apart.
__device__ __forceinline__ uint32_t core_off(int row, int k, int K) {
  return (uint32_t)(((row >> 3) * (K >> 3) + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// Shared-memory matrix descriptor: start address, leading-dimension byte
// offset (between core matrices along K), stride-dimension byte offset
// (between 8-row groups), descriptor version 1 (bits 46-48 = 0b001), no
// swizzle, base offset 0.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9 = 1, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// arrive on the mbarrier once all tcgen05.mma issued so far by this thread complete
__device__ __forceinline__ void mma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}

// Bounded wait for the given phase parity: at most `polls` polls; false when
// the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, int polls = kWaitPolls) {
  for (int i = 0; i < polls; ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes become visible to the tensor cores
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 32 lanes x 16 columns of FP32 from tensor memory (this warp's lane quarter)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ float tanh_fast(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// GELU (tanh form) on a pair of BF16 values with packed BF16 arithmetic:
// 0.5 z (1 + tanh(c (z + 0.044715 z^3))), tanh.approx on the pair
__device__ __forceinline__ __nv_bfloat162 tanh_bf16x2(__nv_bfloat162 x) {
  uint32_t in = *reinterpret_cast<uint32_t*>(&x), out;
  asm("tanh.approx.bf16x2 %0, %1;" : "=r"(out) : "r"(in));
  return *reinterpret_cast<__nv_bfloat162*>(&out);
}
// 2 gelu(z) = z (1 + tanh(c (z + 0.044715 z^3))); the factor 1/2 is folded
// into the next layer's weights (exact in BF16)
__device__ __forceinline__ __nv_bfloat162 gelu2_bf16x2(__nv_bfloat162 z) {
  const __nv_bfloat162 k0 = __float2bfloat162_rn(0.7978845608028654f);
  const __nv_bfloat162 k1 = __float2bfloat162_rn(0.7978845608028654f * 0.044715f);
  const __nv_bfloat162 a = __hmul2(z, __hfma2(__hmul2(z, z), k1, k0));
  return __hfma2(z, tanh_bf16x2(a), z);
}

// (bias and) GELU of 16 accumulator columns into 8 BF16 pairs; without a bias
// the bias came through the MMA (layer 1: two input columns of ones)
template <bool kBias>
__device__ __forceinline__ void bias_gelu16(const float (&d)[16], const float* b, __nv_bfloat162 (&h)[8]) {
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float z0 = kBias ? d[2 * j] + b[2 * j] : d[2 * j];
    const float z1 = kBias ? d[2 * j + 1] + b[2 * j + 1] : d[2 * j + 1];
    h[j] = gelu2_bf16x2(__floats2bfloat162_rn(z0, z1));
  }
}

// store 8 consecutive K values of one row (16 bytes) of a K-major operand
__device__ __forceinline__ void store8_bf16(uint8_t* base, int row, int k0, int K, const float* v) {
  __nv_bfloat162 h[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) h[i] = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
  *reinterpret_cast<uint4*>(base + core_off(row, k0, K)) = *reinterpret_cast<uint4*>(h);
}

// Named barrier of the 128 threads of one tile group (ids 1, 2, ...).
__device__ __forceinline__ void group_sync(int id) { asm volatile("bar.sync %0, 128;" ::"r"(id) : "memory"); }
__device__ __forceinline__ bool group_sync_and(int id, bool v) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 p, %1, 0;\n\t"
      "bar.red.and.pred q, %2, 128, p;\n\t"
      "selp.u32 %0, 1, 0, q;\n\t}\n"
      : "=r"(r)
      : "r"((uint32_t)v), "r"(id)
      : "memory");
  return r != 0;
}

// Forward of the MLP over tiles of 128 rows on the tensor cores.  Src
// provides, for row index i, `bool features(long long i, float (&x)[kIn])`
// (false: no row) and `void output(long long i, float y)`.  A block runs
// kGroups tile groups of 128 threads that share the staged weights: group g
// takes tiles kGroups * blockIdx.x + g, + kGroups * gridDim.x, ... with its
// own operand buffer, mbarrier, 64 accumulator columns and named barrier, so
// one group's epilogue overlaps the other's MMAs.  Thread r of a group owns
// row r of its tiles (TMEM lane r).  The features of the group's next tile
// are loaded while the current tile runs through the three layers.  Returns
// false when an mbarrier wait ran out (uniformly over the group).
template <class Src>
__device__ bool forward_tiles(const Net& net, Src& src, long long ntiles, uint8_t* smem) {
  uint8_t* sW1 = smem;
  uint8_t* sW2 = sW1 + kSmemW1;
  uint8_t* sW3 = sW2 + kSmemW;
  uint8_t* sA0 = sW3 + kSmemW;  // kGroups tile operands
  uint64_t* mbar0 = reinterpret_cast<uint64_t*>(sA0 + kGroups * kSmemA);  // one mbarrier per group
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar0 + kGroups);
  __shared__ float sb[3][kH];
  __shared__ float sw4[kH];
  __shared__ float sxm[kIn], sxi[kIn];
  const int t = threadIdx.x, warp = t >> 5;
  // tile group of this thread (its own tiles, operand, mbarrier, accumulator
  // columns and named barrier) and its row in the group's tiles
  const int grp = t / kTile, r = t % kTile, bar = 1 + grp;

  // weights (BF16, K-major: row = output unit, K = input).  Layer 1: its
  // bias as two BF16 columns (high and low part) against input columns 24-25
  // of ones.  Layers 2-4: weights halved (exact), since the epilogue returns
  // 2 gelu(z).
  for (int i = t; i < kH * kInPad; i += blockDim.x) {
    const int n = i / kInPad, k = i % kInPad;
    __nv_bfloat16 w = __float2bfloat16_rn(0.f);
    if (k < kIn) {
      w = net.pb[kOffW1 + n * kIn + k];
    } else if (k == kIn || k == kIn + 1) {
      const float b = net.p[kOffB1 + n];
      const __nv_bfloat16 hi = __float2bfloat16_rn(b);
      w = k == kIn ? hi : __float2bfloat16_rn(b - __bfloat162float(hi));
    }
    *reinterpret_cast<__nv_bfloat16*>(sW1 + core_off(n, k, kInPad)) = w;
  }
  for (int i = t; i < kH * kH; i += blockDim.x) {
    const int n = i / kH, k = i % kH;
    *reinterpret_cast<__nv_bfloat16*>(sW2 + core_off(n, k, kH)) = __hmul(net.pb[kOffW2 + i], __float2bfloat16_rn(0.5f));
    *reinterpret_cast<__nv_bfloat16*>(sW3 + core_off(n, k, kH)) = __hmul(net.pb[kOffW3 + i], __float2bfloat16_rn(0.5f));
  }
  for (int i = t; i < kH; i += blockDim.x) {
    sb[0][i] = net.p[kOffB1 + i];
    sb[1][i] = net.p[kOffB2 + i];
    sb[2][i] = net.p[kOffB3 + i];
    sw4[i] = 0.5f * __bfloat162float(net.pb[kOffW4 + i]);
  }
  for (int i = t; i < kIn; i += blockDim.x) {
    sxm[i] = net.xmean[i];
    sxi[i] = net.xinv[i];
  }
  const float b4 = net.p[kOffB4];
  const uint32_t mb = smem_u32(mbar0 + grp);
  if (r == 0) {
    mbar_init(mb, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(kH * kGroups)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_async_smem();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = *tslot + (uint32_t)(grp * kH);  // this group's accumulator columns
  const uint32_t tl = tmem + ((uint32_t)((warp & 3) * 32) << 16);  // this warp's lane quarter
  constexpr uint32_t kIdesc = idesc_bf16_f32(kTile, kH);
  uint8_t* sA = sA0 + grp * kSmemA;
  const uint32_t aA = smem_u32(sA), aW[3] = {smem_u32(sW1), smem_u32(sW2), smem_u32(sW3)};
  uint32_t phase = 0;
  bool ok = true;

  const long long stride = (long long)gridDim.x * kGroups;
  long long tile = (long long)blockIdx.x * kGroups + grp;
  float xn[kIn];
  bool vn = tile < ntiles ? src.features(tile * kTile + r, xn) : false;
  for (; tile < ntiles; tile += stride) {
    const long long row = tile * kTile + r;
    const bool valid = vn;
    const float dir = valid ? head_dir(net, xn) : 0.f;  // from the raw features, before the prefetch
    {
      float xs[kInPad];
#pragma unroll
      for (int k = 0; k < kIn; ++k) xs[k] = valid ? (xn[k] - sxm[k]) * sxi[k] : 0.f;
      xs[kIn] = 1.f;  // the two columns of ones that carry layer 1's bias
      xs[kIn + 1] = 1.f;
#pragma unroll
      for (int k = kIn + 2; k < kInPad; ++k) xs[k] = 0.f;
#pragma unroll
      for (int k0 = 0; k0 < kInPad; k0 += 8) store8_bf16(sA, r, k0, kInPad, xs + k0);
    }
    fence_async_smem();
    fence_before_sync();
    group_sync(bar);
    // the next tile's features, in flight during this tile's layers
    {
      const long long nt = tile + stride;
      vn = nt < ntiles ? src.features(nt * kTile + r, xn) : false;
    }
    float y = b4;
#pragma unroll 1
    for (int l = 0; l < 3; ++l) {
      const int K = l == 0 ? kInPad : kH;
      if (r == 0) {
        fence_after_sync();
        for (int k = 0; k < K / 16; ++k) {
          const uint64_t ad = smem_desc(aA + k * 256, 128, (uint32_t)(K / 8) * 128);
          const uint64_t bd = smem_desc(aW[l] + k * 256, 128, (uint32_t)(K / 8) * 128);
          mma_bf16(tmem, ad, bd, kIdesc, k > 0 ? 1u : 0u);
        }
        mma_commit(mb);
      }
      const bool got = mbar_wait(mb, phase, net.wait_polls);
      phase ^= 1u;
      ok = group_sync_and(bar, got);
      if (!ok) break;
      fence_after_sync();
#pragma unroll
      for (int half = 0; half < 2; ++half) {
        // 32 accumulator columns of this row: two loads, one wait
        const int c0 = 32 * half;
        float d0[16], d1[16];
        tmem_ld16(tl + c0, d0);
        tmem_ld16(tl + c0 + 16, d1);
        tmem_wait_ld();
        __nv_bfloat162 h[2][8];
        if (l == 0) {
          bias_gelu16<false>(d0, nullptr, h[0]);
          bias_gelu16<false>(d1, nullptr, h[1]);
        } else {
          bias_gelu16<true>(d0, sb[l] + c0, h[0]);
          bias_gelu16<true>(d1, sb[l] + c0 + 16, h[1]);
        }
        if (l < 2) {
#pragma unroll
          for (int q = 0; q < 2; ++q) {
            *reinterpret_cast<uint4*>(sA + core_off(r, c0 + 16 * q, kH)) = *reinterpret_cast<uint4*>(&h[q][0]);
            *reinterpret_cast<uint4*>(sA + core_off(r, c0 + 16 * q + 8, kH)) = *reinterpret_cast<uint4*>(&h[q][4]);
          }
        } else {
#pragma unroll
          for (int q = 0; q < 2; ++q)
#pragma unroll
            for (int j = 0; j < 8; ++j) {
              const float2 f = __bfloat1622float2(h[q][j]);
              y += f.x * sw4[c0 + 16 * q + 2 * j] + f.y * sw4[c0 + 16 * q + 2 * j + 1];
            }
        }
      }
      if (l < 2) fence_async_smem();
      fence_before_sync();
      group_sync(bar);
    }
    if (!ok) break;
    if (valid) src.output(row, head_out(net, y, dir));
  }
  // after a timed-out wait, the MMAs of that commit may still be running:
  // wait for them (bounded) before the columns are freed
  if (!ok) mbar_wait(mb, phase ^ 1u, kWaitPolls);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(*tslot), "r"(kH * kGroups) : "memory");
  return ok;
}

}  // namespace mlp
}  // namespace tmc
