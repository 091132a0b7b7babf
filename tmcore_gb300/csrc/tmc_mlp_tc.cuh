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

// Bounded wait for the given phase parity; false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
  for (int i = 0; i < (1 << 20); ++i) {
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

// store 8 consecutive K values of one row (16 bytes) of a K-major operand
__device__ __forceinline__ void store8_bf16(uint8_t* base, int row, int k0, int K, const float* v) {
  __nv_bfloat162 h[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) h[i] = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
  *reinterpret_cast<uint4*>(base + core_off(row, k0, K)) = *reinterpret_cast<uint4*>(h);
}

// Forward of the MLP over tiles of 128 rows on the tensor cores.  Src
// provides, for row index i of the current tile, `bool features(long long i,
// float (&x)[kIn])` (false: no row) and `void output(long long i, float y)`.
// 128 threads; thread t owns row t of every tile (TMEM lane t).  Returns
// false (uniformly) when an mbarrier wait ran out.
template <class Src>
__device__ bool forward_tiles(const Net& net, Src& src, long long ntiles, uint8_t* smem) {
  uint8_t* sW1 = smem;
  uint8_t* sW2 = sW1 + kSmemW1;
  uint8_t* sW3 = sW2 + kSmemW;
  uint8_t* sA = sW3 + kSmemW;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sA + kSmemA);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(sA + kSmemA + 8);
  __shared__ float sb[3][kH];
  __shared__ float sw4[kH];
  __shared__ float sxm[kIn], sxi[kIn];
  const int t = threadIdx.x, warp = t >> 5;

  // weights (BF16, K-major: row = output unit, K = input) and biases
  for (int i = t; i < kH * kInPad; i += blockDim.x) {
    const int n = i / kInPad, k = i % kInPad;
    const __nv_bfloat16 w = k < kIn ? net.pb[kOffW1 + n * kIn + k] : __float2bfloat16_rn(0.f);
    *reinterpret_cast<__nv_bfloat16*>(sW1 + core_off(n, k, kInPad)) = w;
  }
  for (int i = t; i < kH * kH; i += blockDim.x) {
    const int n = i / kH, k = i % kH;
    *reinterpret_cast<__nv_bfloat16*>(sW2 + core_off(n, k, kH)) = net.pb[kOffW2 + i];
    *reinterpret_cast<__nv_bfloat16*>(sW3 + core_off(n, k, kH)) = net.pb[kOffW3 + i];
  }
  for (int i = t; i < kH; i += blockDim.x) {
    sb[0][i] = net.p[kOffB1 + i];
    sb[1][i] = net.p[kOffB2 + i];
    sb[2][i] = net.p[kOffB3 + i];
    sw4[i] = __bfloat162float(net.pb[kOffW4 + i]);
  }
  for (int i = t; i < kIn; i += blockDim.x) {
    sxm[i] = net.xmean[i];
    sxi[i] = net.xinv[i];
  }
  const float b4 = net.p[kOffB4];
  const uint32_t mb = smem_u32(mbar);
  if (t == 0) {
    mbar_init(mb, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(kH)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_async_smem();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t tl = tmem + ((uint32_t)(warp * 32) << 16);  // this warp's lane quarter
  constexpr uint32_t kIdesc = idesc_bf16_f32(kTile, kH);
  const uint32_t aA = smem_u32(sA), aW[3] = {smem_u32(sW1), smem_u32(sW2), smem_u32(sW3)};
  uint32_t phase = 0;
  bool ok = true;

  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long row = tile * kTile + t;
    float x[kIn];
    const bool valid = src.features(row, x);
    {
      float xs[kInPad];
#pragma unroll
      for (int k = 0; k < kIn; ++k) xs[k] = valid ? (x[k] - sxm[k]) * sxi[k] : 0.f;
#pragma unroll
      for (int k = kIn; k < kInPad; ++k) xs[k] = 0.f;
#pragma unroll
      for (int k0 = 0; k0 < kInPad; k0 += 8) store8_bf16(sA, t, k0, kInPad, xs + k0);
    }
    fence_async_smem();
    fence_before_sync();
    __syncthreads();
    float y = b4;
#pragma unroll 1
    for (int l = 0; l < 3; ++l) {
      const int K = l == 0 ? kInPad : kH;
      if (t == 0) {
        fence_after_sync();
        for (int k = 0; k < K / 16; ++k) {
          const uint64_t ad = smem_desc(aA + k * 256, 128, (uint32_t)(K / 8) * 128);
          const uint64_t bd = smem_desc(aW[l] + k * 256, 128, (uint32_t)(K / 8) * 128);
          mma_bf16(tmem, ad, bd, kIdesc, k > 0 ? 1u : 0u);
        }
        mma_commit(mb);
      }
      const bool got = mbar_wait(mb, phase);
      phase ^= 1u;
      ok = __syncthreads_and(got ? 1 : 0) != 0;
      if (!ok) break;
      fence_after_sync();
#pragma unroll
      for (int c = 0; c < kH; c += 16) {
        float d[16];
        tmem_ld16(tl + c, d);
        tmem_wait_ld();
        float h[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const float z = d[j] + sb[l][c + j];
          h[j] = gelu_tanh(z, tanh_fast(gelu_arg(z)));
        }
        if (l < 2) {
          store8_bf16(sA, t, c, kH, h);
          store8_bf16(sA, t, c + 8, kH, h + 8);
        } else {
#pragma unroll
          for (int j = 0; j < 16; ++j) y += h[j] * sw4[c + j];
        }
      }
      if (l < 2) fence_async_smem();
      fence_before_sync();
      __syncthreads();
    }
    if (!ok) break;
    if (valid) src.output(row, y * net.yscale);
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kH) : "memory");
  return ok;
}

}  // namespace mlp
}  // namespace tmc
