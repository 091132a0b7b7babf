// Training step of the closure MLP on the tensor cores (tcgen05, inline PTX):
// the forward and the backward of one batch in one kernel, BF16 operands in
// shared memory, FP32 accumulators in tensor memory.
//
// A block of 512 threads takes tiles of 128 rows in turn, four threads per
// row (row r = TMEM lane r), each with 16 of the 64 hidden columns.  Per tile:
//   forward   Z_l = H_{l-1} W_l^T       (M 128, N 64, K 32/64), Z_l kept in TMEM
//   output    y = b4 + w4 . h3,  dy = 2 (p(y) - t) p'(y) / batch with p the
//             output head (p(y) = y for kHeadPlain)
//   backward  dZ3 = dy w4 * gelu'(z3)
//             dH2 = dZ3 W3              (M 128, N 64, K 64) into Z3's columns
//             dZ2 = dH2 * gelu'(z2),    dH1 = dZ2 W2 into Z2's columns
//             dZ1 = dH1 * gelu'(z1)
//   weights   D3 += [dZ3^T; dy] [H2^T; 1; 0; H3^T]^T   (M 128, N 144, K 128 rows)
//             D2 += dZ2^T [H1^T; 1; 0]^T               (M 128, N 80,  K 128)
//             D1 += dZ1^T X^T^T                        (M 128, N 32,  K 128)
// The weight-gradient products run over the tile's rows as K, so every
// operand is stored a second time transposed (row index along K).  Their
// A operands have 64 (or 65) meaningful rows out of the MMA's 128: the rows
// above are whatever lies in the shared memory that follows (never written by
// them, never read back from D).  The rows of ones in the B operands give the
// bias gradients as one more column; D3's row 64 (dy) against H3^T gives the
// output layer's weight gradient and, against the ones, its bias gradient.
// The three D accumulators sum over all of the block's tiles; at the end each
// block writes its partial gradient and loss, which a second kernel sums in a
// fixed order (no atomics: the gradient does not depend on scheduling).
#pragma once

#include "tmc_mlp_tc.cuh"

namespace tmc {
namespace mlp {

constexpr int kTrTile = kTile;       // rows per tile
constexpr int kTrThreads = 512;      // threads per block: four per row, 16 hidden columns each
constexpr int kTrCG = kTrThreads / kTrTile;  // column groups
constexpr int kTrK = kTile;          // K of the weight-gradient products (rows)
constexpr int kTrN3 = 144;           // D3: 64 (H2^T) + 1 (ones) + 15 (zero) + 64 (H3^T)
constexpr int kTrN2 = 80;            // D2: 64 (H1^T) + 1 (ones) + 15 (zero)
constexpr int kTrN1 = kInPad;        // D1: 24 inputs, 2 ones (layer 1 bias hi/lo), 6 zero
constexpr int kTrH3Row = 80;         // first row of H3^T in the D3 B operand
// shared memory (bytes): transposed A operands first, since their unused
// rows run on into whatever follows them
constexpr int kTrAT3 = 0;                        // 9 row groups: dZ3^T (0..63), dy (64)
constexpr int kTrAT2 = kTrAT3 + 9 * 2048;        // dZ2^T
constexpr int kTrAT1 = kTrAT2 + 8 * 2048;        // dZ1^T
constexpr int kTrB3 = kTrAT1 + 8 * 2048;         // [H2^T; 1; 0; H3^T], 144 x 128
constexpr int kTrB2 = kTrB3 + kTrN3 * kTrK * 2;  // [H1^T; 1; 0], 80 x 128
constexpr int kTrXT = kTrB2 + kTrN2 * kTrK * 2;  // X^T (with its columns of ones), 32 x 128
constexpr int kTrA = kTrXT + kTrN1 * kTrK * 2;   // row-major operand: X, H1, H2, then dZ3, dZ2 (128 x 64)
constexpr int kTrW1 = kTrA + kTile * kH * 2;     // W1 [64 out][32 in]
constexpr int kTrW2 = kTrW1 + kSmemW1;           // W2 [64 out][64 in]
constexpr int kTrW3 = kTrW2 + kSmemW;
constexpr int kTrW2T = kTrW3 + kSmemW;           // W2^T [64 in][64 out]
constexpr int kTrW3T = kTrW2T + kSmemW;
constexpr int kTrBar = kTrW3T + kSmemW;          // mbarrier (8 B) and the TMEM address (4 B)
constexpr int kSmemTrain = kTrBar + 16;
// the last A operand's unused rows (16 KB past its start + 16 KB) stay inside
static_assert(kTrAT1 + 2 * 8 * 2048 <= kSmemTrain, "A operand rows run past shared memory");
static_assert(kSmemTrain <= 227 * 1024, "training tile does not fit in shared memory");
// TMEM columns: the three pre-activations (then the dH), and the three
// weight-gradient accumulators
constexpr int kTmZ1 = 0, kTmZ2 = 64, kTmZ3 = 128, kTmD3 = 192, kTmD2 = 352, kTmD1 = 448;
constexpr int kTmCols = 512;
static_assert(kTmD3 + kTrN3 <= kTmD2 && kTmD2 + kTrN2 <= kTmD1 && kTmD1 + kTrN1 <= kTmCols, "TMEM columns overlap");

__device__ __forceinline__ float gelu_f(float z) { return gelu_tanh(z, tanh_fast(gelu_arg(z))); }
__device__ __forceinline__ float gelu_grad_f(float z) {
  const float c = 0.7978845608028654f;
  const float th = tanh_fast(gelu_arg(z));
  return 0.5f * (1.f + th) + 0.5f * z * (1.f - th * th) * c * (1.f + 3.f * 0.044715f * z * z);
}

// one BF16 value at (row n, column k) of a K-major operand with K columns
__device__ __forceinline__ void st_bf16(uint8_t* base, int n, int k, int K, float v) {
  *reinterpret_cast<__nv_bfloat16*>(base + core_off(n, k, K)) = __float2bfloat16_rn(v);
}

// issue the K/16 MMAs of D = A B^T (both K-major, K columns) from one thread
__device__ __forceinline__ void mma_kloop(uint32_t tmem_d, uint32_t a, uint32_t b, int K, uint32_t idesc,
                                          bool accumulate) {
  const uint32_t sbo = (uint32_t)(K / 8) * 128;
  for (int k = 0; k < K / 16; ++k)
    mma_bf16(tmem_d, smem_desc(a + k * 256, 128, sbo), smem_desc(b + k * 256, 128, sbo), idesc,
             (accumulate || k > 0) ? 1u : 0u);
}

// the block's partial gradient from one 64-row accumulator: row m (TMEM lane
// m) holds out-unit m; columns 0..nin-1 the weights, column cb the bias.
// Loads start at multiples of 16 columns; column group cg takes the chunks
// cg, cg + 4, ...
__device__ __forceinline__ void store_dw(uint32_t tl, int m, int cg, int nin, int cb, float* gW, float* gb) {
  const int ncol = (nin > cb ? nin : cb + 1);
  for (int c0 = 16 * cg; c0 < ncol; c0 += 16 * kTrCG) {
    float d[16];
    tmem_ld16(tl + c0, d);
    tmem_wait_ld();
    if (m < kH) {
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        if (c0 + i < nin) gW[m * nin + c0 + i] = d[i];
        if (c0 + i == cb) gb[m] = d[i];
      }
    }
  }
}

// Src: `bool sample(long long i, float (&x)[kIn], float& t)` for row i of the
// batch.  part: [gridDim.x][kParams] partial gradients, ploss: [gridDim.x].
//
// Threads: kTrThreads = 512, four warps per TMEM lane quarter.  Warp w reads
// lane quarter w % 4, so thread t owns row r = 32 (w % 4) + (t % 32) of the
// tile (TMEM lane r) and, with the three other warps of its quarter, splits
// that row's 64 hidden columns: column group cg = w / 4 takes columns
// 16 cg .. 16 cg + 15 of every epilogue (and input columns 8 cg .. 8 cg + 7).
// Each SM sub-partition then has four warps to interleave through the
// epilogues' dependent bias / GELU / BF16 / store chains instead of one.
template <class Src>
__device__ bool train_tiles(const Net& net, const Src& src, long long ntiles, float inv_batch, float* part,
                            double* ploss, uint8_t* smem) {
  uint8_t* const sA = smem + kTrA;
  uint8_t* const sXT = smem + kTrXT;
  uint8_t* const sB2 = smem + kTrB2;
  uint8_t* const sB3 = smem + kTrB3;
  uint8_t* const sAT[3] = {smem + kTrAT1, smem + kTrAT2, smem + kTrAT3};
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + kTrBar);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + kTrBar + 8);
  __shared__ float sb[3][kH], sw4[kH], sxm[kIn], sxi[kIn], sred[4];
  __shared__ float sy[kTrCG][kTile];  // the column groups' partial sums of the output
  const int t = threadIdx.x, warp = t >> 5, quarter = warp & 3, cg = warp >> 2;
  const int r = quarter * 32 + (t & 31);  // this thread's row of the tile (TMEM lane)
  const int cc = 16 * cg;                 // its first hidden column

  // weights (BF16): forward operands K-major by input, backward operands
  // (W^T) K-major by output; layer 1's bias as a high and a low BF16 part
  // against the two input columns of ones
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
    *reinterpret_cast<__nv_bfloat16*>(smem + kTrW1 + core_off(n, k, kInPad)) = w;
  }
  for (int i = t; i < kH * kH; i += blockDim.x) {
    const int n = i / kH, k = i % kH;
    *reinterpret_cast<__nv_bfloat16*>(smem + kTrW2 + core_off(n, k, kH)) = net.pb[kOffW2 + i];
    *reinterpret_cast<__nv_bfloat16*>(smem + kTrW3 + core_off(n, k, kH)) = net.pb[kOffW3 + i];
    *reinterpret_cast<__nv_bfloat16*>(smem + kTrW2T + core_off(k, n, kH)) = net.pb[kOffW2 + i];
    *reinterpret_cast<__nv_bfloat16*>(smem + kTrW3T + core_off(k, n, kH)) = net.pb[kOffW3 + i];
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
  // the constant rows of the B operands: ones at row 64, zeros at 65..79
  for (int i = t; i < 16 * kTrK; i += blockDim.x) {
    const int n = kH + i / kTrK, k = i % kTrK;
    const float v = n == kH ? 1.f : 0.f;
    st_bf16(sB3, n, k, kTrK, v);
    st_bf16(sB2, n, k, kTrK, v);
  }
  const float b4 = net.p[kOffB4];
  const uint32_t mb = smem_u32(mbar);
  if (t == 0) {
    mbar_init(mb, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(kTmCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_async_smem();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t tl = tmem + ((uint32_t)(quarter * 32) << 16);  // this warp's lane quarter
  const uint32_t aA = smem_u32(sA), aXT = smem_u32(sXT), aB2 = smem_u32(sB2), aB3 = smem_u32(sB3);
  const uint32_t aAT1 = smem_u32(sAT[0]), aAT2 = smem_u32(sAT[1]), aAT3 = smem_u32(sAT[2]);
  const uint32_t aW[3] = {smem_u32(smem + kTrW1), smem_u32(smem + kTrW2), smem_u32(smem + kTrW3)};
  const uint32_t aWT2 = smem_u32(smem + kTrW2T), aWT3 = smem_u32(smem + kTrW3T);
  constexpr uint32_t kIdF = idesc_bf16_f32(kTile, kH);
  uint32_t phase = 0;
  bool ok = true;
  double loss = 0.0;
  bool first = true;  // no accumulation into D yet

  // issue (thread 0), commit, and wait for the MMAs of one step
  auto run = [&](auto issue) -> bool {
    if (t == 0) {
      fence_after_sync();
      issue();
      mma_commit(mb);
    }
    const bool got = mbar_wait(mb, phase, net.wait_polls);
    phase ^= 1u;
    const bool all = __syncthreads_and(got) != 0;
    fence_after_sync();
    return all;
  };
  // make this thread's shared-memory operand writes and TMEM reads visible
  // before the next MMA
  auto publish = [&]() {
    fence_async_smem();
    fence_before_sync();
    __syncthreads();
  };

  // the row of the block's next tile, loaded while the current one runs
  float xr[kIn], tr = 0.f;
  bool vr = blockIdx.x < ntiles ? src.sample((long long)blockIdx.x * kTrTile + r, xr, tr) : false;
  for (long long tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    const float tgt = vr ? tr : 0.f;
    const float dir = vr ? head_dir(net, xr) : 0.f;  // from the raw features, before the prefetch
    {
      // the 32 input columns of the row (24 normalised features, 2 ones, 6
      // zeros); this thread stores columns 8 cg .. 8 cg + 7
      float xs[kInPad];
#pragma unroll
      for (int k = 0; k < kIn; ++k) xs[k] = vr ? (xr[k] - sxm[k]) * sxi[k] : 0.f;
      xs[kIn] = xs[kIn + 1] = 1.f;
#pragma unroll
      for (int k = kIn + 2; k < kInPad; ++k) xs[k] = 0.f;
      float v[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) v[k] = cg == 0 ? xs[k] : cg == 1 ? xs[8 + k] : cg == 2 ? xs[16 + k] : xs[24 + k];
      store8_bf16(sA, r, 8 * cg, kInPad, v);
#pragma unroll
      for (int k = 0; k < 8; ++k) st_bf16(sXT, 8 * cg + k, r, kTrK, v[k]);
    }
    publish();
    {
      const long long nt = tile + gridDim.x;
      vr = nt < ntiles ? src.sample(nt * kTrTile + r, xr, tr) : false;
    }
    // forward
#pragma unroll 1
    for (int l = 0; l < 3 && ok; ++l) {
      const int K = l == 0 ? kInPad : kH;
      const uint32_t zc = tmem + (uint32_t)(kTmZ1 + 64 * l);
      ok = run([&] { mma_kloop(zc, aA, aW[l], K, kIdF, false); });
      if (!ok) break;
      // B operand rows of this layer's transposed activations
      uint8_t* const hT = l == 0 ? sB2 : sB3;
      const int n0 = l == 2 ? kTrH3Row : 0;
      float d[16];
      tmem_ld16(tl + (uint32_t)(kTmZ1 + 64 * l + cc), d);
      tmem_wait_ld();
      float h[16];
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const float z = l == 0 ? d[i] : d[i] + sb[l][cc + i];
        h[i] = __bfloat162float(__float2bfloat16_rn(gelu_f(z)));
      }
      if (l < 2) {
        store8_bf16(sA, r, cc, kH, h);
        store8_bf16(sA, r, cc + 8, kH, h + 8);
      } else {
        float yp = 0.f;
#pragma unroll
        for (int i = 0; i < 16; ++i) yp += sw4[cc + i] * h[i];
        sy[cg][r] = yp;
      }
#pragma unroll
      for (int i = 0; i < 16; ++i) st_bf16(hT, n0 + cc + i, r, kTrK, h[i]);
      publish();
    }
    if (!ok) break;
    // output head and loss (every thread of the row forms the same y)
    const float y = b4 + sy[0][r] + sy[1][r] + sy[2][r] + sy[3][r];
    float dpred;
    const float e = head_pred(net, y, dir, dpred) - tgt;
    const float dy = 2.f * e * inv_batch * dpred;
    if (cg == 0) {
      float le = e * e;
      for (int off = 16; off > 0; off >>= 1) le += __shfl_down_sync(0xffffffffu, le, off);
      if ((t & 31) == 0) sred[quarter] = le;
      st_bf16(sAT[2], kH, r, kTrK, dy);
    }
    // dZ3 = dy w4 gelu'(z3): row-major into sA (for dH2), transposed into AT3
    {
      float d[16], g[16];
      tmem_ld16(tl + (uint32_t)(kTmZ3 + cc), d);
      tmem_wait_ld();
#pragma unroll
      for (int i = 0; i < 16; ++i) g[i] = dy * sw4[cc + i] * gelu_grad_f(d[i] + sb[2][cc + i]);
      store8_bf16(sA, r, cc, kH, g);
      store8_bf16(sA, r, cc + 8, kH, g + 8);
#pragma unroll
      for (int i = 0; i < 16; ++i) st_bf16(sAT[2], cc + i, r, kTrK, g[i]);
    }
    publish();
    if (t == 0) loss += (double)(sred[0] + sred[1] + sred[2] + sred[3]) * inv_batch;
    ok = run([&] {
      mma_kloop(tmem + kTmZ3, aA, aWT3, kH, kIdF, false);
      mma_kloop(tmem + kTmD3, aAT3, aB3, kTrK, idesc_bf16_f32(kTile, kTrN3), !first);
    });
    if (!ok) break;
    // dZ2 = dH2 gelu'(z2), dZ1 = dH1 gelu'(z1)
#pragma unroll 1
    for (int l = 1; l >= 0 && ok; --l) {
      const uint32_t dh = (uint32_t)(kTmZ1 + 64 * (l + 1)), zc = (uint32_t)(kTmZ1 + 64 * l);
      {
        float d[16], z[16], g[16];
        tmem_ld16(tl + dh + cc, d);
        tmem_ld16(tl + zc + cc, z);
        tmem_wait_ld();
#pragma unroll
        for (int i = 0; i < 16; ++i) g[i] = d[i] * gelu_grad_f(l == 0 ? z[i] : z[i] + sb[l][cc + i]);
        if (l == 1) {
          store8_bf16(sA, r, cc, kH, g);
          store8_bf16(sA, r, cc + 8, kH, g + 8);
        }
#pragma unroll
        for (int i = 0; i < 16; ++i) st_bf16(sAT[l], cc + i, r, kTrK, g[i]);
      }
      publish();
      if (l == 1)
        ok = run([&] {
          mma_kloop(tmem + kTmZ2, aA, aWT2, kH, kIdF, false);
          mma_kloop(tmem + kTmD2, aAT2, aB2, kTrK, idesc_bf16_f32(kTile, kTrN2), !first);
        });
      else
        ok = run([&] { mma_kloop(tmem + kTmD1, aAT1, aXT, kTrK, idesc_bf16_f32(kTile, kTrN1), !first); });
    }
    first = false;
  }
  // the block's partial gradient (zeros when it had no tile) and loss
  float* const g = part + (size_t)blockIdx.x * kParams;
  if (ok && !first) {
    store_dw(tl + kTmD3, r, cg, kH, kH, g + kOffW3, g + kOffB3);
    store_dw(tl + kTmD2, r, cg, kH, kH, g + kOffW2, g + kOffB2);
    store_dw(tl + kTmD1, r, cg, kIn, kIn, g + kOffW1, g + kOffB1);
    // D3 row 64 (lane 0 of quarter 2): the output layer, 16 columns per group
    {
      float d[16];
      tmem_ld16(tl + (uint32_t)(kTmD3 + kTrH3Row + cc), d);
      tmem_wait_ld();
      if (r == kH)
#pragma unroll
        for (int i = 0; i < 16; ++i) g[kOffW4 + cc + i] = d[i];
    }
    if (cg == 0) {
      float d[16];
      tmem_ld16(tl + (uint32_t)(kTmD3 + kH), d);  // column 64: the ones
      tmem_wait_ld();
      if (r == kH) g[kOffB4] = d[0];
    }
  } else {
    for (int i = t; i < kParams; i += blockDim.x) g[i] = 0.f;
  }
  if (t == 0) ploss[blockIdx.x] = loss;
  // after a timed-out wait, the MMAs of that commit may still be running:
  // wait for them (bounded) before the columns are freed
  if (!ok) mbar_wait(mb, phase ^ 1u, kWaitPolls);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmCols) : "memory");
  return ok;
}

}  // namespace mlp
}  // namespace tmc
