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
// Every operand is stored once, row-major by tile row ([row][column] in
// 8 x 8 core matrices of 16-byte rows).  The forward and dH products read it
// K-major (K = its columns); the weight-gradient products, whose K is the
// tile's rows, read the same bytes MN-major (instruction-descriptor bits 15
// and 16): a core matrix of 8 rows x 8 columns is 8 K-rows of 8 contiguous
// M (or N) elements, and only the strides between core matrices change
// (mn_major below).  The dH products read W2 and W3 MN-major in the same way
// for their transposes.  The weight-gradient A operands have 64 (or 65)
// meaningful M rows out of the MMA's 128: the rows above are whatever lies in
// the shared memory that follows (never written by them, never read back
// from D).  The columns of ones give the bias gradients as one more column;
// D3's row 64 (dy) against H3 gives the output layer's weight gradient and,
// against the ones, its bias gradient.  The three D accumulators sum over all
// of the block's tiles; at the end each block writes its partial gradient and
// loss, which a second kernel sums in a fixed order (no atomics: the gradient
// does not depend on scheduling).
#pragma once

#include "tmc_mlp_tc.cuh"

namespace tmc {
namespace mlp {

constexpr int kTrTile = kTile;       // rows per tile
constexpr int kTrThreads = 512;      // threads per block: four per row, 16 hidden columns each
constexpr int kTrCG = kTrThreads / kTrTile;  // column groups
constexpr int kTrK = kTile;          // K of the weight-gradient products (rows)
constexpr int kTrN3 = 144;           // D3: 64 (H2) + 1 (ones) + 15 (zero) + 64 (H3)
constexpr int kTrN2 = 80;            // D2: 64 (H1) + 1 (ones) + 15 (zero)
constexpr int kTrN1 = kInPad;        // D1: 24 inputs, 2 ones (layer 1 bias hi/lo), 6 zero
constexpr int kTrH3Col = 80;         // first column of H3 in the H2 operand
constexpr int kTrWZ3 = 72;           // columns of the dZ3 operand: dZ3 (0..63), dy (64), 7 unused
// shared memory (bytes): the operands, row-major [rows][width], weights first
constexpr int kTrW1 = 0;                             // W1 [64 out][32 in]
constexpr int kTrW2 = kTrW1 + kSmemW1;               // W2 [64 out][64 in]
constexpr int kTrW3 = kTrW2 + kSmemW;                // W3 [64 out][64 in]
constexpr int kTrH2 = kTrW3 + kSmemW;                // [128][144]: H2, 1, 0, H3
constexpr int kTrH1 = kTrH2 + kTile * kTrN3 * 2;     // [128][80]: H1, 1, 0
constexpr int kTrX = kTrH1 + kTile * kTrN2 * 2;      // [128][32]: X, 1, 1, 0
constexpr int kTrDZ3 = kTrX + kTile * kTrN1 * 2;     // [128][72]: dZ3, dy, 7 unused
constexpr int kTrDZ2 = kTrDZ3 + kTile * kTrWZ3 * 2;  // [128][64]
constexpr int kTrDZ1 = kTrDZ2 + kTile * kH * 2;      // [128][64]
constexpr int kTrBar = kTrDZ1 + kTile * kH * 2;      // mbarrier (8 B) and the TMEM address (4 B)
// Furthest byte an MN-major read of the operand at `base` (width w columns,
// MN extent e, k16 steps of 16 K-rows) reaches: with the core-matrix strides
// as mn_major sets them (K: 16 w bytes per 8 rows; M or N: 128 bytes per 8
// columns), or with the two the other way round.  The weight-gradient A
// operands (M 128 of 64-72 columns) read past their own rows; the block's
// shared memory is sized so that every read stays inside it either way.
constexpr int tr_reach(int base, int w, int e, int k16) {
  const int kg = 16 * w, s = (k16 - 1) * 2 * kg;
  const int as_set = base + s + kg + (e / 8 - 1) * 128 + 128;
  const int swapped = base + s + (e / 8 - 1) * kg + 128 + 128;
  return as_set > swapped ? as_set : swapped;
}
constexpr int tr_max(int a, int b) { return a > b ? a : b; }
constexpr int kSmemTrain =
    tr_max(tr_max(tr_max(kTrBar + 16, tr_reach(kTrDZ3, kTrWZ3, 128, 8)),
                  tr_max(tr_reach(kTrDZ2, kH, 128, 8), tr_reach(kTrDZ1, kH, 128, 8))),
           tr_max(tr_max(tr_reach(kTrH2, kTrN3, kTrN3, 8), tr_reach(kTrH1, kTrN2, kTrN2, 8)),
                  tr_max(tr_reach(kTrX, kTrN1, kTrN1, 8), tr_reach(kTrW3, kH, kH, 4))));
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

// One operand of a product as the MMA descriptors see it: the start of its
// first K-step, the bytes between K-steps (16 K elements), and the two
// core-matrix strides (LBO along K, SBO along M or N).
struct Opnd {
  uint32_t a, step, lbo, sbo;
};
// row-major [rows][w] read K-major (K = its w columns, M or N = its rows)
__device__ __forceinline__ Opnd k_major(uint32_t a, int w) { return Opnd{a, 256u, 128u, (uint32_t)(w / 8) * 128u}; }
// row-major [rows][w] read MN-major (K = its rows, M or N = its columns):
// 8 K-rows of a core matrix are its 8 rows of 16 bytes
__device__ __forceinline__ Opnd mn_major(uint32_t a, int w) {
  const uint32_t kg = (uint32_t)(w / 8) * 128u;  // 8 rows
  return Opnd{a, 2u * kg, kg, 128u};
}
// instruction descriptor with MN-major A (bit 15) and / or B (bit 16)
__host__ __device__ constexpr uint32_t idesc_tr(int M, int N, bool a_mn, bool b_mn) {
  return idesc_bf16_f32(M, N) | (a_mn ? 1u << 15 : 0u) | (b_mn ? 1u << 16 : 0u);
}

// issue the K/16 MMAs of D = A B^T from one thread
__device__ __forceinline__ void mma_steps(uint32_t tmem_d, const Opnd& A, const Opnd& B, int K, uint32_t idesc,
                                          bool accumulate) {
  for (int k = 0; k < K / 16; ++k)
    mma_bf16(tmem_d, smem_desc(A.a + k * A.step, A.lbo, A.sbo), smem_desc(B.a + k * B.step, B.lbo, B.sbo), idesc,
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

// Src: `bool sample(long long i, int cg, float (&x)[8], float (&xd)[4], float& t)`:
// column group cg's part of row i of the batch (TrainSrc in tmc_mlp.cu).
// part: [gridDim.x][kParams] partial gradients, ploss: [gridDim.x].
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
  uint8_t* const sX = smem + kTrX;
  uint8_t* const sH1 = smem + kTrH1;
  uint8_t* const sH2 = smem + kTrH2;
  uint8_t* const sDZ3 = smem + kTrDZ3;
  uint8_t* const sDZ2 = smem + kTrDZ2;
  uint8_t* const sDZ1 = smem + kTrDZ1;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + kTrBar);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + kTrBar + 8);
  __shared__ float sb[3][kH], sw4[kH], sxm[kIn], sxi[kIn], sred[4];
  __shared__ float sy[kTrCG][kTile];  // the column groups' partial sums of the output
  const int t = threadIdx.x, warp = t >> 5, quarter = warp & 3, cg = warp >> 2;
  const int r = quarter * 32 + (t & 31);  // this thread's row of the tile (TMEM lane)
  const int cc = 16 * cg;                 // its first hidden column

  // weights (BF16) K-major by input; layer 1's bias as a high and a low BF16
  // part against the two input columns of ones
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
  // the constant columns of H1 and H2: ones at 64, zeros at 65..79
  for (int i = t; i < 16 * kTile; i += blockDim.x) {
    const int c = kH + i / kTile, row = i % kTile;
    const float v = c == kH ? 1.f : 0.f;
    st_bf16(sH2, row, c, kTrN3, v);
    st_bf16(sH1, row, c, kTrN2, v);
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
  const uint32_t aX = smem_u32(sX), aH1 = smem_u32(sH1), aH2 = smem_u32(sH2);
  const uint32_t aDZ3 = smem_u32(sDZ3), aDZ2 = smem_u32(sDZ2), aDZ1 = smem_u32(sDZ1);
  const uint32_t aW1 = smem_u32(smem + kTrW1), aW2 = smem_u32(smem + kTrW2), aW3 = smem_u32(smem + kTrW3);
  constexpr uint32_t kIdF = idesc_tr(kTile, kH, false, false);
  constexpr uint32_t kIdH = idesc_tr(kTile, kH, false, true);  // dH: W read MN-major as W^T
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

  // this thread's part of the row of the block's next tile, loaded while the
  // current one runs
  float xr[8], xd[4], tr = 0.f;
  bool vr = blockIdx.x < ntiles ? src.sample((long long)blockIdx.x * kTrTile + r, cg, xr, xd, tr) : false;
  for (long long tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    const float tgt = vr ? tr : 0.f;
    const float dir = vr ? head_dir4(net, xd[0], xd[1], xd[2], xd[3]) : 0.f;  // raw features
    {
      // the row's 32 input columns are 24 normalised features, 2 ones and 6
      // zeros; this thread stores columns 8 cg .. 8 cg + 7
      float v[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) v[k] = k < 2 ? 1.f : 0.f;  // column group 3
      if (cg < 3) {
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] = vr ? (xr[k] - sxm[8 * cg + k]) * sxi[8 * cg + k] : 0.f;
      }
      store8_bf16(sX, r, 8 * cg, kInPad, v);
    }
    publish();
    {
      const long long nt = tile + gridDim.x;
      vr = nt < ntiles ? src.sample(nt * kTrTile + r, cg, xr, xd, tr) : false;
    }
    // forward
#pragma unroll 1
    for (int l = 0; l < 3 && ok; ++l) {
      const int K = l == 0 ? kInPad : kH;
      const uint32_t zc = tmem + (uint32_t)(kTmZ1 + 64 * l);
      // A the previous layer K-major, B the weights K-major
      ok = run([&] {
        const Opnd A = l == 0 ? k_major(aX, kTrN1) : l == 1 ? k_major(aH1, kTrN2) : k_major(aH2, kTrN3);
        const Opnd B = l == 0 ? k_major(aW1, kInPad) : l == 1 ? k_major(aW2, kH) : k_major(aW3, kH);
        mma_steps(zc, A, B, K, kIdF, false);
      });
      if (!ok) break;
      float d[16];
      tmem_ld16(tl + (uint32_t)(kTmZ1 + 64 * l + cc), d);
      tmem_wait_ld();
      float h[16];
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const float z = l == 0 ? d[i] : d[i] + sb[l][cc + i];
        h[i] = __bfloat162float(__float2bfloat16_rn(gelu_f(z)));
      }
      // H1 -> sH1, H2 -> sH2 (columns 0..63), H3 -> sH2 (columns 80..143)
      uint8_t* const hb = l == 0 ? sH1 : sH2;
      const int hw = l == 0 ? kTrN2 : kTrN3, c0 = (l == 2 ? kTrH3Col : 0) + cc;
      store8_bf16(hb, r, c0, hw, h);
      store8_bf16(hb, r, c0 + 8, hw, h + 8);
      if (l == 2) {
        float yp = 0.f;
#pragma unroll
        for (int i = 0; i < 16; ++i) yp += sw4[cc + i] * h[i];
        sy[cg][r] = yp;
      }
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
      st_bf16(sDZ3, r, kH, kTrWZ3, dy);
    }
    // dZ3 = dy w4 gelu'(z3)
    {
      float d[16], g[16];
      tmem_ld16(tl + (uint32_t)(kTmZ3 + cc), d);
      tmem_wait_ld();
#pragma unroll
      for (int i = 0; i < 16; ++i) g[i] = dy * sw4[cc + i] * gelu_grad_f(d[i] + sb[2][cc + i]);
      store8_bf16(sDZ3, r, cc, kTrWZ3, g);
      store8_bf16(sDZ3, r, cc + 8, kTrWZ3, g + 8);
    }
    publish();
    if (t == 0) loss += (double)(sred[0] + sred[1] + sred[2] + sred[3]) * inv_batch;
    ok = run([&] {
      mma_steps(tmem + kTmZ3, k_major(aDZ3, kTrWZ3), mn_major(aW3, kH), kH, kIdH, false);
      mma_steps(tmem + kTmD3, mn_major(aDZ3, kTrWZ3), mn_major(aH2, kTrN3), kTrK, idesc_tr(kTile, kTrN3, true, true),
                !first);
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
        uint8_t* const gz = l == 1 ? sDZ2 : sDZ1;
        store8_bf16(gz, r, cc, kH, g);
        store8_bf16(gz, r, cc + 8, kH, g + 8);
      }
      publish();
      if (l == 1)
        ok = run([&] {
          mma_steps(tmem + kTmZ2, k_major(aDZ2, kH), mn_major(aW2, kH), kH, kIdH, false);
          mma_steps(tmem + kTmD2, mn_major(aDZ2, kH), mn_major(aH1, kTrN2), kTrK, idesc_tr(kTile, kTrN2, true, true),
                    !first);
        });
      else
        ok = run([&] {
          mma_steps(tmem + kTmD1, mn_major(aDZ1, kH), mn_major(aX, kTrN1), kTrK, idesc_tr(kTile, kTrN1, true, true),
                    !first);
        });
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
      tmem_ld16(tl + (uint32_t)(kTmD3 + kTrH3Col + cc), d);
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
