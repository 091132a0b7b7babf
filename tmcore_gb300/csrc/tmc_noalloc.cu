// tmc_mass_energy_noalloc: total mass and total energy of a shallow-water
// state from device arrays, for callers that must not allocate device memory.
//
// The per-block partial sums live in the file-scope array g_noalloc_partials
// below instead of memory from cudaMalloc.  The array is part of the library
// image: every GPU that loads the library holds it (TMC_NOALLOC_MAX_ELEMENTS
// bounds it to 3 regions x 8192 blocks x one double-double (hi, lo) block sum
// = 384 KiB) until the process exits.  Its device address is looked up once
// per device with cudaGetSymbolAddress on the first call made while that
// device is current, and cached; cudaDeviceReset on that device unloads the
// library's device image, so the cached address is stale afterwards and the
// entry point must not be called again on that device in the same process.
// Every call reuses the same array, and each call overwrites the entries it
// later reads, so nothing needs clearing; calls that overlap on the GPU
// (several streams, or several host threads on one device) race on it.
#include <cuda_runtime.h>

#include <mutex>

#include "tmc_kernels_impl.cuh"
#include "tmcore_gpu.h"

namespace {

using tmc::DD;
using tmc::dd_add;
using tmc::warp_reduce_dd;

constexpr int kThreads = 256;
constexpr int kPerThread = 4;
constexpr int kMaxBlocks = TMC_NOALLOC_MAX_ELEMENTS / (kThreads * kPerThread);
constexpr int kRegions = 3;  // mass, energy on cells, energy on edges

static __device__ __align__(256) double g_noalloc_partials[kRegions * kMaxBlocks * 2];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
double* g_scratch[kMaxDevices] = {};

// Compensated (double-double) sum of the block's per-thread sums, stored as
// the (hi, lo) pair of one slot.
__device__ __forceinline__ void store_block_sum(DD v, double* slot) {
  __shared__ DD sm[kThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_reduce_dd(v);
  if (lane == 0) sm[warp] = v;
  __syncthreads();
  if (warp == 0) {
    DD w = (lane < kThreads / 32) ? sm[lane] : DD{0.0, 0.0};
    w = warp_reduce_dd(w);
    if (lane == 0) {
      slot[0] = w.hi;
      slot[1] = w.lo;
    }
  }
  __syncthreads();
}

// cells: mass = sum gd*areaCell; energy part sum (gd^2 + 2 gd ghs)*areaCell
// (tmcore_swm_mod.F90:215-231)
__global__ void __launch_bounds__(kThreads) k_cells(const double* gd, const double* ghs, const double* area,
                                                    int64_t n, double* part) {
  DD m{0.0, 0.0}, e{0.0, 0.0};
  for (int k = 0; k < kPerThread; ++k) {
    const int64_t i = (int64_t)blockIdx.x * (kThreads * kPerThread) + (int64_t)k * kThreads + threadIdx.x;
    if (i < n) {
      const double g = gd[i], a = area[i];
      m = dd_add(m, DD{g * a, 0.0});
      e = dd_add(e, DD{(g * g + 2.0 * g * ghs[i]) * a, 0.0});
    }
  }
  store_block_sum(m, part + 2 * (0 * kMaxBlocks + blockIdx.x));
  store_block_sum(e, part + 2 * (1 * kMaxBlocks + blockIdx.x));
}

// edges: energy part sum iap_u^2 * areaEdge
__global__ void __launch_bounds__(kThreads) k_edges(const double* iap, const double* area, int64_t n, double* part) {
  DD e{0.0, 0.0};
  for (int k = 0; k < kPerThread; ++k) {
    const int64_t i = (int64_t)blockIdx.x * (kThreads * kPerThread) + (int64_t)k * kThreads + threadIdx.x;
    if (i < n) e = dd_add(e, DD{iap[i] * iap[i] * area[i], 0.0});
  }
  store_block_sum(e, part + 2 * (2 * kMaxBlocks + blockIdx.x));
}

// one block per region, double-double over the block sums; out = {mass, energy}
__global__ void __launch_bounds__(kThreads) k_final(const double* part, int nb_cells, int nb_edges, double* out) {
  __shared__ double res[kRegions];
  for (int r = 0; r < kRegions; ++r) {
    const int nb = (r < 2) ? nb_cells : nb_edges;
    DD acc{0.0, 0.0};
    for (int b = threadIdx.x; b < nb; b += kThreads)
      acc = dd_add(acc, DD{part[2 * (r * kMaxBlocks + b)], part[2 * (r * kMaxBlocks + b) + 1]});
    __shared__ DD sm[kThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    DD w = warp_reduce_dd(acc);
    if (lane == 0) sm[warp] = w;
    __syncthreads();
    if (warp == 0) {
      w = (lane < kThreads / 32) ? sm[lane] : DD{0.0, 0.0};
      w = warp_reduce_dd(w);
      if (lane == 0) res[r] = w.hi + w.lo;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = res[0];
    out[1] = res[2] + res[1];
  }
}

}  // namespace

extern "C" int tmc_mass_energy_noalloc(const double* gd, const double* ghs, const double* areaCell, int64_t nCells,
                                       const double* iap_u, const double* areaEdge, int64_t nEdges, double* out,
                                       void* stream) {
  if (!gd || !ghs || !areaCell || !iap_u || !areaEdge || !out) return TMC_E_ARG;
  if (nCells <= 0 || nEdges <= 0 || nCells > TMC_NOALLOC_MAX_ELEMENTS || nEdges > TMC_NOALLOC_MAX_ELEMENTS)
    return TMC_E_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return TMC_E_CUDA;
  }
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_partials) != cudaSuccess || !p) {
        cudaGetLastError();
        return TMC_E_CUDA;
      }
      g_scratch[dev] = static_cast<double*>(p);
    }
    scratch = g_scratch[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int per_block = kThreads * kPerThread;
  const int nbc = (int)((nCells + per_block - 1) / per_block), nbe = (int)((nEdges + per_block - 1) / per_block);
  k_cells<<<nbc, kThreads, 0, st>>>(gd, ghs, areaCell, nCells, scratch);
  k_edges<<<nbe, kThreads, 0, st>>>(iap_u, areaEdge, nEdges, scratch);
  k_final<<<1, kThreads, 0, st>>>(scratch, nbc, nbe, out);
  if (cudaGetLastError() != cudaSuccess) return TMC_E_CUDA;
  return TMC_OK;
}
