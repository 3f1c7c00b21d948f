// kernels_sort.cu -- track binning for warp coherence.
//
// A one-thread-per-track BVH traversal wastes most of every warp when the 32
// tracks of a warp start at unrelated positions and go in unrelated
// directions.  Before a step, tracks are counting-sorted by
//     key = direction octant (3 bits) | Morton order of a 2^k-per-axis cell
//           of the world bounding box (3k bits)
// and the step kernel visits them through the resulting permutation.  Each
// track's result is written back at its own index, so the order only changes
// which tracks share a warp, never any result.
#include <cuda_runtime.h>

#include <cstdint>

#include "launch.h"

namespace vgn {
namespace dev {

__device__ __forceinline__ uint32_t spread3(uint32_t v)  // 10 bits -> every third bit
{
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

__global__ void __launch_bounds__(256) bin_keys_kernel(int64_t n, const double *__restrict__ px,
                                                       const double *__restrict__ py, const double *__restrict__ pz,
                                                       const double *__restrict__ dx, const double *__restrict__ dy,
                                                       const double *__restrict__ dz, BinParams b,
                                                       uint32_t *__restrict__ keys, uint32_t *__restrict__ hist)
{
  const uint32_t cmax = (1u << b.kbits) - 1u;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float fx = ((float)px[i] - b.lo[0]) * b.scale[0];
    const float fy = ((float)py[i] - b.lo[1]) * b.scale[1];
    const float fz = ((float)pz[i] - b.lo[2]) * b.scale[2];
    const uint32_t cx = (uint32_t)fminf(fmaxf(fx, 0.f), (float)cmax);
    const uint32_t cy = (uint32_t)fminf(fmaxf(fy, 0.f), (float)cmax);
    const uint32_t cz = (uint32_t)fminf(fmaxf(fz, 0.f), (float)cmax);
    // directions are read only for the octant split (a position-only order never touches them)
    const uint32_t oct =
        b.octants ? ((dx[i] > 0.0 ? 4u : 0u) | (dy[i] > 0.0 ? 2u : 0u) | (dz[i] > 0.0 ? 1u : 0u)) : 0u;
    const uint32_t key = (oct << (3 * b.kbits)) | (spread3(cx) << 2) | (spread3(cy) << 1) | spread3(cz);
    keys[i]            = key;
    atomicAdd(hist + key, 1u);
  }
}

// exclusive scan of the histogram in place (one block)
__global__ void __launch_bounds__(1024) scan_kernel(uint32_t *hist, uint32_t nbins)
{
  __shared__ uint32_t part[1024];
  const uint32_t t     = threadIdx.x;
  const uint32_t chunk = (nbins + 1023u) / 1024u;
  const uint32_t beg = t * chunk, end = min(beg + chunk, nbins);
  uint32_t s = 0;
  for (uint32_t k = beg; k < end; ++k) s += hist[k];
  part[t] = s;
  __syncthreads();
  for (uint32_t off = 1; off < 1024u; off <<= 1) {  // inclusive Hillis-Steele scan of the partial sums
    const uint32_t v = t >= off ? part[t - off] : 0u;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  uint32_t run = part[t] - s;
  for (uint32_t k = beg; k < end; ++k) {
    const uint32_t h = hist[k];
    hist[k]          = run;
    run += h;
  }
}

// Exclusive scan of the histogram in three coalesced passes over 4096-bin tiles: per-tile
// sums, an in-place scan of the tile sums (scan_kernel, at most 512 of them), then each
// tile's own scan offset by its prefix.  Thread t of a block owns bins 4t..4t+3 of the tile.
constexpr uint32_t kScanTile = 4096;
static_assert((8u << 18) / kScanTile <= 512, "tile sums of the largest histogram fit kScanSumWords");

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *total)
{
  __shared__ uint32_t warp_sums[32];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {  // inclusive scan within the warp
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
    if (lane >= (uint32_t)off) x += y;
  }
  if (lane == 31u) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = warp_sums[lane];
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, off);
      if (lane >= (uint32_t)off) w += y;
    }
    warp_sums[lane] = w;  // inclusive over warps
  }
  __syncthreads();
  const uint32_t before = warp ? warp_sums[warp - 1] : 0u;
  if (total) *total = warp_sums[31];
  return before + x - v;
}

__global__ void __launch_bounds__(1024) tile_sum_kernel(const uint32_t *__restrict__ hist, uint32_t nbins,
                                                        uint32_t *__restrict__ sums)
{
  const uint32_t b = blockIdx.x * kScanTile + 4u * threadIdx.x;
  uint32_t s = 0;
#pragma unroll
  for (uint32_t k = 0; k < 4; ++k)
    if (b + k < nbins) s += hist[b + k];
  uint32_t total = 0;
  block_exclusive_scan(s, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) tile_scan_kernel(uint32_t *__restrict__ hist, uint32_t nbins,
                                                         const uint32_t *__restrict__ prefix)
{
  const uint32_t b = blockIdx.x * kScanTile + 4u * threadIdx.x;
  uint32_t v[4];
  uint32_t s = 0;
#pragma unroll
  for (uint32_t k = 0; k < 4; ++k) {
    v[k] = b + k < nbins ? hist[b + k] : 0u;
    s += v[k];
  }
  uint32_t run = prefix[blockIdx.x] + block_exclusive_scan(s, nullptr);
#pragma unroll
  for (uint32_t k = 0; k < 4; ++k) {
    if (b + k < nbins) hist[b + k] = run;
    run += v[k];
  }
}

__global__ void __launch_bounds__(256) scatter_kernel(int64_t n, const uint32_t *__restrict__ keys,
                                                      uint32_t *__restrict__ cursor, uint32_t *__restrict__ perm)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    perm[atomicAdd(cursor + keys[i], 1u)] = (uint32_t)i;
}

}  // namespace dev

// keys [n] | histogram [8 * 2^(3k)] | tile sums [512] | spare [n]
size_t bin_scratch_words(int64_t n, int kbits) { return 2 * (size_t)n + ((size_t)8 << (3 * kbits)) + kScanSumWords; }

// ---- fixed device scratch of vgn_compute_step_batch_static ----------------
// keys [n] | histogram [8 * 2^(3k)] | tile sums [512] | visit permutation [n], at the largest
// n and k the entry point accepts: 2 * 2^20 + 2^18 + 512 words = 9 MiB per device.
static constexpr size_t kStaticScratchWords =
    2 * (size_t)VGN_STATIC_SCRATCH_MAX_TRACKS + ((size_t)8 << (3 * VGN_STATIC_SCRATCH_MAX_KBITS)) + kScanSumWords;
static __device__ __align__(256) uint32_t g_static_scratch[kStaticScratchWords];

size_t static_scratch_words() { return kStaticScratchWords; }

// Address of the buffer in the current context, looked up on every call (no allocation): an
// address kept from an earlier call would go stale after cudaDeviceReset or in another
// context on the same device.
cudaError_t static_scratch(uint32_t **ptr)
{
  void *p             = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
  if (e != cudaSuccess) return e;
  *ptr = static_cast<uint32_t *>(p);
  return cudaSuccess;
}

cudaError_t launch_bin_tracks(int64_t n, const double *px, const double *py, const double *pz, const double *dx,
                              const double *dy, const double *dz, const BinParams &b, uint32_t *scratch,
                              uint32_t *perm, int max_blocks, cudaStream_t s)
{
  const uint32_t nbins = (b.octants ? 8u : 1u) << (3 * b.kbits);
  uint32_t *keys = scratch, *hist = scratch + n;
  cudaError_t e  = cudaMemsetAsync(hist, 0, nbins * sizeof(uint32_t), s);
  if (e != cudaSuccess) return e;
  int64_t blocks = (n + 255) / 256;
  if (blocks > max_blocks) blocks = max_blocks;
  if (blocks < 1) blocks = 1;
  dev::bin_keys_kernel<<<(unsigned)blocks, 256, 0, s>>>(n, px, py, pz, dx, dy, dz, b, keys, hist);
  const uint32_t tiles = (nbins + dev::kScanTile - 1) / dev::kScanTile;  // <= kScanSumWords for kbits <= 6
  uint32_t *sums       = hist + ((size_t)8 << (3 * b.kbits));
  dev::tile_sum_kernel<<<tiles, 1024, 0, s>>>(hist, nbins, sums);
  dev::scan_kernel<<<1, 1024, 0, s>>>(sums, tiles);
  dev::tile_scan_kernel<<<tiles, 1024, 0, s>>>(hist, nbins, sums);
  dev::scatter_kernel<<<(unsigned)blocks, 256, 0, s>>>(n, keys, hist, perm);
  return cudaGetLastError();
}

}  // namespace vgn
