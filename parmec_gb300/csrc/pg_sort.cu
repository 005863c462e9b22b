// pg_sort.cu -- Morton cell keys and a stable LSD radix sort of (key, index).
//
// Used by the session's candidate-list rebuild and by the public
// pg_cell_order entry point (the replacement of partitioning_create,
// partition.ispc:663-746, whose Morton codes quantise each coordinate to 10
// bits, partition.ispc:58-94).  Every kernel takes an optional 'gate': when it
// points at zero the kernel returns at once (used to enqueue a rebuild every
// step but run it only when it is due).
#include <cuda_runtime.h>
#include <cmath>
#include "pg_launch.h"
#include "pg_items.cuh"

namespace {

using namespace pgk;

__device__ __forceinline__ bool closed(const int *gate) { return gate && *gate == 0; }

__global__ void k_cell_keys(const double *x, const double *y, const double *z, int n, Grid g,
                            const int *scene, const double *sox, const double *soy, const double *soz, int shift,
                            unsigned *keys, int *vals, double *rx, double *ry, double *rz, const int *gate)
{
  if (closed(gate)) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) cell_keys_item(i, x, y, z, g, scene, sox, soy, soz, shift, keys, vals, rx, ry, rz);
}

__global__ void __launch_bounds__(SORT_THREADS) k_sort_hist(const unsigned *keys, int n, unsigned *hist,
                                                            int nblocks, int shift, const int *gate)
{
  if (closed(gate)) return;
  __shared__ unsigned h[256];
  sort_hist_tile(keys, n, hist, nblocks, shift, blockIdx.x, h);
}

__global__ void __launch_bounds__(1024) k_sort_scan(unsigned *hist, int nblocks, const int *gate)
{
  if (closed(gate)) return;
  __shared__ unsigned part[1024];
  sort_scan_block(hist, nblocks, part);
}

// The histogram of a large sort (more than PG_SORT_SCAN_ONE_BLOCK tiles) is
// scanned by the whole grid: tile sums | their scan by one block | each tile
// rescanned from its base.  The tile sums sit after the histogram
// (pg_sort_hist_len).
constexpr int SCAN_BLOCK = 256;

__global__ void __launch_bounds__(SCAN_BLOCK) k_scan_tiles(const unsigned *a, int n, unsigned *bs, const int *gate)
{
  if (closed(gate)) return;
  __shared__ unsigned sh[SCAN_BLOCK];
  const unsigned sum = scan_tile_sum(a, n, blockIdx.x, sh);
  if (threadIdx.x == 0) bs[blockIdx.x] = sum;
}

__global__ void __launch_bounds__(1024) k_scan_sums(unsigned *bs, int tiles, const int *gate)
{
  if (closed(gate)) return;
  __shared__ unsigned part[1024];
  block_scan_seq(bs, tiles, part);
}

__global__ void __launch_bounds__(SCAN_BLOCK) k_scan_apply(unsigned *a, int n, const unsigned *bs, const int *gate)
{
  if (closed(gate)) return;
  __shared__ unsigned sh[SCAN_BLOCK];
  scan_tile_apply(a, n, blockIdx.x, bs[blockIdx.x], sh);
}

__global__ void __launch_bounds__(SORT_THREADS) k_sort_scatter(const unsigned *ksrc, const int *vsrc,
                                                               unsigned *kdst, int *vdst, int n,
                                                               const unsigned *hist, int nblocks, int shift,
                                                               const int *gate)
{
  if (closed(gate)) return;
  __shared__ unsigned wcnt[SORT_THREADS / 32][256];
  __shared__ unsigned goff[256];
  sort_scatter_tile(ksrc, vsrc, kdst, vdst, n, hist, nblocks, shift, blockIdx.x, wcnt, goff);
}

} // namespace

int pg_scan_blocks(int n) { return n > 0 ? (n + SCAN_TILE - 1) / SCAN_TILE : 1; }

int pg_sort_passes_exact(int key_bits)
{
  int p = (key_bits + 7) / 8;
  return p < 1 ? 1 : p;
}

int pg_sort_blocks(int n) { return n > 0 ? (n + SORT_TILE - 1) / SORT_TILE : 1; }

size_t pg_sort_hist_len(int n)
{
  const int nb = pg_sort_blocks(n);
  const size_t h = 256 * (size_t)nb;
  return nb <= PG_SORT_SCAN_ONE_BLOCK ? h : h + (size_t)pg_scan_blocks((int)h);
}

int pg_sort_kernel_count(int n, int passes)
{
  return passes * (pg_sort_blocks(n) <= PG_SORT_SCAN_ONE_BLOCK ? 3 : 5);
}

int pg_sort_passes(int bits_per_axis) { return pg_sort_passes_bits(3 * bits_per_axis); }

int pg_sort_passes_bits(int key_bits)
{
  int p = (key_bits + 7) / 8;
  if (p < 2) p = 2;
  if (p & 1) p ++;             // even: the result lands back in the first buffer pair
  return p;
}

void pg_launch_cell_keys(const double *x, const double *y, const double *z, int n, const double org[3],
                         double cell, const int dim[3], unsigned *keys, int *vals,
                         double *rx, double *ry, double *rz, const int *gate, cudaStream_t s,
                         const int *scene, double *const sorg[3], int shift)
{
  if (n <= 0) return;
  Grid g;
  for (int k = 0; k < 3; k ++) { g.org[k] = org ? org[k] : 0.0; g.dim[k] = dim[k]; }
  g.cell = cell;
  k_cell_keys<<<(n + 127) / 128, 128, 0, s>>>(x, y, z, n, g, scene, scene ? sorg[0] : nullptr,
                                              scene ? sorg[1] : nullptr, scene ? sorg[2] : nullptr, shift,
                                              keys, vals, rx, ry, rz, gate);
}

void pg_launch_radix_sort(unsigned *k0, int *v0, unsigned *k1, int *v1, unsigned *hist, int n, int passes,
                          const int *gate, cudaStream_t s)
{
  if (n <= 0) return;
  const int nb = pg_sort_blocks(n);
  for (int p = 0; p < passes; p ++)
  {
    unsigned *ks = (p & 1) ? k1 : k0, *kd = (p & 1) ? k0 : k1;
    int *vs = (p & 1) ? v1 : v0, *vd = (p & 1) ? v0 : v1;
    k_sort_hist<<<nb, SORT_THREADS, 0, s>>>(ks, n, hist, nb, 8 * p, gate);
    if (nb <= PG_SORT_SCAN_ONE_BLOCK) k_sort_scan<<<1, 1024, 0, s>>>(hist, nb, gate);
    else
    {
      const int h = 256 * nb, tiles = pg_scan_blocks(h);
      k_scan_tiles<<<tiles, SCAN_BLOCK, 0, s>>>(hist, h, hist + h, gate);
      k_scan_sums<<<1, 1024, 0, s>>>(hist + h, tiles, gate);
      k_scan_apply<<<tiles, SCAN_BLOCK, 0, s>>>(hist, h, hist + h, gate);
    }
    k_sort_scatter<<<nb, SORT_THREADS, 0, s>>>(ks, vs, kd, vd, n, hist, nb, 8 * p, gate);
  }
}
