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

namespace {

constexpr int SORT_THREADS = 256;
constexpr int SORT_ITEMS = 8;
constexpr int SORT_TILE = SORT_THREADS * SORT_ITEMS;

__device__ __forceinline__ bool closed(const int *gate) { return gate && *gate == 0; }

__device__ __forceinline__ unsigned spread3(unsigned x)
{
  x &= 0x3ff;
  x = (x | (x << 16)) & 0x030000FF;
  x = (x | (x << 8)) & 0x0300F00F;
  x = (x | (x << 4)) & 0x030C30C3;
  x = (x | (x << 2)) & 0x09249249;
  return x;
}

struct Grid { double org[3]; double cell; int dim[3]; };

// key = (scene << shift) | Morton(cell); the cell is taken from the scene's
// own origin when 'scene' is given, else from g.org
__global__ void k_cell_keys(const double *x, const double *y, const double *z, int n, Grid g,
                            const int *scene, const double *sox, const double *soy, const double *soz, int shift,
                            unsigned *keys, int *vals, double *rx, double *ry, double *rz, const int *gate)
{
  if (closed(gate)) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double c[3] = {x[i], y[i], z[i]};
  double o[3] = {g.org[0], g.org[1], g.org[2]};
  unsigned sc = 0;
  if (scene)
  {
    if (scene[i] < 0)                // an entry of no scene: sorts last, owns no cell
    {
      keys[i] = 0xffffffffu;
      vals[i] = i;
      if (rx) { rx[i] = c[0]; ry[i] = c[1]; rz[i] = c[2]; }
      return;
    }
    sc = (unsigned)scene[i];
    o[0] = sox[sc]; o[1] = soy[sc]; o[2] = soz[sc];
  }
  unsigned u[3];
  for (int k = 0; k < 3; k ++)
  {
    double f = floor((c[k] - o[k]) / g.cell);
    if (!(f >= 0.0)) f = 0.0;
    if (f > (double)(g.dim[k] - 1)) f = (double)(g.dim[k] - 1);
    u[k] = (unsigned)f;
  }
  keys[i] = (scene ? (sc << shift) : 0u) | spread3(u[0]) | (spread3(u[1]) << 1) | (spread3(u[2]) << 2);
  vals[i] = i;
  if (rx) { rx[i] = c[0]; ry[i] = c[1]; rz[i] = c[2]; }
}

// per-block digit histograms, stored digit-major: hist[digit*nblocks + block]
__global__ void __launch_bounds__(SORT_THREADS) k_sort_hist(const unsigned *keys, int n, unsigned *hist,
                                                            int nblocks, int shift, const int *gate)
{
  if (closed(gate)) return;
  __shared__ unsigned h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int base = blockIdx.x * SORT_TILE;
  for (int it = 0; it < SORT_ITEMS; it ++)
  {
    int s = base + it * SORT_THREADS + threadIdx.x;
    if (s < n) atomicAdd(&h[(keys[s] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

// exclusive scan of the digit-major histogram, one block of 1024 threads
__global__ void __launch_bounds__(1024) k_sort_scan(unsigned *hist, int nblocks, const int *gate)
{
  if (closed(gate)) return;
  __shared__ unsigned part[1024];
  const int total = 256 * nblocks;
  const int per = (total + 1023) / 1024;
  const int b = threadIdx.x * per;
  const int e = min(b + per, total);
  unsigned sum = 0;
  for (int k = b; k < e; k ++) sum += hist[k];
  part[threadIdx.x] = sum;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1)
  {
    unsigned v = threadIdx.x >= off ? part[threadIdx.x - off] : 0u;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  unsigned run = threadIdx.x ? part[threadIdx.x - 1] : 0u;
  for (int k = b; k < e; k ++)
  {
    unsigned v = hist[k];
    hist[k] = run;
    run += v;
  }
}

// stable scatter: each warp ranks its contiguous sub-tile 32 keys at a time
// (__match_any_sync groups equal digits, popc of lower peers gives the rank)
__global__ void __launch_bounds__(SORT_THREADS) k_sort_scatter(const unsigned *ksrc, const int *vsrc,
                                                               unsigned *kdst, int *vdst, int n,
                                                               const unsigned *hist, int nblocks, int shift,
                                                               const int *gate)
{
  if (closed(gate)) return;
  constexpr int WARPS = SORT_THREADS / 32;
  constexpr int SUB = SORT_TILE / WARPS;
  __shared__ unsigned wcnt[WARPS][256];
  __shared__ unsigned goff[256];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = threadIdx.x; k < WARPS * 256; k += SORT_THREADS) (&wcnt[0][0])[k] = 0;
  goff[threadIdx.x] = hist[threadIdx.x * nblocks + blockIdx.x];
  __syncthreads();
  const int base = blockIdx.x * SORT_TILE + warp * SUB;
  unsigned keyv[SUB / 32];
  int valv[SUB / 32];
  unsigned rank[SUB / 32];
  const unsigned lt = (1u << lane) - 1u;
  for (int r = 0; r < SUB / 32; r ++)
  {
    int s = base + r * 32 + lane;
    bool ok = s < n;
    unsigned key = ok ? ksrc[s] : 0xffffffffu;
    int val = ok ? vsrc[s] : -1;
    unsigned dig = ok ? (key >> shift) & 255u : 256u;      // 256: padding lane, never stored
    unsigned peers = __match_any_sync(0xffffffffu, dig);
    unsigned before = __popc(peers & lt);
    unsigned prev = ok ? wcnt[warp][dig] : 0u;
    __syncwarp();
    if (ok && before == 0) wcnt[warp][dig] = prev + __popc(peers);
    __syncwarp();
    keyv[r] = key;
    valv[r] = ok ? val : -1;
    rank[r] = prev + before;
  }
  __syncthreads();
  {
    unsigned run = 0;
    for (int w = 0; w < WARPS; w ++)
    {
      unsigned c = wcnt[w][threadIdx.x];
      wcnt[w][threadIdx.x] = run;
      run += c;
    }
  }
  __syncthreads();
  for (int r = 0; r < SUB / 32; r ++)
  {
    int s = base + r * 32 + lane;
    if (s >= n) continue;
    unsigned dig = (keyv[r] >> shift) & 255u;
    unsigned pos = goff[dig] + wcnt[warp][dig] + rank[r];
    kdst[pos] = keyv[r];
    vdst[pos] = valv[r];
  }
}

} // namespace

int pg_sort_blocks(int n) { return n > 0 ? (n + SORT_TILE - 1) / SORT_TILE : 1; }

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
    k_sort_scan<<<1, 1024, 0, s>>>(hist, nb, gate);
    k_sort_scatter<<<nb, SORT_THREADS, 0, s>>>(ks, vs, kd, vd, n, hist, nb, 8 * p, gate);
  }
}
