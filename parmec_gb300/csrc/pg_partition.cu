// pg_partition.cu -- public cell-ordering entry point.
//
// pg_cell_order is the GB300 replacement of partitioning_create
// (partition.ispc:663-746): where the reference sorts 30-bit Morton codes of
// the sphere centres (quicksort per task plus a serial merge) and builds a
// radix tree over them, this sorts Morton codes of the centres' grid cells
// with a stable LSD radix sort; sorted cell keys give each cell's range of
// spheres (a cell list).
#include <cuda_runtime.h>
#include <cstdio>
#include "pg_launch.h"
#include "../../include/parmec_gb300.h"

namespace {

int bits_for(const int dim[3])
{
  int m = 1;
  for (int k = 0; k < 3; k ++) m = dim[k] > m ? dim[k] : m;
  int b = 0;
  while ((1 << b) < m) b ++;
  return b > 0 ? b : 1;
}

bool valid(const double *x, const double *y, const double *z, int n, const double origin[3], double cell,
           const int dim[3], const unsigned *keys, const int *order)
{
  if (n < 0 || !origin || !dim || !(cell > 0.0)) return false;
  for (int k = 0; k < 3; k ++) if (dim[k] < 1 || dim[k] > 1024) return false;
  if (n > 0 && (!x || !y || !z || !keys || !order)) return false;
  return true;
}

} // namespace

extern "C" int pg_cell_order(const double *x, const double *y, const double *z, int n,
                             const double origin[3], double cell, const int dim[3],
                             unsigned *keys_out, int *order_out, void *stream)
{
  if (!valid(x, y, z, n, origin, cell, dim, keys_out, order_out)) return PG_ERR_ARGUMENT;
  if (n == 0) return PG_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const int nb = pg_sort_blocks(n);
  unsigned *k1 = nullptr, *hist = nullptr;
  int *v1 = nullptr;
  if (cudaMallocAsync((void **)&k1, sizeof(unsigned) * (size_t)n, s) != cudaSuccess ||
      cudaMallocAsync((void **)&v1, sizeof(int) * (size_t)n, s) != cudaSuccess ||
      cudaMallocAsync((void **)&hist, sizeof(unsigned) * 256 * (size_t)nb, s) != cudaSuccess)
  {
    if (k1) cudaFreeAsync(k1, s);
    if (v1) cudaFreeAsync(v1, s);
    return PG_ERR_CUDA;
  }
  pg_launch_cell_keys(x, y, z, n, origin, cell, dim, keys_out, order_out, nullptr, nullptr, nullptr, nullptr, s);
  pg_launch_radix_sort(keys_out, order_out, k1, v1, hist, n, pg_sort_passes(bits_for(dim)), nullptr, s);
  cudaFreeAsync(k1, s);
  cudaFreeAsync(v1, s);
  cudaFreeAsync(hist, s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
  {
    std::fprintf(stderr, "parmec_gb300: pg_cell_order: %s\n", cudaGetErrorString(e));
    return PG_ERR_CUDA;
  }
  return PG_OK;
}
