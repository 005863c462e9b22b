// pg_partition.cu -- public cell-ordering entry point.
//
// pg_cell_order is the GB300 replacement of partitioning_create
// (partition.ispc:663-746): where the reference sorts 30-bit Morton codes of
// the sphere centres (quicksort per task plus a serial merge) and builds a
// radix tree over them, this sorts Morton codes of the centres' grid cells
// with a stable LSD radix sort; sorted cell keys give each cell's range of
// spheres (a cell list).
#include <cuda_runtime.h>
#include <atomic>
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
      cudaMallocAsync((void **)&hist, sizeof(unsigned) * pg_sort_hist_len(n), s) != cudaSuccess)
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

// ---------------------------------------------------------------------------
// pg_cell_order_static: the same ordering, with no device allocation.
//
// Some callers of this library cannot allocate device memory: coupling codes
// that give the whole device to their own memory pool (so a cudaMalloc here
// would fail or fragment it), and hosts that must not let cudaMalloc/cudaFree
// synchronise the device while their other streams run.  This entry point
// takes its scratch from a file-scope __device__ array instead.  That array is
// part of the library image: every GPU that loads the library holds its
// PG_CELL_ORDER_STATIC_MAX-sized scratch (about 0.55 MB) until the process
// exits.  Every call on a device shares the one array, so calls that overlap
// on the GPU (from different streams or threads) race and must not be made.
// Nothing in the array needs to start at zero: each sort pass writes every
// histogram entry and every key before it reads them.  Each call on a
// stream that is not capturing looks up the array's device address
// (cudaGetSymbolAddress) with the caller's device current; a call on a
// capturing stream uses the address the last such call found on that device.
// So make one call before any stream capture on a device, and again after a
// device reset (a reset may load the library's module at another address).
// ---------------------------------------------------------------------------

#define PG_CELL_ORDER_STATIC_MAX 65536
// sort tiles of the largest call: pg_launch_radix_sort writes 256 histogram
// entries per tile (tile = the sort's SORT_TILE keys, 2048 when this was
// written); the call checks pg_sort_blocks(n) against this bound
#define PG_CELL_ORDER_STATIC_BLOCKS 32
// the histogram of a sort this small is scanned by one block, so the
// scratch needs no room for the grid scan's tile sums (pg_sort_hist_len)
static_assert(PG_CELL_ORDER_STATIC_BLOCKS <= PG_SORT_SCAN_ONE_BLOCK, "static scratch too small for the grid scan");

namespace {

constexpr size_t STATIC_KEYS_OFF = 0;
constexpr size_t STATIC_VALS_OFF = STATIC_KEYS_OFF + sizeof(unsigned) * PG_CELL_ORDER_STATIC_MAX;
constexpr size_t STATIC_HIST_OFF = STATIC_VALS_OFF + sizeof(int) * PG_CELL_ORDER_STATIC_MAX;
constexpr size_t STATIC_BYTES = STATIC_HIST_OFF + sizeof(unsigned) * 256 * PG_CELL_ORDER_STATIC_BLOCKS;

__device__ __align__(256) unsigned char g_cell_order_scratch[STATIC_BYTES];

constexpr int MAX_DEVICES = 64;
std::atomic<unsigned char *> g_scratch_addr[MAX_DEVICES];

// The host-side name g_cell_order_scratch is not a device address; ask the
// runtime for the device address with the device current, unless the stream
// is capturing (then the address found by the last call on this device).
int scratch_address(cudaStream_t s, unsigned char **out)
{
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return PG_ERR_CUDA;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) return PG_ERR_CUDA;
  unsigned char *p = g_scratch_addr[dev].load();
  if (cap == cudaStreamCaptureStatusNone || !p)
  {
    void *q = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&q, g_cell_order_scratch);
    if (e != cudaSuccess || !q)
    {
      std::fprintf(stderr, "parmec_gb300: pg_cell_order_static: cudaGetSymbolAddress failed: %s\n",
                   cudaGetErrorString(e));
      return PG_ERR_CUDA;
    }
    p = (unsigned char *)q;
    g_scratch_addr[dev].store(p);
  }
  *out = p;
  return PG_OK;
}

} // namespace

extern "C" int pg_cell_order_static(const double *x, const double *y, const double *z, int n,
                                    const double origin[3], double cell, const int dim[3],
                                    unsigned *keys_out, int *order_out, void *stream)
{
  if (!valid(x, y, z, n, origin, cell, dim, keys_out, order_out)) return PG_ERR_ARGUMENT;
  if (n > PG_CELL_ORDER_STATIC_MAX)
  {
    std::fprintf(stderr, "parmec_gb300: pg_cell_order_static: n = %d exceeds the static scratch limit of %d "
                         "spheres; use pg_cell_order\n", n, PG_CELL_ORDER_STATIC_MAX);
    return PG_ERR_CAPACITY;
  }
  if (pg_sort_blocks(n) > PG_CELL_ORDER_STATIC_BLOCKS)
  {
    std::fprintf(stderr, "parmec_gb300: pg_cell_order_static: %d sort tiles exceed the static histogram room "
                         "of %d\n", pg_sort_blocks(n), PG_CELL_ORDER_STATIC_BLOCKS);
    return PG_ERR_CAPACITY;
  }
  if (n == 0) return PG_OK;
  cudaStream_t s = (cudaStream_t)stream;
  unsigned char *base = nullptr;
  int r = scratch_address(s, &base);
  if (r != PG_OK) return r;
  unsigned *k1 = (unsigned *)(base + STATIC_KEYS_OFF);
  int *v1 = (int *)(base + STATIC_VALS_OFF);
  unsigned *hist = (unsigned *)(base + STATIC_HIST_OFF);
  pg_launch_cell_keys(x, y, z, n, origin, cell, dim, keys_out, order_out, nullptr, nullptr, nullptr, nullptr, s);
  pg_launch_radix_sort(keys_out, order_out, k1, v1, hist, n, pg_sort_passes(bits_for(dim)), nullptr, s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
  {
    std::fprintf(stderr, "parmec_gb300: pg_cell_order_static: %s\n", cudaGetErrorString(e));
    return PG_ERR_CUDA;
  }
  return PG_OK;
}
