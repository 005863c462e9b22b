// pg_rebuild.cu -- contact candidate lists (replaces partition.ispc's kd-tree).
//
// The reference re-drops every sphere into a frozen kd-tree each step and
// searches it per sphere and per triangle (partition.ispc:600-764,
// condet.ispc:98-516).  Here candidate lists are rebuilt only when a sphere
// or triangle vertex has moved more than 0.45*skin since the last rebuild:
//
//   1. Morton key of each sphere's cell (cell >= 2*rmax + skin)   [pg_sort.cu]
//   2. stable LSD radix sort of (key, sphere) pairs, 8-bit digits  [pg_sort.cu]
//   3. cell start/end ranges over the sorted keys
//   4. per sphere: the spheres of the 27 neighbouring cells and the triangles
//      within r + skin (the master side only: partner particle index larger),
//      sorted in partner order and merged with the previous list so that the
//      contact flag and tangential state follow their contact
//   5. per particle: slave list of master entries that point at it, sorted by
//      master particle then master slot
//
// Every kernel returns at once unless the rebuild flag is set, so the whole
// sequence can be enqueued (or captured) every step at the cost of a few
// empty launches.
#include <cuda_runtime.h>
#include <cstdint>
#include <cmath>
#include "pg_state.h"
#include "pg_math.cuh"
#include "pg_launch.h"
#include "pg_items.cuh"
#include "../../include/parmec_gb300.h"

namespace {

constexpr int TPB = 128;

inline int nblk(int n) { return (n + TPB - 1) / TPB; }

using namespace pgk;

// the whole rebuild as one cooperative launch; returns at once (one empty
// launch per step) unless a rebuild is due
template <int B>
__global__ void __launch_bounds__(B) k_rebuild_coop(PgDev d, int passes, int epasses)
{
  __shared__ RebuildSmem<B> sm;
  if (!d.ellnum || !*(volatile int *)d.rebuild) return;
  rebuild_all<B>(d, passes, epasses, sm, NoHook());
}

// self-test of the bounded grid barrier: the host presets the arrival count
// to the grid size, so no arrival completes the barrier and every block
// waits until the 2 s limit, records PG_ERR_TIMEOUT and leaves
__global__ void k_barrier_probe(PgDev d)
{
  grid_barrier(d);
}

constexpr int RB_THREADS = 256;

// blocks of the cooperative rebuild grid: all that fit at once
int rebuild_grid()
{
  static int grid = 0;
  if (grid) return grid;
  int dev = 0, sms = 0, per = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_rebuild_coop<RB_THREADS>, RB_THREADS, 0) != cudaSuccess)
  {
    cudaGetLastError();
    return 1;
  }
  grid = sms * (per > 0 ? per : 1);
  return grid;
}

// ---- gate of the drop-in condet(): a rebuild is due when a sphere centre or
// a triangle vertex moved more than 0.45*skin since the last rebuild (in the
// session the step kernels raise the same flag as they move things)
__global__ void k_rb_gate(PgDev d)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool need = false;
  if (i < d.ellnum)
  {
    double r0 = d.center[0][i] - d.cref[0][i], r1 = d.center[1][i] - d.cref[1][i], r2 = d.center[2][i] - d.cref[2][i];
    need = !((r0*r0 + r1*r1 + r2*r2) <= d.half_skin_sq);
  }
  if (i < d.trinum)
    for (int v = 0; v < 3; v ++)
    {
      double r0 = d.tri[3*v][i] - d.tref[3*v][i], r1 = d.tri[3*v+1][i] - d.tref[3*v+1][i];
      double r2 = d.tri[3*v+2][i] - d.tref[3*v+2][i];
      need |= !((r0*r0 + r1*r1 + r2*r2) <= d.half_skin_sq);
    }
  if (__syncthreads_or(need) && threadIdx.x == 0) atomicExch(d.rebuild, 1);
}

} // namespace

void pg_launch_rebuild_gate(const PgDev &d, cudaStream_t s)
{
  const int n = d.ellnum > d.trinum ? d.ellnum : d.trinum;
  if (n > 0) k_rb_gate<<<nblk(n), TPB, 0, s>>>(d);
}

void pg_rebuild_grid_params(PgDev &d, const double *ext, double rmax, double rmin)
{
  // default skin: 0.3 rmin for one scene; 0.6 rmin for a pool, whose scenes
  // share one rebuild flag, so that any sphere of any scene moving 0.45 skin
  // rebuilds them all (on 512 shaken boxes: 9 -> 4 rebuilds per 100 steps)
  if (!(d.skin > 0.0)) d.skin = (d.nscene > 1 ? 0.6 : 0.3) * rmin;
  d.half_skin_sq = (0.45 * d.skin) * (0.45 * d.skin);
  d.half_skin_sq_f = (float)d.half_skin_sq;
  double cell = 2.0 * rmax + d.skin;
  double e = 0.0;
  for (int k = 0; k < 3; k ++) e = fmax(e, ext[k]);
  e += 8.0 * cell;
  const int maxdim = 512;
  if (e / cell > maxdim - 4) cell = e / (maxdim - 4);
  d.cell = cell;
  for (int k = 0; k < 3; k ++)
  {
    int n = (int)ceil(ext[k] / cell) + 9;
    if (n > maxdim) n = maxdim;
    if (n < 1) n = 1;
    d.dim[k] = n;
  }
  pg_rebuild_key_bits(d);
}

void pg_rebuild_key_bits(PgDev &d)
{
  int need = 1;
  for (int k = 0; k < 3; k ++) while ((1 << need) < d.dim[k]) need ++;
  d.bits = need;
  int sb = 0;
  while ((1 << sb) < d.nscene) sb ++;
  d.keybits = 3 * need + sb;
}

// bits the radix sort orders: with scene ids one more than the valid keys
// use, so that the 0xffffffff key of a free entry sorts strictly after every
// valid key (a valid key of all ones in the sorted bits would tie with it)
int pg_rebuild_sort_bits(const PgDev &d) { return d.keybits + (d.escene ? 1 : 0); }

cudaError_t pg_launch_barrier_probe(const PgDev &d, cudaStream_t s, int blocks)
{
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(32);
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_barrier_probe, d);
}

void pg_launch_rebuild(const PgDev &d, cudaStream_t s)
{
  if (!d.ellnum) return;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(rebuild_grid());
  cfg.blockDim = dim3(RB_THREADS);
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k_rebuild_coop<RB_THREADS>, d, pg_sort_passes_bits(pg_rebuild_sort_bits(d)),
                     pg_sort_passes_exact(d.sbits));
}

int pg_rebuild_entry_bits(int parnum)
{
  int b = 1;
  while (b < 31 && (1 << b) < parnum) b ++;
  return b + 1;                               // one more: the no-partner key sorts last
}

int pg_rebuild_kernel_count(const PgDev &d)
{
  return d.ellnum ? 1 : 0;
}
