// pg_meshcontact.cu -- mesh-mesh contact between triangles of different
// particles (an extension; off unless pg_session_mesh_contact turns it on).
//
// Every step, before the force sums:
//   1. each mesh triangle's box (its vertices' bounds widened by the swept
//      radius r) and its grid cell, or the "big" range for triangles larger
//      than a cell;
//   2. a stable radix sort of the triangles by cell, and the cell ranges;
//   3. each triangle finds its partners among the triangles of the 27 cells
//      around its own (and among the big ones), keeps those whose boxes
//      overlap with positive measure (two triangles closer than 2r have such
//      boxes; boxes that only touch hold no contact), and sorts them by index.  A pair is found by one triangle
//      only: between two small triangles (or two big ones) by the lower
//      index, between a small and a big one by the small one;
//   4. the pairs, in the order of the finding triangles and their sorted
//      partners (an exclusive scan of the counts gives each triangle's
//      offset);
//   5. one thread per pair: the plane test that settles most pairs as
//      apart; the others are queued (one atomic per warp) and evaluated by a
//      grid-stride loop, so that the narrow phase runs on full warps: the
//      swept-triangle contact (pg_tritri.cuh) and the granular law with the
//      pair's tangential state, carried over from the previous step's pair
//      list by (finder, partner);
//   6. the force of each active pair goes to its two particles (+f to the
//      finder's, -f to the partner's): the entries are sorted by particle
//      (stably, so in pair order) and summed per particle in chunks of
//      PG_TT_CHUNK entries: one warp per chunk, lane L taking entries L,
//      L+32, ... of the chunk from zero and the 32 lane sums added in lane
//      order; then the chunk sums in chunk order from zero, one thread per
//      particle.  A particle with many contacts (a base plate under a whole
//      lattice) spreads over many warps.  k_integrate adds these sums after
//      gravity.
// The CPU oracle restates the same definitions with a brute-force search.
#include <cuda_runtime.h>
#include <cstdio>
#include "pg_items.cuh"
#include "pg_launch.h"
#include "pg_meshcontact.h"
#include "pg_tritri.cuh"

namespace {

constexpr int TPB = 128;
inline int nblk(long long n) { return (int)((n + TPB - 1) / TPB); }

__device__ __forceinline__ bool mesh_tri(const PgDev &d, int t) { return d.triobs[t] >= 0; }

__device__ __forceinline__ void tri_vertices(const PgDev &d, int t, double v[3][3])
{
  for (int a = 0; a < 3; a ++)
    for (int c = 0; c < 3; c ++) v[a][c] = d.tri[3*a + c][t];
}

// box keys: lo < hi on the keys is the FP64 comparison lo < hi
__device__ __forceinline__ unsigned long long lo_key(double x)
{
  const unsigned long long b = pgtt::bits(x);
  return pgtt::nan_b(b) ? ~0ULL : pgtt::okey(b);
}
__device__ __forceinline__ unsigned long long hi_key(double x)
{
  const unsigned long long b = pgtt::bits(x);
  return pgtt::nan_b(b) ? 0ULL : pgtt::okey(b);
}

// 1. boxes and cell keys
__global__ void __launch_bounds__(TPB) k_tt_keys(PgDev d, PgTT g)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.trinum) return;
  unsigned key = g.none;
  if (mesh_tri(d, t))
  {
    double lo[3], hi[3];
    for (int c = 0; c < 3; c ++)
    {
      const double a = d.tri[c][t], b = d.tri[3+c][t], e = d.tri[6+c][t];
      double l = a < b ? a : b, h = a > b ? a : b;
      l = l < e ? l : e;
      h = h > e ? h : e;
      lo[c] = l - g.r;
      hi[c] = h + g.r;
      g.box[c][t] = lo_key(lo[c]);
      g.box[3+c][t] = hi_key(hi[c]);
    }
    if (g.big[t]) key = (unsigned)g.ncells;
    else
    {
      int ix[3];
      for (int c = 0; c < 3; c ++)
      {
        const double q = floor((0.5*(lo[c] + hi[c]) - g.org[c]) / g.h);
        int k = q < 0.0 ? 0 : (q > (double)(g.dim[c]-1) ? g.dim[c]-1 : (int)q);
        ix[c] = k;
      }
      key = (unsigned)((ix[2]*g.dim[1] + ix[1])*g.dim[0] + ix[0]);
    }
    g.cell[t] = (int)key;
  }
  g.keys[0][t] = key;
  g.vals[0][t] = t;
}

// 2. cell ranges over the sorted keys
__global__ void __launch_bounds__(TPB) k_tt_ranges(PgTT g, int n)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const unsigned key = g.keys[0][k];
  if (key == g.none) return;
  if (k == 0 || g.keys[0][k-1] != key) g.cstart[key] = k;
  if (k == n-1 || g.keys[0][k+1] != key) g.cend[key] = k + 1;
}

// 3. partners found by triangle t, sorted by index, in cand[slot][t]
// (sorted in a thread-local array, written once)
__global__ void __launch_bounds__(TPB) k_tt_find(PgDev d, PgTT g)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.trinum) return;
  int cnt = 0;
  int loc[PG_TT_KMAX];
  if (mesh_tri(d, t))
  {
    const int owner = d.triobs[t];
    const bool big = g.big[t] != 0;
    unsigned long long lo[3], hi[3];
    for (int c = 0; c < 3; c ++) { lo[c] = g.box[c][t]; hi[c] = g.box[3+c][t]; }
    auto take = [&](int u) {
      if (u == t || !mesh_tri(d, u) || d.triobs[u] == owner) return;
      const bool ubig = g.big[u] != 0;
      if (big && !ubig) return;                       // found from the small side
      if (big == ubig && u < t) return;               // found by the lower index
      for (int c = 0; c < 3; c ++)
        if (!(lo[c] < g.box[3+c][u] && g.box[c][u] < hi[c])) return;
      if (cnt >= g.kmax) { pgk::set_err(d, PG_ERR_CAPACITY, 40, t, cnt); return; }
      // insertion in index order
      int k = cnt ++;
      while (k > 0 && loc[k-1] > u) { loc[k] = loc[k-1]; k --; }
      loc[k] = u;
    };
    if (!big)
    {
      const int cell = g.cell[t];
      const int ix[3] = {cell % g.dim[0], (cell / g.dim[0]) % g.dim[1], cell / (g.dim[0] * g.dim[1])};
      for (int z = ix[2]-1; z <= ix[2]+1; z ++)
      {
        if (z < 0 || z >= g.dim[2]) continue;
        for (int y = ix[1]-1; y <= ix[1]+1; y ++)
        {
          if (y < 0 || y >= g.dim[1]) continue;
          for (int x = ix[0]-1; x <= ix[0]+1; x ++)
          {
            if (x < 0 || x >= g.dim[0]) continue;
            const int cell = (z*g.dim[1] + y)*g.dim[0] + x;
            for (int k = g.cstart[cell]; k < g.cend[cell]; k ++) take(g.vals[0][k]);
          }
        }
      }
    }
    for (int k = g.cstart[g.ncells]; k < g.cend[g.ncells]; k ++) take(g.vals[0][k]);
  }
  for (int k = 0; k < cnt; k ++) g.cand[(size_t)k * d.trinum + t] = loc[k];
  g.cnt[t] = cnt;
}

// 4a. exclusive scan of the counts in one block (off[n] = total)
__global__ void __launch_bounds__(1024) k_tt_scan(const int *in, int *out, int n, int *total)
{
  __shared__ int part[1024];
  const int tid = threadIdx.x;
  const int per = (n + 1023) / 1024;
  const int b = tid * per, e = b + per < n ? b + per : n;
  int s = 0;
  for (int i = b; i < e; i ++) s += in[i];
  part[tid] = s;
  __syncthreads();
  if (tid == 0)
  {
    int acc = 0;
    for (int k = 0; k < 1024; k ++) { const int v = part[k]; part[k] = acc; acc += v; }
    out[n] = acc;
    *total = acc;
  }
  __syncthreads();
  int acc = part[tid];
  for (int i = b; i < e; i ++) { out[i] = acc; acc += in[i]; }
}

// 4b. the pair list in finder order
__global__ void __launch_bounds__(TPB) k_tt_emit(PgDev d, PgTT g)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.trinum) return;
  const int o = g.off[t], c = g.cnt[t];
  for (int k = 0; k < c; k ++)
  {
    g.pf[o + k] = t;
    g.pu[o + k] = g.cand[(size_t)k * d.trinum + t];
  }
}

// 5a. pairs apart by the plane test get their (zero) results; the others
// are queued
__global__ void __launch_bounds__(TPB) k_tt_cull(PgDev d, PgTT g, int np)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  bool near = false;
  if (k < np)
  {
    double va[3][3], vb[3][3];
    tri_vertices(d, g.pf[k], va);
    tri_vertices(d, g.pu[k], vb);
    const double *A[3] = {va[0], va[1], va[2]}, *B[3] = {vb[0], vb[1], vb[2]};
    near = !pgtt::apart(A, B, g.r, g.r);
    if (!near)
    {
      g.act[k] = 0;
      for (int c = 0; c < 3; c ++) { g.st[c][k] = 0.0; g.f[c][k] = 0.0; g.p[c][k] = 0.0; }
    }
  }
  // warp-aggregated push of the near pairs
  const unsigned m = __ballot_sync(0xffffffffu, near);
  if (!m) return;
  const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(g.qn, __popc(m));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (near) g.queue[base + __popc(m & ((1u << lane) - 1u))] = k;
}

// 5b. contact and granular force of each queued pair
__global__ void __launch_bounds__(TPB) k_tt_pairs(PgDev d, PgTT g, double step)
{
  const int nq = *g.qn;
  for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < nq; w += gridDim.x * blockDim.x)
  {
  const int k = g.queue[w];
  const int f = g.pf[k], u = g.pu[k];
  double va[3][3], vb[3][3];
  tri_vertices(d, f, va);
  tri_vertices(d, u, vb);
  const double *A[3] = {va[0], va[1], va[2]}, *B[3] = {vb[0], vb[1], vb[2]};
  double point[3], normal[3];
  const double depth = pgtt::contact_near(A, B, g.r, g.r, point, normal);
  double st[3] = {0.0, 0.0, 0.0}, fr[3] = {0.0, 0.0, 0.0};
  const bool active = depth > 0.0;
  if (active)
  {
    // the pair's state of the previous step: (finder, partner) in its list
    int lo = g.poff[f], hi = g.poff[f+1];
    while (lo < hi)
    {
      const int mid = (lo + hi) >> 1;
      if (g.ppu[mid] < u) lo = mid + 1;
      else hi = mid;
    }
    if (lo < g.poff[f+1] && g.ppu[lo] == u && g.pact[lo])
      for (int c = 0; c < 3; c ++) st[c] = g.pst[c][lo];
    const int pa = d.triobs[f], pb = d.triobs[u];
    // contact point velocities (forces.ispc:226-246) and their difference
    double vij[3];
    const double za[3] = {point[0]-d.position[0][pa], point[1]-d.position[1][pa], point[2]-d.position[2][pa]};
    const double zb[3] = {point[0]-d.position[0][pb], point[1]-d.position[1][pb], point[2]-d.position[2][pb]};
    for (int c = 0; c < 3; c ++)
    {
      const int c1 = (c+1)%3, c2 = (c+2)%3;
      const double vi = d.angular[3+c1][pa]*za[c2] - d.angular[3+c2][pa]*za[c1] + d.linear[c][pa];
      const double vj = d.angular[3+c1][pb]*zb[c2] - d.angular[3+c2][pb]*zb[c1] + d.linear[c][pb];
      vij[c] = vj - vi;
    }
    const int ij = pgk::pairing(d, d.tricol[f], d.tricol[u]);
    if (d.ikind[ij] != 0) pgk::set_err(d, PG_ERR_UNSUPPORTED, 41, k, ij);
    const double ma = 1.0 / (d.invm[pa] + d.invm[pb]);
    pgtt::granular(d.iparam[0][ij], d.iparam[1][ij], d.iparam[6][ij], d.iparam[2][ij], d.iparam[3][ij], ma,
                   normal, vij, depth, step, st, fr);
  }
  g.act[k] = active ? 1 : 0;
  for (int c = 0; c < 3; c ++)
  {
    g.st[c][k] = st[c];
    g.f[c][k] = fr[c];
    g.p[c][k] = point[c];
  }
  }
}

// resident blocks of k_tt_pairs over every SM
int pairs_blocks()
{
  static int nb = 0;
  if (!nb)
  {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_tt_pairs, TPB, 0);
    nb = (sms > 0 ? sms : 152) * (per > 0 ? per : 4);
  }
  return nb;
}

// 6a. two entries per pair, keyed by particle (inactive: the sentinel)
__global__ void __launch_bounds__(TPB) k_tt_entries(PgDev d, PgTT g, int np)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= np) return;
  const bool on = g.act[k] != 0;
  g.ekeys[0][2*k] = on ? (unsigned)d.triobs[g.pf[k]] : g.enone;
  g.ekeys[0][2*k+1] = on ? (unsigned)d.triobs[g.pu[k]] : g.enone;
  g.evals[0][2*k] = 2*k;
  g.evals[0][2*k+1] = 2*k + 1;
}

// 6b. each particle's range of the sorted entries
__global__ void __launch_bounds__(TPB) k_tt_segments(PgTT g, int n)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const unsigned key = g.ekeys[0][k];
  if (key == g.enone) return;
  if (k == 0 || g.ekeys[0][k-1] != key) g.pfirst[key] = k;
  if (k == n-1 || g.ekeys[0][k+1] != key) g.plast[key] = k + 1;
}

// 6c. chunks per particle
__global__ void __launch_bounds__(TPB) k_tt_chunks(PgDev d, PgTT g)
{
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= d.parnum) return;
  g.nch[w] = (g.plast[w] - g.pfirst[w] + PG_TT_CHUNK - 1) / PG_TT_CHUNK;
}

// 6d. one warp per chunk: lane sums over entries lane, lane+32, ... of the
// chunk, then the lane sums in lane order
__global__ void __launch_bounds__(TPB) k_tt_chunk_sums(PgDev d, PgTT g)
{
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const bool on = c < *g.nchunks;
  int w = 0;
  if (on)
  {
    // the particle whose chunks hold c: the last w with choff[w] <= c
    int lo = 0, hi = d.parnum - 1;
    while (lo < hi)
    {
      const int mid = (lo + hi + 1) >> 1;
      if (g.choff[mid] <= c) lo = mid;
      else hi = mid - 1;
    }
    w = lo;
  }
  double s[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  if (on)
  {
    const int b = g.pfirst[w] + (c - g.choff[w]) * PG_TT_CHUNK;
    const int e = min(b + PG_TT_CHUNK, g.plast[w]);
    const double x[3] = {d.position[0][w], d.position[1][w], d.position[2][w]};
    for (int q = b + lane; q < e; q += 32)
    {
      const int v = g.evals[0][q];
      const int k = v >> 1;
      double f[3] = {g.f[0][k], g.f[1][k], g.f[2][k]};
      if (v & 1) { f[0] = -f[0]; f[1] = -f[1]; f[2] = -f[2]; }
      const double a[3] = {g.p[0][k]-x[0], g.p[1][k]-x[1], g.p[2][k]-x[2]};
      s[0] += f[0]; s[1] += f[1]; s[2] += f[2];
      s[3] += a[1]*f[2] - a[2]*f[1];
      s[4] += a[2]*f[0] - a[0]*f[2];
      s[5] += a[0]*f[1] - a[1]*f[0];
    }
  }
  __shared__ double part[TPB / 32][32][6];
  const int wl = threadIdx.x >> 5;
  for (int k = 0; k < 6; k ++) part[wl][lane][k] = s[k];
  __syncwarp();
  if (on && lane == 0)
  {
    double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int L = 0; L < 32; L ++)
      for (int k = 0; k < 6; k ++) acc[k] += part[wl][L][k];
    for (int k = 0; k < 6; k ++) g.csum[k][c] = acc[k];
  }
}

// 6e. one thread per particle: its chunk sums in chunk order
__global__ void __launch_bounds__(TPB) k_tt_sums(PgDev d, PgTT g)
{
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= d.parnum) return;
  double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  for (int c = g.choff[w]; c < g.choff[w+1]; c ++)
    for (int k = 0; k < 6; k ++) acc[k] += g.csum[k][c];
  for (int k = 0; k < 3; k ++) { d.ttF[k][w] = acc[k]; d.ttT[k][w] = acc[3+k]; }
}

} // namespace

int pg_tt_key_bits(int ncells)
{
  int b = 1;
  while ((1u << b) <= (unsigned)ncells + 1u) b ++;      // ncells + 1 ranges and the sentinel above them
  return b;
}

void pg_tt_find(const PgDev &d, PgTT &g, cudaStream_t s)
{
  const int T = d.trinum;
  if (T <= 0) return;
  k_tt_keys<<<nblk(T), TPB, 0, s>>>(d, g);
  pg_launch_radix_sort(g.keys[0], g.vals[0], g.keys[1], g.vals[1], g.hist, T, g.passes, nullptr, s);
  cudaMemsetAsync(g.cstart, 0, (size_t)(g.ncells + 1) * sizeof(int), s);
  cudaMemsetAsync(g.cend, 0, (size_t)(g.ncells + 1) * sizeof(int), s);
  k_tt_ranges<<<nblk(T), TPB, 0, s>>>(g, T);
  k_tt_find<<<nblk(T), TPB, 0, s>>>(d, g);
  k_tt_scan<<<1, 1024, 0, s>>>(g.cnt, g.off, T, g.np_dev);
}

void pg_tt_forces(const PgDev &d, PgTT &g, cudaStream_t s, int np, double step)
{
  const int T = d.trinum;
  if (np > 0)
  {
    k_tt_emit<<<nblk(T), TPB, 0, s>>>(d, g);
    cudaMemsetAsync(g.qn, 0, sizeof(int), s);
    k_tt_cull<<<nblk(np), TPB, 0, s>>>(d, g, np);
    k_tt_pairs<<<pairs_blocks(), TPB, 0, s>>>(d, g, step);
    k_tt_entries<<<nblk(np), TPB, 0, s>>>(d, g, np);
    pg_launch_radix_sort(g.ekeys[0], g.evals[0], g.ekeys[1], g.evals[1], g.ehist, 2*np, g.epasses, nullptr, s);
  }
  cudaMemsetAsync(g.pfirst, 0, (size_t)d.parnum * sizeof(int), s);
  cudaMemsetAsync(g.plast, 0, (size_t)d.parnum * sizeof(int), s);
  if (np > 0) k_tt_segments<<<nblk(2*(long long)np), TPB, 0, s>>>(g, 2*np);
  k_tt_chunks<<<nblk(d.parnum), TPB, 0, s>>>(d, g);
  k_tt_scan<<<1, 1024, 0, s>>>(g.nch, g.choff, d.parnum, g.nchunks);
  k_tt_chunk_sums<<<nblk(32LL * pg_tt_max_chunks(d.parnum, np)), TPB, 0, s>>>(d, g);
  k_tt_sums<<<nblk(d.parnum), TPB, 0, s>>>(d, g);
}

long long pg_tt_max_chunks(int parnum, int np)
{
  // each particle's entries fill its chunks but the last: at most parnum
  // partial chunks beside 2 np / PG_TT_CHUNK full ones
  return (long long)parnum + (2LL * np) / PG_TT_CHUNK + 1;
}

// kernels of one step's mesh-contact stage
int pg_tt_kernel_count(const PgTT &g, int trinum, int np)
{
  return 5 + pg_sort_kernel_count(trinum, g.passes) + (np > 0 ? 5 + pg_sort_kernel_count(2 * np, g.epasses) : 0) + 4;
}
