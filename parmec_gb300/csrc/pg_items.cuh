// pg_items.cuh -- per-item bodies of the step phases that both the one-kernel-
// per-phase path (pg_step.cu, pg_rebuild.cu, pg_sort.cu) and the persistent
// fused step kernel (pg_mixed.cu) run.  A kernel launches one thread per item
// and calls the body; the persistent kernel walks the same items in
// grid-stride loops between grid barriers.  The bodies are the only copy of
// this code.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "pg_state.h"
#include "pg_math.cuh"
#include "../../include/parmec_gb300.h"

namespace pgk {

constexpr int MAXKN = 96;                       // upper bound of candidate slots per sphere
constexpr int SORT_THREADS = 256;               // radix sort: threads and keys of one tile
constexpr int SORT_ITEMS = 8;
constexpr int SORT_TILE = SORT_THREADS * SORT_ITEMS;

// record the first error with where it happened (site), the index and a value
__device__ __forceinline__ void set_err(const PgDev &d, int code, int site, int index, int value)
{
  if (atomicCAS(d.err, 0, code) == 0)
  {
    d.err[1] = site;
    d.err[2] = index;
    d.err[3] = value;
  }
}

__device__ __forceinline__ unsigned spread3(unsigned x)
{
  x &= 0x3ff;
  x = (x | (x << 16)) & 0x030000FF;
  x = (x | (x << 8)) & 0x0300F00F;
  x = (x | (x << 4)) & 0x030C30C3;
  x = (x | (x << 2)) & 0x09249249;
  return x;
}

// inverse of spread3: every third bit, packed
__device__ __forceinline__ unsigned compact3(unsigned x)
{
  x &= 0x09249249;
  x = (x | (x >> 2)) & 0x030C30C3;
  x = (x | (x >> 4)) & 0x0300F00F;
  x = (x | (x >> 8)) & 0x030000FF;
  x = (x | (x >> 16)) & 0x3ff;
  return x;
}

__device__ __forceinline__ unsigned morton(int x, int y, int z)
{
  return spread3((unsigned)x) | (spread3((unsigned)y) << 1) | (spread3((unsigned)z) << 2);
}

__device__ __forceinline__ unsigned order_key(int code)
{
  return code >= 0 ? (unsigned)code : 0x80000000u + (unsigned)(-code - 1);
}

// ================================================================ triangle work queue
// The contact kernels evaluate a sphere's sphere partners in one pass and
// queue the spheres whose lists go on with triangles (order_key puts them
// last); a second pass evaluates those triangles, one thread per queued
// sphere, so that the long triangle code runs on full warps.

// every thread of the warp calls this; `more`: sphere i has triangles
__device__ __forceinline__ void tri_queue_push(const PgDev &d, bool more, int i)
{
  const unsigned m = __ballot_sync(0xffffffffu, more);
  if (!m) return;
  const int lane = threadIdx.x & 31, lead = __ffs(m) - 1;
  int base = 0;
  if (lane == lead) base = atomicAdd(&d.tcnt[0], __popc(m));
  base = __shfl_sync(0xffffffffu, base, lead);
  if (more) d.twork[base + __popc(m & ((1u << lane) - 1u))] = i;
}

// queue length, read at the start of the triangle pass
__device__ __forceinline__ int tri_queue_len(const PgDev &d) { return *(volatile int *)&d.tcnt[0]; }

// every thread of the block calls this after its triangles; the last block
// of the grid empties the queue for the next step
__device__ __forceinline__ void tri_queue_done(const PgDev &d)
{
  __syncthreads();
  if (threadIdx.x == 0)
  {
    __threadfence();
    if (atomicAdd(&d.tcnt[1], 1) == (int)gridDim.x - 1)
    {
      d.tcnt[0] = 0;
      d.tcnt[1] = 0;
      __threadfence();
    }
  }
}

constexpr int TRI_PASS_BLOCKS = 4 * 152;   // grid of the triangle pass (grid-stride over the queue)

// ================================================================ cell keys and radix sort
struct Grid { double org[3]; double cell; int dim[3]; };

// key = (scene << shift) | Morton(cell); the cell is taken from the scene's
// own origin when 'scene' is given, else from g.org
__device__ __forceinline__ void cell_keys_item(int i, const double *x, const double *y, const double *z, const Grid &g,
                                               const int *scene, const double *sox, const double *soy,
                                               const double *soz, int shift, unsigned *keys, int *vals,
                                               double *rx, double *ry, double *rz)
{
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

// ---- exclusive scans over tiles of SCAN_TILE elements (block-level
// helpers: every thread of the block calls them; blockDim divides SCAN_TILE)
constexpr int SCAN_TILE = 1024;

template <typename T>
__device__ __forceinline__ T scan_tile_sum(const T *a, int n, int tile, T *sh)
{
  const int B = blockDim.x, t = threadIdx.x, per = SCAN_TILE / B;
  const int b = tile * SCAN_TILE + t * per;
  T s = 0;
  for (int k = 0; k < per; k ++) if (b + k < n) s += a[b + k];
  sh[t] = s;
  __syncthreads();
  for (int off = B / 2; off > 0; off >>= 1)
  {
    if (t < off) sh[t] += sh[t + off];
    __syncthreads();
  }
  const T total = sh[0];
  __syncthreads();
  return total;
}

template <typename T>
__device__ __forceinline__ void scan_tile_apply(T *a, int n, int tile, T base, T *sh)
{
  const int B = blockDim.x, t = threadIdx.x, per = SCAN_TILE / B;
  const int b = tile * SCAN_TILE + t * per;
  T v[8];
  T s = 0;
  for (int k = 0; k < per; k ++) { v[k] = (b + k < n) ? a[b + k] : (T)0; s += v[k]; }
  sh[t] = s;
  __syncthreads();
  for (int off = 1; off < B; off <<= 1)
  {
    T x = t >= off ? sh[t - off] : (T)0;
    __syncthreads();
    sh[t] += x;
    __syncthreads();
  }
  T run = base + (t ? sh[t - 1] : (T)0);
  for (int k = 0; k < per; k ++)
  {
    if (b + k < n) a[b + k] = run;
    run += v[k];
  }
  __syncthreads();
}

// exclusive scan of a[0..total) by one block: contiguous chunks per thread
template <typename T>
__device__ __forceinline__ void block_scan_seq(T *a, int total, T *part)
{
  const int B = blockDim.x, t = threadIdx.x;
  const int per = (total + B - 1) / B;
  const int b = t * per;
  const int e = min(b + per, total);
  T sum = 0;
  for (int k = b; k < e; k ++) sum += a[k];
  part[t] = sum;
  __syncthreads();
  for (int off = 1; off < B; off <<= 1)
  {
    T v = t >= off ? part[t - off] : (T)0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  T run = t ? part[t - 1] : (T)0;
  for (int k = b; k < e; k ++)
  {
    T v = a[k];
    a[k] = run;
    run += v;
  }
  __syncthreads();
}

// per-tile digit histogram, stored digit-major: hist[digit*nb + tile].  The
// first 256 threads of the block do the work; every thread must call.
__device__ __forceinline__ void sort_hist_tile(const unsigned *keys, int n, unsigned *hist, int nb, int shift,
                                               int tile, unsigned *h)
{
  const int t = threadIdx.x;
  if (t < 256) h[t] = 0;
  __syncthreads();
  if (t < SORT_THREADS)
  {
    const int base = tile * SORT_TILE;
    for (int it = 0; it < SORT_ITEMS; it ++)
    {
      int s = base + it * SORT_THREADS + t;
      if (s < n) atomicAdd(&h[(keys[s] >> shift) & 255u], 1u);
    }
  }
  __syncthreads();
  if (t < 256) hist[t * nb + tile] = h[t];
  __syncthreads();
}

// exclusive scan of the digit-major histogram by one block
__device__ __forceinline__ void sort_scan_block(unsigned *hist, int nb, unsigned *part)
{
  block_scan_seq(hist, 256 * nb, part);
}

// stable scatter of one tile: each of the first 8 warps ranks its contiguous
// sub-tile 32 keys at a time (__match_any_sync groups equal digits, popc of
// lower peers gives the rank).  wcnt is [8][256], goff [256]; every thread
// of the block must call.
__device__ __forceinline__ void sort_scatter_tile(const unsigned *ksrc, const int *vsrc, unsigned *kdst, int *vdst,
                                                  int n, const unsigned *hist, int nb, int shift, int tile,
                                                  unsigned (*wcnt)[256], unsigned *goff)
{
  constexpr int WARPS = SORT_THREADS / 32;
  constexpr int SUB = SORT_TILE / WARPS;
  const int t = threadIdx.x;
  const int lane = t & 31, warp = t >> 5;
  if (t < SORT_THREADS)
  {
    for (int k = t; k < WARPS * 256; k += SORT_THREADS) (&wcnt[0][0])[k] = 0;
    goff[t] = hist[t * nb + tile];
  }
  __syncthreads();
  const int base = tile * SORT_TILE + warp * SUB;
  unsigned keyv[SUB / 32];
  int valv[SUB / 32];
  unsigned rank[SUB / 32];
  const unsigned lt = (1u << lane) - 1u;
  if (warp < WARPS)
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
  if (t < SORT_THREADS)
  {
    unsigned run = 0;
    for (int w = 0; w < WARPS; w ++)
    {
      unsigned c = wcnt[w][t];
      wcnt[w][t] = run;
      run += c;
    }
  }
  __syncthreads();
  if (warp < WARPS)
    for (int r = 0; r < SUB / 32; r ++)
    {
      int s = base + r * 32 + lane;
      if (s >= n) continue;
      unsigned dig = (keyv[r] >> shift) & 255u;
      unsigned pos = goff[dig] + wcnt[warp][dig] + rank[r];
      kdst[pos] = keyv[r];
      vdst[pos] = valv[r];
    }
  __syncthreads();
}

// surface pair of two colours: binary search of the sorted pairs
// (forces.ispc:98-122; stops where the reference could loop forever)
__device__ __forceinline__ int pairing(const PgDev &d, int i, int j)
{
  int p0 = i, p1 = j, start = 1, end = d.pairnum;
  if (i > j) { p0 = j; p1 = i; }
  while (start < end)
  {
    int mid = ((end-start)>>1) + start;
    int a = d.pairs[2*mid], b = d.pairs[2*mid+1];
    if (p0 > a) { if (start == mid) break; start = mid; }
    else if (p0 == a)
    {
      if (p1 > b) { if (start == mid) break; start = mid; }
      else if (p1 == b) return mid;
      else end = mid;
    }
    else end = mid;
  }
  return 0;
}

// normal damping coefficient of a master sphere i with partner code 'code'
// (forces.ispc:125-135): damper * 2 * sqrt(kn * m), m the reduced mass, or
// the sphere's mass against an obstacle triangle
__device__ __forceinline__ double pair_en(const PgDev &d, int i, int code)
{
  const int pi = d.part[i];
  int pj, colj;
  if (code >= 0) { pj = d.part[code]; colj = d.ellcol[code]; }
  else { pj = d.triobs[-code-1]; colj = d.tricol[-code-1]; }
  const int ij = pairing(d, d.ellcol[i], colj);
  const double ma = pj >= 0 ? 1.0 / (d.invm[pi] + d.invm[pj]) : d.mass[pi];
  const double kn = d.iparam[0][ij];
  return d.iparam[1][ij] * 2.0 * sqrt(kn*ma);
}

// ================================================================ candidate-list rebuild
// 0. clear the cell ranges of the previous sort
__device__ __forceinline__ void rb_clear_item(const PgDev &d, int s)
{
  unsigned key = d.keys[0][s];
  if (key == 0xffffffffu) return;          // entries of no scene own no cell
  d.cstart[key] = 0;
  d.cend[key] = 0;
}

// triangle reference vertices and widened float AABBs
__device__ __forceinline__ void rb_tref_item(const PgDev &d, int t)
{
  for (int k = 0; k < 9; k ++) d.tref[k][t] = d.tri[k][t];
  for (int c = 0; c < 3; c ++)
  {
    double lo = fmin(fmin(d.tri[c][t], d.tri[3+c][t]), d.tri[6+c][t]);
    double hi = fmax(fmax(d.tri[c][t], d.tri[3+c][t]), d.tri[6+c][t]);
    d.tbox[(size_t)c * d.trinum + t] = __double2float_rd(lo);
    d.tbox[(size_t)(3+c) * d.trinum + t] = __double2float_ru(hi);
  }
}

// 3. cell ranges, and the float centre, radius and particle of the sphere at
// each sorted position (the candidate search reads a cell's spheres from
// these contiguous copies)
__device__ __forceinline__ void rb_ranges_item(const PgDev &d, int s)
{
  const int n = d.ellnum;
  unsigned key = d.keys[0][s];
  {
    const int j = d.vals[0][s];
    d.cfs[s] = make_float4((float)d.center[0][j], (float)d.center[1][j], (float)d.center[2][j],
                           (float)d.radii[0][j]);
    d.pfs[s] = d.part[j];
  }
  if (key == 0xffffffffu) return;
  if (s == 0 || d.keys[0][s-1] != key) d.cstart[key] = s;
  if (s == n-1 || d.keys[0][s+1] != key) d.cend[key] = s + 1;
}

// 4. candidate list of sphere i with carried contact state
// Every lane of the warp calls it (valid: i is a sphere index): the triangle
// scan is shared by the warp.
__device__ __forceinline__ void rb_verlet_item(const PgDev &d, int i, bool valid)
{
  const int E = d.ellnum;
  int codes[MAXKN];
  int n = 0, nover = 0, ntri = 0;
  bool over = false;
  double c[3] = {0.0, 0.0, 0.0}, ri = 0.0;
  int pi = 0, sc = -1;
  if (valid)
  {
    for (int k = 0; k < 3; k ++) c[k] = d.center[k][i];
    ri = d.radii[0][i];
    pi = d.part[i];
    sc = d.escene[i];
  }
  const bool live = sc >= 0 && d.sactive[sc] != 0;
  if (live)
  {
    const unsigned prefix = (unsigned)sc << (3 * d.bits);
    // the sphere's cell, from the key the key phase computed, instead of
    // three FP64 divisions again
    const unsigned cm = d.ekey[i] & ((1u << (3 * d.bits)) - 1u);
    const int u[3] = {(int)compact3(cm), (int)compact3(cm >> 1), (int)compact3(cm >> 2)};
    // FP32 prefilter: a neighbour is skipped only when its float distance
    // exceeds the float limit by tol, more than the rounding of the float
    // copies and of the float arithmetic can account for, so the FP64 test
    // below still decides every candidate (the lists are those of the FP64
    // test alone).  Float coordinates carry at most 2^-24 |c| of error;
    // tol = 2^-20 (max|c_i| + 2 cell) bounds the distance error 16 times over
    // for partners within a cell.
    const float cif[3] = {(float)c[0], (float)c[1], (float)c[2]};
    const float rsf = (float)ri + (float)d.skin;
    const float tol = 9.5367431640625e-7f *
                      (fmaxf(fmaxf(fabsf(cif[0]), fabsf(cif[1])), fabsf(cif[2])) + 2.0f * (float)d.cell);
    for (int dz = -1; dz <= 1; dz ++)
      for (int dy = -1; dy <= 1; dy ++)
        for (int dx = -1; dx <= 1; dx ++)
        {
          int x = u[0]+dx, y = u[1]+dy, z = u[2]+dz;
          if (x < 0 || y < 0 || z < 0 || x >= d.dim[0] || y >= d.dim[1] || z >= d.dim[2]) continue;
          unsigned key = prefix | morton(x, y, z);
          int b = d.cstart[key], e = d.cend[key];
          for (int s = b; s < e; s ++)
          {
            const float4 q = d.cfs[s];
            const float f0 = cif[0] - q.x, f1 = cif[1] - q.y, f2 = cif[2] - q.z;
            const float lf = rsf + q.w + tol;
            if (f0*f0 + f1*f1 + f2*f2 >= lf*lf) continue;
            if (d.pfs[s] <= pi) continue;
            int j = d.vals[0][s];
            if ((unsigned)j >= (unsigned)E) continue;
            double q0 = c[0] - d.center[0][j], q1 = c[1] - d.center[1][j], q2 = c[2] - d.center[2][j];
            double lim = ri + d.radii[0][j] + d.skin;
            if (q0*q0 + q1*q1 + q2*q2 < lim*lim)
            {
              if (n < d.kn) codes[n ++] = j;
              else { over = true; nover ++; }
            }
          }
        }
    // insertion sort of the sphere partners
    for (int a = 1; a < n; a ++)
    {
      int v = codes[a], b = a - 1;
      while (b >= 0 && codes[b] > v) { codes[b+1] = codes[b]; b --; }
      codes[b+1] = v;
    }
  }
  // triangles of the sphere's scene within r + skin (AABB in float, then the
  // true closest-point distance), in triangle order
  const float inf = __int_as_float(0x7f800000);
  float clo[3] = {inf, inf, inf}, chi[3] = {-inf, -inf, -inf};
  if (live)
  {
    const float rr = (float)(ri + d.skin) * 1.0001f + 1e-30f;
    for (int k = 0; k < 3; k ++) { clo[k] = __double2float_rd(c[k]) - rr; chi[k] = __double2float_ru(c[k]) + rr; }
  }
  const int T = d.trinum;
  auto box_apart = [&](int t, const float *lo, const float *hi) {
    return d.tbox[t] > hi[0] || d.tbox[(size_t)3 * T + t] < lo[0] ||
           d.tbox[(size_t)T + t] > hi[1] || d.tbox[(size_t)4 * T + t] < lo[1] ||
           d.tbox[(size_t)2 * T + t] > hi[2] || d.tbox[(size_t)5 * T + t] < lo[2];
  };
  auto try_triangle = [&](int t) {
    if (box_apart(t, clo, chi)) return;
    double A[3], B[3], C[3], pnt[3], nrm[3];
    for (int q = 0; q < 3; q ++) { A[q] = d.tri[q][t]; B[q] = d.tri[3+q][t]; C[q] = d.tri[6+q][t]; }
    // the candidate test uses the true closest point: the reference's region
    // formula can only report a larger distance, so this set stays a superset
    double depth = pg::triangle_sphere(A, B, C, c, ri, pnt, nrm, false);
    if (!(depth > -d.skin) && !(depth != depth)) return;
    ntri ++;
    if (n < d.kn) codes[n ++] = -(t + 1);
    else { over = true; nover ++; }
  };
  // when every live lane of the warp is in one scene, the warp tests 32
  // triangles at a time against the box of all its spheres and each lane
  // then tests its own box against the triangles that box reached
  const unsigned full = 0xffffffffu, lm = __ballot_sync(full, live);
  if (!lm) return;
  const int lane = threadIdx.x & 31, sc0 = __shfl_sync(full, sc, __ffs(lm) - 1);
  if (__all_sync(full, !live || sc == sc0))
  {
    float wlo[3], whi[3];
    for (int k = 0; k < 3; k ++)
    {
      wlo[k] = clo[k]; whi[k] = chi[k];
      for (int o = 16; o > 0; o >>= 1)
      {
        wlo[k] = fminf(wlo[k], __shfl_xor_sync(full, wlo[k], o));
        whi[k] = fmaxf(whi[k], __shfl_xor_sync(full, whi[k], o));
      }
    }
    const int tb = d.stbeg[sc0], te = d.stend[sc0];
    for (int t0 = tb; t0 < te; t0 += 32)
    {
      const int t = t0 + lane;
      unsigned hm = __ballot_sync(full, t < te && !box_apart(t, wlo, whi));
      while (hm)
      {
        const int tt = t0 + __ffs(hm) - 1;
        hm &= hm - 1;
        if (live) try_triangle(tt);
      }
    }
  }
  else if (live)
    for (int t = d.stbeg[sc]; t < d.stend[sc]; t ++) try_triangle(t);
  // one atomic per warp for the largest list and triangle counts
  {
    const int cmax = __reduce_max_sync(full, live ? n + nover : 0);
    const int tmax = __reduce_max_sync(full, live ? ntri : 0);
    if (lane == 0)
    {
      if (cmax > 0) atomicMax(&d.stats[1], cmax);
      if (tmax > 0) atomicMax(&d.stats[3], tmax);
    }
  }
  if (!live) return;
  if (over) set_err(d, PG_ERR_CAPACITY, 1, i, n + nover);

  // merge with the previous list (both in partner order)
  const int nold = d.ncnt[i];
  int ocode[MAXKN];
  unsigned char oflag[MAXKN];
  double ost[3][MAXKN];
  // the tangential state lives in the FP64 arrays (FP64 form) or the FP32
  // arrays (mixed form); it moves with its contact either way
  const bool mixed = d.form == PG_FORM_MIXED;
  for (int k = 0; k < nold; k ++)
  {
    size_t idx = (size_t)k * d.estride + i;
    ocode[k] = d.ncode[idx];
    oflag[k] = d.nflag[idx];
    for (int c = 0; c < 3; c ++) ost[c][k] = mixed ? (double)d.nstate_f[c][idx] : d.nstate[c][idx];
  }
  int o = 0;
  for (int k = 0; k < n; k ++)
  {
    unsigned key = order_key(codes[k]);
    while (o < nold && order_key(ocode[o]) < key) o ++;
    size_t idx = (size_t)k * d.estride + i;
    d.ncode[idx] = codes[k];
    if (d.nen) d.nen[idx] = pair_en(d, i, codes[k]);
    const bool kept = o < nold && ocode[o] == codes[k];
    d.nflag[idx] = kept ? oflag[o] : 0;
    for (int c = 0; c < 3; c ++)
    {
      double st = kept ? ost[c][o] : 0.0;
      if (mixed) d.nstate_f[c][idx] = (float)st;
      else d.nstate[c][idx] = st;
    }
  }
  d.ncnt[i] = n;
}

// 5. slave lists (CSR): count entries per sphere in particle order, emit
// (partner, entry) pairs in (master particle, slot) order, then a stable sort
// by partner gives every particle's entries in that order
__device__ __forceinline__ void rb_rzero_item(const PgDev &d, int p) { d.rcnt[p] = 0; }

__device__ __forceinline__ void rb_count_item(const PgDev &d, int q)
{
  d.eoff[q] = d.ncnt[d.eorder[q]];
}

__device__ __forceinline__ void rb_emit_item(const PgDev &d, int q)
{
  const int E = d.ellnum, P = d.parnum;
  const int i = d.eorder[q];
  const int n = d.ncnt[i];
  const int base = d.eoff[q];
  for (int k = 0; k < n; k ++)
  {
    const int code = d.ncode[(size_t)k * d.estride + i];
    const int pj = code >= 0 ? d.part[code] : d.triobs[-code - 1];
    const bool ok = pj >= 0 && pj < P;
    d.skey[0][base + k] = ok ? (unsigned)pj : 0xffffffffu;
    d.sval[0][base + k] = k * d.estride + i;
    if (ok) atomicAdd(&d.rcnt[pj], 1);
  }
}

__device__ __forceinline__ void rb_soff_item(const PgDev &d, int p)
{
  const int n = d.rcnt[p];
  d.soff[p] = n;
  d.rcnt[p] = 0;                 // the placement cursor of the entry scatter
  // one atomic per warp for the largest slave count (of the session and of
  // this rebuild)
  const unsigned am = __activemask();
  const int wmax = __reduce_max_sync(am, n);
  if ((threadIdx.x & 31) == __ffs(am) - 1 && wmax > 0)
  {
    atomicMax(&d.stats[2], wmax);
    atomicMax(&d.smeta[4], wmax);
  }
}

// Slave lists whose longest list has at most PG_SLAVE_PLACE_MAX entries are
// built without the entry sort: every entry goes to its partner's next free
// position (an atomic cursor), then each particle orders its few entries by
// emit position, the order the stable sort by partner gives them.
constexpr int PG_SLAVE_PLACE_MAX = 64;

__device__ __forceinline__ void rb_place_item(const PgDev &d, int e)
{
  const unsigned pj = d.skey[0][e];
  if (pj == 0xffffffffu) return;
  const int at = d.soff[pj] + atomicAdd(&d.rcnt[pj], 1);
  d.skey[1][at] = (unsigned)e;
  d.sval[1][at] = d.sval[0][e];
}

__device__ __forceinline__ void rb_order_item(const PgDev &d, int p, int *dst)
{
  const int b = d.soff[p], n = d.soff[p+1] - b;
  unsigned key[PG_SLAVE_PLACE_MAX];
  int val[PG_SLAVE_PLACE_MAX];
  for (int a = 0; a < n; a ++)
  {
    const unsigned k = d.skey[1][b + a];
    const int v = d.sval[1][b + a];
    int c = a - 1;
    while (c >= 0 && key[c] > k) { key[c+1] = key[c]; val[c+1] = val[c]; c --; }
    key[c+1] = k;
    val[c+1] = v;
  }
  for (int a = 0; a < n; a ++) dst[b + a] = val[a];
}

// sizes of the entry sort (one thread): entries, tiles, histogram length and
// its scan tiles
__device__ __forceinline__ void rb_meta_item(const PgDev &d)
{
  const int n = d.eoff[d.ellnum];
  const int nb = n > 0 ? (n + SORT_TILE - 1) / SORT_TILE : 1;
  d.smeta[0] = n;
  d.smeta[1] = nb;
  d.smeta[2] = 256 * nb;
  d.smeta[3] = (256 * nb + SCAN_TILE - 1) / SCAN_TILE;
}

// end of a rebuild (one thread)
__device__ __forceinline__ void rb_done_item(const PgDev &d)
{
  if (*d.rebuild)
  {
    *d.rebuild = 0;
    d.stats[0] += 1;
  }
}

// ================================================================ cooperative grids
__device__ __forceinline__ unsigned long long global_ns()
{
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// barrier of all blocks of a cooperative grid.  d.gbar = {arrivals,
// generation, abort}.  A block that waits more than 2 s records
// PG_ERR_TIMEOUT and raises abort; every block then leaves its kernel
// (a false return).
static __device__ __noinline__ bool grid_barrier(const PgDev &d)
{
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0)
  {
    volatile unsigned *b = d.gbar;
    int ok = 1;
    const unsigned gen = b[1];
    __threadfence();
    if (b[2] != 0u) ok = 0;
    else
    {
      const unsigned arrived = atomicAdd(d.gbar, 1u) + 1u;
      if (arrived == gridDim.x)
      {
        atomicExch(d.gbar, 0u);
        __threadfence();
        atomicAdd(d.gbar + 1, 1u);
      }
      else
      {
        const unsigned long long t0 = global_ns();
        while (b[1] == gen)
        {
          if (b[2] != 0u) { ok = 0; break; }
          if (global_ns() - t0 > 2000000000ull)
          {
            atomicExch(d.gbar + 2, 1u);
            set_err(d, PG_ERR_TIMEOUT, 20, blockIdx.x, 0);
            ok = 0;
            break;
          }
          __nanosleep(32);
        }
      }
    }
    __threadfence();
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

// exclusive scan of a[0..n) by the whole grid (tile sums | their scan by
// block 0 | tiles), ending with a barrier; false when a barrier gave up
template <typename T>
__device__ bool grid_scan(const PgDev &d, T *a, int n, T *bs, T *sh)
{
  const int tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  for (int t = blockIdx.x; t < tiles; t += gridDim.x)
  {
    const T s = scan_tile_sum(a, n, t, sh);
    if (threadIdx.x == 0) bs[t] = s;
  }
  if (!grid_barrier(d)) return false;
  if (blockIdx.x == 0) block_scan_seq(bs, tiles, sh);
  if (!grid_barrier(d)) return false;
  for (int t = blockIdx.x; t < tiles; t += gridDim.x) scan_tile_apply(a, n, t, bs[t], sh);
  return grid_barrier(d);
}

template <int B>
union RebuildSmem
{
  unsigned h[256];
  struct { unsigned wcnt[SORT_THREADS / 32][256]; unsigned goff[256]; } sc;
  unsigned part[B];
};

struct NoHook
{
  __device__ void operator()(const PgDev &, int) const {}
};

// the whole candidate-list rebuild by a cooperative grid of B-thread blocks
// (B >= 256): clear | keys | key sort (passes) | ranges | lists | slave lists
// (counts | scan | emit | offsets | scan | entry sort (epasses, the result in
// sval[epasses & 1]) ).  'hook' runs for every sphere in the first phase.
// Returns false when a barrier gave up.
template <int B, class Hook>
__device__ bool rebuild_all(const PgDev &d, int passes, int epasses, RebuildSmem<B> &sm, Hook hook)
{
  const int gsz = gridDim.x * B;
  const int g0 = blockIdx.x * B + threadIdx.x;
  const int E = d.ellnum, P = d.parnum, T = d.trinum;
  for (int s = g0; s < E; s += gsz) { rb_clear_item(d, s); hook(d, s); }
  for (int t = g0; t < T; t += gsz) rb_tref_item(d, t);
  if (!grid_barrier(d)) return false;
  Grid g;
  for (int k = 0; k < 3; k ++) { g.org[k] = 0.0; g.dim[k] = d.dim[k]; }
  g.cell = d.cell;
  for (int i = g0; i < E; i += gsz)
  {
    cell_keys_item(i, d.center[0], d.center[1], d.center[2], g, d.escene, d.sorg[0], d.sorg[1], d.sorg[2],
                   3 * d.bits, d.keys[0], d.vals[0], d.cref[0], d.cref[1], d.cref[2]);
    d.ekey[i] = d.keys[0][i];        // the sort reorders keys[]; the search reads its own cell here
  }
  if (!grid_barrier(d)) return false;
  const int nb = d.nsortblocks;
  for (int p = 0; p < passes; p ++)
  {
    unsigned *ks = (p & 1) ? d.keys[1] : d.keys[0], *kd = (p & 1) ? d.keys[0] : d.keys[1];
    int *vs = (p & 1) ? d.vals[1] : d.vals[0], *vd = (p & 1) ? d.vals[0] : d.vals[1];
    for (int tile = blockIdx.x; tile < nb; tile += gridDim.x) sort_hist_tile(ks, E, d.hist, nb, 8 * p, tile, sm.h);
    if (!grid_barrier(d)) return false;
    if (!grid_scan(d, d.hist, 256 * nb, (unsigned *)d.sbs, sm.part)) return false;
    for (int tile = blockIdx.x; tile < nb; tile += gridDim.x)
      sort_scatter_tile(ks, vs, kd, vd, E, d.hist, nb, 8 * p, tile, sm.sc.wcnt, sm.sc.goff);
    if (!grid_barrier(d)) return false;
  }
  for (int s = g0; s < E; s += gsz) rb_ranges_item(d, s);
  if (!grid_barrier(d)) return false;
  for (int i = g0; i - (int)(threadIdx.x & 31) < E; i += gsz) rb_verlet_item(d, i, i < E);
  if (!grid_barrier(d)) return false;
  for (int p = g0; p < P; p += gsz) rb_rzero_item(d, p);
  for (int q = g0; q < E; q += gsz) rb_count_item(d, q);
  if (g0 == 0) { d.eoff[E] = 0; d.smeta[4] = 0; }
  if (!grid_barrier(d)) return false;
  if (!grid_scan(d, d.eoff, E + 1, (int *)d.sbs, (int *)sm.part)) return false;
  for (int q = g0; q < E; q += gsz) rb_emit_item(d, q);
  if (!grid_barrier(d)) return false;
  for (int p = g0; p < P; p += gsz) rb_soff_item(d, p);
  if (g0 == 0) { d.soff[P] = 0; rb_meta_item(d); }
  if (!grid_barrier(d)) return false;
  if (!grid_scan(d, d.soff, P + 1, (int *)d.sbs, (int *)sm.part)) return false;
  if (d.smeta[4] <= PG_SLAVE_PLACE_MAX)
  {
    // short lists: placement and per-particle ordering, the result where
    // the entry sort would leave it (sval[epasses & 1])
    const int n = d.smeta[0];
    for (int e = g0; e < n; e += gsz) rb_place_item(d, e);
    if (!grid_barrier(d)) return false;
    int *dst = d.sval[epasses & 1];
    for (int p = g0; p < P; p += gsz) rb_order_item(d, p, dst);
  }
  else
  {
    const int n = d.smeta[0], nbe = d.smeta[1];
    for (int p = 0; p < epasses; p ++)
    {
      unsigned *ks = (p & 1) ? d.skey[1] : d.skey[0], *kd = (p & 1) ? d.skey[0] : d.skey[1];
      int *vs = (p & 1) ? d.sval[1] : d.sval[0], *vd = (p & 1) ? d.sval[0] : d.sval[1];
      for (int tile = blockIdx.x; tile < nbe; tile += gridDim.x)
        sort_hist_tile(ks, n, d.shist, nbe, 8 * p, tile, sm.h);
      if (!grid_barrier(d)) return false;
      if (!grid_scan(d, d.shist, 256 * nbe, (unsigned *)d.sbs, sm.part)) return false;
      for (int tile = blockIdx.x; tile < nbe; tile += gridDim.x)
        sort_scatter_tile(ks, vs, kd, vd, n, d.shist, nbe, 8 * p, tile, sm.sc.wcnt, sm.sc.goff);
      if (!grid_barrier(d)) return false;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) rb_done_item(d);
  return grid_barrier(d);
}


// ================================================================ per-step scene state
// gravity of scene sc for this step: the step table's row, or the scene's
// base excitation g0 + dir * sum_k amp_k sin(2 pi freq_k t + phase_k) at its
// local time t = (global step - start step) * step.  Written with explicit
// round-to-nearest operations: the same bits whether or not the compiler
// contracts multiply-adds.
__device__ __forceinline__ void excite_item(const PgDev &d, int sc, double step)
{
  const double *tab = d.t_gravity + 3*(size_t)(*d.stepno);
  if (sc == 0 && d.damp_f)
  {
    const double *damp = d.t_damping + 6*(size_t)(*d.stepno);
    for (int k = 0; k < 6; k ++) d.damp_f[k] = (float)damp[k];
  }
  if (!d.sexc_on[sc])
  {
    d.sgrav[3*sc] = tab[0]; d.sgrav[3*sc+1] = tab[1]; d.sgrav[3*sc+2] = tab[2];
    if (d.sgrav_f) { d.sgrav_f[3*sc] = (float)tab[0]; d.sgrav_f[3*sc+1] = (float)tab[1]; d.sgrav_f[3*sc+2] = (float)tab[2]; }
    return;
  }
  const double *e = d.sexc + (size_t)PG_EXC_LEN * sc;
  const double t = __dmul_rn((double)(*d.gstep - d.sstart[sc]), step);
  int nk = (int)e[6];
  if (nk > 8) nk = 8;
  const double two_pi = 2.0 * 3.14159265358979323846;
  double sum = 0.0;
  for (int k = 0; k < nk; k ++)
    sum = __dadd_rn(sum, __dmul_rn(e[8+3*k], sin(__dadd_rn(__dmul_rn(__dmul_rn(two_pi, e[9+3*k]), t), e[10+3*k]))));
  d.sgrav[3*sc] = __dadd_rn(e[0], __dmul_rn(e[3], sum));
  d.sgrav[3*sc+1] = __dadd_rn(e[1], __dmul_rn(e[4], sum));
  d.sgrav[3*sc+2] = __dadd_rn(e[2], __dmul_rn(e[5], sum));
  if (d.sgrav_f)
    for (int k = 0; k < 3; k ++) d.sgrav_f[3*sc+k] = (float)d.sgrav[3*sc+k];
}

// obstacle triangle t moved by its obstacle's velocities (obstacles.ispc:28-78):
// the row of the step table (use_row) or the current obsang/obslin state.
// Returns whether a vertex left its rebuild neighbourhood.
__device__ __forceinline__ bool obstacles_item(const PgDev &d, int t, double step, int use_row)
{
  const int o = d.triown[t];
  if (o < 0) return false;
  // every load that needs only t and o is issued before the scene test, so
  // that one memory latency covers them (the update is a short chain)
  const int sc = d.tscene[t];
  const double *ang, *lin;
  if (use_row)
  {
    const int row = *d.stepno;
    ang = d.t_obs_ang + (size_t)row * d.tab_obs_stride + 3*o;
    lin = d.t_obs_lin + (size_t)row * d.tab_obs_stride + 3*o;
  }
  else
  {
    ang = d.obsang + 3*o;
    lin = d.obslin + 3*o;
  }
  const double *x = d.obspnt + 3*o;
  double V[9], R[9];
  for (int k = 0; k < 9; k ++) { V[k] = d.tri[k][t]; R[k] = d.tref[k][t]; }
  const double a[3] = {ang[0], ang[1], ang[2]}, l[3] = {lin[0], lin[1], lin[2]}, p[3] = {x[0], x[1], x[2]};
  if (sc < 0 || !d.sactive[sc]) return false;
  const bool typo = (d.compat & PG_COMPAT_EXPMAP) != 0;
  bool need = false;
  double y[3], DL[9], z[3];
  y[0] = p[0] + step*l[0];
  y[1] = p[1] + step*l[1];
  y[2] = p[2] + step*l[2];
  pg::expmap(step*a[0], step*a[1], step*a[2], DL, typo);
  for (int v = 0; v < 3; v ++)
  {
    z[0] = V[3*v+0] - p[0];
    z[1] = V[3*v+1] - p[1];
    z[2] = V[3*v+2] - p[2];
    double n0 = DL[0]*z[0]+DL[3]*z[1]+DL[6]*z[2] + y[0];
    double n1 = DL[1]*z[0]+DL[4]*z[1]+DL[7]*z[2] + y[1];
    double n2 = DL[2]*z[0]+DL[5]*z[1]+DL[8]*z[2] + y[2];
    d.tri[3*v+0][t] = n0;
    d.tri[3*v+1][t] = n1;
    d.tri[3*v+2][t] = n2;
    double r0 = n0 - R[3*v+0], r1 = n1 - R[3*v+1], r2 = n2 - R[3*v+2];
    need |= pg::gt_nonneg(r0*r0 + r1*r1 + r2*r2, d.half_skin_sq);
  }
  return need;
}

// obstacle points (after every triangle used the old point), obstacle
// velocity state, and the step counters (one thread)
__device__ __forceinline__ void tail_item(const PgDev &d, double step, int use_row)
{
  const int row = use_row ? *d.stepno : 0;
  const long long gs = use_row ? *d.gstep : 0;
  for (int o = 0; o < d.obsnum; o ++)
  {
    // the obstacle's loads first, then its scene test (one memory latency)
    const int sc = d.oscene[o];
    double *x = d.obspnt + 3*o;
    const double p[3] = {x[0], x[1], x[2]};
    double a[3], v[3];
    if (use_row)
      for (int k = 0; k < 3; k ++)
      {
        a[k] = d.t_obs_ang[(size_t)row * d.tab_obs_stride + 3*o + k];
        v[k] = d.t_obs_lin[(size_t)row * d.tab_obs_stride + 3*o + k];
      }
    else
      for (int k = 0; k < 3; k ++) v[k] = d.obslin[3*o+k];
    if (sc < 0 || !d.sactive[sc]) continue;
    if (use_row)
      for (int k = 0; k < 3; k ++) { d.obsang[3*o+k] = a[k]; d.obslin[3*o+k] = v[k]; }
    x[0] = p[0] + step*v[0]; x[1] = p[1] + step*v[1]; x[2] = p[2] + step*v[2];
  }
  if (use_row)
  {
    *d.stepno = row + 1;
    *d.gstep = gs + 1;
  }
}

} // namespace pgk
