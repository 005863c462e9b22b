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
#include "../../include/parmec_gb300.h"

namespace {

constexpr int TPB = 128;
constexpr int MAXKN = 96;                               // upper bound of slots per sphere

inline int nblk(int n) { return (n + TPB - 1) / TPB; }

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

__device__ __forceinline__ void cell_of(const PgDev &d, int scene, const double *c, int *u)
{
  for (int k = 0; k < 3; k ++)
  {
    double f = floor((c[k] - d.sorg[k][scene]) / d.cell);
    if (!(f >= 0.0)) f = 0.0;                 // also catches NaN
    if (f > (double)(d.dim[k] - 1)) f = (double)(d.dim[k] - 1);
    u[k] = (int)f;
  }
}

__device__ __forceinline__ unsigned morton(int x, int y, int z)
{
  return spread3((unsigned)x) | (spread3((unsigned)y) << 1) | (spread3((unsigned)z) << 2);
}

// ---- 0. clear the cell ranges of the previous sort
__global__ void k_rb_clear(PgDev d)
{
  if (!*d.rebuild) return;
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= d.ellnum) return;
  unsigned key = d.keys[0][s];
  if (key == 0xffffffffu) return;          // entries of no scene own no cell
  d.cstart[key] = 0;
  d.cend[key] = 0;
}

// ---- triangle reference vertices and widened float AABBs
__global__ void k_rb_tref(PgDev d)
{
  if (!*d.rebuild) return;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.trinum) return;
  for (int k = 0; k < 9; k ++) d.tref[k][t] = d.tri[k][t];
  for (int c = 0; c < 3; c ++)
  {
    double lo = fmin(fmin(d.tri[c][t], d.tri[3+c][t]), d.tri[6+c][t]);
    double hi = fmax(fmax(d.tri[c][t], d.tri[3+c][t]), d.tri[6+c][t]);
    d.tbox[(size_t)c * d.trinum + t] = __double2float_rd(lo);
    d.tbox[(size_t)(3+c) * d.trinum + t] = __double2float_ru(hi);
  }
}

// ---- 3. cell ranges
__global__ void k_rb_ranges(PgDev d)
{
  if (!*d.rebuild) return;
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = d.ellnum;
  if (s >= n) return;
  unsigned key = d.keys[0][s];
  if (key == 0xffffffffu) return;
  if (s == 0 || d.keys[0][s-1] != key) d.cstart[key] = s;
  if (s == n-1 || d.keys[0][s+1] != key) d.cend[key] = s + 1;
}

__device__ __forceinline__ unsigned order_key(int code)
{
  return code >= 0 ? (unsigned)code : 0x80000000u + (unsigned)(-code - 1);
}

// ---- 4. candidate lists with carried contact state
__global__ void __launch_bounds__(TPB) k_rb_verlet(PgDev d)
{
  if (!*d.rebuild) return;
  const int E = d.ellnum;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= E) return;
  int codes[MAXKN];
  int n = 0, nsph = 0, nover = 0, ntri = 0;
  bool over = false;
  double c[3] = {d.center[0][i], d.center[1][i], d.center[2][i]};
  const double ri = d.radii[0][i];
  const int pi = d.part[i];
  const int sc = d.escene[i];
  const bool live = sc >= 0 && d.sactive[sc] != 0;
  if (live)
  {
    const unsigned prefix = (unsigned)sc << (3 * d.bits);
    int u[3];
    cell_of(d, sc, c, u);
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
            int j = d.vals[0][s];
            if ((unsigned)j >= (unsigned)E || d.part[j] <= pi) continue;
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
    nsph = n;
    // triangles of the sphere's scene within r + skin (AABB in float, then the
    // true closest-point distance)
    const float rr = (float)(ri + d.skin) * 1.0001f + 1e-30f;
    const float clo[3] = {__double2float_rd(c[0]) - rr, __double2float_rd(c[1]) - rr, __double2float_rd(c[2]) - rr};
    const float chi[3] = {__double2float_ru(c[0]) + rr, __double2float_ru(c[1]) + rr, __double2float_ru(c[2]) + rr};
    const int T = d.trinum;
    for (int t = d.stbeg[sc]; t < d.stend[sc]; t ++)
    {
      if (d.tbox[t] > chi[0] || d.tbox[(size_t)3 * T + t] < clo[0] ||
          d.tbox[(size_t)T + t] > chi[1] || d.tbox[(size_t)4 * T + t] < clo[1] ||
          d.tbox[(size_t)2 * T + t] > chi[2] || d.tbox[(size_t)5 * T + t] < clo[2]) continue;
      double A[3], B[3], C[3], pnt[3], nrm[3];
      for (int q = 0; q < 3; q ++) { A[q] = d.tri[q][t]; B[q] = d.tri[3+q][t]; C[q] = d.tri[6+q][t]; }
      // the candidate test uses the true closest point: the reference's region
      // formula can only report a larger distance, so this set stays a superset
      double depth = pg::triangle_sphere(A, B, C, c, ri, pnt, nrm, false);
      if (!(depth > -d.skin) && !(depth != depth)) continue;
      ntri ++;
      if (n < d.kn) codes[n ++] = -(t + 1);
      else { over = true; nover ++; }
    }
  }
  if (!live) return;
  if (over) set_err(d, PG_ERR_CAPACITY, 1, i, n + nover);
  atomicMax(&d.stats[1], n + nover);
  atomicMax(&d.stats[3], ntri);

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
    size_t idx = (size_t)k * E + i;
    ocode[k] = d.ncode[idx];
    oflag[k] = d.nflag[idx];
    for (int c = 0; c < 3; c ++) ost[c][k] = mixed ? (double)d.nstate_f[c][idx] : d.nstate[c][idx];
  }
  int o = 0;
  for (int k = 0; k < n; k ++)
  {
    unsigned key = order_key(codes[k]);
    while (o < nold && order_key(ocode[o]) < key) o ++;
    size_t idx = (size_t)k * E + i;
    d.ncode[idx] = codes[k];
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
  (void)nsph;
}

// ---- 5. slave lists
__global__ void k_rb_rzero(PgDev d)
{
  if (!*d.rebuild) return;
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < d.parnum) d.rcnt[p] = 0;
}

__global__ void k_rb_rfill(PgDev d)
{
  if (!*d.rebuild) return;
  const int E = d.ellnum;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= E) return;
  const int n = d.ncnt[i];
  for (int k = 0; k < n; k ++)
  {
    int code = d.ncode[(size_t)k * E + i];
    int pj = code >= 0 ? d.part[code] : d.triobs[-code - 1];
    if (pj < 0 || pj >= d.parnum) continue;
    int r = atomicAdd(&d.rcnt[pj], 1);
    if (r < d.kr) d.rref[(size_t)r * d.parnum + pj] = k * E + i;
    else set_err(d, PG_ERR_CAPACITY, 3, pj, r + 1);
  }
}

__global__ void k_rb_rsort(PgDev d)
{
  if (!*d.rebuild) return;
  const int P = d.parnum, E = d.ellnum;
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  int n = d.rcnt[p];
  atomicMax(&d.stats[2], n);
  if (n > d.kr) { n = d.kr; d.rcnt[p] = n; }
  unsigned long long key[MAXKN];
  int ref[MAXKN];
  for (int r = 0; r < n; r ++)
  {
    int v = d.rref[(size_t)r * P + p];
    int i = v % E, k = v / E;
    key[r] = ((unsigned long long)(unsigned)d.part[i] << 32) | (unsigned)k;
    ref[r] = v;
  }
  for (int a = 1; a < n; a ++)
  {
    unsigned long long kv = key[a];
    int rv = ref[a], b = a - 1;
    while (b >= 0 && key[b] > kv) { key[b+1] = key[b]; ref[b+1] = ref[b]; b --; }
    key[b+1] = kv;
    ref[b+1] = rv;
  }
  for (int r = 0; r < n; r ++) d.rref[(size_t)r * P + p] = ref[r];
}

__global__ void k_rb_done(PgDev d)
{
  if (threadIdx.x == 0 && blockIdx.x == 0 && *d.rebuild)
  {
    *d.rebuild = 0;
    d.stats[0] += 1;
  }
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
  if (!(d.skin > 0.0)) d.skin = 0.3 * rmin;
  d.half_skin_sq = (0.45 * d.skin) * (0.45 * d.skin);
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

void pg_launch_rebuild(const PgDev &d, cudaStream_t s)
{
  const int E = d.ellnum;
  if (!E) return;
  k_rb_clear<<<nblk(E), TPB, 0, s>>>(d);
  pg_launch_cell_keys(d.center[0], d.center[1], d.center[2], E, nullptr, d.cell, d.dim, d.keys[0], d.vals[0],
                      d.cref[0], d.cref[1], d.cref[2], d.rebuild, s, d.escene, d.sorg, 3 * d.bits);
  if (d.trinum) k_rb_tref<<<nblk(d.trinum), TPB, 0, s>>>(d);
  pg_launch_radix_sort(d.keys[0], d.vals[0], d.keys[1], d.vals[1], d.hist, E, pg_sort_passes_bits(pg_rebuild_sort_bits(d)),
                       d.rebuild, s);
  k_rb_ranges<<<nblk(E), TPB, 0, s>>>(d);
  k_rb_verlet<<<nblk(E), TPB, 0, s>>>(d);
  k_rb_rzero<<<nblk(d.parnum), TPB, 0, s>>>(d);
  k_rb_rfill<<<nblk(E), TPB, 0, s>>>(d);
  k_rb_rsort<<<nblk(d.parnum), TPB, 0, s>>>(d);
  k_rb_done<<<1, 32, 0, s>>>(d);
}

int pg_rebuild_kernel_count(const PgDev &d)
{
  if (!d.ellnum) return 0;
  return 2 + (d.trinum ? 1 : 0) + 3 * pg_sort_passes_bits(pg_rebuild_sort_bits(d)) + 6;
}
