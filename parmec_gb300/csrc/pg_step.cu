// pg_step.cu -- the per-step DEM kernels (FP64 form).
//
// One step of the reference loop (parmec.cpp:2418-2517) runs as
//   [rebuild of candidate lists, only when some sphere moved > skin/2]
//   k_contacts   per sphere: narrow phase of its candidates, granular force,
//                contact state, master-side partial sums  (condet + contacts_task)
//   k_springs    per spring: nonlinear spring/dashpot/friction force (springs_task)
//   k_integrate  per particle: slave-side sums + gravity + spring flushes,
//                prescribed motion, Lie-group integration, sphere centres
//                (contacts_acc_task + prescribe_* + dynamics_task + ellipsoids_task)
//   k_nodes/k_faces, k_obstacles, k_tail
// All sums run in a fixed order (master list in partner order, then slave
// list in master order), so results repeat bit for bit from run to run.
#include <cuda_runtime.h>
#include "pg_state.h"
#include "pg_math.cuh"
#include "pg_launch.h"
#include "pg_items.cuh"
#include "../../include/parmec_gb300.h"

using namespace pg;

namespace {

constexpr int TPB = 128;

// minimum resident blocks per SM asked of the FP64 particle update and of
// the contact evaluation (register budget against warps in flight)
#ifndef PG_INTEGRATE_MINB
#define PG_INTEGRATE_MINB 1
#endif
#ifndef PG_EVAL_MINB
#define PG_EVAL_MINB 8
#endif
#if PG_INTEGRATE_MINB
#define PG_LB_INTEGRATE __launch_bounds__(TPB, PG_INTEGRATE_MINB)
#else
#define PG_LB_INTEGRATE __launch_bounds__(TPB)
#endif
#if PG_EVAL_MINB
#define PG_LB_EVAL __launch_bounds__(TPB, PG_EVAL_MINB)
#else
#define PG_LB_EVAL __launch_bounds__(TPB)
#endif

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

__device__ __forceinline__ void flag_rebuild(const PgDev &d, bool need)
{
  unsigned m = __ballot_sync(__activemask(), need);
  if (m && (threadIdx.x & 31) == (__ffs(m) - 1)) atomicExch(d.rebuild, 1);
}


// gravity of a particle's scene for this step (written by k_excite)
__device__ __forceinline__ void scene_gravity(const PgDev &d, int sc, double, const double *, double g[3])
{
  g[0] = d.sgrav[3*sc]; g[1] = d.sgrav[3*sc+1]; g[2] = d.sgrav[3*sc+2];
}

// ---------------------------------------------------------------- excitation
// gravity of every scene for this step: the step table's row, or the scene's
// base excitation g0 + dir * sum_k amp_k sin(2 pi freq_k t + phase_k) at its
// local time t = (global step - start step) * step
__global__ void k_excite(PgDev d, double step)
{
  const int sc = blockIdx.x * blockDim.x + threadIdx.x;
  if (sc < d.nscene) pgk::excite_item(d, sc, step);
}

// ---------------------------------------------------------------- isotropic bodies
// A sphere's inertia is j*I and its inverse (1/j)*I, off-diagonals +0.  The
// 3x3 products with them then reduce to j*x per row, except for the sign of
// an exact zero: IEEE gives x + (+-0) = x for x != 0, and a sum of zeros is
// -0 only when every term is -0.  iso_nvmul replays that with integer bit
// tests, so its results equal nvmul's bit for bit (non-finite inputs take
// the full product).
__device__ __forceinline__ void set_piso(const PgDev &d, int i)
{
  if (!d.piso) return;
  const unsigned long long j = dbits(d.inertia[0][i]), ij = dbits(d.inverse[0][i]);
  bool iso = dbits(d.inertia[4][i]) == j && dbits(d.inertia[8][i]) == j &&
             dbits(d.inverse[4][i]) == ij && dbits(d.inverse[8][i]) == ij;
  const int off[6] = {1, 2, 3, 5, 6, 7};
  for (int k = 0; k < 6; k ++)
    iso = iso && dbits(d.inertia[off[k]][i]) == 0 && dbits(d.inverse[off[k]][i]) == 0;
  d.piso[i] = iso ? 1 : 0;
}

__device__ __forceinline__ bool finite_bits(double x) { return finite_d(x); }

// p + 0*a + 0*b as the full product sums them, for finite a and b
__device__ __forceinline__ double zero_terms(double p, double a, double b)
{
  const long long bp = (long long)dbits(p);
  if ((bp << 1) != 0) return p;
  const bool neg = bp < 0 && (long long)dbits(a) < 0 && (long long)dbits(b) < 0;
  return __longlong_as_double(neg ? (long long)0x8000000000000000ull : 0ll);
}

// C = (j*I) B, bit for bit as nvmul with the full matrix
__device__ __forceinline__ void iso_nvmul(double j, const double *B, double *C)
{
  if (finite_bits(B[0]) && finite_bits(B[1]) && finite_bits(B[2]))
  {
    C[0] = zero_terms(j*B[0], B[1], B[2]);
    C[1] = zero_terms(j*B[1], B[0], B[2]);
    C[2] = zero_terms(j*B[2], B[0], B[1]);
  }
  else
  {
    const double M[9] = {j, 0.0, 0.0, 0.0, j, 0.0, 0.0, 0.0, j};
    nvmul(M, B, C);
  }
}

__global__ void k_iso_flags(PgDev d, int p0, int p1)
{
  int i = p0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i < p1) set_piso(d, i);
}

// ---------------------------------------------------------------- invert (parmec.ispc:62-99)
__global__ void k_invert(PgDev d)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.parnum) return;
  double a[9], x[9];
  for (int j = 0; j < 9; j ++) a[j] = d.inertia[j][i];
  for (int j = 0; j < 9; j ++) x[j] = 0.0;
  invert3(a, x);
  for (int j = 0; j < 9; j ++) d.inverse[j][i] = x[j];
  d.invm[i] = 1.0 / d.mass[i];
  set_piso(d, i);
}

// ---------------------------------------------------------------- euler (parmec.ispc:224-272)
__global__ void k_euler(PgDev d, double step)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.parnum) return;
  const bool typo = (d.compat & PG_COMPAT_EXPMAP) != 0;
  double O[3], L1[9], DL[9], L2[9], o[3];
  O[0] = step*d.angular[0][i];
  O[1] = step*d.angular[1][i];
  O[2] = step*d.angular[2][i];
  expmap(O[0], O[1], O[2], DL, typo);
  for (int k = 0; k < 9; k ++) L1[k] = d.rotation[k][i];
  nnmul(L1, DL, L2);
  for (int k = 0; k < 9; k ++) d.rotation[k][i] = L2[k];
  nvmul(L2, O, o);
  d.angular[3][i] = o[0];
  d.angular[4][i] = o[1];
  d.angular[5][i] = o[2];
  d.position[0][i] += step * d.linear[0][i];
  d.position[1][i] += step * d.linear[1][i];
  d.position[2][i] += step * d.linear[2][i];
}

// ---------------------------------------------------------------- shapes (shapes.ispc:29-211)
__device__ __forceinline__ void body_point(const double *x, const double *L, const double *X,
                                           const double *C0, double *c)
{
  double C[3] = {C0[0], C0[1], C0[2]};
  C[0] -= X[0]; C[1] -= X[1]; C[2] -= X[2];     // SCC (X, C)
  nvaddmul(x, L, C, c);
}

// c = x + L (C - X) is x itself, bit for bit, when C and X have the same
// bits and are finite (C - X is +0), every entry of L is finite (each product
// is a zero, so their sum is a zero) and each x[k] is finite and nonzero
// (x + 0 = x).  That is every SPHERE particle, whose sphere centre is its
// reference point; the test runs on the integer pipe and saves the 21 FP64
// instructions of body_point.
__device__ __forceinline__ bool centre_is_position(const double *x, const double *L, const double *X,
                                                   const double *C)
{
  bool ok = true;
  for (int k = 0; k < 3; k ++)
    ok = ok && dbits(C[k]) == dbits(X[k]) && finite_d(X[k]) && finite_d(x[k]) && nonzero_d(x[k]);
  for (int k = 0; k < 9; k ++) ok = ok && finite_d(L[k]);
  return ok;
}

__global__ void k_spheres(PgDev d)
{
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.ellnum) return;
  int j = d.part[e];
  double L[9], X[3], x[3], C[3], c[3];
  for (int k = 0; k < 9; k ++) L[k] = d.rotation[k][j];
  for (int k = 0; k < 3; k ++) { X[k] = d.position[3+k][j]; x[k] = d.position[k][j]; C[k] = d.center[3+k][e]; }
  if (centre_is_position(x, L, X, C)) { c[0] = x[0]; c[1] = x[1]; c[2] = x[2]; }
  else body_point(x, L, X, C, c);
  for (int k = 0; k < 3; k ++) d.center[k][e] = c[k];
}

__global__ void k_nodes(PgDev d, int skip_analytical)
{
  int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= d.nodnum) return;
  int j = d.nodpart[n];
  if (skip_analytical && (d.flags[j] & PG_FLAG_ANALYTICAL)) return;
  double L[9], X[3], x[3], C[3], c[3];
  for (int k = 0; k < 9; k ++) L[k] = d.rotation[k][j];
  for (int k = 0; k < 3; k ++) { X[k] = d.position[3+k][j]; x[k] = d.position[k][j]; C[k] = d.nodes[3+k][n]; }
  body_point(x, L, X, C, c);
  for (int k = 0; k < 3; k ++) d.nodes[k][n] = c[k];
}

__global__ void k_faces(PgDev d)
{
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  bool need = false;
  if (f < d.facnum)
  {
    int t = d.factri[f];
    for (int v = 0; v < 3; v ++)
    {
      int n = d.facnod[v][f];
      double dd = 0.0;
      for (int c = 0; c < 3; c ++)
      {
        double val = d.nodes[c][n];
        d.tri[3*v+c][t] = val;
        if (d.ellnum)                       // the displacement matters only to sphere candidate lists
        {
          double r = val - d.tref[3*v+c][t];
          dd += r*r;
        }
      }
      need |= gt_nonneg(dd, d.half_skin_sq);
    }
  }
  if (d.ellnum) flag_rebuild(d, need);
}

// ---------------------------------------------------------------- obstacles (obstacles.ispc:28-78)
// velocities: row of the step table (use_row) or the current obsang/obslin state
__global__ void k_obstacles(PgDev d, double step, int use_row)
{
  if (d.hs) step = 0.5*(d.hs[0] + d.hs[1]);
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  bool need = false;
  if (t < d.trinum) need = pgk::obstacles_item(d, t, step, use_row);
  if (d.ellnum) flag_rebuild(d, need);
}

// obstacle points (after every triangle used the old point), obstacle
// velocity state, and the step counter
__global__ void k_tail(PgDev d, double step, int use_row)
{
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (d.hs)
  {
    // adaptive: the obstacles move by (step0 + step1)/2; step1 is recorded
    // for the host and becomes the next step's step0
    const double h1 = d.hs[1];
    step = 0.5*(d.hs[0] + h1);
    d.hrec[use_row ? *d.stepno : 0] = h1;
    pgk::tail_item(d, step, use_row);
    d.hs[0] = h1;
    return;
  }
  pgk::tail_item(d, step, use_row);
}

// The row-mode obstacle update with the tail in the same launch: the last
// block to finish (a counter that it resets) runs the tail, after every
// block has read the old obstacle points and the step pair.
__global__ void k_obstacles_tail(PgDev d, double step)
{
  const double step0 = step;
  if (d.hs) step = 0.5*(d.hs[0] + d.hs[1]);
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  bool need = false;
  if (t < d.trinum) need = pgk::obstacles_item(d, t, step, 1);
  if (d.ellnum) flag_rebuild(d, need);
  __shared__ int last;
  __syncthreads();
  if (threadIdx.x == 0)
  {
    __threadfence();
    last = atomicAdd(d.obs_done, 1) == (int)gridDim.x - 1;
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  *d.obs_done = 0;
  if (d.hs)
  {
    const double h1 = d.hs[1];
    const double st = 0.5*(d.hs[0] + h1);
    d.hrec[*d.stepno] = h1;
    pgk::tail_item(d, st, 1);
    d.hs[0] = h1;
    return;
  }
  pgk::tail_item(d, step0, 1);
}

using pgk::pairing;

// ---------------------------------------------------------------- contacts
// One thread per sphere (master side).  For every candidate in its list the
// exact FP64 narrow phase decides whether the contact exists this step:
// a contact persists while depth >= 0 (forces.ispc:191, removal 327-365) and
// is created when depth > 0 (condet.ispc:183); existing sphere pairs use the
// unguarded 1/len (condet.ispc:667), new ones the guarded one (137).
// ADAPT: adaptive stepping; the step comes from d.hs and the master-side
// stiffness terms (forces.ispc:505-522) go to akact/akmax/aemax/akrot.
template <bool GEOM, bool ADAPT>
__global__ void __launch_bounds__(TPB) k_contacts(PgDev d, double step)
{
  const int E = d.ellnum;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= E) return;
  if (ADAPT) step = d.hs[0];
  const int pi = d.part[i];
  const int cnt = d.ncnt[i];
  double fs[3] = {0.0, 0.0, 0.0}, ts[3] = {0.0, 0.0, 0.0};
  double kact0[3] = {0.0, 0.0, 0.0}, krot0[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, kmax0 = 0.0, emax0 = 0.0;
  if (cnt > 0)
  {
    const bool obsc = (d.compat & PG_COMPAT_OBSIDX) != 0;
    double x[3], v[3], oi[3], c[3];
    for (int k = 0; k < 3; k ++)
    {
      x[k] = d.position[k][pi];
      v[k] = d.linear[k][pi];
      oi[k] = d.angular[3+k][pi];
      c[k] = d.center[k][i];
    }
    const double ri = d.radii[0][i];
    const int coli = d.ellcol[i];
    const double invmi = d.invm[pi], massi = d.mass[pi];

    for (int k = 0; k < cnt; k ++)
    {
      const size_t idx = (size_t)k * d.estride + i;
      const int code = d.ncode[idx];
      const bool existing = d.nflag[idx] != 0;
      // Geometry in two stages: the squared distance first; a candidate
      // clearly apart (d2 > (r_i + r_j)^2 (1 + 1e-12), which the rounding of
      // sqrt and of the products cannot bring back to depth >= 0) skips the
      // square root and the division.  Every contact that can be active takes
      // the same operations as the reference's.
      double point[3], normal[3], depth, q[3], len;
      int pj, colj;
      bool apart;
      const double *cjp = nullptr;
      double cj[3];
      if (code >= 0)
      {
        const int j = code;
        pj = d.part[j];
        colj = d.ellcol[j];
        cj[0] = d.center[0][j]; cj[1] = d.center[1][j]; cj[2] = d.center[2][j];
        cjp = cj;
        q[0] = c[0]-cj[0];
        q[1] = c[1]-cj[1];
        q[2] = c[2]-cj[2];
        const double d2 = dot3(q, q);
        const double sr = ri+d.radii[0][j];
        apart = gt_nonneg(d2, (sr*sr) * (1.0 + 1e-12));
        if (!apart)
        {
          len = sqrt(d2);
          depth = sr - len;
        }
      }
      else
      {
        const int t = -code-1;
        double A[3], B[3], C[3];
        for (int kk = 0; kk < 3; kk ++) { A[kk] = d.tri[kk][t]; B[kk] = d.tri[3+kk][t]; C[kk] = d.tri[6+kk][t]; }
        triangle_closest(A, B, C, c, point, (d.compat & PG_COMPAT_TRIEDGE) != 0);
        q[0] = c[0]-point[0];
        q[1] = c[1]-point[1];
        q[2] = c[2]-point[2];
        const double d2 = dot3(q, q);
        apart = gt_nonneg(d2, (ri*ri) * (1.0 + 1e-12));
        if (!apart)
        {
          len = sqrt(d2);
          depth = ri - len;
        }
        pj = d.triobs[t];
        colj = d.tricol[t];
      }
      const bool active = !apart && (existing ? !lt_zero_d(depth) : gt_zero_d(depth));
      if (!active)
      {
        if (existing)
        {
          d.nflag[idx] = 0;
          d.nstate[0][idx] = 0.0; d.nstate[1][idx] = 0.0; d.nstate[2][idx] = 0.0;
        }
        continue;
      }
      if (cjp)
      {
        double ilen = existing ? 1.0/len : (gt_zero_d(len) ? 1.0/len : 1.0);
        point[0] = 0.5*(c[0]+cj[0]);
        point[1] = 0.5*(c[1]+cj[1]);
        point[2] = 0.5*(c[2]+cj[2]);
        normal[0] = ilen*q[0];
        normal[1] = ilen*q[1];
        normal[2] = ilen*q[2];
      }
      else
      {
        double ilen = 1.0/len;
        normal[0] = ilen*q[0];
        normal[1] = ilen*q[1];
        normal[2] = ilen*q[2];
      }

      // contact point velocities (forces.ispc:226-279)
      double z[3], vi[3], vj[3], oj[3], vij[3];
      z[0] = point[0]-x[0]; z[1] = point[1]-x[1]; z[2] = point[2]-x[2];
      vi[0] = oi[1]*z[2]-oi[2]*z[1] + v[0];
      vi[1] = oi[2]*z[0]-oi[0]*z[2] + v[1];
      vi[2] = oi[0]*z[1]-oi[1]*z[0] + v[2];
      if (pj >= 0)
      {
        z[0] = point[0]-d.position[0][pj];
        z[1] = point[1]-d.position[1][pj];
        z[2] = point[2]-d.position[2][pj];
        oj[0] = d.angular[3][pj]; oj[1] = d.angular[4][pj]; oj[2] = d.angular[5][pj];
        vj[0] = oj[1]*z[2]-oj[2]*z[1] + d.linear[0][pj];
        vj[1] = oj[2]*z[0]-oj[0]*z[2] + d.linear[1][pj];
        vj[2] = oj[0]*z[1]-oj[1]*z[0] + d.linear[2][pj];
      }
      else
      {
        int l = -pj-2;
        if (obsc && l >= 0) l = l+1;
        if (l >= 0 && l < d.obsnum)
        {
          z[0] = point[0]-d.obspnt[3*l];
          z[1] = point[1]-d.obspnt[3*l+1];
          z[2] = point[2]-d.obspnt[3*l+2];
          oj[0] = d.obsang[3*l]; oj[1] = d.obsang[3*l+1]; oj[2] = d.obsang[3*l+2];
          vj[0] = oj[1]*z[2]-oj[2]*z[1] + d.obslin[3*l];
          vj[1] = oj[2]*z[0]-oj[0]*z[2] + d.obslin[3*l+1];
          vj[2] = oj[0]*z[1]-oj[1]*z[0] + d.obslin[3*l+2];
        }
        else
        {
          vj[0] = vj[1] = vj[2] = 0.0;
        }
      }
      vij[0] = vj[0] - vi[0];
      vij[1] = vj[1] - vi[1];
      vij[2] = vj[2] - vi[2];

      const int ij = pairing(d, coli, colj);
      if (d.ikind[ij] != 0) set_err(d, PG_ERR_UNSUPPORTED, 4, i, ij);

      // granular force (forces.ispc:125-192)
      double state[3];
      if (existing) { state[0] = d.nstate[0][idx]; state[1] = d.nstate[1][idx]; state[2] = d.nstate[2][idx]; }
      else { state[0] = 0.0; state[1] = 0.0; state[2] = 0.0; }
      // the pair's damping is fixed between uploads: taken from the list
      // entry (computed at the rebuild with the same expression) or here
      double kn = d.iparam[0][ij];
      double en;
      if (d.nen) en = d.nen[idx];
      else
      {
        double ma = pj >= 0 ? 1.0 / (invmi + d.invm[pj]) : massi;
        en = d.iparam[1][ij] * 2.0 * sqrt(kn*ma);
      }
      double vn = dot3(vij, normal);
      double fn = kn*depth + en*vn;
      double f[3];
      f[0] = fn*normal[0];
      f[1] = fn*normal[1];
      f[2] = fn*normal[2];
      double kskn = d.iparam[6][ij];
      double kt = kn * kskn;
      double et = en * kskn;
      double mus = d.iparam[2][ij];
      double mud = d.iparam[3][ij];
      double vt[3], ft[3];
      vt[0] = vij[0] - vn*normal[0];
      vt[1] = vij[1] - vn*normal[1];
      vt[2] = vij[2] - vn*normal[2];
      state[0] += step*vt[0];
      state[1] += step*vt[1];
      state[2] += step*vt[2];
      ft[0] = kt*state[0] + et*vt[0];
      ft[1] = kt*state[1] + et*vt[1];
      ft[2] = kt*state[2] + et*vt[2];
      double flen = sqrt(dot3(ft, ft));
      double lim = mus*fn;
      if (gt_d(flen, lim))
      {
        lim = mud*fn/flen;
        ft[0] *= lim;
        ft[1] *= lim;
        ft[2] *= lim;
      }
      f[0] += ft[0];
      f[1] += ft[1];
      f[2] += ft[2];

      d.nflag[idx] = 1;
      d.nstate[0][idx] = state[0]; d.nstate[1][idx] = state[1]; d.nstate[2][idx] = state[2];
      d.nfrc[0][idx] = f[0]; d.nfrc[1][idx] = f[1]; d.nfrc[2][idx] = f[2];
      d.npnt[0][idx] = point[0]; d.npnt[1][idx] = point[1]; d.npnt[2][idx] = point[2];
      if (GEOM)
      {
        d.nnrm[0][idx] = normal[0]; d.nnrm[1][idx] = normal[1]; d.nnrm[2][idx] = normal[2];
        d.ndep[idx] = depth;
      }

      // master-side accumulation (contacts_acc_task, forces.ispc:490-510)
      double a[3] = {point[0]-x[0], point[1]-x[1], point[2]-x[2]};
      fs[0] += f[0]; fs[1] += f[1]; fs[2] += f[2];
      ts[0] += a[1]*f[2] - a[2]*f[1];
      ts[1] += a[2]*f[0] - a[0]*f[2];
      ts[2] += a[0]*f[1] - a[1]*f[0];
      if (ADAPT)
      {
        kact0[0] += fabs(normal[0]);
        kact0[1] += fabs(normal[1]);
        kact0[2] += fabs(normal[2]);
        kmax0 = kn > kmax0 ? kn : kmax0;
        emax0 = en > emax0 ? en : emax0;
        double L[9], A[3];
        for (int k = 0; k < 9; k ++) L[k] = d.rotation[k][pi];
        nvmul(L, a, A);
        krot_add(krot0, A);
      }
    }
  }
  d.fm[0][pi] = fs[0]; d.fm[1][pi] = fs[1]; d.fm[2][pi] = fs[2];
  d.tm[0][pi] = ts[0]; d.tm[1][pi] = ts[1]; d.tm[2][pi] = ts[2];
  if (ADAPT)
  {
    for (int k = 0; k < 3; k ++) d.akact[k][pi] = kact0[k];
    for (int k = 0; k < 6; k ++) d.akrot[k][pi] = krot0[k];
    d.akmax[pi] = kmax0;
    d.aemax[pi] = emax0;
  }
}

// ---------------------------------------------------------------- contacts in three passes
// The same evaluation as k_contacts, split so that the FP64 work runs on
// full warps: one thread per sphere walks a list whose active contacts sit
// at different slots, so its warp's FP64 instructions ran with a fraction of
// the lanes.
//   k_contacts_probe  one thread per sphere: the squared-distance test of
//                     every sphere candidate; a candidate clearly apart is
//                     settled there (an existing contact ends), every other
//                     slot goes to the work queue (one atomic per warp);
//   k_contacts_eval   one thread per queued slot (a grid-stride loop over
//                     the queue): geometry, the creation/persistence rule,
//                     contact velocities and the granular law, written to
//                     the slot;
//   k_contacts_sum    one thread per sphere: the master-side force, torque
//                     and (adaptive) stiffness sums over its slots in slot
//                     order, as k_contacts sums them.  Without adaptive
//                     stepping k_integrate takes the force and torque sums
//                     itself, in the same order, and this pass is not run.
// Every slot takes the same operations as in k_contacts and the sums the
// same order, so the results are the same bits; the queue's order plays no
// part.
__device__ __forceinline__ void queue_push(int *work, int *count, bool push, int idx)
{
  const unsigned m = __ballot_sync(__activemask(), push);
  if (!m) return;
  const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(count, __popc(m));
  base = __shfl_sync(__activemask(), base, leader);
  if (push) work[base + __popc(m & ((1u << lane) - 1u))] = idx;
}

__global__ void __launch_bounds__(TPB) k_contacts_probe(PgDev d)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int cnt = i < d.ellnum ? d.ncnt[i] : 0;
  double c[3] = {0.0, 0.0, 0.0}, ri = 0.0;
  if (cnt > 0)
  {
    c[0] = d.center[0][i]; c[1] = d.center[1][i]; c[2] = d.center[2][i];
    ri = d.radii[0][i];
  }
  // every lane of the warp takes part in each round's vote
  int kmax = cnt;
  for (int o = 16; o > 0; o >>= 1)
  {
    const int other = __shfl_xor_sync(0xffffffffu, kmax, o);
    kmax = other > kmax ? other : kmax;
  }
  for (int k = 0; k < kmax; k ++)
  {
    bool push = false;
    size_t idx = 0;
    if (k < cnt)
    {
      idx = (size_t)k * d.estride + i;
      const int code = d.ncode[idx];
      push = true;
      if (code >= 0)
      {
        double q[3];
        q[0] = c[0]-d.center[0][code];
        q[1] = c[1]-d.center[1][code];
        q[2] = c[2]-d.center[2][code];
        const double d2 = dot3(q, q);
        const double sr = ri+d.radii[0][code];
        if (gt_nonneg(d2, (sr*sr) * (1.0 + 1e-12)))
        {
          push = false;
          if (d.nflag[idx])
          {
            d.nflag[idx] = 0;
            d.nstate[0][idx] = 0.0; d.nstate[1][idx] = 0.0; d.nstate[2][idx] = 0.0;
          }
        }
      }
    }
    queue_push(d.cwork, d.cwork_n, push, (int)idx);
  }
}

template <bool GEOM, bool ADAPT>
__global__ void PG_LB_EVAL k_contacts_eval(PgDev d, double step)
{
  if (ADAPT) step = d.hs[0];
  const int n = *d.cwork_n;
  const bool obsc = (d.compat & PG_COMPAT_OBSIDX) != 0;
  for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < n; w += gridDim.x * blockDim.x)
  {
    const int idx0 = d.cwork[w];
    const size_t idx = (size_t)idx0;
    const int i = idx0 % d.estride;
    const int pi = d.part[i];
    double x[3], v[3], oi[3], c[3];
    for (int k = 0; k < 3; k ++)
    {
      x[k] = d.position[k][pi];
      v[k] = d.linear[k][pi];
      oi[k] = d.angular[3+k][pi];
      c[k] = d.center[k][i];
    }
    const double ri = d.radii[0][i];
    const int coli = d.ellcol[i];
    const double invmi = d.invm[pi], massi = d.mass[pi];
    const int code = d.ncode[idx];
    const bool existing = d.nflag[idx] != 0;
    double point[3], normal[3], depth = 0.0, q[3], len = 0.0;
    int pj, colj;
    bool apart;
    bool sphere = code >= 0;
    double cj[3];
    if (sphere)
    {
      const int j = code;
      pj = d.part[j];
      colj = d.ellcol[j];
      cj[0] = d.center[0][j]; cj[1] = d.center[1][j]; cj[2] = d.center[2][j];
      q[0] = c[0]-cj[0];
      q[1] = c[1]-cj[1];
      q[2] = c[2]-cj[2];
      const double d2 = dot3(q, q);
      const double sr = ri+d.radii[0][j];
      apart = gt_nonneg(d2, (sr*sr) * (1.0 + 1e-12));
      if (!apart)
      {
        len = sqrt(d2);
        depth = sr - len;
      }
    }
    else
    {
      const int t = -code-1;
      double A[3], B[3], C[3];
      for (int kk = 0; kk < 3; kk ++) { A[kk] = d.tri[kk][t]; B[kk] = d.tri[3+kk][t]; C[kk] = d.tri[6+kk][t]; }
      triangle_closest(A, B, C, c, point, (d.compat & PG_COMPAT_TRIEDGE) != 0);
      q[0] = c[0]-point[0];
      q[1] = c[1]-point[1];
      q[2] = c[2]-point[2];
      const double d2 = dot3(q, q);
      apart = gt_nonneg(d2, (ri*ri) * (1.0 + 1e-12));
      if (!apart)
      {
        len = sqrt(d2);
        depth = ri - len;
      }
      pj = d.triobs[t];
      colj = d.tricol[t];
    }
    const bool active = !apart && (existing ? !lt_zero_d(depth) : gt_zero_d(depth));
    if (!active)
    {
      if (existing)
      {
        d.nflag[idx] = 0;
        d.nstate[0][idx] = 0.0; d.nstate[1][idx] = 0.0; d.nstate[2][idx] = 0.0;
      }
      continue;
    }
    if (sphere)
    {
      double ilen = existing ? 1.0/len : (gt_zero_d(len) ? 1.0/len : 1.0);
      point[0] = 0.5*(c[0]+cj[0]);
      point[1] = 0.5*(c[1]+cj[1]);
      point[2] = 0.5*(c[2]+cj[2]);
      normal[0] = ilen*q[0];
      normal[1] = ilen*q[1];
      normal[2] = ilen*q[2];
    }
    else
    {
      double ilen = 1.0/len;
      normal[0] = ilen*q[0];
      normal[1] = ilen*q[1];
      normal[2] = ilen*q[2];
    }

    // contact point velocities (forces.ispc:226-279)
    double z[3], vi[3], vj[3], oj[3], vij[3];
    z[0] = point[0]-x[0]; z[1] = point[1]-x[1]; z[2] = point[2]-x[2];
    vi[0] = oi[1]*z[2]-oi[2]*z[1] + v[0];
    vi[1] = oi[2]*z[0]-oi[0]*z[2] + v[1];
    vi[2] = oi[0]*z[1]-oi[1]*z[0] + v[2];
    if (pj >= 0)
    {
      z[0] = point[0]-d.position[0][pj];
      z[1] = point[1]-d.position[1][pj];
      z[2] = point[2]-d.position[2][pj];
      oj[0] = d.angular[3][pj]; oj[1] = d.angular[4][pj]; oj[2] = d.angular[5][pj];
      vj[0] = oj[1]*z[2]-oj[2]*z[1] + d.linear[0][pj];
      vj[1] = oj[2]*z[0]-oj[0]*z[2] + d.linear[1][pj];
      vj[2] = oj[0]*z[1]-oj[1]*z[0] + d.linear[2][pj];
    }
    else
    {
      int l = -pj-2;
      if (obsc && l >= 0) l = l+1;
      if (l >= 0 && l < d.obsnum)
      {
        z[0] = point[0]-d.obspnt[3*l];
        z[1] = point[1]-d.obspnt[3*l+1];
        z[2] = point[2]-d.obspnt[3*l+2];
        oj[0] = d.obsang[3*l]; oj[1] = d.obsang[3*l+1]; oj[2] = d.obsang[3*l+2];
        vj[0] = oj[1]*z[2]-oj[2]*z[1] + d.obslin[3*l];
        vj[1] = oj[2]*z[0]-oj[0]*z[2] + d.obslin[3*l+1];
        vj[2] = oj[0]*z[1]-oj[1]*z[0] + d.obslin[3*l+2];
      }
      else
      {
        vj[0] = vj[1] = vj[2] = 0.0;
      }
    }
    vij[0] = vj[0] - vi[0];
    vij[1] = vj[1] - vi[1];
    vij[2] = vj[2] - vi[2];

    const int ij = pairing(d, coli, colj);
    if (d.ikind[ij] != 0) set_err(d, PG_ERR_UNSUPPORTED, 4, i, ij);

    // granular force (forces.ispc:125-192)
    double state[3];
    if (existing) { state[0] = d.nstate[0][idx]; state[1] = d.nstate[1][idx]; state[2] = d.nstate[2][idx]; }
    else { state[0] = 0.0; state[1] = 0.0; state[2] = 0.0; }
    double kn = d.iparam[0][ij];
    double en;
    if (d.nen) en = d.nen[idx];
    else
    {
      double ma = pj >= 0 ? 1.0 / (invmi + d.invm[pj]) : massi;
      en = d.iparam[1][ij] * 2.0 * sqrt(kn*ma);
    }
    double vn = dot3(vij, normal);
    double fn = kn*depth + en*vn;
    double f[3];
    f[0] = fn*normal[0];
    f[1] = fn*normal[1];
    f[2] = fn*normal[2];
    double kskn = d.iparam[6][ij];
    double kt = kn * kskn;
    double et = en * kskn;
    double mus = d.iparam[2][ij];
    double mud = d.iparam[3][ij];
    double vt[3], ft[3];
    vt[0] = vij[0] - vn*normal[0];
    vt[1] = vij[1] - vn*normal[1];
    vt[2] = vij[2] - vn*normal[2];
    state[0] += step*vt[0];
    state[1] += step*vt[1];
    state[2] += step*vt[2];
    ft[0] = kt*state[0] + et*vt[0];
    ft[1] = kt*state[1] + et*vt[1];
    ft[2] = kt*state[2] + et*vt[2];
    double flen = sqrt(dot3(ft, ft));
    double lim = mus*fn;
    if (gt_d(flen, lim))
    {
      lim = mud*fn/flen;
      ft[0] *= lim;
      ft[1] *= lim;
      ft[2] *= lim;
    }
    f[0] += ft[0];
    f[1] += ft[1];
    f[2] += ft[2];

    d.nflag[idx] = 1;
    d.nstate[0][idx] = state[0]; d.nstate[1][idx] = state[1]; d.nstate[2][idx] = state[2];
    d.nfrc[0][idx] = f[0]; d.nfrc[1][idx] = f[1]; d.nfrc[2][idx] = f[2];
    d.npnt[0][idx] = point[0]; d.npnt[1][idx] = point[1]; d.npnt[2][idx] = point[2];
    if (GEOM || ADAPT)
    {
      d.nnrm[0][idx] = normal[0]; d.nnrm[1][idx] = normal[1]; d.nnrm[2][idx] = normal[2];
    }
    if (GEOM) d.ndep[idx] = depth;
  }
}

template <bool ADAPT>
__global__ void __launch_bounds__(TPB) k_contacts_sum(PgDev d)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.ellnum) return;
  const int pi = d.part[i];
  const int cnt = d.ncnt[i];
  double fs[3] = {0.0, 0.0, 0.0}, ts[3] = {0.0, 0.0, 0.0};
  double kact0[3] = {0.0, 0.0, 0.0}, krot0[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, kmax0 = 0.0, emax0 = 0.0;
  if (cnt > 0)
  {
    const double x[3] = {d.position[0][pi], d.position[1][pi], d.position[2][pi]};
    double L[9];
    if (ADAPT) for (int k = 0; k < 9; k ++) L[k] = d.rotation[k][pi];
    for (int k = 0; k < cnt; k ++)
    {
      const size_t idx = (size_t)k * d.estride + i;
      if (!d.nflag[idx]) continue;
      const double f[3] = {d.nfrc[0][idx], d.nfrc[1][idx], d.nfrc[2][idx]};
      const double a[3] = {d.npnt[0][idx]-x[0], d.npnt[1][idx]-x[1], d.npnt[2][idx]-x[2]};
      fs[0] += f[0]; fs[1] += f[1]; fs[2] += f[2];
      ts[0] += a[1]*f[2] - a[2]*f[1];
      ts[1] += a[2]*f[0] - a[0]*f[2];
      ts[2] += a[0]*f[1] - a[1]*f[0];
      if (ADAPT)
      {
        const int code = d.ncode[idx];
        const int pj = code >= 0 ? d.part[code] : d.triobs[-code-1];
        const int ij = pairing(d, d.ellcol[i], code >= 0 ? d.ellcol[code] : d.tricol[-code-1]);
        const double kn = d.iparam[0][ij];
        double en;
        if (d.nen) en = d.nen[idx];
        else
        {
          double ma = pj >= 0 ? 1.0 / (d.invm[pi] + d.invm[pj]) : d.mass[pi];
          en = d.iparam[1][ij] * 2.0 * sqrt(kn*ma);
        }
        kact0[0] += fabs(d.nnrm[0][idx]);
        kact0[1] += fabs(d.nnrm[1][idx]);
        kact0[2] += fabs(d.nnrm[2][idx]);
        kmax0 = kn > kmax0 ? kn : kmax0;
        emax0 = en > emax0 ? en : emax0;
        double A[3];
        nvmul(L, a, A);
        krot_add(krot0, A);
      }
    }
  }
  d.fm[0][pi] = fs[0]; d.fm[1][pi] = fs[1]; d.fm[2][pi] = fs[2];
  d.tm[0][pi] = ts[0]; d.tm[1][pi] = ts[1]; d.tm[2][pi] = ts[2];
  if (ADAPT)
  {
    for (int k = 0; k < 3; k ++) d.akact[k][pi] = kact0[k];
    for (int k = 0; k < 6; k ++) d.akrot[k][pi] = krot0[k];
    d.akmax[pi] = kmax0;
    d.aemax[pi] = emax0;
  }
}

// ---------------------------------------------------------------- springs (forces.ispc:641-1412)
__device__ double look_up(const double *t0, const double *t1, int lo, int hi, double arg, double *slope)
{
  int h0 = hi;
  while (hi > lo+1)
  {
    int mid = lo + (hi-lo)/2;
    if (arg > t0[mid]) lo = mid;
    else hi = mid;
  }
  if (lo+1 == h0) lo --;
  *slope = (t1[lo+1]-t1[lo])/(t0[lo+1]-t0[lo]);
  return t1[lo] + (*slope)*(arg-t0[lo]);
}

__device__ double look_up_slope(int i, const double *t0, const double *t1, int lo, int hi, double arg, double *at)
{
  const double *ti = i == 0 ? t0 : t1;
  const double *tj = i == 0 ? t1 : t0;
  int h0 = hi;
  while (hi > lo+1)
  {
    int mid = lo + (hi-lo)/2;
    if (arg > ti[mid]) lo = mid;
    else hi = mid;
  }
  if (lo+1 == h0) lo --;
  if (at) at[0] = tj[lo] + (tj[lo+1]-tj[lo])*(arg-ti[lo])/(ti[lo+1]-ti[lo]);
  return (t1[lo+1]-t1[lo])/(t0[lo+1]-t0[lo]);
}

// equivalent relative point mass (parmec.ispc:423-482)
__device__ double eqm(const PgDev &d, int part1, const double *point1, int part2, const double *point2,
                      const double *direction)
{
  double Jiv[9], im, A[3], Ask[9], tmp[9], Miv[9];
  for (int k = 0; k < 9; k ++) Jiv[k] = d.inverse[k][part1];
  im = d.invm[part1];
  A[0] = d.position[3][part1] - point1[0];
  A[1] = d.position[4][part1] - point1[1];
  A[2] = d.position[5][part1] - point1[2];
  Ask[0] = 0; Ask[1] = A[2]; Ask[2] = -A[1]; Ask[3] = -A[2]; Ask[4] = 0; Ask[5] = A[0];
  Ask[6] = A[1]; Ask[7] = -A[0]; Ask[8] = 0;
  tnmul(Ask, Jiv, tmp);
  nnmul(tmp, Ask, Miv);
  Miv[0] += im; Miv[4] += im; Miv[8] += im;
  if (part2 >= 0)
  {
    for (int k = 0; k < 9; k ++) Jiv[k] = d.inverse[k][part2];
    im = d.invm[part2];
    A[0] = d.position[3][part2] - point2[0];
    A[1] = d.position[4][part2] - point2[1];
    A[2] = d.position[5][part2] - point2[2];
    Ask[0] = 0; Ask[1] = A[2]; Ask[2] = -A[1]; Ask[3] = -A[2]; Ask[4] = 0; Ask[5] = A[0];
    Ask[6] = A[1]; Ask[7] = -A[0]; Ask[8] = 0;
    tnmul(Ask, Jiv, tmp);
    nnmul(tmp, Ask, Jiv);
    for (int k = 0; k < 9; k ++) Miv[k] = Miv[k] + Jiv[k];
    Miv[0] += im; Miv[4] += im; Miv[8] += im;
  }
  if (direction && dot3(direction, direction) > 0.0)
  {
    nvmul(Miv, direction, tmp);
    return 1.0/dot3(tmp, direction);
  }
  return 1.0/pg::extremum_eigenvalue(Miv, true);
}

// ADAPT: adaptive stepping; the step comes from d.hs and each spring records
// its stiffness terms (forces.ispc:1248-1345) in sad, zeros when its total
// force is zero.  The k arm is taken in the k particle's frame (the reference
// rotates it with the j particle's rotation, forces.ispc:1341).
template <bool ADAPT>
__global__ void __launch_bounds__(TPB) k_springs(PgDev d, double step)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.sprnum) return;
  if (ADAPT) step = d.hs[0];
  const double time = d.t_curtime[*d.stepno];
  const int j = d.sprpart[0][i], k = d.sprpart[1][i];
  double len = 0.0, inv, velocity, spring_force = 0.0, dashpot_force, total_force;
  double Yj[3], Yk[3] = {0.0, 0.0, 0.0}, p[3], q[3], z[3] = {0.0, 0.0, 0.0}, w[3], frc[3], u[3], a[3], b[3] = {0.0, 0.0, 0.0};
  double stiffness = 0.0, damping = 0.0;
  double oj[3], vj[3], xj[3], Xj[3], Lj[9];
  for (int m = 0; m < 3; m ++)
  {
    oj[m] = d.angular[3+m][j]; vj[m] = d.linear[m][j]; xj[m] = d.position[m][j]; Xj[m] = d.position[3+m][j];
  }
  for (int m = 0; m < 9; m ++) Lj[m] = d.rotation[m][j];
  const int flg0 = d.sprflg[i];
  int flg = flg0;

  Yj[0] = d.sprpnt[3][i]; Yj[1] = d.sprpnt[4][i]; Yj[2] = d.sprpnt[5][i];
  Yj[0] = Yj[0] - Xj[0]; Yj[1] = Yj[1] - Xj[1]; Yj[2] = Yj[2] - Xj[2];
  nvaddmul(xj, Lj, Yj, p);
  d.sprpnt[0][i] = p[0]; d.sprpnt[1][i] = p[1]; d.sprpnt[2][i] = p[2];
  u[0] = vj[0]; u[1] = vj[1]; u[2] = vj[2];
  u[0] *= -1.0; u[1] *= -1.0; u[2] *= -1.0;
  a[0] = p[0] - xj[0]; a[1] = p[1] - xj[1]; a[2] = p[2] - xj[2];
  u[0] -= oj[1]*a[2] - oj[2]*a[1];
  u[1] -= oj[2]*a[0] - oj[0]*a[2];
  u[2] -= oj[0]*a[1] - oj[1]*a[0];

  if (k >= 0)
  {
    double ok[3], vk[3], xk[3], Xk[3], Lk[9];
    for (int m = 0; m < 3; m ++)
    {
      ok[m] = d.angular[3+m][k]; vk[m] = d.linear[m][k]; xk[m] = d.position[m][k]; Xk[m] = d.position[3+m][k];
    }
    for (int m = 0; m < 9; m ++) Lk[m] = d.rotation[m][k];
    if (flg & PG_SPRDIR_PROJECT)
    {
      w[0] = d.sprdir[3][i]; w[1] = d.sprdir[4][i]; w[2] = d.sprdir[5][i];
      nvmul(Lk, w, z);
      d.sprdir[0][i] = z[0]; d.sprdir[1][i] = z[1]; d.sprdir[2][i] = z[2];
    }
    Yk[0] = d.sprpnt[9][i]; Yk[1] = d.sprpnt[10][i]; Yk[2] = d.sprpnt[11][i];
    Yk[0] = Yk[0] - Xk[0]; Yk[1] = Yk[1] - Xk[1]; Yk[2] = Yk[2] - Xk[2];
    nvaddmul(xk, Lk, Yk, q);
    d.sprpnt[6][i] = q[0]; d.sprpnt[7][i] = q[1]; d.sprpnt[8][i] = q[2];
    u[0] += vk[0]; u[1] += vk[1]; u[2] += vk[2];
    b[0] = q[0] - xk[0]; b[1] = q[1] - xk[1]; b[2] = q[2] - xk[2];
    u[0] += ok[1]*b[2] - ok[2]*b[1];
    u[1] += ok[2]*b[0] - ok[0]*b[2];
    u[2] += ok[0]*b[1] - ok[1]*b[0];
  }
  else
  {
    q[0] = d.sprpnt[6][i]; q[1] = d.sprpnt[7][i]; q[2] = d.sprpnt[8][i];
    if (flg & PG_SPRDIR_PROJECT) { z[0] = d.sprdir[0][i]; z[1] = d.sprdir[1][i]; z[2] = d.sprdir[2][i]; }
  }

  switch (flg & (PG_SPRDIR_FOLLOWER|PG_SPRDIR_CONSTANT|PG_SPRDIR_PLANAR|PG_SPRDIR_PROJECT))
  {
    case PG_SPRDIR_FOLLOWER:
      w[0] = q[0] - p[0]; w[1] = q[1] - p[1]; w[2] = q[2] - p[2];
      len = sqrt(dot3(w, w));
      inv = len > 0.0 ? 1.0/len : 0.0;
      z[0] = inv*w[0]; z[1] = inv*w[1]; z[2] = inv*w[2];
      d.sprdir[0][i] = z[0]; d.sprdir[1][i] = z[1]; d.sprdir[2][i] = z[2];
      break;
    case PG_SPRDIR_CONSTANT:
      w[0] = q[0] - p[0]; w[1] = q[1] - p[1]; w[2] = q[2] - p[2];
      z[0] = d.sprdir[0][i]; z[1] = d.sprdir[1][i]; z[2] = d.sprdir[2][i];
      len = dot3(w, z);
      break;
    case PG_SPRDIR_PLANAR:
      w[0] = q[0] - p[0]; w[1] = q[1] - p[1]; w[2] = q[2] - p[2];
      inv = w[0]*d.sprdir[3][i]+w[1]*d.sprdir[4][i]+w[2]*d.sprdir[5][i];
      w[0] -= inv*d.sprdir[3][i];
      w[1] -= inv*d.sprdir[4][i];
      w[2] -= inv*d.sprdir[5][i];
      len = sqrt(dot3(w, w));
      inv = len > 0.0 ? 1.0/len : 0.0;
      z[0] = inv*w[0]; z[1] = inv*w[1]; z[2] = inv*w[2];
      d.sprdir[0][i] = z[0]; d.sprdir[1][i] = z[1]; d.sprdir[2][i] = z[2];
      break;
    case PG_SPRDIR_PROJECT:
      w[0] = p[0] - q[0]; w[1] = p[1] - q[1]; w[2] = p[2] - q[2];
      len = dot3(w, z);
      break;
  }

  double offset = 0.0, slope;
  const int ilc = d.sproffset[i];
  if (ilc >= 0) offset = look_up(d.lcurve[0], d.lcurve[1], d.lcidx[ilc], d.lcidx[ilc+1], time, &slope);

  const int unspr = d.unspring[i];
  const double *S0 = d.spring[0], *S1 = d.spring[1];
  const double *U0 = d.unload[0], *U1 = d.unload[1];
  if (unspr <= -2)
  {
    if (d.sprtype[i] == PG_SPRING_NONLINEAR_ELASTIC)
    {
      d.stroke[0][i] = len - d.stroke0[i];
      spring_force = look_up(S0, S1, d.spridx[i], d.spridx[i+1], d.stroke[0][i] - offset, &stiffness);
    }
    else if (d.sprtype[i] == PG_SPRING_GENERAL_NONLINEAR)
    {
      if ((flg & PG_SPRING_YIELDED) == 0)
      {
        d.stroke[0][i] = len - d.stroke0[i];
        spring_force = look_up(S0, S1, d.spridx[i], d.spridx[i+1], d.stroke[0][i] - offset, &stiffness);
        if (spring_force < d.yield[0][i] || spring_force > d.yield[1][i])
        {
          flg |= PG_SPRING_YIELDED;
          if (spring_force < 0)
          {
            d.stroke[1][i] = d.stroke[0][i];
            d.stroke[2][i] = 0.0;
            d.yield[1][i] = 0.0;
          }
          else
          {
            d.stroke[1][i] = 0.0;
            d.stroke[2][i] = d.stroke[0][i];
            d.yield[0][i] = 0.0;
          }
        }
      }
      else
      {
        double s0 = d.stroke[0][i];
        double s1 = len - d.stroke0[i];
        double ds = s1 - s0;
        double f0 = d.sprfrc[1][i];
        d.stroke[0][i] = s1;
        bool loading = false;
        if (f0 * ds > 0)
        {
          if (flg & PG_SPRING_UNLOADING)
          {
            double dfds = look_up_slope(1, U0, U1, d.unidx[i], d.unidx[i+1], f0, nullptr);
            spring_force = f0 + dfds*ds;
            if (spring_force < d.yield[0][i] || spring_force > d.yield[1][i])
            {
              flg &= ~PG_SPRING_UNLOADING;
              loading = true;
            }
          }
          else loading = true;
        }
        else
        {
          double at;
          double dfds = look_up_slope(1, U0, U1, d.unidx[i], d.unidx[i+1], f0, &at);
          stiffness = dfds;
          spring_force = f0 + dfds*ds;
          if (spring_force * f0 < 0.0)
            spring_force = look_up(U0, U1, d.unidx[i], d.unidx[i+1], ds+at, &stiffness);
          if (spring_force < d.yield[0][i] || spring_force > d.yield[1][i])
          {
            flg &= ~PG_SPRING_UNLOADING;
            loading = true;
          }
          else flg |= PG_SPRING_UNLOADING;
        }
        if (loading)
        {
          if (ds < 0) d.stroke[1][i] += ds;
          else d.stroke[2][i] += ds;
          spring_force = look_up(S0, S1, d.spridx[i], d.spridx[i+1], ds < 0 ? d.stroke[1][i] : d.stroke[2][i], &stiffness);
          if (ds < 0) d.yield[0][i] = spring_force;
          else d.yield[1][i] = spring_force;
        }
      }
    }
    velocity = dot3(z, u);
    if (d.dashidx[i]+1 == d.dashidx[i+1])
    {
      double mass = eqm(d, j, Yj, k, Yk, z);
      double ratio = d.dashpot[0][d.dashidx[i]];
      damping = ratio * 2.0 * sqrt(fabs(stiffness) * mass);
      dashpot_force = velocity * damping;
    }
    else
    {
      dashpot_force = look_up(d.dashpot[0], d.dashpot[1], d.dashidx[i], d.dashidx[i+1], velocity, &damping);
    }
    total_force = spring_force + (spring_force == 0.0 ? 0.0 : dashpot_force);
  }
  else if (unspr == -1)
  {
    d.stroke[0][i] = len - d.stroke0[i];
    stiffness = 0.; damping = 0.;
    spring_force = dashpot_force = total_force = 0.;
    velocity = dot3(z, u);
  }
  else
  {
    double s0 = d.stroke[0][i];
    double s1 = len - d.stroke0[i];
    double ds = s1 - s0;
    double f0 = d.sprfrc[1][i];
    double sgn = f0 > 0. ? 1. : -1.;
    d.stroke[0][i] = s1;
    double at;
    double dfds = look_up_slope(1, d.lcurve[0], d.lcurve[1], d.lcidx[unspr], d.lcidx[unspr+1], f0, &at);
    stiffness = dfds;
    spring_force = f0 - sgn*fabs(dfds*ds);
    if (spring_force * f0 < 0.0)
    {
      d.unspring[i] = -1;
      spring_force = 0.;
    }
    damping = 0.; dashpot_force = 0.;
    total_force = spring_force;
    velocity = dot3(z, u);
  }

  frc[0] = z[0] * total_force;
  frc[1] = z[1] * total_force;
  frc[2] = z[2] * total_force;
  d.sprfrc[0][i] = total_force;
  d.sprfrc[1][i] = spring_force;

  const double fric = d.sprfric[i];
  if (fric > 0.0)
  {
    double us[3] = {u[0] - velocity*z[0], u[1] - velocity*z[1], u[2] - velocity*z[2]};
    double flim = fric*fabs(total_force);
    double fsv[3] = {0.0, 0.0, 0.0};
    double kskn = d.sprkskn[i];
    if (kskn == 0.0)
    {
      double ulen = sqrt(dot3(us, us));
      if (ulen > 0.0)
      {
        double coef = flim/ulen;
        fsv[0] = coef*us[0]; fsv[1] = coef*us[1]; fsv[2] = coef*us[2];
      }
    }
    else
    {
      if (spring_force == 0.0) { d.sprsdsp[0][i] = 0.0; d.sprsdsp[1][i] = 0.0; d.sprsdsp[2][i] = 0.0; }
      double ds[3] = {d.sprsdsp[0][i] + us[0]*step, d.sprsdsp[1][i] + us[1]*step, d.sprsdsp[2][i] + us[2]*step};
      double c0 = kskn * fabs(stiffness);
      double c1 = spring_force == 0.0 ? 0.0 : kskn * fabs(damping);
      fsv[0] = c0 * ds[0] + c1 * us[0];
      fsv[1] = c0 * ds[1] + c1 * us[1];
      fsv[2] = c0 * ds[2] + c1 * us[2];
      double flen = sqrt(dot3(fsv, fsv));
      if (flen > flim)
      {
        double coef = flim/flen;
        fsv[0] *= coef; fsv[1] *= coef; fsv[2] *= coef;
        double dl0 = sqrt(dot3(ds, ds));
        coef = flim/(c0*dl0);
        d.sprsdsp[0][i] = coef*ds[0]; d.sprsdsp[1][i] = coef*ds[1]; d.sprsdsp[2][i] = coef*ds[2];
      }
      else
      {
        d.sprsdsp[0][i] = ds[0]; d.sprsdsp[1][i] = ds[1]; d.sprsdsp[2][i] = ds[2];
      }
    }
    d.sprfrc[2][i] = sqrt(dot3(fsv, fsv));
    frc[0] += fsv[0]; frc[1] += fsv[1]; frc[2] += fsv[2];
  }
  if (flg != flg0) d.sprflg[i] = flg;

  d.spr_out[0][i] = frc[0]; d.spr_out[1][i] = frc[1]; d.spr_out[2][i] = frc[2];
  d.spr_out[3][i] = a[1]*frc[2] - a[2]*frc[1];
  d.spr_out[4][i] = a[2]*frc[0] - a[0]*frc[2];
  d.spr_out[5][i] = a[0]*frc[1] - a[1]*frc[0];
  d.spr_out[6][i] = b[1]*frc[2] - b[2]*frc[1];
  d.spr_out[7][i] = b[2]*frc[0] - b[0]*frc[2];
  d.spr_out[8][i] = b[0]*frc[1] - b[1]*frc[0];
  if (ADAPT)
  {
    double v[17];
    for (int m = 0; m < 17; m ++) v[m] = 0.0;
    if (total_force != 0.0)
    {
      double A[3], dt;
      v[0] = fabs(z[0]); v[1] = fabs(z[1]); v[2] = fabs(z[2]);
      v[3] = fabs(stiffness); v[4] = fabs(damping);
      tvmul(Lj, a, A);
      dt = dot3(A, A);
      v[5] = dt - A[0]*A[0]; v[6] = dt - A[1]*A[1]; v[7] = dt - A[2]*A[2];
      v[8] = -A[0]*A[1]; v[9] = -A[0]*A[2]; v[10] = -A[1]*A[2];
      if (k >= 0)
      {
        double Lk[9];
        for (int m = 0; m < 9; m ++) Lk[m] = d.rotation[m][k];
        tvmul(Lk, b, A);
        dt = dot3(A, A);
        v[11] = dt - A[0]*A[0]; v[12] = dt - A[1]*A[1]; v[13] = dt - A[2]*A[2];
        v[14] = -A[0]*A[1]; v[15] = -A[0]*A[2]; v[16] = -A[1]*A[2];
      }
    }
    for (int m = 0; m < 17; m ++) d.sad[m][i] = v[m];
  }
}

// ---------------------------------------------------------------- integrate
// contacts_acc_task (slave side) + gravity + spring flushes (single-task order
// of springs_task) + prescribe_acceleration + dynamics_task +
// prescribe_velocity + ellipsoids_task, one thread per particle.
// ---------------------------------------------------------------- long spring flush runs
// A run longer than PG_SPRING_RUN_LONG springs is summed in three levels:
// chunks of springs in spring order (first element assigned), groups of 32
// chunk sums in order, then the group sums in order (the first-run rule
// applied to them).  Chunks hold 64 springs, doubled until there are at most
// 1,024.  k_spring_run_groups runs one warp per group (grid: groups x runs):
// lane l sums chunk 32 g + l, loading four springs at a time, and the warp
// sums its chunk sums in lane order through shuffles; k_spring_run_totals
// sums each run's group partials in order.  A dependent FP64 add costs tens
// of ns on this part, so the sequential depth stays near 64 + 32 + 32 adds
// for any run length, and the groups of a run spread over the SMs.
constexpr int RUN_GROUP = 32;
constexpr int RUN_MAXCHUNKS = 1024;
constexpr int RUN_GROUPS = RUN_MAXCHUNKS / RUN_GROUP;
constexpr int RUN_SLOT = 12;                   // doubles per group partial: 11 values, has-flag

__device__ __forceinline__ int run_chunk(int len)
{
  int c = 64;
  while ((len + c - 1) / c > RUN_MAXCHUNKS) c *= 2;
  return c;
}

__global__ void __launch_bounds__(RUN_GROUP) k_spring_run_groups(PgDev d)
{
  const unsigned full = 0xffffffffu;
  const int run = blockIdx.x, g = blockIdx.y, lane = threadIdx.x;
  const int4 v = d.sbig[run];
  const int type = v.x & 1, off = type == 0 ? 3 : 6;
  const int len = v.z - v.y, ch = run_chunk(len), nc = (len + ch - 1) / ch;
  if (g * RUN_GROUP >= nc) return;
  const int c = g * RUN_GROUP + lane;
  double a[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  int any = 0;
  if (c < nc)
  {
    const int b = v.y + c * ch, e = min(b + ch, v.z);
    for (int s0 = b; s0 < e; s0 += 4)
    {
      double x[4][6];
      bool ok[4];
      #pragma unroll
      for (int u = 0; u < 4; u ++)
      {
        const int sp = s0 + u < e ? s0 + u : b;
        ok[u] = s0 + u < e && !(type == 1 && d.sprpart[1][sp] < 0);
        x[u][0] = d.spr_out[0][sp]; x[u][1] = d.spr_out[1][sp]; x[u][2] = d.spr_out[2][sp];
        x[u][3] = d.spr_out[off][sp]; x[u][4] = d.spr_out[off+1][sp]; x[u][5] = d.spr_out[off+2][sp];
      }
      #pragma unroll
      for (int u = 0; u < 4; u ++)
        if (ok[u])
        {
          if (!any) for (int k = 0; k < 6; k ++) a[k] = x[u][k];
          else for (int k = 0; k < 6; k ++) a[k] = a[k] + x[u][k];
          any = 1;
        }
    }
  }
  double gs[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  int gany = 0;
  for (int l = 0; l < RUN_GROUP; l ++)
  {
    const int la = __shfl_sync(full, any, l);
    double x[6];
    for (int k = 0; k < 6; k ++) x[k] = __shfl_sync(full, a[k], l);
    if (!la) continue;
    if (!gany) for (int k = 0; k < 6; k ++) gs[k] = x[k];
    else for (int k = 0; k < 6; k ++) gs[k] = gs[k] + x[k];
    gany = 1;
  }
  if (lane == 0)
  {
    double *o = d.sbig_grp + ((size_t)run * RUN_GROUPS + g) * RUN_SLOT;
    for (int k = 0; k < 6; k ++) o[k] = gs[k];
    o[11] = gany ? 1.0 : 0.0;
  }
}

__global__ void k_spring_run_totals(PgDev d)
{
  const int run = blockIdx.x * blockDim.x + threadIdx.x;
  if (run >= d.nbig) return;
  const int4 v = d.sbig[run];
  const int len = v.z - v.y, ch = run_chunk(len), nc = (len + ch - 1) / ch, ng = (nc + RUN_GROUP - 1) / RUN_GROUP;
  double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  bool started = false;
  for (int q = 0; q < ng; q ++)
  {
    const double *o = d.sbig_grp + ((size_t)run * RUN_GROUPS + q) * RUN_SLOT;
    if (o[11] == 0.0) continue;
    if (!started && !v.w) for (int k = 0; k < 6; k ++) acc[k] = o[k];
    else for (int k = 0; k < 6; k ++) acc[k] = acc[k] + o[k];
    started = true;
  }
  for (int k = 0; k < 6; k ++) d.sbig_sum[6*run + k] = acc[k];
}

// Adaptive stiffness partials of the long runs, in the levels of the force
// sums: each chunk sums its springs' terms from zero in spring order (maxima
// for the stiffness and damping), each group the partials of its chunks from
// zero, then the group partials from zero.
__global__ void __launch_bounds__(RUN_GROUP) k_spring_run_groups_adapt(PgDev d)
{
  const unsigned full = 0xffffffffu;
  const int run = blockIdx.x, g = blockIdx.y, lane = threadIdx.x;
  const int4 v = d.sbig[run];
  const int type = v.x & 1, off = type == 0 ? 5 : 11;
  const int len = v.z - v.y, ch = run_chunk(len), nc = (len + ch - 1) / ch;
  if (g * RUN_GROUP >= nc) return;
  const int c = g * RUN_GROUP + lane;
  double q[11] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  if (c < nc)
  {
    const int b = v.y + c * ch, e = min(b + ch, v.z);
    for (int s = b; s < e; s ++)
    {
      if (type == 1 && d.sprpart[1][s] < 0) continue;
      for (int k = 0; k < 3; k ++) q[k] = q[k] + d.sad[k][s];
      for (int k = 0; k < 6; k ++) q[3+k] = q[3+k] + d.sad[off+k][s];
      const double xk = d.sad[3][s], xe = d.sad[4][s];
      q[9] = xk > q[9] ? xk : q[9];
      q[10] = xe > q[10] ? xe : q[10];
    }
  }
  double gq[11] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  for (int l = 0; l < RUN_GROUP; l ++)
  {
    double x[11];
    for (int k = 0; k < 11; k ++) x[k] = __shfl_sync(full, q[k], l);
    if (g * RUN_GROUP + l >= nc) break;
    for (int k = 0; k < 9; k ++) gq[k] = gq[k] + x[k];
    gq[9] = x[9] > gq[9] ? x[9] : gq[9];
    gq[10] = x[10] > gq[10] ? x[10] : gq[10];
  }
  if (lane == 0)
  {
    double *o = d.sbig_grp + ((size_t)run * RUN_GROUPS + g) * RUN_SLOT;
    for (int k = 0; k < 11; k ++) o[k] = gq[k];
  }
}

__global__ void k_spring_run_totals_adapt(PgDev d)
{
  const int run = blockIdx.x * blockDim.x + threadIdx.x;
  if (run >= d.nbig) return;
  const int4 v = d.sbig[run];
  const int len = v.z - v.y, ch = run_chunk(len), nc = (len + ch - 1) / ch, ng = (nc + RUN_GROUP - 1) / RUN_GROUP;
  double p[9] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, km = 0.0, em = 0.0;
  for (int r = 0; r < ng; r ++)
  {
    const double *o = d.sbig_grp + ((size_t)run * RUN_GROUPS + r) * RUN_SLOT;
    for (int k = 0; k < 9; k ++) p[k] = p[k] + o[k];
    km = o[9] > km ? o[9] : km;
    em = o[10] > em ? o[10] : em;
  }
  for (int k = 0; k < 9; k ++) d.sbig_ad[11*run + k] = p[k];
  d.sbig_ad[11*run + 9] = km;
  d.sbig_ad[11*run + 10] = em;
}

// MODE: INT_FUSED runs the whole particle update of one step; the drop-in
// entry points split it as the reference does: INT_FORCES ends with the
// force and torque sums (the tail of forces(), forces.ispc:453-596) and
// INT_DYNAMICS starts from the force and torque arrays (dynamics(),
// dynamics.ispc:30-169, with h = step and h-bar = (step + step1)/2).
// RESTRAIN (restrain.ispc:30-133): v loses its components along the three
// direction rows of restraint q, in order (SUBMUL (v, DOT (v, l), l, v))
__device__ __forceinline__ void restrain_vec(double *v, double *const dir[9], int q)
{
  for (int k = 0; k < 3; k ++)
  {
    const double l[3] = {dir[3*k][q], dir[3*k+1][q], dir[3*k+2][q]};
    const double dt = dot3(v, l);
    v[0] = v[0] - dt*l[0];
    v[1] = v[1] - dt*l[1];
    v[2] = v[2] - dt*l[2];
  }
}

// restrain_velocities_task (restrain.ispc:30-90) for one particle's
// restraints in input order: linear, spatial angular, and referential angular
// velocity against the directions taken to the body frame (L^T a)
__global__ void k_restrain_velocities(PgDev d, const int *first, const int *list, int parnum)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= parnum || first[j] == first[j+1]) return;
  double v[3] = {d.linear[0][j], d.linear[1][j], d.linear[2][j]};
  double O[3] = {d.angular[0][j], d.angular[1][j], d.angular[2][j]};
  double o[3] = {d.angular[3][j], d.angular[4][j], d.angular[5][j]};
  double L[9];
  for (int c = 0; c < 9; c ++) L[c] = d.rotation[c][j];
  for (int rr = first[j]; rr < first[j+1]; rr ++)
  {
    const int q = list[rr];
    restrain_vec(v, d.rstlin, q);
    restrain_vec(o, d.rstang, q);
    double A[3][3];
    for (int k = 0; k < 3; k ++)
    {
      const double a[3] = {d.rstang[3*k][q], d.rstang[3*k+1][q], d.rstang[3*k+2][q]};
      tvmul(L, a, A[k]);
    }
    for (int k = 0; k < 3; k ++)
    {
      const double dt = dot3(O, A[k]);
      O[0] = O[0] - dt*A[k][0];
      O[1] = O[1] - dt*A[k][1];
      O[2] = O[2] - dt*A[k][2];
    }
  }
  for (int c = 0; c < 3; c ++)
  {
    d.linear[c][j] = v[c];
    d.angular[c][j] = O[c];
    d.angular[3+c][j] = o[c];
  }
}

// restrain_forces_task (restrain.ispc:93-133) over the force arrays, for the
// drop-in export
__global__ void k_restrain_forces(PgDev d, const int *first, const int *list, int parnum)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= parnum || first[j] == first[j+1]) return;
  double f[3] = {d.force[0][j], d.force[1][j], d.force[2][j]};
  double t[3] = {d.torque[0][j], d.torque[1][j], d.torque[2][j]};
  for (int rr = first[j]; rr < first[j+1]; rr ++)
  {
    restrain_vec(f, d.rstlin, list[rr]);
    restrain_vec(t, d.rstang, list[rr]);
  }
  for (int c = 0; c < 3; c ++) { d.force[c][j] = f[c]; d.torque[c][j] = t[c]; }
}

// With adaptive stepping the step is split at the step choice:
// INT_FORCES_ADAPT ends with the force sums and the complete stiffness terms
// of every particle (forces.ispc:453-596, 1207-1412); INT_DYN_FUSED starts
// from the force arrays and runs the rest of INT_FUSED with step0 and step1
// from d.hs.
enum { INT_FUSED = 0, INT_FORCES = 1, INT_DYNAMICS = 2, INT_FORCES_ADAPT = 3, INT_DYN_FUSED = 4 };

// F + m*g on the integer pipe when g is a zero and m and F are finite: m*g
// is then a zero of sign sign(m) xor sign(g), and F plus a zero is F, except
// that two zeros sum to -0 only when both are -0 (the gravity components of
// a scene that are zero)
__device__ __forceinline__ double add_times_zero(double F, double m, double g)
{
  const unsigned long long bg = dbits(g);
  if ((bg << 1) != 0 || !finite_d(m) || !finite_d(F)) return F + m*g;
  const unsigned long long bF = dbits(F);
  if ((bF << 1) != 0) return F;
  const bool neg = (bF >> 63) && ((dbits(m) ^ bg) >> 63);
  return __longlong_as_double(neg ? (long long)0x8000000000000000ull : 0ll);
}

// half = step/2 and hstep = (step + step1)/2 come from the host (the same
// IEEE operations), except where the step is chosen on the device
template <int MODE>
__global__ void PG_LB_INTEGRATE k_integrate(PgDev d, double step, double half, double hstep)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool need = false;
  constexpr bool ADAPT = MODE == INT_FORCES_ADAPT;
  constexpr bool FUSED = MODE == INT_FUSED || MODE == INT_DYN_FUSED;
  if (MODE == INT_FORCES_ADAPT || MODE == INT_DYN_FUSED)
  {
    step = d.hs[0];
    half = 0.5*step;
    hstep = 0.5*(step+d.hs[1]);
  }
  if (i < d.parnum && d.pscene[i] >= 0 && d.sactive[d.pscene[i]])
  {
    const int row = *d.stepno;
    const double *damping = d.t_damping + 6*(size_t)row;
    const bool typo = (d.compat & PG_COMPAT_EXPMAP) != 0;
    const int E = d.ellnum;
    double po[3] = {d.position[0][i], d.position[1][i], d.position[2][i]};
    double F[3], T[3];
    const int e = d.pell ? d.pell[i] : -1;
    const double ma = d.mass[i];
    double kact[3] = {0.0, 0.0, 0.0}, krot[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, kmax = 0.0, emax = 0.0;
    double Li[9];
    if (ADAPT)
    {
      for (int k = 0; k < 9; k ++) Li[k] = d.rotation[k][i];
      if (e >= 0)
      {
        for (int k = 0; k < 3; k ++) kact[k] = d.akact[k][i];
        for (int k = 0; k < 6; k ++) krot[k] = d.akrot[k][i];
        kmax = d.akmax[i];
        emax = d.aemax[i];
      }
    }
    if (MODE == INT_DYNAMICS || MODE == INT_DYN_FUSED)
    {
      F[0] = d.force[0][i]; F[1] = d.force[1][i]; F[2] = d.force[2][i];
      T[0] = d.torque[0][i]; T[1] = d.torque[1][i]; T[2] = d.torque[2][i];
    }
    else
    {
    double grav[3];
    scene_gravity(d, d.pscene[i], step, d.t_gravity + 3*(size_t)row, grav);
    if (e >= 0 && !ADAPT && d.cwork)
    {
      // the master side of the sphere's contacts, summed here in slot order
      // as k_contacts_sum sums them into fm and tm in the adaptive mode
      double fs[3] = {0.0, 0.0, 0.0}, ts[3] = {0.0, 0.0, 0.0};
      const int cnt = d.ncnt[e];
      for (int k = 0; k < cnt; k ++)
      {
        const size_t idx = (size_t)k * d.estride + e;
        if (!d.nflag[idx]) continue;
        const double f[3] = {d.nfrc[0][idx], d.nfrc[1][idx], d.nfrc[2][idx]};
        const double a[3] = {d.npnt[0][idx]-po[0], d.npnt[1][idx]-po[1], d.npnt[2][idx]-po[2]};
        fs[0] += f[0]; fs[1] += f[1]; fs[2] += f[2];
        ts[0] += a[1]*f[2] - a[2]*f[1];
        ts[1] += a[2]*f[0] - a[0]*f[2];
        ts[2] += a[0]*f[1] - a[1]*f[0];
      }
      F[0] = fs[0]; F[1] = fs[1]; F[2] = fs[2];
      T[0] = ts[0]; T[1] = ts[1]; T[2] = ts[2];
    }
    else if (e >= 0)
    {
      F[0] = d.fm[0][i]; F[1] = d.fm[1][i]; F[2] = d.fm[2][i];
      T[0] = d.tm[0][i]; T[1] = d.tm[1][i]; T[2] = d.tm[2][i];
    }
    else { F[0] = F[1] = F[2] = 0.0; T[0] = T[1] = T[2] = 0.0; }

    // slave contacts, in master order (forces.ispc:539-569)
    if (E)
    {
      const int rb = d.soff[i], re = d.soff[i+1];
      for (int r = rb; r < re; r ++)
      {
        const int ref = d.rref[r];
        if (!d.nflag[ref]) continue;
        double f[3] = {-d.nfrc[0][ref], -d.nfrc[1][ref], -d.nfrc[2][ref]};
        double a[3] = {d.npnt[0][ref]-po[0], d.npnt[1][ref]-po[1], d.npnt[2][ref]-po[2]};
        F[0] += f[0]; F[1] += f[1]; F[2] += f[2];
        T[0] += a[1]*f[2] - a[2]*f[1];
        T[1] += a[2]*f[0] - a[0]*f[2];
        T[2] += a[0]*f[1] - a[1]*f[0];
        if (ADAPT)
        {
          // slave side (forces.ispc:539-567): the force direction, and the
          // contact's own stiffness and damping (the reference reads slave
          // records whose kcur/ecur nothing sets)
          double u[3] = {f[0], f[1], f[2]};
          double len = sqrt(dot3(u, u));
          if (len != 0.0)
          {
            len = 1.0/len;
            u[0] *= len; u[1] *= len; u[2] *= len;
          }
          else u[0] = u[1] = u[2] = 0.0;
          kact[0] += fabs(u[0]);
          kact[1] += fabs(u[1]);
          kact[2] += fabs(u[2]);
          const int ms = ref % d.estride, code = d.ncode[ref];
          const int ij = pairing(d, d.ellcol[ms], code >= 0 ? d.ellcol[code] : d.tricol[-code-1]);
          const double kc = d.iparam[0][ij];
          double ec;
          if (d.nen) ec = d.nen[ref];
          else ec = d.iparam[1][ij] * 2.0 * sqrt(kc*(1.0 / (d.invm[d.part[ms]] + d.invm[i])));
          kmax = kc > kmax ? kc : kmax;
          emax = ec > emax ? ec : emax;
          double A[3];
          nvmul(Li, a, A);
          krot_add(krot, A);
        }
      }
    }
    F[0] = add_times_zero(F[0], ma, grav[0]);
    F[1] = add_times_zero(F[1], ma, grav[1]);
    F[2] = add_times_zero(F[2], ma, grav[2]);
    if (d.tt_on)
    {
      // mesh-mesh contacts (pg_meshcontact.cu), summed per particle beforehand
      F[0] = F[0] + d.ttF[0][i]; F[1] = F[1] + d.ttF[1][i]; F[2] = F[2] + d.ttF[2][i];
      T[0] = T[0] + d.ttT[0][i]; T[1] = T[1] + d.ttT[1][i]; T[2] = T[2] + d.ttT[2][i];
    }

    // spring force flushes, in the order a single springs_task applies them
    if (d.sprnum)
    {
      for (int ev = d.sev_first[i]; ev < d.sev_first[i+1]; ev ++)
      {
        const int4 v = d.sev[ev];
        const int type = v.x & 1, run = (v.x >> 1) - 1;
        const int off = type == 0 ? 3 : 6;
        double af[3] = {0.0, 0.0, 0.0}, at[3] = {0.0, 0.0, 0.0};
        bool started = false;
        if (run >= 0)
        {
          // a long run, summed in the same order by k_spring_runs
          for (int c = 0; c < 3; c ++) { af[c] = d.sbig_sum[6*run + c]; at[c] = d.sbig_sum[6*run + 3 + c]; }
        }
        else
        for (int s = v.y; s < v.z; s ++)
        {
          if (type == 1 && d.sprpart[1][s] < 0) continue;
          double fr[3] = {d.spr_out[0][s], d.spr_out[1][s], d.spr_out[2][s]};
          double tq[3] = {d.spr_out[off][s], d.spr_out[off+1][s], d.spr_out[off+2][s]};
          if (!started && !v.w)
          {
            af[0] = fr[0]; af[1] = fr[1]; af[2] = fr[2];
            at[0] = tq[0]; at[1] = tq[1]; at[2] = tq[2];
          }
          else
          {
            af[0] += fr[0]; af[1] += fr[1]; af[2] += fr[2];
            at[0] += tq[0]; at[1] += tq[1]; at[2] += tq[2];
          }
          started = true;
        }
        if (type == 0)
        {
          F[0] += af[0]; F[1] += af[1]; F[2] += af[2];
          T[0] += at[0]; T[1] += at[1]; T[2] += at[2];
        }
        else
        {
          F[0] -= af[0]; F[1] -= af[1]; F[2] -= af[2];
          T[0] -= at[0]; T[1] -= at[1]; T[2] -= at[2];
        }
        if (ADAPT)
        {
          // the run's stiffness partials (forces.ispc:1212-1345): sums from
          // zero in spring order, maxima for stiffness and damping
          double p[9] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, km = 0.0, em = 0.0;
          if (run >= 0)
          {
            for (int c = 0; c < 9; c ++) p[c] = d.sbig_ad[11*run + c];
            km = d.sbig_ad[11*run + 9];
            em = d.sbig_ad[11*run + 10];
          }
          else
          {
            const int ao = type == 0 ? 5 : 11;
            for (int s = v.y; s < v.z; s ++)
            {
              if (type == 1 && d.sprpart[1][s] < 0) continue;
              for (int c = 0; c < 3; c ++) p[c] = p[c] + d.sad[c][s];
              for (int c = 0; c < 6; c ++) p[3+c] = p[3+c] + d.sad[ao+c][s];
              const double xk = d.sad[3][s], xe = d.sad[4][s];
              km = xk > km ? xk : km;
              em = xe > em ? xe : em;
            }
          }
          for (int c = 0; c < 3; c ++) kact[c] += p[c];
          for (int c = 0; c < 6; c ++) krot[c] += p[3+c];
          kmax = km > kmax ? km : kmax;
          emax = em > emax ? em : emax;
        }
      }
    }

    // torsion spring torque flushes (trqspr_task, forces.ispc:1667-2055),
    // after every translational spring flush, in the same run rule
    if (d.trqsprnum)
    {
      for (int ev = d.tev_first[i]; ev < d.tev_first[i+1]; ev ++)
      {
        const int4 v = d.tev[ev];
        const int type = v.x & 1;
        double at[3] = {0.0, 0.0, 0.0}, kp[3] = {0.0, 0.0, 0.0};
        bool started = false;
        for (int s = v.y; s < v.z; s ++)
        {
          if (type == 1 && d.trqsprpart[1][s] < 0) continue;
          const double tq[3] = {d.tq_out[0][s], d.tq_out[1][s], d.tq_out[2][s]};
          if (!started && !v.w) { at[0] = tq[0]; at[1] = tq[1]; at[2] = tq[2]; }
          else { at[0] += tq[0]; at[1] += tq[1]; at[2] += tq[2]; }
          if (ADAPT) for (int c = 0; c < 3; c ++) kp[c] = kp[c] + d.tq_k[c][s];
          started = true;
        }
        if (type == 0) { T[0] += at[0]; T[1] += at[1]; T[2] += at[2]; }
        else { T[0] -= at[0]; T[1] -= at[1]; T[2] -= at[2]; }
        if (ADAPT) for (int c = 0; c < 3; c ++) krot[c] += kp[c];
      }
    }

    // prescribe_body_forces (parmec.cpp:2202-2224): the particle's force and
    // torque are exported, then the prescribed ones added
    if ((MODE == INT_FUSED || MODE == INT_FORCES_ADAPT) && d.pbfnum)
    {
      const int q = d.pbf_slot[i];
      if (q >= 0)
        for (int c = 0; c < 3; c ++)
        {
          d.pbfin[c][q] = F[c];
          d.pbfin[3+c][q] = T[c];
          F[c] += d.pbfout[c][q];
          T[c] += d.pbfout[3+c][q];
        }
    }

    }
    if (ADAPT)
    {
      for (int k = 0; k < 3; k ++) d.akact[k][i] = kact[k];
      for (int k = 0; k < 6; k ++) d.akrot[k][i] = krot[k];
      d.akmax[i] = kmax;
      d.aemax[i] = emax;
    }
    if (MODE == INT_FORCES || MODE == INT_FORCES_ADAPT)
    {
      d.force[0][i] = F[0]; d.force[1][i] = F[1]; d.force[2][i] = F[2];
      d.torque[0][i] = T[0]; d.torque[1][i] = T[1]; d.torque[2][i] = T[2];
      return;
    }

    // restrain_forces (restrain.ispc:93-133), in input order; the drop-in
    // entry points run it as its own export
    if (FUSED && d.rstnum)
      for (int rr = d.rst_first[i]; rr < d.rst_first[i+1]; rr ++)
      {
        const int q = d.rst_list[rr];
        restrain_vec(F, d.rstlin, q);
        restrain_vec(T, d.rstang, q);
      }

    // prescribe_acceleration (input.cpp:4247-4341); the drop-in entry points
    // leave prescribed motion to the host, as parmec.cpp does
    const bool prs = FUSED && d.prsnum;
    const int pb = prs ? d.prs_first[i] : 0, pe = prs ? d.prs_first[i+1] : 0;
    for (int pp = pb; pp < pe; pp ++)
    {
      const int q = d.prs_list[pp];
      const double *lin = d.t_prs_lin + (size_t)row * d.tab_prs_stride + 3*q;
      const double *ang = d.t_prs_ang + (size_t)row * d.tab_prs_stride + 3*q;
      if (d.prslin[q] && d.linkind[q] == 1)
      {
        F[0] = ma * lin[0]; F[1] = ma * lin[1]; F[2] = ma * lin[2];
      }
      else if (d.prslin[q] && d.linkind[q] == 0)
      {
        F[0] = 0.0; F[1] = 0.0; F[2] = 0.0;
      }
      if (d.prsang[q] && d.angkind[q] == 1)
      {
        double in[9], acc[3] = {ang[0], ang[1], ang[2]};
        for (int k = 0; k < 9; k ++) in[k] = d.inertia[k][i];
        nvmul(in, acc, T);
      }
      else if (d.prsang[q] && d.angkind[q] == 0)
      {
        T[0] = 0.0; T[1] = 0.0; T[2] = 0.0;
      }
    }

    // dynamics_task (dynamics.ispc:30-169)
    double O[3], o[3], v[3], L1[9], J[9], I[9], im, f[3], t[3], Tb[3], DL[9], L2[9], A[3], B[3];
    double x[3] = {po[0], po[1], po[2]};
    if (!(d.flags[i] & PG_FLAG_SKIP))
    {
      for (int k = 0; k < 3; k ++) { O[k] = d.angular[k][i]; v[k] = d.linear[k][i]; }
      const bool iso = d.piso && d.piso[i];
      const double js = iso ? d.inertia[0][i] : 0.0, is = iso ? d.inverse[0][i] : 0.0;
      for (int k = 0; k < 9; k ++) L1[k] = d.rotation[k][i];
      if (!iso)
        for (int k = 0; k < 9; k ++) { J[k] = d.inertia[k][i]; I[k] = d.inverse[k][i]; }
      im = d.invm[i];
      if (nonzero_d(damping[0]) || nonzero_d(damping[1]) || nonzero_d(damping[2]))
      {
        F[0] -= ma * damping[0] * v[0];
        F[1] -= ma * damping[1] * v[1];
        F[2] -= ma * damping[2] * v[2];
      }
      if (nonzero_d(damping[3]) || nonzero_d(damping[4]) || nonzero_d(damping[5]))
      {
        o[0] = damping[3]*d.angular[3][i];
        o[1] = damping[4]*d.angular[4][i];
        o[2] = damping[5]*d.angular[5][i];
        tvmul(L1, o, t);
        if (iso) iso_nvmul(js, t, Tb); else nvmul(J, t, Tb);
        nvmul(L1, Tb, t);
        T[0] -= t[0]; T[1] -= t[1]; T[2] -= t[2];
      }
      f[0] = F[0]; f[1] = F[1]; f[2] = F[2];
      t[0] = T[0]; t[1] = T[1]; t[2] = T[2];
      tvmul(L1, t, Tb);
      expmap(-half*O[0], -half*O[1], -half*O[2], DL, typo);
      if (iso) iso_nvmul(js, O, A); else nvmul(J, O, A);
      nvmul(DL, A, B);
      B[0] = B[0] + half*Tb[0];
      B[1] = B[1] + half*Tb[1];
      B[2] = B[2] + half*Tb[2];
      if (iso) { iso_nvmul(is, B, A); iso_nvmul(js, A, B); }
      else { nvmul(I, B, A); nvmul(J, A, B); }
      Tb[0] -= A[1]*B[2] - A[2]*B[1];
      Tb[1] -= A[2]*B[0] - A[0]*B[2];
      Tb[2] -= A[0]*B[1] - A[1]*B[0];
      Tb[0] *= step; Tb[1] *= step; Tb[2] *= step;
      if (iso)
      {
        double IT[3];
        iso_nvmul(is, Tb, IT);
        O[0] = O[0] + IT[0]; O[1] = O[1] + IT[1]; O[2] = O[2] + IT[2];
      }
      else nvaddmul(O, I, Tb, O);
      im *= step;
      v[0] = v[0] + im*f[0];
      v[1] = v[1] + im*f[1];
      v[2] = v[2] + im*f[2];
      expmap(hstep*O[0], hstep*O[1], hstep*O[2], DL, typo);
      nnmul(L1, DL, L2);
      nvmul(L2, O, o);
      x[0] += hstep*v[0];
      x[1] += hstep*v[1];
      x[2] += hstep*v[2];

      // prescribe_velocity (input.cpp:4344-4421)
      for (int pp = pb; pp < pe; pp ++)
      {
        const int q = d.prs_list[pp];
        const double *lin = d.t_prs_lin + (size_t)row * d.tab_prs_stride + 3*q;
        const double *ang = d.t_prs_ang + (size_t)row * d.tab_prs_stride + 3*q;
        if (d.prslin[q] && d.linkind[q] == 0) { v[0] = lin[0]; v[1] = lin[1]; v[2] = lin[2]; }
        if (d.prsang[q] && d.angkind[q] == 0)
        {
          double oo[3] = {ang[0], ang[1], ang[2]};
          tvmul(L2, oo, O);
          o[0] = oo[0]; o[1] = oo[1]; o[2] = oo[2];
        }
      }

      for (int k = 0; k < 9; k ++) d.rotation[k][i] = L2[k];
      for (int k = 0; k < 3; k ++)
      {
        d.position[k][i] = x[k];
        d.angular[k][i] = O[k];
        d.angular[3+k][i] = o[k];
        d.linear[k][i] = v[k];
      }
    }
    else
    {
      // skipped particle: prescribe_velocity still applies (it runs after dynamics)
      for (int pp = pb; pp < pe; pp ++)
      {
        const int q = d.prs_list[pp];
        const double *lin = d.t_prs_lin + (size_t)row * d.tab_prs_stride + 3*q;
        const double *ang = d.t_prs_ang + (size_t)row * d.tab_prs_stride + 3*q;
        if (d.prslin[q] && d.linkind[q] == 0)
          for (int k = 0; k < 3; k ++) d.linear[k][i] = lin[k];
        if (d.prsang[q] && d.angkind[q] == 0)
        {
          double Lc[9], oo[3] = {ang[0], ang[1], ang[2]}, Oc[3];
          for (int k = 0; k < 9; k ++) Lc[k] = d.rotation[k][i];
          tvmul(Lc, oo, Oc);
          for (int k = 0; k < 3; k ++) { d.angular[k][i] = Oc[k]; d.angular[3+k][i] = oo[k]; }
        }
      }
      for (int k = 0; k < 9; k ++) L2[k] = d.rotation[k][i];
    }
    d.force[0][i] = F[0]; d.force[1][i] = F[1]; d.force[2][i] = F[2];
    d.torque[0][i] = T[0]; d.torque[1][i] = T[1]; d.torque[2][i] = T[2];

    // ellipsoids_task for this particle's sphere (shapes.ispc:29-98)
    if (FUSED && e >= 0)
    {
      double X[3] = {d.position[3][i], d.position[4][i], d.position[5][i]};
      double C[3] = {d.center[3][e], d.center[4][e], d.center[5][e]}, c[3];
      if (centre_is_position(x, L2, X, C)) { c[0] = x[0]; c[1] = x[1]; c[2] = x[2]; }
      else body_point(x, L2, X, C, c);
      d.center[0][e] = c[0]; d.center[1][e] = c[1]; d.center[2][e] = c[2];
      double r0 = c[0] - d.cref[0][e], r1 = c[1] - d.cref[1][e], r2 = c[2] - d.cref[2][e];
      need = gt_nonneg(r0*r0 + r1*r1 + r2*r2, d.half_skin_sq);
    }
  }
  if (FUSED && d.ellnum) flag_rebuild(d, need);
}

// ---------------------------------------------------------------- torsion springs
// trqspr_task (forces.ispc:1415-2057), one thread per torsion spring: the
// current frame rot1j = Lj [x0 y0 z0], roll/pitch/yaw rates of the relative
// spatial angular velocity, the integrated angles, spring torques from the
// angle lookups (or from the combined angle of a cone), dampers by lookup or
// by a critical damping ratio against the local equivalent inertia
// inv(rot1j (Jj^-1 + Jk^-1) rot1j^T).  The torque rot1j (roll, pitch, yaw)
// goes to tq_out and is flushed to the particles by k_integrate.  The
// pitch-yaw cone's pitch damper reads the pitch ratio (the reference reads
// the roll entry, forces.ispc:1823).
__device__ __forceinline__ double tq_spring(const PgDev &d, int o, int i, double arg, double *kslope)
{
  if (d.krpyidx[o][i+1] > d.krpyidx[o][i])
    return look_up(d.krpy[o][0], d.krpy[o][1], d.krpyidx[o][i], d.krpyidx[o][i+1], arg, kslope);
  *kslope = 0.0;
  return 0.0;
}

__device__ __forceinline__ double tq_damper(const PgDev &d, int o, int i, double rate, double kslope, double inertia)
{
  if (d.drpyidx[o][i]+1 == d.drpyidx[o][i+1])
  {
    const double ratio = d.drpy[o][0][d.drpyidx[o][i]];
    const double dm = - ratio * 2.0 * sqrt(fabs(kslope) * inertia);
    return rate * dm;
  }
  double dm;
  return look_up(d.drpy[o][0], d.drpy[o][1], d.drpyidx[o][i], d.drpyidx[o][i+1], rate, &dm);
}

__global__ void __launch_bounds__(TPB) k_torsion(PgDev d, double step)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.trqsprnum) return;
  if (d.hs) step = d.hs[0];
  const int j = d.trqsprpart[0][i], k = d.trqsprpart[1][i];
  double oj[3] = {d.angular[3][j], d.angular[4][j], d.angular[5][j]}, Lj[9];
  for (int c = 0; c < 9; c ++) Lj[c] = d.rotation[c][j];
  const double zdir0[3] = {d.trqzdir0[0][i], d.trqzdir0[1][i], d.trqzdir0[2][i]};
  const double xdir0[3] = {d.trqxdir0[0][i], d.trqxdir0[1][i], d.trqxdir0[2][i]};
  const double ydir0[3] = {zdir0[1]*xdir0[2] - zdir0[2]*xdir0[1], zdir0[2]*xdir0[0] - zdir0[0]*xdir0[2],
                           zdir0[0]*xdir0[1] - zdir0[1]*xdir0[0]};
  double rot1j[9];
  nvmul(Lj, xdir0, rot1j);
  nvmul(Lj, ydir0, rot1j+3);
  nvmul(Lj, zdir0, rot1j+6);
  for (int c = 0; c < 3; c ++) { d.trqzdir1[c][i] = rot1j[6+c]; d.trqxdir1[c][i] = rot1j[c]; }
  double ok[3] = {0.0, 0.0, 0.0};
  if (k >= 0) { ok[0] = d.angular[3][k]; ok[1] = d.angular[4][k]; ok[2] = d.angular[5][k]; }
  const double ojk[3] = {oj[0]-ok[0], oj[1]-ok[1], oj[2]-ok[2]};
  const double rolldot = dot3(rot1j, ojk), pitchdot = dot3(rot1j+3, ojk), yawdot = dot3(rot1j+6, ojk);
  double roll = d.trqrpy[0][i], pitch = d.trqrpy[1][i], yaw = d.trqrpy[2][i];
  roll += rolldot*step;
  pitch += pitchdot*step;
  yaw += yawdot*step;
  d.trqrpy[0][i] = roll; d.trqrpy[1][i] = pitch; d.trqrpy[2][i] = yaw;
  double Ixx = 0.0, Iyy = 0.0, Izz = 0.0;
  bool ratio = false;
  for (int o = 0; o < 3; o ++) ratio = ratio || d.drpyidx[o][i]+1 == d.drpyidx[o][i+1];
  if (ratio)
  {
    double I[9], tmp[9];
    for (int c = 0; c < 9; c ++) I[c] = d.inverse[c][j];
    if (k >= 0) for (int c = 0; c < 9; c ++) I[c] += d.inverse[c][k];
    ntmul(I, rot1j, tmp);
    nnmul(rot1j, tmp, I);
    invert3(I, tmp);
    Ixx = tmp[0]; Iyy = tmp[4]; Izz = tmp[8];
  }
  double kroll = 0.0, kpitch = 0.0, kyaw = 0.0;
  double trqroll = 0.0, trqpitch = 0.0, trqyaw = 0.0, trqrolltot = 0.0, trqpitchtot = 0.0, trqyawtot = 0.0;
  switch (d.trqcone[i])
  {
    case 0:
    {
      trqroll = tq_spring(d, 0, i, roll, &kroll);
      trqpitch = tq_spring(d, 1, i, pitch, &kpitch);
      trqyaw = tq_spring(d, 2, i, yaw, &kyaw);
      const double trqrolldot = tq_damper(d, 0, i, rolldot, kroll, Ixx);
      const double trqpitchdot = tq_damper(d, 1, i, pitchdot, kpitch, Iyy);
      const double trqyawdot = tq_damper(d, 2, i, yawdot, kyaw, Izz);
      trqrolltot = trqroll + (trqroll == 0.0 ? 0.0 : trqrolldot);
      trqpitchtot = trqpitch + (trqpitch == 0.0 ? 0.0 : trqpitchdot);
      trqyawtot = trqyaw + (trqyaw == 0.0 ? 0.0 : trqyawdot);
      break;
    }
    case 3:                                     // roll-pitch cone
    {
      const double angle = sqrt(roll*roll + pitch*pitch);
      const double angledot = angle > 0.0 ? (rolldot*roll+pitchdot*pitch)/angle : 0.0;
      trqroll = tq_spring(d, 0, i, angle, &kroll);
      kpitch = kroll;
      const double trqrolldot = tq_damper(d, 0, i, angledot, kroll, sqrt(Ixx*Ixx + Iyy*Iyy));
      trqyaw = tq_spring(d, 2, i, yaw, &kyaw);
      const double trqyawdot = tq_damper(d, 2, i, yawdot, kyaw, Izz);
      trqyawtot = trqyaw + (trqyaw == 0.0 ? 0.0 : trqyawdot);
      if (angle > 0.)
      {
        const double xcoef = roll/angle, ycoef = pitch/angle;
        trqrolltot = xcoef*(trqroll + (trqroll == 0.0 ? 0.0 : trqrolldot));
        trqpitchtot = ycoef*(trqroll + (trqroll == 0.0 ? 0.0 : trqrolldot));
        trqpitch = trqroll*ycoef;
        trqroll *= xcoef;
      }
      else { trqrolltot = trqpitchtot = 0.0; trqroll = trqpitch = 0.0; }
      break;
    }
    case 5:                                     // roll-yaw cone
    {
      const double angle = sqrt(roll*roll + yaw*yaw);
      const double angledot = angle > 0.0 ? (rolldot*roll+yawdot*yaw)/angle : 0.0;
      trqroll = tq_spring(d, 0, i, angle, &kroll);
      kyaw = kroll;
      const double trqrolldot = tq_damper(d, 0, i, angledot, kroll, sqrt(Ixx*Ixx + Izz*Izz));
      trqpitch = tq_spring(d, 1, i, pitch, &kpitch);
      const double trqpitchdot = tq_damper(d, 1, i, pitchdot, kpitch, Iyy);
      trqpitchtot = trqpitch + (trqpitch == 0.0 ? 0.0 : trqpitchdot);
      if (angle > 0.)
      {
        const double xcoef = roll/angle, zcoef = yaw/angle;
        trqrolltot = xcoef*(trqroll + (trqroll == 0.0 ? 0.0 : trqrolldot));
        trqyawtot = zcoef*(trqroll + (trqroll == 0.0 ? 0.0 : trqrolldot));
        trqyaw = trqroll*zcoef;
        trqroll *= xcoef;
      }
      else { trqrolltot = trqyawtot = 0.0; trqroll = trqyaw = 0.0; }
      break;
    }
    case 6:                                     // pitch-yaw cone
    {
      trqroll = tq_spring(d, 0, i, roll, &kroll);
      const double trqrolldot = tq_damper(d, 0, i, rolldot, kroll, Ixx);
      const double angle = sqrt(pitch*pitch + yaw*yaw);
      const double angledot = angle > 0.0 ? (pitchdot*pitch+yawdot*yaw)/angle : 0.0;
      trqpitch = tq_spring(d, 1, i, angle, &kpitch);
      kyaw = kpitch;
      const double trqpitchdot = tq_damper(d, 1, i, angledot, kpitch, sqrt(Iyy*Iyy + Izz*Izz));
      trqrolltot = trqroll + (trqroll == 0.0 ? 0.0 : trqrolldot);
      if (angle > 0.)
      {
        const double ycoef = pitch/angle, zcoef = yaw/angle;
        trqpitchtot = ycoef*(trqpitch + (trqpitch == 0.0 ? 0.0 : trqpitchdot));
        trqyawtot = zcoef*(trqpitch + (trqpitch == 0.0 ? 0.0 : trqpitchdot));
        trqyaw = zcoef*trqpitch;
        trqpitch *= ycoef;
      }
      else { trqpitchtot = trqyawtot = 0.0; trqpitch = trqyaw = 0.0; }
      break;
    }
    case 7:                                     // roll-pitch-yaw cone
    {
      const double angle = sqrt(roll*roll + pitch*pitch + yaw*yaw);
      const double angledot = angle > 0.0 ? (rolldot*roll+pitchdot*pitch+yawdot*yaw)/angle : 0.0;
      trqroll = tq_spring(d, 0, i, angle, &kroll);
      kpitch = kyaw = kroll;
      const double trqrolldot = tq_damper(d, 0, i, angledot, kroll, sqrt(Ixx*Ixx + Iyy*Iyy + Izz*Izz));
      if (angle > 0.)
      {
        const double xcoef = roll/angle, ycoef = pitch/angle, zcoef = yaw/angle;
        trqrolltot = xcoef*(trqroll + (trqroll == 0.0 ? 0.0 : trqrolldot));
        trqpitchtot = ycoef*(trqroll + (trqroll == 0.0 ? 0.0 : trqrolldot));
        trqyawtot = zcoef*(trqroll + (trqroll == 0.0 ? 0.0 : trqrolldot));
        trqpitch = ycoef*trqroll;
        trqyaw = zcoef*trqroll;
        trqroll *= xcoef;
      }
      else { trqrolltot = trqpitchtot = trqyawtot = 0.0; trqroll = trqpitch = trqyaw = 0.0; }
      break;
    }
  }
  d.tq_out[0][i] = trqrolltot*rot1j[0] + trqpitchtot*rot1j[3] + trqyawtot*rot1j[6];
  d.tq_out[1][i] = trqrolltot*rot1j[1] + trqpitchtot*rot1j[4] + trqyawtot*rot1j[7];
  d.tq_out[2][i] = trqrolltot*rot1j[2] + trqpitchtot*rot1j[5] + trqyawtot*rot1j[8];
  d.trqrpytot[0][i] = trqrolltot; d.trqrpytot[1][i] = trqpitchtot; d.trqrpytot[2][i] = trqyawtot;
  d.trqrpyspr[0][i] = trqroll; d.trqrpyspr[1][i] = trqpitch; d.trqrpyspr[2][i] = trqyaw;
  if (d.tq_k[0])
  {
    d.tq_k[0][i] = fabs(kroll)*rot1j[0];
    d.tq_k[1][i] = fabs(kpitch)*rot1j[4];
    d.tq_k[2][i] = fabs(kyaw)*rot1j[8];
  }
}

// ---------------------------------------------------------------- partial downloads
// out[c*n + j] = cols[c][idx[j]]: the rows a HISTORY sample reads, gathered
// into one buffer so that one small copy replaces a download of every array
__global__ void k_gather(const double *const *cols, int ncols, const int *idx, int n, double *out)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncols * n) return;
  const int c = t / n, j = t - c * n;
  out[t] = cols[c][idx[j]];
}

// ---------------------------------------------------------------- spring failures
// unspring_task (forces.ispc:2058-2127): the rules in order, by one thread, so
// that rules sharing springs act in the reference's sequence.  A rule is
// checked when stepnum % nsteps == 0 and nfreq > 0: the SUM/MIN/MAX of the
// entity over its tested springs, leaving (lower, upper) counts nfreq down,
// and at zero the monitored springs take the rule's action and the
// activated ones switch on.
__global__ void k_unspring(PgDev d)
{
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int stepnum = *d.ustep;
  for (int i = 0; i < d.unsprnum; i ++)
  {
    if (stepnum % d.unsteps[i]) continue;
    if (d.nfreq[i] == 0) continue;
    const int op = d.unop[i];
    double result = op == PG_OP_MIN ? 1.7976931348623157e308 : (op == PG_OP_MAX ? -1.7976931348623157e308 : 0.0);
    for (int j = d.u_tidx[i]; j < d.u_tidx[i+1]; j ++)
    {
      const int q = d.u_t[j];
      double value = 0.0;
      switch (d.unent[i])
      {
        case PG_HIS_STROKE: value = d.stroke[0][q]; break;
        case PG_HIS_F: value = d.sprfrc[0][q]; break;
        case PG_HIS_SF: value = d.sprfrc[1][q]; break;
        case PG_HIS_FF: value = d.sprfrc[2][q]; break;
      }
      if (d.unabs[i]) value = fabs(value);
      if (op == PG_OP_MIN) result = value < result ? value : result;
      else if (op == PG_OP_MAX) result = value > result ? value : result;
      else result += value;
    }
    if (result < d.unlim[0][i] || result > d.unlim[1][i])
    {
      const int nf = d.nfreq[i] - 1;
      d.nfreq[i] = nf;
      if (nf == 0)
      {
        for (int j = d.u_midx[i]; j < d.u_midx[i+1]; j ++) d.unspring[d.u_m[j]] = d.unaction[i];
        for (int j = d.u_aidx[i]; j < d.u_aidx[i+1]; j ++) d.unspring[d.u_a[j]] = -3;
      }
    }
  }
}

// ---------------------------------------------------------------- adaptive step
// adaptive_timestep (parmec.ispc:397-420): every particle's critical step
// from its stiffness terms, reduced to the smallest.  Non-negative doubles
// order as their bit patterns, so the minimum is an integer atomicMin (NaN
// patterns sort above every finite step and never win, as NaN is dropped by
// the reference's min).
__global__ void __launch_bounds__(TPB) k_adapt_min(PgDev d)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long bits = 0x7fefffffffffffffull;          // DBL_MAX
  if (i < d.parnum && d.pscene[i] >= 0 && d.sactive[d.pscene[i]])
  {
    double kact[3] = {d.akact[0][i], d.akact[1][i], d.akact[2][i]}, krot[6], J[9], om, ra;
    for (int k = 0; k < 6; k ++) krot[k] = d.akrot[k][i];
    for (int k = 0; k < 9; k ++) J[k] = d.inertia[k][i];
    const double h = critical_step(kact, d.akmax[i], d.aemax[i], krot, d.mass[i], J, &om, &ra);
    bits = (unsigned long long)__double_as_longlong(h);
  }
  for (int o = 16; o > 0; o >>= 1)
  {
    const unsigned long long other = __shfl_down_sync(0xffffffffu, bits, o);
    bits = other < bits ? other : bits;
  }
  if ((threadIdx.x & 31) == 0) atomicMin(d.hmin, bits);
}

// ---------------------------------------------------------------- CRITICAL (parmec.ispc:485-888)
// Largest absolute slope of a piecewise-linear table (the spring curve or the
// damping curve of spring j).
__device__ double table_max_slope(const double *t0, const double *t1, int lo, int hi)
{
  double m = 0.0;
  for (int q = lo; q < hi-1; q ++)
  {
    const double k = (t1[q+1]-t1[q]) / (t0[q+1]-t0[q]);
    const double a = fabs(k);
    m = a > m ? a : m;
  }
  return m;
}

// critical_perspring (parmec.ispc:485-544): one thread per spring; the
// equivalent mass of the two reference points along the spring direction,
// the curve's largest slope, the damping ratio given or from the damping
// curve, and the damped step (2/w)(sqrt(1+ksi^2) - ksi).
__global__ void __launch_bounds__(TPB) k_crit_perspring(PgDev d, double *h, double *om, double *ra)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= d.sprnum) return;
  const int i = d.sprpart[0][j], k = d.sprpart[1][j];
  const double pi[3] = {d.sprpnt[3][j], d.sprpnt[4][j], d.sprpnt[5][j]};
  const double pk[3] = {d.sprpnt[9][j], d.sprpnt[10][j], d.sprpnt[11][j]};
  const double dir[3] = {d.sprdir[0][j], d.sprdir[1][j], d.sprdir[2][j]};
  const double kspr = table_max_slope(d.spring[0], d.spring[1], d.spridx[j], d.spridx[j+1]);
  const double mspr = eqm(d, i, pi, k, pk, dir);
  const double omega = sqrt(kspr/mspr);
  double ksi = 0.0;
  if (d.dashidx[j]+1 == d.dashidx[j+1]) ksi = d.dashpot[0][d.dashidx[j]];
  else
  {
    const double espr = table_max_slope(d.dashpot[0], d.dashpot[1], d.dashidx[j], d.dashidx[j+1]);
    if (omega > 0.0) ksi = espr / (2*mspr*omega);
  }
  h[j] = omega > 0.0 ? (2.0/omega)*(sqrt(1.0+ksi*ksi) - ksi) : 1.0;
  om[j] = omega;
  ra[j] = ksi;
}

// critical_perparticle_springs, per-spring part (parmec.ispc:711-745): the
// curve's largest slope and the damping, a critical ratio through the
// equivalent mass or the damping curve's largest slope.  The spring's own
// damping table decides which (the reference indexes dashidx with the
// particle there, parmec.ispc:728).
__global__ void __launch_bounds__(TPB) k_crit_spring_terms(PgDev d, double *ke)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= d.sprnum) return;
  const double kspr = table_max_slope(d.spring[0], d.spring[1], d.spridx[j], d.spridx[j+1]);
  double espr = 0.0;
  if (d.dashidx[j]+1 == d.dashidx[j+1])
  {
    const double Pi[3] = {d.sprpnt[3][j], d.sprpnt[4][j], d.sprpnt[5][j]};
    const double Pk[3] = {d.sprpnt[9][j], d.sprpnt[10][j], d.sprpnt[11][j]};
    const double dir[3] = {d.sprdir[0][j], d.sprdir[1][j], d.sprdir[2][j]};
    const double mass = eqm(d, d.sprpart[0][j], Pi, d.sprpart[1][j], Pk, dir);
    espr = d.dashpot[0][d.dashidx[j]] * 2.0 * sqrt(kspr * mass);
  }
  else espr = table_max_slope(d.dashpot[0], d.dashpot[1], d.dashidx[j], d.dashidx[j+1]);
  ke[2*j] = kspr;
  ke[2*j+1] = espr;
}

// critical_perparticle (parmec.ispc:547-888): one thread per particle.
// Terms in the reference's order: the contacts the particle masters (its
// sphere's list, in list order), the contacts it is the partner of (slave
// list order), then its springs in spring order (the flush events of a
// particle are disjoint spring ranges in ascending order).  Contact normals
// are the recorded ones when the session records geometry, else the
// direction from the partner (sphere centre or contact point) to the
// sphere centre.  The slave side takes the contact's own stiffness and
// damping (the reference reads slave records whose kcur/ecur nothing sets);
// springs are classified by their own flags (the reference reads sprflg
// with the particle index, parmec.ispc:759).  Then time_step_task.
__global__ void __launch_bounds__(TPB) k_crit_perparticle(PgDev d, const double *ke, int use_contacts,
                                                          double *h, double *om, double *ra)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.parnum) return;
  const int E = d.ellnum;
  double kact[3] = {0.0, 0.0, 0.0}, krot[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, kmax = 0.0, emax = 0.0;
  double L[9], po[3] = {d.position[0][i], d.position[1][i], d.position[2][i]};
  for (int k = 0; k < 9; k ++) L[k] = d.rotation[k][i];
  if (use_contacts && E)
  {
    const int e = d.pell ? d.pell[i] : -1;
    if (e >= 0)
    {
      const double c[3] = {d.center[0][e], d.center[1][e], d.center[2][e]};
      for (int k = 0; k < d.ncnt[e]; k ++)
      {
        const size_t idx = (size_t)k * d.estride + e;
        if (!d.nflag[idx]) continue;
        const int code = d.ncode[idx];
        const double pnt[3] = {d.npnt[0][idx], d.npnt[1][idx], d.npnt[2][idx]};
        double n[3];
        if (d.record_geometry)
        {
          n[0] = d.nnrm[0][idx]; n[1] = d.nnrm[1][idx]; n[2] = d.nnrm[2][idx];
        }
        else
        {
          double q[3];
          if (code >= 0) { q[0] = c[0]-d.center[0][code]; q[1] = c[1]-d.center[1][code]; q[2] = c[2]-d.center[2][code]; }
          else { q[0] = c[0]-pnt[0]; q[1] = c[1]-pnt[1]; q[2] = c[2]-pnt[2]; }
          double ln = sqrt(dot3(q, q));
          if (!(ln > 0.0)) ln = 1.0;
          n[0] = q[0]/ln; n[1] = q[1]/ln; n[2] = q[2]/ln;
        }
        const int pj = code >= 0 ? d.part[code] : d.triobs[-code-1];
        const int ij = pairing(d, d.ellcol[e], code >= 0 ? d.ellcol[code] : d.tricol[-code-1]);
        const double kc = d.iparam[0][ij];
        const double ma = pj >= 0 ? 1.0 / (d.invm[i] + d.invm[pj]) : d.mass[i];
        const double ec = d.iparam[1][ij] * 2.0 * sqrt(kc*ma);
        kact[0] += fabs(n[0]);
        kact[1] += fabs(n[1]);
        kact[2] += fabs(n[2]);
        kmax = kc > kmax ? kc : kmax;
        emax = ec > emax ? ec : emax;
        const double a[3] = {pnt[0]-po[0], pnt[1]-po[1], pnt[2]-po[2]};
        double A[3];
        nvmul(L, a, A);
        krot_add(krot, A);
      }
    }
    for (int r = d.soff[i]; r < d.soff[i+1]; r ++)
    {
      const int ref = d.rref[r];
      if (!d.nflag[ref]) continue;
      double u[3] = {-d.nfrc[0][ref], -d.nfrc[1][ref], -d.nfrc[2][ref]};
      double len = sqrt(dot3(u, u));
      if (len != 0.0)
      {
        len = 1.0/len;
        u[0] *= len; u[1] *= len; u[2] *= len;
      }
      else u[0] = u[1] = u[2] = 0.0;
      kact[0] += fabs(u[0]);
      kact[1] += fabs(u[1]);
      kact[2] += fabs(u[2]);
      const int ms = ref % d.estride, code = d.ncode[ref];
      const int ij = pairing(d, d.ellcol[ms], code >= 0 ? d.ellcol[code] : d.tricol[-code-1]);
      const double kc = d.iparam[0][ij];
      const double ec = d.iparam[1][ij] * 2.0 * sqrt(kc*(1.0 / (d.invm[d.part[ms]] + d.invm[i])));
      kmax = kc > kmax ? kc : kmax;
      emax = ec > emax ? ec : emax;
      const double a[3] = {d.npnt[0][ref]-po[0], d.npnt[1][ref]-po[1], d.npnt[2][ref]-po[2]};
      double A[3];
      nvmul(L, a, A);
      krot_add(krot, A);
    }
  }
  if (d.sprnum)
    for (int ev = d.sev_first[i]; ev < d.sev_first[i+1]; ev ++)
    {
      const int4 v = d.sev[ev];
      const int side = v.x & 1;
      for (int s = v.y; s < v.z; s ++)
      {
        if (side == 1 && d.sprpart[1][s] < 0) continue;
        const double dir[3] = {d.sprdir[0][s], d.sprdir[1][s], d.sprdir[2][s]};
        if (dot3(dir, dir) > 0.0)
        {
          if (d.sprflg[s] & PG_SPRDIR_PLANAR)
          {
            double t1[3] = {dir[0] + 0.123, dir[1] + 0.346, dir[2] + 0.789}, t2[3];
            t2[0] = dir[1]*t1[2] - dir[2]*t1[1];
            t2[1] = dir[2]*t1[0] - dir[0]*t1[2];
            t2[2] = dir[0]*t1[1] - dir[1]*t1[0];
            const double i2 = 1.0/sqrt(dot3(t2, t2));
            t2[0] *= i2; t2[1] *= i2; t2[2] *= i2;
            t1[0] = t2[1]*dir[2] - t2[2]*dir[1];
            t1[1] = t2[2]*dir[0] - t2[0]*dir[2];
            t1[2] = t2[0]*dir[1] - t2[1]*dir[0];
            kact[0] += fabs(t1[0]) + fabs(t2[0]);
            kact[1] += fabs(t1[1]) + fabs(t2[1]);
            kact[2] += fabs(t1[2]) + fabs(t2[2]);
          }
          else
          {
            kact[0] += fabs(dir[0]);
            kact[1] += fabs(dir[1]);
            kact[2] += fabs(dir[2]);
          }
        }
        else
        {
          kact[0] += 1.0;
          kact[1] += 1.0;
          kact[2] += 1.0;
        }
        const int o = 6*side;
        const double a[3] = {d.sprpnt[o][s]-po[0], d.sprpnt[o+1][s]-po[1], d.sprpnt[o+2][s]-po[2]};
        double A[3];
        tvmul(L, a, A);
        krot_add(krot, A);
        const double kspr = ke[2*s], espr = ke[2*s+1];
        kmax = kmax > kspr ? kmax : kspr;
        emax = emax > espr ? emax : espr;
      }
    }
  for (int k = 0; k < 3; k ++) d.akact[k][i] = kact[k];
  for (int k = 0; k < 6; k ++) d.akrot[k][i] = krot[k];
  d.akmax[i] = kmax;
  d.aemax[i] = emax;
  double J[9], w, r;
  for (int k = 0; k < 9; k ++) J[k] = d.inertia[k][i];
  h[i] = critical_step(kact, kmax, emax, krot, d.mass[i], J, &w, &r);
  om[i] = w;
  ra[i] = r;
}

// One equivalent mass (the EQM command's eqm export) on particles 0 and
// (part2 >= 0) 1 of the view.
__global__ void k_eqm_one(PgDev d, int part2, const double *pts, double *out)
{
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const double *dir = pts + 6;
  out[0] = eqm(d, 0, pts, part2 >= 0 ? 1 : -1, pts + 3, dot3(dir, dir) > 0.0 ? dir : nullptr);
}

// step1 = factor * the smallest critical step, or step0 when nothing is
// restrained; re-arms the minimum for the next step
__global__ void k_adapt_select(PgDev d)
{
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const double hmin = __longlong_as_double((long long)*d.hmin);
  d.hs[1] = hmin < 1.7976931348623157e308 ? d.hs[2]*hmin : d.hs[0];
  *d.hmin = 0x7fefffffffffffffull;
}

} // namespace

// ================================================================ launchers
void pg_launch_invert(const PgDev &d, cudaStream_t s)
{
  if (d.parnum) k_invert<<<nblk(d.parnum), TPB, 0, s>>>(d);
}

void pg_launch_iso_flags(const PgDev &d, cudaStream_t s, int p0, int p1)
{
  if (p1 > p0 && d.piso) k_iso_flags<<<nblk(p1 - p0), TPB, 0, s>>>(d, p0, p1);
}

void pg_launch_euler(const PgDev &d, cudaStream_t s, double step)
{
  if (d.parnum) k_euler<<<nblk(d.parnum), TPB, 0, s>>>(d, step);
}

void pg_launch_shapes(const PgDev &d, cudaStream_t s, bool skip_analytical)
{
  if (d.ellnum) k_spheres<<<nblk(d.ellnum), TPB, 0, s>>>(d);
  if (d.nodnum) k_nodes<<<nblk(d.nodnum), TPB, 0, s>>>(d, skip_analytical ? 1 : 0);
  if (d.facnum) k_faces<<<nblk(d.facnum), TPB, 0, s>>>(d);
}

void pg_launch_obstacles_state(const PgDev &d, cudaStream_t s, double step)
{
  if (d.obsnum && d.trinum) k_obstacles<<<(d.trinum + 31) / 32, 32, 0, s>>>(d, step, 0);
  if (d.obsnum) k_tail<<<1, 32, 0, s>>>(d, step, 0);
}

// the grid of the queue pass: resident blocks over every SM
static int eval_blocks()
{
  static int nb = 0;
  if (!nb)
  {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_contacts_eval<false, false>, TPB, 0);
    nb = (sms > 0 ? sms : 152) * (per > 0 ? per : 8);
  }
  return nb;
}

void pg_launch_contacts(const PgDev &d, cudaStream_t s, double step)
{
  if (!d.ellnum) return;
  if (d.cwork && d.cwork_n)
  {
    // three passes (probe, queued evaluation, sums; the sums in k_integrate
    // unless adaptive): the same bits as k_contacts
    cudaMemsetAsync(d.cwork_n, 0, sizeof(int), s);
    k_contacts_probe<<<nblk(d.ellnum), TPB, 0, s>>>(d);
    const int nb = eval_blocks();
    if (d.hs)
    {
      if (d.record_geometry) k_contacts_eval<true, true><<<nb, TPB, 0, s>>>(d, step);
      else k_contacts_eval<false, true><<<nb, TPB, 0, s>>>(d, step);
      k_contacts_sum<true><<<nblk(d.ellnum), TPB, 0, s>>>(d);
    }
    else
    {
      // the master-side sums are taken by k_integrate (INT_FUSED, INT_FORCES)
      if (d.record_geometry) k_contacts_eval<true, false><<<nb, TPB, 0, s>>>(d, step);
      else k_contacts_eval<false, false><<<nb, TPB, 0, s>>>(d, step);
    }
    return;
  }
  if (d.hs)
  {
    if (d.record_geometry) k_contacts<true, true><<<nblk(d.ellnum), TPB, 0, s>>>(d, step);
    else k_contacts<false, true><<<nblk(d.ellnum), TPB, 0, s>>>(d, step);
  }
  else if (d.record_geometry) k_contacts<true, false><<<nblk(d.ellnum), TPB, 0, s>>>(d, step);
  else k_contacts<false, false><<<nblk(d.ellnum), TPB, 0, s>>>(d, step);
}

// the FP64 form evaluates the lists in three passes with adaptive stepping,
// two otherwise (one when no work queue is allocated); the mixed form in a
// sphere and a triangle pass (pg_mixed.cu)
int pg_contacts_kernel_count(const PgDev &d)
{
  if (!d.ellnum) return 0;
  if (d.form == PG_FORM_MIXED) return 2;
  return (d.cwork && d.cwork_n) ? (d.hs ? 3 : 2) : 1;
}

void pg_launch_springs(const PgDev &d, cudaStream_t s, double step)
{
  if (!d.sprnum) return;
  if (d.hs) k_springs<true><<<nblk(d.sprnum), TPB, 0, s>>>(d, step);
  else k_springs<false><<<nblk(d.sprnum), TPB, 0, s>>>(d, step);
}

void pg_launch_torsion(const PgDev &d, cudaStream_t s, double step)
{
  if (d.trqsprnum) k_torsion<<<nblk(d.trqsprnum), TPB, 0, s>>>(d, step);
}

void pg_launch_gather(const double *const *cols, int ncols, const int *idx, int n, double *out, cudaStream_t s)
{
  if (ncols > 0 && n > 0) k_gather<<<nblk(ncols * n), TPB, 0, s>>>(cols, ncols, idx, n, out);
}

void pg_launch_unspring(const PgDev &d, cudaStream_t s)
{
  if (d.sprnum && d.unsprnum) k_unspring<<<1, 32, 0, s>>>(d);
}

void pg_launch_spring_runs(const PgDev &d, cudaStream_t s)
{
  if (!(d.sprnum && d.nbig > 0)) return;
  const dim3 grid(d.nbig, RUN_GROUPS);      // runs on x: no 65,535 limit on their count
  const int tb = (d.nbig + 127) / 128;
  k_spring_run_groups<<<grid, RUN_GROUP, 0, s>>>(d);
  k_spring_run_totals<<<tb, 128, 0, s>>>(d);
  if (d.hs)
  {
    k_spring_run_groups_adapt<<<grid, RUN_GROUP, 0, s>>>(d);
    k_spring_run_totals_adapt<<<tb, 128, 0, s>>>(d);
  }
}

void pg_launch_integrate(const PgDev &d, cudaStream_t s, double step)
{
  if (d.parnum) k_integrate<INT_FUSED><<<nblk(d.parnum), TPB, 0, s>>>(d, step, 0.5*step, 0.5*(step+step));
}

void pg_launch_force_sums(const PgDev &d, cudaStream_t s)
{
  if (d.parnum) k_integrate<INT_FORCES><<<nblk(d.parnum), TPB, 0, s>>>(d, 0.0, 0.0, 0.0);
}

void pg_launch_dynamics(const PgDev &d, cudaStream_t s, double step0, double step1)
{
  if (d.parnum) k_integrate<INT_DYNAMICS><<<nblk(d.parnum), TPB, 0, s>>>(d, step0, 0.5*step0, 0.5*(step0+step1));
}

void pg_launch_force_sums_adapt(const PgDev &d, cudaStream_t s)
{
  if (d.parnum) k_integrate<INT_FORCES_ADAPT><<<nblk(d.parnum), TPB, 0, s>>>(d, 0.0, 0.0, 0.0);
}

void pg_launch_adapt_step(const PgDev &d, cudaStream_t s)
{
  if (d.parnum) k_adapt_min<<<nblk(d.parnum), TPB, 0, s>>>(d);
  k_adapt_select<<<1, 32, 0, s>>>(d);
}

void pg_launch_critical_perspring(const PgDev &d, cudaStream_t s, double *h, double *om, double *ra)
{
  if (d.sprnum) k_crit_perspring<<<nblk(d.sprnum), TPB, 0, s>>>(d, h, om, ra);
}

void pg_launch_critical_perparticle(const PgDev &d, cudaStream_t s, double *ke, int use_contacts, double *h,
                                    double *om, double *ra)
{
  if (d.sprnum) k_crit_spring_terms<<<nblk(d.sprnum), TPB, 0, s>>>(d, ke);
  if (d.parnum) k_crit_perparticle<<<nblk(d.parnum), TPB, 0, s>>>(d, ke, use_contacts, h, om, ra);
}

void pg_launch_eqm_one(const PgDev &d, cudaStream_t s, int part2, const double *pts, double *out)
{
  k_eqm_one<<<1, 32, 0, s>>>(d, part2, pts, out);
}

void pg_launch_dynamics_fused(const PgDev &d, cudaStream_t s)
{
  if (d.parnum) k_integrate<INT_DYN_FUSED><<<nblk(d.parnum), TPB, 0, s>>>(d, 0.0, 0.0, 0.0);
}

void pg_launch_restrain_velocities(const PgDev &d, cudaStream_t s)
{
  if (d.parnum && d.rstnum) k_restrain_velocities<<<nblk(d.parnum), TPB, 0, s>>>(d, d.rst_first, d.rst_list, d.parnum);
}

void pg_launch_restrain_forces(const PgDev &d, cudaStream_t s)
{
  if (d.parnum && d.rstnum) k_restrain_forces<<<nblk(d.parnum), TPB, 0, s>>>(d, d.rst_first, d.rst_list, d.parnum);
}

void pg_launch_mesh(const PgDev &d, cudaStream_t s)
{
  if (d.nodnum) k_nodes<<<nblk(d.nodnum), TPB, 0, s>>>(d, 1);
  if (d.facnum) k_faces<<<nblk(d.facnum), TPB, 0, s>>>(d);
}

void pg_launch_obstacles_row(const PgDev &d, cudaStream_t s, double step)
{
  // one warp per block: a few thousand triangles then spread over most SMs,
  // each triangle's update being a chain of FP64 work
  if (d.obsnum && d.trinum) k_obstacles<<<(d.trinum + 31) / 32, 32, 0, s>>>(d, step, 1);
}

void pg_launch_excite(const PgDev &d, cudaStream_t s, double step)
{
  k_excite<<<nblk(d.nscene), TPB, 0, s>>>(d, step);
}

void pg_launch_tail(const PgDev &d, cudaStream_t s, double step)
{
  k_tail<<<1, 32, 0, s>>>(d, step, 1);
}

// the obstacle update and the tail of a step: one launch when the session
// has the completion counter, else the two kernels
void pg_launch_obstacles_tail(const PgDev &d, cudaStream_t s, double step)
{
  if (d.obsnum && d.trinum && d.obs_done) k_obstacles_tail<<<(d.trinum + 31) / 32, 32, 0, s>>>(d, step);
  else
  {
    pg_launch_obstacles_row(d, s, step);
    pg_launch_tail(d, s, step);
  }
}

int pg_obstacles_kernel_count(const PgDev &d)
{
  return 1 + ((d.obsnum && d.trinum && !d.obs_done) ? 1 : 0);
}

int pg_step_kernel_count(const PgDev &d)
{
  int n = 1;                                   // excite
  n += pg_contacts_kernel_count(d);            // contacts: sphere and triangle passes
  if (d.sprnum) n += 1 + (d.nbig > 0 ? 2 : 0) + (d.unsprnum ? 1 : 0);
  if (d.trqsprnum) n += 1;                     // torsion springs
  if (d.parnum) n += 1;                        // integrate
  if (d.nodnum) n += 1;
  if (d.facnum) n += 1;
  n += pg_obstacles_kernel_count(d);           // obstacles and tail
  return n;
}
