// pg_mixed.cu -- the mixed-precision step (PG_FORM_MIXED).
//
// GB300 issues FP64 at 1/64 of its FP32 rate, so this form keeps everything on
// the FP32 pipe:
//   * positions, linear velocities, rotations and sphere radii are compensated
//     FP32 pairs (pg_df.cuh, ~48 significant bits), so that positions are
//     accumulated with FP64-class accuracy and the near-touching gap
//     r_i + r_j - |x_i - x_j| is evaluated without cancellation;
//   * contact normals, velocities, forces, torques, tangential state and the
//     angular dynamics run in FP32.
// Sums keep the FP64 form's order (master list, then slave list), so results
// are reproducible run to run.  The FP64 arrays of the session remain the
// interchange format: uploads convert FP64 -> pairs (k_mx_from64), downloads
// convert back (k_mx_to64).  Scope: sphere particles whose sphere centre is the
// particle's reference point (SPHERE), triangles of obstacles, analytical
// particles; no springs or meshes.
#include <cuda_runtime.h>
#include "pg_state.h"
#include "pg_math.cuh"
#include "pg_df.cuh"
#include "pg_launch.h"
#include "pg_items.cuh"
#include "../../include/parmec_gb300.h"

using namespace pg;

namespace {

constexpr int TPB = 128;
inline int nblk(int n) { return (n + TPB - 1) / TPB; }
// resident blocks per SM asked of the register allocator for the per-phase
// contact and integration kernels (latency-bound gathers: more resident
// warps keep more loads in flight)
#ifndef PG_MX_MIN_BLOCKS
#define PG_MX_MIN_BLOCKS 8
#endif

__device__ __forceinline__ void set_err(const PgDev &d, int code, int site, int index, int value)
{
  if (atomicCAS(d.err, 0, code) == 0) { d.err[1] = site; d.err[2] = index; d.err[3] = value; }
}

__device__ __forceinline__ void flag_rebuild(const PgDev &d, bool need)
{
  unsigned m = __ballot_sync(__activemask(), need);
  if (m && (threadIdx.x & 31) == (__ffs(m) - 1)) atomicExch(d.rebuild, 1);
}

// FP32 expmap: the FP64 form's expression tree in single precision
__device__ __forceinline__ void expmap_f(float O1, float O2, float O3, float *L, bool typo)
{
  float v0 = O1 * O1, v1 = O2 * O2, v2 = O3 * O3;
  float angsq = v0 + v1 + v2, sx, cx;
  if (angsq < 3.0461741978671E-02f)
  {
    sx = 1.0f + (-1.666666666666667E-1f + (8.333333333333333E-3f + (-1.984126984126984E-4f +
         (2.755731922398589E-6f + (-2.505210838544172E-8f + 1.605904383682161E-10f * angsq) * angsq) * angsq)
         * angsq) * angsq) * angsq;
    cx = 0.5f + (-4.166666666666667E-2f + (1.388888888888889E-3f + (-2.480158730158730E-5f +
         (2.755731922398589E-7f + (-2.087675698786810E-9f + 1.147074559772972E-11f * angsq) * angsq) * angsq)
         * angsq) * angsq) * angsq;
  }
  else
  {
    float t = angsq, a = sqrtf(angsq), s, c;
    sincosf(a, &s, &c);
    sx = s / a;
    cx = (1.0f - c) / t;
  }
  float v01 = O1 * O2, v02 = typo ? O2 * O3 : O1 * O3, v12 = O2 * O3;
  float s0 = sx * O1, s1 = sx * O2, s2 = sx * O3;
  L[0] = 1.0f - cx*(v2+v1); L[1] = cx*v01 + s2;  L[2] = cx*v02 - s1;
  L[3] = cx*v01 - s2;       L[4] = 1.0f - cx*(v2+v0); L[5] = cx*v12 + s0;
  L[6] = cx*v02 + s1;       L[7] = cx*v12 - s0;  L[8] = 1.0f - cx*(v1+v0);
}

__device__ __forceinline__ void nvmul_f(const float *A, const float *B, float *C)
{
  C[0] = A[0]*B[0]+A[3]*B[1]+A[6]*B[2];
  C[1] = A[1]*B[0]+A[4]*B[1]+A[7]*B[2];
  C[2] = A[2]*B[0]+A[5]*B[1]+A[8]*B[2];
}

__device__ __forceinline__ void tvmul_f(const float *A, const float *B, float *C)
{
  C[0] = A[0]*B[0]+A[1]*B[1]+A[2]*B[2];
  C[1] = A[3]*B[0]+A[4]*B[1]+A[5]*B[2];
  C[2] = A[6]*B[0]+A[7]*B[1]+A[8]*B[2];
}

// C = M B for the inertia tensor (or its inverse) of particle i: an isotropic
// body (a sphere, scalar s != 0) multiplies by s; any other body reads its
// FP32 tensor at each product, so no 3x3 tensor stays live in registers
__device__ __forceinline__ void inertia_mul(float s, float *const M[9], int i, const float *B, float *C)
{
  if (s != 0.0f)
  {
    C[0] = s*B[0]; C[1] = s*B[1]; C[2] = s*B[2];
  }
  else
  {
    C[0] = M[0][i]*B[0]+M[3][i]*B[1]+M[6][i]*B[2];
    C[1] = M[1][i]*B[0]+M[4][i]*B[1]+M[7][i]*B[2];
    C[2] = M[2][i]*B[0]+M[5][i]*B[1]+M[8][i]*B[2];
  }
}

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

// ------------------------------------------------------------ conversions
// j and 1/j of particle i when its inertia is j*I and its inverse (1/j)*I,
// else 0 (the full FP32 matrices are used then)
__device__ __forceinline__ void set_iso(const PgDev &d, int i)
{
  const double j = d.inertia[0][i], ij = d.inverse[0][i];
  bool iso = j == d.inertia[4][i] && j == d.inertia[8][i] && ij == d.inverse[4][i] && ij == d.inverse[8][i];
  const int off[6] = {1, 2, 3, 5, 6, 7};
  for (int k = 0; k < 6; k ++) iso = iso && d.inertia[off[k]][i] == 0.0 && d.inverse[off[k]][i] == 0.0;
  d.jiso[i] = iso ? (float)j : 0.0f;
  d.iiso[i] = iso ? (float)ij : 0.0f;
}

__global__ void k_mx_from64(PgDev d, int p0, int p1, int e0, int e1)
{
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  int i = p0 + t;
  if (i < p1)
  {
    for (int k = 0; k < 3; k ++)
    {
      df x = df_from(d.position[k][i]); d.xh[k][i] = x.hi; d.xl[k][i] = x.lo;
      df v = df_from(d.linear[k][i]); d.vh[k][i] = v.hi; d.vl[k][i] = v.lo;
      d.Om[k][i] = (float)d.angular[k][i];
      d.om[k][i] = (float)d.angular[3+k][i];
      d.F_f[k][i] = (float)d.force[k][i];
      d.T_f[k][i] = (float)d.torque[k][i];
    }
    for (int k = 0; k < 9; k ++)
    {
      df l = df_from(d.rotation[k][i]); d.Lh[k][i] = l.hi; d.Ll[k][i] = l.lo;
      d.J_f[k][i] = (float)d.inertia[k][i];
      d.I_f[k][i] = (float)d.inverse[k][i];
    }
    d.mass_f[i] = (float)d.mass[i];
    d.invm_f[i] = (float)d.invm[i];
    set_iso(d, i);
  }
  int e = e0 + t;
  if (e < e1)
  {
    df r = df_from(d.radii[0][e]);
    d.rh[e] = r.hi; d.rl[e] = r.lo;
  }
}

__global__ void k_mx_inertia(PgDev d)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.parnum) return;
  for (int k = 0; k < 9; k ++) { d.J_f[k][i] = (float)d.inertia[k][i]; d.I_f[k][i] = (float)d.inverse[k][i]; }
  d.mass_f[i] = (float)d.mass[i];
  d.invm_f[i] = (float)d.invm[i];
  set_iso(d, i);
}

// sphere centres (FP64, for the rebuild's keys and distance tests) and their
// FP32 reference copies, from the particle position pairs; only when a
// rebuild is due -- between rebuilds the mixed step never reads them
__device__ __forceinline__ void mx_centres_item(const PgDev &d, int e)
{
  const int p = d.part[e];
  for (int c = 0; c < 3; c ++)
  {
    d.center[c][e] = df_to({d.xh[c][p], d.xl[c][p]});
    d.cref_f[c][e] = d.xh[c][p];
  }
}

// launched every step and idle unless a rebuild is due: a grid-stride loop
// over a grid of a few blocks per SM, so that the idle launch is short
__global__ void k_mx_centres(PgDev d)
{
  if (!*d.rebuild) return;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < d.ellnum; e += gridDim.x * blockDim.x)
    mx_centres_item(d, e);
}

__global__ void k_mx_to64(PgDev d, int p0, int p1)
{
  int i = p0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p1) return;
  for (int k = 0; k < 3; k ++)
  {
    d.position[k][i] = df_to({d.xh[k][i], d.xl[k][i]});
    d.linear[k][i] = df_to({d.vh[k][i], d.vl[k][i]});
    d.angular[k][i] = (double)d.Om[k][i];
    d.angular[3+k][i] = (double)d.om[k][i];
    d.force[k][i] = (double)d.F_f[k][i];
    d.torque[k][i] = (double)d.T_f[k][i];
  }
  for (int k = 0; k < 9; k ++) d.rotation[k][i] = df_to({d.Lh[k][i], d.Ll[k][i]});
  int e = d.pell[i];
  if (e >= 0) for (int k = 0; k < 3; k ++) d.center[k][e] = d.position[k][i];
}

// ------------------------------------------------------------ contacts
// A sphere's candidate list holds its sphere partners first, then its
// triangles (order_key).  PASS selects the entries one call evaluates:
//   MX_SPHERES   the sphere partners; returns whether triangles follow;
//   MX_TRIANGLES the triangles, continuing the sums the sphere pass stored.
// The force and torque sums take the FP32 additions of a single pass over
// the list, in the same order.
constexpr int MX_SPHERES = 1, MX_TRIANGLES = 2;

template <int PASS>
__device__ __forceinline__ bool mx_contacts_item(const PgDev &d, int i, double step_d)
{
  const int E = d.ellnum;
  const int pi = d.part[i];
  const int cnt = d.ncnt[i];
  bool more = false;
  float fs[3] = {0.0f, 0.0f, 0.0f}, ts[3] = {0.0f, 0.0f, 0.0f};
  if (PASS == MX_TRIANGLES)
    for (int c = 0; c < 3; c ++) { fs[c] = d.fm_f[c][pi]; ts[c] = d.tm_f[c][pi]; }
  if (cnt > 0)
  {
    const float step = (float)step_d;
    const bool obsc = (d.compat & PG_COMPAT_OBSIDX) != 0;
    const bool etypo = (d.compat & PG_COMPAT_TRIEDGE) != 0;
    df x[3];
    float v[3], oi[3];
    for (int k = 0; k < 3; k ++)
    {
      x[k] = {d.xh[k][pi], d.xl[k][pi]};
      v[k] = d.vh[k][pi];
      oi[k] = d.om[k][pi];
    }
    const df ri = {d.rh[i], d.rl[i]};
    const int coli = d.ellcol[i];
    const float invmi = d.invm_f[pi], massi = d.mass_f[pi];
    // the triangle pass starts at the first triangle, so that the j-th
    // triangles of the threads of a warp are evaluated together
    int k0 = 0;
    if (PASS == MX_TRIANGLES)
      while (k0 < cnt && d.ncode[(size_t)k0 * d.estride + i] >= 0) k0 ++;
    for (int k = k0; k < cnt; k ++)
    {
      const size_t idx = (size_t)k * d.estride + i;
      const int code = d.ncode[idx];
      if (PASS == MX_SPHERES && code < 0) { more = true; break; }
      const bool existing = d.nflag[idx] != 0;
      float normal[3], armi[3], armj[3] = {0.0f, 0.0f, 0.0f}, depth;
      bool pos, neg;
      int pj, colj;
      double pnt[3] = {0.0, 0.0, 0.0};
      if (code >= 0)
      {
        const int j = code;
        pj = d.part[j];
        colj = d.ellcol[j];
        df q[3];
        for (int c = 0; c < 3; c ++) q[c] = df_sub(x[c], {d.xh[c][pj], d.xl[c][pj]});
        df d2 = df_add(df_add(df_mul(q[0], q[0]), df_mul(q[1], q[1])), df_mul(q[2], q[2]));
        df len = df_sqrt(d2);
        df dep = df_sub(df_add(ri, {d.rh[j], d.rl[j]}), len);
        depth = df_f(dep);
        pos = df_pos(dep);
        neg = df_neg_(dep);
        float qf[3] = {df_f(q[0]), df_f(q[1]), df_f(q[2])};
        float lenf = df_f(len);
        float ilen = existing ? 1.0f / lenf : (lenf > 0.0f ? 1.0f / lenf : 1.0f);
        for (int c = 0; c < 3; c ++)
        {
          normal[c] = ilen * qf[c];
          armi[c] = -0.5f * qf[c];
          armj[c] = 0.5f * qf[c];
        }
      }
      else
      {
        const int t = -code-1;
        double A[3], B[3], C[3], cd[3], nd[3];
        for (int c = 0; c < 3; c ++)
        {
          A[c] = d.tri[c][t]; B[c] = d.tri[3+c][t]; C[c] = d.tri[6+c][t];
          cd[c] = df_to(x[c]);
        }
        double dd = triangle_sphere(A, B, C, cd, df_to(ri), pnt, nd, etypo);
        depth = (float)dd;
        pos = dd > 0.0;
        neg = dd < 0.0;
        for (int c = 0; c < 3; c ++) { normal[c] = (float)nd[c]; armi[c] = (float)(pnt[c] - cd[c]); }
        pj = d.triobs[t];
        colj = d.tricol[t];
      }
      const bool active = existing ? !neg : pos;
      if (!active)
      {
        if (existing)
        {
          d.nflag[idx] = 0;
          d.nstate_f[0][idx] = 0.0f; d.nstate_f[1][idx] = 0.0f; d.nstate_f[2][idx] = 0.0f;
        }
        continue;
      }
      float vi[3], vj[3], vij[3];
      vi[0] = oi[1]*armi[2]-oi[2]*armi[1] + v[0];
      vi[1] = oi[2]*armi[0]-oi[0]*armi[2] + v[1];
      vi[2] = oi[0]*armi[1]-oi[1]*armi[0] + v[2];
      if (pj >= 0)
      {
        float oj[3] = {d.om[0][pj], d.om[1][pj], d.om[2][pj]};
        vj[0] = oj[1]*armj[2]-oj[2]*armj[1] + d.vh[0][pj];
        vj[1] = oj[2]*armj[0]-oj[0]*armj[2] + d.vh[1][pj];
        vj[2] = oj[0]*armj[1]-oj[1]*armj[0] + d.vh[2][pj];
      }
      else
      {
        int l = -pj-2;
        if (obsc && l >= 0) l = l+1;
        if (l >= 0 && l < d.obsnum)
        {
          float z[3], oj[3];
          for (int c = 0; c < 3; c ++)
          {
            z[c] = (float)(pnt[c] - d.obspnt[3*l+c]);
            oj[c] = (float)d.obsang[3*l+c];
          }
          vj[0] = oj[1]*z[2]-oj[2]*z[1] + (float)d.obslin[3*l];
          vj[1] = oj[2]*z[0]-oj[0]*z[2] + (float)d.obslin[3*l+1];
          vj[2] = oj[0]*z[1]-oj[1]*z[0] + (float)d.obslin[3*l+2];
        }
        else { vj[0] = vj[1] = vj[2] = 0.0f; }
      }
      for (int c = 0; c < 3; c ++) vij[c] = vj[c] - vi[c];
      const int ij = pairing(d, coli, colj);
      if (d.ikind[ij] != 0) set_err(d, PG_ERR_UNSUPPORTED, 4, i, ij);
      float state[3];
      if (existing) { state[0] = d.nstate_f[0][idx]; state[1] = d.nstate_f[1][idx]; state[2] = d.nstate_f[2][idx]; }
      else { state[0] = state[1] = state[2] = 0.0f; }
      float ma = pj >= 0 ? 1.0f / (invmi + d.invm_f[pj]) : massi;
      float kn = d.iparam_f[0][ij];
      float en = d.iparam_f[1][ij] * 2.0f * sqrtf(kn*ma);
      float vn = vij[0]*normal[0] + vij[1]*normal[1] + vij[2]*normal[2];
      float fn = kn*depth + en*vn;
      float kskn = d.iparam_f[6][ij];
      float kt = kn * kskn, et = en * kskn;
      float mus = d.iparam_f[2][ij], mud = d.iparam_f[3][ij];
      float f[3], vt[3], ft[3];
      for (int c = 0; c < 3; c ++)
      {
        f[c] = fn*normal[c];
        vt[c] = vij[c] - vn*normal[c];
        state[c] += step*vt[c];
        ft[c] = kt*state[c] + et*vt[c];
      }
      float flen = sqrtf(ft[0]*ft[0] + ft[1]*ft[1] + ft[2]*ft[2]);
      float lim = mus*fn;
      if (flen > lim)
      {
        lim = mud*fn/flen;
        ft[0] *= lim; ft[1] *= lim; ft[2] *= lim;
      }
      for (int c = 0; c < 3; c ++) f[c] += ft[c];
      d.nflag[idx] = 1;
      for (int c = 0; c < 3; c ++)
      {
        d.nstate_f[c][idx] = state[c];
        d.nfrc_f[c][idx] = f[c];
        d.narm_f[c][idx] = armj[c];
      }
      fs[0] += f[0]; fs[1] += f[1]; fs[2] += f[2];
      ts[0] += armi[1]*f[2] - armi[2]*f[1];
      ts[1] += armi[2]*f[0] - armi[0]*f[2];
      ts[2] += armi[0]*f[1] - armi[1]*f[0];
    }
  }
  for (int c = 0; c < 3; c ++) { d.fm_f[c][pi] = fs[c]; d.tm_f[c][pi] = ts[c]; }
  return more;
}

// the sphere partners of every sphere; spheres whose lists go on with
// triangles are queued for k_tri_mx (queue order does not matter: each
// sphere's triangles are evaluated by one thread, in list order)
__global__ void __launch_bounds__(TPB, PG_MX_MIN_BLOCKS) k_contacts_mx(PgDev d, double step_d)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool more = false;
  if (i < d.ellnum) more = mx_contacts_item<MX_SPHERES>(d, i, step_d);
  pgk::tri_queue_push(d, more, i);
}

// the triangle candidates of the queued spheres, one thread per sphere; the
// last block to finish resets the queue for the next step
__global__ void __launch_bounds__(TPB) k_tri_mx(PgDev d, double step_d)
{
  const int n = pgk::tri_queue_len(d);
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x)
    mx_contacts_item<MX_TRIANGLES>(d, d.twork[q], step_d);
  pgk::tri_queue_done(d);
}

// ------------------------------------------------------------ integrate
// returns whether the particle's sphere left its rebuild neighbourhood
__device__ __forceinline__ bool mx_integrate_item(const PgDev &d, int i, double step_d)
{
  bool need = false;
  if (d.pscene[i] >= 0 && d.sactive[d.pscene[i]])
  {
    const int row = *d.stepno;
    const int sc = d.pscene[i];
    const float grav[3] = {d.sgrav_f[3*sc], d.sgrav_f[3*sc+1], d.sgrav_f[3*sc+2]};
    const float *damping = d.damp_f;
    const bool typo = (d.compat & PG_COMPAT_EXPMAP) != 0;
    const float step = (float)step_d;
    const int e = d.pell[i];
    float F[3] = {0.0f, 0.0f, 0.0f}, T[3] = {0.0f, 0.0f, 0.0f};
    if (e >= 0) for (int c = 0; c < 3; c ++) { F[c] = d.fm_f[c][i]; T[c] = d.tm_f[c][i]; }
    if (d.ellnum)
    {
      const int rb = d.soff[i], re = d.soff[i+1];
      for (int r = rb; r < re; r ++)
      {
        const int ref = d.rref[r];
        if (!d.nflag[ref]) continue;
        float f[3] = {-d.nfrc_f[0][ref], -d.nfrc_f[1][ref], -d.nfrc_f[2][ref]};
        float a[3] = {d.narm_f[0][ref], d.narm_f[1][ref], d.narm_f[2][ref]};
        F[0] += f[0]; F[1] += f[1]; F[2] += f[2];
        T[0] += a[1]*f[2] - a[2]*f[1];
        T[1] += a[2]*f[0] - a[0]*f[2];
        T[2] += a[0]*f[1] - a[1]*f[0];
      }
    }
    const float ma = d.mass_f[i];
    for (int c = 0; c < 3; c ++) F[c] = F[c] + ma * grav[c];

    const int pb = d.prsnum ? d.prs_first[i] : 0, pe = d.prsnum ? d.prs_first[i+1] : 0;
    for (int pp = pb; pp < pe; pp ++)
    {
      const int q = d.prs_list[pp];
      const double *lin = d.t_prs_lin + (size_t)row * d.tab_prs_stride + 3*q;
      const double *ang = d.t_prs_ang + (size_t)row * d.tab_prs_stride + 3*q;
      if (d.prslin[q] && d.linkind[q] == 1) for (int c = 0; c < 3; c ++) F[c] = ma * (float)lin[c];
      else if (d.prslin[q] && d.linkind[q] == 0) F[0] = F[1] = F[2] = 0.0f;
      if (d.prsang[q] && d.angkind[q] == 1)
      {
        float in[9], acc[3] = {(float)ang[0], (float)ang[1], (float)ang[2]};
        for (int k = 0; k < 9; k ++) in[k] = d.J_f[k][i];
        nvmul_f(in, acc, T);
      }
      else if (d.prsang[q] && d.angkind[q] == 0) T[0] = T[1] = T[2] = 0.0f;
    }

    df x[3], v[3], L[9];
    float O[3], o[3], Lf[9];
    for (int c = 0; c < 3; c ++)
    {
      x[c] = {d.xh[c][i], d.xl[c][i]};
      v[c] = {d.vh[c][i], d.vl[c][i]};
      O[c] = d.Om[c][i];
      o[c] = d.om[c][i];
    }
    // isotropic bodies (spheres) have js = j, is = 1/j; others js = is = 0
    const float js = d.jiso[i], is = d.iiso[i];
    for (int k = 0; k < 9; k ++)
    {
      L[k] = {d.Lh[k][i], d.Ll[k][i]};
      Lf[k] = L[k].hi;
    }
    if (!(d.flags[i] & PG_FLAG_SKIP))
    {
      const float half = 0.5f * step, hstep = step;
      if (damping[0] != 0.0f || damping[1] != 0.0f || damping[2] != 0.0f)
        for (int c = 0; c < 3; c ++) F[c] -= ma * damping[c] * v[c].hi;
      if (damping[3] != 0.0f || damping[4] != 0.0f || damping[5] != 0.0f)
      {
        float w[3], t[3], Tb[3];
        for (int c = 0; c < 3; c ++) w[c] = damping[3+c] * o[c];
        tvmul_f(Lf, w, t);
        inertia_mul(js, d.J_f, i, t, Tb);
        nvmul_f(Lf, Tb, t);
        for (int c = 0; c < 3; c ++) T[c] -= t[c];
      }
      float Tb[3], DL[9], A[3], B[3];
      tvmul_f(Lf, T, Tb);
      expmap_f(-half*O[0], -half*O[1], -half*O[2], DL, typo);
      inertia_mul(js, d.J_f, i, O, A);
      nvmul_f(DL, A, B);
      for (int c = 0; c < 3; c ++) B[c] = B[c] + half*Tb[c];
      inertia_mul(is, d.I_f, i, B, A);
      inertia_mul(js, d.J_f, i, A, B);
      Tb[0] -= A[1]*B[2] - A[2]*B[1];
      Tb[1] -= A[2]*B[0] - A[0]*B[2];
      Tb[2] -= A[0]*B[1] - A[1]*B[0];
      for (int c = 0; c < 3; c ++) Tb[c] *= step;
      float IT[3];
      inertia_mul(is, d.I_f, i, Tb, IT);
      for (int c = 0; c < 3; c ++) O[c] = O[c] + IT[c];
      const float im = d.invm_f[i] * step;
      for (int c = 0; c < 3; c ++) v[c] = df_add_f(v[c], im * F[c]);
      expmap_f(hstep*O[0], hstep*O[1], hstep*O[2], DL, typo);
      df L2[9];
      for (int col = 0; col < 3; col ++)
        for (int row3 = 0; row3 < 3; row3 ++)
        {
          df acc = df_mul_f(L[row3], DL[3*col]);
          acc = df_add(acc, df_mul_f(L[3+row3], DL[3*col+1]));
          acc = df_add(acc, df_mul_f(L[6+row3], DL[3*col+2]));
          L2[3*col+row3] = acc;
        }
      for (int k = 0; k < 9; k ++) { L[k] = L2[k]; Lf[k] = L2[k].hi; }
      nvmul_f(Lf, O, o);
      for (int c = 0; c < 3; c ++) x[c] = df_add(x[c], df_mul_f(v[c], hstep));
      for (int pp = pb; pp < pe; pp ++)
      {
        const int q = d.prs_list[pp];
        const double *lin = d.t_prs_lin + (size_t)row * d.tab_prs_stride + 3*q;
        const double *ang = d.t_prs_ang + (size_t)row * d.tab_prs_stride + 3*q;
        if (d.prslin[q] && d.linkind[q] == 0) for (int c = 0; c < 3; c ++) v[c] = df_from(lin[c]);
        if (d.prsang[q] && d.angkind[q] == 0)
        {
          float oo[3] = {(float)ang[0], (float)ang[1], (float)ang[2]};
          tvmul_f(Lf, oo, O);
          o[0] = oo[0]; o[1] = oo[1]; o[2] = oo[2];
        }
      }
      for (int c = 0; c < 3; c ++)
      {
        d.xh[c][i] = x[c].hi; d.xl[c][i] = x[c].lo;
        d.vh[c][i] = v[c].hi; d.vl[c][i] = v[c].lo;
        d.Om[c][i] = O[c];
        d.om[c][i] = o[c];
      }
      for (int k = 0; k < 9; k ++) { d.Lh[k][i] = L[k].hi; d.Ll[k][i] = L[k].lo; }
    }
    for (int c = 0; c < 3; c ++) { d.F_f[c][i] = F[c]; d.T_f[c][i] = T[c]; }
    if (e >= 0)
    {
      // displacement since the last rebuild, in FP32 (the FP64 centres are
      // written only when a rebuild is due)
      float dd = 0.0f;
      for (int c = 0; c < 3; c ++)
      {
        float r = (x[c].hi - d.cref_f[c][e]) + x[c].lo;
        dd += r*r;
      }
      need = dd > d.half_skin_sq_f;
    }
  }
  return need;
}

__global__ void __launch_bounds__(TPB, PG_MX_MIN_BLOCKS) k_integrate_mx(PgDev d, double step_d)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool need = false;
  if (i < d.parnum) need = mx_integrate_item(d, i, step_d);
  if (d.ellnum) flag_rebuild(d, need);
}

// ------------------------------------------------------------ fused step
// One cooperatively launched grid runs a whole step of the mixed form:
//   excitation + sphere contacts | triangle contacts | integration +
//   obstacles | tail
// with a grid barrier at each '|'.  Every block walks the items of a phase in
// a grid-stride loop; the item bodies are the ones the per-phase kernels run,
// so the results do not depend on the launch shape.  The candidate-list
// rebuild, when flagged, is the cooperative rebuild kernel launched before
// each step (pg_launch_fused_mx): inside this kernel's register budget
// (chosen for the step phases) the rebuild ran at a fraction of its speed.
template <int B, int MINB>
__global__ void __launch_bounds__(B, MINB) k_fused_mx(PgDev d, double step)
{
  const int gsz = gridDim.x * B;
  const int g0 = blockIdx.x * B + threadIdx.x;
  const int E = d.ellnum, P = d.parnum, T = d.trinum;
  // excitation and contacts: contacts do not read the scene gravity
  for (int sc = g0; sc < d.nscene; sc += gsz) pgk::excite_item(d, sc, step);
  // sphere partners, queueing spheres with triangles (the loop's trip count
  // is the same for every lane of a warp: the queue push is a warp vote)
  for (int i = g0; i - (int)(threadIdx.x & 31) < E; i += gsz)
  {
    bool more = false;
    if (i < E) more = mx_contacts_item<MX_SPHERES>(d, i, step);
    pgk::tri_queue_push(d, more, i);
  }
  if (!pgk::grid_barrier(d)) return;
  {
    const int n = pgk::tri_queue_len(d);
    for (int q = g0; q < n; q += gsz) mx_contacts_item<MX_TRIANGLES>(d, d.twork[q], step);
  }
  if (!pgk::grid_barrier(d)) return;
  // integration and obstacle triangles touch disjoint state; nothing reads
  // the triangle queue again before the next step's contacts
  if (blockIdx.x == 0 && threadIdx.x == 0) d.tcnt[0] = 0;
  bool need = false;
  for (int i = g0; i < P; i += gsz) need |= mx_integrate_item(d, i, step);
  for (int t = g0; t < T; t += gsz) need |= pgk::obstacles_item(d, t, step, 1);
  if (__syncthreads_or(need) && threadIdx.x == 0 && E) atomicExch(d.rebuild, 1);
  if (!pgk::grid_barrier(d)) return;
  if (blockIdx.x == 0 && threadIdx.x == 0) pgk::tail_item(d, step, 1);
}

typedef void (*FusedKernel)(PgDev, double);

// the launch shapes the autotuner may pick from (threads, minimum blocks per SM)
struct FusedShape { int threads, minb; FusedKernel k; };
const FusedShape fused_shapes[] = {
  {256, 1, k_fused_mx<256, 1>}, {256, 2, k_fused_mx<256, 2>}, {256, 3, k_fused_mx<256, 3>},
  {512, 1, k_fused_mx<512, 1>}, {512, 2, k_fused_mx<512, 2>},
};
constexpr int n_fused_shapes = sizeof(fused_shapes) / sizeof(fused_shapes[0]);

} // namespace

// candidate launch configurations: every shape at every blocks-per-SM count up
// to its occupancy limit (cooperative launches need all blocks resident)
int pg_fused_candidates(PgFusedCfg *out, int cap)
{
  int dev = 0, sms = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  for (int k = 0; k < n_fused_shapes; k ++)
  {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fused_shapes[k].k, fused_shapes[k].threads, 0)
        != cudaSuccess) { cudaGetLastError(); continue; }
    for (int b = 1; b <= per_sm && b <= 4; b ++)
    {
      if (b < fused_shapes[k].minb) continue;
      if (n < cap) out[n] = {k, fused_shapes[k].threads, b * sms};
      n ++;
    }
  }
  return n < cap ? n : cap;
}

cudaError_t pg_launch_fused_mx(const PgDev &d, cudaStream_t s, double step, int nsteps, const PgFusedCfg &c)
{
  if (c.shape < 0 || c.shape >= n_fused_shapes || c.blocks < 1) return cudaErrorInvalidValue;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(c.blocks);
  cfg.blockDim = dim3(fused_shapes[c.shape].threads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  for (int k = 0; k < nsteps; k ++)
  {
    // the rebuild, when flagged (both return at once otherwise)
    pg_launch_mx_centres(d, s);
    pg_launch_rebuild(d, s);
    cudaError_t e = cudaMemsetAsync(d.gbar, 0, 4 * sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    e = cudaLaunchKernelEx(&cfg, fused_shapes[c.shape].k, d, step);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

void pg_launch_mx_from64(const PgDev &d, cudaStream_t s, int p0, int p1, int e0, int e1)
{
  if (p1 < 0) p1 = d.parnum;
  if (e1 < 0) e1 = d.ellnum;
  int n = (p1 - p0) > (e1 - e0) ? (p1 - p0) : (e1 - e0);
  if (n > 0) k_mx_from64<<<nblk(n), TPB, 0, s>>>(d, p0, p1, e0, e1);
}

void pg_launch_mx_inertia(const PgDev &d, cudaStream_t s)
{
  if (d.parnum) k_mx_inertia<<<nblk(d.parnum), TPB, 0, s>>>(d);
}

void pg_launch_mx_to64(const PgDev &d, cudaStream_t s, int p0, int p1)
{
  if (p1 < 0) p1 = d.parnum;
  if (p1 > p0) k_mx_to64<<<nblk(p1 - p0), TPB, 0, s>>>(d, p0, p1);
}

void pg_launch_mx_centres(const PgDev &d, cudaStream_t s)
{
  static int cap = 0;
  if (!cap)
  {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cap = 4 * (sms > 0 ? sms : 152);
  }
  const int nb = nblk(d.ellnum);
  if (d.ellnum) k_mx_centres<<<nb < cap ? nb : cap, TPB, 0, s>>>(d);
}

void pg_launch_contacts_mx(const PgDev &d, cudaStream_t s, double step)
{
  if (!d.ellnum) return;
  k_contacts_mx<<<nblk(d.ellnum), TPB, 0, s>>>(d, step);
  const int nb = nblk(d.ellnum);
  k_tri_mx<<<nb < pgk::TRI_PASS_BLOCKS ? nb : pgk::TRI_PASS_BLOCKS, TPB, 0, s>>>(d, step);
}

void pg_launch_integrate_mx(const PgDev &d, cudaStream_t s, double step)
{
  if (d.parnum) k_integrate_mx<<<nblk(d.parnum), TPB, 0, s>>>(d, step);
}
