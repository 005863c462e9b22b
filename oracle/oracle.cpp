/*
 * oracle.cpp -- TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.
 *
 * A CPU restatement of Parmec's explicit DEM step (the ISPC hot path), used
 * only as the parity checker by tests/, by __graft_entry__.smoke(), and as the
 * timed CPU baseline by bench.py.  Nothing in parmec_gb300/ links or calls it.
 *
 * It follows the reference statement by statement, in the same floating-point
 * operation order, and is compiled with -ffp-contract=off (no fused
 * multiply-add) so that results are reproducible bit for bit:
 *
 *   macros.h:97-1050      vector / 3x3 helpers (same expression trees)
 *   macros.h:1453-1535    expmap (DEFINE_EXPMAP), with the v02 typo switch
 *   dynamics.ispc:30-169  dynamics_task
 *   parmec.ispc:62-99     invert;  224-272 euler_task;  423-482 eqm
 *   shapes.ispc:29-211    ellipsoids_task, nodes_task, faces_task
 *   obstacles.ispc:28-78  obstacles
 *   condet.ispc:98-290    sphere-sphere narrow phase;  294-400 triangle_sphere;
 *                         412-516 drop_triangle;  627-700 update_existing
 *   forces.ispc:98-192    pairing, granural_force;  195-407 contacts_task;
 *                         410-450 look_up(_slope);  453-596 contacts_acc_task;
 *                         641-1412 springs_task (single-task order)
 *   parmec.cpp:2397-2517  the dem() loop body;  input.cpp:4247-4421 prescribe
 *
 * Choices where the reference is not deterministic or not well defined
 * (each one is stated, not hidden):
 *   - Contact set: the exact set {depth > 0} for new pairs (the reference's
 *     kd-tree query can miss pairs, condet.ispc:279-283); existing contacts
 *     persist while depth >= 0 (forces.ispc:191, 327-365).
 *   - Contact list order: per master particle, sorted by partner code
 *     (sphere partners by ellipsoid index, then triangles by index).  The
 *     reference's order depends on lock acquisition (condet.ispc:187-263).
 *     Slave lists are ordered by master particle, then master-list order.
 *   - Sums: sequential in list order (the reference sums 8 SIMD lane partials
 *     then reduce_add, forces.ispc:492-577).
 *   - Friction state: zero when a contact is created and moved with its
 *     contact on removal (the reference leaves state[] uninitialised and does
 *     not move it, condet.ispc:229-260, forces.ispc:339-357).
 *   - pairing(): the binary search of forces.ispc:98-122 can loop forever when
 *     start == mid; the restatement stops the search there (same result when it
 *     terminates).
 *   - Springs with equal (part0, part1) keep their input order (the reference
 *     uses std::sort, parmec.cpp:1683).
 *   - Literals are C++ doubles; ispc may treat unsuffixed literals as float
 *     (affects expmap's series coefficients by <= 1e-16 relative at DEM steps).
 *
 * Parity pins: tests/golden holds the two self-checking decks of the
 * reference (tests/damping.py, tests/spring_curve_tests.py) restated in
 * Python 3, plus analytic known-answer cases; tests/test_reference_pin.py
 * compares the whole step with the reference's own ISPC sources, translated
 * to C++ by oracle/ispc_ref.py and run with parmec.cpp's call sequence.
 *
 * Mesh-mesh contact (or_mesh_contact) is an extension with no counterpart in
 * the reference: its pair search is a brute-force restatement of the
 * device's definitions (pg_meshcontact.cu), and its narrow phase and contact
 * law are the shared functions of parmec_gb300/csrc/pg_tritri.cuh, checked
 * on their own against analytic distances by tests/test_meshcontact.py.
 */
#include "../include/parmec_gb300.h"
#include "../parmec_gb300/csrc/pg_tritri.cuh"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

enum { SPRING = 0, DAMPER, FRISTAT, FRIDYN, FRIROL, FRIDRIL, KSKN };

/* ---------------- macros.h helpers, same expression trees ----------------- */

inline double DOT(const double *a, const double *b) { return a[0]*b[0] + a[1]*b[1] + a[2]*b[2]; }
inline double LEN(const double *a) { return std::sqrt(DOT(a, a)); }

/* NVMUL macros.h:945 */
inline void NVMUL(const double *A, const double *B, double *C)
{
  C[0] = A[0]*B[0]+A[3]*B[1]+A[6]*B[2];
  C[1] = A[1]*B[0]+A[4]*B[1]+A[7]*B[2];
  C[2] = A[2]*B[0]+A[5]*B[1]+A[8]*B[2];
}
/* TVMUL macros.h:966 */
inline void TVMUL(const double *A, const double *B, double *C)
{
  C[0] = A[0]*B[0]+A[1]*B[1]+A[2]*B[2];
  C[1] = A[3]*B[0]+A[4]*B[1]+A[5]*B[2];
  C[2] = A[6]*B[0]+A[7]*B[1]+A[8]*B[2];
}
/* NVADDMUL macros.h:973 */
inline void NVADDMUL(const double *C, const double *A, const double *B, double *D)
{
  D[0] = C[0] + (A[0]*B[0]+A[3]*B[1]+A[6]*B[2]);
  D[1] = C[1] + (A[1]*B[0]+A[4]*B[1]+A[7]*B[2]);
  D[2] = C[2] + (A[2]*B[0]+A[5]*B[1]+A[8]*B[2]);
}
/* NNMUL macros.h:906 */
inline void NNMUL(const double *A, const double *B, double *C)
{
  C[0] = A[0]*B[0]+A[3]*B[1]+A[6]*B[2];
  C[1] = A[1]*B[0]+A[4]*B[1]+A[7]*B[2];
  C[2] = A[2]*B[0]+A[5]*B[1]+A[8]*B[2];
  C[3] = A[0]*B[3]+A[3]*B[4]+A[6]*B[5];
  C[4] = A[1]*B[3]+A[4]*B[4]+A[7]*B[5];
  C[5] = A[2]*B[3]+A[5]*B[4]+A[8]*B[5];
  C[6] = A[0]*B[6]+A[3]*B[7]+A[6]*B[8];
  C[7] = A[1]*B[6]+A[4]*B[7]+A[7]*B[8];
  C[8] = A[2]*B[6]+A[5]*B[7]+A[8]*B[8];
}
/* TNMUL macros.h:919 */
inline void TNMUL(const double *A, const double *B, double *C)
{
  C[0] = A[0]*B[0]+A[1]*B[1]+A[2]*B[2];
  C[1] = A[3]*B[0]+A[4]*B[1]+A[5]*B[2];
  C[2] = A[6]*B[0]+A[7]*B[1]+A[8]*B[2];
  C[3] = A[0]*B[3]+A[1]*B[4]+A[2]*B[5];
  C[4] = A[3]*B[3]+A[4]*B[4]+A[5]*B[5];
  C[5] = A[6]*B[3]+A[7]*B[4]+A[8]*B[5];
  C[6] = A[0]*B[6]+A[1]*B[7]+A[2]*B[8];
  C[7] = A[3]*B[6]+A[4]*B[7]+A[5]*B[8];
  C[8] = A[6]*B[6]+A[7]*B[7]+A[8]*B[8];
}
/* VECSKEW macros.h:1085 */
inline void VECSKEW(const double *V, double *A)
{
  A[0] = 0; A[1] = V[2]; A[2] = -V[1];
  A[3] = -V[2]; A[4] = 0; A[5] = V[0];
  A[6] = V[1]; A[7] = -V[0]; A[8] = 0;
}
/* DET macros.h:1029 */
inline double DET(const double *F)
{
  return F[0]*(F[4]*F[8]-F[5]*F[7]) + F[3]*(F[2]*F[7]-F[1]*F[8]) + F[6]*(F[1]*F[5]-F[2]*F[4]);
}
/* INVERT macros.h:1033 */
inline void INVERT(const double *F, double *INV)
{
  double det = F[0]*(F[4]*F[8]-F[5]*F[7]) + F[3]*(F[2]*F[7]-F[1]*F[8]) + (F[1]*F[5]-F[2]*F[4])*F[6];
  if (det != 0.0)
  {
    det = 1.0 / det;
    INV[0] = (F[4]*F[8]-F[5]*F[7])*det;
    INV[1] = (F[2]*F[7]-F[1]*F[8])*det;
    INV[2] = (F[1]*F[5]-F[2]*F[4])*det;
    INV[3] = (F[5]*F[6]-F[3]*F[8])*det;
    INV[4] = (F[0]*F[8]-F[2]*F[6])*det;
    INV[5] = (F[2]*F[3]-F[0]*F[5])*det;
    INV[6] = (F[3]*F[7]-F[4]*F[6])*det;
    INV[7] = (F[1]*F[6]-F[0]*F[7])*det;
    INV[8] = (F[0]*F[4]-F[1]*F[3])*det;
  }
}

/* DEFINE_EXPMAP macros.h:1453-1535; 'typo' reproduces v02 = Omega2*Omega3 */
inline void expmap(double O1, double O2, double O3, double *L, bool typo)
{
  double angsq, sx, cx, v0, v1, v2, v01, v02, v12, s0, s1, s2;
  v0 = O1 * O1;
  v1 = O2 * O2;
  v2 = O3 * O3;
  angsq = v0 + v1 + v2;
  if (angsq < 3.0461741978671E-02)
  {
    sx = 1.0 +
      (-1.666666666666667E-1 +
       (8.333333333333333E-3 +
        (-1.984126984126984E-4 +
         (2.755731922398589E-6 +
          (-2.505210838544172E-8 +
           1.605904383682161E-10 * angsq
          )*angsq
         )*angsq
        )*angsq
       )*angsq
      )*angsq;
    cx = 0.5 +
      (-4.166666666666667E-2 +
       (1.388888888888889E-3 +
        (-2.480158730158730E-5 +
         (2.755731922398589E-7 +
          (-2.087675698786810E-9 +
           1.147074559772972E-11 * angsq
          )*angsq
         )*angsq
        )*angsq
       )*angsq
      )*angsq;
  }
  else
  {
    double t = angsq;
    angsq = std::sqrt(angsq);
    double s = std::sin(angsq), c = std::cos(angsq);
    sx = s / angsq;
    cx = (1.0 - c) / t;
  }
  v01 = O1 * O2;
  v02 = typo ? O2 * O3 : O1 * O3;
  v12 = O2 * O3;
  s0 = sx * O1;
  s1 = sx * O2;
  s2 = sx * O3;
  L[0] = -cx*(v2+v1);
  L[1] = cx*v01;
  L[2] = cx*v02;
  L[3] = L[1];
  L[4] = -cx*(v2+v0);
  L[5] = cx*v12;
  L[6] = L[2];
  L[7] = L[5];
  L[8] = -cx*(v1+v0);
  L[0] += 1.0;
  L[1] += s2;
  L[2] -= s1;
  L[3] -= s2;
  L[4] += 1.0;
  L[5] += s0;
  L[6] += s1;
  L[7] -= s0;
  L[8] += 1.0;
}

/* cos(acos(r)/3) (largest) or cos(acos(r)/3 + 2 pi/3) (smallest), taken as
 * roots of the triple-angle identity 4c^3 - 3c = r by Newton's method from
 * c = 1 (or -1): the cubic is convex and increasing on [1/2, 1] (concave and
 * increasing on [-1, -1/2]), so the iterates move monotonically to the root
 * and the loop stops when they cease to.  Basic operations only: the same
 * bits on every IEEE machine (the reference's acos and cos come from the ISPC
 * standard library, which nothing pins). */
inline double triple_angle_root(double r, bool largest)
{
  r = r < -1.0 ? -1.0 : (r > 1.0 ? 1.0 : r);
  double c = largest ? 1.0 : -1.0;
  for (int it = 0; it < 100; it ++)
  {
    const double f = (4.0*c*c - 3.0)*c - r;
    const double cn = c - f/(12.0*c*c - 3.0);
    if (largest ? !(cn < c) : !(cn > c)) break;
    c = cn;
  }
  return c;
}

/* extremum_eigenvalue macros.h:1539-1588; the diagonal branch returns the
 * maximum whichever is asked for (reference behaviour) */
inline double extremum_eigenvalue(const double *A, int minimum)
{
  double p1 = A[3]*A[3] + A[6]*A[6] + A[7]*A[7];
  if (p1 == 0.0)
  {
    double r = A[0] > A[4] ? A[0] : A[4];
    return r > A[8] ? r : A[8];
  }
  double q = (A[0]+A[4]+A[8])/3.0;
  double p2 = (A[0]-q)*(A[0]-q) + (A[4]-q)*(A[4]-q) + (A[8]-q)*(A[8]-q) + 2*p1;
  double p = std::sqrt(p2 / 6.0);
  double invp = 1.0 / p;
  double B[9] = {invp*(A[0]-q), invp*A[1], invp*A[2], invp*A[3], invp*(A[4]-q), invp*A[5],
                 invp*A[6], invp*A[7], invp*(A[8]-q)};
  double r = 0.5 * DET(B);
  return q + 2.0 * p * triple_angle_root(r, !minimum);
}

/* NTMUL macros.h:932 */
inline void NTMUL(const double *A, const double *B, double *C)
{
  C[0] = A[0]*B[0]+A[3]*B[3]+A[6]*B[6];
  C[1] = A[1]*B[0]+A[4]*B[3]+A[7]*B[6];
  C[2] = A[2]*B[0]+A[5]*B[3]+A[8]*B[6];
  C[3] = A[0]*B[1]+A[3]*B[4]+A[6]*B[7];
  C[4] = A[1]*B[1]+A[4]*B[4]+A[7]*B[7];
  C[5] = A[2]*B[1]+A[5]*B[4]+A[8]*B[7];
  C[6] = A[0]*B[2]+A[3]*B[5]+A[6]*B[8];
  C[7] = A[1]*B[2]+A[4]*B[5]+A[7]*B[8];
  C[8] = A[2]*B[2]+A[5]*B[5]+A[8]*B[8];
}

/* time_step_task (parmec.ispc:275-383) for one particle.  Position taken: a
 * particle without rotational stiffness (omega_rot = 0, e.g. springs at the
 * mass centre) takes its translational step; the reference divides by zero
 * there and the NaN drops the particle from adaptive_timestep's minimum. */
inline double critical_step(const double kact[3], double kmax, double emax, const double krot[6], double mass,
                            const double J[9], double *omega, double *ratio)
{
  const double nxy = kact[0] > kact[1] ? kact[0] : kact[1];
  const double nxyz = nxy > kact[2] ? nxy : kact[2];
  if (!(nxyz > 0.0)) { *omega = 0.0; *ratio = 0.0; return 1.7976931348623157e308; }
  const double k = kmax;
  const double omegaxyz = std::sqrt(nxyz*k/mass);
  double K[9];
  K[0] = k*krot[0]; K[1] = k*krot[3]; K[2] = k*krot[4];
  K[3] = K[1]; K[4] = k*krot[1]; K[5] = k*krot[5];
  K[6] = K[2]; K[7] = K[5]; K[8] = k*krot[2];
  const double mrot = extremum_eigenvalue(J, 1);
  double L[9], invL[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, tmp[9], A[9], inv;
  L[0] = std::sqrt(J[0]);
  inv = 1.0/L[0];
  L[1] = inv * J[1];
  L[2] = inv * J[2];
  L[3] = 0.0;
  L[4] = std::sqrt(J[4] - L[1]*L[1]);
  inv = 1.0/L[4];
  L[5] = inv * (J[5] - L[2]*L[1]);
  L[6] = 0.0;
  L[7] = 0.0;
  L[8] = std::sqrt(J[8] - (L[2]*L[2] + L[5]*L[5]));
  INVERT(L, invL);
  NTMUL(K, invL, tmp);
  NNMUL(invL, tmp, A);
  const double lambda = extremum_eigenvalue(A, 0);
  const double omegarot = lambda > 0.0 ? std::sqrt(lambda) : 0.0;
  const double damping = emax;
  const double ratioxyz = damping / (2.0*mass*omegaxyz);
  const double hxyz = (2.0/omegaxyz)*(std::sqrt(1.0+ratioxyz*ratioxyz) - ratioxyz);
  double ratiorot = 0.0, hrot = 1.7976931348623157e308;
  if (omegarot > 0.0)
  {
    ratiorot = damping / (2.0*mrot*omegarot);
    hrot = (2.0/omegarot)*(std::sqrt(1.0+ratiorot*ratiorot) - ratiorot);
  }
  *omega = omegaxyz > omegarot ? omegaxyz : omegarot;
  *ratio = ratioxyz > ratiorot ? ratioxyz : ratiorot;
  return hxyz < hrot ? hxyz : hrot;
}

/* krot terms of one body-frame arm A (forces.ispc:514-522, 1262-1268) */
inline void krot_add(double *krot, const double *A)
{
  const double dt = DOT(A, A);
  krot[0] += dt - A[0]*A[0];
  krot[1] += dt - A[1]*A[1];
  krot[2] += dt - A[2]*A[2];
  krot[3] += -A[0]*A[1];
  krot[4] += -A[0]*A[2];
  krot[5] += -A[1]*A[2];
}

/* ---------------- contact records (condet.h:33-64 restated) --------------- */

struct Con
{
  int master;        /* master ellipsoid */
  int slave0;        /* slave particle, or the triangle's triobs code */
  int slave1;        /* slave ellipsoid, or -(triangle+1) */
  int color0, color1;
  double point[3], normal[3], depth;
  double force[3], kcur, ecur;
  double state[3];
};

struct SlaveCon
{
  int mpart, mell;
  double point[3], force[3];
  double kcur, ecur;   /* the contact's own (the reference's slave copy leaves them unset, forces.ispc:383-405) */
};

/* canonical order of a master list: sphere partners by ellipsoid index, then triangles */
inline int64_t con_key(int slave1)
{
  return slave1 >= 0 ? (int64_t)slave1 : ((int64_t)1 << 40) + (int64_t)(-slave1 - 1);
}

} /* namespace */

struct or_ctx
{
  std::vector<std::vector<Con>> master;      /* per particle */
  std::vector<std::vector<SlaveCon>> slave;  /* per particle */
  int threads = 1;
  /* adaptive stepping terms per particle, component-major:
   * kact[3][P], krot[6][P], kmax[P], emax[P] (forces.ispc:453-596) */
  std::vector<double> kact, krot, kmax, emax;
  /* mesh-mesh contact: swept radius (0: off), big-triangle flags, and the
   * previous step's pairs (offsets per finder, partners, active, state) */
  double tt_r = 0.0;
  std::vector<unsigned char> tt_big;
  std::vector<int> tt_poff, tt_ppu;
  std::vector<unsigned char> tt_pact;
  std::vector<double> tt_pst;
};

namespace {

/* ---------------- dynamics.ispc:30-169 ------------------------------------ */
void dynamics_one(pg_scene *s, int i, const double damping[6], double step0, double step1, bool typo)
{
  double half = 0.5*step0;
  double step = 0.5*(step0+step1);
  double O[3], o[3], v[3], L1[9], J[9], I[9], ma, im, f[3], t[3], T[3], DL[9], L2[9], A[3], B[3];

  if (s->flags[i] & PG_FLAG_SKIP) return;

  for (int k = 0; k < 3; k ++) O[k] = s->angular[k][i];
  for (int k = 0; k < 3; k ++) v[k] = s->linear[k][i];
  for (int k = 0; k < 9; k ++) L1[k] = s->rotation[k][i];
  for (int k = 0; k < 9; k ++) J[k] = s->inertia[k][i];
  for (int k = 0; k < 9; k ++) I[k] = s->inverse[k][i];
  im = s->invm[i];

  if (damping[0] != 0.0 || damping[1] != 0.0 || damping[2] != 0.0)
  {
    ma = s->mass[i];
    s->force[0][i] -= ma * damping[0] * v[0];
    s->force[1][i] -= ma * damping[1] * v[1];
    s->force[2][i] -= ma * damping[2] * v[2];
  }
  if (damping[3] != 0.0 || damping[4] != 0.0 || damping[5] != 0.0)
  {
    o[0] = damping[3]*s->angular[3][i];
    o[1] = damping[4]*s->angular[4][i];
    o[2] = damping[5]*s->angular[5][i];
    TVMUL(L1, o, t);
    NVMUL(J, t, T);
    NVMUL(L1, T, t);
    s->torque[0][i] -= t[0];
    s->torque[1][i] -= t[1];
    s->torque[2][i] -= t[2];
  }

  for (int k = 0; k < 3; k ++) f[k] = s->force[k][i];
  for (int k = 0; k < 3; k ++) t[k] = s->torque[k][i];

  TVMUL(L1, t, T);
  expmap(-half*O[0], -half*O[1], -half*O[2], DL, typo);
  NVMUL(J, O, A);
  NVMUL(DL, A, B);
  /* ADDMUL (B, half, T, B) */
  B[0] = B[0] + half*T[0];
  B[1] = B[1] + half*T[1];
  B[2] = B[2] + half*T[2];
  NVMUL(I, B, A);              /* O(t+h/2) */
  NVMUL(J, A, B);
  /* PRODUCTSUB (A, B, T) */
  T[0] -= A[1]*B[2] - A[2]*B[1];
  T[1] -= A[2]*B[0] - A[0]*B[2];
  T[2] -= A[0]*B[1] - A[1]*B[0];
  /* SCALE (T, step0) */
  T[0] *= step0; T[1] *= step0; T[2] *= step0;
  NVADDMUL(O, I, T, O);        /* O(t+h) */
  im *= step0;
  v[0] = v[0] + im*f[0];
  v[1] = v[1] + im*f[1];
  v[2] = v[2] + im*f[2];
  expmap(step*O[0], step*O[1], step*O[2], DL, typo);
  NNMUL(L1, DL, L2);
  for (int k = 0; k < 9; k ++) s->rotation[k][i] = L2[k];
  NVMUL(L2, O, o);
  s->position[0][i] += step*v[0];
  s->position[1][i] += step*v[1];
  s->position[2][i] += step*v[2];
  s->angular[0][i] = O[0];
  s->angular[1][i] = O[1];
  s->angular[2][i] = O[2];
  s->angular[3][i] = o[0];
  s->angular[4][i] = o[1];
  s->angular[5][i] = o[2];
  s->linear[0][i] = v[0];
  s->linear[1][i] = v[1];
  s->linear[2][i] = v[2];
}

/* ---------------- parmec.ispc:224-272 euler_task -------------------------- */
void euler_one(pg_scene *s, int i, double step, bool typo)
{
  double O[3], L1[9], DL[9], L2[9], o[3];
  O[0] = step*s->angular[0][i];
  O[1] = step*s->angular[1][i];
  O[2] = step*s->angular[2][i];
  expmap(O[0], O[1], O[2], DL, typo);
  for (int k = 0; k < 9; k ++) L1[k] = s->rotation[k][i];
  NNMUL(L1, DL, L2);
  for (int k = 0; k < 9; k ++) s->rotation[k][i] = L2[k];
  NVMUL(L2, O, o);
  s->angular[3][i] = o[0];
  s->angular[4][i] = o[1];
  s->angular[5][i] = o[2];
  s->position[0][i] += step * s->linear[0][i];
  s->position[1][i] += step * s->linear[1][i];
  s->position[2][i] += step * s->linear[2][i];
}

/* ---------------- shapes.ispc:29-211 -------------------------------------- */
void ellipsoid_one(pg_scene *s, int i)
{
  double L[9], X[3], x[3], C[3], c[3];
  int j = s->part[i];
  for (int k = 0; k < 9; k ++) L[k] = s->rotation[k][j];
  X[0] = s->position[3][j]; X[1] = s->position[4][j]; X[2] = s->position[5][j];
  x[0] = s->position[0][j]; x[1] = s->position[1][j]; x[2] = s->position[2][j];
  C[0] = s->center[3][i]; C[1] = s->center[4][i]; C[2] = s->center[5][i];
  /* SCC (X, C) */
  C[0] -= X[0]; C[1] -= X[1]; C[2] -= X[2];
  NVADDMUL(x, L, C, c);
  s->center[0][i] = c[0];
  s->center[1][i] = c[1];
  s->center[2][i] = c[2];
}

void node_one(pg_scene *s, int i, bool skip_analytical)
{
  double L[9], X[3], x[3], C[3], c[3];
  int j = s->nodpart[i];
  if (skip_analytical && (s->flags[j] & PG_FLAG_ANALYTICAL)) return;
  for (int k = 0; k < 9; k ++) L[k] = s->rotation[k][j];
  X[0] = s->position[3][j]; X[1] = s->position[4][j]; X[2] = s->position[5][j];
  x[0] = s->position[0][j]; x[1] = s->position[1][j]; x[2] = s->position[2][j];
  C[0] = s->nodes[3][i]; C[1] = s->nodes[4][i]; C[2] = s->nodes[5][i];
  C[0] -= X[0]; C[1] -= X[1]; C[2] -= X[2];
  NVADDMUL(x, L, C, c);
  s->nodes[0][i] = c[0];
  s->nodes[1][i] = c[1];
  s->nodes[2][i] = c[2];
}

void face_one(pg_scene *s, int i)
{
  int j = s->factri[i];
  int k[3] = {s->facnod[0][i], s->facnod[1][i], s->facnod[2][i]};
  for (int v = 0; v < 3; v ++)
    for (int d = 0; d < 3; d ++)
      s->tri[v][d][j] = s->nodes[d][k[v]];
}

void shapes_all(or_ctx *ctx, pg_scene *s, bool skip_analytical)
{
  const int E = s->ellnum, N = s->nodnum, F = s->facnum;
#pragma omp parallel for schedule(static) num_threads(ctx->threads)
  for (int i = 0; i < E; i ++) ellipsoid_one(s, i);
#pragma omp parallel for schedule(static) num_threads(ctx->threads)
  for (int i = 0; i < N; i ++) node_one(s, i, skip_analytical);
#pragma omp parallel for schedule(static) num_threads(ctx->threads)
  for (int i = 0; i < F; i ++) face_one(s, i);
}

/* ---------------- obstacles.ispc:28-78 ------------------------------------ */
void obstacles_all(pg_scene *s, const double *obsang, const double *obslin, double step, bool typo)
{
  double DL[9], y[3];
  for (int i = 0; i < s->obsnum; i ++)
  {
    double *x = s->obspnt + 3*i;
    const double *o = obsang + 3*i;  /* the reference walks these with stride 6 (obstacles.ispc:37),
                                        the values are written with stride 3 (input.cpp:4206);
                                        stride 3 is used here */
    const double *v = obslin + 3*i;
    y[0] = x[0] + step*v[0];
    y[1] = x[1] + step*v[1];
    y[2] = x[2] + step*v[2];
    expmap(step*o[0], step*o[1], step*o[2], DL, typo);
    for (int j = s->trirng[2*i]; j < s->trirng[2*i+1]; j ++)
    {
      double z[3];
      for (int vtx = 0; vtx < 3; vtx ++)
      {
        z[0] = s->tri[vtx][0][j] - x[0];
        z[1] = s->tri[vtx][1][j] - x[1];
        z[2] = s->tri[vtx][2][j] - x[2];
        s->tri[vtx][0][j] = DL[0]*z[0]+DL[3]*z[1]+DL[6]*z[2] + y[0];
        s->tri[vtx][1][j] = DL[1]*z[0]+DL[4]*z[1]+DL[7]*z[2] + y[1];
        s->tri[vtx][2][j] = DL[2]*z[0]+DL[5]*z[1]+DL[8]*z[2] + y[2];
      }
    }
    x[0] = y[0];
    x[1] = y[1];
    x[2] = y[2];
  }
}

/* ---------------- condet.ispc:294-400 (and 519-624) ----------------------- */
inline double clampf(double a, double b, double c) { return a < b ? b : a > c ? c : a; }

double triangle_sphere(double ax, double ay, double az, double bx, double by, double bz,
                       double cx, double cy, double cz, double px, double py, double pz, double r,
                       double point[3], double normal[3], bool edge_typo)
{
  double edge0[3] = {bx-ax, by-ay, bz-az};
  double edge1[3] = {cx-ax, cy-ay, cz-az};
  double v0[3] = {ax-px, ay-py, az-pz};
  double a = DOT(edge0, edge0);
  double b = DOT(edge0, edge1);
  double c = DOT(edge1, edge1);
  double d = DOT(edge0, v0);
  double e = DOT(edge1, v0);
  double det = a*c - b*b;
  double s = b*e - c*d;
  double t = b*d - a*e;

  if (s + t < det)
  {
    if (s < 0.f)
    {
      if (t < 0.f)
      {
        if (d < 0.f) { s = clampf(-d/a, 0.f, 1.f); t = 0.f; }
        else { s = 0.f; t = clampf(-e/c, 0.f, 1.f); }
      }
      else { s = 0.f; t = clampf(-e/c, 0.f, 1.f); }
    }
    else if (t < 0.f) { s = clampf(-d/a, 0.f, 1.f); t = 0.f; }
    else
    {
      double invDet = 1.f / det;
      s *= invDet;
      t *= invDet;
    }
  }
  else
  {
    if (s < 0.f)
    {
      double tmp0 = b+d;
      double tmp1 = c+e;
      if (tmp1 > tmp0)
      {
        double numer = tmp1 - tmp0;
        double denom = a-2*b+c;
        s = clampf(numer/denom, 0.f, 1.f);
        t = 1-s;
      }
      else { t = clampf(-e/c, 0.f, 1.f); s = 0.f; }
    }
    else if (t < 0.f)
    {
      if (a+d > b+e)
      {
        double numer = c+e-b-d;
        double denom = a-2*b+c;
        s = clampf(numer/denom, 0.f, 1.f);
        t = 1-s;
      }
      else
      {
        /* the reference takes -e/c here (condet.ispc:373); -d/a is the ab edge */
        s = edge_typo ? clampf(-e/c, 0.f, 1.f) : clampf(-d/a, 0.f, 1.f);
        t = 0.f;
      }
    }
    else
    {
      double numer = c+e-b-d;
      double denom = a-2*b+c;
      s = clampf(numer/denom, 0.f, 1.f);
      t = 1.f - s;
    }
  }

  point[0] = ax + s*edge0[0] + t*edge1[0];
  point[1] = ay + s*edge0[1] + t*edge1[1];
  point[2] = az + s*edge0[2] + t*edge1[2];
  double q[3] = {px-point[0], py-point[1], pz-point[2]};
  double len = LEN(q);
  double ilen = 1.0/len;
  normal[0] = ilen*q[0];
  normal[1] = ilen*q[1];
  normal[2] = ilen*q[2];
  return r - len;
}

/* sphere-sphere geometry, master perspective (condet.ispc:126-145 new, 654-676 existing) */
double sphere_sphere(const pg_scene *s, int i, int j, bool existing, double point[3], double normal[3])
{
  double p[3], q[3], c[3], len, ilen;
  p[0] = s->center[0][i]; p[1] = s->center[1][i]; p[2] = s->center[2][i];
  c[0] = s->center[0][j]; c[1] = s->center[1][j]; c[2] = s->center[2][j];
  q[0] = p[0]-c[0];
  q[1] = p[1]-c[1];
  q[2] = p[2]-c[2];
  len = LEN(q);
  if (existing) ilen = 1.0/len;
  else ilen = len > 0.0 ? 1.0/len : 1.0;
  point[0] = 0.5*(p[0]+c[0]);
  point[1] = 0.5*(p[1]+c[1]);
  point[2] = 0.5*(p[2]+c[2]);
  normal[0] = ilen*q[0];
  normal[1] = ilen*q[1];
  normal[2] = ilen*q[2];
  return s->radii[0][i]+s->radii[0][j] - len;
}

/* ---------------- exact neighbour search (accelerator for the exact set) -- */
struct Grid
{
  double org[3], h;
  int64_t dim[3];
  std::vector<int64_t> keys;   /* sorted cell keys */
  std::vector<int> items;      /* item index in key order */

  int64_t cell_of(const double *p, int64_t c[3]) const
  {
    for (int k = 0; k < 3; k ++)
    {
      double u = std::floor((p[k] - org[k]) / h);
      if (u < 0) u = 0;
      if (u > (double)(dim[k]-1)) u = (double)(dim[k]-1);
      c[k] = (int64_t)u;
    }
    return (c[2]*dim[1] + c[1])*dim[0] + c[0];
  }

  void range(int64_t key, int &b, int &e) const
  {
    b = (int)(std::lower_bound(keys.begin(), keys.end(), key) - keys.begin());
    e = (int)(std::upper_bound(keys.begin(), keys.end(), key) - keys.begin());
  }
};

void build_sphere_grid(const pg_scene *s, double h, Grid &g)
{
  const int E = s->ellnum;
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int i = 0; i < E; i ++)
    for (int k = 0; k < 3; k ++)
    {
      lo[k] = std::min(lo[k], s->center[k][i]);
      hi[k] = std::max(hi[k], s->center[k][i]);
    }
  g.h = h;
  for (int k = 0; k < 3; k ++)
  {
    g.org[k] = lo[k];
    double n = std::floor((hi[k] - lo[k]) / h) + 1;
    if (n > 1e6) n = 1e6; /* clamped cells stay adjacent-preserving */
    g.dim[k] = (int64_t)n;
  }
  std::vector<std::pair<int64_t,int>> kv(E);
  for (int i = 0; i < E; i ++)
  {
    int64_t c[3];
    double p[3] = {s->center[0][i], s->center[1][i], s->center[2][i]};
    kv[i] = std::make_pair(g.cell_of(p, c), i);
  }
  std::sort(kv.begin(), kv.end());
  g.keys.resize(E);
  g.items.resize(E);
  for (int i = 0; i < E; i ++) { g.keys[i] = kv[i].first; g.items[i] = kv[i].second; }
}

/* ---------------- condet (condet.ispc:627-797) ---------------------------- */
void condet(or_ctx *ctx, pg_scene *s)
{
  const int P = s->parnum, E = s->ellnum, T = s->trinum;

  /* update_existing (condet.ispc:627-700) */
#pragma omp parallel for schedule(dynamic, 64) num_threads(ctx->threads)
  for (int l = 0; l < P; l ++)
  {
    for (Con &con : ctx->master[l])
    {
      int i = con.master, j = con.slave1;
      if (s->radii[1][i] < 0.0)
      {
        if (j < 0)
        {
          int u = -j-1;
          con.depth = triangle_sphere(s->tri[0][0][u], s->tri[0][1][u], s->tri[0][2][u],
                                      s->tri[1][0][u], s->tri[1][1][u], s->tri[1][2][u],
                                      s->tri[2][0][u], s->tri[2][1][u], s->tri[2][2][u],
                                      s->center[0][i], s->center[1][i], s->center[2][i],
                                      s->radii[0][i], con.point, con.normal, (s->compat & PG_COMPAT_TRIEDGE) != 0);
        }
        else if (s->radii[1][j] < 0.0)
        {
          con.depth = sphere_sphere(s, i, j, true, con.point, con.normal);
        }
        else std::abort(); /* ellipsoids: assert(0) in the reference */
      }
      else std::abort();
    }
  }

  if (E == 0) return; /* tree == NULL (condet.ispc:786) */

  double rmax = 0.0;
  for (int i = 0; i < E; i ++) rmax = std::max(rmax, s->radii[0][i]);
  Grid g;
  build_sphere_grid(s, 2.0*rmax > 0.0 ? 2.0*rmax : 1.0, g);

  /* triangles binned into the sphere grid cells their AABB (+rmax) touches */
  std::vector<std::pair<int64_t,int>> tkv;
  for (int t = 0; t < T; t ++)
  {
    double lo[3], hi[3];
    for (int k = 0; k < 3; k ++)
    {
      lo[k] = std::min(std::min(s->tri[0][k][t], s->tri[1][k][t]), s->tri[2][k][t]) - rmax;
      hi[k] = std::max(std::max(s->tri[0][k][t], s->tri[1][k][t]), s->tri[2][k][t]) + rmax;
    }
    int64_t a[3], b[3];
    g.cell_of(lo, a);
    g.cell_of(hi, b);
    for (int64_t z = a[2]; z <= b[2]; z ++)
      for (int64_t y = a[1]; y <= b[1]; y ++)
        for (int64_t x = a[0]; x <= b[0]; x ++)
          tkv.push_back(std::make_pair((z*g.dim[1] + y)*g.dim[0] + x, t));
  }
  std::sort(tkv.begin(), tkv.end());
  std::vector<int64_t> tkeys(tkv.size());
  for (size_t k = 0; k < tkv.size(); k ++) tkeys[k] = tkv[k].first;

  /* new sphere-sphere (condet.ispc:98-290) and sphere-triangle (412-516)
   * contacts, gathered per master sphere so that lists stay private */
#pragma omp parallel for schedule(dynamic, 64) num_threads(ctx->threads)
  for (int i = 0; i < E; i ++)
  {
    int pi = s->part[i];
    std::vector<Con> &ml = ctx->master[pi];
    std::vector<Con> fresh;
    double p[3] = {s->center[0][i], s->center[1][i], s->center[2][i]};
    int64_t c[3];
    g.cell_of(p, c);
    for (int64_t dz = -1; dz <= 1; dz ++)
      for (int64_t dy = -1; dy <= 1; dy ++)
        for (int64_t dx = -1; dx <= 1; dx ++)
        {
          int64_t x = c[0]+dx, y = c[1]+dy, z = c[2]+dz;
          if (x < 0 || y < 0 || z < 0 || x >= g.dim[0] || y >= g.dim[1] || z >= g.dim[2]) continue;
          int b, e;
          g.range((z*g.dim[1] + y)*g.dim[0] + x, b, e);
          for (int k = b; k < e; k ++)
          {
            int j = g.items[k];
            int pj = s->part[j];
            if (pj <= pi) continue;              /* master = smaller particle index */
            if (s->radii[1][j] >= 0.0) std::abort();
            Con con;
            con.depth = sphere_sphere(s, i, j, false, con.point, con.normal);
            if (!(con.depth > 0.0)) continue;
            bool found = false;
            for (const Con &m : ml) if (m.master == i && m.slave0 == pj && m.slave1 == j) { found = true; break; }
            if (found) continue;
            con.master = i; con.slave0 = pj; con.slave1 = j;
            con.color0 = s->ellcol[i]; con.color1 = s->ellcol[j];
            con.force[0] = con.force[1] = con.force[2] = 0.0;
            con.kcur = con.ecur = 0.0;
            con.state[0] = con.state[1] = con.state[2] = 0.0;
            fresh.push_back(con);
          }
        }
    if (T > 0)
    {
      int64_t key = (c[2]*g.dim[1] + c[1])*g.dim[0] + c[0];
      size_t b = std::lower_bound(tkeys.begin(), tkeys.end(), key) - tkeys.begin();
      size_t e = std::upper_bound(tkeys.begin(), tkeys.end(), key) - tkeys.begin();
      for (size_t k = b; k < e; k ++)
      {
        int t = tkv[k].second;
        Con con;
        con.depth = triangle_sphere(s->tri[0][0][t], s->tri[0][1][t], s->tri[0][2][t],
                                    s->tri[1][0][t], s->tri[1][1][t], s->tri[1][2][t],
                                    s->tri[2][0][t], s->tri[2][1][t], s->tri[2][2][t],
                                    p[0], p[1], p[2], s->radii[0][i], con.point, con.normal,
                                    (s->compat & PG_COMPAT_TRIEDGE) != 0);
        if (!(con.depth > 0.0)) continue;
        bool found = false;
        for (const Con &m : ml) if (m.master == i && m.slave1 == -(t+1)) { found = true; break; }
        if (found) continue;
        con.master = i; con.slave0 = s->triobs[t]; con.slave1 = -(t+1);
        con.color0 = s->ellcol[i]; con.color1 = s->tricol[t];
        con.force[0] = con.force[1] = con.force[2] = 0.0;
        con.kcur = con.ecur = 0.0;
        con.state[0] = con.state[1] = con.state[2] = 0.0;
        fresh.push_back(con);
      }
    }
    if (!fresh.empty())
    {
      for (Con &f : fresh) ml.push_back(f);
      std::stable_sort(ml.begin(), ml.end(), [](const Con &a, const Con &b) {
        if (a.master != b.master) return a.master < b.master;
        return con_key(a.slave1) < con_key(b.slave1); });
    }
  }
}

/* ---------------- forces.ispc:98-122 pairing ------------------------------ */
int pairing(int nummat, const int *pairs, int i, int j)
{
  int p0 = i, p1 = j, start = 1, end = nummat;
  if (i > j) { p0 = j; p1 = i; }
  while (start < end)
  {
    int mid = ((end-start)>>1) + start;
    if (p0 > pairs[2*mid]) { if (start == mid) break; start = mid; }
    else if (p0 == pairs[2*mid])
    {
      if (p1 > pairs[2*mid+1]) { if (start == mid) break; start = mid; }
      else if (p1 == pairs[2*mid+1]) return mid;
      else end = mid;
    }
    else end = mid;
  }
  return 0;
}

/* ---------------- forces.ispc:125-192 granural_force ---------------------- */
int granular_force(const pg_scene *s, const double n[3], const double vij[3], double depth,
                   int i, int j, int ij, double state[3], double step, double f[5])
{
  double ma;
  if (j >= 0) ma = 1.0 / (s->invm[i] + s->invm[j]);
  else ma = s->mass[i];

  double kn = s->iparam[SPRING][ij];
  double en = s->iparam[DAMPER][ij] * 2.0 * std::sqrt(kn*ma);
  double vn = DOT(vij, n);
  double fn = kn*depth + en*vn;

  f[0] = fn*n[0];
  f[1] = fn*n[1];
  f[2] = fn*n[2];
  f[3] = kn;
  f[4] = en;

  double kt = kn * s->iparam[KSKN][ij];
  double et = en * s->iparam[KSKN][ij];
  double mus = s->iparam[FRISTAT][ij];
  double mud = s->iparam[FRIDYN][ij];
  double vt[3], ft[3];

  vt[0] = vij[0] - vn*n[0];
  vt[1] = vij[1] - vn*n[1];
  vt[2] = vij[2] - vn*n[2];

  state[0] += step*vt[0];
  state[1] += step*vt[1];
  state[2] += step*vt[2];

  ft[0] = kt*state[0] + et*vt[0];
  ft[1] = kt*state[1] + et*vt[1];
  ft[2] = kt*state[2] + et*vt[2];

  double len = LEN(ft);
  double lim = mus*fn;
  if (len > lim)
  {
    lim = mud*fn/len;
    ft[0] *= lim;
    ft[1] *= lim;
    ft[2] *= lim;
  }
  f[0] += ft[0];
  f[1] += ft[1];
  f[2] += ft[2];

  return depth < 0.0 ? 1 : 0;
}

/* ---------------- forces.ispc:195-407 contacts_task (one particle) -------- */
void contacts_one(pg_scene *s, std::vector<Con> &ml, int i, const double *obsang, const double *obslin,
                  double step, bool obsidx_compat)
{
  double oi[3], v[3], x[3];
  oi[0] = s->angular[3][i]; oi[1] = s->angular[4][i]; oi[2] = s->angular[5][i];
  v[0] = s->linear[0][i]; v[1] = s->linear[1][i]; v[2] = s->linear[2][i];
  x[0] = s->position[0][i]; x[1] = s->position[1][i]; x[2] = s->position[2][i];

  size_t keep = 0;
  for (size_t k = 0; k < ml.size(); k ++)
  {
    Con &con = ml[k];
    double p[3], n[3], z[3], vi[3], vj[3], oj[3], vij[3];
    for (int d = 0; d < 3; d ++) { p[d] = con.point[d]; n[d] = con.normal[d]; }
    z[0] = p[0]-x[0]; z[1] = p[1]-x[1]; z[2] = p[2]-x[2];
    vi[0] = oi[1]*z[2]-oi[2]*z[1] + v[0];
    vi[1] = oi[2]*z[0]-oi[0]*z[2] + v[1];
    vi[2] = oi[0]*z[1]-oi[1]*z[0] + v[2];

    int j = con.slave0;
    if (j >= 0)
    {
      z[0] = p[0]-s->position[0][j];
      z[1] = p[1]-s->position[1][j];
      z[2] = p[2]-s->position[2][j];
      oj[0] = s->angular[3][j]; oj[1] = s->angular[4][j]; oj[2] = s->angular[5][j];
      vj[0] = oj[1]*z[2]-oj[2]*z[1] + s->linear[0][j];
      vj[1] = oj[2]*z[0]-oj[0]*z[2] + s->linear[1][j];
      vj[2] = oj[0]*z[1]-oj[1]*z[0] + s->linear[2][j];
    }
    else
    {
      int l = -j-2;
      if (obsidx_compat && l >= 0) l = l+1;
      if (l >= 0 && l < s->obsnum)
      {
        z[0] = p[0]-s->obspnt[3*l];
        z[1] = p[1]-s->obspnt[3*l+1];
        z[2] = p[2]-s->obspnt[3*l+2];
        oj[0] = obsang[3*l]; oj[1] = obsang[3*l+1]; oj[2] = obsang[3*l+2];
        vj[0] = oj[1]*z[2]-oj[2]*z[1] + obslin[3*l];
        vj[1] = oj[2]*z[0]-oj[0]*z[2] + obslin[3*l+1];
        vj[2] = oj[0]*z[1]-oj[1]*z[0] + obslin[3*l+2];
      }
      else
      {
        /* static boundary; with the index defect a missing obstacle k+1 reads
         * zero-initialised buffers, i.e. a static wall as well */
        oj[0] = oj[1] = oj[2] = 0.0;
        vj[0] = vj[1] = vj[2] = 0.0;
      }
    }
    vij[0] = vj[0] - vi[0];
    vij[1] = vj[1] - vi[1];
    vij[2] = vj[2] - vi[2];

    int ij = pairing(s->pairnum, s->pairs, con.color0, con.color1);
    if (s->ikind[ij] != 0) std::abort(); /* USER_FORCE: assert(0) */
    double f[5];
    int gone = granular_force(s, n, vij, con.depth, i, j, ij, con.state, step, f);
    con.force[0] = f[0]; con.force[1] = f[1]; con.force[2] = f[2];
    con.kcur = f[3]; con.ecur = f[4];
    if (!gone)
    {
      if (keep != k) ml[keep] = con;
      keep ++;
    }
  }
  ml.resize(keep);
}

/* ---------------- forces.ispc:453-596 contacts_acc_task (one particle) ----
 * With 'ad' (adaptive stepping) also the stiffness terms: |normal| (master) or
 * |force direction| (slave) into kact, the contact stiffness and damping into
 * kmax/emax, and the arm terms of L*a into krot, master list first. */
struct AdTerms { double *kact[3], *krot[6], *kmax, *emax; };

void contacts_acc_one(pg_scene *s, const std::vector<Con> &ml, const std::vector<SlaveCon> &sl,
                      int i, const double gravity[3], const AdTerms *ad)
{
  double fs[3] = {0.0, 0.0, 0.0}, ts[3] = {0.0, 0.0, 0.0};
  double po[3] = {s->position[0][i], s->position[1][i], s->position[2][i]};
  double ma = s->mass[i];
  double kact0[3] = {0.0, 0.0, 0.0}, krot0[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, kmax0 = 0.0, emax0 = 0.0;
  double L[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (ad) for (int k = 0; k < 9; k ++) L[k] = s->rotation[k][i];
  for (const Con &m : ml)
  {
    const double *f = m.force;
    double a[3] = {m.point[0]-po[0], m.point[1]-po[1], m.point[2]-po[2]};
    fs[0] += f[0]; fs[1] += f[1]; fs[2] += f[2];
    ts[0] += a[1]*f[2] - a[2]*f[1];
    ts[1] += a[2]*f[0] - a[0]*f[2];
    ts[2] += a[0]*f[1] - a[1]*f[0];
    if (ad)
    {
      kact0[0] += std::fabs(m.normal[0]);
      kact0[1] += std::fabs(m.normal[1]);
      kact0[2] += std::fabs(m.normal[2]);
      kmax0 = m.kcur > kmax0 ? m.kcur : kmax0;
      emax0 = m.ecur > emax0 ? m.ecur : emax0;
      double A[3];
      NVMUL(L, a, A);
      krot_add(krot0, A);
    }
  }
  for (const SlaveCon &m : sl)
  {
    const double *f = m.force;
    double a[3] = {m.point[0]-po[0], m.point[1]-po[1], m.point[2]-po[2]};
    fs[0] += f[0]; fs[1] += f[1]; fs[2] += f[2];
    ts[0] += a[1]*f[2] - a[2]*f[1];
    ts[1] += a[2]*f[0] - a[0]*f[2];
    ts[2] += a[0]*f[1] - a[1]*f[0];
    if (ad)
    {
      double u[3] = {f[0], f[1], f[2]};
      double len = LEN(u);
      if (len != 0.0)
      {
        len = 1.0/len;
        u[0] *= len; u[1] *= len; u[2] *= len;
      }
      else u[0] = u[1] = u[2] = 0.0;
      kact0[0] += std::fabs(u[0]);
      kact0[1] += std::fabs(u[1]);
      kact0[2] += std::fabs(u[2]);
      kmax0 = m.kcur > kmax0 ? m.kcur : kmax0;
      emax0 = m.ecur > emax0 ? m.ecur : emax0;
      double A[3];
      NVMUL(L, a, A);
      krot_add(krot0, A);
    }
  }
  s->force[0][i] = fs[0] + ma * gravity[0];
  s->force[1][i] = fs[1] + ma * gravity[1];
  s->force[2][i] = fs[2] + ma * gravity[2];
  s->torque[0][i] = ts[0];
  s->torque[1][i] = ts[1];
  s->torque[2][i] = ts[2];
  if (ad)
  {
    for (int k = 0; k < 3; k ++) ad->kact[k][i] = kact0[k];
    for (int k = 0; k < 6; k ++) ad->krot[k][i] = krot0[k];
    ad->kmax[i] = kmax0;
    ad->emax[i] = emax0;
  }
}

/* ---------------- forces.ispc:410-450 look_up / look_up_slope ------------- */
double look_up(double *const tab[2], int lo, int hi, double arg, double *slope)
{
  int h0 = hi;
  while (hi > lo+1)
  {
    int mid = lo + (hi-lo)/2;
    if (arg > tab[0][mid]) lo = mid;
    else hi = mid;
  }
  if (lo+1 == h0) lo --;
  *slope = (tab[1][lo+1]-tab[1][lo])/(tab[0][lo+1]-tab[0][lo]);
  return tab[1][lo] + (*slope)*(arg-tab[0][lo]);
}

double look_up_slope(int i, double *const tab[2], int lo, int hi, double arg, double *at)
{
  int h0 = hi;
  while (hi > lo+1)
  {
    int mid = lo + (hi-lo)/2;
    if (arg > tab[i][mid]) lo = mid;
    else hi = mid;
  }
  if (lo+1 == h0) lo --;
  if (at)
  {
    int j = (i == 0 ? 1 : 0);
    at[0] = tab[j][lo] + (tab[j][lo+1]-tab[j][lo])*(arg-tab[i][lo])/(tab[i][lo+1]-tab[i][lo]);
  }
  return (tab[1][lo+1]-tab[1][lo])/(tab[0][lo+1]-tab[0][lo]);
}

/* ---------------- parmec.ispc:423-482 eqm --------------------------------- */
double eqm(const pg_scene *s, int part1, const double *point1, int part2, const double *point2,
           const double *direction)
{
  double Jiv[9], im, A[3], Ask[9], tmp[9], Miv[9], mass;
  for (int k = 0; k < 9; k ++) Jiv[k] = s->inverse[k][part1];
  im = s->invm[part1];
  A[0] = s->position[3][part1] - point1[0];
  A[1] = s->position[4][part1] - point1[1];
  A[2] = s->position[5][part1] - point1[2];
  VECSKEW(A, Ask);
  TNMUL(Ask, Jiv, tmp);
  NNMUL(tmp, Ask, Miv);
  Miv[0] += im; Miv[4] += im; Miv[8] += im;
  if (part2 >= 0)
  {
    for (int k = 0; k < 9; k ++) Jiv[k] = s->inverse[k][part2];
    im = s->invm[part2];
    A[0] = s->position[3][part2] - point2[0];
    A[1] = s->position[4][part2] - point2[1];
    A[2] = s->position[5][part2] - point2[2];
    VECSKEW(A, Ask);
    TNMUL(Ask, Jiv, tmp);
    NNMUL(tmp, Ask, Jiv);
    for (int k = 0; k < 9; k ++) Miv[k] = Miv[k] + Jiv[k]; /* NNADD */
    Miv[0] += im; Miv[4] += im; Miv[8] += im;
  }
  if (direction && DOT(direction, direction) > 0.0)
  {
    NVMUL(Miv, direction, tmp);
    mass = 1.0/DOT(tmp, direction);
  }
  else mass = 1.0/extremum_eigenvalue(Miv, 1);
  return mass;
}

/* ---------------- springs_task's force flushes (forces.ispc:1207-1412) -----
 * Springs are sorted by (part0, part1).  One task adds a run of springs with
 * equal part0 to that particle (+=) and a run with equal part1 to that one
 * (-=), each run summed in spring order, the first run of its kind starting
 * from zero and later ones from their first element.  A run longer than
 * SPRING_RUN_LONG springs is summed in three levels: chunks of springs in
 * spring order, groups of SPRING_RUN_GROUP chunk sums in order, then the
 * group sums in order, as tasks whose boundaries fall on the chunks would
 * flush their partials (the reference adds task partials under a lock, in an
 * order that depends on the tasks, forces.ispc:1272-1327); the GPU uses the
 * same definition.  Chunks hold 64 springs, doubled until there are at most
 * SPRING_RUN_MAXCHUNKS. */
static const int SPRING_RUN_LONG = 64;
static const int SPRING_RUN_MAXCHUNKS = 1024;
static const int SPRING_RUN_GROUP = 32;

static int spring_run_chunk(int len)
{
  int c = 64;
  while ((len + c - 1) / c > SPRING_RUN_MAXCHUNKS) c *= 2;
  return c;
}

struct SprRun { int part, type, b, e, first; long long pos; };

static void add6(double *acc, const double *x, bool assign)
{
  for (int c = 0; c < 6; c ++) acc[c] = assign ? x[c] : acc[c] + x[c];
}

// sum of one run: acc[0..2] force, acc[3..5] torque
static void spring_run_sum(const pg_scene *s, double *const out[9], const SprRun &r, double *acc)
{
  const int off = r.type == 0 ? 3 : 6;
  for (int c = 0; c < 6; c ++) acc[c] = 0.0;
  bool started = false;
  auto element = [&](int i, double *x) {
    x[0] = out[0][i]; x[1] = out[1][i]; x[2] = out[2][i];
    x[3] = out[off][i]; x[4] = out[off+1][i]; x[5] = out[off+2][i];
  };
  auto skipped = [&](int i) { return r.type == 1 && s->sprpart[1][i] < 0; };
  if (r.e - r.b <= SPRING_RUN_LONG)
  {
    for (int i = r.b; i < r.e; i ++)
    {
      if (skipped(i)) continue;
      double x[6];
      element(i, x);
      add6(acc, x, !started && !r.first);
      started = true;
    }
    return;
  }
  const int len = r.e - r.b, ch = spring_run_chunk(len), nc = (len + ch - 1) / ch;
  for (int g0 = 0; g0 < nc; g0 += SPRING_RUN_GROUP)
  {
    double gp[6] = {0, 0, 0, 0, 0, 0};
    bool gany = false;
    for (int c = g0; c < std::min(g0 + SPRING_RUN_GROUP, nc); c ++)
    {
      const int b = r.b + c * ch;
      double part[6] = {0, 0, 0, 0, 0, 0};
      bool any = false;
      for (int i = b; i < std::min(b + ch, r.e); i ++)
      {
        if (skipped(i)) continue;
        double x[6];
        element(i, x);
        add6(part, x, !any);
        any = true;
      }
      if (!any) continue;
      add6(gp, part, !gany);
      gany = true;
    }
    if (!gany) continue;
    add6(acc, gp, !started && !r.first);
    started = true;
  }
}

/* adaptive stepping terms of one run (forces.ispc:1248-1345): per spring
 * |z| (3), |stiffness|, |damping|, then the krot terms of the j arm (6) and
 * of the k arm (6), zero where the spring's total force is zero; the run's
 * partial sums start from zero (long runs chunked as above), its stiffness
 * and damping partials are maxima. */
static void spring_run_adaptive(const pg_scene *s, double *const ad[17], const SprRun &r, double *p, double *km,
                                double *em)
{
  const int off = r.type == 0 ? 5 : 11;
  for (int c = 0; c < 9; c ++) p[c] = 0.0;
  *km = 0.0; *em = 0.0;
  auto skipped = [&](int i) { return r.type == 1 && s->sprpart[1][i] < 0; };
  auto add = [&](int i, double *q, double *qk, double *qe) {
    for (int c = 0; c < 3; c ++) q[c] = q[c] + ad[c][i];
    for (int c = 0; c < 6; c ++) q[3+c] = q[3+c] + ad[off+c][i];
    *qk = ad[3][i] > *qk ? ad[3][i] : *qk;
    *qe = ad[4][i] > *qe ? ad[4][i] : *qe;
  };
  if (r.e - r.b <= SPRING_RUN_LONG)
  {
    for (int i = r.b; i < r.e; i ++) if (!skipped(i)) add(i, p, km, em);
    return;
  }
  const int len = r.e - r.b, ch = spring_run_chunk(len), nc = (len + ch - 1) / ch;
  for (int g0 = 0; g0 < nc; g0 += SPRING_RUN_GROUP)
  {
    double gq[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, gk = 0.0, ge = 0.0;
    for (int c = g0; c < std::min(g0 + SPRING_RUN_GROUP, nc); c ++)
    {
      const int b = r.b + c * ch;
      double q[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, qk = 0.0, qe = 0.0;
      for (int i = b; i < std::min(b + ch, r.e); i ++) if (!skipped(i)) add(i, q, &qk, &qe);
      for (int k = 0; k < 9; k ++) gq[k] = gq[k] + q[k];
      gk = qk > gk ? qk : gk;
      ge = qe > ge ? qe : ge;
    }
    for (int k = 0; k < 9; k ++) p[k] = p[k] + gq[k];
    *km = gk > *km ? gk : *km;
    *em = ge > *em ? ge : *em;
  }
}

static void spring_flush(pg_scene *s, double *const out[9], double *const ad[17], const AdTerms *at)
{
  const int S = s->sprnum;
  std::vector<SprRun> runs;
  int j0 = -1, k0 = -1, jb = 0, kb = 0;
  bool firstj = true, firstk = true;
  for (int i = 0; i < S; i ++)
  {
    const int j = s->sprpart[0][i], k = s->sprpart[1][i];
    if (j0 != j && j0 >= 0) { runs.push_back({j0, 0, jb, i, firstj ? 1 : 0, 2LL*i}); firstj = false; jb = i; }
    if (j0 < 0) jb = i;
    if (k >= 0)
    {
      if (k0 != k && k0 >= 0) { runs.push_back({k0, 1, kb, i, firstk ? 1 : 0, 2LL*i + 1}); firstk = false; kb = i; }
      if (k0 < 0) kb = i;
      k0 = k;
    }
    j0 = j;
  }
  if (j0 >= 0) runs.push_back({j0, 0, jb, S, firstj ? 1 : 0, 2LL*S});
  if (k0 >= 0) runs.push_back({k0, 1, kb, S, firstk ? 1 : 0, 2LL*S + 1});
  for (const SprRun &r : runs)                 /* in stream order */
  {
    double acc[6];
    spring_run_sum(s, out, r, acc);
    const double sg = r.type == 0 ? 1.0 : -1.0;
    for (int c = 0; c < 3; c ++)
    {
      if (sg > 0) { s->force[c][r.part] += acc[c]; s->torque[c][r.part] += acc[3+c]; }
      else { s->force[c][r.part] -= acc[c]; s->torque[c][r.part] -= acc[3+c]; }
    }
    if (at)
    {
      double p[9], km, em;
      spring_run_adaptive(s, ad, r, p, &km, &em);
      for (int c = 0; c < 3; c ++) at->kact[c][r.part] += p[c];
      for (int c = 0; c < 6; c ++) at->krot[c][r.part] += p[3+c];
      at->kmax[r.part] = km > at->kmax[r.part] ? km : at->kmax[r.part];
      at->emax[r.part] = em > at->emax[r.part] ? em : at->emax[r.part];
    }
  }
}

/* ---------------- forces.ispc:641-1412 springs_task (single task) --------- */
void springs_all(pg_scene *s, double step, double time, const AdTerms *at)
{
  const int S = s->sprnum;
  std::vector<double> adv(at ? 17 * (size_t)std::max(S, 1) : 0, 0.0);
  double *ad[17];
  for (int m = 0; m < 17; m ++) ad[m] = at ? adv.data() + (size_t)m * std::max(S, 1) : nullptr;
  double oj[3] = {0}, vj[3] = {0}, xj[3] = {0}, Xj[3] = {0}, Lj[9] = {0};
  double ok[3] = {0}, vk[3] = {0}, xk[3] = {0}, Xk[3] = {0}, Lk[9] = {0};
  int j0 = -1, k0 = -1;
  std::vector<double> outv(9 * (size_t)std::max(S, 1), 0.0);
  double *out[9];
  for (int m = 0; m < 9; m ++) out[m] = outv.data() + (size_t)m * std::max(S, 1);

  for (int i = 0; i < S; i ++)
  {
    double len = 0.0, inv, velocity, spring_force = 0.0, dashpot_force, total_force;
    double Yj[3], Yk[3], p[3], q[3], z[3] = {0.0, 0.0, 0.0}, w[3], frc[3], trq[3], u[3], a[3], b[3];
    double stiffness = 0.0, damping = 0.0;
    int j = s->sprpart[0][i], k = s->sprpart[1][i];

    if (j0 != j)
    {
      oj[0] = s->angular[3][j]; oj[1] = s->angular[4][j]; oj[2] = s->angular[5][j];
      vj[0] = s->linear[0][j]; vj[1] = s->linear[1][j]; vj[2] = s->linear[2][j];
      xj[0] = s->position[0][j]; xj[1] = s->position[1][j]; xj[2] = s->position[2][j];
      Xj[0] = s->position[3][j]; Xj[1] = s->position[4][j]; Xj[2] = s->position[5][j];
      for (int m = 0; m < 9; m ++) Lj[m] = s->rotation[m][j];
    }

    Yj[0] = s->sprpnt[0][3][i];
    Yj[1] = s->sprpnt[0][4][i];
    Yj[2] = s->sprpnt[0][5][i];
    Yj[0] = Yj[0] - Xj[0]; Yj[1] = Yj[1] - Xj[1]; Yj[2] = Yj[2] - Xj[2];
    NVADDMUL(xj, Lj, Yj, p);
    s->sprpnt[0][0][i] = p[0];
    s->sprpnt[0][1][i] = p[1];
    s->sprpnt[0][2][i] = p[2];

    u[0] = vj[0]; u[1] = vj[1]; u[2] = vj[2];
    u[0] *= -1.0; u[1] *= -1.0; u[2] *= -1.0;
    a[0] = p[0] - xj[0]; a[1] = p[1] - xj[1]; a[2] = p[2] - xj[2];
    /* PRODUCTSUB (oj, a, u) */
    u[0] -= oj[1]*a[2] - oj[2]*a[1];
    u[1] -= oj[2]*a[0] - oj[0]*a[2];
    u[2] -= oj[0]*a[1] - oj[1]*a[0];

    if (k >= 0)
    {
      if (k0 != k)
      {
        ok[0] = s->angular[3][k]; ok[1] = s->angular[4][k]; ok[2] = s->angular[5][k];
        vk[0] = s->linear[0][k]; vk[1] = s->linear[1][k]; vk[2] = s->linear[2][k];
        xk[0] = s->position[0][k]; xk[1] = s->position[1][k]; xk[2] = s->position[2][k];
        Xk[0] = s->position[3][k]; Xk[1] = s->position[4][k]; Xk[2] = s->position[5][k];
        for (int m = 0; m < 9; m ++) Lk[m] = s->rotation[m][k];
      }
      if (s->sprflg[i] & PG_SPRDIR_PROJECT)
      {
        w[0] = s->sprdir[3][i]; w[1] = s->sprdir[4][i]; w[2] = s->sprdir[5][i];
        NVMUL(Lk, w, z);
        s->sprdir[0][i] = z[0]; s->sprdir[1][i] = z[1]; s->sprdir[2][i] = z[2];
      }
      Yk[0] = s->sprpnt[1][3][i];
      Yk[1] = s->sprpnt[1][4][i];
      Yk[2] = s->sprpnt[1][5][i];
      Yk[0] = Yk[0] - Xk[0]; Yk[1] = Yk[1] - Xk[1]; Yk[2] = Yk[2] - Xk[2];
      NVADDMUL(xk, Lk, Yk, q);
      s->sprpnt[1][0][i] = q[0];
      s->sprpnt[1][1][i] = q[1];
      s->sprpnt[1][2][i] = q[2];
      u[0] += vk[0]; u[1] += vk[1]; u[2] += vk[2];
      b[0] = q[0] - xk[0]; b[1] = q[1] - xk[1]; b[2] = q[2] - xk[2];
      /* PRODUCTADD (ok, b, u) */
      u[0] += ok[1]*b[2] - ok[2]*b[1];
      u[1] += ok[2]*b[0] - ok[0]*b[2];
      u[2] += ok[0]*b[1] - ok[1]*b[0];
    }
    else
    {
      q[0] = s->sprpnt[1][0][i];
      q[1] = s->sprpnt[1][1][i];
      q[2] = s->sprpnt[1][2][i];
      if (s->sprflg[i] & PG_SPRDIR_PROJECT)
      {
        z[0] = s->sprdir[0][i]; z[1] = s->sprdir[1][i]; z[2] = s->sprdir[2][i];
      }
    }

    switch (s->sprflg[i] & (PG_SPRDIR_FOLLOWER|PG_SPRDIR_CONSTANT|PG_SPRDIR_PLANAR|PG_SPRDIR_PROJECT))
    {
      case PG_SPRDIR_FOLLOWER:
        w[0] = q[0] - p[0]; w[1] = q[1] - p[1]; w[2] = q[2] - p[2];
        len = LEN(w);
        inv = len > 0.0 ? 1.0/len : 0.0;
        z[0] = inv*w[0]; z[1] = inv*w[1]; z[2] = inv*w[2];
        s->sprdir[0][i] = z[0]; s->sprdir[1][i] = z[1]; s->sprdir[2][i] = z[2];
        break;
      case PG_SPRDIR_CONSTANT:
        w[0] = q[0] - p[0]; w[1] = q[1] - p[1]; w[2] = q[2] - p[2];
        z[0] = s->sprdir[0][i]; z[1] = s->sprdir[1][i]; z[2] = s->sprdir[2][i];
        len = DOT(w, z);
        break;
      case PG_SPRDIR_PLANAR:
        w[0] = q[0] - p[0]; w[1] = q[1] - p[1]; w[2] = q[2] - p[2];
        inv = w[0]*s->sprdir[3][i]+w[1]*s->sprdir[4][i]+w[2]*s->sprdir[5][i];
        w[0] -= inv*s->sprdir[3][i];
        w[1] -= inv*s->sprdir[4][i];
        w[2] -= inv*s->sprdir[5][i];
        len = LEN(w);
        inv = len > 0.0 ? 1.0/len : 0.0;
        z[0] = inv*w[0]; z[1] = inv*w[1]; z[2] = inv*w[2];
        s->sprdir[0][i] = z[0]; s->sprdir[1][i] = z[1]; s->sprdir[2][i] = z[2];
        break;
      case PG_SPRDIR_PROJECT:
        w[0] = p[0] - q[0]; w[1] = p[1] - q[1]; w[2] = p[2] - q[2];
        len = DOT(w, z);
        break;
    }

    double offset = 0.0, slope;
    int ilc = s->sproffset[i];
    if (ilc >= 0) offset = look_up(s->lcurve, s->lcidx[ilc], s->lcidx[ilc+1], time, &slope);

    int unspr = s->unspring[i];

    if (unspr <= -2)
    {
      switch (s->sprtype[i])
      {
        case PG_SPRING_NONLINEAR_ELASTIC:
          s->stroke[0][i] = len - s->stroke0[i];
          spring_force = look_up(s->spring, s->spridx[i], s->spridx[i+1], s->stroke[0][i] - offset, &stiffness);
          break;
        case PG_SPRING_GENERAL_NONLINEAR:
          if ((s->sprflg[i] & PG_SPRING_YIELDED) == 0)
          {
            s->stroke[0][i] = len - s->stroke0[i];
            spring_force = look_up(s->spring, s->spridx[i], s->spridx[i+1], s->stroke[0][i] - offset, &stiffness);
            if (spring_force < s->yield[0][i] || spring_force > s->yield[1][i])
            {
              s->sprflg[i] |= PG_SPRING_YIELDED;
              if (spring_force < 0)
              {
                s->stroke[1][i] = s->stroke[0][i];
                s->stroke[2][i] = 0.0;
                s->yield[1][i] = 0.0;
              }
              else
              {
                s->stroke[1][i] = 0.0;
                s->stroke[2][i] = s->stroke[0][i];
                s->yield[0][i] = 0.0;
              }
            }
          }
          else
          {
            double s0 = s->stroke[0][i];
            double s1 = len - s->stroke0[i];
            double ds = s1 - s0;
            double f0 = s->sprfrc[1][i];
            s->stroke[0][i] = s1;
            bool do_loading = false;
            if (f0 * ds > 0)
            {
              if (s->sprflg[i] & PG_SPRING_UNLOADING)
              {
                double dfds = look_up_slope(1, s->unload, s->unidx[i], s->unidx[i+1], f0, NULL);
                spring_force = f0 + dfds*ds;
                if (spring_force < s->yield[0][i] || spring_force > s->yield[1][i])
                {
                  s->sprflg[i] &= ~PG_SPRING_UNLOADING;
                  do_loading = true;
                }
              }
              else do_loading = true;
            }
            else
            {
              double at;
              double dfds = look_up_slope(1, s->unload, s->unidx[i], s->unidx[i+1], f0, &at);
              stiffness = dfds;
              spring_force = f0 + dfds*ds;
              if (spring_force * f0 < 0.0)
              {
                spring_force = look_up(s->unload, s->unidx[i], s->unidx[i+1], ds+at, &stiffness);
              }
              if (spring_force < s->yield[0][i] || spring_force > s->yield[1][i])
              {
                s->sprflg[i] &= ~PG_SPRING_UNLOADING;
                do_loading = true;
              }
              else
              {
                s->sprflg[i] |= PG_SPRING_UNLOADING;
              }
            }
            if (do_loading) /* the 'loading:' label */
            {
              if (ds < 0) s->stroke[1][i] += ds;
              else s->stroke[2][i] += ds;
              spring_force = look_up(s->spring, s->spridx[i], s->spridx[i+1],
                                     ds < 0 ? s->stroke[1][i] : s->stroke[2][i], &stiffness);
              if (ds < 0) s->yield[0][i] = spring_force;
              else s->yield[1][i] = spring_force;
            }
          }
          break;
      }

      velocity = DOT(z, u);

      if (s->dashidx[i]+1 == s->dashidx[i+1])
      {
        double mass = eqm(s, j, Yj, k, Yk, z);
        double ratio = s->dashpot[0][s->dashidx[i]];
        damping = ratio * 2.0 * std::sqrt(std::fabs(stiffness) * mass);
        dashpot_force = velocity * damping;
      }
      else
      {
        dashpot_force = look_up(s->dashpot, s->dashidx[i], s->dashidx[i+1], velocity, &damping);
      }

      total_force = spring_force + (spring_force == 0.0 ? 0.0 : dashpot_force);
    }
    else if (unspr == -1)
    {
      s->stroke[0][i] = len - s->stroke0[i];
      stiffness = 0.;
      damping = 0.;
      spring_force = dashpot_force = total_force = 0.;
      velocity = DOT(z, u);
    }
    else
    {
      double s0 = s->stroke[0][i];
      double s1 = len - s->stroke0[i];
      double ds = s1 - s0;
      double f0 = s->sprfrc[1][i];
      double sgn = f0 > 0. ? 1. : -1.;
      s->stroke[0][i] = s1;
      double at;
      double dfds = look_up_slope(1, s->lcurve, s->lcidx[unspr], s->lcidx[unspr+1], f0, &at);
      stiffness = dfds;
      spring_force = f0 - sgn*std::fabs(dfds*ds);
      if (spring_force * f0 < 0.0)
      {
        s->unspring[i] = -1;
        spring_force = 0.;
      }
      damping = 0.;
      dashpot_force = 0.;
      total_force = spring_force;
      velocity = DOT(z, u);
    }

    frc[0] = z[0] * total_force;
    frc[1] = z[1] * total_force;
    frc[2] = z[2] * total_force;

    s->sprfrc[0][i] = total_force;
    s->sprfrc[1][i] = spring_force;

    double fric = s->sprfric[i];
    if (fric > 0.0)
    {
      double us[3] = {u[0] - velocity*z[0], u[1] - velocity*z[1], u[2] - velocity*z[2]};
      double flim = fric*std::fabs(total_force);
      double fs[3] = {.0, .0, .0};
      double kskn = s->sprkskn[i];
      if (kskn == 0.0)
      {
        double ulen = LEN(us);
        if (ulen > 0.0)
        {
          double coef = flim/ulen;
          fs[0] = coef*us[0]; fs[1] = coef*us[1]; fs[2] = coef*us[2];
        }
      }
      else
      {
        if (spring_force == 0.0)
        {
          s->sprsdsp[0][i] = 0.0; s->sprsdsp[1][i] = 0.0; s->sprsdsp[2][i] = 0.0;
        }
        double ds[3] = {s->sprsdsp[0][i] + us[0]*step, s->sprsdsp[1][i] + us[1]*step, s->sprsdsp[2][i] + us[2]*step};
        double c0 = kskn * std::fabs(stiffness);
        double c1 = spring_force == 0.0 ? 0.0 : kskn * std::fabs(damping);
        fs[0] = c0 * ds[0] + c1 * us[0];
        fs[1] = c0 * ds[1] + c1 * us[1];
        fs[2] = c0 * ds[2] + c1 * us[2];
        double flen = LEN(fs);
        if (flen > flim)
        {
          double coef = flim/flen;
          fs[0] *= coef; fs[1] *= coef; fs[2] *= coef;
          double dl0 = LEN(ds);
          coef = flim/(c0*dl0);
          s->sprsdsp[0][i] = coef*ds[0]; s->sprsdsp[1][i] = coef*ds[1]; s->sprsdsp[2][i] = coef*ds[2];
        }
        else
        {
          s->sprsdsp[0][i] = ds[0]; s->sprsdsp[1][i] = ds[1]; s->sprsdsp[2][i] = ds[2];
        }
      }
      s->sprfrc[2][i] = LEN(fs);
      frc[0] += fs[0]; frc[1] += fs[1]; frc[2] += fs[2];
    }

    /* PRODUCT (a, frc, trq) */
    trq[0] = a[1]*frc[2] - a[2]*frc[1];
    trq[1] = a[2]*frc[0] - a[0]*frc[2];
    trq[2] = a[0]*frc[1] - a[1]*frc[0];

    out[0][i] = frc[0]; out[1][i] = frc[1]; out[2][i] = frc[2];
    out[3][i] = trq[0]; out[4][i] = trq[1]; out[5][i] = trq[2];
    if (at && total_force != 0.0)
    {
      /* the k arm is taken in the k particle's frame; the reference rotates it
       * with the j particle's rotation (forces.ispc:1341) */
      double A[3], dt;
      ad[0][i] = std::fabs(z[0]); ad[1][i] = std::fabs(z[1]); ad[2][i] = std::fabs(z[2]);
      ad[3][i] = std::fabs(stiffness); ad[4][i] = std::fabs(damping);
      TVMUL(Lj, a, A);
      dt = DOT(A, A);
      ad[5][i] = dt - A[0]*A[0]; ad[6][i] = dt - A[1]*A[1]; ad[7][i] = dt - A[2]*A[2];
      ad[8][i] = -A[0]*A[1]; ad[9][i] = -A[0]*A[2]; ad[10][i] = -A[1]*A[2];
      if (k >= 0)
      {
        TVMUL(Lk, b, A);
        dt = DOT(A, A);
        ad[11][i] = dt - A[0]*A[0]; ad[12][i] = dt - A[1]*A[1]; ad[13][i] = dt - A[2]*A[2];
        ad[14][i] = -A[0]*A[1]; ad[15][i] = -A[0]*A[2]; ad[16][i] = -A[1]*A[2];
      }
    }
    if (k >= 0)
    {
      out[6][i] = b[1]*frc[2] - b[2]*frc[1];
      out[7][i] = b[2]*frc[0] - b[0]*frc[2];
      out[8][i] = b[0]*frc[1] - b[1]*frc[0];
      k0 = k;
    }
    j0 = j;
  }
  spring_flush(s, out, ad, at);
}

/* ---------------- forces.ispc:1415-2057 trqspr_task (single task) ---------
 * Per torsion spring: the current frame rot1j = Lj [x0 y0 z0]; roll, pitch
 * and yaw rates from the relative spatial angular velocity; the angles
 * integrate those rates; spring torques from the angle lookups (or from the
 * combined angle of a cone), dampers by lookup or by a critical damping ratio
 * against the local equivalent inertia; the torque rot1j * (roll, pitch,
 * yaw) is added to part0 and subtracted from part1 run by run, as the
 * translational springs are.  Position taken: the pitch-yaw cone's pitch
 * damper reads the pitch ratio (the reference reads the roll entry,
 * forces.ispc:1823). */
void trqspr_all(pg_scene *s, double step, const AdTerms *at)
{
  const int S = s->trqsprnum;
  std::vector<double> out(3 * (size_t)std::max(S, 1), 0.0), kk(3 * (size_t)std::max(S, 1), 0.0);
  for (int i = 0; i < S; i ++)
  {
    const int j = s->trqsprpart[0][i], k = s->trqsprpart[1][i];
    double oj[3] = {s->angular[3][j], s->angular[4][j], s->angular[5][j]}, Lj[9];
    for (int c = 0; c < 9; c ++) Lj[c] = s->rotation[c][j];
    double zdir0[3] = {s->trqzdir0[0][i], s->trqzdir0[1][i], s->trqzdir0[2][i]};
    double xdir0[3] = {s->trqxdir0[0][i], s->trqxdir0[1][i], s->trqxdir0[2][i]};
    double ydir0[3] = {zdir0[1]*xdir0[2] - zdir0[2]*xdir0[1], zdir0[2]*xdir0[0] - zdir0[0]*xdir0[2],
                       zdir0[0]*xdir0[1] - zdir0[1]*xdir0[0]};
    double rot1j[9];
    NVMUL(Lj, xdir0, rot1j);
    NVMUL(Lj, ydir0, rot1j+3);
    NVMUL(Lj, zdir0, rot1j+6);
    for (int c = 0; c < 3; c ++) { s->trqzdir1[c][i] = rot1j[6+c]; s->trqxdir1[c][i] = rot1j[c]; }
    double ok[3] = {0.0, 0.0, 0.0};
    if (k >= 0) { ok[0] = s->angular[3][k]; ok[1] = s->angular[4][k]; ok[2] = s->angular[5][k]; }
    double ojk[3] = {oj[0]-ok[0], oj[1]-ok[1], oj[2]-ok[2]};
    const double rolldot = DOT(rot1j, ojk), pitchdot = DOT(rot1j+3, ojk), yawdot = DOT(rot1j+6, ojk);
    double roll = s->trqrpy[0][i], pitch = s->trqrpy[1][i], yaw = s->trqrpy[2][i];
    roll += rolldot*step;
    pitch += pitchdot*step;
    yaw += yawdot*step;
    s->trqrpy[0][i] = roll; s->trqrpy[1][i] = pitch; s->trqrpy[2][i] = yaw;
    int *const kidx[3] = {s->krpyidx[0], s->krpyidx[1], s->krpyidx[2]};
    int *const didx[3] = {s->drpyidx[0], s->drpyidx[1], s->drpyidx[2]};
    auto ratio_of = [&](int o) { return didx[o][i]+1 == didx[o][i+1]; };
    double Ixx = 0.0, Iyy = 0.0, Izz = 0.0;
    if (ratio_of(0) || ratio_of(1) || ratio_of(2))
    {
      double I[9], tmp[9];
      for (int c = 0; c < 9; c ++) I[c] = s->inverse[c][j];
      if (k >= 0) for (int c = 0; c < 9; c ++) I[c] += s->inverse[c][k];
      NTMUL(I, rot1j, tmp);
      NNMUL(rot1j, tmp, I);
      INVERT(I, tmp);
      Ixx = tmp[0]; Iyy = tmp[4]; Izz = tmp[8];
    }
    auto spring = [&](int o, double arg, double *kslope) {
      if (kidx[o][i+1] > kidx[o][i]) return look_up(s->krpy[o], kidx[o][i], kidx[o][i+1], arg, kslope);
      *kslope = 0.0;
      return 0.0;
    };
    auto damper = [&](int o, int ro, double rate, double kslope, double inertia) {
      if (ratio_of(o))
      {
        const double ratio = s->drpy[ro][0][didx[ro][i]];
        const double d = - ratio * 2.0 * std::sqrt(std::fabs(kslope) * inertia);
        return rate * d;
      }
      double d;
      return look_up(s->drpy[o], didx[o][i], didx[o][i+1], rate, &d);
    };
    double kroll = 0.0, kpitch = 0.0, kyaw = 0.0;
    double trqroll = 0.0, trqpitch = 0.0, trqyaw = 0.0, trqrolltot = 0.0, trqpitchtot = 0.0, trqyawtot = 0.0;
    switch (s->trqcone[i])
    {
      case 0:
      {
        trqroll = spring(0, roll, &kroll);
        trqpitch = spring(1, pitch, &kpitch);
        trqyaw = spring(2, yaw, &kyaw);
        const double trqrolldot = damper(0, 0, rolldot, kroll, Ixx);
        const double trqpitchdot = damper(1, 1, pitchdot, kpitch, Iyy);
        const double trqyawdot = damper(2, 2, yawdot, kyaw, Izz);
        trqrolltot = trqroll + (trqroll == 0.0 ? 0.0 : trqrolldot);
        trqpitchtot = trqpitch + (trqpitch == 0.0 ? 0.0 : trqpitchdot);
        trqyawtot = trqyaw + (trqyaw == 0.0 ? 0.0 : trqyawdot);
        break;
      }
      case 3: /* roll-pitch cone */
      {
        const double angle = std::sqrt(roll*roll + pitch*pitch);
        const double angledot = angle > 0.0 ? (rolldot*roll+pitchdot*pitch)/angle : 0.0;
        trqroll = spring(0, angle, &kroll);
        kpitch = kroll;
        const double trqrolldot = damper(0, 0, angledot, kroll, std::sqrt(Ixx*Ixx + Iyy*Iyy));
        trqyaw = spring(2, yaw, &kyaw);
        const double trqyawdot = damper(2, 2, yawdot, kyaw, Izz);
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
      case 5: /* roll-yaw cone */
      {
        const double angle = std::sqrt(roll*roll + yaw*yaw);
        const double angledot = angle > 0.0 ? (rolldot*roll+yawdot*yaw)/angle : 0.0;
        trqroll = spring(0, angle, &kroll);
        kyaw = kroll;
        const double trqrolldot = damper(0, 0, angledot, kroll, std::sqrt(Ixx*Ixx + Izz*Izz));
        trqpitch = spring(1, pitch, &kpitch);
        const double trqpitchdot = damper(1, 1, pitchdot, kpitch, Iyy);
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
      case 6: /* pitch-yaw cone */
      {
        trqroll = spring(0, roll, &kroll);
        const double trqrolldot = damper(0, 0, rolldot, kroll, Ixx);
        const double angle = std::sqrt(pitch*pitch + yaw*yaw);
        const double angledot = angle > 0.0 ? (pitchdot*pitch+yawdot*yaw)/angle : 0.0;
        trqpitch = spring(1, angle, &kpitch);
        kyaw = kpitch;
        const double trqpitchdot = damper(1, 1, angledot, kpitch, std::sqrt(Iyy*Iyy + Izz*Izz));
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
      case 7: /* roll-pitch-yaw cone */
      {
        const double angle = std::sqrt(roll*roll + pitch*pitch + yaw*yaw);
        const double angledot = angle > 0.0 ? (rolldot*roll+pitchdot*pitch+yawdot*yaw)/angle : 0.0;
        trqroll = spring(0, angle, &kroll);
        kpitch = kyaw = kroll;
        const double trqrolldot = damper(0, 0, angledot, kroll, std::sqrt(Ixx*Ixx + Iyy*Iyy + Izz*Izz));
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
    out[3*i+0] = trqrolltot*rot1j[0] + trqpitchtot*rot1j[3] + trqyawtot*rot1j[6];
    out[3*i+1] = trqrolltot*rot1j[1] + trqpitchtot*rot1j[4] + trqyawtot*rot1j[7];
    out[3*i+2] = trqrolltot*rot1j[2] + trqpitchtot*rot1j[5] + trqyawtot*rot1j[8];
    s->trqrpytot[0][i] = trqrolltot; s->trqrpytot[1][i] = trqpitchtot; s->trqrpytot[2][i] = trqyawtot;
    s->trqrpyspr[0][i] = trqroll; s->trqrpyspr[1][i] = trqpitch; s->trqrpyspr[2][i] = trqyaw;
    kk[3*i+0] = std::fabs(kroll)*rot1j[0];
    kk[3*i+1] = std::fabs(kpitch)*rot1j[4];
    kk[3*i+2] = std::fabs(kyaw)*rot1j[8];
  }
  /* flush: runs of equal part0 added, runs of equal part1 subtracted, in
   * stream order; the first run of a kind starts from zero, later ones from
   * their first element; the adaptive krot partials start from zero */
  int j0 = -1, k0 = -1, jb = 0, kb = 0;
  bool firstj = true, firstk = true;
  auto flush = [&](int part, int type, int b, int e, bool first) {
    double acc[3] = {0.0, 0.0, 0.0}, kp[3] = {0.0, 0.0, 0.0};
    bool started = false;
    for (int i = b; i < e; i ++)
    {
      if (type == 1 && s->trqsprpart[1][i] < 0) continue;
      for (int c = 0; c < 3; c ++)
      {
        acc[c] = (!started && !first) ? out[3*i+c] : acc[c] + out[3*i+c];
        kp[c] = kp[c] + kk[3*i+c];
      }
      started = true;
    }
    for (int c = 0; c < 3; c ++)
    {
      if (type == 0) s->torque[c][part] += acc[c];
      else s->torque[c][part] -= acc[c];
      if (at) at->krot[c][part] += kp[c];
    }
  };
  struct Run { int part, type, b, e, first; long long pos; };
  std::vector<Run> runs;
  for (int i = 0; i < S; i ++)
  {
    const int j = s->trqsprpart[0][i], k = s->trqsprpart[1][i];
    if (j0 != j && j0 >= 0) { runs.push_back({j0, 0, jb, i, firstj ? 1 : 0, 2LL*i}); firstj = false; jb = i; }
    if (j0 < 0) jb = i;
    if (k >= 0)
    {
      if (k0 != k && k0 >= 0) { runs.push_back({k0, 1, kb, i, firstk ? 1 : 0, 2LL*i + 1}); firstk = false; kb = i; }
      if (k0 < 0) kb = i;
      k0 = k;
    }
    j0 = j;
  }
  if (j0 >= 0) runs.push_back({j0, 0, jb, S, firstj ? 1 : 0, 2LL*S});
  if (k0 >= 0) runs.push_back({k0, 1, kb, S, firstk ? 1 : 0, 2LL*S + 1});
  for (const Run &r : runs) flush(r.part, r.type, r.b, r.e, r.first != 0);
}

/* ---------------- forces.ispc:2058-2127 unspring_task (rules in order) ------
 * A rule is checked when stepnum % nsteps == 0 and it has not fired: the SUM,
 * MIN or MAX of an entity (optionally absolute) over its tested springs; a
 * value outside (unlim[0], unlim[1]) counts nfreq down, and at zero the
 * monitored springs take the rule's action (-1: zero force, >= 0: unload
 * along an lcurve) and the activated springs switch on (-3). */
void unspring_all(pg_scene *s, int stepnum)
{
  for (int i = 0; i < s->unsprnum; i ++)
  {
    if (stepnum % s->nsteps[i]) continue;
    if (s->nfreq[i] == 0) continue;
    const int op = s->unop[i];
    double result = op == PG_OP_MIN ? 1.7976931348623157e308 : (op == PG_OP_MAX ? -1.7976931348623157e308 : 0.0);
    for (int j = s->tspridx[i]; j < s->tspridx[i+1]; j ++)
    {
      const int q = s->sprmap[s->tsprings[j]];
      double value = 0.0;
      switch (s->unent[i])
      {
        case PG_HIS_STROKE: value = s->stroke[0][q]; break;
        case PG_HIS_F: value = s->sprfrc[0][q]; break;
        case PG_HIS_SF: value = s->sprfrc[1][q]; break;
        case PG_HIS_FF: value = s->sprfrc[2][q]; break;
      }
      if (s->unabs[i]) value = std::fabs(value);
      if (op == PG_OP_MIN) result = value < result ? value : result;
      else if (op == PG_OP_MAX) result = value > result ? value : result;
      else result += value;
    }
    if (result < s->unlim[0][i] || result > s->unlim[1][i])
    {
      s->nfreq[i] --;
      if (s->nfreq[i] == 0)
      {
        for (int j = s->mspridx[i]; j < s->mspridx[i+1]; j ++) s->unspring[s->sprmap[s->msprings[j]]] = s->unaction[i];
        for (int j = s->actidx[i]; j < s->actidx[i+1]; j ++) s->unspring[s->sprmap[s->activate[j]]] = -3;
      }
    }
  }
}

/* ---------------- restrain.ispc:30-133 ------------------------------------ */
/* v loses its components along the three direction rows of restraint q, in order */
inline void restrain_vec(double *v, double *const dir[9], int q)
{
  for (int k = 0; k < 3; k ++)
  {
    const double l[3] = {dir[3*k][q], dir[3*k+1][q], dir[3*k+2][q]};
    const double dot = DOT(v, l);
    v[0] = v[0] - dot*l[0];
    v[1] = v[1] - dot*l[1];
    v[2] = v[2] - dot*l[2];
  }
}

/* restrain_forces_task, restraints in input order */
void restrain_forces(pg_scene *s)
{
  for (int q = 0; q < s->rstnum; q ++)
  {
    const int j = s->rstpart[q];
    double f[3] = {s->force[0][j], s->force[1][j], s->force[2][j]};
    double t[3] = {s->torque[0][j], s->torque[1][j], s->torque[2][j]};
    restrain_vec(f, s->rstlin, q);
    restrain_vec(t, s->rstang, q);
    for (int c = 0; c < 3; c ++) { s->force[c][j] = f[c]; s->torque[c][j] = t[c]; }
  }
}

/* restrain_velocities_task: linear, spatial and (with the directions taken to
 * the body frame, L^T a) referential angular velocity */
void restrain_velocities(pg_scene *s)
{
  for (int q = 0; q < s->rstnum; q ++)
  {
    const int j = s->rstpart[q];
    double v[3] = {s->linear[0][j], s->linear[1][j], s->linear[2][j]};
    double O[3] = {s->angular[0][j], s->angular[1][j], s->angular[2][j]};
    double o[3] = {s->angular[3][j], s->angular[4][j], s->angular[5][j]};
    double L[9];
    for (int c = 0; c < 9; c ++) L[c] = s->rotation[c][j];
    restrain_vec(v, s->rstlin, q);
    restrain_vec(o, s->rstang, q);
    double A[3][3];
    for (int k = 0; k < 3; k ++)
    {
      const double a[3] = {s->rstang[3*k][q], s->rstang[3*k+1][q], s->rstang[3*k+2][q]};
      TVMUL(L, a, A[k]);
    }
    for (int k = 0; k < 3; k ++)
    {
      const double dot = DOT(O, A[k]);
      O[0] = O[0] - dot*A[k][0];
      O[1] = O[1] - dot*A[k][1];
      O[2] = O[2] - dot*A[k][2];
    }
    for (int c = 0; c < 3; c ++)
    {
      s->linear[c][j] = v[c];
      s->angular[c][j] = O[c];
      s->angular[3+c][j] = o[c];
    }
  }
}

/* ---------------- input.cpp:4247-4341 prescribe_acceleration -------------- */
void prescribe_acceleration(pg_scene *s, const double *lin, const double *ang)
{
  for (int i = 0; i < s->prsnum; i ++)
  {
    int j = s->prspart[i];
    if (s->prslin[i] && s->linkind[i] == 1)
    {
      double ma = s->mass[j];
      s->force[0][j] = ma * lin[3*i];
      s->force[1][j] = ma * lin[3*i+1];
      s->force[2][j] = ma * lin[3*i+2];
    }
    else if (s->prslin[i] && s->linkind[i] == 0)
    {
      s->force[0][j] = 0.0; s->force[1][j] = 0.0; s->force[2][j] = 0.0;
    }
    if (s->prsang[i] && s->angkind[i] == 1)
    {
      double in[9], to[3];
      for (int k = 0; k < 9; k ++) in[k] = s->inertia[k][j];
      NVMUL(in, ang + 3*i, to);
      s->torque[0][j] = to[0]; s->torque[1][j] = to[1]; s->torque[2][j] = to[2];
    }
    else if (s->prsang[i] && s->angkind[i] == 0)
    {
      s->torque[0][j] = 0.0; s->torque[1][j] = 0.0; s->torque[2][j] = 0.0;
    }
  }
}

/* ---------------- input.cpp:4344-4421 prescribe_velocity ------------------ */
void prescribe_velocity(pg_scene *s, const double *lin, const double *ang)
{
  for (int i = 0; i < s->prsnum; i ++)
  {
    int j = s->prspart[i];
    if (s->prslin[i] && s->linkind[i] == 0)
    {
      s->linear[0][j] = lin[3*i]; s->linear[1][j] = lin[3*i+1]; s->linear[2][j] = lin[3*i+2];
    }
    if (s->prsang[i] && s->angkind[i] == 0)
    {
      const double *o = ang + 3*i;
      double L[9], O[3];
      for (int k = 0; k < 9; k ++) L[k] = s->rotation[k][j];
      TVMUL(L, o, O);
      s->angular[0][j] = O[0]; s->angular[1][j] = O[1]; s->angular[2][j] = O[2];
      s->angular[3][j] = o[0]; s->angular[4][j] = o[1]; s->angular[5][j] = o[2];
    }
  }
}

/* slave mirror (forces.ispc:383-405), ordered by master particle */
void build_slaves(or_ctx *ctx, const pg_scene *s)
{
  const int P = s->parnum;
  for (int i = 0; i < P; i ++) ctx->slave[i].clear();
  for (int i = 0; i < P; i ++)
    for (const Con &c : ctx->master[i])
      if (c.slave0 >= 0)
      {
        SlaveCon sc;
        sc.mpart = i; sc.mell = c.master;
        sc.point[0] = c.point[0]; sc.point[1] = c.point[1]; sc.point[2] = c.point[2];
        sc.force[0] = -c.force[0]; sc.force[1] = -c.force[1]; sc.force[2] = -c.force[2];
        sc.kcur = c.kcur; sc.ecur = c.ecur;
        ctx->slave[c.slave0].push_back(sc);
      }
}

const double zeros6[6] = {0, 0, 0, 0, 0, 0};

} /* namespace */

/* ======================================================================== */
/* C entry points used by the tests and the CPU baseline                     */
/* ======================================================================== */
extern "C" {

or_ctx *or_create(const pg_scene *s)
{
  or_ctx *ctx = new or_ctx;
  ctx->master.resize(s->parnum);
  ctx->slave.resize(s->parnum);
  return ctx;
}

void or_destroy(or_ctx *ctx) { delete ctx; }

void or_set_threads(or_ctx *ctx, int threads) { ctx->threads = threads > 0 ? threads : 1; }

/* invert_inertia (parmec.ispc:62-99) */
void or_invert_inertia(or_ctx *ctx, pg_scene *s)
{
#pragma omp parallel for schedule(static) num_threads(ctx->threads)
  for (int i = 0; i < s->parnum; i ++)
  {
    double a[9], x[9];
    for (int j = 0; j < 9; j ++) a[j] = s->inertia[j][i];
    for (int j = 0; j < 9; j ++) x[j] = 0.0;
    INVERT(a, x);
    for (int j = 0; j < 9; j ++) s->inverse[j][i] = x[j];
    s->invm[i] = 1.0 / s->mass[i];
  }
}

/* curtime == 0 block of dem() (parmec.cpp:2397-2405) */
void or_first_half_step(or_ctx *ctx, pg_scene *s, double step, const double *obs_ang, const double *obs_lin)
{
  bool typo = (s->compat & PG_COMPAT_EXPMAP) != 0;
#pragma omp parallel for schedule(static) num_threads(ctx->threads)
  for (int i = 0; i < s->parnum; i ++) euler_one(s, i, 0.5*step, typo);
  shapes_all(ctx, s, false);
  for (int k = 0; k < 3*s->obsnum; k ++)
  {
    s->obsang[k] = obs_ang ? obs_ang[k] : 0.0;
    s->obslin[k] = obs_lin ? obs_lin[k] : 0.0;
  }
  obstacles_all(s, s->obsang, s->obslin, step, typo);
}

/* forces() up to the slave mirror and accumulation, for one step (exported for
 * per-phase parity tests): condet + contacts_task + mirror + contacts_acc_task
 * + springs_task */
void or_condet_forces(or_ctx *ctx, pg_scene *s, double step, double curtime,
                      const double *gravity, const double *obs_ang, const double *obs_lin)
{
  const int P = s->parnum;
  bool obsc = (s->compat & PG_COMPAT_OBSIDX) != 0;
  condet(ctx, s);
#pragma omp parallel for schedule(dynamic, 64) num_threads(ctx->threads)
  for (int i = 0; i < P; i ++) contacts_one(s, ctx->master[i], i, obs_ang, obs_lin, step, obsc);
  build_slaves(ctx, s);
#pragma omp parallel for schedule(dynamic, 64) num_threads(ctx->threads)
  for (int i = 0; i < P; i ++) contacts_acc_one(s, ctx->master[i], ctx->slave[i], i, gravity, nullptr);
  if (s->sprnum) springs_all(s, step, curtime, nullptr);
}

} /* extern "C" */

namespace {

/* ---------------- mesh-mesh contact (extension; pg_meshcontact.cu) -------
 * Pairs in finder order: every mesh triangle t in index order finds, among
 * all triangles u in index order, the partners of another particle whose
 * boxes (widened by r) overlap, by the device's rule (two small or two big
 * triangles: the lower index finds; small and big: the small one finds).
 * Each pair's contact and granular force, with its tangential state from
 * the previous step's pair (finder, partner); then per particle the entries
 * (+f for the finder's particle, -f for the partner's) in pair order, summed
 * in chunks of 1,024 entries (PG_TT_CHUNK): in a chunk by 32 strided lanes
 * from zero and the lane sums added in lane order, then the chunk sums in
 * chunk order from zero; added to the force and torque after gravity. */
int tt_pair_finder(const or_ctx *ctx, const pg_scene *s, int t, int u, const std::vector<double> &box)
{
  if (u == t || s->triobs[u] < 0 || s->triobs[u] == s->triobs[t]) return 0;
  const bool big = ctx->tt_big[t] != 0, ubig = ctx->tt_big[u] != 0;
  if (big && !ubig) return 0;
  if (big == ubig && u < t) return 0;
  const int T = s->trinum;
  for (int c = 0; c < 3; c ++)
    if (!(box[(size_t)c*T + t] < box[(size_t)(3+c)*T + u] && box[(size_t)c*T + u] < box[(size_t)(3+c)*T + t]))
      return 0;
  return 1;
}

void tt_all(or_ctx *ctx, pg_scene *s, double step)
{
  const int T = s->trinum, P = s->parnum;
  const double r = ctx->tt_r;
  std::vector<double> box(6 * (size_t)T, 0.0);
  for (int t = 0; t < T; t ++)
  {
    if (s->triobs[t] < 0) continue;
    for (int c = 0; c < 3; c ++)
    {
      const double a = s->tri[0][c][t], b = s->tri[1][c][t], e = s->tri[2][c][t];
      double l = a < b ? a : b, h = a > b ? a : b;
      l = l < e ? l : e;
      h = h > e ? h : e;
      box[(size_t)c*T + t] = l - r;
      box[(size_t)(3+c)*T + t] = h + r;
    }
  }
  std::vector<int> off(T + 1, 0), pf, pu;
  for (int t = 0; t < T; t ++)
  {
    off[t] = (int)pu.size();
    if (s->triobs[t] < 0) continue;
    for (int u = 0; u < T; u ++)
      if (tt_pair_finder(ctx, s, t, u, box)) { pf.push_back(t); pu.push_back(u); }
  }
  off[T] = (int)pu.size();
  const size_t np = pu.size();
  std::vector<unsigned char> act(np, 0);
  std::vector<double> st(3 * np, 0.0), fr(3 * np, 0.0), pt(3 * np, 0.0);
  for (size_t k = 0; k < np; k ++)
  {
    const int f = pf[k], u = pu[k];
    double va[3][3], vb[3][3];
    for (int a = 0; a < 3; a ++)
      for (int c = 0; c < 3; c ++) { va[a][c] = s->tri[a][c][f]; vb[a][c] = s->tri[a][c][u]; }
    const double *A[3] = {va[0], va[1], va[2]}, *B[3] = {vb[0], vb[1], vb[2]};
    double point[3], normal[3], sk[3] = {0.0, 0.0, 0.0}, fk[3] = {0.0, 0.0, 0.0};
    const double depth = pgtt::contact(A, B, r, r, point, normal);
    const bool active = depth > 0.0;
    if (active)
    {
      if (!ctx->tt_poff.empty())
      {
        const int b0 = ctx->tt_poff[f], b1 = ctx->tt_poff[f+1];
        const int *q = std::lower_bound(ctx->tt_ppu.data() + b0, ctx->tt_ppu.data() + b1, u);
        const int j = (int)(q - ctx->tt_ppu.data());
        if (j < b1 && ctx->tt_ppu[j] == u && ctx->tt_pact[j])
          for (int c = 0; c < 3; c ++) sk[c] = ctx->tt_pst[3*(size_t)j + c];
      }
      const int pa = s->triobs[f], pb = s->triobs[u];
      double vij[3];
      const double za[3] = {point[0]-s->position[0][pa], point[1]-s->position[1][pa], point[2]-s->position[2][pa]};
      const double zb[3] = {point[0]-s->position[0][pb], point[1]-s->position[1][pb], point[2]-s->position[2][pb]};
      for (int c = 0; c < 3; c ++)
      {
        const int c1 = (c+1)%3, c2 = (c+2)%3;
        const double vi = s->angular[3+c1][pa]*za[c2] - s->angular[3+c2][pa]*za[c1] + s->linear[c][pa];
        const double vj = s->angular[3+c1][pb]*zb[c2] - s->angular[3+c2][pb]*zb[c1] + s->linear[c][pb];
        vij[c] = vj - vi;
      }
      const int ij = pairing(s->pairnum, s->pairs, s->tricol[f], s->tricol[u]);
      const double ma = 1.0 / (s->invm[pa] + s->invm[pb]);
      pgtt::granular(s->iparam[SPRING][ij], s->iparam[DAMPER][ij], s->iparam[KSKN][ij], s->iparam[FRISTAT][ij],
                     s->iparam[FRIDYN][ij], ma, normal, vij, depth, step, sk, fk);
    }
    act[k] = active ? 1 : 0;
    for (int c = 0; c < 3; c ++) { st[3*k + c] = sk[c]; fr[3*k + c] = fk[c]; pt[3*k + c] = point[c]; }
  }
  std::vector<std::vector<int>> ent(P);
  for (size_t k = 0; k < np; k ++)
    if (act[k])
    {
      ent[s->triobs[pf[k]]].push_back(2 * (int)k);
      ent[s->triobs[pu[k]]].push_back(2 * (int)k + 1);
    }
  for (int p = 0; p < P; p ++)
  {
    if (ent[p].empty()) continue;
    const double x[3] = {s->position[0][p], s->position[1][p], s->position[2][p]};
    const size_t ne = ent[p].size(), chunk = 1024;
    double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (size_t b = 0; b < ne; b += chunk)
    {
    const size_t e = std::min(ne, b + chunk);
    double part[32][6];
    for (int L = 0; L < 32; L ++)
    {
      double a6[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
      for (size_t q = b + L; q < e; q += 32)
      {
        const int v = ent[p][q], k = v >> 1;
        double f[3] = {fr[3*(size_t)k], fr[3*(size_t)k + 1], fr[3*(size_t)k + 2]};
        if (v & 1) { f[0] = -f[0]; f[1] = -f[1]; f[2] = -f[2]; }
        const double a[3] = {pt[3*(size_t)k]-x[0], pt[3*(size_t)k + 1]-x[1], pt[3*(size_t)k + 2]-x[2]};
        a6[0] += f[0]; a6[1] += f[1]; a6[2] += f[2];
        a6[3] += a[1]*f[2] - a[2]*f[1];
        a6[4] += a[2]*f[0] - a[0]*f[2];
        a6[5] += a[0]*f[1] - a[1]*f[0];
      }
      for (int c = 0; c < 6; c ++) part[L][c] = a6[c];
    }
    double csum[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int L = 0; L < 32; L ++)
      for (int c = 0; c < 6; c ++) csum[c] += part[L][c];
    for (int c = 0; c < 6; c ++) acc[c] += csum[c];
    }
    for (int c = 0; c < 3; c ++)
    {
      s->force[c][p] = s->force[c][p] + acc[c];
      s->torque[c][p] = s->torque[c][p] + acc[3+c];
    }
  }
  ctx->tt_poff = off;
  ctx->tt_ppu = pu;
  ctx->tt_pact = act;
  ctx->tt_pst = st;
}

AdTerms adaptive_terms(or_ctx *ctx, int P)
{
  ctx->kact.assign(3 * (size_t)P, 0.0);
  ctx->krot.assign(6 * (size_t)P, 0.0);
  ctx->kmax.assign((size_t)P, 0.0);
  ctx->emax.assign((size_t)P, 0.0);
  AdTerms at;
  for (int c = 0; c < 3; c ++) at.kact[c] = ctx->kact.data() + (size_t)c * P;
  for (int c = 0; c < 6; c ++) at.krot[c] = ctx->krot.data() + (size_t)c * P;
  at.kmax = ctx->kmax.data();
  at.emax = ctx->emax.data();
  return at;
}

/* one step of the dem() loop body (parmec.cpp:2418-2517) with step0 and
 * step1: condet, forces (with the adaptive terms when at != NULL), the step
 * choice, prescribe, dynamics, shapes, obstacles; returns step1 */
double loop_step(or_ctx *ctx, pg_scene *s, const pg_steptab *tab, int n, double step0, double adaptive,
                 const AdTerms *at)
{
  const int P = s->parnum;
  const bool typo = (s->compat & PG_COMPAT_EXPMAP) != 0;
  const double *grav = tab->gravity ? tab->gravity + 3*(size_t)n : zeros6;
  const double *damp = tab->damping ? tab->damping + 6*(size_t)n : zeros6;
  const double *plin = tab->prs_lin ? tab->prs_lin + (size_t)3*s->prsnum*n : NULL;
  const double *pang = tab->prs_ang ? tab->prs_ang + (size_t)3*s->prsnum*n : NULL;
  double curtime = tab->curtime ? tab->curtime[n] : 0.0;
  bool obsc = (s->compat & PG_COMPAT_OBSIDX) != 0;

  /* partitioning_store + condet + read_gravity_and_damping + forces */
  condet(ctx, s);
#pragma omp parallel for schedule(dynamic, 64) num_threads(ctx->threads)
  for (int i = 0; i < P; i ++) contacts_one(s, ctx->master[i], i, s->obsang, s->obslin, step0, obsc);
  build_slaves(ctx, s);
#pragma omp parallel for schedule(dynamic, 64) num_threads(ctx->threads)
  for (int i = 0; i < P; i ++) contacts_acc_one(s, ctx->master[i], ctx->slave[i], i, grav, at);
  if (ctx->tt_r > 0.0) tt_all(ctx, s, step0);
  if (s->sprnum) springs_all(s, step0, curtime, at);
  if (s->trqsprnum) trqspr_all(s, step0, at);
  if (s->unsprnum) unspring_all(s, tab->stepnum);

  /* prescribe_body_forces (parmec.cpp:2202-2224): export, then add */
  for (int q = 0; q < s->pbfnum; q ++)
  {
    const int p = s->pbfpart[q];
    for (int c = 0; c < 3; c ++)
    {
      s->pbfin[c][q] = s->force[c][p];
      s->pbfin[3+c][q] = s->torque[c][p];
      s->force[c][p] += s->pbfout[c][q];
      s->torque[c][p] += s->pbfout[3+c][q];
    }
  }

  /* adaptive_timestep (parmec.ispc:397-420) */
  double step1 = step0;
  if (at)
  {
    double hmin = 1.7976931348623157e308;
    for (int i = 0; i < P; i ++)
    {
      double kact[3] = {at->kact[0][i], at->kact[1][i], at->kact[2][i]}, krot[6], J[9], om, ra;
      for (int c = 0; c < 6; c ++) krot[c] = at->krot[c][i];
      for (int c = 0; c < 9; c ++) J[c] = s->inertia[c][i];
      double h = critical_step(kact, at->kmax[i], at->emax[i], krot, s->mass[i], J, &om, &ra);
      hmin = h < hmin ? h : hmin;
    }
    if (hmin < 1.7976931348623157e308) step1 = adaptive*hmin;
  }

  /* restrain_forces, prescribe_acceleration, dynamics, prescribe_velocity */
  if (s->rstnum) restrain_forces(s);
  if (s->prsnum && plin && pang) prescribe_acceleration(s, plin, pang);
#pragma omp parallel for schedule(static) num_threads(ctx->threads)
  for (int i = 0; i < P; i ++) dynamics_one(s, i, damp, step0, step1, typo);
  if (s->prsnum && plin && pang) prescribe_velocity(s, plin, pang);

  /* shapes (partial update), obstaclev(curtime+step0), obstacles(0.5*(step0+step1)) */
  shapes_all(ctx, s, true);
  for (int k = 0; k < 3*s->obsnum; k ++)
  {
    s->obsang[k] = tab->obs_ang ? tab->obs_ang[(size_t)3*s->obsnum*n + k] : 0.0;
    s->obslin[k] = tab->obs_lin ? tab->obs_lin[(size_t)3*s->obsnum*n + k] : 0.0;
  }
  obstacles_all(s, s->obsang, s->obslin, 0.5*(step0+step1), typo);
  return step1;
}

} /* namespace */

extern "C" {

/* The loop body of dem() (parmec.cpp:2418-2517) for tab->nsteps steps with a
 * fixed step (adaptive == 0, so step0 == step1 == step). */
int or_run(or_ctx *ctx, pg_scene *s, const pg_steptab *tab, double step)
{
  for (int n = 0; n < tab->nsteps; n ++) loop_step(ctx, s, tab, n, step, 0.0, nullptr);
  return 0;
}

/* The same with adaptive stepping (0 < adaptive <= 1): step n runs with
 * step0 = the previous step's step1 (the first with 'step0') and writes its
 * step1, adaptive * the smallest critical step of the particles, or step0
 * when nothing is restrained, to steps[n]. */
int or_run_adaptive(or_ctx *ctx, pg_scene *s, const pg_steptab *tab, double step0, double adaptive, double *steps)
{
  AdTerms at = adaptive_terms(ctx, s->parnum);
  for (int n = 0; n < tab->nsteps; n ++)
  {
    step0 = loop_step(ctx, s, tab, n, step0, adaptive, &at);
    if (steps) steps[n] = step0;
  }
  return 0;
}

/* restrain_velocities export (restrain.ispc:137), called once per DEM call
 * after invert_inertia (parmec.cpp:2413) */
void or_restrain_velocities(or_ctx *, pg_scene *s) { restrain_velocities(s); }

/* restrain_forces export (restrain.ispc:147) */
void or_restrain_forces(or_ctx *, pg_scene *s) { restrain_forces(s); }

/* Mesh-mesh contact on (radius > 0, with the big-triangle flags of the
 * device's search) or off; the previous step's pairs are dropped. */
void or_mesh_contact(or_ctx *ctx, const pg_scene *s, double radius, const unsigned char *big)
{
  ctx->tt_r = radius > 0.0 ? radius : 0.0;
  ctx->tt_big.assign(big ? big : (const unsigned char *)nullptr, big ? big + s->trinum : nullptr);
  if (!big) ctx->tt_big.assign((size_t)s->trinum, 0);
  ctx->tt_poff.clear();
  ctx->tt_ppu.clear();
  ctx->tt_pact.clear();
  ctx->tt_pst.clear();
}

/* The swept-triangle contact of triangles a and b (9 coordinates each,
 * vertex after vertex): depth, point and normal (pg_tritri.cuh). */
double or_tt_contact(const double *a9, const double *b9, double ra, double rb, double *point, double *normal)
{
  const double *A[3] = {a9, a9 + 3, a9 + 6}, *B[3] = {b9, b9 + 3, b9 + 6};
  return pgtt::contact(A, B, ra, rb, point, normal);
}

/* Pairs and active pairs of the last mesh-contact stage. */
void or_mesh_contact_stats(const or_ctx *ctx, int *pairs, int *active)
{
  *pairs = (int)ctx->tt_ppu.size();
  int a = 0;
  for (unsigned char v : ctx->tt_pact) a += v ? 1 : 0;
  *active = a;
}

/* Per-particle critical step, frequency and damping ratio from the terms of
 * the latest adaptive step (time_step_task, parmec.ispc:275-383). */
int or_critical_terms(or_ctx *ctx, const pg_scene *s, double *h, double *omega, double *ratio)
{
  const int P = s->parnum;
  if ((int)ctx->kmax.size() != P) return -1;
  for (int i = 0; i < P; i ++)
  {
    double kact[3], krot[6], J[9];
    for (int c = 0; c < 3; c ++) kact[c] = ctx->kact[(size_t)c*P + i];
    for (int c = 0; c < 6; c ++) krot[c] = ctx->krot[(size_t)c*P + i];
    for (int c = 0; c < 9; c ++) J[c] = s->inertia[c][i];
    h[i] = critical_step(kact, ctx->kmax[i], ctx->emax[i], krot, s->mass[i], J, &omega[i], &ratio[i]);
  }
  return 0;
}

/* dynamics export (dynamics.ispc:172) for per-kernel parity tests */
void or_dynamics(or_ctx *ctx, pg_scene *s, const double *damping, double step0, double step1)
{
  const bool typo = (s->compat & PG_COMPAT_EXPMAP) != 0;
#pragma omp parallel for schedule(static) num_threads(ctx->threads)
  for (int i = 0; i < s->parnum; i ++) dynamics_one(s, i, damping, step0, step1, typo);
}

/* shapes export (shapes.ispc:214) */
void or_shapes(or_ctx *ctx, pg_scene *s) { shapes_all(ctx, s, false); }

/* obstacles export (obstacles.ispc:28) */
void or_obstacles(or_ctx *, pg_scene *s, double step)
{
  obstacles_all(s, s->obsang, s->obslin, step, (s->compat & PG_COMPAT_EXPMAP) != 0);
}

/* expmap for known-answer tests */
void or_expmap(double o1, double o2, double o3, int typo, double *L) { expmap(o1, o2, o3, L, typo != 0); }

/* triangle_sphere for the closest-point region tests */
double or_triangle_sphere(const double *a, const double *b, const double *c, const double *p, double r,
                          double *point, double *normal, int edge_typo)
{
  return triangle_sphere(a[0], a[1], a[2], b[0], b[1], b[2], c[0], c[1], c[2], p[0], p[1], p[2], r, point, normal,
                         edge_typo != 0);
}

/* equivalent mass (parmec.ispc:423) */
double or_eqm(const pg_scene *s, int part1, const double *point1, int part2, const double *point2,
              const double *direction)
{
  return eqm(s, part1, point1, part2, point2, direction);
}

/* number of master contact points */
int or_contact_count(or_ctx *ctx)
{
  size_t n = 0;
  for (const auto &l : ctx->master) n += l.size();
  return (int)n;
}

/* contacts in canonical order: master particle, then partner code */
int or_contacts(or_ctx *ctx, int cap, int *mpart, int *code, double *point, double *normal,
                double *depth, double *force, double *state)
{
  int n = 0;
  for (size_t i = 0; i < ctx->master.size(); i ++)
    for (const Con &c : ctx->master[i])
    {
      if (n >= cap) return n;
      if (mpart) mpart[n] = (int)i;
      if (code) code[n] = c.slave1;
      for (int d = 0; d < 3; d ++)
      {
        if (point) point[3*n+d] = c.point[d];
        if (normal) normal[3*n+d] = c.normal[d];
        if (force) force[3*n+d] = c.force[d];
        if (state) state[3*n+d] = c.state[d];
      }
      if (depth) depth[n] = c.depth;
      n ++;
    }
  return n;
}

} /* extern "C" */
