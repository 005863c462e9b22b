// pg_math.cuh -- FP64 small-vector algebra for the DEM kernels.
//
// Every helper evaluates the same expression tree as the corresponding macro of
// the reference (macros.h:97-1050, expmap macros.h:1453-1535).  The library is
// compiled with -fmad=false, so no multiply-add is contracted and the FP64 form
// reproduces the CPU restatement bit for bit.
#pragma once

#define PG_DEV __device__ __forceinline__

namespace pg {

PG_DEV double dot3(const double *a, const double *b) { return a[0]*b[0] + a[1]*b[1] + a[2]*b[2]; }

// Comparisons on the integer pipe.  GB300 issues FP64 instructions, DSETP
// included, at 2 lanes per clock per SM; these give the truth values of the
// FP64 comparisons they stand for, from the bit patterns.  The bits are
// taken by a move the compiler cannot see through: with a plain bitcast it
// folds tests such as "bits << 1 != 0" or "exponent != 0x7ff" back into
// FP64 comparisons (DSETP), which issue on the FP64 pipe again.
PG_DEV unsigned long long dbits(double x)
{
  unsigned long long b;
  asm("mov.b64 %0, %1;" : "=l"(b) : "d"(x));
  return b;
}
PG_DEV bool nan_bits(unsigned long long b) { return (b & 0x7fffffffffffffffULL) > 0x7ff0000000000000ULL; }
PG_DEV bool finite_d(double x) { return ((dbits(x) >> 52) & 0x7ff) != 0x7ff; }
// x != 0.0 (true for NaN, as the FP64 comparison)
PG_DEV bool nonzero_d(double x) { return (dbits(x) << 1) != 0; }
// a > b where each of a and b is +0, positive or NaN (never negative or -0,
// as a sum of squares or a square): IEEE order is the bit patterns' order
PG_DEV bool gt_nonneg(double a, double b)
{
  const unsigned long long ua = dbits(a), ub = dbits(b);
  return !nan_bits(ua) && !nan_bits(ub) && ua > ub;
}
// x < 0.0 and x > 0.0: false for NaN and for either zero
PG_DEV bool lt_zero_d(double x) { return dbits(x) - 0x8000000000000001ULL < 0x7ff0000000000000ULL; }
PG_DEV bool gt_zero_d(double x) { return dbits(x) - 1ULL < 0x7ff0000000000000ULL; }
// the IEEE order of non-NaN values as unsigned order, -0 and +0 one key
PG_DEV unsigned long long order_key(unsigned long long b)
{
  if ((b << 1) == 0) b = 0;
  return (long long)b < 0 ? ~b : b | 0x8000000000000000ULL;
}
// a > b for any a and b (false when either is NaN)
PG_DEV bool gt_d(double a, double b)
{
  const unsigned long long ua = dbits(a), ub = dbits(b);
  return !nan_bits(ua) && !nan_bits(ub) && order_key(ua) > order_key(ub);
}

// NVMUL: C = A*B, A column-major 3x3
PG_DEV void nvmul(const double *A, const double *B, double *C)
{
  C[0] = A[0]*B[0]+A[3]*B[1]+A[6]*B[2];
  C[1] = A[1]*B[0]+A[4]*B[1]+A[7]*B[2];
  C[2] = A[2]*B[0]+A[5]*B[1]+A[8]*B[2];
}
// TVMUL: C = A^T*B
PG_DEV void tvmul(const double *A, const double *B, double *C)
{
  C[0] = A[0]*B[0]+A[1]*B[1]+A[2]*B[2];
  C[1] = A[3]*B[0]+A[4]*B[1]+A[5]*B[2];
  C[2] = A[6]*B[0]+A[7]*B[1]+A[8]*B[2];
}
// NVADDMUL: D = C + A*B
PG_DEV void nvaddmul(const double *C, const double *A, const double *B, double *D)
{
  D[0] = C[0] + (A[0]*B[0]+A[3]*B[1]+A[6]*B[2]);
  D[1] = C[1] + (A[1]*B[0]+A[4]*B[1]+A[7]*B[2]);
  D[2] = C[2] + (A[2]*B[0]+A[5]*B[1]+A[8]*B[2]);
}
// NNMUL: C = A*B
PG_DEV void nnmul(const double *A, const double *B, double *C)
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
// TNMUL: C = A^T*B
PG_DEV void tnmul(const double *A, const double *B, double *C)
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

// Rotation matrix of a rotation vector (Lie-group exponential map).  Below ten
// degrees it uses the truncated series sin(x)/x and (1-cos(x))/x^2 in x^2; the
// coefficients are the Taylor coefficients 1/(2k+1)! and 1/(2k+2)!.
// 'typo' reproduces the reference's v02 = O2*O3 (macros.h:1505).
PG_DEV void expmap(double O1, double O2, double O3, double *L, bool typo)
{
  double angsq, sx, cx, v0, v1, v2, v01, v02, v12, s0, s1, s2;
  v0 = O1 * O1;
  v1 = O2 * O2;
  v2 = O3 * O3;
  angsq = v0 + v1 + v2;
  if (gt_nonneg(3.0461741978671E-02, angsq))
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
    angsq = sqrt(angsq);
    double s, c;
    sincos(angsq, &s, &c);
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

PG_DEV double clampd(double a, double b, double c) { return a < b ? b : a > c ? c : a; }

// Closest point of triangle (a,b,c) to sphere centre p, by Voronoi regions of
// the (s,t) parameter plane (condet.ispc:294-400).  Writes the point and the
// unit normal from the point to the centre; returns r - distance.
// 'edge_typo' reproduces the reference's -e/c in the s >= 0, t < 0 region
// beyond edge bc (condet.ispc:373); otherwise the ab-edge parameter -d/a.
// closest point of triangle (A, Bv, Cv) to p (condet.ispc:312-388 regions)
PG_DEV void triangle_closest(const double *A, const double *Bv, const double *Cv, const double *p,
                             double *point, bool edge_typo)
{
  double edge0[3] = {Bv[0]-A[0], Bv[1]-A[1], Bv[2]-A[2]};
  double edge1[3] = {Cv[0]-A[0], Cv[1]-A[1], Cv[2]-A[2]};
  double v0[3] = {A[0]-p[0], A[1]-p[1], A[2]-p[2]};
  double a = dot3(edge0, edge0);
  double b = dot3(edge0, edge1);
  double c = dot3(edge1, edge1);
  double d = dot3(edge0, v0);
  double e = dot3(edge1, v0);
  double det = a*c - b*b;
  double s = b*e - c*d;
  double t = b*d - a*e;
  if (s + t < det)
  {
    if (s < 0.0)
    {
      if (t < 0.0)
      {
        if (d < 0.0) { s = clampd(-d/a, 0.0, 1.0); t = 0.0; }
        else { s = 0.0; t = clampd(-e/c, 0.0, 1.0); }
      }
      else { s = 0.0; t = clampd(-e/c, 0.0, 1.0); }
    }
    else if (t < 0.0) { s = clampd(-d/a, 0.0, 1.0); t = 0.0; }
    else
    {
      double invDet = 1.0 / det;
      s *= invDet;
      t *= invDet;
    }
  }
  else
  {
    if (s < 0.0)
    {
      double tmp0 = b+d;
      double tmp1 = c+e;
      if (tmp1 > tmp0)
      {
        double numer = tmp1 - tmp0;
        double denom = a-2*b+c;
        s = clampd(numer/denom, 0.0, 1.0);
        t = 1-s;
      }
      else { t = clampd(-e/c, 0.0, 1.0); s = 0.0; }
    }
    else if (t < 0.0)
    {
      if (a+d > b+e)
      {
        double numer = c+e-b-d;
        double denom = a-2*b+c;
        s = clampd(numer/denom, 0.0, 1.0);
        t = 1-s;
      }
      else { s = edge_typo ? clampd(-e/c, 0.0, 1.0) : clampd(-d/a, 0.0, 1.0); t = 0.0; }
    }
    else
    {
      double numer = c+e-b-d;
      double denom = a-2*b+c;
      s = clampd(numer/denom, 0.0, 1.0);
      t = 1.0 - s;
    }
  }
  point[0] = A[0] + s*edge0[0] + t*edge1[0];
  point[1] = A[1] + s*edge0[1] + t*edge1[1];
  point[2] = A[2] + s*edge0[2] + t*edge1[2];
}

PG_DEV double triangle_sphere(const double *A, const double *Bv, const double *Cv, const double *p, double r,
                              double *point, double *normal, bool edge_typo)
{
  triangle_closest(A, Bv, Cv, p, point, edge_typo);
  double q[3] = {p[0]-point[0], p[1]-point[1], p[2]-point[2]};
  double len = sqrt(dot3(q, q));
  double ilen = 1.0/len;
  normal[0] = ilen*q[0];
  normal[1] = ilen*q[1];
  normal[2] = ilen*q[2];
  return r - len;
}

// INVERT (macros.h:1033): leaves INV untouched when singular
PG_DEV void invert3(const double *F, double *INV)
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

// NTMUL: C = A*B^T
PG_DEV void ntmul(const double *A, const double *B, double *C)
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

// cos(acos(r)/3) (largest) or cos(acos(r)/3 + 2 pi/3) (smallest) as roots of
// the triple-angle identity 4c^3 - 3c = r.  Newton's method from c = 1 (or
// -1): the cubic is convex and increasing on [1/2, 1] (concave and increasing
// on [-1, -1/2]), so the iterates move monotonically to the root and the loop
// stops when they cease to.  Basic operations only, so every IEEE machine
// gives the same bits (the CPU restatement runs the same steps).
PG_DEV double triple_angle_root(double r, bool largest)
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

// extremum_eigenvalue (macros.h:1539-1588) of a symmetric column-major 3x3:
// the trigonometric formula with the cosines taken by triple_angle_root.  The
// diagonal branch returns the largest diagonal entry whichever is asked for,
// as the reference does (macros.h:1545-1553).
PG_DEV double extremum_eigenvalue(const double *A, bool minimum)
{
  double p1 = A[3]*A[3] + A[6]*A[6] + A[7]*A[7];
  if (p1 == 0.0)
  {
    double r = A[0] > A[4] ? A[0] : A[4];
    return r > A[8] ? r : A[8];
  }
  double q = (A[0]+A[4]+A[8])/3.0;
  double p2 = (A[0]-q)*(A[0]-q) + (A[4]-q)*(A[4]-q) + (A[8]-q)*(A[8]-q) + 2*p1;
  double p = sqrt(p2 / 6.0);
  double invp = 1.0 / p;
  double B[9] = {invp*(A[0]-q), invp*A[1], invp*A[2], invp*A[3], invp*(A[4]-q), invp*A[5],
                 invp*A[6], invp*A[7], invp*(A[8]-q)};
  double r = 0.5 * (B[0]*(B[4]*B[8]-B[5]*B[7]) + B[3]*(B[2]*B[7]-B[1]*B[8]) + B[6]*(B[1]*B[5]-B[2]*B[4]));
  return q + 2.0 * p * triple_angle_root(r, !minimum);
}

// Critical step of one particle (time_step_task, parmec.ispc:275-383) from its
// stiffness terms: translational sqrt(n k / m); rotational from K x = w^2 J x
// through the Cholesky factor of J; each damped as (2/w)(sqrt(1+ksi^2) - ksi).
// A particle without rotational stiffness (w_rot = 0: springs attached at the
// mass centre) takes the translational step; the reference divides by zero
// there and its NaN drops the particle from the minimum.  Returns DBL_MAX when
// nothing restrains the particle.
PG_DEV double critical_step(const double kact[3], double kmax, double emax, const double krot[6], double mass,
                            const double J[9], double *omega, double *ratio)
{
  const double nxy = kact[0] > kact[1] ? kact[0] : kact[1];
  const double nxyz = nxy > kact[2] ? nxy : kact[2];
  if (!(nxyz > 0.0)) { *omega = 0.0; *ratio = 0.0; return 1.7976931348623157e308; }
  const double k = kmax;
  const double omegaxyz = sqrt(nxyz*k/mass);
  double K[9];
  K[0] = k*krot[0]; K[1] = k*krot[3]; K[2] = k*krot[4];
  K[3] = K[1]; K[4] = k*krot[1]; K[5] = k*krot[5];
  K[6] = K[2]; K[7] = K[5]; K[8] = k*krot[2];
  const double mrot = extremum_eigenvalue(J, true);
  double L[9], invL[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, tmp[9], A[9], inv;
  L[0] = sqrt(J[0]);
  inv = 1.0/L[0];
  L[1] = inv * J[1];
  L[2] = inv * J[2];
  L[3] = 0.0;
  L[4] = sqrt(J[4] - L[1]*L[1]);
  inv = 1.0/L[4];
  L[5] = inv * (J[5] - L[2]*L[1]);
  L[6] = 0.0;
  L[7] = 0.0;
  L[8] = sqrt(J[8] - (L[2]*L[2] + L[5]*L[5]));
  invert3(L, invL);
  ntmul(K, invL, tmp);
  nnmul(invL, tmp, A);
  const double lambda = extremum_eigenvalue(A, false);
  const double omegarot = lambda > 0.0 ? sqrt(lambda) : 0.0;
  const double damping = emax;
  const double ratioxyz = damping / (2.0*mass*omegaxyz);
  const double hxyz = (2.0/omegaxyz)*(sqrt(1.0+ratioxyz*ratioxyz) - ratioxyz);
  double ratiorot = 0.0, hrot = 1.7976931348623157e308;
  if (omegarot > 0.0)
  {
    ratiorot = damping / (2.0*mrot*omegarot);
    hrot = (2.0/omegarot)*(sqrt(1.0+ratiorot*ratiorot) - ratiorot);
  }
  *omega = omegaxyz > omegarot ? omegaxyz : omegarot;
  *ratio = ratioxyz > ratiorot ? ratioxyz : ratiorot;
  return hxyz < hrot ? hxyz : hrot;
}

// krot terms of one arm A (body frame): K(1,1), K(2,2), K(3,3), K(2,1),
// K(3,1), K(3,2) (forces.ispc:514-522, 1262-1268)
PG_DEV void krot_add(double *krot, const double *A)
{
  const double dt = dot3(A, A);
  krot[0] += dt - A[0]*A[0];
  krot[1] += dt - A[1]*A[1];
  krot[2] += dt - A[2]*A[2];
  krot[3] += -A[0]*A[1];
  krot[4] += -A[0]*A[2];
  krot[5] += -A[1]*A[2];
}

} // namespace pg
