// pg_tritri.cuh -- mesh-mesh contact between triangles (an extension: the
// reference detects no contact between meshes, partition.ispc:600-646 and
// condet.ispc:786).
//
// Each mesh triangle is swept by a sphere of radius r (a triangle of
// thickness 2r).  Two triangles of different particles touch when their
// distance d is below rA + rB: the contact point is the midpoint of their
// closest points, the normal points from B's closest point to A's, and the
// depth is rA + rB - d.  When the triangles intersect (d = 0) the normal is
// B's face normal turned towards A's centroid and the depth rA + rB.
//
// The distance of two triangles that do not intersect is the smallest of
// the six vertex-triangle and the nine edge-edge distances; an intersection
// shows as an edge of one crossing the other.  Ties keep the first candidate
// in that order, so the result is a function of the inputs alone.  The
// functions are compiled for the device and for the CPU oracle (FP64 with no
// contraction on both), which therefore evaluate the same operations.
#pragma once
#include <math.h>
#include <string.h>

#ifdef __CUDACC__
#define PG_TT __host__ __device__ __forceinline__
#else
#define PG_TT inline
#endif

namespace pgtt {

PG_TT double dot(const double *a, const double *b) { return a[0]*b[0] + a[1]*b[1] + a[2]*b[2]; }
PG_TT void sub(const double *a, const double *b, double *c) { c[0] = a[0]-b[0]; c[1] = a[1]-b[1]; c[2] = a[2]-b[2]; }
PG_TT void cross(const double *a, const double *b, double *c)
{
  c[0] = a[1]*b[2] - a[2]*b[1];
  c[1] = a[2]*b[0] - a[0]*b[2];
  c[2] = a[0]*b[1] - a[1]*b[0];
}

// Comparisons taken from the bit patterns, on the integer pipe of the
// device (the FP64 pipe, which issues comparisons too, is the narrow one);
// each gives the truth value of the IEEE comparison it stands for, NaN
// operands included.  On the device the bits are taken by a move the
// compiler cannot fold back into an FP64 comparison.  The plane test and
// the box keys of the candidate search use them; in the narrow phase, whose
// branches they reshape, plain comparisons measured faster.
PG_TT unsigned long long bits(double x)
{
  unsigned long long b;
#ifdef __CUDA_ARCH__
  asm("mov.b64 %0, %1;" : "=l"(b) : "d"(x));
#else
  memcpy(&b, &x, sizeof b);
#endif
  return b;
}
PG_TT bool nan_b(unsigned long long b) { return (b & 0x7fffffffffffffffULL) > 0x7ff0000000000000ULL; }
// non-NaN values in IEEE order as unsigned order, -0 and +0 one key
PG_TT unsigned long long okey(unsigned long long b)
{
  if ((b << 1) == 0) b = 0;
  return (long long)b < 0 ? ~b : b | 0x8000000000000000ULL;
}
PG_TT bool lt(double x, double y)
{
  const unsigned long long a = bits(x), b = bits(y);
  return !nan_b(a) && !nan_b(b) && okey(a) < okey(b);
}
PG_TT bool gt(double x, double y) { return lt(y, x); }
// x < -y, the sign of y flipped on its bits
PG_TT bool lt_neg(double x, double y)
{
  const unsigned long long a = bits(x), b = bits(y) ^ 0x8000000000000000ULL;
  return !nan_b(a) && !nan_b(b) && okey(a) < okey(b);
}
PG_TT double clamp01(double x) { return x < 0.0 ? 0.0 : (x > 1.0 ? 1.0 : x); }

// Closest point q of triangle (a, b, c) to p: the Voronoi-region method
// (Ericson, Real-Time Collision Detection, 5.1.5).  The region is found
// first and its one division taken at a single place, so that threads of a
// warp in different regions share the division's instructions; each region
// divides the same operands as the textbook branches do.
// (ab = b - a and ac = c - a come with the triangle, computed once for the
// three calls of a triangle pair that use them.)
PG_TT void point_triangle(const double *p, const double *a, const double *b, const double *c,
                          const double *ab, const double *ac, double *q)
{
  double ap[3], bp[3], cp[3];
  sub(p, a, ap); sub(p, b, bp); sub(p, c, cp);
  const double d1 = dot(ab, ap), d2 = dot(ac, ap);
  const double d3 = dot(ab, bp), d4 = dot(ac, bp);
  const double d5 = dot(ab, cp), d6 = dot(ac, cp);
  const double vc = d1*d4 - d3*d2;
  const double vb = d5*d2 - d1*d6;
  const double va = d3*d6 - d5*d4;
  const double e43 = d4 - d3, e56 = d5 - d6;
  // 0: vertex a, 1: vertex b, 2: edge ab, 3: vertex c, 4: edge ac, 5: edge bc, 6: face
  const int region = (d1 <= 0.0 && d2 <= 0.0) ? 0 :
                     (d3 >= 0.0 && d4 <= d3) ? 1 :
                     (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) ? 2 :
                     (d6 >= 0.0 && d5 <= d6) ? 3 :
                     (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) ? 4 :
                     (va <= 0.0 && e43 >= 0.0 && e56 >= 0.0) ? 5 : 6;
  double num = 0.0, den = 1.0;
  if (region == 2) { num = d1; den = d1 - d3; }
  else if (region == 4) { num = d2; den = d2 - d6; }
  else if (region == 5) { num = e43; den = e43 + e56; }
  else if (region == 6) { num = 1.0; den = va + vb + vc; }
  const double x = num / den;
  switch (region)
  {
  case 0: q[0] = a[0]; q[1] = a[1]; q[2] = a[2]; break;
  case 1: q[0] = b[0]; q[1] = b[1]; q[2] = b[2]; break;
  case 3: q[0] = c[0]; q[1] = c[1]; q[2] = c[2]; break;
  case 2: q[0] = a[0] + x*ab[0]; q[1] = a[1] + x*ab[1]; q[2] = a[2] + x*ab[2]; break;
  case 4: q[0] = a[0] + x*ac[0]; q[1] = a[1] + x*ac[1]; q[2] = a[2] + x*ac[2]; break;
  case 5: q[0] = b[0] + x*(c[0]-b[0]); q[1] = b[1] + x*(c[1]-b[1]); q[2] = b[2] + x*(c[2]-b[2]); break;
  default:
  {
    const double v = vb * x, w = vc * x;
    q[0] = a[0] + ab[0]*v + ac[0]*w;
    q[1] = a[1] + ab[1]*v + ac[1]*w;
    q[2] = a[2] + ab[2]*v + ac[2]*w;
  }
  }
}

// Closest points c1 on p1q1 and c2 on p2q2 (Ericson 5.1.9); returns |c1-c2|^2.
// Parallel segments take s = 0.  The divisions of the general case are taken
// at single places (the clamped end's recomputation of s divides whichever
// numerator applies), so that threads of a warp share them.
// (d1 = q1 - p1 and d2 = q2 - p2 come with the triangles' edges, a = d1.d1
// and e = d2.d2 with them.)
PG_TT double segment_segment(const double *p1, const double *d1, double a, const double *p2, const double *d2,
                             double e, double *c1, double *c2)
{
  double r[3];
  sub(p1, p2, r);
  const double f = dot(d2, r);
  double s, t;
  if (a <= 0.0 && e <= 0.0) { s = 0.0; t = 0.0; }
  else if (a <= 0.0) { s = 0.0; t = clamp01(f / e); }
  else
  {
    const double c = dot(d1, r);
    if (e <= 0.0) { t = 0.0; s = clamp01(-c / a); }
    else
    {
      const double b = dot(d1, d2);
      const double den = a*e - b*b;
      const double s0 = (b*f - c*e) / (den != 0.0 ? den : 1.0);
      s = den != 0.0 ? clamp01(s0) : 0.0;
      t = (b*s + f) / e;
      const bool low = t < 0.0, high = t > 1.0;
      if (low || high)
      {
        s = clamp01((low ? -c : b - c) / a);
        t = low ? 0.0 : 1.0;
      }
    }
  }
  c1[0] = p1[0] + d1[0]*s; c1[1] = p1[1] + d1[1]*s; c1[2] = p1[2] + d1[2]*s;
  c2[0] = p2[0] + d2[0]*t; c2[1] = p2[1] + d2[1]*t; c2[2] = p2[2] + d2[2]*t;
  double w[3];
  sub(c1, c2, w);
  return dot(w, w);
}

// A triangle with the differences every test of a pair takes from it: its
// edges from each vertex to the next, ac = c - a, and the plane normal
// n = (b - a) x (c - a).
struct Tri
{
  const double *v[3];
  double e[3][3];                 // e[k] = v[k+1] - v[k]
  double l2[3];                   // e[k].e[k]
  double ac[3], n[3];
};

PG_TT void tri_prep(const double *const t[3], Tri &T)
{
  for (int k = 0; k < 3; k ++) T.v[k] = t[k];
  for (int k = 0; k < 3; k ++) sub(t[(k+1)%3], t[k], T.e[k]);
  for (int k = 0; k < 3; k ++) T.l2[k] = dot(T.e[k], T.e[k]);
  sub(t[2], t[0], T.ac);
  cross(T.e[0], T.ac, T.n);
}

// Does segment pq cross triangle T through its interior or boundary?  The
// end points lie strictly on opposite sides of the plane and the crossing
// point lies inside the triangle (same-side tests).  x: the point.
PG_TT bool segment_crosses(const double *p, const double *q, const Tri &T, double *x)
{
  const double *a = T.v[0];
  double ap[3], aq[3];
  sub(p, a, ap); sub(q, a, aq);
  const double dp = dot(T.n, ap), dq = dot(T.n, aq);
  if (!((dp > 0.0 && dq < 0.0) || (dp < 0.0 && dq > 0.0))) return false;
  const double t = dp / (dp - dq);
  x[0] = p[0] + (q[0]-p[0])*t; x[1] = p[1] + (q[1]-p[1])*t; x[2] = p[2] + (q[2]-p[2])*t;
  for (int k = 0; k < 3; k ++)
  {
    double h[3], m[3];
    sub(x, T.v[k], h);
    cross(T.e[k], h, m);
    if (dot(T.n, m) < 0.0) return false;
  }
  return true;
}

// Distance squared of triangles A (a[0..2]) and B (b[0..2]) with their
// closest points pa on A and pb on B; returns 0 when they intersect (pa =
// pb = the first crossing found).
PG_TT double triangle_triangle(const double *const a[3], const double *const b[3], double *pa, double *pb)
{
  Tri A, B;
  tri_prep(a, A);
  tri_prep(b, B);
  for (int i = 0; i < 3; i ++)
  {
    double x[3];
    if (segment_crosses(a[i], a[(i+1)%3], B, x) || segment_crosses(b[i], b[(i+1)%3], A, x))
    {
      pa[0] = pb[0] = x[0]; pa[1] = pb[1] = x[1]; pa[2] = pb[2] = x[2];
      return 0.0;
    }
  }
  double best = 1.7976931348623157e308;
  for (int i = 0; i < 3; i ++)
  {
    double q[3], w[3];
    point_triangle(a[i], b[0], b[1], b[2], B.e[0], B.ac, q);
    sub(a[i], q, w);
    const double d2 = dot(w, w);
    if (d2 < best) { best = d2; for (int k = 0; k < 3; k ++) { pa[k] = a[i][k]; pb[k] = q[k]; } }
  }
  for (int i = 0; i < 3; i ++)
  {
    double q[3], w[3];
    point_triangle(b[i], a[0], a[1], a[2], A.e[0], A.ac, q);
    sub(q, b[i], w);
    const double d2 = dot(w, w);
    if (d2 < best) { best = d2; for (int k = 0; k < 3; k ++) { pa[k] = q[k]; pb[k] = b[i][k]; } }
  }
  for (int i = 0; i < 3; i ++)
    for (int j = 0; j < 3; j ++)
    {
      double c1[3], c2[3];
      const double d2 = segment_segment(a[i], A.e[i], A.l2[i], b[j], B.e[j], B.l2[j], c1, c2);
      if (d2 < best) { best = d2; for (int k = 0; k < 3; k ++) { pa[k] = c1[k]; pb[k] = c2[k]; } }
    }
  return best;
}

// Are Q's vertices all farther than s from P's plane, on one side?  (The
// plane normal is left unnormalised: distances are compared with s |n|.)
PG_TT bool beyond_plane(const double *const P[3], const double *const Q[3], double s)
{
  double e1[3], e2[3], n[3];
  sub(P[1], P[0], e1); sub(P[2], P[0], e2);
  cross(e1, e2, n);
  const double lim = s * sqrt(dot(n, n));
  int above = 0, below = 0;
  for (int k = 0; k < 3; k ++)
  {
    double w[3];
    sub(Q[k], P[0], w);
    const double h = dot(n, w);
    above += gt(h, lim) ? 1 : 0;
    below += lt_neg(h, lim) ? 1 : 0;
  }
  return above == 3 || below == 3;
}

// Triangles with one wholly beyond the other's plane by ra + rb are apart.
PG_TT bool apart(const double *const a[3], const double *const b[3], double ra, double rb)
{
  return beyond_plane(a, b, ra + rb) || beyond_plane(b, a, ra + rb);
}

// contact() for triangles that are not apart
PG_TT double contact_near(const double *const a[3], const double *const b[3], double ra, double rb,
                          double *point, double *normal)
{
  double pa[3], pb[3];
  const double d2 = triangle_triangle(a, b, pa, pb);
  point[0] = 0.5*(pa[0]+pb[0]); point[1] = 0.5*(pa[1]+pb[1]); point[2] = 0.5*(pa[2]+pb[2]);
  if (d2 > 0.0)
  {
    const double d = sqrt(d2);
    const double id = 1.0 / d;
    normal[0] = (pa[0]-pb[0])*id; normal[1] = (pa[1]-pb[1])*id; normal[2] = (pa[2]-pb[2])*id;
    return (ra + rb) - d;
  }
  double e1[3], e2[3], n[3];
  sub(b[1], b[0], e1); sub(b[2], b[0], e2);
  cross(e1, e2, n);
  const double ln = sqrt(dot(n, n));
  const double il = ln > 0.0 ? 1.0 / ln : 0.0;
  double ca[3], cb[3], w[3];
  for (int k = 0; k < 3; k ++)
  {
    ca[k] = (a[0][k] + a[1][k] + a[2][k]) / 3.0;
    cb[k] = (b[0][k] + b[1][k] + b[2][k]) / 3.0;
  }
  sub(ca, cb, w);
  const double sg = dot(n, w) < 0.0 ? -il : il;
  normal[0] = n[0]*sg; normal[1] = n[1]*sg; normal[2] = n[2]*sg;
  return ra + rb;
}

// Contact of swept triangles A and B (radii ra, rb): returns the depth
// (> 0: touching) with the point and the unit normal from B towards A.
// Triangles apart: depth -1, point and normal zero.
PG_TT double contact(const double *const a[3], const double *const b[3], double ra, double rb,
                     double *point, double *normal)
{
  if (apart(a, b, ra, rb))
  {
    point[0] = point[1] = point[2] = 0.0;
    normal[0] = normal[1] = normal[2] = 0.0;
    return -1.0;
  }
  return contact_near(a, b, ra, rb, point, normal);
}

// The granular contact law (forces.ispc:125-192) for normal n (from the
// partner towards the master), relative velocity vij = v_partner - v_master,
// depth, pair parameters and reduced mass: the force f on the master, and
// the tangential spring state advanced by step * the tangential velocity.
PG_TT void granular(double kn, double damper, double kskn, double mus, double mud, double ma,
                    const double *n, const double *vij, double depth, double step, double *state, double *f)
{
  const double en = damper * 2.0 * sqrt(kn*ma);
  const double vn = dot(vij, n);
  const double fn = kn*depth + en*vn;
  f[0] = fn*n[0];
  f[1] = fn*n[1];
  f[2] = fn*n[2];
  const double kt = kn * kskn;
  const double et = en * kskn;
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
  const double len = sqrt(dot(ft, ft));
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
}

} // namespace pgtt
