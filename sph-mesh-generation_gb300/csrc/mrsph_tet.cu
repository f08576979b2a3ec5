// mrsph_tet.cu — 3D tetrahedralisation of the particles and tet quality (row F3).
//
//   Graphmeshcls::Reconstruct_tets (graph_mesh.cpp:981-1100) hands every
//   particle to TetGen (a Delaunay tetrahedralisation of the convex hull) and
//   drops the tets Check_whether_this_tet_should_be_delete (:675-979) names:
//   all four particles not REAL and aspect ratio above tet_delete_thres = 10
//   (its phi tests are commented out).
//     -> k_tet_star: local Delaunay stars, one warp per particle.  Particle
//        i gift-wraps the tets around itself over its neighbour row, which
//        holds every particle within cutoff * h_i, walking its whole star in
//        the row's Delaunay tetrahedralisation.  A tet is certified when its
//        circumsphere lies inside that ball and no row particle lies inside
//        or on it; then no particle at all does, so it is a Delaunay tet of
//        the whole set and the unique one through its four particles.  Each
//        certified tet is emitted once, by the lowest-id particle whose ball
//        holds it.  Tets that no ball holds (across concavities of the body
//        and on the convex hull, where TetGen keeps large tets) are not
//        produced.
//   Graphmeshcls::Tet_quality_statistics (:1967-2400) -> k_tet_quality: the
//   volume, edge, aspect-ratio, radius-ratio and dihedral-angle statistics
//   and histograms of the kept tets.
// Positions are snapped to the grid 2^(e-52), e the exponent that bounds the
// domain, so that every coordinate is both an exact double and an exact
// integer.  Predicate signs come from an FP64 evaluation with a conservative
// error bound (the permanent bounds of Shewchuk, "Adaptive Precision
// Floating-Point Arithmetic and Fast Robust Geometric Predicates", 1997) and,
// when the bound cannot decide, from exact 320-bit integer arithmetic, so the
// tets do not depend on evaluation order.  Compiled with -fmad=false.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "handle.h"

namespace mrsph {
namespace {

// ------------------------------------------------------------ 320-bit integers
// Two's complement, little-endian 64-bit limbs; wide enough for the insphere
// determinant of 54-bit coordinate differences (< 2^277).
constexpr int BL = 5;
struct BI {
  unsigned long long w[BL];
};

__device__ inline BI bi_from(long long v) {
  BI r;
  const unsigned long long s = v < 0 ? ~0ull : 0ull;
  r.w[0] = (unsigned long long)v;
  for (int k = 1; k < BL; k++) r.w[k] = s;
  return r;
}
__device__ inline BI bi_add(const BI& a, const BI& b) {
  BI r;
  unsigned long long c = 0;
  for (int k = 0; k < BL; k++) {
    const unsigned long long s = a.w[k] + b.w[k];
    const unsigned long long c1 = s < a.w[k];
    r.w[k] = s + c;
    c = c1 | (r.w[k] < s);
  }
  return r;
}
__device__ inline BI bi_neg(const BI& a) {
  BI r;
  unsigned long long c = 1;
  for (int k = 0; k < BL; k++) {
    r.w[k] = ~a.w[k] + c;
    c = (c && r.w[k] == 0) ? 1 : 0;
  }
  return r;
}
__device__ inline BI bi_sub(const BI& a, const BI& b) { return bi_add(a, bi_neg(b)); }
__device__ inline bool bi_negative(const BI& a) { return (long long)a.w[BL - 1] < 0; }
__device__ inline int bi_sign(const BI& a) {
  if (bi_negative(a)) return -1;
  for (int k = 0; k < BL; k++)
    if (a.w[k]) return 1;
  return 0;
}
// a * b, both |.| < 2^(64 BL - 1) with the product in range
__device__ BI bi_mul(const BI& a, const BI& b) {
  const bool na = bi_negative(a), nb = bi_negative(b);
  const BI ua = na ? bi_neg(a) : a, ub = nb ? bi_neg(b) : b;
  BI r;
  for (int k = 0; k < BL; k++) r.w[k] = 0;
  for (int i = 0; i < BL; i++) {
    if (!ua.w[i]) continue;
    unsigned long long carry = 0;
    for (int j = 0; i + j < BL; j++) {
      const unsigned long long lo = ua.w[i] * ub.w[j], hi = __umul64hi(ua.w[i], ub.w[j]);
      unsigned long long s = r.w[i + j] + lo;
      unsigned long long c = s < lo;
      s += carry;
      c += s < carry;
      r.w[i + j] = s;
      carry = hi + c;
    }
  }
  return (na != nb) ? bi_neg(r) : r;
}

// ------------------------------------------------------------ predicates
// Points are snapped doubles; I = integer coordinates (x / grid).
struct Pt {
  double x, y, z;
};
constexpr double kEps = 1.1102230246251565e-16;  // 2^-53
// Conservative error-bound factors of the FP64 evaluations below (the
// published bounds are 7 eps and 16 eps of the same permanents).
constexpr double kO3Bound = 16.0 * kEps;
constexpr double kIsBound = 64.0 * kEps;

__device__ inline long long ival(double v, double inv_g) { return __double2ll_rn(v * inv_g); }

// orient3d(a, b, c, d) = det[a - d; b - d; c - d]: > 0 when d lies below the
// plane of a, b, c seen counter-clockwise from above.
__device__ __noinline__ int orient_x(const Pt& a, const Pt& b, const Pt& c, const Pt& d, double ig) {
  const long long adx = ival(a.x, ig) - ival(d.x, ig), ady = ival(a.y, ig) - ival(d.y, ig),
                  adz = ival(a.z, ig) - ival(d.z, ig);
  const long long bdx = ival(b.x, ig) - ival(d.x, ig), bdy = ival(b.y, ig) - ival(d.y, ig),
                  bdz = ival(b.z, ig) - ival(d.z, ig);
  const long long cdx = ival(c.x, ig) - ival(d.x, ig), cdy = ival(c.y, ig) - ival(d.y, ig),
                  cdz = ival(c.z, ig) - ival(d.z, ig);
  const BI m1 = bi_sub(bi_mul(bi_from(bdy), bi_from(cdz)), bi_mul(bi_from(bdz), bi_from(cdy)));
  const BI m2 = bi_sub(bi_mul(bi_from(cdy), bi_from(adz)), bi_mul(bi_from(cdz), bi_from(ady)));
  const BI m3 = bi_sub(bi_mul(bi_from(ady), bi_from(bdz)), bi_mul(bi_from(adz), bi_from(bdy)));
  const BI det = bi_add(bi_add(bi_mul(bi_from(adx), m1), bi_mul(bi_from(bdx), m2)), bi_mul(bi_from(cdx), m3));
  return bi_sign(det);
}
__device__ int orient3d(const Pt& a, const Pt& b, const Pt& c, const Pt& d, double ig) {
  const double adx = a.x - d.x, ady = a.y - d.y, adz = a.z - d.z;
  const double bdx = b.x - d.x, bdy = b.y - d.y, bdz = b.z - d.z;
  const double cdx = c.x - d.x, cdy = c.y - d.y, cdz = c.z - d.z;
  const double p1 = bdy * cdz, p2 = bdz * cdy, p3 = cdy * adz, p4 = cdz * ady, p5 = ady * bdz, p6 = adz * bdy;
  const double det = adx * (p1 - p2) + bdx * (p3 - p4) + cdx * (p5 - p6);
  const double perm = fabs(adx) * (fabs(p1) + fabs(p2)) + fabs(bdx) * (fabs(p3) + fabs(p4)) +
                      fabs(cdx) * (fabs(p5) + fabs(p6));
  const double bound = kO3Bound * perm;
  if (det > bound) return 1;
  if (-det > bound) return -1;
  return orient_x(a, b, c, d, ig);
}

// insphere(a, b, c, d, e) > 0 when e lies inside the sphere through a, b, c,
// d and orient3d(a, b, c, d) > 0 (the sign flips with the orientation).
__device__ __noinline__ int insphere_x(const Pt& a, const Pt& b, const Pt& c, const Pt& d, const Pt& e, double ig) {
  const long long ex = ival(e.x, ig), ey = ival(e.y, ig), ez = ival(e.z, ig);
  const long long aex = ival(a.x, ig) - ex, aey = ival(a.y, ig) - ey, aez = ival(a.z, ig) - ez;
  const long long bex = ival(b.x, ig) - ex, bey = ival(b.y, ig) - ey, bez = ival(b.z, ig) - ez;
  const long long cex = ival(c.x, ig) - ex, cey = ival(c.y, ig) - ey, cez = ival(c.z, ig) - ez;
  const long long dex = ival(d.x, ig) - ex, dey = ival(d.y, ig) - ey, dez = ival(d.z, ig) - ez;
  auto M = [](long long p, long long q) { return bi_mul(bi_from(p), bi_from(q)); };
  auto lift = [&](long long x, long long y, long long z) { return bi_add(bi_add(M(x, x), M(y, y)), M(z, z)); };
  const BI ab = bi_sub(M(aex, bey), M(bex, aey)), bc = bi_sub(M(bex, cey), M(cex, bey));
  const BI cd = bi_sub(M(cex, dey), M(dex, cey)), da = bi_sub(M(dex, aey), M(aex, dey));
  const BI ac = bi_sub(M(aex, cey), M(cex, aey)), bd = bi_sub(M(bex, dey), M(dex, bey));
  const BI az = bi_from(aez), bz = bi_from(bez), cz = bi_from(cez), dz = bi_from(dez);
  const BI abc = bi_add(bi_sub(bi_mul(az, bc), bi_mul(bz, ac)), bi_mul(cz, ab));
  const BI bcd = bi_add(bi_sub(bi_mul(bz, cd), bi_mul(cz, bd)), bi_mul(dz, bc));
  const BI cda = bi_add(bi_add(bi_mul(cz, da), bi_mul(dz, ac)), bi_mul(az, cd));
  const BI dab = bi_add(bi_add(bi_mul(dz, ab), bi_mul(az, bd)), bi_mul(bz, da));
  const BI det = bi_add(bi_sub(bi_mul(lift(dex, dey, dez), abc), bi_mul(lift(cex, cey, cez), dab)),
                        bi_sub(bi_mul(lift(bex, bey, bez), cda), bi_mul(lift(aex, aey, aez), bcd)));
  return bi_sign(det);
}
__device__ int insphere(const Pt& a, const Pt& b, const Pt& c, const Pt& d, const Pt& e, double ig) {
  const double aex = a.x - e.x, aey = a.y - e.y, aez = a.z - e.z;
  const double bex = b.x - e.x, bey = b.y - e.y, bez = b.z - e.z;
  const double cex = c.x - e.x, cey = c.y - e.y, cez = c.z - e.z;
  const double dex = d.x - e.x, dey = d.y - e.y, dez = d.z - e.z;
  const double ab1 = aex * bey, ab2 = bex * aey, bc1 = bex * cey, bc2 = cex * bey;
  const double cd1 = cex * dey, cd2 = dex * cey, da1 = dex * aey, da2 = aex * dey;
  const double ac1 = aex * cey, ac2 = cex * aey, bd1 = bex * dey, bd2 = dex * bey;
  const double ab = ab1 - ab2, bc = bc1 - bc2, cd = cd1 - cd2, da = da1 - da2, ac = ac1 - ac2, bd = bd1 - bd2;
  const double abc = aez * bc - bez * ac + cez * ab;
  const double bcd = bez * cd - cez * bd + dez * bc;
  const double cda = cez * da + dez * ac + aez * cd;
  const double dab = dez * ab + aez * bd + bez * da;
  const double al = aex * aex + aey * aey + aez * aez, bl = bex * bex + bey * bey + bez * bez;
  const double cl = cex * cex + cey * cey + cez * cez, dl = dex * dex + dey * dey + dez * dez;
  const double det = (dl * abc - cl * dab) + (bl * cda - al * bcd);
  const double Pab = fabs(ab1) + fabs(ab2), Pbc = fabs(bc1) + fabs(bc2), Pcd = fabs(cd1) + fabs(cd2);
  const double Pda = fabs(da1) + fabs(da2), Pac = fabs(ac1) + fabs(ac2), Pbd = fabs(bd1) + fabs(bd2);
  const double Pabc = fabs(aez) * Pbc + fabs(bez) * Pac + fabs(cez) * Pab;
  const double Pbcd = fabs(bez) * Pcd + fabs(cez) * Pbd + fabs(dez) * Pbc;
  const double Pcda = fabs(cez) * Pda + fabs(dez) * Pac + fabs(aez) * Pcd;
  const double Pdab = fabs(dez) * Pab + fabs(aez) * Pbd + fabs(bez) * Pda;
  const double perm = dl * Pabc + cl * Pdab + bl * Pcda + al * Pbcd;
  const double bound = kIsBound * perm;
  if (det > bound) return 1;
  if (-det > bound) return -1;
  return insphere_x(a, b, c, d, e, ig);
}

// ------------------------------------------------------------ tet geometry
// Canonical evaluation over the ascending ids p[0] < p[1] < p[2] < p[3]:
// A_k = P_k - P_3, det = A_0 . (A_1 x A_2), circumcentre P_3 + c.
struct TetGeo {
  double A[3][3], det, c[3], rc, vol_scale;
};
__device__ inline void cross3(const double* u, const double* v, double* w) {
  w[0] = u[1] * v[2] - u[2] * v[1];
  w[1] = u[2] * v[0] - u[0] * v[2];
  w[2] = u[0] * v[1] - u[1] * v[0];
}
__device__ inline double dot3(const double* u, const double* v) { return u[0] * v[0] + u[1] * v[1] + u[2] * v[2]; }

__device__ void tet_geo(const Pt* P, TetGeo& g) {
  const double* p3 = &P[3].x;
  for (int k = 0; k < 3; k++) {
    const double* pk = &P[k].x;
    for (int q = 0; q < 3; q++) g.A[k][q] = pk[q] - p3[q];
  }
  double x12[3], x20[3], x01[3];
  cross3(g.A[1], g.A[2], x12);
  cross3(g.A[2], g.A[0], x20);
  cross3(g.A[0], g.A[1], x01);
  g.det = dot3(g.A[0], x12);
  const double r0 = 0.5 * dot3(g.A[0], g.A[0]), r1 = 0.5 * dot3(g.A[1], g.A[1]), r2 = 0.5 * dot3(g.A[2], g.A[2]);
  for (int q = 0; q < 3; q++) g.c[q] = (r0 * x12[q] + r1 * x20[q] + r2 * x01[q]) / g.det;
  g.rc = sqrt(dot3(g.c, g.c));
  g.vol_scale = sqrt(dot3(g.A[0], g.A[0])) * sqrt(dot3(g.A[1], g.A[1])) * sqrt(dot3(g.A[2], g.A[2]));
}

// Circumsphere inside the certificate ball of the particle at x with
// smoothing length h; flat tets (|det| below 1e-6 of the edge-length
// product) are never certified.
__device__ inline bool tet_in_ball(const TetGeo& g, const Pt* P, const double* x, double h, double cutoff) {
  if (!(fabs(g.det) >= 1.e-6 * g.vol_scale)) return false;
  double v[3];
  const double* p3 = &P[3].x;
  for (int q = 0; q < 3; q++) v[q] = p3[q] + g.c[q] - x[q];
  return sqrt(dot3(v, v)) + g.rc <= cutoff * h * (1.0 - 1.e-6);
}

__device__ inline void sort4(int* v) {
  for (int a = 1; a < 4; a++)
    for (int b = a; b > 0 && v[b - 1] > v[b]; b--) {
      const int t = v[b];
      v[b] = v[b - 1];
      v[b - 1] = t;
    }
}

struct TetIn {
  long long n;
  int cap;
  const double* x;  // snapped positions (n x 3)
  const int* type;
  const double* h;
  const int* rows;  // n x cap ids (list order; self may appear)
  const int* cnt;
  double inv_g;  // 1 / grid
  double cutoff;
  double thres;  // tet_delete_thres
};

__device__ inline Pt load_pt(const TetIn& T, int j) {
  const double* p = T.x + 3 * (long long)j;
  return Pt{p[0], p[1], p[2]};
}

// aspect = longest edge / smallest height (Check_whether_this_tet_should_be_delete,
// graph_mesh.cpp:900-970): longest edge * max_k |grad lambda_k|
__device__ double tet_aspect(const TetGeo& g, const Pt* P) {
  double n[4][3];
  cross3(g.A[1], g.A[2], n[0]);
  cross3(g.A[2], g.A[0], n[1]);
  cross3(g.A[0], g.A[1], n[2]);
  for (int k = 0; k < 3; k++)
    for (int q = 0; q < 3; q++) n[k][q] /= g.det;
  for (int q = 0; q < 3; q++) n[3][q] = -n[0][q] - n[1][q] - n[2][q];
  double hmax = 0.0;
  for (int k = 0; k < 4; k++) hmax = fmax(hmax, sqrt(dot3(n[k], n[k])));
  double e[3], longlen = 0.0;
  for (int k = 0; k < 3; k++) longlen = fmax(longlen, dot3(g.A[k], g.A[k]));
  const double* p0 = &P[0].x;
  const double* p1 = &P[1].x;
  const double* p2 = &P[2].x;
  for (int q = 0; q < 3; q++) e[q] = p1[q] - p0[q];
  longlen = fmax(longlen, dot3(e, e));
  for (int q = 0; q < 3; q++) e[q] = p2[q] - p1[q];
  longlen = fmax(longlen, dot3(e, e));
  for (int q = 0; q < 3; q++) e[q] = p0[q] - p2[q];
  longlen = fmax(longlen, dot3(e, e));
  return sqrt(longlen) * hmax;
}

constexpr int kMaxStar = 128;  // tets around one particle
constexpr int kMaxLink = 224;  // link edges around one particle
constexpr int kMaxOut = kMaxStar;  // tets emitted by one particle (at most its star)
// flags: 2 emit overflow, 4 spilled neighbour row (a star that outgrows
// kMaxStar / kMaxLink stops its walk and is counted in stats[3])

constexpr unsigned kFull = 0xffffffffu;

// FP32 pre-tests relative to particle i (w = d - x_i): they decide a
// candidate only when the FP32 value clears a bound far above its rounding
// error (and above the FP64 error of the circumcentre they use); the rest
// go to the exact predicates, so every decision equals the exact one.
struct Rel {
  float x, y, z, n;  // w and |w|
};
__device__ inline Rel rel(const Pt& p, const Pt& pi) {
  const float x = (float)(p.x - pi.x), y = (float)(p.y - pi.y), z = (float)(p.z - pi.z);
  return Rel{x, y, z, sqrtf(x * x + y * y + z * z)};
}
// Centre c (relative to i) of the sphere through i, a, b, d, and whether it
// is well enough conditioned (|det| >= 1e-3 |A||B||C|) for the pre-test.
__device__ bool sphere_rel(const Pt& pi, const Pt& pa, const Pt& pb, const Pt& pd, float* c, float* cn) {
  const double A[3] = {pa.x - pi.x, pa.y - pi.y, pa.z - pi.z}, B[3] = {pb.x - pi.x, pb.y - pi.y, pb.z - pi.z};
  const double C[3] = {pd.x - pi.x, pd.y - pi.y, pd.z - pi.z};
  double bc[3], ca[3], ab[3];
  cross3(B, C, bc);
  cross3(C, A, ca);
  cross3(A, B, ab);
  const double det = dot3(A, bc);
  const double la = dot3(A, A), lb = dot3(B, B), lc = dot3(C, C);
  if (!(fabs(det) >= 1.e-3 * sqrt(la) * sqrt(lb) * sqrt(lc))) return false;
  double q = 0.0;
  for (int k = 0; k < 3; k++) {
    const double v = (la * bc[k] + lb * ca[k] + lc * ab[k]) / (2.0 * det);
    c[k] = (float)v;
    q += v * v;
  }
  *cn = (float)sqrt(q);
  return true;
}
// +1 inside, -1 outside, 0 undecided: the power |w|^2 - 2 w.c of a sphere
// through i
__device__ inline int power_test(const Rel& w, const float* c, float cn) {
  const float p = w.n * w.n - 2.0f * (w.x * c[0] + w.y * c[1] + w.z * c[2]);
  const float sl = 1.e-5f * (w.n * w.n + 2.0f * w.n * cn);
  return p > sl ? -1 : (p < -sl ? 1 : 0);
}

// Gift-wraps the face (i, a, b) to side s (s * orient3d(i, a, b, d) > 0),
// one warp over the row: the candidate whose sphere through i, a, b holds
// no other candidate.  Along the pencil of spheres through the face's
// circle, "e inside the sphere of d" orders the candidates, so each lane
// takes the first of its share and a shuffle reduction the first of all.
// Returns -1 (on every lane) when no row particle lies on that side.
__device__ int wrap(const TetIn& T, const int* S, int m, const Pt& pi, const Pt& pa, const Pt& pb, int i, int a,
                    int b, int s, int lane) {
  // orient3d(i, a, b, d) = -((a - i) x (b - i)) . (d - i)
  float nf[3], nfn;
  {
    const double A[3] = {pa.x - pi.x, pa.y - pi.y, pa.z - pi.z}, B[3] = {pb.x - pi.x, pb.y - pi.y, pb.z - pi.z};
    double n[3];
    cross3(A, B, n);
    nf[0] = (float)n[0]; nf[1] = (float)n[1]; nf[2] = (float)n[2];
    nfn = (float)sqrt(dot3(n, n));
  }
  int best = -1;
  Pt pbest{0, 0, 0};
  float c[3] = {0.f, 0.f, 0.f}, cn = 0.f;
  bool hc = false;
  for (int q = lane; q < m; q += 32) {
    const int d = S[q];
    if (d == i || d == a || d == b) continue;
    const Pt pd = load_pt(T, d);
    const Rel w = rel(pd, pi);
    const float o = nf[0] * w.x + nf[1] * w.y + nf[2] * w.z, ob = 1.e-5f * nfn * w.n;
    const int side = o > ob ? -1 : (o < -ob ? 1 : orient3d(pi, pa, pb, pd, T.inv_g));
    if (s * side <= 0) continue;
    bool take = best < 0;
    if (!take) {
      const int pt = hc ? power_test(w, c, cn) : 0;
      take = pt != 0 ? pt > 0 : s * insphere(pi, pa, pb, pbest, pd, T.inv_g) > 0;
    }
    if (take) {
      best = d;
      pbest = pd;
      hc = sphere_rel(pi, pa, pb, pd, c, &cn);
    }
  }
  // shuffle reduction; a lane whose partner lies past the warp gets its own
  // candidate back, which is never compared with itself
  for (int off = 16; off > 0; off >>= 1) {
    const int ob = __shfl_down_sync(kFull, best, off);
    const Pt po{__shfl_down_sync(kFull, pbest.x, off), __shfl_down_sync(kFull, pbest.y, off),
                __shfl_down_sync(kFull, pbest.z, off)};
    const float oc0 = __shfl_down_sync(kFull, c[0], off), oc1 = __shfl_down_sync(kFull, c[1], off);
    const float oc2 = __shfl_down_sync(kFull, c[2], off), ocn = __shfl_down_sync(kFull, cn, off);
    const bool ohc = __shfl_down_sync(kFull, (int)hc, off) != 0;
    if (ob < 0 || ob == best) continue;
    bool take = best < 0;
    if (!take) {
      const int pt = hc ? power_test(rel(po, pi), c, cn) : 0;
      take = pt != 0 ? pt > 0 : s * insphere(pi, pa, pb, pbest, po, T.inv_g) > 0;
    }
    if (take) {
      best = ob;
      pbest = po;
      c[0] = oc0; c[1] = oc1; c[2] = oc2; cn = ocn; hc = ohc;
    }
  }
  return __shfl_sync(kFull, best, 0);
}

// Status of tet (i, a, b, d) for particle i: 0 when a row particle lies
// inside or on its sphere (or the four are coplanar), 1 when none does (a
// tet of the row's Delaunay tetrahedralisation), 2 when moreover the sphere
// lies inside i's ball and the tet is not flat (certified: a Delaunay tet
// of all particles).  *degen is set when row particles lie on the sphere
// and none inside it.  Warp-uniform result.
__device__ int tet_status(const TetIn& T, const int* S, int m, int i, int a, int b, int d, const double* xi,
                          double hi, bool* degen, int lane) {
  int v[4] = {i, a, b, d};
  sort4(v);
  Pt P[4];
  for (int k = 0; k < 4; k++) P[k] = load_pt(T, v[k]);
  TetGeo g;
  tet_geo(P, g);
  const int o = orient3d(P[0], P[1], P[2], P[3], T.inv_g);
  if (o == 0) return 0;
  // the sphere's centre relative to i (the pre-test needs |det| >= 1e-3 of the edge product)
  const bool hc = fabs(g.det) >= 1.e-3 * g.vol_scale;
  float c[3];
  double cq = 0.0;
  for (int k = 0; k < 3; k++) {
    const double* p3 = &P[3].x;
    const double v3 = p3[k] + g.c[k] - xi[k];
    c[k] = (float)v3;
    cq += v3 * v3;
  }
  const float cn = (float)sqrt(cq);
  const Pt pi{xi[0], xi[1], xi[2]};
  bool inside = false, on = false;
  for (int q = lane; q < m && !inside; q += 32) {
    const int e = S[q];
    if (e == v[0] || e == v[1] || e == v[2] || e == v[3]) continue;
    const Pt pe = load_pt(T, e);
    const int pt = hc ? power_test(rel(pe, pi), c, cn) : 0;
    const int sg = pt != 0 ? pt : o * insphere(P[0], P[1], P[2], P[3], pe, T.inv_g);
    if (sg > 0) inside = true;
    else if (sg == 0) on = true;
  }
  const bool any_in = __any_sync(kFull, inside), any_on = __any_sync(kFull, on);
  if (any_in || any_on) {
    if (!any_in) *degen = true;
    return 0;
  }
  return tet_in_ball(g, P, xi, hi, T.cutoff) ? 2 : 1;
}

constexpr int kStarWarps = 4;  // warps (particles) per block of k_tet_star

// One warp per particle (grid-stride): its certified star, the tets it
// emits (ascending ids, in star order) into out[i * kMaxOut ...], their
// number into count[i].  stats: [0] open stars, [1] deleted tets, [2] ties,
// [3] stars cut at the per-particle limits.
__global__ void __launch_bounds__(32 * kStarWarps) k_tet_star(TetIn T, int* __restrict__ out,
                                                              int* __restrict__ count, unsigned long long* stats,
                                                              unsigned* flags) {
  __shared__ int s_star[kStarWarps][kMaxStar][3];
  __shared__ int s_le[kStarWarps][kMaxLink][2];
  __shared__ unsigned char s_done[kStarWarps][kMaxLink];
  __shared__ unsigned char s_cert[kStarWarps][kMaxStar];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int(*star)[3] = s_star[wib];
  unsigned char* cert = s_cert[wib];
  int(*le)[2] = s_le[wib];
  unsigned char* ldone = s_done[wib];
  const long long nwarps = (long long)gridDim.x * kStarWarps;
  for (long long i64 = (long long)blockIdx.x * kStarWarps + wib; i64 < T.n; i64 += nwarps) {
    const int i = (int)i64;
    const int* S = T.rows + i64 * T.cap;
    const int m = T.cnt[i];
    const Pt pi = load_pt(T, i);
    const double xi[3] = {pi.x, pi.y, pi.z};
    const double hi = T.h[i];
    bool degen = false, open = false, trunc = false;
    int ns = 0, nl = 0;
    // 1. nearest neighbour a (ties: lower id) and the third point c of the
    // smallest circumcircle through i and a (ties: lower id)
    double best = 1.e300;
    int a = 0x7fffffff;
    for (int q = lane; q < m; q += 32) {
      const int j = S[q];
      if (j == i) continue;
      const Pt pj = load_pt(T, j);
      const double dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
      const double d2 = dx * dx + dy * dy + dz * dz;
      if (d2 < best || (d2 == best && j < a)) { a = j; best = d2; }
    }
    for (int off = 16; off > 0; off >>= 1) {
      const double ob = __shfl_down_sync(kFull, best, off);
      const int oa = __shfl_down_sync(kFull, a, off);
      if (ob < best || (ob == best && oa < a)) { a = oa; best = ob; }
    }
    a = __shfl_sync(kFull, a, 0);
    int c = 0x7fffffff;
    if (a != 0x7fffffff) {
      const Pt pa = load_pt(T, a);
      const double u[3] = {pa.x - pi.x, pa.y - pi.y, pa.z - pi.z};
      const double uu = dot3(u, u);
      double bestr = 1.e300;
      for (int q = lane; q < m; q += 32) {
        const int j = S[q];
        if (j == i || j == a) continue;
        const Pt pj = load_pt(T, j);
        const double v[3] = {pj.x - pi.x, pj.y - pi.y, pj.z - pi.z}, w[3] = {v[0] - u[0], v[1] - u[1], v[2] - u[2]};
        double x[3];
        cross3(u, v, x);
        const double xx = dot3(x, x);
        if (!(xx > 0.0)) continue;
        const double r2 = uu * dot3(v, v) * dot3(w, w) / (4.0 * xx);
        if (r2 < bestr || (r2 == bestr && j < c)) { c = j; bestr = r2; }
      }
      for (int off = 16; off > 0; off >>= 1) {
        const double ob = __shfl_down_sync(kFull, bestr, off);
        const int oc = __shfl_down_sync(kFull, c, off);
        if (ob < bestr || (ob == bestr && oc < c)) { c = oc; bestr = ob; }
      }
      c = __shfl_sync(kFull, c, 0);
    }
    // 2. first tet: the face (i, a, c) wrapped to either side
    if (c != 0x7fffffff) {
      const Pt pa = load_pt(T, a), pc = load_pt(T, c);
      for (int s = 1; s >= -1 && ns == 0; s -= 2) {
        const int d = wrap(T, S, m, pi, pa, pc, i, a, c, s, lane);
        const int st = d >= 0 ? tet_status(T, S, m, i, a, c, d, xi, hi, &degen, lane) : 0;
        if (st > 0) {
          if (lane == 0) {
            star[0][0] = s > 0 ? a : c;
            star[0][1] = s > 0 ? c : a;
            star[0][2] = d;
            cert[0] = st == 2;
          }
          ns = 1;
        }
      }
    }
    __syncwarp();
    if (ns == 0) open = true;
    // 3. breadth-first over the link, through every tet of the row's
    // Delaunay tetrahedralisation around i (certified or not, so that the
    // whole star is reached): every tet (x, y, z) is stored with
    // orient3d(i, x, y, z) > 0; its link edges (x, y), (y, z), (z, x) lead
    // to the tets across the faces (i, x, y) ...  (warp-uniform; lane 0 writes)
    int head = 0;
    while (true) {
      for (; head < ns; head++) {
        for (int k = 0; k < 3; k++) {
          const int u = star[head][k], v = star[head][(k + 1) % 3];
          int f = -1;
          for (int q = 0; q < nl; q++)
            if ((le[q][0] == u && le[q][1] == v) || (le[q][0] == v && le[q][1] == u)) { f = q; break; }
          if (f >= 0) {
            if (lane == 0) ldone[f] = 1;
          } else if (nl < kMaxLink) {
            if (lane == 0) { le[nl][0] = u; le[nl][1] = v; ldone[nl] = 0; }
            nl++;
          } else {
            trunc = true;
          }
          __syncwarp();
        }
      }
      if (trunc) break;
      int f = -1;
      for (int q = 0; q < nl; q++)
        if (!ldone[q]) { f = q; break; }
      if (f < 0) break;
      const int u = le[f][0], v = le[f][1];
      __syncwarp();
      if (lane == 0) ldone[f] = 1;
      __syncwarp();
      const Pt pu = load_pt(T, u), pv = load_pt(T, v);
      // the stored tet (u, v, w) has orient3d(i, u, v, w) > 0: wrap to the other side
      const int d = wrap(T, S, m, pi, pu, pv, i, u, v, -1, lane);
      const int st = d >= 0 ? tet_status(T, S, m, i, u, v, d, xi, hi, &degen, lane) : 0;
      if (st == 0) {
        open = true;
        continue;
      }
      bool dup = false;
      for (int q = 0; q < ns && !dup; q++) {
        const int* t = star[q];
        const bool hu = t[0] == u || t[1] == u || t[2] == u, hv = t[0] == v || t[1] == v || t[2] == v;
        const bool hd = t[0] == d || t[1] == d || t[2] == d;
        dup = hu && hv && hd;
      }
      if (dup) continue;
      if (ns == kMaxStar) {
        trunc = true;
        break;
      }
      if (lane == 0) { star[ns][0] = v; star[ns][1] = u; star[ns][2] = d; cert[ns] = st == 2; }  // orient3d(i, v, u, d) > 0
      ns++;
      __syncwarp();
    }
    // 4. emit the tets whose lowest-id holding ball is i's (lanes over the
    // star, compacted in star order); apply the deletion rule
    int ne = 0;
    unsigned long long ndel = 0;
    for (int base = 0; base < ns; base += 32) {
      const int q = base + lane;
      bool emit = false, del = false;
      int v[4] = {0, 0, 0, 0};
      if (q < ns && cert[q]) {
        v[0] = i; v[1] = star[q][0]; v[2] = star[q][1]; v[3] = star[q][2];
        sort4(v);
        Pt P[4];
        for (int k = 0; k < 4; k++) P[k] = load_pt(T, v[k]);
        TetGeo g;
        tet_geo(P, g);
        int owner = -1;
        for (int k = 0; k < 4 && owner < 0; k++) {
          const double xv[3] = {P[k].x, P[k].y, P[k].z};
          if (tet_in_ball(g, P, xv, T.h[v[k]], T.cutoff)) owner = v[k];
        }
        if (owner == i) {
          const bool all_boundary =
              T.type[v[0]] != 0 && T.type[v[1]] != 0 && T.type[v[2]] != 0 && T.type[v[3]] != 0;
          if (all_boundary && tet_aspect(g, P) > T.thres) del = true;
          else emit = true;
        }
      }
      const unsigned em = __ballot_sync(kFull, emit);
      ndel += __popc(__ballot_sync(kFull, del));
      if (emit) {
        int* o = out + (i64 * kMaxOut + ne + __popc(em & ((1u << lane) - 1u))) * 4;
        for (int k = 0; k < 4; k++) o[k] = v[k];
      }
      ne += __popc(em);
    }
    if (lane == 0) {
      count[i] = ne;
      if (open) atomicAdd(&stats[0], 1ull);
      if (ndel) atomicAdd(&stats[1], ndel);
      if (degen) atomicAdd(&stats[2], 1ull);
      if (trunc) atomicAdd(&stats[3], 1ull);
    }
    __syncwarp();
  }
}

// Snap to the grid: x' = rint(x / g) g (g a power of two, |x / g| < 2^52).
__global__ void k_tet_snap(long long n3, double* __restrict__ x, double inv_g, double g) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n3) x[k] = rint(x[k] * inv_g) * g;
}

__global__ void k_tet_compact(long long n, const int* __restrict__ src, const int* __restrict__ count,
                              const int* __restrict__ off, int* __restrict__ tets) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = count[i];
  const long long o = off[i];
  for (int k = 0; k < 4 * c; k++) tets[4 * o + k] = src[i * kMaxOut * 4 + k];
}

// ------------------------------------------------------------ quality
struct TetStat {
  double vol, vmin, vmax, emin2, emax2, amin, amax, asum, rmin, rmax, rsum, dmin, dmax, dsum;
};
struct TetQIn {
  const double* x;
  const int* tets;
  long long ntet;
  const double* cos_dihed;  // cos(4 k degrees), k = 0..45
  const double* cos_small;  // cos(10, 20, 30, 40 degrees)
  unsigned long long* hist;  // aspect 12, radius 56, dihedral 45, small-dihedral 4
};
constexpr int kAspectBins = 12, kRadiusBins = 56, kDihedBins = 45;
// degrees as the reference converts them: acos(x) / PI * 180 with its PI (glbparam.h:186)
constexpr double kPiRef = 3.1415926;

__device__ void tet_quality_one(const TetQIn& Q, long long t, TetStat& s) {
  Pt P[4];
  for (int k = 0; k < 4; k++) {
    const double* p = Q.x + 3 * (long long)Q.tets[4 * t + k];
    P[k] = Pt{p[0], p[1], p[2]};
  }
  TetGeo g;
  tet_geo(P, g);
  double n[4][3], H[4];
  cross3(g.A[1], g.A[2], n[0]);
  cross3(g.A[2], g.A[0], n[1]);
  cross3(g.A[0], g.A[1], n[2]);
  for (int k = 0; k < 3; k++)
    for (int q = 0; q < 3; q++) n[k][q] /= g.det;
  for (int q = 0; q < 3; q++) n[3][q] = -n[0][q] - n[1][q] - n[2][q];
  double hsum = 0.0, hmax = 0.0;
  for (int k = 0; k < 4; k++) {
    H[k] = sqrt(dot3(n[k], n[k]));
    hsum += H[k];
    hmax = fmax(hmax, H[k]);
    for (int q = 0; q < 3; q++) n[k][q] /= H[k];
  }
  double e2[6], e[3];
  for (int k = 0; k < 3; k++) e2[k] = dot3(g.A[k], g.A[k]);
  const double* p0 = &P[0].x;
  const double* p1 = &P[1].x;
  const double* p2 = &P[2].x;
  for (int q = 0; q < 3; q++) e[q] = p1[q] - p0[q];
  e2[3] = dot3(e, e);
  for (int q = 0; q < 3; q++) e[q] = p2[q] - p1[q];
  e2[4] = dot3(e, e);
  for (int q = 0; q < 3; q++) e[q] = p0[q] - p2[q];
  e2[5] = dot3(e, e);
  double lo = e2[0], hi = e2[0];
  for (int k = 1; k < 6; k++) { lo = fmin(lo, e2[k]); hi = fmax(hi, e2[k]); }
  const double vol = fabs(g.det) / 6.0;
  const double aspect = sqrt(hi) * hmax;
  const double ratio = 3.0 * (1.0 / hsum) / g.rc;
  s.vol += vol;
  s.vmin = fmin(s.vmin, vol);
  s.vmax = fmax(s.vmax, vol);
  s.emin2 = fmin(s.emin2, lo);
  s.emax2 = fmax(s.emax2, hi);
  s.amin = fmin(s.amin, aspect);
  s.amax = fmax(s.amax, aspect);
  s.asum += aspect;
  s.rmin = fmin(s.rmin, ratio);
  s.rmax = fmax(s.rmax, ratio);
  s.rsum += ratio;
  // aspect histogram (aspectratiotable, graph_mesh.cpp:2037-2042, 2349-2353)
  const double tab[11] = {1.5, 2.0, 2.5, 3.0, 4.0, 6.0, 10.0, 15.0, 25.0, 50.0, 100.0};
  int ai = 0;
  while (ai < 11 && aspect > tab[ai]) ai++;
  atomicAdd(&Q.hist[ai], 1ull);
  const double rq = floor(ratio / 0.02);
  const int ri = rq >= 0.0 ? (rq < kRadiusBins - 1 ? (int)rq : kRadiusBins - 1) : 0;
  atomicAdd(&Q.hist[kAspectBins + ri], 1ull);
  // dihedral angles at the six edges: cos = -n_a . n_b
  const int pa[6] = {0, 0, 0, 1, 1, 2}, pb[6] = {1, 2, 3, 2, 3, 3};
  double cmax = -2.0, cmin = 2.0;
  for (int k = 0; k < 6; k++) {
    double cs = -dot3(n[pa[k]], n[pb[k]]);
    cs = fmin(1.0, fmax(-1.0, cs));
    cmax = fmax(cmax, cs);  // smallest angle
    cmin = fmin(cmin, cs);  // largest angle
    int b = 0;
    while (b < kDihedBins - 1 && cs <= Q.cos_dihed[b + 1]) b++;
    atomicAdd(&Q.hist[kAspectBins + kRadiusBins + b], 1ull);
  }
  for (int k = 0; k < 4; k++)
    if (cmax > Q.cos_small[k]) atomicAdd(&Q.hist[kAspectBins + kRadiusBins + kDihedBins + k], 1ull);
  const double dsmall = acos(cmax) / kPiRef * 180.0, dbig = acos(cmin) / kPiRef * 180.0;
  s.dmin = fmin(s.dmin, dsmall);
  s.dmax = fmax(s.dmax, dbig);
  s.dsum += dsmall;
}

__device__ inline void stat_init(TetStat& s) {
  s.vol = s.asum = s.rsum = s.dsum = 0.0;
  s.vmin = s.emin2 = s.amin = s.rmin = s.dmin = 1.e300;
  s.vmax = s.emax2 = s.amax = s.rmax = s.dmax = 0.0;
}
__device__ inline void stat_fold(TetStat& a, const TetStat& b) {
  a.vol += b.vol; a.asum += b.asum; a.rsum += b.rsum; a.dsum += b.dsum;
  a.vmin = fmin(a.vmin, b.vmin); a.emin2 = fmin(a.emin2, b.emin2); a.amin = fmin(a.amin, b.amin);
  a.rmin = fmin(a.rmin, b.rmin); a.dmin = fmin(a.dmin, b.dmin);
  a.vmax = fmax(a.vmax, b.vmax); a.emax2 = fmax(a.emax2, b.emax2); a.amax = fmax(a.amax, b.amax);
  a.rmax = fmax(a.rmax, b.rmax); a.dmax = fmax(a.dmax, b.dmax);
}

// 256 threads, one partial per block folded in thread order (deterministic)
__global__ void __launch_bounds__(256) k_tet_quality(TetQIn Q, TetStat* part) {
  __shared__ TetStat sh[256];
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  TetStat s;
  stat_init(s);
  if (t < Q.ntet) tet_quality_one(Q, t, s);
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) stat_fold(sh[threadIdx.x], sh[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}
__global__ void k_tet_quality_fold(const TetStat* part, int nblk, TetStat* out) {
  TetStat s;
  stat_init(s);
  for (int b = 0; b < nblk; b++) stat_fold(s, part[b]);
  *out = s;
}

int tfail(mrsph_handle* h, int code, const std::string& m) {
  h->err = m;
  return code;
}

}  // namespace
}  // namespace mrsph

using namespace mrsph;

extern "C" int mrsph_tetrahedralize(mrsph_handle* h, int* tets, long long cap, long long* ntet_out,
                                    mrsph_tet_quality* q) {
  if (!h) return MRSPH_ERR_ARG;
  if (!h->eng) return tfail(h, MRSPH_ERR_STATE, "mrsph_set_levelset must come first");
  if (h->prm.dim != 3) return tfail(h, MRSPH_ERR_ARG, "tetrahedralisation is 3D only");
  if (cudaSetDevice(h->prm.device) != cudaSuccess) return tfail(h, MRSPH_ERR_CUDA, "cudaSetDevice failed");
  const long long n = h->eng->num_particles();
  if (n <= 0) return tfail(h, MRSPH_ERR_STATE, "no particles");
  if (n > 0x7fffffffLL / kMaxOut) return tfail(h, MRSPH_ERR_RANGE, "too many particles for one tetrahedralisation");
  const int rowcap = h->eng->neighbor_capacity();
  cudaStream_t s = h->stream;
  std::vector<void*> mem;
  int rc = 0;
  auto A = [&](void** p, size_t bytes) -> bool {
    if (cudaMalloc(p, bytes) != cudaSuccess) return false;
    mem.push_back(*p);
    return true;
  };
  // grid 2^(e-52) with 2^e above every |coordinate| of the domain
  double M = 1.0;
  for (int d = 0; d < 3; d++) M = std::fmax(M, std::fmax(std::fabs(h->prm.box_l[d]), std::fabs(h->prm.box_r[d])));
  int e = 0;
  std::frexp(M, &e);  // M < 2^e
  e += 1;
  const double g = std::ldexp(1.0, e - 52), inv_g = std::ldexp(1.0, 52 - e);
  double *d_x = nullptr, *d_phi = nullptr, *d_h = nullptr, *d_cos = nullptr;
  int *d_type = nullptr, *d_rows = nullptr, *d_cnt = nullptr, *d_out = nullptr, *d_count = nullptr;
  int *d_off = nullptr, *d_blk = nullptr, *d_tets = nullptr;
  unsigned* d_flags = nullptr;
  unsigned long long *d_stats = nullptr, *d_hist = nullptr;
  TetStat *d_part = nullptr, *d_tq = nullptr;
  const size_t NC = (size_t)n * rowcap;
  constexpr int kHist = kAspectBins + kRadiusBins + kDihedBins + 4;
  unsigned long long st[4] = {0, 0, 0, 0}, hist[kHist];
  std::memset(hist, 0, sizeof(hist));
  TetStat tq;
  std::memset(&tq, 0, sizeof(tq));
  long long ntet = 0;
  unsigned flags = 0;
  double cosv[50];
  for (int k = 0; k <= kDihedBins; k++) cosv[k] = std::cos(4.0 * k * kPiRef / 180.0);
  for (int k = 0; k < 4; k++) cosv[46 + k] = std::cos(10.0 * (k + 1) * kPiRef / 180.0);
  if (!A((void**)&d_x, sizeof(double) * 3 * n) || !A((void**)&d_phi, sizeof(double) * n) ||
      !A((void**)&d_h, sizeof(double) * n) || !A((void**)&d_type, sizeof(int) * n) ||
      !A((void**)&d_rows, sizeof(int) * NC) || !A((void**)&d_cnt, sizeof(int) * n) ||
      !A((void**)&d_out, sizeof(int) * 4 * kMaxOut * (size_t)n) || !A((void**)&d_count, sizeof(int) * (n + 1)) ||
      !A((void**)&d_off, sizeof(int) * (n + 1)) || !A((void**)&d_blk, sizeof(int) * scan_blocksums_size(n)) ||
      !A((void**)&d_flags, sizeof(unsigned)) || !A((void**)&d_stats, sizeof(st)) ||
      !A((void**)&d_hist, sizeof(hist)) || !A((void**)&d_cos, sizeof(cosv))) {
    rc = tfail(h, MRSPH_ERR_OOM, "cudaMalloc failed");
    goto done;
  }
  cudaMemsetAsync(d_flags, 0, sizeof(unsigned), s);
  cudaMemsetAsync(d_stats, 0, sizeof(st), s);
  cudaMemsetAsync(d_hist, 0, sizeof(hist), s);
  cudaMemcpyAsync(d_cos, cosv, sizeof(cosv), cudaMemcpyHostToDevice, s);
  rc = h->eng->export_tri(d_x, d_type, d_phi, d_rows, d_cnt, rowcap, d_flags, d_h, false);
  if (rc) { h->err = h->eng->err; goto done; }
  {
    const int nbN = (int)std::min<long long>((n + kStarWarps - 1) / kStarWarps, 152LL * 64);
    k_tet_snap<<<(int)((3 * n + 255) / 256), 256, 0, s>>>(3 * n, d_x, inv_g, g);
    TetIn T;
    T.n = n; T.cap = rowcap; T.x = d_x; T.type = d_type; T.h = d_h; T.rows = d_rows; T.cnt = d_cnt;
    T.inv_g = inv_g; T.cutoff = h->prm.cutoff; T.thres = 10.0;
    k_tet_star<<<nbN, 32 * kStarWarps, 0, s>>>(T, d_out, d_count, d_stats, d_flags);
    cell_scan(d_count, d_off, d_blk, n, 0, s);
    int tot = 0, last = 0;
    cudaMemcpyAsync(&tot, d_off + n - 1, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&last, d_count + n - 1, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&flags, d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(st, d_stats, sizeof(st), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) { rc = tfail(h, MRSPH_ERR_CUDA, "tetrahedralisation failed"); goto done; }
    ntet = (long long)tot + last;
    if (flags & 4u) { rc = tfail(h, MRSPH_ERR_RANGE, "neighbour list spilled; raise neighbor_cap"); goto done; }
    if (flags & 2u) { rc = tfail(h, MRSPH_ERR_RANGE, "a particle emits more tets than the kernel keeps"); goto done; }
    if (ntet > 0) {
      if (!A((void**)&d_tets, sizeof(int) * 4 * ntet)) { rc = tfail(h, MRSPH_ERR_OOM, "cudaMalloc failed"); goto done; }
      k_tet_compact<<<(int)((n + 255) / 256), 256, 0, s>>>(n, d_out, d_count, d_off, d_tets);
      const int nbT = (int)((ntet + 255) / 256);
      if (!A((void**)&d_part, sizeof(TetStat) * nbT) || !A((void**)&d_tq, sizeof(TetStat))) {
        rc = tfail(h, MRSPH_ERR_OOM, "cudaMalloc failed");
        goto done;
      }
      TetQIn Q;
      Q.x = d_x; Q.tets = d_tets; Q.ntet = ntet; Q.cos_dihed = d_cos; Q.cos_small = d_cos + 46; Q.hist = d_hist;
      k_tet_quality<<<nbT, 256, 0, s>>>(Q, d_part);
      k_tet_quality_fold<<<1, 1, 0, s>>>(d_part, nbT, d_tq);
      cudaMemcpyAsync(&tq, d_tq, sizeof(TetStat), cudaMemcpyDeviceToHost, s);
      cudaMemcpyAsync(hist, d_hist, sizeof(hist), cudaMemcpyDeviceToHost, s);
      if (tets && cap >= ntet) cudaMemcpyAsync(tets, d_tets, sizeof(int) * 4 * ntet, cudaMemcpyDeviceToHost, s);
    }
    cudaError_t err = cudaStreamSynchronize(s);
    if (err == cudaSuccess) err = cudaGetLastError();
    if (err != cudaSuccess) { rc = tfail(h, MRSPH_ERR_CUDA, std::string("tetrahedralisation: ") + cudaGetErrorString(err)); goto done; }
  }
  if (ntet_out) *ntet_out = ntet;
  if (q) {
    std::memset(q, 0, sizeof(*q));
    q->ntet = ntet;
    q->nopen = (long long)st[0];
    q->ndeleted = (long long)st[1];
    q->ntie = (long long)st[2];
    q->ntrunc = (long long)st[3];
    q->grid = g;
    if (ntet > 0) {
      q->total_volume = tq.vol; q->min_volume = tq.vmin; q->max_volume = tq.vmax;
      q->min_edge = std::sqrt(tq.emin2); q->max_edge = std::sqrt(tq.emax2);
      q->min_aspect = tq.amin; q->max_aspect = tq.amax; q->avg_aspect = tq.asum / ntet;
      q->min_radius_ratio = tq.rmin; q->max_radius_ratio = tq.rmax; q->avg_radius_ratio = tq.rsum / ntet;
      q->min_dihedral = tq.dmin; q->max_dihedral = tq.dmax; q->avg_min_dihedral = tq.dsum / ntet;
    }
    for (int k = 0; k < kAspectBins; k++) q->aspect_hist[k] = (long long)hist[k];
    for (int k = 0; k < kRadiusBins; k++) q->radius_hist[k] = (long long)hist[kAspectBins + k];
    for (int k = 0; k < kDihedBins; k++) q->dihedral_hist[k] = (long long)hist[kAspectBins + kRadiusBins + k];
    for (int k = 0; k < 4; k++) q->nsmall_dihedral[k] = (long long)hist[kAspectBins + kRadiusBins + kDihedBins + k];
  }
done:
  for (void* p : mem) cudaFree(p);
  return rc;
}
