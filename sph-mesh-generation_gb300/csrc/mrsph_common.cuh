// mrsph_common.cuh — device-side building blocks shared by the FP64-plain and
// FP32-split engines: geometry descriptors, Philox4x32-10, the SPH kernel
// functions and level-set sampling.
#pragma once
#include <cuda_runtime.h>

#include <type_traits>
#include <stdint.h>

namespace mrsph {

constexpr double PI_REF = 3.1415926;  // glbparam.h:186
constexpr int MAX_LS = 4;             // nested level-set levels
constexpr int MAX_CL = 8;             // cell-list levels

enum { REAL_P = 0, SURFACE_P = 1, SINGULARITY_P = 2, SEGMENT_P = 3 };
enum { K_HYP = 0, K_CUB = 1, K_WEN = 2, K_GAU = 3, K_QUI = 4 };
enum { CUT_CELL = 1 };
enum { FLAG_REMAP = 1, FLAG_SEED = 2, FLAG_LEVEL = 4, FLAG_SPILL = 8 };
enum { RNG_SEED = 1, RNG_REMAP = 2 };

// One nested level-set level on the device (dense, margins included).
struct LsLevel {
  double box_l[3], dpkg[3], dcell[3];
  double inv_dpkg[3], inv_dcell[3];  // FP32-split locates with products instead of divisions
  int num_pkg[3], margin, n[3];
  const double4* g64;  // (phi, nx, ny, nz)
  const double* c64;   // curvature
  const float4* g32;
  const float* c32;
  const uint8_t* tag;
  const uint8_t* active;  // per package incl. margins, or nullptr
  // characteristic cell (tag_characteristic + idx_characteristic): 0 none,
  // k + 1 on segment k, -(k + 1) at singularity k; nullptr without any
  const int* chr;
  // FP32-split location (set by the FP32 engine): per axis, for every anchor
  // cell k of the cell list, the package of the anchor's lower corner (.x)
  // and the corner's offset inside that package as FP32 bits (.y); FP32
  // copies of the package and cell sizes
  const int2* anc[3];
  float dpkg_f[3], inv_dpkg_f[3], inv_dcell_f[3];
};

struct LsSet {
  int nls;
  double max_phi, dl0, min_dl, max_dl;
  int law;                              // 0: tanh law of phi; 1: curvature law
  double middle_dl, max_curv, min_curv; // curvature law (|curv| range over CUT cells)
  float max_phi_f, dl0_f, min_dl_f, max_dl_f, middle_dl_f, max_curv_f, min_curv_f;  // FP32 copies
  LsLevel lv[MAX_LS];
  // the geometry's singularity points (3 each) and segments (6 each: first
  // point, second point; z = 0 in 2D), device copies
  int nsing, nseg;
  const double* sing;
  const double* seg;
};

// Cell-list levels (Level_info, level_infor.cpp:35-110): level 0 is the
// coarsest (scale = max_scale), level ncl-1 the finest.  Cells of level l are
// concatenated in one table at offset off[l], row-major (x fastest).
struct CellGeo {
  int ncl;
  double box_l[3];
  double max_scale, min_scale;
  float max_scale_f;
  int n[MAX_CL][3];
  double dcell[MAX_CL][3];
  long long off[MAX_CL + 1];
  double A[3];  // anchor cell of the FP32-split position = finest cell
  float Af[3];
  double ihs[MAX_CL][3];  // 1 / half-cell size (FP32-split keys)
  float ihs_f[MAX_CL][3];
  double idc0[3];         // 1 / level-0 cell size (local h maxima)
  float idc0_f[3];
  float hs_f[MAX_CL][3];  // FP32 half-cell size
  long long nc0;          // level-0 cells
  // sort table: half-size cells (2 per reference cell per axis), row-major per level
  int hn[MAX_CL][3];
  double hs[MAX_CL][3];  // half-cell size = dcell / 2
  long long hoff[MAX_CL + 1];
};

struct Params {
  int dim, kernel;
  double cell_ratio, cutoff, angle_thres, cos_thres, nu_coeff, damp_coeff;
  double box_l[3], box_r[3];
  unsigned long long seed;
  // FP32 copies (the FP32-split kernels read these, not conversions of the above)
  float cell_ratio_f, cutoff_f, cos_thres_f, nu_coeff_f, damp_coeff_f;
};

// Device scalars of a step.  Doubles are kept as their bit patterns so that
// min/max of non-negative values reduce exactly with integer atomics.
struct DevScalars {
  unsigned long long dt1, vmax1, dt2, vmax2, dt_adv;
  float dt_adv_f, hdt_adv_f;  // FP32 dt_adv and dt_adv / 2 (set with dt_adv at the start of a step)
  unsigned long long pairs;
  unsigned long long pairs_total;
  unsigned int remap, nsurf, flags, spill;
  unsigned int step;
  unsigned int maxcnt;  // largest neighbour count of the last density phase
  unsigned int nfix;    // FP32-split: particles queued for the exact re-decision of the density phase
  unsigned int nspill;  // particles whose neighbour list spilled (re-scanned by the force fix-up launches)
  unsigned long long hmax[MAX_CL];  // FP64 bits of the largest h per level (this step)
  unsigned int lcount[MAX_CL];      // particles per level (this step)
};

// ---------------------------------------------------------------- Philox
struct U4 { uint32_t v[4]; };
__host__ __device__ inline U4 philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, unsigned long long seed) {
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
#pragma unroll
  for (int r = 0; r < 10; r++) {
#ifdef __CUDA_ARCH__
    uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
#else
    uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0, hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
#endif
    uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  U4 o; o.v[0] = c0; o.v[1] = c1; o.v[2] = c2; o.v[3] = c3;
  return o;
}
__host__ __device__ inline double u53(uint32_t a, uint32_t b) {
  return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

// ---------------------------------------------------------------- helpers
template <class R> struct V4;
template <> struct V4<double> { using T = double4; };
template <> struct V4<float> { using T = float4; };

__device__ inline double r_sqrt(double x) { return sqrt(x); }
__device__ inline float r_sqrt(float x) { return sqrtf(x); }
__device__ inline double r_exp(double x) { return exp(x); }
__device__ inline float r_exp(float x) { return __expf(x); }
__device__ inline double r_tanh(double x) { return tanh(x); }
__device__ inline float r_tanh(float x) { return tanhf(x); }
__device__ inline double r_fabs(double x) { return fabs(x); }
__device__ inline float r_fabs(float x) { return fabsf(x); }

template <class R> __device__ inline R powern(R a, int n) {
  R res = 1;
  for (int i = 0; i < n; i++) res *= a;
  return res;
}
template <class R> __device__ inline R AMIN1(R a, R b) { return a <= b ? a : b; }
template <class R> __device__ inline R AMAX1(R a, R b) { return a >= b ? a : b; }

__device__ inline unsigned long long dbits(double x) { return (unsigned long long)__double_as_longlong(x); }
__device__ inline double bitsd(unsigned long long b) { return __longlong_as_double((long long)b); }

// ---------------------------------------------------------------- SPH kernels
// particle.cpp:31-807 restated.  D = kernel dimension.  dW returns
// dW/dr / dist (Derivative_kernel_function convention).
template <class R>
__device__ inline R kernel_W(int kind, int D, R dist, R h) {
  const R PI = (R)PI_REF;
  R s = dist / h, C = 0, val = 0;
  if (kind == K_WEN) {
    if (D == 1) return 0;
    if (D == 2) C = (R)1.0 / PI / powern(h, 2) * (R)7. / (R)4.;
    else C = (R)1.0 / PI / powern(h, 3) * (R)21. / (R)16.;
    if (s < 2) val = C * powern(((R)1. - (R)0.5 * s), 4) * ((R)1. + (R)2. * s);
    return val;
  }
  if (kind == K_HYP) {
    if (D == 1) C = (R)1.0 / (R)7.0 / powern(h, 1);
    else if (D == 2) C = (R)1.0 / ((R)3.0 * PI) / powern(h, 2);
    else C = (R)15.0 / ((R)62.0 * PI) / powern(h, 3);
    if (s < 1) val = C * ((R)6.0 - (R)6.0 * s + s * s * s);
    else if (s < 2) val = C * (2 - s) * (2 - s) * (2 - s);
    return val;
  }
  if (kind == K_CUB) {
    if (D == 1) C = (R)0.666666667 / powern(h, 1);
    else if (D == 2) C = (R)0.454728408 / powern(h, 2);
    else C = (R)0.318309886 / powern(h, 3);
    if (s < 1) val = C * (1 - (R)1.5 * s * s + (R)0.75 * s * s * s);
    else if (s < 2) val = C / (R)4.0 * (2 - s) * (2 - s) * (2 - s);
    return val;
  }
  if (kind == K_GAU) {
    R fac = (R)0.5 * 2 / r_sqrt(PI);
    if (D > 1) fac *= (R)0.5 * 2 / r_sqrt(PI);
    if (D > 2) fac *= (R)0.5 * 2 / r_sqrt(PI);
    if (D == 1) C = fac / h;
    else C = fac / powern(h, D);
    if (s < 3) val = r_exp((R)-1. * s * s) * C;
    return val;
  }
  // quintic
  if (D == 1) C = (R)1.0 / (R)120. / powern(h, 1);
  else if (D == 2) C = (R)1.0 / PI * (R)7. / (R)478. / powern(h, 2);
  else C = (R)1.0 / PI * (R)3. / (R)359. / powern(h, 3);
  if (s < 1) val = C * (powern(((R)3. - s), 5) - (R)6. * powern(((R)2. - s), 5) + (R)15. * powern(((R)1. - s), 5));
  else if (s < 2) val = C * (powern(((R)3. - s), 5) - (R)6. * powern(((R)2. - s), 5));
  else if (s < 3) val = C * (powern(((R)3. - s), 5));
  return val;
}

template <class R>
__device__ inline R kernel_dW(int kind, int D, R dist, R h) {
  const R PI = (R)PI_REF;
  R s = dist / h, C = 0, val = 0;
  if (kind == K_WEN) {
    if (D == 1) return 0;
    if (D == 2) C = (R)1.0 / PI / powern(h, 2) * (R)7. / (R)4.;
    else C = (R)1.0 / PI / powern(h, 3) * (R)21. / (R)16.;
    if (s < 2) val = (R)-5. * C * powern(((R)1. - (R)0.5 * s), 3) * s / h / (dist + (R)1.e-15);
    return val;
  }
  if (kind == K_HYP) {
    if (D == 1) C = (R)1.0 / (R)7.0 / powern(h, 2);
    else if (D == 2) C = (R)1.0 / ((R)3.0 * PI) / powern(h, 3);
    else C = (R)15.0 / ((R)62.0 * PI) / powern(h, 4);
    if (s < 1) val = C * ((R)-6.0 + (R)3. * s * s);
    else if (s < 2) val = C * (R)(-3.0) * (2 - s) * (2 - s);
    val /= (dist + (R)1.e-20);
    return val;
  }
  if (kind == K_CUB) {
    if (D == 1) C = (R)0.666666667 / powern(h, 2);
    else if (D == 2) C = (R)0.454728408 / powern(h, 3);
    else C = (R)0.318309886 / powern(h, 4);
    if (s < 1) val = 3 * C * (-s + 3 * (s * s) / 4);
    else if (s < 2) val = (R)(-3 / 4.0) * C * (2 - s) * (2 - s);
    val /= (dist + (R)1.e-20);
    return val;
  }
  if (kind == K_GAU) {
    R fac = (R)0.5 * 2 / r_sqrt(PI);
    if (D > 1) fac *= (R)0.5 * 2 / r_sqrt(PI);
    if (D > 2) fac *= (R)0.5 * 2 / r_sqrt(PI);
    if (D == 1) C = fac / h;
    else C = fac / powern(h, D);
    if (s < 3) val = (R)-2. * s * r_exp((R)-1. * s * s) * C / h / (dist + (R)1.e-15);
    return val;
  }
  if (D == 1) C = (R)1.0 / (R)120. / powern(h, 1);
  else if (D == 2) C = (R)1.0 / PI * (R)7. / (R)478. / powern(h, 2);
  else C = (R)1.0 / PI * (R)3. / (R)359. / powern(h, 3);
  if (s < 1) {
    val = C * ((R)-5. * powern(((R)3. - s), 4) + (R)30. * powern(((R)2. - s), 4) - (R)75. * powern(((R)1. - s), 4));
    val = val / h / (dist + (R)1.e-15);
  } else if (s < 2) {
    val = C * ((R)-5. * powern(((R)3. - s), 4) + (R)30. * powern(((R)2. - s), 4));
    val = val / h / (dist + (R)1.e-15);
  } else if (s < 3) {
    val = C * ((R)-5. * powern(((R)3. - s), 4));
    val = val / h / (dist + (R)1.e-15);
  }
  return val;
}

// ------------------------------------------------- pair arithmetic per path
// FP64 plain keeps the reference's operations (divisions, sqrt) so that its
// results stay within 1e-12 of the FP64 oracle.  FP32-split evaluates the
// same formulas without divisions: 1/h and the normalisation constants are
// hoisted, and reciprocals and square roots come from the hardware
// approximation units (relative error about 1e-7, well inside the FP32
// path's tolerance).
// a run parameter in the path's precision: the double (FP64-plain) or its
// FP32 copy made once on the host (FP32-split; no conversion per thread)
template <class R> __host__ __device__ inline R pick(double d, float f);
template <> __host__ __device__ inline double pick<double>(double d, float) { return d; }
template <> __host__ __device__ inline float pick<float>(double, float f) { return f; }

__device__ inline double r_rcp(double x) { return 1.0 / x; }
__device__ inline float r_rcp(float x) { return __fdividef(1.0f, x); }
__device__ inline double r_div(double a, double b) { return a / b; }
__device__ inline float r_div(float a, float b) { return __fdividef(a, b); }
__device__ inline double pair_dist(double d2) { return sqrt(d2); }
__device__ inline double inv_sq(double r) { return 1. / r / r; }
__device__ inline float inv_sq(float r) { return __fdividef(1.f, r * r); }
__device__ inline float pair_dist(float d2) { return d2 > 0.f ? d2 * rsqrtf(d2) : 0.f; }

// C * h^D of W (particle.cpp:31-401); dW uses the same constants with one
// more power of h for the hyperbolic and cubic kernels.
__host__ __device__ constexpr double kern_norm(int kind, int D) {
  return kind == K_WEN ? (D == 2 ? 1.0 / PI_REF * 7. / 4. : D == 3 ? 1.0 / PI_REF * 21. / 16. : 0.0)
       : kind == K_HYP ? (D == 1 ? 1.0 / 7.0 : D == 2 ? 1.0 / (3.0 * PI_REF) : 15.0 / (62.0 * PI_REF))
       : kind == K_CUB ? (D == 1 ? 0.666666667 : D == 2 ? 0.454728408 : 0.318309886)
       : kind == K_QUI ? (D == 1 ? 1.0 / 120. : D == 2 ? 1.0 / PI_REF * 7. / 478. : 1.0 / PI_REF * 3. / 359.)
       : 0.0;
}

// FP32 W(dist, h) given inv_h = 1/h
__device__ inline float kernel_W_fast(int kind, int D, float dist, float inv_h) {
  const float s = dist * inv_h;
  float ih = inv_h, C;
  float hD = ih;
  if (D >= 2) hD *= ih;
  if (D >= 3) hD *= ih;
  if (kind == K_WEN) {
    if (D == 1) return 0.f;
    C = (float)kern_norm(K_WEN, 2) * hD;
    if (D == 3) C = (float)kern_norm(K_WEN, 3) * hD;
    if (!(s < 2.f)) return 0.f;
    const float t = 1.f - 0.5f * s, t2 = t * t;
    return C * (t2 * t2) * (1.f + 2.f * s);
  }
  if (kind == K_HYP) {
    C = (float)(D == 1 ? kern_norm(K_HYP, 1) : D == 2 ? kern_norm(K_HYP, 2) : kern_norm(K_HYP, 3)) * hD;
    if (s < 1.f) return C * (6.f - 6.f * s + s * s * s);
    if (s < 2.f) { const float t = 2.f - s; return C * t * t * t; }
    return 0.f;
  }
  if (kind == K_CUB) {
    C = (float)(D == 1 ? kern_norm(K_CUB, 1) : D == 2 ? kern_norm(K_CUB, 2) : kern_norm(K_CUB, 3)) * hD;
    if (s < 1.f) return C * (1.f - 1.5f * s * s + 0.75f * s * s * s);
    if (s < 2.f) { const float t = 2.f - s; return C * 0.25f * t * t * t; }
    return 0.f;
  }
  if (kind == K_GAU) {
    const float fac = 0.5f * 2.f / sqrtf((float)PI_REF);
    float f = fac;
    if (D > 1) f *= fac;
    if (D > 2) f *= fac;
    if (!(s < 3.f)) return 0.f;
    return __expf(-s * s) * f * hD;
  }
  C = (float)(D == 1 ? kern_norm(K_QUI, 1) : D == 2 ? kern_norm(K_QUI, 2) : kern_norm(K_QUI, 3)) * hD;
  const float a = 3.f - s, b = 2.f - s, c = 1.f - s;
  const float a5 = a * a * a * a * a, b5 = b * b * b * b * b, c5 = c * c * c * c * c;
  if (s < 1.f) return C * (a5 - 6.f * b5 + 15.f * c5);
  if (s < 2.f) return C * (a5 - 6.f * b5);
  if (s < 3.f) return C * a5;
  return 0.f;
}

// FP32 dW/dr / dist (Derivative_kernel_function, particle.cpp:405-807).
// Reciprocals and the exponential are the correctly rounded / accurate
// forms: the hardware approximations' errors vary smoothly with their input,
// so they would act as a slightly different kernel on every pair of similar
// h and not average out of a near-balanced force sum.
__device__ inline float kernel_dW_fast(int kind, int D, float dist, float h) {
  const float ih = __frcp_rn(h);
  const float s = dist * ih;
  float hD = ih;
  if (D >= 2) hD *= ih;
  if (D >= 3) hD *= ih;
  if (kind == K_WEN) {
    if (D == 1 || !(s < 2.f)) return 0.f;
    const float C = (float)(D == 2 ? kern_norm(K_WEN, 2) : kern_norm(K_WEN, 3)) * hD;
    const float t = 1.f - 0.5f * s;
    return -5.f * C * (t * t * t) * s * ih * __frcp_rn(dist + 1.e-15f);
  }
  if (kind == K_HYP) {
    const float C = (float)(D == 1 ? kern_norm(K_HYP, 1) : D == 2 ? kern_norm(K_HYP, 2) : kern_norm(K_HYP, 3)) *
                    hD * ih;
    float v = 0.f;
    if (s < 1.f) v = C * (-6.f + 3.f * s * s);
    else if (s < 2.f) { const float t = 2.f - s; v = C * -3.f * t * t; }
    return v * __frcp_rn(dist + 1.e-20f);
  }
  if (kind == K_CUB) {
    const float C = (float)(D == 1 ? kern_norm(K_CUB, 1) : D == 2 ? kern_norm(K_CUB, 2) : kern_norm(K_CUB, 3)) *
                    hD * ih;
    float v = 0.f;
    if (s < 1.f) v = 3.f * C * (-s + 0.75f * s * s);
    else if (s < 2.f) { const float t = 2.f - s; v = -0.75f * C * t * t; }
    return v * __frcp_rn(dist + 1.e-20f);
  }
  if (kind == K_GAU) {
    const float fac = 0.5f * 2.f / sqrtf((float)PI_REF);
    float f = fac;
    if (D > 1) f *= fac;
    if (D > 2) f *= fac;
    if (!(s < 3.f)) return 0.f;
    return -2.f * s * expf(-s * s) * f * hD * ih * __frcp_rn(dist + 1.e-15f);
  }
  const float C = (float)(D == 1 ? kern_norm(K_QUI, 1) : D == 2 ? kern_norm(K_QUI, 2) : kern_norm(K_QUI, 3)) * hD;
  const float a = 3.f - s, b = 2.f - s, c = 1.f - s;
  const float a4 = a * a * a * a, b4 = b * b * b * b, c4 = c * c * c * c;
  float v;
  if (s < 1.f) v = C * (-5.f * a4 + 30.f * b4 - 75.f * c4);
  else if (s < 2.f) v = C * (-5.f * a4 + 30.f * b4);
  else if (s < 3.f) v = C * (-5.f * a4);
  else return 0.f;
  return v * ih * __frcp_rn(dist + 1.e-15f);
}

// path dispatch: FP64 keeps the reference arithmetic
__device__ inline double pair_W(int kind, int D, double dist, double h, double) { return kernel_W<double>(kind, D, dist, h); }
__device__ inline float pair_W(int kind, int D, float dist, float, float inv_h) { return kernel_W_fast(kind, D, dist, inv_h); }
__device__ inline double pair_dW(int kind, int D, double dist, double h) { return kernel_dW<double>(kind, D, dist, h); }
__device__ inline float pair_dW(int kind, int D, float dist, float h) { return kernel_dW_fast(kind, D, dist, h); }

// ---------------------------------------------------------------- level set
__device__ inline long long ls_index(const LsLevel& L, int D, int gi, int gj, int gk) {
  long long a0 = gi + 4 * L.margin, a1 = gj + 4 * L.margin, a2 = (D == 3) ? gk + 4 * L.margin : 0;
  return (a2 * L.n[1] + a1) * L.n[0] + a0;
}

// Finest nested level whose interior contains x and whose package is active
// (build extension for a multi-level level set; the reference has one level).
template <int D, class R>
__device__ inline int ls_pick(const LsSet& ls, const double* x) {
  constexpr bool F32 = std::is_same<R, float>::value;
  for (int l = ls.nls - 1; l >= 1; l--) {
    const LsLevel& L = ls.lv[l];
    int pk[3] = {0, 0, 0};
    bool inside = true;
    for (int d = 0; d < D; d++) {
      double cs = x[d] - L.box_l[d];
      double dom = L.dpkg[d] * L.num_pkg[d];
      if (!(cs >= 0.0 && cs < dom)) { inside = false; break; }
      pk[d] = (int)floor(F32 ? cs * L.inv_dpkg[d] : cs / L.dpkg[d]);
      if (pk[d] < 0 || pk[d] >= L.num_pkg[d]) { inside = false; break; }
    }
    if (!inside) continue;
    if (L.active) {
      long long np0 = L.num_pkg[0] + 2 * L.margin, np1 = L.num_pkg[1] + 2 * L.margin;
      long long pidx = ((long long)((D == 3) ? pk[2] + L.margin : 0) * np1 + (pk[1] + L.margin)) * np0 + (pk[0] + L.margin);
      if (!L.active[pidx]) continue;
    }
    return l;
  }
  return 0;
}

template <class R> __device__ inline void ls_fetch(const LsLevel& L, long long a, R& phi, R& nx, R& ny, R& nz, R& c);
template <> __device__ inline void ls_fetch<double>(const LsLevel& L, long long a, double& phi, double& nx, double& ny,
                                                    double& nz, double& c) {
  double4 g = L.g64[a];
  phi = g.x; nx = g.y; ny = g.z; nz = g.w; c = L.c64[a];
}
template <> __device__ inline void ls_fetch<float>(const LsLevel& L, long long a, float& phi, float& nx, float& ny,
                                                   float& nz, float& c) {
  float4 g = __ldg(&L.g32[a]);
  phi = g.x; nx = g.y; ny = g.z; nz = g.w; c = __ldg(&L.c32[a]);
}

// Calculate_particle_infor, particle_mesh_generation.cpp:175-265.  Cell
// location in FP64 (FP64-plain: the reference's divisions; FP32-split:
// products with the reciprocals), weights and accumulation in R.  The
// interpolated normal is not renormalised (reference quirk Q1).
// Interpolation of phi, n and curvature over the 2^D cells around in-package
// position rr of package pos (weights w = rr - floor(rr)), the second half
// of Calculate_particle_infor.
template <int D, class R>
__device__ inline void ls_interp(const LsLevel& L, const int* pos, const int* im, const R* w, R& phi, R* n,
                                 R& curv) {
  R ph = 0, n0 = 0, n1 = 0, n2 = 0, cv = 0;
#pragma unroll
  for (int r = 0; r <= 1; r++)
#pragma unroll
    for (int s = 0; s <= 1; s++)
#pragma unroll
      for (int t = 0; t <= (D == 3 ? 1 : 0); t++) {
        int gi = pos[0] * 4 + im[0] + r, gj = pos[1] * 4 + im[1] + s;
        int gk = (D == 3) ? pos[2] * 4 + im[2] + t : 0;
        long long a = ls_index(L, D, gi, gj, gk);
        R coef = r_fabs(w[0] - (R)(1.0 - r)) * r_fabs(w[1] - (R)(1.0 - s)) *
                 ((D == 3) ? r_fabs(w[2] - (R)(1.0 - t)) : (R)1.0);
        R p_, x_, y_, z_, c_;
        ls_fetch<R>(L, a, p_, x_, y_, z_, c_);
        ph += p_ * coef;
        n0 += x_ * coef;
        n1 += y_ * coef;
        n2 += z_ * coef;
        cv += c_ * coef;
      }
  phi = ph;
  n[0] = n0; n[1] = n1; n[2] = (D == 3) ? n2 : (R)0;
  curv = cv;
}

// Calculate_particle_infor, particle_mesh_generation.cpp:175-265.  Cell
// location in FP64 (FP64-plain: the reference's divisions; FP32-split:
// products with the reciprocals), weights and accumulation in R.  The
// interpolated normal is not renormalised (reference quirk Q1).
template <int D, class R>
__device__ inline void ls_sample(const LsSet& ls, const double* x, R& phi, R* n, R& curv) {
  constexpr bool F32 = std::is_same<R, float>::value;
  const LsLevel& L = ls.lv[ls_pick<D, R>(ls, x)];
  int pos[3] = {0, 0, 0}, im[3] = {0, 0, 0};
  R w[3] = {0, 0, 0};
  for (int d = 0; d < D; d++) {
    double dom = L.dpkg[d] * L.num_pkg[d];
    double cs = AMIN1(AMAX1(x[d] - L.box_l[d], 0.), dom - 1.e-8);
    int p = (int)floor(F32 ? cs * L.inv_dpkg[d] : cs / L.dpkg[d]);
    p = max(-L.margin, min(p, L.num_pkg[d] + L.margin - 1));
    pos[d] = p;
    double csp = cs - L.dpkg[d] * p;
    double rr = (F32 ? csp * L.inv_dcell[d] : csp / L.dcell[d]) - 0.5;
    rr = AMAX1(-0.5, AMIN1(rr, 4.0 - 0.5));
    im[d] = (int)floor(rr);
    w[d] = (R)(rr - (double)im[d]);
  }
  ls_interp<D, R>(L, pos, im, w, phi, n, curv);
}

// FP32-split location of a point given as anchor cell k and FP32 offset o
// (the particle representation): per axis the package P and the position csp
// inside it, from the anchor tables, in FP32 relative to the anchor corner.
template <int D>
__device__ inline void ls_loc_anchor(const LsLevel& L, const int* k, const float* o, int* P, float* csp) {
  for (int d = 0; d < D; d++) {
    const int2 t = __ldg(&L.anc[d][k[d]]);
    const float cs = __int_as_float(t.y) + o[d];
    const float q = floorf(cs * L.inv_dpkg_f[d]);
    P[d] = t.x + (int)q;
    csp[d] = fmaf(-q, L.dpkg_f[d], cs);
  }
}

// near (optional): the location lies within 2^-16 of a cell face of L,
// measured in cells (package faces are cell faces).  The FP32 location is
// within about 2^-22 cells of the exact one, so outside that band its cell is
// the cell of the FP64 location.
template <int D>
__device__ inline void ls_near_face(const LsLevel& L, const float* csp, bool* near) {
  if (!near) return;
  for (int d = 0; d < D; d++) {
    const float u = csp[d] * L.inv_dcell_f[d];
    const float fr = u - floorf(u);
    if (fr < 1.0f / 65536.0f || fr > 1.0f - 1.0f / 65536.0f) *near = true;
  }
}

// ls_pick on the anchor representation: the finest level containing the
// point with an active package, and the point's location on it.  near: see
// ls_near_face, over every level the choice examines.
template <int D>
__device__ inline int ls_pick_anchor(const LsSet& ls, const int* k, const float* o, int* P, float* csp,
                                     bool* near = nullptr) {
  for (int l = ls.nls - 1; l >= 1; l--) {
    const LsLevel& L = ls.lv[l];
    ls_loc_anchor<D>(L, k, o, P, csp);
    ls_near_face<D>(L, csp, near);
    bool inside = true;
    for (int d = 0; d < D; d++) inside = inside && P[d] >= 0 && P[d] < L.num_pkg[d];
    if (!inside) continue;
    if (L.active) {
      long long np0 = L.num_pkg[0] + 2 * L.margin, np1 = L.num_pkg[1] + 2 * L.margin;
      long long pidx = ((long long)((D == 3) ? P[2] + L.margin : 0) * np1 + (P[1] + L.margin)) * np0 + (P[0] + L.margin);
      if (!L.active[pidx]) continue;
    }
    return l;
  }
  ls_loc_anchor<D>(ls.lv[0], k, o, P, csp);
  ls_near_face<D>(ls.lv[0], csp, near);
  return 0;
}

// ls_sample for the FP32-split particle representation: the location runs
// in FP32 relative to the anchor corner (points outside a level's packages
// are clamped to its boundary, as the FP64 location clamps them).
template <int D>
__device__ inline void ls_sample_anchor(const LsSet& ls, const int* k, const float* o, float& phi, float* n,
                                        float& curv) {
  int P[3] = {0, 0, 0};
  float csp[3] = {0.f, 0.f, 0.f};
  const LsLevel& L = ls.lv[ls_pick_anchor<D>(ls, k, o, P, csp)];
  int pos[3] = {0, 0, 0}, im[3] = {0, 0, 0};
  float w[3] = {0.f, 0.f, 0.f};
  for (int d = 0; d < D; d++) {
    int p = P[d];
    float cp = csp[d];
    if (p < 0) { p = 0; cp = 0.f; }
    else if (p >= L.num_pkg[d]) { p = L.num_pkg[d] - 1; cp = L.dpkg_f[d]; }
    pos[d] = p;
    const float rr = fmaxf(-0.5f, fminf(fmaf(cp, L.inv_dcell_f[d], -0.5f), 3.5f));
    im[d] = (int)floorf(rr);
    w[d] = rr - (float)im[d];
  }
  ls_interp<D, float>(L, pos, im, w, phi, n, curv);
}

// ls_tag for the FP32-split particle representation.  near (optional) is
// set when a cell face of a level the lookup examined lies within the FP32
// location's band; the caller then decides in FP64 (ls_tag on the world
// position), as the reference locates the cell.
template <int D>
__device__ inline int ls_tag_anchor(const LsSet& ls, const int* k, const float* o, int* chr = nullptr,
                                    bool* near = nullptr) {
  int P[3] = {0, 0, 0};
  float csp[3] = {0.f, 0.f, 0.f};
  const LsLevel& L = ls.lv[ls_pick_anchor<D>(ls, k, o, P, csp, near)];
  int g[3] = {0, 0, 0};
  for (int d = 0; d < D; d++) {
    int p = P[d], ci;
    if (p < 0) { p = 0; ci = 0; }
    else if (p >= L.num_pkg[d]) { p = L.num_pkg[d] - 1; ci = 3; }
    else ci = max(0, min((int)floorf(csp[d] * L.inv_dcell_f[d]), 3));
    g[d] = p * 4 + ci;
  }
  const long long a = ls_index(L, D, g[0], g[1], g[2]);
  if (chr) *chr = L.chr ? L.chr[a] : 0;
  return L.tag[a];
}

// Get_level_set_char_cell_tag_and_idx (particle_mesh_generation.cpp:552-573)
// via Get_id_pkg_cell (lset_level_infor.cpp:350-366).
template <int D, class R>
__device__ inline int ls_tag(const LsSet& ls, const double* x, int* chr = nullptr) {
  constexpr bool F32 = std::is_same<R, float>::value;
  const LsLevel& L = ls.lv[ls_pick<D, R>(ls, x)];
  int g[3] = {0, 0, 0};
  for (int d = 0; d < D; d++) {
    double dom = L.dpkg[d] * L.num_pkg[d];
    double cs = AMIN1(AMAX1(x[d] - L.box_l[d], 0.), dom - 1.e-8);
    int p = (int)floor(F32 ? cs * L.inv_dpkg[d] : cs / L.dpkg[d]);
    p = max(-L.margin, min(p, L.num_pkg[d] + L.margin - 1));
    double csp = cs - L.dpkg[d] * p;
    int ci = (int)floor(F32 ? csp * L.inv_dcell[d] : csp / L.dcell[d]);
    ci = max(0, min(ci, 3));
    g[d] = p * 4 + ci;
  }
  const long long a = ls_index(L, D, g[0], g[1], g[2]);
  if (chr) *chr = L.chr ? L.chr[a] : 0;
  return L.tag[a];
}

// Levelset::Get_scale, level_set.cpp:311-351.  Law 0: the active tanh law.
// Law 1 (this build's curvature law): at the surface the spacing runs from
// minimum_dl at the largest |curvature| of the CUT cells to middle_dl at the
// smallest, q = clamp((max_curv - |curv|) / (max_curv - min_curv + 1e-20),
// 0, 1), s0 = minimum_dl + q^2 (middle_dl - minimum_dl), and grows with |phi|
// by the tanh law from s0 to maximum_dl.
template <class R>
__device__ inline R get_scale(const LsSet& ls, R phi, R curv) {
  const R min_dl = pick<R>(ls.min_dl, ls.min_dl_f);
  if (phi > 0 || r_fabs(phi) < pick<R>(ls.dl0, ls.dl0_f)) {
    R factor = (R)2.5;
    R lo = min_dl;
    if (ls.law == 1) {
      const R mc = pick<R>(ls.max_curv, ls.max_curv_f);
      R q = (mc - r_fabs(curv)) / (mc - pick<R>(ls.min_curv, ls.min_curv_f) + (R)1.e-20);
      q = AMAX1((R)0., AMIN1(q, (R)1.));
      lo = min_dl + q * q * (pick<R>(ls.middle_dl, ls.middle_dl_f) - min_dl);
    }
    return lo + r_tanh(factor * r_fabs(phi) / pick<R>(ls.max_phi, ls.max_phi_f)) / r_tanh(factor) *
                    (pick<R>(ls.max_dl, ls.max_dl_f) - lo);
  }
  return min_dl;
}

// ---------------------------------------------------------------- reductions
__device__ inline double warp_min(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ inline double warp_max(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ inline unsigned long long warp_sum_u64(unsigned long long v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide min/max of non-negative doubles folded into global bit-pattern
// atomics (exact and order-independent).  All threads of the block must call.
__device__ inline void block_minmax_to_global(double vmin, double vmax, unsigned long long* gmin,
                                              unsigned long long* gmax) {
  __shared__ double smin[32], smax[32];
  vmin = warp_min(vmin);
  vmax = warp_max(vmax);
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { smin[wid] = vmin; smax[wid] = vmax; }
  __syncthreads();
  if (wid == 0) {
    int nw = (blockDim.x + 31) >> 5;
    vmin = lane < nw ? smin[lane] : 1.e300;
    vmax = lane < nw ? smax[lane] : 0.0;
    vmin = warp_min(vmin);
    vmax = warp_max(vmax);
    if (lane == 0) {
      if (gmin) atomicMin(gmin, dbits(vmin));
      if (gmax) atomicMax(gmax, dbits(vmax));
    }
  }
}

__device__ inline void block_sum_u64_to_global(unsigned long long v, unsigned long long* g) {
  __shared__ unsigned long long ss[32];
  v = warp_sum_u64(v);
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) ss[wid] = v;
  __syncthreads();
  if (wid == 0) {
    int nw = (blockDim.x + 31) >> 5;
    v = lane < nw ? ss[lane] : 0ull;
    v = warp_sum_u64(v);
    if (lane == 0 && v) atomicAdd(g, v);
  }
}

}  // namespace mrsph
