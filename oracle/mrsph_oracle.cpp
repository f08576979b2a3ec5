// mrsph_oracle.cpp — CPU FP64 restatement of the reference relaxation path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity checker and the timed CPU
// baseline.  Only tests/, __graft_entry__.smoke() and bench.py (its CPU
// baseline and reference arms) may load it.  The product library
// (sph-mesh-generation_gb300/csrc) never links or calls it.
//
// Parity status: UNPINNED against the reference binary for the relaxation
// step.  The reference (Xiangyu-Hu/SPH-mesh-generation) needs TBB,
// Boost.MPI/Graph/Serialization and voro++ to build, none of which exist
// here, and it ships no tests, golden vectors or fixtures.  This restatement
// is pinned instead by analytic known-answer tests (kernel normalisation,
// zero gradient sum on a lattice, exact bilinear interpolation of linear phi,
// projection onto phi = 0, spacing-law endpoints) in tests/test_oracle_kat.py.
// One piece compiles from the reference's own sources: its marching-cubes
// polygoniser (geometry_tools/polygonise.cpp, oracle/build_ref.py), which
// pins the surface-area restatement below (tests/test_volume_mass.py and the
// golden vectors of tests/golden/make_mc_golden.py).
//
// Every function cites the reference file:line it restates (paths relative to
// the reference's src/).  Arithmetic is FP64 and follows the reference's
// expression order; build with -ffp-contract=off so no multiply-add is fused.
// Deterministic order: each neighbour list is sorted by particle id before any
// summation.  Reference build flags restated: _MESH_GENERATION_, _DOUBLE_,
// _NON_PERI_, _NON_SYM_ (no symmetric-mirror ghosts: the level set bounds the
// domain), one rank.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <array>
#include <set>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const double PI_REF = 3.1415926;  // glbparam.h:186 (#define PI 3.1415926)

enum { REAL_PARTICLE = 0, SURFACE_PARTICLE = 1, SINGULARITY_PARTICLE = 2, SEGMENT_PARTICLE = 3 };
enum { NORMAL_CELL = 0, CUT_CELL = 1 };
enum { K_HYPERBOLIC = 0, K_CUBIC = 1, K_WENDLAND = 2, K_GAUSSIAN = 3, K_QUINTIC = 4 };

// glbfunc.h:42-53
inline double powern(double a, int n) {
  double res = 1;
  for (int i = 0; i < n; i++) res *= a;
  return res;
}
inline double AMAX1(double a, double b) { return a >= b ? a : b; }  // glbfunc.h:56
inline double AMIN1(double a, double b) { return a <= b ? a : b; }  // glbfunc.h:61
inline int IMAX1(int a, int b) { return a >= b ? a : b; }
inline int IMIN1(int a, int b) { return a <= b ? a : b; }
inline int signum(double x) { return (0.0 < x) - (x < 0.0); }  // glbfunc.h:35-39

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), written from the paper.
// Replaces the reference's srand(time)/rand() seeding (reference quirk Q5).
// ---------------------------------------------------------------------------
struct U4 { uint32_t v[4]; };
inline U4 philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint64_t seed) {
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  for (int r = 0; r < 10; r++) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  U4 o; o.v[0] = c0; o.v[1] = c1; o.v[2] = c2; o.v[3] = c3; return o;
}
inline double u53(uint32_t a, uint32_t b) {
  return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}
enum { RNG_SEED = 1, RNG_REMAP = 2 };

// ---------------------------------------------------------------------------
// SPH kernels: particle.cpp:31-807.  D is the kernel dimension (1, 2, 3).
// W  = Kernel_function{,_1D,_2D,_3D}
// dW = Derivative_kernel_function{,_1D,_2D,_3D} (already divided by dist)
// ---------------------------------------------------------------------------
double kernel_W(int kind, int D, double dist, double h) {
  double s = dist / h, C = 0.0, val = 0.0;
  switch (kind) {
    case K_HYPERBOLIC:  // particle.cpp:33-46, 112-125, 201-214, 290-306
      if (D == 1) C = 1.0 / 7.0 / powern(h, 1);
      else if (D == 2) C = 1.0 / (3.0 * PI_REF) / powern(h, 2);
      else C = 15.0 / (62.0 * PI_REF) / powern(h, 3);
      if (s < 1) val = C * (6.0 - 6.0 * s + s * s * s);
      else if (s < 2) val = C * (2 - s) * (2 - s) * (2 - s);
      return val;
    case K_CUBIC:  // particle.cpp:48-63, 127-142, 216-231, 308-330
      if (D == 1) C = 0.666666667 / powern(h, 1);
      else if (D == 2) C = 0.454728408 / powern(h, 2);
      else C = 0.318309886 / powern(h, 3);
      if (s < 1) val = C * (1 - 1.5 * s * s + 0.75 * s * s * s);
      else if (s < 2) val = C / 4.0 * (2 - s) * (2 - s) * (2 - s);
      return val;
    case K_WENDLAND:  // particle.cpp:65-69 (1D unsupported, Q2), 144-157, 233-246, 332-348
      if (D == 1) return 0.0;
      if (D == 2) C = 1.0 / PI_REF / powern(h, 2) * 7. / 4.;
      else C = 1.0 / PI_REF / powern(h, 3) * 21. / 16.;
      if (s < 2) val = C * powern((1. - 0.5 * s), 4) * (1. + 2. * s);
      return val;
    case K_GAUSSIAN: {  // particle.cpp:71-87, 159-176, 248-265, 350-376
      double fac = 0.5 * 2 / std::sqrt(PI_REF);
      if (D > 1) fac *= 0.5 * 2 / std::sqrt(PI_REF);
      if (D > 2) fac *= 0.5 * 2 / std::sqrt(PI_REF);
      if (D == 1) C = fac / h;
      else C = fac / powern(h, D);
      if (s < 3) val = std::exp(-1. * s * s) * C;
      return val;
    }
    case K_QUINTIC:  // particle.cpp:89-106, 178-195, 267-284, 378-400
      if (D == 1) C = 1.0 / 120. / powern(h, 1);
      else if (D == 2) C = 1.0 / PI_REF * 7. / 478. / powern(h, 2);
      else C = 1.0 / PI_REF * 3. / 359. / powern(h, 3);
      if (s < 1) val = C * (powern((3. - s), 5) - 6. * powern((2. - s), 5) + 15. * powern((1. - s), 5));
      else if (s < 2) val = C * (powern((3. - s), 5) - 6. * powern((2. - s), 5));
      else if (s < 3) val = C * (powern((3. - s), 5));
      return val;
  }
  return 0.0;
}

double kernel_dW(int kind, int D, double dist, double h) {
  double s = dist / h, C = 0.0, val = 0.0;
  switch (kind) {
    case K_HYPERBOLIC:  // particle.cpp:405-420, 491-506, 588-603, 686-706
      if (D == 1) C = 1.0 / 7.0 / powern(h, 2);
      else if (D == 2) C = 1.0 / (3.0 * PI_REF) / powern(h, 3);
      else C = 15.0 / (62.0 * PI_REF) / powern(h, 4);
      if (s < 1) val = C * (-6.0 + 3. * s * s);
      else if (s < 2) val = C * (-3.0) * (2 - s) * (2 - s);
      val /= (dist + 1.e-20);
      return val;
    case K_CUBIC:  // particle.cpp:422-439, 508-525, 605-622, 708-730
      if (D == 1) C = 0.666666667 / powern(h, 2);
      else if (D == 2) C = 0.454728408 / powern(h, 3);
      else C = 0.318309886 / powern(h, 4);
      if (s < 1) val = 3 * C * (-s + 3 * (s * s) / 4);
      else if (s < 2) val = -3 / 4.0 * C * (2 - s) * (2 - s);
      val /= (dist + 1.e-20);
      return val;
    case K_WENDLAND:  // particle.cpp:441-444 (1D: 0, Q2), 527-540, 624-637, 732-748
      if (D == 1) return 0.0;
      if (D == 2) C = 1.0 / PI_REF / powern(h, 2) * 7. / 4.;
      else C = 1.0 / PI_REF / powern(h, 3) * 21. / 16.;
      if (s < 2) val = -5. * C * powern((1. - 0.5 * s), 3) * s / h / (dist + 1.e-15);
      return val;
    case K_GAUSSIAN: {  // particle.cpp:446-463, 542-560, 639-658, 750-776
      double fac = 0.5 * 2 / std::sqrt(PI_REF);
      if (D > 1) fac *= 0.5 * 2 / std::sqrt(PI_REF);
      if (D > 2) fac *= 0.5 * 2 / std::sqrt(PI_REF);
      if (D == 1) C = fac / h;
      else C = fac / powern(h, D);
      if (s < 3) val = -2. * s * std::exp(-1. * s * s) * C / h / (dist + 1.e-15);
      return val;
    }
    case K_QUINTIC:  // particle.cpp:465-488, 562-585, 660-683, 778-807
      if (D == 1) C = 1.0 / 120. / powern(h, 1);
      else if (D == 2) C = 1.0 / PI_REF * 7. / 478. / powern(h, 2);
      else C = 1.0 / PI_REF * 3. / 359. / powern(h, 3);
      if (s < 1) {
        val = C * (-5. * powern((3. - s), 4) + 30. * powern((2. - s), 4) - 75. * powern((1. - s), 4));
        val = val / h / (dist + 1.e-15);
      } else if (s < 2) {
        val = C * (-5. * powern((3. - s), 4) + 30. * powern((2. - s), 4));
        val = val / h / (dist + 1.e-15);
      } else if (s < 3) {
        val = C * (-5. * powern((3. - s), 4));
        val = val / h / (dist + 1.e-15);
      }
      return val;
  }
  return 0.0;
}

}  // namespace

// ===========================================================================
// C interface (ctypes).  Structures mirrored in oracle/oracle.py.
// ===========================================================================
extern "C" {

struct orc_level {
  // One level-set level: a dense cell-centred grid of packages of 4^D cells
  // with `margin` packages on every side (lset_level_infor.cpp:17-85).
  double box_l[3];  // corner of interior package (0,0,0)
  double dpkg[3];   // package size (cell size = dpkg/4)
  int num_pkg[3];   // interior packages per axis
  int margin;       // margin packages per side
  double* phi;      // [ntot] input
  double* nx;       // [ntot] output of orc_ls_build
  double* ny;
  double* nz;
  double* curv;
  int* tag;         // tag_interface: NORMAL_CELL / CUT_CELL
  const uint8_t* active;  // per package incl. margins (NULL = all active)
  int* chr;         // [ntot] tag_characteristic (NORMAL / SINGULARITY_CELL / SEGMENT_CELL), or NULL
  int* chr_idx;     // [ntot] idx_characteristic (-1 without), or NULL
};

struct orc_ctx {
  int dim, kernel;
  double cell_ratio;   // glbparam.h:171-183 CELL_RATIO (h = scale*cell_ratio/cutoff)
  double cutoff;       // CUT_OFF
  double angle_thres;  // sph_mesh_generation.cpp:689 (PI*0.4)
  double nu_coeff;     // sph_mesh_generation.cpp:691-694
  double damp_coeff;   // sph_mesh_generation.cpp:696-699
  double min_dl, max_dl, max_phi;
  double box_l[3], box_r[3];
  unsigned long long seed;
  int nls;
  orc_level* ls;
  // cell-list levels, filled by orc_define_levels (sph.cpp:144-180, level_infor.cpp:35-110)
  int ncl;
  double max_scale, min_scale;
  int ini_num_cell[3];
  double cl_dcell[16][3];
  int cl_ncell[16][3];
  double cl_scale[16];
  // spacing law: 0 = the reference's active tanh law; 1 = the curvature law
  // below (max/min |curvature| over CUT cells of all levels, filled from
  // orc_ls_build results by the caller)
  int scale_law;
  double middle_dl, max_curv, min_curv;
  // characteristic points and segments of the geometry (Levelset::singularity,
  // Levelset::segment, read with the level set, level_set.cpp:1100-1125):
  // sing[3 * nsing], seg[6 * nseg] (first point, second point)
  int nsing;
  const double* sing;
  int nseg;
  const double* seg;
};

struct orc_state {
  long long n;
  double *x, *y, *z, *vx, *vy, *vz;
  int *type, *id, *level;
  double *h, *scale, *phi, *curv, *nx, *ny, *nz, *sum, *rho, *vol, *nu;
  double *ax, *ay, *az;  // acceleration of the last force stage
  double dt;             // glbl_timestep
  double max_v;          // glbl_max_v
  long long step;        // run_time counter (RNG stream)
  long long remapped;    // particles re-seeded by the last map phase
};

}  // extern "C"

namespace {

inline int ls_ncell(const orc_level& L, int d) { return (L.num_pkg[d] + 2 * L.margin) * 4; }
inline long long ls_index(const orc_level& L, int D, int gi, int gj, int gk) {
  // global cell index g in [-4*margin, 4*(num_pkg+margin)) -> array index
  long long a0 = gi + 4 * L.margin, a1 = gj + 4 * L.margin, a2 = (D == 3) ? gk + 4 * L.margin : 0;
  long long n0 = ls_ncell(L, 0), n1 = ls_ncell(L, 1);
  return (a2 * n1 + a1) * n0 + a0;
}

// level-set cell size along d
inline double ls_dcell(const orc_level& L, int d) { return L.dpkg[d] / 4.0; }
inline double ls_dl(const orc_level& L, int D) {  // lset_level_infor.cpp:48-51
  double dl = 1.e20;
  for (int d = 0; d < D; d++) dl = AMIN1(ls_dcell(L, d), dl);
  return dl;
}

// ---------------------------------------------------------------------------
// A15 level-set grid build: lset_package.cpp:332-356 (Get_normal),
// :359-390 (Get_BC_normal), :450-470 (Get_interface_tag),
// :664-762 (Is_cut_cell / Get_phi_at_corners), :393-434 (Get_curvature),
// :765-786 (Get_global_scale -> maximum_phi).
// Interior packages get central-difference normals, tags and curvature;
// margin packages get one-sided in-package normals, NORMAL_CELL, curv 0.
// ---------------------------------------------------------------------------
template <int D>
void ls_build(orc_level& L, double* max_phi) {
  const int n0 = ls_ncell(L, 0), n1 = ls_ncell(L, 1), n2 = (D == 3) ? ls_ncell(L, 2) : 1;
  const int m4 = 4 * L.margin;
  double dc[3] = {ls_dcell(L, 0), ls_dcell(L, 1), (D == 3) ? ls_dcell(L, 2) : 1.0};
  auto P = [&](int gi, int gj, int gk) { return L.phi[ls_index(L, D, gi, gj, gk)]; };
  auto interior = [&](int gi, int gj, int gk) {
    bool in = gi >= 0 && gi < 4 * L.num_pkg[0] && gj >= 0 && gj < 4 * L.num_pkg[1];
    if (D == 3) in = in && gk >= 0 && gk < 4 * L.num_pkg[2];
    return in;
  };
  long long ntot = (long long)n0 * n1 * n2;
  for (long long a = 0; a < ntot; a++) { L.tag[a] = NORMAL_CELL; L.curv[a] = 0.0; }
  // normals
#pragma omp parallel for schedule(static)
  for (int ak = 0; ak < n2; ak++)
    for (int aj = 0; aj < n1; aj++)
      for (int ai = 0; ai < n0; ai++) {
        int gi = ai - m4, gj = aj - m4, gk = (D == 3) ? ak - m4 : 0;
        double g[3] = {0, 0, 0};
        if (interior(gi, gj, gk)) {
          g[0] = 0.5 * (P(gi + 1, gj, gk) - P(gi - 1, gj, gk)) / dc[0];
          g[1] = 0.5 * (P(gi, gj + 1, gk) - P(gi, gj - 1, gk)) / dc[1];
          if (D == 3) g[2] = 0.5 * (P(gi, gj, gk + 1) - P(gi, gj, gk - 1)) / dc[2];
        } else {
          int gg[3] = {gi, gj, gk};
          for (int d = 0; d < D; d++) {
            int loc = ((gg[d] % 4) + 4) % 4;  // cell index inside its package
            int e[3] = {0, 0, 0};
            e[d] = 1;
            if (loc == 0)
              g[d] = (P(gi + e[0], gj + e[1], gk + e[2]) - P(gi, gj, gk)) / dc[d];
            else if (loc == 3)
              g[d] = (P(gi, gj, gk) - P(gi - e[0], gj - e[1], gk - e[2])) / dc[d];
            else
              g[d] = 0.5 * (P(gi + e[0], gj + e[1], gk + e[2]) - P(gi - e[0], gj - e[1], gk - e[2])) / dc[d];
          }
        }
        double dist = 0.0;
        dist += g[0] * g[0];
        dist += g[1] * g[1];
        if (D == 3) dist += g[2] * g[2];
        dist = std::sqrt(dist) + 1.e-12;
        double inv = 1. / dist;
        long long a = ls_index(L, D, gi, gj, gk);
        L.nx[a] = g[0] * inv;
        L.ny[a] = g[1] * inv;
        L.nz[a] = (D == 3) ? g[2] * inv : 0.0;
      }
  // cut-cell tags (interior only)
#pragma omp parallel for schedule(static)
  for (int gk = 0; gk < ((D == 3) ? 4 * L.num_pkg[2] : 1); gk++)
    for (int gj = 0; gj < 4 * L.num_pkg[1]; gj++)
      for (int gi = 0; gi < 4 * L.num_pkg[0]; gi++) {
        int ip = gi + 1, im = gi - 1, jp = gj + 1, jm = gj - 1;
        int kp = (D == 3) ? gk + 1 : 0, km = (D == 3) ? gk - 1 : 0;
        double v[3][3][3];
        for (int a = 0; a < 3; a++)
          for (int b = 0; b < 3; b++)
            for (int c = 0; c < 3; c++) {
              int ii = (a == 0) ? im : (a == 1 ? gi : ip);
              int jj = (b == 0) ? jm : (b == 1 ? gj : jp);
              int kk = (c == 0) ? km : (c == 1 ? gk : kp);
              v[a][b][c] = P(ii, jj, kk);
            }
        // corner vectors in the order of lset_package.cpp:726-733; index 0=m,1=centre,2=p
        const int cv[8][8][3] = {
            {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0}, {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}},
            {{0, 0, 2}, {1, 0, 2}, {0, 1, 2}, {1, 1, 2}, {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}},
            {{1, 0, 2}, {2, 0, 2}, {1, 1, 2}, {2, 1, 2}, {1, 0, 1}, {2, 0, 1}, {1, 1, 1}, {2, 1, 1}},
            {{1, 0, 0}, {2, 0, 0}, {1, 1, 0}, {2, 1, 0}, {1, 0, 1}, {2, 0, 1}, {1, 1, 1}, {2, 1, 1}},
            {{0, 2, 0}, {1, 2, 0}, {0, 1, 0}, {1, 1, 0}, {0, 2, 1}, {1, 2, 1}, {0, 1, 1}, {1, 1, 1}},
            {{0, 2, 2}, {1, 2, 2}, {0, 1, 2}, {1, 1, 2}, {0, 2, 1}, {1, 2, 1}, {0, 1, 1}, {1, 1, 1}},
            {{1, 2, 2}, {2, 2, 2}, {1, 1, 2}, {2, 1, 2}, {1, 2, 1}, {2, 2, 1}, {1, 1, 1}, {2, 1, 1}},
            {{1, 2, 0}, {2, 2, 0}, {1, 1, 0}, {2, 1, 0}, {1, 2, 1}, {2, 2, 1}, {1, 1, 1}, {2, 1, 1}}};
        double corner[8];
        for (int u = 0; u < 8; u++) {
          double w[8];
          for (int q = 0; q < 8; q++) {
            int a = cv[u][q][0], b = cv[u][q][1], c = cv[u][q][2];
            if (D == 2) c = 1;  // kp = km = k in 2D (lset_package.cpp:673-676)
            w[q] = v[a][b][c];
          }
          std::sort(w, w + 8);
          double s = 0.0;
          for (int q = 0; q < 8; q++) s += w[q];
          corner[u] = s * 0.125;
        }
        bool cut = false;
        for (int c = 0; c < 8; c++)
          if (signum(corner[c]) != signum(corner[0])) cut = true;
        if (signum(v[1][1][1]) != signum(corner[0])) cut = true;
        L.tag[ls_index(L, D, gi, gj, gk)] = cut ? CUT_CELL : NORMAL_CELL;
      }
  // curvature for cut cells (interior only)
  double cdist = 0.0;
  for (int d = 0; d < D; d++) cdist += dc[d] * dc[d];
  cdist = std::sqrt(cdist);
  double mphi = 0.0;
#pragma omp parallel for schedule(static) reduction(max : mphi)
  for (int gk = 0; gk < ((D == 3) ? 4 * L.num_pkg[2] : 1); gk++)
    for (int gj = 0; gj < 4 * L.num_pkg[1]; gj++)
      for (int gi = 0; gi < 4 * L.num_pkg[0]; gi++) {
        long long a = ls_index(L, D, gi, gj, gk);
        double p0 = L.phi[a];
        if (p0 > 0.) mphi = AMAX1(mphi, std::fabs(p0));
        if (L.tag[a] != CUT_CELL) continue;
        double px = 0, py = 0, pz = 0, pxx = 0, pyy = 0, pzz = 0, pxy = 0, pyz = 0, pxz = 0;
        int i = gi, j = gj, k = gk;
        px = (8.0 * (P(i + 1, j, k) - P(i - 1, j, k)) - (P(i + 2, j, k) - P(i - 2, j, k))) / dc[0] / 12.0;
        pxx = (P(i + 1, j, k) - 2 * P(i, j, k) + P(i - 1, j, k)) / dc[0] / dc[0];
        py = (8.0 * (P(i, j + 1, k) - P(i, j - 1, k)) - (P(i, j + 2, k) - P(i, j - 2, k))) / dc[1] / 12.0;
        pyy = (P(i, j + 1, k) - 2 * P(i, j, k) + P(i, j - 1, k)) / dc[1] / dc[1];
        if (D == 3) {
          pz = (8.0 * (P(i, j, k + 1) - P(i, j, k - 1)) - (P(i, j, k + 2) - P(i, j, k - 2))) / dc[2] / 12.0;
          pzz = (P(i, j, k + 1) - 2 * P(i, j, k) + P(i, j, k - 1)) / dc[2] / dc[2];
        }
        pxy = 0.25 * (P(i + 1, j + 1, k) - P(i - 1, j + 1, k) - P(i + 1, j - 1, k) + P(i - 1, j - 1, k)) / dc[0] / dc[1];
        if (D == 3) {
          pxz = 0.25 * (P(i + 1, j, k + 1) - P(i - 1, j, k + 1) - P(i + 1, j, k - 1) + P(i - 1, j, k - 1)) / dc[0] / dc[2];
          pyz = 0.25 * (P(i, j + 1, k + 1) - P(i, j + 1, k - 1) - P(i, j - 1, k + 1) + P(i, j - 1, k - 1)) / dc[1] / dc[2];
        }
        double c = (px * px * pyy - 2 * px * py * pxy + py * py * pxx + px * px * pzz - 2 * px * pz * pxz +
                    pz * pz * pxx + py * py * pzz - 2 * py * pz * pyz + pz * pz * pyy) /
                   std::pow(px * px + py * py + pz * pz, (double)1.5);
        L.curv[a] = std::fabs(AMIN1(AMAX1(c, -2. / cdist), 2. / cdist));
      }
  *max_phi = mphi;
}

// ---------------------------------------------------------------------------
// Characteristic cells of one level (Levelset_package::Get_singularity_tag,
// lset_package.cpp:515-556; Get_segment_tag, :560-590;
// is_Segment_intersec_AABB, :594-619), after the interface tags.  A
// singularity tags, in every interior package whose half-open box holds it
// (is_in_current_pkg: 0 < x - corner < dpkg + 1e-10 per axis), the interface
// cell (tag_interface != NORMAL) nearest to it, cell centres at
// pkg dpkg + (cell + 0.5) dcell + box_l; equal distances go to the first cell
// in (i, j, k) loop order (the reference sorts with std::sort, whose order
// of equal keys is unspecified).  A segment tags every other interface cell
// whose box it meets, the first segment in order winning.  Points and
// segments are 3-vectors (z = 0 in 2D, where the AABB test reduces to its
// 2D separating axes).
// ---------------------------------------------------------------------------
enum { CHAR_NORMAL = 0, CHAR_SINGULARITY = 1, CHAR_SEGMENT = 2 };  // glbparam.h:48-51

inline bool segment_meets_box(const double* p1, const double* p2, const double* mn, const double* mx) {
  const double EPSILON = 1.e-20;
  double d[3], e[3], cc[3], ad[3];
  for (int k = 0; k < 3; k++) {
    d[k] = (p2[k] - p1[k]) * 0.5;
    e[k] = (mx[k] - mn[k]) * 0.5;
    cc[k] = (p1[k] + d[k]) - (mx[k] + mn[k]) * 0.5;
    ad[k] = std::fabs(d[k]);
  }
  for (int k = 0; k < 3; k++)
    if (std::fabs(cc[k]) > e[k] + ad[k]) return false;
  if (std::fabs(d[1] * cc[2] - d[2] * cc[1]) > e[1] * ad[2] + e[2] * ad[1] + EPSILON) return false;
  if (std::fabs(d[2] * cc[0] - d[0] * cc[2]) > e[2] * ad[0] + e[0] * ad[2] + EPSILON) return false;
  if (std::fabs(d[0] * cc[1] - d[1] * cc[0]) > e[0] * ad[1] + e[1] * ad[0] + EPSILON) return false;
  return true;
}

template <int D>
void ls_characteristics(const orc_ctx& c, orc_level& L) {
  if (!L.chr || !L.chr_idx) return;
  const int n0 = ls_ncell(L, 0), n1 = ls_ncell(L, 1), n2 = (D == 3) ? ls_ncell(L, 2) : 1;
  const long long ntot = (long long)n0 * n1 * n2;
  for (long long a = 0; a < ntot; a++) { L.chr[a] = CHAR_NORMAL; L.chr_idx[a] = -1; }
  double dc[3] = {ls_dcell(L, 0), ls_dcell(L, 1), (D == 3) ? ls_dcell(L, 2) : 0.0};
  auto cell_of_pkg = [&](const int* pk, const int* ce) {
    return ls_index(L, D, 4 * pk[0] + ce[0], 4 * pk[1] + ce[1], (D == 3) ? 4 * pk[2] + ce[2] : 0);
  };
  for (int ic = 0; ic < c.nsing; ic++) {
    const double* p = c.sing + 3 * ic;
    int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int d = 0; d < D; d++) {
      int q = (int)std::floor((p[d] - L.box_l[d]) / L.dpkg[d]);
      lo[d] = IMAX1(0, q - 1);
      hi[d] = IMIN1(L.num_pkg[d] - 1, q + 1);
    }
    for (int pi = lo[0]; pi <= hi[0]; pi++)
      for (int pj = lo[1]; pj <= hi[1]; pj++)
        for (int pk_ = lo[2]; pk_ <= hi[2]; pk_++) {
          const int pk[3] = {pi, pj, pk_};
          bool inside = true;
          for (int d = 0; d < D; d++) {
            const double corner = pk[d] * L.dpkg[d] + L.box_l[d];
            const double dr = p[d] - corner;
            inside = inside && dr < L.dpkg[d] + 1.e-10 && dr > 0.;
          }
          if (!inside) continue;
          double best = 0.0;
          long long besta = -1;
          for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++)
              for (int k = 0; k < ((D == 3) ? 4 : 1); k++) {
                const int ce[3] = {i, j, k};
                const long long a = cell_of_pkg(pk, ce);
                if (L.tag[a] == NORMAL_CELL) continue;
                double dist = 0.0;
                for (int d = 0; d < D; d++) {
                  const double cp = (pk[d] * L.dpkg[d] + (ce[d] + 0.5) * dc[d]) + L.box_l[d];
                  dist += (cp - p[d]) * (cp - p[d]);
                }
                dist = std::sqrt(dist);
                if (besta < 0 || dist < best) { best = dist; besta = a; }
              }
          if (besta >= 0) { L.chr[besta] = CHAR_SINGULARITY; L.chr_idx[besta] = ic; }
        }
  }
  if (c.nseg <= 0) return;
  for (int pk2 = 0; pk2 < ((D == 3) ? L.num_pkg[2] : 1); pk2++)
    for (int pk1 = 0; pk1 < L.num_pkg[1]; pk1++)
      for (int pk0 = 0; pk0 < L.num_pkg[0]; pk0++)
        for (int i = 0; i < 4; i++)
          for (int j = 0; j < 4; j++)
            for (int k = 0; k < ((D == 3) ? 4 : 1); k++) {
              const int pk[3] = {pk0, pk1, pk2}, ce[3] = {i, j, k};
              const long long a = cell_of_pkg(pk, ce);
              if (L.tag[a] == NORMAL_CELL || L.chr[a] == CHAR_SINGULARITY) continue;
              double mn[3] = {0, 0, 0}, mx[3] = {0, 0, 0};
              for (int d = 0; d < D; d++) {
                mn[d] = (pk[d] * L.dpkg[d] + ce[d] * dc[d]) + L.box_l[d];
                mx[d] = mn[d] + dc[d];
              }
              for (int is = 0; is < c.nseg; is++)
                if (segment_meets_box(c.seg + 6 * is, c.seg + 6 * is + 3, mn, mx)) {
                  L.chr[a] = CHAR_SEGMENT;
                  L.chr_idx[a] = is;
                  break;
                }
            }
}

// ---------------------------------------------------------------------------
// Nested level choice (build extension for reference quirk Q9: the reference
// has one level-set level).  The finest level whose interior box contains the
// point and whose package there is active is used; level 0 otherwise.
// ---------------------------------------------------------------------------
template <int D>
int ls_pick(const orc_ctx& c, const double* x) {
  for (int l = c.nls - 1; l >= 1; l--) {
    const orc_level& L = c.ls[l];
    int pk[3] = {0, 0, 0};
    bool inside = true;
    for (int d = 0; d < D; d++) {
      double cs = x[d] - L.box_l[d];
      double dom = L.dpkg[d] * L.num_pkg[d];
      if (!(cs >= 0.0 && cs < dom)) { inside = false; break; }
      pk[d] = (int)std::floor(cs / L.dpkg[d]);
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

// ---------------------------------------------------------------------------
// A2: Calculate_particle_infor, particle_mesh_generation.cpp:175-265.
// Bilinear/trilinear interpolation of phi, n, curv.  The final normal
// "renormalisation" discards its result in the reference (Q1), so n stays the
// raw interpolated normal.
// ---------------------------------------------------------------------------
template <int D>
void sample(const orc_ctx& c, const double* x, double* phi, double* n, double* curv) {
  const orc_level& L = c.ls[ls_pick<D>(c, x)];
  double cs[3] = {0, 0, 0};
  int pos[3] = {0, 0, 0};
  double rr[3] = {0, 0, 0}, w[3] = {0, 0, 0};
  int im[3] = {0, 0, 0};
  const double ICP = 4.0;
  for (int d = 0; d < D; d++) {
    double dom = L.dpkg[d] * L.num_pkg[d];
    cs[d] = AMIN1(AMAX1(x[d] - L.box_l[d], 0.), dom - 1.e-8);
    // get_cell_id, glbfunc.h:196-208 (clamped to the package range incl. margins)
    int p = (int)std::floor(cs[d] / L.dpkg[d]);
    pos[d] = IMAX1(-L.margin, IMIN1(p, L.num_pkg[d] + L.margin - 1));
    double csp = cs[d] - L.dpkg[d] * pos[d];
    rr[d] = csp / ls_dcell(L, d) - 0.5;
    rr[d] = AMAX1(-0.5, AMIN1(rr[d], ICP - 0.5));
    im[d] = (int)std::floor(rr[d]);
    w[d] = rr[d] - (double)im[d];
  }
  double ph = 0., n0 = 0., n1 = 0., n2 = 0., cv = 0.;
  for (int r = 0; r <= 1; r++)
    for (int s = 0; s <= 1; s++)
      for (int t = 0; t <= (D == 3 ? 1 : 0); t++) {
        int gi = pos[0] * 4 + im[0] + r, gj = pos[1] * 4 + im[1] + s;
        int gk = (D == 3) ? pos[2] * 4 + im[2] + t : 0;
        long long a = ls_index(L, D, gi, gj, gk);
        double coef = std::fabs(w[0] - (1.0 - r)) * std::fabs(w[1] - (1.0 - s)) *
                      ((D == 3) ? std::fabs(w[2] - (1.0 - t)) : 1.0);
        ph += L.phi[a] * coef;
        n0 += L.nx[a] * coef;
        n1 += L.ny[a] * coef;
        n2 += L.nz[a] * coef;
        cv += L.curv[a] * coef;
      }
  *phi = ph;
  n[0] = n0; n[1] = n1; n[2] = (D == 3) ? n2 : 0.0;
  *curv = cv;
}

// Get_level_set_char_cell_tag_and_idx, particle_mesh_generation.cpp:552-573,
// via Levelset_levelinfo::Get_id_pkg_cell, lset_level_infor.cpp:350-366.
template <int D>
int cell_tag(const orc_ctx& c, const double* x, int* chr = nullptr, int* chr_idx = nullptr) {
  const orc_level& L = c.ls[ls_pick<D>(c, x)];
  int g[3] = {0, 0, 0};
  for (int d = 0; d < D; d++) {
    double dom = L.dpkg[d] * L.num_pkg[d];
    double cs = AMIN1(AMAX1(x[d] - L.box_l[d], 0.), dom - 1.e-8);
    int p = (int)std::floor(cs / L.dpkg[d]);
    p = IMAX1(-L.margin, IMIN1(p, L.num_pkg[d] + L.margin - 1));
    double csp = cs - L.dpkg[d] * p;
    int ci = (int)std::floor(csp / ls_dcell(L, d));
    ci = IMAX1(0, IMIN1(ci, 3));
    g[d] = p * 4 + ci;
  }
  const long long a = ls_index(L, D, g[0], g[1], g[2]);
  if (chr) *chr = L.chr ? L.chr[a] : CHAR_NORMAL;
  if (chr_idx) *chr_idx = L.chr_idx ? L.chr_idx[a] : -1;
  return L.tag[a];
}

// Levelset::Get_scale, level_set.cpp:311-351.  Law 0: the active tanh law.
// Law 1 (a law of this build, in the spirit of the commented-out curvature
// variants of :319-339): at the surface the spacing runs from minimum_dl at
// the largest |curvature| of the CUT cells to middle_dl at the smallest,
// q = clamp((max_curv - |curv|) / (max_curv - min_curv + 1e-20), 0, 1),
// s0 = minimum_dl + q^2 (middle_dl - minimum_dl), and grows with |phi| by the
// tanh law from s0 to maximum_dl.
inline double get_scale(const orc_ctx& c, int D, double phi, double curv) {
  double dl0 = ls_dl(c.ls[0], D);
  if (phi > 0. || std::fabs(phi) < dl0) {
    double factor = 2.5;
    double lo = c.min_dl;
    if (c.scale_law == 1) {
      double q = (c.max_curv - std::fabs(curv)) / (c.max_curv - c.min_curv + 1.e-20);
      q = AMAX1(0., AMIN1(q, 1.));
      lo = c.min_dl + q * q * (c.middle_dl - c.min_dl);
    }
    return lo + std::tanh(factor * std::fabs(phi) / c.max_phi) / std::tanh(factor) * (c.max_dl - lo);
  }
  return c.min_dl;
}

// Particle_mesh_generation::Set_particle_info, particle_mesh_generation.cpp:361-381
template <int D>
inline void set_info(const orc_ctx& c, orc_state& s, long long i) {
  double h_tmp = get_scale(c, D, s.phi[i], s.curv[i]);
  s.h[i] = h_tmp * c.cell_ratio / c.cutoff;
  // pow(h_tmp, DIM): for DIM = 2 the correctly rounded square, h_tmp*h_tmp
  s.vol[i] = (D == 2) ? h_tmp * h_tmp : std::pow(h_tmp, 3.0);
  s.rho[i] = 1.0 / s.vol[i];  // mass = 1 (Particle_mesh_generation::Initialize :53-63)
}

template <int D>
inline void get_xyz(const orc_state& s, long long i, double* x) {
  x[0] = s.x[i]; x[1] = s.y[i]; x[2] = (D == 3) ? s.z[i] : 0.0;
}
template <int D>
inline void put_xyz(orc_state& s, long long i, const double* x) {
  s.x[i] = x[0]; s.y[i] = x[1]; if (D == 3) s.z[i] = x[2];
}

template <int D>
inline void sample_particle(const orc_ctx& c, orc_state& s, long long i) {
  double x[3], n[3];
  get_xyz<D>(s, i, x);
  sample<D>(c, x, &s.phi[i], n, &s.curv[i]);
  s.nx[i] = n[0]; s.ny[i] = n[1]; s.nz[i] = n[2];
}

// SPH_mesh_generation::Remap_this_particle_to_positive_phase,
// sph_mesh_generation.cpp:1885-1928 (non-MPI box).  Random draws: Philox.
template <int D>
bool remap(const orc_ctx& c, orc_state& s, long long i) {
  double box[3], bl[3], br[3];
  for (int d = 0; d < 3; d++) { bl[d] = c.box_l[d]; br[d] = c.box_r[d]; box[d] = br[d] - bl[d]; }
  for (uint32_t att = 0; att < 10000000u; att++) {
    double x[3] = {0, 0, 0};
    for (int d = 0; d < D; d++) {
      U4 r = philox((uint32_t)s.id[i], (uint32_t)s.step, att, (RNG_REMAP << 8) | d, c.seed);
      double u1 = u53(r.v[0], r.v[1]), u2 = u53(r.v[2], r.v[3]);
      x[d] = u1 * box[d] + u2 * 1.e-3 + bl[d];
      x[d] = AMAX1(bl[d] + 1.e-10, AMIN1(x[d], br[d] - 1.e-10));
    }
    put_xyz<D>(s, i, x);
    sample_particle<D>(c, s, i);
    if (s.phi[i] > s.h[i]) {
      s.type[i] = REAL_PARTICLE;
      set_info<D>(c, s, i);
      return true;
    }
  }
  return false;
}

// ---------------------------------------------------------------------------
// A3: Particle_mesh_generation::Find_and_map_particle :408-467 plus the
// driver loop sph_mesh_generation.cpp:1506-1545 (dispersal, re-sample,
// re-seed of REAL particles with phi < 0).  A particle in a characteristic
// cell (ls_characteristics) goes onto the segment's line or the point; with
// no characteristic points or segments every cell is NORMAL.
// ---------------------------------------------------------------------------
template <int D>
void map_particle(const orc_ctx& c, orc_state& s, long long i, long long* nremap) {
  double x[3];
  get_xyz<D>(s, i, x);
  int chr = CHAR_NORMAL, cidx = -1;
  int tag = cell_tag<D>(c, x, &chr, &cidx);
  int t = s.type[i];
  double nrm[3] = {s.nx[i], s.ny[i], s.nz[i]};
  double phi = s.phi[i];
  auto nlen = [&]() {
    double d = 0.0;
    d += nrm[0] * nrm[0];
    d += nrm[1] * nrm[1];
    if (D == 3) d += nrm[2] * nrm[2];
    return std::sqrt(d);
  };
  if (tag == CUT_CELL && (t == REAL_PARTICLE || t == SURFACE_PARTICLE) && chr == CHAR_NORMAL) {
    t = SURFACE_PARTICLE;
    double dist = std::fabs(phi);
    double div = 1.0 / (nlen() + 1.0e-15);
    for (int d = 0; d < D; d++) {
      double nn = nrm[d] * div;
      double n_d = phi < 0.0 ? nn : -nn;
      x[d] = x[d] + n_d * dist;
    }
  } else if (chr == CHAR_SEGMENT && cidx >= 0) {
    // projection onto the segment's line, particle_mesh_generation.cpp:439-455
    t = SEGMENT_PARTICLE;
    const double* p1 = c.seg + 6 * cidx;
    const double* p2 = p1 + 3;
    double P[3] = {0, 0, 0}, N[3] = {0, 0, 0};
    for (int d = 0; d < D; d++) { P[d] = p2[d] - p1[d]; N[d] = x[d] - p1[d]; }
    double len = 0.0;
    len += P[0] * P[0]; len += P[1] * P[1]; if (D == 3) len += P[2] * P[2];
    len = std::sqrt(len);
    const double inv = 1. / AMAX1(len, 1.e-15);
    double e[3] = {P[0] * inv, P[1] * inv, (D == 3) ? P[2] * inv : 0.0};
    double dist = 0.0;
    dist += N[0] * e[0]; dist += N[1] * e[1]; if (D == 3) dist += N[2] * e[2];
    for (int d = 0; d < D; d++) x[d] = p1[d] + e[d] * dist;
  } else if (chr == CHAR_SINGULARITY && cidx >= 0) {
    // particle_mesh_generation.cpp:456-465
    t = SINGULARITY_PARTICLE;
    for (int d = 0; d < D; d++) x[d] = c.sing[3 * cidx + d];
  } else {
    t = REAL_PARTICLE;
  }
  s.type[i] = t;
  if (t == SURFACE_PARTICLE || t == SEGMENT_PARTICLE) {
    // Get_dispersed_position(0.00001*h), particle_mesh_generation.cpp:385-404
    double dx = 0.00001 * s.h[i];
    double div = 1.0 / (nlen() + 1.0e-15);
    for (int d = 0; d < D; d++) {
      double nn = nrm[d] * div;
      double n_d = phi < 0.0 ? nn : -nn;
      x[d] = x[d] + n_d * dx;
    }
  }
  put_xyz<D>(s, i, x);
  sample_particle<D>(c, s, i);
  if (s.phi[i] < 0. && s.type[i] == REAL_PARTICLE) {
    remap<D>(c, s, i);
    (*nremap)++;
  }
}

// Particle_base::Set_particle_scale, particle.cpp:957-975 (the coarse/finer
// level flags are reported; levels are planned so they never fire).
inline int set_particle_scale(const orc_ctx& c, double h, double* scale) {
  int flag = 0;
  for (;;) {
    if (h * c.cutoff > *scale + 1.e-15) {
      *scale *= 2;
      if (*scale > c.max_scale + 1.e-15) flag = -1;
    } else if (h * c.cutoff < *scale / 2 - 1.e-15) {
      *scale /= 2;
      if (*scale < c.min_scale - 1.e-15) flag = 1;
    } else
      break;
  }
  return flag;
}

// SPH::Map_the_particle_to_tree, sph.cpp:247-276 (level from scale)
inline int level_of_scale(const orc_ctx& c, double scale) {
  int current = 0;
  for (int j = c.ncl - 1; j >= 0; j--) {
    if (std::fabs(scale - c.cl_scale[j]) <= 1.e-10) return j;
    if (j >= 1 && scale > c.cl_scale[j] && scale < c.cl_scale[j - 1]) return j - 1;
  }
  return current;
}

// get_cell_id, glbfunc.h:196-208 with _NON_SYM_ (cell range [0, num_cell))
template <int D>
inline void cell_of(const orc_ctx& c, int lev, const double* x, int* cell) {
  for (int d = 0; d < 3; d++) cell[d] = 0;
  for (int d = 0; d < D; d++) {
    int p = (int)std::floor((x[d] - c.box_l[d]) / c.cl_dcell[lev][d]);
    cell[d] = IMAX1(0, IMIN1(p, c.cl_ncell[lev][d] - 1));
  }
}

// Neighbour set + geometry for one ordered pair, level_infor.cpp:469-506
template <int D>
inline bool is_neighbor(const orc_state& s, long long i, long long j, double cutoff) {
  double dr[3] = {s.x[i] - s.x[j], s.y[i] - s.y[j], (D == 3) ? s.z[i] - s.z[j] : 0.0};
  double dist = 0.0;
  dist += dr[0] * dr[0];
  dist += dr[1] * dr[1];
  if (D == 3) dist += dr[2] * dr[2];
  dist = std::sqrt(dist);
  return (dist <= (s.h[i] * cutoff + 1.e-10)) || (dist <= (s.h[j] * cutoff + 1.e-10));
}

struct Neighbors {
  std::vector<long long> off;  // CSR offsets
  std::vector<int> nb;         // neighbour indices, sorted by particle id
};

// ---------------------------------------------------------------------------
// A5 + A6: cell binning into the multi-resolution tree and neighbour search.
//   Level_info::Update_cell_list level_infor.cpp:325-344 (own level),
//   Level_info::Update_every_level_info :407-464 (parents get all child-cell
//   particles), Level_info::Refresh_neighbor_info :469-506 (3^D own-level
//   cells; cross-level pairs back-inserted into the finer particle's list).
// ---------------------------------------------------------------------------
template <int D>
void build_neighbors(const orc_ctx& c, const orc_state& s, Neighbors& out) {
  const long long n = s.n;
  const int nl = c.ncl;
  std::vector<std::vector<std::vector<int>>> cells(nl);
  auto cid = [&](int l, const int* cc) -> long long {
    return ((long long)cc[2] * c.cl_ncell[l][1] + cc[1]) * c.cl_ncell[l][0] + cc[0];
  };
  for (int l = 0; l < nl; l++) {
    long long nc = (long long)c.cl_ncell[l][0] * c.cl_ncell[l][1] * (D == 3 ? c.cl_ncell[l][2] : 1);
    cells[l].assign(nc, std::vector<int>());
  }
  // own-level binning in index order
  for (long long i = 0; i < n; i++) {
    double x[3]; get_xyz<D>(s, i, x);
    int cc[3]; cell_of<D>(c, s.level[i], x, cc);
    cells[s.level[i]][cid(s.level[i], cc)].push_back((int)i);
  }
  // parents collect all child-cell particles, finest to coarsest
  for (int l = nl - 2; l >= 0; l--) {
    int nc0 = c.cl_ncell[l][0], nc1 = c.cl_ncell[l][1], nc2 = (D == 3) ? c.cl_ncell[l][2] : 1;
    for (int k = 0; k < nc2; k++)
      for (int j = 0; j < nc1; j++)
        for (int i = 0; i < nc0; i++) {
          int pc[3] = {i, j, k};
          auto& dst = cells[l][cid(l, pc)];
          for (int t = 0; t < 2; t++)
            for (int u = 0; u < 2; u++)
              for (int m = 0; m < (D == 3 ? 2 : 1); m++) {
                int ch[3] = {2 * i + t, 2 * j + u, (D == 3) ? 2 * k + m : 0};
                if (ch[0] >= c.cl_ncell[l + 1][0] || ch[1] >= c.cl_ncell[l + 1][1]) continue;
                if (D == 3 && ch[2] >= c.cl_ncell[l + 1][2]) continue;
                auto& src = cells[l + 1][cid(l + 1, ch)];
                dst.insert(dst.end(), src.begin(), src.end());
              }
        }
  }
  std::vector<std::vector<int>> lists(n);
  std::vector<std::vector<std::pair<int, int>>> back(
#ifdef _OPENMP
      omp_get_max_threads()
#else
      1
#endif
  );
#pragma omp parallel for schedule(dynamic, 256)
  for (long long i = 0; i < n; i++) {
#ifdef _OPENMP
    int tid = omp_get_thread_num();
#else
    int tid = 0;
#endif
    int l = s.level[i];
    double x[3]; get_xyz<D>(s, i, x);
    int cc[3]; cell_of<D>(c, l, x, cc);
    int lo[3], hi[3];
    for (int d = 0; d < 3; d++) {
      int span = (d < D) ? 1 : 0;
      lo[d] = IMAX1(cc[d] - span, 0);
      hi[d] = IMIN1(cc[d] + span, (d < D ? c.cl_ncell[l][d] : 1) - 1);
    }
    for (int t = lo[0]; t <= hi[0]; t++)
      for (int u = lo[1]; u <= hi[1]; u++)
        for (int m = lo[2]; m <= hi[2]; m++) {
          int q[3] = {t, u, m};
          for (int j : cells[l][cid(l, q)]) {
            if (is_neighbor<D>(s, i, j, c.cutoff)) {
              lists[i].push_back(j);
              if (s.level[j] != l) back[tid].push_back(std::make_pair(j, (int)i));
            }
          }
        }
  }
  for (auto& b : back)
    for (auto& p : b) lists[p.first].push_back(p.second);
  out.off.assign(n + 1, 0);
  for (long long i = 0; i < n; i++) {
    std::sort(lists[i].begin(), lists[i].end(), [&](int a, int b) { return s.id[a] < s.id[b]; });
    out.off[i + 1] = out.off[i] + (long long)lists[i].size();
  }
  out.nb.resize(out.off[n]);
  for (long long i = 0; i < n; i++) std::copy(lists[i].begin(), lists[i].end(), out.nb.begin() + out.off[i]);
}

// ---------------------------------------------------------------------------
// A7: Particle_mesh_generation::Get_kernel_summation, :690-765
// ---------------------------------------------------------------------------
template <int D>
void density(const orc_ctx& c, orc_state& s, const Neighbors& nb) {
  const double cos_t = std::cos(c.angle_thres);
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < s.n; i++) {
    double sum = 0.;
    int ncount = 0;
    int ti = s.type[i];
    double ni[3] = {s.nx[i], s.ny[i], s.nz[i]};
    for (long long q = nb.off[i]; q < nb.off[i + 1]; q++) {
      int j = nb.nb[q];
      double vec[3] = {s.x[i] - s.x[j], s.y[i] - s.y[j], (D == 3) ? s.z[i] - s.z[j] : 0.0};
      if (ti == REAL_PARTICLE) {
        double dist = 0.0;
        dist += vec[0] * vec[0]; dist += vec[1] * vec[1]; if (D == 3) dist += vec[2] * vec[2];
        dist = std::sqrt(dist);
        sum += kernel_W(c.kernel, D, dist, s.h[i]);
        ncount++;
      } else if (ti == SURFACE_PARTICLE) {
        double dn = 0.0;
        dn += vec[0] * ni[0]; dn += vec[1] * ni[1]; if (D == 3) dn += vec[2] * ni[2];
        double dr[3];
        for (int d = 0; d < 3; d++) dr[d] = vec[d] - ni[d] * dn;
        double dist = 0.0;
        dist += dr[0] * dr[0]; dist += dr[1] * dr[1]; if (D == 3) dist += dr[2] * dr[2];
        dist = std::sqrt(dist);
        int tj = s.type[j];
        if (tj == SURFACE_PARTICLE) {
          double nj[3] = {s.nx[j], s.ny[j], s.nz[j]};
          double ca = 0.0;
          ca += ni[0] * nj[0]; ca += ni[1] * nj[1]; if (D == 3) ca += ni[2] * nj[2];
          if (std::fabs(ca) > cos_t) {
            sum += kernel_W(c.kernel, D - 1, dist, s.h[i]);
            ncount++;
          }
        } else if (tj == SEGMENT_PARTICLE || tj == SINGULARITY_PARTICLE) {
          sum += kernel_W(c.kernel, D - 1, dist, s.h[i]);
          ncount++;
        }
      } else if (ti == SEGMENT_PARTICLE && D == 3) {
        // :740-759: segment and singularity neighbours with the 1D kernel
        double dn = 0.0;
        dn += vec[0] * ni[0]; dn += vec[1] * ni[1]; if (D == 3) dn += vec[2] * ni[2];
        double dr[3];
        for (int d = 0; d < 3; d++) dr[d] = vec[d] - ni[d] * dn;
        double dist = 0.0;
        dist += dr[0] * dr[0]; dist += dr[1] * dr[1]; if (D == 3) dist += dr[2] * dr[2];
        dist = std::sqrt(dist);
        int tj = s.type[j];
        if (tj == SEGMENT_PARTICLE) {
          double nj[3] = {s.nx[j], s.ny[j], s.nz[j]};
          double ca = 0.0;
          ca += ni[0] * nj[0]; ca += ni[1] * nj[1]; if (D == 3) ca += ni[2] * nj[2];
          if (std::fabs(ca) > cos_t) {
            sum += kernel_W(c.kernel, 1, dist, s.h[i]);
            ncount++;
          }
        } else if (tj == SINGULARITY_PARTICLE) {
          sum += kernel_W(c.kernel, 1, dist, s.h[i]);
          ncount++;
        }
      }
    }
    if (ncount > 1) sum = 1. / (sum + 1.e-15);
    s.sum[i] = sum;
  }
}

// ---------------------------------------------------------------------------
// A8: Accumulate_particle_force_real :995-1118, _surf :883-991,
// Map_surface_particle_force :1122-1126.  A9: Set_timestep(stage) :127-145
// and ParallelGetTimestep parallelfunc.cpp:50-58.  A10: Update_velocity_half_step
// :1130-1135.  One rank, so the MPI colour ramp sigma is 1.
// ---------------------------------------------------------------------------
template <int D>
void force_stage(const orc_ctx& c, orc_state& s, const Neighbors& nb, int stage) {
  const double cos_t = std::cos(c.angle_thres);
  const long long n = s.n;
  std::vector<double> axv(n), ayv(n), azv(n);
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < n; i++) {
    int ti = s.type[i];
    double F1[3] = {0, 0, 0}, F2[3] = {0, 0, 0};
    double ni[3] = {s.nx[i], s.ny[i], s.nz[i]};
    double v[3] = {s.vx[i], s.vy[i], (D == 3) ? s.vz[i] : 0.0};
    double rho = s.rho[i], h = s.h[i], sum = s.sum[i], nu = s.nu[i];
    double P = 1.0, mass_j = 1.0, P_j = 1.0, sigma = 1.;
    if (ti == REAL_PARTICLE || ti == SURFACE_PARTICLE || ti == SEGMENT_PARTICLE) {
      for (long long q = nb.off[i]; q < nb.off[i + 1]; q++) {
        int j = nb.nb[q];
        int tj = s.type[j];
        if (ti == SURFACE_PARTICLE && tj == REAL_PARTICLE) continue;
        // Accumulate_particle_force_seg, :769-879: segment and singularity
        // neighbours only, the 1D kernel gradient in 3D (none in 2D)
        if (ti == SEGMENT_PARTICLE && (tj == REAL_PARTICLE || tj == SURFACE_PARTICLE)) continue;
        if (s.id[i] == s.id[j]) continue;
        double h_j = s.h[j], rho_j = s.rho[j], nu_j = s.nu[j];
        double vj[3] = {s.vx[j], s.vy[j], (D == 3) ? s.vz[j] : 0.0};
        double vec[3] = {s.x[i] - s.x[j], s.y[i] - s.y[j], (D == 3) ? s.z[i] - s.z[j] : 0.0};
        double dr[3], dist = 0.0, aw;
        double vol_i = P / powern(rho, 2), vol_j = P_j / powern(rho_j, 2);
        if (ti == REAL_PARTICLE) {
          if (tj != REAL_PARTICLE) for (int d = 0; d < 3; d++) vj[d] = v[d] * -1.0;
          for (int d = 0; d < 3; d++) dr[d] = vec[d];
          dist += dr[0] * dr[0]; dist += dr[1] * dr[1]; if (D == 3) dist += dr[2] * dr[2];
          dist = std::sqrt(dist);
          aw = kernel_dW(c.kernel, D, dist, 0.5 * (h + h_j));
        } else {
          double dn = 0.0;
          dn += vec[0] * ni[0]; dn += vec[1] * ni[1]; if (D == 3) dn += vec[2] * ni[2];
          for (int d = 0; d < 3; d++) dr[d] = vec[d] - ni[d] * dn;
          dist += dr[0] * dr[0]; dist += dr[1] * dr[1]; if (D == 3) dist += dr[2] * dr[2];
          dist = std::sqrt(dist);
          if ((ti == SURFACE_PARTICLE && tj == SURFACE_PARTICLE) ||
              (ti == SEGMENT_PARTICLE && tj == SEGMENT_PARTICLE)) {
            double nj[3] = {s.nx[j], s.ny[j], s.nz[j]};
            double ca = 0.0;
            ca += ni[0] * nj[0]; ca += ni[1] * nj[1]; if (D == 3) ca += ni[2] * nj[2];
            if (std::fabs(ca) <= cos_t) continue;
          }
          if (ti == SEGMENT_PARTICLE) aw = (D == 3) ? kernel_dW(c.kernel, 1, dist, 0.5 * (h + h_j)) : 0.0;
          else aw = kernel_dW(c.kernel, D - 1, dist, 0.5 * (h + h_j));
        }
        double awax[3] = {dr[0] * aw, dr[1] * aw, dr[2] * aw};
        if (stage == 1) {
          double P_ij = sigma * mass_j * sum * (vol_i + vol_j);
          for (int d = 0; d < D; d++) F1[d] = F1[d] + awax[d] * -P_ij;
        } else {
          double eta_i = nu * rho, eta_j = nu_j * rho_j;
          double eta_ij = 2. * eta_j * eta_i / (eta_i + eta_j + 1.e-15);
          double temp0 = aw * eta_ij * mass_j * (1. / rho / rho + 1. / rho_j / rho_j);
          for (int d = 0; d < D; d++) F2[d] = F2[d] + (v[d] - vj[d]) * temp0;
        }
      }
    }
    double a[3] = {0, 0, 0};
    if (ti == REAL_PARTICLE || ti == SURFACE_PARTICLE || ti == SEGMENT_PARTICLE) {
      for (int d = 0; d < D; d++) a[d] = F1[d] + F2[d];
      if (stage == 2)
        for (int d = 0; d < D; d++) a[d] = a[d] + v[d] * c.damp_coeff;
      if (ti == SURFACE_PARTICLE || ti == SEGMENT_PARTICLE) {  // Map_surface_particle_force
        double nf = 0.0;
        nf += a[0] * ni[0]; nf += a[1] * ni[1]; if (D == 3) nf += a[2] * ni[2];
        for (int d = 0; d < D; d++) a[d] = a[d] - ni[d] * nf;
      }
    }
    axv[i] = a[0]; ayv[i] = a[1]; azv[i] = a[2];
  }
  // Set_timestep(stage) + global min/max
  double dtmin = 1.e300, vmax = 0.0;
  std::vector<double> nu_new(n);
#pragma omp parallel for schedule(static) reduction(min : dtmin) reduction(max : vmax)
  for (long long i = 0; i < n; i++) {
    double v[3] = {s.vx[i], s.vy[i], (D == 3) ? s.vz[i] : 0.0};
    double U = 0.0; U += v[0] * v[0]; U += v[1] * v[1]; if (D == 3) U += v[2] * v[2]; U = std::sqrt(U);
    double A = 0.0; A += axv[i] * axv[i]; A += ayv[i] * ayv[i]; if (D == 3) A += azv[i] * azv[i]; A = std::sqrt(A);
    double h = s.h[i];
    double ts = 0.25 * std::sqrt(h / (A + 1.e-15));
    ts = AMIN1(ts, h / 40. / (U + 1.e-15));
    double nu = s.nu[i];
    if (stage == 2) {
      nu = c.nu_coeff * h * U;
      ts = AMIN1(ts, 0.125 * h * h / (nu + 1.e-15));
    }
    nu_new[i] = nu;
    dtmin = AMIN1(dtmin, ts);
    vmax = AMAX1(vmax, U);
  }
  s.dt = dtmin;
  s.max_v = vmax;
  // Update_velocity_half_step
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < n; i++) {
    s.nu[i] = nu_new[i];
    s.ax[i] = axv[i]; s.ay[i] = ayv[i]; if (D == 3) s.az[i] = azv[i];
    double hdt = 0.5 * s.dt;
    s.vx[i] = s.vx[i] + axv[i] * hdt;
    s.vy[i] = s.vy[i] + ayv[i] * hdt;
    if (D == 3) s.vz[i] = s.vz[i] + azv[i] * hdt;
  }
}

// Reset_particle_force(1): v := 0 every step (Q4), particle_mesh_generation.cpp:149-171
template <int D>
void reset_stage1(orc_state& s) {
  for (long long i = 0; i < s.n; i++) {
    s.sum[i] = 0.;
    s.vx[i] = 0.; s.vy[i] = 0.; if (D == 3) s.vz[i] = 0.;
  }
}

// Update_coord_full_step, particle_mesh_generation.cpp:1139-1179 (no periodic wrap)
template <int D>
void advect(orc_state& s) {
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < s.n; i++) {
    if (s.type[i] == SINGULARITY_PARTICLE) continue;
    s.x[i] = s.x[i] + s.vx[i] * s.dt;
    s.y[i] = s.y[i] + s.vy[i] * s.dt;
    if (D == 3) s.z[i] = s.z[i] + s.vz[i] * s.dt;
  }
}

// Phase "map": Update_coord_full_step, Get_particle_info, Find_and_map_particle,
// Set_particle_scale and the scale/level refresh of Prepare_for_the_current_step
// (sph_mesh_generation.cpp:1371-1393, 1984-2022; sph.cpp:456-486).
template <int D>
void phase_map(const orc_ctx& c, orc_state& s, int do_advect) {
  if (do_advect) advect<D>(s);
  long long nremap = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : nremap)
  for (long long i = 0; i < s.n; i++) {
    sample_particle<D>(c, s, i);
    map_particle<D>(c, s, i, &nremap);
  }
  s.remapped = nremap;
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < s.n; i++) {
    set_info<D>(c, s, i);
    set_particle_scale(c, s.h[i], &s.scale[i]);
    s.level[i] = level_of_scale(c, s.scale[i]);
  }
}

// Pre_run, sph_mesh_generation.cpp:1010-1050: sample, Set_particle_info,
// Find_and_map; forces of Pre_run vanish (sum = 0, v = 0), leaving v = 0, nu = 0.
template <int D>
void pre_run(const orc_ctx& c, orc_state& s) {
  long long nremap = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : nremap)
  for (long long i = 0; i < s.n; i++) {
    sample_particle<D>(c, s, i);
    set_info<D>(c, s, i);
    map_particle<D>(c, s, i, &nremap);
  }
  s.remapped = nremap;
  for (long long i = 0; i < s.n; i++) {
    set_particle_scale(c, s.h[i], &s.scale[i]);
    s.level[i] = level_of_scale(c, s.scale[i]);
    s.vx[i] = 0; s.vy[i] = 0; if (D == 3) s.vz[i] = 0;
    s.nu[i] = 0;
  }
  s.dt = 0.0;
}

// Random_particle_distribution, sph_mesh_generation.cpp:1302-1367 (non-MPI)
template <int D>
int seed_particles(const orc_ctx& c, orc_state& s) {
  const orc_level& L0 = c.ls[0];
  double padding = L0.dpkg[0];  // lset_level_info[0]->scale (lset_level_infor.cpp:47)
  double lbl[3], lbr[3];
  for (int d = 0; d < 3; d++) { lbl[d] = L0.box_l[d]; lbr[d] = L0.box_l[d] + L0.dpkg[d] * L0.num_pkg[d]; }
  int fail = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : fail)
  for (long long i = 0; i < s.n; i++) {
    s.type[i] = REAL_PARTICLE;
    s.scale[i] = c.max_scale;  // Particle_mesh_generation::Initialize :53-63
    bool ok = false;
    for (uint32_t att = 0; att < 10000000u && !ok; att++) {
      double x[3] = {0, 0, 0};
      for (int d = 0; d < D; d++) {
        U4 r = philox((uint32_t)s.id[i], 0u, att, (RNG_SEED << 8) | d, c.seed);
        double u1 = u53(r.v[0], r.v[1]), u2 = u53(r.v[2], r.v[3]);
        double box = c.box_r[d] - c.box_l[d];
        x[d] = u1 * box + u2 * 1.e-3 + c.box_l[d];
        x[d] = AMAX1(c.box_l[d] + 1.e-10, AMIN1(x[d], c.box_r[d] - 1.e-10));
        x[d] = AMAX1(lbl[d] + padding, AMIN1(lbr[d] - padding, x[d]));
      }
      put_xyz<D>(s, i, x);
      sample_particle<D>(c, s, i);
      set_info<D>(c, s, i);
      if (s.phi[i] > s.h[i]) ok = true;
    }
    if (!ok) fail++;
  }
  return fail ? -1 : 0;
}

template <int D>
void one_step(const orc_ctx& c, orc_state& s, Neighbors& nb) {
  s.step += 1;
  phase_map<D>(c, s, 1);
  build_neighbors<D>(c, s, nb);
  reset_stage1<D>(s);
  density<D>(c, s, nb);
  force_stage<D>(c, s, nb, 1);
  force_stage<D>(c, s, nb, 2);
}

}  // namespace

// ===========================================================================
extern "C" {

// SPH::Define_level_infor_tight sph.cpp:144-180 + Level_info::Initialize
// level_infor.cpp:35-110 (cell sizes per level), with max/min_scale from
// Initialize_case sph_mesh_generation.cpp:781-787.
int orc_define_levels(orc_ctx* c) {
  const int D = c->dim;
  double domain[3];
  for (int d = 0; d < 3; d++) domain[d] = c->box_r[d] - c->box_l[d];
  c->max_scale = c->max_dl * c->cell_ratio;
  c->min_scale = c->min_dl * c->cell_ratio;
  double ini_scale = c->max_scale;
  double scale_temp = domain[0];
  if (D >= 2) scale_temp = AMIN1(domain[1], scale_temp);
  if (D == 3) scale_temp = AMIN1(domain[2], scale_temp);
  int temp = (int)std::floor(scale_temp / ini_scale);
  if (temp < 1) return -1;
  ini_scale = scale_temp / (double)temp;
  c->max_scale = ini_scale;
  scale_temp = ini_scale;
  int num_level = 1;
  while ((scale_temp + 1.e-6) > c->min_scale) {
    scale_temp /= 2;
    num_level++;
  }
  c->min_scale = scale_temp * 2;
  num_level -= 1;
  if (num_level < 1 || num_level > 16) return -2;
  c->ncl = num_level;
  for (int d = 0; d < 3; d++) c->ini_num_cell[d] = (d < D) ? (int)(domain[d] / c->max_scale) : 1;
  for (int l = 0; l < num_level; l++) {
    double multi = powern(2.0, l);
    double sc = 1.e300;
    for (int d = 0; d < 3; d++) {
      c->cl_ncell[l][d] = (d < D) ? (int)(c->ini_num_cell[d] * multi) : 1;
      c->cl_dcell[l][d] = (d < D) ? domain[d] / c->cl_ncell[l][d] : 1.0;
      if (d < D) sc = AMIN1(sc, c->cl_dcell[l][d]);
    }
    c->cl_scale[l] = sc;
  }
  return 0;
}

int orc_ls_build(orc_ctx* c, int level, double* max_phi) {
  if (c->dim == 2) ls_build<2>(c->ls[level], max_phi);
  else ls_build<3>(c->ls[level], max_phi);
  return 0;
}

// characteristic cells of a built level (needs chr / chr_idx buffers)
int orc_ls_characteristics(orc_ctx* c, int level) {
  if (c->dim == 2) ls_characteristics<2>(*c, c->ls[level]);
  else ls_characteristics<3>(*c, c->ls[level]);
  return 0;
}

void orc_kernel_W(int kind, int D, long long n, const double* dist, double h, double* out) {
  for (long long i = 0; i < n; i++) out[i] = kernel_W(kind, D, dist[i], h);
}
void orc_kernel_dW(int kind, int D, long long n, const double* dist, double h, double* out) {
  for (long long i = 0; i < n; i++) out[i] = kernel_dW(kind, D, dist[i], h);
}
double orc_get_scale(const orc_ctx* c, double phi, double curv) { return get_scale(*c, c->dim, phi, curv); }
int orc_set_particle_scale(const orc_ctx* c, double h, double scale_in, double* scale_out) {
  *scale_out = scale_in;
  return set_particle_scale(*c, h, scale_out);
}

// max / min |curvature| over the CUT cells of one level (Levelset_package::
// Get_global_scale, lset_package.cpp:765-785); min stays 1e20 without CUT cells
void orc_ls_curv_range(const orc_ctx* c, int level, double* cmax, double* cmin) {
  const orc_level& L = c->ls[level];
  long long ntot = 1;
  for (int d = 0; d < 3; d++) ntot *= (d < c->dim) ? ls_ncell(L, d) : 1;
  double mx = 0., mn = 1.e20;
  for (long long a = 0; a < ntot; a++)
    if (L.tag[a] == CUT_CELL) {
      mx = AMAX1(mx, std::fabs(L.curv[a]));
      mn = AMIN1(mn, std::fabs(L.curv[a]));
    }
  *cmax = mx;
  *cmin = mn;
}

void orc_philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, unsigned long long seed, uint32_t* out) {
  U4 r = philox(c0, c1, c2, c3, seed);
  for (int i = 0; i < 4; i++) out[i] = r.v[i];
}

void orc_sample(const orc_ctx* c, long long n, const double* xyz, double* phi, double* nrm, double* curv, int* tag) {
  for (long long i = 0; i < n; i++) {
    double x[3] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
    if (c->dim == 2) {
      sample<2>(*c, x, &phi[i], &nrm[3 * i], &curv[i]);
      if (tag) tag[i] = cell_tag<2>(*c, x);
    } else {
      sample<3>(*c, x, &phi[i], &nrm[3 * i], &curv[i]);
      if (tag) tag[i] = cell_tag<3>(*c, x);
    }
  }
}

int orc_seed(const orc_ctx* c, orc_state* s) {
  return c->dim == 2 ? seed_particles<2>(*c, *s) : seed_particles<3>(*c, *s);
}
void orc_pre_run(const orc_ctx* c, orc_state* s) {
  if (c->dim == 2) pre_run<2>(*c, *s); else pre_run<3>(*c, *s);
}
void orc_phase_map(const orc_ctx* c, orc_state* s, int do_advect) {
  if (c->dim == 2) phase_map<2>(*c, *s, do_advect); else phase_map<3>(*c, *s, do_advect);
}

// per-particle cell key at its own level: (level, cx, cy, cz)
void orc_cells(const orc_ctx* c, const orc_state* s, int* out4) {
  for (long long i = 0; i < s->n; i++) {
    double x[3] = {s->x[i], s->y[i], c->dim == 3 ? s->z[i] : 0.0};
    int cc[3];
    if (c->dim == 2) cell_of<2>(*c, s->level[i], x, cc); else cell_of<3>(*c, s->level[i], x, cc);
    out4[4 * i] = s->level[i];
    out4[4 * i + 1] = cc[0]; out4[4 * i + 2] = cc[1]; out4[4 * i + 3] = cc[2];
  }
}

// Neighbour lists in CSR form (sorted by particle id).  Two-call protocol:
// with nb == NULL only *total is returned.
static Neighbors g_nb_cache;
long long orc_neighbors(const orc_ctx* c, const orc_state* s, long long* off, int* nb, long long cap) {
  if (c->dim == 2) build_neighbors<2>(*c, *s, g_nb_cache); else build_neighbors<3>(*c, *s, g_nb_cache);
  long long tot = g_nb_cache.off[s->n];
  if (off) for (long long i = 0; i <= s->n; i++) off[i] = g_nb_cache.off[i];
  if (nb && cap >= tot) std::copy(g_nb_cache.nb.begin(), g_nb_cache.nb.end(), nb);
  return tot;
}

// Density and force stages on given CSR neighbour lists.
void orc_density(const orc_ctx* c, orc_state* s, const long long* off, const int* nbr) {
  Neighbors nb;
  nb.off.assign(off, off + s->n + 1);
  nb.nb.assign(nbr, nbr + off[s->n]);
  if (c->dim == 2) density<2>(*c, *s, nb); else density<3>(*c, *s, nb);
}
void orc_force(const orc_ctx* c, orc_state* s, const long long* off, const int* nbr, int stage) {
  Neighbors nb;
  nb.off.assign(off, off + s->n + 1);
  nb.nb.assign(nbr, nbr + off[s->n]);
  if (c->dim == 2) force_stage<2>(*c, *s, nb, stage); else force_stage<3>(*c, *s, nb, stage);
}
void orc_reset_stage1(const orc_ctx* c, orc_state* s) {
  if (c->dim == 2) reset_stage1<2>(*s); else reset_stage1<3>(*s);
}

// Full relaxation steps (SPH_run_mesh_generation x nsteps).
long long orc_steps(const orc_ctx* c, orc_state* s, int nsteps) {
  Neighbors nb;
  long long pairs = 0;
  for (int k = 0; k < nsteps; k++) {
    if (c->dim == 2) one_step<2>(*c, *s, nb); else one_step<3>(*c, *s, nb);
    pairs += nb.off[s->n] - s->n;
  }
  return pairs;
}

// ===========================================================================
// A13 CVP: Voronoi::Partitioning (CVP/voronoi.cpp:1376-1446) on a weighted
// point set.  voro++ is replaced by exact in-box Voronoi faces: the face of
// VP k on plane p (a bisector with VP m, or a box wall) is the plane's
// polygon inside the box clipped by every other bisector half-space.
// Per-VP sums run in particle order split into CVP_CHUNK-particle chunks
// (chunk partials, then partials in chunk order); faces are summed in plane
// order (VPs by index, then walls x-, x+, y-, y+, z-, z+).
// ===========================================================================
struct orc_cvp_params {
  int dim, num_vp, max_iter, pressure_step;
  double error_tolerance, relax_ratio;
  double box_l[3], box_r[3];
};
struct orc_cvp_result { int iterations, converged; double error_max, total_energy; };

static const int CVP_CHUNK = 2048;
static const int CVP_MAXV = 64;

static inline double cvp_dot(const double* a, const double* b) {
  double s = 0.0;
  s += a[0] * b[0];
  s += a[1] * b[1];
  s += a[2] * b[2];
  return s;
}

// keep the part of polygon v (nv vertices) with n.x - d <= 0
static int cvp_clip(double (*v)[3], int nv, const double* n, double d, double (*o)[3]) {
  int no = 0;
  for (int a = 0; a < nv; a++) {
    int b = (a + 1) % nv;
    double sa = cvp_dot(n, v[a]) - d, sb = cvp_dot(n, v[b]) - d;
    if (sa <= 0.0) {
      if (no < CVP_MAXV) { o[no][0] = v[a][0]; o[no][1] = v[a][1]; o[no][2] = v[a][2]; }
      no++;
    }
    if ((sa <= 0.0) != (sb <= 0.0)) {
      double t = sa / (sa - sb);
      if (no < CVP_MAXV)
        for (int q = 0; q < 3; q++) o[no][q] = v[a][q] + (v[b][q] - v[a][q]) * t;
      no++;
    }
  }
  return no < CVP_MAXV ? no : CVP_MAXV;
}

// plane p of VP k: unit normal n (outward of k) and offset d (n.x <= d inside).
// p < K: the bisector with point p of vp (VPs, then ghost VPs); p >= K: box
// wall p - K.  K here is the number of points (VPs and ghosts).
static void cvp_plane(const orc_cvp_params& P, const double* vp, int k, int p, double* n, double* d, int K) {
  if (p < K) {
    const double* ck = vp + 3 * k;
    const double* cm = vp + 3 * p;
    double e[3] = {cm[0] - ck[0], cm[1] - ck[1], cm[2] - ck[2]};
    double len = std::sqrt(cvp_dot(e, e));
    double mid[3] = {0.5 * (ck[0] + cm[0]), 0.5 * (ck[1] + cm[1]), 0.5 * (ck[2] + cm[2])};
    for (int q = 0; q < 3; q++) n[q] = e[q] / len;
    *d = cvp_dot(n, mid);
  } else {
    int w = p - K, ax = w / 2, hi = w % 2;
    n[0] = n[1] = n[2] = 0.0;
    n[ax] = hi ? 1.0 : -1.0;
    *d = hi ? P.box_r[ax] : -P.box_l[ax];
  }
}

// face of VP k on plane p: returns 1 and area, normal, dist if non-empty.
// vp holds K points (VPs, then ghost VPs); p < K a point, p >= K wall p - K.
static int cvp_face(const orc_cvp_params& P, const double* vp, int k, int p, double* area, double* nrm, double* dist,
                    int K) {
  double n[3], d;
  cvp_plane(P, vp, k, p, n, &d, K);
  double lo[3], hi[3];
  for (int q = 0; q < 3; q++) {
    lo[q] = q < P.dim ? P.box_l[q] : -0.5;
    hi[q] = q < P.dim ? P.box_r[q] : 0.5;
  }
  double c[3] = {0.5 * (lo[0] + hi[0]), 0.5 * (lo[1] + hi[1]), 0.5 * (lo[2] + hi[2])};
  double S = 0.0;
  for (int q = 0; q < 3; q++) S += (hi[q] - lo[q]) * (hi[q] - lo[q]);
  S = 2.0 * std::sqrt(S);
  // in-plane frame
  int ax = 0;
  if (std::fabs(n[1]) < std::fabs(n[ax])) ax = 1;
  if (std::fabs(n[2]) < std::fabs(n[ax])) ax = 2;
  double e[3] = {0, 0, 0};
  e[ax] = 1.0;
  double u[3] = {n[1] * e[2] - n[2] * e[1], n[2] * e[0] - n[0] * e[2], n[0] * e[1] - n[1] * e[0]};
  double ul = std::sqrt(cvp_dot(u, u));
  for (int q = 0; q < 3; q++) u[q] = u[q] / ul;
  double w[3] = {n[1] * u[2] - n[2] * u[1], n[2] * u[0] - n[0] * u[2], n[0] * u[1] - n[1] * u[0]};
  double off = d - cvp_dot(n, c);
  double p0[3] = {c[0] + n[0] * off, c[1] + n[1] * off, c[2] + n[2] * off};
  double A[CVP_MAXV][3], B[CVP_MAXV][3];
  const double sg[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
  for (int a = 0; a < 4; a++)
    for (int q = 0; q < 3; q++) A[a][q] = p0[q] + u[q] * (sg[a][0] * S) + w[q] * (sg[a][1] * S);
  int nv = 4;
  // box walls (the plane's own wall excluded)
  for (int wq = 0; wq < 6 && nv > 0; wq++) {
    if (p >= K && wq == p - K) continue;
    int axw = wq / 2, hw = wq % 2;
    double wn[3] = {0, 0, 0};
    wn[axw] = hw ? 1.0 : -1.0;
    double wd = hw ? hi[axw] : -lo[axw];
    nv = cvp_clip(A, nv, wn, wd, B);
    for (int a = 0; a < nv; a++) for (int q = 0; q < 3; q++) A[a][q] = B[a][q];
  }
  // other bisectors
  for (int m = 0; m < K && nv > 0; m++) {
    if (m == k || m == p) continue;
    double bn[3], bd;
    cvp_plane(P, vp, k, m, bn, &bd, K);
    nv = cvp_clip(A, nv, bn, bd, B);
    for (int a = 0; a < nv; a++) for (int q = 0; q < 3; q++) A[a][q] = B[a][q];
  }
  if (nv < 3) return 0;
  double ar = 0.0;
  for (int a = 1; a + 1 < nv; a++) {
    double x[3] = {A[a][0] - A[0][0], A[a][1] - A[0][1], A[a][2] - A[0][2]};
    double y[3] = {A[a + 1][0] - A[0][0], A[a + 1][1] - A[0][1], A[a + 1][2] - A[0][2]};
    double cr[3] = {x[1] * y[2] - x[2] * y[1], x[2] * y[0] - x[0] * y[2], x[0] * y[1] - x[1] * y[0]};
    ar += cvp_dot(cr, n);
  }
  ar = 0.5 * std::fabs(ar);
  double ext = S * S;
  if (!(ar > 1.e-13 * ext)) return 0;
  *area = ar;
  nrm[0] = n[0]; nrm[1] = n[1]; nrm[2] = n[2];
  const double* ck = vp + 3 * k;
  double dx[3] = {A[0][0] - ck[0], A[0][1] - ck[1], A[0][2] - ck[2]};
  *dist = std::fabs(cvp_dot(dx, n)) * 2.;
  return 1;
}

static inline double cvp_dist(int D, const double* a, const double* b) {  // get_distance_2p, glbfunc.h:253-261
  double s = 0.0;
  s += (a[0] - b[0]) * (a[0] - b[0]);
  s += (a[1] - b[1]) * (a[1] - b[1]);
  if (D == 3) s += (a[2] - b[2]) * (a[2] - b[2]);
  return std::sqrt(s);
}

// Ghost VPs of the level-set partition, Voronoi_lset::Ghost_VP_generation
// (voronoi_lset.cpp:250-308): every VP k > 0 (the reference's colour > 0
// test leaves VP 0 out) whose packages include one with surface mass, in VP
// order, mirrored across the surface, x - 2 phi n with phi and the
// interpolated normal n at the VP, when phi >= 1e-6 there.
static int cvp_ghosts(const orc_ctx& c, int D, int K, const double* vp, const std::vector<unsigned char>& flag,
                      double* ghost) {
  int G = 0;
  for (int k = 0; k < K; k++) {
    if (!flag[k]) continue;
    double phi, nn[3], cv;
    if (D == 3) sample<3>(c, vp + 3 * k, &phi, nn, &cv);
    else sample<2>(c, vp + 3 * k, &phi, nn, &cv);
    if (phi >= 1.e-6) {
      for (int q = 0; q < 3; q++) ghost[3 * G + q] = q < D ? vp[3 * k + q] - 2. * phi * nn[q] : vp[3 * k + q];
      G++;
    }
  }
  return G;
}

// The partition loop; with a level set (c != NULL) the level-set partition
// Voronoi_lset::Partitioning_for_initial_VP_distribution
// (voronoi_lset.cpp:824-889): each iteration first makes the ghost VPs from
// the previous assignment (the first from the nearest-VP assignment of the
// initial VPs, as Voronoi_lset::Initialize colours the packages), then
// assigns every point to its nearest VP or ghost (label -1 for a ghost: the
// point belongs to no VP), and the ghosts bound the VPs' cells like walls
// (a face with a ghost takes the VP's own pressure).
static int cvp_core(const orc_cvp_params& P, const orc_ctx* c, long long n, const double* xyz, const double* pmass,
                    const double* psurf, double* vp, int* label, double* vp_mass, double* ghost_out, int* nghost_out,
                    orc_cvp_result* res) {
  const int K = P.num_vp, D = P.dim;
  const int GM = c ? K : 0;           // ghost slots
  const int NP = K + GM + 2 * D;      // planes per VP: VPs, ghost slots, walls
  std::vector<double> src(3 * (size_t)(K + GM));
  std::vector<unsigned char> flag(K, 0);
  int G = 0;
  auto nearest = [&](const double* x, int ns) {
    double best = 1.e20;
    int idx = 0;
    for (int k = 0; k < ns; k++) {
      double dd = cvp_dist(D, x, src.data() + 3 * k);
      if (dd < best) { best = dd; idx = k; }
    }
    return idx;
  };
  if (c) {  // Voronoi_lset::Initialize: packages coloured by their nearest VP
    for (int q = 0; q < 3 * K; q++) src[q] = vp[q];
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; i++) label[i] = nearest(xyz + 3 * i, K);
  }
  const long long nchunk = (n + CVP_CHUNK - 1) / CVP_CHUNK;
  std::vector<double> part((size_t)nchunk * K * 5), tmass(nchunk);
  // Set_target_mass (voronoi.cpp:495-510), chunked order
  for (long long c = 0; c < nchunk; c++) {
    double s = 0.0;
    for (long long i = c * CVP_CHUNK; i < std::min(n, (c + 1) * CVP_CHUNK); i++) s += pmass[i];
    tmass[c] = s;
  }
  double total = 0.0;
  for (long long c = 0; c < nchunk; c++) total += tmass[c];
  const double target = total / K;
  std::vector<double> mass(K), mc(3 * K), energy(K), Pk(K), err(K), f(3 * K), hk(K), shift(3 * K), tcvt(K);
  std::vector<double> farea((size_t)K * NP), fnrm((size_t)K * NP * 3), fdist((size_t)K * NP);
  std::vector<int> fex((size_t)K * NP);
  double relax = P.relax_ratio, error_record = 0.0;
  int converged = 0, iter = 0;
  double error_max = 0.0, total_energy = 0.0;
  for (iter = 0; iter <= P.max_iter && converged == 0; iter++) {
    double scale_coeff = 0.25 + 1.75 * (1. - AMIN1((iter - 1) / 500., 1.));
    for (int q = 0; q < 3 * K; q++) src[q] = vp[q];
    G = 0;
    if (c) {
      std::fill(flag.begin(), flag.end(), (unsigned char)0);
      for (long long i = 0; i < n; i++)
        if (psurf[i] > 0. && label[i] > 0) flag[label[i]] = 1;
      G = cvp_ghosts(*c, D, K, vp, flag, src.data() + 3 * K);
    }
    // assignment: Get_CPU_id (voronoi.cpp:480-493) / find_voronoi_cell over
    // VPs and ghosts (voronoi_lset.cpp:435-445), strict <
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; i++) {
      const int idx = nearest(xyz + 3 * i, K + G);
      label[i] = idx < K ? idx : -1;
    }
    // mass, mass centre, energy (voronoi.cpp:617-631)
#pragma omp parallel for schedule(static)
    for (long long c = 0; c < nchunk; c++)
      for (int k = 0; k < K; k++) {
        double m = 0.0, x = 0.0, y = 0.0, z = 0.0, e = 0.0;
        for (long long i = c * CVP_CHUNK; i < std::min(n, (c + 1) * CVP_CHUNK); i++) {
          if (label[i] != k) continue;
          double pm = pmass[i];
          m += pm;
          x = x + xyz[3 * i] * pm;
          y = y + xyz[3 * i + 1] * pm;
          z = z + xyz[3 * i + 2] * pm;
          e += pm * cvp_dist(D, vp + 3 * k, xyz + 3 * i);
        }
        double* q = &part[((size_t)c * K + k) * 5];
        q[0] = m; q[1] = x; q[2] = y; q[3] = z; q[4] = e;
      }
    error_max = 0.0;
    total_energy = 0.0;
    for (int k = 0; k < K; k++) {
      double m = 0.0, x = 0.0, y = 0.0, z = 0.0, e = 0.0;
      for (long long c = 0; c < nchunk; c++) {
        const double* q = &part[((size_t)c * K + k) * 5];
        m += q[0]; x = x + q[1]; y = y + q[2]; z = z + q[3]; e += q[4];
      }
      mass[k] = m;
      energy[k] = e;
      if (m > 0.) {
        double inv = 1. / m;  // voronoi.cpp:672-687
        mc[3 * k] = x * inv;
        mc[3 * k + 1] = y * inv;
        mc[3 * k + 2] = (D == 3) ? z * inv : 0.0;
        Pk[k] = target / m;
      } else {
        // a cell without points (the reference divides by its zero mass):
        // centroid = its position, no pressure; it does not move (below)
        for (int q = 0; q < 3; q++) mc[3 * k + q] = vp[3 * k + q];
        Pk[k] = 0.;
      }
      err[k] = std::fabs(m - target) / target;
    }
    for (int k = 0; k < K; k++) {
      error_max = AMAX1(error_max, err[k]);
      total_energy += energy[k];
    }
    // faces (replacing the voro++ loop, voronoi.cpp:724-790)
#pragma omp parallel for schedule(dynamic, 4)
    for (long long t = 0; t < (long long)K * NP; t++) {
      int k = (int)(t / NP), p = (int)(t % NP);
      fex[t] = 0;
      if (p < K && p == k) continue;
      if (p >= K && p < K + GM && p - K >= G) continue;  // unused ghost slot
      // point index among the K + G points, or wall K + G + w (x-, x+, y-, y+, z-, z+)
      int pp = p < K + GM ? p : K + G + (p - K - GM);
      double ar, nn[3], ds;
      if (cvp_face(P, src.data(), k, pp, &ar, nn, &ds, K + G)) {
        fex[t] = 1;
        farea[t] = ar;
        fnrm[3 * t] = nn[0]; fnrm[3 * t + 1] = nn[1]; fnrm[3 * t + 2] = nn[2];
        fdist[t] = ds;
      }
    }
    for (int k = 0; k < K; k++) {
      double fx = 0.0, fy = 0.0, fz = 0.0, sr = 0.0;
      int nnb = 0;
      for (int p = 0; p < NP; p++) {
        size_t t = (size_t)k * NP + p;
        if (!fex[t]) continue;
        nnb++;
        double nP = (p < K) ? Pk[p] : Pk[k];
        sr += fdist[t];
        double pmid = 0.5 * (Pk[k] + nP);
        double coef = -1 * pmid * farea[t];
        fx = fx + fnrm[3 * t] * coef;
        fy = fy + fnrm[3 * t + 1] * coef;
        fz = fz + fnrm[3 * t + 2] * coef;
      }
      f[3 * k] = fx; f[3 * k + 1] = fy; f[3 * k + 2] = fz;
      hk[k] = scale_coeff * sr / (double)nnb;
    }
    // Check_partition_error (voronoi.cpp:1228-1262)
    error_record = error_record + error_max;
    if (iter % 40 == 0) {
      error_record /= 40.;
      if (error_max <= P.error_tolerance && error_record <= P.error_tolerance) converged = 1;
      error_record = 0.;
    }
    if (converged == 0) {
      // Update_position (voronoi.cpp:830-897)
      double gdt = 1.e20;
      std::vector<double> a(3 * K);
      for (int k = 0; k < K; k++) {
        if (!(mass[k] > 0.)) continue;  // an empty cell neither moves nor limits the step
        double inv = 1. / mass[k];
        for (int q = 0; q < 3; q++) a[3 * k + q] = f[3 * k + q] * inv;
        double acc = 0.0;
        for (int q = 0; q < D; q++) acc += a[3 * k + q] * a[3 * k + q];
        acc = std::sqrt(acc);
        double ts = 0.25 * std::sqrt(hk[k] / (acc + 1.e-20));
        gdt = AMIN1(ts, gdt);
      }
      double gcvt = 1.e20;
      for (int k = 0; k < K; k++) {
        double fac = gdt * gdt * 0.5 * relax;
        for (int q = 0; q < D; q++) {
          double v = P.pressure_step ? vp[3 * k + q] + a[3 * k + q] * fac : vp[3 * k + q];
          vp[3 * k + q] = AMAX1(P.box_l[q] + 1.e-20, AMIN1(v, P.box_r[q] - 1.e-20));
        }
        double sh = 0.0;
        for (int q = 0; q < D; q++) {
          shift[3 * k + q] = mc[3 * k + q] - vp[3 * k + q];
          sh += shift[3 * k + q] * shift[3 * k + q];
        }
        sh = std::sqrt(sh);
        double sc = AMIN1(sh, 1. / 32. * hk[k]);
        tcvt[k] = (mass[k] > 0.) ? sc / (sh + 1.e-20) : 1.e20;
        gcvt = AMIN1(tcvt[k], gcvt);
      }
      // Update_position_CVT (voronoi.cpp:901-992)
      for (int k = 0; k < K; k++)
        for (int q = 0; q < D; q++) {
          double v = vp[3 * k + q] + shift[3 * k + q] * (gcvt * (1 - relax));
          vp[3 * k + q] = AMAX1(P.box_l[q] + 1.e-20, AMIN1(v, P.box_r[q] - 1.e-20));
        }
    }
    if (iter % 600 == 0) relax = 1.02 * relax;
    relax = AMIN1(relax, 0.90);
  }
  if (vp_mass) for (int k = 0; k < K; k++) vp_mass[k] = mass[k];
  if (ghost_out) for (int q = 0; q < 3 * G; q++) ghost_out[q] = src[3 * K + q];
  if (nghost_out) *nghost_out = G;
  if (res) { res->iterations = iter; res->converged = converged; res->error_max = error_max; res->total_energy = total_energy; }
  return 0;
}

int orc_cvp(const orc_cvp_params* Pp, long long n, const double* xyz, const double* pmass, double* vp, int* label,
            double* vp_mass, orc_cvp_result* res) {
  return cvp_core(*Pp, nullptr, n, xyz, pmass, nullptr, vp, label, vp_mass, nullptr, nullptr, res);
}

// level-set partition of weighted points (package centres) with ghost VPs;
// psurf: the points' surface mass; ghost (K x 3, may be NULL) and nghost
// receive the last iteration's ghosts
int orc_cvp_lset(const orc_ctx* c, const orc_cvp_params* Pp, long long n, const double* xyz, const double* pmass,
                 const double* psurf, double* vp, int* label, double* vp_mass, double* ghost, int* nghost,
                 orc_cvp_result* res) {
  return cvp_core(*Pp, c, n, xyz, pmass, psurf, vp, label, vp_mass, ghost, nghost, res);
}

// ===========================================================================
// A14 triangulation (2D): Local_voronoi_diagram / Voronoi_construction::
// Local_VD_generation (voronoi_construction.cpp:6-127) + Graphmeshcls::
// Reconstruct_tris (graph_mesh.cpp:37-409) + Tri_quality_statistics (:411-670).
// voro++ is replaced by exact local Delaunay predicates: j is a Voronoi
// neighbour of i among i's neighbour set S iff some circle through i and j
// has no point of S strictly inside or on it.  Signs are exact (FP64 filter,
// then expansion arithmetic after Priest / Shewchuk 1997), so any correct
// implementation returns the same edges.
// ===========================================================================
namespace xp {
inline void two_sum(double a, double b, double& x, double& y) {
  x = a + b;
  double bv = x - a, av = x - bv, br = b - bv, ar = a - av;
  y = ar + br;
}
inline void two_diff(double a, double b, double& x, double& y) {
  x = a - b;
  double bv = a - x, av = x + bv, br = bv - b, ar = a - av;
  y = ar + br;
}
inline void two_prod(double a, double b, double& x, double& y) {
  x = a * b;
  y = std::fma(a, b, -x);
}
// h = e + b (e nonoverlapping, increasing magnitude); returns length
inline int grow(const double* e, int m, double b, double* h) {
  double Q = b;
  int k = 0;
  for (int i = 0; i < m; i++) {
    double Qn, hh;
    two_sum(Q, e[i], Qn, hh);
    Q = Qn;
    if (hh != 0.0) h[k++] = hh;
  }
  if (Q != 0.0 || k == 0) h[k++] = Q;
  return k;
}
// h = e * b
inline int scale(const double* e, int m, double b, double* h) {
  double Q, hh;
  int k = 0;
  two_prod(e[0], b, Q, hh);
  if (hh != 0.0) h[k++] = hh;
  for (int i = 1; i < m; i++) {
    double T, t, Q2, s;
    two_prod(e[i], b, T, t);
    two_sum(Q, t, Q2, s);
    if (s != 0.0) h[k++] = s;
    double x = T + Q2, bv = x - T;
    s = Q2 - bv;
    Q = x;
    if (s != 0.0) h[k++] = s;
  }
  if (Q != 0.0 || k == 0) h[k++] = Q;
  return k;
}
// running sum acc (length *n) += product of four doubles
inline void acc4(double* acc, int* n, double* tmp, double p, double q, double r, double s, double sign) {
  double e[8], f[8];
  int m;
  two_prod(p, q, e[1], e[0]);
  m = 2;
  m = scale(e, m, r, f);
  m = scale(f, m, s * sign, e);
  for (int i = 0; i < m; i++) {
    int l = grow(acc, *n, e[i], tmp);
    for (int t = 0; t < l; t++) acc[t] = tmp[t];
    *n = l;
  }
}
inline int sign_of(const double* e, int n) {
  for (int i = n - 1; i >= 0; i--)
    if (e[i] != 0.0) return e[i] > 0 ? 1 : -1;
  return 0;
}
}  // namespace xp

// sign of (a-c) x (b-c)
static int orient2d(const double* a, const double* b, const double* c) {
  double acx = a[0] - c[0], bcx = b[0] - c[0], acy = a[1] - c[1], bcy = b[1] - c[1];
  double l = acx * bcy, r = acy * bcx;
  double det = l - r;
  double bound = 1.0e-15 * (std::fabs(l) + std::fabs(r));
  if (det > bound) return 1;
  if (-det > bound) return -1;
  double ax[2], ay[2], bx[2], by[2];
  xp::two_diff(a[0], c[0], ax[1], ax[0]);
  xp::two_diff(a[1], c[1], ay[1], ay[0]);
  xp::two_diff(b[0], c[0], bx[1], bx[0]);
  xp::two_diff(b[1], c[1], by[1], by[0]);
  double acc[80], tmp[80];
  int n = 0;
  for (int u = 0; u < 2; u++)
    for (int v = 0; v < 2; v++) {
      xp::acc4(acc, &n, tmp, ax[u], by[v], 1.0, 1.0, 1.0);
      xp::acc4(acc, &n, tmp, ay[u], bx[v], 1.0, 1.0, -1.0);
    }
  return xp::sign_of(acc, n);
}

// > 0 when d lies inside the circle through a, b, c (a, b, c counter-clockwise)
static int incircle(const double* a, const double* b, const double* c, const double* d) {
  double adx = a[0] - d[0], ady = a[1] - d[1], bdx = b[0] - d[0], bdy = b[1] - d[1];
  double cdx = c[0] - d[0], cdy = c[1] - d[1];
  double al = adx * adx + ady * ady, bl = bdx * bdx + bdy * bdy, cl = cdx * cdx + cdy * cdy;
  double t1 = bdx * cdy, t2 = cdx * bdy, t3 = cdx * ady, t4 = adx * cdy, t5 = adx * bdy, t6 = bdx * ady;
  double det = al * (t1 - t2) + bl * (t3 - t4) + cl * (t5 - t6);
  double perm = (std::fabs(t1) + std::fabs(t2)) * al + (std::fabs(t3) + std::fabs(t4)) * bl +
                (std::fabs(t5) + std::fabs(t6)) * cl;
  double bound = 2.0e-14 * perm;
  if (det > bound) return 1;
  if (-det > bound) return -1;
  double X[3][2], Y[3][2];
  const double* P[3] = {a, b, c};
  for (int q = 0; q < 3; q++) {
    xp::two_diff(P[q][0], d[0], X[q][1], X[q][0]);
    xp::two_diff(P[q][1], d[1], Y[q][1], Y[q][0]);
  }
  static thread_local double acc[4096], tmp[4096];
  int n = 0;
  // det = sum over cyclic (a,b,c): (ax^2 + ay^2) * (bx*cy - cx*by)
  for (int q = 0; q < 3; q++) {
    int r = (q + 1) % 3, s = (q + 2) % 3;
    for (int u = 0; u < 2; u++)
      for (int v = 0; v < 2; v++)
        for (int w = 0; w < 2; w++)
          for (int z = 0; z < 2; z++) {
            xp::acc4(acc, &n, tmp, X[q][u], X[q][v], X[r][w], Y[s][z], 1.0);
            xp::acc4(acc, &n, tmp, Y[q][u], Y[q][v], X[r][w], Y[s][z], 1.0);
            xp::acc4(acc, &n, tmp, X[q][u], X[q][v], X[s][w], Y[r][z], -1.0);
            xp::acc4(acc, &n, tmp, Y[q][u], Y[q][v], X[s][w], Y[r][z], -1.0);
          }
  }
  return xp::sign_of(acc, n);
}

// j is a Voronoi neighbour of i among points S (ids), positions xyz
static bool local_delaunay(const double* xyz, int i, int j, const int* S, int ns) {
  const double* pi = xyz + 3 * (long long)i;
  const double* pj = xyz + 3 * (long long)j;
  int lstar = -1, rstar = -1;
  for (int q = 0; q < ns; q++) {
    int k = S[q];
    if (k == i || k == j) continue;
    const double* pk = xyz + 3 * (long long)k;
    int o = orient2d(pi, pj, pk);
    if (o == 0) {
      // collinear: blocks the edge when strictly between i and j
      double t = (pk[0] - pi[0]) * (pj[0] - pi[0]) + (pk[1] - pi[1]) * (pj[1] - pi[1]);
      double L = (pj[0] - pi[0]) * (pj[0] - pi[0]) + (pj[1] - pi[1]) * (pj[1] - pi[1]);
      if (t > 0 && t < L) return false;
      continue;
    }
    if (o > 0) {
      if (lstar < 0 || incircle(pi, pj, xyz + 3 * (long long)lstar, pk) > 0) lstar = k;
    } else {
      if (rstar < 0 || incircle(pj, pi, xyz + 3 * (long long)rstar, pk) > 0) rstar = k;
    }
  }
  if (lstar < 0 || rstar < 0) return true;
  return incircle(pi, pj, xyz + 3 * (long long)lstar, xyz + 3 * (long long)rstar) < 0;
}

struct orc_tri_quality {
  long long ntri, nedge, nedge_first, ndeleted, nerror;
  double max_angle, min_angle, max_aspect, max_edge, min_edge, max_area, min_area, G_min, G_avg, min_angle_avg;
  double theta_30, total_area;
  long long hist[45];
};

// neighbour CSR (id space, rows sorted, self included or not), positions in id order
long long orc_triangulate(const orc_ctx* c, long long n, const double* xyz, const int* type, const double* phi,
                          const long long* off, const int* nbr, int* tris, long long cap, orc_tri_quality* Q) {
  // 1. local Delaunay edges, symmetrised
  std::vector<std::vector<int>> adj(n);
  std::vector<std::vector<char>> mark(n);
#pragma omp parallel for schedule(dynamic, 64)
  for (long long i = 0; i < n; i++) {
    const int* S = nbr + off[i];
    int ns = (int)(off[i + 1] - off[i]);
    mark[i].assign(ns, 0);
    for (int q = 0; q < ns; q++) {
      int j = S[q];
      if (j == i) continue;
      mark[i][q] = local_delaunay(xyz, (int)i, j, S, ns) ? 1 : 0;
    }
  }
  auto find = [&](long long a, int b) -> int {
    const int* S = nbr + off[a];
    int ns = (int)(off[a + 1] - off[a]);
    int lo = 0, hi = ns - 1;
    while (lo <= hi) {
      int m = (lo + hi) / 2;
      if (S[m] == b) return m;
      if (S[m] < b) lo = m + 1; else hi = m - 1;
    }
    return -1;
  };
  long long nedge1 = 0;
  for (long long i = 0; i < n; i++) {
    const int* S = nbr + off[i];
    int ns = (int)(off[i + 1] - off[i]);
    for (int q = 0; q < ns; q++) {
      int j = S[q];
      if (j == i) continue;
      int p = find(j, (int)i);
      bool e = mark[i][q] || (p >= 0 && mark[j][p]);
      if (e) { adj[i].push_back(j); if (j > i) nedge1++; }
    }
  }
  auto has = [&](const std::vector<std::vector<int>>& A, int a, int b) {
    return std::binary_search(A[a].begin(), A[a].end(), b);
  };
  // 2. pass 1: triangles i > j > k, centroid rule for all-boundary triangles
  std::set<std::pair<int, int>> del;
  std::vector<std::array<int, 3>> kept;
  for (long long i = 0; i < n; i++) {
    for (int j : adj[i]) {
      if (j >= i) break;
      for (int k : adj[i]) {
        if (k >= j) break;
        if (!has(adj, j, k)) continue;
        int I = (int)i;
        bool keep = true;
        if (type[I] != REAL_PARTICLE && type[j] != REAL_PARTICLE && type[k] != REAL_PARTICLE) {
          const double* p1 = xyz + 3 * (long long)I;
          const double* p2 = xyz + 3 * (long long)j;
          const double* p3 = xyz + 3 * (long long)k;
          double cen[3] = {1. / 3. * (p1[0] + p2[0] + p3[0]), 1. / 3. * (p1[1] + p2[1] + p3[1]),
                           1. / 3. * (p1[2] + p2[2] + p3[2])};
          double pc, nn[3], cv;
          sample<2>(*c, cen, &pc, nn, &cv);
          double phi_size = 1. / 3. * (phi[I] + phi[j] + phi[k]);
          if (!(pc > 0.0001 * phi_size)) {
            keep = false;
            double v1[2] = {p2[0] - p1[0], p2[1] - p1[1]};
            double v2[2] = {p3[0] - p2[0], p3[1] - p2[1]};
            double v3[2] = {p1[0] - p3[0], p1[1] - p3[1]};
            double d = std::sqrt(v1[0] * v1[0] + v1[1] * v1[1]);
            std::pair<int, int> e(I, j);
            double d2 = std::sqrt(v2[0] * v2[0] + v2[1] * v2[1]);
            if (d2 > d) { d = d2; e = std::make_pair(j, k); }
            double d3 = std::sqrt(v3[0] * v3[0] + v3[1] * v3[1]);
            if (d3 > d) { d = d3; e = std::make_pair(I, k); }
            del.insert(e);
          }
        }
        if (keep) kept.push_back({I, j, k});
      }
    }
  }
  // 3. rebuild from kept triangles without a deleted edge
  std::vector<std::vector<int>> adj2(n);
  for (auto& t : kept) {
    if (del.count({t[0], t[1]}) || del.count({t[0], t[2]}) || del.count({t[1], t[2]})) continue;
    int e[3][2] = {{t[0], t[1]}, {t[1], t[2]}, {t[0], t[2]}};
    for (auto& q : e) { adj2[q[0]].push_back(q[1]); adj2[q[1]].push_back(q[0]); }
  }
  long long nedge2 = 0;
  for (long long i = 0; i < n; i++) {
    std::sort(adj2[i].begin(), adj2[i].end());
    adj2[i].erase(std::unique(adj2[i].begin(), adj2[i].end()), adj2[i].end());
    for (int j : adj2[i]) if (j > i) nedge2++;
  }
  // 4. pass 2: final triangles = 3-cycles; error checks (graph_mesh.cpp:300-365)
  long long ntri = 0, nerr = 0;
  for (long long i = 0; i < n; i++) {
    for (int j : adj2[i]) {
      if (j >= i) break;
      int common = 0, c0 = -1, c1 = -1;
      for (int k : adj2[i]) {
        if (k == j) continue;
        if (!has(adj2, j, k)) continue;
        if (common == 0) c0 = k; else if (common == 1) c1 = k;
        common++;
        if (k < j) {
          if (tris && ntri < cap) { tris[3 * ntri] = (int)i; tris[3 * ntri + 1] = j; tris[3 * ntri + 2] = k; }
          ntri++;
        }
      }
      if (common > 2 || (common == 2 && has(adj2, c0, c1))) nerr++;
    }
  }
  if (!Q) return ntri;
  // 5. quality statistics (Tri_quality_statistics, graph_mesh.cpp:411-670)
  std::memset(Q, 0, sizeof(*Q));
  Q->ntri = ntri; Q->nedge = nedge2; Q->nedge_first = nedge1; Q->ndeleted = (long long)del.size(); Q->nerror = nerr;
  double maxa = 0., mina = 1.e15, maxasp = 0., maxe = 0., mine = 1.e15, maxar = 0., minar = 1.e15, Gmin = 1.e20;
  double Gsum = 0., minavg = 0., tot = 0.;
  long long th30 = 0;
  const double rad = 180. / std::acos(-1.);
  for (long long t = 0; t < std::min(ntri, cap); t++) {
    const double* v0 = xyz + 3 * (long long)tris[3 * t];
    const double* v1 = xyz + 3 * (long long)tris[3 * t + 1];
    const double* v2 = xyz + 3 * (long long)tris[3 * t + 2];
    double a1[2] = {v1[0] - v0[0], v1[1] - v0[1]}, a2[2] = {v2[0] - v1[0], v2[1] - v1[1]},
           a3[2] = {v0[0] - v2[0], v0[1] - v2[1]};
    double d1 = std::sqrt(a1[0] * a1[0] + a1[1] * a1[1]);
    double d2 = std::sqrt(a2[0] * a2[0] + a2[1] * a2[1]);
    double d3 = std::sqrt(a3[0] * a3[0] + a3[1] * a3[1]);
    double dmax = AMAX1(d1, AMAX1(d2, d3)), dmin = AMIN1(d1, AMIN1(d2, d3));
    maxe = AMAX1(maxe, dmax);
    mine = AMIN1(mine, dmin);
    maxasp = AMAX1(maxasp, dmax / (dmin + 1.e-20));
    double c13 = -(a1[0] * a3[0] + a1[1] * a3[1]) / (d3 * d1 + 1.e-20);
    double al1 = rad * std::acos(c13);
    double al2 = rad * std::acos(-(a1[0] * a2[0] + a1[1] * a2[1]) / (d2 * d1 + 1.e-20));
    double al3 = rad * std::acos(-(a2[0] * a3[0] + a2[1] * a3[1]) / (d3 * d2 + 1.e-20));
    al1 = AMAX1(0., AMIN1(al1, 180.));
    al2 = AMAX1(0., AMIN1(al2, 180.));
    al3 = AMAX1(0., AMIN1(al3, 180.));
    maxa = AMAX1(maxa, AMAX1(al1, AMAX1(al2, al3)));
    double mm = AMIN1(al1, AMIN1(al2, al3));
    mina = AMIN1(mina, mm);
    Q->hist[std::min(44, (int)(al1 / 4.0))]++;
    Q->hist[std::min(44, (int)(al2 / 4.0))]++;
    Q->hist[std::min(44, (int)(al3 / 4.0))]++;
    if (mm < 30.) th30++;
    minavg += mm;
    double area = 0.5 * (d3 * d1) * std::sin(std::acos(c13));
    tot += area;
    maxar = AMAX1(maxar, area);
    minar = AMIN1(minar, area);
    double G = 2. * std::sqrt(3.) * area / (dmax * (d1 + d2 + d3) / 2.);
    Gmin = AMIN1(G, Gmin);
    Gsum = Gsum + G;
  }
  Q->max_angle = maxa; Q->min_angle = mina; Q->max_aspect = maxasp; Q->max_edge = maxe; Q->min_edge = mine;
  Q->max_area = maxar; Q->min_area = minar; Q->G_min = Gmin;
  Q->G_avg = ntri ? Gsum / ntri : 0.0;
  Q->min_angle_avg = ntri ? minavg / ntri : 0.0;
  Q->theta_30 = ntri ? (double)th30 / (double)ntri : 0.0;
  Q->total_area = tot;
  return ntri;
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"

// ===========================================================================
// F1: cut-cell volume, surface area and the particle count of one level-set
// level.  Levelset::Calculate_total_volume_mass (level_set_solver/
// level_set.cpp:930-972) over Levelset_package::Calculate_volume_mass
// (level_set_solver/lset_package.cpp:1283-1397) with GeometryCalculator
// (geometry_tools/geometry_calculator.cpp:12-570), and
// SPH_mesh_generation::Get_num_particles (sph_mesh_generation.cpp:900-940).
//
// Surface area: the reference polygonises each half-cell sub-cube with the
// marching-cubes tables of geometry_tools/polygonise.h.  The polygons follow
// from the signs alone (a face with two diagonal corners below zero cuts
// those two corners off, the rule the tables follow on every ambiguous face,
// checked over all 256 sign cases), so mc_table() below derives them by
// walking the cut edges; each polygon is then split as a fan from its lowest
// edge.  The reference's tables split some polygons along other diagonals,
// so a cell's area may differ in the last digits that a non-planar polygon
// leaves (about 1e-6 of the total area on smooth surfaces); volumes, masses
// and counts do not depend on the split.
// ===========================================================================
namespace {

// cube vertices of a sub-cube in the order of geometry_calculator.cpp:296-297
const int MC_V[8][3] = {{0, 0, 0}, {0, 1, 0}, {1, 1, 0}, {1, 0, 0}, {0, 0, 1}, {0, 1, 1}, {1, 1, 1}, {1, 0, 1}};
// edge endpoints (polygonise.cpp:37-60: the first endpoint is interpolated from)
const int MC_E[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                         {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
const int MC_F[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}};

struct McTable {
  signed char t[256][16];  // edge triples, -1 terminated
};

int mc_edge(int a, int b) {
  for (int e = 0; e < 12; e++)
    if ((MC_E[e][0] == a && MC_E[e][1] == b) || (MC_E[e][0] == b && MC_E[e][1] == a)) return e;
  return -1;
}

// Bit v of a case is set when vertex v lies below zero (polygonise.cpp:19-27).
const McTable& mc_table() {
  static McTable T = [] {
    McTable M;
    for (int ci = 0; ci < 256; ci++) {
      int nb[12][2], nn[12] = {0};
      for (int f = 0; f < 6; f++) {
        int in[4], es[4], cut[4], nc = 0;
        for (int k = 0; k < 4; k++) in[k] = (ci >> MC_F[f][k]) & 1;
        for (int k = 0; k < 4; k++) es[k] = mc_edge(MC_F[f][k], MC_F[f][(k + 1) & 3]);
        for (int k = 0; k < 4; k++)
          if (in[k] != in[(k + 1) & 3]) cut[nc++] = es[k];
        auto link = [&](int a, int b) {
          nb[a][nn[a]++] = b;
          nb[b][nn[b]++] = a;
        };
        if (nc == 2) link(cut[0], cut[1]);
        else if (nc == 4)
          for (int k = 0; k < 4; k++)
            if (in[k]) link(es[(k + 3) & 3], es[k]);
      }
      int n = 0;
      bool seen[12] = {false};
      for (int s = 0; s < 12; s++) {
        if (!nn[s] || seen[s]) continue;
        int cyc[12], m = 0, prev = s, cur = nb[s][0] < nb[s][1] ? nb[s][0] : nb[s][1];
        cyc[m++] = s;
        seen[s] = true;
        while (cur != s) {
          cyc[m++] = cur;
          seen[cur] = true;
          int nxt = nb[cur][0] == prev ? nb[cur][1] : nb[cur][0];
          prev = cur;
          cur = nxt;
        }
        for (int k = 1; k + 1 < m; k++) {
          M.t[ci][n++] = (signed char)cyc[0];
          M.t[ci][n++] = (signed char)cyc[k];
          M.t[ci][n++] = (signed char)cyc[k + 1];
        }
      }
      for (; n < 16; n++) M.t[ci][n] = -1;
    }
    return M;
  }();
  return T;
}

struct P3 {
  double x, y, z;
};

// Polygonise_MQ::VertexInterp, polygonise.cpp:74-92 (isolevel 0)
P3 mc_interp(P3 p1, P3 p2, double v1, double v2) {
  const double iso = 0.0;
  if (std::fabs(iso - v1) < 1.0e-15) return p1;
  if (std::fabs(iso - v2) < 1.0e-15) return p2;
  if (std::fabs(v1 - v2) < 1.0e-15) return p1;
  double mu = (iso - v1) / (v2 - v1);
  return P3{p1.x + mu * (p2.x - p1.x), p1.y + mu * (p2.y - p1.y), p1.z + mu * (p2.z - p1.z)};
}

// GeometryCalculator::get_area_tri, geometry_calculator.cpp:325-350
double mc_tri_area(P3 p1, P3 p2, P3 p3) {
  double v1x = p2.x - p1.x, v1y = p2.y - p1.y, v1z = p2.z - p1.z;
  double v3x = p3.x - p1.x, v3y = p3.y - p1.y, v3z = p3.z - p1.z;
  double d1 = std::sqrt(v1x * v1x + v1y * v1y + v1z * v1z);
  double d3 = std::sqrt(v3x * v3x + v3y * v3y + v3z * v3z);
  double area = 0.5 * (d3 * d1) * std::sin(std::acos((v1x * v3x + v1y * v3y + v1z * v3z) / (d3 * d1 + 1.e-20)));
  if (std::isnan(area)) area = 0.;
  return area;
}

// GeometryCalculator::get_area_MQ, geometry_calculator.cpp:283-321
double mc_area(const double ph[3][3][3], double dx, double dy, double dz) {
  const McTable& T = mc_table();
  double area = 0.0;
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++)
      for (int k = 0; k < 2; k++) {
        P3 p[8];
        double val[8];
        int ci = 0;
        for (int v = 0; v < 8; v++) {
          int vx = i + MC_V[v][0], vy = j + MC_V[v][1], vz = k + MC_V[v][2];
          p[v] = P3{vx * 0.5 * dx, vy * 0.5 * dy, vz * 0.5 * dz};
          val[v] = ph[vx][vy][vz];
          if (val[v] < 0.0) ci |= 1 << v;
        }
        const signed char* t = T.t[ci];
        for (int q = 0; t[q] >= 0; q += 3) {
          P3 a = mc_interp(p[MC_E[t[q]][0]], p[MC_E[t[q]][1]], val[MC_E[t[q]][0]], val[MC_E[t[q]][1]]);
          P3 b = mc_interp(p[MC_E[t[q + 1]][0]], p[MC_E[t[q + 1]][1]], val[MC_E[t[q + 1]][0]], val[MC_E[t[q + 1]][1]]);
          P3 c = mc_interp(p[MC_E[t[q + 2]][0]], p[MC_E[t[q + 2]][1]], val[MC_E[t[q + 2]][0]], val[MC_E[t[q + 2]][1]]);
          area += mc_tri_area(a, b, c);
        }
      }
  return area;
}

// GeometryCalculator::check_volume / check_face / mark_volume / mark_face
// (geometry_calculator.cpp:352-448): 1 all positive, 0 all negative, -1 cut
int gc_mark(const double* v, int n) {
  int flag = 0;
  for (int q = 0; q < n; q++) {
    if (v[q] > 0.0) flag += 1;
    else if (v[q] < 0.0) flag -= 1;
  }
  return flag == n ? 1 : (flag == -n ? 0 : -1);
}

// GeometryCalculator::get_subvolume, geometry_calculator.cpp:505-570
double gc_subvolume(int level_phi, double multi, const double cor[2][2][2]) {
  int flag = gc_mark(&cor[0][0][0], 8);
  if (flag == 1) return multi;
  if (flag == 0) return 0.0;
  double vof = 0.0;
  if (level_phi <= 5) {
    multi *= 0.125;
    level_phi += 1;
    double rf[3][3][3];
    for (int i = 0; i < 2; i++)
      for (int j = 0; j < 2; j++)
        for (int k = 0; k < 2; k++) rf[2 * i][2 * j][2 * k] = cor[i][j][k];
    for (int i = 0; i < 3; i += 2)
      for (int j = 0; j < 3; j += 2) rf[i][j][1] = 0.5 * (rf[i][j][0] + rf[i][j][2]);
    for (int k = 0; k < 3; k++)
      for (int i = 0; i < 3; i += 2) rf[i][1][k] = 0.5 * (rf[i][0][k] + rf[i][2][k]);
    for (int j = 0; j < 3; j++)
      for (int k = 0; k < 3; k++) rf[1][j][k] = 0.5 * (rf[0][j][k] + rf[2][j][k]);
    for (int i = 0; i < 2; i++)
      for (int j = 0; j < 2; j++)
        for (int k = 0; k < 2; k++) {
          double sub[2][2][2];
          for (int r = 0; r < 2; r++)
            for (int s = 0; s < 2; s++)
              for (int t = 0; t < 2; t++) sub[r][s][t] = rf[i + r][j + s][k + t];
          vof += gc_subvolume(level_phi, multi, sub);
        }
  } else {
    double cv = 0.0;
    for (int i = 0; i < 2; i++)
      for (int j = 0; j < 2; j++)
        for (int k = 0; k < 2; k++) cv += cor[i][j][k];
    vof = cv > 0.0 ? 0.75 * multi : (cv == 0.0 ? 0.5 * multi : 0.25 * multi);
  }
  return vof;
}

// GeometryCalculator::get_face, geometry_calculator.cpp:450-503
double gc_face(int level_phi, double multi, const double cor[2][2]) {
  int flag = gc_mark(&cor[0][0], 4);
  if (flag == 1) return multi;
  if (flag == 0) return 0.0;
  double vof = 0.0;
  if (level_phi <= 5) {
    multi *= 0.25;
    level_phi += 1;
    double rf[3][3];
    for (int i = 0; i < 2; i++)
      for (int j = 0; j < 2; j++) rf[2 * i][2 * j] = cor[i][j];
    for (int i = 0; i < 3; i += 2) rf[i][1] = 0.5 * (rf[i][0] + rf[i][2]);
    for (int j = 0; j < 3; j++) rf[1][j] = 0.5 * (rf[0][j] + rf[2][j]);
    for (int i = 0; i < 2; i++)
      for (int j = 0; j < 2; j++) {
        double sub[2][2];
        for (int r = 0; r < 2; r++)
          for (int s = 0; s < 2; s++) sub[r][s] = rf[i + r][j + s];
        vof += gc_face(level_phi, multi, sub);
      }
  } else {
    double cv = 0.0;
    for (int i = 0; i < 2; i++)
      for (int j = 0; j < 2; j++) cv += cor[i][j];
    vof = cv > 0.0 ? 0.75 * multi : (cv == 0.0 ? 0.5 * multi : 0.25 * multi);
  }
  return vof;
}

// GeometryCalculator::Get_corner, geometry_calculator.cpp:12-77: the cell's
// phi on a half-cell lattice from its 3^D neighbourhood p (p[1][1][1 or 0]
// the cell itself); 2D uses z index 0 only (DIM_Z = 0).
void gc_corner(int D, const double p[3][3][3], double c[3][3][3]) {
  const int DZ = D == 3 ? 1 : 0;
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++)
      for (int e = 0; e < 3; e++) c[a][b][e] = 0.;
  c[1][1][DZ] = p[1][1][DZ];
  for (int r = 0; r < 2; r++)
    for (int s = 0; s < 2; s++)
      for (int t = 0; t < 1 + DZ; t++)
        c[2 * r][2 * s][2 * t] = 0.125 * (p[r][s][t] + p[r + 1][s][t] + p[r][s + 1][t] + p[r + 1][s + 1][t] +
                                          p[r][s][t + DZ] + p[r + 1][s][t + DZ] + p[r][s + 1][t + DZ] +
                                          p[r + 1][s + 1][t + DZ]);
  if (DZ)
    for (int r = 0; r < 2; r++)
      for (int s = 0; s < 2; s++)
        c[2 * r][2 * s][1] = 0.25 * (p[r][s][1] + p[r + 1][s][1] + p[r][s + 1][1] + p[r + 1][s + 1][1]);
  for (int s = 0; s < 2; s++)
    for (int t = 0; t < 1 + DZ; t++)
      c[1][2 * s][2 * t] = 0.25 * (p[1][s][t] + p[1][s][t + DZ] + p[1][s + 1][t] + p[1][s + 1][t + DZ]);
  for (int r = 0; r < 2; r++)
    for (int t = 0; t < 1 + DZ; t++)
      c[2 * r][1][2 * t] = 0.25 * (p[r][1][t] + p[r + 1][1][t] + p[r][1][t + DZ] + p[r + 1][1][t + DZ]);
  if (DZ)
    for (int r = 0; r < 2; r++) {
      c[2 * r][1][1] = 0.5 * (p[r][1][1] + p[r + 1][1][1]);
      c[1][2 * r][1] = 0.5 * (p[1][r][1] + p[1][r + 1][1]);
      c[1][1][2 * r] = 0.5 * (p[1][1][r] + p[1][1][r + 1]);
    }
}

// Get_cutcell_volume + Get_surface_area (geometry_calculator.cpp:79-262) of
// one CUT cell from its corner lattice c
void gc_cut_cell(int D, const double c[3][3][3], double dx, double dy, double dz, double* vol, double* area) {
  double H = 0., A = 0.;
  if (D == 3) {
    int marker = gc_mark(&c[0][0][0], 27);
    if (marker == -1) {
      double vof = 0.0;  // get_volume, :262-281
      for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++)
          for (int k = 0; k < 2; k++) {
            double sub[2][2][2];
            for (int r = 0; r < 2; r++)
              for (int s = 0; s < 2; s++)
                for (int t = 0; t < 2; t++) sub[r][s][t] = c[i + r][j + s][k + t];
            vof += gc_subvolume(0, 0.125, sub);
          }
      H = AMIN1(vof, 1.0);
      A = mc_area(c, dx, dy, dz);
    } else {
      H = marker == 1 ? 1.0 : 0.0;
    }
    *vol = H * (dx * dy * dz);
  } else {
    double face[3][3];
    for (int r = 0; r < 3; r++)
      for (int s = 0; s < 3; s++) face[r][s] = c[r][s][0];
    int marker = gc_mark(&face[0][0], 9);
    if (marker == -1) {
      double a = 0.0;  // get_area, :243-260
      for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) {
          double sub[2][2];
          for (int r = 0; r < 2; r++)
            for (int s = 0; s < 2; s++) sub[r][s] = face[i + r][j + s];
          a += gc_face(0, 0.25, sub);
        }
      H = AMIN1(a, 1.0);
      double ext[3][3][3];  // the face extruded over a unit depth (:137-148)
      for (int r = 0; r < 3; r++)
        for (int s = 0; s < 3; s++)
          for (int t = 0; t < 3; t++) ext[r][s][t] = face[r][s];
      A = mc_area(ext, dx, dy, 1.);
    } else {
      H = marker == 1 ? 1.0 : 0.0;
    }
    *vol = H * (dx * dy * 1.);
  }
  *area = A;
}

}  // namespace

extern "C" {

// Marching-cubes table of mc_table(): 256 x 16 edge indices, -1 padded.
void orc_mc_table(signed char* out) { std::memcpy(out, mc_table().t, 256 * 16); }

// Area of the surface of one 3x3x3 corner lattice (get_area_MQ).
double orc_mc_area(const double* c27, double dx, double dy, double dz) {
  double c[3][3][3];
  std::memcpy(c, c27, sizeof(c));
  return mc_area(c, dx, dy, dz);
}

// Volume and area of one CUT cell from its 3^D neighbourhood (27 values,
// [x][y][z], z index 0 in 2D): Get_corner, Get_cutcell_volume, Get_surface_area.
void orc_cut_cell(int D, const double* p27, double dx, double dy, double dz, double* vol, double* area) {
  double p[3][3][3], c[3][3][3];
  std::memcpy(p, p27, sizeof(p));
  gc_corner(D, p, c);
  gc_cut_cell(D, c, dx, dy, dz, vol, area);
}

// Length of segment v0-v1 inside the box [mn, mx]: Segment_AABB_Intersection
// (AABB_calculator.cpp:6-55) clips the segment's parameter range [0, 1] by
// the three slabs in turn (IEEE infinities and NaNs for a segment parallel to
// a slab, which the comparisons then pass or reject) and
// GeometryCalculator::Get_segment_length (geometry_calculator.cpp:571-589)
// returns the clipped piece's length, 0 when it is empty.
double orc_segment_length(const double* mn, const double* mx, const double* v0, const double* v1) {
  double f0 = 0., f1 = 1.;
  for (int d = 0; d < 3; d++) {
    double a = (mn[d] - v0[d]) / (v1[d] - v0[d]);
    double b = (mx[d] - v0[d]) / (v1[d] - v0[d]);
    if (b < a) std::swap(a, b);
    if (b < f0 || a > f1) return 0.;
    f0 = a >= f0 ? a : f0;
    f1 = b <= f1 ? b : f1;
    if (f0 > f1) return 0.;
  }
  double pp[3];
  for (int d = 0; d < 3; d++) pp[d] = ((v1[d] - v0[d]) * f1 + v0[d]) - ((v1[d] - v0[d]) * f0 + v0[d]);
  return std::sqrt(pp[0] * pp[0] + pp[1] * pp[1] + pp[2] * pp[2]);
}

// Calculate_volume_mass over the interior cells of level `level` (after
// orc_ls_build of that level) and Get_num_particles.  cell_vol / cell_area
// (may be NULL) receive per-cell values over the full grid incl. margins
// (zero outside the counted cells).  totals = {total_mass,
// total_mass_surface, total_volume, total_area, total_mass_segment,
// total_length}; counts = {interface cells, mesh particles, surface
// particles, particles, segment particles, singularity particles}.  In 3D a
// SEGMENT cell adds its segment's length inside the cell over its scale
// (lset_package.cpp:1371-1383).
void orc_volume_mass(const orc_ctx* c, int level, double* cell_vol, double* cell_area, double* totals,
                     long long* counts) {
  const int D = c->dim;
  const orc_level& L = c->ls[level];
  const double dl = ls_dl(L, D);
  const double dx = ls_dcell(L, 0), dy = ls_dcell(L, 1), dz = D == 3 ? ls_dcell(L, 2) : 1.0;
  const int n0 = 4 * L.num_pkg[0], n1 = 4 * L.num_pkg[1], n2 = D == 3 ? 4 * L.num_pkg[2] : 1;
  long long ntot = 1;
  for (int d = 0; d < D; d++) ntot *= ls_ncell(L, d);
  std::vector<double> own_v, own_a;
  if (!cell_vol) {
    own_v.resize(ntot);
    cell_vol = own_v.data();
  }
  if (!cell_area) {
    own_a.resize(ntot);
    cell_area = own_a.data();
  }
  std::fill(cell_vol, cell_vol + ntot, 0.0);
  std::fill(cell_area, cell_area + ntot, 0.0);
  // per-cell volumes and areas (the packages of the reference's parallel_for)
#pragma omp parallel for schedule(dynamic, 1)
  for (int gk = 0; gk < n2; gk++)
    for (int gj = 0; gj < n1; gj++)
      for (int gi = 0; gi < n0; gi++) {
        const long long a = ls_index(L, D, gi, gj, gk);
        const double phi = L.phi[a];
        if (!(phi > 0. || std::fabs(phi) < dl)) continue;
        double vol, area = 0.;
        if (L.tag[a] == CUT_CELL) {
          double p[3][3][3] = {}, cr[3][3][3];
          for (int r = 0; r < 3; r++)
            for (int s = 0; s < 3; s++)
              for (int t = 0; t < (D == 3 ? 3 : 1); t++)
                p[r][s][t] = L.phi[ls_index(L, D, gi + r - 1, gj + s - 1, D == 3 ? gk + t - 1 : 0)];
          gc_corner(D, p, cr);
          gc_cut_cell(D, cr, dx, dy, dz, &vol, &area);
        } else {
          vol = (dx * dy) * dz;
        }
        cell_vol[a] = vol;
        cell_area[a] = area;
      }
  // the sums in cell order
  double M = 0., Ms = 0., V = 0., A = 0., Mg = 0., Lg = 0.;
  long long ncut = 0;
  for (int gk = 0; gk < n2; gk++)
    for (int gj = 0; gj < n1; gj++)
      for (int gi = 0; gi < n0; gi++) {
        const long long a = ls_index(L, D, gi, gj, gk);
        if (L.tag[a] == CUT_CELL) ncut++;
        const double phi = L.phi[a];
        if (!(phi > 0. || std::fabs(phi) < dl)) continue;
        const double scale = get_scale(*c, D, phi, L.curv[a]);
        if (L.tag[a] == CUT_CELL) {
          A += cell_area[a];
          Ms += cell_area[a] / powern(scale, D - 1);
        }
        if (D == 3 && L.chr && L.chr[a] == CHAR_SEGMENT) {
          const int g[3] = {gi, gj, gk};
          double mn[3], mx[3];
          for (int d = 0; d < 3; d++) {
            const int pk = g[d] / 4, ce = g[d] % 4;
            mn[d] = (pk * L.dpkg[d] + ce * ls_dcell(L, d)) + L.box_l[d];
            mx[d] = mn[d] + ls_dcell(L, d);
          }
          const double* sg = c->seg + 6 * L.chr_idx[a];
          const double len = orc_segment_length(mn, mx, sg, sg + 3);
          Lg += len;
          Mg += len / scale;
        }
        M += cell_vol[a] / powern(scale, D);
        V += cell_vol[a];
      }
  totals[0] = M;
  totals[1] = Ms;
  totals[2] = V;
  totals[3] = A;
  totals[4] = Mg;
  totals[5] = Lg;
  // Get_num_particles, sph_mesh_generation.cpp:909-923
  const int nsing = c->nsing;
  const long long n_segment = AMAX1(int(Mg * 1. - 0.5 * nsing), 0);
  long long n_surface = AMAX1(int(Ms * 1. - 0.5 * Mg * 1.), 0);
  const long long n_mesh = AMAX1(int(M * 1. - 0.5 * Ms * 1.), 0);
  if (ncut < n_surface) n_surface = ncut;
  counts[0] = ncut;
  counts[1] = n_mesh;
  counts[2] = n_surface;
  counts[3] = n_mesh + n_surface + nsing + n_segment;
  counts[4] = n_segment;
  counts[5] = nsing;
}

}  // extern "C"

// ====================================================================== tets
// 3D tetrahedralisation (row F3; the reference: Graphmeshcls::Reconstruct_tets,
// graph_mesh.cpp:981-1100, TetGen's Delaunay tetrahedralisation of all
// particles, Check_whether_this_tet_should_be_delete, :675-979, and
// Tet_quality_statistics, :1967-2400).  TetGen is not available, so this
// oracle restates the local certified-star construction of the library (per
// particle: gift wrapping over its neighbour row; a tet counts when its
// circumsphere lies in the row's ball of radius cutoff * h and no row
// particle lies inside or on it) on the CPU with its own exact arithmetic;
// the tests pin it against qhull's Delaunay tetrahedralisation (scipy) of
// the same snapped points.
namespace tetorc {
struct Big {  // two's complement, 5 x 64 bits
  unsigned long long w[5];
};
static Big big(long long v) {
  Big r;
  r.w[0] = (unsigned long long)v;
  for (int k = 1; k < 5; k++) r.w[k] = v < 0 ? ~0ull : 0ull;
  return r;
}
static Big add(const Big& a, const Big& b) {
  Big r;
  unsigned __int128 c = 0;
  for (int k = 0; k < 5; k++) {
    c += (unsigned __int128)a.w[k] + b.w[k];
    r.w[k] = (unsigned long long)c;
    c >>= 64;
  }
  return r;
}
static Big neg(const Big& a) {
  Big r;
  for (int k = 0; k < 5; k++) r.w[k] = ~a.w[k];
  return add(r, big(1));
}
static Big sub(const Big& a, const Big& b) { return add(a, neg(b)); }
static bool isneg(const Big& a) { return (long long)a.w[4] < 0; }
static Big mul(const Big& a, const Big& b) {
  const bool na = isneg(a), nb = isneg(b);
  const Big x = na ? neg(a) : a, y = nb ? neg(b) : b;
  unsigned long long r[5] = {0, 0, 0, 0, 0};
  for (int i = 0; i < 5; i++) {
    unsigned __int128 c = 0;
    for (int j = 0; i + j < 5; j++) {
      c += (unsigned __int128)x.w[i] * y.w[j] + r[i + j];
      r[i + j] = (unsigned long long)c;
      c >>= 64;
    }
  }
  Big o;
  for (int k = 0; k < 5; k++) o.w[k] = r[k];
  return na != nb ? neg(o) : o;
}
static int sign(const Big& a) {
  if (isneg(a)) return -1;
  for (int k = 0; k < 5; k++)
    if (a.w[k]) return 1;
  return 0;
}
static Big M2(long long p, long long q) { return mul(big(p), big(q)); }

struct Ctx {
  const double* x;
  double ig;
  long long I(int j, int q) const { return (long long)std::nearbyint(x[3 * (size_t)j + q] * ig); }
};
// exact signs over the integer coordinates (no floating-point filter)
static int orient(const Ctx& C, int a, int b, int c, int d) {
  long long v[3][3];
  const int p[3] = {a, b, c};
  for (int k = 0; k < 3; k++)
    for (int q = 0; q < 3; q++) v[k][q] = C.I(p[k], q) - C.I(d, q);
  const Big m1 = sub(M2(v[1][1], v[2][2]), M2(v[1][2], v[2][1]));
  const Big m2 = sub(M2(v[2][1], v[0][2]), M2(v[2][2], v[0][1]));
  const Big m3 = sub(M2(v[0][1], v[1][2]), M2(v[0][2], v[1][1]));
  return sign(add(add(mul(big(v[0][0]), m1), mul(big(v[1][0]), m2)), mul(big(v[2][0]), m3)));
}
static int insph(const Ctx& C, int a, int b, int c, int d, int e) {
  long long v[4][3];
  const int p[4] = {a, b, c, d};
  for (int k = 0; k < 4; k++)
    for (int q = 0; q < 3; q++) v[k][q] = C.I(p[k], q) - C.I(e, q);
  Big lift[4], mz[4];
  for (int k = 0; k < 4; k++) {
    lift[k] = add(add(M2(v[k][0], v[k][0]), M2(v[k][1], v[k][1])), M2(v[k][2], v[k][2]));
    mz[k] = big(v[k][2]);
  }
  auto xy = [&](int s, int t) { return sub(M2(v[s][0], v[t][1]), M2(v[t][0], v[s][1])); };
  const Big ab = xy(0, 1), bc = xy(1, 2), cd = xy(2, 3), da = xy(3, 0), ac = xy(0, 2), bd = xy(1, 3);
  const Big abc = add(sub(mul(mz[0], bc), mul(mz[1], ac)), mul(mz[2], ab));
  const Big bcd = add(sub(mul(mz[1], cd), mul(mz[2], bd)), mul(mz[3], bc));
  const Big cda = add(add(mul(mz[2], da), mul(mz[3], ac)), mul(mz[0], cd));
  const Big dab = add(add(mul(mz[3], ab), mul(mz[0], bd)), mul(mz[1], da));
  return sign(add(sub(mul(lift[3], abc), mul(lift[2], dab)), sub(mul(lift[1], cda), mul(lift[0], bcd))));
}

static void cross(const double* u, const double* v, double* w) {
  w[0] = u[1] * v[2] - u[2] * v[1];
  w[1] = u[2] * v[0] - u[0] * v[2];
  w[2] = u[0] * v[1] - u[1] * v[0];
}
static double dot(const double* u, const double* v) { return u[0] * v[0] + u[1] * v[1] + u[2] * v[2]; }

// the canonical geometry of a tet over its ascending ids (same terms and
// order as the library's)
struct Geo {
  double A[3][3], det, c[3], rc, vs, P[4][3];
};
static Geo geo(const Ctx& C, const int* v) {
  Geo g;
  for (int k = 0; k < 4; k++)
    for (int q = 0; q < 3; q++) g.P[k][q] = C.x[3 * (size_t)v[k] + q];
  for (int k = 0; k < 3; k++)
    for (int q = 0; q < 3; q++) g.A[k][q] = g.P[k][q] - g.P[3][q];
  double x12[3], x20[3], x01[3];
  cross(g.A[1], g.A[2], x12);
  cross(g.A[2], g.A[0], x20);
  cross(g.A[0], g.A[1], x01);
  g.det = dot(g.A[0], x12);
  const double r0 = 0.5 * dot(g.A[0], g.A[0]), r1 = 0.5 * dot(g.A[1], g.A[1]), r2 = 0.5 * dot(g.A[2], g.A[2]);
  for (int q = 0; q < 3; q++) g.c[q] = (r0 * x12[q] + r1 * x20[q] + r2 * x01[q]) / g.det;
  g.rc = std::sqrt(dot(g.c, g.c));
  g.vs = std::sqrt(dot(g.A[0], g.A[0])) * std::sqrt(dot(g.A[1], g.A[1])) * std::sqrt(dot(g.A[2], g.A[2]));
  return g;
}
static bool in_ball(const Geo& g, const double* x, double h, double cutoff) {
  if (!(std::fabs(g.det) >= 1.e-6 * g.vs)) return false;
  double v[3];
  for (int q = 0; q < 3; q++) v[q] = g.P[3][q] + g.c[q] - x[q];
  return std::sqrt(dot(v, v)) + g.rc <= cutoff * h * (1.0 - 1.e-6);
}
// aspect, inverse heights and unit inward normals
static double heights(const Geo& g, double n[4][3], double H[4], double* hmax, double* hsum) {
  cross(g.A[1], g.A[2], n[0]);
  cross(g.A[2], g.A[0], n[1]);
  cross(g.A[0], g.A[1], n[2]);
  for (int k = 0; k < 3; k++)
    for (int q = 0; q < 3; q++) n[k][q] /= g.det;
  for (int q = 0; q < 3; q++) n[3][q] = -n[0][q] - n[1][q] - n[2][q];
  *hmax = 0.0;
  *hsum = 0.0;
  for (int k = 0; k < 4; k++) {
    H[k] = std::sqrt(dot(n[k], n[k]));
    *hsum += H[k];
    *hmax = std::fmax(*hmax, H[k]);
  }
  double longlen = 0.0, e[3];
  for (int k = 0; k < 3; k++) longlen = std::fmax(longlen, dot(g.A[k], g.A[k]));
  const int ea[3] = {1, 2, 0}, eb[3] = {0, 1, 2};
  for (int k = 0; k < 3; k++) {
    for (int q = 0; q < 3; q++) e[q] = g.P[ea[k]][q] - g.P[eb[k]][q];
    longlen = std::fmax(longlen, dot(e, e));
  }
  return longlen;
}
static void sort4(int* v) { std::sort(v, v + 4); }
}  // namespace tetorc

extern "C" {
struct orc_tet_quality {
  long long ntet, nopen, ndeleted, ntie;
  double grid, total_volume, min_volume, max_volume, min_edge, max_edge, min_aspect, max_aspect, avg_aspect;
  double min_radius_ratio, max_radius_ratio, avg_radius_ratio, min_dihedral, max_dihedral, avg_min_dihedral;
  long long nsmall_dihedral[4], aspect_hist[12], radius_hist[56], dihedral_hist[45];
  long long ntrunc;
};

// xyz (n x 3, FP64), type, h, neighbour rows (CSR off / nbr in id space,
// self may be listed); box_l / box_r bound the coordinates.  Returns the tet
// count (tets filled when cap allows; ascending ids per tet, in the order of
// the emitting particle and its star).  A star stops its walk at the
// library's per-particle limits (128 tets, 224 link edges; counted).
long long orc_tetrahedralize(long long n, const double* xyz_in, const int* type, const double* h,
                             const long long* off, const int* nbr, double cutoff, const double* box_l,
                             const double* box_r, int* tets, long long cap, orc_tet_quality* Q) {
  using namespace tetorc;
  double Mx = 1.0;
  for (int d = 0; d < 3; d++) Mx = std::fmax(Mx, std::fmax(std::fabs(box_l[d]), std::fabs(box_r[d])));
  int e = 0;
  std::frexp(Mx, &e);
  e += 1;
  const double g = std::ldexp(1.0, e - 52), ig = std::ldexp(1.0, 52 - e);
  std::vector<double> X(3 * (size_t)n);
  for (size_t k = 0; k < X.size(); k++) X[k] = std::nearbyint(xyz_in[k] * ig) * g;
  const Ctx C{X.data(), ig};
  std::vector<std::vector<int>> out(n);
  std::vector<int> open(n, 0), tie(n, 0), trunc(n, 0);
  std::vector<long long> ndel(n, 0);
#pragma omp parallel for schedule(dynamic, 64)
  for (long long i64 = 0; i64 < n; i64++) {
    const int i = (int)i64;
    std::vector<int> S;
    for (long long q = off[i]; q < off[i + 1]; q++)
      if (nbr[q] != i) S.push_back(nbr[q]);
    const double* xi = &X[3 * (size_t)i];
    auto d2 = [&](int j) {
      const double* p = &X[3 * (size_t)j];
      const double dx = p[0] - xi[0], dy = p[1] - xi[1], dz = p[2] - xi[2];
      return dx * dx + dy * dy + dz * dz;
    };
    bool degen = false;
    auto wrap = [&](int a, int b, int s) {
      int best = -1;
      for (int d : S) {
        if (d == a || d == b) continue;
        if (s * orient(C, i, a, b, d) <= 0) continue;
        if (best < 0 || s * insph(C, i, a, b, best, d) > 0) best = d;
      }
      return best;
    };
    // 0: a row particle inside or on the sphere (or coplanar); 1: none (a
    // tet of the row's Delaunay tetrahedralisation); 2: also inside i's ball
    // and not flat (certified)
    auto status = [&](int a, int b, int d) {
      int v[4] = {i, a, b, d};
      sort4(v);
      const Geo G = geo(C, v);
      const int o = orient(C, v[0], v[1], v[2], v[3]);
      if (o == 0) return 0;
      bool inside = false, on = false;
      for (int q : S) {
        if (q == v[0] || q == v[1] || q == v[2] || q == v[3]) continue;
        const int s = o * insph(C, v[0], v[1], v[2], v[3], q);
        if (s > 0) { inside = true; break; }
        if (s == 0) on = true;
      }
      if (inside || on) {
        if (!inside) degen = true;
        return 0;
      }
      return in_ball(G, xi, h[i], cutoff) ? 2 : 1;
    };
    // nearest particle, then the smallest circumcircle through i and it
    int a = -1, c = -1;
    double best = 0.0, bestr = 0.0;
    for (int j : S) {
      const double v = d2(j);
      if (a < 0 || v < best || (v == best && j < a)) { a = j; best = v; }
    }
    if (a >= 0) {
      const double* pa = &X[3 * (size_t)a];
      const double u[3] = {pa[0] - xi[0], pa[1] - xi[1], pa[2] - xi[2]};
      const double uu = dot(u, u);
      for (int j : S) {
        if (j == a) continue;
        const double* pj = &X[3 * (size_t)j];
        const double v[3] = {pj[0] - xi[0], pj[1] - xi[1], pj[2] - xi[2]};
        const double w[3] = {v[0] - u[0], v[1] - u[1], v[2] - u[2]};
        double x[3];
        cross(u, v, x);
        const double xx = dot(x, x);
        if (!(xx > 0.0)) continue;
        const double r2 = uu * dot(v, v) * dot(w, w) / (4.0 * xx);
        if (c < 0 || r2 < bestr || (r2 == bestr && j < c)) { c = j; bestr = r2; }
      }
    }
    std::vector<std::array<int, 3>> star;
    std::vector<char> cert;
    if (c >= 0) {
      for (int s = 1; s >= -1 && star.empty(); s -= 2) {
        const int d = wrap(a, c, s);
        const int st = d >= 0 ? status(a, c, d) : 0;
        if (st > 0) {
          star.push_back(s > 0 ? std::array<int, 3>{a, c, d} : std::array<int, 3>{c, a, d});
          cert.push_back(st == 2);
        }
      }
    }
    bool op = star.empty(), ovf = false;
    // link edges (u, v) in the orientation of the tet that registered them
    std::vector<std::array<int, 2>> le;
    std::vector<char> done;
    size_t head = 0;
    while (!ovf) {
      for (; head < star.size(); head++) {
        const auto t = star[head];
        for (int k = 0; k < 3; k++) {
          const int u = t[k], v = t[(k + 1) % 3];
          int f = -1;
          for (size_t q = 0; q < le.size(); q++)
            if ((le[q][0] == u && le[q][1] == v) || (le[q][0] == v && le[q][1] == u)) { f = (int)q; break; }
          if (f >= 0) done[f] = 1;
          else if (le.size() < 224) { le.push_back({u, v}); done.push_back(0); }
          else ovf = true;
        }
      }
      if (ovf) break;
      int f = -1;
      for (size_t q = 0; q < le.size(); q++)
        if (!done[q]) { f = (int)q; break; }
      if (f < 0) break;
      done[f] = 1;
      const int u = le[f][0], v = le[f][1];
      const int d = wrap(u, v, -1);
      const int st = d >= 0 ? status(u, v, d) : 0;
      if (st == 0) { op = true; continue; }
      bool dup = false;
      for (const auto& t : star) {
        auto has = [&](int z) { return t[0] == z || t[1] == z || t[2] == z; };
        if (has(u) && has(v) && has(d)) { dup = true; break; }
      }
      if (dup) continue;
      if (star.size() == 128) { ovf = true; break; }
      star.push_back({v, u, d});
      cert.push_back(st == 2);
    }
    trunc[i] = ovf;
    for (size_t k0 = 0; k0 < star.size(); k0++) {
      if (!cert[k0]) continue;
      const auto& t = star[k0];
      int v[4] = {i, t[0], t[1], t[2]};
      sort4(v);
      const Geo G = geo(C, v);
      int owner = -1;
      for (int k = 0; k < 4 && owner < 0; k++)
        if (in_ball(G, G.P[k], h[v[k]], cutoff)) owner = v[k];
      if (owner != i) continue;
      const bool allb = type[v[0]] != 0 && type[v[1]] != 0 && type[v[2]] != 0 && type[v[3]] != 0;
      if (allb) {
        double n4[4][3], H[4], hmax, hsum;
        const double ll = heights(G, n4, H, &hmax, &hsum);
        if (std::sqrt(ll) * hmax > 10.0) { ndel[i]++; continue; }
      }
      out[i].insert(out[i].end(), v, v + 4);
    }
    open[i] = op;
    tie[i] = degen;
  }
  long long ntet = 0;
  for (long long i = 0; i < n; i++) ntet += (long long)out[i].size() / 4;
  if (tets && cap >= ntet) {
    long long o = 0;
    for (long long i = 0; i < n; i++)
      for (int v : out[i]) tets[o++] = v;
  }
  if (Q) {
    std::memset(Q, 0, sizeof(*Q));
    Q->ntet = ntet;
    Q->grid = g;
    for (long long i = 0; i < n; i++) {
      Q->nopen += open[i];
      Q->ntie += tie[i];
      Q->ndeleted += ndel[i];
      Q->ntrunc += trunc[i];
    }
    double cosd[46], coss[4];
    // degrees as the reference converts them, with its PI (glbparam.h:186)
    const double pi_ref = 3.1415926;
    for (int k = 0; k <= 45; k++) cosd[k] = std::cos(4.0 * k * pi_ref / 180.0);
    for (int k = 0; k < 4; k++) coss[k] = std::cos(10.0 * (k + 1) * pi_ref / 180.0);
    double vmin = 1.e300, vmax = 0, emin = 1.e300, emax = 0, amin = 1.e300, amax = 0, rmin = 1.e300, rmax = 0;
    double dmin = 1.e300, dmax = 0, vsum = 0, asum = 0, rsum = 0, dsum = 0;
    const double tab[11] = {1.5, 2.0, 2.5, 3.0, 4.0, 6.0, 10.0, 15.0, 25.0, 50.0, 100.0};
    for (long long i = 0; i < n; i++)
      for (size_t t = 0; t < out[i].size(); t += 4) {
        const Geo G = geo(C, &out[i][t]);
        double nn[4][3], H[4], hmax, hsum;
        const double hi = heights(G, nn, H, &hmax, &hsum);
        for (int k = 0; k < 4; k++)
          for (int q = 0; q < 3; q++) nn[k][q] /= H[k];
        double lo = 1.e300, e2[3];
        for (int k = 0; k < 3; k++) lo = std::fmin(lo, dot(G.A[k], G.A[k]));
        const int ea[3] = {1, 2, 0}, eb[3] = {0, 1, 2};
        for (int k = 0; k < 3; k++) {
          for (int q = 0; q < 3; q++) e2[q] = G.P[ea[k]][q] - G.P[eb[k]][q];
          lo = std::fmin(lo, dot(e2, e2));
        }
        const double vol = std::fabs(G.det) / 6.0, aspect = std::sqrt(hi) * hmax, ratio = 3.0 * (1.0 / hsum) / G.rc;
        vsum += vol; vmin = std::fmin(vmin, vol); vmax = std::fmax(vmax, vol);
        emin = std::fmin(emin, lo); emax = std::fmax(emax, hi);
        asum += aspect; amin = std::fmin(amin, aspect); amax = std::fmax(amax, aspect);
        rsum += ratio; rmin = std::fmin(rmin, ratio); rmax = std::fmax(rmax, ratio);
        int ai = 0;
        while (ai < 11 && aspect > tab[ai]) ai++;
        Q->aspect_hist[ai]++;
        const double rq = std::floor(ratio / 0.02);
        Q->radius_hist[rq >= 0.0 ? (rq < 55 ? (int)rq : 55) : 0]++;
        const int pa[6] = {0, 0, 0, 1, 1, 2}, pb[6] = {1, 2, 3, 2, 3, 3};
        double cmax = -2.0, cmin = 2.0;
        for (int k = 0; k < 6; k++) {
          const double cs = std::fmin(1.0, std::fmax(-1.0, -dot(nn[pa[k]], nn[pb[k]])));
          cmax = std::fmax(cmax, cs);
          cmin = std::fmin(cmin, cs);
          int b = 0;
          while (b < 44 && cs <= cosd[b + 1]) b++;
          Q->dihedral_hist[b]++;
        }
        for (int k = 0; k < 4; k++)
          if (cmax > coss[k]) Q->nsmall_dihedral[k]++;
        const double ds = std::acos(cmax) / pi_ref * 180.0, db = std::acos(cmin) / pi_ref * 180.0;
        dmin = std::fmin(dmin, ds); dmax = std::fmax(dmax, db); dsum += ds;
      }
    if (ntet > 0) {
      Q->total_volume = vsum; Q->min_volume = vmin; Q->max_volume = vmax;
      Q->min_edge = std::sqrt(emin); Q->max_edge = std::sqrt(emax);
      Q->min_aspect = amin; Q->max_aspect = amax; Q->avg_aspect = asum / ntet;
      Q->min_radius_ratio = rmin; Q->max_radius_ratio = rmax; Q->avg_radius_ratio = rsum / ntet;
      Q->min_dihedral = dmin; Q->max_dihedral = dmax; Q->avg_min_dihedral = dsum / ntet;
    }
  }
  return ntet;
}
}
