// mrsph_api.cu — the C ABI (include/mrsph_relax.h): handle, parameters,
// cell-list level plan, level-set upload/build and the engine dispatch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "engine_iface.h"

#include "handle.h"

using namespace mrsph;

static thread_local std::string g_create_error;

static int fail(mrsph_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg; else g_create_error = msg;
  return code;
}

#define API_CK(h, call)                                                             \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess) return fail(h, MRSPH_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

static double powern_d(double a, int n) {
  double r = 1;
  for (int i = 0; i < n; i++) r *= a;
  return r;
}

// SPH::Define_level_infor_tight (sph.cpp:144-180) + Level_info::Initialize
// (level_infor.cpp:35-110), _NON_SYM_: cells [0, num_cell) per level.
static int plan_levels(mrsph_handle* h) {
  const mrsph_params& p = h->prm;
  const int D = p.dim;
  CellGeo& g = h->geo;
  std::memset(&g, 0, sizeof(g));
  double domain[3];
  for (int d = 0; d < 3; d++) domain[d] = p.box_r[d] - p.box_l[d];
  for (int d = 0; d < D; d++)
    if (!(domain[d] > 0)) return fail(h, MRSPH_ERR_ARG, "box_r must exceed box_l");
  double max_scale = p.max_dl * p.cell_ratio, min_scale = p.min_dl * p.cell_ratio;
  double scale_temp = domain[0];
  if (D >= 2) scale_temp = std::min(domain[1], scale_temp);
  if (D == 3) scale_temp = std::min(domain[2], scale_temp);
  int temp = (int)std::floor(scale_temp / max_scale);
  if (temp < 1) return fail(h, MRSPH_ERR_ARG, "domain smaller than the coarsest cell");
  double ini_scale = scale_temp / (double)temp;
  max_scale = ini_scale;
  scale_temp = ini_scale;
  int num_level = 1;
  while ((scale_temp + 1.e-6) > min_scale) {
    scale_temp /= 2;
    num_level++;
    if (num_level > 64) break;
  }
  min_scale = scale_temp * 2;
  num_level -= 1;
  if (num_level < 1 || num_level > MAX_CL) return fail(h, MRSPH_ERR_RANGE, "too many cell-list levels (max 8)");
  g.ncl = num_level;
  g.max_scale = max_scale;
  g.min_scale = min_scale;
  int ini[3];
  for (int d = 0; d < 3; d++) {
    ini[d] = (d < D) ? (int)(domain[d] / max_scale) : 1;
    g.box_l[d] = (d < D) ? p.box_l[d] : 0.0;
  }
  long long off = 0, hoff = 0;
  for (int l = 0; l < num_level; l++) {
    double multi = powern_d(2.0, l);
    double sc = 1.e300;
    long long nc = 1, hc = 1;
    for (int d = 0; d < 3; d++) {
      g.n[l][d] = (d < D) ? (int)(ini[d] * multi) : 1;
      g.dcell[l][d] = (d < D) ? domain[d] / g.n[l][d] : 1.0;
      if (d < D) sc = std::min(sc, g.dcell[l][d]);
      nc *= g.n[l][d];
      // sort table of half cells: floor(x / (dcell/2)) >> 1 == floor(x / dcell)
      // exactly, since halving commutes with rounding
      g.hn[l][d] = (d < D) ? 2 * g.n[l][d] : 1;
      g.hs[l][d] = (d < D) ? 0.5 * g.dcell[l][d] : 1.0;
      g.ihs[l][d] = 1.0 / g.hs[l][d];
      g.ihs_f[l][d] = (float)g.ihs[l][d];
      g.hs_f[l][d] = (float)g.hs[l][d];
      hc *= g.hn[l][d];
    }
    // the engine keys levels by exponent: scale = max_scale * 2^-l (sph.cpp:247-276)
    if (std::fabs(sc - std::ldexp(max_scale, -l)) > 1.e-10)
      return fail(h, MRSPH_ERR_ARG, "cell-list level scale does not match max_scale/2^l; adjust the domain");
    g.off[l] = off;
    off += nc;
    g.hoff[l] = hoff;
    hoff += hc;
  }
  g.off[num_level] = off;
  g.hoff[num_level] = hoff;
  g.nc0 = (long long)g.n[0][0] * g.n[0][1] * g.n[0][2];
  // cell keys are 32-bit: the half-cell table (counts + starts, 8 bytes per
  // entry; 1.06 G entries for four levels down to 480^3 cells) must index in int
  if (hoff > 2147483000ll) return fail(h, MRSPH_ERR_RANGE, "more than 2^31 half cells over the cell-list levels");
  const int lm = num_level - 1;
  for (int d = 0; d < 3; d++) {
    g.A[d] = g.dcell[lm][d];
    g.idc0[d] = 1.0 / g.dcell[0][d];
    g.idc0_f[d] = (float)g.idc0[d];
    g.Af[d] = (float)g.A[d];
  }
  if (p.precision == MRSPH_FP32_SPLIT) {
    // the FP32 neighbour test's band covers the reference's +1e-10 on the
    // cut-off radius (h cutoff = scale cell_ratio) only for radii >= 1e-4
    if (p.min_dl * p.cell_ratio < 1.e-4)
      return fail(h, MRSPH_ERR_RANGE, "FP32-split needs a smallest cut-off radius (min_dl * cell_ratio) of 1e-4");
    int lim[3] = {D == 2 ? 65536 : 2048, D == 2 ? 65536 : 2048, D == 2 ? 1 : 1024};
    for (int d = 0; d < D; d++)
      if (g.n[lm][d] > lim[d]) return fail(h, MRSPH_ERR_RANGE, "finest cell grid too large for the FP32-split key");
  }
  return 0;
}

extern "C" {

int mrsph_version(void) { return MRSPH_API_VERSION; }

int mrsph_create(const mrsph_params* p, mrsph_handle** out) {
  if (!p || !out) return fail(nullptr, MRSPH_ERR_ARG, "null argument");
  *out = nullptr;
  if (p->dim != 2 && p->dim != 3) return fail(nullptr, MRSPH_ERR_ARG, "dim must be 2 or 3");
  if (p->kernel < 0 || p->kernel > 4) return fail(nullptr, MRSPH_ERR_ARG, "unknown kernel id");
  if (p->precision != MRSPH_FP64_PLAIN && p->precision != MRSPH_FP32_SPLIT)
    return fail(nullptr, MRSPH_ERR_ARG, "unknown precision mode");
  if (p->scale_law != 0 && p->scale_law != 1) return fail(nullptr, MRSPH_ERR_ARG, "scale_law must be 0 or 1");
  if (!(p->cutoff > 0) || !(p->cell_ratio > 0) || !(p->min_dl > 0) || !(p->max_dl >= p->min_dl))
    return fail(nullptr, MRSPH_ERR_ARG, "invalid spacing parameters");
  mrsph_handle* h = new mrsph_handle();
  h->prm = *p;
  int rc = plan_levels(h);
  if (rc) {
    g_create_error = h->err;
    delete h;
    return rc;
  }
  cudaError_t e = cudaSetDevice(p->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    g_create_error = std::string("CUDA: ") + cudaGetErrorString(e);
    delete h;
    return MRSPH_ERR_CUDA;
  }
  *out = h;
  return 0;
}

int mrsph_destroy(mrsph_handle* h) {
  if (!h) return 0;
  cudaSetDevice(h->prm.device);
  // a batch still holding the handle: its queued work finishes first and it
  // forgets the handle (whichever of the two is destroyed first)
  const std::vector<mrsph_batch*> bs = h->batches;
  for (mrsph_batch* b : bs) mrsph_batch_detach(b, h);
  delete h->eng;
  for (void* p : h->ls_allocs) cudaFree(p);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return 0;
}

int mrsph_last_error(mrsph_handle* h, char* buf, size_t len) {
  const std::string& s = h ? h->err : g_create_error;
  if (buf && len) {
    std::strncpy(buf, s.c_str(), len - 1);
    buf[len - 1] = 0;
  }
  return (int)s.size();
}

int mrsph_set_levelset(mrsph_handle* h, int nlevels, const mrsph_levelset_level* lv) {
  if (!h || !lv) return fail(h, MRSPH_ERR_ARG, "null argument");
  if (nlevels < 1 || nlevels > MAX_LS) return fail(h, MRSPH_ERR_RANGE, "1..4 level-set levels supported");
  API_CK(h, cudaSetDevice(h->prm.device));
  const int D = h->prm.dim;
  delete h->eng;
  h->eng = nullptr;
  for (void* p : h->ls_allocs) cudaFree(p);
  h->ls_allocs.clear();
  unsigned long long* d_max = nullptr;
  API_CK(h, cudaMalloc(&d_max, 3 * sizeof(unsigned long long)));  // max phi, max |curv|, min |curv|
  h->ls_allocs.push_back(d_max);
  {
    double init_d[3] = {0.0, 0.0, 1.e20};
    unsigned long long init[3];
    std::memcpy(init, init_d, sizeof(init));
    // ordered before the level-set build kernels on the handle's stream
    API_CK(h, cudaMemcpyAsync(d_max, init, sizeof(init), cudaMemcpyHostToDevice, h->stream));
    API_CK(h, cudaStreamSynchronize(h->stream));
  }
  LsSet& ls = h->ls;
  std::memset(&ls, 0, sizeof(ls));
  ls.nls = nlevels;
  for (int l = 0; l < nlevels; l++) {
    const mrsph_levelset_level& in = lv[l];
    if (!in.phi || in.margin < 1) return fail(h, MRSPH_ERR_ARG, "level set needs phi and margin >= 1");
    LsLevel& L = ls.lv[l];
    LsBuildDesc bd{};
    bd.D = D;
    bd.margin = in.margin;
    L.margin = in.margin;
    long long ntot = 1;
    for (int d = 0; d < 3; d++) {
      L.box_l[d] = in.box_l[d];
      L.dpkg[d] = in.dpkg[d];
      L.num_pkg[d] = in.num_pkg[d];
      L.dcell[d] = in.dpkg[d] / 4.0;
      L.inv_dpkg[d] = 1.0 / L.dpkg[d];
      L.inv_dcell[d] = 1.0 / L.dcell[d];
      L.n[d] = (d < D) ? (in.num_pkg[d] + 2 * in.margin) * 4 : 1;
      if (d < D && in.num_pkg[d] < 1) return fail(h, MRSPH_ERR_ARG, "num_pkg must be positive");
      bd.num_pkg[d] = in.num_pkg[d];
      bd.n[d] = L.n[d];
      bd.dcell[d] = L.dcell[d];
      ntot *= L.n[d];
    }
    h->ls_ntot[l] = ntot;
    double* d_phi = nullptr;
    double4* g64 = nullptr;
    double* c64 = nullptr;
    float4* g32 = nullptr;
    float* c32 = nullptr;
    uint8_t* tag = nullptr;
    uint8_t* act = nullptr;
    API_CK(h, cudaMalloc(&d_phi, sizeof(double) * ntot));
    h->ls_allocs.push_back(d_phi);
    API_CK(h, cudaMalloc(&g64, sizeof(double4) * ntot));
    h->ls_allocs.push_back(g64);
    API_CK(h, cudaMalloc(&c64, sizeof(double) * ntot));
    h->ls_allocs.push_back(c64);
    API_CK(h, cudaMalloc(&g32, sizeof(float4) * ntot));
    h->ls_allocs.push_back(g32);
    API_CK(h, cudaMalloc(&c32, sizeof(float) * ntot));
    h->ls_allocs.push_back(c32);
    API_CK(h, cudaMalloc(&tag, ntot));
    h->ls_allocs.push_back(tag);
    API_CK(h, cudaMemcpyAsync(d_phi, in.phi, sizeof(double) * ntot, cudaMemcpyHostToDevice, h->stream));
    if (in.active) {
      long long np = 1;
      for (int d = 0; d < D; d++) np *= (in.num_pkg[d] + 2 * in.margin);
      API_CK(h, cudaMalloc(&act, np));
      h->ls_allocs.push_back(act);
      API_CK(h, cudaMemcpyAsync(act, in.active, np, cudaMemcpyHostToDevice, h->stream));
    }
    API_CK(h, ls_build_level(bd, d_phi, g64, c64, g32, c32, tag, d_max, h->stream));
    L.g64 = g64;
    L.c64 = c64;
    L.g32 = g32;
    L.c32 = c32;
    L.tag = tag;
    L.active = act;
    L.chr = nullptr;
  }
  // characteristic points and segments (mrsph_set_characteristics) and the
  // characteristic cells of every level
  ls.nsing = (int)(h->sing.size() / 3);
  ls.nseg = (int)(h->seg.size() / 6);
  if (ls.nsing > 0 || ls.nseg > 0) {
    double* d_pts = nullptr;
    const size_t npts = h->sing.size() + h->seg.size();
    API_CK(h, cudaMalloc(&d_pts, sizeof(double) * npts));
    h->ls_allocs.push_back(d_pts);
    if (!h->sing.empty())
      API_CK(h, cudaMemcpyAsync(d_pts, h->sing.data(), sizeof(double) * h->sing.size(), cudaMemcpyHostToDevice,
                                h->stream));
    if (!h->seg.empty())
      API_CK(h, cudaMemcpyAsync(d_pts + h->sing.size(), h->seg.data(), sizeof(double) * h->seg.size(),
                                cudaMemcpyHostToDevice, h->stream));
    ls.sing = d_pts;
    ls.seg = d_pts + h->sing.size();
    for (int l = 0; l < nlevels; l++) {
      int* chr = nullptr;
      API_CK(h, cudaMalloc(&chr, sizeof(int) * h->ls_ntot[l]));
      h->ls_allocs.push_back(chr);
      API_CK(h, ls_build_characteristics(ls.lv[l], D, h->ls_ntot[l], chr, ls.sing, ls.nsing, ls.seg, ls.nseg,
                                         h->stream));
      ls.lv[l].chr = chr;
    }
  }
  unsigned long long mb[3] = {0, 0, 0};
  API_CK(h, cudaMemcpyAsync(mb, d_max, sizeof(mb), cudaMemcpyDeviceToHost, h->stream));
  API_CK(h, cudaStreamSynchronize(h->stream));
  std::memcpy(&ls.max_phi, &mb[0], sizeof(double));
  std::memcpy(&ls.max_curv, &mb[1], sizeof(double));
  std::memcpy(&ls.min_curv, &mb[2], sizeof(double));
  if (!(ls.max_phi > 0)) return fail(h, MRSPH_ERR_ARG, "level set has no positive phi");
  double dl0 = 1.e20;
  for (int d = 0; d < D; d++) dl0 = std::min(ls.lv[0].dcell[d], dl0);
  ls.dl0 = dl0;
  ls.min_dl = h->prm.min_dl;
  ls.max_dl = h->prm.max_dl;
  ls.law = h->prm.scale_law;
  // middel_dl = fac_middel_dl * dl of level 0, fac 5 (level_set.cpp:940, sph_mesh_generation.cpp:271)
  ls.middle_dl = h->prm.middle_dl > 0 ? h->prm.middle_dl : 5.0 * dl0;
  EngineConfig cfg;
  cfg.prm.dim = D;
  cfg.prm.kernel = h->prm.kernel;
  cfg.prm.cell_ratio = h->prm.cell_ratio;
  cfg.prm.cutoff = h->prm.cutoff;
  cfg.prm.angle_thres = h->prm.angle_thres;
  cfg.prm.cos_thres = std::cos(h->prm.angle_thres);
  cfg.prm.nu_coeff = h->prm.nu_coeff;
  cfg.prm.damp_coeff = h->prm.damp_coeff;
  for (int d = 0; d < 3; d++) {
    cfg.prm.box_l[d] = h->prm.box_l[d];
    cfg.prm.box_r[d] = h->prm.box_r[d];
  }
  cfg.prm.seed = h->prm.seed;
  cfg.geo = h->geo;
  cfg.ls = ls;
  cfg.neighbor_cap = h->prm.neighbor_cap;
  cfg.stream = h->stream;
  h->nls = nlevels;
  h->eng = (h->prm.precision == MRSPH_FP64_PLAIN) ? make_engine_fp64(cfg) : make_engine_fp32(cfg);
  return 0;
}

int mrsph_set_characteristics(mrsph_handle* h, int nsing, const double* sing, int nseg, const double* seg) {
  if (!h) return fail(h, MRSPH_ERR_ARG, "null handle");
  if (h->eng) return fail(h, MRSPH_ERR_STATE, "mrsph_set_characteristics must come before mrsph_set_levelset");
  if (nsing < 0 || nseg < 0 || (nsing > 0 && !sing) || (nseg > 0 && !seg))
    return fail(h, MRSPH_ERR_ARG, "bad characteristic point or segment arrays");
  if (nsing > (1 << 20) || nseg > (1 << 20)) return fail(h, MRSPH_ERR_RANGE, "at most 2^20 points and segments");
  h->sing.assign(sing ? sing : nullptr, sing ? sing + 3 * (size_t)nsing : nullptr);
  h->seg.assign(seg ? seg : nullptr, seg ? seg + 6 * (size_t)nseg : nullptr);
  return 0;
}

int mrsph_get_levelset(mrsph_handle* h, int level, double* nx, double* ny, double* nz, double* curv,
                       unsigned char* tag, double* max_phi) {
  if (!h) return fail(h, MRSPH_ERR_ARG, "null handle");
  if (level < 0 || level >= h->nls) return fail(h, MRSPH_ERR_ARG, "no such level");
  API_CK(h, cudaSetDevice(h->prm.device));
  const LsLevel& L = h->ls.lv[level];
  long long ntot = h->ls_ntot[level];
  std::vector<double4> g(ntot);
  API_CK(h, cudaMemcpy(g.data(), L.g64, sizeof(double4) * ntot, cudaMemcpyDeviceToHost));
  for (long long a = 0; a < ntot; a++) {
    if (nx) nx[a] = g[a].y;
    if (ny) ny[a] = g[a].z;
    if (nz) nz[a] = g[a].w;
  }
  if (curv) API_CK(h, cudaMemcpy(curv, L.c64, sizeof(double) * ntot, cudaMemcpyDeviceToHost));
  if (tag) API_CK(h, cudaMemcpy(tag, L.tag, ntot, cudaMemcpyDeviceToHost));
  if (max_phi) *max_phi = h->ls.max_phi;
  return 0;
}

int mrsph_get_characteristics(mrsph_handle* h, int level, int* chr) {
  if (!h || !chr) return fail(h, MRSPH_ERR_ARG, "null argument");
  if (level < 0 || level >= h->nls) return fail(h, MRSPH_ERR_ARG, "no such level");
  API_CK(h, cudaSetDevice(h->prm.device));
  const LsLevel& L = h->ls.lv[level];
  const long long ntot = h->ls_ntot[level];
  if (!L.chr) {
    std::memset(chr, 0, sizeof(int) * ntot);
    return 0;
  }
  API_CK(h, cudaMemcpy(chr, L.chr, sizeof(int) * ntot, cudaMemcpyDeviceToHost));
  return 0;
}

int mrsph_volume_mass(mrsph_handle* h, int level, mrsph_volume_mass_stats* out, double* cell_vol,
                      double* cell_area) {
  if (!h || !out) return fail(h, MRSPH_ERR_ARG, "null argument");
  if (h->nls < 1) return fail(h, MRSPH_ERR_STATE, "mrsph_set_levelset must come first");
  if (level < 0) level += h->nls;
  if (level < 0 || level >= h->nls) return fail(h, MRSPH_ERR_ARG, "no such level");
  API_CK(h, cudaSetDevice(h->prm.device));
  const int D = h->prm.dim;
  const LsLevel& L = h->ls.lv[level];
  const long long ntot = h->ls_ntot[level];
  long long nin = 1;
  for (int d = 0; d < D; d++) nin *= 4LL * L.num_pkg[d];
  if (ntot >= (1LL << 31)) return fail(h, MRSPH_ERR_RANGE, "level set grid above 2^31 cells");
  const long long nb = (nin + 255) / 256;
  // one scratch allocation: cvol, carea, part, tot (doubles), list, cnt, table
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off += (bytes + 255) & ~(size_t)255;
    return o;
  };
  const size_t o_vol = take(sizeof(double) * ntot), o_area = take(sizeof(double) * ntot);
  const size_t o_part = take(sizeof(double) * 6 * nb), o_tot = take(sizeof(double) * 6);
  const size_t o_list = take(sizeof(int) * nin), o_cnt = take(3 * sizeof(unsigned long long));
  const size_t o_tab = take(256 * 16);
  char* buf = nullptr;
  API_CK(h, cudaMalloc(&buf, off));
  struct Free {
    char* p;
    ~Free() { cudaFree(p); }
  } guard{buf};
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  API_CK(h, cudaEventCreate(&e0));
  API_CK(h, cudaEventCreate(&e1));
  struct FreeEv {
    cudaEvent_t a, b;
    ~FreeEv() {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
    }
  } gev{e0, e1};
  double* cvol = reinterpret_cast<double*>(buf + o_vol);
  double* carea = reinterpret_cast<double*>(buf + o_area);
  long long ncut[2] = {0, 0};
  API_CK(h, cudaEventRecord(e0, h->stream));
  API_CK(h, ls_volume_mass(h->ls, level, D, cvol, carea, reinterpret_cast<int*>(buf + o_list),
                           reinterpret_cast<double*>(buf + o_part), reinterpret_cast<signed char*>(buf + o_tab),
                           reinterpret_cast<unsigned long long*>(buf + o_cnt),
                           reinterpret_cast<double*>(buf + o_tot), ncut, h->stream));
  API_CK(h, cudaEventRecord(e1, h->stream));
  double tot[6];
  API_CK(h, cudaMemcpyAsync(tot, buf + o_tot, sizeof(tot), cudaMemcpyDeviceToHost, h->stream));
  if (cell_vol) API_CK(h, cudaMemcpyAsync(cell_vol, cvol, sizeof(double) * ntot, cudaMemcpyDeviceToHost, h->stream));
  if (cell_area)
    API_CK(h, cudaMemcpyAsync(cell_area, carea, sizeof(double) * ntot, cudaMemcpyDeviceToHost, h->stream));
  API_CK(h, cudaStreamSynchronize(h->stream));
  float ms = 0.f;
  API_CK(h, cudaEventElapsedTime(&ms, e0, e1));
  out->total_mass = tot[0];
  out->total_mass_surface = tot[1];
  out->total_volume = tot[2];
  out->total_area = tot[3];
  out->num_interface_cell = ncut[0];
  out->total_mass_segment = tot[4];
  out->total_length = tot[5];
  // Get_num_particles, sph_mesh_generation.cpp:909-923
  const int nsing = (int)(h->sing.size() / 3);
  const long long n_segment = std::max((long long)(int)(tot[4] * 1. - 0.5 * nsing), 0LL);
  long long n_surface = std::max((long long)(int)(tot[1] * 1. - 0.5 * tot[4] * 1.), 0LL);
  const long long n_mesh = std::max((long long)(int)(tot[0] * 1. - 0.5 * tot[1] * 1.), 0LL);
  if (ncut[0] < n_surface) n_surface = ncut[0];
  out->num_particle_mesh = n_mesh;
  out->num_particle_surface = n_surface;
  out->num_particle_segment = n_segment;
  out->num_particle_singularity = nsing;
  out->num_particle = n_mesh + n_surface + nsing + n_segment;
  out->device_ms = ms;
  return 0;
}

#define NEED_ENG(h)                                                                   \
  do {                                                                                \
    if (!(h)) return fail(nullptr, MRSPH_ERR_ARG, "null handle");                     \
    if (!(h)->eng) return fail(h, MRSPH_ERR_STATE, "mrsph_set_levelset must come first"); \
    API_CK(h, cudaSetDevice((h)->prm.device));                                        \
  } while (0)

static int eng_rc(mrsph_handle* h, int rc) {
  if (rc) h->err = h->eng->err;
  return rc;
}

int mrsph_sample_levelset(mrsph_handle* h, long long n, const double* xyz, double* phi, double* norm, double* curv,
                          int* tag) {
  NEED_ENG(h);
  if (n <= 0 || !xyz) return fail(h, MRSPH_ERR_ARG, "no points");
  return eng_rc(h, h->eng->sample(n, xyz, phi, norm, curv, tag));
}

int mrsph_seed(mrsph_handle* h, long long n) {
  NEED_ENG(h);
  return eng_rc(h, h->eng->seed(n));
}

int mrsph_set_state(mrsph_handle* h, long long n, const mrsph_state_in* st, int pre_run) {
  NEED_ENG(h);
  if (!st || !st->xyz || n <= 0) return fail(h, MRSPH_ERR_ARG, "state needs positions");
  if (st->type)
    for (long long i = 0; i < n; i++)
      if (st->type[i] < MRSPH_REAL || st->type[i] > MRSPH_SEGMENT)
        return fail(h, MRSPH_ERR_ARG, "particle type must be REAL, SURFACE, SINGULARITY or SEGMENT");
  if (st->level)
    for (long long i = 0; i < n; i++)
      if (st->level[i] < 0 || st->level[i] >= h->geo.ncl) return fail(h, MRSPH_ERR_ARG, "level out of range");
  return eng_rc(h, h->eng->set_state(n, st, pre_run));
}

int mrsph_step(mrsph_handle* h, int nsteps) {
  NEED_ENG(h);
  return eng_rc(h, h->eng->step(nsteps));
}

int mrsph_step_timed(mrsph_handle* h, int nsteps, double* ms) {
  NEED_ENG(h);
  if (!ms || nsteps < 0) return fail(h, MRSPH_ERR_ARG, "bad arguments");
  return eng_rc(h, h->eng->step_timed(nsteps, ms));
}

int mrsph_profile_steps(mrsph_handle* h, int nsteps, double* phase_ms, int nphase) {
  NEED_ENG(h);
  if (!phase_ms || nsteps < 1 || nphase < 1 || nphase > 8) return fail(h, MRSPH_ERR_ARG, "bad arguments");
  return eng_rc(h, h->eng->profile_steps(nsteps, phase_ms, nphase));
}

int mrsph_run_phase(mrsph_handle* h, int phase) {
  NEED_ENG(h);
  if (phase < MRSPH_PHASE_MAP || phase > MRSPH_PHASE_FORCE2) return fail(h, MRSPH_ERR_ARG, "unknown phase");
  return eng_rc(h, h->eng->run_phase(phase));
}

int mrsph_sync(mrsph_handle* h) {
  if (!h) return fail(nullptr, MRSPH_ERR_ARG, "null handle");
  API_CK(h, cudaSetDevice(h->prm.device));
  API_CK(h, cudaStreamSynchronize(h->stream));
  return 0;
}

int mrsph_get_stats(mrsph_handle* h, mrsph_stats* out) {
  NEED_ENG(h);
  if (!out) return fail(h, MRSPH_ERR_ARG, "null output");
  std::memset(out, 0, sizeof(*out));
  return eng_rc(h, h->eng->stats(out));
}

int mrsph_get_particles(mrsph_handle* h, const mrsph_particle_view* v) {
  NEED_ENG(h);
  if (!v) return fail(h, MRSPH_ERR_ARG, "null view");
  return eng_rc(h, h->eng->get_particles(v));
}

int mrsph_get_cells(mrsph_handle* h, int* level_cell, int* sorted_ids) {
  NEED_ENG(h);
  return eng_rc(h, h->eng->get_cells(level_cell, sorted_ids));
}

int mrsph_get_neighbors(mrsph_handle* h, long long* offsets, int* nb, long long cap, long long* total) {
  NEED_ENG(h);
  return eng_rc(h, h->eng->get_neighbors(offsets, nb, cap, total));
}

int mrsph_upload_positions(mrsph_handle* h, const double* xyz) {
  NEED_ENG(h);
  if (!xyz) return fail(h, MRSPH_ERR_ARG, "null positions");
  return eng_rc(h, h->eng->upload_positions(xyz));
}

int mrsph_download_positions(mrsph_handle* h, double* xyz) {
  NEED_ENG(h);
  if (!xyz) return fail(h, MRSPH_ERR_ARG, "null positions");
  return eng_rc(h, h->eng->download_positions(xyz));
}

}  // extern "C"
