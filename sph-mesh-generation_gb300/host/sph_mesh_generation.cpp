// sph_mesh_generation.cpp — C++ host layer over the C ABI (see the header).
#include "sph_mesh_generation.hpp"

#include <sys/stat.h>

#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iterator>

namespace mrsph_host {

namespace {
constexpr double PI_REF = 3.1415926;  // glbparam.h:186

std::string last_error(mrsph_handle* h) {
  char buf[512] = {0};
  mrsph_last_error(h, buf, sizeof(buf));
  return std::string(buf);
}

// creates d and any missing parent directories
void make_dir(const std::string& d) {
  for (size_t k = 1; k <= d.size(); k++)
    if (k == d.size() || d[k] == '/') mkdir(d.substr(0, k).c_str(), 0755);
}
}  // namespace

mrsph_params default_params(int dim) {
  mrsph_params p{};
  p.dim = dim;
  p.kernel = MRSPH_KERNEL_HYPERBOLIC;
  p.precision = MRSPH_FP64_PLAIN;
  p.cell_ratio = dim == 2 ? 2.0 : 1.45;
  p.cutoff = 2.0;
  p.angle_thres = PI_REF * 0.4;
  p.nu_coeff = 0.1;
  p.damp_coeff = 0.0;
  p.min_dl = 0.01;
  p.max_dl = 0.01;
  for (int d = 0; d < 3; d++) {
    p.box_l[d] = 0.0;
    p.box_r[d] = 1.0;
  }
  p.seed = 0;
  p.neighbor_cap = 0;
  p.device = 0;
  p.scale_law = 0;
  p.middle_dl = 0.0;
  return p;
}

LevelGrid make_level(const std::function<double(double, double, double)>& sdf, int dim,
                     const std::array<double, 3>& box_l, const std::array<double, 3>& dpkg,
                     const std::array<int, 3>& num_pkg, int margin) {
  LevelGrid L;
  L.box_l = box_l;
  L.dpkg = dpkg;
  L.num_pkg = num_pkg;
  L.margin = margin;
  std::array<std::vector<double>, 3> ax;
  for (int d = 0; d < 3; d++) {
    if (d >= dim) {
      ax[d] = {0.0};
      continue;
    }
    const double dcell = dpkg[d] / 4.0;
    for (int pk = -margin; pk < num_pkg[d] + margin; pk++)
      for (int cl = 0; cl < 4; cl++) ax[d].push_back((double)pk * dpkg[d] + ((double)cl + 0.5) * dcell + box_l[d]);
  }
  L.phi.reserve(ax[0].size() * ax[1].size() * ax[2].size());
  for (double z : ax[2])
    for (double y : ax[1])
      for (double x : ax[0]) L.phi.push_back(sdf(x, y, z));
  return L;
}

// package mask of a finer nested level: active where some cell has |phi| < band
static std::vector<unsigned char> nested_active(const LevelGrid& L, double band, int dim) {
  const int m = L.margin;
  const int nx = L.num_pkg[0] + 2 * m, ny = L.num_pkg[1] + 2 * m, nz = dim == 3 ? L.num_pkg[2] + 2 * m : 1;
  const int cx = 4 * nx, cy = 4 * ny;
  std::vector<unsigned char> act((size_t)nx * ny * nz, 0);
  for (int pz = 0; pz < nz; pz++)
    for (int py = 0; py < ny; py++)
      for (int px = 0; px < nx; px++) {
        double mn = 1e300;
        for (int c = 0; c < (dim == 3 ? 4 : 1); c++)
          for (int b = 0; b < 4; b++)
            for (int a = 0; a < 4; a++) {
              const int z = dim == 3 ? 4 * pz + c : 0;
              mn = std::min(mn, std::fabs(L.phi[((size_t)z * cy + (4 * py + b)) * cx + (4 * px + a)]));
            }
        act[((size_t)pz * ny + py) * nx + px] = mn < band ? 1 : 0;
      }
  return act;
}

static double max_phi(const std::vector<LevelGrid>& levels, int dim) {
  double mp = 0.0;
  for (const auto& L : levels) {
    const int m = 4 * L.margin;
    const int cx = 4 * (L.num_pkg[0] + 2 * L.margin), cy = 4 * (L.num_pkg[1] + 2 * L.margin);
    const int cz = dim == 3 ? 4 * (L.num_pkg[2] + 2 * L.margin) : 1;
    for (int z = (dim == 3 ? m : 0); z < (dim == 3 ? cz - m : 1); z++)
      for (int y = m; y < cy - m; y++)
        for (int x = m; x < cx - m; x++) {
          const double v = L.phi[((size_t)z * cy + y) * cx + x];
          if (v > 0) mp = std::max(mp, v);
        }
  }
  return mp;
}

long long particle_count(const std::vector<LevelGrid>& levels, const mrsph_params& p) {
  const int dim = p.dim;
  const double mp = max_phi(levels, dim);
  const LevelGrid& F = levels.back();
  double dl0 = 1e20;
  for (int d = 0; d < dim; d++) dl0 = std::min(dl0, levels[0].dpkg[d] / 4.0);
  double dV = 1.0;
  for (int d = 0; d < dim; d++) dV *= F.dpkg[d] / 4.0;
  const int m = 4 * F.margin;
  const int cx = 4 * (F.num_pkg[0] + 2 * F.margin), cy = 4 * (F.num_pkg[1] + 2 * F.margin);
  const int cz = dim == 3 ? 4 * (F.num_pkg[2] + 2 * F.margin) : 1;
  double tot = 0.0;
  for (int z = (dim == 3 ? m : 0); z < (dim == 3 ? cz - m : 1); z++)
    for (int y = m; y < cy - m; y++)
      for (int x = m; x < cx - m; x++) {
        const double phi = F.phi[((size_t)z * cy + y) * cx + x];
        if (!(phi > 0)) continue;
        // Levelset::Get_scale, level_set.cpp:311-351 (tanh law)
        const double s = p.min_dl + std::tanh(2.5 * std::fabs(phi) / mp) / std::tanh(2.5) * (p.max_dl - p.min_dl);
        tot += dV / std::pow(s, dim);
      }
  return (long long)tot;
}

bool cell_levels_consistent(const double* box_l, const double* box_r, int dim, double max_scale,
                            double min_scale) {
  double dom[3], st = 1e300;
  for (int d = 0; d < dim; d++) {
    dom[d] = box_r[d] - box_l[d];
    st = std::min(st, dom[d]);
  }
  const double temp = std::floor(st / max_scale);
  if (temp < 1) return false;
  const double ini = st / temp;
  double sc = ini;
  int nl = 1;
  while (sc + 1.e-6 > min_scale) {
    sc /= 2;
    nl++;
  }
  nl -= 1;
  int n0[3];
  for (int d = 0; d < dim; d++) n0[d] = (int)(dom[d] / ini);
  for (int l = 0; l < nl; l++) {
    double s = 1e300;
    for (int d = 0; d < dim; d++) s = std::min(s, dom[d] / (n0[d] * std::ldexp(1.0, l)));
    if (std::fabs(s - std::ldexp(ini, -l)) > 1.e-10) return false;
  }
  return true;
}

Case disc_hole_2d(double spacing, int grid, int kernel, double h_over_dx, int precision, unsigned long long seed) {
  Case c;
  c.name = "disc_hole_2d";
  mrsph_params p = default_params(2);
  const int npkg_unit = grid / 4;
  const double dpkg = 1.0 / npkg_unit;
  const double cell_ratio = 2.0 * h_over_dx;
  int margin_pkg = std::max(npkg_unit / 16, 1);
  for (;;) {
    const double bl[2] = {-margin_pkg * dpkg, -margin_pkg * dpkg};
    const double br[2] = {1.0 + margin_pkg * dpkg, 1.0 + margin_pkg * dpkg};
    if (cell_levels_consistent(bl, br, 2, spacing * cell_ratio, spacing * cell_ratio)) break;
    margin_pkg++;
  }
  const double lo = -margin_pkg * dpkg, hi = 1.0 + margin_pkg * dpkg;
  const int npkg = npkg_unit + 2 * margin_pkg;
  p.kernel = kernel;
  p.precision = precision;
  p.min_dl = spacing;
  p.max_dl = spacing;
  p.cell_ratio = cell_ratio;
  p.box_l[0] = p.box_l[1] = lo;
  p.box_r[0] = p.box_r[1] = hi;
  p.box_l[2] = p.box_r[2] = 0.0;
  p.seed = seed;
  auto sdf = [](double X, double Y, double) {
    const double disc = std::sqrt((X - 0.5) * (X - 0.5) + (Y - 0.5) * (Y - 0.5)) - 0.2;
    return std::min(std::min(std::min(X, 1.0 - X), std::min(Y, 1.0 - Y)), disc);
  };
  c.params = p;
  c.levels.push_back(make_level(sdf, 2, {lo, lo, 0.0}, {dpkg, dpkg, 1.0}, {npkg, npkg, 1}));
  c.n_particles = particle_count(c.levels, p);
  c.steps = 200;
  return c;
}

Case torus_3d(double dx_min, double dx_max, int kernel, double h_over_dx, int precision, unsigned long long seed,
              int fine_pkg, int nlevels) {
  Case c;
  c.name = "torus_3d";
  mrsph_params p = default_params(3);
  const int npx0 = fine_pkg >> (nlevels - 1);
  const double dpkg0 = 3.2 / npx0;
  const int npz0 = (int)std::nearbyint(1.2 / dpkg0);
  const double zhalf = 0.5 * npz0 * dpkg0;
  const std::array<double, 3> box_l{{-1.6, -1.6, -zhalf}};
  p.kernel = kernel;
  p.precision = precision;
  p.min_dl = dx_min;
  p.max_dl = dx_max;
  p.cell_ratio = 2.0 * h_over_dx;
  p.box_l[0] = -1.6; p.box_l[1] = -1.6; p.box_l[2] = -zhalf;
  p.box_r[0] = 1.6; p.box_r[1] = 1.6; p.box_r[2] = zhalf;
  p.seed = seed;
  if (!cell_levels_consistent(p.box_l, p.box_r, 3, dx_max * p.cell_ratio, dx_min * p.cell_ratio))
    throw Error(MRSPH_ERR_ARG, "torus box gives an inconsistent cell-list level plan");
  auto sdf = [](double X, double Y, double Z) {
    const double a = std::sqrt(X * X + Y * Y) - 1.0;
    return 0.35 - std::sqrt(a * a + Z * Z);
  };
  for (int l = 0; l < nlevels; l++) {
    const int f = 1 << l;
    const double dp = dpkg0 / f;
    LevelGrid L = make_level(sdf, 3, box_l, {dp, dp, dp}, {npx0 * f, npx0 * f, npz0 * f});
    if (l > 0) L.active = nested_active(L, 4.0 * (dp * 2 / 4.0), 3);
    c.levels.push_back(std::move(L));
  }
  c.params = p;
  c.n_particles = particle_count(c.levels, p);
  c.steps = 500;
  return c;
}

Case box_with_corners(int dim, double spacing, int grid, int kernel, double h_over_dx, int precision,
                      unsigned long long seed, double lo_b, double hi_b, bool edges) {
  if (dim != 2 && dim != 3) throw Error(MRSPH_ERR_ARG, "box_with_corners: dim must be 2 or 3");
  Case c;
  c.name = dim == 3 ? "box_3d" : "box_2d";
  mrsph_params p = default_params(dim);
  const int npkg_unit = grid / 4;
  const double dpkg = 1.0 / npkg_unit;
  const double cell_ratio = 2.0 * h_over_dx;
  int margin_pkg = std::max(npkg_unit / 16, 1);
  for (;;) {
    double bl[3], br[3];
    for (int d = 0; d < 3; d++) {
      bl[d] = -margin_pkg * dpkg;
      br[d] = 1.0 + margin_pkg * dpkg;
    }
    if (cell_levels_consistent(bl, br, dim, spacing * cell_ratio, spacing * cell_ratio)) break;
    margin_pkg++;
  }
  const double lo = -margin_pkg * dpkg, hi = 1.0 + margin_pkg * dpkg;
  const int npkg = npkg_unit + 2 * margin_pkg;
  p.kernel = kernel;
  p.precision = precision;
  p.min_dl = spacing;
  p.max_dl = spacing;
  p.cell_ratio = cell_ratio;
  for (int d = 0; d < 3; d++) {
    p.box_l[d] = d < dim ? lo : 0.0;
    p.box_r[d] = d < dim ? hi : 0.0;
  }
  p.seed = seed;
  auto sdf = [=](double X, double Y, double Z) {
    double out = std::min(std::min(X - lo_b, hi_b - X), std::min(Y - lo_b, hi_b - Y));
    if (dim == 3) out = std::min(out, std::min(Z - lo_b, hi_b - Z));
    return out;
  };
  c.params = p;
  c.levels.push_back(make_level(sdf, dim, {lo, lo, dim == 3 ? lo : 0.0}, {dpkg, dpkg, dim == 3 ? dpkg : 1.0},
                                {npkg, npkg, dim == 3 ? npkg : 1}));
  c.n_particles = particle_count(c.levels, p);
  c.steps = 200;
  const double v[2] = {lo_b, hi_b};
  for (int z = 0; z < (dim == 3 ? 2 : 1); z++)
    for (int y = 0; y < 2; y++)
      for (int x = 0; x < 2; x++) {
        c.singularities.push_back(v[x]);
        c.singularities.push_back(v[y]);
        c.singularities.push_back(dim == 3 ? v[z] : 0.0);
      }
  if (dim == 3 && edges)
    for (int a = 0; a < 2; a++)
      for (int b = 0; b < 2; b++) {
        const double along_x[6] = {lo_b, v[a], v[b], hi_b, v[a], v[b]};
        const double along_y[6] = {v[a], lo_b, v[b], v[a], hi_b, v[b]};
        const double along_z[6] = {v[a], v[b], lo_b, v[a], v[b], hi_b};
        c.segments.insert(c.segments.end(), along_x, along_x + 6);
        c.segments.insert(c.segments.end(), along_y, along_y + 6);
        c.segments.insert(c.segments.end(), along_z, along_z + 6);
      }
  return c;
}

// ------------------------------------------------------------------ solver
SPH_mesh_generation::SPH_mesh_generation(const Case& c, int device) : case_(c) {
  case_.params.device = device;
  if (int rc = mrsph_create(&case_.params, &h_)) throw Error(rc, "mrsph_create: " + last_error(nullptr));
  std::vector<mrsph_levelset_level> lv(case_.levels.size());
  for (size_t l = 0; l < lv.size(); l++) {
    const LevelGrid& L = case_.levels[l];
    for (int d = 0; d < 3; d++) {
      lv[l].box_l[d] = L.box_l[d];
      lv[l].dpkg[d] = L.dpkg[d];
      lv[l].num_pkg[d] = L.num_pkg[d];
    }
    lv[l].margin = L.margin;
    lv[l].phi = L.phi.data();
    lv[l].active = L.active.empty() ? nullptr : L.active.data();
  }
  if (!case_.singularities.empty() || !case_.segments.empty())
    check(mrsph_set_characteristics(h_, (int)(case_.singularities.size() / 3),
                                    case_.singularities.empty() ? nullptr : case_.singularities.data(),
                                    (int)(case_.segments.size() / 6),
                                    case_.segments.empty() ? nullptr : case_.segments.data()),
          "mrsph_set_characteristics");
  check(mrsph_set_levelset(h_, (int)lv.size(), lv.data()), "mrsph_set_levelset");
}

mrsph_tet_quality SPH_mesh_generation::Reconstruct_tets(std::vector<int>& tets) {
  mrsph_tet_quality q{};
  long long nt = 0;
  tets.assign(4 * (size_t)std::max<long long>(8 * n_, 1), 0);
  check(mrsph_tetrahedralize(h_, tets.data(), (long long)(tets.size() / 4), &nt, &q), "mrsph_tetrahedralize");
  if (4 * nt > (long long)tets.size()) {
    tets.assign(4 * (size_t)nt, 0);
    check(mrsph_tetrahedralize(h_, tets.data(), nt, &nt, &q), "mrsph_tetrahedralize");
  }
  tets.resize(4 * (size_t)nt);
  return q;
}

mrsph_cvp_result SPH_mesh_generation::Partitioning(std::vector<double>& vp, const mrsph_cvp_params& p,
                                                   std::vector<int>* labels, std::vector<double>* vp_mass) {
  if ((int)vp.size() != 3 * p.num_vp) throw Error(MRSPH_ERR_ARG, "Partitioning: vp must hold num_vp x 3 values");
  if (labels) labels->assign(n_, 0);
  if (vp_mass) vp_mass->assign(p.num_vp, 0.0);
  mrsph_cvp_result r{};
  check(mrsph_cvp(h_, &p, vp.data(), labels ? labels->data() : nullptr, vp_mass ? vp_mass->data() : nullptr, &r),
        "mrsph_cvp");
  return r;
}

mrsph_cvp_result SPH_mesh_generation::Partitioning_for_initial_VP_distribution(
    const std::vector<double>& xyz, const std::vector<double>& mass, const std::vector<double>& mass_surface,
    std::vector<double>& vp, const mrsph_cvp_params& p, std::vector<int>* labels, std::vector<double>* vp_mass,
    std::vector<double>* ghosts) {
  const long long n = (long long)mass.size();
  if ((long long)xyz.size() != 3 * n || (long long)mass_surface.size() != n)
    throw Error(MRSPH_ERR_ARG, "Partitioning_for_initial_VP_distribution: xyz, mass and mass_surface disagree");
  if ((int)vp.size() != 3 * p.num_vp) throw Error(MRSPH_ERR_ARG, "vp must hold num_vp x 3 values");
  if (labels) labels->assign(n, 0);
  if (vp_mass) vp_mass->assign(p.num_vp, 0.0);
  std::vector<double> g(3 * (size_t)p.num_vp, 0.0);
  int ng = 0;
  mrsph_cvp_result r{};
  check(mrsph_cvp_lset(h_, n, xyz.data(), mass.data(), mass_surface.data(), &p, vp.data(),
                       labels ? labels->data() : nullptr, vp_mass ? vp_mass->data() : nullptr, g.data(), &ng, &r),
        "mrsph_cvp_lset");
  if (ghosts) ghosts->assign(g.begin(), g.begin() + 3 * (size_t)ng);
  return r;
}

SPH_mesh_generation::~SPH_mesh_generation() {
  if (h_) mrsph_destroy(h_);
}

void SPH_mesh_generation::check(int rc, const char* what) {
  if (rc) throw Error(rc, std::string(what) + ": " + last_error(h_));
}

void SPH_mesh_generation::Initialize_case(long long n) {
  n_ = n < 0 ? case_.n_particles : n;
  check(mrsph_seed(h_, n_), "mrsph_seed");
}

mrsph_volume_mass_stats SPH_mesh_generation::Calculate_total_volume_mass(int level) {
  mrsph_volume_mass_stats st{};
  check(mrsph_volume_mass(h_, level, &st, nullptr, nullptr), "mrsph_volume_mass");
  return st;
}

void SPH_mesh_generation::SPH_run_mesh_generation(int nsteps) { check(mrsph_step(h_, nsteps), "mrsph_step"); }

void SPH_mesh_generation::Run_phase(int phase) { check(mrsph_run_phase(h_, phase), "mrsph_run_phase"); }

mrsph_stats SPH_mesh_generation::Stats() {
  mrsph_stats s{};
  check(mrsph_get_stats(h_, &s), "mrsph_get_stats");
  return s;
}

double SPH_mesh_generation::Get_timestep() { return Stats().dt; }

std::vector<double> SPH_mesh_generation::Positions() {
  std::vector<double> xyz((size_t)3 * n_);
  check(mrsph_download_positions(h_, xyz.data()), "mrsph_download_positions");
  return xyz;
}

void SPH_mesh_generation::Particle_fields(std::vector<int>& type, std::vector<double>& h,
                                          std::vector<double>& norm, std::vector<int>& nn) {
  type.assign(n_, 0);
  h.assign(n_, 0.0);
  norm.assign(3 * n_, 0.0);
  mrsph_particle_view v{};
  v.type = type.data();
  v.h = h.data();
  v.norm = norm.data();
  check(mrsph_get_particles(h_, &v), "mrsph_get_particles");
  std::vector<long long> off(n_ + 1, 0);
  long long total = 0;
  check(mrsph_get_neighbors(h_, nullptr, nullptr, 0, &total), "mrsph_get_neighbors");
  std::vector<int> nb(total > 0 ? total : 1);
  check(mrsph_get_neighbors(h_, off.data(), nb.data(), total, &total), "mrsph_get_neighbors");
  nn.assign(n_, 0);
  for (long long i = 0; i < n_; i++) nn[i] = (int)(off[i + 1] - off[i]);
}

std::string SPH_mesh_generation::Save_particle_post_file(const std::string& root, long long run_time, bool first) {
  const std::string dir = root + "/rstfile_particles";
  make_dir(root);
  make_dir(dir);
  {
    std::ofstream lst(dir + "/list.csv", first ? std::ios::trunc : std::ios::app);
    if (first) lst << 1 << "\n";
    lst << run_time << " " << n_ << "\n";
  }
  const std::string path = dir + "/step_" + std::to_string(run_time) + "_rank_0.pst";
  write_pst(path, Positions());
  return path;
}

void SPH_mesh_generation::Load_data_for_post(const std::string& pst, bool pre_run) {
  std::vector<double> xyz = read_pst(pst);
  mrsph_state_in st{};
  st.xyz = xyz.data();
  n_ = (long long)(xyz.size() / 3);
  check(mrsph_set_state(h_, n_, &st, pre_run ? 1 : 0), "mrsph_set_state");
}

double Solver::SPH_Mesh_Generation_Solver(int total_steps, int output_interval, const std::string& output_root) {
  double ms_total = 0.0;
  int done = 0;
  bool first = true;
  const int chunk = output_interval > 0 ? output_interval : total_steps;
  while (done < total_steps) {
    const int k = std::min(chunk, total_steps - done);
    double ms = 0.0;
    int rc = mrsph_step_timed(sim_.handle(), k, &ms);
    if (rc) throw Error(rc, "mrsph_step_timed: " + last_error(sim_.handle()));
    ms_total += ms;
    done += k;
    if (!output_root.empty()) {
      const long long step = (long long)sim_.Stats().step;
      sim_.Save_particle_post_file(output_root, step, first);
      if (write_vtu_) Particle_binary_writer(output_root + "/outdata").Output_particle(n_out_++, sim_, step);
      first = false;
    }
  }
  return ms_total;
}

double Solver::Load_solver(const Initialization& ini, const std::string& output_root) {
  const int every = (int)ini.Get_dt();
  if (every < 1) throw Error(MRSPH_ERR_ARG, "output interval below one step");
  return SPH_Mesh_Generation_Solver(ini.Get_num_timestep() * every, every, output_root);
}

namespace {

// one appended array: its header line and its raw little-endian bytes
struct VtuArray {
  std::string name, type;
  int comps;  // 0: no NumberOfComponents attribute (the cell arrays)
  std::string raw;
};

template <class T>
std::string raw_of(const T* p, size_t count) {
  std::string r(sizeof(T) * count, '\0');
  if (count) std::memcpy(&r[0], p, r.size());  // the library only builds on little-endian hosts
  return r;
}

std::string vtu_text(long long n, long long m, const std::vector<VtuArray>& pd, const std::vector<VtuArray>& cd,
                     const std::vector<VtuArray>& pts, const std::vector<VtuArray>& cells) {
  std::string head, blobs;
  unsigned long long offset = 0;
  auto add = [&](const VtuArray& a) {
    head += "      <DataArray type=\"" + a.type + "\" Name=\"" + a.name + "\"";
    if (a.comps > 0) head += " NumberOfComponents=\"" + std::to_string(a.comps) + "\"";
    head += " format=\"appended\" offset=\"" + std::to_string(offset) + "\"/>\n";
    const uint32_t nb = (uint32_t)a.raw.size();
    blobs += raw_of(&nb, 1) + a.raw;
    offset += 4 + a.raw.size();
  };
  head += "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n";
  head += " <UnstructuredGrid>\n";
  head += "  <Piece NumberOfPoints=\"" + std::to_string(n) + "\" NumberOfCells=\"" + std::to_string(m) + "\">\n";
  head += "    <PointData Vectors=\"vector\">\n";
  for (const auto& a : pd) add(a);
  head += "    </PointData>\n";
  if (!cd.empty()) {
    head += "    <CellData Vectors=\"vector\">\n";
    for (const auto& a : cd) add(a);
    head += "    </CellData>\n";
  }
  head += "    <Points>\n";
  for (const auto& a : pts) add(a);
  head += "    </Points>\n    <Cells>\n";
  for (const auto& a : cells) add(a);
  head += "    </Cells>\n  </Piece>\n </UnstructuredGrid>\n <AppendedData encoding=\"raw\">\n _";
  return head + blobs + "\n </AppendedData>\n</VTKFile>\n";
}

}  // namespace

// the reference's default particle point fields and the positions
void particle_arrays(const ParticleFields& f, std::vector<VtuArray>& pd, std::vector<VtuArray>& pts) {
  const long long n = f.n;
  std::vector<int> ids(n), zeros(n, 0);
  std::vector<float> h(n), nrm(3 * n), pos(3 * n);
  for (long long i = 0; i < n; i++) {
    ids[i] = (int)i;
    h[i] = (float)f.h[i];
    for (int d = 0; d < 3; d++) {
      nrm[3 * i + d] = (float)f.norm[3 * i + d];
      pos[3 * i + d] = (float)f.xyz[3 * i + d];
    }
  }
  pd = {{"id", "Int32", 1, raw_of(ids.data(), n)},       {"local_id", "Int32", 1, raw_of(ids.data(), n)},
        {"type", "Int32", 1, raw_of(f.type, n)},         {"h", "Float32", 1, raw_of(h.data(), n)},
        {"NN", "Int32", 1, raw_of(f.nn, n)},             {"color", "Int32", 1, raw_of(zeros.data(), n)},
        {"norm", "Float32", 3, raw_of(nrm.data(), 3 * n)}};
  pts = {{"Position", "Float32", 3, raw_of(pos.data(), 3 * n)}};
}

std::string particle_vtu(const ParticleFields& f) {
  const long long n = f.n;
  std::vector<VtuArray> pd, pts;
  particle_arrays(f, pd, pts);
  std::vector<int> ids(n), offs(n);
  for (long long i = 0; i < n; i++) {
    ids[i] = (int)i;
    offs[i] = (int)(i + 1);
  }
  std::vector<unsigned char> types(n, 1);  // VTK_VERTEX
  std::vector<VtuArray> cells = {{"connectivity", "Int32", 0, raw_of(ids.data(), n)},
                                 {"offsets", "Int32", 0, raw_of(offs.data(), n)},
                                 {"types", "UInt8", 0, raw_of(types.data(), n)}};
  return vtu_text(n, n, pd, {}, pts, cells);
}

std::string mesh_vtu(const ParticleFields& f, long long ntri, const int* tris) {
  std::vector<VtuArray> pd, pts;
  particle_arrays(f, pd, pts);
  // per-triangle area and aspect ratio (longest / shortest edge) in the plane
  // (Tri_quality_statistics, graph_mesh.cpp:411-670)
  std::vector<float> area(ntri), aspect(ntri);
  std::vector<int> offs(ntri);
  for (long long t = 0; t < ntri; t++) {
    const double* a = f.xyz + 3 * (long long)tris[3 * t];
    const double* b = f.xyz + 3 * (long long)tris[3 * t + 1];
    const double* c = f.xyz + 3 * (long long)tris[3 * t + 2];
    auto len = [](const double* p, const double* q) {
      const double dx = q[0] - p[0], dy = q[1] - p[1];
      return std::sqrt(dx * dx + dy * dy);
    };
    const double e0 = len(a, b), e1 = len(b, c), e2 = len(c, a);
    area[t] = (float)(0.5 * std::fabs((b[0] - a[0]) * (c[1] - a[1]) - (b[1] - a[1]) * (c[0] - a[0])));
    aspect[t] = (float)(std::max(std::max(e0, e1), e2) / std::min(std::min(e0, e1), e2));
    offs[t] = (int)(3 * (t + 1));
  }
  std::vector<unsigned char> types(ntri, 5);  // VTK_TRIANGLE
  std::vector<VtuArray> cd = {{"vol", "Float32", 1, raw_of(area.data(), ntri)},
                              {"aspect", "Float32", 1, raw_of(aspect.data(), ntri)}};
  std::vector<VtuArray> cells = {{"connectivity", "Int32", 0, raw_of(tris, 3 * ntri)},
                                 {"offsets", "Int32", 0, raw_of(offs.data(), ntri)},
                                 {"types", "UInt8", 0, raw_of(types.data(), ntri)}};
  return vtu_text(f.n, ntri, pd, cd, pts, cells);
}

std::string tet_mesh_vtu(const ParticleFields& f, long long ntet, const int* tets) {
  std::vector<VtuArray> pd, pts;
  particle_arrays(f, pd, pts);
  // per-tet volume, aspect ratio (longest edge / smallest height), radius
  // ratio (3 r_in / r_circ) and smallest dihedral angle (Tet_quality_statistics,
  // graph_mesh.cpp:1967-2400)
  std::vector<float> vol(ntet), aspect(ntet), ratio(ntet), mind(ntet);
  std::vector<int> offs(ntet);
  auto cross = [](const double* u, const double* v, double* w) {
    w[0] = u[1] * v[2] - u[2] * v[1];
    w[1] = u[2] * v[0] - u[0] * v[2];
    w[2] = u[0] * v[1] - u[1] * v[0];
  };
  auto dot = [](const double* u, const double* v) { return u[0] * v[0] + u[1] * v[1] + u[2] * v[2]; };
  for (long long t = 0; t < ntet; t++) {
    const double* P[4];
    for (int k = 0; k < 4; k++) P[k] = f.xyz + 3 * (long long)tets[4 * t + k];
    double A[3][3], N[4][3], H[4], c[3];
    for (int k = 0; k < 3; k++)
      for (int q = 0; q < 3; q++) A[k][q] = P[k][q] - P[3][q];
    cross(A[1], A[2], N[0]);
    cross(A[2], A[0], N[1]);
    cross(A[0], A[1], N[2]);
    const double det = dot(A[0], N[0]);
    const double r[3] = {0.5 * dot(A[0], A[0]), 0.5 * dot(A[1], A[1]), 0.5 * dot(A[2], A[2])};
    for (int q = 0; q < 3; q++) c[q] = (r[0] * N[0][q] + r[1] * N[1][q] + r[2] * N[2][q]) / det;
    for (int k = 0; k < 3; k++)
      for (int q = 0; q < 3; q++) N[k][q] /= det;
    for (int q = 0; q < 3; q++) N[3][q] = -(N[0][q] + N[1][q] + N[2][q]);
    double hsum = 0.0, hmax = 0.0, longest = 0.0, cmax = -2.0;
    for (int k = 0; k < 4; k++) {
      H[k] = std::sqrt(dot(N[k], N[k]));
      hsum += H[k];
      hmax = std::max(hmax, H[k]);
    }
    for (int a = 0; a < 4; a++)
      for (int b = a + 1; b < 4; b++) {
        const double e[3] = {P[a][0] - P[b][0], P[a][1] - P[b][1], P[a][2] - P[b][2]};
        longest = std::max(longest, dot(e, e));
        double ua[3], ub[3];
        for (int q = 0; q < 3; q++) { ua[q] = N[a][q] / H[a]; ub[q] = N[b][q] / H[b]; }
        cmax = std::max(cmax, -dot(ua, ub));
      }
    vol[t] = (float)(std::fabs(det) / 6.0);
    aspect[t] = (float)(std::sqrt(longest) * hmax);
    ratio[t] = (float)(3.0 / hsum / std::sqrt(dot(c, c)));
    mind[t] = (float)(std::acos(std::min(std::max(cmax, -1.0), 1.0)) / PI_REF * 180.0);
    offs[t] = (int)(4 * (t + 1));
  }
  std::vector<unsigned char> types(ntet, 10);  // VTK_TETRA
  std::vector<VtuArray> cd = {{"vol", "Float32", 1, raw_of(vol.data(), ntet)},
                              {"aspect", "Float32", 1, raw_of(aspect.data(), ntet)},
                              {"radius_ratio", "Float32", 1, raw_of(ratio.data(), ntet)},
                              {"mindihedangle", "Float32", 1, raw_of(mind.data(), ntet)}};
  std::vector<VtuArray> cells = {{"connectivity", "Int32", 0, raw_of(tets, 4 * ntet)},
                                 {"offsets", "Int32", 0, raw_of(offs.data(), ntet)},
                                 {"types", "UInt8", 0, raw_of(types.data(), ntet)}};
  return vtu_text(f.n, ntet, pd, cd, pts, cells);
}

std::string particle_pvtu(const std::string& piece) {
  std::string t = "<VTKFile type=\"PUnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n"
                  " <PUnstructuredGrid GhostLevel=\"0\">\n  <PPointData>\n";
  const char* names[7] = {"id", "local_id", "type", "h", "NN", "color", "norm"};
  const char* types[7] = {"Int32", "Int32", "Int32", "Float32", "Int32", "Int32", "Float32"};
  for (int k = 0; k < 7; k++)
    t += std::string("    <PDataArray type=\"") + types[k] + "\" Name=\"" + names[k] +
         "\" NumberOfComponents=\"" + (k == 6 ? "3" : "1") + "\"/>\n";
  t += "  </PPointData>\n  <PPoints>\n    <PDataArray type=\"Float32\" Name=\"Position\" "
       "NumberOfComponents=\"3\"/>\n  </PPoints>\n  <Piece Source=\"" + piece +
       "\"/>\n </PUnstructuredGrid>\n</VTKFile>\n";
  return t;
}

std::string mesh_pvtu(const std::string& piece, bool tets) {
  std::string t = particle_pvtu(piece);  // the cell fields go between the point fields and the points
  std::string cells = "  <PCellData>\n    <PDataArray type=\"Float32\" Name=\"vol\" NumberOfComponents=\"1\"/>\n"
                      "    <PDataArray type=\"Float32\" Name=\"aspect\" NumberOfComponents=\"1\"/>\n";
  if (tets)
    cells += "    <PDataArray type=\"Float32\" Name=\"radius_ratio\" NumberOfComponents=\"1\"/>\n"
             "    <PDataArray type=\"Float32\" Name=\"mindihedangle\" NumberOfComponents=\"1\"/>\n";
  cells += "  </PCellData>\n";
  t.insert(t.find("  <PPoints>"), cells);
  return t;
}

void update_pvd(const std::string& path, int n_out, const std::string& timestep, const std::string& dataset) {
  std::vector<std::string> entries;
  if (n_out != 0) {
    std::ifstream in(path);
    std::string ln;
    while (std::getline(in, ln))
      if (ln.find("<DataSet") != std::string::npos) entries.push_back(ln);
  }
  entries.push_back("    <DataSet timestep=\"" + timestep + "\" group=\"\" part=\"0\" file=\"" + dataset + "\"/>");
  std::ofstream out(path, std::ios::trunc);
  out << "<VTKFile type=\"Collection\" version=\"0.1\">\n  <Collection>\n";
  for (const auto& e : entries) out << e << "\n";
  out << "  </Collection>\n</VTKFile>\n";
}

std::string lset_restart_bytes(const LsetRestart& r) {
  std::string b;
  auto I = [&](int v) { b += raw_of(&v, 1); };
  auto D = [&](double v) { b += raw_of(&v, 1); };
  std::array<double, 3> dom;
  for (int d = 0; d < 3; d++) dom[d] = r.box_r[d] - r.box_l[d];
  I(r.dim);
  for (int k = 0; k < 2; k++) {  // domain, box, then the particle box (the same)
    for (int d = 0; d < 3; d++) D(dom[d]);
    for (int d = 0; d < 3; d++) D(r.box_l[d]);
    for (int d = 0; d < 3; d++) D(r.box_r[d]);
  }
  for (int d = 0; d < 3; d++) I(d < r.dim ? 4 * r.num_pkg[d] : 1);  // resolution
  I(0);  // Lmin
  I(0);  // Lmax
  for (int d = 0; d < 3; d++) I(r.num_pkg[d]);  // ini_num_cell
  I(1);  // num_level
  D(1.e-4);  // convergence_error
  I((int)(r.sing.size() / 3));
  for (double v : r.sing) D(v);
  I((int)(r.seg.size() / 6));
  for (double v : r.seg) D(v);
  for (double v : {r.fac_max, r.fac_mid, r.fac_min, r.curv_artificial, r.total_mass, r.total_mass_surface,
                   r.total_mass_segment, r.total_volume, r.total_area, r.total_length, r.max_phi, 0.0, r.max_dl,
                   r.mid_dl, r.min_dl, r.max_curv,
                   r.min_curv})
    D(v);
  I(r.num_interface_cell);
  int total = 1;
  for (int d = 0; d < 3; d++) total *= r.num_pkg[d] + 2 * r.margin[d];
  I(total);
  D(r.dpkg[0]);  // scale
  double dl = 1.e20;
  for (int d = 0; d < r.dim; d++) dl = std::min(dl, r.dcell[d]);
  D(dl);
  for (int d = 0; d < 3; d++) I(r.num_pkg[d]);
  for (int d = 0; d < 3; d++) I(r.num_pkg[d] + 2 * r.margin[d]);
  for (int k = 0; k < 2; k++) {  // global and local package ranges (one rank)
    for (int d = 0; d < 3; d++) I(-r.margin[d]);
    for (int d = 0; d < 3; d++) I(r.num_pkg[d] + r.margin[d]);
  }
  for (int d = 0; d < 3; d++) I(r.margin[d]);
  for (int d = 0; d < 3; d++) D(r.dpkg[d]);
  for (int d = 0; d < 3; d++) D(r.dcell[d]);
  const size_t n = r.phi.size();
  std::vector<double> zero(n, 0.0);
  std::vector<int> izero(n, 0), minus(n, -1);
  const std::vector<double>* fields[6] = {&r.phi, &r.nx, &r.ny, &r.nz, &r.curv, &zero};
  for (const std::vector<double>* v : fields) b += raw_of(v->data(), n);
  b += raw_of(r.tag.data(), n);
  b += r.chr_tag.size() == n ? raw_of(r.chr_tag.data(), n) : raw_of(izero.data(), n);
  b += r.chr_idx.size() == n ? raw_of(r.chr_idx.data(), n) : raw_of(minus.data(), n);
  b += raw_of(r.scale.data(), n);
  return b;
}

namespace {
// Sequential little-endian reader over a file's bytes.
struct ByteReader {
  std::string b;
  size_t o = 0;
  template <class T>
  T get() {
    T v;
    need(sizeof(T));
    std::memcpy(&v, b.data() + o, sizeof(T));
    o += sizeof(T);
    return v;
  }
  template <class T>
  void get_n(std::vector<T>& v, size_t n) {
    need(sizeof(T) * n);
    v.resize(n);
    if (n) std::memcpy(v.data(), b.data() + o, sizeof(T) * n);
    o += sizeof(T) * n;
  }
  void need(size_t k) const {
    if (b.size() - o < k) throw Error(MRSPH_ERR_ARG, "level-set restart: file too short");
  }
};
}  // namespace

LsetRestart Load_lset_restart(const std::string& path) {
  std::ifstream in(path, std::ios::binary);
  if (!in) throw Error(MRSPH_ERR_ARG, "level-set restart: cannot open " + path);
  ByteReader rd;
  rd.b.assign(std::istreambuf_iterator<char>(in), std::istreambuf_iterator<char>());
  LsetRestart r;
  r.dim = rd.get<int>();
  if (r.dim != 2 && r.dim != 3) throw Error(MRSPH_ERR_ARG, "level-set restart: dimension must be 2 or 3");
  for (int d = 0; d < 3; d++) rd.get<double>();  // domain
  for (int d = 0; d < 3; d++) r.box_l[d] = rd.get<double>();
  for (int d = 0; d < 3; d++) r.box_r[d] = rd.get<double>();
  for (int k = 0; k < 9; k++) rd.get<double>();  // particle box: domain, left, right
  for (int k = 0; k < 8; k++) rd.get<int>();     // resolution, Lmin, Lmax, ini_num_cell
  if (rd.get<int>() != 1) throw Error(MRSPH_ERR_ARG, "level-set restart: only one level is read");
  rd.get<double>();  // convergence_error
  const int nsing = rd.get<int>();
  if (nsing < 0) throw Error(MRSPH_ERR_ARG, "level-set restart: negative singularity count");
  rd.get_n(r.sing, 3 * (size_t)nsing);
  const int nseg = rd.get<int>();
  if (nseg < 0) throw Error(MRSPH_ERR_ARG, "level-set restart: negative segment count");
  rd.get_n(r.seg, 6 * (size_t)nseg);
  double* v[] = {&r.fac_max, &r.fac_mid, &r.fac_min, &r.curv_artificial, &r.total_mass, &r.total_mass_surface,
                 &r.total_mass_segment, &r.total_volume, &r.total_area, &r.total_length, &r.max_phi, nullptr,
                 &r.max_dl, &r.mid_dl, &r.min_dl, &r.max_curv, &r.min_curv};
  for (double* p : v) {
    const double x = rd.get<double>();
    if (p) *p = x;  // maximum_psi is not kept
  }
  r.num_interface_cell = rd.get<int>();
  rd.get<int>();     // packages incl. margins
  rd.get<double>();  // scale
  rd.get<double>();  // dl
  for (int d = 0; d < 3; d++) r.num_pkg[d] = rd.get<int>();
  for (int k = 0; k < 15; k++) rd.get<int>();  // package counts incl. margins, global and local ranges
  for (int d = 0; d < 3; d++) r.margin[d] = rd.get<int>();
  for (int d = 0; d < 3; d++) r.dpkg[d] = rd.get<double>();
  for (int d = 0; d < 3; d++) r.dcell[d] = rd.get<double>();
  size_t n = 1;
  for (int d = 0; d < 3; d++) {
    if (r.num_pkg[d] < 1 || (d >= r.dim && r.num_pkg[d] != 1) || r.margin[d] < 0)
      throw Error(MRSPH_ERR_ARG, "level-set restart: bad package counts");
    n *= (size_t)r.num_pkg[d] * (d < r.dim ? 4 : 1);
  }
  std::vector<double> psi;
  std::vector<double>* dbl[] = {&r.phi, &r.nx, &r.ny, &r.nz, &r.curv, &psi};
  for (std::vector<double>* a : dbl) rd.get_n(*a, n);
  rd.get_n(r.tag, n);
  rd.get_n(r.chr_tag, n);
  rd.get_n(r.chr_idx, n);
  rd.get_n(r.scale, n);
  if (rd.o != rd.b.size()) throw Error(MRSPH_ERR_ARG, "level-set restart: trailing bytes");
  return r;
}

long long restart_num_particles(double total_mass, double total_mass_surface, double total_mass_segment,
                                int num_singularity, int num_interface_cell) {
  const long long seg = std::max((long long)(total_mass_segment - 0.5 * num_singularity), 0LL);
  long long surf = std::max((long long)(total_mass_surface - 0.5 * total_mass_segment), 0LL);
  surf = std::min(surf, (long long)num_interface_cell);
  const long long mesh = std::max((long long)(total_mass - 0.5 * total_mass_surface), 0LL);
  return mesh + surf + num_singularity + seg;
}

Case case_from_lset_restart(const LsetRestart& r, int kernel, double h_over_dx, int precision,
                            unsigned long long seed, int scale_law, const double* retarget) {
  const int dim = r.dim;
  Case c;
  c.name = "lset_restart";
  mrsph_params p = default_params(dim);
  p.kernel = kernel;
  p.precision = precision;
  p.min_dl = r.min_dl;
  p.max_dl = r.max_dl;
  p.middle_dl = r.mid_dl;
  if (retarget) {
    double dl = 1.e300;
    for (int d = 0; d < dim; d++) dl = std::min(dl, r.dcell[d]);
    p.min_dl = retarget[0] * dl;
    p.middle_dl = retarget[1] * dl;
    p.max_dl = retarget[2] * dl;
  }
  p.cell_ratio = 2.0 * h_over_dx;
  for (int d = 0; d < 3; d++) {
    p.box_l[d] = d < dim ? r.box_l[d] : 0.0;
    p.box_r[d] = d < dim ? r.box_r[d] : 0.0;
  }
  p.seed = seed;
  p.scale_law = scale_law;
  if (!cell_levels_consistent(p.box_l, p.box_r, dim, p.max_dl * p.cell_ratio, p.min_dl * p.cell_ratio))
    throw Error(MRSPH_ERR_ARG, "the restart's domain and spacing give an inconsistent cell-list level plan "
                               "(sph.cpp:144-180); choose another h_over_dx");
  LevelGrid L;
  const int m = r.margin[0];
  int in[3], pad[3], full[3];
  for (int d = 0; d < 3; d++) {
    L.box_l[d] = p.box_l[d];
    L.dpkg[d] = r.dpkg[d];
    L.num_pkg[d] = d < dim ? r.num_pkg[d] : 1;
    in[d] = r.num_pkg[d] * (d < dim ? 4 : 1);
    pad[d] = d < dim ? 4 * m : 0;
    full[d] = in[d] + 2 * pad[d];
  }
  L.margin = m;
  L.phi.resize((size_t)full[0] * full[1] * full[2]);
  for (int z = 0; z < full[2]; z++)
    for (int y = 0; y < full[1]; y++)
      for (int x = 0; x < full[0]; x++) {
        const int g[3] = {x - pad[0], y - pad[1], z - pad[2]};
        int q[3];
        double off[3];
        for (int d = 0; d < 3; d++) {
          q[d] = std::min(std::max(g[d], 0), in[d] - 1);
          off[d] = (double)(g[d] - q[d]) * (d < dim ? r.dcell[d] : 0.0);
        }
        const double near = r.phi[((size_t)q[2] * in[1] + q[1]) * in[0] + q[0]];
        L.phi[((size_t)z * full[1] + y) * full[0] + x] =
            near - std::sqrt(off[0] * off[0] + off[1] * off[1] + off[2] * off[2]);
      }
  c.levels.push_back(std::move(L));
  c.params = p;
  c.singularities = r.sing;
  c.segments = r.seg;
  c.n_particles = retarget ? particle_count(c.levels, p)
                           : restart_num_particles(r.total_mass, r.total_mass_surface, r.total_mass_segment,
                                                   (int)(r.sing.size() / 3), r.num_interface_cell);
  c.steps = 200;
  return c;
}

std::string Save_lset_restart(SPH_mesh_generation& sim, const std::string& path, int level) {
  const Case& cs = sim.Get_case();
  const mrsph_params& p = cs.params;
  const int dim = p.dim, nls = (int)cs.levels.size();
  level = ((level % nls) + nls) % nls;
  const LevelGrid& lv = cs.levels[level];
  std::array<int, 3> n{{1, 1, 1}};
  for (int d = 0; d < dim; d++) n[d] = (lv.num_pkg[d] + 2 * lv.margin) * 4;
  const int m = 4 * lv.margin;
  std::vector<std::vector<double>> curv(nls);
  std::vector<std::vector<unsigned char>> tag(nls);
  std::vector<double> nx, ny, nz;
  double max_phi = 0.0;
  for (int l = 0; l < nls; l++) {
    const size_t nl = cs.levels[l].phi.size();
    curv[l].assign(nl, 0.0);
    tag[l].assign(nl, 0);
    if (l == level) {
      nx.assign(nl, 0.0);
      ny.assign(nl, 0.0);
      nz.assign(nl, 0.0);
    }
    int rc = mrsph_get_levelset(sim.handle(), l, l == level ? nx.data() : nullptr, l == level ? ny.data() : nullptr,
                                l == level ? nz.data() : nullptr, curv[l].data(), tag[l].data(), &max_phi);
    if (rc) throw Error(rc, "mrsph_get_levelset");
  }
  mrsph_volume_mass_stats vm{};
  int rc = mrsph_volume_mass(sim.handle(), level, &vm, nullptr, nullptr);
  if (rc) throw Error(rc, "mrsph_volume_mass");
  const bool has_chr = !cs.singularities.empty() || !cs.segments.empty();
  std::vector<int> chr;
  if (has_chr) {
    chr.assign(lv.phi.size(), 0);
    rc = mrsph_get_characteristics(sim.handle(), level, chr.data());
    if (rc) throw Error(rc, "mrsph_get_characteristics");
  }
  double dl0 = 1.e20, dl = 1.e20;
  for (int d = 0; d < dim; d++) {
    dl0 = std::min(dl0, cs.levels[0].dpkg[d] / 4.0);
    dl = std::min(dl, lv.dpkg[d] / 4.0);
  }
  double cmax = 0.0, cmin = 1.e20;
  bool any = false;
  for (int l = 0; l < nls; l++)
    for (size_t a = 0; a < curv[l].size(); a++)
      if (tag[l][a] == 1) {
        const double v = std::fabs(curv[l][a]);
        cmax = any ? std::max(cmax, v) : v;
        cmin = any ? std::min(cmin, v) : v;
        any = true;
      }
  const double mid = p.middle_dl > 0 ? p.middle_dl : 5.0 * dl0;
  LsetRestart r;
  r.dim = dim;
  r.sing = cs.singularities;
  r.seg = cs.segments;
  for (int d = 0; d < 3; d++) {
    r.box_l[d] = d < dim ? p.box_l[d] : 0.0;
    r.box_r[d] = d < dim ? p.box_r[d] : 0.0;
    r.num_pkg[d] = d < dim ? lv.num_pkg[d] : 1;
    r.margin[d] = d < dim ? lv.margin : 0;
    r.dpkg[d] = lv.dpkg[d];
    r.dcell[d] = d < dim ? lv.dpkg[d] / 4.0 : lv.dpkg[d];
  }
  r.fac_max = p.max_dl / dl0;
  r.fac_mid = mid / dl0;
  r.fac_min = p.min_dl / dl0;
  r.curv_artificial = std::min(1.0, cmax);
  r.total_mass = vm.total_mass;
  r.total_mass_surface = vm.total_mass_surface;
  r.total_volume = vm.total_volume;
  r.total_area = vm.total_area;
  r.total_mass_segment = vm.total_mass_segment;
  r.total_length = vm.total_length;
  r.max_phi = max_phi;
  r.max_dl = p.max_dl;
  r.mid_dl = mid;
  r.min_dl = p.min_dl;
  r.max_curv = cmax;
  r.min_curv = cmin;
  r.num_interface_cell = (int)vm.num_interface_cell;
  const int z0 = dim == 3 ? m : 0, z1 = dim == 3 ? n[2] - m : 1;
  for (int z = z0; z < z1; z++)
    for (int y = m; y < n[1] - m; y++)
      for (int x = m; x < n[0] - m; x++) {
        const size_t a = ((size_t)z * n[1] + y) * n[0] + x;
        const double phi = lv.phi[a];
        r.phi.push_back(phi);
        r.nx.push_back(nx[a]);
        r.ny.push_back(ny[a]);
        r.nz.push_back(nz[a]);
        r.curv.push_back(curv[level][a]);
        r.tag.push_back(tag[level][a]);
        if (has_chr) {  // k + 1: segment k (SEGMENT_CELL 2); -(k + 1): point k (SINGULARITY_CELL 1)
          const int e = chr[a];
          r.chr_tag.push_back(e > 0 ? 2 : (e < 0 ? 1 : 0));
          r.chr_idx.push_back(e > 0 ? e - 1 : (e < 0 ? -e - 1 : -1));
        }
        double sc = 0.0;  // the scale Calculate_volume_mass leaves in the counted cells
        if (phi > 0 || std::fabs(phi) < dl) {
          double lo = p.min_dl;
          if (p.scale_law == 1) {
            double q = (cmax - std::fabs(curv[level][a])) / (cmax - cmin + 1e-20);
            q = std::min(std::max(q, 0.0), 1.0);
            lo = p.min_dl + q * q * (mid - p.min_dl);
          }
          const double s = lo + std::tanh(2.5 * std::fabs(phi) / max_phi) / std::tanh(2.5) * (p.max_dl - lo);
          sc = (phi > 0 || std::fabs(phi) < dl0) ? s : p.min_dl;
        }
        r.scale.push_back(sc);
      }
  const size_t slash = path.rfind('/');
  if (slash != std::string::npos) make_dir(path.substr(0, slash));
  std::ofstream o(path, std::ios::binary | std::ios::trunc);
  const std::string b = lset_restart_bytes(r);
  o.write(b.data(), (std::streamsize)b.size());
  if (!o) throw Error(MRSPH_ERR_ARG, "cannot write " + path);
  return path;
}

std::string Mesh_binary_writer::Output_mesh(int n_out, SPH_mesh_generation& sim, long long run_time) {
  make_dir(outdir_);
  if (sim.Get_case().params.dim == 3) {
    std::vector<int> tets;
    sim.Reconstruct_tets(tets);
    std::vector<int> type, nn;
    std::vector<double> h, norm;
    sim.Particle_fields(type, h, norm, nn);
    const std::vector<double> xyz = sim.Positions();
    ParticleFields f;
    f.n = sim.num_particles();
    f.xyz = xyz.data();
    f.type = type.data();
    f.h = h.data();
    f.nn = nn.data();
    f.norm = norm.data();
    const std::string piece = "mesh_tets_rank_0_step_" + std::to_string(n_out) + ".vtu";
    const std::string pvtu = "mesh_tets_step_" + std::to_string(n_out) + ".pvtu";
    {
      std::ofstream o(outdir_ + "/" + piece, std::ios::binary | std::ios::trunc);
      const std::string b = tet_mesh_vtu(f, (long long)(tets.size() / 4), tets.data());
      o.write(b.data(), (std::streamsize)b.size());
    }
    {
      std::ofstream o(outdir_ + "/" + pvtu, std::ios::trunc);
      o << mesh_pvtu(piece, true);
    }
    const long long ts = run_time < 0 ? sim.Stats().step : run_time;
    update_pvd(outdir_ + "/mesh_tets.pvd", n_out, std::to_string(ts), "./" + pvtu);
    return outdir_ + "/" + piece;
  }
  long long ntri = 0;
  int rc = mrsph_triangulate(sim.handle(), nullptr, 0, &ntri, nullptr);
  if (rc) throw Error(rc, "mrsph_triangulate");
  std::vector<int> tris(3 * (ntri > 0 ? ntri : 1));
  mrsph_tri_quality q{};
  rc = mrsph_triangulate(sim.handle(), tris.data(), ntri, &ntri, &q);
  if (rc) throw Error(rc, "mrsph_triangulate");
  std::vector<int> type, nn;
  std::vector<double> h, norm;
  sim.Particle_fields(type, h, norm, nn);
  const std::vector<double> xyz = sim.Positions();
  ParticleFields f;
  f.n = sim.num_particles();
  f.xyz = xyz.data();
  f.type = type.data();
  f.h = h.data();
  f.nn = nn.data();
  f.norm = norm.data();
  const std::string piece = "mesh_tris_rank_0_step_" + std::to_string(n_out) + ".vtu";
  const std::string pvtu = "mesh_tris_step_" + std::to_string(n_out) + ".pvtu";
  {
    std::ofstream o(outdir_ + "/" + piece, std::ios::binary | std::ios::trunc);
    const std::string b = mesh_vtu(f, ntri, tris.data());
    o.write(b.data(), (std::streamsize)b.size());
  }
  {
    std::ofstream o(outdir_ + "/" + pvtu, std::ios::trunc);
    o << mesh_pvtu(piece, false);
  }
  const long long ts = run_time < 0 ? sim.Stats().step : run_time;
  update_pvd(outdir_ + "/mesh_tris.pvd", n_out, std::to_string(ts), "./" + pvtu);
  return outdir_ + "/" + piece;
}

std::string Particle_binary_writer::Output_particle(int n_out, SPH_mesh_generation& sim, long long run_time) {
  make_dir(outdir_);
  std::vector<int> type, nn;
  std::vector<double> h, norm;
  sim.Particle_fields(type, h, norm, nn);
  const std::vector<double> xyz = sim.Positions();
  ParticleFields f;
  f.n = sim.num_particles();
  f.xyz = xyz.data();
  f.type = type.data();
  f.h = h.data();
  f.nn = nn.data();
  f.norm = norm.data();
  const std::string piece = "particle_rank_0_step_" + std::to_string(n_out) + ".vtu";
  const std::string pvtu = "particle_step_" + std::to_string(n_out) + ".pvtu";
  {
    std::ofstream o(outdir_ + "/" + piece, std::ios::binary | std::ios::trunc);
    const std::string b = particle_vtu(f);
    o.write(b.data(), (std::streamsize)b.size());
  }
  {
    std::ofstream o(outdir_ + "/" + pvtu, std::ios::trunc);
    o << particle_pvtu(piece);
  }
  const long long t = run_time < 0 ? sim.Stats().step : run_time;
  update_pvd(outdir_ + "/particle.pvd", n_out, std::to_string(t), "./" + pvtu);
  return outdir_ + "/" + piece;
}

std::string repr_double(double v) {
  if (v == 0.0) return std::signbit(v) ? "-0.0" : "0.0";
  char buf[64];
  auto r = std::to_chars(buf, buf + sizeof(buf), v, std::chars_format::scientific);
  std::string sci(buf, r.ptr);  // [-]d[.ddd]e(+|-)XX
  const size_t e = sci.find('e');
  const int exp10 = std::atoi(sci.c_str() + e + 1);
  std::string mant = sci.substr(0, e), sign;
  if (mant[0] == '-') {
    sign = "-";
    mant = mant.substr(1);
  }
  std::string digits;
  for (char c : mant)
    if (c != '.') digits += c;
  if (exp10 >= -4 && exp10 < 16) {  // fixed notation, as repr does
    std::string out;
    const int point = exp10 + 1;    // digits before the decimal point
    if (point <= 0) {
      out = "0." + std::string(-point, '0') + digits;
    } else if (point >= (int)digits.size()) {
      out = digits + std::string(point - digits.size(), '0') + ".0";
    } else {
      out = digits.substr(0, point) + "." + digits.substr(point);
    }
    return sign + out;
  }
  std::string m = digits.substr(0, 1);
  if (digits.size() > 1) m += "." + digits.substr(1);
  char eb[16];
  std::snprintf(eb, sizeof(eb), "e%c%02d", exp10 < 0 ? '-' : '+', exp10 < 0 ? -exp10 : exp10);
  return sign + m + eb;
}

std::string vti_bytes(const std::array<int, 3>& ncell, const std::array<double, 3>& origin,
                      const std::array<double, 3>& spacing, const std::vector<ImageField>& point_data,
                      const std::vector<ImageField>& cell_data) {
  std::string ext;
  for (int d = 0; d < 3; d++) ext += (d ? " 0 " : "0 ") + std::to_string(ncell[d]);
  std::string head = "<VTKFile type=\"ImageData\" version=\"0.1\" byte_order=\"LittleEndian\">\n";
  head += " <ImageData WholeExtent=\"" + ext + "\" Origin=\"" + repr_double(origin[0]) + " " +
          repr_double(origin[1]) + " " + repr_double(origin[2]) + "\" Spacing=\"" + repr_double(spacing[0]) + " " +
          repr_double(spacing[1]) + " " + repr_double(spacing[2]) + "\">\n";
  head += "  <Piece Extent=\"" + ext + "\">\n";
  std::string blobs;
  unsigned long long offset = 0;
  auto block = [&](const char* tag, const std::vector<ImageField>& fs) {
    head += std::string("    <") + tag + " Vectors=\"vector\">\n";
    for (const auto& f : fs) {
      head += "      <DataArray type=\"" + f.type + "\" Name=\"" + f.name +
              "\" NumberOfComponents=\"1\" format=\"appended\" offset=\"" + std::to_string(offset) + "\"/>\n";
      const uint32_t nb = (uint32_t)f.raw.size();
      blobs += raw_of(&nb, 1) + f.raw;
      offset += 4 + f.raw.size();
    }
    head += std::string("    </") + tag + ">\n";
  };
  block("PointData", point_data);
  block("CellData", cell_data);
  head += "  </Piece>\n </ImageData>\n <AppendedData encoding=\"raw\">\n _";
  return head + blobs + "\n </AppendedData>\n</VTKFile>\n";
}

namespace {

// mean of the 2^D cells around each corner of the interior cells; cells are
// (nz, ny, nx) incl. m margin cells per side (nz = 1 in 2D)
std::vector<float> corner_average(const std::vector<double>& c, const std::array<int, 3>& n, int m, int dim) {
  std::vector<float> out;
  if (dim == 2) {
    const int ny = n[1] - 2 * m + 1, nx = n[0] - 2 * m + 1;
    out.resize((size_t)ny * nx);
    for (int y = 0; y < ny; y++)
      for (int x = 0; x < nx; x++) {
        auto C = [&](int dy, int dx) { return c[(size_t)(y + m - 1 + dy) * n[0] + (x + m - 1 + dx)]; };
        out[(size_t)y * nx + x] = (float)(0.25 * (C(0, 0) + C(1, 0) + C(0, 1) + C(1, 1)));
      }
    return out;
  }
  const int nz = n[2] - 2 * m + 1, ny = n[1] - 2 * m + 1, nx = n[0] - 2 * m + 1;
  out.resize((size_t)nz * ny * nx);
  for (int z = 0; z < nz; z++)
    for (int y = 0; y < ny; y++)
      for (int x = 0; x < nx; x++) {
        double acc = 0.0;
        for (int dz = 0; dz < 2; dz++)
          for (int dy = 0; dy < 2; dy++)
            for (int dx = 0; dx < 2; dx++)
              acc += c[((size_t)(z + m - 1 + dz) * n[1] + (y + m - 1 + dy)) * n[0] + (x + m - 1 + dx)];
        out[((size_t)z * ny + y) * nx + x] = (float)(0.125 * acc);
      }
  return out;
}

template <class T, class U>
std::string interior_raw(const std::vector<U>& c, const std::array<int, 3>& n, int m, int dim) {
  std::vector<T> v;
  const int z0 = dim == 3 ? m : 0, z1 = dim == 3 ? n[2] - m : 1;
  for (int z = z0; z < z1; z++)
    for (int y = m; y < n[1] - m; y++)
      for (int x = m; x < n[0] - m; x++) v.push_back((T)c[((size_t)z * n[1] + y) * n[0] + x]);
  return raw_of(v.data(), v.size());
}

}  // namespace

std::string Level_set_binary_writer::Output_lset(int n_out, SPH_mesh_generation& sim, int level,
                                                 long long run_time) {
  make_dir(outdir_);
  const Case& cs = sim.Get_case();
  const mrsph_params& p = cs.params;
  const int dim = p.dim, nls = (int)cs.levels.size();
  if (level < 0 || level >= nls) throw Error(MRSPH_ERR_ARG, "no such level-set level");
  const LevelGrid& lv = cs.levels[level];
  std::array<int, 3> n{{1, 1, 1}};
  for (int d = 0; d < dim; d++) n[d] = (lv.num_pkg[d] + 2 * lv.margin) * 4;
  const size_t ntot = (size_t)n[0] * n[1] * n[2];
  const int m = 4 * lv.margin;
  // curvature and tags of every level (the curvature law's range spans all levels)
  std::vector<std::vector<double>> curv(nls);
  std::vector<std::vector<unsigned char>> tag(nls);
  double max_phi = 0.0;
  for (int l = 0; l < nls; l++) {
    const size_t nl = cs.levels[l].phi.size();
    curv[l].assign(nl, 0.0);
    tag[l].assign(nl, 0);
    int rc = mrsph_get_levelset(sim.handle(), l, nullptr, nullptr, nullptr, curv[l].data(), tag[l].data(), &max_phi);
    if (rc) throw Error(rc, "mrsph_get_levelset");
  }
  // Levelset::Get_scale (level_set.cpp:311-351) on every cell of the level
  double dl0 = 1.e20;
  for (int d = 0; d < dim; d++) dl0 = std::min(dl0, cs.levels[0].dpkg[d] / 4.0);
  double cmax = 0.0, cmin = 1.e20;
  bool any_cut = false;
  for (int l = 0; l < nls; l++)
    for (size_t a = 0; a < curv[l].size(); a++)
      if (tag[l][a] == 1) {
        const double v = std::fabs(curv[l][a]);
        if (!any_cut) {
          cmax = cmin = v;
          any_cut = true;
        } else {
          cmax = std::max(cmax, v);
          cmin = std::min(cmin, v);
        }
      }
  const double mid = p.middle_dl > 0 ? p.middle_dl : 5.0 * dl0;
  std::vector<double> scale(ntot);
  for (size_t a = 0; a < ntot; a++) {
    const double phi = lv.phi[a];
    double lo = p.min_dl;
    if (p.scale_law == 1) {
      double q = (cmax - std::fabs(curv[level][a])) / (cmax - cmin + 1e-20);
      q = std::min(std::max(q, 0.0), 1.0);
      lo = p.min_dl + q * q * (mid - p.min_dl);
    }
    const double s = lo + std::tanh(2.5 * std::fabs(phi) / max_phi) / std::tanh(2.5) * (p.max_dl - lo);
    scale[a] = (phi > 0 || std::fabs(phi) < dl0) ? s : p.min_dl;
  }
  std::vector<double> vol(ntot), area(ntot);
  mrsph_volume_mass_stats vm{};
  int rc = mrsph_volume_mass(sim.handle(), level, &vm, vol.data(), area.data());
  if (rc) throw Error(rc, "mrsph_volume_mass");
  auto fl = [](const std::vector<float>& v) { return raw_of(v.data(), v.size()); };
  std::vector<ImageField> pd = {{"phi", "Float32", fl(corner_average(lv.phi, n, m, dim))},
                                {"curv", "Float32", fl(corner_average(curv[level], n, m, dim))},
                                {"scale", "Float32", fl(corner_average(scale, n, m, dim))}};
  const std::string tags = interior_raw<int>(tag[level], n, m, dim);
  // tag_characteristic: 1 SINGULARITY_CELL, 2 SEGMENT_CELL (glbparam.h:48-51)
  std::vector<int> ctag(ntot, 0);
  if (!cs.singularities.empty() || !cs.segments.empty()) {
    rc = mrsph_get_characteristics(sim.handle(), level, ctag.data());
    if (rc) throw Error(rc, "mrsph_get_characteristics");
    for (int& e : ctag) e = e > 0 ? 2 : (e < 0 ? 1 : 0);
  }
  std::vector<ImageField> cd = {{"interface", "Int32", tags},
                                {"char", "Int32", interior_raw<int>(ctag, n, m, dim)},
                                {"vol", "Float32", interior_raw<float>(vol, n, m, dim)},
                                {"area", "Float32", interior_raw<float>(area, n, m, dim)}};
  std::array<int, 3> nc{{0, 0, 0}};
  std::array<double, 3> origin{{0, 0, 0}}, spacing{{1, 1, 1}};
  for (int d = 0; d < dim; d++) {
    nc[d] = 4 * lv.num_pkg[d];
    origin[d] = lv.box_l[d];
    spacing[d] = lv.dpkg[d] / 4.0;
  }
  const std::string piece = "mesh_lset_rank_0_step_" + std::to_string(n_out) + ".vti";
  {
    std::ofstream o(outdir_ + "/" + piece, std::ios::binary | std::ios::trunc);
    const std::string b = vti_bytes(nc, origin, spacing, pd, cd);
    o.write(b.data(), (std::streamsize)b.size());
  }
  const std::string pvti = "mesh_lset_step_" + std::to_string(n_out) + ".pvti";
  {
    std::string ext;
    for (int d = 0; d < 3; d++) ext += (d ? " 0 " : "0 ") + std::to_string(nc[d]);
    std::ofstream o(outdir_ + "/" + pvti, std::ios::trunc);
    o << "<VTKFile type=\"PImageData\" version=\"0.1\" byte_order=\"LittleEndian\">\n"
      << " <PImageData WholeExtent=\"" << ext << "\" GhostLevel=\"0\" Origin=\"" << repr_double(origin[0]) << " "
      << repr_double(origin[1]) << " " << repr_double(origin[2]) << "\" Spacing=\"" << repr_double(spacing[0]) << " "
      << repr_double(spacing[1]) << " " << repr_double(spacing[2]) << "\">\n  <PPointData>\n";
    for (const auto& f : pd)
      o << "    <PDataArray type=\"" << f.type << "\" Name=\"" << f.name << "\" NumberOfComponents=\"1\"/>\n";
    o << "  </PPointData>\n  <PCellData>\n";
    for (const auto& f : cd)
      o << "    <PDataArray type=\"" << f.type << "\" Name=\"" << f.name << "\" NumberOfComponents=\"1\"/>\n";
    o << "  </PCellData>\n  <Piece Extent=\"" << ext << "\" Source=\"" << piece << "\"/>\n </PImageData>\n</VTKFile>\n";
  }
  const long long t = run_time < 0 ? sim.Stats().step : run_time;
  update_pvd(outdir_ + "/mesh_lset.pvd", n_out, std::to_string(t), "./" + pvti);
  return outdir_ + "/" + piece;
}

void write_pst(const std::string& path, const std::vector<double>& xyz) {
  std::ofstream f(path, std::ios::binary | std::ios::trunc);
  if (!f) throw Error(MRSPH_ERR_ARG, "cannot write " + path);
  const int32_t n = (int32_t)(xyz.size() / 3);
  f.write(reinterpret_cast<const char*>(&n), sizeof(n));
  f.write(reinterpret_cast<const char*>(xyz.data()), (std::streamsize)(sizeof(double) * xyz.size()));
}

std::vector<double> read_pst(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw Error(MRSPH_ERR_ARG, "cannot read " + path);
  int32_t n = 0;
  f.read(reinterpret_cast<char*>(&n), sizeof(n));
  if (!f || n < 0) throw Error(MRSPH_ERR_ARG, path + ": bad particle count");
  std::vector<double> xyz((size_t)3 * n);
  f.read(reinterpret_cast<char*>(xyz.data()), (std::streamsize)(sizeof(double) * xyz.size()));
  if (f.gcount() != (std::streamsize)(sizeof(double) * xyz.size()))
    throw Error(MRSPH_ERR_ARG, path + ": truncated particle file");
  return xyz;
}

}  // namespace mrsph_host

// C entry for the writer tests: the particle VTU bytes of host arrays.
extern "C" long long mrsph_host_particle_vtu(const char* path, long long n, const double* xyz, const int* type,
                                             const double* h, const int* nn, const double* norm) {
  mrsph_host::ParticleFields f;
  f.n = n;
  f.xyz = xyz;
  f.type = type;
  f.h = h;
  f.nn = nn;
  f.norm = norm;
  const std::string b = mrsph_host::particle_vtu(f);
  std::ofstream o(path, std::ios::binary | std::ios::trunc);
  o.write(b.data(), (std::streamsize)b.size());
  return o ? (long long)b.size() : -1;
}

// C entry for the writer tests: the level-set VTI bytes of host arrays
// (point fields at (n0+1) x (n1+1) x (n2+1) corners, cell fields per cell;
// 2D: n2 = 0, one layer).
template <class T>
static std::string host_raw(const T* p, size_t count) {
  std::string r(sizeof(T) * count, '\0');
  if (count) std::memcpy(&r[0], p, r.size());
  return r;
}

extern "C" long long mrsph_host_lset_vti(const char* path, const int* ncell, const double* origin,
                                         const double* spacing, const float* phi, const float* curv,
                                         const float* scale, const int* tag, const float* vol, const float* area,
                                         const int* chr) {
  std::array<int, 3> nc{{ncell[0], ncell[1], ncell[2]}};
  size_t np = 1, ncl = 1;
  for (int d = 0; d < 3; d++) {
    np *= (size_t)(nc[d] + 1);
    ncl *= (size_t)(nc[d] > 0 ? nc[d] : 1);
  }
  std::vector<int> zero(ncl, 0);
  std::vector<mrsph_host::ImageField> pd = {{"phi", "Float32", host_raw(phi, np)},
                                            {"curv", "Float32", host_raw(curv, np)},
                                            {"scale", "Float32", host_raw(scale, np)}};
  std::vector<mrsph_host::ImageField> cd = {{"interface", "Int32", host_raw(tag, ncl)},
                                            {"char", "Int32", host_raw(chr ? chr : zero.data(), ncl)},
                                            {"vol", "Float32", host_raw(vol, ncl)},
                                            {"area", "Float32", host_raw(area, ncl)}};
  const std::string b = mrsph_host::vti_bytes(nc, {{origin[0], origin[1], origin[2]}},
                                              {{spacing[0], spacing[1], spacing[2]}}, pd, cd);
  std::ofstream o(path, std::ios::binary | std::ios::trunc);
  o.write(b.data(), (std::streamsize)b.size());
  return o ? (long long)b.size() : -1;
}

// C entry for the writer tests: the tet-mesh VTU bytes of host arrays.
extern "C" long long mrsph_host_tet_vtu(const char* path, long long n, const double* xyz, const int* type,
                                        const double* h, const int* nn, const double* norm, long long ntet,
                                        const int* tets) {
  mrsph_host::ParticleFields f;
  f.n = n;
  f.xyz = xyz;
  f.type = type;
  f.h = h;
  f.nn = nn;
  f.norm = norm;
  const std::string b = mrsph_host::tet_mesh_vtu(f, ntet, tets);
  std::ofstream o(path, std::ios::binary | std::ios::trunc);
  o.write(b.data(), (std::streamsize)b.size());
  return o ? (long long)b.size() : -1;
}

// C entry for the writer tests: the triangle-mesh VTU bytes of host arrays.
extern "C" long long mrsph_host_mesh_vtu(const char* path, long long n, const double* xyz, const int* type,
                                         const double* h, const int* nn, const double* norm, long long ntri,
                                         const int* tris) {
  mrsph_host::ParticleFields f;
  f.n = n;
  f.xyz = xyz;
  f.type = type;
  f.h = h;
  f.nn = nn;
  f.norm = norm;
  const std::string b = mrsph_host::mesh_vtu(f, ntri, tris);
  std::ofstream o(path, std::ios::binary | std::ios::trunc);
  o.write(b.data(), (std::streamsize)b.size());
  return o ? (long long)b.size() : -1;
}

// C entry for the writer tests: the particle (mesh = 0), triangle-mesh
// (mesh = 1) or tet-mesh (mesh = 2) PVTU text for a piece name; returns its
// length (written when it fits).
extern "C" long long mrsph_host_pvtu(int mesh, const char* piece, char* buf, long long len) {
  const std::string t = mesh ? mrsph_host::mesh_pvtu(piece, mesh == 2) : mrsph_host::particle_pvtu(piece);
  if (buf && len > (long long)t.size()) std::memcpy(buf, t.c_str(), t.size() + 1);
  return (long long)t.size();
}

// C entry for the writer tests: level-set restart bytes of host arrays
// (header values in the order of LsetRestart: box_l[3], box_r[3], dpkg[3],
// dcell[3], fac_max, fac_mid, fac_min, curv_artificial, total_mass,
// total_mass_surface, total_volume, total_area, max_phi, max_dl, mid_dl,
// min_dl, max_curv, min_curv, total_mass_segment, total_length; ints: dim,
// num_pkg[3], margin[3],
// num_interface_cell); nsing points and nseg segments; chr_tag / chr_idx
// may be NULL (NORMAL / -1).
extern "C" long long mrsph_host_lset_restart(const char* path, const double* hd, const int* hi, long long n,
                                             const double* phi, const double* nx, const double* ny,
                                             const double* nz, const double* curv, const int* tag,
                                             const double* scale, int nsing, const double* sing, int nseg,
                                             const double* seg, const int* chr_tag, const int* chr_idx) {
  mrsph_host::LsetRestart r;
  if (nsing > 0) r.sing.assign(sing, sing + 3 * (size_t)nsing);
  if (nseg > 0) r.seg.assign(seg, seg + 6 * (size_t)nseg);
  if (chr_tag) r.chr_tag.assign(chr_tag, chr_tag + n);
  if (chr_idx) r.chr_idx.assign(chr_idx, chr_idx + n);
  for (int d = 0; d < 3; d++) {
    r.box_l[d] = hd[d];
    r.box_r[d] = hd[3 + d];
    r.dpkg[d] = hd[6 + d];
    r.dcell[d] = hd[9 + d];
    r.num_pkg[d] = hi[1 + d];
    r.margin[d] = hi[4 + d];
  }
  double* v[] = {&r.fac_max, &r.fac_mid, &r.fac_min, &r.curv_artificial, &r.total_mass, &r.total_mass_surface,
                 &r.total_volume, &r.total_area, &r.max_phi, &r.max_dl, &r.mid_dl, &r.min_dl, &r.max_curv,
                 &r.min_curv, &r.total_mass_segment, &r.total_length};
  for (int k = 0; k < 16; k++) *v[k] = hd[12 + k];
  r.dim = hi[0];
  r.num_interface_cell = hi[7];
  r.phi.assign(phi, phi + n);
  r.nx.assign(nx, nx + n);
  r.ny.assign(ny, ny + n);
  r.nz.assign(nz, nz + n);
  r.curv.assign(curv, curv + n);
  r.tag.assign(tag, tag + n);
  r.scale.assign(scale, scale + n);
  const std::string b = mrsph_host::lset_restart_bytes(r);
  std::ofstream o(path, std::ios::binary | std::ios::trunc);
  o.write(b.data(), (std::streamsize)b.size());
  return o ? (long long)b.size() : -1;
}

// C entry for the loader tests: the case a level-set restart gives
// (case_from_lset_restart), its phi incl. margins copied to phi (cap
// values at most; retarget: the reference's re-targeting factors); prm
// receives min_dl, max_dl, middle_dl, cell_ratio,
// box_l[3], box_r[3]; cnt receives the particle count, the number of phi
// values, the singularity and segment counts.  Returns 0, or -1 with the
// message in err.
extern "C" int mrsph_host_lset_case(const char* path, int kernel, double h_over_dx, int precision, int scale_law,
                                    double* phi, long long cap, double* prm, long long* cnt, char* err,
                                    long long err_len, int retarget) {
  try {
    const mrsph_host::Case c =
        mrsph_host::case_from_lset_restart(mrsph_host::Load_lset_restart(path), kernel, h_over_dx, precision, 0,
                                           scale_law, retarget ? mrsph_host::kRetargetFactors : nullptr);
    const std::vector<double>& f = c.levels[0].phi;
    if ((long long)f.size() <= cap) std::memcpy(phi, f.data(), f.size() * sizeof(double));
    const double v[] = {c.params.min_dl, c.params.max_dl, c.params.middle_dl, c.params.cell_ratio,
                        c.params.box_l[0], c.params.box_l[1], c.params.box_l[2],
                        c.params.box_r[0], c.params.box_r[1], c.params.box_r[2]};
    std::memcpy(prm, v, sizeof(v));
    cnt[0] = c.n_particles;
    cnt[1] = (long long)f.size();
    cnt[2] = (long long)(c.singularities.size() / 3);
    cnt[3] = (long long)(c.segments.size() / 6);
    return 0;
  } catch (const std::exception& e) {
    if (err && err_len > 0) std::snprintf(err, (size_t)err_len, "%s", e.what());
    return -1;
  }
}
