// mrsph_relax_main.cpp — command-line driver of the C++ host layer, the
// counterpart of the reference's main (src/main.cpp) + Solver for the
// relaxation path: build a workload, seed, relax, write particle restarts.
//
//   mrsph_relax --case disc_hole_2d|torus_3d|box_2d|box_3d [--precision fp32|fp64] [--steps N]
//               [--n N] [--output-every K] [--out DIR] [--count-only] [--cut-cell-count] [--vtu] [--lset]
//               [--lset-restart] [--cvp K] [--cvp-iter M] [--mesh]
//   mrsph_relax --load-lset-restart PATH [--retarget] [--kernel NAME] [--h-over-dx X] [...]
//
// Prints one line of JSON (workload, particles, steps, device milliseconds,
// particle-steps/s, final time step).  --count-only prints the particle count
// of the workload without touching a GPU; --cut-cell-count seeds the count of
// the reference's cut-cell volume pass on the finest level (Get_num_particles)
// instead of the workload's; --vtu also writes the particle VTU series
// (outdata/particle_*.vtu, .pvtu, particle.pvd) at every output; --lset
// writes the level-set image of the finest level (outdata/mesh_lset_*) before
// seeding; --lset-restart writes the level-set restart of the finest level
// (rstfile/levelset.rst, Save_restart_file's level-set part) before seeding.
// box_2d / box_3d are boxes whose corners (and, in 3D, edges) are the
// geometry's singularity points and segments.  --cvp K partitions the
// relaxed particles into K cells (Voronoi::Partitioning, M iterations at
// most, default 4000), the initial VPs at particles 0, n/K, 2n/K, ...; the
// JSON line then carries the result and the final VPs.  --load-lset-restart
// is the reference's restart run (Load_rst_case): the workload is the level
// set of a rstfile/levelset.rst (one level, its characteristic points and
// segments), seeded with Get_num_particles over the file's totals
// (--retarget: the run that re-targets the spacing to 2, 5 and 16 level-set
// cells, _READ_TARGET_FIELD_; seed with --cut-cell-count for the reference's
// count of the recomputed totals); --kernel
// (hyperbolic, cubic, wendland, gaussian, quintic; default wendland) and
// --h-over-dx (default 1.3) set the smoothing kernel and h / dx.  --mesh
// writes the mesh of the relaxed particles (Mesh_binary_writer: triangles in
// 2D, tets in 3D, outdata/mesh_*) and, in 3D, adds the tet count and
// quality to the JSON line.  Exit status 2 on an engine or file error.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "sph_mesh_generation.hpp"

using namespace mrsph_host;

int main(int argc, char** argv) {
  std::string wl = "disc_hole_2d", out, prec, rst, kern = "wendland";
  double hdx = 1.3;
  int steps = -1, every = 0, cvp_k = 0, cvp_iter = 4000;
  long long n = -1;
  bool count_only = false, cut_cell = false, vtu = false, lset = false, lset_rst = false, mesh = false;
  bool retarget = false;
  for (int a = 1; a < argc; a++) {
    const std::string s = argv[a];
    auto val = [&]() -> std::string {
      if (a + 1 >= argc) {
        std::fprintf(stderr, "missing value for %s\n", s.c_str());
        std::exit(1);
      }
      return argv[++a];
    };
    if (s == "--case") wl = val();
    else if (s == "--precision") prec = val();
    else if (s == "--steps") steps = std::atoi(val().c_str());
    else if (s == "--n") n = std::atoll(val().c_str());
    else if (s == "--output-every") every = std::atoi(val().c_str());
    else if (s == "--out") out = val();
    else if (s == "--count-only") count_only = true;
    else if (s == "--cut-cell-count") cut_cell = true;
    else if (s == "--vtu") vtu = true;
    else if (s == "--lset") lset = true;
    else if (s == "--lset-restart") lset_rst = true;
    else if (s == "--cvp") cvp_k = std::atoi(val().c_str());
    else if (s == "--cvp-iter") cvp_iter = std::atoi(val().c_str());
    else if (s == "--load-lset-restart") rst = val();
    else if (s == "--mesh") mesh = true;
    else if (s == "--retarget") retarget = true;
    else if (s == "--kernel") kern = val();
    else if (s == "--h-over-dx") hdx = std::atof(val().c_str());
    else if (s == "--help" || s == "-h") {
      std::printf("usage: mrsph_relax --case disc_hole_2d|torus_3d|box_2d|box_3d [--precision fp32|fp64] [--steps N] [--n N]\n"
                  "                   [--output-every K] [--out DIR] [--count-only] [--cut-cell-count] [--vtu] [--lset]\n"
                  "                   [--lset-restart] [--cvp K] [--cvp-iter M] [--mesh]\n"
                  "       mrsph_relax --load-lset-restart PATH [--retarget] [--kernel NAME] [--h-over-dx X] [...]\n");
      return 0;
    } else {
      std::fprintf(stderr, "unknown argument %s\n", s.c_str());
      return 1;
    }
  }
  try {
    Case c;
    if (!rst.empty()) {
      static const char* names[] = {"hyperbolic", "cubic", "wendland", "gaussian", "quintic"};
      int k = -1;
      for (int q = 0; q < 5; q++)
        if (kern == names[q]) k = q;
      if (k < 0) {
        std::fprintf(stderr, "unknown kernel %s\n", kern.c_str());
        return 1;
      }
      c = case_from_lset_restart(Load_lset_restart(rst), k, hdx,
                                 prec == "fp64" ? MRSPH_FP64_PLAIN : MRSPH_FP32_SPLIT, 0, 0,
                                 retarget ? kRetargetFactors : nullptr);
    } else if (wl == "disc_hole_2d") c = disc_hole_2d(0.02, 64, MRSPH_KERNEL_WENDLAND, 1.3,
                                               prec == "fp32" ? MRSPH_FP32_SPLIT : MRSPH_FP64_PLAIN);
    else if (wl == "torus_3d") c = torus_3d(0.005, 0.02, MRSPH_KERNEL_WENDLAND, 1.3,
                                           prec == "fp64" ? MRSPH_FP64_PLAIN : MRSPH_FP32_SPLIT);
    else if (wl == "box_3d" || wl == "box_2d")
      c = box_with_corners(wl == "box_3d" ? 3 : 2, wl == "box_3d" ? 0.04 : 0.02, wl == "box_3d" ? 32 : 64,
                           MRSPH_KERNEL_HYPERBOLIC, 1.0, prec == "fp32" ? MRSPH_FP32_SPLIT : MRSPH_FP64_PLAIN);
    else {
      std::fprintf(stderr, "unknown case %s\n", wl.c_str());
      return 1;
    }
    if (count_only) {
      std::printf("{\"workload\": \"%s\", \"n_particles\": %lld}\n", c.name.c_str(), c.n_particles);
      return 0;
    }
    if (steps < 0) steps = c.steps;
    SPH_mesh_generation sim(c);
    if (lset)
      Level_set_binary_writer((out.empty() ? std::string(".") : out) + "/outdata")
          .Output_lset(0, sim, (int)c.levels.size() - 1, 0);
    if (lset_rst) Save_lset_restart(sim, (out.empty() ? std::string(".") : out) + "/rstfile/levelset.rst", -1);
    if (cut_cell && n < 0) n = sim.Get_num_particles();
    sim.Initialize_case(n);
    Solver solver(sim);
    solver.Set_vtu_output(vtu);
    double ms;
    if (every > 0 && steps % every == 0) {  // the reference's output schedule
      Initialization ini;
      ini.end_time = steps;
      ini.output_dt = every;
      ms = solver.Load_solver(ini, out);
    } else {
      ms = solver.SPH_Mesh_Generation_Solver(steps, every, out);
    }
    const mrsph_stats st = sim.Stats();
    std::string cvp;
    if (cvp_k > 0) {
      const std::vector<double> x = sim.Positions();
      const long long np = sim.num_particles();
      std::vector<double> vp(3 * (size_t)cvp_k);
      for (int k = 0; k < cvp_k; k++)
        for (int q = 0; q < 3; q++) vp[3 * k + q] = x[3 * (size_t)((long long)k * np / cvp_k) + q];
      mrsph_cvp_params p{};
      p.num_vp = cvp_k;
      p.max_iter = cvp_iter;
      p.pressure_step = 1;
      p.error_tolerance = 0.05;
      p.relax_ratio = 0.8;
      const mrsph_cvp_result r = sim.Partitioning(vp, p);
      char buf[160];
      std::snprintf(buf, sizeof(buf), ", \"cvp\": {\"iterations\": %d, \"converged\": %d, \"error_max\": %.17g, \"vp\": [",
                    r.iterations, r.converged, r.error_max);
      cvp = buf;
      for (size_t q = 0; q < vp.size(); q++) {
        std::snprintf(buf, sizeof(buf), "%s%.17g", q ? ", " : "", vp[q]);
        cvp += buf;
      }
      cvp += "]}";
    }
    if (mesh) {
      const std::string od = (out.empty() ? std::string(".") : out) + "/outdata";
      Mesh_binary_writer(od).Output_mesh(0, sim);
      if (c.params.dim == 3) {
        std::vector<int> tets;
        const mrsph_tet_quality tq = sim.Reconstruct_tets(tets);
        char buf[320];
        std::snprintf(buf, sizeof(buf),
                      ", \"tets\": {\"ntet\": %lld, \"nopen\": %lld, \"ndeleted\": %lld, \"total_volume\": %.17g, "
                      "\"max_aspect\": %.17g, \"avg_aspect\": %.17g, \"min_dihedral\": %.17g}",
                      tq.ntet, tq.nopen, tq.ndeleted, tq.total_volume, tq.max_aspect, tq.avg_aspect,
                      tq.min_dihedral);
        cvp += buf;
      }
    }
    std::printf("{\"workload\": \"%s\", \"n_particles\": %lld, \"steps\": %d, \"device_ms\": %.6f, "
                "\"particle_steps_per_s\": %.6e, \"dt\": %.17g, \"step\": %lld, \"flags\": %d%s}\n",
                c.name.c_str(), sim.num_particles(), steps, ms,
                ms > 0 ? (double)sim.num_particles() * steps / (ms / 1000.0) : 0.0, st.dt, st.step, st.flags,
                cvp.c_str());
  } catch (const Error& e) {
    std::fprintf(stderr, "mrsph_relax: %s (status %d)\n", e.what(), e.code);
    return 2;
  }
  return 0;
}
