// ref_kernels_shim.cpp — TEST INFRASTRUCTURE ONLY.  A C ABI over the
// reference's own Particle_base arithmetic, compiled together with the
// reference's base_cls_particle/particle.cpp (from its sources, with the
// stand-in headers of oracle/ref_stubs/ in place of TBB, Boost and the MPI
// solver classes) into oracle/_ref/libref_kernels_<D>d_<kernel>.so, one
// library per dimension (_DIM2_ / _DIM3_) and kernel macro.  It pins the
// oracle's kernel functions (rows A12: Kernel_function*, particle.cpp:31-401;
// Derivative_kernel_function*, :405-807) and its level law (row A5:
// Set_particle_scale, :957-975) to the code they restate.
#include "glbfunc.h"
#include "particle.h"
#include "sph.h"

extern "C" {

int ref_dim(void) { return DIM; }

// which: 0 = Kernel_function (the build's DIM), 1/2/3 = the _1D/_2D/_3D variant
double ref_kernel_W(int which, double dist, double h) {
  Particle_base p;
  switch (which) {
    case 1: return p.Kernel_function_1D(dist, h);
    case 2: return p.Kernel_function_2D(dist, h);
    case 3: return p.Kernel_function_3D(dist, h);
    default: return p.Kernel_function(dist, h);
  }
}

double ref_kernel_dW(int which, double dist, double h) {
  Particle_base p;
  my_real dr;
  switch (which) {
    case 1: return p.Derivative_kernel_function_1D(dist, dr, h);
    case 2: return p.Derivative_kernel_function_2D(dist, dr, h);
    case 3: return p.Derivative_kernel_function_3D(dist, dr, h);
    default: return p.Derivative_kernel_function(dist, dr, h);
  }
}

// Set_particle_scale from (h, scale): the new scale and the flag it raises
int ref_set_particle_scale(double h, double scale, double max_scale, double min_scale, double* scale_out) {
  Particle_base p;
  SPH sph;
  sph.max_scale = max_scale;
  sph.min_scale = min_scale;
  p.h = h;
  p.scale = scale;
  int flag = 0;
  p.Set_particle_scale(&sph, flag);
  *scale_out = p.scale;
  return flag;
}

}  // extern "C"
