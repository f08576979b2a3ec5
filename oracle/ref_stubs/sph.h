// sph.h (stand-in) — TEST INFRASTRUCTURE ONLY.  The two members of the
// reference's SPH class that Particle_base::Set_particle_scale reads
// (particle.cpp:957-975); shadows the reference's sph.h, which needs MPI.
#pragma once
class SPH {
 public:
  Real max_scale;
  Real min_scale;
};
