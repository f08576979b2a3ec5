// ref_aabb_shim.cpp — TEST INFRASTRUCTURE ONLY.  A C ABI over the reference's
// own segment clipping (geometry_tools/AABB_calculator.cpp, compiled from its
// sources into oracle/_ref/libref_aabb.so): the length of a segment inside a
// box as GeometryCalculator::Get_segment_length (geometry_calculator.cpp:
// 571-589) forms it from Segment_AABB_Intersection.  It pins the oracle's
// orc_segment_length (the SEGMENT cells' lengths of the cut-cell pass).
#include <cmath>

#include "AABB_calculator.h"

extern "C" double ref_segment_length(const double* mn, const double* mx, const double* v0, const double* v1) {
  double p0[3] = {0., 0., 0.}, p1[3] = {0., 0., 0.};
  if (!AABB_calculator::Segment_AABB_Intersection(mn, mx, v0, v1, p0, p1)) return 0.;
  const double d[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
  return std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
}
