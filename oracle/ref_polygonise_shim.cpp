// ref_polygonise_shim.cpp — C ABI around the reference's marching-cubes
// polygoniser (geometry_tools/polygonise.cpp, compiled from the reference's
// own sources by oracle/build_ref.py into oracle/_ref/).
//
// TEST INFRASTRUCTURE ONLY: it pins the oracle's surface-area restatement
// (oracle/mrsph_oracle.cpp, mc_area) against the reference's polygoniser.
// The product library never links it.
#include <cmath>
#include <vector>

#include "polygonise.h"

extern "C" {

// Polygonise_MQ::Polygonise at isolevel 0 of one cube: p24 = 8 vertices
// (x, y, z), val8 = their values.  Writes up to 5 triangles (9 doubles each)
// to tris and returns their number.
int refp_polygonise(const double* p24, const double* val8, double* tris) {
  Polygonise_MQ::GRIDCELL g;
  for (int v = 0; v < 8; v++) {
    g.p[v].x = p24[3 * v];
    g.p[v].y = p24[3 * v + 1];
    g.p[v].z = p24[3 * v + 2];
    g.val[v] = val8[v];
  }
  std::vector<Polygonise_MQ::TRIANGLE> t;
  int n = Polygonise_MQ::Polygonise(g, 0.0, t);
  for (int i = 0; i < n && i < 5; i++)
    for (int k = 0; k < 3; k++) {
      tris[9 * i + 3 * k] = t[i].p[k].x;
      tris[9 * i + 3 * k + 1] = t[i].p[k].y;
      tris[9 * i + 3 * k + 2] = t[i].p[k].z;
    }
  return n;
}

// GeometryCalculator::get_area_MQ (geometry_calculator.cpp:283-321) of a 3x3x3
// corner lattice c27 ([x][y][z]), restated around the reference's polygoniser;
// the triangle area is get_area_tri (:325-350).
double refp_area_mq(const double* c27, double dx, double dy, double dz) {
  static const int V[8][3] = {{0, 0, 0}, {0, 1, 0}, {1, 1, 0}, {1, 0, 0}, {0, 0, 1}, {0, 1, 1}, {1, 1, 1}, {1, 0, 1}};
  double area = 0.0;
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++)
      for (int k = 0; k < 2; k++) {
        double p[24], val[8], tr[45];
        for (int v = 0; v < 8; v++) {
          int vx = i + V[v][0], vy = j + V[v][1], vz = k + V[v][2];
          p[3 * v] = vx * 0.5 * dx;
          p[3 * v + 1] = vy * 0.5 * dy;
          p[3 * v + 2] = vz * 0.5 * dz;
          val[v] = c27[(vx * 3 + vy) * 3 + vz];
        }
        int n = refp_polygonise(p, val, tr);
        for (int q = 0; q < n; q++) {
          const double* a = tr + 9 * q;
          double v1[3] = {a[3] - a[0], a[4] - a[1], a[5] - a[2]};
          double v3[3] = {a[6] - a[0], a[7] - a[1], a[8] - a[2]};
          double d1 = std::sqrt(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
          double d3 = std::sqrt(v3[0] * v3[0] + v3[1] * v3[1] + v3[2] * v3[2]);
          double ar = 0.5 * (d3 * d1) * std::sin(std::acos((v1[0] * v3[0] + v1[1] * v3[1] + v1[2] * v3[2]) /
                                                           (d3 * d1 + 1.e-20)));
          if (std::isnan(ar)) ar = 0.;
          area += ar;
        }
      }
  return area;
}

}  // extern "C"
