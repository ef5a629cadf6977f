// Host maths used to set up the kernels.
#pragma once

#include <vector>

#include "common.cuh"

namespace trvg {

double wigner_3j(int j1, int j2, int j3, int m1, int m2, int m3);
double calc_coupling_coeff_3pt(int ell1, int ell2, int ELL, int m1, int m2,
                               int M);
double calc_coupling_coeff_2pt(int ell, int ELL, int m, int M);
double sph_bessel(int ell, double x);

constexpr double kEpsCoupling = 1.e-9;   // maths.cpp:165

// Natural cubic spline of j_ell on the reference's nodes.
struct SplineHost {
  int ell;
  double split;
  std::vector<double> y, b, c, d;
  explicit SplineHost(int ell);
  // Table view over device (or host) copies of y, b, c and d.
  SplineTable table(const double* dy, const double* db, const double* dc,
                    const double* dd) const;
};

}  // namespace trvg
