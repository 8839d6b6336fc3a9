// osb_closures.h -- the Carpenter boundary-closure weights of the central derivatives, shared
// by the central kernels' launches and the stretched-grid metrics.
#pragma once

#include <algorithm>
#include <cmath>

namespace osb {

// The one-sided fourth-order boundary closure of the central first derivative (Carpenter,
// Gottlieb and Abarbanel, J. Comput. Phys. 1998, doi:10.1006/jcph.1998.6114) as
// Carpenter_scheme.py:91-111 forms it: inv(A_L) A_R, row r for the point r from the wall weighing
// the points m - r (m = 0..5), row 0 the exact third-order rule (the reference rationalises it);
// and the two rows of its second-derivative closure (Carpenter_scheme.py:79-86).
struct Closures {
  double c1[4][6];
  double c2[2][5];
};
inline const Closures& closures() {
  static const Closures cl = [] {
    Closures k{};
    const double R1 = -(2177.0 * std::sqrt(295369.0) - 1166427.0) / 25488.0;
    const double R2 = (66195.0 * std::sqrt(53.0) * std::sqrt(5573.0) - 35909375.0) / 101952.0;
    double L[4][4] = {
        {-(216.0 * R2 + 2160.0 * R1 - 2125.0) / 12960.0, (81.0 * R2 + 675.0 * R1 + 415.0) / 540.0,
         -(72.0 * R2 + 720.0 * R1 + 445.0) / 1440.0, -(108.0 * R2 + 756.0 * R1 + 421.0) / 1296.0},
        {(81.0 * R2 + 675.0 * R1 + 415.0) / 540.0, -(4104.0 * R2 + 32400.0 * R1 + 11225.0) / 4320.0,
         (1836.0 * R2 + 14580.0 * R1 + 7295.0) / 2160.0, -(216.0 * R2 + 2160.0 * R1 + 655.0) / 4320.0},
        {-(72.0 * R2 + 720.0 * R1 + 445.0) / 1440.0, (1836.0 * R2 + 14580.0 * R1 + 7295.0) / 2160.0,
         -(4104.0 * R2 + 32400.0 * R1 + 12785.0) / 4320.0, (81.0 * R2 + 675.0 * R1 + 335.0) / 540.0},
        {-(108.0 * R2 + 756.0 * R1 + 421.0) / 1296.0, -(216.0 * R2 + 2160.0 * R1 + 655.0) / 4320.0,
         (81.0 * R2 + 675.0 * R1 + 335.0) / 540.0, -(216.0 * R2 + 2160.0 * R1 - 12085.0) / 12960.0}};
    double X[4][6] = {
        {-0.5, -(864.0 * R2 + 6480.0 * R1 + 305.0) / 4320.0, (216.0 * R2 + 1620.0 * R1 + 725.0) / 540.0,
         -(864.0 * R2 + 6480.0 * R1 + 3335.0) / 4320.0, 0.0, 0.0},
        {(864.0 * R2 + 6480.0 * R1 + 305.0) / 4320.0, 0.0, -(864.0 * R2 + 6480.0 * R1 + 2315.0) / 1440.0,
         (108.0 * R2 + 810.0 * R1 + 415.0) / 270.0, 0.0, 0.0},
        {-(216.0 * R2 + 1620.0 * R1 + 725.0) / 540.0, (864.0 * R2 + 6480.0 * R1 + 2315.0) / 1440.0, 0.0,
         -(864.0 * R2 + 6480.0 * R1 + 785.0) / 4320.0, -1.0 / 12.0, 0.0},
        {(864.0 * R2 + 6480.0 * R1 + 3335.0) / 4320.0, -(108.0 * R2 + 810.0 * R1 + 415.0) / 270.0,
         (864.0 * R2 + 6480.0 * R1 + 785.0) / 4320.0, 0.0, 8.0 / 12.0, -1.0 / 12.0}};
    // A_L X = A_R by Gauss-Jordan elimination with partial pivoting
    for (int col = 0; col < 4; ++col) {
      int piv = col;
      for (int r = col + 1; r < 4; ++r)
        if (std::fabs(L[r][col]) > std::fabs(L[piv][col])) piv = r;
      for (int j = 0; j < 4; ++j) std::swap(L[col][j], L[piv][j]);
      for (int j = 0; j < 6; ++j) std::swap(X[col][j], X[piv][j]);
      const double inv = 1.0 / L[col][col];
      for (int j = 0; j < 4; ++j) L[col][j] *= inv;
      for (int j = 0; j < 6; ++j) X[col][j] *= inv;
      for (int r = 0; r < 4; ++r) {
        if (r == col) continue;
        const double f = L[r][col];
        for (int j = 0; j < 4; ++j) L[r][j] -= f * L[col][j];
        for (int j = 0; j < 6; ++j) X[r][j] -= f * X[col][j];
      }
    }
    for (int r = 0; r < 4; ++r)
      for (int m = 0; m < 6; ++m) k.c1[r][m] = std::fabs(X[r][m]) < 1e-14 ? 0.0 : X[r][m];
    const double row0[6] = {-11.0 / 6.0, 3.0, -1.5, 1.0 / 3.0, 0.0, 0.0};
    for (int m = 0; m < 6; ++m) k.c1[0][m] = row0[m];
    const double d2[2][5] = {{35.0 / 12.0, -104.0 / 12.0, 114.0 / 12.0, -56.0 / 12.0, 11.0 / 12.0},
                             {11.0 / 12.0, -20.0 / 12.0, 6.0 / 12.0, 4.0 / 12.0, -1.0 / 12.0}};
    for (int r = 0; r < 2; ++r)
      for (int m = 0; m < 5; ++m) k.c2[r][m] = d2[r][m];
    return k;
  }();
  return cl;
}

}  // namespace osb
