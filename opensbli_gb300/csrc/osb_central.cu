// osb_central.cu -- launches of the central 4th-order convective / viscous kernel, compiled
// once per precision (OSB_CENTRAL_T).
#include "osb_internal.h"

#include <algorithm>
#include <cmath>

namespace osb {
namespace {

// The one-sided fourth-order boundary closure of the central first derivative (Carpenter,
// Gottlieb and Abarbanel, J. Comput. Phys. 1998, doi:10.1006/jcph.1998.6114) as
// Carpenter_scheme.py:91-111 forms it: inv(A_L) A_R, row r for the point r from the wall weighing
// the points m - r (m = 0..5), row 0 the exact third-order rule (the reference rationalises it);
// and the two rows of its second-derivative closure (Carpenter_scheme.py:79-86).
struct Closures {
  double c1[4][6];
  double c2[2][5];
};
const Closures& closures() {
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

// Faces whose central derivatives take the one-sided closures (ModifyCentralDerivative walls).
inline bool is_wall(int kind) { return kind == OSB_BC_ISOTHERMAL_WALL || kind == OSB_BC_ADIABATIC_WALL; }

template <typename T, int CONV, int VISC, bool FUSE, int CY, bool BULK, bool WALL = false>
int launch_central_k(osb_ctx* c, Block& bl, int first, const RkFuse& rf) {
  using Fd = CentralFields<T, CONV, VISC>;
  size_t smem = (size_t)Fd::N * CRING * CTile<CY, WALL ? 4 : CH>::CPL * sizeof(T);
  if (BULK) smem += CTile<CY>::RAW * sizeof(float) + 2 * sizeof(unsigned long long);
  auto kern = k_central3d<T, CONV, VISC, FUSE, CY, BULK, WALL>;
  OSB_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  CentralParams cp{};
  const osb_block_desc& d = bl.d;
  cp.gama = d.gama;
  cp.M2 = d.Minf * d.Minf;
  cp.mu_c = d.mu_const;
  cp.invRe = 1.0 / d.Re;
  cp.kheat = 1.0 / (d.Pr * d.Re * d.Minf * d.Minf * (d.gama - 1.0));
  cp.gama_f = (float)cp.gama;
  cp.M2_f = (float)cp.M2;
  cp.mu_c_f = (float)cp.mu_c;
  cp.invRe_f = (float)cp.invRe;
  cp.kheat_f = (float)cp.kheat;
  for (int i = 0; i < 3; ++i) {
    cp.invd[i] = bl.k.invd[i];
    cp.inv2d[i] = bl.k.inv2d[i];
    cp.invd_f[i] = (float)cp.invd[i];
    cp.inv2d_f[i] = (float)cp.inv2d[i];
  }
  if (WALL) {
    cp.wall_lo = is_wall(bl.d.bc[1][0]);
    cp.wall_hi = is_wall(bl.d.bc[1][1]);
    const Closures& cl = closures();
    for (int r = 0; r < 4; ++r)
      for (int m = 0; m < 6; ++m) {
        cp.c1[r][m] = cl.c1[r][m];
        cp.c1f[r][m] = (float)cl.c1[r][m];
      }
    for (int r = 0; r < 2; ++r)
      for (int m = 0; m < 5; ++m) {
        cp.c2[r][m] = cl.c2[r][m];
        cp.c2f[r][m] = (float)cl.c2[r][m];
      }
  }
  const BlockK& k = bl.k;
  // z chunks per column: whole waves of resident CTAs; a chunk starts by staging four planes
  // (two of halo) at about a third of the cost of a computed plane each
  const long cols = (long)((k.n[0] + CX - 1) / CX) * ((k.n[1] + CY - 1) / CY);
  const long slots = (long)resident_ctas(kern, CX * CY, smem) * c->sm_count;
  const int nz = wave_chunks(k.n[2], cols, slots, 1.4, 4);
  const int czc = (k.n[2] + nz - 1) / nz;
  dim3 grid((k.n[0] + CX - 1) / CX, (k.n[1] + CY - 1) / CY, (k.n[2] + czc - 1) / czc);
  timing_begin(c, FAM_CENTRAL);
  kern<<<grid, CX * CY, smem, c->stream>>>(k, cp, first, czc, rf);
  timing_end(c);
  c->launches++;
  return OSB_OK;
}

// Tile height of the FP32 kernels: 8 rows unless the ring holds the KGP form's eleven fields of a
// block whose cross-section already gives every SM several columns (measured: 8 rows are 37 %
// faster on the 64^3 central TGV and equal on the 256^3 TENO5 one; 4 rows are 1.4 % faster for
// the 256^3 KGP form).  The FP64 kernels (FP64-pipe bound, a ring twice as large) keep 4 rows.
template <typename T, int CONV, int VISC, bool FUSE, bool BULK>
int launch_central_h(osb_ctx* c, Block& bl, int first, const RkFuse& rf) {
  if constexpr (CONV == 0 && !BULK) {
    if (is_wall(bl.d.bc[1][0]) || is_wall(bl.d.bc[1][1]))
      return launch_central_k<T, CONV, VISC, FUSE, 4, false, true>(c, bl, first, rf);
  }
  const long cols4 = (long)((bl.k.n[0] + CX - 1) / CX) * ((bl.k.n[1] + 3) / 4);
  if (sizeof(T) == 8 || (CONV == 2 && cols4 >= 2L * c->sm_count))
    return launch_central_k<T, CONV, VISC, FUSE, 4, BULK>(c, bl, first, rf);
  if constexpr (sizeof(T) == 4) return launch_central_k<T, CONV, VISC, FUSE, 8, BULK>(c, bl, first, rf);
  return OSB_OK;
}

// With rf (FP32 path) the kernel applies the RK update instead of storing the residual; its
// planes come in by register loads or, after osb_set_central_staging(1), by bulk copies.
template <typename T, int CONV, int VISC>
int launch_central_t(osb_ctx* c, Block& bl, int first, const RkFuse* rf) {
  if constexpr (sizeof(T) == 4) {
    const bool wall = is_wall(bl.d.bc[1][0]) || is_wall(bl.d.bc[1][1]);
    if (rf && c->central_bulk && !wall) return launch_central_h<T, CONV, VISC, true, true>(c, bl, first, *rf);
    if (rf) return launch_central_h<T, CONV, VISC, true, false>(c, bl, first, *rf);
  }
  return launch_central_h<T, CONV, VISC, false, false>(c, bl, first, RkFuse{});
}

template <typename T>
int launch_central(osb_ctx* c, Block& bl, bool conv, int first, const RkFuse* rf) {
  const int visc = bl.d.viscous;
  if (conv && bl.d.split_form == OSB_SPLIT_KGP) {
    if (visc == OSB_VISC_SUTHERLAND) return launch_central_t<T, 2, 1>(c, bl, first, rf);
    if (visc == OSB_VISC_CONSTANT) return launch_central_t<T, 2, 2>(c, bl, first, rf);
    return launch_central_t<T, 2, 0>(c, bl, first, rf);
  }
  if (conv) {
    if (visc == OSB_VISC_SUTHERLAND) return launch_central_t<T, 1, 1>(c, bl, first, rf);
    if (visc == OSB_VISC_CONSTANT) return launch_central_t<T, 1, 2>(c, bl, first, rf);
    return launch_central_t<T, 1, 0>(c, bl, first, rf);
  }
  if (visc == OSB_VISC_SUTHERLAND) return launch_central_t<T, 0, 1>(c, bl, first, rf);
  if (visc == OSB_VISC_CONSTANT) return launch_central_t<T, 0, 2>(c, bl, first, rf);
  return OSB_OK;
}

}  // namespace

#ifndef OSB_CENTRAL_T
#define OSB_CENTRAL_T double
#define OSB_CENTRAL_NAME central_f64
#endif

int OSB_CENTRAL_NAME(osb_ctx* c, Block& bl, bool conv, int first, const RkFuse* rf) {
  return launch_central<OSB_CENTRAL_T>(c, bl, conv, first, rf);
}

}  // namespace osb
