// osb_central.cu -- launches of the central 4th-order convective / viscous kernel, compiled
// once per precision (OSB_CENTRAL_T).
#include "osb_closures.h"
#include "osb_internal.h"

#include <algorithm>
#include <cmath>

namespace osb {
namespace {

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
  cp.mu_pow = d.viscous == OSB_VISC_POWER_LAW ? d.visc_power : 0.0;
  cp.mu_pow_f = (float)cp.mu_pow;
  cp.forced = d.forcing[0] != 0.0 || d.forcing[1] != 0.0 || d.forcing[2] != 0.0;
  for (int i = 0; i < 3; ++i) {
    cp.force[i] = d.forcing[i];
    cp.force_f[i] = (float)d.forcing[i];
  }
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
    if (visc == OSB_VISC_SUTHERLAND || visc == OSB_VISC_POWER_LAW) return launch_central_t<T, 2, 1>(c, bl, first, rf);
    if (visc == OSB_VISC_CONSTANT) return launch_central_t<T, 2, 2>(c, bl, first, rf);
    return launch_central_t<T, 2, 0>(c, bl, first, rf);
  }
  if (conv) {
    if (visc == OSB_VISC_SUTHERLAND || visc == OSB_VISC_POWER_LAW) return launch_central_t<T, 1, 1>(c, bl, first, rf);
    if (visc == OSB_VISC_CONSTANT) return launch_central_t<T, 1, 2>(c, bl, first, rf);
    return launch_central_t<T, 1, 0>(c, bl, first, rf);
  }
  if (visc == OSB_VISC_SUTHERLAND || visc == OSB_VISC_POWER_LAW) return launch_central_t<T, 0, 1>(c, bl, first, rf);
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
