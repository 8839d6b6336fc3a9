// osb_flux.cu -- launches of the characteristic flux sweeps, compiled once per precision
// (OSB_T), dimension (OSB_ND) and grid kind (OSB_CURV: curvilinear metrics) so the
// instantiations build in parallel.
#include <algorithm>

#include "osb_internal.h"

#ifndef OSB_T
#define OSB_T double
#define OSB_ND 3
#define OSB_NAME flux_f64_3d
#endif
#ifndef OSB_CURV
#define OSB_CURV false
#endif
// 1D blocks have no second sweep to carry the RK update
#define ND_FUSABLE(nd) ((nd) >= 2)

namespace osb {
namespace {

// One y or z sweep over `lines` lines of N interfaces: the lines are cut into segments so the
// CTAs fill the resident slots in nearly whole waves (a segment costs one extra interface and
// the start of its 6-point window, about 1.5 interfaces).
template <typename T, int ND, int D, int SCH, int AVG, bool CURV, bool FUSE, int FLX>
int launch_sweep_k(osb_ctx* c, const BlockK& k, const SchemeParams& sp, int N, int other, const RkFuse& rf) {
  auto kern = k_flux_sweep<T, ND, D, SCH, AVG, CURV, FUSE, FLX>;
  const long slots = (long)resident_ctas(kern, SWEEP_THREADS, 0) * c->sm_count;
  const long gx = (k.n[0] + SWEEP_THREADS - 1) / SWEEP_THREADS;
  int nseg = wave_chunks(N, gx * other, slots, 1.5, 8);
  const int seg = (N + nseg - 1) / nseg;
  nseg = (N + seg - 1) / seg;
  const long gy = (long)other * nseg;
  dim3 grid((unsigned)gx, (unsigned)std::min(gy, 65535L), (unsigned)((gy + 65534) / 65535));
  if (grid.z > 1) return fail(OSB_ENOTSUP, "block too large for the sweep grid");
  kern<<<grid, SWEEP_THREADS, 0, c->stream>>>(k, sp, seg, nseg, 0, rf);
  return OSB_OK;
}

template <typename T, int ND, int D, int SCH, int AVG, bool CURV, int FLX>
int launch_sweep(osb_ctx* c, const BlockK& k, const SchemeParams& sp, int N, int other, const RkFuse* rf) {
  if constexpr (sizeof(T) == 4 && FLX == 0) {
    if (rf) return launch_sweep_k<T, ND, D, SCH, AVG, CURV, true, FLX>(c, k, sp, N, other, *rf);
  }
  return launch_sweep_k<T, ND, D, SCH, AVG, CURV, false, FLX>(c, k, sp, N, other, RkFuse{});
}

// x sweep (writes R), then y[, z] sweeps (accumulate); with rf (FP32 path, 2D/3D) the last
// sweep applies the RK update instead of storing the residual.
template <typename T, int ND, int SCH, int AVG, bool CURV, int FLX = 0>
int launch_flux(osb_ctx* c, Block& bl, const SchemeParams& sp, const RkFuse* rf) {
  BlockK& k = bl.k;
  cudaStream_t st = c->stream;
  // x sweep (writes R)
  {
    constexpr int NF = SweepFields<ND, CURV>::N;
    const size_t smem = (size_t)XWARPS * sizeof(XTile<T, NF, CURV ? ND + 3 : ND + 2>);
    auto kern = k_flux_x<T, ND, SCH, AVG, CURV, FLX>;
    OSB_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int nrows = k.n[1] * k.n[2];
    const long gy = (nrows + 32 * XWARPS - 1) / (32 * XWARPS);
    // osb_set_variant: 0 = segments from the wave model (a segment start costs about four
    // interfaces: the extra interface, the window start and the first chunk's copy), 1 = whole
    // rows, 2 = 64, 3 = 32, 4 = 16, 5 = 48 points per segment
    static const int fixed_seg[6] = {0, 0, 64, 32, 16, 48};
    int xseg;
    if (c->variant == 1) xseg = k.n[0];
    else if (c->variant >= 2 && c->variant <= 5) xseg = fixed_seg[c->variant];
    else {
      const long slots = (long)resident_ctas(kern, 32 * XWARPS, smem) * c->sm_count;
      const int nx = wave_chunks(k.n[0], gy, slots, 4.0, 16);
      xseg = (k.n[0] + nx - 1) / nx;
    }
    // whole flush tiles per segment (sector-aligned stores), at most the row
    xseg = std::max(XOUT, (std::min(xseg, k.n[0]) + XOUT - 1) / XOUT * XOUT);
    // segment 0 also carries the row's head [0, a) before its first sector boundary
    dim3 grid((k.n[0] + xseg - 1) / xseg, (unsigned)gy);
    timing_begin(c, FAM_FLUX_X);
    kern<<<grid, 32 * XWARPS, smem, st>>>(k, sp, 1, xseg, bl.xrows);
    timing_end(c);
    c->launches++;
  }
  // y, z sweeps (accumulate)
  for (int D = 1; D < ND; ++D) {
    const int N = k.n[D];
    const int other = ND == 3 ? (D == 1 ? k.n[2] : k.n[1]) : 1;
    timing_begin(c, D == 1 ? FAM_FLUX_Y : FAM_FLUX_Z);
    const RkFuse* f = D == ND - 1 ? rf : nullptr;
    int rc = OSB_OK;
    if (D == 1) rc = launch_sweep<T, ND, 1, SCH, AVG, CURV, FLX>(c, k, sp, N, other, f);
    else if (ND == 3) rc = launch_sweep<T, ND, (ND == 3 ? 2 : 1), SCH, AVG, CURV, FLX>(c, k, sp, N, other, f);
    timing_end(c);
    if (rc != OSB_OK) return rc;
    c->launches++;
  }
  return OSB_OK;
}

// HLLC-LM flux (Cartesian 2D / 3D blocks, fifth-order reconstructions): the sweeps do not carry
// the RK update for it
template <typename T, int ND>
int dispatch_hllc(osb_ctx* c, Block& bl, const SchemeParams& sp) {
  const int sch = bl.d.scheme, avg = bl.d.averaging;
  if (avg == OSB_AVG_ROE) {
    if (sch == OSB_SCHEME_WENO5_JS) return launch_flux<T, ND, SCH_WENO5_JS, AVG_ROE, false, 1>(c, bl, sp, nullptr);
    if (sch == OSB_SCHEME_WENO5_Z) return launch_flux<T, ND, SCH_WENO5_Z, AVG_ROE, false, 1>(c, bl, sp, nullptr);
    if (sch == OSB_SCHEME_TENO5) return launch_flux<T, ND, SCH_TENO5, AVG_ROE, false, 1>(c, bl, sp, nullptr);
  } else {
    if (sch == OSB_SCHEME_WENO5_JS) return launch_flux<T, ND, SCH_WENO5_JS, AVG_SIMPLE, false, 1>(c, bl, sp, nullptr);
    if (sch == OSB_SCHEME_WENO5_Z) return launch_flux<T, ND, SCH_WENO5_Z, AVG_SIMPLE, false, 1>(c, bl, sp, nullptr);
    if (sch == OSB_SCHEME_TENO5) return launch_flux<T, ND, SCH_TENO5, AVG_SIMPLE, false, 1>(c, bl, sp, nullptr);
  }
  return fail(OSB_ENOTSUP, "the HLLC-LM flux takes the fifth-order WENO / TENO reconstructions");
}

template <typename T, int ND, bool CURV>
int dispatch_flux_nd(osb_ctx* c, Block& bl, const SchemeParams& sp, const RkFuse* rf) {
  const int sch = bl.d.scheme, avg = bl.d.averaging;
  if (bl.d.flux_type == OSB_FLUX_HLLC_LM) {
    if constexpr (!CURV && ND >= 2) return dispatch_hllc<T, ND>(c, bl, sp);
    return fail(OSB_ENOTSUP, "the HLLC-LM flux is implemented for Cartesian 2D and 3D blocks");
  }
  if (avg == OSB_AVG_ROE) {
    if (sch == OSB_SCHEME_WENO5_JS) return launch_flux<T, ND, SCH_WENO5_JS, AVG_ROE, CURV>(c, bl, sp, rf);
    if (sch == OSB_SCHEME_WENO5_Z) return launch_flux<T, ND, SCH_WENO5_Z, AVG_ROE, CURV>(c, bl, sp, rf);
    if (sch == OSB_SCHEME_TENO5) return launch_flux<T, ND, SCH_TENO5, AVG_ROE, CURV>(c, bl, sp, rf);
    if (sch == OSB_SCHEME_TENO6) return launch_flux<T, ND, SCH_TENO6, AVG_ROE, CURV>(c, bl, sp, rf);
  } else {
    if (sch == OSB_SCHEME_WENO5_JS) return launch_flux<T, ND, SCH_WENO5_JS, AVG_SIMPLE, CURV>(c, bl, sp, rf);
    if (sch == OSB_SCHEME_WENO5_Z) return launch_flux<T, ND, SCH_WENO5_Z, AVG_SIMPLE, CURV>(c, bl, sp, rf);
    if (sch == OSB_SCHEME_TENO5) return launch_flux<T, ND, SCH_TENO5, AVG_SIMPLE, CURV>(c, bl, sp, rf);
    if (sch == OSB_SCHEME_TENO6) return launch_flux<T, ND, SCH_TENO6, AVG_SIMPLE, CURV>(c, bl, sp, rf);
  }
  return fail(OSB_ENOTSUP, "unsupported scheme/averaging %d/%d", sch, avg);
}



}  // namespace

int OSB_NAME(osb_ctx* c, Block& bl, const SchemeParams& sp, const RkFuse* rf) {
  return dispatch_flux_nd<OSB_T, OSB_ND, OSB_CURV>(c, bl, sp, ND_FUSABLE(OSB_ND) ? rf : nullptr);
}

}  // namespace osb
