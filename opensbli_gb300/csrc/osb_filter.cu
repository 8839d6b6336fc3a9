// osb_filter.cu -- the non-linear characteristic WENO3 filter applied after every full RK step
// (filters/WENO_filter.py), as the generated Central4-WENO5 benchmark runs it
// (apps/performance_benchmark/Central4-WENO5/opensbli.cpp:386-513, kernels 043-049):
//   1. the filter's own periodic halo exchange (bc_exchanges.h groups 51-56);
//   2. the Ducros sensor kappa on the interior (kernel 044; its halos stay zero);
//   3. per direction the filter flux at every interface i+1/2, i = -1..N-1 (kernels 046-048);
//   4. q += dt * mask * (-sum_d (F_d(i) - F_d(i-1)) / Delta_d), mask = [max kappa over the
//      point and its neighbours >= Ducros_select] (kernel 049).
// The non-linear characteristic TVD filter (filters/TVD_filter.py; the Yee-Sandham-Djomehri
// limiter with Harten's switch, schemes/spatial/shock_capturing.py:619-766) runs the same
// exchange, then per direction its flux at interfaces i = -1..N-1 and the same update without a
// sensor mask, as the generated solver of the TGV app's TVD branch does.
// Compiled once per precision (OSB_FILTER_T).  In the FP32-residual path the filter reads the
// FP32 state, forms the increment in FP32 and adds it to the FP64 state, then refreshes the
// FP32 copy of the points it changed.
#include <algorithm>

#include "osb_internal.h"

#ifndef OSB_FILTER_T
#define OSB_FILTER_T double
#define OSB_FILTER_NAME filter_f64
#define OSB_TVD_STALE_NAME tvd_stale_f64
#endif

namespace osb {
namespace {

constexpr int FT = 256;  // threads per CTA of the filter kernels

// The exchange before the filter: direction d, both sides (they read and write disjoint
// points).  Side 0 copies [0, 4) to [N, N+4), side 1 copies [N-4, N) to [-4, 0), over the
// transverse range [-4, N-4) of the other directions -- the generated iteration range (base
// -4, extent N); no exchange follows the last RK stage, so the halo points outside that range
// keep the values of the exchange after the previous stage.
__global__ void k_filter_halo(BlockK b, int d, int fields) {
  int ext[3];
  for (int e = 0; e < 3; ++e) ext[e] = b.n[e];
  ext[d] = 4;
  const int per = ext[0] * ext[1] * ext[2];
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < 2 * per; t += gridDim.x * blockDim.x) {
    const int side = t >= per;
    const int u = t - side * per;
    int c[3];
    c[0] = u % ext[0];
    c[1] = (u / ext[0]) % ext[1];
    c[2] = u / (ext[0] * ext[1]);
    int src[3], dst[3];
    for (int e = 0; e < 3; ++e) src[e] = dst[e] = c[e] - 4;
    if (side == 0) {
      src[d] = c[d];
      dst[d] = b.n[d] + c[d];
    } else {
      src[d] = b.n[d] - 4 + c[d];
      dst[d] = c[d] - 4;
    }
    const int si = lin(b, src[0], src[1], src[2]), di = lin(b, dst[0], dst[1], dst[2]);
    if (fields & 1)
      for (int v = 0; v < 5; ++v) b.q[v][di] = b.q[v][si];
    if ((fields & 2) && b.qf[0])
      for (int v = 0; v < 5; ++v) b.qf[v][di] = b.qf[v][si];
  }
}

// FP32 path: the last RK stage wrote the other buffer of the FP32 ping-pong pair, whose halo
// shell still holds the state two stages back; the halos the generated step leaves before the
// filter are those of the exchange after the previous stage, which the buffer that stage read
// holds.  Copies that shell (depth D, the block's exchange depth) into the current buffer.
__global__ void k_shell_from(BlockK b, const float* __restrict__ src, int D) {
  const int n0 = b.n[0], n1 = b.n[1], n2 = b.n[2];
  const int e0 = n0 + 2 * D, e1 = n1 + 2 * D, e2 = n2 + 2 * D;
  const int total = e0 * e1 * e2;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    const int x = t % e0 - D, y = (t / e0) % e1 - D, z = t / (e0 * e1) - D;
    if (x >= 0 && x < n0 && y >= 0 && y < n1 && z >= 0 && z < n2) continue;
    const int id = lin(b, x, y, z);
    for (int v = 0; v < 5; ++v) b.qf[v][id] = src[(size_t)v * b.alloc + id];
  }
}

template <typename T>
__device__ __forceinline__ T vel(const BlockK& b, int i, int id) {
  return ld_q<T>(b, 1 + i, id) / ld_q<T>(b, 0, id);
}

// Ducros sensor (kernel 044): (div u)^2 (1/2 - 1/2 tanh(2.5 + 500 div u / |Delta|)) /
// (1e-40 + |curl u|^2 + (div u)^2), central-4 derivatives.  FP32: the 1e-40 (below the FP32
// normal range) becomes 1e-30.
template <typename T>
__global__ void k_ducros(BlockK b, T* kappa, T inv_h) {
  const int n0 = b.n[0], n1 = b.n[1], n2 = b.n[2];
  const int total = n0 * n1 * n2;
  const T id[3] = {inv_delta<T>(b, 0), inv_delta<T>(b, 1), inv_delta<T>(b, 2)};
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    const int x = t % n0, y = (t / n0) % n1, z = t / (n0 * n1);
    const int c = lin(b, x, y, z);
    T du[3][3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const int s = b.st[j];
#pragma unroll
      for (int i = 0; i < 3; ++i)
        du[i][j] = (-L_(2.0 / 3.0) * vel<T>(b, i, c - s) - L_(1.0 / 12.0) * vel<T>(b, i, c + 2 * s) +
                    L_(1.0 / 12.0) * vel<T>(b, i, c - 2 * s) + L_(2.0 / 3.0) * vel<T>(b, i, c + s)) *
                   id[j];
    }
    const T div = du[0][0] + du[1][1] + du[2][2];
    const T wz = -du[0][1] + du[1][0], wx = -du[1][2] + du[2][1], wy = -du[2][0] + du[0][2];
    const T tiny = sizeof(T) == 8 ? L_(1.0e-40) : L_(1.0e-30);
    kappa[c] = (div * div) * (L_(0.5) - L_(0.5) * tanh(L_(2.5) + L_(500.0) * div * inv_h)) /
               (tiny + wz * wz + wx * wx + wy * wy + div * div);
  }
}

// One side of the WENO3-Z filter reconstruction of a wave: f = the split flux at points
// i-1..i+2, side + uses {i-1, i, i+1}, side - {i, i+1, i+2}.  Returns the side's
// contribution to the reconstruction; rj receives its smoothness-sensor term.
// Smoothness of the two-point stencil {lo, hi} (hi = the higher index), as generated:
// 1/4 hi^2 + 1/2 (1/2 lo - hi) lo.
template <typename T>
__device__ __forceinline__ T beta2(T lo, T hi) {
  return L_(0.25) * (hi * hi) + L_(0.5) * (L_(0.5) * lo - hi) * lo;
}

template <typename T, int SIDE>
__device__ __forceinline__ T weno3_side(const T (&f)[4], T eps32, T& rj) {
  // stencil values in the side's own order: a = far-upwind, b = centre, c = downwind
  const T a = SIDE > 0 ? f[0] : f[3], bb = SIDE > 0 ? f[1] : f[2], cc = SIDE > 0 ? f[2] : f[1];
  const T bd = beta2<T>(f[1], f[2]);                                       // downwind pair {i, i+1}
  const T bu = SIDE > 0 ? beta2<T>(f[0], f[1]) : beta2<T>(f[2], f[3]);     // upwind pair
  T ad, au;
  if (sizeof(T) == 8) {
    const T t = fabs(bu - bd) * fabs(bu - bd);
    ad = L_(0.666666666666667) + L_(2.0 / 3.0) * t / ((L_(1.0e-40) + bd) * (L_(1.0e-40) + bd));
    au = L_(0.333333333333333) + L_(1.0 / 3.0) * t / ((L_(1.0e-40) + bu) * (L_(1.0e-40) + bu));
  } else {
    // FP32: epsilon relative to the stencil, and the ratio squared after the division (no
    // underflow of (eps + beta)^2)
    const T tau = fabs(bu - bd);
    const T rd = tau / (eps32 + bd), ru = tau / (eps32 + bu);
    ad = L_(2.0 / 3.0) * (L_(1.0) + rd * rd);
    au = L_(1.0 / 3.0) * (L_(1.0) + ru * ru);
  }
  const T ia = L_(1.0) / (ad + au);
  const T wd = ad * ia, wu = au * ia;
  rj = L_(0.333333333333333) * fabs(-L_(1.0) + L_(3.0) * wu) + L_(0.333333333333333) * fabs(-L_(1.0) + L_(1.5) * wd);
  return (-L_(0.25) * a + L_(0.75) * bb) * wu + (L_(0.25) * bb + L_(0.25) * cc) * wd;
}

// Filter flux at interface i+1/2 along direction D (local frame: w[m] = point i-1+m, normal
// momentum first), kernels 046-048: Roe average of points i, i+1, characteristic projections
// of Q and F, per wave the WENO3-Z reconstruction of CF +/- lambda CS (both sides) minus the
// central 4th-order interpolation of CF, scaled by rj, back-projected with the REV columns.
template <typename T>
__device__ __forceinline__ void filter_flux(const Pt<T, 3> (&w)[4], const SP<T>& sp, T (&fh)[5]) {
  constexpr int ND = 3, NV = 5;
  const T g1 = sp.g1;
  const Pt<T, 3>& L = w[1];
  const Pt<T, 3>& R = w[2];
  const T sL = sqrt(L.q[0]), sR = sqrt(R.q[0]);
  const T rho = sqrt(L.q[0] * R.q[0]);
  const T inv = L_(1.0) / (sL + sR);
  T u[ND], ke = L_(0.0);
#pragma unroll
  for (int i = 0; i < ND; ++i) {
    u[i] = (sL * L.u[i] + sR * R.u[i]) * inv;
    ke += u[i] * u[i];
  }
  const T a = sqrt((-L_(0.5) * ke + ((L.p + L.q[NV - 1]) / sL + (R.p + R.q[NV - 1]) / sR) * inv) * g1);
  const T sfc = sp.sfc;
  const T lam_u = sfc * fmax(fabs(R.u[0]), fabs(L.u[0]));
  const T lam_p = sfc * fmax(fabs(R.u[0] + R.a), fabs(L.u[0] + L.a));
  const T lam_m = sfc * fmax(fabs(R.u[0] - R.a), fabs(L.u[0] - L.a));
  const T ia = L_(1.0) / a, ia2 = ia * ia, irho = L_(1.0) / rho;
  const T phi = g1 * L_(0.5) * ke;
  const T bta = ia * irho * L_(0.70710678118654752440);
  const T alf = rho * ia * L_(0.70710678118654752440);
  T cs[NV][4], cf[NV][4];
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const Pt<T, 3>& s = w[m];
    T Fv[NV];
    Fv[0] = s.q[1];
    Fv[1] = s.u[0] * s.q[1] + s.p;
    Fv[2] = s.u[0] * s.q[2];
    Fv[3] = s.u[0] * s.q[3];
    Fv[4] = s.u[0] * (s.q[4] + s.p);
    T o2[2][NV];
    constexpr int NPASS = sizeof(T) == 4 ? 1 : 2;
#pragma unroll
    for (int pass = 0; pass < NPASS; ++pass) {
      const T* v = pass == 0 ? s.q : Fv;
      T* o = o2[pass];
      const T um = u[0] * v[1] + u[1] * v[2] + u[2] * v[3];
      const T S = phi * v[0] - g1 * um + g1 * v[4];
      const T D = v[1] - u[0] * v[0];
      o[0] = v[0] - S * ia2;
      o[1] = (v[3] - u[2] * v[0]) * irho;
      o[2] = (u[1] * v[0] - v[2]) * irho;
      o[3] = bta * (S + a * D);
      o[4] = bta * (S - a * D);
    }
    if (NPASS == 1) {
      // FP32: L.F = u_n (L.q) + p (L e_1 + u_n L e_E), the two LEV columns in closed form
      const T un = s.u[0], du = un - u[0];
      const T pb = s.p * bta, gd = g1 * du;
      o2[1][0] = un * o2[0][0] - s.p * g1 * ia2 * du;
      o2[1][1] = un * o2[0][1];
      o2[1][2] = un * o2[0][2];
      o2[1][3] = un * o2[0][3] + pb * (a + gd);
      o2[1][4] = un * o2[0][4] + pb * (gd - a);
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      cs[k][m] = o2[0][k];
      cf[k][m] = o2[1][k];  // pass 1 (FP64) or the closed form (FP32)
    }
  }
  T rec[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const T lk = k < ND ? lam_u : (k == ND ? lam_p : lam_m);
    T fp[4], fm[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      fp[m] = cs[k][m] * lk + cf[k][m];
      fm[m] = -cs[k][m] * lk + cf[k][m];
    }
    T eps32 = L_(0.0);
    if (sizeof(T) == 4) {
      const T ms = (cf[k][0] * cf[k][0] + cf[k][1] * cf[k][1] + cf[k][2] * cf[k][2] + cf[k][3] * cf[k][3] +
                    cs[k][1] * cs[k][1] * lk * lk) * L_(0.25);
      eps32 = sp.eps32_rel * ms + L_(1e-30);
    }
    T rp, rm;
    const T rcp = weno3_side<T, 1>(fp, eps32, rp);
    const T rcm = weno3_side<T, -1>(fm, eps32, rm);
    const T rj = fmax(rp, rm);
    rec[k] = (L_(1.0 / 12.0) * (-L_(7.0) * cf[k][1] - L_(7.0) * cf[k][2] + cf[k][0] + cf[k][3]) + (rcm + rcp)) * rj;
  }
  const T rp = rec[3] + rec[4], rmn = rec[3] - rec[4];
  const T F0 = rec[0] + alf * rp;
  fh[0] = F0;
  fh[1] = u[0] * F0 + alf * a * rmn;
  fh[2] = u[1] * F0 - rho * rec[2];
  fh[3] = u[2] * F0 + rho * rec[1];
  const T h0 = (phi + a * a) / g1;
  fh[4] = phi / g1 * rec[0] + rho * u[2] * rec[1] - rho * u[1] * rec[2] + alf * h0 * rp + alf * u[0] * a * rmn;
}

// Filter fluxes along D at interfaces i+1/2, i = -1..N-1, transverse interior; F[v] at the
// index of point i.  Interfaces whose stencil i-3..i+2 sees no kappa above Ducros_check get 0.
template <typename T, int D>
__global__ void k_filter_flux(BlockK b, SchemeParams spd, const T* __restrict__ kappa, T check, T* F0, T* F1, T* F2,
                              T* F3, T* F4) {
  const SP<T> sp(spd);
  int e[3] = {b.n[0], b.n[1], b.n[2]};
  e[D] += 1;
  const int total = e[0] * e[1] * e[2];
  const int s = b.st[D];
  T* F[5] = {F0, F1, F2, F3, F4};
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    int c[3] = {t % e[0], (t / e[0]) % e[1], t / (e[0] * e[1])};
    c[D] -= 1;
    const int id = lin(b, c[0], c[1], c[2]);
    T km = kappa[id - 3 * s];
#pragma unroll
    for (int m = -2; m <= 2; ++m) km = fmax(km, kappa[id + m * s]);
    T fh[5] = {L_(0.0), L_(0.0), L_(0.0), L_(0.0), L_(0.0)};
    if (km > check) {
      Pt<T, 3> w[4];
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const int pid = id + (m - 1) * s;
#pragma unroll
        for (int lv = 0; lv < 5; ++lv) w[m].q[lv] = ld_q<T>(b, gvar_fwd<3, D>(lv), pid);
        make_pt<T, 3>(w[m], sp.gama);
      }
      filter_flux<T>(w, sp, fh);
    }
#pragma unroll
    for (int lv = 0; lv < 5; ++lv) F[gvar_fwd<3, D>(lv)][id] = fh[lv];
  }
}

// ---- TVD filter ---------------------------------------------------------------------------

// A point of the TVD stencil, local frame (normal momentum and velocity first).
template <typename T>
struct TvdPt {
  T r, m[3], e, u[3], a;
};

// Entropy fix of a wave speed with delta_TVD = 1/2 (shock_capturing.py:681-689; generated as
// |z| >= 1/invdelta ? |z| : 1/2 (1/invdelta^2 + z^2) invdelta with invdelta = 2).
template <typename T>
__device__ __forceinline__ T tvd_psi(T z) {
  return fabs(z) >= L_(0.5) ? fabs(z) : L_(0.25) + z * z;  // 1/2 (1/4 + z^2) 2, exactly
}

// Limiter from the jump of this interface (hi) and the one below (lo) (lines 690-704).
template <typename T>
__device__ __forceinline__ T tvd_g(T hi, T lo) {
  const T S = hi > L_(0.0) ? L_(1.0) : (hi < L_(0.0) ? L_(-1.0) : L_(0.0));
  const T t1 = fmax(L_(0.0), fmin(S * lo, L_(2.0) * fabs(hi)));
  const T t2 = fmin(fabs(hi), L_(2.0) * S * lo);
  return S * fmax(t1, t2);
}

// The TVD filter flux at interface i+1/2 follows the generated direction-0 kernel in the local
// frame of each direction: simple averages of u, a, rho over (i-1, i), (i, i+1), (i+1, i+2); the
// characteristic jumps alpha = LEV (q_hi - q_lo) at the three half-points; wave speeds and REV
// at i+1/2; per wave sigma = psi(lambda), the limiters g at i and i+1, gamma, phi =
// 1/2 sigma (g_i + g_i+1) - |sigma + psi(gamma)| alpha, Harten's switch theta = max of
// ((|a_hi| - |a_lo|) / (|a_hi| + |a_lo| + eps))^2 over the two pairs, and F = 1/2 REV
// (kappa theta phi), eps_TVD = 1e-8.  A half-point's jumps serve three interfaces, so they are
// formed once (tvd_half) and the interface combines three of them (tvd_iface).

// Jumps and averages (u_n, u_t1, u_t2, a, rho) of the half-point between lo and hi.
template <typename T>
__device__ __forceinline__ void tvd_half(const TvdPt<T>& lo, const TvdPt<T>& hi, T gm, T (&al)[5], T (&av)[5]) {
  const T g1 = gm - L_(1.0);
  const T c1 = L_(0.35355339059327373), c2 = L_(0.70710678118654746);
  const T u0 = L_(0.5) * (lo.u[0] + hi.u[0]), u1 = L_(0.5) * (lo.u[1] + hi.u[1]), u2 = L_(0.5) * (lo.u[2] + hi.u[2]);
  const T a = L_(0.5) * (lo.a + hi.a), rho = L_(0.5) * (lo.r + hi.r);
  const T ia = L_(1.0) / a, ir = L_(1.0) / rho, ia2 = ia * ia;
  const T q0 = u0 * u0, q1 = u1 * u1, q2 = u2 * u2;
  const T L00 = -L_(0.5) * (L_(-2.0) - q0 * ia2 - q1 * ia2 - q2 * ia2 + q0 * ia2 * gm + q1 * ia2 * gm + q2 * ia2 * gm);
  const T L01 = ia2 * g1 * u0, L02 = ia2 * g1 * u1, L03 = ia2 * g1 * u2, L04 = -ia2 * g1;
  const T kq = -q0 * ia - q1 * ia - q2 * ia + q0 * gm * ia + q1 * gm * ia + q2 * gm * ia;
  const T L30 = c1 * (L_(-2.0) * u0 + kq) * ir, L40 = c1 * (L_(2.0) * u0 + kq) * ir;
  const T L31 = -c2 * (L_(-1.0) - u0 * ia + gm * u0 * ia) * ir, L41 = -c2 * (L_(1.0) - u0 * ia + gm * u0 * ia) * ir;
  const T L32 = -c2 * g1 * u1 * ia * ir, L33 = -c2 * g1 * u2 * ia * ir, L34 = c2 * g1 * ia * ir;
  const T dr = -lo.r + hi.r, d0 = -lo.m[0] + hi.m[0], d1 = -lo.m[1] + hi.m[1], d2 = -lo.m[2] + hi.m[2],
          de = -lo.e + hi.e;
  al[0] = dr * L00 + de * L04 + d0 * L01 + d1 * L02 + d2 * L03;
  al[1] = dr * (-u2 * ir) + d2 * ir;
  al[2] = dr * (u1 * ir) + d1 * (-ir);
  al[3] = dr * L30 + de * L34 + d0 * L31 + d1 * L32 + d2 * L33;
  al[4] = dr * L40 + de * L34 + d0 * L41 + d1 * L32 + d2 * L33;
  av[0] = u0;
  av[1] = u1;
  av[2] = u2;
  av[3] = a;
  av[4] = rho;
}

// Interface flux from the jumps of the half-points below (a0), at (a1) and above (a2) it and
// the averages at it.
template <typename T>
__device__ __forceinline__ void tvd_iface(const T* a0, const T* a1, const T* a2, const T* av, T gm, T kappa,
                                          T (&fh)[5]) {
  const T g1 = gm - L_(1.0), eps = L_(1.0e-8), c2 = L_(0.70710678118654746);
  const T u0 = av[0], u1 = av[1], u2 = av[2], a = av[3], rho = av[4];
  const T ia = L_(1.0) / a;
  const T q0 = u0 * u0, q1 = u1 * u1, q2 = u2 * u2;
  const T ws0 = u0, wsp = a + u0, wsm = -a + u0;
  const T R03 = c2 * rho * ia, R13 = c2 * (a + u0) * rho * ia, R14 = c2 * (-a + u0) * rho * ia;
  const T R23 = c2 * rho * u1 * ia, R33 = c2 * rho * u2 * ia;
  const T R40 = L_(0.5) * q0 + L_(0.5) * q1 + L_(0.5) * q2;
  const T hq = (a * a + L_(0.5) * g1 * (q0 + q1 + q2)) / g1;
  const T R43 = c2 * (hq + a * u0) * rho * ia, R44 = c2 * (hq - a * u0) * rho * ia;
  T ps[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const T s0 = tvd_psi<T>(k < 3 ? ws0 : (k == 3 ? wsp : wsm));
    const T b0 = a0[k], b1 = a1[k], b2 = a2[k];
    const T g0 = tvd_g<T>(b1, b0), gg = tvd_g<T>(b2, b1);
    const T gam = b1 == L_(0.0) ? L_(0.0) : (-g0 + gg) * b1 * s0 / (b1 * b1 + eps);
    const T phi = -fabs(s0 + tvd_psi<T>(gam)) * b1 + L_(0.5) * (g0 + gg) * s0;
    // Harten's switch: the larger of |x0| / y0 and |x1| / y1, squared, with one division
    const T x0 = fabs(-fabs(b0) + fabs(b1)), y0 = fabs(b0) + fabs(b1) + eps;
    const T x1 = fabs(-fabs(b1) + fabs(b2)), y1 = fabs(b1) + fabs(b2) + eps;
    const T th = fmax(x0 * y1, x1 * y0) / (y0 * y1);
    ps[k] = kappa * phi * (th * th);
  }
  fh[0] = L_(0.5) * ps[0] + L_(0.5) * R03 * ps[3] + L_(0.5) * R03 * ps[4];
  fh[1] = L_(0.5) * u0 * ps[0] + L_(0.5) * R13 * ps[3] + L_(0.5) * R14 * ps[4];
  fh[2] = L_(0.5) * u1 * ps[0] + L_(0.5) * (-rho) * ps[2] + L_(0.5) * R23 * ps[3] + L_(0.5) * R23 * ps[4];
  fh[3] = L_(0.5) * u2 * ps[0] + L_(0.5) * rho * ps[1] + L_(0.5) * R33 * ps[3] + L_(0.5) * R33 * ps[4];
  fh[4] = L_(0.5) * R40 * ps[0] + L_(0.5) * (rho * u2) * ps[1] + L_(0.5) * (-rho * u1) * ps[2] + L_(0.5) * R43 * ps[3] +
          L_(0.5) * R44 * ps[4];
}

// Face d of the point -2 velocities: the two other directions e1 < e2, index x_e1 + n_e1 x_e2.
__device__ __forceinline__ void tvd_face_dirs(int d, int& e1, int& e2) {
  e1 = d == 0 ? 1 : 0;
  e2 = d == 2 ? 1 : 2;
}

// u = rhou / rho at index -2 of each direction (the other two interior), from the state the
// last RK stage reads: the value its constituent relations leave there, which the generated
// filter reads at that point.  snap[(3 d + c) * fmax + face index].
template <typename T>
__global__ void k_tvd_stale(BlockK b, T* __restrict__ snap, int fmax) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < 3 * fmax; t += gridDim.x * blockDim.x) {
    const int d = t / fmax, f = t - d * fmax;
    int e1, e2;
    tvd_face_dirs(d, e1, e2);
    if (f >= b.n[e1] * b.n[e2]) continue;
    int c[3];
    c[d] = -2;
    c[e1] = f % b.n[e1];
    c[e2] = f / b.n[e1];
    const int id = lin(b, c[0], c[1], c[2]);
    const T r = ld_q<T>(b, 0, id);
#pragma unroll
    for (int k = 0; k < 3; ++k) snap[(size_t)(3 * d + k) * fmax + f] = ld_q<T>(b, 1 + k, id) / r;
  }
}

// Tile of the TVD flux kernel: TA interfaces along D times TB lines, (TA + 2) TB half-points
// (256: one per thread).  Along x (D = 0) a warp covers consecutive points of a row; along y
// and z it covers 32 consecutive x of the lines, so the state loads and flux stores are
// coalesced either way.
constexpr int TVD_TH = 256;
template <int D>
struct TvdTile {
  static constexpr int TA = D == 0 ? 62 : 8;  // interfaces along D (x: 4 lines of 64 half-points)
  static constexpr int TB = TVD_TH / TA;      // lines
  static constexpr int NH = (TA + 2) * TB;    // half-points
  static constexpr int REC = 11;              // 5 jumps + 5 averages, odd stride
};

// State of point p (index cD along D) in the local frame, u and a as the filter's
// constituent-relation kernel forms them (u = rhou (1/rho), a = sqrt(gama p (1/rho))); at
// index -2 the velocities of the stage snapshot and a = 0, as in the generated solver.
template <typename T, int D>
__device__ __forceinline__ void tvd_point(const BlockK& b, int p, bool stale, const T* __restrict__ snap, int fmax,
                                          int f, T gm, TvdPt<T>& q) {
  constexpr int T1 = (D + 1) % 3, T2 = (D + 2) % 3;
  q.r = ld_q<T>(b, 0, p);
  q.e = ld_q<T>(b, 4, p);
  const T mg[3] = {ld_q<T>(b, 1, p), ld_q<T>(b, 2, p), ld_q<T>(b, 3, p)};
  q.m[0] = mg[D];
  q.m[1] = mg[T1];
  q.m[2] = mg[T2];
  if (stale) {
    q.u[0] = snap[(size_t)(3 * D + D) * fmax + f];
    q.u[1] = snap[(size_t)(3 * D + T1) * fmax + f];
    q.u[2] = snap[(size_t)(3 * D + T2) * fmax + f];
    q.a = L_(0.0);
  } else {
    const T ir = L_(1.0) / q.r;
    q.u[0] = q.m[0] * ir;
    q.u[1] = q.m[1] * ir;
    q.u[2] = q.m[2] * ir;
    const T pr =
        (gm - L_(1.0)) * (-(L_(0.5) * (mg[0] * mg[0]) + L_(0.5) * (mg[1] * mg[1]) + L_(0.5) * (mg[2] * mg[2])) * ir + q.e);
    q.a = sqrt(gm * pr * ir);
  }
}

// TVD filter fluxes along D at interfaces i+1/2, i = -1..N-1, transverse interior; F[v] at the
// index of point i.  Phase 1: every half-point j = i0-1 .. i0+TA of the tile's lines (the
// points j, j+1) into shared memory; phase 2: one thread per interface.
template <typename T, int D>
__global__ void __launch_bounds__(TVD_TH) k_tvd_flux(BlockK b, T gm, T kappa, const T* __restrict__ snap, int fmax,
                                                    T* F0, T* F1, T* F2, T* F3, T* F4) {
  using TT = TvdTile<D>;
  constexpr int TA = TT::TA, TB = TT::TB, REC = TT::REC;
  constexpr int T1 = (D + 1) % 3, T2 = (D + 2) % 3;
  __shared__ T sm[TT::NH * REC];
  int e1, e2;
  tvd_face_dirs(D, e1, e2);
  const int N = b.n[D];
  const int i0 = (int)blockIdx.y * TA - 1;  // first interface of the tile
  const int s = b.st[D];
  // the tile's line `line` -> transverse coordinates (c[e1], c[e2]); false outside the block
  auto line_coords = [&](int line, int (&c)[3]) -> bool {
    if (D == 0) {
      const long L = (long)blockIdx.x * TB + line;
      c[1] = (int)(L % b.n[1]);
      c[2] = (int)(L / b.n[1]);
      return L < (long)b.n[1] * b.n[2];
    }
    c[0] = (int)blockIdx.x * TB + line;
    c[D == 1 ? 2 : 1] = (int)blockIdx.z;
    return c[0] < b.n[0];
  };
  for (int hs = threadIdx.x; hs < TT::NH; hs += TVD_TH) {
    const int line = D == 0 ? hs / (TA + 2) : hs % TB;
    const int a = D == 0 ? hs % (TA + 2) : hs / TB;
    const int j = i0 - 1 + a;  // half-point between points j and j+1
    int c[3];
    if (!line_coords(line, c) || j > N) continue;  // beyond the last interface's needs
    c[D] = j;
    const int p = lin(b, c[0], c[1], c[2]);
    const int f = c[e1] + b.n[e1] * c[e2];
    TvdPt<T> lo, hi;
    tvd_point<T, D>(b, p, j == -2, snap, fmax, f, gm, lo);
    tvd_point<T, D>(b, p + s, false, snap, fmax, f, gm, hi);
    T al[5], av[5];
    tvd_half<T>(lo, hi, gm, al, av);
    T* r = sm + (line * (TA + 2) + a) * REC;
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      r[k] = al[k];
      r[5 + k] = av[k];
    }
  }
  __syncthreads();
  const int t = threadIdx.x;
  if (t >= TA * TB) return;  // x tiles: 248 interfaces for 256 threads
  const int line = D == 0 ? t / TA : t % TB;
  const int a = D == 0 ? t % TA : t / TB;
  const int i = i0 + a;
  int c[3];
  if (!line_coords(line, c) || i > N - 1) return;
  c[D] = i;
  const int id = lin(b, c[0], c[1], c[2]);
  const T* r = sm + (line * (TA + 2) + a) * REC;
  T fh[5];
  tvd_iface<T>(r, r + REC, r + 2 * REC, r + REC + 5, gm, kappa, fh);
  T* F[5] = {F0, F1, F2, F3, F4};
  F[0][id] = fh[0];
  F[1 + D][id] = fh[1];
  F[1 + T1][id] = fh[2];
  F[1 + T2][id] = fh[3];
  F[4][id] = fh[4];
}

// q += dt * mask * (-(F_0(i) - F_0(i-1)) / Delta_0 - (F_2 ...) / Delta_2 - (F_1 ...) / Delta_1)
// on the interior, in the generated operation order (kernel 049); without kappa (TVD filter)
// the mask is 1.  FP32: the increment is
// formed in FP32 and added to the FP64 state; the FP32 copy of a changed point is refreshed.
template <typename T>
struct FilterFluxes {
  const T* f[15];  // direction-major: F_d of variable v at f[5 d + v]
};

template <typename T>
__global__ void k_filter_apply(BlockK b, const T* __restrict__ kappa, FilterFluxes<T> F, double dt, T select) {
  const int n0 = b.n[0], n1 = b.n[1], n2 = b.n[2];
  const int total = n0 * n1 * n2;
  const int sx = b.st[0], sy = b.st[1], sz = b.st[2];
  const T i0 = inv_delta<T>(b, 0), i1 = inv_delta<T>(b, 1), i2 = inv_delta<T>(b, 2);
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    const int x = t % n0, y = (t / n0) % n1, z = t / (n0 * n1);
    const int c = lin(b, x, y, z);
    if (kappa) {
      T km = kappa[c];
      km = fmax(km, kappa[c + sz]);
      km = fmax(km, kappa[c + 2 * sy]);
      km = fmax(km, kappa[c + sx]);
      km = fmax(km, kappa[c - sy]);
      km = fmax(km, kappa[c - sx]);
      km = fmax(km, kappa[c + sy]);
      km = fmax(km, kappa[c + 2 * sz]);
      km = fmax(km, kappa[c + 2 * sx]);
      km = fmax(km, kappa[c - sz]);
      if (!(km >= select)) continue;  // mask 0: the state is unchanged
    }
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const T* f0 = F.f[v];
      const T* f1 = F.f[5 + v];
      const T* f2 = F.f[10 + v];
      const T inc = -(-f0[c - sx] + f0[c]) * i0 - (-f2[c - sz] + f2[c]) * i2 - (-f1[c - sy] + f1[c]) * i1;
      if constexpr (sizeof(T) == 8) {
        b.q[v][c] = inc * dt * 1.0 + b.q[v][c];
      } else {
        const double q = __fma_rn(dt, f2d_exact(inc), b.q[v][c]);
        b.q[v][c] = q;
        b.qf[v][c] = d2f_rn(q);
      }
    }
  }
}

// Largest face of a block (the point -2 velocity snapshot of the TVD filter holds 9 of them in
// the first workspace slot: 9 n_a n_b <= (n_a + 10)(n_b + 10)(n_c + 10), the slot's size).
inline int tvd_fmax(const BlockK& k) {
  return std::max(k.n[1] * k.n[2], std::max(k.n[0] * k.n[2], k.n[0] * k.n[1]));
}

// The TVD filter: its exchange, then per direction the fluxes, then the update (no mask).
template <typename T>
int tvd_filter_t(osb_ctx* c, Block& bl, double dt) {
  BlockK& k = bl.k;
  const long n = (long)k.n[0] * k.n[1] * k.n[2];
  T* base = reinterpret_cast<T*>(bl.filt_ws);
  const T* snap = base;
  T* F[15];
  for (int a = 0; a < 15; ++a) F[a] = base + (size_t)(1 + a) * k.alloc;
  const int fields = sizeof(T) == 8 ? 1 : 2;
  const int fmax = tvd_fmax(k);
  timing_begin(c, FAM_FILTER);
  for (int d = 0; d < 3; ++d) {
    long per = 8L * (d == 0 ? 1 : k.n[0]) * (d == 1 ? 1 : k.n[1]) * (d == 2 ? 1 : k.n[2]);
    k_filter_halo<<<grid_for(c, per, FT), FT, 0, c->stream>>>(k, d, fields);
  }
  const T gm = (T)bl.d.gama, kap = (T)bl.d.tvd_kappa;
  // grids: D = 0 (lines of y, z) x (x tiles); D = 1, 2 (x tiles) x (tiles along D) x (the other)
  const dim3 g0((unsigned)(((long)k.n[1] * k.n[2] + TvdTile<0>::TB - 1) / TvdTile<0>::TB),
                (unsigned)((k.n[0] + 1 + TvdTile<0>::TA - 1) / TvdTile<0>::TA));
  const dim3 g1((unsigned)((k.n[0] + TvdTile<1>::TB - 1) / TvdTile<1>::TB),
                (unsigned)((k.n[1] + 1 + TvdTile<1>::TA - 1) / TvdTile<1>::TA), (unsigned)k.n[2]);
  const dim3 g2((unsigned)((k.n[0] + TvdTile<2>::TB - 1) / TvdTile<2>::TB),
                (unsigned)((k.n[2] + 1 + TvdTile<2>::TA - 1) / TvdTile<2>::TA), (unsigned)k.n[1]);
  k_tvd_flux<T, 0><<<g0, TVD_TH, 0, c->stream>>>(k, gm, kap, snap, fmax, F[0], F[1], F[2], F[3], F[4]);
  k_tvd_flux<T, 1><<<g1, TVD_TH, 0, c->stream>>>(k, gm, kap, snap, fmax, F[5], F[6], F[7], F[8], F[9]);
  k_tvd_flux<T, 2><<<g2, TVD_TH, 0, c->stream>>>(k, gm, kap, snap, fmax, F[10], F[11], F[12], F[13], F[14]);
  FilterFluxes<T> Fd;
  for (int a = 0; a < 15; ++a) Fd.f[a] = F[a];
  k_filter_apply<T><<<grid_for(c, n, FT), FT, 0, c->stream>>>(k, nullptr, Fd, dt, (T)0);
  timing_end(c);
  c->launches += 7;
  return OSB_OK;
}

template <typename T>
int tvd_stale_t(osb_ctx* c, Block& bl) {
  const int fmax = tvd_fmax(bl.k);
  k_tvd_stale<T><<<grid_for(c, 3L * fmax, FT), FT, 0, c->stream>>>(bl.k, reinterpret_cast<T*>(bl.filt_ws), fmax);
  c->launches++;
  return OSB_OK;
}

template <typename T>
int filter_t(osb_ctx* c, Block& bl, double dt) {
  if (bl.d.filter == OSB_FILTER_TVD) return tvd_filter_t<T>(c, bl, dt);
  BlockK& k = bl.k;
  const long n = (long)k.n[0] * k.n[1] * k.n[2];
  T* base = reinterpret_cast<T*>(bl.filt_ws);
  T* kappa = base;
  T* F[15];
  for (int a = 0; a < 15; ++a) F[a] = base + (size_t)(1 + a) * k.alloc;
  const int fields = sizeof(T) == 8 ? 1 : 2;
  timing_begin(c, FAM_FILTER);
  if (sizeof(T) == 4) {
    const int D = bl.d.bc_depth[0][0] > 0 ? bl.d.bc_depth[0][0] : 4;
    const float* prev = c->qf_parity ? bl.qf_base : bl.qf_alt;
    const long shell = (long)(k.n[0] + 2 * D) * (k.n[1] + 2 * D) * (k.n[2] + 2 * D);
    k_shell_from<<<grid_for(c, shell, FT), FT, 0, c->stream>>>(k, prev, D);
    c->launches++;
  }
  for (int d = 0; d < 3; ++d) {
    long per = 8L * (d == 0 ? 1 : k.n[0]) * (d == 1 ? 1 : k.n[1]) * (d == 2 ? 1 : k.n[2]);
    k_filter_halo<<<grid_for(c, per, FT), FT, 0, c->stream>>>(k, d, fields);
  }
  const double h = sqrt(bl.d.delta[0] * bl.d.delta[0] + bl.d.delta[1] * bl.d.delta[1] + bl.d.delta[2] * bl.d.delta[2]);
  k_ducros<T><<<grid_for(c, n, FT), FT, 0, c->stream>>>(k, kappa, (T)(1.0 / h));
  SchemeParams sp = scheme_params(bl.d.gama, bl.d.eps, bl.d.teno_ct, bl.d.shock_filter_control, 1e-12);
  const T check = (T)bl.d.ducros_check;
  const long nf0 = (long)(k.n[0] + 1) * k.n[1] * k.n[2], nf1 = (long)k.n[0] * (k.n[1] + 1) * k.n[2],
             nf2 = (long)k.n[0] * k.n[1] * (k.n[2] + 1);
  k_filter_flux<T, 0><<<grid_for(c, nf0, FT), FT, 0, c->stream>>>(k, sp, kappa, check, F[0], F[1], F[2], F[3], F[4]);
  k_filter_flux<T, 1><<<grid_for(c, nf1, FT), FT, 0, c->stream>>>(k, sp, kappa, check, F[5], F[6], F[7], F[8], F[9]);
  k_filter_flux<T, 2><<<grid_for(c, nf2, FT), FT, 0, c->stream>>>(k, sp, kappa, check, F[10], F[11], F[12], F[13],
                                                                   F[14]);
  FilterFluxes<T> Fd;
  for (int a = 0; a < 15; ++a) Fd.f[a] = F[a];
  k_filter_apply<T><<<grid_for(c, n, FT), FT, 0, c->stream>>>(k, kappa, Fd, dt, (T)bl.d.ducros_select);
  timing_end(c);
  c->launches += 8;
  return OSB_OK;
}

}  // namespace

int OSB_FILTER_NAME(osb_ctx* c, Block& bl, double dt) { return filter_t<OSB_FILTER_T>(c, bl, dt); }
int OSB_TVD_STALE_NAME(osb_ctx* c, Block& bl) { return tvd_stale_t<OSB_FILTER_T>(c, bl); }

}  // namespace osb
