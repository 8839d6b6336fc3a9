// osb_math.cuh -- device numerics of the residual path (characteristic LLF WENO/TENO flux,
// central-4 operators), templated on the arithmetic type T (double: FP64 path, float: FP32
// residual path).
//
// Everything is written in the local frame of the sweep direction: the conserved state of a
// point is (rho, m_n, m_t1[, m_t2], E) with m_n the momentum along the sweep.  For a Cartesian
// direction the eigensystem of physical_models/euler_eigensystem.py:53-166 with k = e_d is the
// k = e_0 system with the momentum components permuted (a cyclic permutation in 3D, a swap in
// 2D, which only flips the sign of one vorticity eigenvector); the characteristic flux is
// invariant under those relabelings, so one set of formulas serves every direction.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace osb {

enum { SCH_WENO5_JS = 1, SCH_WENO5_Z = 2, SCH_TENO5 = 3, SCH_TENO6 = 4, SCH_CENTRAL4 = 5 };
enum { AVG_SIMPLE = 0, AVG_ROE = 1 };

template <typename T> struct Lit;
template <> struct Lit<double> {
  static __device__ __forceinline__ double c(double x) { return x; }
};
template <> struct Lit<float> {
  static __device__ __forceinline__ float c(double x) { return (float)x; }
};
#define L_(x) Lit<T>::c(x)

struct SchemeParams {
  double gama;
  double teno_eps;   // TENO epsilon (reference value 1e-40)
  double teno_ct;    // TENO cut-off
  double sfc;        // shock_filter_control
  double eps32_rel;  // FP32 path: epsilon relative to the stencil's mean square
  // the same constants rounded to FP32 on the host (scheme_params): an FP32 kernel that
  // converted the doubles itself would run the conversions on the FP64 pipe, and under the
  // sweeps' register cap the compiler re-derives such values inside the loop instead of
  // keeping them in registers (measured: six FP64-pipe conversions per point in the FP32 y/z
  // sweeps, 34 % FP64-pipe activity)
  float gama_f, g1_f, teno_eps_f, teno_ct_f, sfc_f, eps32_rel_f;
};

__host__ __device__ inline SchemeParams scheme_params(double gama, double teno_eps, double teno_ct, double sfc,
                                                      double eps32_rel) {
  SchemeParams p;
  p.gama = gama;
  p.teno_eps = teno_eps;
  p.teno_ct = teno_ct;
  p.sfc = sfc;
  p.eps32_rel = eps32_rel;
  p.gama_f = (float)gama;
  p.g1_f = (float)(gama - 1.0);
  p.teno_eps_f = (float)teno_eps;
  p.teno_ct_f = (float)teno_ct;
  p.sfc_f = (float)sfc;
  p.eps32_rel_f = (float)eps32_rel;
  return p;
}

// The constants in the arithmetic type of a kernel.
template <typename T>
struct SP;
template <>
struct SP<double> {
  double gama, g1, teno_eps, teno_ct, sfc, eps32_rel;
  __device__ __forceinline__ explicit SP(const SchemeParams& p)
      : gama(p.gama), g1(p.gama - 1.0), teno_eps(p.teno_eps), teno_ct(p.teno_ct), sfc(p.sfc),
        eps32_rel(p.eps32_rel) {}
};
template <>
struct SP<float> {
  float gama, g1, teno_eps, teno_ct, sfc, eps32_rel;
  __device__ __forceinline__ explicit SP(const SchemeParams& p)
      : gama(p.gama_f), g1(p.g1_f), teno_eps(p.teno_eps_f), teno_ct(p.teno_ct_f), sfc(p.sfc_f),
        eps32_rel(p.eps32_rel_f) {}
};

// ---------------------------------------------------------------------------------------
// Fifth-order reconstruction at the right face of f2 from f0..f4 (offsets -2..+2).
//   WENO5-JS / WENO5-Z: weno.py:71-121 (ENO coefficients, optimal weights 3/10, 3/5, 1/10),
//     139-206 (Jiang-Shu smoothness), 290-376 (JS alpha = d/(1e-6+b)^2; Z alpha =
//     d(1+(|b0-b2|/(1e-40+b))^2)).
//   TENO5: teno.py:96-217, 419-477 (stencils [-1,0,1],[0,1,2],[-2,-1,0], weights 11/20, 4/10,
//     1/20, tau = |b0-b2|, alpha = (1+tau/(eps+b))^6, cut-off alpha/sum < C_T).
// In the FP32 path the epsilon of WENO-Z / TENO (1e-40, below the FP32 normal range) is
// replaced by eps32_rel * mean(f^2) + 1e-30, and TENO's alpha ratios are formed from
// t_r/t_max so that (1+tau/(eps+b))^6 cannot overflow.
template <typename T, int SCH>
__device__ __forceinline__ T recon5(T fm2, T fm1, T f0, T fp1, T fp2, const SP<T>& sp) {
  constexpr bool F32 = sizeof(T) == 4;
  if (SCH == SCH_TENO5) {
    T s0 = fm1 - fp1, c0 = fm1 - L_(2.0) * f0 + fp1;
    T s1 = L_(3.0) * f0 - L_(4.0) * fp1 + fp2, c1 = f0 - L_(2.0) * fp1 + fp2;
    T s2 = fm2 - L_(4.0) * fm1 + L_(3.0) * f0, c2 = fm2 - L_(2.0) * fm1 + f0;
    T b0 = L_(0.25) * s0 * s0 + L_(13.0 / 12.0) * c0 * c0;
    T b1 = L_(0.25) * s1 * s1 + L_(13.0 / 12.0) * c1 * c1;
    T b2 = L_(0.25) * s2 * s2 + L_(13.0 / 12.0) * c2 * c2;
    T tau = fabs(b0 - b2);
    T d0, d1, d2;
    if (F32) {
      T eps = sp.eps32_rel * (fm2 * fm2 + fm1 * fm1 + f0 * f0 + fp1 * fp1 + fp2 * fp2) * L_(0.2) + L_(1e-30);
      T t0 = L_(1.0) + tau / (eps + b0), t1 = L_(1.0) + tau / (eps + b1), t2 = L_(1.0) + tau / (eps + b2);
      T tm = fmax(t0, fmax(t1, t2));
      T r0 = t0 / tm, r1 = t1 / tm, r2 = t2 / tm;
      r0 = r0 * r0 * r0; r0 = r0 * r0;
      r1 = r1 * r1 * r1; r1 = r1 * r1;
      r2 = r2 * r2 * r2; r2 = r2 * r2;
      // alpha_r / sum < C_T  <=>  alpha_r < C_T * sum (sum > 0)
      const T cs = sp.teno_ct * (r0 + r1 + r2);
      d0 = (r0 < cs) ? L_(0.0) : L_(1.0);
      d1 = (r1 < cs) ? L_(0.0) : L_(1.0);
      d2 = (r2 < cs) ? L_(0.0) : L_(1.0);
    } else {
      T eps = sp.teno_eps;
      T t0 = L_(1.0) + tau / (eps + b0), t1 = L_(1.0) + tau / (eps + b1), t2 = L_(1.0) + tau / (eps + b2);
      T a0 = t0 * t0 * t0 * t0 * t0 * t0;
      T a1 = t1 * t1 * t1 * t1 * t1 * t1;
      T a2 = t2 * t2 * t2 * t2 * t2 * t2;
      T inv = L_(1.0) / (a0 + a1 + a2);
      T ct = sp.teno_ct;
      d0 = (a0 * inv < ct) ? L_(0.0) : L_(1.0);
      d1 = (a1 * inv < ct) ? L_(0.0) : L_(1.0);
      d2 = (a2 * inv < ct) ? L_(0.0) : L_(1.0);
    }
    T w0 = L_(11.0 / 20.0) * d0, w1 = L_(4.0 / 10.0) * d1, w2 = L_(1.0 / 20.0) * d2;
    T iw = L_(1.0) / (w0 + w1 + w2);
    T e0 = -L_(1.0 / 6.0) * fm1 + L_(5.0 / 6.0) * f0 + L_(2.0 / 6.0) * fp1;
    T e1 = L_(2.0 / 6.0) * f0 + L_(5.0 / 6.0) * fp1 - L_(1.0 / 6.0) * fp2;
    T e2 = L_(2.0 / 6.0) * fm2 - L_(7.0 / 6.0) * fm1 + L_(11.0 / 6.0) * f0;
    return (w0 * e0 + w1 * e1 + w2 * e2) * iw;
  } else {
    T c0 = f0 - L_(2.0) * fp1 + fp2, s0 = L_(3.0) * f0 - L_(4.0) * fp1 + fp2;
    T c1 = fm1 - L_(2.0) * f0 + fp1, s1 = fm1 - fp1;
    T c2 = fm2 - L_(2.0) * fm1 + f0, s2 = fm2 - L_(4.0) * fm1 + L_(3.0) * f0;
    T b0 = L_(13.0 / 12.0) * c0 * c0 + L_(0.25) * s0 * s0;
    T b1 = L_(13.0 / 12.0) * c1 * c1 + L_(0.25) * s1 * s1;
    T b2 = L_(13.0 / 12.0) * c2 * c2 + L_(0.25) * s2 * s2;
    T a0, a1, a2;
    if (SCH == SCH_WENO5_Z) {
      T eps = F32 ? sp.eps32_rel * (fm2 * fm2 + fm1 * fm1 + f0 * f0 + fp1 * fp1 + fp2 * fp2) * L_(0.2) + L_(1e-30)
                  : L_(1.0e-40);
      T tau = fabs(b0 - b2);
      T r0 = tau / (eps + b0), r1 = tau / (eps + b1), r2 = tau / (eps + b2);
      a0 = L_(0.3) * (L_(1.0) + r0 * r0);
      a1 = L_(0.6) * (L_(1.0) + r1 * r1);
      a2 = L_(0.1) * (L_(1.0) + r2 * r2);
    } else {
      T eps = L_(1.0e-6);
      a0 = L_(0.3) / ((eps + b0) * (eps + b0));
      a1 = L_(0.6) / ((eps + b1) * (eps + b1));
      a2 = L_(0.1) / ((eps + b2) * (eps + b2));
    }
    T inv = L_(1.0) / (a0 + a1 + a2);
    T e0 = L_(1.0 / 3.0) * f0 + L_(5.0 / 6.0) * fp1 - L_(1.0 / 6.0) * fp2;
    T e1 = -L_(1.0 / 6.0) * fm1 + L_(5.0 / 6.0) * f0 + L_(1.0 / 3.0) * fp1;
    T e2 = L_(1.0 / 3.0) * fm2 - L_(7.0 / 6.0) * fm1 + L_(11.0 / 6.0) * f0;
    return (a0 * inv) * e0 + (a1 * inv) * e1 + (a2 * inv) * e2;
  }
}

// Sixth-order TENO at the interface i+1/2 from six points f0..f5 = i-2..i+3 (teno.py:59-194 for
// sides +1 / -1, 220-240 tau_6 = |b3 - (b0 + b2 - 4 b1)/6|, 419-477 cut-off and weights with
// optimal weights 231/500, 3/10, 27/500, 23/125).  Side +1 reconstructs the positive split
// flux, side -1 the negative one.  The reference's side +1 fourth smoothness indicator has its
// 781/720 term unsquared (teno.py:160-161, squared on side -1), and so does this: its generated
// solvers compute it that way.  The FP32 path uses the rescaled epsilon of recon5 and forms
// the cut-off from t_r / max|t|.
template <typename T, int SIDE>
__device__ __forceinline__ T recon6(T fm2, T fm1, T f0, T fp1, T fp2, T fp3, const SP<T>& sp) {
  constexpr bool F32 = sizeof(T) == 4;
  T b0, b1, b2, b3, e0, e1, e2, e3;
  if (SIDE > 0) {
    T s0 = fm1 - fp1, c0 = fm1 - L_(2.0) * f0 + fp1;
    T s1 = L_(3.0) * f0 - L_(4.0) * fp1 + fp2, c1 = f0 - L_(2.0) * fp1 + fp2;
    T s2 = fm2 - L_(4.0) * fm1 + L_(3.0) * f0, c2 = fm2 - L_(2.0) * fm1 + f0;
    b0 = L_(0.25) * s0 * s0 + L_(13.0 / 12.0) * c0 * c0;
    b1 = L_(0.25) * s1 * s1 + L_(13.0 / 12.0) * c1 * c1;
    b2 = L_(0.25) * s2 * s2 + L_(13.0 / 12.0) * c2 * c2;
    T u1 = -L_(11.0) * f0 + L_(18.0) * fp1 - L_(9.0) * fp2 + L_(2.0) * fp3;
    T u2 = L_(2.0) * f0 - L_(5.0) * fp1 + L_(4.0) * fp2 - fp3;
    T u3 = -f0 + L_(3.0) * fp1 - L_(3.0) * fp2 + fp3;
    b3 = L_(1.0 / 36.0) * u1 * u1 + L_(13.0 / 12.0) * u2 * u2 + L_(781.0 / 720.0) * u3;
    e0 = -L_(1.0 / 6.0) * fm1 + L_(5.0 / 6.0) * f0 + L_(2.0 / 6.0) * fp1;
    e1 = L_(2.0 / 6.0) * f0 + L_(5.0 / 6.0) * fp1 - L_(1.0 / 6.0) * fp2;
    e2 = L_(2.0 / 6.0) * fm2 - L_(7.0 / 6.0) * fm1 + L_(11.0 / 6.0) * f0;
    e3 = L_(3.0 / 12.0) * f0 + L_(13.0 / 12.0) * fp1 - L_(5.0 / 12.0) * fp2 + L_(1.0 / 12.0) * fp3;
  } else {
    T s0 = f0 - fp2, c0 = f0 - L_(2.0) * fp1 + fp2;
    T s1 = fm1 - L_(4.0) * f0 + L_(3.0) * fp1, c1 = fm1 - L_(2.0) * f0 + fp1;
    T s2 = L_(3.0) * fp1 - L_(4.0) * fp2 + fp3, c2 = fp1 - L_(2.0) * fp2 + fp3;
    b0 = L_(0.25) * s0 * s0 + L_(13.0 / 12.0) * c0 * c0;
    b1 = L_(0.25) * s1 * s1 + L_(13.0 / 12.0) * c1 * c1;
    b2 = L_(0.25) * s2 * s2 + L_(13.0 / 12.0) * c2 * c2;
    T u1 = -L_(2.0) * fm2 + L_(9.0) * fm1 - L_(18.0) * f0 + L_(11.0) * fp1;
    T u2 = -fm2 + L_(4.0) * fm1 - L_(5.0) * f0 + L_(2.0) * fp1;
    T u3 = -fm2 + L_(3.0) * fm1 - L_(3.0) * f0 + fp1;
    b3 = L_(1.0 / 36.0) * u1 * u1 + L_(13.0 / 12.0) * u2 * u2 + L_(781.0 / 720.0) * u3 * u3;
    e0 = L_(2.0 / 6.0) * f0 + L_(5.0 / 6.0) * fp1 - L_(1.0 / 6.0) * fp2;
    e1 = -L_(1.0 / 6.0) * fm1 + L_(5.0 / 6.0) * f0 + L_(2.0 / 6.0) * fp1;
    e2 = L_(11.0 / 6.0) * fp1 - L_(7.0 / 6.0) * fp2 + L_(1.0 / 3.0) * fp3;
    e3 = L_(1.0 / 12.0) * fm2 - L_(5.0 / 12.0) * fm1 + L_(13.0 / 12.0) * f0 + L_(3.0 / 12.0) * fp1;
  }
  const T tau = fabs(b3 - L_(1.0 / 6.0) * (b0 + b2 - L_(4.0) * b1));
  T a0, a1, a2, a3;
  if (F32) {
    T eps = sp.eps32_rel * (fm2 * fm2 + fm1 * fm1 + f0 * f0 + fp1 * fp1 + fp2 * fp2 + fp3 * fp3) * L_(1.0 / 6.0) +
            L_(1e-30);
    T t0 = L_(1.0) + tau / (eps + b0), t1 = L_(1.0) + tau / (eps + b1), t2 = L_(1.0) + tau / (eps + b2),
      t3 = L_(1.0) + tau / (eps + b3);
    T im = L_(1.0) / fmax(fmax(fabs(t0), fabs(t1)), fmax(fabs(t2), fabs(t3)));
    t0 *= im; t1 *= im; t2 *= im; t3 *= im;
    a0 = t0 * t0 * t0; a0 = a0 * a0;
    a1 = t1 * t1 * t1; a1 = a1 * a1;
    a2 = t2 * t2 * t2; a2 = a2 * a2;
    a3 = t3 * t3 * t3; a3 = a3 * a3;
  } else {
    const T eps = sp.teno_eps;
    T t0 = L_(1.0) + tau / (eps + b0), t1 = L_(1.0) + tau / (eps + b1), t2 = L_(1.0) + tau / (eps + b2),
      t3 = L_(1.0) + tau / (eps + b3);
    a0 = t0 * t0 * t0 * t0 * t0 * t0;
    a1 = t1 * t1 * t1 * t1 * t1 * t1;
    a2 = t2 * t2 * t2 * t2 * t2 * t2;
    a3 = t3 * t3 * t3 * t3 * t3 * t3;
  }
  const T inv = L_(1.0) / (a0 + a1 + a2 + a3);
  const T ct = sp.teno_ct;
  const T w0 = (a0 * inv < ct) ? L_(0.0) : L_(231.0 / 500.0);
  const T w1 = (a1 * inv < ct) ? L_(0.0) : L_(3.0 / 10.0);
  const T w2 = (a2 * inv < ct) ? L_(0.0) : L_(27.0 / 500.0);
  const T w3 = (a3 * inv < ct) ? L_(0.0) : L_(23.0 / 125.0);
  return (w0 * e0 + w1 * e1 + w2 * e2 + w3 * e3) * (L_(1.0) / (w0 + w1 + w2 + w3));
}

// Reconstruction of one characteristic wave at i+1/2 from the positive and negative split
// fluxes at points i-2..i+3.
template <typename T, int SCH>
__device__ __forceinline__ T recon_wave(const T (&fp)[6], const T (&fm)[6], const SP<T>& sp) {
  if (SCH == SCH_TENO6)
    return recon6<T, 1>(fp[0], fp[1], fp[2], fp[3], fp[4], fp[5], sp) +
           recon6<T, -1>(fm[0], fm[1], fm[2], fm[3], fm[4], fm[5], sp);
  return recon5<T, SCH>(fp[0], fp[1], fp[2], fp[3], fp[4], sp) + recon5<T, SCH>(fm[5], fm[4], fm[3], fm[2], fm[1], sp);
}

// Point data carried through a sweep: conserved state in the local frame plus primitives.
template <typename T, int ND>
struct Pt {
  T q[ND + 2];  // rho, m_n, m_t.., E
  T u[ND];      // u_n, u_t..
  T p, a;
};

template <typename T, int ND>
__device__ __forceinline__ void make_pt(Pt<T, ND>& s, T gm) {
  T rho = s.q[0];
  T ir = L_(1.0) / rho;
  T ke = L_(0.0);
#pragma unroll
  for (int i = 0; i < ND; ++i) {
    s.u[i] = s.q[1 + i] * ir;
    ke += s.u[i] * s.u[i];
  }
  s.p = (gm - L_(1.0)) * (s.q[ND + 1] - L_(0.5) * rho * ke);
  s.a = sqrt(gm * s.p * ir);
}

// Characteristic LLF flux at the interface between w[2] and w[3] of a 6-point window
// (offsets -2..+3), local frame.  Restates shock_capturing.py:786-891 and 979-1028 with the
// eigensystems of euler_eigensystem.py for k = e_0.
template <typename T, int ND, int SCH, int AVG>
__device__ __forceinline__ void char_flux(const Pt<T, ND> (&w)[6], const SP<T>& sp, T (&fh)[ND + 2]) {
  constexpr int NV = ND + 2;
  const T g1 = sp.g1;
  const Pt<T, ND>& L = w[2];
  const Pt<T, ND>& R = w[3];
  // ---- averaged state (averaging.py:31-124)
  T rho, u[ND], a;
  if (AVG == AVG_ROE) {
    T sL = sqrt(L.q[0]), sR = sqrt(R.q[0]);
    rho = sqrt(L.q[0] * R.q[0]);
    T inv = L_(1.0) / (sL + sR);
    T ke = L_(0.0);
#pragma unroll
    for (int i = 0; i < ND; ++i) {
      u[i] = (sL * L.u[i] + sR * R.u[i]) * inv;
      ke += u[i] * u[i];
    }
    T H = ((L.q[NV - 1] + L.p) / sL + (R.q[NV - 1] + R.p) / sR) * inv;
    a = sqrt(g1 * (H - L_(0.5) * ke));
  } else {
    rho = L_(0.5) * (L.q[0] + R.q[0]);
#pragma unroll
    for (int i = 0; i < ND; ++i) u[i] = L_(0.5) * (L.u[i] + R.u[i]);
    a = L_(0.5) * (L.a + R.a);
  }
  // ---- LLF wave speeds over points i, i+1 (shock_capturing.py:1000-1028)
  const T sfc = sp.sfc;
  T lam_u = sfc * fmax(fabs(L.u[0]), fabs(R.u[0]));
  T lam_p = sfc * fmax(fabs(L.u[0] + L.a), fabs(R.u[0] + R.a));
  T lam_m = sfc * fmax(fabs(L.u[0] - L.a), fabs(R.u[0] - R.a));

  T rec[NV];
  if (ND == 1) {
    // 1D system, euler_eigensystem.py:85-99, H = a^2/(gama-1) + u^2/2, waves (u-a, u, u+a)
    const T u0 = u[0];
    const T H = a * a / g1 + L_(0.5) * u0 * u0;
    const T den = L_(2.0) * H - u0 * u0;
    const T iden = L_(1.0) / den, ia = L_(1.0) / a;
    T Lm[3][3];
    Lm[0][0] = u0 * (L_(2.0) * H + a * u0 - u0 * u0) * L_(0.5) * ia * iden;
    Lm[0][1] = (-H - a * u0 + L_(0.5) * u0 * u0) * ia * iden;
    Lm[0][2] = iden;
    Lm[1][0] = L_(2.0) * (H - u0 * u0) * iden;
    Lm[1][1] = L_(2.0) * u0 * iden;
    Lm[1][2] = -L_(2.0) * iden;
    Lm[2][0] = u0 * (-L_(2.0) * H + a * u0 + u0 * u0) * L_(0.5) * ia * iden;
    Lm[2][1] = (H - a * u0 - L_(0.5) * u0 * u0) * ia * iden;
    Lm[2][2] = iden;
    const T lam[3] = {lam_m, lam_u, lam_p};
    T fp[3][6], fmn[3][6];
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      const T F0 = w[m].q[1];
      const T F1 = w[m].u[0] * w[m].q[1] + w[m].p;
      const T F2 = w[m].u[0] * (w[m].q[2] + w[m].p);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        T cs = Lm[k][0] * w[m].q[0] + Lm[k][1] * w[m].q[1] + Lm[k][2] * w[m].q[2];
        T cf = Lm[k][0] * F0 + Lm[k][1] * F1 + Lm[k][2] * F2;
        fp[k][m] = L_(0.5) * (cf + lam[k] * cs);
        fmn[k][m] = L_(0.5) * (cf - lam[k] * cs);
      }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) rec[k] = recon_wave<T, SCH>(fp[k], fmn[k], sp);
    fh[0] = rec[0] + rec[1] + rec[2];
    fh[1] = (u0 - a) * rec[0] + u0 * rec[1] + (u0 + a) * rec[2];
    fh[2] = (H - u0 * a) * rec[0] + L_(0.5) * u0 * u0 * rec[1] + (H + u0 * a) * rec[2];
    return;
  }
  // ---- 2D / 3D with k = e_0: waves 0..ND-1 move with u_n, ND with u_n + a, ND+1 with u_n - a
  const T ia = L_(1.0) / a, ia2 = ia * ia, irho = L_(1.0) / rho;
  T ke = L_(0.0);
#pragma unroll
  for (int i = 0; i < ND; ++i) ke += u[i] * u[i];
  const T phi = g1 * L_(0.5) * ke;
  const T bta = ia * irho * L_(0.70710678118654752440);   // 1/(rho a sqrt 2)
  const T alf = rho * ia * L_(0.70710678118654752440);    // rho/(a sqrt 2)
  // projections L*v of a conserved-like vector v (rows of LEV, euler_eigensystem.py):
  //   S = phi*v0 - g1*(u.vm) + g1*vE ; D = v_n - u_n v0
  //   row0 = v0 - S/a^2, row_{1..ND-1} = vorticity rows, row ND = bta(S + a D), row ND+1 = bta(S - a D)
  T fp[NV][6], fmn[NV][6];
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    const Pt<T, ND>& s = w[m];
    T Fv[NV];
    Fv[0] = s.q[1];
    Fv[1] = s.u[0] * s.q[1] + s.p;
#pragma unroll
    for (int i = 1; i < ND; ++i) Fv[1 + i] = s.u[0] * s.q[1 + i];
    Fv[NV - 1] = s.u[0] * (s.q[NV - 1] + s.p);
    T cs[NV], cf[NV];
    // FP32 path: the flux is F = u_n q + p (0, 1, 0.., u_n), so L.F = u_n (L.q) + p (L e_1 + u_n L e_E)
    // with the two LEV columns in closed form; the FP64 path projects F itself (the reference's
    // operation order).
    constexpr int NPASS = sizeof(T) == 4 ? 1 : 2;
#pragma unroll
    for (int pass = 0; pass < NPASS; ++pass) {
      const T* v = pass == 0 ? s.q : Fv;
      T* o = pass == 0 ? cs : cf;
      T um = L_(0.0);
#pragma unroll
      for (int i = 0; i < ND; ++i) um += u[i] * v[1 + i];
      T S = phi * v[0] - g1 * um + g1 * v[NV - 1];
      T D = v[1] - u[0] * v[0];
      o[0] = v[0] - S * ia2;
      if (ND == 2) {
        o[1] = (u[1] * v[0] - v[2]) * irho;
      } else {
        o[1] = (v[3] - u[2] * v[0]) * irho;
        o[2] = (u[1] * v[0] - v[2]) * irho;
      }
      o[ND] = bta * (S + a * D);
      o[ND + 1] = bta * (S - a * D);
    }
    if (NPASS == 1) {
      const T un = s.u[0], du = un - u[0];
      const T pb = s.p * bta, gd = g1 * du;
      cf[0] = un * cs[0] - s.p * g1 * ia2 * du;
#pragma unroll
      for (int k = 1; k < ND; ++k) cf[k] = un * cs[k];
      cf[ND] = un * cs[ND] + pb * (a + gd);
      cf[ND + 1] = un * cs[ND + 1] + pb * (gd - a);
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      const T lk = (k < ND) ? lam_u : (k == ND ? lam_p : lam_m);
      fp[k][m] = L_(0.5) * (cf[k] + lk * cs[k]);
      fmn[k][m] = L_(0.5) * (cf[k] - lk * cs[k]);
    }
  }
#pragma unroll
  for (int k = 0; k < NV; ++k) rec[k] = recon_wave<T, SCH>(fp[k], fmn[k], sp);
  // back to physical space with the REV columns (k = e_0)
  const T rp = rec[ND] + rec[ND + 1], rm = rec[ND] - rec[ND + 1];
  const T F0 = rec[0] + alf * rp;
  fh[0] = F0;
  fh[1] = u[0] * F0 + alf * a * rm;
  const T h0 = (phi + a * a) / g1;
  if (ND == 2) {
    fh[2] = u[1] * F0 - rho * rec[1];
    fh[3] = phi / g1 * rec[0] - rho * u[1] * rec[1] + alf * h0 * rp + alf * u[0] * a * rm;
  } else {
    fh[2] = u[1] * F0 - rho * rec[2];
    fh[3] = u[2] * F0 + rho * rec[1];
    fh[4] = phi / g1 * rec[0] + rho * u[2] * rec[1] - rho * u[1] * rec[2] + alf * h0 * rp + alf * u[0] * a * rm;
  }
}

// HLLC-LM flux at the interface between w[2] and w[3] of a 6-point window (offsets -2..+3),
// Cartesian local frame (HLLCWeno with flux_type 'HLLC-LM', shock_capturing.py:1031-1256):
// the averaged state and eigensystem as char_flux; the characteristic projections CS = L q of
// the six points; per wave the scheme's fifth-order reconstruction from the left (points
// i-2..i+2) and from the right (i+3..i-1, mirrored); back to physical left and right states with
// the REV columns; then u, p, a of each side, the outer wave speeds sL = min(u_av - a_av,
// uL - aL), sR = max(u_av + a_av, uR + aR), the contact speed s*, both outer speeds scaled by
// phi = sin(pi/2 min(1, 10 M)) with M = max |u/a| of the two sides (the low-Mach correction),
// and the flux in the generated central-plus-dissipation form.  The generated right-state
// energy term divides pR by (sL - uR) rho_R, not (sR - uR) rho_R; this follows it.
template <typename T>
__device__ __forceinline__ T lm_sin(T x);
template <>
__device__ __forceinline__ double lm_sin<double>(double x) { return sin(x); }
template <>
__device__ __forceinline__ float lm_sin<float>(float x) { return sinf(x); }

template <typename T, int ND, int SCH, int AVG>
__device__ __forceinline__ void hllc_flux(const Pt<T, ND> (&w)[6], const SP<T>& sp, T (&fh)[ND + 2]) {
  constexpr int NV = ND + 2;
  const T g1 = sp.g1;
  const Pt<T, ND>& L = w[2];
  const Pt<T, ND>& R = w[3];
  T rho, u[ND], a;
  if (AVG == AVG_ROE) {
    T sL = sqrt(L.q[0]), sR = sqrt(R.q[0]);
    rho = sqrt(L.q[0] * R.q[0]);
    T inv = L_(1.0) / (sL + sR);
    T ke = L_(0.0);
#pragma unroll
    for (int i = 0; i < ND; ++i) {
      u[i] = (sL * L.u[i] + sR * R.u[i]) * inv;
      ke += u[i] * u[i];
    }
    T H = ((L.q[NV - 1] + L.p) / sL + (R.q[NV - 1] + R.p) / sR) * inv;
    a = sqrt(g1 * (H - L_(0.5) * ke));
  } else {
    rho = L_(0.5) * (L.q[0] + R.q[0]);
#pragma unroll
    for (int i = 0; i < ND; ++i) u[i] = L_(0.5) * (L.u[i] + R.u[i]);
    a = L_(0.5) * (L.a + R.a);
  }
  const T ia = L_(1.0) / a, ia2 = ia * ia, irho = L_(1.0) / rho;
  T ke = L_(0.0);
#pragma unroll
  for (int i = 0; i < ND; ++i) ke += u[i] * u[i];
  const T phi = g1 * L_(0.5) * ke;
  const T bta = ia * irho * L_(0.70710678118654752440);
  const T alf = rho * ia * L_(0.70710678118654752440);
  T cs[NV][6];
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    const T* v = w[m].q;
    T um = L_(0.0);
#pragma unroll
    for (int i = 0; i < ND; ++i) um += u[i] * v[1 + i];
    T S = phi * v[0] - g1 * um + g1 * v[NV - 1];
    T D = v[1] - u[0] * v[0];
    cs[0][m] = v[0] - S * ia2;
    if (ND == 2) {
      cs[1][m] = (u[1] * v[0] - v[2]) * irho;
    } else {
      cs[1][m] = (v[3] - u[2] * v[0]) * irho;
      cs[2][m] = (u[1] * v[0] - v[2]) * irho;
    }
    cs[ND][m] = bta * (S + a * D);
    cs[ND + 1][m] = bta * (S - a * D);
  }
  T rl[NV], rr[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    rl[k] = recon5<T, SCH>(cs[k][0], cs[k][1], cs[k][2], cs[k][3], cs[k][4], sp);
    rr[k] = recon5<T, SCH>(cs[k][5], cs[k][4], cs[k][3], cs[k][2], cs[k][1], sp);
  }
  // REV columns (k = e_0): characteristic -> conserved, both sides
  T qL[NV], qR[NV];
  const T h0 = (phi + a * a) / g1;
  auto rev = [&](const T (&c)[NV], T (&o)[NV]) {
    const T rp = c[ND] + c[ND + 1], rm = c[ND] - c[ND + 1];
    const T F0 = c[0] + alf * rp;
    o[0] = F0;
    o[1] = u[0] * F0 + alf * a * rm;
    if (ND == 2) {
      o[2] = u[1] * F0 - rho * c[1];
      o[3] = phi / g1 * c[0] - rho * u[1] * c[1] + alf * h0 * rp + alf * u[0] * a * rm;
    } else {
      o[2] = u[1] * F0 - rho * c[2];
      o[3] = u[2] * F0 + rho * c[1];
      o[4] = phi / g1 * c[0] + rho * u[2] * c[1] - rho * u[1] * c[2] + alf * h0 * rp + alf * u[0] * a * rm;
    }
  };
  rev(rl, qL);
  rev(rr, qR);
  const T gm = sp.gama;
  const T irL = L_(1.0) / qL[0], irR = L_(1.0) / qR[0];
  T uL[ND], uR[ND], kL = L_(0.0), kR = L_(0.0);
#pragma unroll
  for (int i = 0; i < ND; ++i) {
    uL[i] = irL * qL[1 + i];
    uR[i] = irR * qR[1 + i];
    kL += uL[i] * uL[i];
    kR += uR[i] * uR[i];
  }
  const T EL = qL[NV - 1], ER = qR[NV - 1];
  const T pL = (-L_(0.5) * kL * qL[0] + EL) * g1, pR = (-L_(0.5) * kR * qR[0] + ER) * g1;
  const T aL = sqrt(gm * irL * pL), aR = sqrt(gm * irR * pR);
  const T un = u[0], uLn = uL[0], uRn = uR[0];
  T sL = fmin(-a + un, -aL + uLn), sR = fmax(a + un, aR + uRn);
  const T ss = (-pL + (-uLn + sL) * qL[0] * uLn - (-uRn + sR) * qR[0] * uRn + pR) /
               ((-uLn + sL) * qL[0] - (-uRn + sR) * qR[0]);
  const T M = fmax(fabs(uLn / aL), fabs(uRn / aR));
  const T lm = lm_sin<T>(L_(0.5) * L_(3.14159265358979323846) * fmin(L_(1.0), L_(10.0) * M));
  sL = lm * sL;
  sR = lm * sR;
  const T mL = (-uLn + sL) * qL[0] / (-ss + sL), mR = (-uRn + sR) * qR[0] / (-ss + sR);
  const T as = fabs(ss);
  if (sL >= L_(0.0)) {
    fh[0] = qL[1];
#pragma unroll
    for (int i = 0; i < ND; ++i) fh[1 + i] = i == 0 ? qL[1] * uLn + pL : qL[1 + i] * uLn;
    fh[NV - 1] = (pL + EL) * uLn;
  } else if (sR <= L_(0.0)) {
    fh[0] = qR[1];
#pragma unroll
    for (int i = 0; i < ND; ++i) fh[1 + i] = i == 0 ? qR[1] * uRn + pR : qR[1 + i] * uRn;
    fh[NV - 1] = (pR + ER) * uRn;
  } else {
    const T hf = L_(0.5);
    fh[0] = hf * qL[1] + hf * qR[1] + hf * (-qL[0] + mL) * sL + hf * (-qR[0] + mR) * sR + hf * (mL - mR) * as;
#pragma unroll
    for (int i = 0; i < ND; ++i) {
      if (i == 0) {
        const T xL = (-uLn + sL) * qL[0] * ss / (-ss + sL), xR = (-uRn + sR) * qR[0] * ss / (-ss + sR);
        fh[1] = hf * pL + hf * pR + hf * (-qL[1] + xL) * sL + hf * (-qR[1] + xR) * sR + hf * (xL - xR) * as +
                hf * qL[1] * uLn + hf * qR[1] * uRn;
      } else {
        const T xL = (-uLn + sL) * qL[0] * uL[i] / (-ss + sL), xR = (-uRn + sR) * qR[0] * uR[i] / (-ss + sR);
        fh[1 + i] = hf * (-qL[1 + i] + xL) * sL + hf * (-qR[1 + i] + xR) * sR + hf * (xL - xR) * as +
                    hf * qL[1 + i] * uLn + hf * qR[1 + i] * uRn;
      }
    }
    const T eL = (-uLn + sL) * ((-uLn + ss) * (pL / ((-uLn + sL) * qL[0]) + ss) + irL * EL) * qL[0] / (-ss + sL);
    const T eR = (-uRn + sR) * ((-uRn + ss) * (pR / ((-uRn + sL) * qR[0]) + ss) + irR * ER) * qR[0] / (-ss + sR);
    fh[NV - 1] = hf * (-EL + eL) * sL + hf * (-ER + eR) * sR + hf * (eL - eR) * as + hf * (pL + EL) * uLn +
                 hf * (pR + ER) * uRn;
  }
}

// Interface flux of a Cartesian sweep: characteristic LLF (FLX 0) or HLLC-LM (FLX 1).
template <typename T, int ND, int SCH, int AVG, int FLX>
__device__ __forceinline__ void cart_flux(const Pt<T, ND> (&w)[6], const SP<T>& sp, T (&fh)[ND + 2]) {
  if constexpr (FLX == 1) {
    hllc_flux<T, ND, SCH, AVG>(w, sp, fh);
  } else {
    char_flux<T, ND, SCH, AVG>(w, sp, fh);
  }
}

// ---------------------------------------------------------------------------------------
// Curvilinear sweeps work in the global frame.  A point carries its conserved state and
// primitives plus the metric row of the sweep direction d, k_i = D_di = d xi_d / d x_i, and
// det J.
template <typename T, int ND>
struct PtC {
  T q[ND + 2];  // rho, rho u_0.., E (global frame)
  T u[ND];
  T p, a;
  T k[ND];      // D_d0 .. D_d(ND-1)
  T J;          // det(d x / d xi)
};

template <typename T, int ND>
__device__ __forceinline__ void make_pt(PtC<T, ND>& s, T gm) {
  T rho = s.q[0];
  T ir = L_(1.0) / rho;
  T ke = L_(0.0);
#pragma unroll
  for (int i = 0; i < ND; ++i) {
    s.u[i] = s.q[1 + i] * ir;
    ke += s.u[i] * s.u[i];
  }
  s.p = (gm - L_(1.0)) * (s.q[ND + 1] - L_(0.5) * rho * ke);
  s.a = sqrt(gm * s.p * ir);
}

// Characteristic LLF flux of the curvilinear form at the interface between w[2] and w[3]:
// contravariant flux F = J [rho U, rho u_i U + p D_di, (E + p) U] with U = D_d . u
// (the conservative metric form of the reference's curvilinear Euler equations,
// equation_types/metric.py with the generated "LFWeno_reconstruction" kernels), eigensystem of
// euler_eigensystem.py:100-165 for the unit direction k = avg(D_d) / |avg(D_d)|, LLF speeds
// from the pointwise J (U +- a |D_d|) over points i, i+1.  The eigenvector matrices are
// applied in factored form: with S = phi v0 - g1 (u . v_m) + g1 v_E, E = v0 - S/a^2,
// w = (v_m - u v0)/rho and Dn = k . v_m - (k . u) v0 the rows of LEV are
//   2D: E, k1 w0 - k0 w1, bta (S + a Dn), bta (S - a Dn)
//   3D: k_i E + (w x k)_i (i = 0..2), bta (S + a Dn), bta (S - a Dn)
// and REV is applied column-wise (see the back-projection below).
template <typename T, int ND, int SCH, int AVG>
__device__ __forceinline__ void char_flux_curv(const PtC<T, ND> (&w)[6], const SP<T>& sp, T (&fh)[ND + 2]) {
  static_assert(ND == 2 || ND == 3, "curvilinear sweeps are 2D or 3D");
  constexpr int NV = ND + 2;
  const T g1 = sp.g1;
  const PtC<T, ND>& L = w[2];
  const PtC<T, ND>& R = w[3];
  T rho, u[ND], a;
  if (AVG == AVG_ROE) {
    T sL = sqrt(L.q[0]), sR = sqrt(R.q[0]);
    rho = sqrt(L.q[0] * R.q[0]);
    T inv = L_(1.0) / (sL + sR);
    T ke = L_(0.0);
#pragma unroll
    for (int i = 0; i < ND; ++i) {
      u[i] = (sL * L.u[i] + sR * R.u[i]) * inv;
      ke += u[i] * u[i];
    }
    T H = ((L.q[NV - 1] + L.p) / sL + (R.q[NV - 1] + R.p) / sR) * inv;
    a = sqrt(g1 * (H - L_(0.5) * ke));
  } else {
    rho = L_(0.5) * (L.q[0] + R.q[0]);
#pragma unroll
    for (int i = 0; i < ND; ++i) u[i] = L_(0.5) * (L.u[i] + R.u[i]);
    a = L_(0.5) * (L.a + R.a);
  }
  // unit direction of the averaged metric row
  T k[ND];
  {
    T kn = L_(0.0);
#pragma unroll
    for (int i = 0; i < ND; ++i) {
      k[i] = L_(0.5) * (L.k[i] + R.k[i]);
      kn += k[i] * k[i];
    }
    kn = L_(1.0) / sqrt(kn);
#pragma unroll
    for (int i = 0; i < ND; ++i) k[i] *= kn;
  }
  // LLF speeds: J U and J U +- a |J D_d| at i and i+1
  const T sfc = sp.sfc;
  T lam_u, lam_p, lam_m;
  {
    T UL = L_(0.0), UR = L_(0.0), mL = L_(0.0), mR = L_(0.0);
#pragma unroll
    for (int i = 0; i < ND; ++i) {
      T kl = L.J * L.k[i], kr = R.J * R.k[i];
      UL += kl * L.u[i];
      UR += kr * R.u[i];
      mL += kl * kl;
      mR += kr * kr;
    }
    mL = sqrt(mL);
    mR = sqrt(mR);
    lam_u = sfc * fmax(fabs(UL), fabs(UR));
    lam_p = sfc * fmax(fabs(UL + L.a * mL), fabs(UR + R.a * mR));
    lam_m = sfc * fmax(fabs(UL - L.a * mL), fabs(UR - R.a * mR));
  }
  const T ia = L_(1.0) / a, ia2 = ia * ia, irho = L_(1.0) / rho;
  T ke = L_(0.0), th = L_(0.0);
#pragma unroll
  for (int i = 0; i < ND; ++i) {
    ke += u[i] * u[i];
    th += k[i] * u[i];
  }
  const T phi = g1 * L_(0.5) * ke;
  const T bta = ia * irho * L_(0.70710678118654752440);
  const T alf = rho * ia * L_(0.70710678118654752440);
  T fp[NV][6], fmn[NV][6];
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    const PtC<T, ND>& s = w[m];
    T U = L_(0.0);
#pragma unroll
    for (int i = 0; i < ND; ++i) U += s.k[i] * s.u[i];
    T Fv[NV];
    Fv[0] = s.J * (s.q[0] * U);
#pragma unroll
    for (int i = 0; i < ND; ++i) Fv[1 + i] = s.J * (s.q[1 + i] * U + s.p * s.k[i]);
    Fv[NV - 1] = s.J * ((s.q[NV - 1] + s.p) * U);
    T cs[NV], cf[NV];
#pragma unroll
    for (int pass = 0; pass < 2; ++pass) {
      const T* v = pass == 0 ? s.q : Fv;
      T* o = pass == 0 ? cs : cf;
      T um = L_(0.0), kv = L_(0.0);
#pragma unroll
      for (int i = 0; i < ND; ++i) {
        um += u[i] * v[1 + i];
        kv += k[i] * v[1 + i];
      }
      T S = phi * v[0] - g1 * um + g1 * v[NV - 1];
      T E = v[0] - S * ia2;
      T Dn = kv - th * v[0];
      T wv[ND];
#pragma unroll
      for (int i = 0; i < ND; ++i) wv[i] = (v[1 + i] - u[i] * v[0]) * irho;
      if (ND == 2) {
        o[0] = E;
        o[1] = k[1] * wv[0] - k[0] * wv[1];
      } else {
        o[0] = k[0] * E + (wv[1] * k[2] - wv[2] * k[1]);
        o[1] = k[1] * E + (wv[2] * k[0] - wv[0] * k[2]);
        o[2] = k[2] * E + (wv[0] * k[1] - wv[1] * k[0]);
      }
      o[ND] = bta * (S + a * Dn);
      o[ND + 1] = bta * (S - a * Dn);
    }
#pragma unroll
    for (int c = 0; c < NV; ++c) {
      const T lk = (c < ND) ? lam_u : (c == ND ? lam_p : lam_m);
      fp[c][m] = L_(0.5) * (cf[c] + lk * cs[c]);
      fmn[c][m] = L_(0.5) * (cf[c] - lk * cs[c]);
    }
  }
  T rec[NV];
#pragma unroll
  for (int c = 0; c < NV; ++c) rec[c] = recon_wave<T, SCH>(fp[c], fmn[c], sp);
  // REV: 2D columns (1, u, phi/g1), rho (0, t, t.u) with t = (k1, -k0), and the acoustic
  // pair alf (1, u +- a k, h0 +- a th); 3D vorticity columns give u (k.r) + rho (k x r) and
  // phi/g1 (k.r) + rho (u x k).r.
  const T rp = rec[ND] + rec[ND + 1], rm = rec[ND] - rec[ND + 1];
  const T h0 = (phi + a * a) / g1;
  if (ND == 2) {
    const T t0 = k[1], t1 = -k[0];
    const T F0 = rec[0] + alf * rp;
    fh[0] = F0;
    fh[1] = u[0] * F0 + alf * a * k[0] * rm + rho * rec[1] * t0;
    fh[2] = u[1] * F0 + alf * a * k[ND - 1] * rm + rho * rec[1] * t1;
    fh[NV - 1] = phi / g1 * rec[0] + rho * (t0 * u[0] + t1 * u[1]) * rec[1] + alf * h0 * rp + alf * a * th * rm;
  } else {
    const T kr = k[0] * rec[0] + k[1] * rec[1] + k[ND - 1] * rec[2];
    const T c0 = k[1] * rec[2] - k[ND - 1] * rec[1];
    const T c1 = k[ND - 1] * rec[0] - k[0] * rec[2];
    const T c2 = k[0] * rec[1] - k[1] * rec[0];
    const T F0 = kr + alf * rp;
    fh[0] = F0;
    fh[1] = u[0] * F0 + rho * c0 + alf * a * k[0] * rm;
    fh[2] = u[1] * F0 + rho * c1 + alf * a * k[1] * rm;
    fh[3] = u[ND - 1] * F0 + rho * c2 + alf * a * k[ND - 1] * rm;
    const T x0 = u[1] * k[ND - 1] - u[ND - 1] * k[1];
    const T x1 = u[ND - 1] * k[0] - u[0] * k[ND - 1];
    const T x2 = u[0] * k[1] - u[1] * k[0];
    fh[NV - 1] = phi / g1 * kr + rho * (x0 * rec[0] + x1 * rec[1] + x2 * rec[2]) + alf * (h0 * rp + a * th * rm);
  }
}

// Central 4th-order first / second derivative weights (scheme.py:83-87), applied to
// differences of the stencil values: the weights of either rule sum to zero, and in this form
// they stay exactly consistent after rounding (a constant field gives exactly zero).  In the
// weighted-sum form the FP32 roundings of 1/12 and 4/3 leave the second-derivative weights
// summing to 7.5e-8, which 1/Delta^2 turns into a systematic source of 7.5e-8 f / Delta^2 (on a
// wall-normal Delta of 2/256 with T ~ 1, 1.2e-3 per point in the Laplacian of T).  The differences
// of neighbouring values are exact when they lie within a factor of two of each other.
template <typename T>
__device__ __forceinline__ T d1w(T fm2, T fm1, T fp1, T fp2) {
  return L_(1.0 / 12.0) * (fm2 - fp2) + L_(2.0 / 3.0) * (fp1 - fm1);
}
template <typename T>
__device__ __forceinline__ T d2w(T fm2, T fm1, T f0, T fp1, T fp2) {
  return L_(4.0 / 3.0) * ((fm1 - f0) + (fp1 - f0)) - L_(1.0 / 12.0) * ((fm2 - f0) + (fp2 - f0));
}

}  // namespace osb
