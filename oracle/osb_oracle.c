/*
 * osb_oracle.c -- CPU restatement of OpenSBLI's explicit residual-and-update path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker the GPU path is compared with; it is
 * loaded by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg, never by
 * the product.  Parity of this restatement with the reference's own generated solver is
 * pinned by tests/test_oracle_golden.py against the committed golden vectors under tests/golden/
 * (states of the reference's own generated OPS C++, compiled with oracle/ops_compat.h, and of
 * its shipped benchmark solvers; tests/golden/make_golden.py writes them).
 *
 * It operates on HOST arrays described by the same osb_block_desc as the CUDA library
 * (include/osb_gb300.h): OPS layout, x fastest, 5 halo points per used direction.
 *
 * Algorithm (each piece cites the reference file it restates):
 *  - constituent relations u_i = rhou_i/rho, p, a, T, mu        (compressible_TGV.py:77-83)
 *  - characteristic LLF flux at i+1/2 per direction:
 *      averaging (simple / Roe)                                   (schemes/spatial/averaging.py:31-124)
 *      eigensystem LEV/REV/eigenvalues (1D, 2D, 3D; k-vector)     (physical_models/euler_eigensystem.py:19-166)
 *      CS = LEV*Q, CF = LEV*F on points i-2..i+3                  (shock_capturing.py:440-502)
 *      lambda_w = sfc * max(|ev_w(i)|, |ev_w(i+1)|)               (shock_capturing.py:1000-1028)
 *      f+/- = (CF +/- lambda*CS)/2                                (shock_capturing.py:979-998)
 *      WENO5-JS / WENO5-Z / TENO5 reconstruction                  (weno.py:36-472, teno.py:59-477)
 *      Fhat = REV * (recon(f+) + recon(f-))                       (shock_capturing.py:859-891)
 *  - HLLC-LM flux from reconstructed states (HLLCWeno)           (shock_capturing.py:1031-1256)
 *  - residual R = -sum_d (Fhat(i+1/2) - Fhat(i-1/2)) / Delta_d    (shock_capturing.py:23-36)
 *  - StoreSome(4) viscous / heat-flux terms, central-4            (optimisations/StoreSome.py, scheme.py:174-258)
 *  - skew-symmetric (Feiereisen) central convective terms         (physical_models/split_forms.py:111-145)
 *  - Kennedy-Gruber-Pirozzoli central convective terms             (physical_models/split_forms.py:178-236)
 *  - non-linear characteristic WENO3 filter with a Ducros sensor    (filters/WENO_filter.py; generated
 *    kernels of apps/performance_benchmark/Central4-WENO5/opensbliblock00_kernels.h:572-2480)
 *  - non-linear characteristic TVD filter (Yee-Sandham-Djomehri)   (filters/TVD_filter.py,
 *    schemes/spatial/shock_capturing.py:619-766)
 *  - low-storage RK3 (rk_LS.py:185-215) and SBLI RK3 (rk_sbli.py:138-154)
 *  - periodic exchange (periodic.py:53-71, opsc.py:1026-1064), zero-gradient
 *    (zero_gradient_outlet.py:11-23), extrapolation (extrapolation.py:29-53), symmetry
 *    (symmetry.py:23-50), Dirichlet (dirichlet.py:27-41), pressure outlet (pressure_outlet.py:35-51),
 *    block interfaces (multi_block.py:48-107)
 *  - TGV reductions (compressible_TGV.py:176-206)
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "../include/osb_gb300.h"

#define NVMAX 5

typedef struct {
  int nd, n[3], hx, hy, hz;
  long ex, ey, ez;
  long st[3]; /* stride per direction */
} geom_t;

static geom_t geom_of(const osb_block_desc* b) {
  geom_t g;
  g.nd = b->ndim;
  for (int d = 0; d < 3; ++d) g.n[d] = d < b->ndim ? b->size[d] : 1;
  g.hx = b->halo;
  g.hy = b->ndim > 1 ? b->halo : 0;
  g.hz = b->ndim > 2 ? b->halo : 0;
  g.ex = g.n[0] + 2 * g.hx;
  g.ey = g.n[1] + 2 * g.hy;
  g.ez = g.n[2] + 2 * g.hz;
  g.st[0] = 1;
  g.st[1] = g.ex;
  g.st[2] = g.ex * g.ey;
  return g;
}

static inline long gid(const geom_t* g, int i, int j, int k) {
  return (long)(i + g->hx) + g->ex * ((long)(j + g->hy) + g->ey * (long)(k + g->hz));
}

static inline long npts_alloc(const geom_t* g) { return g->ex * g->ey * g->ez; }
static double* alloc_like(const geom_t* g);

/* ---- constituent relations ---------------------------------------------------------- */

typedef struct {
  double* u[3];
  double *p, *a, *T, *mu;
} cr_t;

static void cr_alloc(cr_t* c, long n) {
  for (int i = 0; i < 3; ++i) c->u[i] = (double*)calloc(n, sizeof(double));
  c->p = (double*)calloc(n, sizeof(double));
  c->a = (double*)calloc(n, sizeof(double));
  c->T = (double*)calloc(n, sizeof(double));
  c->mu = (double*)calloc(n, sizeof(double));
}

static void cr_free(cr_t* c) {
  for (int i = 0; i < 3; ++i) free(c->u[i]);
  free(c->p); free(c->a); free(c->T); free(c->mu);
}

/* Pointwise primitives over the whole allocated extent (halo points hold whatever the
 * boundary treatment left there; points with rho == 0 are skipped). */
static void cr_compute(const osb_block_desc* b, const geom_t* g, cr_t* c) {
  const int nd = b->ndim, nv = nd + 2;
  const double gm = b->gama;
  long n = npts_alloc(g);
#pragma omp parallel for schedule(static)
  for (long id = 0; id < n; ++id) {
    double rho = b->q[0][id];
    if (rho == 0.0) continue;
    double ke = 0.0;
    for (int i = 0; i < nd; ++i) {
      double ui = b->q[1 + i][id] / rho;
      c->u[i][id] = ui;
      ke += ui * ui;
    }
    double p = (gm - 1.0) * (b->q[nv - 1][id] - 0.5 * rho * ke);
    c->p[id] = p;
    c->a[id] = sqrt(gm * p / rho);
    double T = b->Minf * b->Minf * gm * p / rho;
    c->T[id] = T;
    if (b->viscous == OSB_VISC_SUTHERLAND)
      c->mu[id] = 1.4042 * T * sqrt(T) / (0.40417 + T);
    else if (b->viscous == OSB_VISC_POWER_LAW) /* turbulent_channel.py:93, mu = T**0.7 */
      c->mu[id] = pow(T, b->visc_power);
    else if (b->viscous == OSB_VISC_SUTHERLAND_RATIO) /* katzer_SBLI.py:67 */
      c->mu[id] = pow(T, 1.5) * (1.0 + b->sutherland_s) / (b->sutherland_s + T);
    else
      c->mu[id] = b->mu_const;
  }
}

/* ---- eigensystems (euler_eigensystem.py) --------------------------------------------- */

/* Left/right eigenvectors at the averaged state for unit direction kt (|kt| = 1). */
static void eigensystem(int nd, double gm, const double kt[3], double rho, const double u[3], double a,
                        double L[NVMAX][NVMAX], double R[NVMAX][NVMAX]) {
  const double g1 = gm - 1.0;
  memset(L, 0, sizeof(double) * NVMAX * NVMAX);
  memset(R, 0, sizeof(double) * NVMAX * NVMAX);
  if (nd == 1) {
    /* euler_eigensystem.py:85-99 with H = a^2/(gama-1) + u^2/2 */
    double u0 = u[0];
    double H = a * a / g1 + 0.5 * u0 * u0;
    double den = 2.0 * H - u0 * u0;
    L[0][0] = u0 * (2.0 * H + a * u0 - u0 * u0) / (2.0 * a * den);
    L[0][1] = (-H - a * u0 + 0.5 * u0 * u0) / (a * den);
    L[0][2] = 1.0 / den;
    L[1][0] = 2.0 * (H - u0 * u0) / den;
    L[1][1] = 2.0 * u0 / den;
    L[1][2] = 2.0 / (-den);
    L[2][0] = u0 * (-2.0 * H + a * u0 + u0 * u0) / (2.0 * a * den);
    L[2][1] = (H - a * u0 - 0.5 * u0 * u0) / (a * den);
    L[2][2] = 1.0 / den;
    R[0][0] = 1.0; R[0][1] = 1.0; R[0][2] = 1.0;
    R[1][0] = u0 - a; R[1][1] = u0; R[1][2] = u0 + a;
    R[2][0] = H - u0 * a; R[2][1] = 0.5 * u0 * u0; R[2][2] = H + u0 * a;
    return;
  }
  const double s2 = sqrt(2.0);
  const double alpha = rho / (a * s2), bta = 1.0 / (rho * a * s2);
  const double a2 = a * a;
  if (nd == 2) {
    /* euler_eigensystem.py:100-135 */
    double k0 = kt[0], k1 = kt[1], u0 = u[0], u1 = u[1];
    double phi = g1 * 0.5 * (u0 * u0 + u1 * u1);
    double th = k0 * u0 + k1 * u1;
    R[0][0] = 1.0; R[0][1] = 0.0; R[0][2] = alpha; R[0][3] = alpha;
    R[1][0] = u0; R[1][1] = k1 * rho; R[1][2] = alpha * (u0 + k0 * a); R[1][3] = alpha * (u0 - k0 * a);
    R[2][0] = u1; R[2][1] = -k0 * rho; R[2][2] = alpha * (u1 + k1 * a); R[2][3] = alpha * (u1 - k1 * a);
    R[3][0] = phi / g1; R[3][1] = rho * (k1 * u0 - k0 * u1);
    R[3][2] = alpha * ((phi + a2) / g1 + a * th); R[3][3] = alpha * ((phi + a2) / g1 - a * th);
    L[0][0] = 1.0 - phi / a2; L[0][1] = g1 * u0 / a2; L[0][2] = g1 * u1 / a2; L[0][3] = -g1 / a2;
    L[1][0] = -(k1 * u0 - k0 * u1) / rho; L[1][1] = k1 / rho; L[1][2] = -k0 / rho; L[1][3] = 0.0;
    L[2][0] = bta * (phi - a * th); L[2][1] = bta * (k0 * a - g1 * u0); L[2][2] = bta * (k1 * a - g1 * u1);
    L[2][3] = bta * g1;
    L[3][0] = bta * (phi + a * th); L[3][1] = -bta * (k0 * a + g1 * u0); L[3][2] = -bta * (k1 * a + g1 * u1);
    L[3][3] = bta * g1;
    return;
  }
  /* nd == 3: euler_eigensystem.py:137-165 */
  double k0 = kt[0], k1 = kt[1], k2 = kt[2], u0 = u[0], u1 = u[1], u2 = u[2];
  double phi = g1 * 0.5 * (u0 * u0 + u1 * u1 + u2 * u2);
  double th = k0 * u0 + k1 * u1 + k2 * u2;
  R[0][0] = k0; R[0][1] = k1; R[0][2] = k2; R[0][3] = alpha; R[0][4] = alpha;
  R[1][0] = k0 * u0; R[1][1] = k1 * u0 - k2 * rho; R[1][2] = k2 * u0 + k1 * rho;
  R[1][3] = alpha * (u0 + k0 * a); R[1][4] = alpha * (u0 - k0 * a);
  R[2][0] = k0 * u1 + k2 * rho; R[2][1] = k1 * u1; R[2][2] = k2 * u1 - k0 * rho;
  R[2][3] = alpha * (u1 + k1 * a); R[2][4] = alpha * (u1 - k1 * a);
  R[3][0] = k0 * u2 - k1 * rho; R[3][1] = k1 * u2 + k0 * rho; R[3][2] = k2 * u2;
  R[3][3] = alpha * (u2 + k2 * a); R[3][4] = alpha * (u2 - k2 * a);
  R[4][0] = k0 * phi / g1 + rho * (k2 * u1 - k1 * u2);
  R[4][1] = k1 * phi / g1 + rho * (k0 * u2 - k2 * u0);
  R[4][2] = k2 * phi / g1 + rho * (k1 * u0 - k0 * u1);
  R[4][3] = alpha * ((phi + a2) / g1 + th * a);
  R[4][4] = alpha * ((phi + a2) / g1 - th * a);
  L[0][0] = k0 * (1.0 - phi / a2) - (k2 * u1 - k1 * u2) / rho;
  L[0][1] = k0 * g1 * u0 / a2;
  L[0][2] = k0 * g1 * u1 / a2 + k2 / rho;
  L[0][3] = k0 * g1 * u2 / a2 - k1 / rho;
  L[0][4] = -k0 * g1 / a2;
  L[1][0] = k1 * (1.0 - phi / a2) - (k0 * u2 - k2 * u0) / rho;
  L[1][1] = k1 * g1 * u0 / a2 - k2 / rho;
  L[1][2] = k1 * g1 * u1 / a2;
  L[1][3] = k1 * g1 * u2 / a2 + k0 / rho;
  L[1][4] = -k1 * g1 / a2;
  L[2][0] = k2 * (1.0 - phi / a2) - (k1 * u0 - k0 * u1) / rho;
  L[2][1] = k2 * g1 * u0 / a2 + k1 / rho;
  L[2][2] = k2 * g1 * u1 / a2 - k0 / rho;
  L[2][3] = k2 * g1 * u2 / a2;
  L[2][4] = -k2 * g1 / a2;
  L[3][0] = bta * (phi - th * a);
  L[3][1] = -bta * (g1 * u0 - k0 * a);
  L[3][2] = -bta * (g1 * u1 - k1 * a);
  L[3][3] = -bta * (g1 * u2 - k2 * a);
  L[3][4] = bta * g1;
  L[4][0] = bta * (phi + th * a);
  L[4][1] = -bta * (g1 * u0 + k0 * a);
  L[4][2] = -bta * (g1 * u1 + k1 * a);
  L[4][3] = -bta * (g1 * u2 + k2 * a);
  L[4][4] = bta * g1;
}

/* Pointwise eigenvalues: 1D diag(u-a, u, u+a); 2D diag(U,U,U+ak,U-ak);
 * 3D diag(U,U,U,U+ak,U-ak) with U = k.u (euler_eigensystem.py:88,120,150). */
static void point_ev(int nd, const double k[3], double kmag, const double u[3], double a, double ev[NVMAX]) {
  if (nd == 1) {
    ev[0] = u[0] - a; ev[1] = u[0]; ev[2] = u[0] + a;
    return;
  }
  double U = 0.0;
  for (int i = 0; i < nd; ++i) U += k[i] * u[i];
  for (int i = 0; i < nd; ++i) ev[i] = U;
  ev[nd] = U + a * kmag;
  ev[nd + 1] = U - a * kmag;
}

/* ---- WENO / TENO reconstruction ------------------------------------------------------- */

/* Upwind-biased fifth-order reconstruction at the right face of f[2] from f[0..4] =
 * values at i-2..i+2.  The left-biased reconstruction of the reference (side -1) is this
 * function applied to the mirrored stencil (weno.py:123-136, teno.py:96-107). */
static double recon5(int scheme, const double* f, double teno_eps, double teno_ct) {
  const double fm2 = f[0], fm1 = f[1], f0 = f[2], fp1 = f[3], fp2 = f[4];
  if (scheme == OSB_SCHEME_TENO5) {
    /* teno.py:96-107 (points), 109-123 (ENO), 128-140 (weights), 156-165 (beta), 197-217 */
    double b0 = 0.25 * (fm1 - fp1) * (fm1 - fp1) + (13.0 / 12.0) * (fm1 - 2.0 * f0 + fp1) * (fm1 - 2.0 * f0 + fp1);
    double b1 = 0.25 * (3.0 * f0 - 4.0 * fp1 + fp2) * (3.0 * f0 - 4.0 * fp1 + fp2) +
                (13.0 / 12.0) * (f0 - 2.0 * fp1 + fp2) * (f0 - 2.0 * fp1 + fp2);
    double b2 = 0.25 * (fm2 - 4.0 * fm1 + 3.0 * f0) * (fm2 - 4.0 * fm1 + 3.0 * f0) +
                (13.0 / 12.0) * (fm2 - 2.0 * fm1 + f0) * (fm2 - 2.0 * fm1 + f0);
    double tau = fabs(b0 - b2);
    double t0 = 1.0 + tau / (teno_eps + b0), t1 = 1.0 + tau / (teno_eps + b1), t2 = 1.0 + tau / (teno_eps + b2);
    double a0 = t0 * t0 * t0 * t0 * t0 * t0, a1 = t1 * t1 * t1 * t1 * t1 * t1, a2 = t2 * t2 * t2 * t2 * t2 * t2;
    double inv = 1.0 / (a0 + a1 + a2);
    double d0 = (a0 * inv < teno_ct) ? 0.0 : 1.0;
    double d1 = (a1 * inv < teno_ct) ? 0.0 : 1.0;
    double d2 = (a2 * inv < teno_ct) ? 0.0 : 1.0;
    double w0 = (11.0 / 20.0) * d0, w1 = (4.0 / 10.0) * d1, w2 = (1.0 / 20.0) * d2;
    double iw = 1.0 / (w0 + w1 + w2);
    double e0 = -(1.0 / 6.0) * fm1 + (5.0 / 6.0) * f0 + (2.0 / 6.0) * fp1;
    double e1 = (2.0 / 6.0) * f0 + (5.0 / 6.0) * fp1 - (1.0 / 6.0) * fp2;
    double e2 = (2.0 / 6.0) * fm2 - (7.0 / 6.0) * fm1 + (11.0 / 6.0) * f0;
    return (w0 * e0 + w1 * e1 + w2 * e2) * iw;
  }
  /* WENO5: weno.py:71-121 (ENO coefficients / optimal weights), 139-206 (JS smoothness) */
  double b0 = (13.0 / 12.0) * (f0 - 2.0 * fp1 + fp2) * (f0 - 2.0 * fp1 + fp2) +
              0.25 * (3.0 * f0 - 4.0 * fp1 + fp2) * (3.0 * f0 - 4.0 * fp1 + fp2);
  double b1 = (13.0 / 12.0) * (fm1 - 2.0 * f0 + fp1) * (fm1 - 2.0 * f0 + fp1) + 0.25 * (fm1 - fp1) * (fm1 - fp1);
  double b2 = (13.0 / 12.0) * (fm2 - 2.0 * fm1 + f0) * (fm2 - 2.0 * fm1 + f0) +
              0.25 * (fm2 - 4.0 * fm1 + 3.0 * f0) * (fm2 - 4.0 * fm1 + 3.0 * f0);
  double a0, a1, a2;
  if (scheme == OSB_SCHEME_WENO5_Z) {
    /* weno.py:290-345: tau = |b0 - b2|, alpha = d (1 + (tau/(eps+b))^2), eps = 1e-40 */
    const double eps = 1.0e-40;
    double tau = fabs(b0 - b2);
    double r0 = tau / (eps + b0), r1 = tau / (eps + b1), r2 = tau / (eps + b2);
    a0 = 0.3 * (1.0 + r0 * r0);
    a1 = 0.6 * (1.0 + r1 * r1);
    a2 = 0.1 * (1.0 + r2 * r2);
  } else {
    /* weno.py:348-376: alpha = d / (eps + b)^2, eps = 1e-6 */
    const double eps = 1.0e-6;
    a0 = 0.3 / ((eps + b0) * (eps + b0));
    a1 = 0.6 / ((eps + b1) * (eps + b1));
    a2 = 0.1 / ((eps + b2) * (eps + b2));
  }
  double inv = 1.0 / (a0 + a1 + a2);
  double e0 = (1.0 / 3.0) * f0 + (5.0 / 6.0) * fp1 - (1.0 / 6.0) * fp2;
  double e1 = -(1.0 / 6.0) * fm1 + (5.0 / 6.0) * f0 + (1.0 / 3.0) * fp1;
  double e2 = (1.0 / 3.0) * fm2 - (7.0 / 6.0) * fm1 + (11.0 / 6.0) * f0;
  return (a0 * inv) * e0 + (a1 * inv) * e1 + (a2 * inv) * e2;
}

/* Sixth-order TENO (teno.py:59-194 configuration for sides +1 / -1, 220-240 tau_6, 419-477
 * cut-off and weights) at interface i+1/2 from the six points f[0..5] = i-2..i+3.  Side +1
 * reconstructs the positive split flux, side -1 the negative one.  The reference's side +1
 * fourth smoothness indicator carries its 781/720 term unsquared (teno.py:160-161, unlike side
 * -1 at teno.py:169-171); its generated solver computes it that way and so does this. */
static double recon6(int side, const double* f, double teno_eps, double teno_ct) {
  const double fm2 = f[0], fm1 = f[1], f0 = f[2], fp1 = f[3], fp2 = f[4], fp3 = f[5];
  double b0, b1, b2, b3, e0, e1, e2, e3;
  if (side > 0) {
    b0 = 0.25 * (fm1 - fp1) * (fm1 - fp1) + (13.0 / 12.0) * (fm1 - 2.0 * f0 + fp1) * (fm1 - 2.0 * f0 + fp1);
    b1 = 0.25 * (3.0 * f0 - 4.0 * fp1 + fp2) * (3.0 * f0 - 4.0 * fp1 + fp2) +
         (13.0 / 12.0) * (f0 - 2.0 * fp1 + fp2) * (f0 - 2.0 * fp1 + fp2);
    b2 = 0.25 * (fm2 - 4.0 * fm1 + 3.0 * f0) * (fm2 - 4.0 * fm1 + 3.0 * f0) +
         (13.0 / 12.0) * (fm2 - 2.0 * fm1 + f0) * (fm2 - 2.0 * fm1 + f0);
    double s1 = -11.0 * f0 + 18.0 * fp1 - 9.0 * fp2 + 2.0 * fp3;
    double s2 = 2.0 * f0 - 5.0 * fp1 + 4.0 * fp2 - fp3;
    double s3 = -f0 + 3.0 * fp1 - 3.0 * fp2 + fp3;
    b3 = (1.0 / 36.0) * s1 * s1 + (13.0 / 12.0) * s2 * s2 + (781.0 / 720.0) * s3;
    e0 = -(1.0 / 6.0) * fm1 + (5.0 / 6.0) * f0 + (2.0 / 6.0) * fp1;
    e1 = (2.0 / 6.0) * f0 + (5.0 / 6.0) * fp1 - (1.0 / 6.0) * fp2;
    e2 = (2.0 / 6.0) * fm2 - (7.0 / 6.0) * fm1 + (11.0 / 6.0) * f0;
    e3 = (3.0 / 12.0) * f0 + (13.0 / 12.0) * fp1 - (5.0 / 12.0) * fp2 + (1.0 / 12.0) * fp3;
  } else {
    b0 = 0.25 * (f0 - fp2) * (f0 - fp2) + (13.0 / 12.0) * (f0 - 2.0 * fp1 + fp2) * (f0 - 2.0 * fp1 + fp2);
    b1 = 0.25 * (fm1 - 4.0 * f0 + 3.0 * fp1) * (fm1 - 4.0 * f0 + 3.0 * fp1) +
         (13.0 / 12.0) * (fm1 - 2.0 * f0 + fp1) * (fm1 - 2.0 * f0 + fp1);
    b2 = 0.25 * (3.0 * fp1 - 4.0 * fp2 + fp3) * (3.0 * fp1 - 4.0 * fp2 + fp3) +
         (13.0 / 12.0) * (fp1 - 2.0 * fp2 + fp3) * (fp1 - 2.0 * fp2 + fp3);
    double s1 = -2.0 * fm2 + 9.0 * fm1 - 18.0 * f0 + 11.0 * fp1;
    double s2 = -fm2 + 4.0 * fm1 - 5.0 * f0 + 2.0 * fp1;
    double s3 = -fm2 + 3.0 * fm1 - 3.0 * f0 + fp1;
    b3 = (1.0 / 36.0) * s1 * s1 + (13.0 / 12.0) * s2 * s2 + (781.0 / 720.0) * s3 * s3;
    e0 = (2.0 / 6.0) * f0 + (5.0 / 6.0) * fp1 - (1.0 / 6.0) * fp2;
    e1 = -(1.0 / 6.0) * fm1 + (5.0 / 6.0) * f0 + (2.0 / 6.0) * fp1;
    e2 = (11.0 / 6.0) * fp1 - (7.0 / 6.0) * fp2 + (1.0 / 3.0) * fp3;
    e3 = (1.0 / 12.0) * fm2 - (5.0 / 12.0) * fm1 + (13.0 / 12.0) * f0 + (3.0 / 12.0) * fp1;
  }
  double tau = fabs(b3 - (1.0 / 6.0) * (b0 + b2 - 4.0 * b1));
  double t[4] = {1.0 + tau / (teno_eps + b0), 1.0 + tau / (teno_eps + b1), 1.0 + tau / (teno_eps + b2),
                 1.0 + tau / (teno_eps + b3)};
  double a[4], sum = 0.0;
  for (int r = 0; r < 4; ++r) {
    a[r] = t[r] * t[r] * t[r] * t[r] * t[r] * t[r];
    sum += a[r];
  }
  const double dopt[4] = {231.0 / 500.0, 3.0 / 10.0, 27.0 / 500.0, 23.0 / 125.0};
  const double e[4] = {e0, e1, e2, e3};
  double inv = 1.0 / sum, wsum = 0.0, acc = 0.0;
  for (int r = 0; r < 4; ++r) {
    double w = (a[r] * inv < teno_ct) ? 0.0 : dopt[r];
    wsum += w;
    acc += w * e[r];
  }
  return acc * (1.0 / wsum);
}

/* Reconstruction of one characteristic wave at i+1/2: the positive split flux fp[0..5] and the
 * negative one fm[0..5] (points i-2..i+3). */
static double recon_wave(int scheme, const double* fp, const double* fm, double teno_eps, double teno_ct) {
  if (scheme == OSB_SCHEME_TENO6) return recon6(1, fp, teno_eps, teno_ct) + recon6(-1, fm, teno_eps, teno_ct);
  double mir[5] = {fm[5], fm[4], fm[3], fm[2], fm[1]};
  return recon5(scheme, fp, teno_eps, teno_ct) + recon5(scheme, mir, teno_eps, teno_ct);
}

/* ---- characteristic flux at one interface --------------------------------------------- */

/* Interface i+1/2 along direction d of a Cartesian block: idc = linear index of point i. */
static void char_flux_cart(const osb_block_desc* b, const geom_t* g, const cr_t* c, int d, long idc,
                           double* fhat) {
  const int nd = b->ndim, nv = nd + 2;
  const long s = g->st[d];
  const double gm = b->gama;
  double kt[3] = {0.0, 0.0, 0.0};
  kt[d] = 1.0;
  long iL = idc, iR = idc + s;
  /* averaged state (averaging.py) */
  double rho_av, u_av[3] = {0, 0, 0}, a_av;
  if (b->averaging == OSB_AVG_ROE) {
    double rL = b->q[0][iL], rR = b->q[0][iR];
    double sL = sqrt(rL), sR = sqrt(rR);
    rho_av = sqrt(rL * rR);
    double inv = 1.0 / (sL + sR);
    double ke = 0.0;
    for (int i = 0; i < nd; ++i) {
      u_av[i] = (sL * c->u[i][iL] + sR * c->u[i][iR]) * inv;
      ke += u_av[i] * u_av[i];
    }
    double HL = (b->q[nv - 1][iL] + c->p[iL]) / rL, HR = (b->q[nv - 1][iR] + c->p[iR]) / rR;
    double H = (sL * HL + sR * HR) * inv;
    a_av = sqrt((gm - 1.0) * (H - 0.5 * ke));
  } else {
    rho_av = 0.5 * (b->q[0][iL] + b->q[0][iR]);
    for (int i = 0; i < nd; ++i) u_av[i] = 0.5 * (c->u[i][iL] + c->u[i][iR]);
    a_av = 0.5 * (c->a[iL] + c->a[iR]);
  }
  double L[NVMAX][NVMAX], R[NVMAX][NVMAX];
  eigensystem(nd, gm, kt, rho_av, u_av, a_av, L, R);
  /* LLF wave speeds over points i, i+1 only */
  double lam[NVMAX], evL[NVMAX], evR[NVMAX];
  double uL[3] = {0, 0, 0}, uR[3] = {0, 0, 0};
  for (int i = 0; i < nd; ++i) { uL[i] = c->u[i][iL]; uR[i] = c->u[i][iR]; }
  point_ev(nd, kt, 1.0, uL, c->a[iL], evL);
  point_ev(nd, kt, 1.0, uR, c->a[iR], evR);
  for (int w = 0; w < nv; ++w) lam[w] = b->shock_filter_control * fmax(fabs(evL[w]), fabs(evR[w]));
  /* characteristic projections on points i-2 .. i+3 */
  double fp[NVMAX][6], fm[NVMAX][6];
  for (int m = 0; m < 6; ++m) {
    long id = idc + (long)(m - 2) * s;
    double Q[NVMAX], F[NVMAX];
    double ud = c->u[d][id], p = c->p[id];
    for (int v = 0; v < nv; ++v) Q[v] = b->q[v][id];
    F[0] = Q[1 + d];
    for (int i = 0; i < nd; ++i) F[1 + i] = ud * Q[1 + i] + (i == d ? p : 0.0);
    F[nv - 1] = ud * (Q[nv - 1] + p);
    for (int w = 0; w < nv; ++w) {
      double cs = 0.0, cf = 0.0;
      for (int v = 0; v < nv; ++v) { cs += L[w][v] * Q[v]; cf += L[w][v] * F[v]; }
      fp[w][m] = 0.5 * (cf + lam[w] * cs);
      fm[w][m] = 0.5 * (cf - lam[w] * cs);
    }
  }
  double rec[NVMAX];
  for (int w = 0; w < nv; ++w) {
    rec[w] = recon_wave(b->scheme, fp[w], fm[w], b->eps, b->teno_ct);
  }
  for (int v = 0; v < nv; ++v) {
    double acc = 0.0;
    for (int w = 0; w < nv; ++w) acc += R[v][w] * rec[w];
    fhat[v] = acc;
  }
}

/* HLLC-LM flux at interface i+1/2 of a Cartesian block (HLLCCharacteristic with flux_type
 * 'HLLC-LM', shock_capturing.py:1031-1256, as the generated "HLLCWeno_reconstruction" kernel):
 * the averaged eigensystem; CS = L Q on points i-2..i+3; per wave the scheme's reconstruction of
 * CS from the left (i-2..i+2) and from the right (i-1..i+3, mirrored); the physical states
 * qL = R recL, qR = R recR; then u, p, a of each, the wave speeds sL = min(u_av - a_av, uL - aL),
 * sR = max(u_av + a_av, uR + aR), the contact speed s*, both outer speeds scaled by
 * phi = sin(pi/2 min(1, 10 M)) with M = max(|uL/aL|, |uR/aR|), and the HLLC flux in the
 * generated central-plus-dissipation form.  The generated right-state energy term divides pR by
 * (sL - uR) rho_R, not (sR - uR) rho_R; this follows it. */
static void hllc_flux_cart(const osb_block_desc* b, const geom_t* g, const cr_t* c, int d, long idc,
                           double* fhat) {
  const int nd = b->ndim, nv = nd + 2;
  const long s = g->st[d];
  const double gm = b->gama, g1 = -1 + gm;
  double kt[3] = {0.0, 0.0, 0.0};
  kt[d] = 1.0;
  const long iL = idc, iR = idc + s;
  double rho_av, u_av[3] = {0, 0, 0}, a_av;
  if (b->averaging == OSB_AVG_ROE) {
    const double rL = b->q[0][iL], rR = b->q[0][iR];
    const double sLr = sqrt(rL), sRr = sqrt(rR);
    rho_av = sqrt(rL * rR);
    const double inv = 1.0 / (sLr + sRr);
    double ke = 0.0;
    for (int i = 0; i < nd; ++i) {
      u_av[i] = (sLr * c->u[i][iL] + sRr * c->u[i][iR]) * inv;
      ke += u_av[i] * u_av[i];
    }
    const double HL = (b->q[nv - 1][iL] + c->p[iL]) / rL, HR = (b->q[nv - 1][iR] + c->p[iR]) / rR;
    a_av = sqrt((gm - 1.0) * ((sLr * HL + sRr * HR) * inv - 0.5 * ke));
  } else {
    rho_av = (1.0 / 2.0) * (b->q[0][iL] + b->q[0][iR]);
    for (int i = 0; i < nd; ++i) u_av[i] = (1.0 / 2.0) * (c->u[i][iL] + c->u[i][iR]);
    a_av = (1.0 / 2.0) * (c->a[iL] + c->a[iR]);
  }
  double L[NVMAX][NVMAX], R[NVMAX][NVMAX];
  eigensystem(nd, gm, kt, rho_av, u_av, a_av, L, R);
  double cs[NVMAX][6];
  for (int m = 0; m < 6; ++m) {
    const long id = idc + (long)(m - 2) * s;
    for (int w = 0; w < nv; ++w) {
      double acc = 0.0;
      for (int v = 0; v < nv; ++v) acc += L[w][v] * b->q[v][id];
      cs[w][m] = acc;
    }
  }
  double recL[NVMAX], recR[NVMAX];
  for (int w = 0; w < nv; ++w) {
    const double mir[5] = {cs[w][5], cs[w][4], cs[w][3], cs[w][2], cs[w][1]};
    recL[w] = recon5(b->scheme, cs[w], b->eps, b->teno_ct);
    recR[w] = recon5(b->scheme, mir, b->eps, b->teno_ct);
  }
  double qL[NVMAX], qR[NVMAX];
  for (int v = 0; v < nv; ++v) {
    double aL_ = 0.0, aR_ = 0.0;
    for (int w = 0; w < nv; ++w) {
      aL_ += R[v][w] * recL[w];
      aR_ += R[v][w] * recR[w];
    }
    qL[v] = aL_;
    qR[v] = aR_;
  }
  const double irL = 1.0 / qL[0], irR = 1.0 / qR[0];
  double uL[3] = {0, 0, 0}, uR[3] = {0, 0, 0}, kL = 0.0, kR = 0.0;
  for (int i = 0; i < nd; ++i) {
    uL[i] = irL * qL[1 + i];
    uR[i] = irR * qR[1 + i];
    kL += uL[i] * uL[i];
    kR += uR[i] * uR[i];
  }
  const double EL = qL[nv - 1], ER = qR[nv - 1];
  const double pL = (-0.5 * kL * qL[0] + EL) * g1, pR = (-0.5 * kR * qR[0] + ER) * g1;
  const double aL = sqrt(gm * irL * pL), aR = sqrt(gm * irR * pR);
  const double un = u_av[d], uLn = uL[d], uRn = uR[d];
  double sL = fmin(-a_av + un, -aL + uLn), sR = fmax(a_av + un, aR + uRn);
  const double ss = (-pL + (-uLn + sL) * qL[0] * uLn - (-uRn + sR) * qR[0] * uRn + pR) /
                    ((-uLn + sL) * qL[0] - (-uRn + sR) * qR[0]);
  const double M = fmax(fabs(uLn / aL), fabs(uRn / aR));
  const double phi = sin((1.0 / 2.0) * M_PI * fmin(1.0, 10.0 * M));
  sL = phi * sL;
  sR = phi * sR;
  const double mL = (-uLn + sL) * qL[0] / (-ss + sL), mR = (-uRn + sR) * qR[0] / (-ss + sR);
  const double as = fabs(ss);
  if (sL >= 0) {
    fhat[0] = qL[1 + d];
    for (int i = 0; i < nd; ++i) fhat[1 + i] = i == d ? qL[1 + d] * uLn + pL : qL[1 + i] * uLn;
    fhat[nv - 1] = (pL + EL) * uLn;
  } else if (sR <= 0) {
    fhat[0] = qR[1 + d];
    for (int i = 0; i < nd; ++i) fhat[1 + i] = i == d ? qR[1 + d] * uRn + pR : qR[1 + i] * uRn;
    fhat[nv - 1] = (pR + ER) * uRn;
  } else {
    fhat[0] = (1.0 / 2.0) * qL[1 + d] + (1.0 / 2.0) * qR[1 + d] + (1.0 / 2.0) * (-qL[0] + mL) * sL +
              (1.0 / 2.0) * (-qR[0] + mR) * sR + (1.0 / 2.0) * (mL - mR) * as;
    for (int i = 0; i < nd; ++i) {
      if (i == d) {
        const double xL = (-uLn + sL) * qL[0] * ss / (-ss + sL), xR = (-uRn + sR) * qR[0] * ss / (-ss + sR);
        fhat[1 + i] = (1.0 / 2.0) * pL + (1.0 / 2.0) * pR + (1.0 / 2.0) * (-qL[1 + d] + xL) * sL +
                      (1.0 / 2.0) * (-qR[1 + d] + xR) * sR + (1.0 / 2.0) * (xL - xR) * as +
                      (1.0 / 2.0) * qL[1 + d] * uLn + (1.0 / 2.0) * qR[1 + d] * uRn;
      } else {
        const double xL = (-uLn + sL) * qL[0] * uL[i] / (-ss + sL), xR = (-uRn + sR) * qR[0] * uR[i] / (-ss + sR);
        fhat[1 + i] = (1.0 / 2.0) * (-qL[1 + i] + xL) * sL + (1.0 / 2.0) * (-qR[1 + i] + xR) * sR +
                      (1.0 / 2.0) * (xL - xR) * as + (1.0 / 2.0) * qL[1 + i] * uLn + (1.0 / 2.0) * qR[1 + i] * uRn;
      }
    }
    const double eL = (-uLn + sL) * ((-uLn + ss) * (pL / ((-uLn + sL) * qL[0]) + ss) + irL * EL) * qL[0] / (-ss + sL);
    const double eR = (-uRn + sR) * ((-uRn + ss) * (pR / ((-uRn + sL) * qR[0]) + ss) + irR * ER) * qR[0] / (-ss + sR);
    fhat[nv - 1] = (1.0 / 2.0) * (-EL + eL) * sL + (1.0 / 2.0) * (-ER + eR) * sR + (1.0 / 2.0) * (eL - eR) * as +
                   (1.0 / 2.0) * (pL + EL) * uLn + (1.0 / 2.0) * (pR + ER) * uRn;
  }
}

/* Curvilinear interface flux (k = D_d averaged, contravariant flux scaled by det J), as the
 * generated "LFWeno_reconstruction" kernel of the curvilinear verification case
 * (euler_eigensystem.py:19-51 apply_direction with metrics; metric.py). */
static void char_flux_curv(const osb_block_desc* b, const geom_t* g, const cr_t* c, int d, long idc, double* fhat) {
  const int nd = b->ndim, nv = nd + 2;
  const long s = g->st[d];
  const double gm = b->gama;
  long iL = idc, iR = idc + s;
  const double* J = b->metric[9];
  double rho_av, u_av[3] = {0, 0, 0}, a_av;
  if (b->averaging == OSB_AVG_ROE) {
    double rL = b->q[0][iL], rR = b->q[0][iR];
    double sL = sqrt(rL), sR = sqrt(rR);
    rho_av = sqrt(rL * rR);
    double inv = 1.0 / (sL + sR);
    double ke = 0.0;
    for (int i = 0; i < nd; ++i) {
      u_av[i] = (sL * c->u[i][iL] + sR * c->u[i][iR]) * inv;
      ke += u_av[i] * u_av[i];
    }
    double HL = (b->q[nv - 1][iL] + c->p[iL]) / rL, HR = (b->q[nv - 1][iR] + c->p[iR]) / rR;
    a_av = sqrt((gm - 1.0) * ((sL * HL + sR * HR) * inv - 0.5 * ke));
  } else {
    rho_av = 0.5 * (b->q[0][iL] + b->q[0][iR]);
    for (int i = 0; i < nd; ++i) u_av[i] = 0.5 * (c->u[i][iL] + c->u[i][iR]);
    a_av = 0.5 * (c->a[iL] + c->a[iR]);
  }
  double kav[3] = {0, 0, 0}, kn = 0.0;
  for (int i = 0; i < nd; ++i) {
    kav[i] = 0.5 * (b->metric[3 * d + i][iL] + b->metric[3 * d + i][iR]);
    kn += kav[i] * kav[i];
  }
  kn = 1.0 / sqrt(kn);
  double kt[3] = {kav[0] * kn, kav[1] * kn, kav[2] * kn};
  double L[NVMAX][NVMAX], R[NVMAX][NVMAX];
  eigensystem(nd, gm, kt, rho_av, u_av, a_av, L, R);
  double lam[NVMAX], evL[NVMAX], evR[NVMAX];
  for (int side = 0; side < 2; ++side) {
    long id = side ? iR : iL;
    double k[3] = {0, 0, 0}, km = 0.0, u[3] = {0, 0, 0};
    for (int i = 0; i < nd; ++i) {
      k[i] = J[id] * b->metric[3 * d + i][id];
      km += k[i] * k[i];
      u[i] = c->u[i][id];
    }
    point_ev(nd, k, sqrt(km), u, c->a[id], side ? evR : evL);
  }
  for (int w = 0; w < nv; ++w) lam[w] = b->shock_filter_control * fmax(fabs(evL[w]), fabs(evR[w]));
  double fp[NVMAX][6], fm[NVMAX][6];
  for (int m = 0; m < 6; ++m) {
    long id = idc + (long)(m - 2) * s;
    double Q[NVMAX], F[NVMAX];
    double U = 0.0;
    for (int i = 0; i < nd; ++i) U += b->metric[3 * d + i][id] * c->u[i][id];
    double p = c->p[id], dj = J[id];
    for (int v = 0; v < nv; ++v) Q[v] = b->q[v][id];
    F[0] = dj * (Q[0] * U);
    for (int i = 0; i < nd; ++i) F[1 + i] = dj * (Q[1 + i] * U + p * b->metric[3 * d + i][id]);
    F[nv - 1] = dj * ((Q[nv - 1] + p) * U);
    for (int w = 0; w < nv; ++w) {
      double cs = 0.0, cf = 0.0;
      for (int v = 0; v < nv; ++v) { cs += L[w][v] * Q[v]; cf += L[w][v] * F[v]; }
      fp[w][m] = 0.5 * (cf + lam[w] * cs);
      fm[w][m] = 0.5 * (cf - lam[w] * cs);
    }
  }
  double rec[NVMAX];
  for (int w = 0; w < nv; ++w) {
    rec[w] = recon_wave(b->scheme, fp[w], fm[w], b->eps, b->teno_ct);
  }
  for (int v = 0; v < nv; ++v) {
    double acc = 0.0;
    for (int w = 0; w < nv; ++w) acc += R[v][w] * rec[w];
    fhat[v] = acc;
  }
}

/* ---- central 4th-order operators (scheme.py:83-87 finite_diff_weights) --------------- */

static inline double d1c(const double* f, long id, long s, double invd) {
  return ((1.0 / 12.0) * f[id - 2 * s] - (2.0 / 3.0) * f[id - s] + (2.0 / 3.0) * f[id + s] -
          (1.0 / 12.0) * f[id + 2 * s]) * invd;
}
static inline double d2c(const double* f, long id, long s, double inv2d) {
  return (-(1.0 / 12.0) * f[id - 2 * s] + (4.0 / 3.0) * f[id - s] - 2.5 * f[id] + (4.0 / 3.0) * f[id + s] -
          (1.0 / 12.0) * f[id + 2 * s]) * inv2d;
}
static const double C1[5] = {1.0 / 12.0, -2.0 / 3.0, 0.0, 2.0 / 3.0, -1.0 / 12.0};
/* d^2 f / dx_a dx_b (a != b) as the central-4 derivative along b of the central-4 derivative
 * along a (StoreSome stores du/dx_a and differentiates it again, StoreSome.py:47-67). */
static inline double dmix(const double* f, long id, long sa, long sb, double inva, double invb) {
  double acc = 0.0;
  for (int m = 0; m < 5; ++m) {
    if (m == 2) continue;
    long idb = id + (long)(m - 2) * sb;
    acc += C1[m] * d1c(f, idb, sa, inva);
  }
  return acc * invb;
}

/* ---- one-sided boundary closures of the central derivatives at isothermal-wall faces ----
 * The fourth-order closure of Carpenter, Gottlieb and Abarbanel (J. Comput. Phys. 1998,
 * doi:10.1006/jcph.1998.6114) that Carpenter_scheme.py:91-111 forms as inv(A_L) A_R: its row r
 * (r = 0..3, the points 0..3 next to the wall) weighs the six points r' = m - r (m = 0..5) from
 * the wall plane; row 0 is the exact third-order one-sided rule [-11/6, 3, -3/2, 1/3] (the
 * reference rationalises it).  The second derivative takes the two rows of
 * Carpenter_scheme.py:79-86 at the points 0 and 1 (five points from m - r).  On the far side the
 * rows are mirrored: offsets r - m, first-derivative weights negated. */
static double carp1[4][6];
static const double carp2[2][5] = {{35.0 / 12.0, -104.0 / 12.0, 114.0 / 12.0, -56.0 / 12.0, 11.0 / 12.0},
                                   {11.0 / 12.0, -20.0 / 12.0, 6.0 / 12.0, 4.0 / 12.0, -1.0 / 12.0}};
static int carp_ready = 0;

static void carpenter_init(void) {
  if (carp_ready) return;
  const double R1 = -(2177.0 * sqrt(295369.0) - 1166427.0) / 25488.0;
  const double R2 = (66195.0 * sqrt(53.0) * sqrt(5573.0) - 35909375.0) / 101952.0;
  double AL[4][4] = {
      {-(216.0 * R2 + 2160.0 * R1 - 2125.0) / 12960.0, (81.0 * R2 + 675.0 * R1 + 415.0) / 540.0,
       -(72.0 * R2 + 720.0 * R1 + 445.0) / 1440.0, -(108.0 * R2 + 756.0 * R1 + 421.0) / 1296.0},
      {(81.0 * R2 + 675.0 * R1 + 415.0) / 540.0, -(4104.0 * R2 + 32400.0 * R1 + 11225.0) / 4320.0,
       (1836.0 * R2 + 14580.0 * R1 + 7295.0) / 2160.0, -(216.0 * R2 + 2160.0 * R1 + 655.0) / 4320.0},
      {-(72.0 * R2 + 720.0 * R1 + 445.0) / 1440.0, (1836.0 * R2 + 14580.0 * R1 + 7295.0) / 2160.0,
       -(4104.0 * R2 + 32400.0 * R1 + 12785.0) / 4320.0, (81.0 * R2 + 675.0 * R1 + 335.0) / 540.0},
      {-(108.0 * R2 + 756.0 * R1 + 421.0) / 1296.0, -(216.0 * R2 + 2160.0 * R1 + 655.0) / 4320.0,
       (81.0 * R2 + 675.0 * R1 + 335.0) / 540.0, -(216.0 * R2 + 2160.0 * R1 - 12085.0) / 12960.0}};
  double AR[4][6] = {
      {-0.5, -(864.0 * R2 + 6480.0 * R1 + 305.0) / 4320.0, (216.0 * R2 + 1620.0 * R1 + 725.0) / 540.0,
       -(864.0 * R2 + 6480.0 * R1 + 3335.0) / 4320.0, 0.0, 0.0},
      {(864.0 * R2 + 6480.0 * R1 + 305.0) / 4320.0, 0.0, -(864.0 * R2 + 6480.0 * R1 + 2315.0) / 1440.0,
       (108.0 * R2 + 810.0 * R1 + 415.0) / 270.0, 0.0, 0.0},
      {-(216.0 * R2 + 1620.0 * R1 + 725.0) / 540.0, (864.0 * R2 + 6480.0 * R1 + 2315.0) / 1440.0, 0.0,
       -(864.0 * R2 + 6480.0 * R1 + 785.0) / 4320.0, -1.0 / 12.0, 0.0},
      {(864.0 * R2 + 6480.0 * R1 + 3335.0) / 4320.0, -(108.0 * R2 + 810.0 * R1 + 415.0) / 270.0,
       (864.0 * R2 + 6480.0 * R1 + 785.0) / 4320.0, 0.0, 8.0 / 12.0, -1.0 / 12.0}};
  /* solve A_L X = A_R by Gauss-Jordan elimination with partial pivoting */
  for (int col = 0; col < 4; ++col) {
    int piv = col;
    for (int r = col + 1; r < 4; ++r)
      if (fabs(AL[r][col]) > fabs(AL[piv][col])) piv = r;
    for (int k = 0; k < 4; ++k) { double t = AL[col][k]; AL[col][k] = AL[piv][k]; AL[piv][k] = t; }
    for (int k = 0; k < 6; ++k) { double t = AR[col][k]; AR[col][k] = AR[piv][k]; AR[piv][k] = t; }
    const double inv = 1.0 / AL[col][col];
    for (int k = 0; k < 4; ++k) AL[col][k] *= inv;
    for (int k = 0; k < 6; ++k) AR[col][k] *= inv;
    for (int r = 0; r < 4; ++r) {
      if (r == col) continue;
      const double f = AL[r][col];
      for (int k = 0; k < 4; ++k) AL[r][k] -= f * AL[col][k];
      for (int k = 0; k < 6; ++k) AR[r][k] -= f * AR[col][k];
    }
  }
  for (int r = 0; r < 4; ++r)
    for (int m = 0; m < 6; ++m) carp1[r][m] = fabs(AR[r][m]) < 1e-14 ? 0.0 : AR[r][m];
  const double row0[6] = {-11.0 / 6.0, 3.0, -1.5, 1.0 / 3.0, 0.0, 0.0};
  for (int m = 0; m < 6; ++m) carp1[0][m] = row0[m];
  carp_ready = 1;
}

/* The closure weights (for tests): row r of the first (order 1, 6 weights) or second (order 2,
 * 5 weights) derivative closure. */
int oracle_carpenter(int order, int r, double* w) {
  carpenter_init();
  if (order == 1 && r >= 0 && r < 4) { for (int m = 0; m < 6; ++m) w[m] = carp1[r][m]; return 0; }
  if (order == 2 && r >= 0 && r < 2) { for (int m = 0; m < 5; ++m) w[m] = carp2[r][m]; return 0; }
  return -1;
}

/* Wall-normal stretching metrics of a grid line x1[j], j = 0..n-1: the generated "MetricsEquation
 * evaluation" kernels of a MetricsEquation with direction 1 stretched only (metric.py:183-197,
 * transform_second_derivative metric.py:199-240): x1' = d x1 / d xi_1 by the central 4th-order
 * rule, or the closure rows above in the four rows next to a wall face; D11 = 1 / x1' (and
 * det J = x1'); SD111 = d D11 / d xi_1 by the same rules.  Returns -1 when a row has no rule
 * (no wall at an end) or the line is not strictly monotone. */
int oracle_ystretch_metrics(int n, double delta, const double* x1, int wall_lo, int wall_hi, double* d11,
                            double* sd111) {
  carpenter_init();
  if (n < 12) return -1;
  const double inv = 1.0 / delta;
  for (int pass = 0; pass < 2; ++pass) {
    const double* f = pass == 0 ? x1 : d11;
    double* out = pass == 0 ? d11 : sd111;
    double* tmp = (double*)malloc(sizeof(double) * n);
    for (int j = 0; j < n; ++j) {
      int r = -1, hi = 0;
      if (wall_lo && j < 4) r = j;
      else if (wall_hi && j > n - 5) { r = n - 1 - j; hi = 1; }
      double acc;
      if (r >= 0) {
        acc = 0.0;
        for (int m = 0; m < 6; ++m) {
          if (carp1[r][m] == 0.0) continue;
          const int o = hi ? r - m : m - r;
          acc += (hi ? -carp1[r][m] : carp1[r][m]) * f[j + o];
        }
        acc *= inv;
      } else {
        if (j < 2 || j > n - 3) { free(tmp); return -1; }
        acc = d1c(f, j, 1, inv);
      }
      tmp[j] = acc;
    }
    for (int j = 0; j < n; ++j) {
      if (pass == 0) {
        if (tmp[j] == 0.0 || !isfinite(tmp[j])) { free(tmp); return -1; }
        out[j] = 1.0 / tmp[j];
      } else {
        out[j] = tmp[j];
      }
    }
    free(tmp);
  }
  return 0;
}

/* Closure row of the point with index i along d for derivatives of `order`: 0..3 (first) or
 * 0..1 (second) next to a low wall face, 4 + r next to a high one, -1 for the central rule. */
static inline int modifies_central(int kind) {
  /* every ModifyCentralDerivative face kind (bc_core.py:15-17): walls, the pressure-extrapolation
   * inlet, extrapolation, Dirichlet and pressure-outlet faces; their central derivatives only
   * occur on viscous blocks */
  return kind == OSB_BC_ISOTHERMAL_WALL || kind == OSB_BC_ADIABATIC_WALL || kind == OSB_BC_INLET_PRESSURE_EXTRAP ||
         kind == OSB_BC_EXTRAP0 || kind == OSB_BC_EXTRAP1 || kind == OSB_BC_DIRICHLET ||
         kind == OSB_BC_PRESSURE_OUTLET;
}
static int closure_row(const osb_block_desc* b, const geom_t* g, int d, int i, int order) {
  const int rows = order == 1 ? 4 : 2;
  if (modifies_central(b->bc[d][0]) && i < rows) return i;
  if (modifies_central(b->bc[d][1]) && i > g->n[d] - 1 - rows) return 4 + (g->n[d] - 1 - i);
  return -1;
}

/* Closure sums (without the 1/Delta factors): row code cr of closure_row */
static inline double c1sum(const double* f, long id, long s, int cr) {
  const int r = cr & 3, hi = cr >= 4;
  double acc = 0.0;
  for (int m = 0; m < 6; ++m) {
    if (carp1[r][m] == 0.0) continue;
    const long o = hi ? (long)(r - m) : (long)(m - r);
    acc += (hi ? -carp1[r][m] : carp1[r][m]) * f[id + o * s];
  }
  return acc;
}
static inline double c2sum(const double* f, long id, long s, int cr) {
  const int r = cr & 3, hi = cr >= 4;
  double acc = 0.0;
  for (int m = 0; m < 5; ++m) {
    const long o = hi ? (long)(r - m) : (long)(m - r);
    acc += carp2[r][m] * f[id + o * s];
  }
  return acc;
}

/* First / second derivative along d at the point with coordinates c (index id) */
static inline double d1at(const osb_block_desc* b, const geom_t* g, const double* f, long id, const int* c, int d,
                          double invd) {
  const int cr = closure_row(b, g, d, c[d], 1);
  if (cr < 0) return d1c(f, id, g->st[d], invd);
  return c1sum(f, id, g->st[d], cr) * invd;
}
static inline double d2at(const osb_block_desc* b, const geom_t* g, const double* f, long id, const int* c, int d,
                          double inv2d) {
  const int cr = closure_row(b, g, d, c[d], 2);
  if (cr < 0) return d2c(f, id, g->st[d], inv2d);
  return c2sum(f, id, g->st[d], cr) * inv2d;
}
/* d^2 f / dx_a dx_b: the first derivative along b of the first derivative along a (each with
 * its closure; moving along b keeps the point's index along a) */
static inline double dmixat(const osb_block_desc* b, const geom_t* g, const double* f, long id, const int* c, int a,
                            int bb, double inva, double invb) {
  const int cb = closure_row(b, g, bb, c[bb], 1);
  if (cb < 0) {
    double acc = 0.0;
    for (int m = 0; m < 5; ++m) {
      if (m == 2) continue;
      const long idb = id + (long)(m - 2) * g->st[bb];
      acc += C1[m] * d1at(b, g, f, idb, c, a, inva);
    }
    return acc * invb;
  }
  const int r = cb & 3, hi = cb >= 4;
  double acc = 0.0;
  for (int m = 0; m < 6; ++m) {
    if (carp1[r][m] == 0.0) continue;
    const long o = hi ? (long)(r - m) : (long)(m - r);
    acc += (hi ? -carp1[r][m] : carp1[r][m]) * d1at(b, g, f, id + o * g->st[bb], c, a, inva);
  }
  return acc * invb;
}

/* Viscous stress and heat-flux residual terms (generated "Viscous terms" kernel of the
 * supersonic TGV, Residual1..4 += ...); at isothermal-wall faces the derivatives take the
 * closures above (the generated kernels' idx-conditional branches). */
static void viscous_point(const osb_block_desc* b, const geom_t* g, const cr_t* c, long id, const int* pc, double* r) {
  const int nd = b->ndim;
  double inv[3], inv2[3];
  for (int d = 0; d < nd; ++d) { inv[d] = 1.0 / b->delta[d]; inv2[d] = 1.0 / (b->delta[d] * b->delta[d]); }
  /* stretched y (metric.py:199-240 with only SD111 non-zero): d/dx_1 = D11 d/dxi_1 and
   * d2/dx_1^2 = D11^2 d2/dxi_1^2 + D11 SD111 d/dxi_1 (the generated viscous kernel's
   * D11*D11*d2_u_dy + D11*wk*SD111); mixed derivatives take D11 once */
  double sd = 0.0;
  if (b->ystretch[0]) {
    const double d11 = b->ystretch[0][pc[1]];
    inv[1] *= d11;
    inv2[1] *= d11 * d11;
    sd = b->ystretch[1][pc[1]];
  }
  double du[3][3], lap[3], dmu[3], dT[3], lapT = 0.0;
  for (int i = 0; i < nd; ++i)
    for (int j = 0; j < nd; ++j) du[i][j] = d1at(b, g, c->u[i], id, pc, j, inv[j]);
  double div = 0.0;
  for (int i = 0; i < nd; ++i) div += du[i][i];
  for (int j = 0; j < nd; ++j) {
    dmu[j] = d1at(b, g, c->mu, id, pc, j, inv[j]);
    dT[j] = d1at(b, g, c->T, id, pc, j, inv[j]);
    lapT += d2at(b, g, c->T, id, pc, j, inv2[j]);
  }
  lapT += dT[1] * sd;
  /* lap_i = sum_j d2u_i/dx_j^2 + 1/3 d/dx_i (div u) */
  for (int i = 0; i < nd; ++i) {
    double s = 0.0;
    for (int j = 0; j < nd; ++j) s += d2at(b, g, c->u[i], id, pc, j, inv2[j]);
    s += du[i][1] * sd;
    s += (1.0 / 3.0) * (d2at(b, g, c->u[i], id, pc, i, inv2[i]) + (i == 1 ? du[1][1] * sd : 0.0));
    for (int j = 0; j < nd; ++j) {
      if (j == i) continue;
      int a = i < j ? i : j, bb = i < j ? j : i;
      s += (1.0 / 3.0) * dmixat(b, g, c->u[j], id, pc, a, bb, inv[a], inv[bb]);
    }
    lap[i] = s;
  }
  const double invRe = 1.0 / b->Re;
  const double mu = c->mu[id];
  double tau[3][3];
  for (int i = 0; i < nd; ++i)
    for (int j = 0; j < nd; ++j) tau[i][j] = du[i][j] + du[j][i] - (i == j ? (2.0 / 3.0) * div : 0.0);
  double e = 0.0;
  for (int i = 0; i < nd; ++i) {
    double m = 0.0;
    for (int j = 0; j < nd; ++j) m += tau[i][j] * dmu[j];
    m += mu * lap[i];
    r[1 + i] += m * invRe;
    double ui = c->u[i][id];
    for (int j = 0; j < nd; ++j) e += mu * tau[i][j] * du[i][j] + ui * tau[i][j] * dmu[j];
    e += mu * ui * lap[i];
  }
  double kheat = 1.0 / (b->Pr * b->Re * b->Minf * b->Minf * (b->gama - 1.0));
  double h = mu * lapT;
  for (int j = 0; j < nd; ++j) h += dT[j] * dmu[j];
  r[nd + 1] += e * invRe + h * kheat;
}

/* Skew-symmetric (Feiereisen) central convective terms (split_forms.py:111-145, generated
 * "Convective terms" kernel of the low-Mach TGV):
 *   R_rho  -= sum_j D_j(rhou_j)
 *   R_rhou_i -= D_i p + 1/2 sum_j [ D_j(rhou_i u_j) + u_i D_j(rhou_j) + rhou_j D_j(u_i) ]
 *   R_rhoE -= sum_j [ D_j(p u_j) + 1/2 ( D_j(rhoE u_j) + rhou_j D_j(rhoE/rho) + (rhoE/rho) D_j(rhou_j) ) ]
 * with D_j the central 4th-order first derivative. */
static void central_conv_point(const osb_block_desc* b, const geom_t* g, const cr_t* c, const double* const* tmp,
                               long id, double* r);

/* Kennedy-Gruber-Pirozzoli split convective terms (split_forms.py:178-236; the generated
 * "Convective terms" kernel of the Central4-WENO5 benchmark, opensbliblock00_kernels.h:157-330),
 * D_j the central 4th-order derivative, H = (rhoE + p)/rho, du_i/dx_j pointwise:
 *   R_rho    = -1/2 sum_j [ D_j(rhou_j) + rho du_j/dx_j + u_j D_j(rho) ]
 *   R_rhou_i = -D_i p - 1/4 sum_j [ D_j(u_i rhou_j) + rho D_j(u_i u_j) + u_i D_j(rhou_j) + u_j D_j(rhou_i)
 *                                   + rhou_i du_j/dx_j + rhou_j du_i/dx_j + u_i u_j D_j(rho) ]
 *   R_rhoE   = -1/4 sum_j [ D_j(H rhou_j) + rho D_j(H u_j) + H D_j(rhou_j) + u_j D_j(H rho)
 *                           + rhou_j D_j(H) + H rho du_j/dx_j + H u_j D_j(rho) ] */
static void central_kgp_point(const osb_block_desc* b, const geom_t* g, const cr_t* c, long id, double* r);

/* ---- residual ------------------------------------------------------------------------- */

typedef struct {
  int nblocks;
  osb_block_desc* blocks;
} set_t;

int oracle_residual(const osb_block_desc* b, double* const* Rout) {
  carpenter_init();
  geom_t g = geom_of(b);
  const int nd = b->ndim, nv = nd + 2;
  long n = npts_alloc(&g);
  cr_t c;
  cr_alloc(&c, n);
  cr_compute(b, &g, &c);
  for (int v = 0; v < nv; ++v)
    for (int k = 0; k < g.n[2]; ++k)
      for (int j = 0; j < g.n[1]; ++j)
        for (int i = 0; i < g.n[0]; ++i) Rout[v][gid(&g, i, j, k)] = 0.0;
  if (b->scheme == OSB_SCHEME_CENTRAL4) {
    /* quadratic products needed by the split form (precomputed over the extent) */
    double* tmp[1] = {NULL};
#pragma omp parallel for schedule(static)
    for (int k = 0; k < g.n[2]; ++k)
      for (int j = 0; j < g.n[1]; ++j)
        for (int i = 0; i < g.n[0]; ++i) {
          long id = gid(&g, i, j, k);
          double r[NVMAX] = {0, 0, 0, 0, 0};
          if (b->split_form == OSB_SPLIT_KGP) central_kgp_point(b, &g, &c, id, r);
          else central_conv_point(b, &g, &c, (const double* const*)tmp, id, r);
          for (int v = 0; v < nv; ++v) Rout[v][id] = r[v];
        }
  } else {
    /* interface fluxes per direction, stored like the generated wk arrays */
    double* fh[3][NVMAX];
    for (int d = 0; d < nd; ++d)
      for (int v = 0; v < nv; ++v) fh[d][v] = (double*)calloc(n, sizeof(double));
    /* every loop below writes each point from its own inputs only: the OpenMP split over the
     * outer index leaves the results bit-identical to a serial run */
    for (int d = 0; d < nd; ++d) {
      int lo[3] = {0, 0, 0};
      lo[d] = -1;
#pragma omp parallel for schedule(static)
      for (int k = lo[2]; k < g.n[2]; ++k)
        for (int j = lo[1]; j < g.n[1]; ++j)
          for (int i = lo[0]; i < g.n[0]; ++i) {
            long id = gid(&g, i, j, k);
            double f[NVMAX];
            if (b->metric[9]) char_flux_curv(b, &g, &c, d, id, f);
            else if (b->flux_type == OSB_FLUX_HLLC_LM) hllc_flux_cart(b, &g, &c, d, id, f);
            else char_flux_cart(b, &g, &c, d, id, f);
            for (int v = 0; v < nv; ++v) fh[d][v][id] = f[v];
          }
    }
#pragma omp parallel for schedule(static)
    for (int k = 0; k < g.n[2]; ++k)
      for (int j = 0; j < g.n[1]; ++j)
        for (int i = 0; i < g.n[0]; ++i) {
          long id = gid(&g, i, j, k);
          for (int v = 0; v < nv; ++v) {
            double r = 0.0;
            if (b->metric[9]) {
              /* curvilinear: R = -(sum_d dF_d / Delta_d) / det J */
              for (int d = 0; d < nd; ++d) r += (fh[d][v][id] - fh[d][v][id - g.st[d]]) * (1.0 / b->delta[d]);
              r = -r / b->metric[9][id];
            } else {
              for (int d = 0; d < nd; ++d) {
                /* stretched y: the generated residual's -(F_j - F_j-1) invDelta1 D11 */
                const double sc = (d == 1 && b->ystretch[0]) ? b->ystretch[0][j] : 1.0;
                r -= (fh[d][v][id] - fh[d][v][id - g.st[d]]) * (1.0 / b->delta[d]) * sc;
              }
            }
            Rout[v][id] = r;
          }
        }
    for (int d = 0; d < nd; ++d)
      for (int v = 0; v < nv; ++v) free(fh[d][v]);
  }
  if (b->viscous != OSB_VISC_NONE) {
#pragma omp parallel for schedule(static)
    for (int k = 0; k < g.n[2]; ++k)
      for (int j = 0; j < g.n[1]; ++j)
        for (int i = 0; i < g.n[0]; ++i) {
          long id = gid(&g, i, j, k);
          double r[NVMAX] = {0, 0, 0, 0, 0};
          const int pc[3] = {i, j, k};
          viscous_point(b, &g, &c, id, pc, r);
          for (int v = 1; v < nv; ++v) Rout[v][id] += r[v];
        }
  }
  if (b->forcing[0] != 0.0 || b->forcing[1] != 0.0 || b->forcing[2] != 0.0) {
    /* the channel apps' constant sources (turbulent_channel.py:38-39): -c_i in the momentum
     * equations, -sum_j c_j u_j in the energy equation */
#pragma omp parallel for schedule(static)
    for (int k = 0; k < g.n[2]; ++k)
      for (int j = 0; j < g.n[1]; ++j)
        for (int i = 0; i < g.n[0]; ++i) {
          long id = gid(&g, i, j, k);
          double w = 0.0;
          for (int e = 0; e < nd; ++e) {
            Rout[1 + e][id] -= b->forcing[e];
            w += b->forcing[e] * c.u[e][id];
          }
          Rout[nv - 1][id] -= w;
        }
  }
  cr_free(&c);
  return 0;
}

static void central_conv_point(const osb_block_desc* b, const geom_t* g, const cr_t* c, const double* const* tmp,
                               long id, double* r) {
  (void)tmp;
  const int nd = b->ndim, nv = nd + 2;
  const double* rho = b->q[0];
  const double* rhoE = b->q[nv - 1];
  double inv[3];
  for (int d = 0; d < nd; ++d) inv[d] = 1.0 / b->delta[d];
  double E = rhoE[id] / rho[id];
  double divm = 0.0; /* sum_j d(rhou_j)/dx_j */
  for (int j = 0; j < nd; ++j) divm += d1c(b->q[1 + j], id, g->st[j], inv[j]);
  r[0] -= divm;
  for (int i = 0; i < nd; ++i) {
    double acc = d1c(c->p, id, g->st[i], inv[i]);
    double adv = 0.0, conv = 0.0;
    for (int j = 0; j < nd; ++j) {
      long s = g->st[j];
      double pr = 0.0;
      for (int m = 0; m < 5; ++m) {
        if (m == 2) continue;
        long im = id + (long)(m - 2) * s;
        pr += C1[m] * b->q[1 + i][im] * c->u[j][im];
      }
      conv += pr * inv[j];
      adv += b->q[1 + j][id] * d1c(c->u[i], id, s, inv[j]);
    }
    acc += 0.5 * (conv + c->u[i][id] * divm + adv);
    r[1 + i] -= acc;
  }
  double e = 0.0;
  for (int j = 0; j < nd; ++j) {
    long s = g->st[j];
    double dpu = 0.0, dEu = 0.0, dE = 0.0;
    for (int m = 0; m < 5; ++m) {
      if (m == 2) continue;
      long im = id + (long)(m - 2) * s;
      dpu += C1[m] * c->p[im] * c->u[j][im];
      dEu += C1[m] * rhoE[im] * c->u[j][im];
      dE += C1[m] * rhoE[im] / rho[im];
    }
    e += dpu * inv[j] + 0.5 * (dEu * inv[j] + b->q[1 + j][id] * dE * inv[j]);
  }
  e += 0.5 * divm * E;
  r[nv - 1] -= e;
}

/* central 4th-order derivative of the product f * h along stride s */
static inline double d1p(const double* f, const double* h, long id, long s, double invd) {
  return ((1.0 / 12.0) * f[id - 2 * s] * h[id - 2 * s] - (2.0 / 3.0) * f[id - s] * h[id - s] +
          (2.0 / 3.0) * f[id + s] * h[id + s] - (1.0 / 12.0) * f[id + 2 * s] * h[id + 2 * s]) * invd;
}
/* ... of f * h * k */
static inline double d1p3(const double* f, const double* h, const double* k, long id, long s, double invd) {
  return ((1.0 / 12.0) * f[id - 2 * s] * h[id - 2 * s] * k[id - 2 * s] - (2.0 / 3.0) * f[id - s] * h[id - s] * k[id - s] +
          (2.0 / 3.0) * f[id + s] * h[id + s] * k[id + s] -
          (1.0 / 12.0) * f[id + 2 * s] * h[id + 2 * s] * k[id + 2 * s]) * invd;
}

static void central_kgp_point(const osb_block_desc* b, const geom_t* g, const cr_t* c, long id, double* r) {
  const int nd = b->ndim, nv = nd + 2;
  const double* rho = b->q[0];
  double inv[3];
  for (int d = 0; d < nd; ++d) inv[d] = 1.0 / b->delta[d];
  /* H = (rhoE + p) / rho on the 13-point cross around id */
  double Hs[3][5];
  for (int j = 0; j < nd; ++j)
    for (int m = 0; m < 5; ++m) {
      long im = id + (long)(m - 2) * g->st[j];
      Hs[j][m] = (b->q[nv - 1][im] + c->p[im]) / rho[im];
    }
  const double H0 = Hs[0][2];
  double du[3][3];
  for (int i = 0; i < nd; ++i)
    for (int j = 0; j < nd; ++j) du[i][j] = d1c(c->u[i], id, g->st[j], inv[j]);
  double divu = 0.0, divm = 0.0;
  for (int j = 0; j < nd; ++j) {
    divu += du[j][j];
    divm += d1c(b->q[1 + j], id, g->st[j], inv[j]);
  }
  double drho[3];
  for (int j = 0; j < nd; ++j) drho[j] = d1c(rho, id, g->st[j], inv[j]);
  /* continuity */
  double rc = divm + rho[id] * divu;
  for (int j = 0; j < nd; ++j) rc += c->u[j][id] * drho[j];
  r[0] -= 0.5 * rc;
  /* momentum */
  for (int i = 0; i < nd; ++i) {
    double acc = 0.0;
    for (int j = 0; j < nd; ++j) {
      long s = g->st[j];
      acc += d1p(c->u[i], b->q[1 + j], id, s, inv[j]) + rho[id] * d1p(c->u[i], c->u[j], id, s, inv[j]) +
             c->u[i][id] * d1c(b->q[1 + j], id, s, inv[j]) + c->u[j][id] * d1c(b->q[1 + i], id, s, inv[j]) +
             b->q[1 + i][id] * du[j][j] + b->q[1 + j][id] * du[i][j] + c->u[i][id] * c->u[j][id] * drho[j];
    }
    r[1 + i] -= d1c(c->p, id, g->st[i], inv[i]) + 0.25 * acc;
  }
  /* energy */
  double e = 0.0;
  for (int j = 0; j < nd; ++j) {
    double Hq = 0.0, Hu = 0.0, Hr = 0.0, dH = 0.0;
    for (int m = 0; m < 5; ++m) {
      if (m == 2) continue;
      long im = id + (long)(m - 2) * g->st[j];
      Hq += C1[m] * Hs[j][m] * b->q[1 + j][im];
      Hu += C1[m] * Hs[j][m] * c->u[j][im];
      Hr += C1[m] * Hs[j][m] * rho[im];
      dH += C1[m] * Hs[j][m];
    }
    e += Hq * inv[j] + rho[id] * Hu * inv[j] + H0 * d1c(b->q[1 + j], id, g->st[j], inv[j]) + c->u[j][id] * Hr * inv[j] +
         b->q[1 + j][id] * dH * inv[j] + H0 * rho[id] * du[j][j] + H0 * c->u[j][id] * drho[j];
  }
  r[nv - 1] -= 0.25 * e;
}

/* ---- non-linear WENO filter (filters/WENO_filter.py) ----------------------------------------
 * Applied after every full RK step, as the generated Central4-WENO5 benchmark does
 * (opensbli.cpp:389-513): primitives over the halo'd range, the Ducros sensor kappa on the
 * interior (kernel 044; its halos stay zero), one characteristic WENO3 filter flux per direction
 * and interface i+1/2, i = -1..N-1 (kernels 046-048), then q += dt * mask * (-sum_d dF_d / Delta_d)
 * with mask = [max kappa over the point and its neighbours >= Ducros_select] (kernel 049). */

/* Ducros sensor at interior point id (kernel 044). */
static double ducros_kappa(const osb_block_desc* b, const geom_t* g, const cr_t* c, long id) {
  double inv[3];
  for (int d = 0; d < 3; ++d) inv[d] = 1.0 / b->delta[d];
  double du[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) du[i][j] = d1c(c->u[i], id, g->st[j], inv[j]);
  const double div = du[0][0] + du[1][1] + du[2][2];
  const double h = sqrt(b->delta[0] * b->delta[0] + b->delta[1] * b->delta[1] + b->delta[2] * b->delta[2]);
  const double wz = -du[0][1] + du[1][0], wx = -du[1][2] + du[2][1], wy = -du[2][0] + du[0][2];
  return (div * div) * (0.5 - 0.5 * tanh(2.5 + 500.0 * div / h)) / (1.0e-40 + wz * wz + wx * wx + wy * wy + div * div);
}

/* Filter flux at interface i+1/2 along direction d, idc = point i (kernels 046-048):
 * Roe-averaged eigensystem, CS = L Q and CF = L F on points i-1..i+2, per wave the WENO3-Z
 * reconstruction of both split fluxes CF +/- lambda CS (epsilon 1e-40, optimal weights 2/3,
 * 1/3) minus the central 4th-order interpolation of CF, scaled by the smoothness sensor
 * rj = max over both sides of (|3 w_a - 1| + |3/2 w_b - 1|) / 3; back to physical space with R. */
static void filter_flux(const osb_block_desc* b, const geom_t* g, const cr_t* c, const double* kappa, int d,
                        long idc, double* fhat) {
  const int nd = 3, nv = 5;
  const long s = g->st[d];
  double km = kappa[idc - 3 * s];
  for (int m = -2; m <= 2; ++m) km = fmax(km, kappa[idc + m * s]);
  if (!(km > b->ducros_check)) {
    for (int v = 0; v < nv; ++v) fhat[v] = 0.0;
    return;
  }
  const double gm = b->gama;
  double kt[3] = {0.0, 0.0, 0.0};
  kt[d] = 1.0;
  long iL = idc, iR = idc + s;
  double rL = b->q[0][iL], rR = b->q[0][iR];
  double sL = sqrt(rL), sR = sqrt(rR);
  double rho_av = sqrt(rL * rR);
  double inv = 1.0 / (sL + sR);
  double u_av[3], ke = 0.0;
  for (int i = 0; i < nd; ++i) {
    u_av[i] = (sL * c->u[i][iL] + sR * c->u[i][iR]) * inv;
    ke += u_av[i] * u_av[i];
  }
  double a_av = sqrt((-0.5 * ke + ((c->p[iL] + b->q[nv - 1][iL]) / sL + (c->p[iR] + b->q[nv - 1][iR]) / sR) * inv) *
                     (gm - 1.0));
  double L[NVMAX][NVMAX], R[NVMAX][NVMAX];
  eigensystem(nd, gm, kt, rho_av, u_av, a_av, L, R);
  double lam[NVMAX], evL[NVMAX], evR[NVMAX];
  double uL[3], uR[3];
  for (int i = 0; i < nd; ++i) { uL[i] = c->u[i][iL]; uR[i] = c->u[i][iR]; }
  point_ev(nd, kt, 1.0, uL, c->a[iL], evL);
  point_ev(nd, kt, 1.0, uR, c->a[iR], evR);
  for (int w = 0; w < nv; ++w) lam[w] = b->shock_filter_control * fmax(fabs(evR[w]), fabs(evL[w]));
  double CS[NVMAX][4], CF[NVMAX][4];
  for (int m = 0; m < 4; ++m) {
    long id = idc + (long)(m - 1) * s;
    double Q[NVMAX], F[NVMAX];
    double ud = c->u[d][id], p = c->p[id];
    for (int v = 0; v < nv; ++v) Q[v] = b->q[v][id];
    F[0] = Q[1 + d];
    for (int i = 0; i < nd; ++i) F[1 + i] = ud * Q[1 + i] + (i == d ? p : 0.0);
    F[nv - 1] = ud * (Q[nv - 1] + p);
    for (int w = 0; w < nv; ++w) {
      double cs = 0.0, cf = 0.0;
      for (int v = 0; v < nv; ++v) { cs += L[w][v] * Q[v]; cf += L[w][v] * F[v]; }
      CS[w][m] = cs;
      CF[w][m] = cf;
    }
  }
  double rec[NVMAX];
  for (int w = 0; w < nv; ++w) {
    const double lw = lam[w];
    double fp[4], fm[4];
    for (int m = 0; m < 4; ++m) {
      fp[m] = CS[w][m] * lw + CF[w][m];
      fm[m] = -CS[w][m] * lw + CF[w][m];
    }
    double b0, b1, t, a0, a1, ia, w0, w1, rj, rc = 0.0;
    /* + side: stencils {i, i+1} (weight 2/3) and {i-1, i} (1/3) */
    b0 = (1.0 / 4.0) * (fp[2] * fp[2]) + (1.0 / 2.0) * ((1.0 / 2.0) * fp[1] - fp[2]) * fp[1];
    b1 = (1.0 / 4.0) * (fp[1] * fp[1]) + (1.0 / 2.0) * ((1.0 / 2.0) * fp[0] - fp[1]) * fp[0];
    t = fabs(-b1 + b0) * fabs(-b1 + b0);
    a0 = 0.666666666666667 + (2.0 / 3.0) * t / ((1.0e-40 + b0) * (1.0e-40 + b0));
    a1 = 0.333333333333333 + (1.0 / 3.0) * t / ((1.0e-40 + b1) * (1.0e-40 + b1));
    ia = 1.0 / (a0 + a1);
    w0 = a0 * ia;
    w1 = a1 * ia;
    rj = 0.333333333333333 * fabs(-1.0 + 3 * w1) + 0.333333333333333 * fabs(-1.0 + (3.0 / 2.0) * w0);
    rc = (-(1.0 / 4.0) * fp[0] + (3.0 / 4.0) * fp[1]) * w1 + ((1.0 / 4.0) * fp[1] + (1.0 / 4.0) * fp[2]) * w0 + rc;
    /* - side: stencils {i+1, i+2} (1/3) and {i, i+1} (2/3) */
    b0 = (1.0 / 4.0) * (fm[3] * fm[3]) + (1.0 / 2.0) * ((1.0 / 2.0) * fm[2] - fm[3]) * fm[2];
    b1 = (1.0 / 4.0) * (fm[2] * fm[2]) + (1.0 / 2.0) * ((1.0 / 2.0) * fm[1] - fm[2]) * fm[1];
    t = fabs(-b1 + b0) * fabs(-b1 + b0);
    a0 = 0.333333333333333 + (1.0 / 3.0) * t / ((1.0e-40 + b0) * (1.0e-40 + b0));
    a1 = 0.666666666666667 + (2.0 / 3.0) * t / ((1.0e-40 + b1) * (1.0e-40 + b1));
    ia = 1.0 / (a0 + a1);
    w0 = a0 * ia;
    w1 = a1 * ia;
    rj = fmax(rj, 0.333333333333333 * fabs(-1.0 + 3 * w0) + 0.333333333333333 * fabs(-1.0 + (3.0 / 2.0) * w1));
    rc = (-(1.0 / 4.0) * fm[3] + (3.0 / 4.0) * fm[2]) * w0 + ((1.0 / 4.0) * fm[1] + (1.0 / 4.0) * fm[2]) * w1 + rc;
    rec[w] = ((1.0 / 12.0) * (-7 * CF[w][1] - 7 * CF[w][2] + CF[w][0] + CF[w][3]) + rc) * rj;
  }
  for (int v = 0; v < nv; ++v) {
    double acc = 0.0;
    for (int w = 0; w < nv; ++w) acc += R[v][w] * rec[w];
    fhat[v] = acc;
  }
}

/* The halo exchange the generated code runs between the last RK stage and the filter
 * (bc_exchanges.h groups 51-56 of the Central4-WENO5 benchmark): per direction d, side 0
 * copies [0, 4) to [N, N+4) and side 1 copies [N-4, N) to [-4, 0), over the transverse range
 * [-4, N-4) of the other directions (the generator's iteration range: base -4, extent N), in
 * the order x, y, z.  No exchange follows the last stage, so halo points outside that range
 * keep the values of the exchange after the previous stage. */
static void filter_halos(osb_block_desc* b, const geom_t* g) {
  const int nv = 5;
  for (int d = 0; d < 3; ++d)
    for (int side = 0; side < 2; ++side) {
      int lo[3], ext[3];
      for (int e = 0; e < 3; ++e) {
        lo[e] = -4;
        ext[e] = g->n[e];
      }
      lo[d] = 0;
      ext[d] = 4;
      for (int c2 = 0; c2 < ext[2]; ++c2)
        for (int c1 = 0; c1 < ext[1]; ++c1)
          for (int c0 = 0; c0 < ext[0]; ++c0) {
            int src[3] = {lo[0] + c0, lo[1] + c1, lo[2] + c2}, dst[3];
            for (int e = 0; e < 3; ++e) dst[e] = src[e];
            if (side == 0) {
              dst[d] = g->n[d] + src[d];
            } else {
              src[d] = g->n[d] - 4 + src[d];
              dst[d] = src[d] - g->n[d];
            }
            long si = gid(g, src[0], src[1], src[2]), di = gid(g, dst[0], dst[1], dst[2]);
            for (int v = 0; v < nv; ++v) b->q[v][di] = b->q[v][si];
          }
    }
}

static void weno_filter_block(osb_block_desc* b, double dt) {
  {
    geom_t g = geom_of(b);
    const int nv = 5;
    long n = npts_alloc(&g);
    filter_halos(b, &g);
    cr_t c;
    cr_alloc(&c, n);
    cr_compute(b, &g, &c);
    double* kappa = alloc_like(&g);
    for (int k = 0; k < g.n[2]; ++k)
      for (int j = 0; j < g.n[1]; ++j)
        for (int i = 0; i < g.n[0]; ++i) {
          long id = gid(&g, i, j, k);
          kappa[id] = ducros_kappa(b, &g, &c, id);
        }
    double* F[3][NVMAX];
    for (int d = 0; d < 3; ++d)
      for (int v = 0; v < nv; ++v) F[d][v] = alloc_like(&g);
    for (int d = 0; d < 3; ++d) {
      int lo[3] = {0, 0, 0};
      lo[d] = -1;
      for (int k = lo[2]; k < g.n[2]; ++k)
        for (int j = lo[1]; j < g.n[1]; ++j)
          for (int i = lo[0]; i < g.n[0]; ++i) {
            long id = gid(&g, i, j, k);
            double f[NVMAX];
            filter_flux(b, &g, &c, kappa, d, id, f);
            for (int v = 0; v < nv; ++v) F[d][v][id] = f[v];
          }
    }
    const double i0 = 1.0 / b->delta[0], i1 = 1.0 / b->delta[1], i2 = 1.0 / b->delta[2];
    for (int k = 0; k < g.n[2]; ++k)
      for (int j = 0; j < g.n[1]; ++j)
        for (int i = 0; i < g.n[0]; ++i) {
          long id = gid(&g, i, j, k);
          const long sx = g.st[0], sy = g.st[1], sz = g.st[2];
          double km = kappa[id];
          const long nb[9] = {id + sz, id + 2 * sy, id + sx, id - sy, id - sx, id + sy, id + 2 * sz, id + 2 * sx, id - sz};
          for (int m = 0; m < 9; ++m) km = fmax(km, kappa[nb[m]]);
          const double mask = km >= b->ducros_select ? 1.0 : 0.0;
          for (int v = 0; v < nv; ++v) {
            const double* f0 = F[0][v];
            const double* f1 = F[1][v];
            const double* f2 = F[2][v];
            b->q[v][id] = (-(-f0[id - sx] + f0[id]) * i0 - (-f2[id - sz] + f2[id]) * i2 - (-f1[id - sy] + f1[id]) * i1 * 1.0) *
                              dt * mask + b->q[v][id];
          }
        }
    for (int d = 0; d < 3; ++d)
      for (int v = 0; v < nv; ++v) free(F[d][v]);
    free(kappa);
    cr_free(&c);
  }
}

/* ---- non-linear TVD filter (filters/TVD_filter.py) ------------------------------------------
 * The Yee-Sandham-Djomehri characteristic filter of schemes/spatial/shock_capturing.py:619-766
 * with Harten's switch, applied after every full RK step as the generated solver of the TGV
 * app's TVD branch runs it (apps/compressible_taylor_green_vortex/compressible_TGV.py:210-222;
 * kernels "Constituent Relations evaluation", "TVD reconstruction direction d" and
 * "Non-linear TVD Filter application"): the filter's exchange (filter_halos), u and a on
 * [-1, N+2) of every direction, per direction the flux at interfaces i+1/2, i = -1..N-1, then
 * q += dt * (-(F_0(i) - F_0(i-1)) / Delta_0 - (F_2 ..) / Delta_2 - (F_1 ..) / Delta_1).
 * The interface at -1 reads point -2 of the sweep direction, outside that constituent range:
 * there a keeps its zero initial value and u the value the last RK stage's constituent
 * relations left (rhou / rho of the state at the start of that stage), passed in as stale. */

typedef struct {
  double r, m[3], e, u[3], a; /* local frame: m[0], u[0] normal, then the two transverse */
} tvd_pt;

/* Entropy fix of a wave speed, delta_TVD = 0.5 (shock_capturing.py:681-689). */
static double tvd_psi(double z) {
  const double idl = 1.0 / 0.5; /* invdelta_TVD */
  return fabs(z) >= 1.0 / idl ? fabs(z) : (1.0 / 2.0) * (1.0 / (idl * idl) + z * z) * idl;
}

/* Limiter g from the jumps hi (this interface) and lo (the one below) (lines 690-704). */
static double tvd_g(double hi, double lo) {
  const double S = hi > 0 ? 1.0 : (hi < 0 ? -1.0 : 0.0);
  const double t1 = fmax(0.0, fmin(S * lo, 2 * fabs(hi)));
  const double t2 = fmin(fabs(hi), 2 * S * lo);
  return S * fmax(t1, t2);
}

/* Filter flux at interface i+1/2 from points w[0..3] = i-1..i+2 (local frame), in the
 * operation order of the generated direction-0 kernel: simple averages over (i-1, i), (i, i+1),
 * (i+1, i+2), alpha = LEV (q_hi - q_lo) at each, wave speeds and REV at i+1/2, sigma, g,
 * gamma, phi, Harten's theta, phi* = kappa theta phi, F = 1/2 REV phi*. */
static void tvd_flux(double gm, double kappa, const tvd_pt* w, double* fh) {
  const double g1 = -1 + gm, eps = 1.0e-8;
  const double c1 = 0.35355339059327373, c2 = 0.70710678118654746;
  double al[5][3], ws[5] = {0, 0, 0, 0, 0}, R[5][5];
  memset(R, 0, sizeof(R));
  for (int jb = 0; jb < 3; ++jb) {
    const tvd_pt* lo = &w[jb];
    const tvd_pt* hi = &w[jb + 1];
    const double u0 = (1.0 / 2.0) * (lo->u[0] + hi->u[0]), u1 = (1.0 / 2.0) * (lo->u[1] + hi->u[1]),
                 u2 = (1.0 / 2.0) * (lo->u[2] + hi->u[2]), a = (1.0 / 2.0) * (lo->a + hi->a),
                 rho = (1.0 / 2.0) * (lo->r + hi->r);
    const double ia = 1.0 / a, ir = 1.0 / rho, ia2 = ia * ia;
    const double L00 = -(1.0 / 2.0) * (-2 - (u0 * u0) * ia2 - (u1 * u1) * ia2 - (u2 * u2) * ia2 + (u0 * u0) * ia2 * gm +
                                        (u1 * u1) * ia2 * gm + (u2 * u2) * ia2 * gm);
    const double L01 = ia2 * g1 * u0, L02 = ia2 * g1 * u1, L03 = ia2 * g1 * u2, L04 = -ia2 * g1;
    const double L10 = -u2 * ir, L13 = ir, L20 = u1 * ir, L22 = -ir;
    const double kq = -(u0 * u0) * ia - (u1 * u1) * ia - (u2 * u2) * ia;
    const double L30 = c1 * (-2 * u0 + kq + (u0 * u0) * gm * ia + (u1 * u1) * gm * ia + (u2 * u2) * gm * ia) * ir;
    const double L40 = c1 * (2 * u0 + kq + (u0 * u0) * gm * ia + (u1 * u1) * gm * ia + (u2 * u2) * gm * ia) * ir;
    const double L31 = -c2 * (-1 - u0 * ia + gm * u0 * ia) * ir, L41 = -c2 * (1 - u0 * ia + gm * u0 * ia) * ir;
    const double L32 = -c2 * g1 * u1 * ia * ir, L33 = -c2 * g1 * u2 * ia * ir, L34 = c2 * g1 * ia * ir;
    const double dr = -lo->r + hi->r, d0 = -lo->m[0] + hi->m[0], d1 = -lo->m[1] + hi->m[1],
                 d2 = -lo->m[2] + hi->m[2], de = -lo->e + hi->e;
    al[0][jb] = dr * L00 + de * L04 + d0 * L01 + d1 * L02 + d2 * L03;
    al[1][jb] = dr * L10 + d2 * L13;
    al[2][jb] = dr * L20 + d1 * L22;
    al[3][jb] = dr * L30 + de * L34 + d0 * L31 + d1 * L32 + d2 * L33;
    al[4][jb] = dr * L40 + de * L34 + d0 * L41 + d1 * L32 + d2 * L33;
    if (jb == 1) {
      ws[0] = ws[1] = ws[2] = u0;
      ws[3] = a + u0;
      ws[4] = -a + u0;
      R[0][0] = 1;
      R[0][3] = R[0][4] = c2 * rho * ia;
      R[1][0] = u0;
      R[1][3] = c2 * (a + u0) * rho * ia;
      R[1][4] = c2 * (-a + u0) * rho * ia;
      R[2][0] = u1;
      R[2][2] = -rho;
      R[2][3] = R[2][4] = c2 * rho * u1 * ia;
      R[3][0] = u2;
      R[3][1] = rho;
      R[3][3] = R[3][4] = c2 * rho * u2 * ia;
      R[4][0] = (1.0 / 2.0) * (u0 * u0) + (1.0 / 2.0) * (u1 * u1) + (1.0 / 2.0) * (u2 * u2);
      R[4][1] = rho * u2;
      R[4][2] = -rho * u1;
      const double hq = ((a * a) + (1.0 / 2.0) * (1 - 1 + g1) * ((u0 * u0) + (u1 * u1) + (u2 * u2))) / (1 - 1 + g1);
      R[4][3] = c2 * (hq + a * u0) * rho * ia;
      R[4][4] = c2 * (hq - a * u0) * rho * ia;
    }
  }
  double ps[5];
  for (int k = 0; k < 5; ++k) {
    const double s0 = tvd_psi(ws[k]);
    const double g0 = tvd_g(al[k][1], al[k][0]), gg1 = tvd_g(al[k][2], al[k][1]);
    const double gam = al[k][1] == 0 ? 0 : (-g0 + gg1) * al[k][1] * s0 / ((al[k][1] * al[k][1]) + eps);
    const double s1 = tvd_psi(gam);
    const double phi = -fabs(s0 + s1) * al[k][1] + 0.5 * (g0 + gg1) * s0;
    double t1 = -fabs(al[k][0]) + fabs(al[k][1]), t2 = fabs(al[k][0]) + fabs(al[k][1]) + eps;
    const double th0 = fabs(t1 / t2) * fabs(t1 / t2);
    t1 = -fabs(al[k][1]) + fabs(al[k][2]);
    t2 = fabs(al[k][1]) + fabs(al[k][2]) + eps;
    const double th1 = fabs(t1 / t2) * fabs(t1 / t2);
    ps[k] = kappa * phi * fmax(th0, th1);
  }
  fh[0] = 0.5 * R[0][0] * ps[0] + 0.5 * R[0][3] * ps[3] + 0.5 * R[0][4] * ps[4];
  fh[1] = 0.5 * R[1][0] * ps[0] + 0.5 * R[1][3] * ps[3] + 0.5 * R[1][4] * ps[4];
  fh[2] = 0.5 * R[2][0] * ps[0] + 0.5 * R[2][2] * ps[2] + 0.5 * R[2][3] * ps[3] + 0.5 * R[2][4] * ps[4];
  fh[3] = 0.5 * R[3][0] * ps[0] + 0.5 * R[3][1] * ps[1] + 0.5 * R[3][3] * ps[3] + 0.5 * R[3][4] * ps[4];
  fh[4] = 0.5 * R[4][0] * ps[0] + 0.5 * R[4][1] * ps[1] + 0.5 * R[4][2] * ps[2] + 0.5 * R[4][3] * ps[3] +
          0.5 * R[4][4] * ps[4];
}

/* u at index -2 of each direction (the other two interior): rhou / rho of the current state,
 * one array per velocity component over the whole allocation (only those faces are set). */
static void tvd_stale_capture(const osb_block_desc* b, const geom_t* g, double* const* st) {
  for (int d = 0; d < 3; ++d) {
    int lo[3] = {0, 0, 0}, hi[3] = {g->n[0], g->n[1], g->n[2]};
    lo[d] = -2;
    hi[d] = -1;
    for (int k = lo[2]; k < hi[2]; ++k)
      for (int j = lo[1]; j < hi[1]; ++j)
        for (int i = lo[0]; i < hi[0]; ++i) {
          long id = gid(g, i, j, k);
          for (int c = 0; c < 3; ++c) st[c][id] = b->q[1 + c][id] / b->q[0][id];
        }
  }
}

static void tvd_filter_block(osb_block_desc* b, double dt, double* const* stale) {
  geom_t g = geom_of(b);
  const int nv = 5;
  const double gm = b->gama;
  filter_halos(b, &g);
  double* F[3][NVMAX];
  for (int d = 0; d < 3; ++d)
    for (int v = 0; v < nv; ++v) F[d][v] = alloc_like(&g);
  for (int d = 0; d < 3; ++d) {
    const int t1 = (d + 1) % 3, t2 = (d + 2) % 3;
    int lo[3] = {0, 0, 0};
    lo[d] = -1;
    for (int k = lo[2]; k < g.n[2]; ++k)
      for (int j = lo[1]; j < g.n[1]; ++j)
        for (int i = lo[0]; i < g.n[0]; ++i) {
          const long id = gid(&g, i, j, k);
          const int cd = d == 0 ? i : (d == 1 ? j : k);
          tvd_pt w[4];
          for (int m = 0; m < 4; ++m) {
            const long p = id + (long)(m - 1) * g.st[d];
            const int comp[3] = {d, t1, t2};
            tvd_pt* s = &w[m];
            s->r = b->q[0][p];
            s->e = b->q[4][p];
            for (int c = 0; c < 3; ++c) s->m[c] = b->q[1 + comp[c]][p];
            if (cd + m - 1 == -2) {
              for (int c = 0; c < 3; ++c) s->u[c] = stale[comp[c]][p];
              s->a = 0.0;
            } else {
              /* "Constituent Relations evaluation" of the filter */
              const double inv_rho = 1.0 / b->q[0][p];
              for (int c = 0; c < 3; ++c) s->u[c] = b->q[1 + comp[c]][p] * inv_rho;
              const double p_ = (-1 + gm) * (-(0.5 * (b->q[1][p] * b->q[1][p]) + 0.5 * (b->q[2][p] * b->q[2][p]) +
                                               0.5 * (b->q[3][p] * b->q[3][p])) * inv_rho + b->q[4][p]);
              s->a = sqrt(gm * p_ * inv_rho);
            }
          }
          double f[5];
          tvd_flux(gm, b->tvd_kappa, w, f);
          F[d][0][id] = f[0];
          F[d][1 + d][id] = f[1];
          F[d][1 + t1][id] = f[2];
          F[d][1 + t2][id] = f[3];
          F[d][4][id] = f[4];
        }
  }
  const double i0 = 1.0 / b->delta[0], i1 = 1.0 / b->delta[1], i2 = 1.0 / b->delta[2];
  for (int k = 0; k < g.n[2]; ++k)
    for (int j = 0; j < g.n[1]; ++j)
      for (int i = 0; i < g.n[0]; ++i) {
        const long id = gid(&g, i, j, k);
        const long sx = g.st[0], sy = g.st[1], sz = g.st[2];
        for (int v = 0; v < nv; ++v) {
          const double* f0 = F[0][v];
          const double* f1 = F[1][v];
          const double* f2 = F[2][v];
          b->q[v][id] = (-(-f0[id - sx] + f0[id]) * i0 - (-f2[id - sz] + f2[id]) * i2 - (-f1[id - sy] + f1[id]) * i1 * 1.0) *
                            dt + b->q[v][id];
        }
      }
  for (int d = 0; d < 3; ++d)
    for (int v = 0; v < nv; ++v) free(F[d][v]);
}

/* The filter step of every filtered block.  stale: per block three velocity arrays for the TVD
 * filter's point -2 (NULL: taken from the current state). */
static int filter_impl(osb_block_desc* blocks, int nblocks, double dt, double* const* const* stale) {
  for (int ib = 0; ib < nblocks; ++ib) {
    osb_block_desc* b = &blocks[ib];
    if (b->filter == OSB_FILTER_NONE) continue;
    if (b->ndim != 3) return -1;
    if (b->filter == OSB_FILTER_WENO3) {
      weno_filter_block(b, dt);
    } else if (b->filter == OSB_FILTER_TVD) {
      geom_t g = geom_of(b);
      double* own[3] = {NULL, NULL, NULL};
      if (!stale || !stale[ib]) {
        for (int c = 0; c < 3; ++c) own[c] = alloc_like(&g);
        tvd_stale_capture(b, &g, own);
      }
      tvd_filter_block(b, dt, (stale && stale[ib]) ? stale[ib] : own);
      for (int c = 0; c < 3; ++c) free(own[c]);
    } else {
      return -1;
    }
  }
  return 0;
}

int oracle_filter(osb_block_desc* blocks, int nblocks, double dt) { return filter_impl(blocks, nblocks, dt, NULL); }

/* ---- boundary conditions ---------------------------------------------------------------- */

/* Periodic exchange of one face, as ops_halo_transfer of the generated bc_exchanges.h:
 * side 0 copies interior [0, depth) to the high halo [N, N+depth); side 1 copies
 * [N-depth, N) to [-depth, 0).  Transverse extent covers -depth..N+depth of the other used
 * directions (periodic.py:53-71 with corners). */
static void periodic_face(osb_block_desc* b, const geom_t* g, int d, int side, int depth) {
  const int nd = b->ndim, nv = nd + 2;
  int lo[3], hi[3];
  for (int e = 0; e < 3; ++e) {
    if (e < nd) { lo[e] = -depth; hi[e] = g->n[e] + depth; } else { lo[e] = 0; hi[e] = 1; }
  }
  int N = g->n[d];
  int from0 = side == 0 ? 0 : N - depth;
  int to0 = side == 0 ? N : -depth;
  lo[d] = 0; hi[d] = depth;
  for (int v = 0; v < nv; ++v)
    for (int k = lo[2]; k < hi[2]; ++k)
      for (int j = lo[1]; j < hi[1]; ++j)
        for (int i = lo[0]; i < hi[0]; ++i) {
          int src[3] = {i, j, k}, dst[3] = {i, j, k};
          src[d] += from0; dst[d] += to0;
          b->q[v][gid(g, dst[0], dst[1], dst[2])] = b->q[v][gid(g, src[0], src[1], src[2])];
        }
}

/* Zero-gradient outlet: q(0) = q(1), q(-m) = q(m) for m = 1..depth at side 0 (mirrored at
 * side 1), over the full transverse extent of the boundary plane (zero_gradient_outlet.py). */
static void zero_grad_face(osb_block_desc* b, const geom_t* g, int d, int side, int depth) {
  const int nd = b->ndim, nv = nd + 2;
  int lo[3], hi[3];
  for (int e = 0; e < 3; ++e) {
    if (e < nd) { lo[e] = 0; hi[e] = g->n[e]; } else { lo[e] = 0; hi[e] = 1; }
  }
  int N = g->n[d];
  int base = side == 0 ? 0 : N - 1;
  int sgn = side == 0 ? 1 : -1;
  lo[d] = base; hi[d] = base + 1;
  for (int k = lo[2]; k < hi[2]; ++k)
    for (int j = lo[1]; j < hi[1]; ++j)
      for (int i = lo[0]; i < hi[0]; ++i) {
        long id = gid(g, i, j, k);
        long s = g->st[d] * sgn;
        for (int v = 0; v < nv; ++v) {
          double* q = b->q[v];
          q[id] = q[id + s];
          for (int m = 1; m <= depth; ++m) q[id - m * s] = q[id + m * s];
        }
      }
}

/* Extrapolation boundary (extrapolation.py:29-53 as generated), boundary point b = 0 on side 0,
 * N-1 on side 1, outward step o = -1 / +1.  Order 0: q(b) = q(b-o), then q(b+m o) = q(b-o) for
 * m = 1..depth.  Order 1: q(b+m o) = 2 q(b+(m-1) o) - q(b+(m-2) o) for m = 1..depth, in that
 * order (each layer from the two before it).  Over the interior transverse extent. */
static void extrap_face(osb_block_desc* b, const geom_t* g, int d, int side, int depth, int order) {
  const int nd = b->ndim, nv = nd + 2;
  int lo[3], hi[3];
  for (int e = 0; e < 3; ++e) {
    if (e < nd) { lo[e] = 0; hi[e] = g->n[e]; } else { lo[e] = 0; hi[e] = 1; }
  }
  const int N = g->n[d];
  const int base = side == 0 ? 0 : N - 1;
  lo[d] = base; hi[d] = base + 1;
  const long o = g->st[d] * (side == 0 ? -1 : 1);
  for (int k = lo[2]; k < hi[2]; ++k)
    for (int j = lo[1]; j < hi[1]; ++j)
      for (int i = lo[0]; i < hi[0]; ++i) {
        long id = gid(g, i, j, k);
        for (int v = 0; v < nv; ++v) {
          double* q = b->q[v];
          if (order == 0) {
            q[id] = q[id - o];
            for (int m = 1; m <= depth; ++m) q[id + m * o] = q[id - o];
          } else {
            for (int m = 1; m <= depth; ++m) q[id + m * o] = -q[id + (m - 2) * o] + 2.0 * q[id + (m - 1) * o];
          }
        }
      }
}

/* Visits the transverse points of a face normal to d over the whole allocation of the other
 * used directions (lower direction fastest), calling fn with the point's coordinates (the d
 * coordinate set to `at`) and the transverse index. */
typedef void (*face_fn)(osb_block_desc* b, const geom_t* g, int d, int side, int depth, const int* c, long t);

static void for_face(osb_block_desc* b, const geom_t* g, int d, int side, int depth, int at, face_fn fn) {
  const int nd = b->ndim;
  int lo[3], hi[3];
  for (int e = 0; e < 3; ++e) {
    lo[e] = e < nd ? -b->halo : 0;
    hi[e] = e < nd ? g->n[e] + b->halo : 1;
  }
  lo[d] = at;
  hi[d] = at + 1;
  long t = 0;
  for (int k = lo[2]; k < hi[2]; ++k)
    for (int j = lo[1]; j < hi[1]; ++j)
      for (int i = lo[0]; i < hi[0]; ++i) {
        const int c[3] = {i, j, k};
        fn(b, g, d, side, depth, c, t++);
      }
}

/* Symmetry (symmetry.py:23-50 as generated for a Cartesian block): halo layer m = 1..depth
 * receives the point m inside the boundary plane, the momentum normal to the face times -1.0;
 * the plane itself is unchanged. */
static void symmetry_point(osb_block_desc* b, const geom_t* g, int d, int side, int depth, const int* c, long t) {
  (void)t;
  const int nv = b->ndim + 2;
  const long id = gid(g, c[0], c[1], c[2]);
  const long o = g->st[d] * (side == 0 ? -1 : 1);
  for (int m = 1; m <= depth; ++m)
    for (int v = 0; v < nv; ++v) {
      const double x = b->q[v][id - m * o];
      b->q[v][id + m * o] = v == 1 + d ? -1.0 * x : x;
    }
}

/* Dirichlet (dirichlet.py:27-41): the boundary plane and its depth halo layers take the BC's
 * values, dirichlet[d][side][v][layer][t], layer l at -depth + l (side 0) or N-1 + l (side 1). */
static void dirichlet_point(osb_block_desc* b, const geom_t* g, int d, int side, int depth, const int* c, long t) {
  const int nv = b->ndim + 2;
  long tn = 1;
  for (int e = 0; e < b->ndim; ++e)
    if (e != d) tn *= g->n[e] + 2 * b->halo;
  const double* vals = b->dirichlet[d][side];
  for (int l = 0; l <= depth; ++l) {
    int p[3] = {c[0], c[1], c[2]};
    p[d] = (side == 0 ? -depth : g->n[d] - 1) + l;
    const long id = gid(g, p[0], p[1], p[2]);
    for (int v = 0; v < nv; ++v) b->q[v][id] = vals[((long)v * (depth + 1) + l) * tn + t];
  }
}

/* Pressure outlet (pressure_outlet.py:35-51 as generated): the boundary plane and its depth halo
 * layers take rho and the momentum of the point one inside the plane, and
 * rhoE = back_pressure / (-1.0 + gama) + (1/2 |rhou|^2) / rho of that point. */
static void pressure_outlet_point(osb_block_desc* b, const geom_t* g, int d, int side, int depth, const int* c,
                                  long t) {
  (void)t;
  const int nd = b->ndim, nv = nd + 2;
  const long id = gid(g, c[0], c[1], c[2]);
  const long o = g->st[d] * (side == 0 ? -1 : 1);
  const long in = id - o;
  for (int m = 0; m <= depth; ++m) {
    const long p = id + m * o;
    b->q[0][p] = b->q[0][in];
    for (int i = 0; i < nd; ++i) b->q[1 + i][p] = b->q[1 + i][in];
    double ke = 0.5 * (b->q[1][in] * b->q[1][in]);
    for (int i = 1; i < nd; ++i) ke = ke + 0.5 * (b->q[1 + i][in] * b->q[1 + i][in]);
    b->q[nv - 1][p] = b->back_pressure[d][side] / (-1.0 + b->gama) + ke / b->q[0][in];
  }
}

/* Isothermal wall (isothermal_wall.py:62-131 as generated for conservative variables, with the
 * wall energy rhoE = Twall rho / (gama Minf^2 (gama - 1))): the wall plane takes zero momentum
 * and that energy; with the wall pressure Pw = (gama - 1) rhoE(wall) and the temperature
 * T1 = Minf^2 gama (gama - 1) (rhoE - |rhou|^2 / (2 rho)) / rho of the point next to the wall,
 * halo layer k = 1..depth takes T_k = (k+1) Twall - k T1, rho_k = Minf^2 gama Pw / T_k, the
 * momentum -rho_k u(k) and the energy Pw / (gama - 1) + rho_k |u(k)|^2 / 2, u(k) the velocity of
 * the point k inside the wall. */
static void isothermal_wall_point(osb_block_desc* b, const geom_t* g, int d, int side, int depth, const int* c,
                                  long t) {
  (void)t;
  const int nd = b->ndim, nv = nd + 2;
  const long w = gid(g, c[0], c[1], c[2]);
  const long o = g->st[d] * (side == 0 ? 1 : -1); /* towards the inside */
  const double gm = b->gama, M2 = b->Minf * b->Minf, Tw = b->wall_temperature[d][side];
  for (int i = 0; i < nd; ++i) b->q[1 + i][w] = 0.0;
  b->q[nv - 1][w] = Tw * b->q[0][w] / (gm * M2 * (gm - 1.0));
  const double pw = (gm - 1.0) * b->q[nv - 1][w];
  const long a = w + o;
  double ke = 0.0;
  for (int i = 0; i < nd; ++i) ke += 0.5 * (b->q[1 + i][a] * b->q[1 + i][a]);
  const double Ta = M2 * (gm - 1.0) * (b->q[nv - 1][a] - ke / b->q[0][a]) * gm / b->q[0][a];
  for (int k = 1; k <= depth; ++k) {
    const long in = w + k * o, h = w - k * o;
    double u[3], u2 = 0.0;
    for (int i = 0; i < nd; ++i) {
      u[i] = b->q[1 + i][in] / b->q[0][in];
      u2 += u[i] * u[i];
    }
    const double Tk = -(double)k * Ta + (double)(k + 1) * Tw;
    const double rk = M2 * gm * pw / Tk;
    b->q[0][h] = rk;
    for (int i = 0; i < nd; ++i) b->q[1 + i][h] = -rk * u[i];
    b->q[nv - 1][h] = pw / (gm - 1.0) + 0.5 * u2 * rk;
  }
}

/* Adiabatic wall (adiabatic_wall.py:28-69 as generated): halo layer k takes the density and the
 * energy of the point k inside and its momentum negated; the wall plane takes zero momentum and
 * rhoE = rho(wall) T_w / (gama Minf^2 (gama - 1)) with T_w = (18 T1 - 9 T2 + 2 T3) / 11 the
 * wall temperature of a vanishing one-sided third-order dT/dn, T_k = Minf^2 gama (gama - 1)
 * (rhoE - |rhou|^2 / (2 rho)) / rho of the point k inside. */
static void adiabatic_wall_point(osb_block_desc* b, const geom_t* g, int d, int side, int depth, const int* c,
                                 long t) {
  (void)t;
  const int nd = b->ndim, nv = nd + 2;
  const long w = gid(g, c[0], c[1], c[2]);
  const long o = g->st[d] * (side == 0 ? 1 : -1); /* towards the inside */
  const double gm = b->gama, M2 = b->Minf * b->Minf;
  for (int k = 1; k <= depth; ++k) b->q[0][w - k * o] = b->q[0][w + k * o];
  for (int i = 0; i < nd; ++i) b->q[1 + i][w] = 0.0;
  for (int k = 1; k <= depth; ++k)
    for (int i = 0; i < nd; ++i) b->q[1 + i][w - k * o] = -b->q[1 + i][w + k * o];
  double T[4];
  for (int k = 1; k <= 3; ++k) {
    const long a = w + k * o;
    double ke = 0.0;
    for (int i = 0; i < nd; ++i) ke += 0.5 * (b->q[1 + i][a] * b->q[1 + i][a]);
    T[k] = M2 * (gm - 1.0) * (b->q[nv - 1][a] - ke / b->q[0][a]) * gm / b->q[0][a];
  }
  const double Tw = (18.0 / 11.0) * T[1] - (9.0 / 11.0) * T[2] + (2.0 / 11.0) * T[3];
  b->q[nv - 1][w] = Tw * b->q[0][w] / (gm * M2 * (gm - 1.0));
  for (int k = 1; k <= depth; ++k) b->q[nv - 1][w - k * o] = b->q[nv - 1][w + k * o];
}

/* Block interface (multi_block.py:11-107, identity orientation, matching faces normal to the
 * same direction): the halo layers of face (d, side) receive the neighbour's layers adjacent to
 * its face (d, f->side).  `full` = 0 copies the interior of the face only; `full` = 1 also the
 * transverse halos (depth of this face), which the neighbour has filled by then. */
/* InletPressureExtrapolateBC at a low face (inlet_pressure_extrapolate.py:33-73, the generated
 * "InletPressureExtrapolate boundary" kernel): from the boundary-plane state, |u_i| and the sound
 * speed; where the normal |u| >= a the plane takes the state of halo layer 1 (the inflow the
 * initialisation left there), otherwise the plane keeps its state and rhoE of the plane is
 * copied into the halo layers. */
static void inlet_point(osb_block_desc* b, const geom_t* g, int d, int side, int depth, const int* c, long t) {
  (void)side;
  (void)t;
  const int nd = b->ndim, nv = nd + 2;
  const long id = gid(g, c[0], c[1], c[2]);
  const long s = g->st[d];
  const double gm = b->gama, rhob = b->q[0][id];
  double ub[3] = {0.0, 0.0, 0.0}, usq = 0.0;
  for (int e = 0; e < nd; ++e) {
    ub[e] = fabs(b->q[1 + e][id] / b->q[0][id]);
    usq += ub[e] * ub[e];
  }
  const double pb = (gm - 1.0) * (-0.5 * usq * rhob + b->q[nv - 1][id]);
  const double ab = sqrt(gm * pb / rhob);
  if (ub[d] >= ab) {
    for (int v = 0; v < nv; ++v) b->q[v][id] = b->q[v][id - s];
  } else {
    for (int m = 1; m <= depth; ++m) b->q[nv - 1][id - m * s] = b->q[nv - 1][id];
  }
}

static void interface_face(osb_block_desc* blocks, osb_block_desc* b, const geom_t* g, int d, int side, int depth,
                           int full) {
  const osb_interface* f = &b->iface[d][side];
  osb_block_desc* nb = &blocks[f->block];
  geom_t ng = geom_of(nb);
  const int nv = b->ndim + 2;
  int lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
  for (int e = 0; e < b->ndim; ++e) {
    lo[e] = full ? -depth : 0;
    hi[e] = g->n[e] + (full ? depth : 0);
  }
  lo[d] = 0; hi[d] = depth;
  const int Nn = ng.n[d];
  for (int v = 0; v < nv; ++v)
    for (int k = lo[2]; k < hi[2]; ++k)
      for (int j = lo[1]; j < hi[1]; ++j)
        for (int i = lo[0]; i < hi[0]; ++i) {
          int dst[3] = {i, j, k}, src[3] = {i, j, k};
          int layer = (d == 0 ? i : (d == 1 ? j : k));
          /* a flipped interface (opsc.py:1043-1045: to_dir of the normal direction negated)
           * copies the layers in reverse order along the normal */
          int sl = f->flip ? depth - 1 - layer : layer;
          dst[d] = side == 0 ? -depth + layer : g->n[d] + layer;
          src[d] = f->side == 1 ? Nn - depth + sl : sl;
          b->q[v][gid(g, dst[0], dst[1], dst[2])] = nb->q[v][gid(&ng, src[0], src[1], src[2])];
        }
}

/* Boundary conditions of all blocks, in three passes: (A) interface faces, interior of the
 * face; (B) per block, per direction, periodic and zero-gradient faces (their transverse
 * ranges include the halos, so corners come from the layers filled before); (C) interface
 * faces again with their transverse halos, now filled by the neighbour's own pass (B). */
int oracle_apply_bc(osb_block_desc* blocks, int nblocks, int zero_grad_only) {
  for (int pass = 0; pass < 3; ++pass)
    for (int ib = 0; ib < nblocks; ++ib) {
      osb_block_desc* b = &blocks[ib];
      geom_t g = geom_of(b);
      for (int d = 0; d < b->ndim; ++d)
        for (int side = 0; side < 2; ++side) {
          int kind = b->bc[d][side];
          int depth = b->bc_depth[d][side] > 0 ? b->bc_depth[d][side] : 4;
          if (pass == 1 && kind == OSB_BC_PERIODIC && !zero_grad_only) periodic_face(b, &g, d, side, depth);
          if (pass == 1 && kind == OSB_BC_ZERO_GRAD) zero_grad_face(b, &g, d, side, depth);
          if (pass == 1 && (kind == OSB_BC_EXTRAP0 || kind == OSB_BC_EXTRAP1))
            extrap_face(b, &g, d, side, depth, kind == OSB_BC_EXTRAP1);
          if (pass == 1 && kind == OSB_BC_SYMMETRY)
            for_face(b, &g, d, side, depth, side == 0 ? 0 : g.n[d] - 1, symmetry_point);
          if (pass == 1 && kind == OSB_BC_PRESSURE_OUTLET)
            for_face(b, &g, d, side, depth, side == 0 ? 0 : g.n[d] - 1, pressure_outlet_point);
          if (pass == 1 && kind == OSB_BC_ISOTHERMAL_WALL)
            for_face(b, &g, d, side, depth, side == 0 ? 0 : g.n[d] - 1, isothermal_wall_point);
          if (pass == 1 && kind == OSB_BC_ADIABATIC_WALL)
            for_face(b, &g, d, side, depth, side == 0 ? 0 : g.n[d] - 1, adiabatic_wall_point);
          if (pass == 1 && kind == OSB_BC_INLET_PRESSURE_EXTRAP) {
            if (side != 0) return -1; /* the reference implements the inlet on low faces only */
            for_face(b, &g, d, side, depth, 0, inlet_point);
          }
          if (pass == 1 && kind == OSB_BC_DIRICHLET) {
            if (!b->dirichlet[d][side]) return -1;
            for_face(b, &g, d, side, depth, 0, dirichlet_point);
          }
          if (pass != 1 && kind == OSB_BC_INTERFACE && !zero_grad_only)
            interface_face(blocks, b, &g, d, side, depth, pass == 2);
        }
    }
  return 0;
}

/* ---- time integration ------------------------------------------------------------------ */

static double* alloc_like(const geom_t* g) { return (double*)calloc(npts_alloc(g), sizeof(double)); }

static int stage_impl(osb_block_desc* blocks, int nblocks, int rk_kind, const double* A, const double* B, int stage,
                      double dt, int bc);

int oracle_stage(osb_block_desc* blocks, int nblocks, int rk_kind, const double* A, const double* B, int stage,
                 double dt) {
  return stage_impl(blocks, nblocks, rk_kind, A, B, stage, dt, 1);
}

static int stage_impl(osb_block_desc* blocks, int nblocks, int rk_kind, const double* A, const double* B, int stage,
                      double dt, int bc) {
  /* residuals of every block first (all use the pre-stage state), then the updates */
  double** R = (double**)calloc((size_t)nblocks * NVMAX, sizeof(double*));
  for (int ib = 0; ib < nblocks; ++ib) {
    geom_t g = geom_of(&blocks[ib]);
    for (int v = 0; v < blocks[ib].ndim + 2; ++v) R[ib * NVMAX + v] = alloc_like(&g);
    oracle_residual(&blocks[ib], &R[ib * NVMAX]);
  }
  for (int ib = 0; ib < nblocks; ++ib) {
    osb_block_desc* b = &blocks[ib];
    geom_t g = geom_of(b);
    const int nv = b->ndim + 2;
    for (int v = 0; v < nv; ++v) {
      double* q = b->q[v];
      double* o = b->rkold[v];
      const double* r = R[ib * NVMAX + v];
#pragma omp parallel for schedule(static)
      for (int k = 0; k < g.n[2]; ++k)
        for (int j = 0; j < g.n[1]; ++j)
          for (int i = 0; i < g.n[0]; ++i) {
            long id = gid(&g, i, j, k);
            if (rk_kind == OSB_RK_LOW_STORAGE) {
              o[id] = A[stage] * o[id] + dt * r[id];
              q[id] = B[stage] * o[id] + q[id];
            } else {
              q[id] = A[stage] * dt * r[id] + o[id];
              o[id] = B[stage] * dt * r[id] + o[id];
            }
          }
      free(R[ib * NVMAX + v]);
    }
  }
  free(R);
  if (bc) oracle_apply_bc(blocks, nblocks, 0);
  return 0;
}

#define OSB_MAX_BLOCKS_ORACLE 64

int oracle_step(osb_block_desc* blocks, int nblocks, int rk_kind, int nstages, const double* A, const double* B,
                double dt, int nsteps) {
  for (int it = 0; it < nsteps; ++it) {
    oracle_apply_bc(blocks, nblocks, 0);
    if (rk_kind == OSB_RK_SBLI3) {
      for (int ib = 0; ib < nblocks; ++ib) {
        osb_block_desc* b = &blocks[ib];
        geom_t g = geom_of(b);
        for (int v = 0; v < b->ndim + 2; ++v)
          for (int k = 0; k < g.n[2]; ++k)
            for (int j = 0; j < g.n[1]; ++j)
              for (int i = 0; i < g.n[0]; ++i) {
                long id = gid(&g, i, j, k);
                b->rkold[v][id] = b->q[v][id];
              }
      }
    }
    /* with a WENO-filtered block the generated step (the shipped Central4-WENO5 solver)
     * exchanges no halos after the last stage: the filter's own exchange (filter_halos)
     * follows it; the TVD-filtered solver exchanges after every stage */
    int weno = 0, tvd = 0;
    for (int ib = 0; ib < nblocks; ++ib) {
      weno |= blocks[ib].filter == OSB_FILTER_WENO3;
      tvd |= blocks[ib].filter == OSB_FILTER_TVD;
    }
    if (tvd && nblocks > OSB_MAX_BLOCKS_ORACLE) return -1;
    double** stale[OSB_MAX_BLOCKS_ORACLE];
    for (int ib = 0; ib < nblocks && ib < OSB_MAX_BLOCKS_ORACLE; ++ib) stale[ib] = NULL;
    for (int s = 0; s < nstages; ++s) {
      if (tvd && s == nstages - 1)
        for (int ib = 0; ib < nblocks && ib < OSB_MAX_BLOCKS_ORACLE; ++ib) {
          if (blocks[ib].filter != OSB_FILTER_TVD) continue;
          geom_t g = geom_of(&blocks[ib]);
          stale[ib] = (double**)malloc(3 * sizeof(double*));
          for (int c = 0; c < 3; ++c) stale[ib][c] = alloc_like(&g);
          tvd_stale_capture(&blocks[ib], &g, stale[ib]);
        }
      stage_impl(blocks, nblocks, rk_kind, A, B, s, dt, !(weno && s == nstages - 1));
    }
    int rc = (weno || tvd) ? filter_impl(blocks, nblocks, dt, (double* const* const*)stale) : 0;
    for (int ib = 0; ib < nblocks && ib < OSB_MAX_BLOCKS_ORACLE; ++ib)
      if (stale[ib]) {
        for (int c = 0; c < 3; ++c) free(stale[ib][c]);
        free(stale[ib]);
      }
    if (rc) return -1;
  }
  return 0;
}

/* ---- reductions (compressible_TGV.py:176-206) -------------------------------------------- */

int oracle_reduce(const osb_block_desc* blocks, int nblocks, int what, double* out) {
  double acc = (what == OSB_RED_CFL_DT) ? 1e300 : 0.0;
  for (int ib = 0; ib < nblocks; ++ib) {
    const osb_block_desc* b = &blocks[ib];
    geom_t g = geom_of(b);
    const int nd = b->ndim, nv = nd + 2;
    long n = npts_alloc(&g);
    cr_t c;
    cr_alloc(&c, n);
    cr_compute(b, &g, &c);
    double inv0[3], inv[3];
    for (int d = 0; d < nd; ++d) inv0[d] = inv[d] = 1.0 / b->delta[d];
    for (int k = 0; k < g.n[2]; ++k)
      for (int j = 0; j < g.n[1]; ++j)
        for (int i = 0; i < g.n[0]; ++i) {
          long id = gid(&g, i, j, k);
          if (b->ystretch[0]) inv[1] = inv0[1] * b->ystretch[0][j]; /* d/dx_1 = D11 d/dxi_1 */
          double rho = b->q[0][id];
          if (what == OSB_RED_RHO_SUM) acc += rho;
          else if (what == OSB_RED_KE) {
            double s = 0.0;
            for (int e = 0; e < nd; ++e) s += c.u[e][id] * c.u[e][id];
            acc += 0.5 * s * rho;
          } else if (what == OSB_RED_DILATATION_DISS) {
            double div = 0.0;
            for (int e = 0; e < nd; ++e) div += d1c(c.u[e], id, g.st[e], inv[e]);
            acc += (4.0 / 3.0) * div * div * c.mu[id];
          } else if (what == OSB_RED_ENSTROPHY_DISS) {
            double w2 = 0.0;
            if (nd == 3) {
              double wx = d1c(c.u[2], id, g.st[1], inv[1]) - d1c(c.u[1], id, g.st[2], inv[2]);
              double wy = d1c(c.u[0], id, g.st[2], inv[2]) - d1c(c.u[2], id, g.st[0], inv[0]);
              double wz = d1c(c.u[1], id, g.st[0], inv[0]) - d1c(c.u[0], id, g.st[1], inv[1]);
              w2 = wx * wx + wy * wy + wz * wz;
            } else if (nd == 2) {
              double wz = d1c(c.u[1], id, g.st[0], inv[0]) - d1c(c.u[0], id, g.st[1], inv[1]);
              w2 = wz * wz;
            }
            acc += w2 * c.mu[id];
          } else if (what == OSB_RED_CFL_DT) {
            double s = 0.0;
            for (int e = 0; e < nd; ++e) s += (fabs(c.u[e][id]) + c.a[id]) * inv[e];
            double dtl = 1.0 / s;
            if (dtl < acc) acc = dtl;
          } else if (what == OSB_RED_NAN_COUNT) {
            for (int v = 0; v < nv; ++v)
              if (!isfinite(b->q[v][id])) acc += 1.0;
          }
        }
    cr_free(&c);
  }
  *out = acc;
  return 0;
}
