// osb_resident.cu -- whole calls of osb_step on small 1D blocks in one launch.
//
// A 1D block of a few thousand points (the Sod shock tube: 400) is far too small to fill a GPU;
// per-stage launches (flux, update, boundaries) leave it bound by launch latency.  Here one CTA
// holds a block's state, RK register and interface fluxes in shared memory and runs every stage
// of every requested step itself: boundary treatment, the characteristic flux of every
// interface (one thread per interface, the same char_flux as the sweeps), the residual and the
// RK update (rk_LS.py:204-215 / rk_sbli.py:138-154), separated by CTA barriers that every
// thread reaches.  One CTA per block: blocks of one context advance independently (no
// interfaces).  Both precisions.
#include <algorithm>
#include <vector>

#include "osb_internal.h"

// compiled once per residual precision (OSB_RESIDENT_T), the FP32 one with fast-math intrinsics
// like the other FP32-residual kernels
#ifndef OSB_RESIDENT_T
#define OSB_RESIDENT_T double
#define OSB_RESIDENT_NAME resident_f64
#endif

namespace osb {
namespace {

constexpr int RT = 256;  // threads per CTA

struct RkCoef {
  int kind, nst;
  double A[8], B[8];
};

struct Resident1D {
  BlockK k;
  int bc[2], depth[2];
};

// Boundary treatment of one 1D block held in shared memory (x fastest, halo h): periodic,
// zero-gradient and extrapolation as k_periodic / k_zero_grad / k_extrap; side 0 then side 1.
__device__ void bc_1d(double* q, int E, int h, int N, const Resident1D& r) {
  const int t = threadIdx.x;
  if (r.bc[0] == OSB_BC_PERIODIC) {
    // both sides in one pass (they read the interior only): [0, d) -> [N, N+d), [N-d, N) -> [-d, 0)
    const int d0 = r.depth[0], d1 = r.depth[1];
    for (int u = t; u < 3 * (d0 + d1); u += blockDim.x) {
      const int v = u / (d0 + d1), m = u % (d0 + d1);
      double* f = q + v * E + h;
      if (m < d0) f[N + m] = f[m];
      else f[-d1 + (m - d0)] = f[N - d1 + (m - d0)];
    }
    return;
  }
  if (t < 6) {
    const int side = t / 3, v = t % 3;
    double* f = q + v * E + h;
    const int kind = r.bc[side], depth = r.depth[side];
    const int id = side == 0 ? 0 : N - 1;
    const int s = side == 0 ? 1 : -1;  // inward step
    if (kind == OSB_BC_ZERO_GRAD) {
      f[id] = f[id + s];
      for (int m = 1; m <= depth; ++m) f[id - m * s] = f[id + m * s];
    } else if (kind == OSB_BC_EXTRAP0) {
      f[id] = f[id + s];
      for (int m = 1; m <= depth; ++m) f[id - m * s] = f[id + s];
    } else if (kind == OSB_BC_EXTRAP1) {
      for (int m = 1; m <= depth; ++m) f[id - m * s] = -f[id - (m - 2) * s] + 2.0 * f[id - (m - 1) * s];
    }
  }
}

// T = double: the FP64 path.  T = float: the FP32-residual path -- the state and RK register
// stay FP64 in shared memory next to an FP32 copy of the state; the fluxes come from the FP32
// copy, the residual is the compensated (float-float) flux difference and the update takes
// dt x residual rounded once to FP32 (dt_residual) and applies it with FP64 FMAs, as the fused
// RK epilogue of the per-block path does.
template <typename T, int SCH, int AVG>
__global__ void __launch_bounds__(RT) k_resident_1d(const Resident1D* __restrict__ blocks, SchemeParams spd, RkCoef rk,
                                                    double dt, int nsteps, unsigned long long* bad) {
  constexpr bool F32 = sizeof(T) == 4;
  const Resident1D r = blocks[blockIdx.x];
  const BlockK& b = r.k;
  const SP<T> sp(spd);
  extern __shared__ __align__(16) unsigned char osb_smem[];
  const int N = b.n[0], h = b.off0, E = b.alloc;
  double* q = reinterpret_cast<double*>(osb_smem);   // [3][E]
  double* o = q + 3 * E;                              // [3][E]
  T* F = reinterpret_cast<T*>(o + 3 * E);             // [3][E]: flux at the right face of point i
  float* qf = reinterpret_cast<float*>(F + 3 * E);    // [3][E]: FP32 copy of the state (F32 only)
  for (int u = threadIdx.x; u < 3 * E; u += blockDim.x) {
    q[u] = b.q[u / E][u % E];
    o[u] = b.rk[u / E][u % E];
    if (F32) qf[u] = d2f_rn(q[u]);
  }
  __syncthreads();
  const double invd = b.invd[0];
  const float invd_f = (float)invd;
  const float dt_h = (float)dt, dt_l = (float)(dt - (double)dt_h);
  const T gm = sp.gama;
  for (int step = 0; step < nsteps; ++step) {
    __syncthreads();     // the previous stage's update is complete
    if (rk.kind == 1) {  // SBLI RK3 saves the state at the start of the step
      for (int u = threadIdx.x; u < 3 * N; u += blockDim.x) o[(u / N) * E + h + u % N] = q[(u / N) * E + h + u % N];
    }
    for (int s = 0; s < rk.nst; ++s) {
      __syncthreads();
      bc_1d(q, E, h, N, r);
      __syncthreads();
      if (F32) {
        // the boundary treatment changed the halos and at most the end points: refresh their copy
        for (int u = threadIdx.x; u < 3 * 2 * (h + 2); u += blockDim.x) {
          const int v = u / (2 * (h + 2)), m = u % (2 * (h + 2));
          const int i = m < h + 2 ? m - h : N - 2 + (m - (h + 2));
          qf[v * E + h + i] = d2f_rn(q[v * E + h + i]);
        }
        __syncthreads();
      }
      for (int i = (int)threadIdx.x - 1; i < N; i += blockDim.x) {
        Pt<T, 1> w[6];
#pragma unroll
        for (int m = 0; m < 6; ++m) {
#pragma unroll
          for (int v = 0; v < 3; ++v) {
            const int id = v * E + h + i - 2 + m;
            w[m].q[v] = F32 ? (T)qf[id] : (T)q[id];
          }
          make_pt<T, 1>(w[m], gm);
        }
        T fh[3];
        char_flux<T, 1, SCH, AVG>(w, sp, fh);
#pragma unroll
        for (int v = 0; v < 3; ++v) F[v * E + h + i] = fh[v];
      }
      __syncthreads();
      const double A = rk.A[s], B = rk.B[s];
      const bool a_zero = rk.kind == 0 && A == 0.0;
      for (int i = threadIdx.x; i < N; i += blockDim.x) {
#pragma unroll
        for (int v = 0; v < 3; ++v) {
          const int id = v * E + h + i;
          double ov = o[id], qv = q[id];
          if constexpr (F32) {
            float p, pe;
            ff_flux_diff((float)F[id], (float)F[id - 1], invd_f, p, pe);
            const float hh = __fadd_rn(p, pe);
            const float ll = __fsub_rn(pe, __fsub_rn(hh, p));
            const double x = dt_residual(hh, ll, dt_h, dt_l);  // as rk_point_ff
            if (rk.kind == 0) {
              ov = a_zero ? x : __fma_rn(A, ov, x);
              qv = __fma_rn(B, ov, qv);
            } else {
              qv = __fma_rn(A, x, ov);
              ov = __fma_rn(B, x, ov);
            }
            qf[id] = d2f_rn(qv);
          } else {
            const double r0 = -((double)F[id] - (double)F[id - 1]) * invd;
            if (rk.kind == 0) {
              ov = A * ov + dt * r0;
              qv = B * ov + qv;
            } else {
              qv = A * dt * r0 + ov;
              ov = B * dt * r0 + ov;
            }
          }
          o[id] = ov;
          q[id] = qv;
        }
      }
    }
  }
  __syncthreads();
  bc_1d(q, E, h, N, r);  // the halos a caller observes after the call
  __syncthreads();
  unsigned long long nb = 0;
  for (int u = threadIdx.x; u < 3 * E; u += blockDim.x) {
    b.q[u / E][u % E] = q[u];
    b.rk[u / E][u % E] = o[u];
    if (F32 && b.qf[0]) b.qf[u / E][u % E] = d2f_rn(q[u]);
    const int i = u % E - h;
    if (i >= 0 && i < N && !isfinite(q[u])) ++nb;
  }
  if (nb) atomicAdd(bad, nb);
}

template <typename T, int SCH, int AVG>
int launch_resident(osb_ctx* c, const Resident1D* dev, int nblocks, int maxE, double dt, int nsteps) {
  const Block& f = c->blocks[0];
  SchemeParams sp = scheme_params(f.d.gama, f.d.eps, f.d.teno_ct, f.d.shock_filter_control, 1e-12);
  RkCoef rk{};
  rk.kind = c->rk_kind == OSB_RK_LOW_STORAGE ? 0 : 1;
  rk.nst = c->nst;
  for (int s = 0; s < c->nst; ++s) {
    rk.A[s] = c->A[s];
    rk.B[s] = c->B[s];
  }
  const size_t smem = (size_t)3 * maxE * (2 * sizeof(double) + sizeof(T) + (sizeof(T) == 4 ? sizeof(float) : 0));
  auto kern = k_resident_1d<T, SCH, AVG>;
  OSB_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  timing_begin(c, FAM_PERSISTENT);
  kern<<<nblocks, RT, smem, c->stream>>>(dev, sp, rk, dt, nsteps, c->bad);
  timing_end(c);
  c->launches++;
  return OSB_OK;
}

}  // namespace

#ifndef OSB_RESIDENT_F32
// Largest allocated 1D extent (interior + 2 x 5 halo) the resident path holds: 3 variables x
// (FP64 state, FP64 register, flux, FP32 copy) within the 227 KB of shared memory of a CTA.
constexpr int RESIDENT_MAX_E = 3000;

bool resident_eligible(const osb_ctx* c) {
  if (c->blocks.empty() || c->sched.mode == OSB_SCHED_PER_BLOCK) return false;
  if (c->nst > 8) return false;
  const osb_block_desc& f = c->blocks[0].d;
  for (const auto& bl : c->blocks) {
    const osb_block_desc& d = bl.d;
    if (d.ndim != 1 || d.scheme == OSB_SCHEME_CENTRAL4 || d.viscous != OSB_VISC_NONE || d.metric[9]) return false;
    if (d.scheme != f.scheme || d.averaging != f.averaging) return false;
    if (bl.k.alloc > RESIDENT_MAX_E) return false;
    for (int s = 0; s < 2; ++s)
      if (d.bc[0][s] == OSB_BC_INTERFACE || d.bc[0][s] == OSB_BC_SYMMETRY || d.bc[0][s] == OSB_BC_DIRICHLET ||
          d.bc[0][s] == OSB_BC_PRESSURE_OUTLET)
        return false;
    if (d.flux_type != OSB_FLUX_LLF) return false;
    if ((d.bc[0][0] == OSB_BC_PERIODIC) != (d.bc[0][1] == OSB_BC_PERIODIC)) return false;
  }
  return true;
}

int resident_step(osb_ctx* c, double dt, int nsteps) {
  return c->prec == OSB_PREC_FP32_RESIDUAL ? resident_f32(c, dt, nsteps) : resident_f64(c, dt, nsteps);
}
#endif

int OSB_RESIDENT_NAME(osb_ctx* c, double dt, int nsteps) {
  if (nsteps <= 0) return OSB_OK;
  const int nb = (int)c->blocks.size();
  if (!c->resident || c->resident_n != nb) {
    if (c->resident) cudaFree(c->resident);
    c->resident = nullptr;
    OSB_CK(cudaMalloc(&c->resident, sizeof(Resident1D) * nb));
    c->resident_n = nb;
  }
  std::vector<Resident1D> host(nb);
  int maxE = 0;
  for (int i = 0; i < nb; ++i) {
    const Block& bl = c->blocks[i];
    host[i].k = bl.k;
    for (int s = 0; s < 2; ++s) {
      host[i].bc[s] = bl.d.bc[0][s];
      host[i].depth[s] = bl.d.bc_depth[0][s] > 0 ? bl.d.bc_depth[0][s] : 4;
    }
    maxE = std::max(maxE, (int)bl.k.alloc);
  }
  OSB_CK(cudaMemcpyAsync(c->resident, host.data(), sizeof(Resident1D) * nb, cudaMemcpyHostToDevice, c->stream));
  const Resident1D* dev = reinterpret_cast<const Resident1D*>(c->resident);
  const int sch = c->blocks[0].d.scheme, avg = c->blocks[0].d.averaging;
  if (avg == OSB_AVG_ROE) {
    if (sch == OSB_SCHEME_WENO5_JS) return launch_resident<OSB_RESIDENT_T, SCH_WENO5_JS, AVG_ROE>(c, dev, nb, maxE, dt, nsteps);
    if (sch == OSB_SCHEME_WENO5_Z) return launch_resident<OSB_RESIDENT_T, SCH_WENO5_Z, AVG_ROE>(c, dev, nb, maxE, dt, nsteps);
    if (sch == OSB_SCHEME_TENO5) return launch_resident<OSB_RESIDENT_T, SCH_TENO5, AVG_ROE>(c, dev, nb, maxE, dt, nsteps);
    if (sch == OSB_SCHEME_TENO6) return launch_resident<OSB_RESIDENT_T, SCH_TENO6, AVG_ROE>(c, dev, nb, maxE, dt, nsteps);
  } else {
    if (sch == OSB_SCHEME_WENO5_JS) return launch_resident<OSB_RESIDENT_T, SCH_WENO5_JS, AVG_SIMPLE>(c, dev, nb, maxE, dt, nsteps);
    if (sch == OSB_SCHEME_WENO5_Z) return launch_resident<OSB_RESIDENT_T, SCH_WENO5_Z, AVG_SIMPLE>(c, dev, nb, maxE, dt, nsteps);
    if (sch == OSB_SCHEME_TENO5) return launch_resident<OSB_RESIDENT_T, SCH_TENO5, AVG_SIMPLE>(c, dev, nb, maxE, dt, nsteps);
    if (sch == OSB_SCHEME_TENO6) return launch_resident<OSB_RESIDENT_T, SCH_TENO6, AVG_SIMPLE>(c, dev, nb, maxE, dt, nsteps);
  }
  return fail(OSB_ENOTSUP, "scheme %d not available in the resident 1D path", sch);
}

}  // namespace osb
