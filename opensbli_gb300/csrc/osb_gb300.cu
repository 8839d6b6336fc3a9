// osb_gb300.cu -- C ABI of the GB300 residual-and-update path (include/osb_gb300.h).
//
// A context owns one CUDA stream, the FP64 residual workspace of each block, the reduction
// scratch and an optional CUDA graph of one RK step.  One RK stage is
//     for each block: flux sweeps x, y, z (characteristic LLF WENO/TENO)  | central kernel
//                     [+ central viscous kernel]
//     for each block: RK update
//     for each block: boundary conditions (periodic exchange / zero gradient / interfaces)
// which is the kernel order of the generated stage loop
// (apps/performance_benchmark/TENO6/opensbli.cpp:216-431) with the constituent-relation,
// derivative and residual loops folded into the sweeps and the central kernel.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <mutex>
#include <thread>
#include <algorithm>
#include <vector>

#include "osb_closures.h"
#include "osb_internal.h"

using namespace osb;

namespace osb {

// ---------------------------------------------------------------------------------------
// RK update over the interior (rk_LS.py:204-215 / rk_sbli.py:138-145); counts non-finite
// results into *bad.
__global__ void k_rk(BlockK b, int nv, int kind, double A, double B, double dt, unsigned long long* bad) {
  const long npts = (long)b.n[0] * b.n[1] * b.n[2];
  unsigned long long nb = 0;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < npts; t += (long)gridDim.x * blockDim.x) {
    int i = (int)(t % b.n[0]);
    long r = t / b.n[0];
    int j = (int)(r % b.n[1]);
    int k = (int)(r / b.n[1]);
    long id = lin(b, i, j, k);
    for (int v = 0; v < nv; ++v) {
      double r0 = b.R[v][id];
      double o = b.rk[v][id];
      double q = b.q[v][id];
      if (kind == 0) {
        o = A * o + dt * r0;
        q = B * o + q;
      } else {
        q = A * dt * r0 + o;
        o = B * dt * r0 + o;
      }
      b.rk[v][id] = o;
      b.q[v][id] = q;
      if (!isfinite(q)) ++nb;
    }
  }
  if (nb) atomicAdd(bad, nb);
}

// SBLI RK3 "Save equations": old = q over the interior.
__global__ void k_save(BlockK b, int nv) {
  const long npts = (long)b.n[0] * b.n[1] * b.n[2];
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < npts; t += (long)gridDim.x * blockDim.x) {
    int i = (int)(t % b.n[0]);
    long r = t / b.n[0];
    int j = (int)(r % b.n[1]);
    int k = (int)(r / b.n[1]);
    long id = lin(b, i, j, k);
    for (int v = 0; v < nv; ++v) b.rk[v][id] = b.q[v][id];
  }
}

// FP32-residual path RK update (blocks whose residual kernels do not carry it): the residual
// arrives as a float-float pair, the state and register stay FP64, and the next FP32 state goes
// to rf.qout; conversions use integer operations so only the update runs on the FP64 pipe.
__global__ void k_rk32(BlockK b, int nv, RkFuse rf) {
  const int npts = b.n[0] * b.n[1] * b.n[2];
  unsigned nb = 0;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < npts; t += gridDim.x * blockDim.x) {
    int i = t % b.n[0];
    int r = t / b.n[0];
    int j = r % b.n[1];
    int k = r / b.n[1];
    int id = lin(b, i, j, k);
    for (int v = 0; v < nv; ++v) nb += rk_point(b, rf, v, id, b.Rh[v][id], b.Rl[v][id]);
  }
  if (nb) atomicAdd(rf.bad, (unsigned long long)nb);
}

// (hi + lo) float-float residual -> FP64 array (osb_residual of the FP32-residual path).
__global__ void k_ff_to_double(const float* hi, const float* lo, double* out, long n) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x)
    out[t] = f2d_exact(hi[t]) + f2d_exact(lo[t]);
}

// FP32 shadow <- FP64 state over the whole allocation (halos included).
__global__ void k_q2qf(BlockK b, int nv) {
  const int n = (int)b.alloc;
  const int v = blockIdx.y;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
    b.qf[v][t] = d2f_rn(b.q[v][t]);
}

// Halo arrays a boundary kernel writes: the FP64 state, the FP32 state, or both.
enum { BC_Q = 1, BC_QF = 2, BC_BOTH = 3 };

// Periodic exchange of both faces of direction d (ExchangeSelf, periodic.py:53-71):
// side 0 copies [0, depth) to [N, N+depth), side 1 copies [N-depth, N) to [-depth, 0); the
// transverse ranges include -depth..N+depth of the other used directions (corners).
// blockIdx.y = 2 * variable + side; 32-bit index arithmetic.
__global__ void k_periodic(BlockK b, int nv, int d, int depth0, int depth1, int fields) {
  const int dmax = max(depth0, depth1);
  int ext[3], lo[3];
  for (int e = 0; e < 3; ++e) {
    if (e < b.ndim && e != d) {
      ext[e] = b.n[e] + 2 * dmax;
      lo[e] = -dmax;
    } else {
      ext[e] = 1;
      lo[e] = 0;
    }
  }
  ext[d] = dmax;
  const int side = blockIdx.y & 1, v = blockIdx.y >> 1;
  const int depth = side == 0 ? depth0 : depth1;
  const int N = b.n[d];
  const int per = ext[0] * ext[1] * ext[2];
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < per; t += gridDim.x * blockDim.x) {
    int c[3];
    c[0] = t % ext[0];
    const int r = t / ext[0];
    c[1] = r % ext[1];
    c[2] = r / ext[1];
    if (c[d] >= depth) continue;
    int src[3], dst[3];
    bool skip = false;
    for (int e = 0; e < 3; ++e) {
      src[e] = c[e] + lo[e];
      dst[e] = src[e];
      if (e != d && e < b.ndim && (src[e] < -depth || src[e] >= b.n[e] + depth)) skip = true;
    }
    if (skip) continue;
    if (side == 0) {
      src[d] = c[d];
      dst[d] = N + c[d];
    } else {
      src[d] = N - depth + c[d];
      dst[d] = -depth + c[d];
    }
    const int di = lin(b, dst[0], dst[1], dst[2]), si = lin(b, src[0], src[1], src[2]);
    if (fields & BC_Q) b.q[v][di] = b.q[v][si];
    if ((fields & BC_QF) && b.qf[0]) b.qf[v][di] = b.qf[v][si];
  }
}

// Periodic halos of a block whose faces are all periodic with one depth D: every point of
// [-D, N+D) per used direction outside the interior receives the interior point at the
// wrapped coordinates -- what the direction-by-direction exchange (k_periodic for x, then y,
// then z, transverse ranges including the halos) leaves there -- in one launch.  The shell is
// walked as three disjoint regions (z faces with full x-y extent, y faces over the interior z,
// x faces over the interior y-z), x fastest, 32-bit indices.
__global__ void k_periodic_shell(BlockK b, int nv, int D, int fields) {
  const int nd = b.ndim;
  const int n0 = b.n[0], n1 = nd > 1 ? b.n[1] : 1, n2 = nd > 2 ? b.n[2] : 1;
  const int e0 = n0 + 2 * D, e1 = nd > 1 ? n1 + 2 * D : 1;
  const int cz = nd > 2 ? 2 * D * e1 * e0 : 0;
  const int cy = nd > 1 ? n2 * 2 * D * e0 : 0;
  const int cx = n2 * n1 * 2 * D;
  const int total = cz + cy + cx;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    int x, y = 0, z = 0;
    if (t < cz) {
      x = t % e0 - D;
      const int r = t / e0;
      y = r % e1 - D;
      const int zz = r / e1;
      z = zz < D ? zz - D : n2 + zz - D;
    } else if (t < cz + cy) {
      const int u = t - cz;
      x = u % e0 - D;
      const int r = u / e0;
      const int yy = r % (2 * D);
      y = yy < D ? yy - D : n1 + yy - D;
      z = r / (2 * D);
    } else {
      const int u = t - cz - cy;
      const int xx = u % (2 * D);
      x = xx < D ? xx - D : n0 + xx - D;
      const int r = u / (2 * D);
      y = r % n1;
      z = r / n1;
    }
    const int sx = x < 0 ? x + n0 : (x >= n0 ? x - n0 : x);
    const int sy = y < 0 ? y + n1 : (y >= n1 ? y - n1 : y);
    const int sz = z < 0 ? z + n2 : (z >= n2 ? z - n2 : z);
    const int di = lin(b, x, y, z), si = lin(b, sx, sy, sz);
    if (fields & BC_Q) {
      double vq[5];
      for (int v = 0; v < nv; ++v) vq[v] = b.q[v][si];
      for (int v = 0; v < nv; ++v) b.q[v][di] = vq[v];
    }
    if ((fields & BC_QF) && b.qf[0]) {
      float vf[5];
      for (int v = 0; v < nv; ++v) vf[v] = b.qf[v][si];
      for (int v = 0; v < nv; ++v) b.qf[v][di] = vf[v];
    }
  }
}

// Depth of a block whose faces are all periodic with one depth D not above any of its
// extents (so one wrap lands in the interior), else 0.
static int uniform_periodic_depth(const Block& bl) {
  int D = 0;
  for (int d = 0; d < bl.d.ndim; ++d)
    for (int side = 0; side < 2; ++side) {
      if (bl.d.bc[d][side] != OSB_BC_PERIODIC) return 0;
      const int dep = bl.d.bc_depth[d][side] > 0 ? bl.d.bc_depth[d][side] : 4;
      if (D == 0) D = dep;
      else if (dep != D) return 0;
    }
  for (int d = 0; d < bl.d.ndim; ++d)
    if (bl.k.n[d] < D) return 0;
  return D;
}

// Zero-gradient outlet (zero_gradient_outlet.py:11-23 as generated): on side 0,
// q(0) = q(1) then q(-m) = q(m) for m = 1..depth; mirrored on side 1.  Over the interior
// extent of the other directions.
__global__ void k_zero_grad(BlockK b, int nv, int d, int side, int depth, int fields) {
  int ext[3];
  for (int e = 0; e < 3; ++e) ext[e] = (e == d) ? 1 : b.n[e];
  const long total = (long)ext[0] * ext[1] * ext[2];
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    long r = t;
    int c[3];
    c[0] = (int)(r % ext[0]); r /= ext[0];
    c[1] = (int)(r % ext[1]); r /= ext[1];
    c[2] = (int)r;
    c[d] = side == 0 ? 0 : b.n[d] - 1;
    int id = lin(b, c[0], c[1], c[2]);
    int s = b.st[d] * (side == 0 ? 1 : -1);
    for (int v = 0; v < nv; ++v) {
      if (fields & BC_Q) {
        double* q = b.q[v];
        q[id] = q[id + s];
        for (int m = 1; m <= depth; ++m) q[id - m * s] = q[id + m * s];
      }
      if ((fields & BC_QF) && b.qf[0]) {
        float* f = b.qf[v];
        f[id] = f[id + s];
        for (int m = 1; m <= depth; ++m) f[id - m * s] = f[id + m * s];
      }
    }
  }
}

// Extrapolation boundary (extrapolation.py:29-53 as generated): boundary point b = 0 on side 0,
// N-1 on side 1, outward step o.  Order 0: q(b) = q(b-o), q(b+m o) = q(b-o), m = 1..depth.
// Order 1: q(b+m o) = 2 q(b+(m-1) o) - q(b+(m-2) o), m = 1..depth in order.  Over the interior
// extent of the other directions.
__global__ void k_extrap(BlockK b, int nv, int d, int side, int depth, int order, int fields) {
  int ext[3];
  for (int e = 0; e < 3; ++e) ext[e] = (e == d) ? 1 : b.n[e];
  const int total = ext[0] * ext[1] * ext[2];
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    int c[3];
    c[0] = t % ext[0];
    const int r = t / ext[0];
    c[1] = r % ext[1];
    c[2] = r / ext[1];
    c[d] = side == 0 ? 0 : b.n[d] - 1;
    const int id = lin(b, c[0], c[1], c[2]);
    const int o = b.st[d] * (side == 0 ? -1 : 1);
    for (int v = 0; v < nv; ++v) {
      if (fields & BC_Q) {
        double* q = b.q[v];
        if (order == 0) {
          q[id] = q[id - o];
          for (int m = 1; m <= depth; ++m) q[id + m * o] = q[id - o];
        } else {
          for (int m = 1; m <= depth; ++m) q[id + m * o] = -q[id + (m - 2) * o] + 2.0 * q[id + (m - 1) * o];
        }
      }
      if ((fields & BC_QF) && b.qf[0]) {
        float* f = b.qf[v];
        if (order == 0) {
          f[id] = f[id - o];
          for (int m = 1; m <= depth; ++m) f[id + m * o] = f[id - o];
        } else {
          for (int m = 1; m <= depth; ++m) f[id + m * o] = -f[id + (m - 2) * o] + 2.0f * f[id + (m - 1) * o];
        }
      }
    }
  }
}

// Transverse point t of a face normal to d over the whole allocated extent of the other used
// directions (lower direction fastest): its coordinates, halo included.
__device__ __forceinline__ void face_point(const BlockK& b, int d, int halo, int t, int (&c)[3]) {
  int r = t;
  for (int e = 0; e < 3; ++e) {
    if (e == d) {
      c[e] = 0;
      continue;
    }
    const int ext = e < b.ndim ? b.n[e] + 2 * halo : 1;
    c[e] = r % ext - (e < b.ndim ? halo : 0);
    r /= ext;
  }
}

__host__ __device__ inline int face_extent(const BlockK& b, int d, int halo) {
  int t = 1;
  for (int e = 0; e < b.ndim; ++e)
    if (e != d) t *= b.n[e] + 2 * halo;
  return t;
}

// Symmetry face (symmetry.py:23-50 as generated for a Cartesian block): halo layer k = 1..depth
// receives the point k inside the boundary plane (side 0: -k from +k; side 1: N-1+k from
// N-1-k) with the momentum normal to the face negated; the plane itself is unchanged.  Over the
// whole transverse allocation.
__global__ void k_symmetry(BlockK b, int nv, int d, int side, int depth, int halo, int fields) {
  const int total = face_extent(b, d, halo);
  const int base = side == 0 ? 0 : b.n[d] - 1;
  const int o = b.st[d] * (side == 0 ? -1 : 1);
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    int c[3];
    face_point(b, d, halo, t, c);
    c[d] = base;
    const int id = lin(b, c[0], c[1], c[2]);
    for (int k = 1; k <= depth; ++k)
      for (int v = 0; v < nv; ++v) {
        const bool normal = v == 1 + d;
        if (fields & BC_Q) {
          const double x = b.q[v][id - k * o];
          b.q[v][id + k * o] = normal ? -1.0 * x : x;
        }
        if ((fields & BC_QF) && b.qf[0]) {
          const float x = b.qf[v][id - k * o];
          b.qf[v][id + k * o] = normal ? -x : x;
        }
      }
  }
}

// Pressure outlet (pressure_outlet.py:35-51 as generated): the boundary plane and its `depth`
// halo layers take the density and momentum of the point one inside the plane, and the total
// energy pback / (gama - 1) + (sum_i 1/2 m_i^2) / rho of that point, over the whole transverse
// allocation; the generated operation order, rounded operation by operation.  The FP32 copy
// (between stages of the FP32-residual path) is formed the same way from the FP32 neighbour.
__device__ __forceinline__ double pout_energy(double pback, double gama, const double* m, int nd, double rho) {
  double ke = __dmul_rn(0.5, __dmul_rn(m[0], m[0]));
  for (int i = 1; i < nd; ++i) ke = __dadd_rn(ke, __dmul_rn(0.5, __dmul_rn(m[i], m[i])));
  return __dadd_rn(__ddiv_rn(pback, __dadd_rn(-1.0, gama)), __ddiv_rn(ke, rho));
}
__global__ void k_pressure_outlet(BlockK b, int nv, int d, int side, int depth, int halo, double pback, double gama,
                                  int fields) {
  const int total = face_extent(b, d, halo);
  const int base = side == 0 ? 0 : b.n[d] - 1;
  const int o = b.st[d] * (side == 0 ? -1 : 1);
  const int nd = nv - 2;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    int c[3];
    face_point(b, d, halo, t, c);
    c[d] = base;
    const int id = lin(b, c[0], c[1], c[2]);
    const int in = id - o;
    if (fields & BC_Q) {
      double m[3];
      for (int i = 0; i < nd; ++i) m[i] = b.q[1 + i][in];
      const double rho = b.q[0][in];
      const double E = pout_energy(pback, gama, m, nd, rho);
      for (int k = 0; k <= depth; ++k) {
        const int p = id + k * o;
        b.q[0][p] = rho;
        for (int i = 0; i < nd; ++i) b.q[1 + i][p] = m[i];
        b.q[nv - 1][p] = E;
      }
    }
    if ((fields & BC_QF) && b.qf[0]) {
      double m[3];
      for (int i = 0; i < nd; ++i) m[i] = f2d_exact(b.qf[1 + i][in]);
      const float rho = b.qf[0][in];
      const float E = d2f_rn(pout_energy(pback, gama, m, nd, f2d_exact(rho)));
      for (int k = 0; k <= depth; ++k) {
        const int p = id + k * o;
        b.qf[0][p] = rho;
        for (int i = 0; i < nd; ++i) b.qf[1 + i][p] = b.qf[1 + i][in];
        b.qf[nv - 1][p] = E;
      }
    }
  }
}

// Isothermal no-slip wall (isothermal_wall.py:62-131 as generated for conservative variables,
// wall energy rhoE = Twall rho / (gama Minf^2 (gama - 1))): the wall plane takes zero momentum and
// that energy (its density stays the one the RK update gave it); with the wall pressure
// Pw = (gama - 1) rhoE(wall) and the temperature T1 = Minf^2 gama (gama - 1) (rhoE - |rhou|^2 /
// (2 rho)) / rho of the point next to the wall, halo layer k = 1..depth takes
// T_k = (k+1) Twall - k T1, rho_k = Minf^2 gama Pw / T_k, momentum -rho_k u(k) and energy
// Pw / (gama - 1) + rho_k |u(k)|^2 / 2, u(k) the velocity of the point k inside.  Over the
// transverse range the other faces fill (their layers' depth).  The FP32 shadow is filled from its own values in FP32 arithmetic (its
// halos feed FP32 kernels only); with BC_QF alone the FP64 wall plane is reset too, so the FP64
// state's wall momentum and energy stay the wall's between the FP32 path's stages.
// Explicitly rounded operations in the arithmetic of the array a wall kernel fills.
template <typename A>
struct WOp;
template <>
struct WOp<double> {
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
};
template <>
struct WOp<float> {
  static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
  static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
  static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
};

template <typename A>
__device__ void wall_point(A* const* q, int nd, int w, int o, int depth, A gm, A M2, A Tw) {
  using O = WOp<A>;
  const int nv = nd + 2;
  const A g1 = O::add(gm, A(-1));
  for (int i = 0; i < nd; ++i) q[1 + i][w] = A(0);
  q[nv - 1][w] = O::div(O::mul(Tw, q[0][w]), O::mul(O::mul(gm, M2), g1));
  const A pw = O::mul(g1, q[nv - 1][w]);
  const int a = w + o;
  A ke = A(0);
  for (int i = 0; i < nd; ++i) ke = O::add(ke, O::mul(A(0.5), O::mul(q[1 + i][a], q[1 + i][a])));
  const A ra = q[0][a];
  const A Ta = O::div(O::mul(O::mul(O::mul(M2, g1), O::add(q[nv - 1][a], -O::div(ke, ra))), gm), ra);
  for (int k = 1; k <= depth; ++k) {
    const int in = w + k * o, h = w - k * o;
    A u[3], u2 = A(0);
    for (int i = 0; i < nd; ++i) {
      u[i] = O::div(q[1 + i][in], q[0][in]);
      u2 = O::add(u2, O::mul(u[i], u[i]));
    }
    const A Tk = O::add(O::mul(A(-k), Ta), O::mul(A(k + 1), Tw));
    const A rk = O::div(O::mul(O::mul(M2, gm), pw), Tk);
    q[0][h] = rk;
    for (int i = 0; i < nd; ++i) q[1 + i][h] = -O::mul(rk, u[i]);
    q[nv - 1][h] = O::add(O::div(pw, g1), O::mul(O::mul(A(0.5), u2), rk));
  }
}

// Adiabatic wall (adiabatic_wall.py:28-69 as generated): halo layer k takes the density and
// energy of the point k inside and its momentum negated; the wall plane zero momentum and
// rhoE = rho(wall) T_w / (gama Minf^2 (gama - 1)), T_w = (18 T1 - 9 T2 + 2 T3) / 11 the wall
// temperature of a vanishing one-sided third-order dT/dn (T_k of the point k inside).  `halos`
// false: the wall plane only.
template <typename A>
__device__ void adiabatic_point(A* const* q, int nd, int w, int o, int depth, A gm, A M2, bool halos) {
  using O = WOp<A>;
  const int nv = nd + 2;
  const A g1 = O::add(gm, A(-1));
  if (halos)
    for (int k = 1; k <= depth; ++k) q[0][w - k * o] = q[0][w + k * o];
  for (int i = 0; i < nd; ++i) q[1 + i][w] = A(0);
  if (halos)
    for (int k = 1; k <= depth; ++k)
      for (int i = 0; i < nd; ++i) q[1 + i][w - k * o] = -q[1 + i][w + k * o];
  A T[4];
  for (int k = 1; k <= 3; ++k) {
    const int a = w + k * o;
    A ke = A(0);
    for (int i = 0; i < nd; ++i) ke = O::add(ke, O::mul(A(0.5), O::mul(q[1 + i][a], q[1 + i][a])));
    const A ra = q[0][a];
    T[k] = O::div(O::mul(O::mul(O::mul(M2, g1), O::add(q[nv - 1][a], -O::div(ke, ra))), gm), ra);
  }
  const A Tw = O::add(O::add(O::mul(A(18.0 / 11.0), T[1]), -O::mul(A(9.0 / 11.0), T[2])), O::mul(A(2.0 / 11.0), T[3]));
  q[nv - 1][w] = O::div(O::mul(Tw, q[0][w]), O::mul(O::mul(gm, M2), g1));
  if (halos)
    for (int k = 1; k <= depth; ++k) q[nv - 1][w - k * o] = q[nv - 1][w + k * o];
}

// Both wall kinds over the transverse range of face (d, side), `halo` points beyond the face.
__global__ void k_wall(BlockK b, int nv, int kind, int d, int side, int depth, int halo, double gama, double Minf,
                       double Tw, float gf, float M2f, float Twf, int fields) {
  const int total = face_extent(b, d, halo);
  const int base = side == 0 ? 0 : b.n[d] - 1;
  const int o = b.st[d] * (side == 0 ? 1 : -1);  // towards the inside
  const int nd = nv - 2;
  const double M2 = __dmul_rn(Minf, Minf);
  const bool iso = kind == OSB_BC_ISOTHERMAL_WALL;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    int c[3];
    face_point(b, d, halo, t, c);
    c[d] = base;
    const int w = lin(b, c[0], c[1], c[2]);
    if (fields & BC_Q) {
      if (iso) wall_point<double>(b.q, nd, w, o, depth, gama, M2, Tw);
      else adiabatic_point<double>(b.q, nd, w, o, depth, gama, M2, true);
    } else if (b.qf[0]) {  // FP64 wall plane only (the halos follow when the call returns)
      if (iso) {
        for (int i = 0; i < nd; ++i) b.q[1 + i][w] = 0.0;
        b.q[nv - 1][w] = __ddiv_rn(__dmul_rn(Tw, b.q[0][w]), __dmul_rn(__dmul_rn(gama, M2), __dadd_rn(gama, -1.0)));
      } else {
        adiabatic_point<double>(b.q, nd, w, o, depth, gama, M2, false);
      }
    }
    if ((fields & BC_QF) && b.qf[0]) {
      if (iso) wall_point<float>(b.qf, nd, w, o, depth, gf, M2f, Twf);
      else adiabatic_point<float>(b.qf, nd, w, o, depth, gf, M2f, true);
    }
  }
}

// Dirichlet face (dirichlet.py:27-41): the boundary plane and its `depth` halo layers take the
// values of the BC's equations, vals[v][layer][t] (layer l at -depth + l on side 0, N-1 + l on
// side 1), over the whole transverse allocation.
__global__ void k_dirichlet(BlockK b, int nv, int d, int side, int depth, int halo, const double* __restrict__ vals,
                            int fields) {
  const int tn = face_extent(b, d, halo);
  const int layers = depth + 1;
  const int total = tn * layers;
  const int c0 = side == 0 ? -depth : b.n[d] - 1;
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < total; u += gridDim.x * blockDim.x) {
    const int l = u / tn, t = u - l * tn;
    int c[3];
    face_point(b, d, halo, t, c);
    c[d] = c0 + l;
    const int id = lin(b, c[0], c[1], c[2]);
    for (int v = 0; v < nv; ++v) {
      const double x = vals[((size_t)v * layers + l) * tn + t];
      if (fields & BC_Q) b.q[v][id] = x;
      if ((fields & BC_QF) && b.qf[0]) b.qf[v][id] = d2f_rn(x);
    }
  }
}


// Block interfaces (multi_block.py:11-107, InterfaceBC): the halo layers of face (d, side) of a
// block receive the `depth` layers of its neighbour next to the neighbour's face (d, sside), in
// reverse order along the normal when flip is set (the match flag, opsc.py:1043-1045); the
// transverse range is the interior of the face (full = 0) or that plus `depth` halo points on
// each side (full = 1).  Every interface face of one boundary pass goes in one launch: the faces
// travel by value in the kernel's parameters (their FP32 pointers are the ping-pong buffers
// current at launch time, so a captured graph keeps the right ones per parity), and each thread
// finds its face from the faces' starting offsets.
constexpr int kIfMax = 24;
struct IfFace {
  long begin;                  // first element of this face in the launch's index space
  int d, side, sside, flip, depth, nv;
  int ext[3], lo[3];           // copied box: extents and lower corner (transverse), layers along d
  int dn[3], dst_st[3], dst_off0;
  int sn[3], src_st[3], src_off0;
  double* dq[5];
  const double* sq[5];
  float* dqf[5];
  const float* sqf[5];
};
struct IfBatch {
  int nfaces;
  long total;
  IfFace f[kIfMax];
};

__global__ void k_interface(const __grid_constant__ IfBatch batch, int fields) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < batch.total; t += (long)gridDim.x * blockDim.x) {
    int i = 0;
    while (i + 1 < batch.nfaces && batch.f[i + 1].begin <= t) ++i;
    const IfFace& F = batch.f[i];
    long r = t - F.begin;
    int c[3];
    c[0] = (int)(r % F.ext[0]); r /= F.ext[0];
    c[1] = (int)(r % F.ext[1]); r /= F.ext[1];
    c[2] = (int)(r % F.ext[2]);
    const int v = (int)(r / F.ext[2]);
    int di[3], si[3];
    for (int e = 0; e < 3; ++e) di[e] = si[e] = c[e] + F.lo[e];
    di[F.d] = F.side == 0 ? -F.depth + c[F.d] : F.dn[F.d] + c[F.d];
    const int sl = F.flip ? F.depth - 1 - c[F.d] : c[F.d];
    si[F.d] = F.sside == 1 ? F.sn[F.d] - F.depth + sl : sl;
    const int a = F.dst_off0 + di[0] * F.dst_st[0] + di[1] * F.dst_st[1] + di[2] * F.dst_st[2];
    const int bs = F.src_off0 + si[0] * F.src_st[0] + si[1] * F.src_st[1] + si[2] * F.src_st[2];
    if (fields & BC_Q) F.dq[v][a] = F.sq[v][bs];
    if ((fields & BC_QF) && F.dqf[0]) F.dqf[v][a] = F.sqf[v][bs];
  }
}

// FP32 copy of a metric array (rounded to nearest).
__global__ void k_metric_f32(const double* m, float* out, long n) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x)
    out[t] = d2f_rn(m[t]);
}

// ---------------------------------------------------------------------------------------
// Reductions (compressible_TGV.py:176-206 and the CFL / NaN checks), FP64.
__device__ __forceinline__ double uval(const BlockK& b, int v, long id) { return b.q[v][id] / b.q[0][id]; }

// d u_v / dx_d at the point (row j); a stretched y grid scales the y derivative by D11 of the row
__device__ __forceinline__ double d1g(const BlockK& b, int v, long id, int d, int j) {
  long s = b.st[d];
  const double inv = (d == 1 && b.ys[0]) ? b.invd[1] * b.ys[0][j] : b.invd[d];
  return ((1.0 / 12.0) * uval(b, v, id - 2 * s) - (2.0 / 3.0) * uval(b, v, id - s) + (2.0 / 3.0) * uval(b, v, id + s) -
          (1.0 / 12.0) * uval(b, v, id + 2 * s)) * inv;
}

struct RedParams {
  int what, nv, visc;
  double gama, Minf, mu_const, mu_pow;  // mu_pow: OSB_VISC_POWER_LAW exponent
};

__global__ void k_reduce(BlockK b, RedParams rp, double* partial, int slot) {
  __shared__ double sh[256];
  const long npts = (long)b.n[0] * b.n[1] * b.n[2];
  const bool is_min = rp.what == 4;
  double acc = is_min ? 1e300 : 0.0;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < npts; t += (long)gridDim.x * blockDim.x) {
    int i = (int)(t % b.n[0]);
    long r = t / b.n[0];
    int j = (int)(r % b.n[1]);
    int k = (int)(r / b.n[1]);
    long id = lin(b, i, j, k);
    const int nd = b.ndim;
    double rho = b.q[0][id];
    double u[3] = {0, 0, 0}, ke = 0.0;
    for (int e = 0; e < nd; ++e) { u[e] = b.q[1 + e][id] / rho; ke += u[e] * u[e]; }
    double p = (rp.gama - 1.0) * (b.q[rp.nv - 1][id] - 0.5 * rho * ke);
    double mu = rp.mu_const;
    if (rp.visc == OSB_VISC_SUTHERLAND || rp.visc == OSB_VISC_POWER_LAW) {
      double T = rp.Minf * rp.Minf * rp.gama * p / rho;
      mu = rp.visc == OSB_VISC_POWER_LAW ? pow(T, rp.mu_pow) : 1.4042 * T * sqrt(T) / (0.40417 + T);
    }
    double c = 0.0;
    switch (rp.what) {
      case 0: c = 0.5 * ke * rho; break;
      case 1: {
        double w2 = 0.0;
        if (nd == 3) {
          double wx = d1g(b, 3, id, 1, j) - d1g(b, 2, id, 2, j);
          double wy = d1g(b, 1, id, 2, j) - d1g(b, 3, id, 0, j);
          double wz = d1g(b, 2, id, 0, j) - d1g(b, 1, id, 1, j);
          w2 = wx * wx + wy * wy + wz * wz;
        } else if (nd == 2) {
          double wz = d1g(b, 2, id, 0, j) - d1g(b, 1, id, 1, j);
          w2 = wz * wz;
        }
        c = w2 * mu;
        break;
      }
      case 2: {
        double div = 0.0;
        for (int e = 0; e < nd; ++e) div += d1g(b, 1 + e, id, e, j);
        c = (4.0 / 3.0) * div * div * mu;
        break;
      }
      case 3: c = rho; break;
      case 4: {
        double a = sqrt(rp.gama * p / rho);
        double s = 0.0;
        for (int e = 0; e < nd; ++e) s += (fabs(u[e]) + a) * ((e == 1 && b.ys[0]) ? b.invd[1] * b.ys[0][j] : b.invd[e]);
        c = 1.0 / s;
        break;
      }
      case 5: {
        for (int v = 0; v < rp.nv; ++v)
          if (!isfinite(b.q[v][id])) c += 1.0;
        break;
      }
    }
    acc = is_min ? fmin(acc, c) : acc + c;
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = is_min ? fmin(sh[threadIdx.x], sh[threadIdx.x + s]) : sh[threadIdx.x] + sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[slot + blockIdx.x] = sh[0];
}

__global__ void k_reduce_final(const double* partial, int n, int is_min, double* out) {
  __shared__ double sh[256];
  double acc = is_min ? 1e300 : 0.0;
  for (int t = threadIdx.x; t < n; t += blockDim.x) acc = is_min ? fmin(acc, partial[t]) : acc + partial[t];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = is_min ? fmin(sh[threadIdx.x], sh[threadIdx.x + s]) : sh[threadIdx.x] + sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}



thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

int grid_for(osb_ctx* c, long n, int threads) {
  long g = (n + threads - 1) / threads;
  long cap = (long)c->sm_count * 8;
  return (int)std::max(1L, std::min(g, cap));
}

}  // namespace osb

namespace osb {

void timing_begin(osb_ctx* c, int fam) {
  if (!c->timing) return;
  TimedEvent te;
  te.fam = fam;
  for (int i = 0; i < 2; ++i) {
    cudaEvent_t e;
    if (!c->event_pool.empty()) {
      e = c->event_pool.back();
      c->event_pool.pop_back();
    } else {
      cudaEventCreate(&e);
    }
    (i == 0 ? te.a : te.b) = e;
  }
  cudaEventRecord(te.a, c->stream);
  c->events.push_back(te);
}

void timing_end(osb_ctx* c) {
  if (!c->timing || c->events.empty()) return;
  cudaEventRecord(c->events.back().b, c->stream);
}

}  // namespace osb

namespace {

// Folds completed timed launches into the per-family totals.
int timing_collect(osb_ctx* c) {
  if (c->events.empty()) return OSB_OK;
  OSB_CK(cudaStreamSynchronize(c->stream));
  for (auto& te : c->events) {
    float ms = 0.f;
    OSB_CK(cudaEventElapsedTime(&ms, te.a, te.b));
    c->fam_ms[te.fam] += ms;
    c->fam_count[te.fam] += 1;
    c->event_pool.push_back(te.a);
    c->event_pool.push_back(te.b);
  }
  c->events.clear();
  return OSB_OK;
}

// Residual kernels of one block.  With rf (FP32 path) the last of them applies the RK update
// itself (*fused = true): the central kernel when there is one, else the last sweep of a 2D/3D
// block.
template <typename T>
int residual_t(osb_ctx* c, Block& bl, const RkFuse* rf, bool* fused) {
  SchemeParams sp = scheme_params(bl.d.gama, bl.d.eps, bl.d.teno_ct, bl.d.shock_filter_control, 1e-12);
  if (fused) *fused = false;
  int rc;
  if (bl.d.scheme == OSB_SCHEME_CENTRAL4) {
    if (bl.d.ndim != 3) return fail(OSB_ENOTSUP, "central scheme implemented for 3D blocks");
    rc = sizeof(T) == 4 ? central_f32(c, bl, true, 1, rf) : central_f64(c, bl, true, 1, nullptr);
    if (fused) *fused = rf != nullptr;
  } else {
    const int nd = bl.d.ndim;
    const bool visc = bl.d.viscous != OSB_VISC_NONE;
    // the last sweep of a 3D Cartesian block carries the update (z sweep + update 4.34 against
    // 4.53 ms per step of the 256^3 Euler TGV with the separate k_rk32); the curvilinear sweeps
    // (168 registers) do not: there the extra FP64 state and register loads are not hidden
    // (5.60 against 5.01 ms per step of the 4-block case), nor in 2D, which is unmeasured
    const RkFuse* rs = (sizeof(T) == 4 && !visc && nd == 3 && !bl.k.m[9]) ? rf : nullptr;
    if (bl.k.m[9]) {
      if (sizeof(T) == 4) rc = nd == 2 ? flux_curv_f32_2d(c, bl, sp, rs) : flux_curv_f32_3d(c, bl, sp, rs);
      else rc = nd == 2 ? flux_curv_f64_2d(c, bl, sp, nullptr) : flux_curv_f64_3d(c, bl, sp, nullptr);
    } else if (sizeof(T) == 4) {
      rc = nd == 1 ? flux_f32_1d(c, bl, sp, nullptr) : nd == 2 ? flux_f32_2d(c, bl, sp, rs) : flux_f32_3d(c, bl, sp, rs);
    } else {
      rc = nd == 1 ? flux_f64_1d(c, bl, sp, nullptr) : nd == 2 ? flux_f64_2d(c, bl, sp, nullptr)
                                                          : flux_f64_3d(c, bl, sp, nullptr);
    }
    if (fused) *fused = rs != nullptr;
    if (rc == OSB_OK && visc) {
      if (bl.d.ndim != 3) return fail(OSB_ENOTSUP, "viscous terms implemented for 3D blocks");
      rc = sizeof(T) == 4 ? central_f32(c, bl, false, 0, rf) : central_f64(c, bl, false, 0, nullptr);
      if (fused) *fused = rf != nullptr;
    }
  }
  return rc;
}

int residual(osb_ctx* c, Block& bl) {
  return c->prec == OSB_PREC_FP32_RESIDUAL ? residual_t<float>(c, bl, nullptr, nullptr)
                                           : residual_t<double>(c, bl, nullptr, nullptr);
}


// Interface faces of every block: the interior of each face (full = 0) or the face with its
// transverse halos (full = 1).
int apply_interfaces(osb_ctx* c, int full, int fields) {
  IfBatch batch{};
  auto flush = [&]() {
    if (batch.nfaces == 0) return;
    timing_begin(c, FAM_BC);
    k_interface<<<grid_for(c, batch.total, 256), 256, 0, c->stream>>>(batch, fields);
    timing_end(c);
    c->launches++;
    batch.nfaces = 0;
    batch.total = 0;
  };
  for (size_t ib = 0; ib < c->blocks.size(); ++ib) {
    Block& bl = c->blocks[ib];
    const int nv = bl.d.ndim + 2;
    for (int d = 0; d < bl.d.ndim; ++d)
      for (int side = 0; side < 2; ++side) {
        if (bl.d.bc[d][side] != OSB_BC_INTERFACE) continue;
        const osb_interface& f = bl.d.iface[d][side];
        if (f.block < 0 || f.block >= (int)c->blocks.size())
          return fail(OSB_EINVAL, "interface of block %zu dir %d side %d names block %d of %zu", ib, d, side, f.block,
                      c->blocks.size());
        const Block& nb = c->blocks[f.block];
        for (int e = 0; e < bl.d.ndim; ++e)
          if (e != d && nb.k.n[e] != bl.k.n[e])
            return fail(OSB_EINVAL, "interface of block %zu dir %d: transverse size %d != %d of block %d", ib, d,
                        bl.k.n[e], nb.k.n[e], f.block);
        const int depth = bl.d.bc_depth[d][side] > 0 ? bl.d.bc_depth[d][side] : 4;
        if (depth > nb.k.n[d])
          return fail(OSB_EINVAL, "interface depth %d exceeds the %d points of block %d", depth, nb.k.n[d], f.block);
        if ((bl.k.qf[0] != nullptr) != (nb.k.qf[0] != nullptr))
          return fail(OSB_EINVAL, "interface between blocks of different precision");
        IfFace& F = batch.f[batch.nfaces];
        F.begin = batch.total;
        F.d = d;
        F.side = side;
        F.sside = f.side;
        F.flip = f.flip;
        F.depth = depth;
        F.nv = nv;
        long total = nv;
        for (int e = 0; e < 3; ++e) {
          if (e < bl.d.ndim && e != d) {
            F.lo[e] = full ? -depth : 0;
            F.ext[e] = bl.k.n[e] + (full ? 2 * depth : 0);
          } else {
            F.lo[e] = 0;
            F.ext[e] = 1;
          }
          F.dn[e] = bl.k.n[e];
          F.sn[e] = nb.k.n[e];
          F.dst_st[e] = bl.k.st[e];
          F.src_st[e] = nb.k.st[e];
        }
        F.ext[d] = depth;
        for (int e = 0; e < 3; ++e) total *= F.ext[e];
        F.dst_off0 = bl.k.off0;
        F.src_off0 = nb.k.off0;
        for (int v = 0; v < 5; ++v) {
          F.dq[v] = v < nv ? bl.k.q[v] : nullptr;
          F.sq[v] = v < nv ? nb.k.q[v] : nullptr;
          F.dqf[v] = v < nv ? bl.k.qf[v] : nullptr;
          F.sqf[v] = v < nv ? nb.k.qf[v] : nullptr;
        }
        batch.total += total;
        if (++batch.nfaces == kIfMax) flush();
      }
  }
  flush();
  return OSB_OK;
}

// Faces a single block can apply on its own (every kind but interfaces), with the periodic
// pairing checked: the validation osb_stage_noalloc does before its first launch.
bool block_faces_ok(const osb_block_desc& d, std::string& why) {
  for (int dd = 0; dd < d.ndim; ++dd) {
    const bool p0 = d.bc[dd][0] == OSB_BC_PERIODIC, p1 = d.bc[dd][1] == OSB_BC_PERIODIC;
    if (p0 != p1) {
      why = "periodic boundary on one side only (dir " + std::to_string(dd) + ")";
      return false;
    }
    for (int side = 0; side < 2; ++side)
      if (d.bc[dd][side] == OSB_BC_INTERFACE) {
        why = "block interfaces need osb_step on a context";
        return false;
      }
  }
  return true;
}

// Non-interface boundary faces of one block: the whole periodic halo shell in one launch when
// every face is periodic with one depth, else direction by direction (transverse ranges include
// the halos, so corners come from layers filled before) periodic, zero-gradient, extrapolation,
// symmetry, Dirichlet, pressure-outlet and wall faces.
int apply_block_bc(osb_ctx* c, Block& bl, size_t ib, int fields) {
  const int nv = bl.d.ndim + 2;
  if (const int D = uniform_periodic_depth(bl)) {
    long shell = 1, inner = 1;
    for (int e = 0; e < bl.d.ndim; ++e) {
      shell *= bl.k.n[e] + 2 * D;
      inner *= bl.k.n[e];
    }
    timing_begin(c, FAM_BC);
    k_periodic_shell<<<grid_for(c, shell - inner, 256), 256, 0, c->stream>>>(bl.k, nv, D, fields);
    timing_end(c);
    c->launches++;
    return OSB_OK;
  }
  for (int d = 0; d < bl.d.ndim; ++d) {
    int b0 = bl.d.bc[d][0], b1 = bl.d.bc[d][1];
    int dep0 = bl.d.bc_depth[d][0] > 0 ? bl.d.bc_depth[d][0] : 4;
    int dep1 = bl.d.bc_depth[d][1] > 0 ? bl.d.bc_depth[d][1] : 4;
    if (b0 == OSB_BC_PERIODIC && b1 == OSB_BC_PERIODIC) {
      long tr = 1;
      for (int e = 0; e < bl.d.ndim; ++e)
        if (e != d) tr *= bl.k.n[e] + 2 * std::max(dep0, dep1);
      long per = (long)std::max(dep0, dep1) * tr;
      timing_begin(c, FAM_BC);
      k_periodic<<<dim3(std::max(1, grid_for(c, per, 256) / (2 * nv) + 1), 2 * nv), 256, 0, c->stream>>>(
          bl.k, nv, d, dep0, dep1, fields);
      timing_end(c);
      c->launches++;
      continue;
    }
    for (int side = 0; side < 2; ++side) {
      int kind = bl.d.bc[d][side];
      if (kind == OSB_BC_ZERO_GRAD) {
        long tr = 1;
        for (int e = 0; e < bl.d.ndim; ++e)
          if (e != d) tr *= bl.k.n[e];
        timing_begin(c, FAM_BC);
        k_zero_grad<<<grid_for(c, tr, 128), 128, 0, c->stream>>>(bl.k, nv, d, side, side ? dep1 : dep0, fields);
        timing_end(c);
        c->launches++;
      } else if (kind == OSB_BC_EXTRAP0 || kind == OSB_BC_EXTRAP1) {
        long tr = 1;
        for (int e = 0; e < bl.d.ndim; ++e)
          if (e != d) tr *= bl.k.n[e];
        timing_begin(c, FAM_BC);
        k_extrap<<<grid_for(c, tr, 128), 128, 0, c->stream>>>(bl.k, nv, d, side, side ? dep1 : dep0,
                                                              kind == OSB_BC_EXTRAP1, fields);
        timing_end(c);
        c->launches++;
      } else if (kind == OSB_BC_SYMMETRY) {
        const long tr = face_extent(bl.k, d, bl.d.halo);
        timing_begin(c, FAM_BC);
        k_symmetry<<<grid_for(c, tr, 128), 128, 0, c->stream>>>(bl.k, nv, d, side, side ? dep1 : dep0,
                                                                bl.d.halo, fields);
        timing_end(c);
        c->launches++;
      } else if (kind == OSB_BC_DIRICHLET) {
        const int dep = side ? dep1 : dep0;
        const long tr = (long)face_extent(bl.k, d, bl.d.halo) * (dep + 1);
        timing_begin(c, FAM_BC);
        k_dirichlet<<<grid_for(c, tr, 128), 128, 0, c->stream>>>(bl.k, nv, d, side, dep, bl.d.halo,
                                                                 bl.d.dirichlet[d][side], fields);
        timing_end(c);
        c->launches++;
      } else if (kind == OSB_BC_PRESSURE_OUTLET) {
        const long tr = face_extent(bl.k, d, bl.d.halo);
        timing_begin(c, FAM_BC);
        k_pressure_outlet<<<grid_for(c, tr, 128), 128, 0, c->stream>>>(
            bl.k, nv, d, side, side ? dep1 : dep0, bl.d.halo, bl.d.back_pressure[d][side], bl.d.gama, fields);
        timing_end(c);
        c->launches++;
      } else if (kind == OSB_BC_ISOTHERMAL_WALL || kind == OSB_BC_ADIABATIC_WALL) {
        // over the transverse range the other faces' layers fill (the points beyond them hold
        // whatever the caller left, and a wall point there would divide by their density)
        int th = 1;
        for (int e = 0; e < bl.d.ndim; ++e)
          if (e != d) th = std::max(th, std::max(bl.d.bc_depth[e][0], bl.d.bc_depth[e][1]));
        th = std::min(th, bl.d.halo);
        const long tr = face_extent(bl.k, d, th);
        timing_begin(c, FAM_BC);
        k_wall<<<grid_for(c, tr, 128), 128, 0, c->stream>>>(
            bl.k, nv, kind, d, side, side ? dep1 : dep0, th, bl.d.gama, bl.d.Minf, bl.d.wall_temperature[d][side],
            (float)bl.d.gama, (float)(bl.d.Minf * bl.d.Minf), (float)bl.d.wall_temperature[d][side], fields);
        timing_end(c);
        c->launches++;
      } else if (kind == OSB_BC_PERIODIC) {
        return fail(OSB_EINVAL, "periodic boundary on one side only (block %zu dir %d)", ib, d);
      }
    }
  }
  return OSB_OK;
}

// Boundary conditions of all blocks: interface faces (interior of the face), then each
// block's own faces (apply_block_bc), then the interface faces again with their transverse
// halos, which the neighbour has filled by then.
int apply_bc(osb_ctx* c, int fields = BC_BOTH) {
  bool any_iface = false;
  for (auto& bl : c->blocks)
    for (int d = 0; d < bl.d.ndim; ++d)
      any_iface = any_iface || bl.d.bc[d][0] == OSB_BC_INTERFACE || bl.d.bc[d][1] == OSB_BC_INTERFACE;
  if (any_iface) {
    int rc = apply_interfaces(c, 0, fields);
    if (rc) return rc;
  }
  for (size_t ib = 0; ib < c->blocks.size(); ++ib) {
    int rc = apply_block_bc(c, c->blocks[ib], ib, fields);
    if (rc) return rc;
  }
  if (any_iface) return apply_interfaces(c, 1, fields);
  return OSB_OK;
}

// Whether stages run as the persistent fused launch (osb_batch.cu).
bool use_batch(const osb_ctx* c) {
  if (c->sched.mode == OSB_SCHED_PER_BLOCK) return false;
  return batch_eligible(c, nullptr);
}

// One RK stage of every block; bc = false leaves the boundary treatment after it out (the
// generated step with a filter exchanges no halos after its last stage).
int stage(osb_ctx* c, int s, double dt, bool bc = true) {
  if (use_batch(c)) return batch_stage(c, s, dt);
  const int kind = c->rk_kind == OSB_RK_LOW_STORAGE ? 0 : 1;
  if (c->prec == OSB_PREC_FP32_RESIDUAL) {
    // the last residual kernel of each block applies the RK update and writes the next FP32
    // state into the other buffer; blocks without such a kernel (1D) use k_rk32
    for (auto& bl : c->blocks) {
      RkFuse rf{};
      rf.kind = kind;
      rf.a_zero = (kind == 0 && c->A[s] == 0.0) ? 1 : 0;
      rf.A = c->A[s];
      rf.dt_h = (float)dt;
      rf.dt_l = (float)(dt - (double)rf.dt_h);
      rf.B = c->B[s];
      rf.dt = dt;
      rf.bad = c->bad;
      rf.stall = c->bad + 1;
      float* out = c->qf_parity ? bl.qf_base : bl.qf_alt;
      for (int v = 0; v < bl.d.ndim + 2; ++v) rf.qout[v] = out + (size_t)v * bl.k.alloc;
      bool fused = false;
      int rc = residual_t<float>(c, bl, c->sched.fuse_update ? &rf : nullptr, &fused);
      if (rc) return rc;
      if (!fused) {
        long n = (long)bl.k.n[0] * bl.k.n[1] * bl.k.n[2];
        timing_begin(c, FAM_RK);
        k_rk32<<<grid_for(c, n, 256), 256, 0, c->stream>>>(bl.k, bl.d.ndim + 2, rf);
        timing_end(c);
        c->launches++;
      }
    }
    batch_set_parity(c, c->qf_parity ^ 1);
    // between stages the FP32 kernels read only the FP32 state; the FP64 halos are refreshed
    // when a call returns (osb_step / osb_stage)
    return bc ? apply_bc(c, BC_QF) : OSB_OK;
  }
  for (auto& bl : c->blocks) {
    int rc = residual(c, bl);
    if (rc) return rc;
  }
  for (auto& bl : c->blocks) {
    long n = (long)bl.k.n[0] * bl.k.n[1] * bl.k.n[2];
    timing_begin(c, FAM_RK);
    k_rk<<<grid_for(c, n, 256), 256, 0, c->stream>>>(bl.k, bl.d.ndim + 2, kind, c->A[s], c->B[s], dt, c->bad);
    timing_end(c);
    c->launches++;
  }
  return bc ? apply_bc(c) : OSB_OK;
}

bool any_filter(const osb_ctx* c, int kind) {
  for (const auto& bl : c->blocks)
    if (bl.d.filter == kind) return true;
  return false;
}

// FP32-residual path: refresh the FP32 shadow from the caller's FP64 state (the caller may
// have written q between calls).
int sync_shadow(osb_ctx* c) {
  if (c->prec != OSB_PREC_FP32_RESIDUAL) return OSB_OK;
  for (auto& bl : c->blocks) {
    dim3 grid(grid_for(c, bl.k.alloc, 256), bl.d.ndim + 2);
    k_q2qf<<<grid, 256, 0, c->stream>>>(bl.k, bl.d.ndim + 2);
    c->launches++;
  }
  return OSB_OK;
}

int one_step(osb_ctx* c, double dt) {
  if (use_batch(c)) {
    // periodic images are read in place and the SBLI save is folded into stage 0
    for (int s = 0; s < c->nst; ++s) {
      int rc = batch_stage(c, s, dt);
      if (rc) return rc;
    }
    return OSB_OK;
  }
  int rc = apply_bc(c, c->prec == OSB_PREC_FP32_RESIDUAL ? BC_QF : BC_BOTH);
  if (rc) return rc;
  if (c->rk_kind == OSB_RK_SBLI3) {
    for (auto& bl : c->blocks) {
      long n = (long)bl.k.n[0] * bl.k.n[1] * bl.k.n[2];
      k_save<<<grid_for(c, n, 256), 256, 0, c->stream>>>(bl.k, bl.d.ndim + 2);
      c->launches++;
    }
  }
  // with a WENO-filtered block the last stage exchanges no halos: the filter step's own
  // exchange follows it (the next step starts with the full exchange); the TVD-filtered step
  // exchanges after every stage and keeps the velocities at index -2 that its last stage reads
  const bool fp32 = c->prec == OSB_PREC_FP32_RESIDUAL;
  const bool weno = any_filter(c, OSB_FILTER_WENO3), tvd = any_filter(c, OSB_FILTER_TVD);
  for (int s = 0; s < c->nst; ++s) {
    if (tvd && s == c->nst - 1)
      for (auto& bl : c->blocks) {
        if (bl.d.filter != OSB_FILTER_TVD) continue;
        rc = fp32 ? tvd_stale_f32(c, bl) : tvd_stale_f64(c, bl);
        if (rc) return rc;
      }
    rc = stage(c, s, dt, !(weno && s == c->nst - 1));
    if (rc) return rc;
  }
  if (weno || tvd)
    for (auto& bl : c->blocks) {
      if (bl.d.filter == OSB_FILTER_NONE) continue;
      rc = fp32 ? filter_f32(c, bl, dt) : filter_f64(c, bl, dt);
      if (rc) return rc;
    }
  return OSB_OK;
}

void drop_graph(osb_ctx* c) {
  if (c->gexec) {
    cudaGraphExecDestroy(c->gexec);
    c->gexec = nullptr;
  }
  for (int p = 0; p < 2; ++p)
    if (c->gexec_p[p]) {
      cudaGraphExecDestroy(c->gexec_p[p]);
      c->gexec_p[p] = nullptr;
    }
}

bool check_desc(const osb_block_desc* d, std::string& why) {
  if (d->ndim < 1 || d->ndim > 3) { why = "ndim must be 1, 2 or 3"; return false; }
  if (d->halo != 5) { why = "halo must be 5 (OPS layout)"; return false; }
  for (int i = 0; i < d->ndim; ++i)
    if (d->size[i] < 6) { why = "every used direction needs at least 6 points"; return false; }
  for (int i = d->ndim; i < 3; ++i)
    if (d->size[i] != 1) { why = "unused directions must have size 1"; return false; }
  if (!(d->scheme == OSB_SCHEME_WENO5_JS || d->scheme == OSB_SCHEME_WENO5_Z || d->scheme == OSB_SCHEME_TENO5 ||
        d->scheme == OSB_SCHEME_TENO6 || d->scheme == OSB_SCHEME_CENTRAL4)) { why = "unknown scheme"; return false; }
  if (d->averaging != OSB_AVG_SIMPLE && d->averaging != OSB_AVG_ROE) { why = "unknown averaging"; return false; }
  if (d->viscous == OSB_VISC_SUTHERLAND_RATIO) {
    why = "Sutherland's law with a SuthT / RefT ratio is restated in the oracle only (no GPU kernel)";
    return false;
  }
  if (d->viscous < OSB_VISC_NONE || d->viscous > OSB_VISC_POWER_LAW) { why = "unknown viscosity law"; return false; }
  if (d->viscous == OSB_VISC_POWER_LAW && !(d->visc_power > 0.0)) {
    why = "the power-law viscosity needs a positive exponent (visc_power)";
    return false;
  }
  if ((d->forcing[0] != 0.0 || d->forcing[1] != 0.0 || d->forcing[2] != 0.0) &&
      (d->ndim != 3 || d->viscous == OSB_VISC_NONE || d->metric[9])) {
    why = "the constant forcing terms are applied by the central viscous kernel of 3D Cartesian blocks";
    return false;
  }
  for (int v = 0; v < d->ndim + 2; ++v)
    if (!d->q[v] || !d->rkold[v]) { why = "null state or RK array"; return false; }
  for (int i = 0; i < d->ndim; ++i)
    for (int s = 0; s < 2; ++s) {
      int dep = d->bc_depth[i][s];
      if (dep < 0 || dep > 5) { why = "boundary depth must be 0..5"; return false; }
    }
  if (d->gama <= 1.0) { why = "gama must exceed 1"; return false; }
  bool curv = false;
  for (int i = 0; i < 10; ++i) curv = curv || d->metric[i] != nullptr;
  if (curv) {
    if (d->ndim < 2) { why = "curvilinear blocks are 2D or 3D"; return false; }
    for (int dd = 0; dd < d->ndim; ++dd)
      for (int i = 0; i < d->ndim; ++i)
        if (!d->metric[3 * dd + i]) { why = "metric D" + std::to_string(dd) + std::to_string(i) + " missing"; return false; }
    if (!d->metric[9]) { why = "metric detJ missing"; return false; }
    if (d->scheme == OSB_SCHEME_CENTRAL4 || d->viscous != OSB_VISC_NONE) {
      why = "curvilinear blocks take the characteristic Euler flux only (no central or viscous terms)";
      return false;
    }
  }
  for (int i = 0; i < d->ndim; ++i)
    for (int s = 0; s < 2; ++s) {
      const int k = d->bc[i][s];
      if (k == OSB_BC_INLET_PRESSURE_EXTRAP) {
        why = "the pressure-extrapolation inlet is restated in the oracle only (no GPU kernel)";
        return false;
      }
      if (k < OSB_BC_PERIODIC || k > OSB_BC_ADIABATIC_WALL) { why = "unknown boundary kind"; return false; }
      if (k == OSB_BC_ISOTHERMAL_WALL || k == OSB_BC_ADIABATIC_WALL) {
        if (d->ndim != 3 || i != 1 || d->metric[9] || d->scheme == OSB_SCHEME_CENTRAL4) {
          why = "walls are implemented on the y faces of 3D Cartesian blocks with a shock-capturing scheme";
          return false;
        }
        if (k == OSB_BC_ISOTHERMAL_WALL && !(d->wall_temperature[i][s] > 0.0)) {
          why = "an isothermal wall needs a positive wall temperature";
          return false;
        }
        const int wd = d->bc_depth[i][s] > 0 ? d->bc_depth[i][s] : 4;
        if (wd > d->halo || d->size[i] < 12) {
          why = "walls: depth up to the halo, at least 12 points between the walls";
          return false;
        }
      }
      const int dep = d->bc_depth[i][s] > 0 ? d->bc_depth[i][s] : 4;
      if ((k == OSB_BC_SYMMETRY || k == OSB_BC_DIRICHLET || k == OSB_BC_PRESSURE_OUTLET) &&
          (dep > d->halo || dep >= d->size[i])) {
        why = "symmetry / Dirichlet / pressure-outlet depth must be below the halo and the block size";
        return false;
      }
      if ((k == OSB_BC_SYMMETRY || k == OSB_BC_PRESSURE_OUTLET) && d->metric[9]) {
        why = "the symmetry and pressure-outlet boundaries are implemented for Cartesian blocks";
        return false;
      }
      if (k == OSB_BC_PRESSURE_OUTLET && !(d->back_pressure[i][s] > 0.0)) {
        why = "a pressure outlet needs a positive back pressure";
        return false;
      }
      if (k == OSB_BC_DIRICHLET && !d->dirichlet[i][s]) {
        why = "a Dirichlet face needs its values (osb_block_desc.dirichlet)";
        return false;
      }
      // ExtrapolationBC, DirichletBC and PressureOutletBC are ModifyCentralDerivative faces
      // (bc_core.py:15-17): the reference's central derivatives take the Carpenter closures next
      // to them, which the central kernel implements at y walls only
      if ((k == OSB_BC_EXTRAP0 || k == OSB_BC_EXTRAP1 || k == OSB_BC_DIRICHLET || k == OSB_BC_PRESSURE_OUTLET) &&
          (d->scheme == OSB_SCHEME_CENTRAL4 || d->viscous != OSB_VISC_NONE)) {
        why = "extrapolation, Dirichlet and pressure-outlet faces with central derivatives need the Carpenter "
              "boundary closures (implemented at y walls only)";
        return false;
      }
    }
  if ((d->ystretch[0] != nullptr) != (d->ystretch[1] != nullptr)) {
    why = "a stretched y grid needs both D11 and SD111 (osb_block_desc.ystretch)";
    return false;
  }
  if (d->ystretch[0]) {
    auto wall = [](int k) { return k == OSB_BC_ISOTHERMAL_WALL || k == OSB_BC_ADIABATIC_WALL; };
    if (d->ndim != 3 || d->metric[9] || d->viscous == OSB_VISC_NONE || !wall(d->bc[1][0]) || !wall(d->bc[1][1])) {
      why = "a stretched y grid is implemented for 3D Cartesian viscous blocks with walls on both y faces";
      return false;
    }
  }
  for (int i = 0; i < d->ndim; ++i)
    for (int s = 0; s < 2; ++s) {
      if (d->bc[i][s] != OSB_BC_INTERFACE) continue;
      const osb_interface& f = d->iface[i][s];
      if (f.dir != i || (f.flip != 0 && f.flip != 1)) {
        why = "interfaces connect faces normal to the same direction (flip 0 or 1)";
        return false;
      }
      if (f.side != 0 && f.side != 1) { why = "interface side must be 0 or 1"; return false; }
    }
  if (d->flux_type == OSB_FLUX_HLLC_LM &&
      (d->ndim < 2 || curv || !(d->scheme == OSB_SCHEME_WENO5_JS || d->scheme == OSB_SCHEME_WENO5_Z ||
                                d->scheme == OSB_SCHEME_TENO5))) {
    why = "the HLLC-LM flux is implemented for Cartesian 2D / 3D blocks with WENO5-JS, WENO5-Z or TENO5";
    return false;
  }
  if (d->flux_type != OSB_FLUX_LLF && d->flux_type != OSB_FLUX_HLLC_LM) { why = "unknown flux type"; return false; }
  if (d->split_form != OSB_SPLIT_FEIEREISEN && d->split_form != OSB_SPLIT_KGP) { why = "unknown split form"; return false; }
  if (d->split_form == OSB_SPLIT_KGP && d->scheme != OSB_SCHEME_CENTRAL4) {
    why = "the KGP split form belongs to the central scheme";
    return false;
  }
  if (d->filter != OSB_FILTER_NONE && d->filter != OSB_FILTER_WENO3 && d->filter != OSB_FILTER_TVD) {
    why = "unknown filter";
    return false;
  }
  if (d->filter != OSB_FILTER_NONE) {
    if (d->ndim != 3 || d->scheme != OSB_SCHEME_CENTRAL4 || d->metric[9]) {
      why = "the non-linear filters are implemented for 3D Cartesian blocks of the central scheme";
      return false;
    }
    for (int i = 0; i < 3; ++i)
      for (int s = 0; s < 2; ++s)
        if (d->bc[i][s] != OSB_BC_PERIODIC || d->size[i] < 4) {
          why = "the filter's halo exchange is the periodic one (all faces periodic, >= 4 points)";
          return false;
        }
  }
  if (d->filter == OSB_FILTER_WENO3 && (!(d->ducros_check >= 0.0) || !(d->ducros_select >= 0.0))) {
    why = "Ducros thresholds must be >= 0";
    return false;
  }
  if (d->filter == OSB_FILTER_TVD) {
    if (!std::isfinite(d->tvd_kappa)) { why = "kappa_TVD must be finite"; return false; }
    // the interface at -1 reads index -2, which the stage exchange must fill
    for (int i = 0; i < 3; ++i)
      for (int s = 0; s < 2; ++s)
        if (d->bc_depth[i][s] > 0 && d->bc_depth[i][s] < 2) {
          why = "the TVD filter needs a periodic exchange of depth >= 2";
          return false;
        }
  }
  return true;
}

}  // namespace

// ---------------------------------------------------------------------------------------
extern "C" {

int osb_version(void) { return OSB_VERSION; }

int osb_last_error(char* buf, size_t n) {
  if (!buf || n == 0) return (int)g_err.size();
  size_t m = std::min(n - 1, g_err.size());
  memcpy(buf, g_err.data(), m);
  buf[m] = 0;
  return (int)m;
}

int osb_desc_layout(long long* out, int n) {
  if (!out || n < 20) return fail(OSB_EINVAL, "need 20 slots");
  out[0] = sizeof(osb_block_desc);
  out[1] = offsetof(osb_block_desc, size);
  out[2] = offsetof(osb_block_desc, bc);
  out[3] = offsetof(osb_block_desc, iface);
  out[4] = offsetof(osb_block_desc, gama);
  out[5] = offsetof(osb_block_desc, delta);
  out[6] = offsetof(osb_block_desc, q);
  out[7] = offsetof(osb_block_desc, rkold);
  out[8] = offsetof(osb_block_desc, metric);
  out[9] = offsetof(osb_block_desc, split_form);
  out[10] = offsetof(osb_block_desc, ducros_check);
  out[11] = offsetof(osb_block_desc, tvd_kappa);
  out[12] = offsetof(osb_block_desc, dirichlet);
  out[13] = offsetof(osb_block_desc, flux_type);
  out[14] = offsetof(osb_block_desc, back_pressure);
  out[15] = offsetof(osb_block_desc, wall_temperature);
  out[16] = offsetof(osb_block_desc, ystretch);
  out[17] = offsetof(osb_block_desc, visc_power);
  out[18] = offsetof(osb_block_desc, forcing);
  out[19] = offsetof(osb_block_desc, sutherland_s);
  return OSB_OK;
}

// Stretched wall-normal metrics of a grid line (the generated "MetricsEquation evaluation"
// kernels of a y-stretched MetricsEquation: x1' and D11 = 1 / x1', then SD111 = D11'; each
// derivative the central 4th-order rule, or the Carpenter closure rows in the four rows next to
// a wall face).  Host work only.
int osb_ystretch_metrics(int32_t n, double delta, const double* x1, int32_t wall_lo, int32_t wall_hi, double* d11,
                         double* sd111) {
  if (!x1 || !d11 || !sd111) return fail(OSB_EINVAL, "null argument");
  if (n < 12) return fail(OSB_EINVAL, "a stretched line needs at least 12 points (got %d)", n);
  if (!(delta > 0.0)) return fail(OSB_EINVAL, "delta must be positive");
  const bool inc = x1[1] > x1[0];
  for (int j = 0; j + 1 < n; ++j)
    if (inc ? !(x1[j + 1] > x1[j]) : !(x1[j + 1] < x1[j]))
      return fail(OSB_EINVAL, "the grid line is not strictly monotone (rows %d, %d)", j, j + 1);
  const Closures& cl = closures();
  const double inv = 1.0 / delta;
  // derivative of f at row j: closure rows next to a wall, the central rule elsewhere (which
  // needs j -2 .. j +2 inside the line: a line without walls is refused below)
  auto der = [&](const std::vector<double>& f, int j, double& out) -> bool {
    int r = -1;
    bool hi = false;
    if (wall_lo && j < 4) r = j;
    else if (wall_hi && j > n - 5) { r = n - 1 - j; hi = true; }
    double acc = 0.0;
    if (r >= 0) {
      for (int m = 0; m < 6; ++m) {
        if (cl.c1[r][m] == 0.0) continue;
        const int o = hi ? r - m : m - r;
        acc += (hi ? -cl.c1[r][m] : cl.c1[r][m]) * f[j + o];
      }
    } else {
      if (j < 2 || j > n - 3) return false;
      acc = (1.0 / 12.0) * f[j - 2] - (2.0 / 3.0) * f[j - 1] + (2.0 / 3.0) * f[j + 1] - (1.0 / 12.0) * f[j + 2];
    }
    out = acc * inv;
    return true;
  };
  std::vector<double> xl(x1, x1 + n), dl(n);
  for (int j = 0; j < n; ++j) {
    double xd = 0.0;
    if (!der(xl, j, xd)) return fail(OSB_EINVAL, "row %d: a stretched line needs wall faces at both ends", j);
    if (xd == 0.0 || !std::isfinite(xd)) return fail(OSB_EINVAL, "row %d: the grid line is not strictly monotone", j);
    dl[j] = 1.0 / xd;
    d11[j] = dl[j];
  }
  for (int j = 0; j < n; ++j) {
    double v = 0.0;
    der(dl, j, v);
    sd111[j] = v;
  }
  return OSB_OK;
}

int osb_ctx_create(int device, int precision, osb_ctx** out) {
  if (!out) return fail(OSB_EINVAL, "null out");
  if (precision != OSB_PREC_FP64 && precision != OSB_PREC_FP32_RESIDUAL) return fail(OSB_EINVAL, "bad precision");
  int ndev = 0;
  OSB_CK(cudaGetDeviceCount(&ndev));
  if (device < 0 || device >= ndev) return fail(OSB_EINVAL, "device %d out of range (%d devices)", device, ndev);
  OSB_CK(cudaSetDevice(device));
  osb_ctx* c = new osb_ctx;
  c->device = device;
  c->prec = precision;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) == cudaSuccess) c->sm_count = prop.multiProcessorCount;
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { delete c; return fail(OSB_ECUDA, "stream: %s", cudaGetErrorString(e)); }
  c->red_slots = c->sm_count * 8 + 1;
  e = cudaMalloc(&c->red, sizeof(double) * (c->red_slots + 8) * 64);
  if (e == cudaSuccess) e = cudaMalloc(&c->bad, 2 * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMallocHost(&c->red_host, sizeof(double) * 8);
  if (e == cudaSuccess) e = cudaMemset(c->bad, 0, 2 * sizeof(unsigned long long));
  if (e != cudaSuccess) {
    osb_ctx_destroy(c);
    return fail(OSB_ECUDA, "workspace: %s", cudaGetErrorString(e));
  }
  *out = c;
  return OSB_OK;
}

namespace {

void requests_free(osb_ctx* c) {
  for (int k = 0; k < 2; ++k) {
    if (c->stage_in[k]) cudaFree(c->stage_in[k]);
    if (c->stage_out[k]) cudaFree(c->stage_out[k]);
    c->stage_in[k] = c->stage_out[k] = nullptr;
    for (cudaEvent_t* e : {&c->ev_in[k], &c->ev_used[k], &c->ev_res[k], &c->ev_out[k]})
      if (*e) {
        cudaEventDestroy(*e);
        *e = nullptr;
      }
  }
  if (c->cs_in) cudaStreamDestroy(c->cs_in);
  if (c->cs_out) cudaStreamDestroy(c->cs_out);
  c->cs_in = c->cs_out = nullptr;
  c->stage_bytes = 0;
}

// Bytes of one request: every block's variables, whole allocations, in block order.
size_t request_bytes(const osb_ctx* c) {
  size_t n = 0;
  for (const auto& bl : c->blocks) n += (size_t)(bl.d.ndim + 2) * bl.k.alloc * sizeof(double);
  return n;
}

int requests_setup(osb_ctx* c) {
  const size_t bytes = request_bytes(c);
  if (c->stage_bytes == bytes && c->cs_in) return OSB_OK;
  OSB_CK(cudaStreamSynchronize(c->stream));
  if (c->cs_in) OSB_CK(cudaStreamSynchronize(c->cs_in));
  if (c->cs_out) OSB_CK(cudaStreamSynchronize(c->cs_out));
  requests_free(c);
  OSB_CK(cudaStreamCreateWithFlags(&c->cs_in, cudaStreamNonBlocking));
  OSB_CK(cudaStreamCreateWithFlags(&c->cs_out, cudaStreamNonBlocking));
  for (int k = 0; k < 2; ++k) {
    cudaError_t e = cudaMalloc(&c->stage_in[k], bytes);
    if (e == cudaSuccess) e = cudaMalloc(&c->stage_out[k], bytes);
    if (e != cudaSuccess) {
      requests_free(c);
      return fail(OSB_ECUDA, "request staging (%zu bytes x 4): %s", bytes, cudaGetErrorString(e));
    }
    for (cudaEvent_t* ev : {&c->ev_in[k], &c->ev_used[k], &c->ev_res[k], &c->ev_out[k]})
      OSB_CK(cudaEventCreateWithFlags(ev, cudaEventDisableTiming));
  }
  c->stage_bytes = bytes;
  return OSB_OK;
}

// Copies between the blocks' state arrays and one staging slot (to_state: slot -> state).
int stage_copy(osb_ctx* c, char* slot, bool to_state) {
  size_t off = 0;
  for (auto& bl : c->blocks)
    for (int v = 0; v < bl.d.ndim + 2; ++v) {
      const size_t n = (size_t)bl.k.alloc * sizeof(double);
      if (to_state)
        OSB_CK(cudaMemcpyAsync(bl.k.q[v], slot + off, n, cudaMemcpyDeviceToDevice, c->stream));
      else
        OSB_CK(cudaMemcpyAsync(slot + off, bl.k.q[v], n, cudaMemcpyDeviceToDevice, c->stream));
      off += n;
    }
  return OSB_OK;
}

}  // namespace

int osb_step_requests(osb_ctx* c, int count, const double* const* in, double* const* out, double dt, int nsteps) {
  if (!c || (count > 0 && (!in || !out))) return fail(OSB_EINVAL, "null argument");
  if (count < 0 || nsteps < 0) return fail(OSB_EINVAL, "count or nsteps < 0");
  if (c->blocks.empty()) return fail(OSB_EINVAL, "no blocks");
  if (count == 0) return OSB_OK;
  for (int r = 0; r < count; ++r)
    if (!in[r] || !out[r]) return fail(OSB_EINVAL, "request %d has a null buffer", r);
  OSB_CK(cudaSetDevice(c->device));
  int rc = requests_setup(c);
  if (rc) return rc;
  const size_t bytes = c->stage_bytes;
  // once copies are queued, an error waits for every stream before returning: the caller may
  // free its host buffers as soon as the call returns
  auto drain = [&](int code) -> int {
    cudaStreamSynchronize(c->cs_in);
    cudaStreamSynchronize(c->cs_out);
    cudaStreamSynchronize(c->stream);
    return code;
  };
  auto ck = [&](cudaError_t e, const char* what) -> int {
    return e == cudaSuccess ? OSB_OK : drain(fail(OSB_ECUDA, "%s: %s", what, cudaGetErrorString(e)));
  };
  // request r uses slot r & 1 in each direction; the copy of request r + 1 in and of r - 1 out
  // overlap the steps of request r
  auto h2d = [&](int r) -> int {
    const int k = r & 1;
    int e = OSB_OK;
    if (r >= 2) e = ck(cudaStreamWaitEvent(c->cs_in, c->ev_used[k], 0), "wait");
    if (!e) e = ck(cudaMemcpyAsync(c->stage_in[k], in[r], bytes, cudaMemcpyHostToDevice, c->cs_in), "copy in");
    if (!e) e = ck(cudaEventRecord(c->ev_in[k], c->cs_in), "record");
    return e;
  };
  if ((rc = h2d(0))) return rc;
  for (int r = 0; r < count; ++r) {
    const int k = r & 1;
    if (r + 1 < count && (rc = h2d(r + 1))) return rc;
    if ((rc = ck(cudaStreamWaitEvent(c->stream, c->ev_in[k], 0), "wait"))) return rc;
    if ((rc = stage_copy(c, (char*)c->stage_in[k], true))) return drain(rc);
    if ((rc = ck(cudaEventRecord(c->ev_used[k], c->stream), "record"))) return rc;
    if ((rc = osb_step(c, dt, nsteps))) return drain(rc);
    if (r >= 2 && (rc = ck(cudaStreamWaitEvent(c->stream, c->ev_out[k], 0), "wait"))) return rc;
    if ((rc = stage_copy(c, (char*)c->stage_out[k], false))) return drain(rc);
    if ((rc = ck(cudaEventRecord(c->ev_res[k], c->stream), "record"))) return rc;
    if ((rc = ck(cudaStreamWaitEvent(c->cs_out, c->ev_res[k], 0), "wait"))) return rc;
    if ((rc = ck(cudaMemcpyAsync(out[r], c->stage_out[k], bytes, cudaMemcpyDeviceToHost, c->cs_out), "copy out")))
      return rc;
    if ((rc = ck(cudaEventRecord(c->ev_out[k], c->cs_out), "record"))) return rc;
  }
  OSB_CK(cudaStreamSynchronize(c->cs_out));
  OSB_CK(cudaStreamSynchronize(c->stream));
  return OSB_OK;
}

int osb_ctx_destroy(osb_ctx* c) {
  if (!c) return OSB_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  drop_graph(c);
  for (auto& te : c->events) {
    cudaEventDestroy(te.a);
    cudaEventDestroy(te.b);
  }
  for (auto e : c->event_pool) cudaEventDestroy(e);
  for (auto& bl : c->blocks) {
    if (bl.k.R[0]) cudaFree(bl.k.R[0]);
    if (bl.qf_base) cudaFree(bl.qf_base);  // k.qf may point at either ping-pong buffer
    if (bl.mf_buf) cudaFree(bl.mf_buf);
    if (bl.qf_alt) cudaFree(bl.qf_alt);
    if (bl.filt_ws) cudaFree(bl.filt_ws);
    if (bl.xrows) cudaFree(bl.xrows);
    if (bl.ys_buf) cudaFree(bl.ys_buf);
  }
  batch_free(c);
  requests_free(c);
  if (c->resident) cudaFree(c->resident);
  if (c->red) cudaFree(c->red);
  if (c->bad) cudaFree(c->bad);
  if (c->red_host) cudaFreeHost(c->red_host);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return OSB_OK;
}

int osb_block_add(osb_ctx* c, const osb_block_desc* d, int* block_id) {
  if (!c || !d) return fail(OSB_EINVAL, "null argument");
  std::string why;
  if (!check_desc(d, why)) return fail(OSB_EINVAL, "invalid block descriptor: %s", why.c_str());
  if (!c->blocks.empty()) {
    const osb_block_desc& f = c->blocks[0].d;
    if (f.ndim != d->ndim || f.scheme != d->scheme || f.averaging != d->averaging || f.viscous != d->viscous)
      return fail(OSB_EINVAL, "blocks of one context must share ndim, scheme, averaging and viscosity");
  }
  OSB_CK(cudaSetDevice(c->device));
  Block bl;
  bl.d = *d;
  BlockK& k = bl.k;
  memset(&k, 0, sizeof k);
  k.ndim = d->ndim;
  long ext[3];
  for (int i = 0; i < 3; ++i) {
    k.n[i] = i < d->ndim ? d->size[i] : 1;
    ext[i] = i < d->ndim ? d->size[i] + 2 * d->halo : 1;
    k.invd[i] = i < d->ndim ? 1.0 / d->delta[i] : 0.0;
    k.invdf[i] = (float)k.invd[i];
    k.inv2d[i] = i < d->ndim ? 1.0 / (d->delta[i] * d->delta[i]) : 0.0;
  }
  if (ext[0] * ext[1] * ext[2] >= (1L << 31)) return fail(OSB_EINVAL, "block too large for 32-bit indexing");
  k.st[0] = 1;
  k.st[1] = (int)ext[0];
  k.st[2] = (int)(ext[0] * ext[1]);
  k.alloc = ext[0] * ext[1] * ext[2];
  k.off0 = d->halo + (d->ndim > 1 ? d->halo * k.st[1] : 0) + (d->ndim > 2 ? d->halo * k.st[2] : 0);
  const int nv = d->ndim + 2;
  for (int v = 0; v < nv; ++v) {
    k.q[v] = d->q[v];
    k.rk[v] = d->rkold[v];
  }
  double* R = nullptr;
  OSB_CK(cudaMalloc(&R, sizeof(double) * k.alloc * nv));
  OSB_CK(cudaMemsetAsync(R, 0, sizeof(double) * k.alloc * nv, c->stream));
  for (int v = 0; v < nv; ++v) k.R[v] = R + (size_t)v * k.alloc;
  if (c->prec == OSB_PREC_FP32_RESIDUAL) {
    // the float-float residual reuses the FP64 residual bytes; the FP32 shadow of q is extra
    float* Rf = reinterpret_cast<float*>(R);
    for (int v = 0; v < nv; ++v) {
      k.Rh[v] = Rf + (size_t)(2 * v) * k.alloc;
      k.Rl[v] = Rf + (size_t)(2 * v + 1) * k.alloc;
    }
    float* qf = nullptr;
    cudaError_t e = cudaMalloc(&qf, sizeof(float) * k.alloc * nv);
    if (e != cudaSuccess) {
      cudaFree(R);
      return fail(OSB_ECUDA, "FP32 shadow: %s", cudaGetErrorString(e));
    }
    for (int v = 0; v < nv; ++v) k.qf[v] = qf + (size_t)v * k.alloc;
    bl.qf_base = qf;
    e = cudaMalloc(&bl.qf_alt, sizeof(float) * k.alloc * nv);  // ping-pong partner
    if (e != cudaSuccess) {
      cudaFree(R);
      cudaFree(qf);
      return fail(OSB_ECUDA, "FP32 state: %s", cudaGetErrorString(e));
    }
    OSB_CK(cudaMemsetAsync(bl.qf_alt, 0, sizeof(float) * k.alloc * nv, c->stream));
  }
  for (int i = 0; i < 10; ++i) k.m[i] = d->metric[i];
  if (k.m[9] && c->prec == OSB_PREC_FP32_RESIDUAL) {
    int nm = 0;
    for (int i = 0; i < 10; ++i) nm += k.m[i] ? 1 : 0;
    float* mf = nullptr;
    cudaError_t e = cudaMalloc(&mf, sizeof(float) * k.alloc * nm);
    if (e != cudaSuccess) {
      cudaFree(R);
      cudaFree(bl.qf_base);
      cudaFree(bl.qf_alt);
      return fail(OSB_ECUDA, "FP32 metrics: %s", cudaGetErrorString(e));
    }
    bl.mf_buf = mf;
    for (int i = 0, j = 0; i < 10; ++i) {
      if (!k.m[i]) continue;
      k.mf[i] = mf + (size_t)(j++) * k.alloc;
      k_metric_f32<<<grid_for(c, k.alloc, 256), 256, 0, c->stream>>>(k.m[i], const_cast<float*>(k.mf[i]), k.alloc);
      c->launches++;
    }
    OSB_CK(cudaGetLastError());
  }
  {
    // x-sweep row table: the linear index of every row's x = 0 element, rows grouped by the
    // phase of that element within a 32-byte sector (stable), so each warp's rows share it
    const int nrows = k.n[1] * k.n[2];
    std::vector<int> rows(nrows);
    for (int z = 0, r = 0; z < k.n[2]; ++z)
      for (int y = 0; y < k.n[1]; ++y) rows[r++] = k.off0 + y * k.st[1] + z * k.st[2];
    std::stable_sort(rows.begin(), rows.end(), [](int u, int v) { return (u & 7) < (v & 7); });
    cudaError_t e = cudaMalloc(&bl.xrows, sizeof(int) * nrows);
    if (e == cudaSuccess) e = cudaMemcpy(bl.xrows, rows.data(), sizeof(int) * nrows, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      cudaFree(R);
      if (bl.qf_base) cudaFree(bl.qf_base);
      if (bl.qf_alt) cudaFree(bl.qf_alt);
      if (bl.mf_buf) cudaFree(bl.mf_buf);
      if (bl.xrows) cudaFree(bl.xrows);
      return fail(OSB_ECUDA, "x-sweep row table: %s", cudaGetErrorString(e));
    }
  }
  if (d->filter != OSB_FILTER_NONE) {
    // WENO: kappa (zero halos, written on the interior only); TVD: the point -2 velocities;
    // then the 15 filter-flux arrays
    const size_t bytes = (size_t)16 * k.alloc * (c->prec == OSB_PREC_FP32_RESIDUAL ? sizeof(float) : sizeof(double));
    cudaError_t e = cudaMalloc(&bl.filt_ws, bytes);
    if (e != cudaSuccess) {
      cudaFree(R);
      if (bl.qf_base) cudaFree(bl.qf_base);
      if (bl.qf_alt) cudaFree(bl.qf_alt);
      if (bl.mf_buf) cudaFree(bl.mf_buf);
      cudaFree(bl.xrows);
      return fail(OSB_ECUDA, "filter workspace: %s", cudaGetErrorString(e));
    }
    OSB_CK(cudaMemsetAsync(bl.filt_ws, 0, bytes, c->stream));
  }
  if (d->ystretch[0]) {
    // the stretched grid's D11 and SD111 rows, then their FP32 copies
    const int n1 = k.n[1];
    cudaError_t e = cudaMalloc(&bl.ys_buf, (sizeof(double) + sizeof(float)) * 2 * n1);
    double* yd = static_cast<double*>(bl.ys_buf);
    float* yf = reinterpret_cast<float*>(yd + 2 * n1);
    for (int i = 0; i < 2 && e == cudaSuccess; ++i)
      e = cudaMemcpyAsync(yd + i * n1, d->ystretch[i], sizeof(double) * n1, cudaMemcpyDefault, c->stream);
    if (e != cudaSuccess) {
      cudaFree(R);
      if (bl.qf_base) cudaFree(bl.qf_base);
      if (bl.qf_alt) cudaFree(bl.qf_alt);
      if (bl.mf_buf) cudaFree(bl.mf_buf);
      if (bl.filt_ws) cudaFree(bl.filt_ws);
      if (bl.ys_buf) cudaFree(bl.ys_buf);
      cudaFree(bl.xrows);
      return fail(OSB_ECUDA, "stretched-grid rows: %s", cudaGetErrorString(e));
    }
    k_metric_f32<<<grid_for(c, 2 * n1, 256), 256, 0, c->stream>>>(yd, yf, 2 * n1);
    c->launches++;
    OSB_CK(cudaGetLastError());
    k.ys[0] = yd;
    k.ys[1] = yd + n1;
    k.ysf[0] = yf;
    k.ysf[1] = yf + n1;
  }
  if (c->qf_parity) batch_set_parity(c, 0);  // new tables start from the original buffers
  batch_free(c);
  c->blocks.push_back(bl);
  drop_graph(c);
  if (block_id) *block_id = (int)c->blocks.size() - 1;
  return OSB_OK;
}

int osb_set_rk(osb_ctx* c, int kind, int nstages, const double* A, const double* B) {
  if (!c || !A || !B) return fail(OSB_EINVAL, "null argument");
  if (kind != OSB_RK_LOW_STORAGE && kind != OSB_RK_SBLI3) return fail(OSB_EINVAL, "unknown RK kind");
  if (nstages < 1 || nstages > 8) return fail(OSB_EINVAL, "1..8 stages");
  c->rk_kind = kind;
  c->nst = nstages;
  for (int i = 0; i < nstages; ++i) {
    c->A[i] = A[i];
    c->B[i] = B[i];
  }
  drop_graph(c);
  return OSB_OK;
}

int osb_stage(osb_ctx* c, int s, double dt) {
  if (!c) return fail(OSB_EINVAL, "null ctx");
  if (s < 0 || s >= c->nst) return fail(OSB_EINVAL, "stage %d out of range", s);
  OSB_CK(cudaSetDevice(c->device));
  int rc = sync_shadow(c);
  if (rc) return rc;
  rc = stage(c, s, dt);
  if (rc) return rc;
  if (c->prec == OSB_PREC_FP32_RESIDUAL) {
    rc = apply_bc(c, use_batch(c) ? BC_BOTH : BC_Q);  // halos for observers
    if (rc) return rc;
  }
  OSB_CK(cudaGetLastError());
  return OSB_OK;
}

int osb_apply_bc(osb_ctx* c) {
  if (!c) return fail(OSB_EINVAL, "null ctx");
  OSB_CK(cudaSetDevice(c->device));
  int rc = sync_shadow(c);
  if (rc) return rc;
  rc = apply_bc(c);
  if (rc) return rc;
  OSB_CK(cudaGetLastError());
  return OSB_OK;
}

int osb_step(osb_ctx* c, double dt, int nsteps) {
  if (!c) return fail(OSB_EINVAL, "null ctx");
  if (nsteps < 0) return fail(OSB_EINVAL, "nsteps < 0");
  if (c->blocks.empty()) return fail(OSB_EINVAL, "no blocks");
  OSB_CK(cudaSetDevice(c->device));
  if (resident_eligible(c)) {
    // small 1D blocks: every stage of every step in one launch (no graph needed; the kernel
    // derives its FP32 copy of the state itself)
    int rc = resident_step(c, dt, nsteps);
    if (rc) return rc;
    OSB_CK(cudaGetLastError());
    return OSB_OK;
  }
  int src = sync_shadow(c);
  if (src) return src;
  const bool batch = use_batch(c);
  if (batch && !c->batch.ready) {
    int rc = batch_build(c);  // allocates: never inside a capture
    if (rc) return rc;
  }
  if (!c->graphs || c->timing) {
    for (int it = 0; it < nsteps; ++it) {
      int rc = one_step(c, dt);
      if (rc) return rc;
    }
    if (c->prec == OSB_PREC_FP32_RESIDUAL) {
      int rc = apply_bc(c, batch ? BC_BOTH : BC_Q);  // halos for observers
      if (rc) return rc;
    }
    OSB_CK(cudaGetLastError());
    return OSB_OK;
  }
  if (c->prec == OSB_PREC_FP32_RESIDUAL) {
    // one graph per FP32-buffer parity; a step flips the parity when the stage count is odd
    if (c->g_dt != dt) {
      drop_graph(c);
      c->g_dt = dt;
    }
    for (int it = 0; it < nsteps; ++it) {
      const int p = c->qf_parity;
      if (!c->gexec_p[p]) {
        cudaGraph_t g;
        long long before = c->launches;
        OSB_CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        int rc = one_step(c, dt);
        cudaError_t e = cudaStreamEndCapture(c->stream, &g);
        batch_set_parity(c, p);  // nothing ran yet
        if (rc) {
          if (e == cudaSuccess) cudaGraphDestroy(g);
          return rc;
        }
        if (e != cudaSuccess) return fail(OSB_ECUDA, "graph capture: %s", cudaGetErrorString(e));
        c->g_kernels = c->launches - before;
        c->launches = before;
        e = cudaGraphInstantiate(&c->gexec_p[p], g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(OSB_ECUDA, "graph instantiate: %s", cudaGetErrorString(e));
      }
      OSB_CK(cudaGraphLaunch(c->gexec_p[p], c->stream));
      c->launches += c->g_kernels;
      batch_set_parity(c, p ^ (c->nst & 1));
    }
    {
      int rc = apply_bc(c, batch ? BC_BOTH : BC_Q);  // halos of the FP64 (and FP32) state for observers
      if (rc) return rc;
    }
    OSB_CK(cudaGetLastError());
    return OSB_OK;
  }
  if (!c->gexec || c->g_dt != dt) {
    drop_graph(c);
    cudaGraph_t g;
    long long before = c->launches;
    OSB_CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    int rc = one_step(c, dt);
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (rc) {
      if (e == cudaSuccess) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) return fail(OSB_ECUDA, "graph capture: %s", cudaGetErrorString(e));
    c->g_kernels = c->launches - before;
    c->launches = before;
    e = cudaGraphInstantiate(&c->gexec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(OSB_ECUDA, "graph instantiate: %s", cudaGetErrorString(e));
    c->g_dt = dt;
  }
  for (int it = 0; it < nsteps; ++it) {
    OSB_CK(cudaGraphLaunch(c->gexec, c->stream));
    c->launches += c->g_kernels;
  }
  return OSB_OK;
}

int osb_residual(osb_ctx* c, int block, double* const* out) {
  if (!c || !out) return fail(OSB_EINVAL, "null argument");
  if (block < 0 || block >= (int)c->blocks.size()) return fail(OSB_EINVAL, "block %d out of range", block);
  OSB_CK(cudaSetDevice(c->device));
  Block& bl = c->blocks[block];
  int rc = sync_shadow(c);
  if (rc) return rc;
  rc = residual(c, bl);
  if (rc) return rc;
  for (int v = 0; v < bl.d.ndim + 2; ++v) {
    if (!out[v]) return fail(OSB_EINVAL, "null output array %d", v);
    if (c->prec == OSB_PREC_FP32_RESIDUAL) {
      k_ff_to_double<<<grid_for(c, bl.k.alloc, 256), 256, 0, c->stream>>>(bl.k.Rh[v], bl.k.Rl[v], out[v], bl.k.alloc);
      c->launches++;
    } else {
      OSB_CK(cudaMemcpyAsync(out[v], bl.k.R[v], sizeof(double) * bl.k.alloc, cudaMemcpyDeviceToDevice, c->stream));
    }
  }
  OSB_CK(cudaGetLastError());
  return OSB_OK;
}

int osb_reduce(osb_ctx* c, int what, double* host_out) {
  if (!c || !host_out) return fail(OSB_EINVAL, "null argument");
  if (what < OSB_RED_KE || what > OSB_RED_NAN_COUNT) return fail(OSB_EINVAL, "unknown reduction %d", what);
  if (c->blocks.empty()) return fail(OSB_EINVAL, "no blocks");
  OSB_CK(cudaSetDevice(c->device));
  int slot = 0;
  const int threads = 256;
  for (auto& bl : c->blocks) {
    long n = (long)bl.k.n[0] * bl.k.n[1] * bl.k.n[2];
    int grid = std::min(grid_for(c, n, threads), 64);
    if (slot + grid > (c->red_slots + 8) * 64 - 1) return fail(OSB_ENOTSUP, "too many blocks for the reduction");
    RedParams rp{what, bl.d.ndim + 2, bl.d.viscous, bl.d.gama, bl.d.Minf, bl.d.mu_const, bl.d.visc_power};
    k_reduce<<<grid, threads, 0, c->stream>>>(bl.k, rp, c->red, slot);
    c->launches++;
    slot += grid;
  }
  double* dout = c->red + ((size_t)(c->red_slots + 8) * 64 - 1);
  k_reduce_final<<<1, 256, 0, c->stream>>>(c->red, slot, what == OSB_RED_CFL_DT, dout);
  c->launches++;
  OSB_CK(cudaMemcpyAsync(c->red_host, dout, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  OSB_CK(cudaStreamSynchronize(c->stream));
  *host_out = c->red_host[0];
  return OSB_OK;
}

int osb_sync(osb_ctx* c, int timeout_ms) {
  if (!c) return fail(OSB_EINVAL, "null ctx");
  OSB_CK(cudaSetDevice(c->device));
  auto t0 = std::chrono::steady_clock::now();
  for (;;) {
    cudaError_t e = cudaStreamQuery(c->stream);
    if (e == cudaSuccess) break;
    if (e != cudaErrorNotReady) return fail(OSB_ECUDA, "stream: %s", cudaGetErrorString(e));
    auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0).count();
    if (timeout_ms >= 0 && ms > timeout_ms) return fail(OSB_ETIMEDOUT, "stream not idle after %d ms", timeout_ms);
    std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
  unsigned long long bad[2] = {0, 0};
  OSB_CK(cudaMemcpy(bad, c->bad, sizeof bad, cudaMemcpyDeviceToHost));
  if (bad[0] || bad[1]) {
    OSB_CK(cudaMemset(c->bad, 0, sizeof bad));
    if (bad[1])
      return fail(OSB_ECUDA, "%llu thread blocks of the central kernel gave up waiting for their bulk copies", bad[1]);
    return fail(OSB_ENAN, "%llu non-finite values produced by the RK update", bad[0]);
  }
  return OSB_OK;
}

int osb_set_graphs(osb_ctx* c, int enable) {
  if (!c) return fail(OSB_EINVAL, "null ctx");
  c->graphs = enable != 0;
  if (!c->graphs) drop_graph(c);
  return OSB_OK;
}

int osb_set_schedule(osb_ctx* c, const osb_schedule* sched) {
  if (!c || !sched) return fail(OSB_EINVAL, "null argument");
  if (sched->mode < OSB_SCHED_AUTO || sched->mode > OSB_SCHED_PERSISTENT) return fail(OSB_EINVAL, "unknown mode");
  if (sched->tile_y != 8 && sched->tile_y != 16 && sched->tile_y != 32)
    return fail(OSB_EINVAL, "tile_y must be 8, 16 or 32");
  if (sched->ctas_per_sm < 1 || sched->ctas_per_sm > 16) return fail(OSB_EINVAL, "ctas_per_sm must be 1..16");
  if (sched->order < 0 || sched->order > 2) return fail(OSB_EINVAL, "order must be 0, 1 or 2");
  if (sched->fuse_update != 0 && sched->fuse_update != 1) return fail(OSB_EINVAL, "fuse_update must be 0 or 1");
  if (sched->mode == OSB_SCHED_PERSISTENT) {
    std::string why;
    if (!batch_eligible(c, &why)) return fail(OSB_ENOTSUP, "%s", why.c_str());
  }
  OSB_CK(cudaSetDevice(c->device));
  OSB_CK(cudaStreamSynchronize(c->stream));
  c->sched = *sched;
  batch_free(c);
  drop_graph(c);
  return OSB_OK;
}

int osb_get_schedule(osb_ctx* c, int* mode_out, osb_schedule* sched_out) {
  if (!c || !mode_out) return fail(OSB_EINVAL, "null argument");
  *mode_out = use_batch(c) ? OSB_SCHED_PERSISTENT : OSB_SCHED_PER_BLOCK;
  if (sched_out) *sched_out = c->sched;
  return OSB_OK;
}

int osb_set_variant(osb_ctx* c, int variant) {
  if (!c) return fail(OSB_EINVAL, "null ctx");
  c->variant = variant;
  drop_graph(c);
  return OSB_OK;
}

int osb_set_central_staging(osb_ctx* c, int bulk) {
  if (!c) return fail(OSB_EINVAL, "null ctx");
  if (bulk != 0 && bulk != 1) return fail(OSB_EINVAL, "central staging %d (0 register loads, 1 bulk copies)", bulk);
  c->central_bulk = bulk;
  drop_graph(c);
  return OSB_OK;
}

int osb_timing(osb_ctx* c, int enable) {
  if (!c) return fail(OSB_EINVAL, "null ctx");
  OSB_CK(cudaSetDevice(c->device));
  int rc = timing_collect(c);
  if (rc) return rc;
  c->timing = enable != 0;
  return OSB_OK;
}

int osb_timing_report(osb_ctx* c, double* ms, long long* launches, int n) {
  if (!c || !ms || !launches) return fail(OSB_EINVAL, "null argument");
  OSB_CK(cudaSetDevice(c->device));
  int rc = timing_collect(c);
  if (rc) return rc;
  for (int i = 0; i < n && i < FAM_N; ++i) {
    ms[i] = c->fam_ms[i];
    launches[i] = c->fam_count[i];
    c->fam_ms[i] = 0.0;
    c->fam_count[i] = 0;
  }
  return OSB_OK;
}

int osb_launch_count(osb_ctx* c, long long* out) {
  if (!c || !out) return fail(OSB_EINVAL, "null argument");
  *out = c->launches;
  return OSB_OK;
}

int osb_get_stream(osb_ctx* c, void** stream) {
  if (!c || !stream) return fail(OSB_EINVAL, "null argument");
  *stream = (void*)c->stream;
  return OSB_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// One RK stage without any device allocation (osb_stage_noalloc).
//
// For hosts that cannot call cudaMalloc -- a solver embedded in an application that owns all
// device memory through its own pool, or a caller that must not allocate once it is running --
// the FP64 residual workspace of this variant is a fixed file-scope device array instead of a
// per-context cudaMalloc.  Every GPU that loads this library holds the array until the process
// exits.  All calls share it, so calls that overlap on the GPU (several streams, several host
// threads) race on it; serialise them.  The residual part of the array is fully written by the
// first residual kernel of every call; the non-finite counter at its end is cleared by each call.
namespace {

constexpr size_t kNoAllocDoubles = (size_t)OSB_NOALLOC_MAX_DOUBLES;
// residual workspace followed by the non-finite counter (8 bytes, 256-byte aligned slot)
static __device__ __align__(256) double osb_noalloc_scratch[kNoAllocDoubles + 32];

std::mutex g_noalloc_mu;
double* g_noalloc_ptr[64] = {nullptr};

// Device address of the scratch array on the current device: host code must not use the
// symbol itself (it names a host-side stand-in), so look it up once per device.
int noalloc_scratch(int device, double** out) {
  if (device < 0 || device >= 64) return fail(OSB_EINVAL, "device %d out of range", device);
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[device]) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, osb_noalloc_scratch);
    if (e != cudaSuccess) return fail(OSB_ECUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    g_noalloc_ptr[device] = static_cast<double*>(ptr);
  }
  *out = g_noalloc_ptr[device];
  return OSB_OK;
}

}  // namespace

namespace {

// 4th-order central first derivative of f at linear index id along stride s, the operator
// order of the generated metric kernel: ((-2/3 f[-1] - 1/12 f[+2]) + 1/12 f[-2] + 2/3 f[+1]) / Delta,
// rounded operation by operation (no contraction).
__device__ __forceinline__ double metric_d1(const double* __restrict__ f, int id, int s, double inv) {
  double t = __dadd_rn(__dmul_rn(-(2.0 / 3.0), f[id - s]), -__dmul_rn(1.0 / 12.0, f[id + 2 * s]));
  t = __dadd_rn(t, __dmul_rn(1.0 / 12.0, f[id - 2 * s]));
  t = __dadd_rn(t, __dmul_rn(2.0 / 3.0, f[id + s]));
  return __dmul_rn(t, inv);
}

// Metric arrays at every allocated point: the point's metrics are those evaluated at a source
// point -- the point itself on the interior; its periodic image (fill 0) or the nearest point
// where the stencil fits, index -3..N+2 of each direction (fill 1), in the halos.  At the
// source point J_ij = d x_i / d xi_j from central differences of the coordinates;
// met[3 d + i] = d xi_d / d x_i (the inverse of J), met[9] = det J.
__global__ void k_metrics(BlockK b, const double* __restrict__ x0, const double* __restrict__ x1,
                          const double* __restrict__ x2, double* m0, double* m1, double* m2, double* m3, double* m4,
                          double* m5, double* m6, double* m7, double* m8, double* m9, int fill, int halo) {
  const int nd = b.ndim;
  int ext[3];
  for (int e = 0; e < 3; ++e) ext[e] = e < nd ? b.n[e] + 2 * halo : 1;
  const long total = (long)ext[0] * ext[1] * ext[2];
  const double* x[3] = {x0, x1, x2};
  double* m[10] = {m0, m1, m2, m3, m4, m5, m6, m7, m8, m9};
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    int c[3] = {(int)(t % ext[0]), (int)((t / ext[0]) % ext[1]), (int)(t / ((long)ext[0] * ext[1]))};
    int src[3] = {0, 0, 0};
    for (int e = 0; e < nd; ++e) {
      c[e] -= halo;
      const int n = b.n[e];
      src[e] = fill == OSB_METRIC_PERIODIC ? ((c[e] % n) + n) % n : min(max(c[e], -3), n + 2);
    }
    const int dst = lin(b, c[0], c[1], c[2]);
    const int id = lin(b, src[0], src[1], src[2]);
    double J[3][3];
    for (int i = 0; i < nd; ++i)
      for (int j = 0; j < nd; ++j) J[i][j] = metric_d1(x[i], id, b.st[j], b.invd[j]);
    if (nd == 2) {
      const double det = __dadd_rn(__dmul_rn(J[0][0], J[1][1]), -__dmul_rn(J[0][1], J[1][0]));
      m[0][dst] = __ddiv_rn(J[1][1], det);
      m[1][dst] = __ddiv_rn(-J[0][1], det);
      m[3][dst] = __ddiv_rn(-J[1][0], det);
      m[4][dst] = __ddiv_rn(J[0][0], det);
      m[9][dst] = det;
    } else {
      // cofactors: inv[d][i] = C[i][d] / det
      double C[3][3];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
          C[i][j] = J[i1][j1] * J[i2][j2] - J[i1][j2] * J[i2][j1];
        }
      const double det = J[0][0] * C[0][0] + J[0][1] * C[0][1] + J[0][2] * C[0][2];
      for (int d = 0; d < 3; ++d)
        for (int i = 0; i < 3; ++i) m[3 * d + i][dst] = C[i][d] / det;
      m[9][dst] = det;
    }
  }
}

}  // namespace

extern "C" int osb_metrics(const osb_block_desc* d, const double* const* x, double* const* met, int fill,
                           void* stream) {
  if (!d || !x || !met) return fail(OSB_EINVAL, "null argument");
  if (d->ndim != 2 && d->ndim != 3) return fail(OSB_EINVAL, "metrics are defined for 2D and 3D blocks");
  if (fill != OSB_METRIC_PERIODIC && fill != OSB_METRIC_EDGE) return fail(OSB_EINVAL, "unknown metric fill %d", fill);
  if (d->halo < 5) return fail(OSB_EINVAL, "halo %d < 5", d->halo);
  for (int i = 0; i < d->ndim; ++i) {
    if (!x[i]) return fail(OSB_EINVAL, "coordinate array %d is null", i);
    if (d->size[i] < (fill == OSB_METRIC_PERIODIC ? d->halo : 1))
      return fail(OSB_EINVAL, "direction %d has %d points, fewer than the periodic halo", i, d->size[i]);
    if (!(d->delta[i] > 0.0)) return fail(OSB_EINVAL, "delta[%d] must be > 0", i);
  }
  static const int used2[] = {0, 1, 3, 4, 9};
  if (d->ndim == 2) {
    for (int k : used2)
      if (!met[k]) return fail(OSB_EINVAL, "metric array %d is null", k);
  } else {
    for (int k = 0; k < 10; ++k)
      if (!met[k]) return fail(OSB_EINVAL, "metric array %d is null", k);
  }
  BlockK k;
  memset(&k, 0, sizeof k);
  k.ndim = d->ndim;
  long ext[3];
  for (int i = 0; i < 3; ++i) {
    k.n[i] = i < d->ndim ? d->size[i] : 1;
    ext[i] = i < d->ndim ? d->size[i] + 2 * d->halo : 1;
    k.invd[i] = i < d->ndim ? 1.0 / d->delta[i] : 0.0;
    k.invdf[i] = (float)k.invd[i];
  }
  if (ext[0] * ext[1] * ext[2] >= (1L << 31)) return fail(OSB_EINVAL, "block too large for 32-bit indexing");
  k.st[0] = 1;
  k.st[1] = (int)ext[0];
  k.st[2] = (int)(ext[0] * ext[1]);
  k.alloc = ext[0] * ext[1] * ext[2];
  k.off0 = d->halo + d->halo * k.st[1] + (d->ndim > 2 ? d->halo * k.st[2] : 0);
  int device = 0, sms = 152;
  OSB_CK(cudaGetDevice(&device));
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms <= 0) sms = 152;
  const long blocks = std::min<long>((k.alloc + 255) / 256, (long)sms * 16);
  double* m[10];
  for (int i = 0; i < 10; ++i) m[i] = met[i];
  double* dummy = met[9];  // unused 2D slots are never written
  for (int i = 0; i < 10; ++i)
    if (!m[i]) m[i] = dummy;
  k_metrics<<<(unsigned)blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      k, x[0], x[1], d->ndim > 2 ? x[2] : x[0], m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], m[8], m[9], fill,
      d->halo);
  OSB_CK(cudaGetLastError());
  return OSB_OK;
}

extern "C" int osb_stage_noalloc(const osb_block_desc* d, int rk_kind, double A, double B, double dt,
                                 void* stream) {
  if (!d) return fail(OSB_EINVAL, "null descriptor");
  std::string why;
  if (!check_desc(d, why)) return fail(OSB_EINVAL, "invalid block descriptor: %s", why.c_str());
  if (rk_kind != OSB_RK_LOW_STORAGE && rk_kind != OSB_RK_SBLI3) return fail(OSB_EINVAL, "unknown RK kind");
  for (int i = 0; i < 10; ++i)
    if (d->metric[i]) return fail(OSB_ENOTSUP, "osb_stage_noalloc takes Cartesian blocks only");
  if (d->filter != OSB_FILTER_NONE)
    return fail(OSB_ENOTSUP, "the non-linear filter follows a whole RK step (osb_step), not one stage");
  if (!block_faces_ok(*d, why)) return fail(OSB_ENOTSUP, "osb_stage_noalloc: %s", why.c_str());
  const int nv = d->ndim + 2;
  size_t alloc = 1;
  for (int i = 0; i < d->ndim; ++i) alloc *= (size_t)(d->size[i] + 2 * d->halo);
  if ((size_t)nv * alloc > kNoAllocDoubles)
    return fail(OSB_EINVAL,
                "block needs %zu doubles of residual workspace; the static workspace of osb_stage_noalloc "
                "holds %zu (OSB_NOALLOC_MAX_DOUBLES)", (size_t)nv * alloc, kNoAllocDoubles);
  int device = 0;
  OSB_CK(cudaGetDevice(&device));
  // the stream and every array must belong to the current device, whose workspace is used
  if (stream) {
    int sdev = -1;
    OSB_CK(cudaStreamGetDevice(static_cast<cudaStream_t>(stream), &sdev));
    if (sdev != device) return fail(OSB_EINVAL, "stream belongs to device %d, the current device is %d", sdev, device);
  }
  for (int v = 0; v < nv; ++v)
    for (const void* ptr : {(const void*)d->q[v], (const void*)d->rkold[v]}) {
      cudaPointerAttributes at;
      OSB_CK(cudaPointerGetAttributes(&at, ptr));
      if (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)
        return fail(OSB_EINVAL, "state / RK array of variable %d is not device memory", v);
      if (at.type == cudaMemoryTypeDevice && at.device != device)
        return fail(OSB_EINVAL, "state / RK array of variable %d lives on device %d, the current device is %d", v,
                    at.device, device);
    }
  for (int w = 0; w < 2; ++w) {
    if (!d->ystretch[w]) continue;
    cudaPointerAttributes at;
    OSB_CK(cudaPointerGetAttributes(&at, d->ystretch[w]));
    if ((at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged) ||
        (at.type == cudaMemoryTypeDevice && at.device != device))
      return fail(OSB_EINVAL, "stretched-grid rows %d are not device memory of the current device", w);
  }
  double* scratch = nullptr;
  int rc = noalloc_scratch(device, &scratch);
  if (rc) return rc;
  // a context on the stack: no streams, graphs or workspaces are created
  osb_ctx c;
  c.device = device;
  c.prec = OSB_PREC_FP64;
  c.stream = static_cast<cudaStream_t>(stream);
  c.graphs = false;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) == cudaSuccess && sms > 0)
    c.sm_count = sms;
  c.bad = reinterpret_cast<unsigned long long*>(scratch + kNoAllocDoubles);
  Block bl;
  bl.d = *d;
  BlockK& k = bl.k;
  memset(&k, 0, sizeof k);
  k.ndim = d->ndim;
  long ext[3];
  for (int i = 0; i < 3; ++i) {
    k.n[i] = i < d->ndim ? d->size[i] : 1;
    ext[i] = i < d->ndim ? d->size[i] + 2 * d->halo : 1;
    k.invd[i] = i < d->ndim ? 1.0 / d->delta[i] : 0.0;
    k.invdf[i] = (float)k.invd[i];
    k.inv2d[i] = i < d->ndim ? 1.0 / (d->delta[i] * d->delta[i]) : 0.0;
  }
  k.st[0] = 1;
  k.st[1] = (int)ext[0];
  k.st[2] = (int)(ext[0] * ext[1]);
  k.alloc = ext[0] * ext[1] * ext[2];
  k.off0 = d->halo + (d->ndim > 1 ? d->halo * k.st[1] : 0) + (d->ndim > 2 ? d->halo * k.st[2] : 0);
  for (int v = 0; v < nv; ++v) {
    k.q[v] = d->q[v];
    k.rk[v] = d->rkold[v];
    k.R[v] = scratch + (size_t)v * k.alloc;
  }
  k.ys[0] = d->ystretch[0];  // FP64 path: the caller's rows directly
  k.ys[1] = d->ystretch[1];
  OSB_CK(cudaMemsetAsync(c.bad, 0, sizeof(unsigned long long), c.stream));
  rc = residual(&c, bl);
  if (rc) return rc;
  long n = (long)k.n[0] * k.n[1] * k.n[2];
  k_rk<<<grid_for(&c, n, 256), 256, 0, c.stream>>>(k, nv, rk_kind == OSB_RK_LOW_STORAGE ? 0 : 1, A, B, dt, c.bad);
  // the block's boundary faces, with the kernels osb_apply_bc launches for them
  rc = apply_block_bc(&c, bl, 0, BC_BOTH);
  if (rc) return rc;
  OSB_CK(cudaGetLastError());
  return OSB_OK;
}
