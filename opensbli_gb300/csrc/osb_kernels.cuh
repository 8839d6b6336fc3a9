// osb_kernels.cuh -- CUDA kernels of one RK stage (sm_103a).
//
//   k_flux_x      characteristic flux sweep along x: a warp stages 32 rows x 32 points of the
//                 state in shared memory (coalesced), then each lane sweeps one row
//   k_flux_sweep  characteristic flux sweep along y or z: one thread per line segment,
//                 coalesced along x, 6-point register window, one interface per step
//   k_central3d   central 4th-order terms on a shared-memory tile: skew-symmetric convective
//                 terms and/or viscous stress + heat flux
//   k_rk          low-storage / SBLI RK update, counts non-finite values
//   k_periodic / k_zero_grad / k_interface   boundary conditions
//   k_reduce_*    FP64 diagnostics
#pragma once
#include "osb_math.cuh"

namespace osb {

struct BlockK {
  int n[3];        // interior points per direction (1 for unused directions)
  int ndim;
  int st[3];       // linear strides of the OPS-layout arrays (32-bit: 64-bit integer multiplies
  int off0;        // would compete for the FP64 pipe); linear index of point (0,0,0)
  long alloc;      // allocated points per array (< 2^31, checked at osb_block_add)
  double* q[5];
  double* rk[5];
  double* R[5];    // FP64 residual (FP64 path)
  float* qf[5];    // FP32 shadow of q (FP32-residual path; null otherwise)
  float* Rh[5];    // FP32-residual path: residual as a float-float pair (hi + lo) ...
  float* Rl[5];    // ... stored in the same bytes as the FP64 residual
  const double* m[10];  // curvilinear metrics (D_di at 3*d+i, det J at 9); null: Cartesian
  const float* mf[10];  // FP32 copies of the metrics (FP32-residual path)
  const double* ys[2];  // stretched y grid: D11 and SD111 of the interior rows j; null: uniform
  const float* ysf[2];  // their FP32 copies (FP32-residual path)
  double invd[3];  // 1/Delta
  double inv2d[3]; // 1/Delta^2
  float invdf[3];  // 1/Delta rounded to FP32 on the host (no conversion in FP32 kernels)
};

// Stretched y grid: D11 (w = 0) or SD111 (w = 1) of interior row j in the kernel's type.
template <typename T>
__device__ __forceinline__ T ystr(const BlockK& b, int w, int j);
template <>
__device__ __forceinline__ double ystr<double>(const BlockK& b, int w, int j) { return b.ys[w][j]; }
template <>
__device__ __forceinline__ float ystr<float>(const BlockK& b, int w, int j) { return b.ysf[w][j]; }

// 1/Delta_d in the arithmetic type of a kernel.
template <typename T>
__device__ __forceinline__ T inv_delta(const BlockK& b, int d);
template <>
__device__ __forceinline__ double inv_delta<double>(const BlockK& b, int d) { return b.invd[d]; }
template <>
__device__ __forceinline__ float inv_delta<float>(const BlockK& b, int d) { return b.invdf[d]; }

// ---- FP32-path helpers: no FP64 arithmetic (the FP64 pipe is 1/64 of FP32 on GB300) ----

// Exact float -> double with integer operations (zero and FTZ-flushed denormals map to zero).
__device__ __forceinline__ double f2d_exact(float f) {
  unsigned b = __float_as_uint(f);
  unsigned sign = b & 0x80000000u;
  unsigned e = (b >> 23) & 0xffu;
  unsigned m = b & 0x7fffffu;
  unsigned hi, lo;
  if (e == 0u) {
    hi = sign;
    lo = 0u;
  } else if (e == 255u) {
    hi = sign | 0x7ff00000u | (m >> 3) | (m ? 0x80000u : 0u);
    lo = 0u;
  } else {
    hi = sign | ((e + 896u) << 20) | (m >> 3);
    lo = m << 29;
  }
  return __hiloint2double((int)hi, (int)lo);
}

// double -> float rounded to nearest even with integer operations; results below the FP32
// normal range flush to signed zero (the FP32 path runs flush-to-zero anyway).
__device__ __forceinline__ float d2f_rn(double x) {
  unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  unsigned sign = hi & 0x80000000u;
  int e = (int)((hi >> 20) & 0x7ffu);
  if (e == 0x7ff) return __uint_as_float(sign | 0x7f800000u | ((((hi & 0xfffffu) | lo) != 0u) ? 0x400000u : 0u));
  int fe = e - 896;
  unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);
  unsigned rest = lo & 0x1fffffffu;
  if (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) {
    m += 1u;
    if (m == 0x800000u) {
      m = 0u;
      fe += 1;
    }
  }
  if (fe <= 0) return __uint_as_float(sign);
  if (fe >= 255) return __uint_as_float(sign | 0x7f800000u);
  return __uint_as_float(sign | ((unsigned)fe << 23) | m);
}

// (hi, lo) += a (TwoSum, Knuth), non-contracted operations.
__device__ __forceinline__ void ff_add(float& hi, float& lo, float a, float alo) {
  float S = __fadd_rn(hi, a);
  float w = __fsub_rn(S, hi);
  float E = __fadd_rn(__fsub_rn(hi, __fsub_rn(S, w)), __fsub_rn(a, w));
  E = __fadd_rn(E, __fadd_rn(lo, alo));
  hi = __fadd_rn(S, E);
  lo = __fsub_rn(E, __fsub_rn(hi, S));
}

// -(fnew - fold) * invd as a float-float pair: the difference is exact (TwoSum), the product
// carries its rounding error (FMA).
__device__ __forceinline__ void ff_flux_diff(float fnew, float fold, float invd, float& p, float& pe) {
  float s = __fsub_rn(fnew, fold);
  float v = __fsub_rn(s, fnew);
  float e = __fadd_rn(__fsub_rn(fnew, __fsub_rn(s, v)), __fsub_rn(-fold, v));
  p = __fmul_rn(-s, invd);
  pe = __fadd_rn(__fmaf_rn(-s, invd, -p), __fmul_rn(-e, invd));
}

template <typename T>
__device__ __forceinline__ T ld_q(const BlockK& b, int v, int id);
template <>
__device__ __forceinline__ double ld_q<double>(const BlockK& b, int v, int id) { return __ldg(b.q[v] + id); }
template <>
__device__ __forceinline__ float ld_q<float>(const BlockK& b, int v, int id) { return __ldg(b.qf[v] + id); }

// Local-frame variable order of a sweep along direction D: global index of local variable lv.
template <int ND, int D>
__device__ __forceinline__ int gvar_fwd(int lv) {
  if (lv == 0) return 0;
  if (lv == ND + 1) return ND + 1;
  int t = lv - 1;  // 0 = normal, 1.. = tangential
  if (ND == 3) return 1 + (D + t) % 3;
  if (ND == 2) return 1 + (t == 0 ? D : 1 - D);
  return 1;
}

template <typename T>
__device__ __forceinline__ T ld_m(const BlockK& b, int c, int id);
template <>
__device__ __forceinline__ double ld_m<double>(const BlockK& b, int c, int id) { return __ldg(b.m[c] + id); }
template <>
__device__ __forceinline__ float ld_m<float>(const BlockK& b, int c, int id) { return __ldg(b.mf[c] + id); }

// Fields a sweep along D reads per point: the conserved variables, plus (curvilinear) the
// metric row D_D0..D_D(ND-1) and det J.  gfield maps a field to its local-frame variable
// (Cartesian sweeps) or to a metric component.
template <int ND, bool CURV>
struct SweepFields {
  static constexpr int NV = ND + 2;
  static constexpr int N = CURV ? NV + ND + 1 : NV;
};
template <typename T, int ND, int D, bool CURV>
__device__ __forceinline__ T ld_field(const BlockK& b, int f, int id) {
  constexpr int NV = ND + 2;
  if (!CURV) return ld_q<T>(b, gvar_fwd<ND, D>(f), id);
  if (f < NV) return ld_q<T>(b, f, id);
  if (f < NV + ND) return ld_m<T>(b, 3 * D + (f - NV), id);
  return ld_m<T>(b, 9, id);
}
// Source array of field f (see ld_field).
template <typename T>
__device__ __forceinline__ const T* qptr(const BlockK& b, int v);
template <>
__device__ __forceinline__ const double* qptr<double>(const BlockK& b, int v) { return b.q[v]; }
template <>
__device__ __forceinline__ const float* qptr<float>(const BlockK& b, int v) { return b.qf[v]; }
template <typename T>
__device__ __forceinline__ const T* mptr(const BlockK& b, int c);
template <>
__device__ __forceinline__ const double* mptr<double>(const BlockK& b, int c) { return b.m[c]; }
template <>
__device__ __forceinline__ const float* mptr<float>(const BlockK& b, int c) { return b.mf[c]; }
template <typename T, int ND, int D, bool CURV>
__device__ __forceinline__ const T* field_ptr(const BlockK& b, int f) {
  constexpr int NV = ND + 2;
  if (!CURV) return qptr<T>(b, gvar_fwd<ND, D>(f));
  if (f < NV) return qptr<T>(b, f);
  if (f < NV + ND) return mptr<T>(b, 3 * D + (f - NV));
  return mptr<T>(b, 9);
}

// Asynchronous global -> shared copy of one element (cp.async, sm_80+): many copies stay in
// flight at once instead of one load latency per staged row.
template <typename T>
__device__ __forceinline__ void cp_async_el(T* dst_smem, const T* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
  if (sizeof(T) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

template <typename T, int ND>
__device__ __forceinline__ void set_field(Pt<T, ND>& s, int f, T v) { s.q[f] = v; }
template <typename T, int ND>
__device__ __forceinline__ void set_field(PtC<T, ND>& s, int f, T v) {
  constexpr int NV = ND + 2;
  if (f < NV) s.q[f] = v;
  else if (f < NV + ND) s.k[f - NV] = v;
  else s.J = v;
}
template <typename T, int ND, bool CURV>
struct SweepPt { using type = Pt<T, ND>; };
template <typename T, int ND>
struct SweepPt<T, ND, true> { using type = PtC<T, ND>; };

// Residual update of one variable at linear index id with -(fnew - fold)*invd.
__device__ __forceinline__ void acc_flux(const BlockK& b, int v, int id, double fnew, double fold, double invd,
                                         int first) {
  double d = -(fnew - fold) * invd;
  b.R[v][id] = first ? d : b.R[v][id] + d;
}
__device__ __forceinline__ void acc_flux(const BlockK& b, int v, int id, float fnew, float fold, float invd,
                                         int first) {
  float p, pe;
  ff_flux_diff(fnew, fold, invd, p, pe);
  if (first) {
    float h = __fadd_rn(p, pe);
    b.Rh[v][id] = h;
    b.Rl[v][id] = __fsub_rn(pe, __fsub_rn(h, p));
  } else {
    float h = b.Rh[v][id], l = b.Rl[v][id];
    ff_add(h, l, p, pe);
    b.Rh[v][id] = h;
    b.Rl[v][id] = l;
  }
}
// Split form of acc_flux for sweeps that prefetch the residual they update: r_load reads the
// current value early (its latency hidden behind the flux computation), r_store adds the flux
// difference and writes it back.
__device__ __forceinline__ void r_load(const BlockK& b, int v, int id, double& h, double& l) {
  h = b.R[v][id];
  l = 0.0;
}
__device__ __forceinline__ void r_load(const BlockK& b, int v, int id, float& h, float& l) {
  h = b.Rh[v][id];
  l = b.Rl[v][id];
}
__device__ __forceinline__ void r_store(const BlockK& b, int v, int id, double fnew, double fold, double invd,
                                        double h, double) {
  b.R[v][id] = h + -(fnew - fold) * invd;
}
__device__ __forceinline__ void r_store(const BlockK& b, int v, int id, float fnew, float fold, float invd,
                                        float h, float l) {
  float p, pe;
  ff_flux_diff(fnew, fold, invd, p, pe);
  ff_add(h, l, p, pe);
  b.Rh[v][id] = h;
  b.Rl[v][id] = l;
}

__device__ __forceinline__ void rp_store(const BlockK& b, int v, int id, double c, double h, double) {
  b.R[v][id] = h + c;
}
__device__ __forceinline__ void rp_store(const BlockK& b, int v, int id, float c, float h, float l) {
  ff_add(h, l, c, 0.f);
  b.Rh[v][id] = h;
  b.Rl[v][id] = l;
}

// Fused RK epilogue of the last residual kernel of a stage (FP32-residual path).  There the
// residual of a point is complete, so the kernel applies the FP64 RK update (rk_LS.py:204-215,
// rk_sbli.py:138-145) itself and writes the next stage's FP32 state into the other buffer of a
// ping-pong pair: the kernel reads the current buffer, so no thread sees a partial update.
struct RkFuse {
  int kind;    // 0 low-storage, 1 SBLI
  int a_zero;  // low-storage stage with A = 0 (the first): the register is not read
  double A, B, dt;
  float dt_h, dt_l;  // dt as a float-float pair
  float* qout[5];
  unsigned long long* bad;
  unsigned long long* stall;  // bulk-staging waits that ran out (k_central3d BULK)
};

// The increment dt * R of the FP32-residual path's RK update, from the float-float residual
// (h, l) and dt as a float-float pair: the cross terms h dt_l + l dt_h (relative size 2^-24,
// formed to ~2^-48) are added to h dt_h by one FMA, so the result is dt (h + l) rounded once
// to FP32, |error| <= 2^-24 |dt R| (plus ~2^-47), then widened exactly with integer operations.
// The single rounding is below the residual's own FP32 error: each flux difference in R
// carries ~2^-24 of the flux, and |R| is at most the flux differences it sums.  An FP64
// addition of the pair's two parts would cost more than the two FMAs of the update itself
// on GB300's FP64 pipe.
__device__ __forceinline__ double dt_residual(float h, float l, float dt_h, float dt_l) {
  return f2d_exact(__fmaf_rn(h, dt_h, __fmaf_rn(h, dt_l, __fmul_rn(l, dt_h))));
}

// RK update of one variable from the float-float residual (h, l) with x = dt_residual: two
// FP64 FMAs, the register and the state (rk_LS.py:204-215; rk_sbli.py:138-145).
__device__ __forceinline__ unsigned rk_point_ff(const BlockK& b, const RkFuse& rf, int v, int id, float h, float l,
                                                double q, double o) {
  const double x = dt_residual(h, l, rf.dt_h, rf.dt_l);
  if (rf.kind == 0) {
    o = rf.a_zero ? x : __fma_rn(rf.A, o, x);
    q = __fma_rn(rf.B, o, q);
  } else {
    q = __fma_rn(rf.A, x, o);
    o = __fma_rn(rf.B, x, o);
  }
  b.rk[v][id] = o;
  b.q[v][id] = q;
  rf.qout[v][id] = d2f_rn(q);
  return ((((unsigned)__double2hiint(q) >> 20) & 0x7ffu) == 0x7ffu) ? 1u : 0u;
}
// The first low-storage stage (A = 0): the register becomes x, one FP64 FMA.  Callers take
// this path under a uniform branch; the select in rk_point_ff gives the same values.
__device__ __forceinline__ unsigned rk_point_a0(const BlockK& b, const RkFuse& rf, int v, int id, float h, float l,
                                                double q) {
  const double x = dt_residual(h, l, rf.dt_h, rf.dt_l);
  q = __fma_rn(rf.B, x, q);
  b.rk[v][id] = x;
  b.q[v][id] = q;
  rf.qout[v][id] = d2f_rn(q);
  return ((((unsigned)__double2hiint(q) >> 20) & 0x7ffu) == 0x7ffu) ? 1u : 0u;
}
__device__ __forceinline__ unsigned rk_point(const BlockK& b, const RkFuse& rf, int v, int id, float h, float l) {
  return rk_point_ff(b, rf, v, id, h, l, b.q[v][id], rf.a_zero ? 0.0 : b.rk[v][id]);
}

// Final residual of a point (float-float) from its prefetched partial value plus the last
// flux difference / pointwise contribution.
__device__ __forceinline__ void r_final(float fnew, float fold, float invd, float& h, float& l) {
  float p, pe;
  ff_flux_diff(fnew, fold, invd, p, pe);
  ff_add(h, l, p, pe);
}
__device__ __forceinline__ void rp_final(float c, float& h, float& l) { ff_add(h, l, c, 0.f); }

// Residual update with a pointwise contribution c.
__device__ __forceinline__ void acc_point(const BlockK& b, int v, int id, double c, int first) {
  b.R[v][id] = first ? c : b.R[v][id] + c;
}
__device__ __forceinline__ void acc_point(const BlockK& b, int v, int id, float c, int first) {
  if (first) {
    b.Rh[v][id] = c;
    b.Rl[v][id] = 0.f;
  } else {
    float h = b.Rh[v][id], l = b.Rl[v][id];
    ff_add(h, l, c, 0.f);
    b.Rh[v][id] = h;
    b.Rl[v][id] = l;
  }
}

__device__ __forceinline__ int lin(const BlockK& b, int i, int j, int k) {
  return b.off0 + i * b.st[0] + j * b.st[1] + k * b.st[2];
}

// Global variable of local variable lv of a sweep along D (identity for curvilinear sweeps).
template <int ND, int D, bool CURV>
__device__ __forceinline__ int gvar(int lv) {
  return CURV ? lv : gvar_fwd<ND, D>(lv);
}

// ---------------------------------------------------------------------------------------
// Sweep along y (D=1) or z (D=2): thread = (x, transverse, segment).
// The fields of point j+3 and the residual of point j that iteration j needs are copied with
// cp.async into a per-thread ring of shared-memory slots one iteration ahead, so their latency
// overlaps a whole interface's arithmetic without holding registers (the register file is the
// occupancy limit of these kernels).  A slot is refilled two iterations after it was read.
constexpr int SWEEP_THREADS = 128, SWEEP_RING = 3;
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_prev() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

template <typename T, int ND, int D, int SCH, int AVG, bool CURV, bool FUSE, int FLX = 0>
__global__ void __launch_bounds__(SWEEP_THREADS, sizeof(T) == 4 ? 4 : 1)
    k_flux_sweep(BlockK b, SchemeParams spd, int seg, int nseg, int first, RkFuse rf) {
  constexpr int NV = ND + 2;
  constexpr int NF = SweepFields<ND, CURV>::N;
  constexpr int NR = sizeof(T) == 4 ? 2 * NV : NV;  // residual words of a point: float-float pairs or doubles
  constexpr int NS = NF + NR;
  using P = typename SweepPt<T, ND, CURV>::type;
  __shared__ T ring[SWEEP_RING][NS][SWEEP_THREADS];
  const SP<T> sp(spd);
  const int tid = threadIdx.x;
  const int x = blockIdx.x * blockDim.x + tid;
  const int other = blockIdx.y / nseg, sidx = blockIdx.y % nseg;
  if (x >= b.n[0]) return;
  int c1 = 0, c2 = 0;
  if (ND == 3) {
    if (D == 1) c2 = other + blockIdx.z * 65535; else c1 = other + blockIdx.z * 65535;
    if (D == 1 && c2 >= b.n[2]) return;
    if (D == 2 && c1 >= b.n[1]) return;
  }
  const int s = b.st[D];
  const int base = lin(b, x, c1, c2);
  const int N = b.n[D];
  const int j0 = sidx * seg;
  const int j1 = min(N, j0 + seg);
  if (j0 >= j1) return;
  const T gm = sp.gama;
  const T invd = inv_delta<T>(b, D);
  const bool rd = !first;
  // iteration it (interface j = j0 - 1 + it) reads the fields of point j + 3 and, for j >= j0,
  // the residual of point j (both inside the 5-point halo / the interior)
  auto issue = [&](int it, int slot) {
    const int j = j0 - 1 + it;
    const int idf = base + (j + 3) * s;
#pragma unroll
    for (int f = 0; f < NF; ++f) cp_async_el(&ring[slot][f][tid], field_ptr<T, ND, D, CURV>(b, f) + idf);
    if (rd && j >= j0) {
      const int idr = base + j * s;
#pragma unroll
      for (int lv = 0; lv < NV; ++lv) {
        const int v = gvar<ND, D, CURV>(lv);
        if constexpr (sizeof(T) == 4) {
          cp_async_el(&ring[slot][NF + 2 * lv][tid], b.Rh[v] + idr);
          cp_async_el(&ring[slot][NF + 2 * lv + 1][tid], b.Rl[v] + idr);
        } else {
          cp_async_el(&ring[slot][NF + lv][tid], b.R[v] + idr);
        }
      }
    }
    cp_async_commit();
  };
  issue(0, 0);
  P w[6];
#pragma unroll
  for (int m = 1; m < 6; ++m) {
    int id = base + (j0 - 4 + m) * s;
#pragma unroll
    for (int f = 0; f < NF; ++f) set_field(w[m], f, ld_field<T, ND, D, CURV>(b, f, id));
    make_pt<T, ND>(w[m], gm);
  }
  T fprev[NV];
#pragma unroll
  for (int lv = 0; lv < NV; ++lv) fprev[lv] = L_(0.0);
  unsigned nbad = 0;
  const int nit = j1 - j0 + 1;
  int cur = 0;
  for (int it = 0; it < nit; ++it) {
    const int j = j0 - 1 + it;
    const int nxt = cur == SWEEP_RING - 1 ? 0 : cur + 1;
    if (it + 1 < nit) issue(it + 1, nxt); else cp_async_commit();
    cp_async_wait_prev();  // the group of iteration it has landed
#pragma unroll
    for (int m = 0; m < 5; ++m) w[m] = w[m + 1];
#pragma unroll
    for (int f = 0; f < NF; ++f) set_field(w[5], f, ring[cur][f][tid]);
    make_pt<T, ND>(w[5], gm);
    const int id = base + j * s;
    T oh[NV], ol[NV];
    if (rd && j >= j0) {
#pragma unroll
      for (int lv = 0; lv < NV; ++lv) {
        if constexpr (sizeof(T) == 4) {
          oh[lv] = ring[cur][NF + 2 * lv][tid];
          ol[lv] = ring[cur][NF + 2 * lv + 1][tid];
        } else {
          oh[lv] = ring[cur][NF + lv][tid];
          ol[lv] = L_(0.0);
        }
      }
    }
    T fh[NV];
    T sc = invd;
    if constexpr (CURV) {
      char_flux_curv<T, ND, SCH, AVG>(w, sp, fh);
      sc = invd / w[2].J;
    } else {
      cart_flux<T, ND, SCH, AVG, FLX>(w, sp, fh);
    }
    if (j >= j0) {
      // stretched y grid: -(F_j+1/2 - F_j-1/2) / Delta_1 * D11_j (the generated residual's order)
      if constexpr (D == 1 && !CURV)
        if (b.ys[0]) sc = invd * ystr<T>(b, 0, j);
      if constexpr (FUSE) {
#pragma unroll
        for (int lv = 0; lv < NV; ++lv) {
          r_final(fh[lv], fprev[lv], sc, oh[lv], ol[lv]);
          nbad += rk_point(b, rf, gvar<ND, D, CURV>(lv), id, oh[lv], ol[lv]);
        }
      } else if (first) {
#pragma unroll
        for (int lv = 0; lv < NV; ++lv) acc_flux(b, gvar<ND, D, CURV>(lv), id, fh[lv], fprev[lv], sc, 1);
      } else {
#pragma unroll
        for (int lv = 0; lv < NV; ++lv) r_store(b, gvar<ND, D, CURV>(lv), id, fh[lv], fprev[lv], sc, oh[lv], ol[lv]);
      }
    }
#pragma unroll
    for (int lv = 0; lv < NV; ++lv) fprev[lv] = fh[lv];
    cur = nxt;
  }
  if (FUSE && nbad) atomicAdd(rf.bad, (unsigned long long)nbad);
}

// ---------------------------------------------------------------------------------------
// Sweep along x.  A warp owns 32 rows (fixed y, z; lane = row) and a segment [s0, s1) of x.
// Input: the state of its rows streams through a ring of XRING chunks of XCH columns in shared
// memory; the warp copies chunk k+1 with cp.async (one instruction moves XCH consecutive
// columns of 32 / XCH rows) while its lanes sweep chunk k with a 6-point register window.
// Output: each lane puts the flux of its interfaces into a tile of XOUT columns plus a carry
// column (the interface left of the tile); every XOUT points the warp forms the residual
// differences and stores them row by row in whole 32-byte sectors.  Stores straight from the
// sweep (lane = row) would leave every sector partially written for many iterations and send
// read-modify-write traffic to DRAM.  Segments can be long: each costs one extra interface and
// one window start; the length is chosen on the host (whole waves of resident CTAs) or fixed by
// osb_set_variant.  Row pitches are odd, so the 32 lanes (rows) of a warp hit distinct banks.
constexpr int XCH = 4, XRING = 2, XCOLS = XCH * XRING, XPITCH = XCOLS + 1, XOUT = 8, XOPITCH = XOUT + 1;
constexpr int XWARPS = 2;

template <typename T, int NF, int NO>
struct XTile {
  T in[NF][32][XPITCH];
  T out[NO][32][XOPITCH];  // column 0: carry, 1..XOUT: fluxes at the right faces of the tile's points
  int rowbase[32];
};

template <typename T, int ND, int SCH, int AVG, bool CURV, int FLX = 0>
__global__ void __launch_bounds__(32 * XWARPS) k_flux_x(BlockK b, SchemeParams spd, int first, int xseg,
                                                         const int* __restrict__ xrows) {
  constexpr int NV = ND + 2;
  constexpr int NF = SweepFields<ND, CURV>::N;
  constexpr int NO = CURV ? NV + 1 : NV;  // curvilinear: the point's 1 / (dx J) rides along
  constexpr int RPI = 32 / XCH;           // rows per copy instruction
  constexpr int OPI = 32 / XOUT;          // rows per store instruction
  using P = typename SweepPt<T, ND, CURV>::type;
  const SP<T> sp(spd);
  extern __shared__ __align__(16) unsigned char osb_smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  XTile<T, NF, NO>& t = reinterpret_cast<XTile<T, NF, NO>*>(osb_smem)[warp];
  const int nrows = b.n[1] * b.n[2];
  const int row0 = (blockIdx.y * XWARPS + warp) * 32;
  if (row0 >= nrows) return;  // whole warps only: the lanes below stay converged
  {
    // rows past the block end repeat the last row (computed, never stored); with a row table
    // the rows come grouped by the 32-byte-sector phase of their x = 0 element
    const int row = min(row0 + lane, nrows - 1);
    t.rowbase[lane] = xrows ? xrows[row] : lin(b, 0, row % b.n[1], row / b.n[1]);
  }
  __syncwarp();
  // Segment blockIdx.x of this warp: [0, a + xseg) for 0, then [a + k xseg, a + (k+1) xseg),
  // where x = a is the first point whose element starts a sector in the warp's rows (a = 0
  // without a row table).  Flush tiles of XOUT points are anchored at o0 = a (mod XOUT), and
  // xseg is a whole number of tiles, so every tile store covers whole sectors (the row's head
  // [0, a) is a partial tile of segment 0).
  constexpr int SEC = 32 / (int)sizeof(T);  // elements per 32-byte sector
  const int a = xrows ? (SEC - (t.rowbase[0] & (SEC - 1))) & (SEC - 1) : 0;
  const int kseg = blockIdx.x;
  const int s0 = kseg == 0 ? 0 : min(b.n[0], a + kseg * xseg);
  const int s1 = min(b.n[0], a + (kseg + 1) * xseg);
  if (s0 >= s1) return;  // warp-uniform
  const int o0 = s0 - (((s0 - a) % XOUT) + XOUT) % XOUT;  // tile origin, <= s0
  const int c0 = s0 - 3;          // global x of input column 0
  const int ncols = s1 - s0 + 6;  // columns s0-3 .. s1+2
  auto issue = [&](int k) {       // input chunk k: columns c0 + XCH k .. c0 + XCH k + XCH - 1
    const int rc = k * XCH + (lane % XCH);
    if (rc < ncols) {
      const int pos = rc % XCOLS;
#pragma unroll
      for (int rb = 0; rb < XCH; ++rb) {
        const int r = rb * RPI + lane / XCH;
        const int id = t.rowbase[r] + c0 + rc;
#pragma unroll
        for (int f = 0; f < NF; ++f) cp_async_el(&t.in[f][r][pos], field_ptr<T, ND, 0, CURV>(b, f) + id);
      }
    }
    cp_async_commit();
  };
  const T invd = inv_delta<T>(b, 0);
  // residuals of the tile's points g .. g + XOUT - 1 that lie in [s0, s1), from the out tile
  auto flush = [&](int g) {
    __syncwarp();
    const int cc = lane % XOUT;
    const int p = g + cc;
    if (p >= s0 && p < s1) {
#pragma unroll
      for (int rb = 0; rb < XOUT; ++rb) {
        const int r = rb * OPI + lane / XOUT;
        if (row0 + r < nrows) {
          const int id = t.rowbase[r] + p;
          const T sc = CURV ? t.out[NO - 1][r][cc + 1] : invd;
#pragma unroll
          for (int v = 0; v < NV; ++v) acc_flux(b, v, id, t.out[v][r][cc + 1], t.out[v][r][cc], sc, first);
        }
      }
    }
    __syncwarp();
#pragma unroll
    for (int v = 0; v < NV; ++v) t.out[v][lane][0] = t.out[v][lane][XOUT];
  };
  const int nchunks = (ncols + XCH - 1) / XCH;
  issue(0);
  if (nchunks > 1) issue(1); else cp_async_commit();
  cp_async_wait_prev();  // chunk 0 landed
  __syncwarp();
  const T gm = sp.gama;
  P w[6];
#pragma unroll
  for (int m = 1; m < 6; ++m) {  // columns 0..4: points s0-3 .. s0+1
    if (m - 1 == XCH) {          // column XCH opens chunk 1
      __syncwarp();
      if (2 < nchunks) issue(2); else cp_async_commit();
      cp_async_wait_prev();
      __syncwarp();
    }
#pragma unroll
    for (int f = 0; f < NF; ++f) set_field(w[m], f, t.in[f][lane][(m - 1) % XCOLS]);
    make_pt<T, ND>(w[m], gm);
  }
  for (int j = s0 - 1; j < s1; ++j) {
    const int rc = j - s0 + 6;  // input column of the new point j + 3
    if (rc % XCH == 0) {
      // entering chunk k = rc / XCH: every lane has read chunk k-1, whose slots take chunk k+1
      const int k = rc / XCH;
      __syncwarp();
      if (k + 1 < nchunks) issue(k + 1); else cp_async_commit();
      cp_async_wait_prev();  // chunk k landed
      __syncwarp();
    }
#pragma unroll
    for (int m = 0; m < 5; ++m) w[m] = w[m + 1];
#pragma unroll
    for (int f = 0; f < NF; ++f) set_field(w[5], f, t.in[f][lane][rc % XCOLS]);
    make_pt<T, ND>(w[5], gm);
    T fh[NV];
    if constexpr (CURV) {
      char_flux_curv<T, ND, SCH, AVG>(w, sp, fh);
    } else {
      cart_flux<T, ND, SCH, AVG, FLX>(w, sp, fh);
    }
    // interface j + 1/2 is the right face of point j: out column (j - o0) % XOUT + 1; the face
    // left of the segment lands in the column left of point s0 (the carry column when the
    // segment starts on the tile grid)
    const int dj = j - o0;
    const int oc = dj < 0 ? 0 : dj % XOUT + 1;
#pragma unroll
    for (int v = 0; v < NV; ++v) t.out[v][lane][oc] = fh[v];
    if constexpr (CURV) t.out[NO - 1][lane][oc] = invd / w[2].J;
    if (j >= s0 && (oc == XOUT || j == s1 - 1)) flush(j - (oc - 1));
  }
}

// ---------------------------------------------------------------------------------------
// Central 4th-order terms on a 3D tile (CX x CY x CZ points, halo 2 with edges).
//   CONV: central convective terms, 1 = skew-symmetric (Feiereisen) form, split_forms.py:111-145
//         as generated for the low-Mach TGV ("Convective terms" kernel); 2 = Kennedy-Gruber-
//         Pirozzoli form, split_forms.py:178-236 as generated for the Central4-WENO5 benchmark
//         (its ring holds H = (rhoE + p) / rho where form 1 holds rhoE).
//   VISC: viscous stress and heat flux (StoreSome "Viscous terms" kernel), mu from the
//         modified Sutherland law (VISC == 1) or constant (VISC == 2).
// Constants of the central kernel, derived once on the host in FP64 and handed over in both
// precisions (a conversion or division in FP64 inside an FP32 kernel runs on the FP64 pipe).
struct CentralParams {
  double gama, M2, mu_c, invRe, kheat;  // M2 = Minf^2, kheat = 1 / (Pr Re Minf^2 (gama - 1))
  float gama_f, M2_f, mu_c_f, invRe_f, kheat_f;
  double invd[3], inv2d[3];
  float invd_f[3], inv2d_f[3];
  // isothermal-wall y faces (WALL kernels): low / high face present, and the one-sided
  // closures of the first (rows 0..3, six points from m - r) and second (rows 0..1, five
  // points) derivatives next to a wall (Carpenter_scheme.py)
  int wall_lo, wall_hi;
  double c1[4][6], c2[2][5];
  float c1f[4][6], c2f[2][5];
  // VISC == 1 with mu_pow > 0: the power law mu = T^mu_pow (turbulent_channel.py:93) in place of
  // the modified Sutherland law; forced: the constant sources -c_i (momentum), -c_j u_j (energy)
  double mu_pow, force[3];
  float mu_pow_f, force_f[3];
  int forced;
};
template <typename T>
__device__ __forceinline__ T cpar(double d, float f);
template <>
__device__ __forceinline__ double cpar<double>(double d, float) { return d; }
template <>
__device__ __forceinline__ float cpar<float>(double, float f) { return f; }

// A CTA owns a 32 x CY column of points and streams it through czc planes of z (a launch
// argument, chosen on the host so the CTAs fill whole waves): the planes
// z-2 .. z+2 around the current one sit in a 5-plane ring in shared memory (halo 2 in x and y,
// edges included), the raw state of plane z+3 is loaded into registers while plane z is
// computed, then converted to primitives into the slot plane z-2 vacates.
// The tile height CY is a template argument: 8 rows stage fewer halo points per computed point
// (36 x 12 / 256 against 36 x 8 / 128) and give small blocks more threads per column, 4 rows keep
// the shared-memory ring small when it holds many fields (the KGP form with viscous terms).
// BULK (FP32 state only): the raw planes come in through the bulk-copy (TMA) engine instead --
// one cp.async.bulk per staged row and variable into a two-slot raw buffer in shared memory,
// completion counted on an mbarrier per slot, two planes ahead of the computed one.  The OPS
// row pitch (n + 10 elements) is not a multiple of 16 bytes, which a tiled tensor map needs,
// so each row copy starts at the 16-byte boundary at or below the row's first staged element
// and moves CRW elements; the lead (0..3 elements) is recomputed by the reading thread.
constexpr int CX = 32, CH = 2, CRING = 5;
constexpr int CSX = CX + 2 * CH;
constexpr int CRW = 40;  // elements per bulk row copy: CSX plus a lead of up to 3, in 16-byte units
template <int CY, int HY = CH>
struct CTile {
  static constexpr int CSY = CY + 2 * HY;  // HY: staged rows above and below the tile
  static constexpr int CPL = CSX * CSY;                        // points of one staged plane
  static constexpr int CPP = (CPL + CX * CY - 1) / (CX * CY);  // staged points per thread and plane
  static constexpr int RAW = 2 * 5 * CSY * CRW;                // floats of the two raw plane slots
};

// ---- bulk-copy (TMA) staging: mbarrier and cp.async.bulk wrappers ----
__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned long long* bar, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, 1000;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
  return t;
}
// Waits for the phase of the given parity to complete; gives up after about 0.2 s (false).
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity) {
  if (mbar_test(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (int i = 0; i < (1 << 22); ++i) {
    if (mbar_test(bar, parity)) return true;
    if (global_ns() - t0 > 200000000ull) return false;
  }
  return false;
}
// Orders this thread's earlier generic-proxy accesses of shared memory before its later bulk
// copies into it.
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
// Global -> shared bulk copy of `bytes` (16-byte aligned addresses, a multiple of 16 bytes),
// counted on mbarrier `bar`.
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

template <typename T, int CONV, int VISC>
struct CentralFields {
  // indices into the shared-memory field array
  static constexpr int U0 = 0, U1 = 1, U2 = 2, P = 3;
  static constexpr int TT = 4, MU = 5;
  static constexpr int RHO = VISC ? 6 : 4, M0 = RHO + 1, M1 = RHO + 2, M2 = RHO + 3, E = RHO + 4;
  static constexpr int N = CONV ? (VISC ? 11 : 9) : 6;
};

// BULK: at least as many CTAs per SM as its shared memory (ring, raw slots, mbarriers; 228 KB per
// SM, 1 KB reserved per CTA) admits, so the register allocation does not lower the occupancy.
// Without BULK the minimum is 0 (none declared): an explicit 1 lets the compiler spend twice the
// registers at half the occupancy.
template <int NF, int CY, bool BULK>
constexpr int bulk_ctas() {
  return BULK ? (228 * 1024) / (NF * CRING * CTile<CY>::CPL * 4 + CTile<CY>::RAW * 4 + 16 + 1024) : 0;
}
// WALL: isothermal-wall y faces (cp.wall_lo / cp.wall_hi) -- the tile stages 4 rows above and
// below instead of 2, and the y derivatives of the points next to a wall take the one-sided
// closures (viscous terms of a shock-capturing block; CONV == 0).
template <typename T, int CONV, int VISC, bool FUSE, int CY, bool BULK = false, bool WALL = false>
__global__ void __launch_bounds__(CX * CY, bulk_ctas<CentralFields<T, CONV, VISC>::N, CY, BULK>()) k_central3d(BlockK b, CentralParams cp, int first, int czc, RkFuse rf) {
  static_assert(!BULK || (sizeof(T) == 4 && FUSE), "bulk staging: FP32 state, fused update (error counter)");
  static_assert(!WALL || (CONV == 0 && !BULK), "wall closures: viscous terms of shock-capturing blocks");
  constexpr int CHY = WALL ? 4 : CH;  // staged rows above and below the tile
  constexpr int CPL = CTile<CY, CHY>::CPL, CPP = CTile<CY, CHY>::CPP, CSY = CTile<CY, CHY>::CSY;
  using Fd = CentralFields<T, CONV, VISC>;
  constexpr int FS = CRING * CPL;  // field stride in shared memory
  extern __shared__ __align__(16) unsigned char osb_smem[];
  T* sm = reinterpret_cast<T*>(osb_smem);
  // BULK: raw plane slots after the ring (16-byte aligned: FS * 4 bytes is a multiple of 16),
  // then one mbarrier per slot
  float* raw = reinterpret_cast<float*>(sm + Fd::N * FS);
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(raw + CTile<CY>::RAW);
  const int tx = threadIdx.x % CX, ty = threadIdx.x / CX;
  const int x0 = blockIdx.x * CX, y0 = blockIdx.y * CY;
  const int zb = blockIdx.z * czc, ze = min(b.n[2], zb + czc);
  const T gm = cpar<T>(cp.gama, cp.gama_f);
  const T M2 = cpar<T>(cp.M2, cp.M2_f);
  const T mu_c = cpar<T>(cp.mu_c, cp.mu_c_f);
  const T mu_pw = cpar<T>(cp.mu_pow, cp.mu_pow_f);
  const T invRe = cpar<T>(cp.invRe, cp.invRe_f);
  const T kheat = cpar<T>(cp.kheat, cp.kheat_f);
  // raw state of one plane, CPP points per thread
  T qv[CPP][5];
  auto load_plane = [&](int gz) {
#pragma unroll
    for (int u = 0; u < CPP; ++u) {
      const int idx = threadIdx.x + u * CX * CY;
      const int gx = x0 - CH + idx % CSX, gy = y0 - CHY + idx / CSX;
      if (idx < CPL && gx <= b.n[0] + CH && gy <= b.n[1] + CHY) {
        const int id = lin(b, gx, gy, gz);
#pragma unroll
        for (int v = 0; v < 5; ++v) qv[u][v] = ld_q<T>(b, v, id);
      }
    }
  };
  // primitives of the loaded plane into ring slot `slot`
  auto store_plane = [&](int slot) {
#pragma unroll
    for (int u = 0; u < CPP; ++u) {
      const int idx = threadIdx.x + u * CX * CY;
      const int gx = x0 - CH + idx % CSX, gy = y0 - CHY + idx / CSX;
      if (!(idx < CPL && gx <= b.n[0] + CH && gy <= b.n[1] + CHY)) continue;
      const int at = slot * CPL + idx;
      const T rho = qv[u][0], m0 = qv[u][1], m1 = qv[u][2], m2 = qv[u][3], E = qv[u][4];
      T ir = L_(1.0) / rho;
      T u0 = m0 * ir, u1 = m1 * ir, u2 = m2 * ir;
      T p = (gm - L_(1.0)) * (E - L_(0.5) * rho * (u0 * u0 + u1 * u1 + u2 * u2));
      sm[Fd::U0 * FS + at] = u0;
      sm[Fd::U1 * FS + at] = u1;
      sm[Fd::U2 * FS + at] = u2;
      sm[Fd::P * FS + at] = p;
      if (VISC) {
        T Tt = M2 * gm * p * ir;
        sm[Fd::TT * FS + at] = Tt;
        sm[Fd::MU * FS + at] = (VISC == 1) ? (mu_pw > L_(0.0) ? pow(Tt, mu_pw)
                                                              : L_(1.4042) * Tt * sqrt(Tt) / (L_(0.40417) + Tt))
                                           : mu_c;
      }
      if (CONV) {
        sm[Fd::RHO * FS + at] = rho;
        sm[Fd::M0 * FS + at] = m0;
        sm[Fd::M1 * FS + at] = m1;
        sm[Fd::M2 * FS + at] = m2;
        sm[Fd::E * FS + at] = CONV == 2 ? (E + p) / rho : E;
      }
    }
  };
  auto slot_of = [](int gz) { return (gz + 2 * CRING) % CRING; };
  // BULK: plane gz goes to raw slot (gz - zb + CH) & 1 and completes that slot's phase of
  // parity ((gz - zb + CH) >> 1) & 1; rows past y = n1 + CH are not copied.  A wait that runs
  // out marks the CTA broken (uniformly, through the next barrier): it issues no further copies,
  // counts the event in *rf.stall, and before returning waits (bounded) for the copies it issued.
  const int nrow = min(CSY, b.n[1] + 2 * CH + 1 - y0);
  bool broken = false;
  unsigned pend = 0, ppar = 0;  // raw slots with a copy in flight no wait has seen complete, its parity
  auto rslot = [&](int gz) { return (gz - zb + CH) & 1; };
  auto rpar = [&](int gz) { return (unsigned)((gz - zb + CH) >> 1) & 1u; };
  // The copies of a plane are spread over lanes 0..7 of every warp (one warp issuing all of them
  // measured 10 % slower); thread 0 arms the slot's next phase (arrive + expected bytes) as soon
  // as its wait saw the previous one complete, so the copies need no extra barrier.
  const unsigned plane_bytes = (unsigned)(nrow * 5 * CRW * 4);
  auto issue = [&](int gz) {  // the bookkeeping is uniform
    if (!BULK || broken || gz > ze + CH - 1) return;
    const int s = rslot(gz);
    pend |= 1u << s;
    ppar = (ppar & ~(1u << s)) | (rpar(gz) << s);
    const int lane = threadIdx.x & 31;
    if (lane >= 8) return;
    fence_async_smem();
    for (int c = (threadIdx.x >> 5) * 8 + lane; c < 5 * nrow; c += CY * 8) {
      const int v = c / nrow, r = c - v * nrow;
      const float* src = b.qf[v] + lin(b, x0 - CH, y0 - CH + r, gz);
      const float* al = reinterpret_cast<const float*>(reinterpret_cast<size_t>(src) & ~(size_t)15);
      bulk_copy_g2s(raw + ((s * 5 + v) * CSY + r) * CRW, al, CRW * 4, &bar[s]);
    }
  };
  // the 16-byte phase (0..3 elements) of each variable's array, two bits per variable: a row
  // copy's lead is that phase plus the row's linear index, mod 4
  unsigned phase = 0;
  if constexpr (BULK) {
#pragma unroll
    for (int v = 0; v < 5; ++v) phase |= (unsigned)((reinterpret_cast<size_t>(b.qf[v]) >> 2) & 3) << (2 * v);
  }
  // raw plane gz from its slot into the registers of the staged points (waits for the copy)
  auto fetch_plane = [&](int gz) -> int {
    const int s = rslot(gz);
    int late = 0;
    if (!broken) {
      late = mbar_wait_bounded(&bar[s], rpar(gz)) ? 0 : 1;
      if (!late) pend &= ~(1u << s);
      if (!late && threadIdx.x == 0 && gz + 2 <= ze + CH - 1) mbar_arrive_expect(&bar[s], plane_bytes);
    }
#pragma unroll
    for (int u = 0; u < CPP; ++u) {
      const int idx = threadIdx.x + u * CX * CY;
      const int ry = idx / CSX, cx = idx % CSX;
      if (idx < CPL && x0 - CH + cx <= b.n[0] + CH && y0 - CH + ry <= b.n[1] + CH) {
        const unsigned rl = (unsigned)lin(b, x0 - CH, y0 - CH + ry, gz);
        const float* rrow = raw + (s * 5 * CSY + ry) * CRW + cx;
#pragma unroll
        for (int v = 0; v < 5; ++v) qv[u][v] = rrow[v * CSY * CRW + (int)(((phase >> (2 * v)) + rl) & 3u)];
      }
    }
    return late;
  };
  // the barrier after a staged plane; BULK: also makes `broken` uniform
  auto plane_barrier = [&](int late) {
    if constexpr (BULK) {
      const bool was = broken;
      broken = __syncthreads_or(late) != 0 || was;
      if (broken && !was && threadIdx.x == 0) atomicAdd(rf.stall, 1ull);
    } else {
      __syncthreads();
    }
  };
  if constexpr (BULK) {
    if (threadIdx.x == 0) {
      mbar_init(&bar[0], 1);
      mbar_init(&bar[1], 1);
      mbar_init_fence();
      mbar_arrive_expect(&bar[0], plane_bytes);  // planes zb-2 and zb-1
      mbar_arrive_expect(&bar[1], plane_bytes);
    }
    __syncthreads();
    issue(zb - CH);
    issue(zb - CH + 1);
    // prologue: planes zb-2 .. zb+1 into the ring, each slot refilled two planes ahead
    for (int gz = zb - CH; gz < zb + CH; ++gz) {
      const int late = fetch_plane(gz);
      store_plane(slot_of(gz));
      plane_barrier(late);
      issue(gz + 2);
    }
  } else {
    // prologue: planes zb-2 .. zb+1 into the ring, plane zb+2 into registers
    for (int gz = zb - CH; gz < zb + CH; ++gz) {
      load_plane(gz);
      store_plane(slot_of(gz));
    }
    load_plane(zb + CH);
  }
  const int gx = x0 + tx, gy = y0 + ty;
  const bool active = gx < b.n[0] && gy < b.n[1];
  const T id0 = cpar<T>(cp.invd[0], cp.invd_f[0]), id2 = cpar<T>(cp.invd[2], cp.invd_f[2]);
  const T jd0 = cpar<T>(cp.inv2d[0], cp.inv2d_f[0]), jd2 = cpar<T>(cp.inv2d[2], cp.inv2d_f[2]);
  T id1 = cpar<T>(cp.invd[1], cp.invd_f[1]), jd1 = cpar<T>(cp.inv2d[1], cp.inv2d_f[1]);
  // WALL on a stretched y grid (metric.py:199-240, SD111 the only second-derivative metric):
  // every y derivative of this thread's row takes D11 (d/dx_1 = D11 d/dxi_1, so 1/Delta_1 and
  // 1/Delta_1^2 scale by D11 and D11^2), and the second ones add D11 SD111 d/dxi_1 = SD111 times
  // the scaled first derivative
  T sdy = L_(0.0);
  if constexpr (WALL) {
    if (b.ys[0] && gy < b.n[1]) {
      const T d11 = ystr<T>(b, 0, gy);
      id1 = id1 * d11;
      jd1 = jd1 * (d11 * d11);
      sdy = ystr<T>(b, 1, gy);
    }
  }
  // offsets are written as linear offsets of a virtual (x, y, z) tile with z stride CPL and
  // decoded into (plane, in-plane) parts; they are compile-time constants after unrolling
  const int sx = 1, sy = CSX, sz = CPL;
  const int cxy = (ty + CHY) * CSX + (tx + CH);
  // WALL: the closure rows of this thread's point (wr1: first derivatives, rows 0..3 from a
  // wall; wr2: second derivatives, rows 0..1; -1 the central rule), its weights with the sign of
  // the face applied, and the y offsets m -> yb + ys m of the stencil points
  int wr1 = -1, wr2 = -1, yb1 = 0, ys1 = 1, yb2 = 0, ys2 = 1;
  T cw1[6], cw2[5];
  if constexpr (WALL) {
    const int ny = b.n[1];
    if (gy < ny) {
      if (cp.wall_lo && gy < 4) wr1 = gy;
      else if (cp.wall_hi && gy > ny - 5) wr1 = 4 + (ny - 1 - gy);
      if (cp.wall_lo && gy < 2) wr2 = gy;
      else if (cp.wall_hi && gy > ny - 3) wr2 = 4 + (ny - 1 - gy);
    }
    const int r1 = wr1 & 3, r2 = wr2 & 1;
    const bool hi1 = wr1 >= 4, hi2 = wr2 >= 4;
    yb1 = hi1 ? r1 : -r1;
    ys1 = hi1 ? -1 : 1;
    yb2 = hi2 ? r2 : -r2;
    ys2 = hi2 ? -1 : 1;
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      const T c = r1 == 0 ? cpar<T>(cp.c1[0][m], cp.c1f[0][m])
                  : r1 == 1 ? cpar<T>(cp.c1[1][m], cp.c1f[1][m])
                  : r1 == 2 ? cpar<T>(cp.c1[2][m], cp.c1f[2][m])
                            : cpar<T>(cp.c1[3][m], cp.c1f[3][m]);
      cw1[m] = hi1 ? -c : c;
    }
#pragma unroll
    for (int m = 0; m < 5; ++m) cw2[m] = r2 == 0 ? cpar<T>(cp.c2[0][m], cp.c2f[0][m]) : cpar<T>(cp.c2[1][m], cp.c2f[1][m]);
  }
  for (int gz = zb; gz < ze; ++gz) {
    if constexpr (BULK) {
      const int late = fetch_plane(gz + CH);  // copied during iteration gz - 2
      store_plane(slot_of(gz + CH));
      plane_barrier(late);
      issue(gz + CH + 2);
    } else {
      store_plane(slot_of(gz + CH));  // plane gz+2, loaded during the previous iteration
      __syncthreads();
      if (gz + CH + 1 < ze + CH) load_plane(gz + CH + 1);
    }
    int pbase[2 * CH + 1];
#pragma unroll
    for (int k = 0; k <= 2 * CH; ++k) pbase[k] = slot_of(gz + k - CH) * CPL;
    auto F = [&](int f, int o) -> T {
      const int dz = (o + 2 * sz + sz / 2) / sz - 2;
      return sm[f * FS + pbase[dz + CH] + cxy + (o - dz * sz)];
    };
    // a staged value by plane offset dz and in-plane offset (the closures' y offsets reach 4 rows)
    auto Fp = [&](int f, int dz, int ip) -> T { return sm[f * FS + pbase[dz + CH] + cxy + ip]; };
    // closure sums of the first / second y derivative (without 1/Delta) at plane dz, x offset ox;
    // the first-derivative row 0 has four points (its last two weights are zero and the rows
    // beyond may not be staged).  Every closure row sums to zero, so the sums run over the
    // differences from the stencil's wall-side point m = 0, whose weight drops out: the FP32
    // weights then stay exactly consistent, as in d1w / d2w.
    auto Y1 = [&](int f, int dz, int ox) -> T {
      const T fw = Fp(f, dz, ox + yb1 * sy);
      T acc = L_(0.0);
#pragma unroll
      for (int m = 1; m < 4; ++m) acc += cw1[m] * (Fp(f, dz, ox + (yb1 + ys1 * m) * sy) - fw);
      if ((wr1 & 3) != 0) {
#pragma unroll
        for (int m = 4; m < 6; ++m) acc += cw1[m] * (Fp(f, dz, ox + (yb1 + ys1 * m) * sy) - fw);
      }
      return acc;
    };
    auto Y2 = [&](int f) -> T {
      const T fw = Fp(f, 0, yb2 * sy);
      T acc = L_(0.0);
#pragma unroll
      for (int m = 1; m < 5; ++m) acc += cw2[m] * (Fp(f, 0, (yb2 + ys2 * m) * sy) - fw);
      return acc;
    };
    auto D1 = [&](int f, int s, T inv) -> T {
      if (WALL && s == sy && wr1 >= 0) return Y1(f, 0, 0) * inv;
      return d1w<T>(F(f, -2 * s), F(f, -s), F(f, s), F(f, 2 * s)) * inv;
    };
    auto D2 = [&](int f, int s, T inv) -> T {
      if (WALL && s == sy && wr2 >= 0) return Y2(f) * inv;
      return d2w<T>(F(f, -2 * s), F(f, -s), F(f, 0), F(f, s), F(f, 2 * s)) * inv;
    };
    // mixed derivative: central-4 along sb of the central-4 derivative along sa (WALL: the
    // closures where sa or sb is y; moving along sb keeps the point's row along sa)
    auto DM = [&](int f, int sa, int sb, T ia, T ib) -> T {
      if (WALL && sb == sy && wr1 >= 0) {  // closure along y of the x (sa) derivatives
        auto dx = [&](int dy) -> T {
          const int o = dy * sy;
          return d1w<T>(Fp(f, 0, o - 2 * sa), Fp(f, 0, o - sa), Fp(f, 0, o + sa), Fp(f, 0, o + 2 * sa)) * ia;
        };
        const T gw = dx(yb1);
        T r = L_(0.0);
#pragma unroll
        for (int m = 1; m < 4; ++m) r += cw1[m] * (dx(yb1 + ys1 * m) - gw);
        if ((wr1 & 3) != 0) {
#pragma unroll
          for (int m = 4; m < 6; ++m) r += cw1[m] * (dx(yb1 + ys1 * m) - gw);
        }
        return r * ib;
      }
      if (WALL && sa == sy && wr1 >= 0) {  // central along sb (z) of the closure y derivatives
        const int k = sb / sz;
        return d1w<T>(Y1(f, -2 * k, 0) * ia, Y1(f, -k, 0) * ia, Y1(f, k, 0) * ia, Y1(f, 2 * k, 0) * ia) * ib;
      }
      auto dv = [&](int m) -> T {
        const int o = m * sb;
        return d1w<T>(F(f, o - 2 * sa), F(f, o - sa), F(f, o + sa), F(f, o + 2 * sa)) * ia;
      };
      return d1w<T>(dv(-2), dv(-1), dv(1), dv(2)) * ib;
    };
    // every thread reaches both barriers of an iteration at the same call sites: the point
    // update is guarded, never skipped with a jump past a barrier
    if (active) {
    const int gid = lin(b, gx, gy, gz);
    T oh[5], ol[5];
    if (!first) {
#pragma unroll
      for (int v = (CONV || FUSE) ? 0 : 1; v < 5; ++v) r_load(b, v, gid, oh[v], ol[v]);
    }
    // the fused update's state and register, loaded before the derivative work hides them
    double fq[5], fo[5];
    if constexpr (FUSE) {
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        fq[v] = b.q[v][gid];
        fo[v] = rf.a_zero ? 0.0 : b.rk[v][gid];
      }
    }
    T racc[5] = {L_(0.0), L_(0.0), L_(0.0), L_(0.0), L_(0.0)};
    const int S[3] = {sx, sy, sz};
    const T ID[3] = {id0, id1, id2};
    const T JD[3] = {jd0, jd1, jd2};
    const int UF[3] = {Fd::U0, Fd::U1, Fd::U2};
    if (CONV == 1) {
      // R_rho -= sum_j D_j m_j ; R_m_i -= D_i p + 1/2 sum_j [D_j(m_i u_j) + u_i D_j m_j + m_j D_j u_i]
      // R_E -= sum_j [D_j(p u_j) + 1/2 (D_j(E u_j) + m_j D_j(E/rho) + (E/rho) D_j m_j)]
      const int MF[3] = {Fd::M0, Fd::M1, Fd::M2};
      T divm = L_(0.0);
#pragma unroll
      for (int j = 0; j < 3; ++j) divm += D1(MF[j], S[j], ID[j]);
      racc[0] = -divm;
      T Ec = F(Fd::E, 0) / F(Fd::RHO, 0);
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        T acc = D1(Fd::P, S[i], ID[i]);
        T conv = L_(0.0), adv = L_(0.0);
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const int s = S[j];
          T pr = d1w<T>(F(MF[i], -2 * s) * F(UF[j], -2 * s), F(MF[i], -s) * F(UF[j], -s), F(MF[i], s) * F(UF[j], s),
                        F(MF[i], 2 * s) * F(UF[j], 2 * s));
          conv += pr * ID[j];
          adv += F(MF[j], 0) * D1(UF[i], s, ID[j]);
        }
        acc += L_(0.5) * (conv + F(UF[i], 0) * divm + adv);
        racc[1 + i] = -acc;
      }
      T e = L_(0.0);
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const int s = S[j];
        T dpu = d1w<T>(F(Fd::P, -2 * s) * F(UF[j], -2 * s), F(Fd::P, -s) * F(UF[j], -s), F(Fd::P, s) * F(UF[j], s),
                       F(Fd::P, 2 * s) * F(UF[j], 2 * s));
        T dEu = d1w<T>(F(Fd::E, -2 * s) * F(UF[j], -2 * s), F(Fd::E, -s) * F(UF[j], -s), F(Fd::E, s) * F(UF[j], s),
                       F(Fd::E, 2 * s) * F(UF[j], 2 * s));
        T dE = d1w<T>(F(Fd::E, -2 * s) / F(Fd::RHO, -2 * s), F(Fd::E, -s) / F(Fd::RHO, -s),
                      F(Fd::E, s) / F(Fd::RHO, s), F(Fd::E, 2 * s) / F(Fd::RHO, 2 * s));
        e += dpu * ID[j] + L_(0.5) * (dEu * ID[j] + F(MF[j], 0) * dE * ID[j]);
      }
      e += L_(0.5) * divm * Ec;
      racc[4] = -e;
    }
    if (CONV == 2) {
      // Kennedy-Gruber-Pirozzoli form (Fd::E holds H = (rhoE + p) / rho):
      // R_rho = -1/2 sum_j [D_j m_j + rho du_j/dx_j + u_j D_j rho]
      // R_m_i = -D_i p - 1/4 sum_j [D_j(u_i m_j) + rho D_j(u_i u_j) + u_i D_j m_j + u_j D_j m_i
      //                             + m_i du_j/dx_j + m_j du_i/dx_j + u_i u_j D_j rho]
      // R_E = -1/4 sum_j [D_j(H m_j) + rho D_j(H u_j) + H D_j m_j + u_j D_j(H rho) + m_j D_j H
      //                   + H rho du_j/dx_j + H u_j D_j rho]
      const int MF[3] = {Fd::M0, Fd::M1, Fd::M2};
      auto DP = [&](int f, int g, int s, T inv) -> T {
        return d1w<T>(F(f, -2 * s) * F(g, -2 * s), F(f, -s) * F(g, -s), F(f, s) * F(g, s), F(f, 2 * s) * F(g, 2 * s)) * inv;
      };
      const T rho0 = F(Fd::RHO, 0), H0 = F(Fd::E, 0);
      T dm[3], drho[3], ujj = L_(0.0), divm = L_(0.0);
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        dm[j] = D1(MF[j], S[j], ID[j]);
        drho[j] = D1(Fd::RHO, S[j], ID[j]);
        ujj += D1(UF[j], S[j], ID[j]);
        divm += dm[j];
      }
      T rc = divm + rho0 * ujj;
#pragma unroll
      for (int j = 0; j < 3; ++j) rc += F(UF[j], 0) * drho[j];
      racc[0] = -L_(0.5) * rc;
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const T ui = F(UF[i], 0), mi = F(MF[i], 0);
        T acc = L_(0.0);
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const int s = S[j];
          const T uj = F(UF[j], 0);
          acc += DP(UF[i], MF[j], s, ID[j]) + rho0 * DP(UF[i], UF[j], s, ID[j]) + ui * dm[j] +
                 uj * D1(MF[i], s, ID[j]) + mi * D1(UF[j], s, ID[j]) + F(MF[j], 0) * D1(UF[i], s, ID[j]) +
                 ui * uj * drho[j];
        }
        racc[1 + i] = -(D1(Fd::P, S[i], ID[i]) + L_(0.25) * acc);
      }
      T e = L_(0.0);
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const int s = S[j];
        const T uj = F(UF[j], 0);
        e += DP(Fd::E, MF[j], s, ID[j]) + rho0 * DP(Fd::E, UF[j], s, ID[j]) + H0 * dm[j] +
             uj * DP(Fd::E, Fd::RHO, s, ID[j]) + F(MF[j], 0) * D1(Fd::E, s, ID[j]) +
             H0 * rho0 * D1(UF[j], s, ID[j]) + H0 * uj * drho[j];
      }
      racc[4] = -L_(0.25) * e;
    }
    if (VISC) {
      T du[3][3], lap[3], dmu[3], dT[3], lapT = L_(0.0);
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) du[i][j] = D1(UF[i], S[j], ID[j]);
      const T div = du[0][0] + du[1][1] + du[2][2];
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        dmu[j] = (VISC == 1) ? D1(Fd::MU, S[j], ID[j]) : L_(0.0);
        dT[j] = D1(Fd::TT, S[j], ID[j]);
        lapT += D2(Fd::TT, S[j], JD[j]);
      }
      if constexpr (WALL) lapT += dT[1] * sdy;
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        T s = L_(0.0);
#pragma unroll
        for (int j = 0; j < 3; ++j) s += D2(UF[i], S[j], JD[j]);
        if constexpr (WALL) {
          s += du[i][1] * sdy;
          s += L_(1.0 / 3.0) * (i == 1 ? D2(UF[i], S[i], JD[i]) + du[1][1] * sdy : D2(UF[i], S[i], JD[i]));
        } else {
          s += L_(1.0 / 3.0) * D2(UF[i], S[i], JD[i]);
        }
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          if (j == i) continue;
          const int a = i < j ? i : j, bb = i < j ? j : i;
          s += L_(1.0 / 3.0) * DM(UF[j], S[a], S[bb], ID[a], ID[bb]);
        }
        lap[i] = s;
      }
      const T mu = F(Fd::MU, 0);
      T tau[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) tau[i][j] = du[i][j] + du[j][i] - (i == j ? L_(2.0 / 3.0) * div : L_(0.0));
      T e = L_(0.0);
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        T m = L_(0.0);
#pragma unroll
        for (int j = 0; j < 3; ++j) m += tau[i][j] * dmu[j];
        m += mu * lap[i];
        racc[1 + i] += m * invRe;
        const T ui = F(UF[i], 0);
#pragma unroll
        for (int j = 0; j < 3; ++j) e += mu * tau[i][j] * du[i][j] + ui * tau[i][j] * dmu[j];
        e += mu * ui * lap[i];
      }
      T h = mu * lapT;
#pragma unroll
      for (int j = 0; j < 3; ++j) h += dT[j] * dmu[j];
      racc[4] += e * invRe + h * kheat;
      if (cp.forced) {
        T w = L_(0.0);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const T fi = cpar<T>(cp.force[i], cp.force_f[i]);
          racc[1 + i] -= fi;
          w += fi * F(UF[i], 0);
        }
        racc[4] -= w;
      }
    }
    const int v0 = CONV ? 0 : 1;
    if constexpr (FUSE) {
      // a first (only) residual kernel starts from zero; otherwise from the partial residual
      unsigned nb = 0;
      if (rf.kind == 0 && rf.a_zero) {  // uniform: the first low-storage stage, one FMA per variable
#pragma unroll
        for (int v = 0; v < 5; ++v) {
          float h = first ? racc[v] : oh[v], l = first ? 0.f : ol[v];
          if (!first && v >= v0) rp_final(racc[v], h, l);
          nb += rk_point_a0(b, rf, v, gid, h, l, fq[v]);
        }
      } else {
#pragma unroll
        for (int v = 0; v < 5; ++v) {
          float h = first ? racc[v] : oh[v], l = first ? 0.f : ol[v];
          if (!first && v >= v0) rp_final(racc[v], h, l);
          nb += rk_point_ff(b, rf, v, gid, h, l, fq[v], fo[v]);
        }
      }
      if (nb) atomicAdd(rf.bad, (unsigned long long)nb);
    } else if (first) {
#pragma unroll
      for (int v = v0; v < 5; ++v) acc_point(b, v, gid, racc[v], 1);
    } else {
#pragma unroll
      for (int v = v0; v < 5; ++v) rp_store(b, v, gid, racc[v], oh[v], ol[v]);
    }
    }  // active
    __syncthreads();  // the next iteration overwrites the slot of plane gz-2
  }
  if constexpr (BULK) {
    // only a broken CTA can end with copies in flight: wait for them (bounded) before its
    // shared memory is released
#pragma unroll
    for (int s2 = 0; s2 < 2; ++s2)
      if (pend & (1u << s2)) mbar_wait_bounded(&bar[s2], (ppar >> s2) & 1u);
  }
}

}  // namespace osb
