// osb_batch.cu -- persistent fused RK stage for batches of 2D periodic blocks (FP32-residual
// path).
//
// One launch advances every block of the context by one RK stage.  The grid is persistent
// (ctas_per_sm x SMs CTAs); each CTA claims 32 x ty point tiles of any block from a work list
// (statically strided or through an atomic counter) and, per tile,
//   1. stages the FP32 state of the tile plus 3 points on every side in shared memory, reading
//      the periodic images directly from the opposite interior (equivalent to the periodic
//      halo exchange of periodic.py:53-71, so no boundary kernel runs between stages),
//   2. computes the characteristic LLF fluxes of the 33 x-interfaces of every row and the
//      ty + 1 y-interfaces of every column into shared memory (char_flux, each flux once),
//   3. forms -(dF_x/dx + dF_y/dy) per point as a float-float pair (exact flux differences),
//      applies the FP64 low-storage / SBLI RK update to the caller's state and register (the
//      first low-storage stage, A = 0, does not read the register), and
//      writes the FP32 state of the next stage into the other buffer of a ping-pong pair.
// The residual never goes to HBM.  Tiles read one FP32 buffer and write the other, so a stage
// has no intra-launch dependencies and needs no grid-wide barrier.
//
// The tiling / schedule knobs (ty, CTAs per SM, static or dynamic claiming, work order) are
// the analogue of OPS's cache-blocking tiling parameters (OPS_TILING, OPS_TILESIZE_X/Y) and are
// chosen per workload by opensbli_gb300/autotune.py.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "osb_internal.h"

namespace osb {

constexpr int BTX = 32;        // tile width (points)
constexpr int BTHREADS = 128;  // threads per CTA
constexpr int BH = 3;          // stencil reach of the flux difference

struct BatchBlock {
  int n0, n1;       // interior size
  int st1, off0;    // OPS-layout row stride and linear index of (0, 0)
  float invd0, invd1;
  double* q[4];
  double* rk[4];
  const float* qin[4];
  float* qout[4];
};

__device__ __forceinline__ int wrapi(int x, int n) { return x < 0 ? x + n : (x >= n ? x - n : x); }

template <int SCH, int AVG>
__global__ void __launch_bounds__(BTHREADS) k_batch2d(const BatchBlock* __restrict__ blocks,
                                                      const int4* __restrict__ work, int nwork, int* counter,
                                                      int ty, SchemeParams spd, int kind, double A, double B,
                                                      float dt_h, float dt_l, int save, unsigned long long* bad) {
  constexpr int NV = 4;
  const SP<float> sp(spd);
  extern __shared__ __align__(16) unsigned char osb_smem[];
  const int SP_ = BTX + 2 * BH;  // state pitch (38)
  const int SR = ty + 2 * BH;    // state rows
  float* S = reinterpret_cast<float*>(osb_smem);  // [NV][SR][SP_]
  float* Fx = S + NV * SR * SP_;                  // [NV][ty][BTX + 1]
  float* Fy = Fx + NV * ty * (BTX + 1);           // [NV][ty + 1][BTX]
  __shared__ int s_w;
  const int t = threadIdx.x;
  const float gm = sp.gama;
  unsigned long long nbad = 0;
  for (int it = 0;; ++it) {
    int w;
    if (counter) {
      if (t == 0) s_w = atomicAdd(counter, 1);
      __syncthreads();
      w = s_w;
    } else {
      w = blockIdx.x + it * gridDim.x;
    }
    if (w >= nwork) break;
    const int4 wk = work[w];
    const BatchBlock& bk = blocks[wk.x];
    const int x0 = wk.y, y0 = wk.z;
    const int n0 = bk.n0, n1 = bk.n1;
    // 1. stage the tile (periodic images read from the interior)
    for (int idx = t; idx < NV * SR * SP_; idx += BTHREADS) {
      const int c = idx % SP_, r = (idx / SP_) % SR, v = idx / (SP_ * SR);
      const int gx = wrapi(x0 - BH + c, n0), gy = wrapi(y0 - BH + r, n1);
      S[idx] = __ldg(bk.qin[v] + bk.off0 + gx + gy * bk.st1);
    }
    __syncthreads();
    // 2a. x-interfaces i + 1/2, i = -1 .. 31, of each row: thread = (row, segment)
    {
      const int nseg = BTHREADS / ty;
      const int per = (BTX + 1 + nseg - 1) / nseg;
      const int row = t % ty, seg = t / ty;
      const int i0 = -1 + seg * per, i1 = min(BTX, i0 + per);
      const float* Sr = S + (row + BH) * SP_;
      Pt<float, 2> win[6];
      if (i0 < i1) {
#pragma unroll
        for (int m = 1; m < 6; ++m) {
          const int col = i0 + m - 3 + BH;  // point i0 - 3 + m
#pragma unroll
          for (int v = 0; v < NV; ++v) win[m].q[v] = Sr[v * SR * SP_ + col];
          make_pt<float, 2>(win[m], gm);
        }
      }
      for (int i = i0; i < i1; ++i) {
#pragma unroll
        for (int m = 0; m < 5; ++m) win[m] = win[m + 1];
        const int col = i + 3 + BH;
#pragma unroll
        for (int v = 0; v < NV; ++v) win[5].q[v] = Sr[v * SR * SP_ + col];
        make_pt<float, 2>(win[5], gm);
        float fh[NV];
        char_flux<float, 2, SCH, AVG>(win, sp, fh);
#pragma unroll
        for (int v = 0; v < NV; ++v) Fx[(v * ty + row) * (BTX + 1) + i + 1] = fh[v];
      }
    }
    // 2b. y-interfaces j + 1/2, j = -1 .. ty-1, of each column (local frame: normal = u1)
    {
      const int nseg = BTHREADS / BTX;
      const int per = (ty + 1 + nseg - 1) / nseg;
      const int col = t % BTX, seg = t / BTX;
      const int j0 = -1 + seg * per, j1 = min(ty, j0 + per);
      const float* Sc = S + col + BH;
      Pt<float, 2> win[6];
      if (j0 < j1) {
#pragma unroll
        for (int m = 1; m < 6; ++m) {
          const int r = j0 + m - 3 + BH;
#pragma unroll
          for (int lv = 0; lv < NV; ++lv) win[m].q[lv] = Sc[gvar<2, 1, false>(lv) * SR * SP_ + r * SP_];
          make_pt<float, 2>(win[m], gm);
        }
      }
      for (int j = j0; j < j1; ++j) {
#pragma unroll
        for (int m = 0; m < 5; ++m) win[m] = win[m + 1];
        const int r = j + 3 + BH;
#pragma unroll
        for (int lv = 0; lv < NV; ++lv) win[5].q[lv] = Sc[gvar<2, 1, false>(lv) * SR * SP_ + r * SP_];
        make_pt<float, 2>(win[5], gm);
        float fh[NV];
        char_flux<float, 2, SCH, AVG>(win, sp, fh);
#pragma unroll
        for (int lv = 0; lv < NV; ++lv) Fy[(gvar<2, 1, false>(lv) * (ty + 1) + j + 1) * BTX + col] = fh[lv];
      }
    }
    __syncthreads();
    // 3. residual (float-float) and FP64 RK update of the tile's points
    for (int p = t; p < BTX * ty; p += BTHREADS) {
      const int r = p / BTX, c = p % BTX;
      const int gx = x0 + c, gy = y0 + r;
      if (gx >= n0 || gy >= n1) continue;
      const int id = bk.off0 + gx + gy * bk.st1;
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        float p1, e1, p2, e2;
        ff_flux_diff(Fx[(v * ty + r) * (BTX + 1) + c + 1], Fx[(v * ty + r) * (BTX + 1) + c], bk.invd0, p1, e1);
        ff_flux_diff(Fy[(v * (ty + 1) + r + 1) * BTX + c], Fy[(v * (ty + 1) + r) * BTX + c], bk.invd1, p2, e2);
        float h = __fadd_rn(p1, e1);
        float l = __fsub_rn(e1, __fsub_rn(h, p1));
        ff_add(h, l, p2, e2);
        const double x = dt_residual(h, l, dt_h, dt_l);  // as rk_point_ff
        double q = bk.q[v][id];
        double o;
        if (kind == 0) {
          o = A == 0.0 ? x : __fma_rn(A, bk.rk[v][id], x);
          q = __fma_rn(B, o, q);
        } else {
          o = save ? q : bk.rk[v][id];
          q = __fma_rn(A, x, o);
          o = __fma_rn(B, x, o);
        }
        bk.rk[v][id] = o;
        bk.q[v][id] = q;
        bk.qout[v][id] = d2f_rn(q);
        if ((((unsigned)__double2hiint(q) >> 20) & 0x7ffu) == 0x7ffu) ++nbad;
      }
    }
    __syncthreads();  // the next tile reuses the shared arrays (and s_w)
  }
  if (nbad) atomicAdd(bad, nbad);
}

size_t batch_smem(int ty) {
  const int NV = 4;
  return sizeof(float) * ((size_t)NV * (ty + 2 * BH) * (BTX + 2 * BH) + (size_t)NV * ty * (BTX + 1) +
                          (size_t)NV * (ty + 1) * BTX);
}

namespace {

template <int SCH, int AVG>
int launch_batch_t(osb_ctx* c, const BatchBlock* tab, const SchemeParams& sp, int kind, double A, double B, double dt,
                   int save) {
  const float dt_h = (float)dt, dt_l = (float)(dt - (double)dt_h);
  auto kern = k_batch2d<SCH, AVG>;
  const int ty = c->sched.tile_y;
  const size_t smem = batch_smem(ty);
  OSB_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int* counter = nullptr;
  if (c->sched.dynamic) {
    OSB_CK(cudaMemsetAsync(c->batch.counter, 0, sizeof(int), c->stream));
    counter = c->batch.counter;
  }
  const int grid = std::max(1, std::min(c->batch.nwork, c->sched.ctas_per_sm * c->sm_count));
  timing_begin(c, FAM_PERSISTENT);
  kern<<<grid, BTHREADS, smem, c->stream>>>(tab, c->batch.work, c->batch.nwork, counter, ty, sp, kind, A, B, dt_h,
                                            dt_l, save, c->bad);
  timing_end(c);
  c->launches++;
  OSB_CK(cudaGetLastError());
  return OSB_OK;
}

}  // namespace

bool batch_eligible(const osb_ctx* c, std::string* why) {
  auto no = [&](const char* w) {
    if (why) *why = w;
    return false;
  };
  if (c->prec != OSB_PREC_FP32_RESIDUAL) return no("the persistent stage is an FP32-residual path");
  if (c->blocks.empty()) return no("no blocks");
  for (const auto& bl : c->blocks) {
    if (bl.d.ndim != 2) return no("the persistent stage takes 2D blocks");
    if (bl.k.m[9]) return no("the persistent stage takes Cartesian blocks");
    if (bl.d.scheme == OSB_SCHEME_CENTRAL4 || bl.d.viscous != OSB_VISC_NONE || bl.d.flux_type != OSB_FLUX_LLF)
      return no("the persistent stage takes the characteristic LLF Euler flux");
    for (int d = 0; d < 2; ++d)
      if (bl.d.bc[d][0] != OSB_BC_PERIODIC || bl.d.bc[d][1] != OSB_BC_PERIODIC)
        return no("the persistent stage takes fully periodic blocks");
  }
  return true;
}

// Builds the per-parity block tables, the second FP32 buffer of every block and the tile
// work list for the current schedule.
int batch_build(osb_ctx* c) {
  batch_free(c);
  const int ty = c->sched.tile_y;
  if (ty != 8 && ty != 16 && ty != 32) return fail(OSB_EINVAL, "tile_y must be 8, 16 or 32");
  const int nb = (int)c->blocks.size();
  std::vector<BatchBlock> tab[2];
  for (int ib = 0; ib < nb; ++ib) {
    Block& bl = c->blocks[ib];
    if (!bl.qf_alt) return fail(OSB_EINVAL, "block %d has no FP32 state buffers", ib);
    float* buf[2] = {bl.qf_base, bl.qf_alt};
    for (int p = 0; p < 2; ++p) {
      BatchBlock b;
      memset(&b, 0, sizeof b);
      b.n0 = bl.k.n[0];
      b.n1 = bl.k.n[1];
      b.st1 = bl.k.st[1];
      b.off0 = bl.k.off0;
      b.invd0 = (float)bl.k.invd[0];
      b.invd1 = (float)bl.k.invd[1];
      for (int v = 0; v < 4; ++v) {
        b.q[v] = bl.k.q[v];
        b.rk[v] = bl.k.rk[v];
        b.qin[v] = buf[p] + (size_t)v * bl.k.alloc;
        b.qout[v] = buf[p ^ 1] + (size_t)v * bl.k.alloc;
      }
      tab[p].push_back(b);
    }
  }
  // tile list
  std::vector<int> order(nb);
  std::iota(order.begin(), order.end(), 0);
  auto npts = [&](int i) { return (long)c->blocks[i].k.n[0] * c->blocks[i].k.n[1]; };
  if (c->sched.order == 1)
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return npts(a) > npts(b); });
  std::vector<std::vector<int4>> per(nb);
  for (int ib = 0; ib < nb; ++ib) {
    const BlockK& k = c->blocks[ib].k;
    for (int y = 0; y < k.n[1]; y += ty)
      for (int x = 0; x < k.n[0]; x += BTX) per[ib].push_back(make_int4(ib, x, y, 0));
  }
  std::vector<int4> work;
  if (c->sched.order == 2) {
    // interleaved: one tile of each block in turn
    size_t maxn = 0;
    for (auto& p : per) maxn = std::max(maxn, p.size());
    for (size_t i = 0; i < maxn; ++i)
      for (int ib : order)
        if (i < per[ib].size()) work.push_back(per[ib][i]);
  } else {
    for (int ib : order) work.insert(work.end(), per[ib].begin(), per[ib].end());
  }
  c->batch.nwork = (int)work.size();
  for (int p = 0; p < 2; ++p) {
    OSB_CK(cudaMalloc(&c->batch.tab[p], sizeof(BatchBlock) * nb));
    OSB_CK(cudaMemcpyAsync(c->batch.tab[p], tab[p].data(), sizeof(BatchBlock) * nb, cudaMemcpyHostToDevice,
                           c->stream));
  }
  OSB_CK(cudaMalloc(&c->batch.work, sizeof(int4) * work.size()));
  OSB_CK(cudaMemcpyAsync(c->batch.work, work.data(), sizeof(int4) * work.size(), cudaMemcpyHostToDevice, c->stream));
  OSB_CK(cudaMalloc(&c->batch.counter, sizeof(int)));
  OSB_CK(cudaStreamSynchronize(c->stream));  // host vectors go out of scope
  c->batch.ready = true;
  return OSB_OK;
}

void batch_free(osb_ctx* c) {
  for (int p = 0; p < 2; ++p)
    if (c->batch.tab[p]) {
      cudaFree(c->batch.tab[p]);
      c->batch.tab[p] = nullptr;
    }
  if (c->batch.work) cudaFree(c->batch.work);
  if (c->batch.counter) cudaFree(c->batch.counter);
  c->batch.work = nullptr;
  c->batch.counter = nullptr;
  c->batch.nwork = 0;
  c->batch.ready = false;
}

// Points BlockK::qf of every block at FP32 buffer `parity` (0: the original one).
void batch_set_parity(osb_ctx* c, int parity) {
  c->qf_parity = parity;
  for (auto& bl : c->blocks) {
    float* buf = parity ? bl.qf_alt : bl.qf_base;
    for (int v = 0; v < bl.d.ndim + 2; ++v) bl.k.qf[v] = buf + (size_t)v * bl.k.alloc;
  }
}

// One RK stage of every block in one persistent launch; flips the FP32 buffer parity.
int batch_stage(osb_ctx* c, int s, double dt) {
  if (!c->batch.ready) {
    int rc = batch_build(c);
    if (rc) return rc;
  }
  const Block& f = c->blocks[0];
  SchemeParams sp = scheme_params(f.d.gama, f.d.eps, f.d.teno_ct, f.d.shock_filter_control, 1e-12);
  const int kind = c->rk_kind == OSB_RK_LOW_STORAGE ? 0 : 1;
  const int save = (kind == 1 && s == 0) ? 1 : 0;
  const BatchBlock* tab = c->batch.tab[c->qf_parity];
  const int sch = f.d.scheme, avg = f.d.averaging;
  int rc;
  if (avg == OSB_AVG_ROE) {
    if (sch == OSB_SCHEME_WENO5_JS) rc = launch_batch_t<SCH_WENO5_JS, AVG_ROE>(c, tab, sp, kind, c->A[s], c->B[s], dt, save);
    else if (sch == OSB_SCHEME_WENO5_Z) rc = launch_batch_t<SCH_WENO5_Z, AVG_ROE>(c, tab, sp, kind, c->A[s], c->B[s], dt, save);
    else if (sch == OSB_SCHEME_TENO6) rc = launch_batch_t<SCH_TENO6, AVG_ROE>(c, tab, sp, kind, c->A[s], c->B[s], dt, save);
    else rc = launch_batch_t<SCH_TENO5, AVG_ROE>(c, tab, sp, kind, c->A[s], c->B[s], dt, save);
  } else {
    if (sch == OSB_SCHEME_WENO5_JS) rc = launch_batch_t<SCH_WENO5_JS, AVG_SIMPLE>(c, tab, sp, kind, c->A[s], c->B[s], dt, save);
    else if (sch == OSB_SCHEME_WENO5_Z) rc = launch_batch_t<SCH_WENO5_Z, AVG_SIMPLE>(c, tab, sp, kind, c->A[s], c->B[s], dt, save);
    else if (sch == OSB_SCHEME_TENO6) rc = launch_batch_t<SCH_TENO6, AVG_SIMPLE>(c, tab, sp, kind, c->A[s], c->B[s], dt, save);
    else rc = launch_batch_t<SCH_TENO5, AVG_SIMPLE>(c, tab, sp, kind, c->A[s], c->B[s], dt, save);
  }
  if (rc) return rc;
  batch_set_parity(c, c->qf_parity ^ 1);
  return OSB_OK;
}

}  // namespace osb
