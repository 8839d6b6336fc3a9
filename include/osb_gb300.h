/*
 * osb_gb300.h -- C ABI of the GB300 (sm_103a) residual-and-update path for OpenSBLI.
 *
 * The reference turns a problem script into OPS C++ (opensbli/code_generation/opsc.py:407-460)
 * whose main() runs, per RK stage, constituent-relation loops, one characteristic
 * WENO/TENO reconstruction loop per direction, the residual loop, the central derivative and
 * viscous loops, the RK update loop and the halo exchanges
 * (apps/performance_benchmark/TENO6/opensbli.cpp:206-431).  This library replaces that whole
 * stage: the Python backend (opensbli_gb300/backend.py, standing in for OPSC(alg)) fills one
 * osb_block_desc per OpenSBLI block and drives the steps through the calls below.
 *
 * Conventions
 *  - Every function returns an int status: OSB_OK (0) or a negative OSB_E* code; the text of
 *    the last error of the calling thread is read with osb_last_error().  No C++ exception
 *    crosses this boundary.
 *  - Arrays use the OPS layout the generated code declares (opsc.py:1182-1196): one array per
 *    variable, x fastest, `halo` (=5) points on both sides of every used dimension, FP64.
 *    Pointers in osb_block_desc are DEVICE pointers owned by the caller (borrowed until
 *    osb_ctx_destroy).
 *  - A context serves one host thread and owns one CUDA stream on its device.
 */
#ifndef OSB_GB300_H
#define OSB_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OSB_VERSION 100

#define OSB_OK 0
#define OSB_EINVAL -1      /* bad argument or descriptor */
#define OSB_ECUDA -2       /* CUDA runtime error */
#define OSB_ETIMEDOUT -3   /* osb_sync gave up waiting */
#define OSB_ENOTSUP -4     /* configuration outside the supported path */
#define OSB_ENAN -5        /* non-finite value detected in the state */

/* Convective (shock-capturing) scheme: LFWeno/LFTeno (opensbli/schemes/spatial/weno.py:475,
 * teno.py:480) with characteristic local Lax-Friedrichs splitting; or the central
 * skew-symmetric (Feiereisen) form of physical_models/split_forms.py with StoreSome(4). */
#define OSB_SCHEME_WENO5_JS 1
#define OSB_SCHEME_WENO5_Z 2
#define OSB_SCHEME_TENO5 3
#define OSB_SCHEME_TENO6 4
#define OSB_SCHEME_CENTRAL4 5

/* Averaging for the characteristic system (schemes/spatial/averaging.py:31,65). */
#define OSB_AVG_SIMPLE 0
#define OSB_AVG_ROE 1

/* Viscous terms: none (Euler), modified Sutherland law mu(T) (compressible_TGV.py:82),
 * constant viscosity (split_forms.py viscosity='constant'), or the power law mu = T^visc_power
 * of apps/channel_flow/compressible_TCF_TENO/turbulent_channel.py:93, or Sutherland's law with
 * its ratio S = SuthT / RefT, mu = T^1.5 (1 + S) / (T + S) (apps/katzer_SBLI/katzer_SBLI.py:67;
 * restated in the oracle, refused by the GPU path). */
#define OSB_VISC_NONE 0
#define OSB_VISC_SUTHERLAND 1
#define OSB_VISC_CONSTANT 2
#define OSB_VISC_POWER_LAW 3
#define OSB_VISC_SUTHERLAND_RATIO 4

/* Boundary conditions per face (core/boundary_conditions/). */
#define OSB_BC_PERIODIC 0    /* PeriodicBC -> ExchangeSelf (periodic.py:25-71) */
#define OSB_BC_ZERO_GRAD 1   /* ZeroGradientOutletBC (zero_gradient_outlet.py:11-23) */
#define OSB_BC_INTERFACE 2   /* InterfaceBC between blocks (multi_block.py:48-107) */
#define OSB_BC_EXTRAP0 3     /* ExtrapolationBC order 0 (extrapolation.py:29-38), halo fill only */
#define OSB_BC_EXTRAP1 4     /* ExtrapolationBC order 1 (extrapolation.py:39-53), halo fill only */
#define OSB_BC_SYMMETRY 5    /* SymmetryBC, Cartesian (symmetry.py:23-50): halo layer k = the point k
                                inside, normal momentum negated; the boundary plane unchanged */
#define OSB_BC_DIRICHLET 6   /* DirichletBC (dirichlet.py:27-41): the boundary plane and its halo
                                layers set from osb_block_desc.dirichlet */
#define OSB_BC_PRESSURE_OUTLET 7 /* PressureOutletBC (pressure_outlet.py:35-51), Cartesian: the
                                boundary plane and its halo layers take rho and momentum of the
                                point inside, rhoE from osb_block_desc.back_pressure */
#define OSB_BC_ISOTHERMAL_WALL 8 /* IsothermalWallBC (isothermal_wall.py:62-131) with the wall
                                energy rhoE = Twall rho / (gama Minf^2 (gama - 1)), Twall from
                                osb_block_desc.wall_temperature: no-slip wall plane, halo layer
                                k with T = (k+1) Twall - k T(inside), the wall pressure and the
                                mirrored velocity of the point k inside; the central derivatives
                                of the viscous terms take the one-sided Carpenter closures at the
                                four points next to the wall (Carpenter_scheme.py).  3D
                                Cartesian blocks, walls on y faces, shock-capturing schemes. */
#define OSB_BC_ADIABATIC_WALL 9  /* AdiabaticWallBC (adiabatic_wall.py:28-69): no-slip wall plane with
                                the energy of the wall temperature that makes the one-sided
                                third-order dT/dn vanish, T_w = (18 T1 - 9 T2 + 2 T3) / 11; halo
                                layer k mirrors the point k inside (momentum negated); the same
                                Carpenter closures and scope as OSB_BC_ISOTHERMAL_WALL. */
#define OSB_BC_INLET_PRESSURE_EXTRAP 10 /* InletPressureExtrapolateBC (inlet_pressure_extrapolate.py:11-
                                  73), low x face: where |u_n| >= a at the boundary plane it takes
                                  the inflow state the halo holds, else rhoE of the plane is copied
                                  into the bc_depth halo layers; a ModifyCentralDerivative face
                                  (the viscous terms' Carpenter closures apply).  Restated in the
                                  oracle; the GPU path refuses it (OSB_EINVAL at osb_block_add). */

/* Convective split form of OSB_SCHEME_CENTRAL4 (physical_models/split_forms.py). */
#define OSB_SPLIT_FEIEREISEN 0 /* skew-symmetric form, split_forms.py:111-145 */
#define OSB_SPLIT_KGP 1        /* Kennedy-Gruber-Pirozzoli form, split_forms.py:178-236 */

/* Filter applied after every full RK step (filters/WENO_filter.py, filters/TVD_filter.py). */
#define OSB_FILTER_NONE 0
#define OSB_FILTER_WENO3 1     /* non-linear characteristic WENO3-Z filter with a Ducros sensor */
#define OSB_FILTER_TVD 2       /* non-linear characteristic TVD filter (Yee-Sandham-Djomehri
                                  limiter with Harten's switch, shock_capturing.py:619-766) */

/* Riemann flux of the characteristic WENO / TENO reconstruction (shock_capturing.py). */
#define OSB_FLUX_LLF 0         /* flux-split local Lax-Friedrichs (LFWeno / LFTeno) */
#define OSB_FLUX_HLLC_LM 1     /* HLLC-LM from reconstructed states (HLLCWeno, lines 1031-1256):
                                  Cartesian 2D / 3D blocks, WENO5-JS / WENO5-Z / TENO5 */

/* Residual precision (per context). */
#define OSB_PREC_FP64 0          /* plain FP64 path, parity with the generated solver */
#define OSB_PREC_FP32_RESIDUAL 1 /* FP32 residual arithmetic, FP64 state/RK/reductions */

/* Time integrators (schemes/temporal/rk_LS.py, rk_sbli.py). */
#define OSB_RK_LOW_STORAGE 0     /* RKold = A*RKold + dt*R ; q += B*RKold */
#define OSB_RK_SBLI3 1           /* old = q at step start; q = old + dt*B*R ; old += dt*A*R */

/* Reductions (osb_reduce). */
#define OSB_RED_KE 0             /* sum 0.5*rho*|u|^2 over interior points */
#define OSB_RED_ENSTROPHY_DISS 1 /* sum mu*|curl u|^2 (central-4 derivatives) */
#define OSB_RED_DILATATION_DISS 2/* sum 4/3*mu*(div u)^2 */
#define OSB_RED_RHO_SUM 3        /* sum rho */
#define OSB_RED_CFL_DT 4         /* min over points of 1/sum_d (|u_d|+a)/Delta_d */
#define OSB_RED_NAN_COUNT 5      /* number of non-finite values in the state */

typedef struct osb_ctx osb_ctx;

typedef struct osb_interface {
  int32_t block;   /* index (osb_block_add order) of the neighbouring block */
  int32_t dir;     /* its direction that faces this one */
  int32_t side;    /* its side (0 = low, 1 = high) */
  int32_t flip;    /* 1: InterfaceBC match flag (opsc.py:1043-1045): the normal index of the
                      neighbour runs the other way, so its layers are copied in reverse order
                      (faces of equal sides, e.g. both low faces of a C-mesh wake cut) */
} osb_interface;

typedef struct osb_block_desc {
  int32_t ndim;              /* 1, 2 or 3 */
  int32_t size[3];           /* interior points per direction (1 for unused directions) */
  int32_t halo;              /* halo points on each side of every used direction: 5 */
  int32_t scheme;            /* OSB_SCHEME_* */
  int32_t averaging;         /* OSB_AVG_* */
  int32_t viscous;           /* OSB_VISC_* */
  int32_t bc[3][2];          /* OSB_BC_* per direction, side */
  int32_t bc_depth[3][2];    /* halo layers written by that boundary (4 or 5) */
  osb_interface iface[3][2]; /* neighbour for OSB_BC_INTERFACE faces */
  double gama, Minf, Re, Pr;
  double mu_const;           /* OSB_VISC_CONSTANT: dimensionless viscosity (1.0 in the TGV app) */
  double eps;                /* TENO epsilon (teno.py:369-371) */
  double teno_ct;            /* TENO cut-off C_T (teno.py:373-377) */
  double shock_filter_control; /* LLF wave-speed scale (shock_capturing.py:1008-1019) */
  double delta[3];           /* grid spacing per direction */
  double* q[5];              /* conserved variables rho, rhou0.., rhoE (device, OPS layout) */
  double* rkold[5];          /* RK register (device, OPS layout) */
  const double* metric[10];  /* curvilinear: D00 D01 D02 D10 D11 D12 D20 D21 D22 detJ, or NULL */
  int32_t split_form;        /* OSB_SPLIT_* (central scheme only; 0 = Feiereisen) */
  int32_t filter;            /* OSB_FILTER_* (3D central scheme only; 0 = none) */
  double ducros_check;       /* filter flux where max kappa over the interface stencil > this */
  double ducros_select;      /* filter applied where max kappa around the point >= this */
  double tvd_kappa;          /* OSB_FILTER_TVD: the filter strength kappa_TVD */
  /* OSB_BC_DIRICHLET face (d, side): device array of the conserved variables the BC's
   * equations give on the boundary plane and its bc_depth halo layers, [v][layer][t]: layer l
   * at index -depth + l (side 0) or N-1 + l (side 1) along d, t over the whole allocated
   * extent of the other used directions (lower direction fastest).  NULL elsewhere. */
  const double* dirichlet[3][2];
  int32_t flux_type;         /* OSB_FLUX_* of the shock-capturing schemes (0 = LLF) */
  double back_pressure[3][2]; /* OSB_BC_PRESSURE_OUTLET face (d, side): its back pressure */
  double wall_temperature[3][2]; /* OSB_BC_ISOTHERMAL_WALL face (d, side): Twall */
  /* Stretched wall-normal grid (a MetricsEquation with direction 1 stretched only, applied to the
   * equations: equation_types/metric.py:183-240): D11 = d xi_1 / d x_1 (ystretch[0]) and
   * SD111 = d D11 / d xi_1 (ystretch[1]) of every interior row j = 0 .. size[1]-1, as
   * osb_ystretch_metrics computes them (device arrays of size[1] doubles; host arrays for the
   * oracle); delta[1] is the spacing of xi_1.  The y flux difference and every y derivative of the
   * viscous terms take them: d/dx_1 = D11 d/dxi_1, d2/dx_1^2 = D11^2 d2/dxi_1^2 + D11 SD111 d/dxi_1.
   * NULL for a uniform y grid.  3D Cartesian viscous blocks with wall faces on both y sides only. */
  const double* ystretch[2];
  double visc_power;         /* OSB_VISC_POWER_LAW: the exponent (0.7 in the channel app) */
  /* Constant source terms of the channel apps' momentum and energy equations
   * (turbulent_channel.py:38-39, "- KD(_i,_j)*c_j" and "- Dot(c_j, u_j)"): R(rhou_i) -= c_i,
   * R(rhoE) -= sum_j c_j u_j, applied by the central viscous kernel (3D Cartesian viscous
   * blocks; OSB_EINVAL otherwise). */
  double forcing[3];
  double sutherland_s;       /* OSB_VISC_SUTHERLAND_RATIO: S = SuthT / RefT */
} osb_block_desc;

/* ---- library / context ------------------------------------------------------------- */

/* Library version (OSB_VERSION). */
int osb_version(void);

/* Copies the calling thread's last error message into buf (NUL terminated); returns its
 * length. */
int osb_last_error(char* buf, size_t n);

/* Creates a context on `device` with residual precision OSB_PREC_*; replaces ops_init and
 * the generated OPS declarations (opensbli.cpp:45-160). */
int osb_ctx_create(int device, int precision, osb_ctx** out);

/* Destroys the context, its stream, graphs and workspaces. */
int osb_ctx_destroy(osb_ctx* ctx);

/* Registers one block (ops_decl_block + ops_decl_dat of q / RKold, defdec_data_set.h).
 * Blocks of one context share the scheme, averaging, viscosity and precision; sizes,
 * spacings, boundaries and arrays may differ.  *block_id receives the block index. */
int osb_block_add(osb_ctx* ctx, const osb_block_desc* desc, int* block_id);

/* Selects the time integrator and its coefficients (rk_LS.py:97-132 / rk_sbli.py:75-77).
 * A = stage coefficients (rkA / rknew), B = solution coefficients (rkB / rkold). */
int osb_set_rk(osb_ctx* ctx, int kind, int nstages, const double* A, const double* B);

/* ---- time stepping (the generated time loop, opensbli.cpp:206-431) ------------------- */

/* Advances every block by nsteps full RK steps of size dt.  With graphs enabled the step is
 * captured once into a CUDA graph and replayed.  Asynchronous: returns after queueing. */
int osb_step(osb_ctx* ctx, double dt, int nsteps);

/* Host-memory entry point for independent runs of the context's blocks (the reference's
 * generated solver keeps its state in host memory, opensbli.cpp:86-120 and 206-431): request r
 * copies the state from host buffer in[r] (every block's variables in block order, each the
 * whole allocation including halos, the layout the block descriptors' q arrays have,
 * concatenated), advances it nsteps whole steps (osb_step) and copies the result into out[r].
 * The host-to-device copy of request r+1 and the device-to-host copy of request r-1 run on two
 * copy streams while request r computes (pinned host buffers for the overlap).  in[r] may
 * repeat; out[r] must not be read before the call returns.  Keeps four device staging buffers
 * of one request's size.  Synchronous: returns when every result is in host memory, and on an
 * error only after every copy it queued has finished. */
int osb_step_requests(osb_ctx* ctx, int count, const double* const* in, double* const* out, double dt,
                      int nsteps);

/* Runs one RK stage (index `stage`) on every block: residual, update, boundaries. */
int osb_stage(osb_ctx* ctx, int stage, double dt);

/* Applies the boundary conditions / halo exchanges of every block once
 * (ops_halo_transfer / boundary kernels of the generated code). */
int osb_apply_bc(osb_ctx* ctx);

/* Writes the residual dq/dt of block `block` (before any update) into the caller's device
 * arrays out[nvars] (OPS layout, FP64) -- per-kernel parity hook. */
int osb_residual(osb_ctx* ctx, int block, double* const* out);

/* FP64 global reduction over all blocks of the context (OSB_RED_*); replaces the
 * ops_reduction_result calls of the generated post-processing (opensbli.cpp:450-453). */
int osb_reduce(osb_ctx* ctx, int what, double* host_out);

/* Waits for the context's stream, giving up after timeout_ms (OSB_ETIMEDOUT). */
int osb_sync(osb_ctx* ctx, int timeout_ms);

/* Enables (1) or disables (0) CUDA-graph capture of osb_step. */
int osb_set_graphs(osb_ctx* ctx, int enable);

/* Selects the segment length of the x reconstruction sweep (autotuner hook): 0, < 0 or > 5 the
 * length that fills whole waves of resident CTAs, 1 = whole rows, 2 = 64, 3 = 32, 4 = 16,
 * 5 = 48 points. */
int osb_set_variant(osb_ctx* ctx, int variant);

/* Selects how the FP32-residual path's central kernel (fused RK update) stages the raw state of
 * its z planes: 0 (default) per-thread register loads one plane ahead, 1 bulk copies through the
 * TMA engine (one cp.async.bulk per staged row and variable, completion on an mbarrier per slot,
 * two planes ahead; 20-35 % slower on GB300: the OPS row pitch allows no tiled tensor map, so a
 * plane takes 60 copies of 160 bytes).  Both give bit-identical results.  A bulk-copy wait that
 * runs out (about 0.2 s) ends the kernel's use of the copies and makes the next osb_sync return
 * OSB_ECUDA. */
int osb_set_central_staging(osb_ctx* ctx, int bulk);

/* Stage schedule.  OSB_SCHED_PER_BLOCK runs every block's sweeps, RK update and boundary
 * kernels as separate launches; OSB_SCHED_PERSISTENT runs one fused persistent launch per RK
 * stage over all blocks (FP32-residual path, 2D fully periodic blocks with the characteristic
 * flux: residual kept on chip, periodic images read in place, FP32 state ping-ponged between
 * two buffers); OSB_SCHED_AUTO picks the persistent stage whenever the blocks qualify.  The
 * remaining fields tune the persistent stage: tile height (8, 16 or 32 points; tiles are 32
 * wide), resident CTAs per SM, dynamic (atomic) or static tile claiming, and the tile order
 * (0 block order, 1 largest blocks first, 2 interleaved across blocks).  fuse_update selects,
 * for the per-block FP32-residual path, whether the last residual kernel (the central kernel of
 * a viscous or central block) applies the RK update itself.  The analogue of
 * OPS's cache-blocking tiling parameters (OPS_TILING, OPS_TILESIZE_X / _Y). */
#define OSB_SCHED_AUTO (-1)
#define OSB_SCHED_PER_BLOCK 0
#define OSB_SCHED_PERSISTENT 1
typedef struct osb_schedule {
  int32_t mode;
  int32_t tile_y;
  int32_t ctas_per_sm;
  int32_t dynamic;
  int32_t order;
  int32_t fuse_update; /* per-block FP32 path: 1 = the central kernel applies the RK update */
} osb_schedule;

int osb_set_schedule(osb_ctx* ctx, const osb_schedule* sched);

/* The schedule in effect: *mode_out receives OSB_SCHED_PER_BLOCK or OSB_SCHED_PERSISTENT as
 * resolved for the current blocks (AUTO resolved), *sched_out (optional) the settings. */
int osb_get_schedule(osb_ctx* ctx, int* mode_out, osb_schedule* sched_out);

/* Per-kernel timing, the analogue of OPS's ops_timing_output (opsc.py:826-836): while enabled
 * every kernel launch is bracketed by CUDA events on the context stream (CUDA graphs are
 * bypassed). */
int osb_timing(osb_ctx* ctx, int enable);

/* Writes accumulated milliseconds and launch counts per kernel family (0 flux-x, 1 flux-y,
 * 2 flux-z, 3 central, 4 RK update, 5 boundaries, 6 reductions, 7 persistent stage, 8 filter) into
 * ms[0..n) / launches[0..n) and resets them. */
int osb_timing_report(osb_ctx* ctx, double* ms, long long* launches, int n);

/* Returns the number of kernel launches the context has issued so far. */
int osb_launch_count(osb_ctx* ctx, long long* out);

/* Raw CUDA stream of the context (cudaStream_t), for event timing by the caller. */
int osb_get_stream(osb_ctx* ctx, void** stream);

/* ---- allocation-free variant ---------------------------------------------------------- */

/* Size, in doubles, of the static residual workspace behind osb_stage_noalloc (32 MB). */
#define OSB_NOALLOC_MAX_DOUBLES (4u * 1024u * 1024u)

/* One RK stage (index-free: coefficients A, B given directly) of one block on the caller's
 * stream, for callers that cannot allocate device memory: an application that owns all GPU
 * memory through its own pool, or one that must not call cudaMalloc after start-up.  It calls
 * no cudaMalloc / cudaFree and creates no stream, graph or context; the FP64 residual workspace
 * is a file-scope __device__ array of OSB_NOALLOC_MAX_DOUBLES doubles that every GPU loading
 * the library holds until exit, and blocks whose nvars x allocated points exceed it are
 * rejected with OSB_EINVAL.  The caller passes the state and RK arrays in the descriptor (FP64
 * path only) and, for OSB_RK_SBLI3, copies q into rkold at the start of each step itself.
 *  - Halos: the stage reads q's halos as they are and applies the block's boundary faces only
 *    after its update, so before the first call the caller fills them (one osb_apply_bc on a
 *    context, or its own exchange); later calls leave them filled.
 *  - Faces: periodic, zero-gradient, extrapolation, symmetry, Dirichlet, pressure outlet and
 *    isothermal / adiabatic wall, with the kernels osb_apply_bc uses; a block with an interface
 *    face (or one periodic side) is refused with OSB_ENOTSUP before anything is launched, so the
 *    caller's arrays are untouched.
 *  - Device: the call runs on the current device; `stream` and every array must belong to it
 *    (checked: OSB_EINVAL otherwise).  The first call on a device looks up the workspace address
 *    (cudaGetSymbolAddress) and should come before any stream capture on that device.
 *  - Non-finite values are not reported by this entry point (the context path reports them
 *    through osb_sync / OSB_RED_NAN_COUNT).
 *  - All calls share the workspace: calls that overlap on the GPU race.
 * Asynchronous on `stream` (a cudaStream_t, NULL for the default stream).
 * No counterpart in the reference (OPS always allocates its own datasets). */
int osb_stage_noalloc(const osb_block_desc* desc, int rk_kind, double A, double B, double dt, void* stream);

/* ---- stretched wall-normal grid ------------------------------------------------------ */

/* Metrics of a wall-normal grid line x1[j], j = 0 .. n-1 (the generated "MetricsEquation
 * evaluation" kernels of a MetricsEquation with direction 1 stretched only,
 * equation_types/metric.py:183-240, with the Carpenter closures of
 * core/boundary_conditions/Carpenter_scheme.py in the four rows next to a wall face): with
 * x1' the 4th-order derivative of x1 along xi_1 (spacing delta), d11[j] = 1 / x1'[j] and
 * sd111[j] the same derivative of d11.  wall_lo / wall_hi: 1 where that y face is a wall (the
 * closures apply; the channel apps have walls on both).  Host arrays, no GPU work; n >= 12. */
int osb_ystretch_metrics(int32_t n, double delta, const double* x1, int32_t wall_lo, int32_t wall_hi, double* d11,
                         double* sd111);

/* ---- curvilinear metrics (equation_types/metric.py:183-327) -------------------------- */

#define OSB_METRIC_PERIODIC 0 /* interior, halos the periodic images (a periodic block) */
#define OSB_METRIC_EDGE 1     /* where the stencil fits (-3..N+2), outer layers repeat the nearest */

/* Metric arrays of a 2D or 3D block on the device from its grid coordinates x[0..ndim-1]
 * (device, OPS layout of the descriptor's size and halo, known at every allocated point):
 * J_ij = d x_i / d xi_j with the generated metric kernel's 4th-order central differences and
 * operator order, met[3 d + i] = d xi_d / d x_i (J inverted; 2D: the generated closed form),
 * met[9] = det J -- the arrays osb_block_desc.metric takes.  2D writes slots 0, 1, 3, 4, 9 only.
 * Reads ndim, size, halo and delta of desc.  Asynchronous on `stream`. */
int osb_metrics(const osb_block_desc* desc, const double* const* x, double* const* met, int fill, void* stream);

/* Binding check: writes sizeof(osb_block_desc) and the byte offsets of size, bc, iface, gama,
 * delta, q, rkold, metric, split_form, ducros_check, tvd_kappa, dirichlet, flux_type,
 * back_pressure, wall_temperature, ystretch, visc_power, forcing and sutherland_s into
 * out[0..19] (n >= 20).  Needs no GPU. */
int osb_desc_layout(long long* out, int n);

#ifdef __cplusplus
}
#endif
#endif
