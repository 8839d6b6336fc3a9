// Minimal OPS-API-compatible host runtime used to compile and run the reference's
// generated OPS C++ solvers on the CPU.  TEST INFRASTRUCTURE ONLY (oracle side): nothing in
// the product links it.
//
// OPS itself is not vendored by the reference (it is downloaded by
// environment_and_run_scripts/InstallOPS.sh:24,137) and is not available here.  This header
// implements only the calls the generated code makes (opsc.py:1018-1252,
// core/kernel.py:303-388), written from the semantics visible in that generated code:
//   * ops_decl_dat: x-fastest arrays with d_m/d_p halos, zero initialised;
//   * ops_par_loop: loops over the [start,end) ranges (halo-relative), OpenMP over the
//     outermost dimension, ACC<double> accessors with relative offsets;
//   * ops_decl_halo / ops_halo_transfer: strided slab copies (periodic / interface);
//   * ops_arg_reduce + ops_reduction_result: sum/min/max reductions;
//   * HDF5 calls become no-ops; instead every dat is dumped as raw little-endian doubles.
//
// Run control through the environment (parity harness):
//   OSB_DUMP_DIR         directory for the dumps (default: no dump)
//   OSB_INIT_DIR         if set, the time-advanced dats named in it are loaded from
//                        <dir>/<name>.bin right before the time loop starts
//   OSB_STOP_AFTER_RK=k  dump and exit once the k-th "Temporal solution advancement" loop and
//                        the boundary loops that follow it have run
//   OSB_THREADS          OpenMP threads (default: all)
#ifndef OSB_OPS_COMPAT_H
#define OSB_OPS_COMPAT_H

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <string>
#include <vector>
#include <map>
#include <algorithm>
#include <chrono>
#include <iostream>
#include <cstdarg>
#ifdef _OPENMP
#include <omp.h>
#endif

#if defined(OPS_3D)
#define OSB_NDIM 3
#elif defined(OPS_2D)
#define OSB_NDIM 2
#else
#define OSB_NDIM 1
#endif

#define OPS_READ 0
#define OPS_WRITE 1
#define OPS_RW 2
#define OPS_INC 3
#define OPS_MIN 4
#define OPS_MAX 5

static inline int osb_env_int(const char* name, int dflt) {
  const char* s = getenv(name);
  return s ? atoi(s) : dflt;
}
static inline double osb_env_double(const char* name, double dflt) {
  const char* s = getenv(name);
  return s ? strtod(s, nullptr) : dflt;
}

struct ops_block_core { int dims; std::string name; };
typedef ops_block_core* ops_block;

struct ops_dat_core {
  ops_block block;
  int size[3] = {1, 1, 1};   // interior points
  int d_m[3] = {0, 0, 0};    // negative halo (e.g. -5)
  int d_p[3] = {0, 0, 0};
  long ext[3] = {1, 1, 1};   // allocated extent per dimension
  std::vector<double> data;
  std::string name;
  double* at(int i, int j, int k) {
    return data.data() + (i - d_m[0]) + ext[0] * ((j - d_m[1]) + ext[1] * (long)(k - d_m[2]));
  }
};
typedef ops_dat_core* ops_dat;

struct ops_stencil_core { int dims, points; std::vector<int> offs; std::string name; };
typedef ops_stencil_core* ops_stencil;

struct ops_reduction_core {
  std::string name;
  double value;
  int op;
  bool init;
};
typedef ops_reduction_core* ops_reduction;

enum osb_arg_kind { OSB_ARG_DAT, OSB_ARG_GBL, OSB_ARG_IDX, OSB_ARG_RED };
struct ops_arg {
  osb_arg_kind kind;
  ops_dat dat;
  double* gbl;
  ops_reduction red;
  int acc;
};

static std::vector<ops_dat>& osb_all_dats() { static std::vector<ops_dat> v; return v; }

template <typename T>
struct ACC {
  T* p;
  long sx, sy;
  ACC() : p(nullptr), sx(0), sy(0) {}
  inline T& operator()(int i) const { return p[i]; }
  inline T& operator()(int i, int j) const { return p[i + sx * j]; }
  inline T& operator()(int i, int j, int k) const { return p[i + sx * j + sy * k]; }
};

inline ops_arg ops_arg_dat(ops_dat d, int, ops_stencil, const char*, int acc) {
  ops_arg a; a.kind = OSB_ARG_DAT; a.dat = d; a.gbl = nullptr; a.red = nullptr; a.acc = acc; return a;
}
inline ops_arg ops_arg_gbl(double* x, int, const char*, int acc) {
  ops_arg a; a.kind = OSB_ARG_GBL; a.dat = nullptr; a.gbl = x; a.red = nullptr; a.acc = acc; return a;
}
inline ops_arg ops_arg_gbl(const double* x, int n, const char* t, int acc) {
  return ops_arg_gbl(const_cast<double*>(x), n, t, acc);
}
inline ops_arg ops_arg_idx() {
  ops_arg a; a.kind = OSB_ARG_IDX; a.dat = nullptr; a.gbl = nullptr; a.red = nullptr; a.acc = 0; return a;
}
inline ops_arg ops_arg_reduce(ops_reduction r, int, const char*, int acc) {
  ops_arg a; a.kind = OSB_ARG_RED; a.dat = nullptr; a.gbl = nullptr; a.red = r; a.acc = acc; return a;
}

// One value per kernel argument, convertible to whatever the generated signature expects.
struct osb_argval {
  ACC<double>* acc;
  double* dptr;
  int* iptr;
  operator ACC<double>&() const { return *acc; }
  operator double*() const { return dptr; }
  operator const double*() const { return dptr; }
  operator const int*() const { return iptr; }
};

static inline void ops_init(int, char**, int) {}
static inline void ops_printf(const char* fmt, ...) {
  if (osb_env_int("OSB_QUIET", 0)) return;
  va_list ap; va_start(ap, fmt); vprintf(fmt, ap); va_end(ap);
}
static inline void ops_fprintf(FILE* f, const char* fmt, ...) {
  va_list ap; va_start(ap, fmt); vfprintf(f, fmt, ap); va_end(ap);
}
static inline void ops_timers(double* cpu, double* et) {
  double t = std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
  *cpu = t; *et = t;
}
static inline void ops_partition(const char*) {}
static inline void ops_timing_output(std::ostream&) {}
template <typename T> static inline void ops_decl_const(const char*, int, const char*, T*) {}

static inline ops_block ops_decl_block(int dims, const char* name) {
  ops_block b = new ops_block_core; b->dims = dims; b->name = name; return b;
}

static inline ops_dat ops_decl_dat(ops_block b, int, int* size, int* base, int* d_m, int* d_p,
                                   double*, const char*, const char* name) {
  ops_dat d = new ops_dat_core;
  d->block = b; d->name = name;
  for (int i = 0; i < b->dims; ++i) {
    d->size[i] = size[i]; d->d_m[i] = d_m[i]; d->d_p[i] = d_p[i];
    d->ext[i] = size[i] + d_p[i] - d_m[i];
    (void)base;
  }
  d->data.assign((size_t)(d->ext[0] * d->ext[1] * d->ext[2]), 0.0);
  osb_all_dats().push_back(d);
  return d;
}

static inline ops_stencil ops_decl_stencil(int dims, int points, int* offs, const char* name) {
  ops_stencil s = new ops_stencil_core; s->dims = dims; s->points = points; s->name = name;
  s->offs.assign(offs, offs + dims * points); return s;
}

static inline ops_reduction ops_decl_reduction_handle(int, const char*, const char* name) {
  ops_reduction r = new ops_reduction_core; r->name = name; r->value = 0.0; r->op = -1; r->init = false;
  return r;
}
static inline void ops_reduction_result(ops_reduction r, double* out) {
  *out = r->value; r->init = false; r->value = 0.0;
  if (const char* dir = getenv("OSB_DUMP_DIR")) {
    std::string fn = std::string(dir) + "/reductions.txt";
    FILE* f = fopen(fn.c_str(), "a");
    if (f) { fprintf(f, "%s %.17g\n", r->name.c_str(), *out); fclose(f); }
  }
}

struct ops_halo_core {
  ops_dat from, to;
  int iter[3], from_base[3], to_base[3], from_dir[3], to_dir[3];
};
typedef ops_halo_core* ops_halo;
struct ops_halo_group_core { std::vector<ops_halo> halos; };
typedef ops_halo_group_core* ops_halo_group;

static inline ops_halo ops_decl_halo(ops_dat from, ops_dat to, int* iter, int* fb, int* tb, int* fd, int* td) {
  ops_halo h = new ops_halo_core;
  h->from = from; h->to = to;
  int nd = from->block->dims;
  for (int i = 0; i < 3; ++i) {
    h->iter[i] = i < nd ? iter[i] : 1;
    h->from_base[i] = i < nd ? fb[i] : 0;
    h->to_base[i] = i < nd ? tb[i] : 0;
    h->from_dir[i] = i < nd ? fd[i] : i + 1;
    h->to_dir[i] = i < nd ? td[i] : i + 1;
  }
  return h;
}
static inline ops_halo_group ops_decl_halo_group(int n, ops_halo* hs) {
  ops_halo_group g = new ops_halo_group_core; g->halos.assign(hs, hs + n); return g;
}
// Copy an iter[0] x iter[1] x iter[2] box.  Loop axis a of the box walks "from" axis
// |from_dir[a]|-1 and "to" axis |to_dir[a]|-1; a negative direction walks backwards.
static inline void ops_halo_transfer(ops_halo_group g) {
  for (ops_halo h : g->halos) {
    for (int c = 0; c < h->iter[2]; ++c)
      for (int b = 0; b < h->iter[1]; ++b)
        for (int a = 0; a < h->iter[0]; ++a) {
          int loop[3] = {a, b, c};
          int fi[3] = {0, 0, 0}, ti[3] = {0, 0, 0};
          for (int ax = 0; ax < 3; ++ax) {
            int fa = std::abs(h->from_dir[ax]) - 1, ta = std::abs(h->to_dir[ax]) - 1;
            fi[fa] = h->from_base[fa] + (h->from_dir[ax] > 0 ? loop[ax] : h->iter[ax] - 1 - loop[ax]);
            ti[ta] = h->to_base[ta] + (h->to_dir[ax] > 0 ? loop[ax] : h->iter[ax] - 1 - loop[ax]);
          }
          *h->to->at(ti[0], ti[1], ti[2]) = *h->from->at(fi[0], fi[1], fi[2]);
        }
  }
}

static inline void osb_dump_all(const char* tag) {
  const char* dir = getenv("OSB_DUMP_DIR");
  if (!dir) return;
  for (ops_dat d : osb_all_dats()) {
    std::string fn = std::string(dir) + "/" + d->name + ".bin";
    FILE* f = fopen(fn.c_str(), "wb");
    if (!f) { fprintf(stderr, "cannot write %s\n", fn.c_str()); exit(3); }
    int hdr[8] = {d->block->dims, (int)d->ext[0], (int)d->ext[1], (int)d->ext[2], d->d_m[0], d->d_m[1], d->d_m[2], 0};
    fwrite(hdr, sizeof(int), 8, f);
    fwrite(d->data.data(), sizeof(double), d->data.size(), f);
    fclose(f);
  }
  std::string fn = std::string(dir) + "/done.txt";
  FILE* f = fopen(fn.c_str(), "w");
  if (f) { fprintf(f, "%s\n", tag); fclose(f); }
}

static inline void osb_load_init() {
  const char* dir = getenv("OSB_INIT_DIR");
  if (!dir) return;
  for (ops_dat d : osb_all_dats()) {
    std::string fn = std::string(dir) + "/" + d->name + ".bin";
    FILE* f = fopen(fn.c_str(), "rb");
    if (!f) continue;
    int hdr[8];
    if (fread(hdr, sizeof(int), 8, f) != 8 || hdr[1] != d->ext[0] || hdr[2] != d->ext[1] || hdr[3] != d->ext[2]) {
      fprintf(stderr, "bad init file %s\n", fn.c_str()); exit(3);
    }
    if (fread(d->data.data(), sizeof(double), d->data.size(), f) != d->data.size()) {
      fprintf(stderr, "short init file %s\n", fn.c_str()); exit(3);
    }
    fclose(f);
  }
}

struct osb_run_state {
  int rk_updates = 0;
  int stop_after = -1;
  bool stop_pending = false;
  bool init_loaded = false;
};
static osb_run_state& osb_state() {
  static osb_run_state s;
  static bool once = false;
  if (!once) { once = true; s.stop_after = osb_env_int("OSB_STOP_AFTER_RK", -1); }
  return s;
}

static inline bool osb_is_bc(const char* name) {
  return strstr(name, "boundary") || strstr(name, "BC") || strstr(name, "Boundary");
}
static inline bool osb_is_init(const char* name) {
  return strstr(name, "initialisation") || strstr(name, "Initialisation");
}

static inline void ops_exit() {
  osb_dump_all("exit");
}

static inline double osb_now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Wall-clock timestamp of every completed RK update (plus the start of the time loop) in
// <OSB_DUMP_DIR>/rk_times.txt, for the CPU-baseline timing.
static inline void osb_stamp(const char* what) {
  const char* dir = getenv("OSB_DUMP_DIR");
  if (!dir) return;
  std::string fn = std::string(dir) + "/rk_times.txt";
  FILE* f = fopen(fn.c_str(), "a");
  if (f) { fprintf(f, "%s %.9f\n", what, osb_now()); fclose(f); }
}

static inline void osb_before_loop(const char* name) {
  osb_run_state& st = osb_state();
  if (!st.init_loaded && !osb_is_init(name)) {
    st.init_loaded = true;
    osb_load_init();
    osb_stamp("start");
  }
  if (st.stop_pending && !osb_is_bc(name)) {
    if (!osb_env_int("OSB_NO_DUMP", 0)) osb_dump_all("stop");
    exit(0);
  }
}
static inline void osb_after_loop(const char* name) {
  osb_run_state& st = osb_state();
  if (strstr(name, "Temporal solution advancement")) {
    osb_stamp("rk");
    st.rk_updates++;
    if (st.stop_after >= 0 && st.rk_updates >= st.stop_after) st.stop_pending = true;
  }
}

template <typename F, size_t... I>
static inline void osb_call(F fn, osb_argval* v, std::index_sequence<I...>) {
  fn(v[I]...);
}

template <typename... P, typename... A>
static void ops_par_loop(void (*fn)(P...), const char* name, ops_block blk, int dims, int* range, A... argsin) {
  static_assert(sizeof...(P) == sizeof...(A), "argument count mismatch");
  osb_before_loop(name);
  const int n = sizeof...(A);
  ops_arg args[n] = {argsin...};
  int lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
  for (int d = 0; d < dims; ++d) { lo[d] = range[2 * d]; hi[d] = range[2 * d + 1]; }
  bool has_red = false;
  for (int a = 0; a < n; ++a) {
    if (args[a].kind == OSB_ARG_RED) {
      has_red = true;
      ops_reduction r = args[a].red;
      if (!r->init) {
        r->init = true; r->op = args[a].acc;
        r->value = args[a].acc == OPS_MIN ? 1e308 : (args[a].acc == OPS_MAX ? -1e308 : 0.0);
      }
    }
  }
  int outer = dims - 1;
  int nthreads = 1;
#ifdef _OPENMP
  nthreads = osb_env_int("OSB_THREADS", omp_get_max_threads());
  if (has_red) nthreads = 1;  // keep reductions in sequential order
#endif
  (void)blk;
#pragma omp parallel for num_threads(nthreads) schedule(static)
  for (int o = lo[outer]; o < hi[outer]; ++o) {
    ACC<double> acc[n];
    double redv[n];
    osb_argval v[n];
    int idx[3] = {0, 0, 0};
    for (int a = 0; a < n; ++a) {
      v[a].acc = &acc[a]; v[a].dptr = nullptr; v[a].iptr = idx;
      if (args[a].kind == OSB_ARG_DAT) {
        acc[a].sx = args[a].dat->ext[0];
        acc[a].sy = args[a].dat->ext[0] * args[a].dat->ext[1];
      } else if (args[a].kind == OSB_ARG_GBL) {
        v[a].dptr = args[a].gbl;
      } else if (args[a].kind == OSB_ARG_RED) {
        redv[a] = args[a].red->value;
        v[a].dptr = &redv[a];
      }
    }
    int i0lo = lo[0], i0hi = hi[0];
    int i1lo = dims > 1 ? lo[1] : 0, i1hi = dims > 1 ? hi[1] : 1;
    if (outer == 0) { i0lo = o; i0hi = o + 1; }
    if (outer == 1) { i1lo = o; i1hi = o + 1; }
    int k = outer == 2 ? o : 0;
    for (int j = i1lo; j < i1hi; ++j)
      for (int i = i0lo; i < i0hi; ++i) {
        idx[0] = i; idx[1] = j; idx[2] = k;
        for (int a = 0; a < n; ++a)
          if (args[a].kind == OSB_ARG_DAT) acc[a].p = args[a].dat->at(i, j, k);
        osb_call(fn, v, std::make_index_sequence<sizeof...(P)>{});
      }
    if (has_red) {
      for (int a = 0; a < n; ++a)
        if (args[a].kind == OSB_ARG_RED) args[a].red->value = redv[a];
    }
  }
  osb_after_loop(name);
}

static inline void ops_NaNcheck(ops_dat d) {
  for (double x : d->data)
    if (std::isnan(x)) { fprintf(stderr, "NaN detected in %s\n", d->name.c_str()); exit(2); }
}

// HDF5 entry points: the oracle harness dumps raw arrays instead.
template <typename... T> static inline void ops_fetch_block_hdf5_file(T...) {}
template <typename... T> static inline void ops_fetch_dat_hdf5_file(T...) {}
template <typename... T> static inline void ops_write_const_hdf5(T...) {}
template <typename... T> static inline void ops_get_const_hdf5(T...) {}
static inline ops_dat ops_decl_dat_hdf5(ops_block, int, const char*, const char* name, const char*) {
  fprintf(stderr, "restart from HDF5 (%s) is not supported by the oracle harness\n", name);
  exit(4);
}

#endif
