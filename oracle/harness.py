"""Python side of the oracle: builds and calls the C restatement (osb_oracle.c) and runs the
reference's generated solvers compiled against ops_compat.h.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline, never by the opensbli_gb300 package.
"""
import ctypes
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
REF = os.path.join(HERE, "_ref")

import sys  # noqa: E402

if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from opensbli_gb300 import abi  # noqa: E402
from opensbli_gb300.spec import BlockSpec  # noqa: E402


def oracle_lib_path():
    return os.path.join(BUILD, "libosb_oracle.so")


def build_oracle(force=False):
    """Compile oracle/osb_oracle.c (gcc, no FMA contraction) into oracle/_build."""
    os.makedirs(BUILD, exist_ok=True)
    out = oracle_lib_path()
    src = os.path.join(HERE, "osb_oracle.c")
    if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return out
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp", "-o", out, src, "-lm"]
    subprocess.check_call(cmd)
    return out


_olib = None


def oracle():
    global _olib
    if _olib is None:
        lib = ctypes.CDLL(build_oracle())
        P = ctypes.POINTER
        lib.oracle_residual.argtypes = [P(abi.BlockDesc), P(ctypes.c_void_p)]
        lib.oracle_apply_bc.argtypes = [P(abi.BlockDesc), ctypes.c_int, ctypes.c_int]
        lib.oracle_stage.argtypes = [P(abi.BlockDesc), ctypes.c_int, ctypes.c_int, P(ctypes.c_double),
                                     P(ctypes.c_double), ctypes.c_int, ctypes.c_double]
        lib.oracle_step.argtypes = [P(abi.BlockDesc), ctypes.c_int, ctypes.c_int, ctypes.c_int, P(ctypes.c_double),
                                    P(ctypes.c_double), ctypes.c_double, ctypes.c_int]
        lib.oracle_reduce.argtypes = [P(abi.BlockDesc), ctypes.c_int, ctypes.c_int, P(ctypes.c_double)]
        lib.oracle_filter.argtypes = [P(abi.BlockDesc), ctypes.c_int, ctypes.c_double]
        lib.oracle_carpenter.argtypes = [ctypes.c_int, ctypes.c_int, P(ctypes.c_double)]
        lib.oracle_ystretch_metrics.argtypes = [ctypes.c_int, ctypes.c_double, P(ctypes.c_double), ctypes.c_int,
                                                ctypes.c_int, P(ctypes.c_double), P(ctypes.c_double)]
        _olib = lib
    return _olib


def _ptr(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data


def ystretch_metrics(x1, delta, wall_lo=True, wall_hi=True):
    """(D11, SD111) of a wall-normal grid line by the oracle's restatement of the generated
    metric kernels (oracle_ystretch_metrics)."""
    x = np.ascontiguousarray(x1, dtype=np.float64)
    n = x.shape[0]
    d11, sd = np.zeros(n), np.zeros(n)
    P = ctypes.POINTER(ctypes.c_double)
    if oracle().oracle_ystretch_metrics(n, float(delta), x.ctypes.data_as(P), int(wall_lo), int(wall_hi),
                                        d11.ctypes.data_as(P), sd.ctypes.data_as(P)):
        raise ValueError("oracle_ystretch_metrics refused the line")
    return d11, sd


class OracleBlocks:
    """Host state of several blocks plus the C descriptors that point into it."""

    def __init__(self, specs_states, rkold=None):
        """specs_states: (spec, state) or (spec, state, metrics) per block; metrics is the list
        of 10 metric arrays of osb_block_desc.metric (None where unused)."""
        self.specs = [t[0] for t in specs_states]
        self.q = [[np.ascontiguousarray(a, dtype=np.float64).copy() for a in t[1]] for t in specs_states]
        self.met = [None if len(t) < 3 or t[2] is None else
                    [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in t[2]]
                    for t in specs_states]
        if rkold is None:
            self.rk = [[np.zeros(s.shape) for _ in range(s.nvars)] for s in self.specs]
        else:
            self.rk = [[np.ascontiguousarray(a, dtype=np.float64).copy() for a in r] for r in rkold]
        arr = (abi.BlockDesc * len(self.specs))()
        self.dirichlet = [{k: np.ascontiguousarray(a, dtype=np.float64) for k, a in (s.dirichlet or {}).items()}
                          for s in self.specs]
        self.ys = [None if s.ystretch is None else [np.ascontiguousarray(a, dtype=np.float64) for a in s.ystretch]
                   for s in self.specs]
        for i, s in enumerate(self.specs):
            mp = None if self.met[i] is None else [None if a is None else _ptr(a) for a in self.met[i]]
            dp = {k: _ptr(a) for k, a in self.dirichlet[i].items()} or None
            yp = None if self.ys[i] is None else [_ptr(a) for a in self.ys[i]]
            arr[i] = abi.make_desc(s, [_ptr(a) for a in self.q[i]], [_ptr(a) for a in self.rk[i]], mp, dp, yp)
        self.desc = arr

    def residual(self, ib=0):
        s = self.specs[ib]
        R = [np.zeros(s.shape) for _ in range(s.nvars)]
        ptrs = (ctypes.c_void_p * 5)(*[_ptr(a) for a in R])
        oracle().oracle_residual(ctypes.byref(self.desc[ib]), ptrs)
        return R

    def apply_bc(self):
        oracle().oracle_apply_bc(self.desc, len(self.specs), 0)

    def stage(self, rk_kind, A, B, stage, dt):
        Aa = (ctypes.c_double * len(A))(*A)
        Bb = (ctypes.c_double * len(B))(*B)
        oracle().oracle_stage(self.desc, len(self.specs), rk_kind, Aa, Bb, stage, dt)

    def step(self, rk_kind, A, B, dt, nsteps):
        Aa = (ctypes.c_double * len(A))(*A)
        Bb = (ctypes.c_double * len(B))(*B)
        if oracle().oracle_step(self.desc, len(self.specs), rk_kind, len(A), Aa, Bb, dt, nsteps):
            raise RuntimeError("oracle_step refused the blocks")

    def filter(self, dt):
        """The filter step of the filtered blocks (halos must be filled; the TVD filter takes
        its point -2 velocities from the current state)."""
        if oracle().oracle_filter(self.desc, len(self.specs), dt):
            raise RuntimeError("oracle_filter refused the blocks")

    def reduce(self, what):
        out = ctypes.c_double()
        oracle().oracle_reduce(self.desc, len(self.specs), what, ctypes.byref(out))
        return out.value


# ---------------------------------------------------------------------------------------
# Reference runs (generated OPS C++ under oracle/_ref/<case>, compiled with ops_compat.h)

def ref_available(case):
    return os.path.exists(os.path.join(REF, case, "opensbli.cpp"))


def build_ref(case, force=False, fast=False):
    """Compile a generated reference case.  The parity build uses -O2 -ffp-contract=off; the
    timing build (fast=True, CPU baseline) uses -O3 with the compiler's default contraction."""
    d = os.path.join(REF, case)
    exe = os.path.join(d, "ref_case_O3" if fast else "ref_case")
    src = os.path.join(d, "opensbli.cpp")
    if not os.path.exists(src):
        raise FileNotFoundError("reference sources for %s not generated (oracle/ref_generate.py)" % case)
    deps = max(os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "ops_compat.h")))
    if not force and os.path.exists(exe) and os.path.getmtime(exe) >= deps:
        return exe
    flags = ["-O3"] if fast else ["-O2", "-ffp-contract=off"]
    cmd = ["g++", "-std=c++17"] + flags + ["-fopenmp", "-I", HERE, "-I", d, src, "-o", exe]
    subprocess.check_call(cmd)
    return exe


SHIPPED_TENO6 = os.path.join("apps", "performance_benchmark", "TENO6")


SHIPPED = {"teno6": SHIPPED_TENO6, "c4w5": os.path.join("apps", "performance_benchmark", "Central4-WENO5")}


def reference_root():
    """Directory of the upstream OpenSBLI checkout these recipes read (generator and shipped
    benchmark sources): $OSB_REFERENCE, by default the read-only checkout at /root/reference.
    None where it is absent (a copy of this tree on another machine)."""
    root = os.environ.get("OSB_REFERENCE", "/root/reference")
    return root if os.path.isdir(os.path.join(root, "opensbli")) else None


def build_shipped(name, reference=None, force=False):
    """Compile one of the reference's shipped performance-benchmark solvers (bit-exact
    generated code, from where it lies in the reference checkout: TENO6 or Central4-WENO5)
    against ops_compat.h into oracle/_ref/bench_<name>.
    -O1: at -O2 the benchmark's own out-of-bounds read of its run-mode string (see
    shipped_compat.h) is miscompiled; the floating-point semantics are the same (no FMA
    contraction, no fast math)."""
    reference = reference or reference_root()
    if reference is None:
        raise FileNotFoundError("the upstream checkout is not present (set OSB_REFERENCE)")
    src_dir = os.path.join(reference, SHIPPED[name])
    out_dir = os.path.join(REF, "bench_" + name)
    exe = os.path.join(out_dir, "ref_case")
    if not force and os.path.exists(exe):
        return exe
    if not os.path.exists(os.path.join(src_dir, "opensbli.cpp")):
        raise FileNotFoundError("shipped benchmark sources not found under %s" % src_dir)
    os.makedirs(out_dir, exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-fopenmp", "-include",
           os.path.join(HERE, "shipped_compat.h"), "-I", HERE, "-I", src_dir, os.path.join(src_dir, "opensbli.cpp"),
           "-o", exe]
    subprocess.check_call(cmd, stderr=subprocess.DEVNULL)
    return exe


def build_shipped_teno6(reference=None, force=False):
    return build_shipped("teno6", reference, force)


def run_shipped(name, n, iters, stop_after_rk=None, init=None, timeout=3600):
    """Run a shipped benchmark in its strong-scaling mode (n^3 points, dt =
    0.00084625 * 256 / n) and return its dumped arrays (at exit, or after stop_after_rk RK
    updates).  init: optional {dat_name: array} loaded right before the time loop.  The input
    line carries five tokens: the run-mode string is read into 2 bytes, and a sixth (HDF5)
    token would land in the byte after it."""
    exe = build_shipped(name)
    with tempfile.TemporaryDirectory() as td:
        with open(os.path.join(td, "input"), "w") as f:
            f.write("ss %d %d 1 0\n" % (n, iters))
        e = dict(os.environ)
        e["OSB_QUIET"] = "1"
        e["OSB_DUMP_DIR"] = td
        if stop_after_rk is not None:
            e["OSB_STOP_AFTER_RK"] = str(stop_after_rk)
        if init:
            idir = os.path.join(td, "init")
            os.makedirs(idir)
            for k, a in init.items():
                write_dump(os.path.join(idir, k + ".bin"), a)
            e["OSB_INIT_DIR"] = idir
        subprocess.run([exe], env=e, cwd=td, check=True, timeout=timeout, stdout=subprocess.DEVNULL)
        return {fn[:-4]: read_dump(os.path.join(td, fn)) for fn in os.listdir(td) if fn.endswith(".bin")}


def run_shipped_teno6(n, iters, stop_after_rk=None, timeout=3600):
    return run_shipped("teno6", n, iters, stop_after_rk=stop_after_rk, timeout=timeout)


def read_dump(path):
    hdr = np.fromfile(path, dtype=np.int32, count=8)
    nd = int(hdr[0])
    ext = [int(x) for x in hdr[1:1 + nd]]
    data = np.fromfile(path, dtype=np.float64, offset=32)
    return data.reshape(tuple(reversed(ext)))


def write_dump(path, arr, halo=5):
    nd = arr.ndim
    ext = list(reversed(arr.shape)) + [1] * (3 - nd)
    dm = [-halo] * nd + [0] * (3 - nd)
    hdr = np.array([nd] + ext + dm + [0], dtype=np.int32)
    with open(path, "wb") as f:
        f.write(hdr.tobytes())
        f.write(np.ascontiguousarray(arr, dtype=np.float64).tobytes())


def run_ref(case, env=None, init=None, stop_after_rk=None, threads=None, timeout=3600, fast=False, dump=True):
    """Run a generated reference case; returns {dat_name: array} dumped at the stop point
    plus "_rk_times" (wall-clock stamps: start of the time loop, then every RK update).

    init: optional {dat_name: array} loaded right before the time loop (OSB_INIT_DIR)."""
    exe = build_ref(case, fast=fast)
    with tempfile.TemporaryDirectory() as td:
        e = dict(os.environ)
        e["OSB_QUIET"] = "1"
        e["OSB_DUMP_DIR"] = td
        if env:
            e.update({k: str(v) for k, v in env.items()})
        if threads:
            e["OSB_THREADS"] = str(threads)
            e["OMP_NUM_THREADS"] = str(threads)
        if stop_after_rk is not None:
            e["OSB_STOP_AFTER_RK"] = str(stop_after_rk)
        if not dump:
            e["OSB_NO_DUMP"] = "1"
        if init:
            idir = os.path.join(td, "init")
            os.makedirs(idir)
            for k, v in init.items():
                write_dump(os.path.join(idir, k + ".bin"), v)
            e["OSB_INIT_DIR"] = idir
        subprocess.run([exe], env=e, cwd=td, check=True, timeout=timeout, stdout=subprocess.DEVNULL)
        out = {}
        for fn in os.listdir(td):
            if fn.endswith(".bin"):
                out[fn[:-4]] = read_dump(os.path.join(td, fn))
        red = os.path.join(td, "reductions.txt")
        if os.path.exists(red):
            out["_reductions"] = open(red).read()
        tim = os.path.join(td, "rk_times.txt")
        if os.path.exists(tim):
            out["_rk_times"] = [float(l.split()[1]) for l in open(tim) if l.strip()]
        return out


def state_names(ndim):
    return ["rho_B0"] + ["rhou%d_B0" % i for i in range(ndim)] + ["rhoE_B0"]


def rel_err(a, b):
    """max |a-b| / max |b| (relative to the field's scale)."""
    scale = max(float(np.max(np.abs(b))), 1e-300)
    return float(np.max(np.abs(a - b))) / scale
