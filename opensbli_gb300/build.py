"""In-tree build of libosb_gb300.so for sm_103a.

The flux sweeps are compiled once per (precision, dimension, Cartesian or curvilinear) into
separate objects so the
translation units build in parallel; the objects go to opensbli_gb300/_build and the library
to opensbli_gb300/libosb_gb300.so (both git-ignored).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(HERE, "libosb_gb300.so")
PROBE = os.path.join(HERE, "libosb_probe.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-cudart", "shared", "-I", CSRC, "-I", INCLUDE]

# (object name, source, extra defines)
# The FP32-residual units are compiled with --use_fast_math (approximate reciprocal/sqrt,
# flush-to-zero, FMA contraction); the FP64 parity units keep IEEE division and square root.
FAST = ["--use_fast_math"]
UNITS = [
    ("api", "osb_gb300.cu", []),
    ("central_f64", "osb_central.cu", ["-DOSB_CENTRAL_T=double", "-DOSB_CENTRAL_NAME=central_f64"]),
    ("central_f32", "osb_central.cu", ["-DOSB_CENTRAL_T=float", "-DOSB_CENTRAL_NAME=central_f32"] + FAST),
    ("batch", "osb_batch.cu", FAST),
    ("resident_f64", "osb_resident.cu", ["-DOSB_RESIDENT_T=double", "-DOSB_RESIDENT_NAME=resident_f64"]),
    ("resident_f32", "osb_resident.cu", ["-DOSB_RESIDENT_T=float", "-DOSB_RESIDENT_NAME=resident_f32",
                                          "-DOSB_RESIDENT_F32"] + FAST),
    ("filter_f64", "osb_filter.cu", ["-DOSB_FILTER_T=double", "-DOSB_FILTER_NAME=filter_f64",
                                           "-DOSB_TVD_STALE_NAME=tvd_stale_f64"]),
    ("filter_f32", "osb_filter.cu", ["-DOSB_FILTER_T=float", "-DOSB_FILTER_NAME=filter_f32",
                                          "-DOSB_TVD_STALE_NAME=tvd_stale_f32"] + FAST),
] + [
    ("flux_%s_%dd" % (p, nd), "osb_flux.cu",
     ["-DOSB_T=%s" % ("double" if p == "f64" else "float"), "-DOSB_ND=%d" % nd, "-DOSB_NAME=flux_%s_%dd" % (p, nd)]
     + (FAST if p == "f32" else []))
    for p in ("f64", "f32") for nd in (1, 2, 3)
] + [
    ("flux_curv_%s_%dd" % (p, nd), "osb_flux.cu",
     ["-DOSB_T=%s" % ("double" if p == "f64" else "float"), "-DOSB_ND=%d" % nd, "-DOSB_CURV=true",
      "-DOSB_NAME=flux_curv_%s_%dd" % (p, nd)] + (FAST if p == "f32" else []))
    for p in ("f64", "f32") for nd in (2, 3)
]


def nvcc():
    exe = shutil.which("nvcc")
    if exe is None:
        cand = "/usr/local/cuda/bin/nvcc"
        if os.path.exists(cand):
            return cand
        raise RuntimeError("nvcc not found")
    return exe


def cuda_home():
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(INCLUDE, "osb_gb300.h"))
    files.append(os.path.abspath(__file__))
    return max(os.path.getmtime(f) for f in files)


def build(force=False, jobs=None, verbose=False):
    """Compile every CUDA translation unit for sm_103a and link the shared library."""
    if not force and os.path.exists(LIB) and os.path.exists(PROBE) and os.path.getmtime(LIB) >= _deps():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()

    def compile_unit(u):
        name, src, extra = u
        obj = os.path.join(BUILD, name + ".o")
        cmd = [nv] + ARCH + FLAGS + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr[-4000:]))
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    jobs = jobs or min(len(UNITS) + 1, os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        probe = ex.submit(compile_unit, ("probe", "osb_probe.cu", []))
        objs = list(ex.map(compile_unit, UNITS))
        probe_obj = probe.result()
    link = ["-shared", "-cudart", "shared", "-Xlinker", "-rpath," + os.path.join(cuda_home(), "lib64")]
    subprocess.check_call([nv] + ARCH + link + ["-o", PROBE + ".tmp", probe_obj])
    os.replace(PROBE + ".tmp", PROBE)
    tmp = LIB + ".tmp"
    cmd = [nv] + ARCH + link + ["-o", tmp] + objs
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import time
    t = time.time()
    print(build(force=True, verbose=False), "%.1fs" % (time.time() - t))
