"""Build recipe of the CUDA library libmglet_gpu.so (sm_103a only).

Each translation unit is compiled in parallel with nvcc; the FP64 parity
kernels (plain_*.cu) get -fmad=false so no multiply-add is contracted, the
mixed-precision kernels keep FMA.  The plain flux and Poisson units are
compiled a second time with contraction (-DMG_FMA_BUILD, namespace mg::contract),
the plain form's performance build.  Output goes next to the sources, into
mglet-base_gb300/_build/ (git-ignored), so the library stays in-tree.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)                       # mglet-base_gb300/
CSRC = os.path.join(ROOT, "csrc")
OUT = os.path.join(ROOT, "_build")
LIB = os.path.join(OUT, "libmglet_gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
BASE = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall"]
SOURCES = ["api.cu", "plain_flux.cu", "plain_poisson.cu", "plain_misc.cu", "plain_bound.cu",
           "plain_gc.cu", "plain_level.cu", "mixed.cu", "mixed_flux.cu", "mixed_sip.cu", "noalloc.cu",
           "adjoint.cu", "les.cu", "scalar.cu", "diag.cu", "gc_create.cu", "dist.cu", "mesh_sdf.cu",
           "mixed_level.cu"]
# translation units whose FP64 arithmetic must not be contracted into FMAs
NO_FMA = {"plain_flux.cu", "plain_poisson.cu", "plain_misc.cu", "plain_bound.cu", "plain_gc.cu",
          "plain_level.cu", "noalloc.cu", "les.cu", "scalar.cu"}
# compiled a second time with contraction, into namespace mg::contract (the plain
# form's performance build, MGLET_FORM_PLAIN_FMA)
FMA_TWINS = ["plain_flux.cu", "plain_poisson.cu"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


# translation units with host arithmetic that must not be contracted either
# (the ghost-cell stencil construction)
HOST_NO_FMA = {"gc_create.cu"}


def _flags(src, twin=False):
    f = list(BASE) + ARCH
    if twin:
        f.append("-DMG_FMA_BUILD")
    elif src in NO_FMA:
        f.append("-fmad=false")
    if src in HOST_NO_FMA:
        f += ["-Xcompiler", "-ffp-contract=off"]
    return f


def _needs(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False, extra=None):
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(ROOT), "include", "mglet_gpu.h"))
    jobs = []
    objs = []
    units = [(s, False) for s in SOURCES] + [(s, True) for s in FMA_TWINS]
    for s, twin in units:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OUT, s.replace(".cu", "_fma.o" if twin else ".o"))
        objs.append(obj)
        if force or _needs(obj, [src] + headers):
            cmd = [nvcc()] + _flags(s, twin) + (extra or []) + ["-c", src, "-o", obj]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode != 0:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError("nvcc failed for " + cmd[-3])
    if force or jobs or not os.path.exists(LIB):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
