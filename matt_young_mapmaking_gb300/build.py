"""Build step of the halo painter: the CUDA shared library (sm_103a), the command-line
drop-ins and, for tests and the CPU baseline, the C oracle.

Everything is compiled in place (no install step) so that the library the tests load is
the one in this tree.  Translation units are compiled in parallel; one -gencode only.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
ORACLE = os.path.join(ROOT, "oracle")
BUILD = os.path.join(PKG, "_build")

LIB = os.path.join(PKG, "libp2m_gb300.so")
ORACLE_LIB = os.path.join(ORACLE, "libp2m_oracle.so")
CLI = os.path.join(PKG, "pks2map")
MAPTABLE_CLI = os.path.join(PKG, "make_maptable")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-I" + CSRC, "-I" + INCLUDE]
CU_SOURCES = ["p2m_kernels.cu", "p2m_capi.cu", "p2m_noalloc.cu", "p2m_spectra.cu"]
CPP_SOURCES = ["p2m_tools.cpp", "p2m_outputs.cpp"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".h")]
    return hs + [os.path.join(INCLUDE, "p2m.h"), os.path.join(INCLUDE, "p2m_tools.h")]


def build_lib(force=False, verbose=False):
    """Compile libp2m_gb300.so for sm_103a."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    deps = [os.path.join(CSRC, s) for s in CU_SOURCES + CPP_SOURCES] + _headers()
    if not force and not _stale(LIB, deps):
        return LIB
    jobs = []
    objs = []
    for s in CU_SOURCES:
        o = os.path.join(BUILD, s + ".o")
        objs.append(o)
        jobs.append([nvcc] + ARCH + NVCC_FLAGS + ["-c", os.path.join(CSRC, s), "-o", o])
    for s in CPP_SOURCES:
        o = os.path.join(BUILD, s + ".o")
        objs.append(o)
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I" + CSRC,
                     "-I" + INCLUDE, "-I/usr/local/cuda/include", "-c",
                     os.path.join(CSRC, s), "-o", o])
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-lpthread"])
    return LIB


def build_cli(force=False):
    """The pks2map and make_maptable executables (link against the library)."""
    deps = [LIB] + _headers()
    for src, exe in (("pks2map_cli.cpp", CLI), ("make_maptable_cli.cpp", MAPTABLE_CLI)):
        path = os.path.join(CSRC, src)
        if not os.path.exists(path):
            continue
        if not force and not _stale(exe, deps + [path]):
            continue
        _run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I" + CSRC, "-I" + INCLUDE,
              path, "-o", exe, "-L" + PKG, "-lp2m_gb300", "-Wl,-rpath,$ORIGIN", "-pthread"])
    return CLI


def build_oracle(force=False):
    """The C oracle (test infrastructure): plain C, no FMA contraction, OpenMP threads."""
    src = os.path.join(ORACLE, "p2m_oracle.c")
    deps = [src, os.path.join(ORACLE, "p2m_oracle.h"), os.path.join(CSRC, "p2m_fmath.h")]
    if not force and not _stale(ORACLE_LIB, deps):
        return ORACLE_LIB
    _run(["gcc", "-O2", "-std=c11", "-D_POSIX_C_SOURCE=200809L", "-ffp-contract=off",
          "-fno-fast-math", "-fopenmp", "-fPIC", "-shared", src, "-o", ORACLE_LIB, "-lm"])
    return ORACLE_LIB


def build_all(force=False, verbose=False):
    with ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_lib, force, verbose)
        f2 = ex.submit(build_oracle, force)
        f1.result()
        f2.result()
    build_cli(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print("built", LIB)
