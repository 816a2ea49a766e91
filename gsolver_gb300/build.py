"""Build libgsolver_gb300.so in-tree (gsolver_gb300/_build/) with nvcc for sm_103a.

Every .cu under csrc/ (and every .cpp under csrc/host/) is compiled in parallel, then
linked into one shared library exporting the C ABI of include/gs_abi.h.  Used by
__graft_entry__.build(); also runnable as ``python -m gsolver_gb300.build``.

``--check`` (build(check=True)) builds the GS_CHECK variant into gsolver_gb300/_build_check/:
the hot kernels test their table-driven indices before each access and report a failure as a
status (gs_check_build, gs_selftest_bounds); the package loads it when GS_CHECK=1 is set in
the environment at import.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libgsolver_gb300.so")
OUT_CHECK = os.path.join(HERE, "_build_check")
LIB_CHECK = os.path.join(OUT_CHECK, "libgsolver_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
              "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include")]


def _nvcc():
    n = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(n):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build gsolver_gb300")
    return n


def sources():
    cu = sorted(glob.glob(os.path.join(HERE, "csrc", "*.cu")))
    cpp = sorted(glob.glob(os.path.join(HERE, "csrc", "host", "*.cpp")))
    return cu, cpp


def _deps():
    return sorted(glob.glob(os.path.join(HERE, "csrc", "**", "*"), recursive=True)) + \
        [os.path.join(ROOT, "include", "gs_abi.h"), os.path.abspath(__file__)]


def up_to_date(lib=LIB):
    if not os.path.exists(lib):
        return False
    t = os.path.getmtime(lib)
    return all(os.path.getmtime(d) <= t for d in _deps() if os.path.isfile(d))


def build(force=False, verbose=False, check=False):
    out, lib = (OUT_CHECK, LIB_CHECK) if check else (OUT, LIB)
    if not force and up_to_date(lib):
        return lib
    os.makedirs(out, exist_ok=True)
    nvcc = _nvcc()
    cu, cpp = sources()
    flags = NVCC_FLAGS + (["-DGS_CHECK=1"] if check else [])
    jobs = []
    for s in cu:
        o = os.path.join(out, os.path.basename(s) + ".o")
        jobs.append([nvcc] + ARCH + flags + ["-c", s, "-o", o])
    for s in cpp:
        o = os.path.join(out, "host_" + os.path.basename(s) + ".o")
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
                     "-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, file=sys.stderr)
        return cmd[-1]

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(run, jobs))
    tmp = lib + ".tmp"
    run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcuda", "-lpthread"])
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, check="--check" in sys.argv))
