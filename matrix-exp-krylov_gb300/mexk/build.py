"""Build recipe for the mexk libraries (no cmake).

Produces, under ``matrix-exp-krylov_gb300/_build/``:
  libmexk.so       CUDA kernels + C ABI (nvcc, sm_103a only)
  libmexk_host.so  C++ drop-in API: CSRHost loaders, DeviceContext, ArnoldiRunner
  matrix_exp       drop-in command line program
  csr_tool         loader check tool used by the tests
and builds the oracle (``oracle/_build``; ``oracle/_ref`` when the reference
tree is present). Translation units compile in parallel; a unit is rebuilt
only when a source or header is newer than its object.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ROOT = os.path.dirname(PKG)
INCLUDE = os.path.join(ROOT, "include")
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
OUT = os.path.join(PKG, "_build")
ORACLE = os.path.join(ROOT, "oracle")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-v",
              "--expt-relaxed-constexpr"] + ARCH


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd, log=None):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if log is not None:
        with open(log, "w") as f:
            f.write(" ".join(cmd) + "\n" + p.stdout)
    if p.returncode != 0:
        raise RuntimeError(f"build step failed ({p.returncode}): {' '.join(cmd)}\n{p.stdout[-4000:]}")
    return p.stdout


def have_zlib() -> bool:
    return os.path.exists("/usr/include/zlib.h")


def build_cuda(jobs: int = 8) -> str:
    os.makedirs(OUT, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    objs = []
    todo = []
    for s in srcs:
        o = os.path.join(OUT, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if _newer(o, [s] + headers):
            todo.append((s, o))
    nv = nvcc()

    def comp(so):
        s, o = so
        cmd = [nv] + NVCC_FLAGS + ["-I", INCLUDE, "-I", CSRC, "-c", s, "-o", o]
        _run(cmd, log=o + ".log")

    with cf.ThreadPoolExecutor(max_workers=max(1, jobs)) as ex:
        list(ex.map(comp, todo))
    lib = os.path.join(OUT, "libmexk.so")
    if _newer(lib, objs):
        _run([nv, "-shared"] + ARCH + ["-o", lib] + objs)
    return lib


def build_host() -> None:
    os.makedirs(OUT, exist_ok=True)
    cxx = os.environ.get("CXX", "g++")
    zl = (["-DMEXK_HAVE_ZLIB"], ["-lz"]) if have_zlib() else ([], [])
    hdrs = glob.glob(os.path.join(INCLUDE, "*"))
    host_srcs = [os.path.join(HOST, "csr_host.cpp"), os.path.join(HOST, "arnoldi_runner.cpp")]
    hlib = os.path.join(OUT, "libmexk_host.so")
    base = [cxx, "-O2", "-std=c++17", "-fPIC", "-Wall", "-I", INCLUDE]
    rpath = ["-Wl,-rpath,$ORIGIN", "-L", OUT]
    if _newer(hlib, host_srcs + hdrs + [os.path.join(OUT, "libmexk.so")]):
        _run(base + zl[0] + ["-shared", "-o", hlib] + host_srcs + rpath + ["-lmexk", "-ldl"] + zl[1])
    for name, src in (("matrix_exp", "matrix_exp_main.cpp"), ("csr_tool", "csr_tool.cpp")):
        exe = os.path.join(OUT, name)
        s = os.path.join(HOST, src)
        if _newer(exe, [s, hlib] + hdrs):
            _run(base + ["-o", exe, s] + rpath + ["-lmexk_host", "-lmexk"])


def build_oracle(with_reference: bool | None = None) -> None:
    sys.path.insert(0, ORACLE)
    try:
        import oracle as O  # noqa: WPS433 (test infrastructure build)
    finally:
        sys.path.pop(0)
    O.build(with_reference=with_reference)


def build_all(jobs: int = 8, oracle: bool = True) -> None:
    build_cuda(jobs)
    build_host()
    if oracle:
        build_oracle()


if __name__ == "__main__":
    build_all()
    print("built", OUT)
