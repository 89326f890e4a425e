"""Build libpisces_gb300.so in place (nvcc for sm_103a, g++ for host code).

    python pisces-1_gb300/build.py            # incremental
    python pisces-1_gb300/build.py --force    # rebuild everything

Translation units compile in parallel; objects go to pisces-1_gb300/_build/
(git-ignored) and the library to pisces-1_gb300/libpisces_gb300.so.
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpisces_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

TUNED = os.path.join(HERE, "hx_tuned.tsv")          # launch parameters measured by tune_hx.py
TUNED_INC = os.path.join(BUILD, "pg_hx_tuned.inc")  # the same as C initialisers

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              f"-I{INCLUDE}", f"-I{CSRC}", f"-I{BUILD}", "--expt-relaxed-constexpr"]
# files whose floating-point evaluation order follows the reference exactly
NO_FMA = {"pg_potential.cu", "pg_observables.cu", "pg_dual.cu"}
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", f"-I{INCLUDE}", f"-I{CSRC}"]


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _cuda_home(nvcc):
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def write_tuned_include():
    """hx_tuned.tsv (n, nvec, kind, lag, ctas, form, ...) -> {n, nvec, kind, lag, ctas, form}, lines."""
    rows = []
    if os.path.exists(TUNED):
        with open(TUNED) as f:
            for line in f:
                line = line.strip()
                if not line or line.startswith("#"):
                    continue
                v = line.split()
                rows.append("    {%d, %d, %d, %d, %d, %d}," % tuple(int(x) for x in v[:6]))
    text = "// generated from hx_tuned.tsv by build.py\n" + "\n".join(rows) + ("\n" if rows else "")
    if not os.path.exists(TUNED_INC) or open(TUNED_INC).read() != text:
        with open(TUNED_INC, "w") as f:
            f.write(text)


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _compile(src, force, nvcc):
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + ".o")
    deps = [path] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    deps.append(os.path.join(INCLUDE, "pisces_gb300.h"))
    deps.append(TUNED_INC)
    if not force and os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj, None
    if src.endswith(".cu"):
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", path, "-o", obj]
        if src in NO_FMA:
            cmd.insert(1, "-fmad=false")
    else:
        cmd = ["g++", *CXX_FLAGS, f"-I{_cuda_home(nvcc)}/include", "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, f"{' '.join(cmd)}\n{r.stdout}\n{r.stderr}"
    return obj, None


def build(force: bool = False, verbose: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    write_tuned_include()
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile(s, force, nvcc), sources()))
    errors = [e for _, e in results if e]
    if errors:
        raise RuntimeError("build failed:\n" + "\n".join(errors))
    objs = [o for o, _ in results]
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc, *ARCH, "-shared", "-cudart", "static", "-o", LIB, *objs, "-lpthread", "-lcuda"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            # libcuda is only needed for driver-API entry points; link without it if absent
            cmd = [c for c in cmd if c != "-lcuda"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    try:
        build(force=a.force, verbose=True)
    except RuntimeError as e:
        print(e, file=sys.stderr)
        sys.exit(1)
