"""Build the CUDA engine (libmytrim_gpu.so) in-tree for sm_103a.

Every translation unit is compiled in parallel with nvcc, then linked into
``mytrim_gb300/_lib/libmytrim_gpu.so``.  The FP64 engine is compiled with
``-fmad=false`` so that its multiplies and adds round exactly like the host
replay build of the same source; the FP32 engine uses fast single-precision
intrinsics.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
OUT_DIR = PKG / "_lib"
OBJ_DIR = PKG / "_build"
LIB_NAME = "libmytrim_gpu.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# (source, extra flags)
UNITS = [
    ("mtg_engine64.cu", ["-fmad=false"]),
    ("mtg_engine32.cu", ["--use_fast_math"]),
    ("mtg_surrogate.cu", ["--use_fast_math"]),
    ("mtg_reduce.cu", []),
    ("mtg_api.cu", []),
    ("mtg_noalloc.cu", []),
    ("mtg_setup.cpp", []),
]


def nvcc_path():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def lib_path():
    return OUT_DIR / LIB_NAME


def _compile(unit, flags, nvcc, verbose):
    src = CSRC / unit
    obj = OBJ_DIR / (unit + ".o")
    # host code: no FMA contraction, so the tables built on the host are the same bits
    # on x86 and on Arm (where g++ contracts a*b+c by default) and in the host replay
    cmd = [nvcc, *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
           f"-I{INCLUDE}", f"-I{CSRC}", *flags, "-c", str(src), "-o", str(obj)]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose=False, force=False):
    """Compile and link libmytrim_gpu.so; returns its path."""
    srcs = [CSRC / u for u, _ in UNITS if (CSRC / u).exists()]
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    out = lib_path()
    if not force and out.exists():
        newest = max(p.stat().st_mtime for p in srcs + headers + [Path(__file__)])
        if out.stat().st_mtime >= newest:
            build_frontend()
            return out
    OUT_DIR.mkdir(exist_ok=True)
    OBJ_DIR.mkdir(exist_ok=True)
    nvcc = nvcc_path()
    units = [(u, f) for u, f in UNITS if (CSRC / u).exists()]
    with ThreadPoolExecutor(max_workers=min(8, len(units))) as ex:
        results = list(ex.map(lambda uf: _compile(uf[0], uf[1], nvcc, verbose), units))
    objs = [str(o) for o, _ in results]
    tmp = out.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", str(tmp), *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)
    if verbose:
        for (u, _), (_, log) in zip(units, results):
            sys.stderr.write(f"== {u}\n{log}")
    build_frontend(force=True)
    return out


FRONTENDS = ("runmytrim_gpu", "runstopping_gpu")


def frontend_path(name="runmytrim_gpu"):
    return OUT_DIR / name


def build_frontend(force=False, name=None):
    """Compile the command-line front-ends (host C++ over the C ABI) next to the
    library: runmytrim_gpu and runstopping_gpu.  Returns the path of `name`
    (default runmytrim_gpu)."""
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    for fe in FRONTENDS:
        exe = frontend_path(fe)
        src = PKG / "cpp" / f"{fe}.cpp"
        deps = [src, PKG / "cpp" / "json_lite.h", INCLUDE / "mytrim_gpu.h", lib_path()]
        if not force and exe.exists() and exe.stat().st_mtime >= max(p.stat().st_mtime for p in deps):
            continue
        tmp = exe.with_suffix(".tmp")
        cmd = [cxx, "-O2", "-std=c++17", f"-I{INCLUDE}", f"-I{PKG / 'cpp'}", "-o", str(tmp), str(src),
               f"-L{OUT_DIR}", "-lmytrim_gpu", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"{fe} build failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, exe)
    return frontend_path(name or "runmytrim_gpu")


if __name__ == "__main__":
    p = build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(p)
