"""Build libfacetcu.so (CUDA, sm_103a) in-tree with nvcc.

Translation units are compiled in parallel and linked into
streamsim_gb300/libfacetcu.so.  raster.cu, hemi.cu, lbvh.cu, spectral.cu, energy.cu and image.cu are compiled with
-fmad=false because their float results must round exactly like the
reference's CPU code (no fused multiply-add); host code is compiled with
-ffp-contract=off for the same reason.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfacetcu.so")
CLI_SRC = os.path.join(HERE, "cli", "facetcu_main.cpp")
CLI = os.path.join(HERE, "facetcu")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
EXACT_FP = {"raster.cu", "hemi.cu", "lbvh.cu", "spectral.cu", "energy.cu", "image.cu"}


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libfacetcu")
    return path


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _compile(src):
    obj = os.path.join(BUILD, src + ".o")
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
           "-I", os.path.join(HERE, "..", "include"), "-c", os.path.join(CSRC, src), "-o", obj]
    if src in EXACT_FP:
        cmd.insert(1, "-fmad=false")
    if src.endswith(".cpp"):
        cmd[cmd.index("-c")] = "-x"
        cmd.insert(cmd.index("-x") + 1, "c++")
        cmd.insert(cmd.index("c++") + 1, "-c")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    return obj


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "facetcu.h"))
    deps.append(os.path.abspath(__file__))
    deps.append(CLI_SRC)
    if not os.path.exists(CLI) or os.path.getmtime(CLI) < t:
        return True
    return any(os.path.getmtime(d) > t for d in deps)


def build_cli():
    """The `facetcu` executable (the eFacetRT process seam), linked to
    libfacetcu.so next to it."""
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-std=c++17", "-O2", "-I", os.path.join(HERE, "..", "include"), CLI_SRC,
           "-L", HERE, "-lfacetcu", "-Wl,-rpath,$ORIGIN", "-o", CLI + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"CLI build failed:\n{r.stderr}")
    os.replace(CLI + ".tmp", CLI)
    return CLI


def build(force=False, jobs=None):
    """Compile every translation unit for sm_103a and link libfacetcu.so."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, srcs))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    build_cli()
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
