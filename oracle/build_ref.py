#!/usr/bin/env python3
"""Build recipe for oracle/_ref — TEST INFRASTRUCTURE ONLY.

Compiles the reference's own CPU FacetRT backend (StreamSim HiStream,
models/histream/src/facetrt/facetrtcore.cpp) into oracle/_ref/libfacetrt_ref.so
so that the C restatement in oracle/facet_oracle.c can be pinned against it.

The reference file also holds a Vulkan driver, a GDAL texture loader and a
JSON project loader that need libraries absent here, so the recipe takes the
self-contained CPU span by line range (the same ranges on every run, checked
against anchor lines first), wraps it in the reference header's POD types and
appends the extern "C" wrappers of oracle/ref_shim.inc:

    facetrt_vulkan.h   15-62     Vertex, Direction, SurfaceOptics, Config,
                                 GraphDiagnostics, SolveResult
    facetrtcore.cpp    39-53     Clock/Vec3 aliases
    facetrtcore.cpp    74-630    constants, Scene, geometry, optics helpers
    facetrtcore.cpp    703-1620  CpuRasterizer .. runCpu (with the FacetEB
                                 helpers: latent heat, storage, energy optics)
    facetrtcore.cpp    2458-2497 ShortwaveSpectrum (FacetEB's window integrals)

Everything generated goes to oracle/_ref/ (git-ignored).  The generated
source travels with the repository snapshot, so on a machine without the
reference tree `python oracle/build_ref.py` recompiles it from there.

It is compiled with -ffp-contract=off: the shipped Windows build does not
fuse multiply-adds, and GCC on aarch64 would otherwise fuse them.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SRC = os.path.join(OUT, "facetrt_ref.cpp")
LIB = os.path.join(OUT, "libfacetrt_ref.so")
# The reference tree this recipe compiles from: the one place its path is
# named (tests and the fixture script import it); FACETRT_REFERENCE_ROOT
# overrides it.  Where it is absent the backend is compiled from the extract
# an earlier run generated into oracle/_ref (it travels with the repository
# snapshot), and the tree-only checkers are skipped.
REFERENCE = os.environ.get("FACETRT_REFERENCE_ROOT", "/root/reference")
FACETRT = os.path.join(REFERENCE, "models", "histream", "src", "facetrt")
BASE = os.path.join(REFERENCE, "models", "histream", "src", "base")
PROJECT_SRC = os.path.join(OUT, "project_ref.cpp")
PROJECT_LIB = os.path.join(OUT, "libproject_ref.so")

RANGES = [
    ("facetrt_vulkan.h", 15, 62, "namespace facetvk {", "}"),
    ("facetrtcore.cpp", 39, 53, "namespace {", None),
    ("facetrtcore.cpp", 74, 630, None, None),
    ("facetrtcore.cpp", 703, 1620, None, None),
    ("facetrtcore.cpp", 2458, 2497, None, "}  // namespace"),
]
# (file, line, text the line must start with) — guards against a different
# revision of the reference.
ANCHORS = [
    ("facetrt_vulkan.h", 15, "struct Vertex {"),
    ("facetrt_vulkan.h", 62, "};"),
    ("facetrtcore.cpp", 39, "using Clock"),
    ("facetrtcore.cpp", 74, "constexpr float kPi"),
    ("facetrtcore.cpp", 1212, "class CpuRasterizer"),
    ("facetrtcore.cpp", 1348, "CpuGraph buildCpuGraph("),
    ("facetrtcore.cpp", 1438, "std::vector<float> computeCpuSunlit("),
    ("facetrtcore.cpp", 1476, "facetvk::SolveResult solveCpu("),
    ("facetrtcore.cpp", 1585, "RunResult runCpu("),
    ("facetrtcore.cpp", 1621, "RunResult runGpu("),
    ("facetrtcore.cpp", 631, "std::shared_ptr<const ReflectanceVarianceTexture> loadReflectanceVarianceTexture("),
    ("facetrtcore.cpp", 2458, "struct ShortwaveSpectrum {"),
    ("facetrtcore.cpp", 2497, "};"),
]
PRELUDE = """// GENERATED by oracle/build_ref.py from the reference tree. Not product
// code and not committed: test infrastructure for parity checks only.
#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <filesystem>
#include <fstream>
#include <functional>
#include <iomanip>
#include <iostream>
#include <limits>
#include <memory>
#include <mutex>
#include <numeric>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <unordered_map>
#include <utility>
#include <vector>
"""


def _lines(name):
    with open(os.path.join(FACETRT, name), encoding="utf-8") as f:
        return f.read().split("\n")


def generate():
    cache = {}
    for name, line, text in ANCHORS:
        lines = cache.setdefault(name, _lines(name))
        if not lines[line - 1].lstrip().startswith(text):
            raise SystemExit(f"build_ref: {name}:{line} does not start with {text!r}; "
                             "the reference revision differs from the one this recipe expects")
    parts = [PRELUDE]
    for name, lo, hi, before, after in RANGES:
        lines = cache.setdefault(name, _lines(name))
        if before:
            parts.append(before)
        parts.append(f"// ---- {name}:{lo}-{hi}")
        parts.extend(lines[lo - 1:hi])
        if after:
            parts.append(after)
    with open(os.path.join(HERE, "ref_shim.inc"), encoding="utf-8") as f:
        parts.append(f.read())
    os.makedirs(OUT, exist_ok=True)
    with open(SRC, "w", encoding="utf-8") as f:
        f.write("\n".join(parts) + "\n")


def compile_lib():
    cmd = ["g++", "-O2", "-std=c++20", "-ffp-contract=off", "-fPIC", "-shared",
           "-w", SRC, "-o", LIB]
    subprocess.run(cmd, check=True)


# The project loader (loadProjectScene, facetrtcore.cpp:2038-3025, for the
# reference's XML input) with the CPU span it builds on and the spectral
# models it calls (Compo::resolveSpectrals with fluspect and bsm,
# compo.cpp; Utils::expint, utils.cpp; their types from structs.h and
# structs_cg.h).  GDAL is not available here: oracle/ref_project_stubs.inc
# declares a stand-in that opens ESRI ASCII grids (DEM and texture files in
# that format), and one for the project.json view (nlohmann::json) that
# fails loudly.
PROJECT_RANGES = [
    ("base/structs.h", 122, 128, None, None),
    ("base/structs.h", 148, 186, None, None),
    ("base/structs.h", 195, 206, None, None),
    ("base/structs_cg.h", 45, 48, None, None),
    ("@", 0, 0, "declarations", None),
    ("base/utils.cpp", 459, 471, None, None),
    ("base/compo.cpp", 15, 90, None, None),
    ("base/compo.cpp", 152, 341, None, None),
    ("base/compo.cpp", 436, 479, None, None),
    ("facetrt/facetrt_vulkan.h", 15, 62, "namespace facetvk {", "}"),
    ("facetrt/facetrtcore.cpp", 39, 53, "namespace {", None),
    ("facetrt/facetrtcore.cpp", 74, 630, None, None),
    ("facetrt/facetrtcore.cpp", 631, 702, None, None),
    ("facetrt/facetrtcore.cpp", 703, 1620, None, None),
    ("@", 0, 0, "view", None),
    ("facetrt/facetrtcore.cpp", 2038, 3025, None, "}  // namespace"),
]
PROJECT_ANCHORS = [
    ("base/structs.h", 122, "enum class spectralType"),
    ("base/structs.h", 148, "struct OptCoeff"),
    ("base/structs.h", 195, "struct SpectralXml"),
    ("base/structs_cg.h", 45, "struct  Spectral{"),
    ("base/utils.cpp", 459, "float Utils::expint(float x)"),
    ("base/compo.cpp", 15, "namespace {"),
    ("base/compo.cpp", 152, "float Compo::calctav(float alfa,float nr)"),
    ("base/compo.cpp", 275, "std::vector<Spectral> Compo::resolveSpectrals("),
    ("base/compo.cpp", 436, "void Compo::bsm(OptCoeff bsmCoeff,BSMParam bsm,std::vector<Spectral>& spectrals){"),
    ("facetrt/facetrtcore.cpp", 631,
     "std::shared_ptr<const ReflectanceVarianceTexture> loadReflectanceVarianceTexture("),
    ("facetrt/facetrtcore.cpp", 2038, "std::string readTextFile(const std::string& path)"),
    ("facetrt/facetrtcore.cpp", 2880, "Scene loadProjectScene(const std::string& inputFile)"),
    ("facetrt/facetrtcore.cpp", 3025, "}"),
]


def generate_project():
    src = os.path.join(REFERENCE, "models", "histream", "src")
    read = lambda name: open(os.path.join(src, name), encoding="utf-8").read().split("\n")
    cache = {}
    for name, line, text in PROJECT_ANCHORS:
        lines = cache.setdefault(name, read(name))
        if not lines[line - 1].lstrip().startswith(text):
            raise SystemExit(f"build_ref: {name}:{line} does not start with {text!r}")
    with open(os.path.join(HERE, "ref_project_stubs.inc"), encoding="utf-8") as f:
        stubs = f.read()
    sections = {}
    current = None
    for line in stubs.split("\n"):
        if line.startswith("//@@ "):
            current = line[5:].strip()
            sections[current] = []
        elif current:
            sections[current].append(line)
    parts = [PRELUDE, "#define N1 2001"]
    for name, lo, hi, before, after in PROJECT_RANGES:
        if name == "@":
            parts.extend(sections[before])
            continue
        lines = cache.setdefault(name, read(name))
        if before:
            parts.append(before)
        parts.append(f"// ---- {name}:{lo}-{hi}")
        parts.extend(lines[lo - 1:hi])
        if after:
            parts.append(after)
    with open(os.path.join(HERE, "ref_project_shim.inc"), encoding="utf-8") as f:
        parts.append(f.read())
    os.makedirs(OUT, exist_ok=True)
    with open(PROJECT_SRC, "w", encoding="utf-8") as f:
        f.write("\n".join(parts) + "\n")


def compile_project():
    cmd = ["g++", "-O2", "-std=c++20", "-ffp-contract=off", "-fPIC", "-shared",
           "-w", PROJECT_SRC, "-o", PROJECT_LIB]
    subprocess.run(cmd, check=True)


# The sun of a FacetEB node: the reference's vendored SPA
# (thirdparty/spa.cpp, compiled where it lies) under runFacetEBCore's
# MeteoStep and updateSolarPosition (facetrtcore.cpp:3172-3181, 3290-3327)
# and the Utils date helpers they call (utils.cpp:572-632).
SPA_SRC = os.path.join(OUT, "spa_ref.cpp")
SPA_LIB = os.path.join(OUT, "libspa_ref.so")
THIRDPARTY = os.path.join(REFERENCE, "models", "histream", "src", "thirdparty")
SPA_RANGES = [
    ("@", 0, 0, "declarations", None),
    ("base/utils.cpp", 572, 632, None, None),
    ("@", 0, 0, "open", None),
    ("facetrt/facetrtcore.cpp", 3172, 3181, None, None),
    ("facetrt/facetrtcore.cpp", 3290, 3327, None, None),
    ("@", 0, 0, "close", None),
]
SPA_ANCHORS = [
    ("base/utils.cpp", 572, "double Utils::calculateDeltaT(int year, int month) {"),
    ("base/utils.cpp", 611, "bool Utils::isLeapYear(int year) {"),
    ("base/utils.cpp", 615, "void Utils::calculateMonthAndDay(int kyear, int kdoy, int *kmonth"),
    ("base/utils.cpp", 632, "}"),
    ("facetrt/facetrtcore.cpp", 3172, "struct MeteoStep {"),
    ("facetrt/facetrtcore.cpp", 3290, "const auto updateSolarPosition = [&](const MeteoStep& step) {"),
    ("facetrt/facetrtcore.cpp", 3327, "};"),
]


def _sections(name):
    with open(os.path.join(HERE, name), encoding="utf-8") as f:
        text = f.read()
    sections, current = {}, None
    for line in text.split("\n"):
        if line.startswith("//@@ "):
            current = line[5:].strip()
            sections[current] = []
        elif current:
            sections[current].append(line)
    return sections


def generate_spa():
    src = os.path.join(REFERENCE, "models", "histream", "src")
    read = lambda name: open(os.path.join(src, name), encoding="utf-8").read().split("\n")
    cache = {}
    for name, line, text in SPA_ANCHORS:
        lines = cache.setdefault(name, read(name))
        if not lines[line - 1].lstrip().startswith(text):
            raise SystemExit(f"build_ref: {name}:{line} does not start with {text!r}")
    sections = _sections("ref_spa_shim.inc")
    parts = [PRELUDE]
    for name, lo, hi, before, _ in SPA_RANGES:
        if name == "@":
            parts.extend(sections[before])
            continue
        parts.append(f"// ---- {name}:{lo}-{hi}")
        parts.extend(cache.setdefault(name, read(name))[lo - 1:hi])
    os.makedirs(OUT, exist_ok=True)
    with open(SPA_SRC, "w", encoding="utf-8") as f:
        f.write("\n".join(parts) + "\n")


def compile_spa():
    cmd = ["g++", "-O2", "-std=c++20", "-ffp-contract=off", "-fPIC", "-shared", "-w",
           "-I", THIRDPARTY, SPA_SRC, os.path.join(THIRDPARTY, "spa.cpp"), "-o", SPA_LIB]
    subprocess.run(cmd, check=True)


def main():
    if os.path.isdir(FACETRT):
        generate()
        # the project loader and solar-position oracles are used by CPU
        # tests only, here
        generate_project()
        compile_project()
        generate_spa()
        compile_spa()
    elif not os.path.exists(SRC):
        print("build_ref: reference tree absent and no generated source; skipping",
              file=sys.stderr)
        return 0
    compile_lib()
    print(LIB)
    return 0


if __name__ == "__main__":
    sys.exit(main())
