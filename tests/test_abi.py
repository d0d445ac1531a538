"""The C-ABI library loads, exports include/facetcu.h, and rejects bad calls
without a GPU (no compute is attempted here)."""
import ctypes as C

import numpy as np
import pytest

from streamsim_gb300 import facetcu


def test_library_exports_every_header_symbol(lib):
    names = facetcu.header_symbols()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert missing == []


def test_python_binding_covers_header():
    bound = set(facetcu.SIGNATURES) | set(facetcu.OPTIONAL_SIGNATURES)
    assert set(facetcu.header_symbols()) <= bound


def test_struct_layouts_match_reference_pods():
    # facetvk::Vertex 24 B, Direction 12 B, SurfaceOptics 16 B, CsrEdge 8 B,
    # Config 36 B (bool padded to 4), GraphDiagnostics 24 B
    assert C.sizeof(facetcu.Vertex) == 24
    assert C.sizeof(facetcu.Direction) == 12
    assert C.sizeof(facetcu.SurfaceOptics) == 16
    assert C.sizeof(facetcu.Config) == 36
    assert facetcu.Config.gpu_index.offset == 20
    assert C.sizeof(facetcu.GraphDiagnostics) == 24


def test_call_order_and_arguments_without_gpu(lib):
    h = C.c_void_p()
    assert lib.facetcu_create(C.byref(h)) == facetcu.OK
    try:
        # every call before initialize() is a logic error (facetrt_vulkan.cpp:447)
        v = np.zeros((3, 6), np.float32)
        assert lib.facetcu_set_geometry(h, v.ctypes.data, 3) == facetcu.LOGIC_ERROR
        assert b"initialize()" in lib.facetcu_last_error(h)
        d = facetcu.GraphDiagnostics()
        dirs = np.ones((1, 3), np.float32)
        assert lib.facetcu_build_visibility_graph(h, dirs.ctypes.data, 1, C.byref(d)) == facetcu.LOGIC_ERROR
        # invalid config is rejected before any device work
        cfg = facetcu.Config()
        cfg.raster_width = 0
        cfg.raster_height = 16
        cfg.max_fragments_per_pixel = 8
        assert lib.facetcu_initialize(h, C.byref(cfg)) == facetcu.INVALID_ARGUMENT
        assert b"Raster dimensions" in lib.facetcu_last_error(h)
        cfg.raster_width = 16
        cfg.max_fragments_per_pixel = 0
        assert lib.facetcu_initialize(h, C.byref(cfg)) == facetcu.INVALID_ARGUMENT
        # a valid config on a machine without a GPU reports NO_DEVICE
        if facetcu.device_count() == 0:
            cfg.max_fragments_per_pixel = 8
            assert lib.facetcu_initialize(h, C.byref(cfg)) == facetcu.NO_DEVICE
    finally:
        lib.facetcu_release(h)


def test_null_context_is_rejected(lib):
    assert lib.facetcu_destroy(None) == facetcu.INVALID_ARGUMENT
    assert lib.facetcu_create(None) == facetcu.INVALID_ARGUMENT


def test_host_direction_helpers_match_reference(oracle, reference):
    """makeHemisphereDirections / sunDirection (facetrtcore.cpp:475-498) of the
    library's C++ host code round exactly like the reference's."""
    d = facetcu.hemisphere_directions(40)
    assert np.array_equal(d.view(np.uint32), reference.hemisphere_directions().view(np.uint32))
    assert np.array_equal(d.view(np.uint32), oracle.hemisphere_directions().view(np.uint32))
    for zen, az in [(30, 135), (0, 0), (75, 290), (45.5, 12.25), (89.9, 359.0)]:
        assert np.array_equal(facetcu.sun_direction(zen, az).view(np.uint32),
                              reference.sun_direction(zen, az).view(np.uint32))


def test_cpp_wrapper_compiles_and_maps_errors(tmp_path, lib):
    """include/facetcu.hpp keeps the reference's exception classes."""
    import os
    import shutil
    import subprocess
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    exe = tmp_path / "wrapper_check"
    libdir = os.path.join(root, "streamsim_gb300")
    subprocess.run(["g++", "-std=c++17", "-I", os.path.join(root, "include"),
                    os.path.join(root, "tests", "cpp", "wrapper_check.cpp"), "-L", libdir,
                    "-lfacetcu", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def _build_module_check(tmp_path):
    import os
    import shutil
    import subprocess
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    exe = tmp_path / "module_check"
    libdir = os.path.join(root, "streamsim_gb300")
    subprocess.run(["g++", "-std=c++17", "-I", os.path.join(root, "include"),
                    os.path.join(root, "tests", "cpp", "module_check.cpp"), "-L", libdir,
                    "-lfacetcu", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    return str(exe)


def test_module_seam_readiness_chain(tmp_path, lib):
    """include/facetcu_module.hpp: the reference's Facetrt / FacetrtIO
    (facetrt.h:14-29, facetrtio.h:7-21) and its readiness flags, no run."""
    import subprocess
    r = subprocess.run([_build_module_check(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0 and "module seam ok" in r.stdout, r.stdout + r.stderr
