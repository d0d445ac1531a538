"""facetcu_solve_noalloc: the reference-semantics solve for callers that
cannot allocate device memory (hosts that own the device-memory budget and
hand it out from their own pool, or loops that must not pay cudaMalloc's
implicit synchronisation).  It must give the same radiosity as
facetcu_solve on the same graph and optics, call after call, although every
call reuses the library's one fixed scratch array.  The test allocates the
inputs and outputs itself (through PyTorch) and hands the entry point device
pointers.  This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from streamsim_gb300 import facetcu, scenes
from tests.gpu_helpers import rel_err, require_gpu

pytestmark = pytest.mark.gpu


def _device(torch, a, dtype):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dtype=dtype, device="cuda")


def test_noalloc_matches_solve_on_two_calls_in_a_row():
    require_gpu()
    torch = pytest.importorskip("torch")
    sc = scenes.config1(seed=6, leaves=800, grid=16)
    m = facetcu.FacetrtCuda()
    m.initialize(256, 256, 64)
    m.setGeometry(sc.vertices)
    m.buildVisibilityGraph(scenes.hemisphere_directions())
    sun = scenes.sun_direction(30, 135)
    lit = m.computeSunlitFraction(sun)
    rows, nb, cnt, den, sky = m.graph()
    S = len(den)
    edges = np.empty(2 * len(nb), np.uint32)
    edges[0::2], edges[1::2] = nb, cnt
    d_rows = _device(torch, rows.view(np.int32), torch.int32)
    d_edges = _device(torch, edges.view(np.int32), torch.int32)
    d_den = _device(torch, den.view(np.int32), torch.int32)
    d_sky = _device(torch, sky.view(np.int32), torch.int32)
    d_out = torch.full((S,), 123.0, dtype=torch.float32, device="cuda")  # stale contents
    lib = facetcu.load()

    optics_a = scenes.reference_optics(sc, lit, sun)
    optics_b = optics_a.copy()
    optics_b[:, 3] = 0.0                      # diffuse-only: a different problem
    optics_b[:, 0] *= 0.5
    # an even and an odd sweep count: the caller's buffer ends as either half
    # of the ping-pong pair
    for optics, sky_r, iterations in ((optics_a, 100.0, 64), (optics_b, 80.0, 37)):
        expected = m.solve(optics, sky_r, iterations, 1.0)
        d_optics = _device(torch, optics, torch.float32)
        torch.cuda.synchronize()
        md = C.c_float(-1.0)
        rc = lib.facetcu_solve_noalloc(
            C.c_void_p(d_rows.data_ptr()), C.c_void_p(d_edges.data_ptr()),
            C.c_void_p(d_den.data_ptr()), C.c_void_p(d_sky.data_ptr()), S,
            C.c_void_p(d_optics.data_ptr()), sky_r, iterations, 1.0,
            C.c_void_p(d_out.data_ptr()), C.byref(md), None)
        assert rc == facetcu.OK
        got = d_out.cpu().numpy()
        # same kernel and summation order as facetcu_solve: equal within the
        # solve tests' tolerance (1e-5), in practice bit for bit
        assert rel_err(got, expected["radiosity"]) < 1e-5
        assert md.value == pytest.approx(expected["maxDelta"], rel=1e-5, abs=1e-6)
    m.close()


def test_noalloc_rejects_sizes_beyond_its_array():
    lib = facetcu.load()
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = lib.facetcu_solve_noalloc(dummy, dummy, dummy, dummy,
                                   facetcu.NOALLOC_MAX_SURFACES + 2, dummy, 100.0, 8, 1.0,
                                   dummy, None, None)
    assert rc == facetcu.OVERFLOW_ERROR
    rc = lib.facetcu_solve_noalloc(dummy, dummy, dummy, dummy, 8, dummy, 100.0,
                                   facetcu.NOALLOC_MAX_ITERATIONS + 1, 1.0, dummy, None, None)
    assert rc == facetcu.INVALID_ARGUMENT
