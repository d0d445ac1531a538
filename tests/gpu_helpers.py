"""Shared helpers for the GPU parity tests."""
import numpy as np
import pytest

from oracle.pyoracle import raster_config
from streamsim_gb300 import facetcu


def require_gpu():
    if facetcu.device_count() == 0:
        pytest.fail("GPU test run without a CUDA device")


def model_for(vertices, raster, layers, bounds=None, periodic=(0, 1.0, 1.0)):
    m = facetcu.FacetrtCuda()
    m.initialize(raster, raster, layers, 0, periodic[0], periodic[1], periodic[2])
    m.setGeometry(vertices)
    if bounds is not None:
        m.setRasterBounds(*bounds)
    return m


def oracle_cfg(vertices, raster, layers, bounds=None, periodic=(0, 1.0, 1.0)):
    if bounds is None:
        p = np.asarray(vertices, np.float32).reshape(-1, 6)[:, :3]
        bounds = (p.min(0), p.max(0))
    return raster_config(raster, layers, bounds[0], bounds[1], *periodic)


def graphs_equal(gpu_graph, oracle_graph):
    rows, nb, cnt, den, sky = gpu_graph
    o = oracle_graph
    for name, a, b in (("row_offsets", rows, o.row_offsets), ("neighbors", nb, o.neighbors),
                       ("counts", cnt, o.counts), ("denominators", den, o.denominators),
                       ("sky_counts", sky, o.sky_counts)):
        if not np.array_equal(a, b):
            return name
    return None


def rel_err(a, b, floor=1e-6):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = max(np.max(np.abs(b)), 1e-30)
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), floor * scale))
