"""ctypes bindings of the CPU oracle — TEST INFRASTRUCTURE ONLY.

`Oracle` wraps oracle/facet_oracle.c (the C restatement); `Reference` wraps
oracle/_ref/libfacetrt_ref.so (the reference's own CPU functions, compiled by
oracle/build_ref.py).  Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg use this module; the product never does.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SRC = os.path.join(HERE, "facet_oracle.c")
ORACLE_LIB = os.path.join(HERE, "liborc.so")
REF_LIB = os.path.join(HERE, "_ref", "libfacetrt_ref.so")

u32p = C.POINTER(C.c_uint32)
f32p = C.POINTER(C.c_float)
f64p = C.POINTER(C.c_double)


def build_oracle(force=False):
    """Compile the C restatement (gcc, -ffp-contract=off)."""
    if force or not os.path.exists(ORACLE_LIB) or \
            os.path.getmtime(ORACLE_LIB) < max(os.path.getmtime(ORACLE_SRC),
                                                 os.path.getmtime(os.path.join(HERE, "facet_oracle.h"))):
        subprocess.run(["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fPIC", "-shared",
                        "-pthread", ORACLE_SRC, "-o", ORACLE_LIB, "-lm"], check=True)
    return ORACLE_LIB


def build_reference():
    subprocess.run(["python3", os.path.join(HERE, "build_ref.py")], check=True,
                   stdout=subprocess.DEVNULL)
    return REF_LIB if os.path.exists(REF_LIB) else None


class OrcDirection(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class OrcGraph(C.Structure):
    _fields_ = [("surface_count", C.c_uint32), ("nnz", C.c_uint64),
                ("row_offsets", u32p), ("neighbors", u32p), ("counts", u32p),
                ("denominators", u32p), ("sky_counts", u32p),
                ("fragment_overflow", C.c_uint32), ("max_depth", C.c_uint32),
                ("max_closure_error", C.c_float)]


class OrcRasterConfig(C.Structure):
    _fields_ = [("raster_size", C.c_uint32), ("layers", C.c_uint32),
                ("periodic_count", C.c_uint32), ("periodic_size_x", C.c_float),
                ("periodic_size_z", C.c_float), ("bounds_min", C.c_float * 3),
                ("bounds_max", C.c_float * 3)]


def _ptr(a, t):
    return a.ctypes.data_as(t)


class Graph:
    """Count-form graph as numpy arrays (rows sorted by neighbour)."""

    def __init__(self, row_offsets, neighbors, counts, denominators, sky_counts,
                 fragment_overflow=0, max_closure_error=0.0, max_depth=0):
        self.row_offsets = np.ascontiguousarray(row_offsets, dtype=np.uint32)
        self.neighbors = np.ascontiguousarray(neighbors, dtype=np.uint32)
        self.counts = np.ascontiguousarray(counts, dtype=np.uint32)
        self.denominators = np.ascontiguousarray(denominators, dtype=np.uint32)
        self.sky_counts = np.ascontiguousarray(sky_counts, dtype=np.uint32)
        self.fragment_overflow = int(fragment_overflow)
        self.max_closure_error = float(max_closure_error)
        self.max_depth = int(max_depth)

    @property
    def surface_count(self):
        return len(self.denominators)

    @property
    def nnz(self):
        return len(self.neighbors)

    def sorted_rows(self):
        """Return a copy whose rows are sorted by neighbour."""
        rows = np.repeat(np.arange(self.surface_count, dtype=np.int64),
                         np.diff(self.row_offsets.astype(np.int64)))
        order = np.lexsort((self.neighbors, rows))
        return Graph(self.row_offsets, self.neighbors[order], self.counts[order],
                     self.denominators, self.sky_counts, self.fragment_overflow,
                     self.max_closure_error, self.max_depth)

    def edges_interleaved(self):
        e = np.empty(2 * self.nnz, dtype=np.uint32)
        e[0::2] = self.neighbors
        e[1::2] = self.counts
        return e

    def to_struct(self):
        g = OrcGraph()
        g.surface_count = self.surface_count
        g.nnz = self.nnz
        g.row_offsets = _ptr(self.row_offsets, u32p)
        g.neighbors = _ptr(self.neighbors, u32p)
        g.counts = _ptr(self.counts, u32p)
        g.denominators = _ptr(self.denominators, u32p)
        g.sky_counts = _ptr(self.sky_counts, u32p)
        return g


def raster_config(raster_size, layers, bounds_min, bounds_max, periodic_count=0,
                  periodic_size_x=1.0, periodic_size_z=1.0):
    c = OrcRasterConfig()
    c.raster_size = raster_size
    c.layers = layers
    c.periodic_count = periodic_count
    c.periodic_size_x = periodic_size_x
    c.periodic_size_z = periodic_size_z
    for i in range(3):
        c.bounds_min[i] = float(bounds_min[i])
        c.bounds_max[i] = float(bounds_max[i])
    return c


class Oracle:
    """The C restatement (oracle/facet_oracle.c)."""

    def __init__(self):
        self.lib = C.CDLL(build_oracle())
        L = self.lib
        L.orc_sun_direction.restype = OrcDirection
        L.orc_sun_direction.argtypes = [C.c_float, C.c_float]
        L.orc_hemisphere_directions.argtypes = [C.c_uint32, C.c_void_p]
        L.orc_adaptive_layers.restype = C.c_uint32
        L.orc_adaptive_layers.argtypes = [C.c_uint32] * 4
        L.orc_build_graph.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(OrcRasterConfig),
                                      C.c_void_p, C.c_uint32, C.POINTER(OrcGraph)]
        L.orc_free_graph.argtypes = [C.POINTER(OrcGraph)]
        L.orc_sunlit.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(OrcRasterConfig),
                                 OrcDirection, C.c_void_p]
        L.orc_solve.restype = C.c_float
        L.orc_solve.argtypes = [C.POINTER(OrcGraph), C.c_void_p, C.c_float, C.c_uint32,
                                C.c_float, C.c_void_p]
        L.orc_solve_f64.restype = C.c_uint32
        L.orc_solve_f64.argtypes = [C.POINTER(OrcGraph), C.c_void_p, C.c_double,
                                    C.c_uint32, C.c_double, C.c_void_p]
        L.orc_incident.argtypes = [C.POINTER(OrcGraph), C.c_void_p, C.c_void_p, C.c_float,
                                   C.c_void_p]
        L.orc_energy_closure.argtypes = [C.POINTER(OrcGraph), C.c_void_p, C.c_double,
                                         C.c_void_p, f64p, f64p]
        L.orc_load_tree_with_soil.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, u32p, u32p,
                                              f32p, f32p]
        L.orc_make_optics.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p,
                                      OrcDirection] + [C.c_float] * 5 + [C.c_void_p]
        L.orc_hemisphere_graph.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p,
                                           C.c_uint32, C.c_uint32, C.c_uint32,
                                           C.POINTER(OrcGraph), C.POINTER(C.c_uint64)]
        L.orc_hemisphere_sunlit.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32,
                                            C.c_uint32, OrcDirection, C.c_void_p]
        L.orc_hemisphere_graph_periodic.argtypes = [
            C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
            C.c_uint32, C.c_float, C.c_float, C.c_void_p, C.c_void_p]
        L.orc_hemisphere_sunlit_periodic.argtypes = [
            C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_uint32, OrcDirection, C.c_uint32,
            C.c_float, C.c_float, C.c_void_p]
        L.orc_hemisphere_graph_bvh.argtypes = [
            C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
            C.c_uint32, C.c_float, C.c_float, C.c_uint32, C.c_void_p, C.c_void_p]
        L.orc_hemisphere_sunlit_bvh.argtypes = [
            C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_uint32, OrcDirection, C.c_uint32,
            C.c_float, C.c_float, C.c_uint32, C.c_void_p]
        L.orc_hemisphere_rays.argtypes = [
            C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p,
            C.c_uint32, C.c_int, C.c_void_p, C.c_void_p]
        L.orc_free.argtypes = [C.c_void_p]

    # -- geometry helpers -------------------------------------------------
    def hemisphere_directions(self, count=40):
        out = np.zeros((count, 3), dtype=np.float32)
        self.lib.orc_hemisphere_directions(count, out.ctypes.data)
        return out

    def sun_direction(self, zenith, azimuth):
        d = self.lib.orc_sun_direction(zenith, azimuth)
        return np.array([d.x, d.y, d.z], dtype=np.float32)

    def adaptive_layers(self, facets, periodic, raster, base=64):
        return self.lib.orc_adaptive_layers(facets, periodic, raster, base)

    def load_tree_with_soil(self, path):
        verts = C.c_void_p()
        mats = C.c_void_p()
        nf = C.c_uint32()
        nleaf = C.c_uint32()
        bmin = (C.c_float * 3)()
        bmax = (C.c_float * 3)()
        rc = self.lib.orc_load_tree_with_soil(path.encode(), C.byref(verts), C.byref(mats),
                                              C.byref(nf), C.byref(nleaf), bmin, bmax)
        if rc != 0:
            raise RuntimeError(f"orc_load_tree_with_soil failed: {rc}")
        n = nf.value
        v = np.ctypeslib.as_array(C.cast(verts, f32p), shape=(n * 18,)).copy().reshape(n * 3, 6)
        m = np.ctypeslib.as_array(C.cast(mats, u32p), shape=(n,)).copy()
        self.lib.orc_free(verts)
        self.lib.orc_free(mats)
        return v, m, nleaf.value, np.array(bmin[:], np.float32), np.array(bmax[:], np.float32)

    # -- visibility -----------------------------------------------------
    def _take_graph(self, g):
        S = g.surface_count
        nnz = g.nnz

        def arr(p, n):
            if n == 0:
                return np.zeros(0, np.uint32)
            return np.ctypeslib.as_array(p, shape=(n,)).copy()
        out = Graph(arr(g.row_offsets, S + 1), arr(g.neighbors, nnz), arr(g.counts, nnz),
                    arr(g.denominators, S), arr(g.sky_counts, S), g.fragment_overflow,
                    g.max_closure_error, g.max_depth)
        self.lib.orc_free_graph(C.byref(g))
        return out

    def build_graph(self, vertices, cfg, directions):
        vertices = np.ascontiguousarray(vertices, np.float32)
        directions = np.ascontiguousarray(directions, np.float32)
        g = OrcGraph()
        rc = self.lib.orc_build_graph(vertices.ctypes.data, len(vertices) // 3, C.byref(cfg),
                                      directions.ctypes.data, len(directions), C.byref(g))
        if rc < 0:
            raise RuntimeError(f"orc_build_graph failed: {rc}")
        return self._take_graph(g)

    def sunlit(self, vertices, cfg, sun):
        vertices = np.ascontiguousarray(vertices, np.float32)
        out = np.zeros(2 * (len(vertices) // 3), np.float32)
        d = OrcDirection(*[float(x) for x in sun])
        rc = self.lib.orc_sunlit(vertices.ctypes.data, len(vertices) // 3, C.byref(cfg), d,
                                 out.ctypes.data)
        if rc < 0:
            raise RuntimeError(f"orc_sunlit failed: {rc}")
        return out, rc

    # -- solves ---------------------------------------------------------
    def solve(self, graph, optics, sky, iterations=64, relaxation=1.0):
        optics = np.ascontiguousarray(optics, np.float32)
        out = np.zeros(graph.surface_count, np.float32)
        gs = graph.to_struct()
        md = self.lib.orc_solve(C.byref(gs), optics.ctypes.data, sky, iterations, relaxation,
                                out.ctypes.data)
        return out, md

    def solve_f64(self, graph, optics, sky, max_iterations=2000, tol=1e-13):
        optics = np.ascontiguousarray(optics, np.float32)
        out = np.zeros(graph.surface_count, np.float64)
        gs = graph.to_struct()
        it = self.lib.orc_solve_f64(C.byref(gs), optics.ctypes.data, sky, max_iterations, tol,
                                    out.ctypes.data)
        return out, it

    def incident(self, graph, radiosity, optics, sky):
        radiosity = np.ascontiguousarray(radiosity, np.float32)
        optics = np.ascontiguousarray(optics, np.float32)
        out = np.zeros(graph.surface_count, np.float32)
        gs = graph.to_struct()
        self.lib.orc_incident(C.byref(gs), radiosity.ctypes.data, optics.ctypes.data, sky,
                              out.ctypes.data)
        return out

    def energy_closure(self, graph, optics, sky, radiosity64):
        optics = np.ascontiguousarray(optics, np.float32)
        radiosity64 = np.ascontiguousarray(radiosity64, np.float64)
        lhs = C.c_double()
        rhs = C.c_double()
        gs = graph.to_struct()
        self.lib.orc_energy_closure(C.byref(gs), optics.ctypes.data, sky,
                                    radiosity64.ctypes.data, C.byref(lhs), C.byref(rhs))
        return lhs.value, rhs.value

    def make_optics(self, vertices, leaf_count, sunlit, sun, beam=700.0, leaf_rho=0.10,
                    leaf_tau=0.05, ground_rho=0.20, ground_tau=0.0):
        vertices = np.ascontiguousarray(vertices, np.float32)
        F = len(vertices) // 3
        sunlit = np.ascontiguousarray(sunlit, np.float32)
        out = np.zeros((2 * F, 4), np.float32)
        d = OrcDirection(*[float(x) for x in sun])
        self.lib.orc_make_optics(vertices.ctypes.data, F, leaf_count, sunlit.ctypes.data, d,
                                 beam, leaf_rho, leaf_tau, ground_rho, ground_tau,
                                 out.ctypes.data)
        return out

    # -- hemisphere mode -----------------------------------------------
    def hemisphere_graph(self, vertices, sample_uv, sample_dir, rays, sets, top_k,
                         periodic=(0, 1.0, 1.0)):
        vertices = np.ascontiguousarray(vertices, np.float32)
        sample_uv = np.ascontiguousarray(sample_uv, np.float32)
        sample_dir = np.ascontiguousarray(sample_dir, np.float32)
        g = OrcGraph()
        dropped = C.c_uint64()
        self.lib.orc_hemisphere_graph_periodic(
            vertices.ctypes.data, len(vertices) // 3, sample_uv.ctypes.data,
            sample_dir.ctypes.data, rays, sets, top_k, int(periodic[0]), C.c_float(periodic[1]),
            C.c_float(periodic[2]), C.byref(g), C.byref(dropped))
        return self._take_graph(g), dropped.value

    def hemisphere_sunlit(self, vertices, sample_uv, samples, sets, sun, periodic=(0, 1.0, 1.0)):
        vertices = np.ascontiguousarray(vertices, np.float32)
        sample_uv = np.ascontiguousarray(sample_uv, np.float32)
        out = np.zeros(2 * (len(vertices) // 3), np.float32)
        d = OrcDirection(*[float(x) for x in sun])
        self.lib.orc_hemisphere_sunlit_periodic(
            vertices.ctypes.data, len(vertices) // 3, sample_uv.ctypes.data, samples, sets, d,
            int(periodic[0]), C.c_float(periodic[1]), C.c_float(periodic[2]), out.ctypes.data)
        return out


    def hemisphere_graph_bvh(self, vertices, sample_uv, sample_dir, rays, sets, top_k,
                             periodic=(0, 1.0, 1.0), threads=0):
        """hemisphere_graph with a BVH and host threads (same output)."""
        vertices = np.ascontiguousarray(vertices, np.float32)
        sample_uv = np.ascontiguousarray(sample_uv, np.float32)
        sample_dir = np.ascontiguousarray(sample_dir, np.float32)
        g = OrcGraph()
        dropped = C.c_uint64()
        rc = self.lib.orc_hemisphere_graph_bvh(
            vertices.ctypes.data, len(vertices) // 3, sample_uv.ctypes.data,
            sample_dir.ctypes.data, rays, sets, top_k, int(periodic[0]), C.c_float(periodic[1]),
            C.c_float(periodic[2]), threads, C.byref(g), C.byref(dropped))
        if rc != 0:
            raise MemoryError("orc_hemisphere_graph_bvh: out of host memory")
        return self._take_graph(g), dropped.value

    def hemisphere_sunlit_bvh(self, vertices, sample_uv, samples, sets, sun,
                              periodic=(0, 1.0, 1.0), threads=0):
        """hemisphere_sunlit with a BVH and host threads (same output)."""
        vertices = np.ascontiguousarray(vertices, np.float32)
        sample_uv = np.ascontiguousarray(sample_uv, np.float32)
        out = np.zeros(2 * (len(vertices) // 3), np.float32)
        d = OrcDirection(*[float(x) for x in sun])
        rc = self.lib.orc_hemisphere_sunlit_bvh(
            vertices.ctypes.data, len(vertices) // 3, sample_uv.ctypes.data, samples, sets, d,
            int(periodic[0]), C.c_float(periodic[1]), C.c_float(periodic[2]), threads,
            out.ctypes.data)
        if rc != 0:
            raise MemoryError("orc_hemisphere_sunlit_bvh: out of host memory")
        return out


    def hemisphere_rays(self, vertices, sample_uv, sample_dir, rays, sets, sides, bvh=True):
        """Per-ray (side seen or 0xFFFFFFFF, distance) of the listed sides."""
        vertices = np.ascontiguousarray(vertices, np.float32)
        sides = np.ascontiguousarray(sides, np.uint32)
        hs = np.zeros((len(sides), rays), np.uint32)
        ht = np.zeros((len(sides), rays), np.float32)
        rc = self.lib.orc_hemisphere_rays(
            vertices.ctypes.data, len(vertices) // 3,
            np.ascontiguousarray(sample_uv, np.float32).ctypes.data,
            np.ascontiguousarray(sample_dir, np.float32).ctypes.data, rays, sets,
            sides.ctypes.data, len(sides), int(bool(bvh)), hs.ctypes.data, ht.ctypes.data)
        if rc != 0:
            raise MemoryError("orc_hemisphere_rays: out of host memory")
        return hs, ht


class Reference:
    """The reference's own CPU backend, compiled by oracle/build_ref.py."""

    def __init__(self, path=REF_LIB):
        self.lib = C.CDLL(path)
        L = self.lib
        L.ref_last_error.restype = C.c_char_p
        L.ref_free.argtypes = [C.c_void_p]
        L.ref_hemisphere_directions.argtypes = [C.c_void_p]
        L.ref_sun_direction.argtypes = [C.c_float, C.c_float, C.c_void_p]
        L.ref_adaptive_layers.restype = C.c_uint32
        L.ref_adaptive_layers.argtypes = [C.c_uint32] * 4
        L.ref_load_tree_with_soil.restype = C.c_long
        L.ref_load_tree_with_soil.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, u32p, f32p, f32p]
        L.ref_build_graph.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32,
                                      C.c_uint32, C.c_uint32, C.c_float, C.c_float, C.c_void_p,
                                      C.c_void_p, C.POINTER(C.c_uint64), C.c_void_p, C.c_void_p,
                                      f32p]
        L.ref_sunlit.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32,
                                 C.c_uint32, C.c_uint32, C.c_float, C.c_float, C.c_float,
                                 C.c_float, C.c_void_p]
        L.ref_solve.restype = C.c_float
        L.ref_solve.argtypes = [C.c_uint32] + [C.c_void_p] * 5 + [C.c_float, C.c_uint32,
                                                                 C.c_float, C.c_void_p]
        L.ref_incident.argtypes = [C.c_uint32] + [C.c_void_p] * 6 + [C.c_float, C.c_void_p]
        L.ref_make_optics.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_float,
                                      C.c_float, C.c_void_p]
        L.ref_run_cpu_obj.restype = C.c_long
        L.ref_run_cpu_obj.argtypes = [C.c_char_p, C.c_uint32, C.c_void_p, C.c_void_p,
                                      C.c_void_p, u32p, f32p]

        L.ref_planck.restype = C.c_float
        L.ref_planck.argtypes = [C.c_float, C.c_float]
        L.ref_make_spectral_optics.argtypes = ([C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p,
                                                C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p,
                                                C.c_uint32, C.c_float, C.c_float, C.c_void_p,
                                                C.c_float, C.c_float, C.c_uint32, C.c_void_p])

        L.ref_shortwave_windows.restype = C.c_uint32
        L.ref_shortwave_windows.argtypes = ([C.c_void_p, C.c_void_p, C.c_uint32, C.c_float,
                                             C.c_uint32, C.c_float, C.c_float, C.c_void_p,
                                             C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p,
                                             C.c_void_p])
        L.ref_faceteb_node.restype = C.c_int
        L.ref_faceteb_node.argtypes = ([C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_uint32, C.c_float, C.c_float,
                                        C.c_float] + [C.c_void_p] * 5 +
                                       [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_uint32] + [C.c_void_p] * 4)

    def error(self):
        return self.lib.ref_last_error().decode()

    def shortwave_windows(self, total, cosz, direct=None, diffuse=None, direct_fraction=0.8,
                          width=100, wavelengths=()):
        """The windows of runFacetEBCore (facetrtcore.cpp:3485-3536) and the
        per-band spectral irradiances, through the reference's
        ShortwaveSpectrum: (windows (n, 3), band_direct, band_diffuse)."""
        d = None if direct is None else np.ascontiguousarray(direct, np.float32)
        f = None if diffuse is None else np.ascontiguousarray(diffuse, np.float32)
        n = 0 if d is None or f is None else min(d.size, f.size)
        wl = np.ascontiguousarray(wavelengths, np.float32)
        cap = 4096
        win = np.zeros((cap, 3), np.float32)
        bd = np.zeros(max(wl.size, 1), np.float32)
        bf = np.zeros(max(wl.size, 1), np.float32)
        k = self.lib.ref_shortwave_windows(
            None if d is None else d.ctypes.data, None if f is None else f.ctypes.data, n,
            direct_fraction, width, total, cosz, wl.ctypes.data if wl.size else None, wl.size,
            win.ctypes.data, cap, bd.ctypes.data, bf.ctypes.data)
        return win[:k].astype(np.float64), bd[:wl.size], bf[:wl.size]

    @staticmethod
    def _pack_energy_surface(m):
        head = [len(m.reflectance), len(m.transmittance), len(m.energy_reflectance),
                len(m.energy_transmittance), m.tir_reflectance, m.tir_transmittance,
                m.sunlit_temperature, m.shaded_temperature, m.surface_resistance,
                m.specific_heat, m.density, m.thermal_conductivity, m.soil_moisture,
                m.heat_capacity_per_area, m.soil_temperature_method, float(bool(m.photovoltaic)),
                float(bool(m.vegetation)), m.pv_eta25, m.pv_gamma, m.pv_bifaciality,
                m.convective_scale]
        return np.concatenate([np.asarray(head, np.float32),
                               np.asarray(m.reflectance, np.float32).ravel(),
                               np.asarray(m.transmittance, np.float32).ravel(),
                               np.asarray(m.energy_reflectance, np.float32).ravel(),
                               np.asarray(m.energy_transmittance, np.float32).ravel()])

    ENERGY_FIELDS = ("radiosity", "shortwave_radiosity", "diffuse_radiosity",
                     "longwave_radiosity", "absorbed_shortwave", "incident_shortwave",
                     "net_radiation", "sensible_heat", "latent_heat", "storage_heat",
                     "photovoltaic_power")

    def faceteb_node(self, vertices, leaf_count, graph, sunlit, zenith, azimuth, meteo,
                     temperature, materials=(), material_indices=None, texture_factors=None,
                     strength=0.0, spectrum=None, direct_fraction=0.8, width=100, time_step=1800.0,
                     coupling_iterations=20, tolerance=0.05, relaxation=0.5, vegetation_method=0,
                     sky_temperature=250.0, wavelengths=()):
        """One FacetEB node (runFacetEBCore, facetrtcore.cpp:3462-3908) on the
        reference's CPU functions.  graph = (rows, edges (nnz, 2), denom,
        sky); meteo = (air C, vapour, pressure, wind, shortwave, longwave);
        spectrum = (direct, diffuse) or None.  Returns (fields dict incl.
        temperature and band_output, summary dict)."""
        vertices = np.ascontiguousarray(vertices, np.float32)
        F = len(vertices) // 3
        S = 2 * F
        rows, edges, denom, sky = [np.ascontiguousarray(a, np.uint32) for a in graph]
        lit = np.ascontiguousarray(sunlit, np.float32)
        packed = (np.concatenate([self._pack_energy_surface(m) for m in materials])
                  if materials else np.zeros(1, np.float32))
        mi = None if material_indices is None else np.ascontiguousarray(material_indices, np.uint32)
        tex = None if texture_factors is None else np.ascontiguousarray(texture_factors, np.float32)
        sd = sf = None
        n = 0
        if spectrum is not None:
            sd = np.ascontiguousarray(spectrum[0], np.float32)
            sf = np.ascontiguousarray(spectrum[1], np.float32)
            n = min(sd.size, sf.size)
        met = np.asarray(meteo, np.float32)
        settings = np.asarray([time_step, coupling_iterations, tolerance, relaxation,
                               vegetation_method, sky_temperature, width, direct_fraction],
                              np.float32)
        wl = np.ascontiguousarray(wavelengths, np.float32)
        T = np.ascontiguousarray(temperature, np.float32).copy()
        fields = np.zeros((11, S), np.float32)
        bands = np.zeros((max(wl.size, 1), S), np.float32)
        summary = np.zeros(5, np.float32)
        rc = self.lib.ref_faceteb_node(
            vertices.ctypes.data, F, leaf_count, None if mi is None else mi.ctypes.data,
            None if tex is None else tex.ctypes.data, packed.ctypes.data, len(materials),
            strength, zenith, azimuth, rows.ctypes.data, edges.ctypes.data, denom.ctypes.data,
            sky.ctypes.data, lit.ctypes.data, None if sd is None else sd.ctypes.data,
            None if sf is None else sf.ctypes.data, n, met.ctypes.data, settings.ctypes.data,
            wl.ctypes.data if wl.size else None, wl.size, T.ctypes.data, fields.ctypes.data,
            bands.ctypes.data, summary.ctypes.data)
        if rc != 0:
            raise RuntimeError(self.error())
        out = {k: fields[i] for i, k in enumerate(self.ENERGY_FIELDS)}
        out["temperature"] = T
        out["band_output"] = bands[:wl.size]
        return out, {"coupling_iterations": int(summary[0]), "converged": int(summary[1]),
                     "max_temperature_delta": float(summary[2]),
                     "max_energy_residual": float(summary[3]),
                     "max_energy_residual_equivalent": float(summary[4])}

    def planck(self, wavelength, temperature):
        return float(self.lib.ref_planck(wavelength, temperature))

    @staticmethod
    def _pack_surface(m):
        r = np.asarray(m.reflectance, np.float32).ravel()
        t = np.asarray(m.transmittance, np.float32).ravel()
        head = [r.size, t.size, m.tir_reflectance, m.tir_transmittance, m.sunlit_temperature,
                m.shaded_temperature]
        return np.concatenate([np.asarray(head, np.float32), r, t])

    def make_spectral_optics(self, vertices, leaf_count, sunlit, zenith, azimuth, wavelengths,
                             band, object_surface, ground, materials=(), material_indices=None,
                             texture_factors=None, strength=0.0, sky_temperature=250.0):
        """makeSpectralOptics (facetrtcore.cpp:1057-1126) for one band.
        Surfaces are any objects with reflectance, transmittance,
        tir_reflectance, tir_transmittance, sunlit_temperature and
        shaded_temperature attributes."""
        vertices = np.ascontiguousarray(vertices, np.float32)
        sunlit = np.ascontiguousarray(sunlit, np.float32)
        wl = np.ascontiguousarray(wavelengths, np.float32)
        F = len(vertices) // 3
        packed = np.concatenate([self._pack_surface(m)
                                 for m in [object_surface, ground, *materials]])
        mi = None if material_indices is None else np.ascontiguousarray(material_indices,
                                                                        np.uint32)
        tex = None if texture_factors is None else np.ascontiguousarray(texture_factors,
                                                                       np.float32)
        out = np.zeros((2 * F, 4), np.float32)
        self.lib.ref_make_spectral_optics(
            vertices.ctypes.data, F, leaf_count, None if mi is None else mi.ctypes.data,
            None if tex is None else tex.ctypes.data, packed.ctypes.data, len(materials),
            wl.ctypes.data, wl.size, strength, sky_temperature, sunlit.ctypes.data, zenith,
            azimuth, band, out.ctypes.data)
        return out

    def hemisphere_directions(self):
        out = np.zeros((40, 3), np.float32)
        self.lib.ref_hemisphere_directions(out.ctypes.data)
        return out

    def sun_direction(self, zenith, azimuth):
        out = np.zeros(3, np.float32)
        self.lib.ref_sun_direction(zenith, azimuth, out.ctypes.data)
        return out

    def adaptive_layers(self, facets, periodic, raster, base=64):
        return self.lib.ref_adaptive_layers(facets, periodic, raster, base)

    def load_tree_with_soil(self, path):
        verts = C.c_void_p()
        mats = C.c_void_p()
        nleaf = C.c_uint32()
        bmin = (C.c_float * 3)()
        bmax = (C.c_float * 3)()
        n = self.lib.ref_load_tree_with_soil(path.encode(), C.byref(verts), C.byref(mats),
                                             C.byref(nleaf), bmin, bmax)
        if n < 0:
            raise RuntimeError(self.error())
        v = np.ctypeslib.as_array(C.cast(verts, f32p), shape=(n * 18,)).copy().reshape(n * 3, 6)
        m = np.ctypeslib.as_array(C.cast(mats, u32p), shape=(n,)).copy()
        self.lib.ref_free(verts)
        self.lib.ref_free(mats)
        return v, m, nleaf.value, np.array(bmin[:], np.float32), np.array(bmax[:], np.float32)

    def build_graph(self, vertices, raster, layers, bmin, bmax, periodic=0, px=1.0, pz=1.0):
        vertices = np.ascontiguousarray(vertices, np.float32)
        bmin = np.ascontiguousarray(bmin, np.float32)
        bmax = np.ascontiguousarray(bmax, np.float32)
        ro, ed, de, sk = C.c_void_p(), C.c_void_p(), C.c_void_p(), C.c_void_p()
        ne = C.c_uint64()
        clo = C.c_float()
        F = len(vertices) // 3
        rc = self.lib.ref_build_graph(vertices.ctypes.data, F, bmin.ctypes.data, bmax.ctypes.data,
                                      raster, layers, periodic, px, pz, C.byref(ro), C.byref(ed),
                                      C.byref(ne), C.byref(de), C.byref(sk), C.byref(clo))
        if rc != 0:
            raise RuntimeError(f"reference buildCpuGraph: {self.error()}")
        S = 2 * F
        n = ne.value

        def arr(p, k):
            a = np.ctypeslib.as_array(C.cast(p, u32p), shape=(max(k, 1),))[:k].copy()
            self.lib.ref_free(p)
            return a
        rows = arr(ro, S + 1)
        edges = arr(ed, 2 * n)
        return Graph(rows, edges[0::2], edges[1::2], arr(de, S), arr(sk, S),
                     0, clo.value)

    def sunlit(self, vertices, raster, layers, bmin, bmax, zenith, azimuth, periodic=0,
               px=1.0, pz=1.0):
        vertices = np.ascontiguousarray(vertices, np.float32)
        bmin = np.ascontiguousarray(bmin, np.float32)
        bmax = np.ascontiguousarray(bmax, np.float32)
        F = len(vertices) // 3
        out = np.zeros(2 * F, np.float32)
        rc = self.lib.ref_sunlit(vertices.ctypes.data, F, bmin.ctypes.data, bmax.ctypes.data,
                                 raster, layers, periodic, px, pz, zenith, azimuth,
                                 out.ctypes.data)
        if rc != 0:
            raise RuntimeError(f"reference computeCpuSunlit: {self.error()}")
        return out

    def solve(self, graph, optics, sky, iterations=64, relaxation=1.0):
        optics = np.ascontiguousarray(optics, np.float32)
        edges = graph.edges_interleaved()
        out = np.zeros(graph.surface_count, np.float32)
        md = self.lib.ref_solve(graph.surface_count, graph.row_offsets.ctypes.data,
                                edges.ctypes.data, graph.denominators.ctypes.data,
                                graph.sky_counts.ctypes.data, optics.ctypes.data, sky,
                                iterations, relaxation, out.ctypes.data)
        return out, md

    def incident(self, graph, radiosity, optics, sky):
        optics = np.ascontiguousarray(optics, np.float32)
        radiosity = np.ascontiguousarray(radiosity, np.float32)
        edges = graph.edges_interleaved()
        out = np.zeros(graph.surface_count, np.float32)
        self.lib.ref_incident(graph.surface_count, graph.row_offsets.ctypes.data,
                              edges.ctypes.data, graph.denominators.ctypes.data,
                              graph.sky_counts.ctypes.data, radiosity.ctypes.data,
                              optics.ctypes.data, sky, out.ctypes.data)
        return out

    def make_optics(self, vertices, leaf_count, sunlit, zenith, azimuth):
        vertices = np.ascontiguousarray(vertices, np.float32)
        sunlit = np.ascontiguousarray(sunlit, np.float32)
        F = len(vertices) // 3
        out = np.zeros((2 * F, 4), np.float32)
        self.lib.ref_make_optics(vertices.ctypes.data, F, leaf_count, sunlit.ctypes.data,
                                 zenith, azimuth, out.ctypes.data)
        return out

    def run_cpu_obj(self, path, raster=1024, max_facets=2_000_000):
        rad = np.zeros(2 * max_facets, np.float32)
        sun = np.zeros_like(rad)
        enh = np.zeros_like(rad)
        edges = C.c_uint32()
        clo = C.c_float()
        n = self.lib.ref_run_cpu_obj(path.encode(), raster, rad.ctypes.data, sun.ctypes.data,
                                     enh.ctypes.data, C.byref(edges), C.byref(clo))
        if n < 0:
            raise RuntimeError(self.error())
        S = 2 * n
        return dict(radiosity=rad[:S].copy(), sunlit=sun[:S].copy(),
                    lightEnhancement=enh[:S].copy(), directedEdges=edges.value,
                    closureError=clo.value, facetCount=n)


def reference_available():
    return os.path.exists(REF_LIB)


PROJECT_LIB = os.path.join(HERE, "_ref", "libproject_ref.so")


class ReferenceProject:
    """The reference's own loadProjectScene / facetRTParametersFromInput
    (compiled by oracle/build_ref.py into oracle/_ref/libproject_ref.so;
    built only where the reference tree is present)."""

    HEAD = 24

    def __init__(self, path=PROJECT_LIB):
        self.lib = C.CDLL(path)
        self.lib.ref_project_last_error.restype = C.c_char_p
        self.lib.ref_load_project.argtypes = [C.c_char_p, C.c_void_p] + [C.c_void_p] * 6
        self.lib.ref_project_free.argtypes = [C.c_void_p]

    def _take(self, ptr, n, dtype):
        ct = C.c_float if dtype == np.float32 else C.c_uint32
        a = np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ct)), (max(n, 1),))[:n].copy()
        self.lib.ref_project_free(ptr)
        return a

    @classmethod
    def unpack(cls, packed, count):
        """Split packed surfaces into dicts of their fields."""
        names = ["tir_reflectance", "tir_transmittance", "sunlit_temperature",
                 "shaded_temperature", "surface_resistance", "specific_heat", "density",
                 "thermal_conductivity", "soil_moisture", "heat_capacity_per_area",
                 "soil_temperature_method", "photovoltaic", "vegetation", "pv_eta25", "pv_gamma",
                 "pv_bifaciality", "convective_scale", "output_component", "texture_strength",
                 "texture_repeat"]
        out, at = [], 0
        for _ in range(count):
            h = packed[at:at + cls.HEAD]
            nr, nt, ner, net = (int(x) for x in h[:4])
            d = dict(zip(names, h[4:].tolist()))
            v = packed[at + cls.HEAD:]
            d["reflectance"], v = v[:nr], v[nr:]
            d["transmittance"], v = v[:nt], v[nt:]
            d["energy_reflectance"], v = v[:ner], v[ner:]
            d["energy_transmittance"] = v[:net]
            out.append(d)
            at += cls.HEAD + nr + nt + ner + net
        return out

    def load(self, path):
        info = np.zeros(24, np.float32)
        ptrs = [C.c_void_p() for _ in range(6)]
        rc = self.lib.ref_load_project(os.fsencode(path), info.ctypes.data,
                                       *[C.byref(p) for p in ptrs])
        if rc != 0:
            raise RuntimeError(self.lib.ref_project_last_error().decode())
        F = int(info[0])
        M = int(info[16])
        nb = int(info[17])
        vertices = self._take(ptrs[0], 18 * F, np.float32).reshape(3 * F, 6)
        mi = self._take(ptrs[1], F, np.uint32)
        # sizes of the packed blocks are only known by walking them
        raw_m = C.cast(ptrs[2], C.POINTER(C.c_float))
        raw_p = C.cast(ptrs[3], C.POINTER(C.c_float))

        def walk(raw, count):
            at = 0
            for _ in range(count):
                nr, nt, ner, net = (int(raw[at + k]) for k in range(4))
                at += self.HEAD + nr + nt + ner + net
            return at
        nm, npar = walk(raw_m, M), walk(raw_p, 2)
        materials = self.unpack(self._take(ptrs[2], nm, np.float32), M)
        params = self.unpack(self._take(ptrs[3], npar, np.float32), 2)
        wavelengths = self._take(ptrs[4], nb, np.float32)
        tex = self._take(ptrs[5], F if info[20] else 0, np.float32)
        names = ["facet_count", "leaf_facet_count", "sun_zenith", "sun_azimuth",
                 "periodic_neighbor_count", "periodic_size_x", "periodic_size_z", "raster_size",
                 "raster_layers", "background_angular_strength"]
        d = dict(zip(names, info[:10].tolist()))
        d.update(minimum=info[10:13].tolist(), maximum=info[13:16].tolist(),
                 material_count=M, band_count=nb, sky_temperature=float(info[18]),
                 accelerated_solver=int(info[19]))
        return dict(info=d, vertices=vertices, material_indices=mi, materials=materials,
                    object=params[0], ground=params[1], wavelengths=wavelengths,
                    texture_factors=tex)


SPA_LIB = os.path.join(HERE, "_ref", "libspa_ref.so")


class ReferenceSun:
    """The reference's own SPA (thirdparty/spa.cpp) and FacetEB
    updateSolarPosition (compiled by oracle/build_ref.py into
    oracle/_ref/libspa_ref.so; built only where the reference tree is
    present)."""

    def __init__(self, path=SPA_LIB):
        self.lib = C.CDLL(path)
        self.lib.ref_faceteb_sun.argtypes = [C.c_float] * 5 + [C.POINTER(C.c_float)] * 2
        self.lib.ref_spa_za.argtypes = [C.c_int] * 6 + [C.c_double] * 8 + \
            [C.POINTER(C.c_double)] * 2
        self.lib.ref_delta_t.restype = C.c_double
        self.lib.ref_delta_t.argtypes = [C.c_int, C.c_int]

    def faceteb_sun(self, julian_time, latitude, longitude, pressure, air_temperature):
        """(zenith, azimuth) as float32, or None where the reference throws."""
        z, a = C.c_float(), C.c_float()
        if self.lib.ref_faceteb_sun(julian_time, latitude, longitude, pressure, air_temperature,
                                    C.byref(z), C.byref(a)):
            return None
        return np.float32(z.value), np.float32(a.value)

    def spa_za(self, year, month, day, hour, minute, second, *, delta_t, timezone, longitude,
               latitude, elevation, pressure, temperature, atmos_refract):
        """(SPA error code, zenith, azimuth)."""
        z, a = C.c_double(), C.c_double()
        err = self.lib.ref_spa_za(year, month, day, hour, minute, second, delta_t, timezone,
                                  longitude, latitude, elevation, pressure, temperature,
                                  atmos_refract, C.byref(z), C.byref(a))
        return err, z.value, a.value

    def delta_t(self, year, month):
        return self.lib.ref_delta_t(year, month)
