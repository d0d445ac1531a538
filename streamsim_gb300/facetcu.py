"""ctypes binding of libfacetcu.so (include/facetcu.h) and a host-side class
with the method names of the reference's facetvk::FacetrtVulkan
(models/histream/src/facetrt/facetrt_vulkan.h:70-104).

Errors come back as the reference's exception types: FACETCU_INVALID_ARGUMENT
-> ValueError (std::invalid_argument), FACETCU_LOGIC_ERROR -> LogicError
(std::logic_error), FACETCU_RUNTIME_ERROR -> RuntimeError, FACETCU_OVERFLOW_ERROR
-> OverflowError, anything else -> FacetcuError.  There is no CPU fallback:
if the library is missing, load() raises.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfacetcu.so")

OK = 0
INVALID_ARGUMENT = 1
LOGIC_ERROR = 2
RUNTIME_ERROR = 3
OVERFLOW_ERROR = 4
CUDA_ERROR = 5
NO_DEVICE = 6
OUT_OF_MEMORY = 7
DEVICE_CAPACITY = 8
NOT_CONVERGED = 9
DEVICE_TIMEOUT = 10

PRECISION_FP32 = 0
PRECISION_MIXED = 1
PRECISION_FP64 = 2
WARM_NONE = 0
WARM_GIVEN = 1
WARM_MLP = 2
BATCH_TIME_SWEEPS = 1
BATCH_LEGACY_STEP = 2


class FacetcuError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"[{code}] {message}")
        self.code = code


class LogicError(FacetcuError):
    pass


class NotConverged(FacetcuError):
    pass


class Vertex(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("normal", C.c_float * 3)]


class Direction(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class SurfaceOptics(C.Structure):
    _fields_ = [("reflectance", C.c_float), ("transmittance", C.c_float),
                ("emission", C.c_float), ("direct_irradiance", C.c_float)]


class Config(C.Structure):
    _fields_ = [("raster_width", C.c_uint32), ("raster_height", C.c_uint32),
                ("max_fragments_per_pixel", C.c_uint32), ("edge_hash_capacity", C.c_uint32),
                ("enable_validation", C.c_bool), ("gpu_index", C.c_uint32),
                ("periodic_neighbor_count", C.c_uint32), ("periodic_size_x", C.c_float),
                ("periodic_size_z", C.c_float)]


class GraphDiagnostics(C.Structure):
    _fields_ = [("facet_count", C.c_uint32), ("surface_count", C.c_uint32),
                ("directed_edge_count", C.c_uint32), ("fragment_overflow", C.c_uint32),
                ("hash_overflow", C.c_uint32), ("max_closure_error", C.c_float)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class HemisphereConfig(C.Structure):
    _fields_ = [("rays_per_side", C.c_uint32), ("top_k", C.c_uint32),
                ("sample_sets", C.c_uint32), ("reserved", C.c_uint32)]


class BatchConfig(C.Structure):
    _fields_ = [("band_count", C.c_uint32), ("sun_count", C.c_uint32),
                ("precision", C.c_uint32), ("warm_start", C.c_uint32),
                ("maximum_iterations", C.c_uint32), ("tolerance", C.c_float),
                ("panel_width", C.c_uint32), ("flags", C.c_uint32)]


class MlpTrainConfig(C.Structure):
    _fields_ = [("steps", C.c_uint32), ("batch", C.c_uint32), ("learning_rate", C.c_float),
                ("seed", C.c_uint32)]


class BatchResult(C.Structure):
    _fields_ = [("iterations", C.c_uint32), ("residual_corrections", C.c_uint32),
                ("converged", C.c_uint32), ("max_relative_change", C.c_float),
                ("seconds", C.c_double), ("kernel_launches", C.c_uint32),
                ("sweeps", C.c_uint32), ("sweep_seconds", C.c_double),
                ("sweep_bytes", C.c_double), ("timed_sweeps", C.c_uint32),
                ("graph_launches", C.c_uint32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class SceneInfo(C.Structure):
    _fields_ = [("facet_count", C.c_uint32), ("leaf_facet_count", C.c_uint32),
                ("minimum", C.c_float * 3), ("maximum", C.c_float * 3)]


class SurfaceParameters(C.Structure):
    _fields_ = [("reflectance", C.c_void_p), ("reflectance_count", C.c_uint32),
                ("transmittance", C.c_void_p), ("transmittance_count", C.c_uint32),
                ("tir_reflectance", C.c_float), ("tir_transmittance", C.c_float),
                ("sunlit_temperature", C.c_float), ("shaded_temperature", C.c_float)]


class SpectralParameters(C.Structure):
    _fields_ = [("wavelengths", C.c_void_p), ("band_count", C.c_uint32),
                ("object", SurfaceParameters), ("ground", SurfaceParameters),
                ("materials", C.c_void_p), ("material_count", C.c_uint32),
                ("material_indices", C.c_void_p), ("texture_factors", C.c_void_p),
                ("leaf_facet_count", C.c_uint32), ("background_angular_strength", C.c_float),
                ("sky_temperature", C.c_float), ("accelerated_solver", C.c_uint32)]


class BandResult(C.Structure):
    _fields_ = [("iterations", C.c_uint32), ("max_delta", C.c_float),
                ("thermal_bands", C.c_uint32), ("batched_sweeps", C.c_uint32),
                ("seconds", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ShortwaveSpectrum(C.Structure):
    _fields_ = [("direct", C.c_void_p), ("diffuse", C.c_void_p), ("sample_count", C.c_uint32),
                ("direct_fraction", C.c_float), ("window_width", C.c_uint32)]


class ShortwaveWindow(C.Structure):
    _fields_ = [("direct_normal", C.c_float), ("diffuse", C.c_float), ("energy_band", C.c_uint32)]


class EnergySurfaceParameters(C.Structure):
    _fields_ = [("optics", SurfaceParameters),
                ("energy_reflectance", C.c_void_p), ("energy_reflectance_count", C.c_uint32),
                ("energy_transmittance", C.c_void_p), ("energy_transmittance_count", C.c_uint32),
                ("surface_resistance", C.c_float), ("specific_heat", C.c_float),
                ("density", C.c_float), ("thermal_conductivity", C.c_float),
                ("soil_moisture", C.c_float), ("heat_capacity_per_area", C.c_float),
                ("soil_temperature_method", C.c_int32), ("photovoltaic", C.c_uint32),
                ("vegetation", C.c_uint32), ("pv_eta25", C.c_float), ("pv_gamma", C.c_float),
                ("pv_bifaciality", C.c_float), ("convective_scale", C.c_float)]


class EnergyParameters(C.Structure):
    _fields_ = [("materials", C.c_void_p), ("material_count", C.c_uint32),
                ("material_indices", C.c_void_p), ("texture_factors", C.c_void_p),
                ("leaf_facet_count", C.c_uint32), ("background_angular_strength", C.c_float),
                ("wavelengths", C.c_void_p), ("band_count", C.c_uint32),
                ("sky_temperature", C.c_float), ("time_step", C.c_float),
                ("coupling_iterations", C.c_uint32), ("temperature_tolerance", C.c_float),
                ("temperature_relaxation", C.c_float),
                ("vegetation_temperature_method", C.c_int32), ("solver_iterations", C.c_uint32),
                ("solver_tolerance", C.c_float), ("precision", C.c_uint32)]


class Meteo(C.Structure):
    _fields_ = [("air_temperature", C.c_float), ("vapor_pressure", C.c_float),
                ("pressure", C.c_float), ("wind_speed", C.c_float), ("shortwave", C.c_float),
                ("longwave", C.c_float)]


ENERGY_FIELDS = ("temperature", "radiosity", "shortwave_radiosity", "diffuse_radiosity",
                 "longwave_radiosity", "absorbed_shortwave", "incident_shortwave",
                 "net_radiation", "sensible_heat", "latent_heat", "storage_heat",
                 "photovoltaic_power", "band_output")


class EnergyFields(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in ENERGY_FIELDS]


class EnergyResult(C.Structure):
    _fields_ = [("coupling_iterations", C.c_uint32), ("converged", C.c_uint32),
                ("max_temperature_delta", C.c_float), ("max_energy_residual", C.c_float),
                ("max_energy_residual_equivalent", C.c_float), ("shortwave_sweeps", C.c_uint32),
                ("longwave_sweeps", C.c_uint32), ("band_sweeps", C.c_uint32),
                ("solves", C.c_uint32), ("kernel_launches", C.c_uint32),
                ("seconds", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Sensor(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("perspective", C.c_uint32),
                ("view_zenith", C.c_double), ("view_azimuth", C.c_double), ("fov", C.c_double),
                ("scene_x", C.c_double), ("scene_y", C.c_double), ("position", C.c_double * 3),
                ("sky_temperature", C.c_double), ("temperature_output", C.c_uint32)]


class ImageInfo(C.Structure):
    _fields_ = [("observed_pixels", C.c_uint32), ("output_pixels", C.c_uint32),
                ("naming_zenith", C.c_double), ("naming_azimuth", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def sensor(width=512, height=512, perspective=False, vza=0.0, vaa=0.0, fov=0.0, scene_x=1.0,
           scene_y=1.0, position=(float("nan"),) * 3, sky_temperature=0.0,
           temperature_output=False):
    """A Sensor struct (the project's sensor block; 0 / NaN take the reference's
    defaults)."""
    return Sensor(width, height, 1 if perspective else 0, vza, vaa, fov, scene_x, scene_y,
                  (C.c_double * 3)(*position), sky_temperature, 1 if temperature_output else 0)


class SolarInput(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("year", "month", "day", "hour", "minute", "second")] + \
               [(n, C.c_double) for n in ("delta_t", "timezone", "longitude", "latitude",
                                          "elevation", "pressure", "temperature",
                                          "atmos_refract")]


class ProjectInfo(C.Structure):
    _fields_ = [("facet_count", C.c_uint32), ("leaf_facet_count", C.c_uint32),
                ("material_count", C.c_uint32), ("band_count", C.c_uint32),
                ("sun_zenith", C.c_float), ("sun_azimuth", C.c_float),
                ("periodic_neighbor_count", C.c_uint32), ("periodic_size_x", C.c_float),
                ("periodic_size_z", C.c_float), ("raster_size", C.c_uint32),
                ("raster_layers", C.c_uint32), ("background_angular_strength", C.c_float),
                ("minimum", C.c_float * 3), ("maximum", C.c_float * 3),
                ("sky_temperature", C.c_float), ("accelerated_solver", C.c_uint32)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["minimum"], d["maximum"] = list(self.minimum), list(self.maximum)
        return d


_vp = C.c_void_p
_u32 = C.c_uint32
_ctx = C.c_void_p

# name -> (restype, argtypes) for every symbol of include/facetcu.h
SIGNATURES = {
    "facetcu_hemisphere_directions": (None, [_u32, _vp]),
    "facetcu_sun_direction": (Direction, [C.c_float, C.c_float]),
    "facetcu_create": (C.c_int, [C.POINTER(_vp)]),
    "facetcu_release": (None, [_ctx]),
    "facetcu_last_error": (C.c_char_p, [_ctx]),
    "facetcu_device_count": (C.c_int, [C.POINTER(C.c_int)]),
    "facetcu_initialize": (C.c_int, [_ctx, C.POINTER(Config)]),
    "facetcu_destroy": (C.c_int, [_ctx]),
    "facetcu_get_stream": (C.c_int, [_ctx, C.POINTER(_vp)]),
    "facetcu_set_geometry": (C.c_int, [_ctx, _vp, C.c_uint64]),
    "facetcu_set_raster_bounds": (C.c_int, [_ctx, _vp, _vp]),
    "facetcu_build_visibility_graph": (C.c_int, [_ctx, _vp, _u32, C.POINTER(GraphDiagnostics)]),
    "facetcu_compute_sunlit_fraction": (C.c_int, [_ctx, C.POINTER(Direction), _vp]),
    "facetcu_graph_size": (C.c_int, [_ctx, C.POINTER(_u32), C.POINTER(C.c_uint64)]),
    "facetcu_get_graph": (C.c_int, [_ctx, _vp, _vp, _vp, _vp]),
    "facetcu_set_graph": (C.c_int, [_ctx, _u32, _vp, _vp, _vp, _vp]),
    "facetcu_solve": (C.c_int, [_ctx, _vp, C.c_uint64, C.c_float, _u32, C.c_float, _vp,
                                C.POINTER(_u32), C.POINTER(C.c_float)]),
    "facetcu_solve_accelerated": (C.c_int, [_ctx, _vp, C.c_uint64, C.c_float, _vp, _u32, _u32,
                                            C.c_float, C.c_float, _vp, C.POINTER(_u32),
                                            C.POINTER(C.c_float)]),
    "facetcu_incident_irradiance": (C.c_int, [_ctx, _vp, _vp, C.c_uint64, C.c_float, _vp]),
    "facetcu_solve_batched": (C.c_int, [_ctx, C.POINTER(BatchConfig)] + [_vp] * 8 +
                              [C.POINTER(BatchResult)]),
    "facetcu_solve_batched_device": (C.c_int, [_ctx, C.POINTER(BatchConfig)] + [_vp] * 8 +
                                     [C.POINTER(BatchResult)]),
    "facetcu_build_hemisphere_graph": (C.c_int, [_ctx, C.POINTER(HemisphereConfig), _vp, _vp,
                                                 C.POINTER(GraphDiagnostics),
                                                 C.POINTER(C.c_uint64)]),
    "facetcu_hemisphere_sunlit": (C.c_int, [_ctx, C.POINTER(Direction), _u32, _u32, _vp, _vp]),
    "facetcu_solve_noalloc": (C.c_int, [_vp, _vp, _vp, _vp, _u32, _vp, C.c_float, _u32, C.c_float,
                                        _vp, C.POINTER(C.c_float), _vp]),
}
SIGNATURES.update({
    "facetcu_mlp_parameter_count": (C.c_int, [C.POINTER(_u32)]),
    "facetcu_mlp_reset": (C.c_int, [_ctx, _u32]),
    "facetcu_mlp_get_parameters": (C.c_int, [_ctx, _vp]),
    "facetcu_mlp_set_parameters": (C.c_int, [_ctx, _vp]),
    "facetcu_mlp_forward": (C.c_int, [_ctx, _vp, _u32, _vp]),
    "facetcu_mlp_forward_tensor": (C.c_int, [_ctx, _vp, _u32, _vp]),
    "facetcu_mlp_loss_and_gradient": (C.c_int, [_ctx, _vp, _vp, _u32, C.POINTER(C.c_float), _vp]),
    "facetcu_mlp_train_device": (C.c_int, [_ctx, _vp, _vp, C.c_uint64, C.POINTER(MlpTrainConfig),
                                           C.POINTER(C.c_float)]),
    "facetcu_mlp_samples_device": (C.c_int, [_ctx, C.POINTER(BatchConfig)] + [_vp] * 9),
})
SIGNATURES.update({
    "facetcu_load_tree_with_soil": (C.c_int, [C.c_char_p, _vp, _vp, _u32, C.POINTER(SceneInfo)]),
    "facetcu_make_optics": (C.c_int, [_vp, _u32, _u32, _vp, C.POINTER(Direction), _vp]),
    "facetcu_planck_radiance": (C.c_float, [C.c_float, C.c_float]),
    "facetcu_host_last_error": (C.c_char_p, []),
    "facetcu_run_facetrt_core": (C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p]),
    "facetcu_spectral_optics": (C.c_int, [_ctx, C.POINTER(SpectralParameters), _vp,
                                          C.POINTER(Direction), _u32, _vp]),
    "facetcu_solve_bands": (C.c_int, [_ctx, C.POINTER(SpectralParameters), _vp,
                                      C.POINTER(Direction), _vp, _vp, C.POINTER(BandResult)]),
})
SIGNATURES["facetcu_autotune_batched"] = (C.c_int, [_ctx, C.POINTER(BatchConfig)] + [_vp] * 7 +
                                          [C.c_char_p, C.POINTER(_u32)])
SIGNATURES["facetcu_scene_batch"] = (C.c_int, [_ctx, _vp, _u32, _vp, C.POINTER(GraphDiagnostics)])
SIGNATURES.update({
    "facetcu_project_load": (C.c_int, [C.c_char_p, C.POINTER(_vp)]),
    "facetcu_project_release": (None, [_vp]),
    "facetcu_project_get_info": (C.c_int, [_vp, C.POINTER(ProjectInfo)]),
    "facetcu_project_get_geometry": (C.c_int, [_vp, _vp, _vp, _vp]),
    "facetcu_project_get_material": (C.c_int, [_vp, _u32, C.POINTER(EnergySurfaceParameters),
                                               C.POINTER(_u32)]),
    "facetcu_project_spectral_parameters": (C.c_int, [_vp, C.POINTER(SpectralParameters)]),
    "facetcu_project_xml_view": (C.c_int, [C.c_char_p, _vp, C.c_uint64, C.POINTER(C.c_uint64)]),
    "facetcu_solar_position": (C.c_int, [C.POINTER(SolarInput), C.POINTER(C.c_double),
                                         C.POINTER(C.c_double), C.POINTER(C.c_int32)]),
    "facetcu_faceteb_sun": (C.c_int, [C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
                                      C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "facetcu_dem_height_field": (C.c_int, [C.c_char_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                           C.POINTER(C.c_float), _vp, C.c_uint64]),
})
SIGNATURES["facetcu_render_sensor_image"] = (C.c_int, [_ctx, C.POINTER(Sensor), _vp, _u32, _vp, _vp,
                                                      _vp, C.POINTER(ImageInfo)])
SIGNATURES.update({
    "facetcu_shortwave_windows": (C.c_int, [C.POINTER(ShortwaveSpectrum), C.c_float, C.c_float, _vp,
                                            _u32, _vp, _u32, C.POINTER(_u32), _vp, _vp]),
    "facetcu_energy_surface_defaults": (None, [C.POINTER(EnergySurfaceParameters)]),
    "facetcu_faceteb_node": (C.c_int, [_ctx, C.POINTER(EnergyParameters), C.POINTER(Meteo),
                                       C.POINTER(Direction), _vp, _vp, _u32, _vp, _vp,
                                       C.POINTER(EnergyFields), C.POINTER(EnergyResult)]),
})
OPTIONAL_SIGNATURES = {}
MLP_INPUTS = 12
MLP_OUTPUTS = 64
MLP_PARAMETERS = 26432
WARM_START_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data",
                                  "mlp_warm_start.npy")
NOALLOC_MAX_SURFACES = 1048576
NOALLOC_MAX_ITERATIONS = 4096

_LIB = None


def load(path=LIB_PATH):
    """Load libfacetcu.so; raises if it has not been built (no fallback)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        raise FacetcuError(NO_DEVICE, f"libfacetcu.so not built at {path}; run "
                                      "`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(path)
    for name, (res, args) in {**SIGNATURES, **OPTIONAL_SIGNATURES}.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def header_symbols(header=None):
    """Function names declared in include/facetcu.h."""
    import re
    header = header or os.path.join(HERE, "..", "include", "facetcu.h")
    text = open(header).read()
    return sorted(set(re.findall(r"\b(facetcu_[a-z0-9_]+)\s*\(", text)))


def hemisphere_directions(count=40):
    """makeHemisphereDirections (facetrtcore.cpp:475-489), computed by the library."""
    out = np.zeros((count, 3), np.float32)
    load().facetcu_hemisphere_directions(count, C.c_void_p(out.ctypes.data))
    return out


def sun_direction(zenith_deg, azimuth_deg):
    """sunDirection (facetrtcore.cpp:491-498), computed by the library."""
    d = load().facetcu_sun_direction(zenith_deg, azimuth_deg)
    return np.array([d.x, d.y, d.z], np.float32)


def _host_check(rc):
    if rc != OK:
        msg = (load().facetcu_host_last_error() or b"").decode()
        raise (ValueError if rc == INVALID_ARGUMENT else RuntimeError)(msg)


def load_tree_with_soil(path):
    """loadTreeWithSoil: (vertices (3F, 6) float32, material per facet,
    leaf facet count, minimum (3,), maximum (3,))."""
    lib = load()
    info = SceneInfo()
    _host_check(lib.facetcu_load_tree_with_soil(os.fsencode(path), None, None, 0, C.byref(info)))
    F = info.facet_count
    v = np.zeros((3 * F, 6), np.float32)
    mat = np.zeros(F, np.uint32)
    _host_check(lib.facetcu_load_tree_with_soil(os.fsencode(path), _ptr(v), _ptr(mat), F,
                                                C.byref(info)))
    return (v, mat, info.leaf_facet_count, np.array(info.minimum[:], np.float32),
            np.array(info.maximum[:], np.float32))


def make_optics(vertices, leaf_facet_count, sunlit, sun):
    """makeOptics: (2F, 4) float32 [rho, tau, e, D]."""
    v = _f32(vertices).reshape(-1, 6)
    F = len(v) // 3
    lit = _f32(sunlit)
    if lit.size != 2 * F:
        raise ValueError("sunlit must hold 2 values per facet")
    out = np.zeros((2 * F, 4), np.float32)
    d = Direction(*[float(x) for x in np.ravel(sun)[:3]])
    _host_check(load().facetcu_make_optics(_ptr(v), F, leaf_facet_count, _ptr(lit), C.byref(d),
                                           _ptr(out)))
    return out


def planck_radiance(wavelength, temperature):
    return float(load().facetcu_planck_radiance(wavelength, temperature))


def run_facetrt_core(input_path, output_file=None):
    """runFacetRTCore: 0 on success, 1 on failure (messages on stdout/stderr)."""
    out = os.fsencode(output_file) if output_file else None
    return int(load().facetcu_run_facetrt_core(os.fsencode(input_path), None, out))


class Surface:
    """SurfaceParameters: per-band reflectance/transmittance lists (empty =
    the reference's object/ground fallback), thermal-IR values and the
    sunlit/shaded temperatures."""

    def __init__(self, reflectance=(), transmittance=(), tir_reflectance=0.03,
                 tir_transmittance=0.0, sunlit_temperature=300.0, shaded_temperature=296.0):
        self.reflectance = np.asarray(reflectance, np.float32).ravel()
        self.transmittance = np.asarray(transmittance, np.float32).ravel()
        self.tir_reflectance = tir_reflectance
        self.tir_transmittance = tir_transmittance
        self.sunlit_temperature = sunlit_temperature
        self.shaded_temperature = shaded_temperature

    def struct(self):
        return SurfaceParameters(_ptr(self.reflectance) if self.reflectance.size else None,
                                 self.reflectance.size,
                                 _ptr(self.transmittance) if self.transmittance.size else None,
                                 self.transmittance.size, self.tir_reflectance,
                                 self.tir_transmittance, self.sunlit_temperature,
                                 self.shaded_temperature)


def ground_surface():
    """FacetRTParameters::ground's default (facetrtcore.cpp:143)."""
    return Surface([0.20], [0.0], 0.05, 0.0, 305.0, 295.0)


def spectral_parameters(wavelengths, leaf_facet_count, object_surface=None, ground=None,
                        materials=(), material_indices=None, texture_factors=None,
                        background_angular_strength=0.0, sky_temperature=250.0,
                        accelerated=False):
    """A SpectralParameters struct plus the arrays it points to (keep both)."""
    keep = {"wl": _f32(wavelengths)}
    obj = object_surface or Surface([0.10], [0.05])
    gnd = ground or ground_surface()
    mats = list(materials)
    keep["surfaces"] = [obj, gnd] + mats
    arr = None
    if mats:
        arr = (SurfaceParameters * len(mats))(*[m.struct() for m in mats])
        keep["mats"] = arr
    if material_indices is not None:
        keep["mi"] = np.ascontiguousarray(material_indices, np.uint32)
    if texture_factors is not None:
        keep["tex"] = _f32(texture_factors)
    p = SpectralParameters(_ptr(keep["wl"]), keep["wl"].size, obj.struct(), gnd.struct(),
                           C.cast(arr, C.c_void_p) if arr is not None else None, len(mats),
                           _ptr(keep["mi"]) if "mi" in keep else None,
                           _ptr(keep["tex"]) if "tex" in keep else None, leaf_facet_count,
                           background_angular_strength, sky_temperature, 1 if accelerated else 0)
    return p, keep


class EnergySurface(Surface):
    """SurfaceParameters with the energy-balance fields
    (facetrtcore.cpp:113-138); the defaults are the reference's."""

    def __init__(self, reflectance=(0.10,), transmittance=(0.05,), tir_reflectance=0.03,
                 tir_transmittance=0.0, sunlit_temperature=300.0, shaded_temperature=296.0,
                 energy_reflectance=(), energy_transmittance=(), surface_resistance=120.0,
                 specific_heat=1180.0, density=1800.0, thermal_conductivity=1.55,
                 soil_moisture=0.25, heat_capacity_per_area=60000.0, soil_temperature_method=1,
                 photovoltaic=False, vegetation=True, pv_eta25=0.22, pv_gamma=-0.0035,
                 pv_bifaciality=0.0, convective_scale=1.0):
        super().__init__(reflectance, transmittance, tir_reflectance, tir_transmittance,
                         sunlit_temperature, shaded_temperature)
        self.energy_reflectance = np.asarray(energy_reflectance, np.float32).ravel()
        self.energy_transmittance = np.asarray(energy_transmittance, np.float32).ravel()
        self.surface_resistance = surface_resistance
        self.specific_heat = specific_heat
        self.density = density
        self.thermal_conductivity = thermal_conductivity
        self.soil_moisture = soil_moisture
        self.heat_capacity_per_area = heat_capacity_per_area
        self.soil_temperature_method = soil_temperature_method
        self.photovoltaic = photovoltaic
        self.vegetation = vegetation
        self.pv_eta25 = pv_eta25
        self.pv_gamma = pv_gamma
        self.pv_bifaciality = pv_bifaciality
        self.convective_scale = convective_scale

    def energy_struct(self):
        er, et = self.energy_reflectance, self.energy_transmittance
        return EnergySurfaceParameters(
            self.struct(), _ptr(er) if er.size else None, er.size, _ptr(et) if et.size else None,
            et.size, self.surface_resistance, self.specific_heat, self.density,
            self.thermal_conductivity, self.soil_moisture, self.heat_capacity_per_area,
            self.soil_temperature_method, 1 if self.photovoltaic else 0,
            1 if self.vegetation else 0, self.pv_eta25, self.pv_gamma, self.pv_bifaciality,
            self.convective_scale)


def energy_parameters(leaf_facet_count, materials=(), material_indices=None,
                      texture_factors=None, background_angular_strength=0.0, wavelengths=(),
                      sky_temperature=250.0, time_step=1800.0, coupling_iterations=20,
                      temperature_tolerance=0.05, temperature_relaxation=0.5,
                      vegetation_temperature_method=0, solver_iterations=64, solver_tolerance=0.0,
                      precision=PRECISION_FP32):
    """runFacetEBCore's settings (defaults as the reference's XML defaults,
    facetrtcore.cpp:3196-3233): an EnergyParameters struct plus the arrays it
    points to (keep both)."""
    mats = list(materials)
    keep = {"surfaces": mats, "wl": _f32(wavelengths)}
    arr = None
    if mats:
        arr = (EnergySurfaceParameters * len(mats))(*[m.energy_struct() for m in mats])
        keep["mats"] = arr
    if material_indices is not None:
        keep["mi"] = np.ascontiguousarray(material_indices, np.uint32)
    if texture_factors is not None:
        keep["tex"] = _f32(texture_factors)
    p = EnergyParameters(C.cast(arr, C.c_void_p) if arr is not None else None, len(mats),
                         _ptr(keep["mi"]) if "mi" in keep else None,
                         _ptr(keep["tex"]) if "tex" in keep else None, leaf_facet_count,
                         background_angular_strength,
                         _ptr(keep["wl"]) if keep["wl"].size else None, keep["wl"].size,
                         sky_temperature, time_step, coupling_iterations, temperature_tolerance,
                         temperature_relaxation, vegetation_temperature_method, solver_iterations,
                         solver_tolerance, precision)
    return p, keep


def shortwave_windows(total_shortwave, cos_zenith, direct=None, diffuse=None,
                      direct_fraction=0.8, window_width=100, wavelengths=()):
    """The node's spectral-acceleration windows and per-band spectral
    irradiance: (windows (n, 3) [direct normal, diffuse, centre sample],
    ShortwaveWindow array, band_direct, band_diffuse)."""
    lib = load()
    d = None if direct is None else _f32(direct)
    f = None if diffuse is None else _f32(diffuse)
    n = 0 if d is None or f is None else min(d.size, f.size)
    spec = ShortwaveSpectrum(_ptr(d) if d is not None else None,
                             _ptr(f) if f is not None else None, n, direct_fraction, window_width)
    wl = _f32(wavelengths)
    bd = np.zeros(wl.size, np.float32)
    bf = np.zeros(wl.size, np.float32)
    count = _u32(0)
    lib.facetcu_shortwave_windows(C.byref(spec), total_shortwave, cos_zenith,
                                  _ptr(wl) if wl.size else None, wl.size, None, 0,
                                  C.byref(count), None, None)  # counts the windows
    cap = count.value
    arr = (ShortwaveWindow * max(cap, 1))()
    rc = lib.facetcu_shortwave_windows(C.byref(spec), total_shortwave, cos_zenith,
                                       _ptr(wl) if wl.size else None, wl.size,
                                       C.cast(arr, C.c_void_p), cap, C.byref(count), _ptr(bd),
                                       _ptr(bf))
    _host_check(rc)
    win = np.array([[w.direct_normal, w.diffuse, w.energy_band] for w in arr[:count.value]],
                   np.float64).reshape(-1, 3)
    return win, arr, bd, bf


def _floats(ptr, n):
    return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_float)), (n,)).copy() if n else \
        np.zeros(0, np.float32)


def project_xml_view(path):
    """The XML view of a project.json (facetInputView)."""
    lib = load()
    n = C.c_uint64(0)
    _host_check(lib.facetcu_project_xml_view(os.fsencode(path), None, 0, C.byref(n)))
    buf = C.create_string_buffer(n.value + 1)
    _host_check(lib.facetcu_project_xml_view(os.fsencode(path), buf, n.value + 1, C.byref(n)))
    return buf.value.decode("utf-8")


def solar_position(year, month, day, hour, minute, second, *, timezone, longitude, latitude,
                   delta_t=0.0, elevation=0.0, pressure=1010.0, temperature=10.0,
                   atmos_refract=0.5667):
    """The sun's topocentric (zenith, azimuth) in degrees, azimuth eastward
    from north (spa_data's inputs and SPA_ZA's outputs)."""
    lib = load()
    inp = SolarInput(year, month, day, hour, minute, second, delta_t, timezone, longitude,
                     latitude, elevation, pressure, temperature, atmos_refract)
    z, a, err = C.c_double(), C.c_double(), C.c_int32()
    _host_check(lib.facetcu_solar_position(C.byref(inp), C.byref(z), C.byref(a), C.byref(err)))
    return z.value, a.value


def faceteb_sun(julian_time, latitude, longitude, pressure, air_temperature):
    """updateSolarPosition: a FacetEB node's (zenith, azimuth) as float32."""
    lib = load()
    z, a = C.c_float(), C.c_float()
    _host_check(lib.facetcu_faceteb_sun(julian_time, latitude, longitude, pressure,
                                        air_temperature, C.byref(z), C.byref(a)))
    return np.float32(z.value), np.float32(a.value)


def dem_height_field(path):
    """A DEM as the project loader reads it (readDemHeightField):
    (values (height, width) float32, rows north to south, with nodata set to
    the minimum; minimum)."""
    lib = load()
    w, h, lo = C.c_int32(0), C.c_int32(0), C.c_float(0)
    path = os.fsencode(path)
    _host_check(lib.facetcu_dem_height_field(path, C.byref(w), C.byref(h), C.byref(lo), None, 0))
    out = np.empty((h.value, w.value), np.float32)
    _host_check(lib.facetcu_dem_height_field(path, C.byref(w), C.byref(h), C.byref(lo),
                                             out.ctypes.data, out.size))
    return out, float(lo.value)


class Project:
    """A HiStream XML project read by the library (facetcu_project_load):
    the scene (vertices (3F, 6), material indices, texture factors), its
    materials and the FacetRT parameters."""

    def __init__(self, path):
        self.lib = load()
        self.h = C.c_void_p()
        rc = self.lib.facetcu_project_load(os.fsencode(path), C.byref(self.h))
        _host_check(rc)
        info = ProjectInfo()
        self.lib.facetcu_project_get_info(self.h, C.byref(info))
        self.info = info.as_dict()
        F = info.facet_count
        self.vertices = np.zeros((3 * F, 6), np.float32)
        self.material_indices = np.zeros(F, np.uint32)
        self.texture_factors = np.zeros(F, np.float32)
        self.lib.facetcu_project_get_geometry(self.h, _ptr(self.vertices),
                                              _ptr(self.material_indices),
                                              _ptr(self.texture_factors))

    def material(self, index):
        """Material `index` (material_count: the parameters' object surface,
        material_count + 1: their ground) as a dict of its fields."""
        m = EnergySurfaceParameters()
        comp = _u32(0)
        self._check(self.lib.facetcu_project_get_material(self.h, index, C.byref(m),
                                                          C.byref(comp)))
        o = m.optics
        d = {"reflectance": _floats(o.reflectance, o.reflectance_count),
             "transmittance": _floats(o.transmittance, o.transmittance_count),
             "energy_reflectance": _floats(m.energy_reflectance, m.energy_reflectance_count),
             "energy_transmittance": _floats(m.energy_transmittance,
                                             m.energy_transmittance_count),
             "tir_reflectance": o.tir_reflectance, "tir_transmittance": o.tir_transmittance,
             "sunlit_temperature": o.sunlit_temperature,
             "shaded_temperature": o.shaded_temperature, "output_component": comp.value}
        for k, _ in EnergySurfaceParameters._fields_[5:]:
            d[k] = getattr(m, k)
        return d

    def spectral_parameters(self):
        """SpectralParameters for spectralOptics / solveBands (valid while
        this project lives)."""
        p = SpectralParameters()
        self._check(self.lib.facetcu_project_spectral_parameters(self.h, C.byref(p)))
        return p

    def _check(self, rc):
        if rc != OK:
            raise ValueError("invalid project request")

    def close(self):
        if self.h:
            self.lib.facetcu_project_release(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def device_count():
    lib = load()
    n = C.c_int(0)
    lib.facetcu_device_count(C.byref(n))
    return n.value


def _f32(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    if shape is not None:
        a = a.reshape(shape)
    return a


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


class FacetrtCuda:
    """Host object with the interface of facetvk::FacetrtVulkan.

    Vertices are an (n, 6) float32 array [px, py, pz, nx, ny, nz] (or
    (F, 3, 6)); optics an (S, 4) float32 array [rho, tau, emission, direct].
    """

    def __init__(self):
        self.lib = load()
        h = C.c_void_p()
        rc = self.lib.facetcu_create(C.byref(h))
        if rc != OK:
            raise FacetcuError(rc, "facetcu_create failed")
        self.h = h
        self.diagnostics = None

    def close(self):
        if self.h:
            self.lib.facetcu_release(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc):
        if rc == OK:
            return
        msg = (self.lib.facetcu_last_error(self.h) or b"").decode()
        if rc == INVALID_ARGUMENT:
            raise ValueError(msg)
        if rc == LOGIC_ERROR:
            raise LogicError(rc, msg)
        if rc == RUNTIME_ERROR:
            raise RuntimeError(msg)
        if rc == OVERFLOW_ERROR:
            raise OverflowError(msg)
        if rc == NOT_CONVERGED:
            raise NotConverged(rc, msg)
        raise FacetcuError(rc, msg)

    # -- facetvk::FacetrtVulkan -------------------------------------------
    def initialize(self, raster_width=1024, raster_height=None, max_fragments_per_pixel=64,
                   gpu_index=0, periodic_neighbor_count=0, periodic_size_x=1.0,
                   periodic_size_z=1.0):
        cfg = Config()
        cfg.raster_width = raster_width
        cfg.raster_height = raster_height if raster_height is not None else raster_width
        cfg.max_fragments_per_pixel = max_fragments_per_pixel
        cfg.edge_hash_capacity = 0
        cfg.enable_validation = False
        cfg.gpu_index = gpu_index
        cfg.periodic_neighbor_count = periodic_neighbor_count
        cfg.periodic_size_x = periodic_size_x
        cfg.periodic_size_z = periodic_size_z
        self._check(self.lib.facetcu_initialize(self.h, C.byref(cfg)))
        return self

    def destroy(self):
        self._check(self.lib.facetcu_destroy(self.h))

    def stream(self):
        s = C.c_void_p()
        self._check(self.lib.facetcu_get_stream(self.h, C.byref(s)))
        return s.value

    def setGeometry(self, vertices):
        v = _f32(vertices).reshape(-1, 6)
        self.facet_count = len(v) // 3
        self._check(self.lib.facetcu_set_geometry(self.h, _ptr(v), len(v)))

    def setRasterBounds(self, minimum, maximum):
        mn = _f32(minimum, (3,))
        mx = _f32(maximum, (3,))
        self._check(self.lib.facetcu_set_raster_bounds(self.h, _ptr(mn), _ptr(mx)))

    def buildVisibilityGraph(self, directions):
        d = _f32(directions).reshape(-1, 3)
        diag = GraphDiagnostics()
        rc = self.lib.facetcu_build_visibility_graph(self.h, _ptr(d), len(d), C.byref(diag))
        self.diagnostics = diag.as_dict()
        self._check(rc)
        return self.diagnostics

    def computeSunlitFraction(self, sun):
        sun = _f32(sun, (3,))
        out = np.zeros(2 * self.facet_count, np.float32)
        d = Direction(*[float(x) for x in sun])
        self._check(self.lib.facetcu_compute_sunlit_fraction(self.h, C.byref(d), _ptr(out)))
        return out

    def buildHemisphereGraph(self, sample_uv, sample_dir, rays_per_side, top_k, sample_sets):
        cfg = HemisphereConfig(rays_per_side, top_k, sample_sets, 0)
        uv = _f32(sample_uv)
        dr = _f32(sample_dir)
        if uv.size != 2 * rays_per_side * sample_sets or dr.size != 3 * rays_per_side * sample_sets:
            raise ValueError("sample tables must hold sets * rays_per_side * (2 | 3) floats")
        diag = GraphDiagnostics()
        dropped = C.c_uint64()
        rc = self.lib.facetcu_build_hemisphere_graph(self.h, C.byref(cfg), _ptr(uv), _ptr(dr),
                                                     C.byref(diag), C.byref(dropped))
        self.diagnostics = diag.as_dict()
        self._check(rc)
        return self.diagnostics, dropped.value

    def hemisphereSunlit(self, sun, sample_uv, samples, sample_sets):
        sun = _f32(sun, (3,))
        uv = _f32(sample_uv)
        if uv.size != 2 * samples * sample_sets:
            raise ValueError("sample_uv must hold sets * samples * 2 floats")
        out = np.zeros(2 * self.facet_count, np.float32)
        d = Direction(*[float(x) for x in sun])
        self._check(self.lib.facetcu_hemisphere_sunlit(self.h, C.byref(d), samples, sample_sets,
                                                       _ptr(uv), _ptr(out)))
        return out

    def graph(self):
        """(row_offsets, neighbors, counts, denominators, sky_counts) as numpy arrays."""
        S = C.c_uint32()
        n = C.c_uint64()
        self._check(self.lib.facetcu_graph_size(self.h, C.byref(S), C.byref(n)))
        rows = np.zeros(S.value + 1, np.uint32)
        edges = np.zeros(2 * max(n.value, 1), np.uint32)
        den = np.zeros(S.value, np.uint32)
        sky = np.zeros(S.value, np.uint32)
        self._check(self.lib.facetcu_get_graph(self.h, _ptr(rows), _ptr(edges), _ptr(den), _ptr(sky)))
        e = edges[:2 * n.value]
        return rows, e[0::2].copy(), e[1::2].copy(), den, sky

    def setGraph(self, row_offsets, neighbors, counts, denominators, sky_counts):
        rows = np.ascontiguousarray(row_offsets, np.uint32)
        e = np.empty(2 * max(len(neighbors), 1), np.uint32)
        e[0:2 * len(neighbors):2] = neighbors
        e[1:2 * len(neighbors):2] = counts
        den = np.ascontiguousarray(denominators, np.uint32)
        sky = np.ascontiguousarray(sky_counts, np.uint32)
        self._check(self.lib.facetcu_set_graph(self.h, len(den), _ptr(rows), _ptr(e), _ptr(den),
                                               _ptr(sky)))

    def solve(self, optics, sky_radiosity, iterations=64, relaxation=1.0):
        o = _f32(optics).reshape(-1, 4)
        out = np.zeros(max(len(o), 2 * self.facet_count), np.float32)
        it = C.c_uint32()
        md = C.c_float()
        self._check(self.lib.facetcu_solve(self.h, _ptr(o), len(o), sky_radiosity, iterations,
                                           relaxation, _ptr(out), C.byref(it), C.byref(md)))
        return {"radiosity": out, "iterations": it.value, "maxDelta": md.value}

    def solveAccelerated(self, optics, sky_radiosity, initial=None, maximum_iterations=64,
                         batch_iterations=8, tolerance=1.0e-4, relaxation=1.0):
        o = _f32(optics).reshape(-1, 4)
        init = None if initial is None else _f32(initial)
        if init is not None and len(init) != len(o):
            raise ValueError("Initial radiosity must contain one finite non-negative value per surface")
        out = np.zeros(max(len(o), 2 * self.facet_count), np.float32)
        it = C.c_uint32()
        md = C.c_float()
        self._check(self.lib.facetcu_solve_accelerated(
            self.h, _ptr(o), len(o), sky_radiosity, _ptr(init), maximum_iterations,
            batch_iterations, tolerance, relaxation, _ptr(out), C.byref(it), C.byref(md)))
        return {"radiosity": out, "iterations": it.value, "maxDelta": md.value}

    def incidentIrradiance(self, radiosity, optics, sky_radiosity):
        o = _f32(optics).reshape(-1, 4)
        r = _f32(radiosity)
        if len(r) != len(o):
            raise ValueError("Incident irradiance requires a completed solve and visibility graph")
        out = np.zeros(len(o), np.float32)
        self._check(self.lib.facetcu_incident_irradiance(self.h, _ptr(r), _ptr(o), len(o),
                                                         sky_radiosity, _ptr(out)))
        return out

    # -- batched extension ------------------------------------------------
    def solveBatched(self, reflectance, transmittance, sky, beam, direct_geometry=None,
                     emission=None, precision=PRECISION_FP32, tolerance=1e-6,
                     maximum_iterations=1000, initial=None, panel_width=0, raise_on_nonconvergence=True,
                     flags=0, warm_start=None):
        """reflectance/transmittance/emission: (bands, S); sky, beam: (bands,);
        direct_geometry: (suns, S).  Returns radiosity (suns*bands, S) and the result dict.
        warm_start: None (WARM_GIVEN when `initial` is given, else WARM_NONE) or WARM_MLP."""
        rho = _f32(reflectance)
        tau = _f32(transmittance)
        bands = rho.shape[0]
        S = rho.shape[1]
        if S != 2 * self.facet_count or tau.shape != rho.shape or \
                (emission is not None and np.shape(emission) != rho.shape) or \
                len(np.ravel(sky)) != bands or len(np.ravel(beam)) != bands:
            raise ValueError("band arrays must be (bands, 2 * facets) with one sky/beam per band")
        emis = None if emission is None else _f32(emission)
        dgeo = None if direct_geometry is None else _f32(direct_geometry).reshape(-1, S)
        suns = 1 if dgeo is None else dgeo.shape[0]
        if warm_start is None:
            warm_start = WARM_GIVEN if initial is not None else WARM_NONE
        cfg = BatchConfig(bands, suns, precision, warm_start, maximum_iterations, tolerance,
                          panel_width, flags)
        init = None if initial is None else _f32(initial)
        if init is not None and init.size != suns * bands * S:
            raise ValueError("initial radiosity must hold suns * bands * 2F values")
        out = np.zeros((suns * bands, S), np.float32)
        res = BatchResult()
        rc = self.lib.facetcu_solve_batched(self.h, C.byref(cfg), _ptr(rho), _ptr(tau), _ptr(emis),
                                            _ptr(_f32(sky)), _ptr(_f32(beam)), _ptr(dgeo),
                                            _ptr(init), _ptr(out), C.byref(res))
        if rc == NOT_CONVERGED and not raise_on_nonconvergence:
            return out, res.as_dict()
        self._check(rc)
        return out, res.as_dict()

    # -- scene batches ---------------------------------------------------------
    def sceneBatch(self, models):
        """Make this context the disjoint union of other contexts' geometry and
        graphs; returns the side offsets (len(models) + 1) and diagnostics."""
        handles = (C.c_void_p * len(models))(*[m.h for m in models])
        offsets = np.zeros(len(models) + 1, np.uint32)
        d = GraphDiagnostics()
        self._check(self.lib.facetcu_scene_batch(self.h, C.cast(handles, C.c_void_p), len(models),
                                                 _ptr(offsets), C.byref(d)))
        self.facet_count = int(offsets[-1]) // 2
        return offsets, {k: getattr(d, k) for k, _ in d._fields_}

    # -- spectral optics and the band loop ------------------------------------
    def spectralOptics(self, parameters, sunlit, sun, band):
        """makeSpectralOptics for one band: (2F, 4) float32."""
        lit = _f32(sunlit)
        out = np.zeros((lit.size, 4), np.float32)
        d = Direction(*[float(x) for x in np.ravel(sun)[:3]])
        self._check(self.lib.facetcu_spectral_optics(self.h, C.byref(parameters), _ptr(lit),
                                                     C.byref(d), band, _ptr(out)))
        return out

    def solveBands(self, parameters, sunlit, sun):
        """The runGpu band loop: (band radiosity (bands, 2F), light
        enhancement (2F,), result dict)."""
        lit = _f32(sunlit)
        bands = np.zeros((parameters.band_count, lit.size), np.float32)
        enh = np.zeros(lit.size, np.float32)
        d = Direction(*[float(x) for x in np.ravel(sun)[:3]])
        res = BandResult()
        self._check(self.lib.facetcu_solve_bands(self.h, C.byref(parameters), _ptr(lit),
                                                 C.byref(d), _ptr(bands), _ptr(enh),
                                                 C.byref(res)))
        return bands, enh, res.as_dict()

    # -- FacetEB node --------------------------------------------------------
    def facetebNode(self, parameters, meteo, sun, sunlit, windows, temperature,
                    band_direct=None, band_diffuse=None, fields=ENERGY_FIELDS):
        """One FacetEB time node: (dict of per-side fields, result dict).
        windows is the ShortwaveWindow array of shortwave_windows();
        temperature the state at the node start (2F,); meteo a dict or Meteo."""
        lit = _f32(sunlit)
        S = lit.size
        if isinstance(meteo, dict):
            meteo = Meteo(**meteo)
        out = {}
        for k in fields:
            n = S * parameters.band_count if k == "band_output" else S
            if k == "band_output" and n == 0:
                continue
            out[k] = np.zeros(n, np.float32)
        out["temperature"] = _f32(temperature).copy()
        f = EnergyFields(**{k: _ptr(v) for k, v in out.items()})
        nwin = len(windows) if windows is not None else 0
        bd = None if band_direct is None else _f32(band_direct)
        bf = None if band_diffuse is None else _f32(band_diffuse)
        d = Direction(*[float(x) for x in np.ravel(sun)[:3]])
        res = EnergyResult()
        self._check(self.lib.facetcu_faceteb_node(
            self.h, C.byref(parameters), C.byref(meteo), C.byref(d), _ptr(lit),
            C.cast(windows, C.c_void_p) if nwin else None, nwin, _ptr(bd), _ptr(bf), C.byref(f),
            C.byref(res)))
        if "band_output" in out:
            out["band_output"] = out["band_output"].reshape(parameters.band_count, S)
        return out, res.as_dict()

    # -- sensor images ---------------------------------------------------------
    def renderSensorImage(self, sensor_struct, values, wavelengths):
        """Images of per-side values seen by a sensor: (image (bands, H, W)
        float32, side index (H, W) int32, info dict)."""
        vals = _f32(values).reshape(-1, 2 * self.facet_count) if np.size(values) else \
            np.zeros((0, 2 * self.facet_count), np.float32)
        wl = _f32(wavelengths).ravel()
        nb = len(vals)
        if wl.size < nb:
            raise ValueError("one wavelength per band is required")
        W = sensor_struct.width or 512
        H = sensor_struct.height or 512
        img = np.zeros((nb, H, W), np.float32)
        idx = np.zeros((H, W), np.int32)
        info = ImageInfo()
        self._check(self.lib.facetcu_render_sensor_image(
            self.h, C.byref(sensor_struct), _ptr(vals) if nb else None, nb,
            _ptr(wl) if nb else None, _ptr(img) if nb else None, _ptr(idx), C.byref(info)))
        return img, idx, info.as_dict()

    # -- learned warm start -------------------------------------------------
    def mlpReset(self, seed=1):
        self._check(self.lib.facetcu_mlp_reset(self.h, seed))

    def mlpLoad(self, path=None):
        """Load warm-start weights (a .npy of 26,432 float32; default: the
        weights shipped with the package, trained by train_mlp.py)."""
        self.mlpSetParameters(np.load(path or WARM_START_WEIGHTS))

    def mlpParameters(self):
        p = np.zeros(MLP_PARAMETERS, np.float32)
        self._check(self.lib.facetcu_mlp_get_parameters(self.h, _ptr(p)))
        return p

    def mlpSetParameters(self, params):
        p = _f32(params)
        if p.size != MLP_PARAMETERS:
            raise ValueError("MLP parameter vector must hold 26,432 floats")
        self._check(self.lib.facetcu_mlp_set_parameters(self.h, _ptr(p)))

    def mlpForward(self, x):
        x = _f32(x).reshape(-1, MLP_INPUTS)
        y = np.zeros((len(x), MLP_OUTPUTS), np.float32)
        self._check(self.lib.facetcu_mlp_forward(self.h, _ptr(x), len(x), _ptr(y)))
        return y

    def mlpForwardTensor(self, x):
        """The forward pass on the tensor cores (BF16 activations)."""
        x = _f32(x).reshape(-1, MLP_INPUTS)
        y = np.zeros((len(x), MLP_OUTPUTS), np.float32)
        self._check(self.lib.facetcu_mlp_forward_tensor(self.h, _ptr(x), len(x), _ptr(y)))
        return y

    def mlpLossAndGradient(self, x, target):
        x = _f32(x).reshape(-1, MLP_INPUTS)
        t = _f32(target).reshape(-1, MLP_OUTPUTS)
        if len(t) != len(x):
            raise ValueError("x and target must have the same number of rows")
        loss = C.c_float()
        g = np.zeros(MLP_PARAMETERS, np.float32)
        self._check(self.lib.facetcu_mlp_loss_and_gradient(self.h, _ptr(x), _ptr(t), len(x),
                                                           C.byref(loss), _ptr(g)))
        return loss.value, g

    def mlpTrainDevice(self, x_ptr, t_ptr, n, steps, batch, learning_rate=1e-3, seed=1):
        cfg = MlpTrainConfig(steps, batch, learning_rate, seed)
        loss = C.c_float()
        self._check(self.lib.facetcu_mlp_train_device(self.h, x_ptr, t_ptr, n, C.byref(cfg),
                                                      C.byref(loss)))
        return loss.value

    def mlpSamplesDevice(self, cfg, rho_ptr, tau_ptr, emis_ptr, sky_ptr, beam_ptr, dgeo_ptr,
                         converged_ptr, features_ptr, targets_ptr):
        self._check(self.lib.facetcu_mlp_samples_device(
            self.h, C.byref(cfg), rho_ptr, tau_ptr, emis_ptr, sky_ptr, beam_ptr, dgeo_ptr,
            converged_ptr, features_ptr, targets_ptr))

    def autotuneBatched(self, cfg, rho_ptr, tau_ptr, emis_ptr, sky_ptr, beam_ptr, dgeo_ptr,
                        out_ptr, cache_path=None):
        """Time the panel widths on short solves of these device inputs and keep
        the fastest for later solves with panel_width = 0; returns it."""
        p = C.c_uint32()
        self._check(self.lib.facetcu_autotune_batched(
            self.h, C.byref(cfg), rho_ptr, tau_ptr, emis_ptr, sky_ptr, beam_ptr, dgeo_ptr, out_ptr,
            os.fsencode(cache_path) if cache_path else None, C.byref(p)))
        return p.value

    def solveBatchedDevice(self, cfg, rho_ptr, tau_ptr, emis_ptr, sky_ptr, beam_ptr, dgeo_ptr,
                           init_ptr, out_ptr):
        """Device-pointer variant; all pointers are integers (or None)."""
        res = BatchResult()
        rc = self.lib.facetcu_solve_batched_device(
            self.h, C.byref(cfg), rho_ptr, tau_ptr, emis_ptr, sky_ptr, beam_ptr, dgeo_ptr,
            init_ptr, out_ptr, C.byref(res))
        if rc not in (OK, NOT_CONVERGED):
            self._check(rc)
        return res.as_dict()
