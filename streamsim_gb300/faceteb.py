"""The FacetEB caller: a sequence of time nodes on one scene and graph.

runFacetEBCore (models/histream/src/facetrt/facetrtcore.cpp:3164-4154)
reads a meteorology table, then for every node of [startNode, endNode)
places the sun, rasters it, seeds the temperatures from the air at the
first node, solves the node (shortwave windows, longwave coupling, sensor
bands) and writes the node's energy record; at the end it writes
faceteb.json.  Here each node is one facetcu_faceteb_node call on the
device; this module keeps the reference's host-side sequence and file
formats:

  read_meteorology / default_meteorology   :3243-3273
  time_token                               :3274-3288 (DOY<d>_<hh>-<mm>)
  .facet_steps/components.bin              :3419-3430 (uint8 per facet)
  .facet_steps/energy_T=<token>.bin        :3909-3932 (per side: T, radiosity,
                                           shortwave, longwave, net, sensible,
                                           latent, storage, sunlit, then bands;
                                           float32 little-endian)
  faceteb.json                             :4085-4139

  solar_sun                                :3290-3327 (updateSolarPosition)

The sun of each node is the caller's sun_for(row) or, by default,
updateSolarPosition's: the node's date and local time (2019, UTC+8) at the
site's latitude and longitude, through facetcu_faceteb_sun (the reference
calls NREL's SPA there; the library follows Meeus's published solar
formulas, about 0.01 deg from SPA).
"""
import json
import math
import os

import numpy as np

from . import facetcu


def read_meteorology(path):
    """Rows of a FacetEB meteorology file: a header line, then whitespace
    separated julianTime, air temperature (C), vapour pressure (hPa),
    pressure (hPa), wind speed (m/s), shortwave and longwave (W/m2); rows
    that do not parse are skipped, the node index counts every data row."""
    rows = []
    with open(path) as f:
        f.readline()
        for node, line in enumerate(f):
            parts = line.split()
            try:
                v = [float(x) for x in parts[:7]]
            except ValueError:
                continue
            if len(v) < 7:
                continue
            rows.append({"node": node, "julian_time": v[0], "air_temperature": v[1],
                         "vapor_pressure": v[2], "pressure": v[3], "wind_speed": v[4],
                         "shortwave": v[5], "longwave": v[6]})
    return rows


def default_meteorology(end_node, time_step=1800.0):
    """The reference's table when no file is given: neutral weather, one row
    per node at julianTime 1 + node * dTime / 86400."""
    return [{"node": n, "julian_time": float(np.float32(1.0) + np.float32(n) *
                                              np.float32(time_step) / np.float32(86400.0)),
             "air_temperature": 25.0, "vapor_pressure": 15.0, "pressure": 839.0,
             "wind_speed": 1.0, "shortwave": 0.0, "longwave": 320.0}
            for n in range(end_node)]


def time_token(julian_time):
    """DOY<day>_<hh>-<mm> of a julian time (minutes rounded)."""
    day = int(math.floor(julian_time))
    minutes = int(math.floor((float(julian_time) - day) * 1440.0 + 0.5))  # lround
    if minutes >= 1440:
        day += minutes // 1440
        minutes %= 1440
    return f"DOY{day}_{minutes // 60:02d}-{minutes % 60:02d}"


def solar_sun(latitude=40.0, longitude=116.0):
    """sun_for(row) -> (zenith, azimuth) of updateSolarPosition at the site
    (<Latitude>, <Longitude>; the reference's defaults 40 N, 116 E)."""
    def sun_for(row):
        return facetcu.faceteb_sun(row["julian_time"], latitude, longitude, row["pressure"],
                                   row["air_temperature"])
    return sun_for


def _meteo(row):
    return {k: float(row[k]) for k in ("air_temperature", "vapor_pressure", "pressure",
                                        "wind_speed", "shortwave", "longwave")}


class Run:
    """A FacetEB run on a model whose graph is built.

    materials: facetcu.EnergySurface list (an `output_component` attribute,
    0-5, is written to components.bin); material_indices per facet.
    sun_for(node_row) -> (zenith, azimuth) in degrees; sunlit_for(direction)
    -> per-side sunlit fraction (default: the model's sun raster)."""

    def __init__(self, model, leaf_facet_count, materials, material_indices=None,
                 texture_factors=None, wavelengths=(), spectrum=None, direct_fraction=0.8,
                 window_width=100, sunlit_for=None, **settings):
        self.model = model
        self.leaf = int(leaf_facet_count)
        self.materials = list(materials)
        self.mi = None if material_indices is None else np.asarray(material_indices, np.uint32)
        self.tex = texture_factors
        self.wavelengths = [float(w) for w in wavelengths]
        self.spectrum = spectrum
        self.direct_fraction = direct_fraction
        self.window_width = window_width
        self.sunlit_for = sunlit_for or model.computeSunlitFraction
        self.settings = settings
        self.params, self._keep = facetcu.energy_parameters(
            self.leaf, self.materials, self.mi, self.tex,
            wavelengths=self.wavelengths, **settings)

    def components(self, facet_count):
        """components.bin: 1 for ground facets, else the material's output
        component (0 when unknown)."""
        out = np.zeros(facet_count, np.uint8)
        for f in range(self.leaf):
            m = self.mi[f] if self.mi is not None else None
            if m is not None and m < len(self.materials):
                out[f] = getattr(self.materials[m], "output_component", 0)
        out[self.leaf:] = 1
        return out

    def node(self, row, zenith, azimuth, temperature):
        """One node: (fields, result, sunlit)."""
        sun = facetcu.sun_direction(zenith, azimuth)
        lit = self.sunlit_for(sun)
        d, f = (None, None) if self.spectrum is None else self.spectrum
        _, windows, bd, bf = facetcu.shortwave_windows(
            max(0.0, row["shortwave"]), max(0.0, float(sun[1])), d, f, self.direct_fraction,
            self.window_width, self.wavelengths)
        count = len(facetcu.shortwave_windows(max(0.0, row["shortwave"]), max(0.0, float(sun[1])),
                                              d, f, self.direct_fraction, self.window_width)[0])
        fields, res = self.model.facetebNode(self.params, _meteo(row), sun, lit,
                                             windows if count else None, temperature, bd, bf)
        return fields, res, lit

    def run(self, meteorology, sun_for=None, start_node=0, end_node=None, output_dir=None,
            vertices=None, graph=None, progress=print, latitude=40.0, longitude=116.0):
        """Nodes [start_node, end_node) of the meteorology rows.  Writes the
        reference's step records and faceteb.json under output_dir when
        given.  sun_for defaults to solar_sun(latitude, longitude).  Returns
        the per-node results and the last node's fields."""
        sun_for = sun_for or solar_sun(latitude, longitude)
        end_node = len(meteorology) if end_node is None else end_node
        if end_node > len(meteorology):
            raise RuntimeError("FacetEB time range exceeds meteorology rows")
        F = self.model.facet_count
        S = 2 * F
        steps = None
        if output_dir:
            steps = os.path.join(output_dir, ".facet_steps")
            os.makedirs(steps, exist_ok=True)
            self.components(F).tofile(os.path.join(steps, "components.bin"))
        temperature = None
        results = []
        last = None
        all_converged = True
        for node in range(start_node, end_node):
            row = meteorology[node]
            if temperature is None:
                seed = np.float32(np.clip(np.float32(row["air_temperature"]) +
                                          np.float32(273.15), 220.0, 340.0))
                temperature = np.full(S, seed, np.float32)
            zenith, azimuth = sun_for(row)
            fields, res, lit = self.node(row, zenith, azimuth, temperature)
            temperature = fields["temperature"]
            token = time_token(row["julian_time"])
            all_converged = all_converged and bool(res["converged"])
            results.append(dict(res, node=node, token=token))
            if steps:
                cols = [fields["temperature"], fields["radiosity"], fields["shortwave_radiosity"],
                        fields["longwave_radiosity"], fields["net_radiation"],
                        fields["sensible_heat"], fields["latent_heat"], fields["storage_heat"],
                        lit]
                if self.wavelengths:
                    cols += list(fields["band_output"])
                rec = np.stack([np.asarray(c, np.float32) for c in cols], 1)
                rec.astype("<f4").tofile(os.path.join(steps, f"energy_T={token}.bin"))
            if progress:
                progress(f"FACET_CONVERGENCE\t{node}\t{int(res['converged'])}\t"
                         f"{res['coupling_iterations']}\t{res['max_temperature_delta']}\t"
                         f"{res['max_energy_residual']}\t{res['max_energy_residual_equivalent']}")
            last = (fields, res, lit, token)
        if output_dir and last is not None:
            self._write_result(os.path.join(output_dir, "faceteb.json"), last, all_converged,
                               vertices, graph)
        return results, (last[0] if last else None)

    def _write_result(self, path, last, all_converged, vertices, graph):
        fields, res, lit, token = last
        g = graph or {}
        enhancement = np.maximum(0.0, fields["shortwave_radiosity"] - fields["diffuse_radiosity"])
        doc = {
            "backend": "CUDA GPU Facet RT-EB coupled",
            "componentFile": ".facet_steps/components.bin",
            "facetCount": self.model.facet_count, "leafFacetCount": self.leaf, "time": token,
            "vertexPositions": ([] if vertices is None else
                                np.asarray(vertices, np.float32).reshape(-1, 6)[:, :3]
                                .ravel().tolist()),
            "graph": {"directedEdges": int(g.get("directed_edge_count", 0)),
                      "closureError": float(g.get("max_closure_error", 0.0)),
                      "fragmentOverflow": int(g.get("fragment_overflow", 0)),
                      "hashOverflow": int(g.get("hash_overflow", 0))},
            "iterations": int(max(res["shortwave_sweeps"], res["longwave_sweeps"])),
            "couplingIterations": res["coupling_iterations"],
            "temperatureDelta": res["max_temperature_delta"],
            "converged": all_converged,
            "energyResidual": res["max_energy_residual"], "energyResidualUnits": "W m-2",
            "energyResidualTemperatureEquivalent": res["max_energy_residual_equivalent"],
            "temperatureTolerance": self.params.temperature_tolerance,
            "iterationBudget": self.params.coupling_iterations,
            "sunlit": np.asarray(lit, np.float32).tolist(),
            "radiosity": fields["radiosity"].tolist(),
            "lightEnhancement": enhancement.astype(np.float32).tolist(),
            "temperature": fields["temperature"].tolist(),
            "netRadiation": fields["net_radiation"].tolist(),
            "sensibleHeat": fields["sensible_heat"].tolist(),
            "latentHeat": fields["latent_heat"].tolist(),
            "storageHeat": fields["storage_heat"].tolist(),
            "photovoltaicPower": fields["photovoltaic_power"].tolist(),
        }
        with open(path, "w") as f:
            json.dump(doc, f)
