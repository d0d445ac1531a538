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
  photovoltaic_node_<node>.csv,
  photovoltaic_summary.csv                 :3433-3435, 3847-3860
  faceteb_run.json                         :58-73, 3213-3222, 4030-4041, 4144-4147
  process/<model>_T=<time>.bin / .json     :3936-4021

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
import re
import sys

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


def facet_areas(vertices):
    """facetArea (facetrtcore.cpp:704-716) of every facet, in float32 with
    the reference's operation order: 0.5 sqrt(c . c), c = (b - a) x (c - a)."""
    v = np.asarray(vertices, np.float32).reshape(-1, 3, 6)[:, :, :3]
    ea, eb = v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]
    c0 = ea[:, 1] * eb[:, 2] - ea[:, 2] * eb[:, 1]
    c1 = ea[:, 2] * eb[:, 0] - ea[:, 0] * eb[:, 2]
    c2 = ea[:, 0] * eb[:, 1] - ea[:, 1] * eb[:, 0]
    return np.float32(0.5) * np.sqrt((c0 * c0 + c1 * c1) + c2 * c2)


def _g(x):
    """A number as std::ostream writes it by default (6 significant digits)."""
    return format(float(x), ".6g")


PV_SUMMARY_HEADER = ("node,time,area_m2,temperature_C,incident_W,absorbed_W,electric_W,"
                     "net_longwave_W,sensible_W,storage_W,max_residual_W_m2,energy_kWh\n")
PV_NODE_HEADER = ("area_m2,temperature_C,incident_W_m2,absorbed_W_m2,electric_W_m2,residual_W_m2,"
                  "latent_W_m2,effective_W_m2,net_longwave_W_m2,sensible_W_m2,storage_W_m2,"
                  "facet_index\n")


def utc_timestamp():
    """utcTimestamp (facetrtcore.cpp:42-53): %Y-%m-%dT%H:%M:%SZ."""
    import time
    return time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime())


class RunIndex:
    """faceteb_run.json (FacetRunIndex, facetrtcore.cpp:58-73, 3213-3222,
    3436-3437, 4030-4041, 4144-4147): rewritten after every node, keys in
    sorted order with two-space indents as nlohmann::json writes them; a run
    that stops before its end is marked failed."""

    def __init__(self, path, input_path, start, end, tolerance, budget):
        self.path = path
        self.value = {
            "kind": "faceteb-run", "schemaVersion": 1, "status": "running",
            "startedAt": utc_timestamp(), "input": input_path,
            "requested": {"startNode": start, "endNodeExclusive": end},
            "convergence": {"temperatureTolerance_K": float(np.float32(tolerance)),
                            "iterationBudget": budget,
                            "criterion": "temperatureDelta and residual/thermal-response "
                                         "<= temperatureTolerance"},
            "completed": [], "products": []}
        self.write()

    def write(self):
        with open(self.path, "w") as f:
            f.write(json.dumps(self.value, indent=2, sort_keys=True, ensure_ascii=False) + "\n")

    def node(self, node, token, julian_time, res, tolerance, budget):
        self.value["products"] += [f".facet_steps/energy_T={token}.bin",
                                   f"photovoltaic_node_{node}.csv"]
        f32 = lambda x: float(np.float32(x))
        self.value["completed"].append({
            "node": node, "token": token, "julianTime": f32(julian_time),
            "converged": bool(res["converged"]), "iterations": int(res["coupling_iterations"]),
            "iterationBudget": budget, "temperatureDelta": f32(res["max_temperature_delta"]),
            "temperatureTolerance": f32(tolerance),
            "energyResidual": f32(res["max_energy_residual"]), "energyResidualUnits": "W m-2",
            "energyResidualTemperatureEquivalent": f32(res["max_energy_residual_equivalent"])})
        self.write()

    def finish(self, result_name, converged):
        self.value["products"].append(result_name)
        self.value["status"] = "completed" if converged else "non_converged"
        self.value["finishedAt"] = utc_timestamp()
        self.write()

    def fail(self):
        if self.value.get("status") == "running":
            self.value["status"] = "failed"
            self.value["finishedAt"] = utc_timestamp()
            try:
                self.write()
            except OSError:
                pass


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
            vertices=None, graph=None, progress=print, latitude=40.0, longitude=116.0,
            run_index=None, process=(False, False)):
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
        pv = self._pv_facets() if output_dir else []
        area = facet_areas(vertices) if output_dir and vertices is not None else None
        summary = None
        if output_dir:
            summary = open(os.path.join(output_dir, "photovoltaic_summary.csv"), "w")
            summary.write(PV_SUMMARY_HEADER)
            if run_index is not None:
                run_index.value["products"] += ["photovoltaic_summary.csv",
                                                ".facet_steps/components.bin"]
        energy_kwh = 0.0
        try:
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
                if output_dir and area is not None:
                    energy_kwh, pv_area = self._write_pv(output_dir, node, token, fields, area, pv,
                                                         summary, energy_kwh)
                    for kind, on in (("radiation", process[0]), ("energy", process[1]),
                                     ("photovoltaic", pv_area > 0)):
                        if on:
                            self._write_process(output_dir, kind, node, row, token, zenith, azimuth,
                                                fields, res, F, run_index)
                if run_index is not None:
                    run_index.node(node, token, row["julian_time"], res,
                                   self.params.temperature_tolerance, self.params.coupling_iterations)
                if progress:
                    progress(f"FACET_CONVERGENCE\t{node}\t{int(res['converged'])}\t"
                             f"{res['coupling_iterations']}\t{res['max_temperature_delta']}\t"
                             f"{res['max_energy_residual']}\t{res['max_energy_residual_equivalent']}")
                last = (fields, res, lit, token)
        finally:
            if summary is not None:
                summary.close()
        if output_dir and last is not None:
            self._write_result(os.path.join(output_dir, "faceteb.json"), last, all_converged,
                               vertices, graph)
        return results, (last[0] if last else None)

    def _pv_facets(self):
        """Object facets whose material is photovoltaic (surfaceForFacet)."""
        out = []
        if self.mi is None:
            return out
        for f in range(self.leaf):
            m = int(self.mi[f])
            if m < len(self.materials) and self.materials[m].photovoltaic:
                out.append((f, float(np.float32(self.materials[m].pv_bifaciality))))
        return out

    def _write_pv(self, output_dir, node, token, fields, area, pv, summary, energy_kwh):
        """photovoltaic_node_<node>.csv and the photovoltaic_summary.csv row
        (facetrtcore.cpp:3847-3860): per PV facet its area, front-side
        temperature and fluxes, float arithmetic, double area-weighted sums,
        6 significant digits."""
        f32 = np.float32
        T, ab_, inc_ = fields["temperature"], fields["absorbed_shortwave"], fields["incident_shortwave"]
        pvp, net = fields["photovoltaic_power"], fields["net_radiation"]
        sens, lat, stor = fields["sensible_heat"], fields["latent_heat"], fields["storage_heat"]
        pa = pt = pg = pab = pp = plw = ph = ps = pres = 0.0
        lines = [PV_NODE_HEADER]
        for f, bif in pv:
            k = 2 * f
            a = f32(area[f])
            ab = f32(ab_[k] + ab_[k + 1])
            inc = f32(inc_[k] + inc_[k + 1])
            power = f32(pvp[k])
            lw = f32(net[k] - ab)
            res = f32(f32(f32(f32(net[k] - sens[k]) - lat[k]) - stor[k]) - power)
            tc = f32(T[k] - f32(273.15))
            eff = f32(inc_[k] + f32(f32(bif) * inc_[k + 1]))
            lines.append(",".join(_g(x) for x in (a, tc, inc, ab, power, res, lat[k], eff, lw,
                                                  sens[k], stor[k])) + f",{f}\n")
            pa += float(a)
            pt += float(f32(a * tc))
            pg += float(f32(a * inc))
            pab += float(f32(a * ab))
            pp += float(f32(a * power))
            plw += float(f32(a * lw))
            ph += float(f32(a * f32(sens[k])))
            ps += float(f32(a * f32(stor[k])))
            pres = max(pres, abs(float(res)))
        with open(os.path.join(output_dir, f"photovoltaic_node_{node}.csv"), "w") as f:
            f.write("".join(lines))
        if pa > 0:
            energy_kwh += pp * float(self.settings.get("time_step", 1800.0)) / 3600000.0
            summary.write(",".join([str(node), token] + [_g(x) for x in (
                pa, pt / pa, pg, pab, pp, plw, ph, ps, pres, energy_kwh)]) + "\n")
        return energy_kwh, pa

    def _write_process(self, output_dir, kind, node, row, token, zenith, azimuth, fields, res,
                       facet_count, run_index):
        """process/<model>_T=<token>.bin and .json (facetrtcore.cpp:3936-4021):
        per side 3 floats (radiation: shortwave, final longwave radiosity, net
        radiation; photovoltaic: PV power, temperature, absorbed shortwave)
        or 5 (energy: latent, sensible, storage, temperature, net
        radiation), float32 little-endian, and the metadata."""
        model = "facetrt" if kind == "radiation" else "faceteb"
        stem = model + ("_pv_T=" if kind == "photovoltaic" else "_T=") + token
        folder = os.path.join(output_dir, "process")
        os.makedirs(folder, exist_ok=True)
        if run_index is not None:
            run_index.value["products"] += [f"process/{stem}.bin", f"process/{stem}.json"]
        cols = {"radiation": ("shortwave_radiosity", "longwave_radiosity", "net_radiation"),
                "photovoltaic": ("photovoltaic_power", "temperature", "absorbed_shortwave"),
                "energy": ("latent_heat", "sensible_heat", "storage_heat", "temperature",
                           "net_radiation")}[kind]
        rec = np.stack([np.asarray(fields[c], np.float32) for c in cols], 1)
        rec.astype("<f4").tofile(os.path.join(folder, stem + ".bin"))
        g9 = lambda x: format(float(x), ".9g")
        labels = {
            "photovoltaic": '[{"id":"photovoltaicPower","label":"光伏功率 [W m⁻²]","offset":0},'
                            '{"id":"temperature","label":"温度 [K]","offset":1},'
                            '{"id":"absorbedShortwave","label":"单面吸收短波 [W m⁻²]","offset":2}]',
            "radiation": '[{"id":"shortwaveRadiation","label":"短波辐射 [W m⁻²]","offset":0},'
                         '{"id":"longwaveRadiation","label":"长波辐射 [W m⁻²]","offset":1},'
                         '{"id":"netRadiation","label":"净辐射 [W m⁻²]","offset":2}]',
            "energy": '[{"id":"latentHeat","label":"潜热 [W m⁻²]","offset":0},'
                      '{"id":"sensibleHeat","label":"显热 [W m⁻²]","offset":1},'
                      '{"id":"surfaceHeatFlux","label":"表面热通量 [W m⁻²]","offset":2},'
                      '{"id":"temperature","label":"温度 [K]","offset":3},'
                      '{"id":"netRadiation","label":"净辐射 [W m⁻²]","offset":4}]'}[kind]
        f32 = np.float32
        text = (
            "{\n" + f'  "kind": "facet-{kind}-process",\n' + f'  "model": "{model}",\n'
            + f'  "processType": "{kind}",\n' + '  "geometry": "facet",\n'
            + f'  "node": {node},\n' + f'  "julianTime": {g9(f32(row["julian_time"]))},\n'
            + f'  "time": "{token}",\n' + f'  "solarZenith": {g9(f32(zenith))},\n'
            + f'  "solarAzimuth": {g9(f32(azimuth))},\n' + f'  "facetCount": {facet_count},\n'
            + f'  "surfaceCount": {2 * facet_count},\n'
            + '  "geometryFile": "../faceteb.json",\n'
            + '  "componentFile": "../.facet_steps/components.bin",\n'
            + f'  "dataFile": "{stem}.bin",\n' + '  "dataType": "float32-little-endian",\n'
            + '  "layout": "surface-interleaved",\n' + f'  "recordFloats": {len(cols)},\n'
            + f'  "couplingIterations": {int(res["coupling_iterations"])},\n'
            + f'  "temperatureDelta": {g9(f32(res["max_temperature_delta"]))}'
            + f',\n  "converged": {"true" if res["converged"] else "false"}'
            + f',\n  "energyResidual": {g9(f32(res["max_energy_residual"]))}'
            + ',\n  "energyResidualUnits": "W m-2"'
            + f',\n  "energyResidualTemperatureEquivalent": '
              f'{g9(f32(res["max_energy_residual_equivalent"]))}'
            + f',\n  "temperatureTolerance": {g9(f32(self.params.temperature_tolerance))}'
            + f',\n  "iterationBudget": {self.params.coupling_iterations},\n  "fields": '
            + labels + "\n}\n")
        with open(os.path.join(folder, stem + ".json"), "w", encoding="utf-8") as f:
            f.write(text)

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


# ---- the process entry: runFacetEBCore on an XML project or an OBJ ---------
_ENTITIES = {"&lt;": "<", "&gt;": ">", "&quot;": '"', "&apos;": "'", "&amp;": "&"}
_FLOAT = re.compile(r"[+-]?(?:\d+\.?\d*(?:[eE][+-]?\d+)?|\.\d+(?:[eE][+-]?\d+)?|inf(?:inity)?|nan)",
                    re.IGNORECASE)


def first_xml_tag(xml, tag):
    """firstXmlTag (facetrtcore.cpp:2068-2085): the text of the first
    <tag ...>...</tag>, entities decoded; '' when absent."""
    begin = xml.find("<" + tag)
    if begin < 0:
        return ""
    content = xml.find(">", begin + len(tag) + 1)
    if content < 0:
        return ""
    end = xml.find("</" + tag + ">", content + 1)
    if end < 0:
        return ""
    return re.sub("&(lt|gt|quot|apos|amp);", lambda m: _ENTITIES[m.group(0)], xml[content + 1:end])


def xml_float(xml, tag, fallback):
    """xmlFloat (:2098-2110): std::stof of the trimmed text (its longest
    number prefix), the fallback when empty, unparsable or not finite."""
    text = first_xml_tag(xml, tag).strip()
    m = _FLOAT.match(text)
    if not m:
        return float(fallback)
    v = float(np.float32(float(m.group(0))))
    return v if math.isfinite(v) else float(fallback)


def _scalar_spectrum(path):
    """readScalarSpectrum (:2499-2509): numbers until the first that does not
    parse, negatives and non-finite values as 0, at most 2001."""
    values = []
    try:
        text = open(path).read()
    except OSError:
        return np.zeros(0, np.float32)
    for token in text.split():
        m = _FLOAT.fullmatch(token)
        if not m:
            break
        v = float(np.float32(float(token)))
        values.append(max(0.0, v) if math.isfinite(v) else 0.0)
        if len(values) == 2001:
            break
    return np.asarray(values, np.float32)


def _resolve(input_path, value):
    p = value.strip()
    return p if os.path.isabs(p) else os.path.normpath(os.path.join(os.path.dirname(input_path), p))


def _surface(d):
    keys = ("surface_resistance", "specific_heat", "density", "thermal_conductivity",
            "soil_moisture", "heat_capacity_per_area", "soil_temperature_method", "pv_eta25",
            "pv_gamma", "pv_bifaciality", "convective_scale")
    m = facetcu.EnergySurface(d["reflectance"], d["transmittance"], d["tir_reflectance"],
                              d["tir_transmittance"], d["sunlit_temperature"],
                              d["shaded_temperature"], d["energy_reflectance"],
                              d["energy_transmittance"], photovoltaic=bool(d["photovoltaic"]),
                              vegetation=bool(d["vegetation"]), **{k: d[k] for k in keys})
    m.output_component = int(d["output_component"])
    return m


def run_faceteb_core(input_path, output_file="", progress=print):
    """runFacetEBCore (facetrtcore.cpp:3164-4154) on an XML project (or a
    project.json through its XML view) or an OBJ scene: the scene and
    materials (loadProjectScene / loadTreeWithSoil), the settings of
    :3194-3240 (startTimeNode, endTimeNode, dTime, couplingIterations,
    temperatureTolerance, temperatureRelaxation, spectralAccelerationWidth,
    vegetationTemperatureMethod, Latitude, Longitude, skyTemperature,
    directScatteringRatio), the shortwave spectrum (loadShortwaveSpectrum,
    :2499-2541), the meteorology rows (:3243-3273), one shared visibility
    graph of the 40 hemisphere directions (:3329-3371), then the node
    sequence of Run with each node's sun from its date.  Writes
    .facet_steps/components.bin, .facet_steps/energy_T=<time>.bin per node
    and faceteb.json, the photovoltaic node and summary tables, the run
    index faceteb_run.json and the process/ records (radiation and energy
    when the project asks, photovoltaic when it has PV); prints PROGRESS
    lines and RESULT\t<path>.  Not written: images.  Returns the result
    file."""
    ext = os.path.splitext(input_path)[1].lower()
    is_obj = ext == ".obj"
    if ext == ".json":
        xml = facetcu.project_xml_view(input_path)
    else:
        with open(input_path, encoding="utf-8", errors="replace") as f:
            xml = f.read()
    if output_file:
        result_file = output_file
    else:
        out_dir = first_xml_tag(xml, "outDir") or os.path.dirname(input_path)
        result_file = os.path.normpath(os.path.join(out_dir, "faceteb.json"))
    out_dir = os.path.dirname(result_file) or "."
    os.makedirs(out_dir, exist_ok=True)

    start = max(0, int(round(xml_float(xml, "startTimeNode", 0.0))))
    end = max(start + 1, int(round(xml_float(xml, "endTimeNode", float(start + 1)))))
    dtime = max(1.0, xml_float(xml, "dTime", 1800.0))
    settings = dict(
        coupling_iterations=int(np.clip(round(xml_float(xml, "couplingIterations", 20.0)), 1, 100)),
        temperature_tolerance=float(np.clip(xml_float(xml, "temperatureTolerance", 0.05),
                                            0.001, 10.0)),
        temperature_relaxation=float(np.clip(xml_float(xml, "temperatureRelaxation", 0.5),
                                             0.05, 1.0)),
        vegetation_temperature_method=int(np.clip(
            round(xml_float(xml, "vegetationTemperatureMethod", 0.0)), 0, 1)),
        sky_temperature=float(np.clip(xml_float(xml, "skyTemperature", 250.0), 150.0, 350.0)),
        time_step=dtime)
    index = RunIndex(os.path.join(out_dir, "faceteb_run.json"), input_path, start, end,
                     settings["temperature_tolerance"], settings["coupling_iterations"])
    try:
        return _run_faceteb(xml, input_path, result_file, out_dir, start, end, dtime, settings,
                            index, progress)
    finally:
        index.fail()


def _run_faceteb(xml, input_path, result_file, out_dir, start, end, dtime, settings, index,
                 progress):
    """run_faceteb_core after its settings (the run index is open)."""
    is_obj = os.path.splitext(input_path)[1].lower() == ".obj"
    # isRadiationProcess / isEnergyProcess, isProcess meaning energy (:3199-3205)
    save_radiation = first_xml_tag(xml, "isRadiationProcess").strip() == "1"
    save_energy = first_xml_tag(xml, "isEnergyProcess").strip() == "1"
    if not save_radiation and not save_energy and first_xml_tag(xml, "isProcess").strip() == "1":
        save_energy = True
    process = (save_radiation, save_energy)
    width = int(np.clip(round(xml_float(xml, "spectralAccelerationWidth", 100.0)), 1, 1000))
    latitude = xml_float(xml, "Latitude", 40.0)
    longitude = xml_float(xml, "Longitude", 116.0)
    direct_fraction = float(np.clip(xml_float(xml, "directScatteringRatio", 0.8), 0.0, 1.0))
    esun, esky = first_xml_tag(xml, "esunFileName").strip(), first_xml_tag(xml, "eskyFileName").strip()
    spectrum = None
    if esun and esky:
        spectrum = (_scalar_spectrum(_resolve(input_path, esun)),
                    _scalar_spectrum(_resolve(input_path, esky)))

    meteo_name = first_xml_tag(xml, "filePath").strip()
    if meteo_name:
        path = _resolve(input_path, meteo_name)
        if not os.path.exists(path):
            raise RuntimeError("FacetEB cannot open meteorology: " + meteo_name)
        meteorology = read_meteorology(path)
    else:
        meteorology = []
    if not meteorology:
        meteorology = default_meteorology(end, dtime)
    if end > len(meteorology):
        raise RuntimeError("FacetEB time range exceeds meteorology rows")

    if is_obj:
        vertices, mi, leaf, _, _ = facetcu.load_tree_with_soil(input_path)
        raster, layers, periodic = 1024, 64, (0, 1.0, 1.0)
        materials, mi, tex, strength, wavelengths = [], None, None, 0.0, [550.0]
    else:
        project = facetcu.Project(input_path)
        info = project.info
        vertices, leaf = project.vertices, info["leaf_facet_count"]
        raster, layers = info["raster_size"], info["raster_layers"]
        periodic = (info["periodic_neighbor_count"], info["periodic_size_x"],
                    info["periodic_size_z"])
        materials = [_surface(project.material(i)) for i in range(info["material_count"])]
        mi, tex = project.material_indices, project.texture_factors
        strength = info["background_angular_strength"]
        sp = project.spectral_parameters()
        wl = facetcu.C.cast(sp.wavelengths, facetcu.C.POINTER(facetcu.C.c_float))
        wavelengths = [float(wl[i]) for i in range(sp.band_count)]
        project.close()
    if progress:
        progress("PROGRESS\t3\tFacetEB scene and meteorology loaded")
    model = facetcu.FacetrtCuda()
    model.initialize(raster, raster, layers, 0, *periodic)
    model.setGeometry(vertices)
    if progress:
        progress("PROGRESS\t10\tshared facet visibility graph")
    diag = model.buildVisibilityGraph(facetcu.hemisphere_directions())
    try:
        run = Run(model, leaf, materials, mi, tex, wavelengths=wavelengths, spectrum=spectrum,
                  direct_fraction=direct_fraction, window_width=width,
                  background_angular_strength=strength, **settings)
        results, _ = run.run(meteorology, None, start, end, output_dir=out_dir,
                             vertices=vertices, graph=diag, progress=progress,
                             latitude=latitude, longitude=longitude, run_index=index,
                             process=process)
        written = os.path.join(out_dir, "faceteb.json")
        if os.path.abspath(written) != os.path.abspath(result_file):
            os.replace(written, result_file)
        index.finish(os.path.basename(result_file), all(r["converged"] for r in results))
    finally:
        model.close()
    if progress:
        progress("RESULT\t" + result_file)
    return result_file


def main(argv=None):
    """`python -m streamsim_gb300.faceteb <Input.xml|project.json|scene.obj>
    [faceteb.json]`: the eFacetEB process mode (runFacetEBCore); exit 0, or
    1 with `faceteb: <message>` on stderr."""
    argv = sys.argv[1:] if argv is None else argv
    if not argv:
        print("Usage: python -m streamsim_gb300.faceteb <project> [faceteb.json]", file=sys.stderr)
        return 2
    try:
        run_faceteb_core(argv[0], argv[1] if len(argv) > 1 else "")
        return 0
    except Exception as e:  # the reference prints and returns 1
        print(f"faceteb: {e}", file=sys.stderr)
        return 1


if __name__ == "__main__":
    sys.exit(main())
