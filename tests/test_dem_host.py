"""DEM height fields of XML projects (no GPU).

The reference reads the project's <DEM> with GDAL (readDemHeightField,
models/histream/src/facetrt/facetrtcore.cpp:2652-2697) and raises the ground
grid and every placement by its bilinear height above the minimum
(:2618-2650, :2836-2878, :2989-2993).  Here:
  - the library's reader on the DEM files shipped with the reference
    (assets/dem-library, validation/*.tif: little- and big-endian float32
    GeoTIFF, NaN and -9999 nodata, ASCII grids), against a plain numpy decode;
  - every GeoTIFF layout the reader accepts, written by tests/tiff_writer.py;
  - the reference's own loader (oracle/_ref, its GDAL stand-in opening ASCII
    grids) against the library's, bit for bit, on projects with a DEM, and
    the same project from a GeoTIFF of the same heights;
  - the reference's error messages."""
import os

import numpy as np
import pytest

from streamsim_gb300 import facetcu
from tests import tiff_writer
from tests.test_project_host import _compare, _write_project, ref_project  # noqa: F401

from oracle.build_ref import REFERENCE  # the reference tree the oracle recipe reads


def _reference_file(*parts):
    path = os.path.join(REFERENCE, *parts)
    if not os.path.exists(path):
        pytest.skip("reference DEM files not present")
    return path


def _strip_tiff(path):
    """numpy decode of an uncompressed single-strip float32 GeoTIFF."""
    b = open(path, "rb").read()
    e = "<" if b[:2] == b"II" else ">"
    ifd = int(np.frombuffer(b[4:8], e + "u4")[0])
    n = int(np.frombuffer(b[ifd:ifd + 2], e + "u2")[0])
    tags = {}
    for i in range(n):
        at = ifd + 2 + 12 * i
        tag, typ = np.frombuffer(b[at:at + 4], e + "u2")
        cnt = int(np.frombuffer(b[at + 4:at + 8], e + "u4")[0])
        val = b[at + 8:at + 12]
        if typ == 2:
            off = int(np.frombuffer(val, e + "u4")[0]) if cnt > 4 else None
            tags[int(tag)] = (b[off:off + cnt] if off is not None else val[:cnt]).rstrip(b"\0")
        else:
            tags[int(tag)] = int(np.frombuffer(val[:2] if typ == 3 else val,
                                               e + ("u2" if typ == 3 else "u4"))[0])
    W, H = tags[256], tags[257]
    assert tags[259] == 1 and tags[258] == 32 and tags[339] == 3 and tags[278] >= H
    raw = np.frombuffer(b[tags[273]:tags[273] + 4 * W * H], e + "f4").reshape(H, W)
    nodata = float(tags[42113]) if 42113 in tags else None
    return raw.astype(np.float32), nodata


def _as_loaded(raw, nodata):
    """readDemHeightField's replacement of nodata and non-finite cells."""
    bad = ~np.isfinite(raw)
    if nodata is not None:
        bad |= raw == np.float32(nodata)
    lo = raw[~bad].min()
    out = raw.copy()
    out[bad] = lo
    return out, float(lo)


@pytest.mark.parametrize("parts", [
    ("assets", "dem-library", "slope", "single_slope_60x60m.tif"),
    ("assets", "dem-library", "slope", "compound_slope_60x60m.tif"),
    ("validation", "dem_test_input.tif"),
])
def test_reference_geotiffs(parts):
    path = _reference_file(*parts)
    raw, nodata = _strip_tiff(path)
    want, lo = _as_loaded(raw, nodata)
    got, minimum = facetcu.dem_height_field(path)
    assert np.array_equal(got, want) and minimum == lo


@pytest.mark.parametrize("name", ["flat/flat_65x65.asc", "hill/central_hill_65x65.asc",
                                  "basin/basin_65x65.asc", "rolling/rolling_hills_65x65.asc"])
def test_reference_ascii_grids(name):
    path = _reference_file("assets", "dem-library", *name.split("/"))
    with open(path) as f:
        header = [f.readline().split() for _ in range(6)]
    assert header[0][0].lower() == "ncols"
    nodata = float(header[5][1])
    raw = np.array(open(path).read().split()[12:], np.float64).astype(np.float32)
    raw = raw.reshape(int(header[1][1]), int(header[0][1]))
    want, lo = _as_loaded(raw, nodata)
    got, minimum = facetcu.dem_height_field(path)
    assert np.array_equal(got, want) and minimum == lo


def _terrain(h=37, w=29, seed=0):
    y, x = np.mgrid[0:h, 0:w] / np.array([h - 1, w - 1])[:, None, None]
    z = 120.0 + 9.0 * np.exp(-((x - 0.4) ** 2 + (y - 0.6) ** 2) / 0.05) + 3.0 * np.sin(7 * x)
    z += np.random.default_rng(seed).normal(0, 0.05, z.shape)
    return z


LAYOUTS = {
    "strips_le_f32": dict(dtype="f4", rows_per_strip=5),
    "strips_be_f32_deflate_p3": dict(dtype="f4", order=">", compression=8, predictor=3,
                                     rows_per_strip=8),
    "tiles_le_f32_lzw_p3": dict(dtype="f4", tile=(16, 16), compression=5, predictor=3),
    "tiles_be_f64_lzw_p3": dict(dtype="f8", order=">", tile=(16, 32), compression=5, predictor=3),
    "strips_le_i16_lzw_p2": dict(dtype="i2", scale=100, compression=5, predictor=2,
                                 rows_per_strip=7),
    "strips_be_u16_packbits": dict(dtype="u2", scale=100, order=">", compression=32773),
    "tiles_le_i32_deflate_p2": dict(dtype="i4", scale=1000, tile=(32, 16), compression=32946,
                                    predictor=2),
    "strips_le_u8_p2": dict(dtype="u1", offset=-110, scale=10, predictor=2, rows_per_strip=3),
    "strips_le_f16": dict(dtype="f2", offset=-100),
    "bigtiff_be_f32_tiles_deflate": dict(dtype="f4", order=">", tile=(16, 16), compression=8,
                                         bigtiff=True),
    "planar_le_f32_2bands": dict(dtype="f4", bands=2, planar=2, compression=5, predictor=3,
                                 rows_per_strip=6),
    "chunky_be_i16_3bands_p2": dict(dtype="i2", scale=10, bands=3, order=">", predictor=2,
                                    compression=8),
    "strips_le_i64": dict(dtype="i8", scale=1e6),
    "strips_le_u32_lzw": dict(dtype="u4", scale=1e4, compression=5),
}


@pytest.mark.parametrize("layout", sorted(LAYOUTS))
def test_geotiff_layouts(tmp_path, layout):
    kw = dict(LAYOUTS[layout])
    dtype = np.dtype(kw.pop("dtype"))
    scale, offset, bands = kw.pop("scale", 1.0), kw.pop("offset", 0.0), kw.pop("bands", 1)
    z = (_terrain() + offset) * scale
    img = z.astype(dtype) if dtype.kind == "f" else np.round(z).astype(dtype)
    if bands > 1:  # band 1 is the DEM; the others are noise
        noise = np.random.default_rng(1).integers(0, 100, img.shape + (bands - 1,)).astype(dtype)
        img = np.concatenate([img[:, :, None], noise], axis=2)
    path = tiff_writer.write(str(tmp_path / "d.tif"), img, **kw)
    got, lo = facetcu.dem_height_field(path)
    band1 = (img if bands == 1 else img[:, :, 0]).astype(np.float32)
    assert np.array_equal(got, band1) and lo == band1.min()


def test_lzw_clear_code_and_long_strings(tmp_path):
    # 30,000 float32 cells, half of them repeating: the LZW table fills and
    # clears several times, and runs build long strings
    rng = np.random.default_rng(5)
    z = rng.normal(50, 10, (150, 200)).astype(np.float32)
    z[:, 100:] = 7.25
    path = tiff_writer.write(str(tmp_path / "d.tif"), z, compression=5, rows_per_strip=150)
    got, _ = facetcu.dem_height_field(path)
    assert np.array_equal(got, z)


def test_nodata_and_non_finite_cells(tmp_path):
    z = _terrain().astype(np.float32)
    z[0, :5] = -32768.0
    z[10, 10] = np.nan
    z[11, 3] = np.inf
    path = tiff_writer.write(str(tmp_path / "d.tif"), z, nodata="-32768", tile=(16, 16))
    got, lo = facetcu.dem_height_field(path)
    want, wlo = _as_loaded(z, -32768.0)
    assert np.array_equal(got, want) and lo == wlo and got[0, 0] == lo


def _write_asc(path, z, nodata="-9999", keys=("NCOLS", "NROWS", "XLLCORNER", "YLLCORNER",
                                               "CELLSIZE", "NODATA_VALUE")):
    h, w = z.shape
    vals = dict(zip(keys, [w, h, 0, 0, 1, nodata]))
    with open(path, "w") as f:
        for k in keys:
            f.write(f"{k} {vals[k]}\n")
        for row in z:
            f.write(" ".join(f"{v:.9g}" for v in row) + "\n")
    return path


@pytest.mark.parametrize("case,message", [
    ("missing", "Cannot open DEM: "),
    ("not_raster", "Cannot open DEM: "),
    ("one_row", "DEM must contain at least 2 x 2 cells: "),
    ("all_nodata", "DEM contains no valid elevations: "),
    ("short_ascii", "Cannot read DEM elevations: "),
    ("bad_deflate", "Cannot read DEM elevations: "),
    ("jpeg", "Cannot open DEM: "),
])
def test_reader_errors(tmp_path, case, message):
    path = str(tmp_path / "d")
    if case == "not_raster":
        open(path, "w").write("hello world\n")
    elif case == "one_row":
        _write_asc(path, np.ones((1, 9)))
    elif case == "all_nodata":
        _write_asc(path, np.full((3, 3), -9999.0))
    elif case == "short_ascii":
        _write_asc(path, np.ones((4, 4)))
        open(path, "a").write("1 2 3\n")
        text = open(path).read().split("\n")
        open(path, "w").write("\n".join(text[:7]) + "\n")
    elif case == "bad_deflate":
        tiff_writer.write(path, np.ones((8, 8), np.float32), compression=8)
        b = bytearray(open(path, "rb").read())
        b[10:14] = b"\xff\xff\xff\xff"  # inside the first (only) strip
        open(path, "wb").write(bytes(b))
    elif case == "jpeg":
        tiff_writer.write(path, np.ones((8, 8), np.float32))
        b = bytearray(open(path, "rb").read())
        ifd = int.from_bytes(b[4:8], "little")
        for i in range(int.from_bytes(b[ifd:ifd + 2], "little")):
            at = ifd + 2 + 12 * i
            if int.from_bytes(b[at:at + 2], "little") == 259:
                b[at + 8:at + 10] = (7).to_bytes(2, "little")  # JPEG
        open(path, "wb").write(bytes(b))
    with pytest.raises(RuntimeError) as e:
        facetcu.dem_height_field(path)
    assert str(e.value) == message + path


def test_ascii_grid_header_forms(tmp_path):
    z = _terrain(9, 7).astype(np.float32)  # 9 digits round-trip a float32
    a, _ = facetcu.dem_height_field(_write_asc(str(tmp_path / "a.asc"), z))
    b, _ = facetcu.dem_height_field(_write_asc(
        str(tmp_path / "b.asc"), z, keys=("ncols", "nrows", "xllcenter", "yllcenter", "dx", "dy")))
    assert np.array_equal(a, z) and np.array_equal(a, b)


# ---- projects with a DEM, against the reference's loader -------------------
def _dem_project(root, dem_file, enabled="1", **kw):
    return _write_project(root, coefficients=False, size=(9.0, 7.0), voxel=0.5,
                          extra_control=f"<isDEM>{enabled}</isDEM>",
                          extra_scene=f"<DEM>{dem_file}</DEM>", **kw)


def test_project_on_a_dem_matches_reference(tmp_path, ref_project):  # noqa: F811
    os.makedirs(tmp_path / "terrain")
    z = _terrain().astype(np.float32)  # exact in 9 digits, so .asc == .tif
    z[3, 4] = -9999.0  # nodata -> the minimum
    _write_asc(str(tmp_path / "terrain" / "t.asc"), z)
    path = _dem_project(tmp_path, "terrain/t.asc")
    theirs = ref_project.load(path)
    ours = facetcu.Project(path)
    _compare(ours, theirs)
    v = ours.vertices
    ground = v[3 * ours.info["leaf_facet_count"]:]
    assert ground[:, 1].max() > 5.0 and ground[:, 1].min() >= np.float32(-0.01)
    # the objects stand on the terrain (and are clipped at the domain's
    # height), higher than with the DEM switched off
    flat = facetcu.Project(_dem_project(tmp_path, "terrain/t.asc", enabled="0"))
    leaf, flat_leaf = 3 * ours.info["leaf_facet_count"], 3 * flat.info["leaf_facet_count"]
    assert v[:leaf, 1].mean() > flat.vertices[:flat_leaf, 1].mean() + 1.0
    assert flat.vertices[flat_leaf:, 1].max() == np.float32(-0.01)

    # the same heights as a tiled, predicted LZW GeoTIFF load the same scene
    tiff_writer.write(str(tmp_path / "terrain" / "t.tif"), z, tile=(16, 16), compression=5,
                      predictor=3, nodata="-9999")
    tif = facetcu.Project(_dem_project(tmp_path, "terrain/t.tif"))
    assert np.array_equal(tif.vertices.view(np.uint32), ours.vertices.view(np.uint32))


def test_reference_dem_library_project(tmp_path, ref_project):  # noqa: F811
    src = _reference_file("assets", "dem-library", "rolling", "rolling_hills_65x65.asc")
    path = _dem_project(tmp_path, src)
    _compare(facetcu.Project(path), ref_project.load(path))


def test_project_dem_errors_match_reference(tmp_path, ref_project):  # noqa: F811
    os.makedirs(tmp_path / "terrain")
    _write_asc(str(tmp_path / "terrain" / "n.asc"), np.full((4, 4), -9999.0))
    for name in ("terrain/n.asc", "terrain/missing.asc"):
        path = _dem_project(tmp_path, name)
        with pytest.raises(RuntimeError) as theirs:
            ref_project.load(path)
        with pytest.raises(RuntimeError) as ours:
            facetcu.Project(path)
        assert str(ours.value) == str(theirs.value)


# ---- physical reflectance textures (loadReflectanceVarianceTexture,
# sampledReflectanceVariance, finalizeReflectanceTextureFactors:
# facetrtcore.cpp:623-846), against the reference's own loader ------------
def _texture_project(root, texture_file, strength="0.5", repeat="1.5", objects=None):
    spectral = ("<spectral name=\"tex\" type=\"custom\"><reflectance>0.3</reflectance>"
                "<transmittance>0.1</transmittance>"
                "<physicalTextureEnabled>true</physicalTextureEnabled>"
                f"<physicalTextureFile>{texture_file}</physicalTextureFile>"
                f"<physicalTextureStrength>{strength}</physicalTextureStrength>"
                f"<physicalTextureRepeatSize>{repeat}</physicalTextureRepeatSize></spectral>")
    objects = objects or """
<object objName="House"><componentType>Building</componentType><meshNames>wall, Roof</meshNames>
<spectralNames>tex;concrete</spectralNames><bioNames>wallset</bioNames>
<fileName>models/house.obj</fileName><objectPosition>positions/house.txt</objectPosition></object>
<object objName="Box"><spectralNames>tex</spectralNames><bioNames>wallset</bioNames>
<shapes>1.5,2,0.5</shapes></object>"""
    return _write_project(root, coefficients=False, objects=objects, extra_spectral=spectral)


def _pattern(h=23, w=31):
    y, x = np.mgrid[0:h, 0:w]
    # whole numbers within a byte (30 .. 230)
    return np.floor(30 + 60 * (np.sin(x / 3.0) + 1) + 20 * ((x + y) % 5)).astype(np.float32)


def test_textured_project_matches_reference(tmp_path, ref_project):  # noqa: F811
    os.makedirs(tmp_path / "tex")
    z = _pattern()
    _write_asc(str(tmp_path / "tex" / "a.asc"), z)
    path = _texture_project(tmp_path, "tex/a.asc")
    theirs = ref_project.load(path)
    ours = facetcu.Project(path)
    _compare(ours, theirs)
    f = ours.texture_factors
    assert theirs["texture_factors"].size and np.any(f != 1.0) and np.all(f > 0.0)
    # the same bytes as an 8-bit GeoTIFF give the same factors
    tiff_writer.write(str(tmp_path / "tex" / "a.tif"), z.astype(np.uint8), rows_per_strip=4,
                      compression=5, predictor=2)
    tif = facetcu.Project(_texture_project(tmp_path, "tex/a.tif"))
    assert np.array_equal(tif.texture_factors.view(np.uint32), f.view(np.uint32))


def test_rgb_texture_loads(tmp_path):
    os.makedirs(tmp_path / "tex")
    z = _pattern()
    rgb = np.stack([z, z[::-1], np.roll(z, 3, axis=1)], axis=2).astype(np.uint8)
    tiff_writer.write(str(tmp_path / "tex" / "rgb.tif"), rgb, tile=(16, 16), compression=8)
    f = facetcu.Project(_texture_project(tmp_path, "tex/rgb.tif")).texture_factors
    assert np.any(f != 1.0) and np.all(np.isfinite(f)) and np.all(f > 0.0)


@pytest.mark.parametrize("case", ["constant", "one_row", "missing"])
def test_texture_errors_match_reference(tmp_path, ref_project, case):  # noqa: F811
    os.makedirs(tmp_path / "tex")
    if case == "constant":
        _write_asc(str(tmp_path / "tex" / "t.asc"), np.full((5, 5), 128.0))
    elif case == "one_row":
        _write_asc(str(tmp_path / "tex" / "t.asc"), np.arange(9.0)[None, :])
    path = _texture_project(tmp_path, "tex/t.asc")
    with pytest.raises(RuntimeError) as theirs:
        ref_project.load(path)
    with pytest.raises(RuntimeError) as ours:
        facetcu.Project(path)
    assert str(ours.value) == str(theirs.value)
    assert "reflectance variance texture" in str(ours.value).lower()


@pytest.mark.parametrize("kind", ["gray8", "gray16", "rgb8", "rgba8", "graya8", "palette"])
def test_png_rasters(tmp_path, kind):
    z = _pattern(19, 27)
    if kind == "gray16":
        img = (z * 200).astype(np.uint16)
    elif kind in ("rgb8", "rgba8", "graya8"):
        c = {"rgb8": 3, "rgba8": 4, "graya8": 2}[kind]
        img = np.stack([np.roll(z, k, axis=1) for k in range(c)], axis=2).astype(np.uint8)
    else:
        img = z.astype(np.uint8)
    path = tiff_writer.write_png(str(tmp_path / "t.png"), img, depth=16 if kind == "gray16" else 8,
                                 palette=kind == "palette")
    got, _ = facetcu.dem_height_field(path)  # band 1
    want = (img if img.ndim == 2 else img[:, :, 0]).astype(np.float32)
    assert np.array_equal(got, want)


def test_png_texture_equals_ascii_texture(tmp_path):
    os.makedirs(tmp_path / "tex")
    z = _pattern()
    _write_asc(str(tmp_path / "tex" / "a.asc"), z)
    tiff_writer.write_png(str(tmp_path / "tex" / "a.png"), z.astype(np.uint8))
    a = facetcu.Project(_texture_project(tmp_path, "tex/a.asc")).texture_factors
    b = facetcu.Project(_texture_project(tmp_path, "tex/a.png")).texture_factors
    assert np.any(a != 1.0) and np.array_equal(a.view(np.uint32), b.view(np.uint32))
