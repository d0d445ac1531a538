"""Sensor images from solved radiosity: the products the reference's Node
backend writes after a FacetRT or FacetEB run (writeRadiosityTiffForAngle,
server.mjs:1127-1600), with the raster on the device
(facetcu_render_sensor_image).

  band_names         reflectance / spectral radiance / temperature labels
                     (:1140-1153)
  output_tiff_name   SZA=..._SAA=..._VZA=..._VAA=..._f.tif for FacetRT,
                     T=<time>_VZA=..._VAA=..._f.tif for FacetEB (:706-717)
  write_float_tiff   a baseline little-endian TIFF of float32 bands, pixel
                     interleaved, with the band names in ImageDescription
                     (writeFloatTiff :1907-1975, the same tags and layout)
  facetrt_images     the band images of a facetrt.json band radiosity
  faceteb_images     a FacetEB step record's bands or temperature

The reference's atmosphere correction needs a MODTRAN look-up table that is
not part of the reference tree; images are written without it (as the
reference does when atmosphere.enabled is false).
"""
import os
import struct

import numpy as np

from . import facetcu


def is_optical(wavelength):
    nm = wavelength * 1000 if wavelength <= 2.5 else wavelength
    return nm <= 2500


def band_names(wavelengths, temperature_output=False):
    if temperature_output:
        return ["温度 [K]"]
    return [("Reflectance [-] @ " if is_optical(w) else
             "Spectral radiance [W m-2 sr-1 um-1] @ ") + _js_number(w) + " nm"
            for w in wavelengths]


def _js_number(v):
    """A number as JavaScript's String() writes it (integers without a
    fraction)."""
    v = float(v)
    return str(int(v)) if v.is_integer() else repr(v)


def _angle(v):
    v = float(v)
    return f"{v:.2f}" if np.isfinite(v) else "0.00"


def output_tiff_name(mode, sza=0.0, saa=0.0, vza=0.0, vaa=0.0, time_token=None,
                     atmosphere=False):
    suffix = {"eFacetRT": "_f", "eFacetEB": "_f", "eVoxelRT": "_v",
              "eVoxelEB": "_v"}.get(mode, "") + ("_a" if atmosphere else "")
    if mode in ("eFacetEB", "eVoxelEB"):
        return f"T={time_token or 'UNKNOWN'}_VZA={_angle(vza)}_VAA={_angle(vaa)}{suffix}.tif"
    return (f"SZA={_angle(sza)}_SAA={_angle(saa)}_VZA={_angle(vza)}_VAA={_angle(vaa)}"
            f"{suffix}.tif")


def write_float_tiff(path, image, names=None):
    """image: (bands, H, W) float32.  The reference's layout: header and IFD
    (12 entries, 13 with ExtraSamples for more than one band), the
    BitsPerSample / SampleFormat arrays when they do not fit in the entry,
    the NUL-terminated description, padding to 4 bytes, then the pixels with
    the bands interleaved; non-finite values are written as NaN."""
    img = np.asarray(image, np.float32)
    if img.ndim == 2:
        img = img[None]
    bands, height, width = img.shape
    if min(bands, height, width) <= 0:
        raise ValueError("TIFF size or band count invalid")
    entries = 13 if bands > 1 else 12
    ifd = 8
    data = ifd + 2 + entries * 12 + 4
    extra = []

    def allocate(buf, alignment=2):
        nonlocal data
        pad = (alignment - data % alignment) % alignment
        if pad:
            extra.append((data, b"\0" * pad))
            data += pad
        off = data
        extra.append((off, buf))
        data += len(buf)
        return off

    def shorts(items):
        if len(items) <= 2:
            v = 0
            for i, it in enumerate(items):
                v |= (it & 0xFFFF) << (16 * i)
            return v & 0xFFFFFFFF
        return allocate(struct.pack("<%dH" % len(items), *items))

    bits = shorts([32] * bands)
    formats = shorts([3] * bands)
    extras = shorts([0] * (bands - 1)) if bands > 1 else 0
    labels = [str((names or [])[i]) if names and i < len(names) and names[i] else f"Band {i + 1}"
              for i in range(bands)]
    # Node's 'ascii' Buffer encoding keeps the low byte of each UTF-16 unit
    text = "HiStream image bands: {" + ", ".join(labels) + "}\0"
    desc = bytes(ord(ch) & 0xFF for ch in text.encode("utf-16-le").decode("utf-16-le"))
    desc_off = allocate(desc, 1)
    pad = (4 - data % 4) % 4
    if pad:
        extra.append((data, b"\0" * pad))
        data += pad
    image_off = data
    image_bytes = width * height * bands * 4
    if image_off + image_bytes > 0xFFFFFFFF:
        raise ValueError("TIFF exceeds 4 GiB")
    header = bytearray(image_off)
    header[0:2] = b"II"
    struct.pack_into("<HI", header, 2, 42, ifd)
    struct.pack_into("<H", header, ifd, entries)
    pos = ifd + 2
    for tag, typ, count, value in (
            (256, 4, 1, width), (257, 4, 1, height), (258, 3, bands, bits), (259, 3, 1, 1),
            (262, 3, 1, 1), (270, 2, len(desc), desc_off), (273, 4, 1, image_off),
            (277, 3, 1, bands), (278, 4, 1, height), (279, 4, 1, image_bytes),
            (284, 3, 1, 1)) + (((338, 3, bands - 1, extras),) if bands > 1 else ()) + (
            (339, 3, bands, formats),):
        struct.pack_into("<HHII", header, pos, tag, typ, count, value & 0xFFFFFFFF)
        pos += 12
    struct.pack_into("<I", header, pos, 0)
    for off, buf in extra:
        header[off:off + len(buf)] = buf
    pixels = np.ascontiguousarray(np.moveaxis(img, 0, -1)).astype("<f4")
    pixels[~np.isfinite(pixels)] = np.nan
    tmp = path + ".partial"
    with open(tmp, "wb") as f:
        f.write(header)
        f.write(pixels.tobytes())
    os.replace(tmp, path)
    return path


def read_float_tiff(path):
    """(image (bands, H, W), description) of a TIFF written by
    write_float_tiff."""
    raw = open(path, "rb").read()
    ifd = struct.unpack_from("<I", raw, 4)[0]
    n = struct.unpack_from("<H", raw, ifd)[0]
    tags = {}
    for i in range(n):
        tag, typ, count, value = struct.unpack_from("<HHII", raw, ifd + 2 + 12 * i)
        tags[tag] = (typ, count, value)
    width, height, bands = tags[256][2], tags[257][2], tags[277][2]
    off = tags[273][2]
    pix = np.frombuffer(raw, "<f4", width * height * bands, off).reshape(height, width, bands)
    dtyp, dcount, doff = tags[270]
    desc = raw[doff:doff + dcount - 1].decode("latin-1")
    return np.moveaxis(pix, -1, 0).copy(), desc


def facetrt_images(model, sensor_struct, band_radiosity, wavelengths):
    """Band images of a FacetRT result (band_radiosity (bands, 2F))."""
    return model.renderSensorImage(sensor_struct, band_radiosity, wavelengths)


def faceteb_images(model, sensor_struct, step_path, wavelengths, temperature_output=False):
    """Images of one FacetEB step record (energy_T=<time>.bin: 9 fields then
    the bands per side): the sensor bands, or the temperature as one band
    (its sky at the first thermal wavelength, else 10500 nm)."""
    S = 2 * model.facet_count
    rec = np.fromfile(step_path, "<f4")
    if rec.size % S or rec.size // S < 9:
        raise ValueError("FacetEB step record incomplete: " + os.path.basename(step_path))
    rec = rec.reshape(S, -1)
    if temperature_output:
        thermal = [w for w in wavelengths if not is_optical(w)]
        values, wl = rec[:, 0][None], [thermal[0] if thermal else 10500.0]
        sensor_struct.temperature_output = 1
    else:
        if rec.shape[1] < 9 + len(wavelengths):
            raise ValueError("FacetEB step record lacks the sensor bands: " +
                             os.path.basename(step_path))
        values, wl = rec[:, 9:9 + len(wavelengths)].T, list(wavelengths)
    return model.renderSensorImage(sensor_struct, np.ascontiguousarray(values), wl)
