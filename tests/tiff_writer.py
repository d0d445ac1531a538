"""Small GeoTIFF and PNG writers for the raster reader's tests (test
infrastructure).

Writes one image in any of the layouts facetcu_dem_height_field reads:
classic or BigTIFF, little or big endian, strips or tiles, chunky or planar
samples, no compression, LZW (TIFF 6.0 section 13, with the early code-width
change and a clear code when the table fills), deflate (Python's zlib) or
PackBits, horizontal (2) or floating-point (3) prediction, and the
GDAL_NODATA tag; and non-interlaced PNG with every row filter.  Independent
of the library's decoders."""
import struct
import zlib

import numpy as np

_FORMAT = {"u": 1, "i": 2, "f": 3}


def lzw_encode(data):
    bits = []

    def put(code, width):
        bits.extend((code >> (width - 1 - k)) & 1 for k in range(width))

    def fresh():
        return {bytes([i]): i for i in range(256)}

    table, nxt, width = fresh(), 258, 9
    put(256, width)
    s = b""
    for c in data:
        sc = s + bytes([c])
        if sc in table:
            s = sc
            continue
        put(table[s], width)
        table[sc] = nxt
        nxt += 1
        if nxt == 4094:
            put(256, width)
            table, nxt, width = fresh(), 258, 9
        elif nxt > (1 << width) - 1:
            width += 1
        s = bytes([c])
    if s:
        put(table[s], width)
        nxt += 1
        if nxt == 4094:
            put(256, width)
            width = 9
        elif nxt > (1 << width) - 1:
            width += 1
    put(257, width)
    bits.extend([0] * (-len(bits) % 8))
    return np.packbits(np.array(bits, np.uint8)).tobytes()


def packbits_encode(data):
    out = bytearray()
    i, n = 0, len(data)
    while i < n:
        j = i
        while j + 1 < n and data[j + 1] == data[i] and j - i < 127:
            j += 1
        if j - i >= 2:  # a run of 3..128 equal bytes
            out += bytes([(256 - (j - i)) & 255, data[i]])
            i = j + 1
            continue
        k = i
        while k < n and k - i < 128 and not (k + 2 < n and data[k] == data[k + 1] == data[k + 2]):
            k += 1
        out += bytes([k - i - 1]) + bytes(data[i:k])
        i = k
    return bytes(out)


def _predict(block, predictor, spp, order):
    """block (rows, cols * spp) of samples -> bytes per row after prediction."""
    rows = []
    for row in block:
        if predictor == 2:
            u = row.view(np.dtype(f"u{row.dtype.itemsize}"))
            d = u.copy()
            d[spp:] = u[spp:] - u[:-spp]
            rows.append(d.astype(d.dtype.newbyteorder(order)).tobytes())
        elif predictor == 3:
            n, sb = row.size, row.dtype.itemsize
            be = row.astype(row.dtype.newbyteorder(">")).tobytes()
            planes = np.frombuffer(be, np.uint8).reshape(n, sb).T.reshape(-1).copy()
            d = planes.copy()
            d[spp:] = planes[spp:] - planes[:-spp]
            rows.append(d.tobytes())
        else:
            rows.append(row.astype(row.dtype.newbyteorder(order)).tobytes())
    return b"".join(rows)


def write(path, image, *, order="<", tile=None, rows_per_strip=None, compression=1, predictor=1,
          planar=1, bigtiff=False, nodata=None):
    """image: (H, W) or (H, W, spp) numpy array of the sample type."""
    img = image if image.ndim == 3 else image[:, :, None]
    H, W, spp = img.shape
    kind = img.dtype.kind
    bps = img.dtype.itemsize * 8
    planes = [img] if planar == 1 else [img[:, :, k:k + 1] for k in range(spp)]
    cw, ch = tile if tile else (W, rows_per_strip or H)
    blocks = []
    for plane in planes:
        bspp = plane.shape[2]
        for by in range(0, H, ch):
            for bx in range(0, W, cw):
                if tile:
                    blk = np.zeros((ch, cw, bspp), img.dtype)
                    part = plane[by:by + ch, bx:bx + cw]
                    blk[:part.shape[0], :part.shape[1]] = part
                else:
                    blk = plane[by:by + ch]
                raw = _predict(blk.reshape(blk.shape[0], -1), predictor, bspp, order)
                if compression == 5:
                    raw = lzw_encode(raw)
                elif compression in (8, 32946):
                    raw = zlib.compress(raw)
                elif compression == 32773:
                    raw = packbits_encode(raw)
                blocks.append(raw)
    # layout: header, block data, tag data, IFD
    head = 16 if bigtiff else 8
    data = bytearray()
    offsets = []
    for b in blocks:
        offsets.append(head + len(data))
        data += b
        data += b"\0" * (len(data) % 2)
    long_t = 16 if bigtiff else 4
    tags = [(256, 4, [W]), (257, 4, [H]), (258, 3, [bps] * spp), (259, 3, [compression]),
            (262, 3, [1]), (277, 3, [spp]), (284, 3, [planar]), (339, 3, [_FORMAT[kind]] * spp)]
    if predictor != 1:
        tags.append((317, 3, [predictor]))
    if tile:
        tags += [(322, 3, [cw]), (323, 3, [ch]), (324, long_t, offsets),
                 (325, long_t, [len(b) for b in blocks])]
    else:
        tags += [(273, long_t, offsets), (278, 4, [ch]), (279, long_t, [len(b) for b in blocks])]
    if nodata is not None:
        tags.append((42113, 2, nodata.encode() + b"\0"))
    tags.sort()
    fmt = {3: "H", 4: "I", 16: "Q"}
    size = {2: 1, 3: 2, 4: 4, 16: 8}
    inline = 8 if bigtiff else 4
    extra = bytearray()
    base = head + len(data)
    entries = []
    for tag, typ, vals in tags:
        payload = vals if typ == 2 else struct.pack(order + fmt[typ] * len(vals), *vals)
        count = len(vals)
        if len(payload) <= inline:
            field = payload + b"\0" * (inline - len(payload))
        else:
            field = struct.pack(order + ("Q" if bigtiff else "I"), base + len(extra))
            extra += payload + b"\0" * (len(payload) % 2)
        entries.append(struct.pack(order + ("HHQ" if bigtiff else "HHI"), tag, typ, count) + field)
    ifd = base + len(extra)
    if bigtiff:
        header = (b"II" if order == "<" else b"MM") + struct.pack(order + "HHHQ", 43, 8, 0, ifd)
        ifd_bytes = struct.pack(order + "Q", len(entries)) + b"".join(entries) + \
            struct.pack(order + "Q", 0)
    else:
        header = (b"II" if order == "<" else b"MM") + struct.pack(order + "HI", 42, ifd)
        ifd_bytes = struct.pack(order + "H", len(entries)) + b"".join(entries) + \
            struct.pack(order + "I", 0)
    with open(path, "wb") as f:
        f.write(header + bytes(data) + bytes(extra) + ifd_bytes)
    return path


def write_png(path, image, *, depth=8, palette=False):
    """A non-interlaced PNG of (H, W) or (H, W, C) samples (C = 1 gray,
    2 gray + alpha, 3 RGB, 4 RGBA; palette=True: (H, W) indices into a gray
    palette), every row filtered with one of the five filter types in turn."""
    img = image if image.ndim == 3 else image[:, :, None]
    H, W, C = img.shape
    color = 3 if palette else {1: 0, 2: 4, 3: 2, 4: 6}[C]
    bps = depth // 8
    data = img.astype(">u2" if depth == 16 else np.uint8).reshape(H, W * C).view(np.uint8) \
        if depth == 16 else img.astype(np.uint8).reshape(H, W * C)
    data = np.asarray(data, np.uint8).reshape(H, W * C * bps)
    bpp = C * bps
    rows = []
    prev = np.zeros(W * C * bps, np.int32)
    for y in range(H):
        cur = data[y].astype(np.int32)
        ft = y % 5
        left = np.concatenate([np.zeros(bpp, np.int32), cur[:-bpp]])
        ul = np.concatenate([np.zeros(bpp, np.int32), prev[:-bpp]])
        if ft == 0:
            out = cur
        elif ft == 1:
            out = cur - left
        elif ft == 2:
            out = cur - prev
        elif ft == 3:
            out = cur - (left + prev) // 2
        else:
            p = left + prev - ul
            pa, pb, pc = np.abs(p - left), np.abs(p - prev), np.abs(p - ul)
            pred = np.where((pa <= pb) & (pa <= pc), left, np.where(pb <= pc, prev, ul))
            out = cur - pred
        rows.append(bytes([ft]) + (out & 255).astype(np.uint8).tobytes())
        prev = cur

    def chunk(t, d):
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xffffffff)

    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", W, H, depth, color, 0, 0, 0))
    if palette:
        png += chunk(b"PLTE", bytes(np.repeat(np.arange(256, dtype=np.uint8), 3)))
    raw = zlib.compress(b"".join(rows))
    png += chunk(b"IDAT", raw[:len(raw) // 2]) + chunk(b"IDAT", raw[len(raw) // 2:])
    png += chunk(b"IEND", b"")
    with open(path, "wb") as f:
        f.write(png)
    return path
