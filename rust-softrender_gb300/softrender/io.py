"""Host-side mesh and image I/O for the examples' workflow (examples/suzanne.rs:
24-47 loads an OBJ with tobj and writes the framebuffer as an image).

    load_obj(path or text) -> (positions (n,3), normals (n,3) or None,
                               uvs (n,2) or None, indices (3k,) uint32)
    save_png(path, rgba8)  -- (h, w) uint32 (r in the low byte) or (h, w, 4) uint8
    load_png(path)         -> (h, w) uint32 RGBA8 (8-bit RGB / RGBA, non-interlaced)

Pure Python + numpy + zlib; no image library is needed."""
import struct
import zlib

import numpy as np


# -------------------------------------------------------------------- OBJ
def load_obj(source):
    """Wavefront OBJ: v / vt / vn / f (polygons fan-triangulated from their
    first vertex, as tobj's triangulate option does).  Each distinct
    (v, vt, vn) corner becomes one output vertex.  `source` is a path or the
    file's text (when it contains a newline)."""
    text = source if "\n" in source else open(source).read()
    vs, vts, vns = [], [], []
    corners = {}
    pos, uv, nrm, idx = [], [], [], []
    has_uv = has_n = False

    def corner(tok):
        nonlocal has_uv, has_n
        parts = tok.split("/")
        vi = int(parts[0])
        ti = int(parts[1]) if len(parts) > 1 and parts[1] else 0
        ni = int(parts[2]) if len(parts) > 2 and parts[2] else 0
        vi = vi - 1 if vi > 0 else len(vs) + vi
        ti = (ti - 1 if ti > 0 else len(vts) + ti) if ti else -1
        ni = (ni - 1 if ni > 0 else len(vns) + ni) if ni else -1
        key = (vi, ti, ni)
        if key not in corners:
            corners[key] = len(pos)
            pos.append(vs[vi])
            uv.append(vts[ti] if ti >= 0 else (0.0, 0.0))
            nrm.append(vns[ni] if ni >= 0 else (0.0, 0.0, 0.0))
            has_uv = has_uv or ti >= 0
            has_n = has_n or ni >= 0
        return corners[key]

    for line in text.splitlines():
        t = line.split()
        if not t or t[0].startswith("#"):
            continue
        if t[0] == "v":
            vs.append(tuple(float(x) for x in t[1:4]))
        elif t[0] == "vt":
            vts.append(tuple(float(x) for x in t[1:3]))
        elif t[0] == "vn":
            vns.append(tuple(float(x) for x in t[1:4]))
        elif t[0] == "f":
            c = [corner(tok) for tok in t[1:]]
            for i in range(1, len(c) - 1):
                idx += [c[0], c[i], c[i + 1]]
    return (np.asarray(pos, np.float32).reshape(-1, 3),
            np.asarray(nrm, np.float32).reshape(-1, 3) if has_n else None,
            np.asarray(uv, np.float32).reshape(-1, 2) if has_uv else None,
            np.asarray(idx, np.uint32))


# -------------------------------------------------------------------- PNG
def _chunk(kind, data):
    return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xffffffff)


def _as_rgba(img):
    a = np.asarray(img)
    if a.dtype == np.uint32 and a.ndim == 2:
        a = a.view(np.uint8).reshape(a.shape[0], a.shape[1], 4)
    if a.dtype != np.uint8 or a.ndim != 3 or a.shape[2] != 4:
        raise ValueError("expected (h, w) uint32 RGBA8 or (h, w, 4) uint8")
    return np.ascontiguousarray(a)


def save_png(path, rgba8):
    """Writes an 8-bit RGBA PNG (filter type 0 on every row)."""
    a = _as_rgba(rgba8)
    h, w = a.shape[:2]
    raw = b"".join(b"\x00" + a[y].tobytes() for y in range(h))
    png = (b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)) +
           _chunk(b"IDAT", zlib.compress(raw, 6)) + _chunk(b"IEND", b""))
    with open(path, "wb") as f:
        f.write(png)


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def load_png(path):
    """Reads an 8-bit RGB or RGBA, non-interlaced PNG into (h, w) uint32 RGBA8
    (alpha 255 for RGB)."""
    data = open(path, "rb").read()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG file")
    pos, idat, hdr = 8, b"", None
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        kind = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        if kind == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"IDAT":
            idat += body
        elif kind == b"IEND":
            break
        pos += 12 + n
    w, h, depth, ctype, _, _, interlace = hdr
    if depth != 8 or ctype not in (2, 6) or interlace:
        raise ValueError("only 8-bit RGB / RGBA non-interlaced PNGs are supported")
    bpp = 4 if ctype == 6 else 3
    raw = zlib.decompress(idat)
    stride = w * bpp
    out = np.zeros((h, stride), np.uint8)
    prev = bytearray(stride)
    p = 0
    for y in range(h):
        f = raw[p]
        row = bytearray(raw[p + 1:p + 1 + stride])
        p += 1 + stride
        for i in range(stride):
            a = row[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            if f == 1:
                row[i] = (row[i] + a) & 255
            elif f == 2:
                row[i] = (row[i] + b) & 255
            elif f == 3:
                row[i] = (row[i] + ((a + b) >> 1)) & 255
            elif f == 4:
                row[i] = (row[i] + _paeth(a, b, c)) & 255
        out[y] = np.frombuffer(bytes(row), np.uint8)
        prev = row
    px = out.reshape(h, w, bpp)
    if bpp == 3:
        px = np.concatenate([px, np.full((h, w, 1), 255, np.uint8)], axis=2)
    return np.ascontiguousarray(px).view(np.uint32).reshape(h, w)
