"""File formats of the map-making path (numpy, host side).

.pksc halo catalogues (pksc.f90:46-66): the reference reads a 2-word header (int32
Nhalo, float32 RTHmax) and 7 float32 per halo (x, y, z, vx, vy, vz, RTH); later Peak
Patch catalogues carry a 3-word header (+ float32 zbox) and 10 float32 per halo
(+ xL, yL, zL).  The layout is chosen explicitly or from the file size.

Profile tables (maptable.f90:94,142,156-162): int32 nchit, nmht, nrt, float32 chimint,
chimaxt, mhmint, mhmaxt, rmint, rmaxt, then float32 table(2, nrt, nmht, nchit) in
Fortran order.  Output maps (pks2map.f90:366-385): _dp.bin (int32 ndpdy, float32 dpdy_max, float32
P(<y)[ndpdy]), _fs.map (int32 npix, npix, float32 fov, fov, float32 map), _hp.fits (FITS
BINTABLE, one column of 1024-float rows, RING order).
"""
import os
import struct

import numpy as np

LAYOUTS = {7: 2, 10: 3}  # floats per record -> header words


def detect_layout(nbytes, nhalo):
    """Floats per record of a .pksc file of nbytes holding nhalo records."""
    if nbytes == 8 + 28 * nhalo:
        return 7
    if nbytes == 12 + 40 * nhalo:
        return 10
    raise ValueError("file size %d matches neither 8+28N nor 12+40N for N=%d" % (nbytes, nhalo))


def read_pksc(path, nfloat=None):
    """Returns (header dict, records (N, nfloat) float32)."""
    nbytes = os.path.getsize(path)
    with open(path, "rb") as f:
        head = f.read(12)
    if len(head) < 8:
        raise ValueError("truncated .pksc header")
    nhalo = struct.unpack("<i", head[:4])[0]
    if nhalo < 0:
        raise ValueError("negative halo count")
    if nfloat is None:
        nfloat = detect_layout(nbytes, nhalo)
    if nfloat not in LAYOUTS:
        raise ValueError("nfloat must be 7 or 10")
    hw = LAYOUTS[nfloat]
    need = 4 * hw + 4 * nfloat * nhalo
    if nbytes < need:
        raise ValueError("truncated .pksc: %d bytes, header says %d records (%d bytes)"
                         % (nbytes, nhalo, need))
    rthmax = struct.unpack("<f", head[4:8])[0]
    zbox = struct.unpack("<f", head[8:12])[0] if hw == 3 else None
    rec = np.fromfile(path, dtype="<f4", count=nfloat * nhalo, offset=4 * hw)
    return {"nhalo": nhalo, "rthmax": rthmax, "zbox": zbox, "nfloat": nfloat}, \
        rec.reshape(nhalo, nfloat)


def write_pksc(path, records, zbox=0.0):
    rec = np.ascontiguousarray(records, dtype="<f4")
    n, nfloat = rec.shape
    rthmax = float(rec[:, 6].max()) if n else 0.0
    with open(path, "wb") as f:
        f.write(struct.pack("<if", n, rthmax))
        if nfloat == 10:
            f.write(struct.pack("<f", zbox))
        f.write(rec.tobytes())


def table_header(image):
    """Header of a table image as a dict."""
    h = struct.unpack("<3i6f", bytes(image[:36]))
    keys = ("nchit", "nmht", "nrt", "chimint", "chimaxt", "mhmint", "mhmaxt", "rmint", "rmaxt")
    return dict(zip(keys, h))


def table_array(image):
    """Table values as a (nchit, nmht, nrt, 2) float32 view (C order of the Fortran
    table(2, nrt, nmht, nchit))."""
    h = table_header(image)
    a = np.frombuffer(bytes(image), dtype="<f4", offset=36,
                      count=2 * h["nrt"] * h["nmht"] * h["nchit"])
    return a.reshape(h["nchit"], h["nmht"], h["nrt"], 2)


def read_table(path):
    with open(path, "rb") as f:
        return f.read()


def write_table(path, image):
    with open(path, "wb") as f:
        f.write(bytes(image))


def read_dpdy(path):
    """<out>_dp.bin -> (dpdy_max, P(<y) float32 array)."""
    with open(path, "rb") as f:
        raw = f.read()
    n, mx = struct.unpack("<if", raw[:8])
    return mx, np.frombuffer(raw, dtype="<f4", count=n, offset=8).copy()


def read_flatsky(path):
    """<out>_fs.map -> (fov in radians, (npix, npix) float32 map, index [k, j], j fastest)."""
    with open(path, "rb") as f:
        raw = f.read()
    n1, n2, fov, _ = struct.unpack("<iiff", raw[:16])
    return fov, np.frombuffer(raw, dtype="<f4", count=n1 * n2, offset=16).reshape(n2, n1).copy()


def read_healpix_fits(path):
    """<out>_hp.fits -> (header cards of the BINTABLE as a dict, RING-ordered float32 map).
    Reads the layout the HEALPix writer produces: an empty primary HDU, then a BINTABLE
    whose single column holds TFORM1 = '<repeat>E' floats per row (big endian)."""
    with open(path, "rb") as f:
        raw = f.read()

    def header(at):
        cards = {}
        pos = at
        while True:
            block = raw[pos:pos + 2880]
            if len(block) < 2880:
                raise ValueError("truncated FITS header")
            pos += 2880
            for k in range(36):
                c = block[80 * k:80 * k + 80].decode("ascii")
                key = c[:8].strip()
                if key == "END":
                    return cards, pos
                if c[8:10] == "= ":
                    v = c[10:].split(" /")[0].strip()
                    cards[key] = v.strip("'").strip() if v.startswith("'") else v

    prim, pos = header(0)
    if prim.get("SIMPLE") != "T":
        raise ValueError("not a FITS file")
    ext, pos = header(pos)
    if ext.get("XTENSION") != "BINTABLE":
        raise ValueError("second HDU is not a BINTABLE")
    rows, width = int(ext["NAXIS2"]), int(ext["NAXIS1"])
    data = np.frombuffer(raw, dtype=">f4", count=rows * width // 4, offset=pos)
    return ext, data.astype(np.float32)
