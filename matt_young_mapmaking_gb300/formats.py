"""File formats of the map-making path (numpy, host side).

.pksc halo catalogues (pksc.f90:46-66): the reference reads a 2-word header (int32
Nhalo, float32 RTHmax) and 7 float32 per halo (x, y, z, vx, vy, vz, RTH); later Peak
Patch catalogues carry a 3-word header (+ float32 zbox) and 10 float32 per halo
(+ xL, yL, zL).  The layout is chosen explicitly or from the file size.

Profile tables (maptable.f90:94,142,156-162): int32 nchit, nmht, nrt, float32 chimint,
chimaxt, mhmint, mhmaxt, rmint, rmaxt, then float32 table(2, nrt, nmht, nchit) in
Fortran order.  Output maps (pks2map.f90:366-381): _dp.bin, _fs.map, _hp.fits.
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
