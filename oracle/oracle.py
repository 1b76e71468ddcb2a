"""TEST INFRASTRUCTURE ONLY: ctypes binding of the C oracle (p2m_oracle.c).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this module;
the product never does.  PARITY UNPINNED: the reference has no golden vectors and cannot
be built here (see p2m_oracle.h).
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libp2m_oracle.so")
MAXMAPS = 8


class OrcTable(ctypes.Structure):
    _fields_ = [("nchit", ctypes.c_int32), ("nmht", ctypes.c_int32), ("nrt", ctypes.c_int32),
                ("chimint", ctypes.c_float), ("chimaxt", ctypes.c_float),
                ("mhmint", ctypes.c_float), ("mhmaxt", ctypes.c_float),
                ("rmint", ctypes.c_float), ("rmaxt", ctypes.c_float),
                ("dchit", ctypes.c_float), ("dmht", ctypes.c_float), ("drt", ctypes.c_float),
                ("data", ctypes.c_void_p)]


class OrcParams(ctypes.Structure):
    _fields_ = [("nside", ctypes.c_int32), ("npix_fs", ctypes.c_int32),
                ("fov_deg", ctypes.c_float), ("zmin", ctypes.c_float),
                ("zmax", ctypes.c_float), ("chihview", ctypes.c_float),
                ("model", ctypes.c_int32), ("nmaps", ctypes.c_int32),
                ("profile", ctypes.c_int32 * MAXMAPS), ("table_id", ctypes.c_int32 * MAXMAPS),
                ("fp32_accumulate", ctypes.c_int32), ("nfloat", ctypes.c_int32),
                ("scramble", ctypes.c_int32), ("centre", ctypes.c_int32),
                ("ntasks", ctypes.c_int32)]


class OrcStats(ctypes.Structure):
    _fields_ = [("n_in", ctypes.c_int64), ("n_cut", ctypes.c_int64),
                ("n_painted", ctypes.c_int64), ("hp_updates", ctypes.c_int64),
                ("fs_updates", ctypes.c_int64), ("hp_candidates", ctypes.c_int64),
                ("ring_gaps", ctypes.c_int64), ("centre", ctypes.c_float * 9)]


class OrcCosmo(ctypes.Structure):
    _fields_ = [(k, ctypes.c_float) for k in
                ("omegam", "omegab", "omegal", "h", "fb", "rho_0", "rhocrit_0", "mypi")] + \
               [("rofztable", ctypes.c_float * 10000), ("zofrtable", ctypes.c_float * 10000)] + \
               [(k, ctypes.c_float) for k in
                ("drofztable", "dzofrtable", "rofztable_min", "zofrtable_min")]


_lib = None


def build():
    import sys
    sys.path.insert(0, os.path.dirname(HERE))
    from matt_young_mapmaking_gb300 import build as b
    return b.build_oracle()


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        VP, I32, I64, F, D = (ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_float,
                              ctypes.c_double)
        L.orc_cosmo_init.argtypes = [VP]
        L.orc_zofr.argtypes = [VP, F]
        L.orc_zofr.restype = F
        L.orc_rofz.argtypes = [VP, F]
        L.orc_rofz.restype = F
        L.orc_rhocrit.argtypes = [VP, F]
        L.orc_rhocrit.restype = F
        L.orc_deltacrit.argtypes = [VP, F]
        L.orc_deltacrit.restype = F
        L.orc_table_from_image.argtypes = [VP, VP, I64]
        L.orc_table_from_image.restype = I32
        L.orc_interpolate_table.argtypes = [VP, VP, F, F, ctypes.POINTER(F), I32]
        L.orc_interpolate_table.restype = F
        L.orc_ring_num.argtypes = [I32, D]
        L.orc_ring_num.restype = I32
        L.orc_ring2z.argtypes = [I32, I32]
        L.orc_ring2z.restype = D
        L.orc_pixels_per_ring.argtypes = [I32, I32, VP, VP, VP]
        L.orc_pix2vec_ring.argtypes = [I32, I64, VP]
        L.orc_angdist.argtypes = [VP, VP]
        L.orc_angdist.restype = D
        L.orc_query_disc.argtypes = [I32, VP, D, VP, I64, VP]
        L.orc_query_disc.restype = I64
        L.orc_paint.argtypes = [VP, VP, I32, VP, I64, VP, VP, VP, VP, VP, I64, VP]
        L.orc_paint.restype = I32
        L.orc_map_stats.argtypes = [VP, I64, VP, VP, VP]
        L.orc_map_stats.restype = None
        L.orc_generate_catalogue.argtypes = [ctypes.c_uint64, I64, I64, I32, D, D, D, D, D,
                                             D, VP, I32]
        L.orc_generate_catalogue.restype = I32
        L.orc_paint_parallel.argtypes = [VP, VP, I32, VP, I64, VP, VP, VP, VP, VP, I64, VP,
                                         I32]
        L.orc_paint_parallel.restype = I32
        L.orc_paint_threads.argtypes = [VP, VP, I32, VP, I64, VP, VP, I32, VP, VP]
        L.orc_paint_threads.restype = I32
        L.orc_paint_ranks.argtypes = [VP, VP, I32, VP, I64, VP, I32, VP]
        L.orc_paint_ranks.restype = I32
        L.orc_reduce_ranks.argtypes = [VP, I32, I64, VP, I32]
        L.orc_reduce_ranks.restype = None
        L.orc_zero_ranks.argtypes = [VP, I32, I64]
        L.orc_zero_ranks.restype = None
        L.orc_make_maptable.argtypes = [I32, F, F, I32, I32, I32, VP, I32]
        L.orc_make_maptable.restype = I64
        L.orc_halo_setup.argtypes = [VP, VP, VP, VP]
        L.orc_halo_setup.restype = I32
        _lib = L
    return _lib


def _stats_dict(st):
    return {k: (list(getattr(st, k)) if k == "centre" else getattr(st, k))
            for k, _ in OrcStats._fields_}


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


class Cosmo:
    def __init__(self):
        self.c = OrcCosmo()
        lib().orc_cosmo_init(ctypes.byref(self.c))

    def zofr(self, r):
        return lib().orc_zofr(ctypes.byref(self.c), r)

    def rofz(self, z):
        return lib().orc_rofz(ctypes.byref(self.c), z)

    def rhocrit(self, z):
        return lib().orc_rhocrit(ctypes.byref(self.c), z)

    def deltacrit(self, z):
        return lib().orc_deltacrit(ctypes.byref(self.c), z)


class Table:
    def __init__(self, image):
        self.buf = np.frombuffer(bytes(image), dtype=np.uint8).copy()
        self.t = OrcTable()
        rc = lib().orc_table_from_image(ctypes.byref(self.t), _p(self.buf), self.buf.size)
        if rc:
            raise ValueError("bad table image (%d)" % rc)

    def interpolate(self, cosmo, theta, z, mh, profile):
        m = ctypes.c_float(mh)
        v = lib().orc_interpolate_table(ctypes.byref(cosmo.c), ctypes.byref(self.t), theta, z,
                                        ctypes.byref(m), profile)
        return v, m.value


def make_maptable(model=1, nu=0.0, alpha_cmb=0.0, nchit=0, nmht=0, nrt=0, nthreads=None):
    nthreads = nthreads or os.cpu_count() or 1
    n = lib().orc_make_maptable(model, nu, alpha_cmb, nchit, nmht, nrt, None, nthreads)
    if n < 0:
        raise ValueError("bad table arguments")
    buf = np.zeros(n, dtype=np.uint8)
    lib().orc_make_maptable(model, nu, alpha_cmb, nchit, nmht, nrt, _p(buf), nthreads)
    return buf.tobytes()


def ring_num(nside, z):
    return lib().orc_ring_num(nside, z)


def ring2z(nside, ir):
    return lib().orc_ring2z(nside, ir)


def pixels_per_ring(nside, ring):
    npr, ks, npn = ctypes.c_int(), ctypes.c_int(), ctypes.c_int64()
    lib().orc_pixels_per_ring(nside, ring, ctypes.byref(npr), ctypes.byref(ks), ctypes.byref(npn))
    return npr.value, ks.value, npn.value


def pix2vec_ring(nside, ipix):
    v = np.zeros(3)
    lib().orc_pix2vec_ring(nside, ipix, _p(v))
    return v


def angdist(v1, v2):
    a = np.ascontiguousarray(v1, dtype=np.float64)
    b = np.ascontiguousarray(v2, dtype=np.float64)
    return lib().orc_angdist(_p(a), _p(b))


def query_disc(nside, vec, radius):
    v = np.ascontiguousarray(vec, dtype=np.float64)
    cap = 12 * nside * nside
    out = np.zeros(cap, dtype=np.int64)
    gaps = ctypes.c_int()
    n = lib().orc_query_disc(nside, _p(v), radius, _p(out), cap, ctypes.byref(gaps))
    if n < 0:
        raise ValueError("query_disc error %d" % n)
    return out[:n].copy(), bool(gaps.value)


def params(nside=512, npix_fs=0, fov_deg=10.0, zmin=0.0, zmax=1.25, chihview=0.0, model=1,
           maps=((0, 1),), fp32=False, nfloat=10, scramble=0, centre=0, ntasks=1):
    p = OrcParams()
    p.nside, p.npix_fs, p.fov_deg = nside, npix_fs, fov_deg
    p.zmin, p.zmax, p.chihview, p.model = zmin, zmax, chihview, model
    p.nmaps = len(maps)
    for i, (t, pr) in enumerate(maps):
        p.table_id[i], p.profile[i] = t, pr
    p.fp32_accumulate = 1 if fp32 else 0
    p.nfloat = nfloat
    p.scramble, p.centre, p.ntasks = scramble, centre, ntasks
    return p


def paint(p, tables, records, record_sets=False, set_cap=1 << 24, threads=1):
    """Runs the halo loop.  Returns (hp maps (nmaps, npix) or None, fs maps or None,
    stats dict, (set_rec, set_pix) or None).  threads > 1 (FP64 accumulation only): the
    same results bit for bit, computed on that many threads (orc_paint_parallel)."""
    if threads > 1 and not p.fp32_accumulate:
        return _paint_parallel(p, tables, records, record_sets, set_cap, threads)
    rec = np.ascontiguousarray(records, dtype=np.float32)
    n = rec.shape[0]
    tabs = (OrcTable * len(tables))(*[t.t for t in tables])
    dt = np.float32 if p.fp32_accumulate else np.float64
    hp = np.zeros((p.nmaps, 12 * p.nside * p.nside), dtype=dt) if p.nside > 0 else None
    fs = np.zeros((p.nmaps, p.npix_fs * p.npix_fs), dtype=dt) if p.npix_fs > 0 else None
    st = OrcStats()
    srec = spix = None
    nset = ctypes.c_int64()
    if record_sets:
        srec = np.zeros(set_cap, dtype=np.int64)
        spix = np.zeros(set_cap, dtype=np.int64)
    rc = lib().orc_paint(ctypes.byref(p), tabs, len(tables), _p(rec), n,
                         _p(hp) if hp is not None else None, _p(fs) if fs is not None else None,
                         ctypes.byref(st), _p(srec) if record_sets else None,
                         _p(spix) if record_sets else None, set_cap if record_sets else 0,
                         ctypes.byref(nset))
    if rc:
        raise RuntimeError("oracle paint failed (%d)" % rc)
    stats = _stats_dict(st)
    sets = None
    if record_sets:
        k = min(nset.value, set_cap)
        sets = (srec[:k].copy(), spix[:k].copy())
    return hp, fs, stats, sets


def _paint_parallel(p, tables, records, record_sets, set_cap, threads):
    rec = np.ascontiguousarray(records, dtype=np.float32)
    tabs = (OrcTable * len(tables))(*[t.t for t in tables])
    hp = np.empty((p.nmaps, 12 * p.nside * p.nside)) if p.nside > 0 else None
    fs = np.empty((p.nmaps, p.npix_fs * p.npix_fs)) if p.npix_fs > 0 else None
    st = OrcStats()
    nset = ctypes.c_int64()
    srec = np.empty(set_cap, dtype=np.int64) if record_sets else None
    spix = np.empty(set_cap, dtype=np.int64) if record_sets else None
    rc = lib().orc_paint_parallel(ctypes.byref(p), tabs, len(tables), _p(rec), rec.shape[0],
                                  _p(hp) if hp is not None else None,
                                  _p(fs) if fs is not None else None, ctypes.byref(st),
                                  _p(srec) if record_sets else None,
                                  _p(spix) if record_sets else None,
                                  set_cap if record_sets else 0, ctypes.byref(nset), threads)
    if rc:
        raise RuntimeError("oracle paint failed (%d)" % rc)
    sets = None
    if record_sets:
        if nset.value > set_cap:
            raise RuntimeError("oracle pixel sets: %d pairs, capacity %d" % (nset.value, set_cap))
        sets = (srec[:nset.value], spix[:nset.value])
    return hp, fs, _stats_dict(st), sets


def paint_threads(p, tables, records, nthreads):
    """Threads-as-ranks float painter; returns (hp, fs, stats, (t_setup, t_paint, t_reduce))."""
    rec = np.ascontiguousarray(records, dtype=np.float32)
    tabs = (OrcTable * len(tables))(*[t.t for t in tables])
    hp = np.zeros((p.nmaps, 12 * p.nside * p.nside), dtype=np.float32) if p.nside > 0 else None
    fs = np.zeros((p.nmaps, p.npix_fs * p.npix_fs), dtype=np.float32) if p.npix_fs > 0 else None
    st = OrcStats()
    t = np.zeros(3)
    rc = lib().orc_paint_threads(ctypes.byref(p), tabs, len(tables), _p(rec), rec.shape[0],
                                 _p(hp) if hp is not None else None,
                                 _p(fs) if fs is not None else None, nthreads, ctypes.byref(st),
                                 _p(t))
    if rc:
        raise RuntimeError("oracle paint failed (%d)" % rc)
    return hp, fs, _stats_dict(st), tuple(t)


class RankMaps:
    """Private HEALPix float maps of nranks threads-as-ranks, allocated and written once
    (the reference's per-rank `hpmapl = 0`), for painting repeated samples into them."""

    def __init__(self, p, nranks):
        self.n = p.nmaps * 12 * p.nside * p.nside
        self.maps = [np.empty(self.n, dtype=np.float32) for _ in range(nranks)]
        self.ptrs = (ctypes.c_void_p * nranks)(*[m.ctypes.data for m in self.maps])
        # every rank writes its own map now (in parallel), not while painting
        lib().orc_zero_ranks(self.ptrs, nranks, self.n)

    def zero(self):
        """`hpmapl = 0` of every rank, each rank writing its own maps"""
        lib().orc_zero_ranks(self.ptrs, len(self.maps), self.n)

    def paint(self, p, tables, records):
        rec = np.ascontiguousarray(records, dtype=np.float32)
        tabs = (OrcTable * len(tables))(*[t.t for t in tables])
        st = OrcStats()
        rc = lib().orc_paint_ranks(ctypes.byref(p), tabs, len(tables), _p(rec), rec.shape[0],
                                   self.ptrs, len(self.maps), ctypes.byref(st))
        if rc:
            raise RuntimeError("oracle paint failed (%d)" % rc)
        return _stats_dict(st)

    def reduce(self, nthreads):
        out = np.empty(self.n, dtype=np.float32)
        lib().orc_reduce_ranks(self.ptrs, len(self.maps), self.n, _p(out), nthreads)
        return out


def generate_catalogue(seed, n, nfloat=10, r=(100.0, 3000.0), m=(1e12, 1e15), slope=-0.9,
                       sigma_v=300.0, first=0, threads=None):
    """The synthetic catalogue of the GPU library's generate_catalogue, computed here
    (orc_generate_catalogue): (n, nfloat) float32, bit-identical on the same machine."""
    out = np.empty((n, nfloat), dtype=np.float32)
    rc = lib().orc_generate_catalogue(seed, first, n, nfloat, r[0], r[1], m[0], m[1], slope,
                                      sigma_v, _p(out), threads or os.cpu_count() or 1)
    if rc:
        raise ValueError("generate_catalogue: bad arguments")
    return out


def map_stats(m, dpdy=True):
    """pks2map.f90:321-357 over a float map: (moments[3], rms, dpdy[10000] or None)"""
    a = np.ascontiguousarray(m, dtype=np.float32)
    mom = np.zeros(3)
    rms = ctypes.c_double()
    dp = np.zeros(10000, dtype=np.float32) if dpdy else None
    lib().orc_map_stats(_p(a), a.size, _p(mom), ctypes.byref(rms),
                        _p(dp) if dp is not None else None)
    return mom, rms.value, dp


def fmath(fn, x, y=None):
    """Shared float math on the host (fn: 0 log 1 exp 2 pow 3 asin 4 atan 5 sin 6 cos 7 tan)."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    out = np.empty_like(x)
    yy = np.ascontiguousarray(y, dtype=np.float32) if y is not None else None
    L = lib()
    L.orc_fmath_eval.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                 ctypes.c_int64]
    L.orc_fmath_eval(fn, _p(x), _p(yy) if yy is not None else None, _p(out), x.size)
    return out


def halo_setup(cosmo, p, record):
    r = np.ascontiguousarray(record, dtype=np.float32)
    out = np.zeros(8, dtype=np.float32)
    ok = lib().orc_halo_setup(ctypes.byref(cosmo.c), ctypes.byref(p), _p(r), _p(out))
    return bool(ok), out
