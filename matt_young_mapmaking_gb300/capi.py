"""ctypes binding of the C ABI (include/p2m.h, include/p2m_tools.h).

The Painter class mirrors the reference's map-making interface for the hot path
(pks2map_src/): ``load_table`` is ``loadmaptable`` (maptable.f90:150-172),
``paint_records`` is ``loadpksc`` plus the halo loop (pksc.f90:22-90,
pks2map.f90:134-303), ``project_halo`` is ``projecthalo_flatsky`` followed by
``projecthalo_healpix`` (haloproject.f90:38-156), and ``healpix``/``flatsky`` return the
summed maps (pks2map.f90:313-314).  Every failure raises P2MError; there is no CPU path.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libp2m_gb300.so")

MAXMAPS = 8
NOALLOC_MAXMAPS = 8  # P2M_NOALLOC_MAXMAPS of include/p2m_tools.h
P2M_OK, P2M_ERR_BADARG, P2M_ERR_CUDA, P2M_ERR_CAPACITY = 0, 1, 2, 3
P2M_ERR_IO, P2M_ERR_STATE, P2M_ERR_NOMEM = 5, 6, 7
PREC_FP64, PREC_MIXED, PREC_MIXED_F64, PREC_FIXED = 0, 1, 2, 3
FLAG_RECORD_SETS, FLAG_ALL_HALOS, FLAG_TIMING, FLAG_VALIDATE = 1, 2, 4, 8
STATUS = {0: "OK", 1: "BADARG", 2: "CUDA", 3: "CAPACITY", 4: "TIMEOUT", 5: "IO", 6: "STATE",
          7: "NOMEM"}


class P2MError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("p2m error %s (%d): %s" % (STATUS.get(status, "?"), status, msg))
        self.status = status


class P2MMapStats(ctypes.Structure):
    _fields_ = [("npix", ctypes.c_int64), ("mom", ctypes.c_double * 3), ("rms", ctypes.c_double)]


class P2MConfig(ctypes.Structure):
    _fields_ = [
        ("nside", ctypes.c_int32),
        ("npix_fs", ctypes.c_int32),
        ("fov_deg", ctypes.c_float),
        ("zmin", ctypes.c_float),
        ("zmax", ctypes.c_float),
        ("chihview", ctypes.c_float),
        ("model", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("nmaps", ctypes.c_int32),
        ("map_table", ctypes.c_int32 * MAXMAPS),
        ("map_profile", ctypes.c_int32 * MAXMAPS),
        ("max_records", ctypes.c_int64),
        ("device", ctypes.c_int32),
        ("flags", ctypes.c_int32),
        ("ncones", ctypes.c_int32),
    ]


class P2MTuning(ctypes.Structure):
    _fields_ = [("big_rings", ctypes.c_int32), ("halos_grid", ctypes.c_int32),
                ("full_grid", ctypes.c_int32), ("full_chunk", ctypes.c_int32),
                ("stream_chunk", ctypes.c_int32), ("stream_paint", ctypes.c_int32),
                ("halo_batch", ctypes.c_int32), ("sort_halos", ctypes.c_int32),
                ("halos_threads", ctypes.c_int32), ("ms", ctypes.c_float)]


class P2MStats(ctypes.Structure):
    _fields_ = [
        ("n_records", ctypes.c_int64),
        ("n_shell", ctypes.c_int64),
        ("n_painted", ctypes.c_int64),
        ("n_enumerated", ctypes.c_int64),
        ("hp_candidates", ctypes.c_int64),
        ("hp_updates", ctypes.c_int64),
        ("fs_updates", ctypes.c_int64),
        ("n_recheck", ctypes.c_int64),
        ("val_checked", ctypes.c_int64),
        ("val_bad_set", ctypes.c_int64),
        ("val_bad_index", ctypes.c_int64),
        ("val_max_du", ctypes.c_float),
        ("hp_sum", ctypes.c_double * MAXMAPS),
        ("fs_sum", ctypes.c_double * MAXMAPS),
    ]


_lib = None


def load_library():
    """Load libp2m_gb300.so; raises if it has not been built (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise P2MError(6, "%s is not built; run `python -m matt_young_mapmaking_gb300.build`"
                       % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    P, I32, I64, F, D, VP = (ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_float,
                             ctypes.c_double, ctypes.c_void_p)
    FP = ctypes.POINTER(ctypes.c_float)
    sig = {
        "p2m_create": (I32, [ctypes.POINTER(P2MConfig), ctypes.POINTER(VP)]),
        "p2m_destroy": (None, [VP]),
        "p2m_last_error": (ctypes.c_char_p, [VP]),
        "p2m_load_table": (I32, [VP, I32, VP, I64]),
        "p2m_reset_maps": (I32, [VP]),
        "p2m_paint_records": (I32, [VP, VP, I64, I32]),
        "p2m_host_alloc": (I32, [I64, ctypes.POINTER(VP)]),
        "p2m_host_free": (I32, [VP]),
        "p2m_paint_records_device": (I32, [VP, VP, I64, I32, VP]),
        "p2m_project_halo": (I32, [VP, FP, FP, FP, FP, FP, FP, FP, FP,
                                   ctypes.POINTER(ctypes.c_int32)]),
        "p2m_flush": (I32, [VP]),
        "p2m_get_healpix": (I32, [VP, I32, VP]),
        "p2m_get_flatsky": (I32, [VP, I32, VP]),
        "p2m_get_healpix_device": (I32, [VP, I32, VP, VP]),
        "p2m_bind_healpix_device": (I32, [VP, I32, VP]),
        "p2m_get_stats": (I32, [VP, ctypes.POINTER(P2MStats)]),
        "p2m_synchronize": (I32, [VP]),
        "p2m_get_pixel_sets": (I32, [VP, VP, VP, I64, ctypes.POINTER(ctypes.c_int64)]),
        "p2m_make_maptable": (I32, [I32, I32, F, F, I32, I32, I32, VP,
                                    ctypes.POINTER(ctypes.c_int64)]),
        "p2m_generate_catalogue": (I32, [ctypes.c_uint64, I64, I64, I32, D, D, D, D, D, D, VP]),
        "p2m_philox4x32": (None, [VP, VP, VP]),
        "p2m_fmath_eval_device": (I32, [I32, I32, VP, VP, VP, I64]),
        "p2m_get_timings": (I32, [VP, VP, I32]),
        "p2m_map_sums_noalloc": (I32, [VP, I32, I64, VP, VP]),
        "p2m_set_preprocess": (I32, [VP, I32, I32, I32]),
        "p2m_set_cosmology_tables": (I32, [VP, VP, VP, I32, F, F]),
        "p2m_get_healpix_stats": (I32, [VP, I32, VP, VP]),
        "p2m_get_flatsky_stats": (I32, [VP, I32, VP]),
        "p2m_write_healpix_fits_device": (I32, [VP, I32, ctypes.c_char_p]),
        "p2m_get_centre": (I32, [VP, VP]),
        "p2m_dpdy": (I32, [VP, I64, VP]),
        "p2m_write_dpdy": (I32, [ctypes.c_char_p, VP]),
        "p2m_write_flatsky": (I32, [ctypes.c_char_p, VP, I32, F]),
        "p2m_write_healpix_fits": (I32, [ctypes.c_char_p, VP, I32]),
        "p2m_cl_healpix": (I32, [I32, VP, VP, I32, I32, VP, VP, VP]),
        "p2m_paint_ensemble": (I32, [VP, VP, VP, I32, I32]),
        "p2m_paint_ensemble_device": (I32, [VP, VP, VP, I32, I32, VP]),
        "p2m_get_healpix_cone": (I32, [VP, I32, I32, VP]),
        "p2m_get_tuning": (I32, [VP, ctypes.POINTER(P2MTuning)]),
        "p2m_get_healpix_async": (I32, [VP, I32, VP]),
        "p2m_set_tuning": (I32, [VP, ctypes.POINTER(P2MTuning)]),
        "p2m_autotune": (I32, [VP, VP, I64, I32, I32, ctypes.POINTER(P2MTuning)]),
        "p2m_cl_flatsky": (I32, [I32, VP, VP, I32, F, D, I32, VP, VP, VP, VP, VP]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    """Names the C ABI exports (include/p2m.h and include/p2m_tools.h)."""
    return ["p2m_create", "p2m_destroy", "p2m_last_error", "p2m_load_table", "p2m_reset_maps",
            "p2m_paint_records", "p2m_paint_records_device", "p2m_project_halo", "p2m_flush",
            "p2m_get_healpix", "p2m_get_flatsky", "p2m_get_healpix_device",
            "p2m_bind_healpix_device", "p2m_get_stats",
            "p2m_synchronize", "p2m_get_pixel_sets", "p2m_make_maptable",
            "p2m_generate_catalogue", "p2m_philox4x32", "p2m_fmath_eval_device",
            "p2m_get_timings", "p2m_map_sums_noalloc", "p2m_set_preprocess", "p2m_get_centre",
            "p2m_set_cosmology_tables", "p2m_get_healpix_stats", "p2m_get_flatsky_stats",
            "p2m_write_healpix_fits_device",
            "p2m_dpdy", "p2m_write_dpdy",
            "p2m_write_flatsky", "p2m_write_healpix_fits", "p2m_cl_healpix", "p2m_cl_flatsky",
            "p2m_paint_ensemble", "p2m_paint_ensemble_device", "p2m_get_healpix_cone",
            "p2m_get_tuning", "p2m_set_tuning", "p2m_autotune", "p2m_get_healpix_async",
            "p2m_host_alloc", "p2m_host_free"]


PHASES = ["cut", "setup", "big_scan", "big_items", "flatsky", "big_offsets", "paint", "paint_big",
          "readout"]


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


class Painter:
    """One painter context on one GPU.

    maps: sequence of (table_slot, profile) pairs; profile 1 paints the tSZ column of
    the table with weight 1, profile 2 the optical-depth column with weight -v_los/c.
    """

    def __init__(self, nside=4096, npix_fs=0, fov_deg=10.0, zmin=0.0, zmax=1.25,
                 chihview=0.0, model=1, precision=PREC_MIXED, maps=((0, 1),),
                 max_records=1 << 22, device=0, flags=0, ncones=0):
        self._lib = load_library()
        cfg = P2MConfig()
        cfg.nside, cfg.npix_fs, cfg.fov_deg = nside, npix_fs, fov_deg
        cfg.zmin, cfg.zmax, cfg.chihview, cfg.model = zmin, zmax, chihview, model
        if isinstance(precision, str):
            precision = {"fp64": PREC_FP64, "mixed": PREC_MIXED,
                         "mixed64": PREC_MIXED_F64, "fixed": PREC_FIXED}[precision]
        cfg.precision = precision
        maps = list(maps)
        if not 1 <= len(maps) <= MAXMAPS:
            raise P2MError(1, "1..%d maps" % MAXMAPS)
        cfg.nmaps = len(maps)
        for i, (t, p) in enumerate(maps):
            cfg.map_table[i], cfg.map_profile[i] = t, p
        cfg.max_records, cfg.device, cfg.flags = max_records, device, flags
        cfg.ncones = ncones
        self.ncones = max(ncones, 1)
        self.cfg = cfg
        self.nmaps = len(maps)
        self.nside, self.npix_fs = nside, npix_fs
        h = ctypes.c_void_p()
        st = self._lib.p2m_create(ctypes.byref(cfg), ctypes.byref(h))
        if st != 0:
            msg = self._lib.p2m_last_error(h).decode() if h.value else "create failed"
            if h.value:
                self._lib.p2m_destroy(h)
            raise P2MError(st, msg)
        self._h = h

    # -- plumbing ------------------------------------------------------------------
    def _check(self, st):
        if st != 0:
            raise P2MError(st, self._lib.p2m_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.p2m_destroy(self._h)
        self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # -- the reference's interface ---------------------------------------------------
    def set_preprocess(self, scramble=0, centre=0, ntasks=1):
        """pks2map's scramble / center flags (call right after creation or reset)."""
        self._check(self._lib.p2m_set_preprocess(self._h, scramble, centre, ntasks))

    def centre_info(self):
        """RTHmax, then distance, x, y, z of the largest halo before and after the rotation."""
        v = np.zeros(9, dtype=np.float32)
        self._check(self._lib.p2m_get_centre(self._h, _ptr(v)))
        return v

    def set_cosmology_tables(self, rofz, zofr, rofz_zmax=6.0, zofr_rmax=1.3e4):
        """Replace the r(z) and z(r) tables (10000 floats each, from 0 to rofz_zmax in z
        and to zofr_rmax Mpc in r)."""
        a = np.ascontiguousarray(rofz, dtype=np.float32)
        b = np.ascontiguousarray(zofr, dtype=np.float32)
        if a.shape != b.shape or a.ndim != 1:
            raise P2MError(1, "rofz and zofr must be 1-d arrays of one length")
        self._check(self._lib.p2m_set_cosmology_tables(self._h, _ptr(a), _ptr(b), a.size,
                                                       rofz_zmax, zofr_rmax))

    def map_stats(self, m=0, flatsky=False, dpdy=True):
        """Moments (3), RMS and, for a HEALPix map, the cumulative P(<y) (10000 floats) of
        map m, computed on the device (pks2map.f90:321-357)."""
        st = P2MMapStats()
        if flatsky:
            self._check(self._lib.p2m_get_flatsky_stats(self._h, m, ctypes.byref(st)))
            return list(st.mom), st.rms, None
        dp = np.zeros(NDPDY, dtype=np.float32) if dpdy else None
        self._check(self._lib.p2m_get_healpix_stats(self._h, m, ctypes.byref(st),
                                                    _ptr(dp) if dp is not None else None))
        return list(st.mom), st.rms, dp

    def write_healpix_fits(self, m, path):
        """HEALPix map m to a FITS file, converted and copied out from the device in
        slices that overlap the file write."""
        self._check(self._lib.p2m_write_healpix_fits_device(self._h, m, str(path).encode()))

    def load_table(self, slot, image):
        """loadmaptable: `image` is the table file's bytes (header + table)."""
        buf = np.frombuffer(bytes(image) if not isinstance(image, np.ndarray) else image.tobytes(),
                            dtype=np.uint8)
        self._check(self._lib.p2m_load_table(self._h, slot, _ptr(buf), buf.size))

    def reset(self):
        self._check(self._lib.p2m_reset_maps(self._h))

    def paint_records(self, records):
        """Catalogue records (n, 7) or (n, 10) float32 in host memory."""
        rec = np.ascontiguousarray(records, dtype=np.float32)
        if rec.ndim != 2 or rec.shape[1] not in (7, 10):
            raise P2MError(1, "records must be (n, 7) or (n, 10)")
        self._check(self._lib.p2m_paint_records(self._h, _ptr(rec), rec.shape[0], rec.shape[1]))

    def paint_records_device(self, dptr, n, nfloat, stream=None):
        self._check(self._lib.p2m_paint_records_device(self._h, ctypes.c_void_p(dptr), n, nfloat,
                                                       ctypes.c_void_p(stream or 0)))

    def paint_ensemble(self, records, offsets):
        """Ensemble form: records of independent light-cones, concatenated; cone c owns
        records[offsets[c]:offsets[c + 1]] and is painted to its own maps."""
        rec = np.ascontiguousarray(records, dtype=np.float32)
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        if rec.ndim != 2 or rec.shape[1] not in (7, 10):
            raise P2MError(1, "records must be (n, 7) or (n, 10)")
        if off.ndim != 1 or off.size < 2 or off[-1] != rec.shape[0]:
            raise P2MError(1, "offsets must hold ncones + 1 values ending at the record count")
        self._check(self._lib.p2m_paint_ensemble(self._h, _ptr(rec), _ptr(off), off.size - 1,
                                                 rec.shape[1]))

    def paint_ensemble_device(self, dptr, offsets, nfloat, stream=None):
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        self._check(self._lib.p2m_paint_ensemble_device(self._h, ctypes.c_void_p(dptr), _ptr(off),
                                                        off.size - 1, nfloat,
                                                        ctypes.c_void_p(stream or 0)))

    # -- launch parameters ---------------------------------------------------------
    def tuning(self):
        t = P2MTuning()
        self._check(self._lib.p2m_get_tuning(self._h, ctypes.byref(t)))
        return {k: getattr(t, k) for k, _ in P2MTuning._fields_}

    def set_tuning(self, **kw):
        t = P2MTuning(**{k: v for k, v in self.tuning().items()})
        for k, v in kw.items():
            setattr(t, k, v)
        self._check(self._lib.p2m_set_tuning(self._h, ctypes.byref(t)))

    def autotune(self, dptr, n, nfloat=10, reps=3):
        """Times candidate launch parameters on device records and keeps the fastest
        (include/p2m_tools.h p2m_autotune); returns the choice."""
        t = P2MTuning()
        self._check(self._lib.p2m_autotune(self._h, ctypes.c_void_p(dptr), n, nfloat, reps,
                                           ctypes.byref(t)))
        return {k: getattr(t, k) for k, _ in P2MTuning._fields_}

    def healpix_cone(self, cone, m=0):
        out = np.empty(12 * self.nside * self.nside, dtype=np.float32)
        self._check(self._lib.p2m_get_healpix_cone(self._h, cone, m, _ptr(out)))
        return out

    def project_halo(self, x, y, z, r, chi, m, redshift, v, profile):
        """Queue one halo with precomputed loop quantities; returns (x, y, z)/chi as the
        reference leaves them in its caller."""
        c = [ctypes.c_float(a) for a in (x, y, z, r, chi, m, redshift, v)]
        p = ctypes.c_int32(profile)
        self._check(self._lib.p2m_project_halo(self._h, *[ctypes.byref(a) for a in c],
                                               ctypes.byref(p)))
        return c[0].value, c[1].value, c[2].value

    def flush(self):
        self._check(self._lib.p2m_flush(self._h))

    def healpix(self, m=0):
        """Map m (with an ensemble: every cone's copy, cone-major)."""
        out = np.empty(12 * self.nside * self.nside * self.ncones, dtype=np.float32)
        self._check(self._lib.p2m_get_healpix(self._h, m, _ptr(out)))
        return out

    def healpix_into(self, m, host_ptr):
        """Read map m into host memory at host_ptr (12*nside^2 floats, e.g. pinned)."""
        self._check(self._lib.p2m_get_healpix(self._h, m, ctypes.c_void_p(host_ptr)))

    def healpix_async(self, m, host_ptr):
        """Queue the read-out of map m into host memory at host_ptr (pinned) and return;
        synchronize() waits for it."""
        self._check(self._lib.p2m_get_healpix_async(self._h, m, ctypes.c_void_p(host_ptr)))

    def bind_healpix_device(self, m, dptr):
        """Make device buffer dptr (12*nside^2 floats) the storage of map m."""
        self._check(self._lib.p2m_bind_healpix_device(self._h, m, ctypes.c_void_p(dptr)))

    def healpix_device(self, m, dptr, stream=None):
        self._check(self._lib.p2m_get_healpix_device(self._h, m, ctypes.c_void_p(dptr),
                                                     ctypes.c_void_p(stream or 0)))

    def flatsky(self, m=0):
        out = np.empty(self.npix_fs * self.npix_fs, dtype=np.float32)
        self._check(self._lib.p2m_get_flatsky(self._h, m, _ptr(out)))
        return out

    def synchronize(self):
        self._check(self._lib.p2m_synchronize(self._h))

    def stats(self):
        s = P2MStats()
        self._check(self._lib.p2m_get_stats(self._h, ctypes.byref(s)))
        d = {k: getattr(s, k) for k, _ in P2MStats._fields_ if k not in ("hp_sum", "fs_sum")}
        d["hp_sum"] = list(s.hp_sum)[: self.nmaps]
        d["fs_sum"] = list(s.fs_sum)[: self.nmaps]
        return d

    def timings(self):
        """Device ms per phase of the last paint call / read-out (needs FLAG_TIMING)."""
        ms = np.zeros(len(PHASES))
        self._check(self._lib.p2m_get_timings(self._h, _ptr(ms), len(PHASES)))
        return dict(zip(PHASES, ms.tolist()))

    def pixel_sets(self):
        n = ctypes.c_int64()
        self._check(self._lib.p2m_get_pixel_sets(self._h, None, None, 0, ctypes.byref(n)))
        rec = np.empty(n.value, dtype=np.int64)
        pix = np.empty(n.value, dtype=np.int64)
        self._check(self._lib.p2m_get_pixel_sets(self._h, _ptr(rec), _ptr(pix), n.value,
                                                 ctypes.byref(n)))
        return rec, pix


def make_maptable(model=1, nu=0.0, alpha_cmb=0.0, nchit=0, nmht=0, nrt=0, device=0):
    """make_maptable on the GPU; returns the table file image (bytes)."""
    lib = load_library()
    nb = ctypes.c_int64()
    st = lib.p2m_make_maptable(device, model, nu, alpha_cmb, nchit, nmht, nrt, None,
                               ctypes.byref(nb))
    if st:
        raise P2MError(st, "make_maptable size query failed")
    buf = np.empty(nb.value, dtype=np.uint8)
    st = lib.p2m_make_maptable(device, model, nu, alpha_cmb, nchit, nmht, nrt, _ptr(buf),
                               ctypes.byref(nb))
    if st:
        raise P2MError(st, "make_maptable failed")
    return buf.tobytes()


MAXCONES = 4096
CL_LMAX_MAX = 16384
CL_MAXBINS = 1024


def cl_healpix(map_a, map_b=None, lmax=None, device=0):
    """Angular power spectra of RING-ordered HEALPix maps on the GPU (include/p2m_tools.h
    p2m_cl_healpix).  Returns {"aa": C_l of map_a} plus "ab" and "bb" when map_b is given,
    each an array over l = 0 .. lmax (default 3 nside - 1)."""
    lib = load_library()
    a = np.ascontiguousarray(map_a, dtype=np.float32)
    nside = int(round(np.sqrt(a.size / 12.0)))
    if 12 * nside * nside != a.size:
        raise P2MError(1, "map size %d is not 12 nside^2" % a.size)
    if lmax is None:
        lmax = 3 * nside - 1
    b = None if map_b is None else np.ascontiguousarray(map_b, dtype=np.float32)
    if b is not None and b.size != a.size:
        raise P2MError(1, "maps differ in size")
    out = {k: np.zeros(lmax + 1) for k in (("aa", "ab", "bb") if b is not None else ("aa",))}
    st = lib.p2m_cl_healpix(device, _ptr(a), None if b is None else _ptr(b), nside, lmax,
                            _ptr(out["aa"]), None if b is None else _ptr(out["ab"]),
                            None if b is None else _ptr(out["bb"]))
    if st:
        raise P2MError(st, "p2m_cl_healpix failed")
    return out


def cl_flatsky(map_a, map_b=None, fov_rad=None, ell_max=8000.0, nbins=100, device=0):
    """Binned angular power spectra of npix x npix flat-sky maps over fov_rad (include/
    p2m_tools.h p2m_cl_flatsky).  Returns {"ell", "nmodes", "aa"} plus "ab" and "bb" when
    map_b is given."""
    lib = load_library()
    a = np.ascontiguousarray(map_a, dtype=np.float32).ravel()
    npix = int(round(np.sqrt(a.size)))
    if npix * npix != a.size or fov_rad is None:
        raise P2MError(1, "flat-sky maps are npix^2 floats with a field of view")
    b = None if map_b is None else np.ascontiguousarray(map_b, dtype=np.float32).ravel()
    if b is not None and b.size != a.size:
        raise P2MError(1, "maps differ in size")
    out = {"ell": np.zeros(nbins), "nmodes": np.zeros(nbins, dtype=np.int64),
           "aa": np.zeros(nbins)}
    if b is not None:
        out["ab"], out["bb"] = np.zeros(nbins), np.zeros(nbins)
    st = lib.p2m_cl_flatsky(device, _ptr(a), None if b is None else _ptr(b), npix, fov_rad,
                            ell_max, nbins, _ptr(out["ell"]), _ptr(out["aa"]),
                            None if b is None else _ptr(out["ab"]),
                            None if b is None else _ptr(out["bb"]), _ptr(out["nmodes"]))
    if st:
        raise P2MError(st, "p2m_cl_flatsky failed")
    return out


def generate_catalogue(seed, n, nfloat=10, r=(100.0, 3000.0), m=(1e12, 1e15), slope=-0.9,
                       sigma_v=300.0, first=0):
    """Synthetic catalogue records (n, nfloat) float32 (see include/p2m_tools.h)."""
    lib = load_library()
    out = np.empty((n, nfloat), dtype=np.float32)
    st = lib.p2m_generate_catalogue(seed, first, n, nfloat, r[0], r[1], m[0], m[1], slope,
                                    sigma_v, _ptr(out))
    if st:
        raise P2MError(1, "generate_catalogue: bad arguments")
    return out


NDPDY = 10000


def _status(st, what):
    if st:
        raise P2MError(st, what)


def dpdy(hp_map):
    """P(<y) of a HEALPix map as pks2map computes it (pks2map.f90:340-357)."""
    m = np.ascontiguousarray(hp_map, dtype=np.float32)
    out = np.empty(NDPDY, dtype=np.float32)
    _status(load_library().p2m_dpdy(_ptr(m), m.size, _ptr(out)), "p2m_dpdy")
    return out


def write_outputs(fileout, hp_map=None, nside=0, fs_map=None, npix_fs=0, fov_rad=0.0):
    """The files pks2map writes: <fileout>_dp.bin and _hp.fits from the HEALPix map,
    <fileout>_fs.map from the flat-sky map."""
    lib = load_library()
    if hp_map is not None:
        m = np.ascontiguousarray(hp_map, dtype=np.float32)
        d = dpdy(m)
        _status(lib.p2m_write_dpdy((fileout + "_dp.bin").encode(), _ptr(d)), "_dp.bin")
        _status(lib.p2m_write_healpix_fits((fileout + "_hp.fits").encode(), _ptr(m), nside),
                "_hp.fits")
    if fs_map is not None:
        f = np.ascontiguousarray(fs_map, dtype=np.float32)
        _status(lib.p2m_write_flatsky((fileout + "_fs.map").encode(), _ptr(f), npix_fs,
                                      float(fov_rad)), "_fs.map")
