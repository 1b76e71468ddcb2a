"""Host-side checks that need no GPU: the C ABI library loads and exports every symbol
its headers declare, configuration errors are reported without touching CUDA, the file
formats round-trip, the catalogue generator is deterministic, and the shared float math
is accurate."""
import ctypes
import os
import re

import numpy as np
import pytest

import matt_young_mapmaking_gb300 as p2m
import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in ("p2m.h", "p2m_tools.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(p2m_[a-z0-9_]+)\s*\(", src):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol():
    lib = p2m.load_library()
    declared = declared_functions()
    assert declared >= {"p2m_create", "p2m_paint_records", "p2m_get_healpix"}
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(p2m.exported_symbols()) == declared


def test_bad_configs_rejected_before_cuda():
    lib = p2m.load_library()

    def create(**kw):
        cfg = p2m.P2MConfig()
        cfg.nside, cfg.model, cfg.nmaps, cfg.precision = 64, 1, 1, 1
        cfg.map_profile[0] = 1
        for k, v in kw.items():
            setattr(cfg, k, v)
        h = ctypes.c_void_p()
        st = lib.p2m_create(ctypes.byref(cfg), ctypes.byref(h))
        if h.value:
            lib.p2m_destroy(h)
        return st
    assert create(nside=100) == 1          # not a power of 2
    assert create(nside=16384) == 1        # beyond Nside 8192
    assert create(nside=0, npix_fs=0) == 1  # no map at all
    assert create(model=4) == 1
    assert create(nmaps=9) == 1
    assert create(precision=7) == 1


def test_pksc_roundtrip_and_layout_detection(tmp_path):
    rec10 = p2m.generate_catalogue(3, 257, 10)
    rec7 = np.ascontiguousarray(rec10[:, :7])
    for rec in (rec10, rec7):
        path = str(tmp_path / ("c%d.pksc" % rec.shape[1]))
        p2m.write_pksc(path, rec, zbox=0.5)
        hdr, got = p2m.read_pksc(path)
        assert hdr["nfloat"] == rec.shape[1] and hdr["nhalo"] == 257
        assert np.array_equal(got, rec)
        assert hdr["rthmax"] == rec[:, 6].max()
    assert p2m.detect_layout(8 + 28 * 5, 5) == 7
    assert p2m.detect_layout(12 + 40 * 5, 5) == 10
    with pytest.raises(ValueError):
        p2m.detect_layout(8 + 28 * 5 + 3, 5)


def test_truncated_pksc_raises(tmp_path):
    rec = p2m.generate_catalogue(3, 10, 7)
    path = str(tmp_path / "t.pksc")
    p2m.write_pksc(path, rec)
    with open(path, "r+b") as f:
        f.truncate(8 + 28 * 9)
    with pytest.raises(ValueError):
        p2m.read_pksc(path, nfloat=7)


def test_generator_deterministic_and_offsettable():
    a = p2m.generate_catalogue(7, 1000, 10, r=(100.0, 8000.0), m=(1e12, 3e15))
    b = p2m.generate_catalogue(7, 1000, 10, r=(100.0, 8000.0), m=(1e12, 3e15))
    c = p2m.generate_catalogue(7, 300, 10, r=(100.0, 8000.0), m=(1e12, 3e15), first=700)
    assert np.array_equal(a, b) and np.array_equal(a[700:], c)
    r = np.linalg.norm(a[:, :3].astype(np.float64), axis=1)
    assert r.min() >= 99.9 and r.max() <= 8000.1
    assert np.allclose(a[:, 7:10], a[:, :3] - 0.01 * a[:, 3:6], atol=1e-3)


def test_philox_known_answer():
    # Random123's published known-answer vector for philox4x32-10 with zero counter/key
    lib = p2m.load_library()
    c = (ctypes.c_uint32 * 4)(0, 0, 0, 0)
    k = (ctypes.c_uint32 * 2)(0, 0)
    o = (ctypes.c_uint32 * 4)()
    lib.p2m_philox4x32(c, k, o)
    assert list(o) == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]


@pytest.mark.parametrize("fn,lo,hi,logscale,max_ulp", [
    (0, 1e-30, 1e30, True, 2.0), (1, -87.0, 88.0, False, 1.5), (3, -1.0, 1.0, False, 2.0),
    (4, -50.0, 50.0, False, 2.0), (5, -10.0, 10.0, False, 2.0), (6, -10.0, 10.0, False, 2.0),
    (7, 0.0, 1.5, False, 3.5)])
def test_float_math_accuracy(fn, lo, hi, logscale, max_ulp):
    rng = np.random.default_rng(fn)
    u = rng.random(200_000)
    x = (np.exp(np.log(lo) + u * (np.log(hi) - np.log(lo))) if logscale else lo + u * (hi - lo))
    x = x.astype(np.float32)
    got = oracle.fmath(fn, x).astype(np.float64)
    ref = [np.log, np.exp, None, np.arcsin, np.arctan, np.sin, np.cos, np.tan][fn](x.astype(np.float64))
    r32 = ref.astype(np.float32)
    ulp = np.spacing(np.abs(r32)).astype(np.float64)
    err = np.abs(got - ref) / ulp
    assert err.max() <= max_ulp


def test_pow_accuracy_and_special_cases():
    rng = np.random.default_rng(5)
    x = np.exp(rng.uniform(-7, 7, 100_000)).astype(np.float32)
    for y in (np.float32(1 / 3), np.float32(-0.3), np.float32(-4.5)):
        got = oracle.fmath(2, x, np.full_like(x, y)).astype(np.float64)
        ref = np.power(x.astype(np.float64), float(y))
        ulp = np.spacing(np.abs(ref.astype(np.float32))).astype(np.float64)
        assert (np.abs(got - ref) / ulp).max() <= 8.0
    one = oracle.fmath(2, np.array([3.7, 0.5], np.float32), np.array([1.0, 0.0], np.float32))
    assert one[0] == np.float32(3.7) and one[1] == 1.0


def test_restricted_float_functions_equal_the_general_ones():
    """The painting path's tan for 0 <= x < pi/4 and log for positive normal x give the
    general functions' results bit for bit over their ranges (fn 9 / 7, fn 10 / 0)."""
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.uniform(0.0, 0.78539, 200_000),
                        np.float32(0.78539816) * rng.random(1000) ** 8]).astype(np.float32)
    assert np.array_equal(oracle.fmath(9, x).view(np.uint32), oracle.fmath(7, x).view(np.uint32))
    y = np.exp(rng.uniform(-80.0, 80.0, 200_000)).astype(np.float32)
    y = np.concatenate([y, np.array([1.1754944e-38, 1.0, 3.4e38], np.float32)])
    assert np.array_equal(oracle.fmath(10, y).view(np.uint32), oracle.fmath(0, y).view(np.uint32))


def test_host_alloc_argument_checks():
    """p2m_host_alloc refuses a negative size or a null result pointer before any CUDA
    call; p2m_host_free of NULL is a no-op."""
    lib = p2m.load_library()
    ptr = ctypes.c_void_p(1234)
    assert lib.p2m_host_alloc(-1, ctypes.byref(ptr)) == p2m.capi.P2M_ERR_BADARG
    assert ptr.value is None
    assert lib.p2m_host_alloc(16, None) == p2m.capi.P2M_ERR_BADARG
    assert lib.p2m_host_free(None) == p2m.capi.P2M_OK
