"""GPU angular power spectra (p2m_cl_healpix, p2m_cl_flatsky, through the C ABI) against
the numpy/scipy oracle on the same maps, and the precision report's spectrum ratio of
the mixed painter against the FP64 painter."""
import math

import numpy as np
import pytest

import catalogs
import matt_young_mapmaking_gb300 as p2m
import spectra

pytestmark = pytest.mark.gpu

REL = 1e-9  # FP64 transform against FP64 direct sums


def close(gpu, ref, rel=REL, floor=1e-12):
    gpu, ref = np.asarray(gpu), np.asarray(ref)
    scale = np.abs(ref).max()
    sel = np.abs(ref) > floor * scale
    err = np.abs(gpu - ref)
    assert (err[sel] / np.abs(ref[sel])).max() <= rel, (err[sel] / np.abs(ref[sel])).max()
    assert err[~sel].max(initial=0.0) <= rel * floor * scale


def painted(nside, npix_fs=0, precision="fp64", n=20_000, seed=31):
    rec = catalogs.shell(seed, n, r=(100.0, 3000.0), m=(1e12, 1e15))
    with p2m.Painter(nside=nside, npix_fs=npix_fs, fov_deg=10.0, precision=precision,
                     maps=((0, 1), (0, 2)), max_records=len(rec)) as pt:
        pt.load_table(0, catalogs.table())
        pt.paint_records(rec)
        hp = [pt.healpix(m) for m in range(2)] if nside else None
        fs = [pt.flatsky(m) for m in range(2)] if npix_fs else None
    return hp, fs


@pytest.mark.parametrize("nside,lmax", [(16, 47), (16, 64), (32, 95)])
def test_healpix_random_maps(nside, lmax):
    """White-noise maps; lmax = 64 at Nside 16 exceeds every cap ring's Nyquist m."""
    rng = np.random.default_rng(nside + lmax)
    a = rng.standard_normal(12 * nside * nside).astype(np.float32)
    b = (0.3 * a + rng.standard_normal(a.size)).astype(np.float32)
    g = p2m.cl_healpix(a, b, lmax=lmax)
    r = spectra.cl_healpix(a, b, nside, lmax)
    for k in ("aa", "ab", "bb"):
        close(g[k], r[k])


def test_healpix_painted_map_and_single_map():
    """A painted tSZ map (C_l over many decades), and the one-map form."""
    hp, _ = painted(32)
    g = p2m.cl_healpix(hp[0], None, lmax=95)
    r = spectra.cl_healpix(hp[0], None, 32, 95)
    assert set(g) == {"aa"}
    close(g["aa"], r["aa"])
    g2 = p2m.cl_healpix(hp[0], hp[1], lmax=95)
    r2 = spectra.cl_healpix(hp[0], hp[1], 32, 95)
    for k in ("aa", "ab", "bb"):
        close(g2[k], r2[k], floor=1e-10)


@pytest.mark.parametrize("npix", [256, 96])
def test_flatsky_random_maps(npix):
    """Power-of-two size (shared-memory FFT) and another size (direct DFT)."""
    rng = np.random.default_rng(npix)
    a = rng.standard_normal(npix * npix).astype(np.float32)
    b = (0.5 * a + rng.standard_normal(a.size)).astype(np.float32)
    fov = math.radians(10.0)
    g = p2m.cl_flatsky(a, b, fov_rad=fov, ell_max=3000.0, nbins=40)
    r = spectra.cl_flatsky(a, b, fov, 3000.0, 40)
    assert np.array_equal(g["nmodes"], r["nmodes"])
    np.testing.assert_allclose(g["ell"], r["ell"], rtol=1e-12)
    for k in ("aa", "ab", "bb"):
        close(g[k], r[k])


def test_flatsky_painted_1024():
    _, fs = painted(0, npix_fs=1024, n=40_000)
    fov = math.radians(10.0)
    g = p2m.cl_flatsky(fs[0], fs[1], fov_rad=fov, ell_max=8000.0, nbins=80)
    r = spectra.cl_flatsky(fs[0], fs[1], fov, 8000.0, 80)
    assert np.array_equal(g["nmodes"], r["nmodes"])
    for k in ("aa", "ab", "bb"):
        close(g[k], r[k], floor=1e-10)


def test_mixed_against_fp64_spectrum_ratio():
    """The precision report's C_l ratio: mixed painter over FP64 painter, both maps."""
    nside = 128
    hp64, _ = painted(nside, precision="fp64", n=40_000, seed=32)
    hpm, _ = painted(nside, precision="mixed", n=40_000, seed=32)
    for m in range(2):
        c = p2m.cl_healpix(hpm[m], hp64[m], lmax=3 * nside - 1)
        ratio = c["aa"][1:] / c["bb"][1:]
        assert np.abs(ratio - 1.0).max() < 1e-5, np.abs(ratio - 1.0).max()
        # the cross spectrum is the geometric mean up to the same order
        assert np.abs(c["ab"][1:] / np.sqrt(c["aa"][1:] * c["bb"][1:]) - 1.0).max() < 1e-5
