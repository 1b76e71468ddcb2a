"""The spectra oracle against known answers, and the argument checks of the C-ABI spectra
entry points (rejected before any device call, so no GPU is needed)."""
import math

import numpy as np
import pytest

import matt_young_mapmaking_gb300 as p2m
import spectra


def test_flatsky_single_mode():
    """A cosine of wave vector (3, 4) puts fov^2 / 2 into the bin holding |k| = 5."""
    n, fov = 64, 0.1
    x = np.arange(n)
    m = np.cos(2 * np.pi * (3 * x[:, None] + 4 * x[None, :]) / n).astype(np.float32)
    ell_fund = 2 * np.pi / float(np.float32(fov))
    o = spectra.cl_flatsky(m, None, fov, ell_fund * 10, 20)
    hot = np.nonzero(o["aa"] > 1e-12 * o["aa"].max())[0]
    assert list(hot) == [int(5 * ell_fund / (ell_fund * 10) * 20)]
    # the map is rounded to float32, so the power is exact only to ~1e-8
    assert (o["aa"] * o["nmodes"]).sum() == pytest.approx(float(np.float32(fov)) ** 2 / 2, rel=1e-6)


def test_healpix_single_harmonic():
    """Re Y_32 sampled at Nside 16: C_3 = 1/14 up to the quadrature error, nothing
    elsewhere above 1e-6 of it."""
    sp = pytest.importorskip("scipy.special")
    nside = 16
    rings = spectra.healpix_rings(nside)
    th = np.concatenate([np.full(len(r[1]), r[0]) for r in rings])
    ph = np.concatenate([r[1] for r in rings])
    assert th.size == 12 * nside * nside
    y = sp.sph_harm_y(3, 2, th, ph) if hasattr(sp, "sph_harm_y") else sp.sph_harm(2, 3, ph, th)
    c = spectra.cl_healpix(np.real(y), None, nside, 3 * nside - 1)["aa"]
    assert c[3] == pytest.approx(1.0 / 14.0, rel=2e-3)
    assert np.delete(c, 3).max() < 1e-6 * c[3]


def test_healpix_ring_layout():
    """Ring sizes 4 min(i, N, 4N - i) and equatorial half-pixel shifts alternate."""
    nside = 8
    rings = spectra.healpix_rings(nside)
    sizes = [len(r[1]) for r in rings]
    assert sizes == [4 * min(i, nside, 4 * nside - i) for i in range(1, 4 * nside)]
    assert sum(sizes) == 12 * nside * nside
    dphi = [r[1][0] * len(r[1]) / math.pi for r in rings[nside - 1:3 * nside]]
    assert all(abs(d - (1 - (i % 2))) < 1e-12 for i, d in enumerate(dphi))


@pytest.mark.parametrize("kw", [dict(nside=16, lmax=65), dict(nside=12, lmax=10),
                                dict(nside=16, lmax=-1)])
def test_cl_healpix_rejects_bad_arguments(kw):
    lib = p2m.load_library()
    m = np.zeros(12 * kw["nside"] ** 2, dtype=np.float32)
    out = np.zeros(max(kw["lmax"], 0) + 1)
    st = lib.p2m_cl_healpix(0, m.ctypes.data, None, kw["nside"], kw["lmax"], out.ctypes.data,
                            None, None)
    assert st == p2m.capi.P2M_ERR_BADARG


@pytest.mark.parametrize("npix,nbins", [(16384, 10), (2050, 10), (64, 1025), (64, 0)])
def test_cl_flatsky_rejects_bad_arguments(npix, nbins):
    lib = p2m.load_library()
    m = np.zeros(1, dtype=np.float32)
    nb = max(nbins, 1)
    ell, cl = np.zeros(nb), np.zeros(nb)
    nm = np.zeros(nb, dtype=np.int64)
    st = lib.p2m_cl_flatsky(0, m.ctypes.data, None, npix, 0.1, 8000.0, nbins, ell.ctypes.data,
                            cl.ctypes.data, None, None, nm.ctypes.data)
    assert st == p2m.capi.P2M_ERR_BADARG
