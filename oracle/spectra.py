"""TEST INFRASTRUCTURE ONLY: numpy/scipy restatement of the angular power spectra that
p2m_cl_healpix and p2m_cl_flatsky compute on the GPU.

Only tests/ and bench.py's error report import this module; the product never does.

HEALPix: the pixel-area quadrature of the HEALPix library that the reference vendors,
map2alm without iterations and with unit ring weights
(src/modules/External/alm_map_dd_inc.F90:2978-3224), then alm2cl (:5347-5423):
    a_lm = (4 pi / npix) sum_p f_p conj(Y_lm(theta_p, phi_p)).
It is evaluated here without the GPU's two devices, the phase-stepped ring sums and the
Legendre recursion.  Each ring's sum over phi uses explicit complex exponentials at the
pixel centres of get_pixel_layout (alm_tools.F90:311-349), and lambda_lm(theta) =
Y_lm(theta, 0) comes from scipy.  HEALPix skips terms below l_min_ylm (:882-903); they
are below double precision, and the direct sum keeps them.

Flat sky: numpy's FFT periodogram with the GPU's binning (no reference counterpart).
"""
import math

import numpy as np


def _ylm_theta(lmax, theta):
    """lambda_lm(theta) = Y_lm(theta, 0) for l, m <= lmax: array [l, m, ring] (0 for m > l)."""
    import scipy.special as sp
    ls = np.arange(lmax + 1)[:, None, None]
    ms = np.arange(lmax + 1)[None, :, None]
    th = np.asarray(theta, dtype=np.float64)[None, None, :]
    valid = ms <= ls
    lb, mb, tb = np.broadcast_arrays(ls, ms, th)
    out = np.zeros(lb.shape)
    sel = np.broadcast_to(valid, lb.shape)
    if hasattr(sp, "sph_harm_y"):
        y = sp.sph_harm_y(lb[sel], mb[sel], tb[sel], 0.0)
    else:  # older scipy: sph_harm(m, n, azimuth, polar)
        y = sp.sph_harm(mb[sel], lb[sel], 0.0, tb[sel])
    out[sel] = np.real(y)
    return out


def healpix_rings(nside):
    """(theta, phi of the pixel centres, first pixel) of rings 1 .. 4 nside - 1, RING order."""
    rings = []
    n = nside
    start = 0
    for i in range(1, 4 * n):
        if i < n or i > 3 * n:
            ir = i if i < n else 4 * n - i
            z = 1.0 - ir * ir / (3.0 * n * n)
            if i > 3 * n:
                z = -z
            nph = 4 * ir
            phi = math.pi * (2 * np.arange(nph) + 1) / nph
        else:
            z = (2 * n - i) * (2.0 / (3.0 * n))
            nph = 4 * n
            shift = (i - n + 1) % 2
            phi = math.pi * (2 * np.arange(nph) + shift) / nph
        rings.append((math.acos(z), phi, start))
        start += nph
    return rings


def alm_healpix(maps, nside, lmax):
    """a_lm [map][l, m] (complex, m <= l) by the direct quadrature sum."""
    rings = healpix_rings(nside)
    npix = 12 * nside * nside
    theta = np.array([r[0] for r in rings])
    lam = _ylm_theta(lmax, theta)                      # [l, m, ring]
    ms = np.arange(lmax + 1)
    out = []
    for f in maps:
        f = np.asarray(f, dtype=np.float64)
        F = np.zeros((len(rings), lmax + 1), dtype=np.complex128)
        for r, (_, phi, s) in enumerate(rings):
            vals = f[s:s + len(phi)]
            F[r] = np.exp(-1j * np.outer(ms, phi)) @ vals
        a = np.einsum("lmr,rm->lm", lam, F) * (4.0 * math.pi / npix)
        out.append(a)
    return out


def cl_from_alm(a, b):
    """alm2cl: (Re a_l0 b_l0 + 2 sum_{m>=1} Re a_lm conj b_lm) / (2l + 1)."""
    lmax = a.shape[0] - 1
    cl = np.zeros(lmax + 1)
    for l in range(lmax + 1):
        s = np.sum(a[l, 1:l + 1] * np.conj(b[l, 1:l + 1])).real
        cl[l] = (2.0 * s + (a[l, 0] * b[l, 0]).real) / (2.0 * l + 1.0)
    return cl


def cl_healpix(map_a, map_b, nside, lmax):
    maps = [map_a] if map_b is None else [map_a, map_b]
    al = alm_healpix(maps, nside, lmax)
    out = {"aa": cl_from_alm(al[0], al[0])}
    if map_b is not None:
        out["ab"] = cl_from_alm(al[0], al[1])
        out["bb"] = cl_from_alm(al[1], al[1])
    return out


def cl_flatsky(map_a, map_b, fov_rad, ell_max, nbins):
    """Binned periodogram: bins of ell = 2 pi |k| / fov in (0, ell_max], k = 0 and the
    Nyquist line left out, C = (fov^2 / npix^4) |FFT|^2 averaged over each bin."""
    a = np.asarray(map_a, dtype=np.float64).ravel()
    npix = int(round(math.sqrt(a.size)))
    Fa = np.fft.fft2(a.reshape(npix, npix))
    Fb = None if map_b is None else np.fft.fft2(
        np.asarray(map_b, dtype=np.float64).reshape(npix, npix))
    ell_fund = 2.0 * math.pi / float(np.float32(fov_rad))
    kmax = min(int(math.ceil(ell_max / ell_fund)), npix // 2 - 1)
    k = np.fft.fftfreq(npix) * npix
    k1, k2 = np.meshgrid(k, k, indexing="ij")
    ell = ell_fund * np.sqrt(k1 * k1 + k2 * k2)
    sel = (np.abs(k1) <= kmax) & (np.abs(k2) <= kmax) & ~((k1 == 0) & (k2 == 0)) & (ell <= ell_max)
    b = np.minimum((ell[sel] / ell_max * nbins).astype(np.int64), nbins - 1)
    cnt = np.bincount(b, minlength=nbins).astype(np.float64)
    fov = float(np.float32(fov_rad))
    norm = fov * fov / float(npix) ** 4
    out = {"nmodes": cnt.astype(np.int64)}
    with np.errstate(invalid="ignore", divide="ignore"):
        out["ell"] = np.where(cnt > 0, np.bincount(b, ell[sel], nbins) / cnt,
                              (np.arange(nbins) + 0.5) * ell_max / nbins)
        out["aa"] = np.where(cnt > 0, norm * np.bincount(b, np.abs(Fa[sel]) ** 2, nbins) / cnt, 0)
        if Fb is not None:
            out["ab"] = np.where(cnt > 0, norm * np.bincount(
                b, (Fa[sel] * np.conj(Fb[sel])).real, nbins) / cnt, 0)
            out["bb"] = np.where(cnt > 0, norm * np.bincount(b, np.abs(Fb[sel]) ** 2, nbins) / cnt, 0)
    return out
