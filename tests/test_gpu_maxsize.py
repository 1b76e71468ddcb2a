"""The largest configurations the reference accepts: HEALPix Nside 8192 (805M pixels) and
the 8192^2 flat-sky map of the precision form, against the oracle on the same records."""
import numpy as np
import pytest

import catalogs
from test_gpu_parity import REL_TOL, MASK_FRAC, SUM_TOL, assert_sets_equal, run_gpu, run_oracle

pytestmark = pytest.mark.gpu


def assert_close_sparse(gpu, ref, rel=REL_TOL, what="map"):
    """assert_maps_close restricted to the pixels nonzero in either map: the others are
    zero in both and carry no error."""
    idx = np.union1d(np.flatnonzero(ref), np.flatnonzero(gpu))
    assert idx.size > 0, what
    r = np.asarray(ref[idx], dtype=np.float64)
    g = np.asarray(gpu[idx], dtype=np.float64)
    mx = np.abs(r).max()
    mask = np.abs(r) > MASK_FRAC * mx
    err = np.abs(g - r)
    worst = (err[mask] / np.abs(r[mask])).max()
    assert worst <= rel, "%s: max rel err %.3g" % (what, worst)
    assert err[~mask].max(initial=0.0) <= rel * MASK_FRAC * mx, what
    assert abs(g.sum() - r.sum()) <= SUM_TOL * abs(r.sum()), what


def far_edge_cases():
    """The hand-placed halos (poles, phi = 0, cap boundary) that lie far enough for their
    discs to stay within the recorded pixel-set capacity at Nside 8192."""
    e = catalogs.edge_cases()
    r = np.linalg.norm(e[:, :3].astype(np.float64), axis=1)
    return e[r >= 1200.0]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_healpix_nside_8192(precision):
    rec = np.concatenate([far_edge_cases(),
                          catalogs.shell(41, 1500, r=(800.0, 3000.0), m=(1e12, 1e15))])
    tab = catalogs.table()
    hp, _, st, sets = run_gpu(rec, [tab], precision, 8192)
    rhp, _, rst, rsets = run_oracle(rec, [tab], 8192)
    assert st["hp_updates"] == rst["hp_updates"] > 0
    assert_sets_equal(sets, rsets)
    assert_close_sparse(hp[0], rhp[0], what="Nside 8192 " + precision)


def test_flatsky_8192():
    rec = catalogs.cone(42, 6000, (1.0, 0.0, 0.0), 8.0, r=(1000.0, 3000.0))
    tab = catalogs.table()
    _, fs, st, _ = run_gpu(rec, [tab], "mixed", 0, npix_fs=8192, fov_deg=10.0, flags=0)
    _, rfs, rst, _ = run_oracle(rec, [tab], 0, npix_fs=8192, fov_deg=10.0)
    assert st["fs_updates"] == rst["fs_updates"] > 0
    assert_close_sparse(fs[0], rfs[0], rel=1e-6, what="flat sky 8192^2")
