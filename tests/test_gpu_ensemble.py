"""Ensemble form (p2m_paint_ensemble): independent light-cones painted in one call, each to
its own maps, against the oracle painting each cone's catalogue on its own."""
import numpy as np
import pytest

import catalogs
import matt_young_mapmaking_gb300 as p2m
import oracle
from test_gpu_parity import FLAGS, PRECISIONS, assert_maps_close, assert_sets_equal

pytestmark = pytest.mark.gpu

NSIDE = 64
MAPS = ((0, 1), (0, 2))
# uneven cones, one of them empty, each with its own seed and shell depth
CONES = [(5001, 600, 1500.0), (5002, 4000, 6000.0), (5003, 0, 2000.0), (5004, 9000, 3000.0),
         (5005, 2500, 1000.0)]


def ensemble():
    recs = [catalogs.shell(seed, n, r=(100.0, depth), m=(1e12, 3e15)) if n else
            np.zeros((0, 10), np.float32) for seed, n, depth in CONES]
    off = np.concatenate([[0], np.cumsum([len(r) for r in recs])]).astype(np.int64)
    return recs, off


def oracle_cones(recs, tab):
    out = []
    for r in recs:
        p = oracle.params(nside=NSIDE, maps=MAPS, zmax=6.0, nfloat=10)
        out.append(oracle.paint(p, [oracle.Table(tab)], r, record_sets=True) if len(r) else None)
    return out


def painter(precision, ncones, **kw):
    kw.setdefault("max_records", 1 << 16)
    pt = p2m.Painter(nside=NSIDE, precision=precision, maps=MAPS, zmax=6.0, flags=FLAGS,
                     ncones=ncones, **kw)
    pt.load_table(0, catalogs.table(nu=0.0))
    return pt


def check_cones(pt, recs, off, ref):
    gs = pt.pixel_sets()
    rs_rec, rs_pix = [], []
    for c, r in enumerate(ref):
        for m in range(len(MAPS)):
            got = pt.healpix_cone(c, m)
            if r is None:
                assert not np.any(got), "empty cone %d painted" % c
            else:
                assert_maps_close(got, r[0][m], what="cone %d map %d" % (c, m))
        if r is not None:
            rs_rec.append(r[3][0] + off[c])
            rs_pix.append(r[3][1])
    assert_sets_equal(gs, (np.concatenate(rs_rec), np.concatenate(rs_pix)))
    st = pt.stats()
    assert st["n_painted"] == sum(r[2]["n_painted"] for r in ref if r is not None)
    assert st["hp_updates"] == sum(r[2]["hp_updates"] for r in ref if r is not None)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_ensemble_matches_separate_cones(precision):
    recs, off = ensemble()
    tab = catalogs.table(nu=0.0)
    ref = oracle_cones(recs, tab)
    with painter(precision, len(CONES)) as pt:
        pt.paint_ensemble(np.concatenate(recs), off)
        check_cones(pt, recs, off, ref)
        # the whole-ensemble read-out is the cones' maps one after the other
        full = pt.healpix(0)
        assert full.size == len(CONES) * 12 * NSIDE * NSIDE
        assert np.array_equal(full[12 * NSIDE * NSIDE:2 * 12 * NSIDE * NSIDE], pt.healpix_cone(1, 0))


def test_ensemble_chunks_straddle_cones():
    """max_records of 1024 cuts the call into chunks that start and end inside cones."""
    recs, off = ensemble()
    ref = oracle_cones(recs, catalogs.table(nu=0.0))
    with painter("mixed", len(CONES), max_records=1024) as pt:
        pt.paint_ensemble(np.concatenate(recs), off)
        check_cones(pt, recs, off, ref)


def test_ensemble_device_records_and_reset():
    torch = pytest.importorskip("torch")
    recs, off = ensemble()
    ref = oracle_cones(recs, catalogs.table(nu=0.0))
    d = torch.from_numpy(np.concatenate(recs)).cuda()
    with painter("mixed", len(CONES)) as pt:
        pt.paint_ensemble(np.concatenate(recs), off)  # painted, then cleared by the reset
        pt.reset()
        pt.paint_ensemble_device(d.data_ptr(), off, 10)
        check_cones(pt, recs, off, ref)


def test_plain_records_go_to_cone_zero():
    recs, _ = ensemble()
    with painter("mixed", 3) as pt:
        pt.paint_records(recs[1])
        assert np.any(pt.healpix_cone(0, 0))
        assert not np.any(pt.healpix_cone(1, 0)) and not np.any(pt.healpix_cone(2, 0))


def test_ensemble_argument_checks():
    recs, off = ensemble()
    allrec = np.concatenate(recs)
    with pytest.raises(p2m.P2MError):
        p2m.Painter(nside=NSIDE, npix_fs=64, ncones=4)  # HEALPix only
    with pytest.raises(p2m.P2MError):
        p2m.Painter(nside=NSIDE, ncones=p2m.capi.MAXCONES + 1)
    with painter("mixed", 2) as pt:
        with pytest.raises(p2m.P2MError):  # more cones than the context holds
            pt.paint_ensemble(allrec, off)
        with pytest.raises(p2m.P2MError):  # decreasing offsets
            pt.paint_ensemble(allrec, np.array([0, 9000, 600, len(allrec)]))
        with pytest.raises(p2m.P2MError):
            pt.healpix_cone(2, 0)
        with pytest.raises(p2m.P2MError):
            pt.set_preprocess(scramble=1)
    with painter("mixed", 0) as pt:
        with pytest.raises(p2m.P2MError):  # not an ensemble context
            pt.paint_ensemble(allrec, off)
