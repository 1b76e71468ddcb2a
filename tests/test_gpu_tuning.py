"""Launch parameters (p2m_set_tuning, p2m_autotune): results keep parity with the oracle
at the extremes of every parameter's range and after the autotuner's choice."""
import numpy as np
import pytest

import catalogs
import matt_young_mapmaking_gb300 as p2m
from test_gpu_parity import FLAGS, assert_maps_close, assert_sets_equal, run_oracle

pytestmark = pytest.mark.gpu

MAPS = ((0, 1), (0, 2))


def catalogue():
    """Discs from a few pixels to thousands of rings' worth: both painting paths busy."""
    return np.concatenate([catalogs.edge_cases(),
                           catalogs.shell(51, 30_000, r=(100.0, 8000.0), m=(1e12, 3e15))])


def painter(precision):
    pt = p2m.Painter(nside=512, precision=precision, maps=MAPS, zmax=6.0, flags=FLAGS,
                     max_records=1 << 16)
    pt.load_table(0, catalogs.table(nu=0.0))
    return pt


def check(pt, rec, ref):
    pt.paint_records(rec)
    rhp, _, rst, rsets = ref
    assert_sets_equal(pt.pixel_sets(), rsets)
    for m in range(2):
        assert_maps_close(pt.healpix(m), rhp[m], what="map %d" % m)
    assert pt.stats()["hp_updates"] == rst["hp_updates"]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("tune", [dict(big_rings=0, halos_grid=1, full_grid=1, full_chunk=32),
                                  dict(big_rings=16, halos_grid=2, full_grid=3, full_chunk=100),
                                  dict(big_rings=4096, halos_grid=16, full_grid=32,
                                       full_chunk=65536),
                                  dict(sort_halos=0, halo_batch=32),
                                  dict(sort_halos=1, halo_batch=8),
                                  dict(sort_halos=1, halo_batch=1, big_rings=32),
                                  dict(halos_threads=256, halos_grid=4),
                                  dict(halos_threads=256, halos_grid=1, halo_batch=32)])
def test_tuning_extremes_keep_parity(precision, tune):
    rec = catalogue()
    ref = run_oracle(rec, [catalogs.table(nu=0.0)], 512, maps=MAPS, zmax=6.0)
    with painter(precision) as pt:
        pt.set_tuning(**tune)
        got = pt.tuning()
        assert all(got[k] == v for k, v in tune.items())
        check(pt, rec, ref)


def test_autotune_choice_and_parity():
    torch = pytest.importorskip("torch")
    rec = catalogue()
    ref = run_oracle(rec, [catalogs.table(nu=0.0)], 512, maps=MAPS, zmax=6.0)
    d = torch.from_numpy(rec).cuda()
    with painter("mixed") as pt:
        t = pt.autotune(d.data_ptr(), len(rec), 10, reps=2)
        assert t["big_rings"] in (0, 16, 32, 48, 64, 96, 128, 256)
        assert t["halos_grid"] in (2, 4, 6, 8, 16) and t["full_grid"] in (2, 4, 8, 16)
        assert t["full_chunk"] in (256, 512, 1024, 2048, 4096) and t["ms"] > 0
        assert t["sort_halos"] in (0, 1) and t["halo_batch"] in (8, 16, 32)
        assert t["halos_threads"] in (128, 256)
        assert pt.tuning()["big_rings"] == t["big_rings"]
        assert not np.any(pt.healpix(0))  # the autotuner leaves the maps reset
        check(pt, rec, ref)


def test_tuning_rejects_out_of_range():
    with painter("mixed") as pt:
        for bad in (dict(big_rings=-1), dict(halos_grid=0), dict(full_grid=33),
                    dict(full_chunk=16), dict(halos_threads=192), dict(halos_threads=512)):
            with pytest.raises(p2m.P2MError):
                pt.set_tuning(**bad)
