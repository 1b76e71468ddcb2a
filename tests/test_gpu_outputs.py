"""Map statistics on the device (p2m_get_healpix_stats / p2m_get_flatsky_stats) against the
oracle's restatement of pks2map.f90:321-357 over the same read-out maps, through the C ABI:
moments and RMS to FP64 summation-order rounding, the cumulative P(<y) bit for bit (the
bins are integer counts in the reference's float sequence)."""
import numpy as np
import pytest

import catalogs
import matt_young_mapmaking_gb300 as p2m
import oracle

pytestmark = pytest.mark.gpu

MOM_REL = 1e-11


def check_stats(got, ref, what):
    mom, rms, dp = got
    rmom, rrms, rdp = ref
    for k in range(3):
        assert abs(mom[k] - rmom[k]) <= MOM_REL * abs(rmom[k]) + 1e-300, (what, k, mom[k], rmom[k])
    assert abs(rms - rrms) <= MOM_REL * abs(rrms), (what, rms, rrms)
    if rdp is not None:
        assert dp is not None and np.array_equal(dp.view(np.uint32), rdp.view(np.uint32)), what


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_map_stats_match_oracle(precision):
    rec = catalogs.cone(3, 30_000, (1.0, 0.0, 0.0), 8.0)
    tab = catalogs.table(nu=0.0)
    with p2m.Painter(nside=512, npix_fs=512, fov_deg=10.0, precision=precision,
                     maps=((0, 1), (0, 2)), max_records=len(rec)) as pt:
        pt.load_table(0, tab)
        pt.paint_records(rec)
        for m in range(2):
            hp = pt.healpix(m)
            fs = pt.flatsky(m)
            assert np.abs(hp).max() > 0 and np.abs(fs).max() > 0
            check_stats(pt.map_stats(m), oracle.map_stats(hp), "healpix map %d" % m)
            check_stats(pt.map_stats(m, flatsky=True), oracle.map_stats(fs, dpdy=False),
                        "flat sky map %d" % m)
            # the library's host P(<y) on the same map agrees too
            assert np.array_equal(p2m.dpdy(hp).view(np.uint32), pt.map_stats(m)[2].view(np.uint32))
        # y values spread over many bins, and bin 1 holds the empty sky
        dp = pt.map_stats(0)[2]
        assert 0.5 < dp[0] < 1.0 and np.count_nonzero(np.diff(dp)) > 20


def _mask_date(b):
    i = b.find(b"DATE    = ")
    return b[:i] + b[i + 80:] if i >= 0 else b


@pytest.mark.parametrize("nside", [1, 64, 2048])
def test_device_fits_writer_equals_host_writer(nside, tmp_path):
    """p2m_write_healpix_fits_device (big-endian conversion on the device, copies in
    slices overlapping the file write; 2048 is 3 slices) writes the bytes of the host
    writer p2m_write_healpix_fits on the map a read-out delivers."""
    rec = catalogs.shell(41, 20_000, r=(100.0, 3000.0))
    with p2m.Painter(nside=nside, precision="mixed", max_records=len(rec)) as pt:
        pt.load_table(0, catalogs.table())
        pt.paint_records(rec)
        hp = pt.healpix(0)
        pt.write_healpix_fits(0, tmp_path / "dev.fits")
    p2m.write_outputs(str(tmp_path / "host"), hp_map=hp, nside=nside)
    dev = (tmp_path / "dev.fits").read_bytes()
    host = (tmp_path / "host_hp.fits").read_bytes()
    assert len(dev) == len(host) and len(dev) % 2880 == 0
    assert _mask_date(dev) == _mask_date(host)
    # the data part holds the map, big-endian
    data = np.frombuffer(dev[-(((4 * hp.size + 2879) // 2880) * 2880):][:4 * hp.size], dtype=">f4")
    assert np.array_equal(data.astype(np.float32), hp)
