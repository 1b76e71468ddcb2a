"""The pks2map command line on the GPU: its three output files against the C ABI painter
and the oracle, for both catalogue layouts (10 floats after a 3-word header, 7 after a
2-word header)."""
import os
import subprocess

import numpy as np
import pytest

import catalogs
import matt_young_mapmaking_gb300 as p2m
import oracle

pytestmark = pytest.mark.gpu

PKG = os.path.dirname(p2m.__file__)


def masked_rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    mx = np.abs(b).max()
    m = np.abs(b) > 1e-3 * mx
    return (np.abs(a[m] - b[m]) / np.abs(b[m])).max()


def fe3(v):
    """Fortran 1pe9.3 / 1pe10.3 of the report lines"""
    return "%.3E" % v


@pytest.mark.parametrize("nfloat,profile,scramble,centre,n", [(10, 1, 0, 0, 30_000),
                                                               (7, 2, 0, 0, 30_000),
                                                               (10, 1, 1, 1, 30_000),
                                                               (10, 1, 0, 0, 4_500_000)])
def test_pks2map_command_line(tmp_path, nfloat, profile, scramble, centre, n):
    """n = 4.5e6: the catalogue is read and painted in two steps of up to 4M records"""
    exe = os.path.join(PKG, "pks2map")
    rec = (catalogs.shell(41, n, nfloat=nfloat) if n <= 100_000 else
           p2m.generate_catalogue(41, n, nfloat, r=(100.0, 3000.0), m=(1e12, 1e15)))
    cat = str(tmp_path / "halos.pksc")
    p2m.write_pksc(cat, rec)
    tab = catalogs.table()
    tabfile = str(tmp_path / "table.bin")
    p2m.write_table(tabfile, tab)
    out = str(tmp_path / "map")
    nside, npix, fov, zmax = 256, 64, 10.0, 1.25
    args = [exe, cat, out, tabfile, "0.0", str(nside), str(scramble), str(centre), str(npix), str(fov),
            str(zmax), "0.0", "1", str(profile)]
    r = subprocess.run(args, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    cards, hp = p2m.read_healpix_fits(out + "_hp.fits")
    assert int(cards["NSIDE"]) == nside and hp.size == 12 * nside * nside
    fov_rad, fs = p2m.read_flatsky(out + "_fs.map")
    _, dp = p2m.read_dpdy(out + "_dp.bin")
    assert np.array_equal(dp, p2m.dpdy(hp))

    # the same painting through the C ABI
    with p2m.Painter(nside=nside, npix_fs=npix, fov_deg=fov, zmax=zmax, maps=((0, profile),),
                     max_records=len(rec)) as pt:
        pt.set_preprocess(scramble, centre, 1)
        pt.load_table(0, tab)
        pt.paint_records(rec)
        api_hp, api_fs, st = pt.healpix(0), pt.flatsky(0), pt.stats()
    assert masked_rel(hp, api_hp) <= 1e-6
    assert masked_rel(fs.ravel(), api_fs) <= 1e-6
    assert "Number of halos in map:    %d" % st["n_painted"] in r.stdout

    # and against the oracle
    p = oracle.params(nside=nside, npix_fs=npix, fov_deg=fov, zmax=zmax, maps=((0, profile),),
                      nfloat=nfloat, scramble=scramble, centre=centre)
    ohp, ofs, ost, _ = oracle.paint(p, [oracle.Table(tab)], rec, threads=os.cpu_count() or 1)
    assert masked_rel(hp, ohp[0]) <= 1e-5
    assert masked_rel(fs.ravel(), ofs[0]) <= 1e-6
    assert ost["n_painted"] == st["n_painted"]
    assert ("After rotation largest halo is at" in r.stdout) == bool(centre)

    # the report's moments and RMS (computed on the device) and the P(<y) file against
    # the oracle's restatement of pks2map.f90:321-357 over the written maps
    hmom, hrms, hdp = oracle.map_stats(hp)
    fmom, frms, _ = oracle.map_stats(fs.ravel(), dpdy=False)
    assert np.array_equal(dp.view(np.uint32), hdp.view(np.uint32))
    assert "Flatsky moments:    %s %s %s \n" % tuple(fe3(v) for v in fmom) in r.stdout
    assert "Healpix moments:    %s %s %s \n" % tuple(fe3(v) for v in hmom) in r.stdout
    assert "Healpix RMS:                %s\n" % fe3(hrms) in r.stdout
    assert "Flatsky RMS:                %s\n" % fe3(frms) in r.stdout
