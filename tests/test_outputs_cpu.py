"""Output files of the pks2map command line (host code, no GPU): the P(<y) histogram
against a numpy restatement of pks2map.f90:340-357, the three files read back, and the
command-line usage messages."""
import os
import subprocess

import numpy as np
import pytest

import matt_young_mapmaking_gb300 as p2m

PKG = os.path.dirname(p2m.__file__)


def dpdy_restated(m):
    """pks2map.f90:340-357 in numpy: bin int(y / dy) + 1 with dy = 1e-4 / 1e4 in float,
    counts kept as float (a bin stops at 2^24), normalised by npix, cumulated in float."""
    m = np.asarray(m, dtype=np.float32)
    dy = np.float32(np.float32(1e-4) / np.float32(10000))
    q = m / dy
    ok = (q > -1) & (q < 10000)
    k = np.trunc(q[ok]).astype(np.int64) + 1
    cnt = np.bincount(k, minlength=10001)[1:10001]
    d = np.minimum(cnt, 2 ** 24).astype(np.float32) / np.float32(m.size)
    return np.cumsum(d, dtype=np.float32)


def test_dpdy_matches_restatement():
    rng = np.random.default_rng(5)
    m = np.concatenate([rng.exponential(2e-6, 300_000), -rng.exponential(1e-8, 1000),
                        np.zeros(50_000), [1.0, -1.0, 9.9999e-5, 1e-4]]).astype(np.float32)
    assert np.array_equal(p2m.dpdy(m), dpdy_restated(m))


def test_dpdy_bin_saturates_like_float_counts():
    # more than 2^24 equal values in one bin: float counting stops at 2^24
    m = np.zeros(2 ** 24 + 1000, dtype=np.float32)
    d = p2m.dpdy(m)
    assert d[0] == np.float32(np.float32(2 ** 24) / np.float32(m.size))


def test_output_files_read_back(tmp_path):
    nside, npix = 32, 24
    rng = np.random.default_rng(6)
    hp = rng.normal(size=12 * nside * nside).astype(np.float32) * 1e-5
    fs = rng.normal(size=(npix, npix)).astype(np.float32)
    base = str(tmp_path / "out")
    p2m.write_outputs(base, hp_map=hp, nside=nside, fs_map=fs, npix_fs=npix, fov_rad=0.1745)
    cards, back = p2m.read_healpix_fits(base + "_hp.fits")
    assert cards["TFORM1"] == "1024E" and cards["ORDERING"] == "RING"
    assert int(cards["NSIDE"]) == nside and np.array_equal(back, hp)
    assert os.path.getsize(base + "_hp.fits") % 2880 == 0
    fov, fs_back = p2m.read_flatsky(base + "_fs.map")
    assert np.float32(fov) == np.float32(0.1745) and np.array_equal(fs_back, fs)
    mx, d = p2m.read_dpdy(base + "_dp.bin")
    assert mx == np.float32(1e-4) and np.array_equal(d, dpdy_restated(hp))


def test_small_healpix_fits_uses_single_value_rows(tmp_path):
    hp = np.arange(12 * 4 * 4, dtype=np.float32)  # npix < 1024: rows of one value
    p2m.write_outputs(str(tmp_path / "s"), hp_map=hp, nside=4)
    cards, back = p2m.read_healpix_fits(str(tmp_path / "s_hp.fits"))
    assert cards["TFORM1"] == "1E" and int(cards["NAXIS2"]) == hp.size
    assert np.array_equal(back, hp)


@pytest.mark.parametrize("exe,usage", [
    ("pks2map", "Usage: pks2map <filein> <fileout> <tablefile>"),
    ("make_maptable", "Usage: make_maptable <fileout> <model>")])
def test_command_line_usage(exe, usage):
    path = os.path.join(PKG, exe)
    if not os.path.exists(path):
        pytest.skip("command line not built")
    r = subprocess.run([path], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.startswith(usage)
