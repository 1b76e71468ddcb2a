"""The shipped workloads at full size against the oracle, through the C ABI.

c2 (the headline): 1e7 records (seed 2, shell 100-8000 Mpc, masses 1e12-3e15 Msun/h),
HEALPix Nside 4096, tSZ y (nu = 0 table, profile 1) and kSZ (profile 2), zmax 6, the full
100 x 100 x 200 make_maptable table; the mixed and the plain FP64 paths against the
oracle's FP64 halo loop (pks2map.f90:276-303) on the same records and table image
(and the mixed decisions with FP64 or 64-bit fixed-point accumulation):
  - every (record, pixel) pair of every enumerated disc identical (FLAG_ALL_HALOS:
    also the discs whose table value is zero), ~4e7 pairs;
  - map values within 1e-5 relative wherever |v| > 1e-3 of the map's largest |v|;
  - map totals (integrated Y, net kSZ) within 1e-7 relative.
c4: six Nside 4096 maps (tSZ at 148/200/218/353/545 GHz, each from its own full-size
table, plus kSZ), 2e6 records of the multi-table catalogue (seed 4).
c5: the 64 light-cones of the ensemble form (seeds 5 and 5000 + i), every cone's Nside
1024 map against the oracle painting that cone alone.

The oracle runs on all host cores (orc_paint_parallel, identical to its serial loop)."""
import functools
import os

import numpy as np
import pytest

import matt_young_mapmaking_gb300 as p2m
import oracle

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5
MASK_FRAC = 1e-3
SUM_TOL = 1e-7
SHELL = (100.0, 8000.0)
MASS = (1e12, 3e15)
THREADS = os.cpu_count() or 1
SET_CAP = 1 << 26


@functools.lru_cache(maxsize=None)
def _table(model, nu):
    """the oracle's full-size make_maptable image (100 x 100 x 200)"""
    return oracle.make_maptable(model, nu, 0.0)


@pytest.fixture(scope="module")
def c2():
    rec = p2m.generate_catalogue(2, 10_000_000, 10, r=SHELL, m=MASS)
    tab = _table(1, 0.0)
    p = oracle.params(nside=4096, maps=((0, 1), (0, 2)), zmax=6.0, nfloat=10)
    hp, _, st, sets = oracle.paint(p, [oracle.Table(tab)], rec, record_sets=True,
                                   set_cap=SET_CAP, threads=THREADS)
    keys = _pair_keys(*sets)
    return rec, tab, hp, st, keys


def _pair_keys(srec, spix):
    """(record, pixel) pairs as sorted int64 keys record * 2^28 + pixel on the device
    (records < 2^24, pixels < 12 * 4096^2 < 2^28)"""
    import torch
    r = torch.from_numpy(np.ascontiguousarray(srec)).cuda()
    q = torch.from_numpy(np.ascontiguousarray(spix)).cuda()
    assert int(r.max()) < (1 << 24) and int(q.max()) < (1 << 28)
    return torch.sort(r * (1 << 28) + q).values


def compare_maps(gpu, ref, what):
    """per-pixel (masked) and total checks on the device; returns the measured errors"""
    import torch
    g = torch.as_tensor(np.ascontiguousarray(gpu)).cuda().double()
    r = torch.as_tensor(np.ascontiguousarray(ref)).cuda().double()
    mx = r.abs().max().item()
    assert mx > 0, what
    mask = r.abs() > MASK_FRAC * mx
    err = (g - r).abs()
    worst = (err[mask] / r[mask].abs()).max().item()
    outside = err[~mask].max().item() if (~mask).any() else 0.0
    s_g, s_r = g.sum().item(), r.sum().item()
    tot = abs(s_g - s_r) / abs(s_r)
    assert worst <= REL_TOL, "%s: max rel err %.3g" % (what, worst)
    assert outside <= REL_TOL * MASK_FRAC * mx, "%s: unmasked abs err %.3g" % (what, outside)
    assert tot <= SUM_TOL, "%s: total %.12g vs %.12g (rel %.3g)" % (what, s_g, s_r, tot)
    return worst, tot


@pytest.mark.parametrize("precision", ["mixed", "fp64", "mixed64", "fixed"])
def test_c2_headline_against_oracle(c2, precision, monkeypatch):
    rec, tab, rhp, rst, rkeys = c2
    monkeypatch.setenv("P2M_SET_CAP", str(SET_CAP))
    flags = p2m.FLAG_RECORD_SETS | p2m.FLAG_ALL_HALOS
    with p2m.Painter(nside=4096, precision=precision, maps=((0, 1), (0, 2)), zmax=6.0,
                     flags=flags, max_records=len(rec)) as pt:
        pt.load_table(0, tab)
        pt.paint_records(rec)
        hp = [pt.healpix(0), pt.healpix(1)]
        st = pt.stats()
        gkeys = _pair_keys(*pt.pixel_sets())
    assert st["n_painted"] == rst["n_painted"] > 1_000_000
    assert st["hp_updates"] == rst["hp_updates"] > 30_000_000
    assert gkeys.shape == rkeys.shape, "pixel-set sizes differ"
    assert bool((gkeys == rkeys).all()), "pixel sets differ in %d pairs" % int(
        (gkeys != rkeys).sum())
    for m, name in enumerate(("tSZ y", "kSZ")):
        compare_maps(hp[m], rhp[m], "%s %s" % (precision, name))
    if precision == "mixed":
        # the statistics of pks2map.f90:321-357 on the device over the 201M-pixel y map,
        # whose first P(<y) bin passes the reference's float counter limit of 2^24
        with p2m.Painter(nside=4096, precision=precision, maps=((0, 1), (0, 2)), zmax=6.0,
                         max_records=len(rec)) as pt:
            pt.load_table(0, tab)
            pt.paint_records(rec)
            mom, rms, dp = pt.map_stats(0)
            y = pt.healpix(0)
        rmom, rrms, rdp = oracle.map_stats(y)
        for k in range(3):
            assert abs(mom[k] - rmom[k]) <= 1e-10 * abs(rmom[k])
        assert abs(rms - rrms) <= 1e-10 * rrms
        assert np.array_equal(dp.view(np.uint32), rdp.view(np.uint32))
        assert dp[0] == np.float32(16777216.0) / np.float32(y.size)


def test_c2_gpu_table_is_the_oracle_table():
    """The table the bench paints with (make_maptable on the GPU) is the oracle's table
    image at the full 100 x 100 x 200 size, bit for bit."""
    gpu = p2m.make_maptable(1, 0.0, 0.0)
    ref = _table(1, 0.0)
    assert len(gpu) == len(ref) == 36 + 8 * 100 * 100 * 200
    g, r = p2m.table_array(gpu), p2m.table_array(ref)
    same = (g == r) | (np.isnan(g) & np.isnan(r))
    assert gpu[:36] == ref[:36]
    assert same.all(), "%d of %d entries differ" % ((~same).sum(), same.size)


def test_c4_six_tables_against_oracle():
    freqs = (148.0, 200.0, 218.0, 353.0, 545.0)
    maps = tuple((t, 1) for t in range(len(freqs))) + ((0, 2),)
    tabs = [_table(1, f) for f in freqs]
    rec = p2m.generate_catalogue(4, 2_000_000, 10, r=SHELL, m=MASS)
    p = oracle.params(nside=4096, maps=maps, zmax=6.0, nfloat=10)
    rhp, _, rst, rsets = oracle.paint(p, [oracle.Table(t) for t in tabs], rec,
                                      record_sets=True, set_cap=SET_CAP, threads=THREADS)
    rkeys = _pair_keys(*rsets)
    del rsets
    os.environ["P2M_SET_CAP"] = str(SET_CAP)
    try:
        with p2m.Painter(nside=4096, precision="mixed", maps=maps, zmax=6.0,
                         flags=p2m.FLAG_RECORD_SETS | p2m.FLAG_ALL_HALOS,
                         max_records=len(rec)) as pt:
            for t, tab in enumerate(tabs):
                pt.load_table(t, tab)
            pt.paint_records(rec)
            st = pt.stats()
            gkeys = _pair_keys(*pt.pixel_sets())
            assert st["hp_updates"] == rst["hp_updates"] > 5_000_000
            assert gkeys.shape == rkeys.shape and bool((gkeys == rkeys).all())
            names = ["tsz_%dghz" % f for f in freqs] + ["ksz"]
            for m in range(len(maps)):
                compare_maps(pt.healpix(m), rhp[m], "c4 " + names[m])
    finally:
        del os.environ["P2M_SET_CAP"]


def test_c5_every_cone_against_oracle():
    ncones, nside = 64, 1024
    rng = np.random.default_rng(5)
    counts = np.exp(rng.uniform(np.log(1e4), np.log(1e6), ncones)).astype(np.int64)
    depths = np.exp(rng.uniform(np.log(1000.0), np.log(6000.0), ncones))
    recs = [p2m.generate_catalogue(5000 + i, int(counts[i]), 10, r=(100.0, float(depths[i])),
                                   m=MASS) for i in range(ncones)]
    off = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    tab = _table(1, 0.0)
    with p2m.Painter(nside=nside, precision="mixed", maps=((0, 1),), zmax=6.0,
                     max_records=int(off[-1]), ncones=ncones) as pt:
        pt.load_table(0, tab)
        pt.paint_ensemble(np.concatenate(recs), off)
        allmaps = pt.healpix(0).reshape(ncones, -1)
    p = oracle.params(nside=nside, maps=((0, 1),), zmax=6.0, nfloat=10)
    otab = oracle.Table(tab)
    painted = 0
    for c in range(ncones):
        rhp, _, rst, _ = oracle.paint(p, [otab], recs[c], threads=THREADS)
        if rst["hp_updates"] == 0:
            assert not allmaps[c].any()
            continue
        painted += 1
        compare_maps(allmaps[c], rhp[0], "cone %d" % c)
    assert painted >= ncones // 2
