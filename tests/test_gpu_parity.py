"""GPU painter vs the oracle (same seeded inputs): per-halo pixel sets bit-exact, map
values within 1e-5 relative wherever |value| > 1e-3 of the map maximum, map totals within
1e-7 relative.  All calls go through the C ABI."""
import ctypes

import numpy as np
import pytest

import catalogs
import matt_young_mapmaking_gb300 as p2m
import oracle

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5       # per pixel, where |v| > MASK_FRAC * max|v|
MASK_FRAC = 1e-3
SUM_TOL = 1e-7       # map totals, relative to the oracle's net sum (signed for kSZ)
FLAGS = p2m.FLAG_RECORD_SETS | p2m.FLAG_ALL_HALOS
PRECISIONS = ["fp64", "mixed", "mixed64", "fixed"]


def run_gpu(records, tables, precision, nside, npix_fs=0, maps=((0, 1),), flags=FLAGS,
            **kw):
    with p2m.Painter(nside=nside, npix_fs=npix_fs, precision=precision, maps=maps,
                     flags=flags, max_records=max(len(records), 1024), **kw) as pt:
        for i, t in enumerate(tables):
            pt.load_table(i, t)
        pt.paint_records(records)
        hp = np.stack([pt.healpix(m) for m in range(len(maps))]) if nside else None
        fs = np.stack([pt.flatsky(m) for m in range(len(maps))]) if npix_fs else None
        st = pt.stats()
        sets = pt.pixel_sets() if flags & p2m.FLAG_RECORD_SETS else None
    return hp, fs, st, sets


def run_oracle(records, tables, nside, npix_fs=0, maps=((0, 1),), **kw):
    p = oracle.params(nside=nside, npix_fs=npix_fs, maps=maps, nfloat=records.shape[1], **kw)
    tabs = [oracle.Table(t) for t in tables]
    return oracle.paint(p, tabs, records, record_sets=nside > 0)


def assert_maps_close(gpu, ref, rel=REL_TOL, what="map", sum_tol=SUM_TOL):
    ref = np.asarray(ref, dtype=np.float64)
    gpu = np.asarray(gpu, dtype=np.float64)
    mx = np.abs(ref).max()
    if mx == 0:
        assert np.abs(gpu).max() == 0, what
        return
    mask = np.abs(ref) > MASK_FRAC * mx
    err = np.abs(gpu - ref)
    worst = (err[mask] / np.abs(ref[mask])).max()
    assert worst <= rel, "%s: max rel err %.3g over %d masked pixels" % (what, worst, mask.sum())
    assert err[~mask].max(initial=0.0) <= rel * MASK_FRAC * mx, what
    # the total (integrated Y; the net kSZ sum, positive and negative halos cancelling)
    # relative to the oracle's own net total
    s_ref, s_gpu = ref.sum(), gpu.sum()
    assert abs(s_gpu - s_ref) <= sum_tol * abs(s_ref), \
        "%s: total %.10g vs %.10g (rel %.3g, sum|v| %.6g)" % (
            what, s_gpu, s_ref, abs(s_gpu - s_ref) / abs(s_ref), np.abs(ref).sum())


def assert_sets_equal(gpu_sets, ref_sets):
    g = np.stack(gpu_sets, axis=1)
    r = np.stack(ref_sets, axis=1)
    g = g[np.lexsort((g[:, 1], g[:, 0]))]
    r = r[np.lexsort((r[:, 1], r[:, 0]))]
    assert g.shape == r.shape, "pixel-set sizes differ: gpu %d, oracle %d" % (len(g), len(r))
    assert np.array_equal(g, r), "pixel sets differ in %d entries" % (g != r).any(axis=1).sum()


@pytest.mark.parametrize("precision", PRECISIONS)
def test_config1_tsz_nside512(precision):
    """1e5-halo catalogue, shell 100-3000 Mpc, HEALPix Nside 512, 148 GHz table."""
    rec = catalogs.shell(1, 100_000)
    tab = catalogs.table()
    hp, _, st, sets = run_gpu(rec, [tab], precision, 512)
    rhp, _, rst, rsets = run_oracle(rec, [tab], 512)
    assert_sets_equal(sets, rsets)
    assert st["hp_updates"] == rst["hp_updates"]
    assert st["n_painted"] == rst["n_painted"]
    assert_maps_close(hp[0], rhp[0], rel=1e-6 if precision == "fp64" else REL_TOL)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_tsz_ksz_two_maps_wide_shell(precision):
    """tSZ y (nu = 0) and kSZ from one table, 100-8000 Mpc shell, zmax = 6, Nside 1024."""
    rec = catalogs.shell(2, 40_000, r=(100.0, 8000.0), m=(1e12, 3e15))
    tab = catalogs.table(nu=0.0)
    maps = ((0, 1), (0, 2))
    hp, _, st, sets = run_gpu(rec, [tab], precision, 1024, maps=maps, zmax=6.0)
    rhp, _, rst, rsets = run_oracle(rec, [tab], 1024, maps=maps, zmax=6.0)
    assert_sets_equal(sets, rsets)
    for m in range(2):
        assert_maps_close(hp[m], rhp[m], what="map %d" % m)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_flatsky_and_healpix(precision):
    """Flat-sky 256^2 over 10 deg with halos concentrated in the field, plus HEALPix."""
    rec = catalogs.cone(3, 30_000, (1.0, 0.0, 0.0), 8.0)
    tab = catalogs.table()
    hp, fs, st, sets = run_gpu(rec, [tab], precision, 256, npix_fs=256, fov_deg=10.0)
    rhp, rfs, rst, rsets = run_oracle(rec, [tab], 256, npix_fs=256, fov_deg=10.0)
    assert st["fs_updates"] == rst["fs_updates"] > 0
    assert_sets_equal(sets, rsets)
    # every flat-sky operation is the reference's float sequence: exact up to the
    # order of accumulation
    assert_maps_close(fs[0], rfs[0], rel=1e-6, what="flat sky")
    assert_maps_close(hp[0], rhp[0], what="healpix")


@pytest.mark.parametrize("precision", PRECISIONS)
def test_edge_cases(precision):
    """Poles, phi = 0, cap boundary, very large discs, the radial cut."""
    rec = catalogs.edge_cases()
    tab = catalogs.table()
    maps = ((0, 1), (0, 2))
    hp, _, st, sets = run_gpu(rec, [tab], precision, 128, maps=maps)
    rhp, _, rst, rsets = run_oracle(rec, [tab], 128, maps=maps)
    assert_sets_equal(sets, rsets)
    assert st["n_painted"] == rst["n_painted"]
    for m in range(2):
        assert_maps_close(hp[m], rhp[m], what="map %d" % m)


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("big_rings", ["0", "1000000"])
def test_stored_item_and_fused_paths(precision, big_rings, monkeypatch):
    """Every halo through the stored-item path (threshold 0 rings) or through the fused
    enumerate-and-paint path (threshold above any ring count): the same pixel sets and
    maps as the oracle either way."""
    monkeypatch.setenv("P2M_BIG_RINGS", big_rings)
    rec = np.concatenate([catalogs.edge_cases(), catalogs.shell(21, 20_000, r=(100.0, 8000.0),
                                                                 m=(1e12, 3e15))])
    tab = catalogs.table(nu=0.0)
    maps = ((0, 1), (0, 2))
    hp, _, st, sets = run_gpu(rec, [tab], precision, 256, maps=maps, zmax=6.0)
    rhp, _, rst, rsets = run_oracle(rec, [tab], 256, maps=maps, zmax=6.0)
    assert_sets_equal(sets, rsets)
    assert st["hp_updates"] == rst["hp_updates"]
    for m in range(2):
        assert_maps_close(hp[m], rhp[m], what="map %d" % m)


@pytest.mark.parametrize("precision", ["fp64", "mixed", "fixed"])
@pytest.mark.parametrize("nside", [1, 2, 4, 8, 16])
def test_small_nside(nside, precision):
    """The smallest maps: three to 63 rings, rings of 4 pixels at the poles.  Halos 15-80
    Mpc away have discs of tens of degrees, so that even at Nside 1 some pixel centres
    fall inside."""
    rec = np.concatenate([catalogs.edge_cases(),
                          catalogs.shell(29, 3000, r=(15.0, 80.0), m=(1e13, 3e15)),
                          catalogs.shell(30, 2000)])
    tab = catalogs.table()
    maps = ((0, 1), (0, 2))
    hp, _, st, sets = run_gpu(rec, [tab], precision, nside, maps=maps)
    rhp, _, rst, rsets = run_oracle(rec, [tab], nside, maps=maps)
    assert_sets_equal(sets, rsets)
    assert st["hp_updates"] == rst["hp_updates"] > 0
    for m in range(2):
        assert_maps_close(hp[m], rhp[m], what="map %d" % m)


@pytest.mark.parametrize("scramble,centre,ntasks", [(1, 0, 1), (0, 1, 1), (1, 1, 1), (1, 1, 3)])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_scramble_and_centre(scramble, centre, ntasks, precision):
    """pks2map's scramble (the reference's ranf stream per rank, jumped ahead on the GPU)
    and center (flips and rotations about the largest halo): pixel sets bit-exact against
    the oracle, which runs the generator sequentially."""
    rec = catalogs.shell(23, 20_000)
    tab = catalogs.table()
    maps = ((0, 1), (0, 2))
    with p2m.Painter(nside=256, precision=precision, maps=maps, flags=FLAGS,
                     max_records=len(rec)) as pt:
        pt.set_preprocess(scramble, centre, ntasks)
        pt.load_table(0, tab)
        pt.paint_records(rec)
        hp = np.stack([pt.healpix(m) for m in range(2)])
        st, sets, info = pt.stats(), pt.pixel_sets(), pt.centre_info()
    p = oracle.params(nside=256, maps=maps, nfloat=10, scramble=scramble, centre=centre,
                      ntasks=ntasks)
    rhp, _, rst, rsets = oracle.paint(p, [oracle.Table(tab)], rec, record_sets=True)
    assert_sets_equal(sets, rsets)
    assert st["n_painted"] == rst["n_painted"]
    for m in range(2):
        assert_maps_close(hp[m], rhp[m], what="map %d" % m)
    if centre:
        assert np.array_equal(info, np.array(rst["centre"], dtype=np.float32))


def test_preprocess_needs_one_call():
    rec = catalogs.shell(24, 4000)
    with p2m.Painter(nside=64, max_records=2000) as pt:
        pt.set_preprocess(1, 0, 1)
        pt.load_table(0, catalogs.table())
        with pytest.raises(p2m.P2MError) as e:
            pt.paint_records(rec)  # two chunks of 2000 records
        assert e.value.status == p2m.capi.P2M_ERR_CAPACITY
        # refused before anything was painted: the context paints the first half as usual
        assert pt.stats()["n_records"] == 0
        pt.paint_records(rec[:2000])
        assert pt.stats()["n_records"] == 2000


def too_close_catalogue():
    """A shell catalogue whose first halo sits 15 Mpc from the observer with
    R_TH = 120 Mpc: 4 asin(r / chi) = 3.47 > pi, where query_disc aborts."""
    rec = catalogs.shell(27, 2000).copy()
    rec[0, :3] = [0.0, 0.0, 15.0]
    rec[0, 6] = 120.0
    rec[0, 7:10] = rec[0, :3]
    return rec


@pytest.mark.parametrize("precision", PRECISIONS)
def test_disc_beyond_pi_is_an_error_and_the_context_survives(precision):
    """The set-up kernel raises a device flag for a disc radius above pi (the oracle's
    query_disc refuses it too); the C ABI reports it as an error of the call, which
    paints none of its records, and the same context then paints a good catalogue like
    the oracle, without a reset (the failed call's halos left the painting-order counts)
    and after one."""
    bad = too_close_catalogue()
    p = oracle.params(nside=128, maps=((0, 1),), nfloat=10)
    with pytest.raises(RuntimeError):
        oracle.paint(p, [oracle.Table(catalogs.table())], bad)
    good = bad[1:]
    with p2m.Painter(nside=128, precision=precision, flags=FLAGS,
                     max_records=len(bad)) as pt:
        pt.load_table(0, catalogs.table())
        with pytest.raises(p2m.P2MError, match="radius"):
            pt.paint_records(bad)
        pt.synchronize()  # the flag was reported once and cleared
        pt.paint_records(good)
        hp = [pt.healpix(0)]
        sets = [pt.pixel_sets()]
        with pytest.raises(p2m.P2MError, match="radius"):
            pt.paint_records(bad)
        pt.reset()
        pt.paint_records(good)
        hp.append(pt.healpix(0))
        sets.append(pt.pixel_sets())
    rhp, _, _, rsets = oracle.paint(p, [oracle.Table(catalogs.table())], good,
                                    record_sets=True)
    for k in range(2):
        assert_sets_equal(sets[k], rsets)
        assert_maps_close(hp[k], rhp[0])


@pytest.mark.parametrize("precision", PRECISIONS)
def test_six_maps_five_tables(precision):
    """The multi-table form: tSZ at 148, 200, 218, 353 and 545 GHz, each from its own
    table, plus kSZ, painted in one enumeration."""
    rec = catalogs.shell(25, 20_000, r=(100.0, 3000.0), m=(1e12, 1e15))
    tabs = [catalogs.table(nu=nu) for nu in (148.0, 200.0, 218.0, 353.0, 545.0)]
    maps = tuple((t, 1) for t in range(5)) + ((0, 2),)
    hp, _, st, sets = run_gpu(rec, tabs, precision, 256, maps=maps)
    rhp, _, rst, rsets = run_oracle(rec, tabs, 256, maps=maps)
    assert_sets_equal(sets, rsets)
    for m in range(6):
        assert_maps_close(hp[m], rhp[m], what="map %d" % m)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_eight_maps_eight_tables(precision):
    """The most maps and tables a context holds: tSZ at seven frequencies from seven
    tables and kSZ from an eighth, with flat sky as well."""
    rec = catalogs.cone(31, 15_000, (1.0, 0.0, 0.0), 8.0)
    tabs = [catalogs.table(nu=nu) for nu in (100.0, 143.0, 148.0, 200.0, 218.0, 353.0, 545.0, 0.0)]
    maps = tuple((t, 1) for t in range(7)) + ((7, 2),)
    hp, fs, st, sets = run_gpu(rec, tabs, precision, 128, npix_fs=128, fov_deg=10.0, maps=maps)
    rhp, rfs, rst, rsets = run_oracle(rec, tabs, 128, npix_fs=128, fov_deg=10.0, maps=maps)
    assert_sets_equal(sets, rsets)
    for m in range(8):
        assert_maps_close(hp[m], rhp[m], what="map %d" % m)
        assert_maps_close(fs[m], rfs[m], rel=1e-6, what="flat sky %d" % m)


MAP_SETS = {
    "lone_ksz": ((0, 2),),
    "ksz_then_tsz": ((0, 2), (0, 1)),
    "same_map_twice": ((0, 1), (0, 1)),
    "three_maps": ((0, 1), (1, 2), (1, 1)),
    "three_maps_lone_ksz": ((1, 2), (0, 1), (0, 2)),
}


@pytest.mark.parametrize("precision", ["fp64", "mixed", "fixed"])
@pytest.mark.parametrize("name", list(MAP_SETS))
def test_map_sets_through_pair_tables(name, precision):
    """Map sets whose pairs are not profiles 1 and 2 of one table read gathered pair
    tables (a lone kSZ map, swapped profiles, a map repeated, an odd last map); every map
    must equal the oracle's painting of that (table, profile)."""
    maps = MAP_SETS[name]
    rec = catalogs.shell(27, 20_000, r=(100.0, 3000.0), m=(1e12, 3e15))
    tabs = [catalogs.table(nu=0.0), catalogs.table(nu=148.0)]
    hp, _, st, sets = run_gpu(rec, tabs, precision, 1024, maps=maps)
    rhp, _, rst, rsets = run_oracle(rec, tabs, 1024, maps=maps)
    assert_sets_equal(sets, rsets)
    for m in range(len(maps)):
        assert_maps_close(hp[m], rhp[m], what="%s map %d" % (name, m))


def test_large_flatsky_field():
    """A 1024^2 flat-sky map over 10 degrees (the flat-sky form at reduced side)."""
    rec = catalogs.cone(26, 40_000, (1.0, 0.0, 0.0), 8.0)
    tab = catalogs.table()
    _, fs, st, _ = run_gpu(rec, [tab], "mixed", 0, npix_fs=1024, fov_deg=10.0, flags=0)
    _, rfs, rst, _ = run_oracle(rec, [tab], 0, npix_fs=1024, fov_deg=10.0)
    assert st["fs_updates"] == rst["fs_updates"] > 0
    assert_maps_close(fs[0], rfs[0], rel=1e-6, what="flat sky")


@pytest.mark.parametrize("precision", PRECISIONS)
def test_reset_discards_streamed_unread_paint(precision):
    """A call streamed in chunks paints each chunk as it arrives; a reset before any
    read-out must discard those contributions."""
    a = catalogs.shell(27, 6000)
    b = catalogs.shell(28, 5000)
    tab = catalogs.table()
    with p2m.Painter(nside=128, precision=precision, maps=((0, 1),), flags=FLAGS,
                     max_records=1024) as pt:
        pt.load_table(0, tab)
        pt.paint_records(a)  # six chunks, painted one by one, never read
        pt.reset()
        pt.paint_records(b)
        hp, st, sets = pt.healpix(0), pt.stats(), pt.pixel_sets()
    rhp, _, rst, rsets = run_oracle(b, [tab], 128)
    assert_sets_equal(sets, rsets)
    assert st["hp_updates"] == rst["hp_updates"]
    assert_maps_close(hp, rhp[0])


def test_reset_clears_every_painted_tile():
    """A reset clears everything painted before it.  Catalogues on opposite sides of the
    sky and a full-sky one are painted in turn, with resets, read-outs between paints
    and a bound buffer that starts out holding garbage; every read-out equals the
    oracle's map of what was painted since the last reset."""
    torch = pytest.importorskip("torch")
    a = catalogs.cone(63, 20_000, (1.0, 0.0, 0.0), 30.0)
    b = catalogs.cone(64, 20_000, (-1.0, 0.0, 0.0), 30.0)
    c = catalogs.shell(65, 10_000)
    tab = catalogs.table()
    ra, rb, rc = (run_oracle(r, [tab], 256)[0][0] for r in (a, b, c))
    assert np.abs(ra).max() > 0 and np.abs(rb).max() > 0
    assert not np.any((ra != 0) & (rb != 0))  # disjoint skies
    npix = 12 * 256 * 256
    with p2m.Painter(nside=256, precision="mixed", max_records=1 << 16) as pt:
        pt.load_table(0, tab)
        for rec, ref in ((a, ra), (b, rb), (c, rc), (a, ra), (b, rb)):
            pt.reset()
            pt.paint_records(rec)
            assert_maps_close(pt.healpix(0), ref)
        pt.reset()
        pt.paint_records(a)
        assert_maps_close(pt.healpix(0), ra)
        pt.paint_records(b)  # more painting after a read-out, then a reset
        assert_maps_close(pt.healpix(0), ra + rb)
        pt.reset()
        pt.paint_records(c)
        assert_maps_close(pt.healpix(0), rc)
        dev = torch.full((npix,), 7.0, dtype=torch.float32, device="cuda")
        for k, (rec, ref) in enumerate(((a, ra), (b, rb), (a, ra))):
            pt.reset()
            if k == 0:
                pt.bind_healpix_device(0, dev.data_ptr())
            pt.paint_records(rec)
            pt.healpix_device(0, dev.data_ptr())
            pt.synchronize()
            assert_maps_close(dev.cpu().numpy(), ref)


@pytest.mark.parametrize("model", [1, 2, 3])
def test_profile_models_and_redshift_cuts(model):
    """Each pressure-profile model (its overdensity enters the per-halo mass conversion,
    pks2map.f90:293) with both redshift cuts active."""
    rec = catalogs.shell(29 + model, 20_000, r=(100.0, 6000.0), m=(1e12, 3e15))
    tab = catalogs.table(model=model, nu=0.0)
    maps = ((0, 1), (0, 2))
    kw = dict(model=model, zmin=0.05, zmax=1.5)
    hp, _, st, sets = run_gpu(rec, [tab], "mixed", 1024, maps=maps, **kw)
    rhp, _, rst, rsets = run_oracle(rec, [tab], 1024, maps=maps, **kw)
    assert st["n_shell"] == rst["n_cut"] and st["n_painted"] == rst["n_painted"]
    assert st["hp_updates"] == rst["hp_updates"] > 1000
    assert 0 < st["n_shell"] < len(rec)
    assert_sets_equal(sets, rsets)
    for m in range(2):
        assert_maps_close(hp[m], rhp[m], what="model %d map %d" % (model, m))


def test_fixed_point_maps_are_bit_identical():
    """P2M_PREC_FIXED: the same maps, bit for bit, from repeated runs and from launch
    parameters that route every halo through the other painting kernel (the atomics land
    in a different order each time), HEALPix and flat sky; and within tolerance of FP64."""
    rec = np.concatenate([catalogs.edge_cases(),
                          catalogs.cone(33, 20_000, (1.0, 0.0, 0.0), 8.0, r=(100.0, 3000.0))])
    tab = catalogs.table(nu=0.0)
    maps = ((0, 1), (0, 2))
    runs = []
    for tune in (None, None, dict(big_rings=0, full_grid=3, full_chunk=96),
                 dict(big_rings=4096, halos_grid=1)):
        with p2m.Painter(nside=256, npix_fs=256, fov_deg=10.0, precision="fixed", maps=maps,
                         max_records=len(rec)) as pt:
            if tune:
                pt.set_tuning(**tune)
            pt.load_table(0, tab)
            pt.paint_records(rec)
            runs.append([pt.healpix(m) for m in range(2)] + [pt.flatsky(m) for m in range(2)])
    for r in runs[1:]:
        for a, b in zip(runs[0], r):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    # against the compensated path, which takes the same decisions and profile values,
    # and against FP64 on the single-signed tSZ maps (the signed kSZ sums of this dense
    # cone cancel in places, which magnifies the FP32 profile values' rounding)
    hpm, fsm, _, _ = run_gpu(rec, [tab], "mixed", 256, npix_fs=256, fov_deg=10.0, maps=maps,
                             flags=0)
    hp64, fs64, _, _ = run_gpu(rec, [tab], "fp64", 256, npix_fs=256, fov_deg=10.0, maps=maps,
                               flags=0)
    for m in range(2):
        assert_maps_close(runs[0][m], hpm[m], rel=1e-6, what="healpix %d vs mixed" % m)
        assert_maps_close(runs[0][2 + m], fsm[m], rel=1e-6, what="flat sky %d vs mixed" % m)
    assert_maps_close(runs[0][0], hp64[0], what="healpix tSZ vs fp64")
    assert_maps_close(runs[0][2], fs64[0], rel=1e-6, what="flat sky tSZ vs fp64")


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_async_readout_overlapping_the_next_paint(precision):
    """p2m_get_healpix_async: a catalogue painted while the previous maps are copied out,
    into alternate bound buffers, and into the same buffer (the clear and the painting
    then wait for the copy)."""
    torch = pytest.importorskip("torch")
    a, b = catalogs.shell(61, 20_000), catalogs.shell(62, 15_000)
    tab = catalogs.table()
    ra, rb = run_oracle(a, [tab], 256)[0][0], run_oracle(b, [tab], 256)[0][0]
    npix = 12 * 256 * 256
    dev = [torch.empty(npix, dtype=torch.float32, device="cuda") for _ in range(2)]
    host = [torch.empty(npix, dtype=torch.float32).pin_memory() for _ in range(5)]
    with p2m.Painter(nside=256, precision=precision, max_records=1 << 16) as pt:
        pt.load_table(0, tab)
        for k, rec in enumerate((a, b, a)):  # alternate buffers; the third reuses the first
            pt.reset()
            pt.bind_healpix_device(0, dev[k & 1].data_ptr())
            pt.paint_records(rec)
            pt.healpix_async(0, host[k].data_ptr())
        pt.reset()
        pt.bind_healpix_device(0, dev[0].data_ptr())
        pt.paint_records(b)
        pt.healpix_async(0, host[3].data_ptr())
        pt.reset()  # the same buffer stays bound
        pt.paint_records(a)
        pt.healpix_async(0, host[4].data_ptr())
        pt.synchronize()
    for h, ref in zip(host, (ra, rb, ra, rb, ra)):
        assert_maps_close(h.numpy(), ref)


def test_layout7_chihview_and_bad_records():
    rec = catalogs.shell(5, 20_000, nfloat=7).copy()
    rec[::997, 0] = np.nan
    rec[5::1009, 6] = np.inf
    tab = catalogs.table()
    hp, _, st, sets = run_gpu(rec, [tab], "mixed", 256, chihview=150.0)
    rhp, _, rst, rsets = run_oracle(rec, [tab], 256, chihview=150.0)
    assert_sets_equal(sets, rsets)
    assert st["n_shell"] == rst["n_cut"]
    assert_maps_close(hp[0], rhp[0])


def test_empty_and_fully_cut():
    tab = catalogs.table()
    with p2m.Painter(nside=64, precision="mixed", max_records=1024) as pt:
        pt.load_table(0, tab)
        pt.paint_records(np.zeros((0, 10), np.float32))
        rec = catalogs.shell(6, 1000, r=(5000.0, 6000.0))  # beyond zmax = 1.25
        pt.paint_records(rec)
        m = pt.healpix(0)
        st = pt.stats()
    assert st["n_shell"] == 0 and np.all(m == 0)


def test_maps_without_zero_halos_match():
    """Skipping halos whose table value is identically zero leaves the maps unchanged."""
    rec = catalogs.shell(7, 30_000, r=(100.0, 8000.0))
    tab = catalogs.table(nu=0.0)
    a, _, _, _ = run_gpu(rec, [tab], "mixed", 512, zmax=6.0)
    b, _, _, _ = run_gpu(rec, [tab], "mixed", 512, zmax=6.0, flags=0)
    assert_maps_close(b[0], a[0], rel=1e-6)


def test_chunked_calls_accumulate():
    """Painting a catalogue in several calls equals painting it at once."""
    rec = catalogs.shell(8, 50_000)
    tab = catalogs.table()
    whole, _, _, _ = run_gpu(rec, [tab], "fp64", 256, flags=0)
    with p2m.Painter(nside=256, precision="fp64", max_records=7000) as pt:
        pt.load_table(0, tab)
        pt.paint_records(rec[:20_000])
        pt.paint_records(rec[20_000:])
        parts = pt.healpix(0)
    assert_maps_close(parts, whole[0], rel=1e-6)


def test_project_halo_matches_records():
    """The per-halo entry (projecthalo_* arguments) paints what the record path paints."""
    rec = catalogs.shell(9, 5000, nfloat=7)
    tab = catalogs.table()
    cos = oracle.Cosmo()
    p = oracle.params(nside=256, nfloat=7)
    ref, _, _, _ = run_gpu(rec, [tab], "mixed", 256, flags=0)
    with p2m.Painter(nside=256, precision="mixed", max_records=8192) as pt:
        pt.load_table(0, tab)
        for r in rec:
            ok, q = oracle.halo_setup(cos, p, r)  # radial cut, mass cut, loop quantities
            if not ok:
                continue
            xr, yr, zr = pt.project_halo(q[0], q[1], q[2], q[3], q[4], q[5], q[6], 1.0, 1)
            assert abs(xr - q[0] / q[4]) <= 1e-6 * abs(q[0] / q[4]) + 1e-30
        m = pt.healpix(0)
    assert_maps_close(m, ref[0], rel=1e-6)


def test_fmath_bit_identical_host_device():
    """The shared float math returns the same bits on the GPU and on the host."""
    import torch
    rng = np.random.default_rng(11)
    n = 1 << 18
    cases = {0: (np.exp(rng.uniform(-40, 40, n)), None), 1: (rng.uniform(-80, 80, n), None),
             2: (np.exp(rng.uniform(-8, 8, n)), rng.uniform(-6, 6, n)),
             3: (rng.uniform(-1, 1, n), None), 4: (rng.uniform(-20, 20, n), None),
             5: (rng.uniform(-12, 12, n), None), 6: (rng.uniform(-12, 12, n), None),
             7: (rng.uniform(0, 3.1, n), None), 9: (rng.uniform(0, 0.785, n), None),
             10: (np.exp(rng.uniform(-80, 80, n)), None)}
    lib = p2m.load_library()
    for fn, (x, y) in cases.items():
        x = x.astype(np.float32)
        y = y.astype(np.float32) if y is not None else None
        host = oracle.fmath(fn, x, y)
        dx = torch.from_numpy(x).cuda()
        dy = torch.from_numpy(y).cuda() if y is not None else None
        dout = torch.empty_like(dx)
        rc = lib.p2m_fmath_eval_device(0, fn, dx.data_ptr(), dy.data_ptr() if dy is not None else None,
                                       dout.data_ptr(), n)
        assert rc == 0
        dev = dout.cpu().numpy()
        same = (dev.view(np.uint32) == host.view(np.uint32)) | (np.isnan(dev) & np.isnan(host))
        assert same.all(), "fn %d: %d of %d differ" % (fn, (~same).sum(), n)


def test_fixed_point_conversions_are_exact():
    """P2M_PREC_FIXED's integer conversions: each value rounded to a multiple of 2^-56
    (ties to even), the integers added, the sum rounded to the nearest float (ties to
    even), against the same arithmetic in numpy: random magnitudes from below half a
    unit to 50, exact ties, opposite values and zeros."""
    import torch
    rng = np.random.default_rng(12)
    n = 1 << 18
    mag = 10.0 ** rng.uniform(-18.0, 1.7, n)
    a = (mag * rng.choice([-1.0, 1.0], n)).astype(np.float32)
    b = (10.0 ** rng.uniform(-18.0, 1.7, n) * rng.choice([-1.0, 1.0], n)).astype(np.float32)
    k = rng.integers(0, 1 << 20, n // 8)
    a[: n // 8] = ((2 * k + 1) * 2.0 ** -57).astype(np.float32)  # a 2^56 = k + 1/2
    b[n // 8: n // 4] = -a[n // 8: n // 4]
    a[n // 4: n // 4 + 64] = 0.0
    qa = np.rint(a.astype(np.float64) * 2.0 ** 56).astype(np.int64)
    qb = np.rint(b.astype(np.float64) * 2.0 ** 56).astype(np.int64)
    ref = ((qa + qb).astype(np.float32) * np.float32(2.0 ** -56)).astype(np.float32)
    lib = p2m.load_library()
    dx, dy = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    dout = torch.empty_like(dx)
    assert lib.p2m_fmath_eval_device(0, 8, dx.data_ptr(), dy.data_ptr(), dout.data_ptr(), n) == 0
    dev = dout.cpu().numpy()
    same = dev.view(np.uint32) == ref.view(np.uint32)
    assert same.all(), "%d of %d differ, e.g. a=%r b=%r: %r vs %r" % (
        (~same).sum(), n, a[~same][:1], b[~same][:1], dev[~same][:1], ref[~same][:1])


@pytest.mark.parametrize("model,nu,alpha", [(1, 148.0, 0.0), (1, 0.0, 0.0), (2, 545.0, 0.0),
                                             (3, 218.0, 0.0), (1, 353.0, 1.0)])
def test_maptable_gpu_matches_oracle(model, nu, alpha):
    """The GPU table maker gives the oracle's table image bit for bit (the same float
    sequence and float functions on both sides; the FP64 virial-radius power rounds to
    the same float)."""
    gpu = p2m.make_maptable(model, nu, alpha, nchit=12, nmht=10, nrt=30)
    ref = oracle.make_maptable(model, nu, alpha, nchit=12, nmht=10, nrt=30)
    assert gpu[:36] == ref[:36]
    g = p2m.table_array(gpu)
    r = p2m.table_array(ref)
    same = (g.view(np.uint32) == r.view(np.uint32)) | (np.isnan(g) & np.isnan(r))
    assert same.all(), "%d of %d entries differ" % ((~same).sum(), same.size)


@pytest.mark.parametrize("big_rings", [None, "0"])
def test_fast_path_decisions_match_exact_path(big_rings, monkeypatch):
    """Every disc decision and table index the mixed-precision fast path takes on its own
    agrees with the exact FP64 path (the recheck bands are wide enough), on the fused
    path (default threshold) and on the stored-item path (threshold 0)."""
    if big_rings is not None:
        monkeypatch.setenv("P2M_BIG_RINGS", big_rings)
    rec = catalogs.shell(12, 1_000_000, r=(100.0, 8000.0), m=(1e12, 3e15))
    tab = catalogs.table(nu=0.0, nchit=40, nmht=40, nrt=200)
    with p2m.Painter(nside=4096, precision="mixed", maps=((0, 1), (0, 2)), zmax=6.0,
                     flags=p2m.FLAG_VALIDATE, max_records=len(rec)) as pt:
        pt.load_table(0, tab)
        pt.paint_records(rec)
        pt.flush()
        st = pt.stats()
    assert st["val_checked"] == st["hp_candidates"] > 2_000_000
    assert st["val_bad_set"] == 0
    assert st["val_bad_index"] == 0
    # the largest error of the fast r-index coordinate stays well inside the band half-width
    assert st["val_max_du"] < 0.25 * 2e-4, st
    assert st["n_recheck"] < 2e-3 * st["hp_candidates"]


def test_readout_then_more_painting_accumulates():
    rec = catalogs.shell(13, 40_000)
    tab = catalogs.table()
    whole, _, _, _ = run_gpu(rec, [tab], "mixed", 256, flags=0)
    with p2m.Painter(nside=256, precision="mixed", max_records=len(rec)) as pt:
        pt.load_table(0, tab)
        pt.paint_records(rec[:15_000])
        first = pt.healpix(0)
        pt.paint_records(rec[15_000:])
        both = pt.healpix(0)
    assert np.abs(first).max() > 0
    assert_maps_close(both, whole[0], rel=1e-6)


def test_bound_device_output():
    import torch
    rec = catalogs.shell(14, 20_000)
    tab = catalogs.table()
    ref, _, _, _ = run_gpu(rec, [tab], "mixed", 128, flags=0)
    out = torch.zeros(12 * 128 * 128, dtype=torch.float32, device="cuda")
    with p2m.Painter(nside=128, precision="mixed", max_records=len(rec)) as pt:
        pt.load_table(0, tab)
        pt.bind_healpix_device(0, out.data_ptr())
        pt.paint_records(rec)
        pt.healpix_device(0, out.data_ptr())
        pt.synchronize()
    assert_maps_close(out.cpu().numpy(), ref[0], rel=1e-6)


def test_cosmology_tables_entry_point():
    """p2m_set_cosmology_tables: the reference's own r(z) and z(r) tables (as the oracle
    builds them, cosmology.f90:51-105) leave the maps bit for bit as they were; r(z) scaled
    by 0.8 shrinks the radial cut's shell [rofz(zmin), rofz(zmax)] to 0.8 of its radii;
    bad tables and a call while painted halos await a read-out are refused."""
    rec = catalogs.shell(2, 40_000, r=(100.0, 8000.0), m=(1e12, 3e15))
    tab = catalogs.table(nu=0.0)
    cos = oracle.Cosmo()
    rofz = np.array(cos.c.rofztable, dtype=np.float32)
    zofr = np.array(cos.c.zofrtable, dtype=np.float32)
    maps = ((0, 1), (0, 2))
    kw = dict(nside=256, precision="mixed", maps=maps, zmax=1.25, max_records=len(rec))

    def paint(tables=None):
        with p2m.Painter(**kw) as pt:
            pt.load_table(0, tab)
            if tables is not None:
                pt.set_cosmology_tables(*tables)
            pt.paint_records(rec)
            return [pt.healpix(m) for m in range(2)], pt.stats()

    base, st0 = paint()
    same, st1 = paint((rofz, zofr))
    assert st0["n_shell"] == st1["n_shell"] > 0
    assert all(np.array_equal(a.view(np.uint32), b.view(np.uint32)) for a, b in zip(base, same))
    _, st2 = paint((rofz * np.float32(0.8), zofr))
    chi = np.sqrt((rec[:, :3].astype(np.float64) ** 2).sum(axis=1))
    hi = 0.8 * float(oracle.Cosmo().rofz(1.25))
    expect = int(((chi >= 0.0) & (chi <= hi)).sum())
    assert abs(st2["n_shell"] - expect) <= 2 and st2["n_shell"] < st0["n_shell"]
    with p2m.Painter(**kw) as pt:
        pt.load_table(0, tab)
        with pytest.raises(p2m.P2MError):
            pt.set_cosmology_tables(rofz[:5000], zofr[:5000])
        bad = rofz.copy()
        bad[17] = np.nan
        with pytest.raises(p2m.P2MError):
            pt.set_cosmology_tables(bad, zofr)
        pt.paint_records(rec[:1000])
        with pytest.raises(p2m.P2MError):
            pt.set_cosmology_tables(rofz, zofr)
        pt.reset()
        pt.set_cosmology_tables(rofz, zofr)


@pytest.mark.parametrize("big_rings", ["0", "1000000"])
def test_fixed_point_range_is_reported(big_rings, monkeypatch):
    """P2M_PREC_FIXED holds |value| < 128: a table in units that exceed it makes the
    read-out fail with P2M_ERR_CAPACITY instead of returning saturated maps (both
    painting paths); the same table paints normally with the other precisions."""
    monkeypatch.setenv("P2M_BIG_RINGS", big_rings)
    rec = catalogs.shell(15, 5_000)
    tab = bytearray(catalogs.table())
    vals = np.frombuffer(tab, dtype=np.float32, offset=36)
    big = (vals * np.float32(1e9)).astype(np.float32)  # y ~ 1e-6 .. 1e-4 -> 1e3 .. 1e5
    tab[36:] = big.tobytes()
    with p2m.Painter(nside=128, precision="fixed", max_records=len(rec)) as pt:
        pt.load_table(0, bytes(tab))
        pt.paint_records(rec)
        with pytest.raises(p2m.P2MError) as e:
            pt.healpix(0)
        assert e.value.status == p2m.capi.P2M_ERR_CAPACITY
    with p2m.Painter(nside=128, precision="mixed", max_records=len(rec)) as pt:
        pt.load_table(0, bytes(tab))
        pt.paint_records(rec)
        assert np.abs(pt.healpix(0)).max() >= 128.0


def test_records_from_page_locked_memory():
    """p2m_host_alloc: records painted from a page-locked block (streamed in three steps per
    call, each step's copy overlapping the painting) give the maps of the same records
    painted from ordinary memory; the block is refilled as soon as p2m_paint_records
    returns."""
    lib = p2m.load_library()
    recs = [catalogs.shell(41 + i, 30_000, r=(100.0, 3000.0), m=(1e12, 3e15)) for i in range(2)]
    tab = catalogs.table(nu=0.0)
    maps = ((0, 1), (0, 2))
    ptr = ctypes.c_void_p()
    assert lib.p2m_host_alloc(recs[0].nbytes, ctypes.byref(ptr)) == p2m.capi.P2M_OK
    assert ptr.value
    try:
        blk = np.ctypeslib.as_array((ctypes.c_float * recs[0].size).from_address(ptr.value))
        blk = blk.reshape(recs[0].shape)
        out = []
        for pinned in (True, False):
            with p2m.Painter(nside=512, precision="mixed", maps=maps, zmax=6.0,
                             max_records=10_000) as pt:
                pt.load_table(0, tab)
                for r in recs:
                    if pinned:
                        blk[:] = r
                        pt.paint_records(blk)
                    else:
                        pt.paint_records(r)
                out.append([pt.healpix(m) for m in range(len(maps))])
    finally:
        assert lib.p2m_host_free(ptr) == p2m.capi.P2M_OK
    for m in range(len(maps)):
        assert np.abs(out[1][m]).max() > 0
        assert_maps_close(out[0][m], out[1][m], rel=1e-6, what="map %d" % m, sum_tol=1e-9)
