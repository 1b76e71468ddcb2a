"""The oracle itself, pinned by what can be derived without the reference's binaries
(which cannot be built here): HEALPix geometry identities and known answers, an
independent numpy float32 restatement of the cosmology tables, and hand-built tables for
the interpolation quirks.  Parity with the reference is otherwise unpinned."""
import math

import numpy as np
import pytest

import catalogs
import oracle

f32 = np.float32


# ---------------------------------------------------------------- HEALPix ----------

@pytest.mark.parametrize("nside", [1, 2, 4, 8, 64])
def test_pixels_per_ring_sum_to_npix(nside):
    tot = 0
    for ring in range(1, 4 * nside):
        npr, ks, npn = oracle.pixels_per_ring(nside, ring)
        assert npr == 4 * min(nside, ring, 4 * nside - ring)
        tot += npr
        assert npn == tot
    assert tot == 12 * nside * nside


def test_pix2vec_known_answers_nside1():
    # Gorski et al. 2005: Nside = 1 has 12 base pixels; centres at z = 2/3 (north),
    # 0 (equator, phi offset 0), -2/3 (south), phi = (i + 1/2) pi/2 in the caps
    for i in range(4):
        v = oracle.pix2vec_ring(1, i)
        assert v[2] == pytest.approx(2.0 / 3.0, abs=1e-15)
        phi = math.atan2(v[1], v[0]) % (2 * math.pi)
        assert phi == pytest.approx((i + 0.5) * math.pi / 2, abs=1e-14)
    for i in range(4):
        v = oracle.pix2vec_ring(1, 4 + i)
        assert v[2] == pytest.approx(0.0, abs=1e-15)
        assert math.atan2(v[1], v[0]) % (2 * math.pi) == pytest.approx(i * math.pi / 2, abs=1e-14)
    for i in range(4):
        v = oracle.pix2vec_ring(1, 8 + i)
        assert v[2] == pytest.approx(-2.0 / 3.0, abs=1e-15)


@pytest.mark.parametrize("nside", [4, 16, 128])
def test_pix2vec_unit_and_ring_z(nside):
    rng = np.random.default_rng(nside)
    for ipix in rng.integers(0, 12 * nside * nside, 300):
        v = oracle.pix2vec_ring(nside, int(ipix))
        assert np.linalg.norm(v) == pytest.approx(1.0, abs=1e-14)
    # ring z from pix2vec equals ring2z of its ring, and ring_num maps it back
    for ring in range(1, 4 * nside):
        npr, ks, npn = oracle.pixels_per_ring(nside, ring)
        v = oracle.pix2vec_ring(nside, npn - npr)
        assert v[2] == pytest.approx(oracle.ring2z(nside, ring), abs=1e-14)
        assert oracle.ring_num(nside, v[2]) == ring


def brute_disc(nside, vec, radius):
    v = np.asarray(vec, float)
    out = []
    for p in range(12 * nside * nside):
        if oracle.angdist(v, oracle.pix2vec_ring(nside, p)) <= radius:
            out.append(p)
    return np.array(out, dtype=np.int64)


@pytest.mark.parametrize("seed", range(6))
def test_query_disc_matches_brute_force(seed):
    rng = np.random.default_rng(seed)
    nside = [4, 8, 16][seed % 3]
    v = rng.normal(size=3)
    if seed == 4:
        v = np.array([0.0, 0.0, 1.0])  # disc centred on the pole
    radius = float(rng.uniform(0.05, 1.2))
    got, _ = oracle.query_disc(nside, v, radius)
    assert np.array_equal(np.sort(got), brute_disc(nside, v, radius))


def test_query_disc_whole_sphere_and_ring_order():
    got, _ = oracle.query_disc(8, [0.3, -0.2, 0.5], math.pi)
    assert np.array_equal(np.sort(got), np.arange(12 * 64))
    got, _ = oracle.query_disc(16, [1.0, 0.01, 0.2], 0.3)
    rings = [oracle.ring_num(16, oracle.pix2vec_ring(16, int(p))[2]) for p in got]
    assert rings == sorted(rings)  # emitted ring by ring (discedge2fulldisc)


def test_angdist_known():
    assert oracle.angdist([1, 0, 0], [0, 1, 0]) == pytest.approx(math.pi / 2)
    assert oracle.angdist([2, 0, 0], [-3, 0, 0]) == pytest.approx(math.pi)  # scale-free
    assert oracle.angdist([1, 0, 0], [1, 1e-9, 0]) == pytest.approx(1e-9, rel=1e-12)


# -------------------------------------------------------------- cosmology ----------

def numpy_tables():
    """Independent float32 restatement of cosmology.f90:51-133 (numpy scalars)."""
    om, h = f32(0.25), f32(0.7)
    ckms = 2.99792458e10 / 1e5

    def dzdr(z):
        zp1 = f32(1) + z
        c3 = (zp1 * zp1) * zp1
        s = np.sqrt(((om * c3) + f32(1)) - om)
        return f32(float(h * f32(100)) / ckms * float(s))

    n = 10000
    dz = f32(6.0) / f32(n - 1)
    rofz = np.zeros(n, f32)
    for i in range(2, n + 1):
        z = f32(i - 1) * dz + f32(0)
        rofz[i - 1] = rofz[i - 2] + (f32(1) / dzdr(z)) * dz
    dr = f32(1.3e4) / f32(n - 1)
    zofr = np.zeros(n, f32)
    for i in range(2, n + 1):
        zofr[i - 1] = zofr[i - 2] + dzdr(zofr[i - 2]) * dr
    return rofz, zofr


def test_cosmology_tables_match_numpy_restatement():
    c = oracle.Cosmo()
    rofz, zofr = numpy_tables()
    assert np.array_equal(np.frombuffer(bytes(c.c.rofztable), f32), rofz)
    assert np.array_equal(np.frombuffer(bytes(c.c.zofrtable), f32), zofr)
    assert c.c.mypi == f32(np.pi)  # 4*atan(1.0) in single precision


def test_cosmology_known_values():
    c = oracle.Cosmo()
    # comoving distance to z = 1 for Om = 0.25, h = 0.7 (flat LCDM) is ~3.4 Gpc
    assert 3300 < c.rofz(1.0) < 3500
    for z in (0.1, 0.5, 1.0, 3.0):
        assert c.zofr(c.rofz(z)) == pytest.approx(z, rel=2e-3)
    # rhocrit(0) = 2.775e11 h^2; deltacrit(0) = 18 pi^2 + 82 x - 39 x^2, x = Om - 1
    assert c.rhocrit(0.0) == pytest.approx(2.775e11 * 0.49, rel=1e-6)
    x = 0.25 - 1.0
    assert c.deltacrit(0.0) == pytest.approx(18 * np.pi ** 2 + 82 * x - 39 * x * x, rel=1e-6)


# ----------------------------------------------------------- interpolation ----------

def synthetic_table(nchit=4, nmht=5, nrt=6, fn=None):
    import struct
    fn = fn or (lambda p, r, m, c: 1000.0 * p + 100.0 * c + 10.0 * m + r + 1.0)
    hdr = struct.pack("<3i6f", nchit, nmht, nrt, 1e2, 7e3, 1e13, 1e16, 1e-2, 10.0)
    t = np.zeros((nchit, nmht, nrt, 2), f32)
    for c in range(nchit):
        for m in range(nmht):
            for r in range(nrt):
                for p in range(2):
                    t[c, m, r, p] = fn(p, r, m, c)
    return hdr + t.tobytes(), t


def test_interpolation_weights_pairing():
    """maptable.f90:204-212 pairs the chi fraction with the M+1 corner and the mass
    fraction with the chi+1 corner; fractions are unnormalised log offsets."""
    img, t = synthetic_table()
    tab = oracle.Table(img)
    cos = oracle.Cosmo()
    th = tab.t
    rng = np.random.default_rng(3)
    for _ in range(50):
        z = float(rng.uniform(0.05, 2.0))
        mh = float(10 ** rng.uniform(13.1, 15.9))
        theta = float(rng.uniform(1e-4, 2e-3))
        got, _ = tab.interpolate(cos, theta, z, mh, 1)
        chi = cos.rofz(z)
        r = f32(chi) * f32(math.tan(theta))
        if r > th.rmaxt or chi > th.chimaxt:
            assert got == 0.0
            continue
        r = max(r, f32(th.rmint + 1e-5))
        lr, lc, lm = math.log(r), math.log(chi), math.log(mh)
        ir = int((lr - math.log(th.rmint)) / th.drt) + 1
        ic = int((lc - math.log(th.chimint)) / th.dchit) + 1
        im = int((lm - math.log(th.mhmint)) / th.dmht) + 1
        fr = lr - (math.log(th.rmint) + (ir - 1) * th.drt)
        fc = lc - (math.log(th.chimint) + (ic - 1) * th.dchit)
        fm = lm - (math.log(th.mhmint) + (im - 1) * th.dmht)
        T = lambda a, b, c: float(t[c - 1, b - 1, a - 1, 0])  # noqa: E731 (ir, imh, ichi)
        want = (T(ir, im, ic) * (1 - fr) * (1 - fc) * (1 - fm) + T(ir + 1, im, ic) * fr * (1 - fc) * (1 - fm)
                + T(ir, im + 1, ic) * (1 - fr) * fc * (1 - fm) + T(ir + 1, im + 1, ic) * fr * fc * (1 - fm)
                + T(ir, im, ic + 1) * (1 - fr) * (1 - fc) * fm + T(ir + 1, im, ic + 1) * fr * (1 - fc) * fm
                + T(ir, im + 1, ic + 1) * (1 - fr) * fc * fm + T(ir + 1, im + 1, ic + 1) * fr * fc * fm)
        assert got == pytest.approx(want, rel=2e-5)


def test_interpolation_clamps_mass_in_place():
    img, _ = synthetic_table()
    tab = oracle.Table(img)
    cos = oracle.Cosmo()
    _, m = tab.interpolate(cos, 1e-4, 0.3, 1e12, 1)
    assert m == f32(1e13)  # mhmint + 1e-5 rounds to mhmint (maptable.f90:192)
    _, m = tab.interpolate(cos, 1e-4, 0.3, 1e17, 1)
    assert m == f32(1e16)


# ------------------------------------------------------------ halo loop ----------

def test_loop_counts_and_disc_sizes():
    rec = catalogs.shell(1, 20_000)
    tab = catalogs.table()
    p = oracle.params(nside=256, npix_fs=16)
    hp, fs, st, sets = oracle.paint(p, [oracle.Table(tab)], rec, record_sets=True)
    assert st["n_in"] == 20_000
    assert 0.08 < st["n_painted"] / st["n_in"] < 0.14  # mass cut keeps ~11%
    assert st["hp_updates"] == len(sets[0])
    assert np.array_equal(np.nonzero(hp[0])[0], np.unique(sets[1][np.isin(
        sets[1], np.nonzero(hp[0])[0])]))


def test_fp32_and_fp64_accumulation_agree():
    rec = catalogs.shell(4, 20_000)
    tab = [oracle.Table(catalogs.table())]
    h64, _, _, _ = oracle.paint(oracle.params(nside=128), tab, rec)
    h32, _, _, _ = oracle.paint(oracle.params(nside=128, fp32=True), tab, rec)
    mx = np.abs(h64).max()
    mask = np.abs(h64) > 1e-3 * mx
    assert (np.abs(h32[mask] - h64[mask]) / np.abs(h64[mask])).max() < 1e-5


def test_threads_as_ranks_equals_serial():
    rec = catalogs.shell(5, 16_000)
    tab = [oracle.Table(catalogs.table())]
    h32, _, _, _ = oracle.paint(oracle.params(nside=128, fp32=True), tab, rec)
    ht, _, st, t = oracle.paint_threads(oracle.params(nside=128, fp32=True), tab, rec, 4)
    mx = np.abs(h32).max()
    assert np.abs(ht - h32).max() <= 1e-5 * mx
    assert len(t) == 3


@pytest.mark.parametrize("scramble,centre", [(0, 0), (1, 1)])
def test_parallel_fp64_equals_serial_bit_for_bit(scramble, centre):
    """orc_paint_parallel replays the threads' deposits in halo order: the same FP64 maps
    (HEALPix and flat sky), counters and pixel sets as the serial loop, bit for bit."""
    rec = np.concatenate([catalogs.edge_cases(), catalogs.shell(7, 30_000)])
    tab = [oracle.Table(catalogs.table())]
    maps = ((0, 1), (0, 2))
    p = oracle.params(nside=128, npix_fs=96, fov_deg=20.0, maps=maps, scramble=scramble,
                      centre=centre)
    hs, fs, ss, sets = oracle.paint(p, tab, rec, record_sets=True)
    hp, fp, sp, setp = oracle.paint(p, tab, rec, record_sets=True, threads=5)
    assert ss["hp_updates"] > 300 and ss["fs_updates"] > 0
    assert np.array_equal(hs, hp) and np.array_equal(fs, fp)
    assert ss == sp
    assert np.array_equal(sets[0], setp[0]) and np.array_equal(sets[1], setp[1])


def test_oracle_generator_equals_library_generator():
    """The CPU arms build their catalogues with the oracle's restatement of the library's
    generator: the same records bit for bit (both layouts, an offset first record)."""
    import matt_young_mapmaking_gb300 as p2m
    for nfloat, first in ((10, 0), (7, 123_457)):
        a = oracle.generate_catalogue(2, 200_000, nfloat, r=(100.0, 8000.0), m=(1e12, 3e15),
                                      first=first)
        b = p2m.generate_catalogue(2, 200_000, nfloat, r=(100.0, 8000.0), m=(1e12, 3e15),
                                   first=first)
        assert a.tobytes() == b.tobytes()


def test_golden_fixture_regression():
    """Oracle output on the committed golden inputs is unchanged (regression pin)."""
    import os
    path = os.path.join(os.path.dirname(__file__), "golden", "oracle_small.npz")
    g = np.load(path)
    p = oracle.params(nside=int(g["nside"]), npix_fs=int(g["npix_fs"]), maps=((0, 1), (0, 2)),
                      zmax=6.0)
    hp, fs, st, sets = oracle.paint(p, [oracle.Table(g["table"].tobytes())], g["records"],
                                    record_sets=True)
    assert np.array_equal(hp, g["hp"])
    assert np.array_equal(fs, g["fs"])
    assert np.array_equal(sets[0], g["set_rec"]) and np.array_equal(sets[1], g["set_pix"])


def test_isolated_halo_total_is_the_table_sum_over_its_disc():
    """Self-pinned invariant: one halo's map total equals its profile summed over the
    pixels whose centres lie inside its disc.  The pixels are found by brute force over
    every pixel centre of the sphere (numpy, from the ring layout), and each pixel's
    value is the table at that pixel's angle from the centre."""
    import spectra
    nside = 512
    rec = np.array([[330.0, 140.0, -210.0, 100.0, 50.0, -20.0, 20.0, 0.0, 0.0, 0.0]], np.float32)
    rec[0, 7:10] = rec[0, :3] - 0.01 * rec[0, 3:6]
    tab = catalogs.table(nu=0.0)
    p = oracle.params(nside=nside, npix_fs=0, maps=((0, 1),), zmax=2.0)
    hp, _, st, sets = oracle.paint(p, [oracle.Table(tab)], rec, record_sets=True)
    cos = oracle.Cosmo()
    ok, q = oracle.halo_setup(cos, p, rec[0])
    assert ok
    xh, yh, zh, rh, chi, mh, z, T = (float(v) for v in q)
    centre = np.array([zh, yh, xh]) / chi  # the halo loop's (x, y, z) -> (z, y, x) order
    rings = spectra.healpix_rings(nside)
    th = np.concatenate([np.full(len(r[1]), r[0]) for r in rings])
    ph = np.concatenate([r[1] for r in rings])
    v = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], axis=1)
    cross = np.linalg.norm(np.cross(v, centre / np.linalg.norm(centre)), axis=1)
    ang = np.arctan2(cross, v @ (centre / np.linalg.norm(centre)))
    inside = np.flatnonzero(ang < T)
    assert 50 < inside.size < 5000
    # no pixel centre sits on the boundary within float noise
    assert np.min(np.abs(ang - T)) > 1e-7
    assert np.array_equal(np.sort(sets[1]), inside)
    tabo = oracle.Table(tab)
    total = sum(tabo.interpolate(cos, float(ang[i]), z, mh, 1)[0] for i in inside)
    assert hp[0].sum() == pytest.approx(total, rel=1e-5)
    assert st["hp_updates"] == inside.size
