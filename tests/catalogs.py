"""Seeded synthetic catalogues and tables for the tests (the reference's own catalogue
and tables are not available; these stand in with the benchmark workloads' shells, mass
ranges and record layouts)."""
import functools

import numpy as np

import matt_young_mapmaking_gb300 as p2m
import oracle


def shell(seed, n, nfloat=10, r=(100.0, 3000.0), m=(1e12, 1e15)):
    return p2m.generate_catalogue(seed, n, nfloat, r=r, m=m)


@functools.lru_cache(maxsize=None)
def table(model=1, nu=148.0, alpha=0.0, nchit=24, nmht=20, nrt=60):
    """A reduced-size make_maptable table built by the oracle (same bounds as the
    reference's, fewer entries so it is built in well under a second)."""
    return oracle.make_maptable(model, nu, alpha, nchit=nchit, nmht=nmht, nrt=nrt)


def cone(seed, n, axis, half_angle_deg, r=(100.0, 3000.0), m=(1e13, 1e15), nfloat=10):
    """Halos whose directions lie within half_angle of a record-frame axis."""
    rec = shell(seed, n, nfloat, r=r, m=m).copy()
    rng = np.random.default_rng(seed + 77)
    axis = np.asarray(axis, dtype=np.float64)
    axis /= np.linalg.norm(axis)
    ca = np.cos(np.radians(half_angle_deg))
    cost = 1.0 - rng.random(n) * (1.0 - ca)
    sint = np.sqrt(1.0 - cost * cost)
    phi = rng.random(n) * 2 * np.pi
    # orthonormal frame around axis
    t = np.array([1.0, 0, 0]) if abs(axis[0]) < 0.9 else np.array([0, 1.0, 0])
    e1 = np.cross(axis, t)
    e1 /= np.linalg.norm(e1)
    e2 = np.cross(axis, e1)
    d = (cost[:, None] * axis + sint[:, None] * (np.cos(phi)[:, None] * e1 +
                                                  np.sin(phi)[:, None] * e2))
    rr = np.linalg.norm(rec[:, :3].astype(np.float64), axis=1)
    rec[:, :3] = (d * rr[:, None]).astype(np.float32)
    if nfloat == 10:
        rec[:, 7:10] = rec[:, :3] - 0.01 * rec[:, 3:6]
    return rec


def edge_cases(nfloat=10):
    """Hand-placed halos: on the pole, straddling phi = 0, on the equator, near the
    cap/belt boundary, very close (large discs), at the cut edges."""
    rows = []
    big = 3.0  # RTH in Mpc: M ~ 5e14
    for r in (150.0, 400.0, 1200.0, 2500.0):
        rows.append([0.0, 0.0, r, 100.0, -50.0, 30.0, big])        # north pole (record z)
        rows.append([0.0, 0.0, -r, 10.0, 20.0, -300.0, big])       # south pole
        rows.append([r, 0.0, 0.0, 200.0, 0.0, 0.0, big])           # phi = 0 on the equator
        rows.append([r * 0.8, -1e-4 * r, r * 0.6, 5.0, 5.0, 5.0, big])  # straddling phi = 0
        z = r * 2.0 / 3.0
        rows.append([np.sqrt(r * r - z * z), 0.3, z, -30.0, 0.0, 10.0, big])  # cap boundary
        rows.append([r * 0.5, r * 0.5, r * 0.7071, 0.0, 0.0, 0.0, 1.5])
    rows.append([0.0, 0.0, 101.0, 0.0, 0.0, 0.0, 4.0])  # very large disc
    rows.append([60.0, 0.0, 0.0, 0.0, 0.0, 0.0, 3.0])  # inside zmin cut? (chi = 60)
    a = np.array(rows, dtype=np.float32)
    if nfloat == 10:
        a = np.concatenate([a, a[:, :3] - 0.01 * a[:, 3:6]], axis=1)
    return a
