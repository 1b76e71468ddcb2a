"""Writes tests/golden/oracle_small.npz: a small seeded catalogue, a reduced table, and
the oracle's maps and pixel sets for them (a regression pin of the oracle; the reference
itself ships no golden vectors).  Run from the repository root:
    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle")]

import oracle  # noqa: E402

import matt_young_mapmaking_gb300 as p2m  # noqa: E402


def main():
    rec = p2m.generate_catalogue(21, 3000, 10, r=(100.0, 1500.0), m=(1e12, 3e15))
    table = oracle.make_maptable(1, 0.0, 0.0, nchit=8, nmht=6, nrt=24)
    nside, npix_fs = 128, 32
    p = oracle.params(nside=nside, npix_fs=npix_fs, maps=((0, 1), (0, 2)), zmax=6.0)
    hp, fs, st, sets = oracle.paint(p, [oracle.Table(table)], rec, record_sets=True)
    np.savez_compressed(os.path.join(HERE, "oracle_small.npz"), records=rec,
                        table=np.frombuffer(table, np.uint8), nside=nside, npix_fs=npix_fs,
                        hp=hp, fs=fs, set_rec=sets[0], set_pix=sets[1])
    print("wrote oracle_small.npz:", st)


if __name__ == "__main__":
    main()
