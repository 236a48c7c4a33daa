"""Generates tests/golden/golden_small.npz from the FP64 oracle.

Run from the repository root:  python tests/golden/make_golden.py
Contents: a small lmax = 15 case for spin 0, 1, 2 (alm, random points, direct
synthesis values, adjoint alm of random values) and a pointing case.  The
fixture freezes the oracle's outputs so that GPU tests and oracle changes are
compared against the same numbers.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle as orc  # noqa: E402


def main():
    L = 15
    rng = np.random.default_rng(2024)
    n = orc.nalm(L)
    th = np.arccos(rng.uniform(-1, 1, 64))
    ph = rng.uniform(0, 2 * np.pi, 64)
    out = {"lmax": L, "theta": th, "phi": ph}
    for spin in (0, 1, 2):
        ncomp = 1 if spin == 0 else 2
        a = rng.standard_normal((ncomp, n)) + 1j * rng.standard_normal((ncomp, n))
        a[:, :L + 1] = a[:, :L + 1].real
        for m in range(L + 1):
            b = orc.almidx(L, m, m)
            for l in range(m, min(spin, L + 1)):
                a[:, b + l - m] = 0
        A = a[0] if spin == 0 else a
        v = rng.standard_normal(64 if spin == 0 else (2, 64))
        out[f"alm_s{spin}"] = a
        out[f"map_s{spin}"] = orc.synth_points(L, spin, A, th, ph)
        out[f"val_s{spin}"] = v
        out[f"adj_s{spin}"] = orc.adjoint_synth_points(L, spin, v, th, ph)
    pt = np.arccos(rng.uniform(-0.99, 0.99, 32))
    pp = rng.uniform(0, 2 * np.pi, 32)
    dt = rng.standard_normal(32) * 1e-3
    dp = rng.standard_normal(32) * 1e-3
    thp, php = orc.pointing(pt, pp, dt, dp)
    out.update(ptheta=pt, pphi=pp, dth=dt, dph=dp, thp=thp, php=php)
    np.savez_compressed(os.path.join(os.path.dirname(__file__), "golden_small.npz"), **out)


if __name__ == "__main__":
    main()
