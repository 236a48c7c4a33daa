"""The FP64 CPU restatement of the reference's lensing algorithm
(oracle/fastcpu.c: the timed CPU baseline) against the exact direct-summation
oracle: full lensing chain (deflection, pointing, spin-s synthesis at the
deflected points, rotation) at sampled pixels, within the requested epsilon."""
import numpy as np
import pytest

import oracle
from oracle import oracle as orc


def _exact(lmax, spin, gclm, dls, th, ph):
    ll = np.arange(lmax + 1)
    fl = np.sqrt(ll * (ll + 1.0))
    dl = np.stack([orc.almxfl(d, fl, lmax) for d in dls])
    d = oracle.synth_points_c(lmax, 1, dl, th, ph)
    rt, rp = orc.pointing(th, ph, d[0], d[1])
    v = oracle.synth_points_c(lmax, spin, gclm if spin else gclm[0], rt, rp)
    if spin:
        z = (v[0] + 1j * v[1]) * np.exp(1j * spin * orc.rotation_gamma(th, d[0], d[1]))
        v = np.stack([z.real, z.imag])
    return v, rt, rp


@pytest.mark.parametrize("lmax,spin,eps,curl", [(63, 0, 1e-10, False), (63, 2, 1e-10, True),
                                                (95, 2, 1e-7, False), (95, 0, 1e-5, True)])
def test_fastcpu_lensing_matches_direct_sum(lmax, spin, eps, curl):
    th, p0, nph, ofs, _ = orc.gl_geometry(lmax)
    fc = oracle.FastCPU(lmax, th, p0, int(nph[0]), eps)
    gclm, dls = orc.make_inputs(lmax, spin, seed=8, curl=curl)
    out = fc.lensing(gclm if spin else gclm[:1], dls[0], spin, dclm_scaled=dls[1] if curl else None)
    tpix, ppix = orc.geometry_pixels(th, p0, nph, ofs)
    idx = np.random.default_rng(1).choice(tpix.size, 300, replace=False)
    ref, rt, rp = _exact(lmax, spin, gclm, dls if curl else dls[:1], tpix[idx], ppix[idx])
    got = out[:, idx] if spin else out[idx]
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < eps
    ptg = fc.last_pointing()
    assert np.max(np.abs(ptg[0, idx] - rt)) < 1e-13
    fc.close()
