"""Differentiable lensing at the differentiable-lensing configuration
(spin 0, lmax 1023, float64): gradients of L = ||gclm2lenmap(gclm, dlm) - d||^2,
d = a lensed seeded realisation plus white noise of 10 uK.arcmin, from the
hand-written adjoint (gclm) and pointing-Jacobian VJP (dlm) kernels, against
central finite differences (step 1e-6 relative) on 64 random directions each,
and the gclm gradient against the adjoint operator (dot-product test,
test/test_adjointOperator.py:246-277 pattern)."""
import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

LMAX = 1023
NDIR = 64


def _direction(lmax, rng):
    n = orc.nalm(lmax)
    v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    v[:lmax + 1] = v[:lmax + 1].real  # real-field direction: m = 0 real
    return v / np.linalg.norm(v)


@pytest.fixture(scope="module")
def setup(built_lib):
    import cunusht_gb300 as cu
    from cunusht_gb300.autograd import gclm2lenmap
    lmax = LMAX
    T = cu.get_transformer("GPU")(("gl", {"lmax": lmax}), nuFFTtype=2, epsilon=1e-10, precision="fp64", max_spin=0)
    gclm, dls = orc.make_inputs(lmax, 0, seed=5)
    rng = np.random.default_rng(6)
    g = torch.as_tensor(gclm[0], device="cuda")
    d = torch.as_tensor(dls[0], device="cuda")
    # data: a lensed realisation of another field plus 10 uK.arcmin white noise
    g2, _ = orc.make_inputs(lmax, 0, seed=9)
    data = T.gclm2lenmap(torch.as_tensor(g2[0], device="cuda"), lmax, lmax, dlm_scaled=d, verbose=0)
    pix_arcmin = np.sqrt(4 * np.pi / T.npix()) * 180 * 60 / np.pi
    data = data + torch.as_tensor(rng.standard_normal(data.numel()) * (10.0 / pix_arcmin), device="cuda")
    T.dlm_scaled = None

    def loss(gg, dd):
        out = gclm2lenmap(T, gg, dd)
        return torch.sum((out - data) ** 2)

    return T, lmax, g, d, loss, rng


def _fd(loss, g, d, vg, vd, h):
    with torch.no_grad():
        lp = loss(g + h * vg, d + h * vd).item()
        lm = loss(g - h * vg, d - h * vd).item()
    return (lp - lm) / (2 * h)


def test_gclm_gradient_matches_finite_differences(setup):
    T, lmax, g, d, loss, rng = setup
    gg = g.clone().requires_grad_(True)
    L = loss(gg, d)
    L.backward()
    grad = gg.grad.cpu().numpy()
    h = 1e-6 * float(torch.linalg.norm(g))
    worst = 0.0
    for _ in range(NDIR):
        v = _direction(lmax, rng)
        fd = _fd(loss, g, d, torch.as_tensor(v, device="cuda"), torch.zeros_like(d), h)
        an = float(np.sum((np.conj(grad) * v).real))
        worst = max(worst, abs(fd - an) / (abs(an) + 1e-8 * L.item()))
        assert abs(fd - an) <= 1e-6 * abs(an) + 1e-8 * L.item(), (fd, an)


def test_dlm_gradient_matches_finite_differences(setup):
    T, lmax, g, d, loss, rng = setup
    dd = d.clone().requires_grad_(True)
    L = loss(g, dd)
    L.backward()
    grad = dd.grad.cpu().numpy()
    h = 1e-6 * float(torch.linalg.norm(d))
    for _ in range(NDIR):
        v = _direction(lmax, rng)
        fd = _fd(loss, g, d, torch.zeros_like(g), torch.as_tensor(v, device="cuda"), h)
        an = float(np.sum((np.conj(grad) * v).real))
        assert abs(fd - an) <= 1e-5 * abs(an) + 1e-9 * L.item(), (fd, an)


def test_gclm_gradient_is_twice_the_adjoint(setup):
    """dL/dgclm = 2 A^H (A gclm - d) with A = lensing operator: the gclm
    gradient equals the adjoint operator applied to the map gradient."""
    T, lmax, g, d, loss, rng = setup
    gg = g.clone().requires_grad_(True)
    L = loss(gg, d)
    L.backward()
    # A x and A^H y consistency: <y, A x> = <A^H y, x> with the stored-alm inner product
    y = torch.as_tensor(rng.standard_normal(T.npix()), device="cuda")
    x = torch.as_tensor(_direction(lmax, rng), device="cuda")
    Ax = T.gclm2lenmap(x, lmax, lmax, dlm_scaled=d, verbose=0)
    AHy = T.lenmap2gclm(y, d, None, lmax, lmax, verbose=0)
    lhs = float(torch.sum(y * Ax))
    rhs = orc.alm_dot(AHy.cpu().numpy(), x.cpu().numpy(), lmax)
    np.testing.assert_allclose(lhs, rhs, rtol=1e-9)
    assert torch.all(torch.isfinite(gg.grad))
