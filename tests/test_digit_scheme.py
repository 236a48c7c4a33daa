"""The integer-digit contraction of the tensor-core Legendre synthesis,
restated in numpy (the arithmetic of cunusht_gb300/csrc/legendre_tc.cu,
independent of the GPU):

  lambda sc_l = d0 + d1/256 + d2/256^2 + d3/256^3,  a sc_a = t0 + ... + t3/256^3

with balanced integer digits |d|, |t| <= 128 (exact in bf16), digit products
of equal weight g = i + j summed over a 128-l window (the MMA), weights
4..1 folded by Horner in FP32 and added with weight 0 to a compensated sum.
Pins: the window sums stay below 2^24 (exact in FP32 tensor memory) even for
adversarial digits; keeping g <= 4 leaves about 1e-9 for values spread
below the window bounds; dropping g = 4 costs several times more there (the
reason the kernel keeps five weights)."""
import numpy as np

W = 128


def digits(x):
    """Balanced base-256 digits of x (|x| <= 128), rounding to nearest."""
    d = []
    r = np.asarray(x, dtype=np.float64)
    for _ in range(4):
        q = np.rint(r)
        d.append(q)
        r = (r - q) * 256.0
    return d


def contract(lam, a, ng):
    """sum_l lam_l a_l through the digit scheme: window sums per weight g < ng
    (exact integers), Horner fold of g >= 1 in float32, float64 total."""
    dl, ta = digits(lam), digits(a)
    D = []
    for g in range(ng):
        s = np.zeros(lam.shape[:-1])
        for i in range(4):
            j = g - i
            if 0 <= j <= 3:
                s = s + np.sum(dl[i] * ta[j], axis=-1)
        D.append(s)
    fold = 0.0
    if ng > 1:
        hr = D[ng - 1].astype(np.float32)
        for g in range(ng - 2, 0, -1):
            # the scaling by 2^-8 is exact, so this rounds once, as fmaf does
            hr = hr * np.float32(2.0 ** -8) + D[g].astype(np.float32)
        fold = hr.astype(np.float64) * 2.0 ** -8
    return D[0] + fold, D


def test_window_sums_exact_in_fp32_for_adversarial_digits():
    # every digit at its extreme and of one sign: the largest possible group sums
    lam = np.full((1, W), 128.0 - 128.0 / 255.0)
    a = lam.copy()
    _, D = contract(lam, a, 5)
    for g, s in enumerate(D):
        assert np.all(np.abs(s) < 2 ** 24), (g, s)
        assert np.all(np.float32(s) == s)          # exact in FP32


def test_contraction_error_at_digit_truncation_level():
    """Values spread over two decades below the window bound, as the Legendre
    functions and the alm are within a window (the bound is the largest)."""
    rng = np.random.default_rng(3)
    shape = (400, W)
    lam = rng.uniform(-1, 1, size=shape) * 128 * 10.0 ** -rng.uniform(0, 2, size=shape)
    a = rng.uniform(-1, 1, size=shape) * 128 * 10.0 ** -rng.uniform(0, 2, size=shape)
    exact = np.sum(lam.astype(np.longdouble) * a.astype(np.longdouble), axis=-1)
    rel = lambda got: float(np.linalg.norm(got - exact) / np.linalg.norm(exact))
    e5 = rel(contract(lam, a, 5)[0])
    e4 = rel(contract(lam, a, 4)[0])
    assert e5 < 2e-9, e5                           # digit truncation, 2^-32 of the bounds
    assert e4 > 2.5 * e5, (e4, e5)                 # g = 4 pairs low digits of full size
