"""CPU checks of the two algebraic forms the FP64 kernels evaluate, restated in
NumPy (float64, and float32 arithmetic for the extraction):

* the RHS sweep's stresses of the scaled, shifted velocities w = s u - q
  (s = sqrt(1/(4h)), q = rho/2, rho = (4 visc/h) s): -(w_i + w_i(-e_i))^2 -
  4 rho w_i(-e_i) on the diagonal and -(w_i + w_i(+e_j))(w_j + w_j(+e_i)) -
  2 rho (w_i + w_j) off it equal -1/(4h) times four times the reference's
  stresses up to a constant per component, so their divergence is the
  reference's RHS (oracle.ns.rhs) to rounding;
* the mixed-precision solve's stencil sums (six FP32 neighbours - 6 c) by two
  levels of error-free extraction against powers of two: every extracted sum
  is exact, and the result is within one FP64 rounding (plus 2^-57 of the
  largest term) of the exact value -- at least as close as six FP64 additions.
"""
from fractions import Fraction

import numpy as np
import pytest

from oracle import ns

F32 = np.float32


def shifted_rhs(u, visc, h):
    """du from the shifted stress form (axes of u[c]: z, y, x)."""
    kd = 0.25 / h
    rv = 4 * visc / h
    s = np.sqrt(kd)
    rho = rv * s
    w = s * u - 0.5 * rho
    ax = {0: 2, 1: 1, 2: 0}
    S = {}
    for i in range(3):
        b = np.roll(w[i], 1, axis=ax[i])  # lower neighbour along i
        t = w[i] + b
        S[i, i] = -t * t - 4 * rho * b
    for i in range(3):
        for j in range(i + 1, 3):
            a, bb = w[i], np.roll(w[i], -1, axis=ax[j])
            c, d = w[j], np.roll(w[j], -1, axis=ax[i])
            S[i, j] = S[j, i] = -(a + bb) * (c + d) - 2 * rho * (a + c)
    du = np.zeros_like(u)
    for i in range(3):
        for j in range(3):
            if i == j:
                du[i] += np.roll(S[i, i], -1, axis=ax[i]) - S[i, i]
            else:
                du[i] += S[i, j] - np.roll(S[i, j], 1, axis=ax[j])
    return du


@pytest.mark.parametrize("visc", [1 / 2000, 1 / 100, 0.1])
def test_shifted_stress_form_matches_the_reference_rhs(visc):
    n, l = 12, 1.0
    h = l / n
    u = np.random.default_rng(3).standard_normal((3, n, n, n))
    ref = ns.rhs(u, visc, h)
    got = shifted_rhs(u, visc, h)
    assert np.abs(got - ref).max() <= 1e-14 * np.abs(ref).max()


def _bits(x):
    return int(np.array([x], dtype=F32).view(np.uint32)[0])


def _from_bits(b):
    return np.array([b], dtype=np.uint32).view(F32)[0]


def _extract(sigma, t):
    hi = F32(F32(sigma + t) - sigma)
    return hi, F32(t - hi)


def stencil7_f32(nb, c):
    """(sum of nb) - 6 c of float32 values as a float64: the kernel's steps."""
    t = [F32(v) for v in nb] + [F32(F32(-4) * F32(c)), F32(F32(-2) * F32(c))]
    mb = max(_bits(v) & 0x7FFFFFFF for v in t)
    e1 = min((mb >> 23) + 5, 254)
    s1 = _from_bits(e1 << 23)
    s2 = _from_bits((e1 - 19 if e1 > 20 else 1) << 23)
    h1 = h2 = l2 = F32(0)
    for i in range(8):
        q, t[i] = _extract(s1, t[i])
        assert F32(h1 + q) == Fraction(float(h1)) + Fraction(float(q))  # level 1 sums are exact
        h1 = F32(h1 + q)
    for i in range(8):
        q, t[i] = _extract(s2, t[i])
        assert F32(h2 + q) == Fraction(float(h2)) + Fraction(float(q))  # level 2 sums are exact
        h2 = F32(h2 + q)
    for i in range(8):
        l2 = F32(l2 + t[i])
    hh = float(h1) + float(h2)
    assert Fraction(hh) == Fraction(float(h1)) + Fraction(float(h2))  # h1 + h2 is exact in FP64
    return hh + float(l2)


@pytest.mark.parametrize("kind", ["smooth", "noise", "spread", "equal"])
def test_stencil_extraction_is_exact_to_one_rounding(kind):
    rng = np.random.default_rng({"smooth": 1, "noise": 2, "spread": 3, "equal": 4}[kind])
    for _ in range(400):
        base = rng.standard_normal() * 10.0 ** rng.integers(-20, 20)
        if kind == "smooth":
            v = base * (1 + 1e-3 * rng.standard_normal(7))
        elif kind == "noise":
            v = base * rng.standard_normal(7)
        elif kind == "spread":
            v = base * rng.standard_normal(7) * 2.0 ** rng.integers(-40, 5, 7)
        else:
            v = np.full(7, base)
        v = v.astype(F32)
        nb, c = list(v[:6]), v[6]
        exact = sum(Fraction(float(x)) for x in nb) - 6 * Fraction(float(c))
        got = stencil7_f32(nb, c)
        big = max(abs(float(x)) for x in list(nb) + [4 * float(c)])
        err = abs(Fraction(got) - exact)
        assert err <= abs(exact) * Fraction(1, 2 ** 52) + Fraction(big) / 2 ** 57
        if kind == "equal":
            assert Fraction(got) == exact
