"""GPU parity of the batched 1-D Burgers path (``exc_burgers_*``) against the
oracle ``oracle.burgers``: 1e-12 relative per step for the DNS and the four
LES of ``dns_aided_les``, the exact-closure invariant on the GPU, the
closure terms, fractions and dissipation, the Smagorinsky fit and solve, and
sample independence inside a batch."""
import math

import numpy as np
import pytest

from oracle import burgers as O

pytestmark = pytest.mark.gpu
TWO_PI = 2 * math.pi


@pytest.fixture(scope="module")
def GB(built_lib):
    from exactclosure_gb300 import burgers

    return burgers


def rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def batch(GB, nh, ns, visc, u0=None, kpeak=10, seed=1):
    b = GB.Batch(GB.Grid(TWO_PI, nh), ns, visc)
    if u0 is None:
        b.randomfield(kpeak, 2.0, seed)
    else:
        b.set_velocity(u0)
    return b


@pytest.mark.parametrize("nh,ns,kpeak,seed", [(675, 4, 10, 1), (13500, 3, 10, 5), (96, 2, 3, 9)])
def test_randomfield_matches_oracle(GB, nh, ns, kpeak, seed):
    b = batch(GB, nh, ns, 5e-4, kpeak=kpeak, seed=seed)
    ref = O.randomfields(ns, nh, TWO_PI, kpeak, 2.0, seed)
    assert rel(b.velocity(), ref) < 1e-12
    assert rel(b.velocity(initial=True), ref) < 1e-12


@pytest.mark.parametrize("scheme", ["euler", "rk4"])
def test_dns_steps_match_oracle_per_step(GB, scheme):
    nh, ns, visc = 675, 3, 5e-4
    u0 = O.randomfields(ns, nh, TWO_PI, 10, 2.0, 2)
    b = batch(GB, nh, ns, visc, u0)
    u, t = u0, np.zeros(ns)
    for step in range(6):
        b.advance(0.1, 0.3, scheme, max_steps=1)
        u, t, _ = O.dns(u, visc, TWO_PI, 0.1, 0.3, scheme, max_steps=1, t0=t)
        assert rel(b.velocity(), u) < 1e-12, step
        tg, sg = b.time()
        assert np.abs(tg - t).max() <= 1e-15 * t.max()
        assert (sg == step + 1).all()


def test_dns_to_tstop_matches_oracle(GB):
    nh, ns, visc = 675, 4, 5e-4
    u0 = O.randomfields(ns, nh, TWO_PI, 10, 2.0, 3)
    b = batch(GB, nh, ns, visc, u0)
    m = b.advance(0.05, 0.3)
    u, t, steps = O.dns(u0, visc, TWO_PI, 0.05, 0.3)
    tg, sg = b.time()
    assert (sg == steps).all() and m == steps.max()
    assert np.abs(tg - 0.05).max() < 1e-15
    assert rel(b.velocity(), u) < 1e-11


@pytest.mark.parametrize("nh,nH,ratio,kind", [(675, 45, 2.0, "gaussian"), (675, 135, 2.0, "gaussian"),
                                              (675, 225, 1.0, "tophat"), (675, 27, 0.0, "gaussian")])
def test_dns_aided_les_per_step(GB, nh, nH, ratio, kind):
    ns, visc = 3, 5e-4
    u0 = O.randomfields(ns, nh, TWO_PI, 10, 2.0, 4)
    b = batch(GB, nh, ns, visc, u0)
    b.les_setup(GB.Grid(TWO_PI, nH), ratio, kind)
    state = None
    for step in range(5):
        b.advance(0.1, 0.3, max_steps=1)
        state = O.dns_aided_les(u0, nH, visc, TWO_PI, ratio, kind, 0.1, 0.3, max_steps=1, state=state)
        u, t, steps, V = state
        assert rel(b.velocity(), u) < 1e-12, step
        for k in O.LES_NAMES:
            assert rel(b.les(k), V[k]) < 1e-12, (step, k)


def test_dns_aided_les_full_run(GB):
    """Run to tstop: fields, filtered DNS and errors; the exact closure
    reproduces the filtered DNS on the GPU."""
    nh, nH, ns, visc = 675, 45, 4, 5e-4
    u0 = O.randomfields(ns, nh, TWO_PI, 10, 2.0, 1)
    b = batch(GB, nh, ns, visc, u0)
    out = GB.dns_aided_les(b, GB.Grid(TWO_PI, nH), 2 * TWO_PI / nH, 0.1, 0.3)
    u, t, steps, V = O.dns_aided_les(u0, nH, visc, TWO_PI, 2.0, "gaussian", 0.1, 0.3)
    fil, dfil = O.filtered_dns(u, nH, TWO_PI, 2.0, "gaussian")
    assert rel(out["dns_ref"], u) < 1e-11
    assert rel(out["dns_ref_fil"], fil) < 1e-11
    assert rel(out["dns_fil"], dfil) < 1e-11
    for k in O.LES_NAMES:
        assert rel(out[k], V[k]) < 1e-11, k
    e = b.errors()
    eo = O.compute_errors(V, dfil)
    assert e["swapfil"] < 1e-13
    for k in ("nomodel", "class_m", "class_p"):
        assert abs(e[k] - eo[k]) < 1e-10 * eo[k]
    assert math.isnan(e["smag"])


def test_reference_sizes_short_run(GB):
    """nh = 13500 with the reference's three LES grids (compression 45, 15,
    5), a few steps each, against the oracle."""
    nh, ns, visc = 13500, 2, 5e-4
    u0 = O.randomfields(ns, nh, TWO_PI, 10, 2.0, 11)
    b = batch(GB, nh, ns, visc, u0)
    for nH in (300, 900, 2700):
        b.restart()
        b.les_setup(GB.Grid(TWO_PI, nH), 2.0, "gaussian")
        b.advance(0.1, 0.3, max_steps=3)
        u, _, _, V = O.dns_aided_les(u0, nH, visc, TWO_PI, 2.0, "gaussian", 0.1, 0.3, max_steps=3)
        assert rel(b.velocity(), u) < 1e-12
        for k in O.LES_NAMES:
            assert rel(b.les(k), V[k]) < 1e-12, (nH, k)


def test_samples_are_independent(GB):
    """A sample gives the same bits alone and inside a batch."""
    nh, nH, visc = 675, 45, 5e-4
    u0 = O.randomfields(5, nh, TWO_PI, 10, 2.0, 21)
    b5 = batch(GB, nh, 5, visc, u0)
    b1 = batch(GB, nh, 1, visc, u0[3:4])
    for b in (b5, b1):
        b.les_setup(GB.Grid(TWO_PI, nH), 2.0)
        b.advance(0.05, 0.3)
    assert np.array_equal(b5.velocity()[3], b1.velocity()[0])
    for k in O.LES_NAMES:
        assert np.array_equal(b5.les(k)[3], b1.les(k)[0])


def test_closure_terms_fractions_dissipation(GB):
    nh, nH, ns, visc = 675, 45, 3, 5e-4
    u0 = O.randomfields(ns, nh, TWO_PI, 10, 2.0, 8)
    u, _, _ = O.dns(u0, visc, TWO_PI, 0.05, 0.3)
    b = batch(GB, nh, ns, visc, u)
    b.les_setup(GB.Grid(TWO_PI, nH), 2.0)
    terms, diss, fr = b.closure_terms()
    _, les, dbl = O.kernels(nh, nH, TWO_PI, 2.0, "gaussian")
    ref = O.closure_terms(u, visc, TWO_PI, nH, les, dbl)
    for i in range(5):
        assert rel(terms[:, i], ref[i]) < 1e-12, i
    assert rel(fr, O.compute_fractions(u, visc, TWO_PI, nH, 2.0, "gaussian")) < 1e-12
    dref = O.compute_dissipation(u, visc, TWO_PI, nH, 2.0, "gaussian")
    assert rel(diss.transpose(1, 0, 2), dref) < 1e-12


def test_smagorinsky_fit_and_solve(GB):
    nh, nH, ns, visc = 675, 45, 4, 5e-4
    u0 = O.randomfields(ns, nh, TWO_PI, 10, 2.0, 1)
    b = batch(GB, nh, ns, visc, u0)
    b.advance(0.1, 0.3)
    U, _, _ = O.dns(u0, visc, TWO_PI, 0.1, 0.3)
    b.les_setup(GB.Grid(TWO_PI, nH), 2.0)
    th, fields = b.smagorinsky_fit(want_fields=True)
    f = O.smagorinsky_fields(U, visc, TWO_PI, nH, 2.0, "gaussian")
    for i, k in enumerate(("Sh", "Th", "SH", "TH")):
        assert rel(fields[:, i], f[k]) < 1e-11, k
    tho = O.smagorinsky_theta(f)
    assert abs(th[0] - tho[0]) < 1e-11 * abs(tho[0]) and abs(th[1] - tho[1]) < 1e-11 * abs(tho[1])
    theta = math.sqrt(th[1])
    b.smagorinsky_solve(theta, 0.1, 0.3)
    ub, _, _ = O.solve_smagorinsky(u0, visc, TWO_PI, nH, 2.0, "gaussian", theta, 0.1)
    assert rel(b.les("smag"), ub) < 1e-11
    _, dfil = O.filtered_dns(U, nH, TWO_PI, 2.0, "gaussian")
    e = b.errors()["smag"]
    assert abs(e - np.linalg.norm(ub - dfil) / np.linalg.norm(dfil)) < 1e-9 * e


def test_nonfinite_is_flagged(GB):
    from exactclosure_gb300 import ExcError

    u = O.randomfields(2, 96, TWO_PI, 3, 2.0, 1)
    u[1, 5] = np.nan
    b = batch(GB, 96, 2, 5e-3, u)
    with pytest.raises(ExcError) as ei:
        b.advance(0.01, 0.3)
    assert ei.value.code == 6
    t, s = b.time()
    assert s[1] == 0 and t[0] == pytest.approx(0.01)
