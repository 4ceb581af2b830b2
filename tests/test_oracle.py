"""CPU checks of the oracle: the vectorised restatement against the literal
loop restatement and its golden vectors, and the reference's recorded
invariants (exact closure to round-off, divergence-free random field)."""
import math
from pathlib import Path

import numpy as np
import pytest

from oracle import literal as L
from oracle import ns

GOLDEN = Path(__file__).with_name("golden")


@pytest.fixture(scope="module", params=[6, 12])
def gold(request):
    return dict(np.load(GOLDEN / f"literal_n{request.param}.npz"))


def test_golden_rhs_divergence_projection(gold):
    n, l, visc = int(gold["n"]), float(gold["l"]), float(gold["visc"])
    h = l / n
    u = gold["u"]
    np.testing.assert_allclose(ns.rhs(u, visc, h), gold["rhs"], rtol=0, atol=1e-12 * np.abs(gold["rhs"]).max())
    np.testing.assert_allclose(ns.divergence(u, h), gold["div"], rtol=0, atol=1e-12 * np.abs(gold["div"]).max())
    pu, p = ns.project(u, h, return_p=True)
    np.testing.assert_allclose(pu, gold["proj"], rtol=0, atol=1e-12 * np.abs(u).max())
    np.testing.assert_allclose(p, gold["p"], rtol=0, atol=1e-12 * np.abs(gold["p"]).max())
    k, prhs = ns.projected_rhs(u, visc, h)
    np.testing.assert_allclose(k, gold["k"], rtol=0, atol=1e-12 * np.abs(gold["k"]).max())
    np.testing.assert_allclose(prhs, gold["p_rhs"], rtol=0, atol=1e-12 * np.abs(gold["p_rhs"]).max())


def test_golden_filters_and_closure(gold):
    n, c, l, visc, dt = int(gold["n"]), int(gold["c"]), float(gold["l"]), float(gold["visc"]), float(gold["dt"])
    h = l / n
    u = gold["u"]
    ub = ns.apply_DHpi(u, c, l)
    np.testing.assert_allclose(ub, gold["ubar"], rtol=0, atol=1e-12 * np.abs(ub).max())
    _, prhs = ns.projected_rhs(u, visc, h)
    rd = ns.get_rDHi(ns.get_r(ns.stresstensor(u, visc, h), prhs), c)
    got = np.stack([rd[k] for k in ns.NONSYM9])
    np.testing.assert_allclose(got, gold["rdhi"], rtol=0, atol=1e-12 * np.abs(got).max())
    sd = ns.get_sigmaDH(ns.stresstensor(u, visc, h), c)
    got = np.stack([sd[k] for k in ns.SYM6])
    np.testing.assert_allclose(got, gold["sigmadh"], rtol=0, atol=1e-12 * np.abs(got).max())
    st = ns.step_classic_flux_div(ub, ub, u, prhs, visc, l, c, dt)
    np.testing.assert_allclose(st, gold["cfd"], rtol=0, atol=1e-12 * np.abs(st).max())


def test_literal_gaussian_kernels_match():
    """Filters with the Gaussian FDelta of ``get_kernels`` (src/N.jl:1008-1020)."""
    n, c, l, visc = 6, 3, 1.0, 0.02
    h, H = l / n, l / (n // c)
    rng = np.random.default_rng(1)
    u = ns.project(rng.standard_normal((3, n, n, n)), h)
    fd = ns.gaussian(h, 2 * H, 2)
    assert len(fd) > 1
    uL = [L.Field(L.from_ns(u[i])) for i in range(3)]
    GDH, GDHi = L.get_kernels(c, fd)
    ubL = L.apply_DHpi(uL, n // c, GDH, H)
    ub = ns.apply_DHpi(u, c, l, fd)
    assert max(np.abs(ub[i] - L.to_ns(ubL[i].data)).max() for i in range(3)) < 1e-13


def test_randomfield_divergence_free_and_energy():
    """``navierstokes-test.jl:10-29``: the random field is divergence free."""
    n, l = 16, 1.0
    u = ns.randomfield(n, l, kpeak=4, seed=3)
    h = l / n
    assert np.abs(ns.divergence(u, h)).max() < 1e-12 * np.abs(u).max() / h
    assert abs(ns.kinetic_energy(u) - 1.0) < 1e-3
    k, s = ns.spectrum(u, l)
    assert len(s) == (2 * (n // 2)) // 3 and np.all(s >= 0)


def test_projection_is_idempotent_and_kills_divergence():
    n, l = 12, 2.0
    h = l / n
    rng = np.random.default_rng(2)
    u = rng.standard_normal((3, n, n, n))
    pu = ns.project(u, h)
    assert np.abs(ns.divergence(pu, h)).max() < 1e-12 * np.abs(u).max() / h
    np.testing.assert_allclose(ns.project(pu, h), pu, atol=1e-13 * np.abs(u).max())


@pytest.mark.parametrize("c,kind", [(3, "volume"), (2, "volume"), (4, "volume"), (4, "face"), (3, "face")])
def test_exact_closure_invariant(c, kind):
    """An LES carrying the exact commutator at every RK4 stage stays equal to
    the filtered DNS (the reference's recorded 5.69e-15, navierstokes.jl:33)."""
    n, l, visc = 24, 1.0, 1 / 2000
    u = ns.randomfield(n, l, kpeak=4, seed=0)
    les = [ns.Les(c=c, kind=kind)]
    u1, dts, _ = ns.dnsaid_rk4(u, visc, l, 0.3, 4, les)
    tgt = ns.filtered_target(u1, les[0], l)
    assert ns.rel_l2(les[0].v_exact, tgt) < 1e-13
    assert ns.rel_l2(les[0].v_nomodel, tgt) > 1e-3
    assert all(d > 0 for d in dts)


@pytest.mark.parametrize("c", [2, 3, 4])
def test_flux_form_equals_commutator(c):
    """P_H(delta_H sigma_H(ubar) - delta_H^ns rDHi) == P_H filter(k) - P_H RHS_H(ubar)
    (src/N.jl:1189-1206), including the even-ratio extension."""
    n, l, visc = 24, 1.0, 1 / 1000
    h = l / n
    u = ns.randomfield(n, l, kpeak=3, seed=5)
    k, p = ns.projected_rhs(u, visc, h)
    ub = ns.apply_DHpi(u, c, l)
    m1 = ns.closure(k, ub, visc, l, c, "volume")
    m2 = ns.project(ns.closure_flux_div(u, p, visc, l, c, ub), l / (n // c))
    assert ns.rel_l2(m2, m1) < 1e-13


def test_even_taps_reduce_to_box_and_trapezoid():
    o, w = ns.axis_taps(4, ns.FACE, ns.VOLUME)
    assert list(o) == [1, 2, 3, 4, 5] and np.allclose(w, [1 / 8, 1 / 4, 1 / 4, 1 / 4, 1 / 8])
    o, w = ns.axis_taps(4, ns.CENTRE, ns.VOLUME)
    assert list(o) == [0, 1, 2, 3] and np.allclose(w, 0.25)
    o, w = ns.axis_taps(4, ns.CENTRE, ns.POINT)
    assert list(o) == [1, 2] and np.allclose(w, 0.5)
    o, w = ns.axis_taps(5, ns.CENTRE, ns.POINT)
    assert list(o) == [2]
    o, w = ns.axis_taps(5, ns.FACE, ns.VOLUME)
    assert list(o) == [2, 3, 4, 5, 6] and np.allclose(w, 0.2)


def test_dissipation_matches_energy_decay():
    """dE/dt of the inviscid-free part vanishes, so the kinetic energy decays
    at the discrete viscous dissipation rate (energy budget of the scheme)."""
    n, l, visc = 16, 1.0, 1 / 100
    h = l / n
    u = ns.randomfield(n, l, 3, 2)
    dt = 1e-5
    e0 = ns.kinetic_energy(u)
    e1 = ns.kinetic_energy(ns.step_rk4(u, visc, h, dt))
    eps = ns.dissipation(u, visc, h)
    assert abs((e0 - e1) / dt - eps) < 2e-3 * eps


def test_rk4_fourth_order_in_time():
    n, l, visc = 8, 1.0, 1 / 200
    h = l / n
    u = ns.randomfield(n, l, kpeak=2, seed=1)
    T = 0.02
    ref = u
    for _ in range(64):
        ref = ns.step_rk4(ref, visc, h, T / 64)
    errs = []
    for m in (4, 8):
        v = u
        for _ in range(m):
            v = ns.step_rk4(v, visc, h, T / m)
        errs.append(np.linalg.norm(v - ref))
    order = math.log2(errs[0] / errs[1])
    assert order > 3.5


def test_c_restatement_matches_numpy_oracle():
    """The C/OpenMP restatement (the timed CPU baseline) agrees with the NumPy
    oracle on the full DNS-aided RK4 step, odd/even ratios, both filters."""
    import importlib.util
    from pathlib import Path

    spec = importlib.util.spec_from_file_location("bc", Path(__file__).parents[1] / "oracle" / "build_cpu.py")
    bc = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bc)
    if bc.build() is None:
        pytest.skip("no C compiler")
    from oracle import cpu_ref

    n, l, visc = 24, 1.0, 1 / 2000
    les = [(3, "volume"), (2, "face"), (4, "volume")]
    cs = cpu_ref.CpuCase(n, l, visc, 0.3, les)
    cs.init_random(4, 1.0, 0)
    ref = ns.randomfield(n, l, 4, 0)
    assert ns.rel_l2(cs.velocity(), ref) < 1e-13
    ol = [ns.Les(c=c, kind=k) for c, k in les]
    r1, _, _ = ns.dnsaid_rk4(ref, visc, l, 0.3, 2, ol)
    cs.step(2)
    assert ns.rel_l2(cs.velocity(), r1) < 1e-13
    for i in range(3):
        assert ns.rel_l2(cs.les_field(i, "exact"), ol[i].v_exact) < 1e-13
        assert ns.rel_l2(cs.les_field(i, "nomodel"), ol[i].v_nomodel) < 1e-13
    cs.close()


def test_net_oracle_gradients_by_finite_differences():
    """The analytic backward of the learned-closure net (oracle/net.py)."""
    from oracle import net as onet

    rng = np.random.default_rng(0)
    params = onet.init_params(1, hidden=4)
    params = [(W, rng.normal(0, 0.1, b.shape)) for W, b in params]
    x = rng.normal(size=(1, 4, 4, 4, 3))
    t = rng.normal(size=(1, 4, 4, 4, 3))
    loss, grads = onet.loss_and_grads(params, x, t)
    for li, (W, b) in enumerate(params):
        for idx in [(0, 0, 0), (13, 1, 2), (26, 2, 1)]:
            idx = tuple(min(i, s - 1) for i, s in zip(idx, W.shape))
            eps = 1e-6
            Wp = W.copy()
            Wp[idx] += eps
            pp = list(params)
            pp[li] = (Wp, b)
            lp, _ = onet.loss_and_grads(pp, x, t)
            Wm = W.copy()
            Wm[idx] -= eps
            pp[li] = (Wm, b)
            lm, _ = onet.loss_and_grads(pp, x, t)
            fd = (lp - lm) / (2 * eps)
            assert abs(fd - grads[li][0][idx]) < 1e-6 + 1e-5 * abs(fd)


def test_counter_normal_statistics():
    x = ns.counter_normal(0, 200000)
    assert abs(x.mean()) < 0.01 and abs(x.std() - 1) < 0.01
    assert np.array_equal(ns.counter_normal(5, 10, offset=3), ns.counter_normal(5, 13)[3:])


@pytest.mark.parametrize("doproject", [True, False])
def test_paper_volavg_swap_closure_is_exact(doproject):
    """The paper driver dns_aid_volavg (src/NavierStokes.jl:141-304), restated
    with the reference's own filters: its swap closure (face-filtered flux)
    keeps the LES on the volume-filtered DNS to round-off, with and without
    the projections; the other LES drift."""
    n, c, l, visc = 24, 3, 1.0, 1e-3
    u = ns.randomfield(n, l, -5 / 3, 1, 1.0, profile="power")
    fu = ns.paper_volavg_target(u, l, c, doproject)
    les = {k: fu.copy() for k in ns.PAPER_NAMES}
    u2, les2, _, it = ns.dns_aid_volavg_steps(u, les, visc, l, c, 0.05, 0.4, doproject, max_steps=3)
    assert it == 3
    ref = ns.paper_volavg_target(u2, l, c, doproject)
    assert ns.rel_l2(les2["swapfil"], ref) < 1e-13
    for k in ("nomodel", "classic", "swapfil_symm"):
        assert ns.rel_l2(les2[k], ref) > 1e-4, k


@pytest.mark.parametrize("n,c", [(24, 3), (24, 4), (30, 5), (16, 2)])
def test_surface_line_filter_telescopes(n, c):
    """The face average of the fine off-diagonal flux divergence over a
    coarse face equals the coarse divergence of the line-filtered flux (the
    `linefilter!` of dns_aid_surface, src/NavierStokes.jl:369), for odd and
    even ratios, to round-off."""
    l, visc = 1.0, 1 / 500
    u = ns.randomfield(n, l, 3, 1)
    _, p = ns.project(ns.rhs(u, visc, l / n), l / n, return_p=True)
    a, b = ns.surface_offdiag_identity(u, p, visc, l, c)
    assert ns.rel_l2(b, a) < 1e-13


@pytest.mark.parametrize("c,doproject", [(3, True), (4, False)])
def test_paper_surface_driver_properties(c, doproject):
    """dns_aid_surface (src/NavierStokes.jl:306-468) as restated: the target
    fiu (the face average) is divergence free on the LES grid; the swap flux
    (line filter off the diagonal) is symmetric, so the swap and swap-
    symmetric LES coincide; the swap LES stays closer to fiu than the no-model
    LES; no LES is exact (the normal flux term of a face average is a fine
    difference across the face)."""
    n, l, visc = 24, 1.0, 1e-3
    u = ns.randomfield(n, l, -5 / 3, 1, 1.0, profile="power")
    fiu = ns.face_filter(u, c)
    H = l / (n // c)
    assert np.linalg.norm(ns.divergence(fiu, H)) < 1e-12 * np.linalg.norm(fiu) / H
    les = {k: fiu.copy() for k in ns.PAPER_NAMES}
    u2, les2, _, it = ns.dns_aid_surface_steps(u, les, visc, l, c, 0.05, 0.4, doproject, max_steps=3)
    assert it == 3
    ref = ns.face_filter(u2, c)
    assert ns.rel_l2(les2["swapfil"], les2["swapfil_symm"]) < 1e-14
    e = {k: ns.rel_l2(les2[k], ref) for k in ns.PAPER_NAMES}
    assert e["swapfil"] < e["nomodel"]
    assert min(e.values()) > 1e-6


@pytest.mark.parametrize("dtype,ui,mask", [(np.float64, np.uint64, 0x7FFFFFFFFFFFFFFF), (np.float32, np.uint32, 0x7FFFFFFF)])
def test_magnitude_bit_maximum(dtype, ui, mask):
    """The time step's max |u| is taken on the magnitude bits of the words:
    for non-negative IEEE values the unsigned integer order is the numeric
    order and NaN patterns sort above infinity, so the integer maximum is the
    exact max |u| and a NaN propagates."""
    rng = np.random.default_rng(0)
    x = (rng.standard_normal(10000) * np.exp(rng.uniform(-30, 30, 10000))).astype(dtype)
    x[:5] = [0.0, -0.0, np.finfo(dtype).tiny / 4, -np.finfo(dtype).max, np.finfo(dtype).tiny]

    def bitmax(a):
        return np.array([np.max(a.view(ui) & ui(mask))], dtype=ui).view(dtype)[0]

    assert bitmax(x) == np.max(np.abs(x))
    y = x.copy()
    y[17] = -np.inf
    assert bitmax(y) == np.inf
    y[99] = np.nan
    assert np.isnan(bitmax(y))
