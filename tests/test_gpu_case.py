"""GPU parity of the case-level ABI (RK4 DNS-aided LES with the exact closure
at every stage) against the oracle's ``dnsaid_rk4``: 1e-12 relative L2 per
step in float64; the float32 precision form against its stated budget."""
import numpy as np
import pytest

from oracle import ns

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def NS(built_lib):
    from exactclosure_gb300 import navierstokes

    return navierstokes


def rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.mark.parametrize("n,kpeak,seed", [(16, 4, 0), (32, 4, 1), (24, 3, 2)])
def test_init_random_matches_oracle(NS, n, kpeak, seed):
    cs = NS.Case(n, 1.0, 1 / 2000, 0.3)
    cs.init_random(kpeak, 1.0, seed)
    u = cs.velocity()
    ref = ns.randomfield(n, 1.0, kpeak, seed)
    assert rel(u, ref) < 1e-12
    assert abs(cs.energy() - ns.kinetic_energy(ref)) < 1e-12
    k, s = ns.spectrum(ref, 1.0)
    assert rel(cs.spectrum(), s) < 1e-12
    eps = ns.dissipation(ref, 1 / 2000, 1.0 / n)
    assert abs(cs.dissipation() - eps) < 1e-12 * eps


# ratio 8 after ratio 4: transverse sums coarsened from the ratio-4 ones; two
# LES of ratio 4 share one set of sums
@pytest.mark.parametrize("n,les", [(32, [(4, "volume")]), (24, [(3, "volume"), (2, "face")]),
                                   (32, [(8, "volume"), (4, "face")]),
                                   (32, [(4, "volume"), (8, "volume"), (4, "face")]),
                                   (28, [(2, "volume")]), (44, [(2, "face")])])
def test_rk4_steps_match_oracle_per_step(NS, n, les):
    l, visc, cfl = 1.0, 1 / 2000, 0.3
    u0 = ns.randomfield(n, l, 4, 3)
    cs = NS.Case(n, l, visc, cfl, les=les)
    cs.set_velocity(u0)
    u = u0
    ol = [ns.Les(c=c, kind=k) for c, k in les]
    for le in ol:
        tgt = ns.filtered_target(u, le, l)
        le.v_exact, le.v_nomodel = tgt.copy(), tgt.copy()
    for step in range(3):
        cs.step(1)
        u, dts, _ = _one_step(u, visc, l, cfl, ol)
        assert rel(cs.velocity(), u) < 1e-12, step
        t, dt = cs.time()
        assert abs(dt - dts) <= 1e-14 * dts
        for i, le in enumerate(ol):
            assert rel(cs.les(i, "exact"), le.v_exact) < 1e-12
            assert rel(cs.les(i, "nomodel"), le.v_nomodel) < 1e-12


def test_c1_config_matches_oracle_per_step(NS):
    """The plain-method configuration at its own size: DNS 128^3, nu = 1/2000,
    seeded peak spectrum k0 = 4 with unit energy, RK4 at CFL 0.3, exact
    closure every stage for a 32^3 volume-average LES (ratio 4).  The initial
    field and three RK4 steps of the DNS, the exact-closure LES and the
    no-model LES each agree with the NumPy oracle within 1e-12 relative L2."""
    n, c, l, visc, cfl = 128, 4, 1.0, 1 / 2000, 0.3
    cs = NS.Case(n, l, visc, cfl, les=[(c, "volume")])
    cs.init_random(4.0, 1.0, 0)
    u = ns.randomfield(n, l, 4.0, 0)
    assert rel(cs.velocity(), u) < 1e-12
    cs.set_velocity(u)  # both sides continue from the same bytes
    ol = [ns.Les(c=c, kind="volume")]
    tgt = ns.filtered_target(u, ol[0], l)
    ol[0].v_exact, ol[0].v_nomodel = tgt.copy(), tgt.copy()
    assert rel(cs.les(0, "target"), tgt) < 1e-12
    for step in range(3):
        cs.step(1)
        u, dts, _ = _one_step(u, visc, l, cfl, ol)
        assert rel(cs.velocity(), u) < 1e-12, step
        assert abs(cs.time()[1] - dts) <= 1e-14 * dts
        assert rel(cs.les(0, "exact"), ol[0].v_exact) < 1e-12, step
        assert rel(cs.les(0, "nomodel"), ol[0].v_nomodel) < 1e-12, step
    cs.close()


def _one_step(u, visc, l, cfl, les_list):
    """One step of ns.dnsaid_rk4 continuing existing LES states."""
    saved = [(le.v_exact, le.v_nomodel) for le in les_list]
    n = u.shape[1]
    h = l / n
    dt = ns.propose_timestep(u, visc, cfl, h)
    u0 = u
    ks = []
    les_k = [([], []) for _ in les_list]
    for s in range(4):
        us = u0 if s == 0 else u0 + (ns.RK4_A[s] * dt) * ks[-1]
        k, _ = ns.projected_rhs(us, visc, h)
        ks.append(k)
        for li, le in enumerate(les_list):
            H = l / (n // le.c)
            ub = ns.filtered_target(us, le, l)
            m = ns.closure(k, ub, visc, l, le.c, le.kind)
            ke, kn = les_k[li]
            ve = saved[li][0] if s == 0 else saved[li][0] + (ns.RK4_A[s] * dt) * ke[-1]
            vn = saved[li][1] if s == 0 else saved[li][1] + (ns.RK4_A[s] * dt) * kn[-1]
            ke.append(ns.project(ns.rhs(ve, visc, H), H) + m)
            kn.append(ns.project(ns.rhs(vn, visc, H), H))
    u = u0 + dt / 6 * (ks[0] + 2 * ks[1] + 2 * ks[2] + ks[3])
    for li, le in enumerate(les_list):
        ke, kn = les_k[li]
        le.v_exact = saved[li][0] + dt / 6 * (ke[0] + 2 * ke[1] + 2 * ke[2] + ke[3])
        le.v_nomodel = saved[li][1] + dt / 6 * (kn[0] + 2 * kn[1] + 2 * kn[2] + kn[3])
    return u, dt, None


def test_mediumcase_exact_closure_invariant(NS):
    """The reference's mediumcase grids (DNS 510^3, LES 102^3 and 170^3 by
    volume filters of ratio 5 and 3; radix 17 in every FFT): after two RK4
    steps the exact-closure LES equal the filtered DNS."""
    cs = NS.Case(510, 1.0, 5e-5, 0.3, les=[(5, "volume"), (3, "volume")])
    cs.init_random(5, 0.5, 123)
    cs.step(2)
    cs.sync()
    for i in range(2):
        e_exact, e_nomo = cs.errors(i)
        assert e_exact < 1e-12, (i, e_exact)
    cs.close()


def test_exact_closure_invariant_on_gpu(NS):
    """The exact-closure LES equals the filtered DNS after many steps
    (navierstokes.jl:33 records 5.69e-15 for the reference)."""
    n = 64
    cs = NS.Case(n, 1.0, 1 / 2000, 0.3, les=[(4, "volume"), (2, "face"), (8, "volume")])
    cs.init_random(4, 1.0, 0)
    cs.step(20)
    cs.sync()
    for i in range(3):
        e_exact, e_nomo = cs.errors(i)
        assert e_exact < 1e-12, (i, e_exact)
        assert e_nomo > 1e-4


def test_closure_snapshot_matches_oracle(NS):
    n, c, l, visc = 32, 4, 1.0, 1 / 1000
    u0 = ns.randomfield(n, l, 3, 4)
    cs = NS.Case(n, l, visc, 0.3, les=[(c, "volume")])
    cs.set_velocity(u0)
    cs.step(1)
    m = cs.les(0, "closure")
    k, _ = ns.projected_rhs(u0, visc, l / n)
    ub = ns.apply_DHpi(u0, c, l)
    ref = ns.closure(k, ub, visc, l, c, "volume")
    assert rel(m, ref) < 1e-12


def test_snapshot_pairs_round_trip(NS, tmp_path):
    """Pairs written every 2 steps equal the oracle's (ubar, m) at stage 1 of
    the corresponding steps, after a binary + JSON round trip."""
    from exactclosure_gb300 import snapshots

    n, c, l, visc = 32, 4, 1.0, 1 / 1000
    u0 = ns.randomfield(n, l, 3, 6)
    cs = NS.Case(n, l, visc, 0.3, les=[(c, "volume")])
    cs.set_velocity(u0)
    hp = snapshots.write_pairs(cs, 0, tmp_path, nsnap=2, every=2, stem="run")
    U, M, h = snapshots.read_pairs(hp)
    assert U.shape == (2, 3, 8, 8, 8) and h["ratio"] == c
    les = [ns.Les(c=c)]
    _, _, closures = ns.dnsaid_rk4(u0, visc, l, 0.3, 4, les, record_closure=True)
    for s in range(2):
        _, ub, m = closures[2 * s + 1]  # stage 1 of steps 2 and 4
        assert rel(U[s], ub) < 1e-12
        assert rel(M[s], m) < 1e-12


def test_fixed_dt_and_graph_replay(NS):
    n, l, visc = 16, 1.0, 1 / 500
    u0 = ns.randomfield(n, l, 3, 5)
    cs = NS.Case(n, l, visc, 0.3)
    cs.set_velocity(u0)
    cs.step(4, dt=1e-3)
    ref = u0
    for _ in range(4):
        ref = ns.step_rk4(ref, visc, l / n, 1e-3)
    assert rel(cs.velocity(), ref) < 1e-12
    t, dt = cs.time()
    assert abs(t - 4e-3) < 1e-15 and dt == 1e-3


def test_f32_precision_form_error_budget(NS):
    """FP32 stencil/filter/RK with FP64 divide and diagnostics, against FP64."""
    n, l, visc = 64, 1.0, 1 / 2000
    les = [(4, "volume")]
    c64 = NS.Case(n, l, visc, 0.3, precision=0, les=les)
    c32 = NS.Case(n, l, visc, 0.3, precision=1, les=les)
    c64.init_random(4, 1.0, 0)
    u0 = c64.velocity()
    c32.set_velocity(u0)
    for cs in (c64, c32):
        cs.step(20, dt=2e-4)
    assert rel(c32.velocity(), c64.velocity()) < 1e-4
    assert rel(c32.les(0, "closure"), c64.les(0, "closure")) < 1e-3
    s64, s32 = c64.spectrum(), c32.spectrum()
    assert rel(s32, s64) < 1e-4
    e_exact, _ = c32.errors(0)
    assert e_exact < 1e-4


def test_nonfinite_is_flagged(NS):
    from exactclosure_gb300 import ExcError

    n = 8
    cs = NS.Case(n, 1.0, 1 / 2000, 0.3)
    u = np.zeros((3, n, n, n))
    u[0, 0, 0, 0] = np.nan
    cs.set_velocity(u)
    cs.step(1)
    with pytest.raises(ExcError) as ei:
        cs.sync()
    assert ei.value.code == 6


@pytest.mark.parametrize("n", [32, 48, 64, 128])
def test_f32_dns_unaffected_by_les(NS, n):
    """An LES grid does not act on the DNS: with and without one (the RK stage
    then stores or skips the projected k, or forms the filter sums itself at
    n = 64, 128) the FP32 DNS matches bit for bit."""
    cf = NS.Case(n, 1.0, 1 / 2000, 0.3, precision=1)
    cu = NS.Case(n, 1.0, 1 / 2000, 0.3, precision=1, les=[(4, "volume")])
    u0 = ns.randomfield(n, 1.0, 4, 9)
    cf.set_velocity(u0)
    cu.set_velocity(u0)
    cf.step(5)
    cu.step(5)
    assert np.array_equal(cf.velocity(), cu.velocity())
    assert cf.time() == cu.time()


def test_f32_fused_filter_sums_match_separate_passes(NS):
    """FP32, 192^3: an LES of ratio 4 alone takes its filter sums from the RK
    stage kernel; next to an LES of ratio 3 (two root ratios) the same LES uses
    the separate box-sum passes.  Its exact-closure and no-model states agree
    bit for bit."""
    n = 192
    u0 = ns.randomfield(n, 1.0, 4, 5)
    fused = NS.Case(n, 1.0, 1 / 2000, 0.3, precision=1, les=[(4, "volume")])
    sep = NS.Case(n, 1.0, 1 / 2000, 0.3, precision=1, les=[(4, "volume"), (3, "volume")])
    for cs in (fused, sep):
        cs.set_velocity(u0)
        cs.step(2)
    assert np.array_equal(fused.velocity(), sep.velocity())
    for which in ("exact", "nomodel"):
        assert np.array_equal(fused.les(0, which), sep.les(0, which)), which
    fused.close()
    sep.close()
