"""GPU parity of the reference's own driver ``dnsaid_project``
(``exc_dnsaid_*``, src/N.jl:1239-1332) against the oracle: the power-law
random field, the forward-Euler warm-up, the LES start and the lockstep of
the DNS with the five LES (no model, classic, classic+flux,
classic+flux+div, symmetrised), 1e-12 relative per step; the exact closure
reproduces the filtered DNS (navierstokes.jl:33 records 5.69e-15)."""
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


def test_power_profile_field(NS):
    n = 48
    d = NS.DnsAid(n, 1.0, 1e-3, 3)
    d.init_random("power", -5 / 3, 1.0, 4)
    ref = ns.randomfield(n, 1.0, -5 / 3, 4, 1.0, profile="power")
    assert rel(d.velocity(), ref) < 1e-12


@pytest.mark.parametrize("n,c,use_fdelta", [(48, 3, False), (48, 3, True), (54, 3, True)])
def test_warmup_start_and_lockstep_per_step(NS, n, c, use_fdelta):
    l, visc, cfl = 1.0, 1e-3, 0.4
    m = n // c
    fdelta = ns.gaussian(l / n, 2 * l / m, 2) if use_fdelta else None
    u0 = ns.randomfield(n, l, -5 / 3, 1, 1.0, profile="power")
    d = NS.DnsAid(n, l, visc, c, fdelta)
    d.set_velocity(u0)
    u, t = u0, 0.0
    for k in range(2):
        d.warmup(0.05, cfl, max_steps=1)
        u, t, _ = ns.dnsaid_warmup(u, visc, l, 0.05, cfl, max_steps=1, t0=t)
        assert rel(d.velocity(), u) < 1e-12, k
        assert abs(d.time()[0] - t) <= 1e-15
    d.start()
    les = ns.dnsaid_start(u, l, c, fdelta)
    for key in ns.DNSAID_NAMES:
        assert rel(d.get(key), les[key]) < 1e-12
    t = 0.0
    for k in range(3):
        d.step(0.05, cfl, max_steps=1)
        u, les, t, _ = ns.dnsaid_project_steps(u, les, visc, l, c, 0.05, cfl, fdelta, max_steps=1, t0=t)
        assert rel(d.velocity(), u) < 1e-12, k
        for key in ns.DNSAID_NAMES:
            assert rel(d.get(key), les[key]) < 1e-12, (k, key)
    assert rel(d.get("u_les"), ns.apply_DHpi(u, c, l, fdelta)) < 1e-12


@pytest.mark.parametrize("doproject", [True, False])
def test_paper_volavg_driver_per_step(NS, doproject):
    """The paper's dns_aid_volavg (src/NavierStokes.jl:141-304): start and
    three lockstep steps against the oracle (1e-12); the swap closure (face-
    filtered flux) keeps its LES on the filtered DNS to round-off."""
    n, c, l, visc, cfl = 30, 3, 1.0, 1e-3, 0.4
    u = ns.randomfield(n, l, -5 / 3, 2, 1.0, profile="power")
    d = NS.DnsAid(n, l, visc, c)
    d.set_velocity(u)
    d.set_paper(doproject)
    d.start()
    fu = ns.paper_volavg_target(u, l, c, doproject)
    les = {k: fu.copy() for k in ns.PAPER_NAMES}
    assert rel(d.get("fu"), fu) < 1e-12
    t = 0.0
    for k in range(3):
        d.step(0.05, cfl, max_steps=1)
        u, les, t, _ = ns.dns_aid_volavg_steps(u, les, visc, l, c, 0.05, cfl, doproject, max_steps=1, t0=t)
        assert rel(d.velocity(), u) < 1e-12, k
        for key in ns.PAPER_NAMES:
            assert rel(d.get(key), les[key]) < 1e-12, (k, key)
    e = d.errors()
    assert e["swapfil"] < 1e-13
    for key in ("nomodel", "classic", "swapfil_symm"):
        assert e[key] > 1e-4, key
    d.close()


def test_paper_volavg_host_driver(NS):
    """The reference-shaped driver ``dns_aid_volavg(...) -> (u, relerr)``:
    relative errors at t = 0 and after each step against the oracle's LES,
    the swap closure on the filtered DNS to round-off."""
    n, m, l, visc, cfl, tstop = 30, 10, 1.0, 1e-3, 0.4, 0.004
    u0 = ns.randomfield(n, l, -5 / 3, 3, 1.0, profile="power")
    u, rel_err = NS.dns_aid_volavg(u0, m, visc, True, tstop, cfl, l)
    fu = ns.paper_volavg_target(u0, l, 3, True)
    les = {k: fu.copy() for k in ns.PAPER_NAMES}
    uo, les, t, it = ns.dns_aid_volavg_steps(u0, les, visc, l, 3, tstop, cfl, True)
    assert len(rel_err["time"]) == it + 1 and abs(rel_err["time"][-1] - t) <= 1e-15
    assert rel(u["dns_ref"], uo) < 1e-12
    ref = ns.paper_volavg_target(uo, l, 3, True)
    for k in ns.PAPER_NAMES:
        assert rel(u[k], les[k]) < 1e-12, k
        assert abs(rel_err[k][-1] - rel(les[k], ref)) <= 1e-10 * max(rel(les[k], ref), 1e-30) + 1e-14, k
    assert rel_err["swapfil"].max() < 1e-13
    assert rel_err["nomodel"][0] == 0.0 and rel_err["nomodel"][-1] > 1e-6


def test_exact_closure_invariant_and_errors(NS):
    setup = NS.getsetup(n_dns=72, n_les=24, twarm=0.02, tstop=0.02, visc=1e-3)
    out = NS.dnsaid_project(setup)
    e = out["errors"]
    assert e["u_cfd"] < 1e-13
    for k in ("u_nomo", "u_c", "u_cf", "u_cfd_symm"):
        assert e[k] > 1e-4, k
    eh = NS.compute_errors(out)
    for k in e:
        assert abs(eh[k] - e[k]) <= 1e-10 * max(e[k], 1e-30) + 1e-15


def test_even_ratio_rejected(NS):
    """dnsaid_project's classic closure filters on the fine grid with an odd
    top-hat only: an even ratio is refused at start (the paper drivers take
    it)."""
    from exactclosure_gb300 import ExcError

    d = NS.DnsAid(48, 1.0, 1e-3, 4)
    d.set_velocity(ns.randomfield(48, 1.0, 3, 0))
    with pytest.raises(ExcError) as ei:
        d.start()
    assert ei.value.code == 3
    d.close()


@pytest.mark.parametrize("c,doproject", [(3, True), (3, False), (4, True)])
def test_paper_surface_driver_per_step(NS, c, doproject):
    """The paper's dns_aid_surface (src/NavierStokes.jl:306-468): the face-
    filtered target, start and three lockstep steps of the DNS and the four
    LES against the oracle (1e-12 relative L2 per step); the device relerr
    equals the oracle's |v - fiu| / |fiu|."""
    n, l, visc, cfl = 24, 1.0, 1e-3, 0.4
    u = ns.randomfield(n, l, -5 / 3, 2, 1.0, profile="power")
    d = NS.DnsAid(n, l, visc, c)
    d.set_velocity(u)
    d.set_paper(doproject, "surface")
    d.start()
    fiu = ns.face_filter(u, c)
    les = {k: fiu.copy() for k in ns.PAPER_NAMES}
    assert rel(d.get("fu"), fiu) < 1e-12
    t = 0.0
    for k in range(3):
        d.step(0.05, cfl, max_steps=1)
        u, les, t, _ = ns.dns_aid_surface_steps(u, les, visc, l, c, 0.05, cfl, doproject, max_steps=1, t0=t)
        assert rel(d.velocity(), u) < 1e-12, k
        for key in ns.PAPER_NAMES:
            assert rel(d.get(key), les[key]) < 1e-12, (k, key)
    ref = ns.face_filter(u, c)
    e = d.relerr()
    for key in ns.PAPER_NAMES:
        assert abs(e[key] - rel(les[key], ref)) <= 1e-10 * rel(les[key], ref), key
    d.close()


def test_paper_surface_host_driver(NS):
    """The reference-shaped ``dns_aid_surface(...) -> (u, relerr)``: relerr
    at t = 0 and after every step against the oracle, and an empty relerr
    when tstop <= 0 (the reference's `while t < tstop` loop)."""
    n, m, l, visc, cfl, tstop = 24, 8, 1.0, 1e-3, 0.4, 0.004
    u0 = ns.randomfield(n, l, -5 / 3, 3, 1.0, profile="power")
    u, rel_err = NS.dns_aid_surface(u0, m, visc, True, tstop, cfl, l)
    fiu = ns.face_filter(u0, 3)
    les = {k: fiu.copy() for k in ns.PAPER_NAMES}
    uo, les, t, it = ns.dns_aid_surface_steps(u0, les, visc, l, 3, tstop, cfl, True)
    assert len(rel_err["time"]) == it + 1 and abs(rel_err["time"][-1] - t) <= 1e-15
    assert rel(u["dns_ref"], uo) < 1e-12
    assert rel(u["dns_fil"], ns.face_filter(uo, 3)) < 1e-12
    ref = ns.face_filter(uo, 3)
    for k in ns.PAPER_NAMES:
        assert rel(u[k], les[k]) < 1e-12, k
        assert abs(rel_err[k][-1] - rel(les[k], ref)) <= 1e-10 * rel(les[k], ref), k
    assert rel_err["nomodel"][0] == 0.0
    u_empty, r_empty = NS.dns_aid_surface(u0, m, visc, True, 0.0, cfl, l)
    assert all(len(v) == 0 for v in r_empty.values())
    assert rel(u_empty["dns_fil"], fiu) < 1e-12
    with pytest.raises(ValueError):
        NS.dns_aid_surface(u0, 7, visc, True, tstop, cfl, l)


def test_reference_ratio_5_grid(NS):
    """The reference's own dnsaid_project setup uses n_dns = 500, n_les = 100
    (ratio 5, src/N.jl:718); the radix-5 FFT runs the same ratio here at
    n = 50 -> 10 against the oracle, one warm-up and two lockstep steps."""
    n, c, l, visc, cfl = 50, 5, 1.0, 2e-4, 0.4
    m = n // c
    fdelta = ns.gaussian(l / n, 2 * l / m, 2)
    u0 = ns.randomfield(n, l, -5 / 3, 3, 1.0, profile="power")
    d = NS.DnsAid(n, l, visc, c, fdelta)
    d.set_velocity(u0)
    d.warmup(1.0, cfl, max_steps=1)
    u, t, _ = ns.dnsaid_warmup(u0, visc, l, 1.0, cfl, max_steps=1)
    assert rel(d.velocity(), u) < 1e-12
    d.start()
    les = ns.dnsaid_start(u, l, c, fdelta)
    d.step(1.0, cfl, max_steps=2)
    u, les, _, _ = ns.dnsaid_project_steps(u, les, visc, l, c, 1.0, cfl, fdelta, max_steps=2)
    assert rel(d.velocity(), u) < 1e-12
    for key in ns.DNSAID_NAMES:
        assert rel(d.get(key), les[key]) < 1e-12, key
