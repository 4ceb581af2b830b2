"""CPU checks of the 1-D Burgers oracle (``oracle.burgers``): pinned to the
loop-for-loop restatement of ``dns_aided_les`` (``src/Burgers.jl:350-445``),
the exact-closure invariant, and the library's host-built filter kernels
against the oracle's (no GPU needed)."""
import math

import numpy as np
import pytest

from oracle import burgers as B
from oracle import literal as L

TWO_PI = 2 * math.pi


@pytest.mark.parametrize("nh,nH,ratio,kind", [(45, 9, 2.0, "gaussian"), (45, 15, 1.0, "tophat"),
                                              (45, 5, 0.0, "gaussian")])
def test_batched_oracle_matches_literal(nh, nH, ratio, kind):
    visc = 5e-3
    u0 = B.randomfields(2, nh, TWO_PI, 3, 2.0, 7)
    _, les, dbl = B.kernels(nh, nH, TWO_PI, ratio, kind)
    u, t, steps, V = B.dns_aided_les(u0, nH, visc, TWO_PI, ratio, kind, 0.03, 0.3)
    for s in range(2):
        lit = L.burgers_dns_aided_les(u0[s], nH, visc, TWO_PI, les, dbl, 0.03, 0.3)
        assert np.abs(u[s] - lit["dns_ref"]).max() <= 1e-13 * np.abs(lit["dns_ref"]).max()
        for k in B.LES_NAMES:
            assert np.abs(V[k][s] - lit[k]).max() <= 1e-13 * np.abs(lit[k]).max(), k
    assert (steps > 1).all() and np.allclose(t, 0.03, rtol=0, atol=1e-15)


def test_exact_closure_reproduces_filtered_dns():
    """The classic+flux+div LES equals the filtered DNS to round-off (the
    reference's claim for ``swapfil``), the others do not."""
    nh, nH, visc = 675, 45, 5e-4
    u0 = B.randomfields(3, nh, TWO_PI, 10, 2.0, 1)
    u, _, steps, V = B.dns_aided_les(u0, nH, visc, TWO_PI, 2.0, "gaussian", 0.05, 0.3)
    _, dfil = B.filtered_dns(u, nH, TWO_PI, 2.0, "gaussian")
    e = B.compute_errors(V, dfil)
    assert e["swapfil"] < 1e-13
    assert e["nomodel"] > 1e-3 and e["class_m"] > 1e-3 and e["class_p"] > 1e-4
    assert steps.min() > 20


def test_randomfield_energy_and_mean():
    u = B.randomfields(4, 1350, TWO_PI, 10, 2.0, 1)
    e = np.sum(u**2, axis=1) / 2 * (TWO_PI / 1350)
    assert np.allclose(e, 2.0, rtol=1e-13)
    assert np.abs(u.mean(axis=1)).max() < 1e-12  # no k = 0 mode


def test_rk4_order():
    """``rk4_timestep!`` is fourth order on a smooth field."""
    nh, visc = 64, 0.05
    u0 = B.randomfields(1, nh, TWO_PI, 2, 0.5, 3)
    h = TWO_PI / nh

    def run(dt, n):
        u = u0
        for _ in range(n):
            u = B.rk4_timestep(u, visc, h, dt)
        return u
    ref = run(0.0025, 40)
    e1 = np.abs(run(0.02, 5) - ref).max()
    e2 = np.abs(run(0.01, 10) - ref).max()
    assert 12 < e1 / e2 < 20


def test_smagorinsky_stages_as_written():
    """The reference's Smagorinsky RK4 accumulates its stages in the running
    state; with C = 0 it differs from classic RK4 by O(dt^3) per step."""
    nh, nH, visc = 135, 27, 1e-2
    u0 = B.randomfields(1, nh, TWO_PI, 3, 1.0, 5)
    ub, _, _ = B.solve_smagorinsky(u0, visc, TWO_PI, nH, 0.0, "gaussian", 0.0, 0.02, max_steps=1)
    _, _, dbl = B.kernels(nh, nH, TWO_PI, 0.0, "gaussian")
    v = B.coarse_filter(u0, dbl, nH, True)
    H = TWO_PI / nH
    dt = min(0.3 * B.cfl(v, visc, H)[0], 0.02)
    k1 = B.rhs(v, visc, H)
    k2 = B.rhs(v + dt / 2 * k1, visc, H)
    k3 = B.rhs(v + dt / 2 * (k1 + k2), visc, H)
    k4 = B.rhs(v + dt / 2 * (k1 + k2) + dt * k3, visc, H)
    ref = v + dt / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
    assert np.abs(ub - ref).max() < 1e-14


@pytest.mark.parametrize("nh,nH,ratio,kind", [(13500, 300, 2.0, "gaussian"), (13500, 2700, 2.0, "gaussian"),
                                              (13500, 900, 0.0, "gaussian"), (675, 45, 2.0, "tophat"),
                                              (675, 225, 1.0, "tophat")])
def test_library_kernels_match_oracle(built_lib, nh, nH, ratio, kind):
    """``exc_burgers_kernels`` builds the LES and double kernels on the host."""
    from exactclosure_gb300 import burgers as GB

    (rl, wl), (rd, wd) = GB.filter_kernels(GB.Grid(TWO_PI, nh), GB.Grid(TWO_PI, nH), ratio, kind)
    _, les, dbl = B.kernels(nh, nH, TWO_PI, ratio, kind)
    assert rl == les[0] and rd == dbl[0]
    assert np.abs(wl - les[1]).max() < 1e-16 and np.abs(wd - dbl[1]).max() < 1e-16


def test_library_rejects_even_compression(built_lib):
    from exactclosure_gb300 import ExcError
    from exactclosure_gb300 import burgers as GB

    with pytest.raises(ExcError) as ei:
        GB.filter_kernels(GB.Grid(TWO_PI, 600), GB.Grid(TWO_PI, 300), 2.0)
    assert ei.value.code == 3
    with pytest.raises(ExcError) as ei:
        GB.filter_kernels(GB.Grid(TWO_PI, 600), GB.Grid(TWO_PI, 7), 2.0)
    assert ei.value.code == 3


def test_c_port_matches_numpy_oracle():
    """The C/OpenMP Burgers restatement (the timed CPU baseline) against the
    NumPy oracle."""
    from oracle import build_cpu, cpu_ref

    if build_cpu.build() is None:
        pytest.skip("no C compiler")
    nh, nH, visc = 675, 45, 5e-4
    u0 = B.randomfields(3, nh, TWO_PI, 10, 2.0, 2)
    _, les, dbl = B.kernels(nh, nH, TWO_PI, 2.0, "gaussian")
    u, v, t, steps = cpu_ref.burgers_dnsaid(u0, nH, visc, TWO_PI, les[1], dbl[1], 0.05, 0.3)
    uo, to, so, V = B.dns_aided_les(u0, nH, visc, TWO_PI, 2.0, "gaussian", 0.05, 0.3)
    assert (steps == so).all()
    assert np.abs(u - uo).max() < 1e-11 * np.abs(uo).max()
    for k, name in enumerate(B.LES_NAMES):
        assert np.abs(v[:, k] - V[name]).max() < 1e-11 * np.abs(V[name]).max(), name
