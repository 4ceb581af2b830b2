"""GPU parity at the precision-comparison size: DNS 512^3 in FP64 with the
exact closure for LES grids of ratio 8 (64^3) and 4 (128^3), against the C
restatement of the reference in the oracle (all host threads; a 512^3 RK4
step takes tens of seconds there).  Tolerance: 1e-12 relative L2."""
import numpy as np
import pytest

from oracle import build_cpu, cpu_ref

pytestmark = pytest.mark.gpu

N512 = 512


@pytest.fixture(scope="module")
def NS(built_lib):
    from exactclosure_gb300 import navierstokes

    return navierstokes


@pytest.fixture(scope="module")
def cref():
    build_cpu.build()
    if not cpu_ref.available():
        pytest.fail("the oracle's C restatement did not build")
    return cpu_ref


def rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def _field(n, seed):
    """A non-solenoidal float64 test field with energy at every wavenumber."""
    rng = np.random.default_rng(seed)
    return rng.standard_normal((3, n, n, n))


@pytest.mark.parametrize("engine", [0, 1])
def test_projection_512_f64_matches_c_oracle(NS, cref, engine):
    """project! (src/N.jl:256-307) at 512^3 in FP64 with the default engine
    (0: FP32 FFT solves refined by FP64 residuals) and the FP64 shared-memory
    Stockham passes (1), on a white-noise field."""
    import torch

    n = N512
    u = _field(n, 11)
    ref, pref = cref.project(u)
    g = NS.Grid(1.0, n)
    ps = NS.poissonsolver(g, engine=engine)
    ud = torch.from_numpy(u).cuda()
    pd = torch.empty((n, n, n), dtype=torch.float64, device="cuda")
    ps.project(ud, pd)
    torch.cuda.synchronize()
    assert rel(ud.cpu().numpy(), ref) < 1e-12
    # the pressure is defined up to its (zero) mean on both sides
    assert rel(pd.cpu().numpy(), pref) < 1e-12
    ps.close()
    del ud, pd
    torch.cuda.empty_cache()


def test_rhs_512_f64_matches_c_oracle(NS, cref):
    """tensordivergence(stresstensor(u)) (src/N.jl:94-160) at 512^3, FP64."""
    import torch

    n, visc = N512, 1 / 2000
    u = _field(n, 12)
    ref = cref.rhs(u, visc)
    ud = torch.from_numpy(u).cuda()
    du = torch.empty_like(ud)
    NS.tensordivergence(du, ud, visc, NS.Grid(1.0, n))
    torch.cuda.synchronize()
    assert rel(du.cpu().numpy(), ref) < 1e-12
    del ud, du
    torch.cuda.empty_cache()


def test_c2_config_rk4_step_matches_c_oracle(NS, cref):
    """One RK4 step of the precision-comparison configuration (DNS 512^3,
    nu = 1/2000, seeded peak spectrum k0 = 6, CFL 0.3, exact closure at
    every stage for 64^3 and 128^3 volume-average LES): the DNS, each LES's
    target, exact-closure and no-model states against the C oracle."""
    import torch

    n, visc, cfl = N512, 1 / 2000, 0.3
    les = [(8, "volume"), (4, "volume")]
    cs = NS.Case(n, 1.0, visc, cfl, les=les)
    cs.init_random(6.0, 1.0, 0)
    u0 = cs.velocity()
    cs.set_velocity(u0)
    oc = cref.CpuCase(n, 1.0, visc, cfl, les)
    oc.set_velocity(u0)
    for i in range(len(les)):
        assert rel(cs.les(i, "target"), oc.les_field(i, "target")) < 1e-12, i
    del u0
    cs.step(1)
    cs.sync()
    oc.step(1)
    assert rel(cs.velocity(), oc.velocity()) < 1e-12
    t, dt = cs.time()
    ct, cdt = C_time(cref, oc)
    assert abs(dt - cdt) <= 1e-14 * cdt and abs(t - ct) <= 1e-14 * ct
    for i in range(len(les)):
        for which in ("target", "exact", "nomodel"):
            assert rel(cs.les(i, which), oc.les_field(i, which)) < 1e-12, (i, which)
    oc.close()
    cs.close()
    torch.cuda.empty_cache()


def C_time(cref, oc):
    import ctypes as C

    t, dt = C.c_double(), C.c_double()
    assert cref.lib().cref_time(oc._h, C.byref(t), C.byref(dt)) == 0
    return t.value, dt.value
