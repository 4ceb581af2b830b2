"""GPU parity of the Poisson solver's FFT engines: the register-resident
passes (engine 2, and engine 0 where no mixed-precision solve is built), the
mixed-precision FP64 solve (engine 0 on FP64 grids of 128 and more) and the
shared-memory Stockham passes (engine 1).  Projection and pressure solve
against the oracle (float64: 1e-12 relative; float32 form: 2e-5), and, at grids
too large for the oracle, against each other."""
import numpy as np
import pytest

from oracle import ns

pytestmark = pytest.mark.gpu
TOL64 = 1e-12
TOL32 = 2e-5


@pytest.fixture(scope="module")
def NS(built_lib):
    from exactclosure_gb300 import navierstokes

    return navierstokes


def dev(a, dtype="float64"):
    import torch

    return torch.tensor(np.ascontiguousarray(a), dtype=getattr(torch, dtype), device="cuda")


def host(t):
    import torch

    torch.cuda.synchronize()
    return t.double().cpu().numpy()


def rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


@pytest.mark.parametrize("n,engine", [(32, 0), (48, 0), (64, 0), (96, 0), (128, 2), (128, 0), (192, 0)])
def test_register_projection_f64(NS, n, engine):
    import torch

    l = 2.0
    u = np.random.default_rng(n).standard_normal((3, n, n, n))
    ps = NS.poissonsolver(NS.Grid(l, n), engine=engine)
    ut = dev(u)
    p = torch.empty((n, n, n), dtype=torch.float64, device="cuda")
    ps.project(ut, p)
    ref, pref = ns.project(u, l / n, return_p=True)
    assert rel(host(ut), ref) < TOL64
    assert rel(host(p), pref) < TOL64
    # scalar right-hand side (no fused divergence)
    d = dev(np.random.default_rng(n + 1).standard_normal((n, n, n)))
    q = torch.empty_like(d)
    ps.solve(q, d)
    assert rel(host(q), ns.poisson_solve(host(d), l / n)) < TOL64


@pytest.mark.parametrize("n", [32, 48, 64, 96, 128, 192])
def test_register_projection_f32(NS, n):
    l = 1.0
    u = np.random.default_rng(n).standard_normal((3, n, n, n)).astype(np.float32).astype(np.float64)
    ps = NS.poissonsolver(NS.Grid(l, n), precision=1, engine=0)
    ut = dev(u, "float32")
    ps.project(ut)
    assert rel(host(ut), ns.project(u, l / n)) < TOL32


def engines_agree(NS, n, precision, tol, seed=0, engines=(0, 1)):
    import torch

    dt = "float64" if precision == 0 else "float32"
    g = NS.Grid(1.0, n)
    gen = torch.Generator(device="cuda").manual_seed(seed)
    u = torch.randn((3, n, n, n), generator=gen, device="cuda", dtype=getattr(torch, dt))
    out = []
    for engine in engines:
        ps = NS.poissonsolver(g, precision=precision, engine=engine)
        ut = u.clone()
        p = torch.empty((n, n, n), dtype=u.dtype, device="cuda")
        ps.project(ut, p)
        torch.cuda.synchronize()
        out.append((ut, p))
        ps.close()
    (ua, pa), (ub, pb) = out[0], out[-1]
    eu = float(torch.linalg.vector_norm((ua - ub).double()) / torch.linalg.vector_norm(ub.double()))
    ep = float(torch.linalg.vector_norm((pa - pb).double()) / torch.linalg.vector_norm(pb.double()))
    assert eu < tol and ep < tol, (n, eu, ep)
    # the projected field is divergence free on the grid
    d = torch.empty((n, n, n), dtype=u.dtype, device="cuda")
    NS.divergence(d, ua, g)
    scale = float(torch.linalg.vector_norm(u.double())) * n
    assert float(torch.linalg.vector_norm(d.double())) < (1e-11 if precision == 0 else 2e-5) * scale


@pytest.mark.parametrize("n", [192, 256])
def test_register_engine_matches_stockham_f64(NS, n):
    engines_agree(NS, n, 0, TOL64, engines=(2, 1))


@pytest.mark.parametrize("n", [192, 256, 384, 1024])
def test_mixed_precision_engine_matches_stockham_f64(NS, n):
    """The mixed-precision FP64 solve (FP32 FFT solves refined by FP64
    residuals) against the FP64 Stockham passes, on a white-noise field (the
    hardest right-hand side for the refinement: no decay in the spectrum)."""
    engines_agree(NS, n, 0, TOL64, engines=(0, 1))


@pytest.mark.parametrize("n", [256, 384, 512, 1024])
def test_register_engine_matches_stockham_f32(NS, n):
    engines_agree(NS, n, 1, 1e-5)


def test_engine_argument_checked(NS):
    from exactclosure_gb300 import ExcError

    with pytest.raises(ExcError):
        NS.poissonsolver(NS.Grid(1.0, 32), engine=3)
