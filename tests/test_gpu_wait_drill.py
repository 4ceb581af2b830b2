"""GPU tests of the bounded device waits' give-up path, made safe: a drill
flag makes the producer of a wait never start (the RHS sweep's TMA tiles and
the tensor-core convolution's load warp issue no copy, so no copy or product
is ever in flight), the waits give up after a few polls, the kernels finish,
the fault bit is set and the synchronising status call returns
EXC_ERR_TIMEOUT; afterwards the context is usable and results are correct."""
import numpy as np
import pytest

from oracle import ns

from exactclosure_gb300._lib import ExcError  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def NS(built_lib):
    from exactclosure_gb300 import navierstokes

    return navierstokes


def rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def sync_status():
    """(status, fault flags) of exc_device_sync on torch's current stream."""
    import ctypes as C

    import torch

    from exactclosure_gb300._lib import lib

    v = C.c_int(-1)
    rc = lib().exc_device_sync(C.c_void_p(torch.cuda.current_stream().cuda_stream), C.byref(v))
    return rc, v.value


# 192^3: both sweeps (FP32 2 x 2 kernel with 64-wide tiles, FP64 generic
# kernel) have interior tiles that take their planes by TMA
@pytest.mark.parametrize("prec", [1, 0])
def test_rhs_wait_gives_up_and_reports_timeout(NS, prec):
    import torch

    n, visc = 192, 1 / 2000
    g = NS.Grid(1.0, n)
    dtype = torch.float32 if prec == 1 else torch.float64
    u0 = np.random.default_rng(5).standard_normal((3, n, n, n))
    u = torch.tensor(u0, dtype=dtype, device="cuda")
    du = torch.empty_like(u)
    NS.device_sync()  # no stale fault bits
    NS.debug_wait_drill(1)
    try:
        NS.tensordivergence(du, u, visc, g)
        assert sync_status() == (7, 1)  # EXC_ERR_TIMEOUT, bit 0: the RHS sweep's plane wait
    finally:
        NS.debug_wait_drill(0)
    assert NS.device_faults() == 0  # the sync read and cleared the bit
    # the context is intact: the same sweep without the drill is correct
    NS.tensordivergence(du, u, visc, g)
    assert NS.device_sync() == 0
    with pytest.raises(ExcError):
        NS.debug_wait_drill(4)
    ref = ns.rhs(u.double().cpu().numpy(), visc, 1.0 / n)
    assert rel(du.double().cpu().numpy(), ref) < (1e-12 if prec == 0 else 2e-5)


def test_conv_wait_gives_up_and_reports_timeout(built_lib):
    """The tcgen05 convolution (64^3, 32 -> 32 channels, the hidden layer of
    the learned closure's forward pass): with its load warp drilled, the
    product lane and the epilogue warps give up, no product is issued, the
    tensor memory is freed; fault bit 1, EXC_ERR_TIMEOUT; the next forward
    pass equals one from before the drill."""
    import torch

    from exactclosure_gb300 import learned as LN
    from exactclosure_gb300 import navierstokes as NS

    net = LN.Net(seed=4)
    net.set_conv_engine(0)
    n, batch = 64, 1
    u = torch.tensor(np.random.default_rng(9).normal(0, 1.0, (batch, 3, n, n, n)), device="cuda",
                     dtype=torch.float32)
    before = torch.empty_like(u)
    net.forward(u, before)
    assert NS.device_sync() == 0
    out = torch.empty_like(u)
    NS.debug_wait_drill(2)
    try:
        net.forward(u, out)
        assert sync_status() == (7, 2)  # EXC_ERR_TIMEOUT, bit 1: the tensor-core convolution's waits
    finally:
        NS.debug_wait_drill(0)
    after = torch.empty_like(u)
    net.forward(u, after)
    assert NS.device_sync() == 0
    assert torch.equal(after, before)
    net.close()
