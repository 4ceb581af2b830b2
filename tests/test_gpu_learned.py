"""GPU checks of the learned-closure kernels against the CPU oracle
(oracle/net.py): forward outputs and loss gradients with the same BF16
roundings emulated on the CPU (relative L2 within 2e-3), one Adam step, and
training that lowers the loss."""
import numpy as np
import pytest

from oracle import net as onet

pytestmark = pytest.mark.gpu


def bf16(x):
    """Round to bfloat16 (nearest even), returned as float64."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def to_cl(f):
    """[b, 3, n, n, n] fields -> channel-last [b, z, y, x, 3]."""
    return np.ascontiguousarray(np.moveaxis(f, 1, -1))


def emulated(params, u, m, in_scale, out_scale):
    """Forward and gradients with the GPU's BF16 roundings (FP64 sums)."""
    x0 = bf16(to_cl(u) / in_scale)
    Ws = [(bf16(W), b.astype(np.float64)) for W, b in params]
    pre1 = onet.conv(x0, *Ws[0])
    a1 = bf16(onet.gelu(pre1))
    pre2 = onet.conv(a1, *Ws[1])
    a2 = bf16(onet.gelu(pre2))
    out = onet.conv(a2, *Ws[2])
    tgt = to_cl(m) / out_scale
    diff = out - tgt
    loss = float(np.mean(diff * diff))
    g3 = bf16(2.0 * diff / diff.size)
    _, dW3, db3 = onet.conv_backward(a2, Ws[2][0], g3)
    dx3, _, _ = onet.conv_backward(a2, Ws[2][0], g3)
    # the forward pass keeps GELU'(pre) in BF16 for the backward pass
    gp2 = bf16(dx3 * bf16(onet.gelu_grad(pre2)))
    dx2, dW2, db2 = onet.conv_backward(a1, Ws[1][0], gp2)
    gp1 = bf16(dx2 * bf16(onet.gelu_grad(pre1)))
    _, dW1, db1 = onet.conv_backward(x0, Ws[0][0], gp1)
    return out, loss, [(dW1, db1), (dW2, db2), (dW3, db3)]


@pytest.fixture(scope="module")
def LN(built_lib):
    from exactclosure_gb300 import learned

    return learned


def setup_net(LN, seed=3):
    net = LN.Net(seed=seed)
    params = onet.init_params(seed)
    params = [(bf16(W), np.random.default_rng(seed + i).normal(0, 0.1, b.shape)) for i, (W, b) in enumerate(params)]
    net.set_params(LN.flatten(params))
    params = LN.unflatten(net.get_params().astype(np.float64))
    return net, params


# n = 8: weight-resident convolutions and per-block weight gradients; 12: the
# 4^3-tile convolution and per-tap weight gradients; 10: the row-form
# convolution; 64: the tcgen05 convolutions (tensor-memory accumulators)
@pytest.mark.parametrize("n,batch", [(8, 2), (12, 1), (10, 1), (64, 1)])
def test_forward_and_gradients_match_oracle(LN, n, batch):
    import torch

    from exactclosure_gb300 import navierstokes as NS

    NS.device_faults()

    net, params = setup_net(LN)
    rng = np.random.default_rng(n)
    u = rng.normal(0, 1.3, (batch, 3, n, n, n))
    m = rng.normal(0, 40.0, (batch, 3, n, n, n))
    net.set_scales(1.3, 40.0)
    ut = torch.tensor(u, device="cuda")
    mt = torch.tensor(m, device="cuda")
    out = torch.empty_like(ut)
    net.forward(ut, out)
    torch.cuda.synchronize()
    ref_out, ref_loss, ref_grads = emulated(params, u, m, 1.3, 40.0)
    got = out.cpu().numpy()
    assert rel(to_cl(got) / 40.0, ref_out) < 2e-3
    loss, g = net.gradients(ut, mt)
    assert abs(loss - ref_loss) < 2e-3 * ref_loss
    gp = LN.unflatten(g.astype(np.float64))
    for l in range(3):
        assert rel(gp[l][0], ref_grads[l][0]) < 2e-3, l
        assert rel(gp[l][1], ref_grads[l][1]) < 2e-3, l
    assert NS.device_faults() == 0
    net.close()


def test_conv_engines_agree(LN):
    """On a 64^3 grid the tcgen05 convolutions and the mma.sync ones give the
    same forward output and gradients up to FP32 summation order (and the BF16
    roundings of activations it can flip)."""
    import torch

    from exactclosure_gb300 import navierstokes as NS

    NS.device_faults()
    net, _ = setup_net(LN, seed=3)
    n, batch = 64, 2
    rng = np.random.default_rng(7)
    u = torch.tensor(rng.normal(0, 1.0, (batch, 3, n, n, n)), device="cuda", dtype=torch.float32)
    m = torch.tensor(rng.normal(0, 30.0, (batch, 3, n, n, n)), device="cuda", dtype=torch.float32)
    net.set_scales(1.0, 30.0)
    res = []
    for engine in (0, 1):
        net.set_conv_engine(engine)
        out = torch.empty_like(u)
        net.forward(u, out)
        loss, g = net.gradients(u, m)
        torch.cuda.synchronize()
        res.append((out.double().cpu().numpy(), loss, g.astype(np.float64)))
    (o0, l0, g0), (o1, l1, g1) = res
    assert rel(o0, o1) < 1e-3
    assert abs(l0 - l1) < 1e-4 * l1
    assert rel(g0, g1) < 1e-3
    assert NS.device_faults() == 0
    with pytest.raises(Exception):
        net.set_conv_engine(2)
    net.close()


def test_adam_step_matches_oracle(LN):
    import torch

    net, params = setup_net(LN, seed=5)
    n = 8
    rng = np.random.default_rng(1)
    u = torch.tensor(rng.normal(size=(1, 3, n, n, n)), device="cuda")
    m = torch.tensor(rng.normal(size=(1, 3, n, n, n)), device="cuda")
    p0 = net.get_params().astype(np.float64)
    _, g = net.gradients(u, m)
    net.train_step(u, m, lr=1e-3)
    p1 = net.get_params().astype(np.float64)
    grads = LN.unflatten(g.astype(np.float64))
    ref = onet.adam_step(LN.unflatten(p0), grads, {}, lr=1e-3)
    got = LN.unflatten(p1)
    for l in range(3):
        assert np.allclose(got[l][0], ref[l][0], atol=1e-6, rtol=1e-5)
        assert np.allclose(got[l][1], ref[l][1], atol=1e-6, rtol=1e-5)
    net.close()


def test_learned_closure_beats_no_model_les(LN):
    """Train on (filtered DNS, exact closure) pairs of a GPU DNS-aided run,
    then run an LES with the learned closure from the filtered DNS of a later
    time: its closure error against the exact closure is below the no-model
    closure's (100%), and its velocity error against the filtered DNS is below
    the no-model LES's."""
    import torch

    from exactclosure_gb300 import navierstokes as NS

    n, c = 128, 4
    cs = NS.Case(n, 1.0, 1 / 2000, 0.3, precision=1, les=[(c, "volume")])
    cs.init_random(4.0, 1.0, 0)
    cs.step(10)
    U, M = LN.collect_pairs(cs, 0, nsnap=96, every=1)
    net = LN.Net(seed=1)
    losses = LN.train(net, U[:80], M[:80], steps=400, batch=8, lr=1e-3)
    assert losses[-1] < losses[0]
    # closure error on held-out pairs
    pred = torch.empty_like(U[80:])
    net.forward(U[80:].contiguous(), pred)
    torch.cuda.synchronize()
    e_closure = float((pred - M[80:]).double().norm() / M[80:].double().norm())
    assert e_closure < 0.9
    # LES with the learned closure vs no model, from the filtered DNS
    cs.reset_les()
    cs.attach_net(0, net)
    cs.step(40)
    cs.sync()
    e_learned = cs.les_error(0, "learned")
    e_nomodel = cs.les_error(0, "nomodel")
    e_exact = cs.les_error(0, "exact")
    assert e_exact < 1e-4
    assert e_learned < e_nomodel, (e_learned, e_nomodel)
    net.close()


def test_training_lowers_the_loss(LN):
    """Fit a target produced by another network of the same shape."""
    import torch

    teacher, _ = setup_net(LN, seed=11)
    student = LN.Net(seed=12)
    n, batch = 16, 4
    rng = np.random.default_rng(2)
    u = torch.tensor(rng.normal(size=(batch, 3, n, n, n)), device="cuda", dtype=torch.float32)
    m = torch.empty_like(u)
    teacher.forward(u, m)
    losses = [student.train_step(u, m, lr=3e-3) for _ in range(150)]
    assert losses[-1] < 0.5 * losses[0]
    assert all(np.isfinite(losses))
    teacher.close()
    student.close()


def test_learned_les_fallback_to_no_model(LN):
    """The no-model fallback of the learned-closure LES.  A net whose output
    is zero leaves the learned LES equal to the no-model LES bit for bit and
    the fallback idle; a net scaled to blow the LES up trips the energy band:
    the state goes back to the last one inside the band and the LES runs on
    without the net, finite and inside the band; a reset disengages it."""
    from exactclosure_gb300 import navierstokes as NS

    n, c = 64, 4
    cs = NS.Case(n, 1.0, 1 / 2000, 0.3, precision=1, les=[(c, "volume")])
    cs.init_random(4.0, 1.0, 0)
    net = LN.Net(seed=2)
    net.set_params(np.zeros(net.count, dtype=np.float32))
    cs.reset_les()
    cs.attach_net(0, net)
    cs.step(5)
    cs.sync()
    assert np.array_equal(cs.les(0, "learned"), cs.les(0, "nomodel"))
    assert not cs.fallback_engaged(0)
    # a net whose closure term is about 1e6 times the velocity
    bad = LN.Net(seed=3)
    bad.set_scales(1.0, 1e6)
    e0 = 0.5 * float(np.mean(cs.les(0, "nomodel") ** 2)) * 3
    cs.reset_les()
    cs.attach_net(0, bad)
    cs.set_fallback(0, 0.0, 4.0 * e0)
    cs.step(3)
    cs.sync()
    assert cs.fallback_engaged(0)
    v = cs.les(0, "learned")
    assert np.all(np.isfinite(v))
    assert 0.5 * float(np.mean(v ** 2)) * 3 <= 4.0 * e0
    # without the net's term it runs on like a no-model LES: finite, in the band
    cs.step(2)
    cs.sync()
    assert cs.fallback_engaged(0)
    v = cs.les(0, "learned")
    assert np.all(np.isfinite(v)) and 0.5 * float(np.mean(v ** 2)) * 3 <= 4.0 * e0
    # a reset disengages it
    cs.reset_les()
    assert not cs.fallback_engaged(0)
    net.close()
    bad.close()
    cs.close()
