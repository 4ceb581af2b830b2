"""Learned closure over the libexc C ABI (``exc_net_*`` in include/exc.h): a
3-D convolutional net (3 -> 32 -> 32 -> 3 channels, periodic 3x3x3 kernels,
GELU) trained on (filtered velocity, exact closure) pairs with hand-written
BF16 tensor-core kernels.  No counterpart in the reference."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import EXC_F32, call, lib

# padded layer shapes (KP, NP) and the parameter layout [W1 b1 W2 b2 W3 b3]
SHAPES = ((16, 32), (32, 32), (32, 16))
VALID = ((3, 32), (32, 32), (32, 3))


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _stream():
    import torch

    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _prec(t):
    import torch

    return 0 if t.dtype == torch.float64 else 1


def unflatten(p: np.ndarray):
    """Parameter vector -> [(W[tap, ci, co], b[co]) x 3] with the valid channels."""
    out = []
    o = 0
    for (kp, np_), (ci, co) in zip(SHAPES, VALID):
        W = p[o:o + 27 * kp * np_].reshape(27, kp, np_)
        o += 27 * kp * np_
        b = p[o:o + np_]
        o += np_
        out.append((W[:, :ci, :co].copy(), b[:co].copy()))
    return out


def flatten(params) -> np.ndarray:
    parts = []
    for (kp, np_), (W, b) in zip(SHAPES, params):
        Wp = np.zeros((27, kp, np_), dtype=np.float32)
        Wp[:, :W.shape[1], :W.shape[2]] = W
        bp = np.zeros(np_, dtype=np.float32)
        bp[:b.shape[0]] = b
        parts += [Wp.ravel(), bp]
    return np.concatenate(parts).astype(np.float32)


def collect_pairs(case, les_index: int, nsnap: int, every: int = 1):
    """Step a DNS-aided case and keep (filtered DNS, exact closure) pairs on
    the device: tensors U, M shaped (nsnap, 3, m, m, m) in the case precision."""
    import torch

    m = case.n // case.les_list[les_index][0]
    dt = torch.float64 if case.desc.precision == 0 else torch.float32
    U = torch.empty((nsnap, 3, m, m, m), dtype=dt, device="cuda")
    M = torch.empty_like(U)
    for s in range(nsnap):
        case.step(every)
        case.snapshot(les_index, U[s], M[s])
    case.sync()
    return U, M


def train(net, U, M, steps: int, batch: int = 8, lr: float = 1e-3, seed: int = 0):
    """Adam on random minibatches of the pairs; returns the loss history.
    The input/output scales are the RMS of U and M."""
    import torch

    net.set_scales(float(U.double().pow(2).mean().sqrt()), float(M.double().pow(2).mean().sqrt()))
    g = torch.Generator(device="cpu").manual_seed(seed)
    losses = []
    for _ in range(steps):
        idx = torch.randint(0, U.shape[0], (batch,), generator=g).to(U.device)
        ub = U.index_select(0, idx).contiguous()
        mb = M.index_select(0, idx).contiguous()
        losses.append(net.train_step(ub, mb, lr))
    return losses


class Net:
    def __init__(self, seed: int = 0):
        h = C.c_void_p()
        call("exc_net_create", seed, C.byref(h))
        self._h = h
        self.count = lib().exc_net_param_count()
        self.in_scale = 1.0
        self.out_scale = 1.0

    def set_scales(self, in_scale: float, out_scale: float):
        self.in_scale, self.out_scale = in_scale, out_scale
        call("exc_net_set_scales", self._h, in_scale, out_scale)

    def set_conv_engine(self, engine: int):
        """0: tcgen05 tensor-core convolutions on 64^3 grids (default);
        1: mma.sync convolutions everywhere."""
        call("exc_net_set_conv_engine", self._h, int(engine))

    def get_params(self) -> np.ndarray:
        a = np.empty(self.count, dtype=np.float32)
        call("exc_net_get_params", self._h, a.ctypes.data_as(C.POINTER(C.c_float)), self.count)
        return a

    def set_params(self, p: np.ndarray):
        a = np.ascontiguousarray(p, dtype=np.float32)
        call("exc_net_set_params", self._h, a.ctypes.data_as(C.POINTER(C.c_float)), self.count)

    def forward(self, u, out):
        """out = net(u); u, out CUDA tensors [batch, 3, n, n, n]."""
        call("exc_net_forward", self._h, _prec(u), u.shape[0], u.shape[2], _ptr(u), _ptr(out), _stream())
        return out

    def gradients(self, u, m):
        g = np.empty(self.count, dtype=np.float32)
        loss = C.c_double()
        call("exc_net_gradients", self._h, _prec(u), u.shape[0], u.shape[2], _ptr(u), _ptr(m),
             g.ctypes.data_as(C.POINTER(C.c_float)), C.byref(loss), _stream())
        return loss.value, g

    def train_step(self, u, m, lr: float = 1e-3) -> float:
        loss = C.c_double()
        call("exc_net_train_step", self._h, _prec(u), u.shape[0], u.shape[2], _ptr(u), _ptr(m), lr, C.byref(loss),
             _stream())
        return loss.value

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            lib().exc_net_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
