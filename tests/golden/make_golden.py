"""Generate the golden vectors ``tests/golden/literal_n6.npz`` and ``literal_n12.npz``.

They come from ``oracle.literal``, the loop-for-loop restatement of the
reference's lazy-field operators (1-based ``mod1`` indexing, column-major 3-D
filter kernels; ``src/N.jl``), on a 6^3 grid with LES ratio 3 (the reference's
own odd-ratio regime) and on a 12^3 grid with ratio 3.  The reference itself (Julia) cannot run here, so these
fixtures pin the vectorised oracle and the CUDA path to the literal
semantics.  Run from the repository root: ``python tests/golden/make_golden.py``.
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import literal as L  # noqa: E402
from oracle import ns  # noqa: E402

c, l, visc, dt = 3, 1.0, 0.01, 1e-3


def make(n):
    h, H = l / n, l / (n // c)
    u = ns.counter_normal(7, 3 * n**3).reshape(3, n, n, n)
    u = np.stack([u[i] for i in range(3)])
    uL = [L.Field(L.from_ns(u[i])) for i in range(3)]
    zero = [L.Field(np.zeros((n,) * 3)) for _ in range(3)]
    rhs = L.tensordivergence(zero, L.stresstensor(uL, visc, h), h, False)
    div = L.divergence(uL, h)
    pu, p = L.project(uL, h)
    krhs, prhs = L.project(rhs, h)
    GDH, GDHi = L.get_kernels(c)
    ubar = L.apply_DHpi(uL, n // c, GDH, H)
    rdhi = L.get_rDHi(L.get_r(L.stresstensor(uL, visc, h), prhs), GDHi, n // c)
    sdh = L.get_sigmaDH(L.stresstensor(uL, visc, h), n // c, GDH)
    vL = [L.Field(ubar[i].data.copy()) for i in range(3)]
    cfd = L.step_classic_flux_div(vL, ubar, uL, prhs, visc, h, H, dt, GDHi)
    to = lambda fs: np.stack([L.to_ns(f.data) for f in fs])
    m = n // c
    out = dict(
        n=n, c=c, l=l, visc=visc, dt=dt, u=u,
        rhs=to(rhs), div=L.to_ns(div.data), proj=to(pu), p=L.to_ns(p.data),
        k=to(krhs), p_rhs=L.to_ns(prhs.data), ubar=to(ubar),
        rdhi=np.stack([L.to_ns(L.materialize(r, m).data) for r in rdhi]),
        sigmadh=np.stack([L.to_ns(L.materialize(s, m).data) for s in sdh]),
        cfd=to(cfd),
    )
    np.savez_compressed(Path(__file__).with_name(f"literal_n{n}.npz"), **out)
    print("wrote", n, {k: np.shape(v) for k, v in out.items()})


if __name__ == "__main__":
    for n in (6, 12):
        make(n)
