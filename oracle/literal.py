"""Loop-for-loop restatement of the reference's lazy-field operators.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).  Pure Python, for grids
of a few cells per side: it pins the vectorised oracle ``oracle.ns`` to the
reference's exact index conventions.  It keeps the reference's 1-based
``CartesianIndex`` arithmetic with the periodic ``mod1`` wrap
(``src/N.jl:64-77``), its lazy fields evaluated per access
(``src/N.jl:49-72``), its 3-D filter kernels iterated in column-major order
(``lazyfilter``, ``src/N.jl:655-668``) and its coarse-grain sample point
``factor*Ibar - !stag*a`` (``src/N.jl:686-698``).

Fields are NumPy arrays indexed in the reference's order ``A[i1, i2, i3]``
(0-based storage, 1-based access through ``get``); ``from_ns``/``to_ns``
convert to and from the ``[z, y, x]`` arrays of ``oracle.ns``.
"""
from __future__ import annotations

import itertools

import numpy as np


def from_ns(a):
    return np.ascontiguousarray(np.asarray(a).transpose(2, 1, 0))


def to_ns(a):
    return np.ascontiguousarray(np.asarray(a).transpose(2, 1, 0))


def mod1(i, n):
    return (i - 1) % n + 1


class Field:
    """Materialised periodic field (``Field``, ``src/N.jl:34-42``)."""

    def __init__(self, data):
        self.data = data
        self.n = data.shape[0]

    def __getitem__(self, I):
        n = self.n
        return self.data[mod1(I[0], n) - 1, mod1(I[1], n) - 1, mod1(I[2], n) - 1]


class Lazy:
    """``LazyField``: evaluates ``func(I)`` at every access (``src/N.jl:49-72``)."""

    def __init__(self, func, n):
        self.func = func
        self.n = n

    def __getitem__(self, I):
        return self.func(I)


def right(I, i, r):
    """``right(I, i, r)`` (``src/N.jl:79-80``), ``i`` 1-based."""
    return tuple(I[j] + r if j + 1 == i else I[j] for j in range(3))


def stress(u, visc, h, i, j):
    """``stress(u, visc, i, j)`` (``src/N.jl:106-118``), ``i, j`` 1-based."""

    def f(I):
        ui_rightj = u[i - 1][right(I, j, int(i != j))]
        ui_leftj = u[i - 1][right(I, j, int(i != j) - 1)]
        uj_righti = u[j - 1][right(I, i, int(j != i))]
        uj_lefti = u[j - 1][right(I, i, int(j != i) - 1)]
        etaj_ui = (ui_rightj + ui_leftj) / 2
        etai_uj = (uj_righti + uj_lefti) / 2
        dj_ui = (ui_rightj - ui_leftj) / h
        di_uj = (uj_righti - uj_lefti) / h
        return etaj_ui * etai_uj - visc * (dj_ui + di_uj)

    return Lazy(f, u[0].n)


def stresstensor(u, visc, h):
    """``(s11, s22, s33, s12, s23, s31)`` (``src/N.jl:94-104``)."""
    return tuple(stress(u, visc, h, i, j) for i, j in ((1, 1), (2, 2), (3, 3), (1, 2), (2, 3), (3, 1)))


def _cells(n):
    return itertools.product(range(1, n + 1), repeat=3)


def tensordivergence(du, s, h, doadd):
    """``tensordivergence!`` (``src/N.jl:120-160``), in place on ``du`` data."""
    s11, s22, s33, s12, s23, s31 = s
    s21, s32, s13 = s12, s23, s31
    n = du[0].n
    out = [d.data.copy() for d in du]
    for I in _cells(n):
        I1, I2, I3 = I
        g = lambda k: (du[k][I] if doadd else 0.0)
        out[0][I1 - 1, I2 - 1, I3 - 1] = (g(0) - (s11[(I1 + 1, I2, I3)] - s11[I]) / h
                                          - (s12[I] - s12[(I1, I2 - 1, I3)]) / h
                                          - (s13[I] - s13[(I1, I2, I3 - 1)]) / h)
        out[1][I1 - 1, I2 - 1, I3 - 1] = (g(1) - (s21[I] - s21[(I1 - 1, I2, I3)]) / h
                                          - (s22[(I1, I2 + 1, I3)] - s22[I]) / h
                                          - (s23[I] - s23[(I1, I2, I3 - 1)]) / h)
        out[2][I1 - 1, I2 - 1, I3 - 1] = (g(2) - (s31[I] - s31[(I1 - 1, I2, I3)]) / h
                                          - (s32[I] - s32[(I1, I2 - 1, I3)]) / h
                                          - (s33[(I1, I2, I3 + 1)] - s33[I]) / h)
    return [Field(o) for o in out]


def tensordivergence_nonsym(du, s, h, doadd):
    """``tensordivergence_nonsym!`` (``src/N.jl:162-200``)."""
    s11, s21, s31, s12, s22, s32, s13, s23, s33 = s
    n = du[0].n
    out = [d.data.copy() for d in du]
    for I in _cells(n):
        I1, I2, I3 = I
        g = lambda k: (du[k][I] if doadd else 0.0)
        out[0][I1 - 1, I2 - 1, I3 - 1] = (g(0) - (s11[(I1 + 1, I2, I3)] - s11[I]) / h
                                          - (s12[I] - s12[(I1, I2 - 1, I3)]) / h
                                          - (s13[I] - s13[(I1, I2, I3 - 1)]) / h)
        out[1][I1 - 1, I2 - 1, I3 - 1] = (g(1) - (s21[I] - s21[(I1 - 1, I2, I3)]) / h
                                          - (s22[(I1, I2 + 1, I3)] - s22[I]) / h
                                          - (s23[I] - s23[(I1, I2, I3 - 1)]) / h)
        out[2][I1 - 1, I2 - 1, I3 - 1] = (g(2) - (s31[I] - s31[(I1 - 1, I2, I3)]) / h
                                          - (s32[I] - s32[(I1, I2 - 1, I3)]) / h
                                          - (s33[(I1, I2, I3 + 1)] - s33[I]) / h)
    return [Field(o) for o in out]


def divergence(u, h):
    """``divergence!`` (``src/N.jl:222-238``)."""
    n = u[0].n
    d = np.zeros((n, n, n))
    for I in _cells(n):
        I1, I2, I3 = I
        d[I1 - 1, I2 - 1, I3 - 1] = ((u[0][I] - u[0][(I1 - 1, I2, I3)]) / h
                                     + (u[1][I] - u[1][(I1, I2 - 1, I3)]) / h
                                     + (u[2][I] - u[2][(I1, I2, I3 - 1)]) / h)
    return Field(d)


def pressuregradient(u, p, h):
    """``pressuregradient!`` (``src/N.jl:240-254``)."""
    n = p.n
    out = [x.data.copy() for x in u]
    for I in _cells(n):
        I1, I2, I3 = I
        out[0][I1 - 1, I2 - 1, I3 - 1] -= (p[(I1 + 1, I2, I3)] - p[I]) / h
        out[1][I1 - 1, I2 - 1, I3 - 1] -= (p[(I1, I2 + 1, I3)] - p[I]) / h
        out[2][I1 - 1, I2 - 1, I3 - 1] -= (p[(I1, I2, I3 + 1)] - p[I]) / h
    return [Field(o) for o in out]


def wavenumber_int(n, i):
    """``src/N.jl:31``."""
    return i - 1 - (0 if i <= (n + 1) >> 1 else n)


def project(u, h):
    """``project!`` (``src/N.jl:256-307``); FFTs through NumPy's pocketfft in
    the reference's first-axis-halved ``rfft`` layout."""
    n = u[0].n
    p = divergence(u, h)
    phat = np.fft.rfftn(p.data, axes=(2, 1, 0))  # halves axis 0 (i1), like FFTW
    for i1, i2, i3 in itertools.product(range(1, n // 2 + 2), range(1, n + 1), range(1, n + 1)):
        k1 = i1 - 1
        k2 = wavenumber_int(n, i2)
        k3 = wavenumber_int(n, i3)
        denom = -4 / h**2 * (np.sin(np.pi * k1 / n) ** 2 + np.sin(np.pi * k2 / n) ** 2
                             + np.sin(np.pi * k3 / n) ** 2)
        if denom != 0:
            phat[i1 - 1, i2 - 1, i3 - 1] /= denom
    phat[0, 0, 0] = 0
    pd = np.fft.irfftn(phat, s=(n, n, n), axes=(2, 1, 0))
    return pressuregradient(u, Field(pd), h), Field(pd)


def tophat(c):
    """``tophat`` (``src/N.jl:592-597``)."""
    assert c % 2 == 1
    return [1 / c] * c


def composekernel(f, g):
    """``composekernel`` (``src/N.jl:609-625``), literal double loop."""
    I = len(f) // 2
    J = len(g) // 2
    K = I + J
    out = []
    for k in range(-K, K + 1):
        s = 0.0
        for j in range(-J, J + 1):
            i = k - j
            s += f[I + i] * g[J + j] if abs(i) <= I else 0.0
        out.append(s)
    return out


def kernelproduct(k1, k2, k3):
    """``kernelproduct(::Grid{3}, ...)`` (``src/N.jl:632-637``): ``W[i1,i2,i3]``."""
    return np.asarray(k1)[:, None, None] * np.asarray(k2)[None, :, None] * np.asarray(k3)[None, None, :]


def get_kernels(c, fdelta=(1.0,)):
    """``get_kernels`` (``src/N.jl:1008-1020``) for a given Gaussian ``FDelta``."""
    FH = tophat(c)
    FD = list(fdelta)
    FDH = composekernel(FH, FD)
    GDH = kernelproduct(FDH, FDH, FDH)
    GDHi = tuple(kernelproduct(*[FD if i == j else FDH for j in range(3)]) for i in range(3))
    return GDH, GDHi


def lazyfilter(u, W):
    """``lazyfilter`` (``src/N.jl:655-668``): ``zip(RR, W)`` in column-major order."""
    R = [s // 2 for s in W.shape]

    def f(I):
        s = 0.0
        for r3 in range(-R[2], R[2] + 1):
            for r2 in range(-R[1], R[1] + 1):
                for r1 in range(-R[0], R[0] + 1):
                    w = W[r1 + R[0], r2 + R[1], r3 + R[2]]
                    s += w * u[(I[0] + r1, I[1] + r2, I[2] + r3)]
        return s

    return Lazy(f, u.n)


def lazycoarsegrain(nbar, u, stag):
    """``lazycoarsegrain`` (``src/N.jl:686-698``)."""
    factor = u.n // nbar
    a = factor // 2

    def f(Ib):
        I = tuple(factor * Ib[i] - (not stag[i]) * a for i in range(3))
        return u[I]

    return Lazy(f, nbar)


def materialize(lz, n):
    out = np.zeros((n, n, n))
    for I in _cells(n):
        out[I[0] - 1, I[1] - 1, I[2] - 1] = lz[I]
    return Field(out)


FACES = ((True, False, False), (False, True, False), (False, False, True))
CENTER = (False, False, False)
CORNERS3D = ((False, True, True), (True, False, True), (True, True, False))


def get_r(s, p):
    """``get_r`` (``src/N.jl:1022-1036``)."""
    s11, s22, s33, s12, s23, s31 = s
    r11 = Lazy(lambda I: s11[I] + p[I], p.n)
    r22 = Lazy(lambda I: s22[I] + p[I], p.n)
    r33 = Lazy(lambda I: s33[I] + p[I], p.n)
    return r11, r22, r33, s12, s23, s31


def get_rDHi(r, GDHi, nles):
    """``get_rDHi`` (``src/N.jl:1038-1073``)."""
    r11, r22, r33, r12, r23, r31 = r
    cg = lambda x, W, st: lazycoarsegrain(nles, lazyfilter(x, W), st)
    return (cg(r11, GDHi[0], CENTER), cg(r12, GDHi[0], CORNERS3D[2]), cg(r31, GDHi[0], CORNERS3D[1]),
            cg(r12, GDHi[1], CORNERS3D[2]), cg(r22, GDHi[1], CENTER), cg(r23, GDHi[1], CORNERS3D[0]),
            cg(r31, GDHi[2], CORNERS3D[1]), cg(r23, GDHi[2], CORNERS3D[0]), cg(r33, GDHi[2], CENTER))


def get_sigmaDH(s, nles, GDH):
    """``get_sigmaDH`` (``src/N.jl:1088-1115``)."""
    s11, s22, s33, s12, s23, s31 = s
    cg = lambda x, st: lazycoarsegrain(nles, lazyfilter(x, GDH), st)
    return (cg(s11, CENTER), cg(s22, CENTER), cg(s33, CENTER),
            cg(s12, CORNERS3D[2]), cg(s23, CORNERS3D[0]), cg(s31, CORNERS3D[1]))


def apply_DHpi(u, nles, GDH, H):
    """``apply_DHpi`` (``src/N.jl:1228-1237``)."""
    ub = [materialize(lazycoarsegrain(nles, lazyfilter(u[i], GDH), FACES[i]), nles) for i in range(3)]
    return project(ub, H)[0]


def step_classic_flux_div(v, ubar, u, p, visc, h, H, dt, GDHi, symm=False):
    """``step_DHpi_classic_flux_div[_symm]!`` (``src/N.jl:1189-1226``)."""
    nles = v[0].n
    s_les = stresstensor(v, visc, H)
    s2 = stresstensor(ubar, visc, H)
    sboth = tuple(Lazy(lambda I, a=a, b=b: a[I] - b[I], nles) for a, b in zip(s_les, s2))
    rdhi = get_rDHi(get_r(stresstensor(u, visc, h), p), GDHi, nles)
    zero = [Field(np.zeros((nles,) * 3)) for _ in range(3)]
    du = tensordivergence(zero, sboth, H, False)
    if symm:
        r11, r21, r31, r12, r22, r32, r13, r23, r33 = rdhi
        sym = (r11, r22, r33,
               Lazy(lambda I: (r21[I] + r12[I]) / 2, nles),
               Lazy(lambda I: (r32[I] + r23[I]) / 2, nles),
               Lazy(lambda I: (r31[I] + r13[I]) / 2, nles))
        du = tensordivergence(du, sym, H, True)
    else:
        du = tensordivergence_nonsym(du, rdhi, H, True)
    du, _ = project(du, H)
    return [Field(v[i].data + dt * du[i].data) for i in range(3)]


# ---------------------------------------------------------------------------
# 1-D Burgers (src/Burgers.jl), one sample, 1-based indexing with mod1.

class Field1:
    """Periodic 1-D field (``Field``, ``src/Burgers.jl:33-62``)."""

    def __init__(self, data, h):
        self.data = np.asarray(data, dtype=np.float64)
        self.n = self.data.shape[0]
        self.h = h

    def get(self, i):
        return self.data[mod1(i, self.n) - 1]


class Lazy1:
    """``LazyField`` (``src/Burgers.jl:44-59``): evaluated on every access."""

    def __init__(self, n, h, func):
        self.n, self.h, self.func = n, h, func

    def get(self, i):
        return self.func(i)


def burgers_stress(u, visc):
    """``stress`` (``src/Burgers.jl:89-94``)."""
    def f(i):
        ua = u.get(i - 1)
        ub = u.get(i)
        return -((ua + ub) ** 2) / 8 + visc * (ub - ua) / u.h
    return Lazy1(u.n, u.h, f)


def burgers_lazyfilter(u, kernel):
    """``lazyfilter`` (``src/Burgers.jl:164-172``)."""
    R, w = kernel

    def f(i):
        s = 0.0
        for r in range(-R, R + 1):
            s += w[r + R] * u.get(i + r)
        return s
    return Lazy1(u.n, u.h, f)


def burgers_lazycoarsegrain(nbar, hbar, u, stag):
    """``lazycoarsegrain`` (``src/Burgers.jl:174-180``)."""
    comp = u.n // nbar
    a = comp // 2
    return Lazy1(nbar, hbar, lambda i: u.get(i * comp - (0 if stag else 1) * a))


def burgers_materialize(lz):
    return Field1([lz.get(i) for i in range(1, lz.n + 1)], lz.h)


def burgers_dns_aided_les(ustart, nH, visc, l, les_kernel, double_kernel, tstop, cfl_factor):
    """``dns_aided_les`` (``src/Burgers.jl:350-445``) as written: lazy fields
    materialised where the reference materialises them, forward Euler, the
    LES stepped before the DNS.  Returns the DNS and the four LES fields."""
    nh = len(ustart)
    h, H = l / nh, l / nH
    uh = Field1(ustart, h)
    uH = burgers_materialize(burgers_lazycoarsegrain(nH, H, burgers_lazyfilter(uh, double_kernel), True))
    u = {"dns_ref": Field1(uh.data.copy(), h)}
    for k in ("nomodel", "class_m", "class_p", "swapfil"):
        u[k] = Field1(uH.data.copy(), H)
    t = 0.0
    while t < tstop:
        umax = max(abs(x) for x in u["dns_ref"].data)
        dt = cfl_factor * min(h / umax, h * h / visc)
        dt = min(dt, tstop - t)
        su = burgers_stress(u["dns_ref"], visc)
        fsu = burgers_materialize(burgers_lazycoarsegrain(nH, H, burgers_lazyfilter(su, les_kernel), False))
        vsu = burgers_materialize(burgers_lazycoarsegrain(nH, H, burgers_lazyfilter(su, double_kernel), False))
        VU = burgers_lazyfilter(u["dns_ref"], double_kernel)
        vu = burgers_materialize(burgers_lazycoarsegrain(nH, H, VU, True))
        svu = burgers_stress(vu, visc)
        sVU = burgers_materialize(burgers_lazycoarsegrain(nH, H, burgers_stress(VU, visc), False))
        sig = {
            "nomodel": burgers_stress(u["nomodel"], visc),
            "class_m": Lazy1(nH, H, (lambda s: lambda i: s.get(i) + vsu.get(i) - sVU.get(i))(
                burgers_stress(u["class_m"], visc))),
            "class_p": Lazy1(nH, H, (lambda s: lambda i: s.get(i) + vsu.get(i) - svu.get(i))(
                burgers_stress(u["class_p"], visc))),
            "swapfil": Lazy1(nH, H, (lambda s: lambda i: s.get(i) + fsu.get(i) - svu.get(i))(
                burgers_stress(u["swapfil"], visc))),
        }
        for k in ("nomodel", "class_m", "class_p", "swapfil"):
            du = [(sig[k].get(i + 1) - sig[k].get(i)) / H for i in range(1, nH + 1)]
            u[k] = Field1(u[k].data + dt * np.array(du), H)
        du = [(su.get(i + 1) - su.get(i)) / h for i in range(1, nh + 1)]
        u["dns_ref"] = Field1(u["dns_ref"].data + dt * np.array(du), h)
        t += dt
    return {k: f.data for k, f in u.items()}
