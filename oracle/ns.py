"""Float64 NumPy restatement of the reference's 3-D ``NavierStokes`` operators.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``): what the CUDA path is
compared with, and the timed CPU baseline; never part of the product.

Layout: a scalar field is an ``(n, n, n)`` array indexed ``[z, y, x]`` (C
order, x fastest), which is byte-identical to the reference's column-major
``u[i1, i2, i3]`` (``src/N.jl:29``).  A vector field is ``(3, n, n, n)`` with
the component slowest, like the tuple of three fields of ``src/N.jl:45``.
Direction ``d`` = 0, 1, 2 means x, y, z (the reference's 1, 2, 3).

MAC staggering (from the operators): ``u_d[I]`` sits on the right d-face of
cell I (``src/N.jl:234-236``), ``p[I]`` at the cell centre
(``src/N.jl:250-252``), ``sigma_dd`` at centres and ``sigma_ij`` (i != j) on
the edge ``I + e_i/2 + e_j/2`` (``src/N.jl:106-118``).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

AX = (2, 1, 0)  # direction -> numpy axis of an [z, y, x] array
# Upper-triangle order of the 6 symmetric stress components (src/N.jl:94-104)
SYM6 = ((0, 0), (1, 1), (2, 2), (0, 1), (1, 2), (2, 0))
# Order of the 9 non-symmetric components (src/N.jl:181): s11,s21,s31,s12,...
NONSYM9 = tuple((i, j) for j in range(3) for i in range(3))


def at(a: np.ndarray, d: int, s: int) -> np.ndarray:
    """Periodic shifted view: ``at(a, d, s)[I] == a[I + s*e_d]``.

    Restates the ``mod1`` wrap of ``Base.getindex(::Field{3}, ...)``
    (``src/N.jl:64-67``).
    """
    if s == 0:
        return a
    return np.roll(a, -s, axis=AX[d])


# --------------------------------------------------------------------------
# Grid (src/N.jl:22-32)
# --------------------------------------------------------------------------
@dataclass(frozen=True)
class Grid:
    """Cubic periodic grid ``[0, l]^3`` with ``n`` cells per side (``src/N.jl:22-25``)."""

    l: float
    n: int

    @property
    def h(self) -> float:  # spacing, src/N.jl:30
        return self.l / self.n


def wavenumber_int(n: int, i0: np.ndarray) -> np.ndarray:
    """FFT wavenumber of 0-based index ``i0`` (``src/N.jl:31``)."""
    i = i0 + 1
    return i - 1 - np.where(i <= (n + 1) >> 1, 0, n)


# --------------------------------------------------------------------------
# Stress and divergence (src/N.jl:94-200)
# --------------------------------------------------------------------------
def stress(u: np.ndarray, visc: float, h: float, i: int, j: int) -> np.ndarray:
    """One component of the staggered stress ``sigma_ij`` (``src/N.jl:106-118``)."""
    off = i != j
    ui_rightj = at(u[i], j, int(off))
    ui_leftj = at(u[i], j, int(off) - 1)
    uj_righti = at(u[j], i, int(off))
    uj_lefti = at(u[j], i, int(off) - 1)
    etaj_ui = (ui_rightj + ui_leftj) / 2
    etai_uj = (uj_righti + uj_lefti) / 2
    dj_ui = (ui_rightj - ui_leftj) / h
    di_uj = (uj_righti - uj_lefti) / h
    return etaj_ui * etai_uj - visc * (dj_ui + di_uj)


def stresstensor(u: np.ndarray, visc: float, h: float) -> dict:
    """The 6 symmetric components, keyed ``(i, j)`` (``src/N.jl:94-104``)."""
    s = {}
    for i, j in SYM6:
        s[(i, j)] = stress(u, visc, h, i, j)
        s[(j, i)] = s[(i, j)]
    return s


def tensordivergence(sig: dict, h: float, du: np.ndarray | None = None,
                     doadd: bool = False) -> np.ndarray:
    """``du_i = doadd*du_i - sum_j delta_j sigma_ij`` (``src/N.jl:120-160``).

    ``sig`` maps ``(i, j)`` to the component used in ``du_i`` with the
    derivative along ``j``; a symmetric dict gives ``tensordivergence!`` and a
    9-entry one gives ``tensordivergence_nonsym!`` (``src/N.jl:162-200``).
    Diagonal terms use the forward difference ``s[I+e_i] - s[I]``, off-diagonal
    terms the backward difference ``s[I] - s[I-e_j]``.  ``doadd = False``
    overwrites (Julia's ``false * x`` is a strong zero).
    """
    out = np.empty((3,) + sig[(0, 0)].shape) if du is None or not doadd else du.copy()
    for i in range(3):
        acc = out[i] if doadd else np.zeros_like(sig[(0, 0)])
        for j in range(3):
            s = sig[(i, j)]
            if i == j:
                acc = acc - (at(s, j, 1) - s) / h
            else:
                acc = acc - (s - at(s, j, -1)) / h
        out[i] = acc
    return out


def rhs(u: np.ndarray, visc: float, h: float) -> np.ndarray:
    """Convection-diffusion RHS ``-div sigma(u)`` (``stresstensor`` + ``tensordivergence!``)."""
    return tensordivergence(stresstensor(u, visc, h), h)


def divergence(u: np.ndarray, h: float) -> np.ndarray:
    """Staggered divergence at cell centres (``src/N.jl:222-238``)."""
    d = np.zeros_like(u[0])
    for i in range(3):
        d = d + (u[i] - at(u[i], i, -1)) / h
    return d


def pressuregradient(u: np.ndarray, p: np.ndarray, h: float) -> np.ndarray:
    """``u_i -= (p[I+e_i] - p[I]) / h`` (``src/N.jl:240-254``); returns a new array."""
    out = u.copy()
    for i in range(3):
        out[i] = u[i] - (at(p, i, 1) - p) / h
    return out


# --------------------------------------------------------------------------
# Poisson solver and projection (src/N.jl:202-307)
# --------------------------------------------------------------------------
def laplace_symbol(n: int, h: float) -> np.ndarray:
    """``-4/h^2 * sum_d sin^2(pi k_d / n)`` on the rfft half grid ``[kz, ky, kx]``
    (``src/N.jl:281-291``)."""
    kx = np.arange(n // 2 + 1)
    ky = wavenumber_int(n, np.arange(n))
    s = lambda k: np.sin(np.pi * k / n) ** 2
    return -4 / h**2 * (s(kx)[None, None, :] + s(ky)[None, :, None] + s(ky)[:, None, None])


def poisson_solve(d: np.ndarray, h: float) -> np.ndarray:
    """Pressure ``p`` with ``L p = d`` (mean zero), ``src/N.jl:262-301``."""
    n = d.shape[0]
    phat = np.fft.rfftn(d)
    lam = laplace_symbol(n, h)
    with np.errstate(divide="ignore", invalid="ignore"):
        phat = phat / lam
    phat[0, 0, 0] = 0  # src/N.jl:298
    return np.fft.irfftn(phat, s=d.shape, axes=(0, 1, 2))


def project(u: np.ndarray, h: float, return_p: bool = False):
    """``project!(u, poisson)`` (``src/N.jl:256-307``): returns P(u) [and p]."""
    p = poisson_solve(divergence(u, h), h)
    out = pressuregradient(u, p, h)
    return (out, p) if return_p else out


# --------------------------------------------------------------------------
# Time stepping (src/N.jl:309-356; RK4 tableau src/Burgers.jl:120-142)
# --------------------------------------------------------------------------
def propose_timestep(u: np.ndarray, visc: float, cfl: float, h: float) -> float:
    """``min(cfl*h/umax, cfl*h^2/visc/2D)`` (``src/N.jl:348-356``)."""
    umax = float(np.max(np.abs(u)))
    dt_adv = cfl * h / umax
    dt_visc = cfl * h**2 / visc / (2 * 3)
    return min(dt_adv, dt_visc)


def step_forwardeuler(u, visc, h, dt):
    """``step_forwardeuler!`` (``src/N.jl:309-318``)."""
    return project(u + dt * rhs(u, visc, h), h)


def step_wray3(u, visc, h, dt):
    """``step_wray3!`` (``src/N.jl:320-346``)."""
    a = (8 / 15, 5 / 12, 3 / 4)
    b = (1 / 4, 0.0)
    u0 = u.copy()
    for i in range(3):
        du = rhs(u, visc, h)
        if i > 0:
            u = u0.copy()
        u = project(u + a[i] * dt * du, h)
        if i < 2:
            u0 = u0 + b[i] * dt * du
    return u


RK4_A = (0.0, 0.5, 0.5, 1.0)  # stage abscissae, src/Burgers.jl:120-142
RK4_B = (1.0, 2.0, 2.0, 1.0)  # weights (times dt/6)


def projected_rhs(u, visc, h):
    """``k = P(RHS(u))`` and the pressure ``p`` of that projection, as the DNS
    part of ``dnsaid_project`` computes them (``src/N.jl:1305-1309``)."""
    return project(rhs(u, visc, h), h, return_p=True)


def step_rk4(u, visc, h, dt):
    """Classical RK4 (tableau of ``rk4_timestep!``, ``src/Burgers.jl:120-142``)
    with ``k_s = P(RHS(u_s))``: one FFT projection per stage."""
    u0 = u
    ks = []
    us = u0
    for s in range(4):
        if s > 0:
            us = u0 + (RK4_A[s] * dt) * ks[-1]
        k, _ = projected_rhs(us, visc, h)
        ks.append(k)
    return u0 + dt / 6 * (ks[0] + 2 * ks[1] + 2 * ks[2] + ks[3])


# --------------------------------------------------------------------------
# Random initial field (src/N.jl:366-476)
# --------------------------------------------------------------------------
_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix(x: np.ndarray) -> np.ndarray:
    x = x.astype(np.uint64)
    x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return x ^ (x >> np.uint64(31))


def counter_normal(seed: int, count: int, offset: int = 0) -> np.ndarray:
    """Seeded standard normals from a counter-based generator (the project's
    replacement for Julia's ``Xoshiro``/``randn!``, ``src/N.jl:406``).

    Sample ``m`` uses two splitmix64 hashes of ``seed*phi + 2m (+1)`` mapped to
    uniforms in (0, 1) and the Box–Muller transform.  The CUDA initialiser
    evaluates the same formula per element.
    """
    with np.errstate(over="ignore"):
        m = np.arange(offset, offset + count, dtype=np.uint64)
        base = np.uint64(seed) * np.uint64(0x9E3779B97F4A7C15)
        z1 = _splitmix(base + np.uint64(2) * m)
        z2 = _splitmix(base + np.uint64(2) * m + np.uint64(1))
    u1 = ((z1 >> np.uint64(11)).astype(np.float64) + 0.5) * 2.0**-53
    u2 = ((z2 >> np.uint64(11)).astype(np.float64) + 0.5) * 2.0**-53
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


def peak_profile(k, kpeak):
    """``k^4 exp(-2 (k/kpeak)^2)`` (``src/N.jl:366``)."""
    k = np.asarray(k, dtype=np.float64)
    return k**4 * np.exp(-2 * (k / kpeak) ** 2)


def shell_index(n: int) -> np.ndarray:
    """Squared integer wavenumber ``k1^2+k2^2+k3^2`` on the rfft half grid
    (``applymask!``, ``src/N.jl:375-392``)."""
    kx = np.arange(n // 2 + 1)
    ky = wavenumber_int(n, np.arange(n))
    return kx[None, None, :] ** 2 + ky[None, :, None] ** 2 + ky[:, None, None] ** 2


def conj_weight(n: int) -> np.ndarray:
    """Weight 2 for the rfft x-modes ``1..n/2-1`` whose conjugates are not
    stored, 1 otherwise (``src/N.jl:443``, ``src/N.jl:534-543``)."""
    w = np.ones(n // 2 + 1)
    w[1 : n // 2] = 2.0
    return w


def power_profile(k, p):
    """``k -> (k > 0) * k^p`` (the ``dnsaid_project`` profile, ``src/N.jl:1245``)."""
    k = np.asarray(k, dtype=np.float64)
    return np.where(k > 0, np.power(np.maximum(k, 1.0), p), 0.0)


def randomfield(n: int, l: float, kpeak: float, seed: int, totalenergy: float = 1.0, profile: str = "peak"):
    """``randomfield(peak_profile, ...)`` (``src/N.jl:394-476``) with the
    project's counter-based normals in place of ``randn!``; ``profile =
    "power"`` uses ``power_profile`` with exponent ``kpeak``."""
    h = l / n
    N = n**3
    u = counter_normal(seed, 3 * N).reshape(3, n, n, n)
    u = project(u, h)
    uhat = [np.fft.rfftn(u[c]) / N for c in range(3)]
    E = (np.abs(uhat[0]) ** 2 + np.abs(uhat[1]) ** 2 + np.abs(uhat[2]) ** 2) / 2
    kk = shell_index(n)
    w = conj_weight(n)[None, None, :]
    kmax = n // 2
    kdiag = int(math.floor(math.sqrt(3) * kmax))
    ks = np.arange(kdiag + 1)
    prof = peak_profile(ks, kpeak) if profile == "peak" else power_profile(ks, kpeak)
    totalprofile = prof.sum()
    for k in range(kdiag + 1):
        mask = (k * k <= kk) & (kk < (k + 1) ** 2)
        Eshell = np.sum(E * mask * w)
        E0 = totalenergy * prof[k] / totalprofile
        if not mask.any() or not Eshell > 0:
            continue
        factor = np.sqrt(E0 / Eshell)
        for c in range(3):
            uhat[c] = np.where(mask, factor * uhat[c], uhat[c])
    u = np.stack([np.fft.irfftn(uhat[c], s=(n, n, n), axes=(0, 1, 2)) * N for c in range(3)])
    return project(u, h)


def spectrum(u: np.ndarray, l: float):
    """Shell energy spectrum for shells ``1..div(2*kmax,3)``
    (``spectral_stuff``/``spectrum``, ``src/N.jl:546-590``)."""
    n = u.shape[1]
    N = n**3
    ehat = sum(np.abs(np.fft.rfftn(u[c]) / N) ** 2 / 2 for c in range(3))
    kk = shell_index(n)
    w = conj_weight(n)[None, None, :]
    kcut = (2 * (n // 2)) // 3
    s = np.array([np.sum(ehat * w * ((k * k <= kk) & (kk < (k + 1) ** 2)))
                  for k in range(1, kcut + 1)])
    return 2 * np.pi / l * np.arange(1, kcut + 1), s


def dissipation(u: np.ndarray, visc: float, h: float) -> float:
    """``visc * mean sum_ij (delta_j u_i)^2`` with forward differences: the
    energy drained by the viscous part of ``stress`` (``src/N.jl:106-118``) for
    a divergence-free field; the reference takes it from Turbulox
    (``dns_aid.jl:92-94``)."""
    s = 0.0
    for i in range(3):
        for j in range(3):
            s += float(np.sum(((at(u[i], j, 1) - u[i]) / h) ** 2))
    return visc * s / u[0].size


def kinetic_energy(u: np.ndarray) -> float:
    """Mean kinetic energy ``sum(u^2)/2/N`` (``src/NavierStokes.jl:74``)."""
    return float(np.sum(u * u) / 2 / u[0].size)


# --------------------------------------------------------------------------
# Filters (src/N.jl:592-698, 999-1020) and their even-ratio extension
# --------------------------------------------------------------------------
def tophat(compression: int) -> np.ndarray:
    """``tophat`` (``src/N.jl:592-597``); the reference asserts an odd ratio."""
    assert compression % 2 == 1
    return np.full(compression, 1 / compression)


def gaussian(h: float, delta: float, nsigma: float) -> np.ndarray:
    """``gaussian`` (``src/N.jl:599-607``); ``delta == 0`` gives ``[1]`` like the
    guarded 1-D version (``src/Burgers.jl:149-151``)."""
    if delta < 1e-15:
        return np.ones(1)
    sig = delta / math.sqrt(12)
    r = int(round(nsigma * sig / h))
    x = h * np.arange(-r, r + 1)
    w = np.exp(-(x**2) / (2 * sig**2))
    return w / w.sum()


def composekernel(f: np.ndarray, g: np.ndarray) -> np.ndarray:
    """Full discrete convolution of two centred odd kernels (``src/N.jl:609-625``)."""
    return np.convolve(f, g)


# Position of a quantity along one axis: on a fine face ("stag") or a centre.
FACE, CENTRE = True, False
# Filter mode along one axis: average over the coarse cell or sample the face.
VOLUME, POINT = "volume", "point"


def axis_taps(c: int, stag: bool, mode: str, fdelta: np.ndarray | None = None):
    """1-D coarse-grain-and-filter stencil along one axis.

    Returns ``(offsets, weights)`` such that the coarse sample ``ib`` (0-based)
    is ``sum_t w_t f[(c*ib + o_t) mod n]``.

    Odd ``c`` restates ``lazyfilter`` + ``lazycoarsegrain`` (``src/N.jl:655-698``):
    the sample point is ``c*Ib - !stag*div(c,2)`` (1-based), i.e. 0-based
    ``c*ib + c-1`` for a face and ``c*ib + div(c,2)`` for a centre, and the
    volume mode applies ``tophat(c)`` centred there.  Even ``c`` (no reference
    counterpart; the reference asserts odd ratios, ``src/N.jl:593``) uses the
    same rule -- the exact average of the piecewise-constant fine field over
    the coarse cell extent: on a face axis the ``c+1`` fine faces
    ``c*ib+c-1 -/+ c/2`` with trapezoid weights ``[1/2, 1, ..., 1, 1/2]/c``; on
    a centre axis the ``c`` fine cells ``c*ib .. c*ib+c-1``; a centre point
    sample is the mean of the two fine centres around the coarse centre.  For
    odd ``c`` this is identical to the reference's stencil.  ``fdelta``
    (optional odd Gaussian, ``src/N.jl:1008-1020``) is convolved in.
    """
    a = c // 2
    if stag:
        base = c - 1
        if mode == POINT:
            o, w = [base], [1.0]
        elif c % 2 == 1:
            o, w = list(range(base - a, base + a + 1)), [1 / c] * c
        else:
            o = list(range(base - a, base + a + 1))
            w = [1 / c] * (c + 1)
            w[0] = w[-1] = 0.5 / c
    else:
        if mode == POINT:
            if c % 2 == 1:
                o, w = [a], [1.0]
            else:
                o, w = [a - 1, a], [0.5, 0.5]
        else:
            o, w = list(range(c)), [1 / c] * c
    o = np.array(o)
    w = np.array(w)
    if fdelta is not None and len(fdelta) > 1:
        R = len(fdelta) // 2
        oo = (o[:, None] + np.arange(-R, R + 1)[None, :]).ravel()
        ww = (w[:, None] * fdelta[None, :]).ravel()
        uo = np.unique(oo)
        w = np.array([ww[oo == x].sum() for x in uo])
        o = uo
    return o, w


def filter_coarse(f: np.ndarray, c: int, stags, modes, fdelta=None) -> np.ndarray:
    """Separable filter + coarse-grain of a fine scalar field to ``n/c`` cells.

    ``stags[d]`` / ``modes[d]`` give the position and filter mode along
    direction ``d``.  Restates ``lazycoarsegrain(g_les, lazyfilter(u, G), stag)``
    (``src/N.jl:655-698``) for the separable kernels ``GDH``/``GDHi`` of
    ``get_kernels`` (``src/N.jl:1008-1020``).
    """
    n = f.shape[0]
    m = n // c
    assert m * c == n
    out = f
    for d in range(3):
        o, w = axis_taps(c, stags[d], modes[d], fdelta)
        ax = AX[d]
        base = c * np.arange(m)
        acc = 0.0
        for ot, wt in zip(o, w):
            idx = (base + ot) % n
            acc = acc + wt * np.take(out, idx, axis=ax)
        out = acc
    return out


def positions_u(i: int):
    """``faces[i]`` (``src/N.jl:1001``): face along ``i``, centre elsewhere."""
    return tuple(d == i for d in range(3))


def positions_sigma(i: int, j: int):
    """Centre for ``i == j``; the edge ``corners3D`` otherwise (``src/N.jl:1004``)."""
    if i == j:
        return (False, False, False)
    return tuple(d in (i, j) for d in range(3))


def volume_filter(u: np.ndarray, c: int, fdelta=None) -> np.ndarray:
    """``coarsegrain(faces[i], lazyfilter(u_i, GDH))`` for each component, the
    filter inside ``apply_DHpi`` (``src/N.jl:1228-1237``)."""
    return np.stack([filter_coarse(u[i], c, positions_u(i), (VOLUME,) * 3, fdelta)
                     for i in range(3)])


def face_filter(u: np.ndarray, c: int, fdelta=None) -> np.ndarray:
    """Face (surface) average: the ``c x c`` transverse box of fine faces inside
    each coarse face, sampled at that face.  Restates the semantics of
    Turbulox's ``surfacefilter!(fiu, u, c)`` used by ``dns_aid_surface``
    (``src/NavierStokes.jl:333``); Turbulox itself is not in the reference."""
    return np.stack([filter_coarse(u[i], c, positions_u(i),
                                   tuple(POINT if d == i else VOLUME for d in range(3)), fdelta)
                     for i in range(3)])


def apply_filter(u, c, kind, fdelta=None):
    return volume_filter(u, c, fdelta) if kind == "volume" else face_filter(u, c, fdelta)


def apply_DHpi(u: np.ndarray, c: int, l: float, fdelta=None) -> np.ndarray:
    """``apply_DHpi``: volume filter, coarse-grain at faces, project on the
    coarse grid (``src/N.jl:1228-1237``)."""
    ub = volume_filter(u, c, fdelta)
    return project(ub, l / ub.shape[1])


def get_r(sig: dict, p: np.ndarray) -> dict:
    """Total flux ``r_ij = sigma_ij + delta_ij p`` (``src/N.jl:1022-1036``)."""
    r = dict(sig)
    for i in range(3):
        r[(i, i)] = sig[(i, i)] + p
    return r


def get_rDHi(r: dict, c: int, fdelta=None) -> dict:
    """Face-filtered flux, 9 components keyed ``(i, j)`` = used in ``du_i`` with
    derivative along ``j`` (``src/N.jl:1038-1073``): ``r_ij`` filtered with
    ``GDHi[j]`` (point sample along ``j``, volume elsewhere) and coarse-grained
    at the centre (``i == j``) or the edge ``(i, j)``."""
    out = {}
    for i in range(3):
        for j in range(3):
            modes = tuple(POINT if d == j else VOLUME for d in range(3))
            out[(i, j)] = filter_coarse(r[(i, j)], c, positions_sigma(i, j), modes, fdelta)
    return out


def symmetrize(s9: dict) -> dict:
    """``(r_ij + r_ji)/2`` (``src/N.jl:1075-1086``)."""
    out = {}
    for i, j in SYM6:
        v = s9[(i, i)] if i == j else (s9[(i, j)] + s9[(j, i)]) / 2
        out[(i, j)] = v
        out[(j, i)] = v
    return out


def get_sigmaDH(sig: dict, c: int, fdelta=None) -> dict:
    """Volume-filtered DNS stress at LES centres/edges (``src/N.jl:1088-1115``)."""
    out = {}
    for i, j in SYM6:
        v = filter_coarse(sig[(i, j)], c, positions_sigma(i, j), (VOLUME,) * 3, fdelta)
        out[(i, j)] = v
        out[(j, i)] = v
    return out


def closure_flux_div(u: np.ndarray, p: np.ndarray, visc: float, l: float, c: int,
                     ubar: np.ndarray, fdelta=None) -> np.ndarray:
    """Exact commutator of ``step_DHpi_classic_flux_div!`` (``src/N.jl:1189-1206``)
    before the coarse projection: ``delta_H sigma_H(ubar) - delta_H^ns rDHi``.

    ``u``/``p`` are the DNS velocity and the pressure of its projected RHS,
    ``ubar`` the projected filtered DNS velocity on the LES grid."""
    n = u.shape[1]
    h = l / n
    H = l / ubar.shape[1]
    r = get_r(stresstensor(u, visc, h), p)
    rdhi = get_rDHi(r, c, fdelta)
    m = -rhs(ubar, visc, H)  # +delta_H sigma_H(ubar)
    return tensordivergence(rdhi, H, m, doadd=True)


def closure(kdns: np.ndarray, ubar: np.ndarray, visc: float, l: float, c: int, kind: str,
            fdelta=None) -> np.ndarray:
    """Exact closure commutator on the LES grid at one stage:
    ``m = P_H filter(k_dns) - P_H RHS_H(ubar)`` with ``k_dns = P_h RHS_h(u)``.

    For the volume filter ``P_H filter(k_dns)`` equals
    ``P_H(-delta_H^ns rDHi)`` of ``src/N.jl:1189-1206`` (the box along the
    derivative axis telescopes the fine difference), so ``m`` is the projected
    commutator of the reference's exact closure."""
    H = l / ubar.shape[1]
    return project(apply_filter(kdns, c, kind, fdelta), H) - project(rhs(ubar, visc, H), H)


# --------------------------------------------------------------------------
# LES closure steppers (src/N.jl:1137-1226), forward Euler like the reference
# --------------------------------------------------------------------------
def step_nomodel(v, visc, H, dt):
    """No-model LES step, ``step_forwardeuler!`` on the LES grid (``src/N.jl:1315``)
    in the ``dnsaid_project`` form ``v += dt P(RHS(v))``."""
    return v + dt * project(rhs(v, visc, H), H)


def step_classic(v, u, visc, l, c, dt, fdelta=None):
    """``step_DHpi_classic!`` (``src/N.jl:1137-1162``)."""
    n = u.shape[1]
    h, H = l / n, l / v.shape[1]
    sig_les = stresstensor(v, visc, H)
    s1 = get_sigmaDH(stresstensor(u, visc, h), c, fdelta)
    uf = np.stack([_fine_filter(u[i], c, fdelta) for i in range(3)])
    s2f = stresstensor(uf, visc, h)
    s2 = {k: _lazytensorcoarsegrain(s2f[k], c, k) for k in s2f}
    sall = {k: sig_les[k] + s1[k] - s2[k] for k in sig_les}
    du = project(tensordivergence(sall, H), H)
    return v + dt * du


def _fine_filter(f, c, fdelta=None):
    """``lazyfilter(u, GDH)`` on the fine grid without coarse-graining (odd c)."""
    assert c % 2 == 1, "the classic closure's fine-grid filter is defined for odd ratios"
    w1 = tophat(c) if fdelta is None else composekernel(tophat(c), fdelta)
    R = len(w1) // 2
    out = f
    for d in range(3):
        acc = 0.0
        for r, w in zip(range(-R, R + 1), w1):
            acc = acc + w * at(out, d, r)
        out = acc
    return out


def _lazytensorcoarsegrain(s, c, key):
    """``lazytensorcoarsegrain`` (``src/N.jl:1117-1135``); its sample point
    ``c*Ib - !stag*div(c,2)`` uses ``get_positions(g_les)``."""
    i, j = key
    return filter_coarse(s, c, positions_sigma(i, j), (POINT,) * 3)


def step_classic_flux(v, ubar, u, visc, l, c, dt, fdelta=None):
    """``step_DHpi_classic_flux!`` (``src/N.jl:1164-1187``)."""
    n = u.shape[1]
    h, H = l / n, l / v.shape[1]
    sig_les = stresstensor(v, visc, H)
    s1 = get_sigmaDH(stresstensor(u, visc, h), c, fdelta)
    s2 = stresstensor(ubar, visc, H)
    sall = {k: sig_les[k] + s1[k] - s2[k] for k in sig_les}
    return v + dt * project(tensordivergence(sall, H), H)


def step_classic_flux_div(v, ubar, u, p, visc, l, c, dt, fdelta=None, symm=False):
    """``step_DHpi_classic_flux_div[_symm]!`` (``src/N.jl:1189-1226``)."""
    n = u.shape[1]
    h, H = l / n, l / v.shape[1]
    sig_les = stresstensor(v, visc, H)
    s2 = stresstensor(ubar, visc, H)
    sboth = {k: sig_les[k] - s2[k] for k in sig_les}
    rdhi = get_rDHi(get_r(stresstensor(u, visc, h), p), c, fdelta)
    du = tensordivergence(sboth, H)
    if symm:
        du = tensordivergence(symmetrize(rdhi), H, du, doadd=True)
    else:
        du = tensordivergence(rdhi, H, du, doadd=True)
    return v + dt * project(du, H)


def compute_errors(results: dict, ref: np.ndarray) -> dict:
    """``sqrt(mean_i sum|a_i-b_i|^2/sum|b_i|^2)`` (``src/N.jl:1334-1349``)."""
    out = {}
    for k, a in results.items():
        e = sum(np.sum((a[i] - ref[i]) ** 2) / np.sum(ref[i] ** 2) for i in range(3)) / 3
        out[k] = math.sqrt(e)
    return out


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    """Relative L2 error ``|a-b|/|b|`` over all components."""
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


# --------------------------------------------------------------------------
# DNS-aided driver with RK4 and the exact closure at every stage
# --------------------------------------------------------------------------
@dataclass
class Les:
    """One LES grid attached to a DNS: ratio ``c`` and filter ``kind``."""

    c: int
    kind: str = "volume"
    v_exact: np.ndarray | None = None   # LES driven by the exact closure
    v_nomodel: np.ndarray | None = None  # LES without closure
    snaps: list = field(default_factory=list)


def filtered_target(u, les: Les, l, fdelta=None):
    """The LES target: ``P_H(volume filter u)`` (``apply_DHpi``) or the face
    filter (divergence free by construction, no projection)."""
    ub = apply_filter(u, les.c, les.kind, fdelta)
    if les.kind == "volume":
        ub = project(ub, l / ub.shape[1])
    return ub


def dnsaid_rk4(u: np.ndarray, visc: float, l: float, cfl: float, nsteps: int,
               les_list: list[Les], fdelta=None, record_closure: bool = False,
               dt_fixed: float | None = None):
    """RK4 DNS with LES grids advanced in lockstep (the ``dnsaid_project`` loop,
    ``src/N.jl:1298-1323``, with RK4 stages in place of forward Euler).

    At every stage s: ``k_s = P_h RHS_h(u_s)``; for each LES,
    ``ubar_s = target(u_s)``, ``m_s = P_H filter(k_s) - P_H RHS_H(ubar_s)`` and
    the exact-closure LES stage ``kv_s = P_H RHS_H(v_s) + m_s``; the no-model
    LES uses ``kv_s = P_H RHS_H(v_s)``.  Returns (u, dts, closures)."""
    n = u.shape[1]
    h = l / n
    for les in les_list:
        tgt = filtered_target(u, les, l, fdelta)
        les.v_exact = tgt.copy()
        les.v_nomodel = tgt.copy()
    dts = []
    closures = []
    for _ in range(nsteps):
        dt = dt_fixed if dt_fixed is not None else propose_timestep(u, visc, cfl, h)
        dts.append(dt)
        u0 = u
        ks = []
        les_k = [([], []) for _ in les_list]
        for s in range(4):
            us = u0 if s == 0 else u0 + (RK4_A[s] * dt) * ks[-1]
            k, _p = projected_rhs(us, visc, h)
            ks.append(k)
            for li, les in enumerate(les_list):
                H = l / (n // les.c)
                ub = filtered_target(us, les, l, fdelta)
                m = closure(k, ub, visc, l, les.c, les.kind, fdelta)
                if record_closure and s == 0:
                    closures.append((li, ub, m))
                ke, kn = les_k[li]
                ve = les.v_exact if s == 0 else les.v_exact + (RK4_A[s] * dt) * ke[-1]
                vn = les.v_nomodel if s == 0 else les.v_nomodel + (RK4_A[s] * dt) * kn[-1]
                ke.append(project(rhs(ve, visc, H), H) + m)
                kn.append(project(rhs(vn, visc, H), H))
        u = u0 + dt / 6 * (ks[0] + 2 * ks[1] + 2 * ks[2] + ks[3])
        for li, les in enumerate(les_list):
            ke, kn = les_k[li]
            les.v_exact = les.v_exact + dt / 6 * (ke[0] + 2 * ke[1] + 2 * ke[2] + ke[3])
            les.v_nomodel = les.v_nomodel + dt / 6 * (kn[0] + 2 * kn[1] + 2 * kn[2] + kn[3])
    return u, dts, closures


# --------------------------------------------------------------------------
# The reference's own driver: forward Euler, five LES variants in lockstep
# --------------------------------------------------------------------------
DNSAID_NAMES = ("u_nomo", "u_c", "u_cf", "u_cfd", "u_cfd_symm")


def dnsaid_warmup(u, visc, l, twarm, cfl, max_steps=None, t0=0.0):
    """The warm-up loop of ``dnsaid_project`` (``src/N.jl:1264-1276``).
    Returns (u, t, steps)."""
    h = l / u.shape[1]
    t, it = t0, 0
    while t < twarm and (max_steps is None or it < max_steps):
        dt = min(propose_timestep(u, visc, cfl, h), twarm - t)
        t += dt
        it += 1
        u = step_forwardeuler(u, visc, h, dt)
    return u, t, it


def dnsaid_start(u, l, c, fdelta=None):
    """LES initial states (``src/N.jl:1278-1287``): all five equal
    ``apply_ΔHπ(u)``."""
    ub = apply_DHpi(u, c, l, fdelta)
    return {k: ub.copy() for k in DNSAID_NAMES}


def dnsaid_project_steps(u, les, visc, l, c, tstop, cfl, fdelta=None, max_steps=None, t0=0.0):
    """The lockstep loop of ``dnsaid_project`` (``src/N.jl:1289-1323``):
    the DNS right-hand side is projected (its pressure feeds ``r``), the
    five LES take forward-Euler steps with the DNS time step, then the DNS
    is updated.  Returns (u, les, t, steps)."""
    n = u.shape[1]
    h = l / n
    H = l / (n // c)
    les = {k: v.copy() for k, v in les.items()}
    t, it = t0, 0
    while t < tstop and (max_steps is None or it < max_steps):
        dt = min(propose_timestep(u, visc, cfl, h), tstop - t)
        t += dt
        it += 1
        du, p = project(rhs(u, visc, h), h, return_p=True)
        ub = apply_DHpi(u, c, l, fdelta)
        les["u_nomo"] = step_forwardeuler(les["u_nomo"], visc, H, dt)
        les["u_c"] = step_classic(les["u_c"], u, visc, l, c, dt, fdelta)
        les["u_cf"] = step_classic_flux(les["u_cf"], ub, u, visc, l, c, dt, fdelta)
        les["u_cfd"] = step_classic_flux_div(les["u_cfd"], ub, u, p, visc, l, c, dt, fdelta)
        les["u_cfd_symm"] = step_classic_flux_div(les["u_cfd_symm"], ub, u, p, visc, l, c, dt, fdelta, symm=True)
        u = u + dt * du
    return u, les, t, it


# --------------------------------------------------------------------------
# The paper's volume-average driver `dns_aid_volavg` (src/NavierStokes.jl:141-304)
# --------------------------------------------------------------------------
# The paper module calls Turbulox.jl (not vendored, no pinned version) for its
# filters; they are restated with the reference's own filters of src/N.jl:
# `volumefilter!` as the c^3 top-hat GDH sampled at the LES positions
# (`lazyfilter` + `lazycoarsegrain`, src/N.jl:639-698) and the flux's
# `surfacefilter!(., false)` as GDHi (`get_rΔHi`, src/N.jl:1038-1073).  Parity
# of this path is against this restatement only (no reference vectors).
PAPER_NAMES = ("nomodel", "classic", "swapfil", "swapfil_symm")


def paper_volavg_target(u, l, c, doproject, fdelta=None):
    """``fu``: the volume-filtered DNS, projected when ``doproject``
    (src/NavierStokes.jl:169-170, 290-291)."""
    fu = volume_filter(u, c, fdelta)
    return project(fu, l / fu.shape[1]) if doproject else fu


def dns_aid_volavg_steps(u, les, visc, l, c, tstop, cfl, doproject, fdelta=None, max_steps=None, t0=0.0):
    """Steps of the loop of ``dns_aid_volavg`` (src/NavierStokes.jl:186-288):
    with ``r = sigma(u) + p I`` of the projected DNS right-hand side and
    ``rfu = sigma_H(fu) + p_H I`` (``p_H`` the pressure of the LES
    right-hand side of ``fu``), the closures are the divergences of
    ``fru - rfu`` (classic, volume-filtered flux), ``firu - rfu`` (swap, the
    face-filtered flux) and its symmetric part; each LES takes
    ``v += dt P(RHS_H(v))``, ``v += dt dsigma``, then a projection when
    ``doproject``.  Returns (u, les, t, steps)."""
    n = u.shape[1]
    h = l / n
    m = n // c
    H = l / m
    les = {k: v.copy() for k, v in les.items()}
    t, it = t0, 0
    while t < tstop and (max_steps is None or it < max_steps):
        dt = min(propose_timestep(u, visc, cfl, h), tstop - t)
        t += dt
        it += 1
        du, p = project(rhs(u, visc, h), h, return_p=True)
        r = get_r(stresstensor(u, visc, h), p)
        fru = get_sigmaDH(r, c, fdelta)
        firu = get_rDHi(r, c, fdelta)
        fu = paper_volavg_target(u, l, c, doproject, fdelta)
        sfu = stresstensor(fu, visc, H)
        p_les = poisson_solve(divergence(tensordivergence(sfu, H), H), H)
        rfu = get_r(sfu, p_les)
        s_classic = {k: fru[k] - rfu[k] for k in fru}
        s_swap = {k: firu[k] - rfu[k] for k in firu}
        dsig = {"classic": tensordivergence(s_classic, H), "swapfil": tensordivergence(s_swap, H),
                "swapfil_symm": tensordivergence(symmetrize(s_swap), H)}
        u = u + dt * du
        les["nomodel"] = les["nomodel"] + dt * project(rhs(les["nomodel"], visc, H), H)
        for k in ("classic", "swapfil", "swapfil_symm"):
            v = les[k] + dt * project(rhs(les[k], visc, H), H)
            v = v + dt * dsig[k]
            les[k] = project(v, H) if doproject else v
    return u, les, t, it


# --------------------------------------------------------------------------
# The paper's surface-average driver `dns_aid_surface` (src/NavierStokes.jl:306-468)
# --------------------------------------------------------------------------
# Its filters come from Turbulox.jl (not vendored, no pinned version); they are
# restated from their finite-volume meaning with the separable stencils above:
#   `surfacefilter!(fiu, u, c)`     the face average: the c x c transverse box
#                                   of fine faces inside each coarse face of
#                                   u_i (point sample along i) = face_filter;
#   `surfacefilter!(firu, ru, c, true)`  the flux r_ij (used in du_i, derivative
#                                   along j) filtered like the velocity it
#                                   updates: point sample along i, box along the
#                                   two other axes, at the LES centre (i == j)
#                                   or edge (i, j);
#   `linefilter!(fijru, ru, c)`     r_ij (i != j) point-sampled along i and j,
#                                   averaged along the third axis only.
# Why these: the face average of the fine flux divergence sum_j delta_j r_ij
# over the coarse face of u_i telescopes along each transverse axis j != i
# into a coarse difference of the line average of r_ij (exactly), while the
# normal term delta_i r_ii is a fine-grid difference across the face that no
# coarse difference of a local field reproduces; the swap closure keeps the
# face average of r_ii at the coarse centre for it.  So the swap LES on the
# face filter is exact off the diagonal only (surface_offdiag_identity),
# unlike the volume filter's, whose every term telescopes.
def surface_flux(r: dict, c: int, line: bool, fdelta=None) -> dict:
    """``surfacefilter!(firu, ru, c, true)`` (``line`` False) or the swap flux
    of ``dns_aid_surface`` (``line`` True: ``linefilter!`` off the diagonal,
    the same surface filter on it), 9 components keyed ``(i, j)``
    (src/NavierStokes.jl:368-369, 386-394)."""
    out = {}
    for i in range(3):
        for j in range(3):
            modes = tuple(POINT if (d == i or (line and d == j)) else VOLUME for d in range(3))
            out[(i, j)] = filter_coarse(r[(i, j)], c, positions_sigma(i, j), modes, fdelta)
    return out


def surface_offdiag_identity(u, p, visc, l, c):
    """Both sides of the identity the line filter rests on: the face average
    of the fine off-diagonal flux divergence, and the coarse divergence of the
    line-filtered flux (diagonal terms left out on both sides)."""
    n = u.shape[1]
    h, H = l / n, l / (n // c)
    r = get_r(stresstensor(u, visc, h), p)
    off = {k: (v if k[0] != k[1] else np.zeros_like(v)) for k, v in r.items()}
    fine = tensordivergence(off, h)
    lhs = face_filter(fine, c)
    rl = surface_flux(r, c, True)
    roff = {k: (v if k[0] != k[1] else np.zeros_like(v)) for k, v in rl.items()}
    return lhs, tensordivergence(roff, H)


def dns_aid_surface_steps(u, les, visc, l, c, tstop, cfl, doproject, fdelta=None, max_steps=None, t0=0.0):
    """Steps of the loop of ``dns_aid_surface`` (src/NavierStokes.jl:350-452):
    ``fiu`` the face-filtered DNS (divergence free on the LES grid, never
    projected), ``rfiu = sigma_H(fiu) + p_H I``; closures: the divergences of
    ``firu - rfiu`` (classic), of the swap flux ``diag(firu) + offdiag(fijru) -
    rfiu`` and of its symmetric part; each LES takes ``v += dt P(RHS_H(v))``,
    ``v += dt dsigma`` and a projection when ``doproject``.  Returns
    (u, les, t, steps)."""
    n = u.shape[1]
    h = l / n
    H = l / (n // c)
    les = {k: v.copy() for k, v in les.items()}
    t, it = t0, 0
    while t < tstop and (max_steps is None or it < max_steps):
        dt = min(propose_timestep(u, visc, cfl, h), tstop - t)
        t += dt
        it += 1
        du, p = project(rhs(u, visc, h), h, return_p=True)
        r = get_r(stresstensor(u, visc, h), p)
        firu = surface_flux(r, c, False, fdelta)
        fswap = surface_flux(r, c, True, fdelta)
        fiu = face_filter(u, c, fdelta)
        sfiu = stresstensor(fiu, visc, H)
        p_les = poisson_solve(divergence(tensordivergence(sfiu, H), H), H)
        rfiu = get_r(sfiu, p_les)
        s_classic = {k: firu[k] - rfiu[k] for k in firu}
        s_swap = {k: fswap[k] - rfiu[k] for k in fswap}
        dsig = {"classic": tensordivergence(s_classic, H), "swapfil": tensordivergence(s_swap, H),
                "swapfil_symm": tensordivergence(symmetrize(s_swap), H)}
        u = u + dt * du
        les["nomodel"] = les["nomodel"] + dt * project(rhs(les["nomodel"], visc, H), H)
        for k in ("classic", "swapfil", "swapfil_symm"):
            v = les[k] + dt * project(rhs(les[k], visc, H), H)
            v = v + dt * dsig[k]
            les[k] = project(v, H) if doproject else v
    return u, les, t, it
