"""Float64 NumPy restatement of the reference's 1-D ``Burgers`` module.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``): what the CUDA Burgers
path is compared with, and the timed CPU baseline; never part of the product.

Layout: a batch of samples is a ``(nsample, n)`` array, x fastest -- the
byte layout of the reference's ``zeros(nh, nsample)`` column-major matrices
(``src/Burgers.jl:273-307``).  ``u[:, i]`` sits on the right face of cell i
(staggered, ``points_stag``, ``src/Burgers.jl:82``); stresses sit at cell
centres (``points_coll``, ``:83``).  Index 0 here is the reference's 1.

Every sample advances with its own time step (the reference loops over the
samples, ``src/Burgers.jl:307``); the batched loops below mask finished
samples, which leaves each sample's arithmetic unchanged.
"""
from __future__ import annotations

import math

import numpy as np

from .ns import _splitmix


def spacing(l: float, n: int) -> float:
    """``spacing(g) = g.L / g.n`` (``src/Burgers.jl:31``)."""
    return l / n


def stress(u: np.ndarray, visc: float, h: float) -> np.ndarray:
    """``stress`` (``src/Burgers.jl:89-94``): ``-(u[i-1]+u[i])^2/8 +
    visc (u[i]-u[i-1])/h`` at the centre of cell i."""
    ua = np.roll(u, 1, axis=-1)
    ub = u
    return -((ua + ub) ** 2) / 8 + visc * (ub - ua) / h


def delta_stag(u: np.ndarray, h: float) -> np.ndarray:
    """``δ_stag`` (``src/Burgers.jl:86``): ``(u[i] - u[i-1]) / h``."""
    return (u - np.roll(u, 1, axis=-1)) / h


def delta_coll(p: np.ndarray, h: float) -> np.ndarray:
    """``δ_coll`` (``src/Burgers.jl:87``): ``(p[i+1] - p[i]) / h``."""
    return (np.roll(p, -1, axis=-1) - p) / h


def cfl(u: np.ndarray, visc: float, h: float) -> np.ndarray:
    """``cfl`` (``src/Burgers.jl:97-101``), one value per sample."""
    return np.minimum(h / np.max(np.abs(u), axis=-1), h * h / visc)


def rhs(u, visc, h):
    """``rhs!`` (``src/Burgers.jl:103-109``)."""
    return delta_coll(stress(u, visc, h), h)


def timestep(u, visc, h, dt):
    """``timestep!`` (``src/Burgers.jl:112-118``): forward Euler; ``dt`` per
    sample (shape ``(nsample, 1)``) or scalar."""
    return u + dt * delta_coll(stress(u, visc, h), h)


def rk4_timestep(u, visc, h, dt):
    """``rk4_timestep!`` (``src/Burgers.jl:120-142``), classic RK4 stages."""
    k1 = rhs(u, visc, h)
    k2 = rhs(u + dt / 2 * k1, visc, h)
    k3 = rhs(u + dt / 2 * k2, visc, h)
    k4 = rhs(u + dt * k3, visc, h)
    return u + dt / 6 * (k1 + 2 * k2 + 2 * k3 + k4)


# ---------------------------------------------------------------- filters

def gaussian_weights(h: float, delta: float, nsigma: float = 3.0):
    """``gaussian_weights`` (``src/Burgers.jl:146-156``): ``(R, w)`` with
    ``R = round(nσ σ)``, ``σ^2 = (Δ/h)^2/12``; ``[1]`` for ``Δ < 1e-15``.
    Julia's ``round`` ties to even, as Python's does."""
    s2 = (delta / h) ** 2 / 12
    R = int(round(nsigma * math.sqrt(s2)))
    if delta < 1.0e-15:
        return R, np.ones(1)
    r = np.arange(-R, R + 1, dtype=np.float64)
    w = np.exp(-(r**2) / (2 * s2))
    return R, w / w.sum()


def tophat_weights(comp: int):
    """``tophat_weights`` (``src/Burgers.jl:158-162``); odd ``comp`` only
    (``R = comp ÷ 2`` must give ``2R + 1 == comp`` weights)."""
    assert comp % 2 == 1
    return comp // 2, np.full(comp, 1.0 / comp)


def les_kernel(h: float, H: float, delta_ratio: float, kind: str):
    """The LES kernel of ``dns_aided_les`` (``src/Burgers.jl:356-363``)."""
    delta = H * delta_ratio
    if kind == "tophat":
        lescomp = int(round(delta / h))
        R = lescomp // 2
        return tophat_weights(2 * R + 1)
    if kind == "gaussian":
        return gaussian_weights(h, delta)
    raise ValueError(kind)


def build_doublekernel(F, G):
    """``build_doublekernel`` (``src/Burgers.jl:218-233``): the discrete
    convolution of two centred kernels, summed over j ascending."""
    I, f = F
    J, g = G
    K = I + J
    w = np.zeros(2 * K + 1)
    for k in range(-K, K + 1):
        s = 0.0
        for j in range(-J, J + 1):
            i = k - j
            if abs(i) <= I:
                s += f[I + i] * g[J + j]
        w[k + K] = s
    return K, w


def kernels(nh: int, nH: int, l: float, delta_ratio: float, kind: str):
    """(fvm, les, double) kernels of one LES grid (``src/Burgers.jl:355-364``)."""
    comp = nh // nH
    fvm = tophat_weights(comp)
    les = les_kernel(l / nh, l / nH, delta_ratio, kind)
    return fvm, les, build_doublekernel(fvm, les)


def filter_at(u: np.ndarray, kernel, pos: np.ndarray) -> np.ndarray:
    """``lazyfilter`` (``src/Burgers.jl:164-172``) sampled at fine indices
    ``pos``: ``sum_r w[r+R] u[pos+r]`` with periodic wrap."""
    R, w = kernel
    n = u.shape[-1]
    idx = (pos[:, None] + np.arange(-R, R + 1)[None, :]) % n
    return u[..., idx] @ w


def coarse_positions(nh: int, nH: int, stag: bool) -> np.ndarray:
    """``lazycoarsegrain`` (``src/Burgers.jl:174-180``): coarse cell I reads
    fine index ``I comp - !stag a`` (1-based), ``a = comp ÷ 2``."""
    comp = nh // nH
    a = comp // 2
    I1 = np.arange(1, nH + 1)
    return I1 * comp - (0 if stag else a) - 1


def coarse_filter(u: np.ndarray, kernel, nH: int, stag: bool) -> np.ndarray:
    """``lazycoarsegrain(gH, lazyfilter(u, kernel), stag)``."""
    return filter_at(u, kernel, coarse_positions(u.shape[-1], nH, stag))


def closure_terms(u: np.ndarray, visc: float, l: float, nH: int, les, double):
    """The filtered quantities of one ``dns_aided_les`` step
    (``src/Burgers.jl:397-412``): ``fsu, vsu, vu, sVU, svu`` on the LES grid."""
    nh = u.shape[-1]
    h, H = l / nh, l / nH
    su = stress(u, visc, h)
    fsu = coarse_filter(su, les, nH, False)
    vsu = coarse_filter(su, double, nH, False)
    vu = coarse_filter(u, double, nH, True)
    pc = coarse_positions(nh, nH, False)
    VUl = filter_at(u, double, (pc - 1) % nh)
    VUr = filter_at(u, double, pc)
    sVU = -((VUl + VUr) ** 2) / 8 + visc * (VUr - VUl) / h
    svu = stress(vu, visc, H)
    return fsu, vsu, vu, sVU, svu


# ---------------------------------------------------------- initial field

def uniform01(seed: int, count: int) -> np.ndarray:
    """Counter-based uniforms in (0, 1): ``((splitmix64(seed φ + k) >> 11)
    + 1/2) 2^-53`` -- the project's replacement for ``rand(rng)`` on a
    ``Xoshiro(i)`` stream (``src/Burgers.jl:192``)."""
    with np.errstate(over="ignore"):
        k = np.arange(count, dtype=np.uint64)
        z = _splitmix(np.uint64(seed) * np.uint64(0x9E3779B97F4A7C15) + k)
    return ((z >> np.uint64(11)).astype(np.float64) + 0.5) * 2.0**-53


def randomfield(n: int, l: float, kpeak: float, totalenergy: float, seed: int) -> np.ndarray:
    """``randomfield`` with ``bump_profile`` (``src/Burgers.jl:192-202``):
    ``c_k = (k/k0)^4 exp(-2 (k/k0)^2 + 2πi U_k)``, ``a = irfft(n c, n)``,
    scaled to kinetic energy ``sum(a^2)/2 h``."""
    k = np.arange(n // 2 + 1, dtype=np.float64)
    U = uniform01(seed, n // 2 + 1)
    amp = (k / kpeak) ** 4 * np.exp(-2 * (k / kpeak) ** 2)
    c = amp * (np.cos(2 * np.pi * U) + 1j * np.sin(2 * np.pi * U))
    a = np.fft.irfft(c * n, n)
    etot = np.sum(a**2) / 2 * (l / n)
    return math.sqrt(totalenergy / etot) * a


def randomfields(nsample: int, n: int, l: float, kpeak: float, totalenergy: float, seed: int):
    """Sample s uses the phase stream ``seed + s`` (the reference seeds
    sample i with ``Xoshiro(i)``, ``src/Burgers.jl:308``)."""
    return np.stack([randomfield(n, l, kpeak, totalenergy, seed + s) for s in range(nsample)])


# ---------------------------------------------------------------- solvers

def dns(u0: np.ndarray, visc: float, l: float, tstop: float, cfl_factor: float,
        scheme: str = "euler", max_steps: int | None = None, t0=None):
    """The time loop of ``create_dns`` (``src/Burgers.jl:522-545``): per
    sample ``dt = min(cfl_factor cfl(u), tstop - t)`` until ``t >= tstop``.
    Returns (u, t, steps)."""
    u = u0.copy()
    B, n = u.shape
    h = l / n
    t = np.zeros(B) if t0 is None else t0.copy()
    steps = np.zeros(B, dtype=np.int64)
    while True:
        act = t < tstop
        if max_steps is not None:
            act &= steps < max_steps
        if not act.any():
            break
        dt = np.minimum(cfl_factor * cfl(u, visc, h), tstop - t)
        dt = np.where(act, dt, 0.0)[:, None]
        un = timestep(u, visc, h, dt) if scheme == "euler" else rk4_timestep(u, visc, h, dt)
        u = np.where(act[:, None], un, u)
        t = np.where(act, t + dt[:, 0], t)
        steps += act
    return u, t, steps


LES_NAMES = ("nomodel", "class_m", "class_p", "swapfil")


def dns_aided_les(ustart: np.ndarray, nH: int, visc: float, l: float, delta_ratio: float,
                  kind: str, tstop: float, cfl_factor: float, max_steps: int | None = None,
                  state=None):
    """``dns_aided_les`` (``src/Burgers.jl:350-445``): forward-Euler DNS with
    four LES in lockstep -- no model, classic ``vsu - sVU``, classic+flux
    ``vsu - svu`` and the exact classic+flux+div ``fsu - svu`` (the
    "swapfil" closure) -- each LES stress ``s_H(v) + correction``.

    ``state`` = (u, t, steps, {name: v}) continues an earlier call (the
    GPU runs in chunks of ``max_steps``).  Returns the same tuple."""
    B, nh = ustart.shape
    h, H = l / nh, l / nH
    _, les, double = kernels(nh, nH, l, delta_ratio, kind)
    if state is None:
        u = ustart.copy()
        t = np.zeros(B)
        steps = np.zeros(B, dtype=np.int64)
        v0 = coarse_filter(u, double, nH, True)
        V = {k: v0.copy() for k in LES_NAMES}
    else:
        u, t, steps, V = state
        u, t, steps = u.copy(), t.copy(), steps.copy()
        V = {k: x.copy() for k, x in V.items()}
    done = np.zeros(B, dtype=np.int64)
    while True:
        act = t < tstop
        if max_steps is not None:
            act &= done < max_steps
        if not act.any():
            break
        dt = np.minimum(cfl_factor * cfl(u, visc, h), tstop - t)
        dt = np.where(act, dt, 0.0)
        dtc = dt[:, None]
        fsu, vsu, vu, sVU, svu = closure_terms(u, visc, l, nH, les, double)
        corr = {"nomodel": None, "class_m": (vsu, sVU), "class_p": (vsu, svu),
                "swapfil": (fsu, svu)}
        for name in LES_NAMES:
            s = stress(V[name], visc, H)
            if corr[name] is not None:
                a, b = corr[name]
                s = s + a - b
            vn = V[name] + dtc * delta_coll(s, H)
            V[name] = np.where(act[:, None], vn, V[name])
        un = u + dtc * delta_coll(stress(u, visc, h), h)
        u = np.where(act[:, None], un, u)
        t = np.where(act, t + dt, t)
        steps += act
        done += act
    return u, t, steps, V


def filtered_dns(u: np.ndarray, nH: int, l: float, delta_ratio: float, kind: str):
    """``dns_ref_fil`` and ``dns_fil`` (``src/Burgers.jl:441-442``)."""
    nh = u.shape[-1]
    _, _, double = kernels(nh, nH, l, delta_ratio, kind)
    fil = filter_at(u, double, np.arange(nh))
    return fil, fil[:, coarse_positions(nh, nH, True)]


def compute_errors(V: dict, dns_fil: np.ndarray) -> dict:
    """``compute_errors`` (``src/Burgers.jl:909-916``): Frobenius norm over
    all samples, ``norm(u - dns_fil) / norm(dns_fil)``."""
    nr = np.linalg.norm(dns_fil)
    return {k: float(np.linalg.norm(V[k] - dns_fil) / nr) for k in V}


def compute_fractions(u: np.ndarray, visc: float, l: float, nH: int, delta_ratio: float, kind: str):
    """``compute_fractions`` (``src/Burgers.jl:1022-1116``): mean share of
    |classic|, |flux|, |div| in the total sub-filter stress."""
    nh = u.shape[-1]
    _, les, double = kernels(nh, nH, l, delta_ratio, kind)
    fsu, vsu, vu, sVU, svu = closure_terms(u, visc, l, nH, les, double)
    sc, sf, sd = vsu - sVU, sVU - svu, fsu - vsu
    tot = np.abs(sc) + np.abs(sf) + np.abs(sd) + np.finfo(np.float64).eps
    fr = np.stack([np.abs(sc) / tot, np.abs(sf) / tot, np.abs(sd) / tot])  # (3, B, nH)
    per_sample = fr.sum(axis=2) / nH
    return per_sample.sum(axis=1) / u.shape[0]


def compute_dissipation(u: np.ndarray, visc: float, l: float, nH: int, delta_ratio: float, kind: str):
    """``compute_dissipation`` (``src/Burgers.jl:447-520``): ``δ_stag(vu) σ``
    for the classic, classic+flux and exact closures, shape (3, B, nH)."""
    nh = u.shape[-1]
    _, les, double = kernels(nh, nH, l, delta_ratio, kind)
    fsu, vsu, vu, sVU, svu = closure_terms(u, visc, l, nH, les, double)
    dv = delta_stag(vu, l / nH)
    return np.stack([dv * (vsu - sVU), dv * (vsu - svu), dv * (fsu - svu)])


# ----------------------------------------------------------- Smagorinsky

def smagorinsky_fields(U: np.ndarray, visc: float, l: float, nH: int, delta_ratio: float, kind: str):
    """``smagorinsky_fields`` (``src/Burgers.jl:547-688``) on the DNS grid:
    classic ``Th = filter_d(σ) - σ_h(filter_d u)``, ``Sh = -(Δ^2+H^2)|δu|δu``
    with ``δu`` the fine difference of the double-filtered velocity, and the
    discrete ``TH``, ``SH`` built from the coarse difference
    ``u[i+a] - u[i-a-1]`` over H with the LES-kernel-filtered stress."""
    B, nh = U.shape
    comp = nh // nH
    a = comp // 2
    h, H = l / nh, l / nH
    delta = H * delta_ratio
    _, les, double = kernels(nh, nH, l, delta_ratio, kind)
    allp = np.arange(nh)
    ud = filter_at(U, double, allp)
    sig = stress(U, visc, h)
    s1 = filter_at(sig, double, allp)
    th = s1 - stress(ud, visc, h)
    du = delta_stag(ud, h)
    sh = -(delta**2 + H**2) * np.abs(du) * du
    s1H = filter_at(sig, les, allp)
    ul = np.roll(ud, a + 1, axis=-1)   # ud[i - a - 1]
    ur = np.roll(ud, -a, axis=-1)      # ud[i + a]
    tH = s1H - (-((ul + ur) ** 2) / 8 + visc * (ur - ul) / H)
    dH = (ur - ul) / H
    sH = -(delta**2 + H**2) * np.abs(dH) * dH
    return {"Sh": sh, "Th": th, "D_Sh": sh * du, "D_Th": th * du,
            "SH": sH, "TH": tH, "D_SH": sH * dH, "D_TH": tH * dH, "Ubar": ud}


def smagorinsky_theta(f: dict):
    """``θ^2 = -dot(S, T) / dot(S, S)`` (``smagorinsky.jl:32-45``) for the
    classic and the discrete fit: returns (θ2_classic, θ2_discrete); the
    reference takes ``sqrt``, which fails for a negative fit."""
    def fit(S, T):
        S, T = S.ravel(), T.ravel()
        return float(-np.dot(S, T) / np.dot(S, S))
    return fit(f["Sh"], f["Th"]), fit(f["SH"], f["TH"])


def smagorinsky_rhs(u: np.ndarray, visc: float, H: float, C: float):
    """``smagorinsky_rhs!`` (``src/Burgers.jl:773-786``)."""
    s = stress(u, visc, H)
    du = delta_stag(u, H)
    smag = -C * np.abs(du) * du
    return delta_coll(s - smag, H)


def solve_smagorinsky(ustart: np.ndarray, visc: float, l: float, nH: int, delta_ratio: float,
                      kind: str, theta: float, tstop: float, cfl_factor: float = 0.3,
                      max_steps: int | None = None):
    """``solve_smagorinsky`` (``src/Burgers.jl:690-771``): the filtered
    initial field advanced with the Smagorinsky closure ``C = θ^2 (Δ^2+H^2)``.

    The reference's stages update the running state in place
    (``axpy!(dt/2, k1, ubar)`` then ``axpy!(dt/2, k2, ubar)`` then
    ``axpy!(dt, k3, ubar)``), so stage 3 sees ``u0 + dt/2 (k1 + k2)`` and
    stage 4 ``u0 + dt/2 (k1 + k2) + dt k3``; the update is the classic
    ``u0 + dt/6 (k1 + 2k2 + 2k3 + k4)``.  Restated as written."""
    B, nh = ustart.shape
    H = l / nH
    delta = H * delta_ratio
    C = theta**2 * (delta**2 + H**2)
    _, _, double = kernels(nh, nH, l, delta_ratio, kind)
    ub = coarse_filter(ustart, double, nH, True)
    t = np.zeros(B)
    steps = np.zeros(B, dtype=np.int64)
    while True:
        act = t < tstop
        if max_steps is not None:
            act &= steps < max_steps
        if not act.any():
            break
        dt = np.minimum(cfl_factor * cfl(ub, visc, H), tstop - t)
        dt = np.where(act, dt, 0.0)
        t = np.where(act, t + dt, t)
        d = dt[:, None]
        u0 = ub
        k1 = smagorinsky_rhs(ub, visc, H, C)
        ub = ub + d / 2 * k1
        k2 = smagorinsky_rhs(ub, visc, H, C)
        ub = ub + d / 2 * k2
        k3 = smagorinsky_rhs(ub, visc, H, C)
        ub = ub + d * k3
        k4 = smagorinsky_rhs(ub, visc, H, C)
        un = u0 + d / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
        ub = np.where(act[:, None], un, u0)
        steps += act
    return ub, t, steps
