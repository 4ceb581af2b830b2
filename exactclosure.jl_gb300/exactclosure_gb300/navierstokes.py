"""Host-side mirror of the reference's ``NavierStokes`` module (``src/N.jl``)
over the libexc C ABI.

Operator functions keep the reference's names and argument meaning; fields
are CUDA tensors (torch is used only to own device memory and streams) shaped
``(3, n, n, n)`` / ``(n, n, n)`` in the reference's byte layout (x fastest,
component slowest).  Every call goes through ``libexc.so``; nothing here
computes on the CPU.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from ._lib import (EXC_F32, EXC_F64, EXC_FILTER_FACE, EXC_FILTER_VOLUME, CaseDesc, call, lib)

KINDS = {"volume": EXC_FILTER_VOLUME, "face": EXC_FILTER_FACE}


def _torch():
    import torch  # device memory and streams only

    return torch


def _prec(t) -> int:
    torch = _torch()
    if t.dtype == torch.float64:
        return EXC_F64
    if t.dtype == torch.float32:
        return EXC_F32
    raise TypeError(f"fields must be float64 or float32, got {t.dtype}")


def _ptr(t) -> C.c_void_p:
    if not t.is_cuda or not t.is_contiguous():
        raise ValueError("fields must be contiguous CUDA tensors")
    return C.c_void_p(t.data_ptr())


def _stream():
    return C.c_void_p(_torch().cuda.current_stream().cuda_stream)


def _taps(fdelta):
    if fdelta is None or len(fdelta) <= 1:
        return None, 0
    a = np.ascontiguousarray(fdelta, dtype=np.float64)
    return a.ctypes.data_as(C.POINTER(C.c_double)), len(a)


@dataclass(frozen=True)
class Grid:
    """``Grid{3}(l, n)`` (``src/N.jl:22-25``)."""

    l: float
    n: int

    @property
    def h(self) -> float:
        return self.l / self.n


def tensordivergence(du, u, visc: float, grid: Grid, doadd: bool = False):
    """``tensordivergence!(du, stresstensor(u, visc), doadd)`` (``src/N.jl:94-160``)."""
    call("exc_tensordivergence", _prec(u), grid.n, grid.l, visc, _ptr(u), _ptr(du), int(doadd), _stream())
    return du


def tensordivergence_tensor(du, s, grid: Grid, doadd: bool = False):
    """``tensordivergence!`` (6 components) or ``tensordivergence_nonsym!`` (9)
    with an explicit tensor ``s`` shaped ``(6|9, n, n, n)`` (``src/N.jl:120-200``)."""
    call("exc_tensordivergence_tensor", _prec(s), grid.n, grid.l, s.shape[0], _ptr(s), _ptr(du), int(doadd),
         _stream())
    return du


def stresstensor(s6, u, visc: float, grid: Grid):
    """Materialised ``stresstensor(u, visc)`` (``src/N.jl:94-118``) into ``s6``."""
    call("exc_stresstensor", _prec(u), grid.n, grid.l, visc, _ptr(u), _ptr(s6), _stream())
    return s6


def divergence(d, u, grid: Grid):
    """``divergence!(d, u)`` (``src/N.jl:222-238``)."""
    call("exc_divergence", _prec(u), grid.n, grid.l, _ptr(u), _ptr(d), _stream())
    return d


def pressuregradient(u, p, grid: Grid):
    """``pressuregradient!(u, p)`` (``src/N.jl:240-254``)."""
    call("exc_pressuregradient", _prec(u), grid.n, grid.l, _ptr(u), _ptr(p), _stream())
    return u


class PoissonSolver:
    """``poissonsolver(grid, backend)`` (``src/N.jl:202-220``): owns the
    spectral work array and FFT tables of one grid on the device."""

    def __init__(self, grid: Grid, precision: int = EXC_F64, engine: int = 0):
        self.grid = grid
        self.precision = precision
        h = C.c_void_p()
        call("exc_poisson_create", precision, grid.n, grid.l, C.byref(h))
        self._h = h
        if engine:
            call("exc_poisson_set_engine", h, engine)

    def solve(self, p, d):
        """``p`` with ``L_h p = d`` and zero mean (``src/N.jl:262-301``)."""
        call("exc_poisson_solve", self._h, _ptr(d), _ptr(p), _stream())
        return p

    def project(self, u, p=None):
        """``project!(u, poisson)`` (``src/N.jl:256-307``), in place; the
        pressure goes to ``p`` when given."""
        call("exc_project", self._h, _ptr(u), _ptr(p) if p is not None else None, _stream())
        return u

    def close(self):
        if getattr(self, "_h", None):
            lib().exc_poisson_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def device_faults() -> int:
    """Device fault flags recorded since the last call (0 = none)."""
    v = C.c_int()
    call("exc_device_faults", C.byref(v))
    return v.value


def device_sync(stream=None) -> int:
    """Synchronise the stream (default: torch's current stream) and check the
    device fault flags: raises ExcError (EXC_ERR_TIMEOUT) when a bounded
    device wait gave up, else returns 0."""
    v = C.c_int()
    st = C.c_void_p(stream) if stream is not None else _stream()
    call("exc_device_sync", st, C.byref(v))
    return v.value


def debug_wait_drill(flags: int):
    """Test hook of the bounded device waits (0: normal operation).  Bit 0:
    the RHS sweep's TMA tiles issue no copy; bit 1: the tensor-core
    convolution issues no copy; their waits give up after 64 polls."""
    call("exc_debug_wait_drill", int(flags))


def poissonsolver(grid: Grid, precision: int = EXC_F64, engine: int = 0) -> PoissonSolver:
    return PoissonSolver(grid, precision, engine)


def project(u, poisson: PoissonSolver, p=None):
    return poisson.project(u, p)


def propose_timestep(u, visc: float, cfl: float, grid: Grid) -> float:
    """``propose_timestep`` (``src/N.jl:348-356``)."""
    dt = C.c_double()
    call("exc_propose_timestep", _prec(u), grid.n, grid.l, visc, cfl, _ptr(u), C.byref(dt), _stream())
    return dt.value


def apply_filter(ubar, u, ratio: int, kind: str = "volume", fdelta=None):
    """``lazycoarsegrain(faces[i], lazyfilter(u_i, GDH))`` for each component
    (volume) or the face average (face), materialised into ``ubar``
    (``src/N.jl:655-698``, ``src/N.jl:1228-1237`` without the projection)."""
    t, nt = _taps(fdelta)
    call("exc_filter", _prec(u), u.shape[1], ratio, KINDS[kind], t, nt, _ptr(u), _ptr(ubar), _stream())
    return ubar


def apply_DHpi(ubar, u, poisson_les: PoissonSolver, ratio: int, fdelta=None):
    """``apply_DHpi(ubar, u, poisson, GDH)`` (``src/N.jl:1228-1237``)."""
    apply_filter(ubar, u, ratio, "volume", fdelta)
    return poisson_les.project(ubar)


def get_rDHi(r9, u, p, visc: float, grid: Grid, ratio: int, fdelta=None):
    """``get_rDHi(get_r(stresstensor(u), p), GDHi, g_dns, g_les)``
    (``src/N.jl:1022-1073``), materialised into ``r9`` (9 LES arrays)."""
    t, nt = _taps(fdelta)
    call("exc_closure_flux", _prec(u), grid.n, ratio, grid.l, visc, t, nt, _ptr(u), _ptr(p), _ptr(r9), _stream())
    return r9


def get_sigmaDH(s6, u, visc: float, grid: Grid, ratio: int, fdelta=None):
    """``get_sigmaDH(stresstensor(u), g_dns, g_les, GDH)`` (``src/N.jl:1088-1115``)."""
    t, nt = _taps(fdelta)
    call("exc_filtered_stress", _prec(u), grid.n, ratio, grid.l, visc, t, nt, _ptr(u), _ptr(s6), _stream())
    return s6


class Case:
    """A DNS with attached LES grids advanced by RK4 with the exact closure at
    every stage (the ``dnsaid_project`` loop, ``src/N.jl:1239-1332``), fully
    device resident.  Host arrays are float64 ``(3, n, n, n)``."""

    def __init__(self, n: int, l: float = 1.0, visc: float = 1 / 2000, cfl: float = 0.3,
                 precision: int = EXC_F64, les=(), stream: int | None = None):
        d = CaseDesc()
        d.n, d.l, d.visc, d.cfl, d.precision = n, l, visc, cfl, precision
        d.nles = len(les)
        for i, (ratio, kind) in enumerate(les):
            d.les[i].ratio = ratio
            d.les[i].kind = KINDS[kind] if isinstance(kind, str) else kind
        self.desc = d
        self.n, self.l, self.visc = n, l, visc
        self.les_list = [(r, k) for r, k in les]
        h = C.c_void_p()
        call("exc_case_create", C.byref(d), C.c_void_p(stream) if stream else None, C.byref(h))
        self._h = h

    def _buf(self, shape):
        a = np.empty(shape, dtype=np.float64)
        return a, a.ctypes.data_as(C.POINTER(C.c_double))

    def init_random(self, kpeak: float, energy: float = 1.0, seed: int = 0):
        """``randomfield(peak_profile, ...)`` (``src/N.jl:394-476``)."""
        call("exc_case_init_random", self._h, kpeak, energy, seed)

    def set_velocity(self, u: np.ndarray):
        a = np.ascontiguousarray(u, dtype=np.float64)
        assert a.shape == (3, self.n, self.n, self.n)
        call("exc_case_set_velocity", self._h, a.ctypes.data_as(C.POINTER(C.c_double)))

    def velocity(self) -> np.ndarray:
        a, p = self._buf((3, self.n, self.n, self.n))
        call("exc_case_get_velocity", self._h, p)
        return a

    def les(self, index: int, which: str = "exact") -> np.ndarray:
        """LES field: 'target' (filtered DNS), 'exact', 'nomodel' or 'closure'."""
        w = {"target": 0, "exact": 1, "nomodel": 2, "closure": 3, "learned": 4, "target_last": 5}[which]
        m = self.n // self.les_list[index][0]
        a, p = self._buf((3, m, m, m))
        call("exc_case_get_les", self._h, index, w, p)
        return a

    def get_velocity_into(self, out: np.ndarray):
        """Download the DNS velocity into a caller-owned (e.g. pinned) array."""
        assert out.dtype == np.float64 and out.flags.c_contiguous and out.size == 3 * self.n ** 3
        call("exc_case_get_velocity", self._h, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def device_ptr(self) -> int:
        """Device address of the current DNS velocity (zero-copy callers)."""
        p = C.c_void_p()
        call("exc_case_device_ptr", self._h, 0, C.byref(p))
        return p.value

    def launches_per_step(self) -> int:
        k = C.c_int()
        call("exc_case_launches_per_step", self._h, C.byref(k))
        return k.value

    def reset_les(self):
        """Restart every LES state from the filtered DNS (and the clock from 0)."""
        call("exc_case_reset_les", self._h)

    def les_error(self, index: int, which: str = "exact") -> float:
        """Relative L2 error of an LES state ('exact', 'nomodel', 'learned')
        against the filtered DNS (``compute_errors``, ``src/N.jl:1334-1349``)."""
        e = C.c_double()
        call("exc_case_les_error", self._h, index, {"exact": 1, "nomodel": 2, "learned": 4}[which], C.byref(e))
        return e.value

    def snapshot(self, index: int, u_dev, m_dev):
        """Device copy of (filtered DNS, exact closure) at stage 1 of the last step
        into CUDA tensors of the case precision, shaped (3, m, m, m)."""
        call("exc_case_snapshot", self._h, index, C.c_void_p(u_dev.data_ptr()), C.c_void_p(m_dev.data_ptr()))

    def attach_net(self, index: int, net):
        """Drive a learned-closure LES on LES grid ``index`` (None detaches)."""
        call("exc_case_attach_net", self._h, index, net.handle if net is not None else None)
        self._net = net

    def set_fallback(self, index: int, e_lo: float = 0.0, e_hi: float = float("inf")):
        """No-model fallback of the learned LES on grid ``index``: when its
        kinetic energy is not finite or leaves [e_lo, e_hi], it goes back to
        its last state inside the band and continues without the net."""
        call("exc_case_set_fallback", self._h, index, e_lo, e_hi)

    def fallback_engaged(self, index: int) -> bool:
        v = C.c_int()
        call("exc_case_fallback", self._h, index, C.byref(v))
        return bool(v.value)

    def step(self, nsteps: int = 1, dt: float = 0.0):
        call("exc_case_step", self._h, nsteps, dt)

    def errors(self, index: int) -> tuple[float, float]:
        e = (C.c_double * 2)()
        call("exc_case_errors", self._h, index, e)
        return e[0], e[1]

    def time(self) -> tuple[float, float]:
        t, dt = C.c_double(), C.c_double()
        call("exc_case_time", self._h, C.byref(t), C.byref(dt))
        return t.value, dt.value

    def energy(self) -> float:
        e = C.c_double()
        call("exc_case_energy", self._h, C.byref(e))
        return e.value

    def dissipation(self) -> float:
        """Viscous dissipation ``visc <|grad u|^2>`` of the DNS (FP64)."""
        e = C.c_double()
        call("exc_case_dissipation", self._h, C.byref(e))
        return e.value

    def spectrum(self) -> np.ndarray:
        ns = (2 * (self.n // 2)) // 3
        a, p = self._buf((ns,))
        call("exc_case_spectrum", self._h, p, ns)
        return a

    def sync(self):
        call("exc_case_sync", self._h)

    def close(self):
        if getattr(self, "_h", None):
            lib().exc_case_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# The reference's driver `dnsaid_project` (src/N.jl:1239-1332)
# ---------------------------------------------------------------------------
DNSAID_FIELDS = ("u_les", "u_nomo", "u_c", "u_cf", "u_cfd", "u_cfd_symm")
# the paper's dns_aid_volavg (src/NavierStokes.jl:141-304): target fu, four LES
PAPER_FIELDS = ("fu", "nomodel", "classic", "swapfil", "swapfil_symm")


def gaussian(h: float, delta: float, nsigma: float) -> np.ndarray:
    """``gaussian`` (``src/N.jl:599-607``), a host array like the reference's;
    ``delta == 0`` gives ``[1]``."""
    if delta < 1e-15:
        return np.ones(1)
    sig = delta / np.sqrt(12)
    r = int(round(nsigma * sig / h))
    x = h * np.arange(-r, r + 1)
    w = np.exp(-(x**2) / (2 * sig**2))
    return w / w.sum()


class DnsAid:
    """Handle of ``exc_dnsaid_*``: a DNS with the five LES of
    ``dnsaid_project``, FP64."""

    def __init__(self, n: int, l: float, visc: float, ratio: int, fdelta=None, stream=None):
        from ._lib import DnsAidDesc

        self.n, self.l, self.visc, self.ratio = n, l, visc, ratio
        self.m = n // ratio
        self._fd = None if fdelta is None or len(fdelta) <= 1 else np.ascontiguousarray(fdelta, dtype=np.float64)
        desc = DnsAidDesc(n, l, visc, ratio,
                          None if self._fd is None else self._fd.ctypes.data_as(C.POINTER(C.c_double)),
                          0 if self._fd is None else len(self._fd))
        h = C.c_void_p()
        call("exc_dnsaid_create", C.byref(desc), stream, C.byref(h))
        self._h = h
        self.fields = DNSAID_FIELDS

    def set_paper(self, doproject: bool = True, filter: str = "volume"):
        """Run the paper's volume-average driver ``dns_aid_volavg``
        (src/NavierStokes.jl:141-304), or with ``filter="surface"`` its
        surface-average driver ``dns_aid_surface`` (src/NavierStokes.jl:306-468),
        instead of ``dnsaid_project``; call before ``start``.  Fields:
        ``PAPER_FIELDS``."""
        if filter not in ("volume", "surface"):
            raise ValueError("filter must be 'volume' or 'surface'")
        call("exc_dnsaid_set_paper" if filter == "volume" else "exc_dnsaid_set_surface", self._h,
             1 if doproject else 0)
        self.fields = PAPER_FIELDS

    def init_random(self, profile: str = "power", param: float = -5 / 3, energy: float = 1.0, seed: int = 0):
        call("exc_dnsaid_init_random", self._h, {"peak": 0, "power": 1}[profile], param, energy, seed)

    def set_velocity(self, u: np.ndarray):
        a = np.ascontiguousarray(u, dtype=np.float64)
        call("exc_dnsaid_set_velocity", self._h, a.ctypes.data_as(C.POINTER(C.c_double)))

    def velocity(self) -> np.ndarray:
        out = np.empty((3, self.n, self.n, self.n))
        call("exc_dnsaid_get_velocity", self._h, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def warmup(self, twarm: float, cfl: float, max_steps: int = 0) -> int:
        s = C.c_int()
        call("exc_dnsaid_warmup", self._h, twarm, cfl, max_steps, C.byref(s))
        return s.value

    def start(self):
        call("exc_dnsaid_start", self._h)

    def step(self, tstop: float, cfl: float, max_steps: int = 0) -> int:
        s = C.c_int()
        call("exc_dnsaid_step", self._h, tstop, cfl, max_steps, C.byref(s))
        return s.value

    def time(self):
        t, s = C.c_double(), C.c_int()
        call("exc_dnsaid_time", self._h, C.byref(t), C.byref(s))
        return t.value, s.value

    def get(self, which: str) -> np.ndarray:
        out = np.empty((3, self.m, self.m, self.m))
        call("exc_dnsaid_get", self._h, self.fields.index(which), out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def relerr(self) -> dict:
        """The paper drivers' ``|v - fu| / |fu|`` of the four LES, on the device."""
        e = np.empty(4)
        call("exc_dnsaid_relerr", self._h, e.ctypes.data_as(C.POINTER(C.c_double)))
        return dict(zip(self.fields[1:], e.tolist()))

    def errors(self) -> dict:
        e = np.empty(5)
        call("exc_dnsaid_errors", self._h, e.ctypes.data_as(C.POINTER(C.c_double)))
        return dict(zip(self.fields[1:], e.tolist()))

    def close(self):
        if getattr(self, "_h", None):
            lib().exc_dnsaid_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def getsetup(**kw) -> dict:
    """``getsetup`` (``src/N.jl:712-723``): the reference's defaults (DNS
    500^3, LES 100^3, visc 2e-4, Gaussian width 2H with 2 sigmas), plus the
    driver's warm-up/stop times, CFL and initial spectrum (``src/N.jl:1239-1262``);
    keywords override."""
    s = dict(l=1.0, n_dns=500, n_les=100, visc=2.0e-4, Δ_ratio=2, nσ=2, twarm=0.1, tstop=0.1, cfl=0.4,
             profile=("power", -5 / 3), seed=0)
    s.update(kw)
    return s


def dnsaid_project(setup: dict, stream=None) -> dict:
    """``dnsaid_project`` (``src/N.jl:1239-1332``): warm-up, then the DNS and
    five LES in lockstep; returns ``u_les`` (the filtered DNS) and the five
    LES fields, plus their ``compute_errors``."""
    n, m, l = setup["n_dns"], setup["n_les"], setup["l"]
    ratio = n // m
    H = l / m
    fdelta = gaussian(l / n, setup["Δ_ratio"] * H, setup["nσ"])
    d = DnsAid(n, l, setup["visc"], ratio, fdelta, stream)
    kind, param = setup["profile"]
    d.init_random(kind, param, 1.0, setup["seed"])
    d.warmup(setup["twarm"], setup["cfl"])
    d.start()
    d.step(setup["tstop"], setup["cfl"])
    out = {k: d.get(k) for k in DNSAID_FIELDS}
    out["errors"] = d.errors()
    d.close()
    return out


def testcase(n_dns: int, viscosity: float, seed: int = 123, l: float = 1.0, kpeak: float = 5.0,
             compression=(5, 3), totalenergy: float = 0.5) -> dict:
    """``testcase`` (``src/NavierStokes.jl:14-35``): a DNS grid with one LES
    grid per compression ratio (each must divide ``n_dns``), the peak profile
    with ``kpeak`` and ``totalenergy`` of the initial field, and its seed."""
    if any(n_dns % c for c in compression):
        raise ValueError("every compression must divide n_dns")
    return dict(l=l, n_dns=n_dns, n_les=[n_dns // c for c in compression], compression=list(compression),
                viscosity=viscosity, seed=seed, kpeak=kpeak, totalenergy=totalenergy)


def smallcase() -> dict:
    """``smallcase`` (``src/NavierStokes.jl:37-42``): DNS 90^3, LES 18^3 and 30^3."""
    return testcase(n_dns=90, viscosity=5e-4)


def mediumcase() -> dict:
    """``mediumcase`` (``src/NavierStokes.jl:44-49``): DNS 510^3, LES 102^3 and 170^3."""
    return testcase(n_dns=510, viscosity=5e-5)


def largecase() -> dict:
    """``largecase`` (``src/NavierStokes.jl:51-57``): DNS 810^3, LES 162^3 and 270^3."""
    return testcase(n_dns=810, viscosity=2.5e-5)


def case_for(tc: dict, cfl: float = 0.3, kind: str = "volume", precision: int = EXC_F64, stream=None) -> "Case":
    """A device case for a ``testcase``: the DNS with its LES grids (filter
    ``kind``) and the seeded peak-profile initial field."""
    cs = Case(tc["n_dns"], tc["l"], tc["viscosity"], cfl, precision=precision,
              les=[(c, kind) for c in tc["compression"]], stream=stream)
    cs.init_random(tc["kpeak"], tc["totalenergy"], tc["seed"])
    return cs


def _paper_driver(ustart: np.ndarray, n_les: int, viscosity: float, doproject: bool, tstop: float, cfl: float,
                  l: float, stream, filter: str):
    ustart = np.asarray(ustart)
    if ustart.ndim != 4 or ustart.shape[0] != 3 or not (ustart.shape[1] == ustart.shape[2] == ustart.shape[3]):
        raise ValueError("ustart must have shape (3, n, n, n)")
    n = ustart.shape[1]
    if n_les < 1 or n % n_les:
        raise ValueError(f"n_les = {n_les} must divide the DNS size n = {n}")
    d = DnsAid(n, l, viscosity, n // n_les, None, stream)
    d.set_velocity(ustart)
    d.set_paper(doproject, filter)
    d.start()
    names = PAPER_FIELDS[1:]
    relerr = {k: [] for k in ("time",) + names}
    t, i = 0.0, 0
    # the reference's loop: errors of the initial state in the first pass,
    # then one step per pass while t < tstop
    while t < tstop:
        if i > 0:
            d.step(tstop, cfl, max_steps=1)
            t = d.time()[0]
        e = d.relerr()
        relerr["time"].append(t)
        for k in names:
            relerr[k].append(e[k])
        i += 1
    u = {"dns_ref": d.velocity(), "dns_fil": d.get("fu")}
    for k in names:
        u[k] = d.get(k)
    d.close()
    return u, {k: np.asarray(v, dtype=np.float64) for k, v in relerr.items()}


def dns_aid_volavg(ustart: np.ndarray, n_les: int, viscosity: float, doproject: bool, tstop: float, cfl: float,
                   l: float = 1.0, stream=None):
    """``dns_aid_volavg`` (``src/NavierStokes.jl:141-304``) on the GPU: the
    DNS from ``ustart`` and the four LES (no model, classic, swap,
    swap-symmetric) in lockstep until ``tstop``.  Returns ``(u, relerr)`` like
    the reference: ``u`` with ``dns_ref``, ``dns_fil`` and the four LES fields,
    ``relerr`` with ``time`` and each LES's ``|v - fu| / |fu|`` recorded at
    t = 0 and after every step (empty when ``tstop <= 0``)."""
    return _paper_driver(ustart, n_les, viscosity, doproject, tstop, cfl, l, stream, "volume")


def dns_aid_surface(ustart: np.ndarray, n_les: int, viscosity: float, doproject: bool, tstop: float, cfl: float,
                    l: float = 1.0, stream=None):
    """``dns_aid_surface`` (``src/NavierStokes.jl:306-468``) on the GPU: the
    DNS and four LES on the face-averaged (surface-filtered) DNS ``fiu``;
    classic with the surface-filtered flux, swap with the line-filtered flux
    off the diagonal, its symmetric part.  Returns ``(u, relerr)`` like
    ``dns_aid_volavg``."""
    return _paper_driver(ustart, n_les, viscosity, doproject, tstop, cfl, l, stream, "surface")


def compute_errors(uaid: dict) -> dict:
    """``compute_errors`` (``src/N.jl:1334-1349``) of ``dnsaid_project``
    output (host arrays; the GPU values come from ``DnsAid.errors``)."""
    ref = uaid["u_les"]
    out = {}
    for k in DNSAID_FIELDS[1:]:
        a = uaid[k]
        out[k] = float(np.sqrt(sum(np.sum((a[i] - ref[i]) ** 2) / np.sum(ref[i] ** 2) for i in range(3)) / 3))
    return out
