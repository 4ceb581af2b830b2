"""Host-side mirror of the reference's 1-D ``Burgers`` module
(``src/Burgers.jl``) over the libexc C ABI.

The reference runs its samples one after another (``src/Burgers.jl:307``,
``:530``, ``:605``); here a ``Batch`` holds every sample on the GPU and one
CUDA kernel advances all of them, each with its own time step.  Arrays cross
the boundary as ``(nsample, n)`` float64 NumPy arrays -- the transpose of the
reference's ``(n, nsample)`` column-major matrices, byte for byte the same.
Every computation goes through ``libexc.so``; nothing here computes on the
CPU except bookkeeping.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from ._lib import BurgersDesc, call

GAUSSIAN, TOPHAT = 0, 1
FILTERS = {"gaussian": GAUSSIAN, "tophat": TOPHAT}
EULER, RK4 = 0, 1
FIELDS = {"dns_fil": 0, "nomodel": 1, "class_m": 2, "class_p": 3, "swapfil": 4, "smag": 5}
LABELS = {"dns_ref": "DNS", "dns_ref_fil": "Filtered DNS", "dns_fil": "Filtered DNS",
          "nomodel": "No model", "class_m": "Classic", "class_p": "Classic+Flux",
          "swapfil": "Classic+Flux+Div (ours)"}


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


@dataclass(frozen=True)
class Grid:
    """``Grid(L, n)`` (``src/Burgers.jl:25-31``)."""

    L: float
    n: int

    @property
    def spacing(self) -> float:
        return self.L / self.n


def spacing(g: Grid) -> float:
    return g.L / g.n


def points_stag(g: Grid) -> np.ndarray:
    """``points_stag`` (``src/Burgers.jl:82``)."""
    return np.linspace(0, g.L, g.n + 1)[1:]


def points_coll(g: Grid) -> np.ndarray:
    """``points_coll`` (``src/Burgers.jl:83``)."""
    return points_stag(g) - spacing(g) / 2


def filter_kernels(gh: Grid, gH: Grid, delta_ratio: float, lesfiltertype: str = "gaussian"):
    """((Rl, wl), (Rd, wd)): the LES kernel and the double kernel of
    ``dns_aided_les`` (``src/Burgers.jl:355-364``), built by the library."""
    rl, rd = C.c_int(), C.c_int()
    call("exc_burgers_kernels", gh.n, gH.n, gh.L, delta_ratio, FILTERS[lesfiltertype], C.byref(rl), None,
         C.byref(rd), None)
    wl, wd = np.zeros(2 * rl.value + 1), np.zeros(2 * rd.value + 1)
    call("exc_burgers_kernels", gh.n, gH.n, gh.L, delta_ratio, FILTERS[lesfiltertype], C.byref(rl), _dp(wl),
         C.byref(rd), _dp(wd))
    return (rl.value, wl), (rd.value, wd)


class Batch:
    """``nsample`` periodic Burgers samples resident on the GPU (handle of
    ``exc_burgers_*``)."""

    def __init__(self, g: Grid, nsample: int, visc: float, stream=None):
        self.g, self.ns, self.visc = g, nsample, visc
        h = C.c_void_p()
        desc = BurgersDesc(g.n, nsample, g.L, visc)
        call("exc_burgers_create", C.byref(desc), stream, C.byref(h))
        self._h = h
        self.gH: Grid | None = None

    def close(self):
        if getattr(self, "_h", None):
            call("exc_burgers_destroy", self._h)
            self._h = None

    __del__ = close

    # ---- state
    def randomfield(self, kpeak: float, totalenergy: float, seed: int = 1):
        """``randomfield`` (``src/Burgers.jl:195-202``), sample s seeded
        ``seed + s``."""
        call("exc_burgers_init_random", self._h, kpeak, totalenergy, seed)

    def set_velocity(self, u: np.ndarray):
        a = np.ascontiguousarray(u, dtype=np.float64)
        assert a.shape == (self.ns, self.g.n)
        call("exc_burgers_set_velocity", self._h, _dp(a))

    def velocity(self, initial: bool = False) -> np.ndarray:
        out = np.empty((self.ns, self.g.n))
        call("exc_burgers_get_velocity", self._h, int(initial), _dp(out))
        return out

    def restart(self):
        """Back to the recorded initial field, clocks at zero."""
        call("exc_burgers_restart", self._h)

    def time(self):
        t = np.empty(self.ns)
        s = np.empty(self.ns, dtype=np.int32)
        call("exc_burgers_time", self._h, _dp(t), s.ctypes.data_as(C.POINTER(C.c_int)))
        return t, s

    # ---- stepping
    def les_setup(self, gH: Grid | None, delta_ratio: float = 0.0, lesfiltertype: str = "gaussian"):
        call("exc_burgers_les_setup", self._h, 0 if gH is None else gH.n, delta_ratio, FILTERS[lesfiltertype])
        self.gH = gH

    def advance(self, tstop: float, cfl_factor: float, scheme: str = "euler", max_steps: int = 0) -> int:
        m = C.c_int()
        call("exc_burgers_advance", self._h, tstop, cfl_factor, {"euler": EULER, "rk4": RK4}[scheme], max_steps,
             C.byref(m))
        return m.value

    # ---- outputs
    def les(self, which: str) -> np.ndarray:
        out = np.empty((self.ns, self.gH.n))
        call("exc_burgers_get_les", self._h, FIELDS[which], _dp(out))
        return out

    def filtered(self) -> np.ndarray:
        out = np.empty((self.ns, self.g.n))
        call("exc_burgers_filtered", self._h, _dp(out))
        return out

    def errors(self) -> dict:
        e = np.empty(5)
        call("exc_burgers_errors", self._h, _dp(e))
        return dict(zip(("nomodel", "class_m", "class_p", "swapfil", "smag"), e.tolist()))

    def closure_terms(self, want_terms: bool = True, want_diss: bool = True):
        terms = np.empty((self.ns, 5, self.gH.n)) if want_terms else None
        diss = np.empty((self.ns, 3, self.gH.n)) if want_diss else None
        fr = np.empty(3)
        call("exc_burgers_closure_terms", self._h, None if terms is None else _dp(terms),
             None if diss is None else _dp(diss), _dp(fr))
        return terms, diss, fr

    def smagorinsky_fit(self, want_fields: bool = False):
        th = np.empty(2)
        f = np.empty((self.ns, 4, self.g.n)) if want_fields else None
        call("exc_burgers_smagorinsky_fit", self._h, _dp(th), None if f is None else _dp(f))
        return th, f

    def smagorinsky_solve(self, theta: float, tstop: float, cfl_factor: float = 0.3, max_steps: int = 0,
                          restart: bool = True) -> int:
        m = C.c_int()
        call("exc_burgers_smagorinsky_solve", self._h, theta, tstop, cfl_factor, max_steps, int(restart),
             C.byref(m))
        return m.value


# ---------------------------------------------------------------- drivers

def getsetup(**kw) -> dict:
    """``getsetup`` (``src/Burgers.jl:235-265``); keywords override."""
    s = dict(L=2 * math.pi, nh=100 * 3**3 * 5, nH=tuple(100 * 3**k for k in (1, 2, 3)), Δ_ratios=(2,),
             visc=5.0e-4, kpeak=10, initialenergy=2.0, tstop=0.1, nsample=1000, lesfiltertype="gaussian",
             seed=1)
    s.update(kw)
    return s


def dns_aided_les(batch: Batch, gH: Grid, Δ: float, tstop: float, cfl_factor: float,
                  lesfiltertype: str = "gaussian") -> dict:
    """``dns_aided_les`` (``src/Burgers.jl:350-445``) for every sample of
    ``batch`` from its recorded initial field: the seven fields
    ``dns_ref, dns_ref_fil, dns_fil, nomodel, class_m, class_p, swapfil``."""
    batch.restart()
    batch.les_setup(gH, Δ / gH.spacing, lesfiltertype)
    batch.advance(tstop, cfl_factor, "euler")
    out = {"dns_ref": batch.velocity(), "dns_ref_fil": batch.filtered()}
    for k in ("dns_fil", "nomodel", "class_m", "class_p", "swapfil"):
        out[k] = batch.les(k)
    return out


def run_dns_aided_les(setup: dict, stream=None):
    """``run_dns_aided_les`` (``src/Burgers.jl:267-328``): one result per
    (nH, Δ_ratio) with the fields of every sample."""
    gh = Grid(setup["L"], setup["nh"])
    batch = Batch(gh, setup["nsample"], setup["visc"], stream)
    batch.randomfield(setup["kpeak"], setup["initialenergy"], setup["seed"])
    res = []
    for nH in setup["nH"]:
        for r in setup["Δ_ratios"]:
            gH = Grid(setup["L"], nH)
            fields = dns_aided_les(batch, gH, gH.spacing * r, setup["tstop"], 0.3, setup["lesfiltertype"])
            res.append({"Δ_ratio": r, "nH": nH, "fields": fields, "errors": batch.errors()})
    batch.close()
    return res


def create_dns(setup: dict, cfl_factor: float, scheme: str = "euler", stream=None):
    """``create_dns`` (``src/Burgers.jl:522-545``): (Ustart, U), each
    ``(nsample, nh)``, and the batch holding U."""
    gh = Grid(setup["L"], setup["nh"])
    batch = Batch(gh, setup["nsample"], setup["visc"], stream)
    batch.randomfield(setup["kpeak"], setup["initialenergy"], setup["seed"])
    batch.advance(setup["tstop"], cfl_factor, scheme)
    return batch


def compute_errors(series) -> dict:
    """``compute_errors`` (``src/Burgers.jl:909-916``) of ``run_dns_aided_les``
    results: label and relative error per LES and per (nH, Δ_ratio)."""
    keys = ("nomodel", "class_m", "class_p", "swapfil")
    return {k: {"label": LABELS[k], "e": [s["errors"][k] for s in series]} for k in keys}


def smagorinsky_fields(batch: Batch, setup: dict):
    """``smagorinsky_fields`` + the coefficient fits of ``smagorinsky.jl``
    for every (Δ_ratio, nH): {(Δ_ratio, nH): (θ²_classic, θ²_discrete)}."""
    out = {}
    for r in setup["Δ_ratios"]:
        for nH in setup["nH"]:
            batch.les_setup(Grid(setup["L"], nH), r, setup["lesfiltertype"])
            th, _ = batch.smagorinsky_fit()
            out[(r, nH)] = tuple(th.tolist())
    return out


def solve_smagorinsky(batch: Batch, setup: dict, smagcoeffs: dict, which: int = 1):
    """``solve_smagorinsky`` (``src/Burgers.jl:690-771``) from the batch's
    initial fields with θ = sqrt(θ²[which]); returns {(Δ_ratio, nH): (Ubar,
    relative error against the filtered final DNS)}."""
    out = {}
    for (r, nH), th2 in smagcoeffs.items():
        batch.les_setup(Grid(setup["L"], nH), r, setup["lesfiltertype"])
        batch.smagorinsky_solve(math.sqrt(th2[which]), setup["tstop"], 0.3)
        out[(r, nH)] = (batch.les("smag"), batch.errors()["smag"])
    return out


def compute_fractions(batch: Batch, setup: dict) -> dict:
    """``compute_fractions`` (``src/Burgers.jl:1022-1116``) on the batch's
    current DNS: {(nH, Δ_ratio): (classic, flux, div)}."""
    out = {}
    for nH in setup["nH"]:
        for r in setup["Δ_ratios"]:
            batch.les_setup(Grid(setup["L"], nH), r, setup["lesfiltertype"])
            _, _, fr = batch.closure_terms(False, False)
            out[(nH, r)] = tuple(fr.tolist())
    return out


def compute_dissipation(batch: Batch, setup: dict) -> dict:
    """``compute_dissipation`` (``src/Burgers.jl:447-520``): per (nH,
    Δ_ratio) the dissipation coefficients of the classic, classic+flux and
    exact closures, shape (3, nsample, nH)."""
    out = {}
    for nH in setup["nH"]:
        for r in setup["Δ_ratios"]:
            batch.les_setup(Grid(setup["L"], nH), r, setup["lesfiltertype"])
            _, d, _ = batch.closure_terms(False, True)
            out[(nH, r)] = np.ascontiguousarray(d.transpose(1, 0, 2))
    return out
