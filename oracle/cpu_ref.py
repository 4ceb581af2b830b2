"""ctypes driver of the oracle's C/OpenMP restatement (``oracle/cpu_ref.c``).

TEST INFRASTRUCTURE ONLY: used by the tests as a second oracle and by
``bench.py`` as the timed CPU baseline; never by the product path."""
from __future__ import annotations

import ctypes as C
import os
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libexc_cpu_ref.so"
_lib = None


def available() -> bool:
    return LIB.exists()


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(str(LIB))
        L.cref_threads.restype = C.c_int
        L.cref_create.restype = C.c_void_p
        L.cref_create.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_int,
                                  C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.cref_destroy.argtypes = [C.c_void_p]
        L.cref_init_random.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_uint64]
        L.cref_set_velocity.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.cref_get_velocity.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.cref_get_les.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_double)]
        L.cref_step.argtypes = [C.c_void_p, C.c_int, C.c_double]
        L.cref_stage.argtypes = [C.c_void_p, C.c_int]
        L.cref_init_analytic.argtypes = [C.c_void_p]
        L.cref_init_analytic.restype = C.c_int
        L.cref_time.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.cref_project.argtypes = [C.c_int, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.cref_rhs.argtypes = [C.c_int, C.c_double, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        for f in ("cref_init_random", "cref_set_velocity", "cref_get_velocity", "cref_get_les", "cref_step",
                  "cref_stage", "cref_time", "cref_project", "cref_rhs"):
            getattr(L, f).restype = C.c_int
        _lib = L
    return _lib


class CpuCase:
    """The C restatement of the RK4 DNS-aided LES step (same layout as libexc)."""

    def __init__(self, n, l, visc, cfl, les):
        r = (C.c_int * 4)(*[c for c, _ in les] + [0] * (4 - len(les)))
        k = (C.c_int * 4)(*[0 if kd == "volume" else 1 for _, kd in les] + [0] * (4 - len(les)))
        self.n = n
        self.les = list(les)
        self._h = lib().cref_create(n, l, visc, cfl, len(les), r, k)
        if not self._h:
            raise MemoryError("cref_create failed")

    def init_random(self, kpeak, energy, seed):
        assert lib().cref_init_random(self._h, kpeak, energy, seed) == 0

    def set_velocity(self, u):
        import numpy as np

        a = np.ascontiguousarray(u, dtype=np.float64)
        assert lib().cref_set_velocity(self._h, a.ctypes.data_as(C.POINTER(C.c_double))) == 0

    def velocity(self):
        import numpy as np

        a = np.empty((3, self.n, self.n, self.n))
        assert lib().cref_get_velocity(self._h, a.ctypes.data_as(C.POINTER(C.c_double))) == 0
        return a

    def les_field(self, i, which):
        import numpy as np

        m = self.n // self.les[i][0]
        a = np.empty((3, m, m, m))
        w = {"target": 0, "exact": 1, "nomodel": 2}[which]
        assert lib().cref_get_les(self._h, i, w, a.ctypes.data_as(C.POINTER(C.c_double))) == 0
        return a

    def step(self, nsteps=1, dt=0.0):
        assert lib().cref_step(self._h, nsteps, dt) == 0

    def stage(self, s):
        assert lib().cref_stage(self._h, s) == 0

    def close(self):
        if self._h:
            lib().cref_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def project(u, l=1.0):
    """``project!`` of a float64 ``(3, n, n, n)`` field (a new array) and its
    pressure, by the C restatement on all host threads."""
    import numpy as np

    a = np.array(u, dtype=np.float64, order="C", copy=True)
    n = a.shape[1]
    p = np.empty((n, n, n))
    dp = C.POINTER(C.c_double)
    assert lib().cref_project(n, l, a.ctypes.data_as(dp), p.ctypes.data_as(dp)) == 0
    return a, p


def rhs(u, visc, l=1.0):
    """``tensordivergence(stresstensor(u, visc))`` by the C restatement."""
    import numpy as np

    a = np.ascontiguousarray(u, dtype=np.float64)
    du = np.empty_like(a)
    dp = C.POINTER(C.c_double)
    assert lib().cref_rhs(a.shape[1], l, visc, a.ctypes.data_as(dp), du.ctypes.data_as(dp)) == 0
    return du


def timing_case(n, les, visc, kpeak=None):
    """A full-size CPU case for timing samples: the seeded peak-spectrum
    field of the workload (``kpeak``), or a smooth analytic field when
    ``kpeak`` is None (values do not change the work of a stage)."""
    cs = CpuCase(n, 1.0, visc, 0.3, les)
    if kpeak is None:
        assert lib().cref_init_analytic(cs._h) == 0
    else:
        cs.init_random(kpeak, 1.0, 0)
    cs.stage(0)  # warm-up (page faults, dt)
    return cs


def time_stages(n, les, kpeak, visc, budget_s=20.0, cs=None, max_stages=8):
    """Time whole RK4 stages of the full-size workload on all host threads."""
    own = cs is None
    if own:
        cs = timing_case(n, les, visc, kpeak)
    t0 = time.perf_counter()
    k = 0
    while True:
        cs.stage(1 + (k % 3))
        k += 1
        if time.perf_counter() - t0 > budget_s * 0.5 or k >= max_stages:
            break
    el = time.perf_counter() - t0
    if own:
        cs.close()
    steps = k / 4.0
    threads = lib().cref_threads()
    return {"cell_updates_per_s": n ** 3 * steps / el, "threads": threads,
            "sample": f"C/OpenMP restatement, {k} RK4 stage(s) of the {n}^3 DNS with LES ratios "
                      f"{[c for c, _ in les]} at full size ({k}/4 RK4 steps), {threads} threads"}


def burgers_dnsaid(u0, nH, visc, l, wl, wd, tstop, cfl, max_steps=0, state=None):
    """``dns_aided_les`` in the C restatement (``oracle/cpu_burgers.c``),
    samples in parallel over the host cores.  ``wl``/``wd`` are the LES and
    double kernels (``oracle.burgers.kernels``); ``nH = 0`` runs the DNS
    alone.  Returns (u, v[ns][4][nH], t, steps)."""
    L = lib()
    f = L.cref_burgers_dnsaid
    dp = C.POINTER(C.c_double)
    f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, dp, C.c_int, dp, C.c_int, C.c_double,
                  C.c_double, C.c_int, dp, dp, dp, C.POINTER(C.c_int)]
    f.restype = C.c_int
    import numpy as np

    ns, nh = u0.shape
    if state is None:
        u = np.ascontiguousarray(u0, dtype=np.float64).copy()
        from .burgers import coarse_filter

        v0 = coarse_filter(u, (len(wd) // 2, wd), nH, True) if nH else np.zeros((ns, 1))
        v = np.ascontiguousarray(np.repeat(v0[:, None, :], 4, axis=1)) if nH else np.zeros((ns, 4, 1))
        t = np.zeros(ns)
        steps = np.zeros(ns, dtype=np.int32)
    else:
        u, v, t, steps = (x.copy() for x in state)
    wl = np.ascontiguousarray(wl, dtype=np.float64)
    wd = np.ascontiguousarray(wd, dtype=np.float64)
    f(nh, ns, nH, l, visc, wl.ctypes.data_as(dp), len(wl) // 2, wd.ctypes.data_as(dp), len(wd) // 2, tstop, cfl,
      max_steps if max_steps > 0 else 2**31 - 1, u.ctypes.data_as(dp), v.ctypes.data_as(dp), t.ctypes.data_as(dp),
      steps.ctypes.data_as(C.POINTER(C.c_int)))
    return u, v, t, steps
