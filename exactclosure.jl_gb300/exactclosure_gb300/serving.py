"""Serving form over the libexc C ABI: continuous batching of independent
periodic NS solves of mixed grid sizes (``exc_server_*`` in include/exc.h).

No counterpart in the reference (its driver, ``dnsaid_project`` in
``src/N.jl:1239-1332``, runs one solve at a time); every solve is the same
RK4 step with FFT projection as the plain path, in FP32 (FP64 spectral divide
and diagnostics) or FP64.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import EXC_F32, ServerDesc, ServerInfo, SolveReq, SolveResult, call, lib


class Server:
    def __init__(self, precision: int = EXC_F32, mem_fraction: float = 0.5, slots_per_chunk: int = 0,
                 autotune: bool = True, max_bytes: float = 0.0, max_active_per_size: int = 0):
        d = ServerDesc()
        d.precision, d.mem_fraction, d.slots_per_chunk, d.autotune = precision, mem_fraction, slots_per_chunk, \
            int(autotune)
        d.max_bytes = max_bytes
        h = C.c_void_p()
        call("exc_server_create", C.byref(d), C.byref(h))
        self._h = h
        self.precision = precision
        self._keep = {}
        if max_active_per_size:
            self.set_admission(max_active_per_size)

    def set_admission(self, max_active_per_size: int):
        """Admit a request only while fewer than ``max_active_per_size`` solves
        of its grid size run (0: no bound)."""
        call("exc_server_set_admission", self._h, max_active_per_size)

    def submit(self, n: int, visc: float, nsteps: int, seed: int = 0, kpeak: float = 4.0, energy: float = 1.0,
               l: float = 1.0, cfl: float = 0.3, keep_field: bool = False) -> int:
        q = SolveReq()
        q.n, q.l, q.visc, q.cfl, q.kpeak, q.energy, q.seed, q.nsteps = n, l, visc, cfl, kpeak, energy, seed, nsteps
        buf = None
        if keep_field:
            buf = np.empty((3, n, n, n), dtype=np.float64)
            q.result_host = buf.ctypes.data_as(C.POINTER(C.c_double))
        rid = C.c_int64()
        call("exc_server_submit", self._h, C.byref(q), C.byref(rid))
        if buf is not None:
            self._keep[rid.value] = buf
        return rid.value

    def tick(self) -> tuple[int, int]:
        a, q = C.c_int(), C.c_int()
        call("exc_server_tick", self._h, C.byref(a), C.byref(q))
        return a.value, q.value

    def poll(self, max_results: int = 256) -> list[dict]:
        arr = (SolveResult * max_results)()
        cnt = C.c_int()
        call("exc_server_poll", self._h, arr, max_results, C.byref(cnt))
        out = []
        for i in range(cnt.value):
            r = arr[i]
            out.append(dict(id=r.id, n=r.n, nsteps=r.nsteps, t_submit=r.t_submit, t_admit=r.t_admit,
                            t_finish=r.t_finish, energy=r.energy, sim_time=r.sim_time,
                            field=self._keep.pop(r.id, None)))
        return out

    def drain(self):
        call("exc_server_drain", self._h)

    def stats(self) -> dict:
        s = ServerInfo()
        call("exc_server_stats", self._h, C.byref(s))
        return {f: getattr(s, f) for f, _ in ServerInfo._fields_}

    @staticmethod
    def tuning(precision: int, n: int, slots: int):
        """(engine, col_w, x_rows) the autotuner chose: engine 0 = register-
        resident FFT passes, 1 = Stockham passes."""
        e, w, r = C.c_int(), C.c_int(), C.c_int()
        call("exc_server_tuning", precision, n, slots, C.byref(e), C.byref(w), C.byref(r))
        return e.value, w.value, r.value

    def close(self):
        if getattr(self, "_h", None):
            lib().exc_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
