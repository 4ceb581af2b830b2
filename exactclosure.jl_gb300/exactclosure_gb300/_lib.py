"""ctypes binding of libexc.so (the C ABI declared in include/exc.h).

The library must exist (built by ``exactclosure.jl_gb300/build.py``); a missing
library raises immediately — there is no CPU fallback."""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

LIB_PATH = Path(os.environ.get("EXC_LIB", Path(__file__).resolve().parent.parent / "libexc.so"))

EXC_OK = 0
EXC_F64, EXC_F32 = 0, 1
EXC_FILTER_VOLUME, EXC_FILTER_FACE = 0, 1
EXC_MAX_LES = 4
STATUS = {0: "EXC_OK", 1: "EXC_ERR_ARG", 2: "EXC_ERR_SHAPE", 3: "EXC_ERR_RATIO", 4: "EXC_ERR_OOM",
          5: "EXC_ERR_CUDA", 6: "EXC_ERR_NONFINITE", 7: "EXC_ERR_TIMEOUT", 8: "EXC_ERR_STATE"}


class ExcError(RuntimeError):
    """A non-zero status returned across the C ABI."""

    def __init__(self, code: int, func: str, msg: str):
        super().__init__(f"{func}: {STATUS.get(code, code)}: {msg}")
        self.code = code


class LesDesc(C.Structure):
    _fields_ = [("ratio", C.c_int), ("kind", C.c_int)]


class CaseDesc(C.Structure):
    _fields_ = [("n", C.c_int), ("l", C.c_double), ("visc", C.c_double), ("cfl", C.c_double),
                ("precision", C.c_int), ("nles", C.c_int), ("les", LesDesc * EXC_MAX_LES)]


class BurgersDesc(C.Structure):
    _fields_ = [("nh", C.c_int), ("nsample", C.c_int), ("l", C.c_double), ("visc", C.c_double)]


class DnsAidDesc(C.Structure):
    _fields_ = [("n", C.c_int), ("l", C.c_double), ("visc", C.c_double), ("ratio", C.c_int),
                ("fdelta", C.POINTER(C.c_double)), ("nfdelta", C.c_int)]


class ServerDesc(C.Structure):
    _fields_ = [("precision", C.c_int), ("mem_fraction", C.c_double), ("max_bytes", C.c_double),
                ("slots_per_chunk", C.c_int), ("autotune", C.c_int)]


class SolveReq(C.Structure):
    _fields_ = [("n", C.c_int), ("l", C.c_double), ("visc", C.c_double), ("cfl", C.c_double),
                ("kpeak", C.c_double), ("energy", C.c_double), ("seed", C.c_uint64), ("nsteps", C.c_int),
                ("result_host", C.POINTER(C.c_double))]


class SolveResult(C.Structure):
    _fields_ = [("id", C.c_int64), ("n", C.c_int), ("nsteps", C.c_int), ("t_submit", C.c_double),
                ("t_admit", C.c_double), ("t_finish", C.c_double), ("energy", C.c_double),
                ("sim_time", C.c_double)]


class ServerInfo(C.Structure):
    _fields_ = [("chunks", C.c_int), ("slots", C.c_int), ("active", C.c_int), ("queued", C.c_int),
                ("kernels_per_tick", C.c_int), ("bytes_used", C.c_double), ("bytes_budget", C.c_double),
                ("ticks", C.c_double), ("clock", C.c_double)]


vp = C.c_void_p
dp = C.POINTER(C.c_double)
i32, f64, u64, szt = C.c_int, C.c_double, C.c_uint64, C.c_size_t

# name -> argtypes (every function returns int status unless listed in _RESTYPE)
SIGNATURES = {
    "exc_last_error": [],
    "exc_version": [],
    "exc_tensordivergence": [i32, i32, f64, f64, vp, vp, i32, vp],
    "exc_tensordivergence_tensor": [i32, i32, f64, i32, vp, vp, i32, vp],
    "exc_stresstensor": [i32, i32, f64, f64, vp, vp, vp],
    "exc_divergence": [i32, i32, f64, vp, vp, vp],
    "exc_pressuregradient": [i32, i32, f64, vp, vp, vp],
    "exc_poisson_create": [i32, i32, f64, C.POINTER(vp)],
    "exc_poisson_destroy": [vp],
    "exc_poisson_set_engine": [vp, i32],
    "exc_device_faults": [C.POINTER(i32)],
    "exc_device_sync": [vp, C.POINTER(i32)],
    "exc_debug_wait_drill": [i32],
    "exc_poisson_solve": [vp, vp, vp, vp],
    "exc_project": [vp, vp, vp, vp],
    "exc_project_noalloc": [i32, i32, f64, vp, vp, vp],
    "exc_max_abs": [i32, szt, vp, vp, vp],
    "exc_propose_timestep": [i32, i32, f64, f64, f64, vp, dp, vp],
    "exc_filter": [i32, i32, i32, i32, dp, i32, vp, vp, vp],
    "exc_closure_flux": [i32, i32, i32, f64, f64, dp, i32, vp, vp, vp, vp],
    "exc_filtered_stress": [i32, i32, i32, f64, f64, dp, i32, vp, vp, vp],
    "exc_case_create": [C.POINTER(CaseDesc), vp, C.POINTER(vp)],
    "exc_case_destroy": [vp],
    "exc_case_init_random": [vp, f64, f64, u64],
    "exc_case_set_velocity": [vp, dp],
    "exc_case_get_velocity": [vp, dp],
    "exc_case_get_les": [vp, i32, i32, dp],
    "exc_case_step": [vp, i32, f64],
    "exc_case_errors": [vp, i32, dp],
    "exc_case_time": [vp, dp, dp],
    "exc_case_energy": [vp, dp],
    "exc_case_dissipation": [vp, dp],
    "exc_case_spectrum": [vp, dp, i32],
    "exc_case_device_ptr": [vp, i32, C.POINTER(vp)],
    "exc_case_launches_per_step": [vp, C.POINTER(i32)],
    "exc_case_reset_les": [vp],
    "exc_case_les_error": [vp, i32, i32, dp],
    "exc_case_snapshot": [vp, i32, vp, vp],
    "exc_case_attach_net": [vp, i32, vp],
    "exc_case_set_fallback": [vp, i32, f64, f64],
    "exc_case_fallback": [vp, i32, C.POINTER(i32)],
    "exc_case_sync": [vp],
    "exc_net_create": [u64, C.POINTER(vp)],
    "exc_net_destroy": [vp],
    "exc_net_param_count": [],
    "exc_net_set_scales": [vp, f64, f64],
    "exc_net_set_conv_engine": [vp, i32],
    "exc_net_get_params": [vp, C.POINTER(C.c_float), i32],
    "exc_net_set_params": [vp, C.POINTER(C.c_float), i32],
    "exc_net_forward": [vp, i32, i32, i32, vp, vp, vp],
    "exc_net_gradients": [vp, i32, i32, i32, vp, vp, C.POINTER(C.c_float), dp, vp],
    "exc_net_train_step": [vp, i32, i32, i32, vp, vp, f64, dp, vp],
    "exc_server_create": [C.POINTER(ServerDesc), C.POINTER(vp)],
    "exc_server_destroy": [vp],
    "exc_server_set_admission": [vp, i32],
    "exc_server_submit": [vp, C.POINTER(SolveReq), C.POINTER(C.c_int64)],
    "exc_server_tick": [vp, C.POINTER(i32), C.POINTER(i32)],
    "exc_server_poll": [vp, C.POINTER(SolveResult), i32, C.POINTER(i32)],
    "exc_server_drain": [vp],
    "exc_server_stats": [vp, C.POINTER(ServerInfo)],
    "exc_server_tuning": [i32, i32, i32, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)],
    "exc_dnsaid_create": [C.POINTER(DnsAidDesc), vp, C.POINTER(vp)],
    "exc_dnsaid_destroy": [vp],
    "exc_dnsaid_init_random": [vp, i32, f64, f64, u64],
    "exc_dnsaid_set_velocity": [vp, dp],
    "exc_dnsaid_get_velocity": [vp, dp],
    "exc_dnsaid_warmup": [vp, f64, f64, i32, C.POINTER(i32)],
    "exc_dnsaid_start": [vp],
    "exc_dnsaid_set_paper": [vp, i32],
    "exc_dnsaid_set_surface": [vp, i32],
    "exc_dnsaid_relerr": [vp, dp],
    "exc_dnsaid_step": [vp, f64, f64, i32, C.POINTER(i32)],
    "exc_dnsaid_time": [vp, dp, C.POINTER(i32)],
    "exc_dnsaid_get": [vp, i32, dp],
    "exc_dnsaid_errors": [vp, dp],
    "exc_burgers_kernels": [i32, i32, f64, f64, i32, C.POINTER(i32), dp, C.POINTER(i32), dp],
    "exc_burgers_create": [C.POINTER(BurgersDesc), vp, C.POINTER(vp)],
    "exc_burgers_destroy": [vp],
    "exc_burgers_init_random": [vp, f64, f64, u64],
    "exc_burgers_set_velocity": [vp, dp],
    "exc_burgers_get_velocity": [vp, i32, dp],
    "exc_burgers_time": [vp, dp, C.POINTER(i32)],
    "exc_burgers_restart": [vp],
    "exc_burgers_les_setup": [vp, i32, f64, i32],
    "exc_burgers_advance": [vp, f64, f64, i32, i32, C.POINTER(i32)],
    "exc_burgers_get_les": [vp, i32, dp],
    "exc_burgers_filtered": [vp, dp],
    "exc_burgers_errors": [vp, dp],
    "exc_burgers_closure_terms": [vp, dp, dp, dp],
    "exc_burgers_smagorinsky_fit": [vp, dp, dp],
    "exc_burgers_smagorinsky_solve": [vp, f64, f64, f64, i32, i32, C.POINTER(i32)],
    "exc_burgers_device_ptr": [vp, i32, C.POINTER(vp)],
}
_RESTYPE = {"exc_last_error": C.c_char_p}

_lib = None


def lib() -> C.CDLL:
    """Load libexc.so once; raise if it is missing."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"libexc.so not built at {LIB_PATH}; run exactclosure.jl_gb300/build.py")
        L = C.CDLL(str(LIB_PATH))
        for name, args in SIGNATURES.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = _RESTYPE.get(name, C.c_int)
        _lib = L
    return _lib


def call(name: str, *args) -> None:
    """Call an entry point and raise ExcError on a non-zero status."""
    rc = getattr(lib(), name)(*args)
    if rc != EXC_OK:
        msg = lib().exc_last_error().decode()
        raise ExcError(rc, name, msg)


def declared_symbols() -> list[str]:
    return list(SIGNATURES)
