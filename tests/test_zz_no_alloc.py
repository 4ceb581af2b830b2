"""exc_project_noalloc: the projection for callers that cannot call cudaMalloc
(their device memory belongs to their own pool, they run under a fixed memory
budget, or they cannot afford cudaFree's synchronisation).  Its work array is
a static 4 MiB device array, so it must give the same answer as exc_project
(1e-12 relative L2 in float64) on consecutive calls that reuse that array.

This file is collected last so that a run stopping at the first failure has
already run every other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL64 = 1e-12


def rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def test_noalloc_projection_matches_exc_project_on_consecutive_calls(built_lib):
    import torch

    from exactclosure_gb300._lib import call

    L = 1.0
    st = torch.cuda.Stream()
    # two calls in a row on different grids and inputs: the second call
    # overwrites the first call's tables and spectrum in the shared array;
    # 72 is the largest FP64 grid the 4 MiB array holds
    for n, seed in ((32, 1), (48, 2), (32, 3), (72, 4), (72, 5)):
        rng = np.random.default_rng(seed)
        u0 = torch.tensor(rng.standard_normal((3, n, n, n)), dtype=torch.float64, device="cuda")
        ua, ub = u0.clone(), u0.clone()
        pa = torch.empty((n, n, n), dtype=torch.float64, device="cuda")
        pb = torch.empty_like(pa)
        ps = C.c_void_p()
        call("exc_poisson_create", 0, n, L, C.byref(ps))
        torch.cuda.synchronize()
        try:
            with torch.cuda.stream(st):
                call("exc_project", ps, C.c_void_p(ua.data_ptr()), C.c_void_p(pa.data_ptr()),
                     C.c_void_p(st.cuda_stream))
                call("exc_project_noalloc", 0, n, L, C.c_void_p(ub.data_ptr()), C.c_void_p(pb.data_ptr()),
                     C.c_void_p(st.cuda_stream))
            st.synchronize()
        finally:
            built_lib.exc_poisson_destroy(ps)
        a, b = ua.cpu().numpy(), ub.cpu().numpy()
        assert rel(b, a) < TOL64, (n, rel(b, a))
        assert rel(pb.cpu().numpy(), pa.cpu().numpy()) < TOL64


def test_noalloc_float32_and_size_limit(built_lib):
    import torch

    from exactclosure_gb300._lib import ExcError, call

    # 96 is the largest FP32 grid the 4 MiB array holds
    for n in (24, 96):
        rng = np.random.default_rng(5)
        u0 = torch.tensor(rng.standard_normal((3, n, n, n)), dtype=torch.float32, device="cuda")
        ua, ub = u0.clone(), u0.clone()
        ps = C.c_void_p()
        call("exc_poisson_create", 1, n, 1.0, C.byref(ps))
        try:
            call("exc_project", ps, C.c_void_p(ua.data_ptr()), None, None)
            call("exc_project_noalloc", 1, n, 1.0, C.c_void_p(ub.data_ptr()), None, None)
            torch.cuda.synchronize()
        finally:
            built_lib.exc_poisson_destroy(ps)
        assert rel(ub.cpu().double().numpy(), ua.cpu().double().numpy()) < 2e-5, n
    # beyond the static scratch (the next FFT sizes above the limits: 80 in
    # FP64, 100 in FP32): rejected on the host with a clear error
    for prec, n in ((0, 80), (0, 96), (1, 100)):
        with pytest.raises(ExcError) as ei:
            call("exc_project_noalloc", prec, n, 1.0, C.c_void_p(ub.data_ptr()), None, None)
        assert ei.value.code == 2 and "4 MiB" in str(ei.value), (prec, n)
