"""CPU checks of the C ABI: the library builds for sm_103a, loads, and exports
every symbol include/exc.h declares (no compute calls: there is no GPU)."""
import re
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def header_symbols():
    text = (ROOT / "include" / "exc.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(exc_\w+)\s*\(", text)))


def test_header_matches_binding_table():
    from exactclosure_gb300 import _lib

    assert sorted(_lib.declared_symbols()) == header_symbols()


def test_library_exports_every_declared_symbol(built_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", str(Path(built_lib._name))],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\b(exc_\w+)\b", out))
    missing = [s for s in header_symbols() if s not in exported]
    assert not missing, missing
    for s in header_symbols():
        assert hasattr(built_lib, s)


def test_version_and_error_string(built_lib):
    assert built_lib.exc_version() == 100
    assert isinstance(built_lib.exc_last_error(), bytes)


def test_argument_validation_without_gpu(built_lib):
    """Shape and ratio checks happen on the host before any device call."""
    import ctypes as C

    from exactclosure_gb300 import _lib

    d = _lib.CaseDesc()
    d.n, d.l, d.visc, d.cfl, d.precision, d.nles = 38, 1.0, 1e-3, 0.3, 0, 0  # 38 = 2 19
    h = C.c_void_p()
    assert built_lib.exc_case_create(C.byref(d), None, C.byref(h)) == 2  # EXC_ERR_SHAPE
    d.n, d.nles = 64, 1
    d.les[0].ratio, d.les[0].kind = 5, 0
    assert built_lib.exc_case_create(C.byref(d), None, C.byref(h)) == 3  # EXC_ERR_RATIO
    d.les[0].ratio = 4
    d.visc = -1
    assert built_lib.exc_case_create(C.byref(d), None, C.byref(h)) == 1  # EXC_ERR_ARG
    assert built_lib.exc_case_create(None, None, C.byref(h)) == 1



def test_reference_test_cases():
    """``smallcase`` / ``mediumcase`` / ``largecase`` (src/NavierStokes.jl:37-57):
    DNS 90, 510, 810 with compression 5 and 3; every grid is an FFT size of
    the library (radix 2, 3, 5 and 17 among them)."""
    from exactclosure_gb300 import navierstokes as NS

    cases = {"small": NS.smallcase(), "medium": NS.mediumcase(), "large": NS.largecase()}
    assert [c["n_dns"] for c in cases.values()] == [90, 510, 810]
    assert cases["medium"]["n_les"] == [102, 170] and cases["medium"]["viscosity"] == 5e-5
    assert cases["large"]["n_les"] == [162, 270] and cases["small"]["n_les"] == [18, 30]

    def fft_ok(n):
        m = n
        for f in (2, 3, 5, 7, 11, 13, 17):
            while m % f == 0:
                m //= f
        return m == 1 and n % 2 == 0 and 4 <= n <= 1024

    for c in cases.values():
        assert all(fft_ok(n) for n in [c["n_dns"]] + c["n_les"])
    import pytest

    with pytest.raises(ValueError):
        NS.testcase(n_dns=100, viscosity=1e-3, compression=(3,))
