"""The C-ABI library loads without a GPU and exports every declared entry point."""
import ctypes
import os
import re

from conftest import ROOT


def declared(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\([^;{]*\)\s*;", src)
    return sorted(set(n for n in names if n not in ("if", "return", "sizeof")))


def test_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(os.path.join(ROOT, "upside2-md_gb300", "libupside.so"))
    for h in ("engine_c_library.h", "upside_gb300.h", "upside_main.h"):
        names = declared(h)
        assert len(names) >= (1 if h == "upside_main.h" else 5), h
        for n in names:
            assert hasattr(lib, n), "%s missing from libupside.so (declared in %s)" % (n, h)


def test_drop_in_names_match_reference_interface():
    # the reference C library's entry points (src/engine_c_library.h:12-32)
    want = ["construct_deriv_engine", "free_deriv_engine", "evaluate_energy", "evaluate_deriv", "set_param",
            "get_param_deriv", "get_param", "get_output_dims", "get_output", "get_sens", "get_value_by_name",
            "clamped_spline_solve", "clamped_spline_value", "get_clamped_value_and_deriv",
            "get_clamped_coeff_deriv"]
    assert sorted(want) == sorted(declared("engine_c_library.h"))


def test_clamped_spline_helpers_match_oracle_math(built):
    """Stateless spline helpers run on the host: interpolation and coefficient derivatives."""
    import numpy as np
    lib = ctypes.CDLL(os.path.join(ROOT, "upside2-md_gb300", "libupside.so"))
    N = 12
    vals = np.sin(np.linspace(0, 2, N - 2)).astype(np.float32)
    coeff = np.zeros(N, np.float32)
    assert lib.clamped_spline_solve(N, coeff.ctypes.data, vals.ctypes.data) == 0
    x = np.arange(1, N - 1, dtype=np.float32)  # knots 1..N-2 carry the values
    res = np.zeros(len(x), np.float32)
    lib.clamped_spline_value(N, res.ctypes.data, coeff.ctypes.data, len(x), x.ctypes.data)
    assert np.abs(res - vals).max() < 2e-6
    cd = np.zeros(N, np.float32)
    lib.get_clamped_coeff_deriv.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_float]
    lib.get_clamped_coeff_deriv(N, cd.ctypes.data, coeff.ctypes.data, 4.3)
    # value is linear in the coefficients: dvalue/dcoeff . coeff == value
    v = np.zeros(1, np.float32)
    xx = np.array([4.3], np.float32)
    lib.clamped_spline_value(N, v.ctypes.data, coeff.ctypes.data, 1, xx.ctypes.data)
    assert abs(float(cd @ coeff) - float(v[0])) < 1e-6
    if os.path.exists(os.path.join(ROOT, "oracle", "_ref", "libupside_ref.so")):
        ref = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libupside_ref.so"))
        rc = np.zeros(N, np.float32)
        ref.clamped_spline_solve(N, rc.ctypes.data, vals.ctypes.data)
        assert np.abs(rc - coeff).max() < 1e-6
