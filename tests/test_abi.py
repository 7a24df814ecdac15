"""The C ABI library loads, exports every declared symbol and validates
mixtures on the host (no GPU needed for any of this)."""

import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "mpmc_gb300_flash.h")


@pytest.fixture(scope="module")
def lib():
    from mpmc_hnu_gb300 import build, flash

    build.build()
    return flash.library()


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(mpmc_(?:gpu_flash|flash_server)_\w+)\s*\(", text)))


def test_header_declares_the_abi():
    names = declared_functions()
    from mpmc_hnu_gb300 import flash

    assert set(names) == set(flash.EXPORTED_SYMBOLS)


def test_every_declared_symbol_is_exported(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_abi_version(lib):
    assert lib.mpmc_gpu_flash_abi_version() == 1


def _mixture(tc, pc, omega, kij):
    from mpmc_hnu_gb300.flash import _Mixture

    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (tc, pc, omega, np.asarray(kij).reshape(-1))]
    return _Mixture(len(tc), *(a.ctypes.data for a in arrs)), arrs


@pytest.mark.parametrize("case,code", [
    ("negative_tc", 2), ("asymmetric_kij", 2), ("diagonal_kij", 2), ("nan_omega", 2), ("too_many", 4)])
def test_create_rejects_bad_mixtures_before_touching_the_device(lib, case, code):
    from mpmc_hnu_gb300.flash import _Options

    n = 21 if case == "too_many" else 3
    tc = np.full(n, 300.0)
    pc = np.full(n, 4e6)
    omega = np.full(n, 0.1)
    kij = np.zeros((n, n))
    if case == "negative_tc":
        tc[1] = -5.0
    elif case == "asymmetric_kij":
        kij[0, 1] = 0.05
    elif case == "diagonal_kij":
        kij[2, 2] = 0.01
    elif case == "nan_omega":
        omega[0] = np.nan
    m, keep = _mixture(tc, pc, omega, kij)
    h = ctypes.c_void_p()
    rc = lib.mpmc_gpu_flash_create(ctypes.byref(m), ctypes.byref(_Options(0, 0, 0, 0)), ctypes.byref(h))
    assert rc == code
    assert not h.value
    assert lib.mpmc_gpu_flash_last_error()


def test_null_arguments_are_rejected(lib):
    assert lib.mpmc_gpu_flash_create(None, None, None) == 1
    assert lib.mpmc_gpu_flash_solve(None, 1, None, None, None, None) == 1
    assert lib.mpmc_gpu_flash_solve_device(None, 1, None, None, None, None, None) == 1
    assert lib.mpmc_gpu_flash_destroy(None) == 0


def test_null_arguments_of_the_warm_and_max3_entries(lib):
    """The warm-start and max-3-phase entries validate before any device work."""
    assert lib.mpmc_gpu_flash_solve_warm(None, 1, None, None, None, None, None) == 1
    assert lib.mpmc_gpu_flash_solve_device_warm(None, 1, None, None, None, None, None, None) == 1
    assert lib.mpmc_gpu_flash_solve_max3(None, 1, None, None, None, None, None) == 1
    assert lib.mpmc_gpu_flash_solve_device_max3(None, 1, None, None, None, None, None, None) == 1
    assert b"null handle" in lib.mpmc_gpu_flash_last_error()


def test_null_arguments_of_the_property_chart_entries(lib):
    """The property-chart entries validate before any device work."""
    assert lib.mpmc_gpu_flash_property_chart(None, 1, None, None, None, None) == 1
    assert lib.mpmc_gpu_flash_property_chart_device(None, 1, None, None, None, None, None) == 1
    assert b"null handle" in lib.mpmc_gpu_flash_last_error()


def test_chart_shape():
    from mpmc_hnu_gb300 import flash

    assert flash.chart_shape(10, 1) == (15, 11)
    assert flash.chart_shape(10, 2) == (40, 21)
    assert flash.chart_shape(3, 3) == (30, 10)


def test_null_arguments_of_the_hinted_entries(lib):
    """The hinted entries validate before any device work."""
    assert lib.mpmc_gpu_flash_solve_hinted(None, 1, None, None, None, None, None, None) == 1
    assert lib.mpmc_gpu_flash_solve_device_hinted(None, 1, None, None, None, None, None, None, None) == 1
    assert b"null handle" in lib.mpmc_gpu_flash_last_error()
