"""CPU checks of the C ABI: the library builds, loads, exports every declared symbol and, without
a GPU, refuses to compute instead of falling back to the CPU."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, conf2d, square_mesh


@pytest.fixture(scope="module")
def lib():
    from nlfem_gb300 import _lib
    return _lib.load()


def _declared_c_functions():
    src = open(os.path.join(ROOT, "include", "nlfem_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(nlfem_\w+)\s*\(", src)))


def test_header_lists_match_binding():
    from nlfem_gb300 import _lib
    assert _declared_c_functions() == sorted(_lib.EXPORTED)


def test_all_c_symbols_exported(lib):
    for name in _declared_c_functions():
        assert hasattr(lib, name), name


def test_cpp_compat_symbols_exported(lib):
    from nlfem_gb300 import _lib
    out = subprocess.run(["nm", "-D", "--defined-only", "-C", _lib.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    for sym in ["par_assemble(std::__cxx11::basic_string", "method_retriangulate(double const*",
                "par_evaluateMass(double*, double const*, long*, long const*, double const*, long const*, int, int, int, double*, double const*, int, int, int)",
                "toRef(double const*", "toPhys(double const*", "solve2x2(double const*"]:
        assert sym in out, sym


def test_no_cpu_fallback_without_device(lib):
    from nlfem_gb300 import nlfem, _lib
    if lib.nlfem_device_count() > 0:
        pytest.skip("a CUDA device is present")
    m = square_mesh(4)
    ker = {"function": "constant", "horizon": 0.1, "outputdim": 1}
    with pytest.raises(_lib.NlfemError) as e:
        nlfem.stiffnessMatrix(m, ker, conf2d())
    assert e.value.code == 2


def test_evaluate_mass_no_cpu_fallback_and_checks(lib):
    from nlfem_gb300 import nlfem, _lib, quadrules
    m = square_mesh(4)
    P, w = quadrules.dunavant7()
    ud = np.ones(m["vertices"].shape[0])
    with pytest.raises(ValueError):   # wrong vector length: caught before the library call
        nlfem.evaluateMass(m, ud[:-1], P, w)
    if lib.nlfem_device_count() > 0:
        pytest.skip("a CUDA device is present")
    with pytest.raises(_lib.NlfemError) as e:
        nlfem.evaluateMass(m, ud, P, w)
    assert e.value.code == 2


def test_invalid_configuration_is_reported(lib):
    from nlfem_gb300 import nlfem, _lib
    if lib.nlfem_device_count() == 0:
        pytest.skip("configuration checks run after device discovery")
    m = square_mesh(4)
    with pytest.raises(_lib.NlfemError):
        nlfem.stiffnessMatrix(m, {"function": "nope", "horizon": 0.1, "outputdim": 1}, conf2d())


def test_outdim_mismatch_raises_valueerror():
    from nlfem_gb300 import nlfem
    m = square_mesh(4)
    m["outdim"] = 2
    with pytest.raises(ValueError):
        nlfem.stiffnessMatrix(m, {"function": "constant", "horizon": 0.1, "outputdim": 1}, conf2d())
