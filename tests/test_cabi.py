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
    """The problems' host checks run before device discovery: a configuration error has its own
    code on any machine."""
    from nlfem_gb300 import nlfem, _lib
    m = square_mesh(4)
    with pytest.raises(_lib.NlfemError) as e:
        nlfem.stiffnessMatrix(m, {"function": "nope", "horizon": 0.1, "outputdim": 1}, conf2d())
    assert e.value.code == 4
    with pytest.raises(_lib.NlfemError) as e:   # chk_Conf: 3D takes the barycenter rule only
        from conftest import cube_mesh
        nlfem.stiffnessMatrix(cube_mesh(2), {"function": "constant3D", "horizon": 0.3, "outputdim": 1}, conf2d())
    assert e.value.code == 1


def _zeta(m, rows):
    import scipy.sparse as sp
    indptr = np.cumsum([0] + [len(r) for r in rows])
    m = dict(m)
    m["nZeta"] = 2
    m["ZetaIndicator"] = sp.csr_matrix((np.ones(indptr[-1]), np.concatenate(rows).astype(np.int64), indptr),
                                       shape=(len(rows), 2))
    return m


def test_zeta_subdomain_check(lib):
    """chk_Mesh (checks.cpp:74-84): the first 20 elements must share a subdomain pairwise, or the
    reference aborts; here the library refuses with NLFEM_ERR_INVALID and the reference's words,
    before it looks for a device. The load vector has no such check (the reference runs chk_Mesh
    for the system only)."""
    from nlfem_gb300 import nlfem, _lib
    m = square_mesh(6, 0.1)
    nE = m["elements"].shape[0]
    ker = {"function": "constant", "horizon": 0.1, "outputdim": 1}
    split = [[0] if e % 2 == 0 else [1] for e in range(nE)]   # elements 0 and 1 share none
    with pytest.raises(_lib.NlfemError, match="Zeta") as e:
        nlfem.stiffnessMatrix(_zeta(m, split), ker, conf2d())
    assert e.value.code == 1
    late = [[0, 1] if e < 20 else ([0] if e % 2 == 0 else [1]) for e in range(nE)]   # only later elements split
    ok = [_zeta(m, late), dict(m)]
    if lib.nlfem_device_count() == 0:
        for mm in ok:
            with pytest.raises(_lib.NlfemError) as e:
                nlfem.stiffnessMatrix(mm, ker, conf2d())
            assert e.value.code == 2   # past the host checks: no device
        with pytest.raises(_lib.NlfemError) as e:
            nlfem.loadVector(_zeta(m, split), {"function": "linear"}, conf2d())
        assert e.value.code == 2


def test_outdim_mismatch_raises_valueerror():
    from nlfem_gb300 import nlfem
    m = square_mesh(4)
    m["outdim"] = 2
    with pytest.raises(ValueError):
        nlfem.stiffnessMatrix(m, {"function": "constant", "horizon": 0.1, "outputdim": 1}, conf2d())


def test_reference_configuration_checks(lib):
    """chk_Conf (checks.cpp:105-113), where the reference aborts: the fractional close rule with the
    DG ansatz, and the prototype microelastic kernels with fractional_s other than -0.5. Refused
    with NLFEM_ERR_INVALID before any device work."""
    from nlfem_gb300 import nlfem, _lib
    m = square_mesh(4, 0.2)
    frac = {"function": "fractional", "horizon": 0.2, "outputdim": 1, "fractional_s": 0.4}
    c = conf2d(close="fractional", deg=3)
    c["ansatz"] = "DG"
    with pytest.raises(_lib.NlfemError, match="cannot be used for DG") as e:
        nlfem.stiffnessMatrix(dict(m), frac, c)
    assert e.value.code == 1
    for name, od in (("linearPrototypeMicroelastic", 1), ("linearPrototypeMicroelasticField", 2)):
        k = {"function": name, "horizon": 0.2, "outputdim": od, "fractional_s": 0.4}
        mm = dict(m, outdim=od)
        with pytest.raises(_lib.NlfemError, match="Please set fractional_s") as e:
            nlfem.stiffnessMatrix(mm, k, conf2d(close="fractional", deg=3))
        assert e.value.code == 1
