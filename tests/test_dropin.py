"""The reference's own Python module (cython/nlfem.pyx), compiled unchanged against this library:
its `cdef extern from "Cassemble.h"` finds include/Cassemble.h and it links libnlfem_gpu.so
(nlfem_gb300/dropin.py). The module's C++ source is generated with Cython where the reference
checkout is (build() leaves it in nlfem_gb300/_dropin/) and compiled here.

CPU: the module compiles and imports, and its host-only functions (tensorgauss, get_vertexLabel,
meshFromArrays) agree with nlfem_gb300.nlfem. GPU: its stiffnessMatrix / loadVector / evaluateMass,
whose par_assemble and par_evaluateMass are this library's, equal nlfem_gb300.nlfem's FP64 path
bit for bit and the oracle within rounding."""
import importlib.util
import os
from types import SimpleNamespace

import numpy as np
import pytest

from conftest import conf2d, conf3d, square_mesh, cube_mesh, rel_errors, same_pattern

FP64_TOL = 1e-12


@pytest.fixture(scope="module")
def refmod(tmp_path_factory):
    from nlfem_gb300 import dropin
    if not os.path.exists(dropin.GENERATED_CPP):
        pytest.skip("the reference module's generated C++ (nlfem_gb300/_dropin/nlfem.cpp) is absent: "
                    "build() makes it where the reference checkout and Cython are")
    if not dropin.can_compile():
        pytest.skip("Python.h is absent: the reference module cannot be compiled here")
    out = tmp_path_factory.mktemp("dropin")
    so = dropin.compile_module(dropin.GENERATED_CPP, str(out))
    spec = importlib.util.spec_from_file_location("nlfem", so)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    # the module calls numpy's removed alias np.int (nlfem.pyx:394, 427)
    had = hasattr(np, "int")
    if not had:
        np.int = int
    yield mod
    if not had:
        del np.int


def test_module_exports(refmod):
    for name in ("stiffnessMatrix", "loadVector", "stiffnessMatrix_fromArray", "assemble", "evaluateMass",
                 "meshFromArrays", "get_vertexLabel", "setSolutionLabels", "tensorgauss",
                 "py_retriangulate", "py_toRef", "py_toPhys", "py_solve2x2"):
        assert callable(getattr(refmod, name)), name


def test_host_functions_agree(refmod):
    from nlfem_gb300 import nlfem
    for deg in (2, 3, 5):
        a, b = refmod.tensorgauss(deg), nlfem.tensorgauss(deg)
        np.testing.assert_array_equal(a.points, b.points)
        np.testing.assert_array_equal(a.weights, b.weights)
    m = square_mesh(6, 0.2, jitter=0.1, seed=3)
    el = m["elements"].astype(np.int64)
    lab = m["elementLabels"].astype(np.int64)
    np.testing.assert_array_equal(refmod.get_vertexLabel(el, lab, m["vertices"]),
                                  nlfem.get_vertexLabel(el, lab, m["vertices"]))
    a = refmod.meshFromArrays(el, lab, m["vertices"])
    b = nlfem.meshFromArrays(el, lab, m["vertices"])
    for k in ("elements", "elementLabels", "vertices", "vertexLabels", "outdim"):
        np.testing.assert_array_equal(np.asarray(a[k]), np.asarray(b[k]))


def _ref_mesh(refmod, m):
    return refmod.meshFromArrays(m["elements"].astype(np.int64), m["elementLabels"].astype(np.int64),
                                 m["vertices"])


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["constant", "fractional", "cube"])
def test_stiffness_matrix_through_reference_module(refmod, case, monkeypatch, tmp_path):
    from nlfem_gb300 import nlfem
    from oracle import oracle
    monkeypatch.chdir(tmp_path)     # the module writes its arma files into the working directory
    if case == "constant":
        m, k, c = square_mesh(12, 0.15, jitter=0.2, seed=5), {"function": "constant", "horizon": 0.15, "outputdim": 1}, conf2d()
    elif case == "fractional":
        m = square_mesh(8, 0.2, jitter=0.1, seed=6)
        k = {"function": "fractional", "horizon": 0.2, "outputdim": 1, "fractional_s": 0.4}
        c = conf2d(close="fractional", deg=3)
    else:
        m, k, c = cube_mesh(5, 0.1, jitter=0.1, seed=7), {"function": "constant", "horizon": 0.1, "outputdim": 1}, conf3d()
    rm = _ref_mesh(refmod, m) if case != "cube" else dict(m)
    A = refmod.stiffnessMatrix(rm, k, c)
    assert not [f for f in os.listdir(tmp_path) if f.startswith("tmp_spAd")]   # removed after reading
    B = nlfem.stiffnessMatrix(dict(m), k, dict(c, precision="fp64"))
    A.sort_indices(); B.sort_indices()
    assert same_pattern(A, B)
    np.testing.assert_array_equal(A.data, B.data)
    C = oracle.assemble(m, k, c)["A"]
    assert same_pattern(A, C)
    fro, mx = rel_errors(A, C)
    assert fro < FP64_TOL and mx < FP64_TOL, (fro, mx)


@pytest.mark.gpu
def test_load_vector_and_mass_through_reference_module(refmod, monkeypatch, tmp_path):
    from nlfem_gb300 import nlfem
    from oracle import oracle
    monkeypatch.chdir(tmp_path)
    m = square_mesh(12, 0.1, jitter=0.2, seed=8)
    c = conf2d()
    f = refmod.loadVector(_ref_mesh(refmod, m), {"function": "linear"}, c)
    g = nlfem.loadVector(dict(m), {"function": "linear"}, dict(c, precision="fp64"))
    np.testing.assert_array_equal(f, g)
    h = oracle.assemble(m, None, c, compute="forcing", load={"function": "linear"})["f"]
    assert np.abs(f - h).max() <= 1e-13 * np.abs(h).max()
    nV = m["vertices"].shape[0]
    u = np.random.default_rng(9).normal(size=nV)
    P, w = c["quadrature"]["outer"]["points"], c["quadrature"]["outer"]["weights"]
    lm = SimpleNamespace(elements=m["elements"].astype(np.int64), elementLabels=m["elementLabels"].astype(np.int64),
                         vertices=m["vertices"], vertexLabels=m["vertexLabels"].astype(np.int64), dim=2,
                         nE_Omega=m["elements"].shape[0], K_Omega=nV, K=nV, is_DiscontinuousGalerkin=0)
    a = refmod.evaluateMass(lm, u, P, w)
    b = nlfem.evaluateMass(lm, u, P, w)
    np.testing.assert_array_equal(np.asarray(a), np.asarray(b))


@pytest.mark.gpu
def test_geometry_hooks_through_reference_module(refmod):
    from oracle import oracle
    T = np.array([0.1, 0.2, 0.9, 0.1, 0.3, 0.8])
    x = np.array([0.4, 0.35])
    p = np.asarray(refmod.py_toRef(T, x))
    np.testing.assert_allclose(np.asarray(refmod.py_toPhys(T, p)), x, rtol=0, atol=1e-15)
    A = np.array([2.0, 1.0, 1.0, 3.0]); b = np.array([1.0, 2.0])
    np.testing.assert_allclose(np.asarray(refmod.py_solve2x2(A, b)), np.linalg.solve(A.reshape(2, 2), b), rtol=1e-15)
    for caps in (0, 1):
        n, lst = refmod.py_retriangulate(np.array([0.3, 0.3]), T, 0.2, caps, None)
        k, tri = oracle.retriangulate(np.array([0.3, 0.3]), T, 0.2, caps)
        assert n == k
        np.testing.assert_array_equal(np.asarray(lst)[:2 * 3 * n], np.asarray(tri).ravel()[:2 * 3 * n])
