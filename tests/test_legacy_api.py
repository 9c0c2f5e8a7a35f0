"""The reference's deprecated Python entry points (nlfem.pyx:103-105, 483-636, 678-710): host-side
argument handling, checked on the CPU. The assembly behind them is stiffnessMatrix / loadVector,
whose GPU parity the gpu tests cover."""
import types

import numpy as np
import pytest
import scipy.sparse as sp

from conftest import square_mesh


def _legacy_mesh(n=4):
    m = square_mesh(n, 0.1)
    nE, nV = m["elements"].shape[0], m["vertices"].shape[0]
    keep = m["vertexLabels"] > 0
    return types.SimpleNamespace(
        elements=m["elements"].ravel(), elementLabels=m["elementLabels"], vertices=m["vertices"].ravel(),
        vertexLabels=m["vertexLabels"], nE=nE, nV=nV, nE_Omega=int((m["elementLabels"] > 0).sum()),
        nV_Omega=int(keep.sum()), K=nV, K_Omega=int(keep.sum()), dim=2, is_DiscontinuousGalerkin=0,
        is_NeumannBoundary=0), m


def test_construct_adjacency_graph():
    from nlfem_gb300 import nlfem
    el = np.array([[0, 1, 2], [1, 3, 2], [3, 4, 5]])   # 0-1 share an edge, 1-2 a vertex
    np.testing.assert_array_equal(nlfem.constructAdjaciencyGraph(el),
                                  [[0, 1, 3], [0, 1, 2], [1, 2, 3]])
    np.testing.assert_array_equal(nlfem.constructAdjaciencyGraph(el, ncommon=2),
                                  [[0, 1], [0, 1], [2, 3]])


def test_legacy_assemble_arguments(monkeypatch, tmp_path):
    from nlfem_gb300 import nlfem, quadrules
    calls = {}
    K = 25

    def fake_A(mesh, kernel, conf):
        calls["A"] = (mesh, kernel, conf)
        return sp.identity(K, format="csr")

    def fake_f(mesh, load, conf):
        calls["f"] = (mesh, load, conf)
        return np.arange(K, dtype=float)

    monkeypatch.setattr(nlfem, "stiffnessMatrix", fake_A)
    monkeypatch.setattr(nlfem, "loadVector", fake_f)
    lm, m = _legacy_mesh()
    P, w = quadrules.dunavant7()
    A, f = nlfem.assemble(lm, P, P, w, w, 0.1, path_spAd=str(tmp_path / "A"), model_kernel="parabola",
                          model_f="linear", integration_method="baryCenter", is_PlacePointOnCap=0,
                          tensorGaussDegree=3)
    assert A.shape == (lm.K_Omega, K) and np.array_equal(f, np.arange(lm.K_Omega))
    mesh, kernel, conf = calls["A"]
    np.testing.assert_array_equal(mesh["elements"], m["elements"])
    np.testing.assert_array_equal(mesh["vertices"], m["vertices"])
    assert kernel == {"function": "parabola", "horizon": 0.1, "outputdim": 1, "fractional_s": -1.0}
    assert conf["approxBalls"] == {"method": "baryCenter", "is_PlacePointOnCap": 0}
    assert conf["closeElements"] == "baryCenter" and conf["ansatz"] == "CG"
    assert conf["quadrature"]["tensorGaussDegree"] == 3 and conf["savePath"] == str(tmp_path / "A")
    assert calls["f"][1] == {"function": "linear"} and "savePath" not in calls["f"][2]
    calls.clear()
    A, f = nlfem.assemble(lm, P, P, w, w, 0.1, compute="forcing")
    assert A is None and "A" not in calls and f.shape == (lm.K_Omega,)
    A, f = nlfem.assemble(lm, P, P, w, w, 0.1, compute="system")
    assert f is None and A.shape == (lm.K_Omega, K)


def test_legacy_assemble_reaches_the_library_without_cpu_fallback():
    from nlfem_gb300 import nlfem, quadrules, _lib
    if _lib.load().nlfem_device_count() > 0:
        pytest.skip("a CUDA device is visible")
    lm, _ = _legacy_mesh()
    P, w = quadrules.dunavant7()
    with pytest.raises(_lib.NlfemError):
        nlfem.assemble(lm, P, P, w, w, 0.1)


def test_remove_arma_tmp(tmp_path):
    from nlfem_gb300 import nlfem
    p = tmp_path / "tmp_fd"
    nlfem.write_arma_mat(str(p), np.ones(3))
    nlfem.remove_arma_tmp(str(p))
    assert not p.exists()
