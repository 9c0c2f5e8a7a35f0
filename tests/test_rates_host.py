"""The host side of the convergence-rate run (nlfem_gb300/rates.py, after
examples/test2D/computeRates2D.py:17-111) on the CPU: the oracle stands in for the three GPU calls
(stiffnessMatrix, loadVector, evaluateMass), so the Dirichlet lift, the CG solve, both error
measures and the rates are checked without a device. The GPU run of the same pipeline is in
tests/test_gpu_rates.py."""
import numpy as np
import pytest


@pytest.fixture
def oracle_backed(monkeypatch):
    from nlfem_gb300 import nlfem
    from oracle import oracle
    monkeypatch.setattr(nlfem, "stiffnessMatrix", lambda m, k, c: oracle.assemble(m, k, c)["A"])
    monkeypatch.setattr(nlfem, "loadVector",
                        lambda m, load, c: oracle.assemble(m, None, c, compute="forcing", load=load)["f"])

    def mass(mesh, ud, P, dx):
        return oracle.evaluate_mass(mesh, ud, P, dx)
    monkeypatch.setattr(nlfem, "evaluateMass", mass)


def test_rates_pipeline_on_the_oracle(oracle_backed):
    """The constant kernel reproduces -Laplace on cubics, so the nonlocal solution of the linear
    load is u = x0^2 x1 + x1^2 and the error is P1 discretisation error: second-order rates in
    both measures, and the Dirichlet layer carries u exactly."""
    from nlfem_gb300 import rates
    r = rates.convergence([16, 32, 64])
    assert all(e > 0 for e in r["l2_error"])
    assert all(1.2 < q < 2.6 for q in r["rates"]) and 1.8 < r["rates"][-1] < 2.2, r["rates"]
    assert all(1.2 < q < 2.6 for q in r["mass_rates"]) and 1.8 < r["mass_rates"][-1] < 2.2, r["mass_rates"]
    assert all(k > 0 for k in r["cg_iterations"])


def test_solve_lifts_dirichlet_data(oracle_backed):
    from nlfem_gb300 import meshes, quadrules, rates
    v, e, l = meshes.regular_square(10, 0.1)
    mesh = meshes.mesh_dict(v, e, l)
    P, w = quadrules.dunavant7()
    conf = {"ansatz": "CG", "approxBalls": {"method": "retriangulate", "is_PlacePointOnCap": 1},
            "quadrature": {"outer": {"points": P, "weights": w}, "inner": {"points": P, "weights": w}}}
    k = {"function": "constant", "horizon": 0.1, "outputdim": 1}
    uh, its = rates.solve(mesh, k, conf, {"function": "linear"}, rates.u_quadratic)
    layer = mesh["vertexLabels"] < 0
    np.testing.assert_array_equal(uh[layer], rates.u_quadratic(mesh["vertices"][layer]))
    assert its > 0 and np.isfinite(uh).all()
    # l2_error of the exact interpolant is the interpolation error only, far below the solve's
    ui = rates.u_quadratic(mesh["vertices"])
    assert rates.l2_error(mesh, ui, rates.u_quadratic) < rates.l2_error(mesh, np.zeros_like(ui), rates.u_quadratic)
