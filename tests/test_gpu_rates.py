"""Convergence rates of the solved problem (examples/test2D/computeRates2D.py:17-111): the
mixed-precision operator must give the same L2 error rates as the all-FP64 one."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_mixed_rates_equal_fp64_rates():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from nlfem_gb300 import rates
    ns = [16, 32, 64, 128]
    a = rates.convergence(ns, precision="fp64")
    b = rates.convergence(ns, precision="mixed")
    # second order in L2 for P1 (pre-asymptotic first step excluded)
    assert all(1.9 < r < 2.1 for r in a["rates"][1:]), a
    np.testing.assert_allclose(b["rates"], a["rates"], atol=0.01)
    np.testing.assert_allclose(b["l2_error"], a["l2_error"], rtol=5e-3)
    # the reference's measure, sqrt(d . M d) with the GPU mass product: same rates for both
    # operators (the nodal difference converges at least at second order)
    assert all(r > 1.8 for r in a["mass_rates"][1:]), a
    np.testing.assert_allclose(b["mass_rates"], a["mass_rates"], atol=0.02)


def test_mixed_operator_annihilates_constants():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from nlfem_gb300 import meshes, nlfem, quadrules
    v, e, l = meshes.regular_square(48, 0.1, jitter=0.2, seed=7)
    m = meshes.mesh_dict(v, e, l)
    P, w = quadrules.dunavant7()
    conf = {"ansatz": "CG", "approxBalls": {"method": "retriangulate", "is_PlacePointOnCap": 1},
            "quadrature": {"outer": {"points": P, "weights": w}, "inner": {"points": P, "weights": w}},
            "precision": "mixed"}
    k = {"function": "constant", "horizon": 0.1, "outputdim": 1}
    A = nlfem.stiffnessMatrix(m, k, conf).tocsr()
    # every kept row of A sums to zero up to the conversion of its fixed-point sum to FP64
    rs = np.abs(A @ np.ones(A.shape[1]))
    scale = np.abs(A).max()
    assert rs.max() <= 1e-14 * scale, rs.max() / scale


def test_gpu_solve_matches_host_solve():
    """CG on the GPU (Session.solve) against scipy's CG on the same assembled operator."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from nlfem_gb300 import meshes, rates, quadrules
    v, e, l = meshes.regular_square(32, 0.1)
    m = meshes.mesh_dict(v, e, l)
    P, w = quadrules.dunavant7()
    for prec in ("fp64", "mixed"):
        conf = {"ansatz": "CG", "approxBalls": {"method": "retriangulate", "is_PlacePointOnCap": 1},
                "quadrature": {"outer": {"points": P, "weights": w}, "inner": {"points": P, "weights": w}},
                "precision": prec}
        k = {"function": "constant", "horizon": 0.1, "outputdim": 1}
        uh, it_h = rates.solve(m, k, conf, {"function": "linear"}, rates.u_quadratic)
        ug, it_g = rates.solve_gpu(m, k, conf, {"function": "linear"}, rates.u_quadratic)
        assert np.abs(ug - uh).max() <= 1e-8 * np.abs(uh).max(), prec
        assert abs(it_g - it_h) <= max(5, it_h // 10), (it_g, it_h)
        ug2, _ = rates.solve_gpu(m, k, conf, {"function": "linear"}, rates.u_quadratic)
        assert np.array_equal(ug, ug2)   # deterministic
