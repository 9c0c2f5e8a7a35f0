"""CPU checks of the oracle and of the host-side helpers against the reference's fixtures."""
import json
import os

import numpy as np
import pytest
import scipy.sparse as sp

from conftest import conf2d, conf3d, square_mesh, cube_mesh

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_quadrules_match_reference_configuration():
    from nlfem_gb300 import quadrules
    ref = json.load(open(os.path.join(GOLD, "quadrules_ref.json")))
    P, w = quadrules.dunavant7()
    np.testing.assert_allclose(P, ref["7point"]["points"], atol=1e-13)
    np.testing.assert_allclose(w, ref["7point"]["weights"], atol=1e-13)
    P, w = quadrules.dunavant16()
    np.testing.assert_allclose(P, ref["16point"]["points"], atol=1e-8)
    np.testing.assert_allclose(w, ref["16point"]["weights"], atol=1e-13)


def test_keast_rule_is_degree_4_exact():
    from math import factorial
    from nlfem_gb300 import quadrules
    P, w = quadrules.keast11()
    assert abs(w.sum() - 1.0 / 6.0) < 1e-15
    for a in range(5):
        for b in range(5 - a):
            for c in range(5 - a - b):
                exact = factorial(a) * factorial(b) * factorial(c) / factorial(a + b + c + 3)
                got = np.sum(w * P[:, 0] ** a * P[:, 1] ** b * P[:, 2] ** c)
                assert abs(got - exact) < 1e-14


def test_tensorgauss_matches_reference_class():
    from nlfem_gb300.quadrules import tensorgauss
    ref = np.load(os.path.join(GOLD, "tensorgauss_ref.npz"))
    for deg in (2, 5):
        tg = tensorgauss(deg)
        np.testing.assert_array_equal(tg.points, ref[f"points{deg}"])
        np.testing.assert_array_equal(tg.weights, ref[f"weights{deg}"])


def test_vertex_labels_match_reference():
    from nlfem_gb300.meshes import get_vertexLabel
    d = json.load(open(os.path.join(GOLD, "vertexlabels_ref.json")))
    got = get_vertexLabel(np.array(d["elements"]), np.array(d["elementLabels"]), np.array(d["vertices"]))
    np.testing.assert_array_equal(got, d["vertexLabels"])


def test_cube_split_matches_reference_golden_list():
    from nlfem_gb300.meshes import regular_cube
    d = json.load(open(os.path.join(GOLD, "tets_ref.json")))
    v, e, l = regular_cube(d["n_cells"], 0.1)
    np.testing.assert_array_equal(e, np.array(d["tets"]))


def test_arma_writer_matches_reference_reader():
    ref = np.load(os.path.join(GOLD, "arma_ref.npz"))
    np.testing.assert_array_equal(ref["A_dense"], ref["B_dense"])
    np.testing.assert_array_equal(ref["f"], ref["g"])


def test_arma_roundtrip(tmp_path):
    from nlfem_gb300.nlfem import write_arma_spMat, read_arma_spMat, write_arma_mat, read_arma_mat
    A = sp.random(13, 13, density=0.3, random_state=np.random.RandomState(1), format="csr")
    write_arma_spMat(tmp_path / "A", A)
    B = read_arma_spMat(tmp_path / "A")
    assert abs(A - B).max() == 0
    f = np.arange(13.0)
    write_arma_mat(tmp_path / "f", f)
    np.testing.assert_array_equal(read_arma_mat(tmp_path / "f")[:, 0], f)
    with pytest.raises(ValueError):
        read_arma_mat(tmp_path / "A")


def test_oracle_constant_kernel_invariants():
    from oracle import oracle
    m = square_mesh(12, 0.1)
    ker = {"function": "constant", "horizon": 0.1, "outputdim": 1}
    r = oracle.assemble(m, ker, conf2d(), want_pairs=True)
    A = r["A"]
    assert r["n_errors"] == 0
    assert r["n_pairs"] == len(r["pairs"])
    # the operator annihilates constants on rows whose full stencil is assembled
    keep = m["vertexLabels"] > 0
    assert np.abs(A @ np.ones(A.shape[0]))[keep].max() < 1e-12 * abs(A).max()
    # Dirichlet rows are empty
    assert np.all(np.diff(A.indptr)[~keep] == 0)
    # every outer element interacts with itself
    pairs = set(map(tuple, r["pairs"]))
    for e in range(m["elements"].shape[0]):
        assert (e, e) in pairs


def test_oracle_thread_split_is_rounding_only():
    from oracle import oracle
    m = square_mesh(10, 0.1, jitter=0.2, seed=1)
    ker = {"function": "parabola", "horizon": 0.15, "outputdim": 1}
    a = oracle.assemble(m, ker, conf2d())["A"]
    b = oracle.assemble(m, ker, conf2d(), nthreads=4)["A"]
    assert (a != 0).nnz == (b != 0).nnz
    assert abs(a - b).max() <= 1e-13 * abs(a).max()


def test_oracle_retriangulate_area_and_caps():
    from oracle import oracle
    # a ball deep inside a large triangle: no polygon point -> no interaction (reference quirk)
    T = np.array([0.0, 0.0, 10.0, 0.0, 0.0, 10.0])
    n, tri = oracle.retriangulate(np.array([2.0, 2.0]), T, 0.5)
    assert n == 0
    # triangle fully inside the ball: one sub-triangle, the triangle itself
    T = np.array([0.0, 0.0, 0.1, 0.0, 0.0, 0.1])
    n, tri = oracle.retriangulate(np.array([0.02, 0.02]), T, 1.0)
    assert n == 1 and np.allclose(tri[0].ravel(), T)
    # ball center at a vertex of a large triangle: area close to a quarter disc with caps
    T = np.array([0.0, 0.0, 1.0, 0.0, 0.0, 1.0])
    areas = []
    for caps in (0, 1):
        n, tri = oracle.retriangulate(np.array([0.0, 0.0]), T, 0.3, caps)
        a = sum(abs(np.linalg.det(np.array([t[1] - t[0], t[2] - t[0]]))) / 2 for t in tri)
        areas.append(a)
    assert areas[0] < areas[1] < np.pi * 0.09 / 4


def test_oracle_fractional_and_3d_run():
    from oracle import oracle
    m = square_mesh(6, 0.2)
    ker = {"function": "fractional", "horizon": 0.2, "outputdim": 1, "fractional_s": 0.4}
    r = oracle.assemble(m, ker, conf2d(rule="16", close="fractional", deg=3))
    assert r["n_close"] > 0 and r["n_errors"] == 0
    A = r["A"]
    assert np.all(np.isfinite(A.data))
    m3 = cube_mesh(3, 0.1)
    ker3 = {"function": "constant3D", "horizon": 0.3, "outputdim": 1}
    r3 = oracle.assemble(m3, ker3, conf3d())
    assert r3["A"].nnz > 0


def test_oracle_load_vector_linear():
    from oracle import oracle
    m = square_mesh(8, 0.1)
    f = oracle.assemble(m, None, conf2d(), compute="forcing", load={"function": "linear"})["f"]
    keep = m["vertexLabels"] > 0
    assert np.all(f[~keep] == 0)
    # sum of the load over all basis functions of label>0 elements = integral of f over them
    assert np.all(f[keep] < 0)


def test_oracle_label_kernels_reduce_to_constant():
    """The label- and position-dependent kernels (model.cpp:30-42, 67-114) equal the constant
    kernel, or a multiple of it, where their cases say so."""
    from oracle import oracle
    m = square_mesh(10, 0.1, jitter=0.1, seed=2)
    conf = conf2d()

    def A(mesh, name):
        r = oracle.assemble(mesh, {"function": name, "horizon": 0.1, "outputdim": 1}, conf)
        assert r["n_errors"] == 0
        return r["A"]

    C = A(m, "constant")
    # every quadrature point lies inside the ball: truncation changes nothing
    assert abs(A(m, "constantTruncated") - C).max() == 0
    # labels 1 and -1 never sum to 7
    assert abs(A(m, "labeledNotch") - C).max() == 0
    # 10 lx + ly <= 12 for labels 1 and -1: the constant 0.03 / (4 delta^4)
    assert abs(A(m, "labeled") - C * (0.03 * np.pi / 16)).max() <= 1e-14 * abs(C).max()
    # left of x0 = 0 nothing crosses the notch
    ms = dict(m)
    ms["vertices"] = m["vertices"] - np.array([2.0, 0.5])
    assert abs(A(ms, "notch") - A(ms, "constant")).max() == 0
    assert abs(A(dict(m, vertices=m["vertices"] - 0.5), "notch") - C).max() > 0.1 * abs(C).max()
    # equal labels: the valve is open in both directions
    m1 = dict(m)
    m1["elementLabels"] = np.ones_like(m["elementLabels"])
    m1["vertexLabels"] = np.ones_like(m["vertexLabels"])
    assert abs(A(m1, "labeledValve") - A(m1, "constant")).max() == 0
    # Omega split into labels 1 and 2: closed from 1 towards 2
    m2 = dict(m)
    bx = m["vertices"][m["elements"]].mean(axis=1)[:, 0]
    m2["elementLabels"] = np.where(m["elementLabels"] > 0, np.where(bx < 0.5, 1, 2), -1)
    assert abs(A(m2, "labeledValve") - A(m2, "constant")).max() > 0.1 * abs(C).max()


def test_oracle_labeled_kernel_outside_its_cases_is_nan():
    """Labels 2 and -1 give 10 * 2 - 1 = 19, a case the reference aborts on (model.cpp:86-88)."""
    from oracle import oracle
    m = square_mesh(8, 0.1)
    m["elementLabels"] = np.where(m["elementLabels"] > 0, 2, -1)
    r = oracle.assemble(m, {"function": "labeled", "horizon": 0.1, "outputdim": 1}, conf2d())
    assert np.isnan(r["A"].data).any()


def test_oracle_notruncation_closed_form():
    """noTruncation (integrate_fullyContained, integration.cpp:290-343) with the constant kernel c
    integrates every element pair in full: A = 2 c (|D| M - m m^T) on the kept rows, M the P1 mass
    matrix, m the integrals of the basis functions and |D| the area of the mesh."""
    from oracle import oracle
    m = square_mesh(4, 0.1, jitter=0.1, seed=3)
    conf = conf2d(method="noTruncation")
    ker = {"function": "constant", "horizon": 0.1, "outputdim": 1}
    r = oracle.assemble(m, ker, conf, want_pairs=True)
    nE = m["elements"].shape[0]
    assert r["n_pairs"] == nE * nE
    A = r["A"].toarray()
    V, T = m["vertices"], m["elements"]
    nV = V.shape[0]
    M = np.zeros((nV, nV)); mv = np.zeros(nV); area = 0.0
    for t in T:
        e1, e2 = V[t[1]] - V[t[0]], V[t[2]] - V[t[0]]
        at = 0.5 * abs(e1[0] * e2[1] - e1[1] * e2[0])
        area += at
        M[np.ix_(t, t)] += at / 12 * (np.ones((3, 3)) + np.eye(3))
        mv[t] += at / 3
    c = 4 / (np.pi * 0.1 ** 4)
    B = 2 * c * (area * M - np.outer(mv, mv))
    B[m["vertexLabels"] <= 0] = 0
    assert np.abs(A - B).max() <= 1e-12 * np.abs(B).max()


@pytest.mark.parametrize("method", ["retriangulate_unsymm", "subSetBall", "averageBall", "baryCenterRT"])
def test_oracle_one_sided_rules_annihilate_constants(method):
    """The weight-2 rules with two blocks (integration.cpp:542-704, 1021-1095, 1155-1249): with the
    constant kernel every kept row sums to zero."""
    from oracle import oracle
    m = square_mesh(10, 0.1, jitter=0.15, seed=4)
    ker = {"function": "constant", "horizon": 0.1, "outputdim": 1}
    r = oracle.assemble(m, ker, conf2d(method=method))
    assert r["n_errors"] == 0 and r["n_pairs"] > 0
    A = r["A"]
    keep = m["vertexLabels"] > 0
    assert np.abs(A @ np.ones(A.shape[0]))[keep].max() < 1e-12 * abs(A).max()
    R = oracle.assemble(m, ker, conf2d())["A"]
    assert abs(A - R).max() > 1e-3 * abs(R).max()   # not the retriangulate matrix


def test_oracle_dg_sums_to_cg():
    """DG scatters the same element blocks to element DOFs dV e + a (Cassemble.cpp:580-585,
    637-642) and keeps every row: summed over the vertex copies, its rows and columns give the CG
    matrix and load vector on the kept rows."""
    from oracle import oracle
    m = square_mesh(8, 0.1, jitter=0.15, seed=6)
    ker = {"function": "parabola", "horizon": 0.1, "outputdim": 1}
    cdg = conf2d(); cdg["ansatz"] = "DG"
    D = oracle.assemble(m, ker, cdg)["A"]
    C = oracle.assemble(m, ker, conf2d())["A"]
    T = m["elements"]; nE, nV = T.shape[0], m["vertices"].shape[0]
    assert D.shape == (3 * nE, 3 * nE)
    P = sp.csr_matrix((np.ones(3 * nE), (np.arange(3 * nE), T.ravel())), shape=(3 * nE, nV))
    S = (P.T @ D @ P).toarray()
    keep = m["vertexLabels"] > 0
    S[~keep] = 0
    assert np.abs(S - C.toarray()).max() <= 1e-12 * abs(C).max()
    fd = oracle.assemble(m, None, cdg, compute="forcing", load={"function": "linear"})["f"]
    fc = oracle.assemble(m, None, conf2d(), compute="forcing", load={"function": "linear"})["f"]
    assert fd.shape == (3 * nE,)
    g = P.T @ fd
    assert np.abs(g[keep] - fc[keep]).max() <= 1e-13 * np.abs(fc).max()


def test_oracle_linear_prototype_is_fractional_at_s_minus_half():
    """kernel_linearPrototypeMicroelastic (model.cpp:116-124), 3 / (pi delta^3) / |x - y|, is the
    fractional kernel's formula at s = -1/2 (model.cpp:126-138): 2 - 2s = 3, d + 2s = 1 and
    pow(r, 1) = r, so with the same Duffy tables the two assemblies agree bit for bit."""
    from oracle import oracle
    m = square_mesh(8, 0.1, jitter=0.15, seed=9)
    conf = conf2d(rule="16", close="fractional", deg=3)
    kp = {"function": "linearPrototypeMicroelastic", "horizon": 0.1, "outputdim": 1, "fractional_s": -0.5}
    kf = {"function": "fractional", "horizon": 0.1, "outputdim": 1, "fractional_s": -0.5}
    a = oracle.assemble(m, kp, conf)
    b = oracle.assemble(m, kf, conf)
    assert a["n_close"] > 0 and a["n_close"] == b["n_close"]
    A, B = a["A"], b["A"]
    assert np.array_equal(A.indptr, B.indptr) and np.array_equal(A.indices, B.indices)
    assert np.array_equal(A.data, B.data)


def test_oracle_weak_singular_rule_matches_fractional_rule():
    """integrate_weakSingular (integration.cpp:82-185) integrates the four terms of the bilinear
    form one by one, with xi^(1 - 2s); integrate_fractional integrates (psi(x) - psi(y)) products
    with xi^(3 - 2s). For a weakly singular kernel (here |z|^-1, s = -1/2) the assembled matrices
    are the same sums up to rounding; the blocks are not."""
    from oracle import oracle
    m = square_mesh(8, 0.1, jitter=0.15, seed=9)
    kp = {"function": "linearPrototypeMicroelastic", "horizon": 0.1, "outputdim": 1, "fractional_s": -0.5}
    for deg in (2, 4):
        W = oracle.assemble(m, kp, conf2d(rule="16", close="weakSingular", deg=deg))
        F = oracle.assemble(m, kp, conf2d(rule="16", close="fractional", deg=deg))
        assert W["n_close"] == F["n_close"] > 0
        D = (W["A"] - F["A"]).tocsr()
        assert abs(D).max() <= 1e-13 * abs(F["A"]).max()
    pairs = np.array([[5, 5], [5, 6], [5, 4]])
    bw, _ = oracle.pair_blocks(m, kp, conf2d(rule="16", deg=3), pairs, method="weakSingular")
    bf, _ = oracle.pair_blocks(m, kp, conf2d(rule="16", deg=3), pairs, method="fractional")
    assert np.abs(bw - bf).max() > 1e-6 * np.abs(bf).max()


def _golden_cases_module():
    import importlib.util
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "make_oracle_golden.py")
    spec = importlib.util.spec_from_file_location("make_oracle_golden", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.mark.parametrize("name", ["config1", "tangent", "parabola20", "frac12", "cube5", "labeled10", "average10",
                                  "exact8", "dg10", "weak10", "field8", "linf8"])
def test_oracle_matches_committed_fixtures(name):
    """The oracle against tests/golden/oracle_cases.npz: the same inputs, the same pattern and
    pair list bit for bit, values and load vectors to 1e-13 (libm differences across hosts)."""
    mg = _golden_cases_module()
    fx = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "oracle_cases.npz"))
    case = mg.cases()[name]
    assert str(fx[f"{name}.input_sha"]) == mg.input_hash(*case[:3])
    for k in ("elements", "elementLabels", "vertices", "vertexLabels"):
        np.testing.assert_array_equal(case[0][k], fx[f"{name}.{k}"])
    out = mg.compute(name, case)
    np.testing.assert_array_equal(out[f"{name}.indptr"], fx[f"{name}.indptr"])
    np.testing.assert_array_equal(out[f"{name}.indices"], fx[f"{name}.indices"])
    assert str(out[f"{name}.pairs_sha"]) == str(fx[f"{name}.pairs_sha"])
    d = fx[f"{name}.data"]
    np.testing.assert_allclose(out[f"{name}.data"], d, rtol=1e-13, atol=1e-13 * np.abs(d).max())
    if f"{name}.f" in fx:
        f = fx[f"{name}.f"]
        np.testing.assert_allclose(out[f"{name}.f"], f, rtol=1e-13, atol=1e-15 * np.abs(f).max())


def test_oracle_constant_field_components():
    """kernelField_constant (model.cpp:180-191) is K = c [[1, 0], [1, 0]]. The blocks of a pair
    carry K (termLocal, termNonloc) and the prime blocks, scattered transposed
    (Cassemble.cpp:755-766), carry K^T. With A_s = M + P the scalar constant-kernel matrix split
    into those two parts, the outdim-2 matrix (rows 2v + i, columns 2w + j) has the components
    (0, 0) = A_s, (1, 1) = 0, (1, 0) = M and (0, 1) = P: so (0, 1) + (1, 0) = A_s."""
    from oracle import oracle
    m = square_mesh(8, 0.1, jitter=0.15, seed=3)
    A = oracle.assemble(m, {"function": "constant", "horizon": 0.1, "outputdim": 1}, conf2d())["A"].toarray()
    V = oracle.assemble(m, {"function": "constantField", "horizon": 0.1, "outputdim": 2}, conf2d())["A"].toarray()
    assert V.shape == (2 * A.shape[0], 2 * A.shape[0])
    tol = 1e-14 * np.abs(A).max()
    assert np.abs(V[0::2, 0::2] - A).max() <= tol
    assert np.abs(V[1::2, 1::2]).max() == 0
    assert np.abs(V[0::2, 1::2] + V[1::2, 0::2] - A).max() <= tol
    assert np.abs(V[0::2, 1::2]).max() > 0.1 * np.abs(A).max()   # both parts are present
    assert np.abs(V[1::2, 0::2]).max() > 0.1 * np.abs(A).max()


def _kept_rows(m, od):
    return np.repeat(m["vertexLabels"] > 0, od)


def test_oracle_microelastic_field_annihilates_rigid_motions():
    """kernelField_linearPrototypeMicroelastic (model.cpp:140-153), c z z^T / |z|^3, singular with
    the fractional close rule: translations and the rotation (-x1, x0) make the integrand
    K(x - y)(u(x) - u(y)) vanish pointwise, so every kept row of A u is zero to rounding. A swap
    of component indices anywhere in the blocks or the scatter breaks this."""
    from oracle import oracle
    m = square_mesh(8, 0.1, jitter=0.15, seed=3)
    k = {"function": "linearPrototypeMicroelasticField", "horizon": 0.1, "outputdim": 2, "fractional_s": -0.5}
    r = oracle.assemble(m, k, conf2d(rule="16", close="fractional", deg=3))
    A = r["A"]
    assert r["n_close"] > 0 and not np.isnan(A.data).any()
    V = m["vertices"]
    keep = _kept_rows(m, 2)
    for u in (np.tile([1.0, 0.0], V.shape[0]), np.tile([0.0, 1.0], V.shape[0]),
              np.stack([-V[:, 1], V[:, 0]], axis=1).ravel()):
        assert np.abs(A @ u)[keep].max() <= 1e-12 * abs(A).max() * np.abs(u).max()
    stretch = np.stack([V[:, 0], np.zeros(V.shape[0])], axis=1).ravel()   # not a rigid motion
    assert np.abs(A @ stretch)[keep].max() > 1e-3 * abs(A).max() * 0.01


def test_oracle_microelastic_field_3d_annihilates_rigid_motions():
    """kernelField_linearPrototypeMicroelastic3D (model.cpp:155-178) with the barycenter rule in
    3D: the three translations and three rotations are annihilated on the kept rows."""
    from oracle import oracle
    m = cube_mesh(3, 0.1, jitter=0.1, seed=4)
    k = {"function": "linearPrototypeMicroelasticField3D", "horizon": 0.35, "outputdim": 3}
    # the kernel is singular at x = y and has no close rule: with the same rule inside and out the
    # self pairs meet x = y (NaN, in the reference too), so the inner rule is the 4-point one
    pa, pb = 0.5854101966249685, 0.1381966011250105
    conf = conf3d()
    conf["quadrature"]["inner"] = {"points": np.array([[pb, pb, pb], [pa, pb, pb], [pb, pa, pb], [pb, pb, pa]]),
                                   "weights": np.full(4, 1.0 / 24)}
    A = oracle.assemble(m, k, conf)["A"]
    assert not np.isnan(A.data).any()
    V = m["vertices"]
    n = V.shape[0]
    keep = _kept_rows(m, 3)
    motions = [np.tile(e, n) for e in np.eye(3)]
    for w in np.eye(3):
        motions.append(np.cross(w, V).ravel())
    for u in motions:
        assert np.abs(A @ u)[keep].max() <= 1e-12 * abs(A).max() * np.abs(u).max()


def _forcing_numpy(m, conf, fun, od):
    """compute_f (Cassemble.cpp:149-164) written in numpy: sum_k psi_a(P_k) f(x_k) |det| dx_k."""
    q = conf["quadrature"]["outer"]
    P, w = np.asarray(q["points"]), np.asarray(q["weights"])
    psi = np.column_stack([1 - P.sum(axis=1), P])
    V, T = m["vertices"], m["elements"]
    f = np.zeros(V.shape[0] * od)
    for e, t in enumerate(T):
        if m["elementLabels"][e] <= 0:
            continue
        E = V[t]
        det = abs(np.linalg.det(np.column_stack([E[1] - E[0], E[2] - E[0]])))
        x = E[0] + P @ np.vstack([E[1] - E[0], E[2] - E[0]])
        fx = np.atleast_2d(fun(x.T)).reshape(od, -1)
        for a in range(3):
            if m["vertexLabels"][t[a]] > 0:
                for c in range(od):
                    f[od * t[a] + c] += np.sum(psi[:, a] * fx[c] * w) * det
    return f


@pytest.mark.parametrize("name,od,fun", [
    ("gaussian", 1, lambda x: -4. * (x[0] ** 2 + x[1] ** 2 - 1.) * np.exp(-x[0] ** 2 - x[1] ** 2)),
    ("jump", 1, lambda x: np.where(x[0] + x[1] - 0.5 > -1e-15, -4., 4.)),
    ("tensorsin", 1, lambda x: 32. * np.pi ** 2 * np.sin(x[0] * np.pi * 4) * np.sin(x[1] * np.pi * 4)),
    ("linearField", 2, lambda x: np.array([-np.pi / 2 * (1.0 + 2 * x[0]), -np.pi / 2 * x[1]])),
    ("constantRightField", 2, lambda x: np.array([np.full_like(x[0], 0.1), np.zeros_like(x[0])])),
    ("constantDownField", 2, lambda x: np.array([np.zeros_like(x[0]), np.full_like(x[0], -2 * np.pi)])),
    ("constantBothField", 2, lambda x: np.array([np.full_like(x[0], -np.pi), np.full_like(x[0], -2 * np.pi)])),
])
def test_oracle_forcings(name, od, fun):
    """The forcing terms of model.cpp:201-255 in the oracle's par_forcing against compute_f in
    numpy."""
    from oracle import oracle
    m = square_mesh(10, 0.1, jitter=0.2, seed=8)
    m["outdim"] = od
    f = oracle.assemble(m, None, conf2d(), compute="forcing", load={"function": name})["f"]
    g = _forcing_numpy(m, conf2d(), fun, od)
    assert f.shape == g.shape
    np.testing.assert_allclose(f, g, rtol=1e-12, atol=1e-13 * np.abs(g).max())


def test_oracle_exact_ball_integrates_the_ball_exactly():
    """exactBall (integrate_exact / method_exact / placePointCapCenter, integration.cpp:706-907,
    1300-1351, 1632-1761): the caps-free polygons plus each circular segment at its exact area.
    With the constant kernel c, an outer point whose ball lies inside the mesh sees
    sum over bT of the inner integral = c pi delta^2, so the termLocal blocks of an interior
    element summed over all partners are 2 c pi delta^2 |aT| sum_k dx_k psi_a psi_b. The
    retriangulate rule's cap points only approximate the arcs."""
    from oracle import oracle
    m = square_mesh(16, 0.1, jitter=0.15, seed=7)
    V, T = m["vertices"], m["elements"]
    aT = int(np.argmin(np.linalg.norm(V[T].mean(axis=1) - 0.5, axis=1)))
    pairs = np.array([(aT, b) for b in range(T.shape[0])])
    k = {"function": "constant", "horizon": 0.1, "outputdim": 1}
    conf = conf2d()
    P = np.asarray(conf["quadrature"]["outer"]["points"]); w = np.asarray(conf["quadrature"]["outer"]["weights"])
    psi = np.column_stack([1 - P.sum(axis=1), P])
    E = V[T[aT]]
    det = abs(np.linalg.det(np.column_stack([E[1] - E[0], E[2] - E[0]])))
    c = 4 / (np.pi * 0.1 ** 4)
    want = 2 * c * np.pi * 0.1 ** 2 * det * (psi.T * w) @ psi
    got = oracle.pair_blocks(m, k, conf, pairs, method="exactBall")[0][:, 0].sum(axis=0)
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
    retri = oracle.pair_blocks(m, k, conf, pairs, method="retriangulate")[0][:, 0].sum(axis=0)
    assert np.abs(retri - want / 2).max() > 1e-6 * np.abs(want).max()   # weight 1 there
    # assembled: the one-sided rule's rows still sum to zero
    r = oracle.assemble(m, k, conf2d(method="exactBall"))
    A = r["A"]
    keep = m["vertexLabels"] > 0
    assert r["n_errors"] == 0 and np.abs(A @ np.ones(A.shape[0]))[keep].max() < 1e-12 * abs(A).max()


@pytest.mark.parametrize("method,weight", [("retriangulateLinfty", 1.0), ("retriangulate_unsymmLinfty", 2.0)])
def test_oracle_linf_ball_area(method, weight):
    """The L-infinity ball (method_retriangulateInfty, integration.cpp:1521-1623; the reference
    triangulates the points with CGAL, here the convex hull is fanned) and kernel_constantLinf2D
    (model.cpp:30-33): for an interior element the square of half side delta is covered exactly,
    so the termLocal blocks summed over all partners are weight c 4 delta^2 |aT| sum_k dx psi psi."""
    from oracle import oracle
    m = square_mesh(16, 0.1, jitter=0.15, seed=7)
    V, T = m["vertices"], m["elements"]
    aT = int(np.argmin(np.linalg.norm(V[T].mean(axis=1) - 0.5, axis=1)))
    pairs = np.array([(aT, b) for b in range(T.shape[0])])
    k = {"function": "constantLinf2D", "horizon": 0.1, "outputdim": 1}
    conf = conf2d()
    P = np.asarray(conf["quadrature"]["outer"]["points"]); w = np.asarray(conf["quadrature"]["outer"]["weights"])
    psi = np.column_stack([1 - P.sum(axis=1), P])
    E = V[T[aT]]
    det = abs(np.linalg.det(np.column_stack([E[1] - E[0], E[2] - E[0]])))
    c = 3 / (4 * 0.1 ** 4)
    want = weight * c * 4 * 0.1 ** 2 * det * (psi.T * w) @ psi
    got = oracle.pair_blocks(m, k, conf, pairs, method=method)[0][:, 0].sum(axis=0)
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
    r = oracle.assemble(m, k, conf2d(method=method))
    A = r["A"]
    keep = m["vertexLabels"] > 0
    assert r["n_errors"] == 0 and np.abs(A @ np.ones(A.shape[0]))[keep].max() < 1e-12 * abs(A).max()


def test_oracle_weak_and_fractional_rules_agree_for_the_field_kernel():
    """outdim 2: the weakSingular close rule (integration.cpp:82-185, component loops) and the
    fractional one assemble the same matrix for the weakly singular microelastic field kernel
    (|z|^-1 homogeneous, s = -1/2), as in the scalar case."""
    from oracle import oracle
    m = square_mesh(8, 0.1, jitter=0.15, seed=3)
    k = {"function": "linearPrototypeMicroelasticField", "horizon": 0.1, "outputdim": 2, "fractional_s": -0.5}
    W = oracle.assemble(m, k, conf2d(rule="16", close="weakSingular", deg=3))
    F = oracle.assemble(m, k, conf2d(rule="16", close="fractional", deg=3))
    assert W["n_close"] == F["n_close"] > 0 and W["n_errors"] == 0
    assert abs(W["A"] - F["A"]).max() <= 1e-13 * abs(F["A"]).max()


def test_oracle_dg_sums_to_cg_with_close_pairs():
    """DG with a singular kernel and the fractional close rule: summed over the vertex copies,
    the DG matrix is the CG matrix on the kept rows (the close-pair blocks scatter to element
    DOFs like the others)."""
    from oracle import oracle
    m = square_mesh(8, 0.2, jitter=0.1, seed=5)
    k = {"function": "fractional", "horizon": 0.2, "outputdim": 1, "fractional_s": 0.4}
    cdg = conf2d(rule="16", close="fractional", deg=3)
    cdg["ansatz"] = "DG"
    D = oracle.assemble(m, k, cdg)
    C = oracle.assemble(m, k, conf2d(rule="16", close="fractional", deg=3))
    assert D["n_close"] == C["n_close"] > 0
    T = m["elements"]; nE, nV = T.shape[0], m["vertices"].shape[0]
    P = sp.csr_matrix((np.ones(3 * nE), (np.arange(3 * nE), T.ravel())), shape=(3 * nE, nV))
    S = (P.T @ D["A"] @ P).toarray()
    S[m["vertexLabels"] <= 0] = 0
    assert np.abs(S - C["A"].toarray()).max() <= 1e-11 * abs(C["A"]).max()
