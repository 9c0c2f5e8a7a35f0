"""GPU parity against the oracle: bit-exact sparsity pattern and pair set, FP64 values within
rounding, deterministic runs. All calls go through the C ABI (libnlfem_gpu.so)."""
import ctypes

import numpy as np
import pytest
import scipy.sparse as sp

from conftest import conf2d, conf3d, square_mesh, cube_mesh, labeled_mesh, rel_errors, same_pattern

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12   # relative Frobenius / max-entry error of the FP64 path (summation order only)


@pytest.fixture(scope="module")
def nl():
    from nlfem_gb300 import nlfem, _lib
    lib = _lib.load()
    if lib.nlfem_device_count() == 0:
        pytest.fail("no CUDA device visible: the GPU library cannot run")
    return nlfem


@pytest.fixture(scope="module")
def orc():
    from oracle import oracle
    return oracle


def _cases_retri(rng, n):
    out = []
    for i in range(n):
        T = rng.uniform(-1, 1, 6)
        delta = rng.uniform(0.05, 1.5)
        mode = i % 4
        if mode == 0:
            x = rng.uniform(-1.5, 1.5, 2)
        elif mode == 1:   # center near a vertex
            k = rng.integers(3)
            x = T[2 * k: 2 * k + 2] + rng.normal(0, 1e-3, 2)
        elif mode == 2:   # ball tangent-ish to an edge
            k = rng.integers(3)
            p, q = T[2 * k: 2 * k + 2], T[(2 * k + 2) % 6: (2 * k + 2) % 6 + 2]
            m = 0.5 * (p + q)
            nrm = np.array([q[1] - p[1], p[0] - q[0]])
            nrm /= np.linalg.norm(nrm)
            x = m + nrm * delta * (1 + rng.normal(0, 1e-9))
        else:            # vertex exactly on the sphere
            k = rng.integers(3)
            ang = rng.uniform(0, 2 * np.pi)
            x = T[2 * k: 2 * k + 2] + delta * np.array([np.cos(ang), np.sin(ang)])
        out.append((x, T, delta * delta, int(rng.integers(2))))
    return out


def test_retriangulate_bitexact(nl, orc):
    rng = np.random.Generator(np.random.PCG64(7))
    cases = _cases_retri(rng, 4000)
    for caps in (0, 1):
        sub = [c for c in cases if c[3] == caps]
        X = np.array([c[0] for c in sub]); T = np.array([c[1] for c in sub])
        sq = np.array([c[2] for c in sub])
        for j in range(len(sub)):
            cnt, out = nl.retriangulate_batch(X[j:j + 1], T[j:j + 1], sq[j], caps)
            n, tri = orc.retriangulate_sq(X[j], T[j], sq[j], caps)
            assert cnt[0] == n
            np.testing.assert_array_equal(out[0, :n], tri)


def test_debug_hooks(nl, orc):
    T = np.array([0.1, 0.2, 0.9, 0.1, 0.3, 0.8])
    x = np.array([0.4, 0.35])
    p = nl.py_toRef(T, x)
    np.testing.assert_allclose(nl.py_toPhys(T, p), x, rtol=0, atol=1e-15)
    A = np.array([2.0, 1.0, 1.0, 3.0]); b = np.array([1.0, 2.0])
    np.testing.assert_allclose(nl.py_solve2x2(A, b), np.linalg.solve(A.reshape(2, 2), b), rtol=1e-15)
    n, lst = nl.py_retriangulate(np.array([0.3, 0.3]), T, 0.2, 1)
    m, tri = orc.retriangulate(np.array([0.3, 0.3]), T, 0.2, 1)
    assert n == m
    np.testing.assert_array_equal(lst[: 6 * n], tri.ravel())


KC = {"function": "constant", "horizon": 0.1, "outputdim": 1}


def test_pair_list_config1(nl, orc):
    m = square_mesh(32, 0.1)
    ref = orc.assemble(m, KC, conf2d(), want_pairs=True)
    got = nl.pair_list(m, KC, conf2d())
    rp = ref["pairs"][np.lexsort((ref["pairs"][:, 1], ref["pairs"][:, 0]))]
    np.testing.assert_array_equal(got, rp)


def test_config1_constant_fp64(nl, orc):
    m = square_mesh(32, 0.1)
    A = nl.stiffnessMatrix(m, KC, conf2d())
    B = orc.assemble(m, KC, conf2d())["A"]
    assert same_pattern(A, B)
    fro, mx = rel_errors(A, B)
    assert fro < FP64_TOL and mx < FP64_TOL, (fro, mx)


def test_jittered_parabola_fp64(nl, orc):
    m = square_mesh(20, 0.15, jitter=0.2, seed=4)
    k = {"function": "parabola", "horizon": 0.15, "outputdim": 1}
    A = nl.stiffnessMatrix(m, k, conf2d())
    B = orc.assemble(m, k, conf2d())["A"]
    assert same_pattern(A, B)
    fro, mx = rel_errors(A, B)
    assert fro < FP64_TOL and mx < FP64_TOL, (fro, mx)


def test_no_caps_and_full_search(nl, orc):
    m = square_mesh(8, 0.1, jitter=0.1, seed=2)
    c = conf2d(caps=0)
    A = nl.stiffnessMatrix(m, KC, c); B = orc.assemble(m, KC, c)["A"]
    assert same_pattern(A, B) and rel_errors(A, B)[0] < FP64_TOL
    c = conf2d(); c["is_fullConnectedComponentSearch"] = 1
    A = nl.stiffnessMatrix(m, KC, c); B = orc.assemble(m, KC, c)["A"]
    assert same_pattern(A, B) and rel_errors(A, B)[0] < FP64_TOL


def test_label_zero_bridges(nl, orc):
    m = square_mesh(14, 0.1, jitter=0.1, seed=5)
    lab = m["elementLabels"].copy()
    lab[40:60] = 0
    from nlfem_gb300.meshes import mesh_dict
    m2 = mesh_dict(m["vertices"], m["elements"], lab)
    A = nl.stiffnessMatrix(m2, KC, conf2d()); B = orc.assemble(m2, KC, conf2d())["A"]
    assert same_pattern(A, B) and rel_errors(A, B)[0] < FP64_TOL


@pytest.mark.parametrize("kern", ["constant", "parabola"])
def test_label_zero_bridges_mixed(nl, orc, kern):
    """Mixed path on a mesh with label-0 elements (searched through, never paired), with the
    constant kernel's closed forms and the general kernel."""
    m = square_mesh(16, 0.12, jitter=0.2, seed=7)
    lab = m["elementLabels"].copy()
    lab[60:90] = 0
    from nlfem_gb300.meshes import mesh_dict
    m2 = mesh_dict(m["vertices"], m["elements"], lab)
    k = {"function": kern, "horizon": 0.12, "outputdim": 1}
    A = nl.stiffnessMatrix(m2, k, conf2d(precision="mixed")); B = orc.assemble(m2, k, conf2d())["A"]
    assert same_pattern(A, B)
    fro, mx = rel_errors(A, B)
    assert fro < MIX_TOL and mx < MIX_TOL, (fro, mx)


def test_mixed_no_caps(nl, orc):
    m = square_mesh(18, 0.1, jitter=0.2, seed=11)
    A = nl.stiffnessMatrix(m, KC, conf2d(caps=0, precision="mixed")); B = orc.assemble(m, KC, conf2d(caps=0))["A"]
    assert same_pattern(A, B)
    fro, mx = rel_errors(A, B)
    assert fro < MIX_TOL and mx < MIX_TOL, (fro, mx)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_domain_decomposition_weights(nl, orc, prec):
    """Domain decomposition (Cassemble.cpp:649-657): every pair's blocks weighted by 1 / the number
    of subdomains its elements share. Two subdomains overlap in a strip wider than the ball, so
    every interacting pair shares one; the first 20 elements lie in both (chk_Mesh, checks.cpp:74-84,
    requires them to share one pairwise)."""
    m = square_mesh(14, 0.1, jitter=0.1, seed=8)
    x = m["vertices"][m["elements"]].mean(axis=1)[:, 0]
    rows = [[0, 1] if e < 20 else ([0] if xi < 0.3 else ([1] if xi > 0.7 else [0, 1])) for e, xi in enumerate(x)]
    indptr = np.cumsum([0] + [len(r) for r in rows])
    Z = sp.csr_matrix((np.ones(indptr[-1]), np.concatenate(rows), indptr), shape=(len(rows), 2))
    m["nZeta"] = 2
    m["ZetaIndicator"] = Z
    A = nl.stiffnessMatrix(m, KC, conf2d(precision=prec))
    B = orc.assemble(m, KC, conf2d())["A"]
    assert same_pattern(A, B)
    fro, mx = rel_errors(A, B)
    tol = FP64_TOL if prec == "fp64" else MIX_TOL
    assert fro < tol and mx < tol, (fro, mx)
    m0 = dict(m)
    m0["nZeta"] = 0
    B0 = orc.assemble(m0, KC, conf2d())["A"]
    assert abs(B - B0).max() > 1e-3 * abs(B0).max()   # the weights change the matrix


def test_pair_blocks_match_oracle(nl, orc):
    m = square_mesh(16, 0.1, jitter=0.2, seed=9)
    k = {"function": "parabola", "horizon": 0.1, "outputdim": 1}
    pairs = orc.assemble(m, k, conf2d(), want_pairs=True)["pairs"]
    rng = np.random.Generator(np.random.PCG64(3))
    sel = pairs[rng.choice(len(pairs), 500, replace=False)]
    g, gr = nl.pair_blocks(m, k, conf2d(), sel)
    o, orr = orc.pair_blocks(m, k, conf2d(), sel)
    np.testing.assert_array_equal(gr != 0, orr != 0)
    np.testing.assert_allclose(g, o, rtol=1e-12, atol=1e-12 * np.abs(o).max())


LABEL_KERNELS = ["labeled", "notch", "labeledNotch", "labeledValve", "constantTruncated"]


_labeled_mesh = labeled_mesh


@pytest.mark.parametrize("name,method", [(k, "retriangulate") for k in LABEL_KERNELS] + [("labeledValve", "baryCenter"), ("notch", "baryCenter")])
def test_label_kernels_fp64(nl, orc, name, method):
    """Label- and position-dependent kernels (model.cpp:30-42, 67-114) on the FP64 path."""
    m = _labeled_mesh()
    k = {"function": name, "horizon": 0.1, "outputdim": 1}
    A = nl.stiffnessMatrix(m, k, conf2d(method=method))
    B = orc.assemble(m, k, conf2d(method=method))["A"]
    assert same_pattern(A, B)
    fro, mx = rel_errors(A, B)
    assert fro < FP64_TOL and mx < FP64_TOL, (fro, mx)
    if name != "constantTruncated":   # the kernel matters: not the constant kernel's matrix
        C = orc.assemble(m, KC, conf2d(method=method))["A"]
        assert abs(B - C).max() > 1e-3 * abs(C).max()


def test_label_kernel_pair_blocks(nl, orc):
    m = _labeled_mesh(10, 6)
    k = {"function": "labeled", "horizon": 0.1, "outputdim": 1}
    pairs = orc.assemble(m, k, conf2d(), want_pairs=True)["pairs"]
    g, gr = nl.pair_blocks(m, k, conf2d(), pairs)
    o, orr = orc.pair_blocks(m, k, conf2d(), pairs)
    np.testing.assert_array_equal(gr != 0, orr != 0)
    np.testing.assert_allclose(g, o, rtol=1e-12, atol=1e-12 * np.abs(o).max())


def test_label_kernel_errors(nl):
    from nlfem_gb300._lib import NlfemError
    k = {"function": "labeled", "horizon": 0.1, "outputdim": 1}
    m = square_mesh(8, 0.1, jitter=0.1, seed=1)
    m["elementLabels"] = np.where(m["elementLabels"] > 0, 2, -1)   # 10 * 2 - 1 = 19: the reference aborts
    with pytest.raises(NlfemError, match="outside its domain"):
        nl.stiffnessMatrix(m, k, conf2d())
    with pytest.raises(NlfemError, match="fp64 path only"):
        nl.stiffnessMatrix(_labeled_mesh(8), k, conf2d(precision="mixed"))
    # the session still works after the error
    m = _labeled_mesh(8)
    assert nl.stiffnessMatrix(m, k, conf2d()).nnz > 0


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_tangent_sphere_polygons(nl, orc, prec):
    """Unjittered grid with h = 0.15 and delta = 0.1: element centroids lie at distance delta from
    grid lines, the sphere touches edges up to rounding, and some polygons would need more than 9
    points. Both sides keep the first 9."""
    m = square_mesh(8, 0.1)
    A = nl.stiffnessMatrix(m, KC, conf2d(precision=prec))
    B = orc.assemble(m, KC, conf2d())["A"]
    assert same_pattern(A, B)
    fro, mx = rel_errors(A, B)
    tol = FP64_TOL if prec == "fp64" else 1e-6
    assert fro < tol and mx < tol, (fro, mx)


FURTHER_RULES = ["retriangulate_unsymm", "subSetBall", "averageBall", "baryCenterRT", "noTruncation"]


@pytest.mark.parametrize("method", FURTHER_RULES)
def test_further_rules_fp64(nl, orc, method):
    """retriangulate_unsymm, subSetBall, averageBall, baryCenterRT and noTruncation
    (integration.cpp:290-343, 542-704, 1021-1095, 1155-1249) on the FP64 path: assembled
    matrices, and the blocks and interaction flags of single pairs."""
    n = 6 if method == "noTruncation" else 14   # noTruncation pairs every element with every other
    m = square_mesh(n, 0.1, jitter=0.15, seed=12)
    conf = conf2d(method=method)
    for name in ("constant", "parabola"):
        k = {"function": name, "horizon": 0.1, "outputdim": 1}
        A = nl.stiffnessMatrix(m, k, conf)
        r = orc.assemble(m, k, conf, want_pairs=True)
        B = r["A"]
        assert same_pattern(A, B)
        fro, mx = rel_errors(A, B)
        assert fro < FP64_TOL and mx < FP64_TOL, (name, fro, mx)
    rng = np.random.Generator(np.random.PCG64(5))
    sel = r["pairs"][rng.choice(len(r["pairs"]), min(400, len(r["pairs"])), replace=False)]
    g, gr = nl.pair_blocks(m, k, conf, sel)
    o, orr = orc.pair_blocks(m, k, conf, sel)
    np.testing.assert_array_equal(gr != 0, orr != 0)
    np.testing.assert_allclose(g, o, rtol=1e-12, atol=1e-12 * np.abs(o).max())


def test_further_rules_with_label_kernel(nl, orc):
    m = _labeled_mesh(12, 7)
    k = {"function": "labeledValve", "horizon": 0.1, "outputdim": 1}
    for method in ("retriangulate_unsymm", "averageBall", "baryCenterRT"):
        A = nl.stiffnessMatrix(m, k, conf2d(method=method))
        B = orc.assemble(m, k, conf2d(method=method))["A"]
        assert same_pattern(A, B)
        fro, mx = rel_errors(A, B)
        assert fro < FP64_TOL and mx < FP64_TOL, (method, fro, mx)


def test_further_rules_mixed_precision_refused(nl):
    from nlfem_gb300._lib import NlfemError
    with pytest.raises(NlfemError, match="fp64 path only"):
        nl.stiffnessMatrix(square_mesh(6, 0.1), KC, conf2d(method="subSetBall", precision="mixed"))


def _conf_dg(method="retriangulate", precision="fp64"):
    c = conf2d(method=method, precision=precision)
    c["ansatz"] = "DG"
    return c


@pytest.mark.parametrize("kname,method", [("constant", "retriangulate"), ("parabola", "retriangulate"),
                                          ("constant", "baryCenter"), ("labeledValve", "retriangulate"),
                                          ("constant", "averageBall")])
def test_dg_matches_oracle(nl, orc, kname, method):
    """The DG ansatz (element DOFs dV e + a, every row kept; Cassemble.cpp:580-585, 637-642) on
    the FP64 path, and its sum over vertex copies against the CG assembly."""
    m = _labeled_mesh(10, 14) if kname.startswith("labeled") else square_mesh(10, 0.1, jitter=0.15, seed=14)
    k = {"function": kname, "horizon": 0.1, "outputdim": 1}
    A = nl.stiffnessMatrix(dict(m), k, _conf_dg(method))
    B = orc.assemble(m, k, _conf_dg(method))["A"]
    nE, nV = m["elements"].shape[0], m["vertices"].shape[0]
    assert A.shape == (3 * nE, 3 * nE)
    assert same_pattern(A, B)
    fro, mx = rel_errors(A, B)
    assert fro < FP64_TOL and mx < FP64_TOL, (fro, mx)
    C = nl.stiffnessMatrix(dict(m), k, conf2d(method=method))
    P = sp.csr_matrix((np.ones(3 * nE), (np.arange(3 * nE), m["elements"].ravel())), shape=(3 * nE, nV))
    S = (P.T @ A @ P).toarray()
    S[m["vertexLabels"] <= 0] = 0
    assert np.abs(S - C.toarray()).max() <= 1e-12 * abs(C).max()


@pytest.mark.parametrize("close,kname", [("weakSingular", "fractional"), ("weakSingular", "linearPrototypeMicroelastic")])
def test_dg_singular_kernels(nl, orc, close, kname):
    """DG with a singular kernel: the close pairs (sharing a vertex) take the weakSingular Duffy rule
    (the reference refuses the fractional rule for DG, checks.cpp:105-107), found on the vertex
    table while the rows are element DOFs (Cassemble.cpp:580-585, integration.cpp:82-185); against
    the oracle, and summed over the vertex copies against the CG assembly."""
    m = square_mesh(8, 0.2, jitter=0.1, seed=16)
    s = 0.4 if kname == "fractional" else -0.5
    k = {"function": kname, "horizon": 0.2, "outputdim": 1, "fractional_s": s}
    c = _conf_dg()
    c["closeElements"] = close
    c["quadrature"]["tensorGaussDegree"] = 3
    A = nl.stiffnessMatrix(dict(m), k, c)
    B = orc.assemble(m, k, c)["A"]
    nE, nV = m["elements"].shape[0], m["vertices"].shape[0]
    assert A.shape == (3 * nE, 3 * nE)
    assert same_pattern(A, B)
    fro, mx = rel_errors(A, B)
    assert fro < 1e-11 and mx < 1e-11, (fro, mx)
    cc = dict(c, ansatz="CG")
    C = nl.stiffnessMatrix(dict(m), k, cc)
    P = sp.csr_matrix((np.ones(3 * nE), (np.arange(3 * nE), m["elements"].ravel())), shape=(3 * nE, nV))
    S = (P.T @ A @ P).toarray()
    S[m["vertexLabels"] <= 0] = 0
    assert np.abs(S - C.toarray()).max() <= 1e-11 * abs(C).max()


def test_dg_load_vector(nl, orc):
    m = square_mesh(12, 0.1, jitter=0.2, seed=15)
    f = nl.loadVector(dict(m), {"function": "linear"}, _conf_dg())
    g = orc.assemble(m, None, _conf_dg(), compute="forcing", load={"function": "linear"})["f"]
    assert f.shape == (3 * m["elements"].shape[0],)
    np.testing.assert_allclose(f, g, rtol=1e-13, atol=1e-15 * np.abs(g).max())


def test_dg_session_reassembly_and_cache(nl, orc):
    """A DG session assembles again on its mesh (the row space goes back to the vertices for the
    pair search), and a CG call after a DG call on the same sizes is unchanged."""
    m = square_mesh(10, 0.1, jitter=0.1, seed=16)
    C0 = nl.stiffnessMatrix(dict(m), KC, conf2d())
    s = nl.Session([(dict(m), KC, _conf_dg())])
    s.assemble()
    A1 = s.download(0)
    s.assemble()
    A2 = s.download(0)
    assert same_pattern(A1, A2) and np.array_equal(A1.data, A2.data)
    B = orc.assemble(m, KC, _conf_dg())["A"]
    fro, mx = rel_errors(A1, B)
    assert fro < FP64_TOL and mx < FP64_TOL
    nl.stiffnessMatrix(dict(m), KC, _conf_dg())
    C1 = nl.stiffnessMatrix(dict(m), KC, conf2d())
    assert same_pattern(C0, C1) and np.array_equal(C0.data, C1.data)
    with pytest.raises(Exception, match="CG sessions only"):
        s.solve(0, np.zeros(m["vertices"].shape[0]), np.zeros(m["vertices"].shape[0]))


def test_dg_refusals(nl):
    from nlfem_gb300._lib import NlfemError
    m = square_mesh(6, 0.1)
    with pytest.raises(NlfemError, match="fp64 path only"):
        nl.stiffnessMatrix(dict(m), KC, _conf_dg(precision="mixed"))
    with pytest.raises(NlfemError, match="one at a time"):
        nl.stiffnessMatrix_batch([(dict(m), KC, _conf_dg()), (dict(m), KC, _conf_dg())])


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_linear_prototype_kernel(nl, orc, prec):
    """linearPrototypeMicroelastic (model.cpp:116-124), singular (Cassemble.cpp:89-94), with the
    fractional close-pair rule: the oracle's values, and bit for bit the fractional kernel at
    s = -1/2, whose formula it is."""
    m = square_mesh(10, 0.1, jitter=0.15, seed=9)
    kp = {"function": "linearPrototypeMicroelastic", "horizon": 0.1, "outputdim": 1, "fractional_s": -0.5}
    kf = {"function": "fractional", "horizon": 0.1, "outputdim": 1, "fractional_s": -0.5}
    A = nl.stiffnessMatrix(dict(m), kp, conf2d(rule="16", close="fractional", deg=3, precision=prec))
    B = orc.assemble(m, kp, conf2d(rule="16", close="fractional", deg=3))["A"]
    assert same_pattern(A, B)
    fro, mx = rel_errors(A, B)
    tol = FP64_TOL if prec == "fp64" else MIX_TOL
    assert fro < tol and mx < tol, (fro, mx)
    F = nl.stiffnessMatrix(dict(m), kf, conf2d(rule="16", close="fractional", deg=3, precision=prec))
    assert same_pattern(A, F) and np.array_equal(A.data, F.data)


def test_weak_singular_close_rule(nl, orc):
    """The weakSingular close rule (integration.cpp:82-185) with the weakly singular kernel
    linearPrototypeMicroelastic: the oracle's matrix and close-pair blocks, and the matrix of the
    fractional close rule, which for this kernel is the same sum."""
    from nlfem_gb300._lib import NlfemError
    m = square_mesh(10, 0.1, jitter=0.15, seed=9)
    kp = {"function": "linearPrototypeMicroelastic", "horizon": 0.1, "outputdim": 1, "fractional_s": -0.5}
    cw = conf2d(rule="16", close="weakSingular", deg=3)
    A = nl.stiffnessMatrix(dict(m), kp, cw)
    B = orc.assemble(m, kp, cw)["A"]
    assert same_pattern(A, B)
    fro, mx = rel_errors(A, B)
    assert fro < FP64_TOL and mx < FP64_TOL, (fro, mx)
    F = nl.stiffnessMatrix(dict(m), kp, conf2d(rule="16", close="fractional", deg=3))
    assert abs(A - F).max() <= 1e-12 * abs(F).max()
    T = m["elements"]
    pairs = [(e, f) for e in (3, 40, 77) for f in range(T.shape[0]) if set(T[e]) & set(T[f])]
    g, _ = nl.pair_blocks(m, kp, cw, np.array(pairs), close=True)
    o, _ = orc.pair_blocks(m, kp, cw, np.array(pairs), method="weakSingular")
    np.testing.assert_allclose(g, o, rtol=1e-12, atol=1e-12 * np.abs(o).max())
    # the mixed path: FP32 Duffy rule (weakSingular form) for the close pairs, within the mixed bound
    Am = nl.stiffnessMatrix(dict(m), kp, conf2d(rule="16", close="weakSingular", deg=3, precision="mixed"))
    assert same_pattern(Am, B)
    fro, mx = rel_errors(Am, B)
    assert fro < MIX_TOL and mx < MIX_TOL, (fro, mx)
    with pytest.raises(NlfemError, match="fractional close rule only"):
        nl.stiffnessMatrix(dict(m), kp, conf2d(rule="16", close="weakSingular", deg=3, precision="fp64-onesided"))


@pytest.mark.parametrize("name", ["config1", "tangent", "parabola20", "frac12", "cube5", "labeled10", "average10",
                                  "exact8", "dg10", "weak10", "field8"])
def test_gpu_matches_committed_fixtures(nl, name):
    """The FP64 path against the committed oracle fixtures (tests/golden/oracle_cases.npz, made by
    tests/golden/make_oracle_golden.py): bit-exact pattern, values within rounding."""
    import importlib.util
    import os
    gdir = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    spec = importlib.util.spec_from_file_location("make_oracle_golden", os.path.join(gdir, "make_oracle_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    fx = np.load(os.path.join(gdir, "oracle_cases.npz"))
    _, kernel, conf, load = mg.cases()[name]
    # the stored mesh: the fixture's own inputs, whatever numpy this host runs
    mesh = {k: fx[f"{name}.{k}"] for k in ("elements", "elementLabels", "vertices", "vertexLabels")}
    indptr = fx[f"{name}.indptr"]
    K = indptr.size - 1
    B = sp.csr_matrix((fx[f"{name}.data"], fx[f"{name}.indices"], indptr), shape=(K, K))
    A = nl.stiffnessMatrix(dict(mesh), kernel, conf)
    assert same_pattern(A, B)
    fro, mx = rel_errors(A, B)
    tol = 1e-11 if name == "frac12" else FP64_TOL
    assert fro < tol and mx < tol, (fro, mx)
    if load is not None:
        f = nl.loadVector(dict(mesh, outdim=int(kernel.get("outputdim", 1))), load, conf)
        g = fx[f"{name}.f"]
        np.testing.assert_allclose(f, g, rtol=1e-13, atol=1e-15 * np.abs(g).max())


def test_load_vector(nl, orc):
    m = square_mesh(24, 0.1, jitter=0.2, seed=8)
    f = nl.loadVector(m, {"function": "linear"}, conf2d())
    g = orc.assemble(m, None, conf2d(), compute="forcing", load={"function": "linear"})["f"]
    np.testing.assert_allclose(f, g, rtol=1e-13, atol=1e-15 * np.abs(g).max())


def test_fractional_close_pairs(nl, orc):
    m = square_mesh(12, 0.2)
    k = {"function": "fractional", "horizon": 0.2, "outputdim": 1, "fractional_s": 0.4}
    c = conf2d(rule="16", close="fractional", deg=3)
    A = nl.stiffnessMatrix(m, k, c)
    B = orc.assemble(m, k, c)["A"]
    assert same_pattern(A, B)
    fro, mx = rel_errors(A, B)
    assert fro < 1e-11 and mx < 1e-11, (fro, mx)


def test_fractional_close_blocks(nl, orc):
    m = square_mesh(6, 0.2, jitter=0.2, seed=1)
    k = {"function": "fractional", "horizon": 0.2, "outputdim": 1, "fractional_s": 0.4}
    c = conf2d(rule="16", close="fractional", deg=4)
    e = m["elements"]
    pairs = [(i, i) for i in range(0, 60, 7)]
    for a in range(0, 60, 5):
        for b in range(e.shape[0]):
            if a != b and len(set(e[a]) & set(e[b])) in (1, 2):
                pairs.append((a, b))
    pairs = np.array(pairs)
    g, _ = nl.pair_blocks(m, k, c, pairs, close=True)
    o, _ = orc.pair_blocks(m, k, c, pairs, method="fractional")
    np.testing.assert_allclose(g, o, rtol=1e-11, atol=1e-12 * np.abs(o).max())


def test_3d_barycenter(nl, orc):
    m = cube_mesh(5, 0.1, jitter=0.15, seed=2)
    k = {"function": "constant3D", "horizon": 0.3, "outputdim": 1}
    A = nl.stiffnessMatrix(m, k, conf3d())
    B = orc.assemble(m, k, conf3d())["A"]
    assert same_pattern(A, B)
    fro, mx = rel_errors(A, B)
    assert fro < FP64_TOL and mx < FP64_TOL, (fro, mx)
    f = nl.loadVector(m, {"function": "linear3D"}, conf3d())
    g = orc.assemble(m, None, conf3d(), compute="forcing", load={"function": "linear3D"})["f"]
    np.testing.assert_allclose(f, g, rtol=1e-13, atol=1e-15 * np.abs(g).max())


def test_batch_equals_single(nl):
    probs = []
    for i, (n, d, kn) in enumerate([(10, 0.1, "constant"), (14, 0.13, "parabola"), (8, 0.2, "constant")]):
        probs.append((square_mesh(n, d, jitter=0.2, seed=i), {"function": kn, "horizon": d, "outputdim": 1}, conf2d()))
    As = nl.stiffnessMatrix_batch(probs)
    for (m, k, c), A in zip(probs, As):
        B = nl.stiffnessMatrix(m, k, c)
        assert same_pattern(A, B)
        assert abs(A - B).max() == 0


def test_deterministic_runs(nl):
    m = square_mesh(24, 0.1, jitter=0.2, seed=6)
    k = {"function": "parabola", "horizon": 0.1, "outputdim": 1}
    A = nl.stiffnessMatrix(m, k, conf2d())
    B = nl.stiffnessMatrix(m, k, conf2d())
    assert same_pattern(A, B)
    assert np.array_equal(A.data, B.data)


def test_par_assemble_file_protocol(nl, tmp_path):
    from nlfem_gb300 import _lib
    lib = _lib.load()
    m = square_mesh(10, 0.1)
    c = conf2d()
    A = nl.stiffnessMatrix(m, KC, c)
    el = np.ascontiguousarray(m["elements"].ravel(), np.int64)
    elab = np.ascontiguousarray(m["elementLabels"], np.int64)
    ve = np.ascontiguousarray(m["vertices"].ravel(), np.float64)
    vlab = np.ascontiguousarray(m["vertexLabels"], np.int64)
    P = np.ascontiguousarray(c["quadrature"]["outer"]["points"].ravel()); w = c["quadrature"]["outer"]["weights"]
    dp, lp = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_long)
    D = lambda a: a.ctypes.data_as(dp)
    L = lambda a: a.ctypes.data_as(lp)
    nE, nV = m["elements"].shape[0], m["vertices"].shape[0]
    path = str(tmp_path / "spAd").encode()
    r = lib.nlfem_par_assemble(b"system", path, b"", int((vlab > 0).sum()), nV, L(el), L(elab), D(ve), L(vlab),
                               nE, int((elab > 0).sum()), nV, int((vlab > 0).sum()), D(P), len(w), D(w),
                               D(P), len(w), D(w), ctypes.c_double(0.1 ** 2), 0, 0, b"constant", b"",
                               b"retriangulate", b"retriangulate", 1, 2, 1, None, None, ctypes.c_long(0),
                               None, 0, None, ctypes.c_double(0.0), ctypes.c_double(-1.0), 0, 0)
    assert r == 0, lib.nlfem_last_error()
    B = nl.read_arma_spMat(tmp_path / "spAd")
    assert same_pattern(A, B) and abs(A - B).max() == 0


# ---------------------------------------------------------------- mixed precision
MIX_TOL = 1e-6   # relative Frobenius / max-entry error of the mixed path against the FP64 oracle


def test_certified_geometry_small_triangles(nl, orc):
    """Mesh regime: triangles of size ~delta/20 straddling the sphere, incl. near-tangent edges
    and vertices close to it. Certified FP32 cases must match the exact polygon exactly."""
    rng = np.random.Generator(np.random.PCG64(23))
    delta = 0.1
    n = 60000
    ang = rng.uniform(0, 2 * np.pi, n)
    rad = delta + rng.normal(0, 0.004, n)
    rad[::5] = delta + rng.normal(0, 1e-6, n)[::5]          # vertex near the sphere
    c = np.stack([rad * np.cos(ang), rad * np.sin(ang)], 1)
    h = delta / 20 * rng.uniform(0.5, 1.5, n)
    th = rng.uniform(0, 2 * np.pi, (n, 3))
    T = np.zeros((n, 6))
    T[:, 0:2] = c
    T[:, 2:4] = c + h[:, None] * np.stack([np.cos(th[:, 1]), np.sin(th[:, 1])], 1)
    T[:, 4:6] = c + h[:, None] * np.stack([np.cos(th[:, 2]), np.sin(th[:, 2])], 1)
    T[1::7, 2:4] = T[1::7, 0:2] + (T[1::7, 0:2] / np.linalg.norm(T[1::7, 0:2], axis=1)[:, None])[:, ::-1] * [1, -1] * h[1::7, None]
    x0 = np.array([0.3, -0.2])
    X = np.tile(x0, (n, 1))
    T = T + np.tile(x0, 3)
    for caps in (1, 0):
        cnt, amb, pts = nl.retriangulate_certified_batch(X, T, delta ** 2, caps)
        namb = 0
        for j in range(n):
            if amb[j]:
                namb += 1
                continue
            m, tri = orc.retriangulate_sq(X[j], T[j], delta ** 2, caps)
            exact_pts = 0 if m == 0 else m + 2
            got = cnt[j] if cnt[j] >= 3 else 0
            assert got == exact_pts, (caps, j, cnt[j], m)
            if m:
                R = np.concatenate([tri[0, :1], tri[:, 1], tri[-1:, 2]], axis=0) - X[j]
                # positions: FP32 accuracy, looser along near-tangent edges (values only)
                np.testing.assert_allclose(pts[j, :exact_pts], R, atol=1e-3 * delta)
        # about a third of the cases are built on a decision boundary
        assert namb < 0.45 * n


def test_certified_geometry_mesh_regime(nl, orc):
    """Outer points of mesh elements against the elements near their ball boundary (the cases the
    assembly meets): certified FP32 results equal the exact polygon counts; few fall back."""
    from nlfem_gb300 import meshes, quadrules
    v, e, l = meshes.regular_square(64, 0.1, jitter=0.2, seed=3)
    P, w = quadrules.dunavant7()
    rng = np.random.Generator(np.random.PCG64(4))
    E = v[e]
    bary = E.mean(axis=1)
    X, T = [], []
    for a in rng.choice(len(e), 60, replace=False):
        xs = E[a][0] + (E[a][1] - E[a][0]) * P[:, :1] + (E[a][2] - E[a][0]) * P[:, 1:2]
        d = np.linalg.norm(bary - bary[a], axis=1)
        cand = np.where(np.abs(d - 0.1) < 0.04)[0]
        for x in xs:
            X.append(np.repeat(x[None], len(cand), 0)); T.append(E[cand].reshape(-1, 6))
    X = np.concatenate(X); T = np.concatenate(T)
    cnt, amb, pts = nl.retriangulate_certified_batch(X, T, 0.01, 1)
    ex, _ = nl.retriangulate_batch(X, T, 0.01, 1)
    ok = amb == 0
    got = np.where(cnt >= 3, cnt - 2, 0)
    np.testing.assert_array_equal(got[ok], ex[ok])
    assert (~ok).sum() < 0.01 * (ex > 0).sum()


def test_certified_geometry_never_disagrees(nl, orc):
    """Where the FP32 geometry does not flag a decision as ambiguous, it reproduces the exact
    polygon point count and its points to FP32 accuracy. Half of the cases are built to sit on a
    decision boundary (tangent edges, vertices on the sphere); random cases rarely do."""
    rng = np.random.Generator(np.random.PCG64(17))
    cases = _cases_retri(rng, 4000)
    amb_random = 0
    for j, (x, T, sq, caps) in enumerate(cases):
        c, a, pts = nl.retriangulate_certified_batch(x[None], T[None], sq, caps)
        n, tri = orc.retriangulate_sq(x, T, sq, caps)
        if a[0]:
            amb_random += (j % 4 == 0)
            continue
        exact_pts = 0 if n == 0 else n + 2
        got = c[0] if c[0] >= 3 else 0
        assert got == exact_pts, (j, c[0], n)
        if n:
            R = np.concatenate([tri[0, :1], tri[:, 1], tri[-1:, 2]], axis=0) - x
            np.testing.assert_allclose(pts[0, :exact_pts], R, atol=1e-3 * np.sqrt(sq) + 1e-6)
    assert amb_random < 0.05 * len(cases) / 4


@pytest.mark.parametrize("n,delta,kern,jit", [(32, 0.1, "constant", 0.0), (24, 0.12, "parabola", 0.2),
                                              (20, 0.15, "constant", 0.2)])
def test_mixed_matches_oracle(nl, orc, n, delta, kern, jit):
    m = square_mesh(n, delta, jitter=jit, seed=n)
    k = {"function": kern, "horizon": delta, "outputdim": 1}
    A = nl.stiffnessMatrix(m, k, conf2d(precision="mixed"))
    B = orc.assemble(m, k, conf2d())["A"]
    assert same_pattern(A, B)
    fro, mx = rel_errors(A, B)
    assert fro < MIX_TOL and mx < MIX_TOL, (fro, mx)


def test_mixed_batch_mixed_kernels(nl, orc):
    """A batch mixing constant (closed-form inner sums) and parabola problems equals the single
    assemblies, and each problem matches the oracle."""
    probs = []
    for i, (n, d, kn) in enumerate([(10, 0.1, "constant"), (14, 0.13, "parabola"), (8, 0.2, "constant")]):
        probs.append((square_mesh(n, d, jitter=0.2, seed=i), {"function": kn, "horizon": d, "outputdim": 1},
                      conf2d(precision="mixed")))
    As = nl.stiffnessMatrix_batch(probs)
    for (m, k, c), A in zip(probs, As):
        B = nl.stiffnessMatrix(m, k, c)
        assert same_pattern(A, B)
        assert abs(A - B).max() <= 1e-12 * abs(B).max()
        R = orc.assemble(m, k, conf2d())["A"]
        assert same_pattern(A, R)
        fro, mx = rel_errors(A, R)
        assert fro < MIX_TOL and mx < MIX_TOL, (fro, mx)


def test_mixed_batch_three_kernel_classes(nl, orc):
    """Constant, parabola and fractional (Duffy close pairs) problems in one batch: one pass
    launch per kernel class, each matrix equal to its single assembly."""
    c = conf2d(rule="16", close="fractional", deg=3, precision="mixed")
    probs = [(square_mesh(10, 0.2, jitter=0.1, seed=21), {"function": "constant", "horizon": 0.2, "outputdim": 1}, c),
             (square_mesh(9, 0.2, jitter=0.1, seed=22), {"function": "fractional", "horizon": 0.2, "outputdim": 1,
                                                          "fractional_s": 0.4}, c),
             (square_mesh(8, 0.2, jitter=0.1, seed=23), {"function": "parabola", "horizon": 0.2, "outputdim": 1}, c)]
    As = nl.stiffnessMatrix_batch(probs)
    for (m, k, cc), A in zip(probs, As):
        B = nl.stiffnessMatrix(m, k, cc)
        assert same_pattern(A, B)
        assert abs(A - B).max() <= 1e-12 * abs(B).max()
        R = orc.assemble(m, k, conf2d(rule="16", close="fractional", deg=3))["A"]
        assert same_pattern(A, R)
        fro, mx = rel_errors(A, R)
        assert fro < MIX_TOL and mx < MIX_TOL, (fro, mx)


def test_one_shot_capacity_hints_overflow(nl, orc):
    """One-shot calls reuse the previous call's pattern sizes as scratch capacities when the mesh
    has the same counts. A second mesh with the same counts and a larger ball overflows them; the
    recount must give the exact pattern and values."""
    m = square_mesh(16, 0.1, jitter=0.2, seed=31)
    k1 = {"function": "constant", "horizon": 0.1, "outputdim": 1}
    nl.stiffnessMatrix(m, k1, conf2d(precision="mixed"))
    m2 = square_mesh(16, 0.1, jitter=0.1, seed=32)   # same counts
    k2 = {"function": "constant", "horizon": 0.25, "outputdim": 1}
    A = nl.stiffnessMatrix(m2, k2, conf2d(precision="mixed"))
    B = orc.assemble(m2, k2, conf2d())["A"]
    assert same_pattern(A, B)
    fro, mx = rel_errors(A, B)
    assert fro < MIX_TOL and mx < MIX_TOL, (fro, mx)
    A1 = nl.stiffnessMatrix(m, k1, conf2d(precision="mixed"))   # and back to the smaller one
    B1 = orc.assemble(m, k1, conf2d())["A"]
    assert same_pattern(A1, B1)


@pytest.mark.parametrize("case", ["2d", "2d_J", "3d", "dg"])
def test_evaluate_mass_matches_oracle(nl, orc, case):
    """par_evaluateMass on the GPU (deterministic fixed-point sums) against the oracle's
    sequential restatement."""
    from types import SimpleNamespace
    from nlfem_gb300 import quadrules
    rng = np.random.Generator(np.random.PCG64(7))
    if case == "3d":
        m = cube_mesh(5, 0.1, jitter=0.1, seed=2)
        P, w = quadrules.keast11()
    else:
        m = square_mesh(12, 0.1, jitter=0.2, seed=5)
        P, w = quadrules.dunavant7()
    nE, dV = m["elements"].shape
    dg = case == "dg"
    K = dV * nE if dg else m["vertices"].shape[0]
    ud = rng.standard_normal(K)
    J = nE // 2 if case == "2d_J" else nE
    mesh = SimpleNamespace(elements=m["elements"], elementLabels=m["elementLabels"], vertices=m["vertices"],
                           vertexLabels=m["vertexLabels"], dim=m["vertices"].shape[1], nE_Omega=J,
                           is_DiscontinuousGalerkin=dg, K=K)
    vd = nl.evaluateMass(mesh, ud, P, w)
    ref = orc.evaluate_mass(m, ud, P, w, J=J, is_dg=dg)
    assert np.abs(vd - ref).max() <= 1e-13 * np.abs(ref).max()
    assert np.array_equal(vd, nl.evaluateMass(mesh, ud, P, w))   # deterministic


def test_mixed_pair_list_exact(nl, orc):
    m = square_mesh(24, 0.13, jitter=0.2, seed=3)
    k = {"function": "constant", "horizon": 0.13, "outputdim": 1}
    ref = orc.assemble(m, k, conf2d(), want_pairs=True)
    got = nl.pair_list(m, k, conf2d(precision="mixed"))
    rp = ref["pairs"][np.lexsort((ref["pairs"][:, 1], ref["pairs"][:, 0]))]
    np.testing.assert_array_equal(got, rp)


def test_mixed_fractional(nl, orc):
    m = square_mesh(12, 0.2, jitter=0.1, seed=5)
    k = {"function": "fractional", "horizon": 0.2, "outputdim": 1, "fractional_s": 0.4}
    A = nl.stiffnessMatrix(m, k, conf2d(rule="16", close="fractional", deg=3, precision="mixed"))
    B = orc.assemble(m, k, conf2d(rule="16", close="fractional", deg=3))["A"]
    assert same_pattern(A, B)
    fro, mx = rel_errors(A, B)
    assert fro < MIX_TOL and mx < MIX_TOL, (fro, mx)


def test_mixed_3d(nl, orc):
    m = cube_mesh(5, 0.1, jitter=0.15, seed=2)
    k = {"function": "constant3D", "horizon": 0.3, "outputdim": 1}
    A = nl.stiffnessMatrix(m, k, conf3d(precision="mixed"))
    B = orc.assemble(m, k, conf3d())["A"]
    assert same_pattern(A, B)
    fro, mx = rel_errors(A, B)
    assert fro < MIX_TOL and mx < MIX_TOL, (fro, mx)


def test_mixed_deterministic(nl):
    m = square_mesh(28, 0.1, jitter=0.2, seed=6)
    k = {"function": "parabola", "horizon": 0.1, "outputdim": 1}
    A = nl.stiffnessMatrix(m, k, conf2d(precision="mixed"))
    B = nl.stiffnessMatrix(m, k, conf2d(precision="mixed"))
    assert same_pattern(A, B) and np.array_equal(A.data, B.data)


def test_mixed_pattern_equals_fp64_at_scale(nl):
    """On a mesh too large for the oracle the mixed pattern still equals the FP64 GPU pattern
    (itself bit-exact against the oracle on the smaller meshes above)."""
    m = square_mesh(96, 0.1, jitter=0.2, seed=1)
    A = nl.stiffnessMatrix(m, KC, conf2d(precision="mixed"))
    B = nl.stiffnessMatrix(m, KC, conf2d())
    assert same_pattern(A, B)
    fro, mx = rel_errors(A, B)
    assert fro < MIX_TOL and mx < MIX_TOL, (fro, mx)


@pytest.mark.parametrize("kern", ["parabola", "constant"])
def test_mixed_barycenter_2d(nl, orc, kern):
    m = square_mesh(16, 0.15, jitter=0.2, seed=4)
    k = {"function": kern, "horizon": 0.15, "outputdim": 1}
    A = nl.stiffnessMatrix(m, k, conf2d(method="baryCenter", precision="mixed"))
    B = orc.assemble(m, k, conf2d(method="baryCenter"))["A"]
    assert same_pattern(A, B)
    fro, mx = rel_errors(A, B)
    assert fro < MIX_TOL and mx < MIX_TOL, (fro, mx)


def test_mixed_3d_deterministic_and_fp64_pattern(nl):
    m = cube_mesh(7, 0.1, jitter=0.1, seed=3)
    k = {"function": "constant3D", "horizon": 0.25, "outputdim": 1}
    A1 = nl.stiffnessMatrix(m, k, conf3d(precision="mixed"))
    A2 = nl.stiffnessMatrix(m, k, conf3d(precision="mixed"))
    assert same_pattern(A1, A2) and np.array_equal(A1.data, A2.data)
    B = nl.stiffnessMatrix(m, k, conf3d())
    assert same_pattern(A1, B)
    fro, mx = rel_errors(A1, B)
    assert fro < MIX_TOL and mx < MIX_TOL, (fro, mx)


@pytest.mark.parametrize("case", ["retri2d", "bary3d"])
def test_search_stamp_epochs(nl, case):
    """The pair search's 16-bit per-warp stamp epochs: later assemblies of a session reuse the
    stamps uncleared, and a warp whose epoch wraps clears its own stamps; every assembly, normal
    or replayed from the graph, gives the first one's matrix bit for bit. The epochs are moved
    once, forward (above every epoch used so far), to 16 below the wrap; the assemblies after it
    take the warps that get elements through the wrap."""
    from nlfem_gb300 import _lib
    if case == "retri2d":
        probs = [(square_mesh(40, 0.1, jitter=0.2, seed=11), KC, conf2d(precision="mixed"))]
    else:
        probs = [(cube_mesh(8, 0.1, jitter=0.1, seed=12), {"function": "constant3D", "horizon": 0.2, "outputdim": 1},
                  conf3d(precision="mixed"))]
    s = nl.Session(probs)
    try:
        assert s.lib.nlfem_session_set_search_epoch(s.h, 5) != 0   # no search has run yet
        s.assemble()
        ref = s.download(0)
        _lib.check(s.lib.nlfem_session_set_search_epoch(s.h, 0xfff0))
        for i in range(40):
            graph = i % 2 == 1
            s.assemble(graph=graph)
            A = s.download(0)
            assert same_pattern(A, ref) and np.array_equal(A.data, ref.data), (i, graph)
    finally:
        s.close()


@pytest.mark.parametrize("case", ["retri_batch", "bary3d", "fractional"])
def test_session_graph_replay_bitwise(nl, case):
    if case == "retri_batch":
        probs = [(square_mesh(20, 0.12, jitter=0.2, seed=9), {"function": "parabola", "horizon": 0.12, "outputdim": 1},
                  conf2d(precision="mixed")),
                 (square_mesh(14, 0.2, jitter=0.1, seed=2), {"function": "constant", "horizon": 0.2, "outputdim": 1},
                  conf2d(precision="mixed"))]
    elif case == "bary3d":
        probs = [(cube_mesh(5, 0.1, jitter=0.1, seed=5), {"function": "constant3D", "horizon": 0.3, "outputdim": 1},
                  conf3d(precision="mixed"))]
    else:
        probs = [(square_mesh(10, 0.2, jitter=0.1, seed=3),
                  {"function": "fractional", "horizon": 0.2, "outputdim": 1, "fractional_s": 0.4},
                  conf2d(rule="16", close="fractional", deg=3, precision="mixed"))]
    s = nl.Session(probs)
    try:
        st0 = s.assemble()
        ref = [s.download(i) for i in range(len(probs))]
        s.assemble()   # a repeated assembly builds the pattern in one pass (scratch sized by the first)
        for i, B in enumerate(ref):
            A = s.download(i)
            assert same_pattern(A, B) and np.array_equal(A.data, B.data)
        for _ in range(3):
            st = s.assemble(graph=True)
            assert st["n_pairs"] == st0["n_pairs"] and st["nnz_structural"] == st0["nnz_structural"]
            for i, B in enumerate(ref):
                A = s.download(i)
                assert same_pattern(A, B) and np.array_equal(A.data, B.data)
    finally:
        s.close()
    # a session whose first call already asks for the graph (capture right after the first run)
    s2 = nl.Session(probs)
    try:
        for _ in range(3):
            s2.assemble(graph=True)
            for i, B in enumerate(ref):
                A = s2.download(i)
                assert same_pattern(A, B) and np.array_equal(A.data, B.data)
    finally:
        s2.close()


@pytest.mark.parametrize("n,delta,kern,jit,close", [(32, 0.1, "constant", 0.0, None), (24, 0.12, "parabola", 0.2, None),
                                                    (20, 0.15, "constant", 0.2, None),
                                                    (12, 0.2, "fractional", 0.1, "fractional")])
def test_fp64_onesided_matches_oracle(nl, orc, n, delta, kern, jit, close):
    """The mixed path's algorithm in FP64 arithmetic (precision "fp64-onesided"): one-sided pass,
    closed forms, fixed-point sums with a unit of 2^-52 of the entry scale. It meets the FP64 bar
    against the oracle (1e-12), and its pattern is the reference's."""
    m = square_mesh(n, delta, jitter=jit, seed=n)
    k = {"function": kern, "horizon": delta, "outputdim": 1}
    if kern == "fractional":
        k["fractional_s"] = 0.4
        c = conf2d(rule="16", close=close, deg=3)
    else:
        c = conf2d()
    A = nl.stiffnessMatrix(m, k, dict(c, precision="fp64-onesided"))
    B = orc.assemble(m, k, c)["A"]
    assert same_pattern(A, B)
    fro, mx = rel_errors(A, B)
    assert fro < 1e-12 and mx < 1e-12, (fro, mx)
    # deterministic, like every fixed-point path
    A2 = nl.stiffnessMatrix(m, k, dict(c, precision="fp64-onesided"))
    assert np.array_equal(A.data, A2.data)


def test_fp64_onesided_refusals(nl):
    from nlfem_gb300._lib import NlfemError
    m = cube_mesh(3, 0.2)
    from nlfem_gb300 import quadrules
    P, w = quadrules.keast11()
    c = {"ansatz": "CG", "approxBalls": {"method": "baryCenter"},
         "quadrature": {"outer": {"points": P, "weights": w}, "inner": {"points": P, "weights": w}},
         "precision": "fp64-onesided"}
    with pytest.raises(NlfemError, match="2D retriangulate"):
        nl.stiffnessMatrix(m, {"function": "constant3D", "horizon": 0.2, "outputdim": 1}, c)



FIELD_CASES = {
    # constantField (model.cpp:182-191), retriangulate with caps, jittered
    "constfield": (lambda: square_mesh(12, 0.15, jitter=0.2, seed=21), {"function": "constantField", "horizon": 0.15, "outputdim": 2},
                   lambda: conf2d()),
    # the microelastic field kernel, singular: close pairs by the fractional Duffy rule
    "microfield_frac": (lambda: square_mesh(8, 0.2, jitter=0.1, seed=22),
                        {"function": "linearPrototypeMicroelasticField", "horizon": 0.2, "outputdim": 2, "fractional_s": -0.5},
                        lambda: conf2d(rule="16", close="fractional", deg=3)),
    # the same with the weakSingular close rule
    "microfield_weak": (lambda: square_mesh(8, 0.2, jitter=0.1, seed=23),
                        {"function": "linearPrototypeMicroelasticField", "horizon": 0.2, "outputdim": 2, "fractional_s": -0.5},
                        lambda: conf2d(rule="16", close="weakSingular", deg=3)),
    # 2D barycenter rule with the constant field kernel
    "constfield_bary": (lambda: square_mesh(10, 0.2, jitter=0.15, seed=24), {"function": "constantField", "horizon": 0.2, "outputdim": 2},
                        lambda: conf2d(method="baryCenter")),
    # 3D microelastic field kernel, barycenter (not singular in the reference's lookup); the inner
    # rule avoids the outer points, where the kernel is singular
    "microfield3d": (lambda: cube_mesh(3, 0.1, jitter=0.1, seed=25),
                     {"function": "linearPrototypeMicroelasticField3D", "horizon": 0.35, "outputdim": 3}, lambda: _conf3d_inner4()),
}


def _conf3d_inner4():
    pa, pb = 0.5854101966249685, 0.1381966011250105
    c = conf3d()
    c["quadrature"]["inner"] = {"points": np.array([[pb, pb, pb], [pa, pb, pb], [pb, pa, pb], [pb, pb, pa]]),
                                "weights": np.full(4, 1.0 / 24)}
    return c


@pytest.mark.parametrize("case", list(FIELD_CASES))
def test_vector_kernels_match_oracle(nl, orc, case):
    """Vector-valued kernels (outdim 2 and 3) on the GPU: the reference's general block indexing
    (integration.cpp:345-540, 910-1018, 82-288; Cassemble.cpp:721-770) in FP64 with
    deterministic fixed-point sums. Pattern bit-exact, values within 1e-12 of the oracle (which
    the reference build pins bit for bit)."""
    mk, kernel, mkconf = FIELD_CASES[case]
    m = dict(mk(), outdim=kernel["outputdim"])
    conf = mkconf()
    A = nl.stiffnessMatrix(m, kernel, conf)
    B = orc.assemble(m, kernel, conf)["A"]
    assert A.shape == B.shape == (m["vertices"].shape[0] * kernel["outputdim"],) * 2
    assert same_pattern(A, B)
    fro, mx = rel_errors(A, B)
    assert fro < FP64_TOL and mx < FP64_TOL, (fro, mx)
    A2 = nl.stiffnessMatrix(m, kernel, conf)
    assert np.array_equal(A.data, A2.data)   # deterministic


@pytest.mark.parametrize("load,outdim,dim", [("linearField", 2, 2), ("constantRightField", 2, 2), ("constantDownField", 2, 2),
                                              ("constantBothField", 2, 2), ("linearField3D", 3, 3), ("gaussian", 1, 2),
                                              ("jump", 1, 2), ("tensorsin", 1, 2)])
def test_further_forcings_match_oracle(nl, orc, load, outdim, dim):
    """The vector forcings and the scalar gaussian / jump / tensorsin (model.cpp:201-258) against
    the oracle: within 1e-13 (CUDA's exp and sin may differ from the host's in the last bit)."""
    m = square_mesh(14, 0.1, jitter=0.2, seed=26) if dim == 2 else cube_mesh(3, 0.2, jitter=0.1, seed=27)
    m = dict(m, outdim=outdim)
    conf = conf2d() if dim == 2 else conf3d()
    f = nl.loadVector(m, {"function": load}, conf)
    g = orc.assemble(m, None, conf, compute="forcing", load={"function": load})["f"]
    assert f.shape == g.shape == (m["vertices"].shape[0] * outdim,)
    np.testing.assert_allclose(f, g, rtol=1e-13, atol=1e-14 * np.abs(g).max())


def test_load_vector_domain_decomposition(nl, orc):
    """par_forcing weights each element's contribution by 1 / zeta(aT, aT) (Cassemble.cpp:901-908)."""
    m = square_mesh(12, 0.1, jitter=0.2, seed=28)
    nE = m["elements"].shape[0]
    bx = m["vertices"][m["elements"]].mean(axis=1)[:, 0]
    rows, cols = [], []
    for e in range(nE):   # two overlapping subdomains around x = 0.5
        for z, inside in enumerate((bx[e] < 0.6, bx[e] > 0.4)):
            if inside:
                rows.append(e); cols.append(z)
    Z = sp.csr_matrix((np.ones(len(rows)), (rows, cols)), shape=(nE, 2))
    m = dict(m, nZeta=2, ZetaIndicator=Z)
    f = nl.loadVector(m, {"function": "linear"}, conf2d())
    g = orc.assemble(m, None, conf2d(), compute="forcing", load={"function": "linear"})["f"]
    np.testing.assert_allclose(f, g, rtol=1e-13, atol=1e-15 * np.abs(g).max())
    f0 = nl.loadVector(dict(m, nZeta=0), {"function": "linear"}, conf2d())
    assert not np.allclose(f, f0)


def test_vector_kernel_refusals(nl):
    from nlfem_gb300._lib import NlfemError
    m = dict(square_mesh(4, 0.2), outdim=2)
    k = {"function": "constantField", "horizon": 0.2, "outputdim": 2}
    with pytest.raises(NlfemError, match="fp64 path only"):
        nl.stiffnessMatrix(m, k, conf2d(precision="mixed"))
    with pytest.raises(NlfemError, match="output components"):
        nl.stiffnessMatrix(dict(m, outdim=1), dict(k, outputdim=1), conf2d())



@pytest.mark.parametrize("n,delta,kern,jit", [(10, 0.1, "constant", 0.15), (14, 0.12, "parabola", 0.2), (9, 0.25, "constant", 0.0)])
def test_exact_ball_matches_oracle(nl, orc, n, delta, kern, jit):
    """exactBall (integration.cpp:706-907, 1300-1351, 1632-1761) on the FP64 path: the polygon
    without cap points plus up to three circular segments at their centroids. The pair search takes
    the polygon's interaction test. Within 1e-12 of the oracle (CUDA's acos / sin / pow may differ
    from the host's in the last bit)."""
    m = square_mesh(n, delta, jitter=jit, seed=n + 40)
    k = {"function": kern, "horizon": delta, "outputdim": 1}
    c = conf2d(method="exactBall")
    A = nl.stiffnessMatrix(m, k, c)
    B = orc.assemble(m, k, c)["A"]
    assert same_pattern(A, B)
    fro, mx = rel_errors(A, B)
    assert fro < FP64_TOL and mx < FP64_TOL, (fro, mx)
    pairs = orc.assemble(m, k, c, want_pairs=True)["pairs"]
    sel = pairs[np.random.Generator(np.random.PCG64(n)).choice(len(pairs), min(300, len(pairs)), replace=False)]
    g, gr = nl.pair_blocks(m, k, c, sel)
    o, orr = orc.pair_blocks(m, k, c, sel)
    np.testing.assert_array_equal(gr != 0, orr != 0)
    np.testing.assert_allclose(g, o, rtol=1e-12, atol=1e-12 * np.abs(o).max())


def test_autotune_keeps_the_matrix(nl):
    """The launch-shape autotuner (nlfem_session_autotune) times 1, 2, ... blocks per SM of the
    pair search and the persistent pass and keeps the fastest; the shapes change no bit of the
    matrix (fixed-point sums, per-element search order)."""
    m = square_mesh(48, 0.1, jitter=0.2, seed=61)
    k = {"function": "constant", "horizon": 0.1, "outputdim": 1}
    s = nl.Session([(m, k, conf2d(precision="mixed"))])
    try:
        s.assemble()
        A0 = s.download(0)
        t = s.autotune(reps=1)
        A1 = s.download(0)
        assert t["bfs"] >= 1 and len(t["bfs_ms"]) >= 1
        assert t["pass"] >= 1 and len(t["pass_ms"]) >= 1
        assert all(x > 0 for x in t["bfs_ms"] + t["pass_ms"])
        assert np.array_equal(A0.indptr, A1.indptr) and np.array_equal(A0.indices, A1.indices)
        assert np.array_equal(A0.data, A1.data)
        s.assemble(graph=True)   # a graph captured after tuning replays the tuned shapes
        s.assemble(graph=True)
        assert np.array_equal(s.download(0).data, A0.data)
    finally:
        s.close()


def test_mixed_slot_maps_window_rank_and_hash(nl, orc):
    """The one-sided pass finds matrix slots with window-rank bitmaps when the rows span narrow
    ranges of vertex numbers (a row-by-row numbering) and with per-row hash tables otherwise (here:
    a random vertex numbering). Both give the same matrix, bit for bit after renumbering, and
    both match the oracle within the mixed tolerance."""
    from nlfem_gb300 import _lib, meshes
    v, e, l = meshes.regular_square(64, 0.03, jitter=0.2, seed=21)
    m = meshes.mesh_dict(v, e, l)
    k = {"function": "constant", "horizon": 0.03, "outputdim": 1}
    c = conf2d(precision="mixed")
    A = nl.stiffnessMatrix(dict(m), k, c)
    assert _lib.stats()["slot_map"] == 1
    nV = v.shape[0]
    perm = np.random.default_rng(3).permutation(nV)   # vertex i becomes vertex perm[i]
    v2 = np.empty_like(v)
    v2[perm] = v
    m2 = meshes.mesh_dict(v2, perm[e], l)
    B = nl.stiffnessMatrix(m2, k, c)
    assert _lib.stats()["slot_map"] == 2
    Ac = A.tocoo()   # renumbered entry by entry: slots that cancelled to zero stay stored
    A2 = sp.csr_matrix((Ac.data, (perm[Ac.row], perm[Ac.col])), shape=(nV, nV))
    A2.sort_indices(); B.sort_indices()
    assert same_pattern(A2, B)
    np.testing.assert_array_equal(A2.data, B.data)
    C = orc.assemble(m, k, conf2d())["A"]
    assert same_pattern(A, C)
    fro, mx = rel_errors(A, C)
    assert fro < MIX_TOL and mx < MIX_TOL, (fro, mx)


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_far_component_capacity_retries(nl, orc, prec):
    """The search sizes its pair pool from the mesh's mean element size. A far-away extra triangle
    inflates the bounding box, so that estimate is far too small and the pool overflows: the
    search reruns with the size it counted. The pairs and the matrix are those of the oracle."""
    from nlfem_gb300 import meshes
    v, e, l = meshes.regular_square(32, 0.3, jitter=0.1, seed=31)
    nV = v.shape[0]
    v2 = np.vstack([v, [[50.0, 50.0], [50.01, 50.0], [50.0, 50.01]]])
    e2 = np.vstack([e, [[nV, nV + 1, nV + 2]]])
    l2 = np.concatenate([l, [1]])
    m = meshes.mesh_dict(v2, e2, l2)
    k = {"function": "constant", "horizon": 0.3, "outputdim": 1}
    A = nl.stiffnessMatrix(dict(m), k, conf2d(precision=prec))
    ref = orc.assemble(m, k, conf2d(), want_pairs=True)
    got = nl.pair_list(m, k, conf2d(precision=prec))
    rp = ref["pairs"][np.lexsort((ref["pairs"][:, 1], ref["pairs"][:, 0]))]
    np.testing.assert_array_equal(got, rp)
    assert same_pattern(A, ref["A"])
    fro, mx = rel_errors(A, ref["A"])
    tol = MIX_TOL if prec == "mixed" else FP64_TOL
    assert fro < tol and mx < tol, (fro, mx)


def test_mixed_refuses_elements_far_larger_than_the_horizon(nl, orc):
    """The margins of the mixed path's FP32 geometry hold while every element is at most 16 times
    the horizon (certified.cuh); beyond that the mixed precision is refused and FP64 runs. With a
    horizon this small, a ball around an element's own quadrature point stays inside the element,
    which the retriangulation counts as no polygon, so some elements have no pair at all."""
    from nlfem_gb300._lib import NlfemError
    m = square_mesh(8, 0.005, jitter=0.1, seed=33)
    k = {"function": "constant", "horizon": 0.005, "outputdim": 1}
    with pytest.raises(NlfemError, match="no larger than 16 times the horizon"):
        nl.stiffnessMatrix(dict(m), k, conf2d(precision="mixed"))
    A = nl.stiffnessMatrix(dict(m), k, conf2d())
    B = orc.assemble(m, k, conf2d())["A"]
    assert same_pattern(A, B)
    if B.nnz:
        fro, mx = rel_errors(A, B)
        assert fro < FP64_TOL and mx < FP64_TOL, (fro, mx)
