"""GPU parity against the oracle: bit-exact sparsity pattern and pair set, FP64 values within
rounding, deterministic runs. All calls go through the C ABI (libnlfem_gpu.so)."""
import ctypes

import numpy as np
import pytest
import scipy.sparse as sp

from conftest import conf2d, conf3d, square_mesh, cube_mesh, rel_errors, same_pattern

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
