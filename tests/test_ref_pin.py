"""The CPU restatement and the committed fixtures against the reference's own C++.

oracle/ref.mk compiles the reference's src/*.cpp unmodified against the project-written stand-ins
in oracle/refshim/ (oracle/_ref/libnlfem_ref.so). Where that build exists, these tests check:
* every fixture case of tests/golden/oracle_cases.npz that the reference can assemble is its
  output bit for bit (matrix and load vector), so the GPU tests against those fixtures compare
  with the reference itself;
* the restatement equals the reference bit for bit on further meshes, single-threaded, and to
  rounding with OpenMP (the thread partition changes the order of the final sums);
* the load vector and the retriangulation hook agree bit for bit, par_evaluateMass to rounding
  (the reference adds with omp atomic in its threads' order).
Two fixture cases are not assembled by the reference: "linf8" needs CGAL, and "tangent" makes the
reference write past its 9-point polygon buffer (integration.cpp:1415), which the stack
protector stops. Where the reference build is absent (it needs the reference checkout), the
tests are skipped.
"""
import os
import sys

import numpy as np
import pytest
import scipy.sparse as sp

from conftest import conf2d, conf3d, cube_mesh, labeled_mesh, same_pattern, square_mesh

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

pytestmark = pytest.mark.skipif(
    not os.path.exists(os.path.join(os.path.dirname(HERE), "oracle", "_ref", "libnlfem_ref.so")),
    reason="the reference build oracle/_ref is absent (it needs the reference checkout)")

NOT_IN_REFERENCE = ("linf8", "tangent")


def _bitwise(a, b):
    return np.array_equal(np.asarray(a, np.float64).view(np.int64), np.asarray(b, np.float64).view(np.int64))


def test_fixtures_are_the_references_output():
    from oracle import ref
    import make_oracle_golden as g
    Z = np.load(os.path.join(HERE, "golden", "oracle_cases.npz"))
    checked = 0
    for name, (mesh, kernel, conf, load) in g.cases().items():
        if name in NOT_IN_REFERENCE:
            continue
        m = dict(mesh)
        for k in ("elements", "elementLabels", "vertices", "vertexLabels"):
            m[k] = Z[f"{name}.{k}"]
        A = ref.assemble(m, kernel, conf)["A"]
        A.sort_indices()
        K = A.shape[0]
        B = sp.csr_matrix((Z[f"{name}.data"], Z[f"{name}.indices"], Z[f"{name}.indptr"]), shape=(K, K))
        assert same_pattern(A, B), name
        assert _bitwise(A.data, B.data), name
        if load is not None:
            f = ref.assemble(m, None, conf, compute="forcing", load=load)["f"]
            assert _bitwise(f, Z[f"{name}.f"]), name
        checked += 1
    assert checked == 10


@pytest.mark.parametrize("case", ["jitter24", "parabola16", "frac10", "cube4", "nocaps16"])
def test_oracle_equals_reference(case):
    from oracle import oracle, ref
    kc = {"function": "constant", "horizon": 0.1, "outputdim": 1}
    mesh, kernel, conf = {
        "jitter24": (square_mesh(24, 0.1, jitter=0.2, seed=31), kc, conf2d()),
        "parabola16": (square_mesh(16, 0.12, jitter=0.2, seed=32),
                       {"function": "parabola", "horizon": 0.12, "outputdim": 1}, conf2d(rule="16")),
        "frac10": (square_mesh(10, 0.2, jitter=0.1, seed=33),
                   {"function": "fractional", "horizon": 0.2, "outputdim": 1, "fractional_s": 0.3},
                   conf2d(close="fractional", deg=3)),
        "cube4": (cube_mesh(4, 0.2, jitter=0.1, seed=34), {"function": "constant3D", "horizon": 0.3, "outputdim": 1},
                  conf3d()),
        "nocaps16": (square_mesh(16, 0.1, jitter=0.2, seed=35), kc, conf2d(caps=0)),
    }[case]
    R = ref.assemble(mesh, kernel, conf)["A"]
    O = oracle.assemble(mesh, kernel, conf)["A"]
    R.sort_indices(); O.sort_indices()
    assert same_pattern(R, O)
    assert _bitwise(R.data, O.data)
    # OpenMP: the same pattern, values to rounding (the thread partition orders the final sums)
    R4 = ref.assemble(mesh, kernel, conf, nthreads=4)["A"]
    R4.sort_indices()
    assert same_pattern(R4, O)
    assert abs(R4 - O).max() <= 1e-13 * abs(O).max()


def test_load_vector_and_mass_equal_reference():
    from oracle import oracle, ref
    from nlfem_gb300 import quadrules
    for mesh, conf, load in ((square_mesh(20, 0.1, jitter=0.2, seed=41), conf2d(), "linear"),
                             (cube_mesh(4, 0.2, jitter=0.1, seed=42), conf3d(), "linear3D")):
        fr = ref.assemble(mesh, None, conf, compute="forcing", load={"function": load})["f"]
        fo = oracle.assemble(mesh, None, conf, compute="forcing", load={"function": load})["f"]
        assert _bitwise(fr, fo)
    mesh = square_mesh(16, 0.1, jitter=0.2, seed=43)
    P, w = quadrules.dunavant7()
    u = np.random.Generator(np.random.PCG64(5)).standard_normal(mesh["vertices"].shape[0])
    # the reference adds with omp atomic in its threads' order: equal to rounding
    vr = ref.evaluate_mass(mesh, u, P, w)
    vo = oracle.evaluate_mass(mesh, u, P, w)
    assert np.allclose(vr, vo, rtol=0, atol=1e-14 * abs(vo).max())


def test_retriangulation_equals_reference():
    from oracle import oracle, ref
    rng = np.random.Generator(np.random.PCG64(6))
    for _ in range(2000):
        TE = rng.uniform(-1, 1, 6)
        x = rng.uniform(-1, 1, 2)
        sqd = rng.uniform(0.05, 1.5)
        caps = int(rng.integers(0, 2))
        nr, tr = ref.retriangulate_sq(x, TE, sqd, caps)
        no, to = oracle.retriangulate_sq(x, TE, sqd, caps)
        assert nr == no
        assert _bitwise(tr, to)


def test_load_vector_with_zeta_weights_equals_reference():
    """par_forcing's 1 / zeta(aT, aT) weight (Cassemble.cpp:901-908) in the restatement."""
    from oracle import oracle, ref
    m = square_mesh(12, 0.1, jitter=0.2, seed=44)
    nE = m["elements"].shape[0]
    bx = m["vertices"][m["elements"]].mean(axis=1)[:, 0]
    rows, cols = [], []
    for e in range(nE):
        for z, inside in enumerate((bx[e] < 0.6, bx[e] > 0.4)):
            if inside:
                rows.append(e); cols.append(z)
    Z = sp.csr_matrix((np.ones(len(rows)), (rows, cols)), shape=(nE, 2))
    m = dict(m, nZeta=2, ZetaIndicator=Z)
    fr = ref.assemble(m, None, conf2d(), compute="forcing", load={"function": "linear"})["f"]
    fo = oracle.assemble(m, None, conf2d(), compute="forcing", load={"function": "linear"})["f"]
    assert _bitwise(fr, fo)


def test_zeta_weighted_matrix_equals_reference():
    """The system's 1 / zeta(aT, bT) weights (Cassemble.cpp:648-657) in the restatement, on the
    domain decomposition of the GPU test (two subdomains overlapping in a strip wider than the
    ball; the first 20 elements in both, as chk_Mesh requires)."""
    from oracle import oracle, ref
    m = square_mesh(14, 0.1, jitter=0.1, seed=8)
    x = m["vertices"][m["elements"]].mean(axis=1)[:, 0]
    rows = [[0, 1] if e < 20 else ([0] if xi < 0.3 else ([1] if xi > 0.7 else [0, 1])) for e, xi in enumerate(x)]
    indptr = np.cumsum([0] + [len(r) for r in rows])
    Z = sp.csr_matrix((np.ones(indptr[-1]), np.concatenate(rows), indptr), shape=(len(rows), 2))
    m = dict(m, nZeta=2, ZetaIndicator=Z)
    kc = {"function": "constant", "horizon": 0.1, "outputdim": 1}
    R = ref.assemble(m, kc, conf2d())["A"]
    O = oracle.assemble(m, kc, conf2d())["A"]
    R.sort_indices(); O.sort_indices()
    assert same_pattern(R, O)
    assert _bitwise(R.data, O.data)


def _bridges():
    from nlfem_gb300.meshes import mesh_dict
    m = square_mesh(14, 0.1, jitter=0.1, seed=5)
    lab = m["elementLabels"].copy()
    lab[40:60] = 0
    return mesh_dict(m["vertices"], m["elements"], lab)


def _dg(close, kname, s):
    c = conf2d(close=close, deg=3)
    c["ansatz"] = "DG"
    return (square_mesh(8, 0.2, jitter=0.1, seed=16), {"function": kname, "horizon": 0.2, "outputdim": 1, "fractional_s": s}, c)


def _field(kname, conf, seed, s=None):
    k = {"function": kname, "horizon": 0.2, "outputdim": 2}
    if s is not None:
        k["fractional_s"] = s
    return (square_mesh(8, 0.2, jitter=0.1, seed=seed), k, conf)


WIDENED = {
    # label-0 elements searched through, never paired (Cassemble.cpp:611-633)
    "bridges": lambda: (_bridges(), {"function": "constant", "horizon": 0.1, "outputdim": 1}, conf2d()),
    "bary2d": lambda: (square_mesh(14, 0.15, jitter=0.2, seed=4), {"function": "parabola", "horizon": 0.15, "outputdim": 1},
                       conf2d(method="baryCenter")),
    "fullsearch": lambda: (square_mesh(10, 0.1, jitter=0.1, seed=3), {"function": "constant", "horizon": 0.1, "outputdim": 1},
                           dict(conf2d(), is_fullConnectedComponentSearch=1)),
    "weaksing": lambda: (square_mesh(8, 0.2, jitter=0.1, seed=6),
                         {"function": "fractional", "horizon": 0.2, "outputdim": 1, "fractional_s": 0.4},
                         conf2d(close="weakSingular", deg=3)),
    "prototype": lambda: (square_mesh(8, 0.2, jitter=0.1, seed=6),
                          {"function": "linearPrototypeMicroelastic", "horizon": 0.2, "outputdim": 1, "fractional_s": -0.5},
                          conf2d(close="fractional", deg=3)),
    "dg_weak_fractional": lambda: _dg("weakSingular", "fractional", 0.4),
    "dg_weak_prototype": lambda: _dg("weakSingular", "linearPrototypeMicroelastic", -0.5),
    "field_weak": lambda: _field("linearPrototypeMicroelasticField", conf2d(close="weakSingular", deg=3), 23, -0.5),
    "constfield_bary": lambda: _field("constantField", conf2d(method="baryCenter"), 24),
}
for _r in ("retriangulate_unsymm", "subSetBall", "averageBall", "baryCenterRT", "noTruncation"):
    WIDENED["rule_" + _r] = (lambda r: lambda: (square_mesh(12, 0.12, jitter=0.15, seed=17),
                                                {"function": "parabola", "horizon": 0.12, "outputdim": 1},
                                                conf2d(method=r)))(_r)
for _k in ("labeled", "notch", "labeledNotch", "labeledValve", "constantTruncated"):
    WIDENED["kernel_" + _k] = (lambda k: lambda: (labeled_mesh(10, 6), {"function": k, "horizon": 0.1, "outputdim": 1},
                                                  conf2d()))(_k)


@pytest.mark.parametrize("case", sorted(WIDENED))
def test_widened_rows_equal_reference(case):
    """The restatement against the reference's own C++ on every configuration beyond the headline
    rules that the GPU tests compare with it: label-0 bridges, the 2D barycenter rule, the full
    component search, the weakSingular close rule, the prototype microelastic kernel, DG with
    singular kernels, vector-valued kernels, the further ball rules and the label- and
    position-dependent kernels. Bit for bit, single-threaded."""
    from oracle import oracle, ref
    mesh, kernel, conf = WIDENED[case]()
    if int(kernel.get("outputdim", 1)) > 1:
        mesh = dict(mesh, outdim=int(kernel["outputdim"]))
    R = ref.assemble(mesh, kernel, conf)["A"]
    O = oracle.assemble(mesh, kernel, conf)["A"]
    R.sort_indices(); O.sort_indices()
    assert same_pattern(R, O)
    assert _bitwise(R.data, O.data)
