"""Generates the golden fixtures of tests/golden/ from the reference checkout.

Run here (where the reference is mounted), never on the GPU machine:
    python tests/golden/make_golden.py /path/to/reference

What it pins, and how:
* quadrules_ref.json  - the 7- and 16-point triangle rules exactly as the reference's test
  configuration lists them (examples/test2D/conf/testConfFractional.py:27-77), evaluated from
  that file's AST (the module itself imports quadpy, which is absent).
* tensorgauss_ref.npz - the reference's own ``tensorgauss`` class (cython/nlfem.pyx:108-126),
  executed from its source text, for degrees 2 and 5.
* vertexlabels_ref.json - the reference's ``get_vertexLabel`` (cython/nlfem.pyx:392-402) executed
  from source on a small labelled mesh (np.int aliased to int for NumPy >= 1.24).
* tets_ref.json - the golden 6-tetrahedron split of tests/assembleTest.cpp:257-420.
* arma_ref.npz - the reference's ``read_arma_spMat`` / ``read_arma_mat`` (nlfem.pyx:28-101)
  executed from source on files written by this package's writer: the decoded arrays prove the
  writer speaks the reference's file format.
"""
import ast
import json
import os
import re
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def _pyx_function(src, name, kind="def"):
    m = re.search(rf"^{kind} {name}\b.*?(?=^\S)", src, re.S | re.M)
    if not m:
        raise RuntimeError(f"{name} not found")
    return m.group(0)


def quadrules(ref):
    path = os.path.join(ref, "examples/test2D/conf/testConfFractional.py")
    tree = ast.parse(open(path).read())
    out = {}
    for node in tree.body:
        if isinstance(node, ast.Assign) and getattr(node.targets[0], "id", None) == "quadrules":
            for k, v in zip(node.value.keys, node.value.values):
                key = ast.literal_eval(k)
                if key in ("7point", "16point"):
                    pts = eval(compile(ast.Expression(v.elts[0]), path, "eval"), {"np": np})
                    wts = eval(compile(ast.Expression(v.elts[1]), path, "eval"), {"np": np})
                    out[key] = {"points": np.asarray(pts).tolist(), "weights": np.asarray(wts).tolist()}
    return out


def tensorgauss(ref):
    src = open(os.path.join(ref, "cython/nlfem.pyx")).read()
    ns = {"np": np}
    exec(_pyx_function(src, "tensorgauss", "class"), ns)
    res = {}
    for deg in (2, 5):
        tg = ns["tensorgauss"](deg)
        res[f"points{deg}"] = tg.points
        res[f"weights{deg}"] = tg.weights
    return res


def vertexlabels(ref):
    src = open(os.path.join(ref, "cython/nlfem.pyx")).read()

    class _np_shim:
        def __getattr__(self, k):
            return int if k == "int" else getattr(np, k)

    ns = {"np": _np_shim()}
    exec(_pyx_function(src, "get_vertexLabel"), ns)
    from nlfem_gb300.meshes import regular_square
    v, e, l = regular_square(6, 0.1, jitter=0.2, seed=3)
    l = l.copy()
    l[5] = 0
    l[7] = 2
    return {"elements": e.tolist(), "elementLabels": l.tolist(), "vertices": v.tolist(),
            "vertexLabels": np.asarray(ns["get_vertexLabel"](e, l, v)).tolist()}


def tets(ref):
    src = open(os.path.join(ref, "tests/assembleTest.cpp")).read()
    m = re.search(r"testTetrahedons\s*=\s*\{(.*?)\};", src, re.S)
    rows = re.findall(r"\{\s*([0-9,\s]+)\}", m.group(1))
    return [[int(x) for x in r.split(",")] for r in rows]


def arma(ref):
    src = open(os.path.join(ref, "cython/nlfem.pyx")).read()
    ns = {}
    exec(_pyx_function(src, "read_arma_mat"), ns)
    exec(_pyx_function(src, "read_arma_spMat"), ns)
    import scipy.sparse as sp
    from nlfem_gb300.nlfem import write_arma_spMat, write_arma_mat
    rng = np.random.Generator(np.random.PCG64(11))
    A = sp.random(9, 9, density=0.4, random_state=np.random.RandomState(5), format="csr")
    f = rng.standard_normal(9)
    with tempfile.TemporaryDirectory() as d:
        write_arma_spMat(os.path.join(d, "A"), A)
        write_arma_mat(os.path.join(d, "f"), f)
        B = ns["read_arma_spMat"](os.path.join(d, "A"))
        g = ns["read_arma_mat"](os.path.join(d, "f"))[:, 0]
    return {"A_dense": A.toarray(), "B_dense": B.toarray(), "f": f, "g": g}


def main(ref):
    q = quadrules(ref)
    json.dump(q, open(os.path.join(HERE, "quadrules_ref.json"), "w"), indent=1)
    np.savez_compressed(os.path.join(HERE, "tensorgauss_ref.npz"), **tensorgauss(ref))
    json.dump(vertexlabels(ref), open(os.path.join(HERE, "vertexlabels_ref.json"), "w"))
    json.dump({"n_cells": 3, "tets": tets(ref)}, open(os.path.join(HERE, "tets_ref.json"), "w"))
    np.savez_compressed(os.path.join(HERE, "arma_ref.npz"), **arma(ref))
    print("fixtures written to", HERE)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: python tests/golden/make_golden.py <reference checkout>")
    main(sys.argv[1])
