import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


def conf2d(rule="7", method="retriangulate", close=None, deg=0, caps=1, precision="fp64"):
    from nlfem_gb300 import quadrules
    P, w = quadrules.dunavant7() if rule == "7" else quadrules.dunavant16()
    c = {"ansatz": "CG", "approxBalls": {"method": method, "is_PlacePointOnCap": caps},
         "quadrature": {"outer": {"points": P, "weights": w}, "inner": {"points": P, "weights": w}},
         "precision": precision}
    if close:
        c["closeElements"] = close
    if deg:
        c["quadrature"]["tensorGaussDegree"] = deg
    return c


def conf3d(precision="fp64"):
    from nlfem_gb300 import quadrules
    P, w = quadrules.keast11()
    return {"ansatz": "CG", "approxBalls": {"method": "baryCenter"},
            "quadrature": {"outer": {"points": P, "weights": w}, "inner": {"points": P, "weights": w}},
            "precision": precision}


def square_mesh(n, delta=0.1, jitter=0.0, seed=0):
    from nlfem_gb300 import meshes
    v, e, l = meshes.regular_square(n, delta, jitter=jitter, seed=seed)
    return meshes.mesh_dict(v, e, l)


def cube_mesh(n, delta=0.1, jitter=0.0, seed=0):
    from nlfem_gb300 import meshes
    v, e, l = meshes.regular_cube(n, delta, jitter=jitter, seed=seed)
    return meshes.mesh_dict(v, e, l)


def labeled_mesh(n=14, seed=5):
    """Omega split into labels 3 (x0 < 0.5) and 4, the layer -1, all moved by -0.5 so that the
    notch {x1 = 0, x0 > 0} cuts the right half. Every label pair is a case of the labeled kernel
    (10 lx + ly in {-11, -7, -6, 9, 29, 33, 34, 39, 43, 44}); 3 + 4 = 7 closes labeledNotch."""
    from nlfem_gb300 import meshes
    v, e, l = meshes.regular_square(n, 0.1, jitter=0.1, seed=seed)
    bx = v[e].mean(axis=1)[:, 0]
    lab = np.where(l > 0, np.where(bx < 0.5, 3, 4), -1)
    return meshes.mesh_dict(v - 0.5, e, lab)


def rel_errors(A, B):
    """Relative Frobenius and max-entry errors of A against the reference B."""
    D = (A - B).tocsr()
    fro = np.sqrt((D.multiply(D)).sum()) / np.sqrt((B.multiply(B)).sum())
    mx = abs(D).max() / abs(B).max()
    return float(fro), float(mx)


def same_pattern(A, B):
    A = A.tocsr(); B = B.tocsr()
    A.sort_indices(); B.sort_indices()
    return (A.shape == B.shape and np.array_equal(A.indptr, B.indptr)
            and np.array_equal(A.indices, B.indices))
