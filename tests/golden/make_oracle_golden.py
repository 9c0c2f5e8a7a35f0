"""Oracle fixtures of small assembly cases: tests/golden/oracle_cases.npz.

Run here or anywhere the oracle builds (the reference checkout is not needed):
    python tests/golden/make_oracle_golden.py

Each case stores:
* the mesh arrays, so a host with another numpy assembles the same bits;
* the oracle's CSR (indptr, indices, data);
* the load vector, where the case has a forcing;
* the SHA-256 of the sorted pair list;
* the SHA-256 of the inputs (mesh arrays, kernel, configuration).

The cases are meshes and configurations that the GPU parity tests also assemble. So the fixtures
pin the oracle against drift (tests/test_oracle.py) and give the GPU tests a committed reference
(tests/test_gpu_parity.py).
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

OUT = os.path.join(HERE, "oracle_cases.npz")


def cases():
    """name -> (mesh, kernel, configuration, load or None)."""
    from conftest import conf2d, conf3d, square_mesh, cube_mesh
    kc = {"function": "constant", "horizon": 0.1, "outputdim": 1}
    return {
        # 2D constant kernel, n = 32, delta = 0.1: the configuration the C1 workload names
        "config1": (square_mesh(32, 0.1), kc, conf2d(), {"function": "linear"}),
        # unjittered n = 8: element centroids at distance delta from grid lines (tangent spheres)
        "tangent": (square_mesh(8, 0.1), kc, conf2d(), {"function": "linear"}),
        "parabola20": (square_mesh(20, 0.15, jitter=0.2, seed=4),
                       {"function": "parabola", "horizon": 0.15, "outputdim": 1}, conf2d(), None),
        "frac12": (square_mesh(12, 0.2),
                   {"function": "fractional", "horizon": 0.2, "outputdim": 1, "fractional_s": 0.4},
                   conf2d(rule="16", close="fractional", deg=3), None),
        "cube5": (cube_mesh(5, 0.1, jitter=0.15, seed=2),
                  {"function": "constant3D", "horizon": 0.3, "outputdim": 1}, conf3d(), {"function": "linear3D"}),
        # the rows beyond the reference's default configuration (the CPU pin covers these; the
        # GPU compares against the first five)
        "labeled10": (_labeled_mesh(10, 14), {"function": "labeled", "horizon": 0.1, "outputdim": 1}, conf2d(), None),
        "average10": (square_mesh(10, 0.1, jitter=0.15, seed=12), kc, conf2d(method="averageBall"), None),
        "exact8": (square_mesh(8, 0.1, jitter=0.15, seed=12), kc, conf2d(method="exactBall"), None),
        "dg10": (square_mesh(10, 0.1, jitter=0.15, seed=14),
                 {"function": "parabola", "horizon": 0.1, "outputdim": 1}, dict(conf2d(), ansatz="DG"),
                 {"function": "linear"}),
        "weak10": (square_mesh(10, 0.1, jitter=0.15, seed=9),
                   {"function": "linearPrototypeMicroelastic", "horizon": 0.1, "outputdim": 1, "fractional_s": -0.5},
                   conf2d(rule="16", close="weakSingular", deg=3), None),
        "field8": (dict(square_mesh(8, 0.1, jitter=0.15, seed=3), outdim=2),
                   {"function": "constantField", "horizon": 0.1, "outputdim": 2}, conf2d(), {"function": "constantBothField"}),
        "linf8": (square_mesh(8, 0.1, jitter=0.15, seed=3), {"function": "constantLinf2D", "horizon": 0.1, "outputdim": 1},
                  conf2d(method="retriangulateLinfty"), None),
    }


def _labeled_mesh(n, seed):
    """Labels 3 (x0 < 0.5) and 4 in Omega, -1 in the layer, everything moved by -0.5."""
    from nlfem_gb300 import meshes
    v, e, l = meshes.regular_square(n, 0.1, jitter=0.1, seed=seed)
    bx = v[e].mean(axis=1)[:, 0]
    lab = np.where(l > 0, np.where(bx < 0.5, 3, 4), -1)
    return meshes.mesh_dict(v - 0.5, e, lab)


def input_hash(mesh, kernel, conf):
    h = hashlib.sha256()
    for k in ("elements", "elementLabels", "vertices", "vertexLabels"):
        h.update(np.ascontiguousarray(mesh[k]).tobytes())
    q = conf["quadrature"]
    for part in ("outer", "inner"):
        h.update(np.ascontiguousarray(q[part]["points"], dtype=np.float64).tobytes())
        h.update(np.ascontiguousarray(q[part]["weights"], dtype=np.float64).tobytes())
    rest = {k: v for k, v in conf.items() if k != "quadrature"}
    rest["tensorGaussDegree"] = q.get("tensorGaussDegree", 0)
    h.update(json.dumps([kernel, rest], sort_keys=True).encode())
    return h.hexdigest()


def pair_hash(pairs):
    p = np.asarray(pairs, dtype=np.int64)
    p = p[np.lexsort((p[:, 1], p[:, 0]))]
    return hashlib.sha256(np.ascontiguousarray(p).tobytes()).hexdigest()


def compute(name, case):
    from oracle import oracle
    mesh, kernel, conf, load = case
    r = oracle.assemble(mesh, kernel, conf, want_pairs=True)
    A = r["A"]
    out = {f"{name}.{k}": np.asarray(mesh[k]) for k in ("elements", "elementLabels", "vertices", "vertexLabels")}
    out.update({f"{name}.indptr": A.indptr.astype(np.int64), f"{name}.indices": A.indices.astype(np.int32),
           f"{name}.data": A.data, f"{name}.pairs_sha": np.array(pair_hash(r["pairs"])),
           f"{name}.input_sha": np.array(input_hash(mesh, kernel, conf))})
    if load is not None:
        out[f"{name}.f"] = oracle.assemble(mesh, None, conf, compute="forcing", load=load)["f"]
    return out


def main():
    arrays = {}
    for name, case in cases().items():
        arrays.update(compute(name, case))
    np.savez_compressed(OUT, **arrays)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
