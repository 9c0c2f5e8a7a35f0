"""The assembly workloads the benchmark and the full-size parity checks run (synthetic, seeded).

c1: 2D constant kernel, 2*32^2 right-diagonal triangles of [-delta, 1+delta]^2, delta = 0.1.
c2: the same kernel and rules on 2*256^2 triangles with interior vertices jittered by +-0.2h
    (numpy PCG64, seed 1), delta in {0.05, 0.1}.
c3: fractional kernel s = 0.4, 2*128^2 triangles, delta = 0.1; regular pairs retriangulate with the
    16-point rule, close pairs the Duffy tensor Gauss rule of degree 5.
c4: 3D constant kernel, 6*32^3 tetrahedra of [-delta, 1+delta]^3, barycenter ball, 11-point Keast.
c5: 64 independent 2D problems: n from {32, 48, ..., 192}, delta ~ U[0.05, 0.2], half constant and
    half parabola kernel, jittered +-0.2h (PCG64 seed 2024).
All use continuous P1 elements, caps on, 7-point Dunavant rules unless stated. The element labels
are +1 inside [0,1]^d and -1 in the interaction layer; vertex labels follow get_vertexLabel.
"""
from . import meshes, quadrules

FORCING = {"c1": "linear", "c2": "linear", "c3": "linear", "c4": "linear3D", "c5": "linear"}


def _conf2d(rule, precision, close=None, deg=0):
    P, wts = rule
    c = {"ansatz": "CG", "approxBalls": {"method": "retriangulate", "is_PlacePointOnCap": 1},
         "quadrature": {"outer": {"points": P, "weights": wts}, "inner": {"points": P, "weights": wts}},
         "precision": precision}
    if close:
        c["closeElements"] = close
    if deg:
        c["quadrature"]["tensorGaussDegree"] = deg
    return c


def problems(name, precision="mixed", n=None, delta=0.1):
    """([(mesh, kernel, configuration)], record) of a workload; record names it with its sizes."""
    if name in ("c1", "c2"):
        n = n or (32 if name == "c1" else 256)
        jit = 0.0 if name == "c1" else 0.2
        v, e, l = meshes.regular_square(n, delta, jitter=jit, seed=1)
        mesh = meshes.mesh_dict(v, e, l)
        kernel = {"function": "constant", "horizon": delta, "outputdim": 1}
        desc = (f"2D constant kernel, 2*{n}^2 triangles" + (" jittered +-0.2h (seed 1)" if jit else "") +
                f", delta={delta}, retriangulate+caps, 7-pt Dunavant outer/inner, P1 CG")
        return [(mesh, kernel, _conf2d(quadrules.dunavant7(), precision))], {"workload": desc, "n": n, "delta": delta}
    if name == "c3":
        n = n or 128
        v, e, l = meshes.regular_square(n, delta)
        mesh = meshes.mesh_dict(v, e, l)
        kernel = {"function": "fractional", "horizon": delta, "outputdim": 1, "fractional_s": 0.4}
        desc = (f"2D fractional kernel s=0.4, 2*{n}^2 triangles, delta={delta}; regular pairs "
                f"retriangulate+caps with the 16-pt rule, close pairs Duffy tensor Gauss degree 5 (FP64)")
        return ([(mesh, kernel, _conf2d(quadrules.dunavant16(), precision, close="fractional", deg=5))],
                {"workload": desc, "n": n, "delta": delta})
    if name == "c4":
        n = n or 32
        v, e, l = meshes.regular_cube(n, delta)
        mesh = meshes.mesh_dict(v, e, l)
        kernel = {"function": "constant3D", "horizon": delta, "outputdim": 1}
        P, wts = quadrules.keast11()
        conf = {"ansatz": "CG", "approxBalls": {"method": "baryCenter"},
                "quadrature": {"outer": {"points": P, "weights": wts}, "inner": {"points": P, "weights": wts}},
                "precision": precision}
        desc = (f"3D constant kernel, 6*{n}^3 tetrahedra (Kuhn split) of [-delta,1+delta]^3, delta={delta}, "
                f"barycenter ball, 11-pt Keast outer/inner, P1 CG")
        return [(mesh, kernel, conf)], {"workload": desc, "n": n, "delta": delta}
    if name == "c5":
        probs = []
        for b in meshes.batch_meshes(64, seed=2024):
            k = {"function": b["kernel"], "horizon": b["delta"], "outputdim": 1}
            probs.append((b["mesh"], k, _conf2d(quadrules.dunavant7(), precision)))
        desc = ("64 independent 2D problems in one batch: n from {32,48,...,192} (2*n^2 triangles, jittered "
                "+-0.2h), delta ~ U[0.05,0.2], half constant / half parabola kernel, retriangulate+caps, 7-pt rules "
                "(PCG64 seed 2024)")
        return probs, {"workload": desc, "problems": 64}
    raise ValueError(f"unknown workload {name}")
