"""L2 convergence rates of the solved nonlocal problem (examples/test2D/computeRates2D.py:17-111).

The reference's rate test assembles A and f on a sequence of meshes and solves
A_Omega u = f_Omega - A_Gamma g, with the Dirichlet data g = u_exact on the interaction layer, by
CG. It then measures the L2 error of the discrete solution and reports log2 of successive error
ratios. This module does the same with this package's GPU assembly (either precision). Two error
measures are reported: the L2 norm of u_h - u by a 16-point rule on the host, and the reference's
measure sqrt(d . M d), d the nodal difference, with the GPU mass product (evaluateMass). The
linear solve runs by CG on the host (scipy) or, with solver="gpu", on the GPU on the session's
assembled matrix.

The default problem is the reference's "linear" load f = -2 (x_1 + 1) (model.cpp:240-242) with
the constant kernel. That kernel reproduces -Laplace on cubic polynomials, so the nonlocal
solution is u(x) = x_0^2 x_1 + x_1^2 and the error is pure discretisation error.
"""
import numpy as np

from . import meshes, nlfem, quadrules


def u_quadratic(x):
    return x[..., 0] ** 2 * x[..., 1] + x[..., 1] ** 2


def l2_error(mesh, uh, u_exact, rule=None):
    """L2 norm over the elements with label > 0 of u_h - u_exact, u_h the P1 function with
    vertex values uh; the element quadrature is the 16-point rule unless given."""
    P, w = rule if rule is not None else quadrules.dunavant16()
    P = np.asarray(P, dtype=np.float64)
    w = np.asarray(w, dtype=np.float64)
    E = mesh["elements"][mesh["elementLabels"] > 0]
    V = mesh["vertices"]
    X = V[E]                                              # (nT, 3, 2)
    det = np.abs((X[:, 1, 0] - X[:, 0, 0]) * (X[:, 2, 1] - X[:, 0, 1]) -
                 (X[:, 2, 0] - X[:, 0, 0]) * (X[:, 1, 1] - X[:, 0, 1]))
    psi = np.stack([1.0 - P[:, 0] - P[:, 1], P[:, 0], P[:, 1]], axis=1)      # (nq, 3)
    xq = np.einsum("qa,tad->tqd", psi, X)                                     # (nT, nq, 2)
    uhq = np.einsum("qa,ta->tq", psi, uh[E])
    d = uhq - u_exact(xq)
    return float(np.sqrt(np.sum(det[:, None] * w[None, :] * d * d)))


def mass_error(mesh, uh, u_exact, rule=None):
    """sqrt(d . M d) with d = u_exact - u_h at the vertices and M the P1 mass matrix on the
    elements with label > 0 (the reference's error measure, computeRates2D.py:92-97, on the same
    mesh), with the GPU mass product nlfem.evaluateMass."""
    P, w = rule if rule is not None else quadrules.dunavant7()
    d = u_exact(mesh["vertices"]) - uh
    Md = nlfem.evaluateMass(mesh, d, P, w)
    return float(np.sqrt(max(d @ Md, 0.0)))


def solve_gpu(mesh, kernel, conf, load, u_exact, tol=1e-12):
    """The same with the CG iterations on the GPU, on the session's assembled matrix
    (nlfem.Session.solve). Returns (vertex values of u_h, CG iterations)."""
    f = nlfem.loadVector(mesh, load, conf)
    s = nlfem.Session([(mesh, kernel, conf)])
    try:
        s.assemble()
        g = np.where(mesh["vertexLabels"] < 0, u_exact(mesh["vertices"]), 0.0)
        return s.solve(0, f, g, rtol=tol)
    finally:
        s.close()


def solve(mesh, kernel, conf, load, u_exact, tol=1e-12):
    """Assemble on the GPU, impose g = u_exact on the layer vertices, solve by CG on the host.
    Returns (vertex values of u_h, CG iterations)."""
    from scipy.sparse.linalg import cg
    A = nlfem.stiffnessMatrix(mesh, kernel, conf).tocsr()
    f = nlfem.loadVector(mesh, load, conf)
    lab = mesh["vertexLabels"]
    om, ga = lab > 0, lab < 0
    A_O = A[om][:, om]
    A_I = A[om][:, ga]
    g = u_exact(mesh["vertices"][ga])
    rhs = f[om] - A_I @ g
    it = [0]

    def count(_):
        it[0] += 1
    try:
        x, info = cg(A_O, rhs, x0=np.zeros_like(rhs), rtol=tol, maxiter=20000, callback=count)
    except TypeError:   # scipy < 1.12
        x, info = cg(A_O, rhs, x0=np.zeros_like(rhs), tol=tol, maxiter=20000, callback=count)
    if info != 0:
        raise RuntimeError(f"CG did not converge (info={info})")
    uh = np.zeros(mesh["vertices"].shape[0])
    uh[om] = x
    uh[ga] = g
    return uh, it[0]


def convergence(ns, delta=0.1, precision="fp64", kernel=None, load=None, u_exact=u_quadratic, rule="7",
                solver="host"):
    """L2 errors and rates over the meshes 2*n^2 (n in ns) of [-delta, 1+delta]^2."""
    kernel = kernel or {"function": "constant", "horizon": delta, "outputdim": 1}
    load = load or {"function": "linear"}
    P, w = quadrules.dunavant7() if rule == "7" else quadrules.dunavant16()
    conf = {"ansatz": "CG", "approxBalls": {"method": "retriangulate", "is_PlacePointOnCap": 1},
            "quadrature": {"outer": {"points": P, "weights": w}, "inner": {"points": P, "weights": w}},
            "precision": precision}
    hs, errs, merrs, its = [], [], [], []
    for n in ns:
        v, e, l = meshes.regular_square(n, delta)
        mesh = meshes.mesh_dict(v, e, l)
        uh, k = (solve_gpu if solver == "gpu" else solve)(mesh, kernel, conf, load, u_exact)
        hs.append((1.0 + 2.0 * delta) / n)
        errs.append(l2_error(mesh, uh, u_exact))
        merrs.append(mass_error(mesh, uh, u_exact))
        its.append(k)
    rates = [float(np.log2(errs[i - 1] / errs[i])) for i in range(1, len(errs))]
    mrates = [float(np.log2(merrs[i - 1] / merrs[i])) for i in range(1, len(merrs))]
    return {"n": list(ns), "h": hs, "l2_error": errs, "rates": rates, "mass_error": merrs,
            "mass_rates": mrates, "cg_iterations": its}


if __name__ == "__main__":
    import json
    import sys
    ns = [int(a) for a in sys.argv[1:]] or [16, 32, 64, 128]
    for prec in ("fp64", "mixed"):
        print(prec, json.dumps(convergence(ns, precision=prec)))
