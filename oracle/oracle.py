"""ctypes front-end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle restates the reference's FP64 assembly (see nlfem_oracle.cpp for the file:line map).
Only tests, the smoke check and bench.py's CPU-baseline/reference arm use it, and only as the
checker or the timed CPU baseline; the product path never imports it.

Parity of the assembled values is unpinned by the reference's own tests (they hold no golden
assembled matrices and the reference cannot be built here); see nlfem_oracle.cpp.
"""
import ctypes
import os
import subprocess

import numpy as np
import scipy.sparse as sp

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "libnlfem_oracle.so")
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
_lp = ctypes.POINTER(ctypes.c_long)
_ip = ctypes.POINTER(ctypes.c_int)


class _Result(ctypes.Structure):
    _fields_ = [("K", ctypes.c_long), ("nnz", ctypes.c_long),
                ("indptr", _lp), ("indices", _lp), ("values", _dp), ("fd", _dp),
                ("n_pairs", ctypes.c_long), ("n_candidates", ctypes.c_long),
                ("n_close", ctypes.c_long), ("n_errors", ctypes.c_long),
                ("pairs", _lp), ("seconds", ctypes.c_double)]


def build(force=False):
    """Compile the oracle shared library with its Makefile (gcc, -ffp-contract=off)."""
    src = os.path.join(_HERE, "nlfem_oracle.cpp")
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB


def lib():
    global _lib
    if _lib is None:
        build()
        l = ctypes.CDLL(_LIB)
        l.oracle_par_assemble.restype = ctypes.POINTER(_Result)
        l.oracle_par_assemble.argtypes = [
            ctypes.c_char_p, ctypes.c_int, _lp, _lp, _dp, _lp, ctypes.c_int, ctypes.c_int,
            _dp, ctypes.c_int, _dp, _dp, ctypes.c_int, _dp,
            ctypes.c_double, ctypes.c_int, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p,
            ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
            _dp, ctypes.c_int, _dp, ctypes.c_double, ctypes.c_int, ctypes.c_int, _lp,
            ctypes.c_long, ctypes.c_int]
        l.oracle_free.argtypes = [ctypes.POINTER(_Result)]
        l.oracle_retriangulate.restype = ctypes.c_int
        l.oracle_retriangulate.argtypes = [_dp, _dp, ctypes.c_double, _dp, ctypes.c_int]
        l.oracle_toRef.restype = ctypes.c_int
        l.oracle_toRef.argtypes = [_dp, _dp, _dp]
        l.oracle_pair_blocks.restype = ctypes.c_int
        l.oracle_pair_blocks.argtypes = [
            _lp, _lp, _dp, ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int, _dp, _dp,
            ctypes.c_int, _dp, ctypes.c_double, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int,
            ctypes.c_int, _dp, ctypes.c_int, _dp, ctypes.c_double, _lp, ctypes.c_long, _dp, _ip]
        l.oracle_set_zeta.restype = None
        l.oracle_set_zeta.argtypes = [_lp, _lp, ctypes.c_long]
        l.oracle_evaluate_mass.restype = ctypes.c_int
        l.oracle_evaluate_mass.argtypes = [_dp, _dp, _lp, _lp, _dp, _lp, ctypes.c_int, ctypes.c_int, _dp, _dp,
                                           ctypes.c_int, ctypes.c_int, ctypes.c_int]
        _lib = l
    return _lib


def _d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(_dp)


def _l(a):
    a = np.ascontiguousarray(a, dtype=np.int64)
    return a, a.ctypes.data_as(_lp)


def _null_d():
    return ctypes.cast(None, _dp)


def assemble(mesh, kernel, conf, compute="system", load=None, nthreads=1, subset=None,
             want_pairs=False):
    """Oracle par_assemble. Returns dict with 'A' (CSR) or 'f', plus counters and pairs."""
    keep = []
    el, elp = _l(mesh["elements"]); keep.append(el)
    elab, elabp = _l(mesh["elementLabels"]); keep.append(elab)
    ve, vep = _d(mesh["vertices"]); keep.append(ve)
    vlab, vlabp = _l(mesh["vertexLabels"]); keep.append(vlab)
    dim = el.shape[1] - 1
    nE, nV = el.shape[0], ve.shape[0]
    q = conf["quadrature"]
    Px, Pxp = _d(q["outer"]["points"]); dx, dxp = _d(q["outer"]["weights"])
    if compute == "forcing":
        Py, Pyp, dy, dyp = Px, Pxp, dx, dxp
    else:
        Py, Pyp = _d(q["inner"]["points"]); dy, dyp = _d(q["inner"]["weights"])
    keep += [Px, dx, Py, dy]
    is_dg = conf.get("ansatz", "CG") == "DG"
    # outdim: the kernel's outputdim for the system, the mesh's for the forcing (nlfem.pyx:220-238)
    outdim = int(kernel.get("outputdim", 1)) if (compute == "system" and kernel) else int(mesh.get("outdim", 1))
    K = (nE * (dim + 1) if is_dg else nV) * outdim
    deg = int(q.get("tensorGaussDegree", 0)) if compute == "system" else 0
    Pgp, dgp = _null_d(), _null_d()
    if deg:
        from nlfem_gb300.quadrules import tensorgauss
        tg = tensorgauss(deg)
        Pg, Pgp = _d(tg.points.ravel()); dg, dgp = _d(tg.weights); keep += [Pg, dg]
    sub = None
    subp = ctypes.cast(None, _lp)
    if subset is not None:
        sub, subp = _l(subset); keep.append(sub)
    remote = conf["approxBalls"]["method"] if compute == "system" else ""
    close = conf.get("closeElements", remote) if compute == "system" else ""
    kname = kernel["function"] if (compute == "system" and kernel) else ""
    fname = load["function"] if (compute == "forcing" and load) else ""
    sqdelta = float(kernel["horizon"]) ** 2 if (compute == "system" and kernel) else 0.0
    caps = int(conf["approxBalls"].get("is_PlacePointOnCap", 1))
    s = kernel.get("fractional_s", -1.0) if kernel else -1.0
    full = int(conf.get("is_fullConnectedComponentSearch", 0))
    # domain decomposition (nlfem.pyx:204-214): mesh["nZeta"] > 0 with mesh["ZetaIndicator"] (CSR)
    nZeta = int(mesh.get("nZeta", 0) or 0)
    if nZeta > 0:
        Z = mesh["ZetaIndicator"]
        zi, zip_ = _l(np.asarray(Z.indices)); zp, zpp = _l(np.asarray(Z.indptr))
        keep += [zi, zp]
        lib().oracle_set_zeta(zip_, zpp, nZeta)
    else:
        lib().oracle_set_zeta(ctypes.cast(None, _lp), ctypes.cast(None, _lp), 0)
    r = lib().oracle_par_assemble(
        compute.encode(), K, elp, elabp, vep, vlabp, nE, nV,
        Pxp, Px.shape[0], dxp, Pyp, Py.shape[0], dyp, sqdelta, int(is_dg),
        kname.encode(), fname.encode(), remote.encode(), close.encode(), caps, dim, outdim,
        Pgp, deg, dgp, float(s), full, int(nthreads), subp,
        0 if sub is None else len(sub), int(want_pairs))
    if not r:
        raise ValueError("oracle: unsupported configuration")
    res = r.contents
    out = {"K": res.K, "n_pairs": res.n_pairs, "n_candidates": res.n_candidates,
           "n_close": res.n_close, "n_errors": res.n_errors, "seconds": res.seconds}
    try:
        if compute == "forcing":
            out["f"] = np.ctypeslib.as_array(res.fd, shape=(K,)).copy()
        else:
            nnz = res.nnz
            indptr = np.ctypeslib.as_array(res.indptr, shape=(K + 1,)).copy()
            if nnz:
                indices = np.ctypeslib.as_array(res.indices, shape=(nnz,)).copy()
                values = np.ctypeslib.as_array(res.values, shape=(nnz,)).copy()
            else:
                indices = np.zeros(0, np.int64)
                values = np.zeros(0)
            out["A"] = sp.csr_matrix((values, indices, indptr), shape=(K, K))
            if want_pairs and res.n_pairs:
                out["pairs"] = np.ctypeslib.as_array(res.pairs, shape=(res.n_pairs, 2)).copy()
    finally:
        lib().oracle_free(r)
    return out


def retriangulate(x, TE, delta, caps=1):
    """Oracle method_retriangulate on one (center, triangle): returns (n_sub, (n_sub,3,2))."""
    x, xp = _d(x); TE, TEp = _d(TE)
    out = np.zeros(9 * 3 * 2)
    n = lib().oracle_retriangulate(xp, TEp, float(delta) ** 2, out.ctypes.data_as(_dp), int(caps))
    return n, out[: 6 * n].reshape(n, 3, 2)


def retriangulate_sq(x, TE, sqdelta, caps=1):
    x, xp = _d(x); TE, TEp = _d(TE)
    out = np.zeros(9 * 3 * 2)
    n = lib().oracle_retriangulate(xp, TEp, float(sqdelta), out.ctypes.data_as(_dp), int(caps))
    return n, out[: 6 * n].reshape(n, 3, 2)


def pair_blocks(mesh, kernel, conf, pairs, method=None):
    """Oracle local blocks (n, 4, dV, dV) for explicit (aT, bT) pairs and doesInteract flags."""
    el, elp = _l(mesh["elements"]); elab, elabp = _l(mesh["elementLabels"])
    ve, vep = _d(mesh["vertices"])
    dim = el.shape[1] - 1
    q = conf["quadrature"]
    Px, Pxp = _d(q["outer"]["points"]); dx, dxp = _d(q["outer"]["weights"])
    Py, Pyp = _d(q["inner"]["points"]); dy, dyp = _d(q["inner"]["weights"])
    deg = int(q.get("tensorGaussDegree", 0))
    Pgp, dgp = _null_d(), _null_d()
    keep = []
    if deg:
        from nlfem_gb300.quadrules import tensorgauss
        tg = tensorgauss(deg)
        Pg, Pgp = _d(tg.points.ravel()); dg, dgp = _d(tg.weights); keep += [Pg, dg]
    pr, prp = _l(np.asarray(pairs).reshape(-1, 2))
    n = pr.shape[0]
    dV = dim + 1
    out = np.zeros((n, 4, dV, dV))
    ret = np.zeros(n, dtype=np.int32)
    meth = method or conf["approxBalls"]["method"]
    lib().oracle_pair_blocks(
        elp, elabp, vep, el.shape[0], ve.shape[0], Pxp, Px.shape[0], dxp, Pyp, Py.shape[0], dyp,
        float(kernel["horizon"]) ** 2, kernel["function"].encode(), meth.encode(),
        int(conf["approxBalls"].get("is_PlacePointOnCap", 1)), dim, Pgp, deg, dgp,
        float(kernel.get("fractional_s", -1.0)), prp, n, out.ctypes.data_as(_dp),
        ret.ctypes.data_as(_ip))
    return out, ret


def evaluate_mass(mesh, ud, Px, dx, J=None, outdim=1, is_dg=False):
    """par_evaluateMass (Cassemble.cpp:166-246) on a mesh dict: vd = M ud over the first J
    elements with label > 0 (J defaults to the number of such elements, as nE_Omega)."""
    el, pel = _l(mesh["elements"])
    lab, plab = _l(mesh["elementLabels"])
    V, pV = _d(mesh["vertices"])
    vl, pvl = _l(mesh["vertexLabels"])
    P, pP = _d(Px)
    w, pw = _d(dx)
    u, pu = _d(ud)
    dim = V.shape[1]
    K = (dim + 1) * el.shape[0] if is_dg else V.shape[0]
    vd = np.zeros(K * outdim)
    J = int((lab > 0).sum()) if J is None else int(J)
    lib().oracle_evaluate_mass(vd.ctypes.data_as(_dp), pu, pel, plab, pV, pvl, J, P.shape[0], pP, pw, dim,
                               outdim, int(is_dg))
    return vd
