"""ctypes front-end of the reference's own C++ assembly (TEST INFRASTRUCTURE ONLY).

oracle/ref.mk compiles the reference's src/{Cassemble,integration,model,MeshTypes,mathhelpers}.cpp,
unmodified, against the project-written stand-ins in oracle/refshim/ (an Armadillo subset, the
two METIS calls, CGAL types) into oracle/_ref/libnlfem_ref.so. It pins the CPU restatement
(oracle/nlfem_oracle.cpp) and the committed fixtures to what the reference itself computes.

The build needs the reference's sources, which exist only where the reference checkout is
present; elsewhere available() is False and the callers fall back to the committed fixtures.
assemble() mirrors nlfem.pyx's stiffnessMatrix / loadVector (nlfem.pyx:128-389): the same
derived sizes and arguments to par_assemble, with "mem:" result paths instead of temporary files.
"""
import ctypes
import os
import subprocess

import numpy as np
import scipy.sparse as sp

_HERE = os.path.dirname(os.path.abspath(__file__))
_OUT = os.path.join(_HERE, "_ref")
_LIB = os.path.join(_OUT, "libnlfem_ref.so")
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
_lp = ctypes.POINTER(ctypes.c_long)
_up = ctypes.POINTER(ctypes.c_ulonglong)


def build(ref_path, force=False):
    """Compile the reference against the stand-ins (make -f ref.mk REF=ref_path)."""
    if not os.path.isdir(os.path.join(ref_path, "src")):
        raise FileNotFoundError(f"no reference sources under {ref_path}")
    args = ["make", "-s", "-j8", "-f", os.path.join(_HERE, "ref.mk"), f"REF={os.path.abspath(ref_path)}"]
    if force:
        subprocess.run(args + ["clean"], check=True)
    subprocess.run(args, check=True)
    return _LIB


def available():
    return os.path.exists(_LIB)


def lib():
    global _lib
    if _lib is None:
        if not available():
            raise FileNotFoundError("the reference build oracle/_ref/libnlfem_ref.so is missing (oracle/ref.mk)")
        l = ctypes.CDLL(_LIB)
        l.ref_par_assemble.restype = ctypes.c_double
        l.ref_par_assemble.argtypes = [
            ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int,
            _lp, _lp, _dp, _lp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
            _dp, ctypes.c_int, _dp, _dp, ctypes.c_int, _dp, ctypes.c_double, ctypes.c_int, ctypes.c_int,
            ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int,
            ctypes.c_int, _lp, _lp, ctypes.c_long, _dp, ctypes.c_int, _dp, ctypes.c_double, ctypes.c_double,
            ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_long]
        l.ref_take_sparse.restype = ctypes.c_long
        l.ref_take_sparse.argtypes = [ctypes.c_char_p, _up, _up]
        l.ref_copy_sparse.restype = ctypes.c_int
        l.ref_copy_sparse.argtypes = [ctypes.c_char_p, _dp, _up, _up]
        l.ref_take_dense.restype = ctypes.c_long
        l.ref_take_dense.argtypes = [ctypes.c_char_p, _up, _up]
        l.ref_copy_dense.restype = ctypes.c_int
        l.ref_copy_dense.argtypes = [ctypes.c_char_p, _dp]
        l.ref_evaluate_mass.restype = None
        l.ref_evaluate_mass.argtypes = [_dp, _dp, _lp, _lp, _dp, _lp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        _dp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        l.ref_retriangulate.restype = ctypes.c_int
        l.ref_retriangulate.argtypes = [_dp, _dp, ctypes.c_double, _dp, ctypes.c_int]
        for name in ("ref_toRef", "ref_solve2x2"):
            getattr(l, name).restype = None
            getattr(l, name).argtypes = [_dp, _dp, _dp]
        l.ref_toPhys.restype = None
        l.ref_toPhys.argtypes = [_dp, _dp, ctypes.c_int, _dp]
        _lib = l
    return _lib


def _d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(_dp)


def _l(a):
    a = np.ascontiguousarray(a, dtype=np.int64)
    return a, a.ctypes.data_as(_lp)


def assemble(mesh, kernel, conf, compute="system", load=None, nthreads=1, stack_mb=512):
    """par_assemble of the reference on a mesh dict; returns {'A': CSR} or {'f': ndarray}, plus
    'seconds' (wall time of par_assemble). nthreads sets the OpenMP team (1 gives the canonical
    single-thread summation order)."""
    keep = []
    el, elp = _l(mesh["elements"]); keep.append(el)
    elab, elabp = _l(mesh["elementLabels"]); keep.append(elab)
    ve, vep = _d(mesh["vertices"]); keep.append(ve)
    vlab, vlabp = _l(mesh["vertexLabels"]); keep.append(vlab)
    dim = el.shape[1] - 1
    nE, nV = el.shape[0], ve.shape[0]
    nE_Omega = int(np.sum(elab > 0))
    nV_Omega = int(np.sum(vlab > 0))
    q = conf["quadrature"]
    Px, Pxp = _d(q["outer"]["points"]); dx, dxp = _d(q["outer"]["weights"])
    is_dg = conf.get("ansatz", "CG") == "DG"
    null_l = ctypes.cast(None, _lp)
    null_d = ctypes.cast(None, _dp)
    zi, zp, nZeta = null_l, null_l, 0
    if int(mesh.get("nZeta", 0) or 0) > 0:
        nZeta = int(mesh["nZeta"])
        a, zi = _l(np.asarray(mesh["ZetaIndicator"].indices)); keep.append(a)
        b, zp = _l(np.asarray(mesh["ZetaIndicator"].indptr)); keep.append(b)
    if compute == "system":
        Py, Pyp = _d(q["inner"]["points"]); dy, dyp = _d(q["inner"]["weights"])
        outdim = int(kernel.get("outputdim", 1))
        deg = int(q.get("tensorGaussDegree", 0))
        Pgp, dgp = null_d, null_d
        if deg:
            from nlfem_gb300.quadrules import tensorgauss
            tg = tensorgauss(deg)
            Pg, Pgp = _d(tg.points.ravel()); dg, dgp = _d(tg.weights); keep += [Pg, dg]
        remote = conf["approxBalls"]["method"]
        close = conf.get("closeElements", remote)
        caps = int(conf["approxBalls"].get("is_PlacePointOnCap", 1))
        args = (b"system", b"mem:A", b"", kernel["function"].encode(), b"", remote.encode(), close.encode(),
                caps, float(kernel["horizon"]) ** 2, Pyp, Py.shape[0], dyp, outdim, Pgp, deg, dgp,
                float(mesh.get("diam", 0.0)), float(kernel.get("fractional_s", -1.0)),
                int(conf.get("is_fullConnectedComponentSearch", 0)))
    else:
        outdim = int(mesh.get("outdim", 1))
        args = (b"forcing", b"", b"mem:f", b"", load["function"].encode(), b"", b"", 0, 0.0, Pxp, Px.shape[0],
                dxp, outdim, null_d, 0, null_d, 0.0, -1.0, 0)
    (comp, pA, pf, kname, fname, remote, close, caps, sqdelta, Pyp, nPy, dyp, outdim, Pgp, deg, dgp, diam, s,
     full) = args
    if is_dg:
        K, K_Omega = nE * (dim + 1) * outdim, nE_Omega * (dim + 1) * outdim
    else:
        K, K_Omega = nV * outdim, nV_Omega * outdim
    secs = lib().ref_par_assemble(
        comp, pA, pf, K_Omega, K, elp, elabp, vep, vlabp, nE, nE_Omega, nV, nV_Omega,
        Pxp, Px.shape[0], dxp, Pyp, nPy, dyp, sqdelta, int(is_dg), 0, kname, fname, remote, close, caps,
        dim, outdim, zi, zp, nZeta, Pgp, deg, dgp, diam, s, full, int(conf.get("verbose", 0)),
        int(nthreads), int(stack_mb))
    if secs < 0:
        raise RuntimeError("reference: could not start the assembly thread")
    out = {"K": K, "seconds": secs}
    if compute == "system":
        nr, nc = ctypes.c_ulonglong(), ctypes.c_ulonglong()
        nnz = lib().ref_take_sparse(b"A", ctypes.byref(nr), ctypes.byref(nc))
        if nnz < 0:
            raise RuntimeError("reference: no matrix was saved")
        vals = np.empty(nnz); rows = np.empty(nnz, np.uint64); cptr = np.empty(nc.value + 1, np.uint64)
        lib().ref_copy_sparse(b"A", vals.ctypes.data_as(_dp), rows.ctypes.data_as(_up), cptr.ctypes.data_as(_up))
        # the saved matrix is A^T in compressed columns = A in compressed rows (nlfem.pyx:77-99)
        out["A"] = sp.csr_matrix((vals, rows.astype(np.int64), cptr.astype(np.int64)), shape=(K, K))
    else:
        nr, nc = ctypes.c_ulonglong(), ctypes.c_ulonglong()
        n = lib().ref_take_dense(b"f", ctypes.byref(nr), ctypes.byref(nc))
        if n < 0:
            raise RuntimeError("reference: no load vector was saved")
        f = np.empty(n)
        lib().ref_copy_dense(b"f", f.ctypes.data_as(_dp))
        out["f"] = f.reshape(nc.value, nr.value).T[:, 0].copy()
    return out


def evaluate_mass(mesh, ud, Px, dx, J=None, outdim=1, is_dg=False):
    """par_evaluateMass (Cassemble.cpp:166-246) of the reference on a mesh dict."""
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
    K_Omega = int((vl > 0).sum()) * outdim
    lib().ref_evaluate_mass(vd.ctypes.data_as(_dp), pu, pel, plab, pV, pvl, K_Omega, J, P.shape[0], pP, pw, dim,
                            outdim, int(is_dg))
    return vd


def retriangulate_sq(x, TE, sqdelta, caps=1):
    x, xp = _d(x); TE, TEp = _d(TE)
    out = np.zeros(9 * 3 * 2 + 12)
    n = lib().ref_retriangulate(xp, TEp, float(sqdelta), out.ctypes.data_as(_dp), int(caps))
    return n, out[: 6 * n].reshape(n, 3, 2)
