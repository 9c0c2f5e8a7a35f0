"""Drop-in Python surface of nlfem (cython/nlfem.pyx of the reference) on the GB300 library.

Same functions, dictionary schema, argument meaning and return types as the reference module:

* ``stiffnessMatrix(mesh, kernel, configuration)`` -> scipy CSR (K, K)      (nlfem.pyx:128-274)
* ``loadVector(mesh, load, configuration)`` -> ndarray (K,)                 (nlfem.pyx:276-389)
* ``stiffnessMatrix_fromArray(elements, elementLabels, vertices, kernel, configuration)``
  -> (mesh, A)                                                               (nlfem.pyx:449-481)
* ``meshFromArrays``, ``get_vertexLabel``, ``get_diam``, ``setSolutionLabels`` (nlfem.pyx:392-446)
* ``tensorgauss``, ``read_arma_mat``, ``read_arma_spMat``, ``timestamp``     (nlfem.pyx:18-126)
* ``py_retriangulate``, ``py_toRef``, ``py_toPhys``, ``py_solve2x2``         (nlfem.pyx:712-771)

The assembly runs on the GPU through the C ABI (include/nlfem_gpu.h) and returns the matrix in
memory instead of through a temporary arma file. Errors raise ``ValueError`` where the
reference raises it (output dimension mismatch, bad arma header) and ``NlfemError`` where the
reference would abort the process.

Extra configuration keys (absent from the reference): ``"precision"``: ``"fp64"`` (default,
the reference's arithmetic), ``"mixed"`` (FP32 quadrature with FP64 cut geometry and FP64
accumulation), or ``"fp64-onesided"`` (the mixed path's algorithm in FP64 arithmetic, 2D
retriangulate only: it separates what the precision costs from what the algorithm saves).
"""
import ctypes
import os
import datetime

import numpy as np
import scipy.sparse as sp

from . import _lib
from .meshes import get_vertexLabel, get_diam, meshFromArrays
from .quadrules import tensorgauss

__all__ = ["stiffnessMatrix", "loadVector", "stiffnessMatrix_fromArray", "meshFromArrays",
           "get_vertexLabel", "get_diam", "setSolutionLabels", "tensorgauss", "read_arma_mat",
           "read_arma_spMat", "timestamp", "py_retriangulate", "py_toRef", "py_toPhys",
           "assemble", "constructAdjaciencyGraph", "remove_arma_tmp",
           "py_solve2x2", "stiffnessMatrix_batch", "pair_list", "pair_blocks", "Session",
           "write_arma_spMat", "write_arma_mat"]

_dp = ctypes.POINTER(ctypes.c_double)
_lp = ctypes.POINTER(ctypes.c_long)
_PRECISIONS = {"fp64": _lib.NLFEM_PREC_FP64, "mixed": _lib.NLFEM_PREC_MIXED,
               "fp64-onesided": _lib.NLFEM_PREC_FP64_ONESIDED}
_ip = ctypes.POINTER(ctypes.c_int)


def timestamp():
    """Current timestamp as string, format %m%d_%H-%M-%S (nlfem.pyx:18-26)."""
    return datetime.datetime.now().strftime("%m%d_%H-%M-%S")


# ---------------------------------------------------------------- arma binary files
def read_arma_mat(path, is_verbose=False):
    """Read an ARMA_MAT_BIN_FN008 file (nlfem.pyx:28-58)."""
    with open(path, "rb") as f:
        if f.readline() != b"ARMA_MAT_BIN_FN008\n":
            raise ValueError("in read_arma_mat(), input file is of wrong format.")
        n_rows, n_cols = (int(x) for x in f.readline().decode("utf-8").split())
        data = f.read()
    return np.frombuffer(data[: 8 * n_rows * n_cols], dtype=np.float64).reshape((n_rows, n_cols), order="F").copy()


def read_arma_spMat(path, is_verbose=False):
    """Read an ARMA_SPM_BIN_FN008 file holding A^T in CSC, return A as CSR (nlfem.pyx:60-101)."""
    with open(path, "rb") as f:
        if f.readline() != b"ARMA_SPM_BIN_FN008\n":
            raise ValueError("in read_arma_spMat(), input file is of wrong format.")
        n_rows, n_cols, nnz = (int(x) for x in f.readline().decode("utf-8").split())
        data = f.read()
    values = np.frombuffer(data[: 8 * nnz], dtype=np.float64)
    ptrs = np.frombuffer(data[8 * nnz:], dtype=np.uint64)
    A = sp.csc_matrix((values, ptrs[:nnz], ptrs[nnz:]), shape=(n_rows, n_cols)).transpose()
    return A.tocsr()


def write_arma_spMat(path, A):
    """Write A (K x K) the way par_system saves it: A^T in CSC = A's CSR arrays."""
    A = sp.csr_matrix(A)
    A.sort_indices()
    with open(path, "wb") as f:
        f.write(b"ARMA_SPM_BIN_FN008\n")
        f.write(f"{A.shape[1]} {A.shape[0]} {A.nnz}\n".encode())
        f.write(np.ascontiguousarray(A.data, dtype=np.float64).tobytes())
        f.write(np.ascontiguousarray(A.indices, dtype=np.uint64).tobytes())
        f.write(np.ascontiguousarray(A.indptr, dtype=np.uint64).tobytes())


def write_arma_mat(path, v):
    v = np.asarray(v, dtype=np.float64).reshape(-1)
    with open(path, "wb") as f:
        f.write(b"ARMA_MAT_BIN_FN008\n")
        f.write(f"{v.shape[0]} 1\n".encode())
        f.write(v.tobytes())


# ---------------------------------------------------------------- problem marshalling
class _Problem:
    """Keeps the numpy arrays alive while the C struct points into them."""

    def __init__(self, mesh, kernel, conf, system=True, load=None):
        self.keep = []
        c = _lib.Problem()
        el = self._l(mesh["elements"])
        c.dim = el.shape[1] - 1
        c.nE = el.shape[0]
        c.elements = el.ctypes.data_as(_lp)
        c.elementLabels = self._l(mesh["elementLabels"]).ctypes.data_as(_lp)
        ve = self._d(mesh["vertices"])
        c.nV = ve.shape[0]
        c.vertices = ve.ctypes.data_as(_dp)
        c.vertexLabels = self._l(mesh["vertexLabels"]).ctypes.data_as(_lp)
        c.outdim = int(mesh.get("outdim", 1)) if not system else int(kernel.get("outputdim", 1))
        c.is_dg = int(conf.get("ansatz", "CG") == "DG")
        q = conf["quadrature"]
        Px = self._d(q["outer"]["points"]); dx = self._d(q["outer"]["weights"])
        c.Px, c.dx, c.nPx = Px.ctypes.data_as(_dp), dx.ctypes.data_as(_dp), dx.shape[0]
        if system:
            Py = self._d(q["inner"]["points"]); dy = self._d(q["inner"]["weights"])
        else:
            Py, dy = Px, dx
        c.Py, c.dy, c.nPy = Py.ctypes.data_as(_dp), dy.ctypes.data_as(_dp), dy.shape[0]
        deg = int(q.get("tensorGaussDegree", 0)) if system else 0
        c.tensorGaussDegree = deg
        if deg:
            tg = tensorgauss(deg)
            Pg = self._d(tg.points.ravel()); dg = self._d(tg.weights)
            c.Pg, c.dg = Pg.ctypes.data_as(_dp), dg.ctypes.data_as(_dp)
        if system:
            c.sqdelta = float(kernel["horizon"]) ** 2
            c.fractional_s = float(kernel.get("fractional_s", -1.0))
            c.kernel = self._s(kernel["function"])
            remote = conf["approxBalls"]["method"]
            c.method_remote = self._s(remote)
            c.method_close = self._s(conf.get("closeElements", remote))
            # The reference reads "is_PlacePointOnCap" (nlfem.pyx:172); configurations that
            # spell it "isPlacePointOnCap" therefore always run with caps (default 1).
            c.is_PlacePointOnCap = int(conf["approxBalls"].get("is_PlacePointOnCap", 1))
            c.is_fullConnectedComponentSearch = int(conf.get("is_fullConnectedComponentSearch", 0))
        else:
            c.forcing = self._s(load["function"])
            c.fractional_s = -1.0
        prec = conf.get("precision", "fp64")
        if prec not in _PRECISIONS:
            raise ValueError("configuration['precision'] must be 'fp64', 'mixed' or 'fp64-onesided'")
        c.precision = _PRECISIONS[prec]
        c.verbose = int(conf.get("verbose", 0))
        # domain decomposition (nlfem.pyx:204-214): mesh["nZeta"] > 0 with the element -> subdomain
        # indicator mesh["ZetaIndicator"] (scipy CSR)
        nZeta = int(mesh.get("nZeta", 0) or 0)
        if nZeta > 0:
            Z = mesh["ZetaIndicator"]
            c.zeta_indices = self._l(np.asarray(Z.indices)).ctypes.data_as(_lp)
            c.zeta_indptr = self._l(np.asarray(Z.indptr)).ctypes.data_as(_lp)
            c.nZeta = nZeta
        self.c = c

    def _l(self, a):
        a = np.ascontiguousarray(a, dtype=np.int64)
        self.keep.append(a)
        return a

    def _d(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        self.keep.append(a)
        return a

    def _s(self, s):
        b = ctypes.c_char_p(s.encode("utf-8"))
        self.keep.append(b)
        return b


def _csr_to_scipy(m):
    K, nnz = m.K, m.nnz
    indptr = np.ctypeslib.as_array(m.indptr, shape=(K + 1,)).copy()
    if nnz:
        indices = np.ctypeslib.as_array(m.indices, shape=(nnz,)).copy()
        values = np.ctypeslib.as_array(m.values, shape=(nnz,)).copy()
    else:
        indices = np.zeros(0, dtype=np.int64)
        values = np.zeros(0)
    return sp.csr_matrix((values, indices, indptr), shape=(K, K))


class _CSR32Owner:
    """Keeps the library's CSR arrays alive until the numpy views on them are collected."""

    def __init__(self, lib, m):
        self.lib, self.m = lib, m

    def __del__(self):
        try:
            self.lib.nlfem_csr32_free(ctypes.byref(self.m))
        except Exception:
            pass


def _view(ptr, n, ctype, dtype, owner):
    if n == 0:
        return np.zeros(0, dtype=dtype)
    buf = (ctype * n).from_address(ctypes.cast(ptr, ctypes.c_void_p).value)
    buf._owner = owner   # the array -> buffer -> owner chain frees the memory with the last view
    return np.frombuffer(buf, dtype=dtype)


def _csr32_to_scipy(lib, m):
    """scipy CSR over the library's 32-bit arrays, without copying them."""
    owner = _CSR32Owner(lib, m)
    K, nnz = int(m.K), int(m.nnz)
    indptr = _view(m.indptr, K + 1, ctypes.c_int, np.int32, owner)
    indices = _view(m.indices, nnz, ctypes.c_int, np.int32, owner)
    values = _view(m.values, nnz, ctypes.c_double, np.float64, owner)
    return sp.csr_matrix((values, indices, indptr), shape=(K, K), copy=False)


# ---------------------------------------------------------------- public API
def stiffnessMatrix(mesh, kernel, configuration):
    """Stiffness matrix of the nonlocal operator on the mesh (nlfem.pyx:128-274), on the GPU."""
    if mesh.get("outdim", kernel["outputdim"]) != kernel["outputdim"]:
        raise ValueError("The output dimension of the mesh has to be equal to the output dimension of the kernel.")
    lib = _lib.load()
    p = _Problem(mesh, kernel, configuration, system=True)
    out32 = _lib.CSR32()
    code = lib.nlfem_stiffness_matrix32(ctypes.byref(p.c), ctypes.byref(out32))
    if code == 0:
        A = _csr32_to_scipy(lib, out32)
    else:
        if code != 4:   # NLFEM_ERR_UNSUPPORTED: 2^31 entries or more, 64-bit indices below
            _lib.check(code)
        out = _lib.CSR()
        _lib.check(lib.nlfem_stiffness_matrix(ctypes.byref(p.c), ctypes.byref(out)))
        try:
            A = _csr_to_scipy(out)
        finally:
            lib.nlfem_csr_free(ctypes.byref(out))
    path = configuration.get("savePath")
    if path:
        write_arma_spMat(path, A)
    return A


def evaluateMass(mesh, ud, Px, dx):
    """vd = M ud with the P1 mass matrix (nlfem.pyx:638-671, par_evaluateMass Cassemble.cpp:166-246),
    on the GPU. mesh is the reference's mesh object (elements, elementLabels, vertices,
    vertexLabels, dim, nE_Omega, is_DiscontinuousGalerkin, optional outdim: the first nE_Omega
    elements with a positive label are summed) or a mesh dict (every element with a positive
    label). Px, dx: the quadrature rule on the reference element."""
    if isinstance(mesh, dict):
        get = mesh.get
    else:
        def get(k, default=None):
            return getattr(mesh, k, default)
    elements = np.ascontiguousarray(get("elements"), dtype=np.int64)
    elementLabels = np.ascontiguousarray(get("elementLabels"), dtype=np.int64).ravel()
    vertices = np.ascontiguousarray(get("vertices"), dtype=np.float64)
    vertexLabels = np.ascontiguousarray(get("vertexLabels"), dtype=np.int64).ravel()
    nE, dV = elements.shape
    nV, dim = vertices.shape
    J = get("nE_Omega")
    J = nE if J is None else int(J)
    is_dg = int(bool(get("is_DiscontinuousGalerkin", False)))
    outdim = int(get("outdim", 1) or 1)
    K = dV * nE if is_dg else nV
    u = np.ascontiguousarray(ud, dtype=np.float64).ravel()
    if u.size != K * outdim:
        raise ValueError(f"ud has {u.size} entries, the mesh has {K * outdim} degrees of freedom")
    P = np.ascontiguousarray(Px, dtype=np.float64)
    w = np.ascontiguousarray(dx, dtype=np.float64).ravel()
    vd = np.zeros(K * outdim, dtype=np.float64)
    lib = _lib.load()
    lp = ctypes.POINTER(ctypes.c_long)
    _lib.check(lib.nlfem_evaluate_mass(dim, outdim, is_dg, nE, J, nV, elements.ctypes.data_as(lp),
                                       elementLabels.ctypes.data_as(lp), vertices.ctypes.data_as(_dp),
                                       vertexLabels.ctypes.data_as(lp), int(w.size), P.ctypes.data_as(_dp),
                                       w.ctypes.data_as(_dp), u.ctypes.data_as(_dp), vd.ctypes.data_as(_dp)))
    return vd


def loadVector(mesh, load, configuration):
    """Load vector (nlfem.pyx:276-389), on the GPU."""
    lib = _lib.load()
    p = _Problem(mesh, None, configuration, system=False, load=load)
    K = (int(p.c.dim) + 1) * int(p.c.nE) if p.c.is_dg else int(p.c.nV)   # DG: element DOFs
    fd = np.zeros(K * int(p.c.outdim), dtype=np.float64)
    _lib.check(lib.nlfem_load_vector(ctypes.byref(p.c), fd.ctypes.data_as(_dp)))
    path = configuration.get("savePath")
    if path:
        write_arma_mat(path, fd)
    return fd


def stiffnessMatrix_batch(problems):
    """Many independent assemblies in one pass: problems = [(mesh, kernel, configuration)]."""
    lib = _lib.load()
    ps = [_Problem(m, k, c, system=True) for (m, k, c) in problems]
    arr = (_lib.Problem * len(ps))(*[p.c for p in ps])
    outs32 = (_lib.CSR32 * len(ps))()
    code = lib.nlfem_stiffness_batch32(arr, len(ps), outs32)
    if code == 0:
        res = []
        for i in range(len(ps)):
            m = _lib.CSR32()
            ctypes.pointer(m)[0] = outs32[i]
            res.append(_csr32_to_scipy(lib, m))
        return res
    if code != 4:
        _lib.check(code)
    outs = (_lib.CSR * len(ps))()
    _lib.check(lib.nlfem_stiffness_batch(arr, len(ps), outs))
    res = []
    for i in range(len(ps)):
        try:
            res.append(_csr_to_scipy(outs[i]))
        finally:
            lib.nlfem_csr_free(ctypes.byref(outs[i]))
    return res


class Session:
    """Device-resident assembly: the meshes are uploaded once, assemble() reruns the pipeline."""

    def __init__(self, problems):
        self.lib = _lib.load()
        self.ps = [_Problem(m, k, c, system=True) for (m, k, c) in problems]
        self.arr = (_lib.Problem * len(self.ps))(*[p.c for p in self.ps])
        self.h = ctypes.c_void_p()
        _lib.check(self.lib.nlfem_session_create(self.arr, len(self.ps), ctypes.byref(self.h)))

    def assemble(self, graph=False):
        """Assemble all problems; graph=True replays a captured CUDA graph after the first call."""
        fn = self.lib.nlfem_session_assemble_graph if graph else self.lib.nlfem_session_assemble
        _lib.check(fn(self.h))
        return _lib.stats()

    def autotune(self, reps=2):
        """Times 1, 2, ... blocks per SM for the pair search and the persistent quadrature pass on
        this session's workload, keeps the fastest for the session (and for later sessions of the
        same device and configuration class), and leaves the matrices assembled with it. Returns
        {"bfs": chosen, "pass": chosen, "bfs_ms": [...], "pass_ms": [...]}."""
        t = _lib.Tuning()
        _lib.check(self.lib.nlfem_session_autotune(self.h, int(reps), ctypes.byref(t)))
        return {"bfs": t.bfs_blocks_per_sm, "pass": t.pass_blocks_per_sm,
                "bfs_ms": list(t.bfs_ms[:t.bfs_candidates]), "pass_ms": list(t.pass_ms[:t.pass_candidates])}

    def download(self, i=0):
        out32 = _lib.CSR32()
        code = self.lib.nlfem_session_download32(self.h, i, ctypes.byref(out32))
        if code == 0:
            return _csr32_to_scipy(self.lib, out32)
        if code != 4:
            _lib.check(code)
        out = _lib.CSR()
        _lib.check(self.lib.nlfem_session_download(self.h, i, ctypes.byref(out)))
        try:
            return _csr_to_scipy(out)
        finally:
            self.lib.nlfem_csr_free(ctypes.byref(out))

    def solve(self, i, f, g, rtol=1e-12, maxit=20000):
        """A_Omega u = f_Omega - A_Gamma g by conjugate gradients on the GPU, on problem i's matrix
        of the last assemble() (computeRates2D.py:47-70). f and g are vertex vectors (g read at
        label < 0); returns (u, iterations) with u = g at label < 0."""
        nV = int(self.ps[i].c.nV)
        ff = np.ascontiguousarray(f, dtype=np.float64).ravel()
        gg = np.ascontiguousarray(g, dtype=np.float64).ravel()
        if ff.size != nV or gg.size != nV:
            raise ValueError(f"f and g need {nV} entries")
        u = np.zeros(nV, dtype=np.float64)
        its = ctypes.c_int(0)
        _lib.check(self.lib.nlfem_session_solve(self.h, i, ff.ctypes.data_as(_dp), gg.ctypes.data_as(_dp),
                                                float(rtol), int(maxit), u.ctypes.data_as(_dp), ctypes.byref(its)))
        return u, its.value

    def close(self):
        if self.h:
            self.lib.nlfem_session_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def stiffnessMatrix_fromArray(elements, elementLabels, vertices, kernel, configuration):
    """Mesh dictionary and stiffness matrix from raw arrays (nlfem.pyx:449-481)."""
    mesh = meshFromArrays(np.asarray(elements), np.asarray(elementLabels), np.asarray(vertices),
                          kernel["outputdim"])
    setSolutionLabels(mesh, configuration.get("ansatz", "CG"), kernel["outputdim"])
    return mesh, stiffnessMatrix(mesh, kernel, configuration)


def remove_arma_tmp(path):
    """Deletes a temporary arma file (nlfem.pyx:103-105)."""
    os.remove(path)


def assemble(mesh, Px, Py, dx, dy, delta, path_spAd=None, path_fd=None, compute="systemforcing",
             model_kernel="constant", model_f="constant", integration_method="retriangulate",
             is_PlacePointOnCap=1, tensorGaussDegree=0):
    """The reference's deprecated interface (nlfem.pyx:483-636). mesh is an object with the
    attributes elements, elementLabels, vertices, vertexLabels, nE, nV, dim, K_Omega and
    is_DiscontinuousGalerkin (optional: outdim, is_fullConnectedComponentSearch); the quadrature
    comes as separate arrays and the horizon as delta. The same integration method serves remote
    and close pairs, and fractional_s is -1, as in the reference. Returns (A[:K_Omega],
    f[:K_Omega]) with None for the part `compute` ("system", "forcing" or "systemforcing") leaves
    out; path_spAd / path_fd keep the full arma files."""
    print("This function is deprecated. Please use stiffnessMatrix()")
    dim = int(mesh.dim)
    outdim = int(getattr(mesh, "outdim", 1))
    m = {"elements": np.asarray(mesh.elements, dtype=np.int64).reshape(int(mesh.nE), dim + 1),
         "elementLabels": np.asarray(mesh.elementLabels, dtype=np.int64).ravel(),
         "vertices": np.asarray(mesh.vertices, dtype=np.float64).reshape(int(mesh.nV), dim),
         "vertexLabels": np.asarray(mesh.vertexLabels, dtype=np.int64).ravel(),
         "outdim": outdim}
    conf = {"ansatz": "DG" if getattr(mesh, "is_DiscontinuousGalerkin", 0) else "CG",
            "approxBalls": {"method": integration_method, "is_PlacePointOnCap": int(is_PlacePointOnCap)},
            "closeElements": integration_method,
            "quadrature": {"outer": {"points": np.asarray(Px, dtype=np.float64).reshape(-1, dim),
                                     "weights": np.asarray(dx, dtype=np.float64).ravel()},
                           "inner": {"points": np.asarray(Py, dtype=np.float64).reshape(-1, dim),
                                     "weights": np.asarray(dy, dtype=np.float64).ravel()},
                           "tensorGaussDegree": int(tensorGaussDegree)},
            "is_fullConnectedComponentSearch": int(getattr(mesh, "is_fullConnectedComponentSearch", 0))}
    K_Omega = int(mesh.K_Omega)
    A = f = None
    if compute in ("system", "systemforcing"):
        kernel = {"function": model_kernel, "horizon": float(delta), "outputdim": outdim, "fractional_s": -1.0}
        A = stiffnessMatrix(m, kernel, dict(conf, savePath=path_spAd) if path_spAd else conf)[:K_Omega]
    if compute in ("forcing", "systemforcing"):
        f = loadVector(m, {"function": model_f}, dict(conf, savePath=path_fd) if path_fd else conf)[:K_Omega]
    return A, f


def constructAdjaciencyGraph(elements, ncommon=1):
    """Deprecated in the reference (nlfem.pyx:678-710): (nE, nCols) neighbour table of the
    elements sharing at least ncommon vertices (each element lists itself), padded with nE. The
    assembly does not need it. Neighbours are listed in ascending order."""
    print("Constructing adjaciency graph...")
    print("This function is deprecated, and its use is not required anymore.")
    el = np.asarray(elements, dtype=np.int64)
    nE, dV = el.shape
    nV = int(el.max()) + 1
    G = sp.csr_matrix((np.ones(nE * dV, dtype=np.int64), (el.ravel(), np.repeat(np.arange(nE), dV))), shape=(nV, nE))
    N = (G.T @ G).tocsr()
    N.data = (N.data > ncommon - 1).astype(np.int64)
    N.eliminate_zeros()
    N.sort_indices()
    counts = np.diff(N.indptr)
    neigs = np.full((nE, int(counts.max())), nE, dtype=np.int64)
    for e in range(nE):
        cols = N.indices[N.indptr[e]:N.indptr[e + 1]]
        neigs[e, :cols.size] = cols
    return neigs


def setSolutionLabels(mesh, ansatz="CG", outputdim=1):
    """Solution labels and K of the ansatz space (nlfem.pyx:436-446)."""
    mesh["ansatz"] = ansatz
    mesh["outputdim"] = outputdim
    if ansatz == "CG":
        mesh["solutionLabels"] = np.repeat(mesh["vertexLabels"], outputdim)
        mesh["K"] = mesh["nV"] * outputdim
        mesh["K_Omega"] = mesh["nV_Omega"] * outputdim
    if ansatz == "DG":
        mesh["solutionLabels"] = np.repeat(mesh["elementLabels"], 3 * outputdim)
        mesh["K"] = 3 * mesh["nE"] * outputdim
        mesh["K_Omega"] = 3 * mesh["nE_Omega"] * outputdim


def pair_list(mesh, kernel, configuration):
    """Interacting ordered pairs (aT, bT) of the BFS, sorted, as an (n, 2) int64 array."""
    lib = _lib.load()
    p = _Problem(mesh, kernel, configuration, system=True)
    n = ctypes.c_long()
    ptr = _lp()
    _lib.check(lib.nlfem_pair_list(ctypes.byref(p.c), ctypes.byref(n), ctypes.byref(ptr)))
    try:
        return np.ctypeslib.as_array(ptr, shape=(n.value, 2)).copy() if n.value else np.zeros((0, 2), np.int64)
    finally:
        ctypes.CDLL(None).free(ptr)


def pair_blocks(mesh, kernel, configuration, pairs, close=False):
    """Local blocks (n, 4, dV, dV) and doesInteract flags of explicit (aT, bT) pairs."""
    lib = _lib.load()
    p = _Problem(mesh, kernel, configuration, system=True)
    pr = np.ascontiguousarray(np.asarray(pairs).reshape(-1, 2), dtype=np.int64)
    n = pr.shape[0]
    dV = p.c.dim + 1
    out = np.zeros((n, 4, dV, dV))
    ret = np.zeros(n, dtype=np.int32)
    _lib.check(lib.nlfem_pair_blocks(ctypes.byref(p.c), n, pr.ctypes.data_as(_lp), int(close),
                                     out.ctypes.data_as(_dp), ret.ctypes.data_as(_ip)))
    return out, ret


# ---------------------------------------------------------------- debug helpers (nlfem.pyx:712-771)
def py_retriangulate(x_center, TE, delta, is_placePointOnCaps, pp=None):
    lib = _lib.load()
    x = np.ascontiguousarray(x_center, dtype=np.float64)
    T = np.ascontiguousarray(TE, dtype=np.float64)
    out = np.zeros(9 * 3 * 2)
    cnt = np.zeros(1, dtype=np.int32)
    _lib.check(lib.nlfem_retriangulate_batch(1, x.ctypes.data_as(_dp), T.ctypes.data_as(_dp),
                                             float(delta) ** 2, int(is_placePointOnCaps),
                                             cnt.ctypes.data_as(_ip), out.ctypes.data_as(_dp)))
    return int(cnt[0]), out


def retriangulate_batch(x_centers, TEs, sqdelta, caps=1):
    """Vectorised method_retriangulate: counts (n,) and sub-triangles (n, 9, 3, 2)."""
    lib = _lib.load()
    x = np.ascontiguousarray(x_centers, dtype=np.float64).reshape(-1, 2)
    T = np.ascontiguousarray(TEs, dtype=np.float64).reshape(-1, 6)
    n = x.shape[0]
    out = np.zeros((n, 9, 3, 2))
    cnt = np.zeros(n, dtype=np.int32)
    _lib.check(lib.nlfem_retriangulate_batch(n, x.ctypes.data_as(_dp), T.ctypes.data_as(_dp),
                                             float(sqdelta), int(caps), cnt.ctypes.data_as(_ip),
                                             out.ctypes.data_as(_dp)))
    return cnt, out


def retriangulate_certified_batch(x_centers, TEs, sqdelta, caps=1):
    """FP32 certified retriangulation: counts (n,), ambiguous (n,), points (n, 9, 2) relative to x."""
    lib = _lib.load()
    x = np.ascontiguousarray(x_centers, dtype=np.float64).reshape(-1, 2)
    T = np.ascontiguousarray(TEs, dtype=np.float64).reshape(-1, 6)
    n = x.shape[0]
    pts = np.zeros((n, 9, 2))
    cnt = np.zeros(n, dtype=np.int32)
    amb = np.zeros(n, dtype=np.int32)
    _lib.check(lib.nlfem_retriangulate_certified_batch(n, x.ctypes.data_as(_dp), T.ctypes.data_as(_dp),
                                                       float(sqdelta), int(caps), cnt.ctypes.data_as(_ip),
                                                       amb.ctypes.data_as(_ip), pts.ctypes.data_as(_dp)))
    return cnt, amb, pts


def py_toRef(TE, phys_x):
    lib = _lib.load()
    T = np.ascontiguousarray(TE, dtype=np.float64); x = np.ascontiguousarray(phys_x, dtype=np.float64)
    out = np.zeros(2)
    _lib.check(lib.nlfem_toRef(T.ctypes.data_as(_dp), x.ctypes.data_as(_dp), out.ctypes.data_as(_dp)))
    return out


def py_toPhys(TE, p):
    lib = _lib.load()
    T = np.ascontiguousarray(TE, dtype=np.float64); q = np.ascontiguousarray(p, dtype=np.float64)
    dim = q.shape[0]
    out = np.zeros(dim)
    _lib.check(lib.nlfem_toPhys(T.ctypes.data_as(_dp), q.ctypes.data_as(_dp), dim, out.ctypes.data_as(_dp)))
    return out


def py_solve2x2(A, b):
    lib = _lib.load()
    Am = np.ascontiguousarray(A, dtype=np.float64); bm = np.ascontiguousarray(b, dtype=np.float64)
    out = np.zeros(2)
    _lib.check(lib.nlfem_solve2x2(Am.ctypes.data_as(_dp), bm.ctypes.data_as(_dp), out.ctypes.data_as(_dp)))
    return out
