"""GPU checks of nlfem_load_vector_noalloc through the C ABI: two calls in a row, each
bit-identical to nlfem_load_vector on the same mesh; free device memory unchanged by a call after
the first (the entry point is for callers that cannot let a library allocate); and the size limit
of its static scratch. Collected last, so it also runs after the other GPU tests have used the
device."""
import ctypes

import numpy as np
import pytest

from conftest import conf2d, conf3d, cube_mesh, square_mesh

pytestmark = pytest.mark.gpu

MAX_VERTICES = 1 << 20


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from nlfem_gb300 import _lib, nlfem
    return torch, _lib, _lib.load(), nlfem


def _prepare(env, mesh, conf, forcing, dim):
    """Device copies of the mesh and a result buffer, and a function that runs one call on them."""
    torch, _lib, lib, _ = env
    dev = torch.device("cuda:0")
    T = torch.from_numpy(np.ascontiguousarray(mesh["elements"], dtype=np.int64)).to(dev)
    lT = torch.from_numpy(np.ascontiguousarray(mesh["elementLabels"], dtype=np.int64)).to(dev)
    V = torch.from_numpy(np.ascontiguousarray(mesh["vertices"], dtype=np.float64)).to(dev)
    lV = torch.from_numpy(np.ascontiguousarray(mesh["vertexLabels"], dtype=np.int64)).to(dev)
    nE, nV = T.shape[0], V.shape[0]
    fd = torch.full((nV,), np.nan, dtype=torch.float64, device=dev)
    Px = np.ascontiguousarray(conf["quadrature"]["outer"]["points"], dtype=np.float64)
    dx = np.ascontiguousarray(conf["quadrature"]["outer"]["weights"], dtype=np.float64)
    dp = ctypes.POINTER(ctypes.c_double)
    stream = torch.cuda.current_stream(dev).cuda_stream
    torch.cuda.synchronize(dev)

    def call():
        fd.fill_(np.nan)
        torch.cuda.synchronize(dev)
        r = lib.nlfem_load_vector_noalloc(dim, nE, nV, T.data_ptr(), lT.data_ptr(), V.data_ptr(), lV.data_ptr(),
                                          Px.ctypes.data_as(dp), Px.shape[0], dx.ctypes.data_as(dp),
                                          forcing.encode(), fd.data_ptr(), stream)
        _lib.check(r)

    return call, fd


def _noalloc(env, mesh, conf, forcing, dim):
    call, fd = _prepare(env, mesh, conf, forcing, dim)
    call()
    return fd.cpu().numpy()


def _pow2_edge_mesh():
    """A mesh whose load-vector fixed-point scale 2 (max|x| + 2) |box| / nE is one ulp above a power
    of two: 2^14 triangles on [0, 2 + 2^-51] x [0, 2], so the scale is 2^-9 (1 + 2^-52). A rounded
    log2 gives exactly -9 there and its ceiling -9, the exact ceiling is -8; the ordinary and the
    allocation-free paths must take the same one."""
    from nlfem_gb300 import meshes
    nx, ny = 64, 128
    X, Y = np.meshgrid(np.arange(nx + 1) / 32.0, np.arange(ny + 1) / 64.0, indexing="xy")
    verts = np.stack([X.ravel(), Y.ravel()], axis=1)
    verts[verts[:, 0] == 2.0, 0] = 2.0 + 2.0 ** -51
    j, i = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    c = (j * (nx + 1) + i).ravel()
    elems = np.empty((2 * c.size, 3), dtype=np.int64)
    elems[0::2] = np.stack([c, c + 1, c + 1 + (nx + 1)], axis=1)
    elems[1::2] = np.stack([c, c + 1 + (nx + 1), c + (nx + 1)], axis=1)
    bary = verts[elems].mean(axis=1)
    labels = np.where(np.all((bary > 0.25) & (bary < 1.75), axis=1), 1, -1).astype(np.int64)
    assert elems.shape[0] == 1 << 14
    return meshes.mesh_dict(verts, elems, labels)


def test_noalloc_matches_load_vector_twice(env):
    _, _, _, nl = env
    cases = [
        (square_mesh(40, 0.1, jitter=0.2, seed=5), conf2d(), "linear", 2),
        (cube_mesh(6, 0.2, jitter=0.1, seed=3), conf3d(), "linear3D", 3),
        (square_mesh(17, 0.1, jitter=0.25, seed=11), conf2d(rule="16"), "constant", 2),
        (_pow2_edge_mesh(), conf2d(), "linear", 2),
    ]
    for mesh, conf, forcing, dim in cases:
        want = nl.loadVector(mesh, {"function": forcing}, conf)
        first = _noalloc(env, mesh, conf, forcing, dim)
        second = _noalloc(env, mesh, conf, forcing, dim)
        assert np.array_equal(first.view(np.int64), want.view(np.int64)), forcing
        assert np.array_equal(second.view(np.int64), want.view(np.int64)), forcing


def test_noalloc_call_leaves_free_memory_unchanged(env):
    torch, _, _, nl = env
    mesh, conf = square_mesh(64, 0.1, jitter=0.2, seed=8), conf2d()
    call, fd = _prepare(env, mesh, conf, "linear", 2)
    call()   # the first call on the device may do the one-time set-up
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    call()
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0
    want = nl.loadVector(mesh, {"function": "linear"}, conf)
    assert np.array_equal(fd.cpu().numpy().view(np.int64), want.view(np.int64))


def test_noalloc_rejects_oversize_and_bad_index(env):
    torch, _lib, lib, _ = env
    dev = torch.device("cuda:0")
    dp = ctypes.POINTER(ctypes.c_double)
    from nlfem_gb300 import quadrules
    P, w = quadrules.dunavant7()
    Px = np.ascontiguousarray(P, dtype=np.float64)
    dx = np.ascontiguousarray(w, dtype=np.float64)
    buf = torch.zeros(16, dtype=torch.float64, device=dev)
    # rejected on the host before any device work: the pointers are never read
    r = lib.nlfem_load_vector_noalloc(2, 1, MAX_VERTICES + 1, buf.data_ptr(), buf.data_ptr(), buf.data_ptr(),
                                      buf.data_ptr(), Px.ctypes.data_as(dp), Px.shape[0], dx.ctypes.data_as(dp),
                                      b"linear", buf.data_ptr(), None)
    assert r == 1
    assert b"1048576" in lib.nlfem_last_error()
    # an element that names vertex nV is reported, not read
    mesh = square_mesh(4)
    T = np.ascontiguousarray(mesh["elements"], dtype=np.int64).copy()
    T[int(np.flatnonzero(mesh["elementLabels"] > 0)[0]), 1] = mesh["vertices"].shape[0]
    Td = torch.from_numpy(T).to(dev)
    lT = torch.from_numpy(np.ascontiguousarray(mesh["elementLabels"], dtype=np.int64)).to(dev)
    V = torch.from_numpy(np.ascontiguousarray(mesh["vertices"], dtype=np.float64)).to(dev)
    lV = torch.from_numpy(np.ascontiguousarray(mesh["vertexLabels"], dtype=np.int64)).to(dev)
    fd = torch.zeros(V.shape[0], dtype=torch.float64, device=dev)
    torch.cuda.synchronize(dev)
    r = lib.nlfem_load_vector_noalloc(2, T.shape[0], V.shape[0], Td.data_ptr(), lT.data_ptr(), V.data_ptr(),
                                      lV.data_ptr(), Px.ctypes.data_as(dp), Px.shape[0], dx.ctypes.data_as(dp),
                                      b"linear", fd.data_ptr(), None)
    assert r == 1
    assert b"outside" in lib.nlfem_last_error()
    # and the next good call is still exact
    _, _, _, nl = env
    good = square_mesh(9, 0.1, jitter=0.2, seed=2)
    want = nl.loadVector(good, {"function": "linear"}, conf2d())
    got = _noalloc(env, good, conf2d(), "linear", 2)
    assert np.array_equal(got.view(np.int64), want.view(np.int64))
