"""GPU checks of nlfem_load_vector_noalloc through the C ABI: two calls in a row, each
bit-identical to nlfem_load_vector on the same mesh, and the size limit of its static scratch.
Collected last, so it also runs after the other GPU tests have used the device."""
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


def _noalloc(env, mesh, conf, forcing, dim):
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
    r = lib.nlfem_load_vector_noalloc(dim, nE, nV, T.data_ptr(), lT.data_ptr(), V.data_ptr(), lV.data_ptr(),
                                      Px.ctypes.data_as(dp), Px.shape[0], dx.ctypes.data_as(dp),
                                      forcing.encode(), fd.data_ptr(), stream)
    _lib.check(r)
    return fd.cpu().numpy()


def test_noalloc_matches_load_vector_twice(env):
    _, _, _, nl = env
    cases = [
        (square_mesh(40, 0.1, jitter=0.2, seed=5), conf2d(), "linear", 2),
        (cube_mesh(6, 0.2, jitter=0.1, seed=3), conf3d(), "linear3D", 3),
        (square_mesh(17, 0.1, jitter=0.25, seed=11), conf2d(rule="16"), "constant", 2),
    ]
    for mesh, conf, forcing, dim in cases:
        want = nl.loadVector(mesh, {"function": forcing}, conf)
        first = _noalloc(env, mesh, conf, forcing, dim)
        second = _noalloc(env, mesh, conf, forcing, dim)
        assert np.array_equal(first.view(np.int64), want.view(np.int64)), forcing
        assert np.array_equal(second.view(np.int64), want.view(np.int64)), forcing


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
