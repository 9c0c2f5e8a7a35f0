"""Seeded synthetic meshes for the assembly workloads.

* ``regular_square``: [-delta, 1+delta]^2 with n cells per side, right-diagonal split. Element k of
  cell (i, j) uses corner c = j*(n+1) + i and the triangles (c, c+1, c+1+N), (c, c+1+N, c+N),
  N = n+1, in the element order of src/MeshBuilder.cpp:124-159 (Grid2D::Element).
* ``regular_cube``: [-delta, 1+delta]^3, n cells per side, the 6-tetrahedron split of each cube
  around its main diagonal, in the element order of src/MeshBuilder.cpp (Grid3D::Element) with
  the base tetrahedra of include/MeshBuilder.h:123-129.
* Element labels: +1 if the barycenter lies in the unit square/cube (within 1e-5, the tolerance of
  examples/tutorial/mesh.py:6-20), else -1. Vertex labels follow get_vertexLabel
  (cython/nlfem.pyx:392-402): a vertex takes the smallest nonzero label of its elements.
* Jitter: vertices off the outer bounding box move by U(-j*h, j*h) per coordinate, numpy PCG64.
"""
import numpy as np

__all__ = ["regular_square", "regular_cube", "get_vertexLabel", "get_diam", "meshFromArrays",
           "mesh_dict", "batch_meshes"]


def get_vertexLabel(elements, elementLabels, vertices):
    """Vertex labels from element labels (cython/nlfem.pyx:392-402)."""
    nV = vertices.shape[0]
    vertexLabels = np.zeros(nV, dtype=np.int64)
    for label in np.sort(np.unique(elementLabels))[::-1]:
        if label:
            idx = np.where(elementLabels == label)
            vertexLabels[np.unique(elements[idx].ravel())] = label
    return vertexLabels


def get_diam(elements, vertices):
    """Largest |first-coordinate difference| along element edges (cython/nlfem.pyx:404-415)."""
    dim = vertices.shape[1]
    T = vertices[elements]
    diam = 0.0
    for k in range(dim + 1):
        diff = T[:, k] - T[:, (k + 1) % (dim + 1)]
        diam = max(diam, float(np.max(np.abs(diff[:, 0]))))
    return diam


def meshFromArrays(elements, elementLabels, vertices, outputdim=1):
    """Mesh dictionary from raw arrays (cython/nlfem.pyx:417-434)."""
    vertexLabels = get_vertexLabel(elements, elementLabels, vertices)
    return {
        "dim": elements.shape[1] - 1,
        "nE": elements.shape[0],
        "nV": vertices.shape[0],
        "nE_Omega": int(np.sum(elementLabels > 0)),
        "nV_Omega": int(np.sum(vertexLabels > 0)),
        "elements": np.ascontiguousarray(elements, dtype=np.int64),
        "elementLabels": np.ascontiguousarray(elementLabels, dtype=np.int64),
        "vertices": np.ascontiguousarray(vertices, dtype=np.float64),
        "vertexLabels": vertexLabels,
        "diam": get_diam(elements, vertices),
        "outdim": outputdim,
    }


def _labels(vertices, elements, lo=0.0, hi=1.0):
    bary = vertices[elements].mean(axis=1)
    inside = np.all((bary >= lo - 1e-5) & (bary <= hi + 1e-5), axis=1)
    return np.where(inside, 1, -1).astype(np.int64)


def _jitter(vertices, h, amount, seed, lo, hi):
    if amount <= 0:
        return vertices
    rng = np.random.Generator(np.random.PCG64(seed))
    on_box = np.any(np.isclose(vertices, lo, atol=1e-12 * (1 + abs(lo))) |
                    np.isclose(vertices, hi, atol=1e-12 * (1 + abs(hi))), axis=1)
    shift = rng.uniform(-amount * h, amount * h, size=vertices.shape)
    shift[on_box] = 0.0
    return vertices + shift


def regular_square(n, delta=0.1, jitter=0.0, seed=0):
    """2*n^2 triangles on [-delta, 1+delta]^2; returns (vertices, elements, elementLabels)."""
    N = n + 1
    xs = np.linspace(-delta, 1.0 + delta, N)
    X, Y = np.meshgrid(xs, xs, indexing="xy")
    vertices = np.stack([X.ravel(), Y.ravel()], axis=1)
    j, i = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    c = (j * N + i).ravel()
    elements = np.empty((2 * n * n, 3), dtype=np.int64)
    elements[0::2] = np.stack([c, c + 1, c + 1 + N], axis=1)
    elements[1::2] = np.stack([c, c + 1 + N, c + N], axis=1)
    h = (1.0 + 2.0 * delta) / n
    vertices = _jitter(vertices, h, jitter, seed, -delta, 1.0 + delta)
    return vertices, elements, _labels(vertices, elements)


def regular_cube(n, delta=0.1, jitter=0.0, seed=0):
    """6*n^3 tetrahedra on [-delta, 1+delta]^3; returns (vertices, elements, elementLabels)."""
    N = n + 1
    xs = np.linspace(-delta, 1.0 + delta, N)
    Z, Y, X = np.meshgrid(xs, xs, xs, indexing="ij")
    vertices = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    NN = N * N
    base = np.array([
        [0, 1, 1 + N, 1 + N + NN],
        [0, 1 + N, 1 + N + NN, N],
        [0, 1 + N + NN, N, NN + N],
        [0, 1, 1 + NN, 1 + N + NN],
        [0, 1 + NN, 1 + N + NN, NN],
        [0, 1 + N + NN, NN, NN + N],
    ], dtype=np.int64)
    k, j, i = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    corner = (k * NN + j * N + i).ravel()
    elements = (corner[:, None, None] + base[None, :, :]).reshape(-1, 4)
    h = (1.0 + 2.0 * delta) / n
    vertices = _jitter(vertices, h, jitter, seed, -delta, 1.0 + delta)
    return vertices, elements, _labels(vertices, elements)


def mesh_dict(vertices, elements, elementLabels, outdim=1):
    return meshFromArrays(elements, elementLabels, vertices, outdim)


def batch_meshes(count=64, seed=2024, sizes=tuple(range(32, 193, 16))):
    """Seeded uneven problem set: n from sizes, delta ~ U[0.05, 0.2], kernel constant/parabola."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for p in range(count):
        n = int(rng.choice(sizes))
        delta = float(rng.uniform(0.05, 0.2))
        kernel = "constant" if p % 2 == 0 else "parabola"
        v, e, l = regular_square(n, delta=delta, jitter=0.2, seed=seed * 1000 + p)
        out.append({"n": n, "delta": delta, "kernel": kernel, "mesh": mesh_dict(v, e, l)})
    return out
