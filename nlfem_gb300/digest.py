"""Digests of assembled matrices: compact, size-independent fingerprints for full-size checks.

A full-size stiffness matrix (7.75e7 entries for 2·256² triangles at delta = 0.1) is too large to
keep as a fixture, so the reference assembly of each workload is stored as a digest
(tests/golden/digest_*.npz), and a matrix assembled elsewhere is compared with it:
* pattern: SHA-256 of the sorted CSR row pointers and column indices (int64) - bit-exact check;
* fro / maxabs: Frobenius norm and largest |entry| of the reference matrix;
* Au: the reference matrix applied to a seeded Gaussian vector u. For a difference D of two
  matrices E||D u||^2 = ||D||_F^2, and with one term per row the estimate is tight (its relative
  spread is about sqrt(2 / rows)), so ||A u - Au|| / fro estimates the relative Frobenius error;
* probes: w_k^T A v_k for seeded Gaussian pairs (used where Au would be too large to keep); the
  root mean square of their errors estimates ||D||_F the same way, more coarsely;
* rows: complete rows at seeded positions, for an exact max-entry error over those rows;
* f: the load vector, where the workload has a forcing.
"""
import hashlib

import numpy as np
import scipy.sparse as sp

U_SEED = 20251
PROBE_SEED = 20252
ROW_SEED = 20253


def _csr(A):
    A = sp.csr_matrix(A)
    A.sort_indices()
    return A


def pattern_sha(A):
    A = _csr(A)
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(A.indptr, dtype=np.int64).tobytes())
    h.update(np.ascontiguousarray(A.indices, dtype=np.int64).tobytes())
    return h.hexdigest()


def gaussian(n, seed):
    return np.random.Generator(np.random.PCG64(seed)).standard_normal(n)


def make(A, n_rows=32, n_probes=0, with_au=True, f=None):
    """Digest of the reference matrix A (dict of numpy arrays)."""
    A = _csr(A)
    K = A.shape[0]
    d = {"K": np.int64(K), "nnz": np.int64(A.nnz), "pattern_sha": np.array(pattern_sha(A)),
         "fro": np.float64(np.sqrt(np.dot(A.data, A.data))), "maxabs": np.float64(abs(A.data).max() if A.nnz else 0.0)}
    if with_au:
        d["Au"] = A @ gaussian(K, U_SEED)
    if n_probes:
        p = np.empty(n_probes)
        for k in range(n_probes):
            v = gaussian(K, PROBE_SEED + 2 * k)
            w = gaussian(K, PROBE_SEED + 2 * k + 1)
            p[k] = w @ (A @ v)
        d["probes"] = p
    nonempty = np.flatnonzero(np.diff(A.indptr) > 0)
    rng = np.random.Generator(np.random.PCG64(ROW_SEED))
    rows = np.sort(rng.choice(nonempty, size=min(n_rows, nonempty.size), replace=False)).astype(np.int64)
    ptr = np.zeros(rows.size + 1, np.int64)
    cols, vals = [], []
    for i, r in enumerate(rows):
        a, b = A.indptr[r], A.indptr[r + 1]
        cols.append(A.indices[a:b].astype(np.int64))
        vals.append(A.data[a:b])
        ptr[i + 1] = ptr[i] + (b - a)
    d.update({"rows": rows, "row_ptr": ptr, "row_cols": np.concatenate(cols) if cols else np.zeros(0, np.int64),
              "row_vals": np.concatenate(vals) if vals else np.zeros(0)})
    if f is not None:
        d["f"] = np.asarray(f, dtype=np.float64)
    return d


def compare(A, d, f=None):
    """Errors of matrix A (and load vector f) against digest d:
    {pattern_identical, fro_est, max_rows, [f_max]}; fro_est relative to the reference's Frobenius
    norm, max_rows (the largest entry error over the sampled rows) relative to its largest entry."""
    A = _csr(A)
    K = int(d["K"])
    out = {"pattern_identical": bool(A.shape == (K, K) and pattern_sha(A) == str(d["pattern_sha"]))}
    fro = float(d["fro"])
    if "Au" in d:
        out["fro_est"] = float(np.linalg.norm(A @ gaussian(K, U_SEED) - d["Au"]) / fro)
    elif "probes" in d:
        e = []
        for k in range(len(d["probes"])):
            v = gaussian(K, PROBE_SEED + 2 * k)
            w = gaussian(K, PROBE_SEED + 2 * k + 1)
            e.append(w @ (A @ v) - d["probes"][k])
        out["fro_est"] = float(np.sqrt(np.mean(np.square(e))) / fro)
    worst = 0.0
    rows, ptr, cols, vals = d["rows"], d["row_ptr"], d["row_cols"], d["row_vals"]
    for i, r in enumerate(rows):
        ref = sp.csr_matrix((vals[ptr[i]:ptr[i + 1]], cols[ptr[i]:ptr[i + 1]], [0, ptr[i + 1] - ptr[i]]), shape=(1, K))
        diff = A[int(r)] - ref
        if diff.nnz:
            worst = max(worst, float(abs(diff).max()))
    out["max_rows"] = worst / float(d["maxabs"])
    if f is not None and "f" in d:
        fr = d["f"]
        out["f_max"] = float(abs(np.asarray(f) - fr).max() / max(abs(fr).max(), 1e-300))
    return out


def save(path, digests, meta):
    """Writes digests {prefix: digest} and meta {key: value} into one npz file."""
    arrays = {f"meta.{k}": np.array(v) for k, v in meta.items()}
    for prefix, d in digests.items():
        for k, v in d.items():
            arrays[f"{prefix}.{k}"] = np.asarray(v)
    np.savez_compressed(path, **arrays)


def load(path):
    """(digests {prefix: dict}, meta dict) from a file written by save()."""
    z = np.load(path, allow_pickle=False)
    digests, meta = {}, {}
    for key in z.files:
        prefix, name = key.split(".", 1)
        v = z[key]
        if prefix == "meta":
            meta[name] = v.item() if v.ndim == 0 else v
        else:
            digests.setdefault(prefix, {})[name] = v
    return digests, meta
