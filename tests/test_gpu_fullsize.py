"""Every benchmark workload at its full size against the REFERENCE's own FP64 assembly.

The reference's src/*.cpp, compiled against project-written stand-ins (oracle/ref.mk), assembled
each workload on the CPU; tests/golden/make_ref_digests.py stored a digest of each result
(nlfem_gb300/digest.py): the pattern's hash, A u for a seeded Gaussian u (or bilinear probes per
problem of the batch), complete sampled rows, and the load vector. The GPU assembles the same
workloads here, in both precisions:
* pattern: bit-identical (hash of the sorted CSR);
* FP64 path: relative Frobenius error (estimated from A u, which is tight at these sizes) and
  max-entry error over the sampled rows <= 1e-12 (rounding only: the GPU sums in another order);
* mixed path: both <= 1e-6;
* load vector: <= 1e-12 (max entry, relative).
The 64-problem batch's FP64 check covers every eighth problem (its batch matrices equal the single assemblies bit
for bit, a property the parity tests check); the mixed check covers all 64. A batch digest may hold
only the first problems of the batch (meta problems_done); the checks cover the problems it holds.
"""
import os
import sys

import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
CASES = {"c2": ("c2", 0.1), "c2d05": ("c2", 0.05), "c3": ("c3", 0.1), "c4": ("c4", 0.1), "c5": ("c5", 0.1)}


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from nlfem_gb300 import nlfem
    return nlfem


def _digest(key):
    path = os.path.join(GOLDEN, f"digest_{key}.npz")
    if not os.path.exists(path):
        pytest.skip(f"no reference digest {os.path.basename(path)}")
    from nlfem_gb300 import digest
    return digest.load(path)


@pytest.mark.parametrize("key", list(CASES))
def test_workload_matches_reference(gpu, key):
    from nlfem_gb300 import digest, workloads
    from make_oracle_golden import input_hash
    digests, meta = _digest(key)
    name, delta = CASES[key]
    for precision, tol in (("fp64", 1e-12), ("mixed", 1e-6)):
        probs, _ = workloads.problems(name, precision, delta=delta)
        idx = list(range(len(probs)))
        if precision == "fp64" and len(probs) > 1:
            idx = idx[::8]
        idx = [i for i in idx if f"p{i}" in digests]   # a batch digest may be partial (problems_done)
        for i in idx:
            mesh, kernel, conf = probs[i]
            d = digests[f"p{i}"]
            assert input_hash(mesh, kernel, dict(conf, precision="fp64")) == str(d["input_sha"]), \
                f"{key} problem {i}: the workload's inputs differ from those the reference assembled"
        if len(probs) == 1:
            mats = [gpu.stiffnessMatrix(*probs[0])]
        else:
            mats = gpu.stiffnessMatrix_batch([probs[i] for i in idx])
        for i, A in zip(idx, mats):
            r = digest.compare(A, digests[f"p{i}"])
            assert r["pattern_identical"], (key, precision, i)
            assert r["fro_est"] <= tol, (key, precision, i, r)
            assert r["max_rows"] <= tol, (key, precision, i, r)
    if "f" in digests["p0"]:
        mesh, _, conf = workloads.problems(name, "fp64", delta=delta)[0][0]
        f = gpu.loadVector(mesh, {"function": workloads.FORCING[name]}, conf)
        r = digest.compare(mats[0], digests["p0"], f=f)
        assert r["f_max"] <= 1e-12, r
