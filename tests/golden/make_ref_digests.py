"""Digests of the REFERENCE's own assembly of each full-size workload: tests/golden/digest_*.npz.

Usage (needs the reference checkout; it is compiled by oracle/ref.mk against oracle/refshim/):
    python tests/golden/make_ref_digests.py <reference checkout> [workload ...] [--threads N] [--resume]
workloads: c2 (delta 0.1), c2d05 (delta 0.05), c3, c4, c5 (default: all).

Each file holds, per problem, the digest of nlfem_gb300/digest.py (pattern hash, Frobenius norm,
A u for a seeded Gaussian u or bilinear probes, sampled complete rows), the load vector where the
workload has a forcing, the SHA-256 of the inputs, and the reference's wall time and thread count.
The GPU tests and bench.py compare the GPU assembly of the same workload against these files.
"""
import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, HERE)

WORKLOADS = {"c2": ("c2", 0.1), "c2d05": ("c2", 0.05), "c3": ("c3", 0.1), "c4": ("c4", 0.1), "c5": ("c5", 0.1)}


def path_of(key):
    return os.path.join(HERE, f"digest_{key}.npz")


def make(key, threads, resume=False):
    """Assembles every problem of the workload with the reference and writes the digest file.
    With resume, problems already in an existing file are kept, and the file is rewritten after
    each problem, so a long batch (c5) can be stopped and continued."""
    from nlfem_gb300 import digest, workloads
    from oracle import ref
    from make_oracle_golden import input_hash
    name, delta = WORKLOADS[key]
    probs, rec = workloads.problems(name, "fp64", delta=delta)
    batch = len(probs) > 1
    digests, secs = {}, 0.0
    if resume and os.path.exists(path_of(key)):
        digests, old = digest.load(path_of(key))
        secs = float(old.get("ref_seconds", 0.0))
    for i, (mesh, kernel, conf) in enumerate(probs):
        if f"p{i}" in digests:
            continue
        t0 = time.time()
        r = ref.assemble(mesh, kernel, conf, nthreads=threads)
        secs += r["seconds"]
        f = None
        if not batch:
            f = ref.assemble(mesh, None, conf, compute="forcing", load={"function": workloads.FORCING[name]},
                             nthreads=threads)["f"]
        d = digest.make(r["A"], n_rows=4 if batch else 32, n_probes=16 if batch else 0, with_au=not batch, f=f)
        d["input_sha"] = np.array(input_hash(mesh, kernel, conf))
        digests[f"p{i}"] = d
        print(f"{key} problem {i}: K={int(d['K'])} nnz={int(d['nnz'])} {r['seconds']:.1f}s "
              f"(total {time.time() - t0:.1f}s)", flush=True)
        if resume:
            _save(key, digests, rec, probs, secs, threads)
    _save(key, digests, rec, probs, secs, threads)
    print("wrote", path_of(key), os.path.getsize(path_of(key)), "bytes", flush=True)


def _save(key, digests, rec, probs, secs, threads):
    from nlfem_gb300 import digest
    meta = {"workload": rec["workload"], "problems": len(probs), "problems_done": len(digests),
            "ref_seconds": secs, "ref_threads": threads,
            "source": "reference src/*.cpp compiled by oracle/ref.mk against oracle/refshim"}
    tmp = path_of(key) + ".tmp.npz"
    digest.save(tmp, digests, meta)
    os.replace(tmp, path_of(key))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("reference", help="path of the reference checkout (its src/ and include/)")
    ap.add_argument("workloads", nargs="*", default=list(WORKLOADS))
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    ap.add_argument("--resume", action="store_true", help="keep the problems of an existing file; save after each")
    a = ap.parse_args()
    from oracle import ref
    ref.build(a.reference)
    for key in a.workloads:
        make(key, a.threads, a.resume)


if __name__ == "__main__":
    main()
