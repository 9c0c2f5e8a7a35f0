"""Benchmark of the nonlocal stiffness-matrix assembly on one GB300.

Workload (default, --workload c2): 2D constant kernel at scale - [0,1]^2 plus a delta = 0.1 interaction layer,
right-diagonal triangulation with 2*256^2 triangles, interior vertices jittered by +-0.2h
(numpy PCG64, seed 1), P1 continuous Galerkin, kernel 4/(pi delta^4) on the l2 ball with the
'retriangulate' approximation and caps, 7-point Dunavant outer/inner rules. One step = one full
stiffness-matrix assembly (dual graph, BFS pair search, pattern, quadrature, deterministic
scatter, zero dropping) from the mesh in HBM to the CSR matrix in HBM.

metric: element-pair quadratures/s = interacting ordered element pairs (reference integrate()
calls that contribute) / assembly time. The headline runs the mixed FP32/FP64 path; the all-FP64
GPU path is timed on the same workload beside it, and the relative Frobenius / max-entry error
of the mixed matrix against the FP64 one is reported (the FP64 path itself matches the CPU
oracle to 1e-12 in the parity tests).

--impl reference times the CPU restatement of the reference algorithm (oracle, OpenMP, all host
cores) on a bounded sample of the same workload. --gpus N runs N independent replicas (one per
GPU; the assembly of one problem is not partitioned), value = all pairs / max time over ranks.
Prints one JSON line (rank 0). --workload c1/c3/c4/c5 measures the other configurations the same
way (c1 small 2D, c3 fractional kernel, c4 3D barycenter, c5 64 uneven problems in one batch).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np

METRIC = "element-pair quadratures/s: mixed vs FP64 on one GB300 at <=1e-6 rel err"

# DRAM traffic (read + write bytes) per pair of the quadrature pass, from an ncu capture of one
# launch on a smaller case of the workload: k_pass_mix2d<0> on the 2D constant-kernel workload at
# n = 128 (2.56e7 pairs: 187.7 MB read, 35.0 MB written), k_pass_bary<3> on the 3D one at n = 24
# (2.59e7 pairs: 143.7 MB read, 8.2 MB written). The passes stream their pair lists and reuse the
# mesh from L2, so the traffic grows with the pairs. Reported as roofline.traffic (scaled to this
# run's pairs) with its source.
PASS_TRAFFIC = {
    "c2": ((187.713e6 + 35.046e6) / 25573871, "k_pass_mix2d<0> on the 2D constant-kernel workload at n=128 (2.56e7 pairs)"),
    "c4": ((143.728e6 + 8.242e6) / 25852104, "k_pass_bary<3> on the 3D constant-kernel workload at n=24 (2.59e7 pairs)"),
}
# Algorithmic bytes of the pair search per tested candidate: its 16-bit visited stamp (2 B), its
# incidence entry (4 B), a share of a vertex's stamp and incidence range (about 4 B) and the
# geometry its interaction test reads (the element's coordinates as double-float pairs for the
# retriangulate test, its barycenter's for the barycenter test); per pair, its queue and pool
# entries (8 B).
SEARCH_STAMP_BYTES, SEARCH_INCIDENCE_BYTES = 2 + 4, 4
SEARCH_GEOMETRY_BYTES = {("retriangulate", 2): 2 * 6 * 4, ("baryCenter", 2): 2 * 2 * 4, ("baryCenter", 3): 2 * 3 * 4}
SEARCH_BYTES_PER_PAIR = 8


def search_bytes_per_candidate(conf, dim):
    geo = SEARCH_GEOMETRY_BYTES.get((conf["approxBalls"]["method"], dim), 2 * (dim + 1) * dim * 4)
    return SEARCH_STAMP_BYTES + SEARCH_INCIDENCE_BYTES + geo


def workload(args, precision):
    """Problems [(mesh, kernel, configuration)] and the config record of the chosen workload."""
    from nlfem_gb300 import workloads
    return workloads.problems(args.workload, precision, n=args.n, delta=args.delta)


def reference_digest(args):
    """The digest of the reference's own FP64 assembly of this workload (tests/golden/digest_*.npz,
    made by tests/golden/make_ref_digests.py), or None for sizes that have none."""
    from nlfem_gb300 import digest
    key = {("c2", 0.1): "c2", ("c2", 0.05): "c2d05", ("c3", 0.1): "c3", ("c4", 0.1): "c4",
           ("c5", 0.1): "c5"}.get((args.workload, args.delta))
    if key is None or args.n is not None:
        return None
    path = os.path.join(ROOT, "tests", "golden", f"digest_{key}.npz")
    return digest.load(path) if os.path.exists(path) else None


def vs_reference(mats, dg):
    """Errors of the assembled matrices against the reference digest: the pattern (bit-exact, by
    hash), the relative Frobenius error estimated from A u, and the max-entry error over the
    sampled rows; the worst over the problems of a batch."""
    from nlfem_gb300 import digest
    digests, meta = dg
    res = [digest.compare(A, digests[f"p{i}"]) for i, A in enumerate(mats) if f"p{i}" in digests]
    if not res:
        return None
    return {"pattern_identical": all(r["pattern_identical"] for r in res),
            "fro_est": max(r["fro_est"] for r in res), "max_rows": max(r["max_rows"] for r in res),
            "problems_compared": len(res)}


def search_roofline(st, conf, dim):
    """The pair search against HBM: its algorithmic bytes (search_bytes_per_candidate per tested
    candidate, SEARCH_BYTES_PER_PAIR per pair) over the device time of the search phase (vertex
    incidence, search, pair compaction)."""
    hbm = measured_peaks().get("hbm_gbs")
    ms = st["ms_bfs"]
    per_cand = search_bytes_per_candidate(conf, dim)
    nbytes = per_cand * st["n_candidates"] + SEARCH_BYTES_PER_PAIR * st["n_pairs"]
    gbs = nbytes / (ms / 1000.0) / 1e9 if ms > 0 else None
    return {"bound": "hbm", "kernel": "k_bfs (one warp per outer element)", "candidates": int(st["n_candidates"]),
            "bytes_per_candidate": per_cand, "algorithmic_bytes": int(nbytes), "ms": ms, "achieved": gbs, "peak": hbm, "unit": "GB/s",
            "frac": (gbs / hbm) if (gbs and hbm) else None,
            "note": "latency bound (dependent stamp and incidence loads per step), not bandwidth bound"}


def config_dict(args, extra, problems):
    d = dict(extra)
    d["nE"] = int(sum(m["elements"].shape[0] for m, _, _ in problems))
    d["nV"] = int(sum(m["vertices"].shape[0] for m, _, _ in problems))
    d["precision"] = "mixed (headline) and fp64"
    d["l2"] = "flushed between steps (256 MiB write)"
    d["graph"] = not args.no_graph
    return d


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self.stop = threading.Event()
        self.t = threading.Thread(target=self.run, daemon=True)

    def run(self):
        while not self.stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True,
                                     text=True, timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self.stop.wait(0.2)

    def __enter__(self):
        self.t.start()
        return self

    def __exit__(self, *a):
        self.stop.set()
        self.t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 3 + i and s[3 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def algorithmic_flops(st, conf, kernel, dim=2):
    """Floating-point operations the reference algorithm needs for one assembly (outdim 1),
    counted from integration.cpp with loop invariants hoisted (an FMA counts 2).
    retriangulate (integration.cpp:345-540, 1393-1512), per
      pair 12 (toRef factorisation of bT); (pair, outer point) 198 (toPhys 8, retriangulation 133,
      fold of termLocal/termNonloc/termNonlocPrime 57); (pair, outer point, sub-triangle) 11
      (edge vectors, |det|); inner point of a sub-triangle 51 + k (toPhys 8, toRef 10, basis 2,
      weight 1, innerLocal 2, innerNonloc 6, innerNonlocPrime 6, termLocalPrime 16; k = 0 constant,
      7 parabola).
    baryCenter 3D (integration.cpp:910-1018, 1262-1280), per
      (pair, outer point) 24 + 40 (toPhys 18, distance 6 to the barycenter, fold of termLocal and
      termNonloc 40) and, when the barycenter is inside the ball, per inner point 30 (toPhys 18,
      weight 2, innerLocal 2, innerNonloc 8).
    n_subtri counts each (pair, outer point, sub-triangle) unit once (for baryCenter: each
    (pair, outer point) whose ball contains the barycenter). Close pairs of the singular kernel
    (FP64 Duffy rules) are not included.

    Constant kernels ("constant", "constant3D") take closed forms on the mixed path, and the model
    then counts those instead of the inner-point loops (the same sums, fewer operations):
      retriangulate, per pair 12; (pair, outer point) 30 (class test) + 57 (fold); inside item 10
      (the element's precomputed sums times kc |b|); cut item 133 (polygon) + 26 (basis at the
      first two points, the ten results); cut sub-triangle 11 + 13 (basis at its third point) + 60
      (moment sums);
      baryCenter, per (pair, outer point) 64; item 5.
    Those counts need the item classes (n_items_in / n_items_cut). A batch that mixes kernels is
    counted with the closed forms for every problem (a lower bound)."""
    nPx = len(conf["quadrature"]["outer"]["weights"])
    nPy = len(conf["quadrature"]["inner"]["weights"])
    # a batch mixing constant and other kernels ("mixed") is counted with the closed forms
    # throughout, a lower bound on the operations that ran
    const = kernel["function"] in ("constant", "constant3D", "mixed") and conf.get("precision") == "mixed"
    if conf["approxBalls"]["method"] == "baryCenter":
        if const:
            return st["n_pairs"] * nPx * 64 + st["n_items_in"] * 5
        return st["n_pairs"] * nPx * 64 + st["n_subtri"] * nPy * 30
    if const:
        n_in, n_cut = st["n_items_in"], st["n_items_cut"]
        sub_cut = st["n_subtri"] - n_in
        return st["n_pairs"] * (12 + nPx * 87) + n_in * 10 + n_cut * (133 + 26) + sub_cut * 84
    kf = {"constant": 0, "parabola": 7, "fractional": 0, "mixed": 3.5}.get(kernel["function"], 0)
    return st["n_pairs"] * (12 + nPx * 198) + st["n_subtri"] * (11 + nPy * (51 + kf))


def cpu_sample(problems, seconds, threads):
    """Oracle (CPU restatement, FP64, OpenMP) on a bounded sample of outer elements of each
    problem in turn, until about `seconds` of work; returns (pairs, seconds, elements)."""
    from oracle import oracle
    rng = np.random.Generator(np.random.PCG64(0))
    tot_p = tot_s = 0.0
    tot_e = 0
    budget = seconds / len(problems) if len(problems) > 1 else seconds
    for mesh, kernel, conf in problems:
        conf = dict(conf, precision="fp64")
        nE = mesh["elements"].shape[0]
        k = min(max(threads * 4, 64), nE)
        sub = np.sort(rng.choice(nE, size=k, replace=False))
        r = oracle.assemble(mesh, kernel, conf, nthreads=threads, subset=sub)
        per_el = r["seconds"] / len(sub)
        want = int(min(nE, max(k, budget / max(per_el, 1e-9))))
        if want > k:
            sub = np.sort(rng.choice(nE, size=want, replace=False))
            r = oracle.assemble(mesh, kernel, conf, nthreads=threads, subset=sub)
        tot_p += r["n_pairs"]
        tot_s += r["seconds"]
        tot_e += len(sub)
        if tot_s >= seconds:
            break
    return tot_p, tot_s, tot_e


def run_reference(args):
    problems, extra = workload(args, "fp64")
    threads = os.cpu_count() or 1
    per_step = max(2.0, args.cpu_seconds / max(args.steps, 1))
    for _ in range(min(args.warmup, 1)):
        cpu_sample(problems[:1], 1.0, threads)
    tot_p = tot_s = 0.0
    ns = 0
    for _ in range(args.steps):
        p, s, ns = cpu_sample(problems, per_step, threads)
        tot_p += p
        tot_s += s
    value = tot_p / tot_s
    sample = (f"{ns} outer elements drawn uniformly (seed 0) per step: BFS + quadrature + map scatter of "
              f"their rows, FP64, {threads} OpenMP threads")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "pairs/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * tot_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_dict(args, extra, problems),
            "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def timed_session(problems, steps, warmup, flush, clocks_index=0, dist=None, graph=True):
    """W untimed + K timed assemblies from HBM-resident inputs; L2 flushed before each step.
    With graph=True the steps replay the assembly captured as a CUDA graph during the warm-up
    (every kernel of the step still runs; only the host-side orchestration is replaced).
    Returns (pairs, seconds, last stats, per-step stats, clocks, session)."""
    import torch
    from nlfem_gb300 import nlfem
    sess = nlfem.Session(problems)
    for _ in range(warmup):
        sess.assemble(graph=graph)
    stats = []
    with Clocks(clocks_index) as clk:
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()
        for _ in range(steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            stats.append(sess.assemble(graph=graph))   # device time: CUDA events on its stream
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
    pairs = float(sum(s["n_pairs"] for s in stats))
    secs = float(sum(s["ms_total"] for s in stats)) / 1000.0
    return pairs, secs, stats[-1], stats, clk.summary(), sess


def rel_err(A, B):
    """Relative Frobenius and max-entry error of A against B."""
    A = A.tocsr(); B = B.tocsr()
    A.sort_indices(); B.sort_indices()
    same = (A.shape == B.shape and np.array_equal(A.indptr, B.indptr) and np.array_equal(A.indices, B.indices))
    if same:
        d, b = A.data - B.data, B.data
    else:
        d, b = (A - B).tocsr().data, B.data
    return same, float(np.sqrt(np.sum(d * d)) / np.sqrt(np.sum(b * b))), float(np.max(np.abs(d)) / np.max(np.abs(b)))


def pinned(mesh):
    """The mesh arrays copied into page-locked host memory (torch), as numpy views."""
    import torch
    out = dict(mesh)
    nbytes = 0
    for key in ("elements", "elementLabels", "vertices", "vertexLabels"):
        a = mesh[key]
        t = torch.empty(a.shape, dtype=torch.float64 if a.dtype == np.float64 else torch.int64, pin_memory=True)
        t.numpy()[...] = a
        out[key] = t.numpy()
        nbytes += a.nbytes
    return out, nbytes


def combine_ranks(secs, pairs, dist, device="cpu"):
    """The job's time and work over the ranks: the slowest rank's seconds and all ranks' pairs
    (replicas: value = all pairs / max time)."""
    import torch
    t = torch.tensor([secs], dtype=torch.float64, device=device)
    p = torch.tensor([pairs], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(p, op=dist.ReduceOp.SUM)
    return float(t.item()), float(p.item())


def run_gpu(args, rank=0, world=1, dist=None):
    import ctypes
    import torch
    from nlfem_gb300 import nlfem, _lib
    lib = _lib.load()
    if lib.nlfem_device_count() == 0:
        raise SystemExit("no CUDA device")
    torch.cuda.init()
    dev = torch.cuda.current_device()
    problems, extra = workload(args, "mixed")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    pairs, secs, st, all_st, clocks, sess = timed_session(problems, args.steps, args.warmup, flush, dev, dist,
                                                          graph=not args.no_graph)
    launches = int(sum(s["n_launches"] for s in all_st))
    if dist is not None:
        secs, pairs = combine_ranks(secs, pairs, dist, "cuda")
    value = pairs / secs
    A_mixed = [sess.download(i) for i in range(len(problems))] if rank == 0 else []
    sess.close()
    if rank != 0:
        return

    # roofline of the dominant kernel: algorithmic flops of the step / device time of the
    # quadrature phase, against the FP32 FMA peak measured in this run
    f32, f64 = ctypes.c_double(0.0), ctypes.c_double(0.0)
    _lib.check(lib.nlfem_measure_peaks(ctypes.byref(f32), ctypes.byref(f64)))
    peak32, peak64 = f32.value, f64.value
    kernels = {k["function"] for _, k, _ in problems}
    kernel0 = problems[0][1] if len(kernels) == 1 else {"function": "mixed"}
    conf0 = problems[0][2]
    flops = algorithmic_flops(st, conf0, kernel0)
    achieved = flops / (st["ms_quad"] / 1000.0) / 1e12
    bary = conf0["approxBalls"]["method"] == "baryCenter"
    kname = ("k_pass_bary (one-sided barycenter quadrature + fixed-point scatter, one persistent launch)" if bary else
             "k_pass_mix2d (one-sided quadrature + fixed-point scatter, one persistent launch)")

    # end to end through the public API: pinned host inputs, host CSR out
    pins = [pinned(m) for m, _, _ in problems]
    h2d = sum(nb for _, nb in pins)
    calls = [(pm, k, c) for (pm, _), (_, k, c) in zip(pins, problems)]

    def e2e_call():
        if len(calls) == 1:
            return [nlfem.stiffnessMatrix(*calls[0])]
        return nlfem.stiffnessMatrix_batch(calls)
    # two warm-up calls: results come back in pinned host blocks that the library pools, and a
    # caller holding the previous result while the next call runs uses two of them; the first two
    # calls allocate them (cudaMallocHost of the matrix size), later calls reuse them
    Bs = e2e_call()
    Bs = e2e_call()
    e2e_t, e2e_p, d2h = [], 0, 0
    for _ in range(max(1, min(args.steps, 3))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        Bs = e2e_call()
        e2e_t.append(time.perf_counter() - t0)
        e2e_p += _lib.stats()["n_pairs"]
        d2h = sum(B.data.nbytes + B.indices.nbytes + B.indptr.nbytes for B in Bs)
    e2e = e2e_p / float(np.sum(e2e_t))

    line = {
        "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * secs / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": config_dict(args, extra, problems),
        "pairs_per_step": int(st["n_pairs"]), "nnz": int(sum(A.nnz for A in A_mixed)),
        "nnz_structural": int(st["nnz_structural"]), "close_pairs": int(st["n_close"]),
        "device_bytes": int(st["dev_bytes"]),
        "fp64_fallbacks": int(st["n_ambiguous"]), "subtriangles": int(st["n_subtri"]),
        "phase_ms": {"dual+bfs+pairs+color": st["ms_bfs"], "pattern": st["ms_pattern"],
                     "quadrature+scatter": st["ms_quad"], "finish": st["ms_finish"]},
        "roofline": {"bound": "fp32", "kernel": kname,
                     "achieved": achieved, "peak": peak32, "unit": "TFLOP/s", "frac": achieved / peak32,
                     "traffic": (PASS_TRAFFIC[args.workload][0] * st["n_pairs"]
                                 if args.workload in PASS_TRAFFIC and args.delta == 0.1 else None),
                     "traffic_source": ("ncu DRAM bytes of one launch of " + PASS_TRAFFIC[args.workload][1] +
                                        ", scaled by this run's pairs (not measured in this run)"
                                        if args.workload in PASS_TRAFFIC and args.delta == 0.1 else
                                        "no ncu capture of this workload's pass"),
                     "note": "achieved = flops of the algorithm that ran for the step (FLOP model in "
                             "bench.algorithmic_flops: the reference's inner-point loops, or their closed forms "
                             "for constant kernels; FP64 close pairs not counted) / device time of the "
                             "quadrature phase; peak = FP32 FMA throughput measured in this run (of measured); "
                             "CUDA-core bound path with no GEMM-shaped work, so neither the tensor-core nor the "
                             "HBM peak applies"},
        "search": search_roofline(st, conf0, int(problems[0][0]["vertices"].shape[1])),
        "peaks_measured": {"fp32_tflops": peak32, "fp64_tflops": peak64,
                           "hbm_gbs": measured_peaks().get("hbm_gbs")},
        "e2e": {"value": e2e, "unit": "pairs/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "note": "nlfem.stiffnessMatrix from pinned host mesh arrays to a host scipy CSR, two warm-up "
                        "calls (the pooled pinned result blocks), the previous result held during each call"},
        "clocks": clocks,
        "gpu_launches": launches,
    }

    run64 = world == 1 and not args.no_fp64 and (args.workload != "c5" or args.fp64_steps_set)
    A64 = None
    if run64:
        problems64, _ = workload(args, "fp64")
        p64, s64, st64, _, clk64, sess64 = timed_session(problems64, args.fp64_steps, 1, flush, dev)
        A64 = [sess64.download(i) for i in range(len(problems))]
        errs = [rel_err(A_mixed[i], A64[i]) for i in range(len(problems))]
        sess64.close()
        a64 = algorithmic_flops(st64, problems64[0][2], kernel0) / (st64["ms_quad"] / 1000.0) / 1e12
        line["fp64"] = {"value": p64 / s64, "unit": "pairs/s", "steps": args.fp64_steps,
                        "ms_per_step": 1000.0 * s64 / args.fp64_steps, "mixed_over_fp64": value / (p64 / s64),
                        "roofline": {"bound": "fp64", "achieved": a64, "peak": peak64, "unit": "TFLOP/s",
                                     "frac": a64 / peak64},
                        "clocks": clk64}
        line["rel_err_vs_fp64"] = {"pattern_identical": all(e[0] for e in errs),
                                   "fro": max(e[1] for e in errs), "max": max(e[2] for e in errs),
                                   "per_problem": len(errs) > 1, "bound": 1e-6}
    elif world == 1:
        line["fp64"] = {"skipped": "pass --fp64-steps K to time the all-FP64 path on this workload"}
    # the same one-sided algorithm (classes, closed forms, fixed-point scatter) in FP64 arithmetic:
    # the ratio to it is what the precision alone buys
    A1 = None
    if world == 1 and not args.no_fp64 and args.workload in ("c1", "c2", "c3", "c5"):
        problems1, _ = workload(args, "fp64-onesided")
        p1, s1, st1, _, clk1, sess1 = timed_session(problems1, args.fp64_steps, 1, flush, dev)
        A1 = [sess1.download(i) for i in range(len(problems1))]
        sess1.close()
        a1 = algorithmic_flops(st1, dict(problems1[0][2], precision="mixed"), kernel0) / (st1["ms_quad"] / 1000.0) / 1e12
        line["fp64_same_algorithm"] = {
            "value": p1 / s1, "unit": "pairs/s", "steps": args.fp64_steps, "ms_per_step": 1000.0 * s1 / args.fp64_steps,
            "mixed_over_fp64_same_algorithm": value / (p1 / s1),
            "phase_ms": {"dual+bfs+pairs+color": st1["ms_bfs"], "pattern": st1["ms_pattern"],
                         "quadrature+scatter": st1["ms_quad"], "finish": st1["ms_finish"]},
            "roofline": {"bound": "fp64", "achieved": a1, "peak": peak64, "unit": "TFLOP/s", "frac": a1 / peak64,
                         "note": "the mixed path's FLOP model over the FP64 instance's quadrature phase"},
            "note": "precision \"fp64-onesided\": the headline's one-sided pass, closed forms and fixed-point sums "
                    "in FP64 arithmetic (FP64 class tests, the exact FP64 polygon routine); the plain FP64 arm "
                    "beside it is the reference's two-sided algorithm on the GPU",
            "clocks": clk1}
    dg = reference_digest(args)
    if dg is not None:
        ref = {"oracle": "the reference's own src/*.cpp, FP64, compiled against project-written Armadillo/METIS "
                         "stand-ins (oracle/ref.mk); digest of its assembly of this workload "
                         "(tests/golden/digest_*.npz: pattern hash, A u for a seeded Gaussian u or bilinear probes, "
                         "sampled rows)",
               "ref_cpu_seconds": float(dg[1].get("ref_seconds", 0.0)), "ref_threads": int(dg[1].get("ref_threads", 0)),
               "mixed": vs_reference(A_mixed, dg), "bound_mixed": 1e-6}
        if A64 is not None:
            ref["fp64"] = vs_reference(A64, dg)
        if A1 is not None:
            ref["fp64_same_algorithm"] = vs_reference(A1, dg)
        line["rel_err_vs_oracle"] = ref
    if world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        p, s, ns = cpu_sample(problems, args.cpu_seconds, threads)
        line["cpu_baseline"] = {"value": p / s, "unit": "pairs/s", "cores": threads, "kind": "port",
                                "sample": f"{ns} outer elements (uniform, seed 0): BFS + FP64 quadrature + map "
                                          f"scatter of their rows"}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c3", "c4", "c5"],
                    help="c2 (default): the 2D constant-kernel workload the metric is quoted on")
    ap.add_argument("--n", type=int, default=None, help="mesh cells per side (default per workload)")
    ap.add_argument("--delta", type=float, default=0.1)
    ap.add_argument("--fp64-steps", type=int, default=None)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-graph", action="store_true", help="time normal assemblies instead of CUDA-graph replays")
    args = ap.parse_args()
    args.fp64_steps_set = args.fp64_steps is not None
    if args.fp64_steps is None:
        args.fp64_steps = 1
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return
    if world > 1:
        # replicas only: each rank assembles the full workload on its own GPU, no collective on
        # the data path; the barrier and the max over ranks bracket the timed steps
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
        try:
            run_gpu(args, rank, world, dist)
        finally:
            dist.barrier()
            dist.destroy_process_group()
        return
    run_gpu(args)


if __name__ == "__main__":
    main()
