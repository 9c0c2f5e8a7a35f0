"""Benchmark of the nonlocal stiffness-matrix assembly on one GB300.

Workload (default): 2D constant kernel at scale - [0,1]^2 plus a delta = 0.1 interaction layer,
right-diagonal triangulation with 2*256^2 triangles, interior vertices jittered by +-0.2h
(numpy PCG64, seed 1), P1 continuous Galerkin, kernel 4/(pi delta^4) on the l2 ball with the
'retriangulate' approximation and caps, 7-point Dunavant outer/inner rules. One step = one full
stiffness-matrix assembly (dual graph, BFS pair search, pattern, quadrature, deterministic
scatter, zero dropping) from the mesh in HBM to the CSR matrix in HBM.

metric: element-pair quadratures/s = interacting ordered element pairs / assembly time.
Prints one JSON line (rank 0). --impl reference times the CPU restatement of the reference
(oracle, OpenMP, all host cores) on a bounded sample of the same workload instead.
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

METRIC = "element-pair quadratures/s"


def workload(args):
    from nlfem_gb300 import meshes, quadrules
    v, e, l = meshes.regular_square(args.n, args.delta, jitter=0.2, seed=1)
    mesh = meshes.mesh_dict(v, e, l)
    P, w = quadrules.dunavant7()
    conf = {"ansatz": "CG", "approxBalls": {"method": "retriangulate", "is_PlacePointOnCap": 1},
            "quadrature": {"outer": {"points": P, "weights": w}, "inner": {"points": P, "weights": w}},
            "precision": args.precision}
    kernel = {"function": "constant", "horizon": args.delta, "outputdim": 1}
    return mesh, kernel, conf


def config_dict(args, mesh):
    return {"workload": f"2D constant kernel, 2*{args.n}^2 triangles jittered +-0.2h, delta={args.delta}, "
                        f"retriangulate+caps, 7-pt Dunavant outer/inner, P1 CG",
            "n": args.n, "delta": args.delta, "nE": int(mesh["elements"].shape[0]),
            "nV": int(mesh["vertices"].shape[0]), "precision": args.precision,
            "l2": "flushed between steps (256 MiB write)"}


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.samples = []
        self.stop = threading.Event()
        self.t = threading.Thread(target=self.run, daemon=True)

    def run(self):
        while not self.stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", "0", f"--query-gpu={self.FIELDS}",
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


def cpu_sample(mesh, kernel, conf, seconds, threads):
    """Oracle (CPU restatement, OpenMP) on a bounded sample of outer elements."""
    from oracle import oracle
    nE = mesh["elements"].shape[0]
    rng = np.random.Generator(np.random.PCG64(0))
    k = max(threads * 4, 64)
    sub = np.sort(rng.choice(nE, size=min(k, nE), replace=False))
    r = oracle.assemble(mesh, kernel, conf, nthreads=threads, subset=sub)
    rate = r["n_pairs"] / max(r["seconds"], 1e-9)
    want = int(min(nE, max(k, seconds * rate / max(r["n_pairs"] / len(sub), 1))))
    sub = np.sort(rng.choice(nE, size=want, replace=False))
    r = oracle.assemble(mesh, kernel, conf, nthreads=threads, subset=sub)
    return r["n_pairs"], r["seconds"], len(sub)


def run_reference(args):
    mesh, kernel, conf = workload(args)
    threads = os.cpu_count() or 1
    vals = []
    per_step = max(2.0, args.cpu_seconds / max(args.steps, 1))
    for _ in range(args.warmup if args.warmup < 1 else 1):
        cpu_sample(mesh, kernel, conf, 1.0, threads)
    tot_p = tot_s = 0.0
    ns = 0
    for _ in range(args.steps):
        p, s, ns = cpu_sample(mesh, kernel, conf, per_step, threads)
        tot_p += p
        tot_s += s
        vals.append(p / s)
    value = tot_p / tot_s
    sample = f"{ns} outer elements drawn uniformly (seed 0) of {mesh['elements'].shape[0]}, BFS + quadrature + map scatter per element"
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "pairs/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * tot_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_dict(args, mesh),
            "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gpu(args):
    import torch
    from nlfem_gb300 import nlfem, _lib
    lib = _lib.load()
    if lib.nlfem_device_count() == 0:
        raise SystemExit("no CUDA device")
    torch.cuda.init()
    mesh, kernel, conf = workload(args)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    sess = nlfem.Session([(mesh, kernel, conf)])
    for _ in range(args.warmup):
        st = sess.assemble()
    ms, pairs, stats = [], [], []
    with Clocks() as clk:
        for _ in range(args.steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            st = sess.assemble()
            ms.append(st["ms_total"])
            pairs.append(st["n_pairs"])
            stats.append(st)
    clocks = clk.summary()
    A = sess.download(0)
    sess.close()
    t_ms = float(np.sum(ms))
    value = float(np.sum(pairs)) / (t_ms / 1000.0)
    st = stats[-1]

    # end to end through the public API: pinned host inputs, host CSR out
    pin = {}
    for key in ("elements", "elementLabels", "vertices", "vertexLabels"):
        a = mesh[key]
        t = torch.empty(a.shape, dtype=torch.float64 if a.dtype == np.float64 else torch.int64, pin_memory=True)
        t.numpy()[...] = a
        pin[key] = t.numpy()
    pmesh = dict(mesh)
    pmesh.update(pin)
    h2d = sum(pin[k].nbytes for k in pin)
    for _ in range(1):
        nlfem.stiffnessMatrix(pmesh, kernel, conf)
    e2e_t = []
    e2e_p = 0
    d2h = 0
    for _ in range(max(1, min(args.steps, 3))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        B = nlfem.stiffnessMatrix(pmesh, kernel, conf)
        e2e_t.append(time.perf_counter() - t0)
        e2e_p += _lib.stats()["n_pairs"]
        d2h = B.data.nbytes + B.indices.nbytes + B.indptr.nbytes
    e2e = e2e_p / float(np.sum(e2e_t))

    # roofline: the quadrature kernel, algorithmic FP64 flops per launch / its device time
    flops = algorithmic_flops(st, conf)
    achieved = flops / (st["ms_quad"] / 1000.0) / 1e12
    peaks = measured_peaks()
    peak = args.fp_peak_tflops
    line = {
        "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32+f64", "data": "synthetic",
        "config": config_dict(args, mesh),
        "pairs_per_step": int(pairs[-1]), "nnz": int(A.nnz), "nnz_structural": int(st["nnz_structural"]),
        "fp64_fallbacks": int(st["n_ambiguous"]), "subtriangles": int(st["n_subtri"]),
        "phase_ms": {"dual+bfs+pairs": st["ms_bfs"], "pattern": st["ms_pattern"],
                     "quadrature+scatter": st["ms_quad"], "finish": st["ms_finish"]},
        "roofline": {"bound": args.fp_bound, "kernel": "k_quad (quadrature + scatter)",
                     "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if peak else None, "traffic": None,
                     "note": "algorithmic FP64 flops of the reference arithmetic per step / quadrature phase time; "
                             "peak = nominal CUDA-core FP64 rate (no tensor-core or HBM bound applies)"},
        "e2e": {"value": e2e, "unit": "pairs/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "clocks": clocks,
        "gpu_launches": int(args.launches_per_step * args.steps),
        "hbm_peak_gbs": peaks.get("hbm_gbs"),
    }
    if not args.no_cpu:
        threads = os.cpu_count() or 1
        p, s, ns = cpu_sample(mesh, kernel, conf, args.cpu_seconds, threads)
        line["cpu_baseline"] = {"value": p / s, "unit": "pairs/s", "cores": threads, "kind": "port",
                                "sample": f"{ns} outer elements (uniform, seed 0) of {mesh['elements'].shape[0]}"}
    print(json.dumps(line), flush=True)


def algorithmic_flops(st, conf):
    """FP64 operations of the reference arithmetic for one assembly (counted from the code):
    per (pair, outer point): toPhys 8 + method_retriangulate ~150; per (sub-triangle, inner
    point): toPhys 10, two kernel values 2, toRef 14, basis 2, inner sums 4 + 2*3*4,
    termLocalPrime 9*7; per (pair, outer point) the outer accumulation 3*3*(5+4+4)."""
    nPx = len(conf["quadrature"]["outer"]["weights"])
    nPy = len(conf["quadrature"]["inner"]["weights"])
    per_outer = 8 + 150 + 9 * 13
    per_inner = 10 + 2 + 14 + 2 + 4 + 24 + 63
    return st["n_pairs"] * nPx * per_outer + st["n_subtri"] * nPy * per_inner


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--delta", type=float, default=0.1)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--fp-peak-tflops", type=float, default=1.25)
    ap.add_argument("--fp-bound", default="fp64")
    ap.add_argument("--launches-per-step", type=int, default=40)
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return
    if args.gpus > 1:
        # replicas only: the assembly of one problem is not partitioned across GPUs
        import torch
        import torch.distributed as dist
        local = int(os.environ.get("LOCAL_RANK", "0"))
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        dist.barrier()
        if rank != 0:
            args.no_cpu = True
        run_gpu(args) if rank == 0 else run_gpu_silent(args)
        dist.barrier()
        dist.destroy_process_group()
        return
    run_gpu(args)


def run_gpu_silent(args):
    import contextlib
    import io
    with contextlib.redirect_stdout(io.StringIO()):
        run_gpu(args)


if __name__ == "__main__":
    main()
