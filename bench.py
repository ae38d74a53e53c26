#!/usr/bin/env python3
"""Benchmark: Poisson apply node-terms/s on one GB300, mixed vs FP64 form.

Workload (the FP64-GPU Poisson configuration): Legendre basis k=7, world box
[-32,32]^3, input = sum of 16 seeded Gaussians (centres uniform in [-5,5]^3,
exponents log-uniform in [1,100], coefficients uniform in [-1,1]) projected at
1e-5, PoissonOperator at 1e-5, applied with maxIter = 0 onto the output grid
of the adaptive apply (fixed topology, no norm screening).  The grid is the
adaptive FP64 GPU result, whose topology the parity tests show identical to
the CPU oracle's.

A node-term is one (output node, input node, operator term) triple inside the
operator band with at least one contracted component (the reference's own
screening rules); the count is an integer that equals the oracle's.

  value      node-terms/s of the mixed form with the input tree and the
             operator resident in HBM: per step GenNodes are dropped and
             rebuilt, every output node is computed, then the TopDown and
             BottomUp transforms run (CUDA events on the library stream)
  e2e        the same metric through mrcpp_gb300.apply (the host mirror of
             mrcpp::apply) with host buffers: input-tree upload, level
             norms and the output-tree download inside the timed region
  fp64       the plain FP64 form on the same workload
  roofline   the contraction kernel: algorithmic FLOP (96 (k+1)^4 per node-term)
             per launch / kernel time, against the measured bf16 dense peak
  cpu_baseline  the CPU oracle (port of the reference path) on a bounded sample

--impl reference times the CPU oracle (the reference itself needs Eigen and
cannot be built here) with all host threads on the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

METRIC = "Poisson apply node·terms/s on 1 GB300, mixed vs FP64 form at ≤1e-5 rel error"
UNIT = "node-terms/s"
ORDER, PREC, NGAUSS, SEED = 7, 1e-5, 16, 2026
EXP_RANGE, CENTRE_RANGE, MU = (1.0, 100.0), (-5.0, 5.0), None
WORKLOAD = "poisson-apply legendre k=7 box [-32,32]^3, 16 gaussians (exp 1..100, centres [-5,5]^3), prec 1e-5, fixed output grid (maxIter=0)"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="mw", choices=["mw", "reference"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--small", action="store_true", help="6 Gaussians at 1e-4 (a short launch for ncu captures)")
    p.add_argument("--workload", default="poisson", choices=["poisson", "helmholtz"],
                   help="poisson: the FP64-GPU Poisson configuration (default); helmholtz: the mixed-precision Helmholtz "
                        "configuration (mu=1, k=9, 32 Gaussians with exponents 0.5..500 in [-6,6]^3, prec 1e-6)")
    a = p.parse_args()
    global PREC, NGAUSS, WORKLOAD, ORDER, EXP_RANGE, CENTRE_RANGE, MU, METRIC
    if a.workload == "helmholtz":
        ORDER, PREC, NGAUSS, EXP_RANGE, CENTRE_RANGE, MU = 9, 1e-6, 32, (0.5, 500.0), (-6.0, 6.0), 1.0
        METRIC = "Helmholtz (mu=1) apply node·terms/s on 1 GB300, mixed vs FP64 form"
        WORKLOAD = "helmholtz-apply mu=1 legendre k=9 box [-32,32]^3, 32 gaussians (exp 0.5..500, centres [-6,6]^3), prec 1e-6, fixed output grid (maxIter=0)"
    if a.small:
        PREC, NGAUSS = PREC * 10, 6
        WORKLOAD = WORKLOAD.replace("16 gaussians", "6 gaussians").replace("32 gaussians", "6 gaussians").replace(
            "prec 1e-5", "prec 1e-4").replace("prec 1e-6", "prec 1e-5")
    a.warm = max(a.warmup, 3)
    return a


def dist_setup(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
        pg = dist
    return rank, world, local, pg


def reduce_max(pg, x):
    if pg is None:
        return x
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(pg, x):
    if pg is None:
        return x
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


def barrier(pg):
    if pg is not None:
        pg.barrier()


def make_input():
    import mrcpp_gb300 as mw
    from cases import gaussian_sum

    mra = mw.MRA(box=(-32, 32), order=ORDER, basis=mw.LEGENDRE)
    P = mw.PoissonOperator(mra, PREC) if MU is None else mw.HelmholtzOperator(mra, MU, PREC)
    f = mw.FunctionTree(mra)
    mw.project(PREC, f, gaussian_sum(SEED, NGAUSS, EXP_RANGE, CENTRE_RANGE))
    return mra, P, f


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            parts = [x.strip() for x in l.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def cpu_oracle_rate(mra, P, f, grid, sample, threads, prepared=None):
    """CPU oracle (port of the reference) on every `sample`-th output node of the
    fixed grid.  Only the C oracle call is timed; the node-term count of the
    sample comes from an untimed counting run."""
    import mrcpp_gb300 as mw
    import oracle

    if prepared is None:
        g = mw.FunctionTree(mra)
        mw.copy_grid(g, grid)
        prepared = oracle.Prepared(PREC, g, P, f, max_iter=0)
        prepared.node_terms = prepared.run(threads, count_terms=True, sample=sample, export=False)["node_terms"]
    t0 = time.perf_counter()
    prepared.run(threads, count_terms=False, sample=sample, export=False, fast=True)
    dt = time.perf_counter() - t0
    return prepared.node_terms / dt, dt, prepared.node_terms, prepared


def run_reference(args, rank, world, pg):
    if rank != 0:
        return
    import mrcpp_gb300 as mw
    import oracle

    threads = os.cpu_count() or 1
    mra, P, f = make_input()
    grid = oracle.to_tree(oracle.apply(PREC, mw.FunctionTree(mra), P, f, nthreads=threads, count_terms=False), mra)
    sample = 8
    prep = None
    for _ in range(args.warmup):
        _, _, _, prep = cpu_oracle_rate(mra, P, f, grid, sample, threads, prep)
    rates, times, nts = [], [], []
    for _ in range(args.steps):
        r, dt, nt, prep = cpu_oracle_rate(mra, P, f, grid, sample, threads, prep)
        rates.append(r)
        times.append(dt)
        nts.append(nt)
    value = sum(nts) / sum(times)
    desc = "every %d-th output node of the %d-node fixed grid (%d node-terms per step)" % (sample, grid.n_nodes, nts[0])
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(times), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "out_nodes": grid.n_nodes, "sample": desc},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": desc + "; CPU oracle restating ConvolutionCalculator (reference needs Eigen 3.4, absent)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def load_peaks():
    for p in (os.path.join(ROOT, "MEASURED_PEAKS.json"),):
        if os.path.exists(p):
            with open(p) as fh:
                d = json.load(fh)
            return d.get("bf16_tflops"), d.get("hbm_gbs"), "measured"
    return 1900.0, 6800.0, "fallback"


def load_traffic():
    p = os.path.join(ROOT, "profiles", "contract_poisson_k7_fixed.json")
    if os.path.exists(p):
        with open(p) as fh:
            return json.load(fh)
    return None


def main():
    args = parse()
    rank, world, local, pg = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, world, pg)
        barrier(pg)
        return
    os.environ["MWGPU_DEVICE"] = str(local)
    import ctypes as C

    import mrcpp_gb300 as mw

    mra, P, f = make_input()
    # fixed output grid: the adaptive FP64 apply
    grid = mw.FunctionTree(mra)
    mw.apply(PREC, grid, P, f, precision=mw.FP64)
    L = mw.lib()

    ctx = C.c_void_p()
    cfg = mw.MwgpuConfig()
    cfg.device = local
    cfg.precision = mw.MIXED
    if L.mwgpu_init(C.byref(ctx), C.byref(cfg)) != 0:
        raise SystemExit("mwgpu_init failed: %s" % L.mwgpu_last_error(None).decode())

    def ck(rc):
        if rc != 0:
            raise SystemExit("mwgpu error %d: %s" % (rc, L.mwgpu_last_error(ctx).decode()))

    od = P.desc()
    dop = C.c_void_p()
    ck(L.mwgpu_upload_operator(ctx, C.byref(mra.desc()), C.byref(od), PREC, C.byref(dop)))
    fx = f.export()
    fd = mw.MwgpuTreeDesc(len(fx["child0"]), mw._pi(fx["idx"]), mw._pi(fx["child0"]), mw._pd(fx["coefs"]), mw._pd(fx["norms"]))
    dinp = C.c_void_p()
    ck(L.mwgpu_upload_tree(ctx, C.byref(mra.desc()), C.byref(fd), C.byref(dinp)))
    gx = grid.export()
    gdesc = mw.MwgpuTreeDesc(len(gx["child0"]), mw._pi(gx["idx"]), mw._pi(gx["child0"]), None, None)
    dout = C.c_void_p()
    ck(L.mwgpu_create_tree(ctx, C.byref(mra.desc()), C.byref(gdesc), C.byref(dout)))
    n_out = len(gx["child0"])
    work = np.arange(n_out, dtype=np.int32)
    K = ORDER + 1
    flop_per_nt = 96.0 * K ** 4
    scrub = 256 << 20  # > 129 MB L2

    def step(precision):
        ck(L.mwgpu_set_precision(ctx, precision))
        ck(L.mwgpu_scrub_l2(ctx, scrub))
        ck(L.mwgpu_timer_mark(ctx, 0))
        ck(L.mwgpu_tree_clear_generated(ctx, dinp))
        st = mw.MwgpuLevelStats()
        ck(L.mwgpu_apply_level(ctx, dop, dinp, dout, mw._pi(work), n_out, PREC, -1.0, None, C.byref(st)))
        ck(L.mwgpu_transform(ctx, dout, 0, 0))
        ck(L.mwgpu_transform(ctx, dout, 1, 1))
        ck(L.mwgpu_timer_mark(ctx, 1))
        ms = C.c_double()
        ck(L.mwgpu_timer_elapsed(ctx, 0, 1, C.byref(ms)))
        return ms.value, st

    def timed(precision):
        for _ in range(args.warm):
            step(precision)
        barrier(pg)
        ck(L.mwgpu_sync(ctx))
        l0 = C.c_ulonglong()
        ck(L.mwgpu_launch_count(ctx, C.byref(l0)))
        with ClockSampler(local) as cs:
            res = [step(precision) for _ in range(args.steps)]
        ck(L.mwgpu_sync(ctx))
        l1 = C.c_ulonglong()
        ck(L.mwgpu_launch_count(ctx, C.byref(l1)))
        barrier(pg)
        ms = [r[0] for r in res]
        return ms, res[-1][1], cs.summary(), (l1.value - l0.value)

    ms_mixed, st_mixed, clk, launches = timed(mw.MIXED)
    out_mixed = np.zeros((n_out, 8 * K ** 3))
    ck(L.mwgpu_download_tree(ctx, dout, mw._pd(out_mixed), None))
    ms_fp64, st_fp64, clk64, _ = timed(mw.FP64)
    out_fp64 = np.zeros((n_out, 8 * K ** 3))
    ck(L.mwgpu_download_tree(ctx, dout, mw._pd(out_fp64), None))
    rel_l2 = float(np.linalg.norm(out_mixed - out_fp64) / np.linalg.norm(out_fp64))
    node_err = float((np.linalg.norm(out_mixed - out_fp64, axis=1) / np.linalg.norm(out_fp64, axis=1).max()).max())

    node_terms = st_mixed.node_terms
    t_mixed = reduce_max(pg, statistics.mean(ms_mixed))
    t_fp64 = reduce_max(pg, statistics.mean(ms_fp64))
    total_nt = reduce_sum(pg, node_terms)
    value = total_nt / (t_mixed / 1e3)
    value_fp64 = reduce_sum(pg, st_fp64.node_terms) / (t_fp64 / 1e3)

    # end to end through the public apply (host buffers in, host buffers out)
    e2e_times, h2d, d2h = [], 0, 0
    for i in range(max(args.warmup, 1) + args.steps):
        g = mw.FunctionTree(mra)
        mw.copy_grid(g, grid)
        barrier(pg)
        t0 = time.perf_counter()
        s = mw.apply(PREC, g, P, f, max_iter=0, precision=mw.MIXED)
        dt = time.perf_counter() - t0
        if i >= max(args.warmup, 1):
            e2e_times.append(dt)
            h2d, d2h = s["h2d_bytes"], s["d2h_bytes"]
    t_e2e = reduce_max(pg, statistics.mean(e2e_times))
    e2e_value = total_nt / t_e2e

    # roofline of the contraction kernel (mixed form, last timed launch)
    bf16_peak, hbm_peak, peak_kind = load_peaks()
    achieved = node_terms * flop_per_nt / (st_mixed.contract_ms / 1e3) / 1e12
    tr = load_traffic() if (args.workload == "poisson" and not args.small) else None
    roof = {"bound": "tensor", "achieved": achieved, "peak": bf16_peak, "unit": "TFLOP/s", "frac": achieved / bf16_peak,
            "traffic": (tr or {}).get("dram_bytes_per_launch"), "peak_kind": peak_kind + " bf16 dense burst",
            "kernel": "k_contract<float> (mixed form)", "kernel_ms": st_mixed.contract_ms,
            "flop_per_node_term": flop_per_nt}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rate, dt, nt, _ = cpu_oracle_rate(mra, P, f, grid, 8, threads)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "every 8th output node of the fixed grid (%d node-terms, %.1f s)" % (nt, dt)}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warm,
                "ms_per_step": t_mixed, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32 products, f64 accumulation", "data": "synthetic",
                "config": {"workload": WORKLOAD, "out_nodes": n_out, "node_terms_per_step": int(node_terms),
                           "components_per_step": int(st_mixed.components), "l2": "256 MiB scrub between steps",
                           "parallelism": "replicas" if world > 1 else "single"},
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                        "ms_per_step": t_e2e * 1e3},
                "fp64": {"value": value_fp64, "unit": UNIT, "ms_per_step": t_fp64, "contract_ms": st_fp64.contract_ms},
                "mixed_vs_fp64": {"speedup": value / value_fp64, "rel_l2_error": rel_l2, "max_node_error": node_err},
                "roofline": roof, "cpu_baseline": cpu, "clocks": clk, "gpu_launches": int(launches)}
        print(json.dumps(line), flush=True)
    barrier(pg)


if __name__ == "__main__":
    main()
