"""Benchmark of the lattice max-flow engine on one GB300 (or N replicas).

Default workload: the single large 2-d cut, 2048x2048 Full2d_8, int32
capacities (seeded synthetic image, see latticeflow_gb300/workloads.py).
A step is one complete exact solve: clear the lattice, fill the energies,
push-relabel to a maximum preflow, both canonical cut sets, flow value.

  value  solves/s with the energies already resident in HBM
  e2e    the same through the reference-facing C-ABI call with host buffers:
         addEnergyPotentials from pinned host int64 arrays (H2D inside the
         step) and the minimal cut read back into a pinned host array (D2H
         inside the step), on 3 handles at once by default (--e2e-handles N),
         one host thread and stream each, so that one solve's transfer
         overlaps another's solve, as a server runs them; each handle's
         energies go through the copy engine into a device buffer it keeps
         (--host-stage 1); e2e.one_handle is one handle, solve after solve,
         with the fill kernel reading the pinned arrays in place

The default line also carries: parity (the timed workload's energy and
both cut sets against the oracle), batched_vs_plain (the 512-lattice batch
against 512 plain solves), tv_single_1024 (single-lambda TV of the 1024^2
polygon image through the public call, beside the restated reference on one
core) and serve (p50 / p99 latency of a short Poisson stream of TV
requests).  --workload tv_path times the regularisation path.

Multi-GPU: independent replicas (the path has no exchange step); value is the
solves of all ranks over the max-over-ranks time ("scaling": "weak").

--impl reference times the reference algorithm on the host cores instead:
the CPU restatement of the reference push-relabel (oracle port), one solve per
host core in parallel per step.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "max-flow solves/s & HBM GB/s, batched vs plain on GB300 (exact cut); TV p99 ms"
UNIT = "solves/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="large_cut",
                    choices=["large_cut", "plain_cut", "volume_cut", "batch", "serve", "tv_path"])
    ap.add_argument("--requests", type=int, default=200, help="serve: measured requests")
    ap.add_argument("--rate", type=float, default=200.0, help="serve: mean arrivals per second")
    ap.add_argument("--workers", type=int, default=4, help="serve: server workers")
    ap.add_argument("--max-group", type=int, default=8,
                    help="serve: largest group of same-shape TV requests solved together")
    ap.add_argument("--batch-size", type=int, default=512)
    ap.add_argument("--tv-n", type=int, default=256,
                    help="tv_path: side of the TV image (config 5 names 1024)")
    ap.add_argument("--no-tv-summary", action="store_true",
                    help="skip the single-lambda TV and serving summaries of the default run")
    ap.add_argument("--no-batch-summary", action="store_true",
                    help="skip the batched-vs-plain summary of the default run")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--profile-run", action="store_true",
                    help="only warm-up and timed device-resident solves (for ncu captures)")
    ap.add_argument("--host-loops", action="store_true",
                    help="one launch per pass (the default; kept for the recorded profiling commands)")
    ap.add_argument("--device-loops", action="store_true",
                    help="run the staged passes in device-side loops (CUDA graphs with conditional "
                         "nodes, whose kernels a profiler does not list); one handle only: "
                         "give --e2e-handles 1 with it")
    ap.add_argument("--e2e-handles", type=int, default=3,
                    help="e2e with this many handles (own streams, own host threads) solving "
                         "concurrently, so one solve's host-to-device fill overlaps another's solve; "
                         "timed by the host clock around all of them")
    ap.add_argument("--host-stage", type=int, default=1, choices=[0, 1],
                    help="e2e on several handles: pinned host energies copied into HBM by "
                         "the copy engine first (1, so that the SMs stay free for the other "
                         "handles' solves during a transfer) or read in place by the fill "
                         "kernel (0); e2e.one_handle always reads in place, the faster form "
                         "for solves run one after another")
    ap.add_argument("--tuning", default=None,
                    help="tile_rows,local_sweeps,launches_per_relabel instead of the autotuner "
                         "(e.g. the setting a bench run chose, for a profile run)")
    args = ap.parse_args()
    if args.device_loops and args.e2e_handles > 1:
        # device-side loops run on one handle and one host thread only
        ap.error("--device-loops takes one handle: it cannot be combined with --e2e-handles > 1")
    return args


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_workload(name, seed):
    from latticeflow_gb300 import workloads as W
    if name == "large_cut":
        return W.large_cut(seed)
    if name == "plain_cut":
        return W.plain_cut(seed)
    if name == "volume_cut":
        return W.volume_cut(seed)
    raise ValueError(name)


def workload_config(name, p):
    return {"workload": name, "kernel": p.kernel, "shape": list(p.dims), "capacity": "int32",
            "seed": 0, "l2": "inputs larger than L2 (no flush needed)"}


# ---------------------------------------------------------------- clocks

class ClockSampler(object):
    """nvidia-smi samples during the timed region (read only)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def committed_traffic(kernel_key):
    """DRAM bytes per node visit of a kernel from a committed ncu capture
    (profiles/traffic.json, keyed workload:kernel:tile), if present."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        v = d.get(kernel_key)
        if isinstance(v, dict):
            return v
    return None


def max_over_ranks(x):
    """The largest x over all ranks (replicas time their own work; the job
    takes as long as the slowest).  One process: x itself."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_split(step_fns, steps):
    """Run `steps` steps spread over len(step_fns) host threads, thread j
    calling step_fns[j] (its own handle and stream) for its share, round
    robin; returns the last result of thread 0.  An exception in any thread
    is raised here after every thread has stopped."""
    nh = len(step_fns)
    counts = [steps // nh + (1 if j < steps % nh else 0) for j in range(nh)]
    results = [None] * nh
    errors = []

    def work(j):
        try:
            for _ in range(counts[j]):
                if errors:
                    return
                results[j] = step_fns[j]()
        except BaseException as e:  # re-raised on the calling thread
            errors.append(e)

    threads = [threading.Thread(target=work, args=(j,)) for j in range(nh)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    if errors:
        raise errors[0]
    return results[0]


def replica_value(units_per_rank, world, seconds):
    """Whole-job throughput of `world` replicas: all units over the
    max-over-ranks time."""
    return world * units_per_rank / seconds


# ---------------------------------------------------------------- ours

def run_ours(args):
    import torch
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from latticeflow_gb300 import _build
    _build.build_native()
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import _native as N

    p = make_workload(args.workload, args.seed)
    u, b = p.energies()
    hu = torch.from_numpy(u).pin_memory()
    hb = torch.from_numpy(b).pin_memory()
    du = hu.cuda()
    db = hb.cuda()
    torch.cuda.synchronize()
    L = lf.LatticeFlow(p.kernel, "LatticeEnergyMinimizer", p.dims)
    lib = N.lib()
    h = L._h
    stream = torch.cuda.ExternalStream(L.stream())

    def step_device():
        N.check(lib.lf_clear(h))
        N.check(lib.lf_add_energy_potentials_device(h, ctypes.c_void_p(du.data_ptr()),
                                                    ctypes.c_void_p(db.data_ptr())))
        N.check(lib.lf_run(h))
        return L.flow()

    cut_t = torch.empty(p.n, dtype=torch.int32).pin_memory()  # pinned, like the inputs
    cut = cut_t.numpy()

    def step_e2e():
        N.check(lib.lf_clear(h))
        N.check(lib.lf_add_energy_potentials(h, ctypes.c_void_p(hu.data_ptr()),
                                             ctypes.c_void_p(hb.data_ptr())))
        N.check(lib.lf_run(h))
        N.check(lib.lf_get_cut(h, cut.ctypes.data_as(ctypes.c_void_p)))
        return L.flow()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    def timed(fn, steps, profile):
        barrier()
        torch.cuda.synchronize()
        L.setProfiling(profile)
        prof = {"pr_ms": 0.0, "bfs_ms": 0.0, "reach_ms": 0.0, "pr_tiles": 0, "pr_launches": 0,
                "bfs_passes": 0, "bfs_tiles": 0}
        k0 = L.profile()["kernel_launches"]
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        res = None
        for _ in range(steps):
            res = fn()
            pr = L.profile()
            for k in prof:
                prof[k] += pr[k]
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        launches = L.profile()["kernel_launches"] - k0
        L.setProfiling(False)
        ms = max_over_ranks(ms)
        barrier()
        return ms, res, prof, launches

    tuning = None
    tune_table = None
    if args.device_loops and not args.host_loops:
        L.setParam("device_loops", 1)
    if args.tuning:
        tr_, sw_, lp_ = (int(x) for x in args.tuning.split(","))
        tuning = {"tile_rows": tr_, "local_sweeps": sw_, "launches_per_relabel": lp_}
        for k_, v_ in tuning.items():
            L.setParam(k_, v_)
    elif not args.no_autotune and not args.profile_run:
        from latticeflow_gb300 import autotune
        step_device()
        grid = autotune.VOLUME_GRID if len(p.dims) == 3 else None
        tuning, _, tune_table = autotune.tune(L, autotune.problem_key([p.kernel], p.n), grid=grid)
    if args.profile_run:
        # every solve of the run (warm-up included), with the tile counters
        # that turn a capture's DRAM bytes into bytes per node visit
        tot = {"pr_tiles": 0, "pr_launches": 0, "bfs_tiles": 0, "bfs_passes": 0}
        for _ in range(args.warmup + args.steps):
            step_device()
            pr = L.profile()
            for k in tot:
                tot[k] += pr[k]
        torch.cuda.synchronize()
        tile, _, elem = L.layout()
        print(json.dumps(dict(profile_run=True, flow=L.flow()[0], solves=args.warmup + args.steps,
                              tile=list(tile), elem_bytes=elem, tuning=tuning, **tot)))
        return
    for _ in range(args.warmup):
        step_device()
    sampler = ClockSampler(local)
    sampler.start()
    # value: plain timed steps; then the same steps with CUDA events around
    # every launch for the per-kernel split (events add host work per launch)
    ms, res, _, launches = timed(step_device, args.steps, False)
    clocks = sampler.stop()
    ms_prof, _, prof, _ = timed(step_device, args.steps, True)
    e2e_timing = "CUDA events on the handle's stream"
    L.setParam("host_stage", 0 if args.e2e_handles > 1 else args.host_stage)
    for _ in range(max(1, args.warmup)):
        step_e2e()
    ms_e2e, _, _, _ = timed(step_e2e, args.steps, False)
    ms_e2e_one = ms_e2e
    if args.e2e_handles > 1:
        L.setParam("host_stage", args.host_stage)
        # more handles of the same lattice, tuned alike; each thread's step is
        # the same public calls as step_e2e on its own handle and cut buffer
        extra = []
        for _ in range(args.e2e_handles - 1):
            Lx = lf.LatticeFlow(p.kernel, "LatticeEnergyMinimizer", p.dims)
            for k_, v_ in (tuning or {}).items():
                Lx.setParam(k_, v_)
            Lx.setParam("host_stage", args.host_stage)
            cx = torch.empty(p.n, dtype=torch.int32).pin_memory()
            extra.append((Lx, cx))

        def step_on(Lx, cx):
            def step():
                hx = Lx._h
                N.check(lib.lf_clear(hx))
                N.check(lib.lf_add_energy_potentials(hx, ctypes.c_void_p(hu.data_ptr()),
                                                     ctypes.c_void_p(hb.data_ptr())))
                N.check(lib.lf_run(hx))
                N.check(lib.lf_get_cut(hx, ctypes.c_void_p(cx.data_ptr())))
                return Lx.flow()
            return step

        fns = [step_e2e] + [step_on(Lx, cx) for Lx, cx in extra]
        run_split(fns, max(1, args.warmup) * len(fns))
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        run_split(fns, args.steps)
        torch.cuda.synchronize()
        ms_e2e = max_over_ranks((time.perf_counter() - t0) * 1e3)
        barrier()
        e2e_timing = "host clock around %d handles solving concurrently" % len(fns)
        del extra, fns

    autotune_top = None
    if tune_table:
        autotune_top = [dict(s_, ms=round(1e3 * t_, 3)) for s_, t_ in sorted(tune_table, key=lambda x: x[1])[:4]]
    tile, padded, elem = L.layout()
    nt = tile[0] * tile[1] * tile[2]
    K = 2 * L.nFillingEdges
    peak, peak_kind = measured_peaks()
    pr_bytes = prof["pr_tiles"] * nt * 2 * (K * elem + elem + 4)
    bfs_bytes = prof["bfs_tiles"] * nt * (8 + 4 + 4)
    # a single 2-d lattice with a 3x3 stencil runs the TMA-staged passes
    # (k_pool_pr2d for 32-bit capacities, k_pool_bfs2d for any); other
    # lattices the generic tile kernels
    tma2d = p.kernel in ("Full2d_4", "Full2d_8") and len(p.dims) == 2
    prk = (tuning or {}).get("pr_kernel", 0)
    # a single 3-d lattice with a radius-1 stencil and 32-bit capacities runs
    # the TMA-staged 3-d pass on 4-plane tiles it fits (any height for 6
    # directions, up to 4 rows for 18 and 26)
    rows3 = {"Full3d_6": 8, "Full3d_18": 4, "Full3d_26": 4}.get(p.kernel, 0)
    tma3d = (len(p.dims) == 3 and elem == 4 and prk != 1 and tile[0] == 4
             and tile[1] <= rows3)
    pr_name = ("k_pool_pr2d" if tma2d and elem == 4 else
               "k_pool_pr3d" if tma3d else "k_pool_pr")
    bfs_name = "k_pool_bfs2d" if tma2d else "k_pool_bfs"
    if prof["pr_ms"] >= prof["bfs_ms"]:
        kname, kbytes, kms, klaunch = pr_name, pr_bytes, prof["pr_ms"], prof["pr_launches"]
    else:
        kname, kbytes, kms, klaunch = bfs_name, bfs_bytes, prof["bfs_ms"], prof["bfs_passes"]
    achieved = kbytes / (kms * 1e-3) / 1e9 if kms > 0 else 0.0
    tr = committed_traffic("%s:%s:%s" % (args.workload, kname, "x".join(str(v) for v in tile)))
    klaunch_nodes = (prof["pr_tiles"] if kname.startswith("k_pool_pr") else prof["bfs_tiles"]) * nt / max(1, klaunch)
    roofline = {"bound": "hbm", "kernel": kname, "achieved": round(achieved, 1),
                "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs, copy)",
                # DRAM bytes per node visit from a committed ncu capture of the
                # same kernel and workload, times this run's node visits per launch
                "traffic": int(tr["dram_bytes_per_node_visit"] * klaunch_nodes) if tr else None,
                "traffic_source": tr.get("source") if tr else "no committed capture for this tile shape",
                "algorithmic_bytes_per_launch": int(kbytes / max(1, klaunch)),
                "kernel_ms_share": round(kms / max(ms_prof, 1e-9), 3),
                "launches": int(klaunch)}

    value = replica_value(args.steps, world, ms * 1e-3)
    e2e_value = replica_value(args.steps, world, ms_e2e * 1e-3)
    out = {
        "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded generator, latticeflow_gb300/workloads.py)",
        "config": dict(workload_config(args.workload, p), parallelism="replicas" if world > 1 else "single",
                       tuning=tuning, autotuned=tuning is not None and not args.tuning,
                       autotune_top=autotune_top),
        "e2e": {"value": round(e2e_value, 4), "unit": UNIT,
                "h2d_bytes_per_step": int(u.nbytes + b.nbytes),
                "d2h_bytes_per_step": int(p.n * 4 + 24),  # the cut, flow/supply/energy
                "handles": args.e2e_handles, "timing": e2e_timing,
                "host_read": ("copy engine into HBM, then fill" if args.host_stage else
                              "fill kernel reads the pinned arrays in place")
                             + ("; one_handle: in place" if args.e2e_handles > 1 else ""),
                "one_handle": round(replica_value(args.steps, world, ms_e2e_one * 1e-3), 4)},
        "roofline": roofline,
        "clocks": clocks,
        "gpu_launches": int(launches),
        "solver": {"flow": res[0], "energy": res[1], "profile_ms": {k: (round(v, 3) if isinstance(v, float) else v) for k, v in prof.items()},
                   "tile": list(tile), "elem_bytes": elem},
    }
    if rank == 0:
        out["cpu_baseline"] = cpu_baseline(p)
        out["parity"] = parity_check(p, L)
        if not args.no_batch_summary and not args.profile_run:
            del L
            out["batched_vs_plain"] = batch_summary(args)
        if not args.no_tv_summary and not args.profile_run:
            out["tv_single_1024"] = tv_single_summary()
            out["serve"] = serve_summary(args)
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def make_batch(count, seed=0):
    from latticeflow_gb300 import workloads as W
    return W.batch(count, seed=seed)


def fill_batch(B, probs):
    for i, p in enumerate(probs):
        B.addCapacities(i, p.source, p.sink, p.edge)


def batch_summary(args, steps=3):
    """Batched (one pool) vs sequential plain solves of the same lattices."""
    import torch
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import autotune
    probs = make_batch(args.batch_size)
    B = lf.LatticeBatch()
    for p in probs:
        B.add(p.kernel, p.dims)
    B.setParam("defer_checks", 1)
    fill_batch(B, probs)
    B.run()
    setting, _, _ = autotune.tune(B, autotune.problem_key([p.kernel for p in probs],
                                                          sum(p.n for p in probs)))
    torch.cuda.synchronize()
    tb = []
    for _ in range(steps):
        B.run()
        tb.append(B.runTime())
    plain = []
    for p in probs:
        L = lf.LatticeFlow(p.kernel, "LatticeEnergyMinimizer", p.dims)
        L.addCapacities(p.source, p.sink, p.edge)
        plain.append(L)
    for L in plain[:4]:
        L.run()
    tp = []
    for _ in range(max(1, steps - 1)):
        t = 0.0
        for L in plain:
            L.run()
            t += L.runTime()
        tp.append(t)
    mism = sum(1 for i, L in enumerate(plain)
               if L.flow() != B.flow(i) or not np.array_equal(L.getCut(), B.getCut(i)))
    n = len(probs)
    return {"lattices": n, "nodes": int(sum(p.n for p in probs)),
            "batched_solves_per_s": round(n / min(tb), 2),
            "plain_solves_per_s": round(n / min(tp), 2),
            "speedup": round(min(tp) / min(tb), 2), "tuning": setting,
            "results_differ": mism,
            "timing": "device time of complete solves (CUDA events), best of %d" % steps}


def run_batch(args):
    """--workload batch: 512 uneven lattices, one pool solve per step."""
    import torch
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from latticeflow_gb300 import _build
    _build.build_native()
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import autotune
    probs = make_batch(args.batch_size, seed=args.seed)
    B = lf.LatticeBatch()
    for p in probs:
        B.add(p.kernel, p.dims)
    B.setParam("defer_checks", 1)
    fill_batch(B, probs)
    B.run()
    setting = None
    if not args.no_autotune:
        setting, _, _ = autotune.tune(B, autotune.problem_key([p.kernel for p in probs],
                                                              sum(p.n for p in probs)))
    for _ in range(args.warmup):
        B.run()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    t0 = time.perf_counter()
    dev = 0.0
    for _ in range(args.steps):
        B.run()
        dev += B.runTime()
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    # e2e: host capacities in (one packed call, pinned host arrays), every
    # lattice's minimal cut out (one packed call into a pinned host array)
    def pinned(a):
        t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        return t.numpy()
    src_all = pinned(np.concatenate([p.source for p in probs]))
    snk_all = pinned(np.concatenate([p.sink for p in probs]))
    edge_all = pinned(np.concatenate([p.edge.reshape(-1) for p in probs]))
    cut_buf = pinned(np.zeros(int(sum(p.n for p in probs)), dtype=np.int32))
    # one batch at a time: the fill kernel reading the pinned arrays in place
    # overlaps the transfer with the fill (8.9k against 8.1k solves/s with the
    # copy-engine staging, untuned)
    B.setParam("host_stage", 0)

    def step_e2e():
        B.clear()
        B.addCapacitiesPacked(src_all, snk_all, edge_all)
        B.run()
        B.getCutsPacked(out=cut_buf)

    step_e2e()  # the staging buffer is allocated once
    cut_bytes = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step_e2e()
        cut_bytes += cut_buf.nbytes
    wall_e2e = time.perf_counter() - t0
    n = len(probs)
    dev, wall, wall_e2e = max_over_ranks(dev), max_over_ranks(wall), max_over_ranks(wall_e2e)
    summary = batch_summary(args) if rank == 0 else None
    h2d = int(sum(p.source.nbytes + p.sink.nbytes + p.edge.nbytes for p in probs))
    out = {
        "metric": METRIC, "value": round(replica_value(n * args.steps, world, dev), 3), "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * dev / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded generator, latticeflow_gb300/workloads.py)",
        "config": {"workload": "batch", "lattices": n, "kernels": "Full2d_4 + Full2d_8",
                   "sides": "log-uniform [64, 1024] per axis", "capacity": "int32",
                   "tuning": setting, "autotuned": setting is not None,
                   "l2": "inputs larger than L2 (no flush needed)"},
        "e2e": {"value": round(replica_value(n * args.steps, world, wall_e2e), 3), "unit": UNIT,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": int(cut_bytes / args.steps),
                "host_read": "the fill kernel reads the pinned arrays in place"},
        "wall_ms_per_step": round(1e3 * wall / args.steps, 3),
        "clocks": clocks,
        "batched_vs_plain": summary,
    }
    if rank == 0:
        print(json.dumps(out))


SERVE_SIZES = (128, 256, 512, 1024, 2048)


def run_serve(args):
    """--workload serve: Poisson stream of single-lambda TV requests, sizes
    uniform over {128..2048}^2, lambda log-uniform in [1e-3, 1]."""
    import torch
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from latticeflow_gb300 import _build
    _build.build_native()
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import workloads as W
    rng = np.random.default_rng(args.seed)
    images = {n: W.tv_image(100 + i, n=n, polygons=30) for i, n in enumerate(SERVE_SIZES)}
    S = lf.LatticeServer(workers=args.workers, max_group=args.max_group)
    # warm-up: every size on every worker (engines built, kernels loaded);
    # a round of `workers` simultaneous requests spreads over the workers
    warm = []
    for _ in range(2):
        for n in SERVE_SIZES:
            ts = [S.submit_tv(images[n], 0.01) for _ in range(args.workers)]
            for t in ts:
                S.wait(t)
                S.release(t)
            warm += ts
    sizes = rng.choice(SERVE_SIZES, size=args.requests)
    lams = np.exp(rng.uniform(np.log(1e-3), np.log(1.0), size=args.requests))
    gaps = rng.exponential(1.0 / args.rate, size=args.requests)
    arrive = np.cumsum(gaps)
    tickets = []
    sampler = ClockSampler(local)
    sampler.start()
    t0 = time.perf_counter()
    for i in range(args.requests):
        delay = t0 + arrive[i] - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        tickets.append(S.submit_tv(images[int(sizes[i])], float(lams[i])))
    lat = []
    for t in tickets:
        lat.append(S.wait(t))
        S.release(t)
    makespan = max_over_ranks(time.perf_counter() - t0)
    clocks = sampler.stop()
    st = S.stats()
    S.close()
    lat_ms = np.sort(np.asarray(lat) * 1e3)
    per_size = {}
    for n in SERVE_SIZES:
        m = sizes == n
        if m.any():
            l = np.asarray(lat)[m] * 1e3
            per_size[str(n)] = {"count": int(m.sum()), "p50_ms": round(float(np.percentile(l, 50)), 2),
                                "p99_ms": round(float(np.percentile(l, 99)), 2)}
    out = {
        "metric": METRIC, "value": round(replica_value(args.requests, world, makespan), 3),
        "unit": "solves/s",
        "n_gpus": world, "steps": args.requests, "warmup": len(warm),
        "ms_per_step": round(1e3 * makespan / args.requests, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int64",
        "data": "synthetic (seeded polygon images, latticeflow_gb300/workloads.py)",
        "config": {"workload": "serve", "requests": args.requests, "rate_per_s": args.rate,
                   "sizes": list(SERVE_SIZES), "lambda": "log-uniform [1e-3, 1]",
                   "kernel": "Full2d_4", "workers": args.workers, "max_group": args.max_group},
        "latency_ms": {"p50": round(float(np.percentile(lat_ms, 50)), 2),
                       "p99": round(float(np.percentile(lat_ms, 99)), 2),
                       "max": round(float(lat_ms[-1]), 2)},
        "per_size": per_size, "max_in_flight": st["max_in_flight"],
        "grouping": {"max_group": args.max_group, "groups": st["groups"],
                     "grouped_requests": st["grouped_requests"]},
        "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(out))


TV_PATH_LAMBDAS = 64


def tv_path_lambdas():
    """64 values 1e-3 * 1000^(i/63): 1e-3 .. 1, log-spaced."""
    return np.array([1e-3 * 1000.0 ** (i / (TV_PATH_LAMBDAS - 1)) for i in range(TV_PATH_LAMBDAS)])


def tv_path_cpu_baseline(n, lams, seed, budget_s=30.0):
    """The restated reference path tracker on one host core, on the largest
    image of side n, n/2, n/4, ... whose path its time on a 64x64 image,
    scaled by the fourth power of the side (its observed growth), puts
    within the budget."""
    from oracle import oracle as O
    from latticeflow_gb300 import workloads as W
    O.build_port()
    _, t64, _ = O.port_tv_path("Full2d_4", W.tv_image(seed, n=64, polygons=30), lams)
    m = n
    while m > 64 and t64 * (m / 64.0) ** 4 > budget_s:
        m //= 2
    f = W.tv_image(seed, n=m, polygons=30)
    _, secs, segs = O.port_tv_path("Full2d_4", f, lams)
    return {"value": round(1.0 / secs, 5), "unit": "paths/s", "cores": 1, "kind": "port",
            "sample": "one %d-lambda path of the %dx%d image (%d segments), the reference's "
                      "path tracker restated (oracle/lf_oracle.cpp), %.2f s%s"
                      % (len(lams), m, m, segs, secs,
                         "" if m == n else "; the %dx%d path is beyond the budget" % (n, n)),
            "side": m}


def run_tv_path(args):
    """--workload tv_path: the regularisation path (calculate2dTVPath, the
    reference's path tracker with its region probes on the GPU) of an
    --tv-n square polygon image at 64 lambdas, host arrays in and out.  A
    step is one whole path; value = paths per second."""
    import torch
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from latticeflow_gb300 import _build
    _build.build_native()
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import workloads as W
    n = args.tv_n
    f = W.tv_image(args.seed, n=n, polygons=30)
    lams = tv_path_lambdas()
    for _ in range(args.warmup):
        lf.calculate2dTVPath(f, lams)
    if world > 1:
        dist.barrier()
    sampler = ClockSampler(local)
    sampler.start()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        P, st = lf.calculate2dTVPath(f, lams, return_stats=True)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    wall = max_over_ranks(wall)
    value = replica_value(args.steps, world, wall)
    out = {
        "metric": METRIC, "value": round(value, 5), "unit": "paths/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * wall / args.steps, 2), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int64",
        "data": "synthetic (seeded polygon image, latticeflow_gb300/workloads.py)",
        "config": {"workload": "tv_path", "kernel": "Full2d_4", "shape": [n, n],
                   "lambdas": "64 values 1e-3*1000^(i/63)", "seed": args.seed,
                   "parallelism": "replicas" if world > 1 else "single"},
        "e2e": {"value": round(value, 5), "unit": "paths/s",
                "h2d_bytes_per_step": int(f.nbytes), "d2h_bytes_per_step": int(P.nbytes),
                "note": "the step is the public host-array call itself"},
        "path": {k: (round(float(v), 3) if isinstance(v, float) else v) for k, v in st.items()},
        "clocks": clocks,
    }
    if rank == 0:
        out["cpu_baseline"] = tv_path_cpu_baseline(n, lams, args.seed)
        print(json.dumps(out))


def tv_single_summary(lams=(1e-3, 0.05, 1.0), n=1024):
    """Single-lambda TV of the 1024x1024 polygon image through the public
    call (host arrays), at three lambdas; the restated reference solve of
    the middle one on one host core, and its parity."""
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import workloads as W
    from oracle import oracle as O
    f = W.tv_image(0, n=n, polygons=30)
    lf.calculate2dTV(f[:64, :64], 0.05)  # loads the kernels
    secs, outs = [], []
    for lam in lams:
        t0 = time.perf_counter()
        outs.append(lf.calculate2dTV(f, lam))
        secs.append(time.perf_counter() - t0)
    O.build_port()
    mid = len(lams) // 2
    ref, _, cpu_s = O.port_tv_single("Full2d_4", f, lams[mid])
    ok = float(np.abs(outs[mid] - ref).max()) <= 1e-9 * max(1.0, float(np.abs(ref).max()))
    return {"shape": [n, n], "lambdas": list(lams), "s_per_lambda": [round(x, 4) for x in secs],
            "mean_s": round(float(np.mean(secs)), 4),
            "cpu_port_s": round(cpu_s, 3), "cpu_port_lambda": lams[mid], "cpu_cores": 1,
            "parity": bool(ok),
            "timing": "host clock around the public call (host arrays in and out)"}


def serve_summary(args, requests=30, rate=1.0, workers=4):
    """A short Poisson stream of single-lambda TV requests (config 5 sizes
    {128..2048}^2, lambda log-uniform in [1e-3, 1]) at a rate the server
    sustains on one GPU: p50 / p99 latency (submission to completion) and
    solves per second."""
    import latticeflow_gb300 as lf
    from latticeflow_gb300 import workloads as W
    rng = np.random.default_rng(args.seed + 7)
    images = {n: W.tv_image(100 + i, n=n, polygons=30) for i, n in enumerate(SERVE_SIZES)}
    S = lf.LatticeServer(workers=workers, max_group=8)
    for n in SERVE_SIZES:  # engines built and kernels loaded on every worker
        ts = [S.submit_tv(images[n], 0.01) for _ in range(workers)]
        for t in ts:
            S.wait(t)
            S.release(t)
    sizes = rng.choice(SERVE_SIZES, size=requests)
    lams = np.exp(rng.uniform(np.log(1e-3), np.log(1.0), size=requests))
    arrive = np.cumsum(rng.exponential(1.0 / rate, size=requests))
    t0 = time.perf_counter()
    tickets = []
    for i in range(requests):
        delay = t0 + arrive[i] - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        tickets.append(S.submit_tv(images[int(sizes[i])], float(lams[i])))
    lat = []
    for t in tickets:
        lat.append(S.wait(t))
        S.release(t)
    makespan = time.perf_counter() - t0
    st = S.stats()
    S.close()
    lat_ms = np.asarray(lat) * 1e3
    return {"requests": requests, "rate_per_s": rate, "workers": workers,
            "sizes": list(SERVE_SIZES), "p50_ms": round(float(np.percentile(lat_ms, 50)), 1),
            "p99_ms": round(float(np.percentile(lat_ms, 99)), 1),
            "solves_per_s": round(requests / makespan, 3), "max_in_flight": st["max_in_flight"]}


def cpu_baseline(p, budget_s=12.0):
    """Restated reference push-relabel on one host core, same workload."""
    from oracle import oracle as O
    O.build_port()
    u, b = p.energies()
    times = []
    t0 = time.time()
    while not times or (time.time() - t0 < budget_s and len(times) < 20):
        _, secs = O.port_pr(p.kernel, p.dims, u, b)
        times.append(secs)
    return {"value": round(len(times) / sum(times), 4), "unit": UNIT, "cores": 1, "kind": "port",
            "sample": "%d full solves of the same workload, reference push-relabel restated "
                      "(oracle/lf_oracle.cpp), median %.3f s" % (len(times), float(np.median(times)))}


def parity_check(p, L):
    """The timed workload's result against the oracle (the restated reference
    solver on the same input): minimum energy, minimal and maximal on-sets."""
    from oracle import oracle as O
    O.build_port()
    u, b = p.energies()
    E, cmin, cmax, _, _ = O.port_canonical(p.kernel, p.dims, u, b)
    energy = L.flow()[1]
    ok = energy == E and np.array_equal(L.getCut(), cmin) and np.array_equal(L.getCutMax(), cmax)
    return bool(ok)


# ---------------------------------------------------------------- reference

_W = {}


def _ref_init(workload, seed, batch_size=512, tv_n=256):
    sys.path.insert(0, ROOT)
    _W["tv_n"] = tv_n
    from oracle import oracle as O
    O.port()
    if workload == "batch":
        _W["batch"] = make_batch(batch_size, seed=seed)
        return
    if workload == "tv_path":
        from latticeflow_gb300 import workloads as W
        _W["tv"] = (W.tv_image(seed, n=_W.get("tv_n", 256), polygons=30), tv_path_lambdas())
        return
    p = make_workload(workload, seed)
    _W["p"] = p
    _W["e"] = p.energies()


def _ref_solve(arg):
    from oracle import oracle as O
    if "tv" in _W:
        f, lams = _W["tv"]
        _, secs, _ = O.port_tv_path("Full2d_4", f, lams)
        return secs
    if "batch" in _W:
        secs = 0.0
        for i in arg:
            p = _W["batch"][i]
            _, s = O.port_pr(p.kernel, p.dims, *p.energies())
            secs += s
        return secs
    p = _W["p"]
    u, b = _W["e"]
    _, secs = O.port_pr(p.kernel, p.dims, u, b)
    return secs


def run_reference(args):
    rank, world, local = dist_info()
    if rank != 0:
        return
    import multiprocessing as mp
    from oracle import oracle as O
    O.build_port()
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    if args.workload == "batch":
        p = None
        per_step = args.batch_size
        work = [list(range(c, args.batch_size, cores)) for c in range(cores)]
    elif args.workload == "tv_path":
        p = None
        per_step = cores
        work = list(range(cores))  # one whole path per core
    else:
        p = make_workload(args.workload, args.seed)
        per_step = cores
        work = list(range(cores))
    with ctx.Pool(cores, initializer=_ref_init,
                  initargs=(args.workload, args.seed, args.batch_size, args.tv_n)) as pool:
        for _ in range(args.warmup):
            pool.map(_ref_solve, work, chunksize=1)
        t0 = time.time()
        for _ in range(args.steps):
            pool.map(_ref_solve, work, chunksize=1)
        wall = time.time() - t0
    value = per_step * args.steps / wall
    kind = "port"
    unit = "paths/s" if args.workload == "tv_path" else UNIT
    out = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": unit,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * wall / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int64",
        "data": "synthetic (seeded generator, latticeflow_gb300/workloads.py)",
        "config": (workload_config(args.workload, p) if p is not None else
                   {"workload": "batch", "lattices": args.batch_size}
                   if args.workload == "batch" else
                   {"workload": "tv_path", "kernel": "Full2d_4", "shape": [args.tv_n, args.tv_n],
                    "lambdas": "64 values 1e-3*1000^(i/63)", "seed": args.seed}),
        "cpu_baseline": {"value": round(value, 4), "unit": unit, "cores": cores, "kind": kind,
                         "sample": ("each step: one full solve per host core in parallel"
                                    " (reference push-relabel restated, oracle/lf_oracle.cpp)"
                                    if p is not None else
                                    "each step: all %d lattices spread over the host cores"
                                    " (reference push-relabel restated, oracle/lf_oracle.cpp)"
                                    % args.batch_size if args.workload == "batch" else
                                    "each step: one whole 64-lambda path per host core (the "
                                    "reference's path tracker restated, oracle/lf_oracle.cpp)")},
        "e2e": {"value": round(value, 4), "unit": unit, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "serve":
        run_serve(args)
    elif args.workload == "tv_path":
        run_tv_path(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
