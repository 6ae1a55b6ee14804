#!/usr/bin/env python
"""Benchmark of the tree-code force step on GB300.

Metric: particles/s per force step at <= 1e-4 median relative force error
(median over 4,096 seeded sample particles of |F - F_direct| / |F_direct|,
F_direct an FP64 direct sum on the GPU).

Default workload (the metric's configuration): the 2D N-body force step on
N = 4,194,304 particles in two exponential disks (scale lengths 0.1 and 0.05,
centres 0.6 apart, masses 1/N), Plummer-softened gravity eps = 1e-3, leaf size
64, FP32 expansions and P2P.  A step is one updateTree + solveNbody.  Three
methods are calibrated (untimed) and timed on the same positions:
  learned     the learned-order controller (trained first on independently
              seeded 1M-particle systems; depth and tolerance tau tuned);
  plain_best  the plain order-p FMM autotuned over depth, theta and order;
  plain_p12   the plain FMM at fixed order 12 (fastest depth/theta meeting
              the error target).
Every arm meets the error target on the 4,096 sampled particles; the value is
the faster of learned and plain_best, and "comparison" holds all three with
the learned method's speed-up over each plain one.

Arms:
  --impl ours       (default) the CUDA library on 1..N GPUs (replicas: each
                    rank advances its own independent system; weak scaling)
  --impl reference  the reference's CPU algorithm (the C oracle port of
                    NBodySolverFMM_SYM_MORTON, single-threaded per system as
                    in the reference) on all host cores, each core solving an
                    independent bounded sample of the same workload.
"""
from __future__ import annotations

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

METRIC = "particles/s per force step at 1e-4 rel err: learned-order vs plain FMM, 1 GB300"
UNIT = "particles/s"
TARGET_ERR = 1e-4
N_SAMPLES = 4096
THETAS = (0.4, 0.35, 0.3, 0.25, 0.2, 0.15, 0.1)
# learned-order controller training: systems x pairs sampled per level x Adam steps
CTRL_SYSTEMS = 24
CTRL_PER_LEVEL = 400000
CTRL_STEPS = 12000

WORKLOADS = {
    "nbody_two_disks_4m": dict(n=4194304, dist="two_disks", kernel="gravity", softening=1e-3, max_children=64),
    "nbody_two_disks_1m": dict(n=1048576, dist="two_disks", kernel="gravity", softening=1e-3, max_children=64),
    "tsne_70k": dict(n=70000, dist="tsne", dim=784, clusters=10, perplexity=30.0, kernel="tsne", order=8,
                     theta=0.5, max_children=16, early_exaggeration=12.0, method="tsne", softening=0.0),
    "leapfrog_two_disks_4m": dict(n=4194304, dist="two_disks", kernel="gravity", softening=1e-3, max_children=64,
                                  method="leapfrog", dt=1e-4),
    "tsne_batch_256": dict(n=0, systems=256, n_min=2000, n_max=200000, dim=64, clusters=(5, 20), perplexity=30.0,
                           kernel="tsne", max_children=16, theta=0.5, method="tsne_batch", softening=0.0, dist="tsne",
                           presteps=5),
    "bhmp_mixture_65k": dict(n=65536, dist="mixture", kernel="gravity", softening=1e-3, max_children=16,
                             method="bh", theta=0.5, multipole=True),
    "pm_embedding_70k": dict(n=70000, scale=25.0, n_interp=4, cell_size=1.0, min_intervals=4, method="pm",
                             dist="mixture", kernel="tsne", softening=0.0, max_children=16),
    "bh_mixture_65k": dict(n=65536, dist="mixture", kernel="gravity", softening=1e-3, max_children=16,
                           method="bh", theta=0.5),
}


def positions(w, seed):
    from masterthesislucas_gb300 import datasets
    if w["dist"] == "two_disks":
        p = datasets.two_disks(w["n"], seed=seed)
    else:
        p = datasets.gaussian_mixture(w["n"], seed=seed)
    return np.ascontiguousarray(p.astype(np.float64))


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


class ClockSampler:
    """SM clock, its maximum and the clock event (throttle) reasons, sampled in
    the timed region: every 2 ms by read-only NVML queries through the driver's
    libnvidia-ml (the timed regions last tens of milliseconds), else every 25 ms
    by nvidia-smi."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    # nvmlClocksEventReason* bits (nvml.h)
    BITS = ((0x8, "hw_slowdown"), (0x40, "hw_thermal_slowdown"), (0x20, "sw_thermal_slowdown"),
            (0x4, "sw_power_cap"))

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []
        self.samples = []  # (sm MHz, max MHz, reason bits) from NVML
        self.stop = None
        self.nvml = None

    def _nvml(self):
        import ctypes
        import torch
        uuid = "GPU-" + str(torch.cuda.get_device_properties(self.gpu).uuid)
        lib = ctypes.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            return None
        dev = ctypes.c_void_p()
        mx, sm, bits = ctypes.c_uint(0), ctypes.c_uint(0), ctypes.c_ulonglong(0)
        reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            lib.nvmlDeviceGetCurrentClocksThrottleReasons

        def read():
            if lib.nvmlDeviceGetClockInfo(dev, 1, ctypes.byref(sm)) == 0 and reasons(dev, ctypes.byref(bits)) == 0:
                return float(sm.value), float(mx.value), int(bits.value)
            return None
        if (lib.nvmlDeviceGetHandleByUUID(uuid.encode(), ctypes.byref(dev)) != 0 or
                lib.nvmlDeviceGetMaxClockInfo(dev, 1, ctypes.byref(mx)) != 0 or read() is None):  # NVML_CLOCK_SM
            lib.nvmlShutdown()
            return None
        self.nvml = lib
        return read

    def __enter__(self):
        read = None
        try:
            read = self._nvml()
        except Exception:
            read = None
        if read is not None:
            self.stop = threading.Event()
            first = read()
            if first is not None:
                self.samples.append(first)

            def poll():
                while not self.stop.is_set():
                    r = read()
                    if r is not None:
                        self.samples.append(r)
                    self.stop.wait(0.002)
            self.t = threading.Thread(target=poll, daemon=True)
            self.t.start()
            return self
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "25"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.stop is not None:
            self.stop.set()
            self.t.join(timeout=5)
            self.nvml.nvmlShutdown()
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        for c, m, bits in self.samples:
            sm.append(c)
            mx = m
            reasons.update(name for bit, name in self.BITS if bits & bit)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm), "source": "nvml" if self.samples else "nvidia-smi"}


def median_error(grad, ref):
    e = np.linalg.norm(grad - ref, axis=1) / np.linalg.norm(ref, axis=1)
    return float(np.median(e)), float(np.percentile(e, 90)), float(e.max())


def train_controller(w, seed=0, steps=CTRL_STEPS):
    """The learned-order controller: pair-error samples measured by the method
    on independently seeded 1M-particle systems of the workload's distribution,
    then the MLP trained by the library's own kernels (untimed)."""
    from masterthesislucas_gb300 import learned
    t0 = time.perf_counter()
    X, E = learned.generate(n_systems=CTRL_SYSTEMS, n_particles=1 << 20, kernel=w["kernel"],
                            per_level=CTRL_PER_LEVEL, seed=seed, leaf=w["max_children"])
    t1 = time.perf_counter()
    ctrl, stats = learned.fit(X, E, steps=steps, batch=8192, lr=2e-3, seed=seed)
    stats.update({"samples": int(len(X)), "systems": CTRL_SYSTEMS, "system_n": 1 << 20,
                  "generate_s": round(t1 - t0, 2), "train_s": round(time.perf_counter() - t1, 2),
                  "steps": steps, "orders": list(learned.ORDERS)})
    return ctrl, stats


def run_ours(args, w, rank, world):
    import torch

    from masterthesislucas_gb300 import NBodySolverFMM_SYM_MORTON
    from masterthesislucas_gb300._lib import check, lib, ptr
    from masterthesislucas_gb300.autotune import refine_leaf_p2p, tune, tune_learned

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(device=dev)
    n = w["n"]
    pos_h = positions(w, seed=1000 + rank)
    pos_d = torch.from_numpy(pos_h).to(dev)
    grad_d = torch.zeros((n, 2), dtype=torch.float64, device=dev)
    tot_d = torch.zeros(1, dtype=torch.float64, device=dev)
    # two disjoint seeded samples of sink particles: configurations are chosen on the tuning rows and every
    # reported error is measured on the evaluation rows
    rows, rows_eval = sample_rows(n)
    rows_d = torch.from_numpy(rows).to(dev)
    rows_eval_d = torch.from_numpy(rows_eval).to(dev)
    ref_d = torch.zeros((N_SAMPLES, 2), dtype=torch.float64, device=dev)
    ref_eval_d = torch.zeros((N_SAMPLES, 2), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    # FP64 direct-sum oracle on the sampled sinks (untimed)
    for rd, out in ((rows_d, ref_d), (rows_eval_d, ref_eval_d)):
        check(lib().tc_direct_device(1 if w["kernel"] == "gravity" else 0, w["softening"], 1, ptr(pos_d), n,
                                     ptr(rd), N_SAMPLES, ptr(out), None, None))
    torch.cuda.synchronize()
    ref = ref_d.cpu().numpy()
    ref_eval = ref_eval_d.cpu().numpy()

    def make(theta, order=0, depth=None, controller=None, tau=None, mac="cell", centre="com", m2l="simt",
             leaf_p2p=None):
        kind, _, slack = mac.partition(":")
        lp = args.leaf_p2p if leaf_p2p is None else leaf_p2p
        s = NBodySolverFMM_SYM_MORTON(w["kernel"], max_children=w["max_children"], tree_depth=depth, theta=theta,
                                      softening=w["softening"], precision="fp32", order=order,
                                      device=dev.index, stream=stream.cuda_stream, mac=kind,
                                      slack=float(slack or 1.0), leaf_p2p=lp if order else 0,
                                      centre=centre, m2l=m2l, near_overlap=not args.no_near_overlap)
        if controller is not None:
            s.set_controller(controller, tau)
        return s

    def step(s):
        s.update_tree_device(pos_d)
        s.solve_device(grad_d, tot_d, accumulate=False, scatter=True)

    # reference-order method: largest theta meeting the error target, timed briefly
    ref_order = None
    if not args.skip_reference_order:
        for th in (0.2, 0.15, 0.1):
            s0 = make(th)
            step(s0)
            torch.cuda.synchronize()
            med = median_error(grad_d[rows_d].cpu().numpy(), ref)[0]
            if med <= TARGET_ERR:
                med = median_error(grad_d[rows_eval_d].cpu().numpy(), ref_eval)[0]
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                for _ in range(2):
                    step(s0)
                e1.record(stream)
                torch.cuda.synchronize()
                ms0 = e0.elapsed_time(e1) / 2
                ref_order = {"theta": th, "median_err": med, "ms_per_step": ms0, "particles_per_s": n / ms0 * 1e3,
                             "depth": s0.depth()}
                s0.close()
                break
            s0.close()

    # plain order-p FMM, autotuned over (depth, theta, order); its order-12 line is the fixed-p=12 baseline
    target = TARGET_ERR * 0.9
    tensor_best = None
    if args.order:
        plain = {"depth": args.depth or None, "theta": args.theta or 0.5, "order": args.order,
                 "mac": "cell" if args.mac == "all" else args.mac, "centre": args.centre, "m2l": args.m2l}
        trials = []
    else:
        # expansion engines: about each node's centre of mass with the FP32 SIMT M2L (three opening criteria),
        # and about each cell centre with the tensor-core M2L (bounding-radius criterion)
        engines = []
        if args.engines in ("all", "com"):
            engines.append(("com", "simt", ("cell", "bmax", "bmax_adaptive:0.03") if args.mac == "all"
                            else (args.mac,)))
        if args.engines in ("all", "box"):
            engines.append(("box", "tensor", ("bmax",)))
        plain, trials = None, []
        for centre, m2l, macs in engines:
            best, tr = tune(pos_d, ref, rows_d, kernel=w["kernel"], softening=w["softening"],
                            leaf=w["max_children"], target=target, stream=stream, device=dev.index, macs=macs,
                            leaf_p2p=args.leaf_p2p, centre=centre, m2l=m2l)
            trials += tr
            if m2l == "tensor":
                tensor_best = best
            if best is not None and (plain is None or best["ms"] < plain["ms"]):
                plain = best
        if plain is None:
            raise SystemExit("autotuner found no configuration meeting the error target")
        # the leaf-pair threshold, refined at the chosen configuration
        plain, tr = refine_leaf_p2p(plain, pos_d, ref, rows_d, kernel=w["kernel"], softening=w["softening"],
                                    leaf=w["max_children"], target=target, stream=stream, device=dev.index)
        trials += tr
    p12 = min((t for t in trials if t["order"] == 12 and t["err"] <= target), key=lambda t: t["ms"], default=None)

    # learned-order controller
    learned_cfg, ltrials, ctrl_stats, ctrl = None, [], None, None
    if not args.no_learned:
        ctrl, ctrl_stats = train_controller(w, seed=rank, steps=args.ctrl_steps)
    if ctrl is not None and args.tau:
        from masterthesislucas_gb300.solver import get_depth
        learned_cfg = {"depth": args.learned_depth or get_depth(w["max_children"], n) + 1, "tau": args.tau}
    elif ctrl is not None:
        learned_cfg, ltrials = tune_learned(pos_d, ref, rows_d, ctrl, kernel=w["kernel"], softening=w["softening"],
                                            leaf=w["max_children"], target=target, stream=stream, device=dev.index)
    calib = {"plain_best": plain, "plain_p12": p12, "plain_tensor": tensor_best, "learned_best": learned_cfg, "plain_trials": trials,
             "learned_trials": ltrials, "controller": ctrl_stats, "reference_order": ref_order}

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # 256 MB > L2 (129 MB)

    def timed(s, steps, sample_clocks, judge=None):
        for _ in range(args.warmup):
            step(s)
            if judge is not None:  # the check's first call sets up its kernels: keep it out of the timing
                judge.check_async(pos_d, grad_d, torch.zeros(1, dtype=torch.float64, device=dev), stream)
        torch.cuda.synchronize()
        stages_sync = s.stage_times()
        graph = not args.no_graph
        if graph:
            # the whole step as one CUDA graph over the exact box of these positions
            s.capture_step(pos_d, grad_d, tot_d)
            for _ in range(args.warmup):
                s.launch_step()
            torch.cuda.synchronize()
            if s.async_status():
                graph = False
        if world > 1:
            torch.distributed.barrier()
        ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        judge_err = torch.zeros(steps, dtype=torch.float64, device=dev)
        stage_sum, launches = None, 0
        with ClockSampler(dev.index) as clk:
            for k in range(steps):
                with torch.cuda.stream(stream):
                    flush.fill_(float(k))
                ev0[k].record(stream)
                if graph:
                    s.launch_step()
                    launches += s.launches()
                else:
                    s.update_tree_device(pos_d)
                    launches += s.launches()
                    s.solve_device(grad_d, tot_d, accumulate=False, scatter=True)
                    launches += s.launches()
                if judge is not None:
                    # sampled-error check of this step on the same stream, read after the loop
                    judge.check_async(pos_d, grad_d, judge_err[k:k + 1], stream)
                ev1[k].record(stream)
                st = stages_sync if graph else s.stage_times()
                stage_sum = st if stage_sum is None else {a: stage_sum[a] + st[a] for a in st}
            torch.cuda.synchronize()
        if graph and s.async_status():
            raise SystemExit("a captured step was flagged invalid (box or list capacity)")
        ms = [ev0[k].elapsed_time(ev1[k]) for k in range(steps)]
        judged = None
        if judge is not None:
            # the plain FMM is the fallback: a step whose sampled error missed the target is redone by it, and
            # the redo's device time is added to that step
            errs = judge_err.cpu().numpy()
            failed = [k for k in range(steps) if not errs[k] <= judge.tol]
            for k in failed:
                f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                f0.record(stream)
                judge.plain.update_tree_device(pos_d)
                judge.plain.solve_device(grad_d, tot_d, accumulate=False, scatter=True)
                f1.record(stream)
                torch.cuda.synchronize()
                ms[k] += f0.elapsed_time(f1)
            judge.steps += steps
            judge.recomputed += len(failed)
            judged = {"checked_steps": steps, "fallback_steps": len(failed), "sampled_err_max": float(np.nanmax(errs)),
                      "check_rows": int(len(judge.rows))}
        t_total = sum(ms) / 1e3
        if world > 1:
            t = torch.tensor([t_total], device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            t_total = float(t.item())
        err = median_error(grad_d[rows_eval_d].cpu().numpy(), ref_eval)
        nodes = s.getNodesBufferData(-1).shape[0]
        nn_pairs, near_pairs = s.list_stats()
        return dict(ms=ms, t_total=t_total, judge=judged, stages={a: v / steps for a, v in stage_sum.items()},
                    graph=graph,
                    counters=s.counters(), err=err, clocks=clk.summary() if sample_clocks else None,
                    launches=launches, depth=s.depth(), nonempty_nodes=int(nodes),
                    near_pairs=int(np.asarray(near_pairs, np.int64).sum()))

    # the arms: the learned-order method (headline, when it meets the target) and the plain ones beside it
    arms = {}
    s_plain = make(plain["theta"], order=plain["order"], depth=plain["depth"], mac=plain["mac"],
                   centre=plain["centre"], m2l=plain["m2l"], leaf_p2p=plain.get("leaf_p2p"))
    arms["plain_best"] = timed(s_plain, args.steps, sample_clocks=True)
    arms["plain_best"].update(theta=plain["theta"], order=plain["order"], mac=plain["mac"], centre=plain["centre"],
                              m2l=plain["m2l"], leaf_p2p=plain.get("leaf_p2p", args.leaf_p2p))
    if p12 is not None:
        key = ("depth", "theta", "mac", "centre", "m2l", "leaf_p2p")
        if plain["order"] == 12 and all(p12.get(k) == plain.get(k) for k in key):
            arms["plain_p12"] = arms["plain_best"]
        else:
            s12 = make(p12["theta"], order=12, depth=p12["depth"], mac=p12["mac"], centre=p12["centre"],
                       m2l=p12["m2l"], leaf_p2p=p12.get("leaf_p2p"))
            arms["plain_p12"] = timed(s12, args.steps, sample_clocks=False)
            arms["plain_p12"].update(theta=p12["theta"], order=12, mac=p12["mac"], centre=p12["centre"],
                                     m2l=p12["m2l"])
            s12.close()
    # the tensor-core M2L engine's fastest configuration meeting the target, beside the headline
    if tensor_best is not None and plain.get("m2l") != "tensor":
        st = make(tensor_best["theta"], order=tensor_best["order"], depth=tensor_best["depth"],
                  mac=tensor_best["mac"], centre="box", m2l="tensor")
        arms["plain_tensor"] = timed(st, args.steps, sample_clocks=False)
        arms["plain_tensor"].update(theta=tensor_best["theta"], order=tensor_best["order"], mac=tensor_best["mac"],
                                    centre="box", m2l="tensor")
        st.close()
    s_head, head, s_l = s_plain, "plain_best", None
    if learned_cfg is not None:
        s_l = make(1.0, order=12, depth=learned_cfg["depth"], controller=ctrl, tau=learned_cfg["tau"])
        # the plain FMM is the fallback and the judge: each timed learned step is checked on 64 sampled
        # particles against an FP32 direct sum (about 0.55 ms at 4M; 32 samples proved too noisy a median) and
        # redone by the plain FMM when it misses the target
        from masterthesislucas_gb300.learned import CheckedSolve
        s_fb = make(plain["theta"], order=plain["order"], depth=plain["depth"], mac=plain["mac"],
                    centre=plain["centre"], m2l=plain["m2l"], leaf_p2p=plain.get("leaf_p2p"))
        judge = CheckedSolve(s_l, s_fb, n, kernel=w["kernel"], softening=w["softening"], tol=TARGET_ERR,
                             n_check=64, seed=11, device=dev.index)
        arms["learned"] = timed(s_l, args.steps, sample_clocks=True, judge=judge)
        arms["learned"].update(tau=learned_cfg["tau"], order=12)
        s_fb.close()
        # the headline is the faster of the two methods (both meet the error target)
        if arms["learned"]["t_total"] < arms["plain_best"]["t_total"]:
            s_head, head = s_l, "learned"

    # end to end through the C ABI with pinned host buffers, on the headline arm
    from masterthesislucas_gb300._lib import check as chk
    import ctypes
    pos_pin = torch.empty((n, 2), dtype=torch.float64, pin_memory=True)
    grad_pin = torch.zeros((n, 2), dtype=torch.float64, pin_memory=True)
    ids_pin = torch.empty(n, dtype=torch.int32, pin_memory=True)
    pos_np, grad_np, ids_np = pos_pin.numpy(), grad_pin.numpy(), ids_pin.numpy()
    mn, mx = pos_h.min(0), pos_h.max(0)
    e2e_ms = []
    for k in range(max(2, args.steps // 2) + 2):
        np.copyto(pos_np, pos_h)
        ids_np[:] = np.arange(n, dtype=np.int32)
        grad_np[:] = 0.0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        chk(lib().tc_update_tree(s_head._h, ptr(pos_np), ptr(ids_np), n, ptr(mn), ptr(mx)))
        tot = ctypes.c_double(0.0)
        chk(lib().tc_solve(s_head._h, ctypes.byref(tot), None, ptr(grad_np), n))
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_ms = e2e_ms[2:]
    s_plain.close()
    if s_l is not None:
        s_l.close()
    return dict(head=head, arms=arms, calib=calib, e2e_ms=e2e_ms)


def cpu_baseline(w, theta, n_sample, threads=1, seeds=None):
    """The reference's algorithm (C oracle port), single-threaded per system."""
    import ctypes
    import oracle
    from masterthesislucas_gb300 import datasets

    seeds = seeds or list(range(threads))
    L = oracle.lib()
    jobs = []
    for sd in seeds:
        if w["dist"] == "two_disks":
            p = datasets.two_disks(n_sample, seed=5000 + sd)
        else:
            p = datasets.gaussian_mixture(n_sample, seed=5000 + sd)
        p = np.ascontiguousarray(p.astype(np.float64))
        jobs.append(p)
    depth = oracle.get_depth(w["max_children"], n_sample)
    kern = 1 if w["kernel"] == "gravity" else 0

    def solve(p):
        n = len(p)
        mn, mx = p.min(0), p.max(0)
        codes = np.empty(n, np.uint32)
        ids = np.empty(n, np.int32)
        ps = np.empty((n, 2))
        g = np.zeros((n, 2))
        tot = np.zeros(1)
        L.orc_sym_fmm(kern, w["softening"], w["max_children"], depth, theta, n, oracle._p(p), oracle._p(mn),
                      oracle._p(mx), oracle._p(codes), oracle._p(ids), oracle._p(ps), oracle._p(g), oracle._p(tot),
                      None)

    t0 = time.perf_counter()
    ths = [threading.Thread(target=solve, args=(p,)) for p in jobs]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    dt = time.perf_counter() - t0
    return len(jobs) * n_sample / dt, dt, depth


def run_leapfrog(args, w):
    """N-body time stepping: kick-drift-kick leapfrog (dt = 1e-4) over the
    FMM force on the two rotating disks; the FMM configuration is autotuned on
    the initial positions (untimed).  Reports particles/s per force step,
    steps/s and the FP64 energy drift and momentum over the timed steps."""
    import torch

    from masterthesislucas_gb300._lib import check, lib, ptr
    from masterthesislucas_gb300.autotune import tune
    from masterthesislucas_gb300.nbody import LeapfrogNBody, circular_velocities

    dev = torch.device("cuda", 0)
    n = w["n"]
    m = 1.0 / n
    pos_h = positions(w, seed=1000)
    vel_h = circular_velocities(pos_h, m, w["softening"], centres=[[-0.3, 0.0], [0.3, 0.0]])
    pos_d = torch.from_numpy(pos_h).to(dev)
    rows = np.sort(np.random.default_rng(7).choice(n, N_SAMPLES, replace=False)).astype(np.int64)
    rows_d = torch.from_numpy(rows).to(dev)
    ref_d = torch.zeros((N_SAMPLES, 2), dtype=torch.float64, device=dev)
    check(lib().tc_direct_device(1, w["softening"], 1, ptr(pos_d), n, ptr(rows_d), N_SAMPLES, ptr(ref_d), None, None))
    torch.cuda.synchronize()
    best, _ = tune(pos_d, ref_d.cpu().numpy(), rows_d, kernel="gravity", softening=w["softening"],
                   leaf=w["max_children"], target=TARGET_ERR * 0.9, device=0)
    sim = LeapfrogNBody(pos_h, vel_h, mass=m, dt=w["dt"], softening=w["softening"], max_children=w["max_children"],
                        tree_depth=best["depth"], theta=best["theta"], order=best["order"])
    sim.step(args.warmup)
    d0 = sim.diagnostics()
    torch.cuda.synchronize()
    launches = 0
    with ClockSampler(0) as clk:
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        t0.record()
        for _ in range(args.steps):
            sim.step(1)
            launches += sim.solver.launches()
        torch.cuda.synchronize()
        t1.record()
        torch.cuda.synchronize()
    ms = t0.elapsed_time(t1)
    d1 = sim.diagnostics()
    # force error at the final positions
    x_d = sim.x
    check(lib().tc_direct_device(1, w["softening"], 1, ptr(x_d), n, ptr(rows_d), N_SAMPLES, ptr(ref_d), None, None))
    torch.cuda.synchronize()
    ref_end = ref_d.cpu().numpy() * m
    acc_end = sim.a[rows_d].cpu().numpy()
    err = median_error(acc_end, ref_end)
    sim.close()
    value = n * args.steps / (ms / 1e3)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded two rotating exponential disks, circular velocities from the enclosed mass)",
            "config": {"workload": args.workload, "n": n, "dt": w["dt"], "integrator": "kick-drift-kick leapfrog",
                       "depth": best["depth"], "theta": best["theta"], "order": best["order"],
                       "l2": "inputs exceed L2 (4M particles: 64 MB positions + tree)"},
            "steps_per_s": 1e3 * args.steps / ms,
            "diagnostics": {"energy_start": d0["energy"], "energy_end": d1["energy"],
                            "energy_drift_rel": abs(d1["energy"] - d0["energy"]) / abs(d0["energy"]),
                            "momentum_start": [d0["px"], d0["py"]], "momentum_end": [d1["px"], d1["py"]],
                            "kinetic_end": d1["kinetic"],
                            "potential_end": d1["potential"], "sum": "fp64, fixed order"},
            "error": {"median": err[0], "p90": err[1], "max": err[2], "vs": "fp64 direct sum at the final positions",
                      "samples": N_SAMPLES},
            "gpu_launches": launches, "clocks": clk.summary()}
    print(json.dumps(line))


def batch_order(n):
    """Expansion order per system size for the batched t-SNE, from {4, 8, 12}:
    a fixed size rule (p = 4 below 20k particles, p = 8 above)."""
    return 4 if n < 20000 else 8


def run_tsne_batch(args, w):
    """Batched uneven t-SNE: independent embeddings (N log-uniform in
    [2k, 200k], 64-dim Gaussian-cluster data, perplexity 30, k = 90 CSR P)
    advance one gradient step per CUDA graph launch.  Setup (untimed): P per
    system, a few uncaptured steps so that the embeddings leave their initial
    blob, then each system's tree depth autotuned on its embedding."""
    import torch

    from masterthesislucas_gb300 import affinity, datasets
    from masterthesislucas_gb300.tsne import TSNE, TSNEBatch, tune_depth

    from masterthesislucas_gb300 import shard

    rank, world = int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    rng = np.random.default_rng(2024)
    ns_all = np.exp(rng.uniform(np.log(w["n_min"]), np.log(w["n_max"]), w["systems"])).astype(np.int64)
    ks_all = rng.integers(w["clusters"][0], w["clusters"][1] + 1, len(ns_all))
    # the systems are independent: each rank owns whole systems, no exchange
    mine = shard.shard(ns_all, rank, world)
    ns = ns_all[mine]
    t0 = time.perf_counter()
    systems = []
    for i, n in zip(mine, ns):
        k = int(ks_all[i])
        x, _ = datasets.cluster_data(int(n), w["dim"], k=k, seed=10_000 + i)
        rp, col, val = affinity.build_p_csr(x, perplexity=w["perplexity"], device="cuda")
        y0 = np.random.default_rng(20_000 + i).normal(0.0, 1e-2, (int(n), 2))  # N(0, 1e-4)
        systems.append(TSNE(rp, col, val, y0, early_exaggeration=12.0, max_children=w["max_children"],
                            order=batch_order(int(n))))
    t_p = time.perf_counter() - t0
    for s in systems:
        for _ in range(w["presteps"]):
            s.time_step()
    depths = [tune_depth(s, theta=w["theta"])["depth"] for s in systems]
    t_setup = time.perf_counter() - t0
    batch = TSNEBatch(systems, margin=0.5)
    for _ in range(args.warmup):
        batch.time_step()
    st0 = batch.stats()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    with ClockSampler(local) as clk:
        t1 = time.perf_counter()
        for _ in range(args.steps):
            batch.time_step()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t1
    st1 = batch.stats()
    dev = torch.device("cuda", local)
    dt = shard.max_over_ranks(dt, device=dev)
    total = shard.sum_over_ranks(int(ns.sum()), device=dev)
    value = total * args.steps / dt
    from masterthesislucas_gb300.solver import get_depth
    line = {"metric": "t-SNE gradient steps of a batch of embeddings (particles/s over all systems)",
            "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (64-dim Gaussian clusters per system, P built by the project's kNN/perplexity code)",
            "config": {"workload": args.workload, "systems": int(w["systems"]), "particles": total,
                       "n_min": int(ns_all.min()), "n_max": int(ns_all.max()),
                       "parallelism": f"systems split over {world} rank(s) by particle count, no exchange", "perplexity": w["perplexity"], "k": 90,
                       "leaf_size": w["max_children"], "theta": w["theta"],
                       "orders": {"4": int((ns < 20000).sum()), "8": int((ns >= 20000).sum())},
                       "depth_offsets": np.bincount([d - get_depth(w["max_children"], int(n))
                                                     for d, n in zip(depths, ns)]).tolist(),
                       "iterations_before_timing": w["presteps"] + args.warmup,
                       "timing": "host clock around K batch steps (each one graph launch plus the flag check)",
                       "l2": "inputs exceed L2 (the batch holds %d particles)" % total},
            "steps_per_s": args.steps / dt,
            "graph": {"launches_timed": st1["graph_launches"] - st0["graph_launches"],
                      "captures_timed": st1["captures"] - st0["captures"],
                      "restepped_timed": st1["restepped"] - st0["restepped"],
                      "graph_ms_timed": st1["graph_ms"] - st0["graph_ms"],
                      "restep_ms_timed": st1["restep_ms"] - st0["restep_ms"],
                      "nodes": st1["graph_nodes"], "latency_ms": 1e3 * dt / args.steps},
            "setup_s": {"affinities": round(t_p, 1), "total": round(t_setup, 1)},
            "gpu_launches": st1["kernels_per_launch"] * args.steps,
            "clocks": clk.summary()}
    batch.close()
    for s in systems:
        s.close()
    if rank == 0:
        print(json.dumps(line))


def run_bh(args, w):
    """Barnes-Hut force step (the reference's QuadTree and MAC) on the GPU."""
    import ctypes
    import torch

    from masterthesislucas_gb300._lib import check, lib, ptr

    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    n = w["n"]
    pos_h = positions(w, seed=1000)
    pos_d = torch.from_numpy(pos_h).to(dev)
    grad_d = torch.zeros((n, 2), dtype=torch.float64, device=dev)
    tot_d = torch.zeros(1, dtype=torch.float64, device=dev)
    rows = np.sort(np.random.default_rng(7).choice(n, N_SAMPLES, replace=False)).astype(np.int64)
    rows_d = torch.from_numpy(rows).to(dev)
    ref_d = torch.zeros((N_SAMPLES, 2), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    check(lib().tc_direct_device(1, w["softening"], 1, ptr(pos_d), n, ptr(rows_d), N_SAMPLES, ptr(ref_d), None, None))
    torch.cuda.synchronize()
    ref = ref_d.cpu().numpy()
    cs = ctypes.c_void_p(stream.cuda_stream)

    mp = bool(w.get("multipole"))
    solve_dev = lib().tc_bhmp_solve_device if mp else lib().tc_bh_solve_device
    solve_host = lib().tc_bhmp_solve if mp else lib().tc_bh_solve

    def step():
        check(solve_dev(1, w["softening"], w["max_children"], w["theta"], 0, ptr(pos_d), n, ptr(grad_d), ptr(tot_d),
                        cs))

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    with ClockSampler(0) as clk:
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(float(k))
            ev0[k].record(stream)
            step()
            ev1[k].record(stream)
        torch.cuda.synchronize()
    ms = [ev0[k].elapsed_time(ev1[k]) for k in range(args.steps)]
    err = median_error(grad_d[rows_d].cpu().numpy(), ref)
    # e2e through the host entry point
    import time as _t
    g_h = np.zeros((n, 2))
    tot = ctypes.c_double(0.0)
    e2e = []
    for k in range(3):
        t0 = _t.perf_counter()
        check(solve_host(1, w["softening"], w["max_children"], w["theta"], 0, ptr(pos_h), n, ptr(g_h),
                         ctypes.byref(tot)))
        e2e.append(_t.perf_counter() - t0)
    import oracle
    t0 = _t.perf_counter()
    (oracle.bhmp if mp else oracle.bh)(pos_h, kernel=oracle.KERNEL_GRAVITY, eps=w["softening"],
                                       max_children=w["max_children"], theta=w["theta"])
    cpu_t = _t.perf_counter() - t0
    t_total = sum(ms) / 1e3
    name = "Barnes-Hut with quadrupoles (NBodySolverBHMP)" if mp else "Barnes-Hut (C1, single evaluation)"
    line = {"metric": f"particles/s per {name} force step", "value": n * args.steps / t_total,
            "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * t_total / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded 8-cluster Gaussian mixture)",
            "config": {"workload": args.workload, "n": n, "theta": w["theta"], "leaf_size": w["max_children"],
                       "softening": w["softening"],
                       "method": ("Barnes-Hut + quadrupoles, the reference's QuadTreeMultiPole and MAC" if mp
                                  else "Barnes-Hut, the reference's QuadTree and MAC"),
                       "l2": "256 MB buffer written between timed steps"},
            "error": {"median": err[0], "p90": err[1], "max": err[2], "vs": "fp64 direct sum", "samples": N_SAMPLES},
            "e2e": {"value": n / float(np.median(e2e)), "unit": UNIT, "h2d_bytes_per_step": n * 16,
                    "d2h_bytes_per_step": n * 16 + 8},
            "clocks": clk.summary(),
            "cpu_baseline": {"value": n / cpu_t, "unit": UNIT, "cores": 1, "kind": "port",
                             "sample": f"the full {n}-particle system, reference {'BHMP' if mp else 'BH'} (C port), "
                                       f"{cpu_t:.2f} s"}}
    print(json.dumps(line))


def run_pm(args, w):
    """Particle-mesh (FFT-accelerated interpolation) t-SNE repulsion, NBodySolverPM, on the GPU: the
    reference's settings (4 Lagrange nodes per box, unit boxes, at least 4 boxes per dimension)."""
    import ctypes
    import time as _t
    import torch

    from masterthesislucas_gb300._lib import check, lib, ptr

    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    n = w["n"]
    from masterthesislucas_gb300 import datasets
    pos_h = np.ascontiguousarray(datasets.gaussian_mixture(n, seed=1000).astype(np.float64) * w["scale"])
    pos_d = torch.from_numpy(pos_h).to(dev)
    grad_d = torch.zeros((n, 2), dtype=torch.float64, device=dev)
    tot_d = torch.zeros(1, dtype=torch.float64, device=dev)
    rows = np.sort(np.random.default_rng(7).choice(n, N_SAMPLES, replace=False)).astype(np.int64)
    rows_d = torch.from_numpy(rows).to(dev)
    ref_d = torch.zeros((N_SAMPLES, 2), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    check(lib().tc_direct_device(0, 0.0, 1, ptr(pos_d), n, ptr(rows_d), N_SAMPLES, ptr(ref_d), None, None))
    torch.cuda.synchronize()
    ref = ref_d.cpu().numpy()
    cs = ctypes.c_void_p(stream.cuda_stream)
    prm = (w["n_interp"], w["cell_size"], w["min_intervals"])

    def step():
        check(lib().tc_pm_solve_device(*prm, ptr(pos_d), n, ptr(grad_d), ptr(tot_d), cs))

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    with ClockSampler(0) as clk:
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(float(k))
            ev0[k].record(stream)
            step()
            ev1[k].record(stream)
        torch.cuda.synchronize()
    ms = [ev0[k].elapsed_time(ev1[k]) for k in range(args.steps)]
    err = median_error(grad_d[rows_d].cpu().numpy(), ref)
    g_h = np.zeros((n, 2))
    tot = ctypes.c_double(0.0)
    e2e = []
    for k in range(3):
        t0 = _t.perf_counter()
        check(lib().tc_pm_solve(*prm, ptr(pos_h), n, ptr(g_h), ctypes.byref(tot)))
        e2e.append(_t.perf_counter() - t0)
    import oracle
    t0 = _t.perf_counter()
    oracle.pm_numpy(pos_h, n_interp=prm[0], cell_size=prm[1], min_intervals=prm[2])
    cpu_t = _t.perf_counter() - t0
    t_total = sum(ms) / 1e3
    line = {"metric": "particles/s per particle-mesh (NBodySolverPM) repulsion evaluation", "value": n * args.steps / t_total,
            "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * t_total / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded 8-cluster Gaussian mixture scaled to a t-SNE embedding's extent)",
            "config": {"workload": args.workload, "n": n, "n_interp": prm[0], "cell_size": prm[1],
                       "min_intervals": prm[2], "extent_scale": w["scale"],
                       "method": "FFT-accelerated interpolation (FIt-SNE), the reference's grid, cuFFT convolution",
                       "l2": "256 MB buffer written between timed steps"},
            "error": {"median": err[0], "p90": err[1], "max": err[2], "vs": "fp64 direct sum", "samples": N_SAMPLES},
            "e2e": {"value": n / float(np.median(e2e)), "unit": UNIT, "h2d_bytes_per_step": n * 16,
                    "d2h_bytes_per_step": n * 16 + 8},
            "clocks": clk.summary(),
            "cpu_baseline": {"value": n / cpu_t, "unit": UNIT, "cores": 1, "kind": "port",
                             "sample": f"the full {n}-point system, numpy restatement (pocketfft), {cpu_t:.2f} s"}}
    print(json.dumps(line))


def run_tsne(args, w):
    """t-SNE gradient steps (tree repulsion at order p + CSR attractive + Z + momentum), device resident."""
    import torch

    from masterthesislucas_gb300 import datasets
    from masterthesislucas_gb300._lib import check, lib, ptr
    from masterthesislucas_gb300.affinity import build_p_csr
    from masterthesislucas_gb300.tsne import TSNE

    n = w["n"]
    x, _ = datasets.cluster_data(n, w["dim"], k=w["clusters"], seed=3)
    t0 = time.perf_counter()
    row_ptr, col, val = build_p_csr(x, perplexity=w["perplexity"], device="cuda")
    t_p = time.perf_counter() - t0
    y0 = datasets.tsne_init(n, seed=4, sigma=0.01)
    t = TSNE(row_ptr, col, val, y0, early_exaggeration=w["early_exaggeration"], min_theta=w["theta"],
             max_theta=w["theta"], max_children=w["max_children"], order=args.order or w["order"])
    dev = torch.device("cuda", 0)

    def exact_grad(y, rows):
        """FP64 gradient on sampled rows: 4/Z * direct repulsion + attractive term."""
        yd = torch.from_numpy(np.ascontiguousarray(y)).to(dev)
        rd = torch.from_numpy(rows.astype(np.int64)).to(dev)
        rep = torch.zeros((len(rows), 2), dtype=torch.float64, device=dev)
        z = torch.zeros(1, dtype=torch.float64, device=dev)
        check(lib().tc_direct_device(0, 0.0, 1, ptr(yd), n, ptr(rd), len(rows), ptr(rep), None, None))
        check(lib().tc_direct_device(0, 0.0, 1, ptr(yd), n, None, n, ptr(torch.zeros((n, 2), dtype=torch.float64,
                                                                                   device=dev)), ptr(z), None))
        torch.cuda.synchronize()
        zz = float(z.item())
        g = rep.cpu().numpy() * (4.0 / zz)
        it = t.iteration_counter - 1
        exag = 4.0 * (w["early_exaggeration"] if it < 250 else 1.0)
        for k, i in enumerate(rows):
            js = col[row_ptr[i]:row_ptr[i + 1]]
            d = y[js] - y[i]
            q = 1.0 / (1.0 + (d * d).sum(1))
            g[k] += exag * ((val[row_ptr[i]:row_ptr[i + 1]] * q)[:, None] * d).sum(0)
        return g, zz

    rows = np.sort(np.random.default_rng(9).choice(n, 1024, replace=False))
    errs = []
    steps = args.steps
    for _ in range(args.warmup):
        t.time_step()
    # the warm-up iterations count as t-SNE iterations; the timed ones continue the schedule
    torch.cuda.synchronize()
    st = torch.cuda.Event(enable_timing=True)
    en = torch.cuda.Event(enable_timing=True)
    launches = 0
    ms_total = 0.0
    check_every = max(1, steps // 5)
    with ClockSampler(0) as clk:
        for k in range(steps):
            st.record()
            t.time_step()
            en.record()
            launches += t.launches()
            torch.cuda.synchronize()
            ms_total += st.elapsed_time(en)
            if (k + 1) % check_every == 0:
                y, yp, g = t.embedding()
                ge, zz = exact_grad(yp, rows)   # g was evaluated at the previous embedding
                e = np.linalg.norm(g[rows] - ge, axis=1) / np.linalg.norm(ge, axis=1)
                errs.append({"iteration": t.iteration_counter, "median": float(np.median(e)),
                             "p90": float(np.percentile(e, 90))})
    # final KL(P || Q) with an exact FP64 Z
    y, _, _ = t.embedding()
    yd = torch.from_numpy(y).to(dev)
    z = torch.zeros(1, dtype=torch.float64, device=dev)
    check(lib().tc_direct_device(0, 0.0, 1, ptr(yd), n, None, n,
                                 ptr(torch.zeros((n, 2), dtype=torch.float64, device=dev)), ptr(z), None))
    torch.cuda.synchronize()
    rr = np.repeat(np.arange(n), np.diff(row_ptr).astype(np.int64))
    d2 = ((y[rr] - y[col]) ** 2).sum(1)
    qv = 1.0 / (1.0 + d2) / float(z.item())
    kl = float(np.sum(val * np.log(val / qv)))
    s_per_step = ms_total / 1e3 / steps
    line = {"metric": "t-SNE gradient steps/s (C2: 70k x 784, perplexity 30, order-p FMM repulsion)",
            "value": 1.0 / s_per_step, "unit": "steps/s", "n_gpus": 1, "steps": steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * s_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (10 Gaussian clusters in 784-D clipped to [0,1]; P built here)",
            "config": {"workload": args.workload, "n": n, "perplexity": w["perplexity"], "k": 90,
                       "nnz": int(len(col)), "order": args.order or w["order"], "theta": w["theta"],
                       "early_exaggeration": w["early_exaggeration"], "p_build_s": t_p},
            "particles_per_s": n / s_per_step, "gradient_error_vs_fp64": errs, "final_kl": kl,
            "gpu_launches": launches, "clocks": clk.summary()}
    print(json.dumps(line))


def sample_rows(n, count=N_SAMPLES):
    """Two disjoint seeded samples of `count` sink indices: the tuning rows and the evaluation rows."""
    both = np.random.default_rng(7).choice(n, 2 * count, replace=False).astype(np.int64)
    return np.sort(both[:count]), np.sort(both[count:])


def m2l_flops(order):
    """Flops of one order-p M2L pair as the kernel does it: the kernel derivatives to order 2p by their
    recurrence (about 10 flops each) and the contraction of the multipole with them."""
    K = lambda q: (q + 1) * (q + 2) // 2  # noqa: E731
    return 10 * K(order) + 2 * sum((k + 1) * K(order - k) for k in range(order + 1))


def step_roofline(n, arm, hbm_gbs, fp32_tflops, ms_per_step):
    """Per-stage roofline of one force step: T_roof = sum over stages of max(bytes / HBM peak,
    flops / FP32 peak), from the stage's algorithmic bytes and flops.  Units: sort 100 B per particle (read
    positions, write codes, four 32-bit key/value passes, gather); build 12 B per particle plus the FP32 node
    records and multipoles written; lists 4 B per entry; far field the M2L flops per pair plus the L2L
    coefficient traffic; near field 20 flops per particle pair (16 B per particle: the sink read, its force
    written); L2P 40 B per particle (position, code, near-field force, permutation, FP64 force written) plus
    the leaf expansions, 5 flops per particle and coefficient; the pair-sum reduction 8 B per particle.
    `achieved` is T_roof over the measured step (one graph launch): the near field overlaps the far field,
    so the stage times, each measured by the library's events, add up to more than the step."""
    order = arm.get("order") or 3
    K = (order + 1) * (order + 2) // 2
    nodes, c = arm["nonempty_nodes"], arm["counters"]
    stages = {
        "sort": (100.0 * n, 0.0),
        "build": (12.0 * n + nodes * (4.0 * K + 28.0), 0.0),
        "lists": (4.0 * (c["m2l"] + arm["near_pairs"]), 0.0),
        "far": (8.0 * K * nodes, float(m2l_flops(order)) * c["m2l"]),
        "near": (16.0 * n, 20.0 * c["p2p_pairs"]),
        "l2p": (40.0 * n + 4.0 * K * nodes, 5.0 * (order * (order + 1) // 2) * n),
        "reduce": (8.0 * n, 0.0),
    }
    out, t_roof = {}, 0.0
    for k, (b, f) in stages.items():
        t = max(b / (hbm_gbs * 1e9), f / (fp32_tflops * 1e12)) * 1e3
        t_roof += t
        out[k] = {"roof_ms": round(t, 4), "ms": round(arm["stages"].get(k, 0.0), 4)}
    t_meas = sum(max(v, 0.0) for v in arm["stages"].values())
    return {"t_roof_ms": round(t_roof, 4), "t_stages_ms": round(t_meas, 4), "t_step_ms": round(ms_per_step, 4),
            "achieved": round(t_roof / ms_per_step, 4) if ms_per_step > 0 else None, "stages": out}


def arm_summary(n, steps, a):
    return {"particles_per_s": n * steps / a["t_total"], "ms_per_step": 1e3 * a["t_total"] / steps,
            "depth": a["depth"], "order": a.get("order"), "theta": a.get("theta"), "tau": a.get("tau"),
            "mac": a.get("mac"), "centre": a.get("centre"), "m2l": a.get("m2l"), "median_err": a["err"][0],
            **({"judge": a["judge"]} if a.get("judge") else {})}


def compact_calib(calib):
    """The chosen configurations only; the trial lists go to the record file."""
    keep = ("mac", "centre", "m2l", "depth", "theta", "order", "leaf_p2p", "tau", "ms", "err", "median_err",
            "particles_per_s")
    out = {}
    for k in ("plain_best", "plain_p12", "plain_tensor", "learned_best", "reference_order"):
        v = calib.get(k)
        out[k] = None if v is None else {a: v[a] for a in keep if a in v}
    if calib.get("controller"):
        c = calib["controller"]
        out["controller"] = {a: c[a] for a in ("samples", "systems", "system_n", "steps", "orders") if a in c}
    out["trials"] = {"plain": len(calib.get("plain_trials") or []), "learned": len(calib.get("learned_trials") or [])}
    return out


# DRAM bytes (read + write) of one k_near_p launch, from an ncu capture of the force step at that configuration
# (dram__bytes_read.sum + dram__bytes_write.sum), keyed by (n, depth, order, opening criterion, theta, leaf P2P,
# expansion centre).
NEAR_TRAFFIC = {
    (4194304, 11, 8, "bmax", 0.75, 64, "com"): (75632128 + 12529664,
                                          "ncu dram__bytes_read.sum + dram__bytes_write.sum of one k_near_p launch "
                                          "of the force step at this configuration (P2P only; bit-exact tree)"),
}


def headline_line(args, w, r, world, config, peaks, peak_src, sms):
    n = w["n"]
    head = r["arms"][r["head"]]
    value = n * world * args.steps / head["t_total"]
    e2e_s = float(np.mean(r["e2e_ms"])) / 1e3
    sm_mhz = peaks.get("sm_max_mhz", 2070.0)
    fp32_peak = sms * 128 * 2 * sm_mhz * 1e6 / 1e12  # TFLOP/s, nominal at the max SM clock
    t_near = head["stages"]["near"] / 1e3
    flops = 20.0 * head["counters"]["p2p_pairs"]
    achieved = flops / t_near / 1e12 if t_near > 0 else None
    comparison = {k: arm_summary(n, args.steps, a) for k, a in r["arms"].items()}
    if "learned" in comparison:
        lv = comparison["learned"]["particles_per_s"]
        for k in ("plain_p12", "plain_best"):
            if k in comparison:
                comparison[f"learned_speedup_vs_{k}"] = lv / comparison[k]["particles_per_s"]
    ro = r["calib"].get("reference_order")
    if ro:
        comparison["reference_order_gpu"] = {a: ro[a] for a in ("theta", "median_err", "ms_per_step",
                                                                "particles_per_s", "depth")}
    method = {"learned": "learned-order symmetric Morton FMM: MLP controller (16-64-64-5, BF16 tensor-core "
                         "inference in the list build) picks accept/open and the order in {4,6,8,10,12} per pair",
              "plain_best": "plain fixed-order symmetric Morton FMM (autotuned expansion centre and M2L engine, "
                            "opening criterion, depth, theta and order)"}[r["head"]]
    config = dict(config)
    config.update({"theta": head.get("theta"), "tau": head.get("tau"), "depth": head["depth"], "mac": head.get("mac"),
                   "order": head.get("order"), "method": r["head"],
                   "centre": head.get("centre"), "m2l": head.get("m2l"),
                   "leaf_p2p": head.get("leaf_p2p", config.get("leaf_p2p")),
                   "expansion": ("total-order Cartesian Taylor about the cell centre, M2L on the tensor cores (BF16 "
                                 "hi/lo split, FP32 accumulation) on the deep levels" if head.get("centre") == "box"
                                 else "total-order Cartesian Taylor about the COM, FP32 SIMT M2L"),
                   "tree": "Morton codes, permutation and topology bit-exact to the reference (FP64 quantisation, "
                           "32-bit stable sort)",
                   "autotune": compact_calib(r["calib"]),
                   "error_rows": "chosen on one seeded sample of 4,096 sinks, reported on a disjoint one",
                   "l2": "256 MB buffer written between timed steps (inputs also exceed L2)",
                   "step": ("one CUDA graph launch per step (update + solve captured over the exact box, "
                            "stage times from the uncaptured warm-up steps)" if head.get("graph")
                            else "updateTree + solveNbody calls")})
    key = (n, config["depth"], config["order"], config["mac"], config["theta"], config["leaf_p2p"], config["centre"])
    traffic, traffic_src = NEAR_TRAFFIC.get(key, (None, "no ncu capture of this configuration"))
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * head["t_total"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded two-disk positions; no published dataset for this workload)",
        "config": config,
        "method": method,
        "comparison": comparison,
        "error": {"median": head["err"][0], "p90": head["err"][1], "max": head["err"][2], "vs": "fp64 direct sum",
                  "samples": N_SAMPLES},
        "stages_ms": {k: round(v, 4) for k, v in head["stages"].items()},
        "counters": head["counters"],
        "roofline": {"kernel": "k_near_p (P2P; the L2P is k_l2p_p)", "bound": "fp32",
                     "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": (achieved / fp32_peak) if achieved else None, "traffic": traffic,
                     "traffic_source": traffic_src, "flops_per_pair": 20,
                     "peak_source": f"nominal: {sms} SMs x 128 FP32 lanes x 2 x {sm_mhz:.0f} MHz "
                                    f"(MEASURED_PEAKS.json holds no FP32 figure; HBM peak {peak_src})"},
        "step_roofline": step_roofline(n, head, peaks.get("hbm_gbs", 6800.0), fp32_peak,
                                       1e3 * head["t_total"] / args.steps),
        # H2D: positions, IDs, the gradient the forces add to; D2H: sorted positions, IDs, gradient, pair sum
        "e2e": {"value": n * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": n * 16 + n * 4 + n * 16,
                "d2h_bytes_per_step": n * 16 + n * 4 + n * 16 + 8},
        "gpu_launches": head["launches"],
        "clocks": head["clocks"],
    }


REF_THETA = 0.15
REF_SAMPLE = 65536


def run_reference(args, w, config):
    """The reference's CPU algorithm (the C oracle port of NBodySolverFMM_SYM_MORTON, single-threaded per
    system as the reference is) on every host core, each core solving an independent bounded sample of
    the workload's distribution, at the opening angle the reference's fixed order needs for the error
    target on the full 4M-particle workload (0.15: the GPU run of the same reference-order method,
    which visits the same interactions, measures 1e-4 median error there at that angle).  The error of
    the timed samples against an FP64 direct sum is measured (untimed) and reported."""
    import oracle
    from masterthesislucas_gb300 import datasets

    theta = args.theta or REF_THETA
    threads = os.cpu_count() or 1
    n_s = args.ref_sample
    vals, dts = [], []
    for k in range(args.warmup + args.steps):
        v, dt, depth = cpu_baseline(w, theta, n_s, threads=threads, seeds=[k * 1000 + i for i in range(threads)])
        if k >= args.warmup:
            vals.append(v)
            dts.append(dt)
    # error of the reference method on one timed sample (its first system), 1,024 sampled sinks
    p = np.ascontiguousarray(datasets.two_disks(n_s, seed=5000 + args.warmup * 1000).astype(np.float64)
                             if w["dist"] == "two_disks" else
                             datasets.gaussian_mixture(n_s, seed=5000 + args.warmup * 1000).astype(np.float64))
    kern = 1 if w["kernel"] == "gravity" else 0
    r = oracle.sym_fmm(p, kernel=kern, eps=w["softening"], max_children=w["max_children"], theta=theta,
                       want_nodes=False)
    g = np.zeros_like(p)
    g[r["ids"]] = r["grad"]
    rows = np.sort(np.random.default_rng(9).choice(n_s, 1024, replace=False)).astype(np.int64)
    fd = np.zeros((len(rows), 2))
    oracle.lib().orc_direct_rows(kern, w["softening"], n_s, oracle._p(p), len(rows), oracle._p(rows),
                                 oracle._p(fd), threads)
    err = median_error(g[rows], fd)
    value = float(np.mean(vals))
    config = dict(config)
    config.update({"theta": theta, "sample_n": n_s, "sample_depth": depth, "order": "reference (M0 + M2, C1-C3)"})
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(dts)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded two-disk positions)", "config": config,
            "error": {"median": err[0], "p90": err[1], "max": err[2], "vs": "fp64 direct sum",
                      "samples": len(rows), "on": f"one {n_s}-particle sample"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{threads} independent {n_s}-particle systems of the same distribution "
                                       f"per step, leaf {w['max_children']} (depth {depth}), theta {theta}, "
                                       f"one per core"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def spawn_ranks(n):
    """--gpus N without a launcher: re-run this script under torch.distributed.run with N local ranks."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr", "127.0.0.1", "--master-port", str(29500 + os.getpid() % 1000),
           os.path.abspath(__file__)] + sys.argv[1:]
    return subprocess.call(cmd)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="nbody_two_disks_4m", choices=sorted(WORKLOADS))
    ap.add_argument("--theta", type=float, default=None)
    ap.add_argument("--order", type=int, default=0, help="fix the expansion order instead of autotuning")
    ap.add_argument("--leaf-p2p", type=int, default=64,
                    help="order-p arms: accepted leaf pairs with at most this many particle pairs use P2P")
    ap.add_argument("--mac", default="all",
                    help="opening criterion of the plain arms: cell, bmax, bmax_adaptive:<slack> (per-pair "
                         "orders), or all (autotuned over these)")
    ap.add_argument("--depth", type=int, default=0)
    ap.add_argument("--centre", default="com", choices=["com", "box"],
                    help="with --order: expansion centre (centre of mass, or cell centre)")
    ap.add_argument("--m2l", default="simt", choices=["simt", "tensor", "tensor_all"],
                    help="with --order and --centre box: the M2L engine")
    ap.add_argument("--engines", default="all", choices=["all", "com", "box"],
                    help="autotuned arms: COM-centred with the SIMT M2L, box-centred with the tensor-core M2L")
    ap.add_argument("--no-near-overlap", action="store_true",
                    help="order p: run the near field after the far field on one stream (default: beside it)")
    ap.add_argument("--skip-reference-order", action="store_true")
    ap.add_argument("--cpu-sample", type=int, default=262144)
    ap.add_argument("--ref-sample", type=int, default=REF_SAMPLE,
                    help="--impl reference: particles per core and step")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-order controller arm")
    ap.add_argument("--tau", type=float, default=0.0, help="fix the controller tolerance instead of tuning it")
    ap.add_argument("--no-graph", action="store_true", help="time update + solve calls instead of the captured step")
    ap.add_argument("--learned-depth", type=int, default=0)
    ap.add_argument("--ctrl-steps", type=int, default=CTRL_STEPS, help="controller training steps")
    ap.add_argument("--record", default=os.path.join(ROOT, "_bench_records"),
                    help="directory for the full autotuning record (every trial), kept out of the printed line")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    w = WORKLOADS[args.workload]
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(spawn_ranks(args.gpus))
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    config = {"workload": args.workload, "n": w["n"], "distribution": w["dist"], "kernel": w["kernel"],
              "softening": w["softening"], "leaf_size": w["max_children"],
              "precision": ("fp32 expansions, P2P, MACs and tree moments (cell-relative coordinates formed "
                            "from fp64 positions); fp64 Morton quantisation and pair sum Z"),
              "error_target": TARGET_ERR, "error_samples": N_SAMPLES, "leaf_p2p": args.leaf_p2p,
              "parallelism": f"{world} replica(s), one independent system per GPU, no exchange"}

    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(run_reference(args, w, config)))
        return

    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        dist.init_process_group("nccl")
        if w.get("method") not in (None, "tsne_batch"):
            raise SystemExit(f"--gpus {world}: the {args.workload} workload runs on one GPU; the force-step "
                             "workloads (replicas) and tsne_batch_256 (systems sharded) run on several")
    if w.get("method") == "tsne_batch":
        run_tsne_batch(args, w)
        return
    if w.get("method") == "leapfrog":
        run_leapfrog(args, w)
        return
    if w.get("method") == "bh":
        run_bh(args, w)
        return
    if w.get("method") == "pm":
        run_pm(args, w)
        return
    if w.get("method") == "tsne":
        run_tsne(args, w)
        return
    r = run_ours(args, w, rank, world)
    if rank != 0:
        return
    import torch
    sms = torch.cuda.get_device_properties(int(os.environ.get("LOCAL_RANK", 0))).multi_processor_count
    peaks, peak_src = load_peaks()
    line = headline_line(args, w, r, world, config, peaks, peak_src, sms)
    if not args.no_cpu_baseline:
        ref_th = (r["calib"]["reference_order"] or {}).get("theta", REF_THETA)
        v, dt, depth = cpu_baseline(w, ref_th, args.cpu_sample, threads=1, seeds=[0])
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": f"one {args.cpu_sample}-particle system of the same distribution, "
                                          f"leaf {w['max_children']} (depth {depth}), reference order, "
                                          f"theta {ref_th} (the angle its order needs for the error target), "
                                          f"{dt:.1f} s"}
    if args.record:
        os.makedirs(args.record, exist_ok=True)
        with open(os.path.join(args.record, f"autotune_{args.workload}.json"), "w") as f:
            json.dump({"calib": r["calib"], "arms": {k: {a: v for a, v in arm.items() if a != "ms"}
                                                     for k, arm in r["arms"].items()}}, f, default=str)
    print(json.dumps(line))


if __name__ == "__main__":
    main()
