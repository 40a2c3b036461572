"""Benchmark of the GB300 collision-handling step.

Workload: the self-collision scene - one 129x129-vertex cloth (32,768
triangles), sinusoidal start, velocity -2*grad(phi) of a seeded field,
dt = h = 5e-4 - resolved step by step as the reference's host loop does
(x_cand = x_old + dt*vel, then resolveCollision). A step is one
resolveCollision() on the current state; the trajectory continues across
warm-up and timed steps. Metric: collision-resolved scene-steps per second.

  value  device-resident: inputs in HBM, each step through cc_resolve_device
  e2e    the same steps through cc_resolve with pinned host buffers, copies
         inside the timed region
  L2     flushed (256 MiB write) before every timed step; the working set
         (~8 MB) would otherwise stay in the 129 MB L2

--impl reference times the CPU implementation of the same path (the C
restatement of the reference in oracle/, which is bit-exact to it; the
reference's own sources are not available on the GPU host) on the host
cores. Under torchrun every rank runs an independent replica (different
seed): the path does not shard.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cloth collision steps/s: mixed-prec batched vs FP64 plain, 0 missed CCD"
UNIT = "scene-steps/s"
WORKLOAD = "folded_cloth"
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")


def make_scene(seed):
    from collision_gb300 import scenes
    return scenes.folded_cloth(seed=seed)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rk = int(os.environ.get("RANK", "0"))
    lrk = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rk, lrk


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, device):
        self.device = device
        self.samples = []
        self._stop = threading.Event()
        self._proc = None

    def __enter__(self):
        cmd = ["nvidia-smi", f"--id={self.device}",
               "--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
               "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
               "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200"]
        try:
            self._proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except OSError:
            self._proc = None
        return self

    def _read(self):
        for line in self._proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 6:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self._proc:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except Exception:
                self._proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[2 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def cpu_oracle_rate(seed, budget_s, max_steps):
    """Steps/s of the single-threaded CPU restatement on this workload, from
    the start of the trajectory, within a time budget."""
    from collision_gb300 import scenes
    from oracle.ccopy import OracleSolver
    sc = make_scene(seed)
    o = OracleSolver(sc, record=0)
    x, v, hc = sc.x.copy(), sc.v.copy(), np.zeros(sc.nv, np.uint8)
    n, t_total = 0, 0.0
    while n < max_steps and t_total < budget_s:
        xc = scenes.candidate(sc, x, v)
        t0 = time.perf_counter()
        r = o.step(x, xc, v, hc)
        t_total += time.perf_counter() - t0
        if r["rc"] != 0:
            raise RuntimeError(f"oracle step failed: {r['rc']}")
        x, v, hc = r["x"], r["v"], r["has_collsn"]
        n += 1
    return n / t_total, n, t_total


def run_reference(args):
    ws, rk, _ = dist_env()
    if rk != 0:
        return
    # warm-up steps are part of the trajectory, untimed
    from collision_gb300 import scenes
    from oracle.ccopy import OracleSolver
    sc = make_scene(args.seed)
    o = OracleSolver(sc, record=0)
    x, v, hc = sc.x.copy(), sc.v.copy(), np.zeros(sc.nv, np.uint8)
    times = []
    for step in range(args.warmup + args.steps):
        xc = scenes.candidate(sc, x, v)
        t0 = time.perf_counter()
        r = o.step(x, xc, v, hc)
        dt = time.perf_counter() - t0
        if step >= args.warmup:
            times.append(dt)
        x, v, hc = r["x"], r["v"], r["has_collsn"]
    total = sum(times)
    value = len(times) / total
    sample = f"{WORKLOAD} 129x129, steps {args.warmup}..{args.warmup + args.steps - 1} of the trajectory"
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total / len(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "grid": "129x129", "tris": 32768, "dt": 5e-4, "h": 5e-4,
                       "parallelism": "replicas"},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gpu(args):
    import torch
    ws, rk, lrk = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    dev = lrk if torch.cuda.is_available() else 0
    torch.cuda.set_device(dev)
    from collision_gb300 import scenes
    from collision_gb300._lib import load
    from collision_gb300.solver import CollisionSolver3d
    lib = load()
    seed = args.seed + rk
    sc = make_scene(seed)
    dt = sc.params["dt"]
    stream = torch.cuda.Stream(device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    # ---------------------------------------------- device-resident runs
    def device_run(mode):
        """W untimed + K timed steps from the scene's start, each step
        through cc_resolve_device; returns total timed ms and the counters."""
        s = CollisionSolver3d(dev)
        s.assembleFromScene(sc)
        s.setMode(mode)
        s.setStream(stream.cuda_stream)
        with torch.cuda.stream(stream):
            x = torch.tensor(sc.x, dtype=torch.float64, device=dev)
            v = torch.tensor(sc.v, dtype=torch.float64, device=dev)
            hc = torch.zeros(sc.nv, dtype=torch.uint8, device=dev)
            xc = torch.empty_like(x)
            xo = torch.empty_like(x)
        launches, counters = [], []
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        with torch.cuda.stream(stream):
            for _ in range(args.warmup):
                torch.add(x, v, alpha=dt, out=xc)
                s.resolveCollisionDevice(x, xc, v, hc, xo)
                x, xo = xo, x
        stream.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        s.setProfiling(True)
        with Clocks(dev) as clk, torch.cuda.stream(stream):
            for k in range(args.steps):
                flush.fill_(float(k))
                evs[k][0].record(stream)
                torch.add(x, v, alpha=dt, out=xc)
                s.resolveCollisionDevice(x, xc, v, hc, xo)
                evs[k][1].record(stream)
                c = s.counters()
                counters.append(c)
                launches.append(c["kernel_launches"] + 1)  # + the candidate update
                x, xo = xo, x
            stream.synchronize()
        torch.cuda.synchronize()
        step_ms = [a.elapsed_time(b) for a, b in evs]
        prof = s.profile()
        s.close()
        total_ms = float(sum(step_ms))
        if ws > 1:
            t = torch.tensor([total_ms], dtype=torch.float64, device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            total_ms = float(t.item())
            torch.distributed.barrier()
        return total_ms, step_ms, counters, launches, prof, clk.summary()

    plain_ms, plain_steps, plain_ctr, _, plain_prof, _ = device_run(0)
    total_ms, step_ms, counters, launches, prof, clocks = device_run(1)
    value = ws * args.steps / (total_ms / 1e3)
    plain_value = ws * args.steps / (plain_ms / 1e3)

    # ------------------------------------------------------ end-to-end run
    s2 = CollisionSolver3d(dev)
    s2.assembleFromScene(sc)
    s2.setMode(1)
    s2.setStream(stream.cuda_stream)
    pin = lambda a, dtp: torch.tensor(a, dtype=dtp).pin_memory()
    hx = pin(sc.x, torch.float64)
    hv = pin(sc.v, torch.float64)
    hhc = torch.zeros(sc.nv, dtype=torch.uint8).pin_memory()
    hxc = torch.empty_like(hx).pin_memory()
    hxo = torch.empty_like(hx).pin_memory()
    import ctypes as C
    hcol = C.c_int(0)

    def e2e_step():
        torch.add(hx, hv, alpha=dt, out=hxc)
        st = lib.cc_resolve(s2._h, hx.data_ptr(), hxc.data_ptr(), hv.data_ptr(), hhc.data_ptr(), hxo.data_ptr(),
                            C.byref(hcol))
        if st != 0:
            s2._check(st)
        hx.copy_(hxo)

    for _ in range(args.warmup):
        e2e_step()
    e2e_ms = []
    ev2 = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.fill_(float(k))
            stream.synchronize()
            ev2[k][0].record(stream)
            e2e_step()
            ev2[k][1].record(stream)
        stream.synchronize()
    e2e_total = sum(a.elapsed_time(b) for a, b in ev2)
    if ws > 1:
        t = torch.tensor([e2e_total], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_total = float(t.item())
    e2e_value = ws * args.steps / (e2e_total / 1e3)
    h2d = sc.nv * (3 * 8 * 3 + 1)
    d2h = sc.nv * (3 * 8 * 2 + 1)

    if rk != 0:
        if ws > 1:
            torch.distributed.destroy_process_group()
        return

    # ----------------------------------------------------------- roofline
    peaks = json.load(open(PEAKS)) if os.path.exists(PEAKS) else {}
    hbm = peaks.get("hbm_gbs")
    peak_src = "measured" if hbm else "fallback"
    hbm = hbm or 6800.0
    tot = {k: sum(c[k] for c in counters) for k in counters[0]} if counters else {}
    ptot = {k: sum(c[k] for c in plain_ctr) for k in plain_ctr[0]} if plain_ctr else {}
    # dominant kernel: the CCD narrow phase. Algorithmic bytes per visited
    # pair: the pair (8 B), both leaf ranks (8 B), both elements' point ids
    # (24 B) and the x_old + avgVel records of its up to 6 points (6 x 64 B);
    # plus 64 B per contribution written.
    narrow_ms, narrow_calls = plain_prof.get("narrow_ccd", (0.0, 0))
    ccd_visits = ptot.get("visits", 0)  # all passes; CCD share estimated below
    bytes_per_visit = 8 + 8 + 24 + 6 * 64
    roof = None
    if narrow_calls:
        # visits of CCD passes: total visits minus proximity visits (one
        # proximity pass per step visits about as many pairs as one CCD pass)
        passes = max(ptot.get("passes", 1), 1)
        ccd_share = (passes - args.steps) / passes
        algo = bytes_per_visit * ccd_visits * ccd_share / narrow_calls
        avg_s = narrow_ms / narrow_calls / 1e3
        achieved = algo / avg_s / 1e9
        roof = {"bound": "hbm", "kernel": "k_narrow<true> (CCD narrow phase, plain FP64)", "achieved": achieved,
                "peak": hbm, "unit": "GB/s", "frac": achieved / hbm, "peak_source": peak_src,
                "traffic": None, "note": "FP64-ALU bound: FP64 is ~1.25 TFLOP/s nominal on GB300"}
    cpu = None
    if not args.no_cpu_baseline:
        rate, n, t = cpu_oracle_rate(seed, args.cpu_budget, args.warmup + args.steps)
        cpu = {"value": rate, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"{WORKLOAD} 129x129, first {n} steps of the trajectory ({t:.1f} s)"}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64 (f32 filters)", "data": "synthetic",
            "config": {"workload": WORKLOAD, "grid": "129x129", "tris": 32768, "dt": 5e-4, "h": 5e-4,
                       "path": "mixed: FP32 sub-test filters, FP64 tests (results identical to plain FP64)",
                       "l2": "flushed before every timed step",
                       "parallelism": "replicas" if ws > 1 else "single"},
            "plain_fp64": {"value": plain_value, "ms_per_step": plain_ms / args.steps,
                           "fp64_subtests": int(sum(c.get("fp64_subtests", 0) for c in plain_ctr)),
                           "stages_ms": {k: round(v[0], 3) for k, v in plain_prof.items()}},
            "roofline": roof, "cpu_baseline": cpu, "clocks": clocks,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": int(sum(launches)),
            "step_ms_quantiles": [round(float(q), 3) for q in np.quantile(step_ms, [0, 0.25, 0.5, 0.75, 1.0])],
            "counters": tot, "stages_ms": {k: round(v[0], 3) for k, v in prof.items()}}
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
