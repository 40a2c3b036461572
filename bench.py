"""Benchmark of the GB300 collision-handling step.

Default workload (`batched`): 256 independent cloth-on-obstacle scenes -
sheet resolution 16..128 vertices per side, a fixed sphere (642 points,
r ~ U(0.1, 0.3)) or box (12 triangles) by coin flip, v = (0,0,-U(0.5,3))
+-1 %, dt = h = 1e-3 - all seeded, synthetic. Each cloth starts above its
obstacle by the distance it falls in U(1, 4) steps, so every scene is in
contact from its first steps on and the warm-up and timed steps are contact
steps (--placement freefall puts the cloths 0.05 above a sphere and 0.10
above a box instead, which most take 20-200 steps of free fall to cross).
One step = one resolveCollision() of every scene on its current state, as the
reference's host loop does (x_cand = x_old + dt*vel, then resolve); the
trajectory runs on across warm-up and timed steps. Metric: collision-resolved
scene-steps per second.

  value       mixed precision, batched: all scenes in one solver, inputs in
              HBM, each step through cc_resolve_batch_device
  plain_fp64  the plain FP64 GPU path one scene at a time (one solver per
              scene, cc_resolve_device on each) over the first
              --plain-steps timed steps of the same trajectory; its state
              must equal the batch's bit for bit
  batched_plain_fp64  the whole batch in plain FP64 over the same steps
  e2e         the batched mixed path through cc_resolve_batch with pinned
              host buffers, copies inside the timed region
  missed_ccd  element pairs that still collide after a step, by the exact
              FP64 CCD re-check (cc_check_ccd) after every timed step,
              outside the timed region
  parity_vs_cpu  the CPU baseline's scenes stepped by the oracle (the C
              restatement, bit-exact to the reference) over the same steps
              from the same initial state, against the GPU batch's state for
              those scenes after the same number of steps
  zone cap    the reference's impact-zone loop does not end on some scenes;
              such a scene stops after --zone-cap zone passes, is counted in
              capped_scenes and is left out of the following steps (in every
              arm alike)
  autotune    after the warm-up steps, cc_autotune picks the traversal and
              narrow-phase launch shapes on the state reached (outside the
              timed region); the chosen settings are reported
  L2          flushed (256 MiB write) before every timed step

--workload picks one of the other measured scenes (folded_cloth,
cloth_on_sphere, strings, large) as a batch of one. --impl reference times
the CPU implementation of the same path (the C restatement of the reference
in oracle/, which is bit-exact to it; the reference's own sources are not on
the GPU host) on all host cores, one scene per thread, on the CPU sample of
the workload (batched: every fourth scene by size, 64 of 256). Under
torchrun every rank runs an independent replica (different seed).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cloth collision steps/s: mixed-prec batched vs FP64 plain, 0 missed CCD"
UNIT = "scene-steps/s"
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
# The traversal's DRAM traffic (bytes read + written) per query leaf and
# its threads active per instruction, from one ncu capture of each kernel on
# the batched workload cut to 96 scenes, each a full traversal of all
# 1,298,248 elements: k_traverse_rope_dyn 257.1 MB and k_traverse_rope
# 215.8 MB (the first traversal of the run, the proximity pass of step 1),
# k_traverse (a stack per thread) 221 MB (a free-fall step)
TRAVERSE_DRAM_BYTES_PER_LEAF = {"dyn": 198.0, "rope": 166.2, "stack": 170.4}
TRAVERSE_LANES_ACTIVE = {"dyn": 7.8, "rope": 6.2, "stack": 7.4}
TRAVERSE_KERNEL = {"dyn": "k_traverse_rope_dyn (LBVH broad phase, stackless, persistent warps refilling lanes)",
                   "rope": "k_traverse_rope (LBVH broad phase, stackless along ropes, one thread per query)",
                   "stack": "k_traverse (LBVH broad phase, a stack per thread)"}
# FP64 operations (dadd + dmul + 2 dfma) per queued FP64 sub-test, from one
# ncu capture of both k_subtests launches of a CCD pass of the same 96
# scenes: 85.6 MFLOP for 123,752 point-triangle and 44,900 edge-edge
# sub-tests; GB300's FP64 peak is 1.25 TFLOP/s (nominal: none measured)
SUBTEST_FP64_FLOPS = 507.6
FP64_PEAK_TFLOPS = 1.25
# the CCD filter's algorithmic bytes per visited pair: the pair, two ranks,
# the two elements' point ids, FP32 x_old and avgVel of six points
FILTER_BYTES_PER_VISIT = 8 + 8 + 24 + 6 * 32


def make_workload(name, seed, nscenes=0, large_n=1025, placement="contact"):
    from collision_gb300 import scenes
    if name == "large":
        return [scenes.large(n=large_n, seed=seed)]
    if name == "batched":
        scs = scenes.batched(seed=seed, approach_steps=(1.0, 4.0) if placement == "contact" else None)
    else:
        scs = scenes.workload(name, seed=seed)
    return scs[:nscenes] if nscenes > 0 else scs


def cpu_sample(scs):
    """Indices of the scenes the CPU legs step: every fourth scene in size
    order (the second of each group of four) for batches of 16 or more,
    else all."""
    if len(scs) < 16:
        return list(range(len(scs)))
    order = sorted(range(len(scs)), key=lambda i: scs[i].ne)
    return sorted(order[1::4])


def describe(name, scs, placement=None):
    nv = sum(s.nv for s in scs)
    nt = sum(s.nt for s in scs)
    nb = sum(s.nb for s in scs)
    d = {"workload": name, "scenes": len(scs), "points": nv, "tris": nt, "bonds": nb,
         "dt": sorted({s.params["dt"] for s in scs}), "h": sorted({s.params["thickness"] for s in scs})}
    if name == "batched":
        d["sheet_sides"] = [16, 128]
        d["obstacles"] = {"sphere": sum("sphere" in s.name for s in scs), "box": sum("box" in s.name for s in scs)}
        if placement:
            d["placement"] = ("each cloth above its obstacle by its fall in U(1, 4) steps: contact from the first "
                              "steps" if placement == "contact" else "0.05 above a sphere, 0.10 above a box")
    return d


def dist_env():
    from collision_gb300.replicas import dist_env as env
    return env()


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, device):
        self.device = device
        self.samples = []
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


# ------------------------------------------------------------- CPU (oracle)
ORACLE_ITER_CAP = -3


def one_core_rate(scs, max_steps, budget_s, zone_cap):
    """The CPU restatement on one host core - the reference's own
    single-threaded form - over a sample of the scenes by size: the median
    scene of every sixteenth of them in size order (one scene when there are
    fewer than 16). Same trajectory and bounds as oracle_rate."""
    order = sorted(range(len(scs)), key=lambda i: scs[i].ne)
    one = [scs[i] for i in order[len(order) // 32::16]]
    rate, n, t, steps, _ = oracle_rate(one, max_steps, budget_s, 1, zone_cap)
    return {"value": rate, "unit": UNIT, "cores": 1,
            "sample": f"{len(one)} of {len(scs)} scenes (the median of every sixteenth by size), first {steps} "
                      f"steps ({n} scene-steps, {t:.1f} s)"}


def oracle_rate(scs, max_steps, budget_s, threads, zone_cap, skip_steps=0):
    """Scene-steps/s of the CPU restatement over the trajectory, all scenes
    stepped together (one scene per thread, `threads` at once, largest
    first); the first `skip_steps` steps are run untimed. Stops after
    max_steps timed steps or once budget_s of timed steps has passed. A scene
    whose impact-zone loop reaches zone_cap is left out from then on, as in
    the GPU arms. Returns (rate, scene-steps, seconds, steps, final states:
    (x, v, has_collsn, live) per scene)."""
    from collision_gb300 import scenes
    from oracle.ccopy import OracleSolver
    solvers = [OracleSolver(sc, record=0) for sc in scs]
    for o in solvers:
        o.set_zone_cap(zone_cap)
    state = [(sc.x.copy(), sc.v.copy(), np.zeros(sc.nv, np.uint8)) for sc in scs]
    prev = [None] * len(scs)
    live = [True] * len(scs)
    by_size = sorted(range(len(scs)), key=lambda i: -scs[i].ne)

    def one(i):
        if not live[i]:
            return 0
        x, v, hc = state[i]
        r = solvers[i].step(x, scenes.candidate(scs[i], x, v), v, hc)
        if r["rc"] == ORACLE_ITER_CAP:
            live[i] = False
            return 1
        if r["rc"] != 0:
            raise RuntimeError(f"oracle step failed on scene {i}: {r['rc']}")
        prev[i] = x
        state[i] = (r["x"], r["v"], r["has_collsn"])
        return 1

    done, t_total, steps = 0, 0.0, 0
    with ThreadPoolExecutor(max_workers=threads) as ex:
        for _ in range(skip_steps):
            list(ex.map(one, by_size))
        while steps < max_steps and t_total < budget_s:
            t0 = time.perf_counter()
            n = sum(ex.map(one, by_size))
            t_total += time.perf_counter() - t0
            done += n
            steps += 1
    # the exact CCD re-check of each scene's last step, on the oracle's own
    # results (untimed)
    missed = [solvers[i].check_ccd(prev[i], state[i][0]) if live[i] and prev[i] is not None else 0
              for i in range(len(scs))]
    for o in solvers:
        o.close()
    final = [(x, v, hc, lv, m) for (x, v, hc), lv, m in zip(state, live, missed)]
    return done / t_total, done, t_total, steps, final


def oracle_replay(sc, steps, zone_cap, crmath=False):
    """One scene stepped `steps` times by the oracle (crmath: its build with
    correctly rounded acos/cos/sin/pow); returns (x, v, has_collsn)."""
    from collision_gb300 import scenes
    from oracle.ccopy import OracleSolver
    o = OracleSolver(sc, record=0, crmath=crmath)
    o.set_zone_cap(zone_cap)
    x, v, hc = sc.x.copy(), sc.v.copy(), np.zeros(sc.nv, np.uint8)
    for _ in range(steps):
        r = o.step(x, scenes.candidate(sc, x, v), v, hc)
        if r["rc"] != 0:
            break
        x, v, hc = r["x"], r["v"], r["has_collsn"]
    o.close()
    return x, v, hc


def run_reference(args):
    ws, rk, _ = dist_env()
    if rk != 0:
        return
    scs = make_workload(args.workload, args.seed, args.scenes, args.large_n, args.placement)
    idx = cpu_sample(scs)
    sub = [scs[i] for i in idx]
    threads = os.cpu_count() or 1
    rate, n, t, steps, _ = oracle_rate(sub, args.steps, args.ref_budget, threads, args.zone_cap,
                                       skip_steps=args.warmup)
    sample = (f"{args.workload}: {len(sub)} of {len(scs)} scenes"
              f"{' (every fourth by size)' if len(sub) < len(scs) else ''}, steps {args.warmup}.."
              f"{args.warmup + steps - 1} of the trajectory ({n} scene-steps, {t:.1f} s), one scene per thread")
    line = {"metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": ws, "steps": steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t / max(steps, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": dict(describe(args.workload, scs, args.placement), parallelism="replicas"),
            "impl": "reference",
            "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------- GPU
def run_gpu(args):
    import torch
    ws, rk, lrk = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    dev = lrk
    torch.cuda.set_device(dev)
    from collision_gb300 import _lib
    from collision_gb300.solver import CollisionSolver3d
    from collision_gb300.replicas import max_over_ranks as mor, rank_seed
    seed = rank_seed(args.seed, rk)
    scs = make_workload(args.workload, seed, args.scenes, args.large_n, args.placement)
    nsc = len(scs)
    stream = torch.cuda.Stream(device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    x0 = np.concatenate([s.x for s in scs])
    v0 = np.concatenate([s.v for s in scs])
    dtcol = np.concatenate([np.full((s.nv, 1), s.params["dt"]) for s in scs])
    offs = np.cumsum([0] + [s.nv for s in scs])
    W, K = args.warmup, args.steps
    n_plain = min(K, args.plain_steps) if args.plain_steps > 0 else K

    def device_state():
        with torch.cuda.stream(stream):
            st = dict(x=torch.tensor(x0, device=dev), v=torch.tensor(v0, device=dev),
                      dt=torch.tensor(dtcol, device=dev), hc=torch.zeros(len(x0), dtype=torch.uint8, device=dev))
            st["xc"] = torch.empty_like(st["x"])
            st["xo"] = torch.empty_like(st["x"])
            st["tmp"] = torch.empty_like(st["x"])
        return st

    def candidate(st):
        # x_cand = x_old + dt*vel, two roundings as the reference's host loop
        torch.mul(st["v"], st["dt"], out=st["tmp"])
        torch.add(st["x"], st["tmp"], out=st["xc"])

    def sync_all():
        stream.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(ms):
        return mor(ms, device=dev)

    def apply_tuning(s):
        for kv in args.tune:
            k, v = kv.split("=")
            s.setTuning(getattr(CollisionSolver3d, "TUNE_" + k.strip().upper()), int(v))

    # ------------------------------------------- batched, device-resident
    def drop_capped(s, enabled):
        for q in np.nonzero(s.sceneStatus())[0]:
            s.setSceneEnabled(int(q), False)
            enabled[int(q)] = False

    def batched_run(mode, check):
        s = CollisionSolver3d(dev)
        s.assembleBatch(scs)
        apply_tuning(s)
        s.setMode(mode)
        s.setZoneCap(args.zone_cap)
        s.setStream(stream.cuda_stream)
        st = device_state()
        enabled = np.ones(nsc, dtype=bool)
        cpu_snap = None

        def snap_for_cpu(done):
            # the state of the CPU leg's scenes after as many steps as it ran
            nonlocal cpu_snap
            if cpu is not None and done == cpu["steps"]:
                cpu_snap = (st["x"].cpu().numpy(), st["v"].cpu().numpy(), st["hc"].cpu().numpy(), enabled.copy())

        with torch.cuda.stream(stream):
            for w in range(W):
                candidate(st)
                s.resolveCollisionBatchDevice(st["x"], st["xc"], st["v"], st["hc"], st["xo"])
                drop_capped(s, enabled)
                st["x"], st["xo"] = st["xo"], st["x"]
                snap_for_cpu(w + 1)
        sync_all()
        tuned = s.autotune() if not args.no_autotune else None
        sync_all()
        scene_steps = 0
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
        counters, missed, snap, cpu_missed = [], 0, None, None
        s.setProfiling(True)
        with Clocks(dev) as clk, torch.cuda.stream(stream):
            for k in range(K):
                flush.fill_(float(k))
                scene_steps += int(enabled.sum())
                evs[k][0].record(stream)
                candidate(st)
                s.resolveCollisionBatchDevice(st["x"], st["xc"], st["v"], st["hc"], st["xo"])
                evs[k][1].record(stream)
                counters.append(s.counters())
                drop_capped(s, enabled)
                if check:
                    hits, per = s.checkCCD(st["x"], st["xo"])
                    missed += hits
                    if cpu is not None and W + k + 1 == cpu["steps"]:
                        cpu_missed = per.copy()
                st["x"], st["xo"] = st["xo"], st["x"]
                if k + 1 == n_plain:
                    snap = (st["x"].cpu().numpy(), st["v"].cpu().numpy())
                if check:
                    snap_for_cpu(W + k + 1)
            stream.synchronize()
        torch.cuda.synchronize()
        step_ms = [a.elapsed_time(b) for a, b in evs]
        prof = s.profile()
        rope = ("dyn" if s.getTuning(CollisionSolver3d.TUNE_TRAVERSE_REFILL) > 0 else "rope") \
            if s.getTuning(CollisionSolver3d.TUNE_ROPE_TRAVERSE) else "stack"
        kprof = None
        if mode == 1 and args.kernel_steps > 0:
            # after the timed steps, untimed: a few more steps with every
            # pass's stages timed inside the device loop's graph too
            # (profiling level 2 adds boundary kernels to each pass, so the
            # timed steps run without them), for the per-kernel roofline
            # entries
            s.setProfiling(2)
            kc = []
            with torch.cuda.stream(stream):
                for k in range(args.kernel_steps):
                    candidate(st)
                    s.resolveCollisionBatchDevice(st["x"], st["xc"], st["v"], st["hc"], st["xo"])
                    kc.append(s.counters())
                    drop_capped(s, enabled)
                    st["x"], st["xo"] = st["xo"], st["x"]
                stream.synchronize()
            kprof = dict(prof=s.profile(), counters={k: sum(c[k] for c in kc) for k in kc[0]},
                         steps=args.kernel_steps)
        s.close()
        return dict(total_ms=max_over_ranks(float(sum(step_ms))), step_ms=step_ms, counters=counters,
                    missed=missed, snap=snap, prof=prof, clocks=clk.summary(), scene_steps=scene_steps,
                    capped=int((~enabled).sum()), tuned=tuned, rope=rope, cpu_snap=cpu_snap, cpu_missed=cpu_missed,
                    kprof=kprof)

    # ------------------------------ plain FP64, one scene at a time
    def plain_sequential():
        solvers = []
        for sc in scs:
            s = CollisionSolver3d(dev)
            s.assembleFromScene(sc)
            apply_tuning(s)
            s.setMode(0)
            s.setZoneCap(args.zone_cap)
            s.setStream(stream.cuda_stream)
            solvers.append(s)
        st = device_state()
        seq_enabled = np.ones(nsc, dtype=bool)

        def seq_step():
            candidate(st)
            for i, s in enumerate(solvers):
                a, b = int(offs[i]), int(offs[i + 1])
                if not seq_enabled[i]:  # left out, as in the batch: candidates pass through
                    st["xo"][a:b].copy_(st["xc"][a:b])
                    continue
                try:
                    s.resolveCollisionDevice(st["x"][a:b], st["xc"][a:b], st["v"][a:b], st["hc"][a:b], st["xo"][a:b])
                except _lib.CCError as e:
                    if e.status != CollisionSolver3d.ITER_CAP:
                        raise
                    seq_enabled[i] = False
            st["x"], st["xo"] = st["xo"], st["x"]

        with torch.cuda.stream(stream):
            for _ in range(W):
                seq_step()
        sync_all()
        seq_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n_plain)]
        seq_launches = 0
        seq_scene_steps = 0
        with torch.cuda.stream(stream):
            for k in range(n_plain):
                flush.fill_(float(k))
                seq_scene_steps += int(seq_enabled.sum())
                seq_ev[k][0].record(stream)
                seq_step()
                seq_ev[k][1].record(stream)
                seq_launches += 2 + sum(s.counters()["kernel_launches"] for s in solvers)
            stream.synchronize()
        seq_ms = max_over_ranks(float(sum(a.elapsed_time(b) for a, b in seq_ev)))
        seq_snap = (st["x"].cpu().numpy(), st["v"].cpu().numpy())
        for s in solvers:
            s.close()
        del solvers
        same = bool(np.array_equal(mixed["snap"][0], seq_snap[0]) and np.array_equal(mixed["snap"][1], seq_snap[1]))
        diff = float(np.abs(mixed["snap"][0] - seq_snap[0]).max())
        return dict(ms=seq_ms, scene_steps=seq_scene_steps, launches=seq_launches, same=same, diff=diff)


    # ------------------------------------------------ end to end (host)
    def e2e_run():
        s2 = CollisionSolver3d(dev)
        s2.assembleBatch(scs)
        apply_tuning(s2)
        s2.setMode(1)
        s2.setZoneCap(args.zone_cap)
        s2.setStream(stream.cuda_stream)
        e2e_enabled = np.ones(nsc, dtype=bool)
        pin = lambda a: torch.tensor(a).pin_memory()
        hx, hv, hdt = pin(x0), pin(v0), pin(dtcol)
        hhc = torch.zeros(len(x0), dtype=torch.uint8).pin_memory()
        hxc, hxo = torch.empty_like(hx).pin_memory(), torch.empty_like(hx).pin_memory()
        hcol = np.zeros(nsc, dtype=np.int32)
        import ctypes as C
        lib = s2._lib

        def e2e_call():
            rc = lib.cc_resolve_batch(s2._h, hx.data_ptr(), hxc.data_ptr(), hv.data_ptr(), hhc.data_ptr(),
                                      hxo.data_ptr(), hcol.ctypes.data_as(C.POINTER(C.c_int)))
            if rc not in (0, CollisionSolver3d.ITER_CAP):
                s2._check(rc)
            drop_capped(s2, e2e_enabled)

        def host_candidate():
            np.add(hx.numpy(), hdt.numpy() * hv.numpy(), out=hxc.numpy())

        for _ in range(W):
            host_candidate()
            e2e_call()
            hx.copy_(hxo)
        if not args.no_autotune:
            s2.autotune()
        ev2 = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
        with torch.cuda.stream(stream):
            for k in range(K):
                host_candidate()
                flush.fill_(float(k))
                stream.synchronize()
                ev2[k][0].record(stream)
                e2e_call()
                ev2[k][1].record(stream)
                hx.copy_(hxo)
            stream.synchronize()
        e2e_ms = max_over_ranks(float(sum(a.elapsed_time(b) for a, b in ev2)))
        s2.close()
        return e2e_ms


    # ------------- one scene: both arithmetic modes on the same solver
    def single_scene_pair():
        """Each timed step runs once in plain FP64 and once in mixed
        precision from the same inputs (in alternating order), in one
        solver, so the host's tree emulation is paid once; the two results
        must be equal bit for bit."""
        s = CollisionSolver3d(dev)
        s.assembleFromScene(scs[0])
        apply_tuning(s)
        s.setZoneCap(args.zone_cap)
        s.setStream(stream.cuda_stream)
        s.setMode(1)
        st = device_state()
        tree_us = 0
        with torch.cuda.stream(stream):
            # the approach (untimed steps that bring the scene into contact),
            # then the warm-up
            for _ in range(args.approach + W):
                candidate(st)
                s.resolveCollisionBatchDevice(st["x"], st["xc"], st["v"], st["hc"], st["xo"])
                tree_us += s.counters()["tree_build_us"]
                st["x"], st["xo"] = st["xo"], st["x"]
        sync_all()
        tuned = s.autotune() if not args.no_autotune else None
        ms = {0: 0.0, 1: 0.0}
        same = True
        counters = []
        s.setProfiling(True)
        with Clocks(dev) as clk, torch.cuda.stream(stream):
            for k in range(K):
                candidate(st)
                v0, hc0 = st["v"].clone(), st["hc"].clone()
                outs = {}
                for mode in ((0, 1) if k % 2 == 0 else (1, 0)):
                    st["v"].copy_(v0)
                    st["hc"].copy_(hc0)
                    s.setMode(mode)
                    flush.fill_(float(k))
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    s.resolveCollisionBatchDevice(st["x"], st["xc"], st["v"], st["hc"], st["xo"])
                    e1.record(stream)
                    stream.synchronize()
                    ms[mode] += e0.elapsed_time(e1)
                    outs[mode] = (st["xo"].clone(), st["v"].clone(), st["hc"].clone())
                    if mode == 1:
                        counters.append(s.counters())
                same &= all(bool(torch.equal(a, b)) for a, b in zip(outs[0], outs[1]))
                st["xo"].copy_(outs[1][0])
                st["v"].copy_(outs[1][1])
                st["hc"].copy_(outs[1][2])
                st["x"], st["xo"] = st["xo"], st["x"]
            stream.synchronize()
        prof = s.profile()
        kprof = None
        if args.kernel_steps > 0:
            # untimed, after the timed steps: mixed-precision steps with every
            # pass's stages timed inside the loop graph too
            s.setMode(1)
            s.setProfiling(2)
            with torch.cuda.stream(stream):
                for _ in range(args.kernel_steps):
                    candidate(st)
                    s.resolveCollisionBatchDevice(st["x"], st["xc"], st["v"], st["hc"], st["xo"])
                    st["x"], st["xo"] = st["xo"], st["x"]
                stream.synchronize()
            kprof = {k: round(v[0] / args.kernel_steps, 3) for k, v in s.profile().items() if v[0]}
        s.close()
        tree_us += sum(c["tree_build_us"] for c in counters)
        return dict(mixed_ms=max_over_ranks(ms[1]), plain_ms=max_over_ranks(ms[0]), same=same, tuned=tuned,
                    counters=counters, prof=prof, clocks=clk.summary(), tree_s=tree_us / 1e6, kprof=kprof)

    # ------------------------------------- CPU baseline (rank 0, first)
    # The oracle steps the CPU sample of the scenes from the initial state
    # over the first W + K steps (or its time budget); the GPU batch's state
    # of those scenes after as many steps is compared with its result.
    cpu = None
    if rk == 0 and not args.no_cpu_baseline and nsc > 1:
        threads = os.cpu_count() or 1
        idx = cpu_sample(scs)
        sub = [scs[i] for i in idx]
        rate, n, t, steps, final = oracle_rate(sub, W + K, args.cpu_budget, threads, args.zone_cap)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port", "steps": steps, "idx": idx,
               "final": final,
               "sample": f"{args.workload}: {len(sub)} of {nsc} scenes"
                         f"{' (every fourth by size)' if len(sub) < nsc else ''}, first {steps} steps of the "
                         f"trajectory ({n} scene-steps, {t:.1f} s), one scene per thread"}
        cpu["one_core"] = one_core_rate(scs, steps, args.cpu_budget, args.zone_cap)

    arms = set(args.arms.split(","))
    if nsc == 1 and "plain" in arms:
        pair = single_scene_pair()
        tot = {k: sum(c[k] for c in pair["counters"]) for k in pair["counters"][0]}
        if rk == 0:
            value = ws * K / (pair["mixed_ms"] / 1e3)
            plain_value = ws * K / (pair["plain_ms"] / 1e3)
            line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": W,
                    "ms_per_step": pair["mixed_ms"] / K, "higher_is_better": True, "scaling": "weak",
                    "vs_baseline": None, "dtype": "f64 (f32 filters)", "data": "synthetic",
                    "config": dict(describe(args.workload, scs, args.placement), l2="flushed before every timed step",
                                   path="one scene: mixed precision and plain FP64 on the same inputs"),
                    "plain_fp64": {"value": plain_value, "ms_per_step": pair["plain_ms"] / K,
                                   "state_equal_every_step": pair["same"]},
                    "speedup_vs_plain": value / plain_value, "autotune": pair["tuned"],
                    "approach_steps": args.approach,
                    "tree_build_s": pair["tree_s"], "tree_builds_per_timed_step": tot["tree_builds"] / K,
                    "zone_cap": args.zone_cap, "clocks": pair["clocks"], "counters": tot,
                    "stages_ms": {k: round(v[0], 3) for k, v in pair["prof"].items()},
                    "stages_ms_per_mixed_step": pair["kprof"]}
            print(json.dumps(line), flush=True)
        if ws > 1:
            torch.distributed.destroy_process_group()
        return
    mixed = batched_run(1, check=not args.no_check)
    batch_plain = batched_run(0, check=False) if "batch_plain" in arms else None
    plain = plain_sequential() if "plain" in arms else None
    e2e_ms = e2e_run() if "e2e" in arms else None
    nv = len(x0)
    h2d = nv * (3 * 8 * 3 + 1)   # x_old, x_cand, vel, has_collsn
    d2h = nv * (3 * 8 * 2 + 1) + 4 * nsc  # x_out, vel, has_collsn, has_collision

    if rk != 0:
        if ws > 1:
            torch.distributed.destroy_process_group()
        return

    value = ws * mixed["scene_steps"] / (mixed["total_ms"] / 1e3)
    plain_value = ws * plain["scene_steps"] / (plain["ms"] / 1e3) if plain else None
    batch_plain_value = ws * batch_plain["scene_steps"] / (batch_plain["total_ms"] / 1e3) if batch_plain else None
    e2e_value = ws * mixed["scene_steps"] / (e2e_ms / 1e3) if e2e_ms else None

    # ----------------------------------------------------------- roofline
    peaks = json.load(open(PEAKS)) if os.path.exists(PEAKS) else {}
    hbm = peaks.get("hbm_gbs")
    peak_src = "measured" if hbm else "fallback"
    hbm = hbm or 6800.0
    tot = {k: sum(c[k] for c in mixed["counters"]) for k in mixed["counters"][0]}
    prof = mixed["prof"]
    kern = {}
    ms, calls = prof.get("traverse", (0.0, 0))
    if calls and tot.get("timed_traverse_leaves"):
        # the traversals the "traverse" stage times (the proximity pass's,
        # launched from the host): one read of the hierarchy's FP32 boxes,
        # (2n-1)*24 B for n leaves, and the 8-byte pairs written
        per = (48.0 * tot["timed_traverse_leaves"] + 8.0 * tot["timed_traverse_pairs"]) / calls
        kern["traverse"] = {"kernel": TRAVERSE_KERNEL[mixed["rope"]], "bytes_per_launch": per,
                            "ms_per_launch": ms / calls, "achieved": per / (ms / calls / 1e3) / 1e9,
                            "leaves_per_launch": tot["timed_traverse_leaves"] / calls}
    ms, calls = prof.get("strain", (0.0, 0))
    if calls:
        per = tot["strain_bytes"] / calls
        kern["strain"] = {"kernel": "strain stage: k_strain_setup, k_strain_check and k_strain_window sweeps "
                          "(one CTA per scene), one launch = one step's tail graph", "bytes_per_launch": per,
                          "ms_per_launch": ms / calls, "achieved": per / (ms / calls / 1e3) / 1e9}
    kp = mixed["kprof"]
    if kp:
        # the untimed steps after the timed ones, every stage of every pass
        # timed (inside the loop graph by global-timer boundary kernels)
        kc, kpr = kp["counters"], kp["prof"]
        t_sub = (kpr.get("loop_subtests", (0.0, 0))[0] + kpr.get("ccd_subtests", (0.0, 0))[0]) / 1e3
        if t_sub > 0 and kc.get("fp64_subtests"):
            flops = SUBTEST_FP64_FLOPS * kc["fp64_subtests"]
            kern["ccd_subtests"] = {
                "kernel": "k_subtests_all (the FP64 sub-tests that pass the FP32 filters, both kinds in one launch)",
                "bound": "fp64",
                "flops": flops, "s": t_sub, "achieved_tflops": flops / t_sub / 1e12, "peak_tflops": FP64_PEAK_TFLOPS,
                "frac": flops / t_sub / 1e12 / FP64_PEAK_TFLOPS, "peak_source": "nominal",
                "flops_per_subtest": SUBTEST_FP64_FLOPS, "cr_roots": kc.get("cr_roots"),
                "note": "FP64 pipe 77% busy in the ncu capture: most FP64 issue slots are compares, selects and "
                        "conversions, run at the FP64 rate"}
        t_f = kpr.get("loop_filter", (0.0, 0))[0] / 1e3
        if t_f > 0 and kc.get("moving_visits"):
            b = FILTER_BYTES_PER_VISIT * kc["moving_visits"]
            kern["ccd_filter"] = {"kernel": "k_narrow_filter<1> (FP32 per-pair filters of the CCD passes)",
                                  "bytes": b, "s": t_f, "achieved": b / t_f / 1e9}
    roof = None
    if "traverse" in kern:
        # the traversal is the largest kernel the timed region times per
        # launch with CUDA events (inside the loop graph, only the untimed
        # profiled steps split the stages; their shares are printed as
        # stages_ms_per_step_after)
        kt = kern["traverse"]
        traffic = TRAVERSE_DRAM_BYTES_PER_LEAF[mixed["rope"]] * kt["leaves_per_launch"]
        roof = {"bound": "hbm", "kernel": kt["kernel"], "achieved": kt["achieved"], "peak": hbm, "unit": "GB/s",
                "frac": kt["achieved"] / hbm, "peak_source": peak_src, "traffic": traffic,
                "note": f"latency and divergence bound ({TRAVERSE_LANES_ACTIVE[mixed['rope']]} of 32 lanes active "
                        "per instruction, dependent node loads), not bandwidth bound; traffic = the ncu capture's "
                        "DRAM bytes per query leaf x this launch's leaves", "kernels": kern}
    if roof is not None and tot.get("path_bytes"):
        # the whole step's algorithmic bytes (the path_bytes counter: state in
        # and out, per pass the points, connectivity, hierarchy, pairs and
        # contact records, per strain pass the points and edges) over the
        # timed steps' device time
        achieved = tot["path_bytes"] / (mixed["total_ms"] / 1e3) / 1e9
        roof["path"] = {"bytes_per_scene_step": tot["path_bytes"] / max(mixed["scene_steps"], 1),
                        "achieved": achieved, "frac": achieved / hbm, "unit": "GB/s"}
    parity = None
    if cpu is not None:
        # the oracle's state of each sampled scene against the GPU batch's
        if mixed["cpu_snap"] is None:
            parity = {"equal": None, "note": "no GPU state after the CPU leg's steps (run with the CCD check)"}
        else:
            gx, gv, ghc, gen = mixed["cpu_snap"]
            ndiff, nlive, max_abs, max_rel, capped_mismatch = 0, 0, 0.0, 0.0, 0
            differing = []
            ref_missed = sum(f[4] for f in cpu["final"])
            gpu_missed = None if mixed["cpu_missed"] is None else int(sum(mixed["cpu_missed"][i] for i in cpu["idx"]))
            for j, i in enumerate(cpu["idx"]):
                ox, ov, ohc, olive, _ = cpu["final"][j]
                if not olive or not gen[i]:
                    capped_mismatch += int(olive != bool(gen[i]))
                    continue
                nlive += 1
                a, b = int(offs[i]), int(offs[i + 1])
                eq = (np.array_equal(gx[a:b], ox) and np.array_equal(gv[a:b], ov) and
                      np.array_equal(ghc[a:b], ohc))
                if not eq:
                    ndiff += 1
                    differing.append(i)
                    for g_, o_ in ((gx[a:b], ox), (gv[a:b], ov)):
                        d = np.abs(g_ - o_)
                        max_abs = max(max_abs, float(d.max()))
                        max_rel = max(max_rel, float((d / np.maximum(np.abs(o_), 1e-6)).max()))
            # a differing scene stepped again by the oracle built with
            # correctly rounded acos/cos/sin/pow: equal to the GPU, the
            # difference is glibc's rounding
            explained = 0
            for i in differing:
                a, b = int(offs[i]), int(offs[i + 1])
                cx, cv, chc = oracle_replay(scs[i], cpu["steps"], args.zone_cap, crmath=True)
                explained += int(np.array_equal(gx[a:b], cx) and np.array_equal(gv[a:b], cv) and
                                 np.array_equal(ghc[a:b], chc))
            parity = {"equal": ndiff == 0 and capped_mismatch == 0, "scenes": nlive, "scenes_differing": ndiff,
                      "differing_equal_to_crmath_oracle": explained,
                      "capped_mismatch": capped_mismatch, "steps": cpu["steps"], "max_abs": max_abs,
                      "max_rel": max_rel,
                      "missed_ccd_last_step": {"oracle": ref_missed, "gpu": gpu_missed,
                                               "what": "pairs the exact CCD re-check finds after the last of those "
                                                       "steps on these scenes, on the oracle's and the GPU's states"},
                      "what": "positions, velocities and has_collsn of the CPU sample's scenes after the CPU "
                              "leg's steps, GPU batch (mixed precision) vs the oracle, bit for bit"}
        for k in ("idx", "final", "steps"):
            cpu.pop(k)
    launches = sum(c["kernel_launches"] + 2 for c in mixed["counters"])
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": W,
            "ms_per_step": mixed["total_ms"] / K, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64 (f32 filters)", "data": "synthetic",
            "config": dict(describe(args.workload, scs, args.placement),
                           path="mixed precision, batched: FP32 sub-test filters in front of unchanged FP64 "
                                "tests, all scenes per launch",
                           l2="flushed before every timed step",
                           parallelism="replicas" if ws > 1 else "single"),
            "plain_fp64": None if not plain else {
                "value": plain_value, "steps": n_plain, "ms_per_step": plain["ms"] / n_plain,
                "path": "plain FP64, one scene per call", "gpu_launches": plain["launches"],
                "state_equal_after_steps": plain["same"], "max_abs_diff": plain["diff"]},
            "speedup_vs_plain": value / plain_value if plain else None,
            "batched_plain_fp64": None if not batch_plain else {
                "value": batch_plain_value, "ms_per_step": batch_plain["total_ms"] / K},
            "missed_ccd": None if args.no_check else int(mixed["missed"]),
            "capped_scenes": mixed["capped"], "zone_cap": args.zone_cap,
            "autotune": mixed["tuned"],
            "roofline": roof, "cpu_baseline": cpu, "parity_vs_cpu": parity, "clocks": mixed["clocks"],
            "e2e": None if e2e_value is None else
                   {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": int(launches),
            "step_ms_quantiles": [round(float(q), 3) for q in np.quantile(mixed["step_ms"], [0, .25, .5, .75, 1])],
            "counters": tot, "stages_ms": {k: round(v[0], 3) for k, v in prof.items()}}
    if mixed["kprof"]:
        kp = mixed["kprof"]
        line["stages_ms_per_step_after"] = {
            "steps": kp["steps"], "what": "untimed steps after the timed ones, every pass's stages timed "
                                          "(inside the loop graph by global-timer boundary kernels)",
            "ms": {k: round(v[0] / kp["steps"], 3) for k, v in kp["prof"].items() if v[0]}}
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="batched",
                    choices=["batched", "folded_cloth", "cloth_on_sphere", "strings", "large"])
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--plain-steps", type=int, default=5,
                    help="timed steps of the one-scene-at-a-time run (0: all K)")
    ap.add_argument("--zone-cap", type=int, default=1000)
    ap.add_argument("--arms", default="mixed,batch_plain,plain,e2e",
                    help="arms to run besides the headline batched mixed one (for profiling runs)")
    ap.add_argument("--scenes", type=int, default=0, help="first N scenes of the batched workload (0: all)")
    ap.add_argument("--placement", default="contact", choices=["contact", "freefall"],
                    help="batched workload: cloths within four steps of their obstacles (contact) or 0.05/0.10 "
                         "above them (freefall)")
    ap.add_argument("--large-n", type=int, default=1025, help="cloth vertices per side of the large workload")
    ap.add_argument("--approach", type=int, default=0,
                    help="one-scene workloads: untimed steps of the trajectory before the warm-up (to reach contact)")
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--ref-budget", type=float, default=120.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-check", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--kernel-steps", type=int, default=2,
                    help="untimed steps after the timed ones with every pass's stages timed (roofline.kernels)")
    ap.add_argument("--tune", action="append", default=[], metavar="KNOB=VALUE",
                    help="set a tuning knob on every solver, e.g. STRAIN_BLOCK=128 (names: CollisionSolver3d.TUNE_*)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
