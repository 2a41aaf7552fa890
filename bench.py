"""Benchmark of the AVBD world step on GB300.

Workload (one "step" = one AVBD world step of the whole scene): the dense
pile - a square pyramid of 53 layers (layer k is a k x k grid of 1 m cubes,
51,039 cubes, 1% gap, 1000 kg/m^3, mu 0.6) on the ground, with a 2 m-radius
sphere (5000 kg/m^3) dropped onto the apex at 10 m/s; dt = 1/60 s,
10 iterations, gravity -9.81, 600 steps. Synthetic scene, seeded and
deterministic.

Timing: W warm-up steps, then the scene is packed again and exactly K steps
are timed from its initial state (K = 600 by default: the whole run, from
the standing pyramid to the crushed pile). Each step's device time comes from
CUDA events recorded by the library on its own stream around the whole step;
L2 is flushed (a 256 MB write) between steps, outside those events.
The JSON line also carries the roofline of the dominant kernel (algorithmic
bytes from each step's own pair/manifold/contact counts), the f64 CPU
baseline (the oracle, 1 thread, single steps from states sampled along the
same trajectory), the end-to-end rate through the C ABI with host buffers
(state upload + step + state readback every step, over the same K steps), the
kernel launch count and the SM clocks sampled during the timed region.

`--impl reference` times the reference's CPU algorithm on the host cores
(the oracle restatement: the reference engine is JavaScript and no
JavaScript runtime exists here), on the same workload and metric.
Multi-GPU: the step does not shard (replicas only): each rank runs its own
replica and `value` sums their step rates over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "AVBD steps/s at 51k boxes vs f64 CPU ref; batched & adjoint steps/s at tol"
UNIT = "steps/s"
def workload(layers):
    cubes = layers * (layers + 1) * (2 * layers + 1) // 6
    return (f"pyramid: {layers} layers = {cubes:,} 1 m cubes (1% gap, 1000 kg/m^3, mu 0.6) + ground + r=2 m sphere "
            "(5000 kg/m^3, 10 m/s onto the apex); dt=1/60, 10 iterations, gravity -9.81")


def pkg():
    return importlib.import_module("avbd-sandbox_gb300")


def make_scene(layers):
    sc = pkg().scene
    return sc.pyramid(layers=layers)


def params_for(abi, s, **kw):
    kw.setdefault("body_order", abi.ORDER_PRIORITY)
    return abi.default_params(**s.params, **kw)


def slowest_rank(seconds: float, ws: int, device: str = "cuda") -> float:
    """Replicas only: every rank steps its own copy of the workload, and the
    job's time is the slowest rank's (all_reduce MAX; no collective when ws = 1)."""
    if ws <= 1:
        return seconds
    import torch

    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_rate(steps: int, ws: int, slowest_seconds: float) -> float:
    """Whole-job steps/s: all ranks' steps over the slowest rank's time (weak scaling)."""
    return ws * steps / slowest_seconds


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# ---------------------------------------------------------------------------
# CPU baseline: the f64 oracle, one thread, a bounded sample of the workload
# ---------------------------------------------------------------------------
def cpu_baseline(params, snapshots, budget_s=45.0, window=""):
    """Time the oracle (1 thread) on single steps taken from states of the
    timed window (`snapshots`: (step index, world with warm-start manifolds)),
    in the given order until the budget is spent (at least five when there are
    five). `value` is 1 / the median step time; the mean is reported beside it
    (the window's mean rate is the mean's reciprocal)."""
    from oracle import Oracle

    times, used = [], []
    t_all = time.perf_counter()
    for step_idx, snap in snapshots:
        if len(times) >= 5 and time.perf_counter() - t_all > budget_s:
            break
        o = Oracle(params, snap)
        t0 = time.perf_counter()
        o.step(1)
        times.append(time.perf_counter() - t0)
        used.append(step_idx)
        del o
    med = statistics.median(times)
    mean = sum(times) / len(times)
    return {
        "value": 1.0 / med,
        "unit": UNIT,
        "cores": 1,
        "kind": "port",
        "sample": f"one single-thread f64 step of the oracle from each of the states before steps "
                  f"{sorted(s + 1 for s in used)} of {window} (loaded with their warm-start manifolds); "
                  f"median of {len(times)} steps ({sum(times):.1f} s of CPU work)",
        "ms_per_step_median": med * 1e3,
        "ms_per_step_mean": mean * 1e3,
        "value_from_mean": 1.0 / mean,
        "sampled_ms": [round(t * 1e3, 1) for t in times],
    }


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.proc = None
        self.gpu = gpu_index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for k, name in enumerate(names):
                if f[5 + k].lower() in ("active", "1"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# roofline of the dominant kernel: algorithmic bytes per launch
# ---------------------------------------------------------------------------
def algorithmic_bytes(kind, st, n_dyn, iterations, n_joints=0, n_springs=0):
    """Bytes a launch must move at minimum, from the step's own counts.

    solve (per iteration): each dynamic body reads its state, inertial target,
    mass and moments (72 B) and writes p, q (28 B); each manifold side reads the
    basis and the other body's state (92 B), each contact side reads rA, rB,
    C0, k, lambda (60 B); the dual reads basis + both bodies (148 B) per
    manifold and 60 B, writes 28 B per contact; joints and springs likewise.
    narrowphase: per candidate pair both bodies' pose and size (2 x 56 B) + the
    pair key and previous index (8 B) + the previous manifold header (84 B);
    per live manifold its key, count and basis (132 B written); per contact
    the old record read (60 B) and the new one written (80 B)."""
    N_m, N_c, N_p = st["manifolds"], st["contacts"], st["candidate_pairs"]
    if kind == "solve":
        per_iter = (n_dyn * 100 + N_m * (2 * 92 + 148) + N_c * (2 * 60 + 88) + n_joints * (160 + 2 * 56)
                    + n_springs * (48 + 2 * 56))
        return iterations * per_iter
    if kind == "narrowphase":
        return N_p * 204 + N_m * 132 + N_c * 140
    return None


def read_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def read_traffic(key, units_per_launch):
    """DRAM bytes per launch: the per-unit traffic of a committed ncu capture
    of the same kernel in the same regime (profiles/traffic.json, keyed
    "kernel@regime"), scaled to this run's units per launch; None when no
    capture of that regime is committed."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            d = json.load(f)[key]
        return d["dram_bytes"] / d["units"] * units_per_launch
    except Exception:
        return None


def bench_config(args, n_bodies, ws):
    """The workload description both arms print (the same dict)."""
    return {"workload": workload(args.layers), "bodies": n_bodies,
            "timed_steps": f"steps 1..{args.steps} of the run from its initial state, after {args.warmup} "
                           "untimed warm-up steps",
            "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU",
            "l2": "device timing: L2 flushed between steps (256 MB write), outside the timed step events"}


PHASES = ("broadphase_ms", "narrowphase_ms", "prepare_ms", "coloring_ms", "solve_ms")


def timed_window(gpu, K, flush, n_dyn, iterations, trace=None):
    """K steps from the packed state, each timed by the library's CUDA events
    around the whole step (profiling on), L2 flushed before each step outside
    those events. Returns the per-step times and the window's counters."""
    import torch

    gpu.set_profiling(True)
    rec = {"step_ms": [], "phases": {k: 0.0 for k in PHASES}, "algo": {"solve": 0.0, "narrowphase": 0.0},
           "work": {k: 0 for k in ("candidate_pairs", "manifolds", "contacts", "np_face", "np_edge", "np_exact",
                                   "lanes_per_body", "colors")},
           "peak": {k: 0 for k in ("candidate_pairs", "manifolds", "contacts", "colors", "fp64_bodies")}}
    launches0 = gpu.kernel_launches
    for _ in range(K):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        gpu.step(1)
        p = gpu.last_profile
        rec["step_ms"].append(p["step_ms"])
        for k in PHASES:
            rec["phases"][k] += p[k]
        for kind in rec["algo"]:
            rec["algo"][kind] += algorithmic_bytes(kind, p, n_dyn, iterations)
        for k in rec["work"]:
            rec["work"][k] += p[k]
        for k in rec["peak"]:
            rec["peak"][k] = max(rec["peak"][k], p[k])
        if trace:
            t = dict(p, step=len(rec["step_ms"]))
            for kind in rec["algo"]:
                t[f"algorithmic_bytes_{kind}"] = algorithmic_bytes(kind, p, n_dyn, iterations)
            trace.write(json.dumps(t) + "\n")
    gpu.idle()
    rec["launches"] = gpu.kernel_launches - launches0
    gpu.set_profiling(False)
    return rec


def e2e_window(gpu, start, K, snap_at=()):
    """The same K steps end to end through the C ABI with host buffers: every
    step uploads the state from host f64 arrays (avbd_write_state), steps and
    reads the state back (avbd_read_state). States after the steps in
    `snap_at` are captured with their manifolds, outside the clock."""
    gpu.pack(start)
    host = gpu.read_state()
    e2e_s, snaps = 0.0, []
    for i in range(K):
        t1 = time.perf_counter()
        gpu.write_state(host)
        gpu.step(1)
        gpu.sync_to_cpu(host)
        e2e_s += time.perf_counter() - t1
        if i in snap_at:  # the state after step i + 1 = the state before step i + 2
            snaps.append((i + 1, gpu.read_state(manifolds=True)))
    return e2e_s, snaps


def roofline(rec, K, regime):
    """Roofline of the window's dominant kernel: algorithmic bytes per launch
    (its step's own counts) over its mean launch time, against the measured
    HBM copy bandwidth."""
    phases = {k: v / K for k, v in rec["phases"].items()}
    kinds = {"solve_ms": ("solve", "solve_kernel"), "narrowphase_ms": ("narrowphase", "narrowphase_kernels")}
    dom = max(kinds, key=lambda k: phases[k])
    kind, kname = kinds[dom]
    algo = rec["algo"][kind] / K
    peak, peak_src = read_peaks()
    achieved = algo / (phases[dom] / 1e3) / 1e9
    other_k = "narrowphase_ms" if dom == "solve_ms" else "solve_ms"
    other_kind, other_name = kinds[other_k]
    oach = rec["algo"][other_kind] / K / (phases[other_k] / 1e3) / 1e9
    return {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_src,
            "traffic": read_traffic(f"{kname}@{regime}", algo),
            "algorithmic_bytes_per_launch": algo, "launch_ms": phases[dom],
            "other": {"kernel": other_name, "achieved": oach, "frac": oach / peak, "launch_ms": phases[other_k]}}


def run_gpu(args):
    import torch

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    abi = pkg().abi
    backend = importlib.import_module("avbd-sandbox_gb300.backend")
    s = make_scene(args.layers)
    params = params_for(abi, s)  # direct launches: the per-phase events (phases, roofline)
    world = s.world()
    # the headline: every step replayed as one CUDA graph (the same kernels)
    gpu = backend.GpuBackend(params_for(abi, s, graph=1))
    gpu.pack(world)
    n_dyn = int((world.mass > 0).sum())
    n = world.n_bodies
    K = args.steps
    per_body = 8 * 16  # the caller's f64 arrays: position 3, quaternion 4, velocity, angular and previous velocity 3

    gpu.step(args.warmup)
    gpu.idle()
    gpu.pack(world)  # back to the initial state: the timed steps are steps 1..K of the run
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    with ClockSampler(local) as clk:
        rec = timed_window(gpu, K, flush, n_dyn, params.iterations)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    dev_s = slowest_rank(sum(rec["step_ms"]) / 1e3, ws)
    # the same steps launched directly, for the split by phase and the roofline
    direct = backend.GpuBackend(params)
    direct.pack(world)
    direct.step(args.warmup)
    direct.idle()
    direct.pack(world)
    trace = open(args.trace, "w") if args.trace and rank == 0 else None
    prec = timed_window(direct, K, flush, n_dyn, params.iterations, trace)
    if trace:
        trace.close()
    direct.destroy()

    # end to end over the same K steps; states for the CPU baseline on the way
    cpu = rank == 0 and not args.no_cpu_baseline
    snap_at = sorted({int(round(k * (K - 1) / 5.0)) - 1 for k in range(6)} - {-1}) if cpu else []
    e2e_s, snapshots = e2e_window(gpu, world, K, snap_at)
    if cpu:  # the state before step 1 is the initial state itself
        snapshots = [(0, world)] + snapshots
    e2e_s = slowest_rank(e2e_s, ws)

    value = replica_rate(K, ws, dev_s)
    clocks = clk.summary()
    out = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": ws,
        "steps": K,
        "warmup": args.warmup,
        "ms_per_step": dev_s * 1e3 / K,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 (f64 narrowphase geometry, f64 positions and joint multipliers)",
        "data": "synthetic",
        "config": bench_config(args, n, ws),
        "roofline": roofline(prec, K, "sparse" if K <= 60 else "run"),
        "e2e": {"value": replica_rate(K, ws, e2e_s), "unit": UNIT, "h2d_bytes_per_step": n * per_body,
                "d2h_bytes_per_step": n * per_body,
                "how": "avbd_write_state + avbd_step(1) + avbd_read_state every step over the same steps: the "
                       "caller's f64 arrays copied to and from the device as they are, converted there"},
        "step_launch": "each timed step one CUDA graph (params.graph = 1); phases_ms and the roofline from the "
                       "same steps launched directly, with events between the phases",
        "gpu_launches": rec["launches"],
        "clocks": clocks,
        "phases_ms": {k: v / K for k, v in prec["phases"].items()},
        "phases_total_ms": sum(prec["step_ms"]) / K,
        "wall_s": wall,
        "mean_work_per_step": {k: v / K for k, v in rec["work"].items()},
        "peak_work": rec["peak"],
    }
    if rank == 0 and snapshots:
        ref_params = params_for(abi, s, body_order=abi.ORDER_REFERENCE)
        out["cpu_baseline"] = cpu_baseline(ref_params, snapshots, budget_s=args.cpu_budget,
                                           window=f"the timed steps 1..{K}")
    if args.dense_steps > 0:
        out["dense"] = run_dense(abi, backend, args, s, world, params, flush, n_dyn, ws, rank)
    if args.batched_steps > 0:
        out["batched"] = run_batched(abi, backend, args, flush)
    if rank == 0 and args.adjoint_steps > 0:
        out["adjoint"] = run_adjoint(abi, backend, args)
    if rank == 0 and not args.no_accuracy:
        out["accuracy_vs_oracle"] = run_accuracy(abi, backend)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def run_dense(abi, backend, args, s, world, params, flush, n_dyn, ws, rank):
    """The crushed pile: the run advanced on the device to step D (the state
    after step D, warm-start manifolds included, kept on the host), then
    steps D+1..D+K timed from it like the main window, end to end through the
    C ABI, and the oracle (1 thread) stepped from states of the same window."""
    D, K = args.dense_start, args.dense_steps
    gpu = backend.GpuBackend(params)
    gpu.pack(world)
    gpu.step(D)
    gpu.idle()
    start = gpu.read_state(manifolds=True)
    gpu.pack(start)
    gpu.step(args.warmup)
    gpu.idle()
    gpu.pack(start)
    rec = timed_window(gpu, K, flush, n_dyn, params.iterations)
    dev_s = slowest_rank(sum(rec["step_ms"]) / 1e3, ws)
    cpu = rank == 0 and not args.no_cpu_baseline
    snap_at = sorted({int(round(k * (K - 1) / 5.0)) - 1 for k in range(6)} - {-1}) if cpu else []
    e2e_s, snaps = e2e_window(gpu, start, K, snap_at)
    e2e_s = slowest_rank(e2e_s, ws)
    per_body = 8 * 16  # the caller's f64 body arrays, each way
    out = {"value": replica_rate(K, ws, dev_s), "unit": UNIT, "steps": K, "start_step": D,
           "ms_per_step": dev_s * 1e3 / K,
           "timed_steps": f"steps {D + 1}..{D + K} of the run (the state after step {D} reached on the device "
                          f"and loaded with its warm-start manifolds), after {args.warmup} untimed warm-up steps "
                          "from the same state",
           "e2e": {"value": replica_rate(K, ws, e2e_s), "unit": UNIT, "h2d_bytes_per_step": world.n_bodies * per_body,
                   "d2h_bytes_per_step": world.n_bodies * per_body},
           "roofline": roofline(rec, K, "dense"),
           "gpu_launches": rec["launches"],
           "phases_ms": {k: v / K for k, v in rec["phases"].items()},
           "mean_work_per_step": {k: v / K for k, v in rec["work"].items()}, "peak_work": rec["peak"]}
    if cpu:
        ref_params = params_for(abi, s, body_order=abi.ORDER_REFERENCE)
        cb = cpu_baseline(ref_params, [(0, start)] + snaps, budget_s=args.cpu_budget,
                          window=f"the timed steps {D + 1}..{D + K} (numbered from {D})")
        out["cpu_baseline"] = cb
        out["vs_cpu_baseline"] = out["value"] / cb["value"]
        out["e2e_vs_cpu_baseline"] = out["e2e"]["value"] / cb["value"]
    gpu.destroy()
    return out


def run_batched(abi, backend, args, flush):
    """The batched workload: 512 independent random box piles (body counts
    log-uniform in [64, 8192], edges U[0.3, 2] m, densities log-uniform
    [100, 1e4] kg/m^3, mu U[0.2, 0.9], contact-free column drop), all in one
    context: every phase of a step is one launch over all scenes. Steps 1..K,
    timed like the main workload (per-step device events on the library's
    stream, L2 flushed between steps), in three configurations: the default
    launches; each step replayed as a CUDA graph; and the graph with the
    launch configuration avbd_autotune picked on the run's state after
    K/2 steps. Accuracy: after the tuned run, one more step of the batch
    against the oracle's step of each of a sample of scenes from the same
    state."""
    import torch
    from oracle import Oracle

    sc = pkg().scene
    parts = sc.pile_batch()
    batch = sc.batch_worlds([p.world() for p in parts])
    base = dict(gravity=-9.81, iterations=10, body_order=abi.ORDER_PRIORITY)
    K = args.batched_steps
    n_scenes = len(parts)

    def timed(params):
        gpu = backend.GpuBackend(params)
        gpu.pack(batch)
        gpu.step(args.warmup)
        gpu.idle()
        gpu.pack(batch)
        gpu.set_profiling(True)
        ms, contacts, lanes, graphs = 0.0, 0, 0, 0
        for _ in range(K):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            gpu.step(1)
            p = gpu.last_profile
            ms += p["step_ms"]
            contacts += p["contacts"]
            lanes += p["lanes_per_body"]
            graphs += p["via_graph"]
        gpu.set_profiling(False)
        rec = {"value": n_scenes * K / (ms / 1e3), "unit": "scene-steps/s", "ms_per_step": ms / K,
               "graph_steps": graphs, "mean_contacts": contacts / K, "mean_lanes_per_body": lanes / K}
        return gpu, rec

    out = {"scenes": n_scenes, "bodies": batch.n_bodies, "steps": K,
           "workload": f"{n_scenes} random box piles ({batch.n_bodies:,} bodies) in one context, steps 1..{K}"}
    gpu, out["default"] = timed(abi.default_params(**base))
    gpu.destroy()
    gpu, out["graph"] = timed(abi.default_params(**base, graph=1))
    gpu.destroy()
    # tune on the run's own state half way through
    gpu = backend.GpuBackend(abi.default_params(**base, graph=1))
    gpu.pack(batch)
    gpu.step(K // 2)
    gpu.idle()
    tune = gpu.autotune(3)
    gpu.destroy()
    tuned = abi.default_params(**base, graph=1, schedule=tune["schedule"], lanes_per_body=tune["lanes_per_body"],
                               tail_div=tune["tail_div"], blocks_per_sm=tune["blocks_per_sm"])
    gpu, out["tuned_graph"] = timed(tuned)
    out["autotune"] = dict(tune, tuned_at_step=K // 2)
    best = max(("default", "graph", "tuned_graph"), key=lambda k: out[k]["value"])
    out["value"], out["unit"], out["ms_per_step"], out["best"] = (out[best]["value"], "scene-steps/s",
                                                                   out[best]["ms_per_step"], best)
    # accuracy: every 32nd scene against its own oracle, one step from the state after step K
    state = gpu.read_state(manifolds=True).round_to_device()
    gpu.destroy()
    gpu = backend.GpuBackend(tuned)
    gpu.pack(state)
    gpu.step(1)
    gpu.idle()
    got = gpu.read_state(manifolds=True)
    gpu.destroy()
    worst, same_topo, sample = 0.0, True, list(range(0, n_scenes, 32))
    for k in sample:
        ref = Oracle(tuned, state.scene(k))
        ref.step(1)
        want, g = ref.state(), got.scene(k)
        dyn = want.mass > 0
        worst = max(worst, float(np.abs(g.pos[dyn] - want.pos[dyn]).max()))
        same_topo = same_topo and g.manifold_dict() == want.manifold_dict()
    out["accuracy_vs_oracle"] = {"scenes": sample, "from_step": K, "max_pos_error_m": worst,
                                 "manifolds_identical": same_topo, "tolerance_m": 1e-5}
    return out


def run_adjoint(abi, backend, args):
    """The differentiable wall: 16 x 16 bricks of 0.5 x 0.25 x 0.25 m (hard
    bonds) struck by a 50 kg sphere; the gradient of the mean brick
    displacement after S steps with respect to the sphere's initial velocity
    (3), the bricks' friction and the penalty cap (5 directions).

    adjoint: avbd_adjoint_forward over S steps (every step carries the five
    derivatives) + avbd_adjoint_read + avbd_adjoint_backward, timed on the
    host around the C ABI calls (pack, steps, readback of positions,
    derivatives and gradient included), median of R runs after one warm-up.
    plain: the same scene's FP32 step over the same S steps (device time,
    CUDA events). CPU: the oracle and the tangent oracle over the same steps,
    1 thread. Accuracy: at 30 steps (the horizon where the oracle's central
    differences converge) the device gradient against the tangent oracle's
    exact gradient, and along the sphere's y velocity against the
    differences."""
    import torch
    from oracle import Oracle, TangentOracle

    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import c5_gradients as c5

    sc = pkg().scene
    S, R = args.adjoint_steps, 3
    th = c5.theta0(abi)
    s = sc.brick_wall_c5()
    w = s.world()
    params = c5.params_of(abi, s, th, abi.ORDER_PRIORITY)
    seeds = c5.seeds(abi, s, w)
    gpu = backend.GpuBackend(params)
    times = []
    for r in range(R + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        gpu.adjoint_forward(w, S, seeds)
        pos, tan, _ = gpu.adjoint_read()
        grad = gpu.adjoint_backward(c5.upstream(s, w, pos))
        t = time.perf_counter() - t0
        if r:
            times.append(t)
    adj_s = statistics.median(times)
    # the plain FP32 step of the same scene, same steps
    plain = backend.GpuBackend(params)
    plain.pack(w)
    plain.step(3)
    plain.idle()
    plain.pack(w)
    plain.set_profiling(True)
    ms = 0.0
    for _ in range(S):
        plain.step(1)
        ms += plain.last_profile["step_ms"]
    plain.set_profiling(False)
    plain.destroy()
    # CPU: the oracle and the tangent oracle, same steps
    t0 = time.perf_counter()
    Oracle(params, w).step(S)
    cpu_plain = time.perf_counter() - t0
    o = TangentOracle(params, w)
    for sd in seeds:
        o.seed(*sd)
    t0 = time.perf_counter()
    o.step(S)
    cpu_tan = time.perf_counter() - t0
    # accuracy at the differences' horizon
    T = c5.STEPS
    gpu.adjoint_forward(w, T, seeds)
    pos, tan, _ = gpu.adjoint_read()
    L_dev, g_dev = c5.gradient_from_tangents(s, w, pos, tan, th)
    L_ref, g_ref = c5.tangent_gradient(abi, sc, th, T, abi.ORDER_PRIORITY)
    fd = c5.central_differences(abi, sc, th, T, c5.H[1], abi.ORDER_PRIORITY)
    gpu.destroy()
    scale = float(np.max(np.abs(g_ref)))
    return {
        "workload": "differentiable wall: 256 bricks (16 x 16, 0.5 x 0.25 x 0.25 m, 1000 kg/m^3, hard bonds) + "
                    "50 kg sphere at 8 m/s; gradient of the mean brick displacement w.r.t. the sphere's initial "
                    "velocity (3), brick mu and the penalty cap",
        "bodies": w.n_bodies, "joints": w.n_joints, "steps": S, "directions": abi.TANGENT_DIMS,
        "value": S / adj_s, "unit": "adjoint steps/s",
        "how": f"avbd_adjoint_forward({S} steps, 5 forward-mode tangents, f64 values) + read + "
               f"avbd_adjoint_backward, host-timed around the C ABI calls, median of {R}",
        "ms_per_step": adj_s * 1e3 / S,
        "plain_fp32_step": {"value": S / (ms / 1e3), "unit": "steps/s", "ms_per_step": ms / S,
                            "how": "the same scene's FP32 step, device time (CUDA events)"},
        "cpu_baseline": {"plain_f64": S / cpu_plain, "tangent_f64": S / cpu_tan, "unit": "steps/s", "cores": 1,
                         "kind": "port", "sample": f"the oracle and the tangent oracle over the same {S} steps"},
        "accuracy": {"steps": T, "objective_device": L_dev, "objective_oracle": L_ref,
                     "gradient_device": g_dev.tolist(), "gradient_tangent_oracle": g_ref.tolist(),
                     "max_rel_error_vs_tangent_oracle": float(np.max(np.abs(g_dev - g_ref))) / scale,
                     "central_differences_h5e-5": fd.tolist(),
                     "v0_y_rel_error_vs_differences": abs(g_dev[1] - fd[1]) / abs(fd[1]),
                     "tolerance": "1e-6 relative to the tangent oracle (f64, same operations); 5 % along v0_y "
                                  "against the differences"},
    }


def run_accuracy(abi, backend):
    """The small configurations against the f64 oracle over their whole runs,
    both stepping the same start state (device colouring order replayed by
    the oracle): the 10-cube stack for 300 steps and the heavy chain (26,000:1
    end mass, hard joints) with the 1e3/1e6 spring chain for 1000 steps; the
    worst position error of any dynamic body and of the chain's end mass.
    Beside each, the oracle against itself from a start nudged by 1e-7 m (one
    body, x): these scenes are unstable or chaotic over their full length, so
    that divergence is the yardstick for the device's long-horizon error."""
    from oracle import Oracle

    sc = pkg().scene
    out = {}
    cases = (("cube_stack_300 (beta 10, as configured: sinks through the ground)", sc.cube_stack()),
             ("cube_stack_300 (reference ramps betaLin 1e4, betaAng 100)", sc.cube_stack(beta=None)),
             ("heavy_chain_1000 (50 hard links, 26,000 kg end mass, 1e3/1e6 spring chain)", sc.heavy_chain()))
    for name, s in cases:
        steps = s.meta["steps"]
        params = abi.default_params(**s.params, body_order=abi.ORDER_PRIORITY)
        w = s.world().round_to_device()
        gpu = backend.GpuBackend(params)
        gpu.pack(w)
        o = Oracle(params, w)
        dyn = w.mass > 0
        wn = w.copy()
        wn.pos[int(np.argmax(dyn)), 0] += 1e-7
        on = Oracle(params, wn)
        self_div, self_end = 0.0, 0.0
        worst, worst_end, worst_chain, worst_springs = 0.0, 0.0, 0.0, 0.0
        t0 = time.perf_counter()
        for k in range(steps):
            gpu.step(1)
            o.step(1)
            on.step(1)
            if (k + 1) % 10 == 0 or k + 1 == steps:
                g, r, rn = gpu.read_state(), o.state(), on.state()
                err = np.abs(g.pos[dyn] - r.pos[dyn]).max()
                worst = max(worst, float(err))
                self_div = max(self_div, float(np.abs(rn.pos[dyn] - r.pos[dyn]).max()))
                if "end_body" in s.meta:
                    e = s.meta["end_body"]
                    self_end = max(self_end, float(np.abs(rn.pos[e] - r.pos[e]).max()))
                if "end_body" in s.meta:
                    e = s.meta["end_body"]
                    c0, c1 = s.meta["chain_bodies"]
                    worst_end = max(worst_end, float(np.abs(g.pos[e] - r.pos[e]).max()))
                    worst_chain = max(worst_chain, float(np.abs(g.pos[c0:c1] - r.pos[c0:c1]).max()))
                    sp = np.arange(w.n_bodies) >= c1
                    sp &= dyn
                    worst_springs = max(worst_springs, float(np.abs(g.pos[sp] - r.pos[sp]).max()))
        st = gpu.last_stats
        rec = {"steps": steps, "bodies": w.n_bodies, "max_pos_error_m": worst, "fp64_bodies": st["fp64_bodies"],
               "final_pos_error_m": float(np.abs(gpu.read_state().pos[dyn] - o.state().pos[dyn]).max()),
               "wall_s": time.perf_counter() - t0}
        if "end_body" in s.meta:
            rec["end_mass_max_error_m"] = worst_end
            rec["chain_max_error_m"] = worst_chain
            rec["spring_chain_max_error_m"] = worst_springs
        rec["max_travel_m"] = float(np.abs(o.state().pos[dyn] - w.pos[dyn]).max())
        rec["oracle_vs_oracle_nudged_1e-7m_max_error_m"] = self_div
        if "end_body" in s.meta:
            rec["oracle_vs_oracle_nudged_end_mass_max_error_m"] = self_end
        out[name] = rec
        gpu.destroy()
    return out


def run_reference(args):
    """The reference's CPU engine algorithm (oracle restatement, index-order
    colouring as the reference's CPU solver), one host thread: the reference
    engine is single-threaded sequential Gauss-Seidel. The same window as the
    device arm: W untimed warm-up steps, then the scene is loaded again and
    steps 1..K of the run are timed from its initial state (until K steps or
    the time budget)."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    abi = pkg().abi
    from oracle import Oracle

    s = make_scene(args.layers)
    params = params_for(abi, s, body_order=abi.ORDER_REFERENCE)
    world = s.world()
    o = Oracle(params, world)
    o.step(args.warmup)
    o = Oracle(params, world)  # back to the initial state
    times = []
    while len(times) < args.steps and sum(times) < args.ref_budget:
        t0 = time.perf_counter()
        o.step(1)
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    value = len(times) / tot
    sample = (f"steps 1..{len(times)} of the run from its initial state after {args.warmup} untimed warm-up "
              f"steps, {tot:.1f} s of single-thread f64 work")
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": len(times),
        "warmup": args.warmup, "ms_per_step": tot * 1e3 / len(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(args, world.n_bodies, ws),
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=600)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--layers", type=int, default=53)
    ap.add_argument("--cpu-budget", type=float, default=45.0)
    ap.add_argument("--ref-budget", type=float, default=120.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the small-scene accuracy runs")
    ap.add_argument("--batched-steps", type=int, default=240, help="steps of the 512-scene batch (0: skip)")
    ap.add_argument("--dense-start", type=int, default=300, help="step the crushed-pile window starts after")
    ap.add_argument("--dense-steps", type=int, default=20, help="timed steps of the crushed-pile window (0: skip)")
    ap.add_argument("--adjoint-steps", type=int, default=60, help="steps of the differentiable wall (0: skip)")
    ap.add_argument("--only", default="", choices=["", "adjoint"],
                    help="run one record alone and print it (for profiling): adjoint = the differentiable wall")
    ap.add_argument("--trace", default="", help="write each timed step's profile and counters (JSON lines)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.only == "adjoint":
        import torch

        torch.cuda.set_device(0)
        abi = pkg().abi
        backend = importlib.import_module("avbd-sandbox_gb300.backend")
        print(json.dumps({"adjoint": run_adjoint(abi, backend, args)}), flush=True)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
