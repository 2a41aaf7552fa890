"""Benchmark of the AVBD world step on GB300.

Workload (one "step" = one AVBD world step of the whole scene): the dense
pile - a square pyramid of 53 layers (layer k is a k x k grid of 1 m cubes,
51,039 cubes, 1% gap, 1000 kg/m^3, mu 0.6) on the ground, with a 2 m-radius
sphere (5000 kg/m^3) dropped onto the apex at 10 m/s; dt = 1/60 s,
10 iterations, gravity -9.81. Synthetic scene, seeded and deterministic.

Timing: W warm-up steps, then exactly K steps. Each step's device time comes
from CUDA events recorded by the library on its own stream around the whole
step; L2 is flushed (a 256 MB write) between steps, outside those events.
The JSON line also carries the roofline of the dominant kernel, the f64 CPU
baseline (the oracle, 1 thread, a bounded sample of the same scene), the
end-to-end rate through the C ABI with host buffers, the kernel launch count
and the SM clocks sampled during the timed region.

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

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "AVBD steps/s at 51k boxes vs f64 CPU ref; batched & adjoint steps/s at tol"
UNIT = "steps/s"
WORKLOAD = ("pyramid: 53 layers = 51,039 1 m cubes (1% gap, 1000 kg/m^3, mu 0.6) + ground + r=2 m sphere "
            "(5000 kg/m^3, 10 m/s onto the apex); dt=1/60, 10 iterations, gravity -9.81")


def pkg():
    return importlib.import_module("avbd-sandbox_gb300")


def make_scene(layers):
    sc = pkg().scene
    return sc.pyramid(layers=layers)


def params_for(abi, s, **kw):
    kw.setdefault("body_order", abi.ORDER_PRIORITY)
    return abi.default_params(**s.params, **kw)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# ---------------------------------------------------------------------------
# CPU baseline: the f64 oracle, one thread, a bounded sample of the workload
# ---------------------------------------------------------------------------
def cpu_baseline(scene, params, budget_s=20.0, warm=3, max_steps=30):
    from oracle import Oracle

    o = Oracle(params, scene.world())
    o.step(warm)  # layers settle into contact (they start 1 cm apart)
    times = []
    t_all = time.perf_counter()
    while len(times) < max_steps and (time.perf_counter() - t_all) < budget_s:
        t0 = time.perf_counter()
        o.step(1)
        times.append(time.perf_counter() - t0)
    med = statistics.median(times)
    return {
        "value": 1.0 / med,
        "unit": UNIT,
        "cores": 1,
        "kind": "port",
        "sample": f"steps {warm + 1}..{warm + len(times)} of the same scene from its initial state; median of "
                  f"{len(times)} single-thread steps ({sum(times):.1f} s of CPU work)",
        "ms_per_step": med * 1e3,
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
# roofline of the dominant kernel (algorithmic bytes)
# ---------------------------------------------------------------------------
def algorithmic_bytes(kind, st, n_dyn, iterations, n_joints=0, n_springs=0):
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


def read_traffic(kernel):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f).get(kernel)
    except Exception:
        return None


# ---------------------------------------------------------------------------
def run_gpu(args):
    import ctypes

    import torch

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    abi = pkg().abi
    backend = importlib.import_module("avbd-sandbox_gb300.backend")
    s = make_scene(args.layers)
    params = params_for(abi, s)
    world = s.world()
    gpu = backend.GpuBackend(params)
    gpu.pack(world)
    n_dyn = int((world.mass > 0).sum())

    gpu.step(args.warmup)
    gpu.idle()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    gpu.set_profiling(True)
    launches0 = gpu.kernel_launches
    phase_tot = {k: 0.0 for k in ("broadphase_ms", "narrowphase_ms", "prepare_ms", "coloring_ms", "solve_ms")}
    step_ms = []
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.fill_(1.0)  # L2 flush, outside the step's events
            torch.cuda.synchronize()
            gpu.step(1)
            p = gpu.last_profile
            step_ms.append(p["step_ms"])
            for k in phase_tot:
                phase_tot[k] += p[k]
    gpu.idle()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    launches = gpu.kernel_launches - launches0
    dev_s = sum(step_ms) / 1e3
    if ws > 1:
        t = torch.tensor([dev_s], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        dev_s = float(t.item())
    st = gpu.last_stats
    gpu.set_profiling(False)

    # back-to-back steady state (no flush, no per-step sync), for information
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    gpu.idle()
    t1 = time.perf_counter()
    gpu.step(args.steps)
    gpu.idle()
    b2b = (time.perf_counter() - t1) / args.steps

    # end to end through the C ABI with host buffers: upload state, step, read back
    e2e_steps = max(3, min(args.steps, 20))
    host = gpu.read_state()
    gpu.idle()
    t2 = time.perf_counter()
    for _ in range(e2e_steps):
        gpu.write_state(host)
        gpu.step(1)
        gpu.sync_to_cpu(host)
    e2e_s = (time.perf_counter() - t2) / e2e_steps
    n = world.n_bodies
    per_body = 32 + 4 * 16  # f64 position (D4) + quaternion, velocity, angular velocity, previous velocity (float4)

    # dominant kernel and its roofline
    phases = {k: v / args.steps for k, v in phase_tot.items()}
    kinds = {"solve_ms": ("solve", "solve_kernel"), "narrowphase_ms": ("narrowphase", "narrowphase_kernel")}
    dom = max(kinds, key=lambda k: phases[k])
    kind, kname = kinds[dom]
    algo = algorithmic_bytes(kind, st, n_dyn, params.iterations)
    peak, peak_src = read_peaks()
    achieved = algo / (phases[dom] / 1e3) / 1e9
    traffic = read_traffic(kname)
    value = ws * args.steps / dev_s
    clocks = clk.summary()
    out = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": dev_s * 1e3 / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 (f64 narrowphase geometry, f64 positions and joint multipliers)",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "bodies": n, "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU",
                   "l2": "flushed between steps (256 MB write), outside the timed step events"},
        "roofline": {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_src, "traffic": traffic,
                     "algorithmic_bytes_per_launch": algo, "launch_ms": phases[dom]},
        "e2e": {"value": 1.0 / e2e_s, "unit": UNIT, "h2d_bytes_per_step": n * per_body,
                "d2h_bytes_per_step": n * per_body,
                "how": "avbd_write_state + avbd_step(1) + avbd_read_state per step, pinned staging, host f64 arrays"},
        "gpu_launches": launches,
        "clocks": clocks,
        "phases_ms": phases,
        "back_to_back_steps_per_s": 1.0 / b2b,
        "wall_s": wall,
        "stats": {k: st[k] for k in ("manifolds", "contacts", "candidate_pairs", "colors", "fp64_bodies")},
    }
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(s, params, budget_s=args.cpu_budget)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def run_reference(args):
    """The reference's CPU engine algorithm (oracle restatement), host cores."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    abi = pkg().abi
    from oracle import Oracle

    s = make_scene(args.layers)
    params = params_for(abi, s, body_order=abi.ORDER_REFERENCE)
    o = Oracle(params, s.world())
    o.step(3)
    # each measured step is one step of the same workload; bounded to a few minutes
    n = max(1, min(args.steps, int(args.cpu_budget * 3)))
    o.step(min(args.warmup, 2))
    times = []
    for _ in range(n):
        t0 = time.perf_counter()
        o.step(1)
        times.append(time.perf_counter() - t0)
        if sum(times) > args.cpu_budget * 6:
            break
    tot = sum(times)
    value = len(times) / tot
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": len(times),
        "warmup": 3 + min(args.warmup, 2), "ms_per_step": tot * 1e3 / len(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "bodies": s.world().n_bodies},
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": f"{len(times)} consecutive steps of the same scene after 3 + warm-up steps; the "
                                   "reference engine is single-threaded sequential Gauss-Seidel, so 1 thread"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--layers", type=int, default=53)
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
