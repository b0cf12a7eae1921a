"""Benchmark of the fused colour-gradient LBM step on one GB300 (MLUPS, HBM roofline).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Workload: the D3Q27 liquid jet, 256 x 256 x 1024 fluid nodes (258 x 258 x 1026 lattice
with the ghost frame), inlet disc of diameter 32 at u_z = 0.05 with +-1% seeded noise,
periodic x/y, zero-gradient outflow, tau = 0.51, sigma = 1e-3, FP32 moments.  Synthetic
inputs: the case's own analytic initial condition (no dataset is involved).

One "step" is one time step of the whole lattice (one fused kernel launch).  MLUPS counts
the fluid nodes (nx-2)(ny-2)(nz-2) per step as the reference's MlupsCounter does
(utilities/mlups_count.cuh:24-29).  The state (2 x 2.95 GB) is far larger than the 129 MB
L2, so no explicit L2 flush is needed between timed steps.

--impl reference times the reference algorithm on the host cores instead: the CPU oracle's
FP32 restatement of the reference step (bit-exact with the reference's own code on the
golden fixtures), all host threads, on a z-slab sample of the same jet.

Serving (the "serving" object of the JSON line): a seeded stream of bubble and Rayleigh-Taylor
requests with Poisson arrivals runs once through the continuous-batching server and once one
request at a time through the single-case API (create, initial condition, steps, diagnostics,
destroy); both report cases/s, p50/p99 time to completion and aggregate MLUPS.  The full
workload (--serving full) is 256 requests at 20/s with 500-5000 steps each; the default sample
keeps the size and case distributions but scales every step count by 1/10 and the arrival rate
by 10, so the offered load (node updates per second of arrivals) is the same.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "lightweight-mb-color-gradient-lbm_gb300")
sys.path.insert(0, PKG)

import numpy as np  # noqa: E402

import mbcg  # noqa: E402

METRIC = "MLUPS & % of HBM roofline vs plain FP32; serving cases/s, p50/p99 at stated error"
BYTES_PER_NODE = {mbcg.FP32: 88, mbcg.FP16: 44, mbcg.BF16: 44}
WORKLOAD = "D3Q27 liquid jet 256x256x1024 fluid nodes (tau 0.51, sigma 1e-3, d=32 inlet, 1% noise)"


def jet_workload(precision=mbcg.FP32, nz: int = 1024, q: int = 27) -> mbcg.Params:
    return mbcg.jet_params(256, 256, nz, q=q, precision=precision)


def measured_peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic(kernel_tag: str):
    """DRAM bytes per launch from the committed ncu summary (profiles/<tag>.txt), if any."""
    path = os.path.join(ROOT, "profiles", f"{kernel_tag}.txt")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for line in f:
            if line.startswith("traffic_bytes_per_launch_full:"):
                try:
                    return float(line.split(":", 1)[1].strip().split()[0])
                except ValueError:
                    return None
    return None


class ClockSampler:
    """nvidia-smi clock / throttle samples while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.out = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        self.out.flush()

    def summary(self) -> dict:
        try:
            with open(self.out.name) as f:
                rows = [r.strip().split(",") for r in f if r.strip()]
        except Exception:
            rows = []
        finally:
            try:
                os.unlink(self.out.name)
            except OSError:
                pass
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for nm, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------- replicas (N > 1)
def replica_time(dt: float, world: int, dist, torch, device) -> float:
    """The slowest rank's time: every rank times its own replica between barriers, and the job
    is done when the last one is."""
    if world <= 1:
        return dt
    t = torch.tensor([dt], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_mlups(nodes: int, steps: int, dt_max: float, world: int) -> float:
    """Whole-job MLUPS of `world` independent replicas of `nodes` fluid nodes each."""
    return world * nodes * steps / dt_max / 1e6


def time_device(case: mbcg.Case, steps: int, warmup: int, torch):
    """CUDA-event time of `steps` fused steps on the launching stream (state resident)."""
    stream = torch.cuda.current_stream()
    case.step(warmup, stream)
    torch.cuda.synchronize()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    case.step(steps, stream)
    stop.record(stream)
    torch.cuda.synchronize()
    return start.elapsed_time(stop) / 1000.0


def time_e2e(p: mbcg.Params, steps: int, torch) -> dict:
    """End to end through the C ABI from pinned host memory.  Every step copies its input state
    from the host (H2D), advances it one fused step and copies the result back (D2H).  `value` is
    mbcg_run_host, which overlaps the result of one state going out with the next state coming
    in; `sequential_value` is the same through mbcg_copy_in / mbcg_step / mbcg_copy_out, one call
    after the other."""
    shape = (mbcg.NFIELDS,) + p.shape
    host_in = torch.empty(shape, dtype=torch.float32, pin_memory=True)
    host_out = torch.empty(shape, dtype=torch.float32, pin_memory=True)
    hin, hout = host_in.numpy(), host_out.numpy()
    with mbcg.Case(p) as c:
        c.init()
        c.copy_out(out=hin)
        c.run_host([hin] * 2, [hout] * 2, 1)  # warm-up (allocates the host-run images)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        c.run_host([hin] * steps, [hout] * steps, 1)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        c.copy_in(hin)
        c.step(1)
        c.copy_out(out=hout)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            c.copy_in(hin)
            c.step(1)
            c.copy_out(out=hout)
        torch.cuda.synchronize()
        dt_seq = time.perf_counter() - t0
    nbytes = host_in.numel() * 4
    return {"value": p.active_nodes() * steps / dt / 1e6, "unit": "MLUPS", "h2d_bytes_per_step": nbytes,
            "d2h_bytes_per_step": nbytes, "steps": steps, "api": "mbcg_run_host (transfers of consecutive states overlapped)",
            "sequential_value": p.active_nodes() * steps / dt_seq / 1e6,
            "sequential_api": "mbcg_copy_in + mbcg_step + mbcg_copy_out per step"}


def cpu_sample_params() -> mbcg.Params:
    """z-slab of the jet workload (same x/y extent and boundary kinds, 32 fluid planes)."""
    return mbcg.jet_params(256, 256, 32, q=27)


def cpu_leg(budget_s: float, threads: int, real_bytes: int = 4) -> dict:
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as ol
    p = cpu_sample_params()
    dtype = np.float32 if real_bytes == 4 else np.float64
    a = ol.oracle_init(p, dtype)
    b = a.copy()
    # the reference's cost structure: each source's colour gradient recomputed per direction
    ol.oracle_step(p, a, 1, threads=threads, b=b, reference_cost=True)  # warm
    steps, t0 = 0, time.perf_counter()
    while True:
        ol.oracle_step(p, a, steps + 2, threads=threads, b=b, reference_cost=True)
        a, b = b, a
        steps += 1
        dt = time.perf_counter() - t0
        if dt >= budget_s:
            break
    return {"value": p.active_nodes() * steps / dt / 1e6, "unit": "MLUPS", "cores": threads,
            "kind": "port", "sample": f"{steps} step(s) of a 256x256x32-fluid-node z-slab of the jet, "
                                      f"{'FP32' if real_bytes == 4 else 'FP64'} oracle, {dt:.1f} s"}


def reference_cuda_leg(steps: int, warmup: int, torch) -> dict:
    """The reference's own CUDA build on the same GB300: its unmodified RCSKernel +
    JetBoundaryConditions (kernels.cu:102-131, compiled for sm_103a with the jet's constants by
    oracle/Makefile `cubin`, block 32x4x2 as compile.sh:34-36) on the jet with the same fluid-node
    count (256 x 1024 x 256, the jet along the reference's y axis), timed with CUDA events on the
    launching stream over the same steps and warm-up.  A reported baseline, never the product."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from ref_cuda import RefKernels, cubin_path
    path = cubin_path("jet256")
    if not os.path.exists(path):
        print(f"bench.py: reference CUDA cubin {path} missing (build it with __graft_entry__.build() where "
              f"the reference sources are mounted)", file=sys.stderr)
        return {"unavailable": f"reference cubin {os.path.relpath(path, ROOT)} missing"}
    NX, NY, NZ = 258, 1026, 258
    k = RefKernels(path, (NX, NY, NZ))
    p = mbcg.reference_jet_params(NX, NY, NZ, q=27, tau=0.51, sigma=1e-3, beta=0.7, radius=16.0)
    lib = mbcg.Library.get()
    a = [torch.zeros(NX * NY * NZ, device="cuda") for _ in range(11)]
    m = mbcg.moments_from_tensors(a, NX)
    lib.check(lib.mbcg_init_moments(ctypes.byref(p), ctypes.byref(m), None), "init")
    b = [t.clone() for t in a]
    for _ in range(warmup):
        k.step(a, b)
        a, b = b, a
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(steps):
        k.step(a, b)
        a, b = b, a
    e.record()
    torch.cuda.synchronize()
    ms = s.elapsed_time(e) / steps
    nodes = (NX - 2) * (NY - 2) * (NZ - 2)
    del a, b
    torch.cuda.empty_cache()
    return {"value": nodes / ms / 1e3, "unit": "MLUPS", "ms_per_step": ms, "steps": steps, "warmup": warmup,
            "what": "reference kernels.cu (RCSKernel + JetBoundaryConditions), unmodified, sm_103a cubin, "
                    "D3Q27 jet 256x1024x256 fluid nodes (jet along y), block 32x4x2",
            "roofline_frac": BYTES_PER_NODE[mbcg.FP32] * nodes / (ms * 1e-3) / 1e9 / measured_peak_hbm()[0]}


# ---------------------------------------------------------------- serving workload
# ---------------------------------------------------------------- the other configurations
def configs_leg(torch) -> dict:
    """MLUPS of the plain step on the other configurations (state resident, launch shape measured
    by mbcg_autotune first): the 64^3 D3Q19 periodic bubble (config 0 physics), the
    128 x 128 x 512 D3Q27 Rayleigh-Taylor box (config 1 physics) and the jet in D3Q19."""
    cases = {
        "bubble64_q19": (mbcg.bubble_params(64, q=19), 400),
        "rti128x512_q27": (mbcg.rti_params(128, q=27), 100),
        "jet256x1024_q19": (mbcg.jet_params(256, 256, 1024, q=19), 50),
    }
    out = {}
    for name, (p, steps) in cases.items():
        with mbcg.Case(p) as c:
            c.init()
            c.autotune(repeats=3)
            ms = time_device(c, steps, 3, torch) / steps * 1e3
            w, z = c.shape
        state_bytes = 2 * 11 * 4 * p.nx * p.ny * p.nz
        out[name] = {"mlups": p.active_nodes() / ms / 1e3, "ms_per_step": ms, "block_rows": w, "zchunk": z,
                     "roofline_frac": BYTES_PER_NODE[mbcg.FP32] * p.active_nodes() / (ms * 1e-3) / 1e9 / measured_peak_hbm()[0],
                     "state_bytes": state_bytes, "l2_resident": state_bytes < 129e6}
    return out


def serving_requests(n: int, rate: float, step_scale: float, seed: int = 20240):
    """Seeded request stream: Poisson arrivals at `rate`/s; bubble (config-0 physics, radius L/4,
    L log-uniform in [32, 192]) or Rayleigh-Taylor (config-1 physics, L x L x 4L, L log-uniform
    in [32, 128]) with equal probability; D3Q19 or D3Q27 and FP32 or FP16 moments by coin flip;
    steps uniform in [500, 5000] times step_scale."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for _ in range(n):
        t += rng.exponential(1.0 / rate)
        bubble = rng.random() < 0.5
        q = 19 if rng.random() < 0.5 else 27
        prec = mbcg.FP32 if rng.random() < 0.5 else mbcg.FP16
        steps = max(1, int(round(rng.uniform(500, 5000) * step_scale)))
        if bubble:
            L = int(round(np.exp(rng.uniform(np.log(32), np.log(192)))))
            p = mbcg.bubble_params(L, q=q, radius=0.25 * L, precision=prec)
        else:
            L = int(round(np.exp(rng.uniform(np.log(32), np.log(128)))))
            p = mbcg.rti_params(L, q=q, precision=prec)
        out.append({"t": t, "p": p, "steps": steps, "kind": "bubble" if bubble else "rti", "L": L})
    return out


def _pct(v, q):
    return float(np.percentile(np.asarray(v), q)) if v else None


def serve_batched(reqs, policy=mbcg.POLICY_FIFO) -> dict:
    with mbcg.Server(policy=policy) as srv:
        t0 = time.perf_counter()
        ids = []
        for r in reqs:
            delay = r["t"] - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
            ids.append(srv.submit(r["p"], r["steps"]))
        srv.drain()
        infos = [srv.poll(i) for i in ids]
        st = srv.stats().as_dict()
    ttc = [i.t_done - i.t_submit for i in infos]
    span = max(i.t_done for i in infos) - min(i.t_submit for i in infos)
    work = sum(r["p"].active_nodes() * r["steps"] for r in reqs)
    return {"cases_per_s": len(reqs) / span, "p50_s": _pct(ttc, 50), "p99_s": _pct(ttc, 99), "makespan_s": span,
            "mlups": work / span / 1e6, "failed": sum(i.state != mbcg.REQ_DONE for i in infos),
            "compositions": st["compositions"], "replays": st["replays"], "zchunk_last": st["zchunk"],
            "cost_model_ns_per_plane": st["plane_ns"], "tile_overhead_planes": st["tile_overhead_planes"],
            "arena_peak_gb": st["arena_peak_bytes"] / 1e9,
            "mass": [(i.diag.mass_r, i.diag.mass_b) for i in infos],
            "nonfinite": sum(i.diag.nonfinite for i in infos)}


def serve_sequential(reqs, torch) -> dict:
    t0 = time.perf_counter()
    ttc, done, mass, dev = [], [], [], []
    stream = torch.cuda.current_stream()
    for r in reqs:
        now = time.perf_counter() - t0
        if now < r["t"]:
            time.sleep(r["t"] - now)
        with mbcg.Case(r["p"]) as c:
            c.init()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            c.step(r["steps"], stream)
            e.record(stream)
            d = c.diagnostics(stream)
            e.synchronize()
            dev.append(s.elapsed_time(e) / 1e3)
        fin = time.perf_counter() - t0
        done.append(fin)
        ttc.append(fin - r["t"])
        mass.append((d["mass_r"], d["mass_b"]))
    span = max(done) - reqs[0]["t"]
    work = sum(r["p"].active_nodes() * r["steps"] for r in reqs)
    return {"cases_per_s": len(reqs) / span, "p50_s": _pct(ttc, 50), "p99_s": _pct(ttc, 99), "makespan_s": span,
            "mlups": work / span / 1e6, "mass": mass, "device_s": dev}


def serving_bound(reqs, device_s) -> dict:
    """Ceiling on cases/s for this request stream when every request runs at the plain kernel's
    rate on its own lattice (its measured single-case stepping time) with no other cost: the
    makespan of the best preemptive one-at-a-time schedule with these release times,
    max over k of (a_k + the work released at or after a_k) - a_0."""
    order = sorted(range(len(reqs)), key=lambda i: reqs[i]["t"])
    a = [reqs[i]["t"] for i in order]
    t = [device_s[i] for i in order]
    tail, best = 0.0, 0.0
    for k in range(len(a) - 1, -1, -1):
        tail += t[k]
        best = max(best, a[k] + tail)
    span = best - a[0]
    return {"cases_per_s": len(reqs) / span, "makespan_s": span, "device_s_total": sum(t),
            "how": "release times of the stream, per-request device time of the plain step kernel alone "
                   "(CUDA events around its steps in the sequential run), no set-up, admission or host cost"}


def serving_leg(mode: str, torch) -> dict:
    if mode == "full":
        n, rate, scale = 256, 20.0, 1.0
    else:
        n, rate, scale = 64, 200.0, 0.1
    reqs = serving_requests(n, rate, scale)
    b = serve_batched(reqs)
    bs = serve_batched(reqs, mbcg.POLICY_SJF)
    bs.pop("mass")
    s = serve_sequential(reqs, torch)
    bound = serving_bound(reqs, s.pop("device_s"))
    rel = 0.0
    for (br, bb), (sr, sb) in zip(b.pop("mass"), s.pop("mass")):
        rel = max(rel, abs(br - sr) / abs(sr), abs(bb - sb) / abs(sb))
    return {"workload": ("full: " if mode == "full" else "sample: ") +
            f"{n} requests, Poisson {rate:g}/s, bubble L in [32,192] or RTI LxLx4L L in [32,128] (log-uniform), "
            f"Q19/Q27 and FP32/FP16 by coin flip, steps U[500,5000] x {scale:g}",
            "batched": b, "sequential": s, "cases_per_s_ratio": b["cases_per_s"] / s["cases_per_s"],
            "bound": bound, "bound_ratio": b["cases_per_s"] / bound["cases_per_s"],
            "sequential_bound_ratio": s["cases_per_s"] / bound["cases_per_s"],
            "policy": "FIFO admission with backfill (all requests that fit are live)",
            "batched_sjf": {k: bs[k] for k in ("cases_per_s", "p50_s", "p99_s", "mlups", "makespan_s")},
            "batched_sjf_policy": "shortest job first with aging, live set capped at 4 waves of tiles",
            "accuracy": {"max_rel_phase_mass_diff_batched_vs_sequential": rel,
                         "note": "same physics in both; the batch kernel and the single-case kernel are "
                                 "separate compilations (parity gate rel L2 1e-5, tests/test_gpu_server.py)"}}


def reference_arm(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    budget = float(os.environ.get("MBCG_REF_BUDGET_S", "8"))
    vals = []
    leg = None
    for _ in range(max(args.warmup, 0)):
        cpu_leg(min(budget, 2.0), threads)
    for _ in range(max(args.steps, 1)):
        leg = cpu_leg(budget, threads)
        vals.append(leg["value"])
    v = statistics.median(vals)
    slab = cpu_sample_params()
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": "MLUPS", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": slab.active_nodes() / v / 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (analytic jet initial condition)",
           "config": {"workload": WORKLOAD, "sample": "256x256x32 z-slab per step", "host_threads": threads},
           "cpu_baseline": {"value": v, "unit": "MLUPS", "cores": threads, "kind": "port",
                            "sample": leg["sample"] if leg else ""},
           "e2e": {"value": v, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--cpu-budget", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--forms", default="fp16,bf16")
    ap.add_argument("--nz", type=int, default=1024, help="fluid planes of the jet (profiling uses fewer)")
    ap.add_argument("--q", type=int, default=27, choices=[27, 19], help="lattice of the jet (profiling the D3Q19 step)")
    ap.add_argument("--serving", default="sample", choices=["off", "sample", "full"])
    ap.add_argument("--no-configs", action="store_true", help="skip the bubble / RTI / D3Q19 lines")
    ap.add_argument("--no-ref-cuda", action="store_true", help="skip timing the reference's CUDA kernel")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    if args.impl == "reference":
        reference_arm(args)
        return

    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")

    p = jet_workload(mbcg.FP32, args.nz, args.q)
    peak, peak_kind = measured_peak_hbm()
    # The end-to-end leg runs first: its pinned host buffers are then allocated as a caller does at
    # start-up, before this process has allocated and freed the other legs' ~12 GB (after that,
    # the same leg measured 25-30 % slower, with no change on the device side).
    e2e = time_e2e(p, args.e2e_steps, torch) if rank == 0 and args.e2e_steps > 0 else None
    with mbcg.Case(p) as case:
        case.init()
        launches = case.launches_per_step()
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        with ClockSampler(local) as clk:
            dt = time_device(case, args.steps, args.warmup, torch)
        diag = case.diagnostics()
        status = case.status()
    dt = replica_time(dt, world, dist, torch, "cuda")
    nodes = p.active_nodes()
    mlups = replica_mlups(nodes, args.steps, dt, world)
    per_launch = dt / (args.steps * launches)
    achieved = BYTES_PER_NODE[mbcg.FP32] * nodes / per_launch / 1e9
    traffic = profiled_traffic("step_kernel_jet256_fp32")

    forms = {}
    for name in [f for f in args.forms.split(",") if f]:
        prec = {"fp16": mbcg.FP16, "bf16": mbcg.BF16}[name]
        q = jet_workload(prec, args.nz, args.q)
        with mbcg.Case(q) as c:
            c.init()
            t = time_device(c, args.steps, args.warmup, torch)
        v = nodes * args.steps / t / 1e6
        forms[name] = {"value": v, "unit": "MLUPS", "vs_fp32": v / (mlups / world),
                       "roofline_frac": BYTES_PER_NODE[prec] * nodes / (t / args.steps) / 1e9 / peak}

    serving = serving_leg(args.serving, torch) if rank == 0 and args.serving != "off" else None
    configs = configs_leg(torch) if rank == 0 and not args.no_configs else None
    cpu = cpu64 = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_leg(args.cpu_budget, os.cpu_count() or 1)
        cpu64 = cpu_leg(args.cpu_budget, os.cpu_count() or 1, real_bytes=8)
    ref_cuda = reference_cuda_leg(args.steps, args.warmup, torch) if rank == 0 and not args.no_ref_cuda else None

    if rank == 0:
        out = {
            "metric": METRIC, "value": mlups, "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (analytic jet initial condition, seeded inlet noise)",
            "config": {"workload": (WORKLOAD if args.nz == 1024 else WORKLOAD.replace("x1024", f"x{args.nz}")).replace("D3Q27", f"D3Q{args.q}"), "lattice": [p.nx, p.ny, p.nz], "fluid_nodes": nodes,
                       "precision": "fp32 moments", "l2": "state 2x2.95 GB > 129 MB L2, no flush needed",
                       "parallelism": "replicas" if world > 1 else "single GPU", "zchunk": os.environ.get("MBCG_ZCHUNK", "auto"),
                       "reference_arm_sample": "bench.py --impl reference times the reference arithmetic (FP32 "
                                               "oracle) on the host cores over a 256x256x32-fluid-node z-slab of this "
                                               "jet per step: the same per-node work, a 32-plane sample of the lattice"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "algorithmic_bytes_per_node": BYTES_PER_NODE[mbcg.FP32]},
            "forms": forms,
            "serving": serving,
            "configs": configs,
            "e2e": e2e,
            "cpu_baseline": cpu,
            "cpu_baseline_fp64": cpu64,
            "reference_cuda": ref_cuda,
            "vs_reference_cuda": (mlups / world / ref_cuda["value"]) if ref_cuda and "value" in ref_cuda else None,
            "gpu_launches": args.steps * launches,
            "clocks": clk.summary(),
            "checks": {"mass_r": diag["mass_r"], "mass_b": diag["mass_b"], "nonfinite": diag["nonfinite"],
                       "status": status},
        }
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
