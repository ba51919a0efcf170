#!/usr/bin/env python3
"""Benchmark of the sphere-BVE direct-sum hot path on GB300.

Workload (the configuration the headline metric is quoted on): icosahedral mesh nest 8,
1,966,082 targets and 1,310,720 active sources, relative vorticity = Rossby-Haurwitz wave 4
plus a Gaussian vortex at a seeded random centre (mean removed), Omega = 2 pi.  One step is
one classical RK4 step = 4 velocity sums (2.577e12 interactions each) plus the FP64 stage
combinations, replayed from one CUDA graph, in LPM_MODE_FP32C, with the stage positions
projected onto the sphere (at this resolution the unprojected stage positions of the
reference scheme leave the sphere by more than the nearest-neighbour gap a^2 - x.x_j, and
the Biot-Savart denominator changes sign).

Metric: Ginteractions/s (interactions = N_targets * N_sources - self pairs per sum).
  value : device time of the K steps with the state resident in HBM (CUDA events on the
          solver's stream, L2 flushed with a 256 MB write between steps, outside the events)
  e2e   : the same steps through the C ABI with the state copied from pinned host memory
          before and back after every step (lpm_bve_set_state / lpm_bve_timestep /
          lpm_bve_get_state), timed with CUDA events on the same stream
  roofline: the velocity-sum kernels against the measured FP32 FMA peak (24 flops/pair),
          with the sweep's recorded ncu pipe utilisation beside the contract fraction
  accuracy: the FP32C velocity at the final state against the oracle (FP64) on a target block
  fp64_gpu: the plain FP64 GPU kernel (parity mode) on the same state, on a block of targets
          that fills every SM, and the FP32C/FP64 ratio
  ensemble: config 5 (64 uneven instances at icos nests 3-6), batched persistent launch
          against one solver per instance, a few RK4 steps each
  cpu_baseline: the CPU oracle (the reference loop restated in C, OpenMP over targets) on
          a bounded sample of targets against all sources

--impl reference times the reference's CPU implementation of the path (the C restatement
in oracle/, all host threads) on the same workload, each step a bounded target sample.
Under torchrun (N > 1) every rank runs an independent replica on its own GPU (the path has
no exchange step on one node's replicas), and value = all ranks' interactions / max time.
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
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "lpm-v2_gb300"))

METRIC = "BVE direct-sum Ginteractions/s, FP32-comp vs FP64 on GB300 at <=1e-6 rel err"
UNIT = "Ginteractions/s"
# the PSE operators that have an FP64 form only (their FP32C form would be ill-conditioned):
# --workload sum runs them in FP64 whatever --mode says
FP64_ONLY_SUMS = ("pse_plane_grad", "pse_plane_second", "pse_plane_ddot", "pse_sphere_ddot", "pse_interp")
FLOPS_PER_INTERACTION = 24  # dot 5, a^2-dot 1, x4pi a 1, zeta A/den 2, cross 9, accumulate 6
L2_FLUSH_BYTES = 256 << 20
# DRAM bytes (ncu dram__bytes_read.sum + dram__bytes_write.sum) of one full-size icos nest 8
# sweep launch, from a single-pass ncu capture of this benchmark's own step (ncu cannot run
# inside the timed region, so this is a recorded constant, not a figure of this run)
SWEEP_TRAFFIC_ICOS8 = 264_474_880 + 126_703_360
# Pipe utilisation of the same sweep kernel (ncu --set full of bve_rel_sweep_kernel<128,4,256,4>,
# the autotuner's shape, on this workload at icos nest 7, one launch): the pipe-level counterpart
# of the flop-contract fraction; recorded constants, not figures of this run
SWEEP_PIPES_ICOS7 = {"fma_pipe_active": 0.6801, "xu_pipe_active": 0.6448, "issue_active": 0.5366}
# FP32 CUDA-core nominal peak: 152 SMs x 128 lanes x 2 flops per FMA, per MHz of SM clock
FP32_NOMINAL_TFLOPS_PER_MHZ = 152 * 128 * 2 / 1e6
# FP64: 2 DFMA per clock per SM (4 flops), per MHz
FP64_NOMINAL_TFLOPS_PER_MHZ = 152 * 4 / 1e6
# FP64 parity-mode rate at the headline size: the FP64 sweep on a block of targets that gives
# every SM two 128-thread CTAs (the per-target cost is the same for every target)
FP64_BLOCK_TARGETS = 152 * 2 * 128


def parse_args():
    p = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--nest", type=int, default=8, help="icosahedral refinement level (8 = the metric's size)")
    p.add_argument("--dt", type=float, default=0.01)
    p.add_argument("--accuracy-targets", type=int, default=8192)
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU-baseline sample budget")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-fp64", action="store_true", help="skip the FP64 parity-mode rate at the headline size")
    p.add_argument("--no-ensemble", action="store_true", help="skip the 64-instance ensemble object")
    p.add_argument("--ensemble-steps", type=int, default=10, help="RK4 steps of the ensemble object")
    p.add_argument("--no-size-classes", action="store_true",
                   help="--workload ensemble: skip the per-refinement-level measurements")
    p.add_argument("--workload", choices=["rk4", "ensemble", "stream", "configs", "sum", "remesh"], default="rk4",
                   help="rk4: the headline single-instance step; ensemble: the 64-instance batch")
    p.add_argument("--instances", type=int, default=64)
    p.add_argument("--sum", choices=["bve", "plane", "pse_k8", "pse_gauss", "pse_grad", "pse_div", "pse_plane",
                                     "stream", "plane_stream", "beta", "beta_stream", "swe_plane", "swe_sphere"]
                   + list(FP64_ONLY_SUMS),
                   default="bve",
                   help="--workload sum: which direct sum (one host C-ABI call per step)")
    p.add_argument("--mode", choices=["fp32c", "fp64"], default="fp32c", help="--workload sum: precision mode")
    p.add_argument("--targets", type=int, default=0, help="--workload sum: first N targets only (0: all)")
    return p.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def workload(nest: int):
    import workloads as wl
    c = wl.config_rh54_icos(nest, seed=0)
    n = c["x"].size
    ns = int(c["active"].sum())
    per_sum = n * ns - ns
    return c, n, ns, per_sum


def workload_name(nest, n, ns):
    return (f"sphere BVE RK4 step, icosahedral nest {nest} ({n} targets, {ns} sources), "
            f"RH4 + Gaussian vortex, 4 velocity sums per step in one CUDA graph")


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples (200 ms) during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id: str):
        self.gpu_id = gpu_id
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", self.gpu_id], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def gpu_id_for(torch, dev: int) -> str:
    try:
        u = str(torch.cuda.get_device_properties(dev).uuid)
        return u if u.startswith("GPU-") else f"GPU-{u}"
    except Exception:
        return str(dev)


# ------------------------------------------------------------------ CPU sides
def cpu_sample_rate(c, n, ns, budget_s: float):
    """Times the oracle's BVE sum on a contiguous block of targets against all sources,
    scaled so the sample takes about budget_s seconds.  Returns (Ginter/s, cores, desc)."""
    from oracle import oracle as orc
    args = (c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"])
    start = n // 3
    probe = 64
    t0 = time.perf_counter()
    orc.bve_velocity(*args, ib=start, ie=start + probe)
    dt = max(time.perf_counter() - t0, 1e-6)
    m = int(min(n - start, max(probe, probe * budget_s / dt)))
    t0 = time.perf_counter()
    orc.bve_velocity(*args, ib=start, ie=start + m)
    el = time.perf_counter() - t0
    act = int(c["active"][start:start + m].sum())
    inter = m * ns - act
    cores = os.cpu_count() or 1
    desc = (f"oracle BVE sum (OpenMP, {cores} threads), targets {start + 1}..{start + m} of {n} against all "
            f"{ns} sources ({inter:.3e} interactions, {el:.1f} s)")
    return inter / el / 1e9, cores, desc, m


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    c, n, ns, per_sum = workload(args.nest)
    from oracle import oracle as orc
    # one step = the oracle sum over a fixed block of targets, sized to ~4 s
    rate, cores, desc, m = cpu_sample_rate(c, n, ns, 4.0)
    a = (c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"])
    start = n // 3
    for _ in range(args.warmup):
        orc.bve_velocity(*a, ib=start, ie=start + m)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        orc.bve_velocity(*a, ib=start, ie=start + m)
        times.append(time.perf_counter() - t0)
    inter = m * ns - int(c["active"][start:start + m].sum())
    value = inter * args.steps / sum(times) / 1e9
    sample = (f"each step: the oracle BVE sum for targets {start + 1}..{start + m} against all {ns} sources "
              f"({inter:.3e} interactions)")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_name(args.nest, n, ns), "n_targets": n, "n_sources": ns,
                   "interactions_per_sum": per_sum, "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ GPU side
def run_ours(args):
    import ctypes
    import torch
    import lpm_gpu as lg
    from replicas import max_over_ranks, replica_rate

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()

    c, n, ns, per_sum = workload(args.nest)
    peak = lg.measure_fp32_peak(300.0)
    stream = torch.cuda.Stream()
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    solver = lg.BVESolver(c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"], c["radius"], c["omega"],
                          mode="fp32c")
    solver.set_stream(stream.cuda_stream)
    diag0 = solver.diagnostics()

    for _ in range(args.warmup):
        solver.timestep(args.dt, 1, renormalize=True)

    # ---------------- timed region (state resident in HBM)
    sampler = ClockSampler(gpu_id_for(torch, local))
    sampler.start()
    time.sleep(0.5)
    k_ms0, k_n0 = solver.kernel_timing()
    barrier()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.zero_()
            starts[k].record(stream)
            solver.timestep(args.dt, 1, renormalize=True)
            ends[k].record(stream)
    torch.cuda.synchronize()
    barrier()
    clocks = sampler.stop()
    k_ms1, k_n1 = solver.kernel_timing()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    inter_step = 4 * per_sum
    total_ms = 1e3 * max_over_ranks(sum(step_ms) * 1e-3, dist, "cuda")
    value = replica_rate(inter_step * args.steps, total_ms * 1e-3, dist, "cuda") / 1e9

    # velocity-sum kernels: events around each sum inside the graph
    sums = 4 * args.steps
    sum_ms = (k_ms1 - k_ms0) / sums
    achieved_tflops = FLOPS_PER_INTERACTION * per_sum / (sum_ms * 1e-3) / 1e12

    # ---------------- accuracy of the FP32C velocity at the final state against the oracle
    # (the reference loop restated in C, FP64) on a seeded block of targets
    from oracle import oracle as orc
    st = solver.get_state()
    rng = np.random.default_rng(1)
    m = min(args.accuracy_targets, n)
    ib = int(rng.integers(0, n - m + 1)) + 1
    ref = np.stack(orc.bve_velocity(st["x"], st["y"], st["z"], st["rel_vort"], c["area"], c["active"], c["radius"],
                                    ib=ib - 1, ie=ib - 1 + m))
    got = np.stack([st[k][ib - 1:ib - 1 + m] for k in ("u", "v", "w")])
    rel_linf = float(np.abs(got - ref).max() / np.abs(ref).max())
    rel_l2 = float(np.sqrt(np.sum((got - ref) ** 2) / np.sum(ref ** 2)))
    diag1 = solver.diagnostics()

    # ---------------- the plain FP64 GPU kernel (parity mode) at the same size and state
    fp64 = None
    if not args.no_fp64:
        m64 = min(FP64_BLOCK_TARGETS, n)
        b64 = n // 2 - m64 // 2 + 1
        fa = (st["x"], st["y"], st["z"], st["rel_vort"], c["area"], c["active"], c["radius"])
        lg.bve_sphere_velocity(*fa, i_begin=b64, i_end=b64 + 127, mode="fp64")  # warm-up
        t0 = time.perf_counter()
        lg.bve_sphere_velocity(*fa, i_begin=b64, i_end=b64 + m64 - 1, mode="fp64")
        t64 = time.perf_counter() - t0
        inter64 = m64 * ns - int(c["active"][b64 - 1:b64 - 1 + m64].sum())
        r64 = inter64 / t64 / 1e9
        mhz = clocks.get("sm_mhz") or 2070.0
        fp64 = {"value": r64, "unit": UNIT, "fp32c_over_fp64": value / r64,
                "contract_tflops": FLOPS_PER_INTERACTION * r64 / 1e3,
                "frac_of_nominal_fp64_peak": FLOPS_PER_INTERACTION * r64 / 1e3 / (FP64_NOMINAL_TFLOPS_PER_MHZ * mhz),
                "kernel": "seq_fp64_kernel<BveF64<0>> (one target per thread, sources in ascending order, "
                          "bit-identical to the oracle)",
                "sample": f"targets {b64}..{b64 + m64 - 1} against all {ns} sources ({inter64:.3e} interactions), "
                          "one host C-ABI call, wall clock, copies included",
                "seconds": t64}

    # ---------------- end to end through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        L = lg.lib()
        host = {k: torch.from_numpy(np.ascontiguousarray(st[k])).pin_memory()
                for k in ("x", "y", "z", "rel_vort", "u", "v", "w")}
        ptrs = [ctypes.cast(host[k].data_ptr(), ctypes.POINTER(ctypes.c_double))
                for k in ("x", "y", "z", "rel_vort", "u", "v", "w")]
        es = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ee = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        barrier()
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                flush.zero_()
                es[k].record(stream)
                lg._check(L.lpm_bve_set_state(solver._h, *ptrs))
                lg._check(L.lpm_bve_timestep(solver._h, args.dt, 1, 1))
                lg._check(L.lpm_bve_get_state(solver._h, *ptrs))
                ee[k].record(stream)
        torch.cuda.synchronize()
        barrier()
        e_s = sum(s.elapsed_time(e) for s, e in zip(es, ee)) * 1e-3
        nbytes = 7 * n * 8
        e2e = {"value": replica_rate(inter_step * args.steps, e_s, dist, "cuda") / 1e9, "unit": UNIT,
               "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
               "path": "lpm_bve_set_state + lpm_bve_timestep + lpm_bve_get_state, pinned host buffers"}

    ens = None
    if not args.no_ensemble and world == 1:
        import workloads as wl
        ens = measure_ensemble(torch, lg, wl, args.instances, args.ensemble_steps, 3, args.dt)
        ens.pop("errs", None)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline and world == 1:
        rate, cores, desc, _ = cpu_sample_rate(c, n, ns, args.cpu_seconds)
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port", "sample": desc}

    solver.close()
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": workload_name(args.nest, n, ns), "n_targets": n, "n_sources": ns,
                       "interactions_per_sum": per_sum, "sums_per_step": 4, "mode": "LPM_MODE_FP32C",
                       "renormalize": "stage inputs and new positions projected onto the sphere",
                       "dt": args.dt, "l2": "flushed between steps (256 MB write, outside the timed events)",
                       "parallelism": f"replicas x{world}"},
            "clocks": clocks,
            "gpu_launches": k_n1 - k_n0,
            "roofline": {"bound": "fp32", "achieved": achieved_tflops, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved_tflops / peak,
                         "frac_of_nominal": achieved_tflops / (FP32_NOMINAL_TFLOPS_PER_MHZ * (clocks.get("sm_mhz")
                                                                                            or 2070.0)),
                         "traffic": SWEEP_TRAFFIC_ICOS8 if args.nest == 8 else None,
                         "traffic_unit": "bytes per sweep launch: ncu dram__bytes_read.sum + dram__bytes_write.sum "
                                         "of one full-size launch (a recorded capture, not measured in this run)",
                         "pipes": dict(SWEEP_PIPES_ICOS7, source="ncu --set full of the same sweep kernel on this "
                                       "workload at icos nest 7 (sm__pipe_fma_cycles_active, "
                                       "sm__pipe_xu_cycles_active, smsp__issue_active; recorded, not this run)"),
                         "kernel": "bve_rel_sweep_kernel (+ its prep and finish kernels) per velocity sum",
                         "ms_per_launch": sum_ms, "flops_per_interaction": FLOPS_PER_INTERACTION,
                         "peak_source": "measured in-process FFMA loop (lpm_measure_fp32_peak); "
                                        "frac_of_nominal: 152 SMs x 128 lanes x 2 flops x the median SM clock"},
            "fp64_gpu": fp64,
            "ensemble": ens,
            "accuracy": {"velocity_rel_linf_vs_fp64_oracle": rel_linf, "velocity_rel_l2_vs_fp64_oracle": rel_l2,
                         "reference": "the oracle (the reference BVESphereVelocity loop restated in C, FP64) at "
                                      "the final state",
                         "targets": f"{ib}..{ib + m - 1}",
                         "circulation_drift": diag1["circulation"] - diag0["circulation"],
                         "ke_rel_drift": (diag1["kinetic_energy"] - diag0["kinetic_energy"]) / diag0["kinetic_energy"],
                         "steps_advanced": args.warmup + args.steps},
            "e2e": e2e,
            "cpu_baseline": cpu,
            "step_ms": step_ms,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


# ------------------------------------------------------------------ ensemble
def measure_ensemble(torch, lg, wl, n_instances, steps, warmup, dt, inst=None, check=8):
    """Config 5: `n_instances` independent sphere-BVE instances at seeded random icosahedral
    nests 3-6 (Gaussian vortices with random strength, width and centre, mean removed,
    Omega = 2 pi), FP32C, advanced `steps` RK4 steps (dt, projected stages) as one batch -- one
    persistent launch per stage over a flattened work queue, one CUDA graph per step -- and the
    same instances on separate solvers, one after another.  Both are timed by the host wall
    clock around the step loop, the device synchronised before and after (each step ends with
    a status check).  Returns a dict (Ginteractions/s, the ratio, accuracy against FP64)."""
    if inst is None:
        inst = wl.config_ensemble(n_instances=n_instances, seed=0)
    inter_eval = sum(int(d["x"].size) * int(d["active"].sum()) - int(d["active"].sum()) for d in inst)
    ens = lg.Ensemble(inst, mode="fp32c")
    shape = ens.sweep_shape()
    ens.timestep(dt, max(warmup, 3), renormalize=True)
    torch.cuda.synchronize()
    k0 = ens.kernel_timing()
    t0 = time.perf_counter()
    ens.timestep(dt, steps, renormalize=True)
    torch.cuda.synchronize()
    t_batch = time.perf_counter() - t0
    k1 = ens.kernel_timing()
    # per-instance velocity error of the batched FP32C sums against FP64 (up to `check`
    # instances, a block of up to 4096 targets each)
    st = ens.get_state()
    offs = ens.offsets
    errs = []
    for k in range(0, len(inst), max(1, len(inst) // max(check, 1))):
        a, b = int(offs[k]), int(offs[k + 1])
        d = inst[k]
        m = min(4096, b - a)
        sl = slice(a, b)
        ref = lg.bve_sphere_velocity(st["x"][sl], st["y"][sl], st["z"][sl], st["rel_vort"][sl], d["area"], d["active"],
                                     d["radius"], i_begin=1, i_end=m, mode="fp64")
        got = np.stack([st[c][a:a + m] for c in ("u", "v", "w")])
        r = np.stack([q[:m] for q in ref])
        errs.append(float(np.abs(got - r).max() / np.abs(r).max()))
    ens.close()
    solvers = [lg.BVESolver(d["x"], d["y"], d["z"], d["rel_vort"], d["area"], d["active"], d["radius"],
                            d["rotation_rate"], mode="fp32c") for d in inst]
    for s_ in solvers:
        s_.set_timing(False)
        s_.timestep(dt, max(warmup, 3), renormalize=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s_ in solvers:
        s_.timestep(dt, steps, renormalize=True)
    torch.cuda.synchronize()
    t_seq = time.perf_counter() - t0
    for s_ in solvers:
        s_.close()
    total = 4 * steps * inter_eval
    return {"value": total / t_batch / 1e9, "unit": UNIT, "steps": steps, "instances": len(inst),
            "nests": collections_counter([d["nest"] for d in inst]), "interactions_per_eval": inter_eval,
            "ms_per_step": 1e3 * t_batch / steps,
            "sequential": {"value": total / t_seq / 1e9, "unit": UNIT, "ms_per_step": 1e3 * t_seq / steps,
                           "how": "one BVESolver per instance, each replaying its step graph back to back"},
            "speedup_vs_sequential": t_seq / t_batch,
            "sweep_shape": {"threads": shape[0], "targets_per_thread": shape[1], "ctas_per_sm": shape[2],
                            "items_per_cta_slot": shape[3]},
            "sum_kernel_ms_per_step": (k1[0] - k0[0]) / steps,
            "gpu_launches": k1[1] - k0[1],
            "velocity_rel_linf_vs_fp64_max": max(errs), "instances_checked": len(errs),
            "timing": "host wall clock around the step loop, device synchronised before and after", "errs": errs}


def run_ensemble(args):
    """The 64-instance ensemble (config 5) as its own line, with the same measurement for each
    refinement level of the mix on its own (the per-size-class rates)."""
    import torch
    import lpm_gpu as lg
    import workloads as wl

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    steps = args.steps if args.steps != 5 else 50
    inst = wl.config_ensemble(n_instances=args.instances, seed=0)
    sampler = ClockSampler(gpu_id_for(torch, local))
    sampler.start()
    r = measure_ensemble(torch, lg, wl, args.instances, steps, args.warmup, args.dt, inst=inst)
    clocks = sampler.stop()
    classes = {}
    for nest in ([] if args.no_size_classes else sorted({d["nest"] for d in inst})):
        sub = [d for d in inst if d["nest"] == nest]
        q = measure_ensemble(torch, lg, wl, len(sub), max(2, steps // 5), args.warmup, args.dt, inst=sub, check=2)
        classes[str(nest)] = {"instances": len(sub), "batched": q["value"], "sequential": q["sequential"]["value"],
                              "speedup_vs_sequential": q["speedup_vs_sequential"], "sweep_shape": q["sweep_shape"],
                              "interactions_per_eval": q["interactions_per_eval"], "steps": q["steps"]}
    line = {
        "metric": "BVE ensemble Ginteractions/s (64 uneven instances, batched persistent launch)", "value": r["value"],
        "unit": UNIT, "n_gpus": 1, "steps": steps, "warmup": max(args.warmup, 3),
        "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{len(inst)} sphere-BVE instances, icosahedral nests {r['nests']}, Gaussian vortices "
                               "(shape U[2,8], strength U[2pi,6pi], random centre), dt 0.01, projected stages",
                   "interactions_per_eval": r["interactions_per_eval"], "timing": r["timing"]},
        "clocks": clocks,
        "sequential": r["sequential"],
        "speedup_vs_sequential": r["speedup_vs_sequential"],
        "sum_kernel_ms_per_step": r["sum_kernel_ms_per_step"],
        "sweep_shape": r["sweep_shape"],
        "gpu_launches": r["gpu_launches"],
        "accuracy": {"velocity_rel_linf_vs_fp64_max": r["velocity_rel_linf_vs_fp64_max"],
                     "instances_checked": r["instances_checked"]},
        "size_classes": classes,
    }
    print(json.dumps(line), flush=True)
    return 0


def run_stream(args):
    """The sphere stream functions (SetStreamFunctionsOnMesh, src/SphereBVE.f90:445-485: psi_rel
    and psi_abs, a log-kernel sum called once per reference time step) in LPM_MODE_FP32C
    through the host-buffer C ABI at icosahedral nest `--nest`, on the RK4 workload's
    initial state (absolute vorticity zeta + 2 Omega z / a).  Each step is one call, host
    copies included.  The FP64 mode of the same call is timed on a bounded block of targets,
    and the FP32C result is checked against it on that block."""
    import torch
    import lpm_gpu as lg

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    c, n, ns, per_sum = workload(args.nest)
    omega = 2.0 * np.pi
    absv = c["zeta"] + 2.0 * omega * c["z"]
    a = (c["x"], c["y"], c["z"], c["zeta"], absv, c["area"], c["active"], 1.0)
    for _ in range(max(args.warmup, 3)):
        lg.set_stream_functions_on_mesh(*a, mode="fp32c")
    sampler = ClockSampler(gpu_id_for(torch, local))
    sampler.start()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        pr, pa = lg.set_stream_functions_on_mesh(*a, mode="fp32c")
        times.append(time.perf_counter() - t0)
    clocks = sampler.stop()
    # FP64 on a block of 4096 targets in the middle of the particle range
    ib = n // 3 + 1
    m = 4096
    lg.set_stream_functions_on_mesh(*a, i_begin=ib, i_end=ib + 255, mode="fp64")
    t0 = time.perf_counter()
    r64, a64 = lg.set_stream_functions_on_mesh(*a, i_begin=ib, i_end=ib + m - 1, mode="fp64")
    t64 = time.perf_counter() - t0
    sl = slice(ib - 1, ib - 1 + m)
    err = max(float(np.abs(pr[sl] - r64[sl]).max() / np.abs(r64[sl]).max()),
              float(np.abs(pa[sl] - a64[sl]).max() / np.abs(a64[sl]).max()))
    t = sum(times) / len(times)
    value = per_sum / t / 1e9
    line = {
        "metric": "sphere stream functions Ginteractions/s (psi_rel and psi_abs), FP32C, host-buffer C ABI",
        "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 3),
        "ms_per_step": 1e3 * t, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": f"sphere stream functions, icosahedral nest {args.nest} ({n} targets, {ns} sources), "
                               "RH4 + Gaussian vortex", "interactions_per_call": per_sum,
                   "timing": "host wall clock around each lpm_bve_stream_functions call (H2D of the inputs, "
                             "prep, sweep, finish, D2H of psi_rel and psi_abs)"},
        "clocks": clocks,
        "fp64_same_call": {"value": m * ns / t64 / 1e9, "unit": UNIT, "targets": f"{ib}..{ib + m - 1}"},
        "accuracy": {"psi_rel_linf_vs_fp64": err, "targets": f"{ib}..{ib + m - 1}"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 6 * 8 * n + 4 * ns,
                "d2h_bytes_per_step": 2 * 8 * n},
        "gpu_launches": 4 * args.steps,
    }
    print(json.dumps(line), flush=True)
    return 0


def _best_time(fn, reps=3):
    fn()
    best = 1e300
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        best = min(best, time.perf_counter() - t0)
    return best


def run_configs(args):
    """The other configurations of the path, each timed on the GPU (FP64 parity mode and
    FP32C, through the host-buffer C ABI or the solver handle) and on the host cores (the
    oracle, a bounded block of targets where the full sum would take minutes):
      C1 sphere BVE, icos nest 4, 100 RK4 steps of dt 0.01 (Gaussian vortex, Omega = 2 pi);
      C2 planar velocity, quad nest 7 on [-4,4]^2, Lamb-dipole-like vortices, delta 0 and 0.02;
      C3 PSE sphere Laplacian, cubed sphere nest 7, K8-geodesic and Gaussian-chord kernels.
    Rates are Ginteractions/s; GPU times are host wall clock around the call (copies included)."""
    import torch
    import lpm_gpu as lg
    import workloads as wl
    from oracle import oracle as orc

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    out = {}
    cores = os.cpu_count() or 1
    # C1
    c = wl.config_gauss_vortex_icos(4)
    n, ns = c["x"].size, int(c["active"].sum())
    steps = 100
    per_step = 4 * (n * ns - ns)
    row = {"size": f"icos nest 4: {n} targets, {ns} sources", "interactions_per_step": per_step}
    u0 = lg.set_velocity_from_vorticity(c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"], 1.0)
    for mode in ("fp64", "fp32c"):
        s_ = lg.BVESolver(c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"], 1.0, c["omega"],
                          u0[0], u0[1], u0[2], mode=mode)
        s_.set_timing(False)
        s_.timestep(0.01, 3)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s_.timestep(0.01, steps)
        torch.cuda.synchronize()
        row[f"gpu_{mode}"] = steps * per_step / (time.perf_counter() - t0) / 1e9
        s_.close()
    t0 = time.perf_counter()
    orc.bve_timestep(c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"], u0[0], u0[1], u0[2], 1.0,
                     c["omega"], 0.01, 10)
    row["cpu_oracle"] = 10 * per_step / (time.perf_counter() - t0) / 1e9
    row["cpu_sample"] = "10 RK4 steps, all targets"
    out["C1_sphere_bve_rk4"] = row
    # C2
    c = wl.config_colliding_dipoles(7)
    n, ns = c["x"].size, int(c["active"].sum())
    per = n * ns - ns
    row = {"size": f"quad nest 7 on [-4,4]^2: {n} targets, {ns} sources", "interactions_per_eval": per}
    a = (c["x"], c["y"], c["omega"], c["area"], c["active"])
    m = 4096
    blk = (n // 3, n // 3 + m)
    for delta in (0.0, 0.02):
        for mode in ("fp64", "fp32c"):
            t = _best_time(lambda: lg.planar_incompressible_velocity(*a, delta, mode=mode))
            row[f"gpu_{mode}_delta{delta}"] = per / t / 1e9
        # FP32C velocity error against the oracle on a block of targets, relative to the
        # block's largest velocity
        u, v = lg.planar_incompressible_velocity(*a, delta, i_begin=blk[0] + 1, i_end=blk[1], mode="fp32c")
        ru, rv = orc.plane_velocity(*a, delta, ib=blk[0], ie=blk[1])
        err = max(np.abs(u[blk[0]:blk[1]] - ru).max(), np.abs(v[blk[0]:blk[1]] - rv).max())
        row[f"fp32c_velocity_rel_linf_delta{delta}"] = err / max(np.abs(ru).max(), np.abs(rv).max())
    t = _best_time(lambda: orc.plane_velocity(*a, 0.0, ib=blk[0], ie=blk[1]), reps=1)
    row["cpu_oracle"] = m * ns / t / 1e9
    row["cpu_sample"] = f"delta 0, {m} targets against all sources"
    # the configuration's run: RK4, dt 0.005, 200 steps, delta 0.02, FP32C, through the solver
    s_ = lg.PlaneSolver(*a, delta=0.02, mode="fp32c")
    d0 = s_.diagnostics()
    s_.timestep(0.005, 2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s_.timestep(0.005, 198)
    torch.cuda.synchronize()
    row["gpu_fp32c_rk4_200_steps"] = 198 * 4 * per / (time.perf_counter() - t0) / 1e9
    d1 = s_.diagnostics()
    s_.close()
    row["rk4_circulation_drift"] = d1["circulation"] - d0["circulation"]
    row["rk4_kinetic_energy_rel_drift"] = (d1["kinetic_energy"] - d0["kinetic_energy"]) / d0["kinetic_energy"]
    row["rk4"] = "200 RK4 steps of dt 0.005 (delta 0.02, FP32C solver): rate over the last 198, drifts over all 200"
    out["C2_planar_velocity"] = row
    # C3
    c = wl.config_pse_cubed(7)
    n, ns = c["x"].size, int(c["active"].sum())
    per = n * ns
    row = {"size": f"cubed sphere nest 7: {n} targets, {ns} sources", "interactions_per_eval": per}
    a = (c["x"], c["y"], c["z"], c["f"], c["area"], c["active"])
    exact = -30.0 * wl.y54(c["x"], c["y"], c["z"])  # the Laplacian of the smooth part of f
    for name, kern, eps in (("k8_geodesic", lg.PSE_K8_GEODESIC, c["eps_k8"]),
                            ("gauss_chord", lg.PSE_GAUSS_CHORD, c["eps_gauss"])):
        t = _best_time(lambda: lg.pse_sphere_laplacian_at_particles(*a, eps, 1.0, kern, mode="fp32c"))
        row[f"gpu_fp32c_{name}"] = per / t / 1e9
        t = _best_time(lambda: lg.pse_sphere_laplacian_at_particles(*a, eps, 1.0, kern, mode="fp64"), reps=1)
        row[f"gpu_fp64_{name}"] = per / t / 1e9
        l32 = lg.pse_sphere_laplacian_at_particles(*a, eps, 1.0, kern, mode="fp32c")
        l64 = lg.pse_sphere_laplacian_at_particles(*a, eps, 1.0, kern, mode="fp64")
        row[f"fp32c_rel_linf_vs_fp64_{name}"] = float(np.abs(l32 - l64).max() / np.abs(l64).max())
        row[f"fp64_rel_linf_vs_exact_{name}"] = float(np.abs(l64 - exact).max() / np.abs(exact).max())
        # the same sum on Y54 alone: the PSE discretisation error against the exact Laplacian
        y = (c["x"], c["y"], c["z"], wl.y54(c["x"], c["y"], c["z"]), c["area"], c["active"])
        ly = lg.pse_sphere_laplacian_at_particles(*y, eps, 1.0, kern, mode="fp32c")
        row[f"fp32c_rel_linf_vs_exact_noise_free_{name}"] = float(np.abs(ly - exact).max() / np.abs(exact).max())
        mc = 2048
        t = _best_time(lambda: orc.pse_laplacian(*a, eps, 1.0, kern, ib=n // 3, ie=n // 3 + mc), reps=1)
        row[f"cpu_oracle_{name}"] = mc * ns / t / 1e9
    row["gpu_fp64_sample"] = "every target, in curve order; source tiles beyond r = 7 skipped (all-pairs equivalent)"
    row["exact"] = ("-30 Y54 (the 1e-3 noise in f has no closed-form Laplacian, so the error against it includes "
                    "the PSE estimate of the noise's)")
    row["cpu_sample"] = "2048 targets against all sources"
    out["C3_pse_laplacian"] = row
    line = {"metric": "direct-sum Ginteractions/s per configuration (GPU FP64 / FP32C, CPU oracle)",
            "unit": UNIT, "cpu_cores": cores, "data": "synthetic", "configs": out}
    print(json.dumps(line), flush=True)
    return 0


def sum_oracle_call(kind, v):
    """The oracle restatement of --sum `kind` as f(ib, ie) on 0-based target blocks, from the
    arrays run_sum built (its locals `v`)."""
    from oracle import oracle as orc
    c = v.get("c")
    if kind == "bve":
        return lambda ib, ie: orc.bve_velocity(c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"], 1.0,
                                               ib=ib, ie=ie)
    if kind == "stream":
        return lambda ib, ie: orc.bve_stream(c["x"], c["y"], c["z"], c["zeta"], v["absv"], c["area"], c["active"],
                                             1.0, ib=ib, ie=ie)
    if kind == "plane_stream":
        return lambda ib, ie: orc.plane_stream(c["x"], c["y"], c["omega"], c["area"], c["active"], ib=ib, ie=ie)
    if kind == "plane":
        return lambda ib, ie: orc.plane_velocity(c["x"], c["y"], c["omega"], c["area"], c["active"], 0.0, ib=ib,
                                                 ie=ie)
    if kind == "swe_plane":
        return lambda ib, ie: orc.swe_plane_rhs(c["x"], c["y"], c["omega"], v["div"], v["sh"], c["area"],
                                                c["active"], v["eps"], ib=ib, ie=ie)
    if kind == "swe_sphere":
        return lambda ib, ie: orc.swe_sphere_rhs(c["x"], c["y"], c["z"], c["zeta"], v["div"], v["sh"], c["area"],
                                                 c["active"], 1.0, 1.0, v["eps"], ib=ib, ie=ie)
    if kind == "beta":
        return lambda ib, ie: orc.beta_plane_velocity(c["x"], c["y"], c["zeta"], c["area"], c["active"], ib=ib,
                                                      ie=ie)
    if kind == "beta_stream":
        return lambda ib, ie: orc.beta_plane_stream(c["x"], c["y"], c["zeta"], v["absv"], c["area"], c["active"],
                                                    ib=ib, ie=ie)
    if kind == "pse_plane_grad":
        m = v["m"]
        return lambda ib, ie: orc.pse_plane_gradient(m.x, m.y, v["f"], m.area, m.active, v["eps"], ib=ib, ie=ie)
    if kind == "pse_plane_second":
        m = v["m"]
        return lambda ib, ie: orc.pse_plane_second_partials(m.x, m.y, *v["g"], m.area, m.active, v["eps"], ib=ib,
                                                            ie=ie)
    if kind == "pse_plane_ddot":
        m = v["m"]
        return lambda ib, ie: orc.pse_plane_double_dot(m.x, m.y, *v["g"], m.area, m.active, v["eps"], ib=ib, ie=ie)
    if kind == "pse_sphere_ddot":
        return lambda ib, ie: orc.pse_sphere_double_dot(c["x"], c["y"], c["z"], *v["v"], c["area"], c["active"],
                                                        v["eps"], 1.0, ib=ib, ie=ie)
    if kind == "pse_interp":
        m, q = v["m"], v["q"]
        return lambda ib, ie: orc.pse_interpolate(m.x, m.y, None, v["f"], m.area, m.active, v["eps"], q[0][ib:ie],
                                                  q[1][ib:ie], None, 0)
    if kind == "pse_plane":
        m = v["m"]
        return lambda ib, ie: orc.pse_laplacian(m.x, m.y, None, v["f"], m.area, m.active, v["eps"], 1.0,
                                                orc.PSE_K8_CHORD, ib=ib, ie=ie)
    if kind == "pse_grad":
        return lambda ib, ie: orc.pse_sphere_gradient(c["x"], c["y"], c["z"], v["f"], c["area"], c["active"],
                                                      v["eps"], 1.0, ib=ib, ie=ie)
    if kind == "pse_div":
        vv = v["v"]
        return lambda ib, ie: orc.pse_sphere_divergence(c["x"], c["y"], c["z"], *vv, c["area"], c["active"],
                                                        v["eps"], 1.0, ib=ib, ie=ie)
    kern = orc.PSE_K8_GEODESIC if kind == "pse_k8" else orc.PSE_GAUSS_CHORD
    return lambda ib, ie: orc.pse_laplacian(c["x"], c["y"], c["z"], c["f"], c["area"], c["active"], v["eps"], 1.0,
                                            kern, ib=ib, ie=ie)


def sum_cpu_sample(ocall, n, ns, budget_s: float):
    """Times the oracle on a contiguous block of targets against all sources, sized to about
    budget_s seconds; the cpu_baseline object of a --workload sum line."""
    start, probe = n // 3, 32
    t0 = time.perf_counter()
    ocall(start, min(n, start + probe))
    dt = max(time.perf_counter() - t0, 1e-6)
    m = int(min(n - start, max(probe, probe * budget_s / dt)))
    t0 = time.perf_counter()
    ocall(start, start + m)
    el = time.perf_counter() - t0
    cores = os.cpu_count() or 1
    return {"value": m * ns / el / 1e9, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"oracle (OpenMP, {cores} threads), targets {start + 1}..{start + m} of {n} against all "
                      f"{ns} sources, {el:.1f} s"}


def run_sum(args):
    """One direct sum through its host-buffer C-ABI entry point, `steps` calls after `warmup`
    (a small, few-launch workload for profiling and per-row rates).  --nest is the refinement
    level of the sum's mesh: icosahedral for bve and stream, quad on [-4,4]^2 for plane (Lamb
    dipoles), cubed sphere for pse_* (Y54 plus noise; eps = h^0.75 for K8, 2 x mean edge for
    the Gaussian)."""
    import torch
    import lpm_gpu as lg
    import workloads as wl

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    mode = "fp64" if args.sum in FP64_ONLY_SUMS else args.mode
    if args.sum in ("bve", "stream"):
        c = wl.config_rh54_icos(args.nest, seed=0)
        n, ns = c["x"].size, int(c["active"].sum())
        absv = c["zeta"] + 4.0 * np.pi * c["z"]
        if args.sum == "bve":
            call = lambda ie: lg.bve_sphere_velocity(c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"], 1.0,
                                                     i_end=ie, mode=args.mode)
        else:
            call = lambda ie: lg.set_stream_functions_on_mesh(c["x"], c["y"], c["z"], c["zeta"], absv, c["area"],
                                                              c["active"], 1.0, i_end=ie, mode=args.mode)
        mesh = f"icosahedral nest {args.nest}"
    elif args.sum == "plane_stream":
        c = wl.config_colliding_dipoles(args.nest)
        n, ns = c["x"].size, int(c["active"].sum())
        call = lambda ie: lg.set_stream_function_on_mesh(c["x"], c["y"], c["omega"], c["area"], c["active"],
                                                         i_end=ie, mode=args.mode)
        mesh = f"quad nest {args.nest} on [-4,4]^2"
    elif args.sum == "swe_plane":
        c = wl.config_colliding_dipoles(args.nest)
        n, ns = c["x"].size, int(c["active"].sum())
        div = 0.2 * c["omega"] * np.exp(-(c["x"] ** 2))
        sh = 1.0 + 0.1 * np.cos(c["x"]) * np.sin(c["y"])
        eps = 2.0 * float(np.sqrt(c["area"][c["active"] == 1].max()))
        call = lambda ie: lg.swe_plane_rhs_integrals(c["x"], c["y"], c["omega"], div, sh, c["area"], c["active"],
                                                     eps, i_end=ie, mode=args.mode)
        mesh = f"quad nest {args.nest} on [-4,4]^2 (SWE velocity, double dot and surface Laplacian, eps = 2h)"
    elif args.sum == "swe_sphere":
        c = wl.config_rh54_icos(args.nest, seed=0)
        n, ns = c["x"].size, int(c["active"].sum())
        div = 0.1 * np.cos(3.0 * c["z"]) * np.sin(2.0 * c["x"])
        sh = 1.0 + 0.2 * c["z"]
        eps = 2.0 * float(np.sqrt(c["area"][c["active"] == 1].max()))
        call = lambda ie: lg.swe_sphere_rhs_integrals(c["x"], c["y"], c["z"], c["zeta"], div, sh, c["area"],
                                                      c["active"], 1.0, eps, 1.0, i_end=ie, mode=args.mode)
        mesh = f"icosahedral nest {args.nest} (RH54 vorticity, divergence, surface Laplacian, eps = 2h)"
    elif args.sum == "beta_stream":
        c = wl.config_beta_plane(args.nest)
        n, ns = c["x"].size, int(c["active"].sum())
        absv = c["zeta"] + 10.0 * c["y"]
        call = lambda ie: lg.beta_plane_stream_functions(c["x"], c["y"], c["zeta"], absv, c["area"], c["active"],
                                                         i_end=ie, mode=args.mode)
        mesh = f"beta-plane quad nest {args.nest} on [0,1]x[-1/2,1/2]"
    elif args.sum == "beta":
        c = wl.config_beta_plane(args.nest)
        n, ns = c["x"].size, int(c["active"].sum())
        call = lambda ie: lg.beta_plane_velocity(c["x"], c["y"], c["zeta"], c["area"], c["active"], i_end=ie,
                                                 mode=args.mode)
        mesh = f"beta-plane quad nest {args.nest} on [0,1]x[-1/2,1/2]"
    elif args.sum == "plane":
        c = wl.config_colliding_dipoles(args.nest)
        n, ns = c["x"].size, int(c["active"].sum())
        call = lambda ie: lg.planar_incompressible_velocity(c["x"], c["y"], c["omega"], c["area"], c["active"], 0.0,
                                                            i_end=ie, mode=args.mode)
        mesh = f"quad nest {args.nest} on [-4,4]^2"
    elif args.sum == "pse_plane":
        m = lg.PolyMesh2d(lg.QUAD_RECT_SEED, args.nest, 4.0)
        n, ns = m.n, int(m.active.sum())
        eps = m.max_edge_length ** 0.75
        f = np.exp(-(m.x * m.x + m.y * m.y)) * np.cos(2.0 * m.x)
        call = lambda ie: lg.pse_plane_laplacian_at_particles(m.x, m.y, f, m.area, m.active, eps, kernel=lg.PSE_K8_CHORD,
                                                              i_end=ie, mode=args.mode)
        mesh = f"quad nest {args.nest} on [-4,4]^2, K8 of the chord, eps {eps:.4g}"
    elif args.sum in ("pse_plane_grad", "pse_plane_second", "pse_plane_ddot", "pse_interp"):
        m = lg.PolyMesh2d(lg.QUAD_RECT_SEED, args.nest, 4.0)
        n, ns = m.n, int(m.active.sum())
        eps = m.max_edge_length ** 0.75
        f = np.exp(-(m.x * m.x + m.y * m.y)) * np.cos(2.0 * m.x)
        # a smooth velocity-like pair of fields (the gradient of f, in closed form)
        g = (np.exp(-(m.x * m.x + m.y * m.y)) * (-2.0 * m.x * np.cos(2.0 * m.x) - 2.0 * np.sin(2.0 * m.x)),
             np.exp(-(m.x * m.x + m.y * m.y)) * (-2.0 * m.y * np.cos(2.0 * m.x)))
        if args.sum == "pse_plane_grad":
            call = lambda ie: lg.pse_plane_gradient_at_particles(m.x, m.y, f, m.area, m.active, eps, i_end=ie,
                                                                 mode=mode)
        elif args.sum == "pse_plane_second":
            call = lambda ie: lg.pse_plane_second_partials_at_particles(m.x, m.y, *g, m.area, m.active, eps,
                                                                        i_end=ie, mode=mode)
        elif args.sum == "pse_plane_ddot":
            call = lambda ie: lg.pse_plane_double_dot_product_at_particles(m.x, m.y, *g, m.area, m.active, eps,
                                                                           i_end=ie, mode=mode)
        else:
            # query points: the particles shifted by a third of an edge (seeded), one per particle
            rng = np.random.default_rng(0)
            h = float(np.sqrt(m.area[m.active == 1].max()))
            q = (m.x + rng.uniform(-h / 3, h / 3, n), m.y + rng.uniform(-h / 3, h / 3, n))
            call = lambda ie: lg.pse_interpolate_scalar(m.x, m.y, None, f, m.area, m.active, eps, q[0][:ie],
                                                        q[1][:ie], geometry=lg.GEOMETRY_PLANE, mode=mode)
        mesh = f"quad nest {args.nest} on [-4,4]^2, K8 of the chord, eps {eps:.4g}"
    elif args.sum == "pse_sphere_ddot":
        c = wl.config_pse_cubed(args.nest)
        n, ns = c["x"].size, int(c["active"].sum())
        eps = c["eps_k8"]
        v = wl.y54_surface_gradient(c["x"], c["y"], c["z"])
        call = lambda ie: lg.pse_sphere_double_dot_product_at_particles(c["x"], c["y"], c["z"], *v, c["area"],
                                                                        c["active"], eps, 1.0, i_end=ie, mode=mode)
        mesh = f"cubed sphere nest {args.nest}, eps {eps:.4g} (the surface gradient of y54)"
    elif args.sum in ("pse_grad", "pse_div"):
        c = wl.config_pse_cubed(args.nest)
        n, ns = c["x"].size, int(c["active"].sum())
        eps = c["eps_k8"]
        f = wl.y54(c["x"], c["y"], c["z"])
        v = wl.y54_surface_gradient(c["x"], c["y"], c["z"])
        if args.sum == "pse_grad":
            call = lambda ie: lg.pse_sphere_gradient_at_particles(c["x"], c["y"], c["z"], f, c["area"], c["active"],
                                                                  eps, 1.0, i_end=ie, mode=args.mode)
        else:
            call = lambda ie: lg.pse_sphere_divergence_at_particles(c["x"], c["y"], c["z"], *v, c["area"],
                                                                    c["active"], eps, 1.0, i_end=ie, mode=args.mode)
        mesh = f"cubed sphere nest {args.nest}, eps {eps:.4g} (y54 and its gradient)"
    else:
        c = wl.config_pse_cubed(args.nest)
        n, ns = c["x"].size, int(c["active"].sum())
        kern = lg.PSE_K8_GEODESIC if args.sum == "pse_k8" else lg.PSE_GAUSS_CHORD
        eps = c["eps_k8"] if args.sum == "pse_k8" else c["eps_gauss"]
        call = lambda ie: lg.pse_sphere_laplacian_at_particles(c["x"], c["y"], c["z"], c["f"], c["area"],
                                                               c["active"], eps, 1.0, kern, i_end=ie, mode=args.mode)
        mesh = f"cubed sphere nest {args.nest}, eps {eps:.4g}"
    nt = n if args.targets <= 0 else min(args.targets, n)
    ocall = None if args.no_cpu_baseline else sum_oracle_call(args.sum, locals())
    for _ in range(max(args.warmup, 3)):
        call(nt)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        call(nt)
        times.append(time.perf_counter() - t0)
    t = min(times)
    line = {"metric": f"{args.sum} direct sum Ginteractions/s ({mode}, host-buffer C ABI)",
            "value": nt * ns / t / 1e9, "unit": UNIT, "steps": args.steps, "ms_per_step": 1e3 * t,
            "config": {"workload": f"{args.sum} on {mesh}: {nt} of {n} targets, {ns} sources",
                       "timing": "host wall clock around each call (copies included), best of the steps"}}
    if ocall is not None:
        line["cpu_baseline"] = sum_cpu_sample(ocall, n, ns, 3.0)
    print(json.dumps(line), flush=True)
    return 0


def collections_counter(values):
    out = {}
    for v in values:
        out[str(v)] = out.get(str(v), 0) + 1
    return out


def run_remesh(args):
    """Remesh without rebuilding the solver (lpm_bve_solver_remesh) against the reference's
    Delete + New of the solver per remesh (examples/BVESingleGaussianVortex.f90:218-246), in
    FP32C at icosahedral nest `--nest`.  The new particle set is the mesh's own (positions,
    vorticity, area, mask), loaded after the solver has advanced one step; both paths compute
    the new set's velocity (setVelocityFromVorticity), as New does.  Each timed pass is
    remesh (or create) followed by one RK4 step, synchronised."""
    import torch
    import lpm_gpu as lg

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    c, n, ns, per_sum = workload(args.nest)
    omega = 2.0 * np.pi
    new_set = (c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"])
    s = lg.BVESolver(*new_set, 1.0, omega, mode="fp32c")
    s.timestep(0.01)

    def via_remesh():
        s.remesh(*new_set)
        s.timestep(0.01)
        torch.cuda.synchronize()

    def via_create():
        t = lg.BVESolver(*new_set, 1.0, omega, mode="fp32c")
        t.timestep(0.01)
        torch.cuda.synchronize()
        t.close()

    for _ in range(max(args.warmup, 3)):
        via_remesh()
        via_create()
    tr, tc = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        via_remesh()
        tr.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        via_create()
        tc.append(time.perf_counter() - t0)
    r_ms, c_ms = 1e3 * min(tr), 1e3 * min(tc)
    line = {"metric": "remesh + one RK4 step, ms (FP32C)", "value": r_ms, "unit": "ms", "higher_is_better": False,
            "steps": args.steps, "rebuild_ms": c_ms, "rebuild_over_remesh": c_ms / r_ms,
            "config": {"workload": f"icosahedral nest {args.nest} ({n} particles, {ns} sources): remesh with the "
                                   f"mesh's own set, then one RK4 step (4 velocity sums), against destroy + "
                                   f"create + one step",
                       "timing": "host wall clock, synchronised, best of the steps"}}
    s.close()
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "ensemble":
        return run_ensemble(args)
    if args.workload == "stream":
        return run_stream(args)
    if args.workload == "configs":
        return run_configs(args)
    if args.workload == "sum":
        return run_sum(args)
    if args.workload == "remesh":
        return run_remesh(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
