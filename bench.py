#!/usr/bin/env python
"""Benchmark of the trace-sampling hot path at Hilbert dimension 55296.

Workload (one "step"): the single large radical pair (radical A = two 14N +
five 1H, radical B = one 14N + four 1H; anisotropic hyperfine tensors, tilted
0.05 mT field, J = 0.01 mT, axial D = -0.4 mT, kS = kT = 1/us), M = 512
random-phase sample vectors, Krylov dimension 30, dt = 1 ns, propagated over
a window of --window-ns (default 2000 ns = 2000 dt steps, the configuration's
whole 2 us window). A step is the whole hot path: device Hamiltonian build
(general builder) + batched propagation + sample average.

Metric: sample-steps/s = M * (dt steps per sample) / wall time.
  value  device-resident inputs (spc_trace_sampling_device)
  e2e    through the C ABI with host buffers (spc_build_h + spc_trace_sampling:
         host->device copy of the sample vectors and device->host copy of the
         populations inside the timed region)
--impl reference times the CPU oracle (C++ restatement of the Fortran
reference; the Fortran itself cannot be built here) on all host cores.
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

from spin_dynamics_gb300 import workloads as W  # noqa: E402

# The headline metric as named for this path; `value` is the plain (per-instance) trace
# sampling at dim 55296, `adjoint` / `batched_adjoint` the gradient legs, `accuracy` the
# |Delta Phi_S| check against the oracle on the first vectors of the timed set.
METRIC = "sample-steps/s at dim 55296: batched+adjoint vs plain on GB300 at |\u0394\u03a6S|\u22641e-10"

# DRAM traffic per k_spmm launch (dram__bytes_read.sum + dram__bytes_write.sum)
# from one ncu capture at 64 sample columns (409 MB = 33 MB of Hamiltonian +
# 376 MB that scales with the columns), scaled to the launch's column count.
SPMM_TRAFFIC_H = 33.2e6
SPMM_TRAFFIC_PER_COLUMN = (409.1e6 - 33.2e6) / 64


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=2)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--window-ns", type=float, default=2000.0)
    p.add_argument("--samples", type=int, default=512)
    p.add_argument("--krylov", type=int, default=30)
    p.add_argument("--method", default="auto", choices=["auto", "mgs", "lanczos"],
                   help="Krylov orthogonalisation: auto = Lanczos with MGS fallback when kS == kT")
    p.add_argument("--cpu-samples", type=int, default=0,
                   help="CPU sample size (0 = cores x max(1, 1200 / dt steps): one vector per core at 2 us)")
    p.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--e2e-steps", type=int, default=5,
                   help="steps of the end-to-end leg (at most --steps)")
    p.add_argument("--no-batch", action="store_true", help="skip the batched uneven-set leg")
    p.add_argument("--batch-pairs", type=int, default=256)
    p.add_argument("--batch-orient", type=int, default=64)
    p.add_argument("--batch-tiled-arm", action="store_true",
                   help="also time the per-instance calls kept on the tiled path")
    p.add_argument("--badj-pairs", type=int, default=16, help="pairs of the batched-adjoint leg")
    p.add_argument("--badj-orient", type=int, default=4, help="orientations of the batched-adjoint leg")
    p.add_argument("--batch-window-ns", type=float, default=20.0)
    p.add_argument("--batch-krylov", type=int, default=20)
    p.add_argument("--batch-sample-path", default="auto", choices=["auto", "on", "off"],
                   help="one-CTA-per-sample kernel for the batched call (per-instance calls keep auto)")
    p.add_argument("--no-adjoint", action="store_true", help="skip the adjoint-gradient leg")
    p.add_argument("--no-batch-adjoint", action="store_true", help="skip the batched-adjoint leg")
    p.add_argument("--batch-adjoint-window-ns", type=float, default=10.0)
    p.add_argument("--no-symmetry", action="store_true", help="skip the symmetry-block leg")
    p.add_argument("--no-small", action="store_true", help="skip the small-pair (dim 288) leg")
    p.add_argument("--sym-samples", type=int, default=32)
    p.add_argument("--sym-window-ns", type=float, default=4.0)
    p.add_argument("--sym-directions", type=int, default=2)
    p.add_argument("--no-sym-full-forward", dest="sym_full_forward", action="store_false",
                   help="skip the one-direction plain forward at M = 128 over 1 us")
    p.add_argument("--adjoint-samples", type=int, default=256)
    p.add_argument("--adjoint-window-ns", type=float, default=400.0,
                   help="adjoint window (400 ns = four segments of the 100-step checkpoint spacing)")
    p.add_argument("--adjoint-checkpoint", type=int, default=100)
    p.add_argument("--adjoint-quad", type=int, default=0,
                   help="Gauss-Legendre nodes per step (0 = the library's rule from the norm bound of H)")
    p.add_argument("--adjoint-krylov", type=int, default=30,
                   help="Krylov dimension of the stepwise model (one basis per dt step)")
    p.add_argument("--adjoint-variants", action="store_true",
                   help="also time memory-sized checkpoints, 5 and 8 nodes and m = 16 on a 20-step window")
    return p.parse_args()


def workload_name(args, M, m, tol) -> str:
    return (f"large pair dim 55296 (A: 2x14N+5x1H, B: 14N+4x1H), anisotropic hyperfine, tilted B 0.05 mT, "
            f"J 0.01 mT, D -0.4 mT; M={M}, m={m}, tol={tol:g}, dt 1 ns, window {args.window_ns:g} ns")


def workload(args):
    sysp, B = W.large_pair()
    sim = W.large_sim(M=args.samples, t_end_ns=args.window_ns)
    return sysp, B, sim


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in out.splitlines():
            if line.startswith("Model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


def oracle_csr(sysp, B):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    pyoracle.build()
    e1, e2 = sysp.e1, sysp.e2
    return pyoracle, pyoracle.build_h_general(e1.g_I, e1.A, e1.gammas, e2.g_I, e2.A, e2.gammas, B,
                                              sysp.J, sysp.D, sysp.kS, sysp.kT)


def timed_vectors(args, sysp, rank=0):
    """The headline's M random-phase vectors (rank's own set)."""
    return W.random_phase_samples(sysp.Z, args.samples, seed=7 + rank)


def cpu_sample_size(args, sim, threads):
    steps = int(round(sim.t_end / sim.dt))
    return args.cpu_samples or threads * max(1, round(1200 / steps))


def cpu_leg(args, sysp, B, sim, threads, zk):
    """Time the oracle (fast build) on a bounded sample of the same workload:
    the whole window on the first vectors of the timed set (one per core at
    2 us)."""
    pyoracle, (rp, col, val) = oracle_csr(sysp, B)
    steps = int(round(sim.t_end / sim.dt))
    ns = zk.shape[0]
    t0 = time.perf_counter()
    r = pyoracle.trace_sampling(rp, col, val, zk, sim.dt, sim.t_end, sim.N_krylov, sim.tol,
                                fast=True, threads=threads)
    el = time.perf_counter() - t0
    cpu_leg.last = r  # the oracle populations on these vectors, for the accuracy check
    return {"value": ns * steps / el, "unit": "sample-steps/s", "cores": threads, "kind": "port",
            "sample": f"{ns} samples (the first of the timed set) x {steps} dt steps of the same system "
                      f"(Krylov builds {int(r['n_builds'].sum())}), oracle -O3 native OpenMP, {el:.2f} s, "
                      f"CPU {cpu_model()}"}


def accuracy_check(sampler, method, sysp, B, sim, zk, ref_fast, threads):
    """GPU against the oracle on the first vectors of the timed set over the
    whole window (same system, m, tol), through the timed handle: in the
    headline's Krylov mode and in MGS. Beside them, the oracle's parity build
    (no FMA contraction) against its -O3 FMA build on the same vectors: the
    reference algorithm's own sensitivity to rounding over a long window."""
    from spin_dynamics_gb300.observables import Observables

    pyoracle, (rp, col, val) = oracle_csr(sysp, B)
    ref = pyoracle.trace_sampling(rp, col, val, zk, sim.dt, sim.t_end, sim.N_krylov, sim.tol,
                                  threads=threads)

    def obs(r):
        o = Observables(r["P_S"].copy(), r["P_T0"].copy(), r["P_Tp"].copy(), r["P_Tm"].copy())
        o.get_kinetics(sim.dt, sysp.kS, sysp.kT)
        return o

    def diff(a, b):
        return {"max_abs_dPhi_S": float(np.max(np.abs(a.Phi_S - b.Phi_S))),
                "max_abs_dP_S": float(np.max(np.abs(a.P_S - b.P_S))),
                "max_abs_dP_all": float(max(np.max(np.abs(getattr(a, k) - getattr(b, k)))
                                            for k in ("P_S", "P_T0", "P_Tp", "P_Tm")))}

    o_ref = obs(ref)
    lanczos = method in ("auto", "lanczos") and sysp.kS == sysp.kT
    modes = [("lanczos" if lanczos else "mgs", method)] + ([("mgs", "mgs")] if lanczos else [])
    out = {"samples": int(zk.shape[0]), "vectors": "the first of the timed set",
           "window_ns": round(sim.t_end / sim.dt), "bound": 1e-10, "bound_on": "Phi_S",
           "reference": "oracle parity build (C++ restatement of the Fortran path, no FMA contraction)"}
    try:
        for name, m in modes:
            sampler.set_krylov(m)
            sampler.build_h(sysp, B, "general")
            got = sampler.trace_sampling(zk, sim.dt, sim.t_end, sim.N_krylov, sim.tol)
            got.get_kinetics(sim.dt, sysp.kS, sysp.kT)
            d = diff(got, o_ref)
            d["lanczos_fallbacks"] = int(sampler.stats()["lanczos_fallbacks"])
            d["Phi_S"] = float(got.Phi_S[-1])
            out[name] = d
    finally:
        sampler.set_krylov(method)
    first = out[modes[0][0]]
    out.update(max_abs_dPhi_S=first["max_abs_dPhi_S"], max_abs_dP_S=first["max_abs_dP_S"],
               method=modes[0][0], Phi_S=first["Phi_S"],
               oracle_fast_vs_parity_build=diff(obs(ref_fast), o_ref))
    return out


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._th = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True,
                                     text=True, timeout=5).stdout.strip()
                if out:
                    self.rows.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._th = threading.Thread(target=self._run, daemon=True)
        self._th.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._th:
            self._th.join(timeout=6)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for i, n in enumerate(names):
                if len(r) > 5 + i and r[5 + i].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.rows)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def run_ours(args, rank, world, local_rank):
    import torch
    import torch.distributed as dist

    from spin_dynamics_gb300 import _native as nat
    from spin_dynamics_gb300.dynamics import TraceSampler, num_time_points

    torch.cuda.set_device(local_rank)
    sysp, B, sim = workload(args)
    M, m = sim.N_samples, sim.N_krylov
    T = num_time_points(sim.dt, sim.t_end)
    steps_per_sample = int(round(sim.t_end / sim.dt))
    sampler = TraceSampler(local_rank)
    sampler.set_krylov(args.method)
    zk_host = timed_vectors(args, sysp, rank)
    zk_dev = torch.from_numpy(zk_host).to(f"cuda:{local_rank}")
    out_dev = torch.empty(4 * T, dtype=torch.float64, device=f"cuda:{local_rank}")
    # one stream for the library's launches and the timing events
    stream = torch.cuda.Stream(f"cuda:{local_rank}")
    stream.wait_stream(torch.cuda.current_stream())
    torch.cuda.set_stream(stream)
    sampler.set_stream(stream.cuda_stream)

    def step_device():
        sampler.build_h(sysp, B, "general")
        sampler.trace_sampling_device(zk_dev.data_ptr(), M, sim.dt, sim.t_end, m, sim.tol,
                                      out_dev.data_ptr())

    def barrier():
        if world > 1:
            dist.barrier()

    for _ in range(args.warmup):
        step_device()
    torch.cuda.synchronize()
    # timed region: device-resident inputs, no per-launch timing (build
    # rounds of a repeating shape replay as CUDA graphs)
    launches = 0
    builds = 0
    fallbacks = 0
    barrier()
    torch.cuda.synchronize()
    with Clocks(local_rank) as clk:
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step_device()
            st = sampler.stats()
            launches += st["kernel_launches"] + 4  # + the Hamiltonian build kernels
            builds += st["krylov_builds"]
            fallbacks += st["lanczos_fallbacks"]
        e1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = e0.elapsed_time(e1) / args.steps
    # one more step with per-kernel-class CUDA events, for the kernel shares
    # and the roofline of the dominant kernel (not part of the timed steps)
    prof = {}
    import ctypes as C
    nat.check(nat.lib().spc_set_profiling(sampler.handle, 1))
    step_device()
    torch.cuda.synchronize()
    for k in range(nat.SPC_KERNEL_KINDS):
        a, n, f, b = C.c_double(), C.c_int64(), C.c_double(), C.c_double()
        nat.lib().spc_get_profile(sampler.handle, k, C.byref(a), C.byref(n), C.byref(f), C.byref(b))
        prof[nat.lib().spc_kernel_kind_name(k).decode()] = (a.value, n.value, f.value, b.value)
    nat.check(nat.lib().spc_set_profiling(sampler.handle, 0))
    if world > 1:
        t = torch.tensor([ms], device=f"cuda:{local_rank}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * M * steps_per_sample / (ms / 1e3)

    # e2e through the C ABI with host buffers (pinned), over at most
    # --e2e-steps of the timed steps
    e2e = None
    if not args.no_e2e:
        zk_pin = torch.from_numpy(zk_host).pin_memory()
        zk_np = zk_pin.numpy()
        step_host = lambda: (sampler.build_h(sysp, B, "general"),
                             sampler.trace_sampling(zk_np, sim.dt, sim.t_end, m, sim.tol))
        step_host()
        n_e2e = max(1, min(args.steps, args.e2e_steps))
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(n_e2e):
            res = step_host()[1]
        torch.cuda.synchronize()
        el = (time.perf_counter() - t0) / n_e2e
        if world > 1:
            t = torch.tensor([el], device=f"cuda:{local_rank}")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            el = float(t.item())
        e2e = {"value": world * M * steps_per_sample / el, "unit": "sample-steps/s",
               "h2d_bytes_per_step": int(zk_host.nbytes), "d2h_bytes_per_step": int(4 * T * 8),
               "ms_per_step": el * 1e3, "steps": n_e2e}
    # parity of the timed path: oracle on the first vectors of the timed set
    cpu = accuracy = None
    if rank == 0 and not args.no_cpu:
        threads = host_cores()
        zs = zk_host[:cpu_sample_size(args, sim, threads)]
        cpu = cpu_leg(args, sysp, B, sim, threads, zs)
        accuracy = accuracy_check(sampler, args.method, sysp, B, sim, zs, cpu_leg.last, threads)
    # each secondary leg runs on a handle of its own, released afterwards:
    # buffers a handle holds from an earlier leg would otherwise count against
    # the device memory a later call sizes itself by (checkpoint spacing and
    # node-state caching of the gradient, batch groups)
    sampler.close()
    torch.cuda.empty_cache()

    def leg(skip, fn, *a):
        # a failing secondary leg is recorded in the line, not fatal to it
        if skip:
            return None
        s = TraceSampler(local_rank)
        s.set_krylov(args.method)
        s.set_stream(stream.cuda_stream)
        try:
            return fn(args, s, *a)
        except Exception as e:  # noqa: BLE001
            import traceback
            traceback.print_exc()
            return {"error": f"{type(e).__name__}: {e}"}
        finally:
            torch.cuda.synchronize()
            s.close()
            torch.cuda.empty_cache()

    batched = leg(args.no_batch, batched_leg, local_rank)
    adjoint = leg(args.no_adjoint, adjoint_leg, value / world)
    batch_adjoint = leg(args.no_batch_adjoint, batched_adjoint_leg, local_rank)
    symmetry = leg(args.no_symmetry, symmetry_leg)
    small = leg(args.no_small, small_leg)
    fp64 = C.c_double()
    nat.check(nat.lib().spc_fp64_peak(local_rank, C.byref(fp64)))
    return dict(ms=ms, value=value, e2e=e2e, batched=batched, adjoint=adjoint, batch_adjoint=batch_adjoint,
                symmetry=symmetry, small=small, cpu=cpu, accuracy=accuracy,
                prof=prof, clocks=clk.summary(), launches=launches,
                builds=builds, fallbacks=fallbacks, fp64_peak=fp64.value * 1e12, M=M, steps_per_sample=steps_per_sample,
                sysp=sysp, B=B, sim=sim)


def fp64_peak(device):
    """FP64 FMA peak of the device in FLOP/s, from the library's DFMA probe."""
    import ctypes as C

    from spin_dynamics_gb300 import _native as nat
    v = C.c_double()
    nat.check(nat.lib().spc_fp64_peak(device, C.byref(v)))
    return v.value * 1e12


def batched_leg(args, sampler, local_rank):
    """The uneven set: pairs of dims 16..9216 x field orientations, every job
    with its own Hamiltonian and 32-256 samples (full size by default: 256
    pairs x 64 orientations). Times the batched calls (spc_build_h_batch +
    spc_trace_sampling_batch_device, split into consecutive job groups by
    device memory) against the same jobs as per-instance calls (spc_build_h +
    spc_trace_sampling_device). The FP64 operations the batched run issues,
    at the measured FP64 peak, bound how fast any schedule could run them:
    `ratio_bound_fp64` is the per-instance time over that minimum."""
    import torch

    from spin_dynamics_gb300.dynamics import batch_groups, device_memory, num_time_points, padded_samples

    pairs, dirs, systems, fields, zks = uneven_jobs(args.batch_pairs, args.batch_orient)
    Ms = [z.shape[0] for z in zks]
    dt = 1.0 * 176.08596 / 1000
    t_end = args.batch_window_ns * 176.08596 / 1000
    T = num_time_points(dt, t_end)
    # Krylov dimension by the autotuner (one tile of each of up to 64 evenly
    # spaced jobs, 10 ns), shared by both arms
    pick = list(range(0, len(zks), max(1, len(zks) // 64)))
    sampler.build_h_batch([systems[i] for i in pick], [fields[i] for i in pick], "general")
    m, tune_rates = sampler.autotune_krylov([zks[i] for i in pick], dt, 10 * dt, 1e-5,
                                            candidates=(12, 16, 20, 24, 30, 40))
    offs = np.cumsum([0] + [z.size for z in zks])
    zk_dev = torch.empty(int(offs[-1]), dtype=torch.complex128, device=f"cuda:{local_rank}")
    for k, z in enumerate(zks):  # job by job: no host copy of the whole set
        zk_dev[int(offs[k]):int(offs[k + 1])].copy_(torch.from_numpy(z.reshape(-1)))
    out_dev = torch.empty(len(zks) * 4 * T, dtype=torch.float64, device=f"cuda:{local_rank}")
    # consecutive job groups whose bases and states take at most half the
    # memory left free once the samples and results are resident
    free, _ = device_memory(local_rank)
    groups = batch_groups([4 * s.Z * padded_samples(M) for s, M in zip(systems, Ms)],
                          free * 0.5 / (16.0 * (m + 4)))
    stream = torch.cuda.current_stream()

    def per_instance(jobs=None):
        for k in (range(len(zks)) if jobs is None else jobs):
            sampler.build_h(systems[k], fields[k], "general")
            sampler.trace_sampling_device(zk_dev.data_ptr() + 16 * int(offs[k]), Ms[k], dt, t_end, m,
                                          1e-5, out_dev.data_ptr() + 8 * k * 4 * T)

    def batched():
        sampler.set_sample_path(args.batch_sample_path)
        try:
            for grp in groups:
                sampler.build_h_batch([systems[i] for i in grp], [fields[i] for i in grp], "general")
                sampler.trace_sampling_batch_device(zk_dev.data_ptr() + 16 * int(offs[grp[0]]),
                                                    [Ms[i] for i in grp], dt, t_end, m, 1e-5,
                                                    out_dev.data_ptr() + 8 * grp[0] * 4 * T)
        finally:
            sampler.set_sample_path("auto")

    def timed(fn):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3

    steps = int(round(t_end / dt))
    work = sum(Ms) * steps
    # first run of the leg: allocation and page-in, with per-kernel-class timing
    breakdown = profiled(sampler, batched)
    t_batch = timed(batched)
    per_instance(range(min(len(zks), 64)))  # warm-up of the per-instance calls
    t_single = timed(per_instance)
    out = {}
    if args.batch_tiled_arm:
        # the same per-instance calls kept on the tiled path (small jobs
        # otherwise take the one-CTA-per-sample kernel)
        sampler.set_sample_path("off")
        try:
            t_tiles = timed(per_instance)
        finally:
            sampler.set_sample_path("auto")
        out.update(per_instance_tiled_value=work / t_tiles, ratio_vs_tiled_per_instance=t_tiles / t_batch)
    t_build = timed(lambda: [sampler.build_h_batch([systems[i] for i in grp], [fields[i] for i in grp], "general")
                             for grp in groups])
    flops = sum(v["gflop"] for v in breakdown.values()) * 1e9
    peak = fp64_peak(local_rank)
    t_min = flops / peak
    dims = [4 * s.Z for s in systems]
    out.update({"value": work / t_batch, "per_instance_value": work / t_single,
                "ratio": t_single / t_batch, "ratio_bound_fp64": t_single / t_min,
                "fp64_issued_gflop": flops / 1e9, "fp64_peak_tflops": peak / 1e12,
                "fp64_frac_batched": t_min / t_batch, "fp64_frac_per_instance": t_min / t_single,
                "unit": "sample-steps/s", "jobs": len(zks),
                "pairs": len(pairs), "orientations": len(dirs), "dims": [min(dims), max(dims)],
                "samples": int(sum(Ms)), "dt_steps": steps, "krylov": m, "kernel_breakdown": breakdown,
                "seconds": t_batch, "build_seconds": t_build, "per_instance_seconds": t_single,
                "krylov_autotune_rates": tune_rates, "batches": len(groups),
                "workload": "uneven pairs (2-10 nuclei from 1H/14N, anisotropic) x Fibonacci-sphere "
                            "orientations at 0.05 mT, own Hamiltonian per job"})
    return out


def profiled(sampler, fn):
    """Run fn once with per-kernel-class CUDA-event timing on; returns
    {class: {ms, launches, tflops, gflop}} (an untimed run)."""
    import ctypes as C

    from spin_dynamics_gb300 import _native as nat
    nat.check(nat.lib().spc_set_profiling(sampler.handle, 1))
    fn()
    out = {}
    for k in range(nat.SPC_KERNEL_KINDS):
        a, n, f, b = C.c_double(), C.c_int64(), C.c_double(), C.c_double()
        nat.lib().spc_get_profile(sampler.handle, k, C.byref(a), C.byref(n), C.byref(f), C.byref(b))
        if n.value:
            out[nat.lib().spc_kernel_kind_name(k).decode()] = {
                "ms": round(a.value, 3), "launches": n.value, "gflop": round(f.value / 1e9, 3),
                "tflops": round(f.value / (a.value / 1e3) / 1e12, 4) if a.value else None}
    nat.check(nat.lib().spc_set_profiling(sampler.handle, 0))
    return out


def uneven_jobs(n_pairs, n_orient):
    pairs = W.uneven_pairs(n_pairs)
    dirs = W.fibonacci_sphere(n_orient)
    systems, fields, zks = [], [], []
    for p, (s, M) in enumerate(pairs):
        z = W.random_phase_samples(s.Z, M, seed=100 + p)  # shared by the pair's orientations
        for d in dirs:
            systems.append(s)
            fields.append(d)
            zks.append(z)
    return pairs, dirs, systems, fields, zks


def batched_adjoint_leg(args, sampler, local_rank):
    """Yields and full gradients of every job of the uneven set (pairs x
    orientations) in one spc_yield_gradient_batch call, against one
    spc_yield_gradient call per job and against the plain per-instance
    forward (spc_build_h + spc_trace_sampling, Krylov reuse) of the same
    jobs over the same window. Host vectors in, results out, in every arm."""
    import torch

    pairs, dirs, systems, fields, zks = uneven_jobs(args.badj_pairs, args.badj_orient)
    dt = 1.0 * 176.08596 / 1000
    t_end = args.batch_adjoint_window_ns * 176.08596 / 1000
    m = args.batch_krylov

    def batched():
        return sampler.yield_gradient_batch(systems, fields, zks, dt, t_end, m, n_quad=args.adjoint_quad)

    def per_instance():
        return [sampler.yield_gradient(s, f, z, dt, t_end, m, n_quad=args.adjoint_quad)
                for s, f, z in zip(systems, fields, zks)]

    def plain():
        out = []
        for s, f, z in zip(systems, fields, zks):
            sampler.build_h(s, f, "general")
            out.append(sampler.trace_sampling(z, dt, t_end, m, 1e-5))
        return out

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return r, time.perf_counter() - t0

    gb, t_b = timed(batched)
    st = sampler.stats()
    gi, t_i = timed(per_instance)
    _, t_p = timed(plain)
    steps = st["sample_steps"] // sum(z.shape[0] for z in zks)
    work = sum(z.shape[0] for z in zks) * steps
    dev = max(float(np.max(np.abs(a.raw - b.raw)) / max(np.max(np.abs(b.raw)), 1e-300)) for a, b in zip(gb, gi))
    dims = [4 * s.Z for s in systems]
    return {"value": work / t_b, "unit": "sample-steps/s", "seconds": t_b,
            "per_instance_adjoint_value": work / t_i, "ratio_vs_per_instance_adjoint": t_i / t_b,
            "plain_per_instance_value": work / t_p, "cost_vs_plain_per_instance": t_b / t_p,
            "max_rel_diff_vs_per_instance": dev, "jobs": len(zks), "pairs": len(pairs),
            "orientations": len(dirs), "dims": [min(dims), max(dims)],
            "samples": int(sum(z.shape[0] for z in zks)), "dt_steps": int(steps), "krylov": m,
            "params_per_job": [int(min(g.raw.size for g in gb)), int(max(g.raw.size for g in gb))],
            "workload": "uneven pairs x orientations: Phi_S and dPhi_S/d(B, J, D, kS, kT, every "
                        "hyperfine element) per job"}


def small_leg(args, sampler):
    """The small pair (dim 288: A = 1H, 1H, 14N; B = 14N, 1H; isotropic,
    B = 0.05 mT along z), M = 64, 5 us at dt = 1 ns, m = 20, tol 1e-5 - the
    workload the reference runs on CPU - through spc_build_h +
    spc_trace_sampling (host vectors in, populations out), against the oracle
    on all host cores on the same vectors."""
    import torch

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    sysp, sim = W.small_pair(), W.small_sim(M=64, t_end_ns=5000.0)
    zk = W.random_phase_samples(sysp.Z, sim.N_samples, seed=21)
    steps = int(round(sim.t_end / sim.dt))

    def gpu():
        sampler.build_h(sysp, 0.05, "reference")
        return sampler.trace_sampling(zk, sim.dt, sim.t_end, sim.N_krylov, sim.tol)

    breakdown = profiled(sampler, gpu)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    got = gpu()
    torch.cuda.synchronize()
    t_gpu = time.perf_counter() - t0
    st = sampler.stats()
    pyoracle.build()
    e1, e2 = sysp.e1, sysp.e2
    rp, col, val = pyoracle.build_h_iso(e1.g_I, e1.a_iso, e2.g_I, e2.a_iso, 0.05, sysp.J, sysp.D, sysp.kS,
                                        sysp.kT)
    threads = host_cores()
    t0 = time.perf_counter()
    ref = pyoracle.trace_sampling(rp, col, val, zk, sim.dt, sim.t_end, sim.N_krylov, sim.tol, fast=True,
                                  threads=threads)
    t_cpu = time.perf_counter() - t0
    work = sim.N_samples * steps
    return {"value": work / t_gpu, "unit": "sample-steps/s", "seconds": t_gpu, "rounds": int(st["rounds"]),
            "kernel_launches": int(st["kernel_launches"]), "cpu_value": work / t_cpu, "cpu_cores": threads,
            "max_abs_dP_S_vs_oracle": float(np.max(np.abs(got.P_S - ref["P_S"]))), "kernel_breakdown": breakdown,
            "workload": "small pair dim 288 (isotropic), M=64, 5 us at dt 1 ns, m=20, tol 1e-5"}


def symmetry_leg(args, sampler):
    """The symmetry-reduced large system (full dim 37,748,736 -> 243 total-spin
    blocks of dims 36..112,500): Phi_S and dPhi_S/d(field direction) for
    --sym-directions Fibonacci-sphere directions at 0.05 mT, every (block,
    direction) job in one batched adjoint sweep (split only by device memory),
    against the plain batched forward of the same blocks (Krylov reuse) for
    the first direction. Bounded window and samples per block for the
    gradient, with the configuration's full map (32 directions, M = 128, 1 us)
    projected from its measured rate; the plain forward also runs at the
    configuration's own size for one direction."""
    import torch

    from spin_dynamics_gb300 import symmetry as S
    from spin_dynamics_gb300.dynamics import num_time_points
    from spin_dynamics_gb300.spinsys import SimParam

    sysp = W.symmetric_large_pair()
    sim = SimParam.from_input_units(type="symmetry_dynamics", B=[0.05], init_state="singlet", seed=(42, 99),
                                    N_samples=args.sym_samples, t_end_ns=args.sym_window_ns, dt_ns=1.0,
                                    N_krylov=args.batch_krylov, tol=1e-5, M1=3, M2=2, block_tol=0.0)
    dirs = W.fibonacci_sphere(args.sym_directions, 1.0)
    bl = S.blocks(sysp, 3, 2)
    dims = [4 * Zb for _, _, Zb in bl]

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return r, time.perf_counter() - t0

    g, t_g = timed(lambda: S.symmetrised_yield_gradient(sysp, sim, [0, 0, 0.05], sampler=sampler,
                                                        directions=dirs, n_quad=args.adjoint_quad))
    # the stepwise forward the gradient differentiates, same jobs, yields only
    y, t_f = timed(lambda: S.symmetrised_yield_gradient(sysp, sim, [0, 0, 0.05], sampler=sampler,
                                                        directions=dirs, n_quad=args.adjoint_quad,
                                                        gradient=False))
    _, t_p = timed(lambda: S.symmetrised_dynamics(sysp, sim, sampler=sampler, field=0.05 * dirs[0]))
    work_g = len(bl) * args.sym_samples * len(dirs)
    T_steps = 2 * (num_time_points(sim.dt, sim.t_end) // 2) - 2  # steps of the Simpson grid
    # the configuration's own size for one direction, plain forward: M = 128
    # per block over the whole 1 us window (Krylov reuse, batched blocks)
    full = None
    if args.sym_full_forward:
        sim_f = SimParam.from_input_units(type="symmetry_dynamics", B=[0.05], init_state="singlet",
                                          seed=(42, 99), N_samples=128, t_end_ns=1000.0, dt_ns=1.0,
                                          N_krylov=args.batch_krylov, tol=1e-5, M1=3, M2=2, block_tol=0.0)
        r_f, t_full = timed(lambda: S.symmetrised_dynamics(sysp, sim_f, sampler=sampler, field=0.05 * dirs[0]))
        r_f.get_kinetics(sim_f.dt, sysp.kS, sysp.kT)
        full = {"value": len(bl) * 128 * 1000 / t_full, "seconds": t_full, "samples_per_block": 128,
                "dt_steps": 1000, "directions": 1, "Phi_S": float(r_f.Phi_S[-1]),
                "workload": "all blocks, M = 128 per block, 1 us at dt 1 ns, one direction, plain forward"}
    # the configuration's full gradient map (32 directions, M = 128 per
    # block, 1000 steps) at the bounded leg's measured gradient rate
    work_cfg = len(bl) * 128 * 1000 * 32
    return {"value": work_g * T_steps / t_g, "unit": "sample-steps/s", "seconds": t_g,
            "stepwise_forward_value": work_g * T_steps / t_f, "cost_vs_stepwise_forward": t_g / t_f,
            "max_abs_dPhi_S_gradient_vs_forward_sweep": float(max(abs(a["Phi_S"] - b["Phi_S"]) for a, b in zip(g, y))),
            "plain_batched_forward_value": len(bl) * args.sym_samples * int(round(sim.t_end / sim.dt)) / t_p,
            "blocks": len(bl), "block_dims": [min(dims), max(dims)], "sum_block_dims": int(sum(dims)),
            "full_dim": int(4 * sysp.Z), "samples_per_block": args.sym_samples, "directions": len(dirs),
            "dt_steps": T_steps, "krylov": args.batch_krylov,
            "Phi_S": [d["Phi_S"] for d in g], "dPhi_S_dtheta": [d["dtheta"] for d in g],
            "dPhi_S_dphi": [d["dphi"] for d in g],
            "full_forward_one_direction": full,
            "full_config_gradient_map": {"sample_steps": work_cfg, "directions": 32, "samples_per_block": 128,
                                         "dt_steps": 1000,
                                         "projected_seconds_at_measured_gradient_rate": work_cfg / (work_g * T_steps / t_g)},
            "workload": "symmetry-reduced large pair (14N + 3x4 equivalent 1H | 14N + 2x4 equivalent 1H), "
                        "compass directions at 0.05 mT, batched + adjoint"}


def adjoint_leg(args, sampler, plain_value):
    """Yields and their gradient with respect to all 15 + 9*12 parameters of
    the large pair (spc_yield_gradient, host sample vectors in, gradient out)
    at the adjoint configuration's settings (M = 256, m = 30, checkpoints
    every 100 steps) over --adjoint-window-ns, against the stepwise forward it
    differentiates and the plain Krylov-reuse forward of the headline.

    Projection to the 2000-step window: the gradient runs N forward steps,
    N - K recomputed ones (every segment but the last) and N backward steps
    (costate build, node states, contractions), the stepwise forward N
    steps. With a forward step costing f and a backward step c, the cost
    ratio is (2N - K) f / (N f) + c / f, so from a window of N1 steps to
    N2 = 2000 it grows by (N2 - K)/N2 - (N1 - K)/N1."""
    import torch

    from spin_dynamics_gb300.dynamics import gradient_nodes

    sysp, B = W.large_pair()
    dt = 1.0 * 176.08596 / 1000
    t_end = args.adjoint_window_ns * 176.08596 / 1000
    M, m, K = args.adjoint_samples, args.adjoint_krylov, args.adjoint_checkpoint
    nq = args.adjoint_quad or gradient_nodes(sysp, B, dt)
    zk = W.random_phase_samples(sysp.Z, M, seed=11)
    method = "lanczos" if args.method in ("auto", "lanczos") and sysp.kS == sysp.kT else "mgs"

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return r, time.perf_counter() - t0

    sampler.set_krylov(method)
    out = {}
    try:
        # untimed short run (allocation, page-in) with per-kernel-class timing
        breakdown = profiled(sampler, lambda: sampler.yield_gradient(sysp, B, zk, dt, 20 * dt, m, n_quad=nq,
                                                                     checkpoint_every=10))
        g, t_grad = timed(lambda: sampler.yield_gradient(sysp, B, zk, dt, t_end, m, n_quad=nq,
                                                         checkpoint_every=K))
        st = sampler.stats()
        y, t_fwd = timed(lambda: sampler.stepwise_yields(sysp, B, zk, dt, t_end, m))
        steps = st["sample_steps"] // M
        cost = t_grad / t_fwd
        n2 = 2000
        proj = cost + (n2 - K) / n2 - (steps - K) / steps if steps > K else None
        if args.adjoint_variants:
            # 20-step window: memory-sized checkpoints, 5 and 8 nodes, m = 16 vs m = 30
            t20 = 20 * dt
            _, t_f20 = timed(lambda: sampler.stepwise_yields(sysp, B, zk, dt, t20, m))
            gq, t_q = timed(lambda: sampler.yield_gradient(sysp, B, zk, dt, t20, m, n_quad=nq, checkpoint_every=0))
            g5, t_5 = timed(lambda: sampler.yield_gradient(sysp, B, zk, dt, t20, m, n_quad=5, checkpoint_every=0))
            g8 = sampler.yield_gradient(sysp, B, zk, dt, t20, m, n_quad=8, checkpoint_every=0)
            gs = float(np.max(np.abs(g8.raw)))
            y16 = sampler.stepwise_yields(sysp, B, zk, dt, t20, 16)
            y30 = sampler.stepwise_yields(sysp, B, zk, dt, t20, 30)
            out["variants_20_steps"] = {
                "cost_vs_stepwise_forward_memory_sized": t_q / t_f20,
                "cost_vs_stepwise_forward_memory_sized_5_nodes": t_5 / t_f20,
                "grad_max_rel_diff_vs_8_nodes": {str(nq): float(np.max(np.abs(gq.raw - g8.raw))) / gs,
                                                 "5": float(np.max(np.abs(g5.raw - g8.raw))) / gs},
                "abs_dPhi_S_m16_vs_m30": abs(y16[0] - y30[0])}
    finally:
        sampler.set_krylov(args.method)
    work = M * steps
    out.update({"value": work / t_grad, "unit": "sample-steps/s", "seconds": t_grad,
                "stepwise_forward_value": work / t_fwd, "stepwise_forward_seconds": t_fwd,
                "cost_vs_stepwise_forward": cost,
                "projected_cost_vs_stepwise_forward_2000_steps": proj,
                "cost_vs_plain_forward": t_grad / (work / plain_value),
                "params": int(g.raw.size), "samples": M, "dt_steps": int(steps), "krylov": m,
                "krylov_method": method, "quadrature_nodes": nq,
                "quadrature_nodes_rule": "smallest n with Gauss-Legendre remainder bound <= 1e-8 at the norm "
                                         "bound of H_eff" if not args.adjoint_quad else "fixed",
                "checkpoint_every": K, "segments": -(-int(steps) // K),
                "node_states_kept": bool(st["rounds"]),
                "krylov_builds_per_sample_step": st["krylov_builds"] / max(1, work),
                "kernel_launches": int(st["kernel_launches"]),
                "Phi_S": g.Phi_S, "Phi_S_forward_only": y[0], "abs_dPhi_S_gradient_vs_forward": abs(g.Phi_S - y[0]),
                "kernel_breakdown_20_steps": breakdown,
                "workload": "large pair dim 55296 (anisotropic), gradient of Phi_S over B, J, D, kS, kT "
                            "and every hyperfine tensor element; h2d of the sample vectors inside"})
    return out


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    base = {"metric": METRIC, "unit": "sample-steps/s", "higher_is_better": True,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "vs_baseline": None,
            "dtype": "c128 (complex FP64)", "data": "synthetic (seeded system and random-phase vectors)"}
    if args.impl == "reference":
        if rank != 0:
            return
        sysp, B, sim = workload(args)
        threads = host_cores()
        zs = timed_vectors(args, sysp)[:cpu_sample_size(args, sim, threads)]
        vals = []
        for _ in range(max(1, args.warmup // 3)):
            cpu_leg(args, sysp, B, sim, threads, zs)  # warm-up (page-in, OpenMP pool)
        for _ in range(args.steps):
            vals.append(cpu_leg(args, sysp, B, sim, threads, zs))
        v = float(np.median([x["value"] for x in vals]))
        cb = dict(vals[0])
        cb["value"] = v
        line = dict(base, impl="reference", value=v, ms_per_step=None, scaling="weak",
                    config={"workload": workload_name(args, sim.N_samples, sim.N_krylov, sim.tol),
                            "samples_per_step": cb["sample"]},
                    cpu_baseline=cb,
                    e2e={"value": v, "unit": "sample-steps/s", "h2d_bytes_per_step": 0,
                         "d2h_bytes_per_step": 0})
        print(json.dumps(line))
        return

    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    r = run_ours(args, rank, world, local_rank)
    if rank != 0:
        return
    peaks, peak_src = measured_peaks()
    prof = r["prof"]
    dom = max(prof, key=lambda k: prof[k][0])
    ms_tot, nl, fl, by = prof[dom]
    avg_s = ms_tot / max(nl, 1) / 1e3
    ach_gbs = (by / max(nl, 1)) / avg_s / 1e9 if nl else None
    ach_tf = (fl / max(nl, 1)) / avg_s / 1e12 if nl else None
    cpu, accuracy = r["cpu"], r["accuracy"]
    share = {k: round(v[0] / max(1e-9, sum(x[0] for x in prof.values())), 4) for k, v in prof.items()}
    line = dict(base, value=r["value"], ms_per_step=r["ms"], scaling="weak",
                config={"workload": workload_name(args, r["M"], r["sim"].N_krylov, r["sim"].tol),
                        "samples": r["M"], "dt_steps_per_sample": r["steps_per_sample"],
                        "krylov_builds_per_step": r["builds"] / args.steps,
                        "krylov_method": args.method,
                        "lanczos_fallbacks_per_step": r["fallbacks"] / args.steps,
                        "l2": "inputs larger than L2 (Krylov basis 13.6 GB per build)",
                        "parallelism": f"replicas x{args.gpus}"},
                e2e=r["e2e"], gpu_launches=int(r["launches"]), clocks=r["clocks"],
                roofline={"kernel": dom, "bound": "hbm", "achieved": ach_gbs,
                          "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                          "frac": (ach_gbs / peaks["hbm_gbs"]) if ach_gbs else None,
                          "traffic": (SPMM_TRAFFIC_H + SPMM_TRAFFIC_PER_COLUMN * r["M"])
                          if dom == "spmm" else None,
                          "algorithmic_bytes": (by / max(nl, 1)) if nl else None,
                          "peak_source": peak_src,
                          "fp64": {"achieved_tflops": ach_tf, "peak_tflops": r["fp64_peak"] / 1e12,
                                   "frac": (ach_tf * 1e12 / r["fp64_peak"]) if ach_tf else None,
                                   "peak_source": "measured DFMA probe (spc_fp64_peak)"}},
                kernel_share=share, batched=r["batched"], adjoint=r["adjoint"],
                batched_adjoint=r["batch_adjoint"], symmetry=r["symmetry"], small=r["small"], cpu_baseline=cpu,
                accuracy=accuracy)
    print(json.dumps(line))


if __name__ == "__main__":
    main()
