#!/usr/bin/env python
"""Benchmark of the 2D GPE RK4 stepper (grid-point-steps/s).

Workload (default): 1024^2 periodic box, plain FP64, i dpsi/dt = -1/2 lap psi
+ g|psi|^2 psi - mu psi (g = rho0 = mu = 1), 64 seeded vortices with minimum
separation 4*sqrt(2)*dx, RK4 at dt = 5e-4.  One bench step = SUBSTEPS RK4 steps
(vk_gpe_rk4(ctx, SUBSTEPS)); metric = N^2 * RK4 steps / second.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]

With N > 1 (torchrun) every rank steps its own independent field (replicas:
a single field does not shard), value = all ranks' grid-point-steps / the
slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "RK4 grid-pt-steps/s at 1024^2"
UNIT = "grid-pt-steps/s"
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0
# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the
# FP64 1024^2 passes, recorded from one earlier ncu capture of this workload
# with the bulk row loads (not measured by this script: ncu is not run here)
RECORDED_DRAM_BYTES_1024_FP64 = {"k_x1": 11421952 + 0, "k_x2": 22499328 + 3072, "k_y2_rk4": 44822784 + 64768, "k_y1": 5660416 + 256}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=1024)
    ap.add_argument("--substeps", type=int, default=20)
    ap.add_argument("--no-fp32", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-ensemble", action="store_true")
    ap.add_argument("--no-4096", action="store_true")
    ap.add_argument("--no-argle", action="store_true")
    ap.add_argument("--no-particles", action="store_true")
    ap.add_argument("--no-warmstart", action="store_true")
    return ap.parse_args()


def replica_throughput(ms_local, world, points, S, K, dist=None, device="cpu"):
    """Whole-job throughput of `world` independent replicas: all ranks'
    grid-point steps (points x S RK4 steps x K bench steps each) over the
    slowest rank's time, the MAX over ranks of the per-rank milliseconds.
    Returns (value, ms_max)."""
    import torch
    t = torch.tensor([float(ms_local)], dtype=torch.float64, device=device)
    if dist is not None and world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms_max = float(t.item())
    return world * points * S * K / (ms_max * 1e-3), ms_max


def workload(n, seed):
    from quantumvortices_gb300 import vk
    dx = 2 * math.pi / n
    psi0, _ = vk.ic_vortices(n, n, 64, seed=seed, min_sep=4 * math.sqrt(2) * dx)
    return psi0


def hbm_peak():
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


# ------------------------------------------------------------- clocks --

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------- per-kernel bytes --

def kernel_bytes(tag, n, K, e, disk, stage=None):
    """Bytes one launch of `tag` must move (its own loads + stores) at grid n^2,
    element size e, K = largest kept |k|, disk = # modes with k^2 <= k2max."""
    rows_half, rows_full = K + 1, 2 * K + 1
    if tag == "k_x1":      # Ta (kept columns) in, psi out, rho x-spectrum (kx <= K) out
        return e * (n * rows_full + n * n + n * rows_half)
    if tag == "k_y1":      # Tb in, Tc out
        return e * (2 * n * rows_half)
    if tag == "k_x2":      # Tc in, psi in, Td (kept columns) out
        return e * (n * rows_half + n * n + n * rows_full)
    if tag == "k_y2_rk4":  # Td in; kpsi,str1,str2 in (disk); kpsi out (rows), str2 out (disk), Ta out
        return e * (n * rows_full + 3 * disk + n * rows_full + disk + n * rows_full)
    if tag == "k_xinv":
        return e * (n * rows_full + n * n)
    return None


def kernel_flops(tag, n, K):
    """Nominal FP64 flops of one launch (5 L log2 L per L-point complex FFT;
    the pointwise work is a few flops per point and left out)."""
    f = 5.0 * n * math.log2(n)
    rows = {"k_x1": 1.5 * n, "k_y1": 2.0 * (K + 1), "k_x2": 1.5 * n, "k_y2_rk4": 2.0 * (2 * K + 1),
            "k_xinv": float(n)}.get(tag)
    return None if rows is None else rows * f


def precision_errors(d32, d64):
    """FP32-bulk diagnostics against the FP64 path's (same state, same steps)."""
    return {"rel_err_energy": abs(d32.etot - d64.etot) / abs(d64.etot),
            "rel_err_norm": abs(d32.norm - d64.norm) / abs(d64.norm),
            "rel_l2_err_spectra": float(np.linalg.norm(d32.spec - d64.spec) / np.linalg.norm(d64.spec))}


def fp64_peak_tflops(torch):
    """FP64 throughput of cuBLAS DGEMM (4096^3) on this GPU, TFLOP/s."""
    a = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    b = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(5):
        torch.matmul(a, b)
    e1.record()
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 5 * 1e-3
    del a, b
    return 2.0 * 4096 ** 3 / t / 1e12


def ensemble_bench(torch, K, W, S):
    """192 fields at 256^2 and 48 at 512^2 (16-64 seeded vortices each), FP32
    bulk, stepped together: one CUDA graph per RK4 step.  Two members are
    compared with single-field FP64 runs from the same state after 100 steps."""
    from quantumvortices_gb300 import vk
    sizes = [256] * 192 + [512] * 48
    rng = np.random.default_rng(7)
    ens = vk.Ensemble([vk.params_for(n, dt=5e-4, precision=vk.VK_PREC_FP32) for n in sizes])
    init = []
    for m, n in enumerate(sizes):
        nv = 2 * int(rng.integers(8, 33))
        psi, _ = vk.ic_vortices(n, n, nv, seed=2000 + m, min_sep=4 * math.sqrt(2) * 2 * math.pi / n)
        ens.set_psi(m, psi)
        if m in (0, 192):
            init.append((m, n, psi))
    ext = torch.cuda.ExternalStream(ens.stream)
    for _ in range(W):
        ens.gpe_rk4(S)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = ens.launches
    e0.record(ext)
    for _ in range(K):
        ens.gpe_rk4(S)
    e1.record(ext)
    torch.cuda.synchronize()
    launches = ens.launches - l0
    ms = e0.elapsed_time(e1)
    pts = sum(n * n for n in sizes)
    errs = {}
    for m, n, psi in init:
        ens.set_psi(m, psi)
    ens.gpe_rk4(100)
    for m, n, psi in init:
        s64 = vk.GPESolver(vk.params_for(n, dt=5e-4, precision=vk.VK_PREC_FP64))
        s64.set_psi(psi)
        s64.gpe_rk4(100)
        ref = s64.get_psi()
        d64 = s64.diagnostics_gpe()
        s64.close()
        got = ens.get_psi(m)
        ev = vk.GPESolver(vk.params_for(n, dt=5e-4, precision=vk.VK_PREC_FP64, otoc=False))
        ev.set_psi(got)  # diagnostics of the member's state, evaluated in FP64
        d32 = ev.diagnostics_gpe()
        ev.close()
        errs[f"member{m}_{n}"] = {"rel_l2_psi": float(np.linalg.norm(got - ref) / np.linalg.norm(ref)),
                                  **precision_errors(d32, d64)}
    report = ens.report
    ens.close()
    return {"value": pts * S * K / (ms * 1e-3), "unit": UNIT, "members": "192 x 256^2 + 48 x 512^2",
            "grid_points": pts, "ms_per_rk4_step": ms / (K * S), "gpu_launches": launches,
            "errors_vs_fp64_after_100_steps": errs, "autotune": report}


def argle_bench(torch, n, psi0):
    """ARGLE relaxation at n^2 (the relaxation of the 1024^2 workload: 2000 steps at dt = 1e-3 from the
    64-vortex state), FP64 and FP32: throughput and the residual
    ||kpsi_new - kpsi_old|| / (dt ||kpsi_old||) after the 2000 steps."""
    from quantumvortices_gb300 import vk
    out = {"unit": UNIT, "steps": 2000}
    for nm, prec in (("fp64", vk.VK_PREC_FP64), ("fp32", vk.VK_PREC_FP32)):
        s = vk.GPESolver(vk.params_for(n, dt=1e-3, precision=prec))
        s.set_psi(psi0)
        s.argle(5)
        s.set_psi(psi0)
        ext = torch.cuda.ExternalStream(s.stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        r = s.argle(2000)
        e1.record(ext)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        out[nm] = {"value": n * n * 2000 / (ms * 1e-3), "ms_per_step": ms / 2000, "residual": r}
        s.close()
    return out


def particles_bench(torch, K, W, S, flush):
    """1024^2 FP64 with 16 Gaussian particles (V0 = 10, d = 2 xi,
    M = 5 pi d^2, positions uniform, velocities N(0, 0.1^2), 64 vortices,
    dt = 5e-4): RK4 throughput with the particle forces and the particle RK4
    in every stage, the per-kernel split (the Parseval force pass is
    k_y1_pot), and one diagnostics call with the particle energies."""
    from quantumvortices_gb300 import vk
    n, P = 1024, 16
    dx = 2 * math.pi / n
    d = 2.0 * math.sqrt(2.0) * dx
    p = vk.params_for(n, dt=5e-4, n_particles=P, ppotd=2.0, ppotv0=10.0, gp_mass_part=5.0 * math.pi * d * d)
    psi0 = workload(n, seed=3)
    rng = np.random.default_rng(3)
    s = vk.GPESolver(p)
    s.set_psi(psi0)
    s.particles_set(rng.uniform(0, 2 * math.pi, (P, 2)), rng.normal(0, 0.1, (P, 2)), np.zeros((P, 2)))
    ext = torch.cuda.ExternalStream(s.stream)
    for _ in range(W):
        s.gpe_rk4(S)
    torch.cuda.synchronize()
    ms = 0.0
    l0 = s.launches
    for _ in range(K):
        with torch.cuda.stream(ext):
            flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        s.gpe_rk4(S)
        e1.record(ext)
        torch.cuda.synchronize()
        ms += e0.elapsed_time(e1)
    launches = s.launches - l0
    s.timing_begin()
    s.gpe_rk4(S)
    per = s.timing_end()
    diag = diagnostics_ms(s)
    pos, vel, frc = s.particles_get()
    s.close()
    step_ms = ms / (K * S)
    force_ms = per.get("k_y1_pot", (0.0, 1))[0] / S
    return {"value": n * n * S * K / (ms * 1e-3), "unit": UNIT, "workload": "1024^2 FP64 + 16 Gaussian particles, "
            "V0=10, d=2xi, M=5 pi d^2, 64 vortices, dt=5e-4", "ms_per_rk4_step": step_ms,
            "gpu_launches": launches,
            "force_pass": {"kernel": "k_y1_pot (y transform of rho, dealias, all 16 forces by Parseval, V_tot)",
                           "ms_per_rk4_step": force_ms, "frac_of_step": force_ms / step_ms},
            "kernel_ms": {k: round(v[0] / v[1], 5) for k, v in per.items()},
            "diagnostics_ms": diag, "finite": bool(np.isfinite(pos).all() and np.isfinite(frc).all())}


def diagnostics_ms(s, reps=5):
    """Wall time of one vk_diagnostics call (energies, momentum, norm, the six
    shell spectra, vortex count, particle energies; results copied to the
    host), the median of `reps` calls after one untimed call."""
    s.diagnostics_gpe()
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        s.diagnostics_gpe()
        ts.append(time.perf_counter() - t0)
    return 1e3 * statistics.median(ts)


def argle_time_to_residual(torch, n, psi0):
    """ARGLE wall time (FP64, dt = 1e-3) to a stated residual, checked every
    `chunk` steps (the checks are inside the time):
      * vortex_state: the 64-vortex workload to the residual plain ARGLE has
        after the configured 2000 steps (vortex states never reach 1e-8:
        vortices drift and annihilate while the residual stays near 1e-1);
      * vortex_free: a real density-perturbed state, 1 + 0.3 sum of 12 random
        low-k cosines, to 1e-8 (it relaxes to the uniform ground state)."""
    from quantumvortices_gb300 import vk
    out = {"residual_definition": "||kpsi_new - kpsi_old||_2 / (dt ||kpsi_old||_2), FP64"}
    p = vk.params_for(n, dt=1e-3)
    rng = np.random.default_rng(5)
    x = np.arange(n) * 2 * math.pi / n
    X, Y = np.meshgrid(x, x)
    pert = np.zeros((n, n))
    for _ in range(12):
        kx, ky = rng.integers(0, 5, 2)
        pert += math.cos(rng.uniform(0, 2 * math.pi)) * np.cos(kx * X + ky * Y + rng.uniform(0, 2 * math.pi))
    free = (1.0 + 0.3 * pert / np.abs(pert).max()).astype(np.complex128)
    with vk.GPESolver(p) as s:
        s.set_psi(psi0)
        target = s.argle(2000)
        for name, start, tgt, chunk, cap in (("vortex_state", psi0, target, 50, 4000),
                                             ("vortex_free", free, 1e-8, 10, 20000)):
            s.set_psi(start)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            steps, r = 0, float("inf")
            while steps < cap:
                r = s.argle(chunk)
                steps += chunk
                if r <= tgt:
                    break
            t = time.perf_counter() - t0
            out[name] = {"target_residual": tgt, "reached": bool(r <= tgt), "residual": r, "steps": steps,
                         "time_to_residual_s": t}
    return out


def warmstart_bench(n=512, n_train=512, epochs=6, n_eval=8, batch=8):
    """The learned ARGLE warm start trained in this process at a reduced size
    (n_train solver-generated 512^2 states, 8-128 vortices, 1000 FP32 ARGLE
    steps each; batches of `batch` images) and evaluated on n_eval held-out
    seeds disjoint from the training seeds: ARGLE iterations saved and
    wall-time ratio (features and network included) to the residual plain
    ARGLE reaches after 1000 steps, and the ARGLE functional E - Omega N after
    equal steps."""
    from quantumvortices_gb300 import warmstart as ws
    gen = ws.DataGen(n, 1000)
    net = ws.WarmStartNet(n, n, 32, 4, seed=1, batch=batch)
    try:
        tr = ws.train(net, gen, n_train, epochs, 1e-3, log=lambda *a: None)
        rows = ws.evaluate(net, gen, list(range(900_000, 900_000 + n_eval)), log=lambda *a: None)
        summ = ws.summarize(rows)
    finally:
        net.close()
        gen.close()
    return {"grid": n, "training_states": n_train, "epochs": epochs, "batch": batch, "held_out_seeds": n_eval,
            "reduced_from": "20000 training states / 1000 held-out seeds",
            "generation_s": tr["gen_s"], "train_s": tr["train_s"], "train_tflops": tr["tensor_tflops"],
            **{k: summ[k] for k in ("iterations_saved_frac", "time_ratio_warm_over_plain", "time_ratio_median",
                                     "reached_frac", "rel_grand_diff_same_steps_mean", "grand_lower_frac",
                                     "rel_energy_diff_same_steps_mean")}}


def grid4096_bench(torch, steps=5):
    """One 4096^2 field with 1024 seeded vortices: FP64 and FP32 throughput
    and the FP32-vs-FP64 psi error after 100 RK4 steps."""
    from quantumvortices_gb300 import vk
    n = 4096
    xi0 = math.sqrt(2) * 2 * math.pi / n
    out = {}
    psis, diags = {}, {}
    for nm, prec in (("fp64", vk.VK_PREC_FP64), ("fp32", vk.VK_PREC_FP32)):
        s = vk.GPESolver(vk.params_for(n, dt=5e-4, precision=prec))
        s.set_psi_vortices(1024, 11, xi0, min_sep=4 * xi0)
        s.gpe_rk4(2)
        ext = torch.cuda.ExternalStream(s.stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        s.gpe_rk4(steps)
        e1.record(ext)
        torch.cuda.synchronize()
        out[nm] = n * n * steps / (e0.elapsed_time(e1) * 1e-3)
        s.timing_begin()
        s.gpe_rk4(1)
        per = s.timing_end()
        out[nm + "_kernel_ms"] = {k: round(v[0] / v[1], 5) for k, v in per.items()}
        s.set_psi_vortices(1024, 11, xi0, min_sep=4 * xi0)
        s.gpe_rk4(100)
        psis[nm] = s.get_psi()
        diags[nm] = s.diagnostics_gpe()
        s.close()
    a, b = psis["fp32"], psis["fp64"]
    out["unit"] = UNIT
    out["rel_l2_psi_fp32_vs_fp64_after_100_steps"] = float(np.linalg.norm(a - b) / np.linalg.norm(b))
    out.update(precision_errors(diags["fp32"], diags["fp64"]))
    return out


def count_disk(n):
    ka2 = (n / 3.0) ** 2          # IF (ksqr .GE. kalias**2), src/gpe.f90:571
    k2 = int(math.floor(ka2)) + 1
    while float(k2) >= ka2:
        k2 -= 1
    k = np.array([i if i < n // 2 else i - n for i in range(n)])
    ks = k[:, None] ** 2 + k[None, :] ** 2
    return int((ks <= k2).sum()), int(math.isqrt(k2))


# ---------------------------------------------------------- our arm --

def run_ours(args, rank, world, local_rank):
    import torch
    from quantumvortices_gb300 import vk

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    n, S, K, W = args.n, args.substeps, args.steps, args.warmup
    p = vk.params_for(n, dt=5e-4, precision=vk.VK_PREC_FP64)
    psi0 = workload(n, seed=1 + rank)
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    def timed_loop(solver, K, W):
        ext = torch.cuda.ExternalStream(solver.stream)
        for _ in range(W):
            solver.gpe_rk4(S)
        barrier()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
        l0 = solver.launches
        for i in range(K):
            with torch.cuda.stream(ext):
                flush.zero_()          # L2 flush between timed iterations (outside the events)
            ev[i][0].record(ext)
            solver.gpe_rk4(S)
            ev[i][1].record(ext)
        torch.cuda.synchronize()
        launches = solver.launches - l0
        ms = sum(a.elapsed_time(b) for a, b in ev)
        barrier()
        return ms, launches

    s = vk.GPESolver(p)
    s.set_psi(psi0)
    sampler = ClockSampler(local_rank)
    sampler.start()
    ms, launches = timed_loop(s, K, W)
    clocks = sampler.stop()
    value, ms_max = replica_throughput(ms, world, n * n, S, K, dist, "cuda")

    # per-kernel times (events around every launch, separate pass)
    s.timing_begin()
    s.gpe_rk4(S)
    per = s.timing_end()

    # end to end through the public API with host buffers
    host_in = np.ascontiguousarray(psi0)
    host_out = np.empty_like(host_in)
    e2e_times = []
    for i in range(6):  # the first round (thread-pool start, first-touch) is not timed
        t0 = time.perf_counter()
        s.set_psi(host_in)
        s.gpe_rk4(S)
        s.get_psi(host_out)
        if i > 0:
            e2e_times.append(time.perf_counter() - t0)
    e2e_t = statistics.median(e2e_times)
    diag_ms = diagnostics_ms(s)
    s.close()

    # FP32 bulk path: throughput and error against the FP64 path after S steps
    fp32 = None
    if not args.no_fp32:
        p32 = vk.params_for(n, dt=5e-4, precision=vk.VK_PREC_FP32)
        s32 = vk.GPESolver(p32)
        s32.set_psi(psi0)
        ms32, l32 = timed_loop(s32, K, W)
        s32.set_psi(psi0)
        s32.gpe_rk4(100)
        a = s32.get_psi()
        d32 = s32.diagnostics_gpe()
        s64 = vk.GPESolver(p)
        s64.set_psi(psi0)
        s64.gpe_rk4(100)
        b = s64.get_psi()
        d64 = s64.diagnostics_gpe()
        s32.timing_begin()
        s32.gpe_rk4(S)
        per32 = s32.timing_end()
        s32.close()
        s64.close()
        fp32 = {"value": world * n * n * S * K / (ms32 * 1e-3), "unit": UNIT, "ms_per_step": ms32 / K,
                "rel_l2_psi_vs_fp64_after_100_steps": float(np.linalg.norm(a - b) / np.linalg.norm(b)),
                **precision_errors(d32, d64),
                "kernel_ms": {k: round(v[0] / v[1], 5) for k, v in per32.items()}}

    ens = None if args.no_ensemble else ensemble_bench(torch, K, W, S)
    g4096 = None if args.no_4096 else grid4096_bench(torch)
    argle = None if args.no_argle else argle_bench(torch, n, psi0)
    if argle is not None:
        argle["time_to_residual"] = argle_time_to_residual(torch, n, psi0)
    parts = None if args.no_particles else particles_bench(torch, K, W, S, flush)
    warm = None if args.no_warmstart else warmstart_bench()
    if rank != 0:
        return
    dgemm_tf = fp64_peak_tflops(torch)
    disk, Kk = count_disk(n)
    e = 16
    # dominant kernel of the FP64 step
    tag, (tot, cnt) = max(per.items(), key=lambda kv: kv[1][0])
    per_launch_ms = tot / cnt
    nbytes = kernel_bytes(tag, n, Kk, e, disk)
    peak, peak_kind = hbm_peak()
    achieved = nbytes / (per_launch_ms * 1e-3) / 1e9 if nbytes else None
    flops = kernel_flops(tag, n, Kk)
    f64_tf = flops / (per_launch_ms * 1e-3) / 1e12 if flops else None
    step_ms = ms_max / (K * S)
    canonical = 1344.0 * n * n / (step_ms * 1e-3) / 1e9  # canonical model: 84 field transfers per RK4 step
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": ms_max / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded 64-vortex state)",
        "config": {"workload": f"RK4 {n}^2 plain FP64, 64 vortices, dt=5e-4", "grid": n,
                   "rk4_steps_per_step": S, "parallelism": "replicas" if world > 1 else "single",
                   "l2": "flushed between timed steps (512 MiB write)"},
        "clocks": clocks, "gpu_launches": launches,
        "roofline": {"bound": "fp64", "kernel": tag,
                     "achieved": f64_tf, "peak": dgemm_tf, "unit": "TFLOP/s",
                     "frac": f64_tf / dgemm_tf if f64_tf else None,
                     "peak_source": "cuBLAS DGEMM 4096^3 measured in this run (no FP64 peak is recorded for "
                                    "this GPU); the 1024^2 fields of a step stay in L2, and the passes are "
                                    "bound by the FP64 pipe",
                     "flops_per_launch": flops, "flop_model": "5 L log2 L per L-point complex FFT",
                     "launch_ms": per_launch_ms,
                     "traffic": RECORDED_DRAM_BYTES_1024_FP64.get(tag) if n == 1024 else None,
                     "traffic_source": "recorded ncu capture (dram__bytes_read.sum + dram__bytes_write.sum per "
                                       "launch of this kernel at 1024^2), not measured in this run",
                     "hbm": {"achieved": achieved, "peak": peak, "peak_source": peak_kind, "unit": "GB/s",
                             "frac": achieved / peak if achieved else None,
                             "algorithmic_bytes_per_launch": nbytes,
                             "step_canonical_gbs": canonical, "step_canonical_frac": canonical / peak}},
        "diagnostics": {"ms_per_call": diag_ms, "grid": n,
                        "frac_of_rk4_at_cadence_200": diag_ms / (200.0 * step_ms),
                        "what": "one vk_diagnostics call: energies, momentum, norm, six shell spectra, vortex "
                                "count, results copied to the host"},
        "kernel_ms": {k: round(v[0] / v[1], 5) for k, v in per.items()},
        "kernel_ms_note": "per launch, from a separate pass with an event pair around every launch and no CUDA "
                          "graph; their sum reads a few percent above the graph-replayed step time",
        "e2e": {"value": n * n * S / e2e_t, "unit": UNIT, "h2d_bytes_per_step": n * n * 16,
                "d2h_bytes_per_step": n * n * 16},
        "fp32": fp32,
        "ensemble": ens,
        "grid_4096": g4096,
        "argle": argle,
        "particles": parts,
        "warmstart": warm,
    }
    out["cpu_baseline"] = cpu_baseline(n, psi0, args.cpu_seconds)
    print(json.dumps(out))


def cpu_baseline(n, psi0, seconds):
    """The CPU FP64 oracle (restatement of src/gpe.f90 on the host cores)."""
    from quantumvortices_gb300 import vk
    from oracle.oracle import Oracle
    cores = os.cpu_count() or 1
    p = vk.params_for(n, dt=5e-4)
    o = Oracle.from_vk_params(p, threads=cores)
    o.set_psi(psi0)
    t0 = time.perf_counter()
    o.gpe_rk4(1)
    t1 = time.perf_counter() - t0
    steps = max(1, min(200, int(seconds / max(t1, 1e-6))))
    t0 = time.perf_counter()
    o.gpe_rk4(steps)
    dt = time.perf_counter() - t0
    return {"value": n * n * steps / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{steps} RK4 steps at {n}^2 FP64 (oracle restatement, OpenMP over rows)"}


# ----------------------------------------------------- reference arm --

def run_reference(args, rank):
    """The CPU FP64 restatement of src/gpe.f90 on all host cores.  Parameters
    and the seeded state come from the oracle itself (oracle.derived_params,
    oracle.ic_vortices): this arm loads no product library."""
    if rank != 0:
        return
    from oracle import oracle as orc
    n = args.n
    cores = os.cpu_count() or 1
    psi0, _ = orc.ic_vortices(n, n, 64, seed=1, min_sep=4 * math.sqrt(2) * 2 * math.pi / n)
    o = orc.Oracle(**orc.derived_params(n, dt=5e-4), threads=cores)
    o.set_psi(psi0)
    S = args.substeps  # RK4 steps per bench step, as in the GPU arm
    for _ in range(args.warmup):
        o.gpe_rk4(S)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        o.gpe_rk4(S)
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    value = n * n * S * args.steps / tot
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded 64-vortex state)",
           "config": {"workload": f"RK4 {n}^2 plain FP64, 64 vortices, dt=5e-4", "grid": n,
                      "rk4_steps_per_step": S, "parallelism": "single",
                      "l2": "host caches not flushed (CPU arm)"},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                            "sample": f"{S} RK4 steps at {n}^2 per bench step; the Fortran+FFTW+MPI "
                                      "reference cannot be built here (no gfortran, MPI or FFTW), so the "
                                      "oracle restatement runs on all host cores"},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
