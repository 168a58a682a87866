"""Benchmark: FSI time steps per second of the immersed-boundary step at
800x400 cells x 5 nested levels, FP64, on GB300.

Workload (``plate800x400``): the hinged flat plate of length 1 (51 body points,
twice the grid spacing apart; 10 degrees incidence plus a seeded 0.01 tip
perturbation), Re=500, fine grid 800x400 on [-1,7]x[-2,2], 5 levels, dt=1e-3,
GMRES and FSI tolerances 1e-10.  The plate is the torsional-spring body
(family 2) the reference implements; inputs are synthetic (no dataset is
involved).

``python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]``

GPU arm: W untimed steps from the impulsive start, then K steps timed with CUDA
events on the simulation's stream (the state, about 100 MB per level set, is
larger than L2 only in aggregate; every step re-reads all levels).  ``e2e``
times K more steps through the C ABI with host buffers: each step uploads the
frame fluxes q0 of all levels from pinned memory (the per-step motion input of
motion_potential/motion_rotation, variables.F90:299-360) and reads the force
coefficients and hinge angle back.  With N>1 every rank advances its own
replica of the simulation (the step does not shard; no collective in the data
path) and ``value`` is the sum over ranks.

Reference arm: the reference (Fortran + PETSc + FFTW + MPI) cannot be built in
this image or on the GPU machine, so the CPU restatement in ``oracle/`` (numpy +
scipy.fft, all host cores) is timed on the same workload.  One oracle step takes
tens of seconds, so each "step" is a bounded sample: the non-Krylov part of a
step (predictor on all levels, two vort2flux, correction) measured once per
step plus a few Schur matvecs, scaled to the Krylov matvecs per step this
workload needs.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

METRIC = "FSI steps/s @800x400x5 FP64"
WORKLOAD = "plate800x400"
# Schur matvecs per step of this workload (Krylov iterations + one initial-residual
# product per GMRES cycle, summed over the FSI iterations), counted by the GPU
# arm's ib_get_work (49.8 to 53 over the first steps after warm-up on GB300); the CPU
# arm runs the same algorithm with the matrix-free operator.
MATVECS_PER_STEP = 52.0


def _env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return float(d.get("hbm_gbs", 6800.0)), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region.

    Sampling starts before the region (the first sample is awaited) at 50 ms intervals; each
    sample carries nvidia-smi's timestamp, and the summary keeps the samples that fall inside
    the region marked by begin()/end()."""

    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None
        self.gpu = gpu_index
        self.t0 = self.t1 = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "50"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        deadline = time.time() + 5.0
        while self.p and time.time() < deadline and not self._rows():
            time.sleep(0.02)
        return self

    def begin(self):
        self.t0 = time.time()

    def end(self):
        self.t1 = time.time()
        time.sleep(0.1)   # let a sample taken at the end of the region reach the file

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()

    def _rows(self):
        self.f.flush()
        rows = []
        try:
            for line in Path(self.f.name).read_text().splitlines():
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 10:
                    rows.append(parts)
        except OSError:
            pass
        return rows

    @staticmethod
    def _stamp(text):
        import datetime
        try:
            return datetime.datetime.strptime(text, "%Y/%m/%d %H:%M:%S.%f").timestamp()
        except ValueError:
            return None

    def summary(self):
        rows = self._rows()
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        inside = rows
        where = "all samples"
        if self.t0 is not None and self.t1 is not None:
            sel = [r for r in rows if (self._stamp(r[0]) or 0.0) >= self.t0 - 0.06 and
                   (self._stamp(r[0]) or 0.0) <= self.t1 + 0.06]
            if sel:
                inside, where = sel, "samples inside the timed region"
            else:
                where = "no sample fell inside the timed region; all samples of the run"
        sm = [float(r[2]) for r in inside if r[2].replace(".", "").isdigit()]
        mx = [float(r[3]) for r in inside if r[3].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in inside for i in range(4) if r[6 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(inside), "source": where}


def _dist():
    world = _env_int("WORLD_SIZE", 1)
    rank = _env_int("RANK", 0)
    local = _env_int("LOCAL_RANK", 0)
    return world, rank, local


def reduce_max(t: float, world: int, device: str = "cuda") -> float:
    """Maximum of a per-rank timing over all ranks (the only collective bench.py uses)."""
    if world <= 1:
        return t
    import torch
    import torch.distributed as dist
    x = torch.tensor([t], dtype=torch.float64, device=device)
    dist.all_reduce(x, op=dist.ReduceOp.MAX)
    return float(x.item())


def _barrier_max(t: float, world: int) -> float:
    return reduce_max(t, world, "cuda")


def _barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def _oracle_sample(p, bodies, n_mv: int, workers: int):
    """Time the oracle's non-Krylov part of one step and n_mv Schur matvecs."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import scipy.fft as sfft
    import ib_oracle as O
    po = O.Params(**{k: getattr(p, k) for k in O.Params.__dataclass_fields__ if hasattr(p, k)})
    ob = [O.Body(x=b.x, y=b.y, fam=b.fam, gamma0_deg=b.gamma0_deg, itheta=b.itheta, ktheta=b.ktheta,
                 ctheta=b.ctheta) for b in bodies]
    o = O.IBOracle(po, ob)
    rng = np.random.default_rng(0)
    for k in range(o.L):  # a developed-looking state so nothing is trivially zero
        o.omega[k] = 1e-3 * rng.standard_normal(o.omega[k].shape)
    with sfft.set_workers(workers):
        t0 = time.perf_counter()
        L = o.L
        lastbc = [o.get_bc(o.omega[k + 1], 0.25) for k in range(L - 1)] + [np.zeros(o.nbc)]
        for k in range(L - 1, -1, -1):
            obc = o.get_bc(o.omega[k + 1], 0.25) if k < L - 1 else np.zeros(o.nbc)
            nlx, nly = o.nonlinear(o.omega[k], o.qx[k] + o.q0x[k], o.qy[k] + o.q0y[k], lastbc[k])
            rb = np.zeros_like(o.omega[k])
            o.apply_bc(rb, lastbc[k], o.vfac[k]); o.apply_bc(rb, obc, o.vfac[k])
            rhs = o.rot(nlx, nly)
            o.omega[k] = o.fluid_predictor(o.omega[k], rhs, o.rhs_old[k], rb, k)
            o.rhs_old[k] = rhs
        o.s, o.qx, o.qy = o.vort2flux(o.omega)
        rhsf = o.regT(o.qx[0] + o.q0x[0], o.qy[0] + o.q0y[0], o.compute_rhs())
        o.f_rdst = o.redistribute(rhsf)
        hx, hy = o.reg(rhsf)
        o.omega[0] = o.omega[0] - o.ainv(o.rot(hx, hy))
        o.s, o.qx, o.qy = o.vort2flux(o.omega)
        t_fixed = time.perf_counter() - t0
        x = rng.standard_normal(o.nf)
        o.a_times(x)
        t0 = time.perf_counter()
        for _ in range(n_mv):
            x = o.a_times(x)
            x = x / np.linalg.norm(x)
        t_mv = (time.perf_counter() - t0) / n_mv
    return t_fixed, t_mv


def run_reference(args, world, rank):
    if rank != 0:
        return 0
    from ib_parallel_gb300 import geometry as GEO
    p, bodies = GEO.config_plate_800x400()
    cores = os.cpu_count() or 1
    mv = MATVECS_PER_STEP
    if mv is None:
        print(json.dumps({"impl": "reference", "unavailable": "matvecs per step not yet measured on GB300"}))
        return 0
    per_step = []
    for i in range(args.warmup + args.steps):
        t_fixed, t_mv = _oracle_sample(p, bodies, n_mv=2, workers=cores)
        if i >= args.warmup:
            per_step.append(t_fixed + mv * t_mv)
    T = float(np.mean(per_step))
    value = 1.0 / T
    sample = (f"oracle port (numpy+scipy.fft, {cores} threads): per step the non-Krylov part of a step once "
              f"plus 2 Schur matvecs, scaled to {mv} matvecs/step")
    line = {"metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * T, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "grid": "800x400", "levels": 5, "body_points": 51},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "steps/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_gpu(args, world, rank, local):
    import torch
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", init_method="env://")
    else:
        torch.cuda.set_device(0)
    from ib_parallel_gb300 import geometry as GEO
    from ib_parallel_gb300 import ibgpu as G
    p, bodies = GEO.config_plate_800x400()
    if args.no_autotune:
        p.autotune = 0
    sim = G.Simulation(p, bodies)
    stream = torch.cuda.ExternalStream(sim.stream())
    L = p.mgridlev
    for _ in range(args.warmup):
        sim.advance()
    sim.synchronize()
    mv0, passes0 = sim.work()
    launches0 = G.launch_count()
    ksp_sum, fsi_sum = 0, 0
    _barrier(world)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    if args.host_fsi_loop:
        sim.step_profile(1)
    with Clocks(local) as clk:
        if args.profile_window:
            torch.cuda.profiler.start()
        clk.begin()
        e0.record(stream)
        for _ in range(args.steps):
            sim.advance()
            k, f = sim.counters()
            ksp_sum += k
            fsi_sum += f
        e1.record(stream)
        e1.synchronize()
        clk.end()
        if args.profile_window:
            torch.cuda.profiler.stop()
    if args.host_fsi_loop:
        sim.step_profile(0)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    t_s = _barrier_max(ms / 1e3, world)
    mv1, passes1 = sim.work()
    launches_timed = G.launch_count() - launches0
    mv_per_step = (mv1 - mv0) / args.steps
    passes_timed = [b - a for a, b in zip(passes0, passes1)]
    value = world * args.steps / t_s

    # ---- end to end through the C ABI with host buffers
    q0x = [torch.from_numpy(sim.get_field("q0x", k)).pin_memory() for k in range(L)]
    q0y = [torch.from_numpy(sim.get_field("q0y", k)).pin_memory() for k in range(L)]
    cx = torch.zeros(max(1, sim.nbody), dtype=torch.float64).pin_memory()
    cy = torch.zeros_like(cx)
    th = torch.zeros(max(1, sim.ntors), dtype=torch.float64).pin_memory()
    h2d = sum(t.numel() * 8 for t in q0x + q0y)
    d2h = (2 * sim.nbody + sim.ntors) * 8
    _barrier(world)
    torch.cuda.synchronize()
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(args.steps):
        for k in range(L):
            sim.set_field("q0x", k, q0x[k])
            sim.set_field("q0y", k, q0y[k])
        sim.advance()
        G._check(sim.lib.ib_get_forces(sim.h, G.C.c_void_p(cx.data_ptr()), G.C.c_void_p(cy.data_ptr())))
        G._check(sim.lib.ib_get_body_state(sim.h, G.C.c_void_p(th.data_ptr()), None, None))
    f1.record(stream)
    f1.synchronize()
    e2e_s = _barrier_max(f0.elapsed_time(f1) / 1e3, world)
    e2e_value = world * args.steps / e2e_s

    # ---- roofline of the dominant kernel (the DST-I x pass: largest share of the ncu launch
    # list, profiles/launch_list_plate800x400.md), timed alone: 20 back-to-back full passes
    # over the finest grid with CUDA events on the simulation's stream
    m, n = p.m, p.n
    ns = (m - 1) * (n - 1)
    t_x = sim.time_pass(0, 20)
    t_tri = sim.time_pass(1, 20)
    bytes_x = 16.0 * ns                       # one field read, one written
    achieved = bytes_x / (t_x * 1e-3) / 1e9
    peak, peak_kind = _peaks()
    flops_x = 2.5 * (n - 1) * m * math.log2(2 * m)
    fp64_peak = G.measure_fp64_peak()
    fp_achieved = flops_x / (t_x * 1e-3) / 1e12
    traffic = None
    tpath = ROOT / "profiles" / "dst_traffic_800x400.txt"
    if tpath.exists():
        for line in tpath.read_text().splitlines():
            if line.startswith("k_dst_x dram_bytes_per_launch"):
                try:
                    traffic = float(line.split("=")[1])
                except ValueError:
                    traffic = None
    k_final, f_final = sim.counters()
    result = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded hinged plate, impulsive start)",
        "config": {"workload": WORKLOAD, "grid": "800x400", "levels": 5, "body_points": 51, "Re": 500,
                   "dt": 1e-3, "gmres_rtol": 1e-10, "fsi_tol": 1e-10, "parallelism": f"replicas{world}",
                   "l2": "working set (~330 MB of state, tables and scratch) larger than L2 (129 MB)"},
        "clocks": clk.summary(),
        "e2e": {"value": e2e_value, "unit": "steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": None,
        "work_per_step": {"schur_matvecs": mv_per_step, "ksp_iter": ksp_sum / args.steps,
                          "fsi_iter": fsi_sum / args.steps,
                          "dst_passes": [x / args.steps for x in passes_timed]},
        "roofline": {"bound": "hbm", "kernel": "k_dst_x (DST-I along x, 399 rows of 799)", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                     "peak_source": "of measured (MEASURED_PEAKS.json hbm_gbs, burst; kernel timed alone)"
                     if peak_kind == "measured" else "of fallback 6.8 TB/s",
                     "bytes_per_launch": bytes_x, "avg_launch_us": 1e3 * t_x},
        "fp64_roofline": {"kernel": "k_dst_x", "achieved": fp_achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                          "frac": fp_achieved / fp64_peak, "flops_per_launch": flops_x,
                          "peak_source": "of measured FP64 FMA loop on this GPU (ib_measure_fp64_peak)"},
        "tridiagonal_pass_us": 1e3 * t_tri,
        "schur_stages_us": sim.profile_schur(20),
        "influence": sim.influence_stats(),
        "launch_shapes": sim.launch_shapes(),
        "step_phases_us": _step_phases(sim, 5),
        "step_phases_device_loop_us": _step_phases(sim, 5, device_loop=True),
    }
    if not args.no_matrix_free:
        result["matrix_free"] = _matrix_free_rate(p, bodies, args)
    result["gpu_launches"] = launches_timed
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        t_fixed, t_mv = _oracle_sample(p, bodies, n_mv=4, workers=cores)
        cpu_val = 1.0 / (t_fixed + mv_per_step * t_mv)
        result["cpu_baseline"] = {
            "value": cpu_val, "unit": "steps/s", "cores": cores, "kind": "port",
            "sample": f"oracle port (numpy+scipy.fft, {cores} threads): non-Krylov part of one step "
                      f"({t_fixed:.2f} s) + 4 Schur matvecs ({t_mv * 1e3:.1f} ms each), scaled to the "
                      f"{mv_per_step:.1f} matvecs/step measured above"}
    if rank == 0:
        print(json.dumps(result))
    sim.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def _step_phases(sim, steps, device_loop=False):
    """Device time per step of each phase of ib_advance (CUDA events), over a few more steps:
    the FSI iterations phase by phase from the host, or (device_loop) the device FSI loop as
    one phase."""
    sim.step_profile(3 if device_loop else 1)
    for _ in range(steps):
        sim.advance()
    out = sim.step_profile(0)
    out = {k: v for k, v in out.items() if v > 0.0}
    out["steps"] = steps
    return out


def _matrix_free_rate(p, bodies, args):
    """Steps/s of the same workload with the Schur operator applied matrix-free in every
    Krylov iteration (schur_mode 1), timed the same way over the same number of steps."""
    import dataclasses

    import torch
    from ib_parallel_gb300 import ibgpu as G
    sim = G.Simulation(dataclasses.replace(p, schur_mode=1), bodies)
    stream = torch.cuda.ExternalStream(sim.stream())
    for _ in range(args.warmup):
        sim.advance()
    sim.synchronize()
    mv0, _ = sim.work()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        sim.advance()
    e1.record(stream)
    e1.synchronize()
    mv1, _ = sim.work()
    sim.close()
    return {"value": args.steps / (e0.elapsed_time(e1) / 1e3), "unit": "steps/s",
            "schur_matvecs_per_step": (mv1 - mv0) / args.steps}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-matrix-free", action="store_true",
                    help="skip timing the matrix-free Schur operator beside the default one")
    ap.add_argument("--profile-window", action="store_true",
                    help="bracket the timed steps with cudaProfilerStart/Stop (for ncu --profile-from-start off)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="run with the default launch shapes instead of tuning them by timing at creation (for "
                         "profiler captures, whose replays would mislead the tuner)")
    ap.add_argument("--host-fsi-loop", action="store_true",
                    help="run the timed steps with per-phase timing on, so that the FSI iterations run from the "
                         "host and each of their kernels is a separate launch (a profiler lists kernels inside "
                         "the device loop's graph node only as the graph)")
    args = ap.parse_args()
    world, rank, local = _dist()
    if args.impl == "reference":
        return run_reference(args, world, rank)
    return run_gpu(args, world, rank, local)


if __name__ == "__main__":
    sys.exit(main())
