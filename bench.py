"""Benchmark: FSI time steps per second of the immersed-boundary step at
800x400 cells x 5 nested levels, FP64, on GB300.

Workload (``plate800x400``): the hinged flat plate of length 1 (51 body points,
twice the grid spacing apart; 10 degrees incidence plus a seeded 0.01 tip
perturbation), Re=500, fine grid 800x400 on [-1,7]x[-2,2], 5 levels, dt=1e-3,
GMRES and FSI tolerances 1e-10.  The plate is the torsional-spring body
(family 2) the reference implements; inputs are synthetic (no dataset is
involved).  A second workload, ``cylinder400x200`` (157-point rigid cylinder,
400x200 x 3 levels, Re=100, dt=0.004, the stationary-body direct solve), is
reported in the same line under ``workloads``.

``python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]``

GPU arm: W untimed steps from the impulsive start, then K steps timed with CUDA
events on the simulation's stream (state, tables and the influence band, about
0.5 GB, are larger than L2).  ``e2e`` times K more steps through the C ABI with
host buffers: each step uploads the frame fluxes q0 of all levels from pinned
memory (the per-step motion input of motion_potential/motion_rotation,
variables.F90:299-360) and reads the force coefficients and hinge angle back.
``long_run`` times a fresh simulation over many steps from the impulsive start
with every influence-band build inside the timed region.  With N>1 every rank
advances its own replica of the simulation (the step does not shard; no
collective in the data path) and ``value`` is the sum over ranks.

CPU arms (``--impl reference`` and ``cpu_baseline``): the reference (Fortran +
PETSc + FFTW + MPI) cannot be built in this image or on the GPU machine, so the CPU
restatement in ``oracle/`` (numpy + scipy.fft on all host threads) advances the
same workload through whole time steps from the same impulsive start, with its
own GMRES and FSI loop.  It is a numpy port, a weaker baseline than the
compiled reference would be; it runs the reference's matrix-free Schur
operator, so ``matrix_free`` (the GPU on that same algorithm) is printed beside
it as the algorithm-matched comparison.
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
C1_WORKLOAD = "cylinder400x200"


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


def _oracle(p, bodies):
    sys.path.insert(0, str(ROOT / "oracle"))
    import ib_oracle as O
    po = O.Params(**{k: getattr(p, k) for k in O.Params.__dataclass_fields__ if hasattr(p, k)})
    ob = [O.Body(x=b.x.copy(), y=b.y.copy(), fam=b.fam, gamma0_deg=b.gamma0_deg, itheta=b.itheta,
                 ktheta=b.ktheta, ctheta=b.ctheta, nelem=b.nelem) for b in bodies]
    return O.IBOracle(po, ob)


def _oracle_steps(p, bodies, workers, untimed=0, timed=None, budget_s=None, min_steps=2):
    """Whole time steps of the oracle (IBOracle.advance: predictor, vort2flux, its own GMRES
    and FSI loop, correction) from the impulsive start: `untimed` steps first, then either
    `timed` steps or as many as fit in budget_s (at least min_steps).  Returns the wall time
    of each timed step and the oracle."""
    import scipy.fft as sfft
    o = _oracle(p, bodies)
    times = []
    with sfft.set_workers(workers):
        for _ in range(untimed):
            o.advance()
        t_all = time.perf_counter()
        while True:
            t0 = time.perf_counter()
            o.advance()
            times.append(time.perf_counter() - t0)
            if timed is not None and len(times) >= timed:
                break
            if budget_s is not None and len(times) >= min_steps and time.perf_counter() - t_all >= budget_s:
                break
    return times, o


def run_reference(args, world, rank):
    if rank != 0:
        return 0
    from ib_parallel_gb300 import geometry as GEO
    p, bodies = GEO.config_plate_800x400()
    cores = os.cpu_count() or 1
    times, o = _oracle_steps(p, bodies, cores, untimed=args.warmup, timed=args.steps)
    T = float(np.sum(times))
    value = len(times) / T
    sample = (f"oracle port (numpy + scipy.fft, {cores} threads; the Fortran reference cannot be built here): "
              f"{len(times)} whole time steps ({args.warmup + 1}..{args.warmup + len(times)} from the impulsive "
              f"start, each with its own GMRES and FSI loop; last step {o.ksp_iter} Krylov iterations, "
              f"{o.fsi_iter} FSI iterations), {T:.1f} s")
    line = {"metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * T / len(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded hinged plate)",
            "config": {"workload": WORKLOAD, "grid": "800x400", "levels": 5, "body_points": 51, "Re": 500,
                       "dt": 1e-3, "gmres_rtol": 1e-10, "fsi_tol": 1e-10, "parallelism": "replicas1"},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "steps/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def _algorithmic_bytes(m, n, L, nf):
    """Compulsory DRAM bytes of the reference's step (each array argument of the routines it
    calls read once, each output written once; FP64): the predictor on every level, two
    vort2flux, the correction, and per Krylov iteration one matrix-free Schur product."""
    ns, nu, nv = (m - 1) * (n - 1), (m + 1) * n, m * (n + 1)
    pred = 8.0 * (4 * ns + nu + nv)
    v2f = 8.0 * ((2 * ns + nu + nv) + (L - 1) * (3.25 * ns + nu + nv))
    corr = 8.0 * (3 * ns + nu + nv) + v2f
    fixed = L * pred + v2f + corr
    matvec = 8.0 * 3 * ns + v2f + 49.0 * nf * 56.0
    return fixed, matvec


class _NoGC:
    """Python's cyclic garbage collector held off inside a timed region (a collection there
    would stall the host between two steps, and each step waits on the host once)."""

    def __enter__(self):
        import gc
        self.was = gc.isenabled()
        gc.disable()

    def __exit__(self, *a):
        import gc
        if self.was:
            gc.enable()


def _timed_steps(sim, stream, steps):
    """K steps of sim timed with CUDA events on its stream; returns (seconds, ksp, fsi sums)."""
    import torch
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    ksp_sum = fsi_sum = 0
    with _NoGC():
        e0.record(stream)
        for _ in range(steps):
            sim.advance()
            k, f = sim.counters()
            ksp_sum += k
            fsi_sum += f
        e1.record(stream)
        e1.synchronize()
    return e0.elapsed_time(e1) / 1e3, ksp_sum, fsi_sum


def _e2e_steps(sim, stream, steps, fields=False):
    """K steps through the C ABI with host buffers: each step gives the frame's motion of that
    step, (u, v, angular velocity) from pinned memory through ib_set_frame (the reference's
    per-step input: motion_grid, from which motion_potential and motion_rotation form the frame
    fluxes), or with fields=True uploads the frame fluxes q0 of all levels themselves from pinned
    memory, and reads the force coefficients (and hinge angles) back."""
    import torch
    from ib_parallel_gb300 import ibgpu as G
    L = sim.params.mgridlev
    q0x = [torch.from_numpy(sim.get_field("q0x", k)).pin_memory() for k in range(L)] if fields else []
    q0y = [torch.from_numpy(sim.get_field("q0y", k)).pin_memory() for k in range(L)] if fields else []
    frame = torch.tensor(list(sim.params.motion[:3]), dtype=torch.float64).pin_memory()
    cx = torch.zeros(max(1, sim.nbody), dtype=torch.float64).pin_memory()
    cy = torch.zeros_like(cx)
    th = torch.zeros(max(1, sim.ntors), dtype=torch.float64).pin_memory()
    h2d = sum(t.numel() * 8 for t in q0x + q0y) if fields else frame.numel() * 8
    d2h = (2 * sim.nbody + sim.ntors) * 8
    torch.cuda.synchronize()
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    with _NoGC():
        f0.record(stream)
        for _ in range(steps):
            if fields:
                for k in range(L):
                    sim.set_field("q0x", k, q0x[k])
                    sim.set_field("q0y", k, q0y[k])
            else:
                G._check(sim.lib.ib_set_frame(sim.h, G.C.c_void_p(frame.data_ptr())), "ib_set_frame")
            sim.advance()
            G._check(sim.lib.ib_get_forces(sim.h, G.C.c_void_p(cx.data_ptr()), G.C.c_void_p(cy.data_ptr())))
            if sim.ntors:
                G._check(sim.lib.ib_get_body_state(sim.h, G.C.c_void_p(th.data_ptr()), None, None))
        f1.record(stream)
        f1.synchronize()
    return f0.elapsed_time(f1) / 1e3, h2d, d2h


def _long_run(p, bodies, steps):
    """A fresh simulation timed from its first step over `steps` steps, with every influence-
    band build and rebuild inside the timed region (wall clock around synchronised steps)."""
    import torch
    from ib_parallel_gb300 import ibgpu as G
    sim = G.Simulation(p, bodies)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        sim.advance()
    sim.synchronize()
    T = time.perf_counter() - t0
    st = sim.influence_stats()
    cr = sim.coarse_stats()
    th = sim.body_state()[0]
    sim.close()
    return {"value": steps / T, "unit": "steps/s", "steps": steps, "seconds": T,
            "band_builds": st["builds"], "band_build_ms": st["build_ms"], "fallbacks": st["fallbacks"],
            "coarse_response_solves": cr["solves"], "coarse_response_ms": cr["ms"],
            "final_theta": [float(x) for x in th],
            "note": "from the impulsive start, host wall clock, every band build inside the region"}


def _beam_workload(args):
    """BASELINE's flexible plate as an Euler-Bernoulli beam (geometry.config_beam_800x400: 51
    points, 25 elements, mass ratio 0.5, EI 1e-3, 800x400 x 5 levels, dt 1e-3): device-timed and
    end-to-end steps/s.  Beams run the FSI iterations from the host each step (the captured
    device loop is the torsional body's)."""
    import torch
    from ib_parallel_gb300 import geometry as GEO
    from ib_parallel_gb300 import ibgpu as G
    p, bodies = GEO.config_beam_800x400()
    sim = G.Simulation(p, bodies)
    stream = torch.cuda.ExternalStream(sim.stream())
    for _ in range(max(3, args.warmup)):
        sim.advance()
    sim.synchronize()
    steps = max(args.steps, 20)
    t, ksp, fsi = _timed_steps(sim, stream, steps)
    te, h2d, d2h = _e2e_steps(sim, stream, steps)
    q = sim.beam_state()[0]
    sim.close()
    return {"workload": "beam800x400", "metric": "FSI steps/s @800x400x5 FP64 (Euler-Bernoulli beam)",
            "value": steps / t, "unit": "steps/s", "steps": steps, "ms_per_step": 1e3 * t / steps,
            "e2e": {"value": steps / te, "unit": "steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "work_per_step": {"ksp_iter": ksp / steps, "fsi_iter": fsi / steps},
            "tip_deflection": float(q[-2]) if len(q) else None,
            "config": {"grid": "800x400", "levels": 5, "body_points": 51, "elements": 25, "mass_ratio": 0.5,
                       "stiffness": 1e-3, "Re": 500, "dt": 1e-3}}


def _subdomain_workload(args):
    """The 800x400 plate through the sub-domain precomputed-Schur method (the reference's
    default, sub_domain = T): the precompute of B over the 121 x 51 cloud of
    geometry.subdomain_800x400 (host wall clock), then device-timed and end-to-end steps/s, the
    FSI iterations on the device from the second step; beside it the same steps with the FSI
    iterations run from the host (per-phase timing on), device-timed."""
    import torch
    from ib_parallel_gb300 import geometry as GEO
    from ib_parallel_gb300 import ibgpu as G
    p, bodies = GEO.config_plate_800x400()
    sim = G.Simulation(p, bodies)
    sim.subdomain_setup(*GEO.subdomain_800x400())
    t0 = time.perf_counter()
    sim.subdomain_precompute()
    pre_s = time.perf_counter() - t0
    stream = torch.cuda.ExternalStream(sim.stream())
    for _ in range(max(3, args.warmup)):
        sim.advance()
    sim.synchronize()
    steps = max(args.steps, 20)
    t, ksp, fsi = _timed_steps(sim, stream, steps)
    te, h2d, d2h = _e2e_steps(sim, stream, steps)
    st = sim.subdomain_stats()
    graphs = sim.step_graph_stats()
    theta = float(sim.body_state()[0][0])
    sim.step_profile(1)   # the same context on: the FSI iterations from the host
    for _ in range(2):
        sim.advance()
    sim.synchronize()
    th, _, _ = _timed_steps(sim, stream, steps)
    sim.close()
    return {"workload": "plate800x400_subdomain", "metric": "FSI steps/s @800x400x5 FP64 (sub-domain method)",
            "value": steps / t, "unit": "steps/s", "steps": steps, "ms_per_step": 1e3 * t / steps,
            "e2e": {"value": steps / te, "unit": "steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "host_fsi_loop": {"value": steps / th, "unit": "steps/s", "ms_per_step": 1e3 * th / steps},
            "step_graph": graphs, "precompute_s": pre_s, "subdomain": st,
            "work_per_step": {"ksp_iter": ksp / steps, "fsi_iter": fsi / steps}, "theta_last": theta,
            "config": {"grid": "800x400", "levels": 5, "body_points": 51, "cloud": "121x51 at 0.01",
                       "droptol": "7.0e-3 (single precision)", "Re": 500, "dt": 1e-3}}


def _adjoint_workload(args):
    """The discrete adjoint on the pitching NACA 0012 (geometry.config_pitching_600x300): 400 steps
    of alpha(t) = 10 deg sin(2 pi 0.2 t) in the body's frame, checkpoints every 20 steps; the
    forward and the reverse sweep timed on the host around synchronised calls, the gradient of
    mean lift and drag with respect to (A, f, phi) through the torch.autograd binding, and the
    amplitude derivative checked by a central difference (step 1e-6) of the GPU forward."""
    import torch
    from ib_parallel_gb300 import autodiff as AD
    from ib_parallel_gb300 import geometry as GEO
    from ib_parallel_gb300 import ibgpu as G
    N, K = 400, 20
    p, bodies = GEO.config_pitching_600x300()
    p.autotune = False

    def run(amp, freq, phase, need_grad):
        sim = G.Simulation(p, bodies)
        frames = AD.pitching_frames(N, p.dt, amp, freq, phase)
        t0 = time.perf_counter()
        forces = AD.FrameForces.apply(frames, sim, K)
        t_fwd = time.perf_counter() - t0
        lift, drag = AD.lift_drag(forces, frames)
        out = {"cl": lift.mean(), "cd": drag.mean(), "t_fwd": t_fwd}
        if need_grad:
            t0 = time.perf_counter()
            (lift.mean() + drag.mean()).backward()
            out["t_bwd"] = time.perf_counter() - t0
        sim.close()
        return out

    amp0 = math.radians(10.0)
    params = [torch.tensor(v, dtype=torch.float64, requires_grad=True) for v in (amp0, 0.2, 0.0)]
    r = run(*params, True)
    grads = [float(q.grad) for q in params]
    h = 1e-6
    jp = run(amp0 + h, 0.2, 0.0, False)
    jm = run(amp0 - h, 0.2, 0.0, False)
    fd = (float((jp["cl"] + jp["cd"]).detach()) - float((jm["cl"] + jm["cd"]).detach())) / (2 * h)
    return {"workload": "pitching600x300_adjoint", "metric": "adjoint/forward cost (reverse sweep time over forward time)",
            "value": r["t_bwd"] / r["t_fwd"], "unit": "x", "higher_is_better": False,
            "forward_s": r["t_fwd"], "backward_s": r["t_bwd"], "forward_steps_per_s": N / r["t_fwd"],
            "mean_cl": float(r["cl"].detach()), "mean_cd": float(r["cd"].detach()),
            "gradient_of_mean_cl_plus_cd": {"amplitude_rad": grads[0], "frequency": grads[1], "phase": grads[2]},
            "central_difference_amplitude": {"value": fd, "rel_err": abs(grads[0] - fd) / abs(fd)},
            "config": {"grid": "600x300", "levels": 4, "body": f"NACA 0012, {bodies[0].npts} points (2 grid spacings)",
                       "Re": 200, "dt": 0.002, "steps": N, "checkpoint_every": K,
                       "kinematics": "alpha = 10 deg sin(2 pi 0.2 t) about the quarter chord, in the body frame"}}


def _c1_workload(args):
    """The rigid cylinder (400x200 x 3 levels, 157 points, Re=100, dt=0.004) through the
    stationary-body direct solve: device-timed and end-to-end steps/s, and the oracle timed on
    whole steps after its own preprocessing."""
    import torch
    from ib_parallel_gb300 import geometry as GEO
    from ib_parallel_gb300 import ibgpu as G
    p, bodies = GEO.config_cylinder_400x200()
    p.num_stat = True
    sim = G.Simulation(p, bodies)
    stream = torch.cuda.ExternalStream(sim.stream())
    for _ in range(max(3, args.warmup)):
        sim.advance()
    sim.synchronize()
    steps = max(args.steps, 20)
    t, _, _ = _timed_steps(sim, stream, steps)
    te, h2d, d2h = _e2e_steps(sim, stream, steps)
    cx, cy = sim.forces()
    sim.close()
    out = {"workload": C1_WORKLOAD, "metric": "steps/s @400x200x3 FP64 (direct solve)", "value": steps / t,
           "unit": "steps/s", "steps": steps, "ms_per_step": 1e3 * t / steps,
           "e2e": {"value": steps / te, "unit": "steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
           "config": {"grid": "400x200", "levels": 3, "body_points": 157, "Re": 100, "dt": 0.004,
                      "solve": "num_stat (Cholesky of the assembled Schur matrix at step 1)"},
           "cd_cl_last": [float(cx[0]), float(cy[0])],
           "gmres_note": "with GMRES(30) at rtol 1e-10 the Schur solve of this body (points one grid spacing "
                         "apart, condition ~6e4) does not converge in thousands of iterations, in the oracle "
                         "as on the GPU (ib_advance returns IB_ERR_GMRES); the direct solve is the usable path"}
    if not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        times, o = _oracle_steps(p, bodies, cores, untimed=1, budget_s=8.0, min_steps=5)
        cpu = len(times) / float(np.sum(times))
        out["cpu_baseline"] = {"value": cpu, "unit": "steps/s", "cores": cores, "kind": "port",
                               "sample": f"oracle port, {len(times)} whole steps (2..{len(times) + 1}) after its "
                                         f"step-1 preprocessing, {cores} threads"}
        out["gpu_over_cpu"] = out["value"] / cpu
        out["e2e_over_cpu"] = out["e2e"]["value"] / cpu
    return out


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
    for _ in range(args.warmup):
        sim.advance()
    sim.synchronize()
    mv0, passes0 = sim.work()
    launches0 = G.launch_count()
    _barrier(world)
    torch.cuda.synchronize()
    if args.host_fsi_loop:
        sim.step_profile(1)
    with Clocks(local) as clk:
        if args.profile_window:
            torch.cuda.profiler.start()
        clk.begin()
        t_local, ksp_sum, fsi_sum = _timed_steps(sim, stream, args.steps)
        clk.end()
        if args.profile_window:
            torch.cuda.profiler.stop()
    if args.host_fsi_loop:
        sim.step_profile(0)
    torch.cuda.synchronize()
    t_s = _barrier_max(t_local, world)
    mv1, passes1 = sim.work()
    launches_timed = G.launch_count() - launches0
    mv_per_step = (mv1 - mv0) / args.steps
    passes_timed = [b - a for a, b in zip(passes0, passes1)]
    value = world * args.steps / t_s

    # ---- end to end through the C ABI with host buffers
    _barrier(world)
    e2e_local, h2d, d2h = _e2e_steps(sim, stream, args.steps)
    e2e_s = _barrier_max(e2e_local, world)
    e2e_value = world * args.steps / e2e_s
    _barrier(world)
    e2f_local, h2d_f, d2h_f = _e2e_steps(sim, stream, args.steps, fields=True)
    e2f_s = _barrier_max(e2f_local, world)

    # ---- roofline of the dominant kernel (the DST-I x pass, the largest share of the step's
    # launch list), timed alone: 20 back-to-back full passes over the finest grid with CUDA
    # events on the simulation's stream
    m, n, L = p.m, p.n, p.mgridlev
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
    # the step against HBM on the reference's accounting: the compulsory bytes of the
    # routines it calls, with one matrix-free Schur product per Krylov iteration
    fixed_b, matvec_b = _algorithmic_bytes(m, n, L, sim.nf)
    ksp_per_step = ksp_sum / args.steps
    step_bytes = fixed_b + ksp_per_step * matvec_b
    step_achieved = step_bytes / (t_s / args.steps) / 1e9
    result = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded hinged plate, impulsive start)",
        "config": {"workload": WORKLOAD, "grid": "800x400", "levels": 5, "body_points": 51, "Re": 500,
                   "dt": 1e-3, "gmres_rtol": 1e-10, "fsi_tol": 1e-10, "parallelism": f"replicas{world}",
                   "l2": "working set (~330 MB of state, tables and scratch + 160 MB influence band) larger "
                         "than L2 (129 MB)"},
        "clocks": clk.summary(),
        "e2e": {"value": e2e_value, "unit": "steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "input": "the step's frame motion (u, v, angular velocity) through ib_set_frame"},
        "e2e_q0_fields": {"value": world * args.steps / e2f_s, "unit": "steps/s", "h2d_bytes_per_step": h2d_f,
                          "d2h_bytes_per_step": d2h_f,
                          "input": "the frame fluxes q0 of all levels uploaded by ib_set_field each step"},
        "gpu_launches": launches_timed,
        "work_per_step": {"schur_matvecs": mv_per_step, "ksp_iter": ksp_per_step,
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
        "step_roofline": {"bound": "hbm", "achieved": step_achieved, "peak": peak, "unit": "GB/s",
                          "frac": step_achieved / peak, "bytes_per_step": step_bytes,
                          "fixed_bytes": fixed_b, "bytes_per_krylov_iteration": matvec_b,
                          "krylov_iterations_per_step": ksp_per_step,
                          "note": "compulsory bytes of the reference's step (predictor on every level, two "
                                  "vort2flux, correction, one matrix-free Schur product per Krylov iteration) "
                                  "over the measured step time; the influence matrix replaces the per-iteration "
                                  "work, so this is a step-level figure, not a kernel roofline"},
        "tridiagonal_pass_us": 1e3 * t_tri,
        "nonlinear_stencil_us": {"plain_loads": 1e3 * sim.time_pass(4, 10), "bulk_copies": 1e3 * sim.time_pass(5, 10),
                                 "note": "the predictor's fused nonlinear + rot stencil of all five levels, inputs "
                                         "from HBM; bulk_copies stages the interior tiles' rows with cp.async.bulk "
                                         "(same bits, checked)"},
        "pressure": _pressure_leg(sim, p),
        "schur_stages_us": sim.profile_schur(20),
        "influence": dict(sim.influence_stats(), coarse_responses=sim.coarse_stats()),
        "step_graph": sim.step_graph_stats(),
        "launch_shapes": sim.launch_shapes(),
        "step_phases_us": _step_phases(sim, 5),
        "step_phases_device_loop_us": _step_phases(sim, 5, device_loop=True),
    }
    sim.close()
    result["phase_by_phase"] = _phased_rate(p, bodies, args)
    if not args.no_matrix_free:
        result["matrix_free"] = _matrix_free_rate(p, bodies, args)
    if args.long_steps > 0:
        result["long_run"] = _long_run(p, bodies, args.long_steps)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        times, o = _oracle_steps(p, bodies, cores, budget_s=12.0, min_steps=3)
        cpu_val = len(times) / float(np.sum(times))
        result["cpu_baseline"] = {
            "value": cpu_val, "unit": "steps/s", "cores": cores, "kind": "port",
            "sample": f"oracle port (numpy + scipy.fft, {cores} threads; the Fortran reference cannot be built "
                      f"here): {len(times)} whole time steps from the impulsive start (1..{len(times)}), each "
                      f"with its own GMRES and FSI loop, {np.sum(times):.1f} s"}
        result["speedup_vs_cpu_port"] = {
            "e2e": e2e_value / cpu_val, "device": value / cpu_val,
            "same_algorithm": (result["matrix_free"]["value"] / cpu_val) if "matrix_free" in result else None,
            "note": "same_algorithm: the GPU with the matrix-free Schur operator the port runs"}
    if rank == 0 and world == 1 and not args.no_c1:
        result["workloads"] = {C1_WORKLOAD: _c1_workload(args)}
    if rank == 0 and world == 1 and not args.no_c1:
        result.setdefault("workloads", {})["beam800x400"] = _beam_workload(args)
        result["workloads"]["plate800x400_subdomain"] = _subdomain_workload(args)
        result["workloads"]["pitching600x300_adjoint"] = _adjoint_workload(args)
    if rank == 0 and world == 1 and args.ensemble > 0:
        result.setdefault("workloads", {})["ensemble"] = _ensemble(args)
    if rank == 0:
        print(json.dumps(result))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def _pressure_leg(sim, p):
    """calculate_pressure on the current state (every level), timed with CUDA events on the
    simulation's stream after one untimed call, and the A/B of its x transform (800 x 400 cells
    times the 800 x 800 DST-I matrix) on the FP64 tensor cores and with FP64 FMAs."""
    import torch
    stream = torch.cuda.ExternalStream(sim.stream())
    sim.pressure()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    reps = 5
    for _ in range(reps):
        sim.pressure()
    e1.record(stream)
    e1.synchronize()
    t_mma = sim.time_pass(2, 20)
    t_fma = sim.time_pass(3, 20)
    flops = 2.0 * p.n * p.m * p.m
    return {"recovery_ms": e0.elapsed_time(e1) / reps, "levels": p.mgridlev,
            "x_transform_us": {"dmma": 1e3 * t_mma, "fma": 1e3 * t_fma},
            "x_transform_tflops": {"dmma": flops / (t_mma * 1e-3) / 1e12, "fma": flops / (t_fma * 1e-3) / 1e12},
            "note": "recovery_ms includes copying every level's pressure to the host"}


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


def _phased_rate(p, bodies, args):
    """Steps/s of the same workload with the step run phase by phase (IB_WHOLE_STEP=0 at
    creation: predictor, vort2flux, device FSI loop and correction as separate graphs with a
    host readback between the loop and the correction), timed the same way."""
    import torch
    from ib_parallel_gb300 import ibgpu as G
    old = os.environ.get("IB_WHOLE_STEP")
    os.environ["IB_WHOLE_STEP"] = "0"
    try:
        sim = G.Simulation(p, bodies)
    finally:
        if old is None:
            del os.environ["IB_WHOLE_STEP"]
        else:
            os.environ["IB_WHOLE_STEP"] = old
    stream = torch.cuda.ExternalStream(sim.stream())
    for _ in range(args.warmup):
        sim.advance()
    sim.synchronize()
    t, _, _ = _timed_steps(sim, stream, args.steps)
    stats = sim.step_graph_stats()
    sim.close()
    return {"value": args.steps / t, "unit": "steps/s", "steps_by_kind": stats}


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


def run_ensemble_only(nsim, steps, warmup):
    """The batched ensemble (geometry.config_ensemble): nsim simulations with uneven grids and
    bodies, advanced by ib_batch_advance for `warmup` then `steps` batch steps, and the same
    simulations advanced one at a time through ib_advance for `steps` steps each (the plain GPU
    path run one simulation at a time).  Host wall clock around synchronised calls (every call
    returns with its work complete).  Prints one JSON object."""
    import torch
    from ib_parallel_gb300 import geometry as GEO
    from ib_parallel_gb300 import ibgpu as G
    torch.cuda.set_device(0)
    runs = GEO.config_ensemble(nsim)
    t0 = time.perf_counter()
    batch = G.Batch(runs)
    t_create = time.perf_counter() - t0
    t0 = time.perf_counter()
    for _ in range(warmup):
        batch.advance()
    t_warm = time.perf_counter() - t0
    launches0 = G.launch_count()
    t0 = time.perf_counter()
    for _ in range(steps):
        batch.advance()
    t_batch = time.perf_counter() - t0
    launches = G.launch_count() - launches0
    t0 = time.perf_counter()
    for s in batch.sims:
        for _ in range(steps):
            s.advance()
    t_seq = time.perf_counter() - t0
    grids = {}
    for p, b in runs:
        grids[f"{p.m}x{p.n}"] = grids.get(f"{p.m}x{p.n}", 0) + 1
    out = {"workload": "ensemble", "metric": "sim-steps/s, batched ensemble FP64", "nsim": nsim, "steps": steps,
           "warmup": warmup, "value": nsim * steps / t_batch, "unit": "sim-steps/s",
           "sequential": {"value": nsim * steps / t_seq, "unit": "sim-steps/s",
                          "note": "the same simulations, one at a time through ib_advance"},
           "batch_over_sequential": t_seq / t_batch, "gpu_launches_per_batch_step": launches / steps,
           "create_s": t_create, "warmup_s": t_warm, "grids": grids,
           "body_points": [min(len(b[0].x) for _, b in runs), max(len(b[0].x) for _, b in runs)],
           "config": "seeded per simulation: Re U[100,500], mass ratio logU[0.1,2], stiffness logU[1e-4,1e-2], "
                     "incidence U[0,20] deg, grid U{256x128,384x192,512x256}, 3 levels, dt 2e-3",
           "timing": "host wall clock around synchronised calls, CUDA_DEVICE_MAX_CONNECTIONS=" +
                     os.environ.get("CUDA_DEVICE_MAX_CONNECTIONS", "default")}
    batch.close()
    print(json.dumps(out))
    return 0


def _ensemble(args):
    """Runs the ensemble leg in its own process, with 32 hardware work queues so that the
    simulations' streams run side by side (the variable must be set before CUDA starts)."""
    env = dict(os.environ, CUDA_DEVICE_MAX_CONNECTIONS="32")
    cmd = [sys.executable, str(ROOT / "bench.py"), "--ensemble-only", str(args.ensemble),
           "--steps", str(max(3, min(args.steps, 10))), "--warmup", "3"]
    r = subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=1200)
    if r.returncode != 0:
        return {"error": (r.stderr or r.stdout)[-400:]}
    return json.loads(r.stdout.strip().splitlines()[-1])


def run_roofline_only():
    """The x pass of the roofline alone, 20 launches over cold inputs inside a profiler window
    (ncu --profile-from-start off captures exactly these launches)."""
    import torch
    from ib_parallel_gb300 import geometry as GEO
    from ib_parallel_gb300 import ibgpu as G
    torch.cuda.set_device(0)
    p, bodies = GEO.config_plate_800x400()
    p.autotune = 0
    sim = G.Simulation(p, bodies)
    sim.time_pass(0, 2)
    sim.synchronize()
    torch.cuda.profiler.start()
    t_x = sim.time_pass(0, 20)
    torch.cuda.profiler.stop()
    ns = (p.m - 1) * (p.n - 1)
    print(json.dumps({"kernel": "k_dst_x", "avg_launch_us": 1e3 * t_x, "bytes_per_launch": 16.0 * ns,
                      "achieved_gbs": 16.0 * ns / (t_x * 1e-3) / 1e9}))
    sim.close()
    return 0


def run_profile_leg(which):
    """One short leg inside a cudaProfilerStart/Stop window, for ncu --profile-from-start off:
    'adjoint' brackets the reverse sweep of 20 steps of the pitching NACA 0012 (one segment: the
    recompute, then the 20 reverse steps); 'band' the first step of the 800x400 plate, which builds
    the influence band (capture its first launches with ncu -c); 'subdomain' three steps of the
    800x400 plate through the sub-domain method after its precompute and three warm-up steps, the
    FSI iterations run from the host so that each kernel is a launch of its own."""
    import torch
    from ib_parallel_gb300 import autodiff as AD
    from ib_parallel_gb300 import geometry as GEO
    from ib_parallel_gb300 import ibgpu as G
    if which == "band":
        p, bodies = GEO.config_plate_800x400()
        p.autotune = False
        sim = G.Simulation(p, bodies)
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        sim.advance()
        torch.cuda.profiler.stop()
        print(json.dumps({"leg": "band build (first step)", "influence": sim.influence_stats()}))
        sim.close()
        return 0
    if which == "subdomain":
        p, bodies = GEO.config_plate_800x400()
        p.autotune = False
        sim = G.Simulation(p, bodies)
        sim.subdomain_setup(*GEO.subdomain_800x400())
        sim.subdomain_precompute()
        for _ in range(3):
            sim.advance()
        sim.step_profile(1)
        sim.synchronize()
        torch.cuda.profiler.start()
        for _ in range(3):
            sim.advance()
        sim.synchronize()
        torch.cuda.profiler.stop()
        print(json.dumps({"leg": "sub-domain steps 4-6, FSI iterations from the host",
                          "counters": sim.counters()}))
        sim.close()
        return 0
    p, bodies = GEO.config_pitching_600x300()
    p.autotune = False
    sim = G.Simulation(p, bodies)
    frames = AD.pitching_frames(20, p.dt, math.radians(10.0), 0.2, 0.0).numpy()
    forces = sim.adjoint_forward(frames, 20)
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    t0 = time.perf_counter()
    sim.adjoint_backward(np.ones_like(forces))
    dt = time.perf_counter() - t0
    torch.cuda.profiler.stop()
    print(json.dumps({"leg": which + " backward, 20 steps", "seconds": dt}))
    sim.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-matrix-free", action="store_true",
                    help="skip timing the matrix-free Schur operator beside the default one")
    ap.add_argument("--no-c1", action="store_true", help="skip the 400x200x3 rigid-cylinder workload")
    ap.add_argument("--long-steps", type=int, default=1000,
                    help="steps of the long run from the impulsive start with every band build timed (0: skip)")
    ap.add_argument("--profile-window", action="store_true",
                    help="bracket the timed steps with cudaProfilerStart/Stop (for ncu --profile-from-start off)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="run with the default launch shapes instead of tuning them by timing at creation (for "
                         "profiler captures, whose replays would mislead the tuner)")
    ap.add_argument("--host-fsi-loop", action="store_true",
                    help="run the timed steps with per-phase timing on, so that the FSI iterations run from the "
                         "host and each of their kernels is a separate launch (a profiler lists kernels inside "
                         "the device loop's graph node only as the graph)")
    ap.add_argument("--ensemble", type=int, default=256,
                    help="simulations of the batched-ensemble leg (0: skip)")
    ap.add_argument("--ensemble-only", type=int, default=0, help=argparse.SUPPRESS)
    ap.add_argument("--roofline-only", action="store_true",
                    help="only time the single x pass of the roofline (inside a profiler window: the command "
                         "the ncu traffic capture of that pass runs)")
    ap.add_argument("--profile-leg", choices=["adjoint", "band", "subdomain"], default=None,
                    help="only run one short leg inside a profiler window (the command of an ncu launch list)")
    args = ap.parse_args()
    world, rank, local = _dist()
    if args.profile_leg:
        return run_profile_leg(args.profile_leg)
    if args.roofline_only:
        return run_roofline_only()
    if args.ensemble_only:
        return run_ensemble_only(args.ensemble_only, args.steps, args.warmup)
    if args.impl == "reference":
        return run_reference(args, world, rank)
    return run_gpu(args, world, rank, local)


if __name__ == "__main__":
    sys.exit(main())
