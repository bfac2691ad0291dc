#!/usr/bin/env python
"""Benchmark of the FIPI step on GB300.

Workload (default): 256^3 periodic grid with 20,000 spheres of radius 4 dx,
phi0 = U(-0.05, 0.05), M = eps = sigma = mu = 1, dt = 1e-3 (seeded synthetic
inputs of that shape).  A step is one iteration of the reference's loop body
(Cahn-Hilliard, Stokes projection, two Heun particle stages).

Printed JSON line (rank 0):
  value        mixed-precision steps/s, inputs resident in HBM, CUDA events
               on the library's stream, max over ranks (N replicas: sum)
  e2e          the same metric through the C ABI with host buffers: every
               step uploads the particle state and reads positions, forces
               and the mass back
  fp64         plain FP64 form steps/s and the mixed/FP64 ratio
  error        mixed vs FP64 after `--err-steps` steps from the same state
  roofline     dominant kernel: algorithmic bytes per launch / CUDA-event
               duration against the measured HBM copy bandwidth
  step_roofline  the whole step: the ideal fused pipeline's 44 field passes
               and this design's pass traffic, times steps/s, against it
  cpu_baseline the CPU oracle timed on this host on a bounded sample

`--impl reference` times the reference's CPU path (the oracle) instead.
Under torchrun every rank runs an independent replica (different seed).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))

METRIC = "steps/s 256³+20k particles, mixed vs FP64 at φ err≤1e-4; adjoint/forward ratio"


def peaks():
    try:
        d = json.loads((REPO / "MEASURED_PEAKS.json").read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def aggregate_replicas(elapsed, steps, ws, dist=None, device="cuda"):
    """Whole-job steps/s of `ws` independent replicas: all ranks' steps over
    the slowest rank's time (max over ranks)."""
    if dist is not None and ws > 1:
        import torch

        t = torch.tensor([float(elapsed)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t.item())
    return ws * steps / elapsed, elapsed


def seeded(w, seed):
    import fipi_gb300 as F

    P = w.params()
    c = F.seed_phase(P, seed, w.phi_mean, w.phi_amp)
    p, r, ct = F.seed_particles(P, seed + 1000, w.radius_range, w.theta_range_deg,
                                allow_overlap=w.radius_range is not None)
    return P, c, p, (r if w.radius_range else None), (ct if w.theta_range_deg else None)


def timed_steps(sim, n, torch):
    """Device time of n steps on the library's stream (CUDA events)."""
    stream = torch.cuda.ExternalStream(sim.stream())
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    sim.sync()
    e0.record(stream)
    sim.step_async(n)
    e1.record(stream)
    sim.sync()
    return e0.elapsed_time(e1) / 1e3


def adjoint_ratio(F, P, c, p, r, ct, device, torch, steps, traj_steps):
    """FP64 adjoint cost against the FP64 forward step on the same state,
    both timed with CUDA events on the library's stream.

    adjoint_step: one fipi_adjoint_step (checkpoint load, the step recomputed
    with its intermediates kept, the reverse pass); forward: one plain FP64
    step.  trajectory: fipi_trajectory_forward + fipi_trajectory_backward
    over `traj_steps` steps (sqrt(N) checkpoints) against as many plain
    steps."""
    import numpy as np

    s = F.Simulation(P, "fp64", device=device)
    s.set_phase(c)
    s.set_particles(p, r, ct)
    s.step(2)  # into the SBDF2 regime
    fwd = timed_steps(s, steps, torch) / steps
    s.checkpoint_reserve(2)
    s.checkpoint_save(0)
    s.step(1)
    s.checkpoint_save(1)
    dc = np.random.default_rng(0).standard_normal(s.V)
    stream = torch.cuda.ExternalStream(s.stream())

    def on_stream(fn):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        s.sync()
        e0.record(stream)
        fn()
        e1.record(stream)
        s.sync()
        return e0.elapsed_time(e1) / 1e3

    times = []
    for _ in range(steps + 1):
        s.checkpoint_load(1)
        s.adjoint_seed(dc)
        times.append(on_stream(lambda: s.adjoint_step(0)))
    adj = statistics.median(times[1:])
    s.checkpoint_load(0)
    tf = on_stream(lambda: s.trajectory_forward(traj_steps))
    tb = on_stream(lambda: s.trajectory_backward(dc))
    s.close()
    stride = int(np.ceil(np.sqrt(traj_steps)))
    return {"form": "fp64", "clock": "CUDA events on the library stream (forward and adjoint)",
            "forward_ms": fwd * 1e3, "adjoint_step_ms": adj * 1e3,
            "adjoint_step_over_forward": adj / fwd,
            "trajectory": {"steps": traj_steps, "stride": stride,
                           "slots": -(-traj_steps // stride) + stride + 1,
                           "forward_s": tf, "backward_s": tb,
                           "gradient_over_forward": (tf + tb) / (traj_steps * fwd)}}


def grad_bench(F, name, device, torch, steps=None, fd_steps=None, fd_h=None,
               fd=("phi0", "mobility", "sigma", "cos_theta")):
    """Gradient benchmark of a workload through the FP64 adjoint with sqrt(N)
    checkpointing (fipi_gradient harness, torch loss on the GPU):

      cfg4_128  128^3, 2000 spheres, 200 steps, a checkpoint every 20 steps;
                loss ||S(k) - S_target(k)||^2, the target from a second seed;
                gradients w.r.t. phi0, M, sigma and every cos theta
      cfg5_256  the coated droplet (256^3, 20,000 spheres, g along -z),
                1000 steps, ceil(sqrt(1000)) = 32 checkpoints; loss
                interfacial area + centroid height; gradients w.r.t. sigma
                and every cos theta; the mixed forward against the FP64 one

    Reports the gradient's wall time over the plain FP64 forward's (both
    host wall clocks around synchronous calls), the device memory the
    context holds with its checkpoint slots, and the central-difference
    agreement of each gradient (relative step h).  Config 5's finite
    differences run over its first `fd_steps` steps (default 100): over the
    whole rollout particles cross the attachment force's jump at |d| = r
    (element.cpp:84-89: f_mag drops from -A pi r sigma to 0), where the
    trajectory is not differentiable and a central difference across the
    jump measures the jump, not the derivative (over all 1000 steps the
    differences converge to the adjoint's values as h shrinks: run with
    --grad cfg5_256 --grad-fd-steps 1000 --grad-fd-h 1e-7)."""
    import numpy as np

    from fipi_gb300 import gradcheck as G
    from fipi_gb300 import inputs

    w = F.workload(name)
    nsteps = steps or w.steps
    dev = f"cuda:{device}"
    if name == "cfg5_256":
        P, c0, p0, r, ct = inputs.initial_state(w, 1)
        stride = 0  # ceil(sqrt(N))
        h = fd_h or {"sigma": 1e-6, "cos_theta": 1e-4}
        which = tuple(x for x in fd if x in ("sigma", "cos_theta"))
        fd_n = fd_steps or min(nsteps, 100)

        def loss_fn(c):
            return G.area_plus_height(c, P)
    else:
        P, c0, p0, r, ct = seeded(w, 1)
        stride = 20
        h = fd_h or 1e-6
        which = fd
        fd_n = fd_steps or nsteps
        with F.Simulation(P, "fp64", device=device) as s:  # the target: the same run from a second seed
            Pt, ct0, pt, rt, ctt = seeded(w, 2)
            s.set_phase(ct0)
            s.set_particles(pt, rt, ctt)
            s.step(nsteps)
            target = G.structure_factor(torch.from_numpy(s.get_phase()).to(dev), (P.nz, P.ny, P.nx))

        def loss_fn(c):
            return G.structure_loss(c, target, (P.nz, P.ny, P.nx))
    init = G.InitialState(p0=p0, r=r, cos_theta=np.zeros(w.n_p) if ct is None else ct)
    out = {"workload": name, "steps": nsteps, "grid": f"{w.nx}x{w.ny}x{w.nz}", "particles": w.n_p,
           "loss": "interfacial area + centroid height" if name == "cfg5_256" else "||S(k) - S_target(k)||^2"}
    with F.Simulation(P, "fp64", device=device) as s:
        G._start(s, c0, init)
        s.sync()
        t0 = time.perf_counter()
        s.step(nsteps)
        fwd = time.perf_counter() - t0
        end64 = (s.get_phase(), s.get_velocity(), s.get_particles()[0])
        t0 = time.perf_counter()
        L0, g_c, g_th, g_ct = G.loss_and_grads(s, c0, init, nsteps, loss_fn, stride, dev)
        s.sync()
        tg = time.perf_counter() - t0
        ck = s.checkpoint_bytes()
        hbm = s.device_bytes()
        slots = -(-nsteps // (stride or int(np.ceil(np.sqrt(nsteps))))) + (stride or int(np.ceil(np.sqrt(nsteps)))) + 1
        out.update({"forward_s": fwd, "gradient_s": tg, "gradient_over_forward": tg / fwd,
                    "checkpoint_stride": stride or int(np.ceil(np.sqrt(nsteps))), "checkpoint_slots": slots,
                    "checkpoint_slot_bytes": ck, "device_bytes": hbm, "loss_value": L0,
                    "grad_norms": {"phi0": float(np.linalg.norm(g_c)), "mobility": float(g_th[0]),
                                   "sigma": float(g_th[1]), "cos_theta": float(np.linalg.norm(g_ct))}})
        if which:
            chk = G.fd_all(s, c0, init, fd_n, loss_fn, h, stride if fd_n == nsteps else 0, seed=7, device=dev,
                           which=which, grads=(L0, g_c, g_th, g_ct) if fd_n == nsteps else None)
            out["fd"] = {k: v for k, v in chk.items() if k != "loss"}
            out["fd_steps"] = fd_n
            out["fd_max_rel"] = max(v["rel"] for k, v in chk.items() if k != "loss")
    if name == "cfg5_256":
        with F.Simulation(P, "mixed", device=device) as s:
            G._start(s, c0, init)
            s.step(nsteps)
            a = (s.get_phase(), s.get_velocity(), s.get_particles()[0])
        L = np.array([P.lx, P.ly, P.lz])
        dp = np.abs(a[2] - end64[2]).reshape(-1, 3)
        dp = np.minimum(dp, L - dp)
        out["mixed_vs_fp64"] = {"steps": nsteps,
                                "phi_rel_l2": float(np.linalg.norm(a[0] - end64[0]) / np.linalg.norm(end64[0])),
                                "u_rel_l2": float(np.linalg.norm(a[1] - end64[1]) / np.linalg.norm(end64[1])),
                                "pos_max_abs": float(dp.max())}
    return out


def kernel_stats(sim):
    return sim.kernel_stats()


def launch_count(sim):
    return sim.launch_count()


def set_timing(sim, on):
    sim.set_kernel_timing(on)


def committed_traffic(kernel, workload):
    """DRAM bytes per launch from the committed ncu summary, if it covers this kernel."""
    try:
        for line in (REPO / "profiles" / "dram_traffic.txt").read_text().splitlines():
            if line.startswith("#") or not line.strip():
                continue
            w, k, v = line.split("\t")
            if w == workload and k == kernel:
                return float(v)
    except (OSError, ValueError):
        pass
    return None


# FFT threads of the reference's CPU step: fftw_plan_with_nthreads(4)
# (main.cpp:70 of the reference); everything else there is single-threaded.
CPU_FFT_THREADS = 4


class CpuStep:
    """The reference's CPU step on one workload: the reference itself,
    compiled in place into oracle/_ref where its sources are present
    (kind "reference"), else the oracle's C restatement of it (kind
    "port").  Inputs come from the oracle's restatement of the seeded
    generators, so nothing here loads the CUDA library."""

    def __init__(self, w, threads=CPU_FFT_THREADS):
        sys.path.insert(0, str(REPO / "oracle"))
        import oracle as O

        self.O, self.w, self.threads = O, w, threads
        self.kind, self.ref = "port", None
        if O.reference_available() and w.radius_range is None and w.theta_range_deg is None:
            try:
                self.ref = O.Ref(w.name)
                self.kind = "reference"
            except Exception:
                self.ref = None
        if self.ref is None:
            self.port = O.Port(w.params(), threads=threads)

    def seeded(self, seed):
        return self.O.seeded_state(self.w, seed)

    def set_state(self, c, p, r, ct):
        if self.ref is not None:
            self.ref.init(c, p, r)
        else:
            self.port.set_state(c, p, r, ct)

    def step(self, n):
        st = (self.ref or self.port).step(n)
        if st != 0:
            raise RuntimeError(f"CPU step failed with status {st}")

    def state(self):
        e = self.ref or self.port
        return e.phase(), e.velocity(), e.particles()[0]

    def describe(self):
        if self.kind == "reference":
            return "the reference's own step (compiled in place, FFTW-API shim)"
        return "C restatement of the reference step (full-complex C2C FFTs as the reference)"


def cpu_baseline(w, seed, steps=1):
    """The reference's CPU step on the same workload and seed, 1 warm-up step
    (t = 0, the IMEX start) and `steps` timed steps.  Returns the baseline
    record and the CPU state after those steps (the oracle's end state the
    GPU forms are compared with)."""
    eng = CpuStep(w)
    P, c, p, r, ct = eng.seeded(seed)
    eng.set_state(c, p, r, ct)
    eng.step(1)
    t0 = time.perf_counter()
    eng.step(steps)
    dt = time.perf_counter() - t0
    rec = {"value": steps / dt, "unit": "steps/s", "cores": eng.threads, "kind": eng.kind,
           "sample": f"{steps} step(s) of the {w.name} workload after 1 warm-up step; {eng.describe()}; "
                     f"{eng.threads} threads in the transforms as the reference configures FFTW "
                     f"(main.cpp:70), the rest single-threaded"}
    return rec, eng.state(), 1 + steps


def error_vs_oracle(F, w, P, c, p, r, ct, device, ref_state, nsteps):
    """Both GPU forms after `nsteps` steps from the seeded state, against the
    CPU oracle's state after the same steps: relative L2 of phi, u and
    positions, and the largest position difference."""
    import numpy as np

    rc, ru, rp = ref_state
    L = np.array([P.lx, P.ly, P.lz])
    out = {"steps": nsteps, "oracle": "CPU step of the reference (bench cpu_baseline leg)"}
    for prec in ("fp64", "mixed"):
        with F.Simulation(P, prec, device=device) as s:
            s.set_phase(c)
            s.set_particles(p, r, ct)
            s.step(nsteps)
            gc, gu, gp = s.get_phase(), s.get_velocity(), s.get_particles()[0]
        dp = np.abs(gp - rp).reshape(-1, 3)
        dp = np.minimum(dp, L - dp)
        out[prec] = {"phi_rel_l2": float(np.linalg.norm(gc - rc) / np.linalg.norm(rc)),
                     "u_rel_l2": float(np.linalg.norm(gu - ru) / max(np.linalg.norm(ru), 1e-300)),
                     "pos_rel_l2": float(np.linalg.norm(dp) / np.linalg.norm(rp)),
                     "pos_max_abs": float(dp.max()) if dp.size else 0.0}
    return out


def run_reference(args):
    """The reference's CPU path on the host cores (the oracle's C
    restatement, or the reference compiled in place where its sources are
    present), on the same workload, seed and metric as the GPU arm.  Loads
    no part of the CUDA library: the workload table is plain Python and the
    inputs come from the oracle's restatement of the seeded generators."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from fipi_gb300.params import workload

    w = workload(args.workload)
    warm = min(args.warmup, 1)
    steps = max(1, min(args.steps, 2))
    eng = CpuStep(w)
    P, c, p, r, ct = eng.seeded(1)
    eng.set_state(c, p, r, ct)
    eng.step(warm)
    t0 = time.perf_counter()
    eng.step(steps)
    dt = time.perf_counter() - t0
    v = steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "steps/s", "n_gpus": 0,
        "steps": steps, "warmup": warm, "ms_per_step": 1e3 * dt / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": w.name, "grid": f"{w.nx}x{w.ny}x{w.nz}", "particles": w.n_p},
        "cpu_baseline": {"value": v, "unit": "steps/s", "cores": eng.threads, "kind": eng.kind,
                         "sample": f"{steps} timed step(s) after {warm} warm-up of the {w.name} workload; "
                                   f"{eng.describe()}; {eng.threads} threads in the transforms as the "
                                   f"reference configures FFTW (main.cpp:70), the rest single-threaded"},
        "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_profile(args):
    """Set-up, --warmup steps, then --profile steps of the --form form, nothing
    else: the command ncu captures (launch counts are printed to stderr so the
    capture's -s/-c can skip the set-up and warm-up)."""
    import fipi_gb300 as F

    w = F.workload(args.workload)
    P, c, p, r, ct = seeded(w, 1)
    sim = F.Simulation(P, args.form)
    sim.set_phase(c)
    sim.set_particles(p, r, ct)
    sim.step(args.warmup)
    n0 = launch_count(sim)
    sim.step(args.profile)
    n1 = launch_count(sim)
    print(json.dumps({"profile": args.profile, "form": args.form, "workload": w.name,
                      "launches_before": n0, "launches_per_step": (n1 - n0) / args.profile}),
          file=sys.stderr, flush=True)
    sim.close()
    return 0


def run_gpu(args):
    import numpy as np
    import torch

    import fipi_gb300 as F

    ws, rank, local = dist_env()
    dist = None
    if ws > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(local)
    w = F.workload(args.workload)
    seed = 1 + rank
    P, c, p, r, ct = seeded(w, seed)

    def barrier():
        if dist is not None:
            dist.barrier()
            torch.cuda.synchronize()

    # ---- headline: mixed form, inputs resident
    sim = F.Simulation(P, "mixed", device=local)
    sim.set_phase(c)
    sim.set_particles(p, r, ct)
    sim.step(args.warmup)
    barrier()
    l0 = launch_count(sim)
    with ClockSampler(local) as clk:
        elapsed = timed_steps(sim, args.steps, torch)
    launches = launch_count(sim) - l0
    barrier()
    value, elapsed = aggregate_replicas(elapsed, args.steps, ws, dist)

    # ---- per-kernel CUDA-event timing (separate region; events add overhead)
    set_timing(sim, True)
    sim.step(args.kernel_steps)
    ks = kernel_stats(sim)
    set_timing(sim, False)

    # ---- e2e through the C ABI with host buffers
    pos, fpp, _ = sim.get_particles()
    rr = r if r is not None else np.full(w.n_p, P.r_p)
    cc = ct if ct is not None else np.zeros(w.n_p)
    sim.sync()
    e2e_steps = max(1, min(args.steps, args.e2e_steps))
    # the step is enqueued without waiting; the particle read that follows
    # synchronises and reports any device error of the step
    outs = (np.empty(3 * w.n_p), np.empty(3 * w.n_p), np.empty(3 * w.n_p))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        sim.set_particles(pos, rr, cc, fpp)
        sim.step_async(1)
        pos, fpp, fpi = sim.get_particles(outs)  # set_particles has consumed the last ones
        sim.mass()
    e2e_dt = time.perf_counter() - t0
    e2e_val = ws * e2e_steps / e2e_dt
    h2d = w.n_p * 8 * (3 + 1 + 1 + 3)
    d2h = w.n_p * 8 * 9 + 8
    sim.close()

    # ---- FP64 form and the mixed-vs-FP64 error from one state
    res = {}
    fp64_rate = None
    for prec in ("fp64", "mixed"):
        s = F.Simulation(P, prec, device=local)
        s.set_phase(c)
        s.set_particles(p, r, ct)
        m0 = s.mass()
        s.step(1)
        el = timed_steps(s, args.err_steps - 1, torch)
        if prec == "fp64":
            fp64_rate = (args.err_steps - 1) / el
        res[prec] = (s.get_phase(), s.get_velocity(), s.get_particles()[0], s.mass(), m0, s.free_energy())
        s.close()
    a, b = res["mixed"], res["fp64"]

    # ---- the same runs in the mass-conserving mode (fipi_set_mass_conserving)
    drift_on = {}
    for prec in ("fp64", "mixed"):
        with F.Simulation(P, prec, device=local) as s:
            s.set_phase(c)
            s.set_particles(p, r, ct)
            s.set_mass_conserving(True)
            m0 = s.mass()
            s.step(args.err_steps)
            drift_on[prec] = abs(s.mass() - m0) / (np.abs(c).sum() * P.lx * P.ly * P.lz / w.V)

    # ---- the FP64 form against its own roof: the FP64 FMA pipe (measured
    # here) at the nominal 13 R2C/C2R transforms x 2.5 V log2 V FLOP per step
    fp64_peak = F.fma_peak(local, fp64=True)
    fp32_peak = F.fma_peak(local, fp64=False)
    fp64_flop = 13 * 2.5 * w.V * math.log2(w.V)
    fp64_roof = {"bound": "fp64 pipe", "model": "13 transforms x 2.5 V log2 V FLOP per step",
                 "flop_per_step": fp64_flop, "achieved": fp64_flop * fp64_rate / 1e12,
                 "peak": fp64_peak, "unit": "TFLOP/s", "frac": fp64_flop * fp64_rate / 1e12 / fp64_peak,
                 "peak_source": "measured here: fipi_fma_peak (FP64 FMA chains on every SM, FMA = 2 FLOP)",
                 "fp32_fma_peak_tflops": fp32_peak}

    def rl2(x, y):
        return float(np.linalg.norm(x - y) / np.linalg.norm(y))

    L = np.array([P.lx, P.ly, P.lz])
    dpos = np.abs(a[2] - b[2]).reshape(-1, 3)
    dpos = np.minimum(dpos, L - dpos)
    err = {
        "steps": args.err_steps,
        "phi_rel_l2": rl2(a[0], b[0]),
        "u_rel_l2": rl2(a[1], b[1]),
        "pos_max_abs": float(dpos.max()),
        "free_energy_rel": abs(a[5] - b[5]) / abs(b[5]),
        "mass_drift_mixed": abs(a[3] - a[4]) / (np.abs(c).sum() * P.lx * P.ly * P.lz / w.V),
        "mass_drift_fp64": abs(b[3] - b[4]) / (np.abs(c).sum() * P.lx * P.ly * P.lz / w.V),
        "mass_drift_mass_conserving": drift_on,
    }

    # ---- roofline of the dominant kernel
    hbm, src = peaks()
    # the dominant grid kernel: particle kernels carry no algorithmic bytes
    # (latency-bound, reported as particle updates/s) and never dominate here
    grid = [k for k in ks if k["bytes"] > 0]
    dom = max(grid, key=lambda k: k["ms"]) if grid else None
    top = max(ks, key=lambda k: k["ms"]) if ks else None
    roof = None
    if dom and dom["ms"] > 0:
        per_launch_s = dom["ms"] / dom["launches"] / 1e3
        ach = dom["bytes"] / per_launch_s / 1e9
        roof = {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                "traffic": committed_traffic(dom["name"], w.name), "kernel": dom["name"],
                "peak_source": f"{src} (MEASURED_PEAKS.json hbm_gbs)" if src == "measured" else src,
                "alg_bytes_per_launch": dom["bytes"], "us_per_launch": per_launch_s * 1e6,
                "share_of_step": dom["ms"] / sum(k["ms"] for k in ks),
                "top_kernel_overall": top["name"] if top else None}

    # ---- the whole step against the HBM roofline: the ideal fused pipeline
    # (44 full-grid field passes of V FP32 words per step, one read and one
    # write per transform) and the pass traffic of this design (the
    # algorithmic bytes of every grid-pass launch of a step)
    step_roof = None
    if ks:
        per_rep = value / ws
        ideal = 44 * w.V * 4
        design = sum(k["bytes"] * k["launches"] for k in ks) / args.kernel_steps
        step_roof = {"model": "44 field passes x V x 4 B per step", "bytes_per_step": ideal,
                     "achieved": ideal * per_rep / 1e9, "frac": ideal * per_rep / 1e9 / hbm,
                     "pass_bytes_per_step": design, "pass_achieved": design * per_rep / 1e9,
                     "pass_frac": design * per_rep / 1e9 / hbm, "unit": "GB/s", "peak": hbm}

    # ---- adjoint / forward (FP64 form)
    adj = None
    if args.adj_steps > 0:
        adj = adjoint_ratio(F, P, c, p, r, ct, local, torch, args.adj_steps, args.traj_steps)

    grads = {}
    if rank == 0 and args.grad != "none":
        for name in (("cfg4_128", "cfg5_256") if args.grad == "all" else (args.grad,)):
            grads[name] = grad_bench(F, name, local, torch, steps=args.grad_steps or None,
                                     fd_steps=args.grad_fd_steps or None, fd_h=args.grad_fd_h or None)

    cpu = err_oracle = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cpu, ref_state, nref = cpu_baseline(w, seed)
        err_oracle = error_vs_oracle(F, w, P, c, p, r, ct, local, ref_state, nref)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (k=0 mode, reductions, positions f64)",
            "data": "synthetic (seeded phi0 = U(-0.05,0.05), random non-overlapping spheres)",
            "config": {"workload": w.name, "grid": f"{w.nx}x{w.ny}x{w.nz}", "particles": w.n_p,
                       "form": "mixed", "parallelism": f"replicas x{ws}",
                       "l2": "working set > L2 (inputs larger than L2; no flush needed)"},
            "particle_updates_per_s": value * w.n_p,
            "fp64": {"steps_per_s": fp64_rate * ws, "mixed_over_fp64": value / (fp64_rate * ws),
                     "roofline": fp64_roof},
            "error_mixed_vs_fp64": err,
            "error_vs_oracle": err_oracle,
            "adjoint_over_forward": adj["adjoint_step_over_forward"] if adj else None,
            "adjoint": adj,
            "gradients": grads,
            "e2e": {"value": e2e_val, "unit": "steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches,
            "roofline": roof,
            "step_roofline": step_roof,
            "kernels": sorted([{"name": k["name"], "launches": k["launches"], "ms": round(k["ms"], 4),
                                "gbs": (k["bytes"] * k["launches"] / (k["ms"] / 1e3) / 1e9) if k["ms"] > 0 else None}
                               for k in ks], key=lambda k: -k["ms"]),
            "clocks": clk.summary(),
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="cfg2_256")
    ap.add_argument("--err-steps", type=int, default=1000)
    ap.add_argument("--e2e-steps", type=int, default=50)
    ap.add_argument("--kernel-steps", type=int, default=20)
    ap.add_argument("--adj-steps", type=int, default=5, help="adjoint steps timed (0 = skip)")
    ap.add_argument("--traj-steps", type=int, default=16, help="steps of the checkpointed gradient")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--grad", default="all", choices=["all", "none", "cfg4_128", "cfg5_256"],
                    help="gradient benchmarks of the adjoint (configs 4 and 5)")
    ap.add_argument("--grad-steps", type=int, default=0, help="steps of the gradient benchmarks (0 = the workload's)")
    ap.add_argument("--grad-fd-steps", type=int, default=0,
                    help="steps of the finite-difference checks (0: config 4 all, config 5 the first 100)")
    ap.add_argument("--grad-fd-h", type=float, default=0.0,
                    help="relative step of the finite differences (0: 1e-6; config 5: 1e-6 sigma, 1e-4 cos theta)")
    ap.add_argument("--profile", type=int, default=0, help="only run N steps (for ncu)")
    ap.add_argument("--form", default="mixed", choices=["mixed", "fp64"])
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        return run_reference(args)
    if args.profile > 0:
        return run_profile(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
