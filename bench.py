"""Throughput of one GB300 projection step (Gcell-steps/s), JSON on one line.

Workload (default): the reference's own full-step test case (test/full_test.cpp),
the Ethier-Steinman exact Navier-Stokes solution, on the unit cube at 512^3
cells (513^3 nodes, every face Dirichlet with the exact velocity,
homogeneous-Neumann DCT-I Poisson), Re = 1000, dt = 1e-4 (64/512)^2 (dt
scaled with h^2 as in the large manufactured runs), no forcing (mif::timestep
unchanged). Inputs are the analytic fields at t = 0, generated on the device
(synthetic; no dataset).

Precision of the headline (--precision compensated, the default): float
fields, stencils and transforms, with the velocity state compensated by a
bfloat16 residual per component (MIFGPU_MIXED_COMPENSATED); the eigenvalues
and 1/(lx+ly+lz) are computed in double and applied as a float table; mean
removal and norms in double. The same workload then runs in FP64 and in the
plain float mode over the same window: `matched_error` gives the headline's
L-infinity velocity error against the exact solution over FP64's (the
"matched L-inf error" condition, target <= 2) and the speed-up over FP64.

Extra modes (each prints one JSON line): --configs runs the reference's
benchmark configurations 1-3 at their sizes; --sweep runs the Ethier-Steinman
refinement 32^3 -> 768^3 in FP64 and both float modes (convergence order and
matched error); --velocity runs the reference's own benchmark harness (the
velocity-only step, N = 32..512); --adjoint-only runs the adjoint workload
alone.

Arms:
  --impl gb300      (default) the CUDA library: `value` from CUDA events around
                    K graph-replayed steps with the fields resident in HBM;
                    `e2e` through the drop-in host call mifgpu_timestep_host
                    (pinned host buffers in the reference layout, H2D + step +
                    D2H inside the timed region); `roofline` of the dominant
                    kernel class; `cpu_baseline` of the oracle on a bounded sample.
  --impl reference  the reference's CPU algorithm (the bit-exact C restatement
                    under oracle/, built with the reference's optimisation
                    flags) on every host core, one independent replica per
                    core, on a bounded 128^3 sample of the same workload.
Multi-GPU: the path does not shard; N ranks run N independent replicas
(weak scaling, no collective on the data path).
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

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "mpi-incompressible-fluid_gb300")
ORACLE_DIR = os.path.join(REPO, "oracle")
for _p in (PKG, ORACLE_DIR):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "full-step Gcell/s at 512³, mixed vs FP64 at matched L∞ err; adjoint/fwd ratio"
UNIT = "Gcell-steps/s"

WORKLOADS = {
    # name: (n_global, size, origin, periodic, Re, dt, kind, forcing)
    # The reference's own full-step case (test/full_test.cpp): the Ethier-Steinman
    # exact Navier-Stokes solution on the unit cube, no forcing (mif::timestep as is).
    "cube512": ((513, 513, 513), (1.0, 1.0, 1.0), (0.0, 0.0, 0.0), (False, False, False), 1000.0,
                1e-4 * (64.0 / 512.0) ** 2, 2, 0),
    "cube768": ((769, 769, 769), (1.0, 1.0, 1.0), (0.0, 0.0, 0.0), (False, False, False), 1000.0,
                1e-4 * (64.0 / 768.0) ** 2, 2, 0),
    # SINCOS velocity with its Navier-Stokes forcing (the forcing extension)
    "cube512_sincos": ((513, 513, 513), (1.0, 1.0, 1.0), (0.0, 0.0, 0.0), (False, False, False), 1000.0,
                       1e-4 * (64.0 / 512.0) ** 2, 1, 2),
    "channel512x256x512": ((513, 257, 513), (4 * 3.141592653589793, 2.0, 2 * 3.141592653589793), (0.0, 0.0, 0.0),
                           (True, False, True), 5000.0, 5e-4, 0, 0),
    "cube64": ((65, 65, 65), (1.0, 1.0, 1.0), (0.0, 0.0, 0.0), (False, False, False), 1000.0, 1e-4, 1, 2),
    # profiling case: ~1.5 GB on the device, z lines still DCT-I of 513 points
    "box256x256x512": ((257, 257, 513), (0.5, 0.5, 1.0), (0.0, 0.0, 0.0), (False, False, False), 1000.0,
                       1e-4 * (64.0 / 512.0) ** 2, 1, 2),
    # the same box with the headline's field (Ethier-Steinman, no forcing): the
    # cube512 kernels on a profiling-sized case
    "box256x256x512_es": ((257, 257, 513), (0.5, 0.5, 1.0), (0.0, 0.0, 0.0), (False, False, False), 1000.0,
                          1e-4 * (64.0 / 512.0) ** 2, 2, 0),
    # profiling case for the strided y sweeps of the 512^3 cube: y lines DCT-I of 513 points
    "box256x512x256": ((257, 513, 257), (0.5, 1.0, 0.5), (0.0, 0.0, 0.0), (False, False, False), 1000.0,
                       1e-4 * (64.0 / 512.0) ** 2, 1, 2),
    # profiling case for the x sweeps of the 512^3 cube: x lines DCT-I of 513 points
    "box512x256x256": ((513, 257, 257), (1.0, 0.5, 0.5), (0.0, 0.0, 0.0), (False, False, False), 1000.0,
                       1e-4 * (64.0 / 512.0) ** 2, 1, 2),
}

PRECISIONS = {"fp64": 0, "mixed": 1, "compensated": 2}

# Algorithmic HBM sweeps (full-field reads + writes) per launch of each kernel
# class, in units of one field of the working type (4 B in the float modes,
# 8 B in FP64); times the unit and the cell count give algorithmic bytes.
SWEEPS = {"stage": 11.0, "divergence": 4.0, "x_forward": 2.0, "y_forward": 2.0, "z_fused": 2.0,
          "y_inverse": 2.0, "x_inverse": 2.0, "project": 9.0}
# The compensated state adds its bfloat16 residuals (2 B, half a float sweep
# each): the stages and projections read and write three, the divergence
# reads three.
COMPENSATED_EXTRA = {"stage": 3.0, "divergence": 1.5, "project": 3.0}
LAUNCHES_PER_STEP = {"stage": 3, "divergence": 3, "x_forward": 3, "y_forward": 3, "z_fused": 3, "y_inverse": 3,
                     "x_inverse": 3, "project": 3}


def sweeps(precision: str) -> dict:
    """Per launch (the stage class: the mean of the step's three stages)."""
    out = dict(SWEEPS)
    if precision == "compensated":
        for k, v in COMPENSATED_EXTRA.items():
            out[k] += v
        # The stage kernels of the step a run repeats (the one profile_step
        # times) apply the projection before them (stage_pair_kernel): each
        # also reads phi and writes p + phi (15, 18, 15).
        out["stage"] += 2.0
    return out


def launches_per_step(precision: str) -> dict:
    """In the compensated state the step a run repeats has no projection kernel."""
    out = dict(LAUNCHES_PER_STEP)
    if precision == "compensated":
        out["project"] = 0
    return out


def step_sweeps(precision: str, steps: int = 1) -> float:
    """Per step as built: 33 stage + 3 x (4 divergence + 5 x 2 line sweeps +
    9 projection) = 102 in FP64 and the plain float mode. The compensated
    state, the step a run repeats: stages 15 + 18 + 15 (residuals, and phi and
    p + phi in the stages that project), 3 x 5.5 divergence, 30 line sweeps:
    94.5. A run's first step has a plain Y2 stage (13) and its last ends with
    the projection kernel (12): over a run of `steps` steps the mean is
    94.5 + (12 - 2) / steps (95.0 for 20 steps; 104.5 for one step)."""
    n = launches_per_step(precision)
    rep = sum(v * n[k] for k, v in sweeps(precision).items())
    if precision == "compensated":
        return rep + (12.0 - 2.0) / max(1, steps)
    return rep


# DRAM read + write bytes over algorithmic bytes, from ncu captures of the
# stage, divergence and projection kernels on the 256x256x512 profiling case
# (the compensated stages with the projection inside, of the step a run
# repeats, on its Ethier-Steinman variant: 1.04, 1.03, 1.03) and of the line
# sweeps on the 256x512x256 one: applied to the full launch.
# (The fused z sweep's figure includes its 1/lambda table, one more
# field-sized read.)
MEASURED_TRAFFIC_RATIO = {
    "mixed": {"stage": 1.06, "x_forward": 0.82, "y_forward": 0.81, "z_fused": 1.37, "y_inverse": 0.81,
              "x_inverse": 0.82},
    "compensated": {"stage": 1.03, "divergence": 1.03, "project": 0.99, "x_forward": 0.82, "y_forward": 0.81,
                    "z_fused": 1.37, "y_inverse": 0.81, "x_inverse": 0.82},
}
# FP64 operations of one FP64 step per cell (an FMA counted as two), from the
# DFMA / DADD / DMUL instruction counters of an ncu capture of the
# 256x256x512 case; the 512^3 step's longer x and y transforms add a few per cent.
FP64_FLOPS_PER_CELL_STEP = 1249.0
# The same step with the divergence fused into the x-forward sweep and the
# projection into the x-inverse sweep (the fused dataflow): 90 sweeps.
FUSED_STEP_SWEEPS = 90.0


def measured_peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def bind_gpu_local_cpus(gpu_index: int) -> str:
    """Pins this process to the CPUs local to the GPU (the PCI device's
    local_cpulist), so pinned host buffers allocated afterwards land in the
    memory next to the GPU's host link. Returns what was applied."""
    try:
        bus = subprocess.check_output(["nvidia-smi", "-i", str(gpu_index), "--query-gpu=pci.bus_id",
                                       "--format=csv,noheader"], text=True, timeout=30).strip()
        dom, rest = bus.split(":", 1)
        path = f"/sys/bus/pci/devices/{int(dom, 16):04x}:{rest.lower()}/local_cpulist"
        with open(path) as f:
            spec = f.read().strip()
        cpus = set()
        for part in spec.split(","):
            lo, _, hi = part.partition("-")
            cpus.update(range(int(lo), int(hi or lo) + 1))
        cpus &= os.sched_getaffinity(0)
        if not cpus:
            return "unchanged (no local CPU available)"
        os.sched_setaffinity(0, cpus)
        return f"GPU-local CPUs {spec}"
    except Exception as e:  # no sysfs entry, no nvidia-smi: leave the affinity alone
        return f"unchanged ({type(e).__name__})"


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def allreduce_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(ms_local: float, world: int, cells: int, steps: int) -> tuple:
    """Whole-job throughput of `world` independent replicas: every rank did
    `cells * steps` cell-steps; the job took the slowest rank's time.
    Returns (Gcell-steps/s, max ms)."""
    ms = allreduce_max(ms_local, world)
    return world * cells * steps / (ms / 1e3) / 1e9, ms


# ---------------------------------------------------------------- CPU baseline

CPU_FLAGS = "-Ofast -funroll-all-loops -flto (the reference's Makefile:26 flags without -march=native)"


def cpu_model() -> str:
    try:
        import platform

        with open("/proc/cpuinfo") as f:
            for ln in f:
                if ln.lower().startswith(("model name", "cpu part")):
                    return f"{platform.machine()} {ln.split(':', 1)[1].strip()}"
        return platform.machine()
    except Exception:
        return "unknown"


def _cpu_worker(args):
    """One replica of the CPU step: `warmup` untimed steps, then `steps`
    timed ones; returns (cells per step, [seconds per timed step])."""
    n, warmup, steps, periodic, size, Re, dt, kind, forcing = args
    import oracle as O

    case = O.Case(n_global=(n, n, n), size=size, Re=Re, dt=dt, periodic=periodic, exact_kind=kind, forcing=forcing)
    s = O.OracleFastSolver(case)
    s.set_exact_velocity(0, 0.0, True)
    s.set_exact_pressure(0.0)
    for k in range(warmup):
        s.timestep(k * dt)
    times = []
    for k in range(steps):
        t0 = time.perf_counter()
        s.timestep((warmup + k) * dt)
        times.append(time.perf_counter() - t0)
    return case.cells(), times


def cpu_run(workers: int, n: int, warmup: int, steps: int, workload: str = "cube512"):
    """The reference's step (the oracle's C restatement in its timing build,
    oracle/libmif_oracle_fast.so) on `workers` independent replicas, one per
    core, each an n^3-node sample of the workload family. Returns per timed
    step the whole-job Gcell-steps/s (all replicas' cells over the slowest
    replica's time) and the wall time."""
    import multiprocessing as mp

    import oracle as O

    O.build(with_ref=False, fast=True)
    w = WORKLOADS[workload]
    job = (n, warmup, steps, w[3], w[1], w[4], w[5], w[6], w[7])
    t0 = time.perf_counter()
    if workers == 1:
        res = [_cpu_worker(job)]
    else:
        ctx = mp.get_context("spawn")
        with ctx.Pool(workers) as pool:
            res = pool.map(_cpu_worker, [job] * workers)
    wall = time.perf_counter() - t0
    cells = sum(r[0] for r in res)
    per_step = [cells / max(r[1][k] for r in res) / 1e9 for k in range(steps)]
    return per_step, wall


def cpu_baseline(workers: int = 1, n: int = 129, steps: int = 2):
    """The bounded CPU sample beside the GPU number: one core, a 128^3-cell
    Ethier-Steinman cube (the default workload at a smaller size)."""
    per_step, wall = cpu_run(workers, n, 1, steps)
    return {"value": statistics.median(per_step), "unit": UNIT, "cores": workers, "kind": "port",
            "sample": f"{n - 1}^3-cell Ethier-Steinman cube (the default workload at a smaller size), {steps} timed "
                      f"steps after 1 warm-up, {workers} replica(s); oracle/mif_oracle.c (bit-exact restatement "
                      f"of the reference's step, FFT stand-in for FFTW) built {CPU_FLAGS}; {cpu_model()} "
                      f"(wall {wall:.1f}s)"}


# ------------------------------------------------------------------ adjoint workload

ADJOINT = dict(n=128, L=2 * 3.141592653589793, Re=500.0, dt=2e-3, nsteps=200, every=20, kmax=8, amp=1.0,
               alpha=0.5, seed=1234)


def random_solenoidal(shape_of, n, L, kmax, amp, seed):
    """Seeded divergence-free velocity on the periodic staggered grid: the curl of
    a Gaussian vector potential with |A_k| ~ |k|^-2 (|k| <= kmax), scaled to max |u| = amp.

    Each component is sampled at its own staggered points (offset -h/2 along
    its axis) by a spectral phase shift; ghost points are periodic copies."""
    import numpy as np

    rng = np.random.default_rng(seed)
    k1 = np.fft.fftfreq(n, d=1.0 / n)
    kx, ky, kz = np.meshgrid(k1, k1, k1, indexing="ij")
    kk = np.sqrt(kx ** 2 + ky ** 2 + kz ** 2)
    mask = (kk > 0) & (kk <= kmax)
    spec = np.where(mask, 1.0 / np.maximum(kk, 1.0) ** 2, 0.0)
    A = [np.fft.fftn(rng.standard_normal((n, n, n))) * spec for _ in range(3)]
    w = 2 * np.pi / L
    K = (kx * w, ky * w, kz * w)
    uh = (1j * (K[1] * A[2] - K[2] * A[1]), 1j * (K[2] * A[0] - K[0] * A[2]), 1j * (K[0] * A[1] - K[1] * A[0]))
    h = L / n
    out = {}
    vals = []
    for c, name in enumerate("uvw"):
        shifted = uh[c] * np.exp(-1j * K[c] * h / 2)
        f = np.real(np.fft.ifftn(shifted))  # f[ix, iy, iz] at x = ix h (- h/2 along c)
        vals.append(f)
    scale = amp / max(np.abs(f).max() for f in vals)
    for c, name in enumerate("uvw"):
        ez, ey, ex = shape_of(name)
        ii = (np.arange(ex) - 1) % n
        jj = (np.arange(ey) - 1) % n
        kq = (np.arange(ez) - 1) % n
        f = vals[c] * scale
        out[name] = np.ascontiguousarray(f[np.ix_(ii, jj, kq)].transpose(2, 1, 0))
    return out


def ke_box(s, n, L, box):
    """Kinetic energy 1/2 h^3 sum u_c^2 over the interior staggered points inside
    box, for a periodic n^3 box of side L (the loss of mifgpu_gradient_ke)."""
    import numpy as np

    h = L / n
    tot = 0.0
    for c, nm in enumerate("uvw"):
        a = s.download(nm)
        ez, ey, ex = a.shape
        ax = []
        for d, e in enumerate((ex, ey, ez)):
            x = h * (np.arange(e) - 1.0) - (h / 2 if d == c else 0.0)
            ax.append((x >= box[2 * d]) & (x <= box[2 * d + 1]) & (np.arange(e) >= 1) & (np.arange(e) <= e - 2))
        m = ax[2][:, None, None] & ax[1][None, :, None] & ax[0][None, None, :]
        tot += 0.5 * h ** 3 * float(np.sum(a[m] ** 2))
    return tot


def adjoint_bench(stream):
    """Checkpointed gradient of the kinetic energy in [pi/2, 3pi/2]^3 after 200
    steps of a periodic 128^3 box, in FP32 and FP64: cost against the forward
    steps, FP32 gradient error against FP64, and an FP64 dot-product test."""
    import numpy as np
    import torch

    import mifgpu

    a = ADJOINT
    n = a["n"]
    pi = 3.141592653589793
    box = (pi / 2, 3 * pi / 2) * 3
    res = {"workload": f"periodic {n}^3 box [0,2pi]^3, Re={a['Re']}, dt={a['dt']}, {a['nsteps']} steps, "
                       f"checkpoint every {a['every']}, Taylor-Green forcing alpha={a['alpha']}, "
                       f"k^-2 solenoidal initial velocity |k|<={a['kmax']} max|u|={a['amp']}",
           "loss": "kinetic energy in [pi/2,3pi/2]^3 at the final time"}
    grads = {}
    for prec_name, prec in (("fp32", mifgpu.MIXED), ("fp64", mifgpu.FP64)):
        s = mifgpu.Solver(n_global=(n + 1,) * 3, size=(a["L"],) * 3, Re=a["Re"], dt=a["dt"],
                          periodic=(True, True, True), precision=prec, forcing=mifgpu.FORCING_TAYLOR_GREEN,
                          forcing_amplitude=a["alpha"])
        s.set_stream(stream.cuda_stream)
        st = random_solenoidal(s.shape, n, a["L"], a["kmax"], a["amp"], a["seed"])
        st["p"] = np.zeros(s.shape("p"))
        s.load_state(st)
        s.run(0.0, 3)  # warm-up, graph capture
        s.load_state(st)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s.run(0.0, a["nsteps"])
        e1.record(stream)
        torch.cuda.synchronize()
        fwd_ms = e0.elapsed_time(e1) / a["nsteps"]
        s.load_state(st)
        r = s.gradient_ke(0.0, a["nsteps"], a["every"], box)
        g = {nm: s.adjoint(nm) for nm in "uvwp"}
        grads[prec_name] = (r, g)
        # the backward pass recomputes each segment beside the reverse sweep
        # of the next (two streams): its wall time over the forward steps'
        rev = r["reverse_ms"] / a["nsteps"]
        bwd = r["backward_ms"] / a["nsteps"]
        out = {"forward_ms_per_step": round(fwd_ms, 4), "reverse_ms_per_step": round(rev, 4),
               "backward_ms_per_step": round(bwd, 4),
               "adjoint_step_ratio": round(rev / fwd_ms, 3),
               "backward_ratio": round(bwd / fwd_ms, 3),
               "gradient_pass_ratio": round((r["forward_ms"] + r["backward_ms"]) / (fwd_ms * a["nsteps"]), 3),
               "loss": r["loss"], "dloss_dalpha": r["dloss_dalpha"], "device_gb": round(s.device_bytes() / 1e9, 2)}
        if prec == mifgpu.FP64:
            # dot-product test: <adjoint, delta> against the tangent-linear derivative
            # of the FP64 forward map along a random delta, by central differences at
            # eps and eps/2 and their Richardson extrapolation (removes the eps^2 term)
            rng = np.random.default_rng(5)
            delta = {nm: rng.standard_normal(st[nm].shape) for nm in "uvw"}
            adj = sum(float(np.sum(g[nm] * delta[nm])) for nm in "uvw")

            def loss_at(e):
                s.load_state({nm: st[nm] + e * delta[nm] for nm in "uvw"} | {"p": st["p"]})
                s.run(0.0, a["nsteps"])
                return ke_box(s, n, a["L"], box)

            eps = 1e-6
            d1 = (loss_at(eps) - loss_at(-eps)) / (2 * eps)
            d2 = (loss_at(eps / 2) - loss_at(-eps / 2)) / eps
            dr = (4 * d2 - d1) / 3
            out["dot_product"] = {"adjoint": adj, "tangent_linear_eps": d1, "tangent_linear_eps_half": d2,
                                  "eps": eps, "rel_err_eps": abs(d1 - adj) / abs(adj),
                                  "rel_err_eps_half": abs(d2 - adj) / abs(adj),
                                  "rel_err_richardson": abs(dr - adj) / abs(adj)}
        res[prec_name] = out
        s.close()
        torch.cuda.empty_cache()
    (r32, g32), (r64, g64) = grads["fp32"], grads["fp64"]
    res["fp32_vs_fp64_gradient_max_rel_err"] = max(
        float(np.abs(g32[nm] - g64[nm]).max() / np.abs(g64[nm]).max()) for nm in "uvw")
    res["fp32_vs_fp64_dalpha_rel_err"] = abs(r32["dloss_dalpha"] - r64["dloss_dalpha"]) / abs(r64["dloss_dalpha"])
    return res


# ------------------------------------------------------------------ reference configurations

def solenoidal_noise(shape_of, ncell, L, base, kmax, amp, seed):
    """Seeded divergence-free noise on a staggered grid: the curl of a Gaussian
    vector potential with |A_k| ~ |k|^-2 (integer wavenumbers, 0 < |k| <= kmax),
    periodic over the box, scaled to max |u| = amp. Component c is sampled at
    its own staggered points by a spectral phase shift; array index i along
    axis d maps to grid point (base_d + i) mod ncell_d."""
    import numpy as np

    rng = np.random.default_rng(seed)
    nx, ny, nz = ncell
    kx = np.fft.rfftfreq(nx, 1.0 / nx)
    ky = np.fft.fftfreq(ny, 1.0 / ny)
    kz = np.fft.fftfreq(nz, 1.0 / nz)
    KZ, KY, KX = np.meshgrid(kz, ky, kx, indexing="ij")
    kk = np.sqrt(KX ** 2 + KY ** 2 + KZ ** 2)
    mask = (kk > 0) & (kk <= kmax)
    A = []
    for _ in range(3):
        a = np.zeros(kk.shape, np.complex64)
        m = int(mask.sum())
        a[mask] = (rng.standard_normal(m) + 1j * rng.standard_normal(m)) / kk[mask] ** 2
        A.append(a)
    w = [2 * np.pi / L[d] for d in range(3)]
    K = (KX * w[0], KY * w[1], KZ * w[2])
    uh = (1j * (K[1] * A[2] - K[2] * A[1]), 1j * (K[2] * A[0] - K[0] * A[2]), 1j * (K[0] * A[1] - K[1] * A[0]))
    vals = []
    for c in range(3):
        h = L[c] / ncell[c]
        vals.append(np.fft.irfftn(uh[c] * np.exp(-1j * K[c] * h / 2), s=(nz, ny, nx)).astype(np.float64))
    scale = amp / max(float(np.abs(f).max()) for f in vals)
    out = {}
    for c, name in enumerate("uvw"):
        ez, ey, ex = shape_of(name)
        ii = (base[0] + np.arange(ex)) % nx
        jj = (base[1] + np.arange(ey)) % ny
        kq = (base[2] + np.arange(ez)) % nz
        out[name] = np.ascontiguousarray(vals[c][np.ix_(kq, jj, ii)] * scale)
    return out


def staggered_coords(s, name, n_global, size, origin, periodic):
    """Positions (x, y, z) of a field's points, reference layout (z, y, x)."""
    import numpy as np

    ez, ey, ex = s.shape(name)
    comp = "uvw".index(name) if name in "uvw" else -1
    ax = []
    for d, e in enumerate((ex, ey, ez)):
        h = size[d] / (n_global[d] - 1)
        base = -1 if periodic[d] else 0
        x = origin[d] + h * (base + np.arange(e))
        if d == comp:
            x = x - h / 2
        ax.append(x)
    z, y, x = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    return x, y, z


def timed_run(s, stream, t0, nsteps):
    import torch

    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    s.run(t0, nsteps)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / nsteps


def float_vs_fp64(c):
    """Each float mode's final velocity against the FP64 run's (L-infinity over
    max|u|) and its speed-up; drops the fields."""
    import numpy as np

    umax = max(float(np.abs(c["fp64"]["final"][nm]).max()) for nm in "uvw")
    for pname in ("mixed", "compensated"):
        c[pname + "_vs_fp64_velocity_linf"] = max(
            float(np.abs(c[pname]["final"][nm] - c["fp64"]["final"][nm]).max()) for nm in "uvw") / umax
        c[pname + "_speedup"] = round(c["fp64"]["ms_per_step"] / c[pname]["ms_per_step"], 2)
    for pname in ("fp64", "mixed", "compensated"):
        del c[pname]["final"]


def config_suite(stream):
    """The reference's benchmark configurations 1-3 at their sizes, FP64 and
    mixed: Gcell-steps/s, errors against the analytic solution (config 1) or
    between the two precisions after the run (configs 2 and 3)."""
    import numpy as np
    import torch

    import mifgpu

    pi = 3.141592653589793
    out = {}

    def make(n_global, size, origin, periodic, Re, dt, prec, kind, forcing):
        s = mifgpu.Solver(n_global=n_global, size=size, origin=origin, Re=Re, dt=dt, periodic=periodic,
                          precision=prec, boundary_kind=kind, forcing=forcing)
        s.set_stream(stream.cuda_stream)
        return s

    # 1: 64^3 manufactured cube, SINCOS + forcing, FP64, 10 steps of 1e-4
    c1 = {}
    for pname, prec in (("fp64", mifgpu.FP64), ("mixed", mifgpu.MIXED), ("compensated", mifgpu.MIXED_COMPENSATED)):
        s = make((65,) * 3, (1.0,) * 3, (0.0,) * 3, (False,) * 3, 1000.0, 1e-4, prec, 1, 2)
        s.set_exact_velocity(0, 0.0)
        s.set_exact_pressure(0.0)
        s.run(0.0, 2)
        s.set_exact_velocity(0, 0.0)
        s.set_exact_pressure(0.0)
        ms = timed_run(s, stream, 0.0, 10)
        s.adjust_pressure(10 * 1e-4)
        nrm = s.error_norms(10 * 1e-4)
        c1[pname] = {"ms_per_step": round(ms, 4), "gcell_steps_s": 64 ** 3 / ms / 1e6,
                     "velocity_l2": nrm[1], "velocity_linf": nrm[2], "pressure_l2": nrm[4], "pressure_linf": nrm[5]}
        s.close()
    out["1_cube64_manufactured"] = c1

    # 2: periodic 256^3 Taylor-Green + k^-2 noise (|k| <= 16, 1e-2), Re 1600, dt 2e-3, 100 steps
    n_g = (257,) * 3
    size = (2 * pi,) * 3
    fields = {}
    c2 = {}
    for pname, prec in (("fp64", mifgpu.FP64), ("mixed", mifgpu.MIXED), ("compensated", mifgpu.MIXED_COMPENSATED)):
        s = make(n_g, size, (0.0,) * 3, (True,) * 3, 1600.0, 2e-3, prec, 0, 0)
        if not fields:
            noise = solenoidal_noise(s.shape, (256,) * 3, size, (-1,) * 3, 16, 1e-2, 11)
            for c, nm in enumerate("uvw"):
                x, y, z = staggered_coords(s, nm, n_g, size, (0.0,) * 3, (True,) * 3)
                base = (np.sin(x) * np.cos(y) * np.cos(z) if c == 0 else
                        -np.cos(x) * np.sin(y) * np.cos(z) if c == 1 else 0.0 * x)
                fields[nm] = base + noise[nm]
            fields["p"] = np.zeros(s.shape("p"))
        s.load_state(fields)
        s.run(0.0, 2)
        s.load_state(fields)
        ms = timed_run(s, stream, 0.0, 100)
        c2[pname] = {"ms_per_step": round(ms, 4), "gcell_steps_s": 256 ** 3 / ms / 1e6,
                     "final": {nm: s.download(nm) for nm in "uvw"}}
        s.close()
        torch.cuda.empty_cache()
    float_vs_fp64(c2)
    out["2_tgv256_periodic"] = c2

    # 3: channel [0,4pi]x[0,2]x[0,2pi], 512x256x512, periodic x z, walls in y, Re 5000, dt 5e-4, 50 steps
    n_g = (513, 257, 513)
    size = (4 * pi, 2.0, 2 * pi)
    per = (True, False, True)
    fields = {}
    c3 = {}
    for pname, prec in (("fp64", mifgpu.FP64), ("mixed", mifgpu.MIXED), ("compensated", mifgpu.MIXED_COMPENSATED)):
        s = make(n_g, size, (0.0,) * 3, per, 5000.0, 5e-4, prec, 0, 0)
        if not fields:
            noise = solenoidal_noise(s.shape, (512, 256, 512), size, (-1, 0, -1), 16, 1e-2, 12)
            for nm in "uvw":
                x, y, z = staggered_coords(s, nm, n_g, size, (0.0,) * 3, per)
                fields[nm] = (1.0 - (y - 1.0) ** 2 if nm == "u" else 0.0 * y) + noise[nm]
                del x, z
            fields["p"] = np.zeros(s.shape("p"))
        s.load_state(fields)
        s.run(0.0, 2)
        s.load_state(fields)
        ms = timed_run(s, stream, 0.0, 50)
        c3[pname] = {"ms_per_step": round(ms, 4), "gcell_steps_s": 512 * 256 * 512 / ms / 1e6,
                     "final": {nm: s.download(nm) for nm in "uvw"}}
        s.close()
        torch.cuda.empty_cache()
    float_vs_fp64(c3)
    out["3_channel512x256x512"] = c3
    return out


def sweep(stream, sizes=(32, 64, 128, 256, 512, 768)):
    """Ethier-Steinman refinement (the reference's full-step test case on the
    unit cube): 2 steps of dt = 5e-5 from t = 0 (one time window for every
    size, so the observed order is the spatial one), FP64, mixed and
    compensated, L-infinity velocity and pressure errors against the exact
    solution, observed orders."""
    import torch

    import mifgpu

    T, nt = 1e-4, 2
    rows = []
    for n in sizes:
        row = {"cells": n}
        for pname, prec in (("fp64", mifgpu.FP64), ("mixed", mifgpu.MIXED), ("compensated", mifgpu.MIXED_COMPENSATED)):
            s = mifgpu.Solver(n_global=(n + 1,) * 3, Re=1000.0, dt=T / nt, precision=prec,
                              boundary_kind=mifgpu.FIELD_ETHIER)
            s.set_stream(stream.cuda_stream)
            s.set_exact_velocity(0, 0.0)
            s.set_exact_pressure(0.0)
            s.run(0.0, nt)  # warm-up: captures the graphs the timed run replays
            s.set_exact_velocity(0, 0.0)
            s.set_exact_pressure(0.0)
            ms = timed_run(s, stream, 0.0, nt)
            s.adjust_pressure(T)
            nrm = s.error_norms(T)
            row[pname] = {"velocity_linf": nrm[2], "pressure_linf": nrm[5], "ms_per_step": round(ms, 4)}
            s.close()
            torch.cuda.empty_cache()
        for pname in ("mixed", "compensated"):
            row[pname + "_over_fp64_velocity_linf"] = row[pname]["velocity_linf"] / row["fp64"]["velocity_linf"]
        rows.append(row)
    import math

    for a, b in zip(rows, rows[1:]):
        for pname in ("fp64", "mixed", "compensated"):
            b[pname]["velocity_order"] = math.log(a[pname]["velocity_linf"] / b[pname]["velocity_linf"]) / \
                math.log(b["cells"] / a["cells"])
            b[pname]["pressure_order"] = math.log(a[pname]["pressure_linf"] / b[pname]["pressure_linf"]) / \
                math.log(b["cells"] / a["cells"])
    return {"case": "Ethier-Steinman on [0,1]^3, Re=1000, T=1e-4 in 2 steps (test/full_test.cpp)", "rows": rows}


def velocity_benchmark(stream, sizes=(32, 64, 128, 256, 512), steps=20):
    """The reference's own benchmark harness (test/benchmark.cpp:26-61): the
    velocity-only RK3 step (mif::timestep_velocity) on the unit cube with N
    points per axis, N = 32..512, Re = 1e6, dt = 1e-4, the SINCOS velocity
    with its forcing; its counter is seconds per DoF (N^3) per step. Here:
    graph-replayed steps (mifgpu_run_velocity) timed with CUDA events after
    3 warm-up steps, FP64 and float, and the oracle's timestep_velocity on one
    core (timing build) at the two smallest sizes for comparison."""
    import torch

    import mifgpu
    import oracle as O

    rows = []
    for n in sizes:
        row = {"N": n, "dof": n ** 3}
        for pname, prec in (("fp64", mifgpu.FP64), ("mixed", mifgpu.MIXED)):
            s = mifgpu.Solver(n_global=(n, n, n), Re=1e6, dt=1e-4, precision=prec, boundary_kind=mifgpu.FIELD_SINCOS,
                              forcing=mifgpu.FORCING_VELOCITY)
            s.set_stream(stream.cuda_stream)
            s.set_exact_velocity(0, 0.0)
            s.run_velocity(0.0, 3)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            s.run_velocity(3e-4, steps)
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / steps
            row[pname] = {"ms_per_step": round(ms, 5), "ns_per_dof_step": ms * 1e6 / n ** 3,
                          "gdof_steps_s": n ** 3 / ms / 1e6}
            s.close()
            torch.cuda.empty_cache()
        rows.append(row)
    O.build(with_ref=False, fast=True)
    cpu = []
    for n in sizes[:2]:
        case = O.Case(n_global=(n, n, n), Re=1e6, dt=1e-4, exact_kind=O.KIND_SINCOS)
        o = O.OracleFastSolver(case)
        o.set_exact_velocity(0, 0.0, True)
        o.timestep_velocity(0.0)
        t0 = time.perf_counter()
        for k in range(3):
            o.timestep_velocity((1 + k) * 1e-4)
        el = (time.perf_counter() - t0) / 3
        cpu.append({"N": n, "ms_per_step": round(el * 1e3, 3), "ns_per_dof_step": el * 1e9 / n ** 3,
                    "cores": 1, "build": CPU_FLAGS})
    return {"case": "test/benchmark.cpp: velocity-only RK3 step, unit cube, Re=1e6, dt=1e-4, SINCOS velocity "
                    "with forcing", "rows": rows, "cpu_oracle": cpu}


# ------------------------------------------------------------------ GPU arm

def workload_cells(workload: str) -> int:
    cells = 1
    for n in WORKLOADS[workload][0]:
        cells *= n - 1
    return cells


def line_config(workload: str, precision: str, world: int) -> dict:
    """The `config` of both arms' JSON lines (the same workload and settings)."""
    n_global, size, origin, periodic, Re, dt, kind, forcing = WORKLOADS[workload]
    elem = 8 if precision == "fp64" else 4
    field_gb = 11 * elem * workload_cells(workload) / 1e9
    return {"workload": workload, "n_global": list(n_global), "cells": workload_cells(workload),
            "precision": precision, "periodic": list(periodic), "Re": Re, "dt": dt,
            "parallelism": f"replicas{world}",
            "l2": "inputs larger than L2 (fields ~%.1f GB)" % field_gb}


def make_solver(mifgpu, workload: str, precision: str, stream):
    n_global, size, origin, periodic, Re, dt, kind, forcing = WORKLOADS[workload]
    s = mifgpu.Solver(n_global=n_global, size=size, origin=origin, Re=Re, dt=dt, periodic=periodic,
                      precision=PRECISIONS[precision], boundary_kind=kind, forcing=forcing)
    s.set_stream(stream.cuda_stream)
    s.set_exact_velocity(0, 0.0)
    s.set_exact_pressure(0.0)
    return s


def comparison_run(mifgpu, workload: str, precision: str, stream, n_timed: int, total_steps: int) -> dict:
    """Another precision on the same workload: `n_timed` graph-replayed steps
    timed with CUDA events, and the velocity error against the exact solution
    after `total_steps` steps (the headline run's window)."""
    import torch

    dt = WORKLOADS[workload][5]
    kind = WORKLOADS[workload][6]
    cells = workload_cells(workload)
    s = make_solver(mifgpu, workload, precision, stream)
    s.run(0.0, 1)  # graph capture
    torch.cuda.synchronize()
    a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a0.record(stream)
    s.run(dt, n_timed)
    a1.record(stream)
    torch.cuda.synchronize()
    ms = a0.elapsed_time(a1) / n_timed
    out = {"ms_per_step": round(ms, 4), "value": cells / (ms / 1e3) / 1e9}
    s.run((1 + n_timed) * dt, max(0, total_steps - 1 - n_timed))
    if kind != 0:
        out["velocity_linf"] = s.error_norms(total_steps * dt)[2]
        out["t"] = total_steps * dt
    s.close()
    torch.cuda.empty_cache()
    return out


def run_gpu(args):
    import torch

    import mifgpu

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    import build as pkg_build

    pkg_build.build()
    n_global, size, origin, periodic, Re, dt, kind, forcing = WORKLOADS[args.workload]
    prec = args.precision
    stream = torch.cuda.Stream()
    s = make_solver(mifgpu, args.workload, prec, stream)
    s.synchronize()
    cells = workload_cells(args.workload)
    elem = 8 if prec == "fp64" else 4

    # warm-up (graph capture happens here)
    t = 0.0
    s.run(t, args.warmup)
    t += args.warmup * dt
    torch.cuda.synchronize()

    launches0 = s.launch_count()
    barrier(world)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        s.run(t, args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
    barrier(world)
    t += args.steps * dt
    value, ms = replica_throughput(e0.elapsed_time(e1), world, cells, args.steps)
    launches = s.launch_count() - launches0
    total_steps = args.warmup + args.steps

    # error against the analytic solution after the run (matched-error report)
    linf = None
    if kind != 0:
        norms = s.error_norms(t)
        linf = {"velocity_linf": norms[2], "velocity_l2": norms[1], "t": t}

    # per-kernel-class timing (real steps, launch by launch) -> dominant class
    prof = s.profile_step(t, reps=2)
    t += 2 * dt
    peak, peak_kind = measured_peaks()
    sw = sweeps(prec)
    nl = launches_per_step(prec)
    classes = {k: v for k, v in prof.items() if k in sw}
    dom = max(classes, key=lambda k: classes[k])
    alg_bytes_launch = sw[dom] * elem * cells
    avg_launch_ms = classes[dom] / nl[dom]
    achieved = alg_bytes_launch / (avg_launch_ms / 1e3) / 1e9
    # DRAM traffic per launch from one ncu capture of the same kernels on a
    # profiling case: measured read+write bytes over algorithmic bytes,
    # applied to this launch.
    ratio = MEASURED_TRAFFIC_RATIO.get(prec, {}).get(dom)
    traffic = round(ratio * alg_bytes_launch) if ratio else None
    roofline = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic, "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": alg_bytes_launch, "avg_launch_ms": round(avg_launch_ms, 4)}
    step_ms = ms / args.steps
    ssw = step_sweeps(prec, args.steps)
    step_roofline = ssw * elem * cells / (step_ms / 1e3) / 1e9
    per_kernel = {k: {"ms_per_step": round(v, 4),
                      "gbs": round(sw[k] * nl[k] * elem * cells / (v / 1e3) / 1e9, 1),
                      "frac": round(sw[k] * nl[k] * elem * cells / (v / 1e3) / 1e9 / peak, 4)}
                  for k, v in classes.items() if v > 0}

    # end to end through the drop-in host call, pinned host buffers
    e2e = None
    if not args.no_e2e:
        names = ("u", "v", "w", "p")
        affinity = bind_gpu_local_cpus(local)
        host = {nm: torch.empty(s.shape(nm), dtype=torch.float64, pin_memory=True) for nm in names}
        for nm in names:
            host[nm].numpy()[...] = s.download(nm)
        bi = sum(h.numel() * 8 for h in host.values())

        arrs = [host[nm].numpy() for nm in names]
        for _ in range(2):  # warm
            s.timestep_host(t, *arrs)
            t += dt
        # value: the mean over all timed calls, one per timed step. Single
        # device-to-host copies occasionally take twice their usual time on
        # these hosts, so the calls are timed one by one too and their spread
        # is reported.
        k_e2e = max(1, args.steps)
        calls = []
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(k_e2e):
            tc = time.perf_counter()
            s.timestep_host(t, *arrs)  # returns after the download has landed
            calls.append((time.perf_counter() - tc) * 1e3)
            t += dt
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        el = allreduce_max(el, world)
        e2e = {"value": world * cells * k_e2e / el / 1e9, "unit": UNIT, "h2d_bytes_per_step": bi,
               "d2h_bytes_per_step": bi, "steps": k_e2e, "api": "mifgpu_timestep_host",
               "call_ms": {"min": round(min(calls), 2), "median": round(statistics.median(calls), 2),
                           "max": round(max(calls), 2)},
               "host_buffers": "pinned, allocated after binding to " + affinity}
        # The host link measured on the same buffers with plain copies (one
        # device tensor per field), and the e2e rate it allows: the step plus
        # both transfers at those rates, nothing overlapped.
        dev = {nm: torch.empty_like(host[nm], device="cuda") for nm in names}
        rates = {}
        for direction in ("h2d", "d2h"):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for nm in names:
                if direction == "h2d":
                    dev[nm].copy_(host[nm], non_blocking=True)
                else:
                    host[nm].copy_(dev[nm], non_blocking=True)
            torch.cuda.synchronize()
            rates[direction] = bi / (time.perf_counter() - t0) / 1e9
        del dev
        ceiling_s = step_ms / 1e3 + bi / (rates["h2d"] * 1e9) + bi / (rates["d2h"] * 1e9)
        e2e["link_gbs"] = {k: round(v, 1) for k, v in rates.items()}
        e2e["link_bound_value"] = round(world * cells / ceiling_s / 1e9, 4)
    s.close()
    torch.cuda.empty_cache()

    # the other precisions on the same workload and window
    fp64 = None
    if prec != "fp64" and not args.no_fp64:
        fp64 = comparison_run(mifgpu, args.workload, "fp64", stream, max(1, min(args.steps, 3)), total_steps)
        fp64["speedup_of_headline"] = round(fp64["ms_per_step"] / step_ms, 2)
        # both rooflines of the FP64 step: the FP64 pipe (its FMA rate probed
        # live) and HBM (the as-built sweeps at 8 bytes)
        ms64 = fp64["ms_per_step"]
        peak64 = mifgpu.probe_fp64_fma()
        flops = FP64_FLOPS_PER_CELL_STEP * cells / (ms64 / 1e3) / 1e12
        fp64["fp64_alu_roofline"] = {"achieved_tflops": round(flops, 4), "peak_tflops": round(peak64, 4),
                                     "frac": round(flops / peak64, 4),
                                     "flops_per_cell_step": FP64_FLOPS_PER_CELL_STEP,
                                     "peak_source": "FMA-chain probe (mifgpu_probe_fp64_fma)"}
        hbm64 = step_sweeps("fp64") * 8 * cells / (ms64 / 1e3) / 1e9
        fp64["hbm_roofline"] = {"achieved_gbs": round(hbm64, 1), "peak_gbs": peak, "frac": round(hbm64 / peak, 4)}
    mixed = None
    if prec == "compensated" and not args.no_mixed:
        mixed = comparison_run(mifgpu, args.workload, "mixed", stream, args.steps, total_steps)
        mixed["note"] = "plain float state (stochastically rounded updates), no residual"
    matched = None
    if linf and fp64 and "velocity_linf" in fp64:
        matched = {"velocity_linf": linf["velocity_linf"], "fp64_velocity_linf": fp64["velocity_linf"],
                   "ratio": linf["velocity_linf"] / fp64["velocity_linf"], "target_ratio": 2.0,
                   "speedup_vs_fp64": round(fp64["ms_per_step"] / step_ms, 2), "target_speedup": 1.7,
                   "t": linf["t"]}
        if mixed and "velocity_linf" in mixed:
            matched["plain_mixed_ratio"] = mixed["velocity_linf"] / fp64["velocity_linf"]

    adjoint = None
    if not args.no_adjoint:
        adjoint = adjoint_bench(stream)

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(workers=1)

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(step_ms, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if prec == "fp64" else "f32", "data": "synthetic",
            "config": line_config(args.workload, prec, world),
            "clocks": clk.summary(), "e2e": e2e, "gpu_launches": launches, "roofline": roofline,
            "step_roofline": {"bytes_per_cell_step": ssw * elem, "achieved_gbs": round(step_roofline, 1),
                              "frac": round(step_roofline / peak, 4)},
            "kernel_ms_per_step": {k: round(v, 4) for k, v in prof.items()}, "kernels": per_kernel,
            "error": linf, "matched_error": matched, "fp64": fp64, "mixed": mixed, "adjoint": adjoint,
            "cpu_baseline": cpu,
        }
        if prec == "mixed":
            line["step_roofline"]["fused_dataflow_bytes_per_cell_step"] = FUSED_STEP_SWEEPS * elem
            line["step_roofline"]["fused_dataflow_frac"] = round(step_roofline * FUSED_STEP_SWEEPS / ssw / peak, 4)
        print(json.dumps(line))


def run_reference(args):
    """The reference's CPU step on every host core (one replica per core, a
    bounded 128^3 sample each), on this arm's metric, unit and config."""
    world, rank, local = dist_setup()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    n = 129
    per_step, wall = cpu_run(cores, n, args.warmup, args.steps, args.workload)
    value = statistics.median(per_step) if per_step else 0.0
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": line_config(args.workload, args.precision, world),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{n - 1}^3-cell Ethier-Steinman cube per core (the workload's family at a "
                                       f"smaller size), {args.warmup} warm-up + {args.steps} timed steps per "
                                       f"replica, {cores} independent replicas, value the median over the timed "
                                       f"steps of all replicas' cells over the slowest replica's time; "
                                       f"oracle/mif_oracle.c (bit-exact restatement of the reference's step, FFT "
                                       f"stand-in for FFTW) built {CPU_FLAGS}; {cpu_model()} (wall {wall:.1f}s)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="cube512", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="compensated", choices=sorted(PRECISIONS))
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--configs", action="store_true", help="the reference's configurations 1-3 (one JSON line)")
    ap.add_argument("--sweep", action="store_true", help="Ethier-Steinman refinement 32^3..768^3 (one JSON line)")
    ap.add_argument("--velocity", action="store_true",
                    help="the reference's velocity-only benchmark, N = 32..512 (one JSON line)")
    ap.add_argument("--adjoint-only", action="store_true",
                    help="only the adjoint workload (a profiling aid; prints {'adjoint': ...})")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.configs or args.sweep or args.velocity:
        import torch

        import build as pkg_build

        pkg_build.build()
        stream = torch.cuda.Stream()
        if args.configs:
            print(json.dumps({"configs": config_suite(stream)}))
        elif args.sweep:
            print(json.dumps({"sweep": sweep(stream)}))
        else:
            print(json.dumps({"velocity_benchmark": velocity_benchmark(stream)}))
    elif args.adjoint_only:
        import torch

        import build as pkg_build

        pkg_build.build()
        stream = torch.cuda.Stream()
        print(json.dumps({"adjoint": adjoint_bench(stream)}))
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
