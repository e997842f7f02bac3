"""Benchmark of the GB300-native Nebo evaluator (one JSON line on rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload W]

Default workload (the headline): the deep fused FP64 expression at 256^3 interior + 1 ghost
layer -- out <<= cond(mask,0)(Interp(Grad(Interp(a)))*exp(b)+sin(c)), f <<= BoxFilter(out),
then nebo_sum/max/norm(f) -- on seeded synthetic inputs (a, b, c ~ U(-1,1), mask = 5% of
cells + every boundary cell).  A step is one pass of that chain; the metric is cell-updates
per second (interior cells x steps / time).  Other workloads (--workload heat, heat32) time the
fused heat-equation step.

value    device time of K steps, inputs resident in HBM, CUDA events on the launching stream.
         Every input is larger than L2 (129 MB), so no flush is needed between steps.
e2e      the same steps through the C ABI with host buffers: each step copies its inputs from
         pinned host memory and reads the reductions back.
roofline the dominant kernel's algorithmic bytes per launch / its mean event-timed duration.
cpu_baseline  the oracle (CPU restatement of the reference's serial walk) on a bounded sample.

--impl reference times the reference's CPU path (the oracle port with every host thread;
the reference tree itself does not exist on the GPU host) on the same metric.
Multi-GPU: the path does not shard across GPUs here (replicas only): each rank runs the full
workload on its own GPU and value sums the ranks' cell-updates over the slowest rank's time.
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

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

import __graft_entry__ as graft  # noqa: E402

N_DEFAULT = 256
BYTES_PER_CELL = {  # algorithmic bytes per cell-update of the dominant kernel
    "deep": 8 * 3 + 8 + 1.0 / 8.0,   # a, b, c read, out written, 1 mask bit
    "heat": 8 * 3,                   # T, lambda read, T' written
    "heat32": 4 * 3,
    "patches": 8 * 2,    # T read, T' written (lambda is a scalar per patch)
    "patches32": 4 * 2,  # FP32 state read and written
    # one RK stage, averaged over the two: phi (stencil) + u,v,w,lambda read, state accumulation
    # read/written; stage 2 also reads the step's start state (8 bytes, so 4 on average)
    "transport": 8 * 5 + 8 + 8 + 4,        # FP64: phi, u, v, w, lam, acc read; out written
    "transport32": 4 * 5 + 8 + 8 + 4 + 4,  # FP32 storage: 5 float reads, FP64 acc r/w, float copy written
    # one reverse step: T_k, A_{k+1}, lambda read, glam read and written, A_k written
    "adjoint": 8 * 6,
    # ParticleToCell fill, per particle: x, y, z, size and value read (its entries are not counted)
    "particles": 8 * 5,
}
DOMINANT = {"deep": "deep_chain", "heat": "heat_step_f64", "heat32": "heat_step_f32",
            "patches": "patches_step_f64", "patches32": "patches_step_f32",
            "transport": "transport_stage_f64", "transport32": "transport_stage_f32",
            "adjoint": "heat_adjoint_step", "particles": "particle_to_cell_fill"}


def measured_peak_hbm():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(kernel, workload):
    """DRAM bytes per launch from the committed ncu summary (profiles/traffic.txt), or None."""
    p = os.path.join(REPO, "profiles", "traffic.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        parts = line.split()
        if len(parts) >= 3 and not line.startswith("#") and parts[0] == kernel and parts[1] == workload:
            return float(parts[2])
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every interval_ms while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, bus_id=None, interval_ms=200):
        self.rows = []
        self.proc = None
        self.bus_id = bus_id
        self.interval_ms = interval_ms

    def start(self):
        cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms",
               str(self.interval_ms)]
        if self.bus_id:
            cmd += ["-i", self.bus_id]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([s.strip() for s in line.split(",")])

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                smax.append(float(r[1]))
            except (ValueError, IndexError):
                continue
            for k, name in enumerate(names):
                if len(r) > 4 + k and r[4 + k].lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------------------- workloads
def deep_label(n):
    return f"deep chain {n}^3 + 1 ghost (a SVol; b, c, out, filt XVol; 5% + boundary mask), filter + 4 reductions"


def heat_label(n, dtype):
    return f"heat {n}^3 + 1 ghost, {'FP64 bit-exact' if dtype == 'f64' else 'FP32'} fused RHS + Euler update"


def transport_label(n, dtype):
    prec = {"f64": "FP64", "f32": "FP32 storage, FP64 state accumulation"}.get(
        dtype, "FP64, and FP32 storage with FP64 state accumulation")
    return f"transport {n}^3 + 2 ghosts, Heun RK2 step, {prec}"


def patches_label(count, cells, dtype):
    prec = {"f64": "FP64", "f32": "FP32"}.get(dtype, "FP64 and FP32")
    return (f"{count} heat patches, edges ~ U{{16..96}}, 1 ghost, {cells / 1e6:.1f} M cells, "
            f"{prec}; one persistent launch per step")


def adjoint_label(n, steps):
    return (f"adjoint {n}^3 + 1 ghost, {steps} FP64 steps, sqrt(N) checkpoints; FP64 adjoint state, "
            f"FP32 face products in dJ/dlambda")


def particles_label(n, npart):
    return (f"particles: {n}^3 SVol + 1 ghost, {npart / 1e6:.1f} M particles (edges U(0.5,1.5) cells, "
            f"random order); step = CellToParticle + ParticleToCell, FP64, bit-identical to the reference")


class Deep:
    name = "deep"

    def __init__(self, N, n):
        import torch

        from spatialops_gb300 import workloads as W

        self.N, self.n = N, n
        a, b, c, pts = W.deep_inputs((n, n, n))
        self.host = [torch.from_numpy(x).pin_memory() for x in (a, b, c)]
        words = W.mask_bits_from_points(pts, (n, n, n))
        self.host_mask = torch.from_numpy(words.view(np.int32)).pin_memory()
        self.A = N.Field("SVol", n, 1)
        self.B = N.Field("XVol", n, 1)
        self.C = N.Field("XVol", n, 1)
        for f, h in zip((self.A, self.B, self.C), self.host):
            f.tensor.copy_(h)
        self.words = self.host_mask.to("cuda")
        self.out = N.Field("XVol", n, 1)
        self.filt = N.Field("XVol", n, 1)
        self.red = torch.zeros(4, dtype=torch.float64, device="cuda")
        self.cells = n ** 3
        self.launches_per_step = 2  # chain; filter with the four reductions (ghost shell and final merge in the same grid)
        self.label = deep_label(n)
        self.h2d_bytes = sum(h.numel() * h.element_size() for h in self.host) + self.host_mask.numel() * 4
        self.d2h_bytes = 4 * 8
        self.host_red = torch.zeros(4, dtype=torch.float64).pin_memory()

    def step(self):
        self._chain(self.A, self.B, self.C, self.words)

    def _chain(self, A, B, C, words):
        # nebo_sum, nebo_max (and min), nebo_norm of filt folded into the filter kernel
        self.N.deep_chain(A, B, C, words, self.out, self.filt, reductions=self.red)

    # e2e: every step uploads its inputs (a, b, c, mask words) from pinned host memory and reads
    # its reductions back.  The uploads run on a copy stream into two alternating device input
    # sets, so step k+1's upload overlaps step k's kernels; each upload still happens inside the
    # timed region, after the start event.
    def e2e_begin(self, start_event):
        import torch

        N, n = self.N, self.n
        if not hasattr(self, "sets"):
            self.sets = [(self.A, self.B, self.C, self.words),
                         (N.Field("SVol", n, 1), N.Field("XVol", n, 1), N.Field("XVol", n, 1),
                          torch.empty_like(self.words))]
            self.copy_stream = torch.cuda.Stream()
            self.ready = [torch.cuda.Event(), torch.cuda.Event()]
            self.free = [torch.cuda.Event(), torch.cuda.Event()]
        self.copy_stream.wait_event(start_event)
        self.k = 0

    def step_e2e(self):
        import torch

        i = self.k % 2
        A, B, C, words = self.sets[i]
        cur = torch.cuda.current_stream()
        cs = self.copy_stream
        with torch.cuda.stream(cs):
            if self.k >= 2:
                cs.wait_event(self.free[i])  # step k-2 is done reading this set
            for f, h in zip((A, B, C), self.host):
                f.tensor.copy_(h, non_blocking=True)
            words.copy_(self.host_mask, non_blocking=True)
            self.ready[i].record(cs)
        cur.wait_event(self.ready[i])
        self._chain(A, B, C, words)
        self.free[i].record(cur)
        self.host_red.copy_(self.red, non_blocking=True)
        self.k += 1


class Heat:
    def __init__(self, N, n, dtype):
        import torch

        from spatialops_gb300 import workloads as W

        self.name = "heat" if dtype == "f64" else "heat32"
        self.label = heat_label(n, dtype)
        self.N, self.n = N, n
        lam, T0, dt = W.heat_inputs((n, n, n))
        self.dt = dt
        tdt = torch.float64 if dtype == "f64" else torch.float32
        self.host = [torch.from_numpy(x).to(tdt).pin_memory() for x in (T0, lam)]
        self.T = N.Field("SVol", n, 1, dtype=dtype)
        self.Tt = N.Field("SVol", n, 1, dtype=dtype)
        self.L = N.Field("SVol", n, 1, dtype=dtype)
        self.T.tensor.copy_(self.host[0])
        self.L.tensor.copy_(self.host[1])
        N.fill_periodic(self.T)
        N.fill_periodic(self.L)
        self.cells = n ** 3
        self.launches_per_step = 1
        self.h2d_bytes = sum(h.numel() * h.element_size() for h in self.host)
        self.d2h_bytes = 8
        self.red = torch.zeros(1, dtype=torch.float64, device="cuda")
        self.host_red = torch.zeros(1, dtype=torch.float64).pin_memory()
        self.k = 0

    def reset(self):
        """T back to the initial state (ghosts filled)."""
        self.T.tensor.copy_(self.host[0])
        self.N.fill_periodic(self.T)
        self.k = 0

    def step(self):
        a, b = (self.T, self.Tt) if self.k % 2 == 0 else (self.Tt, self.T)
        self.N.heat_step(a, b, self.L, self.dt)
        self.k += 1

    def step_e2e(self):
        self.T.tensor.copy_(self.host[0], non_blocking=True)
        self.L.tensor.copy_(self.host[1], non_blocking=True)
        self.k = 0
        self.step()
        self.N.reduce_async(self.Tt, "sum", False, self.red)
        self.host_red.copy_(self.red, non_blocking=True)


class Patches:
    """512 heat patches, edges ~ U{16..96}; a step advances every patch once (one launch)."""

    def __init__(self, N, dtype, count=512):
        import torch

        from spatialops_gb300 import workloads as W

        self.name = "patches" if dtype == "f64" else "patches32"  # patches32: FP32 storage
        self.N = N
        shapes = W.patch_shapes(count)
        ins = W.patch_inputs(shapes)
        self.ps = N.PatchSet(shapes, np.array([t[0] for t in ins]), np.array([t[2] for t in ins]), dtype)
        self.ps.autotune()
        self.host = torch.zeros(self.ps.total, dtype=torch.float64).pin_memory()
        for p, (_, T0, _) in enumerate(ins):
            o = int(self.ps.offsets[p])
            self.host[o:o + T0.size].copy_(torch.from_numpy(T0.reshape(-1)))
        self.ps.arena(0).copy_(self.host)
        self.ps.fill_ghosts(0)
        self.cells = int(np.prod(shapes.astype(np.int64), axis=1).sum())
        self.label = patches_label(count, self.cells, dtype)
        self.launches_per_step = 1
        self.h2d_bytes = self.host.numel() * self.host.element_size()
        self.d2h_bytes = 8
        self.red = torch.zeros(1, dtype=torch.float64, device="cuda")
        self.host_red = torch.zeros(1, dtype=torch.float64).pin_memory()
        self.parity = 0
        self.graph_steps = None

    def step(self):
        self.parity = self.ps.run(1, start=self.parity)

    def run(self, k):
        self.parity = self.ps.run(k, start=self.parity)

    def step_e2e(self):
        self.ps.arena(0).copy_(self.host, non_blocking=True)
        self.ps.fill_ghosts(0)
        self.parity = self.ps.run(1, start=0)
        self.ps.sync(self.parity)
        self.red.copy_(self.ps.arena(self.parity)[:1], non_blocking=True)
        self.host_red.copy_(self.red, non_blocking=True)


class TransportWL:
    """Scalar transport at n^3 + 2 ghosts; a step is one Heun RK2 step (two stage kernels)."""

    def __init__(self, N, n, dtype):
        import torch

        from spatialops_gb300 import workloads as W

        self.name = "transport" if dtype == "f64" else "transport32"
        self.label = transport_label(n, dtype)
        self.N, self.n = N, n
        phi, u, v, w, lam, dt, nu = W.transport_inputs_device(n)
        self.t = N.Transport(np.zeros((1, 1, 1)), np.zeros((1, 1, 1)), np.zeros((1, 1, 1)), np.zeros((1, 1, 1)),
                             np.zeros((1, 1, 1)), n, dt, nu, dtype)
        tdt = torch.float64 if dtype == "f64" else torch.float32
        self.t.phi = phi
        self.t.coef = [q.to(tdt).contiguous() for q in (u, v, w, lam)]
        self.host = [phi.cpu().pin_memory()]
        self.cells = n ** 3
        self.launches_per_step = 2
        self.h2d_bytes = self.host[0].numel() * 8
        self.d2h_bytes = 8
        self.red = torch.zeros(4, dtype=torch.float64, device="cuda")
        self.host_red = torch.zeros(4, dtype=torch.float64).pin_memory()
        self.phi_field = N.Field("SVol", n, 2, tensor=self.t.phi)

    def step(self):
        self.t.run(1)

    def run(self, k):
        # k RK2 steps in one nebo_transport_run call, as a time loop runs them: the coefficient
        # ghost fills and the FP32 copy of the state are made once per call, the steps' stage
        # kernels k times
        self.t.run(k)

    def step_e2e(self):
        self.t.phi.copy_(self.host[0], non_blocking=True)
        self.t.run(1)
        self.N.reduce_all(self.phi_field, True, self.red)  # FP64 reductions of the FP64 state
        self.host_red.copy_(self.red, non_blocking=True)


class AdjointWL:
    """Gradient of J = 1/2 sum (T_N - T_target)^2 w.r.t. T0 and lambda: 500 FP64 heat steps at
    192^3 with sqrt(N) checkpointing.  A step is one full gradient (forward sweep with
    checkpoints, segment recomputation, reverse sweep); the metric counts forward cell-steps
    (n^3 * 500) per second of gradient time, and the line adds the gradient / forward time ratio."""

    name = "adjoint"

    def __init__(self, N, n, steps=500):
        import torch

        from spatialops_gb300 import workloads as W

        self.N, self.n, self.nsteps = N, n, steps
        lam, T0, dt, lam_t = W.adjoint_inputs((n, n, n))
        self.dt = dt
        self.host = [torch.from_numpy(x).pin_memory() for x in (T0, lam)]
        self.T0 = N.Field.from_numpy("SVol", T0, 1)
        self.L = N.Field.from_numpy("SVol", lam, 1)
        # target: the same run with the perturbed lambda (on the device)
        self.Tt = N.Field.from_numpy("SVol", T0, 1)
        tmp = N.Field("SVol", n, 1)
        N.heat_run(self.Tt, tmp, N.Field.from_numpy("SVol", lam_t, 1), steps, dt)
        self.cells = n ** 3 * steps
        self.launches_per_step = None
        self.h2d_bytes = sum(h.numel() * h.element_size() for h in self.host)
        self.d2h_bytes = 8
        self.J = 0.0
        self.products = "f32"
        self.label = adjoint_label(n, steps)
        self.metric = "adjoint gradient forward-cell-steps/s"
        self.cells_per_launch = n ** 3

    def step(self):
        self.J, self.gT, self.gl = self.N.heat_gradient(self.T0, self.L, self.Tt, self.nsteps, self.dt,
                                                        products=self.products)

    def gradient_ms(self, products, checkpoint_every=0, forward="f64"):
        """Device time of one gradient with the given face-product precision, checkpoints and
        forward-state precision."""
        import torch

        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        self.N.heat_gradient(self.T0, self.L, self.Tt, self.nsteps, self.dt, checkpoint_every, products=products,
                             forward=forward)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    def step_e2e(self):
        self.T0.tensor.copy_(self.host[0], non_blocking=True)
        self.L.tensor.copy_(self.host[1], non_blocking=True)
        self.step()  # J comes back to the host at the end of the call

    def forward_ms(self, reps=2):
        """Device time of the plain forward run (500 steps, CUDA graph) for the cost ratio."""
        import torch

        N = self.N
        T = N.Field("SVol", self.n, 1)
        tmp = N.Field("SVol", self.n, 1)
        T.tensor.copy_(self.T0.tensor)
        N.heat_run(T, tmp, self.L, self.nsteps, self.dt)  # warm (graph capture)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            N.heat_run(T, tmp, self.L, self.nsteps, self.dt)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps


class ParticlesWL:
    """Particle <-> cell exchange: a 256^3 SVol cell field + 1 ghost and one particle per interior
    cell (16.8 M), edges ~ U(0.5, 1.5) cells, centres uniform with every box inside the window,
    in random order.  A step is CellToParticle (cell field -> one value per particle) then
    ParticleToCell (particle values -> cell field); the metric counts particles per second."""

    name = "particles"

    def __init__(self, N, n):
        import torch

        self.N, self.n = N, n
        self.npart = n ** 3
        gen = torch.Generator(device="cuda").manual_seed(12)
        d = 1.0 / n
        self.spacing, self.low = (d, d, d), (0.5 * d,) * 3
        face = 0.5 * d - d - d / 2
        span = (n + 2) * d
        f64 = dict(device="cuda", dtype=torch.float64)
        self.size = torch.rand(self.npart, generator=gen, **f64) * d + 0.5 * d
        self.pos = [face + self.size / 2 + torch.rand(self.npart, generator=gen, **f64) * (span - self.size)
                    for _ in range(3)]
        self.pval = torch.rand(self.npart, generator=gen, **f64)
        self.gas = N.Field("SVol", n, 1)
        self.gas.tensor.copy_(torch.rand(self.gas.tensor.shape, generator=gen, **f64))
        self.src_field = N.Field("SVol", n, 1)
        self.out_p = torch.empty(self.npart, **f64)
        self.host_in = [t.cpu().pin_memory() for t in (*self.pos, self.size, self.pval, self.gas.tensor)]
        self.host_out = [torch.empty(self.npart, dtype=torch.float64).pin_memory(),
                         torch.empty(self.src_field.tensor.shape, dtype=torch.float64).pin_memory()]
        self.cells = self.npart
        self.cells_per_launch = self.npart
        self.launches_per_step = 7  # gather, count, 3 scan kernels, fill, fold
        self.h2d_bytes = sum(h.numel() * h.element_size() for h in self.host_in)
        self.d2h_bytes = sum(h.numel() * h.element_size() for h in self.host_out)
        self.metric = "particle cell<->particle exchanges/s"
        self.unit = "Gparticle/s"
        self.label = particles_label(n, self.npart)

    def step(self):
        N = self.N
        N.cell_to_particle(self.gas, *self.pos, self.size, self.out_p, self.spacing, self.low)
        N.particle_to_cell(self.pval, *self.pos, self.size, self.src_field, self.spacing, self.low)

    def step_e2e(self):
        for t, h in zip((*self.pos, self.size, self.pval, self.gas.tensor), self.host_in):
            t.copy_(h, non_blocking=True)
        self.step()
        self.host_out[0].copy_(self.out_p, non_blocking=True)
        self.host_out[1].copy_(self.src_field.tensor, non_blocking=True)


def make_workload(N, name, n):
    if name in ("transport", "transport32"):
        return TransportWL(N, n, "f64" if name == "transport" else "f32")
    if name in ("patches", "patches32"):
        return Patches(N, "f64" if name == "patches" else "f32")
    if name == "deep":
        return Deep(N, n)
    if name == "heat":
        return Heat(N, n, "f64")
    if name == "heat32":
        return Heat(N, n, "f32")
    if name == "adjoint":
        return AdjointWL(N, 192 if n == N_DEFAULT else n)
    if name == "particles":
        return ParticlesWL(N, n)
    raise SystemExit(f"unknown workload {name}")


# ----------------------------------------------------------------------------- metric parts
# The metric names several comparisons ("Gcell-upd/s & %HBM peak: batched/FP32 vs plain FP64;
# adjoint/fwd cost ratio").  The headline line carries each of them, timed in the same run with
# CUDA events on the launching stream, each with its own clock record:
#   heat_fp64     the plain FP64 heat RHS + Euler update at 256^3: Gcell-upd/s and %HBM peak
#   patches       512 batched patches x 200 steps: FP32 / FP64 cell-update ratio and the
#                 largest per-patch relative error of the FP32 state against the FP64 one
#   transport     512^3 + 2 ghosts, 50 RK2 steps: FP32-storage / FP64 ratio and relative error
#   adjoint       192^3 x 500 steps: gradient / forward device-time ratios
#   dropin        `<<=` itself (tests/cpp/assign_timing): the deep chain, the box filter and the
#                 heat update written as the reference's users write them, against the hand kernels
def _timed(fn, steps, bus):
    """(ms per step, clocks) of `steps` calls of fn (or one fn(steps) call when fn takes k)."""
    import torch

    sampler = ClockSampler(bus, interval_ms=100)
    sampler.start()
    time.sleep(0.25)
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    fn(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    return e0.elapsed_time(e1) / steps, clocks


def _steps_for(fn, target_s=0.6, cap=4000):
    """How many steps fill about target_s of device time (one warm call of fn(1) measured)."""
    import torch

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    fn(1)
    e1.record()
    torch.cuda.synchronize()
    ms = max(e0.elapsed_time(e1), 1e-3)
    return int(max(3, min(cap, target_s * 1e3 / ms)))


def part_heat(N, bus, peak):
    W = Heat(N, 256, "f64")
    run = lambda k: [W.step() for _ in range(k)]
    run(3)
    k = _steps_for(run)
    ms, clocks = _timed(run, k, bus)
    cells = W.cells
    gbs = BYTES_PER_CELL["heat"] * cells / (ms * 1e-3) / 1e9
    out = {"workload": heat_label(256, "f64"), "gcell_upd_s": cells / (ms * 1e-3) / 1e9, "ms_per_step": ms,
           "steps": k, "alg_gbs": gbs, "hbm_frac": gbs / peak, "hbm_peak_gbs": peak, "clocks": clocks}
    # the same steps in the integer forms, k steps in one nebo_heat_run_ex call each, from the
    # initial state (the exact steps above grew it x1.4 per step; from there the k steps below
    # stay finite and inside the integer forms' ranges):
    #   NEBO_HEAT_FIXED_POINT: FP64 state, fluxes on the integer pipe (two exponent reductions per
    #   call, a 4-byte reset per step);
    #   NEBO_HEAT_FIXED_STATE: the state itself in 64-bit integers (one conversion pass in, one
    #   out per call, both inside the timed region)
    for key, mode in (("fixed_point", "fixed"), ("fixed_state", "fixed_state")):
        runm = lambda kk, m=mode: N.heat_run_ex(W.T, W.Tt, W.L, kk, W.dt, mode=m)
        W.reset()
        runm(3)
        W.reset()
        msf, clocksf = _timed(runm, k, bus)
        gbsf = BYTES_PER_CELL["heat"] * cells / (msf * 1e-3) / 1e9
        out[key] = {"gcell_upd_s": cells / (msf * 1e-3) / 1e9, "ms_per_step": msf, "steps": k,
                    "alg_gbs": gbsf, "hbm_frac": gbsf / peak, "clocks": clocksf,
                    "accuracy": "within 1e-13 relative max-norm of the bit-exact form (tests)"}
    # FP32 storage and arithmetic (the bandwidth path), and its error against the FP64 step after
    # 50 steps from the same state at the stable step 0.15 / max(lambda)
    W32 = Heat(N, 256, "f32")
    run32 = lambda kk: [W32.step() for _ in range(kk)]
    run32(3)
    k32 = _steps_for(run32)
    ms32, clocks32 = _timed(run32, k32, bus)
    gbs32 = BYTES_PER_CELL["heat32"] * cells / (ms32 * 1e-3) / 1e9
    dt_stable = W.dt * 0.75

    def state_after(w, steps):
        w.T.tensor.copy_(w.host[0])
        N.fill_periodic(w.T)
        a, b = w.T, w.Tt
        for _ in range(steps):
            N.heat_step(a, b, w.L, dt_stable)
            a, b = b, a
        return a.tensor[1:-1, 1:-1, 1:-1].double()

    s64, s32 = state_after(W, 50), state_after(W32, 50)
    err = float((s32 - s64).abs().max() / s64.abs().max())
    # the heat configuration itself: 64^3 + 1 ghost, 100 FP64 steps in one nebo_heat_run (a CUDA
    # graph of the 100 launches; the fields fit in L2, so launches and latency bound it)
    from spatialops_gb300 import workloads as WL

    # (dt = 0.15 / max lambda: the configuration's 0.2 grows the checkerboard mode x1.4 per step,
    # and the 2400 timed steps would overflow)
    lam64, T064, dt64 = WL.heat_inputs((64, 64, 64), cfl=0.15)
    T64 = N.Field.from_numpy("SVol", T064, 1)
    Tt64 = N.Field("SVol", (64, 64, 64), 1)
    L64 = N.Field.from_numpy("SVol", lam64, 1)
    c1 = {"workload": "heat 64^3 + 1 ghost, 100 FP64 Euler steps per call, dt = 0.15 / max lambda",
          "steps_per_call": 100, "launches": "one CUDA graph per call (captured once) in every mode"}
    for mode in ("exact", "fixed", "fixed_state"):
        call = (lambda k: [N.heat_run(T64, Tt64, L64, 100, dt64) for _ in range(k)]) if mode == "exact" else \
            (lambda k, m=mode: [N.heat_run_ex(T64, Tt64, L64, 100, dt64, mode=m, use_graph=True) for _ in range(k)])
        call(2)
        ms1, clocks1 = _timed(call, 10, bus)
        c1[mode] = {"ms_per_call": ms1, "us_per_step": ms1 * 10.0,
                    "gcell_upd_s": 64 ** 3 * 100 / (ms1 * 1e-3) / 1e9, "clocks": clocks1}
    out["config_64cubed_100_steps"] = c1
    out["fp32"] = {"gcell_upd_s": cells / (ms32 * 1e-3) / 1e9, "ms_per_step": ms32, "steps": k32,
                   "alg_gbs": gbs32, "hbm_frac": gbs32 / peak, "clocks": clocks32,
                   "fp32_over_fp64": ms / ms32, "rel_err_50_steps_vs_fp64": err,
                   "error_reference": "the bit-exact FP64 step (equal to the oracle bit for bit)"}
    return out


def part_patches(N, bus):
    import torch

    out = {}
    states = {}
    for dtype in ("f64", "f32"):
        W = Patches(N, dtype)
        W.run(3)
        k = _steps_for(W.run)
        ms, clocks = _timed(W.run, k, bus)
        out[dtype] = {"gcell_upd_s": W.cells / (ms * 1e-3) / 1e9, "ms_per_step": ms, "steps": k, "clocks": clocks}
        # 200 steps from the initial state for the error
        W.ps.arena(0).copy_(W.host)
        W.ps.fill_ghosts(0)
        fin = W.ps.run(200, start=0)
        W.ps.sync(fin)
        states[dtype] = [W.ps.window(fin, p).clone() for p in range(W.ps.npatch)]
        cells = W.cells
        del W
        torch.cuda.empty_cache()
    errs = [float((a - b).abs().max() / b.abs().max()) for a, b in zip(states["f32"], states["f64"])]
    return {"workload": patches_label(512, cells, "f64/f32"), "fp64": out["f64"], "fp32": out["f32"],
            "fp32_over_fp64": out["f32"]["gcell_upd_s"] / out["f64"]["gcell_upd_s"],
            "fp32_max_patch_rel_err_200_steps": max(errs), "fp32_median_patch_rel_err_200_steps": float(np.median(errs)),
            "error_reference": "the FP64 patch set (bit-identical to the oracle's serial walk per patch)"}


def part_transport(N, bus):
    import torch

    out, phis = {}, {}
    for dtype in ("f64", "f32"):
        W = TransportWL(N, 512, dtype)
        phi0 = W.t.phi.clone()
        W.run(1)
        k = 10 if dtype == "f64" else 40
        ms, clocks = _timed(W.run, k, bus)
        out[dtype] = {"gcell_upd_s": W.cells / (ms * 1e-3) / 1e9, "ms_per_step": ms, "steps": k, "clocks": clocks}
        W.t.phi.copy_(phi0)
        W.run(50)
        g = 2
        phis[dtype] = W.t.phi[g:-g, g:-g, g:-g].clone()
        del W, phi0
        torch.cuda.empty_cache()
    err = float((phis["f32"] - phis["f64"]).abs().max() / phis["f64"].abs().max())
    return {"workload": transport_label(512, "f64/f32"), "fp64": out["f64"], "fp32": out["f32"],
            "fp32_over_fp64": out["f32"]["gcell_upd_s"] / out["f64"]["gcell_upd_s"],
            "fp32_rel_err_50_steps": err, "error_reference": "the FP64 transport (1e-13 of the oracle on small cases)"}


def part_adjoint(N, bus):
    import torch

    W = AdjointWL(N, 192)
    sampler = ClockSampler(bus, interval_ms=100)
    sampler.start()
    fwd = W.forward_ms()
    W.gradient_ms("f64")  # warm
    g64 = W.gradient_ms("f64")
    g32 = W.gradient_ms("f32")
    W.gradient_ms("f32", N.CHECKPOINT_AUTO)  # warm: the pool grows to hold every state
    gall = W.gradient_ms("f32", N.CHECKPOINT_AUTO)
    W.gradient_ms("f64", forward="f32")  # warm
    gf32 = W.gradient_ms("f64", forward="f32")
    clocks = sampler.stop()
    del W
    torch.cuda.empty_cache()
    return {"workload": adjoint_label(192, 500), "forward_ms": fwd, "gradient_ms_fp64": g64,
            "gradient_ms_f32_products": g32, "gradient_ms_every_state_kept": gall,
            "adjoint_over_forward_fp64": g64 / fwd, "adjoint_over_forward_f32_products": g32 / fwd,
            "adjoint_over_forward_every_state_kept": gall / fwd,
            "gradient_ms_fp32_forward": gf32, "adjoint_over_forward_fp32_forward": gf32 / fwd,
            "fp32_forward_note": "FP32 forward states and checkpoints, FP64 adjoint and products; "
                                 "the ratio is against the FP64 forward run",
            "checkpoints": "ceil(sqrt(500)) = 23",
            "clocks": clocks}


def part_dropin(bus):
    """`<<=` through the drop-in headers (C++ program built by build.py), parsed from its JSON."""
    exe = os.path.join(REPO, "tests", "cpp", "_build", "assign_timing")
    if not os.path.exists(exe):
        return {"unavailable": "tests/cpp/_build/assign_timing not built"}
    sampler = ClockSampler(bus, interval_ms=100)
    sampler.start()
    r = subprocess.run([exe, "256", "10"], capture_output=True, text=True, timeout=600)
    clocks = sampler.stop()
    if r.returncode != 0:
        return {"unavailable": f"assign_timing exited {r.returncode}: {r.stderr.strip()[-200:]}"}
    d = json.loads(r.stdout.strip().splitlines()[-1])
    d["clocks"] = clocks
    d["deep_assign_over_hand_chain"] = d["deep_assign"]["ms"] / d["deep_hand_chain"]["ms"]
    d["filter_assign_over_hand"] = d["filter_assign"]["ms"] / d["filter_hand"]["ms"]
    d["heat_assign_over_hand"] = d["heat_assign"]["ms"] / d["heat_hand"]["ms"]
    # the transport configuration written in Nebo (FP64, 512^3 + 2 ghosts), one RK2 step
    exe_t = os.path.join(REPO, "tests", "cpp", "_build", "configs_dropin")
    if os.path.exists(exe_t):
        r = subprocess.run([exe_t, "transport-time", "512", "3"], capture_output=True, text=True, timeout=600)
        if r.returncode == 0:
            t = json.loads(r.stdout.strip().splitlines()[-1])
            t["assign_over_hand"] = t["transport_assign"]["ms_per_rk2_step"] / t["transport_hand"]["ms_per_rk2_step"]
            d["transport"] = t
        else:
            d["transport"] = {"unavailable": f"configs_dropin exited {r.returncode}: {r.stderr.strip()[-200:]}"}
    return d


def metric_parts(N, bus, peak):
    parts = {}
    for name, fn in (("heat_fp64", lambda: part_heat(N, bus, peak)), ("patches", lambda: part_patches(N, bus)),
                     ("transport", lambda: part_transport(N, bus)), ("adjoint", lambda: part_adjoint(N, bus)),
                     ("dropin", lambda: part_dropin(bus))):
        t0 = time.perf_counter()
        try:
            parts[name] = fn()
        except Exception as e:  # a part that fails is reported, the headline stands
            parts[name] = {"error": f"{type(e).__name__}: {e}"}
        parts[name]["wall_s"] = time.perf_counter() - t0
    return parts


# ----------------------------------------------------------------------------- CPU legs
def _oracle():
    sys.path.insert(0, os.path.join(REPO, "tests"))
    import oracle_dsl as O  # the checker / CPU restatement of the reference's serial walk

    return O


def cpu_run(workload, n_xy, nz, threads):
    """One step of the workload on the CPU oracle over an n_xy x n_xy x nz block; returns seconds."""
    return cpu_stepper(workload, (n_xy, n_xy, nz))(threads)


def cpu_stepper(workload, shape):
    """A sampler: one deep-chain or heat step on the CPU oracle over `shape` (inputs made once);
    sampler(threads) returns seconds."""
    O = _oracle()
    from spatialops_gb300 import workloads as W

    if workload == "deep":
        a, b, c, pts = W.deep_inputs(shape)
        bits = W.mask_bits_from_points(pts, shape)

        def run(threads):
            t0 = time.perf_counter()
            O.deep_run(a, b, c, bits, shape, 1.0, threads)
            return time.perf_counter() - t0

        return run
    lam, T0, dt = W.heat_inputs(shape)

    def run(threads):
        t0 = time.perf_counter()
        O.heat_run(lam, T0, shape, 1, dt, threads)
        return time.perf_counter() - t0

    return run


def cpu_patches(count=512):
    """A sampler: one step of every patch of the 512-patch set by the oracle (each patch's walk
    over z-slabs with the given threads); sampler(threads) returns seconds."""
    O = _oracle()
    from spatialops_gb300 import workloads as W

    shapes = W.patch_shapes(count)
    ins = W.patch_inputs(shapes)
    lams = [np.full_like(T0, lam) for lam, T0, _ in ins]

    def run(threads):
        t0 = time.perf_counter()
        for p, (lam, T0, dt) in enumerate(ins):
            O.heat_run(lams[p], T0, tuple(int(v) for v in shapes[p]), 1, dt, threads)
        return time.perf_counter() - t0

    return run, int(np.prod(shapes.astype(np.int64), axis=1).sum())


def cpu_particles(n, npart):
    """CellToParticle + ParticleToCell of npart particles on an n^3 field by the serial oracle;
    returns seconds."""
    O = _oracle()
    from spatialops_gb300 import workloads as W

    d = 1.0 / n
    c = W.particle_inputs((n, n, n), 1, npart, axes=7, spacing=(d, d, d), low=(0.5 * d,) * 3,
                          size_range=(0.5, 1.5), seed=12)
    t0 = time.perf_counter()
    O.particle_ops(c)
    return time.perf_counter() - t0


def cpu_transport(m):
    """A sampler: one Heun RK2 step of the FP64 transport on an m^3 periodic patch by the oracle
    (inputs made once); sampler(threads) returns seconds."""
    O = _oracle()
    from spatialops_gb300 import workloads as W

    phi, u, v, w, lam, dt, nu = W.transport_inputs(m)

    def run(threads):
        t0 = time.perf_counter()
        O.transport_run(phi, u, v, w, lam, m, 1, dt, nu, threads)
        return time.perf_counter() - t0

    return run


def cpu_gradient(m, steps):
    """A sampler: the heat gradient (forward run plus the reverse sweep) over `steps` steps on an
    m^3 patch by the serial oracle (inputs made once); sampler(threads) returns seconds."""
    O = _oracle()
    from spatialops_gb300 import workloads as W

    n = (m, m, m)
    lam, T0, dt, _ = W.adjoint_inputs(n)

    def run(threads):
        t0 = time.perf_counter()
        TN = O.heat_run(lam, T0, n, steps, dt)
        O.heat_adjoint(T0, lam, TN - T0, n, steps, dt)
        return time.perf_counter() - t0

    return run


# One bounded sample of each workload by the oracle:
# (function(threads) -> seconds, cell-updates per call, what, same size as the device arm).
# The deep chain, the heat step and the patch set run at full size; the transport and the
# gradient on smaller patches (their full sizes take minutes of host time per step).
def cpu_sample(workload, n):
    if workload in ("deep", "heat", "heat32"):
        kind = "deep" if workload == "deep" else "heat"
        return cpu_stepper(kind, (n, n, n)), n ** 3, f"one full {n}^3 {kind} step", True
    if workload in ("patches", "patches32"):
        fn, cells = cpu_patches()
        return fn, cells, "one step of all 512 patches", True
    if workload in ("transport", "transport32"):
        m = 128
        return cpu_transport(m), m ** 3, f"one FP64 RK2 step on a {m}^3 periodic patch", False
    if workload == "adjoint":
        m, steps = 48, 20
        return cpu_gradient(m, steps), m ** 3 * steps, f"gradient over {steps} steps of a {m}^3 patch", False
    raise ValueError(workload)


def cpu_baseline(workload, n, budget_s=10.0):
    """Serial oracle (1 core) on the full workload, repeated until ~budget_s of CPU work."""
    if workload == "particles":
        npart = 2_000_000
        reps, total = 0, 0.0
        while total < budget_s and reps < 20:
            total += cpu_particles(n, npart)
            reps += 1
        return {"value": reps * npart / total / 1e9, "unit": "Gparticle/s", "cores": 1, "kind": "port",
                "sample": f"{reps} x (CellToParticle + ParticleToCell of {npart} particles on the {n}^3 field), "
                          f"serial oracle loops (the reference's operators are serial), {total:.1f} s"}
    if workload in ("deep", "heat", "heat32"):
        step = cpu_stepper("deep" if workload == "deep" else "heat", (n, n, n))
        reps, total = 0, 0.0
        while total < budget_s and reps < 20:
            total += step(1)
            reps += 1
        cells = reps * n ** 3
        return {"value": cells / total / 1e9, "unit": "Gcell-upd/s", "cores": 1, "kind": "port",
                "sample": f"{reps} full {n}^3 step(s) of the {workload} workload, serial oracle walk, {total:.1f} s"}
    fn, units, what, _ = cpu_sample(workload, n)
    reps, total = 0, 0.0
    while total < budget_s and reps < 50:
        total += fn(1)
        reps += 1
    return {"value": reps * units / total / 1e9, "unit": "Gcell-upd/s", "cores": 1, "kind": "port",
            "sample": f"{reps} x ({what}), serial oracle, {total:.1f} s"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    graft._import_pkg()
    threads = os.cpu_count() or 1
    n = args.n
    if args.workload == "particles":
        # the reference's ParticleToCell / CellToParticle are serial loops over the particles
        npart = 1_000_000
        for _ in range(max(args.warmup, 0)):
            cpu_particles(n, npart)
        t = sum(cpu_particles(n, npart) for _ in range(args.steps))
        value = args.steps * npart / t / 1e9
        line = {
            "impl": "reference", "metric": "particle cell<->particle exchanges/s", "value": value,
            "unit": "Gparticle/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": particles_label(n, n ** 3), "sample": f"{npart} particles per step"},
            "cpu_baseline": {"value": value, "unit": "Gparticle/s", "cores": 1, "kind": "port",
                             "sample": f"CellToParticle + ParticleToCell of {npart} particles on the {n}^3 field per "
                                       f"step, oracle restatement of the reference's serial operator loops"},
            "e2e": {"value": value, "unit": "Gparticle/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line), flush=True)
        return 0
    fn, units, what, same = cpu_sample(args.workload, n)
    for _ in range(max(args.warmup, 0)):
        fn(threads)
    t = 0.0
    for _ in range(args.steps):
        t += fn(threads)
    value = args.steps * units / t / 1e9
    w = args.workload
    if w in ("deep", "heat", "heat32"):
        label = deep_label(n) if w == "deep" else heat_label(n, "f64" if w == "heat" else "f32")
    elif w in ("transport", "transport32"):
        label = transport_label(n, "f64" if w == "transport" else "f32")
    elif w in ("patches", "patches32"):
        from spatialops_gb300 import workloads as W

        cells = int(np.prod(W.patch_shapes(512).astype(np.int64), axis=1).sum())
        label = patches_label(512, cells, "f64" if w == "patches" else "f32")
    else:
        label = adjoint_label(192 if n == N_DEFAULT else n, 500)
    metric = "adjoint gradient forward-cell-steps/s" if w == "adjoint" else f"{w} cell-updates/s"
    line = {
        "impl": "reference", "metric": metric, "value": value, "unit": "Gcell-upd/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": label, "cells_per_step": units, "sample": what + " per step", "same_config": same,
                   "sample_dtype": "f64",
                   "note": ("the reference's CPU path runs FP64 here; the device arm's FP32 storage has no CPU "
                            "counterpart" if w.endswith("32") else "")},
        "cpu_baseline": {"value": value, "unit": "Gcell-upd/s", "cores": 1 if w == "adjoint" else threads,
                         "kind": "port",
                         "sample": f"{what} per step, oracle restatement of the reference's serial walk"
                                   + (", serial" if w == "adjoint" else f", z-slabs over {threads} threads")},
        "e2e": {"value": value, "unit": "Gcell-upd/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------------------- main
def max_over_ranks(x, dist, device):
    """x reduced with MAX over the ranks of dist's default group (x itself without a group)."""
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="deep", choices=["deep", "heat", "heat32", "patches", "patches32", "transport",
                                                             "transport32", "adjoint", "particles"])
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parts", action="store_true",
                    help="skip the metric's other comparisons (heat FP64 %%HBM, FP32/FP64 ratios, adjoint ratio, <<=)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)

    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    graft.build() if not os.path.exists(os.path.join(REPO, "spatialops-threadfix_gb300", "_build",
                                                     "libnebo_gb300.so")) else None
    N = graft._import_pkg()
    W = make_workload(N, args.workload, args.n)
    stream = torch.cuda.current_stream()

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
            torch.cuda.synchronize()

    for _ in range(args.warmup):
        W.step()
    barrier()

    bus = None
    try:
        bus = torch.cuda.get_device_properties(local).pci_bus_id
    except Exception:
        bus = None
    sampler = ClockSampler(bus if isinstance(bus, str) else None)
    sampler.start()
    time.sleep(0.3)
    N.profile_enable(True)
    N.profile_report(reset=True)
    launches0 = N.kernel_launch_count()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    if hasattr(W, "run"):
        W.run(args.steps)  # the steps in one library call (replayed as one CUDA graph for patches)
    else:
        for _ in range(args.steps):
            W.step()
    e1.record(stream)
    barrier()
    ms = e0.elapsed_time(e1)
    launches = N.kernel_launch_count() - launches0
    prof = N.profile_report(reset=True)
    N.profile_enable(False)
    clocks = sampler.stop()
    ms = max_over_ranks(ms, dist, "cuda")
    value = world * W.cells * args.steps / (ms * 1e-3) / 1e9

    # e2e: host buffers, copies inside the timed region
    e_steps = max(3, min(args.steps, 50 if W.name != "adjoint" else 3))
    if hasattr(W, "e2e_begin"):
        warm = torch.cuda.Event()
        warm.record(stream)
        W.e2e_begin(warm)
    for _ in range(2):
        W.step_e2e()
    barrier()
    e0.record(stream)
    if hasattr(W, "e2e_begin"):
        W.e2e_begin(e0)
    for _ in range(e_steps):
        W.step_e2e()
    e1.record(stream)
    barrier()
    e2e_ms = e0.elapsed_time(e1)
    e2e_ms = max_over_ranks(e2e_ms, dist, "cuda")
    e2e_value = world * W.cells * e_steps / (e2e_ms * 1e-3) / 1e9

    dom = DOMINANT[W.name]
    peak, peak_kind = measured_peak_hbm()
    roof = None
    if launches == 0 and hasattr(W, "run"):
        # graph replays: the library counts launches when the graph is captured, not replayed
        launches = args.steps * W.launches_per_step
    if dom not in prof and hasattr(W, "run") and W.launches_per_step == 1:
        prof[dom] = {"launches": args.steps, "ms": ms}  # one kernel per step, timed as a whole
    if dom in prof and prof[dom]["launches"]:
        kms = prof[dom]["ms"] / prof[dom]["launches"]
        alg = BYTES_PER_CELL[W.name] * getattr(W, "cells_per_launch", W.cells)
        achieved = alg / (kms * 1e-3) / 1e9
        traffic = ncu_traffic(dom, f"{W.name}{args.n}")
        roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "kernel": dom, "kernel_ms": kms, "alg_bytes_per_launch": alg,
                "peak_source": f"{peak_kind} hbm_gbs (MEASURED_PEAKS.json)" if peak_kind == "measured" else
                "fallback 6.8 TB/s",
                "kernels": {k: {"launches": v["launches"], "ms_per_launch": v["ms"] / max(v["launches"], 1)}
                            for k, v in prof.items()}}

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        cpu = cpu_baseline(W.name, args.n)
    extra = {}
    if W.name == "adjoint":
        fwd = W.forward_ms()
        g64 = W.gradient_ms("f64")
        W.gradient_ms("f32", W.N.CHECKPOINT_AUTO)  # warm: the pool grows to hold every state
        gall = W.gradient_ms("f32", W.N.CHECKPOINT_AUTO)
        extra = {"adjoint_over_forward": (ms / args.steps) / fwd, "forward_ms": fwd,
                 "forward_value": W.cells / (fwd * 1e-3) / 1e9, "J": W.J,
                 "adjoint_over_forward_all_fp64": g64 / fwd,
                 "adjoint_over_forward_every_state_kept": gall / fwd}
    line = {
        "metric": getattr(W, "metric", f"{W.name} cell-updates/s"), "value": value,
        "unit": getattr(W, "unit", "Gcell-upd/s"),
        "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32" if W.name.endswith("32") else "f64",
        "data": "synthetic (seeded)",
        "config": {"workload": getattr(W, "label", f"{W.name} {args.n}^3 + 1 ghost"), "cells_per_step": W.cells,
                   "parallelism": f"replicas x{world}",
                   "l2": "inputs larger than L2 (129 MB); no flush between steps",
                   "timed_calls": ("the K steps in one library call" if hasattr(W, "run")
                                   else "one library call per step")},
        "e2e": {"value": e2e_value, "unit": getattr(W, "unit", "Gcell-upd/s"), "h2d_bytes_per_step": W.h2d_bytes,
                "d2h_bytes_per_step": W.d2h_bytes, "steps": e_steps,
                "copies": ("uploads on a copy stream into 2 alternating input sets, overlapping the previous "
                           "step's kernels" if hasattr(W, "e2e_begin") else "serial with the kernels")},
        "gpu_launches": int(launches),
        "roofline": roof,
        "cpu_baseline": cpu,
        "clocks": clocks,
    }
    line.update(extra)
    if W.name == "deep" and world == 1 and not args.no_parts:
        # the headline workload's buffers go first: the parts need the memory
        del W
        torch.cuda.empty_cache()
        line["metric_parts"] = metric_parts(N, bus if isinstance(bus, str) else None, peak)
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
