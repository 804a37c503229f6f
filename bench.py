"""Benchmark of the GB300 UPPE z-step: grid-pt*steps/s on the large Cartesian filament workload.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload cart_filament_256] [--precision mixed|fp32]

A "step" is one classic RK4 z-step (four right-hand-side evaluations) over the whole grid.
The default workload is the 1025 x 256 x 256 filament (256 x 256 over 3 mm, 800 nm 40 fs pulse at
10 critical powers, Kerr + O2 tunneling ionization + plasma current, 1000 fixed steps over 10 cm;
searay_gb300/workloads.py), the largest workload that fits one GPU.

value: P * K / (device time of K steps), fields resident in HBM, CUDA events on the library's stream.
e2e:   the same metric through the reference-facing call searay_gb300.track() with host (NumPy)
       input and outputs, one call over the workload's whole propagation (its own step count,
       --e2e-steps to change it): grid and handle set-up, the host->device copy of the input plane,
       the steps and the device->host copies of every output inside the timed region; the input
       plane itself (the user's incoming-wave function on the grid) is evaluated before it.
roofline: the kernel class with the largest share of the step, algorithmic bytes per launch over its
       average event-timed duration, against the measured HBM copy bandwidth.
cpu_baseline: the FP64 NumPy oracle (a restatement of the reference path) timed on the host cores:
       its first RK4 step on the same grid (on the 128 x 128 sub-grid for larger Cartesian slices),
       repeated until about 10 s of CPU work.
fwd_adjoint: a forward step that keeps its stage fields plus the vector-Jacobian product of that step
       (uppe_rk4_step_keep + uppe_adjoint_rk4_step_kept), timed together; "recompute" beside it is a
       plain forward step plus the VJP that recomputes the stage states.
fp32:  the same forward and forward+adjoint rates in the plain FP32 form (FP32 phase and density
       sum, SIMT Hankel transforms on cylindrical grids) beside the mixed form of the main line.
err_vs_fp64: both forms' first RK4 step (with the finish: A, J, chi, n_e) against the FP64 oracle's
       on the grid the cpu_baseline leg times (the full grid, or its 128 x 128 sub-grid for larger
       Cartesian slices): max |x - x_ref| / max |x_ref| of the field, its fluence (sum over w of
       |A|^2 per transverse point), its spectrum (sum over the transverse points of |A|^2 per w),
       J, chi and n_e.
kernels: per-class event-timed averages over a replay of the timed steps from the incoming plane.
--impl reference: the reference arm.  The reference (SeaRay) runs through PyOpenCL, which is not
       available on the GPU machine; its CPU path is timed as the oracle port, one bounded RK4 step
       per bench step.
Multi-GPU (torchrun): the path does not shard; every rank runs an independent replica and value is
the sum over ranks divided by the slowest rank's time.
"""
import argparse
import json
import os
import pathlib
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "UPPE grid-pt*steps/s (RK4 z-step)"
UNIT = "grid-pt*steps/s"
# Algorithmic work per launch of each kernel class.  Complex64 fields, 8-byte per-point operator
# K = Re kz + kg (float-float).
# Cartesian grids (bytes per grid point):
#   transverse_inverse: read q, K; write E
#   time_pass: read E; write J
#   transverse_forward_rk (fused slice pass): read J, K, qi and/or qf; write qf or qi; write E for
#   the next evaluation -- 40 / 48 / 48 / 40 bytes for the four RK stages.  The slices at and above
#   the nonlinear cut carry no current (S = 0): there stage 1 reads qi and K and writes qf and E
#   (32 bytes), stage 3 reads qi and K and writes E (24 bytes), and stage 2 and the finish have
#   nothing to do (their q and E are unchanged); see cart_forward_bytes.
CART_BYTES = {
    "transverse_inverse": 8 + 8 + 8,
    "time_pass": 8 + 8,
    "transverse_forward_rk": (40 + 48 + 48 + 40) / 4.0,
}
# Cylindrical grids: the transverse classes are the Hankel GEMMs (complex x real, 4 flops per
# multiply-add): inverse M=N0 rows, N=Nr, K=Nk; forward N=Nr, K=Nr.  Bytes per point as above with
# the RK epilogue of the forward pass writing q and qf (40 / 48 / 48 / 32).
CYL_BYTES = {
    "transverse_inverse": 8 + 8 + 8,
    "time_pass": 8 + 8,
    "transverse_forward_rk": (40 + 48 + 48 + 32) / 4.0,
}


def cart_forward_bytes(vd):
    """Average bytes per grid point of the Cartesian fused evaluation tail over the four RK stages,
    with the slices without current (w >= nonlinear cut, the cut index of the library's
    configuration) counted at what they need: 32 / 0 / 24 / 0 bytes."""
    from searay_gb300.grid import VolumeGrid
    N = vd["wave grid"]
    nl = vd.get("nonlinear band", vd["frequency band"])
    dw = VolumeGrid(vd).dw  # the cut indices of searay_gb300.uppe.DeviceGrid
    jhi = int(nl[1] / dw)
    if is_paraxial(vd) or int(nl[0] / dw) > 0 or not (4 <= jhi < N[0]):
        return CART_BYTES["transverse_forward_rk"]
    f = (N[0] - jhi) / N[0]
    return (1 - f) * CART_BYTES["transverse_forward_rk"] + f * (32 + 0 + 24 + 0) / 4.0


def class_models(vd):
    """{class: {"bytes": B per launch, "flops": F per launch (transverse GEMMs only)}}"""
    N = vd["wave grid"]
    P = N[0] * N[1] * N[2]
    if vd["wave coordinates"] == "cartesian":
        m = {k: {"bytes": b * P} for k, b in CART_BYTES.items()}
        m["transverse_forward_rk"]["bytes"] = cart_forward_bytes(vd) * P
        return m
    Nr, Nk = N[1], vd.get("radial modes", N[1])
    m = {k: {"bytes": b * P} for k, b in CYL_BYTES.items()}
    m["transverse_inverse"]["flops"] = 4.0 * N[0] * N[2] * Nr * Nk
    m["transverse_forward_rk"]["flops"] = 4.0 * N[0] * N[2] * Nr * Nr
    return m


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        time.sleep(0.15)
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in out.strip().splitlines():
            p = [x.strip() for x in line.split(",")]
            if len(p) < 8:
                continue
            try:
                sm.append(float(p[0]))
                smax.append(float(p[1]))
            except ValueError:
                continue
            for n, v in zip(names, p[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    """(HBM GB/s, bf16 dense TFLOP/s burst, source)"""
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


def ncu_traffic(workload):
    """Per-launch DRAM bytes per kernel class from the committed ncu summary, if any."""
    p = ROOT / "profiles" / f"traffic_{workload}.json"
    if p.exists():
        return json.loads(p.read_text())
    return {}


def working_set_mb(vd):
    N = vd["wave grid"]
    P = N[0] * N[1] * N[2]
    return (6 * 8 + 8 + 4) * P / 1e6  # q, qi, qf, k1, E, J (complex64) + K (float2) + Im kz


def is_paraxial(vd):
    return vd.get("propagator", "uppe") == "paraxial"


def build_device(vd, precision):
    from searay_gb300 import grid, ionization, paraxial, uppe
    g = grid.VolumeGrid(vd)
    rates = ionization.RateCoefficients(vd["ionizer"]) if vd.get("ionizer") is not None else None
    env = is_paraxial(vd)
    dev = uppe.DeviceGrid(g, vd, rates, precision, envelope=env)
    dev.set_rotator(vd.get("rotator"))
    chi = vd["dispersion inside"].chi(g.w).astype(np.cdouble)
    if env:  # envelope frame of paraxial_kernel.py:407-411
        n = 1 / vd.get("window speed", 1.0)
        mat = paraxial.Material(dev, g, vd["wave coordinates"], None, chi, vd.get("chi3", 0.0),
                                vd["density reference"], g.w[g.N[0] // 2], n, n, vd["density lambda"])
    else:
        mat = uppe.Material(dev, g, vd["wave coordinates"], None, chi, vd.get("chi3", 0.0), vd["density reference"],
                            vd.get("window speed", 1.0), vd["density lambda"])
    return g, dev, mat


def run_device(args, vd, ws, rank, local, precision, per_class=True):
    import torch
    g, dev, mat = build_device(vd, precision)
    P = int(np.prod(g.N[:3]))
    Lz = vd["size"][2]
    nsteps_cfg = vd["subcycles"]
    dz = Lz / nsteps_cfg
    a = vd["incoming wave"](g.w, g.x1, g.x2)
    if is_paraxial(vd):
        a = np.fft.ifftshift(a, axes=0)  # the envelope solver keeps the frequency axis in FFT order
    a_dev = torch.from_numpy(np.ascontiguousarray(a, dtype=np.complex64)).cuda()
    mat.UpdateMaterial(-Lz / 2 + 0.5 * dz)
    dev.load_field(a_dev)
    step = [0]

    def one_step():
        # fixed step: minimum step = subcycle length, so dz = L/steps exactly (uppe_kernel.py:224-227)
        dev.rk4_step(step[0] * dz, dz, 0.0, dz)
        step[0] += 1

    for _ in range(args.warmup):
        one_step()
    # the timed steps are the workload's own steps 0 .. K-1: back to the incoming plane
    dev.load_field(a_dev)
    step[0] = 0
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    l0 = dev.launches()
    stream = torch.cuda.current_stream()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t0.record(stream)
    for _ in range(args.steps):
        one_step()
    t1.record(stream)
    torch.cuda.synchronize()
    ms = t0.elapsed_time(t1)
    launches = dev.launches() - l0
    if ws > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    finite = not dev.nonfinite()
    # forward + adjoint: K_a vector-Jacobian products of the RK4 step (each recomputes its stage
    # states from the step's input, as the checkpointed backward pass does)
    adj = None
    # the adjoint has no envelope form
    if args.adjoint_steps > 0 and not is_paraxial(vd):
        q = dev.empty_field()
        dev.get_field(q)
        gen = torch.Generator(device="cuda").manual_seed(0)
        lam = torch.randn(q.shape, dtype=torch.complex64, device="cuda", generator=gen)
        out = dev.empty_field()
        for _ in range(2):
            dev.adjoint_step(q, lam, out, step[0] * dz, dz, want_dchi3=False)
        torch.cuda.synchronize()
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        for i in range(args.adjoint_steps):
            dev.adjoint_step(q, lam, out, (step[0] + i) * dz, dz, want_dchi3=False)
            lam, out = out, lam
        a1.record(stream)
        torch.cuda.synchronize()
        adj_ms = a0.elapsed_time(a1) / args.adjoint_steps
        # a forward step that keeps its stage fields plus the VJP of that step from them, timed
        # together (the pair a training step runs)
        pair_ms = None
        dev.set_field(q)
        try:
            for i in range(2):
                dev.rk4_step_keep((step[0] + i) * dz, dz)
                dev.adjoint_step_kept(lam, out, want_dchi3=False)
        except RuntimeError:
            pass
        else:
            torch.cuda.synchronize()
            a0.record(stream)
            for i in range(args.adjoint_steps):
                dev.rk4_step_keep((step[0] + 2 + i) * dz, dz)
                dev.adjoint_step_kept(lam, out, want_dchi3=False)
                lam, out = out, lam
            a1.record(stream)
            torch.cuda.synchronize()
            pair_ms = a0.elapsed_time(a1) / args.adjoint_steps
        adj = (adj_ms, pair_ms)
    # per-kernel-class timing: the timed steps again from the incoming plane (separate region; event
    # records between launches), so that the per-class averages describe the same work
    prof = None
    if per_class:
        dev.load_field(a_dev)
        step[0] = 0
        dev.profile(True)
        for _ in range(args.steps):
            one_step()
        prof = dev.profile_read()
        dev.profile(False)
    dev.close()
    return P, ms, launches, clk, prof, finite, adj


def run_e2e(args, vd, precision):
    """One track() call with host input/outputs over n steps (one diagnostic interval): the
    workload's whole propagation (its own step count) unless --e2e-steps says otherwise.  Returns
    (rate, h2d bytes, d2h bytes, finite, n)."""
    import torch
    from searay_gb300 import paraxial, uppe
    solver = paraxial if is_paraxial(vd) else uppe
    Lz = vd["size"][2]
    dz = Lz / vd["subcycles"]
    n = args.e2e_steps if args.e2e_steps else vd["subcycles"]
    v = dict(vd)
    v["size"] = (vd["size"][0], vd["size"][1], dz * n)
    v["subcycles"] = n
    v["minimum step"] = dz
    v["precision"] = precision
    # the input plane is the user's data: evaluated on the host before the timed region, handed to
    # track() as the incoming wave (its host->device copy and everything after it are timed)
    from searay_gb300 import grid as grid_mod
    g = grid_mod.VolumeGrid(v)
    first = np.ascontiguousarray(vd["incoming wave"](g.w, g.x1, g.x2), dtype=np.complex128)
    v["incoming wave"] = lambda w, x1, x2: first
    warm = dict(v)
    warm["size"] = (vd["size"][0], vd["size"][1], dz * 2)
    warm["subcycles"] = 2
    solver.track(None, None, None, None, warm)
    torch.cuda.synchronize()
    t = time.perf_counter()
    A, J, chi, ne, dom = solver.track(None, None, None, None, v)
    wall = time.perf_counter() - t
    N = v["wave grid"]
    P = int(np.prod(N[:3]))
    # the incoming plane (complex128) and the material tables in; the four complex128 result arrays
    # (every diagnostic plane) out
    h2d = P * 16 + (2 * N[0] + N[0]) * 8 + N[1] * N[2] * 8
    d2h = 4 * P * N[3] * 16
    return P * n / wall, h2d, d2h, bool(np.isfinite(A[..., -1]).all()), n


def aggregate_replicas(ms, points, steps, ws, device):
    """Whole-job rate of N independent replicas (one per rank, no collective on the data path): the
    points*steps of all ranks over the slowest rank's time, taken as the MAX over ranks of ms.
    Returns (rate, ms)."""
    import torch
    if ws > 1:
        t = torch.tensor([ms], device=device, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    return points * steps * ws / (ms / 1e3), ms


def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def oracle_step_time(vd, n_perp=None):
    """Seconds for one FP64 oracle RK4 step (four RHS evaluations + stage arithmetic)."""
    t, _, P, N, _ = oracle_run(sample_volume(vd, n_perp))
    return t, P, N


def sample_volume(vd, n_perp=None):
    """The volume itself, or its n_perp x n_perp (n_perp radial nodes) sub-grid with the box scaled."""
    v = dict(vd)
    if n_perp is not None and n_perp != v["wave grid"][1]:
        N = v["wave grid"]
        f = n_perp / N[1]
        v["wave grid"] = (N[0], n_perp, n_perp if N[2] > 1 else 1, N[3])
        v["size"] = (v["size"][0] * f, v["size"][1] * (f if N[2] > 1 else 1), v["size"][2])
        if v.get("radial modes") is not None:  # keep the same fraction of the radial nodes
            v["radial modes"] = max(1, min(n_perp, int(round(v["radial modes"] * f))))
    return v


def oracle_run(v, min_seconds=0.0, max_steps=1, outputs=False):
    """The FP64 oracle's first RK4 step from the incoming plane on the volume ``v``, repeated until
    ``min_seconds`` of step time or ``max_steps`` steps; returns (seconds, steps, points, grid,
    outputs).  Set-up is not timed.  Every repeat starts again from the incoming plane, so each does
    the same work and stays finite (a collapsing beam overflows after some tens of steps).  With
    ``outputs`` the first step's finish (A, J, chi, n_e, as the oracle's propagator returns them for
    one fixed step) is computed after the timed work; otherwise ``outputs`` is None."""
    from oracle import paraxial_oracle as PO
    from oracle import uppe_oracle as O
    O.set_workers(cpu_cores())
    env = is_paraxial(v)
    orc = PO.ParaxialOracle(v) if env else O.Oracle(v)
    g = orc.g
    dz = v["size"][2] / v["subcycles"]
    orc.mat.update(0.5 * dz)  # the medium at the middle of the first subcycle, as the propagator samples it
    a = v["incoming wave"](g.w, g.x1, g.x2)
    q = g.kspace(np.fft.ifftshift(a, axes=0) if env else a)
    cond = 1.0 if env else orc.conditioner[:, None, None]
    tot, steps, q1 = 0.0, 0, None
    while steps < max(1, max_steps) and (steps == 0 or tot < min_seconds):
        t = time.perf_counter()
        k1 = orc.load_source(q, 0.0)
        qf = q + dz / 6 * k1
        qw = (q + dz / 2 * k1) * cond
        k2 = orc.load_source(qw, dz / 2)
        qf = qf + dz / 3 * k2
        qw = (q + dz / 2 * k2) * cond
        k3 = orc.load_source(qw, dz / 2)
        qf = qf + dz / 3 * k3
        qw = (q + dz * k3) * cond
        k4 = orc.load_source(qw, dz)
        q = (qf + dz / 6 * k4) * cond  # the step's result
        tot += time.perf_counter() - t
        steps += 1
        if q1 is None:
            q1 = q
    out = None
    if outputs:
        if env:  # the envelope solver's step is adaptive (no minimum step): its own propagator, ascending w
            out = orc.propagator(a, 0.0, dz, 1)[:4]
        else:
            out = orc.finish(q1, dz)
    return tot, steps, int(np.prod(g.N[:3])), g.N, out


def cpu_sample(vd):
    """The volume the CPU baseline times: the full grid, or its 128 x 128 sub-grid (same physics, box
    scaled) for larger Cartesian slices."""
    N = vd["wave grid"]
    n_perp = 128 if N[1] * N[2] > 128 * 128 and N[2] > 1 else None
    return sample_volume(vd, n_perp), n_perp is None


def cpu_baseline(vd, min_seconds=10.0, max_steps=200, outputs=False):
    """The FP64 oracle's rate on a bounded sample of the workload (cpu_sample), repeated until about
    ``min_seconds`` of CPU work.  Returns (baseline entry, sample volume, first-step outputs)."""
    N = vd["wave grid"]
    v, full = cpu_sample(vd)
    t, steps, P, Ns, out = oracle_run(v, min_seconds, max_steps, outputs)
    grid = f"{Ns[0]}x{Ns[1]}x{Ns[2]}"
    where = (f"the full {grid} grid" if full else
             f"a {grid} sub-grid (box scaled) of the {N[0]}x{N[1]}x{N[2]} grid")
    return ({"value": P * steps / t, "unit": UNIT, "cores": cpu_cores(), "kind": "port",
             "sample": f"{steps} FP64 oracle RK4 step(s) on {where} ({t:.1f} s)"}, v, out)


def field_metrics(A, J, chi, ne, ref):
    """Errors of one step's outputs against the oracle's: max |x - x_ref| / max |x_ref| of A, J, chi,
    n_e, and of the fluence (sum over w of |A|^2) and the spectrum (sum over x, y of |A|^2)."""
    def rel(x, r):
        s = np.max(np.abs(r))
        return float(np.max(np.abs(x - r)) / s) if s > 0 else float(np.max(np.abs(x)))

    def power(x):
        return x.real.astype(np.float64) ** 2 + x.imag.astype(np.float64) ** 2

    A_ref, J_ref, chi_ref, ne_ref = ref
    pA, pR = power(A), power(A_ref)
    return {"field": rel(A, A_ref), "fluence": rel(pA.sum(axis=0), pR.sum(axis=0)),
            "spectrum": rel(pA.sum(axis=(1, 2)), pR.sum(axis=(1, 2))), "J": rel(J, J_ref),
            "chi": rel(chi, chi_ref), "ne": rel(ne, ne_ref)}


def gpu_first_step_errors(v, ref, precision):
    """One fixed RK4 step with the finish on the device, on the sample volume v, against ref."""
    import torch
    from searay_gb300 import paraxial, uppe
    g, dev, mat = build_device(v, precision)
    try:
        dz = v["size"][2] / v["subcycles"]
        a = v["incoming wave"](g.w, g.x1, g.x2)
        if is_paraxial(v):
            a_dev = torch.from_numpy(np.ascontiguousarray(np.fft.ifftshift(a, axes=0), dtype=np.complex64)).cuda()
            out = paraxial.propagator(dev, mat, a_dev, 1, 0.0, dz)[:4]
            host = [np.fft.fftshift(t.cpu().numpy(), axes=0) for t in out]
        else:
            a_dev = torch.from_numpy(np.ascontiguousarray(a, dtype=np.complex64)).cuda()
            out = uppe.propagator(dev, mat, a_dev, 1, 0.0, dz, dz)[:4]
            host = [t.cpu().numpy() for t in out]
    finally:
        dev.close()
    return field_metrics(*host, ref)


def reduced_volume(vd, n_perp=None, n0=None):
    """The workload on its n_perp x n_perp sub-grid (sample_volume) and/or with n0 frequency nodes at
    the same spacing (the band and the nonlinear band scaled by (n0 - 1) / (N0 - 1)); unchanged when
    both are None.  Small cases of the same kernels for profiling."""
    v = sample_volume(vd, n_perp)
    N = v["wave grid"]
    if n0 is not None and n0 != N[0]:
        f = (n0 - 1) / (N[0] - 1)
        v["wave grid"] = (n0,) + tuple(N[1:])
        v["frequency band"] = (v["frequency band"][0] * f, v["frequency band"][1] * f)
        if "nonlinear band" in v:
            v["nonlinear band"] = (v["nonlinear band"][0] * f, v["nonlinear band"][1] * f)
    return v


def config_of(args, vd, ws):
    """The workload description shared by both arms' lines (marked when reduced for profiling)."""
    c = {"workload": args.workload, "grid": list(vd["wave grid"][:3]), "propagator": vd.get("propagator", "uppe"),
         "parallelism": "replicas" if ws > 1 else "single",
         "l2": f"working set ({working_set_mb(vd):.0f} MB of fields and operator) vs the 129 MB L2"}
    if getattr(args, "n_perp", None) is not None or getattr(args, "n0", None) is not None:
        c["reduced"] = "sub-grid of the workload (--n-perp / --n0): a profiling case, not the workload"
    return c


def reference_arm(args, vd, ws, rank):
    if rank != 0:
        return
    # size the per-step sample so the whole run stays within a few minutes
    budget = 150.0
    chosen = None
    # the full transverse grid where it has at most 128 points per axis, else sub-grids of it
    n_full = vd["wave grid"][1]
    sizes = ([n_full] if n_full <= 128 else []) + [n for n in (128, 64, 32, 16, 8) if n < n_full]
    for n in sizes:
        t, P, N = oracle_step_time(vd, n)
        chosen = (n, t, P, N)
        if t * (args.steps + args.warmup) <= budget:
            break
    n, _, P, N = chosen
    for _ in range(max(0, args.warmup - 1)):
        oracle_step_time(vd, n)
    tot = 0.0
    for _ in range(args.steps):
        t, P, N = oracle_step_time(vd, n)
        tot += t
    value = P * args.steps / tot
    cores = cpu_cores()
    full = list(N[:3]) == list(vd["wave grid"][:3])
    sample = (f"one FP64 RK4 step per bench step on the full {N[0]}x{N[1]}x{N[2]} grid" if full else
              f"one FP64 RK4 step per bench step on a {N[0]}x{N[1]}x{N[2]} sub-grid of the workload "
              "(same physics, box scaled)")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_of(args, vd, ws), "sample_grid": list(N[:3]),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "SeaRay's UPPE path needs PyOpenCL + an OpenCL runtime, absent on the GPU machine; its CPU path is "
                "timed as the FP64 oracle port (pinned to the reference's own outputs at 1e-12).",
    }
    print(json.dumps(line))


def fwd_adjoint_entry(P, ws, fwd_ms, adj):
    """The forward+adjoint rate: the kept-stage pair where it ran, else forward + recomputing VJP."""
    adj_ms, pair_ms = adj
    recompute = {"value": P * ws / ((fwd_ms + adj_ms) / 1e3), "unit": UNIT, "adjoint_ms_per_step": adj_ms,
                 "forward_ms_per_step": fwd_ms,
                 "note": "one forward step plus one vector-Jacobian product of the step; the VJP "
                         "recomputes the step's stage states (checkpointed backward pass)"}
    if pair_ms is None:
        return recompute
    return {"value": P * ws / (pair_ms / 1e3), "unit": UNIT, "ms_per_step": pair_ms,
            "note": "one forward step that keeps its stage fields (rk4_step_keep) and the "
                    "vector-Jacobian product of that step from them (adjoint_step_kept), timed together",
            "recompute": recompute}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cart_filament_256")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp32"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=None,
                    help="steps of the e2e track() call (default: the workload's whole propagation)")
    ap.add_argument("--no-fp32", action="store_true", help="skip the plain FP32 companion rates")
    ap.add_argument("--adjoint-steps", type=int, default=20,
                    help="adjoint (VJP) steps timed for the forward+adjoint rate; 0 to skip")
    ap.add_argument("--n-perp", type=int, default=None,
                    help="run the workload on its n x n transverse sub-grid (box scaled): small cases for profiling")
    ap.add_argument("--n0", type=int, default=None,
                    help="run the workload with n0 = 2^k + 1 frequencies at the same spacing: small cases for profiling")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    from searay_gb300 import workloads
    vd = reduced_volume(workloads.WORKLOADS[args.workload](), args.n_perp, args.n0)
    ws, rank, local = dist_env()
    if args.impl == "reference":
        reference_arm(args, vd, ws, rank)
        return
    import torch
    if ws > 1:
        torch.cuda.set_device(local)
        torch.distributed.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    P, ms, launches, clk, prof, finite, adj = run_device(args, vd, ws, rank, local, args.precision)
    value, ms = aggregate_replicas(ms, P, args.steps, ws, "cuda")
    peak, tpeak, peak_kind = measured_peaks()
    models = class_models(vd)
    tensor_path = vd["wave coordinates"] != "cartesian" and args.precision == "mixed"
    kernels = {}
    for name, (tms, cnt) in prof.items():
        if cnt == 0:
            continue
        entry = {"launch_regions": cnt, "total_ms": tms, "avg_us": 1e3 * tms / cnt}
        if name in models:
            sec = tms / cnt / 1e3
            gbs = models[name]["bytes"] / sec / 1e9
            entry.update({"algo_bytes_per_launch": models[name]["bytes"], "achieved_GBs": gbs, "frac": gbs / peak})
            if "flops" in models[name]:
                tf = models[name]["flops"] / sec / 1e12
                entry.update({"algo_flops_per_launch": models[name]["flops"], "achieved_TFLOPs": tf,
                              "tensor_frac": tf / tpeak if tensor_path else None})
        kernels[name] = entry
    rot = vd.get("rotator")
    if rot is not None and "time_pass" in kernels:
        # the Raman part of the time pass is FP32 arithmetic: per sample and transition 17 flops
        # (pass 1: F h^{2i} into the segment sum, 4; pass 2: u + F rho, u conj(h2), rho |h2|^2 and
        # Im(cq u) into the sample's sum, 13); peak = 2 flops x 128 lanes x SMs x the median SM clock
        N = vd["wave grid"]
        ntr = int(np.count_nonzero(np.asarray(rot.Tj)[2:]))
        Nt = N[0] if is_paraxial(vd) else 2 * N[0] - 2
        flops = 17.0 * Nt * N[1] * N[2] * ntr
        sec = kernels["time_pass"]["avg_us"] / 1e6
        nsm = torch.cuda.get_device_properties(0).multi_processor_count
        fp32_peak = 2 * 128 * nsm * (clk.get("sm_mhz") or 1900) * 1e6 / 1e12
        kernels["time_pass"]["raman"] = {"transitions": ntr, "algo_flops_per_launch": flops,
                                         "achieved_TFLOPs": flops / sec / 1e12, "fp32_peak_TFLOPs": fp32_peak,
                                         "fp32_frac": flops / sec / 1e12 / fp32_peak,
                                         "note": "FP32 peak from the SM count and the median SM clock under load"}
    dom = max((k for k in kernels if k in models), key=lambda k: kernels[k]["total_ms"])
    traffic_rec = ncu_traffic(args.workload)
    traffic = traffic_rec.get(dom)
    traffic_source = (f"profiles/traffic_{args.workload}.json: {traffic_rec.get('source', 'ncu capture')}"
                      if traffic is not None else None)
    share = kernels[dom]["total_ms"] / sum(v["total_ms"] for v in kernels.values())
    if tensor_path and "achieved_TFLOPs" in kernels[dom]:
        roof = {"bound": "tensor", "kernel": dom, "achieved": kernels[dom]["achieved_TFLOPs"], "peak": tpeak,
                "unit": "TFLOP/s", "frac": kernels[dom]["tensor_frac"], "traffic": traffic,
                "traffic_source": traffic_source, "peak_source": peak_kind, "share": share,
                "hbm_frac": kernels[dom]["frac"],
                "note": "algorithmic flops; the split-BF16x3 tensor path executes 3x as many"}
    else:
        roof = {"bound": "hbm", "kernel": dom, "achieved": kernels[dom]["achieved_GBs"], "peak": peak, "unit": "GB/s",
                "frac": kernels[dom]["frac"], "traffic": traffic, "traffic_source": traffic_source,
                "peak_source": peak_kind, "share": share}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (float-float phase and density scan)" if args.precision == "mixed" else "f32",
        "data": "synthetic", "precision": args.precision,
        "config": config_of(args, vd, ws),
        "roofline": roof, "kernels": kernels, "gpu_launches": launches, "clocks": clk, "finite": finite,
    }
    if adj is not None:
        line["fwd_adjoint"] = fwd_adjoint_entry(P, ws, ms / args.steps, adj)
    other = "fp32" if args.precision == "mixed" else "mixed"
    if not args.no_fp32:
        # the other precision form on the same workload: forward and forward+adjoint rates
        P2, ms2, _, _, _, finite2, adj2 = run_device(args, vd, ws, rank, local, other, per_class=False)
        value2, ms2 = aggregate_replicas(ms2, P2, args.steps, ws, "cuda")
        comp = {"value": value2, "unit": UNIT, "ms_per_step": ms2 / args.steps, "finite": finite2,
                "mixed_over_fp32": value / value2 if other == "fp32" else value2 / value}
        if adj2 is not None:
            comp["fwd_adjoint"] = fwd_adjoint_entry(P2, ws, ms2 / args.steps, adj2)
        line[other] = comp
    if rank == 0 and not args.no_e2e:
        e2e, h2d, d2h, ok, n_e2e = run_e2e(args, vd, args.precision)
        line["e2e"] = {"value": e2e * ws, "unit": UNIT, "h2d_bytes_per_step": h2d / n_e2e,
                       "d2h_bytes_per_step": d2h / n_e2e, "steps": n_e2e,
                       "call": "searay_gb300.track (host NumPy in/out), one call over the steps"}
    if rank == 0 and not args.no_cpu_baseline and ws == 1:
        base, v_sample, ref = cpu_baseline(vd, outputs=True)
        line["cpu_baseline"] = base
        # both forms' first step on the sampled grid against the oracle's (set-up outside any timing)
        errs = {p: gpu_first_step_errors(v_sample, ref, p) for p in ("mixed", "fp32")}
        line["err_vs_fp64"] = {"grid": list(v_sample["wave grid"][:3]), "steps": 1, **errs,
                               "metric": "max |x - x_ref| / max |x_ref| after one fixed RK4 step and the finish; "
                                         "fluence = sum over w of |A|^2, spectrum = sum over x, y of |A|^2",
                               "bounds": {"fp32 transforms": 1e-5, "tensor-core transforms": 1e-4}}
        if other in line:
            line[other]["err_vs_fp64"] = errs[other]
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
