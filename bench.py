#!/usr/bin/env python3
"""Benchmark: LSS segment-steps per second on a GB300.

Workload (the batched least-squares-shadowing configuration): 64 segments of
a 32x65x32 channel (Nx x Ny x Nz; 2pi x 2 x pi box, Re 3300, dt 0.005, FP64).
One segment-step is one RK3 time step of the primal, two homogeneous
tangents, one mean-flux-forced tangent (all advanced together) and one
adjoint coupled to the forced tangent with strength 1 (the LSS backward
solve).  A timed "step" advances every segment by one segment-step: the
timed region is a forward sweep of K steps followed by the adjoint sweep of
the same K steps back, exactly the per-segment work of one LSS matvec.

Segment initial states: a seeded synthetic state (laminar profile plus
low-mode noise) run up for 200 steps, plus independent seeded 1e-3
perturbations per segment.  The working set (trajectories of 64 segments,
physical-space fields) is several GB, far larger than the 126 MB L2, so no
L2 flush is needed between steps.

Prints one JSON line.  ``--impl reference`` times the reference algorithm
on the host cores instead (the C restatement in oracle/, one segment per
process, all cores).
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "shadow-channel_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))

GRID = dict(Nx=32, Ny=65, Nz=32, Lx=2 * math.pi, Lz=math.pi, Re=3300.0, flux=2.0, dt=0.005)
NSEG, NTAN, COUPLE = 64, 3, 2
INHOMO = [0, 0, 1]
RUNUP = 200
METRIC = "steps/s fwd+tangent+adjoint, 64 segs 32x32x65 FP64: batched vs plain GPU"
UNIT = "segment-steps/s"
CONFIG = {"workload": "64 LSS segments, 32x65x32 channel (Nx x Ny x Nz), Re 3300, dt 0.005; per segment-step "
                      "1 primal + 2 homogeneous + 1 mean-flux tangent + 1 adjoint (strength 1)",
          "segments": NSEG, "tangents_per_segment": NTAN, "grid": "32x65x32", "dtype": "f64",
          "l2": "working set several GB > 126 MB L2 (no flush needed)"}


def args_parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="run none of the extra measurements (the default runs none either)")
    ap.add_argument("--extras", default="",
                    help="comma list of extra measurements, printed on a second JSON line: exact, uneven, "
                         "large, large5000, grad (default: none)")
    ap.add_argument("--segments", type=int, default=NSEG,
                    help="segments per GPU (default 64; smaller only for profiling captures)")
    ap.add_argument("--runup", type=int, default=RUNUP,
                    help="run-up steps of the parent field (default 200; 0 only for profiling captures)")
    return ap.parse_args()


def emit(line):
    """Print the result as one JSON line of its own: the library (and the
    oracle) write the reference's banners through C stdio, whose buffer is
    flushed first so that no banner text lands on the JSON line."""
    import ctypes
    sys.stdout.flush()
    try:
        ctypes.CDLL(None).fflush(None)
    except (OSError, AttributeError):
        pass
    sys.stdout.write("\n" + json.dumps(line) + "\n")
    sys.stdout.flush()


def grid_args(nsteps):
    g = GRID
    return (g["Nx"], g["Ny"], g["Nz"], g["Lx"], g["Lz"], g["Re"], g["flux"], g["dt"], nsteps)


def segment_states(C_parent, nseg, seed0=1000, amp=1e-3):
    from channel.synthetic import synthetic_state
    g = GRID
    out = np.empty((nseg,) + C_parent.shape, np.complex128)
    for s in range(nseg):
        pert = synthetic_state(g["Nx"], g["Ny"], g["Nz"], seed=seed0 + s, amp=amp, laminar=False)
        out[s] = C_parent + pert
    return out


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
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
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# algorithmic FP64 work (flop, FMA = 2) of the dominant kernels, per launch
# ---------------------------------------------------------------------------

def fft_flops(n):
    return 5.0 * n * math.log2(n)


def phys_inverse_flops(ninst, g, nfields=6):
    """z inverse FFTs of Nx/2 columns plus x inverse FFTs of the row pairs,
    per plane and field (5 N log2 N per complex transform)."""
    Nx, Ny, Nz = g["Nx"], g["Ny"], g["Nz"]
    X, Q, pz, px = Nx // 2, 3 * Ny // 2, 3 * Nz // 2, 3 * Nx // 2
    per_plane = X * fft_flops(pz) + ((pz + 1) // 2) * fft_flops(px)
    return ninst * nfields * Q * per_plane


def segment_step_flops(g):
    """Nominal FP64 flop of one segment-step (primal + 3 tangents + adjoint,
    3 substages): per field and substage the Legendre quadrature
    4 Q (5D + 3R) Nz X (2 right-hand-side + 5 reconstruction contractions of
    a real matrix with complex vectors) and 9 plane transforms (6 inverse + 3
    forward) of X 5 pz log2 pz + pz 2.5 px log2 px each; the adjoint counts
    1.5 quadratures and 15 transforms (9 inverse + 6 forward)."""
    Nx, Ny, Nz = g["Nx"], g["Ny"], g["Nz"]
    X, Q, R, D, pz, px = Nx // 2, 3 * Ny // 2, Ny - 2, Ny - 4, 3 * Nz // 2, 3 * Nx // 2
    quad = 4.0 * Q * (5 * D + 3 * R) * Nz * X
    plane = X * 5 * pz * math.log2(pz) + pz * 2.5 * px * math.log2(px)
    return 3 * ((1 + NTAN) * (quad + 9 * Q * plane) + (1.5 * quad + 15 * Q * plane))


# ncu DRAM bytes (read + write) of one instance of a 24-instance launch at
# 32x65x32 (traffic grows with the instance count; the ncu capture of the
# 8-segment bench case): k_phys_inverse_tc 306.1 MB (97.0 read + 209.1
# write), k_products_tc tangent mode 458.3 MB (411.7 + 46.7; two product
# planes per pass, the third product's fields loaded again)
PHYS_TRAFFIC_PER_INSTANCE_32 = 306.1e6 / 24
PROD_TRAFFIC_PER_INSTANCE_32 = 458.3e6 / 24


def products_fwd_flops(ninst, g):
    """Tangent products and their forward transforms per plane: 3 components
    of u' x w + u x w' (4 multiplies, 3 adds per point) and 3 forward 2D
    transforms (the inverse's nominal FFT flop)."""
    Nx, Ny, Nz = g["Nx"], g["Ny"], g["Nz"]
    Q, pz, px = 3 * Ny // 2, 3 * Nz // 2, 3 * Nx // 2
    return ninst * 3 * Q * 7.0 * pz * px + phys_inverse_flops(ninst, g, nfields=3)


def tc_inverse_mma_flops(ninst, g, nfields=6):
    """bf16 tensor-core flop of one k_phys_inverse_tc launch: per pair of
    fields the radix-2 z-stage GEMM (pz rows x 2 (Nz-1) x 2X, the even and
    odd modes' k-tiles) and x-stage GEMM (px/2 rows x 2X x 2 pz) in m16n8k16
    tiles, each tile 28 digit-pair MMAs."""
    X, Nz = g["Nx"] // 2, g["Nz"]
    pz, px, Q = 3 * Nz // 2, 3 * g["Nx"] // 2, 3 * g["Ny"] // 2
    t = lambda n, d: (n + d - 1) // d
    h = Nz // 2
    nzE, nzO = ((Nz - 1, 0) if pz % 2 else ((h + 1) // 2 + (h - 1) // 2, h // 2 + h // 2))
    ktz = t(2 * nzE, 16) + t(2 * nzO, 16)
    ktx = t(2 * ((X + 1) // 2), 16) + t(2 * (X // 2), 16)
    pzh = pz // 2 if pz % 2 == 0 else pz
    per_pair = 28 * (t(2 * pzh, 16) * ktz * t(2 * X, 8) + t(px // 2, 16) * ktx * t(2 * pz, 8))
    return ninst * Q * t(nfields, 2) * per_pair * 4096.0


def tc_products_mma_flops(ninst, g, ncomp=3):
    """bf16 tensor-core flop of one k_products_tc launch: per component an
    x-stage GEMM (2X x px x pz) and a z-stage GEMM (2 (Nz-1) x 2 pz x X) in
    m16n8k16 tiles of 28 digit-pair MMAs."""
    X, Nz = g["Nx"] // 2, g["Nz"]
    pz, px, Q = 3 * Nz // 2, 3 * g["Nx"] // 2, 3 * g["Ny"] // 2
    t = lambda n, d: (n + d - 1) // d
    per = 28 * (t(2 * X, 16) * t(px, 16) * t(pz, 8) + t(2 * (Nz - 1), 16) * t(2 * pz, 16) * t(X, 8))
    return ninst * Q * ncomp * per * 4096.0


def measured_bf16_peak():
    """bf16 dense TFLOP/s measured on the GB300s (MEASURED_PEAKS.json), else the fallback"""
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"]), "measured (MEASURED_PEAKS.json, cuBLAS bf16 burst)"
    except Exception:
        return 1900.0, "fallback 1.9 PFLOP/s"


def recon_flops(ninst, g):
    """Parity-split reconstruction: (3D + 2R) complex multiply-adds per plane
    pair and (kz, kx) mode, plus 24 flop of wavenumber algebra per point."""
    Nx, Ny, Nz = g["Nx"], g["Ny"], g["Nz"]
    X, Q, R, D = Nx // 2, 3 * Ny // 2, Ny - 2, Ny - 4
    Qh = (Q + 1) // 2
    modes = (Nz - 1) * X
    return ninst * modes * (Qh * (3 * D + 2 * R) * 4 + Q * 24)


# ---------------------------------------------------------------------------
# replicas (one process per GPU; segments never exchange data inside a sweep)
# ---------------------------------------------------------------------------

def max_over_replicas(ms, dist=None):
    """The timed region's duration across the replicas: every rank waits at
    a barrier after its own timed region, and the slowest rank's time is the
    job's (all-reduce MAX over the process group; the rank's own time
    without one)."""
    if dist is None:
        return float(ms)
    import torch
    dist.barrier()
    t = torch.tensor([float(ms)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(world, nseg, K, ms):
    """Whole-job segment-steps per second: every rank advances its own nseg
    segments by K steps (weak scaling) in the slowest rank's ms."""
    return world * nseg * K / (ms * 1e-3)


# ---------------------------------------------------------------------------
# the GB300 arm
# ---------------------------------------------------------------------------

def run_gb300(a):
    global NSEG
    NSEG = a.segments
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    from channel import c_channel as cc

    K, W = a.steps, max(3, a.warmup)
    nsteps = max(K, W)
    assert cc.c_init(*grid_args(nsteps)) == 0, cc.c_last_error_message()
    from channel.synthetic import synthetic_state
    C0 = synthetic_state(GRID["Nx"], GRID["Ny"], GRID["Nz"], seed=0)
    # parent field: run-up through the single-trajectory path (not timed)
    cc.c_destroy()
    assert cc.c_init(*grid_args(1)) == 0
    Cp = C0.copy()
    if a.runup > 0:
        cc.c_primal(a.runup, Cp)
    cc.c_destroy()
    assert cc.c_init(*grid_args(nsteps)) == 0
    Cseg = segment_states(Cp, NSEG)
    IC0 = np.stack([synthetic_state(GRID["Nx"], GRID["Ny"], GRID["Nz"], seed=2000 + i, laminar=False)
                    for i in range(NSEG * NTAN)])
    AC0 = np.stack([synthetic_state(GRID["Nx"], GRID["Ny"], GRID["Nz"], seed=5000 + i, laminar=False)
                    for i in range(NSEG)])
    assert cc.lib.c_batch_init(NSEG, NTAN, COUPLE) == 0, cc.c_last_error_message()
    inh = (ctypes_int_array(INHOMO))
    dev = torch.device("cuda", local)
    dC = torch.from_numpy(Cseg.view(np.float64)).to(dev)
    dIC = torch.from_numpy(IC0.view(np.float64)).to(dev)
    dAC = torch.from_numpy(AC0.view(np.float64)).to(dev)

    def sweep(k):
        rc = cc.lib.c_batch_forward_dev(0, k, dC.data_ptr(), dIC.data_ptr(), inh)
        assert rc == 0, (rc, cc.c_last_error_message())
        rc = cc.lib.c_batch_adjoint_dev(k, 0, dAC.data_ptr(), 1.0)
        assert rc == 0, (rc, cc.c_last_error_message())

    # warm-up (untimed)
    sweep(W)
    torch.cuda.synchronize()
    stream = torch.cuda.ExternalStream(cc.lib.c_stream(), device=dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = cc.c_launch_count()
    with ClockSampler(local) as clk:
        e0.record(stream)
        sweep(K)
        e1.record(stream)
        torch.cuda.synchronize()
    launches = cc.c_launch_count() - launches0
    ms = max_over_replicas(e0.elapsed_time(e1), dist)
    value = replica_value(world, NSEG, K, ms)

    # end to end through the host-array C ABI (H2D of the inputs and D2H of
    # the results inside the timed region), from pinned host buffers
    def pinned(arr):
        buf = torch.empty(arr.nbytes, dtype=torch.uint8, pin_memory=True)
        view = buf.numpy().view(arr.dtype).reshape(arr.shape)
        view[...] = arr
        return buf, view
    pins = [pinned(x) for x in (Cseg, IC0, AC0)]
    hC, hIC, hAC = (v for _, v in pins)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rc1 = cc.lib.c_batch_forward(0, K, hC.ctypes.data, hIC.ctypes.data, inh)
    rc2 = cc.lib.c_batch_adjoint(K, 0, hAC.ctypes.data, 1.0)
    cc.c_synchronize()
    e2e_s = time.perf_counter() - t0
    assert rc1 == 0 and rc2 == 0, cc.c_last_error_message()
    bytes_in = (hC.nbytes + hIC.nbytes + hAC.nbytes)
    e2e = {"value": NSEG * K / e2e_s, "unit": UNIT, "h2d_bytes_per_step": bytes_in // K,
           "d2h_bytes_per_step": bytes_in // K,
           "note": "the sweep entry points copy the segments' C, IC, AC in and out once per call; per-step "
                   "bytes are those copies divided by the K steps of the sweep"}

    # roofline of the dominant kernel: CUDA events on the library stream
    nt = NSEG * NTAN
    k_ms = {name: cc.lib.c_batch_kernel_ms(i, 5) for i, name in
            enumerate(["recon", "phys_inverse", "products_fwd", "solve", "products_adj"])}
    roofline = dominant_roofline(cc, k_ms, nt, value / world)
    autotune = json.loads(cc.lib.c_autotune_report().decode() or "{}")

    extras = set() if a.no_extras else {e.strip() for e in a.extras.split(",") if e.strip()}
    exact = None
    if "exact" in extras and rank == 0:
        exact = exact_adjoint_timing(cc, torch, stream, dAC, K)
    cc.lib.c_batch_destroy()
    cc.c_destroy()
    plain = None
    if not a.no_plain and rank == 0:
        plain = plain_gpu(cc, Cseg[0], IC0[:NTAN], AC0[0], K)

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic seeded states (no dataset; reference restart files absent)",
            "config": CONFIG}
    if plain:
        # the metric's headline: batched segment-steps/s over the plain
        # one-trajectory-per-launch path, both over the same K steps
        line["batched_over_plain"] = (value / world) / plain["value"]
        line["plain_gpu"] = plain
    line.update({"e2e": e2e, "roofline": roofline, "gpu_launches": launches, "clocks": clk.summary()})
    if rank == 0 and not a.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline()
    line["autotune"] = autotune
    extra = {}
    if exact:
        extra["exact_adjoint"] = exact
    if "uneven" in extras and rank == 0:
        extra["uneven_batch"] = uneven_batch(cc)
    if "large" in extras and rank == 0:
        extra["large_grid"] = large_grid(cc)
    if "large5000" in extras and rank == 0:
        extra["large_grid_5000"] = large_grid_horizon(cc)
    if "grad" in extras and rank == 0:
        extra["autograd_32x65x32"] = autograd_config(Cp)
    if rank == 0:
        emit(line)
        if extra:
            emit({"extras_of": METRIC, **extra})
    if dist:
        dist.destroy_process_group()


def products_fwd_bytes(ninst, g):
    """Algorithmic HBM bytes of one tangent-mode k_products_tc launch: each
    tangent's six physical fields in, the primal's six fields shared by the
    segment's NTAN tangents, and the three nonlinear-term components out
    (complex, [Nz][3][Q][X])."""
    Nx, Ny, Nz = g["Nx"], g["Ny"], g["Nz"]
    X, Q, pz, px = Nx // 2, 3 * Ny // 2, 3 * Nz // 2, 3 * Nx // 2
    fields = 6.0 * Q * pz * px * 8
    return ninst * (fields + fields / NTAN + 3.0 * Nz * Q * X * 16)


def phys_inverse_bytes(ninst, g, nfields=6):
    """Algorithmic HBM bytes of one k_phys_inverse_tc launch: the five
    velocity components in (complex, [Nz][5][Q][X]), the physical fields out."""
    Nx, Ny, Nz = g["Nx"], g["Ny"], g["Nz"]
    X, Q, pz, px = Nx // 2, 3 * Ny // 2, 3 * Nz // 2, 3 * Nx // 2
    return ninst * (5.0 * Nz * Q * X * 16 + nfields * Q * pz * px * 8.0)


def measured_hbm_peak():
    """HBM GB/s measured on the GB300s (MEASURED_PEAKS.json), else the fallback"""
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs, STREAM-style copy)"
    except Exception:
        return 6800.0, "fallback 6.8 TB/s"


def dominant_roofline(cc, k_ms, nt, value_per_gpu):
    """Roofline of the dominant kernel of the step, k_products_tc (its
    192-instance tangent launch; 37.5% of the sweeps' kernel time in the ncu
    launch list of this workload, k_phys_inverse_tc 32.8%): achieved
    algorithmic bytes per launch / CUDA-event duration against the measured
    HBM peak, with the tensor-pipe view (bf16 digit-product flop against the
    measured bf16 peak) and the FP64-equivalent view beside it."""
    dom_ms = k_ms["products_fwd"]
    hbm_peak, hbm_src = measured_hbm_peak()
    bf16_peak, bf16_src = measured_bf16_peak()
    at32 = (GRID["Nx"], GRID["Ny"], GRID["Nz"]) == (32, 65, 32)
    nbytes = products_fwd_bytes(nt, GRID)
    gbs = nbytes / (dom_ms * 1e-3) / 1e9
    tc_flops = tc_products_mma_flops(nt, GRID)
    fp64_peak = cc.c_fp64_peak_tflops()
    flops = products_fwd_flops(nt, GRID)
    inv_ms = k_ms["phys_inverse"]
    inv_bytes, inv_tc = phys_inverse_bytes(nt, GRID), tc_inverse_mma_flops(nt, GRID)
    step_flop = segment_step_flops(GRID)
    return {"bound": "hbm", "kernel": f"k_products_tc ({nt} tangent instances, 3 products)",
            "achieved": gbs, "peak": hbm_peak, "unit": "GB/s", "frac": gbs / hbm_peak, "peak_source": hbm_src,
            "traffic": PROD_TRAFFIC_PER_INSTANCE_32 * nt if at32 else None,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of a 24-instance launch, "
                              "scaled by the instance count (bytes per launch)",
            "algorithmic_bytes_per_launch": nbytes, "kernel_ms": k_ms,
            "note": "latency-bound (neither HBM nor a pipe is saturated); tensor and FP64 views below",
            "tensor": {"achieved": tc_flops / (dom_ms * 1e-3) / 1e12, "peak": bf16_peak, "unit": "TFLOP/s",
                       "frac": tc_flops / (dom_ms * 1e-3) / 1e12 / bf16_peak, "peak_source": bf16_src,
                       "mma_flop_per_launch": tc_flops},
            "fp64_equivalent": {"achieved": flops / (dom_ms * 1e-3) / 1e12, "peak": fp64_peak,
                                "unit": "TFLOP/s", "frac": flops / (dom_ms * 1e-3) / 1e12 / fp64_peak,
                                "peak_source": "FP64 FMA probe in this run (c_fp64_peak_tflops)"},
            "phys_inverse_tc": {"kernel": f"k_phys_inverse_tc ({nt} x 6 tangent fields)", "ms": inv_ms,
                                "achieved_gbs": inv_bytes / (inv_ms * 1e-3) / 1e9,
                                "frac_hbm": inv_bytes / (inv_ms * 1e-3) / 1e9 / hbm_peak,
                                "tensor_frac": inv_tc / (inv_ms * 1e-3) / 1e12 / bf16_peak,
                                "traffic": PHYS_TRAFFIC_PER_INSTANCE_32 * nt if at32 else None},
            "step": {"algorithmic_flop_per_segment_step": step_flop,
                     "achieved_tflops": step_flop * value_per_gpu / 1e12,
                     "frac_of_fp64_fma_peak": step_flop * value_per_gpu / 1e12 / fp64_peak}}


def exact_adjoint_timing(cc, torch, stream, dAC, K):
    """The exact discrete adjoint (c_batch_adjoint_exact_dev, the transpose of
    the homogeneous tangent) over the stored K-step trajectories of the batch,
    timed with CUDA events on the library stream beside the reference's
    adjoint (c_batch_adjoint_dev, strength 1) on the same batch."""
    out = {}
    lam = dAC.clone()
    for name, call in (("reference_adjoint", lambda: cc.lib.c_batch_adjoint_dev(K, 0, lam.data_ptr(), 1.0)),
                       ("exact_adjoint", lambda: cc.lib.c_batch_adjoint_exact_dev(K, 0, lam.data_ptr()))):
        assert call() == 0, cc.c_last_error_message()  # warm-up (graph instantiation)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(3):
            assert call() == 0, cc.c_last_error_message()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / 3
        out[name] = {"segment_steps_per_s": NSEG * K / (ms * 1e-3), "ms_per_sweep": ms}
    out["note"] = (f"{NSEG} segments x {K} steps of stored trajectory; the exact adjoint needs one transposed "
                   "product pass per substage where the reference's needs two")
    return out


def ctypes_int_array(vals):
    import ctypes
    return (ctypes.c_int * len(vals))(*vals)


def uneven_batch(cc, n=128, steps=5):
    """128 instances with grids drawn from 16x33x16, 32x65x32, 48x97x48, Re
    from [2000, 4000] and dt at half the CFL limit of a laminar estimate,
    advanced by the same launches (c_multi_*): one primal sweep and one
    adjoint sweep of `steps` steps; instance-steps per second of each."""
    import ctypes
    from channel.synthetic import synthetic_state
    rng = np.random.default_rng(3)
    grids = [(16, 33, 16), (32, 65, 32), (48, 97, 48)]
    pick = rng.integers(0, 3, n)
    Re = rng.uniform(2000.0, 4000.0, n)
    inst = []
    for i in range(n):
        Nx, Ny, Nz = grids[pick[i]]
        # CFL_MAX 2.8 (channel/pass1.c:133) with |u| ~ 1.5 flux/2 at the finest
        # spacing of each direction; half of it
        dx, dz = 2 * math.pi / (1.5 * Nx), math.pi / (1.5 * Nz)
        dy = 1.0 - math.cos(math.pi / (1.5 * Ny))
        dt = 0.5 * 2.8 / (1.5 / dx + 0.1 / dy + 0.1 / dz)
        inst.append((Nx, Ny, Nz, float(Re[i]), min(dt, 0.01)))
    arr = lambda v, t: (t * n)(*v)
    t0 = time.perf_counter()
    rc = cc.lib.c_multi_init(n, arr([x[0] for x in inst], ctypes.c_int), arr([x[1] for x in inst], ctypes.c_int),
                             arr([x[2] for x in inst], ctypes.c_int), arr([2 * math.pi] * n, ctypes.c_double),
                             arr([math.pi] * n, ctypes.c_double), arr([x[3] for x in inst], ctypes.c_double),
                             arr([2.0] * n, ctypes.c_double), arr([x[4] for x in inst], ctypes.c_double), steps, 0, 0)
    assert rc == 0, cc.c_last_error_message()
    init_s = time.perf_counter() - t0
    C = np.concatenate([synthetic_state(*x[:3], seed=i).ravel() for i, x in enumerate(inst)])
    AC = np.concatenate([synthetic_state(*x[:3], seed=500 + i, laminar=False).ravel() for i, x in enumerate(inst)])
    tune = json.loads(cc.lib.c_autotune_report().decode() or "{}")
    t0 = time.perf_counter()
    assert cc.lib.c_multi_primal(0, C.ctypes.data) == 0, cc.c_last_error_message()
    t1 = time.perf_counter()
    assert cc.lib.c_multi_adjoint(steps, 0, AC.ctypes.data, 0.0) == 0, cc.c_last_error_message()
    t2 = time.perf_counter()
    cc.lib.c_multi_destroy()
    counts = {f"{g[0]}x{g[1]}x{g[2]}": int((pick == k).sum()) for k, g in enumerate(grids)}
    return {"instances": n, "grids": counts, "steps": steps, "init_s": init_s,
            "primal_instance_steps_per_s": n * steps / (t1 - t0),
            "adjoint_instance_steps_per_s": n * steps / (t2 - t1), "autotune": tune,
            "note": "host arrays, copies included; one launch per kernel and substage for all instances"}


def autograd_config(C0, nsteps=1000, checkpoint=50):
    """The differentiable single trajectory at 32x65x32, Re 3300, dt 0.005:
    time-mean lower-wall shear over `nsteps` steps from the run-up parent
    field, checkpoints every `checkpoint` steps (channel.autograd), with
    dJ/dRe, dJ/dmeanU and dJ/dC0 (one exact-adjoint sweep) against
    central differences: meanU at relative step 1e-6; C0 along one seeded
    direction of norm |C0| and Re at relative steps 1e-3 .. 1e-6 (headline
    comparisons at 1e-5 and 1e-3, where truncation and rounding noise
    balance; the sweeps show both)."""
    import torch
    from channel import autograd as ag
    from channel.synthetic import synthetic_state
    grid = {k: GRID[k] for k in ("Nx", "Ny", "Nz", "Lx", "Lz", "dt")}
    Re0, U0 = GRID["Re"], GRID["flux"] / 2
    cfg = {"grid": grid, "C0": C0, "nsteps": nsteps, "checkpoint": checkpoint}
    Re = torch.tensor(Re0, dtype=torch.float64, requires_grad=True)
    U = torch.tensor(U0, dtype=torch.float64, requires_grad=True)
    Ct = torch.from_numpy(C0.view(np.float64).reshape(C0.shape + (2,)).copy()).requires_grad_(True)
    J = ag.time_mean_wall_shear(Re, U, cfg, Ct)
    J.backward()
    rep = dict(cfg["report"])
    J_of = lambda r, u, c: ag.primal_objective(grid, r, u, c, nsteps, checkpoint)[0]
    t0 = time.perf_counter()
    # dJ/dRe is small (elasticity ~0.02) and J carries the scheme's rounding
    # noise (~1e-11 relative per step at this grid), so differences in Re
    # are noise-limited below a relative step of ~1e-5: report the sweep
    fd_re = {}
    for hr in (1e-3, 1e-4, 1e-5, 1e-6):
        h = hr * Re0
        fd_re[f"{hr:g}"] = (J_of(Re0 + h, U0, C0) - J_of(Re0 - h, U0, C0)) / (2 * h)
    fdR = fd_re["0.001"]
    hU = 1e-6 * U0
    fdU = (J_of(Re0, U0 + hU, C0) - J_of(Re0, U0 - hU, C0)) / (2 * hU)
    d = synthetic_state(GRID["Nx"], GRID["Ny"], GRID["Nz"], seed=77, laminar=False)
    d *= np.linalg.norm(C0) / np.linalg.norm(d)
    fd_c0 = {}
    for hC in (1e-3, 1e-4, 1e-5, 1e-6):
        fd_c0[f"{hC:g}"] = (J_of(Re0, U0, C0 + hC * d) - J_of(Re0, U0, C0 - hC * d)) / (2 * hC)
    fdC = fd_c0["1e-05"]
    anC = float(np.sum(Ct.grad.numpy() * d.view(np.float64).reshape(Ct.shape)))
    rel = lambda a, b: abs(a - b) / abs(b)
    return {"grid": "32x65x32", "steps": nsteps, "checkpoint_every": checkpoint, "J": float(J.detach()),
            "forward_s": rep["forward_s"], "backward_s": rep["backward_s"],
            "dJ_dRe": float(Re.grad), "fd_dJ_dRe": fdR, "rel_err_Re": rel(float(Re.grad), fdR),
            "fd_dJ_dRe_by_relative_step": fd_re,
            "rel_err_Re_by_relative_step": {k: rel(float(Re.grad), v) for k, v in fd_re.items()},
            "dJ_dmeanU": float(U.grad), "fd_dJ_dmeanU": fdU, "rel_err_meanU": rel(float(U.grad), fdU),
            "dJ_dC0_dir": anC, "fd_dJ_dC0_dir": fdC, "rel_err_C0": rel(anC, fdC),
            "rel_err_C0_by_relative_step": {k: rel(anC, v) for k, v in fd_c0.items()},
            "fd_s": time.perf_counter() - t0,
            "note": "backward = one exact-adjoint sweep giving dJ/dC0, dJ/dmeanU and dJ/dRe, each interval "
                    "recomputed from its checkpoint; central differences: meanU at relative step 1e-6, C0 at 1e-5, "
                    "Re at 1e-3 (the sweeps show truncation at larger steps, rounding noise at smaller)"}


def large_grid(cc, nsteps=8):
    """128x129x128, Lx 4 pi, Lz 2 pi, Re 3300, dt 0.002: the checkpointed
    forward + adjoint (channel.checkpoint) with the HBM-sized interval and a
    short one to expose the recomputation overhead."""
    from channel import checkpoint
    from channel.synthetic import synthetic_state
    grid = dict(Nx=128, Ny=129, Nz=128, Lx=4 * math.pi, Lz=2 * math.pi, Re=3300.0, flux=2.0, dt=0.002)
    C0 = synthetic_state(128, 129, 128, seed=1)
    AC0 = synthetic_state(128, 129, 128, seed=2, laminar=False)
    out = {"grid": "128x129x128", "steps": nsteps,
           "hbm_spacing_for_5000_steps": checkpoint.choose_spacing(grid, 5000)}
    for name, sp in (("one_interval", nsteps), ("interval_2", 2)):
        _, _, rep = checkpoint.forward_adjoint(grid, C0, nsteps, AC0, spacing=sp)
        rep["primal_steps_per_s"] = nsteps / rep["forward_s"]
        rep["adjoint_steps_per_s"] = nsteps / rep["adjoint_s"]
        out[name] = rep
    cc.c_destroy()
    return out


def large_grid_horizon(cc, nsteps=5000):
    """128x129x128 forward + adjoint over the full 5000-step horizon with the
    checkpoint interval sized to the free HBM (channel.checkpoint): the
    primal keeps one checkpoint per interval, the adjoint recomputes each
    interval from its checkpoint; rates and recomputation overhead."""
    from channel import checkpoint
    from channel.synthetic import synthetic_state
    grid = dict(Nx=128, Ny=129, Nz=128, Lx=4 * math.pi, Lz=2 * math.pi, Re=3300.0, flux=2.0, dt=0.002)
    C0 = synthetic_state(128, 129, 128, seed=1)
    AC0 = synthetic_state(128, 129, 128, seed=2, laminar=False)
    spacing = checkpoint.choose_spacing(grid, nsteps)
    _, AC, rep = checkpoint.forward_adjoint(grid, C0, nsteps, AC0, spacing=spacing)
    rep["primal_steps_per_s"] = nsteps / rep["forward_s"]
    rep["adjoint_steps_per_s"] = nsteps / rep["adjoint_s"]
    rep["adjoint_finite"] = bool(np.isfinite(AC).all())
    rep["grid"] = "128x129x128"
    cc.c_destroy()
    return rep


def plain_gpu(cc, C, IC, AC, K):
    """One trajectory per launch sequence through the reference entry points
    (c_primal, three c_tangent calls, c_adjoint coupled to the last tangent)
    for one segment over K steps; segment-steps per second."""
    assert cc.c_init(*grid_args(K)) == 0
    ICs = [IC[t].copy() for t in range(len(IC))]
    cc.c_primal(0, C.copy())  # warm-up
    cc.c_tangent(0, K, IC[0].copy(), 0)
    cc.c_adjoint(K, 0, AC.copy(), 0, 1.0)
    cc.c_synchronize()
    C, AC = C.copy(), AC.copy()
    t0 = time.perf_counter()
    cc.c_primal(0, C)
    for t, x in enumerate(ICs):
        cc.c_tangent(0, K, x, INHOMO[t])
    cc.c_adjoint(K, 0, AC, 0, 1.0)
    cc.c_synchronize()
    dt_ = time.perf_counter() - t0
    cc.c_destroy()
    return {"value": K / dt_, "unit": UNIT, "segments": 1, "steps": K,
            "note": "single-trajectory entry points (c_primal, c_tangent x3, c_adjoint), host arrays"}


# ---------------------------------------------------------------------------
# CPU: the reference algorithm (oracle restatement) on the host cores
# ---------------------------------------------------------------------------

def _segment_case(steps, seed):
    """a constructed oracle instance and one segment's inputs (not timed)"""
    import oracle as O
    ch = O.PortChannel(*grid_args(steps))
    C = O.synthetic_state(GRID["Nx"], GRID["Ny"], GRID["Nz"], seed=seed)
    IC = [O.synthetic_state(GRID["Nx"], GRID["Ny"], GRID["Nz"], seed=seed + 1 + t, laminar=False)
          for t in range(NTAN)]
    AC = O.synthetic_state(GRID["Nx"], GRID["Ny"], GRID["Nz"], seed=seed + 9, laminar=False)
    return ch, C, IC, AC


def _segment_steps(ch, C, IC, AC, steps):
    """the reference sequence of one segment over `steps` steps: primal, the
    tangents (each re-running the primal, as the reference's tangent does),
    the adjoint coupled to the last tangent with strength 1"""
    ch.primal(0, C.copy())
    for t in range(NTAN):
        ch.tangent(0, steps, IC[t].copy(), INHOMO[t])
    ch.adjoint(steps, 0, AC.copy(), 0, 1.0)


def cpu_baseline(steps=2):
    import oracle as O
    O.build_port()
    ch, C, IC, AC = _segment_case(steps, 0)
    t0 = time.perf_counter()
    _segment_steps(ch, C, IC, AC, steps)
    dt_ = time.perf_counter() - t0
    ch.close()
    return {"value": steps / dt_, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"1 segment x {steps} segment-steps (primal, 3 tangents each re-running the primal as "
                      f"the reference does, adjoint with strength 1) at 32x65x32, oracle/chan_port.c, 1 thread, "
                      f"instance constructed before the timed region",
            "seconds": dt_}


REF_STEPS = 2   # segment-steps per process in one sample of the reference arm


def _reference_worker(rank, nsamples, barrier, queue):
    """one host core: constructs its oracle instance once, then for every
    sample waits at the barrier and times REF_STEPS segment-steps"""
    ch, C, IC, AC = _segment_case(REF_STEPS, 200 + 10 * rank)
    for k in range(nsamples):
        barrier.wait()
        t0 = time.clock_gettime(time.CLOCK_MONOTONIC)
        _segment_steps(ch, C, IC, AC, REF_STEPS)
        queue.put((k, rank, t0, time.clock_gettime(time.CLOCK_MONOTONIC)))
    ch.close()


def run_reference(a):
    """The reference algorithm on all host cores: one segment per process
    (as drivers/mpi_wrapper.py runs one segment per rank).  Each process
    builds its oracle instance before any timing; a sample starts every
    process at a barrier and lasts from the first start to the last end."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import multiprocessing as mp
    import oracle as O
    O.build_port()
    cores = os.cpu_count() or 1
    W = max(1, min(a.warmup, 1))
    K = max(2, min(a.steps, 3))
    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(cores)
    queue = ctx.Queue()
    procs = [ctx.Process(target=_reference_worker, args=(r, W + K, barrier, queue)) for r in range(cores)]
    for p in procs:
        p.start()
    spans = {}
    for _ in range(cores * (W + K)):
        k, r, t0, t1 = queue.get()
        s0, s1 = spans.get(k, (t0, t1))
        spans[k] = (min(s0, t0), max(s1, t1))
    for p in procs:
        p.join()
    walls = [spans[k][1] - spans[k][0] for k in range(W, W + K)]
    wall = statistics.median(walls)
    value = cores * REF_STEPS / wall
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0,
            "steps": K, "warmup": W, "ms_per_step": wall * 1e3 / REF_STEPS, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic seeded states",
            "config": CONFIG,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{cores} processes x 1 segment x {REF_STEPS} segment-steps at 32x65x32 "
                                       f"per sample (oracle/chan_port.c, the reference algorithm bit for bit); "
                                       f"instances built before timing; median of {K} samples after {W} warm-up"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    emit(line)


if __name__ == "__main__":
    a = args_parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_gb300(a)
