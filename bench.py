#!/usr/bin/env python
"""3D-CTF filtered-backprojection benchmark (one JSON line on stdout).

Workload: 61 tilts over +-60 deg (2 deg steps), 1024 x 1024 projections at
1.0 A/px, 300 kV, Cs 2.7 mm, defocus 30000 A at the tilt axis, ndf = 10 slabs
(the reference's default width-based slab range), volume 1024 x 1024 x 300.
Input: a seeded synthetic phantom of 2000 Gaussian blobs, analytically
projected and imaged through the CTF at each blob's height (guanaco_gb300.
synthetic), with Gaussian noise -- the reference publishes no dataset for
this path.

A step is one whole 3D-CTF FBP of the tilt series: phase-flip correction of
every tilt into 10 defocus slabs, ramp filtering of every row, backprojection
of every voxel from every tilt.  The metric is voxel-tilt updates per second
(Y * Z * X * T per step).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference's CPU algorithm (the oracle port,
oracle/gno_oracle.c, all host threads) on a bounded sample of the same
workload per step, extrapolated to the whole series.
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

# Load every CUDA kernel when the context is created rather than at its first
# launch, as a latency-sensitive service would: a lazily loaded kernel's first
# launch inside the serving stream can hold up the requests in flight (the
# stream's p99 tail of about 100 ms appeared in fewer runs with eager loading).
# A caller's own setting wins.
os.environ.setdefault("CUDA_MODULE_LOADING", "EAGER")

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = ("3D-CTF FBP Gvoxel·tilt/s, FP16-staged vs FP32 at rel-L2≤1e-3; "
          "serve p50/p99 ms")
UNIT = "Gvoxel·tilt/s"
WL = dict(T=61, H=1024, W=1024, Z=300, D=10, pixel_size=1.0, defocus=30000.0, energy=300.0,
          cs_mm=2.7, blobs=2000, seed=3, tilt_max=60.0, noise=0.1, ctf=True)
WORKLOAD_NAME = ("3D CTF ndf=10: 61 tilts +-60 deg, 1024x1024 projections at 1.0 A/px, "
                 "300 kV, Cs 2.7 mm, df 30000 A, volume 1024x1024x300")
# DRAM bytes (read + written) of one backprojection launch on this workload,
# from an ncu capture whose summary (command included) is committed beside the
# other profiles; the line names the file it came from.
TRAFFIC_CAPTURE = os.path.join("profiles", "bp_dram_3dctf_ndf10.md")


def bp_traffic(form):
    """(bytes per launch, source) from the capture summary, or (None, reason)."""
    path = os.path.join(REPO, TRAFFIC_CAPTURE)
    try:
        with open(path) as f:
            for line in f:
                parts = dict(kv.split("=", 1) for kv in line.split() if "=" in kv)
                if parts.get("form") == form and "dram_bytes_per_launch" in parts:
                    return float(parts["dram_bytes_per_launch"]), TRAFFIC_CAPTURE
    except OSError:
        pass
    return None, f"no capture of the {form} backprojector in {TRAFFIC_CAPTURE}"


def tc_mma_flops():
    """FLOPs of the tensor-core backprojector's MMAs on the workload: per row
    band (256 rows when every 16 x 8 voxel tile reaches at most two slabs per
    tilt, else 128), tile and tilt, the slabs between the lowest and highest
    slab of the tile's four corner voxels inside the volume (the kernel's table
    rule, evaluated here in float32), each two MMAs of M 128 x N rows x K 16.
    (rows, flops)."""
    T, H, W, Z = WL["T"], WL["H"], WL["W"], WL["Z"]
    c, mn, mx, step, nd = slab_setup()
    df = WL["defocus"]
    mind, maxd = np.float32(mn - df), np.float32(mx - df)
    px = np.float32(WL["pixel_size"])
    ds = np.float32(nd * px / (maxd - mind)) if nd > 1 else np.float32(0)
    doff = np.float32(-ds * np.float32(mind / px))
    th = angles_rad()
    co, si = np.cos(th).astype(np.float32), np.sin(th).astype(np.float32)
    d = co * co + si * si
    cos_a, sin_a = co / d, si / d

    def coord(i, n):
        return (i.astype(np.float64) - 0.5 * n + 0.5).astype(np.float32)

    x0 = np.arange(0, W, 16)
    z0 = np.arange(0, Z, 8)
    cx = [coord(x0, W), coord(np.minimum(x0 + 16, W) - 1, W)]
    cz = [coord(z0, Z), coord(np.minimum(z0 + 8, Z) - 1, Z)]
    per_tilt = []
    for t in range(T):
        ks = []
        for x in cx:
            for z in cz:
                h = ((-x[:, None] * sin_a[t]).astype(np.float32)
                     - (z[None, :] * cos_a[t]).astype(np.float32))
                dd = (h * ds).astype(np.float32) + doff
                fl = np.floor(dd)
                k = fl + ((dd - fl) >= 0.5)
                ks.append(np.clip(k, 0, nd - 1))
        per_tilt.append(np.max(ks, 0) - np.min(ks, 0) + 1 if nd > 1
                        else np.ones((len(x0), len(z0))))
    nk = np.stack(per_tilt)
    rows = 256 if nk.max() <= 2 else 128
    slots = float(nk.sum()) * ((H + rows - 1) // rows)
    return rows, slots * 2 * (2 * 128 * rows * 16)


def angles_rad():
    n = WL["T"]
    return np.deg2rad(np.linspace(-WL["tilt_max"], WL["tilt_max"], n)).astype(np.float32)


def voxel_tilts():
    return WL["H"] * WL["Z"] * WL["W"] * WL["T"]


def fft_flops(live_pairs=None):
    """Nominal flops (5 n log2 n per complex n-point transform) of one step's
    correction and filter: per tilt the forward row and column transforms (two
    real rows per complex row, W/2 complex columns); per (tilt, slab) pair
    that some voxel reads (all T D pairs when live_pairs is None) the inverse
    column transforms and the ramp filter's four W-point transforms per row
    pair."""
    T, H, W = WL["T"], WL["H"], WL["W"]
    D = WL["D"] if WL["ctf"] else 1

    def f(n):
        return 5.0 * n * math.log2(n)

    rows = (H + 1) // 2 * 4 * f(W)
    if not WL["ctf"]:
        return T * rows
    pairs = T * D if live_pairs is None else live_pairs
    return T * ((H + 1) // 2 * f(W) + W // 2 * f(H)) + pairs * (W // 2 * f(H) + rows)


def slab_setup():
    import guanaco_gb300 as G

    c = G.get_centre((WL["T"], WL["H"], WL["W"]), None, False)
    mn, mx, step, nd = G.get_defocus_steps(WL["defocus"], WL["D"], None, WL["W"], c,
                                           WL["pixel_size"])
    return c, mn, mx, step, nd


def make_plan(staging):
    import guanaco_gb300 as G

    if not WL["ctf"]:  # plain FBP: ramp filter and backprojection only
        c = G.get_centre((WL["T"], WL["H"], WL["W"]), None, False)
        return G.FbpPlan(WL["T"], WL["H"], WL["W"], angles_rad(), grid_height=WL["Z"],
                         grid_width=WL["W"], centre=c, pixel_size=WL["pixel_size"],
                         input="raw", correct=False, staging=staging)
    c, mn, mx, step, nd = slab_setup()
    df = WL["defocus"]
    return G.FbpPlan(WL["T"], WL["H"], WL["W"], angles_rad(), grid_height=WL["Z"],
                     grid_width=WL["W"], centre=c, pixel_size=WL["pixel_size"], input="raw",
                     correct=True, num_defocus=nd, slab_defocus=G.api.slab_defoci(mn, nd, step),
                     min_defocus=float(mn - df), max_defocus=float(mx - df), energy=WL["energy"],
                     spherical_aberration=WL["cs_mm"], staging=staging)


def make_projections(device):
    from guanaco_gb300 import synthetic

    blobs = synthetic.blob_phantom(WL["blobs"], WL["W"], WL["H"], WL["Z"], WL["seed"])
    return synthetic.tilt_series(blobs, angles_rad(), WL["H"], WL["W"],
                                 pixel_size=WL["pixel_size"],
                                 defocus=WL["defocus"] if WL["ctf"] else None,
                                 energy=WL["energy"], cs_mm=WL["cs_mm"], noise=WL["noise"],
                                 seed=WL["seed"], device=device)


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200", "-f", self.path],
                stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.3)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) < 9:
                    continue
                try:
                    sm.append(float(p[1]))
                    smax.append(float(p[2]))
                except ValueError:
                    continue
                for name, v in zip(names, p[5:9]):
                    if v.lower() == "active":
                        reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------- N replicas
def reduce_max_over_ranks(values, dist, device):
    """Each timing's maximum over the ranks: the slowest replica sets the job's
    time.  ``dist`` is torch.distributed (or None for one rank)."""
    if dist is None:
        return [float(v) for v in values]
    import torch

    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def job_throughput(units_per_step, steps, world, ms):
    """Whole-job Gvoxel·tilt/s: every replica's units over the slowest time."""
    return units_per_step * steps * world / (ms * 1e-3) / 1e9


# --------------------------------------------------------------- our arm
def run_ours(args, rank, world, dist):
    import torch

    import guanaco_gb300 as G  # noqa: F401

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    proj = make_projections(dev)
    torch.cuda.synchronize()
    plans, vols = {}, {}
    large = args.case == "large"

    def ensure(form):
        if form not in plans:
            plans[form] = make_plan(form)
            vols[form] = torch.empty((WL["H"], WL["Z"], WL["W"]), dtype=torch.float32,
                                     device=dev)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def timed(form):
        ensure(form)
        plan, vol = plans[form], vols[form]
        for _ in range(args.warmup):
            plan.execute(proj, vol, stream)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * args.steps + 2)]
        barrier()
        ev[0].record(stream)
        for k in range(args.steps):
            plan.stage(proj, stream)
            ev[2 * k + 1].record(stream)
            plan.backproject(vol, False, stream)
            ev[2 * k + 2].record(stream)
        ev[-1].record(stream)
        barrier()
        total = ev[0].elapsed_time(ev[-1])
        bp = [ev[2 * k + 1].elapsed_time(ev[2 * k + 2]) for k in range(args.steps)]
        plan.check(stream)
        return total, sum(bp) / len(bp)

    clocks = ClockSampler(dev.index)
    clocks.start()
    res, backprojector = {}, {}
    for form in (("f16", "f16t", "f32") if large else ("f32", "f16", "f16t")):
        res[form] = timed(form)
        backprojector[form] = plans[form].backprojector
        if large and form != "f32":  # one plan at a time in HBM at this size
            plans.pop(form).close()
            vols.pop(form)
            torch.cuda.empty_cache()
    # end to end through the public host-buffer entry point: pinned input in,
    # volume out, every step
    from guanaco_gb300 import serve

    h_in_np = serve.pinned_empty(tuple(proj.shape))
    h_in_np[...] = proj.cpu().numpy()
    h_out_np = serve.pinned_empty((WL["H"], WL["Z"], WL["W"]))
    plans["f32"].execute_host(h_in_np, h_out_np, stream)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        plans["f32"].execute_host(h_in_np, h_out_np, stream)
    barrier()
    e2e_ms = (time.perf_counter() - t0) * 1e3
    # the same for the F16T form (its plan is closed after timing at the large size)
    e2e16t_ms = None
    if "f16t" in plans:
        plans["f16t"].execute_host(h_in_np, h_out_np, stream)
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            plans["f16t"].execute_host(h_in_np, h_out_np, stream)
        barrier()
        e2e16t_ms = (time.perf_counter() - t0) * 1e3
    clk = clocks.stop()

    total32, total16, total16t, e2e_ms, e2e16t = reduce_max_over_ranks(
        [res["f32"][0], res["f16"][0], res["f16t"][0], e2e_ms,
         e2e16t_ms if e2e16t_ms is not None else 0.0], dist, dev)
    e2e16t_ms = e2e16t if e2e16t_ms is not None else None
    value32 = job_throughput(voxel_tilts(), args.steps, world, total32)
    value16 = job_throughput(voxel_tilts(), args.steps, world, total16)
    value16t = job_throughput(voxel_tilts(), args.steps, world, total16t)
    e2e_value = job_throughput(voxel_tilts(), args.steps, world, e2e_ms)

    serving = run_serving(dev) if not args.no_serve else None
    parity = cpu = None
    if rank == 0 and not args.no_cpu:
        parity, cpu = oracle_sample(proj, vols)
    if rank != 0:
        return
    import json as _json

    peaks = {}
    try:
        peaks = _json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    p32 = plans["f32"]
    staged_bytes = WL["D"] * WL["T"] * WL["H"] * WL["W"] * 4
    vol_bytes = WL["H"] * WL["Z"] * WL["W"] * 4
    bp_alg = staged_bytes + vol_bytes
    bp_ms = res["f32"][1]
    traffic, traffic_src = bp_traffic("f32")
    achieved = bp_alg / (bp_ms * 1e-3) / 1e9
    # the backprojector's binding resource: shared-memory loads, two 8-byte
    # pixel pairs per (voxel, row pair, tilt) = 8 bytes per voxel-tilt, against
    # 128 bytes per clock per SM at the SM clock sampled during the run
    vt = WL["T"] * WL["H"] * WL["Z"] * WL["W"]
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    sm_mhz = clk.get("sm_mhz") or clk.get("sm_max_mhz")
    smem_peak = sms * 128 * sm_mhz * 1e6 / 1e9 if sm_mhz else None
    smem_achieved = 8 * vt / (bp_ms * 1e-3) / 1e9
    # correction + filter stage (everything before the backprojection): HBM
    # bytes of the fused stage (raw projections in, staged rows out; the
    # flipped spectra pass through L2 tilt by tilt) and its FFT work at the
    # nominal 5 n log2 n flops per complex n-point transform
    stage_ms = total32 / args.steps - bp_ms
    stage_bytes = WL["T"] * WL["H"] * WL["W"] * 4 + staged_bytes
    # (tilt, slab) pairs some voxel reads: only those are phase flipped and filtered
    live = p32.live_slabs(stream)
    live_pairs = int((live[:, 1] - live[:, 0] + 1).sum())
    stage_flops = fft_flops(live_pairs if WL["ctf"] else None)
    # the F16T form's backprojector against the tensor peak: the FLOPs its MMAs
    # execute (weights of two pixels per voxel padded to 32-pixel windows, so
    # most of them multiply zeros) over its event time, and its DRAM traffic
    tc_roofline = None
    if backprojector["f16t"] == 16 and WL["ctf"]:
        tc_rows, tc_flops = tc_mma_flops()
        tc_ms = res["f16t"][1]
        bf16_peak = peaks.get("bf16_tflops", 1900.0)
        tc_traffic, tc_src = bp_traffic("f16t")
        tc_roofline = {
            "kernel": f"k_bp_tc<{tc_rows},...> (tensor-core backprojection)",
            "bound": "tensor",
            "achieved": round(tc_flops / (tc_ms * 1e-3) / 1e12, 1),
            "peak": bf16_peak,
            "peak_source": ("measured (cuBLAS bf16 burst)" if "bf16_tflops" in peaks
                            else "fallback"),
            "unit": "TFLOP/s",
            "frac": round(tc_flops / (tc_ms * 1e-3) / 1e12 / bf16_peak, 4),
            "mma_flops_per_launch": tc_flops,
            "flops_source": "MMA slots counted on the host from the tiles' corner slabs",
            "traffic": tc_traffic if args.case == "3dctf" else None,
            "traffic_source": tc_src if args.case == "3dctf" else "no capture for this case",
            "hbm_frac": (round(tc_traffic / (tc_ms * 1e-3) / 1e9 / hbm_peak, 4)
                         if tc_traffic and args.case == "3dctf" else None),
        }
    line = {
        "metric": METRIC,
        "value": round(value32, 2),
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(total32 / args.steps, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": (f"synthetic: {WL['blobs']}-blob phantom, analytic projections"
                 f"{' through the CTF' if WL['ctf'] else ''}, seeded"),
        "config": {
            "workload": WORKLOAD_NAME,
            "tilts": WL["T"], "projection": [WL["H"], WL["W"]], "volume": [WL["H"], WL["W"], WL["Z"]],
            "ndf": WL["D"], "staging": "f32", "parallelism": f"replicas x{world}",
            "l2": (f"inputs larger than L2: {WL['T'] * WL['H'] * WL['W'] * 4 / 1e6:.0f} MB "
                   f"projections, {WL['D'] * WL['T'] * WL['H'] * WL['W'] * 4 / 1e9:.2f} GB "
                   "staged rows per step"),
        },
        "forms": {
            "f32": {"value": round(value32, 2), "ms_per_step": round(total32 / args.steps, 4),
                    "bp_ms": round(res["f32"][1], 4)},
            "f16": {"value": round(value16, 2), "ms_per_step": round(total16 / args.steps, 4),
                    "bp_ms": round(res["f16"][1], 4),
                    "speedup_vs_f32": round(value16 / value32, 3),
                    "staging": "FP16 records, per-row exponents, CUDA-core backprojection"},
            "f16t": {"value": round(value16t, 2), "ms_per_step": round(total16t / args.steps, 4),
                     "bp_ms": round(res["f16t"][1], 4),
                     "speedup_vs_f32": round(value16t / value32, 3),
                     "staging": ("FP16 rows, one power-of-two scale per tilt, tensor-core "
                                 "backprojection (tcgen05, FP32 accumulation)"),
                     "roofline": tc_roofline,
                     "e2e": ({"value": round(job_throughput(voxel_tilts(), args.steps, world,
                                                            e2e16t_ms), 2),
                              "unit": UNIT, "ms_per_step": round(e2e16t_ms / args.steps, 4)}
                             if e2e16t_ms is not None else None)},
        },
        "e2e": {
            "value": round(e2e_value, 2), "unit": UNIT,
            "h2d_bytes_per_step": int(proj.numel() * 4),
            "d2h_bytes_per_step": int(WL["H"] * WL["Z"] * WL["W"] * 4),
            "ms_per_step": round(e2e_ms / args.steps, 4),
            "api": "gnc_fbp_execute_host (pinned host buffers)",
        },
        "roofline": {
            "kernel": "k_bp_fast (backprojection)",
            "bound": "hbm",
            "achieved": round(achieved, 1),
            "peak": hbm_peak,
            "peak_source": peak_src,
            "unit": "GB/s",
            "frac": round(achieved / hbm_peak, 4),
            "traffic": traffic if args.case == "3dctf" else None,
            "traffic_source": traffic_src if args.case == "3dctf" else "no capture for this case",
            "algorithmic_bytes": bp_alg,
            "kernel_ms": round(bp_ms, 4),
            "binding": {
                "resource": "shared-memory loads (8 B per voxel-tilt)",
                "achieved": round(smem_achieved, 1),
                "peak": round(smem_peak, 1) if smem_peak else None,
                "unit": "GB/s",
                "frac": round(smem_achieved / smem_peak, 4) if smem_peak else None,
                "peak_source": f"{sms} SMs x 128 B/clk x {sm_mhz} MHz (sampled SM clock)",
            },
            "correction_filter_stage": {
                "ms": round(stage_ms, 4),
                "algorithmic_bytes": stage_bytes,
                "achieved": round(stage_bytes / (stage_ms * 1e-3) / 1e9, 1),
                "unit": "GB/s",
                "frac": round(stage_bytes / (stage_ms * 1e-3) / 1e9 / hbm_peak, 4),
                "fft_tflops_nominal": round(stage_flops / (stage_ms * 1e-3) / 1e12, 2),
                "tilt_slab_pairs_computed": f"{live_pairs} of {WL['T'] * WL['D']}",
                "tilt_slab_pair_fraction": round(live_pairs / (WL["T"] * WL["D"]), 4),
                "bound": "FP32 and shared-memory instruction issue of the register FFTs",
            },
        },
        "clocks": clk,
        # kernels of this library launched in the timed region of `value`
        "gpu_launches": int(p32.launches_per_execute * args.steps),
    }
    if serving is not None:
        line["serving"] = serving
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if parity is not None:
        line["parity"] = parity
    print(json.dumps(line))


# ------------------------------------------------------------------ serving
SERVE = dict(requests=2000, seed=5, budget_gb=96, slots=8, load=0.5, burst=192)
SERVE_NAME = ("serving stream: Poisson arrivals, projections 128^2..512^2, 31/41/61 tilts over "
              "+-60 deg, df U[10000, 50000] A, ndf U{1..10}, thickness size/2, FP16 (F16T "
              "rows, tensor-core backprojection where the tiles allow) / FP32 50/50")


def serving_inputs(dev):
    """One seeded blob-phantom tilt series per (size, tilts), page-locked."""
    from guanaco_gb300 import serve, synthetic

    inputs = {}
    for n in (128, 256, 384, 512):
        blobs = synthetic.blob_phantom(max(64, n), n, n, n // 2, seed=n)
        for T in (31, 41, 61):
            ang = np.deg2rad(np.linspace(-60, 60, T)).astype(np.float32)
            t = synthetic.tilt_series(blobs, ang, n, n, defocus=30000.0, noise=0.1, seed=n + T,
                                      device=dev)
            h = serve.pinned_empty((T, n, n))
            h[...] = t.cpu().numpy()
            inputs[(n, T)] = h
    return inputs


def serving_desc(r):
    import guanaco_gb300 as G

    n, T = r["size"], r["tilts"]
    ang = np.deg2rad(np.linspace(-60, 60, T)).astype(np.float32)
    c = G.get_centre((T, n, n), None, False)
    mn, mx, step, nd = G.get_defocus_steps(r["defocus"], r["ndf"], None, n, c, 1.0)
    return G.FbpDesc(T, n, n, ang, grid_height=r["thickness"], grid_width=n, centre=c,
                     pixel_size=1.0, input="raw", correct=True, num_defocus=nd,
                     slab_defocus=G.api.slab_defoci(mn, nd, step),
                     min_defocus=float(mn - r["defocus"]), max_defocus=float(mx - r["defocus"]),
                     energy=300.0, spherical_aberration=2.7, staging=r["staging"])


def drive_stream(srv, stream, descs, inputs, pools, t_base):
    """Submits each request at its arrival time (server clock t_base + arrival);
    returns per-request (latency s, voxel-tilts, info).  Finished requests are
    collected in the order they finish (one wait_any call each, so the client's
    cost per request does not grow with the backlog).  A request whose output
    pool is empty waits until a request of its size finishes (client
    back-pressure); its latency still counts from the scheduled arrival."""
    outstanding = {}
    done = []

    def finish(rid, info):
        r, buf = outstanding.pop(rid)
        pools[r["size"]].append(buf)
        done.append((info["t_done"] - (t_base + r["arrival"]), descs[r["id"]].voxel_tilts, info))

    def collect(timeout):
        got = srv.wait_any(timeout)
        if got is not None:
            finish(*got)
        return got is not None

    for r in stream:
        target = t_base + r["arrival"]
        while True:
            while collect(0.0):
                pass
            now = srv.now()
            if now >= target:
                break
            time.sleep(min(target - now, 2e-4))
        while not pools[r["size"]]:
            collect(None)
        buf = pools[r["size"]].pop()
        rid = srv.submit(descs[r["id"]], inputs[(r["size"], r["tilts"])], buf)
        outstanding[rid] = (r, buf)
    while outstanding:
        collect(None)
    return done


def host_link_gbs(dev, nbytes=256 << 20):
    """Host <-> device copy rate (GB/s, down and up) of one page-locked buffer:
    the link every served request's input and volume cross."""
    import torch

    h = torch.empty(nbytes // 4, dtype=torch.float32).pin_memory()
    d = torch.empty(nbytes // 4, dtype=torch.float32, device=dev)
    rates = []
    for src, dst in ((d, h), (h, d)):
        dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for _ in range(4):
            dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize(dev)
        rates.append(round(4 * nbytes / (time.perf_counter() - t0) / 1e9, 1))
    return rates


def run_serving(dev):
    """The mixed serving stream through the request server: a burst of
    SERVE['burst'] requests, run once to create its shapes' plans and graphs and
    again to measure the capacity, then SERVE['requests'] Poisson arrivals at
    SERVE['load'] of it (new shapes among them still create their plans)."""
    from guanaco_gb300 import serve, synthetic

    inputs = serving_inputs(dev)
    cfg = SERVE
    pools = {n: [serve.pinned_empty((n, n // 2, n)) for _ in range(cfg["slots"] + 8)]
             for n in (128, 256, 384, 512)}
    with serve.Server(budget_bytes=cfg["budget_gb"] << 30, slots=cfg["slots"]) as srv:
        burst = synthetic.request_stream(cfg["burst"], 1e9, seed=cfg["seed"] + 1)
        bdesc = [serving_desc(r) for r in burst]
        drive_stream(srv, burst, bdesc, inputs, pools, srv.now() + 0.01)  # plans, graphs
        capacity = 0.0
        for _ in range(2):  # the better of two warm bursts (one can catch a hiccup)
            t0 = srv.now() + 0.01
            res = drive_stream(srv, burst, bdesc, inputs, pools, t0)
            span = max(i["t_done"] for _, _, i in res) - t0
            capacity = max(capacity, len(burst) / span)
        rate = cfg["load"] * capacity
        stream = synthetic.request_stream(cfg["requests"], rate, seed=cfg["seed"])
        descs = [serving_desc(r) for r in stream]
        link_before = host_link_gbs(dev)
        load_before = os.getloadavg()
        clocks = ClockSampler(dev.index)
        clocks.start()
        t_base = srv.now() + 0.05
        res = drive_stream(srv, stream, descs, inputs, pools, t_base)
        clk = clocks.stop()
        link_after = host_link_gbs(dev)
        load_after = os.getloadavg()
        stats = srv.stats()
    lat = np.array([x[0] for x in res]) * 1e3
    replay = np.array([bool(x[2]["graph"]) for x in res])
    # arrival time of each request (done - latency); new shapes, and so plan
    # creations, cluster early in the stream
    arrived = np.array([x[2]["t_done"] - x[0] for x in res]) - t_base
    late = arrived >= 0.5 * arrived.max()
    # where the latency goes: client (scheduled arrival -> submitted), queue
    # (submitted -> admitted), service (admitted -> volume in host memory)
    parts = {
        "client": np.array([x[2]["t_submit"] - (x[2]["t_done"] - x[0]) for x in res]) * 1e3,
        "queue": np.array([x[2]["t_start"] - x[2]["t_submit"] for x in res]) * 1e3,
        "service": np.array([x[2]["t_done"] - x[2]["t_start"] for x in res]) * 1e3,
    }
    span = max(x[2]["t_done"] for x in res) - t_base
    vt = sum(x[1] for x in res)

    def pct(sel):
        v = lat[sel]
        if v.size == 0:
            return {"requests": 0}
        return {"requests": int(v.size), "p50_ms": round(float(np.percentile(v, 50)), 3),
                "p99_ms": round(float(np.percentile(v, 99)), 3), "max_ms": round(float(v.max()), 3)}

    return {
        "workload": SERVE_NAME,
        "requests": len(res),
        "p50_ms": round(float(np.percentile(lat, 50)), 3),
        "p99_ms": round(float(np.percentile(lat, 99)), 3),
        "max_ms": round(float(lat.max()), 3),
        "mean_ms": round(float(lat.mean()), 3),
        "graph_replays_latency": pct(replay),
        "direct_runs_latency": pct(~replay),
        "second_half_latency": dict(pct(late), direct_runs=int((late & ~replay).sum())),
        "clocks": clk,
        "module_loading": os.environ.get("CUDA_MODULE_LOADING"),
        "host_link_gbs": {"down_up_before": link_before, "down_up_after": link_after},
        # the server's scheduler, builder and completion callbacks are host
        # threads: the host's load average (1, 5, 15 min) and its CPU count
        "host_load": {"before": [round(x, 2) for x in load_before],
                      "after": [round(x, 2) for x in load_after], "cpus": os.cpu_count()},
        "latency_parts_ms": {k: {"p50": round(float(np.percentile(v, 50)), 3),
                                 "p99": round(float(np.percentile(v, 99)), 3)}
                             for k, v in parts.items()},
        "throughput_req_s": round(len(res) / span, 1),
        "value": round(vt / span / 1e9, 2),
        "unit": UNIT,
        "rate_hz": round(rate, 1),
        "load": cfg["load"],
        "burst_capacity_req_s": round(capacity, 1),
        "slots": cfg["slots"],
        "budget_gb": cfg["budget_gb"],
        "graph_replays": int(stats["graph_launches"]),
        "direct_runs": int(stats["direct_launches"]),
        "plans_created": int(stats["plans_created"]),
        "plans_evicted": int(stats["plans_evicted"]),
        "peak_in_flight": int(stats["peak_in_flight"]),
        "failed": int(stats["failed"]),
        "inputs": ("one seeded blob-phantom series per (size, tilts), reused with each "
                   "request's own defocus, ndf and staging; latency from the scheduled arrival "
                   "to the volume in page-locked host memory"),
    }


def cpu_inputs(proj=None):
    """The CPU arms' inputs: the oracle's CTF stack and slab range for the
    workload, and the projections (the bench's own, or a seeded stand-in of
    the same shape: the oracle's run time does not depend on the values)."""
    from oracle import oracle as O

    c, mn, mx, step, nd = slab_setup()
    df = WL["defocus"]
    ctf = (O.ctf_stack(WL["W"], WL["H"], WL["pixel_size"], WL["energy"], mn, nd, step,
                       WL["cs_mm"]) if WL["ctf"] else None)
    if ctf is None:
        mn = mx = df
    if proj is None:
        rng = np.random.default_rng(WL["seed"])
        proj = rng.standard_normal((WL["T"], WL["H"], WL["W"])).astype(np.float32)
    return proj, c, ctf, float(mn - df), float(mx - df)


def cpu_sample(p, c, ctf, rel_mn, rel_mx, threads):
    """One bounded sample of the reference's CPU algorithm (the float oracle,
    OpenMP on `threads` host threads): CTF correction of min(T, threads) tilts
    (one per thread) and ramp filter + backprojection of `threads` Y rows (one
    per thread) of every tilt.  Returns the measured sample time and the whole
    series' time extrapolated from it (correction scales with the tilts, the
    rest with the rows)."""
    from oracle import oracle as O

    ang = angles_rad()
    kt = min(WL["T"], threads)
    nrows = min(WL["H"], threads)
    y0 = WL["H"] // 2 - nrows // 2
    t0 = time.perf_counter()
    if ctf is not None:
        O.fbp_ctf(p, ang, c, WL["pixel_size"], ctf, rel_mn, rel_mx, Z=WL["Z"], rows=(0, 0),
                  tilts=(0, kt), nthreads=threads)
    t1 = time.perf_counter()
    O.fbp_ctf(p, ang, c, WL["pixel_size"], ctf, rel_mn, rel_mx, Z=WL["Z"],
              rows=(y0, y0 + nrows), tilts=(0, 0), nthreads=threads)
    t2 = time.perf_counter()
    series = (t1 - t0) * WL["T"] / kt + (t2 - t1) * WL["H"] / nrows
    desc = ((f"CTF correction of {kt} of {WL['T']} tilts ({t1 - t0:.2f} s) and " if ctf is not None
             else "") + f"ramp filter + backprojection of {nrows} of {WL['H']} rows "
            f"({t2 - t1:.2f} s) on {threads} threads, extrapolated to the whole series")
    return t2 - t0, series, desc


def oracle_sample(proj, vols):
    """Parity of both GPU forms against the FP32 and FP64 oracles on a band of
    rows of the same series (every tilt corrected), and the CPU baseline: one
    cpu_sample of the reference's algorithm, as the reference arm times it."""
    from oracle import oracle as O

    threads = os.cpu_count() or 1
    p, c, ctf, rel_mn, rel_mx = cpu_inputs(proj.cpu().numpy())
    ang = angles_rad()
    nrows = 8
    y0 = WL["H"] // 2 - nrows // 2
    rows = (y0, y0 + nrows)
    v32 = O.fbp_ctf(p, ang, c, WL["pixel_size"], ctf, rel_mn, rel_mx, Z=WL["Z"], rows=rows,
                    nthreads=threads)
    v64 = O.fbp_ctf(p, ang, c, WL["pixel_size"], ctf, rel_mn, rel_mx, Z=WL["Z"], rows=rows,
                    precision="f64", nthreads=threads)
    sl = slice(*rows)
    r64 = v64[sl]
    r32 = v32[sl]

    def rel(a, b):
        return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))

    g32 = vols["f32"][sl].cpu().numpy()
    g16 = vols["f16"][sl].cpu().numpy()
    g16t = vols["f16t"][sl].cpu().numpy()
    parity = {
        "rows_sampled": list(rows),
        "f32_vs_reference_cpu_rel_l2": rel(g32, r32),
        "f32_vs_fp64_oracle_rel_l2": rel(g32, r64),
        "f16_vs_fp64_oracle_rel_l2": rel(g16, r64),
        "f16t_vs_fp64_oracle_rel_l2": rel(g16t, r64),
        "f32_max_abs_vs_fp64": float(np.abs(g32 - r64).max()),
        "reference_cpu_vs_fp64_rel_l2": rel(r32, r64),
    }
    sample_s, series_s, desc = cpu_sample(p, c, ctf, rel_mn, rel_mx, threads)
    cpu = {
        "value": round(voxel_tilts() / series_s / 1e9, 4),
        "unit": UNIT,
        "cores": threads,
        "kind": "port",
        "sample_ms": round(sample_s * 1e3, 1),
        "series_ms_extrapolated": round(series_s * 1e3, 1),
        "sample": "oracle restatement of the reference CPU path (float): " + desc,
    }
    return parity, cpu


# ------------------------------------------------------------ reference arm
def run_reference(args, rank, world):
    if rank != 0:
        return
    import guanaco_gb300 as G  # noqa: F401  (host helpers only: defocus steps)

    threads = os.cpu_count() or 1
    p, c, ctf, rel_mn, rel_mx = cpu_inputs()
    for _ in range(args.warmup):
        cpu_sample(p, c, ctf, rel_mn, rel_mx, threads)
    runs = [cpu_sample(p, c, ctf, rel_mn, rel_mx, threads) for _ in range(args.steps)]
    sample_s = sum(r[0] for r in runs) / len(runs)
    series_s = sum(r[1] for r in runs) / len(runs)
    value = voxel_tilts() / series_s / 1e9
    line = {
        "metric": METRIC, "value": round(value, 4), "unit": UNIT, "impl": "reference",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(sample_s * 1e3, 2),
        "series_ms_extrapolated": round(series_s * 1e3, 2),
        "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded, workload shape)",
        "config": {"workload": WORKLOAD_NAME, "tilts": WL["T"],
                   "projection": [WL["H"], WL["W"]], "volume": [WL["H"], WL["W"], WL["Z"]],
                   "ndf": WL["D"], "staging": "f32", "parallelism": "host threads"},
        "cpu_baseline": {
            "value": round(value, 4), "unit": UNIT, "cores": threads, "kind": "port",
            "sample_ms": round(sample_s * 1e3, 1),
            "series_ms_extrapolated": round(series_s * 1e3, 1),
            "sample": ("per step, one bounded sample: " + runs[-1][2] + "; value = the series' "
                       "voxel-tilts over the extrapolated series time; oracle restatement of "
                       "the reference CPU path (the reference itself needs FFTW and its source "
                       "tree, absent on this host)"),
        },
        "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu", action="store_true", help="skip the oracle parity/CPU sample")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving stream")
    ap.add_argument("--case", choices=["3dctf", "profile", "large", "large_profile",
                                       "plain_256", "single_defocus_512"],
                    default="3dctf",
                    help="profile: the same 1024^2 ndf=10 kernels on 16 tilts and a 64-voxel-"
                         "thick volume, small enough for ncu captures (not a bench line); "
                         "large: 4096^2 projections, ndf=20, 4096x4096x512 volume in one "
                         "HBM pass; large_profile: the 4096^2 kernels on 2 tilts, ndf=10 and "
                         "a 16-voxel-thick volume, for ncu captures (not a bench line); "
                         "plain_256: FBP without CTF, 61 tilts of 256^2 (step 2 deg), "
                         "256x256x128 volume; single_defocus_512: CTF phase flip, one defocus "
                         "(20000 A), 41 tilts of 512^2 (step 3 deg) at 1.35 A/px, "
                         "512x512x256 volume")
    args = ap.parse_args()
    global WORKLOAD_NAME
    if args.case == "large":
        WL.update(T=61, H=4096, W=4096, Z=512, D=20, pixel_size=0.8, defocus=40000.0,
                  blobs=20000, seed=4)
        WORKLOAD_NAME = ("large 3D CTF ndf=20: 61 tilts +-60 deg, 4096x4096 projections at "
                         "0.8 A/px, 300 kV, Cs 2.7 mm, df 40000 A, volume 4096x4096x512")
        args.no_cpu = True
        args.no_serve = True
    if args.case == "plain_256":
        WL.update(T=61, H=256, W=256, Z=128, D=1, pixel_size=1.0, blobs=200, noise=0.05,
                  seed=0, ctf=False)
        WORKLOAD_NAME = ("plain FBP, no CTF: 61 tilts +-60 deg (2 deg steps), 256x256 projections "
                         "at 1.0 A/px, volume 256x256x128")
        args.no_serve = True
    if args.case == "single_defocus_512":
        WL.update(T=41, H=512, W=512, Z=256, D=1, pixel_size=1.35, defocus=20000.0, blobs=500,
                  noise=0.1, seed=1)
        WORKLOAD_NAME = ("single-defocus CTF phase flip: 41 tilts +-60 deg (3 deg steps), "
                         "512x512 projections at 1.35 A/px, 300 kV, Cs 2.7 mm, df 20000 A "
                         "(amplitude contrast not modelled: the phase flip uses the sign of "
                         "the phase-only CTF), volume 512x512x256")
        args.no_serve = True
    if args.case == "large_profile":
        WL.update(T=2, H=4096, W=4096, Z=16, D=10, pixel_size=0.8, defocus=40000.0,
                  blobs=200, seed=4)
        WORKLOAD_NAME = ("profiling case: 2 tilts, 4096x4096 projections at 0.8 A/px, ndf=10, "
                         "df 40000 A, volume 4096x4096x16")
        args.no_cpu = True
        args.no_serve = True
    if args.case == "profile":
        WL.update(T=16, Z=64, blobs=200)
        args.no_serve = True
        WORKLOAD_NAME = "profiling case: " + WORKLOAD_NAME.replace("61 tilts", "16 tilts").replace(
            "x300", "x64")
        args.no_cpu = True
    args.warmup = max(args.warmup, 3)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    dist = None
    if world > 1:
        import torch
        import torch.distributed as tdist

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        tdist.init_process_group("nccl")
        dist = tdist
    try:
        run_ours(args, rank, world, dist)
    finally:
        if dist is not None:
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
