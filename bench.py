"""Benchmark: power spectra per second of the 512^3 CIC workload on GB300.

One step = one pass of the hot path over one particle set: zero the grid,
CIC deposit of 134,217,728 particles onto a 512^3 float32 grid, r2c FFT,
window deconvolution, |delta_k|^2, Legendre ell=0,2,4 and integer-|k|
binning, and the float64 per-bin sums back on the host (k3D, Pk[:,0:3],
Nmodes3D) -- pyl_pk_particles, the reference's canonical
MA -> delta/mean-1 -> Pk caller (Pk_snapshot.py:81-89) in one call.

  value  spectra/s with the positions resident in HBM (device-timed).
  e2e    the same metric through the public API power_spectrum() with the
         positions in pinned host memory: every step copies them to the
         device and reads the spectrum back.
  roofline  the dominant kernel's algorithmic bytes per launch / its mean
         CUDA-event duration, against the measured HBM copy bandwidth.
  cpu_baseline  the reference's CPU path (oracle port: OpenMP atomic deposit
         as MAS_c.c, scipy FFT on all cores as FFTW threads, the serial mode
         loop of Pk) on a bounded sample of the same workload.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Under torchrun (N > 1) every rank runs its own replica (no data exchange);
value is the sum over ranks, timed as the max over ranks.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BOX = 1000.0
METRIC = "P(k)/s @512^3 CIC"
UNIT = "spectra/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mode", default="plain",
                    choices=["plain", "batched", "served", "precision"],
                    help="plain: the headline line; batched: 64 uneven realizations "
                         "overlapped; served: Poisson request streams")
    ap.add_argument("--slots", type=int, default=None,
                    help="contexts in flight (default: 2 batched, 8 served)")
    ap.add_argument("--rates", type=float, nargs="*", default=[50.0, 200.0, 500.0])
    ap.add_argument("--seconds", type=float, default=5.0)
    ap.add_argument("--dims", type=int, default=512)
    ap.add_argument("--particles", type=int, default=512 ** 3)
    ap.add_argument("--mas", default="CIC")
    ap.add_argument("--axis", type=int, default=0)
    ap.add_argument("--positions", default="uniform", choices=["uniform", "zeldovich"])
    ap.add_argument("--sort", default="auto", choices=["auto", "frontier", "two_pass"],
                    help="tile sort of the deposit: chosen on the device from the input "
                         "order (auto), one pass with per-tile cursors, or two staged "
                         "partition passes")
    ap.add_argument("--halos", type=float, default=0.1,
                    help="precision mode: extra fraction of particles in Plummer halos")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--out-dir", default=None,
                    help="precision mode: folder for the per-bin error arrays (.npy)")
    ap.add_argument("--cpu-sample", type=int, default=16,
                    help="CPU baseline runs 1/this of the particles and of the mode loop")
    return ap.parse_args()


def l2_note(a):
    """Whether the step's inputs exceed the 129 MB L2 (then no flush is
    needed between timed steps)."""
    pos_gb, grid_gb = a.particles * 12 / 1e9, 4 * a.dims ** 3 / 1e9
    if pos_gb + grid_gb > 0.129:
        return "inputs larger than L2 (positions %.2f GB, grid %.2f GB) -- no flush" % (pos_gb, grid_gb)
    return ("inputs smaller than L2 (positions %.4f GB, grid %.4f GB): timed steps reuse L2"
            % (pos_gb, grid_gb))


def workload(a):
    return {
        "workload": "%d^3 grid, %d %s particles, %s deposit + %s window, axis %d, "
                    "BoxSize %g" % (a.dims, a.particles, a.positions, a.mas, a.mas, a.axis, BOX),
        "dims": a.dims, "particles": a.particles, "positions": a.positions,
        "mas": a.mas, "axis": a.axis, "box": BOX, "sort": a.sort,
        "l2": l2_note(a),
    }


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# Replicas: every rank runs its own spectra on its own seeded particles; no
# data crosses ranks.  The only collective is the max of the per-rank times.
def replica_seed(rank):
    return 1234 + rank


def max_over_ranks(value, world, device):
    """Max over the ranks of a per-rank time (identity for one rank)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(world, steps, seconds):
    """Whole-job spectra/s: every rank's steps over the slowest rank's time."""
    return world * steps / seconds


# ------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        import tempfile
        self.path = os.path.join(tempfile.gettempdir(), "pyl_clocks_%d.csv" % os.getpid())

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


# -------------------------------------------------------------- roofline
def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def stage_bytes(stage, dims, n, weighted):
    """Algorithmic HBM bytes per launch of each stage."""
    h = dims // 2 + 1
    real = 4 * dims ** 3
    half = 8 * dims * dims * h
    rec = n * (12 + (4 if weighted else 0))   # one particle record (+ weight)
    return {
        "tile_count": n * 12,        # read positions
        "partition": 2 * rec,        # read + write every record once (a one-pass partition)
        "deposit": rec + real,       # read the sorted records, write the grid once
        "mass": n * 4 if weighted else 0,
        "fft_z": real + half,        # read real grid, write half-complex
        "fft_y": 2 * half,           # read + write
        "pk_x": half,                # read only (spectrum not stored)
        "zero": real,
    }.get(stage)


def traffic_table():
    """dram bytes per launch per stage from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    out = {}
    if os.path.exists(p):
        for line in open(p):
            line = line.split("#")[0].split()
            if len(line) >= 3:
                out[(line[0], line[1])] = float(line[2])
    return out


# ------------------------------------------------------------ CPU baseline
def cpu_sample(a, pos_np, threads):
    """Reference CPU path on a bounded sample: returns seconds per spectrum
    (extrapolated) and a description."""
    import numpy as np
    from oracle import oracle as orc
    dims, S = a.dims, a.cpu_sample
    n = pos_np.shape[0]
    ns = n // S
    grid = np.zeros((dims,) * 3, np.float32)
    t0 = time.perf_counter()
    orc.deposit_omp(a.mas, pos_np[:ns], grid, BOX, threads=threads)
    t_dep = (time.perf_counter() - t0) * S
    # the sampled grid stands in for the full one in the steps below
    t0 = time.perf_counter()
    grid /= np.mean(grid, dtype=np.float64)
    grid -= 1.0
    t_norm = time.perf_counter() - t0
    t0 = time.perf_counter()
    dk = orc.FFT3Dr_f(grid, threads)
    t_fft = time.perf_counter() - t0
    rows = max(1, dims // S)
    t0 = time.perf_counter()
    orc.Pk(None, BOX, axis=a.axis, MAS=a.mas, delta_k=dk, rows=(0, rows))
    t_bin = (time.perf_counter() - t0) * dims / rows
    total = t_dep + t_norm + t_fft + t_bin
    desc = ("oracle port on %d threads: OpenMP atomic deposit of 1/%d of the particles "
            "(x%d), overdensity + scipy r2c FFT of the full grid, serial mode loop over "
            "%d of %d kx planes (x%d); per-spectrum %.2f s = deposit %.2f + norm %.2f + "
            "fft %.2f + bin %.2f" % (threads, S, S, rows, dims, dims // rows, total, t_dep,
                                     t_norm, t_fft, t_bin))
    return total, desc


def host_positions(a, seed=1234):
    import numpy as np
    rng = np.random.default_rng(seed)
    pos = rng.random((a.particles, 3), dtype=np.float32)
    pos *= np.float32(BOX)
    np.minimum(pos, np.nextafter(np.float32(BOX), np.float32(0)), out=pos)
    return pos


# ----------------------------------------------------------------- arms
def run_reference(a):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as orc
    orc.build()
    threads = os.cpu_count() or 1
    pos = host_positions(a)
    times = []
    desc = ""
    for i in range(a.warmup + a.steps):
        t, desc = cpu_sample(a, pos, threads)
        if i >= a.warmup:
            times.append(t)
    sec = sum(times) / len(times)
    value = 1.0 / sec
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded uniform positions)",
        "config": workload(a),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": desc},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(a):
    import numpy as np
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from pylians3_gb300 import build_native
    build_native.build()
    import pylians3_gb300 as P
    from pylians3_gb300 import _native, synth
    from pylians3_gb300.Pk_library import _Outputs, MAS_function
    import ctypes

    ctx = _native.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    if a.positions == "uniform":
        pos = synth.uniform(a.particles, BOX, seed=replica_seed(rank))
    else:
        pos = synth.zeldovich(a.dims, BOX, sigma=3.0, seed=replica_seed(rank))
        a.particles = pos.shape[0]
    torch.cuda.synchronize()
    out = _Outputs(a.dims, 0)
    mas = _native.MAS_CODE[a.mas]
    win = MAS_function(a.mas)

    flags = _native.PYL_DEVICE_PTRS | {"auto": 0, "frontier": _native.PYL_SORT_FRONTIER,
                                       "two_pass": _native.PYL_SORT_TWO_PASS}[a.sort]

    def step():
        rc = ctx.lib.pyl_pk_particles(ctx.ptr, ctypes.c_void_p(pos.data_ptr()), a.particles,
                                      None, a.dims, ctypes.c_float(BOX), mas, a.axis, win, 0,
                                      ctypes.byref(out.struct), flags)
        ctx.check(rc)

    for _ in range(a.warmup):
        step()
    ctx.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()
        ctx.synchronize()

    clocks = ClockSampler(local)
    barrier()
    ctx.stage_times(reset=True)
    ctx.set_timing(True)
    l0 = ctx.launches()
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(a.steps):
        step()
    e1.record(stream)
    e1.synchronize()
    clk = clocks.stop()
    launches = ctx.launches() - l0
    stages = ctx.stage_times(reset=True)
    ctx.set_timing(False)
    barrier()
    ms = max_over_ranks(e0.elapsed_time(e1), world, "cuda")
    ms_step = ms / a.steps
    value = job_rate(world, a.steps, ms / 1e3)

    # ---- roofline of the dominant kernel
    peak, peak_kind = peaks()
    kern = {k: v for k, v in stages.items() if k not in ("h2d", "d2h")}
    dom = max(kern, key=lambda k: kern[k][0])
    dom_ms = kern[dom][0] / kern[dom][1]
    algo = stage_bytes(dom, a.dims, a.particles, False)
    achieved = algo / (dom_ms / 1e3) / 1e9
    tr = traffic_table().get((dom, "%s_%d_%s" % (a.mas, a.dims, a.positions)))
    roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)"
            if peak_kind == "measured" else "fallback 6.8 TB/s",
            "traffic": tr, "algorithmic_bytes_per_launch": algo, "ms_per_launch": dom_ms}
    h = a.dims // 2 + 1
    pipe_bytes = (a.particles * 12 + 4 * a.dims ** 3 + 4 * a.dims ** 3 + 2 * 8 * a.dims ** 2 * h)
    stage_ms = {k: v[0] / a.steps for k, v in stages.items()}

    # ---- end to end through the public API with pinned host positions
    e2e = None
    if not a.no_e2e:
        host = P.pinned_empty((a.particles, 3), np.float32)
        host[...] = pos.cpu().numpy()
        for _ in range(2):
            P.power_spectrum(host, a.dims, BOX, a.mas, axis=a.axis, ctx=ctx)
        barrier()
        # one call at a time: copy, compute, read back, then the next
        t0 = time.perf_counter()
        for _ in range(a.steps):
            P.power_spectrum(host, a.dims, BOX, a.mas, axis=a.axis, ctx=ctx)
        single = max_over_ranks(time.perf_counter() - t0, world, "cuda")
        # the public batched call: each step's positions go host -> device
        # while the previous step computes (two contexts in flight)
        P.power_spectra([host] * 2, a.dims, BOX, a.mas, axis=a.axis)
        barrier()
        t0 = time.perf_counter()
        P.power_spectra([host] * a.steps, a.dims, BOX, a.mas, axis=a.axis)
        t1 = time.perf_counter()
        sec = max_over_ranks(t1 - t0, world, "cuda")
        kmax = _native.pk_sizes(a.dims)[0]
        e2e = {"value": job_rate(world, a.steps, sec), "unit": UNIT,
               "h2d_bytes_per_step": a.particles * 12,
               "d2h_bytes_per_step": 8 * (5 * (kmax + 1)),
               "ms_per_step": sec / a.steps * 1e3,
               "api": "pylians3_gb300.power_spectra, pinned host positions, 2 sets in flight",
               "single_call_value": job_rate(world, a.steps, single),
               "single_call_api": "pylians3_gb300.power_spectrum, one call at a time"}
        del host

    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        from oracle import oracle as orc
        orc.build()
        threads = os.cpu_count() or 1
        pos_np = pos.cpu().numpy()
        cpu_sample(a, pos_np, threads)   # warm-up (page faults, thread pools)
        t, desc = cpu_sample(a, pos_np, threads)
        cpu = {"value": 1.0 / t, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": desc}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded %s positions, generated on the device)"
                                     % a.positions,
            "config": workload(a), "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
            "clocks": clk, "gpu_launches": launches,
            "stages_ms_per_step": stage_ms,
            "pipeline_algorithmic_bytes": pipe_bytes,
            "pipeline_frac": pipe_bytes / (ms_step / 1e3) / 1e9 / peak,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


# ------------------------------------------------ batched and served forms
def batched_requests(torch, seed=4242, count=64):
    """64 realizations of uneven size: dims in {128, 192, 256, 384},
    particles log-uniform in [2^20, 2^25], uniform or Zel'dovich (sigma 2-5
    Mpc/h) positions, optional lognormal(0, 0.5) weights, CIC or TSC."""
    import numpy as np
    from pylians3_gb300 import synth
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(count):
        dims = int(rng.choice([128, 192, 256, 384]))
        n = int(2 ** rng.uniform(20, 25))
        if rng.random() < 0.5:
            pos = synth.uniform(n, BOX, seed=seed + i)
        else:
            side = max(2, int(round(n ** (1.0 / 3.0))))
            pos = synth.zeldovich(side, BOX, sigma=float(rng.uniform(2, 5)), seed=seed + i)
        W = None
        if rng.random() < 0.5:
            g = torch.Generator(device="cuda").manual_seed(seed + 1000 + i)
            W = torch.exp(0.5 * torch.randn(pos.shape[0], generator=g, device="cuda"))
        reqs.append(dict(pos=pos, dims=dims, BoxSize=BOX, W=W,
                         MAS=str(rng.choice(["CIC", "TSC"])), axis=int(rng.integers(0, 3))))
    torch.cuda.synchronize()
    return reqs


def run_batched(a):
    import torch
    import pylians3_gb300 as P
    from pylians3_gb300.serving import run_batch
    reqs = batched_requests(torch)
    # autotune the deposit's tile shape and sort granularity per (dims, MAS)
    # at the median particle count of the batch's requests of that kind
    import numpy as np
    from pylians3_gb300 import autotune
    tuned = {}
    groups = {}
    for r in reqs:
        groups.setdefault((r["dims"], r["MAS"]), []).append(int(r["pos"].shape[0]))
    for (dims, mas), ns in sorted(groups.items()):
        default = autotune.current_shape(dims, mas)
        shape, times = autotune.tune(dims, mas, int(np.median(ns)), use_cache=False)
        tuned["%d/%s" % (dims, mas)] = {"shape": list(shape), "default": list(default),
                                        "ms": times.get(shape), "default_ms": times.get(default)}
    for r in reqs[:4]:
        P.power_spectrum(**r)          # plans, mode tables
    ctx = P.context(0)
    for r in reqs:
        P.power_spectrum(**r, ctx=ctx)  # warm every shape once
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for r in reqs:
        P.power_spectrum(**r, ctx=ctx)
    t_seq = time.perf_counter() - t0
    slots = a.slots or 2      # measured best for this mix (1: 1152, 2: 1392, 4: 1339, 8: 1216/s)
    run_batch(reqs, slots=slots)                   # warm the slots
    res, t_srv = run_batch(reqs, slots=slots)
    # the whole batch as one CUDA graph (captured on the first call)
    from pylians3_gb300.pipeline import spectra_batch
    spectra_batch(reqs, ctx=ctx)
    spectra_batch(reqs, ctx=ctx)
    t0 = time.perf_counter()
    reps = 3
    for _ in range(reps):
        spectra_batch(reqs, ctx=ctx)
    t_graph = (time.perf_counter() - t0) / reps
    line = {"mode": "batched", "metric": "realizations/s (64 uneven realizations)",
            "value": len(reqs) / t_graph, "unit": "spectra/s",
            "api": "pipeline.spectra_batch: the 64 requests as one CUDA graph launch",
            "sequential_value": len(reqs) / t_seq, "speedup": t_seq / t_graph,
            "server_value": len(reqs) / t_srv, "server_slots": slots,
            "autotune": tuned,
            "particles_total": int(sum(r["pos"].shape[0] for r in reqs)),
            "config": {"dims": "U{128,192,256,384}", "particles": "2^U(20,25)",
                       "positions": "uniform | zeldovich sigma U(2,5)", "W": "lognormal(0,0.5) half",
                       "mas": "U{CIC,TSC}"}}
    print(json.dumps(line), flush=True)


def served_pool(torch, max_ppc=8):
    """Device-resident particle pools, one per grid size, 8 particles/cell."""
    from pylians3_gb300 import synth
    return {d: synth.uniform(max_ppc * d ** 3, BOX, seed=77 + d) for d in (64, 128, 256, 512)}


def run_served(a):
    import numpy as np
    import torch
    import pylians3_gb300 as P
    from pylians3_gb300.serving import Server
    pool = served_pool(torch)
    torch.cuda.synchronize()

    def stream(rate, seconds, seed):
        rng = np.random.default_rng(seed)
        t, out = 0.0, []
        while True:
            t += rng.exponential(1.0 / rate)
            if t > seconds:
                return out
            d = int(rng.choice([64, 128, 256, 512], p=[0.3, 0.3, 0.3, 0.1]))
            n = int(rng.integers(1, 9)) * d ** 3
            off = int(rng.integers(0, pool[d].shape[0] - n + 1))
            out.append((t, dict(pos=pool[d][off:off + n], dims=d, BoxSize=BOX,
                                MAS=str(rng.choice(["NGP", "CIC", "TSC", "PCS"])),
                                axis=int(rng.integers(0, 3)))))

    # warm the plans and mode tables of every (dims, axis)
    for d in (64, 128, 256, 512):
        for ax in range(3):
            P.power_spectrum(pool[d][:d ** 3], d, BOX, "CIC", axis=ax)
    results = []
    for rate in a.rates:
        reqs = stream(rate, a.seconds, seed=int(rate))
        row = {"rate": rate, "requests": len(reqs)}
        for name, slots in (("served", a.slots or 8), ("queue_only", 1)):
            srv = Server(slots=slots, hbm_budget=150e9)
            t0 = time.perf_counter()
            futs = []
            for t_arr, r in reqs:
                now = time.perf_counter() - t0
                if t_arr > now:
                    time.sleep(t_arr - now)
                futs.append(srv.submit(**r))
            for f in futs:
                f.result()
            wall = time.perf_counter() - t0
            lat = srv.latencies()
            srv.close()
            row[name] = {"spectra_per_s": len(reqs) / wall,
                         "p50_ms": float(np.percentile(lat, 50) * 1e3),
                         "p99_ms": float(np.percentile(lat, 99) * 1e3), "wall_s": wall}
        results.append(row)
    line = {"mode": "served", "metric": "spectra/s and latency under Poisson arrivals",
            "slots": a.slots or 8, "seconds_per_rate": a.seconds, "rates": results,
            "config": {"dims": "{64,128,256,512} p=(.3,.3,.3,.1)", "particles_per_cell": "U{1..8}",
                       "mas": "U{NGP,CIC,TSC,PCS}", "axis": "U{0,1,2}",
                       "positions": "device-resident uniform pools", "hbm_budget_gb": 150}}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------- precision
def run_precision(a):
    """Accuracy of the float32 pipeline variants against the float64 oracle
    on the precision workload: a Zel'dovich lattice (sigma 3 Mpc/h, RSD) on
    dims^3 plus 10% extra particles in 1000 Plummer halos (scale 0.5 Mpc/h),
    deposited with a.mas.  Variants: the default deposit (fixed-point tiles),
    float32 shared atomics, the compensated deposit, and a float64 GPU grid
    (pyl_ma_f64) through the float32 FFT and binning (isolates the FFT).
    The oracle: float64 deposit on all host cores, float64 FFT, float64
    binning.  Per bin, err = max over ell of |P_ell - P_ell^64| / |P_0^64|."""
    import numpy as np
    import torch
    from pylians3_gb300 import build_native
    build_native.build()
    import pylians3_gb300 as P
    from pylians3_gb300 import synth
    from oracle import oracle as orc
    dims = a.dims
    lattice = synth.zeldovich(dims, BOX, sigma=3.0, seed=2027)
    nh = int(lattice.shape[0] * a.halos)
    if nh:
        halos = synth.plummer_halos(nh, 1000, 0.5, BOX, seed=2028)
        pos = torch.cat([lattice, halos])
        del halos
    else:
        pos = lattice
    del lattice
    n = int(pos.shape[0])
    torch.cuda.synchronize()
    spectra, secs = {}, {}
    for name, dep in (("fixed_point_tiles", "auto"), ("float32_atomics", "float"),
                      ("compensated", "compensated")):
        P.power_spectrum(pos, dims, BOX, a.mas, axis=a.axis, deposit=dep)   # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        spectra[name] = P.power_spectrum(pos, dims, BOX, a.mas, axis=a.axis, deposit=dep).Pk
        secs[name] = time.perf_counter() - t0
    g64 = torch.zeros((dims,) * 3, dtype=torch.float64, device="cuda")
    P.MAS_library._deposit(pos, g64, BOX, a.mas, None, 3, True, "float64")
    d = (g64 / g64.mean() - 1.0).to(torch.float32)
    del g64
    spectra["float64_grid_float32_fft"] = P.Pk_library.Pk(d, BOX, axis=a.axis, MAS=a.mas,
                                                         verbose=False).Pk
    del d
    pos_np = pos.cpu().numpy()
    del pos
    torch.cuda.empty_cache()
    t0 = time.perf_counter()
    threads = os.cpu_count() or 1
    grid = orc.MA_f64(pos_np, dims, BOX, a.mas, threads=0)
    del pos_np
    grid /= grid.mean()
    grid -= 1.0
    ref = orc.Pk_f64(grid, BOX, axis=a.axis, MAS=a.mas, threads=threads)
    t_oracle = time.perf_counter() - t0
    del grid
    mid = dims // 2
    rows = {}
    for name, pk in spectra.items():
        err = np.abs(pk - ref.Pk).max(axis=1) / np.abs(ref.Pk[:, 0])
        rows[name] = {
            "max_err_k_le_nyquist": float(err[:mid].max()),
            "median_err_k_le_nyquist": float(np.median(err[:mid])),
            "max_err_all_bins": float(err.max()),
            "bins_over_1e-4": int((err > 1e-4).sum()),
            "seconds": secs.get(name)}
        if a.out_dir:
            np.save(os.path.join(a.out_dir, "precision_err_%s_%s_%d_h%g.npy"
                                 % (name, a.mas, dims, a.halos)), err)
    line = {"mode": "precision", "metric": "per-bin error of P_ell vs the float64 oracle",
            "unit": "max over ell |dP_ell| / |P_0|, per bin", "bins": int(len(ref.Pk)),
            "nyquist_bin": mid, "variants": rows, "oracle_seconds": t_oracle,
            "config": {"workload": "%d^3 Zel'dovich lattice (sigma 3 Mpc/h, RSD) + %g%% in 1000 "
                                   "Plummer halos (a = 0.5 Mpc/h), %s deposit + window, axis %d"
                                   % (dims, 100 * a.halos, a.mas, a.axis),
                       "particles": n, "dims": dims, "mas": a.mas, "axis": a.axis,
                       "oracle": "float64 deposit (all host cores), float64 FFT, float64 sums"}}
    print(json.dumps(line), flush=True)


def main():
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    elif a.mode == "precision":
        if a.out_dir:
            os.makedirs(a.out_dir, exist_ok=True)
        run_precision(a)
    elif a.mode == "batched":
        run_batched(a)
    elif a.mode == "served":
        run_served(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
