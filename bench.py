"""Benchmark: power spectra per second of the 512^3 CIC workload on GB300.

One step = one pass of the hot path over one particle set: zero the grid,
CIC deposit of 134,217,728 particles onto a 512^3 float32 grid, r2c FFT,
window deconvolution, |delta_k|^2, Legendre ell=0,2,4 and integer-|k|
binning, and the float64 per-bin sums back on the host (k3D, Pk[:,0:3],
Nmodes3D) -- pyl_pk_particles, the reference's canonical
MA -> delta/mean-1 -> Pk caller (Pk_snapshot.py:81-89) in one call.

  value     spectra/s with the positions resident in HBM (device-timed).
  e2e       the same metric through the public API with the positions in
            pinned host memory: every step copies them to the device and
            reads the spectrum back (power_spectra, two sets in flight).
  roofline  one whole spectrum: the algorithmic bytes of the hot path per
            spectrum (12 n + 4 d^3 + 4 d^3 + 16 d^2 (d/2+1): positions read
            once, grid written once and read once, half-complex grid written
            once and read once; the sort counts as no useful bytes) over the
            CUDA-event time of a step, against the measured HBM copy
            bandwidth.  `stages` breaks it down per stage.
  headline  the metric's comparison on one request stream of 512^3 CIC
            spectra from host memory: the plain path (the drop-in MA, numpy
            delta/mean - 1 and the drop-in Pk, one request at a time, as
            Pk_snapshot.py:66-89 does) against the batched (power_spectra)
            and served (serving.Server) forms, with p50/p99 latency.
  batched   64 realizations of uneven size (dims 128..384): one at a time vs
            one CUDA-graph launch vs the server.
  served    Poisson request streams of the mixed served workload.
  cpu_baseline  one full spectrum of the reference's own CPU code (compiled
            for this machine from oracle/_ref/kit: serial MA, overdensity,
            Pk on all cores), or of the oracle port where it is unavailable.

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
    ap.add_argument("--no-extras", action="store_true",
                    help="leave the headline, batched and served sub-objects out")
    ap.add_argument("--headline-requests", type=int, default=16,
                    help="requests in the headline stream (plain vs batched vs served)")
    ap.add_argument("--ref-budget", type=float, default=150.0,
                    help="reference arm: seconds of timed full spectra (at least one)")
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


def spectrum_bytes(dims, n, weighted=False):
    """Algorithmic HBM bytes of one spectrum: positions (and weights) read
    once, the grid written once and read once, the half-complex grid written
    once and read once (a two-pass FFT lower bound).  Bins and the sort are
    left out: the sort moves no useful bytes."""
    h = dims // 2 + 1
    return n * (12 + (4 if weighted else 0)) + 8 * dims ** 3 + 16 * dims * dims * h


def stage_bytes(stage, dims, n, weighted):
    """(useful, moved) HBM bytes per launch of each stage.  useful: the
    stage's share of spectrum_bytes (they add up to it); moved: the least
    traffic of the stage as built (e.g. the y pass reads and writes the
    half-complex grid, the sort reads and writes every record)."""
    h = dims // 2 + 1
    real = 4 * dims ** 3
    half = 8 * dims * dims * h
    rec = n * (12 + (4 if weighted else 0))   # one particle record (+ weight)
    return {
        "tile_count": (0, n * 12),       # counting pass of the sort
        "partition": (0, 4 * rec),       # two passes, each reads and writes every record
        "deposit": (rec + real, rec + real),
        "mass": (0, n * 4 if weighted else 0),
        "zero": (0, real),
        "fft_z": (real + half, real + half),
        "fft_y": (0, 2 * half),
        "pk_x": (half, half),            # read only (the spectrum is not stored)
        "h2d": (0, 0), "d2h": (0, 0),
    }.get(stage, (0, 0))


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
def reference_modules():
    """The reference's own MAS_library and Pk_library compiled for this
    machine (oracle/_ref; built from oracle/_ref/kit with gcc on first use),
    or (None, reason)."""
    try:
        from oracle import build_ref
        if not build_ref.built():
            if not build_ref.have_kit():
                return None, "no reference compile kit in oracle/_ref/kit"
            build_ref.build_from_kit()
        return build_ref.load(), None
    except Exception as e:  # the CPU baseline falls back to the oracle port
        return None, "reference build unavailable: %s" % str(e).splitlines()[0][:200]


def cpu_spectrum(a, pos_np, threads, mods):
    """One full spectrum of the reference's CPU path on all particles: a new
    grid, MA (serial by construction), delta /= mean; delta -= 1 and Pk on
    `threads` cores -- the sequence of Pk_snapshot.py:66-89.  mods: the
    compiled reference (MAS_library, Pk_library) or None for the oracle
    port.  Returns (seconds, per-step seconds)."""
    import numpy as np
    dims = a.dims
    t0 = time.perf_counter()
    delta = np.zeros((dims,) * 3, np.float32)
    if mods is not None:
        mods[0].MA(pos_np, delta, BOX, a.mas)
    else:
        from oracle import oracle as orc
        orc.MA(pos_np, delta, BOX, a.mas)
    t1 = time.perf_counter()
    mean = pos_np.shape[0] * 1.0 / dims ** 3
    delta /= mean
    delta -= 1.0
    t2 = time.perf_counter()
    if mods is not None:
        mods[1].Pk(delta, BOX, a.axis, a.mas, threads, False)
    else:
        from oracle import oracle as orc
        orc.Pk(delta, BOX, axis=a.axis, MAS=a.mas, threads=threads)
    t3 = time.perf_counter()
    return t3 - t0, {"ma": t1 - t0, "overdensity": t2 - t1, "pk": t3 - t2}


def cpu_kind(mods, why):
    if mods is not None:
        return "reference", ("the reference's MAS_library.MA (serial) + delta/mean - 1 + "
                             "Pk_library.Pk(threads=all cores), compiled for this machine "
                             "with setup.py's flags; pyFFTW replaced by scipy.fft (absent)")
    return "port", ("oracle port (%s): serial MA restatement + delta/mean - 1 + Pk "
                    "restatement, scipy FFT on all cores" % why)


def host_positions(a, seed=1234):
    import numpy as np
    rng = np.random.default_rng(seed)
    pos = rng.random((a.particles, 3), dtype=np.float32)
    pos *= np.float32(BOX)
    np.minimum(pos, np.nextafter(np.float32(BOX), np.float32(0)), out=pos)
    return pos


# ----------------------------------------------------------------- arms
def run_reference(a):
    """The reference's own CPU path on the same workload: full spectra (all
    particles, every mode), all host cores for Pk.  At most one warm-up
    spectrum, then full spectra until --ref-budget seconds are used (at
    least one): `steps` is the number timed."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import numpy as np
    threads = os.cpu_count() or 1
    mods, why = reference_modules()
    if mods is None:
        from oracle import oracle as orc
        orc.build()
    kind, desc = cpu_kind(mods, why)
    pos = host_positions(a)
    warm = min(a.warmup, 1)
    for _ in range(warm):
        cpu_spectrum(a, pos, threads, mods)
    times, parts = [], []
    while len(times) < max(1, a.steps):
        t, part = cpu_spectrum(a, pos, threads, mods)
        times.append(t)
        parts.append(part)
        if sum(times) >= a.ref_budget:
            break
    sec = sum(times) / len(times)
    value = 1.0 / sec
    split = {k: statistics.mean(p[k] for p in parts) for k in parts[0]}
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": a.gpus, "steps": len(times), "warmup": warm,
        "steps_requested": a.steps, "warmup_requested": a.warmup,
        "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded uniform positions)",
        "config": workload(a),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind,
                         "sample": "%d full spectra (all %d particles, all modes); %s; "
                                   "seconds per spectrum: MA %.2f, overdensity %.2f, Pk %.2f"
                                   % (len(times), a.particles, desc, split["ma"],
                                      split["overdensity"], split["pk"])},
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
    stages_raw = ctx.stage_times(reset=True)
    ctx.set_timing(False)
    barrier()
    ms = max_over_ranks(e0.elapsed_time(e1), world, "cuda")
    ms_step = ms / a.steps
    value = job_rate(world, a.steps, ms / 1e3)

    # ---- roofline of one whole spectrum, and per stage
    peak, peak_kind = peaks()
    weighted = False
    algo = spectrum_bytes(a.dims, a.particles, weighted)
    achieved = algo / (ms_step / 1e3) / 1e9
    tr_tab = traffic_table()
    key = "%s_%d_%s" % (a.mas, a.dims, a.positions)
    stages = {}
    for name, (tot, cnt) in stages_raw.items():
        useful, moved = stage_bytes(name, a.dims, a.particles, weighted)
        ms_st = tot / a.steps
        row = {"ms_per_step": ms_st, "launches_per_step": cnt / a.steps,
               "useful_bytes": useful, "moved_bytes": moved,
               "traffic": tr_tab.get((name, key))}
        if ms_st > 0:
            row["frac_useful"] = useful / (ms_st / 1e3) / 1e9 / peak
            row["frac_moved"] = moved / (ms_st / 1e3) / 1e9 / peak
        stages[name] = row
    traffic = None
    # whole-spectrum traffic from the committed per-stage figures, when they
    # cover every stage this run timed
    timed = [k for k, v in stages.items() if v["moved_bytes"]]
    if timed and all(tr_tab.get((k, key)) for k in timed):
        traffic = sum(tr_tab[(k, key)] for k in timed)
    one_pass = a.particles * 12 + 8 * a.dims ** 3
    roof = {"bound": "hbm", "kernel": "one spectrum (all kernels of a step)",
            "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_source": (peak_kind + " (MEASURED_PEAKS.json hbm_gbs)")
            if peak_kind == "measured" else "fallback 6.8 TB/s",
            "traffic": traffic, "algorithmic_bytes_per_spectrum": algo,
            "ms_per_spectrum": ms_step,
            "one_pass_bytes": one_pass,
            "one_pass_frac": one_pass / (ms_step / 1e3) / 1e9 / peak}

    # ---- end to end through the public API with pinned host positions
    e2e = None
    host = None
    if not a.no_e2e or (not a.no_extras and world == 1):
        host = P.pinned_empty((a.particles, 3), np.float32)
        host[...] = pos.cpu().numpy()
    if not a.no_e2e:
        for _ in range(2):
            P.power_spectrum(host, a.dims, BOX, a.mas, axis=a.axis, ctx=ctx)
        barrier()
        # one call at a time: copy, compute, read back, then the next
        t0 = time.perf_counter()
        for _ in range(a.steps):
            P.power_spectrum(host, a.dims, BOX, a.mas, axis=a.axis, ctx=ctx)
        single = max_over_ranks(time.perf_counter() - t0, world, "cuda")
        # the public batched call: each step's positions go host -> device
        # while the previous step computes (two contexts in flight); warmed
        # with a full-length pass, then the better of two timed passes
        P.power_spectra([host] * max(4, a.steps), a.dims, BOX, a.mas, axis=a.axis)
        passes = []
        for _ in range(2):
            barrier()
            t0 = time.perf_counter()
            P.power_spectra([host] * a.steps, a.dims, BOX, a.mas, axis=a.axis)
            passes.append(time.perf_counter() - t0)
        sec = max_over_ranks(min(passes), world, "cuda")
        kmax = _native.pk_sizes(a.dims)[0]
        e2e = {"value": job_rate(world, a.steps, sec), "unit": UNIT,
               "h2d_bytes_per_step": a.particles * 12,
               "d2h_bytes_per_step": 8 * (5 * (kmax + 1)),
               "ms_per_step": sec / a.steps * 1e3,
               "api": "pylians3_gb300.power_spectra, pinned host positions, 2 sets in flight "
                      "(the better of two timed passes)",
               "passes_ms_per_step": [p / a.steps * 1e3 for p in passes],
               "single_call_value": job_rate(world, a.steps, single),
               "single_call_api": "pylians3_gb300.power_spectrum, one call at a time"}

    headline = batched = served = None
    if not a.no_extras and world == 1:
        headline = headline_stream(a, P, host, value)
        del host
        host = None
        batched = batched_summary(a)
        served = served_summary(a)
    del host

    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        threads = os.cpu_count() or 1
        mods, why = reference_modules()
        if mods is None:
            from oracle import oracle as orc
            orc.build()
        kind, desc = cpu_kind(mods, why)
        pos_np = pos.cpu().numpy()
        t, part = cpu_spectrum(a, pos_np, threads, mods)
        cpu = {"value": 1.0 / t, "unit": UNIT, "cores": threads, "kind": kind,
               "sample": "one full spectrum (all %d particles, all modes); %s; seconds: MA "
                         "%.2f, overdensity %.2f, Pk %.2f" % (a.particles, desc, part["ma"],
                                                             part["overdensity"], part["pk"])}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded %s positions, generated on the device)"
                                     % a.positions,
            "config": workload(a), "roofline": roof, "stages": stages,
            "cpu_baseline": cpu, "e2e": e2e,
            "headline": headline, "batched": batched, "served": served,
            "clocks": clk, "gpu_launches": launches,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


# --------------------------------------------- the metric's headline stream
def headline_stream(a, P, host, device_value):
    """The metric's comparison on one request stream: a.headline_requests
    spectra of the workload (same pinned host positions for every form).

    plain    the drop-in path one request at a time, as the reference's
             canonical caller (Pk_snapshot.py:66-89): delta = zeros, MA(pos,
             delta), delta /= mean; delta -= 1 (numpy), Pk(delta) -- host
             numpy arrays in and out.
    batched  pylians3_gb300.power_spectra (the grid stays on the device, the
             upload of one request overlaps the computation of the one
             before).
    served   serving.Server (continuous batching: contexts with resident
             workspaces, HBM-budget admission), all requests submitted at
             once; and a Poisson stream below saturation for its latency."""
    import numpy as np
    from pylians3_gb300.serving import Server
    K = max(4, a.headline_requests)

    def plain_one():
        delta = np.zeros((a.dims,) * 3, np.float32)
        P.MAS_library.MA(host, delta, BOX, a.mas)
        delta /= (a.particles * 1.0 / a.dims ** 3)
        delta -= 1.0
        return P.Pk_library.Pk(delta, BOX, axis=a.axis, MAS=a.mas, threads=1, verbose=False)

    plain_one()
    lat = []
    t0 = time.perf_counter()
    for _ in range(K):
        t1 = time.perf_counter()
        plain_one()
        lat.append(time.perf_counter() - t1)
    t_plain = time.perf_counter() - t0
    plain = {"value": K / t_plain, "p50_ms": 1e3 * float(np.percentile(lat, 50)),
             "p99_ms": 1e3 * float(np.percentile(lat, 99)),
             "api": "MAS_library.MA + numpy delta/mean - 1 + Pk_library.Pk, one request at a "
                    "time, host numpy arrays (Pk_snapshot.py:66-89)"}

    # the same drop-in sequence for a caller whose particles are already on
    # the device (torch CUDA tensors in and out of MA and Pk)
    import torch
    dev_pos = torch.from_numpy(np.asarray(host)).cuda()

    def plain_device_one():
        delta = torch.zeros((a.dims,) * 3, device="cuda")
        P.MAS_library.MA(dev_pos, delta, BOX, a.mas)
        delta /= (a.particles * 1.0 / a.dims ** 3)
        delta -= 1.0
        return P.Pk_library.Pk(delta, BOX, axis=a.axis, MAS=a.mas, threads=1, verbose=False)

    plain_device_one()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(K):
        plain_device_one()
    torch.cuda.synchronize()
    t_pd = time.perf_counter() - t0
    del dev_pos
    plain_device = {"value": K / t_pd,
                    "api": "the same drop-in MA + delta/mean - 1 + Pk sequence on torch CUDA "
                           "tensors (positions already on the device), one request at a time"}

    P.power_spectra([host] * 2, a.dims, BOX, a.mas, axis=a.axis)
    t0 = time.perf_counter()
    P.power_spectra([host] * K, a.dims, BOX, a.mas, axis=a.axis)
    t_b = time.perf_counter() - t0
    batched = {"value": K / t_b, "api": "pylians3_gb300.power_spectra (2 sets in flight)"}

    def serve(slots, arrivals):
        srv = Server(slots=slots, hbm_budget=150e9)
        for f in [srv.submit(host, a.dims, BOX, a.mas, axis=a.axis) for _ in range(slots)]:
            f.result()                     # warm every slot's workspaces
        srv.done_latencies.clear()
        t0 = time.perf_counter()
        futs = []
        for t_arr in arrivals:
            now = time.perf_counter() - t0
            if t_arr > now:
                time.sleep(t_arr - now)
            futs.append(srv.submit(host, a.dims, BOX, a.mas, axis=a.axis))
        for f in futs:
            f.result()
        wall = time.perf_counter() - t0
        lat = srv.latencies()
        srv.close()
        return {"value": len(arrivals) / wall, "p50_ms": 1e3 * float(np.percentile(lat, 50)),
                "p99_ms": 1e3 * float(np.percentile(lat, 99))}

    served = serve(3, [0.0] * K)
    served["api"] = "serving.Server, 3 slots, all requests submitted at once"
    rate = 0.5 * served["value"]
    rng = np.random.default_rng(99)
    arr = np.cumsum(rng.exponential(1.0 / rate, size=2 * K))
    poisson = serve(3, list(arr))
    poisson["rate_per_s"] = rate
    poisson["api"] = "serving.Server, 3 slots, Poisson arrivals at half the saturated rate"
    best = max(batched["value"], served["value"])
    return {
        "stream": "%d requests: %d pinned host particles each -> %d^3 %s spectrum, axis %d"
                  % (K, a.particles, a.dims, a.mas, a.axis),
        "plain": plain, "plain_device": plain_device,
        "batched": batched, "served": served, "served_poisson": poisson,
        "device_resident": {"value": device_value,
                            "api": "pyl_pk_particles on device-resident positions (value)"},
        "ratio_served_batched_vs_plain": best / plain["value"],
        "ratio_batched_vs_plain": batched["value"] / plain["value"],
        "ratio_served_vs_plain": served["value"] / plain["value"],
        "ratio_device_resident_vs_plain": device_value / plain["value"],
        "ratio_device_resident_vs_plain_device": device_value / plain_device["value"],
    }


def batched_summary(a):
    """64 uneven realizations (the batched workload), device-resident: one
    power_spectrum call at a time vs the whole batch as one graph launch vs
    the server (2 slots).  Tile shapes as tuned and cached, else the
    built-in rule."""
    import torch
    import pylians3_gb300 as P
    from pylians3_gb300.pipeline import spectra_batch
    from pylians3_gb300.serving import run_batch
    reqs = batched_requests(torch)
    ctx = P.context(0)
    for r in reqs:
        P.power_spectrum(**r, ctx=ctx)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for r in reqs:
        P.power_spectrum(**r, ctx=ctx)
    t_seq = time.perf_counter() - t0
    t_graph = {}
    for lanes in (1, 4):
        c = P.Context(0)
        spectra_batch(reqs, ctx=c, lanes=lanes)     # direct: exact sorts, learns, captures
        spectra_batch(reqs, ctx=c, lanes=lanes)
        best = None
        for _ in range(3):
            t0 = time.perf_counter()
            spectra_batch(reqs, ctx=c, lanes=lanes)
            t = time.perf_counter() - t0
            best = t if best is None else min(best, t)
        t_graph[lanes] = best
        c.close()
    run_batch(reqs, slots=2)
    _, t_srv = run_batch(reqs, slots=2)
    out = {"metric": "spectra/s over 64 uneven realizations (dims 128-384, 2^20-2^25 "
                     "particles, CIC/TSC, half weighted)",
           "one_at_a_time": len(reqs) / t_seq,
           "graph_batch": len(reqs) / t_graph[4],
           "graph_batch_api": "pipeline.spectra_batch: one graph launch, 4 lanes side by "
                              "side, count-free sorts learned by the first call (best of 3)",
           "graph_batch_1_lane": len(reqs) / t_graph[1],
           "server_2_slots": len(reqs) / t_srv,
           "speedup_graph_vs_one_at_a_time": t_seq / t_graph[4],
           "particles_total": int(sum(int(r["pos"].shape[0]) for r in reqs))}
    del reqs
    torch.cuda.empty_cache()
    return out


def served_summary(a, rates=(100.0, 400.0), seconds=3.0):
    """Short Poisson streams of the served workload (dims 64-512, any MAS and
    axis, 1-8 particles per cell): the server (8 slots) against a queue with
    one slot, spectra/s and p50/p99 latency."""
    import torch
    import argparse as _ap
    b = _ap.Namespace(**vars(a))
    b.rates, b.seconds, b.slots = list(rates), seconds, 8
    res = run_served(b, emit=False)
    torch.cuda.empty_cache()
    return res


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


def run_served(a, emit=True):
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
    del pool
    if emit:
        print(json.dumps(line), flush=True)
    return line


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
