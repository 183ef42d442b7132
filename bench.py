"""Benchmark of the PaRGO focal hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

Default workload ("hydro8192"): the D8 + pit-removal configuration -- an
8192 x 8192 float32 fBm DEM (seed 1, Hurst 0.75, relief 0-3000 m, 30 m cells)
with 1% of cells lowered by U(0, 5) m and a random-walk nodata blob over 10%,
pit removal with gap 1e-3 m -- one step = pit removal -> Horn slope + D8 on the
float64 levels, outputs: filled DEM (float32), slope (float32), D8 (int8).
Metric: Mcells/s of slope+D8+fill (whole job over all GPUs).

Other workloads (secondary lines, --workload): slope32768 / slope8192 /
slope1024 (fused slope+D8), batch512 (512 uneven rasters, batched vs plain),
sca16384 (SCA on the filled 16384^2 DEM), grad8192 (slope forward+adjoint);
hydro2048 and sca4096 are small cases of the same code for profiler captures.

Multi-GPU: replicas only -- each rank runs the same workload on its own GPU,
nothing is exchanged on the data path; value = all ranks' cells / max time.

The default line also carries, under "sub", the rest of the headline metric
timed in the same run: slope32768 (fused slope + D8 on the 32768^2 DEM, % of
HBM) and batch512 (the batched launch against the per-raster launches).

--impl reference: the reference's own CPU algorithm (the pinned C port of the
reference operators) on the host cores: each step slope + D8 over the full
8192^2 DEM with every core (OpenMP rows) plus the serial raster-order
Gauss-Seidel pit removal on a 1024^2 crop, its per-cell time scaled to the
full raster; once, a one-thread slope + D8 and the fill on 512^2 and 2048^2
crops show how the CPU rates depend on threads and size.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

ND = -9999.0
MEASURED_PEAKS = os.path.join(HERE, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0
# dram__bytes_read.sum + dram__bytes_write.sum per cell of focal_tma_kernel,
# from its ncu capture on 8192^2 (301.3 MB + 289.3 MB over 67108864 cells)
FOCAL_DRAM_BYTES_PER_CELL = (301.330688e6 + 289.264128e6) / 67108864   # tiled kernel, 8192^2 ncu capture
STRIP_DRAM_BYTES_PER_CELL = (289.425152e6 + 284.340224e6) / 67108864   # strip walk, 8192^2 ncu capture
# dram__bytes_read.sum + dram__bytes_write.sum of one batch_strip_kernel launch
# on the batch512 workload (one-pass ncu capture of that launch)
BATCH_STRIP_DRAM_BYTES_512 = 4283454464 + 4787671296
# dram__bytes_read.sum + dram__bytes_write.sum of one fill_tiles_kernel<true>
# launch on the default 8192^2 workload (one-pass ncu capture of that launch)
FILL_DRAM_BYTES_8192 = 2444316416 + 757925632


def hbm_peak():
    try:
        with open(MEASURED_PEAKS) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


# ------------------------------------------------------------------ clocks --
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------- helpers --
def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        backend = "nccl"
        try:
            import torch
            if not torch.cuda.is_available():
                backend = "gloo"
        except Exception:
            backend = "gloo"
        dist.init_process_group(backend=backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, ws, device=None):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device if device is not None else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def pinned(a):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    return t


# --------------------------------------------------------------- workloads --
def make_hydro(rows=8192, cols=8192):
    from pargo_gb300 import synth
    return synth.hydro_dem(rows, cols, seed=1, hurst=0.75, relief=3000.0)


def cpu_fill_crop(dem, side, O=None):
    """The reference's pit removal (raster-order Gauss-Seidel sweeps, serial:
    its OpenMP path races) on a centred side x side crop of `dem`, gap 1e-3.
    Returns (cells, seconds, sweeps)."""
    import oracle
    O = O or oracle.Oracle()
    r0 = max(0, (dem.shape[0] - side) // 2)
    c0 = max(0, (dem.shape[1] - side) // 2)
    crop = np.ascontiguousarray(dem[r0:r0 + side, c0:c0 + side])
    t0 = time.perf_counter()
    _, sweeps = O.fill_gs(crop, ND, gap=1e-3)
    return crop.size, time.perf_counter() - t0, sweeps


def cpu_slope_d8(dem, threads, O=None):
    """The reference's Horn slope and D8 over the whole raster (its OpenMP row
    loop, `threads` threads).  Returns (cells, seconds)."""
    import oracle
    O = O or oracle.Oracle()
    t0 = time.perf_counter()
    O.slope(dem, ND, 30.0, threads=threads)
    O.d8(dem, ND, threads=threads)
    return dem.size, time.perf_counter() - t0


def cpu_sample_hydro(dem, threads, crop=1024, O=None):
    """One bounded CPU sample of the hydro step: slope + D8 over the full
    raster on `threads` cores, and the serial Gauss-Seidel fill on a crop x
    crop crop.  Returns (Mcells/s of the composite, details): the composite
    is the full raster's cells over (slope+D8 time + the crop's fill time per
    cell x the full raster's cells) -- the fill's per-cell cost taken from the
    crop, which favours the CPU (its sweep count grows with the raster)."""
    n_sd8, t_sd8 = cpu_slope_d8(dem, threads, O)
    n_f, t_f, sweeps = cpu_fill_crop(dem, crop, O)
    t_full = t_sd8 + t_f / n_f * dem.size
    return dem.size / t_full / 1e6, {"slope_d8_s": round(t_sd8, 3), "fill_crop_s": round(t_f, 3),
                                     "fill_crop_side": crop, "fill_crop_sweeps": sweeps}


def run_hydro(args, ws, rank, local, side=8192):
    import torch
    from pargo_gb300 import abi
    torch.cuda.set_device(local)
    ctx = abi.Context(local)
    dem = make_hydro(side, side)
    rows, cols = dem.shape
    cells = rows * cols
    stream = torch.cuda.current_stream()
    d = torch.from_numpy(dem).cuda()
    w32 = torch.empty((rows, cols), dtype=torch.float32, device="cuda")
    s32 = torch.empty((rows, cols), dtype=torch.float32, device="cuda")
    c8 = torch.empty((rows, cols), dtype=torch.int8, device="cuda")
    R = abi.raster
    rd, rw, rs, rc = R(d, ND, 30.0), R(w32, ND), R(s32, ND), R(c8, -128)

    def step():
        return ctx.hydro_pipeline(rd, wdem=rw, slope=rs, d8=rc, gap=1e-3, stream=stream)

    for _ in range(args.warmup):
        st = step()
    torch.cuda.synchronize()
    barrier(ws)
    clocks = ClockSampler(local)
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    rounds = 0
    visits = 0
    iters = 0
    rounds_ms = 0.0
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(args.steps):
        st = step()
        rounds += st.rounds
        visits += st.tile_visits
        iters += st.local_iterations
        rounds_ms += st.rounds_ms
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(ws)
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1) / args.steps
    ms = max_over_ranks(ms, ws, torch.device("cuda", local))
    value = ws * cells / (ms * 1e-3) / 1e6

    # end to end through the C ABI with host buffers (pinned), copies inside the timed region
    hd = pinned(dem)
    hw = torch.empty((rows, cols), dtype=torch.float32).pin_memory()
    hs = torch.empty((rows, cols), dtype=torch.float32).pin_memory()
    hc = torch.empty((rows, cols), dtype=torch.int8).pin_memory()
    hr = (R(hd, ND, 30.0), R(hw, ND), R(hs, ND), R(hc, -128))
    ctx.hydro_pipeline(hr[0], wdem=hr[1], slope=hr[2], d8=hr[3], gap=1e-3, stream=stream)
    torch.cuda.synchronize()
    barrier(ws)
    e2e_steps = max(1, min(args.steps, 3))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ctx.hydro_pipeline(hr[0], wdem=hr[1], slope=hr[2], d8=hr[3], gap=1e-3, stream=stream)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks((time.perf_counter() - t0) / e2e_steps, ws, torch.device("cuda", local))
    e2e_value = ws * cells / e2e_s / 1e6

    # roofline of the dominant kernel: the fill relaxation (one persistent
    # launch per step; PARGO_FILL_ROUNDS=1 selects the round launches).
    # Algorithmic bytes: 8 B per cell of the raster per step (4 B DEM read +
    # 4 B level written, the minimum any fill must move), the number of tile
    # visits reported beside it; duration: the relaxation's device time (CUDA
    # events on its stream).  The same 8 B counted once per cell of every tile
    # visit is reported as achieved_per_cell_visit.
    peak, peak_kind = hbm_peak()
    fill_s = rounds_ms * 1e-3 / max(args.steps, 1)  # per step
    achieved = 8.0 * cells / fill_s / 1e9 if fill_s > 0 else 0.0
    achieved_visit = 8.0 * 1024 * visits / max(args.steps, 1) / fill_s / 1e9 if fill_s > 0 else 0.0
    fill_share = rounds_ms / (ms * args.steps) if ms > 0 else None
    roofline = {"bound": "hbm", "kernel": "fill_tiles_kernel<true> (persistent)" if rounds == args.steps
                else "fill_tiles_kernel<false> (rounds)", "achieved": round(achieved, 2), "peak": peak,
                "unit": "GB/s", "frac": round(achieved / peak, 5), "peak_source": peak_kind,
                "algorithmic_bytes_per_cell": 8, "achieved_per_cell_visit": round(achieved_visit, 2),
                "traffic": FILL_DRAM_BYTES_8192 if (side == 8192 and rounds == args.steps) else None,
                "traffic_source": "ncu capture of one launch of this workload" if side == 8192 else None,
                "rounds_per_step": rounds // args.steps,
                "tile_visits_per_step": visits // args.steps,
                "local_iterations_per_visit": round(iters / max(visits, 1), 2), "fill_share_of_step": round(fill_share, 4)
                if fill_share else None}
    # per step: tile bookkeeping, level init, outlet-tile seeding, the
    # relaxation launch(es) and the float64 slope/D8
    launches = args.steps * 4 + rounds

    cpu = None
    if rank == 0 and ws == 1:
        thr = os.cpu_count() or 1
        v, det = cpu_sample_hydro(dem, thr)
        cpu = {"value": round(v, 3), "unit": "Mcells/s", "cores": thr, "kind": "port",
               "sample": "slope + D8 over the full %dx%d DEM (the reference's OpenMP loop, %d threads, %.2f s) and "
                         "the serial Gauss-Seidel fill on a centred 1024x1024 crop (%d sweeps, %.2f s) scaled per "
                         "cell to the full raster; the fill's sweep count grows with raster size, so the CPU's "
                         "true full-size rate is lower still" % (rows, cols, thr, det["slope_d8_s"],
                                                                 det["fill_crop_sweeps"], det["fill_crop_s"])}
    return {
        "metric": "Mcells/s slope+D8+fill", "value": round(value, 2), "unit": "Mcells/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64 levels (emulated on integer pipes), f32 slope",
        "data": "synthetic (seeded fBm, same shapes and value distributions as the named workload)",
        "config": {"workload": "hydro%d: D8 + Planchon-Darboux fill (gap 1e-3 m) + Horn slope, %dx%d "
                               "float32 fBm DEM (seed 1, H 0.75, 0-3000 m, 30 m), 1%% pits, 10%% nodata blob"
                               % (side, side, side),
                   "rows": rows, "cols": cols,
                   "l2": "inputs larger than L2 (%d MB DEM, %d MB float64 levels)" % (cells * 4 >> 20, cells * 8 >> 20)
                   if cells * 4 > (129 << 20) else "DEM smaller than L2 (profiling case)",
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "roofline": roofline, "cpu_baseline": cpu,
        "e2e": {"value": round(e2e_value, 2), "unit": "Mcells/s", "h2d_bytes_per_step": cells * 4,
                "d2h_bytes_per_step": cells * (4 + 4 + 1)},
        "gpu_launches": launches, "clocks": clk,
    }


def run_slope(args, ws, rank, local, side):
    """Fused slope + D8 on a side x side float32 DEM (16-byte aligned rows: TMA path)."""
    import torch
    from pargo_gb300 import abi, synth
    torch.cuda.set_device(local)
    ctx = abi.Context(local)
    dem = synth.slope_dem(side, side, seed=0, hurst=0.8, relief=2000.0)
    cells = side * side
    stream = torch.cuda.current_stream()
    d = torch.from_numpy(dem).cuda()
    del dem
    s = torch.empty((side, side), dtype=torch.float32, device="cuda")
    c = torch.empty((side, side), dtype=torch.int8, device="cuda")
    R = abi.raster
    rd, rs, rc = R(d, ND, 30.0), R(s, ND), R(c, -128)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda") if cells * 9 < (256 << 20) else None
    best, tune_ms = ctx.tune_focal(rd, reps=3)
    forced = os.environ.get("PARGO_FOCAL_VARIANT")
    strip = (int(forced) if forced else best) >= 5   # variants 5 and 6: the strip walk
    for _ in range(args.warmup):
        ctx.slope_d8(rd, rs, rc, stream=stream)
    torch.cuda.synchronize()
    barrier(ws)
    clocks = ClockSampler(local)
    clocks.start()
    times = []
    for _ in range(args.steps):
        if flush is not None:
            flush.fill_(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.slope_d8(rd, rs, rc, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    barrier(ws)
    clk = clocks.stop()
    ms = max_over_ranks(float(np.mean(times)), ws, torch.device("cuda", local))
    peak, kind = hbm_peak()
    achieved = cells * 9.0 / (ms * 1e-3) / 1e9
    return {
        "metric": "Mcells/s slope+D8", "value": round(ws * cells / (ms * 1e-3) / 1e6, 1), "unit": "Mcells/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 (D8 decisions certified, "
        "FP64 fallback)", "data": "synthetic",
        "config": {"workload": "slope%d: fused Horn slope + D8, %dx%d float32 fBm DEM" % (side, side, side),
                   "l2": "flushed between iterations" if flush is not None else "inputs larger than L2"},
        "roofline": {"bound": "hbm", "kernel": "focal_strip_kernel" if strip else "focal_tma_kernel",
                     "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": kind,
                     # DRAM read + write of one launch, scaled by cells from the 8192^2 ncu capture of the
                     # same kernel (the traffic grows with the cell count)
                     "traffic": round((STRIP_DRAM_BYTES_PER_CELL if strip else FOCAL_DRAM_BYTES_PER_CELL) * cells),
                     "traffic_source": "ncu 8192^2 capture scaled per cell",
                     "variant": abi.focal_variant_names()[int(forced) if forced else best],
                     "variant_ms": dict(zip(abi.focal_variant_names(), tune_ms))},
        # the strip walk is a walk launch and a fix-up launch per step; the tiled kernel one
        "gpu_launches": args.steps * (2 if strip else 1), "clocks": clk,
    }


def run_batch(args, ws, rank, local):
    """512 independent fBm rasters (seeds 100-611, sides log-uniform in
    [256, 4096], Hurst U(0.6, 0.9)): fused slope+D8 as ONE persistent batched
    launch vs plain per-raster launches of the same kernel, same buffers."""
    import torch
    from pargo_gb300 import abi, synth
    torch.cuda.set_device(local)
    ctx = abi.Context(local)
    shapes = synth.batch_shapes(512, first_seed=100)
    R = abi.raster
    dems, slopes, codes = [], [], []
    cells = 0
    for (s_, r, c, h) in shapes:
        d = synth.slope_dem(r, c, seed=s_, hurst=h, relief=2000.0)
        pc = (c + 3) // 4 * 4  # 16-byte rows: every raster takes the TMA path
        buf = torch.zeros((r, pc), dtype=torch.float32, device="cuda")
        buf[:, :c] = torch.from_numpy(d).cuda()
        dems.append(buf[:, :c])
        slopes.append(torch.empty((r, pc), dtype=torch.float32, device="cuda")[:, :c])
        codes.append(torch.empty((r, pc), dtype=torch.int8, device="cuda")[:, :c])
        cells += r * c
    stream = torch.cuda.current_stream()
    rd = [R(d, ND, 30.0) for d in dems]
    rs = [R(x, ND) for x in slopes]
    rc = [R(x, -128) for x in codes]

    def batched():
        ctx.batch_slope_d8(rd, rs, rc, stream=stream)

    def plain():
        for a, b, c in zip(rd, rs, rc):
            ctx.slope_d8(a, b, c, stream=stream)

    def timeit(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    # Identical outputs: the batched launch and the per-raster launches give the same bytes.
    batched()
    ref = [(x.clone(), y.clone()) for x, y in zip(slopes, codes)]
    for x, y in zip(slopes, codes):
        x.fill_(0.0)
        y.fill_(0)
    plain()
    identical = all(torch.equal(x, a) and torch.equal(y, b) for (a, b), x, y in zip(ref, slopes, codes))
    del ref

    # the queue's intensity estimate is taken on the first call of a batch
    # description: time that call on its own
    ctx.batch_slope_d8(rd, rs, rc, stream=stream, order=abi.BATCH_BY_SIZE)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    batched()
    torch.cuda.synchronize()
    first_call_ms = (time.perf_counter() - t0) * 1e3
    barrier(ws)
    clocks = ClockSampler(local)
    clocks.start()
    ms_b = timeit(batched)
    ms_p = timeit(plain)
    clk = clocks.stop()
    ms_size = timeit(lambda: ctx.batch_slope_d8(rd, rs, rc, stream=stream, order=abi.BATCH_BY_SIZE))
    ms_b = max_over_ranks(ms_b, ws, torch.device("cuda", local))
    ms_p = max_over_ranks(ms_p, ws, torch.device("cuda", local))
    peak, kind = hbm_peak()
    achieved = cells * 9.0 / (ms_b * 1e-3) / 1e9
    return {
        "metric": "Mcells/s batched slope+D8 (512 uneven rasters); batched vs plain speedup",
        "value": round(ws * cells / (ms_b * 1e-3) / 1e6, 1), "unit": "Mcells/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_b, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (D8 decisions certified, FP64 fallback)",
        "data": "synthetic", "batched_vs_plain_speedup": round(ms_p / ms_b, 3), "plain_ms_per_step": round(ms_p, 4),
        "batched_outputs_identical_to_plain": identical,
        "queue": {"order": "rasters by compute intensity (valid 1, nodata 0), heaviest first, each raster's segments together",
                  "first_call_ms_with_estimate": round(first_call_ms, 3),
                  "ms_per_step_ordered_by_raster_size": round(ms_size, 4)},
        "config": {"workload": "batch512: 512 fBm rasters, seeds 100-611, sides log-uniform [256, 4096], "
                               "Hurst U(0.6, 0.9), %d cells" % cells,
                   "l2": "inputs larger than L2 (%.1f GB per step)" % (cells * 9 / 1e9)},
        "roofline": {"bound": "hbm", "kernel": "batch_strip_kernel (+ batch_strip_fixup_kernel)", "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": kind,
                     "traffic": BATCH_STRIP_DRAM_BYTES_512,
                     "traffic_source": "ncu capture of one batch_strip_kernel launch of this workload",
                     "algorithmic_bytes": cells * 9},
        "gpu_launches": 2 * args.steps, "plain_gpu_launches": args.steps * 512, "clocks": clk,
    }


def run_batch_fill(args, ws, rank, local):
    """Pit removal (gap 1e-3) of the 512 uneven fBm rasters of batch512 as ONE
    persistent relaxation over a mosaic of the batch (pargo_batch_fill) vs a
    pargo_fill call per raster, same buffers, outputs compared byte for byte."""
    import torch
    from pargo_gb300 import abi, synth
    torch.cuda.set_device(local)
    ctx = abi.Context(local)
    shapes = synth.batch_shapes(512, first_seed=100)
    R = abi.raster
    dems, outs = [], []
    cells = 0
    for (s_, r, c, h) in shapes:
        dems.append(torch.from_numpy(synth.slope_dem(r, c, seed=s_, hurst=h, relief=2000.0)).cuda())
        outs.append(torch.empty((r, c), dtype=torch.float32, device="cuda"))
        cells += r * c
    stream = torch.cuda.current_stream()
    rd = [R(d, ND, 30.0) for d in dems]
    ro = [R(o, ND) for o in outs]
    stats = {}

    def batched():
        stats["b"] = ctx.batch_fill(rd, ro, gap=1e-3, stream=stream)

    def plain():
        for a, b in zip(rd, ro):
            ctx.fill(a, b, gap=1e-3, stream=stream)

    batched()
    ref = [o.clone() for o in outs]
    for o in outs:
        o.fill_(0.0)
    plain()
    identical = all(torch.equal(a, b) for a, b in zip(ref, outs))
    del ref
    barrier(ws)
    clocks = ClockSampler(local)
    clocks.start()
    steps = argparse.Namespace(steps=max(1, min(args.steps, 5)), warmup=args.warmup)
    ms_b = timed_steps(batched, steps, stream)
    ms_p = timed_steps(plain, steps, stream)
    clk = clocks.stop()
    ms_b = max_over_ranks(ms_b, ws, torch.device("cuda", local))
    ms_p = max_over_ranks(ms_p, ws, torch.device("cuda", local))
    st = stats["b"]
    peak, kind = hbm_peak()
    fill_ms = st.rounds_ms
    achieved = cells * 8.0 / (fill_ms * 1e-3) / 1e9 if fill_ms > 0 else 0.0
    return {
        "metric": "Mcells/s batched pit removal (512 uneven rasters); batched vs plain speedup",
        "value": round(ws * cells / (ms_b * 1e-3) / 1e6, 1), "unit": "Mcells/s", "n_gpus": ws,
        "steps": steps.steps, "warmup": args.warmup, "ms_per_step": round(ms_b, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64 levels (integer-key arithmetic), f32 output",
        "data": "synthetic", "batched_vs_plain_speedup": round(ms_p / ms_b, 3), "plain_ms_per_step": round(ms_p, 3),
        "batched_outputs_identical_to_plain": identical,
        "config": {"workload": "batchfill512: the batch512 rasters (seeds 100-611, sides log-uniform [256, 4096], "
                               "Hurst U(0.6, 0.9), 0-2000 m, 1-cell nodata border), gap 1e-3, %d cells" % cells,
                   "l2": "inputs larger than L2"},
        "roofline": {"bound": "hbm", "kernel": "fill_tiles_kernel<true> over the batch mosaic",
                     "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 5), "peak_source": kind, "traffic": None,
                     "algorithmic_bytes_per_cell": 8, "relaxation_ms": round(fill_ms, 3),
                     "tile_visits": st.tile_visits},
        # per batched step: mosaic clear + pack, tile bookkeeping, level init,
        # outlet seeding, the persistent relaxation, the per-raster finish
        "gpu_launches": steps.steps * 7, "plain_gpu_launches": steps.steps * 512 * 5, "clocks": clk,
    }


def timed_steps(fn, args, stream, flush=None):
    """W untimed steps, then K steps bracketed by CUDA events on `stream`
    (L2 flushed before each step when `flush` is given); mean ms per step."""
    import torch
    for _ in range(args.warmup):
        fn()
    torch.cuda.synchronize()
    times = []
    for _ in range(args.steps):
        if flush is not None:
            flush.fill_(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    return float(np.mean(times))


def run_sca(args, ws, rank, local, side=16384):
    """D8 specific catchment area on the filled side^2 DEM of the slope
    generator (seed 2, Hurst 0.8, 0-2000 m, 1-cell nodata border, 10 m
    cells): setup (untimed) fills the DEM (gap 1e-3) and derives the int8 D8
    codes on the GPU; a step is one SCA call (float64 output)."""
    import torch
    from pargo_gb300 import abi
    torch.cuda.set_device(local)
    ctx = abi.Context(local)
    from pargo_gb300 import synth
    dem = synth.slope_dem(side, side, seed=2, hurst=0.8, relief=2000.0)
    cells = side * side
    stream = torch.cuda.current_stream()
    R = abi.raster
    d = torch.from_numpy(dem).cuda()
    del dem
    codes = torch.empty((side, side), dtype=torch.int8, device="cuda")
    ctx.hydro_pipeline(R(d, ND, 10.0), d8=R(codes, -128), gap=1e-3, stream=stream)
    del d
    out = torch.empty((side, side), dtype=torch.float64, device="cuda")
    rc, ro = R(codes, -128), R(out, ND)
    barrier(ws)
    clocks = ClockSampler(local)
    clocks.start()
    ms = timed_steps(lambda: ctx.sca(rc, ro, stream=stream), args, stream)
    clk = clocks.stop()
    ms = max_over_ranks(ms, ws, torch.device("cuda", local))
    # end to end with host buffers: codes in, float64 SCA out
    hc = codes.cpu().pin_memory()
    ho = torch.empty((side, side), dtype=torch.float64).pin_memory()
    rh = (R(hc, -128), R(ho, ND))
    ctx.sca(*rh, stream=stream)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_steps = max(1, min(args.steps, 3))
    for _ in range(e2e_steps):
        ctx.sca(*rh, stream=stream)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks((time.perf_counter() - t0) / e2e_steps, ws, torch.device("cuda", local))
    cpu = None
    if rank == 0 and ws == 1:
        # the reference's own algorithm (scaOperator.cpp: in-degree pass, then
        # accumulation sweeps in raster order), restated serially by the
        # oracle, on centred crops of the same codes with a nodata ring:
        # "converged" sweeps until no in-degree is left (what the GPU step
        # computes), "shipped" stops after one accumulation sweep
        import oracle
        O = oracle.Oracle()
        cols = {}
        for name, n, sweeps in (("converged", 1024, 1 << 30), ("converged_512", 512, 1 << 30),
                                ("shipped", 4096, 1)):
            crop = host_codes_crop(hc, n)
            t0 = time.perf_counter()
            _, sw = O.sca_sweeps(crop, -128.0, sweeps)
            dt = time.perf_counter() - t0
            cols[name] = {"crop": n, "sweeps": sw, "s": round(dt, 3), "Mcells_s": round(crop.size / dt / 1e6, 4)}
        crop = host_codes_crop(hc, 2048)
        t0 = time.perf_counter()
        O.sca(crop, -128.0)
        dt = time.perf_counter() - t0
        cols["topological_2048"] = {"crop": 2048, "s": round(dt, 3), "Mcells_s": round(crop.size / dt / 1e6, 3),
                                    "note": "the oracle's O(N) topological accumulation, not the reference's "
                                            "algorithm (informative)"}
        c = cols["converged"]
        cpu = {"value": c["Mcells_s"], "unit": "Mcells/s", "cores": 1, "kind": "port",
               "sample": "1024x1024 crop of the same D8 codes with a nodata ring: the reference's sweep SCA "
                         "(serial restatement), converged after %d accumulation sweeps, %.2f s; the rate falls "
                         "as the crop grows (more sweeps per cell)" % (c["sweeps"], c["s"]),
               "columns": cols}
    peak, kind = hbm_peak()
    achieved = cells * 9.0 / (ms * 1e-3) / 1e9
    return {
        "metric": "Mcells/s D8 SCA", "value": round(ws * cells / (ms * 1e-3) / 1e6, 1), "unit": "Mcells/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64 accumulation (u64 counts)",
        "data": "synthetic",
        "config": {"workload": "sca%d: D8 SCA on the filled %dx%d fBm DEM (seed 2, H 0.8, 0-2000 m, 10 m cells, "
                               "gap 1e-3), int8 codes in, float64 out" % (side, side, side),
                   "l2": "inputs larger than L2"},
        "roofline": {"bound": "hbm", "kernel": "sca_tile_kernel x2 + exit forest (3 kernels) + sca_output_kernel "
                               "(one call)", "achieved": round(achieved, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": kind,
                     "traffic": None, "algorithmic_bytes_per_cell": 9},
        "cpu_baseline": cpu,
        "e2e": {"value": round(ws * cells / e2e_s / 1e6, 1), "unit": "Mcells/s", "h2d_bytes_per_step": cells,
                "d2h_bytes_per_step": cells * 8},
        "gpu_launches": args.steps * 6, "clocks": clk,  # the six kernels of one tiled SCA call
    }


def host_codes_crop(hc, n):
    a = hc.numpy()
    r0 = (a.shape[0] - n) // 2
    c0 = (a.shape[1] - n) // 2
    crop = np.ascontiguousarray(a[r0:r0 + n, c0:c0 + n]).astype(np.float64)
    crop[0, :] = crop[-1, :] = crop[:, 0] = crop[:, -1] = -128.0
    return crop


def run_grad(args, ws, rank, local, side=8192):
    """Differentiable slope: forward + hand-written adjoint of
    L = sum (slope(z) - slope(z + N(0, 0.5 m)))^2 on a side^2 float32 fBm DEM
    (seed 3); a step is one fused loss+gradient call (loss read back)."""
    import torch
    from pargo_gb300 import abi, synth
    torch.cuda.set_device(local)
    ctx = abi.Context(local)
    z = synth.slope_dem(side, side, seed=3, hurst=0.8, relief=2000.0)
    zr = synth.perturbed(z, sigma=0.5, seed=3)
    cells = side * side
    stream = torch.cuda.current_stream()
    R = abi.raster
    dz, dzr = torch.from_numpy(z).cuda(), torch.from_numpy(zr).cuda()
    g = torch.empty((side, side), dtype=torch.float32, device="cuda")
    rz, rzr, rg = R(dz, ND, 30.0), R(dzr, ND, 30.0), R(g, ND)
    barrier(ws)
    clocks = ClockSampler(local)
    clocks.start()
    ms = timed_steps(lambda: ctx.slope_loss_grad(rz, rzr, rg, stream=stream), args, stream)
    clk = clocks.stop()
    ms = max_over_ranks(ms, ws, torch.device("cuda", local))
    hz, hzr = pinned(z), pinned(zr)
    hg = torch.empty((side, side), dtype=torch.float32).pin_memory()
    rh = (R(hz, ND, 30.0), R(hzr, ND, 30.0), R(hg, ND))
    ctx.slope_loss_grad(*rh, stream=stream)
    t0 = time.perf_counter()
    e2e_steps = max(1, min(args.steps, 3))
    for _ in range(e2e_steps):
        ctx.slope_loss_grad(*rh, stream=stream)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks((time.perf_counter() - t0) / e2e_steps, ws, torch.device("cuda", local))
    cpu = None
    if rank == 0 and ws == 1:
        import oracle
        O = oracle.Oracle()
        thr = os.cpu_count() or 1
        t0 = time.perf_counter()
        O.slope(z[:2048], ND, 30.0, threads=thr)
        O.slope(zr[:2048], ND, 30.0, threads=thr)
        dt = time.perf_counter() - t0
        cpu = {"value": round(2048 * side / dt / 1e6, 3), "unit": "Mcells/s", "cores": thr, "kind": "port",
               "sample": "the reference has no adjoint: its forward Horn slope (oracle, OpenMP) on the first 2048 "
                         "rows of z and z_ref, %.2f s" % dt}
    peak, kind = hbm_peak()
    achieved = cells * 12.0 / (ms * 1e-3) / 1e9
    return {
        "metric": "Mcells/s slope forward+backward", "value": round(ws * cells / (ms * 1e-3) / 1e6, 1),
        "unit": "Mcells/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 (loss summed in f64)",
        "data": "synthetic",
        "config": {"workload": "grad%d: fused Horn slope forward + adjoint of sum (slope(z) - slope(z_ref))^2, "
                               "%dx%d float32 fBm DEM (seed 3), z_ref = z + N(0, 0.5 m)" % (side, side, side),
                   "l2": "inputs larger than L2"},
        "roofline": {"bound": "hbm", "kernel": "grad fused forward+adjoint", "achieved": round(achieved, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": kind,
                     "traffic": None, "algorithmic_bytes_per_cell": 12},
        "cpu_baseline": cpu,
        "e2e": {"value": round(ws * cells / e2e_s / 1e6, 1), "unit": "Mcells/s", "h2d_bytes_per_step": cells * 8,
                "d2h_bytes_per_step": cells * 4 + 8},
        "gpu_launches": args.steps, "clocks": clk,
    }


def run_mfd(args, ws, rank, local, side=8192):
    """MFD-md: flow partition weights (exponent 1.1) of the pit-removed side^2
    hydro DEM (seed 1, 30 m cells; levels float64, filled untimed on the GPU)
    into 8 float32 layers, then the MFD SCA of those layers (float64).  A step
    is one pargo_mfd call and one pargo_sca_mfd call."""
    import torch
    from pargo_gb300 import abi
    torch.cuda.set_device(local)
    ctx = abi.Context(local)
    dem = make_hydro(side, side)
    cells = side * side
    stream = torch.cuda.current_stream()
    R = abi.raster
    d = torch.from_numpy(dem).cuda()
    del dem
    lv = torch.empty((side, side), dtype=torch.float64, device="cuda")
    ctx.hydro_pipeline(R(d, ND, 30.0), wdem=R(lv, ND), gap=1e-3, stream=stream)
    del d
    ws_dev = [torch.empty((side, side), dtype=torch.float32, device="cuda") for _ in range(8)]
    out = torch.empty((side, side), dtype=torch.float64, device="cuda")
    rl, rw, ro = R(lv, ND, 30.0), [R(w, ND) for w in ws_dev], R(out, ND)

    def weights():
        ctx.mfd(rl, rw, slp_exp=1.1, stream=stream)

    def sca():
        ctx.sca_mfd(rw, ro, stream=stream)

    barrier(ws)
    clocks = ClockSampler(local)
    clocks.start()
    ms = timed_steps(lambda: (weights(), sca()), args, stream)
    clk = clocks.stop()
    ms_w = timed_steps(weights, argparse.Namespace(steps=args.steps, warmup=1), stream)
    ms_s = timed_steps(sca, argparse.Namespace(steps=args.steps, warmup=1), stream)
    ms = max_over_ranks(ms, ws, torch.device("cuda", local))
    # end to end with host buffers: float64 levels in, 8 float32 layers and float64 SCA out
    hl = lv.cpu().pin_memory()
    hw = [torch.empty((side, side), dtype=torch.float32).pin_memory() for _ in range(8)]
    ho = torch.empty((side, side), dtype=torch.float64).pin_memory()
    rhl, rhw, rho = R(hl, ND, 30.0), [R(w, ND) for w in hw], R(ho, ND)

    def e2e():
        ctx.mfd(rhl, rhw, slp_exp=1.1, stream=stream)
        ctx.sca_mfd(rhw, rho, stream=stream)

    e2e()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_steps = max(1, min(args.steps, 3))
    for _ in range(e2e_steps):
        e2e()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks((time.perf_counter() - t0) / e2e_steps, ws, torch.device("cuda", local))
    cpu = None
    if rank == 0 and ws == 1:
        import oracle
        O = oracle.Oracle()
        a = hl.numpy()
        n = 1024
        r0, c0 = (side - n) // 2, (side - n) // 2
        crop = np.ascontiguousarray(a[r0:r0 + n, c0:c0 + n])
        t0 = time.perf_counter()
        O.sca_mfd(O.mfd(crop, ND, 30.0, 1.1), ND)
        dt = time.perf_counter() - t0
        cpu = {"value": round(crop.size / dt / 1e6, 3), "unit": "Mcells/s", "cores": 1, "kind": "port",
               "sample": "1024x1024 crop of the same levels: the oracle's MFD-md weights + one-sweep MFD SCA "
                         "(serial, as the reference), %.2f s" % dt}
    peak, kind = hbm_peak()
    # the dominant kernel is the MFD SCA (the weights are ~1.5% of the step):
    # 8 float32 weight layers read (32 B) and the float64 SCA written (8 B) per cell
    achieved = cells * 40.0 / (ms_s * 1e-3) / 1e9
    achieved_w = cells * 40.0 / (ms_w * 1e-3) / 1e9
    return {
        "metric": "Mcells/s MFD-md weights + MFD SCA", "value": round(ws * cells / (ms * 1e-3) / 1e6, 1),
        "unit": "Mcells/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 weights, f64 SCA sums", "data": "synthetic",
        "config": {"workload": "mfd%d: MFD-md weights (exponent 1.1) + MFD SCA on the pit-removed %dx%d hydro "
                               "DEM (seed 1, 30 m cells, float64 levels), 8 float32 layers, float64 SCA"
                               % (side, side, side), "l2": "inputs larger than L2"},
        "roofline": {"bound": "hbm", "kernel": "sca_mfd_records_kernel + sca_mfd_band_kernel (MFD SCA: warps walk "
                                               "32-row bands in step)", "achieved": round(achieved, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 5), "peak_source": kind,
                     "traffic": None, "algorithmic_bytes_per_cell": 40, "sca_ms": round(ms_s, 3),
                     "sca_share_of_step": round(ms_s / ms, 4) if ms > 0 else None,
                     "weights_kernel": {"kernel": "mfd_weights_kernel", "ms": round(ms_w, 3),
                                        "achieved": round(achieved_w, 1), "frac": round(achieved_w / peak, 4),
                                        "algorithmic_bytes_per_cell": 40}},
        "cpu_baseline": cpu,
        "e2e": {"value": round(ws * cells / e2e_s / 1e6, 1), "unit": "Mcells/s", "h2d_bytes_per_step": cells * 8,
                "d2h_bytes_per_step": cells * (32 + 8)},
        # per step: weights, SCA in-degrees, the cooperative launch of every
        # frontier round, output (the launch list of this workload shows it)
        "gpu_launches": args.steps * 4, "clocks": clk,
    }


def run_load(args, ws, rank, local, side=32768, grain=16):
    """Load estimator: the intensity-ratio compute layer (grain 16, valid 1,
    nodata 0) of the side^2 float32 hydro DEM (seed 1, 10% nodata blob), then
    its 152-part row decomposition; a step is one pargo_compute_load call
    (the compute layer stays on the device) and one pargo_load_decompose."""
    import torch
    from pargo_gb300 import abi
    torch.cuda.set_device(local)
    ctx = abi.Context(local)
    dem = make_hydro(side, side)
    cells = side * side
    stream = torch.cuda.current_stream()
    R = abi.raster
    d = torch.from_numpy(dem).cuda()
    cr, cc = abi.compute_load_dims(side, side, grain)
    load = torch.empty((cr, cc), dtype=torch.float64, device="cuda")
    rd, rl = R(d, ND), R(load, ND)
    nparts = 152

    def step():
        ctx.compute_load(rd, rl, grain, 0.0, 1.0, stream=stream)
        ctx.load_decompose(rl, (side, side), nparts, stream=stream)

    barrier(ws)
    clocks = ClockSampler(local)
    clocks.start()
    ms = timed_steps(step, args, stream)
    clk = clocks.stop()
    ms_k = timed_steps(lambda: ctx.compute_load(rd, rl, grain, 0.0, 1.0, stream=stream),
                       argparse.Namespace(steps=args.steps, warmup=1), stream)
    ms = max_over_ranks(ms, ws, torch.device("cuda", local))
    hd = pinned(dem)
    hl = torch.empty((cr, cc), dtype=torch.float64).pin_memory()
    rh = (R(hd, ND), R(hl, ND))

    def e2e():
        ctx.compute_load(rh[0], rh[1], grain, 0.0, 1.0, stream=stream)
        ctx.load_decompose(rh[1], (side, side), nparts, stream=stream)

    e2e()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_steps = max(1, min(args.steps, 3))
    for _ in range(e2e_steps):
        e2e()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks((time.perf_counter() - t0) / e2e_steps, ws, torch.device("cuda", local))
    cpu = None
    if rank == 0 and ws == 1:
        import oracle
        O = oracle.Oracle()
        crop = np.ascontiguousarray(dem[:4096])
        t0 = time.perf_counter()
        lo = O.compute_load(crop, ND, grain, 0.0, 1.0)
        O.load_decompose(lo, ND, crop.shape, nparts)
        dt = time.perf_counter() - t0
        cpu = {"value": round(crop.size / dt / 1e6, 3), "unit": "Mcells/s", "cores": 1, "kind": "port",
               "sample": "the first 4096 rows: the oracle's compute layer + decomposition (serial, as the "
                         "reference's Transformation::run), %.2f s" % dt}
    peak, kind = hbm_peak()
    achieved = cells * 4.0 / (ms_k * 1e-3) / 1e9
    return {
        "metric": "Mcells/s load estimate + decomposition", "value": round(ws * cells / (ms * 1e-3) / 1e6, 1),
        "unit": "Mcells/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64 sums", "data": "synthetic",
        "config": {"workload": "load%d: intensity compute layer (grain %d) of the %dx%d float32 hydro DEM (seed 1), "
                               "%d-part row decomposition" % (side, grain, side, side, nparts),
                   "l2": "inputs larger than L2"},
        "roofline": {"bound": "hbm", "kernel": "compute_load_count_kernel<16> (integer loads: a warp counts 32 data columns of a compute row)", "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": kind, "traffic": None,
                     "algorithmic_bytes_per_cell": 4, "kernel_ms": round(ms_k, 3)},
        "cpu_baseline": cpu,
        "e2e": {"value": round(ws * cells / e2e_s / 1e6, 1), "unit": "Mcells/s", "h2d_bytes_per_step": cells * 4,
                "d2h_bytes_per_step": cr * cc * 8},
        "gpu_launches": args.steps * 2, "clocks": clk,
    }


def run_reference(args, ws, rank):
    """The reference's CPU algorithm (the oracle's C port of the reference
    operators; the reference's own build needs its sources, which only the
    build container holds) on this host's cores, on the hydro8192 workload.
    Each step: slope + D8 over the full 8192^2 DEM with every core (the
    reference's OpenMP loop) and the serial Gauss-Seidel fill (its only valid
    mode) on a centred 1024^2 crop; value = the full raster's cells over the
    slope+D8 time plus the crop's per-cell fill time scaled to the full
    raster.  Once, untimed by the steps: slope + D8 on one thread, and the
    fill on 512^2 and 2048^2 crops, to show how its rate falls with size."""
    if rank != 0:
        return None
    import oracle
    O = oracle.Oracle()
    thr = os.cpu_count() or 1
    dem = make_hydro()
    n1, t1 = cpu_slope_d8(dem, 1, O)
    crops = []
    for side in (512, 1024, 2048):
        n, t, sw = cpu_fill_crop(dem, side, O)
        crops.append({"side": side, "sweeps": sw, "s": round(t, 3), "Mcells_s": round(n / t / 1e6, 4)})
    for _ in range(args.warmup):
        cpu_sample_hydro(dem, thr, O=O)
    vals, dets = [], []
    for _ in range(args.steps):
        v, det = cpu_sample_hydro(dem, thr, O=O)
        vals.append(v)
        dets.append(det)
    v = float(np.mean(vals))
    sd8 = float(np.mean([d["slope_d8_s"] for d in dets]))
    fc = float(np.mean([d["fill_crop_s"] for d in dets]))
    sweeps = dets[-1]["fill_crop_sweeps"]
    desc = ("hydro8192: slope + D8 over the full 8192x8192 DEM on %d cores (%.2f s), serial Gauss-Seidel fill "
            "(gap 1e-3) on a centred 1024x1024 crop (%d sweeps, %.2f s), its per-cell time scaled to the full "
            "raster" % (thr, sd8, sweeps, fc))
    return {
        "impl": "reference", "metric": "Mcells/s slope+D8+fill", "value": round(v, 4), "unit": "Mcells/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dem.size / v / 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded fBm, same DEM as the GPU arm)",
        "config": {"workload": desc, "rows": 8192, "cols": 8192,
                   "slope_d8_size": "8192x8192 (full)", "fill_size": "1024x1024 crop (scaled per cell)"},
        "cpu_baseline": {"value": round(v, 4), "unit": "Mcells/s", "cores": thr, "kind": "port", "sample": desc},
        "slope_d8_full_size": {"threads": thr, "s": round(sd8, 3), "Mcells_s": round(dem.size / sd8 / 1e6, 2)},
        "slope_d8_one_thread": {"threads": 1, "s": round(t1, 3), "Mcells_s": round(n1 / t1 / 1e6, 2)},
        "fill_crops": crops,
        # the crops' fill rate fitted as a power of the side and carried to the full raster (informative)
        "fill_rate_extrapolated_8192": {"Mcells_s": round(float(np.exp(np.polyval(np.polyfit(
            np.log([c["side"] for c in crops]), np.log([c["Mcells_s"] for c in crops]), 1), np.log(8192)))), 5),
            "method": "least-squares line through log(rate) against log(side) of the three crops"},
        "e2e": {"value": round(v, 4), "unit": "Mcells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-sub", action="store_true", help="default workload only: skip the slope32768 and "
                    "batch512 sub-records")
    ap.add_argument("--workload", default="hydro8192",
                    choices=["hydro8192", "hydro2048", "slope32768", "slope8192", "slope1024", "batch512",
                             "sca16384", "sca4096", "grad8192", "mfd8192", "mfd2048", "load32768", "load8192",
                             "batchfill512"])
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        out = run_reference(args, ws, rank)
    elif args.workload.startswith("hydro"):
        out = run_hydro(args, ws, rank, local, int(args.workload[5:]))
        if args.workload == "hydro8192" and not args.no_sub:
            # the rest of the headline metric, timed in the same run: slope+D8
            # on the 32768^2 DEM (% of HBM), and the batched launch over 512
            # uneven rasters against the per-raster launches
            import gc
            import torch
            sub = {}
            for name, fn in (("slope32768", lambda: run_slope(args, ws, rank, local, 32768)),
                             ("batch512", lambda: run_batch(args, ws, rank, local)),
                             ("batchfill512", lambda: run_batch_fill(args, ws, rank, local))):
                gc.collect()
                torch.cuda.empty_cache()
                sub[name] = fn()
            out["sub"] = sub
    elif args.workload.startswith("sca"):
        out = run_sca(args, ws, rank, local, int(args.workload[3:]))
    elif args.workload.startswith("load"):
        out = run_load(args, ws, rank, local, int(args.workload[4:]))
    elif args.workload.startswith("mfd"):
        out = run_mfd(args, ws, rank, local, int(args.workload[3:]))
    elif args.workload == "grad8192":
        out = run_grad(args, ws, rank, local)
    elif args.workload == "batch512":
        out = run_batch(args, ws, rank, local)
    elif args.workload == "batchfill512":
        out = run_batch_fill(args, ws, rank, local)
    else:
        out = run_slope(args, ws, rank, local, int(args.workload[5:]))
    if rank == 0 and out is not None:
        print(json.dumps(out))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
