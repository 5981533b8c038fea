"""Throughput benchmark of the tile-matching hot path on GB300.

Workload (one "step"): the same-layer montage batch -- 4096 neighbour pairs
of uint8 overlap strips (W x 2048 or 2048 x W, W ~ U[164, 307]) cut from
2048^2 tiles of the seeded synthetic EM-like generator, +-40 px jitter, 2 %
decoy pairs, CorrPatches with a disc of radius 64 around the nominal offset
and the in-section legality rule.  One step runs the whole batch through
aln_corr_patches_batch.

  value   pairs/s with the strips already resident in HBM (device pointers)
  e2e     pairs/s through the same C-ABI call with pinned HOST buffers:
          host-to-device copies and the result read-back inside the timed region
  plain   the one-pair-per-call path (aln_corr_patches) on a sample of the
          same pairs: pairs/s and p50/p99 latency, with host buffers and with
          device-resident inputs (like for like with `value` and `e2e`)
  roofline  dominant kernel: the DRAM bytes one launch moves (the per-pair
          model checked against ncu dram__bytes) / its CUDA-event duration,
          against the measured HBM copy bandwidth; beside it the FP32 issue
          figure (counted FFT / product flops against the SMs' FMA peak at
          the sampled clock) and the canonical two-pass FFT count
  cpu_baseline  the oracle (FP64 C restatement of the reference) on the host
          cores, on a bounded sample of the same pairs
  configs the other workloads in bounded time, each with its parity table
          against the oracle: c1 plain 512^2 pairs, c3 the thumbnail angle
          sweep, c4 the uneven uint16 batch, c5 the served request stream
          (--no-extras leaves them out)

--impl reference times the reference algorithm's CPU implementation (the
oracle port; the reference's own compiled code exists only where its source
tree is mounted) on the host cores.

Multi-GPU (torchrun): pairs are independent, so every rank runs its own batch
of 4096 pairs (weak scaling, no collective on the data path); the step time
is the max over ranks.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "matched tile pairs/sec batched vs plain per-pair, 1 GB300, peak-exact; p50/p99 ms"
WORKLOAD = ("montage strips: 4096 pairs of W x 2048 / 2048 x W uint8 overlap strips "
            "(W ~ U[164,307]) of 2048^2 synthetic EM tiles, +-40 px jitter, 2% decoys; "
            "CorrPatches, disc radius 64, in-section legality")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--pairs", type=int, default=4096)
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--plain-sample", type=int, default=64)
    ap.add_argument("--cpu-sample", type=int, default=128)
    ap.add_argument("--parity-sample", type=int, default=16)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="montage line only (no c1/c3/c4/c5 figures)")
    ap.add_argument("--workload", default="montage",
                    choices=["montage", "sweep", "served", "uneven"],
                    help="montage: the strip batch (default); sweep: the thumbnail angle "
                         "sweep; served: the Poisson request stream through the server")
    ap.add_argument("--sweep-pairs", type=int, default=1024)
    ap.add_argument("--served-rates", default="2000,5000,10000,20000,50000")
    ap.add_argument("--served-requests", type=int, default=2000)
    ap.add_argument("--served-strips", type=int, default=512)
    ap.add_argument("--served-groups", type=int, default=32)
    ap.add_argument("--served-tiles", type=int, default=0,
                    help="served at tile scale: sweep tiles B keyed by this many distinct tile "
                         "ids (patch tiles by half as many), each reused by 6 neighbours in a "
                         "sliding window of active tiles; spectrum caches bounded by free HBM "
                         "(0: the pooled default, every group keyed once)")
    ap.add_argument("--served-window", type=int, default=32,
                    help="tiles whose neighbour requests are in flight at once (--served-tiles)")
    ap.add_argument("--uneven-pairs", type=int, default=20000)
    ap.add_argument("--c1-pairs", type=int, default=64)
    return ap.parse_args()


# ---------------------------------------------------------------------------
# distributed plumbing
# ---------------------------------------------------------------------------

def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def dist_init(ws, backend):
    if ws <= 1:
        return None
    import torch.distributed as dist
    dist.init_process_group(backend=backend)
    return dist


def max_over_ranks(dist, value, device=None):
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.lines = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# algorithmic bytes (canonical two-pass FFT accounting, one read + one write
# of the array per 1D pass; H = Ny*(Nx/2+1) complex FP32 = 8H bytes)
# ---------------------------------------------------------------------------

def fft_shape(w1, h1, w2, h2):
    """The reference's FFT grid (FFTSize per axis)."""
    def cp2(n):
        p = 1
        while p < n:
            p *= 2
        return p
    return cp2(w1 + w2 - 1), cp2(h1 + h2 - 1)


def solved_grid(pair):
    """(w_s, h_s, Nx, Ny, nseg) of one AlnPair as the library solves it: the
    frame (wide pairs transposed), the transform grid it chooses (the
    smallest power-of-two grid that keeps the disc's lags free of
    wrap-around) and the column segments (0: one column transform)."""
    import alignment_projects_gb300 as aln
    nx, ny, nseg, tr = aln.corr_patches_grid(pair)
    w, h = pair.a.w, pair.a.h
    if tr:
        w, h = h, w
    return w, h, nx, ny, nseg


def alg_bytes_per_pair(grid, e=1):
    """Canonical bytes per kernel (one read + one write of the array per 1D
    pass) for one pair of w x h strips (both the same size here), on the
    transforms the pair is solved with.  One column transform: the two-pass
    count on the Nx x Ny grid (H = Ny (Nx/2+1)).  Segmented columns (nseg
    segments of Ny points): the row pass writes the h rows' spectra, each
    column makes 2 nseg forward transforms, nseg products and one inverse."""
    w, h, Nx, Ny, nseg = grid
    L1 = Nx // 2 + 1
    H = Ny * L1
    inv_rows = 8 * H + 4 * Nx * Ny                    # c2r row pass
    if nseg:
        rows = 2 * (w * h * e + 8 * L1 * h)
        cols = (2 * nseg * 16 + nseg * 24 + 16) * H
    else:
        rows = 2 * (w * h * e + 8 * H)                # r2c row passes, both images
        cols = 16 * H + 16 * H + 24 * H + 16 * H      # column passes b, a; product; c2r column pass
    return {
        "k_rowfft": rows, "k2_rowfft": rows,
        "k_colfft": 16 * H,
        "k_corrcol": cols - 16 * H,
        # fused: b and a columns in one kernel (the segmented form when nseg)
        "k2_corrseg" if nseg else "k2_corrcol": cols,
        "k_lagrow": inv_rows, "k2_lagrow": inv_rows,
    }


def dram_model_per_pair(grid, e=1, wy=129):
    """DRAM bytes per pair the fused kernels move (each array read or written
    once): k2_rowfft reads both strips and writes both row spectra T (rows < h
    only); k2_corrcol and k2_corrseg read both T and write the window rows Q
    (k2_corrseg's re-reads of b's rows shared by neighbouring segments come
    from L2); k2_lagrow reads Q.  Checked against ncu dram__bytes (the
    committed ncu summaries of k2_corrcol and k2_corrseg)."""
    ws, hs, Nx, Ny, nseg = grid
    L1 = Nx // 2 + 1
    cols = 16 * L1 * hs + 8 * L1 * wy
    return {"k2_rowfft": 2 * ws * hs * e + 16 * L1 * hs,
            "k2_corrseg" if nseg else "k2_corrcol": cols,
            "k2_lagrow": 8 * L1 * wy}


def fft_flops(n):
    """Flops of one complex FFT of n points, the standard 5 n log2 n count."""
    return 5.0 * n * max(1, int(n).bit_length() - 1)


def flops_per_pair(grid, wy=129):
    """FP32 flops per pair of the fused FFT kernels (5 n log2 n per complex
    transform, 6 per complex product plus 2 to accumulate it, a real
    transform of n points as a complex one of n/2 plus n/2 split butterflies
    of 10 flops).  Row pass: both images' h rows.  Columns: per column of the
    L+1 spectrum columns, 2 nseg segment transforms of NS points, nseg
    products and one inverse (unsegmented: 2 forward and 1 inverse of Ny).
    Lag rows: one inverse real transform per window row."""
    ws, hs, Nx, Ny, nseg = grid
    L = Nx // 2
    real_fft = fft_flops(L) + 10.0 * L
    rows = 2 * hs * real_fft
    if nseg:
        cols = (L + 1) * ((2 * nseg + 1) * fft_flops(Ny) + 8.0 * nseg * Ny)
    else:
        cols = (L + 1) * (3 * fft_flops(Ny) + 8.0 * Ny)
    return {"k2_rowfft": rows, "k2_corrseg" if nseg else "k2_corrcol": cols,
            "k2_lagrow": wy * real_fft}


def fp32_peak_tflops(sm_mhz, sms=152):
    """FP32 FMA issue peak: SMs x 128 lanes x 2 flops x clock."""
    return sms * 128 * 2 * sm_mhz * 1e6 / 1e12


def fp32_block(flops, seconds, clocks):
    """Counted FP32 flops over `seconds` against the FMA peak at the median
    SM clock sampled in the timed region (max clock if none was sampled)."""
    mhz = (clocks or {}).get("sm_mhz") or (clocks or {}).get("sm_max_mhz") or 2070.0
    peak = fp32_peak_tflops(mhz)
    ach = flops / seconds / 1e12 if seconds > 0 else 0.0
    return {"flops": flops, "achieved_tflops": ach, "peak_tflops": peak,
            "frac": ach / peak, "sm_mhz": mhz,
            "accounting": "5 n log2 n per complex transform, 8 per accumulated product"}


# ---------------------------------------------------------------------------
# CPU baseline (oracle port, all host threads)
# ---------------------------------------------------------------------------

def cpu_pairs_per_s(pairs_host, threads):
    """Run the oracle's CorrPatches on every pair with `threads` host threads
    (ctypes releases the GIL); returns (pairs/s, per-pair seconds)."""
    import concurrent.futures as cf
    import oracle as O
    orc = O.Oracle()
    lg = O.legal(O.RGN_SECTION, 1500, 1500, 30000)
    prepared = []
    for a, b in pairs_host:
        A, VA = O.image_to_points(a)
        B, VB = O.image_to_points(b)
        prepared.append((A, VA, B, VB))

    def one(t):
        A, VA, B, VB = t
        t0 = time.perf_counter()
        o = orc.corr_patches(A, VA, B, VB, 0, 0, 64, lg)
        return time.perf_counter() - t0, o

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        res = list(ex.map(one, prepared))
    wall = time.perf_counter() - t0
    return len(prepared) / wall, [r[0] for r in res], [r[1] for r in res], wall


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


# ---------------------------------------------------------------------------
# reference arm
# ---------------------------------------------------------------------------

def run_reference(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return 0
    import torch
    from alignment_projects_gb300 import synth
    import oracle as O
    O.build()
    dev = "cuda:%d" % local if torch.cuda.is_available() else "cpu"
    threads = host_threads()
    sample = max(threads, args.cpu_sample)
    batch = synth.montage_batch_torch(args.seed, sample, dev)
    host = [(p["a"].cpu().numpy(), p["b"].cpu().numpy()) for p in batch]
    for _ in range(args.warmup):
        cpu_pairs_per_s(host[:threads], threads)
    times = []
    for _ in range(args.steps):
        pps, per, _, wall = cpu_pairs_per_s(host, threads)
        times.append(wall)
    tot = sum(times)
    value = args.steps * len(host) / tot
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "pairs/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * tot / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "pairs_per_step": len(host),
                   "note": "bounded sample of the 4096-pair batch per step"},
        "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": threads, "kind": "port",
                         "sample": "%d montage strip pairs per step (first pairs of the batch),"
                                   " FP64 C restatement of CorrPatches" % len(host)},
        "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def build_pair_array(batch, on_device, host_bufs=None):
    import ctypes as C
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300.native import AlnPair, AlnResult, AlnImage
    n = len(batch)
    arr = (AlnPair * n)()
    lg = aln.legal(aln.RGN_SECTION, 1500, 1500, 30000)
    for k, p in enumerate(batch):
        for slot, key in ((0, "a"), (1, "b")):
            if on_device:
                t = p[key]
                ptr = t.data_ptr()
            else:
                t = host_bufs[k][slot]
                ptr = t.data_ptr()
            im = AlnImage(ptr, aln.U8, t.shape[1], t.shape[0], t.shape[1], 0, 0,
                          1 if on_device else 0)
            if slot == 0:
                arr[k].a = im
            else:
                arr[k].b = im
        arr[k].ox, arr[k].oy, arr[k].radius = p["ox"], p["oy"], p["radius"]
        arr[k].legal = lg
    out = (AlnResult * n)()
    return arr, out


def run_gpu(args):
    import ctypes as C
    import torch
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300 import synth

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = dist_init(ws, "nccl")
    dev = torch.device("cuda", local)
    L = aln.lib()
    ctx = aln.Context(local)

    batch = synth.montage_batch_torch(args.seed + 7919 * rank, args.pairs, dev)
    torch.cuda.synchronize()
    n = len(batch)
    strip_bytes = sum(p["a"].numel() + p["b"].numel() for p in batch)

    # ---- device-resident inputs --------------------------------------------
    arr_d, out_d = build_pair_array(batch, True)

    def step_dev():
        rc = L.aln_corr_patches_batch(ctx.h, n, arr_d, out_d)
        if rc < 0:
            raise RuntimeError(L.aln_last_error(ctx.h).decode())

    for _ in range(args.warmup):
        step_dev()
    ctx.set_profiling(True)
    ctx.profile_reset()
    clk = ClockSampler(local)
    clk.start()
    barrier(dist)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        step_dev()
    e1.record()
    torch.cuda.synchronize()
    barrier(dist)
    ms_dev = e0.elapsed_time(e1)
    clocks = clk.stop()
    prof = ctx.profile()
    cdev = ctx.counters()
    launches = cdev["launches"]
    ctx.set_profiling(False)
    ms_dev = max_over_ranks(dist, ms_dev, dev)
    value = ws * n * args.steps / (ms_dev / 1000.0)

    # ---- roofline of the dominant kernel ------------------------------------
    ours = {k: v for k, v in prof.items()}
    dom = max(ours, key=lambda k: ours[k][1])
    dom_launches, dom_ms = ours[dom]
    grids = [solved_grid(arr_d[k]) for k in range(n)]
    grid_hist, ref_hist = {}, {}
    for g in grids:
        key = "%dx%d" % (g[2], g[3]) + (" in %d segments" % g[4] if g[4] else "")
        grid_hist[key] = grid_hist.get(key, 0) + 1
        rk = "%dx%d" % fft_shape(g[0], g[1], g[0], g[1])
        ref_hist[rk] = ref_hist.get(rk, 0) + 1
    launch_s = dom_ms / dom_launches / 1000.0
    per_launch = args.steps / max(1, dom_launches)
    alg_per_launch = sum(alg_bytes_per_pair(g).get(dom, 0) for g in grids) * per_launch
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        peak = json.load(open(peaks_path))["hbm_gbs"]
        peak_src = "measured"
    else:
        peak, peak_src = 6800.0, "fallback"
    # DRAM bytes one launch of the dominant kernel moves (each array read or
    # written once; the model is checked against ncu dram__bytes)
    traffic = sum(dram_model_per_pair(g).get(dom, 0) for g in grids) * per_launch
    achieved = traffic / launch_s / 1e9
    flops_launch = sum(flops_per_pair(g).get(dom, 0) for g in grids) * per_launch
    # the FFT passes together (row, column and inverse passes with the
    # product), on the same DRAM accounting, over the kernels' summed time
    fft_k = ("k2_rowfft", "k2_corrcol", "k2_corrseg", "k2_lagrow")
    fft_ms = sum(ours[k][1] for k in fft_k if k in ours)
    fft_dram = sum(sum(dram_model_per_pair(g).get(k, 0) for k in fft_k)
                   for g in grids) * args.steps
    fft_flops = sum(sum(flops_per_pair(g).get(k, 0) for k in fft_k)
                    for g in grids) * args.steps
    fft_gbs = fft_dram / (fft_ms / 1000.0) / 1e9 if fft_ms > 0 else None

    # ---- end to end through the C ABI with pinned host buffers -------------
    # host strips in one pinned buffer, pair after pair (a, b), as a tile
    # loader would stage them; the library copies adjacent images at once
    pinned = torch.empty(strip_bytes, dtype=torch.uint8, pin_memory=True)
    host_bufs = []
    off = 0
    for p in batch:
        views = []
        for key in ("a", "b"):
            t = p[key]
            v = pinned[off:off + t.numel()].view(t.shape)
            v.copy_(t)
            off += t.numel()
            views.append(v)
        host_bufs.append(tuple(views))
    arr_h, out_h = build_pair_array(batch, False, host_bufs)

    def step_host():
        rc = L.aln_corr_patches_batch(ctx.h, n, arr_h, out_h)
        if rc < 0:
            raise RuntimeError(L.aln_last_error(ctx.h).decode())

    step_host()
    ctx.set_profiling(True)
    ctx.profile_reset()
    barrier(dist)
    torch.cuda.synchronize()
    e0.record()
    t_host = time.perf_counter()
    for _ in range(args.steps):
        step_host()
    e1.record()
    torch.cuda.synchronize()
    t_host = time.perf_counter() - t_host
    barrier(dist)
    ms_e2e = max_over_ranks(dist, e0.elapsed_time(e1), dev)
    cnt = ctx.counters()
    prof_e2e = ctx.profile()
    ctx.set_profiling(False)
    e2e_value = ws * n * args.steps / (ms_e2e / 1000.0)
    stage_ms = prof_e2e.get("h2d_staging", (0, 0.0))[1] / args.steps
    staging_gbs = strip_bytes / (stage_ms / 1000.0) / 1e9 if stage_ms > 0 else None

    # the host link alone: one pinned-to-device copy of the step's strips
    # (bounds e2e when the copies cannot hide behind the kernels)
    probe = torch.empty(strip_bytes, dtype=torch.uint8, device=dev)
    torch.cuda.synchronize()
    e0.record()
    probe.copy_(pinned, non_blocking=True)
    e1.record()
    torch.cuda.synchronize()
    h2d_gbs = strip_bytes / (e0.elapsed_time(e1) / 1000.0) / 1e9
    # the same bytes as four concurrent copies (several copy engines)
    streams = [torch.cuda.Stream(device=dev) for _ in range(4)]
    q = (strip_bytes + 3) // 4
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k, st in enumerate(streams):
        with torch.cuda.stream(st):
            probe[k * q:(k + 1) * q].copy_(pinned[k * q:(k + 1) * q], non_blocking=True)
    torch.cuda.synchronize()
    h2d_gbs4 = strip_bytes / (time.perf_counter() - t0) / 1e9
    del probe

    # results agree between the two input paths
    same = all((out_d[k].status, out_d[k].peak_x, out_d[k].peak_y, out_d[k].r) ==
               (out_h[k].status, out_h[k].peak_x, out_h[k].peak_y, out_h[k].r)
               for k in range(n))

    line = None
    if rank == 0:
        # ---- plain one-pair-per-call path ------------------------------------
        lat = []
        lg = aln.legal(aln.RGN_SECTION, 1500, 1500, 30000)
        from alignment_projects_gb300.native import AlnResult, AlnImage
        r = AlnResult()
        for k in range(min(args.plain_sample, n)):
            ha, hb = host_bufs[k]
            ia = AlnImage(ha.data_ptr(), aln.U8, ha.shape[1], ha.shape[0], ha.shape[1], 0, 0, 0)
            ib = AlnImage(hb.data_ptr(), aln.U8, hb.shape[1], hb.shape[0], hb.shape[1], 0, 0, 0)
            t0 = time.perf_counter()
            rc = L.aln_corr_patches(ctx.h, C.byref(ia), C.byref(ib), 0, 0, 64, C.byref(lg),
                                    C.byref(r))
            lat.append(time.perf_counter() - t0)
            assert rc >= 0
        lat_ms = sorted(1000.0 * x for x in lat[1:])
        plain_pps = len(lat_ms) / (sum(lat_ms) / 1000.0)
        # the same calls with device-resident inputs (like for like with value)
        lat_d = []
        for k in range(min(args.plain_sample, n)):
            ia, ib = arr_d[k].a, arr_d[k].b
            t0 = time.perf_counter()
            rc = L.aln_corr_patches(ctx.h, C.byref(ia), C.byref(ib), 0, 0, 64, C.byref(lg),
                                    C.byref(r))
            lat_d.append(time.perf_counter() - t0)
            assert rc >= 0
        lat_d_ms = sorted(1000.0 * x for x in lat_d[1:])
        plain_dev_pps = len(lat_d_ms) / (sum(lat_d_ms) / 1000.0)

        # ---- parity on a sample: batch result vs the oracle ------------------
        parity = None
        cpu = None
        threads = host_threads()
        if not args.no_cpu:
            samp = [(host_bufs[k][0].numpy(), host_bufs[k][1].numpy())
                    for k in range(min(n, max(args.cpu_sample, args.parity_sample)))]
            cpu_pps, per, outs, wall = cpu_pairs_per_s(samp, threads)
            per_ms = sorted(1000.0 * x for x in per)
            cpu = {"value": cpu_pps, "unit": "pairs/s", "cores": threads, "kind": "port",
                   "p50_ms_per_pair": per_ms[len(per_ms) // 2],
                   "p99_ms_per_pair": per_ms[min(len(per_ms) - 1, int(0.99 * len(per_ms)))],
                   "sample": "%d of the batch's pairs, FP64 C restatement of CorrPatches, "
                             "%.1f s wall on %d threads" % (len(samp), wall, threads)}
            ok = tot = 0
            max_dr = max_dp = 0.0
            for k, o in enumerate(outs):
                g = out_d[k]
                if o["status"] == 0 and o["r"] - o["second"] > 1e-3:
                    tot += 1
                    ok += (g.peak_x, g.peak_y) == (o["bigx"], o["bigy"])
                    max_dp = max(max_dp, abs(g.dx - o["dx"]), abs(g.dy - o["dy"]))
                max_dr = max(max_dr, abs(g.r - o["r"]))
            parity = {"pairs": len(outs), "peak_exact": ok, "peak_checked": tot,
                      "max_abs_dr": max_dr, "max_abs_dsubpix": max_dp}
        truth_ok = sum(1 for k, p in enumerate(batch)
                       if not p["decoy"] and (out_d[k].peak_x, out_d[k].peak_y) == p["truth"])
        decoys = [k for k, p in enumerate(batch) if p["decoy"]]
        rejected = sum(1 for k in decoys if out_d[k].r < 0.3)
        line = {
            "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_dev / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "pairs_per_step": n,
                       "fft": "transform grids (solved frame, wide pairs transposed): " +
                              ", ".join("%s x%d" % (g, c) for g, c in sorted(grid_hist.items())) +
                              "; the reference's FFTSize grids: " +
                              ", ".join("%s x%d" % (g, c) for g, c in sorted(ref_hist.items())),
                       "l2": "inputs %.2f GB per step > 129 MB L2" % (strip_bytes / 1e9),
                       "parallelism": "replicas x%d" % ws},
            "e2e": {"value": e2e_value, "unit": "pairs/s",
                    "h2d_bytes_per_step": cnt["h2d_bytes"] // args.steps,
                    "d2h_bytes_per_step": cnt["d2h_bytes"] // args.steps,
                    "staging_gbs": staging_gbs,
                    "staging_note": "the library's host-to-device staging (SM copies of the "
                                    "page-locked strips, overlapped with the previous "
                                    "window's kernels), CUDA events on its copy stream",
                    "copy_bound_pairs_per_s": (n / (strip_bytes / (staging_gbs * 1e9))
                                               if staging_gbs else None),
                    "torch_copy_gbs": h2d_gbs, "torch_copy_gbs_4_streams": h2d_gbs4},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                         "peak_source": peak_src, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic,
                         "accounting": "achieved = DRAM bytes per launch (each array read "
                                       "or written once: the per-pair model, checked against "
                                       "ncu dram__bytes in profiles/) / CUDA-event launch time",
                         "avg_launch_ms": dom_ms / dom_launches,
                         "fp32": fp32_block(flops_launch, launch_s, clocks),
                         "canonical_equiv_gbs": alg_per_launch / launch_s / 1e9,
                         "canonical_note": "the canonical two-pass FFT count (one read + one "
                                           "write of the array per 1D pass, on the transforms "
                                           "made) over the same time; the fused kernels keep "
                                           "those passes in registers and shared memory, so "
                                           "this is not a DRAM figure",
                         "fft_passes": {"kernels": list(fft_k), "dram_gbs": fft_gbs,
                                        "frac": fft_gbs / peak if fft_gbs else None,
                                        "fp32": fp32_block(fft_flops, fft_ms / 1000.0,
                                                           clocks)}},
            "cpu_baseline": cpu,
            "clocks": clocks,
            "gpu_launches": launches,
            "kernels_ms": {k: round(v[1], 3) for k, v in sorted(ours.items())},
            "kernels_ms_e2e": {k: round(v[1], 3) for k, v in sorted(prof_e2e.items())},
            "e2e_host_wall_ms_per_step": 1000.0 * t_host / args.steps,
            "host_ms_per_step": {"plan": cdev["host_plan_us"] / 1000.0 / args.steps,
                                 "chunk_prep": cdev["host_prep_us"] / 1000.0 / args.steps,
                                 "note": "device-resident timed region; planning precedes the "
                                         "first launch, chunk preparation overlaps the previous "
                                         "chunk's kernels"},
            "chunks_per_step": cnt["chunks"] / args.steps,
            "h2d_copies_per_step": cnt["h2d_copies"] / args.steps,
            "plain": {"pairs_per_s": plain_pps, "p50_ms": lat_ms[len(lat_ms) // 2],
                      "p99_ms": lat_ms[min(len(lat_ms) - 1, int(0.99 * len(lat_ms)))],
                      "sample": len(lat_ms), "inputs": "host buffers (copies in each call)"},
            "plain_device": {"pairs_per_s": plain_dev_pps,
                             "p50_ms": lat_d_ms[len(lat_d_ms) // 2],
                             "p99_ms": lat_d_ms[min(len(lat_d_ms) - 1,
                                                    int(0.99 * len(lat_d_ms)))],
                             "sample": len(lat_d_ms), "inputs": "device-resident"},
            "batched_over_plain": {"device_inputs": value / plain_dev_pps,
                                   "host_inputs": e2e_value / plain_pps},
            "batch_latency_ms": ms_dev / args.steps,
            "parity": parity,
            "truth": {"found": truth_ok, "of": n - len(decoys), "decoys_rejected": rejected,
                      "decoys": len(decoys)},
            "host_vs_device_inputs_identical": same,
        }
    ctx.close()
    del batch, pinned, host_bufs, arr_h, arr_d
    torch.cuda.empty_cache()
    if line is not None:
        if not args.no_extras:
            line["configs"] = extras(args, local)
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


# ---------------------------------------------------------------------------
# the other configs in bounded time, embedded in the montage line
# ---------------------------------------------------------------------------

def c1_plain(args, local):
    """The plain-pair workload: 512^2 uint8 pairs (FFT 1024^2, full lag window,
    olap >= 32 x 32) through the plain one-pair-per-call path (host and
    device inputs) and as one batch; parity and the CPU port on the host
    cores for the same pairs."""
    import ctypes as C
    import torch
    import alignment_projects_gb300 as aln
    import oracle as O
    from alignment_projects_gb300 import synth
    from alignment_projects_gb300.native import AlnPair, AlnResult
    dev = torch.device("cuda", local)
    L = aln.lib()
    ctx = aln.Context(local)
    pairs = [synth.plain_pair(100 + k, n=512, margin=64) for k in range(args.c1_pairs)]
    lg = aln.legal(aln.RGN_MIN, 32, 32, 0)
    dts = [(torch.from_numpy(p.a).to(dev), torch.from_numpy(p.b).to(dev)) for p in pairs]
    torch.cuda.synchronize()
    r = AlnResult()
    lat_h, lat_d = [], []
    for k, p in enumerate(pairs):
        ia, ib = aln.image(p.a), aln.image(p.b)
        t0 = time.perf_counter()
        assert L.aln_corr_patches(ctx.h, C.byref(ia), C.byref(ib), 0, 0, 4096, C.byref(lg),
                                  C.byref(r)) >= 0
        lat_h.append(time.perf_counter() - t0)
        da, db = dts[k]
        ia = aln.native.AlnImage(da.data_ptr(), aln.U8, 512, 512, 512, 0, 0, 1)
        ib = aln.native.AlnImage(db.data_ptr(), aln.U8, 512, 512, 512, 0, 0, 1)
        t0 = time.perf_counter()
        assert L.aln_corr_patches(ctx.h, C.byref(ia), C.byref(ib), 0, 0, 4096, C.byref(lg),
                                  C.byref(r)) >= 0
        lat_d.append(time.perf_counter() - t0)
    arr = (AlnPair * len(pairs))()
    for k, p in enumerate(pairs):
        da, db = dts[k]
        arr[k].a = aln.native.AlnImage(da.data_ptr(), aln.U8, 512, 512, 512, 0, 0, 1)
        arr[k].b = aln.native.AlnImage(db.data_ptr(), aln.U8, 512, 512, 512, 0, 0, 1)
        arr[k].radius = 4096
        arr[k].legal = lg
    out = (AlnResult * len(pairs))()
    L.aln_corr_patches_batch(ctx.h, len(pairs), arr, out)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    reps = 3
    for _ in range(reps):
        assert L.aln_corr_patches_batch(ctx.h, len(pairs), arr, out) >= 0
    e1.record()
    torch.cuda.synchronize()
    batch_pps = reps * len(pairs) / (e0.elapsed_time(e1) / 1000.0)
    ctx.close()

    def pct(v, q):
        v = sorted(1000.0 * x for x in v[1:])
        return v[min(len(v) - 1, int(q * len(v)))]
    res = {"workload": "512^2 uint8 pairs of the synthetic EM field, offsets U{-64..64}^2, "
                       "noise 8 DN; CorrPatches, full window, olap >= 32 x 32; FFT 1024^2",
           "pairs": len(pairs),
           "plain_host": {"pairs_per_s": (len(lat_h) - 1) / sum(lat_h[1:]),
                          "p50_ms": pct(lat_h, 0.5), "p99_ms": pct(lat_h, 0.99)},
           "plain_device": {"pairs_per_s": (len(lat_d) - 1) / sum(lat_d[1:]),
                            "p50_ms": pct(lat_d, 0.5), "p99_ms": pct(lat_d, 0.99)},
           "batched_device_pairs_per_s": batch_pps,
           "truth": sum(1 for k, p in enumerate(pairs)
                        if (out[k].peak_x, out[k].peak_y) == p.truth)}
    if not args.no_cpu:
        import concurrent.futures as cf
        orc = O.Oracle()
        lo = O.legal(O.RGN_MIN, 32, 32, 0)
        prep = []
        for p in pairs[:args.parity_sample]:
            A, VA = O.image_to_points(p.a)
            B, VB = O.image_to_points(p.b)
            prep.append((A, VA, B, VB))
        threads = host_threads()

        def one(t):
            t0 = time.perf_counter()
            o = orc.corr_patches(t[0], t[1], t[2], t[3], 0, 0, 4096, lo)
            return o, time.perf_counter() - t0
        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(max_workers=threads) as ex:
            got = list(ex.map(one, prep))
        wall = time.perf_counter() - t0
        per = sorted(1000.0 * g[1] for g in got)
        res["cpu_baseline"] = {"value": len(prep) / wall, "unit": "pairs/s", "cores": threads,
                               "kind": "port", "p50_ms_one_core": per[len(per) // 2],
                               "p99_ms_one_core": per[min(len(per) - 1, int(0.99 * len(per)))],
                               "sample": "%d pairs" % len(prep)}
        res["parity"] = corr_parity([out[k] for k in range(len(prep))], [g[0] for g in got])
    return res


def corr_parity(gpu, orc_outs):
    """CorrPatches parity table: integer peak equal wherever the oracle's
    top-two margin exceeds 1e-3, max |dr|, max sub-pixel difference."""
    ok = chk = 0
    dr = dp = 0.0
    for g, o in zip(gpu, orc_outs):
        dr = max(dr, abs(g.r - o["r"]))
        if o["status"] == 0 and o["r"] - o["second"] > 1e-3:
            chk += 1
            ok += (g.peak_x, g.peak_y) == (o["bigx"], o["bigy"])
            dp = max(dp, abs(g.dx - o["dx"]), abs(g.dy - o["dy"]))
    return {"pairs": len(orc_outs), "peak_checked": chk, "peak_exact": ok,
            "max_abs_dr": dr, "max_abs_dsubpix": dp}


def extras(args, local):
    """c1, c3, c4 and c5 in bounded time (rank 0 of the montage run)."""
    import copy
    out = {}
    sub = copy.copy(args)
    sub.steps = min(args.steps, 3)
    sub.warmup = min(args.warmup, 3)
    for name, fn in (("c1_plain", lambda: c1_plain(sub, local)),
                     ("c3_sweep", lambda: run_sweep(sub, embedded=True)),
                     ("c4_uneven", lambda: run_uneven(sub, embedded=True)),
                     ("c5_served", lambda: run_served(sub, embedded=True))):
        t0 = time.perf_counter()
        try:
            out[name] = fn()
        except Exception as e:   # a failing extra must not lose the headline line
            out[name] = {"error": repr(e)[:300]}
        if isinstance(out[name], dict):
            out[name]["bench_wall_s"] = round(time.perf_counter() - t0, 1)
    return out


# ---------------------------------------------------------------------------
# thumbnail angle sweep (--workload sweep)
# ---------------------------------------------------------------------------

SWEEP_WORKLOAD = ("thumbnail angle sweep: pairs of 256^2 FP64 thumbnails (8x box-averaged "
                  "2048^2 synthetic tiles, B rotated U[-10,10] deg, +-30 px, gain 0.9-1.1, "
                  "noise 5, normalised); CThmScan DenovoBestAngle(0, 10, 0.5), ConstXY, "
                  "CorrImagesS, reqArea 3125, no disc, no pretweaks")
SWEEP_REQ_AREA = 3125


def sweep_thumbs(batch):
    """Host thumbnails -> AlnThumbs array (A as a full grid, B as a raster)."""
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300.native import AlnThumbs
    arr = (AlnThumbs * len(batch))()
    keep = []
    for k, p in enumerate(batch):
        ta = np.ascontiguousarray(p["ta"].cpu().numpy())
        tb = np.ascontiguousarray(p["tb"].cpu().numpy())
        keep += [ta, tb]
        arr[k].a = ta.ctypes.data
        arr[k].a_mask = None
        arr[k].a_h, arr[k].a_w = ta.shape
        arr[k].a_stride = ta.shape[1]
        arr[k].a_x0 = arr[k].a_y0 = 0
        arr[k].b = aln.image(tb)
        arr[k].req_area = SWEEP_REQ_AREA
        arr[k].olap1d = 0
    return arr, keep


def sweep_oracle(batch, threads):
    """The oracle's DenovoBestAngle on every pair with `threads` host threads."""
    import concurrent.futures as cf
    import oracle as O
    orc = O.Oracle()
    prep = []
    for p in batch:
        A, VA = O.image_to_points(p["ta"].cpu().numpy())
        B, VB = O.image_to_points(p["tb"].cpu().numpy())
        prep.append((A, VA, B, VB))

    def one(t):
        return orc.thm_search(*t, SWEEP_REQ_AREA, mode=0, ang0=0.0, hfang=10.0, step=0.5)

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        res = list(ex.map(one, prep))
    return res, time.perf_counter() - t0


def run_sweep(args, embedded=False):
    import ctypes as C
    import torch
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300 import synth
    from alignment_projects_gb300.native import AlnThmParams, AlnThmResult

    ws, rank, local = dist_env()
    threads = host_threads()
    if args.impl == "reference":
        if rank != 0:
            return 0
        import oracle as O
        O.build()
        dev = "cuda:%d" % local if torch.cuda.is_available() else "cpu"
        batch = synth.thumb_batch_torch(3, threads, dev)
        sweep_oracle(batch[:1], 1)
        tot = 0.0
        for _ in range(args.steps):
            _, wall = sweep_oracle(batch, threads)
            tot += wall
        value = args.steps * len(batch) / tot
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": value, "unit": "pairs/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * tot / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": SWEEP_WORKLOAD, "pairs_per_step": len(batch),
                       "note": "bounded sample of the 1024-pair sweep per step"},
            "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": threads, "kind": "port",
                             "sample": "%d thumbnail pairs per step, FP64 C restatement of "
                                       "CThmScan + CorrImagesS" % len(batch)},
            "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}), flush=True)
        return 0

    if embedded:
        ws, rank = 1, 0
    torch.cuda.set_device(local)
    dist = None if embedded else dist_init(ws, "nccl")
    dev = torch.device("cuda", local)
    L = aln.lib()
    ctx = aln.Context(local)
    batch = synth.thumb_batch_torch(3 + 7919 * rank, args.sweep_pairs, dev)
    torch.cuda.synchronize()
    n = len(batch)
    arr, keep = sweep_thumbs(batch)
    P = AlnThmParams()
    P.rthresh, P.nbmaxht, P.constxy, P.pretweak, P.usecorrr = 0.3, 0.75, 1, 0, 1
    P.ox, P.oy, P.rx, P.ry = 0, 0, -1, -1
    for i, v in enumerate((1, 0, 0, 0, 1, 0)):
        P.tdfm[i] = v
    out = (AlnThmResult * n)()

    def step(m=n):
        rc = L.aln_thm_search_batch(ctx.h, m, arr, C.byref(P), aln.THM_DENOVO, 0.0, 10.0, 0.5,
                                    out)
        if rc < 0:
            raise RuntimeError(L.aln_last_error(ctx.h).decode())

    for _ in range(args.warmup):
        step(min(n, 64))
    ctx.set_profiling(True)
    ctx.profile_reset()
    c0 = ctx.counters()
    clk = ClockSampler(local)
    clk.start()
    barrier(dist)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    barrier(dist)
    ms = max_over_ranks(dist, e0.elapsed_time(e1), dev)
    clocks = clk.stop()
    prof = ctx.profile()
    c1 = ctx.counters()
    ctx.set_profiling(False)
    value = ws * n * args.steps / (ms / 1000.0)
    calls = sum(o.ncalls for o in out)
    res = [{"A": o.A, "X": o.X, "Y": o.Y, "R": o.R, "err": o.err} for o in out]
    line = None
    if rank == 0:
        truth = sum(1 for r, p in zip(res, batch) if r["err"] == 0 and abs(r["A"] + p["theta"]) < 0.5)
        cpu = parity = None
        if not args.no_cpu:
            samp = batch[:threads]
            orc, wall = sweep_oracle(samp, threads)
            cpu = {"value": len(samp) / wall, "unit": "pairs/s", "cores": threads, "kind": "port",
                   "sample": "%d of the sweep's pairs, FP64 C restatement of CThmScan + "
                             "CorrImagesS, %.1f s wall on %d threads" % (len(samp), wall, threads)}
            parity = sweep_parity(res, orc)
        line = {
            "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": SWEEP_WORKLOAD, "pairs_per_step": n,
                       "fft": "1024 x 1024 (512 x 512 at exactly 0 deg)",
                       "parallelism": "replicas x%d" % ws},
            "e2e": {"value": value, "unit": "pairs/s",
                    "h2d_bytes_per_step": (c1["h2d_bytes"] - c0["h2d_bytes"]) // args.steps,
                    "d2h_bytes_per_step": (c1["d2h_bytes"] - c0["d2h_bytes"]) // args.steps,
                    "note": "the sweep API takes host thumbnails: value is end to end"},
            "correlator_calls_per_s": ws * calls * args.steps / (ms / 1000.0),
            "calls_per_pair": calls / n,
            "cpu_baseline": cpu, "clocks": clocks,
            "gpu_launches": c1["launches"] - c0["launches"],
            "kernels_ms": {k: round(v[1], 3) for k, v in sorted(prof.items())},
            "parity": parity,
            "truth": {"angle_within_0.5deg": truth, "of": n,
                      "err0": sum(1 for r in res if r["err"] == 0)},
        }
        if not embedded:
            print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()
    return line if embedded else 0


def sweep_parity(res, orc):
    """The sweep's parity table against the oracle (oracle/sweep_bar.py):
    pairs whose decisions had no tie must land on the identical angle;
    bar_failures counts pairs outside the bar."""
    from oracle.sweep_bar import SweepStats, check
    st = SweepStats()
    fails = []
    for k, (g, o) in enumerate(zip(res, orc)):
        try:
            st.add(check(g, o, "pair %d" % k))
        except AssertionError:
            fails.append(k)
    t = st.table()
    t["same_err"] = sum(1 for g, o in zip(res, orc) if g["err"] == o["err"])
    t["bar_failures"] = len(fails)
    return t


# ---------------------------------------------------------------------------
# served request stream (--workload served)
# ---------------------------------------------------------------------------

SERVED_WORKLOAD = ("served request stream: Poisson arrivals at swept rates; 70% montage strip "
                   "pairs (CorrPatches, disc 64), 20% thumbnail sweeps (DenovoBestAngle on 256^2 "
                   "thumbnails), 10% 512^2 uint8 patch pairs (CorrPatches, full window); sweep "
                   "and patch tiles B each serve 6 neighbours (spectrum keys); continuous-batching "
                   "server, 2 workers")
SERVED_MIX = (0.7, 0.2, 0.1)


def served_pools(seed, dev, n_strips, n_groups):
    """Host inputs: montage strip pairs, thumbnail groups, patch groups."""
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300 import synth
    strips = [(p["a"].cpu().numpy(), p["b"].cpu().numpy(), p["ox"], p["oy"], p["radius"])
              for p in synth.montage_batch_torch(seed, n_strips, dev)]
    thumbs = []
    for g in range(n_groups):
        tb, tas, _ = synth.neighbour_group_torch(seed * 1000 + g, 6, dev)
        for ta in tas:
            T = aln.native.AlnThumbs()
            T.a = ta.ctypes.data
            T.a_mask = None
            T.a_h, T.a_w = ta.shape
            T.a_stride = ta.shape[1]
            T.a_x0 = T.a_y0 = 0
            T.b = aln.image(tb)
            T.req_area = SWEEP_REQ_AREA
            T.olap1d = 0
            T.b_key = 1_000_000 + g
            T._keep = (ta, tb)
            thumbs.append(T)
    patches = []
    for g in range(n_groups):
        b, a_s, _ = synth.patch_group(seed * 1000 + 500 + g, 6)
        for a in a_s:
            patches.append((a, b, 2_000_000 + g))
    return strips, thumbs, patches


def served_requests(pools, n, seed):
    """n prepared AlnRequest structs drawn with the 70/20/10 mix."""
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300.native import AlnRequest, _thm_params
    strips, thumbs, patches = pools
    rng = np.random.default_rng(seed)
    cls = rng.choice(3, size=n, p=SERVED_MIX)
    lg_s = aln.legal(aln.RGN_SECTION, 1500, 1500, 30000)
    lg_p = aln.legal(aln.RGN_MIN, 32, 32, 0)
    thm = _thm_params()
    reqs, keep = [], [lg_s, lg_p]
    ci = [0, 0, 0]
    for c in cls:
        r = AlnRequest()
        if c == 0:
            a, b, ox, oy, rad = strips[ci[0] % len(strips)]
            r.kind = aln.REQ_PATCHES
            r.pair.a, r.pair.b = aln.image(a), aln.image(b)
            r.pair.ox, r.pair.oy, r.pair.radius = ox, oy, rad
            r.pair.legal = lg_s
        elif c == 1:
            r.kind = aln.REQ_SWEEP
            r.thumbs = thumbs[ci[1] % len(thumbs)]
            r.thm = thm
            r.thm_mode, r.ang0, r.hfang, r.step = aln.THM_DENOVO, 0.0, 10.0, 0.5
        else:
            a, b, key = patches[ci[2] % len(patches)]
            r.kind = aln.REQ_PATCHES
            r.pair.a, r.pair.b = aln.image(a), aln.image(b)
            r.pair.radius = 4096
            r.pair.legal = lg_p
            r.pair.b_key = key
        ci[c] += 1
        reqs.append(r)
    return reqs, cls, keep


class TileWalk:
    """Tile ids 0..n-1 in a random order, `window` of them active at a time;
    each draw takes a random active tile, which retires after `uses` draws
    (its 6 neighbours) and lets the next id in."""

    def __init__(self, n, window, uses, seed):
        self.rng = np.random.default_rng(seed)
        self.order = self.rng.permutation(n)
        self.next = 0
        self.uses = uses
        self.active = []
        while len(self.active) < window and self.next < n:
            self.active.append([int(self.order[self.next]), 0])
            self.next += 1

    def draw(self):
        """(tile id, neighbour index), or None when every tile is used up."""
        if not self.active:
            return None
        k = int(self.rng.integers(len(self.active)))
        tile, used = self.active[k]
        self.active[k][1] += 1
        if self.active[k][1] >= self.uses:
            if self.next < len(self.order):
                self.active[k] = [int(self.order[self.next]), 0]
                self.next += 1
            else:
                self.active.pop(k)
        return tile, used


def served_tile_requests(pools, n_tiles, window, seed):
    """The tile-scale stream: the 70/20/10 mix until every one of n_tiles
    sweep tiles (keys 10^7 + id) has served its 6 neighbours; patch tiles
    (keys 2 * 10^7 + id) walk n_tiles / 2 ids at their own pace.  Pixels come
    from the pools (tile id modulo the pool), so distinct keys hold equal
    pixels -- the cache's promise runs one way only: equal keys, equal
    images."""
    import ctypes as C
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300.native import AlnRequest, AlnThumbs, _thm_params
    strips, thumbs, patches = pools
    rng = np.random.default_rng(seed)
    sweeps = TileWalk(n_tiles, window, 6, seed + 1)
    pw = TileWalk(max(1, n_tiles // 2), window, 6, seed + 2)
    lg_s = aln.legal(aln.RGN_SECTION, 1500, 1500, 30000)
    lg_p = aln.legal(aln.RGN_MIN, 32, 32, 0)
    thm = _thm_params()
    reqs, cls, keep = [], [], [lg_s, lg_p]
    n_groups = len(thumbs) // 6
    ci = 0
    while True:
        c = int(rng.choice(3, p=SERVED_MIX))
        r = AlnRequest()
        if c == 0:
            a, b, ox, oy, rad = strips[ci % len(strips)]
            ci += 1
            r.kind = aln.REQ_PATCHES
            r.pair.a, r.pair.b = aln.image(a), aln.image(b)
            r.pair.ox, r.pair.oy, r.pair.radius = ox, oy, rad
            r.pair.legal = lg_s
        elif c == 1:
            d = sweeps.draw()
            if d is None:
                break
            tile, j = d
            src = thumbs[(tile % n_groups) * 6 + j]
            T = AlnThumbs()
            C.memmove(C.addressof(T), C.addressof(src), C.sizeof(AlnThumbs))
            T.b_key = 10_000_000 + tile
            keep.append(T)
            r.kind = aln.REQ_SWEEP
            r.thumbs = T
            r.thm = thm
            r.thm_mode, r.ang0, r.hfang, r.step = aln.THM_DENOVO, 0.0, 10.0, 0.5
        else:
            d = pw.draw()
            if d is None:
                pw = TileWalk(max(1, n_tiles // 2), window, 6, seed + 3 + len(reqs))
                d = pw.draw()
            tile, j = d
            a, b, _ = patches[(tile % n_groups) * 6 + j]
            r.kind = aln.REQ_PATCHES
            r.pair.a, r.pair.b = aln.image(a), aln.image(b)
            r.pair.radius = 4096
            r.pair.legal = lg_p
            r.pair.b_key = 20_000_000 + tile
        reqs.append(r)
        cls.append(c)
    return reqs, np.array(cls), keep


def served_run(srv, reqs, rate, seed):
    """Submit reqs at Poisson times of `rate` per second; collect every reply.
    Returns (wall seconds first submit -> last reply, replies by index)."""
    import ctypes as C
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300.native import AlnReply
    L = aln.lib()
    n = len(reqs)
    gaps = np.random.default_rng(seed).exponential(1.0 / rate, n)
    t_arr = np.cumsum(gaps) - gaps[0]
    tickets = [0] * n
    index = {}
    done = {}
    lock = threading.Lock()

    def feed():
        t0 = time.perf_counter()
        tk = C.c_ulonglong()
        for i in range(n):
            while time.perf_counter() - t0 < t_arr[i]:
                pass
            rc = L.aln_server_submit(srv.h, C.byref(reqs[i]), C.byref(tk))
            if rc < 0:
                raise RuntimeError("submit refused")
            with lock:
                tickets[i] = tk.value
                index[tk.value] = i

    t_start = time.perf_counter()
    th = threading.Thread(target=feed)
    th.start()
    cap = 4096
    tk_buf = (C.c_ulonglong * cap)()
    rep_buf = (AlnReply * cap)()
    while len(done) < n:
        k = L.aln_server_collect(srv.h, cap, 200, tk_buf, rep_buf)
        for j in range(k):
            with lock:
                i = index.get(tk_buf[j])
            while i is None:   # reply raced ahead of the feeder's bookkeeping
                time.sleep(0)
                with lock:
                    i = index.get(tk_buf[j])
            r = rep_buf[j]
            done[i] = (r.status, r.total_ms, r.queue_ms, r.batch_size)
    wall = time.perf_counter() - t_start
    th.join()
    return wall, done


def run_served(args, embedded=False):
    import torch
    import alignment_projects_gb300 as aln

    ws, rank, local = dist_env()
    if embedded:
        ws, rank = 1, 0
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps({"impl": "reference", "unavailable":
                              "the reference has no request server; its per-pair CPU paths are "
                              "timed by --workload montage and --workload sweep"}), flush=True)
        return 0
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pools = served_pools(5, dev, args.served_strips, args.served_groups)
    torch.cuda.synchronize()
    tiles = getattr(args, "served_tiles", 0) if not embedded else 0
    # tile scale: each worker's spectrum cache bounded by free HBM alone
    srv = aln.Server(local, workers=2, cache_bytes=(1 << 64) - 1 if tiles else 0)
    rates = [float(r) for r in args.served_rates.split(",")]
    # warm-up: every class through the server
    reqs, cls, keep = served_requests(pools, 200, 11)
    served_run(srv, reqs, 2000.0, 12)
    clk = ClockSampler(local)
    clk.start()
    table = []
    for k, rate in enumerate(rates):
        if tiles:
            reqs, cls, keep = served_tile_requests(pools, tiles, args.served_window, 100 + k)
        else:
            reqs, cls, keep = served_requests(pools, args.served_requests, 100 + k)
        c0 = srv.counters()
        free0 = torch.cuda.mem_get_info(local)[0]
        wall, done = served_run(srv, reqs, rate, 200 + k)
        c1 = srv.counters()
        lat = np.array([done[i][1] for i in range(len(reqs))])
        bad = sum(1 for i in range(len(reqs)) if done[i][0] < 0)
        row = {"offered_rate": rate, "requests": len(reqs), "throughput": len(reqs) / wall,
               "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
               "mean_batch": float(np.mean([done[i][3] for i in range(len(reqs))])),
               "errors": bad,
               "spec_hits": c1["spec_hits"] - c0["spec_hits"],
               "spec_fills": c1["spec_fills"] - c0["spec_fills"],
               "spec_evictions": c1["spec_evictions"] - c0["spec_evictions"],
               "cache_gb_after": c1["spec_bytes"] / 1e9,
               "free_hbm_gb_before": free0 / 1e9,
               "free_hbm_gb_after": torch.cuda.mem_get_info(local)[0] / 1e9}
        if tiles:
            row["distinct_sweep_keys"] = int(tiles)
            row["distinct_patch_keys"] = int(max(1, tiles // 2))
        for c, name in enumerate(("strips", "sweeps", "patches")):
            m = cls == c
            if m.any():
                row[name + "_p50_ms"] = float(np.percentile(lat[m], 50))
                row[name + "_p99_ms"] = float(np.percentile(lat[m], 99))
        table.append(row)
    clocks = clk.stop()
    counters = srv.counters()
    srv.close()
    # the plain one-request-per-call path on the same mix
    ctx = aln.Context(local)
    strips, thumbs, patches = pools
    lg_s = aln.legal(aln.RGN_SECTION, 1500, 1500, 30000)
    lg_p = aln.legal(aln.RGN_MIN, 32, 32, 0)
    per = []
    for j in range(9):
        a, b, ox, oy, rad = strips[j]
        t0 = time.perf_counter()
        ctx.corr_patches(a, b, ox, oy, rad, lg_s)
        per.append(time.perf_counter() - t0)
    t_strip = float(np.median(per[1:]))
    per = []
    for j in range(5):
        t0 = time.perf_counter()
        ctx.thm_search_batch([thumbs[j]], mode=aln.THM_DENOVO)
        per.append(time.perf_counter() - t0)
    t_sweep = float(np.median(per[1:]))
    per = []
    for j in range(9):
        a, b, _ = patches[j]
        t0 = time.perf_counter()
        ctx.corr_patches(a, b, 0, 0, 4096, lg_p)
        per.append(time.perf_counter() - t0)
    t_patch = float(np.median(per[1:]))
    ctx.close()
    plain = 1.0 / (SERVED_MIX[0] * t_strip + SERVED_MIX[1] * t_sweep + SERVED_MIX[2] * t_patch)
    best = max(table, key=lambda r: r["throughput"])
    line = {
        "metric": METRIC, "value": best["throughput"], "unit": "requests/s", "n_gpus": 1,
        "steps": len(rates), "warmup": 1, "ms_per_step": None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": SERVED_WORKLOAD, "requests_per_rate": args.served_requests,
                   "rates": rates, "note": "one step = one offered rate; value = best throughput",
                   "tiles": tiles or None,
                   "tile_note": ("sweep tiles B keyed by %d distinct ids, patch tiles by %d, each "
                                 "reused by 6 neighbours (a sliding window of %d active tiles); "
                                 "caches bounded by free HBM" % (tiles, max(1, tiles // 2),
                                                                 args.served_window)
                                 if tiles else "pooled: %d sweep and %d patch keys"
                                 % (args.served_groups, args.served_groups))},
        "e2e": {"value": best["throughput"], "unit": "requests/s",
                "note": "host inputs through the server API: value is end to end"},
        "rates": table,
        "plain": {"requests_per_s": plain, "strip_ms": 1000 * t_strip, "sweep_ms": 1000 * t_sweep,
                  "patch_ms": 1000 * t_patch},
        "served_over_plain": best["throughput"] / plain,
        "server_counters": counters, "clocks": clocks}
    if embedded:
        return line
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# uneven-size uint16 batch (--workload uneven)
# ---------------------------------------------------------------------------

UNEVEN_WORKLOAD = ("uneven-size batch: pairs of uint16 patches (0-4095, mean 2048, std 480), "
                   "long side log-uniform in [64, 1024], aspect 1-4, random orientation, "
                   "offset within a quarter of the short side; CorrPatches, disc radius "
                   "short/2, olap >= 8 x 8; FFT sizes 128..2048 per axis")


def run_uneven(args, embedded=False):
    import ctypes as C
    import torch
    import alignment_projects_gb300 as aln
    import oracle as O
    from alignment_projects_gb300 import synth
    from alignment_projects_gb300.native import AlnPair, AlnResult, AlnImage

    ws, rank, local = dist_env()
    if embedded:
        ws, rank = 1, 0
    threads = host_threads()
    torch.cuda.set_device(local)
    dist = None if embedded else dist_init(ws, "nccl")
    dev = torch.device("cuda", local)
    L = aln.lib()
    ctx = aln.Context(local)
    batch = synth.uneven_batch_torch(4 + 7919 * rank, args.uneven_pairs, dev)
    torch.cuda.synchronize()
    n = len(batch)
    lg = aln.legal(aln.RGN_MIN, 8, 8, 0)

    def pair_array(host):
        arr = (AlnPair * n)()
        for k, p in enumerate(batch):
            ims = []
            for key in ("a", "b"):
                t = host[k][key] if host is not None else p[key]
                ims.append(AlnImage(t.data_ptr(), aln.U16, t.shape[1], t.shape[0], t.shape[1],
                                    0, 0, 0 if host is not None else 1))
            arr[k].a, arr[k].b = ims
            arr[k].ox, arr[k].oy, arr[k].radius = 0, 0, p["radius"]
            arr[k].legal = lg
        return arr, (AlnResult * n)()

    arr_d, out_d = pair_array(None)

    def run(arr, out):
        if L.aln_corr_patches_batch(ctx.h, n, arr, out) < 0:
            raise RuntimeError(L.aln_last_error(ctx.h).decode())

    for _ in range(args.warmup):
        run(arr_d, out_d)
    ctx.set_profiling(True)
    ctx.profile_reset()
    clk = ClockSampler(local)
    clk.start()
    barrier(dist)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        run(arr_d, out_d)
    e1.record()
    torch.cuda.synchronize()
    barrier(dist)
    ms = max_over_ranks(dist, e0.elapsed_time(e1), dev)
    clocks = clk.stop()
    prof = ctx.profile()
    cnt = ctx.counters()
    value = ws * n * args.steps / (ms / 1000.0)
    # the same batch on the fixed cost model's plans (autotuner off), and
    # the tuned plans again, both without the per-launch profiling events of
    # the timed region above (about 1200 launches per step here)
    ctx_fixed = aln.Context(local)
    ctx_fixed.set_tuning(False)
    out_f = (AlnResult * n)()
    if L.aln_corr_patches_batch(ctx_fixed.h, n, arr_d, out_f) < 0:
        raise RuntimeError(L.aln_last_error(ctx_fixed.h).decode())
    ctx.set_profiling(False)

    def timed(c, out):
        torch.cuda.synchronize()
        e0.record()
        for _ in range(args.steps):
            L.aln_corr_patches_batch(c.h, n, arr_d, out)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    ms_fixed = timed(ctx_fixed, out_f)
    ms_tuned = timed(ctx, out_d)
    chunks_fixed = ctx_fixed.counters()["chunks"] / (args.steps + 1)
    ctx_fixed.close()
    fixed_same_peaks = sum(1 for k in range(n) if (out_f[k].peak_x, out_f[k].peak_y) ==
                           (out_d[k].peak_x, out_d[k].peak_y))
    # end to end: the patches in one pinned buffer, pair after pair
    nbytes = sum(2 * (p["a"].numel() + p["b"].numel()) for p in batch)
    pinned = torch.empty(nbytes // 2, dtype=torch.int16, pin_memory=True)
    host, off = [], 0
    for p in batch:
        h = {}
        for key in ("a", "b"):
            t = p[key]
            v = pinned[off:off + t.numel()].view(t.shape)
            v.copy_(t)
            off += t.numel()
            h[key] = v
        host.append(h)
    arr_h, out_h = pair_array(host)
    run(arr_h, out_h)
    ctx.profile_reset()
    torch.cuda.synchronize()
    e0.record()
    for _ in range(args.steps):
        run(arr_h, out_h)
    e1.record()
    torch.cuda.synchronize()
    ms_e2e = max_over_ranks(dist, e0.elapsed_time(e1), dev)
    cnt2 = ctx.counters()
    ctx.set_profiling(False)
    line = None
    if rank == 0:
        same = all((out_d[k].peak_x, out_d[k].peak_y, out_d[k].r) ==
                   (out_h[k].peak_x, out_h[k].peak_y, out_h[k].r) for k in range(n))
        truth = sum(1 for k, p in enumerate(batch)
                    if (out_d[k].peak_x, out_d[k].peak_y) == p["truth"])
        cpu = parity = None
        if not args.no_cpu:
            import concurrent.futures as cf
            orc = O.Oracle()
            lo = O.legal(O.RGN_MIN, 8, 8, 0)
            samp = list(range(0, n, max(1, n // args.cpu_sample)))[:args.cpu_sample]
            prep = []
            for k in samp:
                a = batch[k]["a"].cpu().numpy().astype(np.uint16)
                b = batch[k]["b"].cpu().numpy().astype(np.uint16)
                A, VA = O.image_to_points(a)
                B, VB = O.image_to_points(b)
                prep.append((A, VA, B, VB, batch[k]["radius"]))
            t0 = time.perf_counter()
            with cf.ThreadPoolExecutor(max_workers=threads) as ex:
                outs = list(ex.map(lambda t: orc.corr_patches(t[0], t[1], t[2], t[3], 0, 0,
                                                                t[4], lo), prep))
            wall = time.perf_counter() - t0
            cpu = {"value": len(prep) / wall, "unit": "pairs/s", "cores": threads,
                   "kind": "port", "sample": "%d pairs spread over the batch, FP64 C "
                   "restatement of CorrPatches, %.1f s wall on %d threads"
                   % (len(prep), wall, threads)}
            parity = corr_parity([out_d[k] for k in samp], outs)
        line = {
            "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": UNEVEN_WORKLOAD, "pairs_per_step": n,
                       "input_bytes_per_step": nbytes, "parallelism": "replicas x%d" % ws},
            "e2e": {"value": ws * n * args.steps / (ms_e2e / 1000.0), "unit": "pairs/s",
                    "h2d_bytes_per_step": (cnt2["h2d_bytes"]) // args.steps,
                    "d2h_bytes_per_step": (cnt2["d2h_bytes"]) // args.steps},
            "cpu_baseline": cpu, "clocks": clocks, "gpu_launches": cnt["launches"],
            "autotuner": {"tuned_pairs_per_s": n * args.steps / (ms_tuned / 1000.0),
                          "fixed_plan_pairs_per_s": n * args.steps / (ms_fixed / 1000.0),
                          "tuned_over_fixed": ms_fixed / ms_tuned,
                          "note": "both timed without per-launch profiling events",
                          "classes_timed": ctx.counters()["tune_classes"],
                          "chunks_per_step_tuned": cnt["chunks"] / args.steps,
                          "chunks_per_step_fixed": chunks_fixed,
                          "same_peaks": fixed_same_peaks, "of": n},
            "chunks_per_step": cnt["chunks"] / args.steps,
            "kernels_ms": {k: round(v[1], 3) for k, v in sorted(prof.items())},
            "parity": parity,
            "truth": {"found": truth, "of": n},
            "host_vs_device_inputs_identical": same,
        }
        if not embedded:
            print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()
    return line if embedded else 0


def main():
    args = parse()
    if args.workload == "sweep":
        return run_sweep(args)
    if args.workload == "served":
        return run_served(args)
    if args.workload == "uneven":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the uneven batch's CPU "
                              "baseline is reported in the GPU line (cpu_baseline)"}), flush=True)
            return 0
        return run_uneven(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
