"""Benchmark: dense ampcor offset windows/s on the burst workload.

Workload: 12000 (down) x 8000 (across) complex64 burst pair (speckle + shift
recipe, quadratic offset field up to 3 px, 5 dB), window 128 x 64, half search
32, skip 64, raw oversampling 2, correlation oversampling 32, zoom 16:
184 x 123 = 22 632 windows per step.  Inputs (1.54 GB) exceed the 129 MB L2,
so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun every rank processes its own full burst (weak scaling, no
collective on the data path); rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "offset windows/sec (batched/served vs plain GPU) at ≤0.01 px err; p50/p99 latency"
SIZE = (12000, 8000)
PARAMS = dict(windowSizeHeight=128, windowSizeWidth=64, halfSearchRangeDown=32, halfSearchRangeAcross=32,
              skipSampleDown=64, skipSampleAcross=64, rawDataOversamplingFactor=2,
              corrSurfaceOverSamplingFactor=32, corrSurfaceZoomInWindow=16, derampMethod=1)
WORKLOAD = "burst 12000x8000 c64, window 128x64, half search 32, skip 64, raw 2, ovs 32, zoom 16"
FULL_CHECK = False  # check every window against the oracle (the 2048^2 plain workload runs in full)


def SCENE(H, W):
    from isce2_gb300 import synth
    return synth.scene_burst(H, W)


# the plain CPU-size workload: 2048^2, window 64^2, half search 20, skip 32,
# raw 2, ovs 16, zoom 8, deramp 0 (60 x 60 = 3 600 windows)
PLAIN_SMALL = dict(windowSizeHeight=64, windowSizeWidth=64, halfSearchRangeDown=20, halfSearchRangeAcross=20,
                   skipSampleDown=32, skipSampleAcross=32, rawDataOversamplingFactor=2,
                   corrSurfaceOverSamplingFactor=16, corrSurfaceZoomInWindow=8, derampMethod=0)


def geometry():
    H, W = SIZE
    p = dict(PARAMS)
    hs = p["halfSearchRangeDown"]
    p.update(referenceImageHeight=H, referenceImageWidth=W, secondaryImageHeight=H, secondaryImageWidth=W,
             referenceStartPixelDownStatic=hs, referenceStartPixelAcrossStatic=hs,
             numberWindowDown=(H - 2 * hs - p["windowSizeHeight"]) // p["skipSampleDown"],
             numberWindowAcross=(W - 2 * hs - p["windowSizeWidth"]) // p["skipSampleAcross"])
    return p


def b_win(p) -> int:
    """Algorithmic bytes of one window of the whole path: the complex64
    reference and search chips in, offset + SNR + covariance out."""
    Wh, Ww, hs = p["windowSizeHeight"], p["windowSizeWidth"], p["halfSearchRangeDown"]
    return 8 * (Wh * Ww + (Wh + 2 * hs) * (Ww + 2 * hs)) + 24


def stage_bytes_per_window(p) -> dict:
    """Algorithmic HBM bytes per window of each kernel (its inputs + outputs)."""
    Wh, Ww, hs, raw = p["windowSizeHeight"], p["windowSizeWidth"], p["halfSearchRangeDown"], p["rawDataOversamplingFactor"]
    zoom = min(p["corrSurfaceZoomInWindow"], 2 * raw * hs)
    hz = zoom // (2 * raw)
    zp = 2 * hz * raw
    ref_chip = 8 * Wh * Ww
    search_chip = 8 * (Wh + 2 * hs) * (Ww + 2 * hs)
    zoom_chip = 8 * (Wh + 2 * hz) * (Ww + 2 * hz)
    os_amp = 4 * raw * raw * (Wh * Ww + (Wh + 2 * hz) * (Ww + 2 * hz))
    return {"k_raw": ref_chip + search_chip + 56,
            "k_oversample2": ref_chip + zoom_chip + os_amp,
            "k_corr_os_tma": os_amp + 4 * zp * zp,
            "k_zoom": 4 * zp * zp + 56 + 24}


# --------------------------------------------------------------------------
# CPU leg (oracle port): runs in spawned worker processes only
# --------------------------------------------------------------------------
def _oracle_chunk(args):
    ref_path, sec_path, p, sel = args
    from oracle.ampcor_oracle import OracleParams, run_windows
    ref = np.load(ref_path, mmap_mode="r")
    sec = np.load(sec_path, mmap_mode="r")
    op = OracleParams(**{k: v for k, v in p.items() if k in OracleParams.__dataclass_fields__})
    st = op.constant_gross_starts(0, 0)
    out = run_windows(ref, sec, op, st, sel=np.asarray(sel), batch=8)
    return sel, out["offset"]


def cpu_oracle_timed(pool, cores, ref_path, sec_path, p, sel):
    chunks = [list(c) for c in np.array_split(np.asarray(sel), cores * 2) if len(c)]
    t0 = time.perf_counter()
    res = pool.map(_oracle_chunk, [(ref_path, sec_path, p, c) for c in chunks])
    dt = time.perf_counter() - t0
    idx = np.concatenate([np.asarray(r[0]) for r in res])
    off = np.concatenate([r[1] for r in res])
    return dt, idx, off


# --------------------------------------------------------------------------
# CPU leg (the reference's own CPU code): ISCE2's C++ port of ampcor.F
# (components/zerodop/GPUampcor/src/Ampcor.cpp), built by oracle/build_ref.py
# with an in-memory line accessor and a radix-2 FFT in place of FFTW, run in
# row bands of window rows on every host thread
# --------------------------------------------------------------------------
REF_CPU_NOTE = ("reference C++ CPU ampcor (GPUampcor Ampcor.cpp/AmpcorMethods.cpp, the port of ampcor.F) "
                "with a project radix-2 FFT in place of its FFTW wrapper, one thread per band of window rows")


def host_info() -> dict:
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for l in out.splitlines():
            if l.startswith("Model name:"):
                model = l.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    return {"nproc": os.cpu_count(), "cpu_model": model}


def cpu_reference_exe():
    """Path of the reference CPU build, building it if needed; None if its
    sources were never staged."""
    from oracle import build_ref
    try:
        return build_ref.build()["cpu"]
    except RuntimeError:
        return None


def cpu_reference_rows(exe, sc, p, k0, nrows, threads, tmpdir):
    """Run the reference CPU ampcor on window rows [k0, k0+nrows) of the
    scene.  Only the image rows those windows touch are written out (the
    timed region, measured inside the program, excludes file reading).
    Returns (seconds, windows, accepted windows)."""
    hs, skip, Wh = p["halfSearchRangeDown"], p["skipSampleDown"], p["windowSizeHeight"]
    r0 = p["referenceStartPixelDownStatic"] + k0 * skip - hs
    r1 = p["referenceStartPixelDownStatic"] + (k0 + nrows - 1) * skip - hs + Wh + 2 * hs
    W = sc.reference.shape[1]
    for tag, img in (("ref", sc.reference), ("sec", sc.secondary)):
        fn = os.path.join(tmpdir, f"{tag}.c64")
        np.ascontiguousarray(img[r0:r1]).tofile(fn)
        with open(fn + ".shape", "w") as f:
            f.write(f"{r1 - r0} {W} 8\n")
    summ = os.path.join(tmpdir, "summary.json")
    args = [f"ref={tmpdir}/ref.c64", f"sec={tmpdir}/sec.c64", f"threads={threads}", f"summary={summ}",
            f"numberWindowDown={nrows}", f"referenceStartPixelDownStatic={hs}"]
    for k in ("windowSizeHeight", "windowSizeWidth", "halfSearchRangeDown", "halfSearchRangeAcross",
              "skipSampleDown", "skipSampleAcross", "referenceStartPixelAcrossStatic", "numberWindowAcross",
              "corrSurfaceOverSamplingFactor", "corrSurfaceZoomInWindow"):
        args.append(f"{k}={p[k]}")
    r = subprocess.run([exe, *args], stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference CPU ampcor failed: {r.stderr[-500:]}")
    with open(summ) as f:
        sm = json.load(f)
    return sm["seconds"], sm["windows"], sm["accepted"]


def cpu_reference_timed(exe, sc, p, steps, rows_per_step, threads, seed=0):
    """Seconds and windows over `steps` samples of `rows_per_step` window rows."""
    import tempfile
    nD = p["numberWindowDown"]
    rng = np.random.default_rng(seed)
    tot_s, tot_w, tot_a = 0.0, 0, 0
    with tempfile.TemporaryDirectory() as td:
        for _ in range(steps):
            k0 = int(rng.integers(0, max(1, nD - rows_per_step + 1)))
            s_, w_, a_ = cpu_reference_rows(exe, sc, p, k0, min(rows_per_step, nD - k0), threads, td)
            tot_s += s_
            tot_w += w_
            tot_a += a_
    return tot_s, tot_w, tot_a


def sample_windows(nwin: int, n: int, seed: int = 7) -> np.ndarray:
    return np.sort(np.random.default_rng(seed).choice(nwin, size=min(n, nwin), replace=False))


def write_scene_files(tmpdir: str):
    sc = SCENE(*SIZE)
    rp, sp = os.path.join(tmpdir, "ref.npy"), os.path.join(tmpdir, "sec.npy")
    np.save(rp, sc.reference)
    np.save(sp, sc.secondary)
    return sc, rp, sp


# --------------------------------------------------------------------------
# clocks during the timed region
# --------------------------------------------------------------------------
class ClockSampler:
    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, f[2:]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def batched_path_label(cfg: dict) -> str:
    if cfg.get("mode") == "chain":
        return "batched chain (four stage kernels per wave of mixed windows), CUDA graph replay"
    return (f"batched fused persistent kernel {cfg.get('threads')}x{cfg.get('ctas_per_sm')}, "
            "CUDA graph replay")


def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def measured_peak_bf16():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"]), "measured"
    except (OSError, KeyError, ValueError):
        return 1900.0, "fallback"


def corr_os_flops_per_window(p) -> float:
    """Algorithmic FLOPs of the oversampled correlation of one window:
    2 (raw Wh)(raw Ww)(2 hz raw + 1)^2 (2 per multiply-add)."""
    raw = p["rawDataOversamplingFactor"]
    hs = min(p["halfSearchRangeDown"], p["halfSearchRangeAcross"])
    zoom = min(p["corrSurfaceZoomInWindow"], 2 * raw * hs)
    hz = zoom // (2 * raw)
    return 2.0 * raw * p["windowSizeHeight"] * raw * p["windowSizeWidth"] * (2 * hz * raw + 1) ** 2


def dram_traffic_per_window(kernel: str):
    """DRAM bytes per window of a kernel from the committed ncu summary."""
    try:
        with open(os.path.join(ROOT, "profiles", "dram_bytes_per_window.json")) as f:
            return json.load(f).get(kernel)
    except (OSError, ValueError):
        return None


# --------------------------------------------------------------------------
def run_reference_arm(args, rank, world):
    """The reference's own CPU implementation of the path, timed on the host
    cores on bounded samples of the burst (window rows), same metric."""
    if rank != 0:
        return
    exe = cpu_reference_exe()
    if exe is None:
        print(json.dumps({"impl": "reference", "unavailable": "the reference CPU ampcor sources were not staged "
                          "into oracle/_ref (oracle/build_ref.py needs the ISCE2 tree once)"}), flush=True)
        return
    sc = SCENE(*SIZE)
    p = geometry()
    cores = os.cpu_count() or 1
    rows = min(max(cores, 16), p["numberWindowDown"])  # one band of window rows per thread
    cpu_reference_timed(exe, sc, p, max(args.warmup, 0), cores, cores, seed=100)  # warm-up: one row per thread
    total_t, total_w, acc = cpu_reference_timed(exe, sc, p, args.steps, rows, cores, seed=200)
    v = total_w / total_t
    sample = f"{rows} random window rows ({rows * p['numberWindowAcross']} windows) of the workload per step"
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "windows/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total_t / max(args.steps, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": {"workload": WORKLOAD, "windows_per_step": rows * p["numberWindowAcross"],
                                            "accepted_windows": acc, "host": host_info()},
            "cpu_baseline": {"value": v, "unit": "windows/s", "cores": cores, "kind": "reference",
                             "sample": f"{sample}; {REF_CPU_NOTE}"},
            "e2e": {"value": v, "unit": "windows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def host_link_gbs(dev) -> dict:
    """The host link alone: 1 GiB pinned host -> device copies on one stream,
    CUDA events, after one untimed copy; the best and median of five."""
    import torch

    try:
        hb = torch.ones(1 << 28, dtype=torch.float32).pin_memory()
        db = torch.empty(1 << 28, dtype=torch.float32, device=dev)
        st = torch.cuda.Stream(dev)
        with torch.cuda.stream(st):
            db.copy_(hb, non_blocking=True)
        st.synchronize()
        ms = []
        for _ in range(5):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(st)
            with torch.cuda.stream(st):
                db.copy_(hb, non_blocking=True)
            b.record(st)
            b.synchronize()
            ms.append(a.elapsed_time(b))
        nbytes = hb.numel() * 4
        del hb, db
        return {"bytes": nbytes, "gb_per_s_best": nbytes / min(ms) / 1e6,
                "gb_per_s_median": nbytes / statistics.median(ms) / 1e6}
    except Exception as e:  # a measurement only: the bench line does not depend on it
        return {"error": str(e)[:200]}


def downstream_cull(p, field, dev, peak_gbs):
    """Offset-field outlier culling (Offoutliers) after the burst, outside the
    timed region: the burst's own field (window centres, SNR >= 2, distance
    3 px) and a 4 M-point synthetic field for a bandwidth figure; CUDA
    events over 20 calls of the C ABI on prepared FP64 arrays, the FP64
    oracle timed beside them on the host."""
    import torch
    from isce2_gb300.offsets import offoutliers_device
    from oracle import offoutliers_oracle as orc

    nD, nA = p["numberWindowDown"], p["numberWindowAcross"]
    ld = p["referenceStartPixelDownStatic"] + np.arange(nD) * p["skipSampleDown"] + p["windowSizeHeight"] // 2
    la = p["referenceStartPixelAcrossStatic"] + np.arange(nA) * p["skipSampleAcross"] + p["windowSizeWidth"] // 2
    LD, LA = np.meshgrid(ld.astype(np.float64), la.astype(np.float64), indexing="ij")
    off = field["offset"].reshape(-1, 2).to(torch.float64)
    burst = (torch.as_tensor(LA.ravel(), device=dev), off[:, 1].contiguous(),
             torch.as_tensor(LD.ravel(), device=dev), off[:, 0].contiguous(), field["snr"].reshape(-1).contiguous())
    rng = np.random.default_rng(7)
    m = 4 << 20
    xa, xd = rng.uniform(0, 8000, m).round(), rng.uniform(0, 12000, m).round()
    za, zd = 1.2 + 3e-4 * xa + rng.normal(0, 0.3, m), -0.5 - 1e-4 * xd + rng.normal(0, 0.3, m)
    big_h = (xa, za, xd, zd, rng.gamma(2.0, 3.0, m).astype(np.float32))
    big = tuple(torch.as_tensor(a, device=dev) for a in big_h)
    out = {}
    for name, arrs in (("burst_field", burst), ("field_4m", big)):
        n = arrs[0].numel()
        st = torch.cuda.current_stream(dev)
        call = lambda: offoutliers_device(*arrs[:4], distance=3.0, snr=arrs[4], snr_threshold=2.0, stream=st)
        for _ in range(3):
            r = call()
        torch.cuda.synchronize(dev)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st)
        for _ in range(20):
            r = call()
        b.record(st)
        torch.cuda.synchronize(dev)
        ms = a.elapsed_time(b) / 20
        kept = int(r["count"].item())
        # two passes over 4 FP64 arrays and the FP32 SNR, a flag byte written
        # and read, the kept indices written
        alg = 2 * n * (4 * 8 + 4) + 2 * n + 4 * kept
        h = [x.cpu().numpy() for x in arrs] if name == "burst_field" else list(big_h)
        t0 = time.perf_counter()
        ref = orc.offoutliers(h[0], h[1], h[2], h[3], 3.0, snr=h[4], snr_threshold=2.0)
        cpu_ms = (time.perf_counter() - t0) * 1e3
        out[name] = {"points": n, "kept": kept, "ms": ms, "points_per_s": n / ms * 1e3,
                     "gb_per_s": alg / ms / 1e6, "hbm_frac": alg / ms / 1e6 / peak_gbs,
                     "launches_per_call": 5, "same_as_oracle": bool(np.array_equal(
                         r["index"][:kept].cpu().numpy(), ref["index"])),
                     "oracle_cpu_ms": cpu_ms}
    # offset polynomial (Offsetpoly, 6 terms) of the across offsets
    from isce2_gb300.offsets import offsetpoly_device
    from oracle import offsetpoly_oracle as opo
    for name, arrs in (("burst_field", burst), ("field_4m", big)):
        x, z, y = arrs[0], arrs[1], arrs[2]
        snr64 = arrs[4].to(torch.float64)
        st = torch.cuda.current_stream(dev)
        call = lambda: offsetpoly_device(x, y, z, snr64, ncoef=6, stream=st)
        for _ in range(3):
            r = call()
        torch.cuda.synchronize(dev)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st)
        for _ in range(20):
            r = call()
        b.record(st)
        torch.cuda.synchronize(dev)
        ms = a.elapsed_time(b) / 20
        h = [t.cpu().numpy() for t in (x, y, z, snr64)]
        t0 = time.perf_counter()
        ref = opo.offsetpoly(h[0], h[1], h[2], h[3], 6)
        cpu_ms = (time.perf_counter() - t0) * 1e3
        got = r["coef"].cpu().numpy()
        out["offsetpoly_" + name] = {
            "points": int(x.numel()), "terms": 6, "rank": int(r["rank"].item()), "ms": ms,
            "points_per_s": x.numel() / ms * 1e3, "launches_per_call": 4,
            "max_fit_diff_vs_oracle_px": float(np.abs(opo.evaluate(got, h[0], h[1]) - opo.evaluate(ref, h[0], h[1])).max()),
            "oracle_cpu_ms": cpu_ms}
    out["note"] = ("Offoutliers on the device (ampcor_offoutliers: fit sums, fit, distances, offsets, ordered "
                   "scatter) and Offsetpoly (ampcor_offsetpoly: centring sums, scaled Gram sums, one-thread "
                   "eigen / SVD solve); the oracles are the NumPy restatements on one host core")
    return out


def run_ours(args, rank, world, local_rank):
    import tempfile
    cores = os.cpu_count() or 1
    pool = None
    if rank == 0 and not args.no_cpu_baseline:
        pool = mp.get_context("spawn").Pool(cores)  # created before any CUDA call
    import torch
    import torch.distributed as dist
    from isce2_gb300 import PyCuAmpcor

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    td = tempfile.TemporaryDirectory()
    sc, rp, sp = write_scene_files(td.name)
    p = geometry()
    nwin = p["numberWindowDown"] * p["numberWindowAcross"]
    obj = PyCuAmpcor()
    for k, v in p.items():
        setattr(obj, k, v)
    obj.deviceID = local_rank
    obj.setupParams()
    obj.setConstantGrossOffset(0, 0)
    obj.checkPixelInImageRange()
    ref_d = torch.from_numpy(sc.reference).to(dev)
    sec_d = torch.from_numpy(sc.secondary).to(dev)
    stream = torch.cuda.current_stream(dev)
    out = obj.run_device(ref_d, sec_d, stream=stream)
    for _ in range(args.warmup):
        obj.run_device(ref_d, sec_d, out=out, stream=stream)
    torch.cuda.synchronize(dev)
    if world > 1:
        dist.barrier()
    obj.set_timing(True)
    # inputs smaller than L2 (129 MB) are timed step by step with a 256 MB
    # buffer written between steps (outside the timed events), so every step
    # reads its images from HBM
    flush = (torch.empty(64 << 20, dtype=torch.float32, device=dev)
             if sc.reference.nbytes + sc.secondary.nbytes < (256 << 20) else None)

    def timed(run, st, steps):
        if flush is None:
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(st)
            for _ in range(steps):
                run()
            b.record(st)
            torch.cuda.synchronize(dev)
            return a.elapsed_time(b)
        ev = []
        for _ in range(steps):
            with torch.cuda.stream(st):
                flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(st)
            run()
            b.record(st)
            ev.append((a, b))
        torch.cuda.synchronize(dev)
        return sum(a.elapsed_time(b) for a, b in ev)

    with ClockSampler(local_rank) as clk:
        torch.cuda.synchronize(dev)
        ms_plain = timed(lambda: obj.run_device(ref_d, sec_d, out=out, stream=stream), stream, args.steps)
    stages = obj.read_timing()
    obj.set_timing(False)
    obj.run_status(stream)  # raises if a bounded device wait of a timed run gave up

    # batched path: the same windows through the persistent kernel, tuned
    # launch shape, replayed from a captured CUDA graph
    from isce2_gb300 import AmpcorBatch
    # the batched path correlates the oversampled chips on the tensor cores
    # (split-BF16 by default); the plain chain above stays FP32
    obj_b = PyCuAmpcor()
    for k, v in p.items():
        setattr(obj_b, k, v)
    obj_b.deviceID = local_rank
    obj_b.corrPrecision = args.batched_corr
    obj_b.setupParams()
    obj_b.setConstantGrossOffset(0, 0)
    bstream = torch.cuda.Stream(dev)
    batch = AmpcorBatch(local_rank)
    bout = batch.add(obj_b, ref_d, sec_d)
    if args.batched_shape:
        # a fixed launch shape (profiling: ncu serialises launches, which
        # distorts the tuner's timings)
        batch.set_shape(args.batched_shape)
        tuned = batch.config()
    else:
        tuned = batch.tune(stream=bstream)
    for _ in range(args.warmup):
        batch.run(stream=bstream, graph=True)
    bstream.synchronize()
    if world > 1:
        dist.barrier()
    with ClockSampler(local_rank) as bclk:
        ms_batch = timed(lambda: batch.run(stream=bstream, graph=True), bstream, args.steps)
    batch.synchronize(stream=bstream)
    use_batch = ms_batch < ms_plain
    ms = ms_batch if use_batch else ms_plain
    t = torch.tensor([ms, ms_plain, ms_batch], dtype=torch.float64, device=dev)
    if world > 1:
        dist.barrier()
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms_max, ms_plain_max, ms_batch_max = (float(x) for x in t.tolist())
    value = world * nwin * args.steps / (ms_max / 1e3)
    plain_value = world * nwin * args.steps / (ms_plain_max / 1e3)
    batch_value = world * nwin * args.steps / (ms_batch_max / 1e3)

    # end to end through the public API with host buffers: every step copies
    # its images from pinned host memory and reads its fields back into pinned
    # host memory.  Ingest overlaps compute through a ring of device image
    # buffers: step k's images go up on the copy streams into slot k % NSLOT
    # as soon as the run that last read that slot is done, so copies run up
    # to NSLOT - 1 steps ahead.  The host link moves ~210 GB/s (7.3 ms for a
    # step's 1.54 GB), but single copies now and then take ten times longer;
    # the ring absorbs those instead of stalling the next run.
    nslot = max(2, args.ingest_slots)
    link = host_link_gbs(dev)
    ref_p = torch.from_numpy(sc.reference).pin_memory()
    sec_p = torch.from_numpy(sc.secondary).pin_memory()
    bufs = [(ref_d, sec_d)] + [(torch.empty_like(ref_d), torch.empty_like(sec_d)) for _ in range(nslot - 1)]
    if use_batch:
        best = args.batched_shape or min((v, k) for k, v in tuned["candidates_ms"].items() if v > 0)[1]
        runners = [(batch, bout)]
        for i in range(1, nslot):
            bt = AmpcorBatch(local_rank)
            bo = bt.add(obj_b, bufs[i][0], bufs[i][1])
            bt.set_shape(best)
            runners.append((bt, bo))
    else:
        runners = [(None, out)] + [(None, {k: torch.empty_like(v) for k, v in out.items()}) for _ in range(nslot - 1)]
    out_h = [{k: torch.empty(v.shape, dtype=v.dtype).pin_memory() for k, v in r[1].items()} for r in runners]
    # each image goes up in two row halves, the four parts on four copy
    # streams at once (several copy engines share the host link)
    cstreams = [torch.cuda.Stream(dev) for _ in range(4)]
    copied = [[torch.cuda.Event() for _ in cstreams] for _ in range(nslot)]
    consumed = [torch.cuda.Event() for _ in range(nslot)]
    half = sc.reference.shape[0] // 2
    parts = [(0, slice(0, half)), (0, slice(half, None)), (1, slice(0, half)), (1, slice(half, None))]
    srcs = (ref_p, sec_p)

    def e2e_steps(n, marks=None):
        for k in range(n):
            b = k % nslot
            for i, (cs, ev, (img, rows)) in enumerate(zip(cstreams, copied[b], parts)):
                if k >= nslot:
                    cs.wait_event(consumed[b])
                if marks is not None:
                    marks[k][0][i].record(cs)
                with torch.cuda.stream(cs):
                    bufs[b][img][rows].copy_(srcs[img][rows], non_blocking=True)
                if marks is not None:
                    marks[k][1][i].record(cs)
                ev.record(cs)
                bstream.wait_event(ev)
            bt, dst = runners[b]
            with torch.cuda.stream(bstream):
                if bt is not None:
                    bt.run(stream=bstream, graph=True)
                else:
                    obj.run_device(bufs[b][0], bufs[b][1], out=dst, stream=bstream)
                for key in out_h[b]:
                    out_h[b][key].copy_(dst[key], non_blocking=True)
            consumed[b].record(bstream)
        bstream.synchronize()

    e2e_steps(nslot)
    torch.cuda.synchronize(dev)
    e2e_n = max(args.steps, 10)  # several steps, so the ring's fill is a small part
    # copy start / end on every copy stream, every step (timing events only;
    # the copies and runs are the same as without them)
    marks = [([torch.cuda.Event(enable_timing=True) for _ in cstreams],
              [torch.cuda.Event(enable_timing=True) for _ in cstreams]) for _ in range(e2e_n)]
    origin = torch.cuda.Event(enable_timing=True)
    origin.record(bstream)
    t0 = time.perf_counter()
    e2e_steps(e2e_n, marks)
    e2e_s = time.perf_counter() - t0
    torch.cuda.synchronize(dev)
    if not use_batch:
        obj.run_status(bstream)  # raises if a bounded device wait of any run gave up
    te = torch.tensor([e2e_s], dtype=torch.float64, device=dev)
    if world > 1:
        dist.all_reduce(te, op=dist.ReduceOp.MAX)
    e2e_v = world * nwin * e2e_n / float(te.item())
    step_bytes = sc.reference.nbytes + sc.secondary.nbytes
    copy_ms = [max(origin.elapsed_time(x) for x in m[1]) - min(origin.elapsed_time(x) for x in m[0]) for m in marks]
    copy_med = statistics.median(copy_ms)
    # a step's copy span: first part's start to last part's end on the four
    # copy streams (parts of consecutive steps queue behind one another, so a
    # span can include waiting for the previous step's parts)
    h2d = {"copy_span_ms_median": copy_med, "copy_span_ms_max": max(copy_ms),
           "gb_per_s_over_median_span": step_bytes / copy_med / 1e6,
           "slow_copy_steps": sum(1 for c in copy_ms if c > 2 * copy_med),
           "gb_per_s_over_whole_run": e2e_n * step_bytes / e2e_s / 1e9, "link": link}

    if rank != 0:
        return
    # roofline for the dominant kernel of the reported path
    from isce2_gb300._lib import STAGES, STAGE_KERNELS
    peak, peak_kind = measured_peak_hbm()
    chain_stages = None
    if use_batch and tuned.get("mode") == "chain":
        # stage times of the chain (one extra run with events around every
        # stage launch, outside the timed region)
        batch.set_timing(True)
        batch.run(stream=bstream)
        batch.synchronize(stream=bstream)
        chain_stages = batch.read_timing()
        batch.set_timing(False)
    if use_batch and chain_stages is not None:
        per_win = stage_bytes_per_window(p)
        dom = max(range(len(STAGES)), key=lambda i: chain_stages[STAGES[i]][0])
        plain_kern = STAGE_KERNELS[dom]
        kern = {"k_raw": "k_wave_raw", "k_oversample2": "k_wave_os",
                "k_corr_os_tma": ("k_corr_os_tc (wave)" if args.batched_corr != "fp32" else "k_corr_os_tma (wave)"),
                "k_zoom": "k_wave_zoom"}[plain_kern]
        dom_ms, dom_launches = chain_stages[STAGES[dom]]
        avg_launch_s = dom_ms / 1e3 / max(dom_launches, 1)
        win_per_launch = nwin / max(dom_launches, 1)
        alg = per_win[plain_kern] * win_per_launch
    elif use_batch:
        # one persistent launch per step; algorithmic bytes: B_win per window
        # (reference + search chip complex64 in, 24 B of fields out)
        kern = plain_kern = "k_persist"
        alg = b_win(p) * nwin
        avg_launch_s = ms_batch / 1e3 / args.steps
        win_per_launch = nwin
    else:
        per_win = stage_bytes_per_window(p)
        dom = max(range(len(STAGES)), key=lambda i: stages[STAGES[i]][0])
        kern = plain_kern = STAGE_KERNELS[dom]
        dom_ms, dom_launches = stages[STAGES[dom]]
        avg_launch_s = dom_ms / 1e3 / max(dom_launches, 1)
        win_per_launch = nwin * args.steps / max(dom_launches, 1)
        alg = per_win[kern] * win_per_launch
    achieved = alg / avg_launch_s / 1e9
    # the wave kernels run the plain kernels' bodies; the batched chain's
    # oversampled correlation is the tensor-core kernel unless run in FP32
    tk = "k_corr_os_tc" if (use_batch and plain_kern == "k_corr_os_tma" and args.batched_corr != "fp32") else plain_kern
    trafw = dram_traffic_per_window(tk)
    roof = {"kernel": kern, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind,
            "traffic": (trafw * win_per_launch) if trafw else None,
            "algorithmic_bytes_per_launch": alg, "launch_ms": avg_launch_s * 1e3}
    # the tensor-core stage of the batched chain against the bf16 tensor peak
    roof_tc = None
    if use_batch and chain_stages is not None and args.batched_corr != "fp32":
        tc_ms, tc_launches = chain_stages["oversampled_correlation"]
        if tc_launches:
            tpk, tpk_kind = measured_peak_bf16()
            launch_s = tc_ms / 1e3 / tc_launches
            flops = corr_os_flops_per_window(p) * nwin / tc_launches
            passes = 3 if args.batched_corr == "split-bf16" else 1
            roof_tc = {"kernel": "k_corr_os_tc", "bound": "tensor", "unit": "TFLOP/s",
                       "achieved": flops / launch_s / 1e12, "peak": tpk, "peak_source": tpk_kind,
                       "frac": flops / launch_s / 1e12 / tpk, "algorithmic_flops_per_launch": flops,
                       "launch_ms": launch_s * 1e3, "mma_passes": passes,
                       "note": "algorithmic FLOPs (one pass); the split-BF16 kernel issues three MMA passes"}
    cpu = None
    acc = None
    oracle_cpu = None
    if pool is not None:
        sel = np.arange(nwin) if FULL_CHECK else sample_windows(nwin, max(cores * 32, 256))
        dt, idx, off_o = cpu_oracle_timed(pool, cores, rp, sp, p, sel)
        pool.close()
        oracle_cpu = {"value": len(sel) / dt, "unit": "windows/s", "cores": cores,
                      "sample": (f"all {len(sel)} windows" if FULL_CHECK else f"{len(sel)} random windows")
                      + f" of the workload, FP64 NumPy oracle on {cores} processes"}
        exe = cpu_reference_exe()
        if exe is not None:
            if FULL_CHECK:  # every window row once
                rs, rw, _ = cpu_reference_timed(exe, sc, p, 1, p["numberWindowDown"], cores, seed=300)
                smp = f"all {rw} windows"
            else:
                rows = max(cores, 16)
                rs, rw, _ = cpu_reference_timed(exe, sc, p, 2, rows, cores, seed=300)
                smp = f"2 x {rows} random window rows ({rw} windows) of the burst"
            cpu = {"value": rw / rs, "unit": "windows/s", "cores": cores, "kind": "reference",
                   "sample": f"{smp}; {REF_CPU_NOTE}", "host": host_info()}
        else:
            cpu = dict(oracle_cpu, kind="port")
        g = (bout if use_batch else out)["offset"].reshape(-1, 2).cpu().numpy()[idx]
        e = g - off_o
        acc = {"windows": int(len(idx)), "rms_px": float(np.sqrt(np.mean(e ** 2))),
               "max_px": float(np.abs(e).max()),
               "exact_frac": float(np.mean(np.all(np.abs(e) < 1e-6, axis=1)))}
    downstream = downstream_cull(p, bout if use_batch else out, dev, peak)
    launches = sum(n for _, n in stages.values())
    line = {"metric": METRIC, "value": value, "unit": "windows/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "windows_per_step": nwin,
                       "path": (batched_path_label(tuned) if use_batch else "plain four-kernel chain"),
                       "plain_windows_per_s": plain_value, "batched_windows_per_s": batch_value,
                       "batched_over_plain": batch_value / plain_value, "batched_launch": tuned,
                       "batched_corr_precision": args.batched_corr,
                       "l2": (f"inputs {(sc.reference.nbytes + sc.secondary.nbytes) / 1e9:.2f} GB exceed L2; no flush"
                              if flush is None else "256 MB L2 flush between timed steps (outside the events)"),
                       "parallelism": f"replicas x{world}"},
            "e2e": {"value": e2e_v, "unit": "windows/s", "h2d_bytes_per_step": int(sc.reference.nbytes + sc.secondary.nbytes),
                    "d2h_bytes_per_step": int(nwin * 24), "ingest": "four copy streams (each image in two row halves) overlapped "
                    f"with compute, a ring of {nslot} device image buffers", "h2d": h2d, "steps": e2e_n},
            "gpu_launches": (launches if not use_batch else
                             args.steps * (sum(n for _, n in chain_stages.values()) if chain_stages else 1)),
            "stages_ms_per_step_batched": ({k: v[0] for k, v in chain_stages.items()} if chain_stages else None),
            "stages_ms_per_step": {s: stages[s][0] / args.steps for s in STAGES},
            "roofline": roof, "roofline_tensor_core": roof_tc, "cpu_baseline": cpu, "oracle_cpu": oracle_cpu,
            "accuracy_vs_oracle": acc, "downstream": downstream,
            "clocks": (bclk if use_batch else clk).summary()}
    print(json.dumps(line), flush=True)
    td.cleanup()


# --------------------------------------------------------------------------
# uneven batch: 256 jobs of mixed geometry, plain chain per job vs one
# persistent launch
# --------------------------------------------------------------------------
UNEVEN = ("uneven batch: 256 jobs, sides U[1024,8192], windows {32..128}^2, half search U[8,48], "
          "skips U[16,128], ovs {16,32,64}, raw 2, zoom 16, 10 dB")


def _oracle_job_sample(args):
    ref_path, sec_path, p, sel = args
    from oracle.ampcor_oracle import OracleParams, run_windows
    ref = np.load(ref_path, mmap_mode="r")
    sec = np.load(sec_path, mmap_mode="r")
    op = OracleParams(**{k: v for k, v in p.items() if k in OracleParams.__dataclass_fields__})
    out = run_windows(ref, sec, op, op.constant_gross_starts(0, 0), sel=np.asarray(sel), batch=8)
    return out["offset"], out["raw_gap"]


def run_uneven(args, rank, world, local_rank):
    import tempfile
    cores = os.cpu_count() or 1
    pool = mp.get_context("spawn").Pool(cores) if not args.no_cpu_baseline else None
    import torch
    from isce2_gb300 import AmpcorBatch, PyCuAmpcor, workloads

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    specs = workloads.uneven_jobs(args.jobs)
    t0 = time.perf_counter()
    imgs = [workloads.make_pair_device(s, dev) for s in specs]
    torch.cuda.synchronize(dev)
    gen_s = time.perf_counter() - t0
    nwin = sum(s.windows for s in specs)
    st = torch.cuda.Stream(dev)

    def handle(spec, corr="fp32"):
        obj = PyCuAmpcor()
        for k, v in spec.params().items():
            setattr(obj, k, v)
        obj.deviceID = local_rank
        obj.corrPrecision = corr
        obj.setupParams()
        obj.setConstantGrossOffset(0, 0)
        obj.checkPixelInImageRange()
        return obj

    # plain chain: one handle per job, run alone after warm-up; the step time
    # is the sum over jobs (the per-job handles are freed between jobs, so
    # their workspaces never coexist)
    plain_ms = 0.0
    plain_off = []
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as pclk:
        for spec, (r, s) in zip(specs, imgs):
            obj = handle(spec)
            out = obj.run_device(r, s, stream=st)
            for _ in range(max(args.warmup - 1, 0)):
                obj.run_device(r, s, out=out, stream=st)
            e0.record(st)
            for _ in range(args.steps):
                obj.run_device(r, s, out=out, stream=st)
            e1.record(st)
            st.synchronize()
            plain_ms += e0.elapsed_time(e1)
            plain_off.append(out["offset"])
            del obj

    batch = AmpcorBatch(local_rank)
    bouts = [batch.add(handle(spec, args.batched_corr), r, s) for spec, (r, s) in zip(specs, imgs)]
    tuned = batch.tune(stream=st)
    for _ in range(args.warmup):
        batch.run(stream=st, graph=True)
    st.synchronize()
    with ClockSampler(local_rank) as bclk:
        e0.record(st)
        for _ in range(args.steps):
            batch.run(stream=st, graph=True)
        e1.record(st)
        st.synchronize()
    batch.synchronize(stream=st)
    batch_ms = e0.elapsed_time(e1)
    launches_per_step, chain_stages = 1, None
    if tuned.get("mode") == "chain":
        batch.set_timing(True)
        batch.run(stream=st)
        batch.synchronize(stream=st)
        chain_stages = batch.read_timing()
        batch.set_timing(False)
        launches_per_step = sum(n for _, n in chain_stages.values())
    same = sum(int(torch.equal(a["offset"], b)) for a, b in zip(bouts, plain_off))
    diff = torch.cat([(a["offset"] - b).abs().reshape(-1) for a, b in zip(bouts, plain_off)])
    plain_v = nwin * args.steps / (plain_ms / 1e3)
    batch_v = nwin * args.steps / (batch_ms / 1e3)

    acc = cpu = None
    if pool is not None:
        # FP64 oracle on a sample of windows of the jobs with the smallest images
        order = sorted(range(len(specs)), key=lambda j: specs[j].H * specs[j].W)[:6]
        td = tempfile.TemporaryDirectory()
        tasks, metas = [], []
        for j in order:
            rp, sp = os.path.join(td.name, f"r{j}.npy"), os.path.join(td.name, f"s{j}.npy")
            np.save(rp, imgs[j][0].cpu().numpy())
            np.save(sp, imgs[j][1].cpu().numpy())
            sel = sample_windows(specs[j].windows, 64, seed=j)
            for c in np.array_split(sel, max(1, cores // len(order))):
                if len(c):
                    tasks.append((rp, sp, specs[j].params(), list(c)))
                    metas.append((j, c))
        tc = time.perf_counter()
        res = pool.map(_oracle_job_sample, tasks)
        dt = time.perf_counter() - tc
        pool.close()
        errs, nsum = [], 0
        for (j, c), (off_o, gap) in zip(metas, res):
            g = bouts[j]["offset"].reshape(-1, 2).cpu().numpy()[c]
            keep = gap >= 2e-5
            errs.append((g - off_o)[keep])
            nsum += len(c)
        e = np.concatenate(errs)
        acc = {"windows": int(nsum), "jobs": len(order), "rms_px": float(np.sqrt(np.mean(e ** 2))),
               "max_px": float(np.abs(e).max())}
        cpu = {"value": nsum / dt, "unit": "windows/s", "cores": cores, "kind": "port",
               "sample": f"{nsum} windows of the {len(order)} smallest jobs, FP64 NumPy oracle"}
        td.cleanup()
    classes = {}
    for s in specs:
        k = f"{s.Wh}x{s.Ww}"
        classes[k] = classes.get(k, 0) + s.windows
    line = {"metric": METRIC, "value": batch_v, "unit": "windows/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": batch_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (device generator)",
            "config": {"workload": UNEVEN if args.jobs == 256 else UNEVEN.replace("256 jobs", f"{args.jobs} jobs"),
                       "windows_per_step": nwin, "jobs": len(specs),
                       "path": batched_path_label(tuned),
                       "plain_windows_per_s": plain_v, "batched_windows_per_s": batch_v,
                       "batched_over_plain": batch_v / plain_v, "batched_launch": tuned,
                       "plain_ms_per_step": plain_ms / args.steps,
                       "batched_vs_plain_identical_jobs": same, "batched_vs_plain_max_abs_px": float(diff.max()),
                       "image_gb": sum(2 * s.H * s.W * 8 for s in specs) / 1e9, "generate_s": gen_s,
                       "windows_by_class": classes, "l2": "inputs exceed L2; no flush"},
            "gpu_launches": args.steps * launches_per_step,
            "stages_ms_per_step_batched": ({k: v[0] for k, v in chain_stages.items()} if chain_stages else None),
            "cpu_baseline": cpu, "accuracy_vs_oracle": acc,
            "clocks": bclk.summary(), "clocks_plain": pclk.summary()}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------
# served request stream: Poisson arrivals, continuous batching, p50/p99
# --------------------------------------------------------------------------
SERVING = ("served requests: Poisson arrivals at {rates} req/s, sides log-U[1024,16384], square windows "
           "U[32,256] (even), half search U[8,48], skip = window, ovs 32, zoom 16, HBM budget 150 GB")
SCENE_SIDE = 16384


def run_serving(args, rank, world, local_rank):
    import torch
    from isce2_gb300 import AmpcorServer, PyCuAmpcor, workloads

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    rates = [float(x) for x in args.rates.split(",")]
    # Every request k has its own pair, seeded 5 000 000 + k (the same request
    # k at every rate; only the arrival times differ).  The pairs are made on
    # the GPU once and kept in pinned host memory: requests arrive with their
    # images in host memory and the server copies them in at admission.  The
    # number of requests is capped by a host-memory budget.
    t0 = time.perf_counter()
    n_need = max(int(min(args.max_requests, max(20, r * args.duration))) for r in rates)
    _, all_specs = workloads.serving_requests(max(rates), n_need, max_side=SCENE_SIDE)
    try:
        host_bytes = os.sysconf("SC_PAGE_SIZE") * os.sysconf("SC_PHYS_PAGES")
    except (ValueError, OSError):
        host_bytes = 256 << 30
    on_device = args.serve_from == "device"
    # requests arrive with their images in pinned host memory (the server
    # copies them in at admission, over the host link) or already in device
    # memory (a device-to-device copy at admission), as the plain chain's
    # images are
    budget = min(args.host_gb * 1e9, 0.4 * host_bytes) if not on_device else args.device_request_gb * 1e9
    pairs, used = [], 0
    for sp in all_specs:
        b = 16 * sp.H * sp.W
        if used + b > budget:
            break
        r_d, s_d = workloads.make_pair_device(sp, dev)
        if on_device:
            pairs.append((r_d, s_d))
        else:
            pairs.append((r_d.cpu().pin_memory(), s_d.cpu().pin_memory()))
        del r_d, s_d
        used += b
    torch.cuda.synchronize(dev)
    torch.cuda.empty_cache()
    gen_s = time.perf_counter() - t0
    n_avail = len(pairs)

    from isce2_gb300._lib import AMPCOR_ERR_UNSUPPORTED, AmpcorError

    def handle(spec, corr="fp32"):
        obj = PyCuAmpcor()
        for k, v in spec.params().items():
            setattr(obj, k, v)
        obj.deviceID = local_rank
        obj.corrPrecision = corr
        try:
            obj.setupParams()
        except AmpcorError as e:
            # windows wider than the tensor-core correlation's shared-memory
            # bands (about 150 columns at raw 2) correlate in FP32
            if corr == "fp32" or e.code != AMPCOR_ERR_UNSUPPORTED:
                raise
            obj.corrPrecision = "fp32"
            obj.setupParams()
        obj.setConstantGrossOffset(0, 0)
        return obj

    results = {}
    for rate in rates:
        n = min(n_avail, int(min(args.max_requests, max(20, rate * args.duration))))
        arrivals, specs = workloads.serving_requests(rate, n, max_side=SCENE_SIDE)
        objs = [handle(sp, args.batched_corr) for sp in specs]
        imgs = [(a, b) if on_device else (a.numpy(), b.numpy()) for a, b in pairs[:n]]
        nwin = sum(sp.windows for sp in specs)
        srv = AmpcorServer(local_rank, hbm_budget_bytes=150 * 10 ** 9, step_windows=args.step_windows)
        # warm-up: one request end to end (kernel attributes, pool growth)
        wid = srv.submit(objs[0], *imgs[0])
        while wid not in srv.poll():
            srv.progress()
        srv.take(wid)
        lat, done_t = [], []
        i = 0
        with ClockSampler(local_rank) as clk:
            start = time.perf_counter()
            pending = {}
            while i < n or pending:
                now = time.perf_counter() - start
                while i < n and arrivals[i] <= now:
                    pending[srv.submit(objs[i], *imgs[i])] = arrivals[i]
                    i += 1
                srv.progress()
                for rid in srv.poll():
                    srv.take(rid)
                    t = time.perf_counter() - start
                    lat.append(t - pending.pop(rid))
                    done_t.append(t)
            span = max(done_t) - arrivals[0]
        st = srv.stats()
        del srv, objs  # return the server's memory pool and the handles
        # the same requests through the plain chain, one after another (a
        # fresh handle per request, freed after it, as in the uneven batch)
        plain_s = 0.0
        st_plain = torch.cuda.Stream(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for sp, (r, s_) in zip(specs, pairs[:n]):
            obj = handle(sp)
            rr, ss = (r, s_) if on_device else (r.to(dev), s_.to(dev))
            out = obj.run_device(rr, ss, stream=st_plain)
            e0.record(st_plain)
            obj.run_device(rr, ss, out=out, stream=st_plain)
            e1.record(st_plain)
            st_plain.synchronize()
            plain_s += e0.elapsed_time(e1) / 1e3
            del obj, rr, ss, out
        lat_ms = np.asarray(lat) * 1e3
        results[f"{rate:g}"] = {
            "requests": n, "windows": nwin, "arrival_span_s": float(arrivals[-1] - arrivals[0]),
            "offered_windows_per_s": nwin / float(arrivals[-1] - arrivals[0]),
            "served_windows_per_s": nwin / span, "plain_windows_per_s": nwin / plain_s,
            "p50_ms": float(np.percentile(lat_ms, 50)), "p99_ms": float(np.percentile(lat_ms, 99)),
            "max_ms": float(lat_ms.max()), "peak_active": st["peak_active"], "steps": st["steps_launched"],
            "peak_hbm_gb": st["peak_bytes"] / 1e9, "clocks": clk.summary()}
        del imgs
    top = results[f"{max(rates):g}"]
    line = {"metric": METRIC, "value": top["served_windows_per_s"], "unit": "windows/s", "n_gpus": 1,
            "steps": len(rates), "warmup": 1, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (device generator)",
            "config": {"workload": SERVING.format(rates="/".join(f"{r:g}" for r in rates)),
                       "path": "request server: continuous batching, persistent kernel steps",
                       "step_windows": args.step_windows,
                       "requests": f"{n_avail} pairs seeded 5000000+k in "
                                   f"{'device' if on_device else 'pinned host'} memory "
                                   f"({used / 1e9:.1f} GB), the first n of them at each rate",
                       "request_images": args.serve_from, "batched_corr_precision": args.batched_corr,
                       "generate_s": gen_s, "rates": results,
                       "latency": f"submit at the scheduled arrival (images in {args.serve_from} memory) to "
                                  "fields on the host"},
            "gpu_launches": top["steps"], "clocks": top["clocks"]}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------
# precision stress: 60 dB dynamic range, per-window error against the oracle
# --------------------------------------------------------------------------
PRECISION = ("precision stress 4096x4096 c64: Rayleigh speckle + 200 point targets (1e3 x mean) + dark water "
             "(1e-3 x, 10 % of the area), window 64x64, half search 16, skip 16, raw 2, ovs 64, zoom 16")


def _oracle_diag_chunk(args):
    ref_path, sec_path, p, sel = args
    from oracle.ampcor_oracle import OracleParams, run_windows
    ref = np.load(ref_path, mmap_mode="r")
    sec = np.load(sec_path, mmap_mode="r")
    op = OracleParams(**{k: v for k, v in p.items() if k in OracleParams.__dataclass_fields__})
    out = run_windows(ref, sec, op, op.constant_gross_starts(0, 0), sel=np.asarray(sel), batch=8)
    return sel, out["offset"], out["offset_init"], out["raw_gap"]


def run_precision(args, rank, world, local_rank):
    import tempfile
    cores = os.cpu_count() or 1
    pool = mp.get_context("spawn").Pool(cores)
    import torch
    from isce2_gb300 import AmpcorBatch, PyCuAmpcor, synth

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    n = 4096
    sc = synth.scene_precision(n)
    p = dict(referenceImageHeight=n, referenceImageWidth=n, secondaryImageHeight=n, secondaryImageWidth=n,
             windowSizeHeight=64, windowSizeWidth=64, halfSearchRangeDown=16, halfSearchRangeAcross=16,
             skipSampleDown=16, skipSampleAcross=16, rawDataOversamplingFactor=2,
             corrSurfaceOverSamplingFactor=64, corrSurfaceZoomInWindow=16, derampMethod=1,
             referenceStartPixelDownStatic=16, referenceStartPixelAcrossStatic=16,
             numberWindowDown=(n - 32 - 64) // 16, numberWindowAcross=(n - 32 - 64) // 16)
    nwin = p["numberWindowDown"] * p["numberWindowAcross"]
    obj = PyCuAmpcor()
    for k, v in p.items():
        setattr(obj, k, v)
    obj.setupParams()
    obj.setConstantGrossOffset(0, 0)
    r_d = torch.from_numpy(sc.reference).to(dev)
    s_d = torch.from_numpy(sc.secondary).to(dev)
    st = torch.cuda.Stream(dev)
    out = obj.run_device(r_d, s_d, diag=True, stream=st)
    for _ in range(args.warmup):
        obj.run_device(r_d, s_d, out=out, stream=st)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clk:
        e0.record(st)
        for _ in range(args.steps):
            obj.run_device(r_d, s_d, out=out, stream=st)
        e1.record(st)
        st.synchronize()
    plain_ms = e0.elapsed_time(e1) / args.steps
    stages_fp32 = None
    obj.set_timing(True)
    obj.run_device(r_d, s_d, out=out, stream=st)
    stages_fp32 = {k: v[0] for k, v in obj.read_timing().items()}
    obj.set_timing(False)
    # the oversampler and the oversampled correlation as tensor-core
    # contractions (split-BF16, BF16), each alone and both together
    tcores = {}
    for mode, (osp, corrp) in {"oversampler_split-bf16": ("split-bf16", "fp32"),
                               "oversampler_bf16": ("bf16", "fp32"),
                               "correlation_split-bf16": ("fp32", "split-bf16"),
                               "correlation_bf16": ("fp32", "bf16"),
                               "both_split-bf16": ("split-bf16", "split-bf16")}.items():
        o2 = PyCuAmpcor()
        for k, v in p.items():
            setattr(o2, k, v)
        o2.precision = osp
        o2.corrPrecision = corrp
        o2.setupParams()
        o2.setConstantGrossOffset(0, 0)
        out2 = o2.run_device(r_d, s_d, diag=True, stream=st)
        for _ in range(args.warmup):
            o2.run_device(r_d, s_d, out=out2, stream=st)
        e0.record(st)
        for _ in range(args.steps):
            o2.run_device(r_d, s_d, out=out2, stream=st)
        e1.record(st)
        st.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        o2.set_timing(True)
        o2.run_device(r_d, s_d, out=out2, stream=st)
        tcores[mode] = {"ms": ms, "out": out2, "stages": {k: v[0] for k, v in o2.read_timing().items()}}
        o2.set_timing(False)
    ob = PyCuAmpcor()
    for k, v in p.items():
        setattr(ob, k, v)
    ob.corrPrecision = args.batched_corr
    ob.setupParams()
    ob.setConstantGrossOffset(0, 0)
    batch = AmpcorBatch(local_rank)
    bout = batch.add(ob, r_d, s_d)
    tuned = batch.tune(stream=st)
    batch.run(stream=st, graph=True)
    batch.synchronize(stream=st)
    e0.record(st)
    for _ in range(args.steps):
        batch.run(stream=st, graph=True)
    e1.record(st)
    batch.synchronize(stream=st)
    batch_ms = e0.elapsed_time(e1) / args.steps

    # window classes: a point target inside the reference chip, any water
    # pixel inside it, else speckle
    rng = np.random.default_rng(42)
    tr, tc = rng.integers(0, n, 200), rng.integers(0, n, 200)
    rng = np.random.default_rng(43)
    side = int(np.sqrt(0.1) * n)
    r0, c0 = rng.integers(0, n - side, 2)
    refD = 16 + 16 * (np.arange(nwin) // p["numberWindowAcross"])
    refA = 16 + 16 * (np.arange(nwin) % p["numberWindowAcross"])
    has_t = np.zeros(nwin, bool)
    for a, b in zip(tr, tc):
        has_t |= (a >= refD) & (a < refD + 64) & (b >= refA) & (b < refA + 64)
    has_w = (refD < r0 + side) & (refD + 64 > r0) & (refA < c0 + side) & (refA + 64 > c0)
    cls = np.where(has_t, "target", np.where(has_w, "water", "speckle"))
    S = args.precision_sample
    pick = lambda c, k, seed: np.random.default_rng(seed).choice(  # noqa: E731
        np.flatnonzero(cls == c), min(k, int(np.count_nonzero(cls == c))), replace=False)
    sel = np.sort(np.concatenate([pick("target", S // 2, 4), pick("water", S // 4, 5), pick("speckle", S // 4, 6)]))
    td = tempfile.TemporaryDirectory()
    rp, sp = os.path.join(td.name, "r.npy"), os.path.join(td.name, "s.npy")
    np.save(rp, sc.reference)
    np.save(sp, sc.secondary)
    chunks = [list(c) for c in np.array_split(sel, cores * 2) if len(c)]
    t0 = time.perf_counter()
    res = pool.map(_oracle_diag_chunk, [(rp, sp, p, c) for c in chunks])
    cpu_s = time.perf_counter() - t0
    pool.close()
    idx = np.concatenate([np.asarray(r[0]) for r in res])
    off_o = np.concatenate([r[1] for r in res])
    init_o = np.concatenate([r[2] for r in res])
    gap_o = np.concatenate([r[3] for r in res])

    near = gap_o < 2e-5  # two best raw NCC values within float32 rounding: either peak is valid

    def report(off):
        e = np.abs(off.reshape(-1, 2)[idx] - off_o)
        per = {}
        for c in ("target", "water", "speckle"):
            m = (cls[idx] == c) & ~near
            ec = e[m].max(axis=1)
            per[c] = {"windows": int(m.sum()), "near_ties_excluded": int(np.count_nonzero((cls[idx] == c) & near)),
                      "rms_px": float(np.sqrt(np.mean(e[m] ** 2))), "p99_px": float(np.percentile(ec, 99)),
                      "max_px": float(ec.max()), "frac_over_0.01px": float(np.mean(ec > 0.01))}
        return per

    d = out["diag"].reshape(-1, 8).cpu().numpy()[idx]
    peak_mismatch = int(np.count_nonzero(~np.all(d[:, 0:2] == init_o, axis=1) & ~near))
    line = {"metric": METRIC, "value": nwin / (min(plain_ms, batch_ms) / 1e3), "unit": "windows/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": min(plain_ms, batch_ms),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": {
                "workload": PRECISION, "windows_per_step": nwin,
                "plain_windows_per_s": nwin / (plain_ms / 1e3), "batched_windows_per_s": nwin / (batch_ms / 1e3),
                "batched_launch": tuned, "oracle_windows": int(len(idx)),
                "batched_corr_precision": args.batched_corr,
                "error_vs_fp64_oracle": {"plain_fp32": report(out["offset"].cpu().numpy()),
                                         f"batched_corr_{args.batched_corr}": report(bout["offset"].cpu().numpy()),
                                         **{f"plain_tensor_core_{m}": report(v["out"]["offset"].cpu().numpy())
                                            for m, v in tcores.items()}},
                "tensor_core_modes": {m: {"windows_per_s": nwin / (v["ms"] / 1e3),
                                          "oversample_ms": v["stages"]["oversample"],
                                          "oversampled_correlation_ms": v["stages"]["oversampled_correlation"]}
                                      for m, v in tcores.items()},
                "fp32_stage_ms": stages_fp32,
                "integer_peak_mismatches": peak_mismatch, "near_ties": int(near.sum())},
            "cpu_baseline": {"value": len(idx) / cpu_s, "unit": "windows/s", "cores": cores, "kind": "port",
                             "sample": f"{len(idx)} windows (point-target, water and speckle windows), FP64 oracle"},
            "gpu_launches": None, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    td.cleanup()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--size", default="12000x8000", help="scene size DOWNxACROSS (profiling uses a smaller scene)")
    ap.add_argument("--workload", default="burst", choices=["burst", "plain", "uneven", "serving", "precision"])
    ap.add_argument("--batched-shape", default=None, help="skip the tuner and use this batched launch shape")
    ap.add_argument("--ingest-slots", type=int, default=4,
                    help="device image buffers of the end-to-end ingest ring (copies run this many steps ahead, less one)")
    ap.add_argument("--batched-corr", default="split-bf16", choices=["fp32", "split-bf16", "bf16"],
                    help="oversampled-correlation arithmetic of the batched and served paths")
    ap.add_argument("--precision-sample", type=int, default=1600,
                    help="oracle windows: half with point targets, a quarter water, a quarter speckle")
    ap.add_argument("--rates", default="50,200,500", help="served request rates (req/s)")
    ap.add_argument("--duration", type=float, default=6.0, help="seconds of arrivals per rate")
    ap.add_argument("--max-requests", type=int, default=1200)
    ap.add_argument("--step-windows", type=int, default=8192)
    ap.add_argument("--host-gb", type=float, default=120.0, help="pinned host memory for served request images")
    ap.add_argument("--serve-from", default="device", choices=["device", "host"],
                    help="where served requests' images live when submitted")
    ap.add_argument("--device-request-gb", type=float, default=100.0,
                    help="device memory for served request images (--serve-from device)")
    ap.add_argument("--jobs", type=int, default=256, help="jobs of the uneven batch")
    args = ap.parse_args()
    global SIZE, WORKLOAD, PARAMS, FULL_CHECK, SCENE
    SIZE = tuple(int(x) for x in args.size.lower().split("x"))
    if args.workload == "plain":
        from isce2_gb300 import synth
        SIZE, PARAMS, FULL_CHECK = (2048, 2048), dict(PLAIN_SMALL), True
        WORKLOAD = "plain 2048x2048 c64, window 64x64, half search 20, skip 32, raw 2, ovs 16, zoom 8, deramp 0"
        SCENE = lambda H, W: synth.scene_plain_small(H)  # noqa: E731
    elif SIZE != (12000, 8000):
        WORKLOAD = WORKLOAD.replace("burst 12000x8000", f"burst geometry on {SIZE[0]}x{SIZE[1]}")
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference_arm(args, rank, world)
        return
    if args.workload == "uneven":
        if rank == 0:
            run_uneven(args, rank, world, local_rank)
        return
    if args.workload == "serving":
        if rank == 0:
            run_serving(args, rank, world, local_rank)
        return
    if args.workload == "precision":
        if rank == 0:
            run_precision(args, rank, world, local_rank)
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    run_ours(args, rank, world, local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
