#!/usr/bin/env python3
"""Benchmark of the full-scale convolution back-projection workload.

Workload (one step): a 2048-pixel detector x 1800 views over 180 degrees, 64 detector rows
(slices), raw uint16 frames I = Poisson(20000 exp(-p)) + dark (dark ~ N(100, 3), flat
20000 (1 + 0.02 smooth noise)), 40 random ellipsoids, rotation-centre offset U[-10, 10] px,
Shepp-Logan filter -> 64 slices of 2048 x 2048.  The step runs the whole hot path on the device:
flat/dark log normalisation, padding, FFT filtering, 1/16 sub-sample tables and the
back-projection, in the reference's fixed-point semantics (bit-exact with the reference CPU
routine; the tests prove it).  Synthetic data stand in for beamline data (none is public).

Metric: Tau = time / (pixels per slice x views x slices) in ns per pixel-view (lower is better),
with slices/s alongside.  `value` is device time with inputs resident in HBM; `e2e` is the same
metric through RvStackRunHost with pinned host buffers (host->device frames and device->host
slices inside the timed region).  The CPU baseline is the oracle restatement of the reference
CPU routine (bit-identical to it) with the reference's multi-worker scheme on all host cores.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--slices S]

nvidia-smi clock samples taken during the timed region are summarised in the line (`clocks`);
the raw samples go to RV_BENCH_LOG_DIR (default: the system's temporary directory).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

W_DET, N_VIEWS, N_SLICES = 2048, 1800, 64
PUBLISHED_TAU_NS = 0.029  # RTX A4000, 2048^2 x 1800 views (reference README, Build-220422)
WORKLOAD = "fbp-2048det-1800views-64slices-raw-uint16"
# DRAM bytes (read + write) per pixel-view update of the REF back-projection, from one ncu capture
# of the default variant (three slices per CTA) on 3 slices of this geometry: 2.42 GB + 398 MB
# over 2.265e10 updates; the traffic grows in proportion to the slices processed, so a full
# launch moves this times its updates.
BP_DRAM_BYTES_PER_UPDATE = 1.244e-1


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--slices", type=int, default=N_SLICES, help="slices per step (default: the workload's 64)")
    ap.add_argument("--mode", default="ref", choices=["ref", "lin", "f16", "bf16"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-centre", action="store_true", help="skip the centre-search summary of the default run")
    ap.add_argument("--no-forms", action="store_true", help="skip the reduced-storage and queue summaries")
    ap.add_argument("--no-parity", action="store_true", help="skip the oracle check of the timed output")
    ap.add_argument("--seed", type=int, default=2026)
    ap.add_argument("--workload", default="fbp", choices=["fbp", "centre", "precision", "queue"],
                    help="fbp: the back-projection stack (default); centre: train the centre-proposal network "
                         "and compare the learned search with the full sweep")
    ap.add_argument("--datasets", type=int, default=200, help="centre: evaluation datasets")
    ap.add_argument("--train", type=int, default=20000, help="centre: training scans")
    ap.add_argument("--epochs", type=int, default=10, help="centre: training epochs")
    ap.add_argument("--finetune", type=int, default=64, help="centre: scans labelled by the full sweep")
    ap.add_argument("--net", default=None, help="centre: load network parameters instead of training")
    ap.add_argument("--save-net", default=None, help="centre: write the trained parameters (float32)")
    return ap.parse_args()


# ------------------------------------------------------------------------------ data -------
def centre_of(seed: int) -> float:
    rng = np.random.default_rng(seed)
    return (W_DET - 1) / 2.0 + rng.uniform(-10.0, 10.0)


def make_stack_gpu(seed: int, nslices: int, device, W: int = W_DET, V: int = N_VIEWS, n_spheres: int = 0):
    """Raw frames on the device: [nframes + 1, nslices, W] uint16 stored in an int16 tensor
    (frame 0 flat, 1..V samples, V+1 flat, last = dark).  40 ellipsoids, plus n_spheres small
    high-contrast spheres (radius 1-4 px, attenuation U[0.5, 2]) across the slice heights."""
    import torch
    from recview_gb300 import phantom
    rng = np.random.default_rng(seed)
    ells3 = phantom.random_ellipsoids(rng, 40)
    center = (W - 1) / 2.0 + np.random.default_rng(seed).uniform(-10.0, 10.0)
    fdeg_s = phantom.angle_table(V)
    theta = torch.tensor(np.deg2rad(fdeg_s.astype(np.float64)), device=device)[:, None]
    t = torch.tensor(phantom.detector_coords(W, center), device=device)[None, :]
    ys = phantom.slice_heights(nslices)
    spheres = phantom.random_spheres(rng, n_spheres, W, ys) if n_spheres else np.zeros((0, 5))
    gen = torch.Generator(device=device).manual_seed(seed)
    dark = 100.0 + 3.0 * torch.randn(nslices, W, device=device, generator=gen, dtype=torch.float64)
    flat = torch.tensor(20000.0 * (1.0 + 0.02 * phantom.smooth_noise(rng, (nslices, W), 16.0)), device=device)
    nframes = V + 2
    raw = torch.empty((nframes + 1, nslices, W), dtype=torch.int16, device=device)

    def to_u16(x):
        x = torch.clamp(torch.round(x), 0, 65535).to(torch.int32)
        return torch.where(x > 32767, x - 65536, x).to(torch.int16)

    for s, y in enumerate(ys):
        p = torch.zeros((V, W), dtype=torch.float64, device=device)
        discs = np.concatenate([phantom.ellipsoid_slice(ells3, y), phantom.sphere_slice(spheres, y)], axis=0)
        for x0, z0, a, b, phi, mu in discs:
            sft = x0 * torch.cos(theta) + z0 * torch.sin(theta)
            d = theta - phi
            a2 = (a * torch.cos(d)) ** 2 + (b * torch.sin(d)) ** 2
            u = t - sft
            rad = a2 - u * u
            p += torch.where(rad > 0, 2.0 * mu * a * b * torch.sqrt(torch.clamp(rad, min=0.0)) / a2, 0.0)
        mean = (flat[s][None, :] * torch.exp(-p)).float()
        raw[1:V + 1, s] = to_u16(torch.poisson(mean, generator=gen) + dark[s][None, :])
        fl = flat[s][None, :].expand(2, W).float().contiguous()
        f = torch.poisson(fl, generator=gen) + dark[s][None, :]
        raw[0, s] = to_u16(f[0])
        raw[V + 1, s] = to_u16(f[1])
        raw[nframes, s] = to_u16(dark[s])
    bInc = np.zeros(nframes, np.int8)
    bInc[1:V + 1] = 1
    fdeg = np.zeros(nframes, np.float32)
    fdeg[1:V + 1] = fdeg_s
    fexp = np.arange(nframes, dtype=np.float32)
    return raw, bInc, fdeg, fexp, center


# ------------------------------------------------------------------------------ clocks -----
class ClockSampler:
    """nvidia-smi samples during the timed region (read-only queries)."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        # RV_BENCH_LOG_DIR keeps the raw samples where the caller wants them; by default they are
        # scratch in the system's temporary directory (the JSON line carries their summary)
        log_dir = os.environ.get("RV_BENCH_LOG_DIR") or tempfile.gettempdir()
        self.path = Path(log_dir) / f"clocks_bench_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.path.parent.mkdir(parents=True, exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.proc or not self.path.exists():
            return None
        rows = [r.split(",") for r in self.path.read_text().strip().splitlines() if r.count(",") >= 8]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows]
        smax = max(float(r[2]) for r in rows)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].strip().lower() == "active"})
        loaded = [v for v in sm if v > 0.5 * smax] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": smax, "reasons": reasons,
                "samples": len(rows), "power_w_max": max(float(r[3]) for r in rows if r[3].strip())}


# ------------------------------------------------------------------------------ CPU side ---
def cpu_one_slice(raw_slice: np.ndarray, bInc, fdeg, fexp, center, F, threads: int, use_ref: bool):
    """One slice of the workload on the CPU: GenerateSinogramThread then the reference's CPU
    FBP with `threads` row-band workers.  Returns seconds."""
    from recview_gb300.reconst import ReconInfo
    from tests.rvtest import Oracle, ref_lib
    oracle = Oracle()
    r = raw_slice.copy()
    ri = ReconInfo(r.view(np.int16), fdeg, bInc, center=0, fexp=fexp, iMultiplex=1, maxSinogrLen=r.shape[0])
    rs = ReconInfo(r.view(np.int16), fdeg, bInc, center=center, fFilter=F, maxSinogrLen=r.shape[0],
                   nviews=r.shape[0] - 1)
    t0 = time.perf_counter()
    oracle.generate_sinogram(ri)
    if use_ref:
        import threading
        L = ref_lib()
        infos = []
        for k in range(threads):
            x = abi_copy(rs.ri)
            x.iStartSino, x.iStepSino = k, threads
            infos.append(x)
        th = [threading.Thread(target=L.rvref_fbp, args=(C.byref(x),)) for x in infos]
        for t in th:
            t.start()
        for t in th:
            t.join()
    else:
        oracle.L.rvo_reconstruct_mt(C.byref(rs.ri), threads)
    return time.perf_counter() - t0


def oracle_slice(raw_slice: np.ndarray, bInc, fdeg, fexp, center, F, threads: int, interp: int = 2,
                 ref: bool = True, lin64: bool = False):
    """The oracle on one detector row of raw frames ([nframes + 1, W] uint16 bits):
    GenerateSinogramThread, then the reference's CPU FBP (int32, the bit-exact target) and/or
    the FP64 end-to-end reconstruction (linear interpolation, double accumulation)."""
    from recview_gb300.reconst import ReconInfo
    from tests.rvtest import Oracle
    oracle = Oracle()
    r = np.ascontiguousarray(raw_slice).view(np.int16).copy()
    ri = ReconInfo(r, fdeg, bInc, center=0, fexp=fexp, iMultiplex=1, maxSinogrLen=r.shape[0])
    oracle.generate_sinogram(ri)
    rs = ReconInfo(r, fdeg, bInc, center=center, fFilter=F, iInterpolation=interp, maxSinogrLen=r.shape[0],
                   nviews=r.shape[0] - 1)
    want = oracle.reconstruct(rs, threads=threads).copy() if ref else None
    ref64 = oracle.lin64(rs, threads=threads) if lin64 else None
    return want, ref64


def circle_mask(n: int) -> np.ndarray:
    yy, xx = np.mgrid[:n, :n]
    return (xx - n / 2) ** 2 + (yy - n / 2) ** 2 < (0.45 * n) ** 2


def error_vs_fp64(got: np.ndarray, ref64: np.ndarray) -> dict:
    """Relative L2 and max-abs error inside the reconstruction circle (r < 0.45 of the width)."""
    m = circle_mask(ref64.shape[0])
    a = np.asarray(got, np.float64)[m]
    b = ref64[m]
    d = a - b
    return {"rel_l2_vs_fp64": float(np.linalg.norm(d) / max(np.linalg.norm(b), 1e-300)),
            "max_abs_vs_fp64": float(np.abs(d).max()), "max_abs_fp64": float(np.abs(b).max())}


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the machine type)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.machine()


SCALAR_NOTE = ("the reference's scalar C back-projection loop (source/general.cpp:2147-2158); its MASM SIMD "
               "loops (source/projx64.asm) are x64-only and cannot run on this Arm host")


def cpu_other_configs(seed: int, threads: int, dev) -> dict:
    """The CPU routine on the other configurations' shapes, one slice each, same host threads:
    the 512-pixel x 900-view single slice (int16 sinogram, FBP only) and one 4096 x 3600 slice of
    the precision study (raw frames: normalisation + FBP)."""
    from recview_gb300 import abi, phantom
    from recview_gb300.reconst import ReconInfo, dims
    from tests.rvtest import Oracle
    oracle = Oracle()
    res = {}
    sino, fdeg1 = phantom.sinogram_2d(seed, 512, 900, 255.5)
    F1 = oracle.set_filter(abi.FILT_SHEPP, dims(512).ndim)
    ri = ReconInfo(sino, fdeg1, np.ones(900, np.int8), center=255.5, fFilter=F1)
    oracle.reconstruct(ri, threads=threads)
    t0 = time.perf_counter()
    oracle.reconstruct(ri, threads=threads)
    t = time.perf_counter() - t0
    res["fbp-512det-900views-1slice"] = {"seconds": t, "tau_ns": t * 1e9 / (512.0 * 512 * 900)}
    raw4, bInc4, fdeg4, fexp4, cen4 = make_stack_gpu(seed, 1, dev, W=4096, V=3600)
    raw4h = raw4[:, 0, :].cpu().numpy()
    del raw4
    F4 = oracle.set_filter(abi.FILT_SHEPP, dims(4096).ndim)
    t = cpu_one_slice(raw4h, bInc4, fdeg4, fexp4, cen4, F4, threads, False)
    res["precision-4096det-3600views-1slice"] = {"seconds": t, "tau_ns": t * 1e9 / (4096.0 * 4096 * 3600),
                                                 "includes": "normalisation + FBP"}
    return res


def abi_copy(ri):
    from recview_gb300 import abi
    x = abi.RECONST_INFO()
    C.memmove(C.byref(x), C.byref(ri), C.sizeof(abi.RECONST_INFO))
    return x


def host_slice_data(seed: int):
    """Raw frames of one slice for the CPU side (same distributions as the device data)."""
    from recview_gb300 import phantom
    center = centre_of(seed)
    raw, bInc, fdeg, fexp, _ = phantom.raw_stack(seed, W_DET, N_VIEWS, 1, center, n_ellipsoids=40)
    return raw, bInc, fdeg, fexp, center


def run_reference(args, rank: int, world: int):
    if rank != 0:
        return
    from recview_gb300 import abi
    from recview_gb300.reconst import dims
    from tests.rvtest import Oracle, ref_lib
    threads = os.cpu_count() or 1
    use_ref = ref_lib() is not None
    raw, bInc, fdeg, fexp, center = host_slice_data(args.seed)
    F = Oracle().set_filter(abi.FILT_SHEPP, dims(W_DET).ndim)
    for _ in range(args.warmup):
        cpu_one_slice(raw, bInc, fdeg, fexp, center, F, threads, use_ref)
    ts = [cpu_one_slice(raw, bInc, fdeg, fexp, center, F, threads, use_ref) for _ in range(args.steps)]
    t = float(np.mean(ts))
    tau = t * 1e9 / (W_DET * W_DET * N_VIEWS)
    kind = "reference" if use_ref else "port"
    line = {
        "impl": "reference", "metric": "tau_ns_per_pixel_view", "value": tau, "unit": "ns/(pixel*view)",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": tau / PUBLISHED_TAU_NS,
        "dtype": "f32/i32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "detector": W_DET, "views": N_VIEWS, "slices_per_step": 1,
                   "slices_in_workload": N_SLICES, "filter": "shepp-logan", "l2": "inputs larger than L2"},
        "slices_per_s": 1.0 / t,
        "cpu_baseline": {"value": tau, "unit": "ns/(pixel*view)", "cores": threads, "kind": kind,
                         "cpu_model": cpu_model(),
                         "sample": "1 slice of the workload per step (2048^2 x 1800 views, normalisation + FBP), "
                                   "reference multi-worker scheme (row bands, every worker filters all views); "
                                   + SCALAR_NOTE},
        "e2e": {"value": tau, "unit": "ns/(pixel*view)", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------ GPU side ---
def run_ours(args, rank: int, world: int, local_rank: int):
    import torch
    import recview_gb300 as rv
    from recview_gb300 import abi, replicas
    from recview_gb300.build import build_lib, build_oracle

    build_lib()
    build_oracle()
    torch.cuda.set_device(local_rank)
    _v, _f = C.c_int(), C.c_int()
    rv.lib().RvGetBackprojectionVariant(C.byref(_v), C.byref(_f))
    bp_variant, bp_format = _v.value, _f.value
    dev = torch.device("cuda", local_rank)
    L = rv.lib()
    S = args.slices
    mode = {"ref": abi.MODE_REF, "lin": abi.MODE_LIN, "f16": abi.MODE_LIN_F16, "bf16": abi.MODE_LIN_BF16}[args.mode]
    raw, bInc, fdeg, fexp, center = make_stack_gpu(args.seed + rank, S, dev)
    F = rv.set_filter(abi.FILT_SHEPP, rv.dims(W_DET).ndim)
    st = rv.Stack(ixdim=W_DET, nframes=raw.shape[0] - 1, nslices=S, center=center, bInc=bInc, fdeg=fdeg,
                  fexp=fexp, fFilter=F, mode=mode)
    npix = st.ixdimp * st.ixdimp
    out = torch.empty((S, st.ixdimp, st.ixdimp), dtype=torch.int32 if mode == abi.MODE_REF else torch.float32,
                      device=dev)
    stream = torch.cuda.Stream(device=dev)
    sh = stream.cuda_stream

    barrier, max_over_ranks = replicas.barrier, replicas.max_over_ranks

    for _ in range(args.warmup):
        st.run_device(raw.data_ptr(), out.data_ptr(), sh)
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    t_filter = t_bp = 0.0
    launches = 0
    with ClockSampler(local_rank) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            st.run_device(raw.data_ptr(), out.data_ptr(), sh)
            tf, tb, _tt = st.timings()
            t_filter += tf
            t_bp += tb
            launches += st.launches()
        e1.record(stream)
        torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps)
    clocks = clk.summary()
    updates_step = float(npix) * st.nviews * S
    total_updates = updates_step * world
    tau = ms * 1e6 / total_updates
    bp_ms = t_bp / args.steps
    filt_ms = t_filter / args.steps

    # ---- end to end through the C ABI with pinned host buffers -----------------------------
    e2e = None
    if not args.no_e2e:
        raw_h = torch.empty(raw.shape, dtype=raw.dtype, pin_memory=True)
        raw_h.copy_(raw)
        out_h = torch.empty(out.shape, dtype=out.dtype, pin_memory=True)
        torch.cuda.synchronize()
        L.RvStackRunHost(st.h, C.c_void_p(raw_h.data_ptr()), C.c_void_p(out_h.data_ptr()), C.c_void_p(sh))
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            rc = L.RvStackRunHost(st.h, C.c_void_p(raw_h.data_ptr()), C.c_void_p(out_h.data_ptr()), C.c_void_p(sh))
            assert rc == 0, rv.last_error()
        torch.cuda.synchronize()
        e2e_ms = max_over_ranks((time.perf_counter() - t0) * 1e3 / args.steps)
        barrier()
        e2e = {"value": e2e_ms * 1e6 / total_updates, "unit": "ns/(pixel*view)",
               "h2d_bytes_per_step": int(raw_h.numel() * raw_h.element_size()),
               "d2h_bytes_per_step": int(out_h.numel() * out_h.element_size()),
               "ms_per_step": e2e_ms, "slices_per_s": S * world * 1e3 / e2e_ms}
        del raw_h, out_h

    # ---- roofline of the dominant kernel (back-projection) ----------------------------------
    probe = (C.c_double * 3)()
    L.RvProbeThroughput(probe, 3)
    fp32_tflops, f2i_gops, smem_gbs = probe[0], probe[1], probe[2]
    upd_bp = updates_step / (bp_ms * 1e-3)                      # one k_bp_ref launch per step
    # algorithmic shared-memory bytes: one 4-byte table entry gathered per pixel-view update
    smem_achieved = 4.0 * upd_bp / 1e9
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm = peaks.get("hbm_gbs")
    nviews = st.nviews
    # stage (a) algorithmic bytes per sinogram sample: 2 B uint16 read + 4 B FP32 filtered value
    # written (the row the back-projection interpolates); the REF path materialises that row as the
    # reference's 16-entry int table (64 B per detector pixel), reported as traffic beside it
    filt_bytes = S * nviews * (2.0 * W_DET + 4.0 * st.ixdimp)
    table_bytes = S * nviews * (2.0 * W_DET + 64.0 * st.ixdimp)
    roof_filter = None
    if hbm and filt_ms > 0:
        a = filt_bytes / (filt_ms * 1e-3) / 1e9
        roof_filter = {"bound": "hbm", "achieved": a, "peak": hbm, "unit": "GB/s", "frac": a / hbm,
                       "traffic": table_bytes if mode == abi.MODE_REF else None,
                       "traffic_note": "raw rows in + the 16-entry int tables out (the REF back-projection's "
                                       "gather format), bytes per step" if mode == abi.MODE_REF else None,
                       "table_write_gbs": table_bytes / (filt_ms * 1e-3) / 1e9 if mode == abi.MODE_REF else None,
                       "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)",
                       "note": "HBM is not this kernel's binding resource: its time goes to latency (each row's loads and recheck, the barriers between transform passes)"}

    if rank == 0:
        line = {
            "metric": "tau_ns_per_pixel_view", "value": tau, "unit": "ns/(pixel*view)", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": tau / PUBLISHED_TAU_NS, "dtype": "f32/i32" if mode == abi.MODE_REF else args.mode,
            "data": "synthetic (seeded ellipsoid phantom, Poisson uint16 frames)",
            "config": {"workload": WORKLOAD, "detector": W_DET, "views": nviews, "slices_per_gpu": S,
                       "output": f"{st.ixdimp}x{st.ixdimp} int32 per slice", "filter": "shepp-logan",
                       "mode": args.mode, "centre": round(center, 4), "parallelism": f"replicas x{world}",
                       "l2": "inputs larger than L2 (raw 472 MB, tables 15 GB)",
                       "bp_variant": bp_variant, "table_format": bp_format},
            "slices_per_s": S * world * 1e3 / ms,
            "updates_per_s": total_updates / (ms * 1e-3),
            "stage_ms": {"filter": filt_ms, "backprojection": bp_ms},
            "e2e": e2e,
            "gpu_launches": launches,
            "roofline": {"bound": "smem", "achieved": smem_achieved, "peak": smem_gbs, "unit": "GB/s",
                         "frac": smem_achieved / smem_gbs if smem_gbs else None,
                         "traffic": BP_DRAM_BYTES_PER_UPDATE * updates_step if mode == abi.MODE_REF else None,
                         "kernel": "k_bp_ref_ws" if bp_variant >= 16 else "k_bp_ref", "bytes_per_update": 4,
                         "peak_source": "measured in this run (RvProbeThroughput: conflict-free 32-bit shared loads)",
                         "updates_per_s_bp": upd_bp,
                         "fp32": {"achieved_tflops": 4.0 * upd_bp / 1e12, "peak_tflops": fp32_tflops,
                                  "frac": 4.0 * upd_bp / 1e12 / fp32_tflops if fp32_tflops else None},
                         "f2i_gops_measured": f2i_gops,
                         "hbm_frac": (BP_DRAM_BYTES_PER_UPDATE * upd_bp / 1e9 / hbm) if hbm else None},
            "roofline_filter": roof_filter,
            "clocks": clocks,
        }
        ref64 = slice0 = None
        if mode == abi.MODE_REF and not args.no_parity:
            # what was timed, checked against the oracle after the timed region: the first and the
            # last slice of the stack (the last one is the second half of a slice pair)
            threads = os.cpu_count() or 1
            checked = sorted({0, S - 1})
            t0 = time.perf_counter()
            mism = {}
            for s_ in checked:
                got = out[s_].cpu().numpy()
                want, r64 = oracle_slice(raw[:, s_, :].cpu().numpy(), bInc, fdeg, fexp, center, F, threads,
                                         lin64=(s_ == 0))
                mism[s_] = int(np.count_nonzero(got != want))
                if s_ == 0:
                    ref64, slice0 = r64, got
            line["parity"] = {"slices_checked": checked, "bit_exact": all(v == 0 for v in mism.values()),
                              "mismatched_pixels": [mism[s_] for s_ in checked],
                              "against": "oracle (reference CPU routine restated), np.array_equal on int32",
                              "seconds": time.perf_counter() - t0}
        if not args.no_cpu and world == 1:
            raw_c, bInc_c, fdeg_c, fexp_c, center_c = host_slice_data(args.seed)
            threads = os.cpu_count() or 1
            runs = [cpu_one_slice(raw_c, bInc_c, fdeg_c, fexp_c, center_c, F, threads, False) for _ in range(3)]
            tcpu = float(np.median(runs))
            tau_cpu = tcpu * 1e9 / (W_DET * W_DET * N_VIEWS)
            line["cpu_baseline"] = {"value": tau_cpu, "unit": "ns/(pixel*view)", "cores": threads, "kind": "port",
                                    "cpu_model": cpu_model(),
                                    "sample": "1 of 64 slices (2048^2 x 1800 views, normalisation + FBP), "
                                              "reference multi-worker scheme, median of 3 runs; " + SCALAR_NOTE,
                                    "seconds": tcpu,
                                    "other_configs": cpu_other_configs(args.seed, threads, dev)}
        if not args.no_forms and world == 1 and mode == abi.MODE_REF:
            line["forms"] = forms_summary(raw, bInc, fdeg, fexp, center, F, S, dev, ref64=ref64, ref_slice0=slice0)
            line["queue"] = queue_summary(dev, args.seed)
            line["queue_small_datasets"] = queue_summary(dev, args.seed + 7, QUEUE_SMALL_SHAPES)
            line["dropin"] = dropin_summary(raw, bInc, fdeg, fexp, center, F)
        if not args.no_centre and world == 1 and NET_FILE.exists():
            # the centre-search part of the metric: the shipped network on fresh scans (C5 shapes)
            from recview_gb300 import centre as cs
            net = cs.CentreNet(batch=1)
            net.set_params(np.fromfile(NET_FILE, dtype=np.float32))
            summ = centre_evaluate(net, CENTRE_SCANS, np.random.default_rng(args.seed + 1))
            net.close()
            summ.pop("disagreements", None)
            line["centre_search"] = {"metric": "centre_search_s", "unit": "s/dataset", "value": summ.pop("learned_s"),
                                     "network": str(NET_FILE.relative_to(ROOT)), **summ}
        print(json.dumps(line), flush=True)
    st.close()


def dropin_summary(raw, bInc, fdeg, fexp, center, F, reps: int = 20) -> dict:
    """The reference's own entry points, one slice per call with host buffers, as RecView drives
    its CUDA back-end: CudaSinogramHost normalises a detector row's frames in place, then
    CudaReconstHost reconstructs the slice (same geometry and data as the stack, slice 0)."""
    import time
    import recview_gb300 as rv
    from recview_gb300.reconst import ReconInfo
    nfr = raw.shape[0]
    frames = np.ascontiguousarray(raw[:, 0, :].cpu().numpy())          # [nframes + 1, W] uint16 bits
    out = {}
    ri = ReconInfo(frames.copy(), fdeg, bInc, center=0, fexp=fexp, maxSinogrLen=nfr)
    rv.normalise(ri)                                                    # warm-up
    t0 = time.perf_counter()
    for _ in range(reps):
        ri.rows[:] = frames
        rv.normalise(ri)
    t_norm = (time.perf_counter() - t0) / reps
    sino = ri.rows.copy()
    rr = ReconInfo(sino, fdeg, bInc, center=center, fFilter=F, maxSinogrLen=nfr, nviews=nfr - 1)
    for _ in range(3):
        rr.reset_output()
        rv.reconstruct_slice(rr)
    t0 = time.perf_counter()
    for _ in range(reps):
        rr.reset_output()
        rv.reconstruct_slice(rr)
    t_rec = (time.perf_counter() - t0) / reps
    upd = float(W_DET) * W_DET * N_VIEWS
    out["reconstruct_ms_per_slice"] = t_rec * 1e3
    out["reconstruct_tau_ns"] = t_rec * 1e9 / upd
    out["normalise_ms_per_slice"] = t_norm * 1e3
    out["slices_per_s"] = 1.0 / (t_rec + t_norm)
    out["host_direct"] = bool(rv.lib().RvHostDirectAccess())
    out["note"] = "CudaSinogramHost + CudaReconstHost per slice, host buffers, host wall clock"
    return out


def forms_summary(raw, bInc, fdeg, fexp, center, F, S, dev, steps: int = 3, ref64=None, ref_slice0=None) -> dict:
    """The reduced-storage forms on the same stack: filtered rows stored as FP32 / FP16 / BF16
    (per-row scale), linear interpolation and FP32 accumulation.  With ref64 (the FP64 end-to-end
    oracle of slice 0) each form's slice 0 error is reported, and the REF drop-in's beside them."""
    import torch
    import recview_gb300 as rv
    from recview_gb300 import abi
    out = {}
    if ref64 is not None and ref_slice0 is not None:
        out["error_measure"] = ("slice 0 of the timed stack against the FP64 end-to-end oracle "
                                "(rvo_reconstruct_lin64_mt: the same normalisation, FP64 FFT filter, linear "
                                "interpolation, double accumulation), inside r < 0.45 of the width")
        out["ref"] = {"note": "the bit-exact drop-in (timed as the main figure)", **error_vs_fp64(ref_slice0, ref64)}
    for name, mode in (("lin_fp32", abi.MODE_LIN), ("lin_fp16", abi.MODE_LIN_F16), ("lin_bf16", abi.MODE_LIN_BF16)):
        st = rv.Stack(ixdim=W_DET, nframes=raw.shape[0] - 1, nslices=S, center=center, bInc=bInc, fdeg=fdeg,
                      fexp=fexp, fFilter=F, mode=mode)
        o = torch.empty((S, st.ixdimp, st.ixdimp), dtype=torch.float32, device=dev)
        st.run_device(raw.data_ptr(), o.data_ptr())
        tt, tb = [], []
        for _ in range(steps):
            st.run_device(raw.data_ptr(), o.data_ptr())
            tf_, tb_, tt_ = st.timings()
            tt.append(tt_)
            tb.append(tb_)
        ms = float(np.mean(tt))
        out[name] = {"tau_ns": ms * 1e6 / (float(st.ixdimp) ** 2 * st.nviews * S), "ms_per_step": ms,
                     "backprojection_ms": float(np.mean(tb))}
        if ref64 is not None:
            out[name].update(error_vs_fp64(o[0].cpu().numpy(), ref64))
        st.close()
        del o
    return out


QUEUE_SHAPES = [(1024, 900, 8, 2), (1536, 1800, 4, 2), (2048, 1800, 4, 2), (4096, 900, 2, 2), (1024, 900, 4, 3),
                (512, 1800, 4, 4)]
# many small datasets (1024-pixel detector, 900 views, one slice pair each): one stack's
# back-projection is 256 CTAs, under one wave, so a queue's shared work list can fill the GPU
QUEUE_SMALL_SHAPES = [(1024, 900, 2, 2)] * 48


def queue_summary(dev, seed: int, shapes=None) -> dict:
    """An uneven queue (configuration C3 shapes, scaled to seconds): widths 512-4096, 900/1800
    views, 1-8 slices, zoom x1/x2/x4 ROIs, run as one persistent kernel per wave in a captured graph,
    against the same datasets one stack at a time."""
    import torch
    import recview_gb300 as rv
    from recview_gb300 import abi
    L = rv.lib()
    rng = np.random.default_rng(seed)
    shapes = QUEUE_SHAPES if shapes is None else shapes
    data = []
    for i, (W, V, S, interp) in enumerate(shapes):
        deg = (np.arange(V) * (180.0 / V)).astype(np.float32)
        raw = torch.empty((V + 3, S, W), dtype=torch.int16, device=dev)
        binc = np.zeros(V + 2, np.int8)
        fdeg = np.zeros(V + 2, np.float32)
        fexp = np.zeros(V + 2, np.float32)
        cen = (W - 1) / 2.0 + float(rng.uniform(-20, 20)) / (2 ** (interp - 2))
        fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))  # noqa: E731
        assert L.RvPhantomFrames(700 + i, W, S, fp(deg), V, cen, 40, C.c_void_p(raw.data_ptr()),
                                 C.c_void_p(binc.ctypes.data), fp(fdeg), fp(fexp), None) == 0
        F = rv.set_filter(abi.FILT_SHEPP, rv.dims(W, interp).ndim)
        n = rv.dims(W, interp).ixdimp
        out = torch.empty((S, n, n), dtype=torch.int32, device=dev)
        data.append((W, V, S, interp, cen, raw, binc, fdeg, fexp, F, out))
    q = C.c_void_p()
    assert L.RvQueueCreate(C.byref(q)) == 0
    keep = []
    for (W, V, S, interp, cen, raw, binc, fdeg, fexp, F, out) in data:
        d = abi.RvStackDesc()
        d.ixdim, d.iInterpolation, d.center, d.nframes, d.nslices = W, interp, cen, V + 2, S
        d.bInc = C.cast(C.c_void_p(binc.ctypes.data), C.POINTER(C.c_char))
        d.fdeg = fdeg.ctypes.data_as(C.POINTER(C.c_float))
        d.fexp = fexp.ctypes.data_as(C.POINTER(C.c_float))
        d.fFilter = F.ctypes.data_as(C.POINTER(C.c_float))
        d.mode = abi.MODE_REF
        keep.append(d)
        assert L.RvQueueAdd(q, C.byref(d), C.c_void_p(raw.data_ptr()), C.c_void_p(out.data_ptr())) == 0, rv.last_error()
    chosen = C.c_int(-1)
    assert L.RvQueueAutotune(q, None, C.byref(chosen)) == 0, rv.last_error()
    assert L.RvQueueRun(q, None) == 0, rv.last_error()      # captures the graph
    # both sides by the same clock and statistic: host wall time of the whole run (each call
    # returns after its work is done), median of 3, after one untimed run
    qms, qdev = [], []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        assert L.RvQueueRun(q, None) == 0, rv.last_error()
        qms.append((time.perf_counter() - t0) * 1e3)
        qdev.append(L.RvQueueLastMs(q))
    upd = L.RvQueueUpdates(q)
    L.RvQueueDestroy(q)
    torch.cuda.synchronize()
    queue_out = [x[10].clone() for x in data]
    stacks = [rv.Stack(ixdim=W, nframes=V + 2, nslices=S, center=cen, bInc=binc, fdeg=fdeg, fexp=fexp, fFilter=F,
                       iInterpolation=interp) for (W, V, S, interp, cen, raw, binc, fdeg, fexp, F, out) in data]
    for st, x in zip(stacks, data):
        st.run_device(x[5].data_ptr(), x[10].data_ptr())
    sms = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for st, x in zip(stacks, data):
            st.run_device(x[5].data_ptr(), x[10].data_ptr())
        torch.cuda.synchronize()
        sms.append((time.perf_counter() - t0) * 1e3)
    for st in stacks:
        st.close()
    same = all(torch.equal(a, x[10]) for a, x in zip(queue_out, data))
    qm, sm = float(np.median(qms)), float(np.median(sms))
    return {"datasets": len(data), "shapes_W_V_S_zoom": [list(x[:3]) + [2 ** (x[3] - 2)] for x in data],
            "updates": upd, "queue_ms": qm, "queue_device_ms": float(np.median(qdev)), "queue_tau_ns": qm * 1e6 / upd,
            "one_stack_at_a_time_ms": sm, "speedup_vs_stacks": sm / qm, "autotuned_variant": chosen.value,
            "bit_exact_vs_stacks": bool(same),
            "timing": "host wall clock of the whole run, median of 3, both sides"}


NET_FILE = ROOT / "recview_gb300" / "data" / "centre_net_256x512.f32"


# fresh scans the default run's centre-search summary evaluates (about 0.2 s each); the
# centre workload (--workload centre --datasets N) runs larger evaluations
CENTRE_SCANS = 100


def centre_evaluate(net, n: int, rng) -> dict:
    """Learned search vs the full sweep on n fresh synthetic scans (2048 x 1800, offset U[-40, 40])."""
    from recview_gb300 import centre as cs
    F = cs.sweep_filter(W_DET)
    res = []
    for j in range(n):
        scan = cs.make_scan(9_000_000 + j, float(rng.uniform(-40, 40)), W_DET, N_VIEWS)
        t0 = time.perf_counter()
        grid = cs.getaxis_grid_centre(scan)
        t_axis = time.perf_counter() - t0
        rl = cs.search(net.h, scan, grid, F)
        rf = cs.search(None, scan, grid, F)
        res.append(dict(true=scan.centre, grid=grid, learned=rl.centre, full=rf.centre, trials=rl.trials,
                        fallback=rl.fallback, ms_l=rl.ms, ms_f=rf.ms, axis_ms=t_axis * 1e3, sigma=rl.sigma,
                        proposal=rl.proposal))
        del scan
    ms_l = float(np.mean([r["ms_l"] for r in res]))
    ms_f = float(np.mean([r["ms_f"] for r in res]))
    dis = [r for r in res if abs(r["learned"] - r["full"]) > 0.25]
    return {
        "learned_s": ms_l / 1e3, "full_sweep_s": ms_f / 1e3, "speedup": ms_f / ms_l,
        "agreement_0p25px": 1.0 - len(dis) / len(res), "datasets": len(res),
        "mean_trials": float(np.mean([r["trials"] for r in res])), "full_trials": 81,
        "fallbacks": int(np.sum([r["fallback"] for r in res])),
        "full_vs_true_px": {"p50": float(np.median([abs(r["full"] - r["true"]) for r in res])),
                            "max": float(max(abs(r["full"] - r["true"]) for r in res))},
        "proposal_err_px": {"p50": float(np.median([abs(r["proposal"] - r["true"]) for r in res])),
                            "max": float(max(abs(r["proposal"] - r["true"]) for r in res))},
        "getaxis_ms": float(np.mean([r["axis_ms"] for r in res])),
        "disagreements": [{k: round(float(v), 3) for k, v in r.items()} for r in dis[:8]],
        "criterion": "total variation of the 4x4-box-averaged trial slice (Hann 0.25 filter) inside r < 0.45",
        "grid": "81 trials, 0.5 px apart, centred on GetAxis",
    }


def run_precision(args):
    """Precision study (4096-pixel detector x 3600 views, 32 slices of 4096^2; 40 ellipsoids plus
    200 small high-contrast spheres): the REF drop-in and the FP32 / FP16 / BF16 filtered-row
    forms on the same device-resident raw frames, each timed and each measured against the FP64
    end-to-end oracle on one slice, in one run.

        python bench.py --workload precision [--steps K] [--warmup W]
    """
    import torch
    import recview_gb300 as rv
    from recview_gb300 import abi
    from recview_gb300.build import build_lib
    build_lib()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    W, V, S = 4096, 3600, 32
    raw, bInc, fdeg, fexp, cen = make_stack_gpu(args.seed, S, dev, W=W, V=V, n_spheres=200)
    F = rv.set_filter(abi.FILT_SHEPP, rv.dims(W).ndim)
    es = S // 2   # the error slice: a middle row of the stack
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    want, ref64 = oracle_slice(raw[:, es, :].cpu().numpy(), bInc, fdeg, fexp, cen, F, threads, lin64=True)
    oracle_s = time.perf_counter() - t0
    res = {}
    for name, mode in (("ref", abi.MODE_REF), ("lin_fp32", abi.MODE_LIN), ("lin_fp16", abi.MODE_LIN_F16),
                       ("lin_bf16", abi.MODE_LIN_BF16)):
        st = rv.Stack(ixdim=W, nframes=V + 2, nslices=S, center=cen, bInc=bInc, fdeg=fdeg, fexp=fexp, fFilter=F,
                      mode=mode)
        out = torch.empty((S, st.ixdimp, st.ixdimp), dtype=torch.int32 if mode == abi.MODE_REF else torch.float32,
                          device=dev)
        for _ in range(max(1, args.warmup)):
            st.run_device(raw.data_ptr(), out.data_ptr())
        tt, tf, tb = [], [], []
        for _ in range(args.steps):
            st.run_device(raw.data_ptr(), out.data_ptr())
            a, b, c = st.timings()
            tf.append(a)
            tb.append(b)
            tt.append(c)
        ms = float(np.mean(tt))
        upd = float(st.ixdimp) ** 2 * st.nviews * S
        got = out[es].cpu().numpy()
        res[name] = {"tau_ns": ms * 1e6 / upd, "ms_per_step": ms, "filter_ms": float(np.mean(tf)),
                     "backprojection_ms": float(np.mean(tb)), "updates_per_s": upd / (ms * 1e-3),
                     **error_vs_fp64(got, ref64)}
        if mode == abi.MODE_REF:
            res[name]["bit_exact_vs_reference_routine"] = bool(np.array_equal(got, want))
        st.close()
        del out
        torch.cuda.empty_cache()
    line = {"metric": "tau_ns_per_pixel_view", "value": res["ref"]["tau_ns"], "unit": "ns/(pixel*view)",
            "higher_is_better": False, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "workload": "precision-4096det-3600views-32slices-raw-uint16-200spheres",
            "data": "synthetic (seeded: 40 ellipsoids + 200 spheres of radius 1-4 px, attenuation U[0.5, 2], "
                    "Poisson uint16 frames)",
            "forms": res,
            "error_measure": f"slice {es} against the FP64 end-to-end oracle (rvo_reconstruct_lin64_mt), inside "
                             "r < 0.45 of the width; relative L2 and max-abs",
            "oracle_seconds": oracle_s, "oracle_threads": threads}
    print(json.dumps(line), flush=True)


def c3_draw(seed: int, n: int = 40) -> list[dict]:
    """The uneven queue's datasets: detector width in {1024, 1536, 2048, 4096}, views in
    {900, 1800, 3600}, 1-256 slices, rotation centre (W - 1) / 2 + U[-20, 20] px; every second
    dataset is a zoomed region of interest: 1/4-1/2 of the field kept by trimming (iTrim) and
    reconstructed at x2 or x4 (iInterpolation 3 / 4)."""
    from recview_gb300.reconst import dims
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        W = int(rng.choice([1024, 1536, 2048, 4096]))
        V = int(rng.choice([900, 1800, 3600]))
        S = int(rng.integers(1, 257))
        off = float(rng.uniform(-20.0, 20.0))
        if i % 2:
            frac = float(rng.uniform(0.25, 0.5))
            interp = int(rng.choice([3, 4]))
            T = int(round(W * (1.0 - frac) / 2.0))
        else:
            interp, T = 2, 0
        ixlen = W - 2 * T
        d = dims(ixlen, interp)
        out.append(dict(W=W, V=V, S=S, cen_raw=(W - 1) / 2.0 + off, interp=interp, T=T, ixlen=ixlen, ixdimp=d.ixdimp,
                        ndim=d.ndim, seed=seed * 1000 + i))
    return out


def run_queue(args):
    """The uneven queue: 40 seeded datasets (c3_draw), raw uint16 frames at full detector width
    on the device, the zoomed ones trimmed and zoomed by the library.  The datasets run in
    batches that fit device memory; each batch runs as one queue (per-shape autotuned variants,
    one captured graph, persistent back-projections) and, on the same buffers, one stack at a time
    (RvStackRunDevice per dataset).  Outputs of the two are compared by checksums per dataset, and
    slice 0 of two datasets against the oracle.

        python bench.py --workload queue [--steps K] [--warmup W]
    """
    import torch
    import recview_gb300 as rv
    from recview_gb300 import abi
    from recview_gb300.build import build_lib
    build_lib()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    L = rv.lib()
    specs = c3_draw(args.seed)
    # one device-memory budget for the tables of the queue pool and of each stack (the stacks of
    # a batch live side by side)
    os.environ.setdefault("RV_TABLE_BUDGET_MB", "8192")
    cap = float(os.environ.get("RV_QUEUE_BATCH_GB", "64")) * 1e9
    batches, cur, size = [], [], 0.0
    for i, d in enumerate(specs):
        b = (d["V"] + 3) * d["S"] * d["W"] * 2 + d["S"] * d["ixdimp"] ** 2 * 4
        if cur and size + b > cap:
            batches.append(cur)
            cur, size = [], 0.0
        cur.append(i)
        size += b
    batches.append(cur)

    def checksum(t):
        # per slice: the sum and a position-weighted sum of the int32 values (in int64)
        w = (torch.arange(t[0].numel(), device=t.device, dtype=torch.int64) % 65521) + 1
        out = []
        for sl in range(t.shape[0]):
            x = t[sl].reshape(-1).long()
            out.append((int(x.sum()), int((x * w).sum())))
        return out

    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))  # noqa: E731
    q_total = s_total = qdev_total = sdev_total = 0.0
    upd_total = 0.0
    same_all = True
    variants, oracle_checks = {}, []
    t_start = time.perf_counter()
    for bi, idx in enumerate(batches):
        data = []
        for i in idx:
            d = specs[i]
            deg = (np.arange(d["V"]) * (180.0 / d["V"])).astype(np.float32)
            raw = torch.empty((d["V"] + 3, d["S"], d["W"]), dtype=torch.int16, device=dev)
            binc = np.zeros(d["V"] + 2, np.int8)
            fdeg = np.zeros(d["V"] + 2, np.float32)
            fexp = np.zeros(d["V"] + 2, np.float32)
            assert L.RvPhantomFrames(d["seed"], d["W"], d["S"], fp(deg), d["V"], d["cen_raw"], 40,
                                     C.c_void_p(raw.data_ptr()), C.c_void_p(binc.ctypes.data), fp(fdeg), fp(fexp),
                                     None) == 0, rv.last_error()
            F = rv.set_filter(abi.FILT_SHEPP, d["ndim"])
            out = torch.empty((d["S"], d["ixdimp"], d["ixdimp"]), dtype=torch.int32, device=dev)
            desc = abi.RvStackDesc()
            desc.ixdim, desc.iInterpolation, desc.center = d["ixlen"], d["interp"], d["cen_raw"] - d["T"]
            desc.nframes, desc.nslices = d["V"] + 2, d["S"]
            desc.bInc = C.cast(C.c_void_p(binc.ctypes.data), C.POINTER(C.c_char))
            desc.fdeg, desc.fexp, desc.fFilter = fp(fdeg), fp(fexp), fp(F)
            desc.mode = abi.MODE_REF
            if d["T"]:
                desc.iTrim, desc.iRawWidth = d["T"], d["W"]
            data.append(dict(i=i, raw=raw, out=out, desc=desc, keep=(binc, fdeg, fexp, F)))
        torch.cuda.synchronize()
        # ---- the queue: per-shape autotuning, graph capture, timed replays ----------------------
        q = C.c_void_p()
        assert L.RvQueueCreate(C.byref(q)) == 0
        for x in data:
            assert L.RvQueueAdd(q, C.byref(x["desc"]), C.c_void_p(x["raw"].data_ptr()),
                                C.c_void_p(x["out"].data_ptr())) == 0, rv.last_error()
        chosen = C.c_int(-1)
        assert L.RvQueueAutotune(q, None, C.byref(chosen)) == 0, rv.last_error()
        for k, x in enumerate(data):
            variants[x["i"]] = L.RvQueueItemVariant(q, k)
        assert L.RvQueueRun(q, None) == 0, rv.last_error()          # captures the graph
        qt, qd = [], []
        for _ in range(max(1, args.steps)):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            assert L.RvQueueRun(q, None) == 0, rv.last_error()
            qt.append(time.perf_counter() - t0)
            qd.append(L.RvQueueLastMs(q) * 1e-3)
        upd_total += L.RvQueueUpdates(q)
        L.RvQueueDestroy(q)
        sums_q = [checksum(x["out"]) for x in data]
        # ---- the same datasets one stack at a time ------------------------------------------------
        stacks = []
        for x in data:
            h = C.c_void_p()
            assert L.RvStackCreate(C.byref(x["desc"]), C.byref(h)) == 0, rv.last_error()
            stacks.append(h)
        for h, x in zip(stacks, data):
            assert L.RvStackRunDevice(h, C.c_void_p(x["raw"].data_ptr()), C.c_void_p(x["out"].data_ptr()), None) == 0
        st_t, st_d = [], []
        tm = (C.c_float * 3)()
        for _ in range(max(1, args.steps)):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            dev_s = 0.0
            for h, x in zip(stacks, data):
                assert L.RvStackRunDevice(h, C.c_void_p(x["raw"].data_ptr()), C.c_void_p(x["out"].data_ptr()),
                                          None) == 0, rv.last_error()
                L.RvStackLastTimings(h, tm)
                dev_s += tm[2] * 1e-3
            torch.cuda.synchronize()
            st_t.append(time.perf_counter() - t0)
            st_d.append(dev_s)
        for h in stacks:
            L.RvStackDestroy(h)
        sums_s = [checksum(x["out"]) for x in data]
        same_all &= sums_q == sums_s
        q_total += float(np.median(qt))
        s_total += float(np.median(st_t))
        qdev_total += float(np.median(qd))
        sdev_total += float(np.median(st_d))
        # ---- slice 0 of the smallest zoomed and unzoomed dataset of the first batch vs the oracle
        if bi == 0:
            from tests.rvtest import Oracle
            oracle = Oracle()
            for zoomed in (False, True):
                cand = [x for x in data if (specs[x["i"]]["T"] > 0) == zoomed]
                if not cand:
                    continue
                x = min(cand, key=lambda y: specs[y["i"]]["ixdimp"] ** 2 * specs[y["i"]]["V"])
                d = specs[x["i"]]
                frames = x["raw"][:, 0, :].cpu().numpy().view(np.uint16)
                rows = oracle.bin_frames(frames[:, None, :], d["W"], d["T"], d["interp"], 1)[:, 0, :]
                binc, fdeg, fexp, F = x["keep"]
                want, _ = oracle_slice(rows, binc, fdeg, fexp, d["cen_raw"] - d["T"], F, os.cpu_count() or 1,
                                       interp=d["interp"])
                oracle_checks.append({"dataset": x["i"], "zoomed": zoomed,
                                      "bit_exact": bool(np.array_equal(x["out"][0].cpu().numpy(), want))})
        del data
        torch.cuda.empty_cache()
    line = {"metric": "tau_ns_per_pixel_view", "value": q_total * 1e9 / upd_total, "unit": "ns/(pixel*view)",
            "higher_is_better": False, "n_gpus": 1, "steps": args.steps, "warmup": 1,
            "workload": "queue-40-datasets-uneven-width-views-slices-centre-zoomed-roi",
            "data": "synthetic (seeded ellipsoid phantom frames at full detector width, Poisson uint16)",
            "datasets": len(specs), "batches": len(batches),
            "shapes_W_V_S_zoom_trim": [[d["W"], d["V"], d["S"], 2 ** max(d["interp"] - 2, 0), d["T"]] for d in specs],
            "updates": upd_total, "queue_s": q_total, "one_stack_at_a_time_s": s_total,
            "speedup_vs_stacks": s_total / q_total, "slices_per_s": sum(d["S"] for d in specs) / q_total,
            "device_s": {"queue": qdev_total, "one_stack_at_a_time": sdev_total,
                         "note": "device time between the events bracketing each call (queue graph, or each stack's "
                                 "kernels); wall minus device is the host time between the GPU's work"},
            "autotuned_variant_per_dataset": [variants[i] for i in range(len(specs))],
            "outputs_equal_queue_vs_stacks": bool(same_all), "oracle_checks": oracle_checks,
            "timing": "host wall clock per batch (each call returns after its work), median of the timed runs, summed "
                      "over batches; autotuning and graph capture outside the timed runs",
            "table_budget_mb": int(os.environ["RV_TABLE_BUDGET_MB"]),
            "wall_s": time.perf_counter() - t_start}
    print(json.dumps(line), flush=True)


def run_centre(args):
    """Learned centre search vs the plain full sweep (configuration C5 shapes: 2048-pixel detector,
    1800 views, uint16 Poisson raw frames, true offset U[-40, 40] px)."""
    import torch
    from recview_gb300 import abi
    from recview_gb300 import centre as cs
    from recview_gb300.build import build_lib
    build_lib()
    torch.cuda.set_device(0)
    W = W_DET
    rng = np.random.default_rng(args.seed)
    net = cs.CentreNet(batch=32)
    train = {}
    if args.net:
        net.set_params(np.fromfile(args.net, dtype=np.float32))
        train["source"] = args.net
    else:
        nval = max(256, args.train // 16)
        desc = abi.RvCentreTrainDesc(W=W, views=N_VIEWS, slices=4, n_ellipsoids=40, max_offset=40.0, seed=args.seed)
        t0 = time.perf_counter()
        X, Y = cs.make_samples(desc, 0, args.train + nval)
        train["generate_s"] = time.perf_counter() - t0
        st = cs.fit(net, X, Y, args.train, nval, args.epochs)
        train.update(samples=args.train, held_out=nval, epochs=args.epochs, fit_s=float(st[3]),
                     held_out_err_px={"p50": float(st[0]), "p90": float(st[1]), "p99": float(st[2])})
        if args.finetune:
            # the plain sweep's own optima as targets, mixed with as many generated samples
            F = cs.sweep_filter(W)
            t0 = time.perf_counter()
            xs, ys = [], []
            for j in range(args.finetune):
                scan = cs.make_scan(5_000_000 + j, float(rng.uniform(-40, 40)), W, N_VIEWS)
                r = cs.search(None, scan, cs.getaxis_grid_centre(scan), F)
                xs.append(cs.scan_input(scan))
                ys.append((r.centre - (W - 1) / 2.0) / 16.0)
                del scan
            m = len(xs)
            Xf = torch.cat(xs + [X[:m]], 0).contiguous()
            Yf = torch.cat([torch.tensor(ys, dtype=torch.float32, device="cuda"), Y[:m]], 0).contiguous()
            cs.fit(net, Xf, Yf, 2 * m, 0, 4, lr_max=1e-4, lr_min=1e-5)
            train["finetune_scans"] = m
            train["finetune_s"] = time.perf_counter() - t0
            del Xf, Yf
        del X, Y
        torch.cuda.empty_cache()
        if args.save_net:
            net.get_params().tofile(args.save_net)
    line = {"metric": "centre_search_s", "unit": "s/dataset", "higher_is_better": False, "n_gpus": 1,
            "workload": "centre-search-2048det-1800views-offset-40px",
            "data": "synthetic (seeded ellipsoid phantom, Poisson uint16 frames, true centre offset U[-40, 40] px)"}
    summ = centre_evaluate(net, args.datasets, rng)
    line["value"] = summ.pop("learned_s")
    line.update(summ)
    line["train"] = train
    print(json.dumps(line), flush=True)
    net.close()


def main():
    args = parse()
    if args.workload == "centre":
        run_centre(args)
        return
    if args.workload == "precision":
        run_precision(args)
        return
    if args.workload == "queue":
        run_queue(args)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group(backend="nccl")
    try:
        run_ours(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
