"""Benchmark: input spectra/s of the streaming unpack -> IPFB -> PFB -> xcorr chain.

Workload (the full-chain streaming configuration): 2 antennas x 2 pols of
4-bit packets, 64 contiguous coarse channels, 2^20 spectra per antenna fed in
chunks of 2^15 spectra (IPFB cut 10, the reference's default -> nslice 32788;
--cut 80 gives nslice 32928 = 2^5*3*7^3), PFB osamp 64 (4096 fine channels),
512 fine blocks per job (31 jobs), fine 4x4 visibilities per job.  One step =
the whole 2^20-spectrum stream.  Synthetic seeded data (Gaussian nibbles,
sigma 2.5, clipped to +-7).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference|plain-gpu] [--cut C]

Prints one JSON line (rank 0).  `value` is device-resident throughput; `e2e`
is the same through the public API from pinned host packets with the H2D copy
of the step's packets and the D2H read of the visibilities inside the timed
region; `roofline` is the dominant kernel's achieved HBM bandwidth against
MEASURED_PEAKS.json; `cpu_baseline` the CPU chain on this host's cores over a
bounded sample; `parity` the error of jobs 0-1 and of the IPFB and PFB outputs
against the FP64 oracle (computed after the timed regions); `plain_gpu` the
reference's plain GPU path (its CuPy glue restated in torch around cuFFT and
cuBLAS, baseline/plain_gpu.py) on the same workload.  `--impl reference` times
the reference's CPU path; `--impl plain-gpu` prints the plain GPU path's own
line.
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

METRIC = "input spectra/s, unpack→IPFB→PFB→xcorr on 1 GB300 vs plain GPU path; HBM % roofline"
NANT, NCHAN_RAW, NSPEC, ACCLEN, CUT, OSAMP, NBLOCK, NTAP, THRESH = 2, 64, 2 ** 20, 2 ** 15, 10, 64, 512, 4, 0.45
CHAN0 = 640  # absolute number of the first recorded coarse channel
P = 4096


def workload():
    return ("full-chain streaming: 2 ant x 2 pol 4-bit, 64 coarse ch, 2^20 spectra in 2^15-spectrum chunks, "
            f"cut {CUT} (nslice {ACCLEN + 2 * CUT}), osamp 64 -> 4096 fine ch, 512 fine blocks/job (31 jobs), "
            "fine xcorr")


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
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

    def __exit__(self, *a):
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
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def synth_raw(torch, device, seed=1234):
    """(NANT, NSPEC, 2*NCHAN_RAW) uint8 Gaussian 4-bit packets, made on the device."""
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    shape = (NANT, NSPEC, NCHAN_RAW, 2)
    def nib():
        v = torch.randn(shape, generator=g, device=device, dtype=torch.float32) * 2.5
        return torch.clamp(torch.round(v), -7, 7).to(torch.int16) & 15
    re, im = nib(), nib()
    return ((re << 4) | im).to(torch.uint8).reshape(NANT, NSPEC, 2 * NCHAN_RAW).contiguous()


def stage_bytes(sc):
    """Algorithmic DRAM bytes per launch of each stage for one chunk.
    Unit = one input row (one pol of one spectrum) of 4096 samples."""
    M, nslice, nq = 2 * NANT, ACCLEN + 2 * CUT, sc.nq
    nb = ACCLEN // OSAMP
    L = P * OSAMP
    kind, par = sc.time_filter()
    # rows of each IPFB column the time stage must read: all nslice for the
    # FFT form, the kept rows plus the filter's halo for the FIR/IIR forms
    rows_in = {"fft": nslice, "fir": ACCLEN + 2 * par, "iir": ACCLEN + 2 * par + 3}[kind]
    return {
        "row_ifft": NANT * nslice * 2 * NCHAN_RAW + M * P * nslice * 4,      # packets in, f32 rows out
        # time-axis deconvolution with the PFB fold fused in: IPFB column in,
        # folded/DFT'd fine blocks (W) out
        "time_deconv": M * P * rows_in * 4 + M * nb * L * 4,
        "pfb_fold": 0,                                                      # fused into time_deconv
        "pfb_dft": M * nb * L * 4 + M * nb * nq * 8,                         # W in, band spectra out
        "xcorr": M * nb * nq * 8,                                           # band spectra in
    }


def traffic_per_launch(stage):
    """DRAM bytes (read + write) per launch of `stage`, from the ncu summary
    committed in profiles/ (lines `traffic_per_launch <stage> <bytes>`)."""
    import re
    path = os.path.join(ROOT, "profiles", "dram_traffic_per_launch.txt")
    try:
        for line in open(path):
            m = re.match(r"traffic_per_launch\s+(\w+)\s+(\d+)", line)
            if m and m.group(1) == stage:
                return int(m.group(2))
    except OSError:
        pass
    return None


def replica_ms(ms: float, dist, device) -> float:
    """Step time of the whole job: the slowest replica's (max over ranks)."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(world: int, units_per_rank: float, ms: float) -> float:
    """Units all ranks processed per second (weak scaling: each rank runs the
    same per-replica workload)."""
    return world * units_per_rank / (ms / 1e3)


def run_ours(args):
    import torch
    global NSPEC, NANT
    if args.chunks:
        NSPEC = ACCLEN * args.chunks
    if args.nant:
        NANT = args.nant
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from albatros_axion_detection_gb300 import stream

    channels = np.arange(CHAN0, CHAN0 + NCHAN_RAW)
    raw = synth_raw(torch, dev)
    if args.row_ffts:
        from albatros_axion_detection_gb300 import autotune
        autotune.set_row_ffts_per_cta(args.row_ffts)
    if args.row_prefetch >= 0:
        from albatros_axion_detection_gb300 import autotune
        autotune.set_row_prefetch(args.row_prefetch)
    if args.row_tc >= 0:
        from albatros_axion_detection_gb300 import autotune
        autotune.set_row_tc(args.row_tc)
    if args.pfb_tma >= 0:
        from albatros_axion_detection_gb300 import autotune
        autotune.set_pfb_tma(args.pfb_tma)
    if args.time_filter != "default" or args.row_tile:
        from albatros_axion_detection_gb300 import autotune
        mode = {"iir": 0, "fir": 3, "fft": 1}.get(args.time_filter, autotune.DEFAULT_MODE)
        autotune.set_time_filter(mode, args.row_tile)
    sc = stream.StreamCorrelator(NANT, channels, 0, NCHAN_RAW, ACCLEN, NSPEC // ACCLEN, NBLOCK, OSAMP, CUT, THRESH,
                                 NTAP, nchan_raw=NCHAN_RAW)
    nchunks = NSPEC // ACCLEN
    s = torch.cuda.current_stream(dev)

    def step(src):
        sc.reset()
        for j in range(nchunks):
            sc.push(src, j, final=(j == nchunks - 1))

    def barrier():
        if dist is not None:
            dist.barrier()

    for _ in range(args.warmup):
        step(raw)
    torch.cuda.synchronize()
    step(raw)
    launches_per_step = sc.kernel_launches()  # counter restarts at reset()
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(s)
        for _ in range(args.steps):
            step(raw)
        e1.record(s)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    barrier()
    ms = replica_ms(ms, dist, dev)
    spectra_per_step = NANT * NSPEC
    value = job_throughput(world, spectra_per_step, ms)

    # ---- end to end: pinned host packets -> device, chain, visibilities -> host
    host = torch.empty(raw.shape, dtype=torch.uint8, pin_memory=True)
    host.copy_(raw)
    dev_in = torch.empty_like(raw)
    vis_host = torch.empty(sc.vis_device().shape, dtype=torch.complex64, pin_memory=True)

    copy_stream = torch.cuda.Stream(device=dev)

    def e2e_step():
        sc.reset()
        sc.run_from_host(host, dev_in, copy_stream=copy_stream)  # per-chunk H2D overlapped with the chain
        vis_host.copy_(sc.vis_device(), non_blocking=True)

    for _ in range(max(1, args.warmup // 2)):
        e2e_step()
    torch.cuda.synchronize()
    barrier()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(s)
    for _ in range(args.steps):
        e2e_step()
    f1.record(s)
    torch.cuda.synchronize()
    ms_e2e = replica_ms(f0.elapsed_time(f1) / args.steps, dist, dev)

    # ---- per-stage timing (serialised, separate pass) for the roofline
    sc.profile(True)
    step(raw)
    torch.cuda.synchronize()
    st = sc.stage_times()
    sc.profile(False)
    algo = stage_bytes(sc)
    dom = max(st, key=lambda k: st[k][0])
    tot_ms, nl = st[dom]
    avg_ms = tot_ms / max(nl, 1)
    # bytes per launch: stages run once per chunk (PFB/xcorr: per chunk's blocks)
    per_launch = algo[dom] * nchunks / max(nl, 1)
    peak, peak_kind = peaks()
    achieved = per_launch / (avg_ms / 1e3) / 1e9
    traffic = traffic_per_launch(dom)

    parity = None
    if rank == 0 and not args.no_check and nchunks >= 3 and NANT == 2:
        vis01 = sc.vis_device()[:2].permute(1, 2, 3, 0).cpu().numpy()
        parity = parity_check(raw[:, : 3 * ACCLEN].cpu().numpy(), vis01)

    plain = None
    if rank == 0 and not args.no_plain:
        plain = plain_gpu_leg(args, raw, local)

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline_sample(raw.cpu().numpy(), sc)

    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": "spectra/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded Gaussian 4-bit packets)",
            "config": {"workload": workload(), "spectra_per_step": spectra_per_step, "chunks_per_step": nchunks,
                       "time_stage": "%s %d" % sc.time_filter(),
                       "parallelism": f"replicas x{world}",
                       "l2": "inputs larger than L2 (256 MiB packets, 2 x 4.3 GB IPFB intermediates per step)"},
            "e2e": {"value": job_throughput(world, spectra_per_step, ms_e2e), "unit": "spectra/s",
                    "ms_per_step": ms_e2e, "h2d_bytes_per_step": int(host.numel()),
                    "d2h_bytes_per_step": int(vis_host.numel() * 8)},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                         "algorithmic_bytes_per_launch": per_launch, "avg_launch_ms": avg_ms,
                         "stages_ms_per_step": {k: v[0] for k, v in st.items()},
                         "chain_algorithmic_GBps": sum(algo.values()) * nchunks / (ms / 1e3) / 1e9},
            "gpu_launches": int(launches_per_step * args.steps),
            "clocks": clk.summary(),
        }
        if parity:
            out["parity"] = parity
            out["max_rel_err"] = parity["vis_max_rel_err"]
        if plain:
            out["plain_gpu"] = dict(plain, speedup=value / plain["value"],
                                    e2e_speedup=out["e2e"]["value"] / plain["e2e"]["value"])
        if cpu:
            out["cpu_baseline"] = cpu
        print(json.dumps(out), flush=True)
    sc.close()
    if dist is not None:
        dist.destroy_process_group()


def parity_check(raw3, vis01):
    """Errors of the benchmark's own outputs against the FP64 oracle, over the
    first three chunks (which fully determine jobs 0 and 1):
    - fine visibilities of jobs 0-1 (norm-wise relative, per job);
    - the IPFB timestream: cupy_ipfb on chunk 0's rows of input 0 (with the
      2*cut zero rows before them) against the FP64 IPFB and filter;
    - the PFB band spectra: cupy_pfb_band over job 0's float32 timestream of
      input 0 against the FP64 PFB of the same samples."""
    import torch
    from albatros_axion_detection_gb300 import pfb_gpu_utils as pg
    from oracle import pfb_oracle as po
    t0 = time.perf_counter()
    channels = np.arange(CHAN0, CHAN0 + NCHAN_RAW)
    sel = np.arange(NCHAN_RAW)
    nslice = ACCLEN + 2 * CUT
    filt = po.calculate_filter(po.get_matft(nslice), THRESH)
    ref, (q0, q1) = po.repfb_xcorr_avg(raw3, channels, ACCLEN, 3, NBLOCK, 0, NCHAN_RAW, OSAMP, cut=CUT, filt=filt,
                                       max_jobs=2)
    vis_errs = [float(np.linalg.norm(vis01[..., k] - ref[..., k]) / np.linalg.norm(ref[..., k])) for k in range(2)]
    out = {"vis_rel_err_per_job": vis_errs, "vis_max_rel_err": max(vis_errs), "jobs_checked": [0, 1]}
    # IPFB timestream through cupy_ipfb
    spec = po.unpack_4bit_np(raw3[0], 0, ACCLEN, sel)[0]
    dat = np.zeros((nslice, 2049), np.complex128)
    dat[2 * CUT:] = po.make_continuous(spec, np.arange(ACCLEN), 0, channels, ACCLEN)
    try:
        got = pg.cupy_ipfb(torch.from_numpy(dat.astype(np.complex64)).cuda(), pg.build_filter(nslice, THRESH))
        exp = po.ipfb(dat, filt)
        out["ipfb_timestream_rel_err"] = float(np.linalg.norm(got.cpu().numpy() - exp) / np.linalg.norm(exp))
    except Exception as e:  # a length the library's cupy_ipfb does not run
        out["ipfb_timestream_rel_err"] = None
        out["ipfb_timestream_note"] = str(e).splitlines()[0][:160]
    del dat
    # PFB band spectra through cupy_pfb_band
    lblock = P * OSAMP
    ts = po.stream_timestream(raw3, 0, 0, sel, channels, ACCLEN, 2, CUT, filt)
    ts32 = ts[: (NBLOCK + NTAP - 1) * lblock].astype(np.float32)
    del ts
    win = po.sinc_hamming(NTAP, lblock)
    exp = po.pfb(ts32.astype(np.float64), win, nchan=lblock // 2 + 1, ntap=NTAP)[:, q0:q1]
    got = pg.cupy_pfb_band(torch.from_numpy(ts32).cuda(), win.astype(np.float32), q0, q1, nchan=lblock // 2 + 1)
    out["pfb_band_rel_err"] = float(np.linalg.norm(got.cpu().numpy() - exp) / np.linalg.norm(exp))
    out["oracle"] = "FP64 (pocketfft float64), norm-wise relative error"
    out["check_s"] = time.perf_counter() - t0
    return out


def plain_gpu_leg(args, raw, local):
    """The reference's plain GPU path on the same device-resident packets:
    `value` with the packets already on the device (its per-job D2H of the
    visibilities included, as the reference does it), `e2e` with the packets'
    H2D from pinned host memory inside the timed region too."""
    import torch
    try:
        from baseline import plain_gpu
        plain_gpu.lib()
    except Exception as e:
        return {"unavailable": str(e).splitlines()[0][:160]}
    channels = np.arange(CHAN0, CHAN0 + NCHAN_RAW)
    nchunks = raw.shape[1] // ACCLEN
    chain = plain_gpu.PlainGpuChain(raw.shape[0], channels, ACCLEN, nchunks, NBLOCK, OSAMP, CUT, THRESH, NTAP)
    ms, clk = _timed(torch, lambda: chain.run(raw), args.steps, args.warmup, local)
    host = torch.empty(raw.shape, dtype=torch.uint8, pin_memory=True)
    host.copy_(raw)
    dev_in = torch.empty_like(raw)

    def e2e():
        dev_in.copy_(host, non_blocking=True)
        chain.run(dev_in)
    ms_e2e, _ = _timed(torch, e2e, args.steps, 1, local)
    chain.close()
    spectra = raw.shape[0] * raw.shape[1]
    return {"impl": "plain-gpu", "value": spectra / (ms / 1e3), "unit": "spectra/s", "ms_per_step": ms,
            "e2e": {"value": spectra / (ms_e2e / 1e3), "unit": "spectra/s", "ms_per_step": ms_e2e,
                    "h2d_bytes_per_step": int(host.numel()),
                    "d2h_bytes_per_step": int(chain.vis.size * 8)},
            "what": "reference's CuPy glue restated op for op in torch around cuFFT (R2C/C2R plans, shared work "
                    "area) and cuBLAS CgemmStridedBatched (handle per call), baseline/plain_gpu.py",
            "clocks": clk}


def run_plain(args):
    """--impl plain-gpu: the plain GPU path's own JSON line."""
    import torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    torch.cuda.set_device(local)
    raw = synth_raw(torch, torch.device("cuda", local))
    leg = plain_gpu_leg(args, raw, local)
    out = {"impl": "plain-gpu", "metric": METRIC, "unit": "spectra/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded Gaussian 4-bit packets)",
           "config": {"workload": workload(), "spectra_per_step": int(raw.shape[0] * raw.shape[1])}}
    out.update(leg)
    print(json.dumps(out), flush=True)


BATCH_WORKLOAD = ("uneven batch: 24 files (16 x 4-bit, 8 x 1-bit), 2 ant x 2 pol each, channels from {32,64,128,512}, "
                  "2^14..2^19 spectra, osamp from {16,64}, acclen 2^14 (cut 40) or 2^15 (cut 80), one captured graph")


def _file_job0_error(args):
    """Relative error of job 0 of one file against the FP64 oracle (runs the
    oracle on the file's first two chunks, which fully determine job 0)."""
    import numpy as np
    from oracle import pfb_oracle as po
    raw, channels, acclen, cut, osamp, nblock, bits, vis0 = args
    ref, _ = po.repfb_xcorr_avg(raw, channels, acclen=acclen, nchunks=2, nblock=nblock, chanstart=0,
                                chanend=len(channels), osamp=osamp, cut=cut, bits=bits)
    r = ref[..., 0]
    return float(np.linalg.norm(vis0 - r) / np.linalg.norm(r))


def run_batch(args):
    """The uneven batch in one captured graph (device-resident value; e2e
    with the packets' H2D and the visibilities' D2H inside the graph)."""
    import torch
    from albatros_axion_detection_gb300 import batch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    specs = batch.uneven_batch_specs(seed=2024)
    files = batch.files_from_specs(specs, dev, host_copies=True)
    t0 = time.perf_counter()
    bc = batch.BatchCorrelator(files, lanes=args.lanes, tune=True, vis_to_host=True)
    t_setup = time.perf_counter() - t0
    bc.capture()
    s = torch.cuda.current_stream(dev)
    for _ in range(args.warmup):
        bc.run(io=False)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(s)
        for _ in range(args.steps):
            bc.run(io=False)
        e1.record(s)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    bc.run(io=True)
    torch.cuda.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(s)
    for _ in range(args.steps):
        bc.run(io=True)
    f1.record(s)
    torch.cuda.synchronize()
    ms_e2e = f0.elapsed_time(f1) / args.steps
    spectra = bc.spectra
    out = {
        "metric": METRIC, "value": world * spectra / (ms / 1e3), "unit": "spectra/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded 4-bit Gaussian / 1-bit sign packets)",
        "config": {"workload": BATCH_WORKLOAD, "spectra_per_step": spectra, "files": len(files), "lanes": len(bc.lanes),
                   "parallelism": f"replicas x{world}",
                   "tuned_time_stage": {f"acclen{k[0]}_cut{k[1]}_osamp{k[2]}": v for k, v in bc.tuned.items()},
                   "setup_s": t_setup, "l2": "inputs larger than L2",
                   "workspace_gb_per_lane": [round(w.numel() / 1e9, 3) for w in bc.workspaces if w is not None]},
        "e2e": {"value": world * spectra / (ms_e2e / 1e3), "unit": "spectra/s", "ms_per_step": ms_e2e,
                "h2d_bytes_per_step": bc.h2d_bytes, "d2h_bytes_per_step": bc.d2h_bytes},
        "gpu_launches": int(bc.launches_per_run() * args.steps),
        "clocks": clk.summary(),
    }
    if args.check:
        import multiprocessing as mp
        jobs = []
        for i, f in enumerate(files):
            two = f.host[:, : 2 * f.acclen].numpy().copy()
            vis0 = bc.vis_host[i][0].numpy()  # (M, M, nq) of job 0
            jobs.append((two, f.channels, f.acclen, f.cut, f.osamp, f.nblock, f.bits, vis0))
        with mp.get_context("spawn").Pool(min(4, os.cpu_count() or 1)) as pool:
            errs = pool.map(_file_job0_error, jobs)
        out["per_file_job0_rel_err"] = {f.name: e for f, e in zip(files, errs)}
        out["max_rel_err"] = max(errs)
    bc.close()
    print(json.dumps(out), flush=True)


def _timed(torch, fn, steps, warmup, local, min_s=2.0):
    """ms per call of fn() (CUDA events on the current stream, after warm-up).
    Short calls are repeated until the timed region lasts at least min_s, so
    that the clock sampler (every 200 ms) sees it; the calls actually timed
    are in the returned clock record as `timed_calls`."""
    s = torch.cuda.current_stream()
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    fn()
    torch.cuda.synchronize()
    one = max(time.perf_counter() - t0, 1e-6)
    n = max(int(steps), int(np.ceil(min_s / one)))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(s)
        for _ in range(n):
            fn()
        e1.record(s)
        torch.cuda.synchronize()
    summary = dict(clk.summary(), timed_calls=n)
    return e0.elapsed_time(e1) / n, summary


def _line(metric, value, unit, ms, args, workload, extra):
    out = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "data": "synthetic (seeded)", "config": {"workload": workload}}
    out.update(extra)
    print(json.dumps(out), flush=True)


def run_coarse(args, nant, nchan, nspec, chunk, workload):
    """Exact all-baseline coarse correlation of 4-bit packets (fp16 operands
    on the tcgen05 tensor cores from 9 antennas up, warp-level mma.sync
    below, or int8 mma.sync with --mma-bits 8; int64 sums): configurations
    'plain unpack + xcorr' and 'many-antenna coarse correlator'."""
    import torch
    from albatros_axion_detection_gb300 import correlations
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    g = torch.Generator(device=dev)
    g.manual_seed(4321)
    shape = (nant, nspec, nchan, 2)

    def nib():
        v = torch.randn(shape, generator=g, device=dev, dtype=torch.float32) * 2.5
        return torch.clamp(torch.round(v), -7, 7).to(torch.int16) & 15
    re, im = nib(), nib()
    raw = ((re << 4) | im).to(torch.uint8).reshape(nant, nspec, 2 * nchan).contiguous()
    del re, im
    channels = np.arange(nchan)
    if args.mma_bits:
        from albatros_axion_detection_gb300 import autotune
        autotune.set_coarse_mma_bits(args.mma_bits)
    if args.coarse_tma >= 0:
        from albatros_axion_detection_gb300 import autotune
        autotune.set_coarse_tc_tma(args.coarse_tma)
    fn = lambda: correlations.xcorr_coarse_4bit(raw, 0, nspec, channels, nchan, chunk=chunk, average=False)
    ms, clk = _timed(torch, fn, args.steps, args.warmup, local)
    host = torch.empty(raw.shape, dtype=torch.uint8, pin_memory=True)
    host.copy_(raw)
    dev_in = torch.empty_like(raw)

    def e2e():
        dev_in.copy_(host, non_blocking=True)
        re_, im_ = correlations.xcorr_coarse_4bit(dev_in, 0, nspec, channels, nchan, chunk=chunk, average=False)
        return re_.cpu(), im_.cpu()
    out_re, out_im = e2e()
    ms_e2e, _ = _timed(torch, e2e, args.steps, 1, local)
    spectra = nant * nspec
    bytes_in = raw.numel()
    peak, peak_kind = peaks()
    achieved = bytes_in / (ms / 1e3) / 1e9
    M = 2 * nant
    macs = spectra // nant * nchan * (M * (M + 1) // 2) * 4  # real int MACs, unique pairs
    _line("input spectra/s, exact all-baseline coarse correlation (tensor cores, int64 sums)",
          spectra / (ms / 1e3), "spectra/s", ms, args, workload,
          {"dtype": ("int8" if args.mma_bits == 8 else "fp16 (exact small integers)") + " -> int64", "clocks": clk,
           "e2e": {"value": spectra / (ms_e2e / 1e3), "unit": "spectra/s", "ms_per_step": ms_e2e,
                   "h2d_bytes_per_step": int(bytes_in), "d2h_bytes_per_step": int(out_re.numel() * 16)},
           "roofline": {"bound": "hbm",
                        "kernel": ("coarse_xcorr_kernel (int8 mma.sync)" if args.mma_bits == 8 else
                                   ("coarse_xcorr_tc_tma_kernel (tcgen05, TMA-staged packets)"
                                    if nant <= 16 and args.coarse_tma != 0 and (2 * nchan) % 16 == 0 else
                                    "coarse_xcorr_tc_kernel (tcgen05)") if 9 <= nant <= 32 else
                                   "coarse_xcorr_f16_kernel (fp16 mma.sync)"),
                        "achieved": achieved, "peak": peak,
                        "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                        "int_macs_per_s_unique_pairs": macs / (ms / 1e3)},
           "gpu_launches": None})


def run_ipfb_pfb(args):
    """IPFB + PFB rechannelisation of one input: 4096 rows of 2049 channels
    -> IPFB (threshold 0.45) -> PFB osamp 64 on 64 selected coarse channels."""
    import torch
    from albatros_axion_detection_gb300 import pfb_gpu_utils as pg
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    nslice, nchan, osamp, c0 = 4096, 2049, 64, 640
    g = torch.Generator(device=dev)
    g.manual_seed(99)
    dat = torch.complex(torch.randn(nslice, nchan, generator=g, device=dev),
                        torch.randn(nslice, nchan, generator=g, device=dev)).to(torch.complex64)
    filt = pg.calculate_filter(pg.get_matft(nslice, nchan, 4), 0.45)
    lblock = 4096 * osamp
    # fine PFB window (sinc-Hamming, ntap 4) built on the host in double
    N = 4 * lblock
    i = np.arange(N)
    w = (0.54 - 0.46 * np.cos(2 * np.pi * i / (N - 1))) * np.sinc((i - N / 2) / lblock)
    win = torch.from_numpy(w.astype(np.float32)).to(dev)
    q0, q1 = c0 * osamp, (c0 + 64) * osamp

    def fn():
        ts = pg.cupy_ipfb(dat, filt)
        return pg.cupy_pfb_band(ts.contiguous().reshape(-1), win, q0, q1, nchan=lblock // 2 + 1)
    ms, clk = _timed(torch, fn, args.steps, args.warmup, local)
    _line("input spectra/s, IPFB (lblock 4096) + PFB osamp 64 band of 64 coarse channels, one input",
          nslice / (ms / 1e3), "spectra/s", ms, args,
          "IPFB 4096 rows x 2049 channels (threshold 0.45) + PFB osamp 64 on 64 channels",
          {"dtype": "f32", "clocks": clk, "gpu_launches": None})


def cpu_baseline_sample(raw_np, sc=None, reps=1):
    """The CPU chain over one 2^15-spectrum chunk of both antennas."""
    from oracle import cpu_chain
    channels = np.arange(CHAN0, CHAN0 + NCHAN_RAW)
    q0, q1 = CHAN0 * OSAMP, (CHAN0 + NCHAN_RAW) * OSAMP
    sec, kind, workers = cpu_chain.time_sample(raw_np, np.arange(NCHAN_RAW), channels, NCHAN_RAW, ACCLEN, CUT, OSAMP,
                                               q0, q1, reps=reps)
    return {"value": NANT * ACCLEN / sec, "unit": "spectra/s", "cores": workers, "kind": kind,
            "sample": f"one {ACCLEN}-spectrum chunk of both antennas (unpack, IPFB, PFB, xcorr), {sec:.2f} s"}


def run_reference(args):
    """The reference's CPU path on this host's cores (rank 0 only)."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    rng = np.random.default_rng(1234)
    shape = (NANT, 2 * ACCLEN, NCHAN_RAW, 2)
    nib = lambda: np.clip(np.rint(rng.normal(0, 2.5, shape).astype(np.float32)), -7, 7).astype(np.int64) & 15
    raw = ((nib() << 4) | nib()).astype(np.uint8).reshape(NANT, 2 * ACCLEN, 2 * NCHAN_RAW)
    from oracle import cpu_chain
    channels = np.arange(CHAN0, CHAN0 + NCHAN_RAW)
    q0, q1 = CHAN0 * OSAMP, (CHAN0 + NCHAN_RAW) * OSAMP
    chain = cpu_chain.CpuChain(channels, ACCLEN, CUT, OSAMP, q0, q1, THRESH, NTAP)
    for _ in range(args.warmup):
        chain.run_chunk(raw, np.arange(NCHAN_RAW), NCHAN_RAW, 0)
    t0 = time.perf_counter()
    for k in range(args.steps):
        chain.run_chunk(raw, np.arange(NCHAN_RAW), NCHAN_RAW, k % 2)
    sec = (time.perf_counter() - t0) / args.steps
    value = NANT * ACCLEN / sec
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": "spectra/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded Gaussian 4-bit packets)",
           "config": {"workload": workload(), "step": f"one {ACCLEN}-spectrum chunk of both antennas"},
           "cpu_baseline": {"value": value, "unit": "spectra/s", "cores": chain.workers, "kind": chain.kind,
                            "sample": f"one {ACCLEN}-spectrum chunk of both antennas per step"},
           "e2e": {"value": value, "unit": "spectra/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    global CUT
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference", "plain-gpu"])
    ap.add_argument("--cut", type=int, default=CUT,
                    help="stream: IPFB cut (default 10, the reference's; 80 gives a 7-smooth nslice)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline sample")
    ap.add_argument("--no-check", action="store_true", help="skip the parity check against the FP64 oracle")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain-GPU comparator leg")
    ap.add_argument("--chunks", type=int, default=None,
                    help="stream only this many 2^15-spectrum chunks (smaller case for profiling; "
                         "every launch keeps its full size)")
    ap.add_argument("--nant", type=int, default=None, help="antennas (profiling case; default 2)")
    ap.add_argument("--workload", default="stream",
                    choices=["stream", "uneven-batch", "unpack-xcorr", "coarse-xcorr", "ipfb-pfb"],
                    help="stream: the 2-antenna 2^20-spectrum chain (default); uneven-batch: 24 mixed files; "
                         "unpack-xcorr: 2 ant x 64 ch x 2^17 spectra, 2^14-spectrum averages; coarse-xcorr: "
                         "16 ant x 256 ch x 2^18 spectra all baselines; ipfb-pfb: one-input rechannelisation")
    ap.add_argument("--lanes", type=int, default=4, help="uneven-batch: concurrent CUDA streams")
    ap.add_argument("--time-filter", default="default", choices=["default", "iir", "fir", "fft"],
                    help="stream: IPFB time stage form (default: the library's choice)")
    ap.add_argument("--row-tile", type=int, default=0, help="stream: IIR / FIR row tile (16, 32 or 64)")
    ap.add_argument("--row-ffts", type=int, default=0, help="stream: spectra per row-stage CTA (8, 4 or 2)")
    ap.add_argument("--pfb-tma", type=int, default=-1,
                    help="stream: PFB band DFT tile fetch: 0 plain loads (default), 1 TMA into the FFT buffers, "
                         "2 persistent CTAs with TMA prefetch")
    ap.add_argument("--row-prefetch", type=int, default=-1,
                    help="stream: row stage 0 = one CTA per tile, 1 = persistent prefetching, "
                         "2 (default) = + shared twiddles")
    ap.add_argument("--check", action="store_true", help="uneven-batch: job-0 error of every file vs the FP64 oracle")
    ap.add_argument("--row-tc", type=int, default=-1,
                    help="stream: row stage on the tensor cores (1, library default) or the FFT (0)")
    ap.add_argument("--coarse-tma", type=int, default=-1,
                    help="coarse workloads: tcgen05 packet staging, 1 TMA (library default), 0 register loads")
    ap.add_argument("--mma-bits", type=int, default=0, help="coarse workloads: tensor-core operand bits (16 or 8)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    CUT = args.cut
    if args.impl == "reference":
        run_reference(args)
    elif args.impl == "plain-gpu":
        run_plain(args)
    elif args.workload == "uneven-batch":
        run_batch(args)
    elif args.workload == "unpack-xcorr":
        run_coarse(args, 2, 64, 1 << 17, 1 << 14,
                   "plain unpack + xcorr: 2 ant x 2 pol 4-bit, 64 ch, 2^17 spectra, averages over 2^14 spectra")
        run_coarse(args, 2, 64, 1 << 24, 1 << 14,
                   "plain unpack + xcorr, bandwidth sweep size: 2 ant x 2 pol 4-bit, 64 ch, 2^24 spectra")
    elif args.workload == "coarse-xcorr":
        run_coarse(args, 16, 256, 1 << 18, None,
                   "many-antenna coarse correlator: 16 ant x 2 pol 4-bit, 256 ch, 2^18 spectra, all 528 pairs")
    elif args.workload == "ipfb-pfb":
        run_ipfb_pfb(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
