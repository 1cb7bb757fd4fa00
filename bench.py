#!/usr/bin/env python
"""Rotations/s of the exhaustive FFT correlation scan at 128^3 on GB300.

Workload (default ``shape_ace128``): one seeded synthetic pair, receptor 4000
and ligand 1500 heavy atoms, 128^3 grid at 1.2 A, shape + 18 desolvation
terms (18 folded correlation terms), 9000 uniform rotations scanned in
batches of 64, 4 peaks kept per rotation.  One step = one scan of the whole
rotation set.

Arms
* default: the GPU scan.  ``value`` is device-resident throughput (rotations
  and peaks in HBM, CUDA events on the launching stream); ``e2e`` goes through
  the C ABI with host buffers (``fftdock_scan``: H2D of the rotations, D2H of
  the peaks inside the timed region).
* ``--impl reference``: the reference's CPU path restated by the FP64 oracle
  (one forward + one inverse 3-D FFT per term per rotation, real-space term
  sum, full-grid selection) on every host core, on bounded samples of the
  same workload, in two layouts: one rotation range per single-threaded
  process (the reference's own layout) and one process with threaded FFTs;
  the faster is the arm's value.

Multi-GPU: rotations are independent, every rank scans its own full rotation
set (weak scaling, no collective on the data path).
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

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "rotations/s at 128^3 (1 GB300), exhaustive FFT scan"
UNIT = "rotations/s"


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="shape_ace128")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--n-rot", type=int, default=0, help="scan only this many rotations per step (profiling runs)")
    p.add_argument("--rot-batch", type=int, default=0,
                   help="rotations per pencil/plane launch (default: the workload's, rounded up to 128 by the "
                        "tensor pencil stage)")
    p.add_argument("--pencil", default="auto", choices=["auto", "fft", "tensor"])
    p.add_argument("--precision", default="fp32", choices=["fp32", "bf16"],
                   help="receptor spectra storage (bf16: the precision-study mode)")
    p.add_argument("--cluster", action="store_true",
                   help="translational clustering of each rotation's queue (doClusterTranslations)")
    p.add_argument("--cluster-queue", type=int, default=0,
                   help="queue bound with --cluster (maxNTransInp; default: the reference's maxNTrans * 100)")
    p.add_argument("--cluster-radius", type=float, default=5.0, help="clusterRadiusTrans with --cluster")
    p.add_argument("--n-pairs", type=int, default=0, help="pairs of the pairs256 workload (default 256)")
    p.add_argument("--grid-dims", default="",
                   help="FFT sizes per axis 'nx,ny,nz' instead of the workload's cubic edge (box grids)")
    return p.parse_args()


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def workload(name):
    from proddl2_gb300 import synth
    w = dict(synth.WORKLOADS[name])
    w["name"] = name
    return w


def workload_desc(w, dims=None):
    terms = {"shape_ace": "shape + 18 desolvation types (18 folded terms)", "shape": "shape (1 term)",
             "lj_comp": "the reference's ljComp soft-core LJ (2 terms, weighted ligand entries)",
             "lj_avg": "the reference's ljAvg soft-core LJ (1 term)"}[w["term_set"]]
    grid = ("%d x %d x %d" % tuple(dims)) if dims else ("%d^3" % w["grid_n"])
    return ("%s: receptor %d / ligand %d atoms, %s at %.1f A, %s, %d rotations, %d peaks/rotation"
            % (w["name"], w["n_rec"], w["n_lig"], grid, w["grid_step"], terms, w["n_rot"], w["peaks"]))


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except ValueError:
                continue
            for nm, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def reference_schedule_bytes(n, k, batch):
    """Algorithmic HBM bytes per rotation of the reference FFT schedule:
    each 3-D transform is a plane pass and a line pass over the half spectrum
    M = N^2 (N/2+1) complex; the ligand plane pass writes K M, the line pass
    reads it plus the receptor (shared by `batch` rotations) and writes the
    summed spectrum, the inverse plane pass reads it:
    (2K + 2) M 8 + K M 8 / batch."""
    m = n * n * (n // 2 + 1)
    return (2 * k + 2) * m * 8 + k * m * 8 / batch


FALLBACK_PEAKS = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}


def load_peaks(key):
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d[key]), "measured"
    except Exception:
        return FALLBACK_PEAKS[key], "fallback"


def built_bytes(n, k, n_ent, tensor, batch):
    """Algorithmic HBM bytes per rotation of the pipeline as built (not the
    reference's FFT schedule, which materialises every ligand spectrum):
    pencil stage = receptor operand read once per launch group (tensor form:
    circulant samples [K][N H][N] per 128 rotations; FFT form: spectra
    [K][N][N H] per batch) + the ligand entries + the per-x complex planes it
    writes (N^2 (N/2+1) complex); plane stage = those planes read + the
    per-plane candidate pools (N x 16 value/offset pairs) written."""
    nh = n * (n // 2 + 1)
    plane_bytes = n * nh * 8
    recep = k * nh * n * 8 / (128 if tensor else batch)
    entries = n_ent * 4 * (2 if tensor else 1)
    pencil = recep + entries + plane_bytes
    plane = plane_bytes + n * 16 * 8
    return pencil, plane


# ---------------------------------------------------------------------------
# CPU reference path in the reference's own process layout: one rotation
# range per single-threaded process across the host cores (Makeflow -T local
# over rot-scan tasks, python/lib/PRODDL/dock.py:86-113)
# ---------------------------------------------------------------------------
_CPU_WORKER = None


def _cpu_worker_init(wname):
    global _CPU_WORKER
    from proddl2_gb300 import synth
    w = workload(wname)
    pair = synth.make_pair(w["n_rec"], w["n_lig"], w["n_rot"], seed=1)
    _CPU_WORKER = CpuReference(w, pair, threads=1)


def _cpu_worker_scan(idx):
    t0 = time.perf_counter()
    _CPU_WORKER.rotations(idx)
    return time.perf_counter() - t0


class CpuProcesses:
    """P single-threaded worker processes (spawned, so none inherits a CUDA
    context), each set up with the receptor like a rot-scan process; one
    step = every worker scans its own range of r rotations at the same time."""

    def __init__(self, wname, procs):
        import multiprocessing as mp
        self.procs = procs
        self.pool = mp.get_context("spawn").Pool(procs, initializer=_cpu_worker_init, initargs=(wname,))
        self.next = 0
        self.pool.map(_cpu_worker_scan, [range(0, 0)] * procs, chunksize=1)  # wait for every set-up

    def step(self, r):
        idx = [range(self.next + i * r, self.next + (i + 1) * r) for i in range(self.procs)]
        self.next += self.procs * r
        t0 = time.perf_counter()
        self.pool.map(_cpu_worker_scan, idx, chunksize=1)
        return time.perf_counter() - t0

    def close(self):
        self.pool.terminate()
        self.pool.join()


def cpu_baseline(w, pair, budget_s=20.0):
    """Both CPU layouts of the reference path on this host, bounded samples:
    one range per single-threaded process (the reference's layout) and one
    process whose FFTs use every thread.  Returns (best, both)."""
    cores = os.cpu_count() or 1
    procs = CpuProcesses(w["name"], cores)
    dt = procs.step(1)
    steps = max(1, int(budget_s / 2 / max(dt, 1e-3)))
    t = sum(procs.step(1) for _ in range(steps))
    procs.close()
    proc_rate = cores * steps / t
    ref = CpuReference(w, pair, cores)
    thr_rate, n_s, dt_s = ref.rate(target_s=budget_s / 2)
    layouts = {
        "processes": {"value": proc_rate, "cores": cores,
                      "sample": "%d single-threaded processes x %d rotations (one rotation range each)"
                                % (cores, steps)},
        "threads": {"value": thr_rate, "cores": cores,
                    "sample": "1 process, %d rotations, FFTs on %d threads" % (n_s, cores)},
    }
    best = max(layouts, key=lambda k: layouts[k]["value"])
    return best, layouts, ref.rg.shape[0]


# ---------------------------------------------------------------------------
# CPU reference path (the FP64 oracle, reference schedule)
# ---------------------------------------------------------------------------
class CpuReference:
    def __init__(self, w, pair, threads):
        from oracle import fftdock_oracle as O
        self.O = O
        self.w = w
        self.pair = pair
        self.threads = threads
        self.geom = O.Geometry.centred(w["grid_step"], w["grid_n"])
        if w["term_set"].startswith("lj"):
            from proddl2_gb300 import synth
            ts = O.TERMS_LJ_COMP if w["term_set"] == "lj_comp" else O.TERMS_LJ_AVG
            rl, ll = synth.lj_params(w["n_rec"], 11), synth.lj_params(w["n_lig"], 12)
            lj = O.LjParams(rl[0], rl[1], rl[2], ll[0], ll[1], mix=1, cut=9.0)
            self.rg = O.lj_receptor_terms(self.geom, pair.receptor.xyz, lj, ts)
            self.wts = O.lj_ligand_weights(lj, ts)
        else:
            ts = O.TERMS_SHAPE_ACE if w["term_set"] == "shape_ace" else O.TERMS_SHAPE
            tp = O.TermParams(term_set=ts, ace_matrix=pair.ace)
            # the reference runs one FFTCorrelator per term: shape + each type
            self.rg = O.receptor_terms(self.geom, pair.receptor.xyz, pair.receptor.ace_type, tp, folded=False)
            self.wts = O.ligand_term_weights(pair.ligand.ace_type, tp, folded=False)
        self.rs = O.receptor_spectra(self.rg, workers=threads)
        self.k = w["peaks"]

    def rotations(self, idx):
        for i in idx:
            self.O.scan_rotation(self.geom, self.rg, self.rs, self.pair.ligand.xyz, self.wts,
                                 self.pair.rotations[i % len(self.pair.rotations)], self.k, workers=self.threads)

    def rate(self, target_s=15.0, max_rot=64):
        t0 = time.perf_counter()
        self.rotations([0])
        one = time.perf_counter() - t0
        n = max(2, min(max_rot, int(target_s / max(one, 1e-3))))
        t0 = time.perf_counter()
        self.rotations(range(1, n + 1))
        dt = time.perf_counter() - t0
        return n / dt, n, dt


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from proddl2_gb300 import synth
    w = workload(args.workload)
    cores = os.cpu_count() or 1
    pair = synth.make_pair(w["n_rec"], w["n_lig"], w["n_rot"], seed=1)
    # the reference's layout: one rotation range per single-threaded process
    procs = CpuProcesses(w["name"], cores)
    one = procs.step(1)
    per_proc = max(1, int(3.0 / max(one, 1e-3)))
    for _ in range(args.warmup):
        procs.step(per_proc)
    dt = sum(procs.step(per_proc) for _ in range(args.steps))
    procs.close()
    proc_rate = cores * per_proc * args.steps / dt
    # beside it: one process whose FFTs use every thread (a shorter sample)
    ref = CpuReference(w, pair, cores)
    thr_rate, n_thr, dt_thr = ref.rate(target_s=10.0)
    n_fft = ref.rg.shape[0]
    layouts = {
        "processes": {"value": proc_rate, "cores": cores,
                      "sample": "%d single-threaded processes, %d rotations each per step (one rotation range "
                                "per process, as Makeflow -T local runs rot-scan tasks)" % (cores, per_proc)},
        "threads": {"value": thr_rate, "cores": cores,
                    "sample": "1 process, %d rotations, pocketfft on %d threads" % (n_thr, cores)},
    }
    best = max(layouts, key=lambda k: layouts[k]["value"])
    value = layouts[best]["value"]
    ms_per_step = 1000.0 * dt / args.steps if best == "processes" else 1000.0 * dt_thr / n_thr
    sample = ("%s; %s workload, FP64 oracle, %d FFT terms (reference schedule: forward + inverse 3-D FFT per "
              "term per rotation), scipy pocketfft" % (layouts[best]["sample"], w["name"], n_fft))
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded globules, uniform quaternion rotations)",
        "config": {"workload": workload_desc(w), "mode": "exhaustive",
                   "sample_rotations_per_step": cores * per_proc if best == "processes" else 1},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "layout": best, "sample": sample, "layouts": layouts},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def run_ours(args):
    import numpy as np
    import torch
    import torch.distributed as dist
    from proddl2_gb300 import FFTScan, ScanConfig, synth, _lib

    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    w = workload(args.workload)
    if args.n_rot > 0:
        w["n_rot"] = args.n_rot
    if args.rot_batch > 0:
        w["rot_batch"] = args.rot_batch
    pair = synth.make_pair(w["n_rec"], w["n_lig"], w["n_rot"], seed=1)
    n_rot = w["n_rot"]
    queue = (args.cluster_queue or 100 * w["peaks"]) if args.cluster else 10000
    dims = tuple(int(v) for v in args.grid_dims.split(",")) if args.grid_dims else None
    cfg = ScanConfig(grid_n=w["grid_n"], grid_step=w["grid_step"], term_set=w["term_set"], peaks_per_rot=w["peaks"],
                     rot_batch=w["rot_batch"], ace_matrix=pair.ace, device=local, pencil_mode=args.pencil,
                     precision=args.precision, cluster_trans=args.cluster, max_trans_inp=queue,
                     cluster_radius=args.cluster_radius, grid_dims=dims)
    scan = FFTScan(cfg)
    t0 = time.perf_counter()
    if w["term_set"].startswith("lj"):
        rl, ll = synth.lj_params(w["n_rec"], 11), synth.lj_params(w["n_lig"], 12)
        scan.set_pair_lj(pair.receptor.xyz, rl[0], rl[1], rl[2], pair.ligand.xyz, ll[0], ll[1])
    else:
        scan.set_receptor(pair.receptor.xyz, pair.receptor.ace_type)
    receptor_ms = 1000.0 * (time.perf_counter() - t0)
    if not w["term_set"].startswith("lj"):
        scan.set_ligand(pair.ligand.xyz, pair.ligand.ace_type)

    rot_host = np.ascontiguousarray(pair.rotations.reshape(n_rot, 9))
    d_rot = torch.from_numpy(rot_host).to(dev)
    peak_bytes = _lib.peak_dtype().itemsize
    d_peaks = torch.zeros(n_rot * w["peaks"] * peak_bytes, dtype=torch.uint8, device=dev)
    d_np = torch.zeros(n_rot, dtype=torch.int32, device=dev)
    # a dedicated stream: the library launches on it and the timing events are
    # recorded on it (the legacy default stream would not order against the
    # library's own non-blocking stream)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)

    def step():
        scan.scan_device(d_rot.data_ptr(), n_rot, d_peaks.data_ptr(), d_np.data_ptr(), stream_ptr=stream.cuda_stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)

    gpu_index = int(os.environ.get("CUDA_VISIBLE_DEVICES", str(local)).split(",")[local if world > 1 else 0]) \
        if os.environ.get("CUDA_VISIBLE_DEVICES", "").replace(",", "").isdigit() else local
    sampler = ClockSampler(gpu_index)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize(dev)
    sampler.start()
    scan.profile(True)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize(dev)
    if world > 1:
        dist.barrier()
    clocks = sampler.stop()
    ms_total = ev0.elapsed_time(ev1)
    kstats = scan.kernel_stats()
    scan.profile(False)
    t = torch.tensor([ms_total], dtype=torch.float64, device=dev)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms_total = float(t.item())
    ms_per_step = ms_total / args.steps
    value = n_rot * world / (ms_per_step / 1000.0)

    # end to end through the C ABI with host buffers
    for _ in range(max(1, args.warmup)):
        scan.scan(rot_host)
    torch.cuda.synchronize(dev)
    if world > 1:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        res = scan.scan(rot_host)
    e2e_s = time.perf_counter() - t0
    te = torch.tensor([e2e_s], dtype=torch.float64, device=dev)
    if world > 1:
        dist.all_reduce(te, op=dist.ReduceOp.MAX)
    e2e_s = float(te.item())
    e2e_value = n_rot * world * args.steps / e2e_s
    h2d = rot_host.nbytes
    d2h = res.peaks.nbytes + res.n_peaks.nbytes + 4 * n_rot

    # rooflines from this run's CUDA-event times (per-kernel averages over the
    # timed steps) and the algorithmic figures of the pipeline as built
    info = scan.info()
    launches, pencil_ms = kstats["pencil"]
    plane_launches, plane_ms = kstats["plane"]
    k_terms = info["n_terms"]
    batch = info["rot_batch"]
    avg_launch_ms = pencil_ms / max(launches, 1)
    # one timed stage is one kernel, except the queue + clustering stage:
    # bound, gather, check, 6 x (digit pass + pick), gather, finish
    per_stage = {"finalize": 17 if args.cluster else 1}
    gpu_launches = sum(v[0] * per_stage.get(k, 1) for k, v in kstats.items())
    total_kernel_ms = sum(v[1] for v in kstats.values())
    share = pencil_ms / total_kernel_ms if total_kernel_ms else None
    n = w["grid_n"]
    tensor = info["pencil_path"] == "tensor"
    rot_per_launch = n_rot * args.steps / max(launches, 1)
    pencil_b, plane_b = built_bytes(n, k_terms, info["n_entries"], tensor, batch)
    peak_gbs, gbs_kind = load_peaks("hbm_gbs")
    pencil_gbs = pencil_b * rot_per_launch / (avg_launch_ms / 1000.0) / 1e9
    plane_gbs = plane_b * n_rot * args.steps / max(plane_launches, 1) / (plane_ms / max(plane_launches, 1) / 1000.0) / 1e9
    step_bytes = pencil_b + plane_b
    hbm = {
        "pencil": {"bytes_per_rotation": pencil_b, "achieved": pencil_gbs, "frac": pencil_gbs / peak_gbs},
        "plane": {"bytes_per_rotation": plane_b, "achieved": plane_gbs, "frac": plane_gbs / peak_gbs},
        "whole_step": {"bytes_per_rotation": step_bytes, "achieved": step_bytes * value / 1e9,
                       "frac": step_bytes * value / 1e9 / peak_gbs},
        "peak": peak_gbs, "unit": "GB/s", "peak_source": gbs_kind + " copy bandwidth",
        "basis": "pipeline as built: receptor operand once per launch group + ligand entries + the per-x complex "
                 "planes written by the pencil stage and read by the plane stage + candidate pools; the "
                 "reference's FFT schedule (every ligand spectrum in HBM, %.1f MB per rotation) is that "
                 "schedule's traffic, not a lower bound" % (reference_schedule_bytes(n, k_terms, batch) / 1e6),
    }
    if tensor:
        # executed tcgen05 work per pencil and 128-rotation group: K * W/8
        # chunks of 6 MMAs (real and imaginary output x hi*hi, hi*lo, lo*hi)
        # of 128 x 128 x 16; one of the three split products is the FP32
        # product being emulated
        n_batches = math.ceil(n_rot / batch)
        groups_per_step = sum(math.ceil(min(batch, n_rot - b0) / 128) for b0 in range(0, n_rot, batch))
        nh = n * (n // 2 + 1)
        flops_per_group = nh * k_terms * (info["window_w"] // 8) * 6 * (2.0 * 128 * 128 * 16)
        flops_per_launch = flops_per_group * groups_per_step / n_batches
        executed = flops_per_launch / (avg_launch_ms / 1000.0) / 1e12
        peak, peak_kind = load_peaks("bf16_tflops_sustained")
        roofline = {"bound": "tensor", "achieved": executed, "peak": peak, "unit": "TFLOP/s",
                    "frac": executed / peak, "traffic": None, "kernel": "pencil_tc",
                    "peak_source": peak_kind + " sustained bf16 (the kernel runs inside a seconds-long step)",
                    "useful_achieved": executed / 3.0, "useful_frac": executed / 3.0 / peak,
                    "flops_basis": "executed split-FP16 MMA work: N^2(N/2+1) pencils x K x W/8 chunks x 6 MMAs "
                                   "of 128x128x16 per 128-rotation group (W = %d); useful = executed / 3 (the "
                                   "hi*hi, hi*lo, lo*hi products emulate one FP32 product)" % info["window_w"],
                    "limiter": "the CUDA-core producers of the MMA operands (entry walk, tile conversion "
                               "and build: shared-memory and LSU traffic and its latency); the tensor pipe "
                               "is busy about a third of the time, and halving the MMAs' shared-memory "
                               "operand reads did not change the kernel's time",
                    "kernel_share": share, "hbm": hbm}
    else:
        roofline = {"bound": "hbm", "achieved": pencil_gbs, "peak": peak_gbs, "unit": "GB/s",
                    "frac": pencil_gbs / peak_gbs, "traffic": None, "kernel": "pencil",
                    "peak_source": gbs_kind, "kernel_share": share, "hbm": hbm,
                    "limiter": "FP32 instruction issue (the y/z direct sums and x transforms); HBM traffic is "
                               "the receptor spectra once per batch and the x-planes it writes"}

    if rank != 0:
        scan.close()
        if world > 1:
            dist.destroy_process_group()
        return

    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        best, layouts, n_fft = cpu_baseline(w, pair, budget_s=20.0)
        cpu = {"value": layouts[best]["value"], "unit": UNIT, "cores": layouts[best]["cores"], "kind": "port",
               "layout": best,
               "sample": "%s; FP64 oracle, reference schedule (%d terms, forward + inverse 3-D FFT per term per "
                         "rotation), scipy pocketfft" % (layouts[best]["sample"], n_fft),
               "layouts": layouts}

    metric = METRIC if not dims else "rotations/s on a %d x %d x %d grid (1 GB300), exhaustive FFT scan" % dims
    out = {
        "metric": metric, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic (seeded globules, uniform quaternion rotations)",
        "config": {"workload": workload_desc(w, dims), "rot_batch": batch,
                   "mode": ("exhaustive, translational clustering of a %d-cell queue per rotation (radius %g A)"
                            % (queue, args.cluster_radius)) if args.cluster else "exhaustive",
                   "parallelism": "replicas" if world == 1 else "rotation sets per rank (replicas)",
                   "l2": "inputs larger than L2: %.0f MB receptor spectra + %.0f MB x-planes per batch"
                         % (k_terms * n * n * (n // 2 + 1) * 8 / 1e6, batch * n * n * (n // 2 + 1) * 8 / 1e6),
                   "receptor_setup_ms": receptor_ms,
                   "pencil_stage": info["pencil_path"],
                   "grid_dims": list(scan.grid_dims),
                   "precision": ("split-FP16 tcgen05 GEMM with FP32 accumulation (hi*hi+hi*lo+lo*hi) for the x stage, "
                                 "FP32 FFTs elsewhere" if info["pencil_path"] == "tensor" else "FP32 FFTs")
                                + (", BF16-stored receptor spectra" if args.precision == "bf16" else "")
                                + ", FP64 direct-space rescoring of 16 candidates"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": gpu_launches,
        "kernels_ms_per_step": {k: v[1] / args.steps for k, v in kstats.items()},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "clocks": clocks,
    }
    print(json.dumps(out))
    scan.close()
    if world > 1:
        dist.destroy_process_group()


# ---------------------------------------------------------------------------
# many uneven pairs in one CUDA graph (workload pairs256)
# ---------------------------------------------------------------------------
PAIRS_METRIC = "rotations/s, 256 uneven pairs (grid 48-144^3) scanned from one CUDA graph"


def pairs_workload(args):
    from proddl2_gb300 import synth
    from proddl2_gb300.pairs import PairInput, pair_grid
    w = workload(args.workload)
    n_pairs = args.n_pairs or w["n_pairs"]
    n_rot = args.n_rot or w["n_rot"]
    ace = synth.ace_matrix(18, 1)
    rot = synth.quaternion_rotations(n_rot, seed=2)
    pairs = []
    for rec, lig in synth.uneven_pairs(n_pairs, seed=1):
        pairs.append(PairInput(rec.xyz, lig.xyz, rot, rec.ace_type, lig.ace_type,
                               grid_n=pair_grid(rec.xyz, lig.xyz, w["grid_step"])))
    return w, n_pairs, n_rot, ace, pairs


def pairs_desc(w, n_pairs, n_rot, grids):
    from collections import Counter
    hist = ", ".join("%d^3 x %d" % (n, c) for n, c in sorted(Counter(grids).items()))
    return ("%s: %d pairs, receptors 800-6000 / ligands 300-2000 atoms (log-uniform), grid edge per pair "
            "(%s) at %.1f A, shape + 18 desolvation types, %d rotations per pair, %d peaks/rotation"
            % (w["name"], n_pairs, hist, w["grid_step"], n_rot, w["peaks"]))


def run_pairs(args):
    import torch
    from proddl2_gb300 import FFTScan, ScanConfig
    from proddl2_gb300.pairs import scan_pairs

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    w, n_pairs, n_rot, ace, pairs = pairs_workload(args)
    base = ScanConfig(term_set=w["term_set"], ace_matrix=ace, peaks_per_rot=w["peaks"], rot_batch=w["rot_batch"],
                      device=local)
    # warm-up: the tuned call fixes the plan (streams; per grid edge the
    # rotations per launch and the pencil form)
    t0 = time.perf_counter()
    _, plan = scan_pairs(base, pairs, tune=True)
    tune_call_s = time.perf_counter() - t0
    for _ in range(max(0, args.warmup - 1)):
        scan_pairs(base, pairs, tune=False, plan=plan)
    gpu_index = local
    sampler = ClockSampler(gpu_index)
    sampler.start()
    run_ms, call_s = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        res, rep = scan_pairs(base, pairs, tune=False, plan=plan)
        call_s.append(time.perf_counter() - t0)
        run_ms.append(rep["run_ms"])
    clocks = sampler.stop()
    rot_total = n_pairs * n_rot
    ms_per_step = sum(run_ms) / len(run_ms)
    value = rot_total * world / (ms_per_step / 1000.0)
    e2e_s = sum(call_s) / len(call_s)

    # per-pair sequential launches through the single-pair API (one context per grid edge, made beforehand)
    ctxs = {}
    for p in pairs:
        if p.grid_n not in ctxs:
            ctxs[p.grid_n] = FFTScan(ScanConfig(grid_n=p.grid_n, term_set=w["term_set"], ace_matrix=ace,
                                                peaks_per_rot=w["peaks"], rot_batch=w["rot_batch"], device=local))
    p0 = pairs[0]
    s0 = ctxs[p0.grid_n]
    s0.set_receptor(p0.rec_xyz, p0.rec_type)
    s0.set_ligand(p0.lig_xyz, p0.lig_type)
    s0.scan(p0.rotations)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    seq_n_out = 0
    for p in pairs:
        s = ctxs[p.grid_n]
        s.set_receptor(p.rec_xyz, p.rec_type)
        s.set_ligand(p.lig_xyz, p.lig_type)
        r = s.scan(p.rotations, raise_out_of_grid=False)
        seq_n_out += int((r.n_peaks == 0).sum())
    seq_s = time.perf_counter() - t0
    for s in ctxs.values():
        s.close()
    if rank != 0:
        return
    h2d = sum(p.rec_xyz.nbytes + p.lig_xyz.nbytes + p.rotations.nbytes + p.rec_type.nbytes + p.lig_type.nbytes
              for p in pairs)
    d2h = sum(r.peaks.nbytes + r.n_peaks.nbytes for r in res)
    out = {
        "metric": PAIRS_METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32", "data": "synthetic (seeded globules, uniform quaternion rotations)",
        "config": {"workload": pairs_desc(w, n_pairs, n_rot, [p.grid_n for p in pairs]),
                   "mode": "exhaustive, all pairs in one CUDA graph",
                   "plan": {"streams": plan["n_streams"], "rot_batch_by_grid": plan["rot_batch"],
                            "pencil_form_by_grid": plan["pencil_form"]},
                   "l2": "inputs larger than L2 (per-pair receptor spectra + x-planes rewritten every batch)"},
        "pairs_per_s": n_pairs * world / (ms_per_step / 1000.0),
        "e2e": {"value": rot_total * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "what": "whole fftdock_scan_pairs call: staging, capture, run, copy-out"},
        "tune_call_s": tune_call_s,
        "sequential_per_pair": {"value": rot_total / seq_s, "unit": UNIT, "pairs_per_s": n_pairs / seq_s,
                                "what": "per pair: set_receptor + set_ligand + scan through the single-pair C ABI"},
        "speedup_vs_sequential_e2e": seq_s / e2e_s,
        # per pair: 3 receptor-grid kernels, 6 per receptor term transform, 4 per scan batch
        "gpu_launches": sum(3 + 6 * 18 + 4 * math.ceil(n_rot / plan["rot_batch"][p.grid_n]) for p in pairs),
        "clocks": clocks,
    }
    print(json.dumps(out))


def run_pairs_reference(args):
    rank, _, _ = dist_env()
    if rank != 0:
        return
    from oracle import fftdock_oracle as O
    w, n_pairs, n_rot, ace, pairs = pairs_workload(args)
    threads = os.cpu_count() or 1
    tp = O.TermParams(term_set=O.TERMS_SHAPE_ACE, ace_matrix=ace)
    done, t_total, pi = 0, 0.0, 0
    per_step = 2
    # each step: the reference schedule for a few rotations of the next pair
    for step in range(args.warmup + args.steps):
        p = pairs[pi % len(pairs)]
        pi += 1
        geom = O.Geometry.centred(w["grid_step"], p.grid_n)
        rg = O.receptor_terms(geom, p.rec_xyz, p.rec_type, tp, folded=False)
        rs = O.receptor_spectra(rg, workers=threads)
        wts = O.ligand_term_weights(p.lig_type, tp, folded=False)
        t0 = time.perf_counter()
        for i in range(per_step):
            O.scan_rotation(geom, rg, rs, p.lig_xyz, wts, p.rotations[i], w["peaks"], workers=threads)
        if step >= args.warmup:
            t_total += time.perf_counter() - t0
            done += per_step
    value = done / t_total
    out = {
        "impl": "reference", "metric": PAIRS_METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * t_total / max(1, args.steps),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded globules, uniform quaternion rotations)",
        "config": {"workload": pairs_desc(w, n_pairs, n_rot, [p.grid_n for p in pairs]), "mode": "exhaustive"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "%d rotations of one pair per step (pairs in order), FP64 oracle, 19 FFT terms "
                                   "(reference schedule), scipy pocketfft on %d threads" % (per_step, threads)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


# ---------------------------------------------------------------------------
# precision study (workload precision128): FP32 vs BF16-stored receptor
# spectra on the same rotations
# ---------------------------------------------------------------------------
PRECISION_METRIC = "rotations/s at 128^3, FP32 vs BF16-stored receptor spectra, top-16 rescored in FP64"


def run_precision(args):
    import numpy as np
    import torch
    from proddl2_gb300 import FFTScan, ScanConfig, synth
    from proddl2_gb300.shard import merge_peaks

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    w = workload(args.workload)
    n_rot = args.n_rot or w["n_rot"]
    pair = synth.make_pair(w["n_rec"], w["n_lig"], n_rot, seed=1)
    rot = np.ascontiguousarray(pair.rotations.reshape(n_rot, 9))
    k = w["peaks"]
    sampler = ClockSampler(local)
    sampler.start()
    modes = {}
    for prec in ("fp32", "bf16"):
        cfg = ScanConfig(grid_n=w["grid_n"], grid_step=w["grid_step"], term_set=w["term_set"], peaks_per_rot=k,
                         rot_batch=w["rot_batch"], ace_matrix=pair.ace, device=local, precision=prec)
        with FFTScan(cfg) as s:
            s.set_receptor(pair.receptor.xyz, pair.receptor.ace_type)
            s.set_ligand(pair.ligand.xyz, pair.ligand.ace_type)
            for _ in range(max(1, args.warmup)):
                s.scan(rot[:512])
            t0 = time.perf_counter()
            res = s.scan(rot)
            dt = time.perf_counter() - t0
            vals, offs = s.candidates(rot)
            path = s.info()["pencil_path"]
        # every reported peak is one of the rotation's 16 FP32 candidates,
        # rescored in FP64: compare the two values of the same cell
        n = w["grid_n"]
        cell = res.peaks["cell"].astype(np.int64)
        poff = (cell[..., 0] * n + cell[..., 1]) * n + cell[..., 2]
        score = res.peaks["score"]
        valid = np.arange(k)[None, :] < res.n_peaks[:, None]
        match = poff[:, :, None] == offs[:, None, :]
        assert np.all(match.sum(-1)[valid] == 1)
        v32 = np.where(match, vals[:, None, :], 0.0).sum(-1)
        err = (np.abs(v32 - score) / np.maximum(np.abs(score), 1.0))[valid]
        top = merge_peaks([(0, res.peaks, res.n_peaks)], rot, w["top"])
        modes[prec] = {"rotations_per_s": n_rot / dt, "pencil_stage": path,
                       "max_rel_err": float(err.max()), "median_rel_err": float(np.median(err)),
                       "cells": int(valid.sum()), "top": top}
    clocks = sampler.stop()
    keys = {p: {(tuple(np.round(t["rot"], 12)), tuple(np.round(t["t"], 9))) for t in modes[p]["top"]}
            for p in modes}
    agree = len(keys["fp32"] & keys["bf16"]) / float(w["top"])
    for p in modes:
        del modes[p]["top"]
    if rank != 0:
        return
    out = {
        "metric": PRECISION_METRIC, "value": modes["bf16"]["rotations_per_s"], "unit": UNIT, "n_gpus": world,
        "steps": 1, "warmup": args.warmup, "ms_per_step": 1000.0 * n_rot / modes["bf16"]["rotations_per_s"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32/bf16",
        "data": "synthetic (seeded globules, uniform quaternion rotations)",
        "config": {"workload": workload_desc(w), "mode": "exhaustive, both precisions on the same rotations",
                   "error": "relative error of the FP32-stage value of each reported cell against its FP64 "
                            "direct-space rescoring, max(|E|, 1) scale"},
        "modes": modes,
        "top100_agreement_bf16_vs_fp32": agree,
        "clocks": clocks,
    }
    print(json.dumps(out))


def main():
    args = parse_args()
    pairs_mode = args.workload.startswith("pairs")
    if args.impl == "reference":
        (run_pairs_reference if pairs_mode else run_reference)(args)
    elif args.workload == "precision128":
        run_precision(args)
    else:
        (run_pairs if pairs_mode else run_ours)(args)


if __name__ == "__main__":
    main()
