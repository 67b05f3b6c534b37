#!/usr/bin/env python3
"""Coupling benchmark: IBM coupling cells/s of SolidCloud::interact on one GB300 (and N replicas).

Workload (default): 512^3 uniform hex mesh on [0,1]^3, 16384 spheres / ellipsoids / boxes (lognormal radius,
median 0.004), FP32 fields resident in HBM (seeded synthetic data).  One step = one interact: sparse reset,
enumeration of every solid's touched cells, solid fraction, direct forcing and force/torque reduction.
value = sum over solids of |touched cells| / device time of the step (CUDA events, L2 flushed between steps).
e2e = the same metric through the host-buffer entry point with FP64 fields in OpenFOAM's layout (U read in, As/Fs/Ts/Ct
and force/torque written out), timed over every step.  refgeo_gpu: the reference's own fraction on the GPU, beside the CPU reference arm.

The default method is the learned cut-cell fraction (network + SUBSAMPLE(16^3) fallback outside its band).  The
same run times the plain SUBSAMPLE(10^3) path ("plain") and measures the learned As and per-solid force against a
SUBSAMPLE(16^3) step ("accuracy"; that evaluator's classifications equal the FP64 oracle's).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--config poly3d_512] [--method learned|subsample|refgeo]
  python bench.py --impl reference ...   the CPU restatement of the reference's coupling (its data structures
                                          and REF-GEO fraction), on a bounded sample of the solids spread over
                                          every host thread
With N > 1 (torchrun) every rank runs an independent replica: the path has no exchange step on one mesh per GPU
(replicas only), value = sum over ranks, time = max over ranks.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PEAKS_FALLBACK = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}
# algorithmic bytes per unit (one coupling cell = one (solid, touched cell) pair):
#   U read 12 + As 4 + Fs 12 + Ts 4 + Ct 4 written = 36 B per coupling cell for the whole coupling; per kernel:
ALG_BYTES = {
    "couple_chunks_kernel": ("coupling_cells", 32.0),  # U read 12, As/Ts/Fs written 20
    "claim_kernel": ("coupling_cells", 4.0),       # Ct written
    "finalize_kernel": ("coupling_cells", 8.0),    # Ct and As rewritten for the cells that need it
    "reset_kernel": ("coupling_cells", 24.0),      # previous cells zeroed
    "classify_kernel": ("bbox_cells", 1.0),        # one class byte per bbox cell (+ the cut-cell outputs below)
    "connect_kernel": ("bbox_cells", 1.0),         # class bytes read once
    "mlp_infer_kernel": ("network_cells", 80.0),   # 16 inputs + prior + destination read, fraction written
    "subsample_cells_kernel": ("sampled_cells", 16.0),  # list entry and destination read, fraction written
}
# DRAM bytes per unit measured by ncu (dram__bytes_read.sum + dram__bytes_write.sum of one launch / its units) on the
# 256^3 / 2048-solid learned workload (the full-size workload's distribution at half scale per axis);
# profiles/<kernel>_poly3d_256_learned.md and profiles/launches_poly3d_256_learned.md record the captures
NCU_BYTES_PER_UNIT = {
    "couple_chunks_kernel": 121.3,  # 161.6 MB for 1,332,670 coupling cells: whole 32-byte sectors of the marked chunks
    "classify_kernel": 0.84,        # 3.6 MB for 4,282,843 bbox cells left after the box test
    "subsample_cells_kernel": 52.5,  # 8.1 MB for 154,364 sampled cells
    "learned_stencil_kernel": 11.8,  # 9.0 MB for 760,774 listed cut cells
}
# Warp instructions per unit (ncu smsp__inst_executed.sum of one launch / its units), per (kernel, method); the
# stencil, sampling and classification kernels are bound by instruction issue, and these counts give their issue
# roofline
INST_PER_UNIT = {
    ("learned_stencil_kernel", "learned"): ("learned_cells", 373.0),  # 283.8 M for 760,774 listed cut cells
    ("subsample_cells_kernel", "learned"): ("sampled_cells", 1716.3),  # 264.9 M for 154,364 16^3 cells
    ("classify_kernel", "learned"): ("bbox_cells", 31.08),            # 133.1 M for 4,282,843 bbox cells
    ("classify_kernel", "refgeo"): ("bbox_cells", 37.82),             # 162.0 M for the same bbox cells
}
# FLOPs of the two tensor-core layers per predicted cell: hi and lo BF16 halves of a 16x64 and a 64x64 product
MLP_FLOPS_PER_CELL = 2 * (2 * 16 * 64) + 2 * (2 * 64 * 64)
METHODS = {"refgeo": 0, "subsample": 1, "learned": 2}


def over_ranks(dist, ms_step, cells, device):
    """(max of ms_step, sum of cells) over the ranks of the default process group; unchanged without one.  Each rank
    runs its own replica of the workload, so the job's time is the slowest rank's and its work the sum."""
    if dist is None:
        return ms_step, cells
    import torch
    t = torch.tensor([ms_step], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    c = torch.tensor([cells], dtype=torch.float64, device=device)
    dist.all_reduce(c, op=dist.ReduceOp.SUM)
    return float(t.item()), float(c.item())


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return d, "measured"
    except Exception:
        return PEAKS_FALLBACK, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while the timed region runs."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.FIELDS,
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
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def make_workload(args, lower=None):
    """The workload of --config at --scale with the fraction method of --method.  lower: the solid construction
    (default: the library's host lowering; the CPU reference leg passes the oracle's restatement)."""
    from sdfibm_gb300 import workloads
    w = workloads.CONFIGS[args.config](scale=args.scale, lower=lower)
    w.opt.fraction_method = METHODS[args.method]
    w.opt.exact_forcing = 1 if getattr(args, "exact_forcing", False) else 0
    if args.method == "learned":
        from sdfibm_gb300 import learned
        w.opt.learned_fallback_n = int(learned.load_model()[3].get("band", {}).get("fallback_n", 16))
    elif args.method == "subsample":
        w.opt.subsample_n = args.subsample_n
    return w


def workload_config(w):
    """The `config` of both arms' lines: the workload alone (mesh, solids, fields), identical for the GPU arm and the
    CPU reference arm."""
    kinds = sorted({abi_shape_name(d.shape.type) for d in w.solids})
    return {"workload": "%s: %dx%dx%d uniform hex mesh, %d solids (%s), FP32 velocity field, seeded synthetic"
                        % (w.name, w.mesh.nx, w.mesh.ny, w.mesh.nz, len(w.solids), "/".join(kinds)),
            "n_cells": w.ncells, "n_solids": len(w.solids),
            "l2": "GPU arm: flushed (256 MB write) before every timed step; CPU arm: inputs far above its caches"}


def abi_shape_name(t):
    from sdfibm_gb300 import abi
    return {v: k for k, v in abi.SHAPE_NAMES.items()}.get(int(t), str(t))


def make_cloud(w, method, subsample_n=None, stream=None, timing=False, band=None, params=None):
    """A coupling context of workload w with the given fraction method (the learned model loaded if needed: its
    shipped band, or band = (tau_refine, rho_min); its parameters, or `params`).  With a stream the context replays
    CUDA graphs of its steps; with timing it records per-kernel events instead."""
    import copy

    from sdfibm_gb300 import abi, learned
    from sdfibm_gb300.cloud import SolidCloud
    opt = copy.copy(w.opt)
    opt.fraction_method = METHODS[method]
    if subsample_n:
        opt.subsample_n = subsample_n
    opt.timing = 1 if timing else 0
    opt.graphs = 0 if timing else 1
    cloud = SolidCloud(w.mesh, w.solids, opt, stream=stream)
    if method == "learned":
        p, tau, rho, meta = learned.load_model()
        if band is not None:
            tau, rho = band
        cloud.set_fraction_model(p if params is None else params, tau, rho)
    return cloud


def time_steps(torch, cloud, w, U, f, steps, warmup, flush, stream=None, kernel_times=False):
    """warmup + steps interacts on `stream`; device time per step (CUDA events on that stream around each step, L2
    flushed before it by a 256 MB write on the same stream)."""
    stream = stream or torch.cuda.current_stream()
    with torch.cuda.stream(stream):
        for i in range(warmup):
            cloud.interact(i * w.dt, w.dt, U, f, want_ft=False)
        stream.synchronize()
        ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        cells, bbox, kt, launches, st = [], [], {}, 0, {}
        for i in range(steps):
            flush.fill_(float(i))
            ev0[i].record(stream)
            cloud.interact((warmup + i) * w.dt, w.dt, U, f, want_ft=False)
            ev1[i].record(stream)
            st = cloud.stats()  # synchronises
            cells.append(st["coupling_cells"])
            bbox.append(st["bbox_cells"])
            launches += st["launches"]
            if kernel_times:
                for k, v in cloud.kernel_times().items():
                    kt.setdefault(k, []).append(v)
        stream.synchronize()
    ms = [a.elapsed_time(b) for a, b in zip(ev0, ev1)]
    return dict(ms_step=sum(ms) / len(ms), cells=sum(cells) / len(cells), bbox=sum(bbox) / len(bbox),
                launches=launches, kernel_ms={k: sum(v) / len(v) for k, v in kt.items()}, stats=st)


def reference16(w, U, n=16):
    """Fields and forces of one SUBSAMPLE(n^3) step (its classifications equal the FP64 oracle's)."""
    import copy
    if n > 16:  # about 3 undecided points per 32^3 cell: a recheck list that holds them
        w = copy.copy(w)
        w.opt = copy.copy(w.opt)
        w.opt.recheck_cap = 1 << 26
    ref = make_cloud(w, "subsample", subsample_n=n)
    fr = ref.new_fields()
    FTr = ref.interact(0.0, w.dt, U, fr)
    ref.close()
    return fr, FTr


def converged(torch, w, U, methods):
    """As and per-solid force of each method against a SUBSAMPLE 32^3 step (32768 samples per cut cell)."""
    ref = reference16(w, U, n=32)
    out = {}
    for name, m in methods.items():
        if isinstance(m, tuple):
            c = make_cloud(w, m[0], subsample_n=m[1])
            a = accuracy(torch, w, c, U, ref, reference="SUBSAMPLE 32^3 (32768 samples), same step")
            c.close()
        else:
            a = accuracy(torch, w, m, U, ref, reference="SUBSAMPLE 32^3 (32768 samples), same step")
        out[name] = {k: v for k, v in a.items() if k.startswith("as_") or k.startswith("force_")}
    return out


def accuracy(torch, w, cloud, U, ref, reference="SUBSAMPLE 16^3 (4096 samples), same step"):
    """As and per-solid force of one step of `cloud` against the reference step `ref` (learned.accuracy)."""
    from sdfibm_gb300 import learned
    fr, FTr = ref
    fl = cloud.new_fields()
    torch.cuda.synchronize()  # the fields are zeroed on torch's stream; the context may run on another
    FTl = cloud.interact(0.0, w.dt, U, fl)
    return learned.accuracy(torch, w, fl, FTl, fr, FTr, U, reference=reference)


class CpuReference:
    """The oracle with the reference's data structures and its REF-GEO fraction (the reference's own algorithm for
    this path) on a bounded sample of the workload's solids, the solid loop spread over all host threads (solid i
    on thread i % threads)."""

    def __init__(self, w, solids_per_thread, threads=None):
        import copy

        import numpy as np

        from oracle.oracle import OracleCloud
        self.w = w
        self.threads = threads or os.cpu_count() or 1
        S = len(w.solids)
        rng = np.random.default_rng(123)
        take = sorted(rng.choice(S, size=min(S, solids_per_thread * self.threads), replace=False).tolist())
        sample = []
        for new_id, s in enumerate(take):
            d = type(w.solids[s]).from_buffer_copy(w.solids[s])
            d.id = new_id
            sample.append(d)
        self.nsample, self.S = len(sample), S
        opt = copy.copy(w.opt)
        opt.fraction_method = 0  # REF-GEO
        self.U = w.U_numpy().astype(np.float64).reshape(-1)
        self.oc = OracleCloud(w.mesh, sample, opt, faithful=True)
        self.f = self.oc.new_fields()

    def step(self):
        """One interact; returns (coupling cells, seconds of the timed span, wall seconds)."""
        t0 = time.perf_counter()
        self.oc.interact_threads(self.w.dt, self.U, self.f, self.threads)
        wall = time.perf_counter() - t0
        cells = sum(len(self.oc.touched(i)[0]) for i in range(self.nsample))
        return cells, self.oc.last_seconds(), wall

    def describe(self, value, cells, loop, wall):
        w = self.w
        return {"value": value, "unit": "cells/s", "cores": self.threads, "kind": "port",
                "sample": "%d of %d solids (random, seed 123) on the full %dx%dx%d mesh, interact with the "
                          "reference's data structures (per-solid O(N) cell-type array, std::set, unordered_map "
                          "phi cache, full-mesh nearest-cell search) and its REF-GEO fraction, solids spread over "
                          "%d threads; timed span = solid loop + checkAlpha as solidcloud.cpp:443-451; %d coupling "
                          "cells per step, %.2f s (interact wall %.2f s)"
                          % (self.nsample, self.S, w.mesh.nx, w.mesh.ny, w.mesh.nz, self.threads, cells, loop, wall)}


def cpu_baseline(w, solids_per_thread, threads=None):
    ref = CpuReference(w, solids_per_thread, threads)
    cells, loop, wall = ref.step()
    return ref.describe(cells / loop if loop > 0 else None, cells, loop, wall)


def run_reference(args, rank, world):
    """The CPU reference arm: the oracle's restatement of the reference's own coupling (its data structures and its
    REF-GEO fraction, the only fraction the reference has) on the workload built by the oracle's own lowering, so
    that this process maps no library of the product.  Rank 0 alone runs it."""
    if rank != 0:
        return
    from oracle.oracle import Lowering
    a = argparse.Namespace(**vars(args))
    a.method = "refgeo"
    w = make_workload(a, lower=Lowering)
    ref = CpuReference(w, args.cpu_solids)
    vals = []
    last = None
    for i in range(args.warmup + args.steps):
        cells, loop, wall = ref.step()
        last = (cells, loop, wall)
        if i >= args.warmup:
            vals.append(cells / loop)
    v = sum(vals) / len(vals)
    line = {"impl": "reference", "metric": "IBM coupling cells/s", "value": v, "unit": "cells/s", "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": last[1] * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "method": "refgeo (GeometricTools::calcCellVolume, the reference's only cut-cell fraction)",
            "config": workload_config(w),
            "cpu_baseline": ref.describe(v, *last),
            "e2e": {"value": v, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def issue_peak(clocks, sms):
    """Warp instructions per second the GPU can issue: 4 per cycle per SM (one per sub-partition) at the median SM
    clock sampled during the timed region (the maximum clock when no sample was taken)."""
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0
    return 4.0 * sms * mhz * 1e6


def kernel_rooflines(kmean, units, method, peaks, clocks, sms):
    """Roofline entries of the step's kernels, each against the limit that bounds it: warp-instruction issue for the
    stencil, sampling and classification kernels (INST_PER_UNIT, from ncu), HBM for the coupling kernel, the tensor
    cores for the network.  achieved = work per launch (per-unit figure x units) / average launch time."""
    out = {}
    ip = issue_peak(clocks, sms) / 1e9
    for k, t in kmean.items():
        key = (k, method)
        if key in INST_PER_UNIT and t > 0:
            unit, per = INST_PER_UNIT[key]
            a = per * units[unit] / (t * 1e-3) / 1e9
            out[k] = {"bound": "issue", "achieved": a, "peak": ip, "unit": "G warp-instructions/s", "frac": a / ip,
                      "per_unit": per, "unit_of_work": unit, "units": units[unit], "ms": t,
                      "traffic": NCU_BYTES_PER_UNIT.get(k, 0.0) * units[unit] if k in NCU_BYTES_PER_UNIT else None}
    k = "couple_chunks_kernel"
    if kmean.get(k, 0) > 0:
        a = ALG_BYTES[k][1] * units["coupling_cells"] / (kmean[k] * 1e-3) / 1e9
        out[k] = {"bound": "hbm", "achieved": a, "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": a / peaks["hbm_gbs"],
                  "ms": kmean[k], "traffic": NCU_BYTES_PER_UNIT[k] * units["coupling_cells"]
                  if k in NCU_BYTES_PER_UNIT else None}
    if kmean.get("mlp_infer_kernel", 0) > 0 and units["network_cells"]:
        tf = MLP_FLOPS_PER_CELL * units["network_cells"] / (kmean["mlp_infer_kernel"] * 1e-3) / 1e12
        out["mlp_infer_kernel"] = {"bound": "tensor", "achieved": tf, "peak": peaks["bf16_tflops"],
                                   "unit": "TFLOP/s", "frac": tf / peaks["bf16_tflops"],
                                   "ms": kmean["mlp_infer_kernel"]}
    return out


def e2e_host(torch, cloud, w, steps, cells):
    """The step through the host-buffer entry point with page-locked FP32 host fields, timed over `steps` calls
    after two untimed ones (wall clock around each call: the U upload, the kernels, the write-back of the changed
    cells and the force/torque download)."""
    import numpy as np
    N = w.ncells
    Uh = torch.from_numpy(w.U_numpy()).pin_memory()
    hf = {"As": torch.empty(N, dtype=torch.float32, pin_memory=True),
          "Fs": torch.empty(3 * N, dtype=torch.float32, pin_memory=True),
          "Ts": torch.empty(N, dtype=torch.float32, pin_memory=True),
          "Ct": torch.empty(N, dtype=torch.int32, pin_memory=True)}
    hn = {k: v.numpy() for k, v in hf.items()}
    Uhn = Uh.numpy()
    for i in range(2):
        cloud.interact_host(0.0, w.dt, Uhn, hn)
    h2d = d2h = 0
    ts = []
    st = None
    for i in range(steps):
        t0 = time.perf_counter()
        cloud.interact_host(i * w.dt, w.dt, Uhn, hn)
        ts.append(time.perf_counter() - t0)
        st = cloud.stats()  # outside the timed span
        h2d += st["host_h2d_bytes"]
        d2h += st["host_d2h_bytes"]
    s = sum(ts) / len(ts)
    return {"value": cells / s, "unit": "cells/s", "h2d_bytes_per_step": h2d // steps,
            "d2h_bytes_per_step": d2h // steps, "ms_per_step": s * 1e3, "steps": steps,
            "ms_min_max": [min(ts) * 1e3, max(ts) * 1e3],
            "host_fields": ("page-locked FP32; U read in place at the coupling cells" if h2d // steps < 12 * N else
                            "page-locked FP32; U copied in while the fraction kernels run") +
                           (", changed 8-cell chunks written back in place" if st["host_sparse"]
                            else ", whole fields copied back")}


def e2e_host64(torch, cloud, w, steps, cells):
    """The step through sdfibm_cuda_interact_host64: FP64 host fields in OpenFOAM's own layout (U and Fs one x,y,z
    triple per cell, As / Ts / Ct one double per cell), page-locked as a solver would register its field storage,
    timed over `steps` calls after two untimed ones.  This is the drop-in's host cost: the solver passes its fields as
    they are, with no conversion loop on the host."""
    import numpy as np
    N = w.ncells
    U64 = torch.from_numpy(np.ascontiguousarray(w.U_numpy().T, dtype=np.float64)).pin_memory()
    hf = {"As": torch.empty(N, dtype=torch.float64, pin_memory=True),
          "Fs": torch.empty((N, 3), dtype=torch.float64, pin_memory=True),
          "Ts": torch.empty(N, dtype=torch.float64, pin_memory=True),
          "Ct": torch.empty(N, dtype=torch.float64, pin_memory=True)}
    hn = {k: v.numpy() for k, v in hf.items()}
    Un = U64.numpy()
    for i in range(2):
        cloud.interact_host64(0.0, w.dt, Un, hn)
    h2d = d2h = 0
    ts = []
    st = None
    for i in range(steps):
        t0 = time.perf_counter()
        cloud.interact_host64(i * w.dt, w.dt, Un, hn)
        ts.append(time.perf_counter() - t0)
        st = cloud.stats()  # outside the timed span
        h2d += st["host_h2d_bytes"]
        d2h += st["host_d2h_bytes"]
    s = sum(ts) / len(ts)
    return {"value": cells / s, "unit": "cells/s", "h2d_bytes_per_step": h2d // steps,
            "d2h_bytes_per_step": d2h // steps, "ms_per_step": s * 1e3, "steps": steps,
            "ms_min_max": [min(ts) * 1e3, max(ts) * 1e3],
            "host_fields": "page-locked FP64 in OpenFOAM's layout (volVectorField U/Fs, volScalarField As/Ts/Ct); "
                           "U read at the coupling cells, " +
                           ("changed 8-cell chunks written back in place" if st["host_sparse"]
                            else "whole fields written back")}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="poly3d_512")
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--method", default="learned", choices=sorted(METHODS))
    ap.add_argument("--no-compare", action="store_true",
                    help="skip the plain SUBSAMPLE and REF-GEO timings and the accuracy steps")
    ap.add_argument("--subsample-n", type=int, default=10, help="samples per axis of --method subsample")
    ap.add_argument("--cpu-solids", type=int, default=2, help="solids per host thread in the CPU timing sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="default launch configuration (no autotuner)")
    ap.add_argument("--exact-forcing", action="store_true",
                    help="the reference's FP64 forcing sequence per cell (default: FP64 for the rigid-body "
                         "velocity and U - us, FP32 after it, FP64 force/torque sums)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    w = make_workload(args)
    U = w.U_torch()
    stream = torch.cuda.Stream()
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    cloud = make_cloud(w, args.method, stream=stream)
    with torch.cuda.stream(stream):
        f = cloud.new_fields()
        flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > 129 MB L2
    torch.cuda.synchronize()
    # launch configuration from the project's autotuner (per-kernel CTA counts, classify work-item size), before any
    # timed work; contexts of the same shape below take it from its cache
    tuning = None
    if not args.no_autotune:
        cloud.autotune(w.dt, U, f)
        tuning = cloud.tuning()

    def step(t):
        return cloud.interact(t, w.dt, U, f, want_ft=False)

    with torch.cuda.stream(stream):
        for i in range(args.warmup):
            step(i * w.dt)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    tm = time_steps(torch, cloud, w, U, f, args.steps, 0, flush, stream=stream)
    clk = clocks.stop()
    # per-kernel device times from a second context that records events around every launch (no graphs)
    ct = make_cloud(w, args.method, timing=True)
    ft_ = ct.new_fields()
    if not args.no_autotune:
        ct.autotune(w.dt, U, ft_)
    tk = time_steps(torch, ct, w, U, ft_, min(args.steps, 3), 2, flush, kernel_times=True)
    ct.close()
    del ft_
    ms_step = tm["ms_step"]
    mean_cells = tm["cells"]
    ms_step, job_cells = over_ranks(dist, ms_step, mean_cells, "cuda")
    value = job_cells / (ms_step * 1e-3)
    launches = tm["launches"]
    st = tm["stats"]
    kmean = tk["kernel_ms"]
    units = {"coupling_cells": mean_cells, "bbox_cells": tm["bbox"],
             "learned_cells": st.get("learned_cells", 0) if args.method == "learned" else 0,
             "sampled_cells": st.get("learned_fallback_cells", 0) if args.method == "learned"
             else (st.get("learned_cells", 0) if args.method == "subsample" else 0),
             "cut_cells": st.get("learned_cells", 0),
             # the cells the network predicts (the stencil kernel compacts the in-band cells for it)
             "network_cells": (st.get("learned_cells", 0) - st.get("learned_fallback_cells", 0))
             if args.method == "learned" else 0}

    compare = None
    refgeo = None
    if not args.no_compare:
        # the reference's own fraction (REF-GEO) on the GPU, same workload: the like-for-like figure beside the CPU
        # reference arm
        rg = make_cloud(w, "refgeo", stream=stream)
        with torch.cuda.stream(stream):
            fr_ = rg.new_fields()
        torch.cuda.synchronize()
        if not args.no_autotune:
            rg.autotune(w.dt, U, fr_)
        trg = time_steps(torch, rg, w, U, fr_, args.steps, args.warmup, flush, stream=stream)
        rgt = make_cloud(w, "refgeo", timing=True)
        frt = rgt.new_fields()
        if not args.no_autotune:
            rgt.autotune(w.dt, U, frt)
        krg = time_steps(torch, rgt, w, U, frt, min(args.steps, 3), 2, flush, kernel_times=True)["kernel_ms"]
        rgt.close()
        del frt
        refgeo = {"method": "refgeo (the reference's apex/pyramid fraction; As within 1e-5 of the oracle)",
                  "value": trg["cells"] * world / (trg["ms_step"] * 1e-3), "ms_per_step": trg["ms_step"],
                  "tuning": rg.tuning(),
                  "kernel_ms": {k: round(v, 4) for k, v in sorted(krg.items(), key=lambda x: -x[1])}}
        if not args.no_e2e:
            refgeo["e2e"] = e2e_host64(torch, rg, w, args.steps, trg["cells"] * world)
        rg.close()
        del fr_
    if args.method == "learned" and not args.no_compare:
        ref = reference16(w, U)
        plain = make_cloud(w, "subsample", subsample_n=10, stream=stream)
        with torch.cuda.stream(stream):
            fp = plain.new_fields()
        torch.cuda.synchronize()
        if not args.no_autotune:
            plain.autotune(w.dt, U, fp)
        plain_tuning = plain.tuning()
        tp = time_steps(torch, plain, w, U, fp, args.steps, args.warmup, flush, stream=stream)
        acc_plain = accuracy(torch, w, plain, U, ref)
        plain.close()
        del fp
        pt = make_cloud(w, "subsample", subsample_n=10, timing=True)
        fpt = pt.new_fields()
        if not args.no_autotune:
            pt.autotune(w.dt, U, fpt)
        tp["kernel_ms"] = time_steps(torch, pt, w, U, fpt, min(args.steps, 3), 2, flush, kernel_times=True)["kernel_ms"]
        pt.close()
        del fpt
        plain12 = make_cloud(w, "subsample", subsample_n=12, stream=stream)
        with torch.cuda.stream(stream):
            f12 = plain12.new_fields()
        t12 = time_steps(torch, plain12, w, U, f12, args.steps, args.warmup, flush, stream=stream)
        a12 = accuracy(torch, w, plain12, U, ref)
        plain12.close()
        del f12
        # the plain path at the learned path's accuracy: SUBSAMPLE 16^3, the accuracy reference's own lattice (against the
        # converged 32^3 lattice below, learned and plain 16^3 carry the same As and force errors)
        plain16 = make_cloud(w, "subsample", subsample_n=16, stream=stream)
        with torch.cuda.stream(stream):
            f16 = plain16.new_fields()
        torch.cuda.synchronize()
        if not args.no_autotune:
            plain16.autotune(w.dt, U, f16)
        t16 = time_steps(torch, plain16, w, U, f16, args.steps, args.warmup, flush, stream=stream)
        plain16.close()
        del f16
        acc = accuracy(torch, w, cloud, U, ref)
        # other operating points of the same model: the open band, and its prior alone (what the network adds)
        from sdfibm_gb300 import learned
        p_model = learned.load_model()[0]
        p_prior = p_model.copy()
        p_prior[-65:] = 0.0  # network output zero: a = clamp(P4), the 4^3 sub-cell planar reconstruction
        points = []
        for label, band, params in (("open band (network on every cut cell)", (1e30, 0.0), None),
                                    ("prior alone (4^3 sub-cell planar reconstruction, no network), open band",
                                     (1e30, 0.0), p_prior)):
            c2 = make_cloud(w, "learned", stream=stream, band=band, params=params)
            with torch.cuda.stream(stream):
                f2 = c2.new_fields()
            torch.cuda.synchronize()
            if not args.no_autotune:
                c2.autotune(w.dt, U, f2)
            t2 = time_steps(torch, c2, w, U, f2, args.steps, args.warmup, flush, stream=stream)
            a2 = accuracy(torch, w, c2, U, ref)
            points.append(dict({"band": label, "ms_per_step": t2["ms_step"],
                                "value": t2["cells"] * world / (t2["ms_step"] * 1e-3),
                                "fallback_cells": t2["stats"].get("learned_fallback_cells")}, **a2))
            c2.close()
            del f2
        # every method against a converged lattice (SUBSAMPLE 32^3, 32768 samples per cut cell): how close each is
        # to the true solid fraction, beside the contract's 16^3 reference
        conv = converged(torch, w, U, {"learned": cloud, "plain_10": ("subsample", 10),
                                       "plain_12": ("subsample", 12), "plain_16": ("subsample", 16)})
        del ref
        pick = lambda a: {k: v for k, v in a.items() if k.startswith("as_") or k.startswith("force_")}
        compare = {"plain": dict({"method": "SUBSAMPLE 10^3 samples per cut cell", "ms_per_step": tp["ms_step"],
                                  "tuning": plain_tuning,
                                  "value": tp["cells"] * world / (tp["ms_step"] * 1e-3),
                                  "kernel_ms": {k: round(v, 4) for k, v in tp["kernel_ms"].items()}},
                                 **pick(acc_plain)),
                   "speedup_vs_plain": tp["ms_step"] / tm["ms_step"],
                   "plain_12": dict({"method": "SUBSAMPLE 12^3 samples per cut cell", "ms_per_step": t12["ms_step"],
                                     "value": t12["cells"] * world / (t12["ms_step"] * 1e-3)}, **pick(a12)),
                   "speedup_vs_plain_12": t12["ms_step"] / tm["ms_step"],
                   "plain_16": {"method": "SUBSAMPLE 16^3 samples per cut cell (the accuracy reference's lattice)",
                                "ms_per_step": t16["ms_step"], "value": t16["cells"] * world / (t16["ms_step"] * 1e-3)},
                   "speedup_vs_plain_16": t16["ms_step"] / tm["ms_step"],
                   "learned_cells": st.get("learned_cells"), "fallback_cells": st.get("learned_fallback_cells"),
                   "fallback_share": (st.get("learned_fallback_cells") or 0) / max(1, st.get("learned_cells") or 1),
                   "accuracy": acc, "other_operating_points": points,
                   "against_converged_32": conv}

    # full time step (interact + evolve with its sub-steps and collisions + fixInternal), device time, graphs
    with torch.cuda.stream(stream):
        for i in range(2):
            step(i * w.dt)
            cloud.evolve(i * w.dt, w.dt)
            cloud.fix_internal(f["Ct"], U)
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(stream)
        step(2 * w.dt)
        e1.record(stream)
        cloud.evolve(2 * w.dt, w.dt)
        cloud.fix_internal(f["Ct"], U)
        e2.record(stream)
        stream.synchronize()
    full_ms = e0.elapsed_time(e2)
    evolve_ms = e1.elapsed_time(e2)

    # roofline of the dominant kernel (the one with the largest share of the step), against the limit that binds it
    peaks, peaks_kind = load_peaks()
    kr = kernel_rooflines(kmean, units, args.method, peaks, clk, sms)
    dom = max(kmean, key=lambda k: kmean[k])
    roofline = dict(kr.get(dom, {"bound": "hbm", "achieved": None, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                                 "frac": None, "traffic": None}))
    roofline.update({"kernel": dom, "peak_kind": peaks_kind + (" (HBM, bf16)" if peaks_kind == "measured" else ""),
                     "kernels": kr,
                     "note": "issue = warp instructions per second against 4 per cycle per SM at the sampled SM clock "
                             "(per-unit instruction counts from ncu smsp__inst_executed.sum); the stencil, sampling "
                             "and classification kernels are instruction-bound, the coupling kernel HBM/latency-bound, "
                             "the network tensor-core-bound"})

    e2e = None
    if not args.no_e2e:
        e2e = e2e_host64(torch, cloud, w, args.steps, mean_cells * world)
        e2e["fp32_host_fields"] = e2e_host(torch, cloud, w, args.steps, mean_cells * world)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(w, args.cpu_solids)
    if rank == 0:
        line = {"metric": "IBM coupling cells/s", "value": value, "unit": "cells/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32 fields, f64 geometry and reductions",
                "data": "synthetic",
                "method": {"learned": "learned cut-cell fraction (tensor-core network, SUBSAMPLE fallback outside "
                                      "its band)",
                           "subsample": "SUBSAMPLE %d^3" % args.subsample_n,
                           "refgeo": "refgeo (the reference's apex/pyramid fraction)"}[args.method],
                "config": workload_config(w),
                "details": {"coupling_cells": mean_cells, "bbox_cells": tm["bbox"],
                            "fp64_rechecks": st.get("fp64_rechecks"), "learned_cells": units["learned_cells"],
                            "sampled_cells": units["sampled_cells"], "full_step_ms": full_ms,
                            "evolve_fix_ms": evolve_ms, "cuda_graphs": True,
                            "forcing": "FP64" if args.exact_forcing else "mixed FP64/FP32",
                            "parallelism": "replicas" if world > 1 else "single GPU"},
                "kernel_ms": {k: round(v, 4) for k, v in sorted(kmean.items(), key=lambda x: -x[1])},
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
                "gpu_launches": launches, "tuning": tuning, "refgeo_gpu": refgeo, "learned_vs_plain": compare}
        print(json.dumps(line))
    cloud.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
