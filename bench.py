"""Phase-linking benchmark: pixels/s on the 30-SLC 4096x4096 stack (EMI), 1024x1024 blocks.

One step = the per-block hot path of dolphin's wrapped-phase workflow
(workflows/single.py:215-294) over the whole frame: for each 1024x1024 block
read with its (5, 11) halo, amplitude-dispersion PS selection, GLRT SHP
selection (alpha 0.001) on the Rayleigh scale from the PS pass, and
run_phase_linking (EMI, PS filling, CRLB), outputs trimmed to the block.

Prints one JSON line (rank 0).  ``--impl reference`` times the CPU
implementation instead (the numpy restatement of the reference algorithm:
the reference itself needs jax/numba, which this environment lacks), over
bounded crops of the same workload on all host cores.
"""

from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

# ---- workload (config: 30 SLCs, 4096 x 4096, half-window (5, 11), GLRT 0.001, EMI) ----
NSLC = 30
FRAME = 4096
BLOCK = 1024
HALF = (5, 11)
ALPHA = 0.001
PS_THR = 0.25
SEED = 20261205
METRIC = "phase-linked pixels/sec (N=30, EMI) chosen vs plain GPU form at <=1e-3 rad; GB/s"
# DRAM bytes (read + write) of one k_cov_tc launch on a 1034x1046-pixel block of this
# workload, from an ncu capture (dram__bytes_read.sum 612,392,704 + dram__bytes_write.sum
# 3,772,850,944); the planar coherence output (N^2 floats per pixel) is most of it
COV_TC_TRAFFIC = 612_392_704 + 3_772_850_944
# DRAM bytes (read + write) of one k_solve_reg launch on a 1034x1046-pixel block, scaled
# by the pixel count from an ncu capture of the 778x790 block (614,620 pixels:
# dram__bytes.sum.per_second 239.94 GB/s over 10.005 ms = 2.4006 GB, 3,905.8 B per pixel;
# the planar coherence read, N^2 floats per pixel, is most of it)
SOLVE_TRAFFIC = round(2.4006e9 / 614_620 * 1034 * 1046)
UNIT = "pixels/s"


def block_plan(rows, cols, block, half):
    """Block slices with halo, as StridedBlockManager lays them out (io/_blocks.py:242-348).

    Returns tuples (in_rows, in_cols, trim_rows, trim_cols, out_rows, out_cols): the
    halo-padded input slice, the slice of the block result to keep, and where it goes.
    """
    hy, hx = half
    plan = []
    for r0 in range(0, rows, block):
        r1 = min(rows, r0 + block)
        for c0 in range(0, cols, block):
            c1 = min(cols, c0 + block)
            ir0, ir1 = max(0, r0 - hy), min(rows, r1 + hy)
            ic0, ic1 = max(0, c0 - hx), min(cols, c1 + hx)
            plan.append(((ir0, ir1), (ic0, ic1), (r0 - ir0, r1 - ir0), (c0 - ic0, c1 - ic0), (r0, r1), (c0, c1)))
    return plan


# ---------------------------------------------------------------------------------
# CPU side (oracle restatement), run in spawned worker processes
# ---------------------------------------------------------------------------------
def _cpu_crop_worker(args):
    seed, out_rows, out_cols = args
    os.environ["OMP_NUM_THREADS"] = "1"
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    from dolphin_gb300.simulate import StackConfig, make_stack
    from oracle import phase_link as O

    hy, hx = HALF
    cfg = StackConfig(nslc=NSLC, rows=out_rows + 2 * hy, cols=out_cols + 2 * hx, seed=seed, ps_frac=0.03)
    z = make_stack(cfg)
    t0 = time.perf_counter()
    mean, disp, ps = O.calc_ps_block(np.abs(z), PS_THR, NSLC)
    var = (disp * mean) ** 2
    nb = O.estimate_neighbors_glrt(mean, var, HALF, (1, 1), NSLC, ALPHA)
    O.run_phase_linking(z, HALF, ps_mask=ps, neighbor_arrays=nb, avg_mag=mean)
    dt = time.perf_counter() - t0
    return out_rows * out_cols, dt


def cpu_sample(pool, cores, crop=(64, 128), repeats=1):
    """Time the CPU restatement on `cores` crops in parallel; returns (px/s, description)."""
    jobs = [(SEED + 1000 + i, crop[0], crop[1]) for i in range(cores * repeats)]
    t0 = time.perf_counter()
    res = pool.map(_cpu_crop_worker, jobs)
    wall = time.perf_counter() - t0
    px = sum(r[0] for r in res)
    desc = (f"{len(jobs)} crops of {crop[0]}x{crop[1]} output pixels (+halo) of the N=30 workload, "
            f"one process per core, {wall:.1f}s wall")
    return px / wall, desc


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo), for the baseline's record."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.strip().lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for ln in Path("/proc/cpuinfo").read_text().splitlines():
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def run_reference(args, rank, world):
    """The CPU arm: the numpy restatement of the reference algorithm (the reference's own
    path needs jax/numba, which neither machine has) on all host cores, each step a
    bounded sample of the workload (16 crops of 64x128 output pixels plus halo, one
    process per core)."""
    if rank != 0:
        return
    cores = len(os.sched_getaffinity(0))
    ctx = mp.get_context("spawn")
    t_all = time.perf_counter()
    with ctx.Pool(cores) as pool:
        for _ in range(args.warmup):
            cpu_sample(pool, cores, crop=(16, 32))
        vals, walls, descs = [], [], []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            v, d = cpu_sample(pool, cores)
            walls.append(time.perf_counter() - t0)
            vals.append(v)
            descs.append(d)
    wall_total = time.perf_counter() - t_all
    value = float(np.median(vals))
    crops = cores
    px_step = crops * 64 * 128
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1000.0 * float(np.median(walls)),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": f"N={NSLC} {FRAME}x{FRAME} stack, 1024x1024 blocks, half-window {HALF}, GLRT "
                               f"{ALPHA}, EMI, PS {PS_THR} + fill, CRLB; each step a bounded sample on the CPU: "
                               f"{crops} crops of 64x128 output pixels (+halo) = {px_step} pixels",
                   "pixels_per_step": px_step, "crops_per_step": crops,
                   "warmup_sample": f"{crops} crops of 16x32 output pixels per warm-up step",
                   "timed_wall_s": round(float(sum(walls)), 2), "run_wall_s": round(wall_total, 2),
                   "projected_ms_per_frame": 1000.0 * FRAME * FRAME / value,
                   "cpu_model": cpu_model()},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": descs[-1] + " (numpy restatement of the reference algorithm; the "
                                               "reference needs jax/numba, absent here)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _cpu_case_worker(args):
    """One sub-crop of a CPU-table case, timed in its own process."""
    kind, seed, nslc, out_rows, out_cols, half, use_evd, crlb = args
    os.environ["OMP_NUM_THREADS"] = "1"
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    from dolphin_gb300.simulate import StackConfig, make_stack
    from oracle import phase_link as O

    hy, hx = half
    cfg = StackConfig(nslc=nslc, rows=out_rows + 2 * hy, cols=out_cols + 2 * hx, seed=seed,
                      ps_frac=0.03 if nslc == NSLC else 0.05)
    z = make_stack(cfg)
    t0 = time.perf_counter()
    mean, disp, ps = O.calc_ps_block(np.abs(z), PS_THR, nslc)
    if kind == "ps":
        return out_rows * out_cols, time.perf_counter() - t0
    nb = O.estimate_neighbors_glrt(mean, (disp * mean) ** 2, half, (1, 1), nslc, ALPHA)
    O.run_phase_linking(z, half, ps_mask=ps, neighbor_arrays=nb, avg_mag=mean, use_evd=use_evd, compute_crlb=crlb)
    return out_rows * out_cols, time.perf_counter() - t0


def run_cpu_table(args):
    """The CPU baseline table: the numpy restatement on all host cores, median of 3 timed
    runs after one warm-up, for the 512x512 crop of the N=30 workload (EMI and EVD, CRLB on
    and off), the whole N=10 128x128 configuration, and calc_ps_block alone.  Each run
    splits its frame into one sub-crop (with halo) per core, one process each."""
    cores = len(os.sched_getaffinity(0))
    ctx = mp.get_context("spawn")
    side = int(np.sqrt(cores))
    while cores % side:
        side -= 1
    grid = (side, cores // side)
    cases = [("config 2 crop 512x512, EMI, CRLB", "pl", NSLC, 512, HALF, False, True),
             ("config 2 crop 512x512, EMI, no CRLB", "pl", NSLC, 512, HALF, False, False),
             ("config 2 crop 512x512, EVD, CRLB", "pl", NSLC, 512, HALF, True, True),
             ("config 1 128x128 (N=10, hw (5, 5)), EMI, CRLB", "pl", 10, 128, (5, 5), False, True),
             ("calc_ps_block, config 2 crop 512x512", "ps", NSLC, 512, HALF, False, False)]
    rows = []
    with ctx.Pool(cores) as pool:
        for name, kind, nslc, frame, half, evd, crlb in cases:
            sub = (frame // grid[0], frame // grid[1])
            jobs = [(kind, 20261205 + k, nslc, sub[0], sub[1], half, evd, crlb) for k in range(cores)]
            walls = []
            for rep in range(4):  # one warm-up, then three timed
                t0 = time.perf_counter()
                res = pool.map(_cpu_case_worker, jobs)
                w = time.perf_counter() - t0
                if rep:
                    walls.append(w)
            px = sum(r[0] for r in res)
            med = float(np.median(walls))
            rows.append({"run": name, "pixels": px, "median_wall_s": round(med, 3), "pixels_per_s": px / med,
                         "walls_s": [round(w, 3) for w in walls]})
            print(json.dumps(rows[-1]), flush=True)
    print(json.dumps({"impl": "reference", "workload": "cpu-table", "cores": cores, "cpu_model": cpu_model(),
                      "engine": "numpy restatement of the reference algorithm (oracle/phase_link.py), one "
                                "process per core, OMP/OpenBLAS threads 1 per process",
                      "grid": list(grid), "rows": rows}), flush=True)


# ---------------------------------------------------------------------------------
# GPU side
# ---------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in out.strip().splitlines():
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 6:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[2:6]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(values, dist, device=None):
    """Element-wise maximum of per-rank timings (every rank gets the result)."""
    import torch

    vals = torch.tensor(values, dtype=torch.float64, device=device)
    if dist is not None and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(vals, op=dist.ReduceOp.MAX)
    return vals.tolist()


PL_FIELDS = ("cpx_phase", "temp_coh", "shp_counts", "eigenvalues", "estimator", "crlb_std_dev", "closure_phases")


def frame_outputs(torch, frame, device=None, pin=False):
    """Full-frame arrays for every PhaseLinkOutput field (device, or pinned host)."""
    n = NSLC
    spec = {"cpx_phase": ((n, frame, frame), torch.complex64), "temp_coh": ((frame, frame), torch.float32),
            "shp_counts": ((frame, frame), torch.int32), "eigenvalues": ((frame, frame), torch.float32),
            "estimator": ((frame, frame), torch.uint8), "crlb_std_dev": ((n, frame, frame), torch.float32),
            "closure_phases": ((frame, frame, n - 2), torch.float32)}
    if pin:
        return {k: torch.empty(sh, dtype=dt, pin_memory=True) for k, (sh, dt) in spec.items()}
    return {k: torch.empty(sh, dtype=dt, device=device) for k, (sh, dt) in spec.items()}


def gpu_step(stack, plan, dp, outs, covariance_form="tensor", use_evd=False):
    """One pass of the hot path over every block of a device-resident stack; every
    output field of each block, trimmed to the block, goes into the frame arrays."""
    for (ir, ic, tr, tcl, orr, occ) in plan:
        blk = stack[:, ir[0]:ir[1], ic[0]:ic[1]].contiguous()
        mean, disp, ps = dp.calc_ps_block(blk.abs(), PS_THR, NSLC)
        var = (disp * mean) ** 2
        nb = dp.estimate_neighbors(halfwin_rowcol=HALF, alpha=ALPHA, mean=mean, var=var, nslc=NSLC)
        out = dp.run_phase_linking(blk, HALF, ps_mask=ps, neighbor_arrays=nb, avg_mag=mean, compute_crlb=True,
                                   use_evd=use_evd, covariance_form=covariance_form)
        src = (slice(tr[0], tr[1]), slice(tcl[0], tcl[1]))
        dst = (slice(orr[0], orr[1]), slice(occ[0], occ[1]))
        for k in PL_FIELDS:
            lead = (slice(None),) if k in ("cpx_phase", "crlb_std_dev") else ()
            outs[k][lead + dst] = getattr(out, k)[lead + src]


def fp32_peak_tflops(torch, lib, dev):
    """FP32 FMA throughput of this GPU (TFLOP/s), measured with dpl_fp32_fma_probe: 8 CTAs
    of 256 threads per SM, 8 independent FMA chains per thread; best of 5 launches."""
    from dolphin_gb300 import _lib

    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    blocks, iters = sms * 8, 4096
    out = torch.empty(blocks * 256, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    _lib.check(lib.dpl_fp32_fma_probe(out.data_ptr(), blocks, iters, stream), "dpl_fp32_fma_probe")
    best = float("inf")
    for _ in range(5):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        _lib.check(lib.dpl_fp32_fma_probe(out.data_ptr(), blocks, iters, stream), "dpl_fp32_fma_probe")
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return blocks * 256 * 16.0 * iters / (best / 1000.0) / 1e12


def form_rate(torch, stack, plan, dp, outputs, **kw):
    """Output pixels/s of one timed pass over `plan` (after one untimed pass)."""
    gpu_step(stack, plan, dp, outputs, **kw)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    gpu_step(stack, plan, dp, outputs, **kw)
    e1.record()
    torch.cuda.synchronize()
    px = sum((orr[1] - orr[0]) * (occ[1] - occ[0]) for (*_x, orr, occ) in plan)
    return px / (e0.elapsed_time(e1) / 1000.0)


def run_ours(args, rank, world, pool, cores):
    import torch

    import dolphin_gb300 as dp
    from dolphin_gb300 import _lib
    from dolphin_gb300._build import build_library
    from dolphin_gb300.simulate import StackConfig, make_stack_torch

    build_library()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        if dist is not None:
            dist.barrier()

    frame = args.frame
    cfg = StackConfig(nslc=NSLC, rows=frame, cols=frame, seed=SEED + rank, ps_frac=0.03)
    stack = make_stack_torch(cfg, device=dev)
    plan = block_plan(frame, frame, BLOCK, HALF)
    outs = frame_outputs(torch, frame, dev)
    lib = _lib.load()

    for _ in range(args.warmup):
        gpu_step(stack, plan, dp, outs)
    torch.cuda.synchronize()

    # ---- device-resident timed region ----
    sampler = ClockSampler(local)
    sampler.start()
    tot = (_lib.C.c_double * 2)()
    cnt = (_lib.C.c_int64 * 2)()
    lib.dpl_kernel_timing(1, tot, cnt)
    barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    # each block's status words are copied back and checked, at the end of the region,
    # instead of one host synchronisation per block
    with dp.deferred_checks():
        for _ in range(args.steps):
            gpu_step(stack, plan, dp, outs)
        e1.record()
    torch.cuda.synchronize()
    barrier()
    lib.dpl_kernel_timing(0, tot, cnt)
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1) / args.steps
    cov_ms = tot[0] / max(cnt[0], 1)   # per launch (one launch per block)
    sol_ms = tot[1] / max(cnt[1], 1)
    launches_cov = cnt[0] / args.steps

    # ---- the same stack through the plain GPU form (SIMT covariance fused with the
    # solver) and through EVD, on the first two blocks ----
    sub = plan[:2]
    plain_rate = form_rate(torch, stack, sub, dp, outs, covariance_form="simt")
    chosen_rate = form_rate(torch, stack, sub, dp, outs)
    evd_rate = form_rate(torch, stack, sub, dp, outs, use_evd=True)
    accuracy = fp64_check(torch, dp, stack, plan[0])

    # ---- end-to-end: pinned host stack in, every output field out, through the public API ----
    host_stack = torch.empty(stack.shape, dtype=stack.dtype, pin_memory=True)
    host_stack.copy_(stack)
    host_outs = frame_outputs(torch, frame, pin=True)
    del stack
    torch.cuda.empty_cache()
    dstack = torch.empty(host_stack.shape, dtype=host_stack.dtype, device=dev)

    # pipelined: the stack goes up in row bands (each with its halo) on one copy stream,
    # each block row starts as soon as its band has landed, and its results go down on a
    # second copy stream while the next block row computes.  Consecutive steps overlap
    # too: a band of the next step overwrites the device stack once the block rows that
    # read it (its own and its neighbours', through the halo) are done, and a block row
    # rewrites its results once the previous step's copy of them has left.
    comp = torch.cuda.current_stream()
    copy_in, copy_out = torch.cuda.Stream(device=dev), torch.cuda.Stream(device=dev)
    block_rows = sorted({orr for (*_x, orr, _occ) in plan})
    bands = [(max(0, r0 - HALF[0]), min(frame, r1 + HALF[0])) for (r0, r1) in block_rows]
    nbr = len(block_rows)
    comp_done = [None] * nbr  # block row computed (previous step until overwritten)
    out_done = [None] * nbr   # block row's results on the host

    def e2e_step():
        landed = []
        with torch.cuda.stream(copy_in):
            for b, (b0, b1) in enumerate(bands):
                prev = comp_done[min(b + 1, nbr - 1)]
                if prev is not None:
                    copy_in.wait_event(prev)
                for t in range(NSLC):  # contiguous (rows, cols) slabs of pinned memory
                    dstack[t, b0:b1].copy_(host_stack[t, b0:b1], non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(copy_in)
                landed.append(ev)
        for r, ((r0, r1), ev) in enumerate(zip(block_rows, landed)):
            comp.wait_event(ev)
            if out_done[r] is not None:
                comp.wait_event(out_done[r])
            gpu_step(dstack, [e for e in plan if e[4] == (r0, r1)], dp, outs)
            done = torch.cuda.Event()
            done.record(comp)
            comp_done[r] = done
            with torch.cuda.stream(copy_out):
                copy_out.wait_event(done)
                for k in PL_FIELDS:  # every output; contiguous slabs of pinned memory
                    if k in ("cpx_phase", "crlb_std_dev"):
                        for t in range(NSLC):
                            host_outs[k][t, r0:r1].copy_(outs[k][t, r0:r1], non_blocking=True)
                    else:
                        host_outs[k][r0:r1].copy_(outs[k][r0:r1], non_blocking=True)
                od = torch.cuda.Event()
                od.record(copy_out)
                out_done[r] = od

    e2e_step()
    torch.cuda.synchronize()
    barrier()
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    f0.record()
    copy_in.wait_stream(comp)  # no copy of the timed steps starts before f0
    e2e_steps = max(1, args.steps)
    with dp.deferred_checks():
        for _ in range(e2e_steps):
            e2e_step()
        comp.wait_stream(copy_out)  # the region ends when every result is on the host
        f1.record()
    torch.cuda.synchronize()
    barrier()
    e2e_ms = f0.elapsed_time(f1) / e2e_steps
    h2d = sum((b1 - b0) for (b0, b1) in bands) * NSLC * frame * host_stack.element_size()
    d2h = sum(v.numel() * v.element_size() for v in host_outs.values())

    ms, e2e_ms, cov_ms, sol_ms = max_over_ranks([ms, e2e_ms, cov_ms, sol_ms], dist, dev)
    if rank != 0:
        return
    px = frame * frame * world
    value = px / (ms / 1000.0)
    px_per_launch = sum((ir[1] - ir[0]) * (ic[1] - ic[0]) for (ir, ic, *_r) in plan) / len(plan)
    # solver flops per pixel (EMI), the dominant kernel: Cholesky + inverse of |Gamma|
    # (~N^3), complex Cholesky of A - 0.99 I (4N^3/3), ~7 inverse iterations (8N^2 each),
    # CRLB (~2N^3/3)
    f_sol = NSLC**3 * (1.0 + 4.0 / 3.0 + 2.0 / 3.0) + 7 * 8.0 * NSLC**2
    fp32_nominal = 152 * 128 * 2 * 2.07e9 / 1e12
    fp32_peak = fp32_peak_tflops(torch, lib, dev)
    ach_sol = f_sol * px_per_launch / (sol_ms / 1000.0) / 1e12
    # covariance contraction (tensor cores): F_cov = 4 W N (N + 1) per output pixel
    # (Hermitian half, complex MAC = 8 flops)
    W = (2 * HALF[0] + 1) * (2 * HALF[1] + 1)
    f_cov = 4.0 * W * NSLC * (NSLC + 1)
    ach_cov = f_cov * px_per_launch / (cov_ms / 1000.0) / 1e12
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        pass
    bf16_peak = float(peaks.get("bf16_tflops", 1900.0))
    cpu = None
    if pool is not None:
        cv, cd = cpu_sample(pool, cores)
        cpu = {"value": cv, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": cd + " (numpy restatement of the reference algorithm)"}
    # per block: k_ps_block, k_glrt_scale, k_glrt, k_prep, k_cov_tc, k_solve_reg, k_pixel (LU list),
    # k_eigh (pixels that missed the stopping rule), k_post
    launches_per_step = len(plan) * 9
    b_pl = 8 * NSLC + 8 + 2 + 8 * NSLC + 4 + 2 + 4 + 1 + 4 * NSLC + 4 * (NSLC - 2)
    hbm_peak = float(peaks.get("hbm_gbs", 6768.8))
    e2e_rate = px / (e2e_ms / 1000.0)
    line = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": f"N={NSLC} {frame}x{frame} stack per GPU, {BLOCK}x{BLOCK} blocks with halo, "
                               f"half-window {HALF}, GLRT {ALPHA}, EMI, PS {PS_THR} + fill, CRLB",
                   "l2": "inputs larger than L2 (4 GB stack per GPU)",
                   "form": "chosen: tensor-core covariance (bf16 hi/lo, fp32 accumulate) + FP32 solver",
                   "status_checks": "every block's status copied back and checked at the end of the timed "
                                    "region (deferred_checks), no host synchronisation per block",
                   "e2e_copies": "pinned host stack in by row band, all seven PhaseLinkOutput fields out by "
                                 "block row, overlapping compute within and across steps"},
        "e2e": {"value": px / (e2e_ms / 1000.0), "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches_per_step * args.steps),
        "roofline": {"bound": "fp32", "achieved": ach_sol, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": ach_sol / fp32_peak, "traffic": SOLVE_TRAFFIC if frame == FRAME else None,
                     "kernel": "k_solve_reg", "kernel_ms": sol_ms, "launches_per_step": cnt[1] / args.steps,
                     "fp32_nominal_tflops": fp32_nominal,
                     "note": "dominant kernel (FP32 CUDA cores): algorithmic flops ~(3N^3 + 56N^2) per pixel over "
                             "the CUDA-event launch time on its stream; peak = FP32 FMA rate measured on this GPU "
                             "with dpl_fp32_fma_probe (of measured)"},
        "roofline_covariance": {"bound": "tensor", "achieved": ach_cov, "peak": bf16_peak, "unit": "TFLOP/s",
                                "frac": ach_cov / bf16_peak, "traffic": COV_TC_TRAFFIC if frame == FRAME else None,
                                "kernel": "k_cov_tc", "kernel_ms": cov_ms, "launches_per_step": launches_cov,
                                "note": "algorithmic covariance flops 4*W*N*(N+1) per pixel; peak = measured bf16 "
                                        "dense (of measured)"},
        "accuracy_vs_fp64": accuracy,
        # algorithmic bytes per output pixel, B_PL: the stack 8N, mean and variance 8, PS and
        # nodata masks 2, cpx_phase 8N, temp_coh 4, shp_counts 2, eigenvalue 4, estimator 1,
        # CRLB 4N, closure phases 4(N - 2); the PS pass adds 8N + 9
        "achieved_gbs": {"b_pl_bytes_per_pixel": b_pl, "ps_pass_bytes_per_pixel": 8 * NSLC + 9,
                         "value": (b_pl + 8 * NSLC + 9) * value / 1e9,
                         "e2e": (b_pl + 8 * NSLC + 9) * e2e_rate / 1e9, "unit": "GB/s",
                         "hbm_peak": hbm_peak,
                         "note": "B_PL x pixels/s: far below HBM (the path is compute-bound); of measured"},
        "clocks": clocks,
        "forms": {"blocks": len(sub), "unit": UNIT, "chosen": chosen_rate, "plain": plain_rate,
                  "chosen_over_plain": chosen_rate / plain_rate, "evd_chosen": evd_rate,
                  "note": "chosen = tensor-core covariance + register solver; plain = SIMT covariance fused "
                          "with the shared-memory solver; both EMI unless evd"},
    }
    if cpu:
        line["cpu_baseline"] = cpu
    if world == 1 and frame == FRAME and not args.no_extras:
        # the ministack batch (12 stacks, N = 8..45) and the learned warm start's measured
        # bound, after the timed regions, so that one default run reports them too
        del dstack
        torch.cuda.empty_cache()
        for key, fn in (("batch", lambda: batch_measure(2)), ("learned", lambda: learned_measure(FRAME))):
            try:
                r = fn()
            except Exception as exc:  # reported in the line, the headline figures stand
                line[key] = {"error": f"{type(exc).__name__}: {exc}"}
                continue
            if key == "batch":
                line[key] = {"metric": "phase-linked pixels/sec over 12 ministacks of N = 8..45 (1024x1024 each)",
                             "value": r["graph"], "unit": UNIT, "eager": r["eager"],
                             "per_stack_graph": r["per_stack_graph"], "ministack_ms": r["ministack_ms"],
                             "forms": r["forms"], "note": "value: dpl_phase_link_batch (one work-queue "
                             "covariance launch over all stacks) replayed as one CUDA graph"}
            else:
                line[key] = {k: r[k] for k in ("metric", "value", "unit", "plain", "perfect_start",
                                               "iterations_per_pixel", "fallback_rate", "vs_fp64_block0")}
            torch.cuda.empty_cache()
    print(json.dumps(line), flush=True)


def block_inputs(dp, stack, entry):
    """PS and GLRT inputs of one block of the plan (as gpu_step makes them)."""
    ir, ic = entry[0], entry[1]
    blk = stack[:, ir[0]:ir[1], ic[0]:ic[1]].contiguous()
    mean, disp, ps = dp.calc_ps_block(blk.abs(), PS_THR, NSLC)
    nb = dp.estimate_neighbors(halfwin_rowcol=HALF, alpha=ALPHA, mean=mean, var=(disp * mean) ** 2, nslc=NSLC)
    return blk, mean, disp, ps, nb


def compare_to_fp64(torch, out, ref, ps):
    """Errors of a float32 run against the FP64 form on one block: phase (per pixel, the
    worst SLC) and temporal coherence where the FP64 coherence is above 0.3; EMI/EVD
    flips and where they fall."""
    good = ref.temp_coh > 0.3
    d = torch.angle(out.cpx_phase * ref.cpx_phase.conj()).abs().amax(0)
    t = (out.temp_coh - ref.temp_coh).abs()
    flip = out.estimator != ref.estimator
    psm = ps.bool()
    dg = d[good]
    return {"pixels": int(d.numel()), "coherent": int(good.sum()), "phase_max_rad": float(dg.max()),
            "phase_p99_rad": float(torch.quantile(dg[:2**24].float(), 0.99)),
            "above_1e-3_rad": int((dg > 1e-3).sum()), "temp_coh_max": float(t[good].max()),
            "flips": int(flip.sum()), "flips_on_ps": int((flip & psm).sum()),
            "flips_fp64_emi": int((flip & (ref.estimator == 1)).sum()),
            "flips_phase_max_rad": float(d[flip & good].max()) if (flip & good).any() else 0.0}


def fp64_check(torch, dp, stack, entry):
    """The chosen form against the FP64 GPU form (covariance and solver in double) on
    one 1034x1046 block of the workload."""
    blk, mean, _disp, ps, nb = block_inputs(dp, stack, entry)
    kw = dict(ps_mask=ps, neighbor_arrays=nb, avg_mag=mean, compute_crlb=True)
    out = dp.run_phase_linking(blk, HALF, **kw)
    ref = dp.run_phase_linking(blk, HALF, covariance_form="fp64", **kw)
    r = compare_to_fp64(torch, out, ref, ps)
    r["block"] = [list(entry[0]), list(entry[1])]
    return r


def run_precision(args):
    """The precision workload (N=40, 2048x2048, half-window (7, 7), gamma_inf 0.02 and a
    high-coherence disk): rates of the covariance forms (tensor cores with bf16 hi/lo or
    tf32 operands, SIMT), and on a 512x512 crop holding the disk's edge each form's error
    against the FP64 GPU form, like with like (the SIMT form, whose coherence is never
    stored, keeps the last iterate where the iteration misses its stopping rule, and is
    compared with the FP64 form doing the same)."""
    import torch

    import dolphin_gb300 as dp
    from dolphin_gb300._build import build_library
    from dolphin_gb300.simulate import StackConfig, make_stack_torch

    build_library()
    n, frame, half = 40, 2048, (7, 7)
    cfg = StackConfig(nslc=n, rows=frame, cols=frame, seed=20261206, gamma_inf=0.02, disk_gamma0=0.95,
                      disk_radius=0.125, ps_frac=0.0)
    stack = make_stack_torch(cfg)
    plan = block_plan(frame, frame, BLOCK, half)
    forms = ("tensor", "tf32", "simt")
    rates = {}
    for form in forms:
        def step():
            for (ir, ic, *_r) in plan:
                blk = stack[:, ir[0]:ir[1], ic[0]:ic[1]].contiguous()
                mean, disp, _ps = dp.calc_ps_block(blk.abs(), PS_THR, n)
                nb = dp.estimate_neighbors(halfwin_rowcol=half, alpha=ALPHA, mean=mean, var=(disp * mean) ** 2,
                                           nslc=n)
                dp.run_phase_linking(blk, half, neighbor_arrays=nb, covariance_form=form)
        step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(max(1, args.steps)):
            step()
        e1.record()
        torch.cuda.synchronize()
        rates[form] = frame * frame * max(1, args.steps) / (e0.elapsed_time(e1) / 1000.0)
    r0 = frame // 2 - 256 + int(0.125 * frame) // 2
    crop = stack[:, r0:r0 + 512 + 2 * half[0], r0:r0 + 512 + 2 * half[1]].contiguous()
    cm, cd, _cps = dp.calc_ps_block(crop.abs(), PS_THR, n)
    cnb = dp.estimate_neighbors(halfwin_rowcol=half, alpha=ALPHA, mean=cm, var=(cd * cm) ** 2, nslc=n)
    outs, crop_rates, flags = {}, {}, {}
    for form in ("fp64", "fp64_last") + forms:
        f = torch.zeros(crop.shape[1:], dtype=torch.uint8, device=crop.device)
        kw = dict(covariance_form="fp64" if form.startswith("fp64") else form, eigh_fallback=form != "fp64_last",
                  nonconverged=f)
        dp.run_phase_linking(crop, half, neighbor_arrays=cnb, **kw)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        outs[form] = dp.run_phase_linking(crop, half, neighbor_arrays=cnb, **kw)
        e1.record()
        torch.cuda.synchronize()
        crop_rates[form] = crop.shape[1] * crop.shape[2] / (e0.elapsed_time(e1) / 1000.0)
        flags[form] = int(f.sum())
    errs = {}
    for form in forms:
        ref = outs["fp64_last" if form == "simt" else "fp64"]
        good = ref.temp_coh > 0.3
        d = torch.angle(outs[form].cpx_phase[:, good] * ref.cpx_phase[:, good].conj()).abs()
        t = (outs[form].temp_coh[good] - ref.temp_coh[good]).abs()
        worst = d.max(0).values  # per pixel, over the SLCs
        errs[form] = {"phase_max_rad": float(worst.max()), "phase_p99_rad": float(torch.quantile(worst, 0.99)),
                      "pixels_above_1e-3_rad": int((worst > 1e-3).sum()), "coherent_pixels": int(good.sum()),
                      "temp_coh_max": float(t.max()), "dense_eigensolver_pixels": flags[form],
                      "against": "fp64 with the same fallback" if form != "simt" else "fp64 keeping the last iterate"}
    print(json.dumps({"workload": "precision", "config": {"nslc": n, "frame": frame, "half_window": half,
                                                          "gamma_inf": 0.02, "disk_gamma0": 0.95},
                      "unit": UNIT, "rates": rates, "tensor_over_simt": rates["tensor"] / rates["simt"],
                      "fp64_crop": {"pixels": int(crop.shape[1] * crop.shape[2]), "rates": crop_rates,
                                    "dense_eigensolver_pixels": flags, "errors_vs_fp64": errs}}),
          flush=True)


def glrt_check(torch, mean, disp, nb, nslc, alpha, rows_per_chunk=64):
    """GLRT masks of one block against the float64 statistic: every test evaluated as
    nslc * log1p((s1 - s2)^2 / (4 s1 s2)) in float64 on the float32 scale^2, with the
    reference's window rules (clamped start, validity from the unclamped origin, centre
    excluded).  Returns (tests, tests within 1e-6 relative of the cutoff, masks that
    differ from the float64 decision)."""
    from scipy import stats

    rows, cols = mean.shape
    hy, hx = HALF
    wy, wx = 2 * hy + 1, 2 * hx + 1
    scale2 = ((disp * mean) ** 2 + mean * mean) / 2  # float32, as the kernels compute it
    s64 = scale2.double()
    thr = float(np.float32(stats.chi2.ppf(1 - alpha, df=1)))
    dev = mean.device
    r_idx = torch.arange(rows, device=dev)
    c_idx = torch.arange(cols, device=dev)
    c0 = (c_idx - hx).clamp(min=0).clamp(max=cols - wx)
    wb = torch.arange(wx, device=dev)
    wa = torch.arange(wy, device=dev)
    cc = c0[:, None] + wb[None, :]  # (cols, wx)
    valid_c = ((c_idx[:, None] - hx + wb[None, :]) >= 0) & ((c_idx[:, None] - hx + wb[None, :]) < cols)
    tests = near = differ = 0
    for r_start in range(0, rows, rows_per_chunk):
        rr = r_idx[r_start:r_start + rows_per_chunk]
        r0 = (rr - hy).clamp(min=0).clamp(max=rows - wy)
        ri = r0[:, None] + wa[None, :]  # (R, wy)
        valid_r = ((rr[:, None] - hy + wa[None, :]) >= 0) & ((rr[:, None] - hy + wa[None, :]) < rows)
        s2 = s64[ri[:, None, :, None], cc[None, :, None, :]]  # (R, C, wy, wx)
        s1 = s64[rr][:, :, None, None]
        t = float(nslc) * torch.log1p((s1 - s2) ** 2 / (4.0 * s1 * s2))
        valid = valid_r[:, None, :, None] & valid_c[None, :, None, :]
        valid[:, :, hy, hx] = False
        want = (thr > t) & valid
        got = nb[r_start:r_start + rows_per_chunk].bool()
        tests += int(valid.sum())
        near += int(((t - thr).abs() <= 1e-6 * thr)[valid].sum())
        differ += int((got != want).sum())
    return tests, near, differ


def run_parity(args):
    """The chosen form against the FP64 GPU form over the whole N=30 frame, block by block
    (the FP64 form computes the covariance and the solve in double); GLRT masks against
    the float64 statistic; near-cutoff counts for the GLRT and PS tests."""
    import torch

    import dolphin_gb300 as dp
    from dolphin_gb300._build import build_library
    from dolphin_gb300.simulate import StackConfig, make_stack_torch

    build_library()
    frame = args.frame
    stack = make_stack_torch(StackConfig(nslc=NSLC, rows=frame, cols=frame, seed=SEED, ps_frac=0.03))
    plan = block_plan(frame, frame, BLOCK, HALF)
    errs = {"tensor": [], "simt": []}
    agg = {f: {"phase_max_rad": 0.0, "above_1e-3_rad": 0, "temp_coh_max": 0.0, "flips": 0, "flips_on_ps": 0,
               "flips_fp64_emi": 0, "flips_phase_max_rad": 0.0, "coherent": 0} for f in errs}
    secs = {"tensor": 0.0, "simt": 0.0, "fp64": 0.0}
    glrt = {"tests": 0, "near_cutoff_1e-6": 0, "differ_from_float64": 0}
    ps_near = ps_count = 0
    for entry in plan:
        blk, mean, disp, ps, nb = block_inputs(dp, stack, entry)
        (t0, t1), (c0, c1) = entry[2], entry[3]
        kw = dict(ps_mask=ps, neighbor_arrays=nb, avg_mag=mean, compute_crlb=True)
        outs, ncf = {}, {}
        for form in ("fp64", "tensor", "simt"):
            ncf[form] = torch.zeros(blk.shape[1:], dtype=torch.uint8, device=blk.device)
            torch.cuda.synchronize()
            w0 = time.perf_counter()
            outs[form] = dp.run_phase_linking(blk, HALF, covariance_form=form, nonconverged=ncf[form], **kw)
            torch.cuda.synchronize()
            secs[form] += time.perf_counter() - w0
        trim = (slice(t0, t1), slice(c0, c1))
        ref = outs["fp64"]
        good = ref.temp_coh[trim] > 0.3
        psm = ps.bool()[trim]
        for form in errs:
            o = outs[form]
            d = torch.angle(o.cpx_phase[(slice(None),) + trim] * ref.cpx_phase[(slice(None),) + trim].conj())
            d = d.abs().amax(0)
            errs[form].append(d[good].float())
            tcd = (o.temp_coh[trim] - ref.temp_coh[trim]).abs()[good]
            flip = o.estimator[trim] != ref.estimator[trim]
            a = agg[form]
            a["coherent"] += int(good.sum())
            a["phase_max_rad"] = max(a["phase_max_rad"], float(d[good].max()))
            a["above_1e-3_rad"] += int((d[good] > 1e-3).sum())
            a["temp_coh_max"] = max(a["temp_coh_max"], float(tcd.max()))
            a["flips"] += int(flip.sum())
            a["flips_on_ps"] += int((flip & psm).sum())
            a["flips_fp64_emi"] += int((flip & (ref.estimator[trim] == 1)).sum())
            if (flip & good).any():
                a["flips_phase_max_rad"] = max(a["flips_phase_max_rad"], float(d[flip & good].max()))
            # the pixels above 1e-3 rad, in frame coordinates, with both forms' flags for
            # the dense eigensolver (set where the iteration missed its stopping rule)
            for r, c in (good & (d > 1e-3)).nonzero().tolist()[:20]:
                a.setdefault("above_1e-3_pixels", []).append({
                    "row": entry[4][0] + r, "col": entry[5][0] + c, "rad": float(d[r, c]),
                    "fp64_temp_coh": float(ref.temp_coh[trim][r, c]),
                    "nonconverged": int(ncf[form][trim][r, c]), "fp64_nonconverged": int(ncf["fp64"][trim][r, c])})
        tests, near, differ = glrt_check(torch, mean, disp, nb, NSLC, ALPHA)
        glrt["tests"] += tests
        glrt["near_cutoff_1e-6"] += near
        glrt["differ_from_float64"] += differ
        ps_near += int(((disp[trim] - PS_THR).abs() <= 1e-6 * PS_THR).sum())
        ps_count += int(psm.sum())
        del outs
    for form in errs:
        allv = torch.cat(errs[form])
        agg[form]["phase_p99_rad"] = float(torch.quantile(allv[torch.randperm(allv.numel(), device=allv.device)[:2**24]],
                                                          0.99))
    print(json.dumps({
        "workload": "parity",
        "metric": f"phase error of the chosen form against the FP64 GPU form, N={NSLC} {frame}x{frame}",
        "config": {"workload": f"N={NSLC} {frame}x{frame} stack (seed {SEED}), {BLOCK}x{BLOCK} blocks with halo, "
                               f"half-window {HALF}, GLRT {ALPHA}, EMI, PS {PS_THR} + fill, CRLB; outputs trimmed "
                               "to the blocks as the bench step keeps them", "blocks": len(plan)},
        "chosen": agg["tensor"], "simt": agg["simt"],
        "note": "per pixel the worst SLC's |angle(a conj b)|, on pixels whose FP64 temporal coherence is above 0.3; "
                "flips = EMI/EVD choice differs from the FP64 form's",
        "glrt": glrt, "ps": {"pixels": ps_count, "near_cutoff_1e-6": ps_near},
        "seconds": {k: round(v, 2) for k, v in secs.items()},
    }), flush=True)


def run_peaks(args):
    """FP32 and FP64 FMA rates (dpl_fp32_fma_probe, dpl_fp64_fma_probe: 8 CTAs of 256
    threads per SM, 8 independent chains per thread, best of 5) and the TF32 tensor rate
    (cuBLAS through torch.matmul with TF32 allowed, 8192^3, best of 10) of this GPU."""
    import torch

    from dolphin_gb300 import _lib
    from dolphin_gb300._build import build_library

    build_library()
    lib = _lib.load()
    dev = torch.cuda.current_device()
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    stream = torch.cuda.current_stream().cuda_stream

    def probe(fn, dtype, iters):
        blocks = sms * 8
        out = torch.empty(blocks * 256, dtype=dtype, device="cuda")
        _lib.check(fn(out.data_ptr(), blocks, iters, stream), "probe")
        best = float("inf")
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            _lib.check(fn(out.data_ptr(), blocks, iters, stream), "probe")
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        return blocks * 256 * 16.0 * iters / (best / 1000.0) / 1e12

    torch.backends.cuda.matmul.allow_tf32 = True
    a = torch.randn(8192, 8192, device="cuda")
    b = torch.randn(8192, 8192, device="cuda")
    for _ in range(3):
        a @ b
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(10):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        a @ b
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    print(json.dumps({"workload": "peaks", "unit": "TFLOP/s",
                      "fp32_fma": probe(lib.dpl_fp32_fma_probe, torch.float32, 4096),
                      "fp64_fma": probe(lib.dpl_fp64_fma_probe, torch.float64, 256),
                      "tf32_cublas": 2 * 8192**3 / (best / 1000.0) / 1e12,
                      "gpu": torch.cuda.get_device_name(dev)}), flush=True)


BATCH_DEPTHS = (8, 10, 12, 15, 18, 20, 24, 28, 32, 36, 40, 45)


def run_batch(args):
    """Ministack batch: PS + GLRT + phase linking of 12 stacks of uneven depth, eager and
    as one CUDA-graph replay, with the per-depth covariance form picked by tune_forms."""
    print(json.dumps(batch_measure(args.steps)), flush=True)


def batch_measure(steps):
    """The batch workload's figures as a dict (see run_batch)."""
    import torch

    from dolphin_gb300 import PhaseLinkBatch, tune_forms
    from dolphin_gb300._build import build_library
    from dolphin_gb300.simulate import StackConfig, make_stack_torch

    build_library()
    side, half, seed = 1024, (5, 5), 20261207
    rng = np.random.default_rng(seed)
    taus = rng.uniform(24.0, 96.0, size=len(BATCH_DEPTHS))
    stacks = [make_stack_torch(StackConfig(nslc=n, rows=side, cols=side, seed=seed + k, tau=float(taus[k]),
                                           ps_frac=0.03, outlier_frac=0.4))
              for k, n in enumerate(BATCH_DEPTHS)]
    forms = tune_forms(BATCH_DEPTHS, half)
    px = len(stacks) * side * side

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    reps = max(1, steps)
    # persistent: one dpl_phase_link_batch (the covariance of all 12 stacks in one work-
    # queue launch); per stack: one dpl_phase_link per stack; each eager and as a graph
    eager = PhaseLinkBatch(stacks, half, forms=forms, graph=False)
    eager_ms = timed(eager.run, reps)
    graph = PhaseLinkBatch(stacks, half, forms=forms, graph=True)
    graph_ms = timed(graph.run, reps)
    per_stack = PhaseLinkBatch(stacks, half, forms=forms, graph=True, persistent=False)
    per_stack_ms = timed(per_stack.run, reps)
    # per-ministack latency (eager, one stack per call)
    lat = []
    for _ in range(reps):
        for z in stacks:
            one = PhaseLinkBatch([z], half, forms=forms, graph=False)
            lat.append(timed(one.run, 1))
    return {
        "workload": "batch", "unit": UNIT,
        "config": {"depths": list(BATCH_DEPTHS), "side": side, "half_window": half, "tau_days": taus.round(1).tolist(),
                   "outlier_frac": 0.4, "ps_frac": 0.03},
        "forms": {str(k): v for k, v in forms.items()},
        "eager": px / (eager_ms / 1000.0), "graph": px / (graph_ms / 1000.0),
        "per_stack_graph": px / (per_stack_ms / 1000.0),
        "ms_per_batch": {"eager": eager_ms, "graph": graph_ms, "per_stack_graph": per_stack_ms},
        "note": "eager and graph: the persistent path (dpl_phase_link_batch); per_stack_graph: one dpl_phase_link "
                "per stack in one graph; ministack_ms: each stack alone",
        "ministack_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
    }


SIM_LAYERS, SIM_RADIUS, SIM_SEED = 30, 7, 20261209
SEQ_MINISTACK = 15


def run_learned(args):
    """Learned EMI warm start: train the 190-256-256-40 network on 2 M pixels of N=20
    stacks (the library's GEMM, ReLU, MSE and Adam kernels), then solve the held-out
    4096x4096 N=20 frame (half-window (5, 11), 1024x1024 blocks) with and without the
    warm start; the timed region per block is the solve (and, warm, the network)."""
    print(json.dumps(learned_measure(args.frame)), flush=True)


def learned_measure(frame):
    """The learned warm-start workload's figures as a dict (see run_learned)."""
    import torch

    from dolphin_gb300 import estimate_stack_covariance, run_phase_linking
    from dolphin_gb300._build import build_library
    from dolphin_gb300.learned import WarmStartMLP, make_training_set, process_coherence_warm
    from dolphin_gb300.simulate import StackConfig, make_stack_torch

    build_library()
    n = 20
    train_px = 2_000_000 if frame >= 2048 else 200_000
    t0 = time.perf_counter()
    X, T = make_training_set(train_px, nslc=n, tile=64, seed=20261300)
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    model = WarmStartMLP(nslc=n, seed=0)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(0)
    steps, batch = 3000, 4096
    t0 = time.perf_counter()
    losses = []
    for _ in range(steps):
        idx = torch.randint(0, X.shape[0], (batch,), generator=gen, device="cuda")
        losses.append(model.train_step(X[idx].contiguous(), T[idx].contiguous(), lr=1e-3))
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    del X, T
    z = make_stack_torch(StackConfig(nslc=n, rows=frame, cols=frame, seed=20261208, ps_frac=0.0))
    plan = block_plan(frame, frame, BLOCK, HALF)
    stream = torch.cuda.current_stream()
    kinds = ("plain", "warm", "perfect")
    ms = {k: 0.0 for k in kinds}
    iters = {k: [] for k in kinds}
    worst, px, fallback, fp64 = 0.0, 0, 0, None
    for bi, (ir, ic, *_r) in enumerate(plan):
        blk = z[:, ir[0]:ir[1], ic[0]:ic[1]].contiguous()
        C = estimate_stack_covariance(blk, HALF).reshape(-1, n, n).contiguous()
        res = {}
        for kind in ("plain", "warm"):  # warm-up passes
            res[kind] = process_coherence_warm(C, model if kind == "warm" else None)
        for kind in kinds:
            # perfect: started from the plain solve's own answer, the bound any warm
            # start can reach (the solve minus all but one iteration)
            vs = res["plain"][0].contiguous() if kind == "perfect" else None
            e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            torch.cuda.synchronize()
            e[0].record(stream)
            res[kind] = process_coherence_warm(C, model if kind == "warm" else None, vstart=vs)
            e[1].record(stream)
            torch.cuda.synchronize()
            ms[kind] += e[0].elapsed_time(e[1])
            iters[kind].append(res[kind][5].float().mean().item())
        v0, v1, tc = res["plain"][0], res["warm"][0], res["plain"][4]
        good = (res["plain"][2] == 1) & (tc > 0.3)
        d = torch.angle(v1[good] * v0[good].conj()).abs()
        worst = max(worst, float(d.max().item()) if d.numel() else 0.0)
        # a warm start that misses the stopping rule runs its 49 steps, then plain EMI
        fallback += int((res["warm"][5] >= 50).sum().item())
        if bi == 0:
            # the same block in double precision (covariance and solve) on the GPU
            ref = run_phase_linking(blk, HALF, covariance_form="fp64", compute_crlb=False)
            rv = ref.cpx_phase.reshape(n, -1).T
            ok = good & (ref.temp_coh.reshape(-1) > 0.3)
            dw = torch.angle(v1[ok] * rv[ok].conj()).abs().max(dim=1).values
            dp_ = torch.angle(v0[ok] * rv[ok].conj()).abs().max(dim=1).values
            fp64 = {"pixels": int(ok.sum().item()), "warm_max_rad": float(dw.max().item()),
                    "plain_max_rad": float(dp_.max().item()), "warm_above_1e-3": int((dw > 1e-3).sum().item())}
        px += C.shape[0]
        del C
    line = {
        "workload": "learned", "metric": "EMI solve pixels/sec (N=20) with the learned warm start vs plain",
        "value": px / (ms["warm"] / 1000.0), "unit": UNIT, "plain": px / (ms["plain"] / 1000.0),
        "perfect_start": px / (ms["perfect"] / 1000.0),
        "iterations_per_pixel": {k: float(np.mean(v)) for k, v in iters.items()},
        "fallback_rate": fallback / px, "vs_fp64_block0": fp64,
        "max_phase_diff_rad_coh_gt_0.3": worst, "higher_is_better": True, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"N=20 {frame}x{frame} held-out frame (seed 20261208), half-window {HALF}, "
                               f"{BLOCK}x{BLOCK} blocks; network 190-256-256-40 trained on {train_px} pixels",
                   "training": {"pixels": train_px, "adam_steps": steps, "batch": batch,
                                "loss_first_last": [float(np.mean(losses[:20])), float(np.mean(losses[-20:]))],
                                "data_s": round(t_data, 2), "train_s": round(t_train, 2)}},
    }
    return line


def run_sequential(args):
    """The sequential estimator on the 30-SLC workload: ministacks of 15 real SLCs (the
    second led by the first one's compressed SLC), 1024x1024 blocks with the (5, 11)
    halo, GLRT on the PS pass's mean and dispersion, EMI, PS fill, CRLB, closure phases,
    compressed SLCs, similarity rasters and the averaged coherence."""
    import torch

    import dolphin_gb300 as dp
    from dolphin_gb300._build import build_library
    from dolphin_gb300.simulate import StackConfig, make_stack_torch

    build_library()
    frame = args.frame
    z = make_stack_torch(StackConfig(nslc=NSLC, rows=frame, cols=frame, seed=SEED, ps_frac=0.03))
    mean, disp, ps = dp.calc_ps_block(z.abs(), PS_THR, NSLC)
    kw = dict(ministack_size=SEQ_MINISTACK, half_window=HALF, block_shape=(BLOCK, BLOCK), ps_mask=ps,
              amp_mean=mean, amp_dispersion=disp, shp_method="glrt", shp_alpha=ALPHA)
    stream = torch.cuda.current_stream()

    def timed(fn, steps):
        e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        torch.cuda.synchronize()
        e[0].record(stream)
        for _ in range(steps):
            fn()
        e[1].record(stream)
        torch.cuda.synchronize()
        return e[0].elapsed_time(e[1]) / steps

    def step(src):
        return dp.run_wrapped_phase_sequential(src, **kw)

    for _ in range(max(3, args.warmup)):
        step(z)
    sampler = ClockSampler(torch.cuda.current_device())
    sampler.start()
    ms = timed(lambda: step(z), args.steps)
    clocks = sampler.stop()
    host = torch.empty(z.shape, dtype=z.dtype, pin_memory=True)
    host.copy_(z)
    host_pl = torch.empty(z.shape, dtype=z.dtype, pin_memory=True)
    dev_in = torch.empty_like(z)

    def e2e():
        dev_in.copy_(host, non_blocking=True)
        out = step(dev_in)
        host_pl.copy_(out.pl_slcs, non_blocking=True)

    e2e()
    e2e_ms = timed(e2e, args.steps)
    # each ministack's block loop as one CUDA graph: the first call captures, the
    # following ones copy their inputs in and replay
    for _ in range(2):
        dp.run_wrapped_phase_sequential(z, graph=True, **kw)
    graph_ms = timed(lambda: dp.run_wrapped_phase_sequential(z, graph=True, **kw), args.steps)
    dp.clear_loop_graphs()
    px = frame * frame
    line = {
        "workload": "sequential",
        "metric": f"sequentially phase-linked pixels/sec ({NSLC} SLCs in ministacks of {SEQ_MINISTACK}, EMI)",
        "value": px / (ms / 1000.0), "unit": UNIT, "steps": args.steps, "warmup": max(3, args.warmup),
        "ms_per_step": ms, "higher_is_better": True, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{NSLC} SLCs {frame}x{frame} in ministacks of {SEQ_MINISTACK} (compressed SLC "
                               f"chained), {BLOCK}x{BLOCK} blocks, half-window {HALF}, GLRT {ALPHA}, EMI, PS "
                               "fill, CRLB, closure phases, similarity rasters",
                   "l2": "inputs larger than L2 (4 GB stack)"},
        "e2e": {"value": px / (e2e_ms / 1000.0), "unit": UNIT, "h2d_bytes_per_step": z.numel() * 8,
                "d2h_bytes_per_step": z.numel() * 8},
        "graph": {"value": px / (graph_ms / 1000.0), "unit": UNIT, "ms_per_step": graph_ms,
                  "note": "each ministack's block loop replayed as one CUDA graph (inputs copied into the graph's "
                          "buffers, results copied out)"},
        "clocks": clocks,
    }
    if not args.no_cpu:
        from oracle import phase_link as OP
        from oracle import workflow as OW

        crop = z[:, :48, :96].cpu().numpy()
        t0 = time.perf_counter()
        m_, d_, p_ = OP.calc_ps_block(np.abs(crop), PS_THR, NSLC)
        OW.sequential(crop, SEQ_MINISTACK, HALF, (1, 1), (BLOCK, BLOCK), np.zeros(crop.shape[1:], bool), p_, m_, d_,
                      alpha=ALPHA)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": crop.shape[1] * crop.shape[2] / dt, "unit": UNIT, "cores": 1,
                                "kind": "port", "sample": "numpy restatement of the sequential run on a 48x96 "
                                                          "crop, 1 process"}
    print(json.dumps(line), flush=True)


def run_similarity(args):
    """Phase-similarity raster (similarity.py create_similarities' block computation,
    median, search radius 7) of a 30-interferogram single-reference stack, frame x frame."""
    import torch

    from dolphin_gb300 import _device as D
    from dolphin_gb300 import _lib
    from dolphin_gb300._build import build_library
    from dolphin_gb300.simulate import StackConfig, make_stack_torch

    build_library()
    lib = _lib.load()
    frame, m, radius = args.frame, SIM_LAYERS, SIM_RADIUS
    z = make_stack_torch(StackConfig(nslc=m + 1, rows=frame, cols=frame, seed=SIM_SEED, ps_frac=0.03))
    ifg = (z[1:] * z[:1].conj()).contiguous()
    del z
    unit = torch.empty_like(ifg)
    valid = torch.empty((frame, frame), dtype=torch.uint8, device="cuda")
    out = torch.empty((frame, frame), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    sh = D.stream_handle()

    def step(src):
        _lib.check(lib.dpl_similarity_prep(src.data_ptr(), 1, m, frame, frame, None, 0, unit.data_ptr(), m,
                                           valid.data_ptr(), sh), "dpl_similarity_prep")
        _lib.check(lib.dpl_similarity(unit.data_ptr(), m, frame, frame, radius, 0, out.data_ptr(), sh),
                   "dpl_similarity")

    timing = {}

    def timed(fn, steps):
        e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        torch.cuda.synchronize()
        e[0].record(stream)
        for _ in range(steps):
            fn()
        e[1].record(stream)
        torch.cuda.synchronize()
        return e[0].elapsed_time(e[1]) / steps

    for _ in range(max(3, args.warmup)):
        step(ifg)
    sampler = ClockSampler(torch.cuda.current_device())
    sampler.start()
    ms = timed(lambda: step(ifg), args.steps)
    # the similarity kernel alone, on the phasors just written
    sim_ms = timed(lambda: _lib.check(lib.dpl_similarity(unit.data_ptr(), m, frame, frame, radius, 0,
                                                         out.data_ptr(), sh)), args.steps)
    clocks = sampler.stop()
    # end to end: pinned host stack in, host raster out.  The frame goes up in row bands
    # (each with radius - 1 rows of halo, which make a band's own rows exactly the
    # full frame's) on a copy stream; each band is prepared and summarised as soon as it
    # has landed, and its rows go down on a second copy stream.
    host = torch.empty(ifg.shape, dtype=ifg.dtype, pin_memory=True)
    host.copy_(ifg)
    ref_out = out.clone()
    host_out = torch.empty((frame, frame), dtype=torch.float32, pin_memory=True)
    halo = radius - 1
    nb = 4
    edges = [frame * b // nb for b in range(nb + 1)]
    bands = [(r0, r1, max(0, r0 - halo), min(frame, r1 + halo)) for r0, r1 in zip(edges[:-1], edges[1:])]
    # contiguous (m, band rows, cols) buffers per band, as the C ABI reads them
    b_in = [torch.empty((m, h1 - h0, frame), dtype=ifg.dtype, device="cuda") for (_r0, _r1, h0, h1) in bands]
    b_unit = [torch.empty_like(x) for x in b_in]
    b_out = [torch.empty((h1 - h0, frame), dtype=torch.float32, device="cuda") for (_r0, _r1, h0, h1) in bands]
    copy_in, copy_out = torch.cuda.Stream(), torch.cuda.Stream()

    def e2e():
        landed = []
        copy_in.wait_stream(stream)
        with torch.cuda.stream(copy_in):
            for b, (_r0, _r1, h0, h1) in enumerate(bands):
                for t in range(m):  # contiguous (rows, cols) slabs of pinned memory
                    b_in[b][t].copy_(host[t, h0:h1], non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(copy_in)
                landed.append(ev)
        for b, ((r0, r1, h0, h1), ev) in enumerate(zip(bands, landed)):
            stream.wait_event(ev)
            rows_b = h1 - h0
            _lib.check(lib.dpl_similarity_prep(b_in[b].data_ptr(), 1, m, rows_b, frame, None, 0, b_unit[b].data_ptr(),
                                               m, valid.data_ptr(), sh), "dpl_similarity_prep")
            _lib.check(lib.dpl_similarity(b_unit[b].data_ptr(), m, rows_b, frame, radius, 0, b_out[b].data_ptr(), sh),
                       "dpl_similarity")
            done = torch.cuda.Event()
            done.record(stream)
            with torch.cuda.stream(copy_out):
                copy_out.wait_event(done)
                host_out[r0:r1].copy_(b_out[b][r0 - h0:r1 - h0], non_blocking=True)
        stream.wait_stream(copy_out)

    e2e()
    torch.cuda.synchronize()
    if not torch.equal(host_out, ref_out.cpu()):
        raise RuntimeError("banded similarity differs from the full-frame raster")
    e2e_ms = timed(e2e, args.steps)
    px = frame * frame
    # algorithmic work: K circle offsets x m layers x 4 flops (Re(x conj y)) per pixel
    from dolphin_gb300.similarity import get_circle_idxs

    K = len(get_circle_idxs(radius))
    flops = px * K * m * 4.0
    fp32_peak = fp32_peak_tflops(torch, lib, torch.cuda.current_device())  # measured FMA rate, TFLOP/s
    line = {
        "workload": "similarity", "metric": f"phase-similarity pixels/sec (median, radius {radius}, {m} layers)",
        "value": px / (ms / 1000.0), "unit": UNIT, "steps": args.steps, "warmup": max(3, args.warmup),
        "ms_per_step": ms, "higher_is_better": True, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{m} single-reference interferograms, {frame}x{frame}, median similarity, "
                               f"search radius {radius} ({K} neighbours)", "l2": f"inputs larger than L2 "
                               f"({ifg.numel() * 8 / 1e9:.1f} GB)"},
        "e2e": {"value": px / (e2e_ms / 1000.0), "unit": UNIT, "h2d_bytes_per_step": ifg.numel() * 8,
                "d2h_bytes_per_step": px * 4, "note": f"{nb} row bands with {halo} halo rows, copies overlapping compute"},
        "roofline": {"bound": "fp32", "kernel": "k_similarity", "kernel_ms": sim_ms,
                     "achieved": flops / (sim_ms / 1000.0) / 1e12, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": flops / (sim_ms / 1000.0) / 1e12 / fp32_peak,
                     "note": "algorithmic flops K*m*4 per pixel over the CUDA-event kernel time; peak = FP32 FMA "
                             "rate measured on this GPU with dpl_fp32_fma_probe (of measured)"},
        "clocks": clocks,
    }
    if not args.no_cpu:
        from oracle import similarity as O

        crop = ifg[:, :256, :256].cpu().numpy()
        t0 = time.perf_counter()
        O.median_similarity(crop, radius)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": crop.shape[1] * crop.shape[2] / dt, "unit": UNIT, "cores": 1,
                                "kind": "port", "sample": "numpy restatement on a 256x256 crop, 1 process"}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--frame", type=int, default=FRAME)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the batch and learned figures that the default line adds after its timed regions")
    ap.add_argument("--workload", default="config2",
                    choices=["config2", "precision", "batch", "similarity", "sequential", "learned", "parity",
                             "peaks", "cpu-table"],
                    help="precision: N=40 2048x2048 stack, half-window (7, 7), low gamma_inf with a "
                         "high-coherence disk; rates of the tensor-core and SIMT covariance forms. "
                         "batch: 12 ministacks of N = 8..45, 1024x1024 each, as one CUDA graph. "
                         "similarity: median phase similarity, radius 7, of 30 interferograms. "
                         "sequential: the 30-SLC frame as ministacks of 15 with compressed SLCs. "
                         "learned: EMI with and without the learned warm start, N=20. "
                         "parity: the chosen form against the FP64 GPU form over the whole N=30 frame. "
                         "peaks: FP32, FP64 and TF32 rates of this GPU. "
                         "cpu-table (with --impl reference): the CPU baseline table")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if args.workload == "cpu-table":
            run_cpu_table(args)
        else:
            run_reference(args, rank, world)
        return
    if args.workload == "precision":
        run_precision(args)
        return
    if args.workload == "batch":
        run_batch(args)
        return
    if args.workload == "similarity":
        run_similarity(args)
        return
    if args.workload == "sequential":
        run_sequential(args)
        return
    if args.workload == "learned":
        run_learned(args)
        return
    if args.workload == "parity":
        run_parity(args)
        return
    if args.workload == "peaks":
        run_peaks(args)
        return
    pool = None
    cores = len(os.sched_getaffinity(0))
    if rank == 0 and not args.no_cpu:
        # start the CPU worker pool (spawn) before the first CUDA call
        pool = mp.get_context("spawn").Pool(cores)
    try:
        run_ours(args, rank, world, pool, cores)
    finally:
        if pool is not None:
            pool.terminate()


if __name__ == "__main__":
    main()
