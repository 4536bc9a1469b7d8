"""Benchmark: seconds per gauge configuration of the sLapH hot path.

One step is one gauge configuration through the engine: VdaggerV for every
operator and timeslice, then the full contraction (diluted factors, factor
products, diluted traces, correlator assembly) of the workload's diagram set.

* ``value``: device-resident inputs (eigenvectors, perambulators, noise already
  in HBM when the timed region starts); timed with CUDA events on the engine
  stream (the engine's own stage events) and bracketed by device syncs.
* ``e2e``: the same step through the C ABI from host buffers: host->device
  copies of all inputs and the device->host read of the correlators are
  inside the timed region.
* ``--impl reference``: the CPU restatement of the reference (the oracle,
  OpenMP on the host cores) on a bounded sample of the same workload,
  extrapolated to one configuration.

Inputs are seeded synthetic data with the workload's shapes (the production
ensembles are not available); V totals 22 GB at 32^3 x 64, far above L2, so no
L2 flush is needed between steps.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
for p in (str(REPO), str(REPO / "slaph-contractions_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = "s/gauge-config, VdaggerV+pipi contractions 32³×64: FP64 vs split-prec @1e-10"
UNIT = "s/gauge-config"

# DRAM bytes (read + write) of the tensor-core GEMMs per unit of work, from
# one-pass ncu captures (dram__bytes_read.sum + dram__bytes_write.sum) of the
# full-size 32^3x64 launches; the captures and the derivation are in the
# profile summary named here.  Other workloads have no capture: their
# roofline's traffic is null.
NCU_TRACE_GEMM_DRAM_BYTES_PER_ENTRY = {"cfg3_32x64_pipi": 470.0}  # per dense-group entry
NCU_TRACE_GEMM_TRAFFIC_SOURCE = "profiles/gemm_dram_traffic_cfg3_32x64_pipi.md"
NCU_VDV_GEMM_DRAM_BYTES_PER_UNIT = {"cfg3_32x64_pipi": 0.867e9}  # per (operator, timeslice)
NCU_VDV_GEMM_TRAFFIC_SOURCE = "profiles/gemm_dram_traffic_cfg3_32x64_pipi.md"


def per_correlator_rel_err(out, ref):
    """Largest relative error over correlators, each (one HDF5 dataset, Lt
    values) normalised by its own largest |value|; correlators that are zero in
    ref contribute their absolute error."""
    scale = np.max(np.abs(ref), axis=1)
    diff = np.max(np.abs(out - ref), axis=1)
    rel = np.where(scale > 0, diff / np.where(scale > 0, scale, 1.0), diff)
    return float(np.max(rel)) if rel.size else 0.0


# Host bytes up to which the VdaggerV blocks of a build are kept for the
# comparison of the two paths (32^3x64: 33 operators x 64 timeslices x
# 220^2 x 16 B = 1.6 GB).
VDV_CHECK_MAX_BYTES = 8e9


def vdaggerv_snapshot(eng, n_ops, Lt):
    """Every VdaggerV block (operator, timeslice) of the engine's last build."""
    return [eng.vdaggerv_fetch(op, t) for op in range(n_ops) for t in range(Lt)]


def vdaggerv_max_rel_err(eng, n_ops, Lt, snapshot):
    """Largest error of the snapshot's blocks against the engine's current
    build, each block by the largest |entry| of the current one (its
    absolute error for a zero block)."""
    err, k = 0.0, 0
    for op in range(n_ops):
        for t in range(Lt):
            ref = eng.vdaggerv_fetch(op, t)
            d = float(np.max(np.abs(snapshot[k] - ref)))
            m = float(np.max(np.abs(ref)))
            err = max(err, d / m if m > 0 else d)
            k += 1
    return err


def workload_config(w, n_correlators, single_block_pair, world):
    """The workload's description, printed identically by both arms."""
    return {"workload": w.name, "lattice": f"{w.L}^3x{w.Lt}", "nev": w.nev,
            "n_rnd": w.n_rnd, "dilution": f"TB{w.dilT} EI{w.dilE} DF4",
            "diagrams": sorted({c.split(':')[0] for c in w.correlators}),
            "n_correlators": int(n_correlators), "single_block_pair": single_block_pair,
            "l2": "inputs larger than L2 (eigenvectors alone exceed 129 MB)",
            "parallelism": f"replicas x{world}"}


def load_peaks():
    try:
        return json.loads((REPO / "MEASURED_PEAKS.json").read_text())
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clock and throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
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
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)),
                "power_w_max": float(max(power)) if power else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def dist_setup(n_gpus, backend="nccl"):
    """One process per GPU (torchrun): rank, world size, local rank and the
    process group (None for a single process).  The replicas exchange only
    their timings; gloo serves for tests without GPUs."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
        return rank, world, local, dist
    return rank, world, local, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x):
    """The largest of the ranks' values (the job's time is its slowest rank's)."""
    if dist is None:
        return x
    import torch
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def pageable_nothp_copy(a):
    """A page-aligned numpy copy of a with madvise(MADV_NOHUGEPAGE) applied."""
    import ctypes
    import mmap
    n = a.nbytes
    size = (n + mmap.PAGESIZE - 1) // mmap.PAGESIZE * mmap.PAGESIZE
    buf = mmap.mmap(-1, max(size, mmap.PAGESIZE), flags=mmap.MAP_PRIVATE | mmap.MAP_ANONYMOUS)
    try:
        libc = ctypes.CDLL(None)
        addr = ctypes.addressof(ctypes.c_char.from_buffer(buf))
        libc.madvise(ctypes.c_void_p(addr), ctypes.c_size_t(size), 15)  # MADV_NOHUGEPAGE
    except Exception:
        pass
    out = np.frombuffer(buf, dtype=a.dtype, count=a.size).reshape(a.shape)
    out[...] = a
    return out


def set_device(local):
    import ctypes
    try:
        rt = ctypes.CDLL("libcudart.so")
    except OSError:
        rt = None
    if rt is not None:
        rt.cudaSetDevice(local)


def run_engine(args):
    from slaph_gb300 import GlobalData, synthetic
    from slaph_gb300.engine import Engine

    rank, world, local, dist = dist_setup(args.gpus)
    w = synthetic.CONFIGS[args.workload]
    gd = GlobalData.from_infile(w.write_infile())
    dims = gd.dims
    # Host input buffers: driver-pinned (slaph_host_alloc), or pageable numpy
    # arrays kept out of transparent huge pages (the kernel's collapse of large
    # anonymous mappings moves pages under the GPU's host page-table reads).
    from slaph_gb300.engine import pinned_empty

    def pinned_copy(a):
        if args.host_buffers == "pageable":
            return pageable_nothp_copy(a)
        p = pinned_empty(a.shape, a.dtype)
        p[...] = a
        return p

    t_gen = time.time()
    # Workloads with a period keep that many distinct timeslices on the host
    # (every timeslice is still copied and computed).
    n_distinct = w.v_period if w.v_period > 0 else w.Lt
    pool = [pinned_copy(w.eigenvectors(t)) for t in range(n_distinct)]
    V = [pool[t % n_distinct] for t in range(w.Lt)]
    peram = [pinned_copy(w.perambulator(r)) for r in range(w.n_rnd)]
    noise = pinned_copy(np.stack([w.noise(r) for r in range(w.n_rnd)]))
    precision = 1 if args.precision == "mixed" else 0

    eng = Engine(dims)
    eng.set_operators(gd.plan)
    slots = args.eigenvector_slots if args.eigenvector_slots >= 0 else w.eigenvector_slots
    if slots > 0:
        eng.set_eigenvector_slots(slots)  # streamed: the builds copy from V
    if w.factors_per_block_pair:
        eng.set_factor_lifetime(True)
    # Displaced operators: gauge links of every timeslice, uploaded and
    # HYP-smeared (infile alpha1, alpha2, iterations) per configuration, as
    # create_operators reads and smears them (src/OperatorFactory.cpp:248-260).
    U = None
    if gd.plan.need_gaugefield:
        upool = [pinned_copy(w.gauge_links(t)) for t in range(n_distinct)]
        U = [upool[t % n_distinct] for t in range(w.Lt)]
    hyp = gd.hyp_parameters()
    t_gen = time.time() - t_gen

    def upload_eigenvectors(asynchronous=True):
        # Enqueued on the engine's upload stream; the VdaggerV build waits for
        # each timeslice as it needs it.
        for t, v in enumerate(V):
            eng.set_eigenvectors(t, v, asynchronous)

    def upload_rest(asynchronous=True):
        # Perambulators and noise; the contraction waits for them.
        for r, p in enumerate(peram):
            eng.set_perambulator(r, p, asynchronous)
        for r in range(noise.shape[0]):
            eng.set_random_vector(r, noise[r], asynchronous)

    def upload(asynchronous=True):
        upload_eigenvectors(asynchronous)
        upload_rest(asynchronous)

    def gauge():
        # links of the configuration, smeared on the device (timings[13])
        if U is None:
            return 0.0
        for t, u in enumerate(U):
            eng.set_gauge(t, u)
        if hyp[2] > 0:
            eng.smear_gauge_hyp(*hyp)
            return float(eng.timings()[13])
        return 0.0

    def step():
        gauge()
        eng.vdaggerv_build(precision)
        out = eng.contract(gd.plan_ptr, precision, 0, args.single_block_pair)
        return out

    def device_memory_used():
        import ctypes
        try:
            rt = ctypes.CDLL("libcudart.so")
        except OSError:
            return None
        free, total = ctypes.c_size_t(), ctypes.c_size_t()
        if rt.cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total)) != 0:
            return None
        return (total.value - free.value) / 1e9


    t0 = time.time()
    upload(False)
    first_upload_s = time.time() - t0
    t0 = time.time()
    out = step()  # also builds and uploads the (config-independent) schedule
    first = time.time() - t0
    tim = eng.timings()
    plan_s = tim[4] / 1e3
    for _ in range(max(0, args.warmup - 1)):
        step()

    # ---- device-resident timed region
    barrier(dist)
    sampler = ClockSampler(local)
    sampler.start()
    stage = np.zeros(5)  # VdaggerV, factors, products + traces, assembly, HYP smearing
    launches = 0
    ktim = np.zeros_like(eng.timings())  # per-kernel times and launch counts, over steps
    mem_hw = device_memory_used()
    wall0 = time.time()
    for _ in range(args.steps):
        h = gauge()
        eng.vdaggerv_build(precision)
        eng.contract(gd.plan_ptr, precision, 0, args.single_block_pair)
        tim = eng.timings()
        stage[:4] += tim[:4]
        stage[4] += h
        launches += int(tim[5])
        ktim += tim
        m = device_memory_used()
        if m is not None:
            mem_hw = max(mem_hw or 0.0, m)
    wall = time.time() - wall0
    clocks = sampler.stop()
    dev_s = stage.sum() / 1e3 / args.steps
    dev_s = max_over_ranks(dist, dev_s)

    # ---- end to end from host buffers
    barrier(dist)
    # Configurations streamed as a production run does: the eigenvectors of
    # configuration i+1 are uploaded while configuration i contracts (the
    # contraction does not read them), perambulators and noise before each
    # configuration's build.  Every step's inputs are copied inside the timed
    # region; the results are read back by contract().
    e2e0 = time.time()
    e2e_parts = []
    upload_eigenvectors()
    for i in range(args.steps):
        t_a = time.time()
        upload_rest()
        gauge()
        eng.vdaggerv_build(precision)
        if i + 1 < args.steps:
            upload_eigenvectors()
        t_b = time.time()
        out = eng.contract(gd.plan_ptr, precision, 0, args.single_block_pair)
        e2e_parts.append((t_b - t_a, time.time() - t_b))
    e2e = max_over_ranks(dist, (time.time() - e2e0) / args.steps)
    h2d = (sum(v.nbytes for v in V) + sum(p.nbytes for p in peram) + noise.nbytes
           + (sum(u.nbytes for u in U) if U is not None else 0))
    d2h = out.nbytes

    # ---- the plain FP64 path on the same inputs (outside the timed regions):
    # its time per configuration and every correlator of the split-precision
    # result against it, relative per correlator.
    fp64 = None
    if precision == 1 and not args.no_fp64_check:
        # The VdaggerV blocks of the last split-precision build (the
        # contraction leaves them in place), against the FP64 build of the
        # same eigenvectors below: every operator and timeslice.
        n_vdv_ops = int(gd.plan.n_vdv_ops)
        vdv_snap, vdv_err, vdv_note = None, None, None
        if n_vdv_ops * w.Lt * 16 * w.nev ** 2 <= VDV_CHECK_MAX_BYTES:
            try:
                vdv_snap = vdaggerv_snapshot(eng, n_vdv_ops, w.Lt)
            except Exception as exc:  # reported in the line, never fatal
                vdv_note = f"not compared: {exc}"
        else:
            vdv_note = f"not compared: blocks above {VDV_CHECK_MAX_BYTES:.0e} host bytes"
        w0 = time.time()
        eng.vdaggerv_build(0)
        t_v = eng.timings()
        out64 = eng.contract(gd.plan_ptr, 0, 0, args.single_block_pair)
        t_c = eng.timings()
        wall64 = time.time() - w0
        if vdv_snap is not None:
            try:
                vdv_err = vdaggerv_max_rel_err(eng, n_vdv_ops, w.Lt, vdv_snap)
            except Exception as exc:
                vdv_note = f"not compared: {exc}"
            vdv_snap = None
        # the same (FP64) HYP smearing precedes both builds
        st64 = [t_v[0], t_c[1], t_c[2], t_c[3], stage[4] / args.steps]
        fp64 = {"value": float(sum(st64)) / 1e3, "unit": UNIT,
                "stages_ms": dict(zip(["vdaggerv", "factors", "products_traces", "assembly",
                                       "hyp_smearing"], map(float, st64))),
                "wall_s": wall64,
                "max_rel_err_vs_fp64": per_correlator_rel_err(out, out64),
                "n_correlators": int(out64.shape[0]),
                "error_measure": ("max over correlators of max_t |mixed - fp64| / "
                                  "max_t |fp64| (each HDF5 dataset by its own scale)"),
                "vdaggerv_max_rel_err_vs_fp64": vdv_err,
                "vdaggerv_blocks": n_vdv_ops * w.Lt if vdv_err is not None else 0,
                "vdaggerv_error_measure": (vdv_note or
                                           "max over (operator, timeslice) blocks of "
                                           "max |mixed - fp64| / max |fp64 block|")}

    stats = eng.stats()
    n_ops = gd.plan.n_vdv_ops - (1 if gd.plan.index_of_unity >= 0 else 0)
    vdv_flops = w.flops_vdaggerv(n_ops)
    stage_ms = stage / args.steps
    peaks = load_peaks() or {}
    # The tensor-core kernels run inside a seconds-long step: the sustained
    # bf16 rate is their denominator.
    bf16_peak = peaks.get("bf16_tflops_sustained", 1700.0)
    note = "of measured" if peaks else "of fallback"
    peak_src = ("MEASURED_PEAKS.json bf16_tflops_sustained" if peaks
                else "fallback 1.7 PFLOP/s sustained")
    names = ["vdaggerv", "factors", "products_traces", "assembly", "hyp_smearing"]
    eds = 4 * w.dilE
    K = args.steps
    # Kernels timed on their own by the engine's CUDA events (per step).
    kernels_ms = {"trace_gemm_kernel": ktim[8] / K, "trace_slice_kernels": ktim[10] / K,
                  "trace_df_kernel (residual lists)" if precision == 1 else "trace_kernel":
                  ktim[6] / K,
                  "ozaki_gemm_kernel (VdaggerV GEMM)": ktim[11] / K,
                  "vdaggerv stage (slicing + ozaki_gemm_kernel)" if precision == 1
                  else "vdaggerv stage (vdv_fp64_kernel)": stage_ms[0],
                  "factor stage (q*_kernels, factor GEMMs)": stage_ms[1],
                  "factor products (slicing + product_gemm_kernel)" if precision == 1
                  else "factor products (product_kernel)": ktim[14] / K}
    # Roofline candidates, one kernel each: (time per step in ms, roofline).
    cands = []
    if precision == 1 and ktim[8] > 0:
        # Dense trace groups: per entry 8 (4dilE)^2 FP64-equivalent flops,
        # issued as 21 split-BF16 products.
        flops = 21 * 8.0 * eds * eds * stats[7]
        n_l = ktim[9] / K
        cands.append((ktim[8] / K, {
            "kernel": "trace_gemm_kernel", "bound": "tensor",
            "achieved": flops / (ktim[8] / K / 1e3) / 1e12, "peak": bf16_peak,
            "unit": "TFLOP/s", "peak_source": f"{peak_src} ({note})",
            "launches_per_step": n_l, "launch_ms_avg": ktim[8] / K / n_l,
            "algorithmic_per_launch": flops / n_l,
            "traffic": (NCU_TRACE_GEMM_DRAM_BYTES_PER_ENTRY.get(args.workload, 0) * stats[7] / n_l)
            or None,
            "traffic_source": NCU_TRACE_GEMM_TRAFFIC_SOURCE,
            "fp64_equivalent_tflops": 8.0 * eds * eds * stats[7] / (ktim[8] / K / 1e3) / 1e12,
            "work": "21 split-BF16 products x 8 (4dilE)^2 flops per dense-group trace entry"}))
    if precision == 1 and ktim[11] > 0:
        flops = 21 * vdv_flops  # 21 slice pairs of the real form of every (op, t) product
        n_l = ktim[12] / K
        cands.append((ktim[11] / K, {
            "kernel": "ozaki_gemm_kernel", "bound": "tensor",
            "achieved": flops / (ktim[11] / K / 1e3) / 1e12, "peak": bf16_peak,
            "unit": "TFLOP/s", "peak_source": f"{peak_src} ({note})",
            "launches_per_step": n_l, "launch_ms_avg": ktim[11] / K / n_l,
            "algorithmic_per_launch": flops / n_l,
            "traffic": (NCU_VDV_GEMM_DRAM_BYTES_PER_UNIT.get(args.workload, 0)
                        * n_ops * w.Lt / n_l) or None,
            "traffic_source": NCU_VDV_GEMM_TRAFFIC_SOURCE,
            "fp64_equivalent_tflops": vdv_flops / (ktim[11] / K / 1e3) / 1e12,
            "work": "21 split-BF16 products x 8 nev^2 3L^3 flops per (operator, timeslice)"}))
    ms_dom, roofline = max(cands, key=lambda c: c[0]) if cands else (0.0, {})
    if roofline:
        roofline["frac"] = roofline["achieved"] / roofline["peak"]
        roofline["share_of_step"] = ms_dom / max(stage_ms.sum(), 1e-9)
    others = [c[1] for c in cands if c[1] is not roofline]
    for o in others:
        o["frac"] = o["achieved"] / o["peak"]
    if ktim[6] > 0:
        # The per-entry trace kernel is bound by FP32 instruction issue (its
        # operands are reused from L2), so it gets no HBM roofline.
        ent = stats[6] - stats[7] if precision == 1 else stats[6]
        others.append({
            "kernel": "trace_df_kernel" if precision == 1 else "trace_kernel",
            "bound": "fp32-issue" if precision == 1 else "fp64-issue",
            "ms_per_step": ktim[6] / K, "trace_entries_per_step": ent,
            "fp64_equivalent_tflops": 8.0 * eds * eds * ent / (ktim[6] / K / 1e3) / 1e12,
            "note": ("double-float arithmetic, about 40 FP32 instructions per complex "
                     "multiply-add; operands reused about 14x from L2")})
    line = {
        "metric": METRIC, "value": dev_s * world / world, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_s * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if precision == 0 else "bf16x6-split+f32x2+f64", "data": "synthetic",
        "config": workload_config(w, out.shape[0], args.single_block_pair, world),
        "precision": args.precision,
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h),
                "host_buffers": ("page-locked (slaph_host_alloc)" if args.host_buffers == "pinned"
                                 else "pageable, no transparent huge pages"),
                "uploads": ("asynchronous: eigenvectors of the next configuration during "
                            "the contraction, perambulators and noise before the build"),
                "build_s": [round(a, 4) for a, _ in e2e_parts],
                "contract_s": [round(b, 4) for _, b in e2e_parts],
                "blocking_upload_s": round(first_upload_s, 4)},
        "gpu_launches": launches,
        "stages_ms": dict(zip(names, map(float, stage_ms))),
        "work": {"vdaggerv_tflop": vdv_flops / 1e12, "factor_tflop": stats[4] / 1e12,
                 "product_trace_tflop": stats[5] / 1e12, "factors": stats[0],
                 "products": stats[1], "trace_entries": stats[2], "terms": stats[3]},
        "planning_s": plan_s, "first_step_s": first, "input_generation_s": t_gen,
        "device_memory_used_gb": mem_hw,
        "eigenvectors": (f"streamed through {slots} device slots" if slots > 0
                         else "resident (all timeslices)"),
        "factor_lifetime": "block pair" if w.factors_per_block_pair else "configuration",

        "roofline": roofline, "roofline_others": others, "kernels_ms": kernels_ms,
        "clocks": clocks,
        "wall_s_per_step": wall / args.steps,
    }
    if fp64 is not None:
        line["fp64"] = fp64
        line["fp64_value"] = fp64["value"]
        line["max_rel_err_vs_fp64"] = fp64["max_rel_err_vs_fp64"]
    if rank == 0 and not args.no_cpu_baseline and world == 1:
        line["cpu_baseline"] = cpu_baseline(w, args)
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def run_uneven(args):
    """The uneven batch (synthetic.UNEVEN_CFG4): six configurations of
    different lattice size, Nev, random-vector count and time dilution, one
    after another in one process, each through its own engine.  Per instance:
    the split-precision time per configuration (device stage times, after one
    warm-up configuration that plans and allocates), the plain FP64 path's
    time, and every correlator of the split-precision result against the FP64
    result, relative per correlator."""
    from slaph_gb300 import GlobalData, synthetic
    from slaph_gb300.engine import Engine
    rows = []
    t_all = time.time()
    for w in synthetic.UNEVEN_CFG4:
        gd = GlobalData.from_infile(w.write_infile())
        eng = Engine(gd.dims)
        eng.set_operators(gd.plan)
        for t in range(w.Lt):
            eng.set_eigenvectors(t, w.eigenvectors(t))
        for r in range(w.n_rnd):
            eng.set_perambulator(r, w.perambulator(r))
            eng.set_random_vector(r, w.noise(r))

        def run(precision):
            eng.vdaggerv_build(precision)
            v = eng.timings()[0]
            out = eng.contract(gd.plan_ptr, precision, 0)
            tim = eng.timings()
            return out, (v + tim[1] + tim[2] + tim[3]) / 1e3

        run(1)  # warm-up: planning and allocations
        secs = []
        for _ in range(max(1, args.steps)):
            out, sec = run(1)
            secs.append(sec)
        out64, sec64 = run(0)
        rows.append({"workload": w.name, "lattice": f"{w.L}^3x{w.Lt}", "nev": w.nev,
                     "n_rnd": w.n_rnd, "dilution": f"TB{w.dilT} EI{w.dilE} DF4",
                     "n_correlators": int(out.shape[0]), "value": float(np.mean(secs)),
                     "fp64_value": sec64,
                     "max_rel_err_vs_fp64": per_correlator_rel_err(out, out64)})
        eng.close()
    total = sum(r["value"] for r in rows)
    print(json.dumps({
        "metric": "s/gauge-config, six uneven configurations (24^3x48 and 32^3x64, "
                  "Nev 64-220), split precision vs FP64",
        "value": total / len(rows), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "higher_is_better": False, "dtype": "bf16x6-split+f32x2+f64", "data": "synthetic",
        "config": {"workload": "cfg4_uneven", "instances": len(rows),
                   "order": "one after another in one process, one engine each"},
        "sum_s": total, "fp64_sum_s": sum(r["fp64_value"] for r in rows),
        "max_rel_err_vs_fp64": max(r["max_rel_err_vs_fp64"] for r in rows),
        "instances": rows, "wall_s": time.time() - t_all}))


def _dynamic_schedule(times, threads):
    """Wall time of an OpenMP schedule(dynamic) over `times` in order."""
    free = [0.0] * max(1, threads)
    for t in times:
        i = int(np.argmin(free))
        free[i] += t
    return max(free)


class CpuSample:
    """The oracle (the reference's algorithm restated, OpenMP) timed on the
    host cores on a bounded sample of one configuration, and extrapolated the
    way the reference parallelises it: VdaggerV over timeslices
    (src/OperatorFactory.cpp:220-326), the contraction over block pairs
    (src/Correlators.cpp:86-116)."""

    def __init__(self, w, gd, threads=None):
        import oracle
        oracle.build_oracle.build()
        self.oracle = oracle
        self.w, self.gd = w, gd
        d = gd.dims
        n_bp = (w.Lt // w.dilT) * (w.Lt // w.dilT + 1) // 2
        self.slices = [len(oracle.block_pair_slices(w.Lt, w.dilT, b)) for b in range(n_bp)]
        self.threads = threads or (os.cpu_count() or 1)
        oracle.set_threads(self.threads)
        rng = np.random.default_rng(7)
        # VdaggerV values stand in for the product of the VdaggerV stage; the
        # contraction cost does not depend on them.
        self.vdv = rng.standard_normal((gd.plan.n_vdv_ops, d.Lt, d.nev, 2 * d.nev))
        self.vdv = self.vdv.view(np.complex128)
        self.peram = [np.ascontiguousarray(w.perambulator(r)) for r in range(w.n_rnd)]
        self.noise = np.ascontiguousarray(np.stack([w.noise(r) for r in range(w.n_rnd)]))
        self.nts = min(w.Lt, self.threads)
        self.V = [w.eigenvectors(t) if t < self.nts else None for t in range(w.Lt)]
        unity = gd.plan.index_of_unity
        self.n_computed = gd.plan.n_vdv_ops - (1 if unity >= 0 else 0)
        # The first operators up to and including one computed (non-identity) one.
        self.n_sample_ops = 2 if unity == 0 else 1

    def vdaggerv(self):
        """One computed operator on `nts` timeslices, one per thread."""
        t0 = time.time()
        self.oracle.vdaggerv(self.gd.dims, self.gd.plan, self.V, ts=list(range(self.nts)),
                             n_ops=self.n_sample_ops)
        per = time.time() - t0
        waves = -(-self.w.Lt // self.threads)
        return per * waves * self.n_computed, per

    def contraction(self):
        cold, steady = self.oracle.contract_sample(
            self.gd.dims, self.gd.plan_ptr, self.vdv, self.peram, self.noise,
            list(range(len(self.slices))))
        per_bp = [c + (n - 1) * s for c, s, n in zip(cold, steady, self.slices)]
        return _dynamic_schedule(per_bp, self.threads), cold, steady

    def run(self):
        t0 = time.time()
        vdv_s, vdv_unit = self.vdaggerv()
        con_s, cold, steady = self.contraction()
        sample_wall = time.time() - t0
        w = self.w
        return {
            "value": vdv_s + con_s, "unit": UNIT, "cores": self.threads, "kind": "port",
            "vdaggerv_s": vdv_s, "contraction_s": con_s, "sample_wall_s": sample_wall,
            "sample": (f"oracle, {self.threads} OpenMP threads: VdaggerV of one operator on "
                       f"{self.nts} timeslices ({vdv_unit:.2f} s) scaled by "
                       f"{self.n_computed} operators x {-(-w.Lt // self.threads)} timeslice "
                       f"waves; contraction: per block pair one off-diagonal slice pair from "
                       f"empty caches (max {max(cold):.1f} s) plus (slice pairs - 1) x the same "
                       f"slice pair with factors cached (mean {np.mean(steady):.2f} s), block "
                       f"pairs {self.slices} scheduled dynamically over {self.threads} threads; "
                       f"within 10% below a full single-thread block-pair run at 16^3x32"),
        }


def oracle_global_data(w):
    """The oracle's own parse of the workload infile (no engine library)."""
    from oracle import frontend
    return frontend.GlobalData(w.write_infile())


def cpu_baseline(w, args):
    return CpuSample(w, oracle_global_data(w)).run()


def run_reference(args):
    """The reference's algorithm on the host cores: the oracle (its CPU
    restatement, OpenMP as the reference), with the oracle's own front end, so
    that no engine code is loaded.  Every timed step is one bounded sample of
    the configuration (CpuSample.run); the line's ms_per_step is that sample's
    wall time and value the configuration time it extrapolates to, the factor
    between them given in "extrapolation"."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    from slaph_gb300 import synthetic
    w = synthetic.CONFIGS[args.workload]
    gd = oracle_global_data(w)
    cs = CpuSample(w, gd)
    for _ in range(args.warmup):
        cs.vdaggerv()  # untimed warm-up: page in the inputs, start the thread pool
    vals, walls, cb = [], [], None
    t0 = time.time()
    for _ in range(args.steps):
        cb = cs.run()
        vals.append(cb["value"])
        walls.append(cb["sample_wall_s"])
    timed = time.time() - t0
    v = float(np.mean(vals)) if vals else None
    ms = 1e3 * float(np.mean(walls)) if walls else None
    if cb is not None:
        cb["value"] = v
        cb["sample_wall_s"] = ms / 1e3
    maps = ""
    try:
        maps = Path("/proc/self/maps").read_text()
    except OSError:
        pass
    print(json.dumps({
        "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "impl": "reference",
        "config": workload_config(w, gd.output_doubles() // (2 * w.Lt), args.single_block_pair,
                                  world),
        "timed_region_s": timed,
        "extrapolation": {
            "factor": v / (ms / 1e3) if v and ms else None,
            "model": ("value = VdaggerV wave time x operators x timeslice waves + the "
                      "dynamic schedule over the host threads of, per block pair, one cold "
                      "slice pair + (slice pairs - 1) x one steady slice pair; "
                      "ms_per_step is the wall time of that sample"),
            "hook": ("one block pair per thread, as the reference's "
                     "--single_time_slice_combination (src/global_data.cpp:84-87, "
                     "src/Correlators.cpp:88-90) restricts contract() to one block pair, "
                     "sampled here by one slice pair of each")},
        "engine_library_loaded": "libslaph_gb300" in maps,
        "cpu_baseline": cb,
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def main():
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["engine", "reference"], default="engine")
    ap.add_argument("--workload", default="cfg3_32x64_pipi")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="mixed")
    ap.add_argument("--single-block-pair", type=int, default=-1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--eigenvector-slots", type=int, default=-1,
                    help="stream the eigenvectors through this many device slots "
                         "(0: all resident; default: the workload's setting)")
    ap.add_argument("--no-fp64-check", action="store_true",
                    help="skip the FP64 run and the per-correlator comparison after timing")
    ap.add_argument("--host-buffers", choices=["pinned", "pageable"], default="pinned",
                    help="host input buffers: driver-pinned, or pageable without huge pages")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "cfg4_uneven":
        run_uneven(args)
    else:
        run_engine(args)


if __name__ == "__main__":
    main()
