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


def dist_setup(n_gpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        return rank, world, local, dist
    return rank, world, local, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


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
    t_gen = time.time()
    V = [w.eigenvectors(t) for t in range(w.Lt)]
    peram = [np.ascontiguousarray(w.perambulator(r)) for r in range(w.n_rnd)]
    noise = np.ascontiguousarray(np.stack([w.noise(r) for r in range(w.n_rnd)]))
    t_gen = time.time() - t_gen
    precision = 1 if args.precision == "mixed" else 0

    eng = Engine(dims)
    eng.set_operators(gd.plan)

    def upload():
        for t, v in enumerate(V):
            eng.set_eigenvectors(t, v)
        for r, p in enumerate(peram):
            eng.set_perambulator(r, p)
        for r in range(noise.shape[0]):
            eng.set_random_vector(r, noise[r])

    def step():
        eng.vdaggerv_build(precision)
        out = eng.contract(gd.plan_ptr, precision, 0, args.single_block_pair)
        return out

    upload()
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
    stage = np.zeros(4)
    launches = 0
    wall0 = time.time()
    for _ in range(args.steps):
        step()
        tim = eng.timings()
        stage += tim[:4]
        launches += int(tim[5])
    wall = time.time() - wall0
    clocks = sampler.stop()
    dev_s = stage.sum() / 1e3 / args.steps
    dev_s = max_over_ranks(dist, dev_s)

    # ---- end to end from host buffers
    barrier(dist)
    e2e0 = time.time()
    for _ in range(args.steps):
        upload()
        step()
    e2e = max_over_ranks(dist, (time.time() - e2e0) / args.steps)
    h2d = sum(v.nbytes for v in V) + sum(p.nbytes for p in peram) + noise.nbytes
    d2h = out.nbytes

    stats = eng.stats()
    n_ops = gd.plan.n_vdv_ops - (1 if gd.plan.index_of_unity >= 0 else 0)
    vdv_flops = w.flops_vdaggerv(n_ops)
    stage_ms = stage / args.steps
    peaks = load_peaks()
    # Dominant stage and its roofline.
    names = ["vdaggerv", "factors", "products_traces", "assembly"]
    flops = [vdv_flops, stats[4], stats[5], 0.0]
    dom = int(np.argmax(stage_ms))
    achieved = flops[dom] / (stage_ms[dom] / 1e3) / 1e12 if stage_ms[dom] > 0 else 0.0
    fp64_peak = args.fp64_peak_tflops
    roofline = {
        "kernel": names[dom], "bound": "fp64", "achieved": achieved,
        "peak": fp64_peak, "unit": "TFLOP/s", "frac": achieved / fp64_peak if fp64_peak else None,
        "peak_source": "fp64 rate quoted for GB300 (not in MEASURED_PEAKS.json)",
        "traffic": None,
    }
    if precision == 1 and dom == 0 and peaks:
        roofline.update(bound="tensor", peak=peaks["bf16_tflops"],
                        peak_source="MEASURED_PEAKS.json bf16_tflops (of measured)")
    line = {
        "metric": METRIC, "value": dev_s * world / world, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_s * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if precision == 0 else "bf16-ozaki+f64", "data": "synthetic",
        "config": {"workload": w.name, "lattice": f"{w.L}^3x{w.Lt}", "nev": w.nev,
                   "n_rnd": w.n_rnd, "dilution": f"TB{w.dilT} EI{w.dilE} DF4",
                   "diagrams": sorted({c.split(':')[0] for c in w.correlators}),
                   "n_correlators": int(out.shape[0]), "precision": args.precision,
                   "single_block_pair": args.single_block_pair,
                   "l2": "inputs larger than L2 (eigenvectors alone exceed 129 MB)",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": launches,
        "stages_ms": dict(zip(names, map(float, stage_ms))),
        "work": {"vdaggerv_tflop": vdv_flops / 1e12, "factor_tflop": stats[4] / 1e12,
                 "product_trace_tflop": stats[5] / 1e12, "factors": stats[0],
                 "products": stats[1], "trace_entries": stats[2], "terms": stats[3]},
        "planning_s": plan_s, "first_step_s": first, "input_generation_s": t_gen,
        "roofline": roofline, "clocks": clocks,
    }
    if rank == 0 and not args.no_cpu_baseline and world == 1:
        line["cpu_baseline"] = cpu_baseline(w, gd, args)
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def cpu_baseline(w, gd, args):
    """The oracle (the reference's algorithm restated, OpenMP on all host
    cores) on a bounded sample, extrapolated to one configuration."""
    import oracle
    oracle.build_oracle.build()
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    dims = gd.dims
    # VdaggerV on a few timeslices, scaled by Lt.
    nt = max(1, min(w.Lt, args.cpu_vdv_timeslices))
    ts = list(range(nt))
    V = [w.eigenvectors(t) if t < nt else None for t in range(w.Lt)]
    t0 = time.time()
    oracle.vdaggerv(dims, gd.plan, V, ts=ts)
    vdv_s = (time.time() - t0) * w.Lt / nt
    return {"value": vdv_s, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"VdaggerV on {nt} of {w.Lt} timeslices, scaled by {w.Lt}/{nt}; "
                      "contraction stage not included (lower bound)"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from slaph_gb300 import GlobalData, synthetic
    w = synthetic.CONFIGS[args.workload]
    gd = GlobalData.from_infile(w.write_infile())
    vals = []
    for _ in range(args.warmup + args.steps):
        cb = cpu_baseline(w, gd, args)
        vals.append(cb["value"])
    v = float(np.mean(vals[args.warmup:])) if args.steps else float(vals[-1])
    cb["value"] = v
    print(json.dumps({
        "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": v * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "impl": "reference",
        "config": {"workload": w.name, "lattice": f"{w.L}^3x{w.Lt}", "nev": w.nev},
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
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--single-block-pair", type=int, default=-1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-vdv-timeslices", type=int, default=1)
    ap.add_argument("--fp64-peak-tflops", type=float, default=1.25)
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_engine(args)


if __name__ == "__main__":
    main()
