"""Benchmark: LES cell-steps/s of the GB300 solver on the plain single large domain.

Workload (the configuration the headline metric is quoted on): one urban domain of
600 x 600 x 90 cells, FP32, dx = dy = 4 m, dz = 2 m stretched by 1.04, seeded
rectangular-block buildings (30 % plan coverage), power-law inflow with +-1e-3 m/s
noise, dt = 0.05 s, 50 red-black SOR iterations per step.  A "step" is one full time
step of the reference's solver loop (velnw .. press).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--dims IMxJMxKM] [--no-cpu]

--dims runs a smaller domain of the same kind (profiling captures: ncu wants a small
case); --no-cpu skips the CPU baseline leg.  The headline line uses the defaults.

One JSON line on stdout (rank 0).  Under torchrun each rank advances its own
independent domain (replicas; the single domain does not shard without a halo
exchange), so per-GPU work is fixed as N grows ("scaling": "weak").

--impl reference times the CPU restatement of the reference's les_main (the oracle:
the Fortran reference cannot be compiled on this image, there is no Fortran
compiler) on the host cores, on a bounded sample of the same workload.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "mpi-les_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "LES cell-steps/s"
UNIT = "cell-steps/s"
IM, JM, KM = 600, 600, 90
SOR_ITERS = 50
# algorithmic bytes per cell-step at 50 SOR iterations (each stage's distinct 3-D arrays
# read once and written once; SOR 12 B per cell and iteration)
BYTES_PER_CELL_STEP = 869.0
SOR_BYTES_PER_CELL_ITER = 12.0


def workload_config(im=IM, jm=JM, km=KM):
    return {"workload": f"plain single domain {im}x{jm}x{km} FP32, 50 red-black SOR iterations/step",
            "im": im, "jm": jm, "km": km, "dx_m": 4.0, "dz0_m": 2.0, "dz_ratio": 1.04,
            "buildings": "seeded rectangular blocks, 30% plan coverage, 5-20 cells, 10-60 m",
            "inflow": "5 m/s*(z/100 m)^0.2 + uniform +-1e-3 m/s", "dt_s": 0.05, "sor_iters": SOR_ITERS,
            "l2": "inputs larger than L2 (about 3.8 GB of fields per domain)"}


def scenario(seed=1, im=IM, jm=JM, km=KM):
    import lesgpu
    return lesgpu.Scenario(im=im, jm=jm, km=km, seed=seed)


def read_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        return float(pk["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def read_traffic_per_cell(kernel: str):
    """DRAM bytes per cell and launch of a kernel, from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return float(json.load(f)[kernel]["dram_bytes_per_cell"])
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons while the timed region runs."""

    def __init__(self, dev: int):
        self.dev = dev
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "100", "-i", str(self.dev)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
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
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() in ("active", "0x1") or v == "Active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend="nccl" if os.environ.get("LES_BENCH_GLOO") is None else "gloo")
        pg = dist
    return world, rank, local, pg


def reduce_max(pg, x: float) -> float:
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def cpu_baseline_sample(threads: int | None = None, im=150, jm=150, km=90, steps=3):
    """Time the oracle (CPU restatement of les_main's solver) on a bounded sample."""
    import lesgpu
    from oracle import ref as oref
    sc = scenario(seed=1, im=im, jm=jm, km=km)
    zbm, uin, vin, win = lesgpu.generate_scenario(sc)
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    r = oref.Ref(4, im, jm, km, zbm, uin, vin, win, sqrt_half=0, red64=0, fast=True)
    r.step(1, steps + 1)  # warm-up (n == 1 fill)
    t0 = time.perf_counter()
    for n in range(2, steps + 2):
        r.step(n, steps + 1)
    dt = time.perf_counter() - t0
    r.close()
    return im * jm * km * steps / dt, f"{steps} steps of {im}x{jm}x{km} after 1 warm-up step, {dt:.1f} s"


def run_reference(args):
    world, rank, local, pg = dist_setup()
    if rank != 0:
        return 0
    from oracle import ref as oref
    oref.build()
    import lesgpu
    threads = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(threads)
    # one "step" = one oracle time step on a 300x300x90 sample of the workload's domain
    im, jm, km = 300, 300, 90
    sc = scenario(seed=1, im=im, jm=jm, km=km)
    zbm, uin, vin, win = lesgpu.generate_scenario(sc)
    r = oref.Ref(4, im, jm, km, zbm, uin, vin, win, sqrt_half=0, red64=0, fast=True)
    n = 1
    for _ in range(args.warmup):
        r.step(n, 10**6)
        n += 1
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r.step(n, 10**6)
        n += 1
    dt = time.perf_counter() - t0
    val = im * jm * km * args.steps / dt
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": workload_config(),
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"each step: one oracle time step on a {im}x{jm}x{km} sample of the domain"},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    world, rank, local, pg = dist_setup()
    import numpy as np
    import torch
    torch.cuda.set_device(local)
    import lesgpu
    if not os.path.exists(lesgpu.LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()
    IM, JM, KM = args.dims
    cells = IM * JM * KM
    dom = lesgpu.Domain(IM, JM, KM, lesgpu.Params())
    dom.setup_scenario(scenario(seed=1 + rank, im=IM, jm=JM, km=KM))
    stream = torch.cuda.ExternalStream(dom.stream())
    nmax = args.warmup + args.steps + 10**6
    n = 1
    for _ in range(args.warmup):
        dom.step(n, nmax)
        n += 1
    dom.sync()
    if pg is not None:
        pg.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = dom.launch_count()
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            dom.step(n, nmax)
            n += 1
        ev1.record(stream)
        ev1.synchronize()
    torch.cuda.synchronize()
    launches = dom.launch_count() - l0
    ms = ev0.elapsed_time(ev1)
    ms_max = reduce_max(pg, ms)
    value = world * cells * args.steps / (ms_max / 1e3)
    bad = dom.nonfinite()

    # ---- end to end through the C-ABI with host buffers -----------------------------
    # each step: upload the step's inflow planes (a time-varying inflow, as bondv1 would
    # receive it) from pinned host memory, run the step, and read back the interior
    # u, v, w, p that the reference's per-step output routines consume (main.f95:311-327)
    e2e_steps = max(3, min(args.steps, 20))
    zbm, uin, vin, win = lesgpu.generate_scenario(scenario(seed=1 + rank, im=IM, jm=JM, km=KM))
    pin = [torch.from_numpy(np.asfortranarray(a).ravel(order="F").copy()).pin_memory() for a in (uin, vin, win)]
    outs = [torch.empty((KM, JM, IM), dtype=torch.float32).pin_memory() for _ in range(4)]
    lbi, ubi = (1, 1, 0), (JM, KM, 0)
    lb, ub = (1, 1, 1), (IM, JM, KM)
    import ctypes as C
    lib = dom.lib
    iarr = lambda t: (C.c_int * 3)(*t)
    fptr = lambda t: C.cast(t.data_ptr(), C.POINTER(C.c_float))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for fid, t in zip((lesgpu.UIN, lesgpu.VIN, lesgpu.WIN), pin):
            dom._check(lib.les_gpu_upload(dom._h, fid, fptr(t), iarr(lbi), iarr(ubi)), "upload inflow")
        dom.step(n, nmax)
        n += 1
        for fid, t in zip((lesgpu.U, lesgpu.V, lesgpu.W, lesgpu.P), outs):
            dom._check(lib.les_gpu_download(dom._h, fid, fptr(t), iarr(lb), iarr(ub)), "download")
    e2e_s = time.perf_counter() - t0
    e2e_s = reduce_max(pg, e2e_s)
    e2e_val = world * cells * e2e_steps / e2e_s
    h2d = 3 * JM * KM * 4
    d2h = 4 * cells * 4

    # ---- dominant kernel: one SOR iteration, timed alone ----------------------------
    reps = 100
    sor_ms = dom.profile(lesgpu.PROF_SOR, reps)
    peak, peak_kind = read_peaks()
    alg = SOR_BYTES_PER_CELL_ITER * cells
    achieved = alg / (sor_ms / 1e3) / 1e9
    tpc = read_traffic_per_cell("sor")
    roofline = {"bound": "hbm", "kernel": "SOR iteration (red+black sweep of press)", "achieved": achieved,
                "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                "traffic": (tpc * cells) if tpc else None, "ms_per_launch": sor_ms,
                "alg_bytes_per_launch": alg,
                "step_alg_GBps": BYTES_PER_CELL_STEP * cells / (ms / args.steps / 1e3) / 1e9,
                "step_frac": BYTES_PER_CELL_STEP * cells / (ms / args.steps / 1e3) / 1e9 / peak}
    dom.close()

    line = None
    if rank == 0:
        cpu = None
        if not args.no_cpu:
            try:
                cv, sample = cpu_baseline_sample(threads=1)
                cpu = {"value": cv, "unit": UNIT, "cores": 1, "kind": "port", "sample": sample}
            except Exception as e:  # the baseline must not sink the GPU line
                cpu = {"value": None, "unit": UNIT, "cores": 1, "kind": "port", "sample": f"failed: {e}"}
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic: seeded urban heightmap and power-law inflow (no dataset in the reference)",
                "config": workload_config(IM, JM, KM), "clocks": clk.summary(),
                "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                        "steps": e2e_steps},
                "gpu_launches": launches, "nonfinite": bad, "roofline": roofline, "cpu_baseline": cpu}
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.barrier()
        pg.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--dims", default=f"{IM}x{JM}x{KM}", help="domain IMxJMxKM (default: the workload's)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    args = ap.parse_args()
    args.dims = tuple(int(x) for x in args.dims.lower().split("x"))
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
