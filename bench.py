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

Besides the headline, the line carries the batched ensembles: "batched" (64 domains of
150x150x90, each with its own building seed, inflow direction in [0, 360) and speed in
[2, 10] m/s, stepped together; against one 150x150x90 domain alone) and "uneven" (96
domains with ip, jp in {64..256}, kp in {48, 64, 90}, coverage 15-45%; against the
same domains run one by one).  --mode serve runs the serving stream instead (Poisson
arrivals of such scenarios, 50-500 steps each) and prints its own line with p50/p99
completion latency and an FP64-oracle check of sampled requests.

One JSON line on stdout (rank 0).  Under torchrun each rank advances its own
independent domain (replicas; the single domain does not shard without a halo
exchange), so per-GPU work is fixed as N grows ("scaling": "weak").

--impl reference times the CPU restatement of the reference's les_main (the oracle:
the Fortran reference cannot be compiled on this image, there is no Fortran
compiler) on the host cores, on the same 600x600x90 workload, with inputs from the
oracle's own scenario generator (the GPU library is not loaded).
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


def oracle_domain(im=IM, jm=JM, km=KM, seed=1, prec=4, threads=None):
    """The workload's domain in the oracle's fast build (gfortran semantics: x**0.5 as
    powf, FP32 sums), its inputs made by the oracle's own scenario generator -- nothing
    of the GPU product is loaded.  Returns (Ref, threads in use)."""
    from oracle import ref as oref
    zbm, uin, vin, win = oref.scenario(im, jm, km, seed, fast=True)
    used = oref.set_threads(threads or (os.cpu_count() or 1))
    r = oref.Ref(prec, im, jm, km, zbm, uin, vin, win, sqrt_half=0, red64=0, fast=True)
    return r, used


STAGE_ORDER = ("velnw", "bondv1", "velfg", "feedbf", "les", "adam", "press")


def timed_oracle_steps(r, n0, steps, nmax):
    """Steps n0 .. n0+steps-1 of the oracle, each of the seven subroutines of main.f95's
    order timed (the oracle's step() is exactly this sequence).  Returns (seconds,
    seconds per step of each subroutine)."""
    from oracle import ref as oref
    ids = dict(zip(STAGE_ORDER, (oref.VELNW, oref.BONDV1, oref.VELFG, oref.FEEDBF, oref.LES, oref.ADAM, oref.PRESS)))
    per = {nm: 0.0 for nm in STAGE_ORDER}
    t0 = time.perf_counter()
    for n in range(n0, n0 + steps):
        for nm in STAGE_ORDER:
            ts = time.perf_counter()
            r.stage(ids[nm], n, nmax)
            per[nm] += time.perf_counter() - ts
    dt = time.perf_counter() - t0
    return dt, {nm: round(v / steps, 6) for nm, v in per.items()}


def cpu_baseline_sample(threads: int | None = None, im=150, jm=150, km=90, steps=25):
    """Time the oracle (CPU restatement of les_main's solver) on a bounded sample."""
    r, used = oracle_domain(im, jm, km, threads=threads)
    r.step(1, steps + 1)  # warm-up (n == 1 fill)
    dt, per_step = timed_oracle_steps(r, 2, steps, steps + 1)
    r.close()
    return (im * jm * km * steps / dt, f"{steps} steps of {im}x{jm}x{km} after 1 warm-up step, {dt:.1f} s", used,
            per_step)


def run_reference(args):
    """The reference's CPU path on this host: the oracle's fast build (the Fortran
    reference cannot be compiled here: no Fortran compiler) on the workload's own
    600x600x90 domain, all host threads (OpenMP over k planes, the role les_main_mpi's
    decomposition plays), then the same domain on one thread (les_main's role) for a few
    steps beside it.  Under torchrun only rank 0 runs; the other ranks exit at once."""
    if int(os.environ.get("RANK", "0")) != 0:
        return 0
    from oracle import ref as oref
    oref.build()
    im, jm, km = args.dims  # the workload's 600x600x90 unless --dims says otherwise
    cells = im * jm * km
    nmax = args.warmup + args.steps + 10**6
    r, threads = oracle_domain(im, jm, km)
    n = 1
    for _ in range(args.warmup):
        r.step(n, nmax)
        n += 1
    dt, per_step = timed_oracle_steps(r, n, args.steps, nmax)
    n += args.steps
    val = cells * args.steps / dt
    # one thread, the same domain and state, a few steps
    one_steps = 2
    used1 = oref.set_threads(1)
    dt1, per1 = timed_oracle_steps(r, n, one_steps, nmax)
    r.close()
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: seeded urban heightmap and power-law inflow (the oracle's own generator)",
            "config": workload_config(im, jm, km),
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"each step: one full time step of the {im}x{jm}x{km} domain "
                                       f"(the configuration named in config), {threads} threads",
                             "stage_s_per_step": per_step},
            "single_core": {"value": cells * one_steps / dt1, "unit": UNIT, "cores": used1,
                            "sample": f"{one_steps} further steps of the same {im}x{jm}x{km} domain on one thread "
                                      "(les_main's role)", "stage_s_per_step": per1},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def parity_check(im, jm, km, nsteps=5):
    """A fresh domain of the benchmark's kind stepped nsteps times on the GPU and in the
    FP64 oracle (the reference built with -freal-4-real-8, all host threads): the max
    relative error max|x - x64| / max|x64| of the interior u, v, w, p (contract 1e-4)."""
    import lesgpu
    from oracle import ref as oref
    sc = scenario(seed=1, im=im, jm=jm, km=km)
    d = lesgpu.Domain(im, jm, km, lesgpu.Params())
    d.setup_scenario(sc)
    for n in range(1, nsteps + 1):
        d.step(n, nsteps)
    d.sync()
    lo, hi = (1, 1, 1), (im, jm, km)
    got = {nm: d.download(fid, lo, hi) for nm, fid in (("u", lesgpu.U), ("v", lesgpu.V), ("w", lesgpu.W),
                                                        ("p", lesgpu.P))}
    d.close()
    t0 = time.perf_counter()
    zbm, uin, vin, win = oref.scenario(im, jm, km, 1, fast=True)
    threads = oref.set_threads(os.cpu_count() or 1)
    r = oref.Ref(8, im, jm, km, zbm, uin, vin, win, sqrt_half=0, red64=1, fast=True)
    for n in range(1, nsteps + 1):
        r.step(n, nsteps)
    errs = {}
    for nm, fid in (("u", lesgpu.U), ("v", lesgpu.V), ("w", lesgpu.W), ("p", lesgpu.P)):
        o = r.get(fid, lo, hi)
        errs[nm] = float(abs(got[nm].astype("float64") - o).max() / max(float(abs(o).max()), 1e-30))
    r.close()
    return {"max_rel_err": max(errs.values()), "per_field": errs, "tolerance": 1e-4,
            "against": f"FP64 oracle, {nsteps} steps of {im}x{jm}x{km} from rest, {threads} host threads, "
                       f"{time.perf_counter() - t0:.1f} s"}


def _seconds_synced(fn):
    t0 = time.perf_counter()
    fn()
    return time.perf_counter() - t0


def ensemble(specs, warmup, steps, params=None, persistent=False):
    """Step scenarios together in one batch; returns (cell-steps/s, seconds per step).
    Timed on the host between full device synchronisations (the members run on many
    streams).  persistent: SOR iterations 2..nmaxp of all members in one persistent
    launch over their tiles (les_batch_set_sor_launch)."""
    import lesgpu
    params = params or lesgpu.Params()
    doms = []
    for sc in specs:
        d = lesgpu.Domain(sc.im, sc.jm, sc.km, params)
        d.setup_scenario(sc)
        doms.append(d)
    # SOR tile shape per size class, measured with the GPU shared (before any timing)
    lesgpu.tune_classes(doms, shared=True)
    b = lesgpu.Batch(persistent_sor=persistent)
    for d in doms:
        b.add(d, 1, 10**6)
    for _ in range(warmup):
        b.step()
    b.sync()
    dt = _seconds_synced(lambda: ([b.step() for _ in range(steps)], b.sync()))
    cells = sum(sc.im * sc.jm * sc.km for sc in specs)
    bad = sum(d.nonfinite() for d in doms)
    b.close()
    for d in doms:
        d.close()
    return cells * steps / dt, dt / steps, bad


def one_by_one(specs, warmup, steps, params=None):
    """The same scenarios on the plain path, one domain after the other."""
    import lesgpu
    params = params or lesgpu.Params()
    total_t, work = 0.0, 0
    for sc in specs:
        d = lesgpu.Domain(sc.im, sc.jm, sc.km, params)
        d.setup_scenario(sc)
        lesgpu.tune_classes([d], shared=False)  # the plain path's SOR shape, measured alone
        for n in range(1, warmup + 1):
            d.step(n, 10**6)
        d.sync()
        total_t += _seconds_synced(lambda: ([d.step(n, 10**6) for n in range(warmup + 1, warmup + steps + 1)],
                                            d.sync()))
        work += sc.im * sc.jm * sc.km * steps
        d.close()
    return work / total_t


def uniform_specs(count=64, seed=2024, im=150, jm=150, km=90):
    import random

    import lesgpu
    rng = random.Random(seed)
    return [lesgpu.Scenario(im=im, jm=jm, km=km, seed=rng.getrandbits(48), direction_deg=rng.uniform(0.0, 360.0),
                            u_ref=rng.uniform(2.0, 10.0)) for _ in range(count)]


def uneven_specs(count=96, seed=2025):
    import random

    import lesgpu
    rng = random.Random(seed)
    sizes, kms = (64, 96, 128, 192, 256), (48, 64, 90)
    return [lesgpu.Scenario(im=rng.choice(sizes), jm=rng.choice(sizes), km=rng.choice(kms), seed=rng.getrandbits(48),
                            coverage=rng.uniform(0.15, 0.45), direction_deg=rng.uniform(0.0, 360.0),
                            u_ref=rng.uniform(2.0, 10.0)) for _ in range(count)]


def batched_lines(warmup=3, steps=10):
    """The two ensemble measurements carried by the headline line."""
    uni = uniform_specs()
    v_batch, s_step, bad = ensemble(uni, warmup, steps)
    v_pers, s_pers, bad_p = ensemble(uni, warmup, steps, persistent=True)
    v_alone = one_by_one(uni[:1], warmup, steps)
    batched = {"value": v_batch, "unit": UNIT, "ms_per_step": 1e3 * s_step, "nonfinite": bad + bad_p,
               "workload": "64 domains of 150x150x90, own building seed, inflow direction U[0,360), speed U[2,10] m/s",
               "plain_small_value": v_alone, "vs_plain_small": v_batch / v_alone,
               "persistent_sor": {"value": v_pers, "ms_per_step": 1e3 * s_pers, "vs_plain_small": v_pers / v_alone,
                                  "launch": "SOR iterations 2..nmaxp of all members in one persistent launch over "
                                            "their tile work-list"},
               "timing": "host clock between device synchronisations, after warm-up"}
    une = uneven_specs()
    v_ub, s_ub, bad_u = ensemble(une, warmup, steps)
    v_up, s_up, bad_up = ensemble(une, warmup, steps, persistent=True)
    v_obo = one_by_one(une, warmup, 3)
    uneven = {"value": v_ub, "unit": UNIT, "ms_per_step": 1e3 * s_ub, "nonfinite": bad_u + bad_up,
              "workload": "96 domains, ip, jp in {64,96,128,192,256}, kp in {48,64,90}, coverage U[15,45]%",
              "cells": sum(sc.im * sc.jm * sc.km for sc in une), "one_by_one_value": v_obo,
              "vs_one_by_one": v_ub / v_obo,
              "persistent_sor": {"value": v_up, "ms_per_step": 1e3 * s_up, "vs_one_by_one": v_up / v_obo}}
    return batched, uneven


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
    if args.sor_shape:
        dom.set_sor_shape(*(int(x) for x in args.sor_shape.lower().split("x")))
        sor_shape, sor_tuned_us = dom.sor_shape(), None
    else:
        sor_shape, sor_tuned_us, _ = dom.tune_sor(False)  # measured SOR tile shape (untimed set-up)
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
    # u, v, w, p that the reference's per-step output routines consume (main.f95:311-327).
    # The read-back is les_gpu_download_async into pinned buffers (two sets, alternating):
    # the step's fields are snapshotted in stream order and copied while the next step
    # runs; step n's copies are waited for after step n+1 is queued, the last ones before
    # the clock stops.  Three windows of e2e_steps steps are timed; the line reports the
    # median window (host-side effects make single short windows vary by 10%).
    e2e_steps = max(3, min(args.steps, 20))
    zbm, uin, vin, win = lesgpu.generate_scenario(scenario(seed=1 + rank, im=IM, jm=JM, km=KM))
    pin = [torch.from_numpy(np.asfortranarray(a).ravel(order="F").copy()).pin_memory() for a in (uin, vin, win)]
    outs = [[torch.empty((KM, JM, IM), dtype=torch.float32).pin_memory() for _ in range(4)] for _ in range(2)]
    lbi, ubi = (1, 1, 0), (JM, KM, 0)
    lb, ub = (1, 1, 1), (IM, JM, KM)
    import ctypes as C
    lib = dom.lib
    iarr = lambda t: (C.c_int * 3)(*t)
    fptr = lambda t: C.cast(t.data_ptr(), C.POINTER(C.c_float))
    windows = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        prev = []
        for q in range(e2e_steps):
            for fid, t in zip((lesgpu.UIN, lesgpu.VIN, lesgpu.WIN), pin):
                dom._check(lib.les_gpu_upload(dom._h, fid, fptr(t), iarr(lbi), iarr(ubi)), "upload inflow")
            dom.step(n, nmax)
            n += 1
            cur = []
            for fid, t in zip((lesgpu.U, lesgpu.V, lesgpu.W, lesgpu.P), outs[q % 2]):
                tk = C.c_longlong(-1)
                dom._check(lib.les_gpu_download_async(dom._h, fid, fptr(t), iarr(lb), iarr(ub), C.byref(tk)),
                           "download")
                cur.append(tk.value)
            for tk in prev:  # the previous step's fields are now in host memory
                dom._check(lib.les_gpu_download_wait(dom._h, tk), "download_wait")
            prev = cur
        for tk in prev:
            dom._check(lib.les_gpu_download_wait(dom._h, tk), "download_wait")
        windows.append(reduce_max(pg, time.perf_counter() - t0))
    e2e_s = sorted(windows)[1]
    e2e_val = world * cells * e2e_steps / e2e_s
    h2d = 3 * JM * KM * 4
    d2h = 4 * cells * 4

    # ---- dominant kernel: the fused SOR sweep (49 of a step's 50 iterations), its
    # launches timed with CUDA events on the handle's stream inside passes run as the
    # step runs them ------------------------------------------------------------------
    sweep_ms = dom.profile(lesgpu.PROF_SOR_SWEEP, 4)
    # the other passes of the step, each timed alone with CUDA events on the handle's stream
    stage_ms = {"velnw": dom.profile(lesgpu.PROF_VELNW, 20), "velfg+feedbf": dom.profile(lesgpu.PROF_VELFG, 20),
                "les+adam": dom.profile(lesgpu.PROF_LES, 20), "sor_sweep": sweep_ms,
                "sor_per_iteration_with_first": dom.profile(lesgpu.PROF_SOR, 20),
                "step": dom.profile(lesgpu.PROF_STEP, 10)}
    peak, peak_kind = read_peaks()
    alg = SOR_BYTES_PER_CELL_ITER * cells
    achieved = alg / (sweep_ms / 1e3) / 1e9
    tpc = read_traffic_per_cell("sor")
    roofline = {"bound": "hbm", "kernel": "k_sor_tma: fused red+black SOR sweep of press (49 launches per step)",
                "achieved": achieved,
                "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                "traffic": (tpc * cells) if tpc else None, "ms_per_launch": sweep_ms,
                "alg_bytes_per_launch": alg,
                "sor_tile": {"nx": sor_shape[0], "ny": sor_shape[1], "kchunk": sor_shape[2],
                             "depth": sor_shape[3],
                             "tuner_us": sor_tuned_us},
                "stages_ms": stage_ms,
                "step_alg_GBps": BYTES_PER_CELL_STEP * cells / (ms / args.steps / 1e3) / 1e9,
                "step_frac": BYTES_PER_CELL_STEP * cells / (ms / args.steps / 1e3) / 1e9 / peak}
    dom.close()

    line = None
    parity = None
    if rank == 0 and not args.no_parity:
        try:
            parity = parity_check(IM, JM, KM)
        except Exception as e:  # the check must not sink the GPU line
            parity = {"failed": str(e)}
    if rank == 0:
        cpu = None
        if not args.no_cpu:
            try:
                cv, sample, used, per_step = cpu_baseline_sample(threads=1)
                cpu = {"value": cv, "unit": UNIT, "cores": used, "kind": "port", "sample": sample,
                       "stage_s_per_step": per_step}
            except Exception as e:  # the baseline must not sink the GPU line
                cpu = {"value": None, "unit": UNIT, "cores": 1, "kind": "port", "sample": f"failed: {e}"}
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic: seeded urban heightmap and power-law inflow (no dataset in the reference)",
                "config": workload_config(IM, JM, KM), "clocks": clk.summary(),
                "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                        "steps": e2e_steps, "windows_ms_per_step": [1e3 * w / e2e_steps for w in windows],
                        "window": "median of three windows",
                        "read_back": "les_gpu_download_async of interior u, v, w, p every step (snapshot in "
                                     "stream order, copy overlapping the next step), all waited for"},
                "gpu_launches": launches, "nonfinite": bad, "roofline": roofline, "cpu_baseline": cpu,
                "parity": parity}
        if not args.no_batch:
            try:
                line["batched"], line["uneven"] = batched_lines()
            except Exception as e:  # the ensembles must not sink the headline line
                line["batched"] = {"failed": str(e)}
        if not args.no_serve:
            pool = oracle_pool()  # FP64 checks of served requests (spawned: safe with the GPU in use)
            try:
                line["serve"] = serve_lines(pool)
            except Exception as e:  # the serving run must not sink the headline line
                line["serve"] = {"failed": str(e)}
            pool.close()
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.barrier()
        pg.destroy_process_group()
    return 0


def _oracle_check(job):
    """Oracle runs of one served scenario to its final step (in a spawned worker process;
    the scenario comes from the oracle's own generator): the max relative error of the
    GPU's final u, v, w, p against the FP64 oracle and against the FP32 restatement with
    the GPU's arithmetic (IEEE x**0.5, FP64-accurate sums), and the FP32 restatement's
    own distance from FP64 -- the drift of the reference's precision over the run, which
    on long chaotic runs alone exceeds 1e-4."""
    sc_kw, nsteps, gpu_fields = job
    import numpy as np

    from oracle import ref as oref
    oref.set_threads(2)
    zbm, uin, vin, win = oref.scenario(fast=True, **sc_kw)
    im, jm, km = sc_kw["im"], sc_kw["jm"], sc_kw["km"]
    kw = dict(dx=sc_kw["dx"], dy=sc_kw["dy"], dz_law=sc_kw["dz_law"], dz0=sc_kw["dz0"], dz_ratio=sc_kw["dz_ratio"],
              fast=True)
    r64 = oref.Ref(8, im, jm, km, zbm, uin, vin, win, sqrt_half=0, red64=1, **kw)
    r32 = oref.Ref(4, im, jm, km, zbm, uin, vin, win, sqrt_half=1, red64=1, **kw)
    for n in range(1, nsteps + 1):
        r64.step(n, nsteps)
        r32.step(n, nsteps)

    def rel(a, b):
        return float(np.abs(a.astype(np.float64) - b).max() / max(np.abs(b).max(), 1e-30))

    out = {"gpu_vs_fp64": 0.0, "gpu_vs_fp32": 0.0, "fp32_vs_fp64": 0.0}
    for fid, g in gpu_fields.items():
        o64 = r64.get(fid, (1, 1, 1), (im, jm, km))
        o32 = r32.get(fid, (1, 1, 1), (im, jm, km))
        out["gpu_vs_fp64"] = max(out["gpu_vs_fp64"], rel(g, o64))
        out["gpu_vs_fp32"] = max(out["gpu_vs_fp32"], rel(g, o32))
        out["fp32_vs_fp64"] = max(out["fp32_vs_fp64"], rel(o32, o64))
    r64.close()
    r32.close()
    out["steps"] = nsteps
    out["cells"] = im * jm * km
    return out


def oracle_pool():
    """Worker processes for the FP64 checks of served requests (spawned: safe after the
    GPU is in use), two threads each over the host cores."""
    import multiprocessing as mp
    return mp.get_context("spawn").Pool(processes=max(1, min(8, (os.cpu_count() or 2) // 2)))


def serve_window(rate, seconds, seed, pool, sample_every=20, max_check=None):
    """One serving run: Poisson arrivals of wind scenarios at `rate` for `seconds`,
    admission by free HBM, continuous batching.  Every `sample_every`-th request (5 %)
    is checked against the FP64 oracle at its final step; the checks run on the host
    cores while the GPU keeps serving.  Returns (statistics, pending checks)."""
    import dataclasses

    import lesgpu
    import serve
    reqs = serve.poisson_requests(rate, seconds, seed=seed)
    be = serve.GpuBackend(reserve_bytes=8 << 30)
    sampled = {r.rid for r in reqs[::sample_every][:max_check]}
    checks = []

    def on_done(r, dom):
        if r.rid in sampled:
            fields = {fid: dom.download(fid, (1, 1, 1), (r.im, r.jm, r.km))
                      for fid in (lesgpu.U, lesgpu.V, lesgpu.W, lesgpu.P)}
            checks.append(pool.apply_async(_oracle_check, ((dataclasses.asdict(be.scenario(r)), r.steps, fields),)))

    t_tune = time.perf_counter()
    tuned = be.pretune(reqs)  # the SOR shape of each size class, with the GPU idle
    t_tune = time.perf_counter() - t_tune
    with ClockSampler(0) as clk:
        st = serve.Server(be, max_live=256, setup_workers=4, on_done=on_done).run(reqs)
    be.batch.close()
    st["clocks"] = clk.summary()
    st["rate_hz"] = rate
    st["window_s"] = seconds
    st["sor_tuning"] = {"classes": len(tuned), "seconds": t_tune}
    st["sampled"] = len(sampled)
    return st, checks


def serve_summary(st, checks):
    res = [c.get() for c in checks]
    keep = ("rate_hz", "window_s", "requests", "completed", "rejected", "wall_s", "drain_s", "cell_steps_per_s",
            "latency_s", "service_s", "queue_wait_s", "max_backlog", "mean_live_cells", "clocks")
    out = {k: st[k] for k in keep}
    g64 = [x["gpu_vs_fp64"] for x in res]
    out["oracle_check"] = {
        "requests": len(res), "max_rel_err": max(g64) if g64 else None, "tolerance": 1e-4,
        "within_tolerance": sum(1 for e in g64 if e <= 1e-4),
        "max_vs_fp32_restatement": max((x["gpu_vs_fp32"] for x in res), default=None),
        "reference_precision_drift": [{"steps": x["steps"], "cells": x["cells"], "gpu_vs_fp64": x["gpu_vs_fp64"],
                                       "fp32_vs_fp64": x["fp32_vs_fp64"]} for x in res],
        "sample": "every 20th request (5 percent); u, v, w, p at the request's final step vs the FP64 oracle and "
                  "vs the FP32 restatement; fp32_vs_fp64 is the reference precision's own distance from FP64 "
                  "over the same run"}
    return out


def serve_lines(pool):
    """The serving measurement carried by the headline line: the configuration's 20 req/s
    over a shortened 8 s arrival window (the offered load, about 8e9 cell-steps/s, is
    above what one GPU serves, so latency there is backlog), and 6 req/s over 12 s, a
    rate the GPU sustains, for the service latency; the full 120 s window is
    --mode serve."""
    a = serve_window(20.0, 8.0, 7, pool)
    b = serve_window(6.0, 12.0, 8, pool)
    return {"at_20hz": serve_summary(*a), "sustained": serve_summary(*b),
            "workload": "Poisson arrivals of wind scenarios, ip, jp in {64..256}, kp in {48,64,90}, 50-500 steps, "
                        "own seed, direction and speed; admission by free HBM, continuous batching",
            "latency": "completion latency = arrival to the end of the last step; service = admission to the end "
                       "of the last step; queue wait = arrival to admission"}


def run_serve(args):
    """The serving stream alone: Poisson arrivals, admission by free HBM, continuous batching."""
    pool = oracle_pool()
    import lesgpu
    if not os.path.exists(lesgpu.LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()
    st, checks = serve_window(args.rate, args.serve_seconds, 7, pool, max_check=args.check)
    summ = serve_summary(st, checks)
    pool.close()
    line = {"metric": METRIC, "mode": "serve", "value": st["cell_steps_per_s"], "unit": UNIT, "n_gpus": 1,
            "higher_is_better": True, "dtype": "f32", "data": "synthetic Poisson stream of seeded urban scenarios",
            "config": {"workload": f"serving: Poisson {args.rate} req/s for {args.serve_seconds} s, grids "
                                   "ip,jp in {64..256}, kp in {48,64,90}, 50-500 steps",
                       "rate_hz": args.rate, "window_s": args.serve_seconds}}
    line.update(summ)
    print(json.dumps(line), flush=True)
    return 0


def main():
    # many streams (batched ensembles): let them overlap; must precede CUDA start-up
    os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--dims", default=f"{IM}x{JM}x{KM}", help="domain IMxJMxKM (default: the workload's)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-ensemble measurements")
    ap.add_argument("--no-parity", action="store_true", help="skip the FP64-oracle check of a short run")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving measurement of the headline line")
    ap.add_argument("--sor-shape", default=None,
                    help="NXxNYxKCHUNK[xDEPTH]: fix the SOR tile shape (and iterations per k-march) instead of "
                         "tuning it (for runs under a profiler, whose timings would mislead the tuner)")
    ap.add_argument("--mode", default="plain", choices=["plain", "serve"])
    ap.add_argument("--serve-seconds", type=float, default=120.0, help="serve mode: arrival window")
    ap.add_argument("--rate", type=float, default=20.0, help="serve mode: requests per second")
    ap.add_argument("--check", type=int, default=None,
                    help="serve mode: check at most this many of the sampled requests vs FP64 (default: all)")
    args = ap.parse_args()
    args.dims = tuple(int(x) for x in args.dims.lower().split("x"))
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.mode == "serve":
        return run_serve(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
