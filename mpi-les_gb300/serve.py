"""Serving loop for wind-scenario solves: admission by free HBM, continuous batching.

A request is one urban wind scenario (grid, building seed, inflow direction and speed,
number of steps).  The server admits arrived requests while the device has memory
for their domain (``les_batch_admit``) and a slot is free, sets their domains up on
worker threads while the GPU keeps stepping the live ones, adds them to the batch
between steps, advances every live domain by one step per iteration
(``les_batch_step``: each member's step graph on its own stream, overlapping on the
GPU), and retires finished ones.  Completion latency runs from arrival to the end of
the request's last step.

The scheduling logic talks to a backend object, so it runs on the CPU with a fake
backend in the tests; ``GpuBackend`` is the real one.
"""
from __future__ import annotations

import concurrent.futures as cf
import dataclasses
import math
import random
import time
from collections import deque


@dataclasses.dataclass
class Request:
    rid: int
    arrival_s: float
    im: int
    jm: int
    km: int
    seed: int
    direction_deg: float
    u_ref: float
    coverage: float
    steps: int

    @property
    def cells(self) -> int:
        return self.im * self.jm * self.km


def poisson_requests(rate_hz: float, duration_s: float, seed: int = 0, sizes=(64, 96, 128, 192, 256),
                     kms=(48, 64, 90), steps=(50, 500), speed=(2.0, 10.0), coverage=(0.15, 0.45)) -> list[Request]:
    """Seeded Poisson arrivals; grids, coverage and speeds drawn as in the uneven-size
    ensemble (ip, jp from `sizes`, kp from `kms`)."""
    rng = random.Random(seed)
    out, t, rid = [], 0.0, 0
    while True:
        t += rng.expovariate(rate_hz)
        if t >= duration_s:
            return out
        out.append(Request(rid, t, rng.choice(sizes), rng.choice(sizes), rng.choice(kms), rng.getrandbits(48),
                           rng.uniform(0.0, 360.0), rng.uniform(*speed), rng.uniform(*coverage),
                           rng.randint(*steps)))
        rid += 1


def percentile(xs: list[float], q: float) -> float | None:
    if not xs:
        return None
    s = sorted(xs)
    k = max(0, min(len(s) - 1, int(math.ceil(q / 100.0 * len(s))) - 1))
    return s[k]


class GpuBackend:
    """The solver library: one Domain per request, members of one Batch."""

    def __init__(self, reserve_bytes: int = 4 << 30, params=None):
        import threading

        import lesgpu
        self.lesgpu = lesgpu
        self.batch = lesgpu.Batch()
        self.reserve = reserve_bytes
        # members share the GPU: their SOR march is never split (graphs captured during
        # set-up then match the batch's)
        self.params = params or lesgpu.Params(sor_ksplit=1)
        self.inflight = 0  # bytes of admitted domains whose set-up has not allocated yet
        self.lock = threading.Lock()

    def pretune(self, requests: list[Request]) -> dict:
        """Tune the SOR tile shape of every size class among `requests` for a shared GPU
        (les_gpu_tune_sor), before serving starts: tuning needs an otherwise idle GPU.
        One scratch domain per class; returns {(im, jm, km): (shape, us)}."""
        done = {}
        for r in requests:
            key = (r.im, r.jm, r.km)
            if key in done or self.lesgpu.sor_tuned(*key, True) is not None:
                continue
            d = self.lesgpu.Domain(r.im, r.jm, r.km, self.params)
            try:
                d.setup_scenario(self.scenario(r))
                shape, us, _ = d.tune_sor(True)
                done[key] = (shape, us)
            finally:
                d.close()
        return done

    def footprint(self, r: Request) -> int:
        return int(self.lesgpu.load_library().les_domain_bytes(r.im, r.jm, r.km))

    def admit(self, r: Request) -> bool:
        with self.lock:
            ok = self.lesgpu.Batch.admit(r.im, r.jm, r.km, self.reserve + self.inflight)
            if ok:
                self.inflight += self.footprint(r)
            return ok

    def scenario(self, r: Request):
        return self.lesgpu.Scenario(im=r.im, jm=r.jm, km=r.km, seed=r.seed, coverage=r.coverage, u_ref=r.u_ref,
                                    direction_deg=r.direction_deg)

    def create(self, r: Request):
        try:
            d = self.lesgpu.Domain(r.im, r.jm, r.km, self.params)
        finally:
            with self.lock:
                self.inflight -= self.footprint(r)
        d.setup_scenario(self.scenario(r))
        # the first two steps run here, on the domain's own stream: they capture the
        # domain's step graphs off the stepping thread
        d.pre = min(2, r.steps)
        for n in range(1, d.pre + 1):
            d.step(n, r.steps)
        d.sync()
        return d

    def add(self, dom, steps: int) -> int:
        return self.batch.add(dom, dom.pre + 1, steps)

    def step(self) -> int:
        live = self.batch.step()
        self.batch.sync()
        return live

    def done(self, slot: int) -> bool:
        n, nmax = self.batch.progress(slot)
        return n > nmax

    def remove(self, slot: int):
        return self.batch.remove(slot)

    def release(self, dom):
        dom.close()


class Server:
    def __init__(self, backend, max_live: int = 128, setup_workers: int = 4, on_done=None, on_step=None):
        self.be = backend
        self.max_live = max_live
        self.setup_workers = setup_workers
        self.on_done = on_done  # callback(request, domain) before a finished domain is released
        self.on_step = on_step  # callback({slot: (request, domain)}) after each batch step

    def run(self, requests: list[Request], clock=time.perf_counter, sleep=time.sleep) -> dict:
        """Serve the requests (arrival times relative to the start); returns statistics."""
        pending = deque(sorted(requests, key=lambda r: r.arrival_s))
        setups: dict[cf.Future, Request] = {}
        live: dict[int, tuple[Request, object]] = {}
        done_at: dict[int, float] = {}
        admitted_at: dict[int, float] = {}
        rejected: list[int] = []
        max_backlog, iters, step_cells = 0, 0, 0
        t0 = clock()
        pool = cf.ThreadPoolExecutor(max_workers=self.setup_workers)
        try:
            while pending or setups or live:
                now = clock() - t0
                # admit arrived requests while memory and slots allow (first come, first served);
                # a request that does not fit an idle device never will: refuse it
                while pending and pending[0].arrival_s <= now and len(live) + len(setups) < self.max_live:
                    if self.be.admit(pending[0]):
                        r = pending.popleft()
                        admitted_at[r.rid] = now
                        setups[pool.submit(self.be.create, r)] = r
                    elif not live and not setups:
                        rejected.append(pending.popleft().rid)
                    else:
                        break
                max_backlog = max(max_backlog, sum(1 for r in pending if r.arrival_s <= now))
                # domains whose set-up finished join the batch before the next step
                for fut in [f for f in setups if f.done()]:
                    r = setups.pop(fut)
                    dom = fut.result()
                    live[self.be.add(dom, r.steps)] = (r, dom)
                if live:
                    self.be.step()
                    iters += 1
                    step_cells += sum(r.cells for r, _ in live.values())
                    t_end = clock() - t0
                    if self.on_step:
                        self.on_step(live)
                    for slot in [s for s in live if self.be.done(s)]:
                        r, dom = live.pop(slot)
                        self.be.remove(slot)
                        done_at[r.rid] = t_end
                        if self.on_done:
                            self.on_done(r, dom)
                        self.be.release(dom)
                elif setups:
                    cf.wait(list(setups), timeout=0.05, return_when=cf.FIRST_COMPLETED)
                elif pending:
                    sleep(max(0.0, min(0.05, pending[0].arrival_s - (clock() - t0))))
        finally:
            pool.shutdown(wait=True)
        wall = clock() - t0
        lat = [done_at[r.rid] - r.arrival_s for r in requests if r.rid in done_at]
        wait = [admitted_at[r.rid] - r.arrival_s for r in requests if r.rid in admitted_at]
        # service time: from admission (set-up starts) to the end of the last step
        svc = [done_at[r.rid] - admitted_at[r.rid] for r in requests if r.rid in done_at]
        work = sum(r.cells * r.steps for r in requests if r.rid in done_at)
        last_arrival = max((r.arrival_s for r in requests), default=0.0)
        return {"requests": len(requests), "completed": len(done_at), "rejected": len(rejected), "wall_s": wall,
                "cell_steps": work, "cell_steps_per_s": work / wall if wall > 0 else None,
                "latency_s": {"p50": percentile(lat, 50), "p99": percentile(lat, 99), "max": max(lat) if lat else None},
                "queue_wait_s": {"p50": percentile(wait, 50), "p99": percentile(wait, 99)},
                "service_s": {"p50": percentile(svc, 50), "p99": percentile(svc, 99)},
                "drain_s": wall - last_arrival,
                "max_backlog": max_backlog, "batch_iterations": iters,
                "mean_live_cells": step_cells / iters if iters else 0}
