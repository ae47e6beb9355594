"""The serving scheduler (serve.Server) on the CPU, with a fake backend and clock.

The fake charges simulated time for each batch step in proportion to the live
cells, keeps a device-memory budget and records what the scheduler did, so the
admission and batching rules can be checked without a GPU.
"""
import threading

import pytest

import serve


class FakeClock:
    def __init__(self):
        self.t = 0.0
        self.lock = threading.Lock()

    def __call__(self):
        with self.lock:
            return self.t

    def advance(self, dt):
        with self.lock:
            self.t += dt

    def sleep(self, dt):
        self.advance(max(dt, 1e-4))


class FakeBackend:
    def __init__(self, clock, budget_cells, cost_per_cell=1e-9):
        self.clock = clock
        self.budget = budget_cells
        self.cost = cost_per_cell
        self.used = 0
        self.max_used = 0
        self.slots = {}
        self.next_slot = 0
        self.admitted = []
        self.max_members = 0
        self.lock = threading.Lock()

    def admit(self, r):
        with self.lock:
            ok = self.used + r.cells <= self.budget
            if ok:
                self.used += r.cells  # reserved at admission (set-up allocates)
                self.max_used = max(self.max_used, self.used)
                self.admitted.append(r.rid)
            return ok

    def create(self, r):
        return {"r": r, "n": 0}

    def add(self, dom, steps):
        s = self.next_slot
        self.next_slot += 1
        dom["steps"] = steps
        self.slots[s] = dom
        self.max_members = max(self.max_members, len(self.slots))
        return s

    def step(self):
        cells = sum(d["r"].cells for d in self.slots.values() if d["n"] < d["steps"])
        for d in self.slots.values():
            if d["n"] < d["steps"]:
                d["n"] += 1
        self.clock.advance(cells * self.cost + 1e-4)
        return sum(1 for d in self.slots.values() if d["n"] < d["steps"])

    def done(self, slot):
        d = self.slots[slot]
        return d["n"] >= d["steps"]

    def remove(self, slot):
        return self.slots.pop(slot)

    def release(self, dom):
        with self.lock:
            self.used -= dom["r"].cells


def test_poisson_requests_are_seeded_and_in_range():
    a = serve.poisson_requests(20.0, 10.0, seed=3)
    b = serve.poisson_requests(20.0, 10.0, seed=3)
    assert [(r.arrival_s, r.im, r.steps) for r in a] == [(r.arrival_s, r.im, r.steps) for r in b]
    assert 120 < len(a) < 280  # about 200 expected
    for r in a:
        assert r.im in (64, 96, 128, 192, 256) and r.jm in (64, 96, 128, 192, 256) and r.km in (48, 64, 90)
        assert 50 <= r.steps <= 500 and 0.0 <= r.direction_deg < 360.0 and 2.0 <= r.u_ref <= 10.0
    assert all(x.arrival_s < y.arrival_s for x, y in zip(a, a[1:]))


@pytest.mark.parametrize("budget_cells,max_live", [(40_000_000, 128), (8_000_000, 4)])
def test_server_admits_by_memory_and_completes_all(budget_cells, max_live):
    clock = FakeClock()
    be = FakeBackend(clock, budget_cells)
    reqs = serve.poisson_requests(20.0, 3.0, seed=5, steps=(5, 40))
    stats = serve.Server(be, max_live=max_live, setup_workers=2).run(reqs, clock=clock, sleep=clock.sleep)
    assert stats["completed"] == len(reqs)
    assert be.max_used <= budget_cells
    assert be.max_members <= max_live
    assert be.used == 0
    # first come, first served
    assert be.admitted == sorted(be.admitted)
    # no request completes before its own steps could have run
    assert stats["latency_s"]["p50"] > 0 and stats["latency_s"]["p99"] >= stats["latency_s"]["p50"]
    assert stats["cell_steps"] == sum(r.cells * r.steps for r in reqs)
    # latency = queue wait + service, reported apart
    assert 0 < stats["service_s"]["p50"] <= stats["service_s"]["p99"] <= stats["latency_s"]["max"] + 1e-9
    assert 0 <= stats["queue_wait_s"]["p50"] <= stats["queue_wait_s"]["p99"]
    if max_live == 4:  # slots limited: requests wait to be admitted
        assert stats["queue_wait_s"]["p99"] > 0
    assert stats["drain_s"] >= 0


def test_server_batches_concurrent_requests():
    """Requests that arrive together share batch iterations (continuous batching):
    the number of iterations is the longest request's steps, not the sum."""
    clock = FakeClock()
    be = FakeBackend(clock, 10**12)
    reqs = [serve.Request(i, 0.0, 64, 64, 48, i, 0.0, 5.0, 0.3, 10 + i) for i in range(6)]
    stats = serve.Server(be, setup_workers=6).run(reqs, clock=clock, sleep=clock.sleep)
    assert stats["completed"] == 6
    assert stats["batch_iterations"] < sum(r.steps for r in reqs)


def test_server_refuses_a_request_larger_than_the_device():
    clock = FakeClock()
    be = FakeBackend(clock, budget_cells=1_000_000)
    reqs = [serve.Request(0, 0.0, 256, 256, 90, 1, 0.0, 5.0, 0.3, 10),   # 5.9 M cells: never fits
            serve.Request(1, 0.1, 64, 64, 48, 2, 0.0, 5.0, 0.3, 10)]
    stats = serve.Server(be).run(reqs, clock=clock, sleep=clock.sleep)
    assert stats["rejected"] == 1 and stats["completed"] == 1
