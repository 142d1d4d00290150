"""Serving loop (tandemproject_gb300.serve) and the seeded workloads: the
scheduler's admission and retirement logic on the CPU with a stand-in case,
and on the GPU the property that every result is the same alone and in the mix."""
import numpy as np
import pytest

from tandemproject_gb300.workloads import Request, batch_cases, footprint_bytes, serving_requests


def test_workloads_are_seeded_and_in_range():
    a = serving_requests(20, seed=99)
    b = serving_requests(20, seed=99)
    assert [(r.cfg, r.steps, r.arrival) for r in a] == [(r.cfg, r.steps, r.arrival) for r in b]
    for r in a:
        assert 8 <= r.cfg.thick <= 18 and 0 <= r.cfg.aoa_deg <= 8 and 0.2 <= r.cfg.mach <= 0.4
        assert 200 <= r.steps <= 2000 and 16 <= r.cfg.lzebk[0] + 1 <= 48
        assert 0.3e6 <= r.cfg.npoints <= 25e6
    assert np.all(np.diff([r.arrival for r in a]) > 0)
    cases = batch_cases(16, seed=7)
    sizes = [c.npoints for c, _ in cases]
    assert len(sizes) == 16 and min(sizes) >= 0.8e6 and max(sizes) <= 7e6 and len(set(sizes)) == 16


class FakeCase:
    """CPU stand-in: 'runs' instantly; records the steps it was given."""
    live = 0
    peak = 0

    def __init__(self, cfg, grid):
        self.cfg = cfg
        self.steps = 0
        FakeCase.live += 1
        FakeCase.peak = max(FakeCase.peak, FakeCase.live)

    def idle(self):
        return True

    def step_async(self, k):
        self.steps += k

    def check(self):
        pass

    def forces(self):
        return np.array([float(self.steps), 0.0])

    def close(self):
        FakeCase.live -= 1


def test_scheduler_admits_under_budget_and_finishes_everything():
    from tandemproject_gb300.config import small_case
    from tandemproject_gb300.serve import Server
    reqs = [Request(i, small_case(), 25 + i, 0.001 * i, {}) for i in range(8)]
    fp = lambda cfg: 10
    srv = Server(budget_bytes=30, chunk=7, make_case=FakeCase, make_grid=lambda cfg: (cfg, None), footprint=fp)
    FakeCase.live = FakeCase.peak = 0
    done, summary = srv.run(reqs)
    assert sorted(d["id"] for d in done) == list(range(8))
    for d in done:
        assert d["forces"][0] == d["steps"]  # every step issued, in chunks
        assert d["latency"] >= 0 and d["admitted"] >= d["arrival"] - 1e-9
    assert FakeCase.peak <= 3 and srv.peak_bytes <= 30  # three 10-byte cases fit the 30-byte budget
    assert summary["requests"] == 8 and summary["latency_s"]["p99"] >= summary["latency_s"]["p50"]


def test_footprint_grows_with_points_and_precision():
    from tandemproject_gb300.config import FP64, MIXED, small_case
    a, b = small_case(precision=FP64), small_case(precision=MIXED)
    assert footprint_bytes(b) > footprint_bytes(a) > a.npoints * 93 * 8


@pytest.mark.gpu
def test_results_same_alone_and_in_the_mix(ati_lib):
    from tandemproject_gb300.config import small_case
    from tandemproject_gb300.serve import Server
    from tandemproject_gb300.solver import setup_case
    cfgs = [small_case(lxibk=(48, 120, 48), letbk=(39, 39), lzebk=(12,), precision=1),
            small_case(lxibk=(48, 120, 48), letbk=(39, 39), lzebk=(15,), mach=0.3, aoa_deg=4.0, precision=1),
            small_case(lxibk=(48, 120, 48), letbk=(39, 39), lzebk=(12,), mach=0.2, thick=15.0, precision=0)]
    reqs = [Request(i, c, s, 0.002 * i, {}) for i, (c, s) in enumerate(zip(cfgs, (30, 17, 24)))]
    srv = Server(budget_bytes=8 << 30, chunk=4, keep_state=True)
    done, summary = srv.run(reqs)
    assert summary["requests"] == 3
    for d in done:
        alone = setup_case(cfgs[d["id"]])
        assert alone.folded_blocks() == []  # the server kept the requested grid
        alone.step(reqs[d["id"]].steps)
        for mb, q in enumerate(d["state"]):
            np.testing.assert_array_equal(q, alone.get_state(mb))
        np.testing.assert_array_equal(d["forces"], alone.forces())
        alone.close()


class DivergingCase(FakeCase):
    """A stand-in whose state turns non-finite after `bad_after` steps (the cases with aoa_deg > 5)."""

    def check(self):
        from tandemproject_gb300.solver import AtiError
        if self.cfg.aoa_deg > 5 and self.steps >= 20:
            raise AtiError(4, "non-finite or non-positive density/pressure in the state of case 0")


def test_scheduler_retires_a_diverged_request_and_serves_the_rest():
    from tandemproject_gb300.config import small_case
    from tandemproject_gb300.serve import Server
    reqs = [Request(i, small_case(aoa_deg=8.0 if i in (2, 5) else 0.0), 40 + i, 0.001 * i, {}) for i in range(8)]
    srv = Server(budget_bytes=30, chunk=7, make_case=DivergingCase, make_grid=lambda cfg: (cfg, None),
                 footprint=lambda cfg: 10)
    FakeCase.live = FakeCase.peak = 0
    done, summary = srv.run(reqs)
    assert sorted(d["id"] for d in done) == [0, 1, 3, 4, 6, 7]
    assert summary["failed"] == 2 and sorted(f["id"] for f in summary["failed_requests"]) == [2, 5]
    for f in summary["failed_requests"]:
        assert f["steps_run"] == 21 and f["params"]["aoa_deg"] == 8.0  # retired after the chunk that diverged
    assert FakeCase.live == 0  # every case closed, the failed ones too
    for d in done:
        assert d["forces"][0] == d["steps"]


class PlannedCase(FakeCase):
    """A stand-in that records whether it was given an earlier case's tile plan."""
    made = []

    def __init__(self, cfg, grid, plan=None):
        super().__init__(cfg, grid)
        self.plan = plan
        PlannedCase.made.append((cfg.lxibk, plan))

    def tile_plan(self):
        return ("plan", self.cfg.lxibk)


def test_scheduler_reuses_tile_plans_per_block_shape():
    from tandemproject_gb300.config import small_case
    from tandemproject_gb300.serve import Server
    shapes = [(24, 64, 24), (32, 64, 32), (24, 64, 24), (24, 64, 24), (32, 64, 32)]
    reqs = [Request(i, small_case(lxibk=s), 10, 0.001 * i, {}) for i, s in enumerate(shapes)]
    srv = Server(budget_bytes=100, chunk=5, make_case=PlannedCase, make_grid=lambda cfg: (cfg, None),
                 footprint=lambda cfg: 10)
    PlannedCase.made = []
    done, summary = srv.run(reqs)
    assert len(done) == 5 and summary["tile_plans_reused"] == 3
    # the first case of each shape times its tiles; the later ones get its plan
    assert PlannedCase.made == [((24, 64, 24), None), ((32, 64, 32), None), ((24, 64, 24), ("plan", (24, 64, 24))),
                                ((24, 64, 24), ("plan", (24, 64, 24))), ((32, 64, 32), ("plan", (32, 64, 32)))]


class RefusedCase(FakeCase):
    """A stand-in the library refuses at set-up for the cases of Mach 0.35 (as ati_create does when device memory
    is short)."""

    def __init__(self, cfg, grid):
        from tandemproject_gb300.solver import AtiError
        if cfg.mach == 0.35:
            raise AtiError(3, "cudaMalloc of the case's arena failed: out of memory")
        super().__init__(cfg, grid)


def test_scheduler_retires_a_request_refused_at_set_up_and_serves_the_rest():
    from tandemproject_gb300.config import small_case
    from tandemproject_gb300.serve import Server
    reqs = [Request(i, small_case(mach=0.35 if i == 3 else 0.24), 20 + i, 0.001 * i, {}) for i in range(6)]
    srv = Server(budget_bytes=10, chunk=7, make_case=RefusedCase, make_grid=lambda cfg: (cfg, None),
                 footprint=lambda cfg: 10)  # one case at a time
    FakeCase.live = FakeCase.peak = 0
    done, summary = srv.run(reqs)
    assert sorted(d["id"] for d in done) == [0, 1, 2, 4, 5]
    assert summary["failed"] == 1 and summary["failed_requests"][0]["id"] == 3
    assert summary["failed_requests"][0]["steps_run"] == 0
    # the refused case's memory went back to the budget: held, the next admission would have gone past it
    assert FakeCase.live == 0 and srv.peak_bytes <= 10
