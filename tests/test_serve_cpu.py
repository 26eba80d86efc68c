"""Host logic of the served loop (gallatin_gb300/serve.py) without a GPU: the
job stream and the admission loop, driven by fake launches that finish after
a number of polls proportional to the job's size."""
import numpy as np

from gallatin_gb300.serve import JOB_QUEUE, JOB_VECTOR, footprint, make_jobs, schedule


class FakeRun:
    def __init__(self, polls):
        self.left = polls

    def query(self):
        self.left -= 1
        return self.left <= 0


class Harness:
    """Launches that check the admission rules at the moment they happen."""

    def __init__(self, slots, budget):
        self.slots, self.budget = slots, budget
        self.running = {}    # slot -> (job, run)
        self.order = []
        self.t = 0.0

    def clock(self):
        self.t += 1e-4       # each poll of the loop advances the virtual clock
        return self.t

    def launch(self, job, slot):
        # slots the loop has taken back are free again
        self.running = {s: jr for s, jr in self.running.items() if jr[1].left > 0}
        assert slot not in self.running and 0 <= slot < self.slots
        est = sum(j["est"] for j, _ in self.running.values())
        assert not self.running or est + job["est"] <= self.budget
        assert job["arrival"] <= self.t + 1e-12      # never admitted before it arrives
        run = FakeRun(1 + job["n"] // 50_000)
        self.running[slot] = (job, run)
        self.order.append(job["row"])
        return run


def _rows(jobs):
    return [dict(j, row=r) for r, j in enumerate(jobs)]


def test_job_stream_is_seeded_and_within_its_ranges():
    a, b = make_jobs(300, seed=5), make_jobs(300, seed=5)
    assert a == b
    arrival = np.array([j["arrival"] for j in a])
    assert (np.diff(arrival) > 0).all()
    assert 0.1 < arrival[-1] < 0.2                   # ~2,000 jobs/s
    for j in a:
        lo, hi = (1 << 10, 1 << 24) if j["kind"] == JOB_VECTOR else (1 << 10, 1 << 22)
        assert lo <= j["n"] <= hi


def test_footprint_covers_the_last_two_vector_buffers():
    for n in [1, 1000, 4096, 1 << 20, (1 << 20) + 1, 16 << 20]:
        cap = max(1024, 1 << int(np.ceil(np.log2(n))))
        assert footprint(JOB_VECTOR, n) >= 4 * cap + 2 * cap
    assert footprint(JOB_QUEUE, 1000) >= 32 * 1000


def test_admission_respects_slots_budget_and_arrival_order():
    jobs = _rows(make_jobs(400, seed=5))
    h = Harness(slots=8, budget=1 << 30)
    admit, done, most = schedule(jobs, 8, 1 << 30, h.launch, h.clock)
    assert sorted(h.order) == list(range(400))
    by_arrival = sorted(range(400), key=lambda r: jobs[r]["arrival"])
    assert h.order == by_arrival                     # first come, first admitted
    assert (done >= admit).all() and (admit > 0).all()
    assert 1 < most <= 8


def test_a_job_larger_than_the_budget_runs_alone():
    jobs = _rows([dict(id=0, kind=JOB_VECTOR, n=1 << 20, arrival=0.0),
                  dict(id=1, kind=JOB_VECTOR, n=16 << 20, arrival=1e-6),
                  dict(id=2, kind=JOB_QUEUE, n=1000, arrival=2e-6)])
    budget = footprint(JOB_VECTOR, 16 << 20) // 2
    h = Harness(slots=4, budget=budget)
    admit, done, most = schedule(jobs, 4, budget, h.launch, h.clock)
    assert h.order == [0, 1, 2]
    assert admit[1] >= done[0]                       # waited for job 0 to finish
    assert admit[2] >= done[1]                       # and job 2 for the big one
    assert most == 1


def test_latency_bins_cover_each_value_within_a_fifth():
    """Four bins per power of two: every cycle count maps to a bin whose value
    is within 19% of it, bins grow with the count, and percentiles read from
    a histogram land on the bin of the true percentile."""
    from gallatin_gb300.serve import LAT_BINS, bin_value, hist_percentile, lat_bin
    prev = -1
    for c in list(range(0, 64)) + [int(1.07 ** k) for k in range(60, 400)]:
        b = lat_bin(c)
        assert 0 <= b < LAT_BINS and b >= prev
        prev = b
        if c:
            assert abs(bin_value(b) - c) <= 0.19 * c + 0.5
    rng = np.random.default_rng(1)
    x = (2 ** rng.uniform(8, 20, 100_000)).astype(np.int64)
    h = np.zeros(LAT_BINS, dtype=np.int64)
    np.add.at(h, [lat_bin(v) for v in x], 1)
    for q in (50, 99):
        assert abs(hist_percentile(h, q) - np.percentile(x, q)) <= 0.19 * np.percentile(x, q)
    assert hist_percentile(np.zeros(LAT_BINS), 50) is None


def test_job_grids_and_footprints():
    """Jobs span one CTA per 2^20 vector elements or 2^18 queue operations
    (1-8); a multi-CTA vector job reserves the buffers of each CTA's share."""
    from gallatin_gb300.serve import job_ctas
    assert job_ctas(JOB_VECTOR, 1000) == 1 and job_ctas(JOB_VECTOR, 3 << 20) == 3
    assert job_ctas(JOB_VECTOR, 1 << 30) == 8 and job_ctas(JOB_QUEUE, 1 << 20) == 4
    assert footprint(JOB_VECTOR, 1 << 24) >= 16 * 4 << 20       # 64 MiB of values at least
    assert footprint(JOB_VECTOR, 1 << 24) <= 4 * 3 * (4 << 20) * 8


def test_admission_loop_gives_up_after_its_limit():
    """A job that never finishes ends the loop with TimeoutError once the
    clock passes the limit, instead of polling forever."""
    import pytest

    class Never:
        def query(self):
            return False

    ticks = iter(range(10 ** 6))
    jobs = [{"kind": 0, "n": 1, "arrival": 0.0, "row": 0}]
    with pytest.raises(TimeoutError):
        schedule(jobs, 1, 1 << 30, lambda job, slot: Never(), lambda: float(next(ticks)), limit_s=50.0)
