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
