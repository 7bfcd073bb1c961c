"""Host logic of the served loop (no GPU): admission order, the memory budget,
concurrency, and error delivery, with a fake executor in place of the GPU."""

import threading
import time

import numpy as np
import pytest

from isoext_gb300.serve import MAX_PRIMS, Request, Scheduler, prims_buffer, random_requests


class _Job:
    def __init__(self, rid, need, dur=0.01, fail=False):
        self.rid, self.need, self.dur, self.fail = rid, need, dur, fail


def _fake(log, lock):
    def run(slot, job):
        with lock:
            log.append(("start", job.rid, slot, time.perf_counter()))
        time.sleep(job.dur)
        if job.fail:
            raise ValueError(f"job {job.rid} failed")
        with lock:
            log.append(("end", job.rid, slot, time.perf_counter()))
        return np.full((1, 3), job.rid, np.float32), np.zeros((0, 3), np.int32)

    return run


def test_jobs_overlap_up_to_the_slot_count():
    log, lock = [], threading.Lock()
    s = Scheduler(4, 1 << 30, lambda j: j.need, _fake(log, lock))
    futs = [s.submit(_Job(i, 1, 0.05)) for i in range(12)]
    res = [f.result(timeout=10) for f in futs]
    s.close()
    assert [r.rid for r in res] == list(range(12))
    assert all(r.vertices[0, 0] == r.rid for r in res)
    assert s.max_running == 4
    assert all(r.t_submit <= r.t_start <= r.t_done for r in res)


def test_budget_bounds_the_bytes_admitted():
    log, lock = [], threading.Lock()
    s = Scheduler(8, 100, lambda j: j.need, _fake(log, lock))
    futs = [s.submit(_Job(i, 40, 0.02)) for i in range(10)]
    for f in futs:
        f.result(timeout=10)
    s.close()
    assert s.max_reserved <= 100
    assert s.max_running == 2  # 2 x 40 fit, 3 x 40 do not


def test_admission_is_first_come_first_served():
    log, lock = [], threading.Lock()
    s = Scheduler(4, 100, lambda j: j.need, _fake(log, lock))
    # a large job at the head waits for room; the small ones behind it do not pass it
    jobs = [_Job(0, 60, 0.05), _Job(1, 90, 0.01)] + [_Job(i, 5, 0.01) for i in range(2, 6)]
    futs = [s.submit(j) for j in jobs]
    for f in futs:
        f.result(timeout=10)
    s.close()
    starts = [rid for kind, rid, _, _ in log if kind == "start"]
    assert starts.index(1) < min(starts.index(i) for i in range(2, 6))
    t_end0 = next(t for kind, rid, _, t in log if kind == "end" and rid == 0)
    t_start1 = next(t for kind, rid, _, t in log if kind == "start" and rid == 1)
    assert t_start1 >= t_end0  # 60 + 90 > 100: job 1 waited for job 0's bytes


def test_errors_reach_their_future_and_the_loop_continues():
    log, lock = [], threading.Lock()
    s = Scheduler(2, 1000, lambda j: j.need, _fake(log, lock))
    bad = s.submit(_Job(0, 1, 0.0, fail=True))
    good = s.submit(_Job(1, 1, 0.0))
    with pytest.raises(ValueError, match="job 0 failed"):
        bad.result(timeout=10)
    assert good.result(timeout=10).rid == 1
    s.close()


def test_a_request_larger_than_the_budget_is_refused():
    s = Scheduler(2, 100, lambda j: j.need, _fake([], threading.Lock()))
    with pytest.raises(ValueError, match="budget"):
        s.submit(_Job(0, 101))
    s.close()
    with pytest.raises(RuntimeError, match="closed"):
        s.submit(_Job(1, 1))


def test_prims_buffer_layout():
    p = np.arange(14, dtype=np.float32).reshape(2, 7)
    b = prims_buffer(p)
    assert b.shape == (1 + 7 * MAX_PRIMS,) and b[0] == 2
    assert np.array_equal(b[1:15], p.ravel()) and not b[15:].any()
    with pytest.raises(ValueError):
        prims_buffer(np.zeros((0, 7), np.float32))
    with pytest.raises(ValueError):
        prims_buffer(np.zeros((MAX_PRIMS + 1, 7), np.float32))


def test_request_stream_matches_its_description():
    reqs = random_requests(512, seed=3)
    assert len(reqs) == 512 and [r.rid for r in reqs] == list(range(512))
    assert {r.n for r in reqs} == {64, 96, 128, 192, 256}
    share = sum(r.kind == "mc" for r in reqs) / 512
    assert 0.62 < share < 0.78
    for r in reqs:
        assert 1 <= len(r.prims) <= 16
        assert set(np.unique(r.prims[:, 0])) <= {0.0, 1.0}
        assert (np.abs(r.prims[:, 1:4]) <= 0.5).all()
        assert (r.prims[:, 4:7] > 0).all() and (r.prims[:, 4:7] <= 0.4).all()
    again = random_requests(512, seed=3)
    assert all(np.array_equal(a.prims, b.prims) and a.kind == b.kind and a.n == b.n for a, b in zip(reqs, again))
    assert isinstance(reqs[0], Request)
