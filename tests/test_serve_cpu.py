"""Host logic of the serving loop (peridem_gb300/serve.py) on a fake batch backend: admission
by device budget, chunking that stops every request at exactly its step count, cohort
retirement, oversize requests, and the queueing arithmetic of the one-at-a-time baseline."""
from types import SimpleNamespace

import numpy as np

from peridem_gb300 import serve

BYTES_PER_NODE = 1000


class FakeBatch:
    instances = []

    def __init__(self, setups, configs, precision):
        self.n = len(setups)
        self.steps = [0] * self.n
        self.fin = [False] * self.n
        self.cfg = configs
        self.nb = sum(len(s.pos) * BYTES_PER_NODE for s in setups)
        self.closed = False
        FakeBatch.instances.append(self)

    def step(self, k, sync=True):
        for i in range(self.n):
            if not self.fin[i]:
                self.steps[i] += k

    def poll(self):
        return True

    def finish(self, i):
        self.fin[i] = True

    def sim_state(self, i):
        return {"steps": self.steps[i]}

    def sim_wall(self, i):
        return (np.zeros(6), np.zeros((6, 3)))

    def sim_damage(self, i):
        return np.full(3, float(self.steps[i]))

    def device_bytes(self):
        return self.nb

    def save_sim(self, i):
        return str(self.steps[i]).encode()

    def load_sim(self, blob, i):
        self.steps[i] = int(blob.decode())

    def close(self):
        self.closed = True


def fake_estimate(setups, precision):
    return sum(len(s.pos) * BYTES_PER_NODE for s in setups)


def _req(rid, nodes, steps, arrival=0.0):
    s = SimpleNamespace(pos=np.zeros((nodes, 3)), conn=np.zeros((nodes * 4, 2)))
    return serve.Request(rid, s, {"dt": 1e-8}, steps, arrival)


def _server(capacity, **kw):
    FakeBatch.instances.clear()
    return serve.Server("fp32c", capacity_bytes=capacity, make_batch=FakeBatch, estimate=fake_estimate, **kw)


def test_every_request_stops_at_its_step_count():
    reqs = [_req(i, 100 + 10 * i, st) for i, st in enumerate([7, 130, 64, 1, 99, 500, 33])]
    srv = _server(10 ** 9, chunk_steps=50, max_batch=4)
    res = srv.run(reqs, realtime=False)
    assert [r.rid for r in res] == list(range(len(reqs)))
    for r, q in zip(res, reqs):
        assert r.error is None
        assert r.state["steps"] == q.steps
        assert r.bonds == 2 * len(q.setup.conn)
    assert srv.used == 0 and all(b.closed for b in FakeBatch.instances)
    assert len(FakeBatch.instances) >= 2  # max_batch=4 splits 7 requests


def test_admission_respects_the_budget():
    reqs = [_req(i, 1000, 40) for i in range(6)]
    srv = _server(2500 * BYTES_PER_NODE, chunk_steps=10)
    res = srv.run(reqs, realtime=False)
    assert all(r.error is None for r in res)
    assert srv.peak_used <= 2500 * BYTES_PER_NODE
    assert max(b.n for b in FakeBatch.instances) <= 2


def test_oversize_request_is_rejected_not_blocking():
    reqs = [_req(0, 10, 5), _req(1, 10 ** 6, 5), _req(2, 10, 5)]
    srv = _server(10 ** 5 * BYTES_PER_NODE)
    res = srv.run(reqs, realtime=False)
    assert res[1].error and res[0].error is None and res[2].error is None


def test_realtime_arrivals_are_respected():
    reqs = [_req(i, 50, 20, arrival=0.02 * i) for i in range(4)]
    srv = _server(10 ** 9, chunk_steps=5)
    res = srv.run(reqs)
    for r in res:
        assert r.admitted >= r.arrival - 1e-3
        assert r.done >= r.admitted
    s = serve.summarize(res, max(r.done for r in res))
    assert s["completed"] == 4 and s["ttc_p99_s"] >= s["ttc_p50_s"]


def test_sequential_queue_arithmetic():
    arr = np.array([0.0, 1.0, 1.5, 10.0])
    svc = np.array([2.0, 2.0, 1.0, 0.5])
    ttc = serve.sequential_ttc(arr, svc)
    # done: 2, 4, 5, 10.5
    np.testing.assert_allclose(ttc, [2.0, 3.0, 3.5, 0.5])


class FailingPairBatch(FakeBatch):
    """Fails to build any cohort of more than one request containing request 1."""

    def __init__(self, setups, configs, precision):
        if len(setups) > 1 and any(c.get("tag") == 1 for c in configs):
            raise RuntimeError("cohort build failed")
        super().__init__(setups, configs, precision)


def test_failed_cohort_is_retried_one_by_one():
    reqs = [_req(i, 100, 10) for i in range(4)]
    for r in reqs:
        r.config = dict(r.config, tag=r.rid)
    FakeBatch.instances.clear()
    srv = serve.Server("fp32c", capacity_bytes=10 ** 9, make_batch=FailingPairBatch, estimate=fake_estimate,
                       max_batch=4)
    res = srv.run(reqs, realtime=False)
    assert all(r.error is None and r.state["steps"] == 10 for r in res)
    assert srv.max_batch == 4  # only the failed requests were retried alone


def test_damage_is_read_only_when_asked():
    for keep in (False, True):
        srv = _server(10 ** 9, chunk_steps=4, keep_damage=keep)
        res = srv.run([_req(0, 10, 9), _req(1, 20, 5)])
        for r in res:
            if keep:
                np.testing.assert_array_equal(r.damage, np.full(3, float(r.steps)))
            else:
                assert r.damage is None


class FailingBatch(FakeBatch):
    """A fake handle whose device error word is raised by poll() once any member listed in
    `bad` is in it and `after` chunks have run (as Batch.poll raises PdError on PD_EDEVICE)."""
    bad: set = set()
    after = 1

    def __init__(self, setups, configs, precision):
        super().__init__(setups, configs, precision)
        self.rids = [c["rid"] for c in configs]
        self.chunks = 0

    def step(self, k, sync=True):
        super().step(k, sync)
        self.chunks += 1

    def poll(self):
        if self.chunks >= FailingBatch.after and FailingBatch.bad & set(self.rids):
            raise RuntimeError("[-6] device error word: non-finite force density")
        return True


def _failing_server(capacity, bad, **kw):
    FakeBatch.instances.clear()
    FailingBatch.bad = set(bad)
    return serve.Server("fp32c", capacity_bytes=capacity, make_batch=FailingBatch, estimate=fake_estimate, **kw)


def _req_rid(rid, nodes, steps, arrival=0.0):
    r = _req(rid, nodes, steps, arrival)
    r.config = dict(r.config, rid=rid)
    return r


def test_a_failing_cohort_does_not_stop_the_others():
    """Member 2 makes its handle raise: its cohort is closed and its bytes returned; the other
    members of that cohort run again alone and complete; only member 2 gets the error; the
    other cohort is not affected."""
    reqs = [_req_rid(i, 100, 120) for i in range(6)]
    srv = _failing_server(10 ** 9, bad={2}, chunk_steps=50, max_batch=3)
    res = srv.run(reqs, realtime=False)
    errs = {r.rid: r.error for r in res}
    assert errs[2] is not None and "non-finite" in errs[2]
    for i in (0, 1, 3, 4, 5):
        assert errs[i] is None, (i, errs[i])
        assert res[i].state["steps"] == 120
    assert srv.used == 0
    assert all(b.closed for b in FakeBatch.instances)
    fails = [e for e in srv.log if e[1] == "fail"]
    assert len(fails) == 2  # the cohort of three, then member 2 alone
    assert sorted(fails[0][2]) == [0, 1, 2] and fails[1][2] == [2]


def test_a_failing_request_alone_reports_its_error():
    reqs = [_req_rid(0, 100, 80)]
    srv = _failing_server(10 ** 9, bad={0}, chunk_steps=50, max_batch=4)
    res = srv.run(reqs, realtime=False)
    assert res[0].error is not None and res[0].state is None
    assert srv.used == 0 and not srv.cohorts


def test_compaction_frees_finished_members_memory():
    """A long request shares a cohort with two short ones; three more wait that do not fit. When
    the short ones finish, the cohort is compacted: the long one is saved, the handle closed,
    and it continues in the next cohort with the waiting requests. Every request still stops at
    exactly its step count, the budget is never exceeded and the long request's state passes
    through the checkpoints."""
    reqs = [_req(0, 1000, 200), _req(1, 1000, 20), _req(2, 1000, 20)] + [_req(3 + i, 1000, 30) for i in range(3)]
    srv = _server(3000 * BYTES_PER_NODE, chunk_steps=10, max_batch=3)
    res = srv.run(reqs, realtime=False)
    assert all(r.error is None for r in res)
    assert [r.state["steps"] for r in res] == [q.steps for q in reqs]
    ev = [e for e in srv.log if e[1] == "evict"]
    assert ev and ev[0][2] == [0] and srv.evictions >= 1
    assert srv.peak_used <= 3000 * BYTES_PER_NODE and srv.used == 0
    # without compaction the waiting requests sit until the long one ends
    srv2 = _server(3000 * BYTES_PER_NODE, chunk_steps=10, max_batch=3, compact=0)
    res2 = srv2.run(reqs, realtime=False)
    assert not [e for e in srv2.log if e[1] == "evict"]
    assert [r.state["steps"] for r in res2] == [q.steps for q in reqs]
