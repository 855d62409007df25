"""Serving loop: independent aggregate simulations admitted by device memory, kept resident and
advanced together on one GPU (continuous batching).

The reference runs one simulation per process to completion (run/simulate3d.cpp:37-176) and
has no serving layer; this module is the request loop around the batch entry points of
include/peridem_gb300.h (pd_create_batch, pd_finish_sim, pd_get_sim_state, ...).

How it works:
  * requests arrive over time (`arrival`, seconds after the stream starts) and wait in a FIFO;
  * admission: whenever requests wait and no admission is running, the waiting requests that
    fit in the free device budget (first fit, in arrival order, at most `max_batch`) become one
    cohort: one batch handle on its own CUDA stream, created on a worker thread (the ctypes
    calls release the GIL, so stepping of the resident cohorts goes on meanwhile);
  * stepping: every cohort is advanced in chunks of at most `chunk_steps` steps, cut so that a
    chunk ends exactly where one of its members reaches its step count. Cohorts run on
    separate streams, so their kernels overlap on the device. Within a cohort every phase is
    one launch over all its members (uneven sizes included);
  * completion: at a chunk boundary the members that reached their step count are finished
    (state read back, kept for the caller, their nodes skipped from then on); a cohort whose
    members are all finished is closed and its memory returns to the budget, which admits
    the next waiting requests;
  * compaction: a finished member's memory stays with its cohort's handle until the handle
    closes. When requests wait that do not fit and the finished members of a cohort hold at
    least `compact` of its bytes, the cohort's unfinished members are evicted -- saved to host
    memory at the chunk boundary (pd_save_sim) -- and the handle is closed, so its memory
    returns at once; the evicted members wait at the front of the queue and, once admitted,
    continue from their checkpoints (pd_load_sim), exactly as if never interrupted;
  * failures: a cohort whose handle reports an error (a device error word, a failed read) is
    closed and its memory returned; its unfinished members are queued again, each alone, and a
    member that fails alone gets the error as its result. Other cohorts are not affected.
Each result is what the same simulation computes alone: nothing in a step couples two
simulations of a batch (the tests check this bit for bit).
"""
from __future__ import annotations

import threading
import time
from collections import deque
from dataclasses import dataclass, field, replace

import numpy as np

from .setupdata import Setup


@dataclass
class Request:
    rid: int
    setup: Setup
    config: dict
    steps: int
    arrival: float = 0.0
    checkpoint: bytes | None = None  # set when the request was evicted: its state at that point
    remaining: int | None = None     # steps left after the checkpoint


@dataclass
class Result:
    rid: int
    state: dict | None
    wall: tuple | None
    arrival: float
    admitted: float
    done: float
    steps: int
    n_nodes: int
    bonds: int          # directed bonds of the setup (the bond-update count of one step)
    error: str | None = None
    damage: np.ndarray | None = None  # per-node damage at the last step (keep_damage)

    @property
    def ttc(self) -> float:
        """Time to completion: arrival to result in host memory (s)."""
        return self.done - self.arrival


@dataclass
class _Cohort:
    batch: object
    members: list          # [Request]
    remaining: list        # steps still to run per member
    admitted: float
    nbytes: int
    finished: list = field(default_factory=list)


def directed_bonds(s: Setup) -> int:
    return 2 * int(len(s.conn))


class Server:
    """Continuous-batching server over batch handles.

    make_batch(setups, configs, precision) -> handle with step(n, sync=False), poll(),
    finish(i), sim_state(i), sim_wall(i), device_bytes(), close() (and sim_damage(i) with
    keep_damage; save_sim(i) and load_sim(blob, i) for compaction); the default is
    peridem_gb300.sim.Batch. estimate(setups, precision) -> bytes (default
    peridem_gb300.sim.estimate_bytes)."""

    def __init__(self, precision: str = "fp32c", capacity_bytes: int | None = None, chunk_steps: int = 500,
                 max_batch: int = 32, keep_state: bool = True, make_batch=None, estimate=None, tune=None,
                 keep_damage: bool = False, compact: float = 0.5):
        if make_batch is None or estimate is None:
            from . import sim as _sim
            make_batch = make_batch or _sim.Batch
            estimate = estimate or _sim.estimate_bytes
            if capacity_bytes is None:
                free, _ = _sim.device_memory()
                capacity_bytes = int(free * 0.85)
        if capacity_bytes is None:
            raise ValueError("capacity_bytes is required with a custom backend")
        self.precision = precision
        self.capacity = int(capacity_bytes)
        self.chunk = int(chunk_steps)
        self.max_batch = int(max_batch)
        self.keep_state = keep_state
        self.keep_damage = keep_damage
        self.make_batch = make_batch
        self.estimate = estimate
        self.tune = tune or {}
        self.used = 0
        self.peak_used = 0
        self.cohorts: list[_Cohort] = []
        self.log: list[tuple] = []   # (time, event, detail)
        self.create_s: list[float] = []  # host+device time to build each cohort's handle
        self._solo: set = set()          # requests to admit alone (their cohort failed)
        self.finish_s = 0.0              # time spent reading finished simulations back
        self.compact = float(compact)    # finished share of a cohort's bytes that allows compaction (0: never)
        self.evictions = 0               # simulations saved to host memory and re-queued
        self.max_resident = 0            # most cohorts resident at once
        self._est: dict = {}

    # -- admission ------------------------------------------------------------------------
    def _pick(self, waiting: deque, est: dict) -> list:
        """First fit in arrival order; a request whose cohort failed to build is retried alone."""
        free = self.capacity - self.used
        pick, tot = [], 0
        for r in list(waiting):
            b = est[r.rid]
            alone = r.rid in self._solo
            if alone and pick:
                continue
            if tot + b <= free and len(pick) < self.max_batch:
                pick.append(r)
                tot += b
                if alone:
                    break
        return pick

    def _create(self, reqs: list, out: dict):
        t0 = time.perf_counter()
        try:
            b = self.make_batch([r.setup for r in reqs], [dict(r.config, timesteps=r.steps) for r in reqs],
                                self.precision)
            if self.tune and hasattr(b, "tune"):
                b.tune(**self.tune)
            elif hasattr(b, "graph_mode") and b.graph_mode() == 3:
                # cohorts share the GPU: a persistent launch holds every SM for its steps and
                # would run the cohorts one after another, so small cohorts step with the graph
                b.tune(graphs=1)
            for i, r in enumerate(reqs):  # evicted requests continue from their checkpoints
                if r.checkpoint is not None:
                    b.load_sim(r.checkpoint, i)
            out["batch"] = b
        except Exception as e:  # reported per request
            out["error"] = str(e)
        out["create_s"] = time.perf_counter() - t0

    # -- one cohort -----------------------------------------------------------------------
    def _advance(self, c: _Cohort, results: dict, now, realtime: bool, waiting: deque | None = None) -> bool:
        """Reads back the members that reached their step count, closes the cohort when none is
        left, compacts it when that lets waiting requests in, else enqueues its next chunk.
        Returns whether anything happened."""
        if not c.batch.poll():
            return False
        tdone = now()
        for i, r in enumerate(c.members):
            if c.remaining[i] == 0 and i not in c.finished:
                tf = time.perf_counter()
                c.batch.finish(i)
                st = c.batch.sim_state(i) if self.keep_state else None
                wl = c.batch.sim_wall(i) if self.keep_state else None
                dm = c.batch.sim_damage(i) if self.keep_damage else None
                c.finished.append(i)
                self.finish_s += time.perf_counter() - tf
                results[r.rid] = Result(r.rid, st, wl, r.arrival if realtime else 0.0, c.admitted, now(),
                                        r.steps, len(r.setup.pos), directed_bonds(r.setup), damage=dm)
                self.log.append((tdone, "done", r.rid))
        live = [k for k in c.remaining if k > 0]
        if not live:
            c.batch.close()
            self.used -= c.nbytes
            self.cohorts.remove(c)
            self.log.append((now(), "close", [r.rid for r in c.members]))
            return True
        if waiting and self._should_compact(c, waiting):
            self._evict(c, waiting, now)
            return True
        k = min(self.chunk, min(live))
        c.batch.step(k, sync=False)
        c.remaining = [max(0, x - k) if x > 0 else 0 for x in c.remaining]
        return True

    def _should_compact(self, c: _Cohort, waiting: deque) -> bool:
        """The first waiting request does not fit, and this cohort's finished members hold at
        least `compact` of its bytes."""
        if self.compact <= 0 or not c.finished or not hasattr(c.batch, "save_sim"):
            return False
        if self._est[waiting[0].rid] <= self.capacity - self.used:
            return False
        done = sum(self._est[c.members[i].rid] for i in c.finished)
        return done >= self.compact * sum(self._est[r.rid] for r in c.members)

    def _evict(self, c: _Cohort, waiting: deque, now) -> None:
        """Saves the unfinished members to host memory, closes the handle (its memory returns)
        and puts them back at the front of the queue, in their order."""
        back = []
        for i, r in enumerate(c.members):
            if i in c.finished or c.remaining[i] == 0:
                continue
            back.append(replace(r, checkpoint=c.batch.save_sim(i), remaining=c.remaining[i]))
        c.batch.close()
        self.used -= c.nbytes
        self.cohorts.remove(c)
        self.evictions += len(back)
        self.log.append((now(), "evict", [r.rid for r in back]))
        for r in reversed(back):
            waiting.appendleft(r)

    def _fail(self, c: _Cohort, err: Exception, waiting: deque, results: dict, now, realtime: bool) -> None:
        """A cohort whose handle reported an error (the device error word is per handle, so the
        member that raised it is unknown): the handle is closed and its bytes returned; each
        unfinished member runs again alone from its setup, and one that was already alone gets
        the error as its result. The other cohorts go on."""
        try:
            c.batch.close()
        except Exception:
            pass
        self.used -= c.nbytes
        self.cohorts.remove(c)
        self.log.append((now(), "fail", [r.rid for r in c.members], str(err)))
        again = []
        for i, r in enumerate(c.members):
            if i in c.finished or r.rid in results:
                continue
            if len(c.members) == 1 or r.rid in self._solo:
                results[r.rid] = Result(r.rid, None, None, r.arrival if realtime else 0.0, c.admitted, now(), 0,
                                        len(r.setup.pos), directed_bonds(r.setup), error=str(err))
            else:
                self._solo.add(r.rid)
                again.append(r)
        for r in reversed(again):
            waiting.appendleft(r)

    # -- main loop ------------------------------------------------------------------------
    def run(self, requests: list[Request], realtime: bool = True, idle_sleep: float = 2e-4) -> list[Result]:
        """Serves `requests` (arrival times relative to the start of this call when realtime,
        otherwise all arrive at once) and returns one Result per request, in rid order."""
        reqs = sorted(requests, key=lambda r: (r.arrival, r.rid))
        est = {r.rid: int(self.estimate([r.setup], self.precision)) for r in reqs}
        self._est = est
        results: dict[int, Result] = {}
        waiting: deque = deque()
        nxt = 0
        admit = None  # (thread, out, reqs, reserved bytes, t_start)
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0  # noqa: E731
        while len(results) < len(reqs):
            t = now()
            busy = False
            # arrivals
            while nxt < len(reqs) and (not realtime or reqs[nxt].arrival <= t):
                r = reqs[nxt]
                if est[r.rid] > self.capacity:
                    results[r.rid] = Result(r.rid, None, None, r.arrival if realtime else 0.0, t, t, 0, len(r.setup.pos),
                                            directed_bonds(r.setup), error="larger than the device budget")
                else:
                    waiting.append(r)
                nxt += 1
                busy = True
            # admission finished?
            if admit is not None and not admit[0].is_alive():
                th, out, areqs, reserved, ta = admit
                admit = None
                busy = True
                self.create_s.append(out.get("create_s", 0.0))
                if "batch" in out:
                    b = out["batch"]
                    nb = int(b.device_bytes()) if hasattr(b, "device_bytes") else reserved
                    self.used += nb - reserved
                    self.peak_used = max(self.peak_used, self.used)
                    self.cohorts.append(_Cohort(b, areqs, [r.remaining if r.checkpoint is not None else r.steps
                                                           for r in areqs], now(), nb))
                    self.max_resident = max(self.max_resident, len(self.cohorts))
                    self.log.append((now(), "admit", [r.rid for r in areqs]))
                else:
                    self.used -= reserved
                    if len(areqs) == 1:
                        r = areqs[0]
                        results[r.rid] = Result(r.rid, None, None, r.arrival if realtime else 0.0, ta, now(), 0,
                                                len(r.setup.pos), directed_bonds(r.setup), error=out.get("error"))
                    else:  # retry one by one
                        for r in reversed(areqs):  # retry each of them alone
                            self._solo.add(r.rid)
                            waiting.appendleft(r)
            # start an admission
            if admit is None and waiting:
                pick = self._pick(waiting, est)
                if pick:
                    for r in pick:
                        waiting.remove(r)
                    reserved = sum(est[r.rid] for r in pick)
                    self.used += reserved
                    self.peak_used = max(self.peak_used, self.used)
                    out: dict = {}
                    th = threading.Thread(target=self._create, args=(pick, out), daemon=True)
                    th.start()
                    admit = (th, out, pick, reserved, now())
                    busy = True
            # advance cohorts
            for c in list(self.cohorts):
                try:
                    busy |= self._advance(c, results, now, realtime, waiting)
                except Exception as e:  # a device error of this handle (PdError), a failed read
                    self._fail(c, e, waiting, results, now, realtime)
                    busy = True
            if not busy:
                if realtime and not waiting and not self.cohorts and admit is None and nxt < len(reqs):
                    time.sleep(max(0.0, min(reqs[nxt].arrival - now(), 0.01)))
                else:
                    time.sleep(idle_sleep)
        return [results[r.rid] for r in sorted(reqs, key=lambda r: r.rid)]


def summarize(results: list[Result], wall_s: float) -> dict:
    """sims/hour, aggregate bond-updates/s and time-to-completion percentiles."""
    ok = [r for r in results if r.error is None]
    ttc = np.array([r.ttc for r in ok]) if ok else np.zeros(1)
    bu = float(sum(r.bonds * r.steps for r in ok))
    return dict(requests=len(results), completed=len(ok), failed=len(results) - len(ok),
                wall_s=wall_s, sims_per_hour=len(ok) / wall_s * 3600.0 if wall_s > 0 else 0.0,
                bond_updates=bu, bond_updates_per_s=bu / wall_s if wall_s > 0 else 0.0,
                ttc_p50_s=float(np.percentile(ttc, 50)), ttc_p99_s=float(np.percentile(ttc, 99)),
                ttc_mean_s=float(ttc.mean()))


def sequential_ttc(arrivals: np.ndarray, service_s: np.ndarray) -> np.ndarray:
    """Time to completion of requests served one at a time in arrival order (FIFO queue)."""
    order = np.argsort(arrivals, kind="stable")
    done = np.empty_like(service_s)
    t = 0.0
    for i in order:
        t = max(t, arrivals[i]) + service_s[i]
        done[i] = t
    return done - arrivals
