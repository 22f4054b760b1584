"""Serving loop: integrations requested over time, admitted against an HBM
budget, kept device-resident and advanced together by continuous batching.

A request is one wave-field integration (an `Experiment` plus a step
count).  The loop:

  1. admits arrived requests in arrival order while their device footprint
     (resident fields plus the transient binary64 coefficient buffers of the
     set-up) fits the budget; set-up of a new member runs on its own stream
     while the current batch chunk runs on the batch stream;
  2. advances every active member by one chunk of steps with one batched,
     graph-captured launch per step (chunk = min(chunk_max, fewest steps any
     member has left), so every member stops exactly at its step count);
  3. retires finished members (state copied to the host, memory freed) and
     repeats; new arrivals join at the next chunk boundary.

Latency of a request = completion time - arrival time.  The executor is
pluggable so the scheduling logic is testable without a GPU
(`FakeExecutor`).
"""
import math
import time
from dataclasses import dataclass, field
from typing import Any, List, Optional

import numpy as np


@dataclass
class Request:
    rid: int
    exp: Any                 # configs.Experiment
    steps: int
    arrival: float           # seconds after the start of the run
    cells: int = 0
    admitted: Optional[float] = None
    finished: Optional[float] = None
    result: Any = None
    cancel_at: Optional[float] = None   # the client gives up at this time (s after the start)
    status: str = "queued"              # queued, running, done, cancelled, failed
    error: Optional[str] = None
    ended: Optional[float] = None       # when a cancelled or failed request left

    @property
    def latency(self):
        return None if self.finished is None else self.finished - self.arrival


def poisson_requests(n, rate, seed, steps_range=(50, 1000), spatial=None, spectral=None):
    """n requests with exponential inter-arrival times (mean 1/rate s) and
    step counts uniform in steps_range; dims as the ensemble members."""
    from . import configs
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        steps = int(rng.integers(steps_range[0], steps_range[1] + 1))
        kw = {}
        if spatial:
            kw["spatial"] = spatial
        if spectral:
            kw["spectral"] = spectral
        exp = configs.ensemble_member(rng, steps=steps, **kw)
        out.append(Request(i, exp, steps, t, cells=exp.cells))
    return out


def bytes_per_cell(precision):
    """resident device bytes per cell and transient set-up bytes per cell"""
    elem = 8 if precision == "fp64" else 4
    nlam = 3 if precision == "fp64" else 1
    resident = elem * (2 + 6 + nlam) + elem * 6 / 8.0      # + face-0 planes (<= n/8 of a field)
    transient = 0 if precision == "fp64" else 8 * (6 + 3) + 8 * 6 / 8.0
    return resident, transient


@dataclass
class ServeReport:
    requests: List[Request]
    makespan: float
    cell_updates: int
    peak_bytes: int
    chunks: int
    backlog_max: int
    timeline: list = field(default_factory=list)

    def percentile(self, q):
        lat = sorted(r.latency for r in self.requests if r.status == "done")
        if not lat:
            return None
        k = max(0, min(len(lat) - 1, int(math.ceil(q / 100.0 * len(lat))) - 1))
        return lat[k]

    def summary(self):
        return {"requests": len(self.requests),
                "completed": sum(r.status == "done" for r in self.requests),
                "cancelled": sum(r.status == "cancelled" for r in self.requests),
                "failed": sum(r.status == "failed" for r in self.requests),
                "p50_s": self.percentile(50), "p99_s": self.percentile(99),
                "makespan_s": self.makespan,
                "cell_updates_per_s": self.cell_updates / self.makespan if self.makespan > 0 else None,
                "peak_bytes": self.peak_bytes, "chunks": self.chunks, "backlog_max": self.backlog_max}


class Server:
    """Continuous-batching request loop.  With an executor whose
    `overlap_setup` is true, set-up of admitted requests (`admit_async`) runs
    in a background thread pool while chunks run on the GPU; new members join
    at the next chunk boundary once their set-up has finished.

    One request's trouble does not reach the others: a set-up or a retire
    that raises marks that request "failed" (with the error) and returns its
    memory to the budget; a request whose cancel_at has passed is dropped at
    the next chunk boundary ("cancelled"), before admission, during set-up
    or while running, and its member is discarded.  A failing chunk (the
    batched launch itself) ends the run with the error."""

    def __init__(self, executor, budget_bytes=120e9, chunk_max=50, max_members=64, setup_workers=2):
        self.ex = executor
        self.budget = float(budget_bytes)
        self.chunk_max = int(chunk_max)
        self.max_members = int(max_members)
        self.setup_workers = int(setup_workers)

    def run(self, requests):
        ex = self.ex
        asynchronous = getattr(ex, "overlap_setup", False)
        pool = None
        if asynchronous:
            import concurrent.futures as cf
            pool = cf.ThreadPoolExecutor(self.setup_workers)
        queue = sorted(requests, key=lambda r: r.arrival)
        qi = 0
        active = []            # [request, member, remaining]
        pending = []           # [request, future]
        used = 0.0             # resident bytes of admitted requests
        transient = 0.0        # set-up bytes of requests still being set up
        peak = 0.0
        chunks = 0
        backlog_max = 0
        total = 0
        timeline = []
        t0 = ex.now()
        try:
            while qi < len(queue) or active or pending:
                now = ex.now() - t0
                # ---- admission (arrival order, HBM budget) ----
                while (qi < len(queue) and queue[qi].arrival <= now
                       and len(active) + len(pending) < self.max_members):
                    r = queue[qi]
                    if _gave_up(r, now):
                        _end(r, "cancelled", ex.now() - t0)
                        qi += 1
                        continue
                    need_res, need_tmp = ex.footprint(r)
                    if need_res + need_tmp > self.budget:
                        raise ValueError("request %d needs %.3g B, more than the whole budget"
                                         % (r.rid, need_res + need_tmp))
                    if used + transient + need_res + need_tmp > self.budget:
                        break                                    # wait for memory to free up
                    r.admitted = ex.now() - t0
                    r.status = "running"
                    used += need_res
                    if asynchronous:
                        transient += need_tmp
                        pending.append([r, pool.submit(ex.admit_async, r)])
                    else:
                        try:
                            member = ex.admit(r)
                        except Exception as e:                   # this request only
                            used -= need_res
                            _end(r, "failed", ex.now() - t0, e)
                        else:
                            active.append([r, member, r.steps])
                    peak = max(peak, used + transient + (0 if asynchronous else need_tmp))
                    qi += 1
                # ---- set-ups that finished join the batch (or fail alone) ----
                still = []
                for r, fut in pending:
                    if fut.done():
                        transient -= ex.footprint(r)[1]
                        try:
                            member = fut.result()
                        except Exception as e:
                            used -= ex.footprint(r)[0]
                            _end(r, "failed", ex.now() - t0, e)
                            continue
                        active.append([r, member, r.steps])
                    else:
                        still.append([r, fut])
                pending = still
                # ---- clients that gave up leave at this chunk boundary ----
                gone = [a for a in active if _gave_up(a[0], now)]
                if gone:
                    ex.sync()
                    for a in gone:
                        _discard(ex, a[1])
                        used -= ex.footprint(a[0])[0]
                        _end(a[0], "cancelled", ex.now() - t0)
                    active = [a for a in active if not _gave_up(a[0], now)]
                backlog = sum(1 for r in queue[qi:] if r.arrival <= now)
                backlog_max = max(backlog_max, backlog)
                if not active:
                    if pending:
                        import concurrent.futures as cf
                        cf.wait([f for _, f in pending], return_when=cf.FIRST_COMPLETED)
                    elif qi < len(queue):
                        ex.wait_until(t0 + queue[qi].arrival)
                    continue
                # ---- one chunk for all active members ----
                n = min(self.chunk_max, min(a[2] for a in active))
                ex.step([a[1] for a in active], n)
                chunks += 1
                total += n * sum(a[0].cells for a in active)
                for a in active:
                    a[2] -= n
                done = [a for a in active if a[2] == 0]
                if done:
                    ex.sync()
                    for a in done:
                        r = a[0]
                        used -= ex.footprint(r)[0]
                        try:
                            r.result = ex.retire(a[1])
                        except Exception as e:                   # this request only
                            _end(r, "failed", ex.now() - t0, e)
                            continue
                        r.finished = ex.now() - t0
                        r.status = "done"
                    active = [a for a in active if a[2] > 0]
                timeline.append((ex.now() - t0, len(active), used))
        finally:
            if pool is not None:
                pool.shutdown(wait=True)
        for r, fut in pending:          # only after an error: set-ups still in flight
            if fut.done() and fut.exception() is None:
                _discard(ex, fut.result())
        makespan = ex.now() - t0
        return ServeReport(queue, makespan, total, int(peak), chunks, backlog_max, timeline)


def _gave_up(r, now):
    return r.cancel_at is not None and r.cancel_at <= now


def _end(r, status, t, err=None):
    r.status = status
    r.error = None if err is None else "%s: %s" % (type(err).__name__, err)
    r.ended = t


def _discard(ex, member):
    """free a member without reading its result"""
    getattr(ex, "discard", ex.retire)(member)


class GpuExecutor:
    """Members are `Model`s of libraytracer_gb300.so; a chunk is one
    `Batch.integrate` (persistent, graph-captured launches)."""

    overlap_setup = True   # Server runs admit_async in worker threads

    def __init__(self, precision="fp32", tune=False, batch_tuning=None, persistent=None):
        self.precision = precision
        self.tune = tune
        self.batch_tuning = batch_tuning
        self.persistent = persistent     # consumer threads of the staged classes (None: library default)
        self._batch = None
        self._members = None
        # wall seconds spent per activity (set-up runs in worker threads and overlaps)
        self.times = {"setup": 0.0, "rebuild": 0.0, "step": 0.0, "sync": 0.0, "retire": 0.0}
        self.rebuilds = 0

    def now(self):
        return time.perf_counter()

    def wait_until(self, t):
        d = t - time.perf_counter()
        if d > 0:
            time.sleep(d)

    def footprint(self, r):
        res, tmp = bytes_per_cell(self.precision)
        return res * r.cells, tmp * r.cells

    def admit(self, r):
        from .configs import build_model
        t0 = time.perf_counter()
        m = build_model(r.exp, self.precision, padded=False)   # no padded host array
        self.times["setup"] += time.perf_counter() - t0
        return m

    def admit_async(self, r):
        """set-up in a worker thread: numpy work and the library calls
        release the interpreter lock, so it overlaps the running chunk"""
        return self.admit(r)

    def step(self, members, n):
        from .batch import Batch
        t0 = time.perf_counter()
        if self._members != [id(m) for m in members]:
            self.rebuilds += 1
            if self._batch is not None:
                self._batch.close()
            self._batch = Batch(members)
            if self.batch_tuning:
                self._batch.set_tuning(*self.batch_tuning)
                if self.persistent is not None:
                    self._batch.set_persistent(self.persistent)
            elif self.tune:
                from .autotune import tune_batch
                tune_batch(self._batch)
            self._members = [id(m) for m in members]
        t1 = time.perf_counter()
        self._batch.integrate(n)
        t2 = time.perf_counter()
        self.times["rebuild"] += t1 - t0
        self.times["step"] += t2 - t1

    def sync(self):
        if self._batch is not None:
            t0 = time.perf_counter()
            self._batch.sync()
            self.times["sync"] += time.perf_counter() - t0

    def retire(self, member):
        t0 = time.perf_counter()
        try:
            E = member.get_state()   # interior, in the member's precision
        finally:
            member.close()
        self.times["retire"] += time.perf_counter() - t0
        return E

    def discard(self, member):
        member.close()

    def close(self):
        if self._batch is not None:
            self._batch.close()
            self._batch = None


class SequentialExecutor(GpuExecutor):
    """Baseline: one request at a time, each stepped alone (rt_integrate),
    with the given step schedule (e.g. ("fast", 8, 256, 0) for binary64)."""

    overlap_setup = False  # set-up inline: no overlap in the baseline

    def __init__(self, precision="fp64", schedule=None):
        super().__init__(precision)
        self.schedule = schedule

    def admit(self, r):
        m = super().admit(r)
        if self.schedule:
            m.set_tuning(*self.schedule)
        return m

    def step(self, members, n):
        for m in members:
            m.integrate(n)

    def sync(self):
        pass


class FakeExecutor:
    """Virtual-clock executor for CPU tests of the scheduling logic: a chunk
    of n steps over members costs n * (launch + sum(cells) / rate) seconds,
    admission costs setup_s; results record which steps each member saw."""

    def __init__(self, rate=1e10, launch=1e-5, setup_s=1e-3, bpc=(36.0, 72.0), fail_admit=(), fail_retire=()):
        self.t = 0.0
        self.rate = rate
        self.launch = launch
        self.setup_s = setup_s
        self.bpc = bpc
        self.log = []
        self.fail_admit = set(fail_admit)     # request ids whose set-up raises
        self.fail_retire = set(fail_retire)   # request ids whose result read raises
        self.discarded = []

    def now(self):
        return self.t

    def wait_until(self, t):
        self.t = max(self.t, t)

    def footprint(self, r):
        return self.bpc[0] * r.cells, self.bpc[1] * r.cells

    def admit(self, r):
        self.t += self.setup_s
        if r.rid in self.fail_admit:
            raise RuntimeError("injected set-up failure of request %d" % r.rid)
        return {"rid": r.rid, "steps": 0, "cells": r.cells}

    def step(self, members, n):
        self.t += n * (self.launch + sum(m["cells"] for m in members) / self.rate)
        for m in members:
            m["steps"] += n
        self.log.append((self.t, [m["rid"] for m in members], n))

    def sync(self):
        pass

    def retire(self, member):
        if member["rid"] in self.fail_retire:
            raise RuntimeError("injected result failure of request %d" % member["rid"])
        return member["steps"]

    def discard(self, member):
        self.discarded.append(member["rid"])
