"""Serving loop for phasing requests on one GPU, with continuous batching.

A request is a phasing chunk (its own samples, sites, seed) that needs G MH
generations.  Requests wait in a queue; at every tick the server admits
queued requests whose device footprint (emission, genotype probabilities,
hmm_work scratch, two haplotype buffers) fits the remaining HBM budget, then
runs ONE generation of every resident request in one persistent launch
(glp_run_batch); each request advances by one generation per tick, at its
own generation index, and leaves when it has done G.  Requests therefore
join and leave while others are on the GPU, and their state (haplotypes,
model inputs) stays resident between ticks.

Every random draw is keyed by the request's own seed and generation, and a
sample's chain depends only on its own chunk, so a request's result is the
same alone and in any mix (tests/test_gpu_serve.py checks it bit for bit).

The plain form runs the same ticks with one launch per resident request.

``NativeServer`` runs the same loop inside the library (glp_server_*): the
queue, admission, per-request generation arguments and retirement are C++,
and Python only submits, ticks and polls.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from .batch import DeviceProblem, run_batch


@dataclass
class Request:
    rid: int
    chunk: object            # synth_device.DeviceChunk (model inputs on the device)
    generations: int
    cycles: int
    seed: int
    burnin: int
    arrival: float = 0.0     # seconds after the server clock starts
    admitted: float = -1.0
    finished: float = -1.0
    problem: DeviceProblem | None = None
    gen: int = 0
    vq: tuple | None = None  # (packed codes, codebook): VQ emissions instead of float

    @property
    def updates(self) -> int:
        c = self.chunk
        return c.N * (self.cycles + 1) * c.S * self.generations

    def footprint(self) -> int:
        c = self.chunk
        return c.N * c.S * (16 + 12 + 16) + 2 * c.H * c.wn * 8


@dataclass
class ServeStats:
    latencies: list = field(default_factory=list)
    ticks: int = 0
    updates: int = 0
    busy_s: float = 0.0
    wall_s: float = 0.0
    peak_resident: int = 0
    peak_bytes: int = 0

    def summary(self) -> dict:
        lat = np.array(self.latencies) if self.latencies else np.zeros(1)
        return {"requests": len(self.latencies), "ticks": self.ticks,
                "p50_latency_s": float(np.percentile(lat, 50)),
                "p99_latency_s": float(np.percentile(lat, 99)),
                "updates": self.updates,
                "updates_per_s": self.updates / self.wall_s if self.wall_s else 0.0,
                "busy_updates_per_s": self.updates / self.busy_s if self.busy_s else 0.0,
                "peak_resident": self.peak_resident,
                "peak_bytes": self.peak_bytes}


class Server:
    def __init__(self, dev, budget_bytes: int, plain: bool = False):
        self.dev = dev
        self.budget = budget_bytes
        self.plain = plain
        self.queue: list[Request] = []
        self.active: list[Request] = []
        self.used = 0
        self.stats = ServeStats()

    def submit(self, req: Request) -> None:
        self.queue.append(req)

    def _admit(self, now: float) -> None:
        while self.queue:
            r = self.queue[0]
            need = r.footprint()
            if need > self.budget:
                raise ValueError(f"request {r.rid} needs {need} bytes, more than the budget")
            if self.used + need > self.budget:
                break
            self.queue.pop(0)
            r.problem = DeviceProblem(self.dev, r.chunk, r.cycles, r.seed, r.burnin, vq=r.vq)
            r.admitted = now
            self.used += need
            self.active.append(r)
        self.stats.peak_resident = max(self.stats.peak_resident, len(self.active))
        self.stats.peak_bytes = max(self.stats.peak_bytes, self.used)

    def tick(self, now: float) -> list[Request]:
        """Admit, run one generation of every resident request, retire the
        finished ones.  Returns the requests that finished this tick."""
        self._admit(now)
        if not self.active:
            return []
        t0 = time.perf_counter()
        if self.plain:
            for r in self.active:
                run_batch(self.dev, [r.problem], r.gen)
        else:
            probs = [r.problem for r in self.active]
            gens = {r.gen for r in self.active}
            if len(gens) == 1:
                run_batch(self.dev, probs, gens.pop())
            else:
                self._run_mixed()
        self.dev._c(self.dev.L.glp_finish(self.dev.ctx))
        self.stats.busy_s += time.perf_counter() - t0
        self.stats.ticks += 1
        done = []
        for r in self.active:
            self.stats.updates += r.chunk.N * (r.cycles + 1) * r.chunk.S
            r.gen += 1
        for r in list(self.active):
            if r.gen >= r.generations:
                done.append(r)
                self.active.remove(r)
                self.used -= r.footprint()
                r.result_haps = r.problem.haps
                r.result_like = r.problem.like
                r.problem.close()
        return done

    def _run_mixed(self) -> None:
        """One launch over requests at different generation indices."""
        import ctypes as C
        from . import native as nat
        n = len(self.active)
        args = (nat.GenerationArgs * n)(*[r.problem.args(r.gen) for r in self.active])
        pbs = (C.c_void_p * n)(*[r.problem.pb for r in self.active])
        self.dev._c(self.dev.L.glp_run_batch(self.dev.ctx, n, pbs, args))
        for r in self.active:
            r.problem.swap()

    def serve(self, requests: list[Request], time_limit: float = 600.0) -> ServeStats:
        """Run until every request is done; arrivals follow r.arrival on the
        wall clock started here."""
        pending = sorted(requests, key=lambda r: r.arrival)
        t_start = time.perf_counter()
        while pending or self.queue or self.active:
            now = time.perf_counter() - t_start
            if now > time_limit:
                raise TimeoutError("serving loop exceeded its time limit")
            while pending and pending[0].arrival <= now:
                self.submit(pending.pop(0))
            if not self.queue and not self.active:
                time.sleep(max(0.0, min(pending[0].arrival - now, 0.05)))
                continue
            for r in self.tick(now):
                r.finished = time.perf_counter() - t_start
                self.stats.latencies.append(r.finished - r.arrival)
        self.stats.wall_s = time.perf_counter() - t_start
        return self.stats


class NativeServer(Server):
    """The serving loop of the C ABI (glp_server_create / submit / tick /
    poll): the same admission, generation arguments and retirement as
    ``Server``, run by the library.  A request's device problem is created
    when it is submitted (its model inputs are already on the device)."""

    def __init__(self, dev, budget_bytes: int, plain: bool = False):
        import ctypes as C
        super().__init__(dev, budget_bytes, plain)
        self.srv = C.c_void_p()
        dev._c(dev.L.glp_server_create(dev.ctx, budget_bytes, int(plain), C.byref(self.srv)))
        self._ids: dict[int, int] = {}

    def submit(self, req: Request) -> None:
        import ctypes as C
        from . import native as nat
        L = self.dev.L
        req.problem = DeviceProblem(self.dev, req.chunk, req.cycles, req.seed, req.burnin,
                                    vq=req.vq)
        a = req.problem.args(0)
        rid = C.c_uint64()
        rc = L.glp_server_submit(self.srv, req.problem.pb, C.byref(a), req.generations,
                                 C.byref(rid))
        if rc == nat.GLP_ERR_ARG:
            msg = L.glp_last_error(self.dev.ctx).decode()
            req.problem.close()
            raise ValueError(f"request {req.rid}: {msg}")
        self.dev._c(rc)
        self._ids[req.rid] = rid.value
        self.queue.append(req)

    def _poll(self, req: Request):
        import ctypes as C
        state, done, ptr = C.c_int(), C.c_uint32(), C.c_void_p()
        self.dev._c(self.dev.L.glp_server_poll(self.srv, self._ids[req.rid], C.byref(state),
                                               C.byref(done), C.byref(ptr)))
        return state.value, done.value, ptr.value

    def tick(self, now: float) -> list[Request]:
        import ctypes as C
        from . import native as nat
        L = self.dev.L
        resident, finished = C.c_uint32(), C.c_uint32()
        t0 = time.perf_counter()
        self.dev._c(L.glp_server_tick(self.srv, C.byref(resident), C.byref(finished)))
        if resident.value:
            self.stats.busy_s += time.perf_counter() - t0
        for r in list(self.queue):
            if self._poll(r)[0] != nat.GLP_REQ_QUEUED:
                self.queue.remove(r)
                r.admitted = now
                self.active.append(r)
        self.stats.peak_resident = max(self.stats.peak_resident, len(self.active))
        self.stats.peak_bytes = max(self.stats.peak_bytes,
                                    sum(r.footprint() for r in self.active))
        done = []
        for r in list(self.active):
            state, r.gen, ptr = self._poll(r)
            if state == nat.GLP_REQ_DONE:
                self.active.remove(r)
                p = r.problem
                r.result_haps = p.haps if ptr == p.haps.data_ptr() else p.hnew
                r.result_like = p.like
                p.close()
                self.dev._c(L.glp_server_release(self.srv, self._ids.pop(r.rid)))
                done.append(r)
        ticks, updates, used = C.c_uint64(), C.c_uint64(), C.c_uint64()
        self.dev._c(L.glp_server_stats(self.srv, C.byref(ticks), C.byref(updates),
                                       C.byref(used)))
        self.stats.ticks, self.stats.updates, self.used = ticks.value, updates.value, used.value
        return done

    def close(self) -> None:
        if self.srv:
            self.dev.L.glp_server_destroy(self.srv)
            self.srv = None
