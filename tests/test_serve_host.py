"""Host logic of the serving loop (glphase_gb300/serve.py) without a GPU:
admission against the HBM budget, one generation per resident request per
tick (one launch for the batched form, one per request for the plain form,
a mixed-generation launch when residents are at different generations),
retirement and latency bookkeeping; and the NativeServer wrapper over the
library's glp_server_* calls.  The device calls are faked; the GPU
behaviour (results identical alone and in the mix) is tests/test_gpu_serve.py,
and the library's own scheduling is tests/test_server_core.py."""
from dataclasses import dataclass

import pytest

from glphase_gb300 import serve


@dataclass
class Chunk:
    N: int
    S: int
    H: int

    @property
    def wn(self):
        return (self.S + 63) // 64


class FakeLib:
    def __init__(self, log):
        self.log = log

    def glp_finish(self, ctx):
        self.log.append(("finish",))
        return 0

    def glp_run_batch(self, ctx, n, pbs, args):
        self.log.append(("mixed", n))
        return 0


class FakeDev:
    def __init__(self):
        self.log = []
        self.L = FakeLib(self.log)
        self.ctx = None

    def _c(self, rc):
        assert rc == 0


class FakeProblem:
    def __init__(self, dev, chunk, cycles, seed, burnin, vq=None):
        self.chunk, self.seed = chunk, seed
        self.haps, self.hnew = "a", "b"
        self.like = None
        self.pb = None  # the C problem handle the mixed launch passes
        self.closed = False

    def args(self, generation):
        from glphase_gb300 import native as nat
        a = nat.GenerationArgs()
        a.generation = generation
        return a

    def swap(self):
        self.haps, self.hnew = self.hnew, self.haps

    def close(self):
        self.closed = True


@pytest.fixture
def fake(monkeypatch):
    dev = FakeDev()
    launches = []

    def run_batch(d, problems, generation):
        launches.append((len(problems), generation))
        for p in problems:
            p.swap()

    monkeypatch.setattr(serve, "DeviceProblem", FakeProblem)
    monkeypatch.setattr(serve, "run_batch", run_batch)
    return dev, launches


def request(rid, N=100, S=640, G=3, arrival=0.0):
    return serve.Request(rid, Chunk(N, S, 2 * N), generations=G, cycles=10, seed=rid, burnin=2,
                         arrival=arrival)


def test_footprint_counts_every_buffer():
    r = request(0, N=100, S=640)
    assert r.footprint() == 100 * 640 * (16 + 12 + 16) + 2 * 200 * 10 * 8
    assert r.updates == 100 * 11 * 640 * 3


def test_admission_waits_for_memory(fake):
    dev, launches = fake
    a, b = request(0), request(1)
    srv = serve.Server(dev, budget_bytes=a.footprint() + b.footprint() // 2)
    srv.submit(a)
    srv.submit(b)
    assert srv.tick(0.0) == []           # only a fits
    assert [r.rid for r in srv.active] == [0] and [r.rid for r in srv.queue] == [1]
    srv.tick(0.1)
    done = srv.tick(0.2)                  # a finishes its 3 generations
    assert [r.rid for r in done] == [0] and a.problem.closed and srv.used == 0
    srv.tick(0.3)                         # b admitted once a left
    assert [r.rid for r in srv.active] == [1]
    assert launches == [(1, 0), (1, 1), (1, 2), (1, 0)]
    with pytest.raises(ValueError, match="more than the budget"):
        big = serve.Server(dev, budget_bytes=10)
        big.submit(request(2))
        big.tick(0.0)


def test_batched_ticks_share_one_launch_and_mix_generations(fake):
    dev, launches = fake
    a, b = request(0, G=2), request(1, G=2)
    srv = serve.Server(dev, budget_bytes=1 << 40)
    srv.submit(a)
    srv.tick(0.0)                         # a alone at generation 0
    srv.submit(b)
    srv.tick(0.1)                         # a at 1, b at 0: one mixed launch
    assert ("mixed", 2) in dev.log
    assert launches == [(1, 0)]
    assert a.gen == 2 and b.gen == 1 and srv.active == [b]
    assert srv.stats.updates == a.chunk.N * 11 * a.chunk.S * 2 + b.chunk.N * 11 * b.chunk.S
    assert srv.stats.peak_resident == 2


def test_plain_form_launches_per_request(fake):
    dev, launches = fake
    srv = serve.Server(dev, budget_bytes=1 << 40, plain=True)
    for i in range(3):
        srv.submit(request(i, G=1))
    done = srv.tick(0.0)
    assert launches == [(1, 0), (1, 0), (1, 0)]
    assert sorted(r.rid for r in done) == [0, 1, 2] and srv.active == []


def test_serve_records_latencies(fake):
    dev, _ = fake
    reqs = [request(i, G=2, arrival=0.0) for i in range(4)]
    stats = serve.Server(dev, budget_bytes=1 << 40).serve(reqs, time_limit=30)
    assert len(stats.latencies) == 4 and all(l >= 0 for l in stats.latencies)
    s = stats.summary()
    assert s["requests"] == 4 and s["ticks"] == 2 and s["p99_latency_s"] >= s["p50_latency_s"]


class FakeServerLib(FakeLib):
    """glp_server_* over a small Python model of the library's scheduling:
    FIFO admission under the budget, one generation per resident request
    per tick, retirement, release."""

    def __init__(self, log):
        super().__init__(log)
        self.reqs, self.queue, self.active = {}, [], []
        self.budget = self.used = self.ticks = self.updates = 0
        self.released = []

    def glp_last_error(self, ctx):
        return b"request needs many bytes, more than the budget"

    def glp_server_create(self, ctx, budget, plain, out):
        self.budget = budget
        out._obj.value = 1
        return 0

    def glp_server_submit(self, srv, pb, args, G, rid):
        a = args._obj
        need = a.num_samples * a.num_sites * 44 + 2 * a.num_haps * ((a.num_sites + 63) // 64) * 8
        if need > self.budget:
            return 1
        i = len(self.reqs) + 1
        self.reqs[i] = dict(G=G, gen=0, need=need, state=0, haps=a.haps, hnew=a.hnew,
                            upd=a.num_samples * (a.num_cycles + 1) * a.num_sites)
        self.queue.append(i)
        rid._obj.value = i
        return 0

    def glp_server_tick(self, srv, resident, finished):
        while self.queue and self.used + self.reqs[self.queue[0]]["need"] <= self.budget:
            i = self.queue.pop(0)
            self.used += self.reqs[i]["need"]
            self.reqs[i]["state"] = 1
            self.active.append(i)
        resident._obj.value, finished._obj.value = len(self.active), 0
        if self.active:
            self.ticks += 1
        for i in list(self.active):
            r = self.reqs[i]
            r["gen"] += 1
            self.updates += r["upd"]
            if r["gen"] >= r["G"]:
                r["state"] = 2
                self.used -= r["need"]
                self.active.remove(i)
                finished._obj.value += 1
        return 0

    def glp_server_poll(self, srv, i, state, gen, ptr):
        r = self.reqs[i]
        state._obj.value, gen._obj.value = r["state"], r["gen"]
        ptr._obj.value = r["hnew"] if r["gen"] % 2 else r["haps"]
        return 0

    def glp_server_stats(self, srv, ticks, updates, used):
        ticks._obj.value, updates._obj.value, used._obj.value = \
            self.ticks, self.updates, self.used
        return 0

    def glp_server_release(self, srv, i):
        assert self.reqs[i]["state"] == 2
        self.released.append(i)
        return 0

    def glp_server_destroy(self, srv):
        self.log.append(("destroy",))


class Tensor:
    def __init__(self, addr):
        self.addr = addr

    def data_ptr(self):
        return self.addr


class PtrProblem(FakeProblem):
    _next = 0x1000

    def __init__(self, *a, **k):
        super().__init__(*a, **k)
        PtrProblem._next += 0x100
        self.haps, self.hnew = Tensor(PtrProblem._next), Tensor(PtrProblem._next + 8)

    def args(self, generation):
        a = super().args(generation)
        c = self.chunk
        a.num_samples, a.num_sites, a.num_cycles, a.num_haps = c.N, c.S, 10, c.H
        a.haps, a.hnew = self.haps.data_ptr(), self.hnew.data_ptr()
        return a


def test_native_server_wrapper(monkeypatch):
    """serve.NativeServer over the glp_server_* calls: queued requests move
    to active once the library admits them, finished ones take the buffer
    the library names as their result and are released."""
    dev = FakeDev()
    dev.L = FakeServerLib(dev.log)
    monkeypatch.setattr(serve, "DeviceProblem", PtrProblem)
    a, b, c = request(0, G=1), request(1, G=2), request(2, G=1)
    srv = serve.NativeServer(dev, budget_bytes=a.footprint() + b.footprint())
    for r in (a, b, c):
        srv.submit(r)
    assert [r.rid for r in srv.queue] == [0, 1, 2]
    done = srv.tick(0.0)                  # a and b resident; a finishes
    assert [r.rid for r in done] == [0] and [r.rid for r in srv.active] == [1]
    assert a.result_haps is a.problem.hnew and a.problem.closed
    assert [r.rid for r in srv.queue] == [2]
    done = srv.tick(0.1)                  # b finishes (its result back in haps); c admitted
    assert sorted(r.rid for r in done) == [1, 2]
    assert b.result_haps is b.problem.haps and c.result_haps is c.problem.hnew
    assert dev.L.released == [1, 2, 3] and srv.used == 0 and srv.stats.ticks == 2
    assert srv.stats.peak_resident == 2
    srv.close()
    assert ("destroy",) in dev.log
    big = serve.NativeServer(dev, budget_bytes=10)
    with pytest.raises(ValueError, match="more than the budget"):
        big.submit(request(5))
