"""Host logic of the serving loop (glphase_gb300/serve.py) without a GPU:
admission against the HBM budget, one generation per resident request per
tick (one launch for the batched form, one per request for the plain form,
a mixed-generation launch when residents are at different generations),
retirement and latency bookkeeping.  The device calls are faked; the GPU
behaviour (results identical alone and in the mix) is tests/test_gpu_serve.py."""
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
