"""Serving loop with continuous batching: a request's result is the same
alone and in a mix of requests that arrive while it is on the GPU; the HBM
budget bounds what is resident.  The library's own serving loop
(glp_server_*, through NativeServer) gives the Python loop's results bit for
bit, batched and plain."""
import pytest

from glphase_gb300 import synth, synth_device as sd
from glphase_gb300.hmmlike import HMMLikeCUDA
from glphase_gb300.serve import NativeServer, Request, Server

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev():
    import torch
    torch.cuda.init()
    d = HMMLikeCUDA(0)
    yield d
    d.cleanup()


def make(i, N, S, generations=6, arrival=0.0):
    w = synth.Workload(f"r{i}", N=N, S=S, founders=8, depth=3.0, burnin=3, sampling=3,
                       seed=40 + i)
    return Request(rid=i, chunk=sd.generate(w, N, S, seed=40 + i), generations=generations,
                   cycles=12, seed=900 + i, burnin=3, arrival=arrival)


def test_request_same_alone_and_in_mix(dev):
    import torch
    alone = Server(dev, budget_bytes=1 << 34)
    r = make(0, 60, 700)
    alone.serve([r])
    ref_haps = r.result_haps.clone()
    ref_like = r.result_like.clone()
    # the same request, arriving while three others are being served
    others = [make(1, 25, 130, 9, 0.0), make(2, 80, 1024, 4, 0.0), make(3, 7, 64, 7, 0.0)]
    r2 = make(0, 60, 700, arrival=0.01)
    mix = Server(dev, budget_bytes=1 << 34)
    st = mix.serve(others + [r2])
    assert st.peak_resident >= 2
    assert torch.equal(r2.result_haps, ref_haps)
    assert torch.equal(r2.result_like, ref_like)
    assert len(st.latencies) == 4


def test_budget_limits_residency(dev):
    reqs = [make(i, 30, 300, 3) for i in range(4)]
    one = reqs[0].footprint()
    srv = Server(dev, budget_bytes=int(one * 2.5))
    st = srv.serve(reqs)
    assert st.peak_resident == 2
    assert st.peak_bytes <= int(one * 2.5)
    assert len(st.latencies) == 4


def test_oversized_request_is_rejected(dev):
    r = make(0, 30, 300, 2)
    srv = Server(dev, budget_bytes=r.footprint() - 1)
    with pytest.raises(ValueError):
        srv.serve([r])


SPECS = [(0, 60, 700, 6), (1, 25, 130, 9), (2, 80, 1024, 4), (3, 7, 64, 7), (4, 33, 65, 1)]


@pytest.mark.parametrize("plain", [False, True])
def test_native_server_matches_python_server(dev, plain):
    import torch
    py = [make(i, N, S, G) for i, N, S, G in SPECS]
    ref = Server(dev, budget_bytes=1 << 34).serve(py)
    nat = [make(i, N, S, G) for i, N, S, G in SPECS]
    srv = NativeServer(dev, budget_bytes=1 << 34, plain=plain)
    st = srv.serve(nat)
    srv.close()
    assert st.ticks == ref.ticks == max(G for *_, G in SPECS)
    assert st.updates == ref.updates and st.peak_resident == len(SPECS)
    for a, b in zip(py, nat):
        assert b.gen == a.gen == a.generations
        assert torch.equal(a.result_haps, b.result_haps), a.rid
        assert torch.equal(a.result_like, b.result_like), a.rid


def test_native_server_budget_and_mix(dev):
    import torch
    alone = [make(i, 30, 300, 3) for i in range(4)]
    for r in alone:
        s = NativeServer(dev, budget_bytes=1 << 34)
        s.serve([r])
        s.close()
    reqs = [make(i, 30, 300, 3) for i in range(4)]
    one = reqs[0].footprint()
    srv = NativeServer(dev, budget_bytes=int(one * 2.5))
    st = srv.serve(reqs)
    assert st.peak_resident == 2 and st.peak_bytes <= int(one * 2.5)
    assert len(st.latencies) == 4 and srv.used == 0
    for a, b in zip(alone, reqs):
        assert torch.equal(a.result_haps, b.result_haps)
        assert torch.equal(a.result_like, b.result_like)
    srv.close()
    small = NativeServer(dev, budget_bytes=one - 1)
    with pytest.raises(ValueError, match="more than the budget"):
        small.submit(make(8, 30, 300, 2))
    small.close()
    # a request whose sizes disagree with its problem is refused at submit
    bad = make(7, 30, 300, 2)
    bad.chunk.H = 2 * 30 - 1
    srv = NativeServer(dev, budget_bytes=1 << 34)
    with pytest.raises(ValueError, match="num_haps"):
        srv.submit(bad)
    srv.close()


def test_native_server_mixes_emission_sources(dev):
    """Float and 4-bit VQ requests resident together: the tick launches each
    emission source on its own, and every request's result equals the one
    it gets alone."""
    import numpy as np
    import torch
    from glphase_gb300.glpack import GLPack

    def reqs():
        out = [make(i, N, S, G) for i, N, S, G in SPECS[:4]]
        for r in out[1::2]:
            gp = GLPack(r.chunk.prob.cpu().numpy(), np.random.default_rng(r.rid))
            r.vq = (gp.packed_gls(), gp.code_book())
        return out

    alone = reqs()
    for r in alone:
        s = NativeServer(dev, budget_bytes=1 << 34)
        s.serve([r])
        s.close()
    mix = reqs()
    srv = NativeServer(dev, budget_bytes=1 << 34)
    st = srv.serve(mix)
    srv.close()
    assert st.peak_resident == 4
    for a, b in zip(alone, mix):
        assert torch.equal(a.result_haps, b.result_haps), a.rid
        assert torch.equal(a.result_like, b.result_like), a.rid
