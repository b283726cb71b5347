"""Device parity at the benchmark configurations' own shapes.

The reference fixes the window at NUMSITES = 1,024 sites (src/globals.h:7-23);
this build takes S and the word count at run time, so the CUDA path is
checked against the CPU oracle at the sizes the benchmark runs:

  * plain: 256 samples x 1,024 sites, uniform surrogates, C = 100, the whole
    24-generation schedule (8 annealed + 16 sampling) bit for bit against the
    oracle's loop, plus every sample's per-proposal log-likelihoods of one
    annealed and one full-penalty generation;
  * batched: 10,000 samples x 4,096 sites, C = 100, surrogates from the
    device-built K = 200 Hamming-neighbour table (KNN::ClusterHaps,
    kNN.cpp:99-206), one generation in the annealing ramp and one at full
    penalty; a seeded subset of 256 samples replayed on the oracle; and the
    same shape scored from 4-bit VQ GL codes;
  * panel: 2,000 samples + 10,000 panel haplotypes x 8,192 sites; generation 0
    draws its surrogates from the panel only (the kick-start), generation 1
    from panel and samples with every chain's first proposal from the panel
    (--kickstart, insti.cpp:1505-1511); 256 samples replayed each;
  * uneven: three chunks of 8,192, 12,288 and 16,384 sites in one batched
    launch (glp_run_batch), every sample replayed, and each chunk alone equal
    to its part of the batch.

Tolerances are those of tests/parity_check.py: per-proposal log-likelihood
within 1e-5 relative of the binary32 oracle and of binary64; quadruples,
accept decisions (outside near-ties) and sampled haplotype words exact.
"""
import ctypes as C

import numpy as np
import pytest

from glphase_gb300 import native as nat, synth
from glphase_gb300.batch import anneal_pen
from parity_check import check_samples, report

pytestmark = pytest.mark.gpu


def _engine_generation(eng, pen, seed, gen, nbr=None, lo=0, hi=0, kick=0, kick_first=False):
    """One device-resident generation with its traces; returns host copies
    of the outputs and of the generation's input haplotypes."""
    import torch
    N, C_ = eng.N, eng.C
    evals = torch.full((N, C_ + 1), float("nan"), dtype=torch.float64, device=eng.device)
    acc = torch.zeros((N, C_), dtype=torch.uint8, device=eng.device)
    haps_in = eng.haps.cpu().numpy().view(np.uint64).copy()
    a = eng.args(None, None, pen, seed, gen, eval_trace=evals, accept_trace=acc,
                 neighbors=nbr, kick_first=kick_first)
    if kick:
        a.sample_lo, a.sample_hi, a.kick_start = lo, hi, 1
    eng.launch(a)
    eng.finish()
    out = dict(quad=eng.quad.cpu().numpy().view(np.uint32),
               hnew=eng.hnew.cpu().numpy().view(np.uint64),
               like=eng.like.cpu().numpy(), evals=evals.cpu().numpy(),
               acc=acc.cpu().numpy())
    eng.swap()
    return haps_in, out


def _subset(N, n, seed):
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(N, size=min(n, N), replace=False))


def test_plain_config_full_schedule(oracle_lib):
    """256 x 1,024, uniform surrogates, C = 100: the 24-generation schedule
    equals the oracle's loop bit for bit; one annealed and one full-penalty
    generation checked evaluation by evaluation on every sample."""
    from glphase_gb300 import phase as ph
    from glphase_gb300.hmmlike import Engine
    from phase_oracle import oracle_phase
    O = oracle_lib
    w = synth.CONFIGS["plain"]
    ds = synth.generate(w)
    m, haps = synth.initial_state(ds)
    opts = ph.PhaseOptions(sa_burnin=w.burnin, burnin=0, sampling=w.sampling,
                           cycles=w.cycles, seed=5)
    prob, final = ph.phase(m, haps, opts)
    want_prob, want_haps = oracle_phase(O, m, haps, opts)
    assert np.array_equal(final, want_haps)
    assert np.array_equal(prob, want_prob)
    eng = Engine(m.emit, m.t, m.tran, m.pc, haps, w.cycles)
    try:
        worst = worst64 = 0.0
        for gen in (2, 9):
            pen = float(anneal_pen(gen, w.burnin))
            h_in, out = _engine_generation(eng, pen, 17, gen)
            quad, props = O.sample_surrogates(17, gen, m.N, w.cycles, 0, h_in.shape[0])
            a, b = check_samples(O, m.emit, m.t, m.tran, m.pc, h_in, quad, props, pen, out,
                                 range(m.N), 17, gen)
            worst, worst64 = max(worst, a), max(worst64, b)
    finally:
        eng.dev.cleanup()
    report("plain 256x1024 C=100", worst, worst64, 2 * m.N, generations=24)


def test_batched_config_shape(oracle_lib):
    """10,000 x 4,096, C = 100, K = 200 device kNN surrogates: 256 seeded
    samples of an annealed and of a full-penalty generation replayed on the
    oracle."""
    from glphase_gb300.hmmlike import Engine
    O = oracle_lib
    w = synth.CONFIGS["batched"]
    ds = synth.generate(w)
    m, haps = synth.initial_state(ds)
    assert (m.N, m.S) == (10000, 4096)
    eng = Engine(m.emit, m.t, m.tran, m.pc, haps, w.cycles)
    try:
        nbr = eng.knn(w.knn)
        eng.finish()  # the table is built on the library's stream
        nbr_host = np.ascontiguousarray(nbr.cpu().numpy().view(np.uint32)[:m.N])
        worst = worst64 = 0.0
        checked = 0
        for gen in (3, 9):
            pen = float(anneal_pen(gen, w.burnin))
            h_in, out = _engine_generation(eng, pen, 23, gen, nbr=nbr)
            quad, props = O.sample_surrogates(23, gen, m.N, w.cycles, 0, h_in.shape[0],
                                              nbr=nbr_host)
            sub = _subset(m.N, 256, gen)
            a, b = check_samples(O, m.emit, m.t, m.tran, m.pc, h_in, quad, props, pen, out,
                                 sub, 23, gen)
            worst, worst64 = max(worst, a), max(worst64, b)
            checked += len(sub)
            # the samples outside the subset still finished their chains
            assert np.isfinite(out["evals"][:, 0]).all()
            assert (out["quad"] < h_in.shape[0]).all()
    finally:
        eng.dev.cleanup()
    report("batched 10000x4096 C=100 kNN K=200", worst, worst64, checked)


def test_batched_vq_config_shape(oracle_lib):
    """10,000 x 4,096, C = 100, K = 200 device kNN surrogates, likelihoods
    from 4-bit VQ GL codes (GLPack / GLVQ, trained and packed by the device
    codec): 256 seeded samples of a full-penalty generation replayed on the
    oracle's VQ emission."""
    from glphase_gb300.glpack import GLPack
    from glphase_gb300.hmmlike import Engine, HMMLikeCUDA
    O = oracle_lib
    w = synth.CONFIGS["batched"]
    ds = synth.generate(w)
    m, haps = synth.initial_state(ds)
    codec = HMMLikeCUDA(0)
    try:
        gp = GLPack(m.t, np.random.default_rng(1), device=codec)
        packed, cb = gp.packed_gls(), gp.code_book()
    finally:
        codec.cleanup()
    eng = Engine(m.emit, m.t, m.tran, m.pc, haps, w.cycles, packed=packed, codebook=cb)
    try:
        nbr = eng.knn(w.knn)
        eng.finish()
        nbr_host = np.ascontiguousarray(nbr.cpu().numpy().view(np.uint32)[:m.N])
        gen = 9
        pen = float(anneal_pen(gen, w.burnin))
        h_in, out = _engine_generation(eng, pen, 31, gen, nbr=nbr)
        quad, props = O.sample_surrogates(31, gen, m.N, w.cycles, 0, h_in.shape[0],
                                          nbr=nbr_host)
        sub = _subset(m.N, 256, 77)
        worst, worst64 = check_samples(O, m.emit, m.t, m.tran, m.pc, h_in, quad, props, pen,
                                       out, sub, 31, gen, vq=(packed, cb))
        assert np.isfinite(out["evals"][:, 0]).all()
    finally:
        eng.dev.cleanup()
    report("batched VQ 10000x4096 C=100 kNN K=200", worst, worst64, len(sub))


def test_panel_config_shape(oracle_lib):
    """2,000 samples + 10,000 panel haplotypes x 8,192 sites: generation 0
    from the panel only, generation 1 from everything with each chain's first
    proposal from the panel; 256 samples of each replayed."""
    from glphase_gb300.hmmlike import Engine
    O = oracle_lib
    w = synth.CONFIGS["panel"]
    ds = synth.generate(w)
    m, haps = synth.initial_state(ds)
    N, H = m.N, haps.shape[0]
    assert (N, m.S, H) == (2000, 8192, 2 * 2000 + 10000)
    eng = Engine(m.emit, m.t, m.tran, m.pc, haps, w.cycles)
    try:
        worst = worst64 = 0.0
        checked = 0
        for gen, kick, kick_first in ((0, True, False), (1, False, True)):
            pen = float(anneal_pen(gen, w.burnin))
            h_in, out = _engine_generation(eng, pen, 29, gen, lo=2 * N, hi=H,
                                           kick=kick, kick_first=kick_first)
            lo = 2 * N if kick else 0
            quad, props = O.sample_surrogates(29, gen, N, w.cycles, lo, H,
                                              kick_first=kick_first, H=H)
            if kick:
                assert quad.min() >= 2 * N and props.min() >= 2 * N
            if kick_first:
                assert props[0].min() >= 2 * N
            sub = _subset(N, 256, 40 + gen)
            a, b = check_samples(O, m.emit, m.t, m.tran, m.pc, h_in, quad, props, pen, out,
                                 sub, 29, gen)
            worst, worst64 = max(worst, a), max(worst64, b)
            checked += len(sub)
            # panel rows are never rewritten
            assert np.array_equal(out["hnew"][2 * N:], h_in[2 * N:])
    finally:
        eng.dev.cleanup()
    report("panel 2000+10000x8192 C=100", worst, worst64, checked)


def test_uneven_long_chunks_in_one_batch(oracle_lib):
    """Chunks of 8,192, 12,288 and 16,384 sites in one persistent launch:
    every sample replayed on the oracle, and each chunk alone identical to
    its part of the batch."""
    import torch
    from glphase_gb300 import synth_device as sd
    from glphase_gb300.batch import DeviceProblem
    from glphase_gb300.hmmlike import HMMLikeCUDA
    O = oracle_lib
    dev = HMMLikeCUDA(0)
    shapes = [(96, 8192), (80, 12288), (64, 16384)]
    C_, gen, burnin = 100, 4, 8
    pen = float(anneal_pen(gen, burnin))
    probs = []
    try:
        for i, (N, S) in enumerate(shapes):
            w = synth.Workload(f"u{i}", N=N, S=S, founders=40, depth=4.0, burnin=burnin,
                               sampling=24, seed=60 + i)
            probs.append(DeviceProblem(dev, sd.generate(w, N, S, seed=60 + i), C_,
                                       seed=800 + i, burnin=burnin))
        torch.cuda.synchronize()
        traces = []
        for p in probs:
            ev = torch.full((p.N, C_ + 1), float("nan"), dtype=torch.float64,
                            device=p.haps.device)
            ac = torch.zeros((p.N, C_), dtype=torch.uint8, device=p.haps.device)
            traces.append((ev, ac))
        h_in = [p.haps.cpu().numpy().view(np.uint64).copy() for p in probs]

        def run(members):
            args = []
            for p, (ev, ac) in members:
                a = p.args(gen)
                a.eval_trace, a.accept_trace = ev.data_ptr(), ac.data_ptr()
                args.append(a)
            arr = (nat.GenerationArgs * len(args))(*args)
            pbs = (C.c_void_p * len(args))(*[p.pb for p, _ in members])
            dev._c(dev.L.glp_run_batch(dev.ctx, len(args), pbs, arr))
            dev._c(dev.L.glp_finish(dev.ctx))
            return [dict(quad=p.quad.cpu().numpy().view(np.uint32),
                         hnew=p.hnew.cpu().numpy().view(np.uint64),
                         like=p.like.cpu().numpy(), evals=ev.cpu().numpy(),
                         acc=ac.cpu().numpy()) for p, (ev, ac) in members]

        batched = run(list(zip(probs, traces)))
        worst = worst64 = 0.0
        for p, out, hin in zip(probs, batched, h_in):
            ch = p.chunk
            emit = ch.emit.cpu().numpy()
            prob = ch.prob.cpu().numpy()
            quad, props = O.sample_surrogates(p.seed, gen, p.N, C_, 0, p.H)
            a, b = check_samples(O, emit, prob, ch.tran, ch.pc, hin, quad, props, pen, out,
                                 range(p.N), p.seed, gen)
            worst, worst64 = max(worst, a), max(worst64, b)
        for p, t, out in zip(probs, traces, batched):
            alone = run([(p, t)])[0]
            for k in ("quad", "like", "evals", "acc"):
                assert np.array_equal(out[k], alone[k], equal_nan=True), k
            assert np.array_equal(out["hnew"][:2 * p.N], alone["hnew"][:2 * p.N])
    finally:
        for p in probs:
            p.close()
        dev.cleanup()
    report("uneven chunks 96x8192 + 80x12288 + 64x16384 in one batch", worst, worst64,
           sum(n for n, _ in shapes))
