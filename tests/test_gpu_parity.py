"""GPU parity: the CUDA generation kernel through the C ABI against the CPU
oracle on the same inputs and the same random streams.

Tolerances (stated per the parity contract):
  * per-proposal log-likelihood: |gpu - oracle_fp32| <= 1e-5 * |oracle_fp32|
    (the reference's own FP32 implementation, impute.cpp:327-376), and the
    same bound against the FP64 yardstick;
  * accept decisions identical except where |delta*pen - ln u| < 1e-4;
  * quadruples and sampled haplotype words bit-exact given identical
    decisions (hmm_work runs in the reference's exact binary32 order).
"""
import ctypes as C
import math

import numpy as np
import pytest

from glphase_gb300 import model as mdl, native as nat, synth
from glphase_gb300.hmmlike import HMMLikeCUDA

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5
TIE_TOL = 1e-4


def _p(a):
    return None if a is None else a.ctypes.data


def make_problem(N=24, S=300, C=20, panel=0, seed=3, founders=6, depth=3.0):
    w = synth.Workload("t", N=N, S=S, founders=founders, depth=depth, burnin=1, sampling=1,
                       cycles=C, panel_haps=panel, seed=seed)
    ds = synth.generate(w)
    m, haps = synth.initial_state(ds, seed=seed + 1)
    rng = np.random.default_rng(seed + 2)
    quad, props = synth.uniform_proposals(N, haps.shape[0], C, rng)
    return m, haps, quad, props


def run_gpu(dev, m, haps, quad, props, pen, seed=11, gen=0, flags=0, trace=None):
    N, S = m.N, m.S
    H, wn = haps.shape
    Cc = props.shape[0]
    dev.copy_tran_to_device(m.tran)
    dev.copy_mutation_mat_to_device(m.pc)
    dev.copy_emission_to_device(m.emit, m.t)
    a = nat.GenerationArgs()
    a.num_samples, a.num_sites, a.num_cycles, a.num_haps = N, S, Cc, H
    haps = np.ascontiguousarray(haps)
    hnew = haps.copy()
    quad_in = np.ascontiguousarray(quad, dtype=np.uint32)
    quad_out = np.zeros_like(quad_in)
    props_c = np.ascontiguousarray(props, dtype=np.uint32)
    like = np.zeros(N, np.float64)
    evals = np.full((N, Cc + 1), np.nan, np.float64)
    acc = np.zeros((N, max(Cc, 1)), np.uint8)
    a.haps, a.hnew = _p(haps), _p(hnew)
    a.hap_idxs_in, a.hap_idxs_out, a.props = _p(quad_in), _p(quad_out), _p(props_c)
    a.pen, a.seed, a.generation, a.flags = pen, seed, gen, flags
    if trace is not None:
        slot, u_mh, u_work = (np.ascontiguousarray(x) for x in trace)
        a.trace_slot, a.trace_accept, a.trace_work = _p(slot), _p(u_mh), _p(u_work)
    a.like_out, a.eval_trace, a.accept_trace = _p(like), _p(evals), _p(acc)
    rc = dev.L.glp_run_generation_host(dev.ctx, C.byref(a))
    if rc != nat.GLP_OK:
        raise nat.GlpError(rc, dev.L.glp_last_error(dev.ctx).decode())
    return dict(quad=quad_out, hnew=hnew, like=like, evals=evals, acc=acc[:, :Cc])


@pytest.fixture(scope="module")
def dev():
    d = HMMLikeCUDA(0)
    yield d
    d.cleanup()


def check_against_oracle(O, m, haps, quad, props, pen, out, seed, gen, trace=None,
                         check_work=True):
    N, S = m.N, m.S
    C = props.shape[0]
    pb = O.OracleProblem(haps, m.emit, m.t, m.tran, m.pc, C)
    tr = pb.trace(seed=seed, generation=gen) if trace is None else \
        pb.trace(slot=trace[0], u_mh=trace[1], u_work=trace[2])
    worst = worst64 = 0.0
    for s in range(N):
        like32, like64, own, qf = O.replay_sample(pb, tr, s, quad, props, pen, out["acc"][s])
        g = out["evals"][s]
        assert np.all(np.isfinite(g)), s
        rel = np.abs(g - like32.astype(np.float64)) / np.abs(like32.astype(np.float64))
        rel64 = np.abs(g - like64) / np.abs(like64)
        worst, worst64 = max(worst, rel.max()), max(worst64, rel64.max())
        assert rel.max() <= REL_TOL, (s, rel.max())
        assert rel64.max() <= REL_TOL, (s, rel64.max())
        # decisions identical except at near-ties
        if trace is None:
            slots, us = O.mh_draws(seed, gen, s, C)
        else:
            us = trace[1][s]
        curr = float(like32[0])
        for c in range(C):
            if own[c] != out["acc"][s, c]:
                d = (float(like32[c + 1]) - curr) * pen
                assert abs(d - math.log(max(us[c], 1e-300))) < TIE_TOL, (s, c)
            if out["acc"][s, c]:
                curr = float(like32[c + 1])
        assert np.array_equal(qf, out["quad"][:, s]), s
        assert out["like"][s] == g[np.where(np.r_[1, out["acc"][s]] == 1)[0][-1]]
        if check_work:
            u = O.work_uniforms(seed, gen, s, S) if trace is None else trace[2][s]
            ha, hb = O.hmm_work(m.emit[s], m.t[s], m.tran, m.pc, haps, qf, pen, u)
            assert np.array_equal(ha, out["hnew"][2 * s]), s
            assert np.array_equal(hb, out["hnew"][2 * s + 1]), s
    return worst, worst64


@pytest.mark.parametrize("S", [1, 2, 7, 8, 9, 16, 17, 24, 25, 33, 63, 64, 65, 130, 136, 300,
                               513, 1024, 1088, 1100, 2049])
def test_generation_matches_oracle_sites(dev, oracle_lib, S):
    # past 1,024 sites hmm_work's sampling pass splits a sample's words into
    # 16-word parts: 1,088 and 1,100 sites end on a one- and a two-word part,
    # 2,049 on a part of one word holding one site
    m, haps, quad, props = make_problem(N=16, S=S, C=12)
    out = run_gpu(dev, m, haps, quad, props, 1.0, seed=7, gen=1)
    check_against_oracle(oracle_lib, m, haps, quad, props, 1.0, out, 7, 1)


@pytest.mark.parametrize("lanes", [1, 2, 4, 8, 16, 32])
def test_speculation_width_is_exact(dev, oracle_lib, lanes):
    """Every speculation width gives the sequential chain's results."""
    m, haps, quad, props = make_problem(N=40, S=257, C=30, seed=5)
    dev.set_lanes_per_sample(lanes)
    try:
        out = run_gpu(dev, m, haps, quad, props, 0.3, seed=3, gen=2)
    finally:
        dev.set_lanes_per_sample(0)
    check_against_oracle(oracle_lib, m, haps, quad, props, 0.3, out, 3, 2, check_work=False)
    dev.set_lanes_per_sample(1)
    try:
        ref = run_gpu(dev, m, haps, quad, props, 0.3, seed=3, gen=2)
    finally:
        dev.set_lanes_per_sample(0)
    assert np.array_equal(out["quad"], ref["quad"])
    assert np.array_equal(out["evals"], ref["evals"], equal_nan=True)
    assert np.array_equal(out["hnew"], ref["hnew"])


@pytest.mark.parametrize("S", [700, 1024])
def test_tiny_emissions_take_the_site_by_site_path(dev, oracle_lib, S):
    """Blocks of 8 sites that shrink the state by more than 2^-124 leave the
    range of block normalisation; those evaluations are recomputed site by
    site and still match the oracle."""
    m, haps, quad, props = make_problem(N=16, S=S, C=12, seed=13)
    m.emit = m.emit.copy()
    m.emit[:, 200:240] *= np.float32(1e-7)        # forward half
    m.emit[::2, S - 100:S - 80] *= np.float32(1e-9)  # backward half
    dev.set_block_sites(8)
    try:
        out = run_gpu(dev, m, haps, quad, props, 1.0, seed=7, gen=1)
        assert dev.counters()[3] > 0  # some evaluations took the site-by-site path
    finally:
        dev.set_block_sites(0)
    check_against_oracle(oracle_lib, m, haps, quad, props, 1.0, out, 7, 1)


def confident_problem():
    """Sites 100..159 of every sample scaled by 1e-6: an 8-site block there
    shrinks the state by about 2^-170, beyond one normalisation's 2^-124; a
    4-site block by about 2^-85."""
    m, haps, quad, props = make_problem(N=16, S=700, C=12, seed=13)
    m.emit = m.emit.copy()
    m.emit[:, 100:160] *= np.float32(1e-6)
    return m, haps, quad, props


@pytest.mark.parametrize("sites", [8, 4])
def test_block_sites_match_oracle(dev, oracle_lib, sites):
    m, haps, quad, props = confident_problem()
    dev.set_block_sites(sites)
    try:
        assert dev.block_sites() == sites
        out = run_gpu(dev, m, haps, quad, props, 1.0, seed=7, gen=1)
        ev, redo = dev.counters()[0], dev.counters()[3]
    finally:
        dev.set_block_sites(0)
    if sites == 8:
        assert redo > 0
    else:
        assert redo == 0
    check_against_oracle(oracle_lib, m, haps, quad, props, 1.0, out, 7, 1)


def test_block_sites_switch_automatically(dev):
    m, haps, quad, props = confident_problem()
    dev.set_block_sites(0)
    assert dev.block_sites() == 8
    try:
        run_gpu(dev, m, haps, quad, props, 1.0, seed=7, gen=1)
        ev, redo = dev.counters()[0], dev.counters()[3]
        assert redo * 1000 > ev
        assert dev.block_sites() == 4    # the next launch normalises every 4 sites
        run_gpu(dev, m, haps, quad, props, 1.0, seed=7, gen=2)
        assert dev.counters()[3] == 0
    finally:
        dev.set_block_sites(0)
    assert dev.block_sites() == 8
    with pytest.raises(nat.GlpError):
        dev.set_block_sites(5)


def test_counters_describe_the_generation(dev):
    m, haps, quad, props = make_problem(N=40, S=512, C=20, seed=8)
    run_gpu(dev, m, haps, quad, props, 1.0, seed=2, gen=0)
    ev, rounds, acc, redo, warp_rounds, lanes = dev.counters()
    assert ev >= 40 * 21 and rounds > 0 and 0 <= acc <= 40 * 20
    assert redo == 0  # ordinary emissions never leave the block range
    assert warp_rounds > 0 and 0 < lanes <= 32 * warp_rounds


def test_evals_per_lane_argument(dev):
    for bad in (2, 3):
        with pytest.raises(nat.GlpError):
            dev.set_evals_per_lane(bad)
    dev.set_evals_per_lane(1)
    dev.set_evals_per_lane(0)


@pytest.mark.parametrize("pen", [1.0, 0.25, 0.015625])
def test_penalty_and_hmm_work(dev, oracle_lib, pen):
    m, haps, quad, props = make_problem(N=32, S=500, C=16, seed=9)
    out = run_gpu(dev, m, haps, quad, props, pen, seed=21, gen=3)
    check_against_oracle(oracle_lib, m, haps, quad, props, pen, out, 21, 3)


def test_trace_replay_mode(dev, oracle_lib):
    m, haps, quad, props = make_problem(N=20, S=200, C=25, seed=12)
    rng = np.random.default_rng(4)
    trace = (rng.integers(0, 4, (m.N, 25)).astype(np.uint8), rng.random((m.N, 25)),
             rng.random((m.N, m.S)).astype(np.float32))
    out = run_gpu(dev, m, haps, quad, props, 0.5, trace=trace)
    check_against_oracle(oracle_lib, m, haps, quad, props, 0.5, out, 0, 0, trace=trace)


def test_reference_panel_rows_and_zero_cycles(dev, oracle_lib):
    m, haps, quad, props = make_problem(N=10, S=190, C=0, panel=30, seed=2)
    assert haps.shape[0] == 2 * 10 + 30
    quad = np.random.default_rng(1).integers(20, 50, (4, 10)).astype(np.uint32)
    out = run_gpu(dev, m, haps, quad, props, 1.0, seed=2)
    check_against_oracle(oracle_lib, m, haps, quad, props, 1.0, out, 2, 0)
    assert np.array_equal(out["hnew"][20:], haps[20:])  # panel rows untouched


def test_golden_likelihoods_from_reference(dev, golden):
    """GPU log-likelihoods against values produced by the reference's own
    impute.cpp (tests/golden/reference_vectors.npz), C = 0 evaluations."""
    g = golden
    N, S = int(g["N"]), int(g["S"])

    class M:
        pass
    m = M()
    m.N, m.S, m.emit, m.t, m.tran, m.pc = N, S, g["emit"], g["t"], g["tran"], g["pc"].reshape(4, 4)
    H = g["haps"].shape[0]
    for i in range(len(g["like_ref"])):
        s = int(g["like_sample"][i])
        quad = np.zeros((4, N), np.uint32)
        quad[:, :] = np.array([(2 * ((s + 1) % N)) % H] * 4, np.uint32)[:, None]
        quad[:, s] = g["like_quad"][i]
        out = run_gpu(dev, m, g["haps"], quad, np.zeros((0, N), np.uint32), 1.0,
                      flags=nat.GLP_GEN_NO_WORK)
        ref = float(g["like_ref"][i])
        assert abs(out["evals"][s, 0] - ref) <= REL_TOL * abs(ref), i


def test_golden_hmm_work_from_reference(dev, golden):
    """Sampled haplotype words bit-exact against the reference's hmm_work."""
    g = golden
    N, S = int(g["N"]), int(g["S"])

    class M:
        pass
    m = M()
    m.N, m.S, m.emit, m.t, m.tran, m.pc = N, S, g["emit"], g["t"], g["tran"], g["pc"].reshape(4, 4)
    for k, pen in enumerate(g["pens"]):
        for i in range(len(g["work_sample"])):
            s = int(g["work_sample"][i])
            quad = np.tile(g["work_quad"][i][:, None], (1, N)).astype(np.uint32)
            slot = np.zeros((N, 0), np.uint8)
            u_mh = np.zeros((N, 0), np.float64)
            u_w = np.tile(g["work_u"][i][None, :], (N, 1)).astype(np.float32)
            out = run_gpu(dev, m, g["haps"], quad, np.zeros((0, N), np.uint32), float(pen),
                          trace=(slot, u_mh, u_w))
            assert np.array_equal(out["hnew"][2 * s], g["work_ha"][k, i]), (k, i)
            assert np.array_equal(out["hnew"][2 * s + 1], g["work_hb"][k, i]), (k, i)


def test_index_out_of_range_is_reported(dev):
    m, haps, quad, props = make_problem(N=8, S=100, C=5)
    bad = props.copy()
    bad[2, 3] = haps.shape[0] + 5
    with pytest.raises(nat.GlpError) as e:
        run_gpu(dev, m, haps, quad, bad, 1.0)
    assert e.value.code == nat.GLP_ERR_INDEX
    out = run_gpu(dev, m, haps, quad, props, 1.0)   # context still usable
    assert out["quad"].shape == (4, 8)


def test_argument_errors(dev):
    m, haps, quad, props = make_problem(N=8, S=100, C=5)
    dev.copy_tran_to_device(m.tran)
    a = nat.GenerationArgs()
    a.num_samples, a.num_sites, a.num_cycles, a.num_haps = 8, 101, 5, haps.shape[0]
    h = np.ascontiguousarray(haps)
    q = np.ascontiguousarray(quad)
    p = np.ascontiguousarray(props)
    a.haps, a.hnew, a.hap_idxs_in, a.hap_idxs_out, a.props = _p(h), _p(h.copy()), _p(q), \
        _p(q.copy()), _p(p)
    a.pen = 1.0
    assert dev.L.glp_run_generation_host(dev.ctx, C.byref(a)) == nat.GLP_ERR_STATE
    a.num_sites, a.num_haps = 100, 10
    assert dev.L.glp_run_generation_host(dev.ctx, C.byref(a)) == nat.GLP_ERR_ARG
    a.num_haps, a.pen = haps.shape[0], 0.0
    assert dev.L.glp_run_generation_host(dev.ctx, C.byref(a)) == nat.GLP_ERR_ARG


def test_hmm_work_needs_genotype_probabilities(dev):
    """Emissions set without genotype probabilities (prob NULL, for callers
    that never run hmm_work): a generation with hmm_work is refused with
    GLP_ERR_STATE instead of sampling from stale or unset probabilities, one
    without it (GLP_GEN_NO_WORK) runs, and setting them again restores
    hmm_work."""
    m, haps, quad, props = make_problem(N=8, S=100, C=5)
    run_gpu(dev, m, haps, quad, props, 1.0)          # emissions and probabilities set
    dev.copy_emission_to_device(m.emit, None)        # emissions only
    h = np.ascontiguousarray(haps)
    hn, q = h.copy(), np.ascontiguousarray(quad, dtype=np.uint32)
    qo, p = np.zeros_like(q), np.ascontiguousarray(props, dtype=np.uint32)
    a = nat.GenerationArgs()
    a.num_samples, a.num_sites, a.num_cycles, a.num_haps = m.N, m.S, props.shape[0], h.shape[0]
    a.haps, a.hnew, a.hap_idxs_in, a.hap_idxs_out, a.props = _p(h), _p(hn), _p(q), _p(qo), _p(p)
    a.pen = 1.0
    assert dev.L.glp_run_generation_host(dev.ctx, C.byref(a)) == nat.GLP_ERR_STATE
    assert b"genotype probabilities" in dev.L.glp_last_error(dev.ctx)
    a.flags = nat.GLP_GEN_NO_WORK
    assert dev.L.glp_run_generation_host(dev.ctx, C.byref(a)) == nat.GLP_OK
    out = run_gpu(dev, m, haps, quad, props, 1.0)    # probabilities set again
    assert out["quad"].shape == (4, m.N)


def test_vq_mode_matches_device_reference_semantics(dev, oracle_lib):
    """VQ-decoded emissions (HMMLikeCUDA::hmmLike, hmmLike.cu:53-142)."""
    from glphase_gb300.glpack import GLPack
    O = oracle_lib
    m, haps, quad, props = make_problem(N=24, S=333, C=15, seed=14)
    gp = GLPack(m.t, np.random.default_rng(3))
    packed, cb = gp.packed_gls(), gp.code_book()
    dev.copy_code_book_to_device(cb)
    dev.copy_packed_gls_to_device(packed)
    out = run_gpu(dev, m, haps, quad, props, 1.0, seed=4, flags=nat.GLP_GEN_VQ)
    pb = O.OracleProblem(haps, m.emit, m.t, m.tran, m.pc, 15, packed=packed, codebook=cb,
                         emit_mode=O.EMIT_VQ)
    tr = pb.trace(seed=4, generation=0)
    for s in range(m.N):
        like32, _, own, qf = O.replay_sample(pb, tr, s, quad, props, 1.0, out["acc"][s])
        rel = np.abs(out["evals"][s] - like32) / np.abs(like32)
        assert rel.max() <= REL_TOL, (s, rel.max())
        assert np.array_equal(qf, out["quad"][:, s])
