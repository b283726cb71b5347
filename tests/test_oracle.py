"""The CPU oracle pinned against the reference: golden vectors produced by the
reference's own impute.cpp (tests/golden/make_golden.py), a live comparison
with oracle/_ref where that build exists, and the known-answer tests of the
reference's unit tests (src/testing/*.cpp)."""
import ctypes as C
import math

import numpy as np
import pytest

from glphase_gb300 import model as mdl, synth


def _row(a):
    return np.ascontiguousarray(a)


def test_philox_known_answers():
    """Philox4x32-10 against the published Random123 known-answer vectors."""
    import subprocess, tempfile, os
    from conftest import ROOT
    src = r'''
#include <stdio.h>
#include "glp_rng.h"
int main(){
  glp_u32x4 c={{0,0,0,0}}; glp_u32x4 o=glp_philox4x32_10(c,0,0);
  printf("%08x%08x%08x%08x\n",o.v[0],o.v[1],o.v[2],o.v[3]);
  glp_u32x4 d={{0xffffffffu,0xffffffffu,0xffffffffu,0xffffffffu}};
  o=glp_philox4x32_10(d,0xffffffffu,0xffffffffu);
  printf("%08x%08x%08x%08x\n",o.v[0],o.v[1],o.v[2],o.v[3]);
  glp_u32x4 e={{0x243f6a88u,0x85a308d3u,0x13198a2eu,0x03707344u}};
  o=glp_philox4x32_10(e,0xa4093822u,0x299f31d0u);
  printf("%08x%08x%08x%08x\n",o.v[0],o.v[1],o.v[2],o.v[3]);
  return 0;}
'''
    with tempfile.TemporaryDirectory() as d:
        cfile, exe = os.path.join(d, "k.c"), os.path.join(d, "k")
        open(cfile, "w").write(src)
        subprocess.run(["gcc", "-O2", "-I", os.path.join(ROOT, "glphase_gb300", "csrc"), cfile,
                        "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    assert out == ["6627e8d5e169c58dbc57ac4c9b00dbd8", "408f276d41c83b0ea20bc7c66d5451fd",
                   "d16cfe0994fdcceb5001e42024126ea1"]


def test_hmm_like_matches_reference_golden(oracle_lib, golden):
    O, g = oracle_lib, golden
    for i in range(len(g["like_ref"])):
        s = int(g["like_sample"][i])
        v = O.hmm_like_f32(_row(g["emit"][s]), g["tran"], g["haps"], _row(g["like_quad"][i]))
        assert np.float32(v) == g["like_ref"][i], i


def test_hmm_like_f64_yardstick(oracle_lib, golden):
    O, g = oracle_lib, golden
    for i in range(16):
        s = int(g["like_sample"][i])
        v32 = O.hmm_like_f32(_row(g["emit"][s]), g["tran"], g["haps"], _row(g["like_quad"][i]))
        v64 = O.hmm_like_f64(_row(g["emit"][s]), g["tran"], g["haps"], _row(g["like_quad"][i]))
        assert abs(v32 - v64) <= 1e-5 * abs(v64)
        assert v64 <= 0


def test_hmm_work_matches_reference_golden(oracle_lib, golden):
    O, g = oracle_lib, golden
    for k, pen in enumerate(g["pens"]):
        for i in range(len(g["work_sample"])):
            s = int(g["work_sample"][i])
            ha, hb = O.hmm_work(_row(g["emit"][s]), _row(g["t"][s]), g["tran"], g["pc"],
                                g["haps"], _row(g["work_quad"][i]), float(pen),
                                _row(g["work_u"][i]))
            assert np.array_equal(ha, g["work_ha"][k, i]), (k, i)
            assert np.array_equal(hb, g["work_hb"][k, i]), (k, i)


def test_model_constants_match_reference_initialize(golden):
    """mu, pc, tran, t and emit against Impute::initialize (impute.cpp:182-322)."""
    g = golden
    gl = g["init_gl"]                    # [S][N][2] (het, homAlt), site-major
    Si, Ni = gl.shape[0], gl.shape[1]
    m = mdl.Model(np.ascontiguousarray(gl.transpose(1, 0, 2)), positions=g["init_pos"])
    assert np.array_equal(m.pc.reshape(16), g["init_pc"])
    assert np.array_equal(m.t.reshape(-1), g["init_t"])
    assert np.array_equal(m.emit.reshape(-1), g["init_emit"])
    # Impute keeps the per-interval distance in binary64 where Insti keeps it
    # in binary32 (impute.cpp:275-277 vs insti.cpp:1282-1283)
    np.testing.assert_allclose(m.tran.reshape(-1)[3:], g["init_tran"][3:], rtol=1e-6)


def test_replace_matches_reference_golden(oracle_lib, golden):
    O, g = oracle_lib, golden
    hs = g["replace_haps"]
    hsum = np.zeros(2 * 3 * 100, np.uint32)
    for gen in range(hs.shape[0]):
        for s in range(3):
            O.lib().glpo_replace(np.ascontiguousarray(hs[gen].reshape(-1)), 2, 100, s, hsum)
    assert np.array_equal(hsum, g["replace_hsum"])


@pytest.mark.skipif("not __import__('oracle').ref_available()")
def test_result_matches_live_reference_build(oracle_lib):
    """Impute::result of the reference build (impute.cpp:599-613) against the
    oracle's: allele probabilities [S][2N] identical in binary32, for tallies
    up to 2^26 (where the unsigned-to-float conversion rounds) and sampling
    counts that make 1/sn inexact."""
    O = oracle_lib
    L, R = O.lib(), O.ref()
    rng = np.random.default_rng(43)
    for N, S, sn in ((1, 1, 1), (3, 70, 3), (17, 129, 7), (40, 300, 24), (5, 64, 1000)):
        top = int(rng.choice([sn + 1, 2**20, 2**26]))
        hsum = rng.integers(0, top, 2 * N * S).astype(np.uint32)
        want = np.zeros(2 * N * S, np.float32)
        got = np.zeros(2 * N * S, np.float32)
        R.glpr_result(hsum, N, S, sn, want)
        L.glpo_result(hsum, N, S, sn, got)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (N, S, sn)


@pytest.mark.skipif("not __import__('oracle').ref_available()")
def test_oracle_matches_live_reference_build(oracle_lib):
    """Random inputs straight through the reference's compiled impute.cpp."""
    O = oracle_lib
    R = O.ref()
    rng = np.random.default_rng(17)
    for S in (1, 2, 63, 64, 65, 300):
        H, wn = 12, (S + 63) // 64
        haps = rng.integers(0, 2**63, size=(H, wn), dtype=np.uint64)
        emit = rng.random((S, 4)).astype(np.float32)
        prob = rng.dirichlet([1, 1, 1], S).astype(np.float32)
        tran = np.zeros((S, 3), np.float32)
        r = rng.random(S).astype(np.float32) * 0.01
        tran[:, 0], tran[:, 1], tran[:, 2] = (1 - r) ** 2, r * (1 - r), r * r
        pc = rng.random(16).astype(np.float32)
        for _ in range(8):
            P = rng.integers(0, H, 4).astype(np.uint32)
            a = O.hmm_like_f32(emit, tran, haps, P)
            b = R.glpr_hmm_like(emit, tran, haps, H, wn, S, P)
            assert np.float32(a) == np.float32(b)
            u = rng.random(S).astype(np.float32)
            for pen in (1.0, 0.5):
                ha, hb = O.hmm_work(emit, prob, tran, pc, haps, P, pen, u)
                ra = np.zeros(wn, np.uint64)
                rb = np.zeros(wn, np.uint64)
                R.glpr_hmm_work(emit, prob, tran, pc, haps, H, wn, S, P, pen, u, ra, rb)
                assert np.array_equal(ha, ra) and np.array_equal(hb, rb)


# --- known-answer tests of the reference's unit tests ------------------------

def test_codebook_decode_kat(oracle_lib):
    """src/testing/cuda_tests.cpp:66-96: codebook (i/10, 2i/100); word 1 slot 7
    decodes code 1; word 0x01234567 slot i decodes code i."""
    L = oracle_lib.lib()
    cb = np.array([[i / 10, i * 2 / 100] for i in range(16)], np.float32).reshape(-1)
    gl = np.zeros(3, np.float32)
    L.glpo_unpack_gl_codebook(1, cb, 7, gl)
    np.testing.assert_array_almost_equal(gl, [0.1, 0.02, 0.88], decimal=6)
    for i in range(8):
        L.glpo_unpack_gl_codebook(19088743, cb, i, gl)
        np.testing.assert_allclose(gl, [i / 10, i * 2 / 100, 1 - i / 10 - i * 2 / 100],
                                   rtol=1e-6, atol=1e-7)


def test_fill_emit_kat(oracle_lib):
    """src/testing/cuda_tests.cpp:98-116: all-ones mutation matrix gives
    G0 + 2 G1 + G2 for every state."""
    L = oracle_lib.lib()
    rng = np.random.default_rng(1)
    M = np.ones(16, np.float32)
    for _ in range(10):
        gl = rng.random(3).astype(np.float32)
        em = np.zeros(4, np.float32)
        L.glpo_fill_emit(gl, M, em)
        np.testing.assert_allclose(em, gl[0] + 2 * gl[1] + gl[2], rtol=1e-6)


def test_mutation_matrix_transpose_kat(oracle_lib):
    """src/testing/cuda_tests.cpp:46-63: pc[i][j] = i + 4j lands at M[i + 4j]."""
    L = oracle_lib.lib()
    pc = np.array([[i + 4 * j for j in range(4)] for i in range(4)], np.float32).reshape(-1)
    M = np.zeros(16, np.float32)
    L.glpo_mutation_to_device_layout(pc, M)
    for i in range(4):
        for j in range(4):
            assert M[i + 4 * j] == i + 4 * j


def test_mh_accept_semantics(oracle_lib):
    """src/testing/other_unittests.cpp:256-283 restated on the accept rule:
    better or equal proposals are always accepted, much worse ones are not."""
    L = oracle_lib.lib()
    curr = -100.0
    for i in range(2, 10):
        assert L.glpo_mh_accept(curr + i * 0.01, curr, 1.0, 0.999999) == 1
    assert L.glpo_mh_accept(curr, curr, 1.0, 0.999999) == 1
    assert L.glpo_mh_accept(2 * curr, curr, 1.0, 1e-12) == 0
    # u < exp(delta * pen) boundary, binary64
    d = -0.5
    assert L.glpo_mh_accept(curr + d, curr, 1.0, math.exp(d) * (1 - 1e-12)) == 1
    assert L.glpo_mh_accept(curr + d, curr, 1.0, math.exp(d) * (1 + 1e-12)) == 0
    assert L.glpo_mh_accept(curr + d, curr, 0.25, math.exp(d * 0.25) * 0.999) == 1


@pytest.mark.skipif("not __import__('oracle').ref_available()")
def test_mh_chain_matches_live_reference_build(oracle_lib):
    """MHSampler<unsigned>::SampleHap of the reference (plain MH,
    MHSampler.hpp:81-96, compiled into oracle/_ref) against the oracle's
    accept rule over whole chains: the same decisions, the same reverted
    states, and a uniform consumed exactly when a proposal scores below the
    current likelihood.  Chains mix ties, near ties and large drops, at the
    annealing penalties 1, 0.25 and 0.04."""
    O = oracle_lib
    L, R = O.lib(), O.ref()
    rng = np.random.default_rng(41)
    for t in range(300):
        n = int(rng.integers(1, 120))
        pen = float(rng.choice([1.0, 0.25, 0.04]))
        # proposals around the start's likelihood: equal, a hair above or
        # below, moderately and far below; every other chain with noise added
        steps = rng.choice([0.0, 1e-9, -1e-9, 0.3, -0.3, -5.0, -60.0], size=n)
        like = -1e4 + np.concatenate([[0.0], steps])
        like = np.minimum(like + rng.normal(0, 0.2, n + 1) * (t % 2), 0.0)
        u = rng.random(n + 1)
        acc = np.zeros(n, np.uint8)
        state = np.zeros(n, np.uint32)
        R.glpr_mh_chain(np.ascontiguousarray(like), n, pen, u, u.size, acc, state)
        curr, obj, k = like[0], 0, 0
        for c in range(1, n + 1):
            if like[c] >= curr:
                a = 1
            else:
                a = L.glpo_mh_accept(like[c], curr, pen, u[k])
                k += 1
            if a:
                curr, obj = like[c], c
            assert acc[c - 1] == a and state[c - 1] == obj, (t, c)


def test_hap_packing_round_trip():
    rng = np.random.default_rng(3)
    for S in (1, 63, 64, 65, 200):
        bits = rng.integers(0, 2, size=(5, S)).astype(np.uint8)
        words = mdl.pack_haplotypes(bits)
        assert words.shape == (5, (S + 63) // 64)
        assert np.array_equal(mdl.unpack_haplotypes(words, S), bits)
        # site m -> word m >> 6, bit m & 63 (impute.hpp:53-66)
        for m in range(S):
            assert ((int(words[2, m >> 6]) >> (m & 63)) & 1) == bits[2, m]


def test_generation_reproducible_and_consistent(oracle_lib):
    """A generation from the Philox streams equals per-sample solves."""
    O = oracle_lib
    w = synth.Workload("t", N=12, S=130, founders=5, depth=3, burnin=1, sampling=1, cycles=9,
                       seed=4)
    ds = synth.generate(w)
    m, haps = synth.initial_state(ds)
    rng = np.random.default_rng(0)
    quad, props = synth.uniform_proposals(m.N, haps.shape[0], w.cycles, rng)
    pb = O.OracleProblem(haps, m.emit, m.t, m.tran, m.pc, w.cycles)
    tr = pb.trace(seed=5, generation=2)
    q1, h1, l1 = O.generation(pb, tr, quad, props, 0.5, like=True, nthreads=2)
    q2, h2, l2 = O.generation(pb, tr, quad, props, 0.5, like=True, nthreads=1)
    assert np.array_equal(q1, q2) and np.array_equal(h1, h2) and np.array_equal(l1, l2)
    for s in range(m.N):
        q, curr, likes, acc, ha, hb = O.solve_sample(pb, tr, s, quad, props, 0.5, do_work=True)
        assert np.array_equal(q, q1[:, s])
        assert np.array_equal(ha, h1[2 * s]) and np.array_equal(hb, h1[2 * s + 1])
        assert curr == l1[s]


def test_knn_reference_kat(oracle_lib):
    """KNN::ClusterHaps against src/testing/other_unittests.cpp:103-254."""
    import knn_cases as kc
    O = oracle_lib
    for case in (kc.case_nearest, kc.case_threshold):
        bits, perm, lb, ub, want = case()
        haps = mdl.pack_haplotypes(bits)
        nb = O.knn(haps, kc.NUM_SITES, kc.NUM_CLUSTERS, lb, ub)
        assert [int(perm[i]) for i in nb[0]] == want
    bits, perm, lb, ub, _ = kc.case_threshold()
    mask = O.common_sites(mdl.pack_haplotypes(bits), kc.NUM_SITES, lb, ub)
    _, ncommon = kc.expected_af_threshold()
    assert bin(int(mask[0])).count("1") == ncommon
    af = bits.mean(axis=0)
    assert list(af[:3]) == kc.expected_af_threshold()[0]


def test_knn_lists_are_valid(oracle_lib):
    O = oracle_lib
    rng = np.random.default_rng(8)
    haps = rng.integers(0, 2**63, size=(60, 3), dtype=np.uint64)
    nb = O.knn(haps, 150, 20)
    assert nb.shape == (30, 20)
    for s in range(30):
        assert len(set(nb[s].tolist())) == 20           # unique
        assert all(h // 2 != s for h in nb[s])           # never the sample's own


def test_device_surrogate_streams(oracle_lib):
    """Uniform draws avoid the sample's own pair and cover [lo, hi)."""
    O = oracle_lib
    q, p = O.sample_surrogates(9, 3, 50, 400, 0, 100)
    for s in range(50):
        allh = np.r_[q[:, s], p[:, s]]
        assert not np.any(allh // 2 == s)
        assert allh.max() < 100
    q, p = O.sample_surrogates(9, 3, 50, 400, 100, 130)   # panel-only range
    assert p.min() >= 100 and p.max() < 130
    nbr = np.tile(np.arange(7, dtype=np.uint32)[None, :] + 60, (50, 1))
    q, p = O.sample_surrogates(9, 3, 50, 100, 0, 0, nbr=nbr)
    assert p.min() >= 60 and p.max() < 67
    assert len(np.unique(p)) == 7


def test_kick_start_first_proposal(oracle_lib):
    """--kickstart (insti.cpp:1505-1511): every chain's first proposal is a
    panel haplotype (index >= 2N), the other draws are unchanged."""
    O = oracle_lib
    N, H = 50, 160                      # panel rows 100..159
    q0, p0 = O.sample_surrogates(9, 3, N, 40, 0, H)
    q1, p1 = O.sample_surrogates(9, 3, N, 40, 0, H, kick_first=True)
    assert np.array_equal(q0, q1) and np.array_equal(p0[1:], p1[1:])
    assert p1[0].min() >= 2 * N and p1[0].max() < H
    # with a neighbour list: its panel entries only, in any of them
    nbr = np.tile(np.array([3, 120, 7, 140, 9], np.uint32)[None, :], (N, 1))
    q1, p1 = O.sample_surrogates(9, 3, N, 40, 0, 0, nbr=nbr, kick_first=True, H=H)
    assert set(p1[0].tolist()) == {120, 140}
    assert set(np.unique(p1[1:]).tolist()) <= {3, 120, 7, 140, 9}
    # a list without panel entries falls back to a uniform panel draw
    nbr = np.tile(np.array([3, 7, 9], np.uint32)[None, :], (N, 1))
    _, p1 = O.sample_surrogates(9, 3, N, 40, 0, 0, nbr=nbr, kick_first=True, H=H)
    assert p1[0].min() >= 2 * N and p1[0].max() < H


def test_fp16_gl_storage_exceeds_the_loglik_bound(oracle_lib):
    """Why GLs and emissions stay binary32: rounding either to FP16 before
    the recursion moves the log-likelihood by more than the 1e-5 relative
    bound (measured against the binary64 yardstick on synthetic data at
    depth 2: emission in FP16 up to ~7e-5, GLs in FP16 up to ~4e-5)."""
    O = oracle_lib
    w = synth.Workload("fp16", N=64, S=1024, founders=20, depth=2.0, burnin=1, sampling=1,
                       seed=3)
    ds = synth.generate(w)
    m, haps = synth.initial_state(ds, seed=2)
    e16 = m.emit.astype(np.float16).astype(np.float32)
    e_gl16 = mdl.emission(m.t.astype(np.float16).astype(np.float32), m.pc)
    rng = np.random.default_rng(5)
    worst_e = worst_gl = 0.0
    for _ in range(100):
        s = int(rng.integers(0, m.N))
        q = rng.integers(0, haps.shape[0], 4).astype(np.uint32)
        ref = O.hmm_like_f64(np.ascontiguousarray(m.emit[s]), m.tran, haps, q)
        for emit, name in ((e16, "e"), (e_gl16, "gl")):
            rel = abs(O.hmm_like_f64(np.ascontiguousarray(emit[s]), m.tran, haps, q) - ref)
            rel /= abs(ref)
            if name == "e":
                worst_e = max(worst_e, rel)
            else:
                worst_gl = max(worst_gl, rel)
    assert worst_e > 1e-5 and worst_gl > 1e-5, (worst_e, worst_gl)


def _hap(n, sites=()):
    from glphase_gb300 import model as mdl
    b = np.zeros((1, n), np.uint8)
    for i in sites:
        b[0, i] = 1
    return mdl.pack_haplotypes(b)[0]


def _all_sites(n):
    m = np.zeros((n + 63) // 64, np.uint64)
    for i in range(n):
        m[i >> 6] |= np.uint64(1) << np.uint64(i & 63)
    return m


def test_max_tract_reference_kat(oracle_lib):
    """Haplotype::MaxTractLen's known answers (src/testing/other_unittests.cpp:79-101)."""
    O = oracle_lib
    a, b = _hap(4), _hap(4, (0, 3))
    assert O.max_tract(a, a, _all_sites(4)) == 4
    assert O.max_tract(a, b, _all_sites(4)) == 2
    c, d = _hap(1024), _hap(1024, (23,))
    m = _all_sites(1024)
    assert O.max_tract(c, c, m) == 1024
    assert O.max_tract(c, d, m) == 1000
    assert O.max_tract(d, c, m) == 1000
    d2 = _hap(1024, (23, 1023))
    assert O.max_tract(d2, c, m) == 999


def test_max_tract_skips_sites_outside_the_mask(oracle_lib):
    """Over the common sites only (KNN::CutDownHaps, kNN.cpp:216-257): a
    disagreement at a dropped site neither breaks nor ends a run, and
    dropped sites are not counted."""
    O = oracle_lib
    rng = np.random.default_rng(9)
    for _ in range(50):
        n = int(rng.integers(1, 300))
        a = rng.integers(0, 2, n).astype(np.uint8)
        b = np.where(rng.random(n) < 0.1, 1 - a, a).astype(np.uint8)
        keep = rng.random(n) < 0.7
        from glphase_gb300 import model as mdl
        pa, pb = mdl.pack_haplotypes(a[None])[0], mdl.pack_haplotypes(b[None])[0]
        mask = np.zeros_like(pa)
        for i in np.nonzero(keep)[0]:
            mask[i >> 6] |= np.uint64(1) << np.uint64(i & 63)
        best = run = 0
        for i in np.nonzero(keep)[0]:
            run = 0 if a[i] != b[i] else run + 1
            best = max(best, run)
        assert O.max_tract(pa, pb, mask) == best


def test_knn_tract_metric_lists(oracle_lib):
    """The tract-length metric (insti -T, kNN.cpp:157-164) orders
    neighbours by the longest shared tract, not by the mismatch count:
    a haplotype with one disagreement in its middle is farther than one with
    three near an end."""
    O = oracle_lib
    from glphase_gb300 import model as mdl
    S = 100
    bits = np.zeros((6, S), np.uint8)
    bits[2, 50] = 1            # haplotype 2: one disagreement with haplotype 0, mid-way
    bits[3, [0, 1, 2]] = 1     # haplotype 3: three disagreements at the start
    bits[4, :] = 1             # far from everything
    bits[5, :] = 1
    haps = mdl.pack_haplotypes(bits)
    ham = O.knn(haps, S, 2)
    tract = O.knn(haps, S, 2, metric="tract")
    assert ham[0][0] == 2      # Hamming: 1 < 3
    assert tract[0][0] == 3    # tract: 97 shared sites > 50


# --- the kNN restatement against the reference's own kNN.cpp -----------------

def _knn_cases(rng, n, H_choices, S_max):
    """Random panels with site frequencies spread over (0, 1), and the
    frequency-bound variants of KNN's constructor (plain, an allele-frequency
    window, a minor-allele-frequency cap)."""
    for t in range(n):
        H = int(rng.choice(H_choices))
        S = int(rng.integers(1, S_max))
        K = int(rng.integers(1, H - 1))
        if 2 * ((K + 1) // 2) > H - 2:
            K = H - 2
        bits = (rng.random((H, S)) < rng.random(S)).astype(np.uint8)
        lb, ub, maf = 0.0, 1.0, False
        if t % 3 == 1:
            lb, ub = (float(x) for x in sorted(rng.random(2)))
        elif t % 3 == 2:
            ub, maf = float(rng.random() * 0.5), True
        yield mdl.pack_haplotypes(bits), S, K, lb, ub, maf


@pytest.mark.skipif("not __import__('oracle').ref_knn_available()")
def test_knn_metrics_match_live_reference_build(oracle_lib):
    """Haplotype::MaxTractLen and HammingDist of the reference's compiled
    haplotype.cpp against the oracle's word-wise restatements on random
    pairs (lengths 1 .. 300, sparse and dense disagreements)."""
    O = oracle_lib
    R = O.ref_knn()
    rng = np.random.default_rng(21)
    for _ in range(600):
        n = int(rng.integers(1, 300))
        a = rng.integers(0, 2, n).astype(np.uint8)
        flip = rng.random(n) < rng.choice([0.005, 0.05, 0.3])
        b = np.where(flip, 1 - a, a).astype(np.uint8)
        pa, pb = mdl.pack_haplotypes(a[None])[0], mdl.pack_haplotypes(b[None])[0]
        every = np.zeros_like(pa)
        for i in range(n):
            every[i >> 6] |= np.uint64(1) << np.uint64(i & 63)
        assert O.max_tract(pa, pb, every) == R.glpr_max_tract(a, b, n)
        assert R.glpr_hamming(a, b, n) == int(flip.sum())


@pytest.mark.skipif("not __import__('oracle').ref_knn_available()")
def test_knn_lists_match_live_reference_build(oracle_lib):
    """KNN::ClusterHaps of the reference's compiled kNN.cpp against the
    oracle's lists, both metrics, with and without frequency bounds.

    The reference orders each haplotype's distances with std::sort on the
    distance alone, whose tie order is unspecified; the oracle breaks ties by
    haplotype index.  With at most 16 candidates (H <= 18) libstdc++'s sort
    is a plain insertion sort, which keeps equal distances in index order, so
    there the lists must be identical.  On larger panels the check is
    tie-blind: list A's distances in order, and, where both picked the same
    set for A, list B's distances in order."""
    O = oracle_lib
    rng = np.random.default_rng(23)
    for haps, S, K, lb, ub, maf in _knn_cases(rng, 120, [4, 6, 8, 10, 12, 14, 16, 18], 400):
        for metric in ("hamming", "tract"):
            want = O.ref_knn_lists(haps, S, K, lb, ub, maf, metric)
            got = O.knn(haps, S, K, lb, ub, maf, metric=metric)
            assert np.array_equal(got, want), (haps.shape, S, K, lb, ub, maf, metric)

    def dist(h, o, mask, metric):
        if metric == "hamming":
            return sum(bin(int(x)).count("1") for x in (h ^ o) & mask)
        return sum(bin(int(x)).count("1") for x in mask) - O.max_tract(h, o, mask)

    checked_b = 0
    for haps, S, K, lb, ub, maf in _knn_cases(rng, 4, [300], 700):
        mask = O.common_sites(haps, S, lb, ub, maf)
        for metric in ("hamming", "tract"):
            want = O.ref_knn_lists(haps, S, K, lb, ub, maf, metric)
            got = O.knn(haps, S, K, lb, ub, maf, metric=metric)
            for s in range(0, haps.shape[0] // 2, 7):
                dA = [[dist(haps[2 * s], haps[h], mask, metric) for h in lst[0::2]]
                      for lst in (want[s], got[s])]
                assert dA[0] == dA[1]
                if set(want[s][0::2]) == set(got[s][0::2]):
                    dB = [[dist(haps[2 * s + 1], haps[h], mask, metric) for h in lst[1::2]]
                          for lst in (want[s], got[s])]
                    assert dB[0] == dB[1]
                    checked_b += 1
    assert checked_b > 0
