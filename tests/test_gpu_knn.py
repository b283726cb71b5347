"""Device kNN surrogate restriction and device-side surrogate draws against
the oracle (exact integer results), plus the reference's kNN known answers
(src/testing/other_unittests.cpp:103-254)."""
import ctypes as C

import numpy as np
import pytest

import knn_cases as kc
from glphase_gb300 import model as mdl, native as nat, synth
from glphase_gb300.hmmlike import HMMLikeCUDA

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev():
    d = HMMLikeCUDA(0)
    yield d
    d.cleanup()


def gpu_knn(dev, haps, S, K, lb=0.0, ub=1.0, use_maf=False, metric="hamming"):
    import torch
    H, wn = haps.shape
    half = (K + 1) // 2
    h = torch.from_numpy(np.ascontiguousarray(haps).view(np.int64)).cuda()
    out = torch.zeros((H // 2, 2 * half), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    dev._c(dev.L.glp_set_knn_metric(dev.ctx, nat.KNN_METRICS[metric]))
    dev._c(dev.L.glp_knn_neighbors(dev.ctx, h.data_ptr(), H, S, K, lb, ub, int(use_maf),
                                   out.data_ptr()))
    dev._c(dev.L.glp_finish(dev.ctx))
    return out.cpu().numpy().view(np.uint32)


def test_knn_reference_known_answers(dev):
    for case in (kc.case_nearest, kc.case_threshold):
        bits, perm, lb, ub, want = case()
        nb = gpu_knn(dev, mdl.pack_haplotypes(bits), kc.NUM_SITES, kc.NUM_CLUSTERS, lb, ub)
        assert [int(perm[i]) for i in nb[0]] == want


@pytest.mark.parametrize("H,S,K", [(40, 130, 7), (200, 1000, 20), (1000, 700, 200),
                                   (4000, 4096, 200)])
def test_knn_matches_oracle(dev, oracle_lib, H, S, K):
    rng = np.random.default_rng(H + S)
    # related haplotypes so that distances have many ties and structure
    founders = rng.integers(0, 2, size=(8, S)).astype(np.uint8)
    bits = founders[rng.integers(0, 8, size=H)]
    flip = rng.random((H, S)) < 0.05
    bits = (bits ^ flip).astype(np.uint8)
    haps = mdl.pack_haplotypes(bits)
    want = oracle_lib.knn(haps, S, K)
    got = gpu_knn(dev, haps, S, K)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("H,S,K", [(40, 130, 7), (200, 1000, 20), (1000, 700, 200),
                                   (4000, 4096, 200)])
def test_knn_tract_metric_matches_oracle(dev, oracle_lib, H, S, K):
    """insti -T: the common sites minus the longest shared tract
    (Haplotype::MaxTractLen, haplotype.cpp:62-90; kNN.cpp:157-164)."""
    rng = np.random.default_rng(H + 2 * S)
    founders = rng.integers(0, 2, size=(8, S)).astype(np.uint8)
    bits = founders[rng.integers(0, 8, size=H)]
    flip = rng.random((H, S)) < 0.02
    bits = (bits ^ flip).astype(np.uint8)
    haps = mdl.pack_haplotypes(bits)
    want = oracle_lib.knn(haps, S, K, metric="tract")
    got = gpu_knn(dev, haps, S, K, metric="tract")
    assert np.array_equal(got, want)
    assert not np.array_equal(want, oracle_lib.knn(haps, S, K))  # the metrics differ here


def test_knn_tract_metric_with_frequency_bounds(dev, oracle_lib):
    rng = np.random.default_rng(6)
    bits = (rng.random((300, 500)) < rng.beta(0.5, 0.5, 500)[None, :]).astype(np.uint8)
    haps = mdl.pack_haplotypes(bits)
    for lb, ub, maf in ((0.05, 0.95, False), (0.1, 0.5, True)):
        assert np.array_equal(gpu_knn(dev, haps, 500, 30, lb, ub, maf, metric="tract"),
                              oracle_lib.knn(haps, 500, 30, lb, ub, maf, metric="tract"))


def test_knn_metric_argument(dev):
    assert dev.L.glp_set_knn_metric(dev.ctx, 2) == nat.GLP_ERR_ARG
    assert dev.L.glp_set_knn_metric(dev.ctx, nat.GLP_KNN_HAMMING) == nat.GLP_OK


def test_knn_with_frequency_bounds(dev, oracle_lib):
    rng = np.random.default_rng(5)
    bits = (rng.random((300, 500)) < rng.beta(0.5, 0.5, 500)[None, :]).astype(np.uint8)
    haps = mdl.pack_haplotypes(bits)
    for lb, ub, maf in ((0.05, 0.95, False), (0.1, 0.5, True)):
        assert np.array_equal(gpu_knn(dev, haps, 500, 30, lb, ub, maf),
                              oracle_lib.knn(haps, 500, 30, lb, ub, maf))


def test_device_surrogates_match_oracle(dev, oracle_lib):
    """Generation with the initial quadruples and proposals drawn in the kernel
    (uniform, panel-only and kNN table) equals the oracle run on the same
    draws materialised on the host."""
    from test_gpu_parity import check_against_oracle, make_problem
    O = oracle_lib
    m, haps, _, _ = make_problem(N=24, S=400, C=20, panel=40, seed=6)
    H = haps.shape[0]
    nbr = O.knn(haps, m.S, 10)[:m.N]
    for lo, hi, table, kick in ((0, 0, None, False), (48, H, None, False), (0, 0, nbr, False),
                                (0, 0, None, True), (0, 0, nbr, True)):
        seed, gen = 31, 5
        dev.copy_tran_to_device(m.tran)
        dev.copy_mutation_mat_to_device(m.pc)
        dev.copy_emission_to_device(m.emit, m.t)
        a = nat.GenerationArgs()
        a.num_samples, a.num_sites, a.num_cycles, a.num_haps = m.N, m.S, 20, H
        h = np.ascontiguousarray(haps)
        hnew = h.copy()
        qo = np.zeros((4, m.N), np.uint32)
        evals = np.zeros((m.N, 21), np.float64)
        acc = np.zeros((m.N, 20), np.uint8)
        like = np.zeros(m.N, np.float64)
        a.haps, a.hnew, a.hap_idxs_out = h.ctypes.data, hnew.ctypes.data, qo.ctypes.data
        a.pen, a.seed, a.generation = 0.7, seed, gen
        a.like_out, a.eval_trace, a.accept_trace = like.ctypes.data, evals.ctypes.data, \
            acc.ctypes.data
        a.sample_lo, a.sample_hi = lo, hi
        a.flags = nat.GLP_GEN_KICK_FIRST if kick else 0
        if table is not None:
            tb = np.ascontiguousarray(table)
            a.neighbors, a.neighbors_per_sample = tb.ctypes.data, tb.shape[1]
        rc = dev.L.glp_run_generation_host(dev.ctx, C.byref(a))
        assert rc == 0, dev.L.glp_last_error(dev.ctx)
        quad, props = O.sample_surrogates(seed, gen, m.N, 20, lo, hi if hi else H,
                                          nbr=table, kick_first=kick, H=H)
        if kick:
            assert props[0].min() >= 2 * m.N
        out = dict(quad=qo, hnew=hnew, like=like, evals=evals, acc=acc)
        check_against_oracle(O, m, haps, quad, props, 0.7, out, seed, gen)
