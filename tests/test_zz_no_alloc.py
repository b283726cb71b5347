"""The allocation-free generation entry point (glp_run_generation_noalloc).

It exists for callers that must not allocate device memory -- code whose
device memory belongs to another allocator (a framework's caching allocator,
an arena reserved at start-up) and code that must not stall other streams
through cudaMalloc/cudaFree.  Its scratch is one fixed device array, so this
test checks that two calls in a row (the second reusing what the first left
in that array) give the same results as the allocating entry point
glp_run_generation on the same inputs, and that oversized problems are
refused.  All test buffers are allocated by the test, not by the call.
"""
import ctypes as C

import numpy as np
import pytest

from glphase_gb300 import native as nat, synth
from glphase_gb300.hmmlike import HMMLikeCUDA

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5  # per-proposal log-likelihood, as in the other parity tests


def _problem(seed):
    w = synth.Workload("noalloc", N=48, S=700, founders=7, depth=3.0, burnin=2, sampling=2,
                       cycles=15, seed=seed)
    m, haps = synth.initial_state(synth.generate(w), seed=seed)
    return m, haps


def _outputs(torch, N, C_, H, wn, dev):
    return dict(hnew=torch.zeros((H, wn), dtype=torch.int64, device=dev),
                quad=torch.zeros((4, N), dtype=torch.int32, device=dev),
                like=torch.zeros(N, dtype=torch.float64, device=dev),
                evals=torch.zeros((N, C_ + 1), dtype=torch.float64, device=dev))


def _args(N, S, C_, H, haps, out, pen, seed, gen):
    a = nat.GenerationArgs()
    a.num_samples, a.num_sites, a.num_cycles, a.num_haps = N, S, C_, H
    a.haps, a.hnew = haps.data_ptr(), out["hnew"].data_ptr()
    a.hap_idxs_out = out["quad"].data_ptr()
    a.like_out, a.eval_trace = out["like"].data_ptr(), out["evals"].data_ptr()
    a.pen, a.seed, a.generation = pen, seed, gen
    return a


def test_noalloc_matches_allocating_entry_point_twice():
    import torch
    dev = torch.device("cuda", 0)
    m, haps_np = _problem(21)
    N, S, C_ = m.N, m.S, 15
    H, wn = haps_np.shape
    emit = torch.from_numpy(np.ascontiguousarray(m.emit)).to(dev)
    prob = torch.from_numpy(np.ascontiguousarray(m.t)).to(dev)
    tran = torch.from_numpy(np.ascontiguousarray(m.tran)).to(dev)
    pc = np.ascontiguousarray(m.pc, dtype=np.float32)
    haps = torch.from_numpy(haps_np.view(np.int64)).to(dev)
    torch.cuda.synchronize()

    ref = HMMLikeCUDA(0)
    ref.copy_tran_to_device(m.tran)
    ref.copy_mutation_mat_to_device(m.pc)
    ref.copy_emission_to_device(m.emit, m.t)
    L = ref.L
    cur = haps
    for call, (pen, gen) in enumerate(((0.4, 3), (1.0, 4))):
        want = _outputs(torch, N, C_, H, wn, dev)
        got = _outputs(torch, N, C_, H, wn, dev)
        torch.cuda.synchronize()
        a = _args(N, S, C_, H, cur, want, pen, 77, gen)
        ref._c(L.glp_run_generation(ref.ctx, C.byref(a)))
        ref._c(L.glp_finish(ref.ctx))
        b = _args(N, S, C_, H, cur, got, pen, 77, gen)
        rc = L.glp_run_generation_noalloc(C.byref(b), tran.data_ptr(), pc.ctypes.data,
                                          emit.data_ptr(), prob.data_ptr(), None)
        assert rc == nat.GLP_OK, call
        torch.cuda.synchronize()
        ew, eg = want["evals"].cpu().numpy(), got["evals"].cpu().numpy()
        assert np.all(np.abs(eg - ew) <= REL_TOL * np.abs(ew)), call
        assert torch.equal(got["quad"], want["quad"]), call
        assert torch.equal(got["hnew"][:2 * N], want["hnew"][:2 * N]), call
        lw, lg = want["like"].cpu().numpy(), got["like"].cpu().numpy()
        assert np.all(np.abs(lg - lw) <= REL_TOL * np.abs(lw)), call
        nxt = got["hnew"].clone()
        nxt[2 * N:] = cur[2 * N:]
        cur = nxt
    ref.cleanup()


def test_noalloc_refuses_oversized_problems():
    L = nat.load()
    a = nat.GenerationArgs()
    a.num_samples, a.num_sites, a.num_cycles, a.num_haps = 4000, 4096, 10, 8000
    a.haps = a.hnew = a.hap_idxs_out = 16   # never dereferenced: refused first
    a.pen = 1.0
    dummy = np.zeros(16, np.float32)
    rc = L.glp_run_generation_noalloc(C.byref(a), 16, dummy.ctypes.data, 16, 16, None)
    assert rc == nat.GLP_ERR_TOO_LARGE
