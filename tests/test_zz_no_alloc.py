"""The allocation-free generation entry point (glp_run_generation_noalloc).

It exists for callers that must not allocate device memory -- code whose
device memory belongs to another allocator (a framework's caching allocator,
an arena reserved at start-up) and code that must not stall other streams
through cudaMalloc/cudaFree.  Its scratch is one fixed device array, so these
tests check that

  * two calls in a row (the second reusing what the first left in that
    array) give bit for bit the results of the allocating entry point
    glp_run_generation on the same inputs: the same kernels run, and every
    evaluation is independent of the speculation width;
  * the same holds without hmm_work (GLP_GEN_NO_WORK) and with surrogates
    from a neighbour table and a kick-started first proposal;
  * a call after the first in a context leaves the device's free memory
    unchanged, i.e. it allocates nothing;
  * problems beyond the array, and a kick-started first proposal without
    panel rows, are refused before anything runs.

All test buffers are allocated by the test, not by the call.  The file is
collected last so that a run stopping at the first failure has run every
other test before it.
"""
import ctypes as C

import numpy as np
import pytest

from glphase_gb300 import native as nat, synth
from glphase_gb300.hmmlike import HMMLikeCUDA

pytestmark = pytest.mark.gpu


def _problem(seed, panel=0):
    w = synth.Workload("noalloc", N=48, S=700, founders=7, depth=3.0, burnin=2, sampling=2,
                       cycles=15, panel_haps=panel, seed=seed)
    m, haps = synth.initial_state(synth.generate(w), seed=seed)
    return m, haps


class Inputs:
    """Device copies of one problem's model inputs (torch as plumbing)."""

    def __init__(self, torch, m, haps_np, C_):
        dev = torch.device("cuda", 0)
        self.m, self.N, self.S, self.C = m, m.N, m.S, C_
        self.H, self.wn = haps_np.shape
        self.emit = torch.from_numpy(np.ascontiguousarray(m.emit)).to(dev)
        self.prob = torch.from_numpy(np.ascontiguousarray(m.t)).to(dev)
        self.tran = torch.from_numpy(np.ascontiguousarray(m.tran)).to(dev)
        self.pc = np.ascontiguousarray(m.pc, dtype=np.float32)
        self.haps = torch.from_numpy(haps_np.view(np.int64)).to(dev)
        self.dev = dev

    def outputs(self, torch):
        N, C_, dev = self.N, self.C, self.dev
        return dict(hnew=torch.zeros((self.H, self.wn), dtype=torch.int64, device=dev),
                    quad=torch.zeros((4, N), dtype=torch.int32, device=dev),
                    like=torch.zeros(N, dtype=torch.float64, device=dev),
                    evals=torch.zeros((N, C_ + 1), dtype=torch.float64, device=dev),
                    acc=torch.zeros((N, C_), dtype=torch.uint8, device=dev))

    def args(self, haps, out, pen, seed, gen, flags=0, nbr=None):
        a = nat.GenerationArgs()
        a.num_samples, a.num_sites, a.num_cycles, a.num_haps = self.N, self.S, self.C, self.H
        a.haps, a.hnew = haps.data_ptr(), out["hnew"].data_ptr()
        a.hap_idxs_out = out["quad"].data_ptr()
        a.like_out, a.eval_trace = out["like"].data_ptr(), out["evals"].data_ptr()
        a.accept_trace = out["acc"].data_ptr()
        a.pen, a.seed, a.generation, a.flags = pen, seed, gen, flags
        if nbr is not None:
            a.neighbors, a.neighbors_per_sample = nbr.data_ptr(), nbr.shape[1]
        return a

    def noalloc(self, L, a):
        return L.glp_run_generation_noalloc(C.byref(a), self.tran.data_ptr(),
                                            self.pc.ctypes.data, self.emit.data_ptr(),
                                            self.prob.data_ptr(), None)


def _allocating(torch, inp, flags=0, nbr=None):
    """The allocating entry point on the same inputs, in its own context."""
    ref = HMMLikeCUDA(0)
    ref.copy_tran_to_device(inp.m.tran)
    ref.copy_mutation_mat_to_device(inp.m.pc)
    ref.copy_emission_to_device(inp.m.emit, inp.m.t)

    def run(haps, pen, seed, gen):
        out = inp.outputs(torch)
        torch.cuda.synchronize()
        a = inp.args(haps, out, pen, seed, gen, flags, nbr)
        ref._c(ref.L.glp_run_generation(ref.ctx, C.byref(a)))
        ref._c(ref.L.glp_finish(ref.ctx))
        return out
    return ref, run


def _assert_same(torch, got, want, N, work, call):
    for k in ("evals", "like", "quad", "acc"):
        assert torch.equal(got[k], want[k]), (k, call)
    if work:
        assert torch.equal(got["hnew"][:2 * N], want["hnew"][:2 * N]), call


def _two_calls(torch, inp, flags=0, nbr=None):
    ref, run = _allocating(torch, inp, flags, nbr)
    L = ref.L
    work = not flags & nat.GLP_GEN_NO_WORK
    cur = inp.haps
    try:
        for call, (pen, gen) in enumerate(((0.4, 3), (1.0, 4))):
            want = run(cur, pen, 77, gen)
            got = inp.outputs(torch)
            torch.cuda.synchronize()
            rc = inp.noalloc(L, inp.args(cur, got, pen, 77, gen, flags, nbr))
            assert rc == nat.GLP_OK, (call, rc)
            torch.cuda.synchronize()
            _assert_same(torch, got, want, inp.N, work, call)
            if work:  # the next call starts from this one's haplotypes
                nxt = got["hnew"].clone()
                nxt[2 * inp.N:] = cur[2 * inp.N:]
                cur = nxt
    finally:
        ref.cleanup()


def test_noalloc_matches_allocating_entry_point_twice():
    import torch
    m, haps = _problem(21)
    _two_calls(torch, Inputs(torch, m, haps, 15))


def test_noalloc_without_hmm_work():
    import torch
    m, haps = _problem(22)
    _two_calls(torch, Inputs(torch, m, haps, 15), flags=nat.GLP_GEN_NO_WORK)


def test_noalloc_neighbour_table_and_kick_first():
    import torch
    m, haps = _problem(23, panel=30)
    inp = Inputs(torch, m, haps, 15)
    rng = np.random.default_rng(4)
    table = rng.integers(0, inp.H, size=(inp.N, 12)).astype(np.uint32)
    nbr = torch.from_numpy(table.view(np.int32)).to(inp.dev)
    _two_calls(torch, inp, flags=nat.GLP_GEN_KICK_FIRST, nbr=nbr)


def test_noalloc_call_allocates_nothing():
    """After the first call in a context (the set-up), a call leaves the
    device's free memory exactly as it was."""
    import torch
    m, haps = _problem(24)
    inp = Inputs(torch, m, haps, 15)
    L = nat.load()
    out = inp.outputs(torch)
    torch.cuda.synchronize()
    a = inp.args(inp.haps, out, 1.0, 5, 2)
    assert inp.noalloc(L, a) == nat.GLP_OK       # set-up and module loading
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(0)
    assert inp.noalloc(L, a) == nat.GLP_OK
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0


def test_noalloc_refuses_oversized_and_invalid_problems():
    L = nat.load()
    a = nat.GenerationArgs()
    a.num_samples, a.num_sites, a.num_cycles, a.num_haps = 4000, 4096, 10, 8000
    a.haps = a.hnew = a.hap_idxs_out = 16   # never dereferenced: refused first
    a.pen = 1.0
    dummy = np.zeros(16, np.float32)
    rc = L.glp_run_generation_noalloc(C.byref(a), 16, dummy.ctypes.data, 16, 16, None)
    assert rc == nat.GLP_ERR_TOO_LARGE
    # a kick-started first proposal needs panel rows after the 2N sample rows
    a.num_samples, a.num_sites, a.num_haps = 8, 64, 16
    a.flags = nat.GLP_GEN_KICK_FIRST
    rc = L.glp_run_generation_noalloc(C.byref(a), 16, dummy.ctypes.data, 16, 16, None)
    assert rc == nat.GLP_ERR_ARG
