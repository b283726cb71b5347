"""Many chunks of uneven size in one persistent launch (glp_run_batch): each
chunk's outputs are bit-identical to the same generation run alone through
glp_run_generation, and agree with the oracle."""
import ctypes as C

import numpy as np
import pytest

from glphase_gb300 import native as nat, synth
from glphase_gb300.hmmlike import HMMLikeCUDA

pytestmark = pytest.mark.gpu


class Chunk:
    def __init__(self, dev, N, S, Cc, seed, panel=0):
        import torch
        w = synth.Workload("b", N=N, S=S, founders=7, depth=3.0, burnin=4, sampling=2,
                           cycles=Cc, panel_haps=panel, seed=seed)
        self.m, self.haps = synth.initial_state(synth.generate(w), seed=seed)
        self.N, self.S, self.C = N, S, Cc
        self.H = self.haps.shape[0]
        self.seed = 1000 + seed
        self.pb = C.c_void_p()
        dev._c(dev.L.glp_problem_create(dev.ctx, C.byref(self.pb)))
        t = np.ascontiguousarray(self.m.tran)
        pc = np.ascontiguousarray(self.m.pc)
        e = np.ascontiguousarray(self.m.emit)
        pr = np.ascontiguousarray(self.m.t)
        dev._c(dev.L.glp_problem_set_model(self.pb, t.ctypes.data, pc.ctypes.data,
                                           e.ctypes.data, pr.ctypes.data, N, S))
        self.d_haps = torch.from_numpy(self.haps.view(np.int64)).cuda()
        self.reset()

    def reset(self):
        import torch
        self.d_hnew = self.d_haps.clone()
        self.d_quad = torch.zeros((4, self.N), dtype=torch.int32, device="cuda")
        self.d_like = torch.zeros(self.N, dtype=torch.float64, device="cuda")
        self.d_evals = torch.zeros((self.N, self.C + 1), dtype=torch.float64, device="cuda")
        self.d_acc = torch.zeros((self.N, max(self.C, 1)), dtype=torch.uint8, device="cuda")

    def args(self, pen, gen):
        a = nat.GenerationArgs()
        a.num_samples, a.num_sites, a.num_cycles, a.num_haps = self.N, self.S, self.C, self.H
        a.haps, a.hnew = self.d_haps.data_ptr(), self.d_hnew.data_ptr()
        a.hap_idxs_out = self.d_quad.data_ptr()
        a.pen, a.seed, a.generation = pen, self.seed, gen
        a.like_out, a.eval_trace = self.d_like.data_ptr(), self.d_evals.data_ptr()
        a.accept_trace = self.d_acc.data_ptr()
        return a

    def outputs(self):
        return dict(quad=self.d_quad.cpu().numpy().view(np.uint32).copy(),
                    hnew=self.d_hnew.cpu().numpy().view(np.uint64).copy(),
                    like=self.d_like.cpu().numpy().copy(),
                    evals=self.d_evals.cpu().numpy().copy(),
                    acc=self.d_acc.cpu().numpy()[:, :self.C].copy())


@pytest.fixture(scope="module")
def dev():
    import torch
    torch.cuda.init()
    d = HMMLikeCUDA(0)
    yield d
    d.cleanup()


def test_batch_equals_alone_and_oracle(dev, oracle_lib):
    import torch
    sizes = [(37, 300, 12), (5, 64, 8), (120, 1000, 20), (64, 65, 10), (9, 1, 4), (80, 700, 0)]
    chunks = [Chunk(dev, N, S, Cc, seed=i + 1, panel=6 if i == 2 else 0)
              for i, (N, S, Cc) in enumerate(sizes)]
    torch.cuda.synchronize()
    gen, pen = 3, 0.6
    # the whole batch in one launch
    args = (nat.GenerationArgs * len(chunks))(*[ch.args(pen, gen) for ch in chunks])
    pbs = (C.c_void_p * len(chunks))(*[ch.pb for ch in chunks])
    dev._c(dev.L.glp_run_batch(dev.ctx, len(chunks), pbs, args))
    dev._c(dev.L.glp_finish(dev.ctx))
    batched = [ch.outputs() for ch in chunks]
    # every chunk alone, through the context's own model
    for ch, out in zip(chunks, batched):
        ch.reset()
        dev.copy_tran_to_device(ch.m.tran)
        dev.copy_mutation_mat_to_device(ch.m.pc)
        dev.copy_emission_to_device(ch.m.emit, ch.m.t)
        torch.cuda.synchronize()
        a = ch.args(pen, gen)
        dev._c(dev.L.glp_run_generation(dev.ctx, C.byref(a)))
        dev._c(dev.L.glp_finish(dev.ctx))
        alone = ch.outputs()
        for k in ("quad", "like", "acc"):
            assert np.array_equal(out[k], alone[k]), k
        assert np.array_equal(out["evals"], alone["evals"])
        assert np.array_equal(out["hnew"][:2 * ch.N], alone["hnew"][:2 * ch.N])
    # and against the oracle
    from test_gpu_parity import check_against_oracle
    O = oracle_lib
    for ch, out in zip(chunks, batched):
        quad, props = O.sample_surrogates(ch.seed, gen, ch.N, ch.C, 0, ch.H)
        check_against_oracle(O, ch.m, ch.haps, quad, props, pen, out, ch.seed, gen)
    for ch in chunks:
        dev.L.glp_problem_destroy(ch.pb)


def _device_problems(dev, sizes, cycles, burnin, kick=False):
    from glphase_gb300 import synth_device as sd
    from glphase_gb300.batch import DeviceProblem
    w = synth.Workload("dev", N=1, S=1, founders=9, depth=3.0, burnin=burnin, sampling=2,
                       panel_haps=12 if kick else 0)
    out = []
    for i, (N, S) in enumerate(sizes):
        ch = sd.generate(w, N, S, seed=50 + i)
        out.append(DeviceProblem(dev, ch, cycles, seed=700 + i, burnin=burnin, kick_start=kick))
    return out


@pytest.mark.parametrize("kick", [False, True])
def test_prepared_batch_graph_replay(dev, kick):
    """G generations replayed from one captured CUDA graph (device-side
    advance) equal G generations driven from the host with glp_run_batch."""
    import torch
    from glphase_gb300.batch import PreparedBatch, run_batch
    sizes = [(33, 200), (7, 640), (90, 129), (20, 1024)]
    G = 5
    a = _device_problems(dev, sizes, 9, burnin=3, kick=kick)
    b = _device_problems(dev, sizes, 9, burnin=3, kick=kick)
    torch.cuda.synchronize()
    pb = PreparedBatch(dev, a, generation=0)
    for g in range(G):
        pb.run(graph=(g % 2 == 0))
    dev._c(dev.L.glp_finish(dev.ctx))
    for g in range(G):
        run_batch(dev, b, g)
        dev._c(dev.L.glp_finish(dev.ctx))
    for x, y in zip(a, b):
        assert torch.equal(x.haps, y.haps)
        assert torch.equal(x.quad, y.quad)
        assert torch.equal(x.like, y.like)
    pb.close()
    for p in a + b:
        p.close()


def test_batch_argument_errors(dev):
    ch = Chunk(dev, 6, 100, 4, seed=9)
    a = ch.args(1.0, 0)
    bad = nat.GenerationArgs.from_buffer_copy(a)
    bad.num_sites = 99
    pbs = (C.c_void_p * 2)(ch.pb, ch.pb)
    arr = (nat.GenerationArgs * 2)(a, bad)
    assert dev.L.glp_run_batch(dev.ctx, 2, pbs, arr) == nat.GLP_ERR_STATE
    assert dev.L.glp_run_batch(dev.ctx, 0, pbs, arr) == nat.GLP_ERR_ARG
    dev.L.glp_problem_destroy(ch.pb)
