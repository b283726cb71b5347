"""Device allele tallies (glp_tally / glp_result) against the oracle's
restatement of Impute::replace / Impute::result (bit-exact) and the golden
tallies produced by the reference's own impute.cpp."""
import numpy as np
import pytest

from glphase_gb300.hmmlike import HMMLikeCUDA

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev():
    import torch
    torch.cuda.init()
    d = HMMLikeCUDA(0)
    yield d
    d.cleanup()


def test_tally_matches_oracle_and_result(dev, oracle_lib):
    import torch
    O = oracle_lib
    rng = np.random.default_rng(3)
    N, S, gens = 37, 333, 6
    wn = (S + 63) // 64
    hsum_cpu = np.zeros(2 * N * S, np.uint32)
    hsum = torch.zeros(2 * N * S, dtype=torch.int32, device="cuda")
    for g in range(gens):
        haps = rng.integers(0, 2**63, size=(2 * N, wn), dtype=np.uint64)
        for s in range(N):
            O.lib().glpo_replace(haps.reshape(-1), wn, S, s, hsum_cpu)
        d = torch.from_numpy(haps.view(np.int64)).cuda()
        torch.cuda.synchronize()
        dev._c(dev.L.glp_tally(dev.ctx, d.data_ptr(), N, S, hsum.data_ptr()))
        dev._c(dev.L.glp_finish(dev.ctx))
    assert np.array_equal(hsum.cpu().numpy().view(np.uint32), hsum_cpu)
    prob = torch.zeros(2 * N * S, dtype=torch.float32, device="cuda")
    dev._c(dev.L.glp_result(dev.ctx, hsum.data_ptr(), N, S, gens, prob.data_ptr()))
    dev._c(dev.L.glp_finish(dev.ctx))
    want = np.zeros(2 * N * S, np.float32)
    O.lib().glpo_result(hsum_cpu, N, S, gens, want)
    assert np.array_equal(prob.cpu().numpy(), want)


def test_tally_golden_from_reference(dev, golden):
    """The golden replace tallies came from the reference's Impute::replace."""
    import torch
    hs = golden["replace_haps"]              # [gens][2N=6][wn=2]
    hsum = torch.zeros(2 * 3 * 100, dtype=torch.int32, device="cuda")
    for g in range(hs.shape[0]):
        d = torch.from_numpy(np.ascontiguousarray(hs[g]).view(np.int64)).cuda()
        torch.cuda.synchronize()
        dev._c(dev.L.glp_tally(dev.ctx, d.data_ptr(), 3, 100, hsum.data_ptr()))
        dev._c(dev.L.glp_finish(dev.ctx))
    assert np.array_equal(hsum.cpu().numpy().view(np.uint32), golden["replace_hsum"])
