"""The reference's own device tests (src/testing/cuda_tests.cpp:118-656)
restated against the drop-in boundary: HMMLike -> HMMLikeCUDA ->
glp_run_hmm_on_device, with VQ-packed GLs (GLPack), host-drawn proposals
(UnifSampler) and accept penalty 1.

Panels of 12 haplotypes x 16 words carry all-ones words at designed places
and the GLs of the samples are set to hom-alt (likelihood 100) over the same
words, so the MH chain must settle on the planted parents.  As in the
reference, the checks are stochastic but have a wide margin."""
import numpy as np
import pytest

from glphase_gb300.glpack import GLPack
from glphase_gb300.hmmlike import HMMLike, HMMLikeCUDA, UnifSampler

pytestmark = pytest.mark.gpu

NUM_SITES = 1024
WORD = 64
NW = NUM_SITES // WORD
ALL = np.uint64(0xFFFFFFFFFFFFFFFF)


class Pack:
    """GLPack view in the HMMLike constructor's terms."""

    def __init__(self, gl, rng):
        self.gp = GLPack(gl, rng)
        self.num_sites = gl.shape[1]
        self.num_samps = gl.shape[0]

    def packed_gls(self):
        return self.gp.packed_gls()

    def code_book(self):
        return self.gp.code_book()


def model_mats(num_haps):
    """mutMat and tran built the way cuda_tests.cpp:239-276 builds them."""
    avg_site_dist = 1000
    mu = np.float32(0)
    for i in range(1, num_haps):
        mu = np.float32(float(mu) + 1.0 / i)
    mu = np.float32(1.0) / mu
    rho = np.float32(0.5 * float(mu) * (NUM_SITES - 1) / (NUM_SITES * avg_site_dist))
    mu = np.float32(mu / (np.float32(num_haps) + mu))
    d, o, a = (1 - mu) * (1 - mu), mu * (1 - mu), mu * mu
    pc = np.full((4, 4), o, np.float32)
    for i in range(4):
        pc[i, i], pc[i, 3 - i] = d, a
    tran = np.zeros((NUM_SITES, 3), np.float32)
    r = np.float32(rho * avg_site_dist) / (np.float32(rho * avg_site_dist) + np.float32(4))
    tran[1:] = ((1 - r) * (1 - r), r * (1 - r), r * r)
    return pc, tran


def gls(num_samps, rng):
    """Random GLs, then hom-alt blocks of cuda_tests.cpp:278-303 and 331-342."""
    g = rng.random((num_samps, NUM_SITES, 3)).astype(np.float32)
    hi = np.float32(100)
    g[0, 0:WORD, 2] = hi           # sample 0, word 0
    g[0, 5 * WORD:6 * WORD, 2] = hi  # sample 0, word 5
    g[1, 1 * WORD:2 * WORD, 2] = hi  # sample 1, word 1
    g[1, 7 * WORD:8 * WORD, 2] = hi  # sample 1, word 7
    return g


def panel():
    p = np.zeros((12, NW), np.uint64)
    p[5, 0] = p[6, 0] = p[5, 5] = p[6, 5] = ALL
    p[7, 1] = p[8, 1] = p[7, 7] = p[8, 7] = ALL
    return p


@pytest.fixture(scope="module")
def rng():
    return np.random.default_rng(112)


def test_one_parent_pair_found(rng):
    """cuda_tests.cpp:205-322: one of the father/mother pairs is planted."""
    pc, tran = model_mats(12)
    g = gls(2, rng)
    hap_panel = panel()
    sampler = UnifSampler(rng, 6, 12)
    hm = HMMLike(hap_panel.reshape(-1), 12, Pack(g, rng), 100, tran, pc, sampler, rng)
    first, last, idx = hm.run_hmm_on_samples()
    assert (first, last) == (0, 1)
    assert idx.shape == (8,)
    for i in (0, 2):
        assert (4 < idx[i] < 7) or (4 < idx[i + 1] < 7)
    for i in (4, 6):
        assert (6 < idx[i] < 9) or (6 < idx[i + 1] < 9)


def test_both_parent_pairs_found(rng):
    """cuda_tests.cpp:324-479: father and mother pairs both planted."""
    pc, tran = model_mats(12)
    g = gls(2, rng)
    g[0, 2 * WORD:3 * WORD, 2] = 100
    g[1, 3 * WORD:4 * WORD, 2] = 100
    hp = panel()
    hp[10, 2] = ALL
    hp[11, 3] = ALL
    sampler = UnifSampler(rng, 6, 12)
    hm = HMMLike(hp.reshape(-1), 12, Pack(g, rng), 100, tran, pc, sampler,
                 np.random.default_rng(114))
    _, _, idx = hm.run_hmm_on_samples()
    for i in (0, 2):
        h1, h2 = sorted(idx[i:i + 2])
        assert h2 == 10 and 5 <= h1 <= 6
        h3, h4 = sorted(idx[i + 4:i + 6])
        assert h4 == 11 and 7 <= h3 <= 8


def test_good_quadruple_scores_higher(rng):
    """cuda_tests.cpp:385-428: like({5,10,6,10}) > like({2,2,2,2}), both <= 0."""
    import ctypes as C
    from glphase_gb300 import native as nat
    pc, tran = model_mats(12)
    g = gls(2, rng)
    g[0, 2 * WORD:3 * WORD, 2] = 100
    hp = panel()
    hp[10, 2] = ALL
    pk = Pack(g, rng)
    dev = HMMLikeCUDA(0)
    dev.copy_tran_to_device(tran)
    dev.copy_mutation_mat_to_device(pc)
    dev.copy_code_book_to_device(pk.code_book())
    dev.copy_packed_gls_to_device(pk.packed_gls())
    likes = []
    for quad0 in ([2, 2, 2, 2], [5, 10, 6, 10]):
        quad = np.array([quad0, [0, 0, 0, 0]], np.uint32).T.copy()
        a = nat.GenerationArgs()
        out = np.zeros_like(quad)
        ev = np.zeros((2, 1), np.float64)
        h = np.ascontiguousarray(hp)
        a.num_samples, a.num_sites, a.num_cycles, a.num_haps = 2, NUM_SITES, 0, 12
        a.haps, a.hap_idxs_in, a.hap_idxs_out = h.ctypes.data, quad.ctypes.data, out.ctypes.data
        a.props = quad.ctypes.data
        a.pen, a.flags = 1.0, nat.GLP_GEN_VQ | nat.GLP_GEN_NO_WORK
        a.eval_trace = ev.ctypes.data
        assert dev.L.glp_run_generation_host(dev.ctx, C.byref(a)) == 0
        likes.append(ev[0, 0])
    dev.cleanup()
    assert likes[0] <= 0 and likes[1] <= 0
    assert likes[1] > likes[0]


def test_shim_signatures_round_trip():
    """RunHMMOnDevice rejects mismatched sizes as the reference does
    (hmmLike.cu:407-423), through the C ABI's status codes."""
    import ctypes as C
    from glphase_gb300 import native as nat
    dev = HMMLikeCUDA(0)
    pc, tran = model_mats(12)
    dev.copy_tran_to_device(tran)
    dev.copy_mutation_mat_to_device(pc)
    with pytest.raises(nat.GlpError) as e:   # no GLs copied yet
        dev.run_hmm_on_device(panel().reshape(-1), np.zeros(200, np.uint32), NUM_SITES, 2,
                              100, np.zeros(8, np.uint32), 1)
    assert e.value.code in (nat.GLP_ERR_STATE, nat.GLP_ERR_ARG)
    dev.cleanup()
