"""GL vector quantisation on the device (glp_vq_train / glp_vq_pack) against
the host restatement in glphase_gb300/glpack.py (same comparator, same
summation order, same empty-entry rule: bit for bit) and the reference's
codebook test (glPack_unittests.cpp:127-161)."""
import numpy as np
import pytest

from glphase_gb300.glpack import GLPack, GLVQ
from glphase_gb300.hmmlike import HMMLikeCUDA

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev():
    import torch
    torch.cuda.init()
    d = HMMLikeCUDA(0)
    yield d
    d.cleanup()


def random_gls(N, S, seed, alpha=0.3):
    rng = np.random.default_rng(seed)
    return rng.dirichlet([alpha] * 3, size=(N, S)).astype(np.float32)


def few_distinct_gls(N, S, seed):
    """Only three distinct GL triples: most entries lose their points and
    move onto the points SplitMix64 picks."""
    rng = np.random.default_rng(seed)
    table = np.array([[0.9, 0.1, 0.0], [0.1, 0.8, 0.1], [0.0, 0.05, 0.95]], np.float32)
    return table[rng.integers(0, 3, size=(N, S))]


@pytest.mark.parametrize("N,S,kind,size,seed", [
    (200, 300, "random", 16, 1),      # 60,000 points: 4 blocks, ragged last block
    (7, 9, "random", 16, 2),          # fewer points than one run
    (64, 1024, "few", 16, 3),         # empty entries every update
    (128, 128, "random", 4, 4),       # the 2-bit codebook
])
def test_training_matches_host(dev, N, S, kind, size, seed):
    gl = random_gls(N, S, seed) if kind == "random" else few_distinct_gls(N, S, seed)
    host = GLVQ(gl, np.random.default_rng(10 + seed), size, seed=seed)
    gpu = GLVQ(gl, np.random.default_rng(10 + seed), size, seed=seed, device=dev)
    assert gpu.iterations == host.iterations
    assert np.array_equal(gpu.codebook.view(np.uint32), host.codebook.view(np.uint32))


@pytest.mark.parametrize("bits,S", [(4, 300), (4, 13), (2, 37)])
def test_packing_matches_host(dev, bits, S):
    gl = random_gls(50, S, 7)
    host = GLPack(gl, np.random.default_rng(5), bits=bits, seed=9)
    gpu = GLPack(gl, np.random.default_rng(5), bits=bits, seed=9, device=dev)
    assert np.array_equal(gpu.code_book(), host.code_book())
    got, want = gpu.packed_gls(), host.packed_gls()
    assert got.shape == want.shape == ((S + 32 // bits - 1) // (32 // bits), 50)
    assert np.array_equal(got, want)


def test_codebook_covers_distinct_gls(dev):
    """glPack_unittests.cpp:127-161 on the device-trained codebook: every
    distinct GL pair has an entry within 0.01."""
    gls = np.array([[0, 1 / 16, 15 / 16], [2 / 16, 3 / 16, 11 / 16], [4 / 16, 5 / 16, 7 / 16],
                    [0, 0, 1], [0, 0, 1]], np.float32).reshape(5, 1, 3)
    vq = GLVQ(gls, np.random.default_rng(111), 16, device=dev)
    cb = vq.codebook
    for rr, het, _ in gls.reshape(-1, 3):
        near = (np.abs(cb[:, 0] - rr) < 0.01) & (np.abs(cb[:, 1] - het) < 0.01)
        assert near.any()


def test_argument_errors(dev):
    import ctypes as C
    import torch
    g = torch.zeros(30, dtype=torch.float32, device="cuda")
    cb = np.zeros((17, 2), np.float32)
    rc = dev.L.glp_vq_train(dev.ctx, g.data_ptr(), 10, 17, cb.ctypes.data, 0, 10, None)
    assert rc == 1 and b"codebook_size" in dev.L.glp_last_error(dev.ctx)
    rc = dev.L.glp_vq_pack(dev.ctx, g.data_ptr(), 2, 5, cb.ctypes.data, 16, 3, g.data_ptr())
    assert rc == 1 and b"bits" in dev.L.glp_last_error(dev.ctx)
    # a codebook that cannot converge in one update reports it
    gl = random_gls(20, 30, 1)
    d = torch.from_numpy(gl.reshape(-1, 3)).cuda()
    torch.cuda.synchronize()
    cb16 = np.ascontiguousarray(np.random.default_rng(0).random((16, 2)).astype(np.float32))
    it = C.c_uint32(0)
    rc = dev.L.glp_vq_train(dev.ctx, d.data_ptr(), 600, 16, cb16.ctypes.data, 0, 1, C.byref(it))
    assert rc == 8 and b"failed to converge" in dev.L.glp_last_error(dev.ctx)
