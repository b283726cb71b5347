"""GL packing for the device (glphase_gb300/glpack.py) against the reference's
unit tests (src/testing/glPack_unittests.cpp) and the decode rule of the
device kernel (hmmLike.cu:12-28)."""
import numpy as np

from glphase_gb300.glpack import GLPack, GLVQ, gl2halfchar


def test_8bit_pack_known_answers():
    """glPack_unittests.cpp:27-67: (RR, Het) -> 4-bit halves -> 0, 18, 52."""
    gls = np.array([[0, 1 / 16, 15 / 16], [2 / 16, 3 / 16, 11 / 16], [4 / 16, 5 / 16, 7 / 16],
                    [0, 0, 1], [0, 0, 1]], np.float32).reshape(5, 1, 3)
    packed = GLPack(gls, use_vq=False).packed_gls()
    assert packed.shape == (1, 5)
    first = (packed[0] >> 24) & 0xFF
    assert list(first[:3]) == [0, 18, 52]


def test_8bit_pack_multisite_known_answers():
    """glPack_unittests.cpp:69-117: two sites per sample, codes in the two
    most significant bytes: sample 1 (0, 18), sample 2 (52, 3), sample 3
    (0, 119)."""
    gls = np.array([[[0, 1 / 16, 15 / 16], [2 / 16, 3 / 16, 11 / 16]],
                    [[4 / 16, 5 / 16, 7 / 16], [0.9 / 16, 3.5 / 16, 11.6 / 16]],
                    [[0, 0, 1], [0.5, 0.5, 0]]], np.float32)
    packed = GLPack(gls, use_vq=False).packed_gls()
    b0 = (packed[0] >> 24) & 0xFF
    b1 = (packed[0] >> 16) & 0xFF
    assert list(zip(b0, b1)) == [(0, 18), (52, 3), (0, 119)]


def test_halfchar_rule():
    """GL2HalfChar (glPack.cpp:232-243): floor(max(x - eps, 0) * 16)."""
    x = np.array([0, 1 / 16, 0.5, 15.999 / 16, 1 - 1e-3], np.float32)
    assert list(gl2halfchar(x)) == [0, 0, 7, 15, 15]


def test_vq_codebook_covers_distinct_gls():
    """glPack_unittests.cpp:127-161: every distinct GL pair has a codebook
    entry within 0.01 and FindGLCode returns that entry."""
    gls = np.array([[0, 1 / 16, 15 / 16], [2 / 16, 3 / 16, 11 / 16], [4 / 16, 5 / 16, 7 / 16],
                    [0, 0, 1], [0, 0, 1]], np.float32)
    vq = GLVQ(gls, np.random.default_rng(111), 16)
    cb = vq.codebook
    for rr, het, _ in gls:
        d = np.abs(cb[:, 0] - rr) + np.abs(cb[:, 1] - het)
        match = np.where((np.abs(cb[:, 0] - rr) < 0.01) & (np.abs(cb[:, 1] - het) < 0.01))[0]
        assert len(match) >= 1
        assert int(vq.find_code(rr, het)) == int(match[0]) or d[int(vq.find_code(rr, het))] < 0.02


def test_vq_packing_layout_and_decode():
    """Eight 4-bit codes per word, first site in the most significant nibble,
    laid out [ceil(S/8)][N]; the decode of hmmLike.cu:12-28 recovers the
    codebook entry of each site."""
    rng = np.random.default_rng(3)
    N, S = 5, 21
    gls = rng.dirichlet([1, 1, 1], size=(N, S)).astype(np.float32)
    gp = GLPack(gls, rng)
    packed, cb = gp.packed_gls(), gp.code_book()
    assert packed.shape == ((S + 7) // 8, N)
    for s in range(N):
        for m in range(S):
            code = (int(packed[m // 8, s]) >> (28 - 4 * (m % 8))) & 15
            rr = gls[s, m, 0] / gls[s, m].sum()
            het = gls[s, m, 1] / gls[s, m].sum()
            d = (cb[:, 0] - rr) ** 2 + (cb[:, 1] - het) ** 2
            assert code == int(np.argmin(d))
