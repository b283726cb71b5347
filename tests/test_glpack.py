"""GL packing for the device (glphase_gb300/glpack.py) against the reference's
unit tests (src/testing/glPack_unittests.cpp), the decode rule of the
device kernel (hmmLike.cu:12-28) and, where oracle/_ref holds it, the
reference's own glPack.cpp / glVQ.cpp compiled from its tree."""
import numpy as np
import pytest

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


def _edge_gls(rng, N, S):
    """Random GL trios, unnormalised in part, with some homRef/het values on
    the 1/16 grid where GL2HalfChar's epsilon matters, and one-hot trios."""
    gl = rng.dirichlet([0.3, 0.3, 0.3], (N, S)).astype(np.float32)
    grid = rng.random((N, S)) < 0.2
    k = rng.integers(0, 8, (N, S, 2)).astype(np.float32) / 16
    gl[grid, 0], gl[grid, 1] = k[grid, 0], k[grid, 1]
    gl[grid, 2] = 1 - gl[grid, 0] - gl[grid, 1]
    hot = rng.random((N, S)) < 0.05
    gl[hot] = np.eye(3, dtype=np.float32)[rng.integers(0, 3, int(hot.sum()))]
    scale = np.where(rng.random((N, 1, 1)) < 0.5, rng.random((N, 1, 1)) + 0.1, 1.0)
    return (gl * scale).astype(np.float32)


@pytest.mark.skipif("not __import__('oracle').ref_glpack_available()")
def test_packing_matches_live_reference_build(oracle_lib):
    """GLPack::GetPackedGLs of the reference's compiled glPack.cpp / glVQ.cpp
    against glpack.py, word for word: the 8-bit nibble form, and 2-, 4- and
    8-bit VQ codes packed against the codebook the reference trained (the
    codebook training itself differs by design: binary64 sums in a fixed
    order and a counter-based pick for empty entries).  Site counts that
    leave a partial last word take the array's first GL there, as the
    reference does."""
    O = oracle_lib
    rng = np.random.default_rng(31)
    for N, S in ((1, 1), (1, 9), (3, 4), (7, 33), (29, 282), (40, 256)):
        gl = _edge_gls(rng, N, S)
        want, _ = O.ref_glpack(gl, use_vq=False)
        assert np.array_equal(GLPack(gl, use_vq=False).packed_gls(), want), (N, S)
        for bits in (2, 4, 8):
            want, cb = O.ref_glpack(gl, use_vq=True, bits=bits)
            gp = GLPack(gl, np.random.default_rng(0), use_vq=True, bits=bits)
            gp.vq.codebook = cb.copy()
            assert np.array_equal(gp.packed_gls(), want), (N, S, bits)
