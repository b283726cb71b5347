"""GL packing for the device: the reference's GLPack / GLVQ restated with
numpy (src/glPack.cpp:32-163, src/glVQ.cpp:26-165).

* VQ mode: a 16-entry (homRef, het) codebook trained with Lloyd's algorithm
  (seeded at (0,1), (0,0), (1,0), (1/3,1/3) plus random entries; iterate
  until the assignment variance changes by less than 1 %, at most 1000
  iterations), then eight 4-bit codes per uint32, first site in the most
  significant nibble, laid out [ceil(S/8)][N] (sample-strided).
* 8-bit mode: (homRef, het) each quantised to 4 bits, four sites per uint32.

Inputs are the genotype probabilities [N][S][3] (homRef, het, homAlt) that
Insti hands to GLPack after initialize (src/insti.cpp:1634-1640).
"""
from __future__ import annotations

import numpy as np

F32 = np.float32
EPS32 = np.finfo(np.float32).eps


def _normalise(gl: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    g = np.asarray(gl, dtype=F32)
    s = ((g[..., 0] + g[..., 1]).astype(F32) + g[..., 2]).astype(F32)
    return (g[..., 0] / s).astype(F32), (g[..., 1] / s).astype(F32)


def nearest_code(codebook: np.ndarray, rr: np.ndarray, het: np.ndarray) -> np.ndarray:
    """GLVQ::FindGLCode (glVQ.cpp:214-223): index of the nearest entry, the
    first one on ties (std::min_element)."""
    cb = np.asarray(codebook, dtype=np.float64)
    d = (rr.astype(np.float64)[..., None] - cb[:, 0]) ** 2 + \
        (het.astype(np.float64)[..., None] - cb[:, 1]) ** 2
    return np.argmin(d, axis=-1).astype(np.uint8)


class GLVQ:
    """Codebook training of glVQ.cpp:26-146."""

    def __init__(self, gl: np.ndarray, rng: np.random.Generator, size: int = 16,
                 max_iter: int = 1000):
        if size < 4 or size > 256:
            raise ValueError("codebook size must be in [4, 256]")
        rr, het = _normalise(np.asarray(gl).reshape(-1, 3))
        cb = [(0.0, 1.0), (0.0, 0.0), (1.0, 0.0), (1.0 / 3, 1.0 / 3)]
        for _ in range(4, size):
            a = float(F32(rng.random()))
            cb.append((a, float(F32(rng.random() * (1 - a)))))
        self.codebook = np.array(cb, dtype=F32)
        pts = np.stack([rr, het], axis=1)

        def assign(cbk):
            code = nearest_code(cbk, rr, het)
            var = float(np.sum((pts.astype(np.float64) - cbk[code].astype(np.float64)) ** 2))
            return code, var

        code, cur = assign(self.codebook)
        prev = np.finfo(np.float64).max
        it = 0
        while abs(cur - prev) > cur / 100:
            it += 1
            if it > max_iter:
                raise RuntimeError(f"[GLVQ] Clustering failed to converge within {max_iter} "
                                   "iterations")
            prev = cur
            new = np.zeros_like(self.codebook)
            counts = np.bincount(code, minlength=size)
            sums_rr = np.bincount(code, weights=rr.astype(np.float64), minlength=size)
            sums_het = np.bincount(code, weights=het.astype(np.float64), minlength=size)
            for i in range(size):
                if counts[i]:
                    new[i] = (sums_rr[i] / counts[i], sums_het[i] / counts[i])
                else:
                    j = int(rng.integers(0, len(pts)))
                    new[i] = pts[j]
            self.codebook = new
            code, cur = assign(self.codebook)

    def find_code(self, rr, het):
        return nearest_code(self.codebook, np.asarray(rr, F32), np.asarray(het, F32))


def gl2halfchar(x: np.ndarray) -> np.ndarray:
    """GLPack::GL2HalfChar (glPack.cpp:232-243): floor(max(x - eps, 0) * 16)."""
    x = np.maximum(np.asarray(x, F32) - EPS32, F32(0.0)).astype(F32)
    return np.floor(x * F32(16)).astype(np.uint32)


class GLPack:
    """Packed GLs for the device (src/glPack.hpp:38-78)."""

    def __init__(self, gl: np.ndarray, rng: np.random.Generator | None = None,
                 use_vq: bool = True, bits: int = 4):
        self.gl = np.ascontiguousarray(gl, dtype=F32)
        self.num_samps, self.num_sites = self.gl.shape[0], self.gl.shape[1]
        self.use_vq = use_vq
        self.bits = bits if use_vq else 8
        if use_vq:
            if 8 % bits:
                raise ValueError("bits per GL must divide 8")
            self.vq = GLVQ(self.gl, rng if rng is not None else np.random.default_rng(),
                           2 ** bits)

    @property
    def num_sites_(self):
        return self.num_sites

    def code_book(self) -> np.ndarray:
        return self.vq.codebook.copy()

    def packed_gls(self) -> np.ndarray:
        """[ceil(S/8 or S/4)][N] uint32 (glPack.cpp:112-165)."""
        N, S = self.num_samps, self.num_sites
        per = 32 // self.bits
        nblk = (S + per - 1) // per
        # sites past the end use the very first GL of the array (glPack.cpp:147-149)
        idx = np.arange(nblk * per)
        g = self.gl[:, np.minimum(idx, S - 1), :].copy()
        g[:, idx >= S, :] = self.gl[0, 0, :]
        rr, het = _normalise(g)
        if self.use_vq:
            codes = self.vq.find_code(rr, het).astype(np.uint32)
        else:
            codes = (gl2halfchar(rr) << 4) | gl2halfchar(het)
        codes = codes.reshape(N, nblk, per)
        words = np.zeros((N, nblk), dtype=np.uint32)
        for k in range(per):
            words |= codes[..., k] << np.uint32(32 - self.bits * (k + 1))
        return np.ascontiguousarray(words.T)
