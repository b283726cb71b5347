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
    """GLVQ::FindGLCode with GLVQHelper::EuclidianDist (glVQ.cpp:214-223,
    glVQ.hpp:23-30): differences in binary32, squared and summed in binary64,
    the index of the first smallest square root (std::min_element)."""
    cb = np.asarray(codebook, dtype=F32)
    rr = np.asarray(rr, dtype=F32)
    het = np.asarray(het, dtype=F32)
    out = np.empty(rr.shape, dtype=np.uint8)
    flat_rr, flat_het, flat_out = rr.reshape(-1), het.reshape(-1), out.reshape(-1)
    step = 1 << 20
    for i in range(0, flat_rr.size, step):
        dx = (cb[:, 0][None, :] - flat_rr[i:i + step, None]).astype(np.float64)
        dy = (cb[:, 1][None, :] - flat_het[i:i + step, None]).astype(np.float64)
        flat_out[i:i + step] = np.argmin(np.sqrt(dx * dx + dy * dy), axis=1)
    return out


# Summation order of the device trainer (glp_vq.cuh): point p = b*BLOCK +
# j*THREADS + t belongs to run t of block b; a run adds its points in j order,
# a block its runs in t order, then the blocks in b order (binary64).
_RUN, _THREADS = 64, 256
_BLOCK = _RUN * _THREADS


def ordered_sum(values: np.ndarray) -> float:
    v = np.asarray(values, dtype=np.float64).reshape(-1)
    nblk = max(1, (v.size + _BLOCK - 1) // _BLOCK)
    pad = np.zeros(nblk * _BLOCK, dtype=np.float64)
    pad[:v.size] = v
    runs = np.cumsum(pad.reshape(nblk, _RUN, _THREADS), axis=1)[:, -1, :]
    blocks = np.cumsum(runs, axis=1)[:, -1]
    return float(np.cumsum(blocks)[-1])


_M64 = (1 << 64) - 1


def splitmix64(x: int) -> int:
    """SplitMix64 (Steele, Lea, Flood 2014)."""
    x = (x + 0x9E3779B97F4A7C15) & _M64
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & _M64
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & _M64
    return x ^ (x >> 31)


def empty_point(seed: int, it: int, k: int, P: int) -> int:
    """The point an entry without points moves to at update `it` (the
    reference draws a random point, glVQ.cpp:127-133)."""
    return splitmix64((seed & _M64) ^ ((it << 16) | k)) % P


def initial_codebook(rng: np.random.Generator, size: int) -> np.ndarray:
    """(0,1), (0,0), (1,0), (1/3,1/3), then random (RR, Het(1-RR)) entries
    (glVQ.cpp:38-50)."""
    cb = [(0.0, 1.0), (0.0, 0.0), (1.0, 0.0), (1.0 / 3, 1.0 / 3)]
    for _ in range(4, size):
        a = float(F32(rng.random()))
        cb.append((a, float(F32(rng.random() * (1 - a)))))
    return np.array(cb, dtype=F32)


class GLVQ:
    """Codebook training of glVQ.cpp:26-146: Lloyd iterations from the
    initial entries until the total squared distance changes by at most
    1 %.  A point's entry is the nearest by the reference's comparator; the
    new entry is the binary64 mean of its points (summed in the device
    trainer's fixed order, rounded to binary32); an entry without points
    moves onto the point ``empty_point`` picks.  ``device`` (an
    ``hmmlike.HMMLikeCUDA``) trains with ``glp_vq_train`` on the GPU; the
    result is the same bit for bit."""

    def __init__(self, gl: np.ndarray, rng: np.random.Generator, size: int = 16,
                 max_iter: int = 1000, seed: int = 0, device=None):
        if size < 4 or size > 256:
            raise ValueError("codebook size must be in [4, 256]")
        self.codebook = initial_codebook(rng, size)
        self.seed = seed
        if device is not None:
            self.iterations = self._train_device(device, gl, max_iter)
            return
        rr, het = _normalise(np.asarray(gl).reshape(-1, 3))
        P = rr.size
        rr64, het64 = rr.astype(np.float64), het.astype(np.float64)

        def assign(cbk):
            code = nearest_code(cbk, rr, het)
            dx = (rr - cbk[code, 0]).astype(np.float64)
            dy = (het - cbk[code, 1]).astype(np.float64)
            return code, ordered_sum(dx * dx + dy * dy)

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
            for k in range(size):
                if counts[k]:
                    member = code == k
                    new[k, 0] = F32(ordered_sum(np.where(member, rr64, 0.0)) / counts[k])
                    new[k, 1] = F32(ordered_sum(np.where(member, het64, 0.0)) / counts[k])
                else:
                    j = empty_point(seed, it, k, P)
                    new[k] = (rr[j], het[j])
            self.codebook = new
            code, cur = assign(self.codebook)
        self.iterations = it

    def _train_device(self, dev, gl, max_iter: int) -> int:
        import ctypes as C
        import torch
        g = gl if isinstance(gl, torch.Tensor) else torch.from_numpy(
            np.ascontiguousarray(np.asarray(gl, dtype=F32).reshape(-1, 3)))
        g = g.to(device="cuda", dtype=torch.float32).contiguous()
        torch.cuda.synchronize()
        cb = np.ascontiguousarray(self.codebook)
        iters = C.c_uint32(0)
        dev._c(dev.L.glp_vq_train(dev.ctx, g.data_ptr(), g.numel() // 3, cb.shape[0],
                                  cb.ctypes.data, self.seed, max_iter, C.byref(iters)))
        self.codebook = cb
        return int(iters.value)

    def find_code(self, rr, het):
        return nearest_code(self.codebook, np.asarray(rr, F32), np.asarray(het, F32))


def gl2halfchar(x: np.ndarray) -> np.ndarray:
    """GLPack::GL2HalfChar (glPack.cpp:232-243): floor(max(x - eps, 0) * 16)."""
    x = np.maximum(np.asarray(x, F32) - EPS32, F32(0.0)).astype(F32)
    return np.floor(x * F32(16)).astype(np.uint32)


class GLPack:
    """Packed GLs for the device (src/glPack.hpp:38-78)."""

    def __init__(self, gl: np.ndarray, rng: np.random.Generator | None = None,
                 use_vq: bool = True, bits: int = 4, seed: int = 0, device=None):
        """``device`` (an ``hmmlike.HMMLikeCUDA``): train the codebook and pack
        the codes on the GPU (``glp_vq_train`` / ``glp_vq_pack``), bit for bit
        the host result."""
        self.gl = np.ascontiguousarray(gl, dtype=F32)
        self.num_samps, self.num_sites = self.gl.shape[0], self.gl.shape[1]
        self.use_vq = use_vq
        self.bits = bits if use_vq else 8
        self.device = device if use_vq and 2 ** self.bits <= 16 else None
        if use_vq:
            if 8 % bits:
                raise ValueError("bits per GL must divide 8")
            self._gl_dev = None
            if self.device is not None:
                import torch
                self._gl_dev = torch.from_numpy(self.gl).cuda()
            self.vq = GLVQ(self.gl if self._gl_dev is None else self._gl_dev,
                           rng if rng is not None else np.random.default_rng(), 2 ** bits,
                           seed=seed, device=self.device)

    def code_book(self) -> np.ndarray:
        return self.vq.codebook.copy()

    def packed_gls(self) -> np.ndarray:
        """[ceil(S/8 or S/4)][N] uint32 (glPack.cpp:112-165)."""
        N, S = self.num_samps, self.num_sites
        per = 32 // self.bits
        nblk = (S + per - 1) // per
        if self.device is not None:
            import torch
            dev = self.device
            out = torch.zeros((nblk, N), dtype=torch.int32, device="cuda")
            cb = np.ascontiguousarray(self.vq.codebook, dtype=F32)
            torch.cuda.synchronize()
            dev._c(dev.L.glp_vq_pack(dev.ctx, self._gl_dev.data_ptr(), N, S, cb.ctypes.data,
                                     cb.shape[0], self.bits, out.data_ptr()))
            dev._c(dev.L.glp_finish(dev.ctx))
            return out.cpu().numpy().view(np.uint32)
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
