"""Host-side model set-up: the constants GLPhase's ``Insti::initialize`` hands
to the hot path (src/insti.cpp:1254-1380), restated with numpy in binary32 in
the reference's own order of operations.

Outputs feed the device API unchanged:

* ``tran``  float32 [S][3], row 0 unused (insti.cpp:1277-1300)
* ``pc``    float32 [4][4] mutation matrix (insti.cpp:1307-1315)
* ``t``     float32 [N][S][3] genotype probabilities (homRef, het, homAlt)
  (insti.cpp:1345-1350, stored as ``prob`` after insti.cpp:1382)
* ``emit``  float32 [N][S][4] (insti.cpp:1376-1378)
* initial haplotypes drawn from the GLs (insti.cpp:1353-1372), bit-packed
  hap-major, site m in word m>>6 bit m&63 (impute.hpp:53-66)
"""
from __future__ import annotations

import numpy as np

F32 = np.float32


def mutation_rate(num_haps: int) -> np.float32:
    """mu of insti.cpp:1254-1270: 1 / (sum_{i<hn} 1/i), then mu / (hn + mu).

    ``num_haps`` is hn = 2N before any panel is appended (insti.cpp:1205).
    The sum is kept in binary32 and each term is added in binary64 before
    rounding back, as ``fast mu; mu += 1.0 / i`` does.
    """
    mu = F32(0.0)
    for i in range(1, num_haps):
        mu = F32(float(mu) + 1.0 / i)
    mu = F32(F32(1.0) / mu)
    return mu


def finish_mutation_rate(mu_raw: np.float32, num_haps: int) -> np.float32:
    """``mu = mu / (hn + mu)`` (insti.cpp:1270), binary32."""
    return F32(mu_raw / F32(F32(num_haps) + mu_raw))


def mutation_matrix(mu: np.float32) -> np.ndarray:
    """pc[4][4] of insti.cpp:1307-1315: diagonal (1-mu)^2, one-off mu(1-mu),
    anti-diagonal mu^2."""
    one = F32(1.0)
    d = F32(F32(one - mu) * F32(one - mu))
    o = F32(mu * F32(one - mu))
    a = F32(mu * mu)
    pc = np.empty((4, 4), dtype=F32)
    pc[:] = o
    for i in range(4):
        pc[i, i] = d
        pc[i, 3 - i] = a
    return pc


def transition_from_distances(r_morgans: np.ndarray, inflation: float = 1.0) -> np.ndarray:
    """tran [S][3] from per-interval genetic distances (insti.cpp:1277-1300).

    ``r_morgans[m]`` is the distance between sites m-1 and m (entry 0
    ignored), as ``GeneticMap::GeneticDistance`` returns it
    (geneticMap.cpp:73-79).  r is rounded to binary32, inflated in binary64,
    clamped to 1, then ``(1-r)^2, r(1-r), r^2`` in binary32.
    """
    S = r_morgans.shape[0]
    r = np.asarray(r_morgans, dtype=np.float64).astype(F32)
    r = (r.astype(np.float64) * float(inflation)).astype(F32)
    r = np.minimum(r, F32(1.0))
    one = F32(1.0)
    tran = np.zeros((S, 3), dtype=F32)
    om = (one - r).astype(F32)
    tran[:, 0] = om * om
    tran[:, 1] = r * om
    tran[:, 2] = r * r
    tran[0, :] = 0
    return tran


def transition_from_positions(pos: np.ndarray, mu_raw: np.float32, num_haps: int,
                              density: float = 1.0) -> np.ndarray:
    """tran without a genetic map (insti.cpp:1262-1284): rho from the site
    density, then r = d*rho / (d*rho + hn) per interval, all binary32."""
    S = pos.shape[0]
    first, last = int(pos[0]), int(pos[-1])
    if last == first:
        rho = F32(0.0)
    else:
        rho = F32(0.5 * float(mu_raw) * (S - 1) / (last - first) / density)
    tran = np.zeros((S, 3), dtype=F32)
    one = F32(1.0)
    hn = F32(num_haps)
    for m in range(S - 1, 0, -1):
        tmp = F32(F32(int(pos[m]) - int(pos[m - 1])) * rho)
        r = F32(tmp / F32(tmp + hn))
        om = F32(one - r)
        tran[m] = (F32(om * om), F32(r * om), F32(r * r))
    return tran


def genotype_probs(gl_het_alt: np.ndarray) -> np.ndarray:
    """t = (max(1-het-alt,0), max(het,0), max(alt,0)) per sample and site
    (insti.cpp:1345-1350).  Input [N][S][2] (het, homAlt) as the .bin reader
    stores them (glReader.cpp:202-285); output [N][S][3] binary32."""
    p = np.asarray(gl_het_alt, dtype=F32)
    one = F32(1.0)
    t = np.empty(p.shape[:2] + (3,), dtype=F32)
    t[..., 0] = np.maximum((one - p[..., 0]) - p[..., 1], F32(0.0))
    t[..., 1] = np.maximum(p[..., 0], F32(0.0))
    t[..., 2] = np.maximum(p[..., 1], F32(0.0))
    return t


def emission(t: np.ndarray, pc: np.ndarray) -> np.ndarray:
    """emit[j] = pc[j][0] t0 + pc[j][1] t1 + pc[j][2] t1 + pc[j][3] t2,
    left to right in binary32 (insti.cpp:1376-1378)."""
    t = np.asarray(t, dtype=F32)
    e = np.empty(t.shape[:-1] + (4,), dtype=F32)
    for j in range(4):
        acc = (pc[j, 0] * t[..., 0]).astype(F32)
        acc = (acc + (pc[j, 1] * t[..., 1]).astype(F32)).astype(F32)
        acc = (acc + (pc[j, 2] * t[..., 1]).astype(F32)).astype(F32)
        acc = (acc + (pc[j, 3] * t[..., 2]).astype(F32)).astype(F32)
        e[..., j] = acc
    return e


def num_words(num_sites: int) -> int:
    """wn of insti.cpp:1204."""
    return (num_sites + 63) >> 6


def pack_haplotypes(bits: np.ndarray) -> np.ndarray:
    """Bit-pack [H][S] 0/1 alleles to uint64 [H][wn]: site m -> word m>>6,
    bit m&63 (impute.hpp:53-66, hapPanel.cpp:41-64)."""
    bits = np.asarray(bits, dtype=np.uint8)
    H, S = bits.shape
    wn = num_words(S)
    padded = np.zeros((H, wn * 64), dtype=np.uint8)
    padded[:, :S] = bits
    by = np.packbits(padded.reshape(H, wn, 8, 8), axis=-1, bitorder="little")
    return by.reshape(H, wn * 8).view("<u8").reshape(H, wn).copy()


def unpack_haplotypes(words: np.ndarray, num_sites: int) -> np.ndarray:
    """Inverse of :func:`pack_haplotypes`."""
    words = np.ascontiguousarray(words, dtype="<u8")
    H, wn = words.shape
    by = words.view(np.uint8).reshape(H, wn * 8)
    bits = np.unpackbits(by, axis=-1, bitorder="little")
    return bits[:, :num_sites].copy()


def initial_haplotypes(t: np.ndarray, rng: np.random.Generator) -> np.ndarray:
    """Random starting haplotypes drawn from the GLs (insti.cpp:1353-1372):
    hom-ref with probability t0, else het with probability t1/(t1+t2) (phase
    at random), else hom-alt.  Returns 0/1 alleles [2N][S]."""
    N, S, _ = t.shape
    u1 = rng.random((N, S))
    u2 = rng.random((N, S))
    u3 = rng.random((N, S))
    t0 = t[..., 0].astype(np.float64)
    t1 = t[..., 1].astype(np.float64)
    t2 = t[..., 2].astype(np.float64)
    with np.errstate(invalid="ignore", divide="ignore"):
        het_frac = t1 / (t1 + t2)
    homref = u1 < t0
    het = (~homref) & (u2 < het_frac)
    homalt = (~homref) & (~het)
    ha = (homalt | (het & (u3 < 0.5))).astype(np.uint8)
    hb = (homalt | (het & ~(u3 < 0.5))).astype(np.uint8)
    out = np.empty((2 * N, S), dtype=np.uint8)
    out[0::2] = ha
    out[1::2] = hb
    return out


class Model:
    """Everything ``Insti::initialize`` computes for the hot path."""

    def __init__(self, gl_het_alt: np.ndarray, r_morgans: np.ndarray | None = None,
                 positions: np.ndarray | None = None, inflation: float = 1.0,
                 density: float = 1.0):
        gl = np.asarray(gl_het_alt, dtype=F32)
        self.N, self.S = gl.shape[0], gl.shape[1]
        self.hn = 2 * self.N
        self.wn = num_words(self.S)
        mu_raw = mutation_rate(self.hn)
        if r_morgans is not None:
            self.tran = transition_from_distances(r_morgans, inflation)
        else:
            if positions is None:
                positions = np.arange(self.S)
            self.tran = transition_from_positions(positions, mu_raw, self.hn, density)
        self.mu = finish_mutation_rate(mu_raw, self.hn)
        self.pc = mutation_matrix(self.mu)
        self.t = genotype_probs(gl)
        self.emit = emission(self.t, self.pc)
