"""Seeded synthetic phasing workloads with the shapes and value distributions
of the reference's benchmark configurations (no dataset records are used).

The generator mirrors the reference's own simulator idea
(samples/hapGen/generateGLs.R: Poisson coverage, binomial reads): founders
with allele frequencies ~ Beta(0.5, 0.5); truth haplotypes are Li-Stephens
mosaics of the founders with a per-site switch probability; genotype
likelihoods come from read depth ~ Poisson(lambda) and alt reads ~
Binomial(depth, p_g), p_g in {err, 0.5, 1-err}, normalised to (homRef, het,
homAlt); sites every 200 bp on a uniform 1 cM/Mb map, so neighbouring sites
are 2e-6 Morgans apart.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import model as mdl


@dataclass
class Workload:
    name: str
    N: int                 # GL samples
    S: int                 # sites
    founders: int
    depth: float
    burnin: int            # SA burn-in generations (-B)
    sampling: int          # sampling generations (-m)
    cycles: int = 100      # MH cycles per sample per generation (-C)
    panel_haps: int = 0    # reference-panel haplotypes appended after 2N
    knn: int = 0           # kNN surrogate restriction (0 = uniform sampler)
    seed: int = 1
    switch_rate: float = 1e-3
    base_error: float = 0.01
    site_spacing_bp: int = 200
    cm_per_mb: float = 1.0

    @property
    def generations(self) -> int:
        return self.burnin + self.sampling


# The five workloads of the benchmark, by shape.
CONFIGS = {
    "plain": Workload("plain", N=256, S=1024, founders=40, depth=4.0, burnin=8,
                      sampling=16, seed=11),
    "batched": Workload("batched", N=10000, S=4096, founders=80, depth=2.0,
                        burnin=8, sampling=24, knn=200, seed=12),
    "panel": Workload("panel", N=2000, S=8192, founders=80, depth=4.0, burnin=8,
                      sampling=24, panel_haps=10000, seed=13),
}


@dataclass
class Dataset:
    workload: Workload
    truth: np.ndarray        # [2N + panel][S] 0/1 alleles (panel rows are the panel)
    gl: np.ndarray           # [N][S][3] normalised (homRef, het, homAlt) float32
    r_morgans: np.ndarray    # [S] distance to the previous site (entry 0 = 0)

    @property
    def gl_het_alt(self) -> np.ndarray:
        """[N][S][2] (het, homAlt): what the .bin reader keeps
        (glReader.cpp:202-285)."""
        return self.gl[..., 1:3]


def _mosaic(founders: np.ndarray, n: int, switch: float, rng) -> np.ndarray:
    F, S = founders.shape
    switches = rng.random((n, S)) < switch
    switches[:, 0] = True
    draws = rng.integers(0, F, size=(n, S))
    # index of the last switch at or before each site
    idx = np.where(switches, np.arange(S)[None, :], 0)
    np.maximum.accumulate(idx, axis=1, out=idx)
    src = np.take_along_axis(draws, idx, axis=1)
    return founders[src, np.arange(S)[None, :]]


def _binom_pmf(k: np.ndarray, n: np.ndarray, p: float) -> np.ndarray:
    from scipy.special import gammaln
    logc = gammaln(n + 1) - gammaln(k + 1) - gammaln(n - k + 1)
    return np.exp(logc + k * np.log(p) + (n - k) * np.log1p(-p))


def generate(w: Workload, N: int | None = None, S: int | None = None,
             seed: int | None = None) -> Dataset:
    """Generate a workload (optionally at a reduced N or S for tests)."""
    N = w.N if N is None else N
    S = w.S if S is None else S
    rng = np.random.default_rng(w.seed if seed is None else seed)
    freq = rng.beta(0.5, 0.5, size=S)
    founders = (rng.random((w.founders, S)) < freq[None, :]).astype(np.uint8)
    truth = _mosaic(founders, 2 * N + w.panel_haps, w.switch_rate, rng)
    g = truth[0:2 * N:2].astype(np.int64) + truth[1:2 * N:2]
    depth = rng.poisson(w.depth, size=(N, S))
    palt = np.array([w.base_error, 0.5, 1.0 - w.base_error])[g]
    alt = rng.binomial(depth, palt)
    # GL triple per (depth, alt) pair: binomial pmf per genotype, normalised
    dmax = int(depth.max())
    dd, aa = np.meshgrid(np.arange(dmax + 1), np.arange(dmax + 1), indexing="ij")
    tab = np.stack([_binom_pmf(np.minimum(aa, dd), dd, p)
                    for p in (w.base_error, 0.5, 1.0 - w.base_error)], axis=-1)
    tab /= tab.sum(axis=-1, keepdims=True)
    gl = tab.astype(np.float32)[depth, alt]
    r = np.full(S, w.site_spacing_bp * w.cm_per_mb * 1e-8, dtype=np.float64)
    r[0] = 0.0
    return Dataset(w, truth, gl, r)


def initial_state(ds: Dataset, seed: int = 7):
    """Model constants plus starting haplotypes for a dataset: returns
    (model, haps uint64 [H][wn]) with H = 2N + panel haplotypes; panel rows
    are the bit-packed panel (insti.cpp:1395-1403)."""
    m = mdl.Model(ds.gl_het_alt, r_morgans=ds.r_morgans)
    rng = np.random.default_rng(seed)
    init = mdl.initial_haplotypes(m.t, rng)
    N = m.N
    if ds.workload.panel_haps:
        allbits = np.concatenate([init, ds.truth[2 * N:]], axis=0)
    else:
        allbits = init
    return m, mdl.pack_haplotypes(allbits)


def uniform_proposals(N: int, H: int, C: int, rng: np.random.Generator,
                      only_panel_from: int | None = None) -> tuple[np.ndarray, np.ndarray]:
    """Host draw of the 4 initial parents and C proposals per sample, uniform
    over all haplotypes except the sample's own (UnifSampler::SampleHap,
    sampler.cpp:29-39; RunHMMOnSamples, hmmLike.cpp:90-102).  Returns
    (hap_idxs [4][N], props [C][N]) uint32."""
    def draw(shape):
        own = np.arange(N, dtype=np.int64)
        # uniform over H-2 haps that are not 2i or 2i+1
        x = rng.integers(0, H - 2, size=shape)
        lo = 2 * own
        x = np.where(x >= lo[None, :] if x.ndim == 2 else x >= lo, x + 2, x)
        return x.astype(np.uint32)
    quad = draw((4, N))
    props = draw((C, N))
    if only_panel_from is not None:
        span = H - only_panel_from
        props[0] = (only_panel_from + rng.integers(0, span, size=N)).astype(np.uint32)
    return quad, props
