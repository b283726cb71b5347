"""Device-side generation of large synthetic workloads (the uneven-chunk and
serving configurations hold up to ~1e9 site-samples, too many for the numpy
generator within a benchmark's minutes).  Same model as
:mod:`glphase_gb300.synth`: Beta(0.5, 0.5) allele frequencies, Li-Stephens
mosaics of founders, Poisson depth, binomial reads, normalised GLs; then the
model constants of ``Insti::initialize`` (src/insti.cpp:1254-1380) with the
emission computed on the device in the reference's binary32 operation order
(one elementwise op at a time, no contraction).  torch is plumbing here: the
arrays it produces are handed to the CUDA library by pointer.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import model as mdl
from .synth import Workload


@dataclass
class DeviceChunk:
    N: int
    S: int
    H: int
    wn: int
    emit: "object"      # torch float32 [N][S][4]
    prob: "object"      # torch float32 [N][S][3]
    haps: "object"      # torch int64 [H][wn], bit-packed
    tran: np.ndarray    # [S][3] float32 (host)
    pc: np.ndarray      # [4][4] float32 (host)

    @property
    def nbytes(self) -> int:
        return self.N * self.S * (16 + 12) + 2 * self.H * self.wn * 8


def pack_bits_device(bits):
    """[H][S] uint8 0/1 -> int64 [H][wn]: site m in word m>>6, bit m&63
    (impute.hpp:53-66), via little-endian bytes."""
    import torch
    H, S = bits.shape
    wn = (S + 63) // 64
    pad = torch.zeros((H, wn * 64), dtype=torch.uint8, device=bits.device)
    pad[:, :S] = bits
    w = (1 << torch.arange(8, device=bits.device, dtype=torch.int32)).to(torch.uint8)
    by = (pad.view(H, wn * 8, 8) * w).sum(dim=-1, dtype=torch.int32).to(torch.uint8)
    return by.contiguous().view(torch.int64).view(H, wn)


def generate(w: Workload, N: int, S: int, seed: int, device="cuda") -> DeviceChunk:
    import torch
    rng = np.random.default_rng(seed)
    freq = rng.beta(0.5, 0.5, size=S)
    founders = (rng.random((w.founders, S)) < freq[None, :]).astype(np.uint8)
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    dev = torch.device(device)
    fd = torch.from_numpy(founders).to(dev)
    n = 2 * N + w.panel_haps
    col = torch.arange(S, device=dev)
    switches = torch.rand((n, S), generator=g, device=dev) < w.switch_rate
    switches[:, 0] = True
    draws = torch.randint(0, w.founders, (n, S), generator=g, device=dev)
    idx = torch.where(switches, col[None, :], torch.zeros_like(col)[None, :])
    idx = torch.cummax(idx, dim=1).values
    src = torch.gather(draws, 1, idx)
    del switches, draws, idx
    truth = fd[src, col[None, :]]
    del src
    gt = (truth[0:2 * N:2].to(torch.int64) + truth[1:2 * N:2].to(torch.int64))
    depth = torch.poisson(torch.full((N, S), float(w.depth), device=dev), generator=g)
    palt = torch.tensor([w.base_error, 0.5, 1.0 - w.base_error], device=dev)[gt]
    alt = torch.binomial(depth, palt, generator=g)
    dmax = int(depth.max().item())
    from .synth import _binom_pmf
    dd, aa = np.meshgrid(np.arange(dmax + 1), np.arange(dmax + 1), indexing="ij")
    tab = np.stack([_binom_pmf(np.minimum(aa, dd), dd, p)
                    for p in (w.base_error, 0.5, 1.0 - w.base_error)], axis=-1)
    tab /= tab.sum(axis=-1, keepdims=True)
    tabd = torch.from_numpy(tab.astype(np.float32)).to(dev)
    gl = tabd[depth.long(), alt.long()]            # [N][S][3] float32
    del depth, alt, gt
    # genotype probabilities t (insti.cpp:1345-1350), binary32
    one = torch.tensor(1.0, dtype=torch.float32, device=dev)
    zero = torch.tensor(0.0, dtype=torch.float32, device=dev)
    het, homalt = gl[..., 1], gl[..., 2]
    t = torch.empty((N, S, 3), dtype=torch.float32, device=dev)
    t[..., 0] = torch.maximum((one - het) - homalt, zero)
    t[..., 1] = torch.maximum(het, zero)
    t[..., 2] = torch.maximum(homalt, zero)
    del gl, het, homalt
    hn = 2 * N
    mu = mdl.finish_mutation_rate(mdl.mutation_rate(hn), hn)
    pc = mdl.mutation_matrix(mu)
    r = np.full(S, w.site_spacing_bp * w.cm_per_mb * 1e-8)
    r[0] = 0
    tran = mdl.transition_from_distances(r)
    emit = torch.empty((N, S, 4), dtype=torch.float32, device=dev)
    for j in range(4):   # insti.cpp:1376-1378, left to right
        acc = t[..., 0] * float(pc[j, 0])
        acc = acc + t[..., 1] * float(pc[j, 1])
        acc = acc + t[..., 1] * float(pc[j, 2])
        acc = acc + t[..., 2] * float(pc[j, 3])
        emit[..., j] = acc
    # initial haplotypes from the GLs (insti.cpp:1353-1372)
    u1 = torch.rand((N, S), generator=g, device=dev)
    u2 = torch.rand((N, S), generator=g, device=dev)
    u3 = torch.rand((N, S), generator=g, device=dev)
    t1, t2 = t[..., 1], t[..., 2]
    homref = u1 < t[..., 0]
    het_call = (~homref) & (u2 * (t1 + t2) < t1)
    homalt_call = (~homref) & (~het_call)
    bits = torch.empty((n, S), dtype=torch.uint8, device=dev)
    bits[0:2 * N:2] = (homalt_call | (het_call & (u3 < 0.5))).to(torch.uint8)
    bits[1:2 * N:2] = (homalt_call | (het_call & (u3 >= 0.5))).to(torch.uint8)
    if w.panel_haps:
        bits[2 * N:] = truth[2 * N:]
    del truth, u1, u2, u3
    haps = pack_bits_device(bits)
    del bits
    return DeviceChunk(N=N, S=S, H=n, wn=(S + 63) // 64, emit=emit.contiguous(),
                       prob=t.contiguous(), haps=haps, tran=tran, pc=pc)
