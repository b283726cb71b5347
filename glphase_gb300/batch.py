"""Uneven chunks on one GPU: device-resident problems, one persistent launch
per generation for all of them (glp_run_batch / glp_batch_*), and the
"plain" form that launches each chunk on its own, for comparison.

Each chunk is an independent phasing problem (its own samples, sites, map,
founders and seed); its surrogates are drawn on the device.  A prepared
batch advances every chunk on the device after each generation (haplotype
swap, generation counter, annealing penalty), so generation after
generation replays one captured CUDA graph.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native as nat
from .hmmlike import HMMLikeCUDA


def anneal_pen(generation: int, burnin: int) -> np.float32:
    """pen = min((g + 1) / B, 1)^2 in binary32 (Insti::estimate,
    src/insti.cpp:1670-1671); 1 without burn-in."""
    if not burnin:
        return np.float32(1.0)
    x = np.float32(np.float32(generation + 1.0) / np.float32(burnin))
    x = min(x, np.float32(1.0))
    return np.float32(x * x)


class DeviceProblem:
    """One chunk: model inputs borrowed from device arrays (torch), current
    and new haplotype buffers, outputs."""

    def __init__(self, dev: HMMLikeCUDA, chunk, cycles: int, seed: int, burnin: int,
                 kick_start: bool = False, vq=None):
        import torch
        self.dev = dev
        self.chunk = chunk
        self.N, self.S, self.H, self.C = chunk.N, chunk.S, chunk.H, cycles
        self.seed, self.burnin = seed, burnin
        self.kick_start = kick_start
        self.pb = C.c_void_p()
        dev._c(dev.L.glp_problem_create(dev.ctx, C.byref(self.pb)))
        tran = np.ascontiguousarray(chunk.tran, dtype=np.float32)
        pc = np.ascontiguousarray(chunk.pc, dtype=np.float32)
        dev._c(dev.L.glp_problem_set_model_device(self.pb, tran.ctypes.data, pc.ctypes.data,
                                                  chunk.emit.data_ptr(), chunk.prob.data_ptr(),
                                                  self.N, self.S))
        # vq = (packed [ceil(S/8)][N] uint32, codebook [16][2] float32): the
        # 4-bit GL codes replace the float emission (GLP_GEN_VQ)
        self.flags = 0
        if vq is not None:
            packed = np.ascontiguousarray(vq[0], dtype=np.uint32)
            cb = np.ascontiguousarray(vq[1], dtype=np.float32)
            dev._c(dev.L.glp_problem_set_vq(self.pb, packed.ctypes.data, packed.size,
                                            cb.ctypes.data))
            self.flags = nat.GLP_GEN_VQ
        self.haps = chunk.haps
        self.hnew = chunk.haps.clone()
        self.quad = torch.zeros((4, self.N), dtype=torch.int32, device=chunk.haps.device)
        self.like = torch.zeros(self.N, dtype=torch.float64, device=chunk.haps.device)

    def args(self, generation: int) -> nat.GenerationArgs:
        a = nat.GenerationArgs()
        a.num_samples, a.num_sites, a.num_cycles, a.num_haps = self.N, self.S, self.C, self.H
        a.haps, a.hnew = self.haps.data_ptr(), self.hnew.data_ptr()
        a.hap_idxs_out, a.like_out = self.quad.data_ptr(), self.like.data_ptr()
        a.pen = float(anneal_pen(generation, self.burnin))
        a.seed, a.generation, a.burnin = self.seed, generation, self.burnin
        a.flags = self.flags
        if self.kick_start and generation == 0:
            a.sample_lo, a.sample_hi, a.kick_start = 2 * self.N, self.H, 1
        return a

    def swap(self):
        self.haps, self.hnew = self.hnew, self.haps

    def footprint(self) -> int:
        """Device bytes this chunk holds: emission, genotype probabilities,
        hmm_work scratch and two haplotype buffers."""
        return self.N * self.S * (16 + 12 + 16) + 2 * self.H * ((self.S + 63) // 64) * 8

    def close(self):
        if self.pb:
            self.dev.L.glp_problem_destroy(self.pb)
            self.pb = C.c_void_p()


def run_batch(dev: HMMLikeCUDA, problems, generation: int) -> None:
    """One generation of every problem in one persistent launch (host-side
    descriptors); swaps each problem's haplotype buffers afterwards."""
    n = len(problems)
    args = (nat.GenerationArgs * n)(*[p.args(generation) for p in problems])
    pbs = (C.c_void_p * n)(*[p.pb for p in problems])
    dev._c(dev.L.glp_run_batch(dev.ctx, n, pbs, args))
    for p in problems:
        p.swap()


class PreparedBatch:
    """Device-resident descriptors + a captured CUDA graph per generation."""

    def __init__(self, dev: HMMLikeCUDA, problems, generation: int = 0):
        self.dev = dev
        self.problems = problems
        n = len(problems)
        args = (nat.GenerationArgs * n)(*[p.args(generation) for p in problems])
        pbs = (C.c_void_p * n)(*[p.pb for p in problems])
        self.b = C.c_void_p()
        dev._c(dev.L.glp_batch_prepare(dev.ctx, n, pbs, args, C.byref(self.b)))
        self.generation = generation

    def run(self, graph: bool = True) -> None:
        fn = self.dev.L.glp_batch_run if graph else self.dev.L.glp_batch_launch
        self.dev._c(fn(self.b))
        self.generation += 1
        for p in self.problems:   # the device swapped its descriptors
            p.swap()

    def close(self):
        if self.b:
            self.dev.L.glp_batch_destroy(self.b)
            self.b = C.c_void_p()
