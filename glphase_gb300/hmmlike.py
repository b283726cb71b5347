"""Host-side mirror of the reference's device boundary.

* :class:`HMMLikeCUDA` -- the reference's device API (namespace HMMLikeCUDA,
  src/hmmLike.h:23-38) as methods over one C-ABI context.
* :class:`HMMLike` -- the reference's host driver (src/hmmLike.hpp:122-184,
  src/hmmLike.cpp): copies the model once, pre-draws the 4 initial and C
  proposal haplotypes per sample with the sampler, runs the device MH, and
  returns quadruples transposed to [sample][4].
* :class:`Engine` -- the device-resident generation loop used for
  throughput: haplotypes, quadruples, proposals and outputs stay in HBM and
  each generation is the generation kernel followed by the two hmm_work
  kernels on the same stream (Insti::cudaSolve, src/insti.cpp:1433-1463,
  without the host hmm_work loop).

Every call goes through the CUDA library; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native as nat


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def _check(L, ctx, rc):
    if rc != nat.GLP_OK:
        msg = L.glp_last_error(ctx)
        raise nat.GlpError(rc, msg.decode() if msg else "")


def transpose_hap_idxs(hap_idxs: np.ndarray) -> np.ndarray:
    """[4][N] -> [N][4] flat (HMMLikeHelper::transposeHapIdxs,
    src/hmmLike.cpp:6-22)."""
    h = np.asarray(hap_idxs, dtype=np.uint32).reshape(4, -1)
    return np.ascontiguousarray(h.T).reshape(-1)


class HMMLikeCUDA:
    """The reference's HMMLikeCUDA namespace over one device context."""

    def __init__(self, dev_id: int = 0):
        self.L = nat.load()
        self.ctx = C.c_void_p()
        self.check_device(dev_id)
        _check(self.L, None, self.L.glp_create(dev_id, C.byref(self.ctx)))

    def check_device(self, dev_id: int = 0) -> tuple[int, int, int]:
        n, ma, mi, sms = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        rc = self.L.glp_check_device(dev_id, C.byref(n), C.byref(ma), C.byref(mi), C.byref(sms))
        if rc != nat.GLP_OK:
            raise nat.GlpError(rc, f"device {dev_id}: {n.value} devices, cc "
                                   f"{ma.value}.{mi.value} (an sm_103 GPU is required)")
        return ma.value, mi.value, sms.value

    def _c(self, rc):
        _check(self.L, self.ctx, rc)

    def copy_tran_to_device(self, tran: np.ndarray) -> None:
        t = np.ascontiguousarray(tran, dtype=np.float32).reshape(-1, 3)
        self._c(self.L.glp_set_tran(self.ctx, _ptr(t), t.shape[0]))

    def copy_mutation_mat_to_device(self, pc: np.ndarray) -> None:
        p = np.ascontiguousarray(pc, dtype=np.float32).reshape(16)
        self._c(self.L.glp_set_mutation_mat(self.ctx, _ptr(p)))

    def copy_code_book_to_device(self, codebook) -> None:
        cb = np.ascontiguousarray(np.asarray(codebook, dtype=np.float32).reshape(-1, 2))
        self._c(self.L.glp_set_codebook(self.ctx, _ptr(cb), cb.shape[0]))

    def copy_packed_gls_to_device(self, packed: np.ndarray) -> None:
        p = np.ascontiguousarray(packed, dtype=np.uint32).reshape(-1)
        self._c(self.L.glp_set_packed_gls(self.ctx, _ptr(p), p.size))

    def copy_emission_to_device(self, emit: np.ndarray, prob: np.ndarray | None) -> None:
        e = np.ascontiguousarray(emit, dtype=np.float32)
        N, S = e.shape[0], e.shape[1]
        pr = None if prob is None else np.ascontiguousarray(prob, dtype=np.float32)
        self._c(self.L.glp_set_emission(self.ctx, _ptr(e), None if pr is None else _ptr(pr),
                                        N, S))

    def run_hmm_on_device(self, hap_panel: np.ndarray, extra_prop_haps: np.ndarray,
                          num_sites: int, num_samples: int, num_cycles: int,
                          hap_idxs: np.ndarray, seed: int) -> np.ndarray:
        """In/out hap_idxs [4][N]; returns the updated array."""
        panel = np.ascontiguousarray(hap_panel, dtype=np.uint64).reshape(-1)
        props = np.ascontiguousarray(extra_prop_haps, dtype=np.uint32).reshape(-1)
        out = np.ascontiguousarray(hap_idxs, dtype=np.uint32).reshape(-1).copy()
        self._c(self.L.glp_run_hmm_on_device(self.ctx, _ptr(panel), panel.size, _ptr(props),
                                             num_sites, num_samples, num_cycles, _ptr(out),
                                             seed))
        return out

    def set_lanes_per_sample(self, lanes: int) -> None:
        self._c(self.L.glp_set_lanes_per_sample(self.ctx, lanes))

    def set_evals_per_lane(self, evals: int) -> None:
        self._c(self.L.glp_set_evals_per_lane(self.ctx, evals))

    def set_block_sites(self, sites: int) -> None:
        """Sites per normalisation block: 8, 4, or 0 = automatic."""
        self._c(self.L.glp_set_block_sites(self.ctx, sites))

    def block_sites(self) -> int:
        """The normalisation block size the next launch uses."""
        v = C.c_uint32(0)
        self._c(self.L.glp_get_block_sites(self.ctx, C.byref(v)))
        return int(v.value)

    def counters(self) -> list[int]:
        """[evaluations, rounds, accepts, site-by-site redos, warp rounds,
        active lanes over warp rounds] of the last generation."""
        buf = (C.c_uint64 * 6)()
        self._c(self.L.glp_get_counters(self.ctx, buf, 6))
        return list(buf)

    def kernel_times(self, n: int) -> tuple[list[float], list[float]]:
        """Device ms of the generation kernel and of hmm_work for the last n
        generations launched from this context."""
        g, w = (C.c_float * n)(), (C.c_float * n)()
        self._c(self.L.glp_kernel_times(self.ctx, n, g, w))
        return list(g), list(w)

    def stats(self) -> tuple[int, int, int]:
        ev, rd, ln = C.c_uint64(), C.c_uint64(), C.c_uint32()
        self._c(self.L.glp_get_stats(self.ctx, C.byref(ev), C.byref(rd), C.byref(ln)))
        return ev.value, rd.value, ln.value

    def cleanup(self) -> None:
        if self.ctx:
            self.L.glp_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.cleanup()
        except Exception:
            pass


class HMMLike:
    """Mirror of the reference's HMMLike host driver (src/hmmLike.cpp:32-111).

    ``gl_pack`` provides ``packed_gls()`` ([ceil(S/8)][N] uint32),
    ``code_book()`` ([16][2]), ``num_sites`` and ``num_samps``; ``sampler``
    provides ``sample_hap(sample) -> int``; ``rng`` is a numpy Generator
    standing in for the gsl_rng that seeds each device call.
    """

    def __init__(self, hap_panel: np.ndarray, num_haps: int, gl_pack, num_cycles: int,
                 tran: np.ndarray, mutation_mat: np.ndarray, sampler, rng, dev_id: int = 0):
        assert num_cycles > 0
        self.hap_panel = hap_panel
        self.num_haps = num_haps
        self.gl_pack = gl_pack
        self.num_cycles = num_cycles
        self.sampler = sampler
        self.rng = rng
        self.dev = HMMLikeCUDA(dev_id)
        self.dev.copy_tran_to_device(tran)
        self.dev.copy_mutation_mat_to_device(mutation_mat)
        self.dev.copy_code_book_to_device(gl_pack.code_book())
        self.dev.copy_packed_gls_to_device(gl_pack.packed_gls())

    def update_sampler(self, sampler) -> None:
        if sampler is None:
            raise RuntimeError("HMMLike::UpdateSampler was called with null pointer")
        self.sampler = sampler

    def run_hmm_on_samples(self):
        """Returns (first_samp_idx, last_samp_idx, hap_idxs [N*4])."""
        N = self.gl_pack.num_samps
        hap_idxs = np.zeros((4, N), dtype=np.uint32)
        props = np.zeros((self.num_cycles, N), dtype=np.uint32)
        for s in range(N):
            for j in range(4):
                hap_idxs[j, s] = self.sampler.sample_hap(s)
            for c in range(self.num_cycles):
                props[c, s] = self.sampler.sample_hap(s)
        seed = int(self.rng.integers(0, 2**63))
        out = self.dev.run_hmm_on_device(self.hap_panel, props, self.gl_pack.num_sites, N,
                                         self.num_cycles, hap_idxs, seed)
        return 0, N - 1, transpose_hap_idxs(out)


class UnifSampler:
    """Uniform proposal over all haplotypes except the sample's own
    (UnifSampler::SampleHap, src/sampler.cpp:29-39)."""

    def __init__(self, rng, num_samples: int, num_haps: int):
        assert 2 * num_samples <= num_haps
        self.rng, self.num_samples, self.num_haps = rng, num_samples, num_haps

    def sample_hap(self, exclude_ind: int, only_from_ref: bool = False) -> int:
        while True:
            h = int(self.rng.integers(0, self.num_haps))
            if h // 2 == exclude_ind:
                continue
            if only_from_ref and h < 2 * self.num_samples:
                continue
            return h


class Engine:
    """Device-resident MH generations (torch tensors as device memory)."""

    def __init__(self, emit: np.ndarray, prob: np.ndarray, tran: np.ndarray, pc: np.ndarray,
                 haps: np.ndarray, num_cycles: int, device: int = 0, lanes: int = 0,
                 packed: np.ndarray | None = None, codebook: np.ndarray | None = None,
                 evals: int = 0, block_sites: int = 0):
        import torch
        self.torch = torch
        self.dev = HMMLikeCUDA(device)
        self.device = torch.device("cuda", device)
        self.N, self.S = emit.shape[0], emit.shape[1]
        self.H, self.wn = haps.shape
        self.C = num_cycles
        self.dev.copy_tran_to_device(tran)
        self.dev.copy_mutation_mat_to_device(pc)
        self.dev.copy_emission_to_device(emit, prob)
        self.vq = packed is not None
        if self.vq:
            self.dev.copy_code_book_to_device(codebook)
            self.dev.copy_packed_gls_to_device(packed)
        self.dev.set_lanes_per_sample(lanes)
        self.dev.set_evals_per_lane(evals)
        self.dev.set_block_sites(block_sites)
        h = torch.from_numpy(np.ascontiguousarray(haps).view(np.int64))
        self.haps = h.to(self.device)
        self.hnew = self.haps.clone()
        self.quad = torch.zeros((4, self.N), dtype=torch.int32, device=self.device)
        self.like = torch.zeros(self.N, dtype=torch.float64, device=self.device)
        # a dedicated stream: the legacy default stream has handle 0, which the
        # C ABI reads as "the context's own stream"
        self.stream = torch.cuda.Stream(self.device)
        torch.cuda.current_stream(self.device).synchronize()
        self.dev._c(self.dev.L.glp_set_stream(self.dev.ctx, self.stream.cuda_stream))

    def knn(self, k: int, freq_lb: float = 0.0, freq_ub: float = 1.0, use_maf: bool = False,
            metric: str = "hamming"):
        """Neighbour table of the current haplotypes on the device
        (KNN::ClusterHaps, kNN.cpp:123-206); kept for the in-kernel draws.
        metric "hamming" or "tract" (the common sites minus the longest shared
        tract, insti -T).  Returns the engine's table, which the next call
        rewrites in place (copy it to keep an old one)."""
        torch = self.torch
        half = (k + 1) // 2
        self.dev._c(self.dev.L.glp_set_knn_metric(self.dev.ctx, nat.KNN_METRICS[metric]))
        shape = (self.H // 2, 2 * half)
        # A rebuild writes into the same table on the engine's stream, after
        # the generations already enqueued there have read it.  (A new tensor
        # would come from torch's allocator on its current stream, unordered
        # with the engine's: its memory could be the old table's while a
        # generation still reads it.)
        if getattr(self, "nbr", None) is None or tuple(self.nbr.shape) != shape:
            with torch.cuda.stream(self.stream):
                self.nbr = torch.empty(shape, dtype=torch.int32, device=self.device)
        self.dev._c(self.dev.L.glp_knn_neighbors(self.dev.ctx, self.haps.data_ptr(), self.H,
                                                 self.S, k, freq_lb, freq_ub, int(use_maf),
                                                 self.nbr.data_ptr()))
        return self.nbr

    def args(self, quad_in, props, pen: float, seed: int, generation: int, work: bool = True,
             eval_trace=None, accept_trace=None, neighbors=None,
             kick_first: bool = False) -> nat.GenerationArgs:
        """quad_in / props None: drawn in the kernel (from `neighbors` when
        given, else uniformly over all other haplotypes); kick_first: every
        chain's first proposal from the panel rows (the reference's
        --kickstart)."""
        a = nat.GenerationArgs()
        a.num_samples, a.num_sites, a.num_cycles, a.num_haps = self.N, self.S, self.C, self.H
        a.haps = self.haps.data_ptr()
        a.hnew = self.hnew.data_ptr()
        a.hap_idxs_in = None if quad_in is None else quad_in.data_ptr()
        a.hap_idxs_out = self.quad.data_ptr()
        a.props = None if props is None else props.data_ptr()
        if neighbors is not None:
            a.neighbors, a.neighbors_per_sample = neighbors.data_ptr(), neighbors.shape[1]
        a.pen = pen
        a.seed = seed
        a.generation = generation
        a.flags = ((nat.GLP_GEN_VQ if self.vq else 0) | (0 if work else nat.GLP_GEN_NO_WORK) |
                   (nat.GLP_GEN_KICK_FIRST if kick_first else 0))
        a.like_out = self.like.data_ptr()
        a.eval_trace = None if eval_trace is None else eval_trace.data_ptr()
        a.accept_trace = None if accept_trace is None else accept_trace.data_ptr()
        return a

    def launch(self, a: nat.GenerationArgs) -> None:
        self.dev._c(self.dev.L.glp_run_generation(self.dev.ctx, C.byref(a)))

    def finish(self) -> None:
        self.dev._c(self.dev.L.glp_finish(self.dev.ctx))

    def swap(self) -> None:
        """hnew becomes the current haplotypes (Insti::cudaSolve swap,
        src/insti.cpp:1455); panel rows are identical in both buffers."""
        self.haps, self.hnew = self.hnew, self.haps

    def run_host(self, haps: np.ndarray, quad, props, pen: float,
                 seed: int, generation: int, hnew: np.ndarray, quad_out: np.ndarray,
                 like_out: np.ndarray | None = None, neighbors: np.ndarray | None = None) -> None:
        """The same generation through the host-pointer entry point (quad /
        props None: drawn in the kernel, from `neighbors` when given)."""
        a = nat.GenerationArgs()
        a.num_samples, a.num_sites, a.num_cycles, a.num_haps = self.N, self.S, self.C, self.H
        a.haps, a.hnew = _ptr(haps), _ptr(hnew)
        a.hap_idxs_in = None if quad is None else _ptr(quad)
        a.hap_idxs_out = _ptr(quad_out)
        a.props = None if props is None else _ptr(props)
        if neighbors is not None:
            a.neighbors, a.neighbors_per_sample = _ptr(neighbors), neighbors.shape[1]
        a.pen, a.seed, a.generation = pen, seed, generation
        a.flags = nat.GLP_GEN_VQ if self.vq else 0
        a.like_out = None if like_out is None else _ptr(like_out)
        self.dev._c(self.dev.L.glp_run_generation_host(self.dev.ctx, C.byref(a)))
