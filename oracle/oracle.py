"""ctypes bindings to the CPU oracle (oracle/libglp_oracle.so) and, where they
were built, to the reference's own impute.cpp (oracle/_ref/libglp_ref.so),
kNN surrogate restriction (oracle/_ref/libglp_ref_knn.so), GL packing
(oracle/_ref/libglp_ref_glpack.so) and genetic map (oracle/_ref/libglp_ref_map.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by the CPU-baseline leg of bench.py, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libglp_oracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libglp_ref.so")
REF_KNN_PATH = os.path.join(HERE, "_ref", "libglp_ref_knn.so")
REF_GLPACK_PATH = os.path.join(HERE, "_ref", "libglp_ref_glpack.so")
REF_MAP_PATH = os.path.join(HERE, "_ref", "libglp_ref_map.so")
REF_TREE = "/root/reference"

EMIT_FLOAT = 0
EMIT_VQ = 1

_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")


def build(ref: bool | None = None) -> None:
    """Compile the oracle (and the reference build when the tree exists)."""
    subprocess.run(["make", "-s", "-C", HERE, "libglp_oracle.so"], check=True)
    if ref is None:
        ref = os.path.isdir(os.path.join(REF_TREE, "src"))
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_TREE}"], check=True)


class Problem(C.Structure):
    _fields_ = [("N", C.c_uint32), ("S", C.c_uint32), ("C", C.c_uint32),
                ("H", C.c_uint32), ("wn", C.c_uint32),
                ("haps", C.c_void_p), ("emit", C.c_void_p), ("prob", C.c_void_p),
                ("tran", C.c_void_p), ("pc", C.c_void_p), ("packed", C.c_void_p),
                ("codebook", C.c_void_p), ("emit_mode", C.c_int)]


class Trace(C.Structure):
    _fields_ = [("slot", C.c_void_p), ("u_mh", C.c_void_p), ("u_work", C.c_void_p),
                ("seed", C.c_uint64), ("generation", C.c_uint32)]


_lib = None
_ref = None
_ref_knn = None
_ref_glpack = None
_ref_map = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(ref=False)
        L = C.CDLL(LIB_PATH)
        L.glpo_norm.restype = C.c_float
        L.glpo_hmm_like_f32.restype = C.c_float
        L.glpo_hmm_like_f32.argtypes = [_f32p, _f32p, _u64p, C.c_uint32, C.c_uint32, _u32p]
        L.glpo_hmm_like_f64.restype = C.c_double
        L.glpo_hmm_like_f64.argtypes = [_f32p, _f32p, _u64p, C.c_uint32, C.c_uint32, _u32p]
        L.glpo_unpack_gl_codebook.argtypes = [C.c_uint32, _f32p, C.c_uint32, _f32p]
        L.glpo_fill_emit.argtypes = [_f32p, _f32p, _f32p]
        L.glpo_mutation_to_device_layout.argtypes = [_f32p, _f32p]
        L.glpo_hmm_like_vq.restype = C.c_float
        L.glpo_hmm_like_vq.argtypes = [_u32p, C.c_uint32, C.c_uint32, _f32p, _f32p, _f32p,
                                       _u64p, C.c_uint32, C.c_uint32, _u32p]
        L.glpo_hmm_work.argtypes = [_f32p, _f32p, _f32p, _f32p, _u64p, C.c_uint32,
                                    C.c_uint32, _u32p, C.c_float, _f32p, _u64p, _u64p, _f32p]
        L.glpo_mh_accept.restype = C.c_int
        L.glpo_mh_accept.argtypes = [C.c_double, C.c_double, C.c_double, C.c_double]
        L.glpo_solve_sample.restype = C.c_double
        L.glpo_solve_sample.argtypes = [C.POINTER(Problem), C.POINTER(Trace), C.c_uint32,
                                        _u32p, _u32p, C.c_float, _u32p, C.c_void_p,
                                        C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                        C.c_void_p]
        L.glpo_generation.restype = C.c_int
        L.glpo_generation.argtypes = [C.POINTER(Problem), C.POINTER(Trace), _u32p, _u32p,
                                      C.c_float, C.c_uint32, C.c_uint32, C.c_int, _u32p,
                                      _u64p, C.c_void_p, C.c_int]
        L.glpo_replay_sample.argtypes = [C.POINTER(Problem), C.POINTER(Trace), C.c_uint32,
                                         _u32p, _u32p, C.c_float, _u8p, _f32p, _f64p, _u8p,
                                         _u32p]
        L.glpo_mh_draws.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, _u8p, _f64p]
        L.glpo_work_uniforms.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, _f32p]
        L.glpo_sample_surrogates.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32,
                                             C.c_uint32, C.c_uint32, C.c_void_p, C.c_uint32,
                                             C.c_int, C.c_uint32, _u32p, _u32p]
        L.glpo_common_sites.argtypes = [_u64p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_double,
                                        C.c_double, C.c_int, _u64p]
        L.glpo_knn.restype = C.c_int
        L.glpo_knn.argtypes = [_u64p, C.c_uint32, C.c_uint32, _u64p, C.c_uint32, _u32p]
        L.glpo_knn_metric.restype = C.c_int
        L.glpo_knn_metric.argtypes = [_u64p, C.c_uint32, C.c_uint32, _u64p, C.c_uint32,
                                      C.c_int, _u32p]
        L.glpo_max_tract.restype = C.c_uint32
        L.glpo_max_tract.argtypes = [_u64p, _u64p, _u64p, C.c_uint32]
        L.glpo_replace.argtypes = [_u64p, C.c_uint32, C.c_uint32, C.c_uint32, _u32p]
        L.glpo_result.argtypes = [_u32p, C.c_uint32, C.c_uint32, C.c_uint32, _f32p]
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def ref():
    """The reference's own impute.cpp (built by ``make -C oracle ref``)."""
    global _ref
    if _ref is None:
        R = C.CDLL(REF_PATH)
        R.glpr_hmm_like.restype = C.c_float
        R.glpr_hmm_like.argtypes = [_f32p, _f32p, _u64p, C.c_uint32, C.c_uint32, C.c_uint32,
                                    _u32p]
        R.glpr_hmm_work.argtypes = [_f32p, _f32p, _f32p, _f32p, _u64p, C.c_uint32, C.c_uint32,
                                    C.c_uint32, _u32p, C.c_float, _f32p, _u64p, _u64p]
        R.glpr_initialize.argtypes = [_f32p, _f64p, C.c_uint32, C.c_uint32, C.c_double, _f32p,
                                      _f32p, _f32p, _f32p]
        R.glpr_replace.argtypes = [_u64p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, _u32p]
        R.glpr_result.argtypes = [_u32p, C.c_uint32, C.c_uint32, C.c_uint32, _f32p]
        R.glpr_mh_chain.argtypes = [_f64p, C.c_uint32, C.c_double, _f64p, C.c_uint32, _u8p,
                                    _u32p]
        _ref = R
    return _ref


def ref_knn_available() -> bool:
    return os.path.exists(REF_KNN_PATH)


def ref_knn():
    """The reference's own kNN.cpp / haplotype.cpp (``make -C oracle ref``)."""
    global _ref_knn
    if _ref_knn is None:
        R = C.CDLL(REF_KNN_PATH)
        R.glpr_knn.restype = C.c_int
        R.glpr_knn.argtypes = [_u64p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                               C.c_double, C.c_double, C.c_int, C.c_int, _u32p]
        R.glpr_max_tract.restype = C.c_uint32
        R.glpr_max_tract.argtypes = [_u8p, _u8p, C.c_uint32]
        R.glpr_hamming.restype = C.c_uint32
        R.glpr_hamming.argtypes = [_u8p, _u8p, C.c_uint32]
        _ref_knn = R
    return _ref_knn


def ref_glpack_available() -> bool:
    return os.path.exists(REF_GLPACK_PATH)


def ref_glpack(gl, use_vq=True, bits=4):
    """GLPack of the reference's own glPack.cpp / glVQ.cpp over all samples:
    (packed words [ceil(S / (32 / bits))][N], codebook [2^bits][2]) for GLs
    [N][S][3]; 8-bit nibble form when ``use_vq`` is false.  Its codebook is
    trained from the GLs with the GSL stand-in's counter draws."""
    global _ref_glpack
    if _ref_glpack is None:
        R = C.CDLL(REF_GLPACK_PATH)
        R.glpr_glpack.restype = C.c_int
        R.glpr_glpack.argtypes = [_f32p, C.c_uint32, C.c_uint32, C.c_int, C.c_uint32, _u32p,
                                  _f32p]
        _ref_glpack = R
    gl = _c(gl, np.float32)
    N, S = gl.shape[0], gl.shape[1]
    b = bits if use_vq else 8
    per = 32 // b
    packed = np.zeros(((S + per - 1) // per, N), np.uint32)
    cb = np.zeros((2 ** b, 2), np.float32)
    if _ref_glpack.glpr_glpack(gl, N, S, int(use_vq), b, packed, cb) != 0:
        raise ValueError("the reference's GLPack refused the arguments")
    return packed, cb


def ref_map_available() -> bool:
    return os.path.exists(REF_MAP_PATH)


def ref_genetic_distances(path, positions):
    """GeneticMap of the reference's own geneticMap.cpp on an uncompressed map
    file: (GeneticLocation in cM, GeneticDistance from the previous position
    in Morgans, 0 first) at ``positions``; ValueError where the reference
    throws."""
    global _ref_map
    if _ref_map is None:
        R = C.CDLL(REF_MAP_PATH)
        R.glpr_genetic_distances.restype = C.c_int
        R.glpr_genetic_distances.argtypes = [C.c_char_p, _u32p, C.c_uint32, _f64p, _f64p]
        _ref_map = R
    pos = _c(positions, np.uint32)
    loc = np.zeros(pos.size, np.float64)
    dist = np.zeros(pos.size, np.float64)
    if _ref_map.glpr_genetic_distances(os.fsencode(path), pos, pos.size, loc, dist) != 0:
        raise ValueError("the reference's GeneticMap threw")
    return loc, dist


def ref_knn_lists(haps, S, K, lb=0.0, ub=1.0, use_maf=False, metric="hamming"):
    """KNN::Neighbors of every sample from the reference's own ClusterHaps:
    [H/2][2*ceil(K/2)] (the frequencies come from ``haps`` themselves, as
    the reference computes them from its scaffold)."""
    haps = _c(haps, np.uint64)
    H, wn = haps.shape
    half = (K + 1) // 2
    out = np.zeros((H // 2, 2 * half), np.uint32)
    if ref_knn().glpr_knn(haps, H, wn, S, K, lb, ub, int(use_maf), KNN_METRICS[metric],
                          out) != 0:
        raise ValueError("the reference's KNN refused the arguments")
    return out


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


class OracleProblem:
    """Keeps the numpy arrays alive behind a ``Problem`` struct."""

    def __init__(self, haps, emit, prob, tran, pc, C_cycles, packed=None, codebook=None,
                 emit_mode=EMIT_FLOAT):
        self.haps = _c(haps, np.uint64)
        self.emit = _c(emit, np.float32)
        self.prob = _c(prob, np.float32)
        self.tran = _c(tran, np.float32)
        self.pc = _c(np.asarray(pc).reshape(16), np.float32)
        self.packed = None if packed is None else _c(packed, np.uint32)
        self.codebook = None if codebook is None else _c(np.asarray(codebook).reshape(-1),
                                                         np.float32)
        N, S = self.emit.shape[0], self.emit.shape[1]
        H, wn = self.haps.shape
        self.st = Problem(N, S, C_cycles, H, wn, self.haps.ctypes.data, self.emit.ctypes.data,
                          self.prob.ctypes.data, self.tran.ctypes.data, self.pc.ctypes.data,
                          None if self.packed is None else self.packed.ctypes.data,
                          None if self.codebook is None else self.codebook.ctypes.data,
                          emit_mode)

    def trace(self, seed=0, generation=0, slot=None, u_mh=None, u_work=None):
        keep = []
        def p(a, dt):
            if a is None:
                return None
            a = _c(a, dt)
            keep.append(a)
            return a.ctypes.data
        t = Trace(p(slot, np.uint8), p(u_mh, np.float64), p(u_work, np.float32), seed,
                  generation)
        t._keep = keep
        return t


def hmm_like_f32(emit_row, tran, haps, P):
    haps = _c(haps, np.uint64)
    return float(lib().glpo_hmm_like_f32(_c(emit_row, np.float32), _c(tran, np.float32), haps,
                                         haps.shape[1], emit_row.shape[0], _c(P, np.uint32)))


def hmm_like_f64(emit_row, tran, haps, P):
    haps = _c(haps, np.uint64)
    return float(lib().glpo_hmm_like_f64(_c(emit_row, np.float32), _c(tran, np.float32), haps,
                                         haps.shape[1], emit_row.shape[0], _c(P, np.uint32)))


def hmm_work(emit_row, prob_row, tran, pc, haps, P, pen, u):
    haps = _c(haps, np.uint64)
    S = emit_row.shape[0]
    wn = haps.shape[1]
    ha = np.zeros(wn, np.uint64)
    hb = np.zeros(wn, np.uint64)
    beta = np.zeros(S * 4, np.float32)
    lib().glpo_hmm_work(_c(emit_row, np.float32), _c(prob_row, np.float32), _c(tran, np.float32),
                        _c(np.asarray(pc).reshape(16), np.float32), haps, wn, S,
                        _c(P, np.uint32), pen, _c(u, np.float32), ha, hb, beta)
    return ha, hb


def generation(prob: OracleProblem, trace: Trace, quad, props, pen, first=0, last=None,
               do_work=True, nthreads=0, like=False):
    """Run a whole generation on the CPU.  Returns (quad_out [4][N],
    hnew [H][wn], like_out [N] or None)."""
    N = prob.st.N
    last = N if last is None else last
    quad_out = np.array(quad, dtype=np.uint32, copy=True)
    hnew = prob.haps.copy()
    like_out = np.zeros(N, np.float64) if like else None
    rc = lib().glpo_generation(C.byref(prob.st), C.byref(trace), _c(quad, np.uint32),
                               _c(props, np.uint32), pen, first, last, int(do_work), quad_out,
                               hnew, None if like_out is None else like_out.ctypes.data,
                               nthreads)
    if rc != 0:
        raise MemoryError("oracle generation could not allocate scratch")
    return quad_out, hnew, like_out


def solve_sample(prob: OracleProblem, trace: Trace, sample, quad, props, pen, do_work=False):
    Cc = prob.st.C
    q = np.zeros(4, np.uint32)
    likes = np.zeros(Cc + 1, np.float32)
    acc = np.zeros(max(Cc, 1), np.uint8)
    wn = prob.st.wn
    ha = np.zeros(wn, np.uint64)
    hb = np.zeros(wn, np.uint64)
    beta = np.zeros(prob.st.S * 4, np.float32)
    curr = lib().glpo_solve_sample(C.byref(prob.st), C.byref(trace), sample,
                                   _c(quad, np.uint32), _c(props, np.uint32), pen, q,
                                   likes.ctypes.data, acc.ctypes.data, int(do_work),
                                   ha.ctypes.data, hb.ctypes.data, beta.ctypes.data)
    return q, curr, likes, acc[:Cc], ha, hb


def replay_sample(prob: OracleProblem, trace: Trace, sample, quad, props, pen, gpu_accept):
    Cc = prob.st.C
    like32 = np.zeros(Cc + 1, np.float32)
    like64 = np.zeros(Cc + 1, np.float64)
    own = np.zeros(max(Cc, 1), np.uint8)
    q = np.zeros(4, np.uint32)
    lib().glpo_replay_sample(C.byref(prob.st), C.byref(trace), sample, _c(quad, np.uint32),
                             _c(props, np.uint32), pen,
                             _c(np.asarray(gpu_accept).reshape(-1)[:max(Cc, 1)], np.uint8),
                             like32, like64, own, q)
    return like32, like64, own[:Cc], q


def mh_draws(seed, generation, sample, C_cycles):
    slot = np.zeros(max(C_cycles, 1), np.uint8)
    u = np.zeros(max(C_cycles, 1), np.float64)
    lib().glpo_mh_draws(seed, generation, sample, C_cycles, slot, u)
    return slot[:C_cycles], u[:C_cycles]


def work_uniforms(seed, generation, sample, S):
    u = np.zeros(S, np.float32)
    lib().glpo_work_uniforms(seed, generation, sample, S, u)
    return u


def sample_surrogates(seed, generation, N, C_cycles, lo, hi, nbr=None, kick_first=False,
                      H=None):
    """The surrogates a generation draws on the device, materialised:
    (quad [4][N], props [C][N]).  kick_first: the first proposal of every
    chain from the panel rows [2N, H) (H defaults to hi)."""
    quad = np.zeros((4, N), np.uint32)
    props = np.zeros((max(C_cycles, 1), N), np.uint32)
    if nbr is not None:
        nb = _c(nbr, np.uint32)
        ptr, klen = nb.ctypes.data, nb.shape[1]
    else:
        nb, ptr, klen = None, None, 0
    lib().glpo_sample_surrogates(seed, generation, N, C_cycles, lo, hi, ptr, klen,
                                 int(kick_first), hi if H is None else H, quad, props)
    return quad, props[:C_cycles]


def common_sites(haps, S, lb=0.0, ub=1.0, use_maf=False):
    haps = _c(haps, np.uint64)
    H, wn = haps.shape
    mask = np.zeros(wn, np.uint64)
    lib().glpo_common_sites(haps, H, wn, S, lb, ub, int(use_maf), mask)
    return mask


KNN_METRICS = {"hamming": 0, "tract": 1}


def knn(haps, S, K, lb=0.0, ub=1.0, use_maf=False, metric="hamming"):
    """KNN::ClusterHaps restated: [H/2][2*ceil(K/2)] neighbour lists.
    metric "hamming" (the default) or "tract": the number of common sites
    minus the longest shared tract (insti -T)."""
    haps = _c(haps, np.uint64)
    H, wn = haps.shape
    mask = common_sites(haps, S, lb, ub, use_maf)
    half = (K + 1) // 2
    out = np.zeros((H // 2, 2 * half), np.uint32)
    if lib().glpo_knn_metric(haps, H, wn, mask, K, KNN_METRICS[metric], out) != 0:
        raise ValueError("kNN list longer than the available haplotypes")
    return out


def max_tract(a, b, mask=None):
    """Haplotype::MaxTractLen of two packed haplotypes (uint64 words) over the
    sites set in mask (all sites of the words when None)."""
    a = _c(np.atleast_1d(a), np.uint64)
    b = _c(np.atleast_1d(b), np.uint64)
    if mask is None:
        mask = np.full(a.shape, np.uint64(0xFFFFFFFFFFFFFFFF))
    return int(lib().glpo_max_tract(a, b, _c(mask, np.uint64), a.shape[0]))
