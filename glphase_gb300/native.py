"""ctypes binding of the C ABI in include/glphase_gpu.h.

Loading fails loudly (``NativeLibraryMissing``) when the in-tree CUDA library
has not been built: there is no CPU fallback on the product path.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

GLP_OK = 0
GLP_ERR_ARG = 1
GLP_ERR_CUDA = 2
GLP_ERR_NOMEM = 3
GLP_ERR_STATE = 4
GLP_ERR_INDEX = 5
GLP_ERR_DEVICE = 6
GLP_ERR_TOO_LARGE = 7
GLP_ERR_NO_CONVERGE = 8

GLP_GEN_VQ = 1
GLP_GEN_NO_WORK = 2
GLP_KNN_HAMMING = 0
GLP_KNN_TRACT = 1
KNN_METRICS = {"hamming": GLP_KNN_HAMMING, "tract": GLP_KNN_TRACT}
GLP_GEN_KICK_FIRST = 4

GLP_REQ_QUEUED = 0
GLP_REQ_RESIDENT = 1
GLP_REQ_DONE = 2

EXPORTED = [
    "glp_check_device", "glp_create", "glp_destroy", "glp_last_error", "glp_set_stream",
    "glp_set_tran", "glp_set_mutation_mat", "glp_set_codebook", "glp_set_packed_gls",
    "glp_set_emission", "glp_run_hmm_on_device", "glp_run_generation",
    "glp_run_generation_host", "glp_finish", "glp_set_lanes_per_sample", "glp_get_stats",
    "glp_measure_fp32_peak", "glp_knn_neighbors", "glp_problem_create",
    "glp_problem_destroy", "glp_problem_set_model", "glp_problem_set_vq", "glp_run_batch",
    "glp_problem_set_model_device", "glp_batch_prepare", "glp_batch_run", "glp_batch_launch",
    "glp_batch_destroy", "glp_run_generation_noalloc", "glp_tally", "glp_result",
    "glp_set_evals_per_lane", "glp_get_counters", "glp_kernel_times", "glp_vq_train",
    "glp_vq_pack", "glp_set_block_sites", "glp_get_block_sites", "glp_server_create",
    "glp_server_submit", "glp_server_tick", "glp_server_poll", "glp_server_stats",
    "glp_server_destroy", "glp_server_release", "glp_set_knn_metric",
]


class NativeLibraryMissing(RuntimeError):
    pass


class GlpError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"glphase_gpu error {code}: {msg}")
        self.code = code


class GenerationArgs(C.Structure):
    _fields_ = [
        ("num_samples", C.c_uint32), ("num_sites", C.c_uint32), ("num_cycles", C.c_uint32),
        ("num_haps", C.c_uint32),
        ("haps", C.c_void_p), ("hnew", C.c_void_p),
        ("hap_idxs_in", C.c_void_p), ("hap_idxs_out", C.c_void_p), ("props", C.c_void_p),
        ("pen", C.c_float), ("seed", C.c_uint64), ("generation", C.c_uint32),
        ("flags", C.c_uint32),
        ("trace_slot", C.c_void_p), ("trace_accept", C.c_void_p), ("trace_work", C.c_void_p),
        ("like_out", C.c_void_p), ("eval_trace", C.c_void_p), ("accept_trace", C.c_void_p),
        ("neighbors", C.c_void_p), ("neighbors_per_sample", C.c_uint32),
        ("sample_lo", C.c_uint32), ("sample_hi", C.c_uint32),
        ("burnin", C.c_uint32), ("kick_start", C.c_uint32),
    ]


_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Load the CUDA library (optionally compiling it first)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_build.LIB):
        if build_if_missing:
            _build.build()
        else:
            raise NativeLibraryMissing(
                f"{_build.LIB} is not built; run glphase_gb300/build.py (nvcc, sm_103a)")
    L = C.CDLL(_build.LIB)
    vp, u32, u64, i32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int
    L.glp_check_device.argtypes = [i32, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32),
                                   C.POINTER(i32)]
    L.glp_create.argtypes = [i32, C.POINTER(vp)]
    L.glp_destroy.argtypes = [vp]
    L.glp_destroy.restype = None
    L.glp_last_error.argtypes = [vp]
    L.glp_last_error.restype = C.c_char_p
    L.glp_set_stream.argtypes = [vp, vp]
    L.glp_set_tran.argtypes = [vp, vp, u32]
    L.glp_set_mutation_mat.argtypes = [vp, vp]
    L.glp_set_codebook.argtypes = [vp, vp, u32]
    L.glp_set_packed_gls.argtypes = [vp, vp, C.c_size_t]
    L.glp_set_emission.argtypes = [vp, vp, vp, u32, u32]
    L.glp_run_hmm_on_device.argtypes = [vp, vp, C.c_size_t, vp, u32, u32, u32, vp, u64]
    L.glp_run_generation.argtypes = [vp, C.POINTER(GenerationArgs)]
    L.glp_run_generation_host.argtypes = [vp, C.POINTER(GenerationArgs)]
    L.glp_finish.argtypes = [vp]
    L.glp_set_lanes_per_sample.argtypes = [vp, u32]
    L.glp_set_evals_per_lane.argtypes = [vp, u32]
    L.glp_get_counters.argtypes = [vp, C.POINTER(u64), u32]
    L.glp_kernel_times.argtypes = [vp, u32, C.POINTER(C.c_float), C.POINTER(C.c_float)]
    L.glp_get_stats.argtypes = [vp, C.POINTER(u64), C.POINTER(u64), C.POINTER(u32)]
    L.glp_measure_fp32_peak.argtypes = [vp, C.c_float, C.POINTER(C.c_double)]
    L.glp_knn_neighbors.argtypes = [vp, vp, u32, u32, u32, C.c_double, C.c_double, i32, vp]
    L.glp_problem_create.argtypes = [vp, C.POINTER(vp)]
    L.glp_problem_destroy.argtypes = [vp]
    L.glp_problem_destroy.restype = None
    L.glp_problem_set_model.argtypes = [vp, vp, vp, vp, vp, u32, u32]
    L.glp_problem_set_vq.argtypes = [vp, vp, C.c_size_t, vp]
    L.glp_problem_set_model_device.argtypes = [vp, vp, vp, vp, vp, u32, u32]
    L.glp_batch_prepare.argtypes = [vp, u32, C.POINTER(vp), C.POINTER(GenerationArgs),
                                    C.POINTER(vp)]
    L.glp_batch_run.argtypes = [vp]
    L.glp_batch_launch.argtypes = [vp]
    L.glp_batch_destroy.argtypes = [vp]
    L.glp_batch_destroy.restype = None
    L.glp_run_generation_noalloc.argtypes = [C.POINTER(GenerationArgs), vp, vp, vp, vp, vp]
    L.glp_tally.argtypes = [vp, vp, u32, u32, vp]
    L.glp_result.argtypes = [vp, vp, u32, u32, u32, vp]
    L.glp_vq_train.argtypes = [vp, vp, C.c_uint64, u32, vp, C.c_uint64, u32, vp]
    L.glp_vq_pack.argtypes = [vp, vp, u32, u32, vp, u32, u32, vp]
    L.glp_set_block_sites.argtypes = [vp, u32]
    L.glp_set_knn_metric.argtypes = [vp, i32]
    L.glp_get_block_sites.argtypes = [vp, vp]
    L.glp_run_batch.argtypes = [vp, u32, C.POINTER(vp), C.POINTER(GenerationArgs)]
    L.glp_server_create.argtypes = [vp, u64, i32, C.POINTER(vp)]
    L.glp_server_submit.argtypes = [vp, vp, C.POINTER(GenerationArgs), u32, C.POINTER(u64)]
    L.glp_server_tick.argtypes = [vp, C.POINTER(u32), C.POINTER(u32)]
    L.glp_server_poll.argtypes = [vp, u64, C.POINTER(i32), C.POINTER(u32), C.POINTER(vp)]
    L.glp_server_stats.argtypes = [vp, C.POINTER(u64), C.POINTER(u64), C.POINTER(u64)]
    L.glp_server_release.argtypes = [vp, u64]
    L.glp_server_destroy.argtypes = [vp]
    L.glp_server_destroy.restype = None
    for name in EXPORTED:
        getattr(L, name)
    _lib = L
    return L
