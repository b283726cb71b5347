"""Device-vs-oracle comparison of one generation on a subset of samples
(test infrastructure).

For every checked sample the oracle replays the chain the device ran (same
quadruples, same proposals, the device's accept decisions) and the test
asserts, with the parity contract's tolerances:
  * every per-proposal log-likelihood within REL_TOL relative of the
    reference-order binary32 oracle (impute.cpp:327-376) and of the binary64
    yardstick (float emissions only);
  * the oracle's own accept decisions equal the device's except where
    |delta * pen - ln u| < TIE_TOL (MHSampler.hpp:86-93);
  * the final quadruple and the published log-likelihood bit-exact;
  * the two sampled haplotype rows (hmm_work, impute.cpp:380-485) bit-exact.

Returns the largest relative errors seen, so tests can report them per shape.
"""
from __future__ import annotations

import json
import math
import os

import numpy as np

REL_TOL = 1e-5
TIE_TOL = 1e-4


def check_samples(O, emit, prob, tran, pc, haps, quad, props, pen, out, samples, seed, gen,
                  check_work=True, trace=None, vq=None):
    """emit [N][S][4], prob [N][S][3] (host float32), haps the generation's
    input haplotypes; out: dict(quad [4][N], hnew [H][wn], like [N],
    evals [N][C+1], acc [N][C]) from the device.  vq = (packed codes,
    codebook): the likelihoods score the VQ-decoded emissions (hmmLike.cu:53-142);
    hmm_work still uses the float emissions, as the reference's CPU step does."""
    S = emit.shape[1]
    C = props.shape[0]
    if vq is None:
        pb = O.OracleProblem(haps, emit, prob, tran, pc, C)
    else:
        pb = O.OracleProblem(haps, emit, prob, tran, pc, C, packed=vq[0], codebook=vq[1],
                             emit_mode=O.EMIT_VQ)
    tr = pb.trace(seed=seed, generation=gen) if trace is None else \
        pb.trace(slot=trace[0], u_mh=trace[1], u_work=trace[2])
    worst = worst64 = 0.0
    for s in samples:
        s = int(s)
        like32, like64, own, qf = O.replay_sample(pb, tr, s, quad, props, pen, out["acc"][s])
        g = out["evals"][s]
        assert np.all(np.isfinite(g)), s
        ref32 = like32.astype(np.float64)
        rel = np.abs(g - ref32) / np.abs(ref32)
        worst = max(worst, float(rel.max()))
        assert rel.max() <= REL_TOL, (s, float(rel.max()))
        if vq is None:  # the binary64 yardstick scores the float emissions
            rel64 = np.abs(g - like64) / np.abs(like64)
            worst64 = max(worst64, float(rel64.max()))
            assert rel64.max() <= REL_TOL, (s, float(rel64.max()))
        us = O.mh_draws(seed, gen, s, C)[1] if trace is None else trace[1][s]
        curr = float(like32[0])
        for c in range(C):
            if own[c] != out["acc"][s, c]:
                d = (float(like32[c + 1]) - curr) * pen
                assert abs(d - math.log(max(us[c], 1e-300))) < TIE_TOL, (s, c)
            if out["acc"][s, c]:
                curr = float(like32[c + 1])
        assert np.array_equal(qf, out["quad"][:, s]), s
        last = np.where(np.r_[1, out["acc"][s]] == 1)[0][-1]
        assert out["like"][s] == g[last], s
        if check_work:
            u = O.work_uniforms(seed, gen, s, S) if trace is None else trace[2][s]
            ha, hb = O.hmm_work(emit[s], prob[s], tran, pc, haps, qf, pen, u)
            assert np.array_equal(ha, out["hnew"][2 * s]), s
            assert np.array_equal(hb, out["hnew"][2 * s + 1]), s
    return worst, (worst64 if vq is None else None)


def report(shape: str, worst: float, worst64: float, checked: int, **extra) -> None:
    """Print the largest errors of one shape and, when GLP_PARITY_REPORT
    names a file, append them there as one JSON line."""
    rec = {"shape": shape, "max_rel_vs_fp32_oracle": worst, "max_rel_vs_fp64": worst64,
           "samples_checked": checked, **extra}
    print("PARITY " + json.dumps(rec))
    path = os.environ.get("GLP_PARITY_REPORT")
    if path:
        with open(path, "a") as f:
            f.write(json.dumps(rec) + "\n")
