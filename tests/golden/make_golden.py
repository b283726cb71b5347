"""Generate tests/golden/reference_vectors.npz from the reference's own
impute.cpp, compiled in place by ``make -C oracle ref`` (oracle/_ref).

Run in a checkout where the reference tree exists:

    python tests/golden/make_golden.py

The vectors pin Impute::hmm_like (src/impute.cpp:327-376), Impute::hmm_work
(src/impute.cpp:380-485), the model constants of Impute::initialize
(src/impute.cpp:182-322) and Impute::replace (src/impute.cpp:564-595) on
small seeded synthetic inputs; tests compare the oracle and the CUDA path
against them without needing the reference tree.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from glphase_gb300 import model as mdl, synth  # noqa: E402

OUT = os.path.join(HERE, "reference_vectors.npz")


def main() -> None:
    O.build(ref=True)
    R = O.ref()
    rng = np.random.default_rng(2024)
    w = synth.Workload("golden", N=8, S=200, founders=6, depth=3.0, burnin=2, sampling=2,
                       cycles=20, panel_haps=4, seed=5)
    ds = synth.generate(w)
    m, haps = synth.initial_state(ds, seed=3)
    N, S = m.N, m.S
    H, wn = haps.shape
    emit = np.ascontiguousarray(m.emit)
    t = np.ascontiguousarray(m.t)
    tran = np.ascontiguousarray(m.tran)
    pc = np.ascontiguousarray(m.pc.reshape(16))

    # hmm_like on random quadruples
    nq = 64
    like_sample = rng.integers(0, N, nq).astype(np.uint32)
    like_quad = rng.integers(0, H, (nq, 4)).astype(np.uint32)
    like_ref = np.zeros(nq, np.float32)
    for i in range(nq):
        like_ref[i] = R.glpr_hmm_like(np.ascontiguousarray(emit[like_sample[i]]), tran, haps, H,
                                      wn, S, np.ascontiguousarray(like_quad[i]))

    # hmm_work at two penalties
    nw = 16
    work_sample = rng.integers(0, N, nw).astype(np.uint32)
    work_quad = rng.integers(0, H, (nw, 4)).astype(np.uint32)
    work_u = rng.random((nw, S)).astype(np.float32)
    pens = np.array([1.0, 0.25], np.float32)
    work_ha = np.zeros((len(pens), nw, wn), np.uint64)
    work_hb = np.zeros((len(pens), nw, wn), np.uint64)
    for k, pen in enumerate(pens):
        for i in range(nw):
            s = work_sample[i]
            R.glpr_hmm_work(np.ascontiguousarray(emit[s]), np.ascontiguousarray(t[s]), tran, pc,
                            haps, H, wn, S, np.ascontiguousarray(work_quad[i]), float(pen),
                            np.ascontiguousarray(work_u[i]), work_ha[k, i], work_hb[k, i])

    # model constants of Impute::initialize (positions, no genetic map)
    Ni, Si = 5, 40
    gl_in = rng.dirichlet([1.0, 1.0, 1.0], size=(Si, Ni)).astype(np.float32)
    prob_site_major = np.ascontiguousarray(gl_in[..., 1:3])  # [S][N][2] (het, homAlt)
    pos = np.cumsum(rng.integers(50, 400, Si)).astype(np.float64)
    init_tran = np.zeros(Si * 3, np.float32)
    init_pc = np.zeros(16, np.float32)
    init_emit = np.zeros(Ni * Si * 4, np.float32)
    init_t = np.zeros(Ni * Si * 3, np.float32)
    R.glpr_initialize(prob_site_major.reshape(-1), pos, Ni, Si, 1.0, init_tran, init_pc,
                      init_emit, init_t)

    # replace tallies over a few generations of random haplotypes
    hs = rng.integers(0, 2**63, size=(6, 2 * 3, 2), dtype=np.uint64)
    hsum = np.zeros(2 * 3 * 100, np.uint32)
    for g in range(hs.shape[0]):
        for s in range(3):
            R.glpr_replace(np.ascontiguousarray(hs[g]), 3, 100, 2, s, hsum)

    np.savez_compressed(
        OUT, haps=haps, emit=emit, t=t, tran=tran, pc=pc, N=N, S=S,
        like_sample=like_sample, like_quad=like_quad, like_ref=like_ref,
        work_sample=work_sample, work_quad=work_quad, work_u=work_u, pens=pens,
        work_ha=work_ha, work_hb=work_hb,
        init_gl=prob_site_major, init_pos=pos, init_tran=init_tran, init_pc=init_pc,
        init_emit=init_emit, init_t=init_t,
        replace_haps=hs, replace_hsum=hsum)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
