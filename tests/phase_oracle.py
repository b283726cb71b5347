"""The end-to-end phasing loop of glphase_gb300.phase restated on the CPU
oracle (test infrastructure): the same generations, penalties, surrogate
draws, tallies and result, so the device pipeline can be compared with it
bit for bit and its accuracy checked where no GPU is present (uniform or
kNN sampler, with the reference's recluster rule)."""
from __future__ import annotations

import numpy as np

from glphase_gb300.batch import anneal_pen
from glphase_gb300.phase import knn_builds


def oracle_phase(O, model, haps, opts, nthreads=0):
    """Returns (prob [S][2N] float32, final haplotypes) like phase.phase."""
    N, S, Cc = model.N, model.S, opts.cycles
    H, wn = haps.shape
    cur = np.ascontiguousarray(haps, dtype=np.uint64)
    hsum = np.zeros(2 * N * S, np.uint32)
    tallied_from = opts.sa_burnin + opts.burnin
    builds = set(knn_builds(opts))
    table = None
    for g in range(opts.generations):
        if g in builds:   # KNN::ClusterHaps on the current haplotypes
            table = np.ascontiguousarray(O.knn(cur, S, opts.knn, metric=opts.knn_metric)[:N])
        nbr = table if opts.knn and g >= opts.cluster_start else None
        pb = O.OracleProblem(cur, model.emit, model.t, model.tran, model.pc, Cc)
        panel = H > 2 * N
        lo, hi = (2 * N, H) if (opts.kick_start and panel and g == 0) else (0, H)
        quad, props = O.sample_surrogates(opts.seed, g, N, Cc, lo, hi, nbr=nbr,
                                          kick_first=opts.kick_first and panel, H=H)
        tr = pb.trace(seed=opts.seed, generation=g)
        pen = float(anneal_pen(g, opts.sa_burnin))
        _, cur, _ = O.generation(pb, tr, quad, props, pen, do_work=True, nthreads=nthreads)
        if g >= tallied_from:
            flat = np.ascontiguousarray(cur).reshape(-1)
            for s in range(N):
                O.lib().glpo_replace(flat, wn, S, s, hsum)
    prob = np.zeros(2 * N * S, np.float32)
    O.lib().glpo_result(hsum, N, S, opts.sampling, prob)
    return prob.reshape(S, 2 * N), cur
