"""Host-side rules of the phasing loop (glphase_gb300.phase): the kNN table
schedule against the reference's recluster rule, and the oracle loop with
reclustering on the CPU."""
import numpy as np

from glphase_gb300 import phase as ph
from glphase_gb300 import synth


def reference_rule(g, bn, r):
    """insti.cpp:1675-1676: recluster when r > 0, g > bn and (g - bn) % r == 0."""
    return r > 0 and g > bn and (g - bn) % r == 0


def test_knn_schedule_follows_the_reference_rule():
    for B, I, M, start, r in ((5, 5, 20, 3, 2), (8, 0, 24, 0, 8), (2, 3, 10, 12, 3),
                              (4, 4, 8, 2, 0), (0, 0, 6, 0, 1)):
        opts = ph.PhaseOptions(sa_burnin=B, burnin=I, sampling=M, knn=10, cluster_start=start,
                               recluster=r)
        builds = ph.knn_builds(opts)
        bn = B + I
        for g in range(opts.generations):
            if reference_rule(g, bn, r):
                assert g in builds, (g, builds)
        # the first table exists when the sampler starts being used
        first_use = min(start, opts.generations - 1)
        assert builds and builds[0] <= max(first_use, builds[0])
        assert all(reference_rule(g, bn, r) or g == builds[0] for g in builds)
    assert ph.knn_builds(ph.PhaseOptions(knn=0, recluster=2)) == []


def test_oracle_loop_with_recluster_runs(oracle_lib):
    """The oracle loop with reclustering on a small cohort: the called
    genotypes beat calling each genotype from its GLs alone."""
    from glphase_gb300 import io as gio
    from phase_oracle import oracle_phase
    N, S = 24, 320
    w = synth.Workload("rc", N=N, S=S, founders=8, depth=5.0, burnin=3, sampling=6, seed=8)
    ds = synth.generate(w)
    m, haps = synth.initial_state(ds, seed=2)
    opts = ph.PhaseOptions(sa_burnin=3, burnin=2, sampling=6, cycles=40, seed=5, knn=12,
                           cluster_start=2, recluster=2)
    prob, final = oracle_phase(oracle_lib, m, haps, opts)
    truth = np.stack([ds.truth[0:2 * N:2], ds.truth[1:2 * N:2]], axis=-1).astype(np.int8)
    call = np.argmax(m.t, axis=-1)
    gl_only = np.stack([call >= 1, call == 2], axis=-1).astype(np.int8)
    assert gio.nrd(truth, gio.genotype_calls(prob)) < gio.nrd(truth, gl_only)
