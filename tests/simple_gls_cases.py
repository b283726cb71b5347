"""The reference's simple-GL regression cases (t/10-phase_simple_gls.t:32-68,
t/15-phase_simple_gls_multiallelic.t:27-50) on the committed fixture
tests/golden/phase_cases.npz: 3 samples x 3 sites phased with -C100 -B0
-i10 -m100 with and without the genetic map, the same with the three sites
at one position (biallelic records of a multi-allelic site), and the region
20:101363- with -C100 -B0 -i5 -m5; the phased haplotypes must match the
expected VCF up to each sample's orientation (VCFHapMatch)."""
from __future__ import annotations

import os

import numpy as np

from glphase_gb300 import phase as ph

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "phase_cases.npz")
CASES = ["map", "nomap", "region", "same_map", "same_nomap"]


class _MapDistances:
    """Stands in for io.GeneticMap with the stored distances of the sites."""

    def __init__(self, r):
        self.r = r

    def distances(self, positions):
        assert len(positions) == len(self.r)
        return self.r


def simple_case(name: str, seed: int = 1):
    """(model, starting haplotypes, options, expected GT [N][S][2])."""
    z = np.load(GOLDEN)
    gl, pos = z["simple_gl"], z["simple_pos"]
    if name == "region":
        keep = pos >= 101363
        assert np.array_equal(pos[keep], z["region_pos"])
        gl, pos, expected = gl[:, keep], pos[keep], z["region_expected_gt"]
        opts = ph.PhaseOptions(sa_burnin=0, burnin=5, sampling=5, cycles=100, seed=seed)
    else:
        expected = z["simple_expected_gt"]
        opts = ph.PhaseOptions(sa_burnin=0, burnin=10, sampling=100, cycles=100, seed=seed)
    r = z["simple_r"]
    if name.startswith("same"):
        gl, pos, r = z["same_gl"], z["same_pos"], z["same_r"]
    gmap = _MapDistances(r) if name.endswith("map") and "nomap" not in name else None
    m, haps = ph.prepare(np.ascontiguousarray(gl), pos, gmap, seed=seed)
    return m, haps, opts, expected
