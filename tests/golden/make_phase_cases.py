"""Generate tests/golden/phase_cases.npz from the reference's own regression
inputs and expected outputs (samples/simple_gls, used by
t/10-phase_simple_gls.t), read with glphase_gb300.io.

Run in a checkout where the reference tree exists:

    python tests/golden/make_phase_cases.py [reference root]

Stored: the GLs, positions and genetic-map distances of simple.gls.v1.bin
(3 samples x 3 sites), the expected phased genotypes of the whole file and
of the region 20:101363- (simple.gls.v1.expected.bin.vcf,
simple.gls.v1.region.expected.bin.vcf), and the same for
simple.gls.v1.samePos.bin (three biallelic records at one position,
t/15-phase_simple_gls_multiallelic.t, compared with the same expected
haplotypes), so the device pipeline can be run on them without the
reference tree.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from glphase_gb300 import io as gio  # noqa: E402

OUT = os.path.join(HERE, "phase_cases.npz")


def main(ref_root: str) -> None:
    simple = os.path.join(ref_root, "samples", "simple_gls")
    gmap = gio.read_genetic_map(os.path.join(ref_root, "samples", "geneticMap",
                                             "genetic_map_chr20_combined_b37.txt.gz"))
    d = gio.read_bin(os.path.join(simple, "simple.gls.v1.bin"))
    names, sites, exp_gt = gio.read_vcf_gt(os.path.join(simple, "simple.gls.v1.expected.bin.vcf"))
    assert names == d.names and sites.pos == d.sites.pos
    _, rsites, region_gt = gio.read_vcf_gt(
        os.path.join(simple, "simple.gls.v1.region.expected.bin.vcf"))
    pos = d.sites.positions()
    same = gio.read_bin(os.path.join(simple, "simple.gls.v1.samePos.bin"))
    same_pos = same.sites.positions()
    np.savez_compressed(
        OUT,
        same_gl=same.gl, same_pos=same_pos, same_r=gmap.distances(same_pos),
        same_alt=np.array(same.sites.alt),
        simple_gl=d.gl, simple_pos=pos, simple_r=gmap.distances(pos),
        simple_ref=np.array(d.sites.ref), simple_alt=np.array(d.sites.alt),
        simple_names=np.array(d.names), simple_expected_gt=exp_gt,
        region_pos=np.array(rsites.pos, dtype=np.int64), region_expected_gt=region_gt)
    print("wrote", OUT)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
