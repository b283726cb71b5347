"""The haplotype sets of the reference's kNN unit test
(src/testing/other_unittests.cpp:103-254), restated for the oracle and the
GPU kernel.  Haplotype i carries alt alleles at sites i..i+5 of 24 sites;
haplotype 1 is moved to sites 18..23 so that its nearest are 15 and 14.
The indices 2..15 are shuffled by a fixed permutation (the reference uses
std::random_shuffle) so that the result cannot depend on input order."""
import numpy as np

NUM_CLUSTERS = 4
NUM_HAPS = 16
NUM_SITES = NUM_HAPS + NUM_CLUSTERS * 2


def base_haps():
    h = np.zeros((NUM_HAPS, NUM_SITES), np.uint8)
    for i in range(NUM_HAPS):
        h[i, i:i + NUM_CLUSTERS + 2] = 1
    return h


def shuffled(bits, seed=1):
    perm = np.arange(NUM_HAPS)
    rng = np.random.default_rng(seed)
    perm[2:] = 2 + rng.permutation(NUM_HAPS - 2)
    return bits[perm], perm


def case_nearest():
    h = base_haps()
    for i in range(NUM_SITES - 6, NUM_SITES):
        h[1, i - NUM_SITES + 7] = 0
        h[1, i] = 1
    bits, perm = shuffled(h)
    # neighbours of sample 0 in unshuffled numbering, lb = 0, ub = 1
    return bits, perm, 0.0, 1.0, [2, 15, 3, 14]


def case_threshold():
    h = base_haps()
    for i in (1, 5, 6, 8, 9, 10):
        h[i, 0] = 1
    for i in (5, 6, 8, 11, 12):
        h[i, 2] = 1
    for i in (0, 1, 5, 7, 15, 14, 13):
        h[i, NUM_SITES - 1] = 1
    for i in (0, 1, 2, 3, 4, 5, 8):
        h[i, NUM_SITES - 2] = 1
    bits, perm = shuffled(h)
    return bits, perm, 0.4375, 1.0, [5, 6, 8, 2]


def expected_af_threshold():
    """varAfs[0..2] and the number of common sites at lb = 0.4375."""
    return [0.4375, 0.125, 0.5], 4
