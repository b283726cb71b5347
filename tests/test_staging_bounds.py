"""Bounds of every copy and read of the generation kernel's staging, checked
on the CPU for every site count up to 2,100 and for the benchmark shapes.

The index arithmetic is restated from eval_pair (glp_kernels.cuh): with
nw = floor(S/64) full words, wf = ceil(nw/2) forward and wb = nw - wf
backward words, block t (8 sites) of the forward half is copied from the
transition rows 8t .. 8t+7 and the emission rows 8t .. 8t+7; block t of
the backward half is block n = 8 nw - 1 - t, copied from the transition
rows 8n + 1 .. 8n + 8 and the emission rows 8n .. 8n+7, stored reversed;
block t goes to slot t mod 4 of the direction's ring; the odd lane's sites
above the last full word read the emission row m and transition row m + 1
for m in [64 nw, S).  The transition table has S + 1 rows, the emission row
S, and a group's ring 137 float4 with the backward slots from offset 68.
"""
RING_STRIDE, BWD_OFF, SLOT, SLOTS = 137, 68, 16, 4


def copies(S):
    nw = S >> 6
    wf = (nw + 1) >> 1
    wb = nw - wf
    top = 8 * nw - 1
    for t in range(8 * wf):
        for k in range(8):
            yield "tran", 8 * t + k
            yield "emit", 8 * t + k
            yield "ring", (t % SLOTS) * SLOT + k
            yield "ring", (t % SLOTS) * SLOT + 8 + k
    for t in range(8 * wb):
        n = top - t
        for k in range(8):
            yield "tran", 8 * n + 1 + k
            yield "emit", 8 * n + k
            yield "ring", BWD_OFF + (t % SLOTS) * SLOT + 7 - k
            yield "ring", BWD_OFF + (t % SLOTS) * SLOT + 8 + 7 - k
    for m in range(64 * nw, S):
        yield "emit", m
        yield "tran", m + 1
    # the join reads transition row 64 wf (the identity row S when 64 wf = S)
    yield "tran", 64 * wf


def test_staging_indices_in_bounds():
    for S in list(range(1, 2101)) + [4096, 8192, 12288, 16383, 16384]:
        seen = {"tran": set(), "emit": set()}
        for kind, i in copies(S):
            if kind == "ring":
                assert 0 <= i < RING_STRIDE - 5, (S, i)
            else:
                assert 0 <= i <= (S if kind == "tran" else S - 1), (S, kind, i)
                seen[kind].add(i)
        # every site's emission row is read by exactly one half of an evaluation
        assert seen["emit"] == set(range(S)), S
