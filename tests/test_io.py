"""Input/output either side of the path (glphase_gb300.io): the .bin GL
reader (glReader.cpp:64-82, 215-285), genetic maps (geneticMap.cpp), the
VCF writer (insti.cpp:2098-2167) and NRD (t/VCFComp.pm:116-131); plus the
reference's end-to-end phasing test t/90-phase_simulated_gls.t restated on
the CPU oracle with the reference's own example files."""
import gzip
import os

import numpy as np
import pytest

from glphase_gb300 import io as gio

REF_SAMPLES = "/root/reference/samples/hapGen"


def _bin(N=3, S=5, seed=0):
    rng = np.random.default_rng(seed)
    gl = rng.random((N, S, 2)).astype(np.float32) * 0.5
    sites = gio.Sites(["20"] * S, [100 + 7 * m for m in range(S)],
                      ["A", "C", "AT", "G", "T"][:S], ["G", "T", "A", "GCC", "C"][:S])
    return gio.BinGLs([f"s{i}" for i in range(N)], sites, gl)


@pytest.mark.parametrize("suffix", [".bin", ".bin.gz"])
def test_bin_round_trip(tmp_path, suffix):
    d = _bin()
    path = str(tmp_path / ("x" + suffix))
    gio.write_bin(path, d)
    if suffix.endswith(".gz"):
        with open(path, "rb") as f:
            assert f.read(2) == b"\x1f\x8b"
    r = gio.read_bin(path)
    assert r.names == d.names
    assert r.sites == d.sites
    one = np.float32(1)
    want = np.array([[gio.gl_pair(max(np.float32(0), (one - h) - a), h, a) for h, a in row]
                     for row in d.gl], dtype=np.float32)
    assert np.array_equal(r.gl, want)
    assert np.allclose(r.gl, d.gl, rtol=1e-6, atol=0)
    assert r.gl.dtype == np.float32 and r.gl.shape == (3, 5, 2)


def test_bin_keep_region_and_limit(tmp_path):
    d = _bin()
    path = str(tmp_path / "x.bin")
    gio.write_bin(path, d)
    r = gio.read_bin(path, keep={"s2", "s0"})
    assert r.names == ["s0", "s2"]
    assert np.array_equal(r.gl, gio.read_bin(path).gl[[0, 2]])
    r = gio.read_bin(path, region=("20", 107, 121))
    assert r.sites.pos == [107, 114, 121]
    r = gio.read_bin(path, size_limit=2)
    assert r.sites.pos == [100, 107] and r.not_read == 3
    assert r.gl.shape == (3, 2, 2)


def test_bin_format_errors(tmp_path):
    p = tmp_path / "bad.bin"
    p.write_text("chr\tpos\tallele\n")
    with pytest.raises(ValueError, match="does not contain any sample information"):
        gio.read_bin(str(p))
    p.write_text("chr\tpos\tallele\ta\tb\n20\t5\tAC\t0.1 0.2\n")
    with pytest.raises(ValueError, match="Input line 2 does not have the correct number"):
        gio.read_bin(str(p))
    p.write_text("chr\tpos\tallele\ta\n20\t5\tACG\t0.1 0.2\n")
    with pytest.raises(ValueError, match="Could not parse alleles"):
        gio.read_bin(str(p))
    # Bio::snp_storage_ordered (bio.cpp:47-75): order, one chromosome, no repeats
    head = "chr\tpos\tallele\ta\n"
    p.write_text(head + "20\t5\tAC\t0.1 0.2\n20\t5\tAG\t0.1 0.2\n")
    assert gio.read_bin(str(p)).sites.alt == ["C", "G"]
    for rows, msg in ((["20\t5\tAC", "20\t5\tAC"], "already exists"),
                      (["20\t6\tAC", "20\t5\tAC"], "less than last position"),
                      (["20\t5\tAC", "21\t6\tAC"], "wrong chromosome")):
        p.write_text(head + "".join(r + "\t0.1 0.2\n" for r in rows))
        with pytest.raises(ValueError, match=msg):
            gio.read_bin(str(p))


def test_strtof_rounds_the_decimal_once():
    """std::stof rounds the decimal straight to binary32; a decimal just off
    a binary32 midpoint whose nearest binary64 IS the midpoint must still go
    to its own side (binary64 first, then binary32 would tie to even)."""
    from decimal import Decimal, getcontext
    getcontext().prec = 60
    one, up = np.float32(1), np.nextafter(np.float32(1), np.float32(2))
    m = Decimal(1) + Decimal(2) ** -24                # midpoint of 1 and 1 + 2^-23
    eps = Decimal(2) ** -80
    got = gio.strtof([str(m + eps), str(m - eps), str(m), "0.2", "1e-3", " 0.5", "0"])
    assert got[0] == up and got[1] == one and got[2] == one   # exact tie: to even
    assert np.float32(float(str(m + eps))) == one             # the binary64 route differs
    m3 = Decimal(1) + 3 * Decimal(2) ** -24               # tie between odd and even
    assert gio.strtof([str(m3)])[0] == np.nextafter(up, np.float32(2))
    assert gio.strtof([str(m3 - eps)])[0] == up
    assert list(got[3:]) == [np.float32(0.2), np.float32(1e-3), np.float32(0.5), 0]


def test_nrd_matched_pairs_samples_and_sites_by_name():
    ts = gio.Sites(["1"] * 3, [10, 20, 30], ["A", "C", "G"], ["T", "G", "A"])
    qs = gio.Sites(["1"] * 3, [10, 30, 30], ["A", "G", "G"], ["T", "C", "A"])
    truth = np.array([[[0, 1], [1, 1], [0, 0]], [[1, 1], [0, 0], [0, 1]]], np.int8)
    test = np.array([[[0, 0], [0, 0], [0, 1]], [[1, 0], [0, 0], [0, 0]]], np.int8)
    # test samples in the other order; sites 10 and 30:G>A are shared
    nrd, ns, nsite = gio.nrd_matched(["a", "b"], ts, truth, ["b", "a"], qs, test)
    assert (ns, nsite) == (2, 2)
    # a: 0|1 vs 1|0 agree, 0|0 vs 0|0 not counted; b: 1|1 vs 0|0 differ, 0|1 vs 0|1 -> 1 of 3
    assert nrd == pytest.approx(100 / 3)


def test_parse_region():
    """Bio::Region (bio.cpp:6-24) as --region / -R parse it."""
    assert gio.parse_region("20:101363-") == ("20", 101363, 2 ** 32 - 1)
    assert gio.parse_region("20:5335724-5861377") == ("20", 5335724, 5861377)
    assert gio.parse_region("chrX:1-") == ("chrX", 1, 2 ** 32 - 1)
    assert gio.parse_region("") is None
    for bad, msg in (("20", "Could not parse"), ("20:a-b", "Could not parse"),
                     ("20:-100", "0 is not a valid"), ("20:0-5", "0 is not a valid")):
        with pytest.raises(ValueError, match=msg):
            gio.parse_region(bad)


def test_gl_conversions():
    """Bio::gl2prob / Bio::phred2prob (bio.hpp:154-170) and the GL trio the
    reference keeps (glReader.cpp:202-213)."""
    assert gio.gl2prob(0.0) == 1.0 and gio.gl2prob(2.0) == 1.0
    assert gio.gl2prob(-1.0) == np.float32(np.power(np.float32(10), np.float32(-1)))
    assert gio.phred2prob(0) == 1.0
    assert gio.phred2prob(10) == np.float32(0.1)
    assert gio.phred2prob(370) == np.float32(1e-37) and gio.phred2prob(371) == 0.0
    h, a = gio.gl_pair(np.float32(0.992), np.float32(0.008), np.float32(0))
    s = np.float32(np.float32(0.992) + np.float32(0.008))
    assert (h, a) == (np.float32(np.float32(0.008) / s), np.float32(0))
    assert gio.gl_pair(1, 1, 1) == (np.float32(1 / 3), np.float32(1 / 3))


VCF_HEAD = """##fileformat=VCFv4.2
##FORMAT=<ID=GT,Number=1,Type=String,Description="Genotype">
##FORMAT=<ID={tag},Number=G,Type={kind},Description="likelihoods">
#CHROM\tPOS\tID\tREF\tALT\tQUAL\tFILTER\tINFO\tFORMAT\ta\tb
"""


def test_vcf_gl_and_pl(tmp_path):
    p = tmp_path / "g.vcf"
    p.write_text(VCF_HEAD.format(tag="GL", kind="Float") +
                 "1\t10\t.\tA\tG\t.\t.\t.\tGT:GL\t0/0:0,-1,-2\t./.:.\n"
                 "1\t20\t.\tAC\tA\t.\t.\t.\tGL\t-2,0,-2\t-3,-1,0\n")
    r = gio.read_vcf_gls(str(p))
    assert r.names == ["a", "b"] and r.sites.pos == [10, 20] and r.sites.alt == ["G", "A"]
    t = [gio.gl2prob(v) for v in (0.0, -1.0, -2.0)]
    assert tuple(r.gl[0, 0]) == gio.gl_pair(*t)
    assert tuple(r.gl[1, 0]) == gio.gl_pair(1, 1, 1)      # missing: flat
    p.write_text(VCF_HEAD.format(tag="PL", kind="Integer") +
                 "1\t10\t.\tA\tG\t.\t.\t.\tPL\t0,10,20\t400,0,30\n")
    r = gio.read_vcf_gls(str(p))
    assert tuple(r.gl[0, 0]) == gio.gl_pair(*[gio.phred2prob(v) for v in (0, 10, 20)])
    assert gio.phred2prob(400) == 0.0
    assert tuple(r.gl[1, 0]) == gio.gl_pair(*[gio.phred2prob(v) for v in (400, 0, 30)])
    assert r.gl[1, 0, 0] > 0.99
    p.write_text(VCF_HEAD.format(tag="PL", kind="Integer") +
                 "1\t10\t.\tA\tG,T\t.\t.\t.\tPL\t0,1,2,3,4,5\t0,1,2,3,4,5\n")
    with pytest.raises(ValueError, match="More than two alleles"):
        gio.read_vcf_gls(str(p))
    p.write_text(VCF_HEAD.format(tag="DS", kind="Float"))
    with pytest.raises(ValueError, match="Could not find a known tag"):
        gio.read_vcf_gls(str(p))


def test_genetic_map(tmp_path):
    p = tmp_path / "m.map"
    p.write_text(gio.MAP_HEADER + "\n100 0 0\n200 0 1.5\n400 0 2.5\n")
    gm = gio.read_genetic_map(str(p))
    assert gm.location(100) == 0.0
    assert gm.location(200) == 1.5
    assert gm.location(150) == pytest.approx(0.75)
    assert gm.location(300) == pytest.approx(2.0)
    r = gm.distances([100, 150, 300, 400])
    assert r[0] == 0.0
    assert r[1:] == pytest.approx([0.0075, 0.0125, 0.005])
    with pytest.raises(ValueError, match="is not on genetic map"):
        gm.location(401)
    p.write_text("pos rate cm\n1 0 0\n")
    with pytest.raises(ValueError, match="header of genetic map"):
        gio.read_genetic_map(str(p))
    p.write_text(gio.MAP_HEADER + "\n5 0 0\n5 0 1\n")
    with pytest.raises(ValueError, match="sorted by position"):
        gio.read_genetic_map(str(p))
    p.write_text(gio.MAP_HEADER + "\n5 0\n")
    with pytest.raises(ValueError, match="three columns"):
        gio.read_genetic_map(str(p))
    p.write_text(gio.MAP_HEADER + "\n")
    with pytest.raises(ValueError, match="empty"):
        gio.read_genetic_map(str(p))


@pytest.mark.skipif("not __import__('oracle').ref_map_available()")
def test_genetic_map_matches_live_reference_build(tmp_path, oracle_lib):
    """GeneticMap of the reference's compiled geneticMap.cpp against
    io.GeneticMap on random maps (1 .. 60 rows, cM written with 1 .. 11
    decimals): locations and distances identical in binary64 at map
    positions and between them; the same files and positions refused
    (malformed rows, unsorted positions, positions off the map)."""
    O = oracle_lib
    rng = np.random.default_rng(19)
    path = tmp_path / "m.map"
    for _ in range(150):
        k = int(rng.integers(1, 60))
        pos = np.cumsum(rng.integers(1, 5000, k)) + int(rng.integers(0, 10**6))
        cm = np.cumsum(rng.random(k) * rng.choice([0.001, 0.1, 3.0]))
        rows = [f"{p} {r:.6f} {c:.{int(rng.integers(1, 12))}f}"
                for p, r, c in zip(pos, rng.random(k), cm)]
        path.write_text(gio.MAP_HEADER + "\n" + "\n".join(rows) + "\n")
        q = np.sort(np.concatenate([rng.integers(pos[0], pos[-1] + 1, 40),
                                    pos[rng.integers(0, k, 5)]]))
        loc, dist = O.ref_genetic_distances(str(path), q)
        gm = gio.read_genetic_map(str(path))
        assert np.array_equal([gm.location(int(x)) for x in q], loc)
        assert np.array_equal(gm.distances(q), dist)
    for body, q in ((["5 0 0", "5 0 1"], [5]), (["5 0"], [5]), (["5 0 0", "9 0 1"], [4]),
                    (["5 0 0", "9 0 1"], [10])):
        path.write_text(gio.MAP_HEADER + "\n" + "\n".join(body) + "\n")
        with pytest.raises(ValueError):
            O.ref_genetic_distances(str(path), q)
        with pytest.raises(ValueError):
            gio.read_genetic_map(str(path)).distances(q)


def test_genotype_calls_branches():
    # columns: samples (p0, p1); one site
    prob = np.array([[0.0, 0.0, 0.9, 0.1, 0.1, 0.9, 0.9, 0.9, 0.5, 0.5]], np.float32)
    gt = gio.genotype_calls(prob)
    assert gt[:, 0].tolist() == [[0, 0], [1, 0], [0, 1], [1, 1], [0, 1]]


def test_vcf_record_text(tmp_path):
    sites = gio.Sites(["20", "20"], [5, 9], ["A", "C"], ["G", "T"])
    prob = np.array([[1.0, 0.0, 0.5, 0.5],
                     [0.0, 0.0, 1.0, 1.0]], np.float32)
    path = str(tmp_path / "o.vcf")
    gio.write_vcf(path, sites, ["a", "b"], prob, command_line="test")
    lines = open(path).read().split("\n")
    assert lines[0] == "##fileformat=VCFv4.2"
    assert lines[-1] == ""
    body = [l for l in lines if l and not l.startswith("#")]
    assert body[0] == ("20\t5\t.\tA\tG\t100\tPASS\t.\tGT:GP:APP\t"
                       "1|0:380,0,380:0,380\t0|1:6.02,3.01,6.02:3.01,3.01")
    assert body[1] == ("20\t9\t.\tC\tT\t100\tPASS\t.\tGT:GP:APP\t"
                       "0|0:0,380,380:380,380\t1|1:380,380,0:0,0")
    names, s2, gt = gio.read_vcf_gt(path)
    assert names == ["a", "b"] and s2.pos == [5, 9]
    assert np.array_equal(gt, gio.genotype_calls(prob))
    with pytest.raises(ValueError, match="not between 0 and 1"):
        gio.write_vcf(path, sites, ["a", "b"], prob * 2, command_line="test")


def test_vcf_gz_round_trip(tmp_path):
    rng = np.random.default_rng(4)
    S, N = 40, 7
    prob = rng.random((S, 2 * N)).astype(np.float32)
    sites = gio.Sites(["1"] * S, list(range(10, 10 + S)), ["A"] * S, ["T"] * S)
    path = str(tmp_path / "o.vcf.gz")
    gio.write_vcf(path, sites, [f"n{i}" for i in range(N)], prob)
    with gzip.open(path, "rt") as f:
        assert f.readline().startswith("##fileformat")
    _, _, gt = gio.read_vcf_gt(path)
    assert np.array_equal(gt, gio.genotype_calls(prob))


def test_nrd_definition():
    def g(*d):  # dosages -> alleles
        a = np.array(d)
        return np.stack([(a >= 1), (a == 2)], -1).astype(np.int8)[None]
    t = g(0, 0, 1, 2, 1, 0)
    assert gio.nrd(t, t) == 0.0
    # RR/RR pairs are not counted: one discordance among 3 counted calls
    assert gio.nrd(t, g(0, 0, 1, 2, 2, 0)) == pytest.approx(100 / 3)
    # a false positive at a truth RR site is counted too: 1 of 4
    assert gio.nrd(t, g(1, 0, 1, 2, 1, 0)) == pytest.approx(25.0)
    # phase does not matter, missing calls are skipped
    q = g(0, 0, 1, 2, 1, 0)
    q[0, 2] = (1, 0)
    q[0, 3, 0] = -1
    assert gio.nrd(t, q) == 0.0
    assert np.array_equal(gio.dosages(q)[0], [0, 0, 1, -1, 1, 0])


needs_samples = pytest.mark.skipif(not os.path.isdir(REF_SAMPLES),
                                   reason="reference example files not present")


@needs_samples
def test_reads_reference_example_files():
    d = gio.read_bin(os.path.join(REF_SAMPLES, "ex.bin"))
    assert len(d.names) == 60 and len(d.sites) == 1000
    assert d.names[0] == "samp1"
    assert (d.sites.chrom[0], d.sites.pos[0], d.sites.ref[0], d.sites.alt[0]) == \
        ("20", 45162, "C", "T")
    assert tuple(d.gl[0, 0]) == (np.float32(0.008), np.float32(0.0))
    assert (d.gl >= 0).all() and (d.gl.sum(-1) <= 1.0 + 1e-6).all()
    gm = gio.read_genetic_map(os.path.join(REF_SAMPLES, "ex.map"))
    r = gm.distances(d.sites.positions())
    assert (r >= 0).all() and r[0] == 0
    names, sites, gt = gio.read_vcf_gt(os.path.join(REF_SAMPLES, "ex.vcf.gz"))
    assert names == d.names and sites.pos == d.sites.pos
    assert gt.shape == (60, 1000, 2)
    v = gio.read_vcf_gls(os.path.join(REF_SAMPLES, "ex.gls.vcf.gz"))
    assert v.names == d.names and v.sites.pos == d.sites.pos and v.gl.shape == (60, 1000, 2)
    assert (v.gl >= 0).all() and (v.gl.sum(-1) <= 1.0 + 1e-6).all()


@needs_samples
@pytest.mark.parametrize("source", ["ex.bin", "ex.gls.vcf.gz"])
def test_reference_simulated_gls_nrd(oracle_lib, tmp_path, source):
    """t/90-phase_simulated_gls.t:31-50 restated: phase ex.bin (and the same
    samples' GLs from ex.gls.vcf.gz) with the genetic map at -C100 -m 20 -B5
    -i5, write the VCF, and score it against the truth ex.vcf.gz:
    0 < NRD < 5.5.  Runs the CPU oracle, which the device pipeline matches
    bit for bit (tests/test_gpu_phase.py)."""
    from glphase_gb300 import phase as ph
    from phase_oracle import oracle_phase
    path = os.path.join(REF_SAMPLES, source)
    d = gio.read_bin(path) if source.endswith(".bin") else gio.read_vcf_gls(path)
    gm = gio.read_genetic_map(os.path.join(REF_SAMPLES, "ex.map"))
    opts = ph.PhaseOptions(sa_burnin=5, burnin=5, sampling=20, cycles=100, seed=1)
    m, haps = ph.prepare(d.gl, d.sites.positions(), gm, seed=opts.seed)
    prob, _ = oracle_phase(oracle_lib, m, haps, opts)
    out = str(tmp_path / "simulated_gls.bin.vcf.gz")
    gio.write_vcf(out, d.sites, d.names, prob, command_line="-C100 -m 20 -B5 -i5")
    _, _, called = gio.read_vcf_gt(out)
    _, _, truth = gio.read_vcf_gt(os.path.join(REF_SAMPLES, "ex.vcf.gz"))
    nrd = gio.nrd(truth, called)
    assert 0 < nrd < 5.5, nrd
