"""The reference's own loading and regression cases, restated:

* t/10-phase_simple_gls.t:32-68 and t/15-phase_simple_gls_multiallelic.t --
  simple GLs phased with and without the genetic map, on a region, and with
  all sites at one position, haplotypes compared up to each sample's
  orientation (VCFHapMatch / HapEq, t/VCFComp.pm:48-114), on the CPU oracle
  from the committed fixture (tests/golden/phase_cases.npz); the broken
  input of t/15 (a site twice) is rejected;
* t/91-phase_simulated_gls_with_scaffold.t (reference panel, --kickstart)
  and t/905-phase_simulated_gls_multi.t (split multi-allelic records) on the
  reference's simulated example, scored by NRD against its truth VCF;
* t/92-phase_real_gls_with_pre_haps_multi.t's real GLs (2,495 samples,
  1,024 sites with split multi-allelic records) phased from the .bin without
  pre-existing haplotypes and scored against the chip genotypes;
* src/testing/insti_unittests.cpp:85-184 (Insti.loadGLs) -- sites, GLs
  before and after Insti::initialize, and the reference panel of the
  onlyThree sample files, read from the reference tree when it is present.
"""
import os

import numpy as np
import pytest

from glphase_gb300 import io as gio
from glphase_gb300 import model as mdl

REF = "/root/reference"
SAMPLES = os.path.join(REF, "samples")
HAPGEN = os.path.join(SAMPLES, "hapGen")
ONLY_THREE = os.path.join(SAMPLES, "20_011976121_012173018.bin.onlyThree")
needs_ref = pytest.mark.skipif(not os.path.isdir(SAMPLES),
                               reason="reference sample files not present")


def test_hap_match_rules():
    e = np.array([[[0, 1], [1, 1], [1, 0]]], np.int8)
    assert gio.hap_match(e, e) is None
    assert gio.hap_match(e[:, :, ::-1], e) is None               # whole sample swapped
    assert gio.hap_match(np.array([[[1, 0], [1, 1], [1, 0]]], np.int8), e) is not None
    assert "Allele number 2" in gio.hap_match(np.array([[[0, 0], [1, 1], [1, 0]]], np.int8), e)
    assert gio.hap_match(e[:, :2], e) == "hap files have different lengths"
    two = np.concatenate([e, e[:, :, ::-1]])
    assert gio.hap_match(two, np.concatenate([e, e])) is None    # per-sample orientation


@pytest.mark.parametrize("case", ["map", "nomap", "region", "same_map", "same_nomap"])
def test_simple_gls_phase_like_the_reference(oracle_lib, case):
    """The expected haplotypes for every seed tried with the full schedule,
    and for most seeds on the region, whose 5 sampling generations leave
    sample 3's two hets in the wrong phase now and then, as the reference's
    own run can."""
    from phase_oracle import oracle_phase
    from simple_gls_cases import simple_case
    matches = 0
    for seed in range(1, 9):
        m, haps, opts, expected = simple_case(case, seed)
        prob, _ = oracle_phase(oracle_lib, m, haps, opts)
        matches += gio.hap_match(gio.genotype_calls(prob), expected) is None
    assert matches >= (6 if case == "region" else 8), matches


@needs_ref
def test_phase_cases_fixture_matches_reference_files(tmp_path, monkeypatch):
    import importlib.util
    here = os.path.dirname(os.path.abspath(__file__))
    spec = importlib.util.spec_from_file_location(
        "make_phase_cases", os.path.join(here, "golden", "make_phase_cases.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    monkeypatch.setattr(mod, "OUT", str(tmp_path / "cases.npz"))
    mod.main(REF)
    new = np.load(tmp_path / "cases.npz")
    old = np.load(os.path.join(here, "golden", "phase_cases.npz"))
    assert sorted(new.files) == sorted(old.files)
    for k in new.files:
        assert np.array_equal(new[k], old[k]), k


@needs_ref
@pytest.mark.parametrize("suffix", [".bin", ".vcf.gz"])
def test_load_gls_known_answers(suffix):
    """insti_unittests.cpp:85-172: 3 samples, 1,024 sites on chromosome 20;
    the (het, homAlt) pairs as loaded and the (homRef, het, homAlt) trios
    after Insti::initialize (insti.cpp:1345-1350)."""
    path = ONLY_THREE + suffix
    d = gio.read_bin(path) if suffix == ".bin" else gio.read_vcf_gls(path)
    assert len(d.names) == 3 and len(d.sites) == 1024
    assert set(d.sites.chrom) == {"20"}
    assert [d.sites.pos[i] for i in (0, 5, 1023)] == [11976121, 11977230, 12173018]
    assert [(d.sites.ref[i], d.sites.alt[i]) for i in (0, 5, 1023)] == \
        [("T", "C"), ("A", "G"), ("G", "T")]
    gl = d.gl  # [N][S][2]; the reference's pre-initialize prob is [S][N][2]
    assert gl[0, 0, 0] == 0 and gl[0, 0, 1] == 1
    assert gl[1, 0, 0] == pytest.approx(0.2, rel=4 * 2 ** -23) and gl[1, 0, 1] == 0
    assert (gl[2, 0] == 0).all() and gl[0, 1, 1] == 1 and gl[1, 1, 1] == 0
    assert gl[1, 2, 0] == 1                                      # prob[in*6 - 4]
    t = mdl.genotype_probs(gl)
    assert tuple(t[0, 0]) == (0, 0, 1)
    assert t[1, 0, 0] == pytest.approx(0.8, rel=4 * 2 ** -23)
    assert t[1, 0, 1] == pytest.approx(0.2, rel=4 * 2 ** -23) and t[1, 0, 2] == 0
    assert tuple(t[2, 0]) == (1, 0, 0)
    assert t[0, 1, 1] == 0 and t[0, 1, 2] == 1


@needs_ref
def test_reference_panel_known_answers():
    """insti_unittests.cpp:174-184: after LoadHapLegSamp(legend, hap)
    haplotypes 0 and 2 carry the reference allele and haplotype 3 the
    alternative at sites 0-600; from site 601 haplotypes 0 and 3 carry the
    alternative, 1 and 2 the reference."""
    d = gio.read_bin(ONLY_THREE + ".bin")
    panel = gio.load_reference_panel(ONLY_THREE + ".legend", ONLY_THREE + ".hap", d.sites)
    assert panel.shape == (4, 16)
    bits = mdl.unpack_haplotypes(panel, 1024)
    assert (bits[0, :601] == 0).all() and (bits[2, :601] == 0).all()
    assert (bits[3, :601] == 1).all()
    assert (bits[0, 601:] == 1).all() and (bits[1, 601:] == 0).all()
    assert (bits[2, 601:] == 0).all() and (bits[3, 601:] == 1).all()


def _panel_files(tmp_path, legend_rows, hap_rows, header="id position a0 a1"):
    leg, hap = tmp_path / "p.legend", tmp_path / "p.hap"
    leg.write_text(header + "\n" + "".join(r + "\n" for r in legend_rows))
    hap.write_text("".join(r + "\n" for r in hap_rows))
    return str(leg), str(hap)


def test_reference_panel_rules(tmp_path):
    sites = gio.Sites(["5"] * 3, [100, 200, 300], ["A", "C", "G"], ["T", "G", "A"])
    rows = ["x 50 A C", "x 100 A T", "x 150 C C", "x 200 C G", "x 300 G A"]
    haps = ["1 1", "0 1", "1 0", "1 1", "0 0"]
    leg, hap = _panel_files(tmp_path, rows, haps)
    p = gio.load_reference_panel(leg, hap, sites)
    assert mdl.unpack_haplotypes(p, 3).tolist() == [[0, 1, 0], [1, 1, 0]]
    # a GL site the panel lacks (alleles must match too)
    leg, hap = _panel_files(tmp_path, rows[:4] + ["x 300 G C"], haps)
    with pytest.raises(ValueError, match="Could not find all GL sites"):
        gio.load_reference_panel(leg, hap, sites)
    # a GL site twice
    leg, hap = _panel_files(tmp_path, rows + ["x 300 G A"], haps + ["1 1"])
    with pytest.raises(ValueError, match="too many matching sites"):
        gio.load_reference_panel(leg, hap, sites)
    leg, hap = _panel_files(tmp_path, rows, haps, header="id pos a0 a1")
    with pytest.raises(ValueError, match="header start"):
        gio.load_reference_panel(leg, hap, sites)
    leg, hap = _panel_files(tmp_path, rows, haps[:4] + ["0 0 1"])
    with pytest.raises(ValueError, match="same number of columns"):
        gio.load_reference_panel(leg, hap, sites)
    leg, hap = _panel_files(tmp_path, rows, haps[:4] + ["0 2"])
    with pytest.raises(ValueError, match="not 0 or 1"):
        gio.load_reference_panel(leg, hap, sites)
    # columns are read as atoi reads them
    leg, hap = _panel_files(tmp_path, rows, ["1 1", "0.9 1x", "1 0", "1 1", "a +0"])
    assert mdl.unpack_haplotypes(gio.load_reference_panel(leg, hap, sites), 3).tolist() == \
        [[0, 1, 0], [1, 1, 0]]
    leg, hap = _panel_files(tmp_path, rows[:2] + [""] + rows[2:], haps)
    with pytest.raises(ValueError, match="empty lines"):
        gio.load_reference_panel(leg, hap, sites)


@needs_ref
def test_duplicate_site_input_is_rejected():
    """t/15-phase_simple_gls_multiallelic.t:52-53: insti fails on
    simple.gls.v2.samePos.err.bin, whose last record repeats a site."""
    with pytest.raises(ValueError, match="already exists"):
        gio.read_bin(os.path.join(SAMPLES, "simple_gls", "simple.gls.v2.samePos.err.bin"))


def _read_gls(path):
    return gio.read_bin(path) if path.endswith(".bin") else gio.read_vcf_gls(path)


@needs_ref
@pytest.mark.parametrize("source", ["ex.bin", "ex.gls.vcf.gz"])
def test_reference_panel_kickstart_nrd(oracle_lib, source):
    """t/91-phase_simulated_gls_with_scaffold.t:31-58: ``-g ex.map -C100
    -m10 -B0 -i3 -H ex.haps.gz -L ex.leg -k``: the 120 panel haplotypes
    after the 120 sample rows, every chain's first proposal from the panel;
    NRD against ex.vcf.gz below 5 (2.09 and 3.14 here; seeds 2-4: 2.18-2.43
    and 3.05-3.20)."""
    from glphase_gb300 import phase as ph
    from phase_oracle import oracle_phase
    d = _read_gls(os.path.join(HAPGEN, source))
    gm = gio.read_genetic_map(os.path.join(HAPGEN, "ex.map"))
    opts = ph.PhaseOptions(sa_burnin=0, burnin=3, sampling=10, cycles=100, seed=1,
                           kick_first=True)
    m, haps = ph.prepare(d.gl, d.sites.positions(), gm, seed=opts.seed)
    panel = gio.load_reference_panel(os.path.join(HAPGEN, "ex.leg"),
                                     os.path.join(HAPGEN, "ex.haps.gz"), d.sites)
    assert panel.shape == (120, 16)
    prob, _ = oracle_phase(oracle_lib, m, np.concatenate([haps, panel]), opts)
    _, _, truth = gio.read_vcf_gt(os.path.join(HAPGEN, "ex.vcf.gz"))
    nrd = gio.nrd(truth, gio.genotype_calls(prob))
    assert 0 < nrd < 5, nrd


@needs_ref
@pytest.mark.parametrize("source,truth", [("ex.gls.multi.vcf.gz", "ex.multi.vcf.gz"),
                                          ("ex.gls.almost_multi.vcf.gz",
                                           "ex.almost_multi.vcf.gz")])
def test_multiallelic_simulated_gls_nrd(oracle_lib, source, truth):
    """t/905-phase_simulated_gls_multi.t:29-51: ``-C100 -m20 -B5 -i5 -Fbcf``
    without a map on GLs whose multi-allelic sites are split into biallelic
    records at one position (and on the version with neighbouring
    positions); 0 < NRD < 5.5 (4.93 and 5.08 here; seeds 2-4: 5.03-5.09 and
    5.00-5.07)."""
    from glphase_gb300 import phase as ph
    from phase_oracle import oracle_phase
    d = gio.read_vcf_gls(os.path.join(HAPGEN, source))
    opts = ph.PhaseOptions(sa_burnin=5, burnin=5, sampling=20, cycles=100, seed=1)
    m, haps = ph.prepare(d.gl, d.sites.positions(), None, seed=opts.seed)
    prob, _ = oracle_phase(oracle_lib, m, haps, opts)
    _, sites, want = gio.read_vcf_gt(os.path.join(HAPGEN, truth))
    assert sites.pos == d.sites.pos and sites.alt == d.sites.alt
    nrd = gio.nrd(want, gio.genotype_calls(prob))
    assert 0 < nrd < 5.5, nrd


@needs_ref
def test_real_gls_nrd(oracle_lib):
    """t/92-phase_real_gls_with_pre_haps_multi.t:59-100 without the
    pre-existing haplotypes (a scaffold is outside this path) and from the
    .bin (the tree holds no BCF of these GLs): ``-R20:5335724-5861377 -g
    map -C100 -m10 -B0 -i5``, NRD against the Omni chip genotypes of the
    shared samples and sites below 15 (11.1 here)."""
    from glphase_gb300 import phase as ph
    from phase_oracle import oracle_phase
    src = os.path.join(SAMPLES, "multi_gls")
    d = gio.read_bin(os.path.join(src, "chr20.5335724-5861377.1024_site_subset.HRC.r1.AC5."
                                       "TGPP3_samples.likelihoods.winniFilter.bin"),
                     region=gio.parse_region("20:5335724-5861377"))
    assert len(d.names) == 2495 and len(d.sites) == 1024
    gm = gio.read_genetic_map(os.path.join(SAMPLES, "geneticMap",
                                           "genetic_map_chr20_combined_b37.txt.gz"))
    opts = ph.PhaseOptions(sa_burnin=0, burnin=5, sampling=10, cycles=100, seed=1)
    m, haps = ph.prepare(d.gl, d.sites.positions(), gm, seed=opts.seed)
    prob, _ = oracle_phase(oracle_lib, m, haps, opts)
    tn, ts, tg = gio.read_vcf_gt(os.path.join(
        src, "20.5335724-5861377.chip.omni_broad_sanger_combined.20140818.snps.genotypes.vcf.gz"))
    nrd, ns, nsite = gio.nrd_matched(tn, ts, tg, d.names, d.sites, gio.genotype_calls(prob))
    assert ns > 300 and nsite > 300
    assert 0 < nrd < 15, nrd


@needs_ref
def test_genetic_map_known_answers():
    """other_unittests.cpp:382-418 (GeneticMap errorOK, locationOK,
    distanceOK) on genetic_map_chr20_combined_b37."""
    gm = gio.read_genetic_map(os.path.join(SAMPLES, "geneticMap",
                                           "genetic_map_chr20_combined_b37.txt.gz"))
    for a, b in ((1140749, 1140727), (0, 1140727), (1140727, 70000000)):
        with pytest.raises(ValueError):
            gm.distance(a, b)
    hi, lo = 5.49294973985857, 5.49294697413266
    assert gm.location(1140749) == pytest.approx(hi, rel=4 * 2 ** -52)
    assert gm.location(1140727) == pytest.approx(lo, rel=4 * 2 ** -52)
    assert gm.location(1140730) == pytest.approx(lo + (hi - lo) * 3 / 22, rel=4 * 2 ** -52)
    assert gm.distance(1140727, 1140749) == pytest.approx((hi - lo) / 100, rel=1e-12)
    assert gm.distance(61795, 1140727) == pytest.approx(0.0549294697413266, rel=4 * 2 ** -52)
    assert gm.distance(61795, 62949445) == pytest.approx(1.10205396293913, rel=4 * 2 ** -52)
    assert gm.distance(1140727, 62949445) == pytest.approx(1.0471244931978034,
                                                           rel=4 * 2 ** -52)
    assert gm.distance(1140727, 1140732) == pytest.approx((hi - lo) / 22 * 5 / 100, abs=1e-9)
    assert gm.distance(1140507, 1140732) == pytest.approx(
        ((lo - 5.49291291069285) / 270 * 220 + (hi - lo) / 22 * 5) / 100, abs=1e-8)


@needs_ref
@pytest.mark.parametrize("suffix", [".bin", ".vcf.gz"])
def test_gl_reader_region_and_size_limit(suffix):
    """glReader_tests.cpp:174-224: the region 20:11976121-11976813 and a
    size limit of 3 both keep the first three sites, with their GLs."""
    path = ONLY_THREE + suffix
    read = gio.read_bin if suffix == ".bin" else gio.read_vcf_gls
    full = read(path)
    for d in (read(path, region=("20", 11976121, 11976813)), read(path, size_limit=3)):
        assert d.sites.pos == full.sites.pos[:3] == [11976121, 11976755, 11976813]
        assert np.array_equal(d.gl, full.gl[:, :3])
    assert read(path, size_limit=3).not_read == 1021


@needs_ref
def test_reference_panel_needs_both_files(tmp_path):
    """insti_unittests.cpp:424-441: a hap file without its legend, or a
    legend without its hap file, is refused."""
    from glphase_gb300 import phase as ph
    for leg, hap in ((None, ONLY_THREE + ".hap"), (ONLY_THREE + ".legend", None)):
        with pytest.raises(ValueError, match="both a legend and a hap file"):
            ph.phase_bin(ONLY_THREE + ".bin", ref_legend=leg, ref_hap=hap)
