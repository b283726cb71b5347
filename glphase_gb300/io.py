"""Input and output either side of the phasing path.

* genotype likelihoods in the reference's ``.bin`` format
  (``GLReader::LoadSTBinNames`` / ``LoadSTBinGLs``, src/glReader.cpp:64-82,
  215-285): a tab-separated text file, optionally gzip-compressed, whose
  header is ``chr pos allele name1 name2 ...`` and whose rows are
  ``chrom pos alleles "het homAlt" ...`` (one space-separated pair per
  sample);
* genotype likelihoods in a VCF's GL (log10) or PL (Phred) field
  (``GLReader::LoadBCFGLs``, src/glReader.cpp:100-200; text VCF, optionally
  gzip-compressed, without htslib);
* genetic maps (``GeneticMap``, src/geneticMap.cpp:4-79): header
  ``position COMBINED_rate(cM/Mb) Genetic_Map(cM)``, then space-separated
  rows sorted by position; the genetic location of a site is linearly
  interpolated between map rows, and the distance between two sites is the
  difference in Morgans;
* a reference panel in IMPUTE2 legend + hap form (``Insti::OpenLegend``,
  ``OpenHap``, ``FilterSites``, ``LoadHaps``, src/insti.cpp:855-1184): the
  legend's sites ``id position a0 a1`` and one row of 0/1 alleles per site,
  kept where chrom:pos:ref:alt matches a GL site and packed to the rows that
  follow the 2N sample haplotypes;
* the phased VCF the reference writes (``Insti::save_vcf``,
  src/insti.cpp:2098-2167): GT from the allele probabilities of the two
  haplotypes, GP (genotype) and APP (allele) posteriors Phred-scaled;
* the haplotype match (up to each sample's orientation) and the
  non-reference discordance (NRD) its regression tests score a phased
  VCF by (``VCFNRD``, t/VCFComp.pm:116-131, which reads the ``NRDs`` line of
  ``bcftools stats``): over the genotypes where truth or call is not
  homozygous reference, the percentage whose calls differ.

Host code only; the arrays it returns feed ``model.Model`` and ``phase``.
"""
from __future__ import annotations

import gzip
from dataclasses import dataclass, field

import numpy as np

F32 = np.float32
FLT_MIN_10_EXP = -37  # <cfloat>
MAP_HEADER = "position COMBINED_rate(cM/Mb) Genetic_Map(cM)"
FLT_MAX_10_EXP = 38  # <cfloat>: the Phred value written for probability 0 is 10x this


def _open_read(path: str):
    with open(path, "rb") as f:
        magic = f.read(2)
    if magic == b"\x1f\x8b":
        return gzip.open(path, "rt")
    return open(path, "rt")


def _open_write(path: str):
    if path.endswith(".gz"):
        return gzip.open(path, "wt")
    return open(path, "wt")


@dataclass
class Sites:
    chrom: list[str] = field(default_factory=list)
    pos: list[int] = field(default_factory=list)
    ref: list[str] = field(default_factory=list)
    alt: list[str] = field(default_factory=list)

    _keys: set = field(default_factory=set, repr=False, compare=False)

    def __len__(self) -> int:
        return len(self.pos)

    def push_ordered(self, chrom: str, pos: int, ref: str, alt: str) -> None:
        """Append a site as ``Bio::snp_storage_ordered::push_back``
        (bio.cpp:47-75) does for the GL readers: positions never decrease,
        one chromosome, and no chrom:pos:ref:alt twice (multi-allelic sites
        come as biallelic records at the same position)."""
        if self.pos and pos < self.pos[-1]:
            raise ValueError(f"Tried to insert position [{pos}] that was less than last "
                             f"position [{self.pos[-1]}]")
        if self.chrom and chrom != self.chrom[0]:
            raise ValueError(f"Input snp is wrong chromosome [{chrom}]")
        key = f"{chrom}:{pos}:{ref}:{alt}"
        if key in self._keys:
            raise ValueError(f"Cannot push SNP, it already exists: [{key}]")
        self._keys.add(key)
        self.chrom.append(chrom)
        self.pos.append(pos)
        self.ref.append(ref)
        self.alt.append(alt)

    def positions(self) -> np.ndarray:
        return np.asarray(self.pos, dtype=np.int64)


@dataclass
class BinGLs:
    names: list[str]
    sites: Sites
    gl: np.ndarray          # [N][S][2] (het, homAlt) float32, sample-major
    not_read: int = 0       # sites past size_limit (GLReader::m_numNotRead)


def gl_pair(hom_ref, het, hom_alt) -> tuple[np.float32, np.float32]:
    """What the reference keeps of a GL trio (drop_first_aware_add_gl_trio
    with ST_DROP_FIRST, glReader.cpp:202-213, insti.cpp:219): het / sum and
    homAlt / sum, sum = (homRef + het) + homAlt, all binary32."""
    hr, h, a = F32(hom_ref), F32(het), F32(hom_alt)
    s = F32(F32(hr + h) + a)
    return F32(h / s), F32(a / s)


def strtof(tokens) -> np.ndarray:
    """Decimal strings to binary32 as ``std::stof`` (strtof) rounds them:
    straight from the decimal value to the nearest binary32, ties to even.
    Parsing to binary64 first and rounding that is the same except where the
    binary64 value lands exactly on a binary32 midpoint without the decimal
    being there; those few are settled against the exact decimal."""
    from decimal import Decimal
    toks = list(tokens)
    d = np.array(toks, dtype=np.float64) if toks else np.zeros(0)
    with np.errstate(over="ignore"):
        f = d.astype(F32)
    toward = np.where(d > f.astype(np.float64), np.inf, -np.inf).astype(F32)
    g = np.nextafter(f, toward)
    mid = (f.astype(np.float64) + g.astype(np.float64)) / 2
    tie = (d == mid) & (d != f.astype(np.float64)) & np.isfinite(d)
    for i in np.flatnonzero(tie):
        x, m = Decimal(toks[i].strip()), Decimal(float(mid[i]))
        if x != m:  # the decimal is off the midpoint: round toward its side
            f[i] = g[i] if (x > m) == (g[i] > f[i]) else f[i]
    return f


def gl_pairs(hom_ref: np.ndarray, het: np.ndarray, hom_alt: np.ndarray):
    """``gl_pair`` over arrays (the same binary32 operations elementwise)."""
    hr, h, a = (np.asarray(x, dtype=F32) for x in (hom_ref, het, hom_alt))
    s = (hr + h) + a
    return h / s, a / s


def gl2prob(val) -> np.float32:
    """Bio::gl2prob (bio.hpp:154-161): 10^val in binary32, clamped to [0, 1]."""
    with np.errstate(over="ignore"):
        t = np.power(F32(10), F32(val))
    return F32(min(max(t, F32(0)), F32(1)))


def phred2prob(phred: int) -> np.float32:
    """Bio::phred2prob (bio.hpp:163-170): 0 beyond the binary32 range, else
    10^(-phred/10) with the exponent in binary32 and the power in binary64."""
    if phred > FLT_MIN_10_EXP * -10:
        return F32(0)
    return F32(10.0 ** float(F32(-F32(phred)) / F32(10)))


UINT_MAX = 2 ** 32 - 1


def parse_region(region: str) -> tuple[str, int, int] | None:
    """``Bio::Region`` (bio.cpp:6-24): ``chrom:start-end``, the end may be
    left out (open to the end of the chromosome), the start may not be 0 or
    missing.  Returns (chrom, first, last) for the readers' ``region``, or
    None for an empty string (no region)."""
    import re
    if not region:
        return None
    m = re.fullmatch(r"(\S+):(\d*)-(\d*)", region)
    if not m:
        raise ValueError(f"Could not parse region: [{region}]")
    start = int(m.group(2)) if m.group(2) else 0
    if start == 0:
        raise ValueError("0 is not a valid genomic coordinate")
    end = int(m.group(3)) if m.group(3) else UINT_MAX
    return m.group(1), start, end


def read_bin(path: str, keep: set[str] | None = None,
             region: tuple[str, int, int] | None = None, size_limit: int = 0) -> BinGLs:
    """Read a ``.bin`` file (glReader.cpp:64-82, 215-285).

    ``keep`` restricts the samples (file order is kept), ``region`` =
    (chrom, first, last) keeps the sites inside it, ``size_limit`` > 0 stops
    after that many sites and counts the rest.  The file's site-major GLs
    come back sample-major as the reference keeps them: the trio
    (max(0, 1 - het - homAlt), het, homAlt) through ``gl_pair``.  Format
    errors raise ValueError with the reference's messages.
    """
    with _open_read(path) as fd:
        header = fd.readline().rstrip("\n").split("\t")
        if len(header) < 4:
            raise ValueError(f"Input bin file [{path}] does not contain any sample information")
        names = header[3:]
        idx = [i for i, n in enumerate(names) if not keep or n in keep]
        sites = Sites()
        het_tok: list[str] = []
        alt_tok: list[str] = []
        not_read = 0
        for line_num, line in enumerate(fd, start=2):
            tokens = line.rstrip("\n").split("\t")
            if len(tokens) != 3 + len(names):
                raise ValueError(f"Input line {line_num} does not have the correct number of "
                                 f"columns [{3 + len(names)}]")
            pos = int(tokens[1])
            if region is not None:
                chrom, first, last = region
                if tokens[0] != chrom or pos < first or pos > last:
                    continue
            if size_limit and len(sites) >= size_limit:
                not_read += 1
                continue
            alleles = tokens[2]
            if len(alleles) > 2:
                if " " not in alleles:
                    raise ValueError(f"Could not parse alleles [{alleles}]")
                ref, alt = alleles.split(" ", 1)
            else:
                ref, alt = alleles[0], alleles[1]
            sites.push_ordered(tokens[0], pos, ref, alt)
            for i in idx:
                pair = tokens[3 + i].split()
                if len(pair) < 2:
                    raise ValueError(f"Input line {line_num}: could not parse the GL pair "
                                     f"[{tokens[3 + i]}]")
                het_tok.append(pair[0])
                alt_tok.append(pair[1])
    S, n = len(sites), len(idx)
    # stof of each value, then the trio (max(0, 1 - het - homAlt), het, homAlt)
    # kept as gl_pair keeps it (glReader.cpp:272-283), all in binary32
    h = strtof(het_tok).reshape(S, n)
    a = strtof(alt_tok).reshape(S, n)
    hr = np.maximum((F32(1) - h) - a, F32(0))
    ph, pa = gl_pairs(hr, h, a)
    gl = np.ascontiguousarray(np.stack([ph, pa], axis=-1).transpose(1, 0, 2))
    return BinGLs([names[i] for i in idx], sites, gl, not_read)


def read_vcf_gls(path: str, tags=("GL", "PL"), keep: set[str] | None = None,
                 region: tuple[str, int, int] | None = None, size_limit: int = 0) -> BinGLs:
    """GLs from a VCF (GLReader::LoadBCFGLs, glReader.cpp:100-200): the first
    of ``tags`` the header declares as a FORMAT field; GL values through
    ``gl2prob``, PL through ``phred2prob``, each trio through ``gl_pair``.
    Biallelic records only.  A missing value (".") is read as a flat
    likelihood (the reference would carry a NaN).  Returns the .bin reader's
    structure."""
    declared: set[str] = set()
    names: list[str] = []
    idx: list[int] = []
    tag = None
    sites = Sites()
    rows = []
    not_read = 0
    with _open_read(path) as fd:
        for line in fd:
            if line.startswith("##"):
                if line.startswith("##FORMAT=<ID="):
                    declared.add(line[len("##FORMAT=<ID="):].split(",", 1)[0])
                continue
            cols = line.rstrip("\n").split("\t")
            if line.startswith("#CHROM"):
                names = cols[9:]
                idx = [i for i, n in enumerate(names) if not keep or n in keep]
                tag = next((t for t in tags if t in ("GL", "PL") and t in declared), None)
                if tag is None:
                    raise ValueError("[GLReader] Could not find a known tag")
                continue
            if len(cols) < 9:
                continue
            pos = int(cols[1])
            if region is not None:
                chrom, first, last = region
                if cols[0] != chrom or pos < first or pos > last:
                    continue
            if size_limit and len(sites) >= size_limit:
                not_read += 1
                continue
            alts = [] if cols[4] == "." else cols[4].split(",")
            if len(alts) < 1:
                raise ValueError("Too few alleles in BCF record")
            if len(alts) > 1:
                raise ValueError("More than two alleles per record are not supported. Please "
                                 "break BCF into biallelics using bcftools norm -m -")
            fmt = cols[8].split(":")
            if tag not in fmt:
                raise ValueError(f"no {tag} value at {cols[0]}:{cols[1]}")
            k = fmt.index(tag)
            row = np.empty((len(idx), 2), dtype=F32)
            for j, i in enumerate(idx):
                fields = cols[9 + i].split(":")
                vals = fields[k].split(",") if k < len(fields) else ["."]
                if len(vals) != 3:
                    if vals == ["."]:
                        vals = [".", ".", "."]
                    else:
                        raise ValueError(f"Returned number of values is not correct: {len(vals)}")
                if tag == "GL":
                    trio = [gl2prob(0.0 if v == "." else float(v)) for v in vals]
                else:
                    trio = [phred2prob(0 if v == "." else int(v)) for v in vals]
                row[j] = gl_pair(*trio)
            sites.push_ordered(cols[0], pos, cols[3], alts[0])
            rows.append(row)
    if rows:
        gl = np.ascontiguousarray(np.stack(rows, axis=1))
    else:
        gl = np.zeros((len(idx), 0, 2), dtype=F32)
    return BinGLs([names[i] for i in idx], sites, gl, not_read)


def write_bin(path: str, data: BinGLs) -> None:
    """Write GLs in the ``.bin`` layout read_bin parses (values with nine
    significant digits, which round-trip binary32)."""
    N, S, _ = data.gl.shape
    with _open_write(path) as fd:
        fd.write("\t".join(["chr", "pos", "allele"] + list(data.names)) + "\n")
        for m in range(S):
            ref, alt = data.sites.ref[m], data.sites.alt[m]
            alleles = ref + alt if len(ref) == 1 and len(alt) == 1 else f"{ref} {alt}"
            cols = [data.sites.chrom[m], str(data.sites.pos[m]), alleles]
            cols += [f"{float(data.gl[i, m, 0]):.9g} {float(data.gl[i, m, 1]):.9g}"
                     for i in range(N)]
            fd.write("\t".join(cols) + "\n")


# ---------------------------------------------------------------------------
# Genetic maps


@dataclass
class GeneticMap:
    position: np.ndarray    # int64, strictly increasing
    cm: np.ndarray          # float64 genetic location in cM

    def location(self, pos: int) -> float:
        """GeneticMap::GeneticLocation (geneticMap.cpp:46-70), in cM."""
        p = self.position
        if len(p) == 0:
            return 0.0
        if pos < p[0] or pos > p[-1]:
            raise ValueError(f"Genomic location {pos} is not on genetic map")
        hi = int(np.searchsorted(p, pos, side="left"))
        if p[hi] == pos:
            return float(self.cm[hi])
        lo = hi - 1
        diff_gen = float(self.cm[hi]) - float(self.cm[lo])
        diff_genom = float(p[hi] - p[lo])
        return float(self.cm[lo]) + (pos - int(p[lo])) / diff_genom * diff_gen

    def distance(self, first: int, second: int) -> float:
        """GeneticMap::GeneticDistance (geneticMap.cpp:72-79): Morgans from
        ``first`` to ``second``; ``first`` may not lie after ``second`` and
        both must be on the map."""
        if first > second:
            raise ValueError("first is larger than second")
        return (self.location(second) - self.location(first)) / 100

    def distances(self, positions) -> np.ndarray:
        """r[m] = GeneticDistance(pos[m-1], pos[m]) in Morgans
        (geneticMap.cpp:72-79); r[0] = 0.  This is the input of
        ``model.transition_from_distances``."""
        pos = [int(x) for x in positions]
        r = np.zeros(len(pos), dtype=np.float64)
        loc = [self.location(x) for x in pos]
        for m in range(1, len(pos)):
            if pos[m - 1] > pos[m]:
                raise ValueError("first is larger than second")
            r[m] = (loc[m] - loc[m - 1]) / 100
        return r


def read_genetic_map(path: str) -> GeneticMap:
    """GeneticMap::GeneticMap (geneticMap.cpp:4-44)."""
    pos, cm = [], []
    with _open_read(path) as fd:
        header = fd.readline().rstrip("\n")
        if header != MAP_HEADER:
            raise ValueError("header of genetic map does not look right. Expected "
                             f"'{MAP_HEADER}', but got '{header}'")
        for row_num, line in enumerate(fd, start=2):
            cols = line.rstrip("\n").split(" ")
            if len(cols) != 3:
                raise ValueError(f"Could not find three columns in line {row_num}")
            p = int(cols[0])
            if pos and p <= pos[-1]:
                raise ValueError("Genetic map does not appear to be sorted by position at "
                                 f"line {row_num}")
            pos.append(p)
            cm.append(float(cols[2]))
    if not pos:
        raise ValueError("Genetic map is empty.")
    return GeneticMap(np.asarray(pos, dtype=np.int64), np.asarray(cm, dtype=np.float64))


# ---------------------------------------------------------------------------
# Reference panel (legend + hap)

LEGEND_HEADER = ("id", "position", "a0", "a1")


def read_legend(path: str, chrom: str) -> Sites:
    """Insti::OpenLegend (insti.cpp:1031-1078): the header must start with
    ``id position a0 a1``; every row gives (position, a0, a1) of a site on
    ``chrom`` (the GL sites' chromosome); empty lines are errors."""
    sites = Sites()
    with _open_read(path) as fd:
        for line_num, line in enumerate(fd, start=1):
            line = line.rstrip("\n")
            if not line:
                raise ValueError(f"Error in legend file {path}: empty lines detected.")
            tokens = line.split()
            if line_num == 1:
                if tuple(tokens[:4]) != LEGEND_HEADER:
                    raise ValueError(f"Error in legend file {path}: header start does not "
                                     f"match: {' '.join(LEGEND_HEADER)}")
                continue
            sites.chrom.append(chrom)
            sites.pos.append(int(tokens[1]))
            sites.ref.append(tokens[2])
            sites.alt.append(tokens[3])
    return sites


def _atoi(token: str) -> int:
    """C's atoi: optional sign and the leading digits; 0 without digits."""
    import re
    m = re.match(r"\s*([+-]?\d+)", token)
    return int(m.group(1)) if m else 0


def read_hap(path: str) -> np.ndarray:
    """Insti::OpenHap (insti.cpp:1080-1137): one row per site, one 0/1
    column per haplotype, the same column count on every row; each column is
    read as atoi reads it.  Returns uint8 [sites][haplotypes]."""
    rows = []
    width = None
    with _open_read(path) as fd:
        for line_num, line in enumerate(fd):
            tokens = line.split()
            if width is None:
                width = len(tokens)
            if len(tokens) != width:
                raise ValueError("Every row of hap file must have the same number of columns")
            vals = [_atoi(t) for t in tokens]
            if any(v not in (0, 1) for v in vals):
                raise ValueError(f"All alleles are not 0 or 1 In haplotypes file {path} at "
                                 f"line number {line_num} (0-based)")
            rows.append(vals)
    if not width:
        raise ValueError("num haps is 0.  Haps file empty?")
    return np.asarray(rows, dtype=np.uint8)


def load_reference_panel(legend_path: str, hap_path: str, sites: Sites) -> np.ndarray:
    """The reference panel for the GL sites ``sites``
    (``Insti::LoadHapLegSamp`` with ``InstiPanelType::REFERENCE``,
    insti.cpp:1139-1184): legend rows whose chrom:pos:ref:alt is a GL site
    are kept in legend order (``FilterSites``, insti.cpp:855-925) and every
    GL site must be found exactly once; the kept rows are bit-packed per
    haplotype (``HapPanel::Char2BitVec``, hapPanel.cpp:41-64).  Returns
    uint64 [panel haplotypes][ceil(S/64)], the rows appended after the 2N
    sample haplotypes (insti.cpp:1398)."""
    from .model import pack_haplotypes
    chrom = sites.chrom[0] if len(sites) else ""
    legend = read_legend(legend_path, chrom)
    haps = read_hap(hap_path)
    if len(legend) != haps.shape[0]:
        raise ValueError("legend and hap files have different numbers of sites")
    if len(sites) > len(legend):
        raise ValueError("the reference panel has fewer sites than the GLs")
    gl_keys = {f"{c}:{p}:{r}:{a}" for c, p, r, a in zip(sites.chrom, sites.pos, sites.ref,
                                                        sites.alt)}
    keep = [i for i, (p, r, a) in enumerate(zip(legend.pos, legend.ref, legend.alt))
            if f"{chrom}:{p}:{r}:{a}" in gl_keys]
    if not keep:
        raise ValueError("Error: No sites in loaded panel matched already loaded sites. Is "
                         "your input file sorted?")
    if len(keep) > len(sites):
        raise ValueError("[insti] too many matching sites found")
    if len(keep) != len(sites):
        raise ValueError("[insti] Could not find all GL sites in loaded haplotype panel")
    return pack_haplotypes(haps[keep].T)


# ---------------------------------------------------------------------------
# VCF


def genotype_calls(prob: np.ndarray) -> np.ndarray:
    """The GT of Insti::save_vcf (insti.cpp:2125-2137) for allele
    probabilities ``prob`` [S][2N] (p0, p1 of each sample's two haplotypes,
    Impute::result's layout).  Returns alleles [N][S][2] (int8): the most
    probable of 0|0, het, 1|1 by (1-p0)(1-p1), (1-p0)p1 + p0(1-p1), p0 p1 in
    binary32, ties towards 0|0 then het; a het is 1|0 when p0 > p1."""
    p = np.asarray(prob, dtype=F32)
    S, hn = p.shape
    p0 = p[:, 0::2].T
    p1 = p[:, 1::2].T
    one = F32(1.0)
    prr = (one - p0) * (one - p1)
    pra = (one - p0) * p1 + p0 * (one - p1)
    paa = p0 * p1
    rr = (prr >= pra) & (prr >= paa)
    ra = ~rr & (pra >= prr) & (pra >= paa)
    aa = ~rr & ~ra
    gt = np.zeros((hn // 2, S, 2), dtype=np.int8)
    first_alt = ra & (p0 > p1)
    gt[..., 0] = (aa | first_alt).astype(np.int8)
    gt[..., 1] = (aa | (ra & ~first_alt)).astype(np.int8)
    return gt


def _phred(x: np.float32) -> np.float32:
    if x == 0:
        return F32(FLT_MAX_10_EXP * 10)
    if x == 1:
        return F32(0.0)
    if x > 1 or x < 0:
        raise ValueError(f"error: probability {x} is not between 0 and 1")
    return F32(F32(-10) * np.log10(F32(x)))


def _fmt3(x) -> str:
    """A float the way an ostream with setprecision(3) prints it."""
    return f"{float(x):.3g}"


def write_vcf(path: str, sites: Sites, names: list[str], prob: np.ndarray,
              command_line: str = "", source: str = "glphase_gb300") -> None:
    """Phased VCF of Insti::save_vcf (insti.cpp:2098-2167): one record per
    site with GT:GP:APP per sample, GP = Phred(P(0/0), P(het), P(1/1)) and
    APP = Phred(p0, p1), values printed to three significant digits."""
    p = np.asarray(prob, dtype=F32)
    S, hn = p.shape
    N = hn // 2
    if len(sites) != S or len(names) != N:
        raise ValueError(f"prob is [{S}][{hn}] for {len(sites)} sites and {len(names)} samples")
    gt = genotype_calls(p)
    one = F32(1.0)
    with _open_write(path) as fd:
        fd.write("##fileformat=VCFv4.2\n")
        fd.write(f"##source={source}\n")
        fd.write(f"##phaseAndImputeCall={command_line}\n")
        fd.write(f"##contig=<ID={sites.chrom[0] if S else '.'}>\n")
        fd.write('##FORMAT=<ID=GT,Number=1,Type=String,Description="Genotype">\n')
        fd.write('##FORMAT=<ID=GP,Number=3,Type=Float,Description="Phred-scaled '
                 'genotype posterior probability">\n')
        fd.write('##FORMAT=<ID=APP,Number=2,Type=Float,Description="Phred-scaled '
                 'allelic posterior probability, P(Allele=1|Haplotype)">\n')
        fd.write("#CHROM\tPOS\tID\tREF\tALT\tQUAL\tFILTER\tINFO\tFORMAT")
        for n in names:
            fd.write("\t" + n)
        for m in range(S):
            fd.write(f"\n{sites.chrom[m]}\t{sites.pos[m]}\t.\t{sites.ref[m]}\t{sites.alt[m]}"
                     "\t100\tPASS\t.\tGT:GP:APP")
            for i in range(N):
                p0, p1 = p[m, 2 * i], p[m, 2 * i + 1]
                prr = (one - p0) * (one - p1)
                pra = (one - p0) * p1 + p0 * (one - p1)
                paa = p0 * p1
                ph = [_phred(F32(v)) for v in (prr, pra, paa, p0, p1)]
                fd.write(f"\t{gt[i, m, 0]}|{gt[i, m, 1]}:" + ",".join(_fmt3(v) for v in ph[:3])
                         + ":" + ",".join(_fmt3(v) for v in ph[3:]))
        fd.write("\n")


def read_vcf_gt(path: str):
    """Sample names, sites and GT alleles [N][S][2] (int8, -1 missing) of a
    VCF (phased '|' or unphased '/'; haploid and multi-allelic calls are
    rejected)."""
    names: list[str] = []
    sites = Sites()
    calls = []
    with _open_read(path) as fd:
        for line in fd:
            if line.startswith("##"):
                continue
            cols = line.rstrip("\n").split("\t")
            if line.startswith("#CHROM"):
                names = cols[9:]
                continue
            if not cols or cols == [""]:
                continue
            fmt = cols[8].split(":")
            if "GT" not in fmt:
                raise ValueError(f"no GT field at {cols[0]}:{cols[1]}")
            k = fmt.index("GT")
            sites.chrom.append(cols[0])
            sites.pos.append(int(cols[1]))
            sites.ref.append(cols[3])
            sites.alt.append(cols[4])
            row = np.full((len(names), 2), -1, dtype=np.int8)
            for i, field_ in enumerate(cols[9:]):
                g = field_.split(":")[k].replace("/", "|").split("|")
                if len(g) != 2:
                    raise ValueError(f"not a diploid call: {field_}")
                for j in range(2):
                    if g[j] != ".":
                        a = int(g[j])
                        if a > 1:
                            raise ValueError(f"multi-allelic call: {field_}")
                        row[i, j] = a
            calls.append(row)
    gt = (np.stack(calls, axis=1) if calls else np.zeros((len(names), 0, 2), np.int8))
    return names, sites, gt


def nrd(truth_gt: np.ndarray, test_gt: np.ndarray) -> float:
    """Non-reference discordance in percent (the ``NRDs`` value VCFNRD
    reads from ``bcftools stats``, t/VCFComp.pm:116-131): with genotypes as
    alt-allele counts, the calls where truth and test differ divided by all
    calls except those homozygous reference in both; calls missing in either
    are skipped.  Inputs are GT alleles [N][S][2] over the same samples and
    sites."""
    t = np.asarray(truth_gt)
    q = np.asarray(test_gt)
    if t.shape != q.shape:
        raise ValueError(f"genotype arrays differ in shape: {t.shape} vs {q.shape}")
    ok = (t >= 0).all(axis=-1) & (q >= 0).all(axis=-1)
    dt = t.sum(axis=-1)[ok]
    dq = q.sum(axis=-1)[ok]
    considered = ~((dt == 0) & (dq == 0))
    total = int(considered.sum())
    if total == 0:
        return 0.0
    return 100.0 * int((dt != dq).sum()) / total


def hap_match(test_gt: np.ndarray, expected_gt: np.ndarray) -> str | None:
    """The haplotype comparison of the reference's regression tests
    (``VCFHapMatch`` / ``HapEq``, t/VCFComp.pm:48-114): site by site, each
    sample's two haplotypes must equal the expected ones, or the expected
    ones swapped; a sample is swapped for good at its first mismatch on its
    first haplotype, and any other mismatch fails.  Inputs are GT alleles
    [N][S][2].  Returns None on a match, else the reason."""
    t = np.asarray(test_gt)
    e = np.asarray(expected_gt)
    if t.shape[1] != e.shape[1]:
        return "hap files have different lengths"
    if t.shape[0] != e.shape[0]:
        return "hap files have differing number of haps"
    if t.shape[0] == 0:
        return "hap files have 0 haplotypes"
    flipped = [False] * t.shape[0]
    for m in range(t.shape[1]):
        for i in range(t.shape[0]):
            for j in range(2):
                while t[i, m, j] != e[i, m, (1 - j) if flipped[i] else j]:
                    if not flipped[i] and j == 0:
                        flipped[i] = True
                        continue
                    return (f"Haplotypes do not match at line {m + 1}, at Allele number "
                            f"{2 * i + j + 1}")
    return None


def nrd_matched(truth_names, truth_sites: Sites, truth_gt: np.ndarray,
                test_names, test_sites: Sites, test_gt: np.ndarray) -> tuple[float, int, int]:
    """``nrd`` over what two call sets share, as ``bcftools stats A B -s
    <A's samples>`` pairs them: samples by name, sites by chrom, position,
    ref and alt.  Returns (NRD percent, shared samples, shared sites)."""
    ti = {n: i for i, n in enumerate(test_names)}
    si = {k: i for i, k in enumerate(zip(test_sites.chrom, test_sites.pos, test_sites.ref,
                                         test_sites.alt))}
    sites = [(j, si[k]) for j, k in enumerate(zip(truth_sites.chrom, truth_sites.pos,
                                                   truth_sites.ref, truth_sites.alt))
             if k in si]
    samples = [(i, ti[n]) for i, n in enumerate(truth_names) if n in ti]
    if not sites or not samples:
        return 0.0, len(samples), len(sites)
    tr = np.asarray(truth_gt)[np.ix_([a for a, _ in samples], [a for a, _ in sites])]
    te = np.asarray(test_gt)[np.ix_([b for _, b in samples], [b for _, b in sites])]
    return nrd(tr, te), len(samples), len(sites)


def dosages(gt: np.ndarray) -> np.ndarray:
    """Alt-allele counts [N][S] of GT alleles (-1 where missing)."""
    g = np.asarray(gt)
    return np.where((g >= 0).all(axis=-1), g.sum(axis=-1), -1)
