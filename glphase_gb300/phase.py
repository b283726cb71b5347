"""End-to-end phasing on one GPU: the generation loop of ``Insti::estimate``
(src/insti.cpp:1557-1728) around the device hot path, with the reference's
input and output formats either side (``io``).

Generation g of B + I + M (simulated-annealing burn-in ``-B``, plain
burn-in ``-i``, sampling ``-m``) runs with pen = min((g + 1)/B, 1)^2
(insti.cpp:1670-1671): one device generation -- surrogates drawn in the
kernel, the MH chains, hmm_work -- then the haplotype swap
(insti.cpp:1455).  From generation B + I on, the device tallies add the new
haplotypes (``Impute::replace``, impute.cpp:564-595, insti.cpp:1710-1712);
after the last generation they become the allele probabilities
(``Impute::result``, impute.cpp:599-613) that the VCF writer calls
genotypes from.  Everything stays on the device between generations; only
the final probabilities and haplotypes come back.

The surrogate sampler is uniform over all other haplotypes
(``UnifSampler``), or, from generation ``cluster_start`` on, the K nearest
haplotypes by Hamming distance built on the device from the haplotypes of
that generation (``KNN``, kNN.cpp:99-206); with ``recluster`` = r > 0 the
table is rebuilt from the current haplotypes at every generation g > B + I
with (g - B - I) mod r = 0 (the reference's ``-r``, insti.cpp:1675-1684).
The reference builds its first table from a pre-phased scaffold
(insti.cpp:1576-1586); without one, the first table here comes from the
haplotypes of generation ``cluster_start``.  With reference-panel rows after
the 2N sample haplotypes, ``kick_start`` draws generation 0's surrogates
from the panel only (the README's kick-start) and ``kick_first`` every
chain's first proposal in every generation (the code's ``--kickstart``,
insti.cpp:1505-1511).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import io as gio
from . import model as mdl
from .batch import anneal_pen
from .hmmlike import Engine


@dataclass
class PhaseOptions:
    sa_burnin: int = 5        # -B: generations with the annealed penalty
    burnin: int = 5           # -i: further burn-in generations at pen = 1
    sampling: int = 20        # -m: generations whose haplotypes are tallied
    cycles: int = 100         # -C: MH proposals per sample and generation
    seed: int = 1             # seeds the device's counter-based draws
    knn: int = 0              # K nearest-neighbour surrogates (0: uniform)
    cluster_start: int = 0    # generation from which the kNN sampler is used
    recluster: int = 0        # -r: rebuild the kNN table every r generations after burn-in
    knn_metric: str = "hamming"  # or "tract": -T, common sites minus the longest shared tract
    lanes: int = 0            # speculation width (0: chosen per generation)
    kick_start: bool = False  # generation 0 draws its surrogates from the panel rows only
    kick_first: bool = False  # every chain's first proposal from the panel (--kickstart)
    device: int = 0

    @property
    def generations(self) -> int:
        return self.sa_burnin + self.burnin + self.sampling


def knn_builds(opts: PhaseOptions) -> list[int]:
    """Generations at whose start the kNN table is built from the current
    haplotypes: every g > bn with (g - bn) mod r = 0 for bn = B + I and r =
    ``recluster`` (insti.cpp:1675-1677: not at bn itself), and
    ``cluster_start`` when no table exists by then."""
    if not opts.knn:
        return []
    bn = opts.sa_burnin + opts.burnin
    out = []
    for g in range(opts.generations):
        rebuild = opts.recluster > 0 and g > bn and (g - bn) % opts.recluster == 0
        if rebuild or (g >= opts.cluster_start and not out):
            out.append(g)
    return out


def phase(model: mdl.Model, haps: np.ndarray, opts: PhaseOptions):
    """Run all generations for ``model`` from the packed starting haplotypes
    ``haps`` (uint64 [H][wn], H >= 2N).  Returns (prob [S][2N] float32,
    final haplotypes uint64 [H][wn])."""
    import torch
    if opts.sampling < 1:
        raise ValueError("at least one sampling generation is required")
    N, S = model.N, model.S
    eng = Engine(model.emit, model.t, model.tran, model.pc, haps, opts.cycles,
                 device=opts.device, lanes=opts.lanes)
    dev, L = eng.dev, eng.dev.L
    hsum = torch.zeros(2 * N * S, dtype=torch.int32, device=eng.device)
    prob = torch.zeros(2 * N * S, dtype=torch.float32, device=eng.device)
    torch.cuda.current_stream(eng.device).synchronize()
    tallied_from = opts.sa_burnin + opts.burnin
    builds = set(knn_builds(opts))
    nbr = table = None
    for g in range(opts.generations):
        if g in builds:
            table = eng.knn(opts.knn, metric=opts.knn_metric)
        # the table is the sampler from cluster_start on
        nbr = table if opts.knn and g >= opts.cluster_start else None
        pen = float(anneal_pen(g, opts.sa_burnin))
        a = eng.args(None, None, pen, opts.seed, g, neighbors=nbr,
                     kick_first=opts.kick_first and eng.H > 2 * N)
        if opts.kick_start and g == 0 and eng.H > 2 * N:
            a.sample_lo, a.sample_hi, a.kick_start = 2 * N, eng.H, 1
        eng.launch(a)
        eng.swap()
        if g >= tallied_from:
            dev._c(L.glp_tally(dev.ctx, eng.haps.data_ptr(), N, S, hsum.data_ptr()))
    dev._c(L.glp_result(dev.ctx, hsum.data_ptr(), N, S, opts.sampling, prob.data_ptr()))
    eng.finish()
    out = prob.cpu().numpy().reshape(S, 2 * N)
    final = eng.haps.cpu().numpy().view(np.uint64).reshape(haps.shape)
    dev.cleanup()
    return out, final


def prepare(gl_het_alt: np.ndarray, positions: np.ndarray,
            genetic_map: gio.GeneticMap | None = None, seed: int = 1):
    """Model constants (``Insti::initialize``, insti.cpp:1254-1380) and the
    starting haplotypes drawn from the GLs (insti.cpp:1353-1372): with a
    genetic map the recombination fractions come from it, otherwise from
    the site density.  Returns (model, packed haplotypes [2N][wn])."""
    if genetic_map is not None:
        m = mdl.Model(gl_het_alt, r_morgans=genetic_map.distances(positions))
    else:
        m = mdl.Model(gl_het_alt, positions=np.asarray(positions))
    rng = np.random.default_rng(seed)
    return m, mdl.pack_haplotypes(mdl.initial_haplotypes(m.t, rng))


def phase_bin(bin_path: str, vcf_path: str | None = None, map_path: str | None = None,
              opts: PhaseOptions | None = None, keep: set[str] | None = None,
              command_line: str = "", region: str | tuple[str, int, int] | None = None,
              ref_legend: str | None = None, ref_hap: str | None = None):
    """Phase the samples of a GL file and (optionally) write the phased VCF:
    ``insti -g map -C.. -B.. -i.. -m.. [--region chr:a-b] [-h hap -l legend]
    file.bin`` (or ``-Fbcf file.vcf.gz``) on one GPU.  ``.vcf`` / ``.vcf.gz``
    files are read for their GL or PL field, anything else as ``.bin``;
    ``region`` ("chr:first-last" as ``--region`` takes it, or a (chrom,
    first, last) tuple) keeps the sites inside it; a reference
    panel (legend + hap) becomes the haplotype rows after the 2N sample
    rows.  Returns (prob [S][2N], the parsed input)."""
    opts = opts or PhaseOptions()
    if isinstance(region, str):
        region = gio.parse_region(region)
    if bin_path.endswith((".vcf", ".vcf.gz")):
        data = gio.read_vcf_gls(bin_path, keep=keep, region=region)
    else:
        data = gio.read_bin(bin_path, keep=keep, region=region)
    gmap = gio.read_genetic_map(map_path) if map_path else None
    m, haps = prepare(data.gl, data.sites.positions(), gmap, seed=opts.seed)
    if ref_legend or ref_hap:
        if not (ref_legend and ref_hap):
            raise ValueError("a reference panel needs both a legend and a hap file")
        panel = gio.load_reference_panel(ref_legend, ref_hap, data.sites)
        haps = np.concatenate([haps, panel])
    prob, _ = phase(m, haps, opts)
    if vcf_path:
        gio.write_vcf(vcf_path, data.sites, data.names, prob, command_line=command_line)
    return prob, data
