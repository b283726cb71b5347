#!/usr/bin/env python3
"""Benchmark of the GB300 MH/HMM phasing hot path.

One step = one MH generation over all samples of the workload: C+1
likelihood evaluations per sample (initial quadruple plus C proposals) over
S sites, the MH accept chain, and the fused hmm_work haplotype sampling,
exactly the work of GLPhase's RunHMMOnDevice + hmm_work loop
(src/hmmLike.cu:399-572, src/insti.cpp:1433-1463).  Metric: HMM site-updates
per second, one update = one (sample, proposal, site) forward step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Default workload: 10,000 samples x 4,096 sites, C = 100 (the batched
configuration), seeded synthetic data generated on the host.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FLOPS_PER_UPDATE = 29  # impute.cpp:354-373: 12 mul + 8 add (b terms), 2 pair sums, 4 emission muls, 3 adds
METRIC = "HMM site-updates/s (sample x proposal x site)"
UNIT = "site-updates/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", default="batched")
    ap.add_argument("--samples", type=int, default=0, help="override N (tests)")
    ap.add_argument("--sites", type=int, default=0, help="override S (tests)")
    ap.add_argument("--cycles", type=int, default=100)
    ap.add_argument("--lanes", type=int, default=0, help="lanes per sample (0 = auto)")
    ap.add_argument("--block-sites", type=int, default=0,
                    help="sites per normalisation block (8, 4; 0 = auto)")
    ap.add_argument("--vq", action="store_true", help="score with 4-bit VQ GL codes")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the untimed full-schedule phasing accuracy run")
    ap.add_argument("--knn-metric", choices=["hamming", "tract"], default="hamming",
                    help="kNN distance: Hamming, or the common sites minus the longest "
                         "shared tract (insti -T)")
    ap.add_argument("--recluster", type=int, default=0,
                    help="kNN configurations: rebuild the neighbour table from the current "
                         "haplotypes every R generations after burn-in, inside the timed "
                         "steps (the reference's -r; 0 = its default, never)")
    ap.add_argument("--uniform", action="store_true",
                    help="uniform surrogates instead of the configuration's kNN restriction")
    ap.add_argument("--chunks", type=int, default=64, help="uneven workload: chunk count")
    ap.add_argument("--scale", type=float, default=1.0, help="uneven workload: shrink shapes")
    ap.add_argument("--requests", type=int, default=24, help="serving: request count")
    ap.add_argument("--generations", type=int, default=32, help="serving: generations/request")
    ap.add_argument("--budget-gb", type=float, default=180.0, help="serving: HBM budget")
    ap.add_argument("--serve-limit", type=float, default=600.0)
    ap.add_argument("--no-vs-plain", action="store_true",
                    help="skip the uneven-chunk batched-vs-plain leg of the default line")
    ap.add_argument("--no-serve", action="store_true",
                    help="skip the serving p50/p99 leg of the default line")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def workload(args, rank):
    """This rank's chunk: replicas phase independent chunks (weak scaling)."""
    from glphase_gb300 import replicas, synth
    w = synth.CONFIGS[args.config]
    N = args.samples or w.N
    S = args.sites or w.S
    rp = replicas.plan(w.seed, rank=rank, world=max(rank + 1, dist_env()[0]))
    ds = synth.generate(w, N=N, S=S, seed=rp.data_seed)
    m, haps = synth.initial_state(ds, seed=7 + rank)
    workload.dataset = ds
    return w, m, haps


def knn_k(w, args, H):
    """Neighbours per haplotype of the configuration's kNN sampler, capped
    at what H haplotypes allow (reduced test sizes); 0 = uniform sampler."""
    if not w.knn or args.uniform:
        return 0
    return min(w.knn, (H - 2) // 2 * 2)


def sampler_name(K, metric="hamming"):
    if K:
        by = ("Hamming distance" if metric == "hamming" else
              "common sites minus the longest shared tract (-T)")
        return f"the K={K} nearest haplotypes by {by} (KNN::ClusterHaps)"
    return "uniform over all other haplotypes (UnifSampler)"


def workload_config(args, w, N, S, C, H):
    """The workload definition both arms report under `config` (the arms
    differ in how they run it, which each line says outside `config`)."""
    sampler = sampler_name(knn_k(w, args, H), args.knn_metric)
    K = knn_k(w, args, H)
    rc = (f", rebuilt from the current haplotypes every {args.recluster} generations after "
          f"burn-in" if K and args.recluster else "")
    return {"workload": f"{args.config}: {N} samples x {S} sites x C={C} cycles per "
                        f"generation, surrogates from {sampler}{rc}",
            "samples": N, "sites": S, "cycles": C, "haplotypes": H, "sampler": sampler,
            "recluster_every": args.recluster if K else 0,
            "knn_metric": args.knn_metric if K else None,
            "emission": "vq4" if args.vq else "f32",
            "l2": "inputs larger than L2 (emission %.0f MB)" % (N * S * 16 / 1e6)}


def cpu_model():
    """The host CPU's model name (lscpu; /proc/cpuinfo as a fallback)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def accuracy(w, m, haps, ds, seed, device, recluster=0, knn_metric="hamming"):
    """Phasing accuracy of the workload's full schedule (burn-in + sampling
    generations, the configuration's surrogate sampler, device tallies and
    result; glphase_gb300.phase): NRD of the called genotypes against the
    synthetic truth, beside the NRD of calling each genotype from its GLs
    alone.  Not timed."""
    from glphase_gb300 import io as gio, phase as ph
    N = m.N
    opts = ph.PhaseOptions(sa_burnin=w.burnin, burnin=0, sampling=w.sampling, cycles=w.cycles,
                           seed=seed, knn=w.knn, cluster_start=0, recluster=recluster,
                           knn_metric=knn_metric,
                           kick_start=bool(w.panel_haps), kick_first=bool(w.panel_haps),
                           device=device)
    prob, _ = ph.phase(m, haps, opts)
    truth = np.stack([ds.truth[0:2 * N:2], ds.truth[1:2 * N:2]], axis=-1).astype(np.int8)
    call = np.argmax(m.t, axis=-1)
    gl_only = np.stack([call >= 1, call == 2], axis=-1).astype(np.int8)
    return {"nrd_percent": round(gio.nrd(truth, gio.genotype_calls(prob)), 3),
            "nrd_gl_only_percent": round(gio.nrd(truth, gl_only), 3),
            "generations": opts.generations,
            "sampler": f"kNN K={w.knn}" if w.knn else "uniform",
            "truth": "synthetic haplotypes the GLs were simulated from"}


# DRAM bytes (read + write) of one generation_kernel launch measured by ncu on
# the batched workload itself (N = 10,000, S = 4,096, C = 100, 8 lanes, float
# emission), one launch, no scaling: every speculative round streams its
# sample's emission row again, mostly from DRAM.
NCU_TRAFFIC_BATCHED = 18.977837568e9 + 0.004564480e9


def traffic_per_launch(N, S, C, args):
    if (N, S, C) != (10000, 4096, 100) or args.vq or args.config != "batched":
        return None
    return NCU_TRAFFIC_BATCHED


def hbm_roofline(N, S, H, wn, kernel_ms, traffic, args):
    """The same kernel against the measured HBM copy bandwidth: compulsory
    bytes of one generation kernel launch (every sample's emission rows read
    once, 16 B a site, and the haplotype panel, H x wn words) over its time.
    The kernel re-reads a sample's emission every speculative round, mostly
    from L2; `traffic` is what reached DRAM."""
    peak = None
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        try:
            peak = float(json.load(open(path))["hbm_gbs"])
        except (ValueError, KeyError):
            peak = None
    if peak is None:
        peak = 6800.0
        src = "fallback"
    else:
        src = "measured"
    algo = N * S * 16 + H * wn * 8
    achieved = algo / (kernel_ms * 1e-3) / 1e9
    out = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
           "frac": achieved / peak, "traffic": traffic,
           "note": f"achieved = compulsory bytes ({algo} per launch) over the kernel time; "
                   f"peak = {src} HBM copy bandwidth; traffic = measured DRAM bytes of one "
                   "launch (every speculative round streams its sample's emission row "
                   "again); the kernel is bound by instruction issue (roofline)"}
    if traffic:
        out["traffic_gbs"] = traffic / (kernel_ms * 1e-3) / 1e9
        out["traffic_frac"] = out["traffic_gbs"] / peak
    return out


def pen_for(gen, burnin):
    """Annealing penalty of generation gen (insti.cpp:1670-1671), binary32."""
    from glphase_gb300.batch import anneal_pen
    return float(anneal_pen(gen, burnin))


def surrogates(seed, gen, N, C, H, nbr):
    """The surrogates the kernel draws for generation gen, materialised on
    the host for the CPU reference (same counter-based streams)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    return O.sample_surrogates(seed, gen, N, C, 0, H, nbr=nbr)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        self.gpu = gpu_index
        self.path = tempfile.mktemp(suffix=".csv")

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def cpu_baseline(m, haps, quad, props, C, pen, seconds, seed=1, gen=0):
    """The CPU oracle (reference operation order, OpenMP over samples) on a
    bounded number of samples of one generation."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build(ref=False)
    threads = os.cpu_count() or 1
    pb = O.OracleProblem(haps, m.emit, m.t, m.tran, m.pc, C)
    tr = pb.trace(seed=seed, generation=gen)
    n = min(m.N, max(threads * 2, 16))
    t0 = time.perf_counter()
    O.generation(pb, tr, quad, props, pen, 0, n, True, nthreads=threads)
    dt = time.perf_counter() - t0
    n2 = int(min(m.N, max(n, n * seconds / max(dt, 1e-6))))
    t0 = time.perf_counter()
    O.generation(pb, tr, quad, props, pen, 0, n2, True, nthreads=threads)
    dt = time.perf_counter() - t0
    ups = n2 * (C + 1) * m.S / dt
    # the same on one thread, over about one second's worth of samples
    n1 = int(min(m.N, max(1, n2 / max(dt * threads, 1e-9))))
    t0 = time.perf_counter()
    O.generation(pb, tr, quad, props, pen, 0, n1, True, nthreads=1)
    dt1 = time.perf_counter() - t0
    return {"value": ups, "unit": UNIT, "cores": threads, "kind": "port",
            "cpu_model": cpu_model(),
            "sample": f"{n2} of {m.N} samples of one generation (C={C}, S={m.S}), "
                      f"{dt:.1f} s on {threads} host threads",
            "single_thread_value": n1 * (C + 1) * m.S / dt1,
            "single_thread_sample": f"{n1} samples, {dt1:.1f} s on 1 thread"}, dt


def run_reference(args):
    """The reference's CPU path (the oracle port: impute.cpp's hmm_like and
    hmm_work in their operation order, OpenMP over samples) on the same
    workload and the same surrogate sampler as the GPU arm: for the kNN
    configurations the neighbour table of the starting haplotypes is built by
    the oracle's KNN::ClusterHaps restatement, and every generation draws its
    surrogates from it with the GPU arm's counter-based streams.  The table
    and the draws are set-up, outside the timed region."""
    world, rank, local = dist_env()
    if rank != 0:
        return
    w, m, haps = workload(args, 0)
    C = args.cycles
    N, S = m.N, m.S
    H = haps.shape[0]
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build(ref=False)
    nbr, knn_s = None, None
    K = knn_k(w, args, H)
    if K:
        t0 = time.perf_counter()
        nbr = np.ascontiguousarray(O.knn(haps, S, K, metric=args.knn_metric)[:N])
        knn_s = time.perf_counter() - t0
    seed = 1
    q0, p0 = O.sample_surrogates(seed, 0, N, C, 0, H, nbr=nbr)
    per_step = max(args.cpu_seconds / max(args.steps, 1), 1.0)
    base, _ = cpu_baseline(m, haps, q0, p0, C, 1.0, per_step)
    threads = base["cores"]
    pb = O.OracleProblem(haps, m.emit, m.t, m.tran, m.pc, C)
    n = int(base["sample"].split()[0])

    def gen(g, count):
        quad, props = O.sample_surrogates(seed, g, N, C, 0, H, nbr=nbr)
        return quad, props, pb.trace(seed=seed, generation=g), pen_for(g, w.burnin), count

    def rebuild(g):
        return K and args.recluster and g > w.burnin and (g - w.burnin) % args.recluster == 0

    for g in range(args.warmup):
        quad, props, tr, pen, cnt = gen(g, min(n, 2 * threads))
        O.generation(pb, tr, quad, props, pen, 0, cnt, True, nthreads=threads)
    dt = 0.0
    for i in range(args.steps):
        g = args.warmup + i
        t0 = time.perf_counter()
        if rebuild(g):  # KNN::ClusterHaps on the haplotypes, as the timed GPU step does
            nbr = np.ascontiguousarray(O.knn(haps, S, K, metric=args.knn_metric)[:N])
        dt += time.perf_counter() - t0
        quad, props, tr, pen, cnt = gen(g, n)
        t0 = time.perf_counter()
        O.generation(pb, tr, quad, props, pen, 0, cnt, True, nthreads=threads)
        dt += time.perf_counter() - t0
    value = args.steps * n * (C + 1) * S / dt
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "impl": "reference",
        "config": workload_config(args, w, N, S, C, H),
        "reference_path": "oracle port of the reference CPU path (impute.cpp:327-485, "
                          "MHSampler.hpp:81-96), all host threads; surrogate table "
                          + ("built by the oracle's KNN::ClusterHaps in %.1f s, " % knn_s
                             if knn_s is not None else "")
                          + "draws per generation outside the timed region"
                          + (", rebuilds of the table inside it" if K and args.recluster else ""),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "cpu_model": base["cpu_model"],
                         "sample": f"{n} of {N} samples per step, {args.steps} steps",
                         "single_thread_value": base["single_thread_value"],
                         "single_thread_sample": base["single_thread_sample"]},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import ctypes as C_
    import torch
    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from glphase_gb300 import native as nat, replicas, synth
    from glphase_gb300.hmmlike import Engine

    w, m, haps = workload(args, rank)
    C = args.cycles
    N, S = m.N, m.S
    H, wn = haps.shape
    packed = codebook = None
    if args.vq:
        # the codebook trained and the codes packed by the device codec (bit
        # for bit the host GLPack's result, in a fraction of a second)
        from glphase_gb300.glpack import GLPack
        from glphase_gb300.hmmlike import HMMLikeCUDA
        codec = HMMLikeCUDA(local)
        try:
            gp = GLPack(m.t, np.random.default_rng(1), device=codec)
            packed, codebook = gp.packed_gls(), gp.code_book()
        finally:
            codec.cleanup()
    eng = Engine(m.emit, m.t, m.tran, m.pc, haps, C, device=local, lanes=args.lanes,
                 packed=packed, codebook=codebook,
                 block_sites=args.block_sites)
    dev = torch.device("cuda", local)
    torch.cuda.synchronize()
    # surrogate restriction: the K nearest haplotypes by Hamming distance
    # (KNN::ClusterHaps) computed once on the device from the starting
    # haplotypes; every generation then draws its surrogates in the kernel
    nbr, knn_ms = None, None
    K = knn_k(w, args, H)
    if K:
        k0 = torch.cuda.Event(enable_timing=True)
        k1 = torch.cuda.Event(enable_timing=True)
        k0.record(eng.stream)
        nbr = eng.knn(K, metric=args.knn_metric)
        k1.record(eng.stream)
        eng.finish()
        knn_ms = k0.elapsed_time(k1)
    peak = C_.c_double()
    eng.dev._c(eng.dev.L.glp_measure_fp32_peak(eng.dev.ctx, 200.0, C_.byref(peak)))
    stream = eng.stream
    seed = replicas.plan(w.seed, rank=rank, world=max(world, rank + 1)).rng_seed

    rebuilds = [0]

    def step(g):
        nonlocal nbr
        if nbr is not None and args.recluster and g > w.burnin and \
                (g - w.burnin) % args.recluster == 0:
            nbr = eng.knn(K, metric=args.knn_metric)  # from the current haplotypes
            rebuilds[0] += 1
        a = eng.args(None, None, pen_for(g, w.burnin), seed=seed, generation=g, neighbors=nbr)
        if w.panel_haps and g == 0:
            # the first generation draws its surrogates from the panel only
            a.sample_lo, a.sample_hi, a.kick_start = 2 * N, H, 1
        eng.launch(a)
        eng.swap()

    for g in range(args.warmup):
        step(g)
    eng.finish()
    rebuilds[0] = 0
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.4)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    evs[0].record(stream)
    for i in range(args.steps):
        step(args.warmup + i)
        evs[i + 1].record(stream)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ck = clocks.stop()
    eng.finish()
    per = [evs[i].elapsed_time(evs[i + 1]) for i in range(args.steps)]
    elapsed = evs[0].elapsed_time(evs[-1]) / 1e3
    ev, rounds, lanes = eng.dev.stats()
    cnt = eng.dev.counters()
    elapsed = replicas.max_elapsed(elapsed, device=dev)
    updates_step = N * (C + 1) * S
    value = world * args.steps * updates_step / elapsed
    step_ms = float(np.mean(per))
    # device time of the generation kernel itself (CUDA events the library
    # records around it on the same stream) and of the hmm_work kernels
    gen_t, work_t = eng.dev.kernel_times(args.steps)
    kernel_ms = float(np.mean(gen_t))
    work_ms = float(np.mean(work_t))
    achieved = updates_step * FLOPS_PER_UPDATE / (kernel_ms * 1e-3) / 1e12

    nbr_host = None if nbr is None else np.ascontiguousarray(
        nbr.cpu().numpy().view(np.uint32)[:N])
    # the end-to-end and CPU legs, like the legs after the line's main
    # figures, record an error in the line rather than cost it
    e2e = None
    if not args.no_e2e:
        e2e = extra_leg(lambda: run_e2e(eng, haps, N, S, C, H, wn, w, args, torch, nbr_host))

    base = None
    if rank == 0 and not args.no_cpu_baseline:
        def cpu_leg():
            # the same surrogates the kernel draws, at full penalty
            q0, p0 = surrogates(seed, args.warmup, N, C, H, nbr_host)
            return cpu_baseline(m, haps, q0, p0, C, 1.0, args.cpu_seconds)[0]
        base = extra_leg(cpu_leg)
    sm_count = torch.cuda.get_device_properties(local).multi_processor_count

    if rank == 0:
        sm_mhz = ck.get("sm_mhz")
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": elapsed / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": workload_config(args, w, N, S, C, H),
            "surrogates": ("neighbour table built once on the device from the starting "
                           f"haplotypes ({knn_ms:.1f} ms), drawn in the kernel"
                           if nbr is not None else "drawn in the kernel"),
            "parallelism": f"replicas x{world}" if world > 1 else "1 GPU",
            "speculation": {
                "lanes_per_sample": lanes,
                "positions_per_round": lanes // 2,
                "evaluations_per_step": ev,
                "speculative_rounds": rounds,
                "site_by_site_redos": cnt[3],
                "block_sites": eng.dev.block_sites(),
                "lane_occupancy": round(cnt[5] / max(32 * cnt[4], 1), 4),
                # lane-pair rounds run per counted evaluation: above 1 by the
                # pairs of a chain's last round that score past its end
                "pair_rounds_per_evaluation": round(cnt[5] / 2 / max(cnt[0], 1), 4),
                "useful_fraction": round(N * (C + 1) / max(ev, 1), 4)},
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak.value,
                         "unit": "TFLOP/s", "frac": achieved / peak.value if peak.value else None,
                         "traffic": traffic_per_launch(N, S, C, args),
                         "peak_basis": {
                             "sms": sm_count, "sm_mhz_median": sm_mhz,
                             "fp32_lanes_per_sm": 128,
                             "lanes_x_sms_x_2_x_clock_tflops":
                                 128 * sm_count * 2 * sm_mhz * 1e6 / 1e12 if sm_mhz else None},
                         "note": "29 algorithmic FP32 flops per update over the generation "
                                 "kernel's CUDA-event time; peak = FP32 FMA rate measured on "
                                 "this GPU (glp_measure_fp32_peak, dependent-free FMA chains on "
                                 "every SM); traffic = DRAM bytes of one launch of this "
                                 "workload from one ncu capture"},
            "roofline_hbm": hbm_roofline(N, S, H, wn, kernel_ms, traffic_per_launch(N, S, C, args),
                                         args),
            "clocks": ck,
            "gpu_launches": 3 * args.steps + 2 * rebuilds[0],
            "step_ms": step_ms,
            "kernel_ms": kernel_ms,
            "hmm_work_ms": work_ms,
        }
        if e2e:
            line["e2e"] = e2e
        if base:
            line["cpu_baseline"] = base
        # The legs after the timed steps add to the line; one that fails
        # records its error there instead of costing the line.
        if not args.no_accuracy:
            line["accuracy"] = extra_leg(lambda: accuracy(w, m, haps, workload.dataset, seed,
                                                          local, args.recluster,
                                                          args.knn_metric))
        if world == 1 and args.config == "batched" and not (args.no_vs_plain and args.no_serve):
            # the metric's other halves, on the same GPU after the main leg:
            # batched vs plain GPU form on the uneven chunks, p50/p99 serving
            del eng
            torch.cuda.empty_cache()
            if not args.no_vs_plain:
                line["vs_plain"] = extra_leg(lambda: measure_uneven(args, 4, 2)[0])
            if not args.no_serve:
                line["serving"] = extra_leg(lambda: serving_summary(args))
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def extra_leg(fn):
    """Result of a leg measured after the timed steps, or {"error": ...} when
    it raised (the exception is also printed to stderr)."""
    try:
        return fn()
    except Exception as e:  # noqa: BLE001 - reported in the line and on stderr
        import traceback
        traceback.print_exc()
        return {"error": f"{type(e).__name__}: {e}"}


def serving_summary(args):
    """Serving at 1x the measured capacity, batched and plain, for the
    default line: p50/p99 request latency and throughput of both forms."""
    sv = measure_serve(args, ((1.0, False, False), (1.0, True, False)))
    b1, p1 = sv["results"]["batched@1.0x"], sv["results"]["plain@1.0x"]
    return {"p50_latency_s": b1["p50_latency_s"], "p99_latency_s": b1["p99_latency_s"],
            "updates_per_s": b1["updates_per_s"], "load": "1x measured capacity",
            "plain_p50_latency_s": p1["p50_latency_s"],
            "plain_p99_latency_s": p1["p99_latency_s"],
            "plain_updates_per_s": p1["updates_per_s"],
            "batched_over_plain": b1["updates_per_s"] / max(p1["updates_per_s"], 1e-9),
            **{k: sv[k] for k in ("workload", "capacity_updates_per_s",
                                  "capacity_requests_per_s")}}


def run_e2e(eng, haps, N, S, C, H, wn, w, args, torch, nbr_host):
    """Same metric through the host-pointer C-ABI call: every step copies the
    haplotypes (and the kNN table, when used) in from pinned host memory and
    the quadruples, the new haplotype rows and the log-likelihoods back; the
    surrogates are drawn in the kernel as in the device-resident run."""

    def pinned(shape, dtype):
        t = torch.empty(shape, dtype=dtype, pin_memory=True)
        return t.numpy()

    h = pinned((H, wn), torch.int64).view(np.uint64)
    h[:] = haps
    hn = pinned((H, wn), torch.int64).view(np.uint64)
    hn[:] = haps
    nb = None
    if nbr_host is not None:
        nb = pinned(nbr_host.shape, torch.int32).view(np.uint32)
        nb[:] = nbr_host
    qout = pinned((4, N), torch.int32).view(np.uint32)
    like = pinned((N,), torch.float64)
    cur, nxt = h, hn
    for g in range(args.warmup):
        eng.run_host(cur, None, None, pen_for(g, w.burnin), 99, g, nxt, qout, like, nb)
        nxt[2 * N:] = cur[2 * N:]
        cur, nxt = nxt, cur
    t0 = time.perf_counter()
    for i in range(args.steps):
        g = args.warmup + i
        eng.run_host(cur, None, None, pen_for(g, w.burnin), 99, g, nxt, qout, like, nb)
        cur, nxt = nxt, cur
    dt = time.perf_counter() - t0
    h2d = H * wn * 8 + (0 if nb is None else nb.nbytes)
    d2h = 4 * N * 4 + 2 * N * wn * 8 + N * 8
    return {"value": args.steps * N * (C + 1) * S / dt, "unit": UNIT,
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "api": "glp_run_generation_host (pinned host buffers)"}


def uneven_shapes(n_chunks, seed=4, scale=1.0):
    """Chunk shapes of the uneven workload: sites ~ U{512..16384} in steps of
    64, samples ~ U{100..5000} (scale < 1 shrinks both for tests)."""
    rng = np.random.default_rng(seed)
    S = 64 * rng.integers(8, 257, n_chunks)
    N = rng.integers(100, 5001, n_chunks)
    if scale != 1.0:
        S = np.maximum(64, (S * scale).astype(int) // 64 * 64)
        N = np.maximum(4, (N * scale).astype(int))
    return [(int(n), int(s)) for n, s in zip(N, S)]


def measure_uneven(args, steps, warmup):
    """Batched (one persistent launch per generation, replayed CUDA graph)
    vs plain (one launch per chunk) on the uneven-chunk workload; returns the
    measurements and the clock record of the batched leg."""
    import torch
    from glphase_gb300 import synth, synth_device as sd
    from glphase_gb300.batch import DeviceProblem, PreparedBatch
    from glphase_gb300.hmmlike import HMMLikeCUDA
    C = args.cycles
    shapes = uneven_shapes(args.chunks, scale=args.scale)
    dev = HMMLikeCUDA(0)
    dev.set_lanes_per_sample(args.lanes)
    stream = torch.cuda.Stream()
    dev._c(dev.L.glp_set_stream(dev.ctx, stream.cuda_stream))
    probs = []
    t0 = time.perf_counter()
    for i, (N, S) in enumerate(shapes):
        w = synth.Workload(f"chunk{i}", N=N, S=S, founders=40, depth=4.0, burnin=8,
                           sampling=24, seed=100 + i)
        probs.append(DeviceProblem(dev, sd.generate(w, N, S, seed=100 + i), C,
                                   seed=5000 + i, burnin=8))
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    upd = sum(N * (C + 1) * S for N, S in shapes)

    def timed(fn, n):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(n):
            fn()
        e1.record(stream)
        e1.synchronize()
        dev._c(dev.L.glp_finish(dev.ctx))
        return e0.elapsed_time(e1) / 1e3

    batch = PreparedBatch(dev, probs, generation=0)
    for _ in range(warmup):
        batch.run()
    dev._c(dev.L.glp_finish(dev.ctx))
    clocks = ClockSampler(0)
    clocks.start()
    t_batched = timed(batch.run, steps)
    ck = clocks.stop()
    _, _, lanes_b = dev.stats()
    cnt_b = dev.counters()
    gen = batch.generation
    batch.close()
    singles = [PreparedBatch(dev, [p], generation=gen) for p in probs]

    def plain():
        for sg in singles:
            sg.run(graph=False)
    plain()
    dev._c(dev.L.glp_finish(dev.ctx))
    t_plain = timed(plain, steps)
    for sg in singles:
        sg.close()
    for p in probs:
        p.close()
    dev.cleanup()
    v_b = steps * upd / t_batched
    v_p = steps * upd / t_plain
    res = {"workload": f"uneven: {len(shapes)} chunks, sites U{{512..16384}}/64, "
                       f"samples U{{100..5000}}" + (f" scaled by {args.scale}" if args.scale != 1 else "")
                       + f", C={C}, own seed/founders/map each",
           "chunks": len(shapes), "samples_total": int(sum(n for n, _ in shapes)),
           "updates_per_step": upd, "steps": steps, "warmup": warmup,
           "setup_s": round(setup_s, 1),
           "batched": v_b, "plain": v_p, "ratio": v_b / v_p,
           "batched_ms_per_step": t_batched / steps * 1e3,
           "plain_ms_per_step": t_plain / steps * 1e3,
           "lanes_per_sample": lanes_b,
           "accept_rate": round(cnt_b[2] / max(cnt_b[1], 1), 4),
           "useful_fraction": round(sum(N for N, _ in shapes) * (C + 1) / max(cnt_b[0], 1), 4),
           "form": "batched = one persistent launch per generation replayed from a captured "
                   "CUDA graph; plain = one launch per chunk"}
    return res, ck


def run_uneven(args):
    """The uneven-chunk configuration as its own line."""
    res, ck = measure_uneven(args, args.steps, args.warmup)
    line = {
        "metric": METRIC, "value": res["batched"], "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["batched_ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": {"workload": res["workload"]}, "vs_plain": res,
        "clocks": ck, "gpu_launches": 4 * args.steps,
    }
    print(json.dumps(line), flush=True)


def measure_serve(args, legs):
    """Poisson-arriving phasing requests (uneven-chunk shapes, G generations
    each) served with continuous batching.  legs: (load, plain, native)
    triples -- load in multiples of the measured capacity, plain = one launch
    per resident request per tick, native = the library's own loop
    (glp_server_*).  Returns per-leg summaries and the capacity."""
    import torch
    from glphase_gb300 import synth, synth_device as sd
    from glphase_gb300.hmmlike import HMMLikeCUDA
    from glphase_gb300.serve import NativeServer, Request, Server
    C, G = args.cycles, args.generations
    shapes = uneven_shapes(args.requests, seed=9, scale=args.scale)
    dev = HMMLikeCUDA(0)
    dev.set_lanes_per_sample(args.lanes)
    stream = torch.cuda.Stream()
    dev._c(dev.L.glp_set_stream(dev.ctx, stream.cuda_stream))
    budget = int(args.budget_gb * 1e9)

    def make(i, N, S):
        w = synth.Workload(f"req{i}", N=N, S=S, founders=40, depth=4.0, burnin=8,
                           sampling=24, seed=300 + i)
        return Request(rid=i, chunk=sd.generate(w, N, S, seed=300 + i), generations=G,
                       cycles=C, seed=9000 + i, burnin=8)

    # capacity: saturated throughput of 8 requests resident at once
    reqs = [make(i, N, S) for i, (N, S) in enumerate(shapes)]
    mean_updates = float(np.mean([r.updates for r in reqs]))
    cal = Server(dev, budget)
    for r in reqs[:8]:
        r.generations = 2
        cal.submit(r)
    cal.tick(0.0)
    t0 = time.perf_counter()
    cal.tick(0.0)
    per_gen = sum(r.chunk.N * (C + 1) * r.chunk.S for r in reqs[:8])
    capacity_ups = per_gen / (time.perf_counter() - t0)
    capacity_rps = capacity_ups / mean_updates
    del reqs, cal
    results = {}
    for load, plain, native in legs:
        rng = np.random.default_rng(int(load * 100) + plain)
        gaps = rng.exponential(1.0 / (load * capacity_rps), size=len(shapes))
        reqs = [make(i, N, S) for i, (N, S) in enumerate(shapes)]
        for r, a in zip(reqs, np.cumsum(gaps)):
            r.arrival = float(a)
        torch.cuda.synchronize()
        srv = (NativeServer if native else Server)(dev, budget, plain=plain)
        st = srv.serve(reqs, time_limit=args.serve_limit)
        if native:
            srv.close()
        key = ("native" if native else "plain" if plain else "batched") + f"@{load}x"
        results[key] = st.summary()
        del reqs, srv
        torch.cuda.empty_cache()
    dev.cleanup()
    return {"workload": f"serving: {len(shapes)} Poisson-arriving requests, uneven-chunk "
                        f"shapes" + (f" scaled by {args.scale}" if args.scale != 1 else "")
                        + f", {G} generations each, C={C}, panel off",
            "hbm_budget_gb": args.budget_gb, "capacity_updates_per_s": capacity_ups,
            "capacity_requests_per_s": capacity_rps, "results": results}


def run_serve(args):
    """Serving at 0.5x, 1x and 2x the measured capacity; the plain form and
    the library's own serving loop at 1x beside it."""
    res = measure_serve(args, ((0.5, False, False), (1.0, False, False), (2.0, False, False),
                               (1.0, True, False), (1.0, False, True)))
    r = res["results"]
    b1, p1 = r["batched@1.0x"], r["plain@1.0x"]
    res["batched_over_plain_at_1x"] = b1["updates_per_s"] / p1["updates_per_s"]
    res["native_over_python_loop_at_1x"] = r["native@1.0x"]["updates_per_s"] / b1["updates_per_s"]
    line = {
        "metric": "serving: p50/p99 request latency and site-updates/s", "value":
            b1["updates_per_s"], "unit": UNIT, "n_gpus": 1, "steps": args.requests,
        "warmup": 1, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic", "config": {"workload": res["workload"]},
        "serving": res,
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.config == "uneven":
        run_uneven(args)
    elif args.config == "serve":
        run_serve(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
