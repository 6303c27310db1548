"""Benchmark: BUSseq Gibbs sweeps per second on one GB300 (config 1).

Workload (the configuration the headline metric is quoted on): B = 4 batches
of 2500 cells (N = 10^4), G = 10^4 genes, K = 8 cell types, synthetic counts
drawn from the BUSseq generative model (20% differential genes), plain sampler
(the reference's random-walk MH moves and MH cell-type move).

A step is one full Gibbs sweep.  Reported:
  value      sweeps/s with the counts already in HBM, CUDA events on the
             sampler's stream around K graph-launched sweeps (half burn-in, half
             kept, as in the reference's runs); X and Y are 400 MB each, larger
             than L2, so no flush is needed between sweeps.
  e2e        sweeps/s through the public C ABI from pinned host counts: upload,
             initialisation, K sweeps, posterior summaries and the copy of every
             estimate (including the N x G X and Z) back to the host.
  roofline   the dominant kernel's algorithmic bytes per launch over its mean
             CUDA-event duration, against the measured HBM copy bandwidth.
  cpu_baseline the FP64 OpenMP oracle (the CPU restatement of the same sweep)
             on the host cores: 20 full sweeps of the same data, timed as
             they run (no cell sample, no scaling).

--impl reference runs the CPU arm only (the reference program has no CPU
implementation of the sweep, so its CPU stand-in is the oracle port): every
step is one full oracle sweep of the whole workload, timed, unscaled.  Its
input comes from the generator built on the checker side, so that process
never maps the product library.
Multi-GPU (--gpus N under torchrun): N independent chains, one per GPU
(replicas: a BUSseq chain has no data-parallel split that avoids an
all-reduce per sweep).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CFG1 = dict(n_b=[2500, 2500, 2500, 2500], G=10000, K=8, seed=13580)
# the large uneven workload: 6 batches, 15 % differential genes, phi ~ U(2, 30), HMC block
# update (10 leapfrog steps; --mh runs the plain sampler on it, --gene-accept 1 the per-gene
# decisions)
CFG4 = dict(n_b=[2000, 5000, 8000, 12000, 20000, 3000], G=20000, K=12, seed=13583, sim="wide", hmc=10)
# config-1 data with the HMC block update (10 leapfrog steps) in place of the random-walk
# steps (--gene-accept 1: per-gene decisions)
CFG2 = dict(CFG1, hmc=10)
CFG3 = dict(CFG1, ks=list(range(3, 11)))  # config-1 data fitted by 8 chains, K = 3 .. 10
# the gradient-based sampler whose mixing the config-1 line reports beside the plain sampler's
HMC_QUALITY = dict(hmc=10, gene=True, w_update="mh")
WORKLOADS = {"config1": CFG1, "config2": CFG2, "config3": CFG3, "config4": CFG4}
METRIC = "gibbs_iters_per_s"
UNIT = "sweeps/s"


def _peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def sweep_roofline(N: int, G: int, hmc: int, sweeps_per_s: float, peak_gbs: float) -> dict:
    """The whole sweep against HBM bandwidth, with the bytes of the reference's
    pass structure (one pass over the N x G tensor per conditional that the
    dependency order forces): per entry 12.125 B for Z/X (read Y and X, write X
    and a 1-bit Z), 4.125 B for gamma (X and Z), and 4 B for each of alpha, beta,
    nu, delta, phi and W -- 40.25 B in all; with the HMC update, Z/X, gamma, L + 1
    gradient passes and W: 12.125 + 4.125 + 4 (L + 1) + 4 B."""
    per_entry = 40.25 if hmc <= 0 else 12.125 + 4.125 + 4.0 * (hmc + 1) + 4.0
    bytes_per_sweep = per_entry * float(N) * float(G)
    achieved = bytes_per_sweep * sweeps_per_s / 1e9
    return {"bound": "hbm", "bytes_per_entry": per_entry, "bytes_per_sweep": bytes_per_sweep,
            "achieved": achieved, "peak": peak_gbs, "unit": "GB/s", "frac": achieved / peak_gbs,
            "note": "bytes of the reference's passes over the count tensor x sweeps/s (this build reads "
                    "fewer: the per-kernel figures are in roofline and kernels_ms)"}


def _traffic(kernel: str, workload: str = "config1"):
    """DRAM bytes per launch of `kernel` from the committed ncu summary of this
    workload, or None.  For k_zx: k_zx and k_zx_gp together (the Z/X update)."""
    p = os.path.join(ROOT, "profiles", "dram_traffic_%s.txt" % workload)
    if not os.path.exists(p):
        return None
    want = ("k_zx", "k_zx_gp") if kernel == "k_zx" else (kernel,)
    got = {}
    for line in open(p):
        parts = line.split()
        if len(parts) >= 2 and parts[0] in want and not line.startswith("#"):
            try:
                got[parts[0]] = float(parts[1])
            except ValueError:
                return None
    return sum(got.values()) if len(got) == len(want) else None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(x: float, dist=None, device="cpu") -> float:
    """The largest of one timing over all ranks (every rank gets it); the
    timing of a multi-GPU run is its slowest rank's."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(steps_per_rank: int, world: int, seconds: float) -> float:
    """Sweeps per second of the whole job: every rank runs its own chain (replicas,
    weak scaling), so the units are steps x ranks over the slowest rank's time."""
    return steps_per_rank * world / seconds


def sim_params(cfg):
    """Generator parameters of a workload (the BUSseq model's distributions)."""
    import busseq_gpu_gb300 as bq  # the parameter table only; the library is not loaded
    return dict(bq.CONFIG_SIM[cfg.get("sim", "default")])


def make_data(seed, cfg=CFG1, n_b=None):
    import busseq_gpu_gb300 as bq
    return bq.simulate(n_b if n_b is not None else cfg["n_b"], cfg["G"], cfg["K"], seed, **sim_params(cfg))


def make_data_cpu(seed, cfg=CFG1, n_b=None):
    """The same counts as make_data, from the generator built alone on the
    checker side (oracle/lib/libsim.so): the CPU arms never map the product
    library."""
    from oracle import pyoracle as po
    return po.simulate(n_b if n_b is not None else cfg["n_b"], cfg["G"], cfg["K"], seed, sim_params(cfg))


def cpu_oracle_rate(Y, n_b, K, seed, sweeps: int, warmup: int = 1):
    """FP64 oracle sweeps/s over the whole data set: `warmup` sweeps untimed,
    then `sweeps` timed full sweeps (no sampling, no scaling).  Returns
    (sweeps/s, threads, timed seconds, init seconds)."""
    from oracle import pyoracle as po
    st = po.State(np.ascontiguousarray(Y), n_b, K, seed)
    t0 = time.perf_counter()
    st.init(0.25)
    init_s = time.perf_counter() - t0
    for it in range(warmup):
        st.sweep(it, 0)
    t0 = time.perf_counter()
    for it in range(warmup, warmup + sweeps):
        st.sweep(it, 0)
    dt = time.perf_counter() - t0
    return sweeps / dt, po.num_threads(), dt, init_s


def run_reference(args, rank):
    if rank != 0:
        return 0
    cfg = WORKLOADS[args.workload]
    if args.workload == "config3":
        cfg = dict(cfg, K=max(cfg["ks"]))
    n_b, K, G = list(cfg["n_b"]), cfg["K"], cfg["G"]
    if args.cells > 0:
        n_b = [args.cells] * len(n_b)
    Y, _ = make_data_cpu(cfg["seed"], cfg, n_b)
    value, cores, dt, init_s = cpu_oracle_rate(Y, n_b, K, cfg["seed"], args.steps, args.warmup)
    sample = ("every step one full FP64 oracle sweep over all %d cells x %d genes of the %s data (%d timed "
              "sweeps, %.1f s, after %d untimed; no sampling or scaling)"
              % (sum(n_b), G, args.workload, args.steps, dt, args.warmup))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / value, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (BUSseq generative model)",
        # the reference has only the random-walk sampler: its arm runs that on every workload
        "config": _config(args.workload, n_b, dict(cfg, hmc=0)),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "init_s": init_s,
        "note": "the reference program has no CPU implementation of the sweep; this arm times the FP64 CPU "
                "restatement of it (oracle/oracle.cpp) with all host threads; its input comes from the "
                "generator built on the checker side, so the product library is never loaded",
    }
    print(json.dumps(line))
    return 0


def corrected_cpu_rate(s, n_b, seed, cells_per_batch: int = 40, max_ratio: float = 300.0):
    """The FP64 oracle of the batch-corrected counts on the first cells of each
    batch of a finished run: entries per second on the host cores.  The oracle
    sums every tail term by term (about 40 mean / phi terms per entry), so the
    sample keeps the genes whose means stay within max_ratio times their
    dispersions: a gene whose posterior phi is tiny would otherwise hold the
    host for hours."""
    from oracle import pyoracle as po
    est = s.estimates(with_XZ=True)
    off = np.concatenate([[0], np.cumsum(n_b)])
    rows = np.concatenate([np.arange(off[b], off[b] + min(cells_per_batch, n_b[b])) for b in range(len(n_b))])
    eta = est["alpha"][None, None, :] + est["beta"][None, :, :] + est["nu"][:, None, :]  # [B][K][G]
    mu_max = np.exp(eta.max(axis=(0, 1)) + max(0.0, float(est["delta"][rows].max())))
    genes = np.flatnonzero(mu_max <= max_ratio * est["phi"].min(axis=0))
    if genes.size == 0:
        return None
    sub = {"alpha": est["alpha"][genes], "beta": est["beta"][:, genes], "nu": est["nu"][:, genes],
           "phi": est["phi"][:, genes], "delta": est["delta"][rows], "W": est["W"][rows]}
    nb_s = [min(cells_per_batch, x) for x in n_b]
    X = np.ascontiguousarray(est["X"][rows][:, genes])
    t0 = time.perf_counter()
    po.corrected_counts(X, nb_s, seed, sub)
    secs = time.perf_counter() - t0
    n = X.size
    return {"entries_per_s": n / secs, "cores": po.num_threads(), "kind": "port",
            "sample": "FP64 oracle over the first %d cells of each batch and the %d of %d genes whose means stay "
                      "within %g times their dispersions (%d entries, %.1f s)"
                      % (cells_per_batch, genes.size, est["X"].shape[1], max_ratio, n, secs)}


def _config(name="config1", n_b=None, cfg=None):
    cfg = cfg if cfg is not None else WORKLOADS[name]
    n_b = list(n_b if n_b is not None else cfg["n_b"])
    N, G, K = int(sum(n_b)), cfg["G"], cfg["K"]
    mb = N * G * 4 / 1e6
    gene = bool(cfg.get("gene")) and bool(cfg.get("hmc"))
    sampler = ("HMC block update, %d leapfrog steps%s" % (cfg["hmc"], ", per-gene decisions" if gene else "")
               if cfg.get("hmc") else "plain MH sampler")
    desc = "%s: B=%d batches of %s cells (N=%d), G=%d, K=%d, %s" % (
        name, len(n_b), "/".join(str(n) for n in n_b), N, G, K, sampler)
    return {"workload": desc, "B": len(n_b), "N": N, "G": G, "K": K, "w_update": "mh",
            "sampler": "hmc" if cfg.get("hmc") else "mh", "hmc_leapfrog": cfg.get("hmc", 0), "hmc_gene_accept": gene,
            "parallelism": "replicas (one chain per GPU)",
            "l2": "no flush: X and Y are %.0f MB each, larger than L2" % mb,
            "precision": "f32 likelihood terms, f64 acceptance sums"}


def run_batch(args, cfg, rank, world, local):
    """Config 3: the config-1 data fitted by one chain per K = 3 .. 10 (the BIC
    sweep over K).  Each chain's launch shapes (gene-pass chunk length, Z/X
    unit length and CTAs per SM) come from the autotuner.  The sequential arm
    times each chain alone; the batched arm launches one sweep of all chains as
    one CUDA graph.  Both arms run the same sweeps of the same chains; the
    metric is chain-sweeps per second."""
    import torch
    import busseq_gpu_gb300 as bq

    dev = f"cuda:{local}"
    torch.cuda.set_device(local)
    n_b, G, seed = list(cfg["n_b"]), cfg["G"], cfg["seed"]
    if args.cells > 0:
        n_b = [args.cells] * len(n_b)
    Y, W_true, _ = make_data(seed, cfg, n_b)
    N = int(sum(n_b))
    ks = list(cfg["ks"])
    Yd = torch.from_numpy(Y).to(dev)
    t0 = time.perf_counter()
    tuned = {K: bq.autotune(Yd, n_b, K, seed=seed, sweeps=6, device=local) for K in ks}
    shape = {K: {k: v for k, v in tuned[K].items() if k != "ms_per_sweep"} for K in ks}
    tune_s = time.perf_counter() - t0
    total = args.warmup + args.steps
    burn = args.warmup + args.steps // 2

    def chains():
        return [bq.Sampler(Yd, n_b, K, seed=seed + 7919 * rank + K, device=local, **shape[K]) for K in ks]

    def ev():
        return torch.cuda.Event(enable_timing=True)

    # ---- sequential arm: every chain alone, on its own stream ----------------
    seq_ms, busy_ms = {}, {}
    stream = torch.cuda.Stream(device=local)
    for K, c in zip(ks, chains()):
        c.set_stream(stream.cuda_stream)
        c.begin(total, burn, args.warmup)
        c.sweeps(args.warmup)
        c.synchronize()
        e0, e1 = ev(), ev()
        e0.record(stream)
        c.sweeps(args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
        seq_ms[K] = e0.elapsed_time(e1)
        # the chain's kernels alone: summed event-timed durations per sweep
        busy_ms[K] = sum(c.profile(10).values())
        c.close()
    seq_total = sum(seq_ms.values())

    # ---- batched arm: one graph per sweep holding every chain ---------------
    cs = chains()
    for c in cs:
        c.begin(total, burn, args.warmup)
    b = bq.Batch(cs)
    b.sweeps(args.warmup)
    b.synchronize()
    bstream = torch.cuda.ExternalStream(b.stream, device=dev)
    e0, e1 = ev(), ev()
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        e0.record(bstream)
        b.sweeps(args.steps)
        e1.record(bstream)
        torch.cuda.synchronize()
    bat_ms = e0.elapsed_time(e1)
    b.synchronize()
    b.close()
    bic, launches = {}, 0
    for K, c in zip(ks, cs):
        c.finish()
        bic[K] = c.bic()
        launches += (args.steps - max(0, burn - args.warmup)) * c.launches_per_sweep(True) + \
            max(0, burn - args.warmup) * c.launches_per_sweep(False)
        c.close()
    value = len(ks) * args.steps / (bat_ms / 1000.0)
    seq_value = len(ks) * args.steps / (seq_total / 1000.0)
    del Yd
    torch.cuda.empty_cache()

    # ---- e2e: the whole BIC sweep from pinned host counts --------------------
    Yp = torch.from_numpy(Y).pin_memory()
    Yh = Yp.numpy()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    cs = [bq.Sampler(Yh, n_b, K, seed=seed + 7919 * rank + K, device=local, **shape[K]) for K in ks]
    for c in cs:
        c.begin(args.steps, args.steps // 2, min(args.warmup, args.steps))
    with bq.Batch(cs) as b2:
        b2.sweeps(args.steps)
        b2.synchronize()
    bic_e2e = {}
    d2h = 0
    for K, c in zip(ks, cs):
        c.finish()
        bic_e2e[K] = c.bic()
        d2h += sum(v.nbytes for v in c.estimates(with_XZ=False).values()) + 8
        c.close()
    e2e_s = time.perf_counter() - t0
    if rank == 0:
        k_best = min(bic, key=bic.get)
        line = {
            "metric": "chain_sweeps_per_s", "value": value, "unit": "chain-sweeps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": bat_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (BUSseq generative model, seed %d, K = 8)" % seed,
            "config": {"workload": "config3: the config-1 data (B=4 x %d cells, G=%d) fitted by %d chains, K = %s, "
                                   "batched: one CUDA graph per sweep of all chains" % (n_b[0], G, len(ks), ks),
                       "N": N, "G": G, "Ks": ks, "launch_shapes": {str(K): shape[K] for K in ks},
                       "l2": "no flush: every chain's X and Y are %.0f MB" % (N * G * 4 / 1e6)},
            "sequential": {"value": seq_value, "unit": "chain-sweeps/s", "ms": seq_total,
                           "ms_per_chain": {str(K): v for K, v in seq_ms.items()},
                           "note": "each chain alone for the same %d sweeps" % args.steps},
            "batched_vs_sequential": value / seq_value,
            # What a merged multi-chain launch could recover: it can remove the gaps
            # between kernels (launch latency, tails, idle SMs) but not the kernels'
            # own busy time.  sequential / busy is the speed-up of removing every gap;
            # batched / busy below 1 means the concurrent kernels already overlap.
            "kernel_busy": {
                "ms_per_sweep": {str(K): v for K, v in busy_ms.items()},
                "busy_ms_per_sweep_all_chains": sum(busy_ms.values()),
                "sequential_ms_per_sweep_all_chains": seq_total / args.steps,
                "batched_ms_per_sweep_all_chains": bat_ms / args.steps,
                "gap_free_bound_vs_sequential": (seq_total / args.steps) / sum(busy_ms.values()),
                "batched_over_busy": (bat_ms / args.steps) / sum(busy_ms.values()),
                "note": "busy = sum of each kernel's event-timed duration when its chain runs alone (burn-in "
                        "sweeps, 10 timed)"},
            # per chain-sweep, every chain passes over its own copy of the tensor
            "sweep_roofline": sweep_roofline(N, G, 0, value / world, _peak_hbm()[0]),
            "autotune": {"seconds": tune_s, "ms_per_sweep": {str(K): tuned[K]["ms_per_sweep"] for K in ks}},
            "bic": {str(K): v for K, v in bic.items()}, "k_min_bic": k_best,
            "e2e": {"value": len(ks) * args.steps / e2e_s, "unit": "chain-sweeps/s",
                    "h2d_bytes_per_step": len(ks) * Y.nbytes / args.steps, "d2h_bytes_per_step": d2h / args.steps,
                    "note": "pinned-host upload per chain, init, %d batched sweeps, posterior, estimates and BIC "
                            "per K to the host; k_min_bic %d" % (args.steps, min(bic_e2e, key=bic_e2e.get))},
            "gpu_launches": launches,
            "clocks": clk.summary(),
            "cpu_baseline": None,
        }
        print(json.dumps(line))
    return 0


def ess_run(Y, W_true, n_b, K, seed, n_iter=2000, n_burnin=1000, hmc=0, gene=False, w_update="mh"):
    """One whole job with kept draws: ESS (Geyer, initial monotone sequence) of
    every beta (k >= 1) and nu (b >= 1) coordinate, ESS/s over the wall time of
    the whole job (upload, init, burn-in, kept sweeps, estimates), and the ARI
    of the posterior W against the simulated types."""
    import busseq_gpu_gb300 as bq
    from busseq_gpu_gb300.diagnostics import adjusted_rand_index, ess_geyer

    t0 = time.perf_counter()
    s = bq.Sampler(Y, n_b, K, seed=seed + 1, keep_draws=True, hmc_leapfrog=hmc, hmc_gene_accept=gene and hmc > 0,
                   w_update=w_update)
    s.run(n_iter, n_burnin, min(500, n_burnin))
    est = s.estimates(with_XZ=False)
    wall = time.perf_counter() - t0
    pres = s.preserved()
    hstats = s.hmc_stats() if hmc else None
    s.close()
    out = {"sweeps": n_iter, "burnin": n_burnin, "kept": n_iter - n_burnin, "wall_s": wall,
           "ari_W": adjusted_rand_index(est["W"], W_true), "estimator": "Geyer initial monotone sequence",
           "sampler": ("HMC, %d leapfrog steps%s" % (hmc, ", per-gene decisions" if gene else "")) if hmc
           else "random-walk MH (the reference's)",
           "w_update": "K-way Gibbs draw" if w_update == "gibbs" else "Metropolis, uniform proposal (the reference's)"}
    if hstats:
        out["hmc"] = {k: float(v) for k, v in hstats.items()}
    for name in ("beta", "nu"):
        e = ess_geyer(pres[name].astype(np.float64))
        moving = np.isfinite(e)
        ev = e[moving]
        out[name] = {"coords": int(e.size), "moving": int(moving.sum()),
                     "ess_median": float(np.median(ev)) if ev.size else None,
                     "ess_min": float(ev.min()) if ev.size else None,
                     "ess_per_s_median": float(np.median(ev)) / wall if ev.size else None,
                     "ess_per_s_min": float(ev.min()) / wall if ev.size else None}
    return out


def hmc_vs_mh(Y, W_true, n_b, K, seed, mh_first, seed_offsets=(0, 1000, 2000)):
    """The gradient-based sampler (HMC_QUALITY) against the plain sampler on the
    same data, each run as a whole job of 2000 sweeps (1000 kept) from three
    seeds.  The ARI of a single chain depends on which local mode of the cell
    types the chain settles in (the plain sampler alone ranges 0.81-0.96 over
    these seeds), so the ARIs are compared as means over the three chains of
    each sampler; the ESS/s ratios are the medians of the three per-seed ratios
    (per seed: median over the coordinates, whole-job wall time)."""
    runs = []
    for k, off in enumerate(seed_offsets):
        mh = mh_first if k == 0 else ess_run(Y, W_true, n_b, K, seed + off, hmc=0)
        hq = ess_run(Y, W_true, n_b, K, seed + off, hmc=HMC_QUALITY["hmc"], gene=HMC_QUALITY["gene"],
                     w_update=HMC_QUALITY["w_update"])
        r = {"seed_offset": off, "ari_W_mh": mh["ari_W"], "ari_W_hmc": hq["ari_W"],
             "wall_s_mh": mh["wall_s"], "wall_s_hmc": hq["wall_s"]}
        for name in ("beta", "nu"):
            a, b = hq[name]["ess_per_s_median"], mh[name]["ess_per_s_median"]
            r[name + "_ess_per_s_median_ratio"] = a / b if a and b else None
            r[name + "_ess_median_hmc"] = hq[name]["ess_median"]
            r[name + "_ess_median_mh"] = mh[name]["ess_median"]
        if hq.get("hmc"):
            r["hmc"] = hq["hmc"]
        runs.append(r)
    med = {name: float(np.median([r[name + "_ess_per_s_median_ratio"] or 0.0 for r in runs])) for name in ("beta", "nu")}
    ari_mh = float(np.mean([r["ari_W_mh"] for r in runs]))
    ari_hmc = float(np.mean([r["ari_W_hmc"] for r in runs]))
    return {"sampler": "HMC, %d leapfrog steps%s, W by %s" % (HMC_QUALITY["hmc"],
                                                            ", per-gene decisions" if HMC_QUALITY["gene"] else "",
                                                            HMC_QUALITY["w_update"]),
            "beta_ess_per_s_median_ratio": med["beta"], "nu_ess_per_s_median_ratio": med["nu"],
            "ari_W_hmc_mean": ari_hmc, "ari_W_mh_mean": ari_mh, "ari_diff_mean": ari_hmc - ari_mh,
            "target": "both ESS/s ratios >= 5 with the mean ARI within 0.01 of the plain sampler's or better",
            "met": bool(med["beta"] >= 5 and med["nu"] >= 5 and ari_hmc >= ari_mh - 0.01),
            "runs": runs}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=30)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cells", type=int, default=0,
                    help="cells per batch (default 2500, the config-1 size); smaller only for profiler captures")
    ap.add_argument("--no-ess", action="store_true", help="skip the ESS / ARI run")
    ap.add_argument("--no-hmc-quality", action="store_true",
                    help="config1: skip the gradient-based sampler's ESS / ARI run beside the plain sampler's")
    ap.add_argument("--leapfrog", type=int, default=0,
                    help="leapfrog steps of the HMC block update (overrides the workload's; 0 keeps it)")
    ap.add_argument("--gene-accept", type=int, default=None, choices=[0, 1],
                    help="HMC workloads: 1 accepts or rejects each gene's block on its own (delta by the "
                         "random-walk step), 0 one decision for the whole block (default: the workload's)")
    ap.add_argument("--mh", action="store_true",
                    help="run the plain random-walk sampler even where the workload uses the HMC update")
    ap.add_argument("--workload", default="config1", choices=sorted(WORKLOADS),
                    help="config1 (the headline, default), config2 (config-1 data, HMC block update with 10 "
                         "leapfrog steps), config3 (config-1 data, 8 chains K=3..10 batched in one graph per "
                         "sweep; 1000 steps unless --steps) or config4 (N=50000, G=20000, K=12, uneven batches, "
                         "the same HMC update)")
    ap.add_argument("--only-value", action="store_true",
                    help="measure only the device-resident sweep rate (the short run used under ncu)")
    ap.add_argument("--corrected-counts", action="store_true",
                    help="with --only-value: also run one batch-corrected-count pass after the sweeps")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    args.steps_given = args.steps
    if args.steps is None:
        args.steps = 3000

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank)

    import torch
    import busseq_gpu_gb300 as bq

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()

    cfg = dict(WORKLOADS[args.workload])
    if args.workload == "config3":
        if args.steps_given is None:
            args.steps = 1000
        return run_batch(args, cfg, rank, world, local)
    if args.leapfrog > 0:
        cfg["hmc"] = args.leapfrog
    if args.mh:
        cfg["hmc"] = 0
    if args.gene_accept is not None:
        cfg["gene"] = bool(args.gene_accept)
    n_b, G, K = list(cfg["n_b"]), cfg["G"], cfg["K"]
    seed = cfg["seed"]
    if args.cells > 0:
        n_b = [args.cells] * len(n_b)
    Y, W_true, _ = make_data(seed, cfg, n_b)
    N = int(sum(n_b))

    # ---- value: counts resident in HBM, graph-launched sweeps ---------------
    Yd = torch.from_numpy(Y).to(f"cuda:{local}")
    # a dedicated (non-default) stream shared by the sampler and the events
    stream = torch.cuda.Stream(device=local)
    torch.cuda.set_stream(stream)
    hmc = cfg.get("hmc", 0)
    gene = bool(cfg.get("gene")) and hmc > 0
    s = bq.Sampler(Yd, n_b, K, seed=seed + 7919 * rank, device=local, hmc_leapfrog=hmc, hmc_gene_accept=gene)
    assert stream.cuda_stream != 0
    s.set_stream(stream.cuda_stream)
    total = args.warmup + args.steps
    s.begin(total, args.warmup + args.steps // 2, args.warmup)
    s.sweeps(args.warmup)
    s.synchronize()
    torch.cuda.synchronize()
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        ev0.record(stream)
        s.sweeps(args.steps)
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1)
    s.finish()
    ms_max = max_over_ranks(ms, dist, f"cuda:{local}")
    value = whole_job_rate(args.steps, world, ms_max / 1000.0)
    launches = (args.steps // 2) * s.launches_per_sweep(False) + (args.steps - args.steps // 2) * s.launches_per_sweep(True)

    if args.only_value:
        if args.corrected_counts:  # one corrected-count pass of the finished run (for profiler captures)
            cc = torch.empty((N, G), dtype=torch.int32, device=f"cuda:{local}")
            s.corrected_counts(out=cc)
            torch.cuda.synchronize()
            del cc
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                              "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "config": _config(args.workload, n_b, cfg),
                              "note": "device-resident sweep rate only (--only-value)"}))
        s.close()
        return 0

    # ---- per-kernel durations for the roofline (events on the same stream) --
    prof = s.profile(20)
    big = {k: v for k, v in prof.items() if k in ("k_zx", "k_alpha", "k_beta_nu", "k_delta", "k_phi", "k_w",
                                                  "k_hmc_grad", "k_hmc_dll")}
    # the Z/X update is two launches: k_zx and the Gamma-Poisson draws it leaves to k_zx_gp
    big["k_zx"] = prof.get("k_zx", 0.0) + prof.get("k_zx_gp", 0.0)
    dom = max(big, key=big.get)
    kid = [bq.lib().busseq_kernel_name(i).decode() for i in range(64)].index(dom)
    alg_bytes = s.kernel_bytes(kid)
    n_launch = hmc if dom == "k_hmc_grad" else 1  # launches of the kernel per sweep (one per leapfrog step)
    ms_launch = big[dom] / n_launch
    achieved = alg_bytes / (ms_launch / 1000.0) / 1e9
    peak, peak_kind = _peak_hbm()
    traffic = _traffic(dom, args.workload) if args.cells <= 0 else None

    # ---- batch-corrected counts of the finished run (rank 0, device output) --
    corrected = None
    if rank == 0:
        cc = torch.empty((N, G), dtype=torch.int32, device=f"cuda:{local}")
        s.corrected_counts(out=cc)  # warm-up call
        torch.cuda.synchronize()
        c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        c0.record(stream)
        s.corrected_counts(out=cc)
        c1.record(stream)
        torch.cuda.synchronize()
        cms = c0.elapsed_time(c1)
        corrected = {"ms": cms, "entries_per_s": N * G / (cms / 1000.0), "dtype": "f64",
                     "note": "one call: tables, k_correct over N x G entries, device output"}
        del cc
    # the finished run stays open for the corrected counts' CPU baseline, which
    # runs after the end-to-end job: no host-side leg runs between the GPU timings
    del Yd
    torch.cuda.empty_cache()

    # ---- e2e: pinned host counts through the C ABI ---------------------------
    # inputs and outputs in pinned host memory, allocated before the timed region
    Yp = torch.from_numpy(Y).pin_memory()
    Yh = Yp.numpy()
    torch_dt = {np.dtype(np.float64): torch.float64, np.dtype(np.int32): torch.int32}
    pinned = []

    def pinned_alloc(shape, dtype):
        t = torch.zeros(shape, dtype=torch_dt[np.dtype(dtype)], pin_memory=True)
        pinned.append(t)
        return t.numpy()

    est_out = bq.estimate_buffers(len(n_b), K, G, N, True, pinned_alloc)
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    s2 = bq.Sampler(Yh, n_b, K, seed=seed + 7919 * rank, device=local, hmc_leapfrog=hmc, hmc_gene_accept=gene)
    s2.run(args.steps, args.steps // 2, min(args.warmup, args.steps))
    est = s2.estimates(with_XZ=True, out=est_out)
    t1 = time.perf_counter()
    s2.close()
    e2e_s = t1 - t0
    e2e_value = whole_job_rate(args.steps, world, max_over_ranks(e2e_s, dist, f"cuda:{local}"))
    h2d = Y.nbytes
    d2h = sum(v.nbytes for v in est.values())
    if corrected is not None and world == 1 and not args.no_cpu_baseline:
        corrected["cpu_baseline"] = corrected_cpu_rate(s, n_b, seed + 7919 * rank)
    s.close()

    # ---- mixing and recovery: ESS of beta and nu, ARI of W (rank 0) -------
    quality = None
    if rank == 0 and not args.no_ess:
        quality = ess_run(Y, W_true, n_b, K, seed, hmc=hmc, gene=gene)
        if hmc:
            # the same whole job with the plain random-walk sampler, for the ESS/s ratios
            mh = ess_run(Y, W_true, n_b, K, seed, hmc=0)

            def ratio(name):
                a, r = quality[name]["ess_per_s_median"], mh[name]["ess_per_s_median"]
                return a / r if a and r else None

            quality["vs_mh"] = {"beta_ess_per_s_median_ratio": ratio("beta"),
                                "nu_ess_per_s_median_ratio": ratio("nu"), "ari_W_mh": mh["ari_W"], "mh": mh}
        elif args.workload == "config1" and not args.no_hmc_quality:
            quality["hmc_vs_mh"] = hmc_vs_mh(Y, W_true, n_b, K, seed, quality)

    # ---- CPU baseline (rank 0, N = 1 only): 20 full sweeps of the oracle ----
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        nsw = 20
        rate, cores, secs, _ = cpu_oracle_rate(Y, n_b, K, seed, nsw, 1)
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": "%d full FP64 oracle sweeps over all %d cells x %d genes (%.1f s) after one untimed "
                         "sweep; no sampling or scaling" % (nsw, N, G, secs)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (BUSseq generative model, seed %d)" % seed,
            "config": _config(args.workload, n_b, cfg),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d / args.steps,
                    "d2h_bytes_per_step": d2h / args.steps,
                    "note": "one job per run: pinned-host upload, init, %d sweeps, posterior, all estimates "
                            "(and the last sweep's X and Z) to pinned host buffers" % args.steps},
            "sweep_roofline": sweep_roofline(N, G, hmc, value / world, peak),  # per GPU: replicas
            "roofline": {"bound": "hbm", "kernel": "k_zx + k_zx_gp" if dom == "k_zx" else dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                         "alg_bytes_per_launch": alg_bytes, "ms_per_launch": ms_launch,
                         "launches_per_sweep": n_launch},
            "kernels_ms": {k: v for k, v in prof.items() if v > 0},  # the kernels this sampler launches
            "gpu_launches": launches,
            "clocks": clk.summary(),
            "cpu_baseline": cpu,
            "quality": quality,
            "corrected_counts": corrected,
        }
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
