"""Host logic of bench.py (no GPU): the batch-corrected-count CPU baseline
keeps its oracle sample to genes whose tail sums stay short, and the sweep-level
roofline counts the reference's passes."""
import numpy as np

import bench


class _FakeRun:
    """Stands in for a finished sampler: estimates() of a small state."""

    def __init__(self, est):
        self._est = est

    def estimates(self, with_XZ=True):
        return self._est


def _est(rng, n_b, G, K, tiny_phi_genes=()):
    B, N = len(n_b), sum(n_b)
    alpha = rng.uniform(0.5, 2.5, G)
    beta = np.zeros((K, G))
    beta[1:] = rng.normal(0, 0.5, (K - 1, G))
    nu = np.zeros((B, G))
    nu[1:] = rng.normal(0.3, 0.2, (B - 1, G))
    phi = rng.uniform(5, 20, (B, G))
    for g in tiny_phi_genes:
        phi[1, g] = 1e-6  # a gene whose posterior dispersion collapsed in one batch
    delta = rng.normal(0, 0.1, N)
    W = rng.integers(0, K, N).astype(np.int32)
    X = rng.poisson(5.0, (N, G)).astype(np.int32)
    return {"alpha": alpha, "beta": beta, "nu": nu, "phi": phi, "delta": delta, "W": W, "X": X}


def test_corrected_baseline_skips_genes_with_collapsed_dispersion():
    rng = np.random.default_rng(0)
    n_b, G, K = [12, 10], 30, 3
    est = _est(rng, n_b, G, K, tiny_phi_genes=(3, 17))
    out = bench.corrected_cpu_rate(_FakeRun(est), n_b, 7, cells_per_batch=5)
    assert out is not None and out["entries_per_s"] > 0
    assert "28 of 30 genes" in out["sample"], out["sample"]
    assert "%d entries" % (10 * 28) in out["sample"]


def test_corrected_baseline_keeps_every_gene_of_a_moderate_run():
    rng = np.random.default_rng(1)
    n_b, G, K = [8, 8, 6], 20, 2
    out = bench.corrected_cpu_rate(_FakeRun(_est(rng, n_b, G, K)), n_b, 3, cells_per_batch=4)
    assert "20 of 20 genes" in out["sample"], out["sample"]


def test_sweep_roofline_counts_the_reference_passes():
    r = bench.sweep_roofline(10000, 10000, 0, 594.0, 6786.2)
    assert r["bytes_per_entry"] == 40.25 and r["bytes_per_sweep"] == 40.25e8
    assert abs(r["achieved"] - 40.25e8 * 594.0 / 1e9) < 1e-6 and abs(r["frac"] - r["achieved"] / 6786.2) < 1e-12
    assert bench.sweep_roofline(10000, 10000, 10, 1.0, 1.0)["bytes_per_entry"] == 64.25  # HMC, L = 10


def test_checker_side_generator_matches_the_library():
    import busseq_gpu_gb300 as bq
    from oracle import pyoracle as po
    n_b, G, K, seed = [13, 9, 11], 57, 4, 99
    for name in ("default", "wide"):
        Y, W, _ = bq.simulate(n_b, G, K, seed, **bq.CONFIG_SIM[name])
        Y2, W2 = po.simulate(n_b, G, K, seed, bq.CONFIG_SIM[name])
        assert np.array_equal(Y, Y2) and np.array_equal(W, W2)


def test_reference_arm_is_unscaled_and_never_maps_the_product_library():
    """The reference arm times full oracle sweeps of the whole (here shrunk)
    workload, and its process holds only checker-side libraries."""
    import json
    import subprocess
    import sys
    code = ("import sys, json, io, contextlib; sys.argv = ['bench.py']; import bench\n"
            "class A: workload = 'config1'; cells = 6; steps = 2; warmup = 3; gpus = 1\n"
            "buf = io.StringIO()\n"
            "with contextlib.redirect_stdout(buf): bench.run_reference(A, 0)\n"
            "maps = open('/proc/self/maps').read()\n"
            "print(json.dumps({'line': json.loads(buf.getvalue()), 'product': 'libbusseq_gb300' in maps, "
            "'checker': 'liborc.so' in maps}))\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=bench.ROOT, stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    out = json.loads(r.stdout.strip().splitlines()[-1])
    line = out["line"]
    assert out["checker"] and not out["product"]
    assert line["impl"] == "reference" and line["steps"] == 2 and line["value"] > 0
    assert abs(line["ms_per_step"] - 1000.0 / line["value"]) < 1e-9
    assert "no sampling or scaling" in line["cpu_baseline"]["sample"] and "all 24 cells" in line["cpu_baseline"]["sample"]
