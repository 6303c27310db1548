"""The gradient-based block update on the GPU: its gradient, metric and
log-posterior differences against the FP64 oracle, and the behaviour of HMC
chains (adaptation, acceptance, recovery of the cell types, reproducibility,
checkpoint / resume).

Tolerances: the gradient within 2e-3 posterior standard deviations (scale
sqrt(metric)) plus 1e-4 relative; the metric (observed information) of the eta-coordinates
within 1e-3 relative; the observed information of log phi within 1e-2 relative
+ 0.5 (it sums terms of both signs); log-posterior differences within
5e-3 + 1e-5 |diff| (per-entry float terms of a few units over ~10^5 entries).
"""
import numpy as np
import pytest

import busseq_gpu_gb300 as bq
from oracle import pyoracle as po
from tests.parity_util import oracle_state

pytestmark = pytest.mark.gpu

N_B, G, K, SEED = [60, 45, 70], 300, 4, 31


@pytest.fixture(scope="module")
def warm():
    Y, W_true, _ = bq.simulate(N_B, G, K, SEED)
    mh = bq.Sampler(Y, N_B, K, seed=SEED, p0=0.3)
    mh.begin(30, 30, 0)
    mh.sweeps(30)
    mh.synchronize()
    st = mh.get_state()
    mh.close()
    return Y, W_true, st


def _free_masks():
    off = np.concatenate([[0], np.cumsum(N_B)])[:-1]
    d = np.ones(sum(N_B), bool)
    d[off] = False
    return {"alpha": np.ones(G, bool), "beta": np.arange(K)[:, None] > 0, "nu": np.arange(len(N_B))[:, None] > 0,
            "psi": np.ones((len(N_B), G), bool), "delta": d}


def test_gradient_and_metric_match_oracle(warm):
    Y, _, st = warm
    h = bq.Sampler(Y, N_B, K, seed=SEED, hmc_leapfrog=5)
    h.set_state(st)
    got = h.hmc_gradient(with_metric=True)
    h.close()
    o = oracle_state(Y, np.array(N_B), K, SEED, st)
    want = o.hmc_grad()
    masks = _free_masks()
    for name in ("alpha", "beta", "nu", "psi", "delta"):
        gg, go = got["grad"][name], want["grad"][name]
        mo = np.maximum(want["metric"][name], 1e-2)
        m = np.broadcast_to(masks[name], gg.shape)
        err = np.abs(gg - go)
        tol = 2e-3 * np.sqrt(mo) + 1e-4 * np.abs(go)
        assert np.all(err[m] <= tol[m]), (name, np.max(err[m] / tol[m]))
        assert np.all(gg[~m] == 0)
        mg = got["metric"][name]
        if name == "psi":
            assert np.all(np.abs(mg[m] - mo[m]) <= 1e-2 * mo[m] + 0.5), name
        else:
            np.testing.assert_allclose(mg[m], mo[m], rtol=1e-3, err_msg=name)


def test_logpost_difference_matches_oracle(warm):
    Y, _, st = warm
    rng = np.random.default_rng(3)
    masks = _free_masks()
    B = len(N_B)
    st_b = {k: np.array(v, copy=True) for k, v in st.items()}
    st_b["alpha"] = st["alpha"] + rng.normal(0, 0.01, G).astype(np.float32)
    st_b["beta"] = st["beta"] + (rng.normal(0, 0.01, (K, G)) * masks["beta"]).astype(np.float32)
    st_b["nu"] = st["nu"] + (rng.normal(0, 0.01, (B, G)) * masks["nu"]).astype(np.float32)
    st_b["delta"] = st["delta"] + (rng.normal(0, 0.01, sum(N_B)) * masks["delta"]).astype(np.float32)
    st_b["phi"] = (st["phi"] * np.exp(rng.normal(0, 0.05, (B, G)))).astype(np.float32)
    h = bq.Sampler(Y, N_B, K, seed=SEED, hmc_leapfrog=5)
    h.set_state(st_b)
    got = h.hmc_logpost_diff(st)
    h.close()
    oa = oracle_state(Y, np.array(N_B), K, SEED, st)
    ob = oracle_state(Y, np.array(N_B), K, SEED, st_b)
    want = ob.hmc_logpost() - oa.hmc_logpost()
    assert abs(got - want) <= 5e-3 + 1e-5 * abs(want), (got, want)


def _ari(a, b):
    from busseq_gpu_gb300.diagnostics import adjusted_rand_index
    return adjusted_rand_index(a, b)


def test_hmc_chain_adapts_accepts_and_recovers(warm):
    Y, W_true, _ = warm
    mh = bq.Sampler(Y, N_B, K, seed=SEED)
    mh.run(160, 80, 40)
    ari_mh = _ari(mh.estimates()["W"], W_true)
    mh.close()
    runs = []
    for _ in range(2):
        h = bq.Sampler(Y, N_B, K, seed=SEED, hmc_leapfrog=10, keep_draws=True)
        h.run(160, 80, 40)
        stats = h.hmc_stats()
        est = h.estimates()
        st = h.get_state()
        pres = h.preserved()
        h.close()
        runs.append((stats, est, st, pres))
    stats, est, st, pres = runs[0]
    assert np.isfinite(stats["step_size"]) and stats["step_size"] > 0
    assert 0.4 <= stats["accept_rate_kept"] <= 0.99, stats
    ari = _ari(est["W"], W_true)
    print("HMC", stats, "ARI", ari, "MH ARI", ari_mh)
    assert ari > min(0.7, ari_mh - 0.05)
    # X = Y where Y > 0, Z only where Y == 0, fixed coordinates stay 0
    assert np.array_equal(st["X"][Y > 0], Y[Y > 0]) and not st["Z"][Y > 0].any()
    assert np.all(st["beta"][0] == 0) and np.all(st["nu"][0] == 0)
    off = np.concatenate([[0], np.cumsum(N_B)])[:-1]
    assert np.all(st["delta"][off] == 0)
    # the kept beta draws move (the random-walk sampler leaves most of them in place per sweep)
    moved = np.mean(np.abs(np.diff(pres["beta"], axis=1)) > 0, axis=1)
    assert np.median(moved) > 0.3
    # bit-identical rerun
    for k in st:
        assert np.array_equal(st[k], runs[1][2][k]), k


def test_hmc_checkpoint_resume_is_exact(warm, tmp_path):
    Y, _, _ = warm
    ref = bq.Sampler(Y, N_B, K, seed=SEED, hmc_leapfrog=4)
    ref.run(30, 16, 8)
    st_ref = ref.get_state()
    ref.close()
    a = bq.Sampler(Y, N_B, K, seed=SEED, hmc_leapfrog=4)
    a.begin(30, 16, 8)
    a.sweeps(11)
    path = str(tmp_path / "hmc.ck")
    a.checkpoint_save(path)
    a.close()
    b = bq.Sampler(Y, N_B, K, seed=SEED, hmc_leapfrog=4)
    b.checkpoint_load(path)
    b.sweeps(19)
    b.finish()
    st = b.get_state()
    b.close()
    for k in st_ref:
        assert np.array_equal(st_ref[k], st[k]), k


def test_gradient_accessor_leaves_the_chain_unchanged(warm):
    """Reading the gradient and metric mid-run (after the metric froze) must not
    change the chain: the adapted mass and its information part are kept."""
    Y, _, _ = warm
    ref = bq.Sampler(Y, N_B, K, seed=SEED, hmc_leapfrog=4)
    ref.run(30, 16, 8)
    st_ref = ref.get_state()
    ref.close()
    a = bq.Sampler(Y, N_B, K, seed=SEED, hmc_leapfrog=4)
    a.begin(30, 16, 8)
    a.sweeps(20)
    a.hmc_gradient(with_metric=True)
    a.sweeps(10)
    a.finish()
    st = a.get_state()
    a.close()
    for k in st_ref:
        assert np.array_equal(st_ref[k], st[k]), k


def _perturbed_genes(st, rng):
    """st with alpha, beta, nu and phi moved (delta kept: the per-gene blocks)."""
    masks = _free_masks()
    B = len(N_B)
    st_b = {k: np.array(v, copy=True) for k, v in st.items()}
    st_b["alpha"] = st["alpha"] + rng.normal(0, 0.01, G).astype(np.float32)
    st_b["beta"] = st["beta"] + (rng.normal(0, 0.01, (K, G)) * masks["beta"]).astype(np.float32)
    st_b["nu"] = st["nu"] + (rng.normal(0, 0.01, (B, G)) * masks["nu"]).astype(np.float32)
    st_b["phi"] = (st["phi"] * np.exp(rng.normal(0, 0.05, (B, G)))).astype(np.float32)
    return st_b


def test_gene_logpost_differences_match_oracle(warm):
    """Per-gene decisions: each gene's change of its block log posterior (delta
    held) against the oracle's log posterior of the state that differs in that
    gene only, and their sum against the whole change."""
    Y, _, st = warm
    rng = np.random.default_rng(4)
    st_b = _perturbed_genes(st, rng)
    h = bq.Sampler(Y, N_B, K, seed=SEED, hmc_leapfrog=5, hmc_gene_accept=True)
    h.set_state(st_b)
    got = h.hmc_gene_logpost_diff(st)
    h.close()
    oa = oracle_state(Y, np.array(N_B), K, SEED, st)
    base = oa.hmc_logpost()
    total = oracle_state(Y, np.array(N_B), K, SEED, st_b).hmc_logpost() - base
    assert abs(got.sum() - total) <= 5e-3 + 1e-5 * abs(total), (got.sum(), total)
    for g in rng.choice(G, 5, replace=False):
        st_g = {k: np.array(v, copy=True) for k, v in st.items()}
        st_g["alpha"][g] = st_b["alpha"][g]
        for f in ("beta", "nu", "phi"):
            st_g[f][:, g] = st_b[f][:, g]
        want = oracle_state(Y, np.array(N_B), K, SEED, st_g).hmc_logpost() - base
        assert abs(got[g] - want) <= 2e-3 + 1e-5 * abs(want), (g, got[g], want)


def test_gene_decision_chain(warm, tmp_path):
    """Per-gene decisions: adaptation, acceptance, recovery of the types, the
    invariants, bit-identical reruns and exact checkpoint / resume."""
    Y, W_true, _ = warm
    mh = bq.Sampler(Y, N_B, K, seed=SEED)
    mh.run(160, 80, 40)
    ari_mh = _ari(mh.estimates()["W"], W_true)
    mh.close()
    runs = []
    for _ in range(2):
        h = bq.Sampler(Y, N_B, K, seed=SEED, hmc_leapfrog=10, hmc_gene_accept=True, keep_draws=True)
        h.run(160, 80, 40)
        runs.append((h.hmc_stats(), h.estimates(), h.get_state(), h.preserved()))
        h.close()
    stats, est, st, pres = runs[0]
    ari = _ari(est["W"], W_true)
    print("per-gene HMC", stats, "ARI", ari, "MH ARI", ari_mh)
    assert np.isfinite(stats["step_size"]) and stats["step_size"] > 0
    assert 0.4 <= stats["accept_rate_kept"] <= 0.99, stats
    assert ari > min(0.7, ari_mh - 0.05)
    assert np.array_equal(st["X"][Y > 0], Y[Y > 0]) and not st["Z"][Y > 0].any()
    assert np.all(st["beta"][0] == 0) and np.all(st["nu"][0] == 0)
    off = np.concatenate([[0], np.cumsum(N_B)])[:-1]
    assert np.all(st["delta"][off] == 0)
    moved = np.mean(np.abs(np.diff(pres["beta"], axis=1)) > 0, axis=1)
    assert np.median(moved) > 0.3
    for k in st:
        assert np.array_equal(st[k], runs[1][2][k]), k
    # checkpoint / resume, and a chain with one decision for the whole block refuses it
    ref = bq.Sampler(Y, N_B, K, seed=SEED, hmc_leapfrog=4, hmc_gene_accept=True)
    ref.run(30, 16, 8)
    st_ref = ref.get_state()
    ref.close()
    a = bq.Sampler(Y, N_B, K, seed=SEED, hmc_leapfrog=4, hmc_gene_accept=True)
    a.begin(30, 16, 8)
    a.sweeps(11)
    path = str(tmp_path / "gene.ck")
    a.checkpoint_save(path)
    a.close()
    c = bq.Sampler(Y, N_B, K, seed=SEED, hmc_leapfrog=4)
    with pytest.raises(bq.BusseqError):
        c.checkpoint_load(path)
    c.close()
    b = bq.Sampler(Y, N_B, K, seed=SEED, hmc_leapfrog=4, hmc_gene_accept=True)
    b.checkpoint_load(path)
    b.sweeps(19)
    b.finish()
    st2 = b.get_state()
    b.close()
    for k in st_ref:
        assert np.array_equal(st_ref[k], st2[k]), k
