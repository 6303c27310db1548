"""Parity of every conditional update of the CUDA kernels with the FP64 oracle.

Each test puts the same state on the GPU (through the C ABI) and in the
oracle, runs one stage of the sweep at the same sweep index (so both consume
the same Philox uniforms), and compares.  Fused kernels are checked one
conditional at a time: after a discrete step, the oracle continues from the
kernels' result, so a certified near-tie cannot cascade into later checks.
"""
import numpy as np
import pytest

import busseq_gpu_gb300 as bq
from oracle import pyoracle as po
from tests.parity_util import LR_ATOL, check_discrete, check_mh, lr_ok, oracle_state

pytestmark = pytest.mark.gpu

CASES = {
    # name: (n_b, G, K, seed, warm sweeps)
    "small_init": ([40, 30, 30], 256, 4, 11, 0),
    "small_warm": ([40, 30, 30], 256, 4, 12, 25),
    "demo_warm": ([300, 300, 200, 200], 3000, 5, 13579, 30),
    "ragged_warm": ([9, 61, 17, 33, 5], 333, 5, 7, 15),
    "minimal_warm": ([12, 9], 97, 2, 3, 10),                      # B = 2, K = 2
    "many_types_warm": ([20, 35, 50, 25, 40, 30], 150, 12, 9, 10),  # B = 6, K = 12
    # the headline shape (4 batches, G = 10^4, K = 8) on a cell subset the oracle runs in seconds
    "config1_shape": ([250, 250, 250, 250], 10000, 8, 13580, 20),
    # the large uneven workload's shape: 6 batches in its 2:5:8:12:20:3 ratio, G = 2*10^4,
    # K = 12, 15 % differential genes and phi ~ U(2, 30) ("wide" generator)
    "config4_shape": ([80, 200, 320, 480, 800, 120], 20000, 12, 13583, 10),
}
WIDE = {"config4_shape"}


@pytest.fixture(scope="module", params=list(CASES))
def case(request):
    n_b, G, K, seed, warm = CASES[request.param]
    sim = bq.CONFIG_SIM["wide" if request.param in WIDE else "default"]
    Y, W_true, _ = bq.simulate(n_b, G, K, seed, **sim)
    s = bq.Sampler(Y, n_b, K, seed=seed, p0=0.3)
    if warm:
        s.begin(warm, warm, 0)
        s.sweeps(warm)
        s.synchronize()
    st = s.get_state()
    yield dict(name=request.param, s=s, Y=Y, n_b=np.array(n_b), K=K, seed=seed, st=st)
    s.close()


def _gpu_stage(c, stage, it, n_unchanged=1 << 30):
    s = c["s"]
    s.set_state(c["st"])
    s.run_stage(stage, it, n_unchanged)
    return s.get_state(), s.log_ratios()


def test_stage_zx_gamma_alpha_L_ptau(case):
    c = case
    it, n_unch = 41, 10
    g, lr = _gpu_stage(c, 0, it, n_unch)
    Y, st0 = c["Y"], c["st"]
    o = oracle_state(Y, c["n_b"], c["K"], c["seed"], st0)
    d = po.Debug(o)
    rep = {}
    # Z / X (BUSseq_gpu.cu:484-512)
    o.step("zx", it, debug=d)
    y0 = Y == 0
    check_discrete("X", g["X"], o.X, d.mg_zx, mask=y0, report=rep)
    check_discrete("Z", g["Z"], o.Z, d.mg_zx, mask=y0, report=rep)
    assert np.array_equal(g["X"][~y0], Y[~y0]) and not g["Z"][~y0].any()
    assert np.all(g["X"][y0 & (g["Z"] == 0)] == 0)
    assert np.all(g["Z"][y0 & (g["X"] > 0)] == 1)
    # gamma0, gamma1, continuing from the kernels' X and Z
    o.X[:] = g["X"]
    o.Z[:] = g["Z"]
    o.step("gamma", it, debug=d)
    B = len(c["n_b"])
    f0 = check_mh("gamma0", st0["gamma"][0], g["gamma"][0], o.gamma[0], lr["gamma"][0], d.lr_gamma[0],
                  d.mg_gamma[0], report=rep, scale=d.sc_gamma[0])
    same0 = (g["gamma"][0] != st0["gamma"][0]) == (o.gamma[0] != st0["gamma"][0])
    check_mh("gamma1", st0["gamma"][1], g["gamma"][1], o.gamma[1], lr["gamma"][1], d.lr_gamma[1],
             d.mg_gamma[1], mask=same0, report=rep, scale=d.sc_gamma[1])
    # alpha (BUSseq_gpu.cu:602-632)
    o.step("alpha", it, debug=d)
    check_mh("alpha", st0["alpha"], g["alpha"], o.alpha, lr["alpha"], d.lr_alpha, d.mg_alpha, report=rep,
             scale=d.sc_alpha)
    # L from the old beta, p, tau0 (BUSseq_gpu.cu:634-648)
    o.step("L", it, debug=d)
    check_discrete("L", g["L"][1:], o.L[1:], d.mg_L[1:], report=rep)
    # p, tau0 from the kernels' L (BUSseq_gpu.cu:650-668): each is compared unless its
    # own Gamma rejection step is a certified near-tie (margin <= 1e-5)
    o.L[:] = g["L"]
    o.step("ptau", it, debug=d)
    checked = d.mg_ptau > 1e-5
    np.testing.assert_allclose(g["p_tau0"][checked], o.p_tau0[checked], rtol=1e-5)
    rep["p_tau0_checked"] = int(checked.sum())
    print(c["name"], rep, "gamma0 flips", f0)


def test_stage_beta_nu(case):
    c = case
    it = 57
    g, lr = _gpu_stage(c, 1, it)
    st0 = c["st"]
    o = oracle_state(c["Y"], c["n_b"], c["K"], c["seed"], st0)
    d = po.Debug(o)
    rep = {}
    o.step("beta", it, debug=d)
    check_mh("beta", st0["beta"][1:], g["beta"][1:], o.beta[1:], lr["beta"][1:], d.lr_beta[1:], d.mg_beta[1:],
             report=rep, scale=d.sc_beta[1:])
    assert np.all(g["beta"][0] == 0)
    o.beta[:] = g["beta"]
    o.step("nu", it, debug=d)
    check_mh("nu", st0["nu"][1:], g["nu"][1:], o.nu[1:], lr["nu"][1:], d.lr_nu[1:], d.mg_nu[1:], report=rep,
             scale=d.sc_nu[1:])
    assert np.all(g["nu"][0] == 0)
    print(c["name"], rep)


def test_stage_delta(case):
    c = case
    it = 63
    g, lr = _gpu_stage(c, 2, it)
    st0 = c["st"]
    o = oracle_state(c["Y"], c["n_b"], c["K"], c["seed"], st0)
    d = po.Debug(o)
    o.step("delta", it, debug=d)
    first = np.zeros(len(st0["delta"]), bool)
    first[np.concatenate([[0], np.cumsum(c["n_b"])[:-1]])] = True
    rep = {}
    check_mh("delta", st0["delta"], g["delta"], o.delta, lr["delta"], d.lr_delta, d.mg_delta, mask=~first,
             report=rep, scale=d.sc_delta)
    assert np.array_equal(g["delta"][first], st0["delta"][first])
    print(c["name"], rep)


def test_stage_phi(case):
    c = case
    it = 71
    g, lr = _gpu_stage(c, 3, it)
    st0 = c["st"]
    o = oracle_state(c["Y"], c["n_b"], c["K"], c["seed"], st0)
    d = po.Debug(o)
    o.step("phi", it, debug=d)
    rep = {}
    check_mh("phi", st0["phi"], g["phi"], o.phi, lr["phi"], d.lr_phi, d.mg_phi, report=rep, scale=d.sc_phi)
    print(c["name"], rep)


def test_stage_W_mh(case):
    c = case
    it = 83
    g, lr = _gpu_stage(c, 4, it)
    st0 = c["st"]
    o = oracle_state(c["Y"], c["n_b"], c["K"], c["seed"], st0)
    d = po.Debug(o)
    o.step("W", it, w_update=0, debug=d)
    dlr = np.abs(lr["W"] - d.lr_W)
    assert np.all(lr_ok(lr["W"], d.lr_W, d.sc_W)), dlr.max()
    flip = g["W"] != o.W
    assert np.all(d.mg_W[flip] <= dlr[flip] + 1e-6), (np.flatnonzero(flip), d.mg_W[flip], dlr[flip])
    print(c["name"], "W moved", int((g["W"] != st0["W"]).sum()), "flips", int(flip.sum()), "max dlr", dlr.max())


def test_stage_W_gibbs(case):
    c = case
    it = 89
    Y = c["Y"]
    s = bq.Sampler(Y, c["n_b"], c["K"], seed=c["seed"], w_update="gibbs")
    try:
        s.set_state(c["st"])
        s.run_stage(4, it)
        g = s.get_state()
        lr = s.log_ratios()
    finally:
        s.close()
    o = oracle_state(Y, c["n_b"], c["K"], c["seed"], c["st"])
    d = po.Debug(o)
    o.step("W", it, w_update=1, debug=d)
    # Where both drew the same type, the log weight of that type relative to the
    # current one (K sums over the genes in float) must agree within the log-ratio
    # tolerance (with the size of its float pieces); the largest such error eps
    # measured on this very case bounds how
    # far a boundary of the categorical distribution function can move (by at
    # most max |d log w_j - d log w_k| <= 2 eps), so a differing draw is a
    # certified near-tie only where the oracle's uniform lies within 2 eps of a
    # boundary, and such draws are at most 0.1 % of the cells.
    same = g["W"] == o.W
    dlr = np.abs(lr["W"] - d.lr_W)
    assert np.all(lr_ok(lr["W"][same], d.lr_W[same], d.sc_W[same])), dlr[same].max()
    eps = float(dlr[same].max()) if same.any() else LR_ATOL
    rep = {"max_dlr": eps}
    check_discrete("W_gibbs", g["W"], o.W, d.mg_W, tol=2.0 * eps + 1e-9, max_frac=1e-3, report=rep)
    print(c["name"], rep)


def test_stage_pi_and_order(case):
    c = case
    it = 97
    g, _ = _gpu_stage(c, 5, it)
    st0 = c["st"]
    o = oracle_state(c["Y"], c["n_b"], c["K"], c["seed"], st0)
    d = po.Debug(o)
    o.step("pi", it, debug=d)
    ok = d.mg_pi.min(axis=1) > 1e-5
    np.testing.assert_allclose(g["pi"][ok], o.pi[ok], rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(g["pi"].sum(axis=1), 1.0, rtol=1e-5)
