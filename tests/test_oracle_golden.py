"""Pin the FP64 oracle against the reference's OWN kernels.

tests/golden/ref_kernels.npz holds seeded inputs and the outputs of the
reference BUSseq_gpu.cu kernels run on a GPU (tests/golden/make_ref_golden.py,
oracle/ref_harness.cpp).  Every formula the oracle restates and the kernels of
this package implement is compared here, on the CPU, at FP64 tolerance.
"""
import numpy as np
import pytest

from oracle import pyoracle as po

RTOL = 1e-10


def _unpack(d):
    B, K, G, N = (int(x) for x in d["in_dims"])
    n_b = d["in_n_b"]
    off = np.concatenate([[0], np.cumsum(n_b)])
    bat = np.repeat(np.arange(B), n_b)
    s = dict(B=B, K=K, G=G, N=N, n_b=n_b, off=off, bat=bat)
    for k in d.files:
        if k.startswith("in_"):
            s[k[3:]] = d[k]
    s["Y"] = s["Y"].reshape(N, G)
    s["X"] = s["X"].reshape(N, G)
    s["Z"] = s["Z"].reshape(N, G)
    s["beta"] = s["beta"].reshape(K, G)
    s["beta_prop"] = s["beta_prop"].reshape(K - 1, G)
    s["nu"] = s["nu"].reshape(B, G)
    s["nu_prop"] = s["nu_prop"].reshape(B - 1, G)
    s["phi"] = s["phi"].reshape(B, G)
    s["phi_prop"] = s["phi_prop"].reshape(B, G)
    s["gamma"] = s["gamma"].reshape(2, B)
    s["gamma_prop"] = s["gamma_prop"].reshape(2, B)
    s["pi"] = s["pi"].reshape(B, K)
    return s


def _close(got, want, rtol=RTOL, atol=1e-11):
    got, want = np.asarray(got, float), np.asarray(want, float)
    scale = np.maximum(np.abs(want), 1.0)
    err = np.abs(got - want) / scale
    assert np.all(err <= rtol + atol), "max scaled err %.3g" % err.max()


@pytest.fixture(scope="module")
def S(golden):
    return _unpack(golden)


def test_alpha_terms(S, golden):
    L = po.lib()
    ref = golden["out_alpha_terms"].reshape(S["G"], S["N"])
    got = np.zeros_like(ref)
    for g in range(S["G"]):
        for i in range(S["N"]):
            b = S["bat"][i]
            m = S["beta"][S["W"][i], g] + S["nu"][b, g] + S["delta"][i]
            got[g, i] = L.orc_term_shift(S["alpha"][g], S["alpha_prop"][g], m, S["phi"][b, g], int(S["X"][i, g]))
    _close(got, ref)


def test_beta_terms(S, golden):
    L = po.lib()
    K, G, N = S["K"], S["G"], S["N"]
    ref = golden["out_beta_terms"].reshape(K - 1, G, N)
    got = np.zeros_like(ref)
    for k in range(1, K):
        for g in range(G):
            for i in range(N):
                if S["W"][i] != k:
                    continue
                b = S["bat"][i]
                m = S["alpha"][g] + S["nu"][b, g] + S["delta"][i]
                got[k - 1, g, i] = L.orc_term_shift(S["beta"][k, g], S["beta_prop"][k - 1, g], m,
                                                    S["phi"][b, g], int(S["X"][i, g]))
    _close(got, ref)


def test_nu_terms(S, golden):
    L = po.lib()
    B, G = S["B"], S["G"]
    ref = golden["out_nu_terms"]
    got = []
    for b in range(1, B):
        for g in range(G):
            for i in range(S["off"][b], S["off"][b + 1]):
                m = S["alpha"][g] + S["beta"][S["W"][i], g] + S["delta"][i]
                got.append(L.orc_term_shift(S["nu"][b, g], S["nu_prop"][b - 1, g], m, S["phi"][b, g],
                                            int(S["X"][i, g])))
    _close(got, ref)


def test_delta_terms(S, golden):
    L = po.lib()
    N, G = S["N"], S["G"]
    ref = golden["out_delta_terms"].reshape(N, G)
    got = np.zeros_like(ref)
    for i in range(N):
        b = S["bat"][i]
        for g in range(G):
            m = S["alpha"][g] + S["beta"][S["W"][i], g] + S["nu"][b, g]
            got[i, g] = L.orc_term_shift(S["delta"][i], S["delta_prop"][i], m, S["phi"][b, g], int(S["X"][i, g]))
    _close(got, ref)


def test_phi_terms(S, golden):
    L = po.lib()
    B, G = S["B"], S["G"]
    ref = golden["out_phi_terms"]
    got = []
    for b in range(B):
        for g in range(G):
            for i in range(S["off"][b], S["off"][b + 1]):
                eta = np.exp(S["alpha"][g] + S["beta"][S["W"][i], g] + S["nu"][b, g] + S["delta"][i])
                got.append(L.orc_term_phi(S["phi"][b, g], S["phi_prop"][b, g], eta, int(S["X"][i, g])))
    _close(got, ref, rtol=1e-9)


def test_W_terms(S, golden):
    L = po.lib()
    N, G = S["N"], S["G"]
    ref = golden["out_W_terms"].reshape(N, G)
    got = np.zeros_like(ref)
    for i in range(N):
        b = S["bat"][i]
        for g in range(G):
            m = S["alpha"][g] + S["nu"][b, g] + S["delta"][i]
            got[i, g] = L.orc_term_shift(S["beta"][S["W"][i], g], S["beta"][S["W_prop"][i], g], m, S["phi"][b, g],
                                         int(S["X"][i, g]))
    _close(got, ref)


def test_gamma_terms(S, golden):
    L = po.lib()
    B, G = S["B"], S["G"]
    r0, r1 = golden["out_gamma0_terms"], golden["out_gamma1_terms"]
    g0, g1 = [], []
    for b in range(B):
        for i in range(S["off"][b], S["off"][b + 1]):
            for g in range(G):
                X, Z = int(S["X"][i, g]), int(S["Z"][i, g])
                g0.append(L.orc_term_gamma0(S["gamma"][0, b], S["gamma_prop"][0, b], S["gamma"][1, b], X, Z))
                g1.append(L.orc_term_gamma1(S["gamma"][0, b], S["gamma"][1, b], S["gamma_prop"][1, b], X, Z))
    _close(g0, r0)
    _close(g1, r1)


def _oracle_state_from(S):
    st = po.State(S["Y"], S["n_b"], S["K"], seed=1)
    st.X[:] = S["X"]
    st.Z[:] = S["Z"].astype(np.uint8)
    st.W[:] = S["W"]
    st.alpha[:] = S["alpha"]
    st.beta[:] = S["beta"]
    st.nu[:] = S["nu"]
    st.delta[:] = S["delta"]
    st.phi[:] = S["phi"]
    st.gamma[:] = S["gamma"]
    st.pi[:] = S["pi"]
    return st


def test_bic(S, golden):
    st = _oracle_state_from(S)
    bic, ll = st.bic()
    _close(ll, golden["out_ll_partial"].reshape(S["K"], S["N"]), rtol=1e-11)
    part = golden["out_ll_partial"].reshape(S["K"], S["N"])
    # reference fill_log_likelihood_2 per cell, then BUSseq_gpu.cu:1833
    ll2 = golden["out_ll2_terms"]
    mx = part.max(axis=0)
    mine = mx + np.log((S["pi"][S["bat"]].T * np.exp(part - mx)).sum(axis=0))
    _close(mine, ll2, rtol=1e-12)
    B, G, N, K = S["B"], S["G"], S["N"], S["K"]
    nparam = (B + G) * K + 2 * B + G * (B * 2 - 1) + N - B
    want = -2 * ll2.sum() + np.log(G * N) * nparam
    _close([bic], [want], rtol=1e-12)


def test_init_given_W(S, golden):
    st = _oracle_state_from(S)
    st.W[:] = golden["out_init_W"]
    raw, bm = st.init_given_W()
    np.testing.assert_array_equal(st.Y.sum(axis=1), golden["out_libsize"])
    _close(st.delta, golden["out_init_delta"], rtol=1e-12)
    _close(raw.ravel(), golden["out_init_raw_means"], rtol=1e-11)
    _close(st.nu.ravel(), golden["out_init_nu"], rtol=1e-11)
    _close(st.phi.ravel(), golden["out_init_phi"])
    _close(st.pi.ravel(), golden["out_init_pi"])
    _close(bm, golden["out_init_batch_means"], rtol=1e-11)
    # alpha = mu_alpha = raw[0][0], beta_k = raw[0][k] - raw[0][0]  (BUSseq_gpu.cu:456, :1227)
    _close(st.alpha, raw[0, 0])
    _close(st.beta[1:], raw[0, 1:] - raw[0, 0][None, :])
    _close(st.mu_nu[1:], bm[1:] - bm[0], rtol=1e-11)


def test_mode(S, golden):
    counts = golden["in_mode_counts"].reshape(S["K"], S["N"])
    np.testing.assert_array_equal(np.argmax(counts, axis=0), golden["out_mode_W"])
