"""Chain-level comparison of two BUSseq chains -- TEST INFRASTRUCTURE ONLY.

Summarises the kept draws of a chain (posterior mean, batch-means standard
error and ESS-based Monte Carlo standard error of every scalar) and compares
two chains that ran on the same data: this project's sampler and the
reference's own kernels (oracle/ref_chain.cpp).  The chains use different
random number generators, so agreement can only be statistical: per scalar,
z = (mean_a - mean_b) / sqrt(se_a^2 + se_b^2), and the fraction of scalars
with |z| > 3 is reported per parameter block.

Cell-type labels are only defined up to a permutation.  The types of chain b
are matched to those of chain a by the Hungarian assignment on the confusion
matrix of the two posterior-mode labelings.  alpha, beta, L, p and tau0 depend
on which type is the baseline (type 0 has beta = 0); they are compared
directly only when the assignment keeps type 0 as the baseline.  The
label-free type means alpha_g + beta_gk are always compared.

Blocks and their layouts follow the reference's preserved files
(BUSseq_gpu.cu:1845-2018): gamma [2B], alpha [G], L and beta [(K-1)G],
p_tau0 [2], nu [(B-1)G], delta [N], phi [BG], pi [BK], W [N].
"""
from __future__ import annotations

import numpy as np

BLOCKS = ("gamma", "alpha", "beta", "L", "p_tau0", "nu", "delta", "phi", "pi", "typemean")


def batch_means_se(draws: np.ndarray) -> np.ndarray:
    """Batch-means standard error of the mean of every row (scalars x sweeps),
    with floor(sqrt(n)) batches of equal length (the first n mod batches
    draws are dropped)."""
    x = np.asarray(draws, dtype=np.float64)
    n = x.shape[1]
    nb = max(2, int(np.floor(np.sqrt(n))))
    m = n // nb
    xb = x[:, n - nb * m:].reshape(x.shape[0], nb, m).mean(axis=2)
    return xb.std(axis=1, ddof=1) / np.sqrt(nb)


def ess_se(draws: np.ndarray) -> np.ndarray:
    """Monte Carlo standard error sd / sqrt(ESS), ESS by Geyer's initial
    monotone sequence; 0 for rows that do not move."""
    from busseq_gpu_gb300.diagnostics import ess_geyer  # numpy only: the library is not loaded
    x = np.asarray(draws, dtype=np.float64)
    e = ess_geyer(x)
    sd = x.std(axis=1, ddof=1)
    out = np.zeros(x.shape[0])
    ok = np.isfinite(e) & (sd > 0)
    out[ok] = sd[ok] / np.sqrt(e[ok])
    return out


def posterior_mode(W_draws: np.ndarray, K: int) -> np.ndarray:
    """Posterior mode of every cell's type, ties to the smallest type
    (BUSseq_gpu.cu:944-959)."""
    counts = np.stack([(W_draws == k).sum(axis=1) for k in range(K)], axis=1)
    return counts.argmax(axis=1).astype(np.int32)


def summarise(pres: dict, B: int, K: int, G: int) -> dict:
    """Per-block mean, batch-means SE, ESS SE and sd from a chain's kept draws
    (a dict in the reference's preserved layouts)."""
    out = {}
    n = pres["alpha"].shape[1]
    blocks = {k: np.asarray(pres[k], dtype=np.float64) for k in ("gamma", "alpha", "beta", "L", "p_tau0", "nu",
                                                                   "delta", "phi", "pi")}
    beta_full = np.concatenate([np.zeros((G, n)), blocks["beta"]], axis=0)  # [K*G][n], type 0 first
    blocks["typemean"] = beta_full + np.tile(blocks["alpha"], (K, 1))      # alpha_g + beta_gk, [k*G + g]
    for name, x in blocks.items():
        out[name] = {"mean": x.mean(axis=1), "se_bm": batch_means_se(x), "se_ess": ess_se(x),
                     "sd": x.std(axis=1, ddof=1)}
    out["W_mode"] = posterior_mode(np.asarray(pres["W"]), K)
    out["n_kept"] = n
    return out


def match_types(W_a: np.ndarray, W_b: np.ndarray, K: int) -> np.ndarray:
    """perm[k_b] = k_a maximising the agreement of the two labelings."""
    from scipy.optimize import linear_sum_assignment
    conf = np.zeros((K, K), np.int64)
    np.add.at(conf, (np.asarray(W_b), np.asarray(W_a)), 1)
    rows, cols = linear_sum_assignment(-conf)
    perm = np.empty(K, np.int64)
    perm[rows] = cols
    return perm


def permute_block(name: str, v: np.ndarray, perm: np.ndarray, B: int, K: int, G: int) -> np.ndarray:
    """Block `name` of chain b laid out with chain a's type labels."""
    if name == "pi":
        out = np.empty_like(v)
        for b in range(B):
            out[b * K + perm] = v[b * K:(b + 1) * K]
        return out
    if name == "typemean":
        out = np.empty_like(v)
        for k in range(K):
            out[perm[k] * G:(perm[k] + 1) * G] = v[k * G:(k + 1) * G]
        return out
    if name in ("beta", "L"):  # rows k = 1..K-1; valid only when perm[0] == 0
        out = np.empty_like(v)
        for k in range(1, K):
            out[(perm[k] - 1) * G:perm[k] * G] = v[(k - 1) * G:k * G]
        return out
    return v


def compare(a: dict, b: dict, B: int, K: int, G: int, W_true=None) -> dict:
    """Statistical comparison of chain summaries a and b (from summarise)."""
    from busseq_gpu_gb300.diagnostics import adjusted_rand_index as ari
    perm = match_types(a["W_mode"], b["W_mode"], K)
    base_kept = bool(perm[0] == 0)
    rec = {"perm_b_to_a": [int(x) for x in perm], "baseline_type_matched": base_kept, "blocks": {}}
    if W_true is not None:
        rec["ari_a"] = ari(a["W_mode"], W_true)
        rec["ari_b"] = ari(b["W_mode"], W_true)
        rec["ari_diff"] = rec["ari_a"] - rec["ari_b"]
    rec["ari_a_vs_b"] = ari(a["W_mode"], b["W_mode"])
    for name in BLOCKS:
        if name in ("alpha", "beta", "L", "p_tau0") and not base_kept:
            continue
        sa, sb = a[name], b[name]
        mb = permute_block(name, sb["mean"], perm, B, K, G)
        stats = {}
        for kind in ("se_bm", "se_ess"):
            se = np.sqrt(sa[kind] ** 2 + permute_block(name, sb[kind], perm, B, K, G) ** 2)
            d = sa["mean"] - mb
            z = np.where(se > 0, d / np.where(se > 0, se, 1.0), np.where(d == 0, 0.0, np.inf))
            stats[kind] = {"frac_abs_z_gt_3": float(np.mean(np.abs(z) > 3)), "median_abs_z": float(np.median(np.abs(z))),
                           "max_abs_z": float(np.max(np.abs(z)))}
        # the same test where both chains' ESS (sd / MCSE)^2 reach a floor: the
        # MCSE of a chain with only a few effective draws is itself unreliable
        sb_se = permute_block(name, sb["se_ess"], perm, B, K, G)
        sb_sd = permute_block(name, sb["sd"], perm, B, K, G)
        ess_a = np.where(sa["se_ess"] > 0, (sa["sd"] / np.where(sa["se_ess"] > 0, sa["se_ess"], 1.0)) ** 2, 0.0)
        ess_b = np.where(sb_se > 0, (sb_sd / np.where(sb_se > 0, sb_se, 1.0)) ** 2, 0.0)
        se = np.sqrt(sa["se_ess"] ** 2 + sb_se ** 2)
        z = np.where(se > 0, (sa["mean"] - mb) / np.where(se > 0, se, 1.0), 0.0)
        stats["median_ess"] = [float(np.median(ess_a)), float(np.median(ess_b))]
        for floor in (30, 100):
            m = (ess_a >= floor) & (ess_b >= floor) & (se > 0)
            stats["ess_ge_%d" % floor] = {"coords": int(m.sum()),
                                          "frac_abs_z_gt_3": float(np.mean(np.abs(z[m]) > 3)) if m.any() else None,
                                          "mean_z": float(np.mean(z[m])) if m.any() else None}
        stats["mean_z"] = float(np.mean(z[se > 0])) if (se > 0).any() else 0.0
        sd = np.sqrt(0.5 * (sa["sd"] ** 2 + sb_sd ** 2))
        dd = np.abs(sa["mean"] - mb)
        rel = dd[sd > 0] / sd[sd > 0]
        stats["coords"] = int(sa["mean"].size)
        stats["median_abs_diff_over_sd"] = float(np.median(rel)) if rel.size else 0.0
        stats["max_abs_diff"] = float(dd.max())
        rec["blocks"][name] = stats
    return rec


def to_npz_dict(prefix: str, s: dict) -> dict:
    out = {prefix + "W_mode": s["W_mode"], prefix + "n_kept": np.array(s["n_kept"])}
    for name in BLOCKS:
        for kind in ("mean", "se_bm", "se_ess", "sd"):
            out["%s%s/%s" % (prefix, name, kind)] = np.asarray(s[name][kind], dtype=np.float64)
    return out


def from_npz(z, prefix: str) -> dict:
    s = {"W_mode": z[prefix + "W_mode"], "n_kept": int(z[prefix + "n_kept"])}
    for name in BLOCKS:
        s[name] = {kind: z["%s%s/%s" % (prefix, name, kind)] for kind in ("mean", "se_bm", "se_ess", "sd")}
    return s
