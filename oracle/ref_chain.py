"""Whole-chain comparison with the reference's own kernels -- TEST INFRASTRUCTURE.

Runs, on one GPU, on the same synthetic data (the BUSseq generative model at the
demo size: batches of 300/300/200/200 cells, G = 3000, K = 5, seed 13579):

  1. the reference chain: oracle/lib/ref_chain replays the reference program's
     initialisation, burn-in and kept sweeps with the reference's kernels from
     oracle/_ref/busseq_ref.cubin (pi drawn on the host; see ref_chain.cpp);
  2. this project's sampler (the plain MH sampler, the reference's moves), with
     the same run lengths, started from the reference chain's initial state
     (so both chains have the same distribution at every sweep, and the
     cell-type labels agree);

and compares the two chains with oracle/chain_compare.py: ARI of the
posterior-mode cell types against the simulated types, and per-scalar z-scores
of the posterior means.  Writes <out>/ref_chain_<name>.json (the record) and
<out>/ref_chain_<name>.npz (per-scalar means and standard errors of both
chains, the types; what tests/test_ref_chain_parity.py replays).

The cubin is compiled from the reference source by oracle/build.py where that
source exists and travels with the checkout otherwise.

usage: python oracle/ref_chain.py [--iters 1000 --burnin 500 --unchanged 300]
                                  [--out DIR] [--name config0]
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

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)

CONFIG0 = dict(n_b=[300, 300, 200, 200], G=3000, K=5, seed=13579)
# a small problem on which the reference's sweep takes ~0.1 s, so that long
# chains give every block enough effective draws for a Monte Carlo error test
SMALL = dict(n_b=[60, 50, 40, 50], G=300, K=4, seed=2468)
CASES = {"config0": CONFIG0, "small": SMALL}


def _ref_binary(Y, n_b, K, seed, n_iter, n_burnin, n_unchanged, workdir, timeout, env=None):
    from oracle import build
    cubin = build.build_ref_cubin()
    exe = build.build_ref_chain()
    if not cubin or not os.path.exists(cubin) or not exe:
        raise RuntimeError("the reference cubin or oracle/lib/ref_chain is not available")
    ypath = os.path.join(workdir, "Y.i32")
    if not os.path.exists(ypath):
        np.ascontiguousarray(Y, dtype=np.int32).tofile(ypath)
    G = Y.shape[1]
    cmd = [exe, cubin, ypath, str(G), str(K), str(seed), str(n_iter), str(n_burnin), str(n_unchanged), workdir,
           *[str(n) for n in n_b]]
    t0 = time.perf_counter()
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=timeout,
                       env=dict(os.environ, **(env or {})))
    wall = time.perf_counter() - t0
    info = json.loads(r.stdout.strip().splitlines()[-1]) if r.stdout.strip() else {}
    if r.returncode != 0:
        raise RuntimeError("ref_chain failed (rc %d): %s %s" % (r.returncode, r.stderr[-2000:], info))
    info["wall_s"] = wall
    return info


def _read_init(workdir, Y, B, K, G):
    def ini(name, dtype):
        return np.fromfile(os.path.join(workdir, "init_%s.bin" % name), dtype=dtype)

    return {"X": np.ascontiguousarray(Y, dtype=np.int32), "Z": np.zeros(Y.shape, np.uint8),
            "W": ini("W", np.int32), "L": ini("L", np.int32).astype(np.int8).reshape(K, G),
            "alpha": ini("alpha", np.float64), "mu_alpha": ini("mu_alpha", np.float64),
            "beta": ini("beta", np.float64).reshape(K, G), "nu": ini("nu", np.float64).reshape(B, G),
            "mu_nu": np.concatenate([[0.0], ini("mu_nu", np.float64)]), "delta": ini("delta", np.float64),
            "mu_delta": ini("mu_delta", np.float64), "phi": ini("phi", np.float64).reshape(B, G),
            "gamma": ini("gamma", np.float64).reshape(2, B), "pi": ini("pi", np.float64).reshape(B, K),
            "p_tau0": ini("p", np.float64)}


def _read_preserved(workdir, n_b, K, G, n):
    B, N = len(n_b), int(sum(n_b))

    def rd(name, dtype, rows):
        return np.fromfile(os.path.join(workdir, "preserved_%s.bin" % name), dtype=dtype).reshape(rows, n)

    return {"gamma": rd("gamma", np.float64, 2 * B), "alpha": rd("alpha", np.float64, G),
            "L": rd("L", np.int32, (K - 1) * G), "beta": rd("beta", np.float64, (K - 1) * G),
            "p_tau0": rd("p", np.float64, 2), "nu": rd("nu", np.float64, (B - 1) * G),
            "delta": rd("delta", np.float64, N), "phi": rd("phi", np.float64, B * G),
            "W": rd("W", np.int32, N), "pi": rd("pi", np.float64, B * K)}


def _write_start(workdir, st):
    """A state of this sampler as the reference runner's start files."""
    files = {"X": (st["X"], np.int32), "Z": (st["Z"], np.int32), "W": (st["W"], np.int32), "L": (st["L"], np.int32),
             "alpha": (st["alpha"], np.float64), "beta": (st["beta"], np.float64), "nu": (st["nu"], np.float64),
             "delta": (st["delta"], np.float64), "phi": (st["phi"], np.float64), "gamma": (st["gamma"], np.float64),
             "pi": (st["pi"], np.float64), "p": (st["p_tau0"], np.float64)}
    for name, (v, dt) in files.items():
        np.ascontiguousarray(v, dtype=dt).ravel().tofile(os.path.join(workdir, "start_%s.bin" % name))


def run_stationary(Y, n_b, K, seed, start_sweeps, n_iter, n_burnin, timeout):
    """Both samplers from one state in the posterior's bulk: this sampler runs
    `start_sweeps` sweeps from the reference's initial state; from the state it
    reaches, each sampler then runs n_iter sweeps (n_burnin not kept) with p and
    tau0 updated throughout, and the kept draws are compared."""
    import busseq_gpu_gb300 as bq
    B, G = len(n_b), Y.shape[1]
    with tempfile.TemporaryDirectory() as wd:
        info0 = _ref_binary(Y, n_b, K, seed, 1, 0, 0, wd, timeout, env={"REF_CHAIN_INIT_ONLY": "1"})
        init = _read_init(wd, Y, B, K, G)
        t0 = time.perf_counter()
        s = bq.Sampler(Y, n_b, K, seed=seed, p0=info0["p0"], keep_draws=True)
        s.set_state(init)
        s.begin(start_sweeps + n_iter, start_sweeps + n_burnin, 0)
        s.sweeps(start_sweeps)
        s.synchronize()
        start = s.get_state()
        s.sweeps(n_iter)
        s.finish()
        ours_wall = time.perf_counter() - t0
        ours = s.preserved()
        s.close()
        _write_start(wd, start)
        info = _ref_binary(Y, n_b, K, seed, n_iter, n_burnin, 0, wd, timeout, env={"REF_CHAIN_START_DIR": wd})
        ref = _read_preserved(wd, n_b, K, G, n_iter - n_burnin)
    info["start"] = {"sweeps_of_this_sampler_from_the_reference_init": start_sweeps}
    return ref, info, ours, {"wall_s": ours_wall, "sweeps_per_s": (start_sweeps + n_iter) / ours_wall}


def run_reference(Y, n_b, K, seed, n_iter, n_burnin, n_unchanged, workdir, timeout):
    info = _ref_binary(Y, n_b, K, seed, n_iter, n_burnin, n_unchanged, workdir, timeout)
    B, N, n = len(n_b), int(sum(n_b)), n_iter - n_burnin

    def rd(name, dtype, rows):
        return np.fromfile(os.path.join(workdir, "preserved_%s.bin" % name), dtype=dtype).reshape(rows, n)

    pres = {"gamma": rd("gamma", np.float64, 2 * B), "alpha": rd("alpha", np.float64, G),
            "L": rd("L", np.int32, (K - 1) * G), "beta": rd("beta", np.float64, (K - 1) * G),
            "p_tau0": rd("p", np.float64, 2), "nu": rd("nu", np.float64, (B - 1) * G),
            "delta": rd("delta", np.float64, N), "phi": rd("phi", np.float64, B * G),
            "W": rd("W", np.int32, N), "pi": rd("pi", np.float64, B * K)}

    return pres, info, _read_init(workdir, Y, B, K, G)


def run_ours(Y, n_b, K, seed, p0, n_iter, n_burnin, n_unchanged, init=None):
    """This sampler's chain, started from `init` (the reference's initial
    state) when given, else from its own initialisation."""
    import busseq_gpu_gb300 as bq
    t0 = time.perf_counter()
    s = bq.Sampler(Y, n_b, K, seed=seed, p0=p0, keep_draws=True)
    if init is not None:
        s.set_state(init)
    s.run(n_iter, n_burnin, n_unchanged)
    wall = time.perf_counter() - t0
    pres = s.preserved()
    s.close()
    return pres, {"wall_s": wall, "sweeps_per_s": n_iter / wall}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--iters", type=int, default=1000)
    ap.add_argument("--burnin", type=int, default=500)
    ap.add_argument("--unchanged", type=int, default=300)
    ap.add_argument("--out", default=os.path.join(ROOT, "gpurun_out"))
    ap.add_argument("--name", default="config0")
    ap.add_argument("--data", default="config0", choices=sorted(CASES),
                    help="config0: 300/300/200/200 cells, G = 3000, K = 5; small: 60/50/40/50 cells, G = 300, K = 4")
    ap.add_argument("--timeout", type=int, default=3000, help="seconds allowed for the reference chain")
    ap.add_argument("--start-sweeps", type=int, default=0,
                    help="> 0: compare the stationary chains: this sampler first runs this many sweeps from the "
                         "reference's initial state, then both samplers run --iters sweeps from the state reached "
                         "(--unchanged is then 0)")
    ap.add_argument("--own-init", action="store_true",
                    help="start this sampler from its own initialisation instead of the reference's initial state")
    args = ap.parse_args()
    from oracle import chain_compare as cc
    import busseq_gpu_gb300 as bq

    cfg = CASES[args.data]
    n_b, G, K, seed = cfg["n_b"], cfg["G"], cfg["K"], cfg["seed"]
    B = len(n_b)
    Y, W_true, _ = bq.simulate(n_b, G, K, seed)
    os.makedirs(args.out, exist_ok=True)
    if args.start_sweeps > 0:
        ref_pres, ref_info, ours_pres, ours_info = run_stationary(Y, n_b, K, seed, args.start_sweeps, args.iters,
                                                                  args.burnin, args.timeout)
    else:
        with tempfile.TemporaryDirectory() as wd:
            ref_pres, ref_info, init = run_reference(Y, n_b, K, seed, args.iters, args.burnin, args.unchanged, wd,
                                                     args.timeout)
        ours_pres, ours_info = run_ours(Y, n_b, K, seed, ref_info["p0"], args.iters, args.burnin, args.unchanged,
                                        None if args.own_init else init)
    sa = cc.summarise(ref_pres, B, K, G)
    sb = cc.summarise(ours_pres, B, K, G)
    rec = cc.compare(sa, sb, B, K, G, W_true)
    rec.update({
        "what": "whole-chain comparison: the reference's kernels (a) against this sampler (b), same data, run "
                "lengths, seed and initial p; z = (mean_a - mean_b) / sqrt(se_a^2 + se_b^2) per scalar",
        "start": (("both chains from one state in the posterior's bulk: this sampler ran %d sweeps from the "
                   "reference's initial state, and both samplers continue from the state it reached (X, Z, W, L and "
                   "every parameter; the priors of the reference's initialisation); p and tau0 updated throughout"
                   % args.start_sweeps) if args.start_sweeps > 0 else
                  "both chains from their own initialisation" if args.own_init else
                  "this sampler started from the reference chain's initial state (W, L, every parameter, X = Y, "
                  "Z = 0), so both chains have the same distribution at every sweep"),
        "data": "BUSseq generative model, batches %s, G = %d, K = %d, seed %d (%s)" % (n_b, G, K, seed, args.data),
        "n_iter": args.iters, "n_burnin": args.burnin,
        "n_unchanged": 0 if args.start_sweeps > 0 else args.unchanged,
        "reference": ref_info, "ours": ours_info,
        "pi_in_reference_chain": "host Dirichlet(count + 2) draws; update_pi (BUSseq_gpu.cu:866-890) not launched",
    })
    npz = {"W_true": W_true.astype(np.int32)}
    npz.update(cc.to_npz_dict("a/", sa))
    npz.update(cc.to_npz_dict("b/", sb))
    np.savez_compressed(os.path.join(args.out, "ref_chain_%s.npz" % args.name),
                        **{k: (v.astype(np.float32) if v.dtype == np.float64 else v) for k, v in npz.items()})
    with open(os.path.join(args.out, "ref_chain_%s.json" % args.name), "w") as f:
        json.dump(rec, f, indent=1)
    print(json.dumps({k: rec[k] for k in ("ari_a", "ari_b", "ari_diff", "ari_a_vs_b", "baseline_type_matched")}))
    for name, st in rec["blocks"].items():
        e30 = st["ess_ge_30"]
        print("%-9s coords %6d  |z|>3 (batch means) %.4f  (ESS) %.4f  ESS>=30: %d coords %s  median ESS %.0f/%.0f"
              % (name, st["coords"], st["se_bm"]["frac_abs_z_gt_3"], st["se_ess"]["frac_abs_z_gt_3"], e30["coords"],
                 "%.4f" % e30["frac_abs_z_gt_3"] if e30["frac_abs_z_gt_3"] is not None else "-", *st["median_ess"]))
    print("reference %.3f s/sweep (%s), ours %.1f sweeps/s" % (ref_info["seconds_per_sweep"],
                                                              "graphs" if ref_info["graphs"] else "launches",
                                                              ours_info["sweeps_per_s"]))
    return 0


if __name__ == "__main__":
    sys.exit(main())
