"""Generate tests/golden/ref_kernels.npz from the REFERENCE's own kernels.

Run on a machine with a GPU, after ``oracle/build.py`` has produced
``oracle/_ref/busseq_ref.cubin`` (compiled from the reference's BUSseq_gpu.cu
where it lies) and ``oracle/lib/ref_harness`` (the driver-API loader):

    python tests/golden/make_ref_golden.py --out tests/golden/ref_kernels.npz

Inputs are seeded and small; they are stored in the fixture next to the
reference's outputs so the CPU tests can replay them through the FP64 oracle.
"""
from __future__ import annotations

import argparse
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)


def make_inputs(seed: int = 20241203):
    rng = np.random.default_rng(seed)
    B, K, G = 3, 4, 32
    n_b = np.array([20, 16, 12], np.int32)
    N = int(n_b.sum())
    off = np.concatenate([[0], np.cumsum(n_b)])
    alpha = rng.uniform(0.5, 2.5, G)
    beta = np.zeros((K, G))
    beta[1:] = rng.normal(0.0, 1.0, (K - 1, G)) * (rng.random((K - 1, G)) < 0.5)
    nu = np.zeros((B, G))
    nu[1:] = rng.normal(0.5, 0.3, (B - 1, G))
    delta = rng.normal(0.0, 0.2, N)
    delta[off[:-1]] = 0.0
    phi = rng.uniform(2.0, 20.0, (B, G))
    W = rng.integers(0, K, N).astype(np.int32)
    bat = np.repeat(np.arange(B), n_b)
    mu = np.exp(alpha[None, :] + beta[W] + nu[bat] + delta[:, None])
    Xtrue = rng.negative_binomial(phi[bat], phi[bat] / (phi[bat] + mu)).astype(np.int32)
    drop = rng.random((N, G)) < 1.0 / (1.0 + np.exp(0.5 + 0.2 * Xtrue))
    Y = np.where(drop, 0, Xtrue).astype(np.int32)
    Y[:, 0] = np.maximum(Y[:, 0], 1)  # every cell has a positive library size
    X = Y.copy()
    imp = (Y == 0) & (rng.random((N, G)) < 0.5)
    X[imp] = rng.integers(1, 12, int(imp.sum()))
    Z = np.where(Y == 0, np.where(X > 0, 1, rng.integers(0, 2, (N, G))), 0).astype(np.int32)
    gamma = np.stack([rng.normal(0.0, 0.5, B), -rng.uniform(0.05, 0.5, B)])
    gamma_prop = np.stack([gamma[0] + 0.1 * rng.normal(size=B), -rng.gamma(2.0, 0.1, B)])
    inputs = {
        "dims": np.array([B, K, G, N], np.int32),
        "n_b": n_b,
        "Y": Y.ravel(), "X": X.ravel(), "Z": Z.ravel(), "W": W,
        "W_prop": rng.integers(0, K, N).astype(np.int32),
        "alpha": alpha, "alpha_prop": alpha + 0.1 * rng.normal(size=G),
        "beta": beta.ravel(), "beta_prop": (beta[1:] + 0.1 * rng.normal(size=(K - 1, G))).ravel(),
        "nu": nu.ravel(), "nu_prop": (nu[1:] + 0.1 * rng.normal(size=(B - 1, G))).ravel(),
        "delta": delta, "delta_prop": delta + 0.1 * rng.normal(size=N),
        "phi": phi.ravel(), "phi_prop": rng.gamma(phi, 1.0).ravel(),
        "gamma": gamma.ravel(), "gamma_prop": gamma_prop.ravel(),
        "pi": rng.dirichlet(np.full(K, 2.0), B).ravel(),
        "mode_counts": rng.integers(0, 50, (K, N)).astype(np.int32).ravel(),
    }
    return inputs


def write_records(path, arrays):
    with open(path, "wb") as f:
        for name, a in arrays.items():
            nb = name.encode()
            if a.dtype == np.float64:
                dt, data = 0, np.ascontiguousarray(a, np.float64)
            else:
                dt, data = 1, np.ascontiguousarray(a, np.int32)
            f.write(struct.pack("<I", len(nb)))
            f.write(nb)
            f.write(struct.pack("<BQ", dt, data.size))
            f.write(data.tobytes())


def read_records(path):
    out = {}
    with open(path, "rb") as f:
        while True:
            h = f.read(4)
            if len(h) < 4:
                break
            (nl,) = struct.unpack("<I", h)
            name = f.read(nl).decode()
            dt, cnt = struct.unpack("<BQ", f.read(9))
            dtype = np.float64 if dt == 0 else np.int32
            out[name] = np.frombuffer(f.read(cnt * np.dtype(dtype).itemsize), dtype=dtype).copy()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(ROOT, "tests", "golden", "ref_kernels.npz"))
    args = ap.parse_args()
    from oracle import build
    cubin = build.REF_CUBIN
    harness = build.build_harness()
    if not (cubin and os.path.exists(cubin)):
        sys.exit("reference cubin missing: run oracle/build.py where the reference source exists")
    if not harness:
        sys.exit("could not build the harness (needs libcuda)")
    inputs = make_inputs()
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        write_records(fin, inputs)
        subprocess.run([harness, cubin, fin, fout], check=True)
        outputs = read_records(fout)
    pack = {"in_" + k: v for k, v in inputs.items()}
    pack.update({"out_" + k: v for k, v in outputs.items()})
    os.makedirs(os.path.dirname(args.out), exist_ok=True)
    np.savez_compressed(args.out, **pack)
    print("wrote", args.out, "with", len(outputs), "reference outputs")


if __name__ == "__main__":
    main()
