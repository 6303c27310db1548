"""Time the reference implementation's Gibbs sweep on this GPU (measurement only).

Writes the counts of a synthetic data set from the BUSseq generative model
(the package's simulator) to a temporary file and runs oracle/lib/ref_sweep_timer,
which replays the reference's launch sequence of one sweep with the reference's
own kernels (oracle/_ref/busseq_ref.cubin).  Prints the timer's JSON line.

    python oracle/time_reference.py --cells 2500 --genes 10000 --types 8 --batches 4 --sweeps 3
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--cells", type=int, default=2500, help="cells per batch")
    ap.add_argument("--batches", type=int, default=4)
    ap.add_argument("--genes", type=int, default=10000)
    ap.add_argument("--types", type=int, default=8)
    ap.add_argument("--seed", type=int, default=13580)
    ap.add_argument("--sweeps", type=int, default=3)
    a = ap.parse_args()

    from oracle import build as obuild
    import busseq_gpu_gb300 as bq

    cubin = obuild.build_ref_cubin()
    timer = obuild.build_ref_timer()
    if not cubin or not os.path.exists(cubin) or not timer:
        print('{"unavailable": "reference cubin or timer not built"}')
        return 0
    n_b = [a.cells] * a.batches
    Y, _, _ = bq.simulate(n_b, a.genes, a.types, a.seed)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "Y.i32")
        Y.astype("int32").tofile(path)
        cmd = [timer, cubin, path, str(a.genes), str(a.types), str(a.seed), str(a.sweeps)] + [str(n) for n in n_b]
        out = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    sys.stdout.write(out.stdout)
    return out.returncode


if __name__ == "__main__":
    sys.exit(main())
