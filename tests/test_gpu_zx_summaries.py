"""Posterior summaries of the imputation (E[X] and P(Z = 1) over the kept
sweeps), accumulated on the device by the Z/X kernel.

The reference: the same chain advanced one sweep at a time, its Z and X read
after every kept sweep and averaged on the host.  Sums of integers, so the
comparison is exact (up to the final float conversion of the means).
"""
import os
import subprocess

import numpy as np
import pytest

import busseq_gpu_gb300 as bq

pytestmark = pytest.mark.gpu

N_B, G, K, SEED = [40, 35, 30], 150, 3, 77
N_ITER, N_BURN = 16, 8


@pytest.fixture(scope="module")
def data():
    Y, _, _ = bq.simulate(N_B, G, K, SEED)
    return Y


def test_summaries_match_host_averages(data):
    Y = data
    s = bq.Sampler(Y, N_B, K, seed=SEED, zx_summaries=True)
    s.begin(N_ITER, N_BURN, 4)
    xs = np.zeros(Y.shape, np.int64)
    zn = np.zeros(Y.shape, np.int64)
    for it in range(N_ITER):
        s.sweeps(1)
        if it >= N_BURN:
            st = s.get_state()
            xs += st["X"]
            zn += st["Z"]
    s.finish()
    got = s.zx_summaries()
    s.close()
    n = N_ITER - N_BURN
    np.testing.assert_array_equal(got["x_mean"], (xs / n).astype(np.float32))
    np.testing.assert_array_equal(got["z_prob"], (zn / n).astype(np.float32))
    assert np.all(got["z_prob"][Y > 0] == 0) and np.all(got["x_mean"][Y > 0] == Y[Y > 0])
    assert got["z_prob"][Y == 0].max() > 0  # some dropouts were imputed


def test_summaries_off_by_default_and_refused(data):
    s = bq.Sampler(data, N_B, K, seed=SEED)
    s.run(10, 5, 2)
    with pytest.raises(bq.BusseqError):
        s.zx_summaries()
    s.close()


def test_summaries_survive_checkpoint_resume(data, tmp_path):
    Y = data
    ref = bq.Sampler(Y, N_B, K, seed=SEED, zx_summaries=True)
    ref.run(N_ITER, N_BURN, 4)
    want = ref.zx_summaries()
    ref.close()
    a = bq.Sampler(Y, N_B, K, seed=SEED, zx_summaries=True)
    a.begin(N_ITER, N_BURN, 4)
    a.sweeps(12)
    path = str(tmp_path / "zx.ck")
    a.checkpoint_save(path)
    a.close()
    # a chain without the summaries cannot take this checkpoint
    c = bq.Sampler(Y, N_B, K, seed=SEED)
    with pytest.raises(bq.BusseqError):
        c.checkpoint_load(path)
    c.close()
    b = bq.Sampler(Y, N_B, K, seed=SEED, zx_summaries=True)
    b.checkpoint_load(path)
    b.sweeps(N_ITER - 12)
    b.finish()
    got = b.zx_summaries()
    b.close()
    for k in want:
        np.testing.assert_array_equal(want[k], got[k])


def test_cli_writes_summary_tables(data, tmp_path):
    Y = data
    cnt, dim = tmp_path / "counts.txt", tmp_path / "dim.txt"
    np.savetxt(cnt, Y, fmt="%d", delimiter=" ")
    dim.write_text("\n".join(str(x) for x in N_B))
    r = subprocess.run([bq.CLI_PATH, "-B", "3", "-N", str(dim), "-G", str(G), "-K", str(K), "-s", "5", "-c", str(cnt),
                        "-i", "20", "-b", "10", "-u", "5", "-o", str(tmp_path / "out"), "--posterior-zx"],
                       stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    xm = np.loadtxt(str(tmp_path / "out") + "_post_X_mean.txt").reshape(Y.shape)
    zp = np.loadtxt(str(tmp_path / "out") + "_post_Z_prob.txt").reshape(Y.shape)
    # the device formatter prints each value as printf("%f") of the float
    with open(str(tmp_path / "out") + "_post_Z_prob.txt") as f:
        first = f.readline().rstrip("\n").split("\t")
    assert first == ["%f" % float(np.float32(v)) for v in zp[0]]
    assert np.all(xm[Y > 0] == Y[Y > 0]) and np.all(zp[Y > 0] == 0)
    assert np.all((zp >= 0) & (zp <= 1)) and zp.max() > 0
    assert os.path.exists(str(tmp_path / "out") + "_post_X.txt")
