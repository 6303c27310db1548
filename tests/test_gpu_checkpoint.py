"""Checkpoint / resume on the GPU: a run stopped mid-way, saved, and resumed in
a new handle reproduces the uninterrupted run bit for bit (the draws are keyed
by the sweep index, so nothing else needs to be carried)."""
import numpy as np
import pytest

import busseq_gpu_gb300 as bq

pytestmark = pytest.mark.gpu

N_B, G, K, SEED = [60, 45, 70], 300, 4, 2718


@pytest.fixture(scope="module")
def data():
    Y, _, _ = bq.simulate(N_B, G, K, SEED)
    return Y


def _state_equal(a, b):
    for k in a:
        assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), k


@pytest.mark.parametrize("stop", [7, 27])  # inside burn-in, inside the kept sweeps
def test_resume_reproduces_uninterrupted_run(data, tmp_path, stop):
    Y = data
    ref = bq.Sampler(Y, N_B, K, seed=SEED, keep_draws=True)
    ref.run(40, 20, 10)
    est_ref, pres_ref, st_ref = ref.estimates(), ref.preserved(), ref.get_state()
    ref.close()

    path = str(tmp_path / "chain.ck")
    a = bq.Sampler(Y, N_B, K, seed=SEED, keep_draws=True)
    a.begin(40, 20, 10)
    a.sweeps(stop)
    a.checkpoint_save(path)
    a.close()

    b = bq.Sampler(Y, N_B, K, seed=SEED, keep_draws=True)
    b.checkpoint_load(path)
    b.sweeps(40 - stop)
    b.finish()
    _state_equal(st_ref, b.get_state())
    est = b.estimates()
    for k in est_ref:
        assert np.array_equal(est_ref[k], est[k]), k
    pres = b.preserved()
    for k in pres_ref:
        assert np.array_equal(pres_ref[k], pres[k]), k
    b.close()


def test_state_only_checkpoint_and_mismatches(data, tmp_path):
    Y = data
    a = bq.Sampler(Y, N_B, K, seed=SEED)
    a.begin(12, 6, 3)
    a.sweeps(12)
    a.finish()
    st = a.get_state()
    path = str(tmp_path / "done.ck")
    a.checkpoint_save(path)
    a.close()
    # a finished run restores its estimates too
    b = bq.Sampler(Y, N_B, K, seed=SEED)
    b.checkpoint_load(path)
    _state_equal(st, b.get_state())
    b.close()
    # another seed, other counts or other dimensions are refused
    c = bq.Sampler(Y, N_B, K, seed=SEED + 1)
    with pytest.raises(bq.BusseqError):
        c.checkpoint_load(path)
    c.close()
    Y2 = Y.copy()
    Y2[0, 0] += 1
    d = bq.Sampler(Y2, N_B, K, seed=SEED)
    with pytest.raises(bq.BusseqError):
        d.checkpoint_load(path)
    d.close()
    e = bq.Sampler(Y[:, :G - 1].copy(), N_B, K, seed=SEED)
    with pytest.raises(bq.BusseqError):
        e.checkpoint_load(path)
    e.close()
    with pytest.raises(bq.BusseqError):
        f = bq.Sampler(Y, N_B, K, seed=SEED)
        try:
            f.checkpoint_load(str(tmp_path / "missing.ck"))
        finally:
            f.close()


def test_cli_stop_and_resume_matches_uninterrupted(tmp_path):
    import os
    import subprocess
    n_b, G, K = [30, 25, 20], 120, 3
    Y, _, _ = bq.simulate(n_b, G, K, 99)
    cnt, dim = tmp_path / "counts.txt", tmp_path / "dim.txt"
    np.savetxt(cnt, Y, fmt="%d", delimiter=" ")
    dim.write_text("\n".join(str(x) for x in n_b))
    base = [bq.CLI_PATH, "-B", "3", "-N", str(dim), "-G", str(G), "-K", str(K), "-s", "99", "-c", str(cnt),
            "-i", "40", "-b", "20", "-u", "10", "-p"]

    def run(*extra):
        r = subprocess.run(base + list(extra), stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        return r

    run("-o", str(tmp_path / "full"))
    ck = str(tmp_path / "run.ck")
    r = run("-o", str(tmp_path / "part"), "--checkpoint=" + ck, "--checkpoint-every=5", "--stop-after=27")
    assert "stopped after sweep 27 of 40" in r.stderr
    assert not os.path.exists(str(tmp_path / "part") + "_post_W.txt")
    r = run("-o", str(tmp_path / "part"), "--resume=" + ck)
    assert "resumed from" in r.stderr and "at sweep 27 of 40" in r.stderr
    names = sorted(f[len("full"):] for f in os.listdir(tmp_path) if f.startswith("full"))
    assert len(names) == 23
    for suffix in names:
        with open(str(tmp_path / "full") + suffix) as a, open(str(tmp_path / "part") + suffix) as b:
            assert a.read() == b.read(), suffix
