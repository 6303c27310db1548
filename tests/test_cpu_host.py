"""CPU-only checks: the C ABI library loads and exports every declared symbol,
the count parser, the generator, the command line's argument checks (which
run before any GPU call), and the oracle's own samplers."""
import os
import re
import subprocess

import numpy as np
import pytest

import busseq_gpu_gb300 as bq
from oracle import pyoracle as po

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    text = open(os.path.join(ROOT, "include", "busseq_gb300.h")).read()
    return sorted(set(re.findall(r"\b(busseq_[a-z_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    path = bq.library_path()
    assert os.path.exists(path)
    out = subprocess.run(["nm", "-D", "--defined-only", path], stdout=subprocess.PIPE, text=True).stdout
    exported = set(l.split()[-1] for l in out.splitlines() if l.strip())
    missing = [s for s in _declared_symbols() if s not in exported]
    assert not missing, missing
    lib = bq.lib()
    for s in _declared_symbols():
        assert hasattr(lib, s)


def test_read_counts_roundtrip_and_errors(tmp_path):
    rng = np.random.default_rng(0)
    Y = rng.integers(0, 5000, (37, 23)).astype(np.int32)
    p = tmp_path / "c.txt"
    with open(p, "w") as f:
        for row in Y:
            f.write(" ".join(str(x) for x in row) + "\n")
    np.testing.assert_array_equal(bq.read_counts(str(p), 37, 23), Y)
    # tabs, CRLF and a missing trailing newline are fine
    p2 = tmp_path / "c2.txt"
    p2.write_text("\r\n".join("\t".join(str(x) for x in row) for row in Y))
    np.testing.assert_array_equal(bq.read_counts(str(p2), 37, 23), Y)
    with pytest.raises(bq.BusseqError):
        bq.read_counts(str(p), 37, 24)            # too few numbers
    bad = tmp_path / "bad.txt"
    bad.write_text("1 2 x 4\n")
    with pytest.raises(bq.BusseqError):
        bq.read_counts(str(bad), 1, 4)
    neg = tmp_path / "neg.txt"
    neg.write_text("1 -2 3 4\n")
    with pytest.raises(bq.BusseqError):
        bq.read_counts(str(neg), 1, 4)
    with pytest.raises(bq.BusseqError):
        bq.read_counts(str(tmp_path / "absent.txt"), 1, 1)


def test_read_counts_large_parallel(tmp_path):
    Y, _, _ = bq.simulate([700, 500], 900, 3, 5)
    p = tmp_path / "big.txt"
    np.savetxt(p, Y, fmt="%d", delimiter=" ")
    np.testing.assert_array_equal(bq.read_counts(str(p), 1200, 900), Y)


def test_binary_counts_roundtrip_and_errors(tmp_path):
    Y, _, _ = bq.simulate([400, 300], 700, 3, 9)
    p = str(tmp_path / "y.bin")
    bq.write_counts_binary(p, Y)
    np.testing.assert_array_equal(bq.read_counts(p, 700, 700), Y)
    with open(p, "rb") as f:
        head = f.read(24)
    assert head[:8] == b"BUSSEQY1"
    assert np.frombuffer(head[8:], "<i8").tolist() == [700, 700]
    with pytest.raises(bq.BusseqError):
        bq.read_counts(p, 700, 699)              # other dimensions
    trunc = str(tmp_path / "t.bin")
    with open(p, "rb") as f, open(trunc, "wb") as g:
        g.write(f.read(24 + 4 * 1000))
    with pytest.raises(bq.BusseqError):
        bq.read_counts(trunc, 700, 700)          # truncated payload
    neg = np.array(Y)
    neg[3, 5] = -1
    pn = str(tmp_path / "n.bin")
    bq.write_counts_binary(pn, neg)
    with pytest.raises(bq.BusseqError):
        bq.read_counts(pn, 700, 700)             # negative count


def test_gzip_counts_text_and_binary(tmp_path):
    import gzip
    Y, _, _ = bq.simulate([60, 50], 90, 3, 21)
    txt, binf = str(tmp_path / "y.txt"), str(tmp_path / "y.bin")
    np.savetxt(txt, Y, fmt="%d", delimiter=" ")
    bq.write_counts_binary(binf, Y)
    for src in (txt, binf):
        with open(src, "rb") as f, gzip.open(src + ".gz", "wb") as g:
            g.write(f.read())
        np.testing.assert_array_equal(bq.read_counts(src + ".gz", 110, 90), Y)
        with pytest.raises(bq.BusseqError):
            bq.read_counts(src + ".gz", 110, 91)     # other dimensions
    with open(txt + ".gz", "rb") as f:
        data = f.read()
    bad = str(tmp_path / "bad.gz")
    with open(bad, "wb") as f:
        f.write(data[: len(data) // 2])              # a truncated stream
    with pytest.raises(bq.BusseqError):
        bq.read_counts(bad, 110, 90)


def test_documented_python_api_exists():
    """The names the integration notes and the README call exist on the package."""
    for name in ("run", "begin", "sweeps", "finish", "estimates", "bic", "write_outputs", "corrected_counts",
                 "checkpoint_save", "checkpoint_load", "zx_summaries", "hmc_stats", "hmc_gradient",
                 "hmc_logpost_diff", "hmc_gene_logpost_diff", "get_state", "set_state", "preserved", "profile",
                 "set_stream", "synchronize", "close"):
        assert callable(getattr(bq.Sampler, name, None)), name
    for name in ("simulate", "read_counts", "write_counts_binary", "autotune_chunk", "autotune", "Batch",
                 "estimate_buffers"):
        assert callable(getattr(bq, name, None)), name


def test_simulate_deterministic_and_model_shaped():
    a = bq.simulate([50, 40, 30], 400, 4, 123)
    b = bq.simulate([50, 40, 30], 400, 4, 123)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    Y, W, X = a
    assert Y.shape == (120, 400) and W.shape == (120,)
    assert np.all((Y == 0) | (Y == X))
    assert np.all(Y.sum(1) > 0)
    assert set(np.unique(W)) <= set(range(4))
    # dropout is more frequent for small counts
    small, large = (X > 0) & (X <= 2), X >= 20
    assert (Y[small] == 0).mean() > (Y[large] == 0).mean()


def _cli(*args):
    return subprocess.run([bq.CLI_PATH, *args], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                          timeout=60)


def test_cli_argument_checks_match_reference(tmp_path):
    # BUSseq_gpu.cu:1120-1134: messages and exit status -1
    r = _cli("-s", "1", "-i", "10", "-b", "20")
    assert r.returncode == 255 and r.stdout.splitlines() == [
        "Seed is 1", "Burn-in iterations must be less than total number of iterations."]
    r = _cli("-s", "1", "-B", "1")
    assert r.returncode == 255 and r.stdout.splitlines()[-1] == "The batch number must be greater than one."
    dim = tmp_path / "dim.txt"
    dim.write_text("3 10")
    r = _cli("-s", "2", "-B", "2", "-N", str(dim), "-K", "5")
    assert r.returncode == 255
    assert r.stdout.splitlines()[-1] == "The sample size in any batch must be greater than the assumed cell type number."
    r = _cli("-z")
    # BUSseq_gpu.cu:1088, byte for byte (the reference's own flag names included)
    assert r.returncode == 1 and r.stdout == (
        "Error Usage: %s [-b batch] [-n sample_size_file] [-g gene] [-k celltype] [-c count_data_file)] "
        "[-i iterations] [-b burnin] [-u unchanged_iterations] [-p print_preserved] [-o output_prefix] \n"
        % bq.CLI_PATH)


def test_cli_hmc_flags_are_checked():
    for bad in ("--hmc=0", "--hmc=abc", "--hmc=2000"):
        r = _cli(bad, "-s", "1")
        assert r.returncode == 1 and "--hmc takes a number of leapfrog steps" in r.stderr, bad
    r = _cli("--hmc-gene", "-s", "1")
    assert r.returncode == 1 and "--hmc-gene needs --hmc=L" in r.stderr


def test_cli_missing_count_file_fails_cleanly(tmp_path):
    dim = tmp_path / "dim.txt"
    dim.write_text("10 10")
    r = _cli("-s", "3", "-B", "2", "-N", str(dim), "-G", "5", "-K", "2", "-c", str(tmp_path / "none.txt"))
    assert r.returncode == 1
    assert "Start reading file." in r.stdout and "cannot open count file" in r.stderr


def test_oracle_sampler_moments():
    g = po.sample_gamma(7, 2.5, 100000)
    assert abs(g.mean() - 2.5) < 0.03 and abs(g.var() - 2.5) < 0.08
    g = po.sample_gamma(8, 0.4, 100000)
    assert abs(g.mean() - 0.4) < 0.01
    p = po.sample_poisson(9, 3.3, 100000)
    assert abs(p.mean() - 3.3) < 0.03 and abs(p.var() - 3.3) < 0.08
    p = po.sample_poisson(10, 250.0, 100000)
    assert abs(p.mean() - 250) < 0.3 and abs(p.var() / 250 - 1) < 0.03
    nb = po.sample_negbin(11, 40.0, 4.0, 100000)  # Gamma-Poisson
    assert abs(nb.mean() - 40) < 0.5 and abs(nb.var() / (40 + 1600 / 4) - 1) < 0.05
    nb = po.sample_negbin(12, 24.0, 3.0, 100000)  # distribution-function inversion (mu < 32, phi >= 1)
    assert abs(nb.mean() - 24) < 0.25 and abs(nb.var() / (24 + 576 / 3) - 1) < 0.05
    for seed, mu in ((13, 31.5), (14, 32.5)):  # either side of the switch, phi = 1 (a long tail)
        nb = po.sample_negbin(seed, mu, 1.0, 200000)
        assert abs(nb.mean() - mu) < 0.5 and abs(nb.var() / (mu + mu * mu) - 1) < 0.05, (mu, nb.mean(), nb.var())


def test_philox_known_answers():
    # Random123 known-answer vectors for Philox4x32-10
    assert po.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert po.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert po.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == [
        0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]
    u = po.uniforms(1, 4, 17, 3, 8)
    assert np.all((u > 0) & (u < 1))


def test_oracle_chain_runs_and_recovers_types():
    """A short FP64 oracle chain on a tiny data set: invariants and clustering."""
    n_b, G, K = [60, 50], 200, 3
    Y, W_true, _ = bq.simulate(n_b, G, K, 31)
    st = po.State(Y, n_b, K, seed=31)
    st.init(0.3)
    for it in range(80):
        st.sweep(it, n_unchanged=20)
    assert np.all(st.X[Y > 0] == Y[Y > 0]) and not st.Z[Y > 0].any()
    assert np.all(st.delta[[0, 60]] == 0) and np.all(st.beta[0] == 0)
    assert np.allclose(st.pi.sum(1), 1)
    from collections import Counter
    agree = 0
    for k in range(K):
        c = Counter(W_true[st.W == k])
        agree += c.most_common(1)[0][1] if c else 0
    assert agree / len(W_true) > 0.8
