"""The command line with binary count input: a run from the binary file writes
the same output files as the run from the reference's text format."""
import os
import subprocess

import numpy as np
import pytest

import busseq_gpu_gb300 as bq

pytestmark = pytest.mark.gpu


def test_binary_and_text_counts_give_identical_outputs(tmp_path):
    n_b, G, K = [30, 25, 20], 90, 3
    Y, _, _ = bq.simulate(n_b, G, K, 4)
    txt, binf, dim = tmp_path / "c.txt", str(tmp_path / "c.bin"), tmp_path / "dim.txt"
    np.savetxt(txt, Y, fmt="%d", delimiter=" ")
    bq.write_counts_binary(binf, Y)
    dim.write_text("\n".join(str(x) for x in n_b))
    for src, tag in ((str(txt), "t"), (binf, "b")):
        r = subprocess.run([bq.CLI_PATH, "-B", "3", "-N", str(dim), "-G", str(G), "-K", str(K), "-s", "3", "-c", src,
                            "-i", "20", "-b", "10", "-u", "5", "-p", "-o", str(tmp_path / tag)],
                           stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
    names = sorted(f[1:] for f in os.listdir(tmp_path) if f.startswith("t_"))
    assert len(names) == 23
    for suffix in names:
        with open(str(tmp_path / "t") + suffix) as a, open(str(tmp_path / "b") + suffix) as b:
            assert a.read() == b.read(), suffix


def test_post_x_z_text_is_byte_exact(tmp_path):
    """_post_X.txt and _post_Z.txt are formatted on the device; their bytes equal
    the host layout (tab-separated decimal integers, one row per cell)."""
    n_b, G, K = [40, 35, 30], 333, 3
    Y, _, _ = bq.simulate(n_b, G, K, 12)
    s = bq.Sampler(Y, n_b, K, seed=12)
    s.run(12, 6, 3)
    st = s.get_state()
    prefix = str(tmp_path / "o")
    s.write_outputs(prefix)
    s.close()
    for name, M in (("_post_X.txt", st["X"]), ("_post_Z.txt", st["Z"])):
        with open(prefix + name, "rb") as f:
            got = f.read()
        want = "".join("\t".join(str(int(v)) for v in row) + "\n" for row in M).encode()
        assert got == want, name


def test_preserved_files_are_byte_exact(tmp_path):
    """The -p tables are formatted on the device ("%f" of the float draws, ints
    for L and W); their bytes equal printf's layout of the kept draws."""
    n_b, G, K = [30, 25, 20], 90, 3
    Y, _, _ = bq.simulate(n_b, G, K, 5)
    s = bq.Sampler(Y, n_b, K, seed=5, keep_draws=True)
    s.run(16, 8, 4)
    pres = s.preserved()
    prefix = str(tmp_path / "o")
    s.write_outputs(prefix, True)
    s.close()
    files = {"gamma": "_preserved_gamma.txt", "alpha": "_preserved_alpha.txt", "L": "_preserved_L.txt",
             "beta": "_preserved_beta.txt", "p_tau0": "_preserved_p.txt", "nu": "_preserved_nu.txt",
             "delta": "_preserved_delta.txt", "phi": "_preserved_phi.txt", "W": "_preserved_W.txt",
             "pi": "_preserved_pi.txt"}
    for key, name in files.items():
        M = pres[key]
        fmt = (lambda v: "%d" % v) if M.dtype.kind == "i" else (lambda v: "%f" % v)
        want = "".join("\t".join(fmt(v) for v in row) + "\n" for row in M).encode()
        with open(prefix + name, "rb") as f:
            assert f.read() == want, name


@pytest.mark.parametrize("gene", [False, True])
def test_cli_hmc_matches_the_library_chain(tmp_path, gene):
    """--hmc=L (and --hmc-gene) run the gradient-based update: the posterior
    means the command line writes are those of the same chain run through the
    library (same seed and initial p)."""
    import ctypes
    n_b, G, K = [30, 25, 20], 90, 3
    Y, _, _ = bq.simulate(n_b, G, K, 5)
    txt, dim = tmp_path / "c.txt", tmp_path / "dim.txt"
    np.savetxt(txt, Y, fmt="%d", delimiter=" ")
    dim.write_text("\n".join(str(x) for x in n_b))
    args = [bq.CLI_PATH, "-B", "3", "-N", str(dim), "-G", str(G), "-K", str(K), "-s", "5", "-c", str(txt),
            "-i", "20", "-b", "10", "-u", "5", "-o", str(tmp_path / "h"), "--hmc=4"] + (["--hmc-gene"] if gene else [])
    r = subprocess.run(args, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    alpha = np.loadtxt(str(tmp_path / "h") + "_post_alpha.txt")
    phi = np.loadtxt(str(tmp_path / "h") + "_post_phi.txt")
    libc = ctypes.CDLL(None)
    libc.srand(5)
    p0 = libc.rand() * 0.5 / 2147483647.0  # the command line's initial p (glibc rand)
    s = bq.Sampler(Y, n_b, K, seed=5, p0=p0, hmc_leapfrog=4, hmc_gene_accept=gene)
    s.run(20, 10, 5)
    est = s.estimates()
    s.close()
    np.testing.assert_allclose(alpha, est["alpha"], rtol=0, atol=1e-6)
    np.testing.assert_allclose(phi, est["phi"], rtol=0, atol=1e-6)
