"""Batches of chains (one CUDA graph per sweep holding every chain) and the
launch-shape autotuners.

A chain run inside a batch must make exactly the draws it makes alone: the
batch only changes how its kernels are launched (graph branches that run
concurrently with the other chains'), not what they compute.  So every state
array and estimate is compared bit for bit with a solo run of the same chain.
"""
import numpy as np
import pytest

import busseq_gpu_gb300 as bq

pytestmark = pytest.mark.gpu

N_B, G = [60, 45, 70], 300
KS = [2, 3, 4, 5]
N_ITER, N_BURN, N_UNCH = 24, 12, 6


@pytest.fixture(scope="module")
def data():
    Y, _, _ = bq.simulate(N_B, G, 4, 17)
    return Y


def _solo(Y, K, seed, **kw):
    s = bq.Sampler(Y, N_B, K, seed=seed, **kw)
    s.run(N_ITER, N_BURN, N_UNCH)
    out = (s.get_state(), s.estimates(with_XZ=False), s.bic())
    s.close()
    return out


def test_batch_matches_solo_runs(data):
    Y = data
    chains = [bq.Sampler(Y, N_B, K, seed=100 + K, keep_draws=True) for K in KS]
    for c in chains:
        c.begin(N_ITER, N_BURN, N_UNCH)
    with bq.Batch(chains) as b:
        b.sweeps(5)            # inside burn-in
        b.sweeps(N_ITER - 5)   # across the burn-in boundary to the end
        b.synchronize()
    for K, c in zip(KS, chains):
        c.finish()
        st, est, bic = c.get_state(), c.estimates(with_XZ=False), c.bic()
        c.close()
        st0, est0, bic0 = _solo(Y, K, 100 + K, keep_draws=True)
        for k in st0:
            assert np.array_equal(st0[k], st[k]), (K, k)
        for k in est0:
            assert np.array_equal(est0[k], est[k]), (K, k)
        assert bic == bic0


def test_batch_with_hmc_chain_matches_solo(data):
    Y = data
    a = bq.Sampler(Y, N_B, 3, seed=7)
    h = bq.Sampler(Y, N_B, 4, seed=8, hmc_leapfrog=4)
    for c in (a, h):
        c.begin(N_ITER, N_BURN, N_UNCH)
    with bq.Batch([a, h]) as b:
        b.sweeps(N_ITER)
        b.synchronize()
    for c, K, seed, kw in ((a, 3, 7, {}), (h, 4, 8, {"hmc_leapfrog": 4})):
        c.finish()
        st = c.get_state()
        c.close()
        st0, _, _ = _solo(Y, K, seed, **kw)
        for k in st0:
            assert np.array_equal(st0[k], st[k]), (K, k)


def test_batch_refuses_mismatched_chains(data):
    Y = data
    a = bq.Sampler(Y, N_B, 3, seed=1)
    c = bq.Sampler(Y, N_B, 3, seed=2)
    a.begin(20, 10, 5)
    c.begin(30, 10, 5)
    with pytest.raises(bq.BusseqError):
        bq.Batch([a, c])
    c.begin(20, 10, 5)
    a.sweeps(2)
    with pytest.raises(bq.BusseqError):
        bq.Batch([a, c])  # not at the same sweep
    with pytest.raises(bq.BusseqError):
        bq.Batch([a, a])
    c.sweeps(2)
    with bq.Batch([a, c]) as b:
        b.sweeps(18)
        with pytest.raises(bq.BusseqError):
            b.sweeps(1)  # past the run length
        b.synchronize()
    a.finish()
    c.finish()
    a.close()
    c.close()


def test_autotune_picks_a_candidate_and_the_choice_is_a_valid_chain(data):
    Y = data
    best, ms = bq.autotune_chunk(Y, N_B, 4, seed=3, candidates=(32, 64, 128, 256), sweeps=4)
    assert best in (32, 64, 128, 256)
    assert set(ms) == {32, 64, 128, 256} and all(v > 0 for v in ms.values())
    assert ms[best] == min(ms.values())
    # a chain with another chunk length makes the same draws up to float
    # reassociation of the per-chunk partial sums; its run completes and its
    # estimates are finite
    s = bq.Sampler(Y, N_B, 4, seed=3, chunk_cells=best)
    s.run(20, 10, 5)
    est = s.estimates(with_XZ=False)
    s.close()
    assert np.all(np.isfinite(est["alpha"])) and np.all(np.isfinite(est["phi"]))


def test_launch_shape_autotune_and_shapes_keep_the_draws(data):
    """busseq_autotune returns shapes from its candidate sets; a chain with other
    Z/X unit lengths and CTA counts imputes exactly the same X and Z in its
    first sweep (the draws come from each entry's own stream; only the order
    of the gamma statistics' partial sums moves, which the first sweep's Z/X
    update does not read)."""
    Y = data
    t = bq.autotune(Y, N_B, 4, seed=3, sweeps=3)
    assert t["chunk_cells"] in (64, 128, 192, 256) and t["zx_unit"] in (128, 256, 384, 512)
    assert t["zx_ctas_per_sm"] in (2, 3, 4) and t["ms_per_sweep"] > 0
    states = []
    for kw in ({}, {"zx_unit": 48, "zx_ctas_per_sm": 1}, {"zx_unit": t["zx_unit"], "zx_ctas_per_sm": t["zx_ctas_per_sm"]}):
        s = bq.Sampler(Y, N_B, 4, seed=3, **kw)
        s.begin(4, 4, 0)
        s.sweeps(1)
        s.synchronize()
        states.append(s.get_state())
        s.close()
    for st in states[1:]:
        np.testing.assert_array_equal(st["X"], states[0]["X"])
        np.testing.assert_array_equal(st["Z"], states[0]["Z"])
