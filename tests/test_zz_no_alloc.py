"""The allocation-free BIC entry point (busseq_bic_noalloc) against busseq_bic.

busseq_bic_noalloc is for callers that cannot call cudaMalloc (all device
memory owned by a pool or arena they do not control, or a footprint fixed
after start-up): it takes device pointers from the caller and keeps its
per-(cell, type) scratch in a fixed static device array.  This file is named
so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

import busseq_gpu_gb300 as bq

pytestmark = pytest.mark.gpu

BIC_RTOL = 1e-10  # the tolerance of the other BIC tests (double precision on both sides)


def _noalloc_fn():
    f = bq.lib().busseq_bic_noalloc
    f.argtypes = [C.POINTER(bq.Dims)] + [C.c_void_p] * 10
    f.restype = C.c_int
    return f


def _case(n_b, G, K, seed):
    Y, _, _ = bq.simulate(n_b, G, K, seed)
    s = bq.Sampler(Y, n_b, K, seed=seed)
    s.run(24, 12, 6)
    est = s.estimates(with_XZ=False)
    want = s.bic()
    s.close()
    return Y, est, want


def test_bic_noalloc_matches_busseq_bic_twice():
    torch = pytest.importorskip("torch")
    fn = _noalloc_fn()
    # two calls in a row share the static scratch; the second one runs on a
    # stream of the caller's (not the default stream)
    cases = [([40, 30, 30], 150, 3, 5, False), ([25, 35], 90, 2, 6, True)]
    for n_b, G, K, seed, own_stream in cases:
        Y, est, want = _case(n_b, G, K, seed)
        dev = torch.device("cuda", 0)
        t = {k: torch.from_numpy(np.ascontiguousarray(est[k], dtype=np.float64)).to(dev)
             for k in ("alpha", "beta", "nu", "delta", "phi", "gamma", "pi")}
        Yd = torch.from_numpy(Y).to(dev)
        out = torch.full((2,), float("nan"), dtype=torch.float64, device=dev)
        nb = np.array(n_b, np.int32)
        dims = bq.Dims(len(n_b), K, G, nb.ctypes.data_as(C.POINTER(C.c_int32)))
        torch.cuda.synchronize()
        stream = torch.cuda.Stream(device=dev) if own_stream else None
        rc = fn(C.byref(dims), Yd.data_ptr(), t["alpha"].data_ptr(), t["beta"].data_ptr(), t["nu"].data_ptr(),
                t["delta"].data_ptr(), t["phi"].data_ptr(), t["gamma"].data_ptr(), t["pi"].data_ptr(),
                out.data_ptr(), stream.cuda_stream if stream is not None else None)
        assert rc == 0, bq.lib().busseq_last_error().decode()
        if stream is not None:
            stream.synchronize()
        torch.cuda.synchronize()
        got, ll = (float(v) for v in out.cpu())
        assert abs(got - want) <= BIC_RTOL * abs(want), (got, want)
        # out[1] is the log-likelihood of the BIC: BIC = -2 LL + log(G N) * nparam
        B, N = len(n_b), sum(n_b)
        nparam = (B + G) * K + 2 * B + G * (2 * B - 1) + N - B
        ll_want = -(want - np.log(G * N) * nparam) / 2.0
        assert abs(ll - ll_want) <= BIC_RTOL * abs(want), (ll, ll_want)


def test_bic_noalloc_in_a_captured_graph():
    """A call made during stream capture, after one outside capture on the
    device, records its launches into the graph; a replay computes the BIC.
    The call outside capture has a smaller K (less shared memory per CTA) than
    the captured one."""
    torch = pytest.importorskip("torch")
    fn = _noalloc_fn()
    dev = torch.device("cuda", 0)

    def prepared(n_b, G, K, seed):
        Y, est, want = _case(n_b, G, K, seed)
        t = {k: torch.from_numpy(np.ascontiguousarray(est[k], dtype=np.float64)).to(dev)
             for k in ("alpha", "beta", "nu", "delta", "phi", "gamma", "pi")}
        Yd = torch.from_numpy(Y).to(dev)
        out = torch.full((2,), float("nan"), dtype=torch.float64, device=dev)
        nb = np.array(n_b, np.int32)
        dims = bq.Dims(len(n_b), K, G, nb.ctypes.data_as(C.POINTER(C.c_int32)))
        args = [Yd.data_ptr()] + [t[k].data_ptr() for k in ("alpha", "beta", "nu", "delta", "phi", "gamma", "pi")]
        keep = (Y, t, Yd, nb, dims)
        return dims, args + [out.data_ptr()], out, want, keep

    d1, a1, o1, w1, k1 = prepared([25, 30], 80, 2, 11)
    torch.cuda.synchronize()
    assert fn(C.byref(d1), *a1, None) == 0, bq.lib().busseq_last_error().decode()
    torch.cuda.synchronize()
    assert abs(float(o1[0].cpu()) - w1) <= BIC_RTOL * abs(w1)

    d2, a2, o2, w2, k2 = prepared([30, 40, 35], 120, 8, 9)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        rc = fn(C.byref(d2), *a2, torch.cuda.current_stream().cuda_stream)
    assert rc == 0, bq.lib().busseq_last_error().decode()
    torch.cuda.synchronize()
    assert np.isnan(float(o2[0].cpu()))  # captured, not yet run
    g.replay()
    torch.cuda.synchronize()
    got = float(o2[0].cpu())
    assert abs(got - w2) <= BIC_RTOL * abs(w2), (got, w2)


def test_bic_noalloc_rejects_oversize():
    fn = _noalloc_fn()
    nb = np.array([1 << 17, 1 << 17, 1 << 17], np.int32)  # N above the static limit
    dims = bq.Dims(3, 2, 10, nb.ctypes.data_as(C.POINTER(C.c_int32)))
    rc = fn(C.byref(dims), *([C.c_void_p(16)] * 9), None)
    assert rc == bq.BusseqError(-1, "").code
    assert "exceed the fixed scratch" in bq.lib().busseq_last_error().decode()
