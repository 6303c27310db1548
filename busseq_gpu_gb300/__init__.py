"""GB300-native BUSseq Gibbs sampler.

Python front-end over the C ABI of ``libbusseq_gb300.so`` (include/busseq_gb300.h).
The compute path is the library's sm_103a CUDA kernels; there is no CPU
fallback: if the library has not been built, or no GPU is present, the calls
fail loudly.

    from busseq_gpu_gb300 import Sampler, simulate
    Y, W_true, _ = simulate([300, 300, 200, 200], G=3000, K=5, seed=13579)
    s = Sampler(Y, [300, 300, 200, 200], K=5, seed=13579)
    s.run(n_iter=4000, n_burnin=2000, n_unchanged=500)
    est = s.estimates()
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

__all__ = [
    "Sampler", "BusseqError", "simulate", "read_counts", "lib", "library_path", "CONFIG_SIM", "STAGES",
    "W_MH", "W_GIBBS",
]

_PKG = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_PKG, "lib", "libbusseq_gb300.so")
CLI_PATH = os.path.join(_PKG, "bin", "busseq")

W_MH = 0
W_GIBBS = 1
STAGES = {"zx_gamma_alpha_L": 0, "beta_nu": 1, "delta": 2, "phi": 3, "W": 4, "pi": 5}

_PI32 = C.POINTER(C.c_int32)
_PU8 = C.POINTER(C.c_uint8)
_PI8 = C.POINTER(C.c_int8)
_PF = C.POINTER(C.c_float)
_PD = C.POINTER(C.c_double)


class Dims(C.Structure):
    _fields_ = [("B", C.c_int32), ("K", C.c_int32), ("G", C.c_int64), ("n_b", _PI32)]


class Options(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("p0", C.c_double), ("w_update", C.c_int32), ("keep_draws", C.c_int32),
                ("device", C.c_int32), ("chunk_cells", C.c_int32), ("hmc_leapfrog", C.c_int32),
                ("zx_summaries", C.c_int32), ("hmc_gene_accept", C.c_int32), ("test_nb_inv_cap", C.c_int32),
                ("zx_unit", C.c_int32), ("zx_ctas_per_sm", C.c_int32), ("reserved", C.c_int32 * 2)]


class Estimates(C.Structure):
    _fields_ = [("Z", _PI32), ("X", _PI32), ("gamma", _PD), ("alpha", _PD), ("L", _PD), ("beta", _PD),
                ("p_tau0", _PD), ("nu", _PD), ("delta", _PD), ("phi", _PD), ("W", _PI32), ("pi", _PD)]


class Preserved(C.Structure):
    _fields_ = [("gamma", _PD), ("alpha", _PD), ("L", _PI32), ("beta", _PD), ("p_tau0", _PD), ("nu", _PD),
                ("delta", _PD), ("phi", _PD), ("W", _PI32), ("pi", _PD)]


class State(C.Structure):
    _fields_ = [("X", _PI32), ("Z", _PU8), ("W", _PI32), ("L", _PI8), ("alpha", _PF), ("mu_alpha", _PF),
                ("beta", _PF), ("nu", _PF), ("mu_nu", _PF), ("delta", _PF), ("mu_delta", _PF), ("phi", _PF),
                ("gamma", _PF), ("pi", _PF), ("p_tau0", _PF)]


class LogRatios(C.Structure):
    _fields_ = [("gamma", _PD), ("alpha", _PD), ("beta", _PD), ("nu", _PD), ("delta", _PD), ("phi", _PD),
                ("W", _PD)]


class SimParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("alpha_lo", "alpha_hi", "de_frac", "beta_lo", "beta_hi", "nu_step",
                                          "nu_sd", "delta_sd", "phi_lo", "phi_hi", "pi_conc", "gamma0", "gamma1")]


class BusseqError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("busseq error %d: %s" % (code, msg))
        self.code = code


_lib = None


def library_path() -> str:
    return _LIB_PATH


def lib():
    """Load libbusseq_gb300.so (built in-tree by __graft_entry__.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        raise BusseqError(-4, "%s is not built; run __graft_entry__.build() first" % _LIB_PATH)
    L = C.CDLL(_LIB_PATH)
    H = C.c_void_p
    sigs = {
        "busseq_create": ([C.POINTER(Dims), C.c_void_p, C.c_int32, C.POINTER(Options), C.POINTER(H)], C.c_int),
        "busseq_destroy": ([H], None),
        "busseq_run": ([H, C.c_int32, C.c_int32, C.c_int32], C.c_int),
        "busseq_begin": ([H, C.c_int32, C.c_int32, C.c_int32], C.c_int),
        "busseq_sweeps": ([H, C.c_int32], C.c_int),
        "busseq_finish": ([H], C.c_int),
        "busseq_synchronize": ([H], C.c_int),
        "busseq_get_estimates": ([H, C.POINTER(Estimates)], C.c_int),
        "busseq_get_preserved": ([H, C.POINTER(Preserved)], C.c_int),
        "busseq_bic": ([H, _PD], C.c_int),
        "busseq_corrected_counts": ([H, C.c_void_p, C.c_int32], C.c_int),
        "busseq_get_zx_summaries": ([H, C.c_void_p, C.c_void_p], C.c_int),
        "busseq_write_zx_summaries": ([H, C.c_char_p], C.c_int),
        "busseq_batch_create": ([C.POINTER(C.c_void_p), C.c_int32, C.POINTER(H)], C.c_int),
        "busseq_batch_sweeps": ([H, C.c_int32], C.c_int),
        "busseq_batch_synchronize": ([H], C.c_int),
        "busseq_batch_stream": ([H], C.c_void_p),
        "busseq_batch_destroy": ([H], None),
        "busseq_autotune_chunk": ([C.POINTER(Dims), C.c_void_p, C.c_int32, C.POINTER(Options), _PI32, C.c_int32,
                                   C.c_int32, _PI32, _PD], C.c_int),
        "busseq_autotune": ([C.POINTER(Dims), C.c_void_p, C.c_int32, C.POINTER(Options), C.c_int32, _PD], C.c_int),
        "busseq_get_state": ([H, C.POINTER(State)], C.c_int),
        "busseq_set_state": ([H, C.POINTER(State)], C.c_int),
        "busseq_run_stage": ([H, C.c_int32, C.c_int32, C.c_int32], C.c_int),
        "busseq_get_log_ratios": ([H, C.POINTER(LogRatios)], C.c_int),
        "busseq_set_stream": ([H, C.c_void_p], C.c_int),
        "busseq_checkpoint_save": ([H, C.c_char_p], C.c_int),
        "busseq_checkpoint_load": ([H, C.c_char_p], C.c_int),
        "busseq_get_progress": ([H, _PI32, _PI32, _PI32], C.c_int),
        "busseq_hmc_stats": ([H, _PD], C.c_int),
        "busseq_hmc_gradient": ([H, _PD, _PD], C.c_int),
        "busseq_hmc_logpost_diff": ([H, C.POINTER(State), _PD], C.c_int),
        "busseq_hmc_gene_logpost_diff": ([H, C.POINTER(State), _PD], C.c_int),
        "busseq_profile": ([H, C.c_int32, _PD, C.c_int32, _PI32], C.c_int),
        "busseq_kernel_name": ([C.c_int32], C.c_char_p),
        "busseq_kernel_bytes": ([H, C.c_int32], C.c_double),
        "busseq_launches_per_sweep": ([H, C.c_int32], C.c_int),
        "busseq_read_counts": ([C.c_char_p, C.c_int64, C.c_int64, _PI32], C.c_int),
        "busseq_write_counts_binary": ([C.c_char_p, C.c_int64, C.c_int64, _PI32], C.c_int),
        "busseq_write_outputs": ([H, C.c_char_p, C.c_int32], C.c_int),
        "busseq_simulate": ([C.POINTER(Dims), C.POINTER(SimParams), C.c_uint64, _PI32, _PI32, _PI32], C.c_int),
        "busseq_last_error": ([], C.c_char_p),
        "busseq_sample_draws": ([C.c_int32, C.c_double, C.c_double, C.c_uint64, C.c_int64, C.c_void_p], C.c_int),
        "busseq_version": ([], C.c_char_p),
    }
    for name, (args, res) in sigs.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def _check(rc: int) -> None:
    if rc != 0:
        raise BusseqError(rc, lib().busseq_last_error().decode())


def _p(a, t):
    return a.ctypes.data_as(t)


# Parameters of the generative model behind each benchmark configuration.
CONFIG_SIM = {
    "default": dict(alpha_lo=0.5, alpha_hi=2.5, de_frac=0.2, beta_lo=1.5, beta_hi=3.0, nu_step=0.5, nu_sd=0.2,
                    delta_sd=0.2, phi_lo=5.0, phi_hi=20.0, pi_conc=2.0, gamma0=-0.5, gamma1=-0.2),
}
CONFIG_SIM["wide"] = dict(CONFIG_SIM["default"], de_frac=0.15, phi_lo=2.0, phi_hi=30.0)


def simulate(n_b, G: int, K: int, seed: int, **params):
    """Draw (Y [N,G] int32, W_true [N], X_true [N,G]) from the BUSseq model on the host."""
    prm = dict(CONFIG_SIM["default"])
    prm.update(params)
    n_b = np.ascontiguousarray(n_b, dtype=np.int32)
    N = int(n_b.sum())
    Y = np.zeros((N, G), np.int32)
    W = np.zeros(N, np.int32)
    X = np.zeros((N, G), np.int32)
    d = Dims(len(n_b), K, G, _p(n_b, _PI32))
    sp = SimParams(**prm)
    _check(lib().busseq_simulate(C.byref(d), C.byref(sp), int(seed), _p(Y, _PI32), _p(W, _PI32), _p(X, _PI32)))
    return Y, W, X


SAMPLE_KINDS = {"gamma": (0, np.float32), "poisson": (1, np.int32), "negbin": (2, np.int32),
                "negbin_gamma_poisson": (3, np.int32), "negbin_inversion": (4, np.int32)}


def sample_draws(kind: str, a: float, b: float = 0.0, seed: int = 0, n: int = 100000) -> np.ndarray:
    """n draws of one device sampler (busseq_sample_draws), for distribution tests."""
    code, dt = SAMPLE_KINDS[kind]
    out = np.zeros(n, dt)
    _check(lib().busseq_sample_draws(code, float(a), float(b), int(seed), int(n), out.ctypes.data_as(C.c_void_p)))
    return out


def read_counts(path: str, N: int, G: int) -> np.ndarray:
    """An N x G count file: the reference's text format, or binary counts
    (recognised by their magic)."""
    out = np.zeros((N, G), np.int32)
    _check(lib().busseq_read_counts(path.encode(), N, G, _p(out, _PI32)))
    return out


def write_counts_binary(path: str, Y) -> None:
    """Y (N x G) as a binary count file that read_counts and the command line load
    without parsing."""
    Yc = np.ascontiguousarray(Y, dtype=np.int32)
    _check(lib().busseq_write_counts_binary(path.encode(), Yc.shape[0], Yc.shape[1], _p(Yc, _PI32)))


def autotune_chunk(Y, n_b, K: int, seed: int = 0, candidates=(64, 128, 192, 256), sweeps: int = 8,
                   hmc_leapfrog: int = 0, device: int = 0):
    """Gene-pass chunk length (cells per CTA of the gene passes) chosen by timing
    ``sweeps`` burn-in sweeps of a scratch chain for every candidate.  Returns
    (best, {candidate: ms per sweep})."""
    n_b = np.ascontiguousarray(n_b, dtype=np.int32)
    on_dev = hasattr(Y, "data_ptr") and getattr(Y, "is_cuda", False)
    if on_dev:
        yptr, G = C.c_void_p(Y.data_ptr()), int(Y.shape[1])
    else:
        Yh = np.ascontiguousarray(Y, dtype=np.int32)
        yptr, G = Yh.ctypes.data_as(C.c_void_p), int(Yh.shape[1])
    dims = Dims(len(n_b), int(K), G, _p(n_b, _PI32))
    opt = Options(seed=int(seed) & 0xFFFFFFFFFFFFFFFF, p0=0.25, w_update=W_MH, keep_draws=0, device=int(device),
                  chunk_cells=0, hmc_leapfrog=int(hmc_leapfrog))
    cand = np.ascontiguousarray(candidates, dtype=np.int32)
    ms = np.zeros(cand.size)
    best = C.c_int32()
    _check(lib().busseq_autotune_chunk(C.byref(dims), yptr, int(on_dev), C.byref(opt), _p(cand, _PI32),
                                       int(cand.size), int(sweeps), C.byref(best), _p(ms, _PD)))
    return int(best.value), {int(c): float(m) for c, m in zip(cand, ms)}


def autotune(Y, n_b, K: int, seed: int = 0, sweeps: int = 8, hmc_leapfrog: int = 0, device: int = 0) -> dict:
    """Launch shapes (gene-pass chunk length, Z/X work-unit length, Z/X CTAs
    per SM) chosen by busseq_autotune's coordinate descent over burn-in sweeps
    of scratch chains.  Returns the keyword arguments for Sampler and the
    time per sweep they gave: {"chunk_cells", "zx_unit", "zx_ctas_per_sm",
    "ms_per_sweep"}."""
    n_b = np.ascontiguousarray(n_b, dtype=np.int32)
    on_dev = hasattr(Y, "data_ptr") and getattr(Y, "is_cuda", False)
    if on_dev:
        yptr, G = C.c_void_p(Y.data_ptr()), int(Y.shape[1])
    else:
        Yh = np.ascontiguousarray(Y, dtype=np.int32)
        yptr, G = Yh.ctypes.data_as(C.c_void_p), int(Yh.shape[1])
    dims = Dims(len(n_b), int(K), G, _p(n_b, _PI32))
    opt = Options(seed=int(seed) & 0xFFFFFFFFFFFFFFFF, p0=0.25, w_update=W_MH, keep_draws=0, device=int(device),
                  chunk_cells=0, hmc_leapfrog=int(hmc_leapfrog))
    ms = C.c_double()
    _check(lib().busseq_autotune(C.byref(dims), yptr, int(on_dev), C.byref(opt), int(sweeps), C.byref(ms)))
    return {"chunk_cells": int(opt.chunk_cells), "zx_unit": int(opt.zx_unit),
            "zx_ctas_per_sm": int(opt.zx_ctas_per_sm), "ms_per_sweep": float(ms.value)}


def estimate_buffers(B: int, K: int, G: int, N: int, with_XZ: bool = True, alloc=np.zeros) -> dict:
    """Arrays of the shapes and types Sampler.estimates() fills; ``alloc(shape,
    dtype)`` may return pinned host memory (for instance through torch) to speed
    up the copies of X and Z."""
    o = {"gamma": alloc((2, B), np.float64), "alpha": alloc((G,), np.float64),
         "L": alloc((max(K - 1, 1), G), np.float64), "beta": alloc((K, G), np.float64),
         "p_tau0": alloc((2,), np.float64), "nu": alloc((B, G), np.float64), "delta": alloc((N,), np.float64),
         "phi": alloc((B, G), np.float64), "W": alloc((N,), np.int32), "pi": alloc((B, K), np.float64)}
    if with_XZ:
        o["X"] = alloc((N, G), np.int32)
        o["Z"] = alloc((N, G), np.int32)
    return o


class Batch:
    """Chains (Samplers on one GPU, begun with the same run length) whose sweeps
    are launched together as one CUDA graph per sweep; each chain's draws are
    those it makes alone."""

    def __init__(self, samplers):
        self.samplers = list(samplers)
        arr = (C.c_void_p * len(self.samplers))(*[s._h.value if hasattr(s._h, "value") else s._h
                                                  for s in self.samplers])
        h = C.c_void_p()
        _check(lib().busseq_batch_create(arr, len(self.samplers), C.byref(h)))
        self._h = h

    def sweeps(self, count: int):
        _check(lib().busseq_batch_sweeps(self._h, int(count)))

    def synchronize(self):
        _check(lib().busseq_batch_synchronize(self._h))

    @property
    def stream(self) -> int:
        return int(lib().busseq_batch_stream(self._h) or 0)

    def close(self):
        if getattr(self, "_h", None):
            lib().busseq_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Sampler:
    """One BUSseq chain on one GPU (mirrors the reference program's pipeline:
    read counts -> initialise -> sweeps -> posterior -> files)."""

    def __init__(self, Y, n_b, K: int, seed: int = 0, p0: float = 0.25, w_update: str | int = "mh",
                 keep_draws: bool = False, device: int = 0, chunk_cells: int = 0, hmc_leapfrog: int = 0,
                 zx_summaries: bool = False, hmc_gene_accept: bool = False, test_nb_inv_cap: int = 0,
                 zx_unit: int = 0, zx_ctas_per_sm: int = 0):
        L = lib()
        self.n_b = np.ascontiguousarray(n_b, dtype=np.int32)
        self.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        self.B, self.K = len(self.n_b), int(K)
        self.N = int(self.n_b.sum())
        if isinstance(w_update, str):
            w_update = {"mh": W_MH, "gibbs": W_GIBBS}[w_update]
        opt = Options(seed=int(seed) & 0xFFFFFFFFFFFFFFFF, p0=float(p0), w_update=int(w_update),
                      keep_draws=int(bool(keep_draws)), device=int(device), chunk_cells=int(chunk_cells),
                      hmc_leapfrog=int(hmc_leapfrog), zx_summaries=int(bool(zx_summaries)),
                      hmc_gene_accept=int(bool(hmc_gene_accept)), test_nb_inv_cap=int(test_nb_inv_cap),
                      zx_unit=int(zx_unit), zx_ctas_per_sm=int(zx_ctas_per_sm))
        on_dev = hasattr(Y, "data_ptr") and getattr(Y, "is_cuda", False)
        if on_dev:
            assert Y.dtype.__str__().endswith("int32") and Y.is_contiguous() and Y.dim() == 2
            self.G = int(Y.shape[1])
            yptr = C.c_void_p(Y.data_ptr())
        else:
            Yh = np.ascontiguousarray(Y, dtype=np.int32)
            self.G = int(Yh.shape[1])
            yptr = Yh.ctypes.data_as(C.c_void_p)
            self._Yh = Yh
        if (Y.shape[0] if on_dev else self._Yh.shape[0]) != self.N:
            raise ValueError("Y has %d rows, n_b sums to %d" % (Y.shape[0], self.N))
        self._dims = Dims(self.B, self.K, self.G, _p(self.n_b, _PI32))
        h = C.c_void_p()
        _check(L.busseq_create(C.byref(self._dims), yptr, int(on_dev), C.byref(opt), C.byref(h)))
        self._h = h
        self._Yh = None
        self.n_kept = 0

    # -- lifecycle -----------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            lib().busseq_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def run(self, n_iter: int, n_burnin: int, n_unchanged: int):
        _check(lib().busseq_run(self._h, n_iter, n_burnin, n_unchanged))
        self.n_kept = n_iter - n_burnin

    def begin(self, n_iter: int, n_burnin: int, n_unchanged: int):
        _check(lib().busseq_begin(self._h, n_iter, n_burnin, n_unchanged))
        self.n_kept = n_iter - n_burnin

    def sweeps(self, count: int):
        _check(lib().busseq_sweeps(self._h, count))

    def synchronize(self):
        _check(lib().busseq_synchronize(self._h))

    def finish(self):
        _check(lib().busseq_finish(self._h))

    # -- results ---------------------------------------------------------------
    def estimate_buffers(self, with_XZ: bool = True, alloc=np.zeros) -> dict:
        return estimate_buffers(self.B, self.K, self.G, self.N, with_XZ, alloc)

    def estimates(self, with_XZ: bool = True, out: dict | None = None) -> dict:
        """Posterior estimates (and the last sweep's X and Z), into ``out`` when
        given (arrays from estimate_buffers)."""
        o = out if out is not None else self.estimate_buffers(with_XZ)
        e = Estimates()
        for k, v in o.items():
            if k in ("X", "Z"):
                continue
            assert v.flags.c_contiguous
            setattr(e, k, _p(v, _PI32 if v.dtype == np.int32 else _PD))
        if "X" in o:
            assert o["X"].flags.c_contiguous and o["Z"].flags.c_contiguous
            e.X, e.Z = _p(o["X"], _PI32), _p(o["Z"], _PI32)
        _check(lib().busseq_get_estimates(self._h, C.byref(e)))
        return o

    def preserved(self) -> dict:
        B, K, G, N, n = self.B, self.K, self.G, self.N, self.n_kept
        o = {"gamma": np.zeros((2 * B, n)), "alpha": np.zeros((G, n)), "L": np.zeros(((K - 1) * G, n), np.int32),
             "beta": np.zeros(((K - 1) * G, n)), "p_tau0": np.zeros((2, n)), "nu": np.zeros(((B - 1) * G, n)),
             "delta": np.zeros((N, n)), "phi": np.zeros((B * G, n)), "W": np.zeros((N, n), np.int32),
             "pi": np.zeros((B * K, n))}
        p = Preserved()
        for k, v in o.items():
            setattr(p, k, _p(v, _PI32 if v.dtype == np.int32 else _PD))
        _check(lib().busseq_get_preserved(self._h, C.byref(p)))
        return o

    def checkpoint_save(self, path: str):
        """Writes the chain and the run in progress to `path` (busseq_checkpoint_save)."""
        _check(lib().busseq_checkpoint_save(self._h, os.fsencode(path)))

    def checkpoint_load(self, path: str):
        """Restores a checkpoint written for the same counts, dimensions, seed and
        options; a run in progress continues with sweeps() / finish()."""
        _check(lib().busseq_checkpoint_load(self._h, os.fsencode(path)))
        kept = self._read_run_lengths(path)  # the Python side mirrors the restored run's length
        if kept is not None:
            self.n_kept = kept

    @staticmethod
    def _read_run_lengths(path: str):
        import struct
        with open(path, "rb") as f:
            head = f.read(8 + 4 + 4 * 11)
        if len(head) < 56 or head[:8] != b"BUSSEQCK":
            return None
        (_ver, _B, _K, _wu, _kd, begun, _fin, n_iter, n_burnin, _nu, _ih, _idev) = struct.unpack("<I11i", head[8:56])
        return (n_iter - n_burnin) if begun else None

    def bic(self) -> float:
        v = C.c_double()
        _check(lib().busseq_bic(self._h, C.byref(v)))
        return v.value

    def zx_summaries(self) -> dict:
        """Posterior mean of X and P(Z = 1) per entry over the kept sweeps (needs
        zx_summaries=True and a finished run)."""
        xm = np.zeros((self.N, self.G), np.float32)
        zp = np.zeros((self.N, self.G), np.float32)
        _check(lib().busseq_get_zx_summaries(self._h, xm.ctypes.data_as(C.c_void_p), zp.ctypes.data_as(C.c_void_p)))
        return {"x_mean": xm, "z_prob": zp}

    def corrected_counts(self, out=None) -> np.ndarray:
        """Batch-corrected counts [N, G] (int32): the last sweep's imputed counts
        mapped by randomised quantile matching onto NB(exp(alpha + beta_w), phi_1),
        with the posterior means and the posterior-mode types.  ``out`` may be
        a CUDA tensor (int32, N x G, contiguous) to keep the result on the
        device."""
        if out is not None and hasattr(out, "data_ptr"):
            if tuple(out.shape) != (self.N, self.G) or not out.is_contiguous() or out.element_size() != 4:
                raise ValueError("out must be a contiguous int32 tensor of shape (N, G)")
            _check(lib().busseq_corrected_counts(self._h, C.c_void_p(out.data_ptr()), 1))
            return out
        res = np.empty((self.N, self.G), np.int32)
        _check(lib().busseq_corrected_counts(self._h, res.ctypes.data_as(C.c_void_p), 0))
        return res

    def write_outputs(self, prefix: str, print_preserved: bool = False):
        _check(lib().busseq_write_outputs(self._h, prefix.encode(), int(print_preserved)))

    # -- state and stages ------------------------------------------------------
    def _state_arrays(self):
        B, K, G, N = self.B, self.K, self.G, self.N
        return {"X": np.zeros((N, G), np.int32), "Z": np.zeros((N, G), np.uint8), "W": np.zeros(N, np.int32),
                "L": np.zeros((K, G), np.int8), "alpha": np.zeros(G, np.float32),
                "mu_alpha": np.zeros(G, np.float32), "beta": np.zeros((K, G), np.float32),
                "nu": np.zeros((B, G), np.float32), "mu_nu": np.zeros(B, np.float32),
                "delta": np.zeros(N, np.float32), "mu_delta": np.zeros(N, np.float32),
                "phi": np.zeros((B, G), np.float32), "gamma": np.zeros((2, B), np.float32),
                "pi": np.zeros((B, K), np.float32), "p_tau0": np.zeros(2, np.float32)}

    @staticmethod
    def _ptr_for(v):
        return {np.int32: _PI32, np.uint8: _PU8, np.int8: _PI8, np.float32: _PF}[v.dtype.type]

    def get_state(self) -> dict:
        o = self._state_arrays()
        s = State()
        for k, v in o.items():
            setattr(s, k, _p(v, self._ptr_for(v)))
        _check(lib().busseq_get_state(self._h, C.byref(s)))
        return o

    def _state_struct(self, st: dict):
        """A State structure pointing at (converted copies of) the arrays in `st`,
        and the list that keeps those copies alive."""
        ref = self._state_arrays()
        s = State()
        keep = []
        for k, v in ref.items():
            if k not in st:
                continue
            a = np.ascontiguousarray(st[k], dtype=v.dtype).reshape(v.shape)
            keep.append(a)
            setattr(s, k, _p(a, self._ptr_for(a)))
        return s, keep

    def set_state(self, st: dict):
        s, keep = self._state_struct(st)
        _check(lib().busseq_set_state(self._h, C.byref(s)))
        del keep

    def run_stage(self, stage, it: int, n_unchanged: int = 1 << 30):
        if isinstance(stage, str):
            stage = STAGES[stage]
        _check(lib().busseq_run_stage(self._h, int(stage), int(it), int(n_unchanged)))

    def log_ratios(self) -> dict:
        B, K, G, N = self.B, self.K, self.G, self.N
        o = {"gamma": np.zeros((2, B)), "alpha": np.zeros(G), "beta": np.zeros((K, G)), "nu": np.zeros((B, G)),
             "delta": np.zeros(N), "phi": np.zeros((B, G)), "W": np.zeros(N)}
        r = LogRatios()
        for k, v in o.items():
            setattr(r, k, _p(v, _PD))
        _check(lib().busseq_get_log_ratios(self._h, C.byref(r)))
        return o

    # -- measurement -------------------------------------------------------------
    def set_stream(self, stream_ptr: int | None):
        _check(lib().busseq_set_stream(self._h, C.c_void_p(stream_ptr) if stream_ptr else None))

    def profile(self, n_sweeps: int) -> dict:
        """Mean event-timed milliseconds per sweep of every kernel (summed over
        its launches in a sweep); kernels the sampler does not launch read 0."""
        ms = np.zeros(64)
        n = C.c_int32()
        _check(lib().busseq_profile(self._h, n_sweeps, _p(ms, _PD), 64, C.byref(n)))
        return {lib().busseq_kernel_name(i).decode(): float(ms[i]) for i in range(n.value)}

    # ---- gradient-based block update (hmc_leapfrog > 0) ----------------------
    def _hmc_split(self, flat):
        G, K, B, N = self.G, self.K, self.B, self.N
        o, at = {}, 0
        for name, shape in (("alpha", (G,)), ("beta", (K, G)), ("nu", (B, G)), ("psi", (B, G)), ("delta", (N,))):
            n = int(np.prod(shape))
            o[name] = flat[at:at + n].reshape(shape)
            at += n
        return o

    def hmc_stats(self) -> dict:
        out = np.zeros(4)
        _check(lib().busseq_hmc_stats(self._h, _p(out, _PD)))
        return {"step_size": out[0], "accept_rate_kept": out[1], "last_accept_prob": out[2], "last_dH": out[3]}

    def hmc_gradient(self, with_metric: bool = True) -> dict:
        """Gradient (and metric) of the block log posterior at the current state."""
        n = self.G * (1 + self.K + 2 * self.B) + self.N
        g = np.zeros(n)
        m = np.zeros(n) if with_metric else None
        _check(lib().busseq_hmc_gradient(self._h, _p(g, _PD), _p(m, _PD) if m is not None else None))
        out = {"grad": self._hmc_split(g)}
        if m is not None:
            out["metric"] = self._hmc_split(m)
        return out

    def hmc_logpost_diff(self, from_state: dict) -> float:
        """Block log posterior of the current state minus that of `from_state`."""
        st, keep = self._state_struct(from_state)
        out = C.c_double()
        _check(lib().busseq_hmc_logpost_diff(self._h, C.byref(st), C.byref(out)))
        del keep
        return float(out.value)

    def hmc_gene_logpost_diff(self, from_state: dict) -> np.ndarray:
        """Per gene (hmc_gene_accept chains): the change of gene g's block log
        posterior from `from_state` (which must carry the current delta)."""
        st, keep = self._state_struct(from_state)
        out = np.zeros(self.G)
        _check(lib().busseq_hmc_gene_logpost_diff(self._h, C.byref(st), _p(out, _PD)))
        del keep
        return out

    def kernel_bytes(self, i: int) -> float:
        return float(lib().busseq_kernel_bytes(self._h, i))

    def launches_per_sweep(self, kept: bool) -> int:
        return int(lib().busseq_launches_per_sweep(self._h, int(kept)))
