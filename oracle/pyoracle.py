"""ctypes wrapper of the FP64 oracle (oracle/oracle.cpp) -- test infrastructure.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline / reference
arm import this module.  The product package never does.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

STAGE_ZX_GAMMA_ALPHA_L = 0
STAGE_BETA_NU = 1
STAGE_DELTA = 2
STAGE_PHI = 3
STAGE_W = 4
STAGE_PI = 5
N_STAGES = 6

_PD = C.POINTER(C.c_double)
_PI32 = C.POINTER(C.c_int32)
_PU8 = C.POINTER(C.c_uint8)
_PI8 = C.POINTER(C.c_int8)


class OrcState(C.Structure):
    _fields_ = [
        ("B", C.c_int32), ("K", C.c_int32), ("G", C.c_int64), ("N", C.c_int64),
        ("n_b", _PI32), ("Y", _PI32), ("X", _PI32), ("Z", _PU8), ("W", _PI32), ("L", _PI8),
        ("alpha", _PD), ("mu_alpha", _PD), ("beta", _PD), ("nu", _PD), ("mu_nu", _PD),
        ("delta", _PD), ("mu_delta", _PD), ("phi", _PD), ("gamma", _PD), ("pi", _PD),
        ("p_tau0", _PD), ("seed", C.c_uint64),
    ]


_DEBUG_FIELDS = ["lr_gamma", "lr_alpha", "lr_beta", "lr_nu", "lr_delta", "lr_phi", "lr_W",
                 "mg_zx", "mg_gamma", "mg_alpha", "mg_L", "mg_beta", "mg_nu", "mg_delta",
                 "mg_phi", "mg_W", "mg_ptau", "mg_pi",
                 "sc_gamma", "sc_alpha", "sc_beta", "sc_nu", "sc_delta", "sc_phi", "sc_W"]


class OrcDebug(C.Structure):
    _fields_ = [(f, _PD) for f in _DEBUG_FIELDS]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = C.CDLL(path)
        L.orc_init.argtypes = [C.POINTER(OrcState), C.c_double]
        L.orc_init_given_W.argtypes = [C.POINTER(OrcState), _PD, _PD]
        L.orc_stage.argtypes = [C.POINTER(OrcState), C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(OrcDebug)]
        L.orc_step.argtypes = [C.POINTER(OrcState), C.c_char_p, C.c_int, C.c_int, C.POINTER(OrcDebug)]
        L.orc_sweep.argtypes = [C.POINTER(OrcState), C.c_int, C.c_int, C.c_int]
        L.orc_bic.argtypes = [C.POINTER(OrcState), _PD]
        L.orc_bic.restype = C.c_double
        L.orc_uniforms.argtypes = [C.c_uint64, C.c_uint32, C.c_uint64, C.c_uint32, C.c_int, _PD]
        L.orc_philox.argtypes = [C.POINTER(C.c_uint32), C.c_uint32, C.c_uint32, C.POINTER(C.c_uint32)]
        L.orc_sample_gamma.argtypes = [C.c_uint64, C.c_double, C.c_int, _PD]
        L.orc_sample_poisson.argtypes = [C.c_uint64, C.c_double, C.c_int, _PI32]
        L.orc_sample_negbin.argtypes = [C.c_uint64, C.c_double, C.c_double, C.c_int, _PI32]
        for f in ("orc_term_shift",):
            getattr(L, f).argtypes = [C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]
            getattr(L, f).restype = C.c_double
        L.orc_term_phi.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int]
        L.orc_term_phi.restype = C.c_double
        L.orc_term_gamma0.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int, C.c_int]
        L.orc_term_gamma0.restype = C.c_double
        L.orc_term_gamma1.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int, C.c_int]
        L.orc_term_gamma1.restype = C.c_double
        L.orc_hmc_logpost.argtypes = [C.POINTER(OrcState)]
        L.orc_hmc_logpost.restype = C.c_double
        L.orc_hmc_grad.argtypes = [C.POINTER(OrcState)] + [_PD] * 10
        L.orc_corrected_counts.argtypes = [C.POINTER(OrcState), _PI32, _PD]
        L.orc_num_threads.restype = C.c_int
        L.orc_set_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def _ptr(a, t):
    return a.ctypes.data_as(t)


class State:
    """Host state in double precision, owned by numpy arrays."""

    FLOAT_FIELDS = ["alpha", "mu_alpha", "beta", "nu", "mu_nu", "delta", "mu_delta", "phi", "gamma", "pi", "p_tau0"]

    def __init__(self, Y, n_b, K, seed):
        Y = np.ascontiguousarray(Y, dtype=np.int32)
        self.N, self.G = Y.shape
        self.n_b = np.ascontiguousarray(n_b, dtype=np.int32)
        self.B = len(self.n_b)
        self.K = int(K)
        assert int(self.n_b.sum()) == self.N
        self.seed = int(seed)
        N, G, B, K = self.N, self.G, self.B, self.K
        self.Y = Y
        self.X = Y.copy()
        self.Z = np.zeros((N, G), np.uint8)
        self.W = np.zeros(N, np.int32)
        self.L = np.zeros((K, G), np.int8)
        self.alpha = np.zeros(G)
        self.mu_alpha = np.zeros(G)
        self.beta = np.zeros((K, G))
        self.nu = np.zeros((B, G))
        self.mu_nu = np.zeros(B)
        self.delta = np.zeros(N)
        self.mu_delta = np.zeros(N)
        self.phi = np.full((B, G), 5.0)
        self.gamma = np.zeros((2, B))
        self.pi = np.full((B, K), 1.0 / K)
        self.p_tau0 = np.array([0.25, 0.005])

    def c(self) -> OrcState:
        s = OrcState()
        s.B, s.K, s.G, s.N = self.B, self.K, self.G, self.N
        s.n_b = _ptr(self.n_b, _PI32)
        s.Y = _ptr(self.Y, _PI32)
        s.X = _ptr(self.X, _PI32)
        s.Z = _ptr(self.Z, _PU8)
        s.W = _ptr(self.W, _PI32)
        s.L = _ptr(self.L, _PI8)
        for f in self.FLOAT_FIELDS:
            arr = getattr(self, f)
            assert arr.dtype == np.float64 and arr.flags.c_contiguous, f
            setattr(s, f, _ptr(arr, _PD))
        s.seed = self.seed
        self._keep = s
        return s

    def copy(self) -> "State":
        o = State.__new__(State)
        for k, v in self.__dict__.items():
            if k == "_keep":
                continue
            setattr(o, k, v.copy() if isinstance(v, np.ndarray) else v)
        return o

    # ---- operations -------------------------------------------------------
    def init(self, p0: float) -> None:
        lib().orc_init(C.byref(self.c()), float(p0))

    def init_given_W(self):
        raw = np.zeros((self.B, self.K, self.G))
        bm = np.zeros(self.B)
        lib().orc_init_given_W(C.byref(self.c()), _ptr(raw, _PD), _ptr(bm, _PD))
        return raw, bm

    def stage(self, stage: int, it: int, n_unchanged: int = 0, w_update: int = 0, debug: "Debug | None" = None):
        d = debug.c() if debug is not None else None
        r = lib().orc_stage(C.byref(self.c()), stage, it, n_unchanged, w_update, C.byref(d) if d else None)
        if r != 0:
            raise ValueError("bad stage %r" % stage)

    def step(self, which: str, it: int, w_update: int = 0, debug: "Debug | None" = None):
        d = debug.c() if debug is not None else None
        r = lib().orc_step(C.byref(self.c()), which.encode(), it, w_update, C.byref(d) if d else None)
        if r != 0:
            raise ValueError("bad step %r" % which)

    def sweep(self, it: int, n_unchanged: int, w_update: int = 0):
        lib().orc_sweep(C.byref(self.c()), it, n_unchanged, w_update)

    def hmc_logpost(self) -> float:
        """Log posterior of (alpha, beta, nu, delta, log phi) given the rest, up to a constant."""
        return lib().orc_hmc_logpost(C.byref(self.c()))

    def hmc_grad(self) -> dict:
        """Gradient of hmc_logpost (psi = log phi) and the diagonal metric."""
        G, K, B, N = self.G, self.K, self.B, self.N
        o = {"alpha": np.zeros(G), "beta": np.zeros((K, G)), "nu": np.zeros((B, G)), "delta": np.zeros(N),
             "psi": np.zeros((B, G))}
        m = {k: np.zeros_like(v) for k, v in o.items()}
        lib().orc_hmc_grad(C.byref(self.c()), *[_ptr(o[k], _PD) for k in ("alpha", "beta", "nu", "delta", "psi")],
                           *[_ptr(m[k], _PD) for k in ("alpha", "beta", "nu", "delta", "psi")])
        return {"grad": o, "metric": m}

    def bic(self):
        ll = np.zeros((self.K, self.N))
        v = lib().orc_bic(C.byref(self.c()), _ptr(ll, _PD))
        return v, ll


def corrected_counts(X, n_b, seed, est):
    """Oracle of the batch-corrected counts from the imputed counts X [N, G] and
    the estimates (alpha [G], beta [K, G], nu [B, G], delta [N], phi [B, G],
    W [N]).  Returns (counts [N, G] int32, margin [N, G]): margin is the
    relative distance of each entry's probability position from the nearer
    bracketing tail value of the corrected distribution, negative where the
    position underflowed and was floored at 1e-280."""
    X = np.ascontiguousarray(X, dtype=np.int32)
    beta = np.ascontiguousarray(est["beta"], dtype=np.float64)
    st = State(X, n_b, beta.shape[0], seed)
    st.W = np.ascontiguousarray(est["W"], dtype=np.int32)
    for f in ("alpha", "nu", "delta", "phi"):
        setattr(st, f, np.ascontiguousarray(est[f], dtype=np.float64))
    st.beta = beta
    out = np.zeros(X.shape, np.int32)
    mg = np.zeros(X.shape)
    lib().orc_corrected_counts(C.byref(st.c()), _ptr(out, _PI32), _ptr(mg, _PD))
    return out, mg


class Debug:
    def __init__(self, st: State):
        B, K, G, N = st.B, st.K, st.G, st.N
        shapes = {
            "lr_gamma": (2, B), "lr_alpha": (G,), "lr_beta": (K, G), "lr_nu": (B, G), "lr_delta": (N,),
            "lr_phi": (B, G), "lr_W": (N,), "mg_zx": (N, G), "mg_gamma": (2, B), "mg_alpha": (G,),
            "mg_L": (K, G), "mg_beta": (K, G), "mg_nu": (B, G), "mg_delta": (N,), "mg_phi": (B, G),
            "mg_W": (N,), "mg_ptau": (2,), "mg_pi": (B, K),
            "sc_gamma": (2, B), "sc_alpha": (G,), "sc_beta": (K, G), "sc_nu": (B, G), "sc_delta": (N,),
            "sc_phi": (B, G), "sc_W": (N,),
        }
        for k, shp in shapes.items():
            setattr(self, k, np.full(shp, np.inf if k.startswith("mg") else 0.0 if k.startswith("sc") else np.nan))

    def c(self) -> OrcDebug:
        d = OrcDebug()
        for f in _DEBUG_FIELDS:
            setattr(d, f, _ptr(getattr(self, f), _PD))
        self._keep = d
        return d


def uniforms(seed: int, sid: int, entity: int, it: int, n: int) -> np.ndarray:
    out = np.zeros(n)
    lib().orc_uniforms(seed, sid, entity, it, n, _ptr(out, _PD))
    return out


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*[int(x) & 0xFFFFFFFF for x in ctr])
    o = (C.c_uint32 * 4)()
    lib().orc_philox(c, int(key[0]) & 0xFFFFFFFF, int(key[1]) & 0xFFFFFFFF, o)
    return [int(x) for x in o]


def sample_gamma(seed, a, n):
    out = np.zeros(n)
    lib().orc_sample_gamma(seed, a, n, _ptr(out, _PD))
    return out


def sample_poisson(seed, lam, n):
    out = np.zeros(n, np.int32)
    lib().orc_sample_poisson(seed, lam, n, _ptr(out, _PI32))
    return out


def sample_negbin(seed, mu, phi, n):
    out = np.zeros(n, np.int32)
    lib().orc_sample_negbin(seed, mu, phi, n, _ptr(out, _PI32))
    return out


class _SimParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("alpha_lo", "alpha_hi", "de_frac", "beta_lo", "beta_hi", "nu_step",
                                          "nu_sd", "delta_sd", "phi_lo", "phi_hi", "pi_conc", "gamma0", "gamma1")]


class _Dims(C.Structure):
    _fields_ = [("B", C.c_int32), ("K", C.c_int32), ("G", C.c_int64), ("n_b", _PI32)]


_sim = None


def simulate(n_b, G: int, K: int, seed: int, params: dict):
    """(Y [N, G], W_true [N]) from the generator built alone (oracle/lib/libsim.so):
    the same counts as the product library's generator for the same seed and
    parameters, without loading that library."""
    global _sim
    if _sim is None:
        _sim = C.CDLL(_build.build_sim())
        _sim.busseq_simulate.argtypes = [C.POINTER(_Dims), C.POINTER(_SimParams), C.c_uint64, _PI32, _PI32, _PI32]
        _sim.sim_last_error.restype = C.c_char_p
    n_b = np.ascontiguousarray(n_b, dtype=np.int32)
    N = int(n_b.sum())
    Y = np.zeros((N, G), np.int32)
    W = np.zeros(N, np.int32)
    d = _Dims(len(n_b), int(K), int(G), _ptr(n_b, _PI32))
    sp = _SimParams(**params)
    rc = _sim.busseq_simulate(C.byref(d), C.byref(sp), int(seed), _ptr(Y, _PI32), _ptr(W, _PI32), None)
    if rc != 0:
        raise RuntimeError("simulate: %s" % _sim.sim_last_error().decode())
    return Y, W


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def num_threads() -> int:
    return int(lib().orc_num_threads())
