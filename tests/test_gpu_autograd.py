"""The hand-written adjoint kernel behind a torch.autograd.Function (test
harness only), checked by torch.autograd.gradcheck.

BlockLogPost maps the free coordinates theta = (alpha, beta_{k>=1},
nu_{b>=1}, delta of every cell but the first of its batch, psi = log phi)
to the block log posterior of the gradient-based update.  Its forward value
is the FP64 oracle's log posterior (oracle/oracle.cpp, orc_hmc_logpost); its
backward is the GPU's gradient (k_hmc_grad + k_hmc_assemble through
busseq_hmc_gradient).  gradcheck compares that backward with central
differences of the forward (step h = 1e-3, in FP64), so it checks the
kernel's gradient against finite differences of the oracle's log posterior.

Tolerance: |gpu - fd| <= 2e-3 sqrt(max observed information) + 1e-3 |fd|,
the gradient tolerance of the other HMC tests (the kernels sum float terms),
with the central-difference truncation error (h^2/6 times a third derivative
of the size of the information) far below it.
"""
import numpy as np
import pytest

import busseq_gpu_gb300 as bq
from tests.parity_util import oracle_state

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

N_B, G, K, SEED = [14, 12], 24, 3, 41


class Layout:
    """Packing of the free coordinates of the block into one vector."""

    def __init__(self, n_b, G, K):
        self.B, self.G, self.K = len(n_b), G, K
        off = np.concatenate([[0], np.cumsum(n_b)])[:-1]
        self.free_delta = np.ones(int(sum(n_b)), bool)
        self.free_delta[off] = False
        self.sizes = [G, (K - 1) * G, (self.B - 1) * G, int(self.free_delta.sum()), self.B * G]

    def pack(self, alpha, beta, nu, delta, psi):
        return np.concatenate([np.ravel(alpha), np.ravel(beta[1:]), np.ravel(nu[1:]), np.ravel(delta)[self.free_delta],
                               np.ravel(psi)])

    def unpack(self, theta, base):
        """A state dict (float64) with the block replaced by theta."""
        t = np.asarray(theta, np.float64)
        parts = np.split(t, np.cumsum(self.sizes)[:-1])
        st = {k: np.array(v, np.float64, copy=True) for k, v in base.items() if k not in ("X", "Z", "W", "L")}
        st.update({k: base[k] for k in ("X", "Z", "W", "L")})
        st["alpha"] = parts[0].copy()
        beta = np.zeros((self.K, self.G))
        beta[1:] = parts[1].reshape(self.K - 1, self.G)
        nu = np.zeros((self.B, self.G))
        nu[1:] = parts[2].reshape(self.B - 1, self.G)
        delta = np.asarray(base["delta"], np.float64).copy()
        delta[self.free_delta] = parts[3]
        st.update(beta=beta, nu=nu, delta=delta, phi=np.exp(parts[4].reshape(self.B, self.G)))
        return st


class BlockLogPost(torch.autograd.Function):
    """forward: the FP64 oracle's block log posterior; backward: the GPU adjoint."""

    @staticmethod
    def forward(ctx, theta, env):
        st = env["layout"].unpack(theta.detach().cpu().numpy(), env["base"])
        ctx.env = env
        ctx.st = st
        o = oracle_state(env["Y"], np.array(N_B), K, SEED, st)
        return torch.tensor(o.hmc_logpost(), dtype=torch.float64)

    @staticmethod
    def backward(ctx, gout):
        env, st = ctx.env, ctx.st
        s = env["sampler"]
        s.set_state({k: (v.astype(np.float32) if v.dtype == np.float64 else v) for k, v in st.items()})
        g = s.hmc_gradient(with_metric=False)["grad"]
        v = env["layout"].pack(g["alpha"], g["beta"], g["nu"], g["delta"], g["psi"])
        return gout * torch.from_numpy(v).to(torch.float64), None


def test_adjoint_kernel_passes_gradcheck_against_the_oracle():
    Y, _, _ = bq.simulate(N_B, G, K, SEED)
    mh = bq.Sampler(Y, N_B, K, seed=SEED, p0=0.3)
    mh.begin(12, 12, 0)
    mh.sweeps(12)
    mh.synchronize()
    base = mh.get_state()
    mh.close()
    lay = Layout(N_B, G, K)
    theta0 = lay.pack(base["alpha"], base["beta"], base["nu"], base["delta"], np.log(base["phi"]))
    theta = torch.tensor(theta0, dtype=torch.float64, requires_grad=True)
    h = bq.Sampler(Y, N_B, K, seed=SEED, hmc_leapfrog=5)
    try:
        o = oracle_state(Y, np.array(N_B), K, SEED, lay.unpack(theta0, base))
        metric = o.hmc_grad()["metric"]
        info = max(float(np.max(m)) for m in metric.values())
        env = {"layout": lay, "base": base, "Y": Y, "sampler": h}
        f = lambda t: BlockLogPost.apply(t, env)  # noqa: E731
        assert torch.autograd.gradcheck(f, (theta,), eps=1e-3, atol=2e-3 * np.sqrt(info), rtol=1e-3,
                                        raise_exception=True)
        # one backward through the wrapper equals the kernel's gradient
        lp = f(theta)
        lp.backward()
        s_st = lay.unpack(theta0, base)
        h.set_state({k: (v.astype(np.float32) if v.dtype == np.float64 else v) for k, v in s_st.items()})
        g = h.hmc_gradient(with_metric=False)["grad"]
        want = lay.pack(g["alpha"], g["beta"], g["nu"], g["delta"], g["psi"])
        np.testing.assert_array_equal(theta.grad.numpy(), want)
    finally:
        h.close()
