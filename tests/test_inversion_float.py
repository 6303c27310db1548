"""The NB proposal's distribution-function inversion runs in single precision
on the device for means below 32 (and dispersions >= 1).  This restates its
recurrence in numpy float32 -- P(0) = (phi / (phi + mu))^phi, then
P(k+1) = P(k) q (phi + k) / (k + 1), with F summed until it passes u -- and
checks it against the same search in double precision on random and on
stress draws (means 24..32, dispersions 100..1000, the largest exponent of
P(0)).  numpy's float32 exp and log1p stand in for the device's, which have
errors of the same order."""
import numpy as np

f32 = np.float32


def _inv_f32(mu, phi, u):
    q = f32(mu) / (f32(phi) + f32(mu))
    p = f32(np.exp(f32(phi) * f32(np.log1p(-q))))
    F, k = p, 0
    while u > F and k < 1024:
        p = f32(p * (q * f32(f32(phi + k) / f32(k + 1))))
        k += 1
        Fn = f32(F + p)
        if Fn == F:
            break
        F = Fn
    return k


def _inv_f64(mu, phi, u):
    q = mu / (phi + mu)
    p = np.exp(phi * np.log1p(-q))
    F, k = p, 0
    while u > F and k < 1024:
        p = p * (q * ((phi + k) / (k + 1)))
        k += 1
        F = F + p
    return k


def _draws(rng, n, mu_lo, mu_hi, phi_lo, phi_hi):
    bad = 0
    for _ in range(n):
        mu = rng.uniform(mu_lo, mu_hi)
        phi = float(np.exp(rng.uniform(np.log(phi_lo), np.log(phi_hi))))
        u = f32((int(rng.integers(0, 2 ** 23)) * 2 + 1) * 2.0 ** -24)  # the kernels' uniform grid
        bad += _inv_f32(mu, phi, u) != _inv_f64(mu, phi, float(u))
    return bad


def test_float_inversion_matches_double():
    rng = np.random.default_rng(7)
    assert _draws(rng, 1500, 0.5, 32.0, 1.0, 1000.0) == 0
    assert _draws(rng, 1500, 24.0, 32.0, 100.0, 1000.0) == 0
