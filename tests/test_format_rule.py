"""The rule the device formatter uses for printf("%f") of a float (CPU check of
the algorithm): with v = m 2^e, R = round-half-even(m 10^6 2^e) in integers,
printed as sign, R // 10^6, '.', R % 10^6 zero-padded.  Compared with Python's
correctly rounded "%f" on edge values: exact ties, negative zero, subnormals,
values near the limit the device path covers (|v| < 2^43)."""
import struct

import numpy as np


def f6(v: float) -> str:
    bits = struct.unpack("<I", struct.pack("<f", v))[0]
    neg = bits >> 31
    E = (bits >> 23) & 0xFF
    frac = bits & 0x7FFFFF
    m = (frac | 0x800000) if E else frac
    e = E - 150 if E else -149
    t = m * 1000000
    if e >= 0:
        assert e <= 19
        R = t << e
    else:
        sh = -e
        if sh >= 64:
            R = 0
        else:
            q, rem, half = t >> sh, t & ((1 << sh) - 1), 1 << (sh - 1)
            R = q + (1 if rem > half or (rem == half and q & 1) else 0)
    return ("-" if neg else "") + "%d.%06d" % (R // 1000000, R % 1000000)


def test_rule_matches_printf_on_edge_values():
    vals = [0.0, -0.0, 1.0, -1.0, 0.5, 1 / 128, 3 / 128, 5 / 128, -7 / 128, 1e-7, 4e-7, 5e-7, 6e-7, -5e-7,
            1.5e-45, -1.4e-45, 1.17549435e-38, 0.1, 0.2, 0.3, 123.456789, 99999.9999995, 2.0 ** 42, -(2.0 ** 42),
            8388607.5, 16777215.0, 3.4028e12]
    rng = np.random.default_rng(0)
    vals += list(rng.normal(0, 3, 2000)) + list(rng.uniform(-1e-5, 1e-5, 500)) + list(rng.uniform(0, 5e4, 500))
    for v in vals:
        f = float(np.float32(v))
        assert f6(f) == "%f" % f, (v, f6(f), "%f" % f)
