"""Division operand pairs whose quotient lies as close to a rounding midpoint as quotients of
doubles can: for an odd 53-bit significand B and a small odd c, M = c / B mod 2^54 is odd,
and a = (M B - c) / 2^54 is an integer; where M has 54 significant bits and a 53, the
quotient a / B = M / 2^54 - c / (2^54 B) sits c * 2^-54 ulp from the midpoint M / 2^54 (or
on the other side for -c).  A correctly rounded division must still round these to the right
neighbour; a faithful one would not.  Operands are scaled by random powers of two within the
tame range (2^-200 <= |x| < 2^201) and given random signs.
"""
import numpy as np

_P54 = 1 << 54


def midpoint_cases(rng, n, emax=90):
    a_out, b_out = [], []
    while len(a_out) < n:
        B = int(rng.integers(1 << 52, 1 << 53)) | 1
        c = int(rng.integers(1, 64)) * 2 + 1
        sgn = 1 if rng.random() < 0.5 else -1
        M = (sgn * c * pow(B, -1, _P54)) % _P54
        if M < (1 << 53) or not (M & 1):
            continue
        num = M * B - sgn * c
        assert num % _P54 == 0
        a = num // _P54
        if not ((1 << 52) <= a < (1 << 53)):
            continue
        ea, eb = rng.integers(-emax, emax + 1, 2)
        sa = -1.0 if rng.random() < 0.5 else 1.0
        sb = -1.0 if rng.random() < 0.5 else 1.0
        a_out.append(sa * np.ldexp(float(a), int(ea) - 52))
        b_out.append(sb * np.ldexp(float(B), int(eb) - 52))
    return np.array(a_out), np.array(b_out)
