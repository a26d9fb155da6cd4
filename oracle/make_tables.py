"""ORACLE -- test infrastructure only.  Writes oracle/oracle_tables.h, the
constants of the FP64 Box-Muller transform restated in rng_oracle.c
(Tang's table-driven logarithm, ACM TOMS 15(2), 1989, and sin / cos of
pi v by angle addition over pi n / 64), each the nearest double of a
50-digit mpmath evaluation -- computed independently of the library's own
table generator, so that a test can compare the two sets entry by entry.

    python oracle/make_tables.py
"""
import os

import mpmath

mpmath.mp.dps = 50
HERE = os.path.dirname(os.path.abspath(__file__))


def dbl(x):
    """Nearest double of an mpmath number (correct rounding via its exact
    rational value)."""
    from fractions import Fraction
    sign, man, exp, _ = mpmath.mpf(x)._mpf_
    v = Fraction(int(man))*Fraction(2)**int(exp)
    return float(-v if sign else v)


def tables():
    c = [mpmath.mpf(3)/4 + mpmath.mpf(j)/128 for j in range(97)]
    t = {'ORC_LOG_C': [dbl(x) for x in c],
         'ORC_LOG_INVC': [dbl(1/x) for x in c],
         'ORC_LOG_LNC': [dbl(mpmath.log(x)) for x in c]}
    hi, lo = [], []
    for k in range(-35, 1):
        v = k*mpmath.log(2)
        h = dbl(v)
        hi.append(h)
        lo.append(dbl(v - mpmath.mpf(h)))
    t['ORC_KLN2_HI'], t['ORC_KLN2_LO'] = hi, lo
    t['ORC_SINPI_N'] = [0.0 if n % 64 == 0 else dbl(mpmath.sinpi(mpmath.mpf(n)/64)) for n in range(-64, 65)]
    t['ORC_COSPI_N'] = [0.0 if (n + 32) % 64 == 0 else dbl(mpmath.cospi(mpmath.mpf(n)/64)) for n in range(-64, 65)]
    t['ORC_PI_HI'] = dbl(mpmath.pi)
    return t


def main():
    t = tables()
    out = ['/* ORACLE -- test infrastructure only.  Written by oracle/make_tables.py:\n'
           ' * nearest doubles of 50-digit mpmath values. */\n#pragma once\n\n']
    for name, v in t.items():
        if isinstance(v, float):
            out.append('static const double %s = %r;\n' % (name, v))
            continue
        out.append('static const double %s[%d] = {\n' % (name, len(v)))
        for i in range(0, len(v), 3):
            out.append('    ' + ', '.join(repr(x) if x != 0 else '0.0' for x in v[i:i + 3]) + ',\n')
        out.append('};\n')
    with open(os.path.join(HERE, 'oracle_tables.h'), 'w') as f:
        f.write(''.join(out))


if __name__ == '__main__':
    main()
