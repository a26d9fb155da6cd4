"""Write fp64_tables.h: the tables of the FP64 Box-Muller transform in rng.cuh.

    python sdepy_gb300/csrc/make_fp64_tables.py

Every value is computed with Python's decimal module at 60 significant
digits and rounded once to the nearest double (float(Decimal) rounds
correctly), so each table entry is within half an ulp of the true value:

* logarithm (Tang's table-driven method, ACM TOMS 15(2), 1989): for
  c_j = 0.75 + j/128, j = 0..96, the exact c_j, 1/c_j and ln c_j; and the
  two-double split k ln 2 = hi + lo for k = -35..0;
* sin(pi v), cos(pi v) by angle addition: sin(pi n/64), cos(pi n/64) for
  n = -64..64; and pi split as hi + lo;
* sin x, cos x for the characteristic function (sde_process.cu): the same
  table, 64/pi, and pi/64 split into three doubles for the Cody-Waite
  reduction x = k pi/64 + r.

Pi comes from Machin's formula pi = 16 atan(1/5) - 4 atan(1/239), the
logarithm from the atanh series ln x = 2 atanh((x-1)/(x+1)), sine and cosine
from their Taylor series.
"""
import os
from decimal import Decimal, getcontext

getcontext().prec = 60
HERE = os.path.dirname(os.path.abspath(__file__))


def atan_inv(n):
    """atan(1/n) by its Taylor series."""
    x = Decimal(1)/n
    x2 = x*x
    s, t, k = Decimal(0), x, 0
    while True:
        term = t/(2*k + 1)
        if term == 0 or abs(term) < Decimal(10)**-70:
            break
        s += term if k % 2 == 0 else -term
        t *= x2
        k += 1
    return s


PI = 16*atan_inv(5) - 4*atan_inv(239)


def ln(x):
    x = Decimal(x)
    y = (x - 1)/(x + 1)
    y2 = y*y
    s, t, k = Decimal(0), y, 0
    while True:
        term = t/(2*k + 1)
        if abs(term) < Decimal(10)**-70:
            break
        s += term
        t *= y2
        k += 1
    return 2*s


LN2 = ln(2)


def sin_cos(x):
    x = Decimal(x)
    s, c = Decimal(0), Decimal(0)
    t, k = Decimal(1), 0   # x^k / k!
    while True:
        if abs(t) < Decimal(10)**-70 and k > 2:
            break
        if k % 2 == 1:
            s += t if (k // 2) % 2 == 0 else -t
        else:
            c += t if (k // 2) % 2 == 0 else -t
        k += 1
        t = t*x/k
    return s, c


def d(x):
    return float(x)


def fmt(v):
    return repr(v) if v != 0 else '0.0'


def main():
    cval = [Decimal(3)/4 + Decimal(j)/128 for j in range(97)]
    rows = []
    rows.append('// sin(pi v), cos(pi v) and ln(u) tables of the FP64 Box-Muller transform\n'
                '// (rng.cuh).  Written by make_fp64_tables.py; every entry is the nearest\n'
                '// double of a 60-digit decimal evaluation.\n#pragma once\n\nnamespace sdegpu {\n')

    def arr(name, vals, comment):
        rows.append('// %s\nstatic __device__ const double %s[%d] = {\n' % (comment, name, len(vals)))
        for i in range(0, len(vals), 3):
            rows.append('    ' + ', '.join(fmt(v) for v in vals[i:i + 3]) + ',\n')
        rows.append('};\n\n')

    arr('F64_LOG_C', [d(c) for c in cval], 'c_j = 0.75 + j/128, j = 0..96 (exact)')
    arr('F64_LOG_INVC', [d(1/c) for c in cval], '1 / c_j')
    arr('F64_LOG_LNC', [d(ln(c)) for c in cval], 'ln c_j')
    khi, klo = [], []
    for k in range(-35, 1):
        v = k*LN2
        hi = d(v)
        khi.append(hi)
        klo.append(d(v - Decimal(hi)))
    arr('F64_KLN2_HI', khi, 'k ln 2 = hi + lo, k = -35..0 (index k + 35)')
    arr('F64_KLN2_LO', klo, '')
    sn, cs = [], []
    for n in range(-64, 65):
        s, c = sin_cos(PI*n/64)
        sn.append(d(s))
        cs.append(d(c))
    # exact zeros where the true value is zero
    sn[0] = sn[64] = sn[128] = 0.0
    cs[32] = cs[96] = 0.0
    arr('F64_SINPI_N', sn, 'sin(pi n/64), n = -64..64 (index n + 64)')
    arr('F64_COSPI_N', cs, 'cos(pi n/64)')
    pi_hi = d(PI)
    pi_lo = d(PI - Decimal(pi_hi))
    rows.append('// pi = hi + lo\nstatic constexpr double F64_PI_HI = %r;\nstatic constexpr double F64_PI_LO = %r;\n\n'
                % (pi_hi, pi_lo))
    q = PI/64
    q1 = d(q)
    q2 = d(q - Decimal(q1))
    q3 = d(q - Decimal(q1) - Decimal(q2))
    rows.append('// 64 / pi, and pi / 64 = c1 + c2 + c3\n'
                'static constexpr double F64_INV_PIO64 = %r;\n'
                'static constexpr double F64_PIO64_1 = %r;\n'
                'static constexpr double F64_PIO64_2 = %r;\n'
                'static constexpr double F64_PIO64_3 = %r;\n\n' % (d(64/PI), q1, q2, q3))
    rows.append('}  // namespace sdegpu\n')
    with open(os.path.join(HERE, 'fp64_tables.h'), 'w') as f:
        f.write(''.join(rows))


if __name__ == '__main__':
    main()
