"""Correctly rounded sin/cos/tan/sinh/cosh of doubles, for constant folding.

The reference writes element constants into its kernel source as literals
(ufo/methods.py:117-123, :150-156, :202-208).  A C compiler folds a math call
whose argument is a literal at compile time, and GCC does so with MPFR, i.e.
the result is the double nearest to the exact value.  The same call on a
runtime value goes to the C library, which may differ in the last bit.  To
reproduce the folded constants bit for bit this module evaluates the
functions in ~70-digit decimal arithmetic (standard library ``decimal``) and
rounds once to the nearest double.  Methods: Machin's formula for pi,
argument reduction modulo pi/2, Taylor series for sin/cos on [-pi/4, pi/4],
and exp by Taylor series after halving the argument.
"""
import decimal
import math
from decimal import Decimal

_PREC = 80
_ctx = decimal.Context(prec=_PREC)


def _atan_inv(n, ctx):
    """atan(1/n) by its Taylor series."""
    x = ctx.divide(Decimal(1), Decimal(n))
    x2 = ctx.multiply(x, x)
    term = x
    total = x
    k = 1
    eps = Decimal(10) ** (-(ctx.prec + 5))
    while True:
        term = ctx.multiply(term, -x2)
        k += 2
        t = ctx.divide(term, Decimal(k))
        if abs(t) < eps:
            break
        total = ctx.add(total, t)
    return total


def _pi(ctx):
    return ctx.subtract(ctx.multiply(Decimal(16), _atan_inv(5, ctx)),
                        ctx.multiply(Decimal(4), _atan_inv(239, ctx)))


_PI = _pi(decimal.Context(prec=_PREC + 40))


def _sin_cos_small(r, ctx):
    """(sin r, cos r) by Taylor series for |r| <= pi/4."""
    r2 = ctx.multiply(r, r)
    eps = Decimal(10) ** (-(ctx.prec + 5))
    s = term = r
    k = 1
    while True:
        term = ctx.divide(ctx.multiply(term, -r2), Decimal((k + 1) * (k + 2)))
        k += 2
        if abs(term) < eps:
            break
        s = ctx.add(s, term)
    c = term = Decimal(1)
    k = 0
    while True:
        term = ctx.divide(ctx.multiply(term, -r2), Decimal((k + 1) * (k + 2)))
        k += 2
        if abs(term) < eps:
            break
        c = ctx.add(c, term)
    return s, c


def _sin_cos(x):
    ctx = decimal.Context(prec=_PREC + 20)
    d = Decimal(x)  # exact value of the double
    half_pi = ctx.divide(_PI, Decimal(2))
    q = int(ctx.divide(d, half_pi).to_integral_value(rounding=decimal.ROUND_HALF_EVEN))
    r = ctx.subtract(d, ctx.multiply(Decimal(q), half_pi))
    s, c = _sin_cos_small(r, ctx)
    q %= 4
    if q == 0:
        return s, c
    if q == 1:
        return c, -s
    if q == 2:
        return -s, -c
    return -c, s


def _exp(d, ctx):
    k = 0
    while abs(d) > Decimal('0.01'):
        d = ctx.divide(d, Decimal(2))
        k += 1
    eps = Decimal(10) ** (-(ctx.prec + 5))
    total = term = Decimal(1)
    n = 0
    while True:
        n += 1
        term = ctx.divide(ctx.multiply(term, d), Decimal(n))
        if abs(term) < eps:
            break
        total = ctx.add(total, term)
    for _ in range(k):
        total = ctx.multiply(total, total)
    return total


def _round(d):
    return float(format(d, 'e')) if d != 0 else 0.0


def _special(x, fn):
    if math.isnan(x) or math.isinf(x):
        return fn(x) if not math.isinf(x) or fn in (math.sinh, math.cosh) else float('nan')
    return None


def sin(x):
    x = float(x)
    if not math.isfinite(x):
        return float('nan')
    if x == 0.0:
        return x
    return _round(_sin_cos(x)[0])


def cos(x):
    x = float(x)
    if not math.isfinite(x):
        return float('nan')
    return _round(_sin_cos(x)[1])


def tan(x):
    x = float(x)
    if not math.isfinite(x):
        return float('nan')
    if x == 0.0:
        return x
    s, c = _sin_cos(x)
    ctx = decimal.Context(prec=_PREC + 20)
    return _round(ctx.divide(s, c))


def sinh(x):
    x = float(x)
    if not math.isfinite(x) or abs(x) > 700:
        return math.sinh(x)
    if x == 0.0:
        return x
    ctx = decimal.Context(prec=_PREC + 20)
    e = _exp(Decimal(x), ctx)
    return _round(ctx.divide(ctx.subtract(e, ctx.divide(Decimal(1), e)), Decimal(2)))


def cosh(x):
    x = float(x)
    if not math.isfinite(x) or abs(x) > 700:
        return math.cosh(x)
    ctx = decimal.Context(prec=_PREC + 20)
    e = _exp(Decimal(x), ctx)
    return _round(ctx.divide(ctx.add(e, ctx.divide(Decimal(1), e)), Decimal(2)))
