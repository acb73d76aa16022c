"""The C-expression compiler (ufo_gb300/cexpr.py) and the lowering of user
pass methods (time-dependent kickers) on the CPU.

C semantics are checked against C itself: every expression is compiled by gcc
(strict IEEE, no contraction) into a function of the same variables, and the
program's value must equal the C function's bit for bit."""
import ctypes
import os
import subprocess
import tempfile

import numpy as np
import pytest

import helpers as H

EXPRS = [
    '(turn == 20) ? 0.05 : 0.',
    '((turn >= parameters[0]) && (turn < parameters[0] + 1.5) )? 0.05 * '
    'sin(3.1415 * ((float)turn - parameters[0]) / 1.5): 0.',
    '1/2 + turn/3 + turn%4',
    '7/turn',
    '(float)x * (float)y',           # float * float: rounded to float
    '(float)x + 1',                  # int converted to float, float sum
    '3.1415f * turn',                # float literal and int -> float
    '(float)turn - parameters[0]',   # float - double: double
    '(int)(x * 1e4) / 3',            # truncation, then int division
    '-x * oodppo + !turn',
    'x > 0 ? (float)px : py',        # ?: arithmetic conversion (float, double)
    'turn > 3 ? 2 : 0.5f',           # ?: int and float branches
    'fabs(x) < 0.02 && fabs(y) < 0.005 || turn < 2',
    'sqrt(x * x + y * y) - exp(-turn / 10.) + log(1. + dp)',
    'cos(x) * tan(y / 2)',
    'parameters[1] * parameters[0] / (1 + turn)',
]

@pytest.fixture(scope='module')
def cfuncs():
    src = ['#include <math.h>']
    for i, e in enumerate(EXPRS):
        src.append(f'double f{i}(int turn, double x, double px, double y, double py, double z, '
                   f'double dp, double oodppo, const double *parameters) '
                   f'{{ return (double)({e}); }}')
    d = tempfile.mkdtemp()
    c, so = os.path.join(d, 'e.c'), os.path.join(d, 'e.so')
    with open(c, 'w') as f:
        f.write('\n'.join(src) + '\n')
    subprocess.run(['gcc', '-O0', '-ffp-contract=off', '-fno-fast-math', '-shared', '-fPIC',
                    '-o', so, c, '-lm'], check=True)
    lib = ctypes.CDLL(so)
    fns = []
    for i in range(len(EXPRS)):
        f = getattr(lib, f'f{i}')
        f.restype = ctypes.c_double
        f.argtypes = [ctypes.c_int] + [ctypes.c_double] * 7 + [ctypes.POINTER(ctypes.c_double)]
        fns.append(f)
    return fns


def test_expressions_match_c(cfuncs):
    from ufo_gb300 import cexpr as X
    rng = np.random.default_rng(3)
    for i, e in enumerate(EXPRS):
        code, _, _ = X.compile_expr(e, allow_params=True)
        for _ in range(40):
            turn = int(rng.integers(1, 40))
            x, px, y, py, z, dp = rng.normal(size=6) * [1e-2, 1e-3, 1e-2, 1e-3, 0, 1e-3]
            o = 1.0 / (1.0 + dp)
            params = np.array([5.0 + rng.random(), rng.normal()])
            want = cfuncs[i](turn, x, px, y, py, z, dp, o,
                             params.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
            got = X.evaluate(code, (x, px, y, py, z, dp, o, turn), params)
            assert np.float64(got).tobytes() == np.float64(want).tobytes() or \
                (np.isnan(got) and np.isnan(want)), (e, turn, got, want)


def test_howto_kickers_lower_to_dynamic_kicks():
    """The HOWTO's kickers compile to one dynamic kick each; the trigger time
    bound as a parameter becomes a per-seed literal of the program."""
    import kickers
    import ufo_gb300 as u
    from ufo_gb300 import compiler as C, cexpr as X
    line = u.Line('L', [kickers.NLKGate('NLK', knl=[0., 5e-2]), u.Drift('D', length=1.0)])
    p = C.compile_line(line, u.FIVED | u.KICK, ['x', 'px'], [-1])
    assert [int(r[0]) for r in p.ops] == [C.OP_DYNKICK, C.OP_DRIFT, C.OP_OBSERVE]
    nn, ns, words = (int(v) for v in p.ops[0, 3:6])
    assert (nn, ns) == (2, 0) and words == p.ops[1, 2]
    # coefficient 0 is the literal 0., coefficient 1 the gate program
    assert list(p.table[0, :3]) == [1.0, X.PUSH, 0.0]
    line = u.Line('L', [kickers.NLKPulse('NLK', knl=[0., 5e-2], tau=1.5)])
    rows = np.array([[0., 0., 5.0], [0., 0., 5.25]])
    p = C.compile_line(line, u.FIVED | u.KICK, ['x', 'px', ('NLK', 't0')], [-1], rows)
    t0 = p.table[:, 3:int(p.ops[0, 5])]
    assert np.any(t0[0] == 5.0) and np.any(t0[1] == 5.25)  # the parameter, per seed
    assert X.SIN in set(p.table[0, 4:int(p.ops[0, 5]):2].astype(int))


def test_static_user_values_fold_to_plain_kicks():
    """C text that reads neither the turn nor the particle is folded per seed
    (the reference's compiler computes it once): the element stays a plain
    kick."""
    import ufo_gb300 as u
    from ufo_gb300 import compiler as C

    class Scaled(u.Multipole):
        def method(self, k1=None, **kwargs):
            return super().method(k1=f'({k1 or self.knl[1]} * 2.0)', **kwargs)
    p = C.compile_line(u.Line('L', [Scaled('S', knl=[0., 0.25])]), u.KICK, [], [-1])
    assert int(p.ops[0, 0]) == C.OP_KICK and p.table[0, 0] == 0.5


@pytest.mark.parametrize('text,err', [
    ('((turn == 2) ? px : 0.)', 'px and py'),
    ('turn == 2 ? 0.1 : 0.', 'parentheses'),
    ('(foo(turn))', 'unknown name'),
    ('(parameters[7])', 'outside the parameter list'),
])
def test_rejected_user_values(text, err):
    import ufo_gb300 as u
    from ufo_gb300 import compiler as C

    class K(u.Multipole):
        def method(self, **kwargs):
            return super().method(k1=text, **kwargs)
    with pytest.raises((NotImplementedError, IndexError), match=err):
        C.compile_line(u.Line('L', [K('K', knl=[0., 1.])]), u.KICK, [], [-1])


def test_dynamic_values_outside_thin_multipoles_rejected():
    import ufo_gb300 as u
    from ufo_gb300 import compiler as C

    class Q(u.Quadrupole):
        def method(self, **kwargs):
            return super().method(k1='((turn < 5) ? 1.0 : 1.1)', **kwargs)
    with pytest.raises(NotImplementedError, match='thin multipole'):
        C.compile_line(u.Line('L', [Q('Q', length=0.3, k1=1.0)]), u.KICK, [], [-1])


def test_oracle_reproduces_reference_kickers():
    """The oracle's evaluation of the kickers' C text against the reference's
    tracks (the same check the generic oracle test makes, named here)."""
    for name in ('nlk_gate', 'nlk_pulse'):
        c = H.case(name)
        out = H.oracle_case(c)
        assert np.array_equal(out['tracks'], H.arr(name, 'out/tracks'), equal_nan=True)


def _random_expr(rng, depth):
    """A random expression of the grammar, free of C undefined behaviour:
    integer arithmetic only between small leaves, integer division and % only
    by non-zero literals, (int) casts only of bounded values.  Returns
    (text, type, is_leaf)."""
    if depth == 0 or rng.random() < 0.25:
        k = rng.integers(7)
        if k == 0:
            return str(int(rng.integers(1, 10))), 'i', True
        if k == 1:
            return repr(float(rng.normal())), 'd', True
        if k == 2:
            return f'{rng.random():.6f}f', 'f', True
        if k == 3:
            return 'turn', 'i', True
        if k == 4:
            return f'parameters[{int(rng.integers(2))}]', 'd', True
        return str(rng.choice(['x', 'px', 'y', 'dp', 'oodppo'])), 'd', True
    k = rng.integers(9)
    a, ta, la = _random_expr(rng, depth - 1)
    if k == 0:
        op = str(rng.choice(['-', '!']))
        return f'{op}({a})', ('i' if op == '!' else ta), False
    if k == 1:
        c = str(rng.choice(['float', 'double']))
        return f'({c})({a})', c[0], False
    if k == 2:  # bounded integer cast
        return f'(int)(fabs({a}) < 1e6 ? ({a}) : 0.)', 'i', False
    if k == 3:
        f = str(rng.choice(['fabs', 'sin', 'cos', 'exp', 'sqrt', 'log']))
        arg = f'fabs({a})' if f in ('sqrt', 'log') else a
        return f'{f}({arg})', 'd', False
    b, tb, lb = _random_expr(rng, depth - 1)
    if k == 4:
        c, _, _ = _random_expr(rng, depth - 1)
        return f'(({c}) ? ({a}) : ({b}))', max(ta, tb, key='ifd'.index), False
    if k == 5:
        op = str(rng.choice(['<', '<=', '>', '>=', '==', '!=', '&&', '||']))
        return f'(({a}) {op} ({b}))', 'i', False
    op = str(rng.choice(['+', '-', '*', '/']))
    if ta == 'i' and tb == 'i':
        if op == '/' or not (la and lb):
            # integer division by a non-zero literal, or mix in a double
            return (f'(({a}) / {int(rng.integers(1, 10))})' if op == '/' and la
                    else f'(({a}) {op} (({b}) * 1.5))'), 'd' if op != '/' or not la else 'i', False
        return f'({a} {op} {b})', 'i', False
    if op == '%':
        op = '+'
    t = max(ta, tb, key='ifd'.index)
    return f'(({a}) {op} ({b}))', t, False


def test_random_expressions_match_c():
    """400 random expressions (seeded), each compiled by gcc and by the
    expression compiler, evaluated at 8 points: bit-identical values."""
    from ufo_gb300 import cexpr as X
    rng = np.random.default_rng(11)
    exprs = [_random_expr(rng, 4)[0] for _ in range(400)]
    src = ['#include <math.h>']
    for i, e in enumerate(exprs):
        src.append(f'double g{i}(int turn, double x, double px, double y, double py, double z, '
                   f'double dp, double oodppo, const double *parameters) '
                   f'{{ return (double)({e}); }}')
    d = tempfile.mkdtemp()
    c, so = os.path.join(d, 'r.c'), os.path.join(d, 'r.so')
    with open(c, 'w') as f:
        f.write('\n'.join(src) + '\n')
    subprocess.run(['gcc', '-O0', '-ffp-contract=off', '-fno-fast-math', '-w', '-shared', '-fPIC',
                    '-o', so, c, '-lm'], check=True)
    lib = ctypes.CDLL(so)
    pts = []
    for _ in range(8):
        v = rng.normal(size=6) * [1e-2, 1e-3, 1e-2, 1e-3, 0, 1e-3]
        pts.append((int(rng.integers(1, 40)), *v, 1.0 / (1.0 + v[5]),
                    np.array([5.0 + rng.random(), rng.normal()])))
    for i, e in enumerate(exprs):
        fn = getattr(lib, f'g{i}')
        fn.restype = ctypes.c_double
        fn.argtypes = [ctypes.c_int] + [ctypes.c_double] * 7 + [ctypes.POINTER(ctypes.c_double)]
        code, _, _ = X.compile_expr(e, allow_params=True)
        for turn, x, px, y, py, z, dp, o, prm in pts:
            want = fn(turn, x, px, y, py, z, dp, o,
                      prm.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
            got = X.evaluate(code, (x, px, y, py, z, dp, o, turn), prm)
            assert np.float64(got).tobytes() == np.float64(want).tobytes() or \
                (np.isnan(got) and np.isnan(want)), (e, turn, got, want)


def test_turn_outside_tracking_kernels_rejected():
    """The reference's closed-orbit and optics kernels declare no ``turn``:
    element text that reads it cannot build there, and is refused here."""
    import kickers
    import ufo_gb300 as u
    from ufo_gb300 import compiler as C, drivers
    gate = C.compile_line(u.Line('L', [kickers.NLKGate('N', knl=[0., 1e-3])]), u.KICK, [], [-1])
    window = C.compile_line(u.Line('L', [u.Aperture('A', window='turn < 5 || x*x < 1e-4')]),
                            u.KICK, [], [-1])
    circle = C.compile_line(u.Line('L', [u.Aperture('A', window='x*x + y*y < 1e-4')]),
                            u.KICK, [], [-1])
    assert C.reads_turn(gate) and C.reads_turn(window) and not C.reads_turn(circle)
    with pytest.raises(RuntimeError, match='turn'):
        drivers._no_turn(gate, 'closed-orbit')
    drivers._no_turn(circle, 'optics')


def test_coordinate_columns_are_not_lattice_values():
    import ufo_gb300 as u
    from ufo_gb300 import compiler as C

    class K(u.Multipole):
        def method(self, **kwargs):
            return super().method(k1='((turn > 2) ? parameters[0] : 0.)', **kwargs)
    with pytest.raises(NotImplementedError, match='particle coordinate'):
        C.compile_line(u.Line('L', [K('K', knl=[0., 1.])]), u.KICK, ['x', ('K', 'dx')], [-1])


@pytest.mark.gpu
def test_malformed_dynamic_kick_tables_rejected_before_launch():
    """ufo_prog_create and ufo_prog_set_table check every dynamic-kick program
    on the host: a length past the op's table words or an op without operands
    is an error, and no kernel runs."""
    import kickers
    import ufo_gb300 as u
    from ufo_gb300 import capi, cexpr, compiler as C
    line = u.Line('L', [kickers.NLKGate('N', knl=[0., 1e-3]), u.Drift('D', length=1.0)])
    prog = C.compile_line(line, u.KICK, [], [-1])
    ctx = u.context(0)
    good = capi.DeviceProgram(ctx, prog)  # well formed
    # table: [1, PUSH, 0.0, 6, VAR, 7, PUSH, 20, EQ, 0, ...]
    for pos, value in ((0, 99.0), (4, float(cexpr.NEG))):
        bad = prog.table.copy()
        bad[0, pos] = value
        with pytest.raises(RuntimeError, match='dynamic-kick'):
            good.set_table(bad)  # a replacement table is checked the same way
        keep = prog.table[0, pos]
        prog.table[0, pos] = value
        with pytest.raises(RuntimeError, match='dynamic-kick'):
            capi.DeviceProgram(ctx, prog)
        prog.table[0, pos] = keep
    good.set_table(prog.table)
