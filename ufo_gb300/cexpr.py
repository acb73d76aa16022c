"""Restricted C expressions compiled to postfix stack programs.

The reference builds its kernels from C text: aperture windows are pasted into
``if ({window} == 0) x = NAN;`` (ufo/elements.py:517-518) and a user element's
``method()`` may hand any C expression to its base class as a strength
(the time-dependent kicker of HOWTO.md:84-200 passes
``(turn == 20) ? k1 : 0.``).  This module parses such text with C's operator
precedence and C's typing, and emits a program that the kernels evaluate per
particle (ops.cuh: ``eval_prog``; the Python evaluator below follows the same
rules).

Grammar: number literals (``f`` suffix: float), the variables
``x px y py z dp oodppo`` (double) and ``turn`` (int), ``parameters[i]`` (the
i-th column of the parameter list, resolved per seed by the compiler),
``NAN``, unary ``- + !``, casts ``(float) (double) (ufloat) (int)``, ``* / %``,
``+ -``, ``< <= > >=``, ``== !=``, ``&& ||``, ``?:`` and the calls ``fabs sqrt
sin cos tan exp log``.

Typing follows C: operands of a binary operator convert to the wider of int,
float and double; int/int divides with truncation and ``%`` takes ints; integer
results are never -0 (``0 - a`` for negation, ``+ 0`` after products,
truncation and remainders); a float
result is rounded to float32 (emitted as an explicit F32 op, so the FP64
evaluators reproduce float arithmetic exactly: a double result of two floats
rounds once to the correctly rounded float).  Calls take and return double
(the C library functions, which the reference's kernels call through the C
compiler here).  Anything else raises ``NotImplementedError``: the reference
accepted arbitrary OpenCL C, which a data-driven kernel cannot run.
"""
import math
import re

import numpy as np

# stack opcodes (shared with the CUDA kernels and the C oracle)
PUSH, VAR, NEG, NOT, ADD, SUB, MUL, DIV, IDIV, IMOD, LT, LE, GT, GE, EQ, NE, AND, OR, \
    FABS, SQRT, SEL, SIN, COS, TAN, EXP, LOG, F32, TRUNC, PARAM = range(1, 30)
UNARY = (NEG, NOT, FABS, SQRT, SIN, COS, TAN, EXP, LOG, F32, TRUNC)
CALLS = {'fabs': FABS, 'sqrt': SQRT, 'sin': SIN, 'cos': COS, 'tan': TAN, 'exp': EXP,
         'log': LOG}
VARS = {'x': 0, 'px': 1, 'y': 2, 'py': 3, 'z': 4, 'dp': 5, 'oodppo': 6, 'turn': 7}
INT_VARS = {'turn'}
CASTS = {'float': 'f', 'double': 'd', 'ufloat': 'd', 'int': 'i'}
_RANK = {'i': 0, 'f': 1, 'd': 2}

_TOK = re.compile(r'\s*(?:(?P<num>(?:\d+\.\d*|\.\d+|\d+)(?:[eE][+-]?\d+)?[fF]?)'
                  r'|(?P<id>[A-Za-z_]\w*)|(?P<op>&&|\|\||==|!=|<=|>=|[-+*/%<>!()?:\[\]]))')


def f32(v):
    """Round a double to the nearest float32 (as a double)."""
    return float(np.float32(v))


def tokenize(text, what='expression'):
    pos = 0
    out = []
    text = str(text).rstrip()
    while pos < len(text):
        m = _TOK.match(text, pos)
        if not m or m.end() == pos:
            raise NotImplementedError(f'{what}: cannot parse {text[pos:]!r}')
        pos = m.end()
        if m.group('num') is not None:
            raw = m.group('num')
            s = raw.rstrip('fF')
            if s != raw:
                out.append(('num', f32(float(s)), 'f'))
            elif any(c in s for c in '.eE'):
                out.append(('num', float(s), 'd'))
            else:
                out.append(('num', int(s), 'i'))
        elif m.group('id') is not None:
            out.append(('id', m.group('id'), None))
        else:
            out.append(('op', m.group('op'), None))
    return out


class Parser:
    """Recursive-descent parser; ``code`` is a list of (opcode, value)."""
    # binary operators by precedence level, lowest first
    LEVELS = [('||',), ('&&',), ('==', '!='), ('<', '<=', '>', '>='), ('+', '-'), ('*', '/', '%')]
    MUL_LEVEL = 5

    def __init__(self, toks, what='expression', allow_params=False):
        self.t = toks
        self.i = 0
        self.code = []
        self.what = what
        self.allow_params = allow_params

    def peek(self, k=0):
        j = self.i + k
        return self.t[j] if j < len(self.t) else (None, None, None)

    def take(self, op=None):
        tok = self.peek()
        if op is not None and (tok[0] != 'op' or tok[1] != op):
            raise NotImplementedError(f'{self.what}: expected {op!r}')
        self.i += 1
        return tok

    def fail(self, msg):
        raise NotImplementedError(f'{self.what}: {msg}')

    def parse(self):
        t = self.ternary()
        if self.i != len(self.t):
            self.fail('trailing tokens')
        return t

    def _convert(self, pos, t, to):
        """Convert the operand whose code ends at ``pos`` from type t to
        ``to`` (only int -> float rounds)."""
        if t == 'i' and to == 'f':
            self.code.insert(pos, (F32, 0.0))
            return 1
        return 0

    def ternary(self):
        t = self.binary(0)
        tok = self.peek()
        if tok[0] == 'op' and tok[1] == '?':
            self.take('?')
            ta = self.ternary()
            mark = len(self.code)  # end of the first branch
            self.take(':')
            tb = self.ternary()
            to = max(ta, tb, key=_RANK.get)
            self._convert(mark, ta, to)
            self._convert(len(self.code), tb, to)
            self.code.append((SEL, 0.0))
            return to
        return t

    def binary(self, level):
        if level == len(self.LEVELS):
            return self.unary()
        left = self.binary(level + 1)
        while True:
            tok = self.peek()
            if tok[0] != 'op' or tok[1] not in self.LEVELS[level]:
                return left
            op = self.take()[1]
            mark = len(self.code)  # end of the left operand
            right = self.binary(level + 1)
            if op in ('&&', '||'):
                self.code.append((AND if op == '&&' else OR, 0.0))
                left = 'i'
                continue
            if op == '%':
                if left != 'i' or right != 'i':
                    self.fail('% on floating-point operands')
                self.code.append((IMOD, 0.0))
                left = 'i'
                continue
            to = max(left, right, key=_RANK.get)
            mark += self._convert(mark, left, to)
            self._convert(len(self.code), right, to)
            if op in ('==', '!=', '<', '<=', '>', '>='):
                self.code.append(({'==': EQ, '!=': NE, '<': LT, '<=': LE, '>': GT,
                                   '>=': GE}[op], 0.0))
                left = 'i'
                continue
            if op == '/':
                self.code.append((IDIV if to == 'i' else DIV, 0.0))
            else:
                self.code.append(({'+': ADD, '-': SUB, '*': MUL}[op], 0.0))
                if op == '*' and to == 'i':  # 0 * -n is 0, not -0
                    self.code += [(PUSH, 0.0), (ADD, 0.0)]
            if to == 'f':
                self.code.append((F32, 0.0))
            left = to

    def unary(self):
        tok = self.peek()
        if tok[0] == 'op' and tok[1] in ('-', '+', '!'):
            op = self.take()[1]
            start = len(self.code)
            t = self.unary()
            if op == '-' and t == 'i':  # ints have no -0: 0 - a
                self.code.insert(start, (PUSH, 0.0))
                self.code.append((SUB, 0.0))
            elif op == '-':
                self.code.append((NEG, 0.0))
            elif op == '!':
                self.code.append((NOT, 0.0))
                t = 'i'
            return t
        # cast: '(' type ')' unary
        if (tok[0] == 'op' and tok[1] == '(' and self.peek(1)[0] == 'id' and
                self.peek(1)[1] in CASTS and self.peek(2)[:2] == ('op', ')')):
            self.take('(')
            to = CASTS[self.take()[1]]
            self.take(')')
            t = self.unary()
            if to == 'i' and t != 'i':
                self.code.append((TRUNC, 0.0))
            elif to == 'f' and t != 'f':
                self.code.append((F32, 0.0))
            return to
        return self.primary()

    def primary(self):
        tok = self.take()
        if tok[0] == 'num':
            self.code.append((PUSH, float(tok[1])))
            return tok[2]
        if tok[0] == 'op' and tok[1] == '(':
            t = self.ternary()
            self.take(')')
            return t
        if tok[0] == 'id':
            name = tok[1]
            if name in CALLS:
                self.take('(')
                self.ternary()  # any arithmetic type converts to double exactly
                self.take(')')
                self.code.append((CALLS[name], 0.0))
                return 'd'
            if name == 'NAN':
                self.code.append((PUSH, float('nan')))
                return 'd'
            if name in VARS:
                self.code.append((VAR, float(VARS[name])))
                return 'i' if name in INT_VARS else 'd'
            if name == 'parameters' and self.allow_params:
                self.take('[')
                n = self.take()
                if n[0] != 'num' or n[2] != 'i':
                    self.fail('parameters[] needs an integer literal index')
                self.take(']')
                self.code.append((PARAM, float(n[1])))
                return 'd'
            self.fail(f'unknown name {name!r}')
        self.fail(f'unexpected {tok[1]!r}')


def top_level(toks):
    """Precedence level (index into Parser.LEVELS) of the loosest operator
    outside brackets: -1 for ?:, None when the text is a primary, unary, cast
    or call expression.  Text pasted next to a tighter operator keeps its
    meaning only when this is None or the multiplicative level."""
    depth = 0
    best = None
    prev = None
    for kind, v, _ in toks:
        if kind == 'op' and v in ('(', '['):
            depth += 1
        elif kind == 'op' and v in (')', ']'):
            depth -= 1
        elif kind == 'op' and depth == 0:
            binary = prev is not None and (prev[0] in ('num', 'id') or
                                           (prev[0] == 'op' and prev[1] in (')', ']')))
            if v in ('?', ':'):
                lvl = -1
            elif binary or v not in ('-', '+', '!'):
                lvl = next((i for i, ops in enumerate(Parser.LEVELS) if v in ops), None)
            else:
                lvl = None
            if lvl is not None and (best is None or lvl < best):
                best = lvl
        prev = (kind, v)
    return best


def compile_expr(text, what='expression', allow_params=False):
    """Program of one C expression.  Returns (code, type, top_level)."""
    toks = tokenize(text, what)
    p = Parser(toks, what, allow_params)
    t = p.parse()
    return p.code, t, top_level(toks)


def depth(code):
    d = m = 0
    for op, _ in code:
        if op in (PUSH, VAR, PARAM):
            d += 1
        elif op in UNARY:
            pass
        elif op == SEL:
            d -= 2
        else:
            d -= 1
        m = max(m, d)
    return m


def is_constant(code):
    """True when the program reads no particle variable (and no turn)."""
    return not any(op == VAR for op, _ in code)


def has_calls(code):
    return any(op in (FABS, SQRT, SIN, COS, TAN, EXP, LOG) for op, _ in code)


def _call(op, a, correctly_rounded):
    if op == FABS:
        return abs(a)
    if op == SQRT:
        return math.sqrt(a) if a >= 0 else (a if a != a else math.nan)
    name = {SIN: 'sin', COS: 'cos', TAN: 'tan', EXP: 'exp', LOG: 'log'}[op]
    if correctly_rounded:
        from . import crmath
        fn = getattr(crmath, name, None)
        if fn is not None:
            try:
                return fn(a)
            except (ValueError, OverflowError):
                pass
    # the C library (Python's math calls it); domain errors as C returns them
    try:
        return getattr(math, name)(a)
    except OverflowError:
        return math.inf
    except ValueError:
        return -math.inf if (name == 'log' and a == 0) else math.nan


def evaluate(code, vars=(0., 0., 0., 0., 0., 0., 1., 0), params=(), correctly_rounded=False):
    """Value of a program (C semantics in FP64).  ``vars`` = x, px, y, py, z,
    dp, oodppo, turn; ``params`` the parameter row.  ``correctly_rounded``
    evaluates calls correctly rounded (what a C compiler does when it folds a
    call on literal arguments); otherwise the C library's results."""
    vals = [float(v) for v in vars]
    st = []
    for op, v in code:
        if op == PUSH:
            st.append(v)
        elif op == VAR:
            st.append(vals[int(v)])
        elif op == PARAM:
            st.append(float(params[int(v)]))
        elif op == NEG:
            st.append(-st.pop())
        elif op == NOT:
            st.append(1.0 if st.pop() == 0 else 0.0)
        elif op == F32:
            st.append(f32(st.pop()))
        elif op == TRUNC:
            a = st.pop()
            st.append(float(math.trunc(a)) if math.isfinite(a) else a)
        elif op in (FABS, SQRT, SIN, COS, TAN, EXP, LOG):
            st.append(_call(op, st.pop(), correctly_rounded))
        elif op == SEL:
            b = st.pop()
            a = st.pop()
            c = st.pop()
            st.append(a if c != 0 else b)
        else:
            b = st.pop()
            a = st.pop()
            with np.errstate(all='ignore'):
                A, B = np.float64(a), np.float64(b)
                if op == ADD:
                    r = float(A + B)
                elif op == SUB:
                    r = float(A - B)
                elif op == MUL:
                    r = float(A * B)
                elif op == DIV:
                    r = float(A / B)
                elif op == IDIV:
                    r = float(math.trunc(a / b)) if b != 0 else math.nan
                elif op == IMOD:
                    r = float(math.fmod(a, b)) + 0.0 if b != 0 else math.nan
                elif op == LT:
                    r = float(a < b)
                elif op == LE:
                    r = float(a <= b)
                elif op == GT:
                    r = float(a > b)
                elif op == GE:
                    r = float(a >= b)
                elif op == EQ:
                    r = float(a == b)
                elif op == NE:
                    r = float(a != b)
                elif op == AND:
                    r = float(a != 0 and b != 0)
                else:
                    r = float(a != 0 or b != 0)
            st.append(r)
    return st[-1]
