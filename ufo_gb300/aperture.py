"""Aperture windows: the reference's C keep-condition, parsed to a stack program.

The reference pastes the window text into ``if ({window} == 0) x = NAN;``
(ufo/elements.py:517-518) without parentheses around ``window``, so the C
operator precedence of the concatenated text decides what is tested (for
``'a && b'`` the test is ``a && (b == 0)``).  This module parses exactly that
concatenated text with C precedence and C's int/double typing and emits a
postfix program that the kernels evaluate per particle.  Supported: number
literals, the variables ``x px y py z dp oodppo turn``, unary ``- + !``,
``* / %`` (``%`` on ints only), ``+ -``, ``< <= > >=``, ``== !=``, ``&& ||``,
``?:`` and the calls ``fabs`` and ``sqrt``.  Anything else raises
``NotImplementedError``: the reference accepted arbitrary OpenCL C there, which
a data-driven kernel cannot run.
"""
import re

# stack opcodes (shared with the CUDA kernels and the C oracle)
PUSH, VAR, NEG, NOT, ADD, SUB, MUL, DIV, IDIV, IMOD, LT, LE, GT, GE, EQ, NE, AND, OR, \
    FABS, SQRT, SEL = range(1, 22)
VARS = {'x': 0, 'px': 1, 'y': 2, 'py': 3, 'z': 4, 'dp': 5, 'oodppo': 6, 'turn': 7}
INT_VARS = {'turn'}
MAX_STACK = 16

_TOK = re.compile(r'\s*(?:(?P<num>(?:\d+\.\d*|\.\d+|\d+)(?:[eE][+-]?\d+)?[fF]?)'
                  r'|(?P<id>[A-Za-z_]\w*)|(?P<op>&&|\|\||==|!=|<=|>=|[-+*/%<>!()?:]))')


def _tokenize(text):
    pos = 0
    out = []
    text = text.rstrip()
    while pos < len(text):
        m = _TOK.match(text, pos)
        if not m or m.end() == pos:
            raise NotImplementedError(f'aperture window: cannot parse {text[pos:]!r}')
        pos = m.end()
        if m.group('num') is not None:
            s = m.group('num').rstrip('fF')
            is_int = not any(c in s for c in '.eE')
            out.append(('num', int(s) if is_int else float(s), is_int))
        elif m.group('id') is not None:
            out.append(('id', m.group('id'), None))
        else:
            out.append(('op', m.group('op'), None))
    return out


class _Parser:
    # binary operators by precedence level, lowest first
    LEVELS = [('||',), ('&&',), ('==', '!='), ('<', '<=', '>', '>='), ('+', '-'), ('*', '/', '%')]

    def __init__(self, toks):
        self.t = toks
        self.i = 0
        self.code = []  # list of (opcode, value)

    def peek(self):
        return self.t[self.i] if self.i < len(self.t) else (None, None, None)

    def take(self, op=None):
        tok = self.peek()
        if op is not None and (tok[0] != 'op' or tok[1] != op):
            raise NotImplementedError(f'aperture window: expected {op!r}')
        self.i += 1
        return tok

    def parse(self):
        is_int = self.ternary()
        if self.i != len(self.t):
            raise NotImplementedError('aperture window: trailing tokens')
        return is_int

    def ternary(self):
        is_int = self.binary(0)
        tok = self.peek()
        if tok[0] == 'op' and tok[1] == '?':
            self.take('?')
            a_int = self.ternary()
            self.take(':')
            b_int = self.ternary()
            self.code.append((SEL, 0.0))
            return a_int and b_int
        return is_int

    def binary(self, level):
        if level == len(self.LEVELS):
            return self.unary()
        left = self.binary(level + 1)
        while True:
            tok = self.peek()
            if tok[0] != 'op' or tok[1] not in self.LEVELS[level]:
                return left
            op = self.take()[1]
            right = self.binary(level + 1)
            both_int = left and right
            if op in ('&&', '||', '==', '!=', '<', '<=', '>', '>='):
                code = {'&&': AND, '||': OR, '==': EQ, '!=': NE, '<': LT, '<=': LE,
                        '>': GT, '>=': GE}[op]
                left = True
            elif op == '/':
                code = IDIV if both_int else DIV
                left = both_int
            elif op == '%':
                if not both_int:
                    raise NotImplementedError('aperture window: % on doubles')
                code = IMOD
                left = True
            else:
                code = {'+': ADD, '-': SUB, '*': MUL}[op]
                left = both_int
            self.code.append((code, 0.0))

    def unary(self):
        tok = self.peek()
        if tok[0] == 'op' and tok[1] in ('-', '+', '!'):
            op = self.take()[1]
            is_int = self.unary()
            if op == '-':
                self.code.append((NEG, 0.0))
            elif op == '!':
                self.code.append((NOT, 0.0))
                is_int = True
            return is_int
        return self.primary()

    def primary(self):
        tok = self.take()
        if tok[0] == 'num':
            self.code.append((PUSH, float(tok[1])))
            return tok[2]
        if tok[0] == 'op' and tok[1] == '(':
            is_int = self.ternary()
            self.take(')')
            return is_int
        if tok[0] == 'id':
            name = tok[1]
            if name in ('fabs', 'sqrt'):
                self.take('(')
                self.ternary()
                self.take(')')
                self.code.append((FABS if name == 'fabs' else SQRT, 0.0))
                return False
            if name == 'NAN':
                self.code.append((PUSH, float('nan')))
                return False
            if name in VARS:
                self.code.append((VAR, float(VARS[name])))
                return name in INT_VARS
            raise NotImplementedError(f'aperture window: unknown name {name!r}')
        raise NotImplementedError(f'aperture window: unexpected {tok[1]!r}')


def _depth(code):
    d = m = 0
    for op, _ in code:
        if op in (PUSH, VAR):
            d += 1
        elif op in (NEG, NOT, FABS, SQRT):
            pass
        elif op == SEL:
            d -= 2
        else:
            d -= 1
        m = max(m, d)
    return m


def compile_window(window):
    """Postfix program for the reference's loss test ``{window} == 0``.
    Returns a list of (opcode, value); the particle is lost when it
    evaluates to non-zero."""
    text = f'{window} == 0'
    p = _Parser(_tokenize(text))
    p.parse()
    if _depth(p.code) > MAX_STACK:
        raise NotImplementedError('aperture window: expression too deep')
    return p.code


def evaluate(code, x=0., px=0., y=0., py=0., z=0., dp=0., oodppo=1., turn=0):
    """Reference evaluator of a compiled window (used by tests)."""
    import math
    vals = [x, px, y, py, z, dp, oodppo, float(turn)]
    st = []
    for op, v in code:
        if op == PUSH:
            st.append(v)
        elif op == VAR:
            st.append(vals[int(v)])
        elif op == NEG:
            st.append(-st.pop())
        elif op == NOT:
            st.append(1.0 if st.pop() == 0 else 0.0)
        elif op == FABS:
            st.append(abs(st.pop()))
        elif op == SQRT:
            a = st.pop()
            st.append(math.sqrt(a) if a >= 0 else float('nan'))
        elif op == SEL:
            b = st.pop(); a = st.pop(); c = st.pop()
            st.append(a if c != 0 else b)
        else:
            b = st.pop(); a = st.pop()
            if op == ADD: r = a + b
            elif op == SUB: r = a - b
            elif op == MUL: r = a * b
            elif op == DIV:
                r = a / b if b != 0 else (math.copysign(math.inf, a * b) if a != 0 and a == a else math.nan)
            elif op == IDIV: r = float(int(a / b)) if b != 0 else math.nan
            elif op == IMOD: r = float(math.fmod(a, b)) if b != 0 else math.nan
            elif op == LT: r = float(a < b)
            elif op == LE: r = float(a <= b)
            elif op == GT: r = float(a > b)
            elif op == GE: r = float(a >= b)
            elif op == EQ: r = float(a == b)
            elif op == NE: r = float(a != b)
            elif op == AND: r = float(a != 0 and b != 0)
            else: r = float(a != 0 or b != 0)
            st.append(r)
    return st[-1] != 0
