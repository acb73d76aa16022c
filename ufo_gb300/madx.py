"""Loader for the MAD-X dialect the reference reads (ufo/mad.py:14-147).

Statements are ``LABEL: TYPE, KEY=VALUE, ...;`` and ``LABEL: LINE=(a, b, ...);``.
Values are numbers, ``{a, b, ...}`` vectors or double-quoted strings.  The
element table (which MAD-X keys each type accepts) is the reference's
(ufo/mad.py:103-113); unknown statement types are skipped with a warning and
unknown keys raise, as there.  This loader also accepts exponents in numbers
(``1e-4``), which the reference's tokenizer does not.
"""
import re
import warnings

_NUM = r'[+-]?(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?'
_TOKEN = re.compile(
    r'(?P<VEC>\{[^}]*\})|(?P<STR>"[^"]*")|(?P<NUM>' + _NUM + r')'
    r'|(?P<DEF>:=)|(?P<COLON>:)|(?P<OPEN>\()|(?P<CLOSE>\))|(?P<COMMA>,)|(?P<ASSIGN>=)'
    r'|(?P<END>;)|(?P<ID>[A-Za-z_][A-Za-z0-9_.]*)|(?P<WS>\s+)|(?P<BAD>.)')


def _tokens(text):
    for m in _TOKEN.finditer(text):
        kind = m.lastgroup
        val = m.group()
        if kind == 'WS':
            continue
        if kind == 'BAD':
            raise RuntimeError(f'{val!r} unexpected')
        if kind == 'NUM':
            val = float(val)
        elif kind == 'VEC':
            inner = val[1:-1].strip()
            val = [float(v) for v in inner.split(',') if v.strip()] if inner else []
        elif kind == 'STR':
            val = val[1:-1]
        if kind == 'DEF':
            kind = 'ASSIGN'
        yield kind, val


def _elements():
    import ufo_gb300 as u
    return {
        'MARKER': (u.Marker, {}),
        'DRIFT': (u.Drift, {'L': 'length'}),
        'QUADRUPOLE': (u.Quadrupole, {'L': 'length', 'K1': 'k1'}),
        'SBEND': (u.Sbend, {'L': 'length', 'ANGLE': 'angle', 'K1': 'k1', 'E1': 'e1',
                            'E2': 'e2', 'HGAP': 'hgap', 'FINT': 'fint'}),
        'RBEND': (u.Rbend, {'L': 'length', 'ANGLE': 'angle', 'K1': 'k1', 'E1': 'e1',
                            'E2': 'e2'}),
        'SEXTUPOLE': (u.Sextupole, {'L': 'length', 'K2': 'k2', 'K2S': 'k2s'}),
        'OCTUPOLE': (u.Octupole, {'L': 'length', 'K3': 'k3', 'K3S': 'k3s'}),
        'MULTIPOLE': (u.Multipole, {'KNL': 'knl', 'KSL': 'ksl'}),
        'APERTURE': (u.Aperture, {'WINDOW': 'window'}),
    }


def loads(text):
    """Parse MAD-X dialect text into ``{label: element or Line}``."""
    from .lattice import Line
    table = _elements()
    toks = list(_tokens(text))
    out = {}
    i = 0

    def expect(kind):
        nonlocal i
        if i >= len(toks) or toks[i][0] != kind:
            got = toks[i][1] if i < len(toks) else 'end of file'
            raise RuntimeError(f'{got!r} unexpected')
        i += 1
        return toks[i - 1][1]

    while i < len(toks):
        label = expect('ID')
        expect('COLON')
        kind = expect('ID').upper()
        if kind == 'LINE':
            expect('ASSIGN')
            expect('OPEN')
            line = Line(label)
            while True:
                name = expect('ID')
                if name not in out:
                    raise RuntimeError(f'{name!r} used before definition')
                line.append(out[name])
                if toks[i][0] == 'CLOSE':
                    i += 1
                    break
                expect('COMMA')
            expect('END')
            out[label] = line
        elif kind in table:
            cls, keys = table[kind]
            kwargs = {}
            while toks[i][0] != 'END':
                expect('COMMA')
                key = expect('ID').upper()
                expect('ASSIGN')
                if i >= len(toks) or toks[i][0] not in ('NUM', 'VEC', 'STR'):
                    raise RuntimeError(f'{toks[i][1]!r} unexpected')
                val = toks[i][1]
                i += 1
                if key not in keys:
                    raise TypeError(f'{kind} does not accept {key}')
                kwargs[keys[key]] = val
            expect('END')
            out[label] = cls(label, **kwargs)
        else:
            warnings.warn(f"unknown statement '{kind}'")
            while toks[i][0] != 'END':
                i += 1
            i += 1
    return out


def load(path):
    """Parse a MAD-X dialect file (ufo/mad.py:101-147)."""
    with open(path) as f:
        return loads(f.read())
