"""ctypes wrapper and build recipe for the C parity oracle (ufo_oracle.c).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker.  The product path (ufo_gb300)
never imports this module.

The wrapper turns a flattened line plus the reference's parameter list into
per-seed element records.  Attribute resolution follows the reference's
element ``method()``s (``value or self.value``, ufo/elements.py) and
parameter binding follows ufo/lattice.py:107-110; transcendentals that the
reference's C compiler would fold (literal arguments) are precomputed here,
correctly rounded, exactly as GCC folds them.  Elements whose class has its
own ``method()`` (time-dependent kickers) are called as the reference's
Line.method calls them; the C text they return is parsed with ufo_gb300's
expression parser (cexpr) and evaluated here in C with the C library's math,
as the reference's compiled kernel evaluates it.
"""
import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, '_build')
SO = os.path.join(BUILD, 'libufo_oracle.so')
CFLAGS = ['-O2', '-std=gnu11', '-fPIC', '-shared', '-ffp-contract=off', '-fno-fast-math',
          '-fopenmp']

TYPES = {'marker': 0, 'drift': 1, 'multipole': 2, 'quadrupole': 3, 'sbend': 4, 'rbend': 5,
         'sextupole': 6, 'octupole': 7, 'wire': 8, 'aperture': 9}

OELEM = np.dtype([
    ('type', 'i4'), ('slices', 'i4'), ('nknl', 'i4'), ('nksl', 'i4'), ('ndkn', 'i4'),
    ('ndks', 'i4'), ('mp_off', 'i4'), ('nfrac', 'i4'), ('frac_off', 'i4'), ('pre_dump', 'i4'),
    ('ap_off', 'i4'), ('ap_len', 'i4'), ('fold_off', 'i4'), ('fold_achro', 'i4'),
    ('length', 'f8'), ('angle', 'f8'), ('k1', 'f8'), ('e1', 'f8'), ('e2', 'f8'),
    ('hgap', 'f8'), ('fint', 'f8'), ('dx', 'f8'), ('dy', 'f8'), ('k2', 'f8'), ('k2s', 'f8'),
    ('k3', 'f8'), ('k3s', 'f8'), ('wx', 'f8'), ('wy', 'f8'), ('wk', 'f8')])
assert OELEM.itemsize == 14 * 4 + 16 * 8

ACHROMATIC, KICK, FIVED = 64, 8, 2


def build(force=False):
    """Compile ufo_oracle.c (gcc, strict IEEE) into oracle/_build/."""
    src = os.path.join(HERE, 'ufo_oracle.c')
    if not force and os.path.exists(SO) and os.path.getmtime(SO) >= os.path.getmtime(src):
        return SO
    os.makedirs(BUILD, exist_ok=True)
    tmp = SO + f'.{os.getpid()}.tmp'
    subprocess.run(['gcc', *CFLAGS, '-o', tmp, src, '-lm'], check=True)
    os.replace(tmp, SO)
    return SO


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        f = _lib.oracle_track
        f.restype = ctypes.c_int
        P = ctypes.c_void_p
        f.argtypes = [P, ctypes.c_int, ctypes.c_int, P, P, P, P, ctypes.c_int, ctypes.c_int,
                      ctypes.c_double, P, P, ctypes.c_long, ctypes.c_int, ctypes.c_int,
                      ctypes.c_long, ctypes.c_int, P, P, P, ctypes.c_int]
    return _lib


# ---- correctly rounded folding (what GCC does to literal math calls) ----

def _fold(name, x, literal):
    import importlib
    cr = importlib.import_module('ufo_gb300.crmath')
    fn = getattr(cr, name) if literal else getattr(math, name)
    try:
        return fn(float(x))
    except (ValueError, OverflowError):
        return math.nan if name != 'cosh' else math.inf


def _sqrt(x):
    with np.errstate(all='ignore'):
        return float(np.sqrt(np.float64(x)))


def _div(a, b):
    with np.errstate(all='ignore'):
        return float(np.float64(a) / np.float64(b))


class Prepared:
    """Per-seed element records of a line, ready for oracle_track."""

    def __init__(self, line, flags, parameters, where, seed_values, dp=0.0):
        from ufo_gb300 import compiler, aperture
        flat = line.flatten() if hasattr(line, 'flatten') else list(line)
        parameters = list(parameters)
        self.flags = flags
        binds = compiler.element_bindings(flat, parameters)
        per, pre = compiler.fractures(len(flat), list(where))
        seed_values = np.zeros((1, max(len(parameters), 1))) if seed_values is None else \
            np.asarray(seed_values, np.float64)
        S = seed_values.shape[0]
        n = len(flat)
        self.n_elem = n
        self.n_seeds = S
        elems = np.zeros(S * n, dtype=OELEM)
        mp, fr, fold, ap = [], [], [], []
        for idx, f in enumerate(per):
            pass
        frac_off = []
        for idx in range(n):
            frac_off.append(len(fr))
            fr.extend(per[idx])
        ap_off = {}
        for idx, e in enumerate(flat):
            if e.kind == 'aperture':
                code = aperture.compile_window(e.window)
                ap_off[idx] = (len(ap), len(code))
                for opc, v in code:
                    ap += [float(opc), float(v)]
        achro = bool(flags & ACHROMATIC)
        # FIVED pastes dp as a literal (ufo/track.py:99-101), so oodppo is a
        # compile-time constant and the C compiler folds what it feeds: the
        # thick maps' and fringe edges' transcendentals, as in ACHROMATIC mode
        fived = bool(flags & FIVED)
        o_lit = float(np.float64(1.0) / (np.float64(dp) + np.float64(1.0)))
        fold_mode = achro or fived
        for s in range(S):
            for idx, e in enumerate(flat):
                r = elems[s * n + idx]
                prm = binds[idx]
                lit = {}
                if _user_method(e):
                    self._dynamic_multipole(r, e, prm, flags, per[idx], seed_values[s], ap)
                    r['nfrac'] = len(per[idx])
                    r['frac_off'] = frac_off[idx]
                    r['pre_dump'] = int(pre[idx])
                    continue

                def get(name, default=0.0):
                    if name in prm:
                        lit[name] = False
                        return float(seed_values[s, prm[name]])
                    lit[name] = True
                    v = getattr(e, name, default)
                    return v

                r['type'] = TYPES[e.kind]
                r['nfrac'] = len(per[idx])
                r['frac_off'] = frac_off[idx]
                r['pre_dump'] = int(pre[idx])
                r['mp_off'] = len(mp)
                r['fold_off'] = len(fold)
                if e.kind == 'aperture':
                    r['ap_off'], r['ap_len'] = ap_off[idx]
                    continue
                if e.kind == 'marker':
                    continue
                if e.kind == 'wire':
                    r['wx'], r['wy'], r['wk'] = get('x'), get('y'), get('k')
                    continue
                r['length'] = get('length')
                if e.kind == 'drift':
                    continue
                r['dx'], r['dy'] = get('dx'), get('dy')
                if e.kind == 'multipole':
                    knl = [float(v) for v in e.knl]
                    ksl = [float(v) for v in e.ksl]
                    for p, col in prm.items():
                        if p[:1] == 'k' and p[1:].isdigit():
                            knl[int(p[1:])] = float(seed_values[s, col])
                        if p[:1] == 'k' and p[-1:] == 's' and p[1:-1].isdigit():
                            ksl[int(p[1:-1])] = float(seed_values[s, col])
                    r['nknl'], r['nksl'] = len(knl), len(ksl)
                    mp += knl + ksl
                    continue
                r['slices'] = int(e.slices)
                dkn = [float(v) for v in e.dkn]
                dks = [float(v) for v in e.dks]
                for p, col in prm.items():
                    if p[:2] == 'dk' and p[2:].isdigit():
                        i = int(p[2:])
                        dkn += [0.0] * (i + 1 - len(dkn))
                        dkn[i] = float(seed_values[s, col])
                    if p[:2] == 'dk' and p[-1:] == 's' and p[2:-1].isdigit():
                        i = int(p[2:-1])
                        dks += [0.0] * (i + 1 - len(dks))
                        dks[i] = float(seed_values[s, col])
                r['ndkn'], r['ndks'] = len(dkn), len(dks)
                mp += dkn + dks
                for a in ('k1', 'k2', 'k3', 'k2s', 'k3s', 'angle', 'e1', 'e2', 'hgap', 'fint'):
                    if hasattr(e, a):
                        r[a] = get(a)
                # folded transcendentals (8 edge slots, then per-piece thick slots)
                pieces = []
                f0 = 0.0
                for f in list(per[idx]) + [1.0]:
                    pieces.append(f - f0)
                    f0 = f
                fl = [0.0] * 8
                if e.kind in ('sbend', 'rbend'):
                    L, A = float(r['length']), float(r['angle'])
                    fringe = float(r['hgap']) * float(r['fint'])
                    lit_edge = all(lit.get(a, True) for a in ('length', 'angle', 'hgap', 'fint'))
                    for j, en in enumerate(('e1', 'e2')):
                        ev = float(r[en])
                        elit = lit.get(en, True) and (e.kind == 'sbend' or lit.get('angle', True))
                        if e.kind == 'rbend':
                            ev = ev + (A * 0.5)
                        c, sn, t = _fold('cos', ev, elit), _fold('sin', ev, elit), \
                            _fold('tan', ev, elit)
                        tpsi = 0.0
                        if fold_mode:
                            curv = _div(A, L)
                            if not achro:  # angle / (L) * oodppo
                                curv = float(np.float64(curv) * np.float64(o_lit))
                            with np.errstate(all='ignore'):
                                psi = float(np.float64(ev) - np.float64(2 * curv) *
                                            np.float64(fringe) / np.float64(c) *
                                            (np.float64(1.) + np.float64(sn) * np.float64(sn)))
                            tpsi = _fold('tan', psi, elit and lit_edge)
                        fl[4 * j:4 * j + 4] = [c, sn, t, tpsi]
                thick = not (flags & KICK) and e.kind in ('quadrupole', 'sbend', 'rbend')
                if e.kind in ('sbend', 'rbend') and fold_mode:
                    r['fold_achro'] = 1  # the edges' tan(psi) come from the fold slots
                if thick and fold_mode:
                    r['fold_achro'] = 1
                    L = float(r['length'])
                    k1 = float(r['k1'])
                    tl = lit.get('length', True) and lit.get('k1', True)
                    o = 1.0 if achro else o_lit
                    for f in pieces:
                        with np.errstate(all='ignore'):
                            Lf = float(np.float64(L) * np.float64(f))
                        if e.kind == 'quadrupole':
                            with np.errstate(all='ignore'):
                                k2 = _sqrt(abs(k1) if achro else
                                           abs(float(np.float64(k1) * np.float64(o))))
                            k2l = Lf * k2
                            fl += [_fold('cos', k2l, tl), _fold('sin', k2l, tl),
                                   _fold('cosh', k2l, tl), _fold('sinh', k2l, tl)]
                        else:
                            A = float(r['angle'])
                            tlb = tl and lit.get('angle', True)
                            Af = float(np.float64(A) * np.float64(f))
                            curv = _div(Af, Lf)
                            kv = k1
                            if not achro:  # curvature and k carry oodppo
                                with np.errstate(all='ignore'):
                                    curv = float(np.float64(curv) * np.float64(o))
                                    kv = float(np.float64(k1) * np.float64(o))
                            k2 = _sqrt(abs(kv))
                            k2l = Lf * k2
                            v = [_fold('cos', k2l, tlb), _fold('sin', k2l, tlb),
                                 _fold('cosh', k2l, tlb), _fold('sinh', k2l, tlb)]
                            with np.errstate(all='ignore'):
                                cc = np.float64(curv) * np.float64(curv)
                                if not achro:  # k += curvature * curvature / oodppo
                                    cc = cc / np.float64(o)
                                kx = float(np.float64(kv) + cc)
                            k2 = _sqrt(abs(kx))
                            k2l = Lf * k2
                            v += [_fold('cos', k2l, tlb), _fold('sin', k2l, tlb),
                                  _fold('cosh', k2l, tlb), _fold('sinh', k2l, tlb)]
                            fl += v
                fold += fl
        self.elems = elems
        self.ap_list = ap
        self.mp = np.array(mp + [0.0], dtype=np.float64)
        self.fr = np.array(fr + [0.0], dtype=np.float64)
        self.fold = np.array(fold + [0.0], dtype=np.float64)
        self.ap = np.array(ap + [0.0], dtype=np.float64)


    @staticmethod
    def _dynamic_multipole(r, e, prm, flags, fracture, row, ap):
        """A multipole subclass with its own method(): called as
        ufo/lattice.py:107-113 calls it (bound parameters as the text
        ``parameters[i]``); the values it hands its base class (C text or
        numbers) become one program per coefficient (the base class
        ufo/elements.py:152-167: ``knl`` / ``kN`` overrides, ``dx or
        self.dx``)."""
        from ufo_gb300 import cexpr, elements
        if e.kind != 'multipole':
            raise NotImplementedError('user pass methods of thin multipoles only')
        out = e.method(flags=flags, fracture=list(fracture),
                       **{name: f'parameters[{col}]' for name, col in prm.items()})
        vals = [p for p in out if isinstance(p, elements.PassMethod)][0].values
        knl = list(vals['knl']) if vals.get('knl') is not None else list(e.knl)
        ksl = list(vals['ksl']) if vals.get('ksl') is not None else list(e.ksl)
        for p, v in vals.items():
            if p[:1] == 'k' and p[1:].isdigit():
                knl[int(p[1:])] = v
            if p[:1] == 'k' and p[-1:] == 's' and p[1:-1].isdigit():
                ksl[int(p[1:-1])] = v

        def program(v):
            if isinstance(v, str):
                code, _, _ = cexpr.compile_expr(v, allow_params=True)
                return [(cexpr.PUSH, float(row[int(x)])) if op == cexpr.PARAM else (op, x)
                        for op, x in code]
            return [(cexpr.PUSH, float(v))]

        def number(name):
            v = vals.get(name) or getattr(e, name)
            return cexpr.evaluate(program(v)) if isinstance(v, str) else float(v)
        r['type'] = 10
        r['dx'], r['dy'] = number('dx'), number('dy')
        r['nknl'], r['nksl'] = len(knl), len(ksl)
        r['ap_off'] = len(ap)
        for v in knl + ksl:
            code = program(v)
            ap.append(float(len(code)))
            for op, x in code:
                ap += [float(op), float(x)]
        r['ap_len'] = len(ap) - r['ap_off']


def _user_method(e):
    from ufo_gb300 import elements
    return type(e).method is not elements.Element.method


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def track(line, flags, coords, turns, parameters=(), where=(-1,), seed=None, seed_values=None,
          mode=0, dp=0.0, tracks=True, threads=None, count=None, dump_end=None):
    """Run the oracle.  coords: [n, 6].  Returns dict with tracks [n, count*turns, 6]
    (or None), lost [n] uint32 and final [n, 6]."""
    where = list(where)
    prep = Prepared(line, flags, parameters, where, seed_values, dp=dp)
    coords = np.ascontiguousarray(coords, dtype=np.float64)
    n = coords.shape[0]
    count = len(where) if count is None else count
    dump_end = (-1 in where) if dump_end is None else dump_end
    tr = np.zeros((n, count * turns, 6), dtype=np.float64) if tracks else None
    lost = np.zeros(n, dtype=np.uint32)
    final = np.zeros((n, 6), dtype=np.float64)
    seed_arr = None if seed is None else np.ascontiguousarray(seed, dtype=np.int32)
    threads = threads or len(os.sched_getaffinity(0))
    lib().oracle_track(_ptr(prep.elems), prep.n_elem, prep.n_seeds, _ptr(prep.mp), _ptr(prep.fr),
                       _ptr(prep.fold), _ptr(prep.ap), int(flags), int(bool(flags & FIVED)),
                       float(dp), _ptr(coords), _ptr(seed_arr), n, int(turns), int(mode),
                       int(count), int(bool(dump_end)), _ptr(tr), _ptr(lost), _ptr(final),
                       int(threads))
    return {'tracks': tr, 'lost': lost, 'final': final}
