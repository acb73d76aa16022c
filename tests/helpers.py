"""Shared test helpers: golden-fixture access and case runners."""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
if REPO not in sys.path:
    sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(HERE, 'golden'))

import latjson  # noqa: E402

COORDS = ('x', 'px', 'y', 'py', 'z', 'dp')
_gold = None


def golden():
    global _gold
    if _gold is None:
        with open(os.path.join(HERE, 'golden', 'cases.json')) as f:
            meta = json.load(f)
        arrs = dict(np.load(os.path.join(HERE, 'golden', 'golden.npz')))
        _gold = (meta, arrs)
    return _gold


def cases(kind=None):
    meta, _ = golden()
    return [c for c in meta['cases'] if kind is None or c['kind'] == kind]


def case(name):
    for c in cases():
        if c['name'] == name:
            return c
    raise KeyError(name)


def arr(name, key):
    return golden()[1][f'{name}/{key}']


def line_of(c):
    """The case's lattice; elements recorded as user subclasses (kickers
    whose method() is their own) are rebuilt from tests/kickers.py."""
    meta, _ = golden()
    items = meta['lattices'][c['lattice']]
    line = latjson.load(items)
    for i, d in enumerate(items):
        if 'subclass' in d:
            import kickers
            e = line[i]
            extra = {k: c[k] for k in ('t0', 'tau') if k in c}
            line[i] = getattr(kickers, d['subclass'])(e.label, knl=e.knl, ksl=e.ksl, dx=e.dx,
                                                       dy=e.dy, **extra)
    return line


def coords_from_pool(pool, params, flags, dp=0.0):
    n = pool.shape[0]
    coords = np.zeros((n, 6))
    for j, name in enumerate(COORDS):
        if name in params:
            coords[:, j] = pool[:, params.index(name)]
    if flags & 2:  # FIVED
        coords[:, 4] = 0.0
        coords[:, 5] = dp
    return coords


def oracle_case(c, perturb=0.0):
    """Run a golden track/sa case through the C oracle; ``perturb`` scales the
    initial coordinates by (1 + perturb)."""
    from oracle import oracle as O
    line = line_of(c)
    params = latjson.params_load(c['parameters'])
    pool = arr(c['name'], 'in/pool').astype(np.float64)
    coords = coords_from_pool(pool, params, c['flags'], c.get('dp', 0.0)) * (1.0 + perturb)
    n = pool.shape[0]
    if c['kind'] == 'track':
        return O.track(line, c['flags'], coords, c['turns'], parameters=params, where=c['where'],
                       seed=np.arange(n), seed_values=pool, mode=0, dp=c.get('dp', 0.0))
    return O.track(line, c['flags'], coords, c['turns'], parameters=params, where=[],
                   seed=np.arange(n), seed_values=pool, mode=1, dp=c.get('dp', 0.0),
                   tracks=False, count=0, dump_end=False)


def gpu_case(c, extra_flags=0):
    """Run a golden track/sa case through the public API on the GPU."""
    import ufo_gb300 as u
    line = line_of(c)
    params = latjson.params_load(c['parameters'])
    pool = arr(c['name'], 'in/pool')
    flags = c['flags'] | extra_flags
    if c['kind'] == 'track':
        t = u.Track(line, flags=flags, turns=c['turns'], particles=pool.shape[0],
                    parameters=params, where=c['where'], dp=c.get('dp', 0.0))
        t.parameters[:] = pool
        t.run()
        return t
    s = u.StableAperture(line, flags=flags, turns=c['turns'], particles=pool.shape[0],
                         parameters=params, dp=c.get('dp', 0.0))
    s.parameters[:] = pool
    s.run()
    return s


def program_is_exact(prog):
    """True when no op of the program evaluates a transcendental per particle
    (those use the GPU's libm, which may differ from the host C library in
    the last bit)."""
    from ufo_gb300 import compiler as C
    for row in prog.ops:
        kind, flags = int(row[0]), int(row[1])
        if kind in (C.OP_THICKQ, C.OP_THICKB) and not flags & C.F_CONST:
            return False
        if kind == C.OP_EDGE and flags & C.F_RTPSI:
            return False
        if kind == C.OP_WIRE:
            return False
        if kind == C.OP_DYNKICK and _dynkick_calls(prog.table[0], int(row[2]), int(row[5])):
            return False
    return True


def _dynkick_calls(table, off, words):
    """True when a dynamic kick's coefficient programs call a libm function."""
    from ufo_gb300 import cexpr as X
    q = off
    while q < off + words:
        n = int(table[q])
        ops = table[q + 1:q + 1 + 2 * n:2].astype(int)
        if any(op in (X.SIN, X.COS, X.TAN, X.EXP, X.LOG) for op in ops):
            return True
        q += 1 + 2 * n
    return False


def track_rel_err(a, b):
    """max |a-b| over written slots, relative to each coordinate's max |b|."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = np.nanmax(np.abs(b).reshape(-1, b.shape[-1]), axis=0)
    scale = np.where(scale > 0, scale, 1.0)
    d = np.abs(a - b) / scale
    both_nan = np.isnan(a) & np.isnan(b)
    d = np.where(both_nan, 0.0, d)
    return float(np.nanmax(np.where(np.isnan(d), np.inf, d))) if d.size else 0.0


def tolerance(turns):
    """FP64 agreement bar: 1e-12 relative after one turn, growing linearly to
    1e-9 after 1000 turns."""
    return 1e-12 * max(1, turns)


def per_particle_err(a, b):
    """Relative error per particle (scale: each coordinate's max |b|)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = np.nanmax(np.abs(b).reshape(-1, b.shape[-1]), axis=0)
    scale = np.where(scale > 0, scale, 1.0)
    d = np.abs(a - b) / scale
    d = np.where(np.isnan(a) & np.isnan(b), 0.0, d)
    d = np.where(np.isnan(d), np.inf, d)
    return d.reshape(d.shape[0], -1).max(axis=1)


def regular_mask(c, tol):
    """Particles whose reference trajectory is regular at the tested length:
    re-tracking with the start perturbed by 1e-15 (relative) moves them by
    less than tol/10.  Chaotic particles amplify any rounding difference, so
    no FP64 implementation other than the reference's own operation order can
    be held to a fixed tolerance on them."""
    a = oracle_case(c)['tracks']
    b = oracle_case(c, perturb=1e-15)['tracks']
    # escaping particles end in overflow, where the turn of inf - inf = NaN is
    # a threshold effect rather than a relative error: not regular either
    with np.errstate(invalid='ignore'):
        escaped = (np.isinf(a) | (np.abs(np.nan_to_num(a)) > 1e10)).reshape(a.shape[0], -1)
    return (per_particle_err(b, a) <= tol / 10) & ~escaped.any(axis=1)


def first_turn_slots(c):
    meta_where = c['where']
    return max(1, len(meta_where))
