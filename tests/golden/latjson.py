"""Flattened-lattice <-> JSON for the golden fixtures.

A lattice is stored as the list of its flattened elements with the attributes
the tracker reads, so fixtures made from the reference's element objects can
be rebuilt with ufo_gb300's classes on a machine without the reference.
"""
ATTRS = {
    'Marker': [],
    'Drift': ['length'],
    'Multipole': ['knl', 'ksl', 'dx', 'dy'],
    'Quadrupole': ['slices', 'length', 'k1', 'dx', 'dy', 'dkn', 'dks'],
    'Sbend': ['slices', 'length', 'angle', 'k1', 'e1', 'e2', 'hgap', 'fint', 'dx', 'dy', 'dkn',
              'dks'],
    'Rbend': ['slices', 'length', 'angle', 'k1', 'e1', 'e2', 'hgap', 'fint', 'dx', 'dy', 'dkn',
              'dks'],
    'Sextupole': ['slices', 'length', 'k2', 'k2s', 'dx', 'dy', 'dkn', 'dks'],
    'Octupole': ['slices', 'length', 'k3', 'k3s', 'dx', 'dy', 'dkn', 'dks'],
    'Wire': ['x', 'y', 'k'],
    'Aperture': ['window'],
}


def _val(v):
    if isinstance(v, (list, tuple)):
        return [float(x) for x in v]
    if isinstance(v, str):
        return v
    if isinstance(v, int) and not isinstance(v, bool):
        return v
    return float(v)


def dump(line):
    out = []
    for e in line.flatten():
        # a user subclass (e.g. a kicker overriding method()) is stored as its
        # library base class; its own behaviour is described by the case
        cls = next(c.__name__ for c in type(e).__mro__ if c.__name__ in ATTRS)
        d = {'class': cls, 'label': e.label}
        if cls != type(e).__name__:
            d['subclass'] = type(e).__name__
        for a in ATTRS[cls]:
            d[a] = _val(e.__dict__[a])
        out.append(d)
    return out


def load(items, m=None):
    if m is None:
        import ufo_gb300 as m
    els = []
    for d in items:
        d = dict(d)
        cls = getattr(m, d.pop('class'))
        label = d.pop('label')
        d.pop('subclass', None)
        els.append(cls(label, **d))
    return m.Line('RING', els)


def params_dump(params):
    return [list(p) if isinstance(p, tuple) else p for p in params]


def params_load(params):
    return [tuple(p) if isinstance(p, list) else p for p in params]
