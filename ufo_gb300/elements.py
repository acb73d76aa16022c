"""Lattice element classes.

The constructors, attribute names, ``parameters`` lists and the scalar
multipole accessors (``dkN`` / ``dkNs`` / ``kN`` / ``kNs``) follow the
reference's element classes (ufo/elements.py:14-522) so that user scripts and
MAD-X files load unchanged.  What differs is what an element produces: the
reference's ``method()`` returns OpenCL C source strings
(ufo/elements.py:98-106, 152-167, 200-219, 260-285, 326-352, 392-413,
447-468, 494-500, 517-518); here ``lower()`` hands the element's resolved
attributes to :mod:`ufo_gb300.compiler`, which emits rows of the opcode table
that the sm_103a kernels interpret.

One deliberate deviation: the reference uses shared mutable default lists
(``dkn=[]``) so every element built without errors aliases one list; here each
element gets its own copy.
"""
import ufo_gb300

#: attribute names that the tracker reads for each element type, in the order
#: the reference lists them in ``self.parameters``
_SCALAR_ATTRS = ('length', 'angle', 'k1', 'e1', 'e2', 'hgap', 'fint', 'dx', 'dy',
                 'k2', 'k2s', 'k3', 'k3s', 'x', 'y', 'k')


def _dk_index(name, prefix):
    """Return (order, skew) for names like ``dk3`` / ``dk3s`` (prefix 'dk') or
    ``k2`` / ``k2s`` (prefix 'k'); None when ``name`` is not such a name.
    Mirrors the name tests of ufo/elements.py:16-23 and :135-140."""
    n = len(prefix)
    if name[:n] != prefix:
        return None
    if name[n:].isdigit():
        return int(name[n:]), False
    if name[-1:] == 's' and name[n:-1].isdigit():
        return int(name[n:-1]), True
    return None


class PassMethod:
    """What ``Element.method()`` returns: the element and the attribute values
    its pass method was called with."""
    __slots__ = ('element', 'values')

    def __init__(self, element, values):
        self.element = element
        self.values = values


class Element:
    """Base element.  ``lower()`` is what the compiler calls.  Subclasses may
    override ``method()`` (the reference's plugin point) as long as they return
    their base class's ``method()`` result; the values they pass it may be C
    expressions (see ``method``)."""

    kind = 'element'

    def __str__(self):
        return self.label

    def __repr__(self):
        msg = f'{self.label: <8}: {type(self).__name__.upper(): <12} '
        return msg + '   '.join(f'{p}={self.__dict__.get(p)}' for p in self.parameters)

    # dkN / dkNs scalar access to the error lists (ufo/elements.py:36-54)
    def __setattr__(self, name, value):
        idx = _dk_index(name, 'dk')
        if idx is not None and 'dkn' in self.__dict__:
            order, skew = idx
            (self.dks if skew else self.dkn)[order] = value
            return
        object.__setattr__(self, name, value)

    def __getattr__(self, name):
        idx = _dk_index(name, 'dk')
        if idx is not None and 'dkn' in self.__dict__:
            order, skew = idx
            return (self.dks if skew else self.dkn)[order]
        raise AttributeError(name)

    def method(self, flags=0, fracture=None, **kwargs):
        """The reference's plugin point (ufo/elements.py), which returned
        OpenCL source.  Here it returns ``[PassMethod(self, values)]``: a
        subclass overriding it (a time-dependent kicker, HOWTO.md:84-200) calls
        ``super().method(k1='(C expression)', **kwargs)`` as it would with the
        reference, and the compiler lowers the values it passed (numbers, or C
        expressions of ``turn``, the coordinates and ``parameters[i]``)."""
        values = dict(kwargs)
        values['flags'] = flags
        values['fracture'] = fracture
        return [PassMethod(self, values)]

    def lower(self):
        """Return a dict of resolved attributes for the compiler."""
        return {'kind': self.kind}

    def survey(self, x0=None, alpha0=0.):
        raise NotImplementedError('survey() (element positions) is not part of the tracking library')


class Marker(Element):
    """A marker element (no-op)."""
    kind = 'marker'

    def __init__(self, label):
        self.label = label
        self.parameters = []


class Drift(Element):
    """A drift.  The EXACT flag selects the exact-Hamiltonian pass."""
    kind = 'drift'

    def __init__(self, label, length=0.):
        self.label = label
        self.length = length
        self.parameters = ['length']


class Multipole(Element):
    """A thin multipole with integrated normal/skew strengths ``knl``/``ksl``
    and an alignment offset (ufo/elements.py:116-176)."""
    kind = 'multipole'

    def __init__(self, label, knl=None, ksl=None, dx=0., dy=0.):
        self.label = label
        self.knl = list(knl) if knl is not None else []
        self.ksl = list(ksl) if ksl is not None else []
        self.dx = dx
        self.dy = dy
        self.parameters = ['knl', 'ksl', 'dx', 'dy']

    # kN / kNs scalar access to knl / ksl (ufo/elements.py:132-150)
    def __setattr__(self, name, value):
        idx = _dk_index(name, 'k')
        if idx is not None and 'knl' in self.__dict__:
            order, skew = idx
            (self.ksl if skew else self.knl)[order] = value
            return
        super().__setattr__(name, value)

    def __getattr__(self, name):
        idx = _dk_index(name, 'k')
        if idx is not None and 'knl' in self.__dict__:
            order, skew = idx
            return (self.ksl if skew else self.knl)[order]
        return super().__getattr__(name)


class Quadrupole(Element):
    """A thick normal quadrupole (ufo/elements.py:178-227)."""
    kind = 'quadrupole'

    def __init__(self, label, slices=None, length=0., k1=0., dx=0., dy=0., dkn=None, dks=None):
        self.label = label
        self.slices = slices if slices else ufo_gb300.DEFAULT_QUADRUPOLE_SLICES
        self.length = length
        self.k1 = k1
        self.dx = dx
        self.dy = dy
        self.dkn = list(dkn) if dkn is not None else []
        self.dks = list(dks) if dks is not None else []
        self.parameters = ['length', 'k1', 'dx', 'dy', 'dkn', 'dks']


class Sbend(Element):
    """A sector bend with edge focusing (ufo/elements.py:229-293)."""
    kind = 'sbend'

    def __init__(self, label, slices=None, length=0., angle=0., k1=0., e1=0., e2=0., hgap=0.,
                 fint=0., dx=0., dy=0., dkn=None, dks=None):
        self.label = label
        self.slices = slices if slices else ufo_gb300.DEFAULT_BEND_SLICES
        self.length = length
        self.angle = angle
        self.k1 = k1
        self.e1 = e1
        self.e2 = e2
        self.hgap = hgap
        self.fint = fint
        self.dx = dx
        self.dy = dy
        self.dkn = list(dkn) if dkn is not None else []
        self.dks = list(dks) if dks is not None else []
        self.parameters = ['length', 'angle', 'k1', 'e1', 'e2', 'hgap', 'fint', 'dx', 'dy',
                           'dkn', 'dks']


class Rbend(Sbend):
    """A rectangular bend: an Sbend whose edge angles are e + angle/2
    (ufo/elements.py:295-366, edges at :349-350)."""
    kind = 'rbend'

    def __init__(self, label, slices=None, length=0., angle=0., k1=0., e1=0., e2=0., hgap=0,
                 fint=0, dx=0., dy=0., dkn=None, dks=None):
        super().__init__(label, slices=slices, length=length, angle=angle, k1=k1, e1=e1, e2=e2,
                         hgap=hgap, fint=fint, dx=dx, dy=dy, dkn=dkn, dks=dks)


class Sextupole(Element):
    """A thick sextupole, always teapot-sliced (ufo/elements.py:368-421)."""
    kind = 'sextupole'

    def __init__(self, label, length=0., slices=None, k2=0., k2s=0., dx=0., dy=0., dkn=None,
                 dks=None):
        self.label = label
        self.length = length
        self.slices = slices if slices else ufo_gb300.DEFAULT_SEXTUPOLE_SLICES
        self.k2 = k2
        self.k2s = k2s
        self.dx = dx
        self.dy = dy
        self.dkn = list(dkn) if dkn is not None else []
        self.dks = list(dks) if dks is not None else []
        self.parameters = ['length', 'k2', 'k2s', 'dx', 'dy', 'dkn', 'dks']


class Octupole(Element):
    """A thick octupole, always teapot-sliced (ufo/elements.py:423-476)."""
    kind = 'octupole'

    def __init__(self, label, length=0., slices=None, k3=0., k3s=0., dx=0., dy=0., dkn=None,
                 dks=None):
        self.label = label
        self.length = length
        self.slices = slices if slices else ufo_gb300.DEFAULT_OCTUPOLE_SLICES
        self.k3 = k3
        self.k3s = k3s
        self.dx = dx
        self.dy = dy
        self.dkn = list(dkn) if dkn is not None else []
        self.dks = list(dks) if dks is not None else []
        self.parameters = ['length', 'k3', 'k3s', 'dx', 'dy', 'dkn', 'dks']


class Wire(Element):
    """Kick k/r from a wire parallel to the beam at (x, y) (ufo/elements.py:478-503)."""
    kind = 'wire'

    def __init__(self, label, x=0., y=0., k=0.):
        self.label = label
        self.x = x
        self.y = y
        self.k = k
        self.parameters = ['x', 'y', 'k']


class Aperture(Element):
    """Particles for which the C expression ``window`` is false get x = NaN
    (ufo/elements.py:505-522).  The window is kept as the reference's C
    expression text and parsed by :mod:`ufo_gb300.aperture`."""
    kind = 'aperture'

    def __init__(self, label, window=0):
        self.label = label
        self.window = window
        self.parameters = ['aperture']
