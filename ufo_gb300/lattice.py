"""Lines and lattices (the reference's ufo/lattice.py:19-150, tracking part).

``Line`` is a ``list`` of elements and nested lines with the reference's
helpers: ``flatten`` (ufo/lattice.py:121-124), ``find`` (:54-61), ``locate``
(:63-72) and the ``count`` / ``length`` / ``angle`` properties (:41-52).
``Line.method`` keeps the reference's signature (:86-119) but returns the
lowered opcode segments instead of OpenCL source strings.
"""
from . import madx


class Lattice:
    """A collection of elements and lines, optionally loaded from a MAD-X
    dialect file (ufo/lattice.py:19-26)."""

    def __init__(self, path=None):
        if path:
            self.__dict__.update(madx.load(path))

    def __repr__(self):
        return '\n'.join(repr(v) for v in self.__dict__.values())


class Line(list):
    """A list of elements or other lines."""

    def __init__(self, label, line=None):
        self.label = label
        super().__init__(line if line is not None else [])

    def __str__(self):
        return self.label

    def __repr__(self):
        return f'{self.label: <8}: LINE         {[str(e) for e in self]}'

    @property
    def count(self):
        return sum(getattr(e, 'count', 1.) for e in self)

    @property
    def length(self):
        return sum(getattr(e, 'length', 0.) for e in self)

    @property
    def angle(self):
        return sum(getattr(e, 'angle', 0.) for e in self)

    def find(self, what):
        """Indices (in the flattened line) of the elements with what(e) true."""
        return [i for i, e in enumerate(self.flatten()) if what(e)]

    def locate(self, element):
        """Position in metres of a flat index whose fractional part is a
        fraction of that element's length; -1 is the end of the line."""
        if element == -1:
            return self.length
        s = 0
        for idx, e in enumerate(self.flatten()):
            if int(element) == idx:
                return s + (element - int(element)) * e.length
            s += getattr(e, 'length', 0.)
        return None

    def flatten(self, reverse=False):
        """All nested lines expanded into their elements."""
        flat = []
        for e in self:
            if getattr(e, 'flatten', None):
                flat.extend(e.flatten())
            else:
                flat.append(e)
        return flat

    def method(self, fracture=None, flags=0, parameters=None):
        """Lower the line to opcode segments, one per fracture interval.  Kept
        for scripts that call ``method()`` to check a lattice compiles."""
        from . import compiler
        prog = compiler.compile_line(self, flags=flags, parameters=parameters or [],
                                     where=fracture or [])
        return prog.segments


class Beam:
    """Beam description (ufo/lattice.py:152-164): energy in eV, particle mass
    in eV, bunch charge, current, emittances, bunch length and energy spread.
    ``gamma`` is (1 + energy) / mass as the reference computes it (the 1 eV
    offset is below 1e-9 relative at GeV energies)."""

    def __init__(self, energy=3e9, particle_mass=None, bunch_charge=1e-9, beam_current=0.25,
                 ex=1e-9, ey=1e-9, bunch_length=6e-3, energy_spread=1e-3):
        from .constants import electron_mass
        self.energy = energy
        self.particle_mass = electron_mass if particle_mass is None else particle_mass
        self.gamma = (1. + energy) / self.particle_mass
        self.bunch_charge = bunch_charge
        self.beam_current = beam_current
        self.ex = ex
        self.ey = ey
        self.bunch_length = bunch_length
        self.energy_spread = energy_spread
