"""The MAD-X loader on the reference's own lattice files.

tests/golden/madx/ holds copies of the reference's optics/*.mad input files
(alba, fodo, fodo2, elements, bend, oct): plain lattice descriptions, the
inputs of the golden cases.  tests/golden/make_golden.py built every golden
lattice by loading one of these files with the reference's own loader
(ufo.Lattice(path=...), ufo/mad.py:101-147) and stored the flattened result
as JSON.  Loading the same file with this library's loader must give the same
flattened lattice: the same element classes, labels and attribute values,
bit for bit."""
import os

import pytest

import helpers as H
import latjson

MADX = os.path.join(H.HERE, 'golden', 'madx')

# golden case -> (file, line) it was built from (make_golden.py)
SOURCES = [
    ('fodo_kick_6d', 'fodo.mad', 'RING'),
    ('fodo2_thick_edges', 'fodo2.mad', 'RING'),
    ('alba_thick', 'alba.mad', 'RING'),
    ('alba_optics_fp64', 'alba.mad', 'RING'),
    ('elements_kick', 'elements.mad', 'TEST'),
    ('rbend_thick', 'bend.mad', 'RRING'),
    ('oct_kick', 'oct.mad', 'RING'),
]


@pytest.mark.parametrize('case,path,name', SOURCES)
def test_loader_reproduces_reference_lattice(case, path, name):
    import ufo_gb300 as u
    line = getattr(u.Lattice(path=os.path.join(MADX, path)), name)
    meta, _ = H.golden()
    ref = meta['lattices'][H.case(case)['lattice']]
    got = latjson.dump(line)
    assert len(got) == len(ref)
    for i, (g, r) in enumerate(zip(got, ref)):
        assert g == r, (i, g, r)


def test_loader_lattice_tracks_like_the_golden_case():
    """The loaded ALBA ring compiles to the same program as the golden case's
    JSON lattice (same opcode table and constants)."""
    import numpy as np
    import ufo_gb300 as u
    from ufo_gb300 import compiler as C
    c = H.case('alba_kick')
    a = C.compile_line(u.Lattice(path=os.path.join(MADX, 'alba.mad')).RING, c['flags'],
                       where=c['where'])
    b = C.compile_line(H.line_of(c), c['flags'], where=c['where'])
    assert np.array_equal(a.ops, b.ops)
    assert np.array_equal(a.table, b.table)
