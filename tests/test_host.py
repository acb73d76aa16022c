"""Host-side logic: compiler folding and binding rules, aperture parsing,
correctly rounded constant math, MAD-X loading, workloads."""
import math

import numpy as np
import pytest

import helpers as H
import ufo_gb300 as u
from ufo_gb300 import aperture as A
from ufo_gb300 import compiler as C
from ufo_gb300 import crmath, workloads as W


def test_crmath_matches_mpmath():
    mp = pytest.importorskip('mpmath')
    mp.mp.prec = 200
    rng = np.random.default_rng(1)
    xs = list(rng.uniform(-3, 3, 300)) + [0.1034762088, 0.1963495408 / 1.3738850810, 1e-8, 2.5]
    for x in xs:
        for name in ('sin', 'cos', 'tan', 'sinh', 'cosh'):
            want = float(getattr(mp, name)(mp.mpf(float(x))))
            assert getattr(crmath, name)(x) == want, (name, x)


def test_aperture_precedence_follows_c():
    # 'a && b' pasted into `if (a && b == 0)` tests a && (b == 0)
    code = A.compile_window('fabs(x) < 0.02 && fabs(y) < 0.005')
    assert A.evaluate(code, x=0.01, y=0.01)          # a true, b false -> lost
    assert not A.evaluate(code, x=0.01, y=0.001)     # a true, b true -> kept
    assert not A.evaluate(code, x=0.05, y=0.01)      # a false -> kept
    circle = A.compile_window('x*x + y*y < 1e-4')
    assert A.evaluate(circle, x=0.02) and not A.evaluate(circle, x=0.005)
    assert A.evaluate(A.compile_window(0))            # default window loses everything
    assert A.evaluate(A.compile_window('1/2 > 0'))    # C integer division: 0 > 0 false -> lost
    with pytest.raises(NotImplementedError):
        A.compile_window('my_function(x) < 1')


def test_teapot_constants_follow_reference_text():
    # knl = ((k*L)*f)/N, outer = (L*f)/(2*(1+N)), inner = ((L*f - 2*outer)*px)/(N-1)
    q = u.Quadrupole('q', length=0.3, k1=1.2, slices=4)
    prog = C.compile_line(u.Line('l', [q]), u.KICK, where=[-1])
    row = prog.ops[0]
    assert row[0] == C.OP_TEAPOT
    tab = prog.table[0]
    L, f, N, k = 0.3, 1.0, 4, 1.2
    outer = (L * f) / (2 * (1 + N))
    assert tab[0] == outer
    A_, d = (L * f - 2. * outer), N - 1.
    assert tab[1] == A_ and tab[2] == d and tab[3] == 1.0 / d and tab[4] == A_ / d
    assert tab[5] == ((0. + k) * L) * f / N


def test_structural_zero_masks():
    q = u.Quadrupole('q', length=0.3, k1=1.2, slices=4, dkn=[0., 0., 0.5])
    prog = C.compile_line(u.Line('l', [q]), u.KICK, where=[-1])
    slices, nn, ns, mn, ms = prog.ops[0][3:8]
    assert (slices, nn, ns) == (4, 6, 0)   # pad([0,0,.5], 2) appends 3 zeros
    assert mn == 0b110                     # k1 at index 1, dk2 at index 2


def test_parameter_zero_in_one_seed_is_not_trimmed():
    q = u.Quadrupole('q', length=0.3, k1=1.2, slices=4)
    rows = np.array([[0.0], [0.3]])
    prog = C.compile_line(u.Line('l', [q]), u.KICK, [('q', 'dk2')], [-1], seed_values=rows)
    assert prog.ops[0][6] & 0b100
    prog0 = C.compile_line(u.Line('l', [q]), u.KICK, [('q', 'dk2')], [-1],
                           seed_values=rows[:1])
    assert not prog0.ops[0][6] & 0b100


def test_parameter_binding_quirks():
    line = u.Line('l', [u.Drift('d', length=1.0), u.Quadrupole('q', length=0.3, k1=1.)])
    # 'dp'[0] == 'd' binds to the element labelled 'd' (ufo/lattice.py:109)
    with pytest.raises(TypeError):
        C.compile_line(line, 0, ['dp'], [-1])
    binds = C.element_bindings(line.flatten(), [('q', 'k1'), (1, 'dx'), ('q', 'k1')])
    assert binds[1] == {'k1': 2, 'dx': 1}


def test_fractures_follow_reference():
    per, pre = C.fractures(4, [0, 0.5, 1.25, 2.75, -1])
    assert pre == [True, False, False, False]
    assert per[0] == [0.5] and per[1] == [0.25] and per[2] == [0.75] and per[3] == []


def test_user_method_returning_opencl_rejected():
    """An override that returns its own OpenCL (not its base class's
    method() result) cannot run in the data-driven kernels."""
    class Raw(u.Multipole):
        def method(self, **kw):
            return ['x += 1;']
    with pytest.raises(NotImplementedError):
        C.compile_line(u.Line('l', [Raw('n', knl=[0, 1])]), 0, [], [-1])


def test_line_method_lowers_every_element_type():
    """What the reference's tests/elements.py checks (every element type of
    elements.mad lowers), in thick and kick modes, and fractures split the
    program into one segment per interval."""
    line = H.line_of(H.case('elements_kick'))
    kinds = {e.kind for e in line.flatten()}
    assert kinds == {'drift', 'quadrupole', 'sbend', 'sextupole', 'multipole', 'marker'}
    for flags in (0, u.KICK, u.KICK | u.EXACT, u.LINEAR | u.ACHROMATIC):
        segs = line.method(flags=flags)
        assert len(segs) == 1 and len(segs[0]) > 0
    assert len(line.method(fracture=[1.5, 4.25], flags=u.KICK)) == 3  # bend, sextupole
    assert len(line.method(fracture=[3.5], flags=u.KICK)) == 1  # a marker drops it (thin)


def test_madx_loader():
    lat = u.Lattice()
    from ufo_gb300 import madx
    d = madx.loads('QF: QUADRUPOLE, L=0.3, K1= 1.2e0;\nO: DRIFT, L=1;\n'
                   'B: SBEND, L=1.5, ANGLE=0.19, E1=0.1, HGAP=0.01, FINT=0.5;\n'
                   'M: MULTIPOLE, KNL={0, 0, 3.5};\nX: FOO, A=1;\n'
                   'C: LINE=(QF, O, B, M);\nR: LINE=(C, C);')
    assert isinstance(d['R'], u.Line) and len(d['R'].flatten()) == 8
    assert d['B'].hgap == 0.01 and d['M'].knl == [0, 0, 3.5]
    with pytest.raises(TypeError):
        madx.loads('Q: QUADRUPOLE, K9=1;')
    assert lat is not None


def test_golden_lattices_rebuild():
    for c in H.cases():
        line = H.line_of(c)
        assert len(line.flatten()) > 0


def test_workloads_shapes():
    r1 = W.c1_ring(u)
    assert len(r1.flatten()) == 128
    r2 = W.c2_ring(u)
    assert len(r2.flatten()) == 1024
    M = W._linear_map(r2, 0.0)
    assert abs((M[0, 0] + M[1, 1]) / 2) < 1 and abs((M[2, 2] + M[3, 3]) / 2) < 1
    assert W.c3_grid().shape == (196608, 6)
    parts, turns = W.c4_sizes()
    assert parts.min() >= 256 and parts.max() <= 8192 and turns.min() >= 1000


def test_flop_counts():
    p1 = C.compile_line(W.c1_ring(u), u.KICK, where=[-1])
    # teapot N=4: 2 outer drifts (4 each) + 3 inner drifts x*(px*A)/3 (6 each);
    # quad kick 5, bend weak focusing 2 per slice; 4 plain drifts (4 each)
    quad = 2 * 4 + 3 * 6 + 4 * 5
    bend = 2 * 4 + 3 * 6 + 4 * 2
    assert p1.flops == 16 * (2 * quad + 2 * bend + 4 * 4)


def test_fma_drift_merging_conserves_length_and_flops():
    """FMA programs fold plain drifts into neighbouring teapot outer drifts:
    the total drift length per turn, the element count and the reference
    flop count are unchanged, the executed count drops by the merged drifts'
    two FMAs each, and strict programs are not touched."""
    import numpy as np
    import ufo_gb300 as u
    from ufo_gb300 import compiler as C, workloads as W

    def drift_length(p):
        tot = 0.0
        for r in p.ops:
            kind, fl, off = int(r[0]), int(r[1]), int(r[2])
            c = p.table[0, off:]
            if kind == C.OP_DRIFT:
                assert int(r[3]) == C.DF_MUL
                tot += c[0]
            elif kind == C.OP_TEAPOT:
                N, nn, ns, mn, ms = (int(v) for v in r[3:8])
                inner = (N - 1) * (c[1] if (fl >> C.SH_FINNER) & 3 == C.DF_MUL else c[4])
                exit_ = c[0]
                if fl & C.F_SPLITO:
                    k = 1 + ((1 if (fl >> C.SH_FINNER) & 3 == C.DF_MUL else 4) if N > 1 else 0)
                    k += bin(mn).count('1') + bin(ms).count('1') + (1 if fl & C.F_WEAK else 0)
                    exit_ = c[k]
                tot += c[0] + exit_ + (inner if N > 1 else 0.0)
        return tot

    for ring in (W.c2_ring(u), W.c3_ring(u)):
        strict = C.compile_line(ring, u.KICK, where=[-1])
        fma = C.compile_line(ring, u.KICK | u.FMA, where=[-1], linearize=False)
        assert len(fma.ops) < len(strict.ops)
        merged = sum(int(r[0]) == C.OP_DRIFT for r in strict.ops) - \
            sum(int(r[0]) == C.OP_DRIFT for r in fma.ops)
        assert merged > 0
        assert fma.flops == strict.flops and fma.n_elements == strict.n_elements
        assert fma.flops_fast == strict.flops_fast - 4 * merged
        assert abs(drift_length(fma) - drift_length(strict)) < 1e-9 * drift_length(strict)
    assert not np.any(C.compile_line(W.c2_ring(u), u.KICK | u.FMA, where=[-1]).ops[:, 0] ==
                      C.OP_DRIFT)
    assert not np.any(C.compile_line(W.c2_ring(u), u.KICK, where=[-1]).ops[:, 1] & C.F_SPLITO)


def test_fma_programs_append_dense_power_series_for_general_kicks():
    """FMA programs append to every general kick (here: C4-style errors of
    orders 3-6 on every magnet) the dense series a_n = RN(kn_n * RN(1/n!)),
    then b_n, n up to the highest order, structural zeros as +0.0, after all
    other constants (F_PSER); quadrupole/sextupole short forms and strict
    programs get none."""
    import math
    import numpy as np
    import ufo_gb300 as u
    from ufo_gb300 import compiler as C, workloads as W
    ring = W.c1_ring(u)
    params = W.c4_parameters(ring)
    rows = W.c4_seed_rows(ring, 3)
    fma = C.compile_line(ring, u.KICK | u.FMA, params, [], seed_values=rows)
    strict = C.compile_line(ring, u.KICK, params, [], seed_values=rows)
    assert not any(int(r[1]) & C.F_PSER for r in strict.ops)
    rf = []
    fact = 1.0
    for k in range(8):
        if k:
            fact *= float(k)
        rf.append(1.0 / fact)
    n_series = 0
    for r in fma.ops:
        kind, fl = int(r[0]), int(r[1])
        if kind != C.OP_TEAPOT:
            continue
        N, nn, ns, mn, ms = (int(v) for v in r[3:8])
        general = ms or not ((nn == 2 and mn == 2) or (nn == 3 and mn == 4) or mn == 0)
        assert bool(fl & C.F_PSER) == bool(general and (mn | ms))
        if not fl & C.F_PSER:
            continue
        n_series += 1
        fi = (fl >> C.SH_FINNER) & 3
        first = int(r[2]) + 1 + (0 if N <= 1 else 4 if fi == C.DF_DIV else 1)
        tail = int(r[2]) + (first - int(r[2])) + bin(mn).count('1') + bin(ms).count('1') + \
            (1 if fl & C.F_WEAK else 0) + (1 if fl & C.F_SPLITO else 0)
        M = (mn | ms).bit_length()
        coef = fma.table[:, first:first + bin(mn).count('1') + bin(ms).count('1')]
        ser = fma.table[:, tail:tail + 2 * M]
        q = 0
        for part, mask in ((0, mn), (1, ms)):
            for j in range(M):
                got = ser[:, part * M + j]
                if mask >> j & 1:
                    assert np.array_equal(got, coef[:, q] * rf[j])
                    q += 1
                else:
                    assert np.all(got == 0.0) and not np.any(np.signbit(got))
    assert n_series > 0
    assert math.isclose(rf[5], 1 / 120, rel_tol=1e-15)


@pytest.mark.parametrize('yoshida', [False, True])
def test_fma_linear_elements_compose_their_drifts_and_weak_kicks(yoshida):
    """FMA programs replace each kick-free teapot (or Yoshida) element, here
    the C2 ring's bends with their merged neighbouring drifts, by one linear
    op: a 2x2 matrix for (x, px) and a drift for (y, py), composed on the host.
    Applied to test vectors it equals the element's own sequence of drifts and
    weak-focusing kicks to rounding."""
    ring = W.c2_ring(u)
    fl = u.KICK | u.FMA | (u.YOSHIDA if yoshida else 0)
    lin = C.compile_line(ring, fl, where=[-1])
    ref = C.compile_line(ring, fl, where=[-1], linearize=False)
    assert lin.flops == ref.flops and lin.flops_fast < ref.flops_fast
    # the bends' zero-angle edges (structural zeros) leave with them
    linear_elems = {e for e, r in zip(lin.op_elem, lin.ops) if int(r[0]) == C.OP_LINEAR}
    keep = [i for i, r in enumerate(ref.ops) if not (
        int(r[0]) == C.OP_EDGE and ref.op_elem[i] in linear_elems and
        not int(r[1]) & (C.F_T1 | C.F_T2 | C.F_RTPSI))]
    assert len(keep) == len(lin.ops) < len(ref.ops)
    ref_ops = ref.ops[keep]
    rng = np.random.default_rng(3)
    v = rng.standard_normal((4, 16)) * np.array([[1e-3], [1e-4], [1e-3], [1e-4]])
    n = 0
    for a, b in zip(lin.ops, ref_ops):
        if int(a[0]) != C.OP_LINEAR:  # the same op (its table offset may move)
            assert np.array_equal(np.delete(a, 2), np.delete(b, 2))
            continue
        n += 1
        assert int(b[0]) == C.OP_TEAPOT
        m = lin.table[0, int(a[2]):int(a[2]) + 5]
        c = ref.table[0, int(b[2]):]
        N, fl_b = int(b[3]), int(b[1])
        x, px, y, py = v.copy()
        if fl_b & C.F_YOSHIDA:
            wk = c[7] if fl_b & C.F_WEAK else 0.0
            for _ in range(N):
                x, y = x + px * c[0], y + py * c[0]
                for k in range(3):
                    px = px - x * (wk * c[4 + k])
                    x, y = x + px * c[1 + k], y + py * c[1 + k]
        else:
            fi = (fl_b >> C.SH_FINNER) & 3
            Li = c[1] if fi == C.DF_MUL else c[4]
            ck = 1 + (0 if N <= 1 else (4 if fi == C.DF_DIV else 1))
            wk = c[ck] if fl_b & C.F_WEAK else 0.0
            Lx = c[ck + (1 if fl_b & C.F_WEAK else 0)] if fl_b & C.F_SPLITO else c[0]
            x, y = x + px * c[0], y + py * c[0]
            for sl in range(N):
                px = px - x * wk
                L = Li if sl < N - 1 else Lx
                x, y = x + px * L, y + py * L
        xl = m[0] * v[0] + m[1] * v[1]
        pxl = m[2] * v[0] + m[3] * v[1]
        yl = v[2] + v[3] * m[4]
        for got, want in ((xl, x), (pxl, px), (yl, y)):
            assert np.max(np.abs(got - want)) <= 1e-15 * np.max(np.abs(want)) + 1e-19
    assert n == 128
