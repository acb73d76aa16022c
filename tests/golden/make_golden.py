"""Generate the golden fixtures by running the REFERENCE implementation.

Run where the reference is importable (it needs its source tree; the GPU machine
does not have it):

    python tests/golden/make_golden.py /path/to/reference

The reference (bellaz89/ufo) generates OpenCL C and runs it through pyopencl.
pyopencl is not installed here, so oracle/refshim provides a stand-in module
that compiles the generated kernel source with gcc (strict IEEE) and runs it
on the host cores over the reference's own atomic work queue; the reference's
Python code runs unmodified.  For every case this script stores the inputs
(flattened lattice as JSON, flags, parameter names and values, where, turns)
and the reference's outputs, plus the MAD-X known-answer values that the
reference's own tests pin (parsed from its tests/*.py).
"""
import hashlib
import json
import math
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)
import latjson  # noqa: E402

COORDS = ('x', 'px', 'y', 'py', 'z', 'dp')


def main(ref):
    os.environ.setdefault('PYTHONDONTWRITEBYTECODE', '1')
    sys.dont_write_bytecode = True
    sys.path.insert(0, os.path.join(REPO, 'oracle', 'refshim'))
    sys.path.insert(0, ref)
    import ufo
    from ufo_gb300 import workloads as W

    optics = os.path.join(ref, 'optics')
    cases = []
    arrays = {}
    lattices = {}

    def lat(path, name='RING'):
        return getattr(ufo.Lattice(path=os.path.join(optics, path)), name)

    def add(name, kind, line, flags, meta, outs, inputs):
        meta = dict(meta)
        items = latjson.dump(line)
        key = hashlib.sha1(json.dumps(items).encode()).hexdigest()[:12]
        lattices[key] = items
        meta.update(name=name, kind=kind, flags=int(flags), lattice=key)
        cases.append(meta)
        for k, v in inputs.items():
            arrays[f'{name}/in/{k}'] = np.asarray(v)
        for k, v in outs.items():
            arrays[f'{name}/out/{k}'] = np.asarray(v)

    def track_case(name, line, flags, turns, n, params, where, scale=1e-3, seed=0, dp=0.0,
                   pool=None):
        flags |= ufo.DOUBLE_PRECISION
        tr = ufo.Track(line, flags=flags, turns=turns, particles=n, parameters=params,
                       where=list(where), dp=dp)
        rng = np.random.default_rng(seed)
        if pool is None:
            pool = rng.normal(size=tr.parameters.shape) * scale
        tr.parameters[:] = pool
        tr.run(threads=min(n, 8))
        add(name, 'track', line, flags, dict(turns=turns, particles=n,
                                             parameters=latjson.params_dump(params),
                                             where=list(where), dp=dp),
            {'tracks': tr.tracks}, {'pool': pool})

    def sa_case(name, line, flags, turns, pool, params, dp=0.0):
        flags |= ufo.DOUBLE_PRECISION
        n = pool.shape[0]
        sa = ufo.StableAperture(line, flags=flags, turns=turns, particles=n, parameters=params,
                                dp=dp)
        sa.parameters[:] = pool
        sa.run(threads=8)
        add(name, 'sa', line, flags, dict(turns=turns, particles=n,
                                          parameters=latjson.params_dump(params), dp=dp),
            {'lost': sa.lost}, {'pool': pool})

    six = ['x', 'px', 'y', 'py', 'dp']
    # --- tracking through every element kind, both integrators, all flags
    track_case('fodo_fived', lat('fodo.mad'), ufo.FIVED, 10, 2, ['x'], [-1],
               pool=np.full((2, 1), 1e-3))
    track_case('fodo_kick_6d', lat('fodo.mad'), ufo.KICK, 50, 16, six, [-1])
    track_case('fodo_kick_where', lat('fodo.mad'), ufo.KICK, 5, 8, six, [0, 0.5, 1.25, 2.75, -1])
    track_case('fodo_thick_where', lat('fodo.mad'), 0, 5, 8, six, [0, 0.5, 1.25, 2.75, -1])
    track_case('fodo2_thick_edges', lat('fodo2.mad'), 0, 20, 8, six, [-1])
    track_case('fodo2_kick_edges', lat('fodo2.mad'), ufo.KICK, 20, 8, six, [-1])
    track_case('alba_thick', lat('alba.mad'), 0, 10, 8, six, [-1])
    track_case('alba_kick', lat('alba.mad'), ufo.KICK, 10, 8, six, [-1])
    track_case('alba_kick_exact', lat('alba.mad'), ufo.KICK | ufo.EXACT, 10, 8, six, [-1])
    # FIVED pastes dp as a literal: the C compiler folds the thick maps' and
    # fringe edges' transcendentals (the HOWTO's own mode)
    four = ['x', 'px', 'y', 'py']
    track_case('alba_fived_thick', lat('alba.mad'), ufo.FIVED, 10, 8, four, [-1])
    track_case('alba_fived_thick_dp', lat('alba.mad'), ufo.FIVED, 10, 8, four, [-1], dp=1e-3)
    track_case('alba_linear_achro', lat('alba.mad'), ufo.LINEAR | ufo.ACHROMATIC, 3, 4, six, [-1])
    track_case('alba_achro_thick', lat('alba.mad'), ufo.ACHROMATIC, 3, 4, six, [-1])
    track_case('elements_kick', lat('elements.mad', 'TEST'), ufo.KICK, 30, 8, six, [-1, 1.5])
    track_case('elements_thick', lat('elements.mad', 'TEST'), 0, 30, 8, six, [-1, 1.5])
    track_case('rbend_thick', lat('bend.mad', 'RRING'), 0, 30, 8, six, [-1])
    track_case('rbend_kick', lat('bend.mad', 'RRING'), ufo.KICK, 30, 8, six, [-1])
    track_case('oct_kick', lat('oct.mad'), ufo.KICK, 30, 8, six, [-1], scale=1e-2)
    track_case('alba_kick_params', lat('alba.mad'), ufo.KICK, 5, 8,
               six + [('QF1', 'k1'), ('SD1', 'dx'), (5, 'dk3'), ('QD2', 'dk2s'), ('BE', 'e1')],
               [-1])
    track_case('alba_thick_params', lat('alba.mad'), 0, 5, 8,
               six + [('QF1', 'k1'), ('SD1', 'dx'), ('BE', 'angle'), ('BE', 'e1')], [-1])
    mixed = ufo.Line('l', [
        ufo.Drift('dr1', length=0.5), ufo.Aperture('ap', window='x*x + y*y < 1e-4'),
        ufo.Quadrupole('q', length=0.3, k1=1.2, slices=4),
        ufo.Wire('w', x=0.01, y=0.02, k=1e-5),
        ufo.Aperture('ap2', window='fabs(x) < 0.02 && fabs(y) < 0.005'),
        ufo.Drift('d2', length=0.5), ufo.Quadrupole('qd', length=0.3, k1=-1.2, slices=4),
        ufo.Multipole('m', knl=[0, 0, 3., 10., 1e3, 1e5], ksl=[0, 0.1, 0, 5., 0., 2e4], dx=1e-4),
        ufo.Octupole('o', length=0.2, k3=300., slices=3, dkn=[0., 0., 20.]),
        ufo.Sextupole('s', length=0.2, k2=40., k2s=7., slices=5, dx=2e-4, dy=-1e-4)])
    track_case('mixed_kick', mixed, ufo.KICK, 50, 32, six, [-1, 4.5], scale=5e-3)
    sa_case('mixed_sa', mixed, ufo.KICK, 200, np.random.default_rng(5).normal(size=(64, 5)) * 5e-3,
            six)
    # C1 ring (the benchmark's FODO) and C4-style error seeds through parameters
    c1 = W.c1_ring(ufo)
    track_case('c1_kick', c1, ufo.KICK, 100, 64, six, [-1], seed=11,
               pool=W.c1_beam(64, seed=11)[:, [0, 1, 2, 3, 5]])
    c1e = W.c1_ring(ufo, aperture=True)
    mags = [i for i, e in enumerate(c1e.flatten()) if type(e).__name__ in ('Quadrupole', 'Sbend')]
    params = six + [(i, a) for i in mags for a in ('dx', 'dy', 'dk2', 'dk2s')]
    rng = np.random.default_rng(7)
    n_seeds, per = 6, 8
    rows = []
    for s in range(n_seeds):
        vals = []
        for i in mags:
            e = c1e.flatten()[i]
            km = abs(e.k1) if type(e).__name__ == 'Quadrupole' else abs(e.angle / e.length)
            mo = 1 if type(e).__name__ == 'Quadrupole' else 0
            vals += [rng.normal(0, 50e-6), rng.normal(0, 50e-6),
                     rng.normal(0, 1e-3) * km / W.R0 ** (2 - mo),
                     rng.normal(0, 1e-3) * km / W.R0 ** (2 - mo)]
        rows.append(vals)
    beam = W.c1_beam(n_seeds * per, seed=12)[:, [0, 1, 2, 3, 5]] * 20
    pool = np.concatenate([beam, np.repeat(np.array(rows), per, axis=0)], axis=1)
    track_case('c1_seeds_kick', c1e, ufo.KICK, 30, n_seeds * per, params, [-1], pool=pool)
    # dynamic aperture on the C1 ring with aperture + dk2 errors
    c3 = W.c1_ring(ufo, aperture=True)
    rng = np.random.default_rng(13)
    for e in c3.flatten():
        if type(e).__name__ in ('Quadrupole', 'Sbend'):
            km = abs(e.k1) if type(e).__name__ == 'Quadrupole' else abs(e.angle / e.length)
            mo = 1 if type(e).__name__ == 'Quadrupole' else 0
            e.dx, e.dy = rng.normal(0, 50e-6), rng.normal(0, 50e-6)
            e.dkn = [0., 0., rng.normal(0, 5e-3) * km / W.R0 ** (2 - mo)]
            e.dks = [0., 0., rng.normal(0, 5e-3) * km / W.R0 ** (2 - mo)]
    grid = W.c3_grid(48, 48)[:, [0, 1, 2, 3, 5]]
    sa_case('c3_da_sa', c3, ufo.KICK, 512, grid, six)
    # HOWTO 12x12 ALBA stable-aperture example in FP64 (HOWTO.md:330-351)
    g = np.linspace(-0.04, 0.04, 12)
    xx, yy = np.meshgrid(g, g)
    sa_case('alba_sa_12x12', lat('alba.mad'), ufo.FIVED, 1000,
            np.stack([xx.ravel(), yy.ravel()], 1), ['x', 'y'])
    sa_case('alba_sa_12x12_kick', lat('alba.mad'), ufo.FIVED | ufo.KICK, 1000,
            np.stack([xx.ravel(), yy.ravel()], 1), ['x', 'y'])

    # --- optics: tunes, chromaticity by finite differences, thick vs kick, align
    def optics_case(name, line, flags, where, periodic=True, params=(), pval=None, attrs=None,
                    consumers=False):
        o = ufo.Optics(line, where=list(where), periodic=periodic, parameters=list(params),
                       flags=flags)
        if pval is not None:
            o.parameters[0] = pval
        if attrs:
            for k, v in attrs.items():
                setattr(o, k, v)
        o.run(threads=1)
        outs = {k: getattr(o, k) for k in ('track', 'bx', 'by', 'ax', 'ay', 'dx', 'dpx', 'dy',
                                           'dpy', 'mux', 'muy')}
        for k in ('qx', 'qy'):
            if hasattr(o, k):
                outs[k] = np.float64(getattr(o, k))
        if consumers:
            # the reference's host consumers of the optics output
            # (ufo/radiation.py, ufo/chroma.py)
            rad = ufo.emittance(o)
            for k in ('I1', 'I2', 'I4', 'I5', 'Jx', 'Jt', 'U0', 'Ex'):
                outs[f'rad_{k}'] = np.float64(getattr(rad, k))
            (dqx0, dqy0), (dqx, dqy) = ufo.chromaticity(o)
            outs['chroma'] = np.array([dqx0, dqy0, dqx, dqy], dtype=np.float64)
        add(name, 'optics', line, flags, dict(where=list(where), periodic=periodic,
                                              parameters=list(params),
                                              pval=None if pval is None else float(pval),
                                              attrs=attrs or {}), outs, {})
        return o

    alba = lat('alba.mad')
    optics_case('alba_optics_fp32', alba, ufo.LINEAR | ufo.ACHROMATIC, [])
    o64 = optics_case('alba_optics_fp64', lat('alba.mad'),
                      ufo.LINEAR | ufo.ACHROMATIC | ufo.DOUBLE_PRECISION, [])
    where_q = lat('alba.mad').find(lambda e: hasattr(e, 'k1') or hasattr(e, 'k2'))
    optics_case('alba_optics_where', lat('alba.mad'),
                ufo.LINEAR | ufo.ACHROMATIC | ufo.DOUBLE_PRECISION, where_q[:40])
    for tag, dpv in (('0', 0.0), ('1', 1e-4)):
        optics_case(f'alba_chroma_fd_{tag}', lat('alba.mad'), ufo.LINEAR | ufo.DOUBLE_PRECISION,
                    [], params=['dp'], pval=dpv)
    optics_case('alba_optics_propagate', lat('alba.mad'),
                ufo.LINEAR | ufo.ACHROMATIC | ufo.DOUBLE_PRECISION, [-1], periodic=False,
                attrs=dict(ax0=float(o64.ax[-1]), ay0=float(o64.ay[-1]), bx0=float(o64.bx[-1]),
                           by0=float(o64.by[-1]), dx0=float(o64.dx[-1]),
                           dpx0=float(o64.dpx[-1])))
    # radiation integrals and analytic chromaticity, as the reference's tests
    # call them (tests/radiation.py:17-21, tests/chroma.py:12-17)
    bends = lat('alba.mad').find(lambda e: hasattr(e, 'angle'))
    mags = lat('alba.mad').find(lambda e: hasattr(e, 'k1') or hasattr(e, 'k2'))
    for tag, fl in (('fp32', ufo.LINEAR | ufo.ACHROMATIC),
                    ('fp64', ufo.LINEAR | ufo.ACHROMATIC | ufo.DOUBLE_PRECISION)):
        optics_case(f'alba_radiation_{tag}', lat('alba.mad'), fl, bends, consumers=True)
        optics_case(f'alba_chroma_{tag}', lat('alba.mad'), fl, mags, consumers=True)
    ufo.DEFAULT_QUADRUPOLE_SLICES, ufo.DEFAULT_BEND_SLICES = 16, 48
    tk = lat('alba.mad')
    ufo.DEFAULT_QUADRUPOLE_SLICES, ufo.DEFAULT_BEND_SLICES = 8, 8
    optics_case('alba_kick_16_48', tk,
                ufo.LINEAR | ufo.ACHROMATIC | ufo.KICK | ufo.DOUBLE_PRECISION, [])
    al = ufo.Lattice(path=os.path.join(optics, 'align.mad'))
    al.QF.dx = 1e-4
    optics_case('align_fodo', al.FODO, ufo.LINEAR | ufo.ACHROMATIC | ufo.DOUBLE_PRECISION, [-1])
    optics_case('align_equiv', al.EQUIVALENT, ufo.LINEAR | ufo.ACHROMATIC | ufo.DOUBLE_PRECISION,
                [-1])

    # --- time-dependent user elements: subclasses overriding method() with C
    # text of `turn` (the two kickers of HOWTO.md:84-200, on the ALBA ring)
    class NLKGate(ufo.Multipole):
        def method(self, k1=None, **kwargs):
            k1 = k1 or self.knl[1]
            return super().method(k1=f'((turn == 20) ? {k1} : 0.)', **kwargs)

    class NLKPulse(ufo.Multipole):
        def __init__(self, label, t0=0., tau=0., **kwargs):
            super().__init__(label, **kwargs)
            self.tau = tau
            self.t0 = t0
            self.parameters += ['tau', 't0']

        def method(self, k1=None, t0=None, tau=None, **kwargs):
            k1, t0, tau = k1 or self.knl[1], t0 or self.t0, tau or self.tau
            k = (f'((turn >= {t0}) && (turn < {t0} + {tau}) )? '
                 f'{k1} * sin(3.1415 * ((float)turn - {t0}) / {tau}): 0.')
            return super().method(k1=f'({k})', **kwargs)

    class SkewKick(ufo.Multipole):
        # a sextupole term every third turn and a skew quadrupole that flips
        # sign after turn 4: higher orders and the skew Horner of a
        # time-dependent kick
        def method(self, k2=None, k1s=None, **kwargs):
            k2, k1s = k2 or self.knl[2], k1s or self.ksl[1]
            return super().method(k2=f'((turn % 3 == 0) ? {k2} : 0.)',
                                  k1s=f'((turn > 4) ? {k1s} : -{k1s})', **kwargs)

    rng = np.random.default_rng(7)
    betax, ex0 = 11.26, 4.3e-9
    for name, kicker, turns, n, params, extra in (
            ('nlk_gate', NLKGate('NLK', knl=[0., 5e-2]), 40, 32, ['x', 'px'], {}),
            ('nlk_pulse', NLKPulse('NLK', knl=[0., 5e-2], tau=1.5), 15, 28,
             ['x', 'px', ('NLK', 't0')], {'tau': 1.5}),
            ('skew_kick', SkewKick('SK', knl=[0., 0., 40.0], ksl=[0., 2e-2]), 12, 16,
             ['x', 'px'], {})):
        ring = lat('alba.mad')
        ring.insert(0, kicker)
        fl = ufo.FIVED | ufo.KICK | ufo.DOUBLE_PRECISION
        tr = ufo.Track(ring, flags=fl, turns=turns, particles=n, parameters=params, where=[-1])
        pool = np.zeros(tr.parameters.shape)
        pool[:, 0] = rng.normal(size=n) * np.sqrt(0.5 * betax * ex0)
        pool[:, 1] = rng.normal(size=n) * np.sqrt(0.5 * ex0 / betax)
        if len(params) > 2:  # the trigger-time scan of the HOWTO, one t0 per 4 particles
            pool[:, 2] = 5.0 + np.repeat(np.linspace(0., 1., 7, endpoint=False), 4)
        tr.parameters[:] = pool
        tr.run(threads=8)
        add(name, 'track', ring, fl, dict(turns=turns, particles=n,
                                          parameters=latjson.params_dump(params), where=[-1],
                                          dp=0.0, kicker=type(kicker).__name__, **extra),
            {'tracks': tr.tracks}, {'pool': pool})

    # --- closed orbit (reference: Nelder-Mead, 200 iterations)
    co_l = lat('alba.mad')
    co_l_d = {e.label: e for e in co_l.flatten()}
    co_l_d['QD1'].dx = 1e-4
    co_l_d['QD1'].dy = 1e-4
    co = ufo.ClosedOrbit(co_l, particles=1, flags=ufo.DOUBLE_PRECISION)
    co.run()
    add('alba_co_qd1', 'co', co_l, ufo.DOUBLE_PRECISION, dict(particles=1, parameters=[]),
        {'orbits': co.orbits}, {'pool': co.parameters})
    sx = lat('alba.mad')
    sexts = sx.find(lambda e: type(e).__name__ == 'Sextupole')[:12]
    prm = [(e, 'dx') for e in sexts]
    co = ufo.ClosedOrbit(sx, particles=len(sexts), flags=ufo.FIVED | ufo.DOUBLE_PRECISION,
                         parameters=prm)
    co.parameters[:, :] = np.identity(len(sexts)) * 1e-3
    co.run(threads=8)
    add('alba_co_sext_dx', 'co', sx, ufo.FIVED | ufo.DOUBLE_PRECISION,
        dict(particles=len(sexts), parameters=latjson.params_dump(prm)),
        {'orbits': co.orbits}, {'pool': co.parameters})

    # --- known-answer values from the reference's own tests (MAD-X runs)
    def floats(path, pattern):
        txt = open(os.path.join(ref, 'tests', path)).read()
        return [float(v) for v in re.findall(pattern, txt)]
    madx = {}
    txt = open(os.path.join(ref, 'tests', 'tracking.py')).read()
    arr = re.search(r'np\.array\(\[(.*?)\]\)', txt, re.S).group(1)
    madx['tracking_fodo_x'] = [float(v) for v in arr.replace('\n', ' ').split(',')]
    madx['alba_qx'], madx['alba_qy'] = floats('optics.py', r'q[xy] = ([-\d.]+)')
    madx['alba_dqx'], madx['alba_dqy'] = floats('optics3.py', r'dq[xy]_mad = ([-\d.]+)')
    rad = dict(re.findall(r'^\s*(I[1245]|alpha_c)\s*=\s*([-\d.e]+)',
                          open(os.path.join(ref, 'tests', 'radiation.py')).read(), re.M))
    for k, v in rad.items():
        madx[f'alba_{k}'] = float(v)
    madx['alba_dqx_sext'], madx['alba_dqy_sext'] = floats('chroma.py', r'dq[xy] = ([-\d.]+)')

    with open(os.path.join(HERE, 'cases.json'), 'w') as f:
        json.dump({'cases': cases, 'lattices': lattices, 'madx': madx,
                   'generator': 'tests/golden/make_golden.py (reference through oracle/refshim)'},
                  f)
    np.savez_compressed(os.path.join(HERE, 'golden.npz'), **arrays)
    print(f'{len(cases)} cases, {sum(a.nbytes for a in arrays.values()) / 1e6:.2f} MB raw')


if __name__ == '__main__':
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get('UFO_REFERENCE', '../reference'))
