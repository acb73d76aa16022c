"""Synthetic lattices and beams of the benchmark workloads (seeded, numpy RNG).

Every builder takes the element module ``m`` (this package, or any module with
the same element classes) so that identical lattices can be built for
cross-checks.

C1  plain FODO ring: 16 cells [QF(0.3, +1.2), D 1.0, B(1.5, 2pi/32), D 1.0,
    QD(0.3, -1.2), D 1.0, B, D 1.0], 4 teapot slices, 128 elements.
C2  light-source-like ring, 32 cells of 4 bends (1.38 m, 2pi/128), 10 quads
    (0.25 m, |k1| ~ U(0.8, 2.2), alternating sign), 6 sextupoles (0.2 m,
    |k2| ~ U(20, 60), SF > 0, SD < 0), 11 drifts and a 10 mm circular
    aperture: 32 elements per cell, 1024 in the ring.  The magnets alone
    need 9.22 m per cell, more than a 268.8 m circumference allows
    (8.4 m per cell), so cells are 12 m (384 m ring).  One cell's strengths
    are drawn from a seeded RNG (redrawn until the cell is linearly stable in
    both planes at dp = 0 and +-1%) and repeated 32 times.
C3  dynamic-aperture grid on the C1 ring with C4-style errors of seed 0 and a
    10 mm circular aperture per cell: 256 x 256 polar grid, r in [0, 25 mm],
    theta in [0, pi/2], dp in {-2%, 0, +2%}.
C4  error seeds of the C1 ring: dx, dy ~ N(0, 50 um) per magnet; normal and
    skew errors of MAD orders 3..6 (this code's indices 2..5),
    dk_j = eps * K_main / r0^(j - m), eps ~ N(0, 1e-4), r0 = 10 mm, m the
    main order; particles per seed log-uniform in [256, 8192], turns uniform
    in [1000, 4096].
"""
import math

import numpy as np

R0 = 0.01          # reference radius of the relative multipole errors [m]
APERTURE = 'x*x + y*y < 1e-4'


def c1_ring(m, slices=4, aperture=False, errors=None):
    """C1 FODO ring.  ``errors``: dict label -> {attr: value} applied per
    magnet (C4 seeds); ``aperture`` adds a 10 mm aperture after each QF."""
    cells = []
    ang = 2 * math.pi / 32
    for c in range(16):
        el = [m.Quadrupole(f'QF{c}', length=0.3, k1=1.2, slices=slices),
              m.Drift(f'D{c}a', length=1.0),
              m.Sbend(f'B{c}a', length=1.5, angle=ang, slices=slices),
              m.Drift(f'D{c}b', length=1.0),
              m.Quadrupole(f'QD{c}', length=0.3, k1=-1.2, slices=slices),
              m.Drift(f'D{c}c', length=1.0),
              m.Sbend(f'B{c}b', length=1.5, angle=ang, slices=slices),
              m.Drift(f'D{c}d', length=1.0)]
        if aperture:
            el.insert(1, m.Aperture(f'AP{c}', window=APERTURE))
        cells.extend(el)
    if errors:
        for e in cells:
            for a, v in errors.get(e.label, {}).items():
                setattr(e, a, v)
    return m.Line('RING', cells)


def c1_magnets(line):
    return [e for e in line.flatten() if type(e).__name__ in ('Quadrupole', 'Sbend')]


def c4_error_names():
    """Per-magnet attributes that carry C4 errors."""
    names = ['dx', 'dy']
    for j in range(2, 6):
        names += [f'dk{j}', f'dk{j}s']
    return names


def c4_seed_errors(rng, magnets):
    """One C4 error seed: {label: {attr: value}}."""
    out = {}
    for e in magnets:
        if type(e).__name__ == 'Quadrupole':
            kmain, mo = abs(e.k1), 1
        else:
            kmain, mo = abs(e.angle / e.length), 0
        d = {'dx': rng.normal(0, 50e-6), 'dy': rng.normal(0, 50e-6),
             'dkn': [0.0] * 6, 'dks': [0.0] * 6}
        for j in range(2, 6):
            d['dkn'][j] = rng.normal(0, 1e-4) * kmain / R0 ** (j - mo)
            d['dks'][j] = rng.normal(0, 1e-4) * kmain / R0 ** (j - mo)
        out[e.label] = d
    return out


def c4_parameters(line):
    """Reference-style parameter list binding every C4 error of every magnet
    (by flat index) -- the seed table columns."""
    flat = line.flatten()
    params = []
    for i, e in enumerate(flat):
        if type(e).__name__ in ('Quadrupole', 'Sbend'):
            params += [(i, a) for a in c4_error_names()]
    return params


def c4_seed_rows(line, n_seeds, seed=4):
    """[n_seeds, P] values for c4_parameters(line)."""
    rng = np.random.default_rng(seed)
    flat = line.flatten()
    mags = [(i, e) for i, e in enumerate(flat) if type(e).__name__ in ('Quadrupole', 'Sbend')]
    rows = np.zeros((n_seeds, len(mags) * 10))
    for s in range(n_seeds):
        errs = c4_seed_errors(rng, [e for _, e in mags])
        col = 0
        for _, e in mags:
            d = errs[e.label]
            rows[s, col] = d['dx']
            rows[s, col + 1] = d['dy']
            col += 2
            for j in range(2, 6):
                rows[s, col] = d['dkn'][j]
                rows[s, col + 1] = d['dks'][j]
                col += 2
    return rows


def c4_sizes(n_seeds=512, seed=44):
    rng = np.random.default_rng(seed)
    parts = np.exp(rng.uniform(math.log(256), math.log(8192), n_seeds)).astype(np.int64)
    turns = rng.integers(1000, 4097, n_seeds)
    return parts, turns


def gaussian_beam(n, sx, spx, sy, spy, sdp, seed=1):
    rng = np.random.default_rng(seed)
    c = np.zeros((n, 6))
    c[:, 0] = rng.normal(0, sx, n)
    c[:, 1] = rng.normal(0, spx, n)
    c[:, 2] = rng.normal(0, sy, n)
    c[:, 3] = rng.normal(0, spy, n)
    c[:, 5] = rng.normal(0, sdp, n)
    return c


def c1_beam(n=1024, seed=1):
    return gaussian_beam(n, 1e-4, 1e-5, 1e-4, 1e-5, 1e-3, seed)


def c2_beam(n=65536, seed=2):
    return gaussian_beam(n, 50e-6, 5e-6, 5e-6, 0.5e-6, 1e-3, seed)


def c3_grid(nr=256, nt=256, dps=(-0.02, 0.0, 0.02)):
    r = np.linspace(0, 0.025, nr)
    t = np.linspace(0, math.pi / 2, nt)
    rr, tt = np.meshgrid(r, t, indexing='ij')
    out = []
    for dp in dps:
        c = np.zeros((nr * nt, 6))
        c[:, 0] = (rr * np.cos(tt)).ravel()
        c[:, 2] = (rr * np.sin(tt)).ravel()
        c[:, 5] = dp
        out.append(c)
    return np.concatenate(out)


def c3_ring(m, slices=4):
    """C1 ring + 10 mm aperture after each QF + the C4 errors of seed 0."""
    base = c1_ring(m, slices=slices, aperture=True)
    rng = np.random.default_rng(4)
    errs = c4_seed_errors(rng, c1_magnets(base))
    for e in base.flatten():
        if e.label in errs:
            d = errs[e.label]
            e.dx, e.dy = d['dx'], d['dy']
            e.dkn, e.dks = list(d['dkn']), list(d['dks'])
    return base


# ----------------------------------------------------------------- C2

def _c2_cell(m, c, rng, slices):
    kq = rng.uniform(0.8, 2.2, 10)
    ks = rng.uniform(20.0, 60.0, 6)
    sgn = [1 if i % 2 == 0 else -1 for i in range(10)]
    ang = 2 * math.pi / 128
    dl = (12.0 - (4 * 1.38 + 10 * 0.25 + 6 * 0.2)) / 11
    q = [m.Quadrupole(f'Q{c}_{i}', length=0.25, k1=sgn[i] * kq[i], slices=slices) for i in range(10)]
    s = [m.Sextupole(f'S{c}_{i}', length=0.2, k2=(1 if i % 2 == 0 else -1) * ks[i], slices=slices)
         for i in range(6)]
    b = [m.Sbend(f'B{c}_{i}', length=1.38, angle=ang, slices=slices) for i in range(4)]
    d = [m.Drift(f'D{c}_{i}', length=dl) for i in range(11)]
    seq = [q[0], d[0], s[0], b[0], d[1], q[1], s[1], d[2], q[2], b[1], d[3], q[3], s[2], d[4],
           q[4], d[5], q[5], s[3], d[6], q[6], b[2], d[7], q[7], s[4], d[8], q[8], b[3], d[9],
           s[5], q[9], d[10], m.Aperture(f'AP{c}', window=APERTURE)]
    return seq


def _cell_stable(cell_line, dp):
    """|trace|/2 < 1 in both planes of the cell's linear map (finite
    differences of a pure-Python pass through the teapot-sliced cell)."""
    M = _linear_map(cell_line, dp)
    cx = (M[0, 0] + M[1, 1]) / 2
    cy = (M[2, 2] + M[3, 3]) / 2
    return abs(cx) < 0.98 and abs(cy) < 0.98


def _linear_map(line, dp):
    """4x4 linear map of a teapot-sliced line at energy offset dp (drifts,
    quadrupole kicks scaled by 1/(1+dp), bend weak focusing; sextupoles and
    apertures have no linear part on the dp-independent zero orbit)."""
    o = 1.0 / (1.0 + dp)
    M = np.eye(4)

    def drift(L):
        D = np.eye(4)
        D[0, 1] = D[2, 3] = L
        return D

    for e in line.flatten():
        t = type(e).__name__
        if t == 'Drift':
            M = drift(e.length) @ M
        elif t in ('Quadrupole', 'Sbend'):
            N, L = e.slices, e.length
            k = getattr(e, 'k1', 0.0) * L / N * o
            w = (e.angle ** 2 * L / N / L / L) if t == 'Sbend' else 0.0
            K = np.eye(4)
            K[1, 0] = -k - w
            K[3, 2] = k
            outer = L / (2 * (1 + N))
            inner = (L - 2 * outer) / (N - 1)
            S = drift(outer)
            for i in range(N):
                S = K @ S
                S = (drift(inner) if i < N - 1 else drift(outer)) @ S
            M = S @ M
        elif t == 'Sextupole':
            M = drift(e.length) @ M
    return M


def c2_ring(m, seed=2, slices=4):
    """C2 ring (see module docstring).  One cell's strengths are drawn (and
    redrawn until the cell is stable at dp = 0, +-1%) and the cell is repeated
    32 times, so the ring is stable whenever the cell is (32 different random
    cells are almost never stable as a product)."""
    import ufo_gb300 as U
    rng = np.random.default_rng(seed)
    for _ in range(1000):
        st = rng.bit_generator.state
        probe = U.Line('cell', _c2_cell(U, 0, rng, slices))
        if all(_cell_stable(probe, dp) for dp in (-0.01, 0.0, 0.01)):
            break
    else:
        raise RuntimeError('no stable C2 cell found')
    cells = []
    for c in range(32):
        rng.bit_generator.state = st
        cells.extend(_c2_cell(m, c, rng, slices))
    return m.Line('RING', cells)


# ----------------------------------------------------------------- C5

def c5_ring(m, seed=5, slices=4):
    """C5: the C2 ring with one C4-style error seed on every magnet (dx, dy ~
    N(0, 50 um); normal and skew errors of MAD orders 3..6 relative to the
    main field at r0 = 10 mm)."""
    ring = c2_ring(m, slices=slices)
    rng = np.random.default_rng(seed)
    for e in ring.flatten():
        t = type(e).__name__
        if t not in ('Quadrupole', 'Sbend', 'Sextupole'):
            continue
        if t == 'Quadrupole':
            kmain, mo = abs(e.k1), 1
        elif t == 'Sextupole':
            kmain, mo = abs(e.k2), 2
        else:
            kmain, mo = abs(e.angle / e.length), 0
        e.dx, e.dy = rng.normal(0, 50e-6), rng.normal(0, 50e-6)
        e.dkn = [0.0] * 6
        e.dks = [0.0] * 6
        for j in range(2, 6):
            e.dkn[j] = rng.normal(0, 1e-4) * kmain / R0 ** (j - mo)
            e.dks[j] = rng.normal(0, 1e-4) * kmain / R0 ** (j - mo)
    return ring


def c5_parameters(ring):
    """The 320 quadrupole k1 and 192 sextupole k2 of the C5 ring (flat index,
    attribute) and their values."""
    flat = ring.flatten()
    q = [(i, 'k1') for i, e in enumerate(flat) if type(e).__name__ == 'Quadrupole']
    s = [(i, 'k2') for i, e in enumerate(flat) if type(e).__name__ == 'Sextupole']
    vals = [flat[i].k1 for i, _ in q] + [flat[i].k2 for i, _ in s]
    return q + s, np.array(vals, dtype=np.float64)
