"""CPU restatement of the build's 4th-order Yoshida integrator (flag YOSHIDA).
Test infrastructure only: the GPU tests compare the library against it.

PARITY UNPINNED: the reference has no Yoshida mode, so there is neither a
reference implementation nor golden vectors to pin this restatement to.  It
follows the published method (H. Yoshida, Phys. Lett. A 150 (1990) 262)
applied to the reference's teapot slice (ufo/methods.py:79-97): each of the N
slices of length h = L/N becomes

    drift c0 h, kick w0, drift c1 h, kick w1, drift c2 h, kick w2, drift c3 h

with w1 = 1/(2 - 2^(1/3)), w0 = 1 - 2 w1, c = (w1/2, (w0+w1)/2, (w0+w1)/2, w1/2).
A kick of weight w applies w times the slice kick of integrated strength
k L / N (the reference's complex Horner, ufo/methods.py:45-76, written here as
S(z) = sum_n (kn_n + i ks_n) z^n / n!, px -= o Re S, py += o Im S) and w times
its weak focusing px -= x angle^2 / (L N) (ufo/methods.py:84).  Alignment,
edges and apertures are the reference's (ufo/methods.py:22-26, :199-211,
ufo/elements.py:505-522).  Elements are read from their attributes, not from
the GPU compiler's tables; numpy, vectorised over particles.  KICK mode
without fringe fields or EXACT drifts (what the build supports).
"""
import math

import numpy as np

W1 = 1.0 / (2.0 - 2.0 ** (1.0 / 3.0))
W0 = 1.0 - 2.0 * W1
CS = (W1 / 2.0, (W0 + W1) / 2.0, (W0 + W1) / 2.0, W1 / 2.0)
DS = (W1, W0, W1)


def _strengths(e):
    """(normal, skew) integrated-per-metre coefficient lists of a thick magnet
    (ufo/elements.py method(): main strength added to the padded dkn; the
    sextupole/octupole skew list is dks alone, the reference's quirk)."""
    t = type(e).__name__
    kn, ks = list(e.dkn), list(e.dks)
    main = {'Quadrupole': (1, 'k1'), 'Sbend': (1, 'k1'), 'Rbend': (1, 'k1'),
            'Sextupole': (2, 'k2'), 'Octupole': (3, 'k3')}[t]
    order, attr = main
    while len(kn) <= order:
        kn.append(0.0)
    kn[order] += getattr(e, attr)
    return kn, ks


def _kick(x, y, kn, ks, scale, o, achro):
    z = x + 1j * y
    n = max(len(kn), len(ks))
    S = np.zeros_like(z)
    for j in range(n - 1, -1, -1):
        c = (kn[j] if j < len(kn) else 0.0) + 1j * (ks[j] if j < len(ks) else 0.0)
        S = S * z + c * scale / math.factorial(j)
    f = 1.0 if achro else o
    return -f * S.real, f * S.imag


def _teapot_yoshida(s, e, kn, ks, angle, o, achro):
    x, px, y, py = s
    L, N = float(e.length), int(e.slices)
    h = L / N
    W = angle * angle / (L * N) if angle else 0.0
    for _ in range(N):
        for i in range(3):
            x, y = x + px * CS[i] * h, y + py * CS[i] * h
            dpx, dpy = _kick(x, y, kn, ks, h, o, achro)
            px, py = px + DS[i] * dpx, py + DS[i] * dpy
            px = px - DS[i] * W * x
        x, y = x + px * CS[3] * h, y + py * CS[3] * h
    return x, px, y, py


def _edge(s, e, angle, edge, o, achro):
    x, px, y, py = s
    curv = angle / e.length * (1.0 if achro else o)
    t = math.tan(edge)
    return x, px + x * curv * t, y, py - y * curv * t


def track(line, coords, turns, achromatic=False):
    """Final coordinates [n, 6] after ``turns`` turns (lost particles: NaN x)."""
    c = np.array(coords, np.float64)
    x, px, y, py, dp = c[:, 0].copy(), c[:, 1].copy(), c[:, 2].copy(), c[:, 3].copy(), c[:, 5]
    o = 1.0 / (dp + 1.0)
    flat = line.flatten()
    for _ in range(turns):
        for e in flat:
            t = type(e).__name__
            if t == 'Marker':
                continue
            if t == 'Drift':
                x, y = x + px * e.length, y + py * e.length
                continue
            if t == 'Aperture':
                keep = eval(e.window, {'__builtins__': {}}, {'x': x, 'y': y})  # noqa: S307
                x = np.where(keep, x, np.nan)
                continue
            if t not in ('Quadrupole', 'Sbend', 'Rbend', 'Sextupole', 'Octupole'):
                raise NotImplementedError(t)
            x, y = x - e.dx, y - e.dy
            kn, ks = _strengths(e)
            s = (x, px, y, py)
            bend = t in ('Sbend', 'Rbend')
            angle = float(e.angle) if bend else 0.0
            if bend:
                s = _edge(s, e, angle, e.e1 + (angle / 2 if t == 'Rbend' else 0.0), o, achromatic)
            s = _teapot_yoshida(s, e, kn, ks, angle, o, achromatic)
            if bend:
                s = _edge(s, e, angle, e.e2 + (angle / 2 if t == 'Rbend' else 0.0), o, achromatic)
            x, px, y, py = s
            x, y = x + e.dx, y + e.dy
    out = c.copy()
    out[:, 0], out[:, 1], out[:, 2], out[:, 3] = x, px, y, py
    return out
