"""Gradients of closed orbit, tunes, chromaticity and multi-turn amplitudes
with respect to element strengths (quadrupole k1, sextupole k2, octupole k3).

The GPU side (csrc/diff.cu) is a tangent map and a hand-written adjoint of the
one-turn map; this module turns a compiled line into the differentiator's
opcode list and wires the kernels into ``torch.autograd.Function``s:

``OpticsFunction``      k -> (closed orbit x, px, y, py at dp = 0, Qx, Qy,
                        chromaticities dQx/dp, dQy/dp).  Closed orbit by Newton
                        iteration on the exact one-turn Jacobian; tunes from the
                        one-turn matrix at the closed orbit with the reference's
                        branch rule (ufo/optics.py:162-199); chromaticity by
                        central differences of the tunes in dp (the reference's
                        own method is a one-sided difference, tests/optics3.py).
                        Backward: implicit differentiation of the fixed point
                        F(z*) = z* plus the adjoint of the tangent-augmented map
                        (second order) at dp = 0 and +-h.
``AmplitudeFunction``   k -> final x^2 + y^2 of each particle after T turns;
                        backward: the checkpointed multi-turn adjoint.

The reference has no derivatives; its only Jacobian-like computation is the
finite difference of tunes in dp (tests/optics3.py:13-23) and the linear-map
columns tracked by Optics (ufo/optics.py:100-103).
"""
import math

import numpy as np

from . import compiler as C

D_NOP, D_DRIFT, D_TEAPOT, D_KICK, D_ALIGN, D_EDGE = range(6)
MAXC = 16


def _torch():
    import torch
    return torch


class DiffProgram:
    """Differentiator opcode list of a compiled line.

    ``values`` is one row of parameter values, or [S, P] rows (one per seed):
    the opcode list is shared and the constant table holds one row per seed."""

    def __init__(self, line, flags, parameters, values=None, dp_attrs=('k1', 'k2', 'k3')):
        parameters = list(parameters)
        self.parameters = parameters
        vals = np.zeros((1, max(1, len(parameters)))) if values is None else \
            np.atleast_2d(np.asarray(values, np.float64))
        if values is not None and vals.shape[1] != len(parameters):
            vals = vals.reshape(-1, len(parameters))
        prog = C.compile_line(line, flags, parameters, [], seed_values=vals)
        self.prog = prog
        flat = line.flatten() if hasattr(line, 'flatten') else list(line)
        # element index -> (parameter slot, coefficient order)
        slot = {}
        for i, p in enumerate(parameters):
            if not isinstance(p, tuple):
                raise ValueError('only lattice parameters (element, attribute) are differentiated')
            key, attr = p
            if attr not in dp_attrs:
                raise NotImplementedError(f'derivatives with respect to {attr!r}')
            idx = key if isinstance(key, int) else [j for j, e in enumerate(flat) if e.label == key]
            for j in (idx if isinstance(idx, list) else [idx]):
                slot[j] = (i, {'k1': 1, 'k2': 2, 'k3': 3}[attr])
        rows = [self._lower(prog, row, flat, slot) for row in prog.table]
        ops, kicks = rows[0][0], rows[0][2]
        self.ops = np.ascontiguousarray(np.array(ops, np.int32).reshape(-1, 8))
        self.tab = np.ascontiguousarray(np.array([r[1] + [0.0] for r in rows], np.float64))
        self.n_seeds = self.tab.shape[0]
        self.tab_stride = self.tab.shape[1]
        self.kicks_per_turn = kicks
        self.n_params = len(parameters)

    @staticmethod
    def _lower(prog, row, flat, slot):
        ops, tab = [], []
        kicks = 0
        for r, elem in zip(prog.ops, prog.op_elem):
            kind, fl, off = int(r[0]), int(r[1]), int(r[2])
            c = row[off:]
            achro = 1 if fl & C.F_ACHRO else 0
            if kind in (C.OP_NOP, C.OP_OBSERVE, C.OP_APERTURE):
                continue
            if kind == C.OP_DRIFT:
                if fl & C.F_EXACT:
                    raise NotImplementedError('exact drifts are not differentiated')
                form = int(r[3])
                L = c[0] if form == C.DF_MUL else c[0] * c[1] if form == C.DF_MUL2 else c[3]
                ops.append([D_DRIFT, 0, len(tab), 0, 0, -1, 0, 0])
                tab += [L]
            elif kind == C.OP_ALIGN:
                ops.append([D_ALIGN, 0, len(tab), 0, 0, -1, 0, 0])
                tab += [c[0] if fl & C.F_AX else 0.0, c[1] if fl & C.F_AY else 0.0]
            elif kind == C.OP_EDGE:
                if fl & C.F_RTPSI:
                    raise NotImplementedError('fringe-field edges with chromatic psi')
                ops.append([D_EDGE, 0, len(tab), 0, 0, -1, 0, achro])
                tab += [c[0], c[1] if fl & C.F_T1 else 0.0, c[2] if fl & C.F_T2 else 0.0]
            elif kind in (C.OP_TEAPOT, C.OP_KICK):
                tp = kind == C.OP_TEAPOT
                if tp:
                    N, nn, ns, mn, ms = (int(v) for v in r[3:8])
                    if fl & C.F_EXACT:
                        raise NotImplementedError('exact drifts are not differentiated')
                    Lo = c[0]
                    fi = (fl >> C.SH_FINNER) & 3
                    k = 1
                    if N > 1:
                        Li = c[1] if fi == C.DF_MUL else c[4]
                        k += 1 if fi == C.DF_MUL else 4
                    else:
                        Li = 0.0
                    ck = c[k:]
                else:
                    N = 1
                    nn, ns, mn, ms = (int(v) for v in r[3:7])
                    Lo = Li = 0.0
                    ck = c
                M = max(nn, ns, 1)
                if M > MAXC:
                    raise NotImplementedError(f'more than {MAXC} multipole orders')
                cr, ci = np.zeros(M), np.zeros(M)
                q = 0
                for j in range(nn):
                    if mn >> j & 1:
                        cr[j] = ck[q]
                        q += 1
                for j in range(ns):
                    if ms >> j & 1:
                        ci[j] = ck[q]
                        q += 1
                W = ck[q] if tp and fl & C.F_WEAK else 0.0
                ps, pm = slot.get(elem, (-1, 0))
                if pm >= M:  # the coefficient was truncated away (LINEAR): no effect
                    ps = -1
                if ps >= 0:
                    e = flat[elem]
                    dKdk = (float(e.length) / N) if tp else 1.0
                else:
                    dKdk = 0.0
                ops.append([D_TEAPOT if tp else D_KICK, 0, len(tab), N, M, ps, pm, achro])
                tab += [Lo, Li, W, dKdk] + list(cr) + list(ci)
                kicks += N
            else:
                raise NotImplementedError(f'{C.OP_NAMES[kind]} elements are not differentiated')
        return ops, tab, kicks


class DiffEngine:
    """Device copy of a DiffProgram and the two kernels."""

    def __init__(self, dprog, device=0):
        torch = _torch()
        from . import capi
        self.capi = capi
        self.lib = capi.load()
        self.dev = torch.device('cuda', device)
        self.p = dprog
        self.ops = torch.from_numpy(dprog.ops).to(self.dev)
        self.tab = torch.from_numpy(dprog.tab).to(self.dev)

    def _ptr(self, t):
        return self.capi.ptr(t.data_ptr()) if t is not None else None

    def forward(self, z0, o, turns, tangent=False, ck=None, seed=None):
        """z0 [J, 4], o [J], seed [J] (constant-table row of each job, default 0)
        -> (zT [J, 20] on host, state for ``reverse``)."""
        torch = _torch()
        z0 = torch.as_tensor(np.ascontiguousarray(z0, np.float64), device=self.dev)
        o = torch.as_tensor(np.ascontiguousarray(o, np.float64), device=self.dev)
        J = z0.shape[0]
        sd = None
        if seed is not None:
            seed = np.ascontiguousarray(seed, np.int32)
            if seed.shape != (J,) or seed.min(initial=0) < 0 or \
                    seed.max(initial=0) >= self.p.n_seeds:
                raise ValueError('seed must hold one valid table row per job')
            sd = torch.as_tensor(seed, device=self.dev)
        ck = ck or max(1, turns)
        nck = turns // ck + 1
        ckpt = torch.zeros((J, nck, 20), dtype=torch.float64, device=self.dev)
        zT = torch.zeros((J, 20), dtype=torch.float64, device=self.dev)
        rc = self.lib.ufo_diff_forward(
            self._ptr(self.ops), self.ops.shape[0], self._ptr(self.tab), self.p.tab_stride,
            self._ptr(sd), self.p.n_params, self.p.kicks_per_turn, J, self._ptr(z0), self._ptr(o),
            int(turns), int(ck), int(bool(tangent)), self._ptr(ckpt), self._ptr(zT), None)
        if rc:
            raise RuntimeError(f'ufo_diff_forward failed ({rc})')
        torch.cuda.synchronize(self.dev)
        return zT.cpu().numpy(), (ckpt, o, turns, ck, tangent, sd)

    def reverse(self, state, zbar, Tbar=None):
        """Cotangents of the final state -> (cotangent of z0 [J, 4],
        parameter cotangents [J, n_params])."""
        torch = _torch()
        ckpt, o, turns, ck, tangent, sd = state
        J = ckpt.shape[0]
        zbar = torch.as_tensor(np.ascontiguousarray(zbar, np.float64), device=self.dev)
        Tb = None
        if tangent:
            Tb = torch.as_tensor(np.ascontiguousarray(Tbar, np.float64).reshape(J, 16),
                                 device=self.dev)
        seg = torch.empty((J, ck, 20), dtype=torch.float64, device=self.dev)
        tape = torch.empty((J, max(1, self.p.kicks_per_turn), 10), dtype=torch.float64,
                           device=self.dev)
        zbar0 = torch.empty((J, 4), dtype=torch.float64, device=self.dev)
        pbar = torch.empty((J, max(1, self.p.n_params)), dtype=torch.float64, device=self.dev)
        rc = self.lib.ufo_diff_reverse(
            self._ptr(self.ops), self.ops.shape[0], self._ptr(self.tab), self.p.tab_stride,
            self._ptr(sd), self.p.n_params, self.p.kicks_per_turn, J, self._ptr(o), int(turns),
            int(ck), int(bool(tangent)),
            self._ptr(ckpt), self._ptr(zbar), self._ptr(Tb), self._ptr(seg), self._ptr(tape),
            self._ptr(zbar0), self._ptr(pbar), None)
        if rc:
            raise RuntimeError(f'ufo_diff_reverse failed ({rc})')
        torch.cuda.synchronize(self.dev)
        return zbar0.cpu().numpy(), pbar[:, :self.p.n_params].cpu().numpy()


# ----------------------------------------------------------------- optics

def tune_and_grad(M, plane):
    """Tune of one plane from the one-turn matrix with the reference's branch
    rule (ufo/optics.py:163-174, :185-196) and dQ/d(M_aa), dQ/d(M_bb)."""
    a = 0 if plane == 0 else 2
    c = (M[a, a] + M[a + 1, a + 1]) * 0.5
    if abs(c) > 1:
        return math.nan, 0.0
    s = math.copysign(math.sqrt(1 - c * c), M[a, a + 1])
    nu = math.atan2(s, c)
    if nu < 0:
        nu += 2 * math.pi
    dnu_dc = -1.0 / s
    return nu / (2 * math.pi), 0.5 * dnu_dc / (2 * math.pi)


def closed_orbits(engine, dps, z0=None, max_iter=30, seed=None):
    """Newton closed orbits at each dp (4D, one-turn map with dp fixed), job i
    on constant-table row ``seed[i]``.
    Returns (z* [len(dps), 4], J [len(dps), 4, 4], final residual [len(dps)])."""
    dps = np.asarray(dps, np.float64)
    n = len(dps)
    o = 1.0 / (dps + 1.0)
    z = np.zeros((n, 4)) if z0 is None else np.array(z0, np.float64)
    best = np.full(n, np.inf)
    zbest = z.copy()
    active = np.ones(n, bool)  # per-job stopping: a job's iterates do not depend on the batch
    for _ in range(max_iter):
        out, _ = engine.forward(z, o, 1, tangent=True, seed=seed)
        F = out[:, :4]
        J = out[:, 4:].reshape(n, 4, 4)
        res = F - z
        nrm = np.max(np.abs(res), axis=1)
        better = active & (nrm < best)
        best = np.where(better, nrm, best)
        zbest[better] = z[better]
        active = better & (nrm > 0)
        if not np.any(active):
            break
        dz = np.zeros_like(z)
        dz[active] = np.linalg.solve(J[active] - np.eye(4)[None], -res[active, :, None])[:, :, 0]
        z = np.where(active[:, None], z + dz, z)
    # the Jacobian at the final iterate
    out, _ = engine.forward(zbest, o, 1, tangent=True, seed=seed)
    return zbest, out[:, 4:].reshape(n, 4, 4), best


class OpticsModel:
    """Closed orbit, tunes and chromaticity of a line as functions of the
    element strengths named in ``parameters``."""

    def __init__(self, line, flags, parameters, h_dp=1e-5, device=0):
        self.line = line
        self.flags = flags
        self.parameters = list(parameters)
        self.h = h_dp
        self.device = device

    def engine(self, values):
        return DiffEngine(DiffProgram(self.line, self.flags, self.parameters, values),
                          self.device)

    def evaluate(self, values):
        eng = self.engine(values)
        dps = [0.0, self.h, -self.h]
        z, J, res = closed_orbits(eng, dps)
        q = np.array([[tune_and_grad(J[i], p)[0] for p in (0, 1)] for i in range(3)])
        xi = (q[1] - q[2]) / (2 * self.h)
        out = np.concatenate([z[0], q[0], xi])
        return out, (eng, z, J, dps)

    def evaluate_many(self, values):
        """evaluate() for S rows of parameter values in one batch of launches
        (the S x 3 closed-orbit problems run as one job list).  -> out [S, 8]."""
        values = np.atleast_2d(np.asarray(values, np.float64))
        S = values.shape[0]
        eng = self.engine(values)
        dps = np.tile([0.0, self.h, -self.h], S)
        seed = np.repeat(np.arange(S, dtype=np.int32), 3)
        z, J, _ = closed_orbits(eng, dps, seed=seed)
        q = np.array([[tune_and_grad(J[i], p)[0] for p in (0, 1)] for i in range(3 * S)])
        q = q.reshape(S, 3, 2)
        xi = (q[:, 1] - q[:, 2]) / (2 * self.h)
        return np.concatenate([z.reshape(S, 3, 4)[:, 0], q[:, 0], xi], axis=1)

    def vjp(self, saved, gbar):
        """Vector-Jacobian product of evaluate() for the 8 output cotangents."""
        eng, z, J, dps = saved
        gbar = np.asarray(gbar, np.float64)
        zco_bar = gbar[:4]
        qbar = gbar[4:6]
        xibar = gbar[6:8]
        Mbar = np.zeros((3, 4, 4))
        for i, w in ((0, 1.0), (1, 1.0 / (2 * self.h)), (2, -1.0 / (2 * self.h))):
            for p in (0, 1):
                coeff = (qbar[p] if i == 0 else 0.0) + (xibar[p] * w if i else 0.0)
                if coeff == 0.0:
                    continue
                _, dq = tune_and_grad(J[i], p)
                a = 0 if p == 0 else 2
                Mbar[i, a, a] += coeff * dq
                Mbar[i, a + 1, a + 1] += coeff * dq
        o = 1.0 / (np.asarray(dps) + 1.0)
        # (1) adjoint of the tangent-augmented one-turn map at fixed z*
        _, st = eng.forward(z, o, 1, tangent=True)
        v, ka = eng.reverse(st, np.zeros((3, 4)), Mbar.reshape(3, 16))
        # (2) implicit differentiation of F(z*) = z*: lambda = (I - J)^-T (zbar + v)
        zb = v.copy()
        zb[0] += zco_bar
        lam = np.linalg.solve(np.transpose(np.eye(4)[None] - J, (0, 2, 1)), zb[:, :, None])[:, :, 0]
        _, st = eng.forward(z, o, 1, tangent=False)
        _, kb = eng.reverse(st, lam)
        return (ka + kb).sum(axis=0)


def _function_classes():
    torch = _torch()

    class OpticsFunction(torch.autograd.Function):
        """k (float64 tensor of the parameter values) -> tensor[8]:
        closed orbit (x, px, y, py), Qx, Qy, dQx/dp, dQy/dp."""

        @staticmethod
        def forward(ctx, k, model):
            out, saved = model.evaluate(k.detach().cpu().numpy())
            ctx.model = model
            ctx.saved = saved
            return torch.as_tensor(out, dtype=torch.float64)

        @staticmethod
        def backward(ctx, g):
            kbar = ctx.model.vjp(ctx.saved, g.detach().cpu().numpy())
            return torch.as_tensor(kbar, dtype=torch.float64), None

    class AmplitudeFunction(torch.autograd.Function):
        """k -> x_T^2 + y_T^2 of every particle after ``turns`` turns
        (checkpoints every ``ck`` turns)."""

        @staticmethod
        def forward(ctx, k, model, coords, turns, ck):
            eng = model.engine(k.detach().cpu().numpy())
            coords = np.asarray(coords, np.float64)
            o = 1.0 / (coords[:, 5] + 1.0)
            zT, st = eng.forward(coords[:, :4], o, turns, tangent=False, ck=ck)
            ctx.eng, ctx.st, ctx.zT = eng, st, zT
            return torch.as_tensor(zT[:, 0] ** 2 + zT[:, 2] ** 2, dtype=torch.float64)

        @staticmethod
        def backward(ctx, g):
            g = g.detach().cpu().numpy()
            zT = ctx.zT
            zbar = np.zeros((zT.shape[0], 4))
            zbar[:, 0] = 2 * zT[:, 0] * g
            zbar[:, 2] = 2 * zT[:, 2] * g
            _, pbar = ctx.eng.reverse(ctx.st, zbar)
            return torch.as_tensor(pbar.sum(axis=0), dtype=torch.float64), None, None, None, None

    return OpticsFunction, AmplitudeFunction


_FUNCS = None


def functions():
    global _FUNCS
    if _FUNCS is None:
        _FUNCS = _function_classes()
    return _FUNCS


def optics(k, model):
    """Differentiable closed orbit / tunes / chromaticity (see OpticsFunction)."""
    return functions()[0].apply(k, model)


def amplitudes(k, model, coords, turns, ck=64):
    """Differentiable final amplitudes of a bunch (see AmplitudeFunction)."""
    return functions()[1].apply(k, model, coords, turns, ck)
