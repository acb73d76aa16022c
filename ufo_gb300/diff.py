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
from .flags import FMA

D_NOP, D_DRIFT, D_TEAPOT, D_KICK, D_ALIGN, D_EDGE, D_THICK = range(7)
KHDR = 6  # kick constants: Lo (entry), Li, W, dK/dk/pm!, dK/dk/(pm-1)!, Lx (exit), then a, b
DT_BEND = 1  # D_THICK flag: sector bend (weak focusing h^2 and the dispersion term)
DE_RTPSI = 1  # D_EDGE flag: fringe-field angle psi depends on the job's dp
# tape slots a thick element takes per turn (tangent mode stores the entry
# state and all 16 tangent entries: two slots of 10 fields)
THICK_SLOTS = 2


def thick_functions(K, L):
    """The thick-map functions of the focusing strength K (q'' = -K q) over a
    length L, for either sign of K, and their derivatives in K:
        C = cos(sqrt(K) L) (cosh for K < 0), Sw = sin(sqrt(K) L)/sqrt(K)
        (sinh(sqrt(-K) L)/sqrt(-K)), D1 = (1 - C)/K (the bend's dispersion
        function); dC = -L Sw/2, dSw = (L C - Sw)/(2K), dD1 = (L Sw/2 - D1)/K.
    Power series in u = K L^2 for |u| < 1 (no cancellation near K = 0),
    closed forms above.  Arrays broadcast.  The same arithmetic as the
    device code (csrc/diff.cu: thick_fns)."""
    K = np.asarray(K, np.float64)
    L = np.asarray(L, np.float64)
    u = K * L * L
    small = np.abs(u) < 1.0
    # series: sum over n of (-u)^n / (2n)!, /(2n+1)!, /(2n+2)!; derivative
    # series n (-1)^n u^(n-1) / (2n+1)! and / (2n+2)!
    c = np.zeros_like(u)
    sw = np.zeros_like(u)
    d1 = np.zeros_like(u)
    dsw = np.zeros_like(u)
    dd1 = np.zeros_like(u)
    us = np.where(small, u, 0.0)
    for n in range(13, -1, -1):
        sg = -1.0 if n % 2 else 1.0
        c = c * us + sg / math.factorial(2 * n)
        sw = sw * us + sg / math.factorial(2 * n + 1)
        d1 = d1 * us + sg / math.factorial(2 * n + 2)
        if n >= 1:
            dsw = dsw * us + sg * n / math.factorial(2 * n + 1)
            dd1 = dd1 * us + sg * n / math.factorial(2 * n + 2)
    C_s, Sw_s, D1_s = c, L * sw, L * L * d1
    dSw_s, dD1_s = L ** 3 * dsw, L ** 4 * dd1
    with np.errstate(invalid='ignore', divide='ignore'):
        w = np.sqrt(np.abs(K))
        foc = K > 0
        C_c = np.where(foc, np.cos(w * L), np.cosh(w * L))
        Sw_c = np.where(foc, np.sin(w * L), np.sinh(w * L)) / w
        D1_c = (1.0 - C_c) / K
        dSw_c = (L * C_c - Sw_c) / (2 * K)
        dD1_c = (0.5 * L * Sw_c - D1_c) / K
    C = np.where(small, C_s, C_c)
    Sw = np.where(small, Sw_s, Sw_c)
    D1 = np.where(small, D1_s, D1_c)
    dSw = np.where(small, dSw_s, dSw_c)
    dD1 = np.where(small, dD1_s, dD1_c)
    return C, Sw, D1, -0.5 * L * Sw, dSw, dD1


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
        # the differentiator has its own (fused) arithmetic: it takes the FMA-mode
        # program, whose plain drifts are folded into the magnets' outer drifts
        prog = C.compile_line(line, flags | FMA, parameters, [], seed_values=vals,
                              linearize=False)
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
        ops, tab, kicks = self._lower(prog, flat, slot)
        ops, tab = self._trim(np.array(ops, np.int32).reshape(-1, 8), tab)
        self.ops = np.ascontiguousarray(ops)
        self.tab = np.ascontiguousarray(tab)
        self.n_seeds = self.tab.shape[0]
        self.tab_stride = self.tab.shape[1]
        self.kicks_per_turn = kicks
        self.n_params = len(parameters)

    @staticmethod
    def _trim(ops, tab):
        """Drop trailing multipole orders that are zero in every seed (the
        reference pads coefficient lists with zeros), keeping the order a
        parameter scales; the constant table is repacked."""
        out_ops, cols = [], []
        for op in ops:
            kind, off, M, ps, pm = int(op[0]), int(op[2]), int(op[4]), int(op[5]), int(op[6])
            op = op.copy()
            op[2] = len(cols)
            if kind in (D_TEAPOT, D_KICK):
                h = KHDR
                hdr = list(range(off, off + h))
                a = tab[:, off + h:off + h + M]
                b = tab[:, off + h + M:off + h + 2 * M]
                nz = np.nonzero(np.any(a != 0, axis=0) | np.any(b != 0, axis=0))[0]
                Mt = max(int(nz.max()) + 1 if len(nz) else 1, pm + 1 if ps >= 0 else 1)
                op[4] = Mt
                cols += hdr + list(range(off + h, off + h + Mt)) + \
                    list(range(off + h + M, off + h + M + Mt))
            else:
                n = {D_DRIFT: 1, D_ALIGN: 2, D_EDGE: 6 if op[1] & DE_RTPSI else 3,
                     D_THICK: 3}.get(kind, 0)
                cols += list(range(off, off + n))
            out_ops.append(op)
        cols.append(tab.shape[1] - 1)
        return np.array(out_ops, np.int32).reshape(-1, 8), tab[:, cols]

    @staticmethod
    def _lower(prog, flat, slot):
        """Opcode list and constant columns for all seed rows of ``prog.table``
        at once: each constant is an array over the rows (or a scalar)."""
        T = prog.table
        ops, tab = [], []
        kicks = 0
        for r, elem in zip(prog.ops, prog.op_elem):
            kind, fl, off = int(r[0]), int(r[1]), int(r[2])

            def c(k, off=off):
                return T[:, off + k]

            achro = 1 if fl & C.F_ACHRO else 0
            if kind in (C.OP_NOP, C.OP_OBSERVE, C.OP_APERTURE):
                continue
            if kind == C.OP_DRIFT:
                if fl & C.F_EXACT:
                    raise NotImplementedError('exact drifts are not differentiated')
                form = int(r[3])
                L = c(0) if form == C.DF_MUL else c(0) * c(1) if form == C.DF_MUL2 else c(3)
                ops.append([D_DRIFT, 0, len(tab), 0, 0, -1, 0, 0])
                tab += [L]
            elif kind == C.OP_ALIGN:
                ops.append([D_ALIGN, 0, len(tab), 0, 0, -1, 0, 0])
                tab += [c(0) if fl & C.F_AX else 0.0, c(1) if fl & C.F_AY else 0.0]
            elif kind == C.OP_EDGE:
                if fl & C.F_RTPSI:
                    # fringe field with a chromatic angle: tan(psi) per job,
                    # psi = e - 2 (A o) fint' / cos(e) (1 + sin^2 e) (SLAC-75;
                    # ufo/methods.py:199-211)
                    ops.append([D_EDGE, DE_RTPSI, len(tab), 0, 0, -1, 0, achro])
                    tab += [c(0), c(1) if fl & C.F_T1 else 0.0, c(2), c(3), c(4), c(5)]
                else:
                    ops.append([D_EDGE, 0, len(tab), 0, 0, -1, 0, achro])
                    tab += [c(0), c(1) if fl & C.F_T1 else 0.0, c(2) if fl & C.F_T2 else 0.0]
            elif kind in (C.OP_TEAPOT, C.OP_KICK):
                if fl & C.F_YOSHIDA:
                    raise NotImplementedError('Yoshida elements are not differentiated')
                tp = kind == C.OP_TEAPOT
                if tp:
                    N, nn, ns, mn, ms = (int(v) for v in r[3:8])
                    if fl & C.F_EXACT:
                        raise NotImplementedError('exact drifts are not differentiated')
                    Lo = c(0)
                    fi = (fl >> C.SH_FINNER) & 3
                    k = 1
                    if N > 1:
                        Li = c(1) if fi == C.DF_MUL else c(4)
                        k += 1 if fi == C.DF_MUL else 4
                    else:
                        Li = 0.0
                else:
                    N = 1
                    nn, ns, mn, ms = (int(v) for v in r[3:7])
                    Lo = Li = 0.0
                    k = 0
                M = max(nn, ns, 1)
                fac = [float(math.factorial(n)) for n in range(M)]
                cr, ci = [0.0] * M, [0.0] * M
                q = k
                for j in range(nn):
                    if mn >> j & 1:
                        cr[j] = c(q) / fac[j]
                        q += 1
                for j in range(ns):
                    if ms >> j & 1:
                        ci[j] = c(q) / fac[j]
                        q += 1
                W = c(q) if tp and fl & C.F_WEAK else 0.0
                # exit outer drift: its own constant when a drift was merged into it
                qx = q + (1 if tp and fl & C.F_WEAK else 0)
                Lx = c(qx) if tp and fl & C.F_SPLITO else Lo
                ps, pm = slot.get(elem, (-1, 0))
                if pm >= M:  # the coefficient was truncated away (LINEAR): no effect
                    ps = -1
                if ps >= 0:
                    e = flat[elem]
                    dKdk = (float(e.length) / N) if tp else 1.0
                else:
                    dKdk = 0.0
                g0 = dKdk / fac[pm] if ps >= 0 else 0.0
                g1 = dKdk / fac[pm - 1] if ps >= 0 and pm >= 1 else 0.0
                ops.append([D_TEAPOT if tp else D_KICK, 0, len(tab), N, M, ps, pm, achro])
                tab += [Lo, Li, W, g0, g1, Lx] + cr + ci
                kicks += N
            elif kind in (C.OP_THICKQ, C.OP_THICKB):
                # the exact thick maps (ufo/methods.py:99-134, :136-196): per
                # plane q' = C q + Sw pq (+ dispersion), pq' = -K Sw q + C pq
                # with K_x = o (k1 + h^2), K_y = -o k1 (o = 1 when ACHROMATIC)
                if kind == C.OP_THICKQ:
                    k1, L, h, fl_d = c(0), c(1), 0.0, 0
                else:
                    h, k1, L, fl_d = c(0), c(1), c(2), DT_BEND
                ps, pm = slot.get(elem, (-1, 0))
                if pm != 1:  # thick maps read k1 only
                    ps = -1
                ops.append([D_THICK, fl_d, len(tab), 0, 0, ps, 1, achro])
                tab += [L, k1, h]
                kicks += THICK_SLOTS
            else:
                raise NotImplementedError(f'{C.OP_NAMES[kind]} elements are not differentiated')
        S = T.shape[0]
        tab = np.stack([np.broadcast_to(np.asarray(v, np.float64), (S,)) for v in tab + [0.0]],
                       axis=1) if tab else np.zeros((S, 1))
        return ops, tab, kicks


class DiffEngine:
    """Device copy of a DiffProgram and the two kernels.  Kernels run on
    torch's current stream; ``device_ms`` and ``launches`` accumulate their
    CUDA-event time and count."""

    def __init__(self, dprog, device=0, tape_budget=None):
        torch = _torch()
        from . import capi
        # bytes of device memory for the reverse tape; default: 40% of the free
        # memory at reverse time, at most 128 GiB (more memory = more
        # checkpoint segments re-tracked in parallel)
        self.tape_budget = tape_budget
        self.capi = capi
        self.lib = capi.load()
        self.dev = torch.device('cuda', device)
        self.p = dprog
        self.ops = torch.from_numpy(dprog.ops).to(self.dev)
        self.tab = torch.from_numpy(dprog.tab).to(self.dev)
        self.device_ms = 0.0
        self.launches = 0

    def _ptr(self, t):
        return self.capi.ptr(t.data_ptr()) if t is not None else None

    def _run(self, fn, name):
        torch = _torch()
        st = torch.cuda.current_stream(self.dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        rc = fn(self.capi.ptr(st.cuda_stream))
        e1.record(st)
        if rc:
            raise RuntimeError(f'{name} failed ({rc})')
        e1.synchronize()
        self.device_ms += e0.elapsed_time(e1)
        self.launches += 1

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
        ckpt = torch.zeros((nck, 20, J), dtype=torch.float64, device=self.dev)
        zT = torch.zeros((J, 20), dtype=torch.float64, device=self.dev)
        self._run(lambda st: self.lib.ufo_diff_forward(
            self._ptr(self.ops), self.ops.shape[0], self._ptr(self.tab), self.p.tab_stride,
            self._ptr(sd), self.p.n_params, self.p.kicks_per_turn, J, self._ptr(z0), self._ptr(o),
            int(turns), int(ck), int(bool(tangent)), self._ptr(ckpt), self._ptr(zT), st),
            'ufo_diff_forward')
        return zT.cpu().numpy(), (ckpt, o, turns, ck, tangent, sd)

    def reverse(self, state, zbar, Tbar=None, sum_jobs=False):
        """Cotangents of the final state -> (cotangent of z0 [J, 4],
        parameter cotangents [J, n_params], or their sum over jobs [n_params]
        with ``sum_jobs``)."""
        torch = _torch()
        ckpt, o, turns, ck, tangent, sd = state
        J = ckpt.shape[2]
        zbar = torch.as_tensor(np.ascontiguousarray(zbar, np.float64), device=self.dev)
        Tb = None
        if tangent:
            Tb = torch.as_tensor(np.ascontiguousarray(Tbar, np.float64).reshape(J, 16),
                                 device=self.dev)
        nf = 10 if tangent else 4
        seg_len = min(ck, turns)
        W = (J + 31) // 32  # the tape is warp-blocked: [turn][warp][kick][field][lane]
        seg_bytes = seg_len * max(1, self.p.kicks_per_turn) * nf * W * 32 * 8
        n_seg = (turns - 1) // ck + 1
        budget = self.tape_budget
        if budget is None:
            torch.cuda.empty_cache()  # cached but unused blocks count as free here
            free, _ = torch.cuda.mem_get_info(self.dev)
            budget = min(128 << 30, int(0.4 * free))
        if tangent:
            G = 1
        else:
            # segments taped at once: bounded by memory and by parallelism (the
            # taping pass runs two lanes per job; about 1.5 warps per SM
            # sub-partition fill the GPU, more only queue), then balanced so
            # the groups are equal
            smsp = 4 * torch.cuda.get_device_properties(self.dev).multi_processor_count
            warps_per_seg = -(-2 * J // 32)
            g_par = max(1, round(1.5 * smsp / warps_per_seg))
            G = int(max(1, min(n_seg, budget // max(1, seg_bytes), g_par)))
            groups = -(-n_seg // G)
            G = -(-n_seg // groups)
        tape = torch.empty((G * seg_len, W, max(1, self.p.kicks_per_turn), nf, 32),
                           dtype=torch.float64, device=self.dev)
        self.last_tape_segments = G
        zbar0 = torch.empty((J, 4), dtype=torch.float64, device=self.dev)
        pbar = torch.empty((max(1, self.p.n_params), J), dtype=torch.float64, device=self.dev)
        self._run(lambda st: self.lib.ufo_diff_reverse(
            self._ptr(self.ops), self.ops.shape[0], self._ptr(self.tab), self.p.tab_stride,
            self._ptr(sd), self.p.n_params, self.p.kicks_per_turn, J, self._ptr(o), int(turns),
            int(ck), int(bool(tangent)), self._ptr(ckpt), self._ptr(zbar), self._ptr(Tb),
            self._ptr(tape), G, self._ptr(zbar0), self._ptr(pbar), st), 'ufo_diff_reverse')
        pb = pbar[:self.p.n_params]
        pb = pb.sum(dim=1) if sum_jobs else pb.T
        return zbar0.cpu().numpy(), pb.cpu().numpy()


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
    element strengths named in ``parameters``; one or many rows of strengths
    (error seeds) at a time."""

    def __init__(self, line, flags, parameters, h_dp=1e-4, device=0):
        self.line = line
        self.flags = flags
        self.parameters = list(parameters)
        self.h = h_dp
        self.device = device

    def engine(self, values):
        return DiffEngine(DiffProgram(self.line, self.flags, self.parameters, values),
                          self.device)

    def evaluate_batch(self, values):
        """values [S, P] -> (out [S, 8], saved).  The S x 3 closed-orbit problems
        (dp = 0, +h, -h per row) run as one job list; each job stops on its own,
        so a row's result does not depend on the other rows."""
        values = np.atleast_2d(np.asarray(values, np.float64))
        S = values.shape[0]
        eng = self.engine(values)
        dps = np.tile([0.0, self.h, -self.h], S)
        seed = np.repeat(np.arange(S, dtype=np.int32), 3)
        z, J, _ = closed_orbits(eng, dps, seed=seed)
        q = np.array([[tune_and_grad(J[i], p)[0] for p in (0, 1)] for i in range(3 * S)])
        q = q.reshape(S, 3, 2)
        xi = (q[:, 1] - q[:, 2]) / (2 * self.h)
        out = np.concatenate([z.reshape(S, 3, 4)[:, 0], q[:, 0], xi], axis=1)
        return out, (eng, z, J, dps, seed, S)

    def evaluate(self, values):
        """One row of strengths -> (out [8], saved)."""
        out, saved = self.evaluate_batch(np.asarray(values, np.float64).reshape(1, -1))
        return out[0], saved

    def evaluate_many(self, values):
        return self.evaluate_batch(values)[0]

    def vjp(self, saved, gbar):
        """Vector-Jacobian products of evaluate_batch().  ``gbar`` holds output
        cotangents [8] (one row), [S, 8] or [S, R, 8] (R cotangent vectors per
        row, e.g. R = 8 unit vectors for the whole Jacobian); the result has the
        same leading shape with P parameter cotangents.  All S x R x 3 jobs run
        in one tangent-adjoint and one plain-adjoint launch pair."""
        eng, z, J, dps, seed, S = saved
        g = np.asarray(gbar, np.float64)
        lead = g.shape[:-1]
        G = g.reshape(S, -1, 8)
        R = G.shape[1]
        # xi = (Q(+h) - Q(-h)) / 2h: weights of the xi cotangent per dp job
        w = np.array([0.0, 1.0 / (2 * self.h), -1.0 / (2 * self.h)])
        # dQ/dc for every (row, dp) and plane
        dq = np.array([[tune_and_grad(J[i], p)[1] for p in (0, 1)] for i in range(3 * S)])
        dq = dq.reshape(S, 1, 3, 2)
        coeff = G[:, :, None, 6:8] * w[None, None, :, None]           # [S, R, 3, 2]
        coeff[:, :, 0] += G[:, :, 4:6]
        coeff = coeff * dq
        Mbar = np.zeros((S, R, 3, 4, 4))
        for p, a in ((0, 0), (1, 2)):
            Mbar[..., a, a] += coeff[..., p]
            Mbar[..., a + 1, a + 1] += coeff[..., p]
        jobs = (np.arange(S)[:, None, None] * 3 + np.arange(3)[None, None, :]) + \
            np.zeros((1, R, 1), np.int64)                                # [S, R, 3]
        jobs = jobs.reshape(-1)
        zj, Jj, sj = z[jobs], J[jobs], seed[jobs]
        o = 1.0 / (dps[jobs] + 1.0)
        # (1) adjoint of the tangent-augmented one-turn map at fixed z*
        _, st = eng.forward(zj, o, 1, tangent=True, seed=sj)
        v, ka = eng.reverse(st, np.zeros((len(jobs), 4)), Mbar.reshape(-1, 16))
        # (2) implicit differentiation of F(z*) = z*: lambda = (I - J)^-T (zbar + v)
        zb = v.reshape(S, R, 3, 4).copy()
        zb[:, :, 0] += G[:, :, :4]
        zb = zb.reshape(-1, 4)
        lam = np.linalg.solve(np.transpose(np.eye(4)[None] - Jj, (0, 2, 1)),
                              zb[:, :, None])[:, :, 0]
        _, st = eng.forward(zj, o, 1, tangent=False, seed=sj)
        _, kb = eng.reverse(st, lam)
        kbar = (ka + kb).reshape(S, R, 3, -1).sum(axis=2)
        return kbar.reshape(*lead, -1)


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
            _, pbar = ctx.eng.reverse(ctx.st, zbar, sum_jobs=True)
            return torch.as_tensor(pbar, dtype=torch.float64), None, None, None, None

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
