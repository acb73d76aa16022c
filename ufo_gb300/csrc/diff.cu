// diff.cu -- tangent map and hand-written adjoint of the one-turn map.
//
// Differentiation runs on its own opcode list (built by ufo_gb300/diff.py from
// the compiled line): drifts, teapot elements, thin kicks, alignments, edges
// (with a fringe angle that may depend on dp) and the exact thick quadrupole
// and sector-bend maps.  Every kick of the reference (ufo/methods.py:45-76, the
// Horner scheme) is the complex polynomial
//     S(z) = o * sum_n (a_n + i b_n) z^n,   z = x + i y,
//     a_n = kn_n / n!,  b_n = ks_n / n!,
//     px -= Re S,   py += Im S,
// so its derivatives follow from S' and S'' (Cauchy-Riemann); one Horner pass
// gives S, S' and S''/2 together.  A teapot slice is kick, weak focusing
// (px -= W x), drift.  Element strengths enter linearly: one parameter per
// element scales coefficient `pm`; the table carries dK/dk / pm! and
// dK/dk / (pm-1)! for the S and S' terms.
//
// diff_forward: z (and optionally the 4x4 tangent T = dz/dz0) through `turns`
//   turns, writing the state (and T) every `ck` turns as checkpoints.
// Reverse pass, given the output cotangents zbar (and Tbar), over the
//   checkpoint segments from the last to the first:
//   * plain (multi-turn) mode: diff_tape re-tracks G segments at once
//     (G x J independent jobs: the segments only need their checkpoints) onto
//     a "rich" tape holding x, y and S'(z) at every kick; diff_reverse_plain
//     then walks those G segments backwards, job by job, with the cheap
//     reverse kick the stored S' allows.  The cotangent state is carried in
//     zbar0 from one group of segments to the next.
//   * tangent mode (optics, one turn): diff_reverse re-tracks each segment
//     onto a tape of x, y and the x/y rows of T and reverses it in one kernel.
//   Both accumulate the cotangent of the start state and of every element
//   parameter.
// Per-job buffers that grow with the work (checkpoints, tape, parameter
// cotangents) are laid out job-fastest, so a warp's 32 jobs touch 32
// consecutive doubles.  Arithmetic is FP64 with fused multiply-adds (gradients
// need FP64 accuracy, not the reference's rounding).  One thread per job.
#include <cuda_runtime.h>

#include <cstdint>

namespace ufo_diff {

enum : int { D_NOP = 0, D_DRIFT, D_TEAPOT, D_KICK, D_ALIGN, D_EDGE, D_THICK };
constexpr int KHDR = 6;   // kick constants: Lo, Li, W, g0, g1, Lx (exit), then a[M], b[M]
constexpr int DT_BEND = 1;      // D_THICK flag: sector bend (h^2 focusing, dispersion term)
constexpr int DE_RTPSI = 1;     // D_EDGE flag: fringe angle psi depends on the job's dp
constexpr int THICK_SLOTS = 2;  // tape slots of a thick element per turn

struct DOp {
  int kind, flags, toff, N, M, pslot, pm, achro;
};

struct DiffArgs {
  const DOp *ops;
  int n_ops;
  const double *tab;      // constants, [n_seeds][tab_stride]
  const int32_t *seed;    // [job] constant-table row, or null (row 0)
  int64_t tab_stride;
  int n_params;
  int kicks_per_turn;
  int n_jobs;
  const double *z0;       // [job][4]
  const double *o;        // [job] 1/(1+dp)
  int turns, ck;          // turns, checkpoint interval
  int tangent;            // propagate T
  double *ckpt;           // [turns/ck + 1][20][job]
  double *zT;             // [job][20] final state (+T)
  const double *zbar;     // [job][4] output cotangents
  const double *Tbar;     // [job][16] (tangent only)
  double *tape;           // [G*ck][warp][kicks_per_turn][nf][lane], nf = 10 (tangent) or 4
  double *zbar0;          // [job][4] cotangent of the start state
  double *pbar;           // [n_params][job]
};

struct St {
  double x, px, y, py;
  double T[16];  // rows x, px, y, py; columns = start coordinates
};

// S(z)/o, S'(z)/o and S''(z)/(2o) by one Horner pass over the power series
// (ND = highest derivative wanted)
template <int ND>
__device__ __forceinline__ void series(const double *__restrict__ a, int M, double x, double y,
                                       double &s0r, double &s0i, double &s1r, double &s1i,
                                       double &s2r, double &s2i) {
  const double *b = a + M;
  s0r = __ldg(a + M - 1);
  s0i = __ldg(b + M - 1);
  s1r = s1i = s2r = s2i = 0.0;
  for (int n = M - 2; n >= 0; --n) {
    if (ND >= 2) {
      const double tr = fma(s2r, x, fma(-s2i, y, s1r));
      s2i = fma(s2r, y, fma(s2i, x, s1i));
      s2r = tr;
    }
    if (ND >= 1) {
      const double tr = fma(s1r, x, fma(-s1i, y, s0r));
      s1i = fma(s1r, y, fma(s1i, x, s0i));
      s1r = tr;
    }
    const double tr = fma(s0r, x, fma(-s0i, y, __ldg(a + n)));
    s0i = fma(s0r, y, fma(s0i, x, __ldg(b + n)));
    s0r = tr;
  }
}

__device__ __forceinline__ void fwd_drift(St &s, double L, bool tangent) {
  s.x = fma(s.px, L, s.x);
  s.y = fma(s.py, L, s.y);
  if (tangent)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      s.T[j] = fma(s.T[4 + j], L, s.T[j]);
      s.T[8 + j] = fma(s.T[12 + j], L, s.T[8 + j]);
    }
}

__device__ __forceinline__ void fwd_weak(St &s, double W, bool tangent) {
  s.px = fma(-W, s.x, s.px);
  if (tangent)
#pragma unroll
    for (int j = 0; j < 4; ++j) s.T[4 + j] = fma(-W, s.T[j], s.T[4 + j]);
}

__device__ __forceinline__ void fwd_kick(St &s, const double *a, int M, double o, bool tangent) {
  double sr, si, ar, ai, br, bi;
  if (tangent) {
    series<1>(a, M, s.x, s.y, sr, si, ar, ai, br, bi);
    ar *= o;
    ai *= o;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const double dx = s.T[j], dy = s.T[8 + j];
      s.T[4 + j] -= fma(ar, dx, -ai * dy);
      s.T[12 + j] += fma(ai, dx, ar * dy);
    }
  } else {
    series<0>(a, M, s.x, s.y, sr, si, ar, ai, br, bi);
  }
  s.px = fma(-o, sr, s.px);
  s.py = fma(o, si, s.py);
}

// The exact thick maps (ufo/methods.py:99-134 quadrupole, :136-196 sector
// bend) per plane: q' = C q + Sw pq + disp D1, pq' = -K Sw q + C pq + disp Sw,
// with the plane's focusing strength K (q'' = -K q; K_x = o (k1 + h^2),
// K_y = -o k1, o = 1 when achromatic), C = cos(sqrt(K) L) (cosh for K < 0),
// Sw = sin(sqrt(K) L) / sqrt(K) (sinh), D1 = (1 - C) / K, and the bend's
// horizontal dispersion disp = dp h o.  Power series in u = K L^2 for
// |u| < 1 (no cancellation near K = 0), closed forms above; the derivatives
// in K are dC = -L Sw / 2, dSw = (L C - Sw) / (2K), dD1 = (L Sw / 2 - D1) / K.
// Same arithmetic as ufo_gb300/diff.py: thick_functions.
template <bool DERIV>
__device__ __forceinline__ void thick_fns(double K, double L, double &C, double &Sw, double &D1,
                                          double &dC, double &dSw, double &dD1) {
  const double u = K * L * L;
  if (fabs(u) < 1.0) {
    // Horner over n = 13..0 of (-u)^n / (2n)!, / (2n+1)!, / (2n+2)! (and
    // n (-1)^n u^(n-1) / (2n+1)!, / (2n+2)! for the derivatives)
    double c = 0.0, sw = 0.0, d1 = 0.0, ds = 0.0, dd = 0.0;
    double f2n = 1.0;  // (2n)! for n = 13, built downwards from the top
#pragma unroll
    for (int k = 1; k <= 26; ++k) f2n *= k;
#pragma unroll
    for (int n = 13; n >= 0; --n) {
      const double sg = (n & 1) ? -1.0 : 1.0;
      const double i0 = sg / f2n;                              // 1/(2n)!
      const double i1 = i0 / (2 * n + 1);                      // 1/(2n+1)!
      const double i2 = i1 / (2 * n + 2);                      // 1/(2n+2)!
      c = fma(c, u, i0);
      sw = fma(sw, u, i1);
      d1 = fma(d1, u, i2);
      if (DERIV && n >= 1) {
        ds = fma(ds, u, n * i1);
        dd = fma(dd, u, n * i2);
      }
      if (n > 0) f2n /= static_cast<double>((2 * n) * (2 * n - 1));
    }
    C = c;
    Sw = L * sw;
    D1 = L * L * d1;
    if (DERIV) {
      dSw = L * L * L * ds;
      dD1 = L * L * L * L * dd;
    }
  } else {
    const double w = sqrt(fabs(K));
    if (K > 0) {
      double sn, cs;
      sincos(w * L, &sn, &cs);
      C = cs;
      Sw = sn / w;
    } else {
      C = cosh(w * L);
      Sw = sinh(w * L) / w;
    }
    D1 = (1.0 - C) / K;
    if (DERIV) {
      dSw = (L * C - Sw) / (2.0 * K);
      dD1 = (0.5 * L * Sw - D1) / K;
    }
  }
  if (DERIV) dC = -0.5 * L * Sw;
}

// one plane of a thick element forward; with `tangent` the plane's two
// tangent rows tq, tp (4 columns each) too
__device__ __forceinline__ void thick_plane_fwd(double &q, double &pq, double *tq, double *tp,
                                                double K, double L, double disp, bool tangent) {
  double C, Sw, D1, dC, dSw, dD1;
  thick_fns<false>(K, L, C, Sw, D1, dC, dSw, dD1);
  const double A = -K * Sw;
  const double q0 = q;
  q = fma(C, q0, fma(Sw, pq, disp * D1));
  pq = fma(A, q0, fma(C, pq, disp * Sw));
  if (tangent)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const double t = tq[j];
      tq[j] = fma(C, t, Sw * tp[j]);
      tp[j] = fma(A, t, C * tp[j]);
    }
}

// reverse of one plane of a thick element at the entry state (q, pq) and
// entry tangent rows (tq, tp; tangent mode): cotangents (qb, pqb) and the
// tangent-row cotangents (bq, bp) are mapped back through the transposed map;
// returns the cotangent of the plane's focusing strength K
__device__ __forceinline__ double thick_plane_rev(double &qb, double &pqb, double *bq, double *bp,
                                                  const double *tq, const double *tp, double q,
                                                  double pq, double K, double L, double disp,
                                                  bool tangent) {
  double C, Sw, D1, dC, dSw, dD1;
  thick_fns<true>(K, L, C, Sw, D1, dC, dSw, dD1);
  const double A = -K * Sw, dA = fma(-K, dSw, -Sw);
  double Kb = fma(qb, fma(dC, q, fma(dSw, pq, disp * dD1)),
                  pqb * fma(dA, q, fma(dC, pq, disp * dSw)));
  if (tangent)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      Kb = fma(bq[j], fma(dC, tq[j], dSw * tp[j]), fma(bp[j], fma(dA, tq[j], dC * tp[j]), Kb));
      const double b = bq[j];
      bq[j] = fma(C, b, A * bp[j]);
      bp[j] = fma(Sw, b, C * bp[j]);
    }
  const double b = qb;
  qb = fma(C, b, A * pqb);
  pqb = fma(Sw, b, C * pqb);
  return Kb;
}

// tan of an edge's vertical angle: constant, or the fringe-field psi of the
// job's curvature (psi = e - 2 curv fint' / cos(e) (1 + sin^2 e), SLAC-75)
__device__ __forceinline__ double edge_t2(int flags, const double *c, double curv) {
  if (flags & DE_RTPSI)
    return tan(__ldg(c + 2) - 2.0 * curv * __ldg(c + 3) / __ldg(c + 4) * __ldg(c + 5));
  return __ldg(c + 2);
}

// tape slot of field f of kick k in turn tt (counted from the start of the
// group of segments being taped); rich-tape fields: x, y, Re S', Im S'.
// Warp-blocked: one warp's values for one turn are a contiguous run (the
// reverse walk prefetches them in bulk), a kick's field a 256-byte line.
constexpr int TLANES = 32;
__device__ __forceinline__ int64_t tidx(const DiffArgs &a, int tt, int k, int f, int nf, int j) {
  const int64_t warps = (a.n_jobs + TLANES - 1) / TLANES;
  return (((static_cast<int64_t>(tt) * warps + j / TLANES) * a.kicks_per_turn + k) * nf + f) *
             TLANES + (j % TLANES);
}

// one turn forward (one lane per job); with `tape` (tangent mode) x, y and
// the x/y rows of T at every kick are recorded as turn `tt`
__device__ void turn_forward(St &s, const DiffArgs &a, const double *T0, double o, bool tangent,
                             int j, int tt, bool tape) {
  int kidx = 0;
  const int nf = 10;
  for (int i = 0; i < a.n_ops; ++i) {
    const DOp op = a.ops[i];
    const double *c = T0 + op.toff;
    const double oo = op.achro ? 1.0 : o;
    switch (op.kind) {
      case D_DRIFT:
        fwd_drift(s, __ldg(c), tangent);
        break;
      case D_ALIGN:
        s.x -= __ldg(c);
        s.y -= __ldg(c + 1);
        break;
      case D_EDGE: {
        const double curv = __ldg(c) * oo, e1 = __ldg(c + 1), e2 = edge_t2(op.flags, c, curv);
        const double x0 = s.x, y0 = s.y;
        s.px = fma(x0 * curv, e1, s.px);
        s.py = fma(-(y0 * curv), e2, s.py);
        if (tangent)
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            s.T[4 + q] = fma(s.T[q] * curv, e1, s.T[4 + q]);
            s.T[12 + q] = fma(-(s.T[8 + q] * curv), e2, s.T[12 + q]);
          }
        break;
      }
      case D_KICK:
      case D_TEAPOT: {
        const bool tp = op.kind == D_TEAPOT;
        const int N = tp ? op.N : 1;
        const double Lo = __ldg(c), Li = __ldg(c + 1), W = __ldg(c + 2), Lx = __ldg(c + 5);
        if (tp) fwd_drift(s, Lo, tangent);
        for (int sl = 0; sl < N; ++sl) {
          const int k = kidx++;
          if (tape) {  // tangent tape (the plain rich tape is written by the pair kernels)
            double *t = a.tape;
            t[tidx(a, tt, k, 0, nf, j)] = s.x;
            t[tidx(a, tt, k, 1, nf, j)] = s.y;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              t[tidx(a, tt, k, 2 + q, nf, j)] = s.T[q];
              t[tidx(a, tt, k, 6 + q, nf, j)] = s.T[8 + q];
            }
          }
          fwd_kick(s, c + KHDR, op.M, oo, tangent);
          if (tp && W != 0.0) fwd_weak(s, W, tangent);
          if (tp) fwd_drift(s, sl < N - 1 ? Li : Lx, tangent);
        }
        break;
      }
      case D_THICK: {
        const double L = __ldg(c), k1 = __ldg(c + 1), h = __ldg(c + 2);
        const int k = kidx;
        kidx += THICK_SLOTS;
        if (tape) {  // entry state and tangent: x, y, T rows x, y | px, py, T rows px, py
          double *t = a.tape;
          t[tidx(a, tt, k, 0, nf, j)] = s.x;
          t[tidx(a, tt, k, 1, nf, j)] = s.y;
          t[tidx(a, tt, k + 1, 0, nf, j)] = s.px;
          t[tidx(a, tt, k + 1, 1, nf, j)] = s.py;
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            t[tidx(a, tt, k, 2 + q, nf, j)] = s.T[q];
            t[tidx(a, tt, k, 6 + q, nf, j)] = s.T[8 + q];
            t[tidx(a, tt, k + 1, 2 + q, nf, j)] = s.T[4 + q];
            t[tidx(a, tt, k + 1, 6 + q, nf, j)] = s.T[12 + q];
          }
        }
        const double disp = (op.flags & DT_BEND) ? (1.0 / o - 1.0) * h * oo : 0.0;
        thick_plane_fwd(s.x, s.px, s.T, s.T + 4, oo * fma(h, h, k1), L, disp, tangent);
        thick_plane_fwd(s.y, s.py, s.T + 8, s.T + 12, -oo * k1, L, 0.0, tangent);
        break;
      }
      default:
        break;
    }
  }
}

struct Bar {
  double x, px, y, py;
  double T[16];
};

__device__ __forceinline__ void rev_drift(Bar &b, double L, bool tangent) {
  b.px = fma(b.x, L, b.px);
  b.py = fma(b.y, L, b.py);
  if (tangent)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      b.T[4 + j] = fma(b.T[j], L, b.T[4 + j]);
      b.T[12 + j] = fma(b.T[8 + j], L, b.T[12 + j]);
    }
}

__device__ __forceinline__ void rev_weak(Bar &b, double W, bool tangent) {
  b.x = fma(-W, b.px, b.x);
  if (tangent)
#pragma unroll
    for (int j = 0; j < 4; ++j) b.T[j] = fma(-W, b.T[4 + j], b.T[j]);
}

// z^n for small n
__device__ __forceinline__ void zpow(double x, double y, int n, double &zr, double &zi) {
  zr = 1.0;
  zi = 0.0;
  for (int k = 0; k < n; ++k) {
    const double tr = fma(zr, x, -zi * y);
    zi = fma(zr, y, zi * x);
    zr = tr;
  }
}

// reverse of one kick at the taped (x, y) [and tangent rows]; adds the
// cotangents of the op's parameter coefficient to g0 (S term, weight z^pm) and
// g1 (S' term, weight z^(pm-1)), both still to be scaled by dK/dk / n!
__device__ __forceinline__ void rev_kick(Bar &b, const DiffArgs &a, int tt, int k, int j,
                                         const double *co, int M, double o, bool tangent, int pm,
                                         double &g0, double &g1) {
  const int nf = 10;
  const double x = a.tape[tidx(a, tt, k, 0, nf, j)], y = a.tape[tidx(a, tt, k, 1, nf, j)];
  double s0r, s0i, a1, b1, a2, b2;
  series<2>(co, M, x, y, s0r, s0i, a1, b1, a2, b2);
  a1 *= o;
  b1 *= o;
  // state: px' = px - Re S, py' = py + Im S
  double xb = fma(-b.px, a1, b.py * b1);
  double yb = fma(b.px, b1, b.py * a1);
  if (pm >= 0) {  // dS/dc = o z^pm / pm!
    double zr, zi;
    zpow(x, y, pm, zr, zi);
    g0 += o * fma(-b.px, zr, b.py * zi);
  }
  if (tangent) {
    a2 *= 2.0 * o;
    b2 *= 2.0 * o;
    double Ab = 0.0, Bb = 0.0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const double dx = a.tape[tidx(a, tt, k, 2 + q, nf, j)];
      const double dy = a.tape[tidx(a, tt, k, 6 + q, nf, j)];
      const double pxb = b.T[4 + q], pyb = b.T[12 + q];
      // T_px -= a1 dx - b1 dy ; T_py += b1 dx + a1 dy
      b.T[q] += fma(-pxb, a1, pyb * b1);
      b.T[8 + q] += fma(pxb, b1, pyb * a1);
      Ab += fma(-pxb, dx, pyb * dy);
      Bb += fma(pxb, dy, pyb * dx);
    }
    // a1 + i b1 = S'(z): d/dx = S'' , d/dy = i S''
    xb += fma(Ab, a2, Bb * b2);
    yb += fma(-Ab, b2, Bb * a2);
    if (pm >= 1) {  // dS'/dc = o z^(pm-1) / (pm-1)!
      double zr, zi;
      zpow(x, y, pm - 1, zr, zi);
      g1 += o * fma(Ab, zr, Bb * zi);
    }
  }
  b.x += xb;
  b.y += yb;
}

// reverse of turn `tt` of the segment from its tape; accumulates parameter
// cotangents
__device__ void turn_reverse(Bar &b, const DiffArgs &a, const double *T0, double o, bool tangent,
                             int j, int tt) {
  int kidx = a.kicks_per_turn;
  for (int i = a.n_ops - 1; i >= 0; --i) {
    const DOp op = a.ops[i];
    const double *c = T0 + op.toff;
    const double oo = op.achro ? 1.0 : o;
    switch (op.kind) {
      case D_DRIFT:
        rev_drift(b, __ldg(c), tangent);
        break;
      case D_ALIGN:
        break;  // translation: cotangents unchanged
      case D_EDGE: {
        const double curv = __ldg(c) * oo, e1 = __ldg(c + 1), e2 = edge_t2(op.flags, c, curv);
        b.x = fma(b.px * curv, e1, b.x);
        b.y = fma(-(b.py * curv), e2, b.y);
        if (tangent)
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            b.T[q] = fma(b.T[4 + q] * curv, e1, b.T[q]);
            b.T[8 + q] = fma(-(b.T[12 + q] * curv), e2, b.T[8 + q]);
          }
        break;
      }
      case D_KICK:
      case D_TEAPOT: {
        const bool tp = op.kind == D_TEAPOT;
        const int N = tp ? op.N : 1;
        const double Lo = __ldg(c), Li = __ldg(c + 1), W = __ldg(c + 2), Lx = __ldg(c + 5);
        const int pm = op.pslot >= 0 ? op.pm : -1;
        double g0 = 0.0, g1 = 0.0;
        for (int sl = N - 1; sl >= 0; --sl) {
          if (tp) rev_drift(b, sl < N - 1 ? Li : Lx, tangent);
          if (tp && W != 0.0) rev_weak(b, W, tangent);
          rev_kick(b, a, tt, --kidx, j, c + KHDR, op.M, oo, tangent, pm, g0, g1);
        }
        if (tp) rev_drift(b, Lo, tangent);
        if (op.pslot >= 0) {
          double &p = a.pbar[static_cast<int64_t>(op.pslot) * a.n_jobs + j];
          p = fma(g0, __ldg(c + 3), fma(g1, __ldg(c + 4), p));
        }
        break;
      }
      case D_THICK: {
        const double L = __ldg(c), k1 = __ldg(c + 1), h = __ldg(c + 2);
        kidx -= THICK_SLOTS;
        const int nf = 10;
        const double *t = a.tape;
        double ex[4], epx[4], ey[4], epy[4];  // entry tangent rows
        if (tangent)
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            ex[q] = t[tidx(a, tt, kidx, 2 + q, nf, j)];
            ey[q] = t[tidx(a, tt, kidx, 6 + q, nf, j)];
            epx[q] = t[tidx(a, tt, kidx + 1, 2 + q, nf, j)];
            epy[q] = t[tidx(a, tt, kidx + 1, 6 + q, nf, j)];
          }
        const double x = t[tidx(a, tt, kidx, 0, nf, j)], y = t[tidx(a, tt, kidx, 1, nf, j)];
        const double px = t[tidx(a, tt, kidx + 1, 0, nf, j)];
        const double py = t[tidx(a, tt, kidx + 1, 1, nf, j)];
        const double disp = (op.flags & DT_BEND) ? (1.0 / o - 1.0) * h * oo : 0.0;
        const double kbx = thick_plane_rev(b.x, b.px, b.T, b.T + 4, ex, epx, x, px,
                                           oo * fma(h, h, k1), L, disp, tangent);
        const double kby = thick_plane_rev(b.y, b.py, b.T + 8, b.T + 12, ey, epy, y, py, -oo * k1,
                                           L, 0.0, tangent);
        if (op.pslot >= 0) {  // dK_x/dk1 = o, dK_y/dk1 = -o
          double &p = a.pbar[static_cast<int64_t>(op.pslot) * a.n_jobs + j];
          p = fma(oo, kbx - kby, p);
        }
        break;
      }
      default:
        break;
    }
  }
}

// z^pm for the parameter weight of the reverse kick: closed forms for the
// quadrupole and sextupole orders
__device__ __forceinline__ void zpow_small(double x, double y, int pm, double &zr, double &zi) {
  if (pm == 1) {
    zr = x;
    zi = y;
  } else if (pm == 2) {
    zr = fma(x, x, -y * y);
    zi = 2.0 * x * y;
  } else if (pm == 0) {
    zr = 1.0;
    zi = 0.0;
  } else {
    zpow(x, y, pm, zr, zi);
  }
}

// The reverse walk reads the tape backwards from HBM with one warp per SM,
// one dependent access per kick.  Lane 0 asks the copy engine to bring the
// warp's next chunks (CHUNK kicks, 64 KiB) into L2 ahead of use: fire and
// forget, nothing waits on it.
constexpr int CHUNK = 64;

__device__ __forceinline__ void prefetch_l2_bulk(const double *p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// chunk [k0, k0 + CHUNK) of turn tt (clipped at 0) of this lane's warp
__device__ __forceinline__ void prefetch_chunk(const DiffArgs &a, int tt, int k0, int j) {
  const int lo = k0 < 0 ? 0 : k0;
  const int hi = min(k0 + CHUNK, a.kicks_per_turn);  // stay inside this warp's turn
  if (hi <= lo || (j % TLANES) != 0) return;
  prefetch_l2_bulk(a.tape + tidx(a, tt, lo, 0, 4, j),
                   static_cast<uint32_t>((hi - lo) * 4 * TLANES * sizeof(double)));
}

__device__ void save_ckpt(const St &s, const DiffArgs &a, int c, int j, bool tangent) {
  double *d = a.ckpt + static_cast<int64_t>(c) * 20 * a.n_jobs + j;
  d[0] = s.x;
  d[a.n_jobs] = s.px;
  d[2 * a.n_jobs] = s.y;
  d[3 * a.n_jobs] = s.py;
  if (tangent)
#pragma unroll
    for (int k = 0; k < 16; ++k) d[(4 + k) * static_cast<int64_t>(a.n_jobs)] = s.T[k];
}

__device__ void load_ckpt(St &s, const DiffArgs &a, int c, int j, bool tangent) {
  const double *d = a.ckpt + static_cast<int64_t>(c) * 20 * a.n_jobs + j;
  s.x = d[0];
  s.px = d[a.n_jobs];
  s.y = d[2 * a.n_jobs];
  s.py = d[3 * a.n_jobs];
#pragma unroll
  for (int k = 0; k < 16; ++k)
    s.T[k] = tangent ? d[(4 + k) * static_cast<int64_t>(a.n_jobs)] : 0.0;
}

__global__ void diff_forward(DiffArgs a) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.n_jobs) return;
  const bool tangent = a.tangent;
  St s;
  s.x = a.z0[4 * j]; s.px = a.z0[4 * j + 1]; s.y = a.z0[4 * j + 2]; s.py = a.z0[4 * j + 3];
#pragma unroll
  for (int k = 0; k < 16; ++k) s.T[k] = (k % 5 == 0) ? 1.0 : 0.0;
  const double o = a.o[j];
  const double *T0 = a.tab + (a.seed ? static_cast<int64_t>(a.seed[j]) : 0) * a.tab_stride;
  const bool ck = a.ckpt != nullptr;
  for (int t = 0; t < a.turns; ++t) {
    if (ck && t % a.ck == 0) save_ckpt(s, a, t / a.ck, j, tangent);
    turn_forward(s, a, T0, o, tangent, j, 0, false);
  }
  if (ck && a.turns % a.ck == 0) save_ckpt(s, a, a.turns / a.ck, j, tangent);
  double *d = a.zT + 20 * static_cast<int64_t>(j);
  d[0] = s.x; d[1] = s.px; d[2] = s.y; d[3] = s.py;
#pragma unroll
  for (int k = 0; k < 16; ++k) d[4 + k] = tangent ? s.T[k] : 0.0;
}

__global__ void diff_reverse(DiffArgs a) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.n_jobs) return;
  const bool tangent = a.tangent;
  const double o = a.o[j];
  const double *T0 = a.tab + (a.seed ? static_cast<int64_t>(a.seed[j]) : 0) * a.tab_stride;
  for (int k = 0; k < a.n_params; ++k) a.pbar[static_cast<int64_t>(k) * a.n_jobs + j] = 0.0;
  Bar b;
  b.x = a.zbar[4 * j]; b.px = a.zbar[4 * j + 1]; b.y = a.zbar[4 * j + 2]; b.py = a.zbar[4 * j + 3];
#pragma unroll
  for (int k = 0; k < 16; ++k) b.T[k] = tangent ? a.Tbar[16 * j + k] : 0.0;
  const int last_seg = (a.turns - 1) / a.ck;
  for (int sg = last_seg; sg >= 0; --sg) {
    const int t0 = sg * a.ck;
    const int t1 = min(a.turns, t0 + a.ck);
    St s;
    load_ckpt(s, a, sg, j, tangent);
    for (int t = t0; t < t1; ++t) turn_forward(s, a, T0, o, tangent, j, t - t0, true);
    for (int t = t1 - 1; t >= t0; --t) turn_reverse(b, a, T0, o, tangent, j, t - t0);
  }
  a.zbar0[4 * j] = b.x; a.zbar0[4 * j + 1] = b.px; a.zbar0[4 * j + 2] = b.y;
  a.zbar0[4 * j + 3] = b.py;
}

// ---------------------------------------------------------------- lane pairs
// Plain (non-tangent) mode runs every job on two lanes of a warp: the even
// lane carries the horizontal plane (x, px), the odd lane the vertical one
// (y, py), so a warp holds 16 jobs and a sweep of J jobs has twice the warps
// (the SM sub-partitions are what the one-thread-per-job sweep leaves idle).
// Each quantity is computed by the same IEEE operations, in the same order, as
// in the one-lane code above; the lanes exchange values by warp shuffles where
// a quantity needs both planes (z = x + iy of a kick, the complex Horner
// steps, the momentum cotangents of the reverse kick).  Lanes of a job past
// the end keep running on a clamped job (every shuffle has all 32 lanes) and
// write nothing.
constexpr unsigned ALL_LANES = 0xffffffffu;

struct Half {
  double u, pu;  // this lane's plane: (x, px) on even lanes, (y, py) on odd lanes
};

__device__ __forceinline__ double other(double v) { return __shfl_xor_sync(ALL_LANES, v, 1); }

// S(z)/o (and S'(z)/o with ND = 1) split over the pair: `r0` / `r1` are this
// lane's part (real on even lanes, imaginary on odd lanes)
template <int ND>
__device__ __forceinline__ void series_pair(const double *__restrict__ a, int M, double x, double y,
                                            bool even, double &r0, double &r1) {
  const double *b = a + M;
  const double p = even ? x : y, q = even ? y : x;
  r0 = even ? __ldg(a + M - 1) : __ldg(b + M - 1);
  r1 = 0.0;
  for (int n = M - 2; n >= 0; --n) {
    const double o0 = other(r0);
    const double sr0 = even ? r0 : o0, si0 = even ? o0 : r0;
    if (ND >= 1) {
      const double o1 = other(r1);
      const double sr1 = even ? r1 : o1, si1 = even ? o1 : r1;
      // re: fma(s1r, x, fma(-s1i, y, s0r)); im: fma(s1r, y, fma(s1i, x, s0i))
      r1 = fma(sr1, p, fma(even ? -si1 : si1, q, even ? sr0 : si0));
    }
    const double c = even ? __ldg(a + n) : __ldg(b + n);
    r0 = fma(sr0, p, fma(even ? -si0 : si0, q, c));
  }
}

// a kick element of the pair with its M coefficients (this lane's part: the
// normal list on even lanes, the skew list on odd lanes) loaded into
// registers once for all N slices; the unrolled Horner issues no loads
template <int M>
__device__ __forceinline__ void kick_elem_pair(Half &h, const DiffArgs &a, const double *c, bool tp,
                                               int N, double oo, bool even, int j, bool write,
                                               int tt, bool tape, int &kidx) {
  double cf[M];
  const double *src = c + KHDR + (even ? 0 : M);
#pragma unroll
  for (int n = 0; n < M; ++n) cf[n] = __ldg(src + n);
  const double Lo = __ldg(c), Li = __ldg(c + 1), W = __ldg(c + 2), Lx = __ldg(c + 5);
  if (tp) h.u = fma(h.pu, Lo, h.u);
  for (int sl = 0; sl < N; ++sl) {
    const int k = kidx++;
    const double w = other(h.u);
    const double x = even ? h.u : w, y = even ? w : h.u;
    const double p = even ? x : y, q = even ? y : x;
    double r0 = cf[M - 1], r1 = 0.0;
    if (tape) {
#pragma unroll
      for (int n = M - 2; n >= 0; --n) {
        const double o0 = other(r0), o1 = other(r1);
        const double sr0 = even ? r0 : o0, si0 = even ? o0 : r0;
        const double sr1 = even ? r1 : o1, si1 = even ? o1 : r1;
        r1 = fma(sr1, p, fma(even ? -si1 : si1, q, even ? sr0 : si0));
        r0 = fma(sr0, p, fma(even ? -si0 : si0, q, cf[n]));
      }
      if (write) {
        double *t0 = a.tape + tidx(a, tt, k, 0, 4, j);
        t0[even ? 0 : TLANES] = h.u;
        t0[(even ? 2 : 3) * TLANES] = oo * r1;
      }
    } else {
#pragma unroll
      for (int n = M - 2; n >= 0; --n) {
        const double o0 = other(r0);
        const double sr0 = even ? r0 : o0, si0 = even ? o0 : r0;
        r0 = fma(sr0, p, fma(even ? -si0 : si0, q, cf[n]));
      }
    }
    h.pu = fma(even ? -oo : oo, r0, h.pu);
    if (tp && W != 0.0 && even) h.pu = fma(-W, h.u, h.pu);
    if (tp) h.u = fma(h.pu, sl < N - 1 ? Li : Lx, h.u);
  }
}

// one turn forward of the pair; with `tape` the rich tape is written as turn
// `tt` of the group (x, Re S' by the even lane; y, Im S' by the odd lane)
__device__ void turn_forward_pair(Half &h, const DiffArgs &a, const double *T0, double o,
                                  bool even, int j, bool write, int tt, bool tape) {
  int kidx = 0;
  for (int i = 0; i < a.n_ops; ++i) {
    const DOp op = a.ops[i];
    const double *c = T0 + op.toff;
    const double oo = op.achro ? 1.0 : o;
    switch (op.kind) {
      case D_DRIFT:
        h.u = fma(h.pu, __ldg(c), h.u);
        break;
      case D_ALIGN:
        h.u -= __ldg(c + (even ? 0 : 1));
        break;
      case D_EDGE: {
        const double curv = __ldg(c) * oo;
        const double t = h.u * curv;
        h.pu = fma(even ? t : -t, even ? __ldg(c + 1) : edge_t2(op.flags, c, curv), h.pu);
        break;
      }
      case D_THICK: {
        const double L = __ldg(c), k1 = __ldg(c + 1), hh = __ldg(c + 2);
        const int k = kidx;
        kidx += THICK_SLOTS;
        if (tape && write) {  // entry state: x, px by the even lane; y, py by the odd lane
          double *t0 = a.tape + tidx(a, tt, k, 0, 4, j);
          t0[even ? 0 : TLANES] = h.u;
          t0[(even ? 2 : 3) * TLANES] = h.pu;
        }
        const double K = even ? oo * fma(hh, hh, k1) : -oo * k1;
        const double disp = (even && (op.flags & DT_BEND)) ? (1.0 / o - 1.0) * hh * oo : 0.0;
        thick_plane_fwd(h.u, h.pu, nullptr, nullptr, K, L, disp, false);
        break;
      }
      case D_KICK:
      case D_TEAPOT: {
        const bool tp = op.kind == D_TEAPOT;
        const int N = tp ? op.N : 1;
        switch (op.M) {  // common orders: coefficients in registers
          case 1: kick_elem_pair<1>(h, a, c, tp, N, oo, even, j, write, tt, tape, kidx); continue;
          case 2: kick_elem_pair<2>(h, a, c, tp, N, oo, even, j, write, tt, tape, kidx); continue;
          case 3: kick_elem_pair<3>(h, a, c, tp, N, oo, even, j, write, tt, tape, kidx); continue;
          case 4: kick_elem_pair<4>(h, a, c, tp, N, oo, even, j, write, tt, tape, kidx); continue;
          case 5: kick_elem_pair<5>(h, a, c, tp, N, oo, even, j, write, tt, tape, kidx); continue;
          case 6: kick_elem_pair<6>(h, a, c, tp, N, oo, even, j, write, tt, tape, kidx); continue;
          case 7: kick_elem_pair<7>(h, a, c, tp, N, oo, even, j, write, tt, tape, kidx); continue;
          case 8: kick_elem_pair<8>(h, a, c, tp, N, oo, even, j, write, tt, tape, kidx); continue;
          default: break;
        }
        const double Lo = __ldg(c), Li = __ldg(c + 1), W = __ldg(c + 2), Lx = __ldg(c + 5);
        if (tp) h.u = fma(h.pu, Lo, h.u);
        for (int sl = 0; sl < N; ++sl) {
          const int k = kidx++;
          const double w = other(h.u);
          const double x = even ? h.u : w, y = even ? w : h.u;
          double s0, s1;
          if (tape) {
            series_pair<1>(c + KHDR, op.M, x, y, even, s0, s1);
            if (write) {
              double *t0 = a.tape + tidx(a, tt, k, 0, 4, j);
              t0[even ? 0 : TLANES] = h.u;
              t0[(even ? 2 : 3) * TLANES] = oo * s1;
            }
          } else {
            series_pair<0>(c + KHDR, op.M, x, y, even, s0, s1);
          }
          h.pu = fma(even ? -oo : oo, s0, h.pu);
          if (tp && W != 0.0 && even) h.pu = fma(-W, h.u, h.pu);
          if (tp) h.u = fma(h.pu, sl < N - 1 ? Li : Lx, h.u);
        }
        break;
      }
      default:
        break;
    }
  }
}

// reverse of a kick element of the pair with the tape values of its N slices
// (x, y, Re S', Im S') loaded up front, before the dependent cotangent chain
template <int N>
__device__ __forceinline__ void rev_elem_pair(Half &bh, const DiffArgs &a, const double *c, bool tp,
                                              double oo, bool even, int j, bool write, int tt,
                                              int pm, int &kidx, double &g0) {
  double tx[N], ty[N], ta[N], tb[N];
#pragma unroll
  for (int q = 0; q < N; ++q) {
    const double *t0 = a.tape + tidx(a, tt, kidx - 1 - q, 0, 4, j);
    tx[q] = t0[0];
    ty[q] = t0[TLANES];
    ta[q] = t0[2 * TLANES];
    tb[q] = t0[3 * TLANES];
  }
  const double Lo = __ldg(c), Li = __ldg(c + 1), W = __ldg(c + 2), Lx = __ldg(c + 5);
#pragma unroll
  for (int q = 0; q < N; ++q) {  // slice N-1-q
    if (tp) bh.pu = fma(bh.u, q > 0 ? Li : Lx, bh.pu);
    if (tp && W != 0.0 && even) bh.u = fma(-W, bh.pu, bh.u);
    --kidx;
    if (write && even && kidx % CHUNK == 0 && kidx >= 2 * CHUNK)
      prefetch_chunk(a, tt, kidx - 2 * CHUNK, j);
    const double a1 = ta[q], b1 = tb[q];
    const double w = other(bh.pu);
    const double pxb = even ? bh.pu : w, pyb = even ? w : bh.pu;
    bh.u = fma(even ? -pxb : pxb, even ? a1 : b1, fma(pyb, even ? b1 : a1, bh.u));
    if (pm >= 0) {
      double zr, zi;
      zpow_small(tx[q], ty[q], pm, zr, zi);
      g0 = fma(-pxb, zr, fma(pyb, zi, g0));
    }
  }
  if (tp) bh.pu = fma(bh.u, Lo, bh.pu);
}

// reverse of turn `tt` of the group from the rich tape, split over the pair
// (cotangents of x, px on even lanes, of y, py on odd lanes)
__device__ void turn_reverse_pair(Half &bh, const DiffArgs &a, const double *T0, double o,
                                  bool even, int j, bool write, int tt) {
  int kidx = a.kicks_per_turn;
  const int top = ((a.kicks_per_turn - 1) / CHUNK) * CHUNK;
  if (write && even) {
    prefetch_chunk(a, tt, top, j);
    prefetch_chunk(a, tt, top - CHUNK, j);
  }
  for (int i = a.n_ops - 1; i >= 0; --i) {
    const DOp op = a.ops[i];
    const double *c = T0 + op.toff;
    const double oo = op.achro ? 1.0 : o;
    switch (op.kind) {
      case D_DRIFT:
        bh.pu = fma(bh.u, __ldg(c), bh.pu);
        break;
      case D_ALIGN:
        break;
      case D_EDGE: {
        const double curv = __ldg(c) * oo;
        const double t = bh.pu * curv;
        bh.u = fma(even ? t : -t, even ? __ldg(c + 1) : edge_t2(op.flags, c, curv), bh.u);
        break;
      }
      case D_THICK: {
        const double L = __ldg(c), k1 = __ldg(c + 1), hh = __ldg(c + 2);
        kidx -= THICK_SLOTS;
        const int m = ((kidx + THICK_SLOTS - 1) / CHUNK) * CHUNK;  // a chunk start in range
        if (write && even && m >= kidx && m >= 2 * CHUNK) prefetch_chunk(a, tt, m - 2 * CHUNK, j);
        const double *t0 = a.tape + tidx(a, tt, kidx, 0, 4, j);
        const double q = t0[even ? 0 : TLANES], pq = t0[(even ? 2 : 3) * TLANES];
        const double K = even ? oo * fma(hh, hh, k1) : -oo * k1;
        const double disp = (even && (op.flags & DT_BEND)) ? (1.0 / o - 1.0) * hh * oo : 0.0;
        const double kb = thick_plane_rev(bh.u, bh.pu, nullptr, nullptr, nullptr, nullptr, q, pq,
                                          K, L, disp, false);
        const double kb_other = other(kb);  // every lane: the shuffle needs the whole warp
        if (op.pslot >= 0 && write && even) {  // dK_x/dk1 = o, dK_y/dk1 = -o
          double &p = a.pbar[static_cast<int64_t>(op.pslot) * a.n_jobs + j];
          p = fma(oo, kb - kb_other, p);
        }
        break;
      }
      case D_KICK:
      case D_TEAPOT: {
        const bool tp = op.kind == D_TEAPOT;
        const int N = tp ? op.N : 1;
        const double Lo = __ldg(c), Li = __ldg(c + 1), W = __ldg(c + 2), Lx = __ldg(c + 5);
        const int pm = op.pslot >= 0 ? op.pm : -1;
        double g0 = 0.0;
        bool done = true;
        switch (N) {  // common slice counts: the element's tape values up front
          case 1: rev_elem_pair<1>(bh, a, c, tp, oo, even, j, write, tt, pm, kidx, g0); break;
          case 2: rev_elem_pair<2>(bh, a, c, tp, oo, even, j, write, tt, pm, kidx, g0); break;
          case 4: rev_elem_pair<4>(bh, a, c, tp, oo, even, j, write, tt, pm, kidx, g0); break;
          case 8: rev_elem_pair<8>(bh, a, c, tp, oo, even, j, write, tt, pm, kidx, g0); break;
          default: done = false; break;
        }
        for (int sl = N - 1; !done && sl >= 0; --sl) {
          if (tp) bh.pu = fma(bh.u, sl < N - 1 ? Li : Lx, bh.pu);
          if (tp && W != 0.0 && even) bh.u = fma(-W, bh.pu, bh.u);
          --kidx;
          if (write && even && kidx % CHUNK == 0 && kidx >= 2 * CHUNK)
            prefetch_chunk(a, tt, kidx - 2 * CHUNK, j);
          const double *t0 = a.tape + tidx(a, tt, kidx, 0, 4, j);
          const double a1 = t0[2 * TLANES], b1 = t0[3 * TLANES];
          const double w = other(bh.pu);
          const double pxb = even ? bh.pu : w, pyb = even ? w : bh.pu;
          // x: fma(-pxb, a1, fma(pyb, b1, xb)); y: fma(pxb, b1, fma(pyb, a1, yb))
          bh.u = fma(even ? -pxb : pxb, even ? a1 : b1, fma(pyb, even ? b1 : a1, bh.u));
          if (pm >= 0) {
            double zr, zi;
            zpow_small(t0[0], t0[TLANES], pm, zr, zi);
            g0 = fma(-pxb, zr, fma(pyb, zi, g0));
          }
        }
        if (tp && !done) bh.pu = fma(bh.u, Lo, bh.pu);
        if (op.pslot >= 0 && write && even) {
          double &p = a.pbar[static_cast<int64_t>(op.pslot) * a.n_jobs + j];
          p = fma(g0 * oo, __ldg(c + 3), p);
        }
        break;
      }
      default:
        break;
    }
  }
}

// pair index of this thread: job j (clamped), lane parity, whether it writes
__device__ __forceinline__ void pair_of(int64_t t, int64_t jobs, int64_t &job, bool &even,
                                        bool &write) {
  job = t >> 1;
  even = (t & 1) == 0;
  write = job < jobs;
  if (!write) job = jobs - 1;
}

__global__ void diff_forward_pair(DiffArgs a) {
  const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if ((t & ~static_cast<int64_t>(31)) >= 2 * static_cast<int64_t>(a.n_jobs)) return;  // whole warp past the end
  int64_t jl;
  bool even, write;
  pair_of(t, a.n_jobs, jl, even, write);
  const int j = static_cast<int>(jl);
  Half h;
  h.u = a.z0[4 * j + (even ? 0 : 2)];
  h.pu = a.z0[4 * j + (even ? 1 : 3)];
  const double o = a.o[j];
  const double *T0 = a.tab + (a.seed ? static_cast<int64_t>(a.seed[j]) : 0) * a.tab_stride;
  const bool ck = a.ckpt != nullptr;
  const int f0 = even ? 0 : 2;
  for (int tt = 0; tt < a.turns; ++tt) {
    if (ck && tt % a.ck == 0 && write) {
      double *d = a.ckpt + static_cast<int64_t>(tt / a.ck) * 20 * a.n_jobs + j;
      d[f0 * static_cast<int64_t>(a.n_jobs)] = h.u;
      d[(f0 + 1) * static_cast<int64_t>(a.n_jobs)] = h.pu;
    }
    turn_forward_pair(h, a, T0, o, even, j, write, 0, false);
  }
  if (write) {
    if (ck && a.turns % a.ck == 0) {
      double *d = a.ckpt + static_cast<int64_t>(a.turns / a.ck) * 20 * a.n_jobs + j;
      d[f0 * static_cast<int64_t>(a.n_jobs)] = h.u;
      d[(f0 + 1) * static_cast<int64_t>(a.n_jobs)] = h.pu;
    }
    double *d = a.zT + 20 * static_cast<int64_t>(j);
    d[f0] = h.u;
    d[f0 + 1] = h.pu;
    if (even)
      for (int k = 4; k < 20; ++k) d[k] = 0.0;
  }
}

__global__ void diff_tape_pair(DiffArgs a, int sg0, int G) {
  const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  const int64_t pairs = static_cast<int64_t>(G) * a.n_jobs;
  if ((t & ~static_cast<int64_t>(31)) >= 2 * pairs) return;
  int64_t q;
  bool even, write;
  pair_of(t, pairs, q, even, write);
  const int g = static_cast<int>(q / a.n_jobs), j = static_cast<int>(q % a.n_jobs);
  const int sg = sg0 + g;
  const int t0 = sg * a.ck;
  const bool live = t0 < a.turns;  // uniform per segment: whole warps agree unless G spans
  const int t1 = live ? min(a.turns, t0 + a.ck) : t0;
  const double o = a.o[j];
  const double *T0 = a.tab + (a.seed ? static_cast<int64_t>(a.seed[j]) : 0) * a.tab_stride;
  Half h;
  const int f0 = even ? 0 : 2;
  const int sl = live ? sg : 0;
  const double *d = a.ckpt + static_cast<int64_t>(sl) * 20 * a.n_jobs + j;
  h.u = d[f0 * static_cast<int64_t>(a.n_jobs)];
  h.pu = d[(f0 + 1) * static_cast<int64_t>(a.n_jobs)];
  // a warp may straddle two segments (J not a multiple of 16): every lane runs
  // the longer count; lanes past their own segment end do not write
  const int tmax = __reduce_max_sync(ALL_LANES, t1 - t0);
  for (int k = 0; k < tmax; ++k)
    turn_forward_pair(h, a, T0, o, even, j, write && k < t1 - t0, g * a.ck + k, true);
}

__global__ void diff_reverse_plain_pair(DiffArgs a, int sg0, int sg_hi) {
  const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if ((t & ~static_cast<int64_t>(31)) >= 2 * static_cast<int64_t>(a.n_jobs)) return;
  int64_t jl;
  bool even, write;
  pair_of(t, a.n_jobs, jl, even, write);
  const int j = static_cast<int>(jl);
  const double o = a.o[j];
  const double *T0 = a.tab + (a.seed ? static_cast<int64_t>(a.seed[j]) : 0) * a.tab_stride;
  const int f0 = even ? 0 : 2;
  Half bh;
  bh.u = a.zbar0[4 * j + f0];
  bh.pu = a.zbar0[4 * j + f0 + 1];
  for (int sg = sg_hi; sg >= sg0; --sg) {
    const int t0 = sg * a.ck;
    const int t1 = min(a.turns, t0 + a.ck);
    for (int tt = t1 - 1; tt >= t0; --tt)
      turn_reverse_pair(bh, a, T0, o, even, j, write, (sg - sg0) * a.ck + (tt - t0));
  }
  if (write) {
    a.zbar0[4 * j + f0] = bh.u;
    a.zbar0[4 * j + f0 + 1] = bh.pu;
  }
}

}  // namespace ufo_diff

// ---------------------------------------------------------------- C ABI
extern "C" {

// All pointers are device pointers; `ops` int32[n_ops][8] (DOp), `tab` f64.
// Asynchronous on `stream`.  Returns 0, -1 (bad arguments) or -2 (launch
// error).
// the kernels use no shared memory: give the whole on-chip store to L1, where
// the opcode list and one seed's constants (~200 kB for a 1,000-element ring)
// then stay resident
static void prefer_l1() {
  static bool done = false;
  if (done) return;
  cudaFuncSetAttribute(ufo_diff::diff_forward, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
  cudaFuncSetAttribute(ufo_diff::diff_reverse, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
  cudaFuncSetAttribute(ufo_diff::diff_forward_pair,
                       cudaFuncAttributePreferredSharedMemoryCarveout, 0);
  cudaFuncSetAttribute(ufo_diff::diff_tape_pair, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
  cudaFuncSetAttribute(ufo_diff::diff_reverse_plain_pair,
                       cudaFuncAttributePreferredSharedMemoryCarveout, 0);
  done = true;
}

int ufo_diff_forward(const int32_t *ops, int n_ops, const double *tab, int64_t tab_stride,
                     const int32_t *seed, int n_params, int kicks_per_turn, int n_jobs,
                     const double *z0, const double *o, int turns, int ck, int tangent,
                     double *ckpt, double *zT, void *stream) {
  if (n_jobs <= 0) return 0;
  if (!ops || n_ops < 0 || !tab || !z0 || !o || !zT || turns < 0 || ck < 1) return -1;
  prefer_l1();
  ufo_diff::DiffArgs a{};
  a.ops = reinterpret_cast<const ufo_diff::DOp *>(ops);
  a.n_ops = n_ops;
  a.tab = tab;
  a.tab_stride = tab_stride;
  a.seed = seed;
  a.n_params = n_params;
  a.kicks_per_turn = kicks_per_turn;
  a.n_jobs = n_jobs;
  a.z0 = z0;
  a.o = o;
  a.turns = turns;
  a.ck = ck;
  a.tangent = tangent;
  a.ckpt = ckpt;
  a.zT = zT;
  const int tpb = 32;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (tangent) {
    ufo_diff::diff_forward<<<(n_jobs + tpb - 1) / tpb, tpb, 0, st>>>(a);
  } else {  // two lanes per job
    const int64_t threads = 2 * static_cast<int64_t>(n_jobs);
    ufo_diff::diff_forward_pair<<<static_cast<unsigned>((threads + tpb - 1) / tpb), tpb, 0, st>>>(a);
  }
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int ufo_diff_reverse(const int32_t *ops, int n_ops, const double *tab, int64_t tab_stride,
                     const int32_t *seed, int n_params, int kicks_per_turn, int n_jobs,
                     const double *o, int turns, int ck, int tangent, const double *ckpt,
                     const double *zbar, const double *Tbar, double *tape, int tape_segments,
                     double *zbar0, double *pbar, void *stream) {
  if (n_jobs <= 0) return 0;
  if (!ops || n_ops < 0 || !tab || !o || !ckpt || !zbar || !tape || !zbar0 ||
      (n_params > 0 && !pbar) || turns < 1 || ck < 1 || (tangent && !Tbar) || tape_segments < 1)
    return -1;
  prefer_l1();
  ufo_diff::DiffArgs a{};
  a.ops = reinterpret_cast<const ufo_diff::DOp *>(ops);
  a.n_ops = n_ops;
  a.tab = tab;
  a.tab_stride = tab_stride;
  a.seed = seed;
  a.n_params = n_params;
  a.kicks_per_turn = kicks_per_turn;
  a.n_jobs = n_jobs;
  a.o = o;
  a.turns = turns;
  a.ck = ck;
  a.tangent = tangent;
  a.ckpt = const_cast<double *>(ckpt);
  a.zbar = zbar;
  a.Tbar = Tbar;
  a.tape = tape;
  a.zbar0 = zbar0;
  a.pbar = pbar;
  const int tpb = 32;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (tangent) {
    ufo_diff::diff_reverse<<<(n_jobs + tpb - 1) / tpb, tpb, 0, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
  }
  // plain mode: groups of up to tape_segments segments, last group first
  if (n_params > 0 &&
      cudaMemsetAsync(pbar, 0, sizeof(double) * n_params * static_cast<size_t>(n_jobs), st) !=
          cudaSuccess)
    return -2;
  if (cudaMemcpyAsync(zbar0, zbar, sizeof(double) * 4 * static_cast<size_t>(n_jobs),
                      cudaMemcpyDeviceToDevice, st) != cudaSuccess)
    return -2;
  const int last_seg = (turns - 1) / ck;
  for (int hi = last_seg; hi >= 0; hi -= tape_segments) {
    const int lo = hi - tape_segments + 1 < 0 ? 0 : hi - tape_segments + 1;
    const int G = hi - lo + 1;
    const int64_t threads = 2 * static_cast<int64_t>(G) * n_jobs;  // two lanes per job
    ufo_diff::diff_tape_pair<<<static_cast<unsigned>((threads + tpb - 1) / tpb), tpb, 0, st>>>(
        a, lo, G);
    const int64_t rthreads = 2 * static_cast<int64_t>(n_jobs);
    ufo_diff::diff_reverse_plain_pair<<<static_cast<unsigned>((rthreads + tpb - 1) / tpb), tpb, 0,
                                        st>>>(a, lo, hi);
    if (cudaGetLastError() != cudaSuccess) return -2;
  }
  return 0;
}

}  // extern "C"
