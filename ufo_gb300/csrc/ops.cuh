// ops.cuh -- FP64 element pass methods interpreted from the opcode table.
//
// Each op reproduces one template of the reference's code generator
// (ufo/methods.py) with the reference's C evaluation order, so that in the
// default (strict) mode every coordinate is bit-identical to the reference's
// FP64 kernel.  Strict mode uses __dmul_rn/__dadd_rn/... (never contracted);
// FMA mode contracts multiply-add pairs and replaces divisions by constants.
//
// Structurally-zero terms (coefficients that are 0 in every seed) were dropped
// by the compiler.  For finite x, y the dropped terms contribute exact zeros;
// when x or y is not finite, a 0*x term is NaN in the reference, so those
// cases run the untrimmed expression (`slow` paths below).
#pragma once
#include <cstdint>

namespace ufo {

enum : int {
  OP_NOP = 0, OP_DRIFT, OP_KICK, OP_TEAPOT, OP_ALIGN, OP_EDGE, OP_THICKQ, OP_THICKB, OP_WIRE,
  OP_APERTURE, OP_OBSERVE, OP_DYNKICK, OP_LINEAR
};
enum : int { DF_MUL = 0, DF_MUL2 = 1, DF_DIV = 2 };
enum : int {
  F_ACHRO = 1 << 0, F_EXACT = 1 << 1, F_WEAK = 1 << 2, F_RTPSI = 1 << 3, F_T1 = 1 << 4,
  F_T2 = 1 << 5, F_CONST = 1 << 6, F_AX = 1 << 7, F_AY = 1 << 8, F_T1Z = 1 << 9,
  F_T2Z = 1 << 10, F_WEAKZ = 1 << 11, F_YOSHIDA = 1 << 12, F_CIRCLE = 1 << 13, F_SPLITO = 1 << 14,
  F_PSER = 1 << 15
};
constexpr int SH_FOUTER = 16, SH_FINNER = 18;

struct Op {
  int kind, flags, toff, i0, i1, i2, i3, i4;
};

#define UFO_DEV __device__ __forceinline__

UFO_DEV double mul(double a, double b) { return __dmul_rn(a, b); }
UFO_DEV double add(double a, double b) { return __dadd_rn(a, b); }
UFO_DEV double sub(double a, double b) { return __dsub_rn(a, b); }
UFO_DEV double dvd(double a, double b) { return __ddiv_rn(a, b); }
UFO_DEV double fma_(double a, double b, double c) { return __fma_rn(a, b, c); }
UFO_DEV double ld(const double *p) { return __ldg(p); }

// not finite: exponent field all ones (integer test, no FP64 pipe)
UFO_DEV bool nf(double v) { return (__double2hiint(v) & 0x7ff00000) == 0x7ff00000; }

// Correctly rounded a/d given r = RN(1/d): q0 = RN(a*r) is within an ulp of a/d
// and Markstein's correction q = RN(q0 + RN(a - q0*d)*r) (the remainder is
// exact under FMA) returns RN(a/d) (P. Markstein, IBM J. Res. Dev. 34 (1990);
// Muller et al., Handbook of Floating-Point Arithmetic, ch. 4).  Operands far
// from the unit range, zeros and non-finite values take IEEE division.
__device__ __noinline__ double div_ieee(double a, double d) { return __ddiv_rn(a, d); }

UFO_DEV double divc(double a, double d, double r) {
  const unsigned e = static_cast<unsigned>(__double2hiint(a)) & 0x7ff00000u;
  if (e < 0x07700000u || e > 0x77f00000u) return div_ieee(a, d);
  const double q0 = mul(a, r);
  const double rem = fma_(-q0, d, a);
  return fma_(rem, r, q0);
}

// reciprocals of the Horner orders 1..32, RN(1/k)
__constant__ double c_rcp_order[33];
// reciprocal factorials RN(1/n!), n = 0..32 (FMA-mode power-series kicks)
__constant__ double c_rcp_fact[33];

UFO_DEV double div_order(double a, int order) {
  if (order == 1) return a;
  if (order == 2) return mul(a, 0.5);
  if (order == 4) return mul(a, 0.25);
  return divc(a, static_cast<double>(order), c_rcp_order[order]);
}

struct State {
  double x, px, y, py, z, dp, o, opdp;  // o = 1/(1+dp); opdp = 1+dp (exact drift)
  int turn;
  bool bad_o;  // oodppo not finite: every kick takes the untrimmed path
};

// ---------------------------------------------------------------- drifts
// methods.drift (ufo/methods.py:28-43) on the pasted length text
template <bool FMA>
UFO_DEV void drift(State &s, int form, bool exact, const double *c) {
  if (exact) {
    // l = {length} / sqrt(opdp*opdp - px*px - py*py): the length text folds to c[0]
    const double l = dvd(ld(c), __dsqrt_rn(sub(sub(mul(s.opdp, s.opdp), mul(s.px, s.px)),
                                                mul(s.py, s.py))));
    if (FMA) {
      s.x = fma_(s.px, l, s.x);
      s.y = fma_(s.py, l, s.y);
    } else {
      s.x = add(s.x, mul(s.px, l));
      s.y = add(s.y, mul(s.py, l));
    }
    return;
  }
  if (form == DF_MUL) {  // x += px * L
    const double L = ld(c);
    if (FMA) {
      s.x = fma_(s.px, L, s.x);
      s.y = fma_(s.py, L, s.y);
    } else {
      s.x = add(s.x, mul(s.px, L));
      s.y = add(s.y, mul(s.py, L));
    }
  } else if (form == DF_MUL2) {  // x += px * L * f  ==  x + ((px*L)*f)
    const double L = ld(c), f = ld(c + 1);
    if (FMA) {
      s.x = fma_(mul(s.px, L), f, s.x);
      s.y = fma_(mul(s.py, L), f, s.y);
    } else {
      s.x = add(s.x, mul(mul(s.px, L), f));
      s.y = add(s.y, mul(mul(s.py, L), f));
    }
  } else {  // x += px * (A) / d  ==  x + ((px*A)/d)
    if (FMA) {
      const double aod = ld(c + 3);
      s.x = fma_(s.px, aod, s.x);
      s.y = fma_(s.py, aod, s.y);
    } else {
      const double A = ld(c), d = ld(c + 1), r = ld(c + 2);
      if (nf(s.px) || nf(s.py)) {
        s.x = add(s.x, dvd(mul(s.px, A), d));
        s.y = add(s.y, dvd(mul(s.py, A), d));
      } else {
        s.x = add(s.x, divc(mul(s.px, A), d, r));
        s.y = add(s.y, divc(mul(s.py, A), d, r));
      }
    }
  }
}

UFO_DEV int drift_nconst(int form, bool exact) {
  return exact ? 1 : (form == DF_MUL ? 1 : form == DF_MUL2 ? 2 : 4);
}

// ---------------------------------------------------------------- kicks
// methods.kick (ufo/methods.py:45-76).  Normal part, with a = dpx, b = dpy:
//   a = c[n-1]*o; b = 0
//   for order = n-1..1: na = (a*x - b*y)/order; nb = (a*y + b*x)/order;
//                        a = c[order-1]*o + na; b = nb
//   px -= a; py += b
// Skew part, with a = dpy, b = dpx:
//   na = (b*y + a*x)/order; nb = (b*x - a*y)/order; a = s[order-1]*o + na
//   px -= b; py += a
// `c` holds the structurally non-zero coefficients in ascending order.

// untrimmed evaluation (reference semantics incl. 0*x terms): `coef(j)` gives
// coefficient j of the list
template <bool SKEW, class Coef>
UFO_DEV void horner_any(const State &s, int n, Coef coef, bool achro, double &pxd,
                        double &pyd) {
  double a = achro ? coef(n - 1) : mul(coef(n - 1), s.o);
  double b = 0.0;
  for (int order = n - 1; order > 0; --order) {
    double na, nb;
    if (!SKEW) {
      na = dvd(sub(mul(a, s.x), mul(b, s.y)), static_cast<double>(order));
      nb = dvd(add(mul(a, s.y), mul(b, s.x)), static_cast<double>(order));
    } else {
      na = dvd(add(mul(b, s.y), mul(a, s.x)), static_cast<double>(order));
      nb = dvd(sub(mul(b, s.x), mul(a, s.y)), static_cast<double>(order));
    }
    a = achro ? add(coef(order - 1), na) : add(mul(coef(order - 1), s.o), na);
    b = nb;
  }
  if (!SKEW) {
    pxd = a;
    pyd = b;
  } else {
    pxd = b;
    pyd = a;
  }
}

// the untrimmed kick on table coefficients (non-finite x/y): coefficient j is
// its value if bit j of the mask is set, else a literal 0.
template <bool SKEW>
UFO_DEV void horner_full(const State &s, int n, uint32_t mask, const double *c, bool achro,
                         double &pxd, double &pyd) {
  horner_any<SKEW>(s, n, [&](int j) -> double {
    if (!((mask >> j) & 1u)) return 0.0;
    return ld(c + __popc(mask & ((1u << j) - 1u)));
  }, achro, pxd, pyd);
}

// trimmed evaluation: za/zb mark exact (structural) zeros
// One step of the recurrence.  After the top non-zero coefficient m the shape
// is fixed: the first step (order m) has b == 0 exactly, every later step has
// both accumulators non-zero; steps differ only in the divisor (1, 2, 4 or a
// general order) and in whether coefficient order-1 is added.  Each
// combination is a separate instantiation selected by a switch, so no FP64
// instruction is predicated.
template <bool FMA, bool SKEW, bool FIRST, int DK, bool COEF>
UFO_DEV void hstep(const State &s, double &a, double &b, int order, const double *cp, double o1) {
  double na, nb;
  if (FIRST) {  // b is an exact zero
    na = mul(a, s.x);
    nb = SKEW ? -mul(a, s.y) : mul(a, s.y);
  } else if (!SKEW) {
    na = FMA ? fma_(a, s.x, -mul(b, s.y)) : sub(mul(a, s.x), mul(b, s.y));
    nb = FMA ? fma_(a, s.y, mul(b, s.x)) : add(mul(a, s.y), mul(b, s.x));
  } else {
    na = FMA ? fma_(b, s.y, mul(a, s.x)) : add(mul(b, s.y), mul(a, s.x));
    nb = FMA ? fma_(b, s.x, -mul(a, s.y)) : sub(mul(b, s.x), mul(a, s.y));
  }
  if (DK == 1) {
    na = mul(na, 0.5);
    nb = mul(nb, 0.5);
  } else if (DK == 2) {
    na = mul(na, 0.25);
    nb = mul(nb, 0.25);
  } else if (DK == 3) {
    const double r = c_rcp_order[order];
    if (FMA) {
      na = mul(na, r);
      nb = mul(nb, r);
    } else {
      const double d = static_cast<double>(order);
      na = divc(na, d, r);
      nb = divc(nb, d, r);
    }
  }
  if (COEF) {
    const double cc = ld(cp);  // achromatic: o1 == 1.0 and cc*1.0 == cc exactly
    a = FMA ? fma_(cc, o1, na) : add(mul(cc, o1), na);
  } else {
    a = na;
  }
  b = nb;
}

template <bool FMA, bool SKEW>
UFO_DEV void horner_trim(const State &s, int n, uint32_t mask, const double *c, bool achro,
                         double &pxd, bool &zpx, double &pyd, bool &zpy) {
  (void)n;
  if (mask == 0u) {
    pxd = pyd = 0.0;
    zpx = zpy = true;
    return;
  }
  const int m = 31 - __clz(mask);  // top non-zero coefficient
  int k = __popc(mask) - 1;        // its index in c
  const double o1 = achro ? 1.0 : s.o;
  double a = mul(ld(c + k), o1), b = 0.0;
  --k;
  for (int order = m; order > 0; --order) {
    const int dk = order == 1 ? 0 : order == 2 ? 1 : order == 4 ? 2 : 3;
    const bool coef = (mask >> (order - 1)) & 1u;
    const double *cp = c + (k < 0 ? 0 : k);
    switch ((order == m ? 1 : 0) | (dk << 1) | (coef ? 8 : 0)) {
      case 0: hstep<FMA, SKEW, false, 0, false>(s, a, b, order, cp, o1); break;
      case 1: hstep<FMA, SKEW, true, 0, false>(s, a, b, order, cp, o1); break;
      case 2: hstep<FMA, SKEW, false, 1, false>(s, a, b, order, cp, o1); break;
      case 3: hstep<FMA, SKEW, true, 1, false>(s, a, b, order, cp, o1); break;
      case 4: hstep<FMA, SKEW, false, 2, false>(s, a, b, order, cp, o1); break;
      case 5: hstep<FMA, SKEW, true, 2, false>(s, a, b, order, cp, o1); break;
      case 6: hstep<FMA, SKEW, false, 3, false>(s, a, b, order, cp, o1); break;
      case 7: hstep<FMA, SKEW, true, 3, false>(s, a, b, order, cp, o1); break;
      case 8: hstep<FMA, SKEW, false, 0, true>(s, a, b, order, cp, o1); break;
      case 9: hstep<FMA, SKEW, true, 0, true>(s, a, b, order, cp, o1); break;
      case 10: hstep<FMA, SKEW, false, 1, true>(s, a, b, order, cp, o1); break;
      case 11: hstep<FMA, SKEW, true, 1, true>(s, a, b, order, cp, o1); break;
      case 12: hstep<FMA, SKEW, false, 2, true>(s, a, b, order, cp, o1); break;
      case 13: hstep<FMA, SKEW, true, 2, true>(s, a, b, order, cp, o1); break;
      case 14: hstep<FMA, SKEW, false, 3, true>(s, a, b, order, cp, o1); break;
      default: hstep<FMA, SKEW, true, 3, true>(s, a, b, order, cp, o1); break;
    }
    if (coef) --k;
  }
  // normal: a = dpx, b = dpy; skew: a = dpy, b = dpx.  b is an exact zero
  // only when the kick has a single (order 0) coefficient.
  if (!SKEW) {
    pxd = a; zpx = false;
    pyd = b; zpy = (m == 0);
  } else {
    pxd = b; zpx = (m == 0);
    pyd = a; zpy = false;
  }
}

struct PxPy { double px, py; };

// FMA mode, sextupole kick with t = (K*o)/2 and t2 = 2t = K*o:
//   px -= t (x^2 - y^2),  py += t2 x y
// 2 DMUL + 3 DFMA instead of the reference's form's 2 DMUL + 4 DFMA
UFO_DEV void sext_fma(State &s, double t, double t2) {
  const double d = fma_(s.x, s.x, -mul(s.y, s.y));
  const double xy = mul(s.x, s.y);
  s.px = fma_(-t, d, s.px);
  s.py = fma_(t2, xy, s.py);
}

// FMA mode, general multipole.  The reference's kick (ufo/methods.py:45-76)
// runs one real Horner pass for the normal and one for the skew list, dividing
// by the order at every step; both are the one complex polynomial
//   S(z) = sum_n (kn_n + i ks_n) z^n / n!,   px -= o Re S,  py += o Im S,
// evaluated here by a single complex Horner pass over the power-series
// coefficients (4 DFMA and 2 scalings per order instead of ~14 instructions).
// Coefficients absent from the table (structural zeros) enter as 0.  (pr, pi)
// is S/o.
UFO_DEV void poly_cplx(double x, double y, uint32_t mn, uint32_t ms, const double *c,
                       double &pr, double &pi) {
  const uint32_t mm = mn | ms;
  const double *cs = c + __popc(mn);
  int n = 31 - __clz(mm);
  {
    const uint32_t below = (1u << n) - 1u;
    const double cr = ((mn >> n) & 1u) ? ld(c + __popc(mn & below)) : 0.0;
    const double ci = ((ms >> n) & 1u) ? ld(cs + __popc(ms & below)) : 0.0;
    const double rf = c_rcp_fact[n];
    pr = mul(cr, rf);
    pi = mul(ci, rf);
  }
  for (--n; n >= 0; --n) {
    const uint32_t below = (1u << n) - 1u;
    const double cr = ((mn >> n) & 1u) ? ld(c + __popc(mn & below)) : 0.0;
    const double ci = ((ms >> n) & 1u) ? ld(cs + __popc(ms & below)) : 0.0;
    const double rf = c_rcp_fact[n];
    const double tr = fma_(pr, x, fma_(-pi, y, mul(cr, rf)));
    pi = fma_(pr, y, fma_(pi, x, mul(ci, rf)));
    pr = tr;
  }
}

// px -= f Re S/o, py += f Im S/o with f = w o (w = 1 for a plain kick);
// mn | ms != 0.  Out of line: inlined, its live values would cost every
// interpreter instantiation occupancy.
__device__ __noinline__ PxPy kick_cplx_ool(double x, double y, double px, double py, double f,
                                           uint32_t mn, uint32_t ms, const double *c) {
  double pr, pi;
  poly_cplx(x, y, mn, ms, c, pr, pi);
  return {fma_(-f, pr, px), fma_(f, pi, py)};
}

// The same kick from a dense power series prepared on the host (F_PSER:
// a_n = RN(kn_n * RN(1/n!)), then b_n, n < M): the products poly_cplx forms at
// every order are loaded instead, so the result is the same bit for bit with
// 4 FMAs per order.
__device__ __noinline__ PxPy kick_pser_ool(double x, double y, double px, double py, double f,
                                           int M, const double *c) {
  double pr = ld(c + M - 1), pi = ld(c + 2 * M - 1);
  for (int n = M - 2; n >= 0; --n) {
    const double tr = fma_(pr, x, fma_(-pi, y, ld(c + n)));
    pi = fma_(pr, y, fma_(pi, x, ld(c + M + n)));
    pr = tr;
  }
  return {fma_(-f, pr, px), fma_(f, pi, py)};
}

// terms of the dense series of a kick with masks mn, ms (highest order + 1)
UFO_DEV int pser_len(uint32_t mn, uint32_t ms) { return 32 - __clz(mn | ms); }

UFO_DEV void kick_cplx(State &s, uint32_t mn, uint32_t ms, const double *c, bool achro,
                       double w = 1.0) {
  const double f = mul(achro ? 1.0 : s.o, w);
  const PxPy r = kick_cplx_ool(s.x, s.y, s.px, s.py, f, mn, ms, c);
  s.px = r.px;
  s.py = r.py;
}

// quadrupole / sextupole shapes have their own short forms
UFO_DEV bool kick_is_general(int nn, int ns, uint32_t mn, uint32_t ms) {
  if (ms != 0u) return true;
  return !((nn == 2 && mn == 2u) || (nn == 3 && mn == 4u) || mn == 0u);
}

// one kick; `bad` selects the untrimmed path.  nn/ns: list lengths, mn/ms: masks
template <bool FMA>
UFO_DEV void kick(State &s, int nn, int ns, uint32_t mn, uint32_t ms, const double *c,
                  bool achro, bool bad) {
  const double *cs = c + __popc(mn);
  if (FMA && !bad && kick_is_general(nn, ns, mn, ms)) {
    kick_cplx(s, mn, ms, c, achro);
    return;
  }
  if (bad) {
    if (nn) {
      double a, b;
      horner_full<false>(s, nn, mn, c, achro, a, b);
      s.px = sub(s.px, a);
      s.py = add(s.py, b);
    }
    if (ns) {
      double a, b;
      horner_full<true>(s, ns, ms, cs, achro, a, b);
      s.px = sub(s.px, a);
      s.py = add(s.py, b);
    }
    return;
  }
  if (nn) {
    if (nn == 2 && mn == 2u) {
      // quadrupole: px -= (K*o)*x; py += (K*o)*y
      const double t = achro ? ld(c) : mul(ld(c), s.o);
      if (FMA) {
        s.px = fma_(-t, s.x, s.px);
        s.py = fma_(t, s.y, s.py);
      } else {
        s.px = sub(s.px, mul(t, s.x));
        s.py = add(s.py, mul(t, s.y));
      }
    } else if (nn == 3 && mn == 4u) {
      // sextupole: a = ((K*o)*x)/2 = ((K*o)*0.5)*x exactly (power-of-two scaling)
      const double t = mul(achro ? ld(c) : mul(ld(c), s.o), 0.5);
      if (FMA) {
        sext_fma(s, t, add(t, t));
      } else {
        const double a = mul(t, s.x), b = mul(t, s.y);
        s.px = sub(s.px, sub(mul(a, s.x), mul(b, s.y)));
        s.py = add(s.py, add(mul(a, s.y), mul(b, s.x)));
      }
    } else {
      double a, b;
      bool za, zb;
      horner_trim<FMA, false>(s, nn, mn, c, achro, a, za, b, zb);
      if (!za) s.px = sub(s.px, a);
      if (!zb) s.py = add(s.py, b);
    }
  }
  if (ns) {
    double a, b;
    bool za, zb;
    horner_trim<FMA, true>(s, ns, ms, cs, achro, a, za, b, zb);
    if (!za) s.px = sub(s.px, a);
    if (!zb) s.py = add(s.py, b);
  }
}

// weak focusing of a teapot slice: px -= x * W (ufo/methods.py:84)
template <bool FMA>
UFO_DEV void weak(State &s, int flags, double W, bool bad) {
  if (flags & F_WEAK) {
    s.px = FMA ? fma_(-s.x, W, s.px) : sub(s.px, mul(s.x, W));
  } else if (bad) {
    s.px = sub(s.px, mul(s.x, 0.0));  // structurally zero: only NaN/inf propagate
  }
}


// out-of-line kick (defined at the end of this file)
struct P4 { double x, px, y, py; };
template <bool FMA>
__device__ __noinline__ PxPy kick_ool(double x, double y, double px, double py, double o,
                                      bool bad_o, int nn, int ns, uint32_t mn, uint32_t ms,
                                      const double *c, bool achro, bool bad);

// ---------------------------------------------------------------- teapot
// methods.teapot (ufo/methods.py:79-97): outer drift, N-1 x (kick, weak,
// inner drift), kick, weak, outer drift.  Table: [outer][inner][kick][W], then the exit
// outer drift when it differs from the entry (F_SPLITO: an FMA-mode program folded a
// neighbouring plain drift into one of them).
//
// The FP64 pipe of this GPU charges a predicated-off instruction like an
// executed one, so no runtime `if` may guard FP64 arithmetic in the hot path:
// every variant (kick pattern x inner-drift form x weak term) is its own
// instantiation reached through a switch, and the rare paths (non-finite
// coordinates, general multipoles) are out-of-line calls.
//
// Kick pattern.  The reference recomputes (K*oodppo) in every slice; it is
// the same value each time, so it is formed once per element.
//   1: quadrupole  px -= t*x, py += t*y            t = K*o
//   2: sextupole   a = t*x, b = t*y; px -= a*x - b*y; py += a*y + b*x,
//                  t = (K*o)*0.5 (scaling by 0.5 commutes with rounding)
//   3: no kick terms (bend without gradient)
//   0: general Horner (out of line; FMA mode: one complex Horner pass, kick_cplx)
// Achromatic coefficients are multiplied by 1.0 instead of o (exact), so the
// choice needs no branch.

template <bool FMA>
UFO_DEV void drift_L(State &s, double L) {
  if (FMA) {
    s.x = fma_(s.px, L, s.x);
    s.y = fma_(s.py, L, s.y);
  } else {
    s.x = add(s.x, mul(s.px, L));
    s.y = add(s.y, mul(s.py, L));
  }
}

// x += px * (A) / d  ==  x + ((px*A)/d); FMA mode: x + px*(A/d)
template <bool FMA>
UFO_DEV void drift_div(State &s, const double *c) {
  if (FMA) {
    const double aod = ld(c + 3);
    s.x = fma_(s.px, aod, s.x);
    s.y = fma_(s.py, aod, s.y);
  } else {
    const double A = ld(c), d = ld(c + 1), r = ld(c + 2);
    s.x = add(s.x, divc(mul(s.px, A), d, r));
    s.y = add(s.y, divc(mul(s.py, A), d, r));
  }
}

// one slice with the untrimmed (reference) expressions: non-finite x or y
template <bool FMA>
__device__ __noinline__ PxPy slow_slice(double x, double y, double px, double py, double o,
                                        bool bad_o, int nn, int ns, uint32_t mn, uint32_t ms,
                                        const double *ck, bool achro, bool has_weak, double W);

template <bool FMA, int PAT, bool WEAK>
UFO_DEV void tp_slice(State &s, int nn, int ns, uint32_t mn, uint32_t ms, const double *ck,
                      bool achro, double t, double t2, double W, const double *ps = nullptr) {
  if (s.bad_o || nf(s.x) || nf(s.y)) {
    const PxPy r = slow_slice<FMA>(s.x, s.y, s.px, s.py, s.o, s.bad_o, nn, ns, mn, ms, ck, achro,
                                   WEAK, W);
    s.px = r.px;
    s.py = r.py;
    return;
  }
  if (PAT == 0) {
    if (FMA && ps) {  // t: the strength factor o (1 when achromatic)
      const PxPy r = kick_pser_ool(s.x, s.y, s.px, s.py, t, pser_len(mn, ms), ps);
      s.px = r.px;
      s.py = r.py;
    } else if (FMA && (mn | ms) != 0u) {
      kick_cplx(s, mn, ms, ck, achro);
    } else {
      const PxPy r = kick_ool<FMA>(s.x, s.y, s.px, s.py, s.o, s.bad_o, nn, ns, mn, ms, ck, achro,
                                   false);
      s.px = r.px;
      s.py = r.py;
    }
  } else if (PAT == 1) {
    if (FMA) {
      s.px = fma_(-t, s.x, s.px);
      s.py = fma_(t, s.y, s.py);
    } else {
      s.px = sub(s.px, mul(t, s.x));
      s.py = add(s.py, mul(t, s.y));
    }
  } else if (PAT == 2) {
    if (FMA) {
      sext_fma(s, t, t2);
    } else {
      const double a = mul(t, s.x), b = mul(t, s.y);
      s.px = sub(s.px, sub(mul(a, s.x), mul(b, s.y)));
      s.py = add(s.py, add(mul(a, s.y), mul(b, s.x)));
    }
  }
  if (WEAK) s.px = FMA ? fma_(-s.x, W, s.px) : sub(s.px, mul(s.x, W));
}

template <bool FMA, int PAT, bool DIVIN, bool WEAK>
UFO_DEV void teapot_v(State &s, const Op &op, const double *c) {
  const int N = op.i0, nn = op.i1, ns = op.i2;
  const uint32_t mn = static_cast<uint32_t>(op.i3), ms = static_cast<uint32_t>(op.i4);
  const bool achro = op.flags & F_ACHRO;
  const double Lo = ld(c);
  const double *ci = c + 1;
  const double *ck = ci + (N > 1 ? (DIVIN ? 4 : 1) : 0);
  const double W = WEAK ? ld(ck + __popc(mn) + __popc(ms)) : 0.0;
  const double o1 = achro ? 1.0 : s.o;
  double t = 0.0, t2 = 0.0;
  if (PAT == 1) t = mul(ld(ck), o1);
  if (PAT == 2) {  // t = (K*o)*0.5; the FMA form's 2t is K*o itself (exact)
    const double ko = mul(ld(ck), o1);
    t = mul(ko, 0.5);
    if (FMA) t2 = ko;
  }
  // general kicks of FMA programs: the dense series after every other constant
  const double *ps = nullptr;
  if (FMA && PAT == 0 && (op.flags & F_PSER)) {
    ps = ck + __popc(mn) + __popc(ms) + (WEAK ? 1 : 0) + ((op.flags & F_SPLITO) ? 1 : 0);
    t = o1;
  }
  const double Li = DIVIN ? 0.0 : ld(ci);
  drift_L<FMA>(s, Lo);
  for (int sl = 1; sl < N; ++sl) {
    tp_slice<FMA, PAT, WEAK>(s, nn, ns, mn, ms, ck, achro, t, t2, W, ps);
    if (DIVIN)
      drift_div<FMA>(s, ci);
    else
      drift_L<FMA>(s, Li);
  }
  tp_slice<FMA, PAT, WEAK>(s, nn, ns, mn, ms, ck, achro, t, t2, W, ps);
  // exit outer drift: its own constant after the others when a following
  // drift was merged into it (FMA programs)
  double Lx = Lo;
  if (op.flags & F_SPLITO) Lx = ld(ck + __popc(mn) + __popc(ms) + (WEAK ? 1 : 0));
  drift_L<FMA>(s, Lx);
}

// ---------------------------------------------------------------- Yoshida
// The build's 4th-order integrator (H. Yoshida, Phys. Lett. A 150 (1990) 262;
// no reference counterpart): each of the N slices of length h = L*f/N is
//   drift c0 h, kick w0, drift c1 h, kick w1, drift c2 h, kick w2, drift c3 h
// with c = (w1/2, (w0+w1)/2, (w0+w1)/2, w1/2), w = (w1, w0, w1),
// w1 = 1/(2 - 2^(1/3)), w0 = 1 - 2 w1.  A kick of weight w applies w times the
// slice's teapot kick (coefficients (k*L*f)/N) and w times its weak focusing.
// Table: [c0 h, c1 h, c2 h, c3 h][w0, w1, w2][kick][W].  The weighted kick
// strengths of the quadrupole/sextupole patterns are formed once per element.
template <bool FMA, int PAT, bool WEAK>
UFO_DEV void y_kick(State &s, int nn, int ns, uint32_t mn, uint32_t ms, const double *ck,
                    bool achro, double w, double t, double t2, double Ww,
                    const double *ps = nullptr) {
  if (PAT == 0 && FMA && ps) {
    const PxPy r = kick_pser_ool(s.x, s.y, s.px, s.py, mul(achro ? 1.0 : s.o, w),
                                 pser_len(mn, ms), ps);
    s.px = r.px;
    s.py = r.py;
  } else if (PAT == 0 && FMA && (mn | ms) != 0u) {
    kick_cplx(s, mn, ms, ck, achro, w);
  } else if (PAT == 0) {
    // unweighted kick from zero momenta: r = (-dpx, +dpy)
    const PxPy r = kick_ool<FMA>(s.x, s.y, 0.0, 0.0, s.o, s.bad_o, nn, ns, mn, ms, ck, achro,
                                 false);
    if (FMA) {
      s.px = fma_(w, r.px, s.px);
      s.py = fma_(w, r.py, s.py);
    } else {
      s.px = add(s.px, mul(w, r.px));
      s.py = add(s.py, mul(w, r.py));
    }
  } else if (PAT == 1) {
    if (FMA) {
      s.px = fma_(-t, s.x, s.px);
      s.py = fma_(t, s.y, s.py);
    } else {
      s.px = sub(s.px, mul(t, s.x));
      s.py = add(s.py, mul(t, s.y));
    }
  } else if (PAT == 2) {
    if (FMA) {
      sext_fma(s, t, t2);
    } else {
      const double a = mul(t, s.x), b = mul(t, s.y);
      s.px = sub(s.px, sub(mul(a, s.x), mul(b, s.y)));
      s.py = add(s.py, add(mul(a, s.y), mul(b, s.x)));
    }
  }
  if (WEAK) s.px = FMA ? fma_(-s.x, Ww, s.px) : sub(s.px, mul(s.x, Ww));
}

template <bool FMA, int PAT, bool WEAK>
UFO_DEV void yoshida_v(State &s, const Op &op, const double *c) {
  const int N = op.i0, nn = op.i1, ns = op.i2;
  const uint32_t mn = static_cast<uint32_t>(op.i3), ms = static_cast<uint32_t>(op.i4);
  const bool achro = op.flags & F_ACHRO;
  const double d0 = ld(c), d1 = ld(c + 1), d2 = ld(c + 2), d3 = ld(c + 3);
  const double w0 = ld(c + 4), w1 = ld(c + 5), w2 = ld(c + 6);
  const double *ck = c + 7;
  double t0 = 0.0, t1 = 0.0, t2 = 0.0, W0 = 0.0, W1 = 0.0, W2 = 0.0;
  if (PAT == 1 || PAT == 2) {
    const double o1 = achro ? 1.0 : s.o;
    double t = mul(ld(ck), o1);
    if (PAT == 2) t = mul(t, 0.5);
    t0 = mul(t, w0);
    t1 = mul(t, w1);
    t2 = mul(t, w2);
  }
  // doubled strengths of the FMA sextupole form
  const double u0 = (FMA && PAT == 2) ? add(t0, t0) : 0.0;
  const double u1 = (FMA && PAT == 2) ? add(t1, t1) : 0.0;
  const double u2 = (FMA && PAT == 2) ? add(t2, t2) : 0.0;
  if (WEAK) {
    const double W = ld(ck + __popc(mn) + __popc(ms));
    W0 = mul(W, w0);
    W1 = mul(W, w1);
    W2 = mul(W, w2);
  }
  const double *ps = (FMA && PAT == 0 && (op.flags & F_PSER))
                         ? ck + __popc(mn) + __popc(ms) + (WEAK ? 1 : 0)
                         : nullptr;
  for (int sl = 0; sl < N; ++sl) {
    drift_L<FMA>(s, d0);
    y_kick<FMA, PAT, WEAK>(s, nn, ns, mn, ms, ck, achro, w0, t0, u0, W0, ps);
    drift_L<FMA>(s, d1);
    y_kick<FMA, PAT, WEAK>(s, nn, ns, mn, ms, ck, achro, w1, t1, u1, W1, ps);
    drift_L<FMA>(s, d2);
    y_kick<FMA, PAT, WEAK>(s, nn, ns, mn, ms, ck, achro, w2, t2, u2, W2, ps);
    drift_L<FMA>(s, d3);
  }
}

// exact-Hamiltonian teapot (rare): generic, out of line
template <bool FMA>
__device__ __noinline__ P4 teapot_exact_ool(double x, double px, double y, double py,
                                            double opdp, double o, bool bad_o, Op op,
                                            const double *c);

template <bool FMA, bool FULL>
UFO_DEV void teapot(State &s, const Op &op, const double *c) {
  if (FULL && (op.flags & F_EXACT)) {
    const P4 r = teapot_exact_ool<FMA>(s.x, s.px, s.y, s.py, s.opdp, s.o, s.bad_o, op, c);
    s.x = r.x; s.px = r.px; s.y = r.y; s.py = r.py;
    return;
  }
  const int nn = op.i1, ns = op.i2;
  const uint32_t mn = static_cast<uint32_t>(op.i3);
  const int pat = ns != 0 ? 0 : (nn == 2 && mn == 2u) ? 1 : (nn == 3 && mn == 4u) ? 2
                 : mn == 0u ? 3 : 0;
  if (op.flags & F_YOSHIDA) {
    switch (pat | ((op.flags & F_WEAK) ? 4 : 0)) {
      case 0: yoshida_v<FMA, 0, false>(s, op, c); break;
      case 1: yoshida_v<FMA, 1, false>(s, op, c); break;
      case 2: yoshida_v<FMA, 2, false>(s, op, c); break;
      case 3: yoshida_v<FMA, 3, false>(s, op, c); break;
      case 4: yoshida_v<FMA, 0, true>(s, op, c); break;
      case 5: yoshida_v<FMA, 1, true>(s, op, c); break;
      case 6: yoshida_v<FMA, 2, true>(s, op, c); break;
      default: yoshida_v<FMA, 3, true>(s, op, c); break;
    }
    return;
  }
  const int fi = (op.flags >> SH_FINNER) & 3;
  const int v = pat | (fi == DF_DIV ? 4 : 0) | ((op.flags & F_WEAK) ? 8 : 0);
  switch (v) {
    case 0: teapot_v<FMA, 0, false, false>(s, op, c); break;
    case 1: teapot_v<FMA, 1, false, false>(s, op, c); break;
    case 2: teapot_v<FMA, 2, false, false>(s, op, c); break;
    case 3: teapot_v<FMA, 3, false, false>(s, op, c); break;
    case 4: teapot_v<FMA, 0, true, false>(s, op, c); break;
    case 5: teapot_v<FMA, 1, true, false>(s, op, c); break;
    case 6: teapot_v<FMA, 2, true, false>(s, op, c); break;
    case 7: teapot_v<FMA, 3, true, false>(s, op, c); break;
    case 8: teapot_v<FMA, 0, false, true>(s, op, c); break;
    case 9: teapot_v<FMA, 1, false, true>(s, op, c); break;
    case 10: teapot_v<FMA, 2, false, true>(s, op, c); break;
    case 11: teapot_v<FMA, 3, false, true>(s, op, c); break;
    case 12: teapot_v<FMA, 0, true, true>(s, op, c); break;
    case 13: teapot_v<FMA, 1, true, true>(s, op, c); break;
    case 14: teapot_v<FMA, 2, true, true>(s, op, c); break;
    default: teapot_v<FMA, 3, true, true>(s, op, c); break;
  }
}

// ---------------------------------------------------------------- edge
// methods.edge (ufo/methods.py:199-211):
//   curvature = A (* o);  psi = e - 2*curv*fringe/cos(e)*(1 + sin(e)^2)
//   px += x*curv*tan(e);  py -= y*curv*tan(psi)
// table: [A, T1, T2] or, per-particle psi, [A, T1, e, fringe, cos e, 1+sin^2 e]
// Generic form (all flags at run time): used out of line for the rare cases.
template <bool FULL>
UFO_DEV void edge(State &s, int flags, const double *c) {
  const bool achro = flags & F_ACHRO;
  if (!(flags & (F_T1 | F_T2)) && !(s.bad_o || nf(s.x) || nf(s.y))) return;
  const double curv = achro ? ld(c) : mul(ld(c), s.o);
  double t2;
  if (FULL && (flags & F_RTPSI)) {
    const double psi = sub(ld(c + 2), mul(dvd(mul(mul(2.0, curv), ld(c + 3)), ld(c + 4)),
                                          ld(c + 5)));
    t2 = tan(psi);
  } else {
    t2 = ld(c + 2);
  }
  const double x0 = s.x, y0 = s.y;
  const bool bad = nf(x0) || nf(y0) || nf(curv);
  if (flags & F_T1)
    s.px = add(s.px, mul(mul(x0, curv), ld(c + 1)));
  else if (bad)
    s.px = add(s.px, mul(mul(x0, curv), 0.0));
  if (flags & F_T2)
    s.py = sub(s.py, mul(mul(y0, curv), t2));
  else if (bad)
    s.py = sub(s.py, mul(mul(y0, curv), 0.0));
}

__device__ __noinline__ PxPy edge_ool(double x, double y, double px, double py, double o,
                                      bool bad_o, int flags, const double *c);

// hot-path edge with a constant tan(psi): T1/T2 presence known per variant
template <bool FMA, bool T1, bool T2>
UFO_DEV void edge_v(State &s, int flags, const double *c) {
  const bool achro = flags & F_ACHRO;
  if (!T1 && !T2) {
    if (s.bad_o || nf(s.x) || nf(s.y)) {
      const PxPy r = edge_ool(s.x, s.y, s.px, s.py, s.o, s.bad_o, flags, c);
      s.px = r.px;
      s.py = r.py;
    }
    return;
  }
  const double curv = mul(ld(c), achro ? 1.0 : s.o);
  if (nf(s.x) || nf(s.y) || nf(curv)) {
    const PxPy r = edge_ool(s.x, s.y, s.px, s.py, s.o, s.bad_o, flags, c);
    s.px = r.px;
    s.py = r.py;
    return;
  }
  const double x0 = s.x, y0 = s.y;
  if (T1) s.px = FMA ? fma_(mul(x0, curv), ld(c + 1), s.px) : add(s.px, mul(mul(x0, curv), ld(c + 1)));
  if (T2) s.py = FMA ? fma_(-mul(y0, curv), ld(c + 2), s.py) : sub(s.py, mul(mul(y0, curv), ld(c + 2)));
}

template <bool FMA, bool FULL>
UFO_DEV void edge_dispatch(State &s, int flags, const double *c) {
  if (FULL && (flags & F_RTPSI)) {
    const PxPy r = edge_ool(s.x, s.y, s.px, s.py, s.o, s.bad_o, flags, c);
    s.px = r.px;
    s.py = r.py;
    return;
  }
  switch ((flags & F_T1 ? 1 : 0) | (flags & F_T2 ? 2 : 0)) {
    case 0: edge_v<FMA, false, false>(s, flags, c); break;
    case 1: edge_v<FMA, true, false>(s, flags, c); break;
    case 2: edge_v<FMA, false, true>(s, flags, c); break;
    default: edge_v<FMA, true, true>(s, flags, c); break;
  }
}

// ---------------------------------------------------------------- thick
struct Trig { double C, S, CH, SH; };

UFO_DEV Trig trig(double k2l) {
  Trig t;
  sincos(k2l, &t.S, &t.C);
  t.CH = cosh(k2l);
  t.SH = sinh(k2l);
  return t;
}

// methods.quadrupole thick branch (ufo/methods.py:103-134);
// table [k, L*f, (k2, C, S, CH, SH)]
UFO_DEV void thick_quad(State &s, int flags, const double *c) {
  const double k = ld(c), Lf = ld(c + 1);
  double k2;
  Trig t;
  if (flags & F_CONST) {
    k2 = ld(c + 2);
    t.C = ld(c + 3); t.S = ld(c + 4); t.CH = ld(c + 5); t.SH = ld(c + 6);
  } else {
    k2 = __dsqrt_rn(fabs((flags & F_ACHRO) ? k : mul(k, s.o)));
    t = trig(mul(Lf, k2));
  }
  const double x0 = s.x, px0 = s.px, y0 = s.y, py0 = s.py;
  if (k > 0.) {
    s.x = add(mul(t.C, x0), dvd(mul(t.S, px0), k2));
    s.px = add(mul(mul(-t.S, x0), k2), mul(t.C, px0));
    s.y = add(mul(t.CH, y0), dvd(mul(t.SH, py0), k2));
    s.py = add(mul(mul(t.SH, y0), k2), mul(t.CH, py0));
  } else {
    s.x = add(mul(t.CH, x0), dvd(mul(t.SH, px0), k2));
    s.px = add(mul(mul(t.SH, x0), k2), mul(t.CH, px0));
    s.y = add(mul(t.C, y0), dvd(mul(t.S, py0), k2));
    s.py = add(mul(mul(-t.S, y0), k2), mul(t.C, py0));
  }
}

// methods.sbend thick branch (ufo/methods.py:140-196); table
// [A/L, k1, L*f, (kv, k2v, Cv, Sv, CHv, SHv, kx, k2x, Cx, Sx, CHx, SHx, |kx|)]
UFO_DEV void thick_bend(State &s, int flags, const double *c) {
  const bool achro = flags & F_ACHRO;
  const double Lf = ld(c + 2);
  const double curv = achro ? ld(c) : mul(ld(c), s.o);
  double k, k2;
  Trig t;
  const double x0 = s.x, px0 = s.px, y0 = s.y, py0 = s.py;
  if (flags & F_CONST) {
    k = ld(c + 3); k2 = ld(c + 4);
    t.C = ld(c + 5); t.S = ld(c + 6); t.CH = ld(c + 7); t.SH = ld(c + 8);
  } else {
    k = achro ? ld(c + 1) : mul(ld(c + 1), s.o);
    k2 = __dsqrt_rn(fabs(k));
    t = trig(mul(Lf, k2));
  }
  if (k > 0.) {
    s.y = add(mul(t.CH, y0), dvd(mul(t.SH, py0), k2));
    s.py = add(mul(mul(t.SH, y0), k2), mul(t.CH, py0));
  }
  if (k < 0.) {
    s.y = add(mul(t.C, y0), dvd(mul(t.S, py0), k2));
    s.py = add(mul(mul(-t.S, y0), k2), mul(t.C, py0));
  }
  if (k == 0.) s.y = add(s.y, mul(Lf, py0));
  double ak;
  if (flags & F_CONST) {
    k = ld(c + 9); k2 = ld(c + 10);
    t.C = ld(c + 11); t.S = ld(c + 12); t.CH = ld(c + 13); t.SH = ld(c + 14);
    ak = ld(c + 15);
  } else {
    k = add(k, achro ? mul(curv, curv) : dvd(mul(curv, curv), s.o));
    k2 = __dsqrt_rn(fabs(k));
    t = trig(mul(Lf, k2));
    ak = fabs(k);
  }
  if (k > 0.) {
    s.x = add(mul(t.C, x0), dvd(mul(t.S, px0), k2));
    s.x = add(s.x, dvd(mul(mul(s.dp, curv), sub(1., t.C)), ak));
    s.px = add(mul(mul(-t.S, x0), k2), mul(t.C, px0));
    s.px = add(s.px, dvd(mul(mul(s.dp, curv), t.S), k2));
  }
  if (k < 0.) {
    s.x = add(mul(t.CH, x0), dvd(mul(t.SH, px0), k2));
    s.x = add(s.x, dvd(mul(mul(s.dp, curv), sub(t.CH, 1.)), ak));
    s.px = add(mul(mul(t.SH, x0), k2), mul(t.CH, px0));
    s.px = add(s.px, dvd(mul(mul(s.dp, curv), t.SH), k2));
  }
  if (k == 0.) s.x = add(s.x, mul(Lf, px0));
}

// ---------------------------------------------------------------- wire
// methods.wire (ufo/methods.py:230-241); table [xw, yw, k]
UFO_DEV void wire(State &s, const double *c) {
  const double wx = ld(c), wy = ld(c + 1), wk = ld(c + 2);
  const double alpha = atan2(sub(wy, s.y), sub(wx, s.x));
  const double B = dvd(wk, hypot(sub(wx, s.x), sub(wy, s.y)));
  double sa, ca;
  sincos(alpha, &sa, &ca);
  s.px = add(s.px, mul(B, ca));
  s.py = add(s.py, mul(B, sa));
}

// ---------------------------------------------------------------- expressions
// stack programs of C expressions (ufo_gb300/cexpr.py): the table holds
// (opcode, value) pairs.  Opcodes 3,4,19,20,22-28 are unary, 21 is ?:, 1 and 2
// push a literal or a variable, the rest are binary.
UFO_DEV bool prog_unary(int op) { return op == 3 || op == 4 || op == 19 || op == 20 ||
                                         (op >= 22 && op <= 28); }

// value of a program in `out`; false (and `out` untouched) when the program
// would leave its stack of DEPTH slots
template <int DEPTH>
UFO_DEV bool eval_prog(const State &s, const double *c, int n, double &out) {
  double st[DEPTH];
  int sp = 0;
  for (int i = 0; i < n; ++i) {
    const int op = static_cast<int>(ld(c + 2 * i));
    const double v = ld(c + 2 * i + 1);
    // depth guards: a malformed program stops instead of leaving the stack
    const int need = (op == 1 || op == 2) ? 0 : prog_unary(op) ? 1 : op == 21 ? 3 : 2;
    if (sp < need || ((op == 1 || op == 2) && sp >= DEPTH)) return false;
    if (op == 1) { st[sp++] = v; continue; }
    if (op == 2) {
      const int k = static_cast<int>(v);
      st[sp++] = k == 0 ? s.x : k == 1 ? s.px : k == 2 ? s.y : k == 3 ? s.py : k == 4 ? s.z
               : k == 5 ? s.dp : k == 6 ? s.o : static_cast<double>(s.turn);
      continue;
    }
    if (prog_unary(op)) {
      const double a = st[sp - 1];
      double r;
      switch (op) {
        case 3: r = -a; break;
        case 4: r = a == 0 ? 1. : 0.; break;
        case 19: r = fabs(a); break;
        case 20: r = __dsqrt_rn(a); break;
        case 22: r = sin(a); break;
        case 23: r = cos(a); break;
        case 24: r = tan(a); break;
        case 25: r = exp(a); break;
        case 26: r = log(a); break;
        case 27: r = static_cast<double>(__double2float_rn(a)); break;  // (float)
        default: r = add(trunc(a), 0.0); break;                         // (int): no -0
      }
      st[sp - 1] = r;
      continue;
    }
    if (op == 21) {
      const double b = st[--sp], a = st[--sp], cc = st[--sp];
      st[sp++] = cc != 0 ? a : b;
      continue;
    }
    const double b = st[--sp], a = st[--sp];
    double r;
    switch (op) {
      case 5: r = add(a, b); break;
      case 6: r = sub(a, b); break;
      case 7: r = mul(a, b); break;
      case 8: r = dvd(a, b); break;
      // integer / and %: truncated, and never -0 (C ints have none)
      case 9: r = b != 0 ? add(trunc(dvd(a, b)), 0.0) : __longlong_as_double(0x7ff8000000000000ll);
        break;
      case 10: r = b != 0 ? add(fmod(a, b), 0.0) : __longlong_as_double(0x7ff8000000000000ll);
        break;
      case 11: r = a < b; break;
      case 12: r = a <= b; break;
      case 13: r = a > b; break;
      case 14: r = a >= b; break;
      case 15: r = a == b; break;
      case 16: r = a != b; break;
      case 17: r = (a != 0) && (b != 0); break;
      default: r = (a != 0) || (b != 0); break;
    }
    st[sp++] = r;
  }
  if (sp < 1) return false;
  out = st[sp - 1];
  return true;
}

// ``{window} == 0`` of an aperture (ufo_gb300/aperture.py): true when lost
UFO_DEV bool aperture_lost(const State &s, const double *c, int n) {
  double v;
  return eval_prog<16>(s, c, n, v) && v != 0;
}

UFO_DEV void align(State &s, int flags, const double *c) {
  if (flags & F_AX) s.x = sub(s.x, ld(c));
  if (flags & F_AY) s.y = sub(s.y, ld(c + 1));
}

}  // namespace ufo

namespace ufo {

// ------------------------------------------------------- out-of-line paths
// Rare or heavy ops run out of line with by-value arguments, so the caller's
// particle state stays in registers and the hot interpreter loop keeps a
// small register footprint (the FP64 pipe is per SM: all of a launch's warps
// must be resident at once).
template <bool FMA>
__device__ __noinline__ PxPy kick_ool(double x, double y, double px, double py, double o,
                                      bool bad_o, int nn, int ns, uint32_t mn, uint32_t ms,
                                      const double *c, bool achro, bool bad) {
  State s{};
  s.x = x; s.y = y; s.px = px; s.py = py; s.o = o; s.bad_o = bad_o;
  kick<FMA>(s, nn, ns, mn, ms, c, achro, bad);
  return {s.px, s.py};
}

__device__ __noinline__ P4 thick_quad_ool(double x, double px, double y, double py, double o,
                                          int flags, const double *c) {
  State s{};
  s.x = x; s.px = px; s.y = y; s.py = py; s.o = o;
  thick_quad(s, flags, c);
  return {s.x, s.px, s.y, s.py};
}

__device__ __noinline__ P4 thick_bend_ool(double x, double px, double y, double py, double dp,
                                          double o, int flags, const double *c) {
  State s{};
  s.x = x; s.px = px; s.y = y; s.py = py; s.dp = dp; s.o = o;
  thick_bend(s, flags, c);
  return {s.x, s.px, s.y, s.py};
}

__device__ __noinline__ P4 wire_ool(double x, double px, double y, double py, const double *c) {
  State s{};
  s.x = x; s.px = px; s.y = y; s.py = py;
  wire(s, c);
  return {s.x, s.px, s.y, s.py};
}

__device__ __noinline__ bool aperture_ool(double x, double px, double y, double py, double z,
                                          double dp, double o, int turn, const double *c, int n) {
  State s{};
  s.x = x; s.px = px; s.y = y; s.py = py; s.z = z; s.dp = dp; s.o = o; s.turn = turn;
  return aperture_lost(s, c, n);
}

// A thin kick whose coefficients are programs (a user pass method's C text,
// ufo_gb300/compiler.py: _dyn_kick): table [n, (opcode, value) x n] per
// coefficient, normal then skew, `words` entries in all.  The reference's
// untrimmed Horner in its operation order (methods.kick, ufo/methods.py:45-76)
// in both arithmetic modes.  Every read stays within the op's `words` table
// entries; a malformed program yields a NaN coefficient.
__device__ __noinline__ PxPy dynkick_ool(double x, double px, double y, double py, double z,
                                         double dp, double o, int turn, int nn, int ns,
                                         bool achro, int words, const double *c) {
  State s{};
  s.x = x; s.px = px; s.y = y; s.py = py; s.z = z; s.dp = dp; s.o = o; s.turn = turn;
  auto coef = [&](int j) -> double {
    double v = __longlong_as_double(0x7ff8000000000000ll);
    int q = 0;
    for (int k = 0; k <= j; ++k) {
      if (q >= words) return v;
      const double len = ld(c + q);
      if (!(len >= 1.0 && len <= 0.5 * (words - q - 1))) return v;
      if (k == j) {
        eval_prog<32>(s, c + q + 1, static_cast<int>(len), v);
        return v;
      }
      q += 1 + 2 * static_cast<int>(len);
    }
    return v;
  };
  if (nn) {
    double a, b;
    horner_any<false>(s, nn, coef, achro, a, b);
    s.px = sub(s.px, a);
    s.py = add(s.py, b);
  }
  if (ns) {
    double a, b;
    horner_any<true>(s, ns, [&](int j) { return coef(nn + j); }, achro, a, b);
    s.px = sub(s.px, a);
    s.py = add(s.py, b);
  }
  return {s.px, s.py};
}

__device__ __noinline__ PxPy edge_ool(double x, double y, double px, double py, double o,
                                      bool bad_o, int flags, const double *c) {
  State s{};
  s.x = x; s.y = y; s.px = px; s.py = py; s.o = o; s.bad_o = bad_o;
  edge<true>(s, flags, c);
  return {s.px, s.py};
}

}  // namespace ufo

namespace ufo {

template <bool FMA>
__device__ __noinline__ PxPy slow_slice(double x, double y, double px, double py, double o,
                                        bool bad_o, int nn, int ns, uint32_t mn, uint32_t ms,
                                        const double *ck, bool achro, bool has_weak, double W) {
  State s{};
  s.x = x; s.y = y; s.px = px; s.py = py; s.o = o; s.bad_o = bad_o;
  kick<FMA>(s, nn, ns, mn, ms, ck, achro, true);
  s.px = sub(s.px, mul(s.x, has_weak ? W : 0.0));
  return {s.px, s.py};
}

// the generic teapot with exact drifts (EXACT flag)
template <bool FMA>
__device__ __noinline__ P4 teapot_exact_ool(double x, double px, double y, double py,
                                            double opdp, double o, bool bad_o, Op op,
                                            const double *c) {
  State s{};
  s.x = x; s.px = px; s.y = y; s.py = py; s.opdp = opdp; s.o = o; s.bad_o = bad_o;
  const int N = op.i0, nn = op.i1, ns = op.i2;
  const uint32_t mn = static_cast<uint32_t>(op.i3), ms = static_cast<uint32_t>(op.i4);
  const bool achro = op.flags & F_ACHRO;
  const double *co = c, *ci = c + 1, *ck = ci + (N > 1 ? 1 : 0);
  const bool has_weak = op.flags & F_WEAK;
  const double W = has_weak ? ld(ck + __popc(mn) + __popc(ms)) : 0.0;
  drift<FMA>(s, DF_MUL, true, co);
  for (int sl = 0; sl < N; ++sl) {
    const bool bad = s.bad_o || nf(s.x) || nf(s.y);
    kick<FMA>(s, nn, ns, mn, ms, ck, achro, bad);
    if (has_weak)
      s.px = FMA ? fma_(-s.x, W, s.px) : sub(s.px, mul(s.x, W));
    else if (bad)
      s.px = sub(s.px, mul(s.x, 0.0));
    if (sl < N - 1) drift<FMA>(s, DF_MUL, true, ci);
  }
  drift<FMA>(s, DF_MUL, true, co);
  return {s.x, s.px, s.y, s.py};
}

}  // namespace ufo
