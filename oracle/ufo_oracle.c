/*
 * ufo_oracle.c -- CPU restatement of the reference's FP64 tracking arithmetic.
 *
 * TEST INFRASTRUCTURE. This file is the parity oracle: the tests, the smoke
 * check and the CPU baseline of bench.py run it to check the CUDA kernels.
 * The product path (ufo_gb300) never links or calls it.
 *
 * It restates, operation for operation, the OpenCL C that the reference
 * generates:
 *   align            ufo/methods.py:22-26
 *   drift (+EXACT)   ufo/methods.py:28-43
 *   kick (Horner)    ufo/methods.py:45-76
 *   teapot           ufo/methods.py:79-97
 *   quadrupole       ufo/methods.py:99-134    (KICK -> teapot, else thick)
 *   sbend            ufo/methods.py:136-196
 *   edge             ufo/methods.py:199-211
 *   sextupole/octup. ufo/methods.py:213-227   (dks passed, k2s/k3s ignored)
 *   wire             ufo/methods.py:230-241
 *   aperture         ufo/elements.py:517-518
 *   element wrappers ufo/elements.py:98-106,152-167,200-219,260-285,326-352,
 *                    392-413,447-468,494-500
 *   Track scaffold   ufo/track.py:84-114      (loss = isnan(x) per turn)
 *   SA scaffold      ufo/sa.py:93-126         (loss = |x|>1 || |y|>1 || isnan(x))
 * Every expression is written with the reference's C association
 * (left-to-right, no contraction: compile with -ffp-contract=off), and it
 * works from element attributes, not from the opcode table the GPU path uses.
 * Transcendentals that a C compiler folds because their arguments are
 * literals arrive precomputed (correctly rounded) in `fold`; all others call
 * the C library at run time, as the reference's kernel does.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define F_LINEAR 1
#define F_FIVED 2
#define F_EXACT 4
#define F_KICK 8
#define F_ACHRO 64

enum { T_MARKER = 0, T_DRIFT, T_MULTIPOLE, T_QUAD, T_SBEND, T_RBEND, T_SEXT, T_OCT, T_WIRE,
       T_APERTURE, T_DYNMULT };

/* one flat element of one seed; lists live in `mp`, fractures in `frac`,
 * folded transcendentals in `fold`, aperture programs in `ap` */
typedef struct {
    int32_t type, slices;
    int32_t nknl, nksl, ndkn, ndks, mp_off;   /* knl | ksl | dkn | dks */
    int32_t nfrac, frac_off, pre_dump;        /* fracture fractions, dump before */
    int32_t ap_off, ap_len;                   /* (opcode, value) pairs */
    int32_t fold_off, fold_achro;             /* folded constants offset; set when oodppo
                                                 is a compile-time constant */
    double length, angle, k1, e1, e2, hgap, fint, dx, dy, k2, k2s, k3, k3s, wx, wy, wk;
} oelem;

typedef struct { double x, px, y, py, z, dp, oodppo; int turn; } state;

static void align_(state *s, double dx, double dy) { s->x -= dx; s->y -= dy; }

/* drift length text: form 0 "c0", 1 "c0 * c1" (Drift element piece),
 * 2 "(c0) / c1" (teapot inner drift) */
static void drift_(state *s, int flags, int form, double c0, double c1) {
    if (flags & F_EXACT) {
        double lc = form == 1 ? c0 * c1 : form == 2 ? c0 / c1 : c0;
        double opdp = 1. + s->dp;
        double l = lc / sqrt(opdp * opdp - s->px * s->px - s->py * s->py);
        s->x += s->px * l;
        s->y += s->py * l;
    } else if (form == 1) {
        s->x += s->px * c0 * c1;
        s->y += s->py * c0 * c1;
    } else if (form == 2) {
        s->x += s->px * c0 / c1;
        s->y += s->py * c0 / c1;
    } else {
        s->x += s->px * c0;
        s->y += s->py * c0;
    }
}

static void kick_(state *s, int flags, const double *knl, int nn, const double *ksl, int ns) {
    const int ach = flags & F_ACHRO;
    const double o = s->oodppo;
    if (nn) {
        int mo = (flags & F_LINEAR) ? (nn < 2 ? nn : 2) : nn;
        double dpx = ach ? knl[mo - 1] : knl[mo - 1] * o;
        double dpy = 0.;
        for (int order = mo - 1; order > 0; --order) {
            double aux = (dpx * s->x - (dpy * s->y)) / order;
            double ndpy = (dpx * s->y + (dpy * s->x)) / order;
            dpx = ach ? (knl[order - 1] + aux) : (knl[order - 1] * o + aux);
            dpy = ndpy;
        }
        s->px -= dpx;
        s->py += dpy;
    }
    if (ns) {
        int mo = (flags & F_LINEAR) ? (ns < 2 ? ns : 2) : ns;
        double dpy = ach ? ksl[mo - 1] : ksl[mo - 1] * o;
        double dpx = 0.;
        for (int order = mo - 1; order > 0; --order) {
            double aux = (dpx * s->y + (dpy * s->x)) / order;
            double ndpx = (dpx * s->x - (dpy * s->y)) / order;
            dpy = ach ? (ksl[order - 1] + aux) : (ksl[order - 1] * o + aux);
            dpx = ndpx;
        }
        s->px -= dpx;
        s->py += dpy;
    }
}

/* teapot over the pasted length text "L * f" */
static void teapot_(state *s, int flags, double L, double f, int N, const double *knl0, int nn,
                    const double *ksl0, int ns, int has_angle, double A) {
    double kn[64], ks[64];
    const double Lf = L * f;
    const double outer = N == 1 ? (Lf / 2.) : (Lf / (2 * (1 + N)));
    const double inner_a = Lf - 2. * outer;
    const double inner_d = N - 1.;
    double weak;
    if (has_angle) {
        const double Af = A * f;
        weak = Af * Af * Lf / N / Lf / Lf;
    } else {
        weak = 0.0 * Lf / N / Lf / Lf;
    }
    for (int j = 0; j < nn; ++j) kn[j] = knl0[j] * L * f / N;
    for (int j = 0; j < ns; ++j) ks[j] = ksl0[j] * L * f / N;
    drift_(s, flags, 0, outer, 0.);
    for (int c = 0; c < N - 1; ++c) {
        kick_(s, flags, kn, nn, ks, ns);
        s->px -= s->x * weak;
        drift_(s, flags, 2, inner_a, inner_d);
    }
    kick_(s, flags, kn, nn, ks, ns);
    s->px -= s->x * weak;
    drift_(s, flags, 0, outer, 0.);
}

/* edge: curvature = angle/(L) (* oodppo); psi = e - 2*curv*fringe/cos(e)*(1+sin^2 e)
 * fold[0..3] = cos(e), sin(e), tan(e), tan(psi) (the last only if achromatic) */
/* fold[3] holds tan(psi) when oodppo is a compile-time constant (ACHROMATIC,
 * or FIVED's literal dp): `folded` */
static void edge_(state *s, int flags, double L, double angle, double e, double fringe,
                  const double *fold, int folded) {
    double curvature = (flags & F_ACHRO) ? angle / L : angle / L * s->oodppo;
    double tpsi;
    if ((flags & F_ACHRO) || folded) {
        tpsi = fold[3];
    } else {
        double psi = e - 2 * curvature * fringe / fold[0] * (1. + fold[1] * fold[1]);
        tpsi = tan(psi);
    }
    s->px += s->x * curvature * fold[2];
    s->py -= s->y * curvature * tpsi;
}

static void thick_quad_(state *s, int flags, double L, double f, double k1, const double *fold) {
    const double x0 = s->x, px0 = s->px, y0 = s->y, py0 = s->py;
    const double k = k1;
    const double k2 = (flags & F_ACHRO) ? sqrt(fabs(k)) : sqrt(fabs(k * s->oodppo));
    const double k2l = L * f * k2;
    double C, CH, S, SH;
    if (fold) { C = fold[0]; S = fold[1]; CH = fold[2]; SH = fold[3]; }
    else { C = cos(k2l); CH = cosh(k2l); S = sin(k2l); SH = sinh(k2l); }
    if (k > 0.) {
        s->x = C * x0 + S * px0 / k2;
        s->px = -S * x0 * k2 + C * px0;
        s->y = CH * y0 + SH * py0 / k2;
        s->py = SH * y0 * k2 + CH * py0;
    } else {
        s->x = CH * x0 + SH * px0 / k2;
        s->px = SH * x0 * k2 + CH * px0;
        s->y = C * y0 + S * py0 / k2;
        s->py = -S * y0 * k2 + C * py0;
    }
}

static void thick_bend_(state *s, int flags, double L, double f, double angle, double k1,
                        const double *fold) {
    const int ach = flags & F_ACHRO;
    const double x0 = s->x, px0 = s->px, y0 = s->y, py0 = s->py;
    const double Lf = L * f;
    const double curvature = ach ? angle * f / (Lf) : angle * f / (Lf) * s->oodppo;
    double k = ach ? k1 : k1 * s->oodppo;
    double k2 = sqrt(fabs(k));
    double k2l = Lf * k2;
    double C, CH, S, SH;
    if (fold) { C = fold[0]; S = fold[1]; CH = fold[2]; SH = fold[3]; }
    else { C = cos(k2l); CH = cosh(k2l); S = sin(k2l); SH = sinh(k2l); }
    if (k > 0.) {
        s->y = CH * y0 + SH * py0 / k2;
        s->py = SH * y0 * k2 + CH * py0;
    }
    if (k < 0.) {
        s->y = C * y0 + S * py0 / k2;
        s->py = -S * y0 * k2 + C * py0;
    }
    if (k == 0.) s->y += Lf * py0;
    k += ach ? curvature * curvature : curvature * curvature / s->oodppo;
    k2 = sqrt(fabs(k));
    k2l = Lf * k2;
    if (fold) { C = fold[4]; S = fold[5]; CH = fold[6]; SH = fold[7]; }
    else { C = cos(k2l); CH = cosh(k2l); S = sin(k2l); SH = sinh(k2l); }
    if (k > 0.) {
        s->x = C * x0 + S * px0 / k2;
        s->x += s->dp * curvature * (1. - C) / fabs(k);
        s->px = -S * x0 * k2 + C * px0;
        s->px += s->dp * curvature * S / k2;
    }
    if (k < 0.) {
        s->x = CH * x0 + SH * px0 / k2;
        s->x += s->dp * curvature * (CH - 1.) / fabs(k);
        s->px = SH * x0 * k2 + CH * px0;
        s->px += s->dp * curvature * SH / k2;
    }
    if (k == 0.) s->x += Lf * px0;
}

static void wire_(state *s, double wx, double wy, double wk) {
    double alpha = atan2(wy - s->y, wx - s->x);
    double B = (wk) / hypot(wx - s->x, wy - s->y);
    s->px += B * cos(alpha);
    s->py += B * sin(alpha);
}

/* value of a C-expression stack program (opcodes of ufo_gb300/cexpr.py) */
static double eval_(const state *s, const double *prog, int n) {
    double st[32];
    int sp = 0;
    const double vars[8] = {s->x, s->px, s->y, s->py, s->z, s->dp, s->oodppo, (double)s->turn};
    for (int i = 0; i < n; ++i) {
        int op = (int)prog[2 * i];
        double v = prog[2 * i + 1];
        double a, b, c;
        switch (op) {
        case 1: st[sp++] = v; break;
        case 2: st[sp++] = vars[(int)v]; break;
        case 3: st[sp - 1] = -st[sp - 1]; break;
        case 4: st[sp - 1] = st[sp - 1] == 0 ? 1. : 0.; break;
        case 19: st[sp - 1] = fabs(st[sp - 1]); break;
        case 20: st[sp - 1] = sqrt(st[sp - 1]); break;
        case 22: st[sp - 1] = sin(st[sp - 1]); break;
        case 23: st[sp - 1] = cos(st[sp - 1]); break;
        case 24: st[sp - 1] = tan(st[sp - 1]); break;
        case 25: st[sp - 1] = exp(st[sp - 1]); break;
        case 26: st[sp - 1] = log(st[sp - 1]); break;
        case 27: st[sp - 1] = (double)(float)st[sp - 1]; break;
        case 28: st[sp - 1] = trunc(st[sp - 1]) + 0.0; break;  /* (int): no -0 */
        case 21: b = st[--sp]; a = st[--sp]; c = st[--sp]; st[sp++] = c != 0 ? a : b; break;
        default:
            b = st[--sp];
            a = st[--sp];
            switch (op) {
            case 5: c = a + b; break;
            case 6: c = a - b; break;
            case 7: c = a * b; break;
            case 8: c = a / b; break;
            case 9: c = b != 0 ? (double)(long long)(a / b) : NAN; break;
            case 10: c = b != 0 ? fmod(a, b) + 0.0 : NAN; break;
            case 11: c = a < b; break;
            case 12: c = a <= b; break;
            case 13: c = a > b; break;
            case 14: c = a >= b; break;
            case 15: c = a == b; break;
            case 16: c = a != b; break;
            case 17: c = (a != 0) && (b != 0); break;
            default: c = (a != 0) || (b != 0); break;
            }
            st[sp++] = c;
        }
    }
    return st[sp - 1];
}

/* the loss test ``{window} == 0`` (see ufo_gb300/aperture.py) */
static int aperture_lost_(const state *s, const double *prog, int n) {
    return eval_(s, prog, n) != 0;
}

typedef struct {
    double *tracks;
    long slots;      /* count * turns */
    long track_idx;
    long p;
} dumper;

static void dump_(dumper *d, const state *s, int fived) {
    if (!d->tracks) { d->track_idx++; return; }
    double *t = d->tracks + (d->p * d->slots + d->track_idx) * 6;
    t[0] = s->x;
    t[1] = s->px;
    t[2] = s->y;
    t[3] = s->py;
    if (!fived) {
        t[4] = s->z;
        t[5] = s->dp;
    }
    d->track_idx++;
}

/* one pass through the line: element methods with their fractures, dumps
 * between fracture chunks (ufo/lattice.py:98-119, ufo/track.py:69-78) */
static void one_turn_(state *s, int flags, const oelem *el, int n, const double *mp,
                      const double *fr, const double *fold, const double *ap, dumper *d,
                      int fived, int dump_end) {
    double knl[128], ksl[128];
    for (int e = 0; e < n; ++e) {
        const oelem *q = el + e;
        const double *m = mp + q->mp_off;
        const double *fl = fold + q->fold_off;
        if (q->pre_dump) dump_(d, s, fived);
        int np = q->nfrac + 1;
        double f0 = 0.;
        /* thin elements ignore fractures (ufo/elements.py:152-167, 494-500, 517-518) */
        switch (q->type) {
        case T_MARKER:
            break;
        case T_MULTIPOLE:
            align_(s, q->dx, q->dy);
            kick_(s, flags, m, q->nknl, m + q->nknl, q->nksl);
            align_(s, -(q->dx), -(q->dy));
            break;
        case T_WIRE:
            wire_(s, q->wx, q->wy, q->wk);
            break;
        case T_APERTURE:
            if (aperture_lost_(s, ap + q->ap_off, q->ap_len)) s->x = NAN;
            break;
        case T_DYNMULT: {
            /* a multipole whose coefficients are C text of a user pass method:
             * each evaluated where the reference's kick statement reads it */
            align_(s, q->dx, q->dy);
            const double *pq = ap + q->ap_off;
            for (int j = 0; j < q->nknl + q->nksl && j < 256; ++j) {
                const int len = (int)pq[0];
                const double v = eval_(s, pq + 1, len);
                if (j < q->nknl) knl[j] = v; else ksl[j - q->nknl] = v;
                pq += 1 + 2 * len;
            }
            kick_(s, flags, knl, q->nknl, ksl, q->nksl);
            align_(s, -(q->dx), -(q->dy));
            break;
        }
        default:
            for (int i = 0; i < np; ++i) {
                const double f1 = i < q->nfrac ? fr[q->frac_off + i] : 1.;
                const double f = f1 - f0;
                f0 = f1;
                if (i > 0) dump_(d, s, fived);
                if (i == 0 && q->type != T_DRIFT) {
                    align_(s, q->dx, q->dy);
                    if (q->type == T_SBEND || q->type == T_RBEND) {
                        double e1 = q->type == T_RBEND ? q->e1 + (q->angle * 0.5) : q->e1;
                        edge_(s, flags, q->length, q->angle, e1, (q->hgap * q->fint), fl,
                              q->fold_achro);
                    }
                }
                /* multipole lists: knl = pad(dkn, order), knl[order-1] += main */
                const double *dkn = m + q->nknl + q->nksl;
                const double *dks = dkn + q->ndkn;
                switch (q->type) {
                case T_DRIFT:
                    drift_(s, flags, 1, q->length, f);
                    break;
                case T_QUAD:
                case T_SBEND:
                case T_RBEND:
                case T_SEXT:
                case T_OCT: {
                    int mo = q->type == T_SEXT ? 3 : q->type == T_OCT ? 4 : 2;
                    int nn = q->ndkn + (q->ndkn > mo ? q->ndkn : mo);
                    for (int j = 0; j < nn; ++j) knl[j] = j < q->ndkn ? dkn[j] : 0.;
                    for (int j = 0; j < q->ndks; ++j) ksl[j] = dks[j];
                    double main = q->type == T_SEXT ? q->k2 : q->type == T_OCT ? q->k3 : q->k1;
                    knl[mo - 1] = (knl[mo - 1] + main);
                    int bend = q->type == T_SBEND || q->type == T_RBEND;
                    if ((flags & F_KICK) || q->type == T_SEXT || q->type == T_OCT) {
                        teapot_(s, flags, q->length, f, q->slices, knl, nn, ksl, q->ndks, bend,
                                q->angle);
                    } else if (q->type == T_QUAD) {
                        thick_quad_(s, flags, q->length, f, q->k1,
                                    q->fold_achro ? fl + 8 + 4 * i : NULL);
                    } else {
                        thick_bend_(s, flags, q->length, f, q->angle, q->k1,
                                    q->fold_achro ? fl + 8 + 8 * i : NULL);
                    }
                    break;
                }
                default:
                    break;
                }
                if (i == np - 1 && q->type != T_DRIFT) {
                    if (q->type == T_SBEND || q->type == T_RBEND) {
                        double e2 = q->type == T_RBEND ? q->e2 + (q->angle * 0.5) : q->e2;
                        edge_(s, flags, q->length, q->angle, e2, (q->hgap * q->fint), fl + 4,
                              q->fold_achro);
                    }
                    align_(s, -(q->dx), -(q->dy));
                }
            }
        }
    }
    if (dump_end) dump_(d, s, fived);
}

/*
 * Track / StableAperture driver.
 *   elems   [n_seeds][n_elem]   per-seed element attributes
 *   coords  [n][6]              x, px, y, py, z, dp at the start
 *   seed    [n] or NULL         seed row of every particle
 *   mode    0: Track (loss = isnan(x)); 1: StableAperture
 *   tracks  [n][count*turns][6] or NULL; lost [n] or NULL; final [n][6] or NULL
 * Returns 0.
 */
int oracle_track(const oelem *elems, int n_elem, int n_seeds, const double *mp, const double *fr,
                 const double *fold, const double *ap, int flags, int fived, double dp_fived,
                 const double *coords, const int32_t *seed, long n, int turns, int mode,
                 long count, int dump_end, double *tracks, uint32_t *lost, double *final,
                 int threads) {
    (void)n_seeds;
#pragma omp parallel for schedule(dynamic, 4) num_threads(threads)
    for (long p = 0; p < n; ++p) {
        const int sd = seed ? seed[p] : 0;
        const oelem *el = elems + (long)sd * n_elem;
        state s;
        s.x = coords[p * 6 + 0];
        s.px = coords[p * 6 + 1];
        s.y = coords[p * 6 + 2];
        s.py = coords[p * 6 + 3];
        s.z = coords[p * 6 + 4];
        s.dp = coords[p * 6 + 5];
        if (fived) {
            s.z = 0.;
            s.dp = dp_fived;
        }
        s.oodppo = 1. / (s.dp + 1.);
        dumper d = {tracks, count * turns, 0, p};
        int turn;
        for (turn = 0; turn < turns; turn++) {
            s.turn = turn;
            one_turn_(&s, flags, el, n_elem, mp, fr, fold, ap, &d, fived, dump_end);
            if (mode == 0) {
                if (isnan(s.x)) break;
            } else {
                if (fabs(s.x) > 1. || fabs(s.y) > 1. || isnan(s.x)) break;
            }
        }
        if (lost) lost[p] = (uint32_t)turn;
        if (final) {
            final[p * 6 + 0] = s.x;
            final[p * 6 + 1] = s.px;
            final[p * 6 + 2] = s.y;
            final[p * 6 + 3] = s.py;
            final[p * 6 + 4] = s.z;
            final[p * 6 + 5] = s.dp;
        }
    }
    return 0;
}

int oracle_version(void) { return 1; }
