// diff.cu -- tangent map and hand-written adjoint of the one-turn map.
//
// Differentiation runs on its own opcode list (built by ufo_gb300/diff.py from
// the compiled line): drifts, teapot elements, thin kicks, alignments and
// constant edges.  Every kick of the reference (ufo/methods.py:45-76, the
// Horner scheme) is the complex polynomial
//     S(z) = o * sum_n (c_n + i s_n) z^n / n!,   z = x + i y,
//     px -= Re S,   py += Im S,
// so its derivatives follow from S' and S'' (Cauchy-Riemann).  A teapot slice is
// kick, weak focusing (px -= W x), drift.  Element strengths enter linearly:
// one parameter per element scales coefficient `pm` with dK/dk (= L*f/N).
//
// diff_forward: z (and optionally the 4x4 tangent T = dz/dz0) through `turns`
//   turns, writing the state (and T) every `ck` turns as checkpoints.
// diff_reverse: given the output cotangents zbar (and Tbar), walks the turns
//   backwards: each checkpoint segment is re-tracked once to recover its turn
//   starts, each turn is re-tracked onto a tape (x, y and the x/y rows of T at
//   every kick) and then reversed; accumulates the cotangent of the start state
//   and of every element parameter.
// Arithmetic is FP64 with fused multiply-adds (gradients need FP64 accuracy,
// not the reference's rounding).  One thread per job.
#include <cuda_runtime.h>

#include <cstdint>

namespace ufo_diff {

enum : int { D_NOP = 0, D_DRIFT, D_TEAPOT, D_KICK, D_ALIGN, D_EDGE };
constexpr int MAXC = 16;  // multipole orders handled by the differentiator

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
  double *ckpt;           // [job][turns/ck + 1][20]
  double *zT;             // [job][20] final state (+T)
  const double *zbar;     // [job][4] output cotangents
  const double *Tbar;     // [job][16] (tangent only)
  double *seg;            // [job][ck][20] turn starts of one segment
  double *tape;           // [job][kicks_per_turn][10]
  double *zbar0;          // [job][4] cotangent of the start state
  double *pbar;           // [job][n_params]
};

struct St {
  double x, px, y, py;
  double T[16];  // rows x, px, y, py; columns = start coordinates
};

__device__ __forceinline__ double fact(int n) {
  double f = 1.0;
  for (int k = 2; k <= n; ++k) f *= k;
  return f;
}

// S^(d)(z) / o for d = 0, 1, 2: sum_n C_n z^(n-d) / (n-d)!
__device__ void poly(const double *cr, const double *ci, int M, double x, double y, int d,
                     double &re, double &im) {
  re = 0.0;
  im = 0.0;
  for (int n = M - 1; n >= d; --n) {  // Horner in z with the 1/(n-d)! weights
    const double w = 1.0 / fact(n - d);
    const double tr = fma(re, x, -im * y), ti = fma(re, y, im * x);
    re = tr + cr[n] * w;
    im = ti + ci[n] * w;
  }
}

__device__ __forceinline__ void fwd_kick(St &s, const double *cr, const double *ci, int M,
                                         double o, bool tangent) {
  double sr, si;
  poly(cr, ci, M, s.x, s.y, 0, sr, si);
  if (tangent) {
    double a, b;
    poly(cr, ci, M, s.x, s.y, 1, a, b);
    a *= o;
    b *= o;
    for (int j = 0; j < 4; ++j) {
      const double dx = s.T[j], dy = s.T[8 + j];
      s.T[4 + j] -= fma(a, dx, -b * dy);
      s.T[12 + j] += fma(b, dx, a * dy);
    }
  }
  s.px -= o * sr;
  s.py += o * si;
}

__device__ __forceinline__ void fwd_drift(St &s, double L, bool tangent) {
  s.x = fma(s.px, L, s.x);
  s.y = fma(s.py, L, s.y);
  if (tangent)
    for (int j = 0; j < 4; ++j) {
      s.T[j] = fma(s.T[4 + j], L, s.T[j]);
      s.T[8 + j] = fma(s.T[12 + j], L, s.T[8 + j]);
    }
}

__device__ __forceinline__ void fwd_weak(St &s, double W, bool tangent) {
  s.px = fma(-W, s.x, s.px);
  if (tangent)
    for (int j = 0; j < 4; ++j) s.T[4 + j] = fma(-W, s.T[j], s.T[4 + j]);
}

// teapot constants: [Lo, Li, W, dKdk, cr[M], ci[M]]
__device__ void load_coefs(const double *c, int M, double *cr, double *ci) {
  for (int n = 0; n < MAXC; ++n) {
    cr[n] = n < M ? c[n] : 0.0;
    ci[n] = n < M ? c[M + n] : 0.0;
  }
}

// one turn forward; with `tape` the state at every kick is recorded
__device__ void turn_forward(St &s, const DiffArgs &a, const double *T0, double o, bool tangent,
                             double *tape) {
  int kidx = 0;
  double cr[MAXC], ci[MAXC];
  for (int i = 0; i < a.n_ops; ++i) {
    const DOp op = a.ops[i];
    const double *c = T0 + op.toff;
    const double oo = op.achro ? 1.0 : o;
    switch (op.kind) {
      case D_DRIFT:
        fwd_drift(s, c[0], tangent);
        break;
      case D_ALIGN:
        s.x -= c[0];
        s.y -= c[1];
        break;
      case D_EDGE: {
        const double curv = c[0] * oo;
        const double x0 = s.x, y0 = s.y;
        s.px = fma(x0 * curv, c[1], s.px);
        s.py = fma(-(y0 * curv), c[2], s.py);
        if (tangent)
          for (int j = 0; j < 4; ++j) {
            s.T[4 + j] = fma(s.T[j] * curv, c[1], s.T[4 + j]);
            s.T[12 + j] = fma(-(s.T[8 + j] * curv), c[2], s.T[12 + j]);
          }
        break;
      }
      case D_KICK:
      case D_TEAPOT: {
        const bool tp = op.kind == D_TEAPOT;
        const int N = tp ? op.N : 1;
        const double Lo = tp ? c[0] : 0.0, Li = tp ? c[1] : 0.0, W = tp ? c[2] : 0.0;
        load_coefs(c + 4, op.M, cr, ci);
        if (tp) fwd_drift(s, Lo, tangent);
        for (int sl = 0; sl < N; ++sl) {
          if (tape) {
            double *t = tape + 10 * (kidx++);
            t[0] = s.x;
            t[1] = s.y;
            if (tangent)
              for (int j = 0; j < 4; ++j) {
                t[2 + j] = s.T[j];
                t[6 + j] = s.T[8 + j];
              }
          }
          fwd_kick(s, cr, ci, op.M, oo, tangent);
          if (tp && W != 0.0) fwd_weak(s, W, tangent);
          if (tp) fwd_drift(s, sl < N - 1 ? Li : Lo, tangent);
        }
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
    for (int j = 0; j < 4; ++j) {
      b.T[4 + j] = fma(b.T[j], L, b.T[4 + j]);
      b.T[12 + j] = fma(b.T[8 + j], L, b.T[12 + j]);
    }
}

__device__ __forceinline__ void rev_weak(Bar &b, double W, bool tangent) {
  b.x = fma(-W, b.px, b.x);
  if (tangent)
    for (int j = 0; j < 4; ++j) b.T[j] = fma(-W, b.T[4 + j], b.T[j]);
}

// reverse of one kick at recorded (x, y) [and tangent rows]; returns the
// cotangent of the op's parameter coefficient (order pm)
__device__ double rev_kick(Bar &b, const double *t, const double *cr, const double *ci, int M,
                           double o, bool tangent, int pm) {
  const double x = t[0], y = t[1];
  double a1, b1;
  poly(cr, ci, M, x, y, 1, a1, b1);
  a1 *= o;
  b1 *= o;
  // state: px' = px - Re S, py' = py + Im S
  double xb = -b.px * a1 + b.py * b1;
  double yb = b.px * b1 + b.py * a1;
  // parameter (real coefficient of order pm): dS/dc = o z^pm / pm!
  double gr = 0.0;
  if (pm >= 0) {
    double zr = 1.0, zi = 0.0;
    for (int k = 0; k < pm; ++k) {
      const double tr = zr * x - zi * y;
      zi = zr * y + zi * x;
      zr = tr;
    }
    const double w = o / fact(pm);
    gr = -b.px * zr * w + b.py * zi * w;
  }
  if (tangent) {
    double a2 = 0.0, b2 = 0.0;
    if (M > 2) poly(cr, ci, M, x, y, 2, a2, b2);
    a2 *= o;
    b2 *= o;
    double Ab = 0.0, Bb = 0.0;
    for (int j = 0; j < 4; ++j) {
      const double dx = t[2 + j], dy = t[6 + j];
      const double pxb = b.T[4 + j], pyb = b.T[12 + j];
      // T_px -= a1 dx - b1 dy ; T_py += b1 dx + a1 dy
      b.T[j] += -pxb * a1 + pyb * b1;
      b.T[8 + j] += pxb * b1 + pyb * a1;
      Ab += -pxb * dx + pyb * dy;
      Bb += pxb * dy + pyb * dx;
    }
    // a1 + i b1 = S'(z): d/dx = S'' , d/dy = i S''
    xb += Ab * a2 + Bb * b2;
    yb += -Ab * b2 + Bb * a2;
    if (pm >= 1) {  // dS'/dc = o z^(pm-1) / (pm-1)!
      double zr = 1.0, zi = 0.0;
      for (int k = 0; k < pm - 1; ++k) {
        const double tr = zr * x - zi * y;
        zi = zr * y + zi * x;
        zr = tr;
      }
      const double w = o / fact(pm - 1);
      gr += Ab * zr * w + Bb * zi * w;
    }
  }
  b.x += xb;
  b.y += yb;
  return gr;
}

// reverse of one turn using its tape; accumulates parameter cotangents
__device__ void turn_reverse(Bar &b, const DiffArgs &a, const double *T0, double o, bool tangent,
                             const double *tape, double *pbar) {
  int kidx = a.kicks_per_turn;
  double cr[MAXC], ci[MAXC];
  for (int i = a.n_ops - 1; i >= 0; --i) {
    const DOp op = a.ops[i];
    const double *c = T0 + op.toff;
    const double oo = op.achro ? 1.0 : o;
    switch (op.kind) {
      case D_DRIFT:
        rev_drift(b, c[0], tangent);
        break;
      case D_ALIGN:
        break;  // translation: cotangents unchanged
      case D_EDGE: {
        const double curv = c[0] * oo;
        b.x = fma(b.px * curv, c[1], b.x);
        b.y = fma(-(b.py * curv), c[2], b.y);
        if (tangent)
          for (int j = 0; j < 4; ++j) {
            b.T[j] = fma(b.T[4 + j] * curv, c[1], b.T[j]);
            b.T[8 + j] = fma(-(b.T[12 + j] * curv), c[2], b.T[8 + j]);
          }
        break;
      }
      case D_KICK:
      case D_TEAPOT: {
        const bool tp = op.kind == D_TEAPOT;
        const int N = tp ? op.N : 1;
        const double Lo = tp ? c[0] : 0.0, Li = tp ? c[1] : 0.0, W = tp ? c[2] : 0.0;
        const double dKdk = c[3];
        load_coefs(c + 4, op.M, cr, ci);
        double g = 0.0;
        for (int sl = N - 1; sl >= 0; --sl) {
          if (tp) rev_drift(b, sl < N - 1 ? Li : Lo, tangent);
          if (tp && W != 0.0) rev_weak(b, W, tangent);
          const double *t = tape + 10 * (--kidx);
          g += rev_kick(b, t, cr, ci, op.M, oo, tangent, op.pslot >= 0 ? op.pm : -1);
        }
        if (tp) rev_drift(b, Lo, tangent);
        if (op.pslot >= 0) pbar[op.pslot] += g * dKdk;
        break;
      }
      default:
        break;
    }
  }
}

__device__ void load_state(St &s, const double *src, bool tangent) {
  s.x = src[0]; s.px = src[1]; s.y = src[2]; s.py = src[3];
  if (tangent)
    for (int k = 0; k < 16; ++k) s.T[k] = src[4 + k];
}

__device__ void save_state(const St &s, double *dst, bool tangent) {
  dst[0] = s.x; dst[1] = s.px; dst[2] = s.y; dst[3] = s.py;
  if (tangent)
    for (int k = 0; k < 16; ++k) dst[4 + k] = s.T[k];
}

__global__ void diff_forward(DiffArgs a) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.n_jobs) return;
  const bool tangent = a.tangent;
  St s;
  s.x = a.z0[4 * j]; s.px = a.z0[4 * j + 1]; s.y = a.z0[4 * j + 2]; s.py = a.z0[4 * j + 3];
  for (int k = 0; k < 16; ++k) s.T[k] = (k % 5 == 0) ? 1.0 : 0.0;
  const double o = a.o[j];
  const double *T0 = a.tab + (a.seed ? static_cast<int64_t>(a.seed[j]) : 0) * a.tab_stride;
  const int nck = a.turns / a.ck + 1;
  double *ck = a.ckpt ? a.ckpt + static_cast<int64_t>(j) * nck * 20 : nullptr;
  for (int t = 0; t < a.turns; ++t) {
    if (ck && t % a.ck == 0) save_state(s, ck + 20 * (t / a.ck), tangent);
    turn_forward(s, a, T0, o, tangent, nullptr);
  }
  if (ck && a.turns % a.ck == 0) save_state(s, ck + 20 * (a.turns / a.ck), tangent);
  save_state(s, a.zT + 20 * j, tangent);
}

__global__ void diff_reverse(DiffArgs a) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.n_jobs) return;
  const bool tangent = a.tangent;
  const double o = a.o[j];
  const double *T0 = a.tab + (a.seed ? static_cast<int64_t>(a.seed[j]) : 0) * a.tab_stride;
  const int nck = a.turns / a.ck + 1;
  const double *ck = a.ckpt + static_cast<int64_t>(j) * nck * 20;
  double *seg = a.seg + static_cast<int64_t>(j) * a.ck * 20;
  double *tape = a.tape + static_cast<int64_t>(j) * a.kicks_per_turn * 10;
  double *pbar = a.pbar + static_cast<int64_t>(j) * a.n_params;
  for (int k = 0; k < a.n_params; ++k) pbar[k] = 0.0;
  Bar b;
  b.x = a.zbar[4 * j]; b.px = a.zbar[4 * j + 1]; b.y = a.zbar[4 * j + 2]; b.py = a.zbar[4 * j + 3];
  for (int k = 0; k < 16; ++k) b.T[k] = tangent ? a.Tbar[16 * j + k] : 0.0;
  const int last_seg = (a.turns - 1) / a.ck;
  for (int sg = last_seg; sg >= 0; --sg) {
    const int t0 = sg * a.ck;
    const int t1 = min(a.turns, t0 + a.ck);
    St s;
    load_state(s, ck + 20 * sg, tangent);
    for (int t = t0; t < t1; ++t) {  // recover the segment's turn starts
      save_state(s, seg + 20 * (t - t0), tangent);
      if (t + 1 < t1) turn_forward(s, a, T0, o, tangent, nullptr);
    }
    for (int t = t1 - 1; t >= t0; --t) {
      load_state(s, seg + 20 * (t - t0), tangent);
      turn_forward(s, a, T0, o, tangent, tape);  // tape this turn
      turn_reverse(b, a, T0, o, tangent, tape, pbar);
    }
  }
  a.zbar0[4 * j] = b.x; a.zbar0[4 * j + 1] = b.px; a.zbar0[4 * j + 2] = b.y;
  a.zbar0[4 * j + 3] = b.py;
}

}  // namespace ufo_diff

// ---------------------------------------------------------------- C ABI
extern "C" {

// All pointers are device pointers; `ops` int32[n_ops][8] (DOp), `tab` f64.
// Asynchronous on `stream`.  Returns 0 or a CUDA error code (negative).
int ufo_diff_forward(const int32_t *ops, int n_ops, const double *tab, int64_t tab_stride,
                     const int32_t *seed, int n_params, int kicks_per_turn, int n_jobs,
                     const double *z0, const double *o, int turns, int ck, int tangent,
                     double *ckpt, double *zT, void *stream) {
  if (n_jobs <= 0) return 0;
  if (!ops || !tab || !z0 || !o || !zT || turns < 0 || ck < 1) return -1;
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
  ufo_diff::diff_forward<<<(n_jobs + tpb - 1) / tpb, tpb, 0, static_cast<cudaStream_t>(stream)>>>(a);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int ufo_diff_reverse(const int32_t *ops, int n_ops, const double *tab, int64_t tab_stride,
                     const int32_t *seed, int n_params, int kicks_per_turn, int n_jobs,
                     const double *o, int turns, int ck, int tangent, const double *ckpt,
                     const double *zbar, const double *Tbar, double *seg, double *tape,
                     double *zbar0, double *pbar, void *stream) {
  if (n_jobs <= 0) return 0;
  if (!ops || !tab || !o || !ckpt || !zbar || !seg || !tape || !zbar0 || !pbar || turns < 1 ||
      ck < 1 || (tangent && !Tbar))
    return -1;
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
  a.seg = seg;
  a.tape = tape;
  a.zbar0 = zbar0;
  a.pbar = pbar;
  const int tpb = 32;
  ufo_diff::diff_reverse<<<(n_jobs + tpb - 1) / tpb, tpb, 0, static_cast<cudaStream_t>(stream)>>>(a);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

}  // extern "C"
