// ufo_gb300.cu -- tracking kernels and the C ABI (include/ufo_gb300.h).
//
// One thread tracks one particle with its state in registers; all lanes of a
// warp walk the same opcode table, so element dispatch is warp-uniform.  The
// per-seed FP64 constants are read through the read-only cache (each warp's
// lanes usually share a seed, so loads broadcast).
//
// track_kernel is persistent: a grid of a few warps per SM pulls particles from
// a device counter.  At each turn boundary the lanes whose particle finished
// (lost, or its turn count reached) write their results and refill from the
// counter with one warp-aggregated atomicAdd (ballot + popc + rank), so warps
// stay full while survival is uneven -- the FP64 pipe charges a warp
// instruction the same whether 1 or 32 lanes are active.  This is the
// reference's atomic work queue (ufo/track.py:110-112, ufo/sa.py:122-124) at
// lane granularity instead of work-item granularity.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "../../include/ufo_gb300.h"
#include "ops.cuh"

namespace ufo {

struct Parked {        // a particle in flight, moved between lanes or CTAs
  double x, px, y, py, z, dp;
  int64_t p;
  int turn, target;
  int seed;
  int pad;
};

struct TrackArgs {
  const Op *ops;
  int n_ops;
  const double *table;
  int64_t stride;
  int n_seeds;
  int n_dumps;
  const double *coords;
  const int32_t *seed;
  const int32_t *pturns;
  int64_t n;
  int turns;
  int mode;
  int flags;
  int64_t slots;
  int every;
  double *tracks;
  uint32_t *lost;
  double *final_state;
  // queue[0]: particles handed out so far.  The compacting kernel also uses
  // queue[1]: particles finished, queue[2]: CTAs that left, queue[3] / [4]:
  // the particle pool's head and tail tickets (all zeroed by each launch)
  unsigned long long *queue;
  // particle pool of the compacting kernel (null: CTAs exchange nothing): a
  // bounded ring of pool_cap slots; pool_seq[slot] = 2 e while the slot is free
  // for ticket e * pool_cap + slot, 2 e + 1 once that ticket's particle is in it
  Parked *pool;
  unsigned long long *pool_seq;
  long long pool_cap;
  // compacting kernel: chunks of 32 consecutive particles are handed out in
  // the order c -> (c * spread) mod (n / 32) (spread coprime to n / 32; 0: in
  // order; a last partial chunk comes last), so that a warp still takes
  // neighbours (which tend to survive or be lost together) while the chunks of
  // a region that survives are spread over every SM
  unsigned long long spread;
};

UFO_DEV void load_particle(State &s, const TrackArgs &a, int64_t p) {
  const double *c = a.coords + p * 6;
  s.x = c[0];
  s.px = c[1];
  s.y = c[2];
  s.py = c[3];
  s.z = c[4];
  s.dp = c[5];
  s.o = dvd(1., add(s.dp, 1.));  // oodppo = 1. / (dp + 1.)  (ufo/track.py:103)
  s.opdp = add(1., s.dp);        // opdp = 1. + dp            (ufo/methods.py:32)
  s.turn = 0;
  s.bad_o = nf(s.o);
}

UFO_DEV void store_final(const State &s, const TrackArgs &a, int64_t p) {
  if (a.lost) a.lost[p] = static_cast<uint32_t>(s.turn);
  if (a.final_state) {
    double *f = a.final_state + p * 6;
    f[0] = s.x; f[1] = s.px; f[2] = s.y; f[3] = s.py; f[4] = s.z; f[5] = s.dp;
  }
}

UFO_DEV void observe(const State &s, const TrackArgs &a, int64_t p, int k) {
  if (!a.tracks) return;
  if ((s.turn + 1) % a.every) return;
  const int64_t slot = static_cast<int64_t>((s.turn + 1) / a.every - 1) * a.n_dumps + k;
  if (slot < 0 || slot >= a.slots) return;
  double *t = a.tracks + (p * a.slots + slot) * 6;
  t[0] = s.x; t[1] = s.px; t[2] = s.y; t[3] = s.py;
  if (!(a.flags & UFO_TRACK_FIVED)) { t[4] = s.z; t[5] = s.dp; }
}

// one pass through the line
// FULL = false: the lean interpreter for programs made only of drifts, teapot
// elements, kicks, alignments, constant edges, circular apertures and
// observation points (chosen on the host); it carries far fewer live values.
template <bool FMA, bool FULL>
UFO_DEV void one_turn(State &s, const TrackArgs &a, const double *tab, int64_t p) {
  for (int i = 0; i < a.n_ops; ++i) {
    const int4 w0 = __ldg(reinterpret_cast<const int4 *>(a.ops + i));
    const int4 w1 = __ldg(reinterpret_cast<const int4 *>(a.ops + i) + 1);
    const Op op{w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
    const double *c = tab + op.toff;
    switch (op.kind) {
      case OP_TEAPOT:
        teapot<FMA, FULL>(s, op, c);
        break;
      case OP_DRIFT:
        if (FULL && (op.flags & F_EXACT))
          drift<FMA>(s, DF_MUL, true, c);
        else if (op.i0 == DF_MUL)
          drift_L<FMA>(s, ld(c));
        else if (op.i0 == DF_DIV)
          drift_div<FMA>(s, c);
        else
          drift<FMA>(s, DF_MUL2, false, c);
        break;
      case OP_KICK: {
        const bool bad = s.bad_o || nf(s.x) || nf(s.y);
        if (FMA && !bad && (op.flags & F_PSER)) {  // dense series after the coefficients
          const uint32_t mn = static_cast<uint32_t>(op.i2), ms = static_cast<uint32_t>(op.i3);
          const PxPy r = kick_pser_ool(s.x, s.y, s.px, s.py, (op.flags & F_ACHRO) ? 1.0 : s.o,
                                       pser_len(mn, ms), c + __popc(mn) + __popc(ms));
          s.px = r.px;
          s.py = r.py;
          break;
        }
        const PxPy r = kick_ool<FMA>(s.x, s.y, s.px, s.py, s.o, s.bad_o, op.i0, op.i1,
                                     static_cast<uint32_t>(op.i2), static_cast<uint32_t>(op.i3),
                                     c, op.flags & F_ACHRO, bad);
        s.px = r.px;
        s.py = r.py;
        break;
      }
      case OP_ALIGN:
        switch ((op.flags & F_AX ? 1 : 0) | (op.flags & F_AY ? 2 : 0)) {
          case 1: s.x = sub(s.x, ld(c)); break;
          case 2: s.y = sub(s.y, ld(c + 1)); break;
          case 3: s.x = sub(s.x, ld(c)); s.y = sub(s.y, ld(c + 1)); break;
          default: break;
        }
        break;
      case OP_EDGE:
        edge_dispatch<FMA, FULL>(s, op.flags, c);
        break;
      case OP_THICKQ:
        if (FULL) {
          const P4 r = thick_quad_ool(s.x, s.px, s.y, s.py, s.o, op.flags, c);
          s.x = r.x; s.px = r.px; s.y = r.y; s.py = r.py;
        }
        break;
      case OP_THICKB:
        if (FULL) {
          const P4 r = thick_bend_ool(s.x, s.px, s.y, s.py, s.dp, s.o, op.flags, c);
          s.x = r.x; s.px = r.px; s.y = r.y; s.py = r.py;
        }
        break;
      case OP_WIRE:
        if (FULL) {
          const P4 r = wire_ool(s.x, s.px, s.y, s.py, c);
          s.x = r.x; s.px = r.px; s.y = r.y; s.py = r.py;
        }
        break;
      case OP_APERTURE: {
        bool lost;
        if (!FULL || (op.flags & F_CIRCLE))  // (x*x + y*y < c) == 0
          lost = !(add(mul(s.x, s.x), mul(s.y, s.y)) < ld(c));
        else
          lost = aperture_ool(s.x, s.px, s.y, s.py, s.z, s.dp, s.o, s.turn, c, op.i0);
        if (lost) s.x = __longlong_as_double(0x7ff8000000000000ll);
        break;
      }
      case OP_OBSERVE:
        observe(s, a, p, op.i0);
        break;
      case OP_LINEAR: {
        // a kick-free teapot element of an FMA program composed on the host:
        // (x, px) through a 2x2 matrix, (y, py) through a drift
        const double m11 = ld(c), m12 = ld(c + 1), m21 = ld(c + 2), m22 = ld(c + 3);
        const double x0 = s.x;
        s.x = fma_(m11, x0, mul(m12, s.px));
        s.px = fma_(m21, x0, mul(m22, s.px));
        s.y = fma_(s.py, ld(c + 4), s.y);
        break;
      }
      case OP_DYNKICK:
        if (FULL) {
          const PxPy r = dynkick_ool(s.x, s.px, s.y, s.py, s.z, s.dp, s.o, s.turn, op.i0, op.i1,
                                     op.flags & F_ACHRO, op.i2, c);
          s.px = r.px;
          s.py = r.py;
        }
        break;
      default:
        break;
    }
  }
}

UFO_DEV bool is_lost(const State &s, int mode) {
  if (mode == UFO_MODE_TRACK) return isnan(s.x);
  return fabs(s.x) > 1. || fabs(s.y) > 1. || isnan(s.x);
}

template <bool FMA, bool FULL>
__global__ void __launch_bounds__(32) track_kernel(TrackArgs a) {
  const unsigned ALL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned lt_mask = (1u << lane) - 1u;
  int64_t p = -1;
  bool exhausted = false;
  State s{};
  int target = 0;
  const double *tab = a.table;
  while (true) {
    // lanes without a particle take the next ones from the queue
    const unsigned need = __ballot_sync(ALL, p < 0 && !exhausted);
    if (need) {
      const int leader = __ffs(need) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(a.queue, static_cast<unsigned long long>(__popc(need)));
      base = __shfl_sync(ALL, base, leader);
      if (p < 0 && !exhausted) {
        const int64_t q = static_cast<int64_t>(base) + __popc(need & lt_mask);
        if (q < a.n) {
          p = q;
          load_particle(s, a, p);
          target = a.pturns ? a.pturns[p] : a.turns;
          const int64_t sd = a.seed ? static_cast<int64_t>(a.seed[p]) : 0;
          tab = a.table + sd * a.stride;
          if (sd < 0 || sd >= a.n_seeds) {  // seed outside the table: not tracked
            if (a.lost) a.lost[p] = 0xffffffffu;
            p = -1;
          } else if (target <= 0) {  // nothing to track
            store_final(s, a, p);
            p = -1;
          }
        } else {
          exhausted = true;
        }
      }
      continue;  // re-check: a lane that got a zero-turn particle needs another
    }
    if (__all_sync(ALL, p < 0)) break;
    if (p >= 0) {
      one_turn<FMA, FULL>(s, a, tab, p);
      const bool lost = is_lost(s, a.mode);
      if (!lost) ++s.turn;
      if (lost || s.turn >= target) {
        store_final(s, a, p);
        p = -1;
      }
    }
  }
}

// ------------------------------------------------- CTA-compacting variant
// The same persistent loop with many warps per CTA, and one more step once
// the work counter is exhausted: at every turn boundary the CTA packs its
// surviving particles into its lowest warps through shared memory (a ballot
// + popc rank within each warp, a prefix over the warps), so the survivors of
// an uneven scan keep filling whole warps instead of thinning out across all
// of them.  Moving a particle between lanes is a copy of its state: every
// particle's arithmetic, and so every result bit, is the one of the other
// kernels.
// Phase A (work left in the counter): each warp refills its own lanes, no
// barrier, exactly as track_kernel.  A warp that finds the counter exhausted
// (itself, or through the CTA's flag another warp set) enters phase B, where
// the CTA meets at one barrier per turn: every warp reaches phase B (the flag
// is set once and only read afterwards), so every barrier is reached by the
// whole CTA.  Emptied warps stay in the loop (they take part in the barriers
// and issue no FP64 work) until the CTA has no particle left.
// Phase B also balances the CTAs (when the launch gives a pool): the counter
// runs out while each CTA holds whatever its lanes took, and an SM's turn
// time grows with its busy warps, so the CTA holding the most survivors would
// set the launch's time.  Every 4 turns each CTA compares its particles with
// the share of the unfinished ones per CTA still running (rounded up to whole
// warps): a CTA above it puts the excess into the pool, a CTA below it takes
// from the pool.  The pool is a bounded ring with one sequence word per slot
// (the multi-producer multi-consumer queue of D. Vyukov): warp 0 of a CTA
// reserves free slots or claims filled ones with one CAS on the tail or head
// ticket and gives up when the CAS or a slot's state says no, so no CTA ever
// waits for another.  A CTA leaves when it holds no particle and the pool is
// empty or its head slot is still being filled; the CTA filling it still
// runs (it keeps at least one particle) and takes its own particles back
// before it can leave, so no particle stays behind in the pool.
constexpr int CTA_MAX_WARPS = 16;

UFO_DEV void park(Parked &d, const State &s, int64_t p, int target, int sd) {
  d.x = s.x; d.px = s.px; d.y = s.y; d.py = s.py; d.z = s.z; d.dp = s.dp;
  d.p = p; d.turn = s.turn; d.target = target; d.seed = sd;
}

UFO_DEV void unpark(const Parked &d, const TrackArgs &a, State &s, int64_t &p, int &target,
                    int &sd, const double *&tab) {
  s.x = d.x; s.px = d.px; s.y = d.y; s.py = d.py; s.z = d.z; s.dp = d.dp;
  s.o = dvd(1., add(s.dp, 1.));  // as load_particle: the same bits
  s.opdp = add(1., s.dp);
  s.bad_o = nf(s.o);
  s.turn = d.turn;
  p = d.p;
  target = d.target;
  sd = d.seed;
  tab = a.table + static_cast<int64_t>(sd) * a.stride;
}

UFO_DEV unsigned long long vload(const unsigned long long *q) {
  return *static_cast<const volatile unsigned long long *>(q);
}

// Warp 0: the number of consecutive slots from ticket t0 (at most `want`)
// whose sequence word is `state` (0: free for that ticket, 1: filled with it).
UFO_DEV int pool_run(const TrackArgs &a, unsigned long long t0, int want, unsigned state) {
  const unsigned long long cap = static_cast<unsigned long long>(a.pool_cap);
  const int lane = threadIdx.x & 31;
  int n = 0;
  while (n < want) {
    const unsigned long long t = t0 + n + lane;
    const bool ok = vload(a.pool_seq + t % cap) == 2 * (t / cap) + state;
    const unsigned run = __ballot_sync(0xffffffffu, ok);
    const int k = run == 0xffffffffu ? 32 : __ffs(~run) - 1;
    n += k;
    if (k < 32) break;
  }
  return n < want ? n : want;
}

template <bool FMA, bool FULL>
__global__ void __launch_bounds__(CTA_MAX_WARPS * 32, 1) track_kernel_cta(TrackArgs a) {
  extern __shared__ Parked parked[];  // one slot per thread of the CTA
  // lanes with a particle per warp, double-buffered by barrier phase (a warp
  // one phase ahead writes the other buffer)
  __shared__ int warp_active[2][CTA_MAX_WARPS];
  __shared__ int exhausted_flag;  // set once the work counter is exhausted
  __shared__ unsigned long long seen[2];  // particles finished, CTAs that left
  __shared__ unsigned long long xfer_base;  // first pool ticket moved
  __shared__ int xfer_n, xfer_leave;        // particles moved; the CTA leaves
  const unsigned ALL = 0xffffffffu;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  const int nthreads = static_cast<int>(blockDim.x);
  const unsigned lt_mask = (1u << lane) - 1u;
  volatile int *flag = &exhausted_flag;
  if (threadIdx.x == 0) *flag = 0;
  __syncthreads();
  int64_t p = -1;
  int sd = 0;
  State s{};
  int target = 0;
  const double *tab = a.table;
  // ---- phase A: refill from the counter, no barrier
  bool exhausted = false;
  while (true) {
    if (*flag) exhausted = true;  // another warp found the counter exhausted
    while (!exhausted) {
      const unsigned need = __ballot_sync(ALL, p < 0);
      if (!need) break;
      const int leader = __ffs(need) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(a.queue, static_cast<unsigned long long>(__popc(need)));
      base = __shfl_sync(ALL, base, leader);
      if (base + __popc(need) > static_cast<unsigned long long>(a.n)) {
        exhausted = true;
        if (lane == leader) *flag = 1;  // the counter only grows: final
      }
      if (p < 0) {
        const int64_t q = static_cast<int64_t>(base) + __popc(need & lt_mask);
        if (q < a.n) {
          p = q;
          const unsigned long long full = static_cast<unsigned long long>(a.n) / 32u;
          const unsigned long long chunk = static_cast<unsigned long long>(q) / 32u;
          if (a.spread && chunk < full)
            p = static_cast<int64_t>(((chunk * a.spread) % full) * 32u + (q & 31));
          load_particle(s, a, p);
          target = a.pturns ? a.pturns[p] : a.turns;
          sd = a.seed ? a.seed[p] : 0;
          tab = a.table + static_cast<int64_t>(sd) * a.stride;
          if (sd < 0 || sd >= a.n_seeds) {  // seed outside the table: not tracked
            if (a.lost) a.lost[p] = 0xffffffffu;
            p = -1;
            if (a.pool) atomicAdd(a.queue + 1, 1ull);  // finished (rare)
          } else if (target <= 0) {  // nothing to track
            store_final(s, a, p);
            p = -1;
            if (a.pool) atomicAdd(a.queue + 1, 1ull);
          }
        }
      }
    }
    if (exhausted) break;  // warp-uniform
    bool done = false;
    if (p >= 0) {  // a lane's particle needs no refill this turn
      one_turn<FMA, FULL>(s, a, tab, p);
      const bool lost = is_lost(s, a.mode);
      if (!lost) ++s.turn;
      if (lost || s.turn >= target) {
        store_final(s, a, p);
        p = -1;
        done = true;
      }
    }
    if (a.pool) {  // launch-uniform: count the warp's finished particles
      const unsigned f = __ballot_sync(ALL, done);
      if (f && lane == 0) atomicAdd(a.queue + 1, static_cast<unsigned long long>(__popc(f)));
    }
  }
  // ---- phase B: one barrier per turn, survivors packed into the lowest warps
  for (int k = 0;; ++k) {
    const bool exchange = a.pool != nullptr && gridDim.x > 1;  // launch-uniform
    const bool balance = exchange && (k & 3) == 0;             // CTA-uniform
    if (balance && threadIdx.x == 0) {  // read before the barrier: no extra one
      seen[0] = vload(a.queue + 1);
      seen[1] = vload(a.queue + 2);
    }
    const unsigned act = __ballot_sync(ALL, p >= 0);
    if (lane == 0) warp_active[k & 1][warp] = __popc(act);
    __syncthreads();
    int total = 0, busy = 0, before = 0;
    for (int w = 0; w < nwarps; ++w) {
      const int c = warp_active[k & 1][w];
      if (w < warp) before += c;
      total += c;
      busy += c > 0;
    }
    if (total == 0 && !exchange) break;  // CTA-uniform: every thread read the same counts
    // particles to move through the pool: > 0 take up to want, < 0 give -want
    int want = 0;  // CTA-uniform
    if (exchange) {
      if (total == 0) {
        want = nthreads;
      } else if (balance) {
        const long long running = static_cast<long long>(gridDim.x) - static_cast<long long>(seen[1]);
        const long long unfinished = a.n - static_cast<long long>(seen[0]);
        if (running > 0 && unfinished > 0) {
          const long long share = (unfinished + running - 1) / running;
          const long long whole = (share + 31) / 32 * 32;  // the warps the share needs
          if (total > whole) {
            want = -static_cast<int>(total - whole);
          } else if (total < share) {
            const long long room = (whole < nthreads ? whole : nthreads) - total;
            want = room > 0 ? static_cast<int>(room) : 0;
          }
        }
      }
    }
    if (want != 0) {  // CTA-uniform: every lane's particle goes through the slots
      if (p >= 0) park(parked[before + __popc(act & lt_mask)], s, p, target, sd);
      p = -1;  // the state lives in the slot now (nothing held across the pool step)
      s = State{};
      if (warp == 0) {
        int n = 0, leave = 0;
        unsigned long long t0 = 0;
        if (want < 0) {  // reserve free slots at the tail
          if (lane == 0) t0 = vload(a.queue + 4);
          t0 = __shfl_sync(ALL, t0, 0);
          n = pool_run(a, t0, -want, 0);
          if (n > 0 && lane == 0 && atomicCAS(a.queue + 4, t0, t0 + n) != t0) n = -1;
        } else {  // claim filled slots at the head
          if (lane == 0) t0 = vload(a.queue + 3);
          t0 = __shfl_sync(ALL, t0, 0);
          n = pool_run(a, t0, want, 1);
          leave = total == 0 && n == 0;  // empty, or its head is still being filled
          if (n > 0 && lane == 0 && atomicCAS(a.queue + 3, t0, t0 + n) != t0) n = -1;
        }
        n = __shfl_sync(ALL, n, 0);  // -1: another CTA moved the ticket first
        if (lane == 0) {
          xfer_base = t0;
          xfer_n = n > 0 ? n : 0;
          xfer_leave = leave;
          if (leave) atomicAdd(a.queue + 2, 1ull);
        }
        __threadfence();  // the claimed slots' contents before their readers
      }
      __syncthreads();
      const int moved = xfer_n;
      const unsigned long long t0 = xfer_base;
      const unsigned long long cap = static_cast<unsigned long long>(a.pool_cap);
      int keep = total;
      if (want < 0) {  // the highest parked particles go to the reserved slots
        keep = total - moved;
        if (static_cast<int>(threadIdx.x) < moved) {
          const unsigned long long t = t0 + threadIdx.x;
          a.pool[t % cap] = parked[keep + threadIdx.x];
          __threadfence();
          *static_cast<volatile unsigned long long *>(a.pool_seq + t % cap) = 2 * (t / cap) + 1;
        }
      }
      if (static_cast<int>(threadIdx.x) < keep) {
        unpark(parked[threadIdx.x], a, s, p, target, sd, tab);
      } else if (want > 0 && static_cast<int>(threadIdx.x) < keep + moved) {
        const unsigned long long t = t0 + (threadIdx.x - keep);
        const unsigned long long *w = reinterpret_cast<const unsigned long long *>(a.pool + t % cap);
        Parked d;
        unsigned long long *dw = reinterpret_cast<unsigned long long *>(&d);
#pragma unroll
        for (int i = 0; i < static_cast<int>(sizeof(Parked) / 8); ++i) dw[i] = __ldcg(w + i);
        unpark(d, a, s, p, target, sd, tab);
        __threadfence();  // the slot is read before it is handed back
        *static_cast<volatile unsigned long long *>(a.pool_seq + t % cap) = 2 * (t / cap + 1);
      }
      if (xfer_leave) break;  // CTA-uniform: no particle in the CTA
      // the slots are rewritten only after the next phase's barrier
    } else if ((total + 31) / 32 < busy) {  // CTA-uniform: packing frees a warp
      if (p >= 0) park(parked[before + __popc(act & lt_mask)], s, p, target, sd);
      __syncthreads();
      p = -1;
      if (static_cast<int>(threadIdx.x) < total) unpark(parked[threadIdx.x], a, s, p, target, sd, tab);
      // the slots are rewritten only after the next phase's barrier
    }
    bool done = false;
    if (p >= 0) {
      one_turn<FMA, FULL>(s, a, tab, p);
      const bool lost = is_lost(s, a.mode);
      if (!lost) ++s.turn;
      if (lost || s.turn >= target) {
        store_final(s, a, p);
        p = -1;
        done = true;
      }
    }
    if (exchange) {  // count the warp's finished particles
      const unsigned f = __ballot_sync(ALL, done);
      if (f && lane == 0) atomicAdd(a.queue + 1, static_cast<unsigned long long>(__popc(f)));
    }
  }
}

// plain variant: one thread per particle, no refill (the reference's
// one-work-item-per-particle launch shape, used for comparisons)
template <bool FMA, bool FULL>
__global__ void __launch_bounds__(128) track_plain_kernel(TrackArgs a) {
  const int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (p >= a.n) return;
  State s{};
  load_particle(s, a, p);
  const int target = a.pturns ? a.pturns[p] : a.turns;
  const int64_t sd = a.seed ? static_cast<int64_t>(a.seed[p]) : 0;
  if (sd < 0 || sd >= a.n_seeds) {  // seed outside the table: not tracked
    if (a.lost) a.lost[p] = 0xffffffffu;
    return;
  }
  const double *tab = a.table + sd * a.stride;
  while (s.turn < target) {
    one_turn<FMA, FULL>(s, a, tab, p);
    if (is_lost(s, a.mode)) break;
    ++s.turn;
  }
  store_final(s, a, p);
}

// ---------------------------------------------------------------- closed orbit
// The reference's ClosedOrbit (ufo/co.py:18-124, :146-250): per orbit, a fixed
// number of Nelder-Mead steps (reflection 1, contraction 0.5, expansion 2) on
// the squared one-turn residual of (x, px, y, py) with z = 0, dp = 0,
// oodppo = 1, starting from the simplex {v, v + 1e-4 e_j}.  Every step is the
// reference's, in its IEEE operation order (no contraction), and the one-turn
// map is the strict interpreter, so the orbits are the reference's bit for
// bit.  One thread per orbit; the simplex lives in local memory (indexed by
// the run-time vertex numbers).
template <bool FULL>
UFO_DEV double co_residual(const double *v, const TrackArgs &a, const double *tab) {
  State s{};
  s.x = v[0]; s.px = v[1]; s.y = v[2]; s.py = v[3];
  s.z = 0.0; s.dp = 0.0; s.o = 1.0; s.opdp = 1.0;
  s.turn = 0;
  s.bad_o = false;
  one_turn<false, FULL>(s, a, tab, 0);
  double r = mul(sub(v[0], s.x), sub(v[0], s.x));
  r = add(r, mul(sub(v[1], s.px), sub(v[1], s.px)));
  r = add(r, mul(sub(v[2], s.y), sub(v[2], s.y)));
  r = add(r, mul(sub(v[3], s.py), sub(v[3], s.py)));
  return r;
}

UFO_DEV void co_simplex_sum(const double (*sx)[4], double *psum) {
  for (int j = 0; j < 4; ++j) {
    psum[j] = 0.0;
    for (int i = 0; i < 5; ++i) psum[j] = add(psum[j], sx[i][j]);
  }
}

// trial vertex through the face opposite `ihi`, scaled by `fac`; replaces
// `ihi` if better
template <bool FULL>
UFO_DEV double co_try(double (*sx)[4], double *y, double *psum, int ihi, double fac,
                      const TrackArgs &a, const double *tab) {
  const double fac1 = dvd(sub(1.0, fac), 4.0);
  const double fac2 = sub(fac1, fac);
  double t[4];
  for (int j = 0; j < 4; ++j) t[j] = sub(mul(psum[j], fac1), mul(sx[ihi][j], fac2));
  const double yt = co_residual<FULL>(t, a, tab);
  if (yt < y[ihi]) {
    y[ihi] = yt;
    for (int j = 0; j < 4; ++j) {
      psum[j] = add(psum[j], sub(t[j], sx[ihi][j]));
      sx[ihi][j] = t[j];
    }
  }
  return yt;
}

template <bool FULL>
__global__ void __launch_bounds__(32) co_amoeba_kernel(TrackArgs a, const double *start,
                                                       double *orbits, int iterations) {
  const int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (p >= a.n) return;
  const int64_t sd = a.seed ? static_cast<int64_t>(a.seed[p]) : 0;
  double *out = orbits + 4 * p;
  if (sd < 0 || sd >= a.n_seeds) {  // seed outside the table: no orbit
    for (int j = 0; j < 4; ++j) out[j] = __longlong_as_double(0x7ff8000000000000ll);
    return;
  }
  const double *tab = a.table + sd * a.stride;
  double sx[5][4], y[5], psum[4];
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 4; ++j) sx[i][j] = start[4 * p + j];
  for (int j = 0; j < 4; ++j) sx[j + 1][j] = add(sx[j + 1][j], 1e-4);
  for (int i = 0; i < 5; ++i) y[i] = co_residual<FULL>(sx[i], a, tab);
  co_simplex_sum(sx, psum);
  int iter = 0, ilo = 0;
  while (true) {
    ilo = 1;
    int ihi, inhi;
    if (y[1] > y[2]) {
      inhi = 2;
      ihi = 1;
    } else {
      inhi = 1;
      ihi = 2;
    }
    for (int i = 0; i < 5; ++i) {
      if (y[i] < y[ilo]) ilo = i;
      if (y[i] > y[ihi]) {
        inhi = ihi;
        ihi = i;
      } else if (y[i] > y[inhi] && i != ihi) {
        inhi = i;
      }
    }
    if (iter >= iterations) break;
    double yt = co_try<FULL>(sx, y, psum, ihi, -1.0, a, tab);
    ++iter;
    if (yt <= y[ilo]) {
      yt = co_try<FULL>(sx, y, psum, ihi, 2.0, a, tab);
    } else if (yt >= y[inhi]) {
      const double ysave = y[ihi];
      yt = co_try<FULL>(sx, y, psum, ihi, 0.5, a, tab);
      if (yt >= ysave) {  // shrink towards the best vertex
        for (int i = 0; i < 5; ++i) {
          if (i == ilo) continue;
          for (int j = 0; j < 4; ++j) {
            psum[j] = mul(add(sx[i][j], sx[ilo][j]), 0.5);
            sx[i][j] = psum[j];
          }
          y[i] = co_residual<FULL>(psum, a, tab);
        }
        iter += 4;
        co_simplex_sum(sx, psum);
      }
    }
  }
  for (int j = 0; j < 4; ++j) out[j] = sx[ilo][j];
}

// FP64 pipe peak probe: 8 independent DFMA chains per thread
__global__ void __launch_bounds__(256) dfma_peak_kernel(double *out, int iters, double b, double c) {
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = threadIdx.x * 1e-3 + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fma_(a[k], b, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s = add(s, a[k]);
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// FP64 pipe probe: CH independent DFMA chains per thread; only the first
// `lanes` lanes of each warp run the chains (the rest skip the loop), so the
// useful rate shows what inactive lanes cost
template <int CH>
__global__ void __launch_bounds__(32) dfma_probe_kernel(double *out, int iters, int lanes,
                                                        double b, double c) {
  double a[CH];
#pragma unroll
  for (int k = 0; k < CH; ++k) a[k] = threadIdx.x * 1e-3 + k;
  if (static_cast<int>(threadIdx.x & 31) < lanes) {
    for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int k = 0; k < CH; ++k) a[k] = fma_(a[k], b, c);
    }
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < CH; ++k) s = add(s, a[k]);
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace ufo

// ======================================================================= C ABI

struct ufo_ctx {
  int device;
  int sm_count;
  int warps_per_sm;  // resident warps per SM of the persistent grid
  cudaStream_t stream;
  unsigned long long *queue;
  ufo::Parked *pool;               // the compacting kernel's particle pool
  unsigned long long *pool_seq;    // and its slots' sequence words
  std::atomic<int64_t> launches;
};

struct ufo_prog {
  ufo_ctx *ctx;
  int device;  // copied: destruction must not touch the context
  ufo::Op *ops;
  int n_ops;
  double *table;
  int64_t stride;
  int n_seeds;
  int n_dumps;
  bool full;  // needs the full interpreter (thick, wire, exact, ...)
  std::vector<int32_t> host_ops;  // for validating replacement tables
};

namespace {
thread_local char g_err[512] = "";

int fail(int code, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
  return code;
}

int cuda_fail(cudaError_t e, const char *what) {
  return fail(UFO_E_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define UFO_CUDA(call)                                  \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

// per-device set-up state; host threads making their first call on a device
// at the same time serialise on this mutex
std::mutex g_setup_mutex;
bool g_const_ready[64] = {};

// Upload the constant tables to the current device, once per device.
int ensure_constants(int device) {
  if (device < 0 || device >= 64) return fail(UFO_E_ARG, "device %d out of range", device);
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (g_const_ready[device]) return UFO_OK;
  double r[33];
  r[0] = 0.0;
  for (int k = 1; k <= 32; ++k) r[k] = 1.0 / static_cast<double>(k);
  UFO_CUDA(cudaMemcpyToSymbol(ufo::c_rcp_order, r, sizeof r));
  double rf[33];
  double fact = 1.0;  // n! is exact in FP64 for n <= 22; above, one rounding per step
  for (int k = 0; k <= 32; ++k) {
    if (k > 0) fact *= static_cast<double>(k);
    rf[k] = 1.0 / fact;
  }
  UFO_CUDA(cudaMemcpyToSymbol(ufo::c_rcp_fact, rf, sizeof rf));
  g_const_ready[device] = true;
  return UFO_OK;
}

int popc32(uint32_t v) { return __builtin_popcount(v); }

bool mask_fits(int n, int32_t mask) {
  if (n < 0 || n > 32) return false;
  const uint32_t m = static_cast<uint32_t>(mask);
  return n == 32 || (m >> n) == 0u;
}

// constants of the dense power series of a general kick (F_PSER): 2 per
// order up to the highest coefficient; -1 if the flag is set without one
int64_t pser_consts(int flags, int32_t mn, int32_t ms) {
  if (!(flags & ufo::F_PSER)) return 0;
  const uint32_t m = static_cast<uint32_t>(mn) | static_cast<uint32_t>(ms);
  if (m == 0u) return -1;
  return 2 * static_cast<int64_t>(32 - __builtin_clz(m));
}

int drift_consts(int form, bool exact) {
  if (exact) return 1;
  return form == ufo::DF_MUL ? 1 : form == ufo::DF_MUL2 ? 2 : form == ufo::DF_DIV ? 4 : -1;
}

// Number of table constants an op reads (exactly what the kernels read), or
// -1 if the op's shape is invalid.  Every op must fit inside the stride so
// that no kernel read leaves its seed's row.
int64_t op_consts(const int32_t *w) {
  const int kind = w[0], flags = w[1];
  const bool exact = flags & ufo::F_EXACT;
  switch (kind) {
    case ufo::OP_NOP:
    case ufo::OP_OBSERVE:
      return 0;
    case ufo::OP_DRIFT:
      return drift_consts(w[3], exact);
    case ufo::OP_KICK: {
      if (!mask_fits(w[3], w[5]) || !mask_fits(w[4], w[6])) return -1;
      const int64_t ps = pser_consts(flags, w[5], w[6]);
      if (ps < 0) return -1;
      return popc32(w[5]) + popc32(w[6]) + ps;
    }
    case ufo::OP_TEAPOT: {
      const int64_t ps = pser_consts(flags, w[6], w[7]);
      if (ps < 0) return -1;
      if (flags & ufo::F_YOSHIDA) {  // [4 drifts][3 weights][kick][W][series]
        if (exact || w[3] < 1 || !mask_fits(w[4], w[6]) || !mask_fits(w[5], w[7])) return -1;
        return 7 + popc32(w[6]) + popc32(w[7]) + ((flags & ufo::F_WEAK) ? 1 : 0) + ps;
      }
      if (w[3] < 1 || !mask_fits(w[4], w[6]) || !mask_fits(w[5], w[7])) return -1;
      if ((flags & ufo::F_PSER) && exact) return -1;
      const int fo = (flags >> ufo::SH_FOUTER) & 3, fi = (flags >> ufo::SH_FINNER) & 3;
      const int co = drift_consts(fo, exact), ci = w[3] > 1 ? drift_consts(fi, exact) : 0;
      if (co < 0 || ci < 0) return -1;
      return co + ci + popc32(w[6]) + popc32(w[7]) + ((flags & ufo::F_WEAK) ? 1 : 0) +
             ((flags & ufo::F_SPLITO) ? 1 : 0) + ps;
    }
    case ufo::OP_ALIGN:
      return 2;
    case ufo::OP_EDGE:
      return (flags & ufo::F_RTPSI) ? 6 : 3;
    case ufo::OP_THICKQ:
      return (flags & ufo::F_CONST) ? 7 : 2;
    case ufo::OP_THICKB:
      return (flags & ufo::F_CONST) ? 16 : 3;
    case ufo::OP_WIRE:
      return 3;
    case ufo::OP_APERTURE:
      if (flags & ufo::F_CIRCLE) return 1;
      return w[3] >= 0 ? 2 * static_cast<int64_t>(w[3]) : -1;
    case ufo::OP_DYNKICK:
      if (w[3] < 0 || w[4] < 0 || w[3] > 32 || w[4] > 32 || w[5] < w[3] + w[4]) return -1;
      return w[5];
    case ufo::OP_LINEAR:
      return 5;
    default:
      return -1;
  }
}

// simulate an expression stack program (row 0 of the table; the opcodes are
// the same in every row): every pop must find an operand and the depth must
// stay within the kernel's `depth` slots
bool prog_ok(const double *prog, int n, int depth) {
  int sp = 0;
  for (int i = 0; i < n; ++i) {
    const double code = prog[2 * i];
    if (!(code >= 1 && code <= 28) || code != static_cast<int>(code)) return false;
    const int op = static_cast<int>(code);
    if (op == 2) {
      const double v = prog[2 * i + 1];
      if (!(v >= 0 && v <= 7)) return false;
    }
    if (op == 1 || op == 2) {
      if (++sp > depth) return false;
    } else if (op == 3 || op == 4 || op == 19 || op == 20 || (op >= 22 && op <= 28)) {
      if (sp < 1) return false;
    } else if (op == 21) {
      if (sp < 3) return false;
      sp -= 2;
    } else {
      if (sp < 2) return false;
      sp -= 1;
    }
  }
  return n == 0 || sp >= 1;
}

bool aperture_ok(const double *prog, int n) { return prog_ok(prog, n, 16); }

// the coefficient programs of a dynamic kick: n_coef of them, exactly filling
// `words` table entries, each a valid program of at least one op
bool dynkick_ok(const double *c, int n_coef, int64_t words) {
  int64_t q = 0;
  for (int j = 0; j < n_coef; ++j) {
    if (q >= words) return false;
    const double len = c[q];
    if (!(len >= 1 && len <= 4096) || len != static_cast<int>(len)) return false;
    const int n = static_cast<int>(len);
    if (q + 1 + 2 * n > words || !prog_ok(c + q + 1, n, 32)) return false;
    q += 1 + 2 * n;
  }
  return q == words;
}

// ops the lean interpreter does not carry
bool needs_full(const int32_t *ops, int n_ops) {
  for (int i = 0; i < n_ops; ++i) {
    const int32_t *w = ops + i * UFO_OP_WORDS;
    const int kind = w[0], flags = w[1];
    if (kind == ufo::OP_THICKQ || kind == ufo::OP_THICKB || kind == ufo::OP_WIRE) return true;
    if ((kind == ufo::OP_DRIFT || kind == ufo::OP_TEAPOT) && (flags & ufo::F_EXACT)) return true;
    if (kind == ufo::OP_EDGE && (flags & ufo::F_RTPSI)) return true;
    if (kind == ufo::OP_APERTURE && !(flags & ufo::F_CIRCLE)) return true;
    if (kind == ufo::OP_DYNKICK) return true;
  }
  return false;
}

// `table` may be NULL (constants on the device): the expression programs of
// apertures and dynamic kicks are then not checked.
int validate_ops(const int32_t *ops, int n_ops, int64_t stride, int n_dumps,
                 const double *table) {
  for (int i = 0; i < n_ops; ++i) {
    const int32_t *w = ops + i * UFO_OP_WORDS;
    if (w[0] < ufo::OP_NOP || w[0] > ufo::OP_LINEAR)
      return fail(UFO_E_ARG, "op %d: unknown kind %d", i, w[0]);
    // an observation point writes slot (turn / every) * n_dumps + index
    if (w[0] == ufo::OP_OBSERVE && (w[3] < 0 || w[3] >= n_dumps))
      return fail(UFO_E_ARG, "op %d: observation index %d outside [0, %d)", i, w[3], n_dumps);
    const int64_t nc = op_consts(w);
    if (nc < 0) return fail(UFO_E_ARG, "op %d (kind %d): invalid shape", i, w[0]);
    if (w[2] < 0 || w[2] + nc > stride)
      return fail(UFO_E_ARG, "op %d: constants [%d, %lld) outside stride %lld", i, w[2],
                  static_cast<long long>(w[2] + nc), static_cast<long long>(stride));
    if (w[0] == ufo::OP_APERTURE && !(w[1] & ufo::F_CIRCLE) && table &&
        !aperture_ok(table + w[2], w[3]))
      return fail(UFO_E_ARG, "op %d: malformed aperture program", i);
    if (w[0] == ufo::OP_DYNKICK && table && !dynkick_ok(table + w[2], w[3] + w[4], w[5]))
      return fail(UFO_E_ARG, "op %d: malformed dynamic-kick programs", i);
  }
  return UFO_OK;
}

// Chunk hand-out order of the compacting kernel: c -> (c * m) mod n_chunks
// with m coprime to the number of whole 32-particle chunks, near it / golden
// ratio: a permutation whose early values sample the whole input evenly (a
// dynamic-aperture grid is ordered by amplitude, and its surviving chunks
// would otherwise all go to the first SMs to start).
unsigned long long spread_multiplier(int64_t n_particles) {
  const int64_t n = n_particles / 32;
  // chunk * m < n^2 must fit 64 bits: beyond 2^31 chunks (far more particles
  // than device memory holds) the chunks go out in order
  if (n < 3 || n >= (int64_t{1} << 31)) return 0;
  unsigned long long m = static_cast<unsigned long long>(0.6180339887498949 * static_cast<double>(n));
  const unsigned long long un = static_cast<unsigned long long>(n);
  auto gcd = [](unsigned long long x, unsigned long long y) {
    while (y) {
      const unsigned long long t = x % y;
      x = y;
      y = t;
    }
    return x;
  };
  if (m < 1) m = 1;
  while (gcd(m, un) != 1) ++m;  // ends: m = n - 1 is coprime to n
  return m;
}

// The launch shared by every entry point: fill the kernel arguments and start
// the persistent (or plain) kernel on `stream`; `queue` is the work counter.
int launch_kernels(ufo::TrackArgs &a, bool full, int sm_count, int warps_per_sm,
                   cudaStream_t stream) {
  const bool fma = a.flags & UFO_TRACK_FMA;
  if (a.flags & UFO_TRACK_PLAIN) {
    const unsigned blocks = static_cast<unsigned>((a.n + 127) / 128);
    if (fma)
      full ? ufo::track_plain_kernel<true, true><<<blocks, 128, 0, stream>>>(a)
           : ufo::track_plain_kernel<true, false><<<blocks, 128, 0, stream>>>(a);
    else
      full ? ufo::track_plain_kernel<false, true><<<blocks, 128, 0, stream>>>(a)
           : ufo::track_plain_kernel<false, false><<<blocks, 128, 0, stream>>>(a);
  } else if (a.flags & UFO_TRACK_COMPACT) {
    // the work counter, the finished and departed counts, the pool's tickets
    UFO_CUDA(cudaMemsetAsync(a.queue, 0, 5 * sizeof(unsigned long long), stream));
    // one CTA per SM (as many SMs as the particles' warps allow) of up to
    // warps_per_sm warps (at most 16); survivors are packed within each CTA
    const int64_t warps = (a.n + 31) / 32;
    const int64_t ctas = warps < sm_count ? warps : sm_count;
    int wpc = warps_per_sm < 1 ? 1 : warps_per_sm > ufo::CTA_MAX_WARPS ? ufo::CTA_MAX_WARPS
                                                                          : warps_per_sm;
    if (ctas * wpc > warps) wpc = static_cast<int>((warps + ctas - 1) / ctas);
    a.spread = spread_multiplier(a.n);
    const unsigned g = static_cast<unsigned>(ctas), tpb = static_cast<unsigned>(wpc * 32);
    if (a.pool) {
      // as many slots as the CTAs have lanes: the particles in flight once the
      // counter is exhausted (the pool array holds sm_count * CTA_MAX_WARPS * 32)
      a.pool_cap = static_cast<long long>(g) * tpb;
      UFO_CUDA(cudaMemsetAsync(a.pool_seq, 0, sizeof(unsigned long long) * a.pool_cap, stream));
    }
    const size_t smem = sizeof(ufo::Parked) * tpb;
    if (fma)
      full ? ufo::track_kernel_cta<true, true><<<g, tpb, smem, stream>>>(a)
           : ufo::track_kernel_cta<true, false><<<g, tpb, smem, stream>>>(a);
    else
      full ? ufo::track_kernel_cta<false, true><<<g, tpb, smem, stream>>>(a)
           : ufo::track_kernel_cta<false, false><<<g, tpb, smem, stream>>>(a);
  } else {
    UFO_CUDA(cudaMemsetAsync(a.queue, 0, sizeof(unsigned long long), stream));
    // one warp per block so the block scheduler spreads warps evenly over the
    // SMs (the FP64 pipe is per SM); at most warps_per_sm resident per SM
    int64_t warps = (a.n + 31) / 32;
    const int64_t max_warps = static_cast<int64_t>(sm_count) * warps_per_sm;
    if (warps > max_warps) warps = max_warps;
    const unsigned g = static_cast<unsigned>(warps);
    if (fma)
      full ? ufo::track_kernel<true, true><<<g, 32, 0, stream>>>(a)
           : ufo::track_kernel<true, false><<<g, 32, 0, stream>>>(a);
    else
      full ? ufo::track_kernel<false, true><<<g, 32, 0, stream>>>(a)
           : ufo::track_kernel<false, false><<<g, 32, 0, stream>>>(a);
  }
  UFO_CUDA(cudaGetLastError());
  return UFO_OK;
}

ufo::TrackArgs make_args(const ufo::Op *ops, int n_ops, const double *table, int64_t stride,
                         int n_seeds, int n_dumps, const double *d_coords, const int32_t *d_seed,
                         const int32_t *d_pturns, int64_t n, int turns, int mode, int flags,
                         int64_t slots, int every, double *d_tracks, uint32_t *d_lost,
                         double *d_final, unsigned long long *queue) {
  ufo::TrackArgs a;
  a.ops = ops;
  a.n_ops = n_ops;
  a.table = table;
  a.stride = stride;
  a.n_seeds = n_seeds;
  a.n_dumps = n_dumps;
  a.coords = d_coords;
  a.seed = d_seed;
  a.pturns = d_pturns;
  a.n = n;
  a.turns = turns;
  a.mode = mode;
  a.flags = flags;
  a.slots = d_tracks ? slots : 0;
  a.every = every < 1 ? 1 : every;
  a.tracks = d_tracks;
  a.lost = d_lost;
  a.final_state = d_final;
  a.queue = queue;
  a.pool = nullptr;
  a.pool_seq = nullptr;
  a.pool_cap = 0;
  a.spread = 0;
  return a;
}

int launch_track(ufo_ctx *ctx, const ufo_prog *prog, const double *d_coords, const int32_t *d_seed,
                 const int32_t *d_pturns, int64_t n, int turns, int mode, int flags, int64_t slots,
                 int every, double *d_tracks, uint32_t *d_lost, double *d_final,
                 cudaStream_t stream) {
  if (n <= 0) return UFO_OK;
  ufo::TrackArgs a = make_args(prog->ops, prog->n_ops, prog->table, prog->stride, prog->n_seeds,
                               prog->n_dumps, d_coords, d_seed, d_pturns, n, turns, mode, flags,
                               slots, every, d_tracks, d_lost, d_final, ctx->queue);
  a.pool = ctx->pool;
  a.pool_seq = ctx->pool_seq;
  const int rc = launch_kernels(a, prog->full, ctx->sm_count, ctx->warps_per_sm, stream);
  if (rc == UFO_OK) ctx->launches.fetch_add(1);
  return rc;
}

int check_track_args(ufo_ctx *ctx, const ufo_prog *prog, int64_t n, int turns, int mode,
                     int64_t slots, int every) {
  if (!ctx || !prog) return fail(UFO_E_ARG, "null context or program");
  if (prog->ctx != ctx) return fail(UFO_E_ARG, "program belongs to another context");
  if (n < 0) return fail(UFO_E_ARG, "negative particle count");
  if (turns < 0) return fail(UFO_E_ARG, "negative turn count");
  if (mode != UFO_MODE_TRACK && mode != UFO_MODE_SA) return fail(UFO_E_ARG, "bad mode %d", mode);
  if (slots < 0) return fail(UFO_E_ARG, "negative slot count");
  if (every < 1) return fail(UFO_E_ARG, "every must be >= 1");
  return UFO_OK;
}
}  // namespace

extern "C" {

const char *ufo_last_error(void) { return g_err; }

int ufo_device_count(int *count) {
  if (!count) return fail(UFO_E_ARG, "null count");
  UFO_CUDA(cudaGetDeviceCount(count));
  return UFO_OK;
}

int ufo_ctx_create(int device, ufo_ctx **out) {
  if (!out) return fail(UFO_E_ARG, "null output");
  *out = nullptr;
  int n = 0;
  UFO_CUDA(cudaGetDeviceCount(&n));
  if (device < 0 || device >= n) return fail(UFO_E_ARG, "device %d of %d", device, n);
  UFO_CUDA(cudaSetDevice(device));
  int rc = ensure_constants(device);
  if (rc) return rc;
  ufo_ctx *c = new (std::nothrow) ufo_ctx;
  if (!c) return fail(UFO_E_NOMEM, "host allocation");
  c->device = device;
  c->launches = 0;
  cudaDeviceProp prop;
  cudaError_t e = cudaGetDeviceProperties(&prop, device);
  if (e != cudaSuccess) { delete c; return cuda_fail(e, "cudaGetDeviceProperties"); }
  c->sm_count = prop.multiProcessorCount;
  c->warps_per_sm = 16;
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { delete c; return cuda_fail(e, "cudaStreamCreate"); }
  e = cudaMalloc(&c->queue, 64);
  if (e != cudaSuccess) {
    cudaStreamDestroy(c->stream);
    delete c;
    return fail(UFO_E_NOMEM, "cudaMalloc(queue): %s", cudaGetErrorString(e));
  }
  // one pool slot per lane of the largest compacting grid
  const size_t slots = static_cast<size_t>(c->sm_count) * ufo::CTA_MAX_WARPS * 32;
  c->pool = nullptr;
  c->pool_seq = nullptr;
  if (cudaMalloc(&c->pool, sizeof(ufo::Parked) * slots) != cudaSuccess ||
      cudaMalloc(&c->pool_seq, sizeof(unsigned long long) * slots) != cudaSuccess) {
    cudaFree(c->pool);
    cudaFree(c->queue);
    cudaStreamDestroy(c->stream);
    delete c;
    return fail(UFO_E_NOMEM, "cudaMalloc(particle pool of %zu slots)", slots);
  }
  *out = c;
  return UFO_OK;
}

void ufo_ctx_destroy(ufo_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  cudaFree(ctx->queue);
  cudaFree(ctx->pool);
  cudaFree(ctx->pool_seq);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
}

int ufo_fp64_peak(ufo_ctx *ctx, double *gflops) {
  if (!ctx || !gflops) return fail(UFO_E_ARG, "null argument");
  UFO_CUDA(cudaSetDevice(ctx->device));
  const int blocks = ctx->sm_count * 4, threads = 256, iters = 4096;
  double *buf = nullptr;
  if (cudaMalloc(&buf, sizeof(double) * blocks * threads) != cudaSuccess)
    return fail(UFO_E_NOMEM, "cudaMalloc(peak buffer)");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  cudaError_t err = cudaSuccess;
  for (int rep = 0; rep < 4 && err == cudaSuccess; ++rep) {
    cudaEventRecord(e0, ctx->stream);
    ufo::dfma_peak_kernel<<<blocks, threads, 0, ctx->stream>>>(buf, iters, 0.999999, 1e-7);
    cudaEventRecord(e1, ctx->stream);
    err = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  if (err == cudaSuccess) err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  if (err != cudaSuccess) return cuda_fail(err, "fp64 peak probe");
  *gflops = 2.0 * blocks * threads * static_cast<double>(iters) * 8 / (best * 1e6);
  return UFO_OK;
}

int ufo_fp64_probe(ufo_ctx *ctx, int warps_per_sm, int chains, int lanes, double *gflops) {
  if (!ctx || !gflops) return fail(UFO_E_ARG, "null argument");
  if (warps_per_sm < 1 || warps_per_sm > 32) return fail(UFO_E_ARG, "warps_per_sm in [1, 32]");
  if (lanes < 1 || lanes > 32) return fail(UFO_E_ARG, "lanes in [1, 32]");
  if (chains != 1 && chains != 2 && chains != 4 && chains != 8)
    return fail(UFO_E_ARG, "chains in {1, 2, 4, 8}");
  UFO_CUDA(cudaSetDevice(ctx->device));
  const int blocks = ctx->sm_count * warps_per_sm, iters = 32768 / chains;
  double *buf = nullptr;
  if (cudaMalloc(&buf, sizeof(double) * blocks * 32) != cudaSuccess)
    return fail(UFO_E_NOMEM, "cudaMalloc(probe buffer)");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  cudaError_t err = cudaSuccess;
  for (int rep = 0; rep < 4 && err == cudaSuccess; ++rep) {
    cudaEventRecord(e0, ctx->stream);
    switch (chains) {
      case 1: ufo::dfma_probe_kernel<1><<<blocks, 32, 0, ctx->stream>>>(buf, iters, lanes, 0.999999, 1e-7); break;
      case 2: ufo::dfma_probe_kernel<2><<<blocks, 32, 0, ctx->stream>>>(buf, iters, lanes, 0.999999, 1e-7); break;
      case 4: ufo::dfma_probe_kernel<4><<<blocks, 32, 0, ctx->stream>>>(buf, iters, lanes, 0.999999, 1e-7); break;
      default: ufo::dfma_probe_kernel<8><<<blocks, 32, 0, ctx->stream>>>(buf, iters, lanes, 0.999999, 1e-7); break;
    }
    cudaEventRecord(e1, ctx->stream);
    err = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  if (err == cudaSuccess) err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  if (err != cudaSuccess) return cuda_fail(err, "fp64 probe");
  // useful flops: active lanes only
  *gflops = 2.0 * blocks * lanes * static_cast<double>(iters) * chains / (best * 1e6);
  return UFO_OK;
}

int ufo_launch_count(ufo_ctx *ctx, int64_t *count) {
  if (!ctx || !count) return fail(UFO_E_ARG, "null argument");
  *count = ctx->launches.load();
  return UFO_OK;
}

// the op shapes, and every seed row's expression programs
static int validate_rows(const int32_t *ops, int n_ops, int64_t stride, int n_dumps,
                         const double *table, int n_seeds) {
  for (int r = 0; r < n_seeds; ++r) {
    const int rc =
        validate_ops(ops, n_ops, stride, n_dumps, table + static_cast<int64_t>(r) * stride);
    if (rc) return rc;
  }
  return UFO_OK;
}

int ufo_prog_create(ufo_ctx *ctx, const int32_t *ops, int n_ops, const double *table,
                    int64_t stride, int n_seeds, int n_dumps, ufo_prog **out) {
  if (!ctx || !ops || !table || !out) return fail(UFO_E_ARG, "null argument");
  *out = nullptr;
  if (n_ops < 0 || stride < 1 || n_seeds < 1 || n_dumps < 0)
    return fail(UFO_E_ARG, "bad program sizes");
  int rc = validate_rows(ops, n_ops, stride, n_dumps, table, n_seeds);
  if (rc) return rc;
  UFO_CUDA(cudaSetDevice(ctx->device));
  ufo_prog *p = new (std::nothrow) ufo_prog;
  if (!p) return fail(UFO_E_NOMEM, "host allocation");
  p->ctx = ctx;
  p->device = ctx->device;
  p->n_ops = n_ops;
  p->stride = stride;
  p->n_seeds = n_seeds;
  p->n_dumps = n_dumps;
  p->full = needs_full(ops, n_ops);
  p->host_ops.assign(ops, ops + static_cast<size_t>(n_ops) * UFO_OP_WORDS);
  p->ops = nullptr;
  p->table = nullptr;
  const size_t ob = sizeof(ufo::Op) * (n_ops > 0 ? n_ops : 1);
  const size_t tb = sizeof(double) * static_cast<size_t>(stride) * n_seeds;
  if (cudaMalloc(&p->ops, ob) != cudaSuccess || cudaMalloc(&p->table, tb) != cudaSuccess) {
    cudaFree(p->ops);
    cudaFree(p->table);
    delete p;
    return fail(UFO_E_NOMEM, "cudaMalloc(program %zu + %zu bytes)", ob, tb);
  }
  cudaError_t e = cudaMemcpyAsync(p->ops, ops, sizeof(ufo::Op) * n_ops, cudaMemcpyHostToDevice,
                                  ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(p->table, table, tb, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    cudaFree(p->ops);
    cudaFree(p->table);
    delete p;
    return cuda_fail(e, "program upload");
  }
  *out = p;
  return UFO_OK;
}

int ufo_prog_set_table(ufo_prog *prog, const double *table, int n_seeds) {
  if (!prog || !table) return fail(UFO_E_ARG, "null argument");
  if (n_seeds != prog->n_seeds) return fail(UFO_E_ARG, "seed count changed");
  const int rc = validate_rows(prog->host_ops.data(), prog->n_ops, prog->stride, prog->n_dumps,
                               table, n_seeds);
  if (rc) return rc;
  UFO_CUDA(cudaSetDevice(prog->ctx->device));
  const size_t tb = sizeof(double) * static_cast<size_t>(prog->stride) * n_seeds;
  UFO_CUDA(cudaMemcpyAsync(prog->table, table, tb, cudaMemcpyHostToDevice, prog->ctx->stream));
  UFO_CUDA(cudaStreamSynchronize(prog->ctx->stream));
  return UFO_OK;
}

void ufo_prog_destroy(ufo_prog *prog) {
  // may run after the context is gone (any destruction order is allowed), so
  // only the copied device id is used; cudaFree waits for work in flight
  if (!prog) return;
  cudaSetDevice(prog->device);
  cudaDeviceSynchronize();
  cudaFree(prog->ops);
  cudaFree(prog->table);
  delete prog;
}

int ufo_track_device(ufo_ctx *ctx, const ufo_prog *prog, const double *d_coords,
                     const int32_t *d_seed, const int32_t *d_pturns, int64_t n, int turns,
                     int mode, int flags, int64_t slots, int every, double *d_tracks,
                     uint32_t *d_lost, double *d_final, void *stream) {
  int rc = check_track_args(ctx, prog, n, turns, mode, slots, every);
  if (rc) return rc;
  if (n > 0 && !d_coords) return fail(UFO_E_ARG, "null coordinates");
  UFO_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  return launch_track(ctx, prog, d_coords, d_seed, d_pturns, n, turns, mode, flags, slots, every,
                      d_tracks, d_lost, d_final, st);
}

int ufo_track(ufo_ctx *ctx, const ufo_prog *prog, const double *coords, const int32_t *seed,
              const int32_t *pturns, int64_t n, int turns, int mode, int flags, int64_t slots,
              int every, double *tracks, uint32_t *lost, double *final_state) {
  int rc = check_track_args(ctx, prog, n, turns, mode, slots, every);
  if (rc) return rc;
  if (n == 0) return UFO_OK;
  if (!coords) return fail(UFO_E_ARG, "null coordinates");
  if (seed) {
    for (int64_t i = 0; i < n; ++i)
      if (seed[i] < 0 || seed[i] >= prog->n_seeds)
        return fail(UFO_E_ARG, "particle %lld: seed %d outside [0, %d)",
                    static_cast<long long>(i), seed[i], prog->n_seeds);
  }
  UFO_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  const size_t cb = sizeof(double) * 6 * n;
  const size_t tb = tracks ? sizeof(double) * 6 * static_cast<size_t>(slots) * n : 0;
  double *d_coords = nullptr, *d_tracks = nullptr, *d_final = nullptr;
  int32_t *d_seed = nullptr, *d_pturns = nullptr;
  uint32_t *d_lost = nullptr;
  auto cleanup = [&]() {
    cudaFree(d_coords); cudaFree(d_tracks); cudaFree(d_final);
    cudaFree(d_seed); cudaFree(d_pturns); cudaFree(d_lost);
  };
  if (cudaMalloc(&d_coords, cb) != cudaSuccess ||
      (tb && cudaMalloc(&d_tracks, tb) != cudaSuccess) ||
      (final_state && cudaMalloc(&d_final, cb) != cudaSuccess) ||
      (seed && cudaMalloc(&d_seed, sizeof(int32_t) * n) != cudaSuccess) ||
      (pturns && cudaMalloc(&d_pturns, sizeof(int32_t) * n) != cudaSuccess) ||
      (lost && cudaMalloc(&d_lost, sizeof(uint32_t) * n) != cudaSuccess)) {
    cleanup();
    return fail(UFO_E_NOMEM, "device buffers for %lld particles", static_cast<long long>(n));
  }
  cudaError_t e = cudaMemcpyAsync(d_coords, coords, cb, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && seed)
    e = cudaMemcpyAsync(d_seed, seed, sizeof(int32_t) * n, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && pturns)
    e = cudaMemcpyAsync(d_pturns, pturns, sizeof(int32_t) * n, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && tb) e = cudaMemsetAsync(d_tracks, 0, tb, st);
  if (e != cudaSuccess) {
    cleanup();
    return cuda_fail(e, "upload");
  }
  rc = launch_track(ctx, prog, d_coords, d_seed, d_pturns, n, turns, mode, flags, slots, every,
                    d_tracks, d_lost, d_final, st);
  if (rc) {
    cleanup();
    return rc;
  }
  e = cudaSuccess;
  if (tb) e = cudaMemcpyAsync(tracks, d_tracks, tb, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && lost)
    e = cudaMemcpyAsync(lost, d_lost, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && final_state)
    e = cudaMemcpyAsync(final_state, d_final, cb, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cleanup();
  if (e != cudaSuccess) return cuda_fail(e, "track");
  return UFO_OK;
}

}  // extern "C"

// ============================================ allocation-free entry point
//
// ufo_track_noalloc serves callers that cannot call cudaMalloc: programs whose
// device memory belongs to another allocator (a framework's memory pool or a
// fixed arena) or that must not allocate while running, such as an online
// model inside an accelerator control loop that may neither stall on nor fail
// in an allocation mid-operation.  The caller owns every buffer it passes; the
// only scratch this path needs -- the staged opcode table the kernel
// interprets and the persistent kernel's work counter -- lives in the
// file-scope array below, which every GPU that loads this library holds
// (256 B + UFO_NOALLOC_MAX_OPS * 32 B = 256.25 KiB) until the process exits.
namespace {

struct NoallocScratch {
  unsigned long long queue;        // work counter, cleared by every call
  unsigned long long pad[31];      // keeps the table 256-byte aligned
  ufo::Op ops[UFO_NOALLOC_MAX_OPS];
};
static __device__ __align__(256) NoallocScratch g_noalloc_scratch;

struct NoallocDevice {
  bool ready;
  NoallocScratch *scratch;  // device address of g_noalloc_scratch
  int sm_count;
};
NoallocDevice g_noalloc_dev[64];

// Once per device, with that device current: resolve the array's device
// address (in host code its name is only a host-side stand-in) and upload the
// constant tables.  Runs on a device's first call.
int noalloc_setup(int device) {
  if (device < 0 || device >= 64) return fail(UFO_E_ARG, "device %d out of range", device);
  int rc = ensure_constants(device);
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  NoallocDevice &d = g_noalloc_dev[device];
  if (d.ready) return UFO_OK;
  void *ptr = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
  int sms = 0;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");
  d.scratch = static_cast<NoallocScratch *>(ptr);
  d.sm_count = sms;
  d.ready = true;
  return UFO_OK;
}

}  // namespace

extern "C" int ufo_track_noalloc(const int32_t *ops, int n_ops, const double *d_table,
                                 int64_t stride, int n_seeds, int n_dumps, const double *d_coords,
                                 const int32_t *d_seed, const int32_t *d_pturns, int64_t n,
                                 int turns, int mode, int flags, int64_t slots, int every,
                                 double *d_tracks, uint32_t *d_lost, double *d_final,
                                 void *stream) {
  if (!ops && n_ops > 0) return fail(UFO_E_ARG, "null opcode table");
  if (n_ops < 0 || n_ops > UFO_NOALLOC_MAX_OPS)
    return fail(UFO_E_ARG,
                "opcode table of %d ops exceeds the allocation-free entry point's maximum of %d",
                n_ops, UFO_NOALLOC_MAX_OPS);
  if (!d_table || stride < 1 || n_seeds < 1 || n_dumps < 0)
    return fail(UFO_E_ARG, "bad constant table (pointer, stride or seed count)");
  if (n < 0 || turns < 0) return fail(UFO_E_ARG, "negative particle or turn count");
  if (mode != UFO_MODE_TRACK && mode != UFO_MODE_SA) return fail(UFO_E_ARG, "bad mode %d", mode);
  if (slots < 0 || every < 1) return fail(UFO_E_ARG, "bad observation slots or stride");
  if (n > 0 && !d_coords) return fail(UFO_E_ARG, "null coordinates");
  // the constants are on the device: op shapes and observation indices are
  // checked here, expression programs are not (see the header)
  int rc = validate_ops(ops, n_ops, stride, n_dumps, nullptr);
  if (rc) return rc;
  int device = 0;
  UFO_CUDA(cudaGetDevice(&device));
  rc = noalloc_setup(device);
  if (rc) return rc;
  if (n == 0) return UFO_OK;
  NoallocDevice &d = g_noalloc_dev[device];
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (n_ops > 0)
    UFO_CUDA(cudaMemcpyAsync(d.scratch->ops, ops, sizeof(ufo::Op) * n_ops,
                             cudaMemcpyHostToDevice, st));
  ufo::TrackArgs a = make_args(d.scratch->ops, n_ops, d_table, stride, n_seeds, n_dumps,
                               d_coords, d_seed, d_pturns, n, turns, mode,
                               flags & ~UFO_TRACK_PLAIN, slots, every, d_tracks, d_lost, d_final,
                               &d.scratch->queue);
  return launch_kernels(a, needs_full(ops, n_ops), d.sm_count, 16, st);
}

// ===================================================== tuning and graphs

struct ufo_graph {
  ufo_ctx *ctx;
  int device;  // copied: destruction must not touch the context
  cudaGraph_t graph;
  cudaGraphExec_t exec;
};

extern "C" int ufo_closed_orbit(ufo_ctx *ctx, const ufo_prog *prog, const double *start,
                                const int32_t *seed, int64_t n, int iterations, double *orbits) {
  int rc = check_track_args(ctx, prog, n, 1, UFO_MODE_TRACK, 0, 1);
  if (rc) return rc;
  if (n == 0) return UFO_OK;
  if (!start || !orbits) return fail(UFO_E_ARG, "null start or orbit buffer");
  if (iterations < 0) return fail(UFO_E_ARG, "negative iteration count");
  if (seed) {
    for (int64_t i = 0; i < n; ++i)
      if (seed[i] < 0 || seed[i] >= prog->n_seeds)
        return fail(UFO_E_ARG, "orbit %lld: seed %d outside [0, %d)",
                    static_cast<long long>(i), seed[i], prog->n_seeds);
  }
  UFO_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  const size_t vb = sizeof(double) * 4 * n;
  double *d_start = nullptr, *d_orbits = nullptr;
  int32_t *d_seed = nullptr;
  auto cleanup = [&]() { cudaFree(d_start); cudaFree(d_orbits); cudaFree(d_seed); };
  if (cudaMalloc(&d_start, vb) != cudaSuccess || cudaMalloc(&d_orbits, vb) != cudaSuccess ||
      (seed && cudaMalloc(&d_seed, sizeof(int32_t) * n) != cudaSuccess)) {
    cleanup();
    return fail(UFO_E_NOMEM, "device buffers for %lld orbits", static_cast<long long>(n));
  }
  cudaError_t e = cudaMemcpyAsync(d_start, start, vb, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && seed)
    e = cudaMemcpyAsync(d_seed, seed, sizeof(int32_t) * n, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) {
    cleanup();
    return cuda_fail(e, "upload");
  }
  ufo::TrackArgs a = make_args(prog->ops, prog->n_ops, prog->table, prog->stride, prog->n_seeds,
                               prog->n_dumps, nullptr, d_seed, nullptr, n, 1, UFO_MODE_TRACK, 0, 0,
                               1, nullptr, nullptr, nullptr, ctx->queue);
  const unsigned blocks = static_cast<unsigned>((n + 31) / 32);
  if (prog->full)
    ufo::co_amoeba_kernel<true><<<blocks, 32, 0, st>>>(a, d_start, d_orbits, iterations);
  else
    ufo::co_amoeba_kernel<false><<<blocks, 32, 0, st>>>(a, d_start, d_orbits, iterations);
  e = cudaGetLastError();
  if (e == cudaSuccess) {
    ctx->launches.fetch_add(1);
    e = cudaMemcpyAsync(orbits, d_orbits, vb, cudaMemcpyDeviceToHost, st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cleanup();
  if (e != cudaSuccess) return cuda_fail(e, "closed orbit");
  return UFO_OK;
}

extern "C" int ufo_ctx_set_tuning(ufo_ctx *ctx, int warps_per_sm) {
  if (!ctx) return fail(UFO_E_ARG, "null context");
  if (warps_per_sm < 1 || warps_per_sm > 32)
    return fail(UFO_E_ARG, "warps_per_sm %d outside [1, 32]", warps_per_sm);
  ctx->warps_per_sm = warps_per_sm;
  return UFO_OK;
}

// Capture one tracking launch (counter reset + persistent kernel) into a CUDA
// graph; ufo_graph_launch replays it on the same device buffers.
extern "C" int ufo_graph_create(ufo_ctx *ctx, const ufo_prog *prog, const double *d_coords,
                                const int32_t *d_seed, const int32_t *d_pturns, int64_t n,
                                int turns, int mode, int flags, int64_t slots, int every,
                                double *d_tracks, uint32_t *d_lost, double *d_final,
                                ufo_graph **out) {
  if (!out) return fail(UFO_E_ARG, "null output");
  *out = nullptr;
  int rc = check_track_args(ctx, prog, n, turns, mode, slots, every);
  if (rc) return rc;
  if (n <= 0) return fail(UFO_E_ARG, "empty launch");
  if (!d_coords) return fail(UFO_E_ARG, "null coordinates");
  UFO_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t cap;
  UFO_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    rc = launch_track(ctx, prog, d_coords, d_seed, d_pturns, n, turns, mode, flags, slots, every,
                      d_tracks, d_lost, d_final, cap);
    e = cudaStreamEndCapture(cap, &graph);
  }
  cudaStreamDestroy(cap);
  if (rc) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(e, "stream capture");
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, graph, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(graph);
    return cuda_fail(e, "cudaGraphInstantiate");
  }
  ufo_graph *g = new (std::nothrow) ufo_graph;
  if (!g) {
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    return fail(UFO_E_NOMEM, "host allocation");
  }
  g->ctx = ctx;
  g->device = ctx->device;
  g->graph = graph;
  g->exec = exec;
  *out = g;
  return UFO_OK;
}

extern "C" int ufo_graph_launch(ufo_graph *g, void *stream) {
  if (!g) return fail(UFO_E_ARG, "null graph");
  UFO_CUDA(cudaSetDevice(g->ctx->device));
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : g->ctx->stream;
  UFO_CUDA(cudaGraphLaunch(g->exec, st));
  g->ctx->launches.fetch_add(1);
  return UFO_OK;
}

extern "C" void ufo_graph_destroy(ufo_graph *g) {
  if (!g) return;
  cudaSetDevice(g->device);
  cudaDeviceSynchronize();
  cudaGraphExecDestroy(g->exec);
  cudaGraphDestroy(g->graph);
  delete g;
}
