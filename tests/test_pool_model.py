"""A model check of the compacting kernel's particle pool.

track_kernel_cta (ufo_gb300/csrc/ufo_gb300.cu) lets its CTAs even out their
particles through a bounded ring with one sequence word per slot: a donor
reserves free slots with a CAS on the tail ticket and publishes each slot
after writing it; a taker claims published slots with a CAS on the head
ticket and frees each slot after reading it; a CTA leaves once it holds no
particle and the pool is empty or its head slot is still being filled.  The
kernel never waits for another CTA.  Its correctness rests on the
interleavings of those steps across CTAs, which a GPU run samples only a few
of.  This file restates the protocol step by step as Python generators (one
per CTA, yielding at every access to shared state) and runs them under many
random schedules, checking that every particle is finished exactly once,
that nothing is left in the pool, that no slot is overwritten before it is
read and that every CTA leaves.  The restatement follows the kernel's phase-B
loop; it is a test of the protocol, not of the CUDA code.
"""
import random

import pytest


class Shared:
    def __init__(self, cap, n_particles, n_ctas):
        self.cap = cap
        self.seq = [0] * cap        # 2e: free for ticket e*cap+slot; 2e+1: holds it
        self.slot = [None] * cap
        self.head = 0
        self.tail = 0
        self.finished = 0
        self.left = 0
        self.n = n_particles
        self.n_ctas = n_ctas
        self.done = {}              # particle -> times finished
        self.moved = 0


def cta(sh, parts, lanes, period):
    """One CTA's phase B.  `parts`: [particle id, turns left] pairs (the
    particles its lanes hold when the work counter runs out)."""
    parts = [list(p) for p in parts]
    k = 0
    while True:
        balance = k % period == 0
        if balance:
            seen = (sh.finished, sh.left)
            yield
        total = len(parts)
        want = 0
        if total == 0:
            want = lanes
        elif balance:
            running = sh.n_ctas - seen[1]
            unfinished = sh.n - seen[0]
            if running > 0 and unfinished > 0:
                share = -(-unfinished // running)
                whole = -(-share // 32) * 32
                if total > whole:
                    want = -(total - whole)
                elif total < share:
                    want = max(0, min(whole, lanes) - total)
        leave = False
        if want < 0:                       # reserve free slots at the tail
            t0 = sh.tail
            yield
            n = 0
            while n < -want:
                t = t0 + n
                ok = sh.seq[t % sh.cap] == 2 * (t // sh.cap)
                yield
                if not ok:
                    break
                n += 1
            if n and sh.tail != t0:        # the CAS fails: another CTA moved the tail
                n = 0
            elif n:
                sh.tail = t0 + n
            yield
            give, parts = parts[total - n:], parts[:total - n]
            for i, p in enumerate(give):   # each donor thread: write, fence, publish
                t = t0 + i
                assert sh.seq[t % sh.cap] == 2 * (t // sh.cap), 'slot overwritten'
                sh.slot[t % sh.cap] = p
                yield
                sh.seq[t % sh.cap] = 2 * (t // sh.cap) + 1
                sh.moved += 1
                yield
        elif want > 0:                     # claim filled slots at the head
            h = sh.head
            yield
            n = 0
            while n < want:
                t = h + n
                ok = sh.seq[t % sh.cap] == 2 * (t // sh.cap) + 1
                yield
                if not ok:
                    break
                n += 1
            leave = total == 0 and n == 0
            if n and sh.head != h:         # the CAS fails: try again later
                n = 0
            elif n:
                sh.head = h + n
            if leave:
                sh.left += 1
            yield
            for i in range(n):             # each taker thread: read, fence, free
                t = h + i
                assert sh.seq[t % sh.cap] == 2 * (t // sh.cap) + 1, 'slot not filled'
                p = sh.slot[t % sh.cap]
                sh.slot[t % sh.cap] = None
                parts.append(p)
                yield
                sh.seq[t % sh.cap] = 2 * (t // sh.cap + 1)
                yield
        if leave:
            assert not parts
            return
        # one turn for the CTA's particles
        keep = []
        fin = 0
        for p in parts:
            p[1] -= 1
            if p[1] <= 0:
                sh.done[p[0]] = sh.done.get(p[0], 0) + 1
                fin += 1
            else:
                keep.append(p)
        parts = keep
        if fin:
            sh.finished += fin
        yield
        k += 1


def run_model(seed, n_ctas=6, lanes=96, period=4, cta_fn=cta):
    rng = random.Random(seed)
    # uneven hold-outs: some CTAs start empty, some full, long and short lives
    holdings = []
    pid = 0
    for c in range(n_ctas):
        m = rng.choice([0, 5, lanes // 2, lanes, lanes])
        ps = []
        for _ in range(m):
            ps.append((pid, rng.choice([1, 2, 3, 40, 120])))
            pid += 1
        holdings.append(ps)
    sh = Shared(cap=n_ctas * lanes, n_particles=pid, n_ctas=n_ctas)
    gens = [cta_fn(sh, h, lanes, period) for h in holdings]
    alive = list(range(n_ctas))
    steps = 0
    while alive:
        i = rng.choice(alive)
        try:
            next(gens[i])
        except StopIteration:
            alive.remove(i)
        steps += 1
        assert steps < 5_000_000, 'no progress'
    return sh


@pytest.mark.parametrize('n_ctas,lanes,period', [(3, 64, 1), (6, 96, 4), (12, 64, 2)])
def test_pool_protocol_finishes_every_particle_once(n_ctas, lanes, period):
    moved = 0
    for seed in range(300):
        sh = run_model(seed, n_ctas, lanes, period)
        assert sorted(sh.done) == list(range(sh.n)), seed
        assert all(v == 1 for v in sh.done.values()), seed
        assert sh.head == sh.tail, seed            # nothing left in the pool
        assert all(s is None for s in sh.slot), seed
        assert sh.left == sh.n_ctas, seed
        assert sh.finished == sh.n, seed
        moved += sh.moved
    assert moved > 0                               # the CTAs did exchange particles


def test_pool_model_catches_a_wrong_leave_rule():
    """The same model with a CTA leaving as soon as it is empty (ignoring
    particles waiting in the pool) strands particles on some schedules: the
    sweep above is wide enough to see such a mistake."""
    import inspect
    src = inspect.getsource(cta)
    bad = src.replace('leave = total == 0 and n == 0', 'leave = total == 0')
    assert bad != src
    ns = dict(globals())
    exec(bad, ns)
    stranded = 0
    for seed in range(300):
        try:
            sh = run_model(seed, cta_fn=ns['cta'])
        except AssertionError:
            stranded += 1
            continue
        stranded += sh.head != sh.tail or len(sh.done) != sh.n
    assert stranded > 0
