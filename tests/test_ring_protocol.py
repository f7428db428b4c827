"""(CPU) Models of the shared-memory rings of the whole-run kernel
(numericalflowiteration_gb300/csrc/run_split_1d.cu: issue, copy_part,
start_step, refill) and of the 2D/3D split trace (simulate_nd), run under
random interleavings of the CTA's warps.

The ring is one stream of chunks over the run: chunk g sits in slot
g % R; chunk j of step n holds slabs [max(0, k_hi - S + 1), k_hi],
k_hi = n - 1 - j S.  The last warp to release a slot refills it with chunk
g + R (of this step, or of step n + 1 without its newest slab n, which the
field solve of step n writes); thread 0, after the barriers of step n - 1,
issues the newest slab of chunk 0 and the first chunks whose predecessor
was not in the previous step.  Checked: every chunk armed once and each
of its slabs copied exactly once, no slot re-armed while a warp still
reads it, no slab copied before the step that writes it has finished, and
no warp left waiting (no deadlock).  Two planted mistakes must be caught.
"""
import random

import pytest

R = 3  # kRing


class ProtocolError(AssertionError):
    pass


def check(cond, *what):
    if not cond:
        raise ProtocolError(what)


def simulate(n0, n1, S, W, seed, newest_early=False, refill_early=False):
    rnd = random.Random(seed)

    def nchunks(n):
        return (n + S - 1) // S if n > 0 else 0

    def chunk_range(n, j):
        k_hi = n - 1 - j * S
        return max(0, k_hi - S + 1), k_hi

    armed, copied, busy = {}, {}, {}
    released = [0] * R

    def copy_part(g, n, j, k_from, k_to, final_upto):
        check(armed.get(g) == (n, j), "copy into a chunk that is not armed", g)
        for k in range(k_from, k_to + 1):
            check(k not in copied[g], "slab copied twice", g, k)
            check(k <= final_upto, "slab copied before its step finished", g, k, final_upto)
            copied[g].add(k)

    def issue(g, n, j, k_last, final_upto):
        s = g % R
        check(s not in busy, "slot re-armed while in use", g, busy)
        check(g not in armed, "chunk armed twice", g)
        armed[g], copied[g], busy[s] = (n, j), set(), g
        lo, _ = chunk_range(n, j)
        if k_last >= lo:
            copy_part(g, n, j, lo, k_last, final_upto)

    gbase = gprev = 0
    for n in range(n0, n1 + 1):
        nc = nchunks(n)
        # thread 0 after the barriers of step n - 1: slabs <= n - 1 are final
        for j in range(min(R, nc)):
            g = gbase + j
            pred_prev = n != n0 and g >= R and g - R >= gprev
            lo, hi = chunk_range(n, j)
            if not pred_prev:
                issue(g, n, j, hi, n - 1)
            elif j == 0 and not newest_early:
                copy_part(g, n, 0, hi, hi, n - 1)
        pos = [0] * W  # next chunk of each warp
        while any(p < nc for p in pos):
            ready = []
            for w in range(W):
                if pos[w] < nc:
                    g = gbase + pos[w]
                    lo, hi = chunk_range(n, pos[w])
                    if g in armed and copied[g] == set(range(lo, hi + 1)) and busy.get(g % R) == g:
                        ready.append(w)
            check(ready, "deadlock: no warp's data is complete", n, pos)
            w = rnd.choice(ready)
            j = pos[w]
            g = gbase + j
            pos[w] += 1
            s = g % R
            released[s] += 1
            if released[s] == (W - 1 if refill_early and W > 1 else W):
                released[s] = 0
                del busy[s]
                jj = j + R
                if jj < nc:
                    issue(g + R, n, jj, chunk_range(n, jj)[1], n - 1)
                elif n + 1 <= n1 and jj - nc < nchunks(n + 1):
                    j1 = jj - nc
                    hi1 = chunk_range(n + 1, j1)[1]
                    # during step n only slabs <= n - 1 are final
                    k_last = hi1 if (j1 > 0 or newest_early) else hi1 - 1
                    issue(g + R, n + 1, j1, k_last, n - 1)
        gprev, gbase = gbase, gbase + nc
    check(set(armed) == set(range(gbase)), "chunks never armed", sorted(set(range(gbase)) - set(armed)))
    for g, (n, j) in armed.items():
        lo, hi = chunk_range(n, j)
        check(copied[g] == set(range(lo, hi + 1)), "chunk not completely copied", g)
    check(not busy, "slots left armed", busy)
    return gbase


RANGES = [(0, 0), (0, 1), (0, 5), (0, 40), (3, 30), (1, 1), (10, 11), (0, 120), (57, 200)]


@pytest.mark.parametrize("S", [1, 2, 3, 5, 10, 32])
def test_ring_protocol_holds(S):
    for n0, n1 in RANGES:
        for W in (1, 2, 8):
            for seed in range(3):
                total = simulate(n0, n1, S, W, seed)
                assert total == sum((n + S - 1) // S for n in range(max(n0, 1), n1 + 1))


def simulate_nd(n, batches, S, W, seed, no_wrap=False):
    """The per-step ring of the 2D/3D split trace
    (numericalflowiteration_gb300/csrc/trace_split_nd.cu): a stream of
    batches x nchunks chunks, chunk g = chunk g mod nchunks of batch
    g / nchunks in slot g mod R; the first R issued up front, then the last
    warp to release a slot issues chunk g + R, i.e. chunk (j + R) mod
    nchunks, while g + R < total.  Each warp waits for chunk g on its slot
    with phase parity (g / R) & 1; checked: the slot then holds chunk g
    (so the parity is unambiguous) with the slabs of chunk g mod nchunks."""
    rnd = random.Random(seed)
    nchunks = (n + S - 1) // S if n > 0 else 0
    total = batches * nchunks
    holds = {}   # slot -> (g, j) of the chunk it holds
    issued = []
    released = [0] * R

    def issue(g, j):
        s = g % R
        check(s not in holds, "slot re-armed while in use", g, holds)
        holds[s] = (g, j)
        issued.append(g)

    for g0 in range(min(R, total)):
        issue(g0, g0 % nchunks)
    pos = [0] * W
    while any(p < total for p in pos):
        ready = [w for w in range(W) if pos[w] < total and holds.get(pos[w] % R, (None,))[0] == pos[w]]
        check(ready, "deadlock", pos, holds)
        w = rnd.choice(ready)
        g = pos[w]
        j = g % nchunks
        check(holds[g % R] == (g, j), "slot holds another chunk", g, holds[g % R])
        pos[w] += 1
        s = g % R
        released[s] += 1
        if released[s] == W:
            released[s] = 0
            del holds[s]
            if g + R < total:
                jr = j + R
                if not no_wrap:
                    while jr >= nchunks:
                        jr -= nchunks
                issue(g + R, jr)
    check(issued == list(range(total)), "stream not issued in order", issued[:10])
    check(not holds, "slots left armed", holds)


@pytest.mark.parametrize("S", [1, 2, 3, 15, 16])
def test_nd_ring_protocol_holds(S):
    for n in (0, 1, 2, 5, 17, 40, 100):
        for batches in (1, 2, 3, 7):
            for W in (1, 4, 16):
                for seed in range(2):
                    simulate_nd(n, batches, S, W, seed)


def test_planted_mistakes_are_caught():
    with pytest.raises(ProtocolError, match="another chunk"):
        simulate_nd(5, 4, 2, 4, 0, no_wrap=True)
    with pytest.raises(ProtocolError, match="before its step finished"):
        simulate(0, 40, 4, 8, 0, newest_early=True)
    with pytest.raises(ProtocolError):
        for seed in range(20):
            simulate(0, 40, 4, 8, seed, refill_early=True)
