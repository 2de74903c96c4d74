"""A CPU model of the mbarrier protocol of the warp-specialised tcgen05
convolution (``k_conv3d_tc`` in pybella_gb300/csrc/bella_cnn.cu), run under
random interleavings of its roles.

The kernel's roles meet only on mbarriers whose phases are told apart by parity
alone, so a waiter must never fall two phases behind a barrier it waits on.  The
model keeps the kernel's ring sizes (read from the source), its work shares
(one contiguous share of (row block, x-plane) items per CTA, cut into runs) and
its hand-offs:

* producers stage input plane i into slot i % TC_SLOTS once the MMAs of plane
  i - TC_SLOTS are complete (completion ring entry (i - TC_SLOTS) % TC_DRING);
  the copies' completion arrives on the slot's ``full`` barrier later, in order;
* the MMA thread waits for ``full``, acquires the accumulators of the output
  planes it starts (waiting for the epilogue to release plane o - TC_LIVE), issues
  one MMA window per input plane -- TC_RING accumulator blocks, the window of
  outputs w, w-1, w-2 at blocks tc_win(w) + 0, 1, 2 -- and commits to completion
  entry i % TC_DRING (completions happen later, in issue order);
* epilogue warps wait for the completion of input plane q+1 of the run, read
  output plane q from its blocks (``tc_blocks``: one, or two at the wrap),
  release them.

Checked: no deadlock, no parity alias, a window never wraps, every contribution
lands in one of its output's blocks, an output plane is read only after all
its contributions are complete, a slot or accumulator block is reused only
after its last reader is done.
"""
import os
import random
import re

import pytest

from conftest import ROOT


def _const(name):
    src = open(os.path.join(ROOT, "pybella_gb300", "csrc", "bella_cnn.cu")).read()
    return int(re.search(r"constexpr int %s = (\d+);" % name, src).group(1))


S, D, R, LIVE = _const("TC_SLOTS"), _const("TC_DRING"), _const("TC_RING"), _const("TC_LIVE")


def tc_win(w):
    """First accumulator block of the window whose first output is w (the kernel's tc_win)."""
    return (1 - w) % LIVE


def tc_blocks(o):
    """The accumulator blocks of output o (the kernel's tc_blocks)."""
    a = (-o) % LIVE
    return [LIVE if a == LIVE - 1 else a + 1] + ([LIVE + 1] if a == 0 else [0] if a == LIVE - 1 else [])
NPROD, NEPI = _const("TC_PROD_WARPS"), 8


class Bar:
    def __init__(self, count, name):
        self.count, self.pending, self.done, self.name = count, count, 0, name

    def arrive(self):
        self.pending -= 1
        assert self.pending >= 0, self.name
        if self.pending == 0:
            self.done += 1
            self.pending = self.count

    def ready(self, k):
        """Waiting for completion k (0-based) by its parity k & 1."""
        assert self.done <= k + 1, "parity alias on %s: %d completions, waiting for %d" % (self.name, self.done, k)
        return self.done == k + 1


def _runs(cta, work, nx, nblk):
    out, idx, hi = [], cta * work, min(cta * work + work, nblk * nx)
    while idx < hi:
        fb, ia = divmod(idx, nx)
        ib = min(nx, ia + (hi - idx))
        out.append((fb, ia, ib))
        idx += ib - ia
    return out


def _simulate(nx, xseg, work, nblk, cta, seed):
    rng = random.Random(seed)
    runs = _runs(cta, work, nx, nblk)
    full = [Bar(NPROD, "full%d" % k) for k in range(S)]
    done = [Bar(1, "done%d" % k) for k in range(D)]
    free = [Bar(NEPI, "free%d" % k) for k in range(LIVE)]
    inputs = [p for (_, ia, ib) in runs for p in range(ia - 1, ib + 1)]
    owner, contrib, slot_data = {}, {}, {}
    commits, landings = [], [[] for _ in range(NPROD)]

    def producer(w):
        for i, _ in enumerate(inputs):
            slot, prev = i % S, i - S
            if prev >= 0:
                while not done[prev % D].ready(prev // D):
                    yield
            slot_data[(slot, w)] = i
            landings[w].append(slot)
            yield

    def mma():
        i = obase = acq = 0
        for (_, ia, ib) in runs:
            for p in range(ia - 1, ib + 1):
                slot = i % S
                while not full[slot].ready(i // S):
                    yield
                assert all(slot_data[(slot, w)] == i for w in range(NPROD)), "slot holds another plane"
                if 0 <= p < nx:
                    s0 = (p // xseg) * xseg
                    qlo, qhi = max(p - 1, ia, s0), min(p + 1, ib - 1, s0 + xseg - 1)
                    if qlo <= qhi:
                        olo, ohi = obase + qlo - ia, obase + qhi - ia
                        while acq <= ohi:
                            if acq >= LIVE:
                                while not free[acq % LIVE].ready(acq // LIVE - 1):
                                    yield
                            acq += 1
                        w = obase + p + 1 - ia                  # the window's first output
                        assert tc_win(w) + (w - olo) <= R - 1, "window wraps"
                        for o in range(olo, ohi + 1):
                            if o not in contrib:                # first contribution: claim the blocks
                                for b in tc_blocks(o):
                                    assert b not in owner or contrib[owner[b]] == "done", "reused too early"
                                    owner[b] = o
                                contrib[o] = 0
                            blk = tc_win(w) + (w - o)
                            assert blk in tc_blocks(o) and owner[blk] == o, ("contribution in a foreign block", o, blk)
                            contrib[o] += 1
                commits.append(i % D)
                i += 1
                yield
            obase += ib - ia

    def epilogue(w):
        o = ibase = 0
        for (_, ia, ib) in runs:
            for q in range(ia, ib):
                j = ibase + (q - ia + 2)
                while not done[j % D].ready(j // D):
                    yield
                assert all(owner[b] == o for b in tc_blocks(o))
                want = sum(1 for pp in (q - 1, q, q + 1) if 0 <= pp < nx and pp // xseg == q // xseg)
                assert contrib[o] == want, ("incomplete plane", q, contrib[o], want)
                yield
                free[o % LIVE].arrive()
                if free[o % LIVE].pending == free[o % LIVE].count:
                    contrib[o] = "done"
                o += 1
            ibase += ib - ia + 2

    def asynchronous():
        while True:
            for w in range(NPROD):
                if landings[w] and rng.random() < 0.3:
                    full[landings[w].pop(0)].arrive()
            if commits and rng.random() < 0.5:
                done[commits.pop(0)].arrive()
            yield

    # seeds pick which role runs slow, so that every waiter is made to lag
    slow = ("none", "epilogue", "producer", "mma", "async")[seed % 5]
    weight = {"producer": 1.0, "mma": 1.0, "epilogue": 1.0, "async": 1.0}
    if slow in weight:
        weight[slow] = 0.05
    actors = [("producer", producer(w)) for w in range(NPROD)] + [("mma", mma())] + \
             [("epilogue", epilogue(w)) for w in range(NEPI)]
    bg = ("async", asynchronous())
    steps = 0
    while actors:
        steps += 1
        assert steps < 5_000_000, "deadlock"
        pool = actors + [bg]
        role, a = rng.choices(pool, weights=[weight[r] for r, _ in pool])[0]
        try:
            next(a)
        except StopIteration:
            actors.remove((role, a))


@pytest.mark.parametrize("nx,xseg,nblk,grid", [(129, 129, 35, 152), (40, 8, 3, 7), (24, 12, 2, 3), (9, 9, 1, 1),
                                               (12, 12, 9, 152), (25, 5, 3, 4)])
def test_tc_convolution_protocol(nx, xseg, nblk, grid):
    items = nblk * nx
    grid = min(grid, items)
    work = -(-items // grid)
    ctas = range(grid) if grid <= 8 else (0, 1, grid // 2, grid - 1)
    for cta in ctas:
        for seed in range(5):
            _simulate(nx, xseg, work, nblk, cta, seed)
