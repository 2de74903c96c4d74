"""A CPU model of the stage ring of the tcgen05 weight-gradient kernel
(``k_wgrad_tc`` in pybella_gb300/csrc/bella_cnn.cu), run under random MMA
completion delays.

The kernel keeps ``nst`` stages (two or three, WG_MAX_STAGES at most).  Per item
i of a CTA's share: every thread waits for its own copies of item i, the block
meets at a barrier, one thread issues item i's MMAs and commits them to the
stage's mbarrier ``bar[i % nst]``; then every thread waits (mbarrier parity
((i-1) / nst) & 1) for the MMAs of item i-1 and stages item i+nst-1 into stage
(i-1) % nst.  The model checks that a stage is overwritten only after the MMAs
that read it have completed, that the MMAs of an item read the data of that item,
and that no parity wait can see a later phase of the same parity (which would
make it wait for ever).
"""
import os
import random
import re

import pytest

from conftest import ROOT


def _const(name):
    src = open(os.path.join(ROOT, "pybella_gb300", "csrc", "bella_cnn.cu")).read()
    return int(re.search(r"constexpr int %s = (\d+);" % name, src).group(1))


MAXST = _const("WG_MAX_STAGES")


def _simulate(n_it, nst, seed):
    rng = random.Random(seed)
    stage_item = [None] * nst          # which item's data each stage holds
    completions = [0] * nst            # completed phases of bar[k]
    pending = []                       # issued MMA groups, completing in issue order: (item, stage)
    reads_done = set()

    def drain(force=False):
        while pending and (force or rng.random() < 0.5):
            item, st = pending.pop(0)
            assert stage_item[st] == item, "MMAs read a stage restaged under them"
            reads_done.add(item)
            completions[st] += 1

    def wait(st, phase):
        # try_wait.parity: true once phase `phase` of bar[st] has completed; a count two
        # phases ahead would read as incomplete again (parity alias)
        while True:
            assert completions[st] <= phase + 1, "parity alias"
            if completions[st] == phase + 1:
                return
            drain(force=not pending or rng.random() < 0.3)
            assert pending or completions[st] == phase + 1, "wait for an MMA group never issued"

    def stage(it, st):
        if stage_item[st] is not None:
            assert stage_item[st] in reads_done, "stage overwritten before its MMAs completed"
        stage_item[st] = it

    for k in range(nst - 1):           # prologue: items 0 .. nst-2 (empty copy groups past the share)
        if k < n_it:
            stage(k, k)
    for i in range(n_it):
        b = i % nst
        assert stage_item[b] == i, "item's copies not in its stage"
        pending.append((i, b))         # issue + commit to bar[b]
        drain()
        nxt = i + nst - 1
        if i >= 1 and nxt < n_it:
            wait((i - 1) % nst, (i - 1) // nst)
        if nxt < n_it:
            stage(nxt, nxt % nst)
    drain(force=True)
    assert reads_done == set(range(n_it))
    assert sum(completions) == n_it


@pytest.mark.parametrize("nst", sorted({2, MAXST}))
@pytest.mark.parametrize("n_it", [0, 1, 2, 3, 5, 30, 31])
def test_wgrad_stage_ring(nst, n_it):
    for seed in range(20):
        _simulate(n_it, nst, seed)
