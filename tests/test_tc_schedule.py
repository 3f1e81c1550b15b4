"""Model check of the tensor-core far-field kernel's barrier protocol (planes_tc_kernel in
mma_gb300/csrc/hankel_tc.cu), on the CPU.

The warp programs -- TMA producer, MMA issuer, generator groups that interleave the previous
tile's epilogue chunks with their K-blocks -- are replayed under random interleavings with the
mbarrier semantics the kernel relies on: a phase counter, pending arrivals, transaction bytes, and
try_wait.parity(p) passing when the most recently completed phase has parity p.  Checked:
no deadlock; no parity wait passing on a phase two behind the one intended (the failure of a
per-tile K-block assignment, where a group's consecutive K-blocks can be more than STAGES
apart); no stage overwritten before its MMAs consumed it; no accumulator reused before drained.
The kernel's constants are mirrored here: STAGES 4, 16 generator warps, two accumulators, two
epilogue chunks per warp, groups of 64/MM warps, at most STAGES groups.
"""
import random

import pytest

STAGES, NGEN, NACC, EPI = 4, 16, 2, 2


class Bar:
    def __init__(self, count):
        self.count, self.pending, self.tx, self.phase = count, count, 0, 0

    def arrive(self, tx=0):
        self.tx += tx
        self.pending -= 1
        self._complete()

    def complete_tx(self, b):
        self.tx -= b
        self._complete()

    def _complete(self):
        if self.pending == 0 and self.tx == 0:
            self.phase += 1
            self.pending = self.count

    def passes(self, parity):
        return (self.phase & 1) != parity


def simulate(MM, nkb, tiles, seed, per_tile_assignment=False):
    rnd = random.Random(seed)
    RC = 128 // MM
    GW = RC // 2
    NG = min(NGEN // GW, STAGES)
    full = [Bar(1 + GW) for _ in range(STAGES)]
    empty = [Bar(1) for _ in range(STAGES)]
    accf = [Bar(1) for _ in range(NACC)]
    acce = [Bar(NGEN) for _ in range(NACC)]
    owner = [None] * STAGES
    consumed, drained, acc_tile, errs = set(), {}, [None] * NACC, []

    def wait(bar, parity, needed_phase):
        if bar.passes(parity):
            if needed_phase >= 0 and bar.phase < needed_phase + 1:
                errs.append("parity wait passed %d phases early" % (needed_phase + 1 - bar.phase))
            return True
        return False

    def producer():
        it = 0
        for _ in range(tiles):
            for _ in range(nkb):
                s, n = it % STAGES, it // STAGES
                while not wait(empty[s], (n & 1) ^ 1, n - 1):
                    yield
                full[s].arrive(tx=2)
                yield
                full[s].complete_tx(1)
                yield
                full[s].complete_tx(1)
                it += 1

    def mma():
        it = 0
        for tt in range(tiles):
            a = tt % NACC
            while not wait(acce[a], ((tt // NACC) & 1) ^ 1, tt // NACC - 1):
                yield
            if acc_tile[a] is not None and drained.get(acc_tile[a], 0) < NGEN:
                errs.append("accumulator reused before drained")
            acc_tile[a] = tt
            for _ in range(nkb):
                s, n = it % STAGES, it // STAGES
                while not wait(full[s], n & 1, n):
                    yield
                if owner[s] != it:
                    errs.append("stage %d holds K-block %r, the MMA wants %d" % (s, owner[s], it))
                consumed.add(it)
                yield
                empty[s].arrive()
                it += 1
            accf[a].arrive()

    def generator(gw):
        grp = gw // GW

        def gen(it):
            s, n = it % STAGES, it // STAGES
            while not wait(empty[s], (n & 1) ^ 1, n - 1):
                yield
            if it >= STAGES and it - STAGES not in consumed:
                errs.append("stage overwritten before K-block %d was consumed" % (it - STAGES))
            owner[s] = it
            yield
            full[s].arrive()

        def epi(tt, j):
            a = tt % NACC
            if j == 0:
                while not wait(accf[a], (tt // NACC) & 1, tt // NACC):
                    yield
            yield
            if j == EPI - 1:
                drained[tt] = drained.get(tt, 0) + 1
                acce[a].arrive()

        prev = -1
        for tt in range(tiles):
            it0, j = tt * nkb, 0
            if grp < NG:
                kb = grp if per_tile_assignment else (grp + NG - it0 % NG) % NG
                while kb < nkb:
                    yield from gen(it0 + kb)
                    if prev >= 0 and j < EPI:
                        yield from epi(tt - 1, j)
                        j += 1
                    kb += NG
            while prev >= 0 and j < EPI:
                yield from epi(tt - 1, j)
                j += 1
            prev = tt
        for j in range(EPI):
            yield from epi(tiles - 1, j)

    procs = [producer(), mma()] + [generator(g) for g in range(NGEN)]
    live, steps = list(range(len(procs))), 0
    while live and not errs:
        i = rnd.choice(live)
        try:
            next(procs[i])
        except StopIteration:
            live.remove(i)
        steps += 1
        if steps > 400000:
            errs.append("deadlock")
    return errs


@pytest.mark.parametrize("MM", [8, 16, 32])
@pytest.mark.parametrize("nkb", [1, 3, 7, 16])
def test_schedule_is_safe(MM, nkb):
    for seed in range(3):
        for tiles in (1, 3):
            assert simulate(MM, nkb, tiles, seed) == []


def test_per_tile_assignment_is_caught():
    """The model finds the hazard of assigning K-blocks to groups by their number within the tile."""
    found = any(simulate(32, 7, 2, seed, per_tile_assignment=True) for seed in range(4))
    assert found
