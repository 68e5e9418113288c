"""A model of the multi-block team's hand-off protocol, run under random
interleavings on the CPU.

Each block of a team iterates: expand (write its stage region of iteration i
into ring slot i % kStageRing) -> publish (its ready word for iteration i, its
part of cut i; the first block also clears cut slot i - 2*kCutLag - 2) -> wait
for its producer's ready word (block (b + i) % blocks) -> wait for cut
i - kCutLag to be complete and test it -> push (read the producer's region).
The scheduler advances one enabled block by one step at a time, in a random
order.  The invariants the kernel's comments state are checked at every step:
a region is read only while it holds the iteration the reader expects, a cut
slot is published into only when it is clear or holds the same iteration, a
slot is cleared only after every block has tested it, ready words are never
lapped, and no interleaving deadlocks.  The ring sizes come from
engine_types.h; planted mistakes (a ring one slot shorter, a clear one
iteration earlier) must be caught.
"""
import os
import random
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _constants():
    src = open(os.path.join(ROOT, "cuda_a_star_gb300", "csrc", "engine_types.h")).read()
    get = lambda name: int(re.search(r"constexpr uint32_t %s = (\d+);" % name, src).group(1))
    return get("kStageRing"), get("kCutLag"), get("kCuts")


class Violation(Exception):
    pass


def simulate(blocks, iters, ring, lag, cuts, clear_lag, seed):
    rng = random.Random(seed)
    it = [0] * blocks
    phase = ["expand"] * blocks
    region = [[None] * ring for _ in range(blocks)]      # iteration held by each region
    ready = [[0] * ring for _ in range(blocks)]           # (iteration + 1) published
    slot = [set() for _ in range(cuts)]                   # (iteration, block) published since the clear
    tested = [-1] * blocks                                # last cut iteration each block tested
    done = 0
    while done < blocks:
        enabled = []
        for b in range(blocks):
            if it[b] >= iters:
                continue
            i, ph = it[b], phase[b]
            if ph == "wait_ready":
                p = (b + i) % blocks
                if p != b and ready[p][i % ring] < i + 1:
                    continue
            elif ph == "wait_cut":
                c = i - lag
                if c >= 0 and len({x for x in slot[c % cuts] if x[0] == c}) < blocks:
                    continue
            enabled.append(b)
        if not enabled:
            raise Violation("deadlock")
        b = rng.choice(enabled)
        i, ph = it[b], phase[b]
        if ph == "expand":
            region[b][i % ring] = i
            phase[b] = "publish"
        elif ph == "publish":
            w = ready[b][i % ring]
            if w > i + 1:
                raise Violation("ready word lapped")
            ready[b][i % ring] = i + 1
            s = slot[i % cuts]
            if any(x[0] != i for x in s):
                raise Violation("cut slot %d published into while it holds another iteration" % (i % cuts))
            s.add((i, b))
            if b == 0 and i >= clear_lag:
                c = i - clear_lag
                if any(tested[x] < c for x in range(blocks)):
                    raise Violation("cut %d cleared before every block tested it" % c)
                slot[c % cuts] = {x for x in slot[c % cuts] if x[0] != c}
            phase[b] = "wait_ready"
        elif ph == "wait_ready":
            p = (b + i) % blocks
            if p != b and ready[p][i % ring] != i + 1:
                raise Violation("ready word of iteration %d lapped" % i)
            phase[b] = "wait_cut"
        elif ph == "wait_cut":
            c = i - lag
            if c >= 0:
                s = slot[c % cuts]
                if {x[1] for x in s if x[0] == c} != set(range(blocks)) or any(x[0] != c for x in s):
                    raise Violation("cut %d tested while its slot holds other publications" % c)
                tested[b] = c
            phase[b] = "push"
        else:  # push
            p = (b + i) % blocks
            if region[p][i % ring] != i:
                raise Violation("region of iteration %d overwritten before its push" % i)
            it[b] += 1
            phase[b] = "expand"
            if it[b] == iters:
                done += 1
    return True


@pytest.mark.parametrize("blocks", [2, 3, 5, 8])
def test_protocol_holds_under_random_interleavings(blocks):
    ring, lag, cuts = _constants()
    assert ring >= lag + 2 and cuts > 3 * lag + 2
    for seed in range(150):
        simulate(blocks, 40, ring, lag, cuts, 2 * lag + 2, seed)


def test_model_catches_a_ring_one_slot_short():
    ring, lag, cuts = _constants()
    found = False
    for seed in range(400):
        try:
            simulate(4, 40, lag + 1, lag, cuts, 2 * lag + 2, seed)
        except Violation:
            found = True
            break
    assert found


def test_model_catches_an_early_cut_clear():
    ring, lag, cuts = _constants()
    found = False
    for seed in range(400):
        try:
            simulate(4, 40, ring, lag, cuts, 2 * lag + 1, seed)
        except Violation:
            found = True
            break
    assert found
