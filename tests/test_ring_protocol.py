"""The logits kernel's plane-granular W ring (ll_kernel for K = 112 and 128, tc_kernels.cu), as a
discrete model with mbarrier parity semantics: one producer thread fills six plane slots in ring
order, one or two MMA-issuing threads (two with an even chunk count, one chunk of each pair each)
wait for a plane before its first product and release its slot after its last. Random copy and
MMA latencies; the MMAs read their plane when they execute in the tensor pipe (in issue order,
both issuers interleaved) and a commit arrives once everything issued before it executed. The
model checks that no fill overwrites a slot before its release, that every product reads its
own (chunk, plane) fill, and that the schedule never deadlocks. The kernel's
constants are restated here: the fill position of plane fill u of chunk j (wpos), the product
order (kOrder), the products' W planes (prod_w) and the steps that wait and release."""
import random

import pytest

K_ORDER = [2, 1, 4, 0, 3, 5]          # products in issue order
WAIT_STEPS, RELEASE_STEPS = (0, 1, 3), (0, 2, 5)
NSLOT = 6


def prod_w(pr):
    return 2 if pr == 2 else (1 if pr in (1, 4) else 0)


class Bar:
    """mbarrier: a phase completes after `count` arrivals; try_wait.parity(p) succeeds once the
    phase with parity p has completed."""

    def __init__(self, count=1):
        self.count, self.pending, self.phase = count, count, 0

    def arrive(self):
        self.pending -= 1
        assert self.pending >= 0
        if self.pending == 0:
            self.phase += 1
            self.pending = self.count

    def ready(self, parity):
        return (self.phase & 1) != parity


def simulate(n_chunks, my_tiles, seed, pipe_depth=4):
    rng = random.Random(seed)
    two = n_chunks % 2 == 0
    wpos = (lambda j, u: 6 * (j >> 1) + 2 * u + (j & 1)) if two else (lambda j, u: 3 * j + u)
    w_full = [Bar() for _ in range(NSLOT)]
    w_empty = [Bar() for _ in range(NSLOT)]
    content = [None] * NSLOT
    busy = [False] * NSLOT
    copies = []  # [cycles left, slot, (chunk, plane)]
    # the tensor pipe: products and commits in issue order, both issuers' interleaved; a product
    # reads its W plane when it executes, a commit arrives once everything before it executed
    pipe = []  # [cycles left, "mma", slot, (chunk, plane)] or [0, "commit", slot, None]

    def producer():
        j = 0
        group = 2 if two else 1
        for _ in range(my_tiles):
            for _ in range(0, n_chunks, group):
                for u in range(3):
                    for g in range(group):
                        pos = wpos(j + g, u)
                        ws = pos % NSLOT
                        while not w_empty[ws].ready(((pos // NSLOT) & 1) ^ 1):
                            yield
                        assert not busy[ws], ("fill over an unreleased slot", pos)
                        busy[ws] = True
                        copies.append([rng.randint(1, 40), ws, (j + g, 2 - u)])
                j += group

    def issue(item):
        while len(pipe) >= pipe_depth:
            yield
        pipe.append(item)

    def issuer(role):
        j = 0
        for _ in range(my_tiles):
            for ch in range(n_chunks):
                if two and (ch & 1) != role:
                    j += 1
                    continue
                for st, pr in enumerate(K_ORDER):
                    u = 2 - prod_w(pr)
                    pos = wpos(j, u)
                    ws = pos % NSLOT
                    if st in WAIT_STEPS:
                        while not w_full[ws].ready((pos // NSLOT) & 1):
                            yield
                    for _ in range(2):  # K / 16 MMAs per product, two are enough for the model
                        yield from issue([rng.randint(1, 6), "mma", ws, (j, prod_w(pr))])
                    if st in RELEASE_STEPS:
                        yield from issue([0, "commit", ws, None])
                j += 1

    actors = [producer(), issuer(0)] + ([issuer(1)] if two else [])
    done = [False] * len(actors)
    for _ in range(10 ** 6):
        if all(done) and not pipe:
            return
        for c in copies:
            c[0] -= 1
        for c in [c for c in copies if c[0] <= 0]:
            copies.remove(c)
            content[c[1]] = c[2]
            w_full[c[1]].arrive()
        if pipe:
            head = pipe[0]
            head[0] -= 1
            if head[0] <= 0:
                pipe.pop(0)
                if head[1] == "mma":
                    assert content[head[2]] == head[3], ("stale plane read", head[3], content[head[2]])
                else:
                    busy[head[2]] = False
                    w_empty[head[2]].arrive()
        order = list(range(len(actors)))
        rng.shuffle(order)
        for i in order:
            if not done[i]:
                try:
                    next(actors[i])
                except StopIteration:
                    done[i] = True
    raise AssertionError("deadlock")


def test_each_plane_waited_before_first_use_and_released_after_last():
    for u in range(3):
        steps = [st for st, pr in enumerate(K_ORDER) if 2 - prod_w(pr) == u]
        assert steps[0] in WAIT_STEPS and steps[-1] in RELEASE_STEPS
        assert not (set(steps[1:]) & set(WAIT_STEPS)) and not (set(steps[:-1]) & set(RELEASE_STEPS))
    assert sorted(K_ORDER) == list(range(6))


@pytest.mark.parametrize("n_chunks", [1, 2, 3, 8, 16])
@pytest.mark.parametrize("my_tiles", [1, 3])
def test_plane_ring_schedule(n_chunks, my_tiles):
    for seed in range(8):
        simulate(n_chunks, my_tiles, seed)
