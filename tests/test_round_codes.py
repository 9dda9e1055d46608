"""Host model of the peel's 4-bit round codes (csrc/peel.cu: code_mark,
code_round, mark_prev_dead and the level changes' marks).

The listed peel classifies a triangle's partner edges from a code per edge
instead of the edge's sub-round stamp: 0xF never marked, y & 3 marked for
sub-round y, bit 3 set once peeled.  A code is written when its edge is
marked (the stamp y is written at the same moment), edges marked without an
item (no triangle left) are dead at once, and the items of sub-round r-1 turn
dead at some point during sub-round r, concurrently with its reads.  This
model replays random peel schedules with those rules, reads the codes at
random moments of each sub-round (before or after each dead mark of the
previous round), and checks that every read classifies the edge exactly as
its true stamp does: alive, peeling now, marked for the next sub-round, or
peeled before.  The GPU tests check the kernel itself against the oracle.
"""
import random

ALIVE, DEAD = 0xF, 0x8


def code_round(c, r):
    """The classification code_round() returns: -1 alive, r, r + 1, -2 dead."""
    if c == ALIVE:
        return -1
    if c == (r & 3):
        return r
    if c == ((r + 1) & 3):
        return r + 1
    return -2


def truth(stamp, r):
    if stamp == -1:
        return -1
    if stamp in (r, r + 1):
        return stamp
    assert stamp < r
    return -2


def run_schedule(seed, n_edges=64, n_rounds=40):
    rng = random.Random(seed)
    stamp = [-1] * n_edges
    code = [ALIVE] * n_edges
    items = {}  # sub-round -> edges queued with an item
    itemless = set()  # edges that never appear in a list as a live partner
    # sub-round 0's frontier, marked by a level change before it starts
    front = rng.sample(range(n_edges), 4)
    for e in front:
        with_item = rng.random() < 0.8
        stamp[e] = 0
        code[e] = 0 if with_item else DEAD
        if not with_item:
            itemless.add(e)
    items[0] = [e for e in front if e not in itemless]
    checks = 0
    for r in range(n_rounds):
        # sub-round r: the dead marks of round r-1's items interleave with reads
        pending = list(items.get(r - 1, []))
        rng.shuffle(pending)
        alive = [e for e in range(n_edges) if stamp[e] == -1]
        newly = rng.sample(alive, min(len(alive), rng.randint(0, 4)))
        events = [("dead", e) for e in pending] + [("mark", e) for e in newly] + [("read", None)] * 12
        rng.shuffle(events)
        items[r + 1] = []
        for kind, e in events:
            if kind == "dead":
                code[e] |= DEAD
            elif kind == "mark":
                with_item = rng.random() < 0.8
                stamp[e] = r + 1
                code[e] = ((r + 1) & 3) if with_item else DEAD
                if with_item:
                    items[r + 1].append(e)
                else:
                    itemless.add(e)
            else:
                for x in range(n_edges):
                    if x in itemless:
                        continue  # never read as a live partner (its triangles are gone)
                    got, want = code_round(code[x], r), truth(stamp[x], r)
                    # an edge marked during r reads as alive until its mark lands
                    assert got == want, (seed, r, x, stamp[x], code[x], got, want)
                    checks += 1
        if not any(stamp[e] == -1 for e in range(n_edges)) and not items.get(r + 1):
            break
    return checks


def test_round_codes_classify_like_the_stamps():
    total = sum(run_schedule(seed) for seed in range(300))
    assert total > 100000


def test_dead_mark_is_needed_two_rounds_later():
    # an item of round r-1 still coded (r-1) & 3 reads dead in r and r+1 ...
    r = 9
    c = (r - 1) & 3
    assert code_round(c, r) == -2 and code_round(c, r + 1) == -2
    # ... but as "marked for the next sub-round" in r+2: the dead mark must
    # land during round r (it does: every round ends with a grid barrier)
    assert code_round(c, r + 2) == r + 3
    assert code_round(c | DEAD, r + 2) == -2
