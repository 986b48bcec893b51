"""The conflict-resolution rounds of the reinsertion kernel (k_resolve) on the
CPU, against the reference's sequential apply loop
(src/bvh2/reinsertion.rs:176-208): proposals in priority order, each
accepted when none of its five conflict nodes was touched by an accepted
earlier one.

Both forms of the kernel's rounds are modelled: the global form (claims of
round r in owner array r % 3, the next round's array reset by the claims) and
the shared-memory form (one claim word per conflict node: a check, a reset of
the unresolved proposals' claims, a claim).  Inside a round the kernel's
threads run in no fixed order, and an accept's touched flags may or may not be
seen by other proposals in the same round; the models visit proposals in a
random order and make every touch visible at once, which covers both.  The
accepted sets must equal the sequential loop's on every input, including
heavy conflicts and conflict sets that repeat a node."""
import numpy as np


def sequential(confs, keys):
    touched, acc = set(), set()
    for j in sorted(range(len(keys)), key=lambda q: keys[q]):
        if any(c in touched for c in confs[j]):
            continue
        touched.update(confs[j])
        acc.add(j)
    return acc


def rounds_shared(confs, keys, rng):
    P = len(keys)
    st = [0] * P
    own, touched = {}, set()
    for rnd in range(P + 3):
        for j in rng.permutation(P):
            if st[j]:
                continue
            if any(c in touched for c in confs[j]):
                st[j] = 2
            elif rnd > 0 and all(own.get(c) == keys[j] for c in confs[j]):
                st[j] = 1
                touched.update(confs[j])
        for j in range(P):
            if st[j] == 0:
                for c in confs[j]:
                    own[c] = None
        rem = 0
        for j in rng.permutation(P):
            if st[j] == 0:
                for c in confs[j]:
                    if own.get(c) is None or keys[j] < own[c]:
                        own[c] = keys[j]
                rem += 1
        if rem == 0:
            return {j for j in range(P) if st[j] == 1}
    raise AssertionError("rounds did not end")


def rounds_global(confs, keys, rng):
    P = len(keys)
    st = [0] * P
    owner = [{}, {}, {}]
    touched = set()
    # the searches reset the round-0 claim words of every listed proposal
    for j in range(P):
        for c in confs[j]:
            owner[0][c] = None
    for rnd in range(P + 3):
        prev, cur, nxt = owner[(rnd + 2) % 3], owner[rnd % 3], owner[(rnd + 1) % 3]
        rem = 0
        for j in rng.permutation(P):
            if st[j]:
                continue
            if any(c in touched for c in confs[j]):
                st[j] = 2
                continue
            if rnd > 0 and all(prev.get(c) == keys[j] for c in confs[j]):
                st[j] = 1
                touched.update(confs[j])
                continue
            for c in confs[j]:
                if cur.get(c) is None or keys[j] < cur[c]:
                    cur[c] = keys[j]
                nxt[c] = None
            rem += 1
        if rem == 0:
            return {j for j in range(P) if st[j] == 1}
    raise AssertionError("rounds did not end")


def _case(rng, P, nodes):
    confs = [tuple(int(x) for x in rng.integers(0, nodes, size=5)) for _ in range(P)]
    # priority keys: area gain descending then candidate rank (unique)
    gains = rng.integers(0, 4, size=P)  # many equal gains
    keys = [((3 - int(g)) << 32) | k for k, g in enumerate(gains)]
    return confs, keys


def test_rounds_accept_the_sequential_set():
    rng = np.random.default_rng(1234)
    for trial in range(400):
        P = int(rng.integers(0, 60))
        nodes = int(rng.integers(3, 80))  # few nodes: dense conflicts
        confs, keys = _case(rng, P, nodes)
        want = sequential(confs, keys)
        assert rounds_shared(confs, keys, rng) == want, trial
        assert rounds_global(confs, keys, rng) == want, trial


def test_rounds_on_chains_of_conflicts():
    """Proposal k conflicts with k + 1 only (a chain): the sequential loop
    accepts every other one in priority order; the rounds resolve the chain
    from its head."""
    rng = np.random.default_rng(7)
    for P in (1, 2, 5, 33, 100):
        confs = [(k, k + 1, 10_000 + k, 20_000 + k, 30_000 + k) for k in range(P)]
        for order in (list(range(P)), list(reversed(range(P))), list(rng.permutation(P))):
            keys = [0] * P
            for rank, j in enumerate(order):
                keys[j] = rank
            want = sequential(confs, keys)
            assert rounds_shared(confs, keys, rng) == want
            assert rounds_global(confs, keys, rng) == want
