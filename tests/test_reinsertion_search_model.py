"""The reinsertion search's push rule (FindSearch in
obvhs_gb300/csrc/reinsertion.cu) against find_reinsertion as the reference
runs it (src/bvh2/reinsertion.rs:233-334), on the CPU.

The kernel does not push two children whose bound already fails (the
reference pushes them and pops and prunes both at once), unless a push would
be lost to the clamped stack (StackStack: a push onto a full stack writes a
slot no pop reads) or would overflow the bound; then it pushes as the
reference does.  The two searches are run on random trees with tiny stacks,
so that the clamp and the overflow are reached often, in both stack modes;
they must find the same target and gain and overflow alike.  (Keeping the top
two entries in registers and loading children's records early change no
result: the logical stack is the same.)"""
import numpy as np

F = np.float32


def half_area(b):
    d = b[3:] - b[:3]
    return F(F(F(d[0] + d[1]) * d[2]) + F(d[0] * d[1]))


def union(a, b):
    return np.concatenate([np.minimum(a[:3], b[:3]), np.maximum(a[3:], b[3:])]).astype(F)


def sibling(i):
    return i + 1 if i & 1 else i - 1


def random_tree(rng, m):
    """A BVH2 in the reference's layout: root 0, children pairs (first,
    first + 1) with first odd; leaves with random boxes, inner boxes the
    unions."""
    boxes, first, parents = {}, {}, {}
    nxt = [1]

    def build(node, leaves):
        if len(leaves) == 1:
            c = rng.uniform(-10, 10, 3).astype(F)
            e = rng.uniform(0.01, 2.0, 3).astype(F)
            boxes[node] = np.concatenate([c, c + e]).astype(F)
            first[node] = None
            return
        k = int(rng.integers(1, len(leaves)))
        f = nxt[0]
        nxt[0] += 2
        first[node] = f
        parents[f] = parents[f + 1] = node
        build(f, leaves[:k])
        build(f + 1, leaves[k:])
        boxes[node] = union(boxes[f], boxes[f + 1])

    parents[0] = 0
    build(0, list(range(m)))
    return boxes, first, parents


def search(tree, node, room, error_mode, skip):
    """find_reinsertion with a stack that accepts `room` entries (clamped:
    further pushes are lost; error_mode: a push beyond them overflows).
    skip: the kernel's rule for children whose bound fails at the push."""
    boxes, first, parents = tree
    st = []
    overflow = False
    lost = 0

    def push(a, i):
        nonlocal overflow, lost
        if len(st) >= room:
            if error_mode:
                overflow = True
            lost += 1
            return
        st.append((a, i))

    box = boxes[node]
    node_area = half_area(box)
    parent = parents[node]
    area_diff = half_area(boxes[parent])
    sib = sibling(node)
    pivot_bbox = boxes[sib]
    pivot = parent
    best_to, best_diff = 0, F(0)
    push(area_diff, sib)
    while True:
        while st and not overflow:
            a, i = st.pop()
            if F(a - node_area) <= best_diff:
                continue
            reinsert = F(a - half_area(union(boxes[i], box)))
            if reinsert > best_diff:
                best_to, best_diff = i, reinsert
            if first[i] is not None:
                child = F(reinsert + half_area(boxes[i]))
                if skip and F(child - node_area) <= best_diff and len(st) + 2 <= room:
                    continue
                push(child, first[i])
                push(child, first[i] + 1)
        if overflow:
            return (0, F(0), True), lost
        if pivot != parent:
            pivot_bbox = union(pivot_bbox, boxes[sib])
            area_diff = F(area_diff + F(half_area(boxes[pivot]) - half_area(pivot_bbox)))
        up = parents[pivot]
        if up == pivot:
            break
        sib = sibling(pivot)
        pivot = up
        push(area_diff, sib)
    if best_to == sibling(node) or best_to == parents[node]:
        best_to, best_diff = 0, F(0)
    return (best_to, best_diff, False), lost


def test_skipped_pushes_change_no_search():
    rng = np.random.default_rng(99)
    compared = overflows = clamped = 0
    for trial in range(24):
        tree = random_tree(rng, int(rng.integers(2, 64)))
        nodes = sorted(tree[0])[1:]
        pick = rng.choice(nodes, size=min(len(nodes), 24), replace=False)
        for room in (1, 2, 3, 4, 6, 9, 191):
            for error_mode in (False, True):
                for node in pick:
                    ref, lost = search(tree, int(node), room, error_mode, skip=False)
                    got, _ = search(tree, int(node), room, error_mode, skip=True)
                    assert got == ref, (trial, room, error_mode, int(node))
                    compared += 1
                    overflows += ref[2]
                    clamped += lost > 0 and not error_mode
    # both limits were reached many times
    assert compared > 4000 and overflows > 100 and clamped > 100, (compared, overflows, clamped)
