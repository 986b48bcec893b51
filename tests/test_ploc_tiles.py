"""The tile arithmetic of the cooperative PLOC passes (k_ploc_coop, k_ploc_seg
with ploc_tile_offsets / ploc_tile_fused / ploc_tile_write in
obvhs_gb300/csrc/ploc.cu), on the CPU.

A pass over `count` clusters with radius r and ipt items per thread cuts the
list into tiles of chunk = PT * ipt - 2r clusters (tile_chunk).  A tile
stages the boxes of [base - 2r, base + chunk + 2r), computes the merge
offsets of [base - r, base + chunk + r) (its clusters and the r either side
whose offsets the mutual-pair test reads), and thread tid owns the items
base + tid * ipt + k, k < ipt, that lie in the tile and the list.  Checked
for every radius the builder accepts and many list lengths: each cluster is
an item of exactly one tile; the offset span is exactly PT * ipt clusters;
every box a radius search reads and every offset the mutual test reads lies
inside what the tile staged or computed, and inside the shared arrays
(BOXS boxes, PCHUNK + 64 offsets); the tile count fits the status scratch
(n / TILE_MIN tiles)."""
import numpy as np

PT, PITEMS = 256, 4
PCHUNK = PT * PITEMS
BOXS = PCHUNK + 4 * 32
MERGE_SLOTS = PCHUNK + 2 * 32
TILE_MIN = PT - 2 * 32


def tile_chunk(ipt, r):
    return PT * ipt - 2 * r


def check_pass(count, ipt, r):
    chunk = tile_chunk(ipt, r)
    ntiles = -(-count // chunk)
    assert ntiles <= -(-count // TILE_MIN)
    owner = np.zeros(count, np.int32)
    for t in range(ntiles):
        base = t * chunk
        box_lo, box_span = base - 2 * r, chunk + 4 * r
        m_lo, m_span = base - r, chunk + 2 * r
        assert m_span == PT * ipt and box_span <= BOXS and m_span <= MERGE_SLOTS
        # radius searches: cluster j of the offset span reads boxes j - r .. j + r
        j = np.arange(m_lo, m_lo + m_span)
        j = j[(j >= 0) & (j < count)]
        lo = np.maximum(j - r, 0)
        hi = np.minimum(j + r, count - 1)
        assert (lo >= box_lo).all() and (hi < box_lo + box_span).all()
        # the items of the tile's threads
        tid = np.arange(PT)[:, None]
        k = np.arange(PITEMS)[None, :]
        i = base + tid * ipt + k
        own = (k < ipt) & (i < count) & (i < base + chunk)
        items = i[own]
        np.add.at(owner, items, 1)
        # the mutual test reads the offsets of i and of its partner i + off, |off| <= r
        assert (items - r >= m_lo).all() and (items + r < m_lo + m_span).all()
    assert (owner == 1).all(), (count, ipt, r)


def test_every_cluster_in_one_tile_and_every_read_inside_the_tile():
    rng = np.random.default_rng(3)
    counts = sorted({2, 3, 5, 31, 255, 256, 257, 1000, 1023, 1024, 1025, 4096, 65537,
                     *map(int, rng.integers(2, 200_000, size=12))})
    for r in (1, 2, 7, 14, 16, 31, 32):
        for ipt in (1, 2, 4):
            for count in counts:
                check_pass(count, ipt, r)
