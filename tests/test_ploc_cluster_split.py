"""The slice arithmetic of the cluster PLOC kernel (k_ploc_cluster) on the
CPU: for every live-cluster count it accepts and both cluster sizes, every
slice fits one CTA's window, every active slice is non-empty, and each
slice's +-2r halo (r <= 32) lies inside its two neighbours' slices, as the
kernel's shared-memory indexing assumes.  The constants are read from the
source so the check follows them."""
import os
import re

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "obvhs_gb300", "csrc", "ploc.cu")


def _const(src, name):
    m = re.search(r"constexpr\s+\w+\s+" + name + r"\s*=\s*([0-9]+)", src)
    assert m, name
    return int(m.group(1))


def _split(count, ncta, min_slice):
    active = min(ncta, max(1, count // min_slice))
    return active, (count + active - 1) // active


def test_slices_and_halos_fit():
    src = open(CSRC).read()
    cap, halo, min_slice = _const(src, "CL_CAP"), _const(src, "CL_HALO"), _const(src, "CL_MIN_SLICE")
    stride = cap + 2 * halo
    assert min_slice >= halo and halo >= 2 * 32
    for ncta in (8, 16):
        counts = list(range(1, 4 * min_slice * ncta)) + list(range(4 * min_slice * ncta, cap * ncta + 1, 97))
        counts.append(cap * ncta)
        for count in counts:
            act, sl = _split(count, ncta, min_slice)
            assert 1 <= act <= ncta and sl <= cap
            lens = [min(sl, count - me * sl) if me < act else 0 for me in range(ncta)]
            assert sum(lens) == count and all(n > 0 for n in lens[:act])
            if act > 1:
                # halos of up to 2r = halo clusters come from one neighbour
                assert min(lens[:act]) >= halo
            for me in range(act):
                base, n = me * sl, lens[me]
                # window positions of the slice and its halos
                assert halo - min(base, halo) >= 0 and halo + n + halo <= stride
            # the next pass's owner of every emitted index exists
            for total in {1, max(1, count // 2), count}:
                a2, s2 = _split(total, ncta, min_slice)
                assert (total - 1) // s2 < a2 and s2 <= cap


def test_hand_off_to_the_single_cta_tail_fits_it():
    """The cluster kernel writes its slices back and hands the last passes to
    the single-CTA tail at CL_TAIL_AT live clusters: the tail's shared memory
    holds TAIL_MAX clusters, and the written slices cover [0, count) exactly
    (each CTA writes min(slice, count - base) clusters at base)."""
    src = open(CSRC).read()
    hdr = open(os.path.join(os.path.dirname(CSRC), "build.h")).read()
    tail_at = _const(src, "CL_TAIL_AT")
    tail_max = _const(hdr, "TAIL_MAX")
    min_slice = _const(src, "CL_MIN_SLICE")
    assert 1 < tail_at <= tail_max
    for ncta in (8, 16):
        for count in range(2, tail_at + 1):
            act, sl = _split(count, ncta, min_slice)
            covered = []
            for me in range(ncta):
                base = me * sl
                n = min(sl, count - base) if me < act else 0
                covered.extend(range(base, base + n))
            assert covered == list(range(count))
