"""Host logic of the Cholesky-direct mode (ccsdt_debug_slab_schedule; no GPU): the triplet order
by blocks of occupied indices and the least-recently-used slab cache.  Every batch must find all
of its slabs resident, and the number of slabs formed must fall as the cache grows."""
import numpy as np
import pytest


def _triplets(o):
    return np.array([(i, j, k) for i in range(o) for j in range(i, o) for k in range(j, o)], dtype=np.int32)


def test_order_is_a_permutation_by_occupied_blocks(built):
    from exachem_gb300.ccsd_t import slab_schedule
    o, C = 11, 6
    tri = _triplets(o)
    order, builds = slab_schedule(o, C, 2, tri)
    assert sorted(order.tolist()) == list(range(len(tri)))
    b = C // 3
    keys = [(tri[t, 0] // b, tri[t, 1] // b, tri[t, 2] // b, *tri[t]) for t in order]
    assert keys == sorted(keys)


@pytest.mark.parametrize("o", [7, 16])
def test_cache_forms_each_slab_once_when_it_holds_all(built, o):
    from exachem_gb300.ccsd_t import slab_schedule
    tri = _triplets(o)
    for batch in (1, 4):
        _, builds = slab_schedule(o, max(o, 3 * batch), batch, tri)
        assert builds == o


def test_builds_fall_as_the_cache_grows(built):
    from exachem_gb300.ccsd_t import slab_schedule
    o = 24
    tri = _triplets(o)
    counts = [slab_schedule(o, C, 1, tri)[1] for C in (3, 6, 12, 24)]
    assert counts[-1] == o
    assert all(a >= b for a, b in zip(counts, counts[1:])), counts
    # blocks of C / 3: roughly o (o / b)^2 / 6 formations, far below one per triplet
    assert counts[0] < len(tri) and counts[1] < 0.5 * len(tri)


def test_schedule_rejects_batches_larger_than_the_cache(built):
    from exachem_gb300.ccsd_t import CCSDTError, slab_schedule
    tri = _triplets(6)
    with pytest.raises(CCSDTError):
        slab_schedule(6, 6, 3, tri)            # 3 triplets may need 9 slabs
    with pytest.raises(CCSDTError):
        slab_schedule(6, 2, 1, tri)
    bad = tri.copy()
    bad[0] = (2, 1, 3)
    with pytest.raises(CCSDTError):
        slab_schedule(6, 6, 1, bad)
