"""Layout arithmetic of the TMA energy kernel (csrc/energy_tma.cuh), restated on the CPU: the
lane -> orbit map of a work unit covers its 512 orbits once, and each of the eighteen shared-
memory reads an orbit makes (cube q's value from the P12, P34 and P56 boxes, laid out [slowest]
[middle][fastest] = [a'][c'][b'], [b'][a'][c'], [c'][b'][a']) touches at most two addresses per
bank across a warp; the box coordinates a unit loads are the six orderings of its block triple
in each array."""
import itertools

PERMS = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]   # c_perm, slot order


def lanes(g):
    """(la, lb, lc) of the 32 lanes of orbit warp g (kernel: la = w + 4 (g % 2), lb = u,
    lc = (u + w + g / 2) % 8 with u = lane % 8, w = lane / 8)."""
    return [((lane >> 3) + 4 * (g & 1), lane & 7, ((lane & 7) + (lane >> 3) + (g >> 1)) & 7) for lane in range(32)]


def box_offset(arr, x, y, z):
    """element of cube-local (x, y, z) = (a', b', c') in the box of array arr"""
    return [(x * 8 + z) * 8 + y, (y * 8 + x) * 8 + z, (z * 8 + y) * 8 + x][arr]


def test_orbit_warps_cover_the_unit_once():
    orbits = [o for g in range(16) for o in lanes(g)]
    assert len(orbits) == 512 and len(set(orbits)) == 512
    assert all(0 <= c < 8 for o in orbits for c in o)


def test_every_read_is_at_most_two_way_per_bank():
    for g in range(16):
        L = lanes(g)
        for q, P in enumerate(PERMS):
            for arr in range(3):
                banks = {}
                for loc in L:
                    x, y, z = loc[P[0]], loc[P[1]], loc[P[2]]
                    addr = (arr * 6 + q) * 512 + box_offset(arr, x, y, z)
                    banks.setdefault(addr % 32, set()).add(addr)
                assert max(len(a) for a in banks.values()) <= 2, (g, q, arr)


def test_boxes_are_the_orderings_of_the_block_triple():
    """Box b = (pass, q) loads blocks (q2, q1, q0) as (fastest, middle, slowest): for P12[a][c][b]
    (P[0], P[2], P[1]) as (slowest, middle, fastest), P34[b][a][c] (P[1], P[0], P[2]),
    P56[c][b][a] (P[2], P[1], P[0]).  Over the six cubes each array's boxes are the six orderings
    of the unit's three blocks."""
    X, Y, Z = 3, 5, 9
    blk = (X, Y, Z)
    for pas in range(3):
        seen = set()
        for P in PERMS:
            q0 = (P[0], P[1], P[2])[pas]
            q1 = (P[2], P[0], P[1])[pas]
            q2 = (P[1], P[2], P[0])[pas]
            seen.add((blk[q0], blk[q1], blk[q2]))
        assert seen == set(itertools.permutations(blk))
