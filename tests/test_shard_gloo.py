"""Multi-rank path on CPU: two gloo ranks split the occupied triplets with the library's own
ccsdt_shard_triplets (host-only), evaluate their shard with the oracle, and sum the partial
energies with an all_reduce - the pattern of the reference's rank loop and final reduce
(ccsd_t_fused_driver.hpp:368-483, ccsd_t.cpp:262-263).  Checks that the shards are disjoint,
cover every triplet, and that the reduced energy equals the single-rank energy."""
import ctypes
import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _shard(lib, o, index, count):
    n = ctypes.c_long()
    assert lib.ccsdt_shard_triplets(o, index, count, ctypes.byref(n), None) == 0
    tri = np.zeros((n.value, 3), np.int32)
    assert lib.ccsdt_shard_triplets(o, index, count, ctypes.byref(n),
                                    tri.ctypes.data_as(ctypes.POINTER(ctypes.c_int))) == 0
    return tri


def _rank(rank, world, port, o, v, seed, q):
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    import torch
    import torch.distributed as dist
    import oracle
    from exachem_gb300.ccsd_t import load_library
    from exachem_gb300.generator import generate
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        lib = load_library()
        tri = _shard(lib, o, rank, world)
        d = generate(o, v, seed)
        e4, e5 = oracle.triplets(d, tri)
        part = torch.tensor([e4.sum(), e5.sum(), float(len(tri))], dtype=torch.float64)
        dist.all_reduce(part)
        counts = [None] * world
        dist.all_gather_object(counts, tri.tolist())
        if rank == 0:
            q.put((part.tolist(), counts))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_two_gloo_ranks_sum_to_single_rank_energy(built, world):
    import torch.multiprocessing as mp
    import oracle
    from exachem_gb300.ccsd_t import all_triplets
    from exachem_gb300.generator import generate
    o, v, seed = 7, 22, 11
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, o, v, seed, q)) for r in range(world)]
    for p in procs:
        p.start()
    try:
        (e4, e5, n), shards = q.get(timeout=240)
    finally:
        for p in procs:
            p.join(timeout=60)
    assert all(p.exitcode == 0 for p in procs)
    allt = sorted(map(tuple, all_triplets(o).tolist()))
    got = sorted(tuple(t) for s in shards for t in s)
    assert got == allt and n == len(allt)                       # disjoint and complete
    ref4, ref5 = oracle.energy(generate(o, v, seed))
    assert e4 == pytest.approx(ref4, rel=1e-12, abs=0)
    assert e5 == pytest.approx(ref5, rel=1e-12, abs=0)


def test_shard_listing_matches_lexicographic_round_robin(built):
    from exachem_gb300.ccsd_t import all_triplets, load_library
    lib = load_library()
    for o, count in [(1, 1), (5, 3), (9, 4), (12, 7)]:
        allt = all_triplets(o)
        for index in range(count):
            assert np.array_equal(_shard(lib, o, index, count), allt[index::count])
    n = ctypes.c_long()
    assert lib.ccsdt_shard_triplets(5, 3, 3, ctypes.byref(n), None) != 0    # index outside [0, count)
    assert lib.ccsdt_shard_triplets(0, 0, 1, ctypes.byref(n), None) != 0
