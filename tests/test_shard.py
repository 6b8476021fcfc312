"""Multi-rank sharding on the CPU (gloo, world size 2): strip-aligned
location ranges, pairs dealt largest-first, and the gather of result records
to rank 0 in location order.  Each rank correlates its share with the oracle
(no GPU here); the gathered array must equal one run over all locations,
which holds because shards never split a strip."""
import os
import socket
import tempfile

import numpy as np
import pytest
import torch.multiprocessing as mp

from xcorr_gb300 import shard


def test_strip_ranges_cover_and_align():
    for nlocs, sl, world in [(96, 8, 2), (1000, 20, 3), (7, 3, 4), (0, 5, 2), (50, 0, 3)]:
        rs = shard.strip_ranges(nlocs, sl, world)
        assert len(rs) == world and rs[0][0] == 0 and rs[-1][1] == nlocs
        for (a0, a1), (b0, b1) in zip(rs, rs[1:]):
            assert a1 == b0
        for w0, w1 in rs:
            assert sl == 0 or w0 % sl == 0 or w0 == nlocs


def test_deal_pairs_balances():
    counts = [40000, 500, 12000, 12000, 9000, 700, 30000]
    owner = shard.deal_pairs(counts, 2)
    assert sorted(i for o in owner for i in o) == list(range(len(counts)))
    loads = [sum(counts[i] for i in o) for o in owner]
    assert max(loads) - min(loads) <= max(counts) // 2


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_path):
    import torch.distributed as dist
    import golden_util as gu
    import xcorr_oracle as xo
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    g = gu.load("xs32")
    m, s, locs, d, xoff, yoff, ast = gu.case_inputs("xs32", g)
    ranges = shard.strip_ranges(len(locs), d["nxl"], world)
    w0, w1 = ranges[rank]
    p = xo.params(d["xsearch"], d["ysearch"], d["ri"], d["interp_flag"], d["ifc"])
    mine = xo.run(p, m, s, locs[w0:w1], xoff, yoff, ast, precision=xo.F32, strip_len=d["nxl"], nthreads=2)
    full = shard.gather_results(mine, ranges)
    if rank == 0:
        np.save(out_path, np.frombuffer(full.tobytes(), dtype=np.uint8))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_gather_equals_one_run():
    import golden_util as gu
    import xcorr_oracle as xo
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "full.npy")
        mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
        got = np.frombuffer(np.load(out).tobytes(), dtype=xo.RESULT_DTYPE)
    g = gu.load("xs32")
    m, s, locs, d, xoff, yoff, ast = gu.case_inputs("xs32", g)
    p = xo.params(d["xsearch"], d["ysearch"], d["ri"], d["interp_flag"], d["ifc"])
    ref = xo.run(p, m, s, locs, xoff, yoff, ast, precision=xo.F32, strip_len=d["nxl"], nthreads=2)
    assert got.tobytes() == ref.tobytes()
