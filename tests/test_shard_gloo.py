"""One answer from a query partitioned by rows over two ranks (gloo, world size 2, on CPU): each
rank computes the partial state of its row range (the oracle stands in for the GPU here), the
states are gathered to rank 0 and folded in rank order (reffine_gb300.shard), and the folded
answer equals the single-rank answer on the whole table: integers exactly, FP64 within 1e-12.

Covers the partition plans of the four benchmark shapes: filter + sum and the 6-group group-by
(row ranges; the group-by's AVG columns evaluated on the folded state), the join (build side
replicated on every rank, probe rows by range) and the hash group-by (row ranges; partial
key-sorted tables folded by key)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASES = ["filter_sum", "groupby", "join", "hashgroup"]


def _port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _workload(name):
    from reffine_gb300 import workloads as W
    if name == "filter_sum":
        t = W.filter_sum_table(200_003, seed=51)
        return W.filter_sum_query(t.get_data_type()), [t]
    if name == "groupby":
        t = W.groupby_table(200_003, seed=52)
        return W.groupby_query(t.get_data_type()), [t]
    if name == "join":
        b, p = W.join_tables(5_000, 200_003, seed=53)
        return W.join_query(b.get_data_type(), p.get_data_type()), [b, p]
    t = W.hashgroup_table(200_003, 30_000, 1.1, seed=54)
    return W.hashgroup_query(t.get_data_type()), [t]


def _ree_result(t):
    """The grouped query on the reference's form (keys sorted and run-end encoded), by the oracle."""
    from oracle import loopgen
    from reffine_gb300 import workloads as W
    ree = W.ree_sorted(t)
    return loopgen.Query(W.hashgroup_query(ree.get_data_type()))(ree)


def _rank_main(rank, world, port, name, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as td
    from oracle import loopgen
    from reffine_gb300 import shard
    td.init_process_group("gloo", rank=rank, world_size=world)
    try:
        fn, tabs = _workload(name)
        drive = tabs[-1]
        lo, hi = shard.row_range(len(drive), rank, world)
        mine = tabs[:-1] + [drive.rows(lo, hi)]  # a join's build side is replicated
        if name == "hashgroup":
            part = _ree_result(mine[0])
            part = {"cols": part["cols"], "len": part["len"]}
        else:
            state_fn, _ = shard.split_reduce(fn)
            part = loopgen.Query(state_fn)(*mine)
        parts = [None] * world if rank == 0 else None
        td.gather_object(part, parts, dst=0)
        if rank == 0:
            if name == "hashgroup":
                got = shard.fold_tables(parts, ["sum", "sum"])
            else:
                _, finish = shard.split_reduce(fn)
                got = finish(shard.fold_states(parts, shard.leaf_ops(fn)))
            q.put((name, got))
    finally:
        td.destroy_process_group()


@pytest.mark.parametrize("name", CASES)
def test_two_rank_fold_equals_one_rank_answer(name):
    torch = pytest.importorskip("torch")
    sys.path.insert(0, ROOT)
    from oracle import loopgen
    from parity import assert_same, assert_table_same
    fn, tabs = _workload(name)
    ref = _ree_result(tabs[0]) if name == "hashgroup" else loopgen.Query(fn)(*tabs)
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _port()
    ps = [mp.Process(target=_rank_main, args=(r, 2, port, name, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = q.get(timeout=300)
    for p in ps:
        p.join(120)
    assert all(p.exitcode == 0 for p in ps)
    assert got[0] == name
    if name == "hashgroup":
        assert_table_same(got[1], ref)
    else:
        assert_same(got[1], ref)


def test_row_ranges_cover_the_table_once():
    from reffine_gb300.shard import row_range
    for n in (0, 1, 7, 100, 100_003):
        for world in (1, 2, 3, 8):
            rs = [row_range(n, r, world) for r in range(world)]
            assert rs[0][0] == 0 and rs[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(rs, rs[1:]))
            assert max(h - l for l, h in rs) - min(h - l for l, h in rs) <= 1
