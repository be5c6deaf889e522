"""The N-GPU form of bench.py is replicas only (every rank renders its own copy
of the frame; nothing is exchanged on the data path). Its host logic runs here
as two gloo ranks on the CPU: the process group comes up from the torchrun
environment, the ranks meet at the barriers around the timed region, the
reported time is the slowest rank's, and the reference arm does its work on
rank 0 only."""
import multiprocessing as mp
import os
import socket


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, port: int, out) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(rank),
                      LOCAL_RANK=str(rank))
    import time

    import bench

    world, r, local = bench.dist_setup(None)
    bench.barrier(world)
    time.sleep(0.05 * (r + 1))  # rank 1 is the slower one
    slowest = bench.max_over_ranks(10.0 + r, world)
    bench.barrier(world)
    t0 = time.perf_counter()
    bench.run_reference(None, world, r) if r == 1 else None  # rank 1 of the reference arm does no work
    idle_s = time.perf_counter() - t0
    import torch.distributed as dist

    dist.destroy_process_group()
    out.put((r, world, local, slowest, idle_s))


def test_two_replica_ranks_time_the_slowest_and_rank0_reports():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        res = sorted(out.get(timeout=180) for _ in range(2))
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert [x[0] for x in res] == [0, 1]
    assert all(x[1] == 2 and x[2] == x[0] for x in res)
    assert all(x[3] == 11.0 for x in res)  # both ranks report the slowest rank's time
    assert res[1][4] < 1.0  # the reference arm's rank 1 returns at once
    assert all(p.exitcode == 0 for p in procs)



def test_profiled_traffic_keys():
    """The bench's traffic figures come from the committed extend summary: one
    pair of keys for frames on the fast tree and one for the reference's tree,
    each read from its own line (one key is a suffix of the other)."""
    import bench

    fast = bench.profiled_traffic("dram_bytes_per_extension_ray")
    ref = bench.profiled_traffic("reference_tree_dram_bytes_per_extension_ray")
    l2_fast = bench.profiled_traffic("l2_bytes_per_extension_ray")
    l2_ref = bench.profiled_traffic("reference_tree_l2_bytes_per_extension_ray")
    assert None not in (fast, ref, l2_fast, l2_ref)
    assert 0 < fast < ref and 0 < l2_fast < l2_ref
    assert fast < l2_fast and ref < l2_ref
