"""The multi-GPU path runs independent work per rank with no data-path
collective: replicas of one grid (each rank runs the whole hot path on its
own GPU), or a batch of charts split between the ranks, whose per-chart
results rank 0 gathers.  What crosses ranks is the timing (a barrier around
the timed region and the slowest rank's time, from which rank 0 reports the
whole job's throughput) and, for charts, one gather of their results.  This
checks that host logic with two `gloo` ranks on the CPU, each running its
share through the oracle."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, out_dir):
    import time
    import torch.distributed as dist
    sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle"),
                    os.path.join(ROOT, "surface-remesher_gb300", "python")]
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank,
                           world_size=ws)
    import bench
    import oracle
    from workloads import small_case
    assert bench.dist_env() == (ws, rank, rank)
    sites, _, _ = small_case(256, 200 + 100 * rank, seed=30 + rank)
    dist.barrier()
    t0 = time.perf_counter()
    labels = oracle.pba_label(sites)
    t = time.perf_counter() - t0 + 0.05 * rank  # rank 1 is the slow one
    dist.barrier()
    slowest, tag = bench.max_over_ranks([t, rank], ws)
    seen = [None] * ws
    dist.all_gather_object(seen, t)
    rate = bench.job_rate(256 * 256, 1, ws, slowest)
    # the reference arm: rank 0 alone runs it; the others return at once
    if rank != 0:
        assert bench.run_reference(None) == 0
    np.savez(os.path.join(out_dir, "rank%d.npz" % rank), slowest=slowest, tag=tag,
             seen=np.array(seen), rate=rate, labels_ok=bool((labels[..., 0] >= 0).all()))
    dist.destroy_process_group()


def test_two_gloo_replicas_report_the_slowest_rank(tmp_path):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ws = 2
    mp.start_processes(_rank_main, args=(ws, _free_port(), str(tmp_path)), nprocs=ws,
                       join=True, start_method="spawn")
    r = [np.load(os.path.join(tmp_path, "rank%d.npz" % k)) for k in range(ws)]
    assert all(bool(x["labels_ok"]) for x in r)
    for x in r:
        assert float(x["slowest"]) == max(r[0]["seen"]) == max(r[1]["seen"])
        assert float(x["tag"]) == ws - 1
        assert np.isclose(float(x["rate"]), 256 * 256 * ws / float(x["slowest"]) / 1e9)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks([1.5, 2], 1) == [1.5, 2.0]
    assert bench.job_rate(10 ** 9, 2, 1, 4.0) == 0.5


def _charts():
    from workloads import small_case
    out = []
    for i, (n, m) in enumerate(((256, 300), (256, 150), (512, 900), (256, 500), (512, 400))):
        out.append(small_case(n, m, seed=60 + i))
    return out


def _chart_result(oracle, sites, rho, mask):
    labels, st = oracle.gcvt(sites, rho, mask, 1, 6, mode=oracle.EXACT, fixed_iters=6)
    return {"n": int(sites.shape[0]), "iterations": int(st["iterations"]),
            "energy": float(st["last_energy"]),
            "labels": int(np.frombuffer(labels.tobytes(), np.uint32).astype(np.uint64).sum())}


def _shard_main(rank, ws, port, out_dir):
    import torch.distributed as dist
    sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle"),
                    os.path.join(ROOT, "surface-remesher_gb300", "python")]
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank,
                            world_size=ws)
    import bench
    import oracle
    charts = _charts()
    weights = [int(c[0].shape[0]) ** 2 for c in charts]
    mine = bench.shard_charts(weights, ws, rank)
    res = [_chart_result(oracle, *charts[i]) for i in mine]
    got = bench.gather_charts(res, mine, ws, len(charts))
    if rank == 0:
        np.save(os.path.join(out_dir, "gathered.npy"), np.array(got, dtype=object),
                allow_pickle=True)
    else:
        assert got is None
    dist.destroy_process_group()


def test_charts_shard_across_two_gloo_ranks(tmp_path):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle"),
                    os.path.join(ROOT, "surface-remesher_gb300", "python")]
    import bench
    import oracle
    charts = _charts()
    weights = [int(c[0].shape[0]) ** 2 for c in charts]
    # every chart on exactly one rank, the heavy ones spread
    parts = [bench.shard_charts(weights, 2, r) for r in range(2)]
    assert sorted(parts[0] + parts[1]) == list(range(len(charts)))
    loads = [sum(weights[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(weights)
    assert bench.shard_charts(weights, 1, 0) == list(range(len(charts)))
    ws = 2
    mp.start_processes(_shard_main, args=(ws, _free_port(), str(tmp_path)), nprocs=ws,
                       join=True, start_method="spawn")
    got = list(np.load(os.path.join(tmp_path, "gathered.npy"), allow_pickle=True))
    want = [_chart_result(oracle, *c) for c in charts]
    assert got == want
