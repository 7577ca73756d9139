"""Replicas-only multi-GPU logic on the host: two gloo ranks on the CPU."""
import os
import socket

import numpy as np
import pytest


def test_read_ranges_partition_the_reads():
    from pysa_gb300.shard import read_range
    for reads in (0, 1, 7, 100, 257):
        for world in (1, 2, 3, 8):
            got = [read_range(reads, r, world) for r in range(world)]
            assert got[0][0] == 0 and got[-1][1] == reads
            assert all(a[1] == b[0] for a, b in zip(got, got[1:]))
            sizes = [b - a for a, b in got]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        read_range(4, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist
    from pysa_gb300.ais import combine_logZf
    from pysa_gb300.shard import (combined_logz, gather_rows, read_range,
                                  slowest)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    start, stop = read_range(11, rank, world)
    # stand-in result rows: what a rank's Solver run returns per read
    rows = [{"read": k, "best_energy": -float(k), "log_Zf": 0.1 * k}
            for k in range(start, stop)]
    allrows = gather_rows(rows)
    t = slowest(1.0 + rank)
    lz = combined_logz(allrows)
    want = combine_logZf({"log_Zf": np.arange(11) * 0.1})
    ok = ([r["read"] for r in allrows] == list(range(11)) and t == world
          and abs(lz - want) < 1e-12)
    with open(os.path.join(out_dir, f"r{rank}"), "w") as f:
        f.write("ok" if ok else f"bad {allrows} {t} {lz} {want}")
    dist.destroy_process_group()


def test_two_gloo_ranks_gather_rows_time_and_logz(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2,
                       start_method="spawn", join=True)
    for r in range(2):
        assert (tmp_path / f"r{r}").read_text() == "ok"
