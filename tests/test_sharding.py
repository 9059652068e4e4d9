"""Event sharding across ranks (the multi-GPU partitioning), tested on the
CPU with two gloo ranks: each rank samples a disjoint event range with the
oracle's replay of the GPU streams (gpu_event_offset semantics); the hadron
lists gathered on rank 0 equal the single-rank run bit for bit.  No
collective touches the data path; the gather only assembles the result."""
import os
import socket

import numpy as np
import torch.distributed as dist
import torch.multiprocessing as mp

import oracle_lib as O
from iss_gb300 import surfaces as S

N_EVENTS = 12


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _sample(event_offset, n_events):
    g = O.load_golden("yields_viscous_14moment.npz")
    lrf = g["lrf"]
    y = g["yields"].astype(np.float32)
    cdf, tot = O.cdf(y)
    oc = O.OracleConfig(g["params"], S.TABLE_DIR, n_events=n_events, seed=77,
                        event_offset=event_offset)
    cnt = O.counts(oc, g["species"], tot)
    coef = O.cell_coeffs(oc, lrf).astype(np.float32)
    had, _ = O.sample_replay(oc, g["species"], lrf, coef, cdf, cnt)
    return had


def _rank(rank, world, port, out_path):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    per = N_EVENTS // world
    mine = _sample(rank * per, per)
    gathered = [None] * world
    dist.all_gather_object(gathered, mine.tobytes())
    if rank == 0:
        with open(out_path, "wb") as f:
            f.write(b"".join(gathered))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_event_shards_reproduce_single_rank(tmp_path):
    out = tmp_path / "gathered.bin"
    port = _free_port()
    mp.start_processes(_rank, args=(2, port, str(out)), nprocs=2, join=True, start_method="spawn")
    single = _sample(0, N_EVENTS)
    assert out.read_bytes() == single.tobytes()
    assert len(single) > 0
