"""Replica plumbing of bench.py under torchrun, on CPU with gloo (world size 2).

The step has no data-path exchange on one GPU per box, so N GPUs run N
independent replicas: every rank times its own copy, the timing is the
maximum over ranks (all-reduce MAX) behind a barrier, value = N x the zone
updates of one replica / that maximum, and only rank 0 prints.  The reference
arm runs on rank 0 alone; the other ranks leave without work.
"""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

CHILD = r"""
import io, json, os, sys, contextlib, types
sys.path.insert(0, {root!r})
import bench
rank, ws = bench.dist_init()
bench.barrier(ws)
# each replica reports its own time; the job time is the slowest rank's
ms = 10.0 + 5.0 * rank
ms_max = bench.allmax(ms, ws)
bench.barrier(ws)
buf = io.StringIO()
with contextlib.redirect_stdout(buf):
    bench.reference_arm(types.SimpleNamespace(ref_n=8, steps=1, warmup=0), rank, ws) if rank != 0 else None
print(json.dumps({{"rank": rank, "ws": ws, "ms_max": ms_max, "ref_out": buf.getvalue()}}))
import torch.distributed as dist
dist.destroy_process_group()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_replicas_take_the_max_over_ranks_and_only_rank0_reports():
    pytest.importorskip("torch.distributed")
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2",
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD.format(root=str(ROOT))], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=300)
        assert p.returncode == 0, err[-2000:]
        outs.append(json.loads(out.strip().splitlines()[-1]))
    assert [o["rank"] for o in outs] == [0, 1]
    assert all(o["ws"] == 2 for o in outs)
    assert all(o["ms_max"] == 15.0 for o in outs)  # the slower replica's time on every rank
    assert outs[1]["ref_out"] == ""  # the reference arm does no work off rank 0


def test_single_process_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    env = dict(os.environ)
    try:
        os.environ.pop("WORLD_SIZE", None)
        os.environ.pop("RANK", None)
        assert bench.dist_init() == (0, 1)
        assert bench.allmax(3.5, 1) == 3.5
    finally:
        os.environ.clear()
        os.environ.update(env)
