"""Multi-GPU form of the path: independent replicas, no data-path collective.

bench.py --gpus N runs one process per GPU, each advancing its own scenario
(its own seed), and reduces once after the timed region: the slowest rank's
time and the sum of particle-steps.  Here the same code runs as two `gloo`
ranks on the CPU, each replica stepped by the CPU restatement.
"""
import os
import socket
import subprocess
import sys

import pytest

from conftest import ORACLE, PKG, ROOT

WORKER = r'''
import os, sys, json
sys.path[:0] = [{pkg!r}, {oracle!r}, {root!r}]
import torch.distributed as dist
import bench
from bmc import scenarios
import oracle

rank, world = int(os.environ["RANK"]), int(os.environ["WORLD_SIZE"])
dist.init_process_group("gloo", init_method="tcp://127.0.0.1:{port}", rank=rank, world_size=world)
seed = bench.replica_seed(world, rank)
scen = scenarios.small_ring(3000 + 1000 * rank, seed=seed, feeds=True)
o = oracle.Oracle(scen)
o.init_particles()
steps = 5
o.run(steps)
psteps = float(scen.n_particles * steps)
t, total = bench.aggregate_replicas(dist, 1.0 + rank, psteps, device="cpu")
dist.barrier()
print(json.dumps({{"rank": rank, "seed": seed, "t": t, "total": total, "local": psteps}}))
dist.destroy_process_group()
'''


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_replicas_aggregate(tmp_path):
    pytest.importorskip("torch.distributed")
    import json

    code = WORKER.format(pkg=PKG, oracle=ORACLE, root=ROOT, port=free_port())
    script = tmp_path / "replica.py"
    script.write_text(code)
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1")
        procs.append(subprocess.Popen([sys.executable, str(script)], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=300)
        assert p.returncode == 0, err[-2000:]
        outs.append(json.loads(out.strip().splitlines()[-1]))
    seeds = {o["seed"] for o in outs}
    assert len(seeds) == 2 and None not in seeds          # each replica its own scenario
    for o in outs:
        assert o["t"] == 2.0                                # slowest rank's time
        assert o["total"] == 3000 * 5 + 4000 * 5            # particle-steps of all ranks


def test_single_replica_keeps_workload_seed():
    import bench

    assert bench.replica_seed(1, 0) is None
    assert bench.aggregate_replicas(None, 3.0, 7.0) == (3.0, 7.0)


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0"], env=env, capture_output=True, text=True,
                       timeout=300, cwd=ROOT)
    assert r.returncode == 0 and r.stdout.strip() == ""
