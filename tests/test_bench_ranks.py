"""Replica plumbing of bench.py on two CPU ranks over gloo: the process
group comes up from the launcher's environment, the barrier releases both
ranks, the step time is the maximum over ranks and the whole-job value
counts every replica; the reference arm does its work on rank 0 only."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_SCRIPT = r'''
import json, os, sys
sys.path.insert(0, sys.argv[1])
import bench
ws, rank, local = bench.dist_init(2)
bench.barrier(ws)
ms = bench.max_over_ranks(ws, 10.0 + rank)
value = bench.whole_job_value(ws, 1000, ms)
ref = bench.run_reference(None) if rank != 0 else 'skipped'
bench.barrier(ws)
import torch.distributed as dist
backend = dist.get_backend()
dist.destroy_process_group()
print(json.dumps({'rank': rank, 'ws': ws, 'ms': ms, 'value': value, 'backend': backend, 'ref': ref}))
'''


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def test_two_ranks_over_gloo():
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE='2', MASTER_ADDR='127.0.0.1',
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES='')
        procs.append(subprocess.Popen([sys.executable, '-c', RANK_SCRIPT, ROOT], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=240)
        assert p.returncode == 0, err[-2000:]
        outs.append(json.loads(out.strip().splitlines()[-1]))
    for o in outs:
        assert o['ws'] == 2 and o['backend'] == 'gloo'
        assert o['ms'] == 11.0                                  # the slower rank's time
        assert abs(o['value'] - 2 * 1000 / 0.011) < 1e-6 * o['value']
    assert outs[1]['ref'] is None and outs[0]['ref'] == 'skipped'  # rank 1 leaves the reference arm at once
