"""Clones split over processes, on the CPU with torch.distributed (gloo,
world size 2): each rank owns a contiguous block of clones, the per-clone
log-weights are all-gathered, every rank draws the same copy table (the
oracle's systematic resampling), and clbm_shard_plan drives the exchange
(send / recv between ranks, local copies within a rank) -- the reference's
MPI clone transfers (src/mpi_LBM_GK_pops_perturb.cpp:650-699).  After the
exchange every rank must hold exactly what one process gathering
states[labels[j]] would hold.  Also: the plan's host-side checks, and the
bench's multi-rank path (gloo reference arm: rank 0 alone prints)."""
import ctypes as C
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def systematic_labels(orc, logw: np.ndarray, u: float) -> np.ndarray:
    nc = logw.size
    copies = np.zeros(nc, dtype=np.int32)
    labels = np.zeros(nc, dtype=np.int32)
    table = np.zeros(2 * nc, dtype=np.int32)
    lw = np.ascontiguousarray(logw, dtype=np.float64)
    res = orc.lib().orc_clone_systematic(nc, lw.ctypes.data_as(C.c_void_p), C.c_double(u),
                                         copies.ctypes.data_as(C.c_void_p),
                                         labels.ctypes.data_as(C.c_void_p),
                                         table.ctypes.data_as(C.c_void_p))
    assert res.status == 0
    return labels


def _worker(rank, world, port, nc, n, seed, out_dir):
    for p in (REPO, REPO / "cloning-lbm-mpi_gb300", REPO / "oracle"):
        sys.path.insert(0, str(p))
    import torch
    import torch.distributed as dist
    import clbm
    import oracle
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    local = nc // world
    rng = np.random.default_rng(seed)
    every = rng.standard_normal((nc, n))          # the states of every clone (checker's copy)
    logw = rng.normal(0.0, 1.5, nc)
    mine = every[rank * local:(rank + 1) * local].copy()
    # this shard's weights only, then the all-gather
    lw = torch.from_numpy(logw[rank * local:(rank + 1) * local].copy())
    parts = [torch.empty(local, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(parts, lw)
    gathered = torch.cat(parts).numpy()
    assert np.array_equal(gathered, logw)
    labels = systematic_labels(oracle, gathered, 0.37)
    # every rank drew the same table
    lt = torch.from_numpy(labels.astype(np.int64))
    tabs = [torch.empty_like(lt) for _ in range(world)]
    dist.all_gather(tabs, lt)
    assert all(torch.equal(t, lt) for t in tabs)
    plan = clbm.shard_plan(labels, world, rank)
    # sends and receives, matched by destination slot (the tag); non-blocking
    # sends so that the two ranks never wait on each other's order
    reqs = []
    for src, dst, peer in plan["sends"]:
        buf = torch.from_numpy(mine[src - rank * local].copy())
        reqs.append(dist.isend(buf, int(peer), tag=int(dst)))
    recv = {}
    for src, dst, peer in plan["recvs"]:
        buf = torch.empty(n, dtype=torch.float64)
        dist.recv(buf, int(peer), tag=int(dst))
        recv[int(dst)] = buf.numpy()
    for r in reqs:
        r.wait()
    before = mine.copy()
    for src, dst, _ in plan["locals"]:
        mine[dst - rank * local] = before[src - rank * local]
    for dst, v in recv.items():
        mine[dst - rank * local] = v
    expect = every[labels[rank * local:(rank + 1) * local]]
    assert np.array_equal(mine, expect)
    counts = np.array([len(plan["sends"]), len(plan["recvs"]), len(plan["locals"])])
    np.save(os.path.join(out_dir, f"counts{rank}.npy"), counts)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("nc,seed", [(16, 1), (64, 2), (2, 3)])
def test_clone_exchange_over_two_ranks(orc, clbm_lib, tmp_path, nc, seed):
    import torch.multiprocessing as mp
    mp.spawn(_worker, args=(2, free_port(), nc, 45, seed, str(tmp_path)), nprocs=2, join=True)
    c0, c1 = (np.load(tmp_path / f"counts{r}.npy") for r in range(2))
    assert c0[0] == c1[1] and c0[1] == c1[0]  # every send has its receive


def test_plan_matches_a_single_process_gather(clbm_lib):
    rng = np.random.default_rng(5)
    for nshards in (1, 2, 4, 8):
        nc = 8 * nshards
        parents = rng.choice(nc, size=nc // 2, replace=False)
        labels = np.arange(nc, dtype=np.int32)
        for j in range(nc):
            if j not in parents:
                labels[j] = rng.choice(parents)
        labels[parents] = parents
        seen = []
        for s in range(nshards):
            p = clbm_lib.shard_plan(labels, nshards, s)
            for src, dst, peer in p["sends"]:
                assert src // (nc // nshards) == s and peer == dst // (nc // nshards) != s
            for src, dst, peer in p["recvs"]:
                assert dst // (nc // nshards) == s and peer == src // (nc // nshards) != s
                seen.append((src, dst))
            for src, dst, peer in p["locals"]:
                assert peer == s and src // (nc // nshards) == dst // (nc // nshards) == s
                seen.append((src, dst))
            for k in p:
                assert np.all(np.diff(p[k][:, 1]) > 0)  # ascending destination slot
        expect = sorted((int(labels[j]), j) for j in range(nc) if labels[j] != j)
        assert sorted(seen) == expect


def test_plan_rejects_bad_tables(clbm_lib):
    with pytest.raises(clbm_lib.ClbmError):
        clbm_lib.shard_plan(np.array([0, 0, 1, 3]), 2, 0)   # slot 1 is a parent but not its own
    with pytest.raises(clbm_lib.ClbmError):
        clbm_lib.shard_plan(np.arange(6), 4, 0)             # 6 clones do not split in 4 blocks
    with pytest.raises(clbm_lib.ClbmError):
        clbm_lib.shard_plan(np.arange(4), 2, 2)             # no shard 2


def test_bench_reference_arm_under_two_ranks(orc):
    """torchrun with 2 processes on the host (gloo): rank 0 alone prints the
    reference arm's line, both ranks exit 0."""
    env = dict(os.environ, OMP_NUM_THREADS="1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), str(REPO / "bench.py"),
           "--impl", "reference", "--workload", "c1", "--steps", "1", "--warmup", "0", "--gpus", "2"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=REPO, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port"
