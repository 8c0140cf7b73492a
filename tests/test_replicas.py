"""Replicas across ranks: partition of independent instances, gather of their
summaries, max-over-ranks timing. CPU only: world_size 2 over gloo, with the
oracle march standing in for the GPU solve of each instance."""
import os
import socket

import numpy as np
import pytest

from angularspectrum_heterogeneous_gb300 import replicas as R

import scenarios as S


def test_partition_covers_every_instance_once():
    rng = np.random.default_rng(0)
    costs = rng.integers(1, 100, size=37).astype(float)
    for world in (1, 2, 3, 8, 40):
        parts = R.partition(costs, world)
        assert len(parts) == world
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        # LPT bound: no rank carries more than the mean load plus one instance
        assert max(loads) <= costs.sum() / world + costs.max() + 1e-9


def test_partition_is_deterministic_and_balanced():
    costs = [128 * 128 * 256, 384 * 384 * 1024, 192 * 192 * 512, 256 * 256 * 1024,
             128 * 128 * 512, 384 * 384 * 256]
    a = R.partition(costs, 2)
    assert a == R.partition(list(costs), 2)
    loads = [sum(costs[i] for i in p) for p in a]
    assert max(loads) / min(loads) < 1.5
    assert R.partition([], 3) == [[], [], []]
    with pytest.raises(ValueError):
        R.partition(costs, 0)


def _instances():
    out = []
    for k, (nx, nt, amp) in enumerate([(8, 16, 1e5), (10, 16, 3e5), (8, 24, 2e5),
                                        (12, 16, 5e4), (8, 16, 4e5)]):
        out.append(R.Instance(index=k, shape=(nx, nx, nt), steps=2, payload=(amp, 10 + k)))
    return out


def _solve(inst):
    import oracle.asm_oracle as O
    nx, ny, nt = inst.shape
    amp, seed = inst.payload
    u0 = S.seeded_field(inst.shape, seed=seed, amp=amp)
    p = O.OracleParams(**dict(S.BASE, propDist=inst.steps * S.BASE["dZmin"]))
    return O.solve(u0, p, precision="fp64")


def _summary(inst, res):
    field, pnp, ppp, pI, pIloss, zaxis, pax = res
    return {"ppp": float(ppp.max()), "pnp": float(pnp.min()), "pI": float(pI.sum()),
            "nz": int(len(zaxis))}


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        res = R.run_instances(_instances(), _solve, _summary)
        slowest = R.max_over_ranks(1.5 + rank)
        q.put((rank, res, slowest))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_ranks_gather_every_instance():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    world, port = 2, _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = {}
    for _ in range(world):
        rank, res, slowest = q.get(timeout=240)
        got[rank] = (res, slowest)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    insts = _instances()
    # rank 0 holds every instance's summary; rank 1 only its own share
    assert sorted(got[0][0]) == [i.index for i in insts]
    share1 = R.partition([i.voxel_steps for i in insts], world)[1]
    assert sorted(got[1][0]) == share1
    assert {k for k, v in got[0][0].items() if v["rank"] == 1} == set(share1)
    # same numbers as a single-process run of each instance
    for inst in insts:
        ref = _summary(inst, _solve(inst))
        s = got[0][0][inst.index]
        for key in ("ppp", "pnp", "pI", "nz"):
            assert s[key] == ref[key], (inst.index, key)
    # max over ranks of (1.5 + rank)
    assert got[0][1] == got[1][1] == 2.5
