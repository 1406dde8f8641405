"""Multi-rank path on the CPU: two gloo ranks each step their own contiguous
column range (no data crosses ranks during the run) and reduce only the
scalar statistics at the end.  The oracle stands in for each rank's device
solver; the gathered states must equal a single-process run, column for
column, and the reduced statistics the single-process ones."""
import os
import socket
import sys

import numpy as np
import pytest

from sedgpu import shard, synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NSTEPS = 6


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, outdir):
    for p in (os.path.join(ROOT, "mossco-code_gb300"), os.path.join(ROOT, "oracle")):
        if p not in sys.path:
            sys.path.insert(0, p)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    import oracle
    from sedgpu import shard as sh
    from sedgpu import synth as sy
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        cs = sy.make_workload("uneven_1024x1024",
                              cols=np.arange(0, 1024 * 1024, 1024 * 1024 // 160)[:160])
        mine, (c0, c1) = sh.shard(cs, rank, world)
        c = mine.conc.copy()
        rc, st, fl = oracle.OracleModel(mine).run(c, nsteps=NSTEPS, percol=True, nthreads=1)
        assert rc == 0
        st["column_steps"] = int(np.count_nonzero(mine.kact)) * NSTEPS
        red = sh.reduce_stats(st)
        np.savez(os.path.join(outdir, f"rank{rank}.npz"), conc=c, fluxes=fl,
                 c0=c0, c1=c1, attempts=red["attempts"], accepted=red["accepted"],
                 column_steps=red["column_steps"], max_col=red["max_col_attempts"],
                 min_dt=red["min_dt"])
    finally:
        dist.destroy_process_group()


def test_partition_balances_work_and_covers_the_grid():
    kact = np.array([0, 30, 30, 0, 10, 60, 60, 5, 0, 30], dtype=np.int32)
    for world in (1, 2, 3, 4):
        parts = shard.partition(kact, world)
        assert parts[0][0] == 0 and parts[-1][1] == kact.size
        assert all(a[1] == b[0] for a, b in zip(parts, parts[1:]))
        work = [int(kact[a:b].sum()) for a, b in parts]
        assert max(work) <= kact.sum() / world + kact.max()


def test_two_gloo_ranks_equal_one_process(oracle_mod, tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    cs = synth.make_workload("uneven_1024x1024",
                             cols=np.arange(0, 1024 * 1024, 1024 * 1024 // 160)[:160])
    ref = cs.conc.copy()
    rc, sref, fref = oracle_mod.OracleModel(cs).run(ref, nsteps=NSTEPS, percol=True,
                                                   nthreads=1)
    assert rc == 0
    got = np.empty_like(ref)
    fl = np.empty_like(fref)
    reds = []
    for r in range(2):
        d = np.load(tmp_path / f"rank{r}.npz")
        c0, c1 = int(d["c0"]), int(d["c1"])
        got[:, :, c0:c1] = d["conc"]
        fl[:, c0:c1] = d["fluxes"]
        reds.append(d)
    np.testing.assert_array_equal(got, ref)
    np.testing.assert_array_equal(fl, fref)
    for d in reds:   # every rank holds the same whole-grid statistics
        assert int(d["attempts"]) == sref["attempts"]
        assert int(d["accepted"]) == sref["accepted"]
        assert int(d["column_steps"]) == int(np.count_nonzero(cs.kact)) * NSTEPS
        assert int(d["max_col"]) == sref["max_col_attempts"]
        assert float(d["min_dt"]) == sref["min_dt"]


def _pel_rank_main(rank, world, port, outdir):
    for p in (os.path.join(ROOT, "mossco-code_gb300"), os.path.join(ROOT, "oracle")):
        if p not in sys.path:
            sys.path.insert(0, p)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    import pel_oracle
    from sedgpu import pelagic as pl
    from sedgpu import shard as sh
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        pcs = pl.make_pelagic_workload("pelagic_cpu_16x16")
        mine, (c0, c1) = sh.shard_pelagic(pcs, rank, world)
        c = mine.conc.copy()
        rc, st, _ = pel_oracle.PelOracle(mine).run(c, nthreads=1, nruns=2)
        assert rc == 0
        st["column_steps"] = mine.water_columns() * 2
        red = sh.reduce_stats(st)
        np.savez(os.path.join(outdir, f"pel{rank}.npz"), conc=c, c0=c0, c1=c1,
                 attempts=red["attempts"], column_steps=red["column_steps"],
                 max_cell=red["max_cell_attempts"])
    finally:
        dist.destroy_process_group()


def test_pelagic_two_gloo_ranks_equal_one_process(tmp_path):
    """The pelagic grid split the same way (columns balanced by water
    cells): two ranks' Runs gathered equal one process's Runs."""
    import pel_oracle
    import torch.multiprocessing as mp
    from sedgpu import pelagic
    pel_oracle.build()
    port = _free_port()
    mp.spawn(_pel_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    pcs = pelagic.make_pelagic_workload("pelagic_cpu_16x16")
    ref = pcs.conc.copy()
    rc, sref, _ = pel_oracle.PelOracle(pcs).run(ref, nthreads=1, nruns=2)
    assert rc == 0
    got = np.empty_like(ref)
    for r in range(2):
        d = np.load(tmp_path / f"pel{r}.npz")
        got[:, :, int(d["c0"]):int(d["c1"])] = d["conc"]
        assert int(d["attempts"]) == sref["attempts"]
        assert int(d["column_steps"]) == 2 * pcs.water_columns()
        assert int(d["max_cell"]) == sref["max_cell_attempts"]
    np.testing.assert_array_equal(got, ref)
    parts = shard.partition(pcs.water().sum(axis=0), 2)
    w = [int(pcs.water()[:, a:b].sum()) for a, b in parts]
    assert abs(w[0] - w[1]) <= pcs.knum


def test_partition_edge_cases():
    """More ranks than columns, no active column, no column: the ranges stay
    contiguous and cover the grid; a rank may get an empty range."""
    for kact, world in ((np.array([5]), 3), (np.zeros(6, dtype=np.int32), 2),
                        (np.ones(4, dtype=np.int32), 8), (np.array([], dtype=np.int32), 2)):
        parts = shard.partition(kact, world)
        assert len(parts) == world
        assert parts[0][0] == 0 and parts[-1][1] == kact.size
        assert all(a[1] == b[0] and a[0] <= a[1] for a, b in zip(parts, parts[1:]))
        assert sum(b - a for a, b in parts) == kact.size


def _cpl_rank_main(rank, world, port, outdir):
    for p in (os.path.join(ROOT, "mossco-code_gb300"), os.path.join(ROOT, "oracle")):
        if p not in sys.path:
            sys.path.insert(0, p)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch
    import torch.distributed as dist
    import pel_oracle
    from sedgpu import pelagic as pl
    from sedgpu import shard as sh
    from sedgpu import synth as sy
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        pcs = pl.make_pelagic_workload("pelagic_cpu_16x16")
        cs = sy.make_columns(inum=16, jnum=16, kmin=5, kmax=15, total=0.18, land=0.2,
                             poc="loguniform", days=1, seed=3, name="soil16")
        pmine, smine, (c0, c1) = sh.shard_coupled(pcs, cs, rank, world)
        assert pmine.ncol == smine.ncol == c1 - c0
        rc, S, V, present = pel_oracle.cpl_run(pmine.conc, {"detN": 3, "din": 0})
        assert rc == 0
        # the only cross-rank traffic: one scalar, the columns mapped
        n = torch.tensor([float(pmine.ncol)])
        dist.all_reduce(n)
        np.savez(os.path.join(outdir, f"cpl{rank}.npz"), S=S, V=V, c0=c0, c1=c1,
                 total=float(n.item()))
    finally:
        dist.destroy_process_group()


def test_coupled_two_gloo_ranks_equal_one_process(tmp_path):
    """A coupled pelagic / soil grid sharded by shard_coupled: each rank
    maps its own columns (the same range of both grids) and the gathered
    soil fields equal one process's connector Run."""
    import pel_oracle
    import torch.multiprocessing as mp
    from sedgpu import pelagic
    pel_oracle.build()
    port = _free_port()
    mp.spawn(_cpl_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    pcs = pelagic.make_pelagic_workload("pelagic_cpu_16x16")
    rc, S, V, _ = pel_oracle.cpl_run(pcs.conc, {"detN": 3, "din": 0})
    assert rc == 0
    gS, gV = np.full_like(S, np.nan), np.full_like(V, np.nan)
    for r in range(2):
        d = np.load(tmp_path / f"cpl{r}.npz")
        a, b = int(d["c0"]), int(d["c1"])
        gS[:, a:b], gV[:, a:b] = d["S"], d["V"]
        assert float(d["total"]) == pcs.ncol
    np.testing.assert_array_equal(gS, S)
    np.testing.assert_array_equal(gV, V)


def test_shard_coupled_balances_both_grids():
    from sedgpu import pelagic
    pcs = pelagic.make_pelagic_workload("pelagic_cpu_16x16")
    cs = synth.make_columns(inum=16, jnum=16, kmin=5, kmax=15, total=0.18, land=0.2,
                            poc="loguniform", days=1, seed=3, name="soil16")
    work = cs.kact + shard.PEL_CELL_WEIGHT * pcs.water().sum(axis=0)
    for world in (1, 2, 3, 7):
        ranges = [shard.shard_coupled(pcs, cs, r, world)[2] for r in range(world)]
        assert ranges[0][0] == 0 and ranges[-1][1] == cs.ncol
        assert all(a[1] == b[0] for a, b in zip(ranges, ranges[1:]))
        w = [work[a:b].sum() for a, b in ranges]
        assert max(w) - min(w) <= 2 * work.max()
    small = pcs.subset(np.arange(10))
    with pytest.raises(ValueError):
        shard.shard_coupled(small, cs, 0, 2)
