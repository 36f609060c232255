"""Multi-rank host logic on CPU: LPT sharding and the per-iteration sum over
ranks (gloo, world size 2), checked against a single-process accumulation of
the same chunks.  The per-chunk work here is the CPU restatement (the oracle),
standing in for the engine that each rank runs on its GPU."""
import os
import socket
import tempfile

import numpy as np
import pytest

from lyspeq_gb300 import distributed as D


def test_shard_lpt_covers_every_item_once_and_balances():
    rng = np.random.default_rng(3)
    n = rng.integers(200, 1200, size=257)
    ns = rng.integers(60, 200, size=257)
    costs = [D.chunk_cost(a, b) for a, b in zip(n, ns)]
    for world in (1, 2, 3, 8):
        sh = D.shard_lpt(costs, world)
        flat = sorted(i for s in sh for i in s)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in s) for s in sh]
        # LPT bound: max load <= mean + largest item
        assert max(loads) <= sum(costs) / world + max(costs) + 1e-6
        assert sh == D.shard_lpt(costs, world)


def test_shard_lpt_rejects_bad_world():
    with pytest.raises(ValueError):
        D.shard_lpt([1.0], 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_plan_costs_follow_the_chunks(engine_lib):
    """Costs from lqg_chunk_plan before any engine: chunk_cost(n, stored
    matrices) of each golden chunk, 0 for one the engine would reject."""
    import golden_cases as G
    c = G.load("desi_sub")
    chunks = list(c.chunks) + [(c.chunks[0][0], c.chunks[0][1], c.chunks[0][2], 12345)]   # no such table
    offs = np.cumsum([0] + [len(x[0]) for x in chunks])
    cat = lambda j: np.concatenate([np.asarray(x[j], dtype=np.float64) for x in chunks])
    costs = D.plan_costs(c.bins, c.tables, cat(0), cat(1), cat(2), offs, [x[3] for x in chunks],
                         c.max_forest_length)
    want = [D.chunk_cost(m[0], m[2] // c.bins.nk * m[3]) for m in c.meta] + [0.0]
    assert costs == want and all(x > 0 for x in costs[:-1])


def _rank_main(rank, world, port, out_path):
    import torch.distributed as dist
    from lyspeq_gb300 import synth
    from oracle import qmle_port as P

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w = synth.make_workload("tiny")
    s = P.Settings(max_forest_length=w.max_forest_length, cont_logl_order=1, cont_l_order=-1)
    chunks = P.chunks_from_spectra(w.spectra, w.bins, w.table_index(), s)
    tvs = [P.table_view(t, w.bins, w.nv, w.lenv, w.nzp) for t in w.tables]
    costs = [D.chunk_cost(len(c.wave), 40) for c in chunks]
    mine = D.shard_lpt(costs, world)[rank]
    res = []
    for i in mine:
        ch = chunks[i]
        d, b, t, f = P.chunk_iteration(ch, w.bins, tvs[ch.res_index], np.zeros(w.bins.nkz), s)
        res.append((ch.fisher_index_start, d, b, t, f))
    fsum, dbt = P.accumulate(w.bins.nkz, res)
    F, d, b, t = D.allreduce_sums(fsum, dbt[0], dbt[1], dbt[2])
    if rank == 0:
        np.savez(out_path, F=F, dbt=np.stack([d, b, t]), n=len(chunks))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_sum_to_the_single_process_result():
    import torch.multiprocessing as mp
    from lyspeq_gb300 import synth
    from oracle import qmle_port as P

    with tempfile.TemporaryDirectory() as tmp:
        out = os.path.join(tmp, "r0.npz")
        mp.start_processes(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True,
                           start_method="spawn")
        got = np.load(out)
    w = synth.make_workload("tiny")
    s = P.Settings(max_forest_length=w.max_forest_length, cont_logl_order=1, cont_l_order=-1)
    chunks = P.chunks_from_spectra(w.spectra, w.bins, w.table_index(), s)
    tvs = [P.table_view(t, w.bins, w.nv, w.lenv, w.nzp) for t in w.tables]
    res = []
    for ch in chunks:
        d, b, t, f = P.chunk_iteration(ch, w.bins, tvs[ch.res_index], np.zeros(w.bins.nkz), s)
        res.append((ch.fisher_index_start, d, b, t, f))
    fsum, dbt = P.accumulate(w.bins.nkz, res)
    assert int(got["n"]) == len(chunks)
    scale = np.max(np.abs(fsum))
    assert np.max(np.abs(got["F"] - fsum)) <= 1e-12 * scale
    assert np.max(np.abs(got["dbt"] - dbt)) <= 1e-12 * np.max(np.abs(dbt))
