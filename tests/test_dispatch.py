"""Multi-GPU work division (dispatch.py) on CPU ranks: world_size-2 gloo process groups on
127.0.0.1.  The per-rank compute is the CPU oracle, so what is under test is the partition (cost
queues, k tiles, exciton ranges) and the host gathers: rank 0 must reproduce the one-process
results exactly (batched spectra and the assembled H) or to rounding (the split eps sum)."""
import os
import socket

import numpy as np
import pytest

OMEGA = np.arange(200) * 8.0 / 200
GAMMA = 0.05


def _dispatch():
    import __graft_entry__ as entry
    entry.load_package()
    from importlib import import_module
    return import_module("bse_gb300.dispatch")


def test_plan_batch_covers_and_balances(synth):
    d = _dispatch()
    probs = synth.random_batch_problems(n_models=64, seed=77)
    costs = [d.batch_cost(p) for p in probs]
    for ws in (1, 2, 3, 4, 8):
        q = d.plan_batch(costs, ws)
        assert sorted(i for qq in q for i in qq) == list(range(len(probs)))
        loads = [sum(costs[i] for i in qq) for qq in q]
        # greedy longest-first: no queue exceeds the mean by more than the largest single model
        assert max(loads) <= sum(costs) / ws + max(costs) + 1e-6
        assert q == d.plan_batch(costs, ws)          # deterministic


def test_ranges_and_tile_rows():
    d = _dispatch()
    for n, ws in ((10, 3), (7, 8), (144, 2)):
        rr = d.ranges(n, ws)
        assert rr[0][0] == 0 and rr[-1][1] == n and all(a[1] == b[0] for a, b in zip(rr, rr[1:]))
    rows = d.tile_rows(n_h=12, nk=4, lo=1, hi=3)
    assert rows.tolist() == [1, 2, 5, 6, 9, 10]
    with pytest.raises(ValueError):
        d.assemble_rows([(0, 2, np.zeros((6, 12))), (1, 4, np.zeros((9, 12)))], nk=4, n_h=12)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, out_q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        import __graft_entry__ as entry
        entry.load_package()
        from importlib import import_module
        d = import_module("bse_gb300.dispatch")
        synth = import_module("bse_gb300.synth")
        orc = entry.load_oracle()
        res = {}
        # batched models
        probs = [synth.hbn_problem(grid=3), synth.magnetic4_problem(grid=3), synth.hbn_problem(grid=5),
                 synth.collinear_problem(grid=3), synth.hbn_problem(grid=4)]
        e2 = d.solve_batch(probs, OMEGA, GAMMA, rank, ws,
                           solve_queue=lambda ps, om, g: [orc.solve(p, om, g)["eps2"] for p in ps])
        res["batch"] = e2
        res["queue"] = d.plan_batch([d.batch_cost(p) for p in probs], ws)[rank]
        # kernel build by k tiles (the oracle builds the whole H; each rank keeps its tile's rows)
        for name, prob in (("mag", synth.magnetic4_problem(grid=4)), ("coll", synth.collinear_problem(grid=4))):
            def rows(p, lo, hi):
                H, _ = orc.build(p, orc.bands(p))
                return H[d.tile_rows(H.shape[0], p.nk, lo, hi)]
            res["H_" + name] = d.build_sharded(prob, rank, ws, build_rows=rows)
        # eps split over excitons
        prob = synth.magnetic4_problem(grid=4)
        ref = orc.solve(prob, OMEGA, GAMMA)
        res["eps"] = d.eps_sharded(ref["E_opt"], ref["f"], ref["F"], OMEGA, GAMMA, rank, ws,
                                   eps_part=lambda E, f, F, om, g: orc.eps(E, f, F, om, g))
        if rank == 0:
            out_q.put(res)
        else:
            out_q.put({"rank": rank, "queue": res["queue"], "none": [res[k] is None for k in res if k != "queue"]})
    finally:
        dist.destroy_process_group()


def test_world_size_2_gloo(synth, oracle):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.SimpleQueue()
    port = _free_port()
    pc = mp.start_processes(_worker, args=(2, port, q), nprocs=2, join=False, start_method="spawn")
    got = [q.get(), q.get()]          # read before joining: a child blocks on a full pipe
    while not pc.join(timeout=60):
        pass
    r0 = next(g for g in got if "batch" in g)
    r1 = next(g for g in got if "rank" in g)
    assert all(r1["none"])                                    # results only on rank 0
    assert sorted(r0["queue"] + r1["queue"]) == list(range(5))
    probs = [synth.hbn_problem(grid=3), synth.magnetic4_problem(grid=3), synth.hbn_problem(grid=5),
             synth.collinear_problem(grid=3), synth.hbn_problem(grid=4)]
    for i, p in enumerate(probs):
        assert np.array_equal(r0["batch"][i], oracle.solve(p, OMEGA, GAMMA)["eps2"])
    for name, p in (("mag", synth.magnetic4_problem(grid=4)), ("coll", synth.collinear_problem(grid=4))):
        H, _ = oracle.build(p, oracle.bands(p))
        assert np.array_equal(r0["H_" + name], H)
    ref = oracle.solve(synth.magnetic4_problem(grid=4), OMEGA, GAMMA)
    e2, e1 = r0["eps"]
    assert np.abs(e2 - ref["eps2"]).max() <= 1e-12 * np.abs(ref["eps2"]).max()
    assert np.abs(e1 - ref["eps1"]).max() <= 1e-12 * np.abs(ref["eps1"]).max()
