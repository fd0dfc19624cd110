"""The N > 1 path of bench.py on CPU ranks (gloo, world size 2): replicas
report the slowest rank's time, and the reference arm prints from rank 0
only.  (One GPU per box in this build, so the GPU side of the replicas runs
in the driver's scaling runs, not here.)"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out.put((rank, bench.reduce_max(10.0 * (rank + 1), dist)))
    finally:
        dist.destroy_process_group()


def test_reduce_max_over_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == {0: 20.0, 1: 20.0}


def test_reference_arm_silent_on_other_ranks(capsys):
    sys.path.insert(0, ROOT)
    import bench

    class A:
        steps, warmup, gpus = 1, 0, 2
    assert bench.run_reference(A(), rank=1) == 0
    assert capsys.readouterr().out == ""


# ---------------------------------------------------------------------------
# Grid-partitioned stages: two gloo ranks, each running the CPU restatement
# on its own grids plus read-only copies of its neighbours, exchanging the
# copies' boxes at every connect and all-reducing the residual maximum, give
# the one-rank result bit for bit.

def _part_case(walls):
    import numpy as np
    from mglet_gb300 import abi, cases
    w = {1: abi.BC_FIX, 2: abi.BC_OP1} if walls else None
    case = cases.periodic_box(4, 2, 2, n=8, walls=w)
    u, v, w_, p = cases.taylor_green(case)
    u, v, w_ = cases.add_noise(case, (u, v, w_), amplitude=1e-2, seed=42)
    if walls:
        u = u + 1.0
    return case, [u, v, w_, p]


def _part_params(fixed):
    from mglet_gb300 import abi
    if fixed:
        return abi.make_flow_params(gmol=1e-2, epcorr=1e-12, nouter=4, ninner=3, nouter_min=4)
    return abi.make_flow_params(gmol=1e-2, epcorr=1e-6, nouter=30, ninner=3, nouter_min=0)


def _run_oracle(case, fields, prm, walls, part=None, exchange=None, steps=2):
    import numpy as np
    from oracle import binding
    from mglet_gb300 import abi
    sub = part.sub if part else case
    o = binding.Oracle(sub, prm)
    if part:
        o.set_partition(part, exchange)
    for nm, a in zip("UVWP", fields):
        o.set(nm, part.scatter(a) if part else a)
    if walls:
        one = np.ones(sub.kk * sub.jj)
        for g in range(sub.ngrid):
            if sub.bctype[g, 0] == abi.BC_FIX:
                o.set_buffer("U", g + 1, 1, one)
    o.connect(0, 2, "U", "V", "W", "P", corners=True)
    rk = binding.rk_scheme("williamson")
    stats = []
    for it in range(1, steps + 1):
        for irk in (1, 2, 3):
            st = o.timeintegrate_flow(it, it, 0.0, 2e-3, irk, rk)
            stats.append((st.ipc, st.nouter_done, st.maxrhs))
    info = o.itinfo(2e-3)
    out = {nm: o.get(nm) for nm in "UVWP"}
    return out, stats, (info.cflmax, info.divmax, info.energy)


def _part_worker(rank, world, port, walls, fixed, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "mglet-base_gb300"))
    from mglet_gb300 import dist as mdist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        case, fields = _part_case(walls)
        part = mdist.Partition(case, world, rank)
        ex = mdist.TorchExchange(dist)
        out, stats, info = _run_oracle(case, fields, _part_params(fixed), walls, part, ex)
        owned = {nm: part.owned_part(a) for nm, a in out.items()}
        q.put((rank, owned, stats, info, part.nowned, int(part.halo.sum()), ex.error))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("walls,fixed", [(False, True), (False, False), (True, True)],
                         ids=["periodic-fixed", "periodic-converged", "walls-fixed"])
def test_partitioned_stages_match_one_rank(oracle_lib, walls, fixed):
    """Two RK3 steps of a 4 x 2 x 2 tiling on two gloo ranks (dist_grids:
    8 grids each, the neighbours as halo copies) equal the one-rank run bit
    for bit on every owned grid; with the convergence test active the
    all-reduced maximum residual stops both ranks after the same outer
    iteration; CFL and divergence maxima agree exactly, the energy (summed
    across ranks in another order) to 1e-14."""
    import numpy as np
    torch = pytest.importorskip("torch")
    case, fields = _part_case(walls)
    ref, ref_stats, ref_info = _run_oracle(case, fields, _part_params(fixed), walls)
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_part_worker, args=(r, 2, port, walls, fixed, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    npg = case.kk * case.jj * case.ii
    seen = set()
    for rank, owned, stats, info, nowned, nhalo, err in res:
        assert err is None
        assert nowned == 8 and nhalo > 0
        assert stats == ref_stats
        assert info[0] == ref_info[0] and info[1] == ref_info[1]
        assert abs(info[2] - ref_info[2]) <= 1e-14 * abs(ref_info[2])
        for nm, (gids, vals) in owned.items():
            for gid, row in zip(gids, vals):
                assert np.array_equal(row, ref[nm][gid * npg:(gid + 1) * npg]), (rank, nm, gid)
                seen.add(int(gid))
    assert seen == set(range(case.ngrid))


def test_dist_grids_follows_the_reference_split():
    """Per level an even share, the remainders round-robin with the position
    carried over levels, contiguous runs (grids_mod.F90:344-394)."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "mglet-base_gb300"))
    from mglet_gb300.dist import dist_grids
    level = np.array([1] * 10 + [2] * 5)
    own = dist_grids(level, 4)
    # level 1: 10 = 3 + 3 + 2 + 2 (remainder to ranks 0, 1); level 2: 5 =
    # 1 + 1 + 2 + 1 (remainder continues at rank 2)
    assert own[:10].tolist() == [0, 0, 0, 1, 1, 1, 2, 2, 3, 3]
    assert own[10:].tolist() == [0, 1, 2, 2, 3]
