"""The library's grid partition (mglet_gpu_set_partition) on the GPU: two
ranks emulated as two contexts on one GPU, each driven by its own host
thread; the exchange function moves the packed boxes between them through
host memory (no kernel of one context waits for the other -- the host
threads meet in the exchange function).  Two RK3 steps give, on every
owned grid, the one-context result bit for bit."""
import queue
import threading

import numpy as np
import pytest

from mglet_gb300 import abi, cases, dist

pytestmark = pytest.mark.gpu


class _Board:
    """Mailboxes and a reduction point shared by the emulated ranks."""

    def __init__(self, world):
        self.world = world
        self.box = {(a, b): queue.Queue() for a in range(world) for b in range(world)}
        self.bar = threading.Barrier(world, timeout=120)
        self.vals = [None] * world


class _ThreadExchange:
    def __init__(self, board, rank):
        self.board, self.rank = board, rank
        self.error = None
        self.fn = dist.EXCHANGE_FN(self._call)

    def _call(self, user, op, npeers, peers, sendbuf, sendn, recvbuf, recvn):
        try:
            b = self.board
            if op == 0:
                for q in range(npeers):
                    b.box[(self.rank, peers[q])].put(dist._arr(sendbuf[q], sendn[q]).copy())
                for q in range(npeers):
                    got = b.box[(peers[q], self.rank)].get(timeout=120)
                    dist._arr(recvbuf[q], recvn[q])[:] = got
                return 0
            a = dist._arr(sendbuf[0], sendn[0])
            b.vals[self.rank] = a.copy()
            b.bar.wait()
            red = np.max(b.vals, axis=0) if op == 1 else np.sum(b.vals, axis=0)
            b.bar.wait()
            a[:] = red
            return 0
        except Exception as ex:
            self.error = ex
            return 1


def _setup(gpu_lib, case, fields, prm, part=None, ex=None):
    sub = part.sub if part else case
    s = gpu_lib.Solver(sub, prm)
    if part:
        s.set_partition(part, ex)
    for nm, a in zip("UVWP", fields):
        s.set(nm, part.scatter(a) if part else a)
    return s


def _steps(gpu_lib, s, out, key):
    # the first connect already exchanges, so it runs on the rank's thread
    s.connect(0, 2, "U", "V", "W", "P", corners=True)
    rk = gpu_lib.rk_scheme("williamson")
    stats = []
    for it in (1, 2):
        for irk in (1, 2, 3):
            st = s.timeintegrate_flow(it, it, 0.0, 2e-3, irk, rk)
            stats.append((st.ipc, st.maxrhs))
    info = s.itinfo(2e-3)
    out[key] = ({nm: s.get(nm) for nm in "UVWP"}, stats, (info.cflmax, info.divmax, info.energy))


def test_two_contexts_match_one(gpu_lib):
    case = cases.periodic_box(4, 2, 2, n=8)
    u, v, w, p = cases.taylor_green(case)
    u, v, w = cases.add_noise(case, (u, v, w), amplitude=1e-2, seed=42)
    fields = [u, v, w, p]
    prm = abi.make_flow_params(gmol=1e-2, epcorr=1e-6, nouter=30, ninner=3, nouter_min=0)
    out = {}
    ref = _setup(gpu_lib, case, fields, prm)
    _steps(gpu_lib, ref, out, "ref")
    board = _Board(2)
    parts = [dist.Partition(case, 2, r) for r in range(2)]
    exs = [_ThreadExchange(board, r) for r in range(2)]
    solvers = [_setup(gpu_lib, case, fields, prm, parts[r], exs[r]) for r in range(2)]
    errors = []

    def run(r):
        try:
            _steps(gpu_lib, solvers[r], out, r)
        except Exception as ex:   # surfaced below
            errors.append(ex)

    threads = [threading.Thread(target=run, args=(r,)) for r in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    assert not errors and all(e.error is None for e in exs), (errors, [e.error for e in exs])
    rfields, rstats, rinfo = out["ref"]
    npg = case.kk * case.jj * case.ii
    seen = set()
    for r in range(2):
        flds, stats, info = out[r]
        assert stats == rstats
        assert info[:2] == rinfo[:2]
        for nm in "UVWP":
            gids, vals = parts[r].owned_part(flds[nm])
            for gid, row in zip(gids, vals):
                assert np.array_equal(row, rfields[nm][gid * npg:(gid + 1) * npg]), (r, nm, gid)
                seen.add(int(gid))
    assert seen == set(range(case.ngrid))
    for s in solvers + [ref]:
        s.close()


def test_partition_refused_for_the_mixed_form(gpu_lib):
    case = cases.periodic_box(2, 1, 1, n=8)
    part = dist.Partition(case, 2, 0)
    s = gpu_lib.Solver(part.sub, abi.make_flow_params(gmol=1e-2, form=abi.FORM_MIXED))
    board = _Board(2)
    with pytest.raises(gpu_lib.MgletError):
        s.set_partition(part, _ThreadExchange(board, 0))
