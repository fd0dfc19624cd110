"""Grid-partitioned runs over several ranks (one GPU each).

The reference gives every MPI rank whole grids, level by level in
contiguous runs (dist_grids, src/core/grids_mod.F90:344-394), and its
connect sends and receives the halo boxes between ranks
(src/core/connect/connect2_mod.F90:406-548); the pressure solve all-reduces
the maximum residual (src/flow/pressuresolver_mod.F90:295).

Here a rank's context holds the grids it owns followed by read-only copies
of the remote grids next to them ("halo grids"); `Partition` builds that
sub-case and the per-peer box tables, and the library refreshes the copies
at every connect through an exchange function (mglet_gpu_set_partition).
`TorchExchange` is that function over a torch.distributed process group
(host buffers: gloo directly, NCCL through staging tensors on the device).

The box a copy needs from its owner, per direction d towards one of this
rank's grids: the two interior layers next to the face, edge or corner of d
along the axes d points along, and the whole extent (ghosts included) along
the others, which covers every source box of connect, its edge and corner
rescue copies included.  One grid level only.
"""
import ctypes as C

import numpy as np

from . import abi, cases


def dist_grids(level, nprocs):
    """Owning rank (0-based) of every grid: per level, in grid order, an
    even share per rank, the remainders handed out round-robin with the
    position carried from level to level (grids_mod.F90:344-394)."""
    level = np.asarray(level)
    owner = np.full(len(level), -1, dtype=np.int64)
    rest_proc = 0
    for lvl in sorted(set(int(v) for v in level)):
        grids = [g for g in range(len(level)) if level[g] == lvl]
        n = len(grids) // nprocs
        count = [n] * nprocs
        for _ in range(len(grids) % nprocs):
            count[rest_proc] += 1
            rest_proc = (rest_proc + 1) % nprocs
        iproc, handed = 0, 0
        for g in grids:
            while count[iproc] < 1:
                iproc += 1
            if handed < count[iproc]:
                owner[g] = iproc
                handed += 1
            if handed == count[iproc]:
                iproc += 1
                handed = 0
    return owner


def _box(case, d):
    """The box of a grid that its neighbour in direction d = (di, dj, dk)
    reads: [k0, k1, j0, j1, i0, i1], 1-based inclusive."""
    out = []
    for comp, n in ((d[2], case.kk), (d[1], case.jj), (d[0], case.ii)):
        if comp < 0:
            out += [3, 4]
        elif comp > 0:
            out += [n - 3, n - 2]
        else:
            out += [1, n]
    return out


class Partition:
    """Rank `rank`'s share of `case` among `nprocs` ranks.

    sub       the rank's Case: owned grids, then halo copies, each group in
              global grid order, NBRGRID renumbered (neighbours outside the
              rank's set become 0);
    gids      0-based global id of every grid of sub;
    halo      int32 flags (1 = copy of a remote grid);
    send, recv  int32 rows [peer, grid of sub (1-based), k0, k1, j0, j1, i0,
              i1], both sides of a pair listing the same boxes in the same
              order."""

    def __init__(self, case, nprocs, rank):
        if int(case.level.min()) != int(case.level.max()):
            raise ValueError("grid partitions cover one level")
        self.case, self.nprocs, self.rank = case, nprocs, rank
        owner = dist_grids(case.level, nprocs)
        self.owner = owner
        owned = [g for g in range(case.ngrid) if owner[g] == rank]
        ghost = set()
        for g in owned:
            for s in range(26):
                nb = int(case.nbrgrid[g, s]) - 1
                if nb >= 0 and owner[nb] != rank:
                    ghost.add(nb)
        gids = owned + sorted(ghost)
        self.gids = np.array(gids, dtype=np.int64)
        self.nowned = len(owned)
        local = {g: q for q, g in enumerate(gids)}
        self.halo = np.array([0] * len(owned) + [1] * len(ghost), dtype=np.int32)
        send, recv = [], []
        for g in range(case.ngrid):
            for s in range(1, 27):
                nb = int(case.nbrgrid[g, s - 1]) - 1
                if nb < 0:
                    continue
                box = _box(case, cases.slot_offset(s))
                if owner[g] == rank and owner[nb] != rank:
                    send.append([int(owner[nb]), local[g] + 1] + box)
                elif owner[g] != rank and owner[nb] == rank:
                    recv.append([int(owner[g]), local[g] + 1] + box)
        self.send = np.array(send, dtype=np.int32).reshape(-1, 8)
        self.recv = np.array(recv, dtype=np.int32).reshape(-1, 8)
        self.sub = self._subcase(case, gids, local)

    @staticmethod
    def _subcase(case, gids, local):
        nb = np.zeros((len(gids), 26), dtype=np.int32)
        for q, g in enumerate(gids):
            for s in range(26):
                n = int(case.nbrgrid[g, s]) - 1
                nb[q, s] = local[n] + 1 if n >= 0 and n in local else 0
        sel1 = lambda a, w: np.concatenate([a[g * w:(g + 1) * w] for g in gids])
        return cases.Case(
            ngrid=len(gids), kk=case.kk, jj=case.jj, ii=case.ii,
            mgdims=case.mgdims[gids], level=case.level[gids], bctype=case.bctype[gids],
            nbrgrid=nb, gridpos=case.gridpos[gids],
            x=sel1(case.x, case.ii), y=sel1(case.y, case.jj), z=sel1(case.z, case.kk),
            dx=sel1(case.dx, case.ii), dy=sel1(case.dy, case.jj), dz=sel1(case.dz, case.kk),
            ddx=sel1(case.ddx, case.ii), ddy=sel1(case.ddy, case.jj), ddz=sel1(case.ddz, case.kk))

    def scatter(self, flat):
        """The rank's part (owned grids and copies) of a global flat field."""
        npg = self.case.kk * self.case.jj * self.case.ii
        v = flat.reshape(self.case.ngrid, npg)
        return np.ascontiguousarray(v[self.gids].ravel())

    def owned_part(self, flat_sub):
        """(global ids, [nowned, points]) of the owned grids of a sub field."""
        npg = self.case.kk * self.case.jj * self.case.ii
        return self.gids[:self.nowned], flat_sub.reshape(-1, npg)[:self.nowned]


EXCHANGE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_int32),
                          C.POINTER(C.POINTER(C.c_double)), C.POINTER(C.c_int64),
                          C.POINTER(C.POINTER(C.c_double)), C.POINTER(C.c_int64))


def _arr(ptr, n):
    return np.ctypeslib.as_array(ptr, shape=(int(n),)) if n else np.zeros(0)


class TorchExchange:
    """The exchange function over a torch.distributed process group: op 0
    posts every send and receive at once and waits, op 1 / 2 all-reduce
    (max / sum).  With an NCCL group the host buffers are staged through
    tensors on `device`."""

    def __init__(self, dist, device=None, group=None):
        self.dist, self.group = dist, group
        self.device = device
        self.error = None
        self.fn = EXCHANGE_FN(self._call)

    def _t(self, a):
        import torch
        t = torch.from_numpy(a)
        return t.to(self.device) if self.device is not None else t

    def _call(self, user, op, npeers, peers, sendbuf, sendn, recvbuf, recvn):
        try:
            d = self.dist
            if op == 0:
                reqs, back = [], []
                for q in range(npeers):
                    s = self._t(_arr(sendbuf[q], sendn[q]))
                    r_host = _arr(recvbuf[q], recvn[q])
                    r = self._t(r_host) if self.device is not None else self._t(r_host)
                    reqs.append(d.isend(s, int(peers[q]), group=self.group))
                    reqs.append(d.irecv(r, int(peers[q]), group=self.group))
                    back.append((r_host, r))
                for rq in reqs:
                    rq.wait()
                if self.device is not None:
                    for h, r in back:
                        h[:] = r.cpu().numpy()
                return 0
            a = _arr(sendbuf[0], sendn[0])
            t = self._t(a.copy())
            d.all_reduce(t, op=d.ReduceOp.MAX if op == 1 else d.ReduceOp.SUM, group=self.group)
            a[:] = t.cpu().numpy()
            return 0
        except Exception as ex:   # reported through the library's status
            self.error = ex
            return 1
