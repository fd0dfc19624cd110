"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product path.  The oracle's
parity status against the reference is stated in mglet_oracle.cpp's header.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")


def build(quiet=True):
    """Compile the oracle with its Makefile (g++, -ffp-contract=off)."""
    r = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    if not quiet:
        print(r.stdout)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        _lib = C.CDLL(LIB)
        vp = C.c_void_p
        _lib.oracle_last_error.restype = C.c_char_p
        _lib.oracle_idim3d.restype = C.c_int64
        _lib.oracle_idim3d.argtypes = [vp]
        _lib.oracle_create.argtypes = [vp, vp, C.POINTER(vp)]
        for fn in ("oracle_tstle4", "oracle_destroy"):
            getattr(_lib, fn).argtypes = [vp]
        _lib.oracle_set_field.argtypes = [vp, C.c_char_p, vp, C.c_int64]
        _lib.oracle_get_field.argtypes = [vp, C.c_char_p, vp, C.c_int64]
        _lib.oracle_get_sip_index.argtypes = [vp, vp, vp, C.c_int64]
        _lib.oracle_get_conns.argtypes = [vp, vp, C.c_int64, C.POINTER(C.c_int64)]
        _lib.oracle_rkstep.argtypes = [vp, C.c_char_p, C.c_char_p, C.c_char_p, C.c_double,
                                       C.c_double]
        _lib.oracle_connect.argtypes = [vp, C.c_int, C.c_int] + [C.c_char_p] * 6 + [
            C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int64)]
        _lib.oracle_divcal.argtypes = [vp, C.c_char_p, C.c_double]
        _lib.oracle_laplacephi.argtypes = [vp, C.c_char_p, C.c_char_p]
        _lib.oracle_mgpoisl.argtypes = [vp, C.c_double, C.c_int, C.c_int, vp]
        _lib.oracle_timeintegrate_flow.argtypes = [vp, C.c_int, C.c_int, C.c_double, C.c_double,
                                                   C.c_int, vp, vp]
        _lib.oracle_itinfo.argtypes = [vp, C.c_double, vp]
        _lib.oracle_set_partition.argtypes = [vp, vp, C.c_int32, vp, C.c_int32, vp, vp, vp]
        _lib.oracle_set_buffer.argtypes = [vp, C.c_char_p, C.c_int, C.c_int, vp, C.c_int64]
        _lib.oracle_set_bc_real.argtypes = [vp, C.c_int, C.c_int, C.c_double]
        _lib.oracle_bound_flow.argtypes = [vp, C.c_int]
        _lib.oracle_get_buffer.argtypes = [vp, C.c_char_p, C.c_int, C.c_int, vp, C.c_int64]
        _lib.oracle_set_hierarchy.argtypes = [vp, vp, vp]
        _lib.oracle_parent.argtypes = [vp, C.c_int] + [C.c_char_p] * 6 + [C.c_int]
        _lib.oracle_ftoc.argtypes = [vp, C.c_int, C.c_char_p, C.c_char_p, C.c_char]
        _lib.oracle_ftoc_multiple.argtypes = [vp, C.c_int] + [C.c_char_p] * 6
        _lib.oracle_set_body_force.argtypes = [vp, vp, vp, vp, C.c_int64]
        _lib.oracle_set_lesmodel.argtypes = [vp, C.c_int, C.c_double]
        _lib.oracle_set_scalars.argtypes = [vp, C.c_int, vp, vp, vp, C.c_double]
        _lib.oracle_timeintegrate_scalar.argtypes = [vp, C.c_double, C.c_int, vp]
        _lib.oracle_set_buoyancy.argtypes = [vp, vp, C.c_double, C.c_int]
        _lib.oracle_set_coriolis.argtypes = [vp, vp]
        _lib.oracle_set_scalar_bc.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp]
        _lib.oracle_add_scalar_source.argtypes = [vp, C.c_int, C.c_char_p, C.c_double]
        _lib.oracle_set_scastencils.argtypes = [vp, C.c_int, C.c_int, vp, vp, vp]
        _lib.oracle_set_scalar_geometry.argtypes = [vp, C.c_int, C.c_int, vp, vp]
        _lib.oracle_par_ftoc_norm.argtypes = [vp, C.c_int] + [C.c_char_p] * 3 + [C.c_int]
        _lib.oracle_ctof.argtypes = [vp, C.c_int, C.c_char_p, C.c_char_p]
        _lib.oracle_bound_pressure.argtypes = [vp, C.c_int, C.c_char_p, C.c_int]
        _lib.oracle_set_stencils.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp, C.c_int64, vp,
                                             C.c_int64, vp, C.c_int64]
        _lib.oracle_set_ghostcell.argtypes = [vp]
        _lib.oracle_setpointvalues.argtypes = [vp, C.c_int]
        _lib.oracle_gc_mode.argtypes = [vp, C.c_char_p]
        _lib.oracle_rk_init.argtypes = [C.c_char_p, vp]
        _lib.oracle_rk_get_coeffs.argtypes = [vp, C.c_int] + [C.POINTER(C.c_double)] * 4
        _lib.oracle_set_threads.argtypes = [C.c_int]
        _lib.oracle_max_threads.restype = C.c_int
    return _lib


def _b(s):
    return None if s is None else s.encode()


class OracleError(RuntimeError):
    pass


def _check(rc):
    if rc != 0:
        raise OracleError(f"oracle status {rc}: {lib().oracle_last_error().decode()}")


def rk_scheme(name):
    from mglet_gb300.abi import RKScheme
    rk = RKScheme()
    _check(lib().oracle_rk_init(name.encode(), C.byref(rk)))
    return rk


def rk_coeffs(rk, irk):
    vals = [C.c_double() for _ in range(4)]
    _check(lib().oracle_rk_get_coeffs(C.byref(rk), irk, *[C.byref(v) for v in vals]))
    return tuple(v.value for v in vals)


def set_threads(n):
    lib().oracle_set_threads(int(n))


def max_threads():
    return lib().oracle_max_threads()


class Oracle:
    """One oracle context: the FP64 CPU restatement of the stage."""

    def __init__(self, case, params):
        from mglet_gb300.abi import GridDesc  # noqa: F401  (struct layout)
        self.case = case
        self._desc = case.desc()
        self._params = params
        h = C.c_void_p()
        _check(lib().oracle_create(C.byref(self._desc), C.byref(params), C.byref(h)))
        self.h = h
        self.n = lib().oracle_idim3d(h)

    def close(self):
        if self.h:
            lib().oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        _check(lib().oracle_set_field(self.h, name.encode(), a.ctypes.data, a.size))

    def get(self, name, n=None):
        n = self.n if n is None else n
        a = np.empty(n, dtype=np.float64)
        _check(lib().oracle_get_field(self.h, name.encode(), a.ctypes.data, n))
        return a

    def sip_index(self):
        mip = np.empty(self.n, dtype=np.int64)
        idx = np.empty(self.n, dtype=np.int64)
        _check(lib().oracle_get_sip_index(self.h, mip.ctypes.data, idx.ctypes.data, self.n))
        return mip, idx

    def conns(self):
        nrows = C.c_int64()
        _check(lib().oracle_get_conns(self.h, None, 0, C.byref(nrows)))
        rows = np.zeros((nrows.value, 4), dtype=np.int32)
        _check(lib().oracle_get_conns(self.h, rows.ctypes.data, nrows.value, C.byref(nrows)))
        return rows

    def tstle4(self):
        _check(lib().oracle_tstle4(self.h))

    def rkstep(self, p, dp, rhs, frhs, dtfu):
        _check(lib().oracle_rkstep(self.h, p.encode(), dp.encode(), rhs.encode(), frhs, dtfu))

    def connect(self, ilevel=0, layers=1, v1=None, v2=None, v3=None, s1=None, s2=None, s3=None,
                corners=False, normal=False, forward=0):
        n = C.c_int64()
        _check(lib().oracle_connect(self.h, ilevel, layers, _b(v1), _b(v2), _b(v3), _b(s1),
                                    _b(s2), _b(s3), int(corners), int(normal), int(forward),
                                    C.byref(n)))
        return n.value

    def divcal(self, div, fak):
        _check(lib().oracle_divcal(self.h, div.encode(), fak))

    def laplacephi(self, res, phi):
        _check(lib().oracle_laplacephi(self.h, res.encode(), phi.encode()))

    def mgpoisl(self, dt, ittot=1, irk=1):
        from mglet_gb300.abi import StageStats
        st = StageStats()
        _check(lib().oracle_mgpoisl(self.h, dt, ittot, irk, C.byref(st)))
        return st

    def timeintegrate_flow(self, itstep, ittot, timeph, dt, irk, rk):
        from mglet_gb300.abi import StageStats
        st = StageStats()
        _check(lib().oracle_timeintegrate_flow(self.h, itstep, ittot, timeph, dt, irk,
                                               C.byref(rk), C.byref(st)))
        return st

    def set_buffer(self, name, igrid, iface, plane):
        """Boundary buffer of U, V or W on face iface (1..6) of grid igrid
        (1-based): a (kk,jj), (kk,ii) or (jj,ii) plane, first index fastest."""
        a = np.ascontiguousarray(plane, dtype=np.float64).ravel(order="F")
        _check(lib().oracle_set_buffer(self.h, _b(name), igrid, iface,
                                       a.ctypes.data_as(C.c_void_p), a.size))

    def set_bc_real(self, igrid, iface, value):
        """The real parameter of an OP1 face (the far-field pressure)."""
        _check(lib().oracle_set_bc_real(self.h, igrid, iface, value))

    def bound_flow(self, ilevel=0):
        _check(lib().oracle_bound_flow(self.h, ilevel))

    def get_buffer(self, name, igrid, iface, shape):
        a = np.zeros(int(np.prod(shape)), dtype=np.float64)
        _check(lib().oracle_get_buffer(self.h, _b(name), igrid, iface,
                                       a.ctypes.data_as(C.c_void_p), a.size))
        return a.reshape(shape, order="F")

    def set_hierarchy(self, iparent, position):
        ip = np.ascontiguousarray(iparent, dtype=np.int32)
        ps = np.ascontiguousarray(position, dtype=np.int32)
        _check(lib().oracle_set_hierarchy(self.h, ip.ctypes.data_as(C.c_void_p),
                                          ps.ctypes.data_as(C.c_void_p)))

    def parent(self, ilevel, v=None, s=(), normal=False):
        v = list(v) if v else [None] * 3
        s = list(s) + [None] * (3 - len(s))
        _check(lib().oracle_parent(self.h, ilevel, *[_b(n) for n in v + s], int(normal)))

    def ftoc(self, ilevel, ff, fc, flag):
        _check(lib().oracle_ftoc(self.h, ilevel, _b(ff), _b(fc), flag.encode()))

    def ftoc_multiple(self, ilevel, v=None, s=()):
        v = list(v) if v else [None] * 3
        s = list(s) + [None] * (3 - len(s))
        _check(lib().oracle_ftoc_multiple(self.h, ilevel, *[_b(n) for n in v + s]))

    def set_scalars(self, prmol, kayscrawford=None, source=None, prturb=1.0):
        """Scalars T1..Tn with molecular Prandtl numbers prmol, the
        Kays/Crawford switch and a constant source each."""
        n = len(prmol)
        pr = np.ascontiguousarray(prmol, dtype=np.float64)
        kc = np.ascontiguousarray(kayscrawford if kayscrawford is not None else [0] * n, dtype=np.int32)
        so = np.ascontiguousarray(source if source is not None else [0.0] * n, dtype=np.float64)
        self._sca = (pr, kc, so)
        _check(lib().oracle_set_scalars(self.h, n, pr.ctypes.data_as(C.c_void_p), kc.ctypes.data_as(C.c_void_p),
                                        so.ctypes.data_as(C.c_void_p), prturb))

    def timeintegrate_scalar(self, dt, irk, rk):
        _check(lib().oracle_timeintegrate_scalar(self.h, dt, irk, C.byref(rk)))

    def set_buoyancy(self, gravity, beta, iscalar=1):
        g = np.ascontiguousarray(gravity, dtype=np.float64)
        self._g = g
        _check(lib().oracle_set_buoyancy(self.h, g.ctypes.data_as(C.c_void_p), beta, iscalar))

    def add_scalar_source(self, isca, value, field=None):
        _check(lib().oracle_add_scalar_source(self.h, isca, field.encode() if field else None, value))

    def set_scastencils(self, igrid, xpoli, xpolr, xpolrvel):
        """Scalar ghost-cell list of grid igrid (1-based): per cell 9 integers
        {intcell, body, nstencils, six stencil cells} and 8 reals {areabyvol,
        six coefficients, acoeffvel}, for the 'C' (xpolr) and 'P' (xpolrvel)
        forms."""
        xi = np.ascontiguousarray(xpoli, dtype=np.int64)
        xr = np.ascontiguousarray(xpolr, dtype=np.float64)
        xv = np.ascontiguousarray(xpolrvel, dtype=np.float64)
        _check(lib().oracle_set_scastencils(self.h, igrid, len(xi) // 9, xi.ctypes.data_as(C.c_void_p),
                                            xr.ctypes.data_as(C.c_void_p), xv.ctypes.data_as(C.c_void_p)))

    def set_scalar_geometry(self, isca, flags, values):
        """Per body of the ghost-cell IB the scalar's condition: flag 0 fixed
        value, 1 fixed flux, and its value."""
        fl = np.ascontiguousarray(flags, dtype=np.int32)
        va = np.ascontiguousarray(values, dtype=np.float64)
        _check(lib().oracle_set_scalar_geometry(self.h, isca, len(fl), fl.ctypes.data_as(C.c_void_p),
                                                va.ctypes.data_as(C.c_void_p)))

    def set_scalar_bc(self, igrid, iface, kind, types=()):
        ty = np.ascontiguousarray(list(types) + [0] * 9, dtype=np.int32)
        _check(lib().oracle_set_scalar_bc(self.h, igrid, iface, kind, ty.ctypes.data_as(C.c_void_p)))

    def set_coriolis(self, omega):
        om = np.ascontiguousarray(omega, dtype=np.float64)
        self._om = om
        _check(lib().oracle_set_coriolis(self.h, om.ctypes.data_as(C.c_void_p)))

    def set_lesmodel(self, model, cm=-1.0):
        """0 none, 1 smagorinsky, 2 wale, 5 sigma; cm < 0 takes the model's default."""
        _check(lib().oracle_set_lesmodel(self.h, model, cm))

    def set_body_force(self, fx, fy, fz):
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in (fx, fy, fz)]
        _check(lib().oracle_set_body_force(self.h, *[x.ctypes.data_as(C.c_void_p) for x in a], a[0].size))

    def par_ftoc_norm(self, ilevel, v1="U", v2="V", v3="W", sum=False):
        _check(lib().oracle_par_ftoc_norm(self.h, ilevel, _b(v1), _b(v2), _b(v3), int(sum)))

    def ctof(self, ilevel, ff, fc):
        _check(lib().oracle_ctof(self.h, ilevel, _b(ff), _b(fc)))

    def bound_pressure(self, ilevel, dp, with_bp=False):
        _check(lib().oracle_bound_pressure(self.h, ilevel, _b(dp), int(with_bp)))

    def set_stencils(self, igrid, comp, ncells, xpoli, xpolr, xpolrvel=None):
        """Ghost-cell lists of grid igrid (1-based): comp 1..3 (u, v, w) with
        xpoli [intcell, n, stcell x n], xpolr / xpolrvel [coeff x n, const];
        comp 4 the flux correction, xpoli [foundnr, intcell], xpolr
        [ax1, ax2, ay1, ay2, az1, az2, acoeff] per cell."""
        xi = np.ascontiguousarray(xpoli, dtype=np.int64)
        xr = np.ascontiguousarray(xpolr, dtype=np.float64)
        xv = np.ascontiguousarray(xpolrvel if xpolrvel is not None else [], dtype=np.float64)
        _check(lib().oracle_set_stencils(self.h, igrid, comp, ncells, xi.ctypes.data_as(C.c_void_p),
                                         xi.size, xr.ctypes.data_as(C.c_void_p), xr.size,
                                         xv.ctypes.data_as(C.c_void_p), xv.size))

    def set_ghostcell(self):
        _check(lib().oracle_set_ghostcell(self.h))

    def setpointvalues(self, comp_new=True):
        _check(lib().oracle_setpointvalues(self.h, 1 if comp_new else 0))

    def gc_mode(self, mode):
        """One ghost-cell operation on U, V, W: 'F', 'C', 'S', 'R', 'X', 'Y',
        'Z' (setibvalues_level / setpointvalues_all), 'I' (setibvalues), 'M'
        (maskbp, also P)."""
        _check(lib().oracle_gc_mode(self.h, _b(mode)))

    def set_partition(self, part, exchange):
        """The same partition hooks as the library's mglet_gpu_set_partition."""
        self._part = (part, exchange)
        halo = np.ascontiguousarray(part.halo, dtype=np.int32)
        send = np.ascontiguousarray(part.send, dtype=np.int32)
        recv = np.ascontiguousarray(part.recv, dtype=np.int32)
        self._part_arrays = (halo, send, recv)
        fnp = C.cast(exchange.fn, C.c_void_p)
        _check(lib().oracle_set_partition(self.h, halo.ctypes.data, len(send), send.ctypes.data,
                                          len(recv), recv.ctypes.data, fnp, None))

    def itinfo(self, dt):
        from mglet_gb300.abi import ItInfo
        out = ItInfo()
        _check(lib().oracle_itinfo(self.h, dt, C.byref(out)))
        return out
