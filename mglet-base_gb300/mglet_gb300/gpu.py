"""ctypes binding of libmglet_gpu.so, shaped like the reference's modules.

`Solver` wraps one mglet_ctx and exposes the calls timeloop_mod makes
(timeintegrate_flow, itinfo) plus the module-level procedures
(tstle4, rkstep, connect, divcal, laplacephi, mgpoisl).  There is no CPU
fallback: if the CUDA library is missing or no GPU is present, every
constructor raises.
"""
import ctypes as C
import os

import numpy as np

from . import abi
from .build import LIB

_lib = None

# Every symbol declared in include/mglet_gpu.h.
EXPORTS = [
    "mglet_rk_init", "mglet_rk_get_coeffs", "mglet_gpu_create", "mglet_gpu_destroy",
    "mglet_gpu_idim3d", "mglet_gpu_set_field", "mglet_gpu_get_field",
    "mglet_gpu_timeintegrate_flow", "mglet_gpu_tstle4", "mglet_gpu_rkstep", "mglet_gpu_connect",
    "mglet_gpu_divcal", "mglet_gpu_laplacephi", "mglet_gpu_mgpoisl", "mglet_gpu_itinfo",
    "mglet_gpu_synchronize", "mglet_gpu_kernel_launches", "mglet_gpu_last_error",
    "mglet_gpu_abi_version", "mglet_gpu_stream", "mglet_gpu_profile", "mglet_gpu_profile_get",
    "mglet_gpu_profile_names", "mglet_gpu_divmax_noalloc", "mglet_gpu_bound_flow",
    "mglet_gpu_set_buffer", "mglet_gpu_set_bc_real", "mglet_gpu_set_stencils",
    "mglet_gpu_set_ghostcell", "mglet_gpu_setibvalues", "mglet_gpu_getibvalues",
    "mglet_gpu_setpointvalues", "mglet_gpu_maskbp", "mglet_gpu_get_buffer",
    "mglet_gpu_set_hierarchy", "mglet_gpu_parent", "mglet_gpu_ftoc", "mglet_gpu_ftoc_multiple",
    "mglet_gpu_ctof", "mglet_gpu_bound_pressure", "mglet_gpu_par_ftoc_norm",
    "mglet_gpu_set_body_force", "mglet_gpu_adjoint_rk_stage", "mglet_gpu_energy_gradient",
    "mglet_gpu_set_lesmodel", "mglet_gpu_set_scalars", "mglet_gpu_timeintegrate_scalar",
    "mglet_gpu_set_buoyancy", "mglet_gpu_set_coriolis", "mglet_gpu_set_scalar_bc",
    "mglet_gpu_add_scalar_source", "mglet_gpu_fp64_roof", "mglet_gpu_tuning",
    "mglet_gpu_force_variant", "mglet_create_flowstencils", "mglet_flowstencils_size",
    "mglet_flowstencils_copy", "mglet_flowstencils_free", "mglet_gpu_set_partition",
    "mglet_gpu_test_wait_timeout", "mglet_gpu_test_barrier_timeout", "mglet_gpu_set_scastencils",
    "mglet_gpu_set_scalar_geometry", "mglet_create_scastencils", "mglet_scastencils_size",
    "mglet_scastencils_copy", "mglet_scastencils_free", "mglet_mesh_create",
    "mglet_mesh_distance", "mglet_mesh_free",
]


class MgletError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"mglet_gpu status {code}: {msg}")
        self.code = code


def load(path=None):
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB
    if not os.path.exists(path):
        raise RuntimeError(f"{path} not built: run __graft_entry__.build() "
                           "(the GPU path has no CPU fallback)")
    L = C.CDLL(path)
    vp = C.c_void_p
    cp = C.c_char_p
    L.mglet_gpu_last_error.restype = C.c_char_p
    L.mglet_gpu_abi_version.restype = C.c_int32
    L.mglet_gpu_idim3d.restype = C.c_int64
    L.mglet_gpu_idim3d.argtypes = [vp]
    L.mglet_gpu_kernel_launches.restype = C.c_int64
    L.mglet_gpu_kernel_launches.argtypes = [vp]
    L.mglet_rk_init.argtypes = [cp, vp]
    L.mglet_rk_get_coeffs.argtypes = [vp, C.c_int32] + [C.POINTER(C.c_double)] * 4
    L.mglet_gpu_create.argtypes = [vp, vp, C.c_int32, C.POINTER(vp)]
    L.mglet_gpu_destroy.argtypes = [vp]
    L.mglet_gpu_set_field.argtypes = [vp, cp, vp, C.c_int64]
    L.mglet_gpu_get_field.argtypes = [vp, cp, vp, C.c_int64]
    L.mglet_gpu_timeintegrate_flow.argtypes = [vp, C.c_int32, C.c_int32, C.c_double, C.c_double,
                                               C.c_int32, vp, vp]
    L.mglet_gpu_tstle4.argtypes = [vp]
    L.mglet_gpu_rkstep.argtypes = [vp, cp, cp, cp, C.c_double, C.c_double]
    L.mglet_gpu_connect.argtypes = [vp, C.c_int32, C.c_int32] + [cp] * 6 + [C.c_int32] * 3
    L.mglet_gpu_divcal.argtypes = [vp, cp, C.c_double]
    L.mglet_gpu_laplacephi.argtypes = [vp, cp, cp]
    L.mglet_gpu_mgpoisl.argtypes = [vp, C.c_double, C.c_int32, C.c_int32, vp]
    L.mglet_gpu_itinfo.argtypes = [vp, C.c_double, vp]
    L.mglet_gpu_bound_flow.argtypes = [vp, C.c_int32]
    L.mglet_gpu_set_buffer.argtypes = [vp, cp, C.c_int32, C.c_int32, vp, C.c_int64]
    L.mglet_gpu_set_bc_real.argtypes = [vp, C.c_int32, C.c_int32, C.c_double]
    L.mglet_gpu_get_buffer.argtypes = [vp, cp, C.c_int32, C.c_int32, vp, C.c_int64]
    L.mglet_gpu_set_hierarchy.argtypes = [vp, vp, vp]
    L.mglet_gpu_parent.argtypes = [vp, C.c_int32] + [cp] * 6 + [C.c_int32]
    L.mglet_gpu_ftoc.argtypes = [vp, C.c_int32, cp, cp, C.c_char]
    L.mglet_gpu_ftoc_multiple.argtypes = [vp, C.c_int32] + [cp] * 6
    L.mglet_gpu_ctof.argtypes = [vp, C.c_int32, cp, cp]
    L.mglet_gpu_par_ftoc_norm.argtypes = [vp, C.c_int32, cp, cp, cp, C.c_int32]
    L.mglet_gpu_set_body_force.argtypes = [vp, vp, vp, vp, C.c_int64]
    L.mglet_gpu_set_lesmodel.argtypes = [vp, C.c_int32, C.c_double]
    L.mglet_gpu_set_scalars.argtypes = [vp, C.c_int32, vp, vp, vp, C.c_double]
    L.mglet_gpu_set_buoyancy.argtypes = [vp, vp, C.c_double, C.c_int32]
    L.mglet_gpu_set_coriolis.argtypes = [vp, vp]
    L.mglet_gpu_set_scalar_bc.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, vp]
    L.mglet_gpu_add_scalar_source.argtypes = [vp, C.c_int32, C.c_char_p, C.c_double]
    L.mglet_gpu_timeintegrate_scalar.argtypes = [vp, C.c_double, C.c_int32, vp]
    L.mglet_gpu_adjoint_rk_stage.argtypes = [vp, C.c_int32, C.c_double, vp]
    L.mglet_gpu_energy_gradient.argtypes = [vp, C.c_int32, C.c_int32, C.c_double, vp,
                                            C.POINTER(C.c_double)]
    L.mglet_gpu_bound_pressure.argtypes = [vp, C.c_int32, cp, C.c_int32]
    L.mglet_gpu_set_stencils.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, vp, C.c_int64, vp,
                                         C.c_int64, vp, C.c_int64]
    for fn in ("mglet_gpu_set_ghostcell", "mglet_gpu_setibvalues", "mglet_gpu_getibvalues",
               "mglet_gpu_maskbp"):
        getattr(L, fn).argtypes = [vp]
    L.mglet_gpu_setpointvalues.argtypes = [vp, C.c_int32]
    L.mglet_gpu_synchronize.argtypes = [vp]
    L.mglet_gpu_stream.restype = vp
    L.mglet_gpu_stream.argtypes = [vp]
    L.mglet_gpu_profile.argtypes = [vp, C.c_int32]
    L.mglet_gpu_profile_get.argtypes = [vp, cp, C.POINTER(C.c_double), C.POINTER(C.c_int64)]
    L.mglet_gpu_profile_names.argtypes = [vp, cp, C.c_int64]
    L.mglet_gpu_divmax_noalloc.argtypes = [vp, vp, vp, C.c_int32, C.c_int32, C.c_int32,
                                           C.c_int32, vp, vp, vp, vp, vp]
    L.mglet_gpu_fp64_roof.argtypes = [C.c_int32, C.POINTER(C.c_double)]
    L.mglet_gpu_tuning.argtypes = [vp, cp, C.c_int64]
    L.mglet_gpu_force_variant.argtypes = [vp, cp, C.c_int32]
    L.mglet_gpu_test_wait_timeout.argtypes = [vp]
    L.mglet_gpu_test_barrier_timeout.argtypes = [vp]
    L.mglet_gpu_set_scastencils.argtypes = [vp, C.c_int32, C.c_int32, vp, vp, vp]
    L.mglet_gpu_set_scalar_geometry.argtypes = [vp, C.c_int32, C.c_int32, vp, vp]
    L.mglet_create_scastencils.argtypes = [vp, vp, C.POINTER(vp)]
    L.mglet_scastencils_size.argtypes = [vp, C.c_int32, C.POINTER(C.c_int32)]
    L.mglet_scastencils_copy.argtypes = [vp, C.c_int32, vp, vp, vp]
    L.mglet_scastencils_free.argtypes = [vp]
    L.mglet_mesh_create.argtypes = [vp, C.c_int64, C.POINTER(vp)]
    L.mglet_mesh_distance.argtypes = [vp, vp, C.c_int64, vp, vp]
    L.mglet_mesh_free.argtypes = [vp]
    L.mglet_create_flowstencils.argtypes = [vp, vp, C.POINTER(vp)]
    L.mglet_flowstencils_size.argtypes = [vp, C.c_int32, C.c_int32, C.POINTER(C.c_int32),
                                          C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    L.mglet_flowstencils_copy.argtypes = [vp, C.c_int32, C.c_int32, vp, vp, vp]
    L.mglet_flowstencils_free.argtypes = [vp]
    L.mglet_gpu_set_partition.argtypes = [vp, vp, C.c_int32, vp, C.c_int32, vp, vp, vp]
    _lib = L
    return L


def fp64_roof(device=0):
    """Measured FP64 issue rates of the device (thread instructions per
    second): {"dfma": .., "dadd": .., "dmul": ..}."""
    out = (C.c_double * 3)()
    _check(load().mglet_gpu_fp64_roof(device, out))
    return {"dfma": out[0], "dadd": out[1], "dmul": out[2]}


def _check(rc):
    if rc != 0:
        raise MgletError(rc, load().mglet_gpu_last_error().decode())


def rk_scheme(name="williamson"):
    rk = abi.RKScheme()
    _check(load().mglet_rk_init(name.encode(), C.byref(rk)))
    return rk


def rk_coeffs(rk, irk):
    v = [C.c_double() for _ in range(4)]
    _check(load().mglet_rk_get_coeffs(C.byref(rk), irk, *[C.byref(x) for x in v]))
    return tuple(x.value for x in v)


def _b(s):
    return None if s is None else s.encode()


class Solver:
    """One GPU context holding a case's fields and solver state."""

    def __init__(self, case, params, device=0):
        L = load()
        self.case = case
        self._desc = case.desc()
        self.params = params
        h = C.c_void_p()
        _check(L.mglet_gpu_create(C.byref(self._desc), C.byref(params), device, C.byref(h)))
        self.h = h
        self.n = L.mglet_gpu_idim3d(h)

    def close(self):
        if getattr(self, "h", None):
            load().mglet_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        _check(load().mglet_gpu_set_field(self.h, name.encode(), a.ctypes.data, a.size))

    def get(self, name, n=None, out=None):
        n = self.n if n is None else n
        a = np.empty(n, dtype=np.float64) if out is None else out
        _check(load().mglet_gpu_get_field(self.h, name.encode(), a.ctypes.data, n))
        return a

    def set_ptr(self, name, ptr, n):
        _check(load().mglet_gpu_set_field(self.h, name.encode(), ptr, n))

    def get_ptr(self, name, ptr, n):
        _check(load().mglet_gpu_get_field(self.h, name.encode(), ptr, n))

    def timeintegrate_flow(self, itstep, ittot, timeph, dt, irk, rk):
        st = abi.StageStats()
        _check(load().mglet_gpu_timeintegrate_flow(self.h, itstep, ittot, timeph, dt, irk,
                                                   C.byref(rk), C.byref(st)))
        return st

    def tstle4(self):
        _check(load().mglet_gpu_tstle4(self.h))

    def rkstep(self, p, dp, rhs, frhs, dtfu):
        _check(load().mglet_gpu_rkstep(self.h, p.encode(), dp.encode(), rhs.encode(), frhs, dtfu))

    def connect(self, ilevel=0, layers=1, v1=None, v2=None, v3=None, s1=None, s2=None, s3=None,
                corners=False, normal=False, forward=0):
        _check(load().mglet_gpu_connect(self.h, ilevel, layers, _b(v1), _b(v2), _b(v3), _b(s1),
                                        _b(s2), _b(s3), int(corners), int(normal), int(forward)))

    def divcal(self, div, fak):
        _check(load().mglet_gpu_divcal(self.h, div.encode(), fak))

    def laplacephi(self, res, phi):
        _check(load().mglet_gpu_laplacephi(self.h, res.encode(), phi.encode()))

    def mgpoisl(self, dt, ittot=1, irk=1):
        st = abi.StageStats()
        _check(load().mglet_gpu_mgpoisl(self.h, dt, ittot, irk, C.byref(st)))
        return st

    def bound_flow(self, ilevel=0):
        _check(load().mglet_gpu_bound_flow(self.h, ilevel))

    def set_buffer(self, name, igrid, iface, plane):
        """Boundary buffer of U, V or W on face iface of grid igrid (1-based):
        a (kk,jj), (kk,ii) or (jj,ii) plane, first index fastest."""
        a = np.ascontiguousarray(plane, dtype=np.float64).ravel(order="F")
        _check(load().mglet_gpu_set_buffer(self.h, name.encode(), igrid, iface,
                                           a.ctypes.data_as(C.c_void_p), a.size))

    def set_bc_real(self, igrid, iface, value):
        _check(load().mglet_gpu_set_bc_real(self.h, igrid, iface, value))

    def get_buffer(self, name, igrid, iface, shape):
        """The boundary buffer plane of a field, shape (first, second) index."""
        a = np.zeros(int(np.prod(shape)), dtype=np.float64)
        _check(load().mglet_gpu_get_buffer(self.h, name.encode(), igrid, iface,
                                           a.ctypes.data_as(C.c_void_p), a.size))
        return a.reshape(shape, order="F")

    # -- grid hierarchies ---------------------------------------------------
    def set_hierarchy(self, iparent, position):
        ip = np.ascontiguousarray(iparent, dtype=np.int32)
        ps = np.ascontiguousarray(position, dtype=np.int32)
        _check(load().mglet_gpu_set_hierarchy(self.h, ip.ctypes.data_as(C.c_void_p),
                                              ps.ctypes.data_as(C.c_void_p)))

    def parent(self, ilevel, v=None, s=(), normal=False):
        v = list(v) if v else [None] * 3
        s = list(s) + [None] * (3 - len(s))
        e = lambda n: None if n is None else n.encode()
        _check(load().mglet_gpu_parent(self.h, ilevel, *[e(n) for n in v + s], int(normal)))

    def ftoc(self, ilevel, ff, fc, flag):
        _check(load().mglet_gpu_ftoc(self.h, ilevel, ff.encode(), fc.encode(), flag.encode()))

    def ftoc_multiple(self, ilevel, v=None, s=()):
        v = list(v) if v else [None] * 3
        s = list(s) + [None] * (3 - len(s))
        e = lambda n: None if n is None else n.encode()
        _check(load().mglet_gpu_ftoc_multiple(self.h, ilevel, *[e(n) for n in v + s]))

    def ctof(self, ilevel, ff, fc):
        _check(load().mglet_gpu_ctof(self.h, ilevel, ff.encode(), fc.encode()))

    def set_scalars(self, prmol, kayscrawford=None, source=None, prturb=1.0):
        n = len(prmol)
        pr = np.ascontiguousarray(prmol, dtype=np.float64)
        kc = np.ascontiguousarray(kayscrawford if kayscrawford is not None else [0] * n, dtype=np.int32)
        so = np.ascontiguousarray(source if source is not None else [0.0] * n, dtype=np.float64)
        _check(load().mglet_gpu_set_scalars(self.h, n, pr.ctypes.data_as(C.c_void_p),
                                            kc.ctypes.data_as(C.c_void_p), so.ctypes.data_as(C.c_void_p),
                                            prturb))

    def timeintegrate_scalar(self, dt, irk, rk):
        _check(load().mglet_gpu_timeintegrate_scalar(self.h, dt, irk, C.byref(rk)))

    def set_buoyancy(self, gravity, beta, iscalar=1):
        g = np.ascontiguousarray(gravity, dtype=np.float64)
        _check(load().mglet_gpu_set_buoyancy(self.h, g.ctypes.data_as(C.c_void_p), beta, iscalar))

    def set_coriolis(self, omega):
        om = np.ascontiguousarray(omega, dtype=np.float64)
        _check(load().mglet_gpu_set_coriolis(self.h, om.ctypes.data_as(C.c_void_p)))

    def add_scalar_source(self, isca, value, field=None):
        _check(load().mglet_gpu_add_scalar_source(self.h, isca, field.encode() if field else None, value))

    def set_scalar_bc(self, igrid, iface, kind, types=()):
        ty = np.ascontiguousarray(list(types) + [0] * 9, dtype=np.int32)
        _check(load().mglet_gpu_set_scalar_bc(self.h, igrid, iface, kind, ty.ctypes.data_as(C.c_void_p)))

    def set_lesmodel(self, model, cm=-1.0):
        """0 none, 1 smagorinsky, 2 wale, 5 sigma; cm < 0 takes the model's default."""
        _check(load().mglet_gpu_set_lesmodel(self.h, model, cm))

    def set_body_force(self, fx, fy, fz):
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in (fx, fy, fz)]
        _check(load().mglet_gpu_set_body_force(self.h, *[x.ctypes.data_as(C.c_void_p) for x in a],
                                               a[0].size))

    def adjoint_rk_stage(self, irk, dt, rk):
        _check(load().mglet_gpu_adjoint_rk_stage(self.h, irk, dt, C.byref(rk)))

    def energy_gradient(self, nsteps, ncheck, dt, rk):
        """J (the itinfo kinetic energy after nsteps steps) and dJ/d(body
        force) as three flat arrays."""
        e = C.c_double(0.0)
        _check(load().mglet_gpu_energy_gradient(self.h, nsteps, ncheck, dt, C.byref(rk), C.byref(e)))
        return e.value, tuple(self.get(n) for n in ("GFX", "GFY", "GFZ"))

    def par_ftoc_norm(self, ilevel, v1="U", v2="V", v3="W", sum=False):
        _check(load().mglet_gpu_par_ftoc_norm(self.h, ilevel, v1.encode(), v2.encode(), v3.encode(),
                                              int(sum)))

    def bound_pressure(self, ilevel, dp, with_bp=False):
        _check(load().mglet_gpu_bound_pressure(self.h, ilevel, dp.encode(), int(with_bp)))

    def set_stencils(self, igrid, comp, ncells, xpoli, xpolr, xpolrvel=None):
        xi = np.ascontiguousarray(xpoli, dtype=np.int64)
        xr = np.ascontiguousarray(xpolr, dtype=np.float64)
        xv = np.ascontiguousarray(xpolrvel if xpolrvel is not None else [], dtype=np.float64)
        _check(load().mglet_gpu_set_stencils(self.h, igrid, comp, ncells,
                                             xi.ctypes.data_as(C.c_void_p), xi.size,
                                             xr.ctypes.data_as(C.c_void_p), xr.size,
                                             xv.ctypes.data_as(C.c_void_p), xv.size))

    def set_ghostcell(self):
        _check(load().mglet_gpu_set_ghostcell(self.h))

    def setpointvalues(self, comp_new=True):
        _check(load().mglet_gpu_setpointvalues(self.h, 1 if comp_new else 0))

    def gc_mode(self, mode):
        """'I' setibvalues, 'R' getibvalues, 'M' maskbp (the oracle's names)."""
        fn = {"I": "mglet_gpu_setibvalues", "R": "mglet_gpu_getibvalues",
              "M": "mglet_gpu_maskbp"}[mode]
        _check(getattr(load(), fn)(self.h))

    def itinfo(self, dt):
        out = abi.ItInfo()
        rc = load().mglet_gpu_itinfo(self.h, dt, C.byref(out))
        if rc not in (0, abi.MGLET_ERR_EXPLODED):
            _check(rc)
        return out

    def synchronize(self):
        _check(load().mglet_gpu_synchronize(self.h))

    @property
    def stream(self):
        """cudaStream_t (as an int) the context issues its work on."""
        return load().mglet_gpu_stream(self.h)

    def profile(self, enable=True):
        _check(load().mglet_gpu_profile(self.h, int(enable)))

    def profile_names(self):
        buf = C.create_string_buffer(4096)
        _check(load().mglet_gpu_profile_names(self.h, buf, 4096))
        return [x for x in buf.value.decode().split(",") if x]

    def profile_get(self, kernel):
        ms = C.c_double()
        n = C.c_int64()
        _check(load().mglet_gpu_profile_get(self.h, kernel.encode(), C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def set_partition(self, part, exchange):
        """A rank's share of a partitioned run (dist.Partition) with its
        exchange function (dist.TorchExchange or any EXCHANGE_FN owner)."""
        self._part = (part, exchange)
        halo = np.ascontiguousarray(part.halo, dtype=np.int32)
        send = np.ascontiguousarray(part.send, dtype=np.int32)
        recv = np.ascontiguousarray(part.recv, dtype=np.int32)
        self._part_arrays = (halo, send, recv)
        fnp = C.cast(exchange.fn, C.c_void_p)
        _check(load().mglet_gpu_set_partition(self.h, halo.ctypes.data, len(send), send.ctypes.data,
                                              len(recv), recv.ctypes.data, fnp, None))

    def tuning(self):
        buf = C.create_string_buffer(2048)
        _check(load().mglet_gpu_tuning(self.h, buf, len(buf)))
        return buf.value.decode()

    def test_wait_timeout(self):
        _check(load().mglet_gpu_test_wait_timeout(self.h))

    def set_scastencils(self, igrid, xpoli, xpolr, xpolrvel):
        """Scalar ghost-cell list of grid igrid (1-based): per cell 9 integers
        and 8 reals (see mglet_gpu_set_scastencils)."""
        xi = np.ascontiguousarray(xpoli, dtype=np.int64)
        xr = np.ascontiguousarray(xpolr, dtype=np.float64)
        xv = np.ascontiguousarray(xpolrvel, dtype=np.float64)
        _check(load().mglet_gpu_set_scastencils(self.h, igrid, len(xi) // 9, xi.ctypes.data_as(C.c_void_p),
                                                xr.ctypes.data_as(C.c_void_p), xv.ctypes.data_as(C.c_void_p)))

    def set_scalar_geometry(self, isca, flags, values):
        """Per body the scalar's condition: flag 0 fixed value, 1 fixed flux."""
        fl = np.ascontiguousarray(flags, dtype=np.int32)
        va = np.ascontiguousarray(values, dtype=np.float64)
        _check(load().mglet_gpu_set_scalar_geometry(self.h, isca, len(fl), fl.ctypes.data_as(C.c_void_p),
                                                    va.ctypes.data_as(C.c_void_p)))

    def test_barrier_timeout(self):
        _check(load().mglet_gpu_test_barrier_timeout(self.h))

    def force_variant(self, kernel, variant):
        _check(load().mglet_gpu_force_variant(self.h, kernel.encode(), variant))

    @property
    def launches(self):
        return load().mglet_gpu_kernel_launches(self.h)


def create_scastencils(case, geo, arealist, bodyid):
    """The scalar ghost-cell lists of every grid (mglet_create_scastencils,
    host code, no device needed) from the blocking fields (geometry.block)
    and, per cut cell, its interface area and body id.  Returns per grid
    (xpoli, xpolr, xpolrvel), the layout mglet_gpu_set_scastencils takes."""
    L = load()
    keep = {"bp": np.ascontiguousarray(geo["bp"], dtype=np.float64),
            "bzelltyp": np.ascontiguousarray(geo["bzelltyp"], dtype=np.int32),
            "icells": np.ascontiguousarray(geo["icells"], dtype=np.int32),
            "nvecs": np.ascontiguousarray(geo["nvecs"], dtype=np.float64).reshape(-1),
            "arealist": np.ascontiguousarray(arealist, dtype=np.float64),
            "bodyid": np.ascontiguousarray(bodyid, dtype=np.int32)}
    g = abi.ScaGeometry()
    for n, a in keep.items():
        setattr(g, n, a.ctypes.data_as(C.c_void_p))
    desc = case.desc()
    h = C.c_void_p()
    _check(L.mglet_create_scastencils(C.byref(desc), C.byref(g), C.byref(h)))
    out = []
    try:
        for ig in range(1, case.ngrid + 1):
            n = C.c_int32()
            _check(L.mglet_scastencils_size(h, ig, C.byref(n)))
            xi = np.zeros(9 * n.value, dtype=np.int64)
            xr, xv = np.zeros(8 * n.value), np.zeros(8 * n.value)
            _check(L.mglet_scastencils_copy(h, ig, xi.ctypes.data_as(C.c_void_p), xr.ctypes.data_as(C.c_void_p),
                                            xv.ctypes.data_as(C.c_void_p)))
            out.append((xi, xr, xv))
    finally:
        L.mglet_scastencils_free(h)
    return out


def create_flowstencils(case, geo):
    """The ghost-cell stencil lists of every grid from the blocking fields
    (geometry.block): mglet_create_flowstencils, host code, no device needed.
    Returns lists[g] = {1: (ncells, xpoli, xpolr, xpolrvel), 2: .., 3: ..,
    4: (ncells, xpoli, xpolr)}, the layout mglet_gpu_set_stencils takes."""
    L = load()
    f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    keep = {n: f64(geo[n]) for n in ("bp", "bu", "bv", "bw", "areau", "areav", "areaw")}
    keep["bzelltyp"] = np.ascontiguousarray(geo["bzelltyp"], dtype=np.int32)
    keep["icells"] = np.ascontiguousarray(geo["icells"], dtype=np.int32)
    keep["nvecs"] = f64(geo["nvecs"]).reshape(-1)
    keep["ucell"] = f64(geo["ucell"]).reshape(-1)
    g = abi.IbGeometry()
    for n, a in keep.items():
        setattr(g, n, a.ctypes.data_as(C.c_void_p))
    desc = case.desc()
    h = C.c_void_p()
    _check(L.mglet_create_flowstencils(C.byref(desc), C.byref(g), C.byref(h)))
    out = []
    try:
        for ig in range(1, case.ngrid + 1):
            gl = {}
            for comp in (1, 2, 3, 4):
                n = C.c_int32()
                nxi, nxr = C.c_int64(), C.c_int64()
                _check(L.mglet_flowstencils_size(h, ig, comp, C.byref(n), C.byref(nxi), C.byref(nxr)))
                xi = np.zeros(nxi.value, dtype=np.int64)
                xr = np.zeros(nxr.value)
                xv = np.zeros(nxr.value) if comp < 4 else None
                _check(L.mglet_flowstencils_copy(h, ig, comp, xi.ctypes.data_as(C.c_void_p),
                                                 xr.ctypes.data_as(C.c_void_p),
                                                 xv.ctypes.data_as(C.c_void_p) if xv is not None
                                                 else None))
                gl[comp] = (n.value, xi, xr, xv) if comp < 4 else (n.value, xi, xr)
            out.append(gl)
    finally:
        L.mglet_flowstencils_free(h)
    return out
