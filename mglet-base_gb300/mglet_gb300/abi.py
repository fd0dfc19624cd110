"""ctypes mirror of include/mglet_gpu.h (structs and status codes).

The same structs describe a case to the GPU library and, in the tests, to
the CPU oracle, so both receive byte-identical grid descriptions.
"""
import ctypes as C

MGLET_OK = 0
MGLET_ERR_ARG = 1
MGLET_ERR_UNSUPPORTED = 2
MGLET_ERR_CUDA = 3
MGLET_ERR_NAME = 4
MGLET_ERR_SIZE = 5
MGLET_ERR_EXPLODED = 6
MGLET_ERR_NOMEM = 7

BC_FIX, BC_OP1, BC_NOS, BC_SLI, BC_CON, BC_PAR, BC_CO1 = 2, 3, 5, 6, 7, 8, 19

PSOLVER_SIP, PSOLVER_SOR, PSOLVER_CLASSIC = 0, 1, 2
FORM_PLAIN, FORM_MIXED, FORM_PLAIN_FMA = 0, 1, 2

_i32p = C.POINTER(C.c_int32)
_f64p = C.POINTER(C.c_double)


class GridDesc(C.Structure):
    _fields_ = [
        ("ngrid", C.c_int32),
        ("mgdims", _i32p),
        ("level", _i32p),
        ("bctype", _i32p),
        ("nbrgrid", _i32p),
        ("gradpflag", _i32p),
        ("x", _f64p), ("y", _f64p), ("z", _f64p),
        ("dx", _f64p), ("dy", _f64p), ("dz", _f64p),
        ("ddx", _f64p), ("ddy", _f64p), ("ddz", _f64p),
    ]


class FlowParams(C.Structure):
    _fields_ = [
        ("gmol", C.c_double),
        ("rho", C.c_double),
        ("gradp", C.c_double * 3),
        ("psolver", C.c_int32),
        ("ninner", C.c_int32),
        ("nouter", C.c_int32),
        ("nouter_min", C.c_int32),
        ("epcorr", C.c_double),
        ("omega", C.c_double),
        ("form", C.c_int32),
        ("reserved", C.c_int32),
    ]


class RKScheme(C.Structure):
    _fields_ = [
        ("nrk", C.c_int32),
        ("reserved", C.c_int32),
        ("cflmax", C.c_double),
        ("a", C.c_double * 6),
        ("b", C.c_double * 6),
        ("c", C.c_double * 6),
    ]


class StageStats(C.Structure):
    _fields_ = [
        ("ipc", C.c_int32),
        ("nouter_done", C.c_int32),
        ("maxrhs", C.c_double),
        ("prefak", C.c_double),
    ]


class ItInfo(C.Structure):
    _fields_ = [
        ("cflmax", C.c_double),
        ("divmax", C.c_double),
        ("energy", C.c_double),
        ("exploded", C.c_int32),
        ("reserved", C.c_int32),
    ]


class IbGeometry(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("bp", "bu", "bv", "bw", "areau", "areav", "areaw",
                                          "bzelltyp", "icells", "nvecs", "ucell")]


class ScaGeometry(C.Structure):
    """mglet_sca_geometry: the inputs of create_scastencils."""
    _fields_ = [(n, C.c_void_p) for n in ("bp", "bzelltyp", "icells", "nvecs", "arealist", "bodyid")]


def make_flow_params(gmol, rho=1.0, gradp=(0.0, 0.0, 0.0), psolver=PSOLVER_SIP, ninner=5,
                     nouter=9, nouter_min=0, epcorr=1e-10, omega=1.1, form=FORM_PLAIN):
    p = FlowParams()
    p.gmol = gmol
    p.rho = rho
    for q in range(3):
        p.gradp[q] = gradp[q]
    p.psolver = psolver
    p.ninner = ninner
    p.nouter = nouter
    p.nouter_min = nouter_min
    p.epcorr = epcorr
    p.omega = omega
    p.form = form
    return p
