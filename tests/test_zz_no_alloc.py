"""The allocation-free divergence maximum (mglet_gpu_divmax_noalloc).

Callers whose device memory belongs to another runtime (for instance an
OpenMP-offload Fortran build that maps the fields itself) or that must not
let cudaMalloc/cudaFree synchronise the device inside the time loop hand the
library raw device pointers; this entry point then computes itinfo's
divmax with a static device scratch array and allocates nothing.  The test
calls it through the C ABI on device buffers owned by the caller (torch
tensors here) and checks it against the context-based mglet_gpu_itinfo,
twice in a row, on a uniform tiling and on one whose cell widths differ from
grid to grid (so that a wrong per-grid offset into rddx/rddy/rddz shows),
checks that a call leaves the device's free memory unchanged, plus the size
limit.  This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

from mglet_gb300 import abi, cases

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _fields(case, seed):
    u, v, w, p = cases.taylor_green(case)
    return cases.add_noise(case, (u, v, w), amplitude=5e-2, seed=seed) + [p]


def _ref_divmax(gpu_lib, case, fields):
    s = gpu_lib.Solver(case, abi.make_flow_params(gmol=1e-3))
    for nm, a in zip("UVWP", fields):
        s.set(nm, a)
    s.connect(0, 2, "U", "V", "W", "P", corners=True)
    out = {nm: s.get(nm) for nm in "UVW"}
    d = s.itinfo(1e-3).divmax
    s.close()
    return d, out


def _cases():
    # uniform spacing, and the same tiling with cell widths that differ per
    # grid and axis
    return [cases.periodic_box(3, 2, 2, n=12), cases.stretch(cases.periodic_box(3, 2, 2, n=12))]


@pytest.mark.parametrize("which", [0, 1], ids=["uniform", "stretched"])
def test_divmax_noalloc_matches_itinfo(gpu_lib, which):
    import torch
    lib = gpu_lib.load()
    case = _cases()[which]
    if which == 1:
        # the per-grid spacing really differs, so the offsets matter
        assert not np.allclose(case.ddx[:case.ii], case.ddx[case.ii:2 * case.ii])
    dev = torch.device("cuda", 0)
    rdd = [torch.from_numpy(1.0 / a).to(dev) for a in (case.ddx, case.ddy, case.ddz)]
    out = torch.full((1,), -1.0, dtype=torch.float64, device=dev)
    for call, seed in enumerate((42, 7)):
        ref, flds = _ref_divmax(gpu_lib, case, _fields(case, seed))
        u, v, w = (torch.from_numpy(flds[nm]).to(dev) for nm in "UVW")
        torch.cuda.synchronize()
        rc = lib.mglet_gpu_divmax_noalloc(u.data_ptr(), v.data_ptr(), w.data_ptr(), case.ngrid,
                                          case.kk, case.jj, case.ii, rdd[0].data_ptr(),
                                          rdd[1].data_ptr(), rdd[2].data_ptr(), out.data_ptr(),
                                          None)
        assert rc == 0, lib.mglet_gpu_last_error().decode()
        torch.cuda.synchronize()
        got = float(out.item())
        assert ref > 0
        assert abs(got - ref) <= RTOL * ref, (call, got, ref)


def test_divmax_noalloc_allocates_nothing(gpu_lib):
    """After a first call (which looks up the scratch array's address), a
    further call changes neither the device's free memory nor torch's
    allocation count."""
    import torch
    lib = gpu_lib.load()
    case = cases.periodic_box(2, 2, 2, n=8)
    dev = torch.device("cuda", 0)
    u, v, w = (torch.from_numpy(a).to(dev) for a in _fields(case, 3)[:3])
    rdd = [torch.from_numpy(1.0 / a).to(dev) for a in (case.ddx, case.ddy, case.ddz)]
    out = torch.zeros(1, dtype=torch.float64, device=dev)

    def call():
        rc = lib.mglet_gpu_divmax_noalloc(u.data_ptr(), v.data_ptr(), w.data_ptr(), case.ngrid,
                                          case.kk, case.jj, case.ii, rdd[0].data_ptr(),
                                          rdd[1].data_ptr(), rdd[2].data_ptr(), out.data_ptr(),
                                          None)
        assert rc == 0, lib.mglet_gpu_last_error().decode()
        torch.cuda.synchronize()

    call()
    free0, _ = torch.cuda.mem_get_info(dev)
    alloc0 = torch.cuda.memory_allocated(dev)
    call()
    call()
    free1, _ = torch.cuda.mem_get_info(dev)
    assert free1 == free0
    assert torch.cuda.memory_allocated(dev) == alloc0


def test_divmax_noalloc_rejects_too_many_grids(gpu_lib):
    lib = gpu_lib.load()
    dummy = C.c_void_p(16)   # never dereferenced: the size check comes first
    rc = lib.mglet_gpu_divmax_noalloc(dummy, dummy, dummy, 65537, 28, 28, 28, dummy, dummy,
                                      dummy, dummy, None)
    assert rc == abi.MGLET_ERR_SIZE
    assert "MGLET_NOALLOC_MAX_GRIDS" in lib.mglet_gpu_last_error().decode()
