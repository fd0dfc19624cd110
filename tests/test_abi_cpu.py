"""The C-ABI library loads and exports every symbol of include/mglet_gpu.h,
and its host-only entry points agree with the oracle -- no GPU needed."""
import ctypes as C
import os
import re

import pytest

from mglet_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header_symbols():
    src = open(os.path.join(ROOT, "include", "mglet_gpu.h")).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w]+\*?\s+\**(mglet_\w+)\s*\(", src, re.M)))


@pytest.fixture(scope="module")
def lib():
    from mglet_gb300 import build, gpu
    build.build()
    return gpu.load()


def test_exports_every_header_symbol(lib):
    from mglet_gb300 import gpu
    syms = _header_symbols()
    assert len(syms) >= 19
    assert set(gpu.EXPORTS) <= set(syms)
    for s in syms:
        assert hasattr(lib, s), s
    assert lib.mglet_gpu_abi_version() == 1


def test_struct_sizes_match_header():
    # the layouts the C compiler gives these structs (x86-64 / aarch64 LP64)
    assert C.sizeof(abi.GridDesc) == 4 + 4 + 5 * 8 + 9 * 8
    assert C.sizeof(abi.FlowParams) == 8 + 8 + 24 + 4 * 4 + 8 + 8 + 4 + 4
    assert C.sizeof(abi.RKScheme) == 4 + 4 + 8 + 18 * 8
    assert C.sizeof(abi.StageStats) == 4 + 4 + 8 + 8
    assert C.sizeof(abi.ItInfo) == 3 * 8 + 4 + 4


@pytest.mark.parametrize("name", ["williamson", "berland", "carpenter", "bernardini"])
def test_rk_init_matches_oracle(lib, oracle_lib, name):
    from mglet_gb300 import gpu
    a = gpu.rk_scheme(name)
    b = oracle_lib.rk_scheme(name)
    assert a.nrk == b.nrk
    assert a.cflmax == b.cflmax
    for q in range(6):
        assert a.a[q] == b.a[q] and a.b[q] == b.b[q] and a.c[q] == b.c[q]
    for irk in range(1, a.nrk + 1):
        assert gpu.rk_coeffs(a, irk) == oracle_lib.rk_coeffs(b, irk)


def test_rk_init_rejects_unknown(lib):
    from mglet_gb300 import gpu
    with pytest.raises(gpu.MgletError) as e:
        gpu.rk_scheme("euler")
    assert e.value.code == abi.MGLET_ERR_ARG


def test_create_fails_loudly_without_usable_device(lib):
    """No silent CPU fallback: creating a context either succeeds on a GPU
    or reports an error (here: no device, or a bad device index)."""
    from mglet_gb300 import cases, gpu
    import torch
    case = cases.periodic_box(1, 1, 1, n=8)
    prm = abi.make_flow_params(gmol=1e-3)
    dev = 0 if not torch.cuda.is_available() else 10_000
    with pytest.raises(gpu.MgletError) as e:
        gpu.Solver(case, prm, device=dev)
    assert e.value.code in (abi.MGLET_ERR_CUDA, abi.MGLET_ERR_ARG)
