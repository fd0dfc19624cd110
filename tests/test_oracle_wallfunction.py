"""The Werner-Wengle wall function of NOS faces in the oracle (no GPU).

tstle4_diff calls swcle3d (src/flow/tstle4_mod.F90:315-316, 1756-1844),
which subtracts tauwin(u, dds)/rho/dds (src/flow/wernerwengle_mod.F90:64-87,
constants :13-28) from the two tangential components in the layer next to
each NOS (code 5) wall, over the face's rows 2..n-1.  kon and diff treat NOS
and SLI alike (only CON and OP1 change their ranges), so tstle4 on a case
with NOS walls minus tstle4 on the same case relabelled SLI is the wall
term.  It is pinned against a loop transcription in Python scalars
(math.pow is C's pow, as the reference's real ** real), in the laminar
sublayer, the fully turbulent regime and a mix of both.
"""
import dataclasses
import math

import numpy as np
import pytest

from mglet_gb300 import abi, cases

ALL_NOS = {f: abi.BC_NOS for f in range(1, 7)}


def ww_constants(gmol, rho):
    """init_wernerwengle (wernerwengle_mod.F90:13-28)."""
    cwa, cwb = 8.3, 1.0 / 7.0
    cpo1, cpo2 = 1.0 - cwb, 1.0 + cwb
    return dict(
        gmol=gmol, rho=rho, cwb=cwb,
        cpo4=cpo2 / cwa * math.pow(gmol / rho, cwb),
        cpo5=0.5 * cpo1 * math.pow(cwa, cpo2 / cpo1) * math.pow(gmol / rho, cpo2),
        cpo6=0.5 * gmol / rho * math.pow(cwa, 2.0 / cpo1),
        cpo8=2.0 / cpo2)


def swcle3d_one(q, dds, u):
    """tauwin(u, dds)/rho/dds; also returns whether the point is turbulent."""
    vz = math.copysign(1.0, u)
    un = abs(u)
    if un >= q["cpo6"] / dds:
        ddsb = math.pow(dds, -q["cwb"])
        tau = vz * q["rho"] * math.pow(ddsb * (q["cpo4"] * un + q["cpo5"] / dds), q["cpo8"])
        return tau / q["rho"] / dds, True
    return vz * 2.0 * q["gmol"] * un / dds / q["rho"] / dds, False


def wall_terms(case, q, u, v, w):
    """swcle3d over every grid: the values 0 - term - term ... in the
    reference's face order, and a mask of the points written."""
    sh = (case.ngrid, case.ii, case.jj, case.kk)
    U, V, W = (a.reshape(sh) for a in (u, v, w))
    E = {n: np.zeros(sh) for n in "UVW"}
    M = {n: np.zeros(sh, dtype=bool) for n in "UVW"}
    nturb = nlam = 0
    kk, jj, ii = case.kk, case.jj, case.ii
    for g in range(case.ngrid):
        off = g * ii
        ddx = case.ddx[off:off + ii]
        ddy = case.ddy[g * jj:(g + 1) * jj]
        ddz = case.ddz[g * kk:(g + 1) * kk]
        bc = case.bctype[g]
        todo = []
        for side, f in ((0, 0), (1, 1)):          # front i = 3, back i = ii-2
            if bc[f] == abi.BC_NOS:
                i = ii - 2 if side else 3
                todo += [(c, (i - 1, j - 1, k - 1), ddx[i - 1]) for j in range(2, jj) for k in range(2, kk)
                         for c in "VW"]
        for side, f in ((0, 2), (1, 3)):          # right j = 3, left j = jj-2
            if bc[f] == abi.BC_NOS:
                j = jj - 2 if side else 3
                todo += [(c, (i - 1, j - 1, k - 1), ddy[j - 1]) for i in range(2, ii) for k in range(2, kk)
                         for c in "UW"]
        for side, f in ((0, 4), (1, 5)):          # bottom k = 3, top k = kk-2
            if bc[f] == abi.BC_NOS:
                k = kk - 2 if side else 3
                todo += [(c, (i - 1, j - 1, k - 1), ddz[k - 1]) for i in range(2, ii) for j in range(2, jj)
                         for c in "UV"]
        src = {"U": U, "V": V, "W": W}
        for c, (i, j, k), dds in todo:
            t, turb = swcle3d_one(q, float(dds), float(src[c][g, i, j, k]))
            E[c][g, i, j, k] = E[c][g, i, j, k] - t
            M[c][g, i, j, k] = True
            nturb += turb
            nlam += not turb
    return ({n: E[n].ravel() for n in "UVW"}, {n: M[n].ravel() for n in "UVW"}, nturb, nlam)


def wall_case(walls=ALL_NOS):
    return cases.periodic_box(2, 2, 1, n=8, length=(2.0, 2.0, 1.0), walls=walls)


def relabel_sli(case):
    return dataclasses.replace(case, bctype=np.where(case.bctype == abi.BC_NOS, abi.BC_SLI,
                                                     case.bctype).astype(np.int32))


def wall_fields(case, amplitude, seed, gmol):
    rng = np.random.default_rng(seed)
    f = {n: amplitude * rng.standard_normal(case.idim3d) for n in "UVWP"}
    f["G"] = np.full(case.idim3d, gmol)
    return f


@pytest.mark.parametrize("gmol,amplitude,regime", [(1e-2, 0.3, "laminar"), (1e-5, 1.0, "turbulent"),
                                                   (1e-3, 1.0, "both")])
def test_wall_function_matches_loop_transcription(oracle_lib, gmol, amplitude, regime):
    case = wall_case()
    prm = abi.make_flow_params(gmol=gmol, epcorr=1e-12, nouter=4, ninner=2, nouter_min=0)
    fields = wall_fields(case, amplitude, 31, gmol)
    o, s = oracle_lib.Oracle(case, prm), oracle_lib.Oracle(relabel_sli(case), prm)
    for x in (o, s):
        for n, a in fields.items():
            x.set(n, a)
        x.tstle4()
    E, M, nturb, nlam = wall_terms(case, ww_constants(gmol, 1.0), fields["U"], fields["V"], fields["W"])
    assert {"laminar": nturb == 0 and nlam > 0, "turbulent": nlam < 0.01 * nturb,
            "both": nlam > 100 and nturb > 100}[regime], (nturb, nlam)
    for n in "UVW":
        a, b = o.get(n + "O"), s.get(n + "O")
        assert np.array_equal(a[~M[n]], b[~M[n]]), n            # nothing off the wall rows
        rows = M[n] & (b == 0.0)                                 # rows outside the flux ranges
        assert rows.sum() > 0
        assert np.array_equal(a[rows], E[n][rows]), n
        scale = np.abs(a).max()
        assert np.abs(a[M[n]] - (b[M[n]] + E[n][M[n]])).max() <= 1e-13 * scale, n


def test_wall_stage_with_turbulent_wall_function_is_divergence_free(oracle_lib):
    """A stage with the wall function in its turbulent branch: the wall
    shear enters the momentum update only, the projection still leaves the
    field divergence free to the solver residual."""
    case = wall_case({5: abi.BC_NOS, 6: abi.BC_NOS})
    prm = abi.make_flow_params(gmol=1e-5, epcorr=1e-13, nouter=60, ninner=5, nouter_min=0)
    o = oracle_lib.Oracle(case, prm)
    u, v, w, p = cases.taylor_green(case)
    for nm, a in zip("UVWP", (u + 0.5, v, w, p)):
        o.set(nm, a)
    o.connect(0, 2, "U", "V", "W", "P", corners=True)
    st = o.timeintegrate_flow(1, 1, 0.0, 1e-2, 1, oracle_lib.rk_scheme("williamson"))
    res = st.maxrhs / st.prefak
    assert res < 1e-9
    assert o.itinfo(1e-2).divmax <= 1.01 * res + 1e-13


def test_body_force_enters_tstle4(oracle_lib):
    """The steady body force (a source term the reference does not have) is
    added to uo, vo, wo over the flux ranges of tstle4, after gradp: on a
    fluid at rest it is the whole of uo, vo, wo there, and nothing outside."""
    case = cases.periodic_box(2, 1, 1, n=8, length=(2.0, 1.0, 1.0))
    o = oracle_lib.Oracle(case, abi.make_flow_params(gmol=1e-2, epcorr=1e-12, nouter=4, ninner=2))
    rng = np.random.default_rng(12)
    f = [rng.standard_normal(case.idim3d) for _ in range(3)]
    for n in "UVWP":
        o.set(n, case.zeros())
    o.set_body_force(*f)
    o.tstle4()
    inner = np.zeros((case.ngrid, case.ii, case.jj, case.kk), dtype=bool)
    inner[:, 2:-2, 2:-2, 2:-2] = True       # every face CON: 3..n-2 for every component
    inner = inner.ravel()
    for n, fv in zip(("UO", "VO", "WO"), f):
        a = o.get(n)
        assert np.array_equal(a[inner], fv[inner]), n
        assert not np.any(a[~inner]), n
