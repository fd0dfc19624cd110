"""Grid hierarchies with the ghost-cell IB in the oracle (no GPU).

* gc_restrict (src/ib/gc_restrict_mod.F90): with the ghost-cell IB, ftoc's
  P and R restrictions weigh the fine cells by BP (P: BP-weighted volume
  mean, 0 where all eight are blocked; R: BP-weighted sum over the full
  coarse volume); U, V, W and S keep the no-IB means.  Pinned against a
  numpy transcription of restrict_p / restrict_r.
* par_ftoc_norm (src/ib/par_ftoc_mod.F90): the face-normal velocity of each
  PAR face, area-averaged (or summed) over 2x2 fine faces, written into the
  parent (inside it, or onto its boundary face and then also onto the
  neighbour across that face).  Pinned against a numpy transcription of
  pack_single / unpack_single with the destinations of init_par_ftoc, on
  full refinements (every PAR on a coarse face) and single fine grids
  (PAR faces inside the parent).
* The multi-level ghost-cell schedule (setibvalues with ftoc and
  par_ftoc_norm between the level sweeps, setpointvalues and setsdivfield
  per level) runs inside the multi-level stage, whose projection leaves
  every grid divergence free to the solver residual.
"""
import numpy as np
import pytest

from mglet_gb300 import abi, cases
from test_oracle_levels import _fine, _g1, _g3, prepare_levels


def _prm(**kw):
    base = dict(gmol=1e-2, epcorr=1e-12, nouter=4, ninner=2, nouter_min=0)
    base.update(kw)
    return abi.make_flow_params(**base)


def gc_hierarchy(octants=None, body=True, seed=5):
    case = cases.refined_box(2, 2, 2, n=8, refine=(1,), octants=octants)
    fine = _fine(case)
    bp, lists = cases.block_body(case, (5, 5, 5), (7, 6, 7), seed=seed,
                                 grids=fine if body else [])
    return case, bp, lists


def load_gc(s, case, bp, lists, fields=None):
    s.set_hierarchy(case.iparent, case.position)
    for nm, a in (fields or {}).items():
        s.set(nm, a)
    s.set("BP", bp)
    for g, gl in enumerate(lists):
        for comp in (1, 2, 3):
            n, xi, xr, xv = gl[comp]
            s.set_stencils(g + 1, comp, n, xi, xr, xv)
        n, fi, fr = gl[4]
        s.set_stencils(g + 1, 4, n, fi, fr)
    s.set_ghostcell()


def _gc_restrict_ref(case, ff, fc, bp, flag):
    kk, jj, ii = case.kk, case.jj, case.ii
    out = fc.copy()
    for g in _fine(case):
        Fv, B = _g3(case, ff, g), _g3(case, bp, g)
        C3 = _g3(case, out, case.iparent[g] - 1)
        ddx, ddy, ddz = (_g1(case.ddx, g, ii), _g1(case.ddy, g, jj), _g1(case.ddz, g, kk))
        ipos, jpos, kpos = case.position[g]
        for i in range(3, ii - 2, 2):
            for j in range(3, jj - 2, 2):
                for k in range(3, kk - 2, 2):
                    cols = [(j, i), (j, i + 1), (j + 1, i), (j + 1, i + 1)]
                    if flag == "P":
                        vol = {(c, kq): B[c[1] - 1, c[0] - 1, kq - 1] * ddz[kq - 1] * ddy[c[0] - 1] * ddx[c[1] - 1]
                               for c in cols for kq in (k, k + 1)}
                        pv = {key: Fv[key[0][1] - 1, key[0][0] - 1, key[1] - 1] * v for key, v in vol.items()}
                        order = [(c, k) for c in cols] + [(c, k + 1) for c in cols]
                        spv = 0.0
                        sv = 0.0
                        for key in order:
                            spv = spv + pv[key]
                        for key in order:
                            sv = sv + vol[key]
                        val = spv / sv if sv > 0.0 else 0.0
                    else:
                        order = [(c, k) for c in cols] + [(c, k + 1) for c in cols]
                        spv = 0.0
                        for (c, kq) in order:
                            spv = spv + (Fv[c[1] - 1, c[0] - 1, kq - 1] * B[c[1] - 1, c[0] - 1, kq - 1]
                                         * ddz[kq - 1] * ddy[c[0] - 1] * ddx[c[1] - 1])
                        val = spv / ((ddx[i - 1] + ddx[i]) * (ddy[j - 1] + ddy[j]) * (ddz[k - 1] + ddz[k]))
                    ic, jc, kc = ipos + (i - 3) // 2, jpos + (j - 3) // 2, kpos + (k - 3) // 2
                    C3[ic - 1, jc - 1, kc - 1] = val
    return out


@pytest.mark.parametrize("flag", ["P", "R"])
def test_gc_restriction(oracle_lib, flag):
    case, bp, lists = gc_hierarchy()
    bp = bp.copy()
    rng = np.random.default_rng(3)
    bp[rng.random(case.idim3d) < 0.3] = 0.0
    for g in _fine(case):                # one block with all eight cells blocked
        _g3(case, bp, g)[2:4, 2:4, 2:4] = 0.0
    o = oracle_lib.Oracle(case, _prm())
    load_gc(o, case, bp, lists)
    ff, fc = rng.standard_normal(case.idim3d), rng.standard_normal(case.idim3d)
    o.set("RHS", ff)
    o.set("RES", fc)
    o.ftoc(2, "RHS", "RES", flag)
    assert np.array_equal(o.get("RES"), _gc_restrict_ref(case, ff, fc, bp, flag))


def test_gc_t_restriction_is_refused(oracle_lib):
    from oracle.binding import OracleError
    case, bp, lists = gc_hierarchy()
    o = oracle_lib.Oracle(case, _prm())
    load_gc(o, case, bp, lists)
    with pytest.raises(OracleError):
        o.ftoc(2, "RHS", "RES", "T")


def _par_ftoc_ref(case, u, v, w, use_sum):
    kk, jj, ii = case.kk, case.jj, case.ii
    sh = (case.ngrid, ii, jj, kk)
    src = [a.reshape(sh) for a in (u, v, w)]
    out = [a.copy() for a in (u, v, w)]
    dst = [a.reshape(sh) for a in out]
    for g in _fine(case):
        p = case.iparent[g] - 1
        ipos, jpos, kpos = case.position[g]
        ddx, ddy, ddz = (_g1(case.ddx, g, ii), _g1(case.ddy, g, jj), _g1(case.ddz, g, kk))
        for iface in range(1, 7):
            if case.bctype[g, iface - 1] != abi.BC_PAR:
                continue
            d = (iface - 1) // 2
            F = src[d][g]
            # the fine face plane and its two in-plane directions, as 2-D arrays
            lay = {1: 1, 2: ii - 3, 3: 1, 4: jj - 3, 5: 1, 6: kk - 3}[iface]   # 0-based
            if d == 0:
                plane, a1, a2 = F[lay, 2:jj - 2, 2:kk - 2], ddy[2:jj - 2], ddz[2:kk - 2]
            elif d == 1:
                plane, a1, a2 = F[2:ii - 2, lay, 2:kk - 2], ddx[2:ii - 2], ddz[2:kk - 2]
            else:
                plane, a1, a2 = F[2:ii - 2, 2:jj - 2, lay], ddx[2:ii - 2], ddy[2:jj - 2]
            f00, f10, f01, f11 = plane[0::2, 0::2], plane[1::2, 0::2], plane[0::2, 1::2], plane[1::2, 1::2]
            b0, b1 = a1[0::2, None], a1[1::2, None]
            c0, c1 = a2[None, 0::2], a2[None, 1::2]
            if use_sum:
                if d == 2:
                    val = f00 + f01 + f10 + f11
                else:
                    val = f00 + f10 + f01 + f11
            else:
                if d == 2:   # (i, j): order (j,i), (j+1,i), (j,i+1), (j+1,i+1)
                    sua = f00 * b0 * c0 + f01 * b0 * c1 + f10 * b1 * c0 + f11 * b1 * c1
                else:        # (j, k) or (i, k): (a,b), (a+1,b), (a,b+1), (a+1,b+1)
                    sua = f00 * b0 * c0 + f10 * b1 * c0 + f01 * b0 * c1 + f11 * b1 * c1
                val = sua / ((b0 + b1) * (c0 + c1))
            pos = (ipos, jpos, kpos)[d]
            nf = (ii, jj, kk)[d]
            odd = iface % 2 == 1
            recv = iface
            one_connect = not nf > (case.ii, case.jj, case.kk)[d]   # parent dims equal here
            if pos == 3 and one_connect:
                if not odd:
                    recv = -1
            elif pos > 3 and odd:
                recv = -1

            def put(gc, ifr):
                lo = [ipos, jpos, kpos]
                hi = [ipos + (ii - 4) // 2 - 1, jpos + (jj - 4) // 2 - 1, kpos + (kk - 4) // 2 - 1]
                if ifr < 0:
                    if odd:
                        lo[d] = hi[d] = (ipos, jpos, kpos)[d] - 1
                    else:
                        lo[d] = hi[d]
                else:
                    lo[d] = hi[d] = 2 if ifr % 2 == 1 else (ii, jj, kk)[d] - 2
                t = [slice(lo[q] - 1, hi[q]) for q in range(3)]
                dst[d][gc][t[0], t[1], t[2]] = val.reshape(
                    [hi[q] - lo[q] + 1 for q in range(3)])

            put(p, recv)
            if recv > 0:
                nb = case.nbrgrid[p, iface - 1]
                if nb > 0:
                    put(nb - 1, iface + 1 if odd else iface - 1)
    return out


@pytest.mark.parametrize("octants", [None, [(0, 0, 0)], [(1, 1, 1)], [(1, 0, 1)]])
@pytest.mark.parametrize("use_sum", [False, True])
def test_par_ftoc_norm(oracle_lib, octants, use_sum):
    case = cases.refined_box(2, 2, 2, n=8, refine=(1,), octants=octants)
    o = oracle_lib.Oracle(case, _prm())
    o.set_hierarchy(case.iparent, case.position)
    rng = np.random.default_rng(4)
    f = {n: rng.standard_normal(case.idim3d) for n in "UVW"}
    for n, a in f.items():
        o.set(n, a)
    o.par_ftoc_norm(2, sum=use_sum)
    ref = _par_ftoc_ref(case, f["U"], f["V"], f["W"], use_sum)
    for n, r in zip("UVW", ref):
        assert np.array_equal(o.get(n), r), n
        assert not np.array_equal(r, f[n]), n          # something was written


def _divmax(o, case):
    o.divcal("RES", 1.0)
    r = o.get("RES").reshape(case.ngrid, case.ii, case.jj, case.kk)[:, 2:-2, 2:-2, 2:-2]
    return np.abs(r).max()


@pytest.mark.parametrize("octants", [None, [(0, 0, 0)]])
@pytest.mark.parametrize("body", [False, True])
def test_multilevel_ghostcell_stage(oracle_lib, octants, body):
    """Three RK stages of the multi-level ghost-cell schedule.  Without a
    body (BP = 1, empty lists) every part of it still runs (setibvalues with
    its level sweeps, ftoc and par_ftoc_norm, setpointvalues per level, the
    BP-weighted restrictions) and the projection leaves every grid
    divergence free to the solver residual.  With the synthetic body the
    random stencils make the Neumann problem incompatible (as they do on
    one level), so that run is checked for finite fields and a solve that
    ran to its iteration limit without breaking down."""
    from oracle.binding import rk_scheme
    case, bp, lists = gc_hierarchy(octants=octants, body=body)
    prm = _prm(epcorr=1e-11, nouter=200 if not body else 20, ninner=5)
    o = oracle_lib.Oracle(case, prm)
    rng = np.random.default_rng(6)
    fields = {n: 0.1 * rng.standard_normal(case.idim3d) for n in "UVW"}
    fields["U"] = fields["U"] + 1.0
    load_gc(o, case, bp, lists, fields)
    for lvl in (1, 2):
        o.connect(lvl, 2, v1="U", v2="V", v3="W", s1="P", corners=True)
    prepare_levels(o, case)
    o.setpointvalues(True)               # flow_mod.F90:83, before the first stage
    rk = rk_scheme("williamson")
    for irk in (1, 2, 3):
        st = o.timeintegrate_flow(1, 1, 0.0, 1e-2, irk, rk)
        for n in ("U", "V", "W", "P", "PWU"):
            assert np.isfinite(o.get(n)).all(), n
        if not body:
            assert st.maxrhs / st.prefak < 1e-11 and st.nouter_done < 200
        else:
            assert st.nouter_done == 20 and np.isfinite(st.maxrhs)
    if not body:
        assert _divmax(o, case) < 1e-9
