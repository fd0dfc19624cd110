"""A channel with a sphere: the multi-level ghost-cell configuration.

Channel 8D x 4D x 4D (D the sphere diameter, at (2D, 2D, 2D)), uniform
inflow u = 1 through FIX front faces, OP1 outflow at the back, periodic in
y and z; level 1 tiles it with 16 x 8 x 8 grids, levels 2 and 3 refine
around the sphere (cases.body_refined), the sphere is blocked from its
signed distance (geometry.block) and its ghost-cell lists are built by the
library (gpu.create_flowstencils).  `scale` shrinks the tiling and the grid
size for bounded samples of the same case.

The set-up runs the reference's initialisation order for a ghost-cell
case: the hierarchy, BP and the lists (create_flowstencils with setsdivfield,
gc_flowstencils_mod.F90:37-100), the FIX buffers (setboundarybuffers),
the initial field, per level connect, then ftoc / connect / parent /
bound_flow and setpointvalues before the first stage
(src/flow/flow_mod.F90:123-172, timeintegration_mod.F90:89-122).
"""
import numpy as np

from . import abi, cases, geometry


class SphereChannel:
    """tiles level-1 grids of n^3 cells, each grid_size wide; the sphere
    (`diameter`) sits a quarter of the channel length downstream of the
    inflow, on the channel axis.  The defaults are the full configuration."""

    def __init__(self, tiles=(16, 8, 8), n=24, grid_size=0.5, diameter=1.0, refine_radii=(1.0, 1.0),
                 re=300.0, samples=8):
        nx, ny, nz = tiles
        d = diameter
        self.length = (nx * grid_size, ny * grid_size, nz * grid_size)
        self.center = (self.length[0] / 4.0, self.length[1] / 2.0, self.length[2] / 2.0)
        self.diameter = d
        self.case = cases.body_refined(nx, ny, nz, n=n, length=self.length, center=self.center,
                                       refine_radii=refine_radii,
                                       walls={1: abi.BC_FIX, 2: abi.BC_OP1})
        self.body = geometry.Sphere(self.center, d / 2.0)
        self.geo = geometry.block(self.case, self.body, samples=samples)
        self.nu = 1.0 * d / re
        self._lists = None

    @property
    def lists(self):
        if self._lists is None:
            from . import gpu
            self._lists = gpu.create_flowstencils(self.case, self.geo)
        return self._lists

    def flow_params(self, form=abi.FORM_PLAIN, **kw):
        base = dict(gmol=self.nu, rho=1.0, epcorr=1e-8, nouter=9, ninner=5, nouter_min=0,
                    form=form)
        base.update(kw)
        return abi.make_flow_params(**base)

    def dt(self, cfl=0.5):
        """The time step of CFL `cfl` at the inflow velocity on the finest
        level (targetcflmax of timeloop_mod.F90:105-121 at the start)."""
        return cfl * float(self.case.ddx.min()) / 1.0

    def levels(self):
        return range(int(self.case.level.min()), int(self.case.level.max()) + 1)

    def setup(self, s):
        """Loads the case into a solver (the GPU Solver, or any object with
        the same calls) and runs the steps before the first stage."""
        case = self.case
        s.set_hierarchy(case.iparent, case.position)
        s.set("BP", self.geo["bp"])
        for g, gl in enumerate(self.lists):
            for comp in (1, 2, 3):
                nc, xi, xr, xv = gl[comp]
                s.set_stencils(g + 1, comp, nc, xi, xr, xv)
            nc, fi, fr = gl[4]
            s.set_stencils(g + 1, 4, nc, fi, fr)
        s.set_ghostcell()
        one = np.ones(case.kk * case.jj)
        for g in range(case.ngrid):
            if case.bctype[g, 0] == abi.BC_FIX:
                s.set_buffer("U", g + 1, 1, one)
        u = np.ones(case.idim3d)
        zero = np.zeros(case.idim3d)
        for nm, a in zip("UVWP", (u, zero, zero, zero)):
            s.set(nm, a)
        for lvl in self.levels():
            s.connect(lvl, 2, v1="U", v2="V", v3="W", s1="P", corners=True)
        for lvl in range(int(case.level.max()), int(case.level.min()), -1):
            s.ftoc_multiple(lvl, v=("U", "V", "W"), s=("P",))
        for lvl in self.levels():
            s.connect(lvl, 1, v1="U", v2="V", v3="W", normal=True, forward=1)
            s.parent(lvl, v=("U", "V", "W"), s=("P",))
            s.bound_flow(lvl)
        s.setpointvalues(True)
