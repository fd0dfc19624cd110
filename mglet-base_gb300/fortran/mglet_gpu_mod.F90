! mglet_gpu_mod.F90 -- ISO_C_BINDING interface to libmglet_gpu.so
! (include/mglet_gpu.h) for the reference's Fortran callers.
!
! The module keeps the call shapes of the reference's hot-path modules so
! that timeloop_mod (src/timeloop_mod.F90:229-317) can call
!     CALL gpu_timeintegrate_flow(itstep, ittot, timeph, dt, irk, rkscheme)
! in place of timeintegrate_flow (src/flow/timeintegration_mod.F90:22).
! Field arrays are passed as the flat field_t%arr (src/core/field_t), so a
! host<->device copy is one memcpy of idim3d reals (REAL64 build).
! Every nonzero status goes to errr(__FILE__, __LINE__), as for the other C
! helpers of the reference (src/core/err_mod.F90:57-100).
MODULE mglet_gpu_mod
    USE, INTRINSIC :: ISO_C_BINDING
    USE err_mod, ONLY: errr
    IMPLICIT NONE(type, external)
    PRIVATE

    TYPE, BIND(C) :: mglet_grid_desc
        INTEGER(c_int32_t) :: ngrid
        TYPE(c_ptr) :: mgdims, level, bctype, nbrgrid, gradpflag
        TYPE(c_ptr) :: x, y, z, dx, dy, dz, ddx, ddy, ddz
    END TYPE mglet_grid_desc

    TYPE, BIND(C) :: mglet_flow_params
        REAL(c_double) :: gmol, rho, gradp(3)
        INTEGER(c_int32_t) :: psolver, ninner, nouter, nouter_min
        REAL(c_double) :: epcorr, omega
        INTEGER(c_int32_t) :: form, reserved
    END TYPE mglet_flow_params

    TYPE, BIND(C) :: mglet_rk_scheme
        INTEGER(c_int32_t) :: nrk, reserved
        REAL(c_double) :: cflmax, a(6), b(6), c(6)
    END TYPE mglet_rk_scheme

    TYPE, BIND(C) :: mglet_stage_stats
        INTEGER(c_int32_t) :: ipc, nouter_done
        REAL(c_double) :: maxrhs, prefak
    END TYPE mglet_stage_stats

    TYPE, BIND(C) :: mglet_itinfo
        REAL(c_double) :: cflmax, divmax, energy
        INTEGER(c_int32_t) :: exploded, reserved
    END TYPE mglet_itinfo

    ! Blocking fields of the ghost-cell IB for create_flowstencils (pointers
    ! to field_t%arr of BP, BU, BV, BW, AREAU, AREAV, AREAW, BZELLTYP, icells,
    ! nvecs(4, ncells), ucell(3, ncells))
    TYPE, BIND(C) :: mglet_ib_geometry
        TYPE(c_ptr) :: bp, bu, bv, bw, areau, areav, areaw, bzelltyp, icells, nvecs, ucell
    END TYPE mglet_ib_geometry

    ! create_scastencils' inputs: BP, BZELLTYP, per grid the cut-cell count,
    ! per cut cell its plane, interface area and body id (gc_t)
    TYPE, BIND(C) :: mglet_sca_geometry
        TYPE(c_ptr) :: bp, bzelltyp, icells, nvecs, arealist, bodyid
    END TYPE mglet_sca_geometry

    INTERFACE
        INTEGER(c_int) FUNCTION mglet_rk_init(name, rk) BIND(C, name="mglet_rk_init")
            IMPORT :: c_int, c_char, mglet_rk_scheme
            CHARACTER(kind=c_char), INTENT(in) :: name(*)
            TYPE(mglet_rk_scheme), INTENT(out) :: rk
        END FUNCTION mglet_rk_init

        INTEGER(c_int) FUNCTION mglet_gpu_create(desc, prm, device, ctx) &
                BIND(C, name="mglet_gpu_create")
            IMPORT :: c_int, c_int32_t, c_ptr, mglet_grid_desc, mglet_flow_params
            TYPE(mglet_grid_desc), INTENT(in) :: desc
            TYPE(mglet_flow_params), INTENT(in) :: prm
            INTEGER(c_int32_t), VALUE :: device
            TYPE(c_ptr), INTENT(out) :: ctx
        END FUNCTION mglet_gpu_create

        INTEGER(c_int) FUNCTION mglet_gpu_destroy(ctx) BIND(C, name="mglet_gpu_destroy")
            IMPORT :: c_int, c_ptr
            TYPE(c_ptr), VALUE :: ctx
        END FUNCTION mglet_gpu_destroy

        INTEGER(c_int) FUNCTION mglet_gpu_set_field(ctx, name, host, n) &
                BIND(C, name="mglet_gpu_set_field")
            IMPORT :: c_int, c_ptr, c_char, c_double, c_int64_t
            TYPE(c_ptr), VALUE :: ctx
            CHARACTER(kind=c_char), INTENT(in) :: name(*)
            REAL(c_double), INTENT(in) :: host(*)
            INTEGER(c_int64_t), VALUE :: n
        END FUNCTION mglet_gpu_set_field

        INTEGER(c_int) FUNCTION mglet_gpu_get_field(ctx, name, host, n) &
                BIND(C, name="mglet_gpu_get_field")
            IMPORT :: c_int, c_ptr, c_char, c_double, c_int64_t
            TYPE(c_ptr), VALUE :: ctx
            CHARACTER(kind=c_char), INTENT(in) :: name(*)
            REAL(c_double), INTENT(inout) :: host(*)
            INTEGER(c_int64_t), VALUE :: n
        END FUNCTION mglet_gpu_get_field

        INTEGER(c_int) FUNCTION mglet_gpu_timeintegrate_flow(ctx, itstep, ittot, timeph, dt, &
                irk, rk, stats) BIND(C, name="mglet_gpu_timeintegrate_flow")
            IMPORT :: c_int, c_int32_t, c_ptr, c_double, mglet_rk_scheme, mglet_stage_stats
            TYPE(c_ptr), VALUE :: ctx
            INTEGER(c_int32_t), VALUE :: itstep, ittot, irk
            REAL(c_double), VALUE :: timeph, dt
            TYPE(mglet_rk_scheme), INTENT(in) :: rk
            TYPE(mglet_stage_stats), INTENT(out) :: stats
        END FUNCTION mglet_gpu_timeintegrate_flow

        INTEGER(c_int) FUNCTION mglet_gpu_connect(ctx, ilevel, layers, v1, v2, v3, s1, s2, s3, &
                corners, normal, forward) BIND(C, name="mglet_gpu_connect")
            IMPORT :: c_int, c_int32_t, c_ptr
            TYPE(c_ptr), VALUE :: ctx
            INTEGER(c_int32_t), VALUE :: ilevel, layers, corners, normal, forward
            TYPE(c_ptr), VALUE :: v1, v2, v3, s1, s2, s3    ! C strings or C_NULL_PTR
        END FUNCTION mglet_gpu_connect

        INTEGER(c_int) FUNCTION mglet_gpu_bound_flow(ctx, ilevel) BIND(C, name="mglet_gpu_bound_flow")
            IMPORT :: c_int, c_int32_t, c_ptr
            TYPE(c_ptr), VALUE :: ctx
            INTEGER(c_int32_t), VALUE :: ilevel
        END FUNCTION mglet_gpu_bound_flow

        INTEGER(c_int) FUNCTION mglet_gpu_set_buffer(ctx, name, igrid, iface, host, n) &
                BIND(C, name="mglet_gpu_set_buffer")
            IMPORT :: c_int, c_int32_t, c_int64_t, c_ptr, c_char, c_double
            TYPE(c_ptr), VALUE :: ctx
            CHARACTER(kind=c_char), INTENT(in) :: name(*)
            INTEGER(c_int32_t), VALUE :: igrid, iface
            REAL(c_double), INTENT(in) :: host(*)
            INTEGER(c_int64_t), VALUE :: n
        END FUNCTION mglet_gpu_set_buffer

        INTEGER(c_int) FUNCTION mglet_gpu_set_bc_real(ctx, igrid, iface, value) &
                BIND(C, name="mglet_gpu_set_bc_real")
            IMPORT :: c_int, c_int32_t, c_ptr, c_double
            TYPE(c_ptr), VALUE :: ctx
            INTEGER(c_int32_t), VALUE :: igrid, iface
            REAL(c_double), VALUE :: value
        END FUNCTION mglet_gpu_set_bc_real

        INTEGER(c_int) FUNCTION mglet_gpu_set_stencils(ctx, igrid, comp, ncells, xpoli, nxi, &
                xpolr, nxr, xpolrvel, nxrv) BIND(C, name="mglet_gpu_set_stencils")
            IMPORT :: c_int, c_int32_t, c_int64_t, c_ptr, c_double
            TYPE(c_ptr), VALUE :: ctx
            INTEGER(c_int32_t), VALUE :: igrid, comp, ncells
            INTEGER(c_int64_t), INTENT(in) :: xpoli(*)
            INTEGER(c_int64_t), VALUE :: nxi, nxr, nxrv
            REAL(c_double), INTENT(in) :: xpolr(*), xpolrvel(*)
        END FUNCTION mglet_gpu_set_stencils

        INTEGER(c_int) FUNCTION mglet_gpu_set_ghostcell(ctx) BIND(C, name="mglet_gpu_set_ghostcell")
            IMPORT :: c_int, c_ptr
            TYPE(c_ptr), VALUE :: ctx
        END FUNCTION mglet_gpu_set_ghostcell

        INTEGER(c_int) FUNCTION mglet_gpu_setibvalues(ctx) BIND(C, name="mglet_gpu_setibvalues")
            IMPORT :: c_int, c_ptr
            TYPE(c_ptr), VALUE :: ctx
        END FUNCTION mglet_gpu_setibvalues

        INTEGER(c_int) FUNCTION mglet_gpu_setpointvalues(ctx, comp_new) &
                BIND(C, name="mglet_gpu_setpointvalues")
            IMPORT :: c_int, c_int32_t, c_ptr
            TYPE(c_ptr), VALUE :: ctx
            INTEGER(c_int32_t), VALUE :: comp_new
        END FUNCTION mglet_gpu_setpointvalues

        INTEGER(c_int) FUNCTION mglet_gpu_set_hierarchy(ctx, iparent, position) &
                BIND(C, name="mglet_gpu_set_hierarchy")
            IMPORT :: c_int, c_int32_t, c_ptr
            TYPE(c_ptr), VALUE :: ctx
            INTEGER(c_int32_t), INTENT(in) :: iparent(*), position(*)
        END FUNCTION mglet_gpu_set_hierarchy

        INTEGER(c_int) FUNCTION mglet_gpu_parent(ctx, ilevel, v1, v2, v3, s1, s2, s3, normal) &
                BIND(C, name="mglet_gpu_parent")
            IMPORT :: c_int, c_int32_t, c_ptr
            TYPE(c_ptr), VALUE :: ctx
            INTEGER(c_int32_t), VALUE :: ilevel, normal
            TYPE(c_ptr), VALUE :: v1, v2, v3, s1, s2, s3    ! C strings or C_NULL_PTR
        END FUNCTION mglet_gpu_parent

        INTEGER(c_int) FUNCTION mglet_gpu_ftoc(ctx, ilevel, ff, fc, flag) BIND(C, name="mglet_gpu_ftoc")
            IMPORT :: c_int, c_int32_t, c_ptr, c_char
            TYPE(c_ptr), VALUE :: ctx
            INTEGER(c_int32_t), VALUE :: ilevel
            CHARACTER(kind=c_char), INTENT(in) :: ff(*), fc(*)
            CHARACTER(kind=c_char), VALUE :: flag
        END FUNCTION mglet_gpu_ftoc

        INTEGER(c_int) FUNCTION mglet_gpu_ctof(ctx, ilevel, ff, fc) BIND(C, name="mglet_gpu_ctof")
            IMPORT :: c_int, c_int32_t, c_ptr, c_char
            TYPE(c_ptr), VALUE :: ctx
            INTEGER(c_int32_t), VALUE :: ilevel
            CHARACTER(kind=c_char), INTENT(in) :: ff(*), fc(*)
        END FUNCTION mglet_gpu_ctof

        INTEGER(c_int) FUNCTION mglet_gpu_set_scalars(ctx, nsca, prmol, kayscrawford, source, &
                prturb) BIND(C, name="mglet_gpu_set_scalars")
            IMPORT :: c_int, c_int32_t, c_ptr, c_double
            TYPE(c_ptr), VALUE :: ctx
            INTEGER(c_int32_t), VALUE :: nsca
            REAL(c_double), INTENT(in) :: prmol(*), source(*)
            INTEGER(c_int32_t), INTENT(in) :: kayscrawford(*)
            REAL(c_double), VALUE :: prturb
        END FUNCTION mglet_gpu_set_scalars

        INTEGER(c_int) FUNCTION mglet_gpu_timeintegrate_scalar(ctx, dt, irk, rk) &
                BIND(C, name="mglet_gpu_timeintegrate_scalar")
            IMPORT :: c_int, c_int32_t, c_ptr, c_double, mglet_rk_scheme
            TYPE(c_ptr), VALUE :: ctx
            REAL(c_double), VALUE :: dt
            INTEGER(c_int32_t), VALUE :: irk
            TYPE(mglet_rk_scheme), INTENT(in) :: rk
        END FUNCTION mglet_gpu_timeintegrate_scalar

        INTEGER(c_int) FUNCTION mglet_gpu_set_scalar_bc(ctx, igrid, iface, kind, types) &
                BIND(C, name="mglet_gpu_set_scalar_bc")
            IMPORT :: c_int, c_int32_t, c_ptr
            TYPE(c_ptr), VALUE :: ctx
            INTEGER(c_int32_t), VALUE :: igrid, iface, kind
            INTEGER(c_int32_t), INTENT(in) :: types(*)
        END FUNCTION mglet_gpu_set_scalar_bc

        INTEGER(c_int) FUNCTION mglet_gpu_add_scalar_source(ctx, isca, field, value) &
                BIND(C, name="mglet_gpu_add_scalar_source")
            IMPORT :: c_int, c_int32_t, c_ptr, c_double, c_char
            TYPE(c_ptr), VALUE :: ctx
            INTEGER(c_int32_t), VALUE :: isca
            CHARACTER(kind=c_char), INTENT(in) :: field(*)
            REAL(c_double), VALUE :: value
        END FUNCTION mglet_gpu_add_scalar_source

        INTEGER(c_int) FUNCTION mglet_gpu_set_lesmodel(ctx, model, cm) &
                BIND(C, name="mglet_gpu_set_lesmodel")
            IMPORT :: c_int, c_int32_t, c_ptr, c_double
            TYPE(c_ptr), VALUE :: ctx
            INTEGER(c_int32_t), VALUE :: model
            REAL(c_double), VALUE :: cm
        END FUNCTION mglet_gpu_set_lesmodel

        INTEGER(c_int) FUNCTION mglet_gpu_set_body_force(ctx, fx, fy, fz, n) &
                BIND(C, name="mglet_gpu_set_body_force")
            IMPORT :: c_int, c_int64_t, c_ptr, c_double
            TYPE(c_ptr), VALUE :: ctx
            REAL(c_double), INTENT(in) :: fx(*), fy(*), fz(*)
            INTEGER(c_int64_t), VALUE :: n
        END FUNCTION mglet_gpu_set_body_force

        INTEGER(c_int) FUNCTION mglet_gpu_energy_gradient(ctx, nsteps, ncheck, dt, rk, energy) &
                BIND(C, name="mglet_gpu_energy_gradient")
            IMPORT :: c_int, c_int32_t, c_ptr, c_double, mglet_rk_scheme
            TYPE(c_ptr), VALUE :: ctx
            INTEGER(c_int32_t), VALUE :: nsteps, ncheck
            REAL(c_double), VALUE :: dt
            TYPE(mglet_rk_scheme), INTENT(in) :: rk
            REAL(c_double), INTENT(out) :: energy
        END FUNCTION mglet_gpu_energy_gradient

        INTEGER(c_int) FUNCTION mglet_gpu_par_ftoc_norm(ctx, ilevel, v1, v2, v3, sum) &
                BIND(C, name="mglet_gpu_par_ftoc_norm")
            IMPORT :: c_int, c_int32_t, c_ptr, c_char
            TYPE(c_ptr), VALUE :: ctx
            INTEGER(c_int32_t), VALUE :: ilevel, sum
            CHARACTER(kind=c_char), INTENT(in) :: v1(*), v2(*), v3(*)
        END FUNCTION mglet_gpu_par_ftoc_norm

        INTEGER(c_int) FUNCTION mglet_gpu_bound_pressure(ctx, ilevel, dp, with_bp) &
                BIND(C, name="mglet_gpu_bound_pressure")
            IMPORT :: c_int, c_int32_t, c_ptr, c_char
            TYPE(c_ptr), VALUE :: ctx
            INTEGER(c_int32_t), VALUE :: ilevel, with_bp
            CHARACTER(kind=c_char), INTENT(in) :: dp(*)
        END FUNCTION mglet_gpu_bound_pressure

        INTEGER(c_int) FUNCTION mglet_gpu_tstle4(ctx) BIND(C, name="mglet_gpu_tstle4")
            IMPORT :: c_int, c_ptr
            TYPE(c_ptr), VALUE :: ctx
        END FUNCTION mglet_gpu_tstle4

        INTEGER(c_int) FUNCTION mglet_gpu_rkstep(ctx, p, dp, rhsp, frhs, dtfu) &
                BIND(C, name="mglet_gpu_rkstep")
            IMPORT :: c_int, c_ptr, c_char, c_double
            TYPE(c_ptr), VALUE :: ctx
            CHARACTER(kind=c_char), INTENT(in) :: p(*), dp(*), rhsp(*)
            REAL(c_double), VALUE :: frhs, dtfu
        END FUNCTION mglet_gpu_rkstep

        INTEGER(c_int) FUNCTION mglet_gpu_divcal(ctx, div, fak) BIND(C, name="mglet_gpu_divcal")
            IMPORT :: c_int, c_ptr, c_char, c_double
            TYPE(c_ptr), VALUE :: ctx
            CHARACTER(kind=c_char), INTENT(in) :: div(*)
            REAL(c_double), VALUE :: fak
        END FUNCTION mglet_gpu_divcal

        INTEGER(c_int) FUNCTION mglet_gpu_laplacephi(ctx, res, phi) &
                BIND(C, name="mglet_gpu_laplacephi")
            IMPORT :: c_int, c_ptr, c_char
            TYPE(c_ptr), VALUE :: ctx
            CHARACTER(kind=c_char), INTENT(in) :: res(*), phi(*)
        END FUNCTION mglet_gpu_laplacephi

        INTEGER(c_int) FUNCTION mglet_gpu_mgpoisl(ctx, dt, ittot, irk, stats) &
                BIND(C, name="mglet_gpu_mgpoisl")
            IMPORT :: c_int, c_int32_t, c_ptr, c_double, mglet_stage_stats
            TYPE(c_ptr), VALUE :: ctx
            REAL(c_double), VALUE :: dt
            INTEGER(c_int32_t), VALUE :: ittot, irk
            TYPE(mglet_stage_stats), INTENT(out) :: stats
        END FUNCTION mglet_gpu_mgpoisl

        INTEGER(c_int) FUNCTION mglet_gpu_maskbp(ctx) BIND(C, name="mglet_gpu_maskbp")
            IMPORT :: c_int, c_ptr
            TYPE(c_ptr), VALUE :: ctx
        END FUNCTION mglet_gpu_maskbp

        INTEGER(c_int) FUNCTION mglet_gpu_getibvalues(ctx) BIND(C, name="mglet_gpu_getibvalues")
            IMPORT :: c_int, c_ptr
            TYPE(c_ptr), VALUE :: ctx
        END FUNCTION mglet_gpu_getibvalues

        INTEGER(c_int) FUNCTION mglet_gpu_adjoint_rk_stage(ctx, irk, dt, rk) &
                BIND(C, name="mglet_gpu_adjoint_rk_stage")
            IMPORT :: c_int, c_int32_t, c_ptr, c_double, mglet_rk_scheme
            TYPE(c_ptr), VALUE :: ctx
            INTEGER(c_int32_t), VALUE :: irk
            REAL(c_double), VALUE :: dt
            TYPE(mglet_rk_scheme), INTENT(in) :: rk
        END FUNCTION mglet_gpu_adjoint_rk_stage

        INTEGER(c_int) FUNCTION mglet_create_scastencils(desc, geo, out) &
                BIND(C, name="mglet_create_scastencils")
            IMPORT :: c_int, c_ptr, mglet_grid_desc, mglet_sca_geometry
            TYPE(mglet_grid_desc), INTENT(in) :: desc
            TYPE(mglet_sca_geometry), INTENT(in) :: geo
            TYPE(c_ptr), INTENT(out) :: out
        END FUNCTION mglet_create_scastencils

        INTEGER(c_int) FUNCTION mglet_scastencils_size(s, igrid, ncells) &
                BIND(C, name="mglet_scastencils_size")
            IMPORT :: c_int, c_int32_t, c_ptr
            TYPE(c_ptr), VALUE :: s
            INTEGER(c_int32_t), VALUE :: igrid
            INTEGER(c_int32_t), INTENT(out) :: ncells
        END FUNCTION mglet_scastencils_size

        INTEGER(c_int) FUNCTION mglet_scastencils_copy(s, igrid, xpoli, xpolr, xpolrvel) &
                BIND(C, name="mglet_scastencils_copy")
            IMPORT :: c_int, c_int32_t, c_int64_t, c_ptr, c_double
            TYPE(c_ptr), VALUE :: s
            INTEGER(c_int32_t), VALUE :: igrid
            INTEGER(c_int64_t), INTENT(out) :: xpoli(*)
            REAL(c_double), INTENT(out) :: xpolr(*), xpolrvel(*)
        END FUNCTION mglet_scastencils_copy

        INTEGER(c_int) FUNCTION mglet_scastencils_free(s) BIND(C, name="mglet_scastencils_free")
            IMPORT :: c_int, c_ptr
            TYPE(c_ptr), VALUE :: s
        END FUNCTION mglet_scastencils_free

        INTEGER(c_int) FUNCTION mglet_create_flowstencils(desc, geo, out) &
                BIND(C, name="mglet_create_flowstencils")
            IMPORT :: c_int, c_ptr, mglet_grid_desc, mglet_ib_geometry
            TYPE(mglet_grid_desc), INTENT(in) :: desc
            TYPE(mglet_ib_geometry), INTENT(in) :: geo
            TYPE(c_ptr), INTENT(out) :: out
        END FUNCTION mglet_create_flowstencils

        INTEGER(c_int) FUNCTION mglet_flowstencils_size(s, igrid, comp, ncells, nxi, nxr) &
                BIND(C, name="mglet_flowstencils_size")
            IMPORT :: c_int, c_int32_t, c_int64_t, c_ptr
            TYPE(c_ptr), VALUE :: s
            INTEGER(c_int32_t), VALUE :: igrid, comp
            INTEGER(c_int32_t), INTENT(out) :: ncells
            INTEGER(c_int64_t), INTENT(out) :: nxi, nxr
        END FUNCTION mglet_flowstencils_size

        INTEGER(c_int) FUNCTION mglet_flowstencils_copy(s, igrid, comp, xpoli, xpolr, xpolrvel) &
                BIND(C, name="mglet_flowstencils_copy")
            IMPORT :: c_int, c_int32_t, c_int64_t, c_ptr, c_double
            TYPE(c_ptr), VALUE :: s
            INTEGER(c_int32_t), VALUE :: igrid, comp
            INTEGER(c_int64_t), INTENT(out) :: xpoli(*)
            REAL(c_double), INTENT(out) :: xpolr(*), xpolrvel(*)
        END FUNCTION mglet_flowstencils_copy

        INTEGER(c_int) FUNCTION mglet_flowstencils_free(s) BIND(C, name="mglet_flowstencils_free")
            IMPORT :: c_int, c_ptr
            TYPE(c_ptr), VALUE :: s
        END FUNCTION mglet_flowstencils_free

        INTEGER(c_int) FUNCTION mglet_gpu_set_partition(ctx, halo, nsend, send, nrecv, recv, &
                fn, user) BIND(C, name="mglet_gpu_set_partition")
            IMPORT :: c_int, c_int32_t, c_ptr, c_funptr
            TYPE(c_ptr), VALUE :: ctx
            INTEGER(c_int32_t), INTENT(in) :: halo(*), send(*), recv(*)
            INTEGER(c_int32_t), VALUE :: nsend, nrecv
            TYPE(c_funptr), VALUE :: fn
            TYPE(c_ptr), VALUE :: user
        END FUNCTION mglet_gpu_set_partition

        INTEGER(c_int) FUNCTION mglet_gpu_itinfo(ctx, dt, out) BIND(C, name="mglet_gpu_itinfo")
            IMPORT :: c_int, c_ptr, c_double, mglet_itinfo
            TYPE(c_ptr), VALUE :: ctx
            REAL(c_double), VALUE :: dt
            TYPE(mglet_itinfo), INTENT(out) :: out
        END FUNCTION mglet_gpu_itinfo

        INTEGER(c_int) FUNCTION mglet_gpu_ftoc_multiple(ctx, ilevel, v1, v2, v3, s1, s2, s3) &
                BIND(C, name="mglet_gpu_ftoc_multiple")
            IMPORT :: c_int, c_int32_t, c_ptr
            TYPE(c_ptr), VALUE :: ctx
            INTEGER(c_int32_t), VALUE :: ilevel
            TYPE(c_ptr), VALUE :: v1, v2, v3, s1, s2, s3
        END FUNCTION mglet_gpu_ftoc_multiple

        INTEGER(c_int) FUNCTION mglet_gpu_get_buffer(ctx, name, igrid, iface, host, n) &
                BIND(C, name="mglet_gpu_get_buffer")
            IMPORT :: c_int, c_int32_t, c_int64_t, c_ptr, c_char, c_double
            TYPE(c_ptr), VALUE :: ctx
            CHARACTER(kind=c_char), INTENT(in) :: name(*)
            INTEGER(c_int32_t), VALUE :: igrid, iface
            REAL(c_double), INTENT(out) :: host(*)
            INTEGER(c_int64_t), VALUE :: n
        END FUNCTION mglet_gpu_get_buffer

        INTEGER(c_int) FUNCTION mglet_gpu_divmax_noalloc(u, v, w, ngrid, kk, jj, ii, rddx, rddy, &
                rddz, divmax, stream) BIND(C, name="mglet_gpu_divmax_noalloc")
            IMPORT :: c_int, c_int32_t, c_ptr
            TYPE(c_ptr), VALUE :: u, v, w, rddx, rddy, rddz, divmax, stream
            INTEGER(c_int32_t), VALUE :: ngrid, kk, jj, ii
        END FUNCTION mglet_gpu_divmax_noalloc

        INTEGER(c_int) FUNCTION mglet_gpu_synchronize(ctx) BIND(C, name="mglet_gpu_synchronize")
            IMPORT :: c_int, c_ptr
            TYPE(c_ptr), VALUE :: ctx
        END FUNCTION mglet_gpu_synchronize

        INTEGER(c_int64_t) FUNCTION mglet_gpu_idim3d(ctx) BIND(C, name="mglet_gpu_idim3d")
            IMPORT :: c_int64_t, c_ptr
            TYPE(c_ptr), VALUE :: ctx
        END FUNCTION mglet_gpu_idim3d

        TYPE(c_ptr) FUNCTION mglet_gpu_last_error() BIND(C, name="mglet_gpu_last_error")
            IMPORT :: c_ptr
        END FUNCTION mglet_gpu_last_error

        INTEGER(c_int) FUNCTION mglet_rk_get_coeffs(rk, irk, frhs, fu, dtrk, dtrki) &
                BIND(C, name="mglet_rk_get_coeffs")
            IMPORT :: c_int, c_int32_t, c_double, mglet_rk_scheme
            TYPE(mglet_rk_scheme), INTENT(in) :: rk
            INTEGER(c_int32_t), VALUE :: irk
            REAL(c_double), INTENT(out) :: frhs, fu, dtrk, dtrki
        END FUNCTION mglet_rk_get_coeffs

        INTEGER(c_int) FUNCTION mglet_gpu_tuning(ctx, buf, buflen) BIND(C, name="mglet_gpu_tuning")
            IMPORT :: c_int, c_int64_t, c_ptr, c_char
            TYPE(c_ptr), VALUE :: ctx
            CHARACTER(kind=c_char), INTENT(out) :: buf(*)
            INTEGER(c_int64_t), VALUE :: buflen
        END FUNCTION mglet_gpu_tuning

        INTEGER(c_int) FUNCTION mglet_gpu_set_scastencils(ctx, igrid, ncells, xpoli, xpolr, &
                xpolrvel) BIND(C, name="mglet_gpu_set_scastencils")
            IMPORT :: c_int, c_int32_t, c_int64_t, c_ptr, c_double
            TYPE(c_ptr), VALUE :: ctx
            INTEGER(c_int32_t), VALUE :: igrid, ncells
            INTEGER(c_int64_t), INTENT(in) :: xpoli(*)
            REAL(c_double), INTENT(in) :: xpolr(*), xpolrvel(*)
        END FUNCTION mglet_gpu_set_scastencils

        INTEGER(c_int) FUNCTION mglet_gpu_set_scalar_geometry(ctx, isca, nbody, flag, value) &
                BIND(C, name="mglet_gpu_set_scalar_geometry")
            IMPORT :: c_int, c_int32_t, c_ptr, c_double
            TYPE(c_ptr), VALUE :: ctx
            INTEGER(c_int32_t), VALUE :: isca, nbody
            INTEGER(c_int32_t), INTENT(in) :: flag(*)
            REAL(c_double), INTENT(in) :: value(*)
        END FUNCTION mglet_gpu_set_scalar_geometry

        INTEGER(c_int) FUNCTION mglet_gpu_force_variant(ctx, kernel, variant) &
                BIND(C, name="mglet_gpu_force_variant")
            IMPORT :: c_int, c_int32_t, c_ptr, c_char
            TYPE(c_ptr), VALUE :: ctx
            CHARACTER(kind=c_char), INTENT(in) :: kernel(*)
            INTEGER(c_int32_t), VALUE :: variant
        END FUNCTION mglet_gpu_force_variant
    END INTERFACE

    ! mglet_flow_params%form: the FP64 form bit for bit with the reference, the
    ! batched mixed-precision form, the FP64 form with multiply-add contraction
    INTEGER(c_int32_t), PARAMETER :: MGLET_FORM_PLAIN = 0, MGLET_FORM_MIXED = 1, &
        MGLET_FORM_PLAIN_FMA = 2

    TYPE(c_ptr), SAVE :: gctx = C_NULL_PTR
    TYPE(mglet_rk_scheme), SAVE :: grk

    PUBLIC :: mglet_grid_desc, mglet_flow_params, mglet_rk_scheme, mglet_stage_stats, &
        mglet_itinfo, gpu_init, gpu_finish, gpu_upload, gpu_download, &
        gpu_timeintegrate_flow, gpu_itinfo, gpu_upload_buffer, gpu_set_pinf, &
        gpu_upload_stencils, gpu_start_ghostcell, gpu_set_hierarchy, gpu_ftoc, gpu_ctof, &
        gpu_bound_pressure, gpu_par_ftoc_norm, gpu_set_lesmodel, gpu_set_body_force, &
        gpu_energy_gradient, gpu_set_scalars, gpu_timeintegrate_scalar, gpu_set_scalar_bc, &
        gpu_add_scalar_source, gpu_tstle4, gpu_rkstep, gpu_divcal, gpu_laplacephi, gpu_mgpoisl, &
        gpu_maskbp, gpu_getibvalues, gpu_adjoint_rk_stage, mglet_ib_geometry, &
        gpu_create_flowstencils, gpu_ftoc_multiple, gpu_download_buffer, gpu_synchronize, &
        gpu_tuning, gpu_force_variant, MGLET_FORM_PLAIN, MGLET_FORM_MIXED, MGLET_FORM_PLAIN_FMA, &
        gpu_set_scastencils, gpu_set_scalar_geometry, mglet_sca_geometry, gpu_create_scastencils

CONTAINS
    ! Called once after init_flow: builds the device state from the same
    ! tables grids.h5 provides (one rank, one level, noib).
    SUBROUTINE gpu_init(desc, prm, rkname)
        TYPE(mglet_grid_desc), INTENT(in) :: desc
        TYPE(mglet_flow_params), INTENT(in) :: prm
        CHARACTER(len=*), INTENT(in) :: rkname
        IF (mglet_gpu_create(desc, prm, 0_c_int32_t, gctx) /= 0) CALL errr(__FILE__, __LINE__)
        IF (mglet_rk_init(TRIM(rkname)//C_NULL_CHAR, grk) /= 0) CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_init

    SUBROUTINE gpu_finish()
        IF (mglet_gpu_destroy(gctx) /= 0) CALL errr(__FILE__, __LINE__)
        gctx = C_NULL_PTR
    END SUBROUTINE gpu_finish

    ! map_arr_to_device equivalent for one field_t%arr
    SUBROUTINE gpu_upload(name, arr)
        CHARACTER(len=*), INTENT(in) :: name
        REAL(c_double), INTENT(in) :: arr(:)
        IF (mglet_gpu_set_field(gctx, TRIM(name)//C_NULL_CHAR, arr, &
            INT(SIZE(arr), c_int64_t)) /= 0) CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_upload

    SUBROUTINE gpu_download(name, arr)
        CHARACTER(len=*), INTENT(in) :: name
        REAL(c_double), INTENT(inout) :: arr(:)
        IF (mglet_gpu_get_field(gctx, TRIM(name)//C_NULL_CHAR, arr, &
            INT(SIZE(arr), c_int64_t)) /= 0) CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_download

    ! One boundary buffer plane (field_t%get_buffer(buf, igrid, iface)), for
    ! FIX inflow values and OP1 inflow tangential velocities; call after
    ! setboundarybuffers has filled the host copy.
    SUBROUTINE gpu_upload_buffer(name, igrid, iface, buf)
        CHARACTER(len=*), INTENT(in) :: name
        INTEGER, INTENT(in) :: igrid, iface
        REAL(c_double), INTENT(in) :: buf(:, :)
        IF (mglet_gpu_set_buffer(gctx, TRIM(name)//C_NULL_CHAR, INT(igrid, c_int32_t), &
            INT(iface, c_int32_t), buf, INT(SIZE(buf), c_int64_t)) /= 0) &
            CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_upload_buffer

    ! OP1 far-field pressure of one face (get_bcprms with nreal = 1)
    SUBROUTINE gpu_set_pinf(igrid, iface, pinf)
        INTEGER, INTENT(in) :: igrid, iface
        REAL(c_double), INTENT(in) :: pinf
        IF (mglet_gpu_set_bc_real(gctx, INT(igrid, c_int32_t), INT(iface, c_int32_t), pinf) /= 0) &
            CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_set_pinf

    ! The grid hierarchy (gridinfo%iparent, i/j/kposition of every grid):
    ! needed before gpu_parent, gpu_ftoc, gpu_ctof, a multi-level mgpoisl and
    ! a multi-level gpu_timeintegrate_flow.
    SUBROUTINE gpu_set_hierarchy(iparent, position)
        INTEGER(c_int32_t), INTENT(in) :: iparent(:), position(:, :)   ! position(3, ngrid)
        IF (mglet_gpu_set_hierarchy(gctx, iparent, position) /= 0) CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_set_hierarchy

    ! Drop-in for ftoc(ilevel, ff, fc, flag) on the device copies
    SUBROUTINE gpu_ftoc(ilevel, ff, fc, flag)
        INTEGER, INTENT(in) :: ilevel
        CHARACTER(len=*), INTENT(in) :: ff, fc
        CHARACTER(len=1), INTENT(in) :: flag
        IF (mglet_gpu_ftoc(gctx, INT(ilevel, c_int32_t), TRIM(ff)//C_NULL_CHAR, &
            TRIM(fc)//C_NULL_CHAR, flag) /= 0) CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_ftoc

    ! Drop-in for ctof(ilevel, ff, fc) on the device copies
    SUBROUTINE gpu_ctof(ilevel, ff, fc)
        INTEGER, INTENT(in) :: ilevel
        CHARACTER(len=*), INTENT(in) :: ff, fc
        IF (mglet_gpu_ctof(gctx, INT(ilevel, c_int32_t), TRIM(ff)//C_NULL_CHAR, &
            TRIM(fc)//C_NULL_CHAR) /= 0) CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_ctof

    ! The scalars of scacore_mod (device fields T1..Tn)
    SUBROUTINE gpu_set_scalars(prmol, kayscrawford, source, prturb)
        REAL(c_double), INTENT(in) :: prmol(:), source(:), prturb
        INTEGER(c_int32_t), INTENT(in) :: kayscrawford(:)
        IF (mglet_gpu_set_scalars(gctx, INT(SIZE(prmol), c_int32_t), prmol, kayscrawford, source, &
            prturb) /= 0) CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_set_scalars

    ! The scalar condition of a boundary face, as get_bcprms hands
    ! bound_scalar_mod.F90 its scbtype: kind 1 SWA, 2 SIO; scbtype(l) 0 value,
    ! 1 flux; the value or flux goes in with gpu_upload_buffer under the
    ! scalar's name
    SUBROUTINE gpu_set_scalar_bc(igrid, iface, kind, scbtype)
        INTEGER, INTENT(in) :: igrid, iface, kind
        INTEGER(c_int32_t), INTENT(in) :: scbtype(:)
        IF (mglet_gpu_set_scalar_bc(gctx, INT(igrid, c_int32_t), INT(iface, c_int32_t), &
            INT(kind, c_int32_t), scbtype) /= 0) CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_set_scalar_bc

    ! One entry of sca%sources (timeintegrate_scalar_mod.F90:549-634): an
    ! empty field name is a constant source, else value * that field
    SUBROUTINE gpu_add_scalar_source(isca, field, value)
        INTEGER, INTENT(in) :: isca
        CHARACTER(len=*), INTENT(in) :: field
        REAL(c_double), INTENT(in) :: value
        IF (mglet_gpu_add_scalar_source(gctx, INT(isca, c_int32_t), TRIM(field)//c_null_char, value) /= 0) &
            CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_add_scalar_source

    ! Drop-in for timeintegrate_scalar (src/scalar/timeintegrate_scalar_mod.F90:17)
    SUBROUTINE gpu_timeintegrate_scalar(dt, irk)
        REAL(c_double), INTENT(in) :: dt
        INTEGER, INTENT(in) :: irk
        IF (mglet_gpu_timeintegrate_scalar(gctx, dt, INT(irk, c_int32_t), grk) /= 0) &
            CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_timeintegrate_scalar

    ! init_lesmodel (src/flow/lesmodel_mod.F90:34-84): model 0 none,
    ! 1 smagorinsky, 2 wale; cm < 0 takes the model's default constant
    SUBROUTINE gpu_set_lesmodel(model, cm)
        INTEGER, INTENT(in) :: model
        REAL(c_double), INTENT(in) :: cm
        IF (mglet_gpu_set_lesmodel(gctx, INT(model, c_int32_t), cm) /= 0) CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_set_lesmodel

    ! A steady body force per unit mass (flat fields of idim3d reals)
    SUBROUTINE gpu_set_body_force(fx, fy, fz)
        REAL(c_double), INTENT(in) :: fx(:), fy(:), fz(:)
        IF (mglet_gpu_set_body_force(gctx, fx, fy, fz, INT(SIZE(fx), c_int64_t)) /= 0) &
            CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_set_body_force

    ! The kinetic energy after nsteps steps and its gradient with respect to
    ! the body force (device fields GFX, GFY, GFZ; gpu_download them)
    SUBROUTINE gpu_energy_gradient(nsteps, ncheck, dt, energy)
        INTEGER, INTENT(in) :: nsteps, ncheck
        REAL(c_double), INTENT(in) :: dt
        REAL(c_double), INTENT(out) :: energy
        IF (mglet_gpu_energy_gradient(gctx, INT(nsteps, c_int32_t), INT(ncheck, c_int32_t), dt, &
            grk, energy) /= 0) CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_energy_gradient

    ! Drop-in for par_ftoc_norm(ilevel, v1, v2, v3[, sum]) on the device copies
    SUBROUTINE gpu_par_ftoc_norm(ilevel, v1, v2, v3, sum)
        INTEGER, INTENT(in) :: ilevel
        CHARACTER(len=*), INTENT(in) :: v1, v2, v3
        LOGICAL, OPTIONAL, INTENT(in) :: sum
        INTEGER(c_int32_t) :: s
        s = 0
        IF (PRESENT(sum)) THEN
            IF (sum) s = 1
        END IF
        IF (mglet_gpu_par_ftoc_norm(gctx, INT(ilevel, c_int32_t), TRIM(v1)//C_NULL_CHAR, &
            TRIM(v2)//C_NULL_CHAR, TRIM(v3)//C_NULL_CHAR, s) /= 0) CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_par_ftoc_norm

    ! Drop-in for bound_pressure(ilevel, dp[, bp]) on the device copies
    SUBROUTINE gpu_bound_pressure(ilevel, dp, with_bp)
        INTEGER, INTENT(in) :: ilevel
        CHARACTER(len=*), INTENT(in) :: dp
        LOGICAL, INTENT(in) :: with_bp
        INTEGER(c_int32_t) :: wb
        wb = 0
        IF (with_bp) wb = 1
        IF (mglet_gpu_bound_pressure(gctx, INT(ilevel, c_int32_t), TRIM(dp)//C_NULL_CHAR, wb) /= 0) &
            CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_bound_pressure

    ! Ghost-cell lists of one grid and component (the uxpoli/uxpolr/uxpolrvel,
    ! .., fxpoli/fxpolr arrays of gc_flowstencils_mod after
    ! create_flowstencils); comp 4 is the flux correction (xpolrvel unused).
    SUBROUTINE gpu_upload_stencils(igrid, comp, ncells, xpoli, xpolr, xpolrvel)
        INTEGER, INTENT(in) :: igrid, comp, ncells
        INTEGER(c_int64_t), INTENT(in) :: xpoli(:)
        REAL(c_double), INTENT(in) :: xpolr(:), xpolrvel(:)
        IF (mglet_gpu_set_stencils(gctx, INT(igrid, c_int32_t), INT(comp, c_int32_t), &
            INT(ncells, c_int32_t), xpoli, INT(SIZE(xpoli), c_int64_t), xpolr, &
            INT(SIZE(xpolr), c_int64_t), xpolrvel, INT(SIZE(xpolrvel), c_int64_t)) /= 0) &
            CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_upload_stencils

    ! After BP and all lists are uploaded: rebuild the Poisson coefficients,
    ! build SDIV, and initialise the point values (setpointvalues with new
    ! extrapolation, as the reference's flow initialisation does).
    ! The end of init_flow (src/flow/flow_mod.F90:83-84): point values and
    ! ghost values once before the first stage.  With grid hierarchies call
    ! gpu_set_hierarchy first.
    SUBROUTINE gpu_start_ghostcell()
        IF (mglet_gpu_set_ghostcell(gctx) /= 0) CALL errr(__FILE__, __LINE__)
        IF (mglet_gpu_setpointvalues(gctx, 1_c_int32_t) /= 0) CALL errr(__FILE__, __LINE__)
        IF (mglet_gpu_setibvalues(gctx) /= 0) CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_start_ghostcell

    ! Drop-in for timeintegrate_flow (src/flow/timeintegration_mod.F90:22)
    SUBROUTINE gpu_timeintegrate_flow(itstep, ittot, timeph, dt, irk, ipc)
        INTEGER, INTENT(in) :: itstep, ittot, irk
        REAL(c_double), INTENT(in) :: timeph, dt
        INTEGER, INTENT(out) :: ipc
        TYPE(mglet_stage_stats) :: st
        IF (mglet_gpu_timeintegrate_flow(gctx, INT(itstep, c_int32_t), INT(ittot, c_int32_t), &
            timeph, dt, INT(irk, c_int32_t), grk, st) /= 0) CALL errr(__FILE__, __LINE__)
        ipc = st%ipc
    END SUBROUTINE gpu_timeintegrate_flow

    ! Drop-in for tstle4(uo, vo, wo, u, v, w, u, v, w, p, g) on the device
    ! fields (src/flow/tstle4_mod.F90:13)
    SUBROUTINE gpu_tstle4()
        IF (mglet_gpu_tstle4(gctx) /= 0) CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_tstle4

    ! Drop-in for rkstep(p, dp, rhsp, frhs, dtfu) (src/core/rungekutta_mod.F90:315)
    SUBROUTINE gpu_rkstep(p, dp, rhsp, frhs, dtfu)
        CHARACTER(len=*), INTENT(in) :: p, dp, rhsp
        REAL(c_double), INTENT(in) :: frhs, dtfu
        IF (mglet_gpu_rkstep(gctx, TRIM(p)//C_NULL_CHAR, TRIM(dp)//C_NULL_CHAR, &
            TRIM(rhsp)//C_NULL_CHAR, frhs, dtfu) /= 0) CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_rkstep

    ! Drop-in for ib%divcal(div, u, v, w, fak) (src/ib/noib_mod.F90:253)
    SUBROUTINE gpu_divcal(div, fak)
        CHARACTER(len=*), INTENT(in) :: div
        REAL(c_double), INTENT(in) :: fak
        IF (mglet_gpu_divcal(gctx, TRIM(div)//C_NULL_CHAR, fak) /= 0) CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_divcal

    ! Drop-in for laplacephi(res, phi) (src/flow/laplacephi_mod.F90:14)
    SUBROUTINE gpu_laplacephi(res, phi)
        CHARACTER(len=*), INTENT(in) :: res, phi
        IF (mglet_gpu_laplacephi(gctx, TRIM(res)//C_NULL_CHAR, TRIM(phi)//C_NULL_CHAR) /= 0) &
            CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_laplacephi

    ! Drop-in for mgpoisl(u, v, w, p, dt, ittot, irk)
    ! (src/flow/pressuresolver_mod.F90:160)
    SUBROUTINE gpu_mgpoisl(dt, ittot, irk, ipc)
        REAL(c_double), INTENT(in) :: dt
        INTEGER, INTENT(in) :: ittot, irk
        INTEGER, INTENT(out) :: ipc
        TYPE(mglet_stage_stats) :: st
        IF (mglet_gpu_mgpoisl(gctx, dt, INT(ittot, c_int32_t), INT(irk, c_int32_t), st) /= 0) &
            CALL errr(__FILE__, __LINE__)
        ipc = st%ipc
    END SUBROUTINE gpu_mgpoisl

    ! Drop-ins for maskbp(u, v, w, p) and getibvalues(u, v, w)
    ! (src/flow/timeintegration_mod.F90:255, gc_flowstencils_mod.F90:1393)
    SUBROUTINE gpu_maskbp()
        IF (mglet_gpu_maskbp(gctx) /= 0) CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_maskbp

    SUBROUTINE gpu_getibvalues()
        IF (mglet_gpu_getibvalues(gctx) /= 0) CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_getibvalues

    ! The adjoint of one stage (device fields LU.., GFX..; no reference
    ! counterpart)
    SUBROUTINE gpu_adjoint_rk_stage(irk, dt)
        INTEGER, INTENT(in) :: irk
        REAL(c_double), INTENT(in) :: dt
        IF (mglet_gpu_adjoint_rk_stage(gctx, INT(irk, c_int32_t), dt, grk) /= 0) &
            CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_adjoint_rk_stage

    ! Replaces create_flowstencils (gc_flowstencils_mod.F90:37): builds every
    ! grid's lists from the blocking fields and uploads them; call
    ! gpu_start_ghostcell afterwards.
    ! Drop-in for create_scastencils(gc): builds every grid's scalar list
    ! from the cut cells and uploads it
    SUBROUTINE gpu_create_scastencils(desc, geo)
        TYPE(mglet_grid_desc), INTENT(in) :: desc
        TYPE(mglet_sca_geometry), INTENT(in) :: geo
        TYPE(c_ptr) :: s
        INTEGER :: ig
        INTEGER(c_int32_t) :: nc
        INTEGER(c_int64_t), ALLOCATABLE :: xi(:)
        REAL(c_double), ALLOCATABLE :: xr(:), xv(:)
        IF (mglet_create_scastencils(desc, geo, s) /= 0) CALL errr(__FILE__, __LINE__)
        DO ig = 1, desc%ngrid
            IF (mglet_scastencils_size(s, INT(ig, c_int32_t), nc) /= 0) CALL errr(__FILE__, __LINE__)
            ALLOCATE(xi(MAX(9 * nc, 1)), xr(MAX(8 * nc, 1)), xv(MAX(8 * nc, 1)))
            IF (mglet_scastencils_copy(s, INT(ig, c_int32_t), xi, xr, xv) /= 0) &
                CALL errr(__FILE__, __LINE__)
            CALL gpu_set_scastencils(ig, INT(nc), xi(1:9 * nc), xr(1:8 * nc), xv(1:8 * nc))
            DEALLOCATE(xi, xr, xv)
        END DO
        IF (mglet_scastencils_free(s) /= 0) CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_create_scastencils

    SUBROUTINE gpu_create_flowstencils(desc, geo)
        TYPE(mglet_grid_desc), INTENT(in) :: desc
        TYPE(mglet_ib_geometry), INTENT(in) :: geo
        TYPE(c_ptr) :: s
        INTEGER :: ig, comp
        INTEGER(c_int32_t) :: nc
        INTEGER(c_int64_t) :: nxi, nxr
        INTEGER(c_int64_t), ALLOCATABLE :: xi(:)
        REAL(c_double), ALLOCATABLE :: xr(:), xv(:)
        IF (mglet_create_flowstencils(desc, geo, s) /= 0) CALL errr(__FILE__, __LINE__)
        DO ig = 1, desc%ngrid
            DO comp = 1, 4
                IF (mglet_flowstencils_size(s, INT(ig, c_int32_t), INT(comp, c_int32_t), nc, nxi, &
                    nxr) /= 0) CALL errr(__FILE__, __LINE__)
                ALLOCATE(xi(MAX(nxi, 1_c_int64_t)), xr(MAX(nxr, 1_c_int64_t)), &
                    xv(MAX(nxr, 1_c_int64_t)))
                IF (mglet_flowstencils_copy(s, INT(ig, c_int32_t), INT(comp, c_int32_t), xi, xr, &
                    xv) /= 0) CALL errr(__FILE__, __LINE__)
                CALL gpu_upload_stencils(ig, comp, INT(nc), xi(1:nxi), xr(1:nxr), xv(1:nxr))
                DEALLOCATE(xi, xr, xv)
            END DO
        END DO
        IF (mglet_flowstencils_free(s) /= 0) CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_create_flowstencils

    ! Drop-in for ftoc_multiple(ilevel, v1, v2, v3, s1, s2, s3): blank names
    ! leave a slot out
    SUBROUTINE gpu_ftoc_multiple(ilevel, v1, v2, v3, s1, s2, s3)
        INTEGER, INTENT(in) :: ilevel
        CHARACTER(len=*), INTENT(in) :: v1, v2, v3, s1, s2, s3
        ! one NUL-terminated name per column (field names are short)
        CHARACTER(kind=c_char), TARGET :: n(64, 6)
        TYPE(c_ptr) :: p(6)
        INTEGER :: q
        CALL put(1, v1); CALL put(2, v2); CALL put(3, v3)
        CALL put(4, s1); CALL put(5, s2); CALL put(6, s3)
        DO q = 1, 6
            p(q) = C_NULL_PTR
            IF (n(1, q) /= C_NULL_CHAR) p(q) = C_LOC(n(1, q))
        END DO
        IF (mglet_gpu_ftoc_multiple(gctx, INT(ilevel, c_int32_t), p(1), p(2), p(3), p(4), p(5), &
            p(6)) /= 0) CALL errr(__FILE__, __LINE__)
    CONTAINS
        SUBROUTINE put(col, name)
            INTEGER, INTENT(in) :: col
            CHARACTER(len=*), INTENT(in) :: name
            INTEGER :: c, l
            l = MIN(LEN_TRIM(name), 63)
            DO c = 1, l
                n(c, col) = name(c:c)
            END DO
            n(l + 1, col) = C_NULL_CHAR
        END SUBROUTINE put
    END SUBROUTINE gpu_ftoc_multiple

    ! field_t%get_buffer(buf, igrid, iface) of the device copy
    SUBROUTINE gpu_download_buffer(name, igrid, iface, buf)
        CHARACTER(len=*), INTENT(in) :: name
        INTEGER, INTENT(in) :: igrid, iface
        REAL(c_double), INTENT(out) :: buf(:)
        IF (mglet_gpu_get_buffer(gctx, TRIM(name)//C_NULL_CHAR, INT(igrid, c_int32_t), &
            INT(iface, c_int32_t), buf, INT(SIZE(buf), c_int64_t)) /= 0) &
            CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_download_buffer

    ! The scalar ghost-cell list of grid igrid as create_scastencils leaves
    ! it: ncells cells of 9 integers (scaxpoli) and 8 reals (scaxpolr,
    ! scaxpolrvel)
    SUBROUTINE gpu_set_scastencils(igrid, ncells, xpoli, xpolr, xpolrvel)
        INTEGER, INTENT(in) :: igrid, ncells
        INTEGER(c_int64_t), INTENT(in) :: xpoli(:)
        REAL(c_double), INTENT(in) :: xpolr(:), xpolrvel(:)
        IF (mglet_gpu_set_scastencils(gctx, INT(igrid, c_int32_t), INT(ncells, c_int32_t), xpoli, &
            xpolr, xpolrvel) /= 0) CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_set_scastencils

    ! sca%geometries of scalar isca: per body flag (0 fixed value, 1 fixed
    ! flux) and value
    SUBROUTINE gpu_set_scalar_geometry(isca, flag, value)
        INTEGER, INTENT(in) :: isca
        INTEGER(c_int32_t), INTENT(in) :: flag(:)
        REAL(c_double), INTENT(in) :: value(:)
        IF (mglet_gpu_set_scalar_geometry(gctx, INT(isca, c_int32_t), INT(SIZE(flag), c_int32_t), &
            flag, value) /= 0) CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_set_scalar_geometry

    SUBROUTINE gpu_synchronize()
        IF (mglet_gpu_synchronize(gctx) /= 0) CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_synchronize

    ! The launch variants the mixed form's tuner chose, as text
    SUBROUTINE gpu_tuning(text)
        CHARACTER(len=*), INTENT(out) :: text
        CHARACTER(kind=c_char) :: buf(4096)
        INTEGER :: q
        IF (mglet_gpu_tuning(gctx, buf, INT(SIZE(buf), c_int64_t)) /= 0) &
            CALL errr(__FILE__, __LINE__)
        text = ''
        DO q = 1, MIN(LEN(text), SIZE(buf))
            IF (buf(q) == C_NULL_CHAR) EXIT
            text(q:q) = buf(q)
        END DO
    END SUBROUTINE gpu_tuning

    SUBROUTINE gpu_force_variant(kernel, variant)
        CHARACTER(len=*), INTENT(in) :: kernel
        INTEGER, INTENT(in) :: variant
        IF (mglet_gpu_force_variant(gctx, TRIM(kernel)//C_NULL_CHAR, INT(variant, c_int32_t)) /= 0) &
            CALL errr(__FILE__, __LINE__)
    END SUBROUTINE gpu_force_variant

    SUBROUTINE gpu_itinfo(dt, cflmax, divmax, energy, exploded)
        REAL(c_double), INTENT(in) :: dt
        REAL(c_double), INTENT(out) :: cflmax, divmax, energy
        INTEGER, INTENT(inout) :: exploded
        TYPE(mglet_itinfo) :: info
        INTEGER(c_int) :: rc
        rc = mglet_gpu_itinfo(gctx, dt, info)
        IF (rc /= 0 .AND. rc /= 6) CALL errr(__FILE__, __LINE__)
        cflmax = info%cflmax
        divmax = info%divmax
        energy = info%energy
        IF (info%exploded /= 0) exploded = 1
    END SUBROUTINE gpu_itinfo
END MODULE mglet_gpu_mod
