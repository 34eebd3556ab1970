! Fortran 2003 interface (ISO_C_BINDING) of the C ABI in elastic_gb300.h,
! for the reference's Fortran driver: `use elastic_gb300` and link with
! -lelastic_gb300.  Every routine returns the ELX_* status of the C call
! (elx_destroy / elx_host_structure_destroy return nothing); a non-zero
! status is where the reference would call stop_mef.
!
! Arrays are passed as the driver's pool slices (ia(i_ix), ia(i_x), ...):
! by reference, Fortran layout, 1-based index contents -- the C side reads
! them as they are.  Optional outputs of the C ABI (NULL there) are
! type(c_ptr), value arguments here: pass c_null_ptr to leave them out,
! or c_loc(array) to have them filled.
!
! Entry points and the reference routines they replace (see the header for
! the argument meanings):
!   elx_set_structure / elx_build_structure  reord + numeq + csrstruct (Main.f:412-491)
!   elx_assemble       pform_mec isw = 2 (Pform.f:1-254, Main.f:791-802)
!   elx_solve          solv (Solv.f:13-440, Main.f:820-826)
!   elx_set_loads      pload_mec + the 2-D edge loads of pform_mec isw = 4
!   elx_update         update_mec (Predict.f:183-209)
!   elx_stress         tform_mec isw = 3 (Pform.f:258-421, Main.f:893-901)
!   elx_write_vtk      write_mesh_res_mec (Write_vtk.f:742-985)
module elastic_gb300
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: ELX_OK = 0, ELX_ERR_ZERO_DIAG = 1, &
      ELX_ERR_NO_CONVERGENCE = 2, ELX_ERR_BAD_DET = 3, ELX_ERR_OOM = 4, &
      ELX_ERR_TIMEOUT = 5, ELX_ERR_ARG = 6, ELX_ERR_BAD_ELEMENT = 7, &
      ELX_ERR_CUDA = 8, ELX_ERR_STATE = 9
  integer(c_int32_t), parameter :: ELX_SOLVER_PCG = 1, ELX_SOLVER_GMRES = 2, &
      ELX_SOLVER_BICGSTAB = 4, ELX_SOLVER_BICGSTAB_NOPREC = 5
  integer(c_int32_t), parameter :: ELX_PREC_FP64 = 0, ELX_PREC_MIXED = 1
  integer(c_int32_t), parameter :: ELX_VTK_VTU_ASCII = 0, ELX_VTK_LEGACY_BINARY = 1
  integer(c_int32_t), parameter :: ELX_VTK_DESLOC = 1, ELX_VTK_STRESS = 2

  type, bind(C) :: elx_opts
    integer(c_int32_t) :: device = 0
    integer(c_int32_t) :: verbose = 0
    integer(c_int64_t) :: hbm_budget = 0
  end type elx_opts

  type, bind(C) :: elx_info
    integer(c_int32_t) :: iters, status
    real(c_double)     :: xkx, norm_x, norm_r, norm_m_r, conv, seconds, mflops
    integer(c_int32_t) :: refinements, inner_iters
  end type elx_info

  interface
    integer(c_int) function elx_create(ctx, opts) bind(C, name='elx_create')
      import :: c_ptr, c_int, elx_opts
      type(c_ptr), intent(out) :: ctx
      type(elx_opts), intent(in) :: opts
    end function

    subroutine elx_destroy(ctx) bind(C, name='elx_destroy')
      import :: c_ptr
      type(c_ptr), value :: ctx
    end subroutine

    type(c_ptr) function elx_last_error(ctx) bind(C, name='elx_last_error')
      import :: c_ptr
      type(c_ptr), value :: ctx
    end function

    integer(c_int64_t) function elx_device_bytes(ctx) bind(C, name='elx_device_bytes')
      import :: c_ptr, c_int64_t
      type(c_ptr), value :: ctx
    end function

    integer(c_int) function elx_set_mesh(ctx, ndm, ndf, nen, numel, nnode, ix, x, ie, e, &
                                         prop, numat) bind(C, name='elx_set_mesh')
      import :: c_ptr, c_int, c_int32_t, c_double
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: ndm, ndf, nen, numel, nnode, prop, numat
      integer(c_int32_t), intent(in) :: ix(*), ie(*)
      real(c_double), intent(in) :: x(*), e(*)
    end function

    integer(c_int) function elx_set_structure(ctx, neq, nad, id, ia, ja) &
        bind(C, name='elx_set_structure')
      import :: c_ptr, c_int, c_int32_t, c_int64_t
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: neq
      integer(c_int64_t), value :: nad
      integer(c_int32_t), intent(in) :: id(*), ia(*), ja(*)
    end function

    integer(c_int) function elx_build_structure(ctx, bc, reorder) &
        bind(C, name='elx_build_structure')
      import :: c_ptr, c_int, c_int32_t
      type(c_ptr), value :: ctx
      integer(c_int32_t), intent(in) :: bc(*)
      integer(c_int32_t), value :: reorder
    end function

    integer(c_int) function elx_get_sizes(ctx, neq, nad, ncolors) bind(C, name='elx_get_sizes')
      import :: c_ptr, c_int, c_int32_t, c_int64_t
      type(c_ptr), value :: ctx
      integer(c_int32_t), intent(out) :: neq, ncolors
      integer(c_int64_t), intent(out) :: nad
    end function

    integer(c_int) function elx_get_structure(ctx, perm, id, ia, ja) &
        bind(C, name='elx_get_structure')
      import :: c_ptr, c_int, c_int32_t
      type(c_ptr), value :: ctx
      integer(c_int32_t), intent(out) :: perm(*), id(*), ia(*), ja(*)
    end function

    integer(c_int) function elx_assemble(ctx, u, b0, b, ad, al) bind(C, name='elx_assemble')
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: u(*), b0(*)
      real(c_double), intent(out) :: b(*)
      type(c_ptr), value :: ad, al      ! c_null_ptr: keep K on the device
    end function

    integer(c_int) function elx_solve(ctx, solver, precision, tol, maxit, ngram, b, x, info) &
        bind(C, name='elx_solve')
      import :: c_ptr, c_int, c_int32_t, c_double, elx_info
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: solver, precision, maxit, ngram
      real(c_double), value :: tol
      real(c_double), intent(in) :: b(*)
      real(c_double), intent(out) :: x(*)
      type(elx_info), intent(out) :: info
    end function

    integer(c_int) function elx_solve_block(ctx, nrhs, precision, tol, maxit, width, b, x, &
                                            info) bind(C, name='elx_solve_block')
      import :: c_ptr, c_int, c_int32_t, c_double, elx_info
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: nrhs, precision, maxit, width
      real(c_double), value :: tol
      real(c_double), intent(in) :: b(*)        ! b(neq, nrhs)
      real(c_double), intent(out) :: x(*)       ! x(neq, nrhs)
      type(elx_info), intent(out) :: info(*)    ! info(nrhs)
    end function

    integer(c_int) function elx_set_loads(ctx, f, eload, loadvec, nload) &
        bind(C, name='elx_set_loads')
      import :: c_ptr, c_int, c_int32_t, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: f(*)         ! f(ndf, nnode)
      type(c_ptr), value :: eload, loadvec       ! c_null_ptr: no edge loads
      integer(c_int32_t), value :: nload
    end function

    integer(c_int) function elx_update(ctx, x, u) bind(C, name='elx_update')
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: x(*)
      real(c_double), intent(inout) :: u(*)
    end function

    integer(c_int) function elx_stress(ctx, u, tx0, t) bind(C, name='elx_stress')
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: ctx
      type(c_ptr), value :: u, tx0               ! u: c_null_ptr = the resident u
      real(c_double), intent(out) :: t(*)        ! t(ntn, nnode)
    end function

    integer(c_int) function elx_write_vtk(ctx, path, format, fields, bytes) &
        bind(C, name='elx_write_vtk')
      import :: c_ptr, c_int, c_int32_t, c_int64_t, c_char
      type(c_ptr), value :: ctx
      character(kind=c_char), intent(in) :: path(*)  ! NUL-terminated
      integer(c_int32_t), value :: format, fields
      integer(c_int64_t), intent(out) :: bytes
    end function
  end interface
end module elastic_gb300
