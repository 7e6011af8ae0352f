!-----------------------------------------------------------------------
! openmhd_gb300.f90 -- iso_c_binding interfaces to libopenmhd_gb300.so for
! OpenMHD-style Fortran drivers.
!
! `use openmhd_gb300` gives generic subroutines with the reference's names and
! argument lists (u2v, limiter, flux_solver, rk_tvd21/22, rk_std21/22,
! glm_ss2, set_dt, bc, flux_resistive, set_dt_resistive), resolved by array
! rank between the 2D and 3D forms.  Arrays are the drivers' own column-major
! arrays; host arrays are mirrored to the GPU by the library, device arrays
! (CUDA Fortran, compile with -D_CUDA) are used in place.  A failure prints
! the reference's message and stops, as the reference routines do.
!
! Link: gfortran main.f90 model.f90 ... -L<dir> -lopenmhd_gb300 -lcudart
!-----------------------------------------------------------------------
#ifdef _CUDA
#define DEVATTR , device
#else
#define DEVATTR
#endif
module openmhd_gb300
  use iso_c_binding
  implicit none
  private
  public :: u2v, limiter, flux_solver, rk_tvd21, rk_tvd22, rk_std21, rk_std22
  public :: glm_ss2, set_dt, bc, flux_resistive, set_dt_resistive

  interface
     integer(c_int) function c_u2v_2d(U, V, ix, jx) bind(C, name="omhd_u2v_2d")
       import :: c_int, c_double
       real(c_double) DEVATTR, intent(in) :: U(*)
       real(c_double) DEVATTR :: V(*)
       integer(c_int), value :: ix, jx
     end function
     integer(c_int) function c_u2v_3d(U, V, ix, jx, kx) bind(C, name="omhd_u2v_3d")
       import :: c_int, c_double
       real(c_double) DEVATTR, intent(in) :: U(*)
       real(c_double) DEVATTR :: V(*)
       integer(c_int), value :: ix, jx, kx
     end function
     integer(c_int) function c_limiter_2d(wk, wL, wR, ix, jx, dir, type) bind(C, name="omhd_limiter_2d")
       import :: c_int, c_double
       real(c_double) DEVATTR, intent(in) :: wk(*)
       real(c_double) DEVATTR :: wL(*), wR(*)
       integer(c_int), value :: ix, jx, dir, type
     end function
     integer(c_int) function c_limiter_3d(wk, wL, wR, ix, jx, kx, dir, type) bind(C, name="omhd_limiter_3d")
       import :: c_int, c_double
       real(c_double) DEVATTR, intent(in) :: wk(*)
       real(c_double) DEVATTR :: wL(*), wR(*)
       integer(c_int), value :: ix, jx, kx, dir, type
     end function
     integer(c_int) function c_flux_2d(F, VL, VR, ch, ix, jx, dir, type) bind(C, name="omhd_flux_solver_2d")
       import :: c_int, c_double
       real(c_double) DEVATTR :: F(*)
       real(c_double) DEVATTR, intent(in) :: VL(*), VR(*)
       real(c_double), value :: ch
       integer(c_int), value :: ix, jx, dir, type
     end function
     integer(c_int) function c_flux_3d(F, VL, VR, ch, ix, jx, kx, dir, type) bind(C, name="omhd_flux_solver_3d")
       import :: c_int, c_double
       real(c_double) DEVATTR :: F(*)
       real(c_double) DEVATTR, intent(in) :: VL(*), VR(*)
       real(c_double), value :: ch
       integer(c_int), value :: ix, jx, kx, dir, type
     end function
     integer(c_int) function c_rk_2d(U, U1, F, G, dt, dx, ix, jx) bind(C, name="omhd_rk_tvd21_2d")
       import :: c_int, c_double
       real(c_double) DEVATTR :: U(*), U1(*)
       real(c_double) DEVATTR, intent(in) :: F(*), G(*)
       real(c_double), value :: dt, dx
       integer(c_int), value :: ix, jx
     end function
     integer(c_int) function c_rk22_2d(U, U1, F, G, dt, dx, ix, jx) bind(C, name="omhd_rk_tvd22_2d")
       import :: c_int, c_double
       real(c_double) DEVATTR :: U(*), U1(*)
       real(c_double) DEVATTR, intent(in) :: F(*), G(*)
       real(c_double), value :: dt, dx
       integer(c_int), value :: ix, jx
     end function
     integer(c_int) function c_std21_2d(U, U1, F, G, dt, dx, ix, jx) bind(C, name="omhd_rk_std21_2d")
       import :: c_int, c_double
       real(c_double) DEVATTR :: U(*), U1(*)
       real(c_double) DEVATTR, intent(in) :: F(*), G(*)
       real(c_double), value :: dt, dx
       integer(c_int), value :: ix, jx
     end function
     integer(c_int) function c_std22_2d(U, F, G, dt, dx, ix, jx) bind(C, name="omhd_rk_std22_2d")
       import :: c_int, c_double
       real(c_double) DEVATTR :: U(*)
       real(c_double) DEVATTR, intent(in) :: F(*), G(*)
       real(c_double), value :: dt, dx
       integer(c_int), value :: ix, jx
     end function
     integer(c_int) function c_rk_3d(U, U1, F, G, H, dt, dx, ix, jx, kx) bind(C, name="omhd_rk_tvd21_3d")
       import :: c_int, c_double
       real(c_double) DEVATTR :: U(*), U1(*)
       real(c_double) DEVATTR, intent(in) :: F(*), G(*), H(*)
       real(c_double), value :: dt, dx
       integer(c_int), value :: ix, jx, kx
     end function
     integer(c_int) function c_rk22_3d(U, U1, F, G, H, dt, dx, ix, jx, kx) bind(C, name="omhd_rk_tvd22_3d")
       import :: c_int, c_double
       real(c_double) DEVATTR :: U(*), U1(*)
       real(c_double) DEVATTR, intent(in) :: F(*), G(*), H(*)
       real(c_double), value :: dt, dx
       integer(c_int), value :: ix, jx, kx
     end function
     integer(c_int) function c_std21_3d(U, U1, F, G, H, dt, dx, ix, jx, kx) bind(C, name="omhd_rk_std21_3d")
       import :: c_int, c_double
       real(c_double) DEVATTR :: U(*), U1(*)
       real(c_double) DEVATTR, intent(in) :: F(*), G(*), H(*)
       real(c_double), value :: dt, dx
       integer(c_int), value :: ix, jx, kx
     end function
     integer(c_int) function c_std22_3d(U, F, G, H, dt, dx, ix, jx, kx) bind(C, name="omhd_rk_std22_3d")
       import :: c_int, c_double
       real(c_double) DEVATTR :: U(*)
       real(c_double) DEVATTR, intent(in) :: F(*), G(*), H(*)
       real(c_double), value :: dt, dx
       integer(c_int), value :: ix, jx, kx
     end function
     integer(c_int) function c_glm_2d(U, ch, dt, ix, jx) bind(C, name="omhd_glm_ss2_2d")
       import :: c_int, c_double
       real(c_double) DEVATTR :: U(*)
       real(c_double), value :: ch, dt
       integer(c_int), value :: ix, jx
     end function
     integer(c_int) function c_glm_3d(U, ch, dt, ix, jx, kx) bind(C, name="omhd_glm_ss2_3d")
       import :: c_int, c_double
       real(c_double) DEVATTR :: U(*)
       real(c_double), value :: ch, dt
       integer(c_int), value :: ix, jx, kx
     end function
     integer(c_int) function c_set_dt_2d(U, V, vmax, dt, dx, cfl, ix, jx) bind(C, name="omhd_set_dt_2d")
       import :: c_int, c_double
       real(c_double) DEVATTR, intent(in) :: U(*), V(*)
       real(c_double), intent(out) :: vmax, dt
       real(c_double), value :: dx, cfl
       integer(c_int), value :: ix, jx
     end function
     integer(c_int) function c_set_dt_3d(U, V, vmax, dt, dx, cfl, ix, jx, kx) bind(C, name="omhd_set_dt_3d")
       import :: c_int, c_double
       real(c_double) DEVATTR, intent(in) :: U(*), V(*)
       real(c_double), intent(out) :: vmax, dt
       real(c_double), value :: dx, cfl
       integer(c_int), value :: ix, jx, kx
     end function
     integer(c_int) function c_bc_2d(U, ix, jx, kind, flip) bind(C, name="omhd_bc_2d")
       import :: c_int, c_double
       real(c_double) DEVATTR :: U(*)
       integer(c_int), value :: ix, jx
       integer(c_int), intent(in) :: kind(4), flip(4)
     end function
     integer(c_int) function c_bc_3d(U, ix, jx, kx, kind, flip) bind(C, name="omhd_bc_3d")
       import :: c_int, c_double
       real(c_double) DEVATTR :: U(*)
       integer(c_int), value :: ix, jx, kx
       integer(c_int), intent(in) :: kind(6), flip(6)
     end function
     integer(c_int) function c_resist_2d(F, U, x, y, dx, ix, jx, dir, eta) bind(C, name="omhd_flux_resistive_2d")
       import :: c_int, c_double
       real(c_double) DEVATTR :: F(*)
       real(c_double) DEVATTR, intent(in) :: U(*), x(*), y(*)
       real(c_double), value :: dx
       integer(c_int), value :: ix, jx, dir, eta
     end function
     integer(c_int) function c_resist_3d(F, U, x, y, z, dx, ix, jx, kx, dir, eta) bind(C, name="omhd_flux_resistive_3d")
       import :: c_int, c_double
       real(c_double) DEVATTR :: F(*)
       real(c_double) DEVATTR, intent(in) :: U(*), x(*), y(*), z(*)
       real(c_double), value :: dx
       integer(c_int), value :: ix, jx, kx, dir, eta
     end function
     integer(c_int) function c_set_dt_resistive(dt, dx, cfl, eta) bind(C, name="omhd_set_dt_resistive")
       import :: c_int, c_double
       real(c_double), intent(inout) :: dt
       real(c_double), value :: dx, cfl
       integer(c_int), value :: eta
     end function
     subroutine c_abort_on_error(on) bind(C, name="omhd_set_abort_on_error")
       import :: c_int
       integer(c_int), value :: on
     end subroutine
  end interface

  interface u2v
     module procedure u2v_2d, u2v_3d
  end interface
  interface limiter
     module procedure limiter_2d, limiter_3d
  end interface
  interface flux_solver
     module procedure flux_solver_2d, flux_solver_3d
  end interface
  interface rk_tvd21
     module procedure rk_tvd21_2d, rk_tvd21_3d
  end interface
  interface rk_tvd22
     module procedure rk_tvd22_2d, rk_tvd22_3d
  end interface
  interface rk_std21
     module procedure rk_std21_2d, rk_std21_3d
  end interface
  interface rk_std22
     module procedure rk_std22_2d, rk_std22_3d
  end interface
  interface glm_ss2
     module procedure glm_ss2_2d, glm_ss2_3d
  end interface
  interface set_dt
     module procedure set_dt_2d, set_dt_3d
  end interface
  interface bc
     module procedure bc_2d, bc_3d
  end interface
  interface flux_resistive
     module procedure flux_resistive_2d, flux_resistive_3d
  end interface

contains

  ! every routine below fails like the reference: the library prints the
  ! reference's message and ends the program (omhd_set_abort_on_error(1))
  subroutine u2v_2d(U, V, ix, jx)
    integer, intent(in) :: ix, jx
    real(8) DEVATTR, intent(in) :: U(ix, jx, 9)
    real(8) DEVATTR, intent(out) :: V(ix, jx, 4)
    call check(c_u2v_2d(U, V, ix, jx))
  end subroutine
  subroutine u2v_3d(U, V, ix, jx, kx)
    integer, intent(in) :: ix, jx, kx
    real(8) DEVATTR, intent(in) :: U(ix, jx, kx, 9)
    real(8) DEVATTR, intent(out) :: V(ix, jx, kx, 4)
    call check(c_u2v_3d(U, V, ix, jx, kx))
  end subroutine
  subroutine limiter_2d(wk, wL, wR, ix, jx, dir, type)
    integer, intent(in) :: ix, jx, dir, type
    real(8) DEVATTR, intent(in) :: wk(ix, jx)
    real(8) DEVATTR, intent(inout) :: wL(ix, jx), wR(ix, jx)
    call check(c_limiter_2d(wk, wL, wR, ix, jx, dir, type))
  end subroutine
  subroutine limiter_3d(wk, wL, wR, ix, jx, kx, dir, type)
    integer, intent(in) :: ix, jx, kx, dir, type
    real(8) DEVATTR, intent(in) :: wk(ix, jx, kx)
    real(8) DEVATTR, intent(inout) :: wL(ix, jx, kx), wR(ix, jx, kx)
    call check(c_limiter_3d(wk, wL, wR, ix, jx, kx, dir, type))
  end subroutine
  subroutine flux_solver_2d(F, VL, VR, ch, ix, jx, dir, type)
    integer, intent(in) :: ix, jx, dir, type
    real(8) DEVATTR, intent(out) :: F(ix, jx, 9)
    real(8) DEVATTR, intent(in) :: VL(ix, jx, 9), VR(ix, jx, 9)
    real(8), intent(in) :: ch
    call check(c_flux_2d(F, VL, VR, ch, ix, jx, dir, type))
  end subroutine
  subroutine flux_solver_3d(F, VL, VR, ch, ix, jx, kx, dir, type)
    integer, intent(in) :: ix, jx, kx, dir, type
    real(8) DEVATTR, intent(out) :: F(ix, jx, kx, 9)
    real(8) DEVATTR, intent(in) :: VL(ix, jx, kx, 9), VR(ix, jx, kx, 9)
    real(8), intent(in) :: ch
    call check(c_flux_3d(F, VL, VR, ch, ix, jx, kx, dir, type))
  end subroutine
  subroutine rk_tvd21_2d(U, U1, F, G, dt, dx, ix, jx)
    integer, intent(in) :: ix, jx
    real(8) DEVATTR :: U(ix, jx, 9), U1(ix, jx, 9)
    real(8) DEVATTR, intent(in) :: F(ix, jx, 9), G(ix, jx, 9)
    real(8), intent(in) :: dt, dx
    call check(c_rk_2d(U, U1, F, G, dt, dx, ix, jx))
  end subroutine
  subroutine rk_tvd22_2d(U, U1, F, G, dt, dx, ix, jx)
    integer, intent(in) :: ix, jx
    real(8) DEVATTR :: U(ix, jx, 9), U1(ix, jx, 9)
    real(8) DEVATTR, intent(in) :: F(ix, jx, 9), G(ix, jx, 9)
    real(8), intent(in) :: dt, dx
    call check(c_rk22_2d(U, U1, F, G, dt, dx, ix, jx))
  end subroutine
  subroutine rk_std21_2d(U, U1, F, G, dt, dx, ix, jx)
    integer, intent(in) :: ix, jx
    real(8) DEVATTR :: U(ix, jx, 9), U1(ix, jx, 9)
    real(8) DEVATTR, intent(in) :: F(ix, jx, 9), G(ix, jx, 9)
    real(8), intent(in) :: dt, dx
    call check(c_std21_2d(U, U1, F, G, dt, dx, ix, jx))
  end subroutine
  subroutine rk_std22_2d(U, F, G, dt, dx, ix, jx)
    integer, intent(in) :: ix, jx
    real(8) DEVATTR :: U(ix, jx, 9)
    real(8) DEVATTR, intent(in) :: F(ix, jx, 9), G(ix, jx, 9)
    real(8), intent(in) :: dt, dx
    call check(c_std22_2d(U, F, G, dt, dx, ix, jx))
  end subroutine
  subroutine rk_tvd21_3d(U, U1, F, G, H, dt, dx, ix, jx, kx)
    integer, intent(in) :: ix, jx, kx
    real(8) DEVATTR :: U(ix, jx, kx, 9), U1(ix, jx, kx, 9)
    real(8) DEVATTR, intent(in) :: F(ix, jx, kx, 9), G(ix, jx, kx, 9), H(ix, jx, kx, 9)
    real(8), intent(in) :: dt, dx
    call check(c_rk_3d(U, U1, F, G, H, dt, dx, ix, jx, kx))
  end subroutine
  subroutine rk_tvd22_3d(U, U1, F, G, H, dt, dx, ix, jx, kx)
    integer, intent(in) :: ix, jx, kx
    real(8) DEVATTR :: U(ix, jx, kx, 9), U1(ix, jx, kx, 9)
    real(8) DEVATTR, intent(in) :: F(ix, jx, kx, 9), G(ix, jx, kx, 9), H(ix, jx, kx, 9)
    real(8), intent(in) :: dt, dx
    call check(c_rk22_3d(U, U1, F, G, H, dt, dx, ix, jx, kx))
  end subroutine
  subroutine rk_std21_3d(U, U1, F, G, H, dt, dx, ix, jx, kx)
    integer, intent(in) :: ix, jx, kx
    real(8) DEVATTR :: U(ix, jx, kx, 9), U1(ix, jx, kx, 9)
    real(8) DEVATTR, intent(in) :: F(ix, jx, kx, 9), G(ix, jx, kx, 9), H(ix, jx, kx, 9)
    real(8), intent(in) :: dt, dx
    call check(c_std21_3d(U, U1, F, G, H, dt, dx, ix, jx, kx))
  end subroutine
  subroutine rk_std22_3d(U, F, G, H, dt, dx, ix, jx, kx)
    integer, intent(in) :: ix, jx, kx
    real(8) DEVATTR :: U(ix, jx, kx, 9)
    real(8) DEVATTR, intent(in) :: F(ix, jx, kx, 9), G(ix, jx, kx, 9), H(ix, jx, kx, 9)
    real(8), intent(in) :: dt, dx
    call check(c_std22_3d(U, F, G, H, dt, dx, ix, jx, kx))
  end subroutine
  subroutine glm_ss2_2d(U, ch, dt, ix, jx)
    integer, intent(in) :: ix, jx
    real(8) DEVATTR :: U(ix, jx, 9)
    real(8), intent(in) :: ch, dt
    call check(c_glm_2d(U, ch, dt, ix, jx))
  end subroutine
  subroutine glm_ss2_3d(U, ch, dt, ix, jx, kx)
    integer, intent(in) :: ix, jx, kx
    real(8) DEVATTR :: U(ix, jx, kx, 9)
    real(8), intent(in) :: ch, dt
    call check(c_glm_3d(U, ch, dt, ix, jx, kx))
  end subroutine
  subroutine set_dt_2d(U, V, vmax, dt, dx, cfl, ix, jx)
    integer, intent(in) :: ix, jx
    real(8) DEVATTR, intent(in) :: U(ix, jx, 9), V(ix, jx, 4)
    real(8), intent(out) :: vmax, dt
    real(8), intent(in) :: dx, cfl
    call check(c_set_dt_2d(U, V, vmax, dt, dx, cfl, ix, jx))
  end subroutine
  subroutine set_dt_3d(U, V, vmax, dt, dx, cfl, ix, jx, kx)
    integer, intent(in) :: ix, jx, kx
    real(8) DEVATTR, intent(in) :: U(ix, jx, kx, 9), V(ix, jx, kx, 4)
    real(8), intent(out) :: vmax, dt
    real(8), intent(in) :: dx, cfl
    call check(c_set_dt_3d(U, V, vmax, dt, dx, cfl, ix, jx, kx))
  end subroutine
  subroutine bc_2d(U, ix, jx)          ! 2D_basic/bc.f90: periodic on all sides
    integer, intent(in) :: ix, jx
    real(8) DEVATTR :: U(ix, jx, 9)
    integer(c_int) :: kind(4) = 0, flip(4) = 0
    call check(c_bc_2d(U, ix, jx, kind, flip))
  end subroutine
  subroutine bc_3d(U, ix, jx, kx)      ! 3D_basic/bc.f90: periodic on all sides
    integer, intent(in) :: ix, jx, kx
    real(8) DEVATTR :: U(ix, jx, kx, 9)
    integer(c_int) :: kind(6) = 0, flip(6) = 0
    call check(c_bc_3d(U, ix, jx, kx, kind, flip))
  end subroutine
  subroutine flux_resistive_2d(F, U, x, y, dx, ix, jx, dir)   ! eta of 2D_reconnection
    integer, intent(in) :: ix, jx, dir
    real(8) DEVATTR :: F(ix, jx, 9)
    real(8) DEVATTR, intent(in) :: U(ix, jx, 9), x(ix), y(jx)
    real(8), intent(in) :: dx
    call check(c_resist_2d(F, U, x, y, dx, ix, jx, dir, 1))
  end subroutine
  subroutine flux_resistive_3d(F, U, x, y, z, dx, ix, jx, kx, dir)   ! Harris-xz eta
    integer, intent(in) :: ix, jx, kx, dir
    real(8) DEVATTR :: F(ix, jx, kx, 9)
    real(8) DEVATTR, intent(in) :: U(ix, jx, kx, 9), x(ix), y(jx), z(kx)
    real(8), intent(in) :: dx
    call check(c_resist_3d(F, U, x, y, z, dx, ix, jx, kx, dir, 2))
  end subroutine
  subroutine set_dt_resistive(dt, dx, cfl)
    real(8), intent(inout) :: dt
    real(8), intent(in) :: dx, cfl
    call check(c_set_dt_resistive(dt, dx, cfl, 1))
  end subroutine

  subroutine check(st)
    integer(c_int), intent(in) :: st
    if (st /= 0) then
       write(6, *) 'openmhd_gb300: status ', st
       stop
    endif
  end subroutine
end module openmhd_gb300
