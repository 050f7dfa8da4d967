!-----------------------------------------------------------------------
!  mhd_gpu_binding.f90
!  iso_c_binding interface of libmhdgpu.so (include/mhd_gpu.h) for the
!  unchanged Fortran driver of mhd3d3.f90.  Compile with the driver
!  (mpif90 -r8 ... mhd_gpu_binding.f90 mhd3d3.f90 -L<lib> -lmhdgpu).
!
!  The reference's `call step` (mhd3d3.f90:3286) becomes
!     call gpu_step(tau)
!  after `call gpu_init` at the end of `initialization` (mhd3d3.f90:3375),
!  and `call gpu_fetch` before `outputxyz` / `diag_*` (mhd3d3.f90:3289-3298).
!-----------------------------------------------------------------------
module mhd_gpu_binding
   use iso_c_binding
   implicit none

   type, bind(C) :: mhd_params
      integer(c_int32_t) :: nx0, ny0, nz0
      integer(c_int32_t) :: nord, reconop, stepop
      integer(c_int32_t) :: bc(3)
      integer(c_int32_t) :: precision, dt_mode, tvd_shift
      real(c_double)     :: gam, cfl, pdmb, eps, alpha, beta
      real(c_double)     :: tau
      integer(c_int32_t) :: emf
      integer(c_int32_t) :: reserved(7)
   end type mhd_params

   interface
      integer(c_int) function mhd_init(prm, rho, vx, vy, vz, p, bi, bj, bk, dx, dy, dz, h) &
            bind(C, name="mhd_init")
         import :: c_int, c_double, c_ptr, mhd_params
         type(mhd_params), intent(in) :: prm
         real(c_double), intent(in) :: rho(*), vx(*), vy(*), vz(*), p(*)
         real(c_double), intent(in) :: bi(*), bj(*), bk(*), dx(*), dy(*), dz(*)
         type(c_ptr), intent(out) :: h
      end function mhd_init

      integer(c_int) function mhd_step(h, tau, status) bind(C, name="mhd_step")
         import :: c_int, c_double, c_ptr, c_int32_t
         type(c_ptr), value :: h
         real(c_double), intent(inout) :: tau
         integer(c_int32_t), intent(out) :: status
      end function mhd_step

      integer(c_int) function mhd_step_n(h, n, tau, status) bind(C, name="mhd_step_n")
         import :: c_int, c_double, c_ptr, c_int32_t
         type(c_ptr), value :: h
         integer(c_int32_t), value :: n
         real(c_double), intent(out) :: tau
         integer(c_int32_t), intent(out) :: status
      end function mhd_step_n

      integer(c_int) function mhd_fetch(h, rho, vx, vy, vz, p, bx, by, bz, bi, bj, bk) &
            bind(C, name="mhd_fetch")
         import :: c_int, c_double, c_ptr
         type(c_ptr), value :: h
         real(c_double), intent(out) :: rho(*), vx(*), vy(*), vz(*), p(*)
         real(c_double), intent(out) :: bx(*), by(*), bz(*), bi(*), bj(*), bk(*)
      end function mhd_fetch

      integer(c_int) function mhd_set_tau(h, tau) bind(C, name="mhd_set_tau")
         import :: c_int, c_double, c_ptr
         type(c_ptr), value :: h
         real(c_double), value :: tau
      end function mhd_set_tau

      integer(c_int) function mhd_free(h) bind(C, name="mhd_free")
         import :: c_int, c_ptr
         type(c_ptr), value :: h
      end function mhd_free

      integer(c_int) function mhd_diagnostics(h, out) bind(C, name="mhd_diagnostics")
         import :: c_int, c_double, c_ptr
         type(c_ptr), value :: h
         real(c_double), intent(out) :: out(*)
      end function mhd_diagnostics
   end interface

   type(c_ptr), save :: gpu_handle = c_null_ptr

contains

   !..the driver's deck scalars and module arrays -> device (end of initialization)
   subroutine gpu_init(nx0, ny0, nz0, nord, reconop, stepop, bcs, prec, gam, cfl, pdmb, eps, &
                       alpha, beta, tau, rho, vx, vy, vz, p, bi, bj, bk, dx, dy, dz)
      integer, intent(in) :: nx0, ny0, nz0, nord, reconop, stepop, bcs(3), prec
      real(c_double), intent(in) :: gam, cfl, pdmb, eps, alpha, beta, tau
      real(c_double), intent(in) :: rho(*), vx(*), vy(*), vz(*), p(*), bi(*), bj(*), bk(*)
      real(c_double), intent(in) :: dx(*), dy(*), dz(*)
      type(mhd_params) :: prm
      integer(c_int) :: rc
      prm%nx0 = nx0; prm%ny0 = ny0; prm%nz0 = nz0
      prm%nord = nord; prm%reconop = reconop; prm%stepop = stepop
      prm%bc = bcs; prm%precision = prec; prm%dt_mode = 0; prm%tvd_shift = 0
      prm%gam = gam; prm%cfl = cfl; prm%pdmb = pdmb; prm%eps = eps
      prm%alpha = alpha; prm%beta = beta; prm%tau = tau; prm%emf = 0; prm%reserved = 0
      rc = mhd_init(prm, rho, vx, vy, vz, p, bi, bj, bk, dx, dy, dz, gpu_handle)
      if (rc /= 0) stop 'mhd_init failed'
   end subroutine gpu_init

   !..replaces `call step`: tau goes in as the driver's module tau (for RK with
   !  the deck dt, a changed positive tau becomes the fixed dt tau0) and comes
   !  back as the module tau after the step (AB: its CFL dt)
   subroutine gpu_step(tau)
      real(c_double), intent(inout) :: tau
      integer(c_int32_t) :: status
      integer(c_int) :: rc
      rc = mhd_step(gpu_handle, tau, status)
      if (rc /= 0) stop 'mhd_step failed'
      if (iand(status, 3) /= 0) stop 'NaN or negative density (device check)'
   end subroutine gpu_step

   !..sets the fixed RK dt (the module tau0) outright, e.g. after a restart
   subroutine gpu_set_tau(tau)
      real(c_double), intent(in) :: tau
      integer(c_int) :: rc
      rc = mhd_set_tau(gpu_handle, tau)
      if (rc /= 0) stop 'mhd_set_tau failed'
   end subroutine gpu_set_tau

   subroutine gpu_fetch(rho, vx, vy, vz, p, bx, by, bz, bi, bj, bk)
      real(c_double), intent(out) :: rho(*), vx(*), vy(*), vz(*), p(*), bx(*), by(*), bz(*)
      real(c_double), intent(out) :: bi(*), bj(*), bk(*)
      integer(c_int) :: rc
      rc = mhd_fetch(gpu_handle, rho, vx, vy, vz, p, bx, by, bz, bi, bj, bk)
      if (rc /= 0) stop 'mhd_fetch failed'
   end subroutine gpu_fetch

   !..device diagnostics for the driver's diag_* step (mhd3d3.f90:3137-3160):
   !  mass and total energy (compensated FP64 sums), max |div B|, min rho
   !  (diag_rho_neg) and the CFL dt (get_dt)
   subroutine gpu_diagnostics(mass, energy, divb_max, rho_min, dt_cfl)
      real(c_double), intent(out) :: mass, energy, divb_max, rho_min, dt_cfl
      real(c_double) :: out(5)
      integer(c_int) :: rc
      rc = mhd_diagnostics(gpu_handle, out)
      if (rc /= 0) stop 'mhd_diagnostics failed'
      mass = out(1); energy = out(2); divb_max = out(3); rho_min = out(4); dt_cfl = out(5)
   end subroutine gpu_diagnostics

   subroutine gpu_free()
      integer(c_int) :: rc
      rc = mhd_free(gpu_handle)
      gpu_handle = c_null_ptr
   end subroutine gpu_free

end module mhd_gpu_binding
