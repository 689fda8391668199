! Fortran interface to libp3x's Fortran-layout P3 entry (include/p3x.h).
!
! p3x_main_f takes the arguments of the reference's C-bound Fortran entry
! p3_main_c (components/eamxx/src/physics/p3/p3_iso_c.f90:132-183) in the same
! order and meaning: host arrays in the (its:ite, kts:kte) column-fastest
! layout, level kts at the model top.  The library copies them to the GPU,
! runs the FP64 P3 step there and copies the results back; elapsed_s returns
! the device time of the step.  Status codes are the P3X_* values of p3x.h
! (0 = success).
!
! p3x_init replaces p3_init_c (p3_iso_c.f90:43-130): pass c_null_ptr to build
! the lookup tables in-process, or the address of a NUL-terminated path of a
! "VERSION 4.1.1" ice-table file.  info receives 0 or the negative status.
module p3x_mod
  use iso_c_binding, only: c_int, c_bool, c_double, c_ptr
  implicit none
  private
  public :: p3x_init, p3x_finalize, p3x_main_f

  interface
    function p3x_init(table_file, info) bind(C, name="p3x_init") result(status)
      import :: c_int, c_ptr
      type(c_ptr), value :: table_file
      integer(c_int), intent(out) :: info
      integer(c_int) :: status
    end function p3x_init

    function p3x_finalize() bind(C, name="p3x_finalize") result(status)
      import :: c_int
      integer(c_int) :: status
    end function p3x_finalize

    function p3x_main_f(qc, nc, qr, nr, th_atm, qv, dt, qi, qm, ni, bm, pres, dz, nc_nuceat_tend, &
                        nccn_prescribed, ni_activated, inv_qc_relvar, it, precip_liq_surf, precip_ice_surf, &
                        its, ite, kts, kte, diag_eff_radius_qc, diag_eff_radius_qi, diag_eff_radius_qr, &
                        rho_qi, do_predict_nc, do_prescribed_ccn, dpres, inv_exner, qv2qi_depos_tend, &
                        precip_liq_flux, precip_ice_flux, cld_frac_r, cld_frac_l, cld_frac_i, &
                        liq_ice_exchange, vap_liq_exchange, vap_ice_exchange, qv_prev, t_prev, elapsed_s) &
        bind(C, name="p3x_main_f") result(status)
      import :: c_int, c_bool, c_double
      integer(c_int), value :: its, ite, kts, kte, it
      logical(c_bool), value :: do_predict_nc, do_prescribed_ccn
      real(c_double), value :: dt
      real(c_double), intent(inout), dimension(its:ite, kts:kte) :: qc, nc, qr, nr, th_atm, qv, qi, qm, &
                                                                    ni, bm
      real(c_double), intent(in), dimension(its:ite, kts:kte) :: pres, dz, nc_nuceat_tend, &
                                                                 nccn_prescribed, ni_activated, &
                                                                 inv_qc_relvar, dpres, inv_exner, &
                                                                 cld_frac_r, cld_frac_l, cld_frac_i, &
                                                                 qv_prev, t_prev
      real(c_double), intent(out), dimension(its:ite) :: precip_liq_surf, precip_ice_surf
      real(c_double), intent(out), dimension(its:ite, kts:kte) :: diag_eff_radius_qc, diag_eff_radius_qi, &
                                                                  diag_eff_radius_qr, rho_qi, &
                                                                  qv2qi_depos_tend, liq_ice_exchange, &
                                                                  vap_liq_exchange, vap_ice_exchange
      real(c_double), intent(out), dimension(its:ite, kts:kte+1) :: precip_liq_flux, precip_ice_flux
      real(c_double), intent(out) :: elapsed_s
      integer(c_int) :: status
    end function p3x_main_f
  end interface
end module p3x_mod
