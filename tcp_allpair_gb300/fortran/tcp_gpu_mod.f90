! tcp_gpu_mod.f90 -- ISO_C_BINDING interfaces to libtcpgpu.so (include/tcp_gpu.h)
! and drop-in wrappers with the argument lists of the reference's step routines.
!
! A maintainer replaces force.f90 / vverlet.f90 in the reference's Makefile by
! this file, keeps data.f90 / main.f90 / init.f90 / result.f90, and links
! -L<pkg>/_build -ltcpgpu.  The wrappers keep the reference's names and
! arguments; NS, COMM, gsend/gemit/grec/pme and PSI are accepted and ignored
! (one GPU, no MPI ranks on the compute path).  Not compiled in this
! repository's tests: no Fortran compiler exists on either build machine.
MODULE TCP_GPU
  USE ISO_C_BINDING
  USE DATASTR
  IMPLICIT NONE

  TYPE, BIND(C) :: tcp_params
     REAL(C_DOUBLE) :: xm(2), q(2), tau, alpha_lgv, a, box(3), Te, Ti, rs, rc
     INTEGER(C_INT) :: K(3), order
     REAL(C_DOUBLE) :: dx_ee, dx_ei, dx_ii, dv_e, dv_i
     INTEGER(C_INT) :: ei_model
     REAL(C_DOUBLE) :: lambda_ei, charge_scale
     INTEGER(C_INT) :: precision, reciprocal, ewald_nmax2, thermo, thermo_period
     INTEGER(C_INT64_T) :: seed
  END TYPE tcp_params

  TYPE, BIND(C) :: tcp_energies
     REAL(C_DOUBLE) :: Ur, Uo, Um, Epot, mv2el, mv2ion
  END TYPE tcp_energies

  TYPE(C_PTR), SAVE :: ctx = C_NULL_PTR

  ! tcp_set_flags bits (include/tcp_gpu.h)
  INTEGER(C_INT), PARAMETER :: TCP_FLAG_RDF = 1, TCP_FLAG_VDF = 2, TCP_FLAG_ENERGY = 4, &
       TCP_FLAG_DETERMINISTIC = 8

  INTERFACE
     INTEGER(C_INT) FUNCTION tcp_create(p, nel, nion, device, out) BIND(C, NAME='tcp_create')
       IMPORT :: C_INT, C_PTR, tcp_params
       TYPE(tcp_params), INTENT(IN) :: p
       INTEGER(C_INT), VALUE :: nel, nion, device
       TYPE(C_PTR), INTENT(OUT) :: out
     END FUNCTION
     INTEGER(C_INT) FUNCTION tcp_ewald_self(c, alpha, uo) BIND(C, NAME='tcp_ewald_self')
       IMPORT :: C_INT, C_PTR, C_DOUBLE
       TYPE(C_PTR), VALUE :: c
       REAL(C_DOUBLE), INTENT(OUT) :: alpha, uo
     END FUNCTION
     INTEGER(C_INT) FUNCTION tcp_upload(c, species, xx, xv, ff, stride) BIND(C, NAME='tcp_upload')
       IMPORT :: C_INT, C_PTR, C_LONG
       TYPE(C_PTR), VALUE :: c, xx, xv, ff
       INTEGER(C_INT), VALUE :: species
       INTEGER(C_LONG), VALUE :: stride
     END FUNCTION
     INTEGER(C_INT) FUNCTION tcp_download(c, species, xx, xv, ff, stride) BIND(C, NAME='tcp_download')
       IMPORT :: C_INT, C_PTR, C_LONG
       TYPE(C_PTR), VALUE :: c, xx, xv, ff
       INTEGER(C_INT), VALUE :: species
       INTEGER(C_LONG), VALUE :: stride
     END FUNCTION
     INTEGER(C_INT) FUNCTION tcp_force_direct(c, ur) BIND(C, NAME='tcp_force_direct')
       IMPORT :: C_INT, C_PTR, C_DOUBLE
       TYPE(C_PTR), VALUE :: c
       REAL(C_DOUBLE), INTENT(OUT) :: ur
     END FUNCTION
     INTEGER(C_INT) FUNCTION tcp_force_spme(c, um) BIND(C, NAME='tcp_force_spme')
       IMPORT :: C_INT, C_PTR, C_DOUBLE
       TYPE(C_PTR), VALUE :: c
       REAL(C_DOUBLE), INTENT(OUT) :: um
     END FUNCTION
     INTEGER(C_INT) FUNCTION tcp_spme_sum(c) BIND(C, NAME='tcp_spme_sum')
       IMPORT :: C_INT, C_PTR
       TYPE(C_PTR), VALUE :: c
     END FUNCTION
     INTEGER(C_INT) FUNCTION tcp_remove_rigidmtn(c) BIND(C, NAME='tcp_remove_rigidmtn')
       IMPORT :: C_INT, C_PTR
       TYPE(C_PTR), VALUE :: c
     END FUNCTION
     INTEGER(C_INT) FUNCTION tcp_vverlet1(c, dt) BIND(C, NAME='tcp_vverlet1')
       IMPORT :: C_INT, C_PTR, C_DOUBLE
       TYPE(C_PTR), VALUE :: c
       REAL(C_DOUBLE), VALUE :: dt
     END FUNCTION
     INTEGER(C_INT) FUNCTION tcp_vverlet2(c, dt, mv2el, mv2ion) BIND(C, NAME='tcp_vverlet2')
       IMPORT :: C_INT, C_PTR, C_DOUBLE
       TYPE(C_PTR), VALUE :: c
       REAL(C_DOUBLE), VALUE :: dt
       REAL(C_DOUBLE), INTENT(OUT) :: mv2el, mv2ion
     END FUNCTION
     INTEGER(C_INT) FUNCTION tcp_set_flags(c, flags) BIND(C, NAME='tcp_set_flags')
       IMPORT :: C_INT, C_PTR
       TYPE(C_PTR), VALUE :: c
       INTEGER(C_INT), VALUE :: flags
     END FUNCTION
     INTEGER(C_INT) FUNCTION tcp_histograms(c, rdf, vdf, reset) BIND(C, NAME='tcp_histograms')
       IMPORT :: C_INT, C_PTR, C_DOUBLE
       TYPE(C_PTR), VALUE :: c
       REAL(C_DOUBLE), INTENT(OUT) :: rdf(*), vdf(*)
       INTEGER(C_INT), VALUE :: reset
     END FUNCTION
     INTEGER(C_INT) FUNCTION tcp_md_steps(c, dt, nsteps, e) BIND(C, NAME='tcp_md_steps')
       IMPORT :: C_INT, C_PTR, C_DOUBLE, tcp_energies
       TYPE(C_PTR), VALUE :: c
       REAL(C_DOUBLE), VALUE :: dt
       INTEGER(C_INT), VALUE :: nsteps
       TYPE(tcp_energies), INTENT(OUT) :: e
     END FUNCTION
     INTEGER(C_INT) FUNCTION tcp_md_steps_records(c, dt, nsteps, exx, exv, eff, estride, ixx, ixv, iff, istride, e) &
          BIND(C, NAME='tcp_md_steps_records')
       IMPORT :: C_INT, C_PTR, C_DOUBLE, C_LONG, tcp_energies
       TYPE(C_PTR), VALUE :: c, exx, exv, eff, ixx, ixv, iff
       REAL(C_DOUBLE), VALUE :: dt
       INTEGER(C_INT), VALUE :: nsteps
       INTEGER(C_LONG), VALUE :: estride, istride
       TYPE(tcp_energies), INTENT(OUT) :: e
     END FUNCTION
     ! derivatives (no counterpart in the reference)
     INTEGER(C_INT) FUNCTION tcp_adjoint_energy(c, e, dedl, deds) BIND(C, NAME='tcp_adjoint_energy')
       IMPORT :: C_INT, C_PTR, C_DOUBLE
       TYPE(C_PTR), VALUE :: c
       REAL(C_DOUBLE), INTENT(OUT) :: e, dedl, deds
     END FUNCTION
     INTEGER(C_INT) FUNCTION tcp_hvp(c, w, hw, dfdl_w) BIND(C, NAME='tcp_hvp')
       IMPORT :: C_INT, C_PTR, C_DOUBLE
       TYPE(C_PTR), VALUE :: c
       REAL(C_DOUBLE), INTENT(IN) :: w(3, *)
       REAL(C_DOUBLE), INTENT(OUT) :: hw(3, *)
       REAL(C_DOUBLE), INTENT(OUT) :: dfdl_w
     END FUNCTION
     INTEGER(C_INT) FUNCTION tcp_reverse_md(c, dt, nsteps, every, j, djdl) BIND(C, NAME='tcp_reverse_md')
       IMPORT :: C_INT, C_PTR, C_DOUBLE
       TYPE(C_PTR), VALUE :: c
       REAL(C_DOUBLE), VALUE :: dt
       INTEGER(C_INT), VALUE :: nsteps, every
       REAL(C_DOUBLE), INTENT(OUT) :: j, djdl
     END FUNCTION
     FUNCTION tcp_last_error() BIND(C, NAME='tcp_last_error')
       IMPORT :: C_PTR
       TYPE(C_PTR) :: tcp_last_error
     END FUNCTION
  END INTERFACE

CONTAINS

  SUBROUTINE tcp_stop_on(status, where)
    INTEGER(C_INT), INTENT(IN) :: status
    CHARACTER(*), INTENT(IN) :: where
    IF (status /= 0) THEN
       PRINT *, " *** libtcpgpu error in ", where, " status ", status
       STOP
    END IF
  END SUBROUTINE

  ! Sync the host PT records into the device state (rec = qel or qion)
  SUBROUTINE tcp_push(species, rec, n)
    INTEGER, INTENT(IN) :: species, n
    TYPE(PT), TARGET, INTENT(IN) :: rec(n)
    INTEGER(C_LONG) :: stride
    IF (n == 0) RETURN
    stride = 104
    IF (n > 1) stride = TRANSFER(C_LOC(rec(2)), 0_C_LONG) - TRANSFER(C_LOC(rec(1)), 0_C_LONG)
    CALL tcp_stop_on(tcp_upload(ctx, species, C_LOC(rec(1)%xx), C_LOC(rec(1)%xv), C_LOC(rec(1)%ff), stride), &
         "tcp_upload")
  END SUBROUTINE

  ! nsteps MD steps on qel / qion updated in place (the body of main.f90:81-153
  ! with the records read before and written after, one wait for the device)
  SUBROUTINE tcp_steps_records(dt, nsteps, qel, nel, qion, nion, e)
    REAL(C_DOUBLE), INTENT(IN) :: dt
    INTEGER, INTENT(IN) :: nsteps, nel, nion
    TYPE(PT), TARGET, INTENT(INOUT) :: qel(nel), qion(nion)
    TYPE(tcp_energies), INTENT(OUT) :: e
    INTEGER(C_LONG) :: estr, istr
    TYPE(C_PTR) :: exx, exv, eff, ixx, ixv, iff
    estr = 104
    istr = 104
    exx = C_NULL_PTR; exv = C_NULL_PTR; eff = C_NULL_PTR
    ixx = C_NULL_PTR; ixv = C_NULL_PTR; iff = C_NULL_PTR
    IF (nel > 0) THEN
      exx = C_LOC(qel(1)%xx); exv = C_LOC(qel(1)%xv); eff = C_LOC(qel(1)%ff)
      IF (nel > 1) estr = TRANSFER(C_LOC(qel(2)), 0_C_LONG) - TRANSFER(C_LOC(qel(1)), 0_C_LONG)
    END IF
    IF (nion > 0) THEN
      ixx = C_LOC(qion(1)%xx); ixv = C_LOC(qion(1)%xv); iff = C_LOC(qion(1)%ff)
      IF (nion > 1) istr = TRANSFER(C_LOC(qion(2)), 0_C_LONG) - TRANSFER(C_LOC(qion(1)), 0_C_LONG)
    END IF
    CALL tcp_stop_on(tcp_md_steps_records(ctx, dt, INT(nsteps, C_INT), exx, exv, eff, estr, ixx, ixv, iff, istr, e), &
         "tcp_md_steps_records")
  END SUBROUTINE

  ! NS%RDF_* / NS%VDF_* += the device histograms since the last pull, which are
  ! then zeroed; called before DUMP (main.f90:155-157), which reads and
  ! resets the NS arrays (result.f90:209-278)
  SUBROUTINE tcp_pull_histograms(NS)
    TYPE(NM) :: NS
    REAL(C_DOUBLE) :: rdf(3 * SIZE(NS%RDF_ee)), vdf(2 * SIZE(NS%VDF_e))
    INTEGER :: m
    m = SIZE(NS%RDF_ee)
    CALL tcp_stop_on(tcp_histograms(ctx, rdf, vdf, 1_C_INT), "tcp_histograms")
    NS%RDF_ee = NS%RDF_ee + rdf(1:m)
    NS%RDF_ei = NS%RDF_ei + rdf(m + 1:2 * m)
    NS%RDF_ii = NS%RDF_ii + rdf(2 * m + 1:3 * m)
    NS%VDF_e = NS%VDF_e + vdf(1:m)
    NS%VDF_i = NS%VDF_i + vdf(m + 1:2 * m)
  END SUBROUTINE

  SUBROUTINE tcp_pull(species, rec, n)
    INTEGER, INTENT(IN) :: species, n
    TYPE(PT), TARGET, INTENT(INOUT) :: rec(n)
    INTEGER(C_LONG) :: stride
    IF (n == 0) RETURN
    stride = 104
    IF (n > 1) stride = TRANSFER(C_LOC(rec(2)), 0_C_LONG) - TRANSFER(C_LOC(rec(1)), 0_C_LONG)
    CALL tcp_stop_on(tcp_download(ctx, species, C_LOC(rec(1)%xx), C_LOC(rec(1)%xv), C_LOC(rec(1)%ff), stride), &
         "tcp_download")
  END SUBROUTINE

END MODULE TCP_GPU

! ---- drop-in replacements with the reference's argument lists -------------

! EWALD_SELF(NS,param,sys,PSI,COMM), force.f90:4-49: also creates the context
SUBROUTINE EWALD_SELF(NS, param, sys, PSI, COMM)
  USE TCP_GPU
  IMPLICIT NONE
  TYPE(NM):: NS
  TYPE(PM):: param
  TYPE(ST):: sys
  TYPE(MP):: COMM
  REAL(KIND=DP) :: PSI(*)
  TYPE(tcp_params) :: p
  REAL(C_DOUBLE) :: a, uo
  p%xm = param%xm; p%q = param%q; p%tau = param%tau; p%alpha_lgv = param%alpha
  p%a = 0.0D0; p%box = param%box; p%Te = param%Te; p%Ti = param%Ti
  p%rs = param%rs; p%rc = param%rc; p%K = param%K; p%order = 4
  p%dx_ee = NS%dx_ee; p%dx_ei = NS%dx_ei; p%dx_ii = NS%dx_ii; p%dv_e = NS%dv_e; p%dv_i = NS%dv_i
  p%ei_model = 0; p%lambda_ei = param%rs; p%charge_scale = 1.0D0
  p%precision = 0; p%reciprocal = 1; p%ewald_nmax2 = 0; p%thermo_period = 1; p%seed = 0
  p%thermo = 0
  IF (param%thermo == 'ISOKIN') p%thermo = 1
  IF (param%thermo == 'BEREND') p%thermo = 2
  IF (param%thermo == 'STOCH ') p%thermo = 3
  IF (.NOT. C_ASSOCIATED(ctx)) THEN
    CALL tcp_stop_on(tcp_create(p, NS%NTel, NS%NTion, 0, ctx), "tcp_create")
    ! the reference accumulates RDF and VDF in every force call and kick
    CALL tcp_stop_on(tcp_set_flags(ctx, IOR(IOR(TCP_FLAG_RDF, TCP_FLAG_VDF), TCP_FLAG_ENERGY)), "tcp_set_flags")
  END IF
  CALL tcp_stop_on(tcp_ewald_self(ctx, a, uo), "EWALD_SELF")
  param%a = a
  param%rc2 = param%rc**2
  sys%Uo = uo
END SUBROUTINE EWALD_SELF

! Force_direct_self(NS,qel,qion,param,sys), force.f90:52-180 (whole system)
SUBROUTINE Force_direct_self(NS, qel, qion, param, sys)
  USE TCP_GPU
  IMPLICIT NONE
  TYPE(NM):: NS
  TYPE(PT):: qel(NS%Nel), qion(NS%Nion)
  TYPE(PM):: param
  TYPE(ST):: sys
  REAL(C_DOUBLE) :: ur
  CALL tcp_stop_on(tcp_force_direct(ctx, ur), "Force_direct_self")
  sys%Ur = ur
END SUBROUTINE Force_direct_self

! Force_SPME4(NS,param,sys,COMM,PSI,gsend,pme), force.f90:652-929
SUBROUTINE Force_SPME4(NS, param, sys, COMM, PSI, gsend, pme)
  USE TCP_GPU
  IMPLICIT NONE
  TYPE(NM):: NS
  TYPE(PM):: param
  TYPE(ST):: sys
  TYPE(MP):: COMM
  REAL(KIND=DP) :: PSI(*)
  TYPE(GH):: gsend(*), pme(*)
  REAL(C_DOUBLE) :: um
  CALL tcp_stop_on(tcp_force_spme(ctx, um), "Force_SPME4")
  sys%Um = um
END SUBROUTINE Force_SPME4

! SPME_SUM(NS,qel,qion,sys,COMM,pme,grec), force.f90:932-969
SUBROUTINE SPME_SUM(NS, qel, qion, sys, COMM, pme, grec)
  USE TCP_GPU
  IMPLICIT NONE
  TYPE(NM):: NS
  TYPE(PT):: qel(NS%Nel), qion(NS%Nion)
  TYPE(ST):: sys
  TYPE(MP):: COMM
  TYPE(GH):: pme(*), grec(*)
  CALL tcp_stop_on(tcp_spme_sum(ctx), "SPME_SUM")
END SUBROUTINE SPME_SUM

! REMOVE_RIGIDMTN(NS,qel,qion,COMM), force.f90:974-1007
SUBROUTINE REMOVE_RIGIDMTN(NS, qel, qion, COMM)
  USE TCP_GPU
  IMPLICIT NONE
  TYPE(NM):: NS
  TYPE(PT):: qel(NS%Nel), qion(NS%Nion)
  TYPE(MP):: COMM
  CALL tcp_stop_on(tcp_remove_rigidmtn(ctx), "REMOVE_RIGIDMTN")
END SUBROUTINE REMOVE_RIGIDMTN

! VVerletNotemp1(NS,qel,qion,param,dt,gsend), vverlet.f90:132-171
SUBROUTINE VVerletNotemp1(NS, qel, qion, param, dt, gsend)
  USE TCP_GPU
  IMPLICIT NONE
  TYPE(NM):: NS
  TYPE(PT):: qel(NS%Nel), qion(NS%Nion)
  TYPE(PM):: param
  REAL(KIND=DP) :: dt
  TYPE(GH):: gsend(*)
  CALL tcp_stop_on(tcp_vverlet1(ctx, dt), "VVerletNotemp1")
END SUBROUTINE VVerletNotemp1

! VVerletNotemp2(NS,qel,qion,param,sys,dt), vverlet.f90:174-223 (and the
! ISOKIN/BEREND variants: the thermostat is selected at EWALD_SELF)
SUBROUTINE VVerletNotemp2(NS, qel, qion, param, sys, dt)
  USE TCP_GPU
  IMPLICIT NONE
  TYPE(NM):: NS
  TYPE(PT):: qel(NS%Nel), qion(NS%Nion)
  TYPE(PM):: param
  TYPE(ST):: sys
  REAL(KIND=DP) :: dt
  REAL(C_DOUBLE) :: a, b
  CALL tcp_stop_on(tcp_vverlet2(ctx, dt, a, b), "VVerletNotemp2")
  sys%mv2el = a
  sys%mv2ion = b
END SUBROUTINE VVerletNotemp2
