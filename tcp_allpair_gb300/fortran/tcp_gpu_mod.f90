! tcp_gpu_mod.f90 -- ISO_C_BINDING interfaces to libtcpgpu.so (include/tcp_gpu.h)
! and drop-in wrappers with the argument lists of the reference's step routines.
!
! A maintainer replaces force.f90 / vverlet.f90 in the reference's Makefile by
! this file, keeps data.f90 / main.f90 / init.f90 / result.f90 unchanged, and
! links -L<pkg>/_build -ltcpgpu.  Every routine main.f90 and init.f90 call in
! force.f90 / vverlet.f90 is defined here with the reference's name and dummy
! arguments (tests/test_fortran_shim.py checks this against the reference's
! sources); COMM, grec/gemit/pme and PSI are accepted and ignored (one GPU, no
! MPI ranks on the compute path).  The GPU build's own parameters (precision,
! e-i model, spline order, alpha, Kelbg length, device) come from
! ./tcp_gpu.prm or TCP_GPU_* environment variables (tcp_params_from_env).
! Not compiled in this repository's tests: no Fortran compiler exists on
! either build machine.
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

  ! Who holds the current state.  host_owns: the host records were written
  ! last (after EWALD_SELF: Init / restart read, Vinit, Finit's x - dt v), so
  ! the next routine that can see them uploads them.  dev_forces: the device
  ! computed forces since then (Finit's force calls), so the records' ff are
  ! stale and are not uploaded.  After the first half kick the device owns the
  ! state; the second half kick refreshes the records every sync_every steps
  ! (1 by default: the reference's host arrays are current after every step,
  ! and DUMP / SAMPLING / Restart read them, main.f90:155-168).
  LOGICAL, SAVE :: host_owns = .TRUE., dev_forces = .FALSE.
  INTEGER(C_INT), SAVE :: sync_every = 1
  INTEGER, SAVE :: nkick2 = 0

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
     INTEGER(C_INT) FUNCTION tcp_params_from_env(p, device, sync_every) BIND(C, NAME='tcp_params_from_env')
       IMPORT :: C_INT, tcp_params
       TYPE(tcp_params), INTENT(INOUT) :: p
       INTEGER(C_INT), INTENT(INOUT) :: device, sync_every
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

  ! byte distance between consecutive records (never an assumed constant)
  INTEGER(C_LONG) FUNCTION pt_stride(rec, n)
    INTEGER, INTENT(IN) :: n
    TYPE(PT), TARGET, INTENT(IN) :: rec(n)
    pt_stride = 104
    IF (n > 1) pt_stride = TRANSFER(C_LOC(rec(2)), 0_C_LONG) - TRANSFER(C_LOC(rec(1)), 0_C_LONG)
  END FUNCTION

  INTEGER(C_LONG) FUNCTION gh_stride(g, n)
    INTEGER, INTENT(IN) :: n
    TYPE(GH), TARGET, INTENT(IN) :: g(n)
    gh_stride = 24
    IF (n > 1) gh_stride = TRANSFER(C_LOC(g(2)), 0_C_LONG) - TRANSFER(C_LOC(g(1)), 0_C_LONG)
  END FUNCTION

  ! Upload one species' records: positions and velocities, and the forces
  ! unless the device computed them since the host last wrote the records.
  SUBROUTINE tcp_push(species, rec, n)
    INTEGER, INTENT(IN) :: species, n
    TYPE(PT), TARGET, INTENT(IN) :: rec(n)
    TYPE(C_PTR) :: ff
    IF (n == 0) RETURN
    ff = C_NULL_PTR
    IF (.NOT. dev_forces) ff = C_LOC(rec(1)%ff)
    CALL tcp_stop_on(tcp_upload(ctx, INT(species, C_INT), C_LOC(rec(1)%xx), C_LOC(rec(1)%xv), ff, &
         pt_stride(rec, n)), "tcp_upload")
  END SUBROUTINE

  ! Positions from the gsend array of Force_SPME4 (electrons, then ions),
  ! which Finit fills with x - dt v (init.f90:171-185).
  SUBROUTINE tcp_push_gh(g, nel, nion)
    INTEGER, INTENT(IN) :: nel, nion
    TYPE(GH), TARGET, INTENT(IN) :: g(nel + nion)
    IF (nel > 0) CALL tcp_stop_on(tcp_upload(ctx, 0_C_INT, C_LOC(g(1)%xx), C_NULL_PTR, C_NULL_PTR, &
         gh_stride(g, nel + nion)), "tcp_upload")
    IF (nion > 0) CALL tcp_stop_on(tcp_upload(ctx, 1_C_INT, C_LOC(g(nel + 1)%xx), C_NULL_PTR, C_NULL_PTR, &
         gh_stride(g, nel + nion)), "tcp_upload")
  END SUBROUTINE

  SUBROUTINE tcp_pull(species, rec, n)
    INTEGER, INTENT(IN) :: species, n
    TYPE(PT), TARGET, INTENT(INOUT) :: rec(n)
    IF (n == 0) RETURN
    CALL tcp_stop_on(tcp_download(ctx, INT(species, C_INT), C_LOC(rec(1)%xx), C_LOC(rec(1)%xv), &
         C_LOC(rec(1)%ff), pt_stride(rec, n)), "tcp_download")
  END SUBROUTINE

  ! The caller changed qel / qion on the host after the run started (for
  ! example a restart read in the middle of a run): the next routine that can
  ! see the records uploads them.
  SUBROUTINE tcp_gpu_host_changed()
    host_owns = .TRUE.
    dev_forces = .FALSE.
  END SUBROUTINE

  ! Records current before the first half kick of the run
  SUBROUTINE tcp_sync_in(NS, qel, qion)
    TYPE(NM) :: NS
    TYPE(PT) :: qel(NS%Nel), qion(NS%Nion)
    IF (.NOT. host_owns) RETURN
    CALL tcp_push(0, qel, NS%Nel)
    CALL tcp_push(1, qion, NS%Nion)
    host_owns = .FALSE.
  END SUBROUTINE

  ! End of a step (second half kick): records and histograms back to the host
  SUBROUTINE tcp_sync_out(NS, qel, qion)
    TYPE(NM) :: NS
    TYPE(PT) :: qel(NS%Nel), qion(NS%Nion)
    nkick2 = nkick2 + 1
    IF (sync_every <= 0) RETURN
    IF (MOD(nkick2, sync_every) /= 0) RETURN
    CALL tcp_pull(0, qel, NS%Nel)
    CALL tcp_pull(1, qion, NS%Nion)
    CALL tcp_pull_histograms(NS)
  END SUBROUTINE

  ! nsteps MD steps on qel / qion updated in place (the body of main.f90:81-153
  ! with the records read before and written after, one wait for the device):
  ! the fast route for a caller that may replace its loop by one call
  SUBROUTINE tcp_steps_records(dt, nsteps, qel, nel, qion, nion, e)
    REAL(C_DOUBLE), INTENT(IN) :: dt
    INTEGER, INTENT(IN) :: nsteps, nel, nion
    TYPE(PT), TARGET, INTENT(INOUT) :: qel(nel), qion(nion)
    TYPE(tcp_energies), INTENT(OUT) :: e
    INTEGER(C_LONG) :: estr, istr
    TYPE(C_PTR) :: exx, exv, eff, ixx, ixv, iff
    estr = pt_stride(qel, nel)
    istr = pt_stride(qion, nion)
    exx = C_NULL_PTR; exv = C_NULL_PTR; eff = C_NULL_PTR
    ixx = C_NULL_PTR; ixv = C_NULL_PTR; iff = C_NULL_PTR
    IF (nel > 0) THEN
      exx = C_LOC(qel(1)%xx); exv = C_LOC(qel(1)%xv); eff = C_LOC(qel(1)%ff)
    END IF
    IF (nion > 0) THEN
      ixx = C_LOC(qion(1)%xx); ixv = C_LOC(qion(1)%xv); iff = C_LOC(qion(1)%ff)
    END IF
    CALL tcp_stop_on(tcp_md_steps_records(ctx, dt, INT(nsteps, C_INT), exx, exv, eff, estr, ixx, ixv, iff, istr, e), &
         "tcp_md_steps_records")
    host_owns = .FALSE.
  END SUBROUTINE

  ! NS%RDF_* / NS%VDF_* += the device histograms since the last pull, which are
  ! then zeroed; DUMP (result.f90:209-278) reads and resets the NS arrays
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

END MODULE TCP_GPU

! ---- drop-in replacements with the reference's argument lists -------------

! EWALD_SELF(NS,param,sys,PSI,COMM), force.f90:4-49: also creates the context
! from param, NS and the GPU build's own knobs (tcp_params_from_env)
SUBROUTINE EWALD_SELF(NS, param, sys, PSI, COMM)
  USE TCP_GPU
  IMPLICIT NONE
  TYPE(NM):: NS
  TYPE(PM):: param
  TYPE(ST):: sys
  REAL(KIND=DP) :: PSI(*)
  TYPE(MP):: COMM
  TYPE(tcp_params) :: p
  REAL(C_DOUBLE) :: a, uo
  INTEGER(C_INT) :: device
  p%xm = param%xm(1:2); p%q = param%q(1:2); p%tau = param%tau; p%alpha_lgv = param%alpha
  p%a = 0.0D0; p%box = param%box; p%Te = param%Te; p%Ti = param%Ti
  p%rs = param%rs; p%rc = param%rc; p%K = param%K; p%order = 4
  p%dx_ee = NS%dx_ee; p%dx_ei = NS%dx_ei; p%dx_ii = NS%dx_ii; p%dv_e = NS%dv_e; p%dv_i = NS%dv_i
  p%ei_model = 0; p%lambda_ei = param%rs; p%charge_scale = 1.0D0
  p%precision = 0; p%reciprocal = 1; p%ewald_nmax2 = 0; p%thermo_period = 1; p%seed = 0
  p%thermo = 0
  IF (param%thermo == 'ISOKIN') p%thermo = 1
  IF (param%thermo == 'BEREND') p%thermo = 2
  IF (param%thermo == 'STOCH ') p%thermo = 3
  device = 0
  CALL tcp_stop_on(tcp_params_from_env(p, device, sync_every), "tcp_params_from_env")
  IF (.NOT. C_ASSOCIATED(ctx)) THEN
    CALL tcp_stop_on(tcp_create(p, NS%NTel, NS%NTion, device, ctx), "tcp_create")
    ! the reference accumulates RDF and VDF in every force call and kick
    CALL tcp_stop_on(tcp_set_flags(ctx, IOR(IOR(TCP_FLAG_RDF, TCP_FLAG_VDF), TCP_FLAG_ENERGY)), "tcp_set_flags")
  END IF
  CALL tcp_stop_on(tcp_ewald_self(ctx, a, uo), "EWALD_SELF")
  param%a = a
  param%rc2 = param%rc**2
  sys%Uo = uo
  host_owns = .TRUE.
  dev_forces = .FALSE.
END SUBROUTINE EWALD_SELF

! Force_direct_self(NS,qel,qion,param,sys), force.f90:52-180, for the whole
! system (the rectangles of Force_direct_ext are part of it on one GPU).
! Finit passes one more argument (PRE_data, init.f90:195), ignored here as by
! the reference.
SUBROUTINE Force_direct_self(NS, qel, qion, param, sys)
  USE TCP_GPU
  IMPLICIT NONE
  TYPE(NM):: NS
  TYPE(PT):: qel(NS%Nel), qion(NS%Nion)
  TYPE(PM):: param
  TYPE(ST):: sys
  REAL(C_DOUBLE) :: ur
  IF (host_owns) THEN            ! Finit: the records hold x - dt v (init.f90:171-185)
    CALL tcp_push(0, qel, NS%Nel)
    CALL tcp_push(1, qion, NS%Nion)
  END IF
  CALL tcp_stop_on(tcp_force_direct(ctx, ur), "Force_direct_self")
  sys%Ur = ur
  IF (host_owns) dev_forces = .TRUE.
END SUBROUTINE Force_direct_self

! Force_direct_ext(NS,qel,qion,param,grec,gemit,Ur,Ne,Ni), force.f90:183-343:
! the pairs with another rank's particles.  One GPU holds every particle and
! Force_direct_self sums every pair, so there is no other rank: Ur = 0 and
! gemit is left as it is.  (With one process main.f90 does not call it.)
SUBROUTINE Force_direct_ext(NS, qel, qion, param, grec, gemit, Ur, Ne, Ni)
  USE TCP_GPU
  IMPLICIT NONE
  TYPE(NM):: NS
  TYPE(PT):: qel(NS%Nel), qion(NS%Nion)
  TYPE(PM):: param
  TYPE(GH):: grec(*), gemit(*)
  REAL(KIND=DP) :: Ur
  INTEGER :: Ne, Ni
  Ur = 0.0D0
END SUBROUTINE Force_direct_ext

! Force_direct_sum(NS,qel,qion,grec), force.f90:346-372: adds the reactions a
! remote rank computed; on one GPU they are added inside the pair kernel.
SUBROUTINE Force_direct_sum(NS, qel, qion, grec)
  USE TCP_GPU
  IMPLICIT NONE
  TYPE(NM):: NS
  TYPE(PT):: qel(NS%Nel), qion(NS%Nion)
  TYPE(GH):: grec(*)
END SUBROUTINE Force_direct_sum

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
  IF (host_owns) CALL tcp_push_gh(gsend, NS%Nel, NS%Nion)   ! Finit's x - dt v
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

! VVerletNotemp1(NS,qel,qion,param,dt,gsend), vverlet.f90:132-171.  The first
! call of a run uploads the host records (positions and velocities; forces
! too unless Finit computed them on the device).
SUBROUTINE VVerletNotemp1(NS, qel, qion, param, dt, gsend)
  USE TCP_GPU
  IMPLICIT NONE
  TYPE(NM):: NS
  TYPE(PT):: qel(NS%Nel), qion(NS%Nion)
  TYPE(PM):: param
  REAL(KIND=DP) :: dt
  TYPE(GH):: gsend(*)
  CALL tcp_sync_in(NS, qel, qion)
  CALL tcp_stop_on(tcp_vverlet1(ctx, dt), "VVerletNotemp1")
END SUBROUTINE VVerletNotemp1

! VVerletStoch1(NS,qel,qion,param,dt,gsend), vverlet.f90:9-59: the Langevin
! first half kick (the context was created with thermo = STOCH, so
! tcp_vverlet1 applies the damping and the noise)
SUBROUTINE VVerletStoch1(NS, qel, qion, param, dt, gsend)
  USE TCP_GPU
  IMPLICIT NONE
  TYPE(NM):: NS
  TYPE(PT):: qel(NS%Nel), qion(NS%Nion)
  TYPE(PM):: param
  REAL(KIND=DP) :: dt
  TYPE(GH):: gsend(*)
  CALL tcp_sync_in(NS, qel, qion)
  CALL tcp_stop_on(tcp_vverlet1(ctx, dt), "VVerletStoch1")
END SUBROUTINE VVerletStoch1

! VVerletNotemp2(NS,qel,qion,param,sys,dt), vverlet.f90:174-223
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
  CALL tcp_sync_out(NS, qel, qion)
END SUBROUTINE VVerletNotemp2

! VVerletStoch2(NS,qel,qion,param,sys,dt), vverlet.f90:62-127
SUBROUTINE VVerletStoch2(NS, qel, qion, param, sys, dt)
  USE TCP_GPU
  IMPLICIT NONE
  TYPE(NM):: NS
  TYPE(PT):: qel(NS%Nel), qion(NS%Nion)
  TYPE(PM):: param
  TYPE(ST):: sys
  REAL(KIND=DP) :: dt
  REAL(C_DOUBLE) :: a, b
  CALL tcp_stop_on(tcp_vverlet2(ctx, dt, a, b), "VVerletStoch2")
  sys%mv2el = a
  sys%mv2ion = b
  CALL tcp_sync_out(NS, qel, qion)
END SUBROUTINE VVerletStoch2

! VVerletBerend2(NS,qel,qion,param,sys,dt,COMM), vverlet.f90:227-298
SUBROUTINE VVerletBerend2(NS, qel, qion, param, sys, dt, COMM)
  USE TCP_GPU
  IMPLICIT NONE
  TYPE(NM):: NS
  TYPE(PT):: qel(NS%Nel), qion(NS%Nion)
  TYPE(PM):: param
  TYPE(ST):: sys
  REAL(KIND=DP) :: dt
  TYPE(MP):: COMM
  REAL(C_DOUBLE) :: a, b
  CALL tcp_stop_on(tcp_vverlet2(ctx, dt, a, b), "VVerletBerend2")
  sys%mv2el = a
  sys%mv2ion = b
  CALL tcp_sync_out(NS, qel, qion)
END SUBROUTINE VVerletBerend2

! VVerletIsokin2(NS,qel,qion,param,sys,dt,COMM), vverlet.f90:301-372
SUBROUTINE VVerletIsokin2(NS, qel, qion, param, sys, dt, COMM)
  USE TCP_GPU
  IMPLICIT NONE
  TYPE(NM):: NS
  TYPE(PT):: qel(NS%Nel), qion(NS%Nion)
  TYPE(PM):: param
  TYPE(ST):: sys
  REAL(KIND=DP) :: dt
  TYPE(MP):: COMM
  REAL(C_DOUBLE) :: a, b
  CALL tcp_stop_on(tcp_vverlet2(ctx, dt, a, b), "VVerletIsokin2")
  sys%mv2el = a
  sys%mv2ion = b
  CALL tcp_sync_out(NS, qel, qion)
END SUBROUTINE VVerletIsokin2
