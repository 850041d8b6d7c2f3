!==============================================================!
! Fortran 2008 interface to libchgpu.so (include/chgpu.h and !
! include/chgpu_closure.h).                                   !
! Lets a Fortran driver shaped like channel.f90 call the GB300 !
! time step through iso_c_binding.  Compile with the driver    !
! and link -lchgpu (channel_gb300/_build/libchgpu.so).        !
!==============================================================!
MODULE chgpu_interface
  USE, INTRINSIC :: iso_c_binding
  IMPLICIT NONE

  INTEGER(C_INT), PARAMETER :: CHGPU_FP64 = 0, CHGPU_MIXED = 1, CHGPU_FP64DD = 2
  INTEGER(C_INT), PARAMETER :: CHGPU_EXPORT_ALL = 0, CHGPU_EXPORT_LARGE = 1, CHGPU_EXPORT_SMALL = 2

  ! Mirrors chgpu_params field by field (C layout).
  TYPE, BIND(C) :: chgpu_params
    INTEGER(C_INT)       :: nx, ny, nz
    REAL(C_DOUBLE)       :: alfa0, beta0
    REAL(C_DOUBLE)       :: ni
    REAL(C_DOUBLE)       :: a, ymin, ymax
    INTEGER(C_INT)       :: cpi, cpi_type
    REAL(C_DOUBLE)       :: gamma
    REAL(C_DOUBLE)       :: meanpx, meanpz
    REAL(C_DOUBLE)       :: meanflowx, meanflowz
    REAL(C_DOUBLE)       :: u0, uN
    REAL(C_DOUBLE)       :: deltat, cflmax, time
    REAL(C_DOUBLE)       :: dt_field, dt_save, t_max
    INTEGER(C_INT)       :: time_from_restart
    INTEGER(C_LONG_LONG) :: nstep
    INTEGER(C_INT)       :: npy
    INTEGER(C_INT)       :: precision
  END TYPE chgpu_params

  ! Mirrors chgpu_stats: line(1:11) is one Runtimedata record.
  TYPE, BIND(C) :: chgpu_stats
    REAL(C_DOUBLE)       :: line(11)
    REAL(C_DOUBLE)       :: fr(3)
    REAL(C_DOUBLE)       :: corrpx, corrpz, meanpx, meanpz
    REAL(C_DOUBLE)       :: cfl, deltat, time
    INTEGER(C_LONG_LONG) :: istep
  END TYPE chgpu_stats

  ! Mirrors chgpu_export_opts (out2bin's -f, -l/-s, z_threshold, -u).
  TYPE, BIND(C) :: chgpu_export_opts
    INTEGER(C_INT)       :: fluct_only, part, z_threshold
    REAL(C_FLOAT)        :: undersample
  END TYPE chgpu_export_opts

  ! Mirrors chgpu_mlp_norm (include/chgpu_closure.h).
  INTEGER(C_INT), PARAMETER :: CHGPU_MLP_NPARAMS = 9734
  TYPE, BIND(C) :: chgpu_mlp_norm
    REAL(C_FLOAT)        :: mu_in(10), sd_in(10), mu_out(6), sd_out(6)
  END TYPE chgpu_mlp_norm

  INTERFACE
    INTEGER(C_INT) FUNCTION chgpu_create(p, h) BIND(C, name="chgpu_create")
      IMPORT :: C_INT, C_PTR, chgpu_params
      TYPE(chgpu_params), INTENT(IN) :: p
      TYPE(C_PTR), INTENT(OUT) :: h
    END FUNCTION
    INTEGER(C_INT) FUNCTION chgpu_destroy(h) BIND(C, name="chgpu_destroy")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: h
    END FUNCTION
    ! V is the reference's V(-1:ny+1,-nz:nz,0:nx,1:3), complex(C_DOUBLE_COMPLEX)
    INTEGER(C_INT) FUNCTION chgpu_upload_field(h, V) BIND(C, name="chgpu_upload_field")
      IMPORT :: C_INT, C_PTR, C_DOUBLE_COMPLEX
      TYPE(C_PTR), VALUE :: h
      COMPLEX(C_DOUBLE_COMPLEX), INTENT(IN) :: V(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION chgpu_download_field(h, V) BIND(C, name="chgpu_download_field")
      IMPORT :: C_INT, C_PTR, C_DOUBLE_COMPLEX
      TYPE(C_PTR), VALUE :: h
      COMPLEX(C_DOUBLE_COMPLEX), INTENT(OUT) :: V(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION chgpu_start(h, time, deltat, st) BIND(C, name="chgpu_start")
      IMPORT :: C_INT, C_PTR, C_DOUBLE, chgpu_stats
      TYPE(C_PTR), VALUE :: h
      REAL(C_DOUBLE), VALUE :: time, deltat
      TYPE(chgpu_stats), INTENT(OUT) :: st
    END FUNCTION
    INTEGER(C_INT) FUNCTION chgpu_set_wall_velocity(h, u0, uN) BIND(C, name="chgpu_set_wall_velocity")
      IMPORT :: C_INT, C_PTR, C_DOUBLE
      TYPE(C_PTR), VALUE :: h
      REAL(C_DOUBLE), VALUE :: u0, uN
    END FUNCTION
    INTEGER(C_INT) FUNCTION chgpu_buildrhs(h, ode, compute_cfl) BIND(C, name="chgpu_buildrhs")
      IMPORT :: C_INT, C_PTR, C_DOUBLE
      TYPE(C_PTR), VALUE :: h
      REAL(C_DOUBLE), INTENT(IN) :: ode(3)
      INTEGER(C_INT), VALUE :: compute_cfl
    END FUNCTION
    INTEGER(C_INT) FUNCTION chgpu_linsolve(h, lambda) BIND(C, name="chgpu_linsolve")
      IMPORT :: C_INT, C_PTR, C_DOUBLE
      TYPE(C_PTR), VALUE :: h
      REAL(C_DOUBLE), VALUE :: lambda
    END FUNCTION
    INTEGER(C_INT) FUNCTION chgpu_outstats(h, st) BIND(C, name="chgpu_outstats")
      IMPORT :: C_INT, C_PTR, chgpu_stats
      TYPE(C_PTR), VALUE :: h
      TYPE(chgpu_stats), INTENT(OUT) :: st
    END FUNCTION
    INTEGER(C_INT) FUNCTION chgpu_step(h, st) BIND(C, name="chgpu_step")
      IMPORT :: C_INT, C_PTR, chgpu_stats
      TYPE(C_PTR), VALUE :: h
      TYPE(chgpu_stats), INTENT(OUT) :: st
    END FUNCTION
    ! bodyforce hook: F(-1:ny+1,-nz:nz,0:nx,1:3) like V; pass C_NULL_PTR via
    ! chgpu_clear_body_force below to switch it off
    INTEGER(C_INT) FUNCTION chgpu_set_body_force(h, F) BIND(C, name="chgpu_set_body_force")
      IMPORT :: C_INT, C_PTR, C_DOUBLE_COMPLEX
      TYPE(C_PTR), VALUE :: h
      COMPLEX(C_DOUBLE_COMPLEX), INTENT(IN) :: F(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION chgpu_clear_body_force(h, nullF) BIND(C, name="chgpu_set_body_force")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: h, nullF
    END FUNCTION
    ! asynchronous snapshot: start the copy, later get a pointer to the host copy
    INTEGER(C_INT) FUNCTION chgpu_snapshot_async(h) BIND(C, name="chgpu_snapshot_async")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: h
    END FUNCTION
    INTEGER(C_INT) FUNCTION chgpu_snapshot_wait(h, V) BIND(C, name="chgpu_snapshot_wait")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: h
      TYPE(C_PTR), INTENT(OUT) :: V
    END FUNCTION
    ! mean and variance profiles (var_history.f90) accumulated on the device
    INTEGER(C_INT) FUNCTION chgpu_stats_reset(h) BIND(C, name="chgpu_stats_reset")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: h
    END FUNCTION
    INTEGER(C_INT) FUNCTION chgpu_stats_accumulate(h) BIND(C, name="chgpu_stats_accumulate")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: h
    END FUNCTION
    INTEGER(C_INT) FUNCTION chgpu_profiles(h, mean, var, nsamples) BIND(C, name="chgpu_profiles")
      IMPORT :: C_INT, C_PTR, C_DOUBLE, C_LONG_LONG
      TYPE(C_PTR), VALUE :: h
      REAL(C_DOUBLE), INTENT(OUT) :: mean(*), var(*)
      INTEGER(C_LONG_LONG), INTENT(OUT) :: nsamples
    END FUNCTION
    ! out2bin: vec(3,nxtot,0:ny,nztot) of the current field
    INTEGER(C_INT) FUNCTION chgpu_export_dims(h, undersample, dims) BIND(C, name="chgpu_export_dims")
      IMPORT :: C_INT, C_PTR, C_FLOAT
      TYPE(C_PTR), VALUE :: h
      REAL(C_FLOAT), VALUE :: undersample
      INTEGER(C_INT), INTENT(OUT) :: dims(3)
    END FUNCTION
    INTEGER(C_INT) FUNCTION chgpu_export_physical(h, opts, vec) BIND(C, name="chgpu_export_physical")
      IMPORT :: C_INT, C_PTR, C_DOUBLE, chgpu_export_opts
      TYPE(C_PTR), VALUE :: h
      TYPE(chgpu_export_opts), INTENT(IN) :: opts
      REAL(C_DOUBLE), INTENT(OUT) :: vec(*)
    END FUNCTION
    ! transform tiles timed on this handle (optional; results do not depend on them)
    INTEGER(C_INT) FUNCTION chgpu_autotune(h) BIND(C, name="chgpu_autotune")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: h
    END FUNCTION
    INTEGER(C_INT) FUNCTION chgpu_set_step_halves(h, halves) BIND(C, name="chgpu_set_step_halves")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: h
      INTEGER(C_INT), VALUE :: halves
    END FUNCTION
    TYPE(C_PTR) FUNCTION chgpu_last_error(h) BIND(C, name="chgpu_last_error")
      IMPORT :: C_PTR
      TYPE(C_PTR), VALUE :: h
    END FUNCTION
    ! ---- learned closure (include/chgpu_closure.h) ----
    INTEGER(C_INT) FUNCTION chgpu_mlp_create(seed, m) BIND(C, name="chgpu_mlp_create")
      IMPORT :: C_INT, C_LONG_LONG, C_PTR
      INTEGER(C_LONG_LONG), VALUE :: seed
      TYPE(C_PTR), INTENT(OUT) :: m
    END FUNCTION
    INTEGER(C_INT) FUNCTION chgpu_mlp_destroy(m) BIND(C, name="chgpu_mlp_destroy")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: m
    END FUNCTION
    ! theta(CHGPU_MLP_NPARAMS): W1(16,64) W2(64,64) b2(64) W3(64,64) b3(64) W4(64,6) b4(6), column-major view of W[o][i]
    INTEGER(C_INT) FUNCTION chgpu_mlp_set_params(m, theta) BIND(C, name="chgpu_mlp_set_params")
      IMPORT :: C_INT, C_PTR, C_FLOAT
      TYPE(C_PTR), VALUE :: m
      REAL(C_FLOAT), INTENT(IN) :: theta(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION chgpu_mlp_set_norm(m, nm) BIND(C, name="chgpu_mlp_set_norm")
      IMPORT :: C_INT, C_PTR, chgpu_mlp_norm
      TYPE(C_PTR), VALUE :: m
      TYPE(chgpu_mlp_norm), INTENT(IN) :: nm
    END FUNCTION
    ! enable = 1: the network's stresses enter every convolution pass; 0: the plain solver
    INTEGER(C_INT) FUNCTION chgpu_closure_attach(h, m, enable) BIND(C, name="chgpu_closure_attach")
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: h, m
      INTEGER(C_INT), VALUE :: enable
    END FUNCTION
  END INTERFACE

CONTAINS

  ! dns.in values as read_dnsin leaves them -> chgpu_params
  FUNCTION chgpu_params_from(nx, ny, nz, alfa0, beta0, ni, a, ymin, ymax, cpi, cpi_type, gamma, meanpx, meanpz, &
                             meanflowx, meanflowz, u0, uN, deltat, cflmax, time, dt_field, dt_save, t_max, &
                             time_from_restart, nstep, npy, precision) RESULT(p)
    INTEGER(C_INT), INTENT(IN) :: nx, ny, nz, cpi_type, npy, precision
    REAL(C_DOUBLE), INTENT(IN) :: alfa0, beta0, ni, a, ymin, ymax, gamma, meanpx, meanpz, meanflowx, meanflowz
    REAL(C_DOUBLE), INTENT(IN) :: u0, uN, deltat, cflmax, time, dt_field, dt_save, t_max
    LOGICAL, INTENT(IN) :: cpi, time_from_restart
    INTEGER(C_SIZE_T), INTENT(IN) :: nstep
    TYPE(chgpu_params) :: p
    p%nx = nx; p%ny = ny; p%nz = nz; p%alfa0 = alfa0; p%beta0 = beta0; p%ni = ni
    p%a = a; p%ymin = ymin; p%ymax = ymax
    p%cpi = MERGE(1, 0, cpi); p%cpi_type = cpi_type; p%gamma = gamma
    p%meanpx = meanpx; p%meanpz = meanpz; p%meanflowx = meanflowx; p%meanflowz = meanflowz
    p%u0 = u0; p%uN = uN; p%deltat = deltat; p%cflmax = cflmax; p%time = time
    p%dt_field = dt_field; p%dt_save = dt_save; p%t_max = t_max
    p%time_from_restart = MERGE(1, 0, time_from_restart)
    p%nstep = INT(nstep, C_LONG_LONG); p%npy = npy; p%precision = precision
  END FUNCTION chgpu_params_from

END MODULE chgpu_interface
