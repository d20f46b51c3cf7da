! oakg.F90 -- Fortran interface to the GB300 local ensemble square-root analysis (liboakg.so).
!
! A thin ISO_C_BINDING layer over include/oakg.h, for Fortran host code of OAK
! (gher-uliege/OAK 1.7): one bind(C) interface per entry point of the header, the structures
! it passes by pointer, and wrappers that keep the argument lists of the Fortran routines the
! library replaces:
!
!   gpu_analysis     <- analysis(xf,Hxf,yo,Sf,HSf,R,xa,Sa,amplitudes)      rrsqrt.F90:196-208
!   gpu_locAnalysis  <- locAnalysis(zoneSize,selectObservations,xf,Hxf,yo,Sf,HSf,R,xa,Sa,
!                                   amplitudes,localise_obs)                rrsqrt.F90:433-466
!   gpu_locAnalysis_r4  <- the same for the reference's single-precision build (real(4))
!   gpu_locAnalysis_adjoint  gradients of a cost of the analysis mean (no reference
!                            counterpart: the reference has no derivative code)
!
! Differences from the reference routines:
!   - R is class(Covar) in the reference; here it is the diagonal of DiagCovar (the
!     observation error variances), covariance.F90:70-79.
!   - selectObservations is a procedure argument in the reference, which cannot cross a C
!     interface; gpu_locAnalysis takes the data it evaluates instead (type oakg_geometry):
!     the coordinates of each zone's first element, the observation coordinates and the
!     correlation / maximum lengths, with the weight kind, metric and loctype of
!     selectObservations (assimilation.F90:3683-3771).
!   - real is real(c_double) (the reference's PRECISION=double build, -fdefault-real-8), or
!     real(c_float) in gpu_locAnalysis_r4 (PRECISION=single).
!   - A non-zero status stops the program with the library's message, as the reference stops
!     on errors (ERROR_STOP, ppdef.h:22); the bind(C) interfaces return the status instead.
!   - Call the wrappers from one thread (inside !$omp master, then !$omp barrier, where the
!     caller runs in an OpenMP team as the reference's locAnalysis does).
!
! The reference's own C interface (oak_init, oak_assim, oak_done, assimilation.F90:4885-4935)
! is exported under the same names by the library; its interfaces are declared here too.
!
! Build:  gfortran -c oakg.F90  (any Fortran 2018 compiler: optional arguments of bind(C)
!         interfaces pass NULL when absent), link with -L<lib dir> -loakg.

module oakg
  use iso_c_binding
  implicit none
  private :: check, c2f

  ! status codes
  integer(c_int), parameter :: OAKG_OK = 0, OAKG_ERR_ARGS = 1, OAKG_ERR_CUDA = 2, &
       OAKG_ERR_NAN = 3, OAKG_ERR_EIG = 4, OAKG_ERR_NOMEM = 5, OAKG_ERR_TIMEOUT = 6, &
       OAKG_ERR_INIT = 7, OAKG_ERR_NOTIMPL = 8
  ! where array pointers live
  integer(c_int32_t), parameter :: OAKG_MEM_HOST = 0, OAKG_MEM_DEVICE = 1
  ! observation weight kinds
  integer(c_int32_t), parameter :: OAKG_WEIGHT_GAUSS_CUTOFF = 0, OAKG_WEIGHT_GASPARI_COHN = 1
  ! metrics (metrictype)
  integer(c_int32_t), parameter :: OAKG_METRIC_CARTESIAN = 0, OAKG_METRIC_SPHERICAL = 1, &
       OAKG_METRIC_SPHERICAL_APPROX = 2
  ! precision of the local analysis
  integer(c_int32_t), parameter :: OAKG_PREC_FP64 = 0, OAKG_PREC_MIXED = 1, &
       OAKG_PREC_MIXED_FP64EIG = 2
  ! oakg_loc%flags
  integer(c_int32_t), parameter :: OAKG_FLAG_AMPL_ALWAYS = 1, OAKG_FLAG_BRUTE_SEARCH = 2, &
       OAKG_FLAG_SIMT_UPDATE = 4, OAKG_FLAG_SIMT_GRAM = 8

  ! struct oakg_dims (the ensemble size is the C member N; Fortran names are case-blind)
  type, bind(C) :: oakg_dims
    integer(c_int64_t) :: n = 0       ! state vector size
    integer(c_int32_t) :: nens = 0    ! ensemble size (columns of Sf)
    integer(c_int32_t) :: pad0 = 0
    integer(c_int64_t) :: m = 0       ! number of observations
    integer(c_int64_t) :: ldS = 0     ! leading dimension of Sf and Sa
    integer(c_int64_t) :: ldH = 0     ! leading dimension of HSf
    integer(c_int32_t) :: mem = OAKG_MEM_HOST
    integer(c_int32_t) :: pad1 = 0
  end type oakg_dims

  ! struct oakg_loc
  type, bind(C) :: oakg_loc
    integer(c_int32_t) :: weight = OAKG_WEIGHT_GAUSS_CUTOFF
    integer(c_int32_t) :: metric = OAKG_METRIC_SPHERICAL
    integer(c_int32_t) :: loctype = 1
    integer(c_int32_t) :: localise_obs = 1
    integer(c_int32_t) :: rotate = 1
    integer(c_int32_t) :: precision = OAKG_PREC_FP64
    integer(c_int32_t) :: flags = 0
    integer(c_int32_t) :: pad0 = 0
    real(c_double) :: cell_size = 0
  end type oakg_loc

  ! struct oakg_obsoper (sparse observation operator in row form)
  type, bind(C) :: oakg_obsoper
    integer(c_int64_t) :: m = 0
    integer(c_int32_t) :: K = 0
    integer(c_int32_t) :: pad0 = 0
    type(c_ptr) :: index = c_null_ptr
    type(c_ptr) :: weight = c_null_ptr
    type(c_ptr) :: shift = c_null_ptr
  end type oakg_obsoper

  ! What selectObservations evaluates (assimilation.F90:3683-3771), as data: the argument of
  ! gpu_locAnalysis in place of the procedure argument.
  type :: oakg_geometry
    real(c_double), allocatable :: zone_xyzt(:,:)   ! (4, nzones): x,y,z,t of each zone's first element
    real(c_double), allocatable :: obs_x(:), obs_y(:), obs_z(:), obs_t(:)  ! obsGridX/Y/Z/T
    real(c_double), allocatable :: corr_len(:)      ! hCorrLengthToObs at each zone's first element
    real(c_double), allocatable :: max_len(:)       ! hMaxCorrLengthToObs likewise
    type(oakg_loc) :: loc                           ! weight kind, metric, loctype, precision
  end type oakg_geometry

  interface
    integer(c_int) function oakg_analysis(dims, xf, Hxf, yo, Sf, HSf, r_diag, xa, Sa, ampl) &
         bind(C, name="oakg_analysis")
      import
      type(oakg_dims), intent(in) :: dims
      real(c_double), intent(in) :: xf(*), Hxf(*), yo(*), Sf(*), HSf(*), r_diag(*)
      real(c_double), intent(out) :: xa(*)
      real(c_double), intent(out), optional :: Sa(*), ampl(*)
    end function oakg_analysis

    integer(c_int) function oakg_locanalysis(dims, loc, nzones, zone_size, xf, Hxf, yo, Sf, &
         HSf, r_diag, zone_xyzt, obs_x, obs_y, obs_z, obs_t, corr_len, max_len, xa, Sa, ampl, &
         nobs) bind(C, name="oakg_locanalysis")
      import
      type(oakg_dims), intent(in) :: dims
      type(oakg_loc), intent(in) :: loc
      integer(c_int32_t), value :: nzones
      integer(c_int32_t), intent(in) :: zone_size(*)
      real(c_double), intent(in) :: xf(*), Hxf(*), yo(*), Sf(*), HSf(*), r_diag(*), zone_xyzt(*)
      real(c_double), intent(in), optional :: obs_x(*), obs_y(*), obs_z(*), obs_t(*)
      real(c_double), intent(in) :: corr_len(*), max_len(*)
      real(c_double), intent(out) :: xa(*)
      real(c_double), intent(out), optional :: Sa(*), ampl(*)
      integer(c_int32_t), intent(out), optional :: nobs(*)
    end function oakg_locanalysis

    integer(c_int) function oakg_locanalysis_f32(dims, loc, nzones, zone_size, xf, Hxf, yo, &
         Sf, HSf, r_diag, zone_xyzt, obs_x, obs_y, obs_z, obs_t, corr_len, max_len, xa, Sa, &
         ampl, nobs) bind(C, name="oakg_locanalysis_f32")
      import
      type(oakg_dims), intent(in) :: dims
      type(oakg_loc), intent(in) :: loc
      integer(c_int32_t), value :: nzones
      integer(c_int32_t), intent(in) :: zone_size(*)
      real(c_float), intent(in) :: xf(*), Hxf(*), yo(*), Sf(*), HSf(*), r_diag(*)
      real(c_double), intent(in) :: zone_xyzt(*)
      real(c_double), intent(in), optional :: obs_x(*), obs_y(*), obs_z(*), obs_t(*)
      real(c_double), intent(in) :: corr_len(*), max_len(*)
      real(c_float), intent(out) :: xa(*)
      real(c_float), intent(out), optional :: Sa(*), ampl(*)
      integer(c_int32_t), intent(out), optional :: nobs(*)
    end function oakg_locanalysis_f32

    integer(c_int) function oakg_locanalysis_adjoint(dims, loc, nzones, zone_size, Hxf, yo, &
         Sf, HSf, r_diag, zone_xyzt, obs_x, obs_y, obs_z, obs_t, corr_len, max_len, &
         inflation, dJ_dxa, dJ_dyo, dJ_dr, dJ_dlen, dJ_dinfl) &
         bind(C, name="oakg_locanalysis_adjoint")
      import
      type(oakg_dims), intent(in) :: dims
      type(oakg_loc), intent(in) :: loc
      integer(c_int32_t), value :: nzones
      integer(c_int32_t), intent(in) :: zone_size(*)
      real(c_double), intent(in) :: Hxf(*), yo(*), Sf(*), HSf(*), r_diag(*), zone_xyzt(*)
      real(c_double), intent(in), optional :: obs_x(*), obs_y(*), obs_z(*), obs_t(*)
      real(c_double), intent(in) :: corr_len(*), max_len(*)
      real(c_double), value :: inflation
      real(c_double), intent(in) :: dJ_dxa(*)
      real(c_double), intent(out), optional :: dJ_dyo(*), dJ_dr(*)
      real(c_double), intent(out) :: dJ_dlen, dJ_dinfl
    end function oakg_locanalysis_adjoint

    integer(c_int) function oakg_analysis_noalloc(dims, xf, Hxf, yo, Sf, HSf, r_diag, xa, Sa, &
         ampl, stream) bind(C, name="oakg_analysis_noalloc")
      import
      type(oakg_dims), intent(in) :: dims
      real(c_double), intent(in) :: xf(*), Hxf(*), yo(*), Sf(*), HSf(*), r_diag(*)
      real(c_double), intent(out) :: xa(*)
      real(c_double), intent(out), optional :: Sa(*), ampl(*)
      type(c_ptr), value :: stream
    end function oakg_analysis_noalloc

    integer(c_int) function oakg_ensemble_prologue(dims, Ef, ldE, H, xf, Sf, Hxf, HSf) &
         bind(C, name="oakg_ensemble_prologue")
      import
      type(oakg_dims), intent(in) :: dims
      real(c_double), intent(in) :: Ef(*)
      integer(c_int64_t), value :: ldE
      type(oakg_obsoper), intent(in) :: H
      real(c_double), intent(out) :: xf(*), Sf(*), Hxf(*), HSf(*)
    end function oakg_ensemble_prologue

    integer(c_int) function oakg_ensemble_epilogue(dims, xf, xa, Sa, inflation, &
         max_correction, Ea, ldE) bind(C, name="oakg_ensemble_epilogue")
      import
      type(oakg_dims), intent(in) :: dims
      real(c_double), intent(in) :: xf(*), xa(*), Sa(*)
      real(c_double), value :: inflation
      real(c_double), intent(in), optional :: max_correction(*)
      real(c_double), intent(out) :: Ea(*)
      integer(c_int64_t), value :: ldE
    end function oakg_ensemble_epilogue

    integer(c_int) function oakg_locanalysis_smw(dims, loc, nzones, zone_size, xf, Hxf, yo, &
         Sf, HSf, r_diag, k, B, ldB, zone_xyzt, obs_x, obs_y, obs_z, obs_t, corr_len, max_len, &
         xa, Sa, ampl, nobs) bind(C, name="oakg_locanalysis_smw")
      import
      type(oakg_dims), intent(in) :: dims
      type(oakg_loc), intent(in) :: loc
      integer(c_int32_t), value :: nzones
      integer(c_int32_t), intent(in) :: zone_size(*)
      real(c_double), intent(in) :: xf(*), Hxf(*), yo(*), Sf(*), HSf(*), r_diag(*)
      integer(c_int32_t), value :: k
      real(c_double), intent(in) :: B(*)
      integer(c_int64_t), value :: ldB
      real(c_double), intent(in) :: zone_xyzt(*)
      real(c_double), intent(in), optional :: obs_x(*), obs_y(*), obs_z(*), obs_t(*)
      real(c_double), intent(in) :: corr_len(*), max_len(*)
      real(c_double), intent(out) :: xa(*)
      real(c_double), intent(out), optional :: Sa(*), ampl(*)
      integer(c_int32_t), intent(out), optional :: nobs(*)
    end function oakg_locanalysis_smw

    integer(c_int) function oakg_analysis_smw(dims, xf, Hxf, yo, Sf, HSf, r_diag, k, B, ldB, &
         xa, Sa, ampl) bind(C, name="oakg_analysis_smw")
      import
      type(oakg_dims), intent(in) :: dims
      real(c_double), intent(in) :: xf(*), Hxf(*), yo(*), Sf(*), HSf(*), r_diag(*)
      integer(c_int32_t), value :: k
      real(c_double), intent(in) :: B(*)
      integer(c_int64_t), value :: ldB
      real(c_double), intent(out) :: xa(*)
      real(c_double), intent(out), optional :: Sa(*), ampl(*)
    end function oakg_analysis_smw

    integer(c_int) function oakg_ens2sqrt(dims, E, ldE, mean, S) bind(C, name="oakg_ens2sqrt")
      import
      type(oakg_dims), intent(in) :: dims
      real(c_double), intent(in) :: E(*)
      integer(c_int64_t), value :: ldE
      real(c_double), intent(out) :: mean(*), S(*)
    end function oakg_ens2sqrt

    integer(c_int) function oakg_sqrt2ens(dims, mean, S, theta, E, ldE) &
         bind(C, name="oakg_sqrt2ens")
      import
      type(oakg_dims), intent(in) :: dims
      real(c_double), intent(in) :: mean(*), S(*)
      real(c_double), intent(in), optional :: theta(*)
      real(c_double), intent(out) :: E(*)
      integer(c_int64_t), value :: ldE
    end function oakg_sqrt2ens

    integer(c_int) function oakg_ens_analysis(dims, Ef, ldE, HEf, ldHE, yo, r_diag, Ea, xa, &
         ampl) bind(C, name="oakg_ens_analysis")
      import
      type(oakg_dims), intent(in) :: dims
      real(c_double), intent(in) :: Ef(*)
      integer(c_int64_t), value :: ldE
      real(c_double), intent(in) :: HEf(*)
      integer(c_int64_t), value :: ldHE
      real(c_double), intent(in) :: yo(*), r_diag(*)
      real(c_double), intent(out) :: Ea(*)
      real(c_double), intent(out), optional :: xa(*), ampl(*)
    end function oakg_ens_analysis

    integer(c_int) function oakg_biased_locanalysis(dims, loc, nzones, zone_size, gamma, H, &
         xf, bf, Hxf, yo, Sf, HSf, r_diag, zone_xyzt, obs_x, obs_y, obs_z, obs_t, corr_len, &
         max_len, xa, ba, Sa) bind(C, name="oakg_biased_locanalysis")
      import
      type(oakg_dims), intent(in) :: dims
      type(oakg_loc), intent(in) :: loc
      integer(c_int32_t), value :: nzones
      integer(c_int32_t), intent(in) :: zone_size(*)
      real(c_double), value :: gamma
      type(oakg_obsoper), intent(in) :: H
      real(c_double), intent(in) :: xf(*), bf(*), Hxf(*), yo(*), Sf(*), HSf(*), r_diag(*)
      real(c_double), intent(in) :: zone_xyzt(*)
      real(c_double), intent(in), optional :: obs_x(*), obs_y(*), obs_z(*), obs_t(*)
      real(c_double), intent(in) :: corr_len(*), max_len(*)
      real(c_double), intent(out) :: xa(*), ba(*)
      real(c_double), intent(out), optional :: Sa(*)
    end function oakg_biased_locanalysis

    integer(c_int) function oakg_zone_layout(n, partition, nzones, mem, zone_size, &
         zone_index, inv_index) bind(C, name="oakg_zone_layout")
      import
      integer(c_int64_t), value :: n
      integer(c_int32_t), intent(in) :: partition(*)
      integer(c_int32_t), value :: nzones, mem
      integer(c_int32_t), intent(out) :: zone_size(*), zone_index(*)
      integer(c_int32_t), intent(out), optional :: inv_index(*)
    end function oakg_zone_layout

    integer(c_int) function oakg_partition_compact(n, labels, mem, partition, nzones) &
         bind(C, name="oakg_partition_compact")
      import
      integer(c_int64_t), value :: n
      integer(c_int32_t), intent(in) :: labels(*)
      integer(c_int32_t), value :: mem
      integer(c_int32_t), intent(out) :: partition(*)
      integer(c_int32_t), intent(out), optional :: nzones
    end function oakg_partition_compact

    integer(c_int) function oakg_permute_rows(n, ncols, index, X, ldX, Y, ldY, mem) &
         bind(C, name="oakg_permute_rows")
      import
      integer(c_int64_t), value :: n
      integer(c_int32_t), value :: ncols
      integer(c_int32_t), intent(in) :: index(*)
      real(c_double), intent(in) :: X(*)
      integer(c_int64_t), value :: ldX
      real(c_double), intent(out) :: Y(*)
      integer(c_int64_t), value :: ldY
      integer(c_int32_t), value :: mem
    end function oakg_permute_rows

    integer(c_int) function oakg_sea_index(npts, mask, mem, sea, nsea) &
         bind(C, name="oakg_sea_index")
      import
      integer(c_int64_t), value :: npts
      integer(c_int8_t), intent(in) :: mask(*)
      integer(c_int32_t), value :: mem
      integer(c_int64_t), intent(out) :: sea(*)
      integer(c_int64_t), intent(out), optional :: nsea
    end function oakg_sea_index

    integer(c_int) function oakg_obsoper_to_zone_order(count, index, inv_index, n, mem) &
         bind(C, name="oakg_obsoper_to_zone_order")
      import
      integer(c_int64_t), value :: count
      integer(c_int64_t), intent(inout) :: index(*)
      integer(c_int32_t), intent(in) :: inv_index(*)
      integer(c_int64_t), value :: n
      integer(c_int32_t), value :: mem
    end function oakg_obsoper_to_zone_order

    integer(c_int) function oakg_obsoper_rectilinear(ndim, shape, coords, sea, offset, m, pos, &
         mem, index, weight) bind(C, name="oakg_obsoper_rectilinear")
      import
      integer(c_int32_t), value :: ndim
      integer(c_int32_t), intent(in) :: shape(*)
      real(c_double), intent(in) :: coords(*)
      integer(c_int64_t), intent(in), optional :: sea(*)
      integer(c_int64_t), value :: offset, m
      real(c_double), intent(in) :: pos(*)
      integer(c_int32_t), value :: mem
      integer(c_int64_t), intent(out) :: index(*)
      real(c_double), intent(out) :: weight(*)
    end function oakg_obsoper_rectilinear

    integer(c_int) function oakg_ens_locanalysis(dims, loc, nzones, zone_size, Ef, ldE, H, yo, &
         r_diag, zone_xyzt, obs_x, obs_y, obs_z, obs_t, corr_len, max_len, inflation, &
         max_correction, Ea) bind(C, name="oakg_ens_locanalysis")
      import
      type(oakg_dims), intent(in) :: dims
      type(oakg_loc), intent(in) :: loc
      integer(c_int32_t), value :: nzones
      integer(c_int32_t), intent(in) :: zone_size(*)
      real(c_double), intent(in) :: Ef(*)
      integer(c_int64_t), value :: ldE
      type(oakg_obsoper), intent(in) :: H
      real(c_double), intent(in) :: yo(*), r_diag(*), zone_xyzt(*)
      real(c_double), intent(in), optional :: obs_x(*), obs_y(*), obs_z(*), obs_t(*)
      real(c_double), intent(in) :: corr_len(*), max_len(*)
      real(c_double), value :: inflation
      real(c_double), intent(in), optional :: max_correction(*)
      real(c_double), intent(out) :: Ea(*)
    end function oakg_ens_locanalysis

    integer(c_int) function oakg_plan_locanalysis(plan, dims, loc, nzones, zone_size, xf, Hxf, &
         yo, Sf, HSf, r_diag, zone_xyzt, obs_x, obs_y, obs_z, obs_t, corr_len, max_len, xa, Sa, &
         ampl, nobs, tune) bind(C, name="oakg_plan_locanalysis")
      import
      type(c_ptr), intent(out) :: plan
      type(oakg_dims), intent(in) :: dims
      type(oakg_loc), intent(in) :: loc
      integer(c_int32_t), value :: nzones
      integer(c_int32_t), intent(in) :: zone_size(*)
      real(c_double), intent(in) :: xf(*), Hxf(*), yo(*), Sf(*), HSf(*), r_diag(*), zone_xyzt(*)
      real(c_double), intent(in), optional :: obs_x(*), obs_y(*), obs_z(*), obs_t(*)
      real(c_double), intent(in) :: corr_len(*), max_len(*)
      real(c_double), intent(out) :: xa(*)
      real(c_double), intent(out), optional :: Sa(*), ampl(*)
      integer(c_int32_t), intent(out), optional :: nobs(*)
      integer(c_int32_t), value :: tune
    end function oakg_plan_locanalysis

    integer(c_int) function oakg_plan_execute(plan, stream) bind(C, name="oakg_plan_execute")
      import
      type(c_ptr), value :: plan, stream
    end function oakg_plan_execute

    integer(c_int) function oakg_plan_info(plan, cell_size, graph_nodes, tune_cell, tune_ms, &
         ntune) bind(C, name="oakg_plan_info")
      import
      type(c_ptr), value :: plan
      real(c_double), intent(out), optional :: cell_size
      integer(c_int64_t), intent(out), optional :: graph_nodes
      real(c_double), intent(out), optional :: tune_cell(*), tune_ms(*)
      integer(c_int32_t), value :: ntune
    end function oakg_plan_info

    integer(c_int) function oakg_plan_schedule(plan, index_order_ms, count_order_ms) &
         bind(C, name="oakg_plan_schedule")
      import
      type(c_ptr), value :: plan
      real(c_double), intent(out), optional :: index_order_ms, count_order_ms
    end function oakg_plan_schedule

    subroutine oakg_plan_destroy(plan) bind(C, name="oakg_plan_destroy")
      import
      type(c_ptr), value :: plan
    end subroutine oakg_plan_destroy

    integer(c_size_t) function oakg_last_error(buf, len) bind(C, name="oakg_last_error")
      import
      character(kind=c_char), intent(out) :: buf(*)
      integer(c_size_t), value :: len
    end function oakg_last_error

    integer(c_int) function oakg_last_status() bind(C, name="oakg_last_status")
      import
    end function oakg_last_status

    integer(c_int) function oakg_release() bind(C, name="oakg_release")
      import
    end function oakg_release

    integer(c_int) function oakg_last_timings(ms, n) bind(C, name="oakg_last_timings")
      import
      real(c_double), intent(out) :: ms(*)
      integer(c_int), value :: n
    end function oakg_last_timings

    integer(c_int) function oakg_set_stream(stream) bind(C, name="oakg_set_stream")
      import
      type(c_ptr), value :: stream
    end function oakg_set_stream

    integer(c_int64_t) function oakg_launch_count() bind(C, name="oakg_launch_count")
      import
    end function oakg_launch_count

    integer(c_int) function oakg_fp64_peak(tflops) bind(C, name="oakg_fp64_peak")
      import
      real(c_double), intent(out) :: tflops
    end function oakg_fp64_peak

    integer(c_int) function oakg_read_variable(spec, values, capacity, count, shape, ndim, &
         valex) bind(C, name="oakg_read_variable")
      import
      character(kind=c_char), intent(in) :: spec(*)
      real(c_double), intent(out), optional :: values(*)
      integer(c_int64_t), value :: capacity
      integer(c_int64_t), intent(out) :: count
      integer(c_int64_t), intent(out) :: shape(*)
      integer(c_int32_t), intent(out) :: ndim
      real(c_double), intent(out) :: valex
    end function oakg_read_variable

    ! OAK's own C interface (assimilation.F90:4911-4933), exported by the library
    subroutine oak_init(fname) bind(C, name="oak_init")
      import
      character(kind=c_char), intent(in) :: fname(*)
    end subroutine oak_init

    subroutine oak_assim(ntime, n, r, Ef, Ea) bind(C, name="oak_assim")
      import
      integer(c_int), value :: ntime, n, r
      real(c_double) :: Ef(*)
      real(c_double) :: Ea(*)
    end subroutine oak_assim

    subroutine oak_done() bind(C, name="oak_done")
      import
    end subroutine oak_done
  end interface

contains

  ! The library's message as a Fortran string.
  function c2f() result(msg)
    character(len=512) :: msg
    character(kind=c_char) :: buf(512)
    integer(c_size_t) :: len, i
    len = oakg_last_error(buf, int(512, c_size_t))
    msg = ''
    do i = 1, min(len, int(511, c_size_t))
      msg(i:i) = buf(i)
    end do
  end function c2f

  ! A failed call stops the program, as the reference does on errors.
  subroutine check(status, where)
    integer(c_int), intent(in) :: status
    character(len=*), intent(in) :: where
    if (status /= OAKG_OK) then
      write(0, '(A,": status ",I0,": ",A)') where, status, trim(c2f())
      error stop 1
    end if
  end subroutine check

  ! analysis (rrsqrt.F90:196-208) on the GPU, with R = DiagCovar(R) (covariance.F90:70-79).
  subroutine gpu_analysis(xf, Hxf, yo, Sf, HSf, R, xa, Sa, amplitudes)
    real(c_double), intent(in) :: xf(:), Hxf(:), yo(:), R(:)
    real(c_double), intent(in), contiguous :: Sf(:,:), HSf(:,:)
    real(c_double), intent(out) :: xa(:)
    real(c_double), intent(out), optional, contiguous :: Sa(:,:)
    real(c_double), intent(out), optional :: amplitudes(:)
    type(oakg_dims) :: dims
    dims%n = size(xf)
    dims%nens = size(Sf, 2)
    dims%m = size(yo)
    dims%ldS = size(Sf, 1)
    dims%ldH = max(size(HSf, 1), 1)
    dims%mem = OAKG_MEM_HOST
    call check(oakg_analysis(dims, xf, Hxf, yo, Sf, HSf, R, xa, Sa, amplitudes), 'gpu_analysis')
  end subroutine gpu_analysis

  ! locAnalysis (rrsqrt.F90:433-466) on the GPU. zoneSize, xf, Hxf, yo, Sf, HSf, xa, Sa,
  ! amplitudes and localise_obs as in the reference; R = DiagCovar(R); geometry replaces
  ! selectObservations. The state is in zone order (initPartition, assimilation.F90:578-641).
  subroutine gpu_locAnalysis(zoneSize, geometry, xf, Hxf, yo, Sf, HSf, R, xa, Sa, amplitudes, &
       localise_obs)
    integer(c_int32_t), intent(in) :: zoneSize(:)
    type(oakg_geometry), intent(in) :: geometry
    real(c_double), intent(in) :: xf(:), Hxf(:), yo(:), R(:)
    real(c_double), intent(in), contiguous :: Sf(:,:), HSf(:,:)
    real(c_double), intent(out) :: xa(:)
    real(c_double), intent(out), optional, contiguous :: Sa(:,:), amplitudes(:,:)
    logical, intent(in), optional :: localise_obs
    type(oakg_dims) :: dims
    type(oakg_loc) :: loc
    dims%n = size(xf)
    dims%nens = size(Sf, 2)
    dims%m = size(yo)
    dims%ldS = size(Sf, 1)
    dims%ldH = max(size(HSf, 1), 1)
    dims%mem = OAKG_MEM_HOST
    loc = geometry%loc
    loc%localise_obs = 1
    if (present(localise_obs)) then
      if (.not. localise_obs) loc%localise_obs = 0
    end if
    call check(oakg_locanalysis(dims, loc, int(size(zoneSize), c_int32_t), zoneSize, xf, Hxf, &
         yo, Sf, HSf, R, geometry%zone_xyzt, geometry%obs_x, geometry%obs_y, geometry%obs_z, &
         geometry%obs_t, geometry%corr_len, geometry%max_len, xa, Sa, amplitudes), &
         'gpu_locAnalysis')
  end subroutine gpu_locAnalysis

  ! gpu_locAnalysis for the reference's single-precision build (PRECISION=single: real is
  ! real(4)); the geometry stays real(c_double).
  subroutine gpu_locAnalysis_r4(zoneSize, geometry, xf, Hxf, yo, Sf, HSf, R, xa, Sa, &
       amplitudes, localise_obs)
    integer(c_int32_t), intent(in) :: zoneSize(:)
    type(oakg_geometry), intent(in) :: geometry
    real(c_float), intent(in) :: xf(:), Hxf(:), yo(:), R(:)
    real(c_float), intent(in), contiguous :: Sf(:,:), HSf(:,:)
    real(c_float), intent(out) :: xa(:)
    real(c_float), intent(out), optional, contiguous :: Sa(:,:), amplitudes(:,:)
    logical, intent(in), optional :: localise_obs
    type(oakg_dims) :: dims
    type(oakg_loc) :: loc
    dims%n = size(xf)
    dims%nens = size(Sf, 2)
    dims%m = size(yo)
    dims%ldS = size(Sf, 1)
    dims%ldH = max(size(HSf, 1), 1)
    dims%mem = OAKG_MEM_HOST
    loc = geometry%loc
    loc%localise_obs = 1
    if (present(localise_obs)) then
      if (.not. localise_obs) loc%localise_obs = 0
    end if
    call check(oakg_locanalysis_f32(dims, loc, int(size(zoneSize), c_int32_t), zoneSize, xf, &
         Hxf, yo, Sf, HSf, R, geometry%zone_xyzt, geometry%obs_x, geometry%obs_y, &
         geometry%obs_z, geometry%obs_t, geometry%corr_len, geometry%max_len, xa, Sa, &
         amplitudes), 'gpu_locAnalysis_r4')
  end subroutine gpu_locAnalysis_r4

  ! Gradients of a cost J(xa) of gpu_locAnalysis's mean, given dJ/dxa: with respect to the
  ! observations (dJ_dyo), their error variances (dJ_dr), a common factor on the correlation
  ! and maximum lengths (dJ_dlen) and the prior anomaly inflation (dJ_dinfl). Sf and HSf are
  ! the anomalies before the inflation.
  subroutine gpu_locAnalysis_adjoint(zoneSize, geometry, Hxf, yo, Sf, HSf, R, inflation, &
       dJ_dxa, dJ_dyo, dJ_dr, dJ_dlen, dJ_dinfl)
    integer(c_int32_t), intent(in) :: zoneSize(:)
    type(oakg_geometry), intent(in) :: geometry
    real(c_double), intent(in) :: Hxf(:), yo(:), R(:), dJ_dxa(:)
    real(c_double), intent(in), contiguous :: Sf(:,:), HSf(:,:)
    real(c_double), intent(in) :: inflation
    real(c_double), intent(out), optional :: dJ_dyo(:), dJ_dr(:)
    real(c_double), intent(out) :: dJ_dlen, dJ_dinfl
    type(oakg_dims) :: dims
    dims%n = size(Sf, 1)
    dims%nens = size(Sf, 2)
    dims%m = size(yo)
    dims%ldS = size(Sf, 1)
    dims%ldH = max(size(HSf, 1), 1)
    dims%mem = OAKG_MEM_HOST
    call check(oakg_locanalysis_adjoint(dims, geometry%loc, int(size(zoneSize), c_int32_t), &
         zoneSize, Hxf, yo, Sf, HSf, R, geometry%zone_xyzt, geometry%obs_x, geometry%obs_y, &
         geometry%obs_z, geometry%obs_t, geometry%corr_len, geometry%max_len, inflation, &
         dJ_dxa, dJ_dyo, dJ_dr, dJ_dlen, dJ_dinfl), 'gpu_locAnalysis_adjoint')
  end subroutine gpu_locAnalysis_adjoint

end module oakg
