!! m_euler2d_gb300.f90 -- ISO_C_BINDING interface to libeuler2d_gb300.so
!! (include/euler2d_gb300.h) and a drop-in replacement of the procedures of
!! serial_ref/m_run.f90 that serial_ref/main.f90 calls.
!!
!! Build (with any Fortran 2003 compiler, against the reference's own
!! m_precision / m_constants / m_parameters modules, and instead of m_run.f90):
!!   gfortran -c m_precision.f90 m_constants.f90 m_parameters.f90 m_monitoring.f90
!!   gfortran -c m_euler2d_gb300.f90 main.f90
!!   gfortran -o euler2d *.o -L<path>/_build/<machine> -leuler2d_gb300 -Wl,-rpath,<path>/_build/<machine>
!! (or -leuler2d_gb300_fma, the build with fused multiply-adds)
!! main.f90 is used unchanged.  No Fortran compiler exists where this project
!! is built and tested, so this file is shipped uncompiled.
module m_euler2d_gb300_abi

  use iso_c_binding
  implicit none

  type, bind(C) :: e2d_params
     integer(c_int) :: nx, ny
     real(c_double) :: gamma0, cfl, smallr, smallc
     integer(c_int) :: niter_riemann, iorder, slope_type
     integer(c_int) :: boundary_type_xmin, boundary_type_xmax
     integer(c_int) :: boundary_type_ymin, boundary_type_ymax
     integer(c_int) :: implementation_version, riemann_solver, precision
  end type e2d_params

  interface
     integer(c_int) function e2d_default_params(p) bind(C, name="e2d_default_params")
       import :: c_int, e2d_params
       type(e2d_params), intent(out) :: p
     end function e2d_default_params

     integer(c_int) function e2d_arithmetic(mode) bind(C, name="e2d_arithmetic")
       import :: c_int
       integer(c_int), intent(out) :: mode   ! 0: exact build, 1: fused multiply-adds
     end function e2d_arithmetic

     integer(c_int) function e2d_create(p, h) bind(C, name="e2d_create")
       import :: c_int, c_ptr, e2d_params
       type(e2d_params), intent(in) :: p
       type(c_ptr), intent(out) :: h
     end function e2d_create

     integer(c_int) function e2d_destroy(h) bind(C, name="e2d_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
     end function e2d_destroy

     integer(c_int) function e2d_init_implode(h) bind(C, name="e2d_init_implode")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
     end function e2d_init_implode

     integer(c_int) function e2d_upload_state(h, which, host) bind(C, name="e2d_upload_state")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
       integer(c_int), value :: which
       type(c_ptr), value :: host
     end function e2d_upload_state

     integer(c_int) function e2d_download_state(h, which, host) bind(C, name="e2d_download_state")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
       integer(c_int), value :: which
       type(c_ptr), value :: host
     end function e2d_download_state

     integer(c_int) function e2d_compute_dt(h, useU, dt) bind(C, name="e2d_compute_dt")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
       integer(c_int), value :: useU
       type(c_ptr), value :: dt          ! c_loc of a real(fp_kind) scalar
     end function e2d_compute_dt

     integer(c_int) function e2d_make_boundaries(h, which) bind(C, name="e2d_make_boundaries")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
       integer(c_int), value :: which
     end function e2d_make_boundaries

     integer(c_int) function e2d_godunov_unsplit(h, nStep, dt) bind(C, name="e2d_godunov_unsplit")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       integer(c_int), value :: nStep
       real(c_double), value :: dt
     end function e2d_godunov_unsplit

     integer(c_int) function e2d_advance(h, nStep0, nsteps, dt_log) bind(C, name="e2d_advance")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
       integer(c_int), value :: nStep0, nsteps
       type(c_ptr), value :: dt_log
     end function e2d_advance
  end interface

end module m_euler2d_gb300_abi

!! The m_run module of serial_ref, with the same public names, backed by the
!! GB300 library.  u and u2 stay host arrays for saveVTK; the time-stepping
!! state lives on the GPU and is downloaded only when saveVTK needs it.
module m_run

  use m_precision
  use m_constants
  use m_parameters
  use m_euler2d_gb300_abi
  use iso_c_binding

  implicit none

  real(fp_kind), dimension(:,:,:), allocatable, target :: u, u2
  type(HydroPar)    :: hydroParams
  integer(int_kind) :: nStepmax, nOutput
  real(fp_kind)     :: tEnd
  integer(int_kind), parameter :: ghostWidth = 2
  integer(int_kind) :: imin=0, imax=0, jmin=0, jmax=0
  integer(int_kind) :: implementationVersion = 0
  character(len=8)  :: riemann_solver = 'approx'
  type(c_ptr)       :: run = c_null_ptr

contains

  subroutine check(rc, what)
    integer(c_int), intent(in) :: rc
    character(len=*), intent(in) :: what
    if (rc /= 0) then
       write(*,*) 'euler2d_gb300 error in ', what, ': code ', rc
       stop
    end if
  end subroutine check

  subroutine initHydroParameters()
    integer(int_kind) :: narg, ios
    character(LEN=80) :: inputFilename
    integer(int_kind) :: nx, ny, niter_riemann=10, iorder, slope_type
    integer(int_kind) :: boundary_type_xmin=1, boundary_type_xmax=1, boundary_type_ymin=1, boundary_type_ymax=1
    real(fp_kind)     :: gamma0, cfl, smallr, smallc
    namelist/run/tEnd,nStepmax,nOutput
    namelist/mesh/nx,ny,boundary_type_xmin,boundary_type_xmax,boundary_type_ymin,boundary_type_ymax
    namelist/hydro/gamma0,cfl,smallr,smallc,niter_riemann,iorder,slope_type
    namelist/other/implementationVersion
    namelist/gb300/riemann_solver

    narg = COMMAND_ARGUMENT_COUNT()
    if (narg .ne. 1) then
       write(*,*)'You should provide an input parameter file (with a namelist)'
       stop
    end if
    call GET_COMMAND_ARGUMENT(1,inputFilename)
    open(1,file=inputFilename)
    read(1,NML=run)
    read(1,NML=mesh)
    read(1,NML=hydro)
    read(1,NML=other,iostat=ios)   ! optional groups
    rewind(1)
    read(1,NML=gb300,iostat=ios)
    close(1)

    hydroParams%nx = nx
    hydroParams%ny = ny
    hydroParams%boundary_type_xmin = boundary_type_xmin
    hydroParams%boundary_type_xmax = boundary_type_xmax
    hydroParams%boundary_type_ymin = boundary_type_ymin
    hydroParams%boundary_type_ymax = boundary_type_ymax
    imin = 1
    jmin = 1
    imax = nx+2*ghostWidth
    jmax = ny+2*ghostWidth
    hydroParams%isize = imax - imin + 1
    hydroParams%jsize = jmax - jmin + 1
    hydroParams%dx = 1.0_fp_kind / nx
    hydroParams%dy = 1.0_fp_kind / ny
    hydroParams%gamma0 = gamma0
    hydroParams%cfl = cfl
    hydroParams%smallr = smallr
    hydroParams%smallc = smallc
    hydroParams%niter_riemann = niter_riemann
    hydroParams%iorder = iorder
    hydroParams%slope_type = slope_type
    hydroParams%smallp  = smallc * smallc / gamma0
    hydroParams%smallpp = smallr * hydroParams%smallp
    hydroParams%gamma6  = (gamma0 + ONE_F) / (TWO_F * gamma0)
  end subroutine initHydroParameters

  subroutine printHydroParameters()
    write(*,*) 'Simulation run parameters:'
    write(*,*) 'nx : ', hydroParams%nx
    write(*,*) 'ny : ', hydroParams%ny
    write(*,*) 'nStepmax,tEnd,nOutput : ',nStepmax,tEnd,nOutput
    write(*,*) 'implementationVersion, riemann_solver : ', implementationVersion, ' ', trim(riemann_solver)
  end subroutine printHydroParameters

  subroutine run_init()
    type(e2d_params) :: p
    call check(e2d_default_params(p), 'default_params')
    p%nx = hydroParams%nx
    p%ny = hydroParams%ny
    p%gamma0 = real(hydroParams%gamma0, c_double)
    p%cfl = real(hydroParams%cfl, c_double)
    p%smallr = real(hydroParams%smallr, c_double)
    p%smallc = real(hydroParams%smallc, c_double)
    p%niter_riemann = hydroParams%niter_riemann
    p%iorder = hydroParams%iorder
    p%slope_type = hydroParams%slope_type
    p%boundary_type_xmin = hydroParams%boundary_type_xmin
    p%boundary_type_xmax = hydroParams%boundary_type_xmax
    p%boundary_type_ymin = hydroParams%boundary_type_ymin
    p%boundary_type_ymax = hydroParams%boundary_type_ymax
    p%implementation_version = implementationVersion
    p%riemann_solver = 0
    if (trim(riemann_solver) == 'hllc') p%riemann_solver = 2
    p%precision = int(storage_size(1.0_fp_kind) / 8, c_int)
    call check(e2d_create(p, run), 'create')
    allocate( u (hydroParams%isize, hydroParams%jsize, NBVAR) )
    allocate( u2(hydroParams%isize, hydroParams%jsize, NBVAR) )
    call check(e2d_init_implode(run), 'init_implode')
    call check(e2d_download_state(run, 0_c_int, c_loc(u)), 'download_state')
    u2 = 0.0
  end subroutine run_init

  subroutine run_cleanup()
    call check(e2d_destroy(run), 'destroy')
    run = c_null_ptr
    deallocate(u)
    deallocate(u2)
  end subroutine run_cleanup

  !! compute_dt of serial_ref/m_run.f90:248; the running max lives in the run.
  subroutine compute_dt(params, dt, useU)
    type(HydroPar)   , intent(in)  :: params
    real(fp_kind)    , intent(out), target :: dt
    integer(int_kind), intent(in)  :: useU
    call check(e2d_compute_dt(run, int(useU, c_int), c_loc(dt)), 'compute_dt')
  end subroutine compute_dt

  !! make_boundaries of serial_ref/m_run.f90:561; main.f90 calls it on u only.
  subroutine make_boundaries(params, data)
    type(HydroPar), intent(in) :: params
    real(fp_kind), dimension(params%isize, params%jsize, nbVar), intent(inout), target :: data
    integer(c_int) :: which
    which = 0
    if (c_associated(c_loc(data), c_loc(u2))) which = 1
    call check(e2d_make_boundaries(run, which), 'make_boundaries')
  end subroutine make_boundaries

  !! godunov_unsplit of serial_ref/m_run.f90:187 (u -> u2 if nStep even).
  subroutine godunov_unsplit(nStep, dt)
    integer      , intent(in) :: nStep
    real(fp_kind), intent(in) :: dt
    call check(e2d_godunov_unsplit(run, int(nStep, c_int), real(dt, c_double)), 'godunov_unsplit')
  end subroutine godunov_unsplit

  !! saveVTK of serial_ref/m_run.f90:653: fetch the state from the GPU first.
  subroutine saveVTK(data, iStep)
    real(fp_kind), dimension(hydroParams%isize, hydroParams%jsize, NBVAR), intent(inout), target :: data
    integer(int_kind) :: iStep
    integer(c_int) :: which
    integer :: j, iVar
    character(LEN=8) :: filenum
    character(LEN=7) :: floatType
    floatType = 'Float32'
    if (useDoublePrecision()) floatType = 'Float64'
    which = 0
    if (c_associated(c_loc(data), c_loc(u2))) which = 1
    call check(e2d_download_state(run, which, c_loc(data)), 'download_state')
    write (filenum,'(i8.8)') iStep
    open(10, file='euler2d_'//filenum//'.vti')
    write(10,'(a)') '<?xml version="1.0"?>'
    write(10,'(a)') '<VTKFile type="ImageData" version="0.1" byte_order="LittleEndian">'
    write(10,'(a,6(I7),a)') '  <ImageData WholeExtent="',1,hydroParams%nx+1,1,hydroParams%ny+1,1,2,'"'
    write(10,'(a)') ' Origin="0 0 0" Spacing="1 1 1">'
    write(10,'(a,6(I7),a)') '  <Piece Extent="',1,hydroParams%nx+1,1,hydroParams%ny+1,1,2,'">'
    write(10,'(a)') '   <PointData>'
    write(10,'(a)') '    </PointData>'
    write(10,'(a)') '    <CellData>'
    do iVar=1,NBVAR
       write(10,'(a)') '    <DataArray type="'//floatType//'" Name="'//varNames(iVar)//'" format="ascii" >'
       do j=jmin+ghostWidth,jmax-ghostWidth
          write(10,*) data(imin+ghostWidth:imax-ghostWidth,j,iVar)
       end do
       write(10,'(a)') '    </DataArray>'
    end do
    write(10,'(a)') '    </CellData>'
    write(10,'(a)') '  </Piece>'
    write(10,'(a)') '  </ImageData>'
    write(10,'(a)') '</VTKFile>'
    close(10)
  end subroutine saveVTK

end module m_run
