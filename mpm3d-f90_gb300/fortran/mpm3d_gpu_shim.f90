!-------------------------------------------------------------------------
! mpm3d_gpu_shim.f90 -- ISO_C_BINDING layer between the MPM3D-F90 host and
! libmpm3d_gpu (include/mpm3d_gpu.h).
!
! Use: compile this file with the reference sources and link
! libmpm3d_gpu.so. In MPM3D.f90, call gpu_init(FileInp) after InputPara and
! keep the time loop as it is: the step subroutines of update_step.f90
! (GridMomentumInitial, ApplyBoundaryConditions, ParticleStressUpdate,
! GridMomentumUpdate, IntegrateMomentum, ParticlePositionUpdate,
! GridMomentumMUSL, UpdateDT, SmoothStressbyGrid, Lagr_NodContact) and calcEnergy /
! dynamicRelaxationDamping of Particle.f90 are replaced by the gpu_* routines
! below, one C call each.
! gpu_sync_scalars copies DT, CurrentTime, energies and momentum back into
! the ParticleData globals; gpu_fetch_particles refreshes particle_list
! before OutCurve / OutAnim.
!
! The library parses the same .mpm file (mpm_deck_load) and derives the
! set-up itself, so the device state starts from exactly the deck the host
! read.
!-------------------------------------------------------------------------
module mpm3d_gpu
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: MPM_FP64_STRICT = 0, MPM_FP64_NATIVE = 1, MPM_MIXED = 2
  integer(c_int), parameter :: PH_GRID_MOMENTUM_INITIAL = 1, PH_APPLY_BOUNDARY = 2, &
       PH_PARTICLE_STRESS_UPDATE = 3, PH_GRID_MOMENTUM_UPDATE = 4, &
       PH_INTEGRATE_MOMENTUM = 5, PH_PARTICLE_POSITION_UPDATE = 6, &
       PH_GRID_MOMENTUM_MUSL = 7, PH_CALC_ENERGY = 8, PH_UPDATE_DT = 9, &
       PH_DR_DAMPING = 10, PH_BEGIN_STEP = 11, PH_SMOOTH_STRESS = 12, PH_CONTACT = 13
  integer(c_int), parameter :: F_XP = 1, F_VXP = 3, F_VOL = 7, F_SM = 10, F_SEQV = 11, &
       F_SD = 12, F_EPEFF = 14, F_CELSIUS = 15, F_IE = 18, F_CP = 20, F_FAILURE = 22, &
       F_SPRE = 26

  type(c_ptr), save :: ctx = c_null_ptr
  type(c_ptr), save :: deck = c_null_ptr
  ! page-locked download buffer of gpu_fetch_particles (9 * nb_particle)
  type(c_ptr), save :: hbuf = c_null_ptr
  integer(c_int64_t), save :: hbuf_n = 0

  interface
     integer(c_int) function mpm_deck_load(path, out, errbuf, errlen) bind(C, name="mpm_deck_load")
       import :: c_int, c_ptr, c_char
       character(kind=c_char), dimension(*) :: path
       type(c_ptr) :: out
       character(kind=c_char), dimension(*) :: errbuf
       integer(c_int), value :: errlen
     end function
     subroutine mpm_deck_free(d) bind(C, name="mpm_deck_free")
       import :: c_ptr
       type(c_ptr), value :: d
     end subroutine
     integer(c_int) function mpm_create(d, precision, device, out) bind(C, name="mpm_create")
       import :: c_int, c_ptr
       type(c_ptr), value :: d
       integer(c_int), value :: precision, device
       type(c_ptr) :: out
     end function
     subroutine mpm_destroy(c) bind(C, name="mpm_destroy")
       import :: c_ptr
       type(c_ptr), value :: c
     end subroutine
     integer(c_int) function mpm_step_phase(c, phase) bind(C, name="mpm_step_phase")
       import :: c_int, c_ptr
       type(c_ptr), value :: c
       integer(c_int), value :: phase
     end function
     integer(c_int) function mpm_step(c) bind(C, name="mpm_step")
       import :: c_int, c_ptr
       type(c_ptr), value :: c
     end function
     integer(c_int) function mpm_get_scalars(c, out16) bind(C, name="mpm_get_scalars")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: c
       real(c_double), dimension(16) :: out16
     end function
     integer(c_int) function mpm_download(c, field, out) bind(C, name="mpm_download")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: c
       integer(c_int), value :: field
       real(c_double), dimension(*) :: out
     end function
     integer(c_int) function mpm_deck_pin(d, on) bind(C, name="mpm_deck_pin")
       import :: c_int, c_ptr
       type(c_ptr), value :: d
       integer(c_int), value :: on
     end function
     type(c_ptr) function mpm_host_alloc(bytes) bind(C, name="mpm_host_alloc")
       import :: c_ptr, c_int64_t
       integer(c_int64_t), value :: bytes
     end function
     subroutine mpm_host_free(p) bind(C, name="mpm_host_free")
       import :: c_ptr
       type(c_ptr), value :: p
     end subroutine
     integer(c_int) function mpm_sync(c) bind(C, name="mpm_sync")
       import :: c_int, c_ptr
       type(c_ptr), value :: c
     end function
  end interface

contains

  subroutine check(st, what)
    integer(c_int), intent(in) :: st
    character(*), intent(in) :: what
    if (st /= 0) then
       write(*, *) '*** libmpm3d_gpu error ', st, ' in ', what
       stop 'GPU step failed'
    end if
  end subroutine check

  ! Parse the deck in the library and create the device context.
  subroutine gpu_init(fileinp, precision)
    character(*), intent(in) :: fileinp
    integer, intent(in), optional :: precision
    character(kind=c_char, len=256) :: err
    integer(c_int) :: prec
    prec = MPM_FP64_STRICT
    if (present(precision)) prec = precision
    call check(mpm_deck_load(trim(fileinp)//c_null_char, deck, err, 256_c_int), 'mpm_deck_load')
    ! the particle arrays page-locked for the upload in mpm_create
    call check(mpm_deck_pin(deck, 1_c_int), 'mpm_deck_pin')
    call check(mpm_create(deck, prec, -1_c_int, ctx), 'mpm_create')
    call check(mpm_deck_pin(deck, 0_c_int), 'mpm_deck_pin')
  end subroutine gpu_init

  subroutine gpu_finalize()
    if (c_associated(hbuf)) call mpm_host_free(hbuf)
    hbuf = c_null_ptr
    hbuf_n = 0
    call mpm_destroy(ctx)
    call mpm_deck_free(deck)
    ctx = c_null_ptr
    deck = c_null_ptr
  end subroutine gpu_finalize

  ! MPM3D.f90:72-74 (istep + 1, CurrentTime + DT) on the device copy
  subroutine gpu_begin_step()
    call check(mpm_step_phase(ctx, PH_BEGIN_STEP), 'BeginStep')
  end subroutine
  subroutine gpu_GridMomentumInitial()
    call check(mpm_step_phase(ctx, PH_GRID_MOMENTUM_INITIAL), 'GridMomentumInitial')
  end subroutine
  subroutine gpu_ApplyBoundaryConditions()
    call check(mpm_step_phase(ctx, PH_APPLY_BOUNDARY), 'ApplyBoundaryConditions')
  end subroutine
  subroutine gpu_ParticleStressUpdate()
    call check(mpm_step_phase(ctx, PH_PARTICLE_STRESS_UPDATE), 'ParticleStressUpdate')
  end subroutine
  subroutine gpu_GridMomentumUpdate()
    call check(mpm_step_phase(ctx, PH_GRID_MOMENTUM_UPDATE), 'GridMomentumUpdate')
  end subroutine
  subroutine gpu_IntegrateMomentum()
    call check(mpm_step_phase(ctx, PH_INTEGRATE_MOMENTUM), 'IntegrateMomentum')
  end subroutine
  subroutine gpu_ParticlePositionUpdate()
    call check(mpm_step_phase(ctx, PH_PARTICLE_POSITION_UPDATE), 'ParticlePositionUpdate')
  end subroutine
  subroutine gpu_GridMomentumMUSL()
    call check(mpm_step_phase(ctx, PH_GRID_MOMENTUM_MUSL), 'GridMomentumMUSL')
  end subroutine
  subroutine gpu_calcEnergy()
    call check(mpm_step_phase(ctx, PH_CALC_ENERGY), 'calcEnergy')
  end subroutine
  subroutine gpu_UpdateDT()
    call check(mpm_step_phase(ctx, PH_UPDATE_DT), 'UpdateDT')
  end subroutine
  subroutine gpu_dynamicRelaxationDamping()
    call check(mpm_step_phase(ctx, PH_DR_DAMPING), 'dynamicRelaxationDamping')
  end subroutine
  subroutine gpu_SmoothStressbyGrid()
    call check(mpm_step_phase(ctx, PH_SMOOTH_STRESS), 'SmoothStressbyGrid')
  end subroutine
  subroutine gpu_Lagr_NodContact()
    call check(mpm_step_phase(ctx, PH_CONTACT), 'Lagr_NodContact')
  end subroutine

  ! One whole step (the fused kernel sequence) instead of the phases above.
  subroutine gpu_step()
    call check(mpm_step(ctx), 'mpm_step')
  end subroutine

  ! Copy the loop scalars back into the ParticleData globals.
  subroutine gpu_sync_scalars()
    use ParticleData, only: istep, CurrentTime, DT, EngKinetic, EngInternal, Momentum
    real(c_double) :: s(16)
    call check(mpm_get_scalars(ctx, s), 'mpm_get_scalars')
    istep = int(s(1))
    CurrentTime = s(2)
    DT = s(3)
    EngKinetic = s(4)
    EngInternal = s(5)
    Momentum = s(6:8)
  end subroutine gpu_sync_scalars

  ! Refresh particle_list (positions, velocities, stresses, energies) for the
  ! output writers of DataOut.f90.
  subroutine gpu_fetch_particles()
    use ParticleData, only: particle_list, nb_particle
    real(c_double), pointer :: buf(:)
    integer :: n, c
    n = nb_particle
    ! a page-locked buffer, kept for the next fetch: the copies run at the
    ! link's bandwidth instead of through the driver's staging
    if (hbuf_n < 9_c_int64_t * n) then
       if (c_associated(hbuf)) call mpm_host_free(hbuf)
       hbuf = mpm_host_alloc(8_c_int64_t * 9_c_int64_t * n)
       if (.not. c_associated(hbuf)) stop 'page-locked buffer allocation failed'
       hbuf_n = 9_c_int64_t * n
    end if
    call c_f_pointer(hbuf, buf, [9 * n])
    call check(mpm_download(ctx, F_XP, buf), 'Xp')
    do c = 1, 3
       particle_list(:)%Xp(c) = buf((c - 1) * n + 1:c * n)
    end do
    call check(mpm_download(ctx, F_VXP, buf), 'VXp')
    do c = 1, 3
       particle_list(:)%VXp(c) = buf((c - 1) * n + 1:c * n)
    end do
    call check(mpm_download(ctx, F_SD, buf), 'SD')
    particle_list(:)%SDxx = buf(1:n)
    particle_list(:)%SDyy = buf(n + 1:2 * n)
    particle_list(:)%SDzz = buf(2 * n + 1:3 * n)
    particle_list(:)%SDxy = buf(3 * n + 1:4 * n)
    particle_list(:)%SDyz = buf(4 * n + 1:5 * n)
    particle_list(:)%SDxz = buf(5 * n + 1:6 * n)
    call check(mpm_download(ctx, F_SM, buf), 'SM')
    particle_list(:)%SM = buf(1:n)
    call check(mpm_download(ctx, F_SEQV, buf), 'Seqv')
    particle_list(:)%Seqv = buf(1:n)
    call check(mpm_download(ctx, F_VOL, buf), 'VOL')
    particle_list(:)%VOL = buf(1:n)
    call check(mpm_download(ctx, F_EPEFF, buf), 'epeff')
    particle_list(:)%epeff = buf(1:n)
    call check(mpm_download(ctx, F_IE, buf), 'ie')
    particle_list(:)%ie = buf(1:n)
    call check(mpm_download(ctx, F_CELSIUS, buf), 'celsius_t')
    particle_list(:)%celsius_t = buf(1:n)
    call check(mpm_download(ctx, F_SPRE, buf), 'Spre')
    particle_list(:)%Spre = buf(1:n)
    nullify(buf)
  end subroutine gpu_fetch_particles

end module mpm3d_gpu
