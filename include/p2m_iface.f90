! p2m_iface.f90 -- ISO_C_BINDING interface of the GB300 halo painter (include/p2m.h) for
! the reference's Fortran host, pks2map.f90.
!
! The reference calls projecthalo_flatsky and projecthalo_healpix per halo
! (pks2map.f90:300-301) after loadmaptable (maptable.f90:150-172) and loadpksc
! (pksc.f90:22-90), and sums the ranks' maps with MPI_Allreduce (pks2map.f90:313-314).
! With this module the host either
!   (a) replaces the halo loop (pks2map.f90:134-303) by one p2m_paint_records call on the
!       catalogue as read, or
!   (b) keeps its loop and replaces the two projecthalo calls by p2m_project_halo, whose
!       by-reference arguments are those of the projecthalo routines,
! and reads the maps with p2m_get_healpix / p2m_get_flatsky.  Every function returns a
! status (P2M_OK = 0); p2m_last_error gives the message.
!
! The derived types mirror the C structs field for field (bind(C) types take the C
! layout, padding included); tests/test_fortran_iface.py checks the field order and kinds
! and every interface's name, argument count and passing against the C headers.
module p2m_iface
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: P2M_MAXMAPS = 8
  integer(c_int), parameter :: P2M_MAXCONES = 4096

  integer(c_int), parameter :: P2M_OK = 0, P2M_ERR_BADARG = 1, P2M_ERR_CUDA = 2, &
                               P2M_ERR_CAPACITY = 3, P2M_ERR_TIMEOUT = 4, P2M_ERR_IO = 5, &
                               P2M_ERR_STATE = 6, P2M_ERR_NOMEM = 7

  integer(c_int), parameter :: P2M_PREC_FP64 = 0, P2M_PREC_MIXED = 1, &
                               P2M_PREC_MIXED_F64 = 2, P2M_PREC_FIXED = 3

  integer(c_int), parameter :: P2M_LAYOUT_7 = 7, P2M_LAYOUT_10 = 10

  integer(c_int), parameter :: P2M_FLAG_RECORD_SETS = 1, P2M_FLAG_ALL_HALOS = 2, &
                               P2M_FLAG_TIMING = 4, P2M_FLAG_VALIDATE = 8

  ! p2m_config of include/p2m.h: the pks2map command-line parameters (pks2map.f90:62-82)
  ! plus the painter's own fields
  type, bind(C) :: p2m_config
     integer(c_int)       :: nside
     integer(c_int)       :: npix_fs
     real(c_float)        :: fov_deg
     real(c_float)        :: zmin
     real(c_float)        :: zmax
     real(c_float)        :: chihview
     integer(c_int)       :: model
     integer(c_int)       :: precision
     integer(c_int)       :: nmaps
     integer(c_int)       :: map_table(P2M_MAXMAPS)
     integer(c_int)       :: map_profile(P2M_MAXMAPS)
     integer(c_long_long) :: max_records
     integer(c_int)       :: device
     integer(c_int)       :: flags
     integer(c_int)       :: ncones
  end type p2m_config

  ! p2m_stats of include/p2m.h: counters and map sums since the last reset
  type, bind(C) :: p2m_stats
     integer(c_long_long) :: n_records
     integer(c_long_long) :: n_shell
     integer(c_long_long) :: n_painted
     integer(c_long_long) :: n_enumerated
     integer(c_long_long) :: hp_candidates
     integer(c_long_long) :: hp_updates
     integer(c_long_long) :: fs_updates
     integer(c_long_long) :: n_recheck
     integer(c_long_long) :: val_checked
     integer(c_long_long) :: val_bad_set
     integer(c_long_long) :: val_bad_index
     real(c_float)        :: val_max_du
     real(c_double)       :: hp_sum(P2M_MAXMAPS)
     real(c_double)       :: fs_sum(P2M_MAXMAPS)
  end type p2m_stats

  ! p2m_map_stats of include/p2m.h: moments and RMS of one map (pks2map.f90:321-334)
  type, bind(C) :: p2m_map_stats
     integer(c_long_long) :: npix
     real(c_double)       :: mom(3)
     real(c_double)       :: rms
  end type p2m_map_stats

  interface
     integer(c_int) function p2m_create(cfg, ctx) bind(C, name="p2m_create")
       import :: c_int, c_ptr, p2m_config
       type(p2m_config), intent(in) :: cfg
       type(c_ptr), intent(out)     :: ctx
     end function p2m_create

     subroutine p2m_destroy(ctx) bind(C, name="p2m_destroy")
       import :: c_ptr
       type(c_ptr), value :: ctx
     end subroutine p2m_destroy

     ! C string owned by the context (convert with c_f_pointer)
     type(c_ptr) function p2m_last_error(ctx) bind(C, name="p2m_last_error")
       import :: c_ptr
       type(c_ptr), value :: ctx
     end function p2m_last_error

     ! loadmaptable (maptable.f90:150-172): the table file's bytes
     integer(c_int) function p2m_load_table(ctx, slot, image, nbytes) &
          bind(C, name="p2m_load_table")
       import :: c_int, c_ptr, c_long_long
       type(c_ptr), value          :: ctx
       integer(c_int), value       :: slot
       type(c_ptr), value          :: image
       integer(c_long_long), value :: nbytes
     end function p2m_load_table

     ! set_rofztable / set_zofrtable (cosmology.f90:51-105): n = 10000 values each
     integer(c_int) function p2m_set_cosmology_tables(ctx, rofz, zofr, n, rofz_zmax, &
          zofr_rmax) bind(C, name="p2m_set_cosmology_tables")
       import :: c_int, c_ptr, c_float
       type(c_ptr), value         :: ctx
       real(c_float), intent(in)  :: rofz(*), zofr(*)
       integer(c_int), value      :: n
       real(c_float), value       :: rofz_zmax, zofr_rmax
     end function p2m_set_cosmology_tables

     ! `fsmapl = 0; hpmapl = 0` (pks2map.f90:278-279)
     integer(c_int) function p2m_reset_maps(ctx) bind(C, name="p2m_reset_maps")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function p2m_reset_maps

     ! the scramble and center flags (pks2map.f90:75-76, :162-262)
     integer(c_int) function p2m_set_preprocess(ctx, scramble, centre, ntasks) &
          bind(C, name="p2m_set_preprocess")
       import :: c_int, c_ptr
       type(c_ptr), value    :: ctx
       integer(c_int), value :: scramble, centre, ntasks
     end function p2m_set_preprocess

     ! the halo loop (pks2map.f90:134-303) over nrec records of nfloat = 7 or 10 floats,
     ! header removed (pksc.f90:46-66)
     integer(c_int) function p2m_paint_records(ctx, records, nrec, nfloat) &
          bind(C, name="p2m_paint_records")
       import :: c_int, c_ptr, c_long_long, c_float
       type(c_ptr), value          :: ctx
       real(c_float), intent(in)   :: records(*)
       integer(c_long_long), value :: nrec
       integer(c_int), value       :: nfloat
     end function p2m_paint_records

     ! page-locked host memory for the records (c_f_pointer gives the Fortran array);
     ! p2m_paint_records copies from it without the driver's staging
     integer(c_int) function p2m_host_alloc(bytes, ptr) bind(C, name="p2m_host_alloc")
       import :: c_int, c_ptr, c_long_long
       integer(c_long_long), value :: bytes
       type(c_ptr), intent(out)    :: ptr
     end function p2m_host_alloc

     integer(c_int) function p2m_host_free(ptr) bind(C, name="p2m_host_free")
       import :: c_int, c_ptr
       type(c_ptr), value :: ptr
     end function p2m_host_free

     ! projecthalo_flatsky + projecthalo_healpix (haloproject.f90:38,83) with their
     ! by-reference arguments; x, y, z come back divided by chi
     integer(c_int) function p2m_project_halo(ctx, x, y, z, r, chi, m, redshift, v, &
          profile) bind(C, name="p2m_project_halo")
       import :: c_int, c_ptr, c_float
       type(c_ptr), value           :: ctx
       real(c_float), intent(inout) :: x, y, z
       real(c_float), intent(in)    :: r, chi, m, redshift, v
       integer(c_int), intent(in)   :: profile
     end function p2m_project_halo

     integer(c_int) function p2m_flush(ctx) bind(C, name="p2m_flush")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function p2m_flush

     ! ensemble form: cone c owns records offsets(c+1)+1 .. offsets(c+2) (0-based offsets)
     integer(c_int) function p2m_paint_ensemble(ctx, records, offsets, ncones, nfloat) &
          bind(C, name="p2m_paint_ensemble")
       import :: c_int, c_ptr, c_float, c_long_long
       type(c_ptr), value               :: ctx
       real(c_float), intent(in)        :: records(*)
       integer(c_long_long), intent(in) :: offsets(*)
       integer(c_int), value            :: ncones, nfloat
     end function p2m_paint_ensemble

     ! the summed maps (MPI_Allreduce, pks2map.f90:313-314): 12 nside^2 floats in RING
     ! order, or npix_fs^2 floats with j (theta) fastest
     integer(c_int) function p2m_get_healpix(ctx, map, out) bind(C, name="p2m_get_healpix")
       import :: c_int, c_ptr, c_float
       type(c_ptr), value         :: ctx
       integer(c_int), value      :: map
       real(c_float), intent(out) :: out(*)
     end function p2m_get_healpix

     integer(c_int) function p2m_get_flatsky(ctx, map, out) bind(C, name="p2m_get_flatsky")
       import :: c_int, c_ptr, c_float
       type(c_ptr), value         :: ctx
       integer(c_int), value      :: map
       real(c_float), intent(out) :: out(*)
     end function p2m_get_flatsky

     integer(c_int) function p2m_get_healpix_cone(ctx, cone, map, out) &
          bind(C, name="p2m_get_healpix_cone")
       import :: c_int, c_ptr, c_float
       type(c_ptr), value         :: ctx
       integer(c_int), value      :: cone, map
       real(c_float), intent(out) :: out(*)
     end function p2m_get_healpix_cone

     ! halo counts and map totals (pks2map.f90:310,321-327)
     integer(c_int) function p2m_get_stats(ctx, stats) bind(C, name="p2m_get_stats")
       import :: c_int, c_ptr, p2m_stats
       type(c_ptr), value           :: ctx
       type(p2m_stats), intent(out) :: stats
     end function p2m_get_stats

     ! moments, RMS and the cumulative P(<y) (10000 values) of pks2map.f90:321-357,
     ! computed on the device
     integer(c_int) function p2m_get_healpix_stats(ctx, map, stats, dpdy) &
          bind(C, name="p2m_get_healpix_stats")
       import :: c_int, c_ptr, c_float, p2m_map_stats
       type(c_ptr), value               :: ctx
       integer(c_int), value            :: map
       type(p2m_map_stats), intent(out) :: stats
       real(c_float), intent(out)       :: dpdy(*)
     end function p2m_get_healpix_stats

     integer(c_int) function p2m_get_flatsky_stats(ctx, map, stats) &
          bind(C, name="p2m_get_flatsky_stats")
       import :: c_int, c_ptr, p2m_map_stats
       type(c_ptr), value               :: ctx
       integer(c_int), value            :: map
       type(p2m_map_stats), intent(out) :: stats
     end function p2m_get_flatsky_stats

     ! output_map of the HEALPix map to a FITS file (pks2map.f90:381-385) from the device;
     ! path is a NUL-terminated string (trim(name)//c_null_char)
     integer(c_int) function p2m_write_healpix_fits_device(ctx, map, path) &
          bind(C, name="p2m_write_healpix_fits_device")
       import :: c_int, c_ptr, c_char
       type(c_ptr), value                 :: ctx
       integer(c_int), value              :: map
       character(kind=c_char), intent(in) :: path(*)
     end function p2m_write_healpix_fits_device

     integer(c_int) function p2m_synchronize(ctx) bind(C, name="p2m_synchronize")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function p2m_synchronize

     ! the dP/dy histogram of pks2map.f90:338-357 (10000 bins of 1e-8, cumulated)
     integer(c_int) function p2m_dpdy(map, npix, dpdy) bind(C, name="p2m_dpdy")
       import :: c_int, c_float, c_long_long
       real(c_float), intent(in)   :: map(*)
       integer(c_long_long), value :: npix
       real(c_float), intent(out)  :: dpdy(*)
     end function p2m_dpdy

     ! angular power spectra of two RING maps, l = 0..lmax (validation)
     integer(c_int) function p2m_cl_healpix(device, map_a, map_b, nside, lmax, cl_aa, &
          cl_ab, cl_bb) bind(C, name="p2m_cl_healpix")
       import :: c_int, c_float, c_double
       integer(c_int), value       :: device, nside, lmax
       real(c_float), intent(in)   :: map_a(*), map_b(*)
       real(c_double), intent(out) :: cl_aa(*), cl_ab(*), cl_bb(*)
     end function p2m_cl_healpix
  end interface
end module p2m_iface
