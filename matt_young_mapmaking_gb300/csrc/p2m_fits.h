/*
 * p2m_fits.h -- the parts of the HEALPix FITS writer (p2m_outputs.cpp) shared by the
 * host writer and the device-map writer (p2m_capi.cu).  Internal.
 */
#ifndef P2M_FITS_H
#define P2M_FITS_H

#include <cstdint>
#include <cstdio>

/* the primary HDU and the BINTABLE header of a RING map of 12 nside^2 floats, as the
   reference's output_map writes them (fits_s_inc.f90:787-960); the big-endian floats
   follow, then p2m_fits_put_padding */
int32_t p2m_fits_put_header(FILE *fp, int32_t nside);
int32_t p2m_fits_put_padding(FILE *fp, int32_t nside);

#endif
