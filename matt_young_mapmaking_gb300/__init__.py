"""GB300-native drop-in for Peak Patch's map-making hot path (pks2map).

Halos from a .pksc catalogue are painted as tSZ / kSZ profiles (make_maptable tables)
onto HEALPix (RING) and flat-sky maps by hand-written sm_103a CUDA kernels behind the C
ABI of include/p2m.h.  This package holds the Python binding of that ABI, the file
formats and the build step.
"""
from .capi import (FLAG_ALL_HALOS, FLAG_RECORD_SETS, FLAG_TIMING, FLAG_VALIDATE, MAXMAPS, PHASES,
                   PREC_FIXED, PREC_FP64, PREC_MIXED,
                   P2MConfig, P2MError, Painter, exported_symbols, generate_catalogue,
                   load_library, make_maptable)
from .capi import cl_flatsky, cl_healpix, dpdy, write_outputs
from .formats import (detect_layout, read_dpdy, read_flatsky, read_healpix_fits, read_pksc,
                      read_table, table_array, table_header, write_pksc, write_table)

__all__ = ["FLAG_ALL_HALOS", "FLAG_RECORD_SETS", "FLAG_TIMING", "FLAG_VALIDATE", "PHASES",
           "MAXMAPS", "PREC_FIXED", "PREC_FP64", "PREC_MIXED",
           "P2MConfig", "P2MError", "Painter", "exported_symbols", "generate_catalogue",
           "load_library", "make_maptable", "detect_layout", "read_pksc", "read_table",
           "table_array", "table_header", "write_pksc", "write_table", "dpdy", "write_outputs",
           "cl_healpix", "cl_flatsky",
           "read_dpdy", "read_flatsky", "read_healpix_fits"]
