/* Minimal stand-in for <hdf5.h>: the typedefs trace_h5io.h uses in its
 * declarations. The HDF5 reader/writer itself is never compiled. */
#ifndef ORACLE_REF_STUB_HDF5_H
#define ORACLE_REF_STUB_HDF5_H
#include "mpi.h"
typedef unsigned long long hsize_t;
typedef long long hid_t;
typedef int herr_t;
typedef enum { H5FD_MPIO_INDEPENDENT = 0, H5FD_MPIO_COLLECTIVE = 1 } H5FD_mpio_xfer_t;
#endif
