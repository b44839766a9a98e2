/* Minimal stand-in for <mpi.h>: just the handle types the reference's
 * tracer/operator headers name in declarations. Nothing here is called. */
#ifndef ORACLE_REF_STUB_MPI_H
#define ORACLE_REF_STUB_MPI_H
typedef int MPI_Comm;
typedef int MPI_Info;
#endif
