/* Project-written stand-in for <mpi.h>, used ONLY to compile the reference's
 * sequential sources (src/main_seq.cpp, src/SetupParticleSystem.cpp) into the
 * test oracle under oracle/_ref.  The sequential path never calls MPI; every
 * stub aborts so an accidental call cannot go unnoticed. */
#pragma once
#include <cstdio>
#include <cstdlib>
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
#define MPI_COMM_WORLD ((MPI_Comm)0)
#define MPI_INT ((MPI_Datatype)1)
#define MPI_LONG_DOUBLE ((MPI_Datatype)2)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
static inline int pdref_mpi_unavailable(const char* fn) {
  std::fprintf(stderr, "oracle/_ref: %s called, but the sequential oracle has no MPI\n", fn);
  std::abort();
  return 1;
}
#define PDREF_MPI_STUB(name) static inline int name(...) { return pdref_mpi_unavailable(#name); }
PDREF_MPI_STUB(MPI_Init)
PDREF_MPI_STUB(MPI_Finalize)
PDREF_MPI_STUB(MPI_Comm_rank)
PDREF_MPI_STUB(MPI_Comm_size)
PDREF_MPI_STUB(MPI_Barrier)
PDREF_MPI_STUB(MPI_Bcast)
PDREF_MPI_STUB(MPI_Gather)
PDREF_MPI_STUB(MPI_Gatherv)
PDREF_MPI_STUB(MPI_Scatter)
PDREF_MPI_STUB(MPI_Scatterv)
PDREF_MPI_STUB(MPI_Send)
PDREF_MPI_STUB(MPI_Recv)
PDREF_MPI_STUB(MPI_Sendrecv)
PDREF_MPI_STUB(MPI_Wtime)
#undef PDREF_MPI_STUB
