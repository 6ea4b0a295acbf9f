/* Project-written stand-in for <parmetis.h> (types + one aborting stub) so the
 * reference's include/SetupParticleSystem.h compiles for the sequential oracle. */
#pragma once
#include "mpi.h"
typedef int idx_t;
typedef float real_t;
static inline int ParMETIS_V3_PartKway(...) { return pdref_mpi_unavailable("ParMETIS_V3_PartKway"); }
