// Drop-in replacement for the reference's include/mechanics.cuh.
//
// Put include/compat ahead of the reference's include directory and the
// reference's GPU driver (src/main.cu, which #includes "mechanics.cuh" after
// SetupParticleSystem.h) compiles unmodified against the GB300 library:
//   nvcc -Iinclude/compat -Iinclude -I<reference>/include src/main.cu \
//        -Lpath/to/_build -lpd_dropin -lpd_gb300
// Particle is then the reference's own struct (same layout as the
// drop-in's), so the drop-in's definition is skipped.
#pragma once
#define PD_DROPIN_HAVE_PARTICLE
#include "pd_dropin.h"
