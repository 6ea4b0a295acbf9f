// pd_dropin.h -- C++ drop-in with the reference's own names and signatures.
//
// A program written against EricYJA/2D_PD_GPU's sequential / GPU surface
// (include/SetupParticleSystem.h, the mechanics functions of
// src/main_seq.cpp, include/mechanics.cuh, include/util.h) compiles against
// this header instead and links libpd_dropin.so (+ libpd_gb300.so).  The
// setup and bookkeeping functions keep the reference's host semantics; the
// hot path -- computeVelocity / compute_velocity_GPU_host and findNeighbor
// -- runs on the GPU through the C ABI of pd_gb300.h.  Device state is kept
// resident between calls in a context cached per particle vector (the
// reference re-allocates and re-uploads everything on every call,
// include/mechanics.cuh:963-1135).
//
// MPI/ParMETIS declarations of SetupParticleSystem.h (:28-38) are omitted:
// the drop-in is single-GPU, single-process.
#pragma once
#include <set>
#include <string>
#include <unordered_map>
#include <vector>

#include "pd_gb300.h"

using namespace std;  // as the reference headers (include/SetupParticleSystem.h:9)

#ifndef PD_DROPIN_HAVE_PARTICLE
#define PD_DROPIN_HAVE_PARTICLE
// Same members and order as include/SetupParticleSystem.h:11-22.
struct Particle {
  int globalID;
  int partitionID;
  long double volume;
  double damageStatus;
  vector<long double> initialPositions;
  vector<long double> currentPositions;
  vector<int> neighbors;
  set<int> nneighbors;
};
#endif

#ifndef MATRIX_H
#define MATRIX_H
// Same data members and methods as include/matrix.h:7-26 (the reference's
// include guard is reused, so a program that already includes the
// reference's matrix.h keeps its own definition).
class matrix {
 public:
  int ndim;
  vector<vector<long double>> elements;
  matrix();
  matrix(int ndim, const vector<long double>& values);
  matrix matrixAdd(const matrix& M);
  matrix matrixSub(const matrix& M);
  matrix timeScalar(long double constant);
  vector<long double> timeVector(const vector<long double>& V);
  matrix timeMatrix(const matrix& M);
  matrix transpose();
  matrix inverse2D();
  matrix inverse3D();
};
#endif

// ---- setup (include/SetupParticleSystem.h:24-46)
vector<Particle> computeInitialPositions(int numParticlesRow, long double dx, int ndim, vector<long double>& boxlimit);
vector<Particle> readMeshFile(vector<long double>& boxlimit, long double& dx);
void defineParticleIDmap(const vector<Particle>& localParticles, unordered_map<int, int>& globalLocalIDmap);
// GPU cell list; same families (cutoff 1.01*dx*horizon, ascending ids) and
// 2-hop sets as src/SetupParticleSystem.cpp:100-136.
void findNeighbor(vector<Particle>& globalParticles, long double dx, long double horizon, int ndim);
void defineBoundarySet(int ndim, long double dx, const vector<long double>& boxlimit, vector<set<int>>& boundarySet,
                       const vector<Particle> localParticles);
void outputLocalParticlesPositions(int rank, const vector<Particle>& localParticles, int ndim, int step);

// ---- util (include/util.h:20-39)
void storeVelocity(int ndim, std::vector<std::vector<long double>>& particles, const std::string& filename);

// ---- mechanics (src/main_seq.cpp:15-470, include/mechanics.cuh:867-881)
void applyDispBC(int ndim, vector<int>& boundarySet, vector<long double>& dispBC, vector<Particle>& localParticles,
                 vector<vector<long double>>& velocity, vector<vector<long double>>& acce);
void applyVelocityBC(int ndim, vector<int>& boundarySet, vector<long double> v0, vector<vector<long double>>& velocity,
                     vector<vector<long double>>& acce);
void applyFixedBC(int ndim, vector<int>& boundarySet, vector<Particle>& localParticles);
void buildLocalNeighborlist(int ndim, double dx, double horizon, vector<Particle>& localParticles,
                            const unordered_map<int, int>& globalLocalIDmap, vector<vector<Particle*>>& Neighborslist);
matrix getStiffnessTensor(int ndim, double E, double nv);
void updatePositions(int ndim, vector<Particle>& localParticles, long double stepSize, long double massDensity,
                     vector<vector<long double>>& velocity, vector<vector<long double>>& acce,
                     vector<vector<long double>>& netF);
// The hot path: net force and velocity-Verlet kick on the GPU (FP64).
// n1 = n2 = 0 selects the classic model; other weights the reference's
// bond-associated model (per-bond shape tensors, weight length
// horizon * dx).  acce is left as given (the reference CPU semantics,
// src/main_seq.cpp:463-466).
void computeVelocity(int ndim, double n1, double n2, double horizon, double dx, long double massDensity,
                     matrix& StiffnessTensor, long double stepSize, vector<vector<long double>>& velocity,
                     vector<vector<Particle*>>& Neighborslist, vector<vector<long double>>& acce,
                     vector<vector<long double>>& netF, vector<Particle>& localParticles,
                     const unordered_map<int, int>& globalLocalIDmap, vector<vector<double>>& bondDamage);
// Same, with the reference GPU wrapper's semantics: acce := netF / massDensity
// on return (include/mechanics.cuh:854-864).
void compute_velocity_GPU_host(int ndim, double n1, double n2, double horizon, double dx, double massDensity,
                               matrix& StiffnessTensor, double stepSize, vector<vector<long double>>& velocity,
                               vector<vector<Particle*>>& Neighborslist, vector<vector<long double>>& acce,
                               vector<vector<long double>>& netF, vector<Particle>& allParticles,
                               const unordered_map<int, int>& globalLocalIDmap, vector<vector<double>>& bondDamage);

// The reference's Mazars damage (src/main_seq.cpp:473-598) on the GPU
// (pd_mazars_*): from the particles' current positions, updates the per-bond
// thresholds and damage in place and sets each Particle::damageStatus.  The
// tensile / compressive strain parts start at zero (the reference leaves
// them uninitialised).
void computeDamageStatus(int ndim, double n1, double n2, double dx, double horizon,
                         vector<vector<double>>& bondDamageThreshold, vector<Particle>& localParticles,
                         const vector<vector<Particle*>>& Neighborslist, vector<vector<double>>& bondDamage,
                         const unordered_map<int, int>& globalLocalIDmap);

// ---- drop-in controls (no reference counterpart)
// Critical stretch for the GPU contexts the drop-in creates (default 0: no
// bond breaking, as the reference).  Broken bonds then persist across calls,
// and pd_dropin_damage() reports broken / family per particle.
void pd_dropin_set_critical_stretch(double s_c);
void pd_dropin_damage(const vector<Particle>& localParticles, vector<double>& damage);
// Releases the cached device contexts.
void pd_dropin_release();
