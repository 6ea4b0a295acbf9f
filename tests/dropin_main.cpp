// Test driver for the C++ drop-in (include/pd_dropin.h): the reference's
// sequential main (src/main_seq.cpp:601-715) written against the drop-in's
// functions, classic weights (n1 = n2 = 0), with the step loop run
// `nsteps` times instead of breaking after one step.  Reads
// 2D_Hassa_test_mesh.dat from the working directory and writes
//   output/velocity_step_0_after_seq_ref.txt    (storeVelocity, after step 1)
//   output/LocalParticlesPositions_rank_0step_0.txt
//   dropin_state.bin: per step int32 step, then u, v, netF as n x 2 doubles
// Usage: dropin_main <nsteps> <gpu-wrapper 0/1> [n1 n2]
//        dropin_main mazars <n1>: the reference's Mazars damage
//        (computeDamageStatus) at the two imposed displacement fields of the
//        reference fixture (same field as oracle/ref_harness.cpp), writing
//        dropin_mazars.bin: per level thresholds, bond damage (family order)
//        and damageStatus as doubles.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <sys/stat.h>

#include "pd_dropin.h"

static int mazars_main(double n1) {
  vector<Particle> P;
  long double dx = 1.0, horizon = 3.0;
  vector<long double> boxlimit(4);
  P = readMeshFile(boxlimit, dx);
  findNeighbor(P, dx, horizon, 2);
  for (auto& p : P) p.partitionID = 0;
  const int n = (int)P.size();
  unordered_map<int, int> g2l;
  defineParticleIDmap(P, g2l);
  vector<vector<Particle*>> NL;
  buildLocalNeighborlist(2, (double)dx, (double)horizon, P, g2l, NL);
  const long double E = 3.5e4, tensileStrength = 3.0;
  const long double damageThreshold = tensileStrength / E;
  vector<vector<double>> bondDamage(n + 1), thr(n);
  for (int i = 0; i < n; ++i) {
    thr[i].resize(NL[i].size(), damageThreshold);
    bondDamage[i].resize(NL[i].size(), 0.0);
  }
  bondDamage[n].resize(30, 0.0);
  FILE* fo = fopen("dropin_mazars.bin", "wb");
  for (int level = 1; level <= 2; ++level) {
    const long double e = level == 1 ? 1.0e-4L : 1.4e-4L, a = 4.0e-4L, ph = level == 1 ? 0.0L : 1.3L;
    for (auto& p : P) {
      const long double X = p.initialPositions[0], Y = p.initialPositions[1];
      p.currentPositions[0] = X + e * (X + 0.3L * Y) + a * sinl(0.23L * X + 0.11L * Y + ph);
      p.currentPositions[1] = Y + (-0.4L * e * Y + a * cosl(0.19L * Y - 0.07L * X + ph));
    }
    computeDamageStatus(2, n1, n1, (double)dx, (double)horizon, thr, P, NL, bondDamage, g2l);
    for (int i = 0; i < n; ++i) fwrite(thr[i].data(), sizeof(double), thr[i].size(), fo);
    for (int i = 0; i < n; ++i) fwrite(bondDamage[i].data(), sizeof(double), NL[i].size(), fo);
    for (const auto& p : P) fwrite(&p.damageStatus, sizeof(double), 1, fo);
  }
  fclose(fo);
  pd_dropin_release();
  std::cout << "dropin mazars ok " << n << " particles" << std::endl;
  return 0;
}

int main(int argc, char** argv) {
  if (argc > 2 && std::strcmp(argv[1], "mazars") == 0) return mazars_main(atof(argv[2]));
  const int nsteps = argc > 1 ? atoi(argv[1]) : 1;
  const bool gpu_wrapper = argc > 2 && atoi(argv[2]) != 0;
  vector<Particle> allParticles;
  int ndim = 2;
  long double dx = 1.0, horizon = 3.0;
  double n1 = argc > 3 ? atof(argv[3]) : 0.0, n2 = argc > 4 ? atof(argv[4]) : 0.0;
  vector<long double> boxlimit(2 * ndim);
  allParticles = readMeshFile(boxlimit, dx);
  findNeighbor(allParticles, dx, horizon, ndim);
  for (auto& p : allParticles) p.partitionID = 0;
  const int n = (int)allParticles.size();
  unordered_map<int, int> globalLocalIDmap;
  defineParticleIDmap(allParticles, globalLocalIDmap);
  vector<set<int>> boundarySet(2 * ndim);
  defineBoundarySet(ndim, dx, boxlimit, boundarySet, allParticles);
  vector<vector<long double>> netF(n, vector<long double>(ndim, 0.0)), velocity(n, vector<long double>(ndim, 0.0)),
      acce(n, vector<long double>(ndim, 0.0));
  vector<int> boundaryBottom(boundarySet[2].begin(), boundarySet[2].end());
  vector<int> boundaryTop(boundarySet[3].begin(), boundarySet[3].end());
  vector<vector<Particle*>> Neighborslist;
  vector<vector<double>> bondDamage(n + 1);
  vector<long double> vt = {0.0, 5.0};
  long double stepSize = 1.0e-9, massDensity = 2.5e-6;
  long double E = 3.5e4, nv = 0.2;
  matrix StiffnessTensor = getStiffnessTensor(ndim, E, nv);
  buildLocalNeighborlist(ndim, dx, horizon, allParticles, globalLocalIDmap, Neighborslist);
  for (int i = 0; i < n; ++i) bondDamage[i].resize(Neighborslist[i].size(), 0.0);
  mkdir("output", 0755);
  FILE* fo = fopen("dropin_state.bin", "wb");
  fwrite(&n, sizeof(int), 1, fo);
  for (int j = 0; j < nsteps; ++j) {
    if (!boundaryTop.empty()) applyVelocityBC(ndim, boundaryTop, vt, velocity, acce);
    updatePositions(ndim, allParticles, stepSize, massDensity, velocity, acce, netF);
    applyFixedBC(ndim, boundaryBottom, allParticles);
    if (gpu_wrapper)
      compute_velocity_GPU_host(ndim, n1, n2, (double)horizon, (double)dx, (double)massDensity, StiffnessTensor,
                                (double)stepSize, velocity, Neighborslist, acce, netF, allParticles, globalLocalIDmap,
                                bondDamage);
    else
      computeVelocity(ndim, n1, n2, (double)horizon, (double)dx, massDensity, StiffnessTensor, stepSize, velocity,
                      Neighborslist, acce, netF, allParticles, globalLocalIDmap, bondDamage);
    if (j == 0) {
      storeVelocity(ndim, velocity, "./output/velocity_step_0_after_seq_ref.txt");
      outputLocalParticlesPositions(0, allParticles, ndim, j);
    }
    const int32_t s = j + 1;
    fwrite(&s, sizeof(s), 1, fo);
    for (const auto& p : allParticles)
      for (int m = 0; m < 2; ++m) {
        const double u = (double)(p.currentPositions[m] - p.initialPositions[m]);
        fwrite(&u, sizeof(u), 1, fo);
      }
    for (const auto& r : velocity)
      for (int m = 0; m < 2; ++m) {
        const double v = (double)r[m];
        fwrite(&v, sizeof(v), 1, fo);
      }
    for (const auto& r : netF)
      for (int m = 0; m < 2; ++m) {
        const double f = (double)r[m];
        fwrite(&f, sizeof(f), 1, fo);
      }
  }
  fclose(fo);
  pd_dropin_release();
  std::cout << "dropin ok " << n << " particles" << std::endl;
  return 0;
}
