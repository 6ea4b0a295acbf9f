// Timing driver for the reference's own published problem: the Hassa mesh
// (2D_Hassa_test_mesh.dat in the working directory) with the reference GPU
// main's parameters and call sequence (src/main.cu:533-648): readMeshFile,
// findNeighbor, defineParticleIDmap, defineBoundarySet, getStiffnessTensor,
// buildLocalNeighborlist, then per step applyVelocityBC -> updatePositions
// -> applyFixedBC -> compute_velocity_GPU_host, the last timed with
// std::chrono around the call as the reference times it
// (src/main.cu:627-637; its published figure is output/gpu_output.txt:9).
// Here the call goes to the GB300 drop-in (include/pd_dropin.h).
//
// Second, the same problem as a device-resident context through the C ABI:
// pd_step_timed(1) (drift, pass A, pass B on the device; CUDA events).
//
// Usage: pd_hassa_timing <n1> <n2> <calls>
// Prints one JSON line: particles, bonds, the first call's seconds (it
// creates the device context and uploads the problem), the median and best
// of the following calls, and the device-only step time.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "pd_dropin.h"
#include "pd_gb300.h"

static void die(const char* what, int rc, pd_ctx* ctx) {
  std::fprintf(stderr, "%s failed (%d): %s\n", what, rc, ctx ? pd_last_error(ctx) : "");
  std::exit(1);
}

int main(int argc, char** argv) {
  const double n1 = argc > 1 ? std::atof(argv[1]) : 10.0, n2 = argc > 2 ? std::atof(argv[2]) : 10.0;
  const int calls = std::max(2, argc > 3 ? std::atoi(argv[3]) : 5);
  // src/main.cu:539-560 (the parameters of the reference's GPU main)
  const int ndim = 2;
  long double dx = 1.0, horizon = 3.0;
  vector<long double> boxlimit(2 * ndim);
  vector<Particle> allParticles = readMeshFile(boxlimit, dx);
  findNeighbor(allParticles, dx, horizon, ndim);
  for (auto& p : allParticles) p.partitionID = 0;
  const int n = (int)allParticles.size();
  unordered_map<int, int> globalLocalIDmap;
  defineParticleIDmap(allParticles, globalLocalIDmap);
  vector<set<int>> boundarySet(2 * ndim);
  defineBoundarySet(ndim, dx, boxlimit, boundarySet, allParticles);
  vector<int> boundaryBottom(boundarySet[2].begin(), boundarySet[2].end());
  vector<int> boundaryTop(boundarySet[3].begin(), boundarySet[3].end());
  vector<vector<long double>> netF(n, vector<long double>(ndim, 0.0)), velocity(n, vector<long double>(ndim, 0.0)),
      acce(n, vector<long double>(ndim, 0.0));
  vector<vector<Particle*>> Neighborslist;
  vector<vector<double>> bondDamage(n + 1);
  const vector<long double> vt = {0.0, 5.0};
  const long double stepSize = 1.0e-9, massDensity = 2.5e-6, E = 3.5e4, nv = 0.2;
  matrix StiffnessTensor = getStiffnessTensor(ndim, (double)E, (double)nv);
  buildLocalNeighborlist(ndim, (double)dx, (double)horizon, allParticles, globalLocalIDmap, Neighborslist);
  long bonds = 0;
  for (int i = 0; i < n; ++i) {
    bondDamage[i].resize(Neighborslist[i].size(), 0.0);
    bonds += (long)Neighborslist[i].size();
  }
  std::vector<double> secs;
  for (int j = 0; j < calls; ++j) {
    applyVelocityBC(ndim, boundaryTop, vt, velocity, acce);
    updatePositions(ndim, allParticles, stepSize, massDensity, velocity, acce, netF);
    applyFixedBC(ndim, boundaryBottom, allParticles);
    const auto t0 = std::chrono::high_resolution_clock::now();
    compute_velocity_GPU_host(ndim, n1, n2, (double)horizon, (double)dx, (double)massDensity, StiffnessTensor,
                              (double)stepSize, velocity, Neighborslist, acce, netF, allParticles, globalLocalIDmap,
                              bondDamage);
    const auto t1 = std::chrono::high_resolution_clock::now();
    secs.push_back(std::chrono::duration<double>(t1 - t0).count());
  }
  pd_dropin_release();
  std::vector<double> warm(secs.begin() + 1, secs.end());
  std::sort(warm.begin(), warm.end());

  // the same problem, device-resident, through the C ABI
  pd_params p;
  pd_default_params(&p);
  p.E = (double)E;
  p.nu = (double)nv;
  p.rho = (double)massDensity;
  p.dt = (double)stepSize;
  p.n1 = n1;
  p.n2 = n2;
  p.weight_len = (double)(horizon * dx);
  pd_ctx* ctx = nullptr;
  int rc = pd_create(&p, &ctx);
  if (rc != PD_OK) die("pd_create", rc, ctx);
  std::vector<double> x(2 * (size_t)n), vol((size_t)n);
  for (int i = 0; i < n; ++i) {
    x[2 * i] = (double)allParticles[i].initialPositions[0];
    x[2 * i + 1] = (double)allParticles[i].initialPositions[1];
    vol[i] = (double)allParticles[i].volume;
  }
  if ((rc = pd_set_particles(ctx, n, x.data(), vol.data())) != PD_OK) die("pd_set_particles", rc, ctx);
  if ((rc = pd_build_families(ctx, 1.01 * (double)(dx * horizon), 0, nullptr)) != PD_OK)
    die("pd_build_families", rc, ctx);
  std::vector<uint8_t> group((size_t)n, 0);
  for (int i : boundaryTop) group[i] = 1;
  for (int i : boundaryBottom) group[i] = 2;
  const int32_t kinds[2] = {PD_BC_VELOCITY, PD_BC_FIXED};
  const double vals[4] = {0.0, 5.0, 0.0, 0.0};
  if ((rc = pd_set_bc(ctx, 2, kinds, vals, group.data())) != PD_OK) die("pd_set_bc", rc, ctx);
  float ms = 0.f;
  if ((rc = pd_step_timed(ctx, 3, &ms)) != PD_OK) die("pd_step_timed", rc, ctx);  // warm-up
  std::vector<float> dev;
  for (int r = 0; r < 10; ++r) {
    if ((rc = pd_step_timed(ctx, 1, &ms)) != PD_OK) die("pd_step_timed", rc, ctx);
    dev.push_back(ms);
  }
  std::sort(dev.begin(), dev.end());
  pd_destroy(ctx);
  std::printf(
      "{\"particles\": %d, \"bonds\": %ld, \"n1\": %g, \"n2\": %g, \"calls\": %d, \"first_call_s\": %.6e, "
      "\"median_call_s\": %.6e, \"best_call_s\": %.6e, \"device_step_ms_median\": %.6e, \"device_step_ms_best\": "
      "%.6e}\n",
      n, bonds, n1, n2, calls, secs[0], warm[warm.size() / 2], warm[0], (double)dev[dev.size() / 2], (double)dev[0]);
  return 0;
}
