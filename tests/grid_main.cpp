// Test driver: the drop-in's computeInitialPositions (include/pd_dropin.h),
// dumped in the format of the reference harness's `grid` mode
// (oracle/ref_harness.cpp): int32 n, int32 ndim, boxlimit[2 ndim], then per
// particle int32 globalID, int32 partitionID, initialPositions[ndim],
// currentPositions[ndim], volume, each long double v as the two doubles
// hi = (double)v, lo = (double)(v - hi).
//
// Usage: grid_main <numParticlesRow> <dx> <ndim> <out.bin>
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "pd_dropin.h"

int main(int argc, char** argv) {
  if (argc != 5) return 2;
  const int rows = std::atoi(argv[1]), ndim = std::atoi(argv[3]);
  const long double dx = std::strtold(argv[2], nullptr);
  vector<long double> boxlimit(2 * ndim);
  vector<Particle> P = computeInitialPositions(rows, dx, ndim, boxlimit);
  FILE* fo = std::fopen(argv[4], "wb");
  if (!fo) return 2;
  auto i32 = [&](int32_t v) { std::fwrite(&v, sizeof v, 1, fo); };
  auto ld = [&](long double v) {
    const double hi = (double)v, lo = (double)(v - (long double)hi);
    std::fwrite(&hi, sizeof hi, 1, fo);
    std::fwrite(&lo, sizeof lo, 1, fo);
  };
  i32((int32_t)P.size());
  i32(ndim);
  for (long double b : boxlimit) ld(b);
  for (const auto& p : P) {
    i32(p.globalID);
    i32(p.partitionID);
    for (int d = 0; d < ndim; ++d) ld(p.initialPositions[d]);
    for (int d = 0; d < ndim; ++d) ld(p.currentPositions[d]);
    ld(p.volume);
  }
  std::fclose(fo);
  return 0;
}
