// Test oracle only: drives the reference's own sequential CPU path.
//
// This harness is linked with the unmodified reference sources
// src/main_seq.cpp (its main renamed with -Dmain=pdref_seq_main),
// src/SetupParticleSystem.cpp and src/matrix.cpp, compiled where they lie by
// oracle/Makefile (target `ref`) into oracle/_ref/.  It calls the reference
// functions in the order of the reference's step loop
// (src/main_seq.cpp:680-715):
//     applyVelocityBC -> updatePositions -> applyFixedBC -> computeVelocity
// and dumps displacements, velocities, net force and acceleration at full
// precision (binary doubles), so that the project's C restatement (oracle/
// pd_oracle.c) and the CUDA path can be checked against the reference itself.
//
// Three input modes:
//   hassa <mesh_dir> <out_dir> <n1> <n2> <nsteps> <out.bin>
//       exactly the reference main (src/main_seq.cpp:601-715): reads
//       2D_Hassa_test_mesh.dat from <mesh_dir>, dx=1, horizon=3, dt=1e-9,
//       rho=2.5e-6, E=3.5e4, nu=0.2, top velocity (0,5), bottom fixed; also
//       writes the reference's own 6-digit golden files under <out_dir>/output/.
//   plate <in.bin> <out.bin>
//       particles, parameters, optional families and BC lists from a binary
//       file written by tests/golden/make_golden.py (format below).
//   mazars <mesh_dir> <n1> <n2> <out.bin>
//       the reference's Mazars damage (computeDamageStatus, src/main_seq.cpp:
//       473-598) on the Hassa mesh, thresholds initialised as the reference
//       main does (tensileStrength / E, :659-673), called on two imposed
//       displacement fields in turn (mazars_field below); dumps u, the bond
//       thresholds, bond damage and damageStatus after each call.
//   grid <numParticlesRow> <dx> <ndim> <out.bin>
//       the reference's computeInitialPositions (src/SetupParticleSystem.cpp:
//       62-98); dumps int32 n, int32 ndim, then boxlimit[2 ndim], and per
//       particle int32 globalID, int32 partitionID, initialPositions[ndim],
//       currentPositions[ndim], volume -- every long double v as two doubles
//       hi = (double)v, lo = (double)(v - hi) (exact for x86's 64-bit
//       extended mantissa).
//
// Never part of the product: only tests/ and the fixture script run it.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <set>
#include <unordered_map>
#include <unistd.h>
#include <sys/stat.h>

#include "matrix.h"
#include "SetupParticleSystem.h"

// Functions defined in the reference's src/main_seq.cpp (external linkage).
void applyVelocityBC(int ndim, vector<int>& boundarySet, vector<long double> v0,
                     vector<vector<long double>>& velocity, vector<vector<long double>>& acce);
void applyFixedBC(int ndim, vector<int>& boundarySet, vector<Particle>& localParticles);
void buildLocalNeighborlist(int ndim, double dx, double horizon, vector<Particle>& localParticles,
                            const unordered_map<int, int>& globalLocalIDmap,
                            vector<vector<Particle*>>& Neighborslist);
matrix getStiffnessTensor(int ndim, double E, double nv);
void updatePositions(int ndim, vector<Particle>& localParticles, long double stepSize,
                     long double massDensity, vector<vector<long double>>& velocity,
                     vector<vector<long double>>& acce, vector<vector<long double>>& netF);
void computeVelocity(int ndim, double n1, double n2, double horizon, double dx,
                     long double massDensity, matrix& StiffnessTensor, long double stepSize,
                     vector<vector<long double>>& velocity, vector<vector<Particle*>>& Neighborslist,
                     vector<vector<long double>>& acce, vector<vector<long double>>& netF,
                     vector<Particle>& localParticles, const unordered_map<int, int>& globalLocalIDmap,
                     vector<vector<double>>& bondDamage);
void storeVelocity(int ndim, std::vector<std::vector<long double>>& particles, const std::string& filename);
void computeDamageStatus(int ndim, double n1, double n2, double dx, double horizon,
                         vector<vector<double>>& bondDamageThreshold, vector<Particle>& localParticles,
                         const vector<vector<Particle*>>& Neighborslist, vector<vector<double>>& bondDamage,
                         const unordered_map<int, int>& globalLocalIDmap);

namespace {

struct Reader {
  FILE* f;
  template <typename T> T get() {
    T v;
    if (fread(&v, sizeof(T), 1, f) != 1) { fprintf(stderr, "ref_harness: truncated input\n"); exit(2); }
    return v;
  }
  template <typename T> void arr(T* p, size_t n) {
    if (n && fread(p, sizeof(T), n, f) != n) { fprintf(stderr, "ref_harness: truncated input\n"); exit(2); }
  }
};

struct Writer {
  FILE* f;
  template <typename T> void put(T v) { fwrite(&v, sizeof(T), 1, f); }
  void vec2(const vector<vector<long double>>& a) {
    for (const auto& r : a) { put<double>((double)r[0]); put<double>((double)r[1]); }
  }
};

// Dump one step: int32 step, then u, v, netF, acce as N x 2 doubles each.
// u = currentPositions - initialPositions is formed in long double before the
// rounding to double, so it keeps the reference's full precision.
void dump_step(Writer& w, int step, const vector<Particle>& P, const vector<vector<long double>>& v,
               const vector<vector<long double>>& f, const vector<vector<long double>>& a) {
  w.put<int32_t>(step);
  for (const auto& p : P)
    for (int m = 0; m < 2; ++m) w.put<double>((double)(p.currentPositions[m] - p.initialPositions[m]));
  w.vec2(v); w.vec2(f); w.vec2(a);
}

void dump_families(Writer& w, const vector<Particle>& P) {
  int64_t nnz = 0;
  for (const auto& p : P) nnz += (int64_t)p.neighbors.size();
  w.put<int64_t>(nnz);
  int64_t off = 0;
  w.put<int64_t>(0);
  for (const auto& p : P) { off += (int64_t)p.neighbors.size(); w.put<int64_t>(off); }
  for (const auto& p : P) for (int j : p.neighbors) w.put<int32_t>(j);
}

// The reference step loop body (src/main_seq.cpp:686-699), generalised to
// several velocity-BC groups (the reference applies one, boundaryTop).
struct Problem {
  int ndim = 2;
  double dx = 1, horizon = 3, n1 = 0, n2 = 0, E = 0, nu = 0, rho = 0, dt = 0;
  vector<Particle> P;
  vector<vector<int>> vbc_idx;
  vector<vector<long double>> vbc_val;
  vector<int> fixed_idx;
};

int run_steps(Problem& pb, int nsteps, int dump_every, Writer& w, bool dump_fam, const vector<double>* v0) {
  const int n = (int)pb.P.size();
  unordered_map<int, int> g2l;
  defineParticleIDmap(pb.P, g2l);
  vector<vector<Particle*>> NL;
  buildLocalNeighborlist(pb.ndim, pb.dx, pb.horizon, pb.P, g2l, NL);
  matrix C = getStiffnessTensor(pb.ndim, pb.E, pb.nu);
  vector<vector<long double>> netF(n, vector<long double>(2, 0.0)), vel(n, vector<long double>(2, 0.0)),
      acce(n, vector<long double>(2, 0.0));
  if (v0)
    for (int i = 0; i < n; ++i) { vel[i][0] = (*v0)[2 * i]; vel[i][1] = (*v0)[2 * i + 1]; }
  vector<vector<double>> bondDamage(n + 1);
  for (int i = 0; i < n; ++i) bondDamage[i].resize(NL[i].size(), 0.0);
  bondDamage[n].resize(30, 0.0);
  if (dump_fam) dump_families(w, pb.P);
  long double stepSize = pb.dt, massDensity = pb.rho;
  for (int s = 0; s < nsteps; ++s) {
    for (size_t g = 0; g < pb.vbc_idx.size(); ++g)
      if (!pb.vbc_idx[g].empty()) applyVelocityBC(pb.ndim, pb.vbc_idx[g], pb.vbc_val[g], vel, acce);
    updatePositions(pb.ndim, pb.P, stepSize, massDensity, vel, acce, netF);
    applyFixedBC(pb.ndim, pb.fixed_idx, pb.P);
    computeVelocity(pb.ndim, pb.n1, pb.n2, pb.horizon, pb.dx, massDensity, C, stepSize, vel, NL, acce, netF,
                    pb.P, g2l, bondDamage);
    if ((s + 1) % dump_every == 0 || s + 1 == nsteps) dump_step(w, s + 1, pb.P, vel, netF, acce);
  }
  return 0;
}

// Imposed displacement field of the Mazars fixture, level 1 or 2 (mm): a
// homogeneous stretch-shear plus a smooth ripple.  Part of the mesh exceeds
// the 3 / 3.5e4 threshold at level 1; level 2 stretches more but shifts the
// ripple, so some bonds unload (their history threshold holds) while others
// load further.
void mazars_field(int level, long double X, long double Y, long double* ux, long double* uy) {
  const long double e = level == 1 ? 1.0e-4L : 1.4e-4L, a = 4.0e-4L, ph = level == 1 ? 0.0L : 1.3L;
  *ux = e * (X + 0.3L * Y) + a * sinl(0.23L * X + 0.11L * Y + ph);
  *uy = -0.4L * e * Y + a * cosl(0.19L * Y - 0.07L * X + ph);
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) { fprintf(stderr, "usage: see header\n"); return 2; }
  std::string mode = argv[1];
  if (mode == "hassa") {
    if (argc != 8) { fprintf(stderr, "hassa <mesh_dir> <out_dir> <n1> <n2> <nsteps> <out.bin>\n"); return 2; }
    const std::string mesh_dir = argv[2], out_dir = argv[3];
    Problem pb;
    pb.n1 = atof(argv[4]); pb.n2 = atof(argv[5]);
    const int nsteps = atoi(argv[6]);
    // Parameters of the reference main (src/main_seq.cpp:607-660).
    long double dx = 1.0, horizon = 3.0;
    vector<long double> boxlimit(4);
    if (chdir(mesh_dir.c_str()) != 0) { perror("chdir mesh_dir"); return 2; }
    pb.P = readMeshFile(boxlimit, dx);
    findNeighbor(pb.P, dx, horizon, 2);
    for (auto& p : pb.P) p.partitionID = 0;
    if (chdir(out_dir.c_str()) != 0) { perror("chdir out_dir"); return 2; }
    mkdir("output", 0755);
    vector<set<int>> bset(4);
    defineBoundarySet(2, dx, boxlimit, bset, pb.P);
    pb.dx = (double)dx; pb.horizon = (double)horizon;
    pb.E = 3.5e4; pb.nu = 0.2; pb.rho = 2.5e-6; pb.dt = 1.0e-9;
    pb.vbc_idx.push_back(vector<int>(bset[3].begin(), bset[3].end()));
    pb.vbc_val.push_back({0.0, 5.0});
    pb.fixed_idx.assign(bset[2].begin(), bset[2].end());
    FILE* fo = fopen(argv[7], "wb");
    if (!fo) { perror("out"); return 2; }
    Writer w{fo};
    w.put<int32_t>((int32_t)pb.P.size());
    for (const auto& p : pb.P) { w.put<double>((double)p.initialPositions[0]); w.put<double>((double)p.initialPositions[1]); w.put<double>((double)p.volume); }
    for (int b = 0; b < 4; ++b) {
      w.put<int32_t>((int32_t)bset[b].size());
      for (int k : bset[b]) w.put<int32_t>(k);
    }
    // Same loop as run_steps but also writes the reference's own golden text
    // files after the first step (src/main_seq.cpp:703, :711).
    const int n = (int)pb.P.size();
    unordered_map<int, int> g2l;
    defineParticleIDmap(pb.P, g2l);
    vector<vector<Particle*>> NL;
    buildLocalNeighborlist(2, pb.dx, pb.horizon, pb.P, g2l, NL);
    matrix C = getStiffnessTensor(2, pb.E, pb.nu);
    vector<vector<long double>> netF(n, vector<long double>(2, 0.0)), vel(n, vector<long double>(2, 0.0)),
        acce(n, vector<long double>(2, 0.0));
    vector<vector<double>> bondDamage(n + 1);
    for (int i = 0; i < n; ++i) bondDamage[i].resize(NL[i].size(), 0.0);
    bondDamage[n].resize(30, 0.0);
    dump_families(w, pb.P);
    long double stepSize = 1.0e-9, massDensity = 2.5e-6;
    for (int s = 0; s < nsteps; ++s) {
      applyVelocityBC(2, pb.vbc_idx[0], pb.vbc_val[0], vel, acce);
      updatePositions(2, pb.P, stepSize, massDensity, vel, acce, netF);
      applyFixedBC(2, pb.fixed_idx, pb.P);
      computeVelocity(2, pb.n1, pb.n2, pb.horizon, pb.dx, massDensity, C, stepSize, vel, NL, acce, netF, pb.P,
                      g2l, bondDamage);
      if (s == 0) {
        storeVelocity(2, vel, "./output/velocity_step_0_after_seq_ref.txt");
        outputLocalParticlesPositions(0, pb.P, 2, 0);
      }
      dump_step(w, s + 1, pb.P, vel, netF, acce);
    }
    fclose(fo);
    return 0;
  }
  if (mode == "grid") {
    if (argc != 6) { fprintf(stderr, "grid <numParticlesRow> <dx> <ndim> <out.bin>\n"); return 2; }
    const int rows = atoi(argv[2]), ndim = atoi(argv[4]);
    const long double dx = strtold(argv[3], nullptr);
    vector<long double> boxlimit(2 * ndim);
    vector<Particle> P = computeInitialPositions(rows, dx, ndim, boxlimit);
    FILE* fo = fopen(argv[5], "wb");
    if (!fo) { perror("out"); return 2; }
    Writer w{fo};
    auto ld = [&](long double v) {
      const double hi = (double)v;
      w.put<double>(hi);
      w.put<double>((double)(v - (long double)hi));
    };
    w.put<int32_t>((int32_t)P.size());
    w.put<int32_t>(ndim);
    for (long double b : boxlimit) ld(b);
    for (const auto& p : P) {
      w.put<int32_t>(p.globalID);
      w.put<int32_t>(p.partitionID);
      for (int d = 0; d < ndim; ++d) ld(p.initialPositions[d]);
      for (int d = 0; d < ndim; ++d) ld(p.currentPositions[d]);
      ld(p.volume);
    }
    fclose(fo);
    return 0;
  }
  if (mode == "plate") {
    if (argc != 4) { fprintf(stderr, "plate <in.bin> <out.bin>\n"); return 2; }
    FILE* fi = fopen(argv[2], "rb");
    if (!fi) { perror("in"); return 2; }
    Reader r{fi};
    // Input format (little-endian):
    //   char[4] "PDRF", int32 version(=1), int32 n, int32 families_from_file,
    //   double dx, horizon, n1, n2, E, nu, rho, dt, int32 nsteps, int32 dump_every,
    //   double x_ref[n][2], double vol[n],
    //   version 2 only: int32 has_state; if has_state: double u0[n][2], v0[n][2]
    //     (initial displacement and velocity; version 1 starts at rest),
    //   if families_from_file: int64 row_ptr[n+1], int32 col[row_ptr[n]],
    //   int32 n_vbc; n_vbc x { int32 cnt, double vx, vy, int32 idx[cnt] },
    //   int32 n_fixed, int32 idx[n_fixed]
    char magic[4];
    r.arr(magic, 4);
    if (memcmp(magic, "PDRF", 4) != 0) { fprintf(stderr, "bad magic\n"); return 2; }
    const int version = r.get<int32_t>();
    if (version != 1 && version != 2) { fprintf(stderr, "bad version\n"); return 2; }
    Problem pb;
    const int n = r.get<int32_t>();
    const int fam_from_file = r.get<int32_t>();
    pb.dx = r.get<double>(); pb.horizon = r.get<double>(); pb.n1 = r.get<double>(); pb.n2 = r.get<double>();
    pb.E = r.get<double>(); pb.nu = r.get<double>(); pb.rho = r.get<double>(); pb.dt = r.get<double>();
    const int nsteps = r.get<int32_t>(), dump_every = r.get<int32_t>();
    vector<double> x(2 * (size_t)n), vol(n);
    r.arr(x.data(), x.size());
    r.arr(vol.data(), vol.size());
    vector<double> u0, v0;
    if (version == 2 && r.get<int32_t>() != 0) {
      u0.resize(2 * (size_t)n);
      v0.resize(2 * (size_t)n);
      r.arr(u0.data(), u0.size());
      r.arr(v0.data(), v0.size());
    }
    pb.P.resize(n);
    for (int i = 0; i < n; ++i) {
      Particle& p = pb.P[i];
      p.globalID = i; p.partitionID = 0; p.damageStatus = 0.0;
      p.volume = vol[i];
      p.initialPositions = {x[2 * i], x[2 * i + 1]};
      p.currentPositions = p.initialPositions;
      if (!u0.empty()) {  // current = reference + u0 in long double, so u = u0 exactly
        p.currentPositions[0] += (long double)u0[2 * i];
        p.currentPositions[1] += (long double)u0[2 * i + 1];
      }
    }
    if (fam_from_file) {
      vector<int64_t> rp(n + 1);
      r.arr(rp.data(), rp.size());
      vector<int32_t> col(rp[n]);
      r.arr(col.data(), col.size());
      for (int i = 0; i < n; ++i) pb.P[i].neighbors.assign(col.begin() + rp[i], col.begin() + rp[i + 1]);
    } else {
      findNeighbor(pb.P, (long double)pb.dx, (long double)pb.horizon, 2);
    }
    const int nv = r.get<int32_t>();
    for (int g = 0; g < nv; ++g) {
      const int cnt = r.get<int32_t>();
      const double vx = r.get<double>(), vy = r.get<double>();
      vector<int> idx(cnt);
      r.arr(idx.data(), idx.size());
      pb.vbc_idx.push_back(idx);
      pb.vbc_val.push_back({vx, vy});
    }
    const int nf = r.get<int32_t>();
    pb.fixed_idx.resize(nf);
    r.arr(pb.fixed_idx.data(), pb.fixed_idx.size());
    fclose(fi);
    FILE* fo = fopen(argv[3], "wb");
    if (!fo) { perror("out"); return 2; }
    Writer w{fo};
    w.put<int32_t>(n);
    run_steps(pb, nsteps, dump_every, w, true, v0.empty() ? nullptr : &v0);
    fclose(fo);
    return 0;
  }
  if (mode == "mazars") {
    if (argc != 6) { fprintf(stderr, "mazars <mesh_dir> <n1> <n2> <out.bin>\n"); return 2; }
    const double n1 = atof(argv[3]), n2 = atof(argv[4]);
    long double dx = 1.0, horizon = 3.0;
    vector<long double> boxlimit(4);
    if (chdir(argv[2]) != 0) { perror("chdir mesh_dir"); return 2; }
    vector<Particle> P = readMeshFile(boxlimit, dx);
    findNeighbor(P, dx, horizon, 2);
    for (auto& p : P) p.partitionID = 0;
    const int n = (int)P.size();
    unordered_map<int, int> g2l;
    defineParticleIDmap(P, g2l);
    vector<vector<Particle*>> NL;
    buildLocalNeighborlist(2, (double)dx, (double)horizon, P, g2l, NL);
    // src/main_seq.cpp:659-676
    const long double E = 3.5e4, tensileStrength = 3.0;
    const long double damageThreshold = tensileStrength / E;
    vector<vector<double>> bondDamage(n + 1), bondDamageThreshold(n);
    for (int i = 0; i < n; ++i) {
      bondDamageThreshold[i].resize(NL[i].size(), damageThreshold);
      bondDamage[i].resize(NL[i].size(), 0.0);
    }
    bondDamage[n].resize(30, 0.0);
    FILE* fo = fopen(argv[5], "wb");
    if (!fo) { perror("out"); return 2; }
    Writer w{fo};
    w.put<int32_t>(n);
    dump_families(w, P);
    for (int level = 1; level <= 2; ++level) {
      for (auto& p : P) {
        long double ux, uy;
        mazars_field(level, p.initialPositions[0], p.initialPositions[1], &ux, &uy);
        p.currentPositions[0] = p.initialPositions[0] + ux;
        p.currentPositions[1] = p.initialPositions[1] + uy;
      }
      computeDamageStatus(2, n1, n2, (double)dx, (double)horizon, bondDamageThreshold, P, NL, bondDamage, g2l);
      w.put<int32_t>(level);
      for (const auto& p : P)
        for (int m = 0; m < 2; ++m) w.put<double>((double)(p.currentPositions[m] - p.initialPositions[m]));
      for (int i = 0; i < n; ++i) for (double t : bondDamageThreshold[i]) w.put<double>(t);
      for (int i = 0; i < n; ++i) for (size_t k = 0; k < NL[i].size(); ++k) w.put<double>(bondDamage[i][k]);
      for (const auto& p : P) w.put<double>(p.damageStatus);
    }
    fclose(fo);
    return 0;
  }
  fprintf(stderr, "unknown mode %s\n", mode.c_str());
  return 2;
}
