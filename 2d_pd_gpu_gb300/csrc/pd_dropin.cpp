// C++ drop-in (include/pd_dropin.h): the reference's function names over the
// C ABI of pd_gb300.h.  Host bookkeeping keeps the reference's semantics
// (cited per function); the force/kick and the family search run on the GPU.
#include "pd_dropin.h"

#include <cmath>
#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>

namespace {

double g_s_c = 0.0;

void check(int rc, pd_ctx* ctx, const char* what) {
  if (rc != PD_OK) throw std::runtime_error(std::string(what) + ": " + pd_last_error(ctx));
}

// Device context for one particle vector, created on first use and kept.
struct Cached {
  pd_ctx* ctx = nullptr;
  const Particle* data = nullptr;
  size_t n = 0;
  double rho = 0.0, dt = 0.0, s_c = 0.0, n1 = 0.0, n2 = 0.0, wlen = 1.0, C[9] = {0};
  double *u = nullptr, *v = nullptr, *a = nullptr, *f = nullptr;  // pinned staging
  ~Cached() {
    pd_host_free(u);
    pd_host_free(v);
    pd_host_free(a);
    pd_host_free(f);
    pd_destroy(ctx);
  }
};

std::map<const vector<Particle>*, std::unique_ptr<Cached>>& cache() {
  static std::map<const vector<Particle>*, std::unique_ptr<Cached>> m;
  return m;
}

Cached& context_for(vector<Particle>& P, const vector<vector<Particle*>>& NL, long double rho, long double dt,
                    const matrix& Cm, double n1, double n2, double wlen) {
  auto& slot = cache()[&P];
  const size_t n = P.size();
  double C[9];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) C[3 * r + c] = (double)Cm.elements.at(r).at(c);
  if (!slot || slot->data != P.data() || slot->n != n) {
    slot.reset(new Cached());
    Cached& k = *slot;
    pd_params p;
    pd_default_params(&p);
    p.rho = (double)rho;
    p.dt = (double)dt;
    p.s_c = g_s_c;
    p.n1 = n1;
    p.n2 = n2;
    p.weight_len = wlen;
    check(pd_create(&p, &k.ctx), nullptr, "pd_create");
    vector<double> x(2 * n), vol(n);
    for (size_t i = 0; i < n; ++i) {
      x[2 * i] = (double)P[i].initialPositions[0];
      x[2 * i + 1] = (double)P[i].initialPositions[1];
      vol[i] = (double)P[i].volume;
    }
    check(pd_set_particles(k.ctx, (int64_t)n, x.data(), vol.data()), k.ctx, "pd_set_particles");
    // families from the caller's neighbour pointers (buildLocalNeighborlist)
    vector<int64_t> rp(n + 1, 0);
    vector<int32_t> col;
    for (size_t i = 0; i < n; ++i) {
      for (const Particle* q : NL.at(i)) col.push_back((int32_t)(q - P.data()));
      rp[i + 1] = (int64_t)col.size();
    }
    check(pd_set_families(k.ctx, rp.data(), col.data()), k.ctx, "pd_set_families");
    void* b;
    for (double** dst : {&k.u, &k.v, &k.a, &k.f}) {
      check(pd_host_alloc((int64_t)(2 * n * sizeof(double)), &b), k.ctx, "pd_host_alloc");
      *dst = static_cast<double*>(b);
    }
    k.data = P.data();
    k.n = n;
    k.rho = p.rho;
    k.dt = p.dt;
    k.s_c = p.s_c;
    k.n1 = n1;
    k.n2 = n2;
    k.wlen = wlen;
    std::copy(C, C + 9, k.C);
    check(pd_set_stiffness(k.ctx, C), k.ctx, "pd_set_stiffness");
  }
  Cached& k = *slot;
  if (k.rho != (double)rho || k.dt != (double)dt || k.s_c != g_s_c || k.n1 != n1 || k.n2 != n2 ||
      k.wlen != wlen || !std::equal(C, C + 9, k.C)) {
    pd_params p;
    check(pd_get_params(k.ctx, &p), k.ctx, "pd_get_params");
    p.rho = (double)rho;
    p.dt = (double)dt;
    p.s_c = g_s_c;
    p.n1 = n1;
    p.n2 = n2;
    p.weight_len = wlen;
    k.n1 = n1;
    k.n2 = n2;
    k.wlen = wlen;
    check(pd_set_params(k.ctx, &p), k.ctx, "pd_set_params");
    check(pd_set_stiffness(k.ctx, C), k.ctx, "pd_set_stiffness");
    k.rho = p.rho;
    k.dt = p.dt;
    k.s_c = p.s_c;
    std::copy(C, C + 9, k.C);
  }
  return k;
}

void gpu_velocity(double n1, double n2, double wlen, long double rho, const matrix& C, long double dt,
                  vector<vector<long double>>& velocity, vector<vector<Particle*>>& NL,
                  vector<vector<long double>>& acce, vector<vector<long double>>& netF, vector<Particle>& P,
                  bool gpu_semantics) {
  Cached& k = context_for(P, NL, rho, dt, C, n1, n2, wlen);
  const size_t n = P.size();
  for (size_t i = 0; i < n; ++i)
    for (int m = 0; m < 2; ++m) {
      // displacement formed in long double before rounding (keeps the
      // precision the absolute long double positions carry)
      k.u[2 * i + m] = (double)(P[i].currentPositions[m] - P[i].initialPositions[m]);
      k.v[2 * i + m] = (double)velocity[i][m];
      k.a[2 * i + m] = (double)acce[i][m];
    }
  check(pd_compute_velocity(k.ctx, k.u, k.v, k.a, k.f), k.ctx, "pd_compute_velocity");
  for (size_t i = 0; i < n; ++i)
    for (int m = 0; m < 2; ++m) {
      velocity[i][m] = k.v[2 * i + m];
      netF[i][m] = k.f[2 * i + m];
      if (gpu_semantics) acce[i][m] = k.a[2 * i + m];
    }
}

}  // namespace

// ------------------------------------------------------------------- matrix

matrix::matrix() : ndim(0) {}

matrix::matrix(int nd, const vector<long double>& values) : ndim(nd), elements(nd, vector<long double>(nd)) {
  for (int r = 0; r < nd; ++r)
    for (int c = 0; c < nd; ++c) elements[r][c] = values[r * nd + c];
}

matrix matrix::matrixAdd(const matrix& M) {
  matrix o(ndim, vector<long double>(ndim * ndim, 0.0));
  for (int r = 0; r < ndim; ++r)
    for (int c = 0; c < ndim; ++c) o.elements[r][c] = elements[r][c] + M.elements[r][c];
  return o;
}

matrix matrix::matrixSub(const matrix& M) {
  matrix o(ndim, vector<long double>(ndim * ndim, 0.0));
  for (int r = 0; r < ndim; ++r)
    for (int c = 0; c < ndim; ++c) o.elements[r][c] = elements[r][c] - M.elements[r][c];
  return o;
}

matrix matrix::timeScalar(long double s) {
  matrix o(ndim, vector<long double>(ndim * ndim, 0.0));
  for (int r = 0; r < ndim; ++r)
    for (int c = 0; c < ndim; ++c) o.elements[r][c] = elements[r][c] * s;
  return o;
}

vector<long double> matrix::timeVector(const vector<long double>& V) {
  vector<long double> o(ndim, 0.0);
  for (int r = 0; r < ndim; ++r)
    for (int c = 0; c < ndim; ++c) o[r] += elements[r][c] * V[c];
  return o;
}

matrix matrix::timeMatrix(const matrix& M) {
  matrix o(ndim, vector<long double>(ndim * ndim, 0.0));
  for (int r = 0; r < ndim; ++r)
    for (int c = 0; c < ndim; ++c)
      for (int k = 0; k < ndim; ++k) o.elements[r][c] += elements[r][k] * M.elements[k][c];
  return o;
}

matrix matrix::transpose() {
  matrix o(ndim, vector<long double>(ndim * ndim, 0.0));
  for (int r = 0; r < ndim; ++r)
    for (int c = 0; c < ndim; ++c) o.elements[c][r] = elements[r][c];
  return o;
}

matrix matrix::inverse2D() {
  matrix o(ndim, vector<long double>(ndim * ndim, 0.0));
  const long double d = elements[0][0] * elements[1][1] - elements[0][1] * elements[1][0];
  o.elements[0][0] = elements[1][1] / d;
  o.elements[0][1] = -elements[0][1] / d;
  o.elements[1][0] = -elements[1][0] / d;
  o.elements[1][1] = elements[0][0] / d;
  return o;
}

matrix matrix::inverse3D() {
  const auto& e = elements;
  const long double c00 = e[1][1] * e[2][2] - e[1][2] * e[2][1];
  const long double c01 = e[1][0] * e[2][2] - e[1][2] * e[2][0];
  const long double c02 = e[1][0] * e[2][1] - e[1][1] * e[2][0];
  const long double d = e[0][0] * c00 - e[0][1] * c01 + e[0][2] * c02;
  matrix o(ndim, vector<long double>(ndim * ndim, 0.0));
  o.elements[0][0] = c00 / d;
  o.elements[0][1] = -(e[0][1] * e[2][2] - e[0][2] * e[2][1]) / d;
  o.elements[0][2] = (e[0][1] * e[1][2] - e[0][2] * e[1][1]) / d;
  o.elements[1][0] = -c01 / d;
  o.elements[1][1] = (e[0][0] * e[2][2] - e[0][2] * e[2][0]) / d;
  o.elements[1][2] = -(e[0][0] * e[1][2] - e[0][2] * e[1][0]) / d;
  o.elements[2][0] = c02 / d;
  o.elements[2][1] = -(e[0][0] * e[2][1] - e[0][1] * e[2][0]) / d;
  o.elements[2][2] = (e[0][0] * e[1][1] - e[0][1] * e[1][0]) / d;
  return o;
}

// -------------------------------------------------------------------- setup

// src/SetupParticleSystem.cpp:62-98 (grid, x fastest, box centred on -floor(n/2) dx)
vector<Particle> computeInitialPositions(int numParticlesRow, long double dx, int ndim, vector<long double>& boxlimit) {
  vector<Particle> out;
  const int total = (int)std::pow(numParticlesRow, ndim);
  vector<long double> lo(ndim);
  for (int d = 0; d < ndim; ++d) {
    lo[d] = -1.0L * std::floor(numParticlesRow / 2) * dx;
    boxlimit[2 * d] = lo[d];
    boxlimit[2 * d + 1] = lo[d] + (numParticlesRow - 1) * dx;
  }
  out.reserve(total);
  for (int i = 0; i < total; ++i) {
    Particle p;
    vector<long double> c(ndim);
    for (int d = 0; d < ndim; ++d) {
      const int k = d == 0 ? i % numParticlesRow : (int)(i / std::pow(numParticlesRow, d));
      c[d] = lo[d] + k * dx;
    }
    p.globalID = i;
    p.partitionID = 0;
    p.damageStatus = 0.0;
    p.volume = std::pow(dx, ndim);
    p.initialPositions = c;
    p.currentPositions = c;
    out.push_back(p);
  }
  return out;
}

// src/SetupParticleSystem.cpp:11-60: the Hassa mesh from the working
// directory, two side notches (|x| > 17.5 and |y| < 2) removed as the pre-crack.
vector<Particle> readMeshFile(vector<long double>& boxlimit, long double& dx) {
  vector<Particle> out;
  std::ifstream in("2D_Hassa_test_mesh.dat");
  if (!in.is_open()) std::cerr << "Error: Could not open the mesh file '2D_Hassa_test_mesh.dat'" << std::endl;
  std::string line;
  std::getline(in, line);
  int id = 0;
  while (std::getline(in, line)) {
    std::istringstream ss(line);
    long double x, y, a;
    if (!(ss >> x >> y >> a)) continue;
    if (std::fabs(x) > 17.5 && std::fabs(y) < 2.0) continue;
    Particle p;
    p.globalID = id++;
    p.partitionID = 0;
    p.damageStatus = 0.0;
    p.initialPositions = {x, y};
    p.currentPositions = {x, y};
    p.volume = a;
    out.push_back(p);
  }
  dx = 1.0;
  boxlimit[0] = -34.5;
  boxlimit[1] = 34.5;
  boxlimit[2] = -29.5;
  boxlimit[3] = 29.5;
  return out;
}

// src/SetupParticleSystem.cpp:504-510
void defineParticleIDmap(const vector<Particle>& P, unordered_map<int, int>& m) {
  m.clear();
  int k = 0;
  for (const auto& p : P) m[p.globalID] = k++;
}

// src/SetupParticleSystem.cpp:100-136, with the O(N^2) pair loop replaced by
// the GPU cell list (pd_build_families).
void findNeighbor(vector<Particle>& G, long double dx, long double horizon, int ndim) {
  if (ndim != 2) throw std::invalid_argument("findNeighbor: the GPU family build is 2-D");
  const size_t n = G.size();
  pd_params p;
  pd_default_params(&p);
  pd_ctx* ctx = nullptr;
  check(pd_create(&p, &ctx), nullptr, "pd_create");
  vector<double> x(2 * n), vol(n);
  for (size_t i = 0; i < n; ++i) {
    x[2 * i] = (double)G[i].initialPositions[0];
    x[2 * i + 1] = (double)G[i].initialPositions[1];
    vol[i] = G[i].volume > 0 ? (double)G[i].volume : 1.0;
  }
  const double cutoff = (double)(1.01L * dx * horizon);
  int rc = pd_set_particles(ctx, (int64_t)n, x.data(), vol.data());
  if (rc == PD_OK) rc = pd_build_families(ctx, cutoff, 0, nullptr);
  int64_t nnz = 0;
  vector<int64_t> rp(n + 1);
  vector<int32_t> col;
  if (rc == PD_OK) rc = pd_num_bonds(ctx, &nnz);
  if (rc == PD_OK) {
    col.resize((size_t)nnz);
    rc = pd_get_families(ctx, rp.data(), col.data());
  }
  if (rc != PD_OK) {
    std::string msg = pd_last_error(ctx);
    pd_destroy(ctx);
    throw std::runtime_error("findNeighbor: " + msg);
  }
  pd_destroy(ctx);
  for (size_t i = 0; i < n; ++i) G[i].neighbors.assign(col.begin() + rp[i], col.begin() + rp[i + 1]);
  for (auto& pi : G) {  // 2-hop sets (used by the reference's ghost exchange)
    pi.nneighbors.clear();
    for (int pj : pi.neighbors) {
      pi.nneighbors.insert(G[pj].neighbors.begin(), G[pj].neighbors.end());
      pi.nneighbors.erase(pj);
    }
    for (int pj : pi.neighbors) pi.nneighbors.erase(pj);
    pi.nneighbors.erase(pi.globalID);
  }
}

// src/SetupParticleSystem.cpp:513-529
void defineBoundarySet(int ndim, long double dx, const vector<long double>& boxlimit, vector<set<int>>& boundarySet,
                       const vector<Particle> P) {
  for (size_t k = 0; k < P.size(); ++k) {
    if (P[k].neighbors.size() > 17) continue;
    for (int d = 0; d < ndim; ++d) {
      const long double c = P[k].initialPositions[d];
      if (c < boxlimit[2 * d] + dx / 2.0)
        boundarySet[2 * d].insert((int)k);
      else if (c > boxlimit[2 * d + 1] - dx / 2.0)
        boundarySet[2 * d + 1].insert((int)k);
    }
  }
}

// src/SetupParticleSystem.cpp:646-658
void outputLocalParticlesPositions(int rank, const vector<Particle>& P, int ndim, int step) {
  std::ofstream o("./output/LocalParticlesPositions_rank_" + std::to_string(rank) + "step_" + std::to_string(step) +
                  ".txt");
  o << "ID, x, y, ux, uy " << std::endl;
  for (const auto& p : P) {
    o << p.globalID << ",";
    for (int d = 0; d < ndim; ++d) o << p.initialPositions[d] << ",";
    o << p.currentPositions[0] - p.initialPositions[0] << ",";
    o << p.currentPositions[1] - p.initialPositions[1] << std::endl;
  }
}

// include/util.h:20-39
void storeVelocity(int ndim, std::vector<std::vector<long double>>& particles, const std::string& filename) {
  std::ofstream o(filename);
  if (!o) {
    std::cerr << "Error opening file: " << filename << std::endl;
    return;
  }
  for (const auto& p : particles) {
    if ((int)p.size() >= ndim) {
      for (int d = 0; d < ndim; ++d) o << p[d] << (d < ndim - 1 ? " " : "");
      o << std::endl;
    } else {
      std::cerr << "Skipping particle with insufficient data.\n";
    }
  }
  std::cout << "Current velocity data stored in " << filename << std::endl;
}

// ---------------------------------------------------------------- mechanics

// src/main_seq.cpp:15-26
void applyDispBC(int ndim, vector<int>& S, vector<long double>& d, vector<Particle>& P,
                 vector<vector<long double>>& velocity, vector<vector<long double>>& acce) {
  for (int pi : S)
    for (int m = 0; m < ndim; ++m) {
      P[pi].currentPositions[m] = P[pi].initialPositions[m] + d[m];
      velocity[pi][m] = 0.0;
      acce[pi][m] = 0.0;
    }
}

// src/main_seq.cpp:28-36
void applyVelocityBC(int ndim, vector<int>& S, vector<long double> v0, vector<vector<long double>>& velocity,
                     vector<vector<long double>>& acce) {
  for (int pi : S)
    for (int m = 0; m < ndim; ++m) {
      velocity[pi][m] = v0[m];
      acce[pi][m] = 0.0;
    }
}

// src/main_seq.cpp:38-46
void applyFixedBC(int ndim, vector<int>& S, vector<Particle>& P) {
  for (int pi : S)
    for (int m = 0; m < ndim; ++m) P[pi].currentPositions[m] = P[pi].initialPositions[m];
}

// src/main_seq.cpp:49-68
void buildLocalNeighborlist(int, double, double, vector<Particle>& P, const unordered_map<int, int>& g2l,
                            vector<vector<Particle*>>& NL) {
  for (size_t i = 0; i < P.size(); ++i) {
    vector<Particle*> row;
    for (int nb : P[i].neighbors) {
      auto it = g2l.find(nb);
      if (it != g2l.end()) {
        row.push_back(&P[it->second]);
      } else {
        std::cout << "Error in buildLocalNeighborlist: Key " << nb << " not found in globalLocalIDmap." << std::endl;
        std::cout << " pi = " << P[i].globalID << std::endl;
      }
    }
    NL.push_back(row);
  }
}

// src/main_seq.cpp:180-201
matrix getStiffnessTensor(int ndim, double E, double nv) {
  matrix C;
  if (ndim == 2) {
    C = matrix(3, {1.0, nv, 0.0, nv, 1.0, 0.0, 0.0, 0.0, 1 - nv}).timeScalar(E / (1 - std::pow(nv, 2)));
  } else if (ndim == 3) {
    C = matrix(6, {1.0 - nv, nv, nv, 0.0, 0.0, 0.0, nv, 1.0 - nv, nv, 0.0, 0.0, 0.0, nv, nv, 1.0 - nv, 0.0, 0.0, 0.0,
                   0.0, 0.0, 0.0, 1 - 2 * nv, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1 - 2 * nv, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0,
                   1 - 2 * nv})
            .timeScalar(E / (1 + nv) / (1 - 2 * nv));
  }
  return C;
}

// src/main_seq.cpp:386-393
void updatePositions(int ndim, vector<Particle>& P, long double dt, long double rho,
                     vector<vector<long double>>& velocity, vector<vector<long double>>& acce,
                     vector<vector<long double>>& netF) {
  for (size_t i = 0; i < P.size(); ++i)
    for (int m = 0; m < ndim; ++m) {
      acce[i][m] = netF[i][m] / rho;
      P[i].currentPositions[m] += velocity[i][m] * dt + 0.5 * acce[i][m] * std::pow(dt, 2);
    }
}

void computeVelocity(int, double n1, double n2, double horizon, double dx, long double massDensity,
                     matrix& StiffnessTensor, long double stepSize, vector<vector<long double>>& velocity,
                     vector<vector<Particle*>>& Neighborslist, vector<vector<long double>>& acce,
                     vector<vector<long double>>& netF, vector<Particle>& localParticles,
                     const unordered_map<int, int>&, vector<vector<double>>&) {
  gpu_velocity(n1, n2, horizon * dx, massDensity, StiffnessTensor, stepSize, velocity, Neighborslist, acce, netF, localParticles,
               false);
}

void compute_velocity_GPU_host(int, double n1, double n2, double horizon, double dx, double massDensity,
                               matrix& StiffnessTensor, double stepSize, vector<vector<long double>>& velocity,
                               vector<vector<Particle*>>& Neighborslist, vector<vector<long double>>& acce,
                               vector<vector<long double>>& netF, vector<Particle>& allParticles,
                               const unordered_map<int, int>&, vector<vector<double>>&) {
  gpu_velocity(n1, n2, horizon * dx, massDensity, StiffnessTensor, stepSize, velocity, Neighborslist, acce, netF, allParticles,
               true);
}

void computeDamageStatus(int, double n1, double n2, double dx, double horizon,
                         vector<vector<double>>& bondDamageThreshold, vector<Particle>& localParticles,
                         const vector<vector<Particle*>>& Neighborslist, vector<vector<double>>& bondDamage,
                         const unordered_map<int, int>&) {
  vector<Particle>& P = localParticles;
  const size_t n = P.size();
  // the particle vector's context (computeVelocity's, or a new one whose
  // material parameters computeVelocity replaces later: Mazars needs none)
  auto it = cache().find(&P);
  const bool have = it != cache().end() && it->second && it->second->data == P.data() && it->second->n == n;
  matrix C = have ? matrix() : getStiffnessTensor(2, 1.0, 0.0);
  if (have) {
    C = matrix(3, vector<long double>(9, 0.0));
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) C.elements[r][c] = it->second->C[3 * r + c];
  }
  Cached& k = context_for(P, const_cast<vector<vector<Particle*>>&>(Neighborslist),
                          have ? it->second->rho : 1.0L, have ? it->second->dt : 1.0L, C, n1, n2, horizon * dx);
  for (size_t i = 0; i < n; ++i)
    for (int m = 0; m < 2; ++m) k.u[2 * i + m] = (double)(P[i].currentPositions[m] - P[i].initialPositions[m]);
  check(pd_set_state(k.ctx, k.u, nullptr, nullptr), k.ctx, "pd_set_state");
  vector<double> thr, bd;
  for (size_t i = 0; i < n; ++i) {
    const size_t deg = Neighborslist.at(i).size();
    if (bondDamageThreshold.at(i).size() < deg || bondDamage.at(i).size() < deg)
      throw std::runtime_error("computeDamageStatus: bondDamageThreshold / bondDamage rows shorter than the families");
    thr.insert(thr.end(), bondDamageThreshold[i].begin(), bondDamageThreshold[i].begin() + deg);
    bd.insert(bd.end(), bondDamage[i].begin(), bondDamage[i].begin() + deg);
  }
  pd_mazars_params mp;
  pd_mazars_default_params(&mp);
  if (!thr.empty()) mp.kappa0 = thr[0];
  check(pd_mazars_init(k.ctx, &mp), k.ctx, "pd_mazars_init");
  check(pd_mazars_set(k.ctx, thr.data(), bd.data()), k.ctx, "pd_mazars_set");
  check(pd_mazars_update(k.ctx), k.ctx, "pd_mazars_update");
  vector<double> status(n);
  check(pd_mazars_get(k.ctx, thr.data(), bd.data(), status.data()), k.ctx, "pd_mazars_get");
  size_t o = 0;
  for (size_t i = 0; i < n; ++i) {
    const size_t deg = Neighborslist[i].size();
    std::copy(thr.begin() + o, thr.begin() + o + deg, bondDamageThreshold[i].begin());
    std::copy(bd.begin() + o, bd.begin() + o + deg, bondDamage[i].begin());
    o += deg;
    P[i].damageStatus = status[i];
  }
  if (bondDamage.size() > n) bondDamage[n].resize(30, 0.0);  // the reference's ghost row (src/main_seq.cpp:596)
}

void pd_dropin_set_critical_stretch(double s_c) { g_s_c = s_c; }

void pd_dropin_damage(const vector<Particle>& P, vector<double>& damage) {
  auto it = cache().find(&P);
  damage.assign(P.size(), 0.0);
  if (it == cache().end() || !it->second) return;
  check(pd_get_damage(it->second->ctx, damage.data()), it->second->ctx, "pd_get_damage");
}

void pd_dropin_release() { cache().clear(); }
