/* TEST ORACLE -- not part of the product; see pd_oracle.h.
 *
 * Restatement of the reference's sequential step, classic form:
 *   reference (src/main_seq.cpp)            restated here
 *   applyVelocityBC        :28-36           drift(), BC group kind VELOCITY
 *   updatePositions        :386-393         drift()
 *   applyFixedBC           :38-46           drift(), BC group kind FIXED
 *   computeShapeTensors    :71-156          pass_a(): K (cached), N per particle
 *   computeStressTensor    :204-268         pass_a(): F = N K^-1, eps, sigma
 *   matrix::inverse2D      src/matrix.cpp:116-129   kinv_of() (+ det guard)
 *   computeForceDensityStates :271-380      pass_a(): S = sigma K^-1
 *   computeVelocity        :396-470         pass_b(): f_i = sum_j V_j (S_i+S_j) xi_ij, kick
 *   findNeighbor  src/SetupParticleSystem.cpp:100-121   pdo_build_families()
 * With n1 = n2 = 0 every bond-associated weight is exactly 1
 * (exp(0) * pow(x, 0) = 1), K_{i,nb} = K_i for all nb, and
 *   T_ij = (1/V_h) sum_nb V_nb sigma_i K_i^-1 xi_ij = S_i xi_ij,
 * so the reference's net force sum_j (T_ij - T_ji) V_j is
 *   f_i = S_i m_i + sum_j V_j S_j xi_ij,   m_i = sum_j V_j xi_ij.
 * The canonical form evaluated here is f_i = W_i mt_i + sum_j W_j xi_ij with
 * W = V S and mt = m / V (same quantity, one fewer multiply per bond).
 *
 * State is the displacement u = y - x (FP64), not the absolute position y.
 *
 * Additions of the drop-in (no reference counterpart): a bond breaks for
 * good when |eta| > (1+s_c)|xi| (stretch > s_c); broken bonds leave
 * K, N and the force; damage_i = broken_i / family_i (the reference
 * accumulates damage as a per-bond average, src/main_seq.cpp:588); a
 * relative determinant guard sets S_i = 0 for a particle whose remaining
 * bonds give a singular K (the reference divides by zero on the CPU,
 * src/matrix.cpp:121-126), and so does material-point failure: damage above
 * damage_fail (a particle held by a few bonds has a small K and a stiffness
 * the time step cannot follow).
 */
#include "pd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static void set_threads(int32_t nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
}

void pdo_stiffness(double E, double nu, double c[3]) {
  const double pre = E / (1.0 - nu * nu);
  c[0] = pre;
  c[1] = nu * pre;
  c[2] = (1.0 - nu) * pre;
}

/* ---------------------------------------------------------------- families */

static double orient(double ax, double ay, double bx, double by, double px, double py) {
  const double d1 = (bx - ax) * (py - ay);
  const double d2 = (by - ay) * (px - ax);
  return d1 - d2;
}

/* Proper crossing of segment P-Q with segment A-B (touching does not count). */
static int crosses(double px, double py, double qx, double qy, const double* c) {
  const double o1 = orient(c[0], c[1], c[2], c[3], px, py);
  const double o2 = orient(c[0], c[1], c[2], c[3], qx, qy);
  const double o3 = orient(px, py, qx, qy, c[0], c[1]);
  const double o4 = orient(px, py, qx, qy, c[2], c[3]);
  return ((o1 > 0.0 && o2 < 0.0) || (o1 < 0.0 && o2 > 0.0)) &&
         ((o3 > 0.0 && o4 < 0.0) || (o3 < 0.0 && o4 > 0.0));
}

typedef struct grid {
  double x0, y0, inv_cs;
  int64_t gx, gy;
  int64_t* start; /* [gx*gy+1] */
  int64_t* items; /* [n] particle ids sorted by cell, ascending id within a cell */
} grid;

static int64_t cell_coord(double v, double v0, double inv_cs, int64_t g) {
  int64_t c = (int64_t)floor((v - v0) * inv_cs);
  if (c < 0) c = 0;
  if (c >= g) c = g - 1;
  return c;
}

static int grid_build(grid* G, int64_t n, const double* x, double cutoff) {
  double xmin = INFINITY, xmax = -INFINITY, ymin = INFINITY, ymax = -INFINITY;
  for (int64_t i = 0; i < n; ++i) {
    xmin = fmin(xmin, x[2 * i]); xmax = fmax(xmax, x[2 * i]);
    ymin = fmin(ymin, x[2 * i + 1]); ymax = fmax(ymax, x[2 * i + 1]);
  }
  const double cs = cutoff * 1.0000001;
  G->x0 = xmin; G->y0 = ymin; G->inv_cs = 1.0 / cs;
  G->gx = (int64_t)floor((xmax - xmin) / cs) + 1;
  G->gy = (int64_t)floor((ymax - ymin) / cs) + 1;
  const int64_t nc = G->gx * G->gy;
  G->start = (int64_t*)calloc((size_t)nc + 1, sizeof(int64_t));
  G->items = (int64_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
  if (!G->start || !G->items) return -1;
  for (int64_t i = 0; i < n; ++i) {
    const int64_t c = cell_coord(x[2 * i + 1], G->y0, G->inv_cs, G->gy) * G->gx +
                      cell_coord(x[2 * i], G->x0, G->inv_cs, G->gx);
    G->start[c + 1]++;
  }
  for (int64_t c = 0; c < nc; ++c) G->start[c + 1] += G->start[c];
  int64_t* fill = (int64_t*)malloc((size_t)nc * sizeof(int64_t) + 1);
  if (!fill) return -1;
  memcpy(fill, G->start, (size_t)nc * sizeof(int64_t));
  for (int64_t i = 0; i < n; ++i) {
    const int64_t c = cell_coord(x[2 * i + 1], G->y0, G->inv_cs, G->gy) * G->gx +
                      cell_coord(x[2 * i], G->x0, G->inv_cs, G->gx);
    G->items[fill[c]++] = i;
  }
  free(fill);
  return 0;
}

/* Neighbours of particle i, ascending id, into out (capacity cap); returns count. */
static int64_t family_of(const grid* G, int64_t i, const double* x, double cutoff, int32_t n_cracks,
                         const double* cracks, int32_t* out, int64_t cap) {
  const double xi = x[2 * i], yi = x[2 * i + 1];
  const int64_t cx = cell_coord(xi, G->x0, G->inv_cs, G->gx);
  const int64_t cy = cell_coord(yi, G->y0, G->inv_cs, G->gy);
  int64_t cnt = 0;
  for (int64_t dy = -1; dy <= 1; ++dy) {
    const int64_t yy = cy + dy;
    if (yy < 0 || yy >= G->gy) continue;
    for (int64_t dx = -1; dx <= 1; ++dx) {
      const int64_t xx = cx + dx;
      if (xx < 0 || xx >= G->gx) continue;
      const int64_t c = yy * G->gx + xx;
      for (int64_t k = G->start[c]; k < G->start[c + 1]; ++k) {
        const int64_t j = G->items[k];
        if (j == i) continue;
        const double rx = x[2 * j] - xi, ry = x[2 * j + 1] - yi;
        const double d2 = rx * rx + ry * ry;
        if (!(sqrt(d2) < cutoff)) continue;
        int cut = 0;
        for (int32_t q = 0; q < n_cracks && !cut; ++q) cut = crosses(xi, yi, x[2 * j], x[2 * j + 1], cracks + 4 * q);
        if (cut) continue;
        if (out) {
          if (cnt >= cap) return -1;
          /* insertion keeps ascending order (findNeighbor scans j upward) */
          int64_t p = cnt;
          while (p > 0 && out[p - 1] > (int32_t)j) { out[p] = out[p - 1]; --p; }
          out[p] = (int32_t)j;
        }
        ++cnt;
      }
    }
  }
  return cnt;
}

int pdo_build_families(int64_t n, const double* x, double cutoff, int32_t n_cracks, const double* cracks,
                       int64_t* row_ptr, int32_t* col, int64_t cap, int64_t* nnz_out, int32_t nthreads) {
  set_threads(nthreads);
  grid G;
  if (grid_build(&G, n, x, cutoff) != 0) return -2;
  int64_t* cnt = (int64_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) cnt[i] = family_of(&G, i, x, cutoff, n_cracks, cracks, NULL, 0);
  int64_t nnz = 0;
  for (int64_t i = 0; i < n; ++i) {
    if (row_ptr) row_ptr[i] = nnz;
    nnz += cnt[i];
  }
  if (row_ptr) row_ptr[n] = nnz;
  if (nnz_out) *nnz_out = nnz;
  int rc = 0;
  if (col) {
    if (nnz > cap) rc = -1;
    else {
      int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
      for (int64_t i = 0; i < n; ++i) {
        int32_t buf[1024];
        const int64_t c = family_of(&G, i, x, cutoff, n_cracks, cracks, buf, 1024);
        if (c != cnt[i]) { bad |= 1; continue; }
        memcpy(col + row_ptr[i], buf, (size_t)c * sizeof(int32_t));
      }
      if (bad) rc = -3;
    }
  }
  free(cnt); free(G.start); free(G.items);
  return rc;
}

/* ------------------------------------------------------------------ physics */

/* K^-1 and mt of particle i over its alive bonds.  Returns 1 if singular. */
static int kinv_of(const pdo_problem* pb, const pdo_state* st, int64_t i) {
  const double xi = pb->x[2 * i], yi = pb->x[2 * i + 1];
  double k11 = 0.0, k12 = 0.0, k22 = 0.0, mx = 0.0, my = 0.0;
  int64_t nal = 0;
  for (int64_t s = pb->row_ptr[i]; s < pb->row_ptr[i + 1]; ++s) {
    if (!st->alive[s]) continue;
    const int64_t j = pb->col[s];
    const double ex = pb->x[2 * j] - xi, ey = pb->x[2 * j + 1] - yi;
    const double t = pb->vol[j] * ex, u = pb->vol[j] * ey;
    k11 = fma(t, ex, k11);
    k12 = fma(t, ey, k12);
    k22 = fma(u, ey, k22);
    mx = mx + t;
    my = my + u;
    ++nal;
  }
  const double det = fma(k11, k22, -(k12 * k12));
  double* ki = st->kinv + 3 * i;
  double* mt = st->mt + 2 * i;
  const int64_t fam = pb->row_ptr[i + 1] - pb->row_ptr[i];
  const int failed = fam > 0 && (double)st->broken[i] / (double)fam > pb->damage_fail;
  if (nal == 0 || failed || !(det > pb->det_guard * (k11 * k22))) {
    ki[0] = ki[1] = ki[2] = 0.0;
    mt[0] = mt[1] = 0.0;
    st->singular[i] = 1;
    return 1;
  }
  const double r = 1.0 / det;
  ki[0] = k22 * r;
  ki[1] = -k12 * r;
  ki[2] = k11 * r;
  const double rv = 1.0 / pb->vol[i];
  mt[0] = mx * rv;
  mt[1] = my * rv;
  st->singular[i] = 0;
  return 0;
}

int pdo_init(const pdo_problem* pb, pdo_state* st) {
  set_threads(pb->nthreads);
  const int64_t n = pb->n, nnz = pb->row_ptr[n];
  memset(st->u, 0, (size_t)n * 2 * sizeof(double));
  memset(st->v, 0, (size_t)n * 2 * sizeof(double));
  memset(st->f, 0, (size_t)n * 2 * sizeof(double));
  memset(st->alive, 1, (size_t)nnz);
  memset(st->broken, 0, (size_t)n * sizeof(int32_t));
  memset(st->damage, 0, (size_t)n * sizeof(double));
  memset(st->w, 0, (size_t)n * 4 * sizeof(double));
  memset(st->hg, 0, (size_t)n * 2 * sizeof(double));
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) kinv_of(pb, st, i);
  return 0;
}

/* Start of a step: velocity BC, drift, fixed BC (src/main_seq.cpp:686-692). */
static void drift(const pdo_problem* pb, pdo_state* st) {
  const double dt = pb->dt, dt2 = dt * dt, inv_rho = 1.0 / pb->rho;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < pb->n; ++i) {
    const int g = pb->bc ? pb->bc[i] : 0;
    const int kind = g ? pb->group_kind[g - 1] : PDO_BC_NONE;
    double* v = st->v + 2 * i;
    double* u = st->u + 2 * i;
    if (kind == PDO_BC_VELOCITY) {
      v[0] = pb->group_val[2 * (g - 1)];
      v[1] = pb->group_val[2 * (g - 1) + 1];
    }
    for (int m = 0; m < 2; ++m) {
      const double a = st->f[2 * i + m] * inv_rho;
      u[m] = u[m] + (v[m] * dt + (0.5 * a) * dt2);
    }
    if (kind == PDO_BC_FIXED) {
      u[0] = 0.0;
      u[1] = 0.0;
    }
  }
}

/* Stretch test + D accumulation + stress (per particle); returns bonds broken.
 * With u the displacement, eta = xi + d, d = u_j - u_i:
 *   N = sum V eta (x) xi = K + D,  D = sum V d (x) xi,  F - I = D K^-1,
 * and stretch > s_c  <=>  |eta|^2 - |xi|^2 = d.(2 xi + d) > ((1+s_c)^2 - 1)|xi|^2.
 * Both forms avoid the cancellation of eta - xi / F - I (the reference keeps
 * absolute positions in 80-bit long double instead). */
static int64_t pass_a(const pdo_problem* pb, pdo_state* st) {
  double c[3];
  pdo_stiffness(pb->E, pb->nu, c);
  const double s2 = pb->s_c > 0.0 ? pb->s_c * (2.0 + pb->s_c) : INFINITY;
  int64_t nbroke = 0;
#pragma omp parallel for schedule(static) reduction(+ : nbroke)
  for (int64_t i = 0; i < pb->n; ++i) {
    const double xi = pb->x[2 * i], yi = pb->x[2 * i + 1];
    const double ui = st->u[2 * i], wi = st->u[2 * i + 1];
    double d11 = 0.0, d12 = 0.0, d21 = 0.0, d22 = 0.0, ax = 0.0, ay = 0.0;
    int32_t newly = 0;
    for (int64_t s = pb->row_ptr[i]; s < pb->row_ptr[i + 1]; ++s) {
      if (!st->alive[s]) continue;
      const int64_t j = pb->col[s];
      const double ex = pb->x[2 * j] - xi, ey = pb->x[2 * j + 1] - yi;
      const double dx = st->u[2 * j] - ui, dy = st->u[2 * j + 1] - wi;
      const double q = fma(dx, fma(2.0, ex, dx), dy * fma(2.0, ey, dy));
      const double lim = s2 * fma(ex, ex, ey * ey);
      if (q > lim) {
        st->alive[s] = 0;
        ++newly;
        continue;
      }
      const double t0 = pb->vol[j] * ex, t1 = pb->vol[j] * ey;
      d11 = fma(dx, t0, d11);
      d12 = fma(dx, t1, d12);
      d21 = fma(dy, t0, d21);
      d22 = fma(dy, t1, d22);
      ax = fma(pb->vol[j], dx, ax);
      ay = fma(pb->vol[j], dy, ay);
    }
    {
      const double k2 = 2.0 * pb->k_hg;
      st->hg[2 * i] = k2 * ax;
      st->hg[2 * i + 1] = k2 * ay;
    }
    if (newly) {
      st->broken[i] += newly;
      const int64_t fam = pb->row_ptr[i + 1] - pb->row_ptr[i];
      st->damage[i] = (double)st->broken[i] / (double)fam;
      kinv_of(pb, st, i);
      nbroke += newly;
    }
    double* w = st->w + 4 * i;
    if (st->singular[i]) {
      w[0] = w[1] = w[2] = w[3] = 0.0;
      continue;
    }
    const double* ki = st->kinv + 3 * i;
    const double k11 = ki[0], k12 = ki[1], k22 = ki[2];
    /* G = D K^-1 = F - I */
    const double g11 = fma(d11, k11, d12 * k12), g12 = fma(d11, k12, d12 * k22);
    const double g21 = fma(d21, k11, d22 * k12), g22 = fma(d21, k12, d22 * k22);
    const double e11 = g11, e22 = g22, e12 = 0.5 * (g12 + g21);
    const double s11 = fma(c[0], e11, c[1] * e22);
    const double s22 = fma(c[1], e11, c[0] * e22);
    const double s12 = c[2] * e12;
    const double vi = pb->vol[i], kh = -pb->k_hg;
    /* W = V (sigma K^-1 - k_hg G): correspondence stress plus the
       zero-energy-mode penalty's -k G xi part */
    w[0] = vi * fma(kh, g11, fma(s11, k11, s12 * k12));
    w[1] = vi * fma(kh, g12, fma(s11, k12, s12 * k22));
    w[2] = vi * fma(kh, g21, fma(s12, k11, s22 * k12));
    w[3] = vi * fma(kh, g22, fma(s12, k12, s22 * k22));
  }
  return nbroke;
}

/* Force gather + Verlet kick (src/main_seq.cpp:402-468). */
static void pass_b(const pdo_problem* pb, pdo_state* st) {
  const double dt = pb->dt, inv_rho = 1.0 / pb->rho;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < pb->n; ++i) {
    const double xi = pb->x[2 * i], yi = pb->x[2 * i + 1];
    const double* wi = st->w + 4 * i;
    const double* mt = st->mt + 2 * i;
    double fx = fma(wi[0], mt[0], fma(wi[1], mt[1], st->hg[2 * i]));
    double fy = fma(wi[2], mt[0], fma(wi[3], mt[1], st->hg[2 * i + 1]));
    for (int64_t s = pb->row_ptr[i]; s < pb->row_ptr[i + 1]; ++s) {
      if (!st->alive[s]) continue;
      const int64_t j = pb->col[s];
      const double ex = pb->x[2 * j] - xi, ey = pb->x[2 * j + 1] - yi;
      const double* wj = st->w + 4 * j;
      fx = fma(wj[0], ex, fx);
      fx = fma(wj[1], ey, fx);
      fy = fma(wj[2], ex, fy);
      fy = fma(wj[3], ey, fy);
    }
    double* f = st->f + 2 * i;
    double* v = st->v + 2 * i;
    const double ao0 = f[0] * inv_rho, ao1 = f[1] * inv_rho;
    const double an0 = fx * inv_rho, an1 = fy * inv_rho;
    v[0] = v[0] + (0.5 * (ao0 + an0)) * dt;
    v[1] = v[1] + (0.5 * (ao1 + an1)) * dt;
    f[0] = fx;
    f[1] = fy;
  }
}

/* ------------------------------------------------- bond-associated mode
 * The reference's default model (n1, n2 != 0; src/main_seq.cpp:71-156,
 * :271-380): every bond b = (i, nb) has its own shape tensors
 *   K_b = sum_k w(b,k) V_k xi_k (x) xi_k,  N_b = K_b + D_b,
 *   w(b,k) = exp(-n1 |L_b - L_k| / (horizon dx)) (0.5 + 0.5 cos(b,k))^n2,
 * its own stress sigma_b (F_b = N_b K_b^-1) and P_b = sigma_b K_b^-1, and
 *   T_ij = (1/V_h) sum_b w(j,b) V_b P_b xi_ij,   f_i = sum_j (T_ij - T_ji) V_j.
 * The reference re-derives P_b for every (i, j, b) triple (O(n^3) per
 * particle); here P_b is formed once per bond and T once per bond (O(n^2)).
 * No bond breaking or penalty in this mode (the reference has neither). */
static double ba_weight(const pdo_problem* pb, double bx, double by, double lb, double kx, double ky, double lk) {
  double c = (bx * kx + by * ky) / (lb * lk);
  if (c > 1.0) c = 1.0;
  else if (c < -1.0) c = -1.0;
  const double lr = fabs(lb - lk) / pb->wlen;
  return exp(-pb->n1 * lr) * pow(0.5 + 0.5 * c, pb->n2);
}

static void ba_pass_a(const pdo_problem* pb, pdo_state* st) {
  double c[3];
  pdo_stiffness(pb->E, pb->nu, c);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < pb->n; ++i) {
    const int64_t r0 = pb->row_ptr[i], n = pb->row_ptr[i + 1] - r0;
    if (n == 0) continue;
    double ex[256], ey[256], el[256], vv[256], dx[256], dy[256], P[256][4];
    if (n > 256) continue; /* caller checks the family size */
    const double xi = pb->x[2 * i], yi = pb->x[2 * i + 1], ui = st->u[2 * i], wi = st->u[2 * i + 1];
    double vh = 0.0;
    for (int64_t k = 0; k < n; ++k) {
      const int64_t j = pb->col[r0 + k];
      ex[k] = pb->x[2 * j] - xi;
      ey[k] = pb->x[2 * j + 1] - yi;
      el[k] = sqrt(ex[k] * ex[k] + ey[k] * ey[k]);
      vv[k] = pb->vol[j];
      dx[k] = st->u[2 * j] - ui;
      dy[k] = st->u[2 * j + 1] - wi;
      vh = vh + vv[k];
    }
    for (int64_t b = 0; b < n; ++b) {
      double k11 = 0.0, k12 = 0.0, k22 = 0.0, d11 = 0.0, d12 = 0.0, d21 = 0.0, d22 = 0.0;
      for (int64_t k = 0; k < n; ++k) {
        const double wv = ba_weight(pb, ex[b], ey[b], el[b], ex[k], ey[k], el[k]) * vv[k];
        const double t0 = wv * ex[k], t1 = wv * ey[k];
        k11 = fma(t0, ex[k], k11);
        k12 = fma(t0, ey[k], k12);
        k22 = fma(t1, ey[k], k22);
        d11 = fma(dx[k], t0, d11);
        d12 = fma(dx[k], t1, d12);
        d21 = fma(dy[k], t0, d21);
        d22 = fma(dy[k], t1, d22);
      }
      const double det = fma(k11, k22, -(k12 * k12));
      if (!(det > pb->det_guard * (k11 * k22))) {
        P[b][0] = P[b][1] = P[b][2] = P[b][3] = 0.0;
        continue;
      }
      const double r = 1.0 / det;
      const double q11 = k22 * r, q12 = -k12 * r, q22 = k11 * r;
      const double g11 = fma(d11, q11, d12 * q12), g12 = fma(d11, q12, d12 * q22);
      const double g21 = fma(d21, q11, d22 * q12), g22 = fma(d21, q12, d22 * q22);
      const double e11 = g11, e22 = g22, e12 = 0.5 * (g12 + g21);
      const double s11 = fma(c[0], e11, c[1] * e22);
      const double s22 = fma(c[1], e11, c[0] * e22);
      const double s12 = c[2] * e12;
      P[b][0] = fma(s11, q11, s12 * q12);
      P[b][1] = fma(s11, q12, s12 * q22);
      P[b][2] = fma(s12, q11, s22 * q12);
      P[b][3] = fma(s12, q12, s22 * q22);
    }
    const double rv = 1.0 / vh;
    for (int64_t jj = 0; jj < n; ++jj) {
      double m11 = 0.0, m12 = 0.0, m21 = 0.0, m22 = 0.0;
      for (int64_t b = 0; b < n; ++b) {
        const double wv = ba_weight(pb, ex[jj], ey[jj], el[jj], ex[b], ey[b], el[b]) * vv[b];
        m11 = fma(wv, P[b][0], m11);
        m12 = fma(wv, P[b][1], m12);
        m21 = fma(wv, P[b][2], m21);
        m22 = fma(wv, P[b][3], m22);
      }
      double* t = st->tb + 2 * (r0 + jj);
      t[0] = fma(m11 * rv, ex[jj], (m12 * rv) * ey[jj]);
      t[1] = fma(m21 * rv, ex[jj], (m22 * rv) * ey[jj]);
    }
  }
}

static void ba_pass_b(const pdo_problem* pb, pdo_state* st) {
  const double dt = pb->dt, inv_rho = 1.0 / pb->rho;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < pb->n; ++i) {
    double fx = 0.0, fy = 0.0;
    for (int64_t s = pb->row_ptr[i]; s < pb->row_ptr[i + 1]; ++s) {
      const int64_t j = pb->col[s], r = st->rev[s];
      const double vj = pb->vol[j];
      fx = fma(st->tb[2 * s] - st->tb[2 * r], vj, fx);
      fy = fma(st->tb[2 * s + 1] - st->tb[2 * r + 1], vj, fy);
    }
    double* f = st->f + 2 * i;
    double* v = st->v + 2 * i;
    const double ao0 = f[0] * inv_rho, ao1 = f[1] * inv_rho;
    const double an0 = fx * inv_rho, an1 = fy * inv_rho;
    v[0] = v[0] + (0.5 * (ao0 + an0)) * dt;
    v[1] = v[1] + (0.5 * (ao1 + an1)) * dt;
    f[0] = fx;
    f[1] = fy;
  }
}

int pdo_reverse_bonds(int64_t n, const int64_t* row_ptr, const int32_t* col, int64_t* rev) {
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (int64_t i = 0; i < n; ++i)
    for (int64_t s = row_ptr[i]; s < row_ptr[i + 1]; ++s) {
      const int64_t j = col[s];
      int64_t lo = row_ptr[j], hi = row_ptr[j + 1], found = -1;
      while (lo < hi) {
        const int64_t mid = lo + (hi - lo) / 2;
        if (col[mid] < i) lo = mid + 1;
        else if (col[mid] > i) hi = mid;
        else { found = mid; break; }
      }
      rev[s] = found;
      if (found < 0) bad |= 1;
    }
  return bad ? -1 : 0;
}

int64_t pdo_step(const pdo_problem* pb, pdo_state* st, int32_t nsteps) {
  set_threads(pb->nthreads);
  int64_t nb = 0;
  const int ba = pb->n1 != 0.0 || pb->n2 != 0.0;
  for (int32_t s = 0; s < nsteps; ++s) {
    drift(pb, st);
    if (ba) {
      ba_pass_a(pb, st);
      ba_pass_b(pb, st);
    } else {
      nb += pass_a(pb, st);
      pass_b(pb, st);
    }
  }
  return nb;
}

/* ------------------------------------------------------- Mazars damage
 * computeDamageStatus (src/main_seq.cpp:473-598).  The 2x2 symmetric
 * eigen-decomposition follows Eigen's SelfAdjointEigenSolver contract
 * (ascending eigenvalues, unit eigenvector columns) in closed form:
 * mean -+ sqrt(((p - q)/2)^2 + o^2), eigenvector (o, lambda - p) / norm, the
 * axes when o = 0. */
static void sym_eig2(double p, double o, double q, double lam[2], double vec[2][2]) {
  const double mean = 0.5 * (p + q), h = 0.5 * (p - q);
  const double rad = sqrt(h * h + o * o);
  lam[0] = mean - rad;
  lam[1] = mean + rad;
  if (o == 0.0) {
    const int swap = p > q;
    vec[0][0] = swap ? 0.0 : 1.0;
    vec[1][0] = swap ? 1.0 : 0.0;
    vec[0][1] = swap ? 1.0 : 0.0;
    vec[1][1] = swap ? 0.0 : 1.0;
    return;
  }
  for (int k = 0; k < 2; ++k) {
    const double x = o, y = lam[k] - p;
    const double nrm = sqrt(x * x + y * y);
    vec[0][k] = x / nrm;
    vec[1][k] = y / nrm;
  }
}

/* Equivalent strain and the (alpha_t, alpha_c) split of a strain e, as the
 * reference forms them (:525-566). */
typedef struct mz_point {
  double eq, at, ac;
} mz_point;

static mz_point mazars_point(double e11, double e12, double e22) {
  double lam[2], v[2][2];
  sym_eig2(e11, e12, e22, lam, v);
  double s2 = 0.0;
  for (int i = 0; i < 2; ++i)
    if (lam[i] > 0.0) s2 += lam[i] * lam[i];
  mz_point r = {s2 > 0.0 ? sqrt(s2) : 0.0, 0.0, 0.0};
  if (!(r.eq > 0.0)) return r;
  double st[2][2] = {{0.0, 0.0}, {0.0, 0.0}}, sc[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
  for (int i = 0; i < 2; ++i) {
    if (lam[i] > 0.0) {
      for (int j = 0; j < 2; ++j)
        for (int k = 0; k < 2; ++k) st[j][k] += lam[i] * v[j][i] * v[k][i];
    } else if (lam[i] < 0.0) {
      for (int j = 0; j < 2; ++j)
        for (int k = 0; k < 2; ++k) sc[j][k] += lam[i] * v[j][i] * v[k][i];
    }
  }
  double tl[2], tv[2][2], cl[2], cv[2][2];
  sym_eig2(st[0][0], 0.5 * (st[0][1] + st[1][0]), st[1][1], tl, tv);
  sym_eig2(sc[0][0], 0.5 * (sc[0][1] + sc[1][0]), sc[1][1], cl, cv);
  for (int i = 0; i < 2; ++i) {
    if (tl[i] > 0.0) r.at += tl[i] * (tl[i] + cl[i]) / (r.eq * r.eq);
    if (cl[i] > 0.0) r.ac += cl[i] * (tl[i] + cl[i]) / (r.eq * r.eq);
  }
  return r;
}

/* Bond update (:539-584): only where eq exceeds the bond's threshold. */
static void mazars_bond(const mz_point* p, const pdo_mazars* mp, double* thr, double* bd) {
  if (!(p->eq > *thr)) return;
  const double k = *thr;
  const double dt = 1.0 - k * (1 - mp->a_t) / p->eq - mp->a_t / exp(mp->b_t * (p->eq - k));
  const double dc = 1.0 - k * (1 - mp->a_c) / p->eq - mp->a_c / exp(mp->b_c * (p->eq - k));
  *bd = p->at * dt + p->ac * dc;
  *thr = p->eq;
}

int pdo_mazars_update(const pdo_problem* pb, const pdo_state* st, const pdo_mazars* mp, double* thr, double* bd,
                      double* status) {
  const int ba = pb->n1 != 0.0 || pb->n2 != 0.0;
  int bad = 0;
  set_threads(pb->nthreads);
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (int64_t i = 0; i < pb->n; ++i) {
    const int64_t r0 = pb->row_ptr[i], n = pb->row_ptr[i + 1] - r0;
    const double xi = pb->x[2 * i], yi = pb->x[2 * i + 1], ui = st->u[2 * i], wi = st->u[2 * i + 1];
    if (!ba) {
      /* classic: one strain per particle, D over the intact bonds as pass A */
      double d11 = 0.0, d12 = 0.0, d21 = 0.0, d22 = 0.0;
      for (int64_t s = r0; s < r0 + n; ++s) {
        if (!st->alive[s]) continue;
        const int64_t j = pb->col[s];
        const double ex = pb->x[2 * j] - xi, ey = pb->x[2 * j + 1] - yi;
        const double dx = st->u[2 * j] - ui, dy = st->u[2 * j + 1] - wi;
        const double t0 = pb->vol[j] * ex, t1 = pb->vol[j] * ey;
        d11 = fma(dx, t0, d11);
        d12 = fma(dx, t1, d12);
        d21 = fma(dy, t0, d21);
        d22 = fma(dy, t1, d22);
      }
      mz_point p = {0.0, 0.0, 0.0};
      if (!st->singular[i]) {
        const double* ki = st->kinv + 3 * i;
        const double k11 = ki[0], k12 = ki[1], k22 = ki[2];
        const double g11 = fma(d11, k11, d12 * k12), g12 = fma(d11, k12, d12 * k22);
        const double g21 = fma(d21, k11, d22 * k12), g22 = fma(d21, k12, d22 * k22);
        p = mazars_point(g11, 0.5 * (g12 + g21), g22);
      }
      for (int64_t s = r0; s < r0 + n; ++s) mazars_bond(&p, mp, thr + s, bd + s);
    } else {
      if (n > 256) {
        bad = 1;
        continue;
      }
      double ex[256], ey[256], el[256], vv[256], dx[256], dy[256];
      for (int64_t k = 0; k < n; ++k) {
        const int64_t j = pb->col[r0 + k];
        ex[k] = pb->x[2 * j] - xi;
        ey[k] = pb->x[2 * j + 1] - yi;
        el[k] = sqrt(ex[k] * ex[k] + ey[k] * ey[k]);
        vv[k] = pb->vol[j];
        dx[k] = st->u[2 * j] - ui;
        dy[k] = st->u[2 * j + 1] - wi;
      }
      for (int64_t b = 0; b < n; ++b) {
        double k11 = 0.0, k12 = 0.0, k22 = 0.0, d11 = 0.0, d12 = 0.0, d21 = 0.0, d22 = 0.0;
        for (int64_t k = 0; k < n; ++k) {
          const double wv = ba_weight(pb, ex[b], ey[b], el[b], ex[k], ey[k], el[k]) * vv[k];
          const double t0 = wv * ex[k], t1 = wv * ey[k];
          k11 = fma(t0, ex[k], k11);
          k12 = fma(t0, ey[k], k12);
          k22 = fma(t1, ey[k], k22);
          d11 = fma(dx[k], t0, d11);
          d12 = fma(dx[k], t1, d12);
          d21 = fma(dy[k], t0, d21);
          d22 = fma(dy[k], t1, d22);
        }
        mz_point p = {0.0, 0.0, 0.0};
        const double det = fma(k11, k22, -(k12 * k12));
        if (det > pb->det_guard * (k11 * k22)) {
          const double r = 1.0 / det;
          const double q11 = k22 * r, q12 = -k12 * r, q22 = k11 * r;
          const double g11 = fma(d11, q11, d12 * q12), g12 = fma(d11, q12, d12 * q22);
          const double g21 = fma(d21, q11, d22 * q12), g22 = fma(d21, q12, d22 * q22);
          p = mazars_point(g11, 0.5 * (g12 + g21), g22);
        }
        mazars_bond(&p, mp, thr + r0 + b, bd + r0 + b);
      }
    }
    double sum = 0.0;
    for (int64_t s = r0; s < r0 + n; ++s) sum += bd[s] / (double)n;
    status[i] = sum;
  }
  return bad ? -1 : 0;
}

