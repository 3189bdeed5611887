// Synthetic implicit-Euler FEM beam QPs: the inputs the solver is measured on.
//
// Restates the system the reference's MPRGP FEM driver hands to the solver
// (src/CollisionHandle/MprgpFemSolver.cpp:315-356 via
// src/ElasticSolver/FEMSystem.cpp:167-193) for a linear material
// (FEMEnergy.cpp:657 evalFLinear; Lame parameters as FEMEnergy.cpp:383-384)
// with lumped mass (vertex mass += rho*V/4 per tet, FEMMesh.cpp:501-511):
//   A = M + h^2 K,   b = M (x0 + h v0) + h^2 M g + h^2 K X
// where X is the rest shape and x0 = X shifted so the lowest layer sits at
// y = -lift.  Constraints follow LinearConCollider's plane form n.x + p >= 0
// (LinearConCollider.h:21): a floor y >= 0 on every vertex plus seeded random
// planes.  The mesh is an a x b x c grid of cubes, each split into the six
// Kuhn tetrahedra around its (1,1,1) diagonal, so every interior vertex has
// 14 neighbours and its block row of A holds 15 3x3 blocks.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/mprgp_gpu.h"

namespace {

inline uint64_t mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  uint64_t z = x;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
// Uniform in (0, 1] from (seed, stream, index).
inline double unif(uint64_t seed, uint64_t stream, uint64_t i) {
  const uint64_t h = mix64(mix64(seed ^ (stream * 0xD1B54A32D192ED03ull)) + i);
  return ((double)(h >> 11) + 1.0) * 0x1.0p-53;
}
inline double gauss(uint64_t seed, uint64_t stream, uint64_t i) {  // Box-Muller
  const double u1 = unif(seed, stream, 2 * i), u2 = unif(seed, stream, 2 * i + 1);
  return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
}

struct Grid {
  int a, b, c, nx, ny, nz, nv;
  explicit Grid(const mprgp_beam_params &p)
      : a(p.a), b(p.b), c(p.c), nx(p.a + 1), ny(p.b + 1), nz(p.c + 1),
        nv((p.a + 1) * (p.b + 1) * (p.c + 1)) {}
  int id(int i, int j, int k) const { return i + nx * (j + ny * k); }
};

// Sorted neighbour list (including the vertex itself) of vertex (i,j,k).
int neighbours(const Grid &G, int i, int j, int k, int *out) {
  static const int off[15][3] = {{0, 0, 0},   {1, 0, 0},  {-1, 0, 0},  {0, 1, 0},  {0, -1, 0},
                                 {0, 0, 1},   {0, 0, -1}, {1, 1, 0},   {-1, -1, 0}, {1, 0, 1},
                                 {-1, 0, -1}, {0, 1, 1},  {0, -1, -1}, {1, 1, 1},  {-1, -1, -1}};
  int n = 0;
  for (const auto &o : off) {
    const int ii = i + o[0], jj = j + o[1], kk = k + o[2];
    if (ii < 0 || jj < 0 || kk < 0 || ii >= G.nx || jj >= G.ny || kk >= G.nz) continue;
    out[n++] = G.id(ii, jj, kk);
  }
  std::sort(out, out + n);
  return n;
}

bool valid(const mprgp_beam_params *p) {
  return p && p->a > 0 && p->b > 0 && p->c > 0 && p->edge > 0 && p->rho > 0 &&
         p->poisson < 0.5 && p->extra_planes_min >= 0 &&
         p->extra_planes_max >= p->extra_planes_min && p->extra_planes_max <= 2 &&
         p->plane_band >= 0.0 && p->max_tilt >= 0.0 && p->max_tilt <= 1.5707963267948966 &&
         (double)(p->a + 1) * (p->b + 1) * (p->c + 1) < 2.0e8;
}

// Number of global planes of this beam: seeded in [min, max].
int global_count(const mprgp_beam_params *p) {
  const int span = p->extra_planes_max - p->extra_planes_min + 1;
  const int e = p->extra_planes_min + (int)(unif(p->seed, 11, 0) * span);
  return std::min(e, p->extra_planes_max);
}

// Seeded global planes (n, p), n.x + p >= 0, with normals uniform on the
// upper hemisphere.  Each plane cuts at most `lift` deep into x0, like the
// floor: contact in a time-stepped simulation penetrates by about one step's
// motion.  `active_frac` (0..1) moves the plane from touching the deepest
// vertex (0) to the full `lift` penetration (1).
void global_planes(const mprgp_beam_params *p, const double *x0, int nv,
                   std::vector<std::array<double, 4>> &out) {
  out.clear();
  const int G = global_count(p);
  for (int t = 0; t < G; ++t) {
    double n[3];
    if (p->plane_mode == 2) {  // walls x >= x_min + lift, z >= z_min + lift
      n[0] = (t == 0) ? 1.0 : 0.0;
      n[1] = 0.0;
      n[2] = (t == 0) ? 0.0 : 1.0;
    } else {
      // cos(theta) uniform on [cos(max_tilt), 1]: uniform area on the cap
      const double cmin = std::cos(p->max_tilt);
      const double ny = cmin + (1.0 - cmin) * unif(p->seed, 21, (uint64_t)t);
      const double ph = 6.283185307179586 * unif(p->seed, 22, (uint64_t)t);
      const double r = std::sqrt(std::max(0.0, 1.0 - ny * ny));
      n[0] = r * std::cos(ph);
      n[1] = ny;
      n[2] = r * std::sin(ph);
    }
    double dmin = 1e300;
    for (int v = 0; v < nv; ++v)
      dmin = std::min(dmin, n[0] * x0[3LL * v] + n[1] * x0[3LL * v + 1] + n[2] * x0[3LL * v + 2]);
    const double depth = p->lift * std::min(1.0, std::max(0.0, p->active_frac));
    out.push_back({n[0], n[1], n[2], -(dmin + depth)});
  }
}

// Contact facets: a seeded fraction `active_frac` of the vertices in the
// lowest `facet_layers` layers each get extra_planes_min..max planes through
// their start position, normals uniform on the upper-hemisphere cap within
// max_tilt of +y.  They are active from the start; no plane sits close to a
// free vertex.
int facet_count(const mprgp_beam_params *p, int v) {
  const int ny = p->b + 1, nx = p->a + 1;
  const int j = (v / nx) % ny;
  if (j >= p->facet_layers) return 0;
  if (unif(p->seed, 31, (uint64_t)v) > p->active_frac) return 0;
  const int span = p->extra_planes_max - p->extra_planes_min + 1;
  const int e = p->extra_planes_min + (int)(unif(p->seed, 32, (uint64_t)v) * span);
  return std::min(e, p->extra_planes_max);
}
void facet_normal(const mprgp_beam_params *p, int v, int t, double n[3]) {
  const uint64_t key = 4ull * (uint64_t)v + (uint64_t)t;
  const double cmin = std::cos(p->max_tilt);
  const double ny = cmin + (1.0 - cmin) * unif(p->seed, 33, key);
  const double ph = 6.283185307179586 * unif(p->seed, 34, key);
  const double r = std::sqrt(std::max(0.0, 1.0 - ny * ny));
  n[0] = r * std::cos(ph);
  n[1] = ny;
  n[2] = r * std::sin(ph);
}

int extra_count(const mprgp_beam_params *p, const std::vector<std::array<double, 4>> &gp,
                const double *x0, int v) {
  int e = 0;
  for (const auto &P : gp) {
    const double s = P[0] * x0[3LL * v] + P[1] * x0[3LL * v + 1] + P[2] * x0[3LL * v + 2] + P[3];
    if (s < p->plane_band) ++e;
  }
  return e;
}

}  // namespace

extern "C" {

void mprgp_beam_default(mprgp_beam_params *p) {
  p->a = 4;
  p->b = 4;
  p->c = 16;
  p->edge = 0.05;
  p->young = 1e5;
  p->poisson = 0.45;
  p->rho = 1000.0;
  p->dt = 0.01;
  p->gravity = -9.8;
  p->lift = 0.01;
  p->v0_sigma = 0.1;
  p->extra_planes_max = 0;
  p->extra_planes_min = 0;
  p->active_frac = 1.0;
  p->plane_band = 0.025;
  p->max_tilt = 1.5707963267948966;
  p->plane_mode = 2;
  p->facet_layers = 1;
  p->seed = 1;
}

int mprgp_beam_sizes(const mprgp_beam_params *p, int *nv, int *nnzb, int *nplanes) {
  if (!valid(p)) return MPRGP_INVALID;
  const Grid G(*p);
  long long nb = 0, np = 0;
  int nb_buf[15];
  std::vector<double> x0(3LL * G.nv);
  for (int k = 0; k < G.nz; ++k)
    for (int j = 0; j < G.ny; ++j)
      for (int i = 0; i < G.nx; ++i) {
        const int v = G.id(i, j, k);
        x0[3LL * v] = i * p->edge;
        x0[3LL * v + 1] = j * p->edge - p->lift;
        x0[3LL * v + 2] = k * p->edge;
      }
  std::vector<std::array<double, 4>> gp;
  if (p->plane_mode != 1) global_planes(p, x0.data(), G.nv, gp);
  for (int k = 0; k < G.nz; ++k)
    for (int j = 0; j < G.ny; ++j)
      for (int i = 0; i < G.nx; ++i) {
        nb += neighbours(G, i, j, k, nb_buf);
        np += 1 + (p->plane_mode != 1 ? extra_count(p, gp, x0.data(), G.id(i, j, k))
                                       : facet_count(p, G.id(i, j, k)));
      }
  if (nb > 0x7fffffffLL || np > 0x7fffffffLL) return MPRGP_INVALID;
  if (nv) *nv = G.nv;
  if (nnzb) *nnzb = (int)nb;
  if (nplanes) *nplanes = (int)np;
  return MPRGP_OK;
}

int mprgp_beam_mesh(const mprgp_beam_params *p, int *tets, double *X, double *x0, double *v0) {
  if (!valid(p) || !tets || !X) return MPRGP_INVALID;
  const Grid G(*p);
  static const int perm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  long long t4 = 0;
  for (int k = 0; k < p->c; ++k)
    for (int j = 0; j < p->b; ++j)
      for (int i = 0; i < p->a; ++i)
        for (int t = 0; t < 6; ++t) {
          int o[4][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {1, 1, 1}};
          o[1][perm[t][0]] = 1;
          o[2][perm[t][0]] = 1;
          o[2][perm[t][1]] = 1;
          for (int a = 0; a < 4; ++a) tets[t4++] = G.id(i + o[a][0], j + o[a][1], k + o[a][2]);
        }
  for (int v = 0; v < G.nv; ++v) {
    const int i = v % G.nx, j = (v / G.nx) % G.ny, k = v / (G.nx * G.ny);
    for (int d = 0; d < 3; ++d) {
      const long long q = 3LL * v + d;
      X[q] = (d == 0 ? i : d == 1 ? j : k) * p->edge;
      if (x0) x0[q] = X[q] + (d == 1 ? -p->lift : 0.0);
      if (v0) v0[q] = p->v0_sigma * gauss(p->seed, 7, (uint64_t)q);
    }
  }
  return MPRGP_OK;
}

int mprgp_beam_build(const mprgp_beam_params *p, int *row_ptr, int *cols, double *vals,
                     double *b, double *x0, int *plane_ptr, double *planes) {
  if (!valid(p) || !row_ptr || !cols || !vals || !b || !x0) return MPRGP_INVALID;
  const Grid G(*p);
  const int nv = G.nv;
  // Pattern.
  row_ptr[0] = 0;
  int nb_buf[15];
  for (int k = 0; k < G.nz; ++k)
    for (int j = 0; j < G.ny; ++j)
      for (int i = 0; i < G.nx; ++i) {
        const int v = G.id(i, j, k);
        const int cnt = neighbours(G, i, j, k, nb_buf);
        row_ptr[v + 1] = row_ptr[v] + cnt;
        std::memcpy(cols + row_ptr[v], nb_buf, sizeof(int) * cnt);
      }
  const long long nnzb = row_ptr[nv];
  std::memset(vals, 0, sizeof(double) * 9 * nnzb);
  auto block = [&](int r, int cidx) -> double * {
    for (int q = row_ptr[r]; q < row_ptr[r + 1]; ++q)
      if (cols[q] == cidx) return vals + 9LL * q;
    return nullptr;
  };

  const double h = p->edge;
  const double lam = p->poisson * p->young / ((1.0 + p->poisson) * (1.0 - 2.0 * p->poisson));
  const double mu = p->young / (2.0 * (1.0 + p->poisson));
  const double h2 = p->dt * p->dt;
  std::vector<double> mass(nv, 0.0);
  std::vector<double> KX(3LL * nv, 0.0);  // K * X (rest shape)
  auto rest = [&](int v, int d) -> double {
    const int i = v % G.nx, j = (v / G.nx) % G.ny, k = v / (G.nx * G.ny);
    return (d == 0 ? i : d == 1 ? j : k) * h;
  };
  static const int perm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  // Shape-function gradients are the same for every cube of a given
  // permutation (the grid is uniform), so compute each tet's element matrix
  // once per permutation.
  std::array<std::array<double, 144>, 6> Ke;
  std::array<double, 6> vol;
  std::array<std::array<std::array<int, 3>, 4>, 6> corner;  // offsets of the 4 vertices
  for (int t = 0; t < 6; ++t) {
    int o[4][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {1, 1, 1}};
    o[1][perm[t][0]] = 1;
    o[2][perm[t][0]] = 1;
    o[2][perm[t][1]] = 1;
    for (int a = 0; a < 4; ++a)
      for (int d = 0; d < 3; ++d) corner[t][a][d] = o[a][d];
    double Dm[3][3];  // columns x_a - x_0
    for (int a = 1; a < 4; ++a)
      for (int d = 0; d < 3; ++d) Dm[d][a - 1] = (o[a][d] - o[0][d]) * h;
    const double det = Dm[0][0] * (Dm[1][1] * Dm[2][2] - Dm[1][2] * Dm[2][1]) -
                       Dm[0][1] * (Dm[1][0] * Dm[2][2] - Dm[1][2] * Dm[2][0]) +
                       Dm[0][2] * (Dm[1][0] * Dm[2][1] - Dm[1][1] * Dm[2][0]);
    double inv[3][3];  // Dm^-1
    inv[0][0] = (Dm[1][1] * Dm[2][2] - Dm[1][2] * Dm[2][1]) / det;
    inv[0][1] = (Dm[0][2] * Dm[2][1] - Dm[0][1] * Dm[2][2]) / det;
    inv[0][2] = (Dm[0][1] * Dm[1][2] - Dm[0][2] * Dm[1][1]) / det;
    inv[1][0] = (Dm[1][2] * Dm[2][0] - Dm[1][0] * Dm[2][2]) / det;
    inv[1][1] = (Dm[0][0] * Dm[2][2] - Dm[0][2] * Dm[2][0]) / det;
    inv[1][2] = (Dm[0][2] * Dm[1][0] - Dm[0][0] * Dm[1][2]) / det;
    inv[2][0] = (Dm[1][0] * Dm[2][1] - Dm[1][1] * Dm[2][0]) / det;
    inv[2][1] = (Dm[0][1] * Dm[2][0] - Dm[0][0] * Dm[2][1]) / det;
    inv[2][2] = (Dm[0][0] * Dm[1][1] - Dm[0][1] * Dm[1][0]) / det;
    double gradN[4][3];  // row a of Dm^-1 is grad N_a, a = 1..3
    for (int d = 0; d < 3; ++d) {
      gradN[1][d] = inv[0][d];
      gradN[2][d] = inv[1][d];
      gradN[3][d] = inv[2][d];
      gradN[0][d] = -(inv[0][d] + inv[1][d] + inv[2][d]);
    }
    const double V = std::fabs(det) / 6.0;
    vol[t] = V;
    // K_ab[i][j] = V (lam dNa_i dNb_j + mu dNa_j dNb_i + mu (dNa . dNb) delta_ij)
    for (int a = 0; a < 4; ++a)
      for (int bb = 0; bb < 4; ++bb) {
        const double dd = gradN[a][0] * gradN[bb][0] + gradN[a][1] * gradN[bb][1] +
                          gradN[a][2] * gradN[bb][2];
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j)
            Ke[t][(3 * a + i) * 12 + 3 * bb + j] =
                V * (lam * gradN[a][i] * gradN[bb][j] + mu * gradN[a][j] * gradN[bb][i] +
                     (i == j ? mu * dd : 0.0));
      }
  }
  for (int k = 0; k < p->c; ++k)
    for (int j = 0; j < p->b; ++j)
      for (int i = 0; i < p->a; ++i)
        for (int t = 0; t < 6; ++t) {
          int vid[4];
          for (int a = 0; a < 4; ++a)
            vid[a] = G.id(i + corner[t][a][0], j + corner[t][a][1], k + corner[t][a][2]);
          for (int a = 0; a < 4; ++a) {
            mass[vid[a]] += p->rho * vol[t] / 4.0;
            for (int bb = 0; bb < 4; ++bb) {
              double *blk = block(vid[a], vid[bb]);
              for (int ii = 0; ii < 3; ++ii)
                for (int jj = 0; jj < 3; ++jj) {
                  const double kv = Ke[t][(3 * a + ii) * 12 + 3 * bb + jj];
                  blk[3 * ii + jj] += h2 * kv;
                  KX[3LL * vid[a] + ii] += kv * rest(vid[bb], jj);
                }
            }
          }
        }
  for (int v = 0; v < nv; ++v) {
    double *blk = block(v, v);
    for (int d = 0; d < 3; ++d) blk[4 * d] += mass[v];
  }
  // x0, v0, b.
  for (int v = 0; v < nv; ++v)
    for (int d = 0; d < 3; ++d) {
      const long long q = 3LL * v + d;
      const double X = rest(v, d);
      const double x = X + (d == 1 ? -p->lift : 0.0);
      const double vel = p->v0_sigma * gauss(p->seed, 7, (uint64_t)q);
      x0[q] = x;
      b[q] = mass[v] * (x + p->dt * vel) + h2 * mass[v] * (d == 1 ? p->gravity : 0.0) +
             h2 * KX[q];
    }
  // Planes: the floor y >= 0 on every vertex, then the beam's global planes
  // on the vertices within `plane_band` of them at x0 (a proximity query, as
  // LinearConCollider::handle(plane) adds constraints, LinearConCollider.cpp:140-161).
  if (plane_ptr && planes) {
    std::vector<std::array<double, 4>> gp;
    if (p->plane_mode != 1) global_planes(p, x0, nv, gp);
    plane_ptr[0] = 0;
    long long q = 0;
    for (int v = 0; v < nv; ++v) {
      double *pl = planes + 4 * q;
      pl[0] = 0.0; pl[1] = 1.0; pl[2] = 0.0; pl[3] = 0.0;
      ++q;
      if (p->plane_mode != 1) {
        for (const auto &P : gp) {
          const double s = P[0] * x0[3LL * v] + P[1] * x0[3LL * v + 1] + P[2] * x0[3LL * v + 2] + P[3];
          if (s >= p->plane_band) continue;
          pl = planes + 4 * q;
          pl[0] = P[0]; pl[1] = P[1]; pl[2] = P[2]; pl[3] = P[3];
          ++q;
        }
      } else {
        const int e = facet_count(p, v);
        for (int t = 0; t < e; ++t) {
          double n[3];
          facet_normal(p, v, t, n);
          pl = planes + 4 * q;
          pl[0] = n[0]; pl[1] = n[1]; pl[2] = n[2];
          // through the vertex's start position (projected onto the floor)
          const double y0 = std::max(0.0, x0[3LL * v + 1]);
          pl[3] = -(n[0] * x0[3LL * v] + n[1] * y0 + n[2] * x0[3LL * v + 2]);
          ++q;
        }
      }
      plane_ptr[v + 1] = (int)q;
    }
  }
  return MPRGP_OK;
}

}  // extern "C"
