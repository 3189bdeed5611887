// oracle/beam_oracle.h -- CPU restatement of the synthetic beam QP inputs.
//
// TEST INFRASTRUCTURE ONLY (see mprgp_oracle.h).  The CPU side of the
// measurements -- the reference arm and the CPU baseline -- builds its QPs
// here, so that it runs without the GPU library.  A CPU test checks that
// these QPs equal the library's mprgp_beam_build output bit for bit.
//
// The system is the one the reference's MPRGP FEM driver hands to the solver
// (src/CollisionHandle/MprgpFemSolver.cpp:315-356 through
// src/ElasticSolver/FEMSystem.cpp:167-193) for a linear material
// (FEMEnergy.cpp:657; Lame parameters as FEMEnergy.cpp:383-384) and lumped
// mass (rho V / 4 per tet corner, FEMMesh.cpp:501-511):
//   A = M + h^2 K,   b = M (x0 + h v0) + h^2 M g + h^2 K X.
// Mesh: a x b x c cubes of edge `edge`, each split into the six Kuhn tets
// around its (1,1,1) diagonal; vertex (i,j,k) has id i + nx (j + ny k).
// Planes (n, p) mean n.x + p >= 0 (LinearConCollider.h:21): the floor y >= 0
// on every vertex, then walls / tilted planes / contact facets by mode.
//
// Every floating-point expression is written in the order the GPU library's
// generator evaluates it, so that the two agree bit for bit when both are
// compiled without contraction of products into fused multiply-adds.
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <vector>

namespace oracle {

struct BeamSpec {
  int a = 4, b = 4, c = 16;
  double edge = 0.05, young = 1e5, poisson = 0.45, rho = 1000.0, dt = 0.01, gravity = -9.8;
  double lift = 0.01, v0_sigma = 0.1;
  int planes_max = 0, planes_min = 0;
  double active_frac = 1.0;
  uint64_t seed = 1;
  double band = 0.025, max_tilt = 1.5707963267948966;
  int mode = 2, facet_layers = 1;
};

struct BeamQPData {
  int nv = 0;
  std::vector<int> row_ptr, cols, plane_ptr;
  std::vector<double> vals, b, x0, planes;
};

namespace beamgen {

inline uint64_t hash64(uint64_t x) {  // splitmix64 finalizer
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
// Uniform in (0, 1]: 53 hash bits of (seed, stream, index).
inline double uniform01(uint64_t seed, uint64_t stream, uint64_t i) {
  const uint64_t h = hash64(hash64(seed ^ (stream * 0xD1B54A32D192ED03ull)) + i);
  return ((double)(h >> 11) + 1.0) * 0x1.0p-53;
}
// Standard normal by Box-Muller from two uniforms.
inline double normal(uint64_t seed, uint64_t stream, uint64_t i) {
  const double r = std::sqrt(-2.0 * std::log(uniform01(seed, stream, 2 * i)));
  return r * std::cos(6.283185307179586 * uniform01(seed, stream, 2 * i + 1));
}

// Unit normal on the cap within max_tilt of +y, cos(theta) uniform.
inline void cap_normal(double max_tilt, double u_cos, double u_phi, double n[3]) {
  const double cmin = std::cos(max_tilt);
  const double ny = cmin + (1.0 - cmin) * u_cos;
  const double phi = 6.283185307179586 * u_phi;
  const double r = std::sqrt(std::max(0.0, 1.0 - ny * ny));
  n[0] = r * std::cos(phi);
  n[1] = ny;
  n[2] = r * std::sin(phi);
}

inline bool spec_ok(const BeamSpec &s) {
  return s.a > 0 && s.b > 0 && s.c > 0 && s.edge > 0 && s.rho > 0 && s.poisson < 0.5 &&
         s.planes_min >= 0 && s.planes_max >= s.planes_min && s.planes_max <= 2 &&
         s.band >= 0.0 && s.max_tilt >= 0.0 && s.max_tilt <= 1.5707963267948966 &&
         (double)(s.a + 1) * (s.b + 1) * (s.c + 1) < 2.0e8;
}

// Corner offsets of Kuhn tet t of a cube: (0,0,0), then one, two and three
// unit steps along the axes in the order of permutation t, ending at (1,1,1).
inline void kuhn_corners(int t, int o[4][3]) {
  static const int order[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2},
                                  {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  for (int q = 0; q < 4; ++q)
    for (int d = 0; d < 3; ++d) o[q][d] = q == 3 ? 1 : 0;
  o[1][order[t][0]] = 1;
  o[2][order[t][0]] = 1;
  o[2][order[t][1]] = 1;
}

// Global planes of modes 0 and 2, each cutting `lift * active_frac` into the
// deepest vertex of x0.
inline std::vector<std::array<double, 4>> global_planes(const BeamSpec &s,
                                                        const std::vector<double> &x0) {
  std::vector<std::array<double, 4>> out;
  const int span = s.planes_max - s.planes_min + 1;
  const int count = std::min(s.planes_min + (int)(uniform01(s.seed, 11, 0) * span), s.planes_max);
  const size_t nv = x0.size() / 3;
  for (int t = 0; t < count; ++t) {
    double n[3];
    if (s.mode == 2) {  // walls x >= .., z >= ..
      n[0] = t == 0 ? 1.0 : 0.0;
      n[1] = 0.0;
      n[2] = t == 0 ? 0.0 : 1.0;
    } else {
      cap_normal(s.max_tilt, uniform01(s.seed, 21, (uint64_t)t), uniform01(s.seed, 22, (uint64_t)t),
                 n);
    }
    double lowest = 1e300;
    for (size_t v = 0; v < nv; ++v)
      lowest = std::min(lowest, n[0] * x0[3 * v] + n[1] * x0[3 * v + 1] + n[2] * x0[3 * v + 2]);
    const double depth = s.lift * std::min(1.0, std::max(0.0, s.active_frac));
    out.push_back({n[0], n[1], n[2], -(lowest + depth)});
  }
  return out;
}

// Mode 1: the number of contact facets of vertex v.
inline int facets_of(const BeamSpec &s, int v) {
  const int nx = s.a + 1, ny = s.b + 1;
  if ((v / nx) % ny >= s.facet_layers) return 0;
  if (uniform01(s.seed, 31, (uint64_t)v) > s.active_frac) return 0;
  const int span = s.planes_max - s.planes_min + 1;
  return std::min(s.planes_min + (int)(uniform01(s.seed, 32, (uint64_t)v) * span), s.planes_max);
}

}  // namespace beamgen

// Builds the beam QP of spec s.  Returns false for an invalid spec.
inline bool build_beam(const BeamSpec &s, BeamQPData &q) {
  using namespace beamgen;
  if (!spec_ok(s)) return false;
  const int nx = s.a + 1, ny = s.b + 1, nz = s.c + 1;
  const int nv = nx * ny * nz;
  q.nv = nv;
  auto vid = [&](int i, int j, int k) { return i + nx * (j + ny * k); };
  auto rest = [&](int v, int d) {
    const int idx = d == 0 ? v % nx : d == 1 ? (v / nx) % ny : v / (nx * ny);
    return idx * s.edge;
  };
  // Block pattern: the vertex and its Kuhn-split neighbours, ascending.
  static const int nbr[15][3] = {{0, 0, 0},  {1, 0, 0},   {-1, 0, 0}, {0, 1, 0},   {0, -1, 0},
                                 {0, 0, 1},  {0, 0, -1},  {1, 1, 0},  {-1, -1, 0}, {1, 0, 1},
                                 {-1, 0, -1}, {0, 1, 1},  {0, -1, -1}, {1, 1, 1},  {-1, -1, -1}};
  q.row_ptr.assign(nv + 1, 0);
  q.cols.clear();
  for (int v = 0; v < nv; ++v) {
    const int i = v % nx, j = (v / nx) % ny, k = v / (nx * ny);
    std::vector<int> row;
    for (const auto &o : nbr) {
      const int ii = i + o[0], jj = j + o[1], kk = k + o[2];
      if (ii >= 0 && jj >= 0 && kk >= 0 && ii < nx && jj < ny && kk < nz)
        row.push_back(vid(ii, jj, kk));
    }
    std::sort(row.begin(), row.end());
    q.cols.insert(q.cols.end(), row.begin(), row.end());
    q.row_ptr[v + 1] = (int)q.cols.size();
  }
  q.vals.assign(9 * q.cols.size(), 0.0);
  auto blk = [&](int r, int col) {
    const int *lo = q.cols.data() + q.row_ptr[r], *hi = q.cols.data() + q.row_ptr[r + 1];
    return q.vals.data() + 9 * (std::lower_bound(lo, hi, col) - q.cols.data());
  };

  // Element matrices: one per Kuhn permutation (the grid is uniform).
  const double lam = s.poisson * s.young / ((1.0 + s.poisson) * (1.0 - 2.0 * s.poisson));
  const double mu = s.young / (2.0 * (1.0 + s.poisson));
  const double h2 = s.dt * s.dt;
  double Ke[6][12][12], vol[6];
  int corner[6][4][3];
  for (int t = 0; t < 6; ++t) {
    kuhn_corners(t, corner[t]);
    double E[3][3];  // edge vectors x_q - x_0 as columns
    for (int q3 = 1; q3 < 4; ++q3)
      for (int d = 0; d < 3; ++d) E[d][q3 - 1] = (corner[t][q3][d] - corner[t][0][d]) * s.edge;
    const double det = E[0][0] * (E[1][1] * E[2][2] - E[1][2] * E[2][1]) -
                       E[0][1] * (E[1][0] * E[2][2] - E[1][2] * E[2][0]) +
                       E[0][2] * (E[1][0] * E[2][1] - E[1][1] * E[2][0]);
    // rows of E^-1 (adjugate / det) are the gradients of shape functions 1..3
    double G[4][3];
    G[1][0] = (E[1][1] * E[2][2] - E[1][2] * E[2][1]) / det;
    G[1][1] = (E[0][2] * E[2][1] - E[0][1] * E[2][2]) / det;
    G[1][2] = (E[0][1] * E[1][2] - E[0][2] * E[1][1]) / det;
    G[2][0] = (E[1][2] * E[2][0] - E[1][0] * E[2][2]) / det;
    G[2][1] = (E[0][0] * E[2][2] - E[0][2] * E[2][0]) / det;
    G[2][2] = (E[0][2] * E[1][0] - E[0][0] * E[1][2]) / det;
    G[3][0] = (E[1][0] * E[2][1] - E[1][1] * E[2][0]) / det;
    G[3][1] = (E[0][1] * E[2][0] - E[0][0] * E[2][1]) / det;
    G[3][2] = (E[0][0] * E[1][1] - E[0][1] * E[1][0]) / det;
    for (int d = 0; d < 3; ++d) G[0][d] = -(G[1][d] + G[2][d] + G[3][d]);
    const double V = std::fabs(det) / 6.0;
    vol[t] = V;
    // linear elasticity: K_ab[i][j] = V (lam Ga_i Gb_j + mu Ga_j Gb_i + mu Ga.Gb delta_ij)
    for (int qa = 0; qa < 4; ++qa)
      for (int qb = 0; qb < 4; ++qb) {
        const double gg = G[qa][0] * G[qb][0] + G[qa][1] * G[qb][1] + G[qa][2] * G[qb][2];
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j)
            Ke[t][3 * qa + i][3 * qb + j] =
                V * (lam * G[qa][i] * G[qb][j] + mu * G[qa][j] * G[qb][i] + (i == j ? mu * gg : 0.0));
      }
  }
  // Assembly, cube by cube (x fastest), tet by tet: mass, h^2 K and K X.
  std::vector<double> mass(nv, 0.0), KX(3 * (size_t)nv, 0.0);
  for (int k = 0; k < s.c; ++k)
    for (int j = 0; j < s.b; ++j)
      for (int i = 0; i < s.a; ++i)
        for (int t = 0; t < 6; ++t) {
          int id[4];
          for (int qa = 0; qa < 4; ++qa)
            id[qa] = vid(i + corner[t][qa][0], j + corner[t][qa][1], k + corner[t][qa][2]);
          for (int qa = 0; qa < 4; ++qa) {
            mass[id[qa]] += s.rho * vol[t] / 4.0;
            for (int qb = 0; qb < 4; ++qb) {
              double *B = blk(id[qa], id[qb]);
              for (int r = 0; r < 3; ++r)
                for (int cc = 0; cc < 3; ++cc) {
                  const double kv = Ke[t][3 * qa + r][3 * qb + cc];
                  B[3 * r + cc] += h2 * kv;
                  KX[3 * (size_t)id[qa] + r] += kv * rest(id[qb], cc);
                }
            }
          }
        }
  for (int v = 0; v < nv; ++v) {
    double *B = blk(v, v);
    for (int d = 0; d < 3; ++d) B[4 * d] += mass[v];
  }
  q.x0.assign(3 * (size_t)nv, 0.0);
  q.b.assign(3 * (size_t)nv, 0.0);
  for (int v = 0; v < nv; ++v)
    for (int d = 0; d < 3; ++d) {
      const size_t r = 3 * (size_t)v + d;
      const double x = rest(v, d) + (d == 1 ? -s.lift : 0.0);
      const double vel = s.v0_sigma * normal(s.seed, 7, (uint64_t)r);
      q.x0[r] = x;
      q.b[r] = mass[v] * (x + s.dt * vel) + h2 * mass[v] * (d == 1 ? s.gravity : 0.0) + h2 * KX[r];
    }
  // Constraints: the floor, then the global planes within `band` of the
  // vertex at x0 (modes 0, 2) or the vertex's contact facets (mode 1).
  std::vector<std::array<double, 4>> gp;
  if (s.mode != 1) gp = global_planes(s, q.x0);
  q.plane_ptr.assign(nv + 1, 0);
  q.planes.clear();
  for (int v = 0; v < nv; ++v) {
    const double *xv = q.x0.data() + 3 * (size_t)v;
    q.planes.insert(q.planes.end(), {0.0, 1.0, 0.0, 0.0});
    if (s.mode != 1) {
      for (const auto &P : gp)
        if (P[0] * xv[0] + P[1] * xv[1] + P[2] * xv[2] + P[3] < s.band)
          q.planes.insert(q.planes.end(), {P[0], P[1], P[2], P[3]});
    } else {
      for (int t = 0, e = facets_of(s, v); t < e; ++t) {
        const uint64_t key = 4ull * (uint64_t)v + (uint64_t)t;
        double n[3];
        cap_normal(s.max_tilt, uniform01(s.seed, 33, key), uniform01(s.seed, 34, key), n);
        const double y0 = std::max(0.0, xv[1]);  // through x0 lifted onto the floor
        q.planes.insert(q.planes.end(), {n[0], n[1], n[2], -(n[0] * xv[0] + n[1] * y0 + n[2] * xv[2])});
      }
    }
    q.plane_ptr[v + 1] = (int)(q.planes.size() / 4);
  }
  return true;
}

}  // namespace oracle
