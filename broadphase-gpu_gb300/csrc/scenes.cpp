// scenes.cpp - deterministic synthetic collision scenes (host C++).
// See scenes.h for the scene shapes; nothing here touches the GPU.
#include "scenes.h"

#include <cmath>
#include <cstring>
#include <vector>

namespace {

struct Rng {
  uint64_t s[4];
  explicit Rng(uint64_t seed) {
    uint64_t x = seed;
    for (int i = 0; i < 4; ++i) s[i] = x = stq_splitmix64(x);
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {  // xoshiro256**
    const uint64_t r = rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  // uniform in [0, 1) with 53 random bits
  double uniform() { return double(next() >> 11) * 0x1.0p-53; }
  double uniform(double a, double b) { return a + (b - a) * uniform(); }
  double normal() {  // Box-Muller, first variate
    double u1 = 1.0 - uniform();  // (0, 1]
    double u2 = uniform();
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  }
};

struct Grid {
  int64_t nV, nE, nF;
};

Grid grid_counts(int g) {
  const int64_t m = g - 1;
  return Grid{int64_t(g) * g, 3 * m * m + 2 * m, 2 * m * m};
}

// Topology of one g x g sheet whose first vertex has global index `base`.
// Vertex (r, c) = base + r*g + c at (x, y) = (c, r) / (g - 1).
void grid_topology(int g, int32_t base, int32_t *E, int32_t *F) {
  int64_t e = 0, f = 0;
  auto vid = [&](int r, int c) { return int32_t(base + r * g + c); };
  for (int r = 0; r < g; ++r)  // along x
    for (int c = 0; c + 1 < g; ++c) {
      E[2 * e] = vid(r, c);
      E[2 * e + 1] = vid(r, c + 1);
      ++e;
    }
  for (int r = 0; r + 1 < g; ++r)  // along y
    for (int c = 0; c < g; ++c) {
      E[2 * e] = vid(r, c);
      E[2 * e + 1] = vid(r + 1, c);
      ++e;
    }
  for (int r = 0; r + 1 < g; ++r)  // cell diagonals
    for (int c = 0; c + 1 < g; ++c) {
      E[2 * e] = vid(r, c);
      E[2 * e + 1] = vid(r + 1, c + 1);
      ++e;
    }
  for (int r = 0; r + 1 < g; ++r)
    for (int c = 0; c + 1 < g; ++c) {
      const int32_t a = vid(r, c), b = vid(r, c + 1), cc = vid(r + 1, c),
                    d = vid(r + 1, c + 1);
      F[3 * f] = a, F[3 * f + 1] = b, F[3 * f + 2] = d;
      ++f;
      F[3 * f] = a, F[3 * f + 1] = d, F[3 * f + 2] = cc;
      ++f;
    }
}

// Smoothly interpolated lattice noise in [-1, 1] at frequency `freq`.
struct ValueNoise {
  int freq;
  std::vector<double> lattice;  // (freq+1)^2 values
  ValueNoise(int f, Rng &rng) : freq(f), lattice((f + 1) * (f + 1)) {
    for (double &v : lattice) v = rng.uniform(-1.0, 1.0);
  }
  static double fade(double t) { return t * t * (3.0 - 2.0 * t); }
  double at(double x, double y) const {
    double fx = x * freq, fy = y * freq;
    int ix = int(std::floor(fx)), iy = int(std::floor(fy));
    if (ix >= freq) ix = freq - 1;
    if (iy >= freq) iy = freq - 1;
    if (ix < 0) ix = 0;
    if (iy < 0) iy = 0;
    double tx = fade(fx - ix), ty = fade(fy - iy);
    auto L = [&](int i, int j) { return lattice[j * (freq + 1) + i]; };
    double a = L(ix, iy) + (L(ix + 1, iy) - L(ix, iy)) * tx;
    double b = L(ix, iy + 1) + (L(ix + 1, iy + 1) - L(ix, iy + 1)) * tx;
    return a + (b - a) * ty;
  }
};

}  // namespace

extern "C" {

uint64_t stq_splitmix64(uint64_t x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

void stq_grid_counts(int g, int64_t *nV, int64_t *nE, int64_t *nF) {
  Grid c = grid_counts(g);
  *nV = c.nV, *nE = c.nE, *nF = c.nF;
}

int stq_cloth_pair_grid_for(int64_t boxes) {
  int g = 2;
  while (true) {
    Grid c = grid_counts(g + 1);
    if (2 * (c.nV + c.nE + c.nF) > boxes) break;
    ++g;
  }
  // pick the closer of g and g + 1
  Grid a = grid_counts(g), b = grid_counts(g + 1);
  int64_t na = 2 * (a.nV + a.nE + a.nF), nb = 2 * (b.nV + b.nE + b.nF);
  return (boxes - na <= nb - boxes) ? g : g + 1;
}

void stq_scene_cloth_pair(int g, double z_offset, double angle_deg,
                          double sigma, uint64_t seed, double *V0, double *V1,
                          int32_t *E, int32_t *F) {
  const Grid c = grid_counts(g);
  const double pi = 3.141592653589793;
  const double th = angle_deg * pi / 180.0, ct = std::cos(th), st = std::sin(th);
  for (int sheet = 0; sheet < 2; ++sheet) {
    double *P = V0 + 3 * c.nV * sheet;
    for (int r = 0; r < g; ++r)
      for (int col = 0; col < g; ++col) {
        const double x = double(col) / (g - 1), y = double(r) / (g - 1);
        const double z = 0.02 * std::sin(2 * pi * 3 * x) * std::cos(2 * pi * 2 * y);
        double *p = P + 3 * (int64_t(r) * g + col);
        if (sheet == 0) {
          p[0] = x, p[1] = y, p[2] = z;
        } else {  // rotate about z around the sheet centre, lift by z_offset
          const double dx = x - 0.5, dy = y - 0.5;
          p[0] = 0.5 + ct * dx - st * dy;
          p[1] = 0.5 + st * dx + ct * dy;
          p[2] = z + z_offset;
        }
      }
    grid_topology(g, int32_t(c.nV * sheet), E + 2 * c.nE * sheet,
                  F + 3 * c.nF * sheet);
  }
  Rng rng(seed);
  for (int64_t i = 0; i < 3 * 2 * c.nV; ++i) V1[i] = V0[i] + sigma * rng.normal();
}

void stq_scene_crumpled(int sheets, int g, double amp, double sigma,
                        uint64_t seed, double *V0, double *V1, int32_t *E,
                        int32_t *F) {
  const Grid c = grid_counts(g);
  Rng rng(seed);
  for (int s = 0; s < sheets; ++s) {
    ValueNoise n1(4, rng), n2(8, rng), n3(16, rng);
    // uniform random rotation from a normalised Gaussian quaternion
    double q[4], qn = 0;
    for (double &v : q) v = rng.normal(), qn += v * v;
    qn = std::sqrt(qn);
    for (double &v : q) v /= qn;
    const double w = q[0], x = q[1], y = q[2], z = q[3];
    const double R[9] = {1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y),
                         2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
                         2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)};
    double t[3];
    for (double &v : t) v = rng.uniform(0.5, 1.0);
    double *P = V0 + 3 * c.nV * s;
    for (int r = 0; r < g; ++r)
      for (int col = 0; col < g; ++col) {
        const double u = double(col) / (g - 1), v = double(r) / (g - 1);
        const double h = amp * (n1.at(u, v) + 0.5 * n2.at(u, v) + 0.25 * n3.at(u, v)) / 1.75;
        const double l[3] = {u - 0.5, v - 0.5, h};
        double *p = P + 3 * (int64_t(r) * g + col);
        for (int k = 0; k < 3; ++k)
          p[k] = t[k] + R[3 * k] * l[0] + R[3 * k + 1] * l[1] + R[3 * k + 2] * l[2];
      }
    grid_topology(g, int32_t(c.nV * s), E + 2 * c.nE * s, F + 3 * c.nF * s);
  }
  for (int64_t i = 0; i < 3 * sheets * c.nV; ++i) V1[i] = V0[i] + sigma * rng.normal();
}

void stq_scene_step(int64_t nV, double sigma, uint64_t seed, double *V0,
                    double *V1) {
  Rng rng(seed);
  for (int64_t i = 0; i < 3 * nV; ++i) {
    V0[i] = V1[i];
    V1[i] = V1[i] + sigma * rng.normal();
  }
}

void stq_scene_random_boxes(int64_t n, double sliver_frac, uint64_t seed,
                            void *boxes_out) {
  struct Box {
    int32_t id;
    float min[3], max[3];
    int32_t v[3];
    int32_t ref_id;
  };
  static_assert(sizeof(Box) == 44, "box layout");
  Box *boxes = static_cast<Box *>(boxes_out);
  Rng rng(seed);
  const int64_t nverts = n / 6 > 0 ? n / 6 : 1;
  const double mu = std::log(0.002), sg = 0.5;
  for (int64_t k = 0; k < n; ++k) {
    Box &b = boxes[k];
    double ctr[3], ext[3];
    for (double &v : ctr) v = rng.uniform();
    for (double &v : ext) v = std::exp(mu + sg * rng.normal());
    if (rng.uniform() < sliver_frac) ext[rng.next() % 3] *= 200.0;
    for (int a = 0; a < 3; ++a) {
      float lo = float(ctr[a] - 0.5 * ext[a]), hi = float(ctr[a] + 0.5 * ext[a]);
      b.min[a] = std::nextafter(lo, -INFINITY);
      b.max[a] = std::nextafter(hi, INFINITY);
    }
    const int t = int(k % 6);  // 0: vertex, 1-3: edge, 4-5: face
    const int32_t a0 = int32_t(rng.next() % nverts), a1 = int32_t(rng.next() % nverts),
                  a2 = int32_t(rng.next() % nverts);
    if (t == 0) {
      b.v[0] = a0, b.v[1] = -a0 - 1, b.v[2] = -a0 - 1;
    } else if (t <= 3) {
      b.v[0] = a0, b.v[1] = a1, b.v[2] = -a0 - 1;
    } else {
      b.v[0] = a0, b.v[1] = a1, b.v[2] = a2;
    }
    b.id = int32_t(k);
    b.ref_id = int32_t(k);
  }
}

}  // extern "C"
