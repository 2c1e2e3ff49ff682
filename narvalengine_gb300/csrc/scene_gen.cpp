// Procedural scene inputs (see scene_gen.h).
//
// Simplex noise follows the published 3-D algorithm of Perlin's simplex noise as
// described by S. Gustavson, "Simplex noise demystified" (2005): skew the input onto
// the simplicial grid with F = 1/3, unskew with G = 1/6, rank the offsets to pick the
// simplex, and sum the four corner contributions (0.6 - |d|^2)^4 (g . d) with the 12
// cube-edge gradients, scaled by 32. The permutation table is a seeded shuffle.

#include "scene_gen.h"

#include <math.h>
#include <string.h>

#include <algorithm>
#include <thread>
#include <unordered_map>

namespace negen {
namespace {

uint64_t splitmix64(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

const int kGrad[12][3] = {{1, 1, 0},  {-1, 1, 0},  {1, -1, 0}, {-1, -1, 0}, {1, 0, 1},  {-1, 0, 1},
                          {1, 0, -1}, {-1, 0, -1}, {0, 1, 1},  {0, -1, 1},  {0, 1, -1}, {0, -1, -1}};

inline int fastfloor(double x) {
  double f = floor(x);
  return (int)f;
}

}  // namespace

double hash_u01(uint64_t seed, uint64_t i) {
  uint64_t s = seed ^ (i * 0xD1B54A32D192ED03ull);
  uint64_t v = splitmix64(s);
  return (double)(v >> 11) * (1.0 / 9007199254740992.0);
}

Simplex::Simplex(uint64_t seed) {
  uint8_t p[256];
  for (int i = 0; i < 256; i++) p[i] = (uint8_t)i;
  uint64_t s = seed;
  for (int i = 255; i > 0; i--) {
    int j = (int)(splitmix64(s) % (uint64_t)(i + 1));
    std::swap(p[i], p[j]);
  }
  for (int i = 0; i < 512; i++) perm[i] = p[i & 255];
}

double Simplex::noise(double xin, double yin, double zin) const {
  const double F3 = 1.0 / 3.0, G3 = 1.0 / 6.0;
  double s = (xin + yin + zin) * F3;
  int i = fastfloor(xin + s), j = fastfloor(yin + s), k = fastfloor(zin + s);
  double t = (double)(i + j + k) * G3;
  double x0 = xin - ((double)i - t), y0 = yin - ((double)j - t), z0 = zin - ((double)k - t);
  int i1, j1, k1, i2, j2, k2;
  if (x0 >= y0) {
    if (y0 >= z0) { i1 = 1; j1 = 0; k1 = 0; i2 = 1; j2 = 1; k2 = 0; }
    else if (x0 >= z0) { i1 = 1; j1 = 0; k1 = 0; i2 = 1; j2 = 0; k2 = 1; }
    else { i1 = 0; j1 = 0; k1 = 1; i2 = 1; j2 = 0; k2 = 1; }
  } else {
    if (y0 < z0) { i1 = 0; j1 = 0; k1 = 1; i2 = 0; j2 = 1; k2 = 1; }
    else if (x0 < z0) { i1 = 0; j1 = 1; k1 = 0; i2 = 0; j2 = 1; k2 = 1; }
    else { i1 = 0; j1 = 1; k1 = 0; i2 = 1; j2 = 1; k2 = 0; }
  }
  double x1 = x0 - i1 + G3, y1 = y0 - j1 + G3, z1 = z0 - k1 + G3;
  double x2 = x0 - i2 + 2.0 * G3, y2 = y0 - j2 + 2.0 * G3, z2 = z0 - k2 + 2.0 * G3;
  double x3 = x0 - 1.0 + 3.0 * G3, y3 = y0 - 1.0 + 3.0 * G3, z3 = z0 - 1.0 + 3.0 * G3;
  int ii = i & 255, jj = j & 255, kk = k & 255;
  int g0 = perm[ii + perm[jj + perm[kk]]] % 12;
  int g1 = perm[ii + i1 + perm[jj + j1 + perm[kk + k1]]] % 12;
  int g2 = perm[ii + i2 + perm[jj + j2 + perm[kk + k2]]] % 12;
  int g3 = perm[ii + 1 + perm[jj + 1 + perm[kk + 1]]] % 12;
  auto corner = [](int g, double x, double y, double z) {
    double t = 0.6 - x * x - y * y - z * z;
    if (t < 0) return 0.0;
    t *= t;
    return t * t * (kGrad[g][0] * x + kGrad[g][1] * y + kGrad[g][2] * z);
  };
  double n = corner(g0, x0, y0, z0) + corner(g1, x1, y1, z1) + corner(g2, x2, y2, z2) + corner(g3, x3, y3, z3);
  return 32.0 * n;
}

void fbm_grid(const uint32_t res[3], const FbmParams& p, std::vector<float>& out) {
  const uint32_t W = res[0], H = res[1], D = res[2];
  out.assign((size_t)W * H * D, 0.0f);
  Simplex sx(p.seed);
  const double cx = W * 0.5, cy = H * 0.5, cz = D * 0.5;
  auto slab = [&](uint32_t z0, uint32_t z1) {
    for (uint32_t z = z0; z < z1; z++)
      for (uint32_t y = 0; y < H; y++)
        for (uint32_t x = 0; x < W; x++) {
          double px = x + 0.5, py = y + 0.5, pz = z + 0.5;
          double dx = px - cx, dy = py - cy, dz = pz - cz;
          double r = sqrt(dx * dx + dy * dy + dz * dz);
          double fall = 1.0 - r / p.falloff_radius;
          float v = 0.0f;
          if (fall > 0.0) {
            double sum = 0.0, amp = 1.0, f = p.frequency;
            for (int o = 0; o < p.octaves; o++) {
              sum += amp * sx.noise(px * f, py * f, pz * f);
              amp *= p.gain;
              f *= p.lacunarity;
            }
            if (sum < 0.0) sum = 0.0;
            v = (float)(sum * fall);
          }
          out[((size_t)z * H + y) * W + x] = v;
        }
  };
  unsigned nt = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
  if ((size_t)W * H * D < (1u << 18)) nt = 1;
  std::vector<std::thread> ts;
  uint32_t per = (D + nt - 1) / nt;
  for (unsigned t = 0; t < nt; t++) {
    uint32_t a = t * per, b = std::min(D, a + per);
    if (a >= b) break;
    ts.emplace_back(slab, a, b);
  }
  for (auto& t : ts) t.join();
}

void icosphere(const IcoParams& p, std::vector<float>& positions, std::vector<uint32_t>& indices) {
  const double phi = (1.0 + sqrt(5.0)) / 2.0;
  std::vector<double> v = {-1, phi, 0, 1, phi, 0, -1, -phi, 0, 1, -phi, 0, 0, -1, phi, 0, 1, phi,
                           0, -1, -phi, 0, 1, -phi, phi, 0, -1, phi, 0, 1, -phi, 0, -1, -phi, 0, 1};
  for (size_t i = 0; i < v.size(); i += 3) {
    double l = sqrt(v[i] * v[i] + v[i + 1] * v[i + 1] + v[i + 2] * v[i + 2]);
    v[i] /= l; v[i + 1] /= l; v[i + 2] /= l;
  }
  std::vector<uint32_t> f = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4, 11, 10, 2, 10, 7, 6,
                             7, 1, 8, 3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8, 3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6, 7,
                             9, 8, 1};
  for (int s = 0; s < p.subdivisions; s++) {
    std::unordered_map<uint64_t, uint32_t> mid;
    mid.reserve(f.size());
    std::vector<uint32_t> nf;
    nf.reserve(f.size() * 4);
    auto midpoint = [&](uint32_t a, uint32_t b) {
      uint64_t key = a < b ? ((uint64_t)a << 32 | b) : ((uint64_t)b << 32 | a);
      auto it = mid.find(key);
      if (it != mid.end()) return it->second;
      double x = (v[3 * a] + v[3 * b]) * 0.5, y = (v[3 * a + 1] + v[3 * b + 1]) * 0.5, z = (v[3 * a + 2] + v[3 * b + 2]) * 0.5;
      double l = sqrt(x * x + y * y + z * z);
      v.push_back(x / l); v.push_back(y / l); v.push_back(z / l);
      uint32_t id = (uint32_t)(v.size() / 3 - 1);
      mid.emplace(key, id);
      return id;
    };
    for (size_t i = 0; i < f.size(); i += 3) {
      uint32_t a = f[i], b = f[i + 1], c = f[i + 2];
      uint32_t ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
      uint32_t t[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
      nf.insert(nf.end(), t, t + 12);
    }
    f.swap(nf);
  }
  Simplex sx(p.seed);
  positions.resize(v.size());
  for (size_t i = 0; i < v.size(); i += 3) {
    double r = 1.0;
    if (p.amplitude != 0.0) r = 1.0 + p.amplitude * sx.noise(v[i] * p.frequency, v[i + 1] * p.frequency, v[i + 2] * p.frequency);
    positions[i] = (float)(v[i] * r);
    positions[i + 1] = (float)(v[i + 1] * r);
    positions[i + 2] = (float)(v[i + 2] * r);
  }
  indices = f;
}

}  // namespace negen
