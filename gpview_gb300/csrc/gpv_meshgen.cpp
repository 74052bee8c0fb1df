// gpv_meshgen.cpp -- seeded synthetic closed meshes (UV-sphere, noisy torus, Y_lm star,
// superellipsoid) with the shapes of the benchmark workloads.  Host code only, plain C++ with no
// CUDA: it is compiled into libgpview.so (the gpv_gen_* entry points of include/gpview.h) and, from
// this same file, into the CPU oracle's library, so that a CPU-only process (the reference arm of
// the benchmark) generates bit-identical inputs without loading the GPU library.  Every value is
// computed in double with the C library's math functions and rounded to float once.
#include <cmath>
#include <cstdint>
#include <unordered_map>
#include <vector>

#ifdef GPV_MESHGEN_ORACLE
// Built into the CPU oracle's library: the same functions under orc_gen_* names, so a process
// that loads both libraries never confuses the two.
#define GPV_GEN(name) orc_gen_##name
extern "C" {
int64_t orc_gen_uvsphere(uint64_t, int32_t, int32_t, const float *, float, float, float *);
int64_t orc_gen_torus(uint64_t, int32_t, int32_t, const float *, float, float, float, float *);
int64_t orc_gen_star(uint64_t, int32_t, const float *, float, float, const float *, float *);
int64_t orc_gen_superellipsoid(uint64_t, int32_t, int32_t, const float *, const float *, float,
                               float, const float *, float *);
}
#else
#include "../../include/gpview.h"
#define GPV_GEN(name) gpv_gen_##name
#endif

namespace {
// ---- random numbers ------------------------------------------------------------------------------
struct Rng {
  uint64_t s[4];
  static uint64_t splitmix(uint64_t &x) {
    uint64_t z = (x += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
  }
  explicit Rng(uint64_t seed) {
    for (int i = 0; i < 4; ++i) s[i] = splitmix(seed);
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {  // xoshiro256**
    const uint64_t r = rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  double normal() {  // Marsaglia polar method
    for (;;) {
      double u = 2.0 * uniform() - 1.0, v = 2.0 * uniform() - 1.0;
      double q = u * u + v * v;
      if (q > 0.0 && q < 1.0) return u * std::sqrt(-2.0 * std::log(q) / q);
    }
  }
};

void emit_tri(float *out, int64_t t, const float *a, const float *b, const float *c) {
  float *o = out + 9 * t;
  for (int k = 0; k < 3; ++k) { o[k] = a[k]; o[3 + k] = b[k]; o[6 + k] = c[k]; }
}

// UV grid with single pole vertices: ring j (1..nlat-1) has nlon vertices; pole 0 (top) and
// pole 1 (bottom) are separate.  Writes 2*nlon*(nlat-1) triangles from a vertex array laid out
// as [top, bottom, ring1..., ring(nlat-1)...].
int64_t emit_uv_mesh(const std::vector<float> &P, int nlon, int nlat, float *tris) {
  const int64_t T = 2ll * nlon * (nlat - 1);
  if (!tris) return T;
  auto ring = [&](int j, int i) -> const float * {
    return &P[3 * (2 + (size_t)(j - 1) * nlon + (size_t)(i % nlon))];
  };
  const float *top = &P[0], *bot = &P[3];
  int64_t t = 0;
  for (int i = 0; i < nlon; ++i) emit_tri(tris, t++, top, ring(1, i), ring(1, i + 1));
  for (int j = 1; j < nlat - 1; ++j)
    for (int i = 0; i < nlon; ++i) {
      emit_tri(tris, t++, ring(j, i), ring(j + 1, i), ring(j + 1, i + 1));
      emit_tri(tris, t++, ring(j, i), ring(j + 1, i + 1), ring(j, i + 1));
    }
  for (int i = 0; i < nlon; ++i) emit_tri(tris, t++, bot, ring(nlat - 1, i + 1), ring(nlat - 1, i));
  return t;
}

// 3-D value noise: hashed lattice values in [-1,1], smoothstep trilinear interpolation.
struct ValueNoise {
  uint64_t seed;
  double lattice(int64_t x, int64_t y, int64_t z) const {
    uint64_t h = seed ^ ((uint64_t)x * 0x9e3779b97f4a7c15ull) ^ ((uint64_t)y * 0xc2b2ae3d27d4eb4full) ^
                 ((uint64_t)z * 0x165667b19e3779f9ull);
    uint64_t k = h;
    h = Rng::splitmix(k);
    return (double)(h >> 11) * (2.0 / 9007199254740992.0) - 1.0;
  }
  static double fade(double t) { return t * t * (3.0 - 2.0 * t); }
  double eval(double x, double y, double z) const {
    double fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
    int64_t ix = (int64_t)fx, iy = (int64_t)fy, iz = (int64_t)fz;
    double tx = fade(x - fx), ty = fade(y - fy), tz = fade(z - fz);
    double c[2][2][2];
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 2; ++b)
        for (int d = 0; d < 2; ++d) c[a][b][d] = lattice(ix + a, iy + b, iz + d);
    double x00 = c[0][0][0] + (c[1][0][0] - c[0][0][0]) * tx;
    double x10 = c[0][1][0] + (c[1][1][0] - c[0][1][0]) * tx;
    double x01 = c[0][0][1] + (c[1][0][1] - c[0][0][1]) * tx;
    double x11 = c[0][1][1] + (c[1][1][1] - c[0][1][1]) * tx;
    double y0 = x00 + (x10 - x00) * ty, y1 = x01 + (x11 - x01) * ty;
    return y0 + (y1 - y0) * tz;
  }
  double fbm(double x, double y, double z, int octaves) const {
    double sum = 0.0, amp = 1.0, norm = 0.0, f = 4.0;
    for (int o = 0; o < octaves; ++o) {
      sum += amp * eval(x * f, y * f, z * f);
      norm += amp;
      amp *= 0.5;
      f *= 2.0;
    }
    return sum / norm;
  }
};

// Real spherical harmonic Y_lm (orthonormal), l <= 6.
double real_sh(int l, int m, double theta, double phi) {
  const int am = m < 0 ? -m : m;
  const double x = std::cos(theta);
  // associated Legendre P_l^am(x) by the standard recurrences
  double pmm = 1.0;
  if (am > 0) {
    double somx2 = std::sqrt((1.0 - x) * (1.0 + x)), fact = 1.0;
    for (int i = 1; i <= am; ++i) { pmm *= -fact * somx2; fact += 2.0; }
  }
  double plm;
  if (l == am) plm = pmm;
  else {
    double pmmp1 = x * (2 * am + 1) * pmm;
    if (l == am + 1) plm = pmmp1;
    else {
      double pll = 0.0;
      for (int ll = am + 2; ll <= l; ++ll) {
        pll = ((2 * ll - 1) * x * pmmp1 - (ll + am - 1) * pmm) / (ll - am);
        pmm = pmmp1;
        pmmp1 = pll;
      }
      plm = pll;
    }
  }
  double num = 1.0, den = 1.0;
  for (int i = l - am + 1; i <= l + am; ++i) den *= i;
  (void)num;
  const double K = std::sqrt((2 * l + 1) / (4.0 * M_PI) / den);
  if (m == 0) return K * plm;
  if (m > 0) return std::sqrt(2.0) * K * std::cos(m * phi) * plm;
  return std::sqrt(2.0) * K * std::sin(am * phi) * plm;
}

}  // namespace

extern "C" {

int64_t GPV_GEN(uvsphere)(uint64_t seed, int32_t nlon, int32_t nlat, const float center[3],
                         float radius, float jitter_sigma, float *tris) {
  if (nlon < 3 || nlat < 2) return 0;
  if (!tris) return 2ll * nlon * (nlat - 1);
  Rng rng(seed);
  std::vector<float> P(3 * (2 + (size_t)nlon * (nlat - 1)));
  auto put = [&](size_t vi, double th, double ph) {
    double r = radius + (jitter_sigma > 0 ? jitter_sigma * rng.normal() : 0.0);
    P[3 * vi + 0] = (float)(center[0] + r * std::sin(th) * std::cos(ph));
    P[3 * vi + 1] = (float)(center[1] + r * std::sin(th) * std::sin(ph));
    P[3 * vi + 2] = (float)(center[2] + r * std::cos(th));
  };
  put(0, 0.0, 0.0);
  put(1, M_PI, 0.0);
  for (int j = 1; j < nlat; ++j)
    for (int i = 0; i < nlon; ++i)
      put(2 + (size_t)(j - 1) * nlon + i, M_PI * j / nlat, 2.0 * M_PI * i / nlon);
  return emit_uv_mesh(P, nlon, nlat, tris);
}

int64_t GPV_GEN(torus)(uint64_t seed, int32_t nu, int32_t nv, const float center[3], float R,
                      float r, float noise_amp, float *tris) {
  if (nu < 3 || nv < 3) return 0;
  const int64_t T = 2ll * nu * nv;
  if (!tris) return T;
  ValueNoise vn{Rng(seed).next()};
  std::vector<float> P(3 * (size_t)nu * nv);
  for (int a = 0; a < nu; ++a)
    for (int b = 0; b < nv; ++b) {
      double A = 2.0 * M_PI * a / nu, Bq = 2.0 * M_PI * b / nv;
      double nx = std::cos(Bq) * std::cos(A), ny = std::cos(Bq) * std::sin(A), nz = std::sin(Bq);
      double px = (R + r * std::cos(Bq)) * std::cos(A), py = (R + r * std::cos(Bq)) * std::sin(A),
             pz = r * std::sin(Bq);
      double d = noise_amp * vn.fbm(px + 1.7, py + 2.3, pz + 3.1, 4);
      size_t vi = (size_t)a * nv + b;
      P[3 * vi + 0] = (float)(center[0] + px + d * nx);
      P[3 * vi + 1] = (float)(center[1] + py + d * ny);
      P[3 * vi + 2] = (float)(center[2] + pz + d * nz);
    }
  int64_t t = 0;
  for (int a = 0; a < nu; ++a)
    for (int b = 0; b < nv; ++b) {
      const float *p00 = &P[3 * ((size_t)a * nv + b)];
      const float *p10 = &P[3 * ((size_t)((a + 1) % nu) * nv + b)];
      const float *p11 = &P[3 * ((size_t)((a + 1) % nu) * nv + (b + 1) % nv)];
      const float *p01 = &P[3 * ((size_t)a * nv + (b + 1) % nv)];
      emit_tri(tris, t++, p00, p10, p11);
      emit_tri(tris, t++, p00, p11, p01);
    }
  return t;
}

int64_t GPV_GEN(star)(uint64_t seed, int32_t subdiv, const float center[3], float radius,
                     float amp, const float scale[3], float *tris) {
  if (subdiv < 0 || subdiv > 10) return 0;
  int64_t T = 20;
  for (int s = 0; s < subdiv; ++s) T *= 4;
  if (!tris) return T;
  // icosahedron
  const double ph = (1.0 + std::sqrt(5.0)) / 2.0;
  std::vector<double> V = {-1, ph, 0, 1, ph, 0, -1, -ph, 0, 1, -ph, 0, 0, -1, ph, 0, 1, ph,
                           0, -1, -ph, 0, 1, -ph, ph, 0, -1, ph, 0, 1, -ph, 0, -1, -ph, 0, 1};
  for (size_t i = 0; i < V.size(); i += 3) {
    double n = std::sqrt(V[i] * V[i] + V[i + 1] * V[i + 1] + V[i + 2] * V[i + 2]);
    V[i] /= n; V[i + 1] /= n; V[i + 2] /= n;
  }
  std::vector<int32_t> F = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4,
                            11, 10, 2, 10, 7, 6, 7, 1, 8, 3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8,
                            3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6, 7, 9, 8, 1};
  for (int s = 0; s < subdiv; ++s) {
    std::unordered_map<uint64_t, int32_t> mid;
    mid.reserve(F.size());
    std::vector<int32_t> NF;
    NF.reserve(F.size() * 4);
    auto midpoint = [&](int32_t a, int32_t b) -> int32_t {
      uint64_t key = a < b ? ((uint64_t)a << 32 | (uint32_t)b) : ((uint64_t)b << 32 | (uint32_t)a);
      auto it = mid.find(key);
      if (it != mid.end()) return it->second;
      double x = V[3 * a] + V[3 * b], y = V[3 * a + 1] + V[3 * b + 1], z = V[3 * a + 2] + V[3 * b + 2];
      double n = std::sqrt(x * x + y * y + z * z);
      int32_t id = (int32_t)(V.size() / 3);
      V.push_back(x / n); V.push_back(y / n); V.push_back(z / n);
      mid.emplace(key, id);
      return id;
    };
    for (size_t f = 0; f < F.size(); f += 3) {
      int32_t a = F[f], b = F[f + 1], c = F[f + 2];
      int32_t ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
      int32_t nf[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
      NF.insert(NF.end(), nf, nf + 12);
    }
    F.swap(NF);
  }
  // star-shaped radius r = radius * (1 + amp * sum a_lm Y_lm), a_lm ~ N(0, 1/l^2), l = 1..6
  Rng rng(seed);
  std::vector<double> coef;
  for (int l = 1; l <= 6; ++l)
    for (int m = -l; m <= l; ++m) coef.push_back(rng.normal() / l);
  std::vector<float> P(V.size());
  for (size_t i = 0; i < V.size(); i += 3) {
    double x = V[i], y = V[i + 1], z = V[i + 2];
    double th = std::acos(z < -1 ? -1 : (z > 1 ? 1 : z)), phv = std::atan2(y, x);
    double s = 0.0;
    size_t c = 0;
    for (int l = 1; l <= 6; ++l)
      for (int m = -l; m <= l; ++m) s += coef[c++] * real_sh(l, m, th, phv);
    double f = 1.0 + amp * s;
    if (f < 0.25) f = 0.25;  // keeps the surface star-shaped and closed
    double r = radius * f;
    P[i] = (float)(center[0] + scale[0] * r * x);
    P[i + 1] = (float)(center[1] + scale[1] * r * y);
    P[i + 2] = (float)(center[2] + scale[2] * r * z);
  }
  int64_t t = 0;
  for (size_t f = 0; f < F.size(); f += 3)
    emit_tri(tris, t++, &P[3 * (size_t)F[f]], &P[3 * (size_t)F[f + 1]], &P[3 * (size_t)F[f + 2]]);
  return t;
}

int64_t GPV_GEN(superellipsoid)(uint64_t seed, int32_t nlon, int32_t nlat, const float center[3],
                               const float semi[3], float e1, float e2, const float rot[9],
                               float *tris) {
  (void)seed;
  if (nlon < 3 || nlat < 2) return 0;
  if (!tris) return 2ll * nlon * (nlat - 1);
  auto spow = [](double v, double e) { return (v < 0 ? -1.0 : 1.0) * std::pow(std::fabs(v), e); };
  std::vector<float> P(3 * (2 + (size_t)nlon * (nlat - 1)));
  auto put = [&](size_t vi, double eta, double om) {
    double ce = spow(std::cos(eta), e1), se = spow(std::sin(eta), e1);
    double x = semi[0] * ce * spow(std::cos(om), e2);
    double y = semi[1] * ce * spow(std::sin(om), e2);
    double z = semi[2] * se;
    for (int a = 0; a < 3; ++a)
      P[3 * vi + a] = (float)(center[a] + rot[3 * a] * x + rot[3 * a + 1] * y + rot[3 * a + 2] * z);
  };
  put(0, M_PI / 2, 0.0);
  put(1, -M_PI / 2, 0.0);
  for (int j = 1; j < nlat; ++j)
    for (int i = 0; i < nlon; ++i)
      put(2 + (size_t)(j - 1) * nlon + i, M_PI / 2 - M_PI * j / nlat, 2.0 * M_PI * i / nlon);
  return emit_uv_mesh(P, nlon, nlat, tris);
}

}  // extern "C"
