/**
 * @file synthetic_xs.h
 * @brief Seeded synthetic multigroup cross sections for the benchmark
 *        workloads (pin cells and pin lattices with 2-70 groups).
 *
 * The construction, per material:
 *   - sigma_t[g] ~ U[0.2, 1.5] /cm;
 *   - for every origin group g the total out-scatter s_g ~ U[0.3, 0.95] *
 *     sigma_t[g] is spread over destination groups with random weights that
 *     decay away from the diagonal.  Destinations are h >= g (down-scatter
 *     and self-scatter) except for origins in the up-scatter set, the last
 *     ceil(27*G/70) groups (groups 5-7 for G=7, the last 27 for G=70), whose
 *     destinations are every h >= first up-scatter group;
 *   - fuel only: nu_sigma_f[g] ~ U[0.005, 0.3] /cm, sigma_f = nu_sigma_f/2.43,
 *     chi positive on groups 1..min(3,G) and normalised to 1;
 *   - moderator: nu_sigma_f = sigma_f = chi = 0.
 * A perturbed copy multiplies sigma_t[g] and row g of the scattering matrix by
 * the same lognormal(0, sigma) factor, so the scattering row sum stays below
 * sigma_t.
 *
 * The random stream is splitmix64, so the same seed gives the same numbers
 * on every host (x86 and Arm).  Scattering is returned origin-major,
 * xs[orig*G + dest], the order Material::setSigmaS takes
 * (src/Material.cpp:721-735).
 */
#ifndef OPENMOC_GB300_SYNTHETIC_XS_H_
#define OPENMOC_GB300_SYNTHETIC_XS_H_

#include <cmath>
#include <cstdint>
#include <vector>

namespace openmoc_gb300 {

struct SplitMix64 {
  uint64_t state;
  explicit SplitMix64(uint64_t seed) : state(seed) {}
  uint64_t next() {
    uint64_t z = (state += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
  }
  /* uniform in [0, 1) with 53 random bits */
  double uniform() { return (double) (next() >> 11) * (1.0 / 9007199254740992.0); }
  double uniform(double lo, double hi) { return lo + (hi - lo) * uniform(); }
  /* standard normal by Box-Muller */
  double normal() {
    double u1 = uniform();
    double u2 = uniform();
    if (u1 < 1e-300) u1 = 1e-300;
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  }
};

struct MaterialXS {
  int num_groups = 0;
  bool fissile = false;
  std::vector<double> sigma_t;     /* [G] */
  std::vector<double> sigma_s;     /* [G*G] origin-major: [orig*G + dest] */
  std::vector<double> nu_sigma_f;  /* [G] */
  std::vector<double> sigma_f;     /* [G] */
  std::vector<double> chi;         /* [G] */
};

/** First (0-based) group of the up-scatter set for G groups. */
inline int upscatter_start(int G) {
  int n_up = (27 * G + 69) / 70;   /* ceil(27*G/70) */
  if (G == 7) n_up = 3;            /* groups 5-7 */
  if (n_up >= G) n_up = G - 1;
  if (n_up < 1) n_up = (G > 1) ? 1 : 0;
  return G - n_up;
}

inline MaterialXS make_synthetic_xs(uint64_t seed, int G, bool fissile) {
  SplitMix64 rng(seed);
  MaterialXS m;
  m.num_groups = G;
  m.fissile = fissile;
  m.sigma_t.assign(G, 0.0);
  m.sigma_s.assign((size_t) G * G, 0.0);
  m.nu_sigma_f.assign(G, 0.0);
  m.sigma_f.assign(G, 0.0);
  m.chi.assign(G, 0.0);
  for (int g = 0; g < G; g++)
    m.sigma_t[g] = rng.uniform(0.2, 1.5);
  const int up0 = upscatter_start(G);
  std::vector<double> w(G);
  for (int g = 0; g < G; g++) {
    double row = rng.uniform(0.3, 0.95) * m.sigma_t[g];
    int h0 = (g >= up0) ? up0 : g;
    double wsum = 0.0;
    for (int h = 0; h < G; h++) {
      w[h] = 0.0;
      if (h < h0) continue;
      double dist = (double) (h > g ? h - g : g - h);
      w[h] = rng.uniform(0.05, 1.0) * std::exp(-0.5 * dist);
      if (h == g) w[h] += 1.0;   /* self-scatter dominant */
      wsum += w[h];
    }
    for (int h = 0; h < G; h++)
      m.sigma_s[(size_t) g * G + h] = row * w[h] / wsum;
  }
  if (fissile) {
    for (int g = 0; g < G; g++) {
      m.nu_sigma_f[g] = rng.uniform(0.005, 0.3);
      m.sigma_f[g] = m.nu_sigma_f[g] / 2.43;
    }
    int nchi = G < 3 ? G : 3;
    double csum = 0.0;
    for (int g = 0; g < nchi; g++) {
      m.chi[g] = rng.uniform(0.1, 1.0);
      csum += m.chi[g];
    }
    for (int g = 0; g < nchi; g++)
      m.chi[g] /= csum;
  }
  return m;
}

/** Copy of m with sigma_t[g] and scattering row g scaled by one lognormal
 *  factor per group. */
inline MaterialXS perturb_xs(const MaterialXS& m, uint64_t seed, double sigma) {
  SplitMix64 rng(seed);
  MaterialXS p = m;
  const int G = m.num_groups;
  for (int g = 0; g < G; g++) {
    double f = std::exp(sigma * rng.normal());
    p.sigma_t[g] *= f;
    for (int h = 0; h < G; h++)
      p.sigma_s[(size_t) g * G + h] *= f;
  }
  return p;
}

}  // namespace openmoc_gb300

#endif
