// Seeded synthetic inputs for the multigrid workloads: right-hand sides and
// log-normal diffusion coefficients.
//
// Both are defined as functions of POSITION, not of node or element numbering,
// so any two grid managers that build the same mesh (UG's own refinement and
// the structured generator in meshgen.cpp) assemble bit-identical systems even
// though they enumerate nodes differently.
//
//  * rhs_uniform(seed, key)  : i.i.d. uniform[-1,1] keyed by the node's integer
//                              lattice coordinates on the finest level.
//  * LogNormalField           : k(x) = exp(g(x)), g a zero-mean Gaussian field
//                              with exponential covariance var*exp(-|r|/corr),
//                              sampled by random Fourier features (Rahimi &
//                              Recht 2007): g(x) = sqrt(2 var/M) sum_m
//                              cos(w_m.x + phi_m), with w_m drawn from the
//                              covariance's spectral density (a multivariate
//                              Cauchy law with scale 1/corr) and phi_m uniform.
#pragma once
#include <cmath>
#include <cstdint>
#include <vector>

#ifdef __CUDACC__
#define UGFX_HD __host__ __device__
#else
#define UGFX_HD
#endif

namespace ugfx {

// splitmix64 (Steele, Lea, Flood 2014): a 64-bit mixing function.
UGFX_HD inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Uniform double in [0,1) from the top 53 bits.
UGFX_HD inline double u01(uint64_t z) { return double(z >> 11) * (1.0 / 9007199254740992.0); }

// Key for an integer lattice point (ix,iy,iz), each < 2^20.
UGFX_HD inline uint64_t lattice_key(int64_t ix, int64_t iy, int64_t iz) {
  return (uint64_t(ix) << 42) ^ (uint64_t(iy) << 21) ^ uint64_t(iz);
}

// i.i.d. uniform[-1,1] value attached to (seed, key).
UGFX_HD inline double rhs_uniform(uint64_t seed, uint64_t key) {
  return 2.0 * u01(mix64(mix64(seed) ^ key)) - 1.0;
}

// Sequential generator used to draw the field's features.
struct SplitMix {
  uint64_t s;
  explicit SplitMix(uint64_t seed) : s(seed) {}
  uint64_t next() { s += 0x9E3779B97F4A7C15ull; uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull; z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31); }
  double uniform() { return u01(next()); }
  // standard normal by Box-Muller (one value per call, the sine branch dropped)
  double normal() {
    double u1 = uniform(), u2 = uniform();
    if (u1 < 1e-300) u1 = 1e-300;
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  }
};

struct LogNormalField {
  int dim = 3, M = 0;
  double amp = 0.0;
  std::vector<double> w;    // M x dim frequencies
  std::vector<double> phi;  // M phases

  LogNormalField() = default;
  LogNormalField(uint64_t seed, int dim_, double corr, double var, int M_ = 256) : dim(dim_), M(M_) {
    SplitMix r(mix64(seed ^ 0x5eedf1e1dull));
    w.resize(size_t(M) * dim);
    phi.resize(M);
    for (int m = 0; m < M; ++m) {
      double z0 = std::fabs(r.normal());
      if (z0 < 1e-12) z0 = 1e-12;
      for (int d = 0; d < dim; ++d) w[size_t(m) * dim + d] = r.normal() / (corr * z0);
      phi[m] = 6.283185307179586 * r.uniform();
    }
    amp = std::sqrt(2.0 * var / M);
  }
  double g(const double *x) const {
    double s = 0.0;
    for (int m = 0; m < M; ++m) {
      double a = phi[m];
      for (int d = 0; d < dim; ++d) a += w[size_t(m) * dim + d] * x[d];
      s += std::cos(a);
    }
    return amp * s;
  }
  double k(const double *x) const { return M ? std::exp(g(x)) : 1.0; }
};

}  // namespace ugfx
