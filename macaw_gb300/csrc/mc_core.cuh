// mc_core.cuh -- arithmetic shared by host and device code of the tracker.
//
// Every function here runs as the same sequence of IEEE-754 operations on
// the host (compiled with -ffp-contract=off) and on sm_103a (compiled with
// -fmad=false), so FP64 particle histories are reproducible bit for bit
// between the two.  No libm/libdevice transcendental is used on the FP64
// path: the natural log is evaluated from its atanh series, and angles are
// sampled by rejection instead of sin/cos.
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define MC_HD __host__ __device__ __forceinline__
#else
#define MC_HD inline
#endif

namespace mc {

#ifdef __CUDACC__
// float <-> double by integer operations, for the mixed-precision walk and
// the quotient below: on this GPU a conversion instruction issues on the
// narrow FP64 pipe, an integer operation on the full-rate ALU.  widen() is
// exact for every normal float (zero and subnormals give a signed zero);
// narrow() rounds to nearest even like a conversion for results in the
// normal float range and gives a signed zero below it (|x| < 2^-126) --
// positions, directions and cross sections never leave that range except
// through zero.
__device__ __forceinline__ double widen(float f) {
  const uint32_t b = __float_as_uint(f);
  const uint32_t e = (b >> 23) & 0xffu;
  const uint64_t sign = (uint64_t)(b & 0x80000000u) << 32;
  if (e == 0u) return __longlong_as_double((long long)sign);
  return __longlong_as_double(
      (long long)(sign | ((uint64_t)(e + 896u) << 52) | ((uint64_t)(b & 0x7fffffu) << 29)));
}

__device__ __forceinline__ float narrow(double d) {
  const uint64_t b = (uint64_t)__double_as_longlong(d);
  const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7ffu) - 896;
  if (e <= 0) return __uint_as_float(sign);
  const uint64_t m = b & 0xfffffffffffffull;
  const uint32_t lo = (uint32_t)(m & 0x1fffffffu);  // 29 dropped bits
  uint32_t r = ((uint32_t)e << 23) + (uint32_t)(m >> 29);
  if (lo > 0x10000000u || (lo == 0x10000000u && (r & 1u))) ++r;  // may carry into the exponent
  if (e >= 255) r = 0x7f800000u;
  return __uint_as_float(sign | r);
}

#endif

// num / den by Markstein's division sequence (P. Markstein, "Computation of
// elementary functions on the IBM RISC System/6000 processor", IBM J. Res.
// Dev. 34(1), 1990): the correctly rounded float reciprocal of den, one
// Newton step in FP64, and the quotient corrected by its residual.  Within
// an ulp of the IEEE quotient, in five FP64 operations, fewer than a
// division costs on this GPU's narrow FP64 pipe (the lattice's FP64 walk
// launches: 1.12 ms against 1.25 ms with divisions).  A den whose float
// lies outside [2^-100, 2^100] takes the IEEE division.  Host and device
// give the same bits: the device's narrow() rounds like the host's
// conversion in that range, and __frcp_rn is the IEEE reciprocal.  The
// oracle computes the same sequence (oracle_quotient).
MC_HD double quotient(double num, double den) {
#ifdef __CUDA_ARCH__
  const float df = narrow(den);
#else
  const float df = (float)den;
#endif
  const float da = fabsf(df);
  if (!(da >= 0x1p-100f && da <= 0x1p100f)) return num / den;
#ifdef __CUDA_ARCH__
  const double y0 = widen(__frcp_rn(df));
#else
  const double y0 = (double)(1.0f / df);
#endif
  const double y1 = fma(y0, fma(-den, y0, 1.0), y0);
  const double q0 = num * y1;
  return fma(fma(-den, q0, num), y1, q0);
}

// ---------------------------------------------------------------------------
// Random numbers.  Same scheme as OpenMC 0.13, which MaCaw drives through
// openmc::prn(p->current_seed()) (src/raykernels/CollisionKernel.C:150) and
// openmc::initialize_history (src/userobjects/OpenMCStudy.C:326): the state
// of a 64-bit LCG (multiplier 6364136223846793005, increment
// 1442695040888963407) is permuted by PCG's RXS-M-XS output function
// (O'Neill 2014); histories own disjoint stretches of the sequence, a
// stride of 152917 states per particle id, reached by Brown's (1994)
// arbitrary-stride skip-ahead; each purpose has its own stream, seeded with
// master + stream.
constexpr uint64_t kPrnMult = 6364136223846793005ULL;
constexpr uint64_t kPrnAdd = 1442695040888963407ULL;
constexpr uint64_t kPrnStride = 152917ULL;
constexpr int kStreamTracking = 0;
constexpr int kStreamSource = 2;

// k * 2^-53 for an integer k < 2^53, exactly.  On the device it is built
// from the bits (the leading one's position gives the exponent) with
// integer operations: the conversion and the multiply would issue on this
// GPU's narrow FP64 pipe, and births draw about fifteen numbers each.  Both
// forms are exact, so they give the same bits.
MC_HD double unit53(uint64_t k) {
#ifdef __CUDA_ARCH__
  if (k == 0) return 0.0;
  const int p = 63 - __clzll((long long)k);  // leading one, 0..52
  const uint64_t b = ((uint64_t)(p + 970) << 52) | ((k << (52 - p)) & 0xfffffffffffffULL);
  return __longlong_as_double((long long)b);
#else
  return (double)k * 0x1.0p-53;
#endif
}

MC_HD double prn(uint64_t& s) {
  s = kPrnMult * s + kPrnAdd;
  uint64_t w = ((s >> ((s >> 59u) + 5u)) ^ s) * 12605985483714917081ULL;
  w = (w >> 43u) ^ w;
  return unit53(w >> 11);
}

// Affine map seed -> G*seed + C equal to n steps of the LCG.
struct Skip {
  uint64_t G, C;
};

// The maps for 2^k steps, k = 0..63 (each the previous one applied twice).
struct SkipTable {
  uint64_t G[64], C[64];
};
constexpr SkipTable make_skip_table() {
  SkipTable t{};
  uint64_t g = kPrnMult, c = kPrnAdd;
  for (int k = 0; k < 64; ++k) {
    t.G[k] = g;
    t.C[k] = c;
    c = (g + 1ULL) * c;
    g = g * g;
  }
  return t;
}
#ifdef __CUDACC__
__constant__ SkipTable kSkipTable = make_skip_table();
#endif

// The maps of the LCG commute, so composing the 2^k-step maps of n's set
// bits in any order gives the same (G, C); on the device the 2^k maps come
// from the table instead of being squared up on the way.
MC_HD Skip skip_ahead(uint64_t n) {
  uint64_t G = 1, C = 0;
#ifdef __CUDA_ARCH__
  for (int k = 0; n > 0; ++k, n >>= 1) {
    if (n & 1ULL) {
      const uint64_t g = kSkipTable.G[k], c = kSkipTable.C[k];
      G = G * g;
      C = C * g + c;
    }
  }
#else
  uint64_t g = kPrnMult, c = kPrnAdd;
  while (n > 0) {
    if (n & 1ULL) {
      G = G * g;
      C = C * g + c;
    }
    c = (g + 1ULL) * c;
    g = g * g;
    n >>= 1;
  }
#endif
  return Skip{G, C};
}

MC_HD uint64_t stream_seed(const Skip& k, uint64_t master, int stream) {
  return k.G * (master + (uint64_t)stream) + k.C;
}

// ---------------------------------------------------------------------------
// Bit casts.
MC_HD uint64_t dbits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t b;
  memcpy(&b, &x, 8);
  return b;
#endif
}
MC_HD double bitsd(uint64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double x;
  memcpy(&x, &b, 8);
  return x;
#endif
}

MC_HD double dinf() { return bitsd(0x7ff0000000000000ULL); }
MC_HD double dnan() { return bitsd(0x7ff8000000000000ULL); }

// Natural log: x = 2^e * m with m in [sqrt(1/2), sqrt(2)),
// ln m = 2 atanh(f) = 2f (1 + f^2/3 + f^4/5 + ... + f^22/23), f = (m-1)/(m+1),
// |f| <= 0.1716; ln x = e*ln2_hi + (ln m + e*ln2_lo) with ln2 split so that
// e*ln2_hi is exact.  Error stays within a few ulp.
MC_HD double log64(double x) {
  if (!(x > 0.0)) {
    if (x == 0.0) return -dinf();
    return dnan();
  }
  if (x == dinf()) return x;
  uint64_t b = dbits(x);
  int e = (int)((b >> 52) & 0x7ffULL);
  if (e == 0) {
    double y = x * 18014398509481984.0;  // 2^54
    b = dbits(y);
    e = (int)((b >> 52) & 0x7ffULL) - 54;
  }
  e -= 1023;
  double m = bitsd((b & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL);
  if (m > 1.4142135623730951) {
    m = m * 0.5;
    e += 1;
  }
  // Horner steps and the final sums as fused multiply-adds (one rounding
  // each, the same in the oracle's oracle_log), the quotient by quotient()
  const double f = quotient(m - 1.0, m + 1.0);
  const double s = f * f;
  double p = 0.043478260869565216;        // 1/23
  p = fma(s, p, 0.047619047619047616);    // 1/21
  p = fma(s, p, 0.05263157894736842);     // 1/19
  p = fma(s, p, 0.058823529411764705);    // 1/17
  p = fma(s, p, 0.06666666666666667);     // 1/15
  p = fma(s, p, 0.07692307692307693);     // 1/13
  p = fma(s, p, 0.09090909090909091);     // 1/11
  p = fma(s, p, 0.1111111111111111);      // 1/9
  p = fma(s, p, 0.14285714285714285);     // 1/7
  p = fma(s, p, 0.2);                     // 1/5
  p = fma(s, p, 0.3333333333333333);      // 1/3
  p = s * p;
  const double t = 2.0 * f;
  const double r = fma(t, p, t);
  const double de = (double)e;
  return fma(de, 0.6931471803691238, fma(de, 1.9082149292705877e-10, r));
}

// exp for the host-side table generators only (not on the tracking path):
// x = k ln2 + r, |r| <= ln2/2, Taylor series of e^r to degree 14, scaled
// by 2^k through the exponent bits.
MC_HD double exp64(double x) {
  if (x != x) return x;
  if (x > 709.0) return dinf();
  if (x < -708.0) return 0.0;
  double kd = x * 1.4426950408889634;
  kd = (kd >= 0.0) ? (double)(int64_t)(kd + 0.5) : -(double)(int64_t)(-kd + 0.5);
  const double r = (x - kd * 0.6931471803691238) - kd * 1.9082149292705877e-10;
  double p = 1.0 / 87178291200.0;  // 1/14!
  p = 1.0 / 6227020800.0 + r * p;
  p = 1.0 / 479001600.0 + r * p;
  p = 1.0 / 39916800.0 + r * p;
  p = 1.0 / 3628800.0 + r * p;
  p = 1.0 / 362880.0 + r * p;
  p = 1.0 / 40320.0 + r * p;
  p = 1.0 / 5040.0 + r * p;
  p = 1.0 / 720.0 + r * p;
  p = 1.0 / 120.0 + r * p;
  p = 1.0 / 24.0 + r * p;
  p = 1.0 / 6.0 + r * p;
  p = 0.5 + r * p;
  p = 1.0 + r * p;
  p = 1.0 + r * p;
  const int64_t k = (int64_t)kd;
  // 2^k as a double (k in [-1022, 1023] here, after the range checks)
  if (k < -1020) return p * bitsd((uint64_t)(k + 1023 + 60) << 52) * 0x1.0p-60;
  return p * bitsd((uint64_t)(k + 1023) << 52);
}

MC_HD double fmax0(double a) { return a > 0.0 ? a : 0.0; }

// ---------------------------------------------------------------------------
// Sampling without sin/cos: a uniform azimuth is the doubled angle of a point
// drawn uniformly in the unit disk (von Neumann 1951); the Maxwell cos^2
// term is the squared cosine of the angle of a point in the unit quarter disk.
MC_HD void sample_azimuth(uint64_t& s, double& c, double& sn) {
  for (int it = 0; it < 10000; ++it) {
    const double a = 2.0 * prn(s) - 1.0;
    const double b = 2.0 * prn(s) - 1.0;
    const double r2 = a * a + b * b;
    if (r2 > 0.0 && r2 <= 1.0) {
      const double inv = quotient(1.0, r2);
      c = (a * a - b * b) * inv;
      sn = (2.0 * a * b) * inv;
      return;
    }
  }
  c = 1.0;  // not reached in practice: acceptance is pi/4 per try
  sn = 0.0;
}

MC_HD double sample_cos2_quarter(uint64_t& s) {
  for (int it = 0; it < 10000; ++it) {
    const double a = prn(s);
    const double b = prn(s);
    const double r2 = a * a + b * b;
    if (r2 > 0.0 && r2 <= 1.0) return quotient(a * a, r2);
  }
  return 0.5;
}

// Watt fission spectrum as a Maxwellian plus a shift (the form OpenMC's
// watt_spectrum uses), redrawn outside [E_lo, E_hi).
MC_HD double sample_watt(uint64_t& s, double a, double b, double E_lo, double E_hi) {
  for (int it = 0; it < 1000; ++it) {
    const double r1 = prn(s);
    const double r2 = prn(s);
    const double c2 = sample_cos2_quarter(s);
    const double w = -a * (mc::log64(r1) + mc::log64(r2) * c2);
    const double E = w + a * a * b / 4.0 + (2.0 * prn(s) - 1.0) * sqrt(a * a * b * w);
    if (E < E_hi && E >= E_lo) return E;
  }
  return E_hi * 0.5;
}

// Rotate direction u by polar cosine mu and azimuth (cos phi, sin phi): the
// textbook change-of-direction formula used by OpenMC's rotate_angle.
MC_HD void rotate_dir(double& u0, double& v0, double& w0, double mu, double cphi, double sphi) {
  const double u = u0, v = v0, w = w0;
  const double a = sqrt(fmax0(1.0 - mu * mu));
  double b = sqrt(fmax0(1.0 - w * w));
  if (b > 1e-10) {
    u0 = mu * u + a * (u * w * cphi - v * sphi) / b;
    v0 = mu * v + a * (v * w * cphi + u * sphi) / b;
    w0 = mu * w - a * b * cphi;
  } else {
    b = sqrt(1.0 - v * v);
    u0 = mu * u + a * (u * v * cphi + w * sphi) / b;
    v0 = mu * v - a * b * cphi;
    w0 = mu * w + a * (v * w * cphi - u * sphi) / b;
  }
}

// 2-D problems (CollisionKernel z_coord, CollisionKernel.C:60-61,200-202;
// OpenMCStudy.C:355-356): a direction loses its z component and is
// renormalised in the plane (a direction along z becomes +x).
MC_HD void planar_dir(double& u, double& v, double& w) {
  w = 0.0;
  const double n2 = u * u + v * v;
  if (n2 > 0.0) {
    const double n = sqrt(n2);
    u = u / n;
    v = v / n;
  } else {
    u = 1.0;
    v = 0.0;
  }
}

// ---------------------------------------------------------------------------
// Per-history trace hash (FNV-1a over 64-bit words).
constexpr uint64_t kFnvOffset = 14695981039346656037ULL;
constexpr uint64_t kFnvPrime = 1099511628211ULL;
MC_HD uint64_t fnv(uint64_t h, uint64_t v) { return (h ^ v) * kFnvPrime; }

// History end states.
enum Status : int {
  kAlive = 0,
  kLeaked = 1,
  kAbsorbed = 2,
  kCutoff = 3,
  kStuck = 4,
  kLost = 5,
  kBadXS = 6,
};

// Segments a history may walk before it is ended as stuck, unless the
// caller sets a limit (mc_set_segment_limit): a straight flight crosses of
// the order of cbrt(n_tet) elements, and the default allows 4096 such
// flights, at least 65,536 and at most 10,000,000 segments.
inline int64_t default_segment_limit(int64_t n_tet) {
  int64_t c = 1;
  while (c * c * c < n_tet) ++c;
  int64_t l = 4096 * c;
  return l < 65536 ? 65536 : l > 10000000 ? 10000000 : l;
}
constexpr int kMaxZeroRun = 10000;
constexpr double kLocateTol = 1e-9;

}  // namespace mc
