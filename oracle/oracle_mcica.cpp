// Test infrastructure: the oracle's restatement of McICA's stochastic cloud
// generator (mcica_subcol_gen_lw.f90 / mcica_subcol_gen_sw.f90,
// generate_stochastic_clouds[_sw]) with its two random-number generators,
// kissvec (mcica_subcol_gen_lw.f90 kissvec) and the Mersenne Twister of
// mcica_random_numbers.f90 (module MersenneTwister).  Integer arithmetic is
// the reference's 32-bit two's-complement arithmetic (MiMA builds with -i4),
// real arithmetic FP64 (-r8).  Only the tests call it.
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

// kissvec (mcica_subcol_gen_lw.f90, end of module): four 32-bit states per
// column, one draw per call; m(k, n) = ieor(k, ishft(k, n)) with a logical
// shift, the sum wrapping on 32 bits, then kiss * 2.328306e-10 + 0.5.
struct Kiss {
  uint32_t s1, s2, s3, s4;
  static uint32_t m(uint32_t k, int n) { return k ^ (n > 0 ? (k << n) : (k >> -n)); }
  double next() {
    s1 = 69069u * s1 + 1327217885u;
    s2 = m(m(m(s2, 13), -17), 5);
    s3 = 18000u * (s3 & 65535u) + (s3 >> 16);
    s4 = 30903u * (s4 & 65535u) + (s4 >> 16);
    const int32_t kiss = (int32_t)(s1 + s2 + (s3 << 16) + s4);
    return (double)kiss * 2.328306e-10 + 0.5;
  }
};

// MersenneTwister (mcica_random_numbers.f90): MT19937 with the scalar seeding
// (initialize_scalar), its twist, tempering and getRandomReal, which maps the
// signed 32-bit draw to [0, 1] as its unsigned value / (2^32 - 1).
struct Twister {
  uint32_t st[624];
  int cur = 624;
  explicit Twister(int32_t seed) {
    st[0] = (uint32_t)seed;
    for (uint32_t i = 1; i < 624; ++i) st[i] = 1812433253u * (st[i - 1] ^ (st[i - 1] >> 30)) + i;
  }
  static uint32_t twist(uint32_t u, uint32_t v) {
    const uint32_t mix = (u & 0x80000000u) | (v & 0x7fffffffu);
    return (mix >> 1) ^ ((v & 1u) ? 0x9908b0dfu : 0u);
  }
  void next_state() {
    for (int k = 0; k < 624 - 397; ++k) st[k] = st[k + 397] ^ twist(st[k], st[k + 1]);
    for (int k = 624 - 397; k < 623; ++k) st[k] = st[k + 397 - 624] ^ twist(st[k], st[k + 1]);
    st[623] = st[396] ^ twist(st[623], st[0]);
    cur = 0;
  }
  uint32_t next_int() {
    if (cur >= 624) next_state();
    uint32_t x = st[cur++];
    x ^= x >> 11;
    x ^= (x << 7) & 0x9d2c5680u;
    x ^= (x << 15) & 0xefc60000u;
    return x ^ (x >> 18);
  }
  double next_real() { return (double)next_int() / 4294967295.0; }
};

}  // namespace

extern "C" {

// The first n tempered draws of the Mersenne Twister seeded with seed.
void orc_mt_ints(int32_t seed, int n, uint32_t* out) {
  Twister t(seed);
  for (int i = 0; i < n; ++i) out[i] = t.next_int();
}

// generate_stochastic_clouds[_sw] for ncol columns of nlay layers (arrays
// (ncol, nlay), column fastest, layer 1 at the surface): nsub sub-columns
// (the g-points), overlap icld (1 random, 2 maximum/random, 3 maximum), irng
// (0 kissvec seeded from the bottom four layer pressures, else the Mersenne
// Twister seeded with permuteseed), permuteseed (kissvec: draws skipped).
// band[g]: the 0-based band of sub-column g (ngb - ngb(1) with the SW's
// offset); fields: nfield arrays (nband, ncol, nlay) of band optics copied to
// cloudy sub-columns, clear[f] their clear-sub-column value.  Outputs
// (nsub, ncol, nlay): cover 0 / 1, ice and liquid water paths, and the
// nfield fields.  Returns 0, 3 for an icld outside 0..3, 6 where kissvec's
// seeding needs the layers ordered from the surface up (the reference stops).
int orc_mcica_subcol(int ncol, int nlay, int nsub, int icld, int irng, int permuteseed, const double* play,
                     const double* cldfr, const double* ciwp, const double* clwp, int nband, const int* band,
                     int nfield, const double* fields, const double* clear, double* cld_out, double* ciwp_out,
                     double* clwp_out, double* fields_out) {
  if (icld == 0) return 0;
  if (icld < 0 || icld > 3) return 3;
  if (irng != 0) irng = 1;
  const double cldmin = 1.0e-20;
  const size_t N = (size_t)ncol;
  auto at = [&](const double* a, int i, int l) { return a[(size_t)i + N * (size_t)l]; };
  auto sub = [&](int g, int i, int l) { return (size_t)g + (size_t)nsub * ((size_t)i + N * (size_t)l); };
  std::vector<double> cldf((size_t)ncol * nlay);
  for (int l = 0; l < nlay; ++l)
    for (int i = 0; i < ncol; ++i) {
      const double c = at(cldfr, i, l);
      cldf[(size_t)i + N * l] = c < cldmin ? 0.0 : c;
    }
  std::vector<double> cdf((size_t)nsub * ncol * nlay);
  if (irng == 0) {
    std::vector<Kiss> kiss(ncol);
    for (int i = 0; i < ncol; ++i) {
      if (nlay < 4) return 6;
      const double p1 = at(play, i, 0) * 1.e2, p2 = at(play, i, 1) * 1.e2;
      if (p1 < p2) return 6;
      uint32_t s[4];
      for (int k = 0; k < 4; ++k) {
        const double p = at(play, i, k) * 1.e2;
        s[k] = (uint32_t)(int32_t)((p - (double)(int64_t)p) * 1000000000.0);
      }
      kiss[i] = Kiss{s[0], s[1], s[2], s[3]};
    }
    for (int r = 0; r < permuteseed; ++r)
      for (int i = 0; i < ncol; ++i) kiss[i].next();
    if (icld == 3) {
      for (int g = 0; g < nsub; ++g)
        for (int i = 0; i < ncol; ++i) {
          const double v = kiss[i].next();
          for (int l = 0; l < nlay; ++l) cdf[sub(g, i, l)] = v;
        }
    } else {
      for (int g = 0; g < nsub; ++g)
        for (int l = 0; l < nlay; ++l)
          for (int i = 0; i < ncol; ++i) cdf[sub(g, i, l)] = kiss[i].next();
    }
  } else {
    Twister mt(permuteseed);
    for (int g = 0; g < nsub; ++g)
      for (int i = 0; i < ncol; ++i) {
        if (icld == 3) {
          const double v = mt.next_real();
          for (int l = 0; l < nlay; ++l) cdf[sub(g, i, l)] = v;
        } else {
          for (int l = 0; l < nlay; ++l) cdf[sub(g, i, l)] = mt.next_real();
        }
      }
  }
  if (icld == 2) {
    for (int l = 1; l < nlay; ++l)
      for (int i = 0; i < ncol; ++i) {
        const double cm = cldf[(size_t)i + N * (l - 1)];
        for (int g = 0; g < nsub; ++g) {
          const double below = cdf[sub(g, i, l - 1)];
          if (below > 1.0 - cm)
            cdf[sub(g, i, l)] = below;
          else
            cdf[sub(g, i, l)] = cdf[sub(g, i, l)] * (1.0 - cm);
        }
      }
  }
  const size_t total = (size_t)nsub * N * nlay, per_band = (size_t)nband * N * nlay;
  for (int l = 0; l < nlay; ++l)
    for (int i = 0; i < ncol; ++i) {
      const double c = cldf[(size_t)i + N * l];
      for (int g = 0; g < nsub; ++g) {
        const size_t q = sub(g, i, l);
        const bool cloudy = cdf[q] >= 1.0 - c;
        cld_out[q] = cloudy ? 1.0 : 0.0;
        ciwp_out[q] = cloudy ? at(ciwp, i, l) : 0.0;
        clwp_out[q] = cloudy ? at(clwp, i, l) : 0.0;
        for (int f = 0; f < nfield; ++f)
          fields_out[f * total + q] =
              cloudy ? fields[f * per_band + (size_t)band[g] + (size_t)nband * ((size_t)i + N * l)] : clear[f];
      }
    }
  return 0;
}

}  // extern "C"
