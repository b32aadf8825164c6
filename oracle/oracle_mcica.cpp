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

// ---------------------------------------------------------------------------
// Jump-ahead of the Mersenne Twister (the F2-linear jump of Haramoto,
// Matsumoto, Nishimura, Panneton and L'Ecuyer, "Efficient jump ahead for
// F2-linear random number generators", 2008): the state J words ahead is
// g(T) applied to the state, T the one-word transition and g(x) = x^J mod
// phi(x), phi the characteristic polynomial of T (degree 19937).  A prototype
// of the host side of a device generator that starts each sub-column's
// stream at its own offset; the tests check it against the serial stream.
// ---------------------------------------------------------------------------

// The transition one word at a time: 624 words in a ring, the next word
// x[k + 624] = x[k + 397] ^ twist(x[k], x[k + 1]) written over x[k].
struct MtRing {
  uint32_t x[624];
  int k = 0;
  uint32_t step() {
    const uint32_t v = x[(k + 397) % 624] ^ Twister::twist(x[k], x[(k + 1) % 624]);
    x[k] = v;
    k = (k + 1) % 624;
    return v;
  }
  static uint32_t temper(uint32_t y) {
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    return y ^ (y >> 18);
  }
};

// Polynomials over GF(2), bit i of word i / 64 the coefficient of x^i.
struct Poly {
  std::vector<uint64_t> w;
  explicit Poly(int nbits = 0) : w((size_t)(nbits + 64) / 64, 0) {}
  bool bit(int i) const { return (size_t)(i >> 6) < w.size() && ((w[(size_t)i >> 6] >> (i & 63)) & 1u); }
  void flip(int i) {
    if ((size_t)(i >> 6) >= w.size()) w.resize((size_t)(i >> 6) + 1, 0);
    w[(size_t)i >> 6] ^= (uint64_t)1 << (i & 63);
  }
  int deg() const {
    for (size_t j = w.size(); j-- > 0;)
      if (w[j]) return (int)(j * 64) + 63 - __builtin_clzll(w[j]);
    return -1;
  }
  // this ^= src * x^sh
  void add_shifted(const Poly& src, int sh) {
    const int ds = src.deg();
    if (ds < 0) return;
    const size_t need = (size_t)(ds + sh) / 64 + 1;
    if (w.size() < need) w.resize(need, 0);
    const int q = sh >> 6, r = sh & 63;
    for (size_t j = 0; j < src.w.size(); ++j) {
      const uint64_t v = src.w[j];
      if (!v) continue;
      w[j + q] ^= v << r;
      if (r && j + q + 1 < w.size()) w[j + q + 1] ^= v >> (64 - r);
    }
  }
};

// The remainder of a modulo m.
static void poly_mod(Poly& a, const Poly& m) {
  const int dm = m.deg();
  for (int d = a.deg(); d >= dm; d = a.deg()) a.add_shifted(m, d - dm);
}

// The square of a over GF(2): coefficient i moves to 2i.
static Poly poly_square(const Poly& a) {
  Poly r(2 * (a.deg() + 1));
  for (int i = 0, d = a.deg(); i <= d; ++i)
    if (a.bit(i)) r.flip(2 * i);
  return r;
}

// phi(x): the minimal polynomial of the bit sequence of the generator's
// words (their top bits), by Berlekamp-Massey over 2 x 19937 + 64 bits; for
// MT19937 it is the characteristic polynomial of the transition (degree
// 19937).  Computed once.
static const Poly& mt_charpoly() {
  static Poly phi = [] {
    const int N = 2 * 19937 + 64;
    MtRing g;
    Twister t(5489);
    for (int i = 0; i < 624; ++i) g.x[i] = t.st[i];
    std::vector<uint8_t> s(N);
    for (int i = 0; i < N; ++i) s[i] = (uint8_t)(g.step() >> 31);
    // connection polynomial C (s_n = sum_{j=1..L} c_j s_{n-j})
    std::vector<uint8_t> C(N + 1, 0), B(N + 1, 0), T;
    C[0] = B[0] = 1;
    int L = 0, m = 1;
    for (int n = 0; n < N; ++n) {
      uint8_t d = s[n];
      for (int j = 1; j <= L; ++j) d ^= (uint8_t)(C[j] & s[n - j]);
      if (!d) {
        ++m;
      } else if (2 * L <= n) {
        T = C;
        for (int j = 0; j + m <= N; ++j) C[j + m] ^= B[j];
        L = n + 1 - L;
        B = T;
        m = 1;
      } else {
        for (int j = 0; j + m <= N; ++j) C[j + m] ^= B[j];
        ++m;
      }
    }
    // phi(x) = x^L C(1/x)
    Poly p(L);
    for (int j = 0; j <= L; ++j)
      if (C[j]) p.flip(L - j);
    return p;
  }();
  return phi;
}

// x^J mod phi(x), square and multiply from the top bit of J.
static Poly mt_jump_poly(uint64_t J) {
  const Poly& phi = mt_charpoly();
  Poly r(1);
  r.flip(0);
  for (int b = 63; b >= 0; --b) {
    r = poly_square(r);
    poly_mod(r, phi);
    if ((J >> b) & 1u) {
      Poly x(r.deg() + 2);
      x.add_shifted(r, 1);
      r = x;
      poly_mod(r, phi);
    }
  }
  return r;
}

// g(T) applied to the ring by Horner's rule: acc = T(acc) ^ g_k * start,
// k from deg g down to 0.  The result is aligned to k = 0.
static void mt_apply(const Poly& g, MtRing& ring) {
  MtRing acc;
  for (int i = 0; i < 624; ++i) acc.x[i] = 0;
  for (int k = g.deg(); k >= 0; --k) {
    acc.step();
    if (g.bit(k))
      for (int i = 0; i < 624; ++i) acc.x[(acc.k + i) % 624] ^= ring.x[(ring.k + i) % 624];
  }
  MtRing out;
  for (int i = 0; i < 624; ++i) out.x[i] = acc.x[(acc.k + i) % 624];
  ring = out;
}

}  // namespace

extern "C" {

// The first n tempered draws of the Mersenne Twister seeded with seed.
void orc_mt_ints(int32_t seed, int n, uint32_t* out) {
  Twister t(seed);
  for (int i = 0; i < n; ++i) out[i] = t.next_int();
}

// The n tempered draws that follow the first `jump` draws of the Mersenne
// Twister seeded with seed, reached by the jump-ahead above (no draw of the
// first `jump` is made).  Returns the degree of phi (19937).
int orc_mt_jump_ints(int32_t seed, uint64_t jump, int n, uint32_t* out) {
  MtRing ring;
  Twister t(seed);
  for (int i = 0; i < 624; ++i) ring.x[i] = t.st[i];
  mt_apply(mt_jump_poly(jump), ring);
  for (int i = 0; i < n; ++i) out[i] = MtRing::temper(ring.step());
  return mt_charpoly().deg();
}

// The start states of nsub sub-column streams `stride` words apart (McICA's
// Mersenne Twister path draws sub-column g from word g * ncol * nlay of the
// stream): one jump polynomial x^stride mod phi, applied in a chain, each
// start reached from the one before.  out (nsub, n): the first n draws from
// each start.
void orc_mt_subcol_starts(int32_t seed, uint64_t stride, int nsub, int n, uint32_t* out) {
  MtRing ring;
  Twister t(seed);
  for (int i = 0; i < 624; ++i) ring.x[i] = t.st[i];
  const Poly g = mt_jump_poly(stride);
  for (int s = 0; s < nsub; ++s) {
    if (s) mt_apply(g, ring);
    MtRing r = ring;
    for (int i = 0; i < n; ++i) out[(size_t)s * n + i] = MtRing::temper(r.step());
  }
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
