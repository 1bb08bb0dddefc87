// Host check of the integer-pipe binary64 division, square root and multiplication
// (cato_intdiv.cuh): the same source as the device code, with the FP32 seeds computed by the host's IEEE float division and
// square root, compared bit for bit with the host's hardware a / b and sqrt(a).
//
// The device seeds are hardware approximations, so every family runs with the host seeds moved by
// up to 8 units in the last place either way (cato_gpu_check_divsqrt measures the hardware seeds
// against the same correctly rounded values over all their inputs).
//
// usage: intdiv_check <random cases per family and seed offset>
// Prints one line per family ("<family> tested <n> fallback <n> bad <n>") and exits 1 on any
// mismatch.  Families: random normal operands over the full exponent range and over a narrow
// one; significands near powers of two, near each other and with few bits set; quotients and
// roots next to rounding midpoints; every FP32 seed (all 2^23 truncated significands) with the
// largest truncation error; the exact power-of-two scalings; products over the full exponent
// range and of significands with few bits set (exact products and ties).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#define CATO_INTDIV_SEED_HOOK
#include "../fvleg_2d_gb300/csrc/cato_intdiv.cuh"

namespace cato {
namespace intdiv {
int seed_offset_ulps = 0;  // ulps added to the host seeds (the device uses approximations)
}  // namespace intdiv
}  // namespace cato

using namespace cato::intdiv;

static std::mt19937_64 rng(20261203);
static unsigned long long tested, fallback, bad;

static void reset() { tested = fallback = bad = 0; }
static void report(const char* fam) {
  printf("%s tested %llu fallback %llu bad %llu\n", fam, tested, fallback, bad);
}

static void check_div(double a, double b) {
  bool ok;
  const uint64_t q = div_bits(bits_of(a), bits_of(b), ok);
  if (!ok) { ++fallback; return; }
  ++tested;
  if (q != bits_of(a / b)) {
    if (bad < 5) printf("div mismatch %a / %a: %a, hardware %a\n", a, b, double_of(q), a / b);
    ++bad;
  }
}

static void check_sqrt(double a) {
  bool ok;
  const uint64_t r = sqrt_bits(bits_of(a), ok);
  if (!ok) { ++fallback; return; }
  ++tested;
  if (r != bits_of(std::sqrt(a))) {
    if (bad < 5) printf("sqrt mismatch %a: %a, hardware %a\n", a, double_of(r), std::sqrt(a));
    ++bad;
  }
}

static void check_mul(double a, double b) {
  bool ok;
  const uint64_t r = mul_bits(bits_of(a), bits_of(b), ok);
  if (!ok) { ++fallback; return; }
  ++tested;
  if (r != bits_of(a * b)) {
    if (bad < 5) printf("mul mismatch %a * %a: %a, hardware %a\n", a, b, double_of(r), a * b);
    ++bad;
  }
}

static double random_double(int emin, int emax, bool sign = true) {
  const uint64_t m = rng() & kFrac;
  const uint64_t e = (uint64_t)(emin + (int)(rng() % (uint64_t)(emax - emin + 1)));
  const uint64_t s = sign ? (rng() & 0x8000000000000000ULL) : 0;
  return double_of(s | (e << 52) | m);
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? atol(argv[1]) : 1000000;
  int fail = 0;
  static const int kOffsets[] = {0, -8, -4, -2, -1, 1, 2, 4, 8};

  reset();
  for (const int off : kOffsets) {
    seed_offset_ulps = off;
    for (long i = 0; i < n; ++i) check_div(random_double(1, 2046), random_double(1, 2046));
    for (long i = 0; i < n; ++i) check_div(random_double(960, 1090), random_double(960, 1090));
  }
  report("div_random");
  fail |= bad != 0;

  reset();
  for (const int off : kOffsets) {
  seed_offset_ulps = off;
  for (long i = 0; i < n; ++i) {
    uint64_t ma = rng() & kFrac, mb = rng() & kFrac;
    switch (rng() % 6) {
      case 0: mb &= 0xfff; break;                                   // b just above 2^k
      case 1: mb = kFrac - (mb & 0xfff); break;                     // b just below 2^k
      case 2: ma = (mb + (rng() % 9) - 4) & kFrac; break;           // a close to b
      case 3: ma &= ~((1ULL << (rng() % 50)) - 1); mb &= ~((1ULL << (rng() % 50)) - 1); break;
      case 4: ma = kFrac - (ma & 0xff); break;
      default: ma &= 0xff; break;
    }
    const double a = double_of(((uint64_t)(1022 + rng() % 3) << 52) | ma);
    const double b = double_of((1023ULL << 52) | mb);
    check_div(a, b);
  }
  for (long i = 0; i < n; ++i) {  // a / b next to a rounding midpoint of the quotient
    const double b = random_double(1000, 1046), q = random_double(1020, 1026);
    const long double mid = ((long double)q + (long double)double_of(bits_of(q) + 1)) / 2;
    const double a = (double)(mid * (long double)b);
    check_div(a, b);
    check_div(std::nextafter(a, 0.0), b);
    check_div(std::nextafter(a, 1e300), b);
    check_div(q * b, b);
  }
  }
  report("div_structured");
  fail |= bad != 0;

  reset();
  for (const int off : kOffsets) {
  seed_offset_ulps = off;
  for (long i = 0; i < n; ++i) check_sqrt(random_double(1, 2046, false));
  for (long i = 0; i < n; ++i) {  // next to a rounding midpoint of the root, and exact squares
    const double s = random_double(1000, 1046, false);
    const long double mid = ((long double)s + (long double)double_of(bits_of(s) + 1)) / 2;
    const double a = (double)(mid * mid);
    check_sqrt(a);
    check_sqrt(std::nextafter(a, 0.0));
    check_sqrt(std::nextafter(a, 1e300));
    check_sqrt(s * s);
  }
  }
  report("sqrt");
  fail |= bad != 0;

  reset();  // the exact scalings against the products, over all exponent classes
  for (long i = 0; i < 4 * n; ++i) {
    const uint64_t u = rng();
    const uint64_t cls = rng() % 4;
    double x = double_of(u);
    if (cls == 1) x = double_of((u & 0x800fffffffffffffULL) | ((rng() % 5) << 52));      // tiny
    if (cls == 2) x = double_of((u & 0x800fffffffffffffULL) | ((0x7fcULL + rng() % 4) << 52));
    if (x != x) continue;
    ++tested;
    const bool ok = bits_of(scale_down<1>(x)) == bits_of(x * 0.5) &&
                    bits_of(scale_down<2>(x)) == bits_of(x * 0.25) &&
                    bits_of(scale_down<3>(x)) == bits_of(x * 0.125) &&
                    bits_of(scale_up1(x)) == bits_of(x * 2.0);
    if (!ok) {
      if (bad < 5) printf("scale mismatch %a\n", x);
      ++bad;
    }
  }
  report("scale");
  fail |= bad != 0;

  reset();  // every seed: b (a) = 1.t followed by 29 one bits (largest truncation), and zeros
  for (const int off : {-8, 0, 8}) {
  seed_offset_ulps = off;
  for (uint64_t t = 0; t < (1ULL << 23); ++t) {
    for (const uint64_t low : {0ULL, (1ULL << 29) - 1}) {
      const uint64_t m = (t << 29) | low;
      const double b = double_of((1023ULL << 52) | m);
      check_div(double_of((1023ULL << 52) | (rng() & kFrac)), b);
      check_div(double_of((1023ULL << 52) | kFrac), b);
      check_div(b, b);
      check_sqrt(b);
      check_sqrt(double_of((1024ULL << 52) | m));
    }
  }
  }
  seed_offset_ulps = 0;
  report("seeds");
  fail |= bad != 0;

  reset();  // products: random operands, few significant bits (exact products, ties), overflow
  for (long i = 0; i < 4 * n; ++i) {
    check_mul(random_double(1, 2046), random_double(1, 2046));
    check_mul(random_double(900, 1150), random_double(900, 1150));
    uint64_t ma = rng() & kFrac, mb = rng() & kFrac;
    switch (rng() % 5) {
      case 0: mb = (1ULL << (rng() % 52)); break;                    // b = 1 + 2^-k
      case 1: mb = (1ULL << (rng() % 52)) | (1ULL << (rng() % 52)); ma |= 1; break;
      case 2: ma &= ~((1ULL << (rng() % 53)) - 1); mb &= ~((1ULL << (rng() % 53)) - 1); break;
      case 3: ma = kFrac - (ma & 0xff); mb = kFrac - (mb & 0xff); break;  // near 2 x 2
      default: ma &= 0xfff; break;
    }
    const uint64_t s2 = rng() & 0x8000000000000000ULL;
    const double a = double_of(s2 | ((uint64_t)(1000 + rng() % 47) << 52) | ma);
    const double b = double_of(((uint64_t)(1000 + rng() % 47) << 52) | mb);
    check_mul(a, b);
    // near the ends of the normal range: subnormal and overflowing products fall back
    check_mul(random_double(1, 30), random_double(990, 1030));
    check_mul(random_double(2020, 2046), random_double(1020, 1030));
  }
  report("mul");
  fail |= bad != 0;
  return fail;
}
