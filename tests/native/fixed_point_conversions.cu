// Host-side check of the f32 <-> int64 conversions the FIt-SNE charges use
// (bhtsne_gb300/csrc/common.cuh): round to nearest even, saturation as the
// IEEE conversion. References: a long double (at least 64-bit significand) holds
// every int64 exactly, so one rounding to float is the correctly rounded value;
// llrintf rounds to nearest even in the default rounding mode. Exit status 0
// when every case matches.
#include "common.cuh"

#include <cmath>
#include <cstdio>
#include <random>

using bhg::f32_bits;
using bhg::f32_from_bits;

int main(int argc, char** argv) {
  const long long cases = argc > 1 ? atoll(argv[1]) : 4000000;
  std::mt19937_64 g(1);
  long long bad = 0, n = 0;
  auto i2f = [&](long long v) {
    const float ref = (float)(long double)v;
    const float got = bhg::i64_to_f32_rn(v);
    if (f32_bits(ref) != f32_bits(got)) {
      if (bad < 5) printf("i64 -> f32 %lld: expected %a, got %a\n", v, ref, got);
      ++bad;
    }
    ++n;
  };
  auto f2i = [&](float x) {
    long long ref;
    if (std::isnan(x)) ref = (long long)0x8000000000000000ull;
    else if (x >= 9.2233720368547758e18f) ref = 0x7FFFFFFFFFFFFFFFll;
    else if (x < -9.2233720368547758e18f) ref = (long long)0x8000000000000000ull;
    else ref = llrintf(x);
    const long long got = bhg::f32_to_i64_rn(x);
    if (ref != got) {
      if (bad < 5) printf("f32 -> i64 %a: expected %lld, got %lld\n", x, ref, got);
      ++bad;
    }
    ++n;
  };
  const long long edges[] = {0, 1, 2, 3, (1ll << 24) - 1, 1ll << 24, (1ll << 24) + 1, (1ll << 24) + 2,
                             (1ll << 24) + 3, (1ll << 25) + 2, (1ll << 25) + 6, (1ll << 62) - 1, 1ll << 62,
                             0x7FFFFFFFFFFFFFFFll, (long long)0x8000000000000000ull};
  for (long long v : edges) {
    i2f(v);
    i2f(-v);
  }
  for (long long i = 0; i < cases; ++i) {
    const int bits = (int)(g() % 64);
    long long v = (long long)(g() >> (63 - bits));
    if (g() & 1) v = -v;
    i2f(v);
    if (bits > 26) i2f((v & ~((1ll << (bits - 24)) - 1)) | (1ll << (bits - 25)));  // an exact tie
    f2i(f32_from_bits((uint32_t)g()));
  }
  const float fedges[] = {0.f, -0.f, 0.5f, -0.5f, 1.5f, 2.5f, -2.5f, 0.49999997f, 0.50000006f, 8388607.5f,
                          16777216.f, 9.2233715e18f, -9.2233715e18f, 9.2233720e18f, -9.2233720e18f, INFINITY,
                          -INFINITY, NAN, 3.4e38f, 1e-30f};
  for (float x : fedges) f2i(x);
  for (uint32_t ex = 100; ex < 200; ++ex)  // every exponent that reaches the integer range, strided mantissas
    for (uint32_t m = 0; m < (1u << 23); m += 997) {
      f2i(f32_from_bits((ex << 23) | m));
      f2i(f32_from_bits(0x80000000u | (ex << 23) | m));
    }
  printf("%lld cases, %lld mismatches\n", n, bad);
  return bad != 0;
}
