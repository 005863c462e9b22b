// Checks the bit-pattern comparisons of pg_tritri.cuh (host build) against
// the IEEE comparisons they stand for: every pair of a set of edge values
// (zeros of both signs, subnormals, infinities, NaNs) and seeded random bit
// patterns, half of them near one another.  Prints the number of mismatches.
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <cmath>
#include <random>
#include "../parmec_gb300/csrc/pg_tritri.cuh"

static double from_bits(unsigned long long b) { double x; memcpy(&x, &b, 8); return x; }

int main(int argc, char **argv)
{
  const long n = argc > 1 ? atol(argv[1]) : 1000000;
  const double edge[] = {0.0, -0.0, 1.0, -1.0, INFINITY, -INFINITY, NAN, -NAN, 5e-324, -5e-324,
                         1e308, -1e308, 2.2e-308, -2.2e-308, 0.5, 1.0000000000000002, 0.9999999999999999};
  long bad = 0, cases = 0;
  auto check = [&](double a, double b) {
    cases ++;
    bad += pgtt::lt(a, b) != (a < b);
    bad += pgtt::gt(a, b) != (a > b);
    bad += pgtt::lt_neg(a, b) != (a < -b);
  };
  for (double a : edge) for (double b : edge) check(a, b);
  std::mt19937_64 g(12345);
  for (long i = 0; i < n; i ++)
  {
    unsigned long long x = g(), y = g();
    switch (i & 3)
    {
    case 1: y = x ^ (g() & 0xff); break;                     // close values
    case 2: y = x ^ 0x8000000000000000ULL; break;            // opposite signs
    case 3: x &= 0x800fffffffffffffULL; break;               // zeros and subnormals
    }
    check(from_bits(x), from_bits(y));
  }
  printf("%ld %ld\n", cases, bad);
  return 0;
}
