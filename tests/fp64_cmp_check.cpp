// Checks every helper of fp64_cmp.h against the C comparison operators (and
// the sign flip against the unary minus) on
// signed zeros, subnormals, normals around the model constants, infinities,
// NaNs of both signs and random bit patterns.  Prints the number of
// mismatches and exits non-zero when there is any.
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <random>
#include <vector>

#include "fp64_cmp.h"

using namespace pihm::cmp;

int main() {
  // the positive constants the kernels compare against, and a few others
  const double consts[] = {1e-4 /* depression storage */, 1e-3, 0.5e-4, 1.0, 700.0, 70.0, 0.1, 5e-8,
                           0.01, 3.0e-8, DBL_MIN, DBL_TRUE_MIN, DBL_MAX, 0.5, 2.0};
  std::vector<double> v = {0.0, -0.0, DBL_TRUE_MIN, -DBL_TRUE_MIN, DBL_MIN, -DBL_MIN,
                           std::nextafter(DBL_MIN, 0.0), -std::nextafter(DBL_MIN, 0.0),
                           DBL_MAX, -DBL_MAX, INFINITY, -INFINITY,
                           std::numeric_limits<double>::quiet_NaN(),
                           -std::numeric_limits<double>::quiet_NaN(),
                           from_bits(0x7FF0000000000001ull), from_bits(0xFFF0000000000001ull),
                           from_bits(0x7FFFFFFFFFFFFFFFull), from_bits(0xFFFFFFFFFFFFFFFFull),
                           from_bits(0x7FF8000000000000ull), from_bits(0xFFF8000000000000ull)};
  for (double c : consts) {
    for (double s : {1.0, -1.0}) {
      v.push_back(s * c);
      v.push_back(s * std::nextafter(c, 0.0));
      v.push_back(s * std::nextafter(c, INFINITY));
      v.push_back(s * c * 0.5);
      v.push_back(s * c * 3.0);
    }
  }
  std::mt19937_64 rng(12345);
  std::uniform_real_distribution<double> u(-10.0, 10.0);
  for (int k = 0; k < 2000; k++) v.push_back(from_bits(rng()));
  for (int k = 0; k < 2000; k++) v.push_back(u(rng));
  for (int k = 0; k < 500; k++) v.push_back(u(rng) * 1e-300);

  long bad = 0;
  auto check = [&](bool got, bool want, const char *what, double x, double y) {
    if (got != want) {
      if (bad < 20)
        std::printf("mismatch %s x=%a y=%a got %d want %d\n", what, x, y, (int)got, (int)want);
      bad++;
    }
  };
  for (double x : v) {
    check(gt0(x), x > 0.0, "gt0", x, 0.0);
    check(ge0(x), x >= 0.0, "ge0", x, 0.0);
    check(lt0(x), x < 0.0, "lt0", x, 0.0);
    check(le0(x), x <= 0.0, "le0", x, 0.0);
    check(eq0(x), x == 0.0, "eq0", x, 0.0);
    check(isnan_(x), std::isnan(x), "isnan_", x, 0.0);
    // the unary minus, bit for bit
    const double nx = -x;
    check(bits(neg_if(x, true)) == bits(nx), true, "neg_if", x, 0.0);
    check(bits(neg_if(x, false)) == bits(x), true, "neg_if0", x, 0.0);
    for (double c : consts) {
      check(gt_c(x, c), x > c, "gt_c", x, c);
      check(ge_c(x, c), x >= c, "ge_c", x, c);
      check(lt_c(x, c), x < c, "lt_c", x, c);
      check(le_c(x, c), x <= c, "le_c", x, c);
      check(abs_lt_c(x, c), std::fabs(x) < c, "abs_lt_c", x, c);
      check(gt_nc(x, -c), x > -c, "gt_nc", x, -c);
    }
  }
  // every ordered pair of a sample (the random part thinned to keep it quick)
  std::vector<double> w(v.begin(), v.begin() + 80);
  for (size_t k = 80; k < v.size(); k += 7) w.push_back(v[k]);
  for (double x : w)
    for (double y : w) {
      check(lt_v(x, y), x < y, "lt_v", x, y);
      check(le_v(x, y), x <= y, "le_v", x, y);
      check(gt_v(x, y), x > y, "gt_v", x, y);
      check(ge_v(x, y), x >= y, "ge_v", x, y);
    }
  std::printf("%zu values, %ld mismatches\n", v.size(), bad);
  return bad ? 1 : 0;
}
