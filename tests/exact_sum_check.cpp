// Checks the exact parallel running sum of the resampling fallback on the
// CPU: the window algorithm of the kernel `exact_running_sums`
// (dust2_gb300/csrc/filter_kernels.cu), run here one emulated block at a
// time over the same integer helpers (dust2gpu/exact_sum.hpp), must give
// the plain loop s_j = fl(s_{j-1} + w_j) bit for bit.  Prints one line
// "cases C bad B windows_per_1000 W" and exits non-zero on a mismatch.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <random>
#include <vector>

#include "dust2gpu/exact_sum.hpp"

namespace es = dust2gpu::exact_sum;
using dust2gpu::math::bits_of;

// The kernel's loop, with its block of nb threads emulated in order.
static std::vector<double> windowed(const std::vector<double>& w, int nb,
                                    long* windows) {
  const int n = static_cast<int>(w.size());
  std::vector<double> ser(n);
  std::vector<std::uint64_t> r(nb);
  std::vector<char> tie(nb);
  ser[0] = w[0];
  double sum = w[0];
  int j0 = 0;
  while (j0 < n - 1) {
    ++*windows;
    const es::grid gr = es::grid_of(sum);
    if (!gr.ok) {
      for (int j = j0 + 1; j < n; ++j) {
        sum = sum + w[j];
        ser[j] = sum;
      }
      break;
    }
    for (int t = 0; t < nb; ++t) {
      const int j = j0 + 1 + t;
      bool tt = false;
      r[t] = j < n ? es::grid_units(w[j], gr.e_grid, &tt) : 0;
      tie[t] = tt;
    }
    std::uint64_t acc = 0;
    int first = nb;
    std::vector<std::uint64_t> m(nb);
    for (int t = 0; t < nb; ++t) {
      acc = es::sat_add(acc, r[t]);
      m[t] = gr.count + acc;
      const int j = j0 + 1 + t;
      if (first == nb && j < n && es::is_break(m[t], tie[t])) {
        first = t;
      }
    }
    for (int t = 0; t < first; ++t) {
      const int j = j0 + 1 + t;
      if (j < n) {
        ser[j] = es::grid_value(gr, m[t]);
      }
    }
    const int jb = j0 + 1 + first;
    if (first < 32 && jb < n) {
      const int stop = std::min(n - 1, j0 + 128);
      double a = ser[jb - 1];
      for (int q = jb; q <= stop; ++q) {
        a = a + w[q];
        ser[q] = a;
      }
      sum = a;
      j0 = stop;
    } else if (first < nb && jb < n) {
      sum = ser[jb - 1] + w[jb];
      ser[jb] = sum;
      j0 = jb;
    } else {
      j0 = std::min(n - 1, j0 + nb);
      sum = ser[j0];
    }
  }
  return ser;
}

int main() {
  std::mt19937_64 rng(1);
  std::uniform_real_distribution<double> U(0, 1);
  long bad = 0, cases = 0, windows = 0, elements = 0;
  for (int rep = 0; rep < 2000; ++rep) {
    const int kind = rep % 10;
    const int n = 1 + static_cast<int>(rng() % (rep % 3 == 0 ? 40000 : 3000));
    std::vector<double> w(n);
    for (int j = 0; j < n; ++j) {
      double x;
      switch (kind) {
      case 0: x = std::exp(-30 * U(rng)); break;                 // filter-like
      case 1: x = std::exp(-700 * U(rng)); break;                // wide range
      case 2: x = 1.0; break;                                     // equal
      case 3: x = static_cast<double>(rng() % 4) * 0.5; break;    // halfway cases
      case 4: x = std::ldexp(1.0, -static_cast<int>(rng() % 1100)); break;
      case 5: x = std::ldexp(static_cast<double>(rng() % 1000),
                             static_cast<int>(rng() % 60) - 30); break;
      case 6: x = U(rng) < 0.9 ? 0.0 : U(rng); break;             // sparse
      case 7: x = std::ldexp(U(rng), static_cast<int>(rng() % 2000) - 1074);
        break;                                                    // subnormal..huge
      case 8: x = U(rng) * 1e300; break;                          // overflow to Inf
      default: x = (rep % 20 == 9) ? U(rng) - 0.3 : U(rng); break; // negatives
      }
      w[j] = x;
    }
    const int nb = (rep % 2) ? 1024 : 128;
    const std::vector<double> a = windowed(w, nb, &windows);
    elements += n;
    ++cases;
    double s = 0;
    for (int j = 0; j < n; ++j) {
      s = s + w[j];
      if (bits_of(s) != bits_of(a[j])) {
        if (bad < 5) {
          std::printf("mismatch: kind %d n %d j %d\n", kind, n, j);
        }
        ++bad;
        break;
      }
    }
  }
  std::printf("cases %ld bad %ld windows_per_1000 %.2f\n", cases, bad,
              1000.0 * static_cast<double>(windows) /
              static_cast<double>(elements));
  return bad == 0 ? 0 : 1;
}
