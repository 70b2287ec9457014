// Host check of crocodile_gb300/csrc/fft32.h: the register-blocked Stockham
// stages (radix 16, one first stage of radix 2, 4 or 8), run thread by
// thread as the kernels run them (all threads' loads of a stage before any
// store, one buffer, the two-level twiddle table), against a direct DFT in
// double precision for
// N = 64 .. 8192 and both signs.  Prints the worst error relative to the
// transform's norm; exit status 0 when it is below 1e-6.
#include <cmath>
#include <cstdio>
#include <vector>

#include "fft32.h"

using namespace cg::f32;

int main() {
  double worst = 0;
  unsigned seed = 12345;
  auto rnd = [&]() {
    seed = seed * 1664525u + 1013904223u;
    return (float)((seed >> 8) * (1.0 / 16777216.0) - 0.5);
  };
  for (int logn = 6; logn <= 13; ++logn) {
    const int N = 1 << logn, T = N / 16;
    for (int sign = -1; sign <= 1; sign += 2) {
      std::vector<cf> in(N), buf(N), tw(N);
      for (auto &c : in) c = {rnd(), rnd()};
      for (int j = 0; j < N; ++j) {
        const double a = sign * 2.0 * M_PI * j / N;
        tw[j] = {(float)std::cos(a), (float)std::sin(a)};
      }
      // the kernels' two-level table: w^j = A[j mod 64] * C[j / 64] for N > 64
      std::vector<cf> A(64), Cc(N / 64 + 1);
      for (int a = 0; a < 64; ++a) A[a] = tw[a % N];
      for (int c = 0; c * 64 < N; ++c) Cc[c] = tw[c * 64];
      auto twf = [&](int j) { return N > 64 ? cf_mul(A[j & 63], Cc[j >> 6]) : tw[j]; };
      std::vector<std::vector<cf>> regs(T, std::vector<cf>(16));
      const int ns = stage_count(logn);
      for (int s = 0; s < ns; ++s) {
        const std::vector<cf> &src = s == 0 ? in : buf;
        auto ld = [&](int e) { return src[e]; };
        for (int t = 0; t < T; ++t) stage_load(logn, s, t, ld, twf, regs[t].data());
        auto st = [&](int e, cf v) { buf[e] = v; };
        for (int t = 0; t < T; ++t) {
          stage_dft(logn, s, sign, regs[t].data());
          stage_store(logn, s, t, st, regs[t].data());
        }
      }
      double num = 0, den = 0;
      const int kstep = N > 512 ? N / 512 : 1;  // direct DFT on a sample of outputs
      for (int k = 0; k < N; k += kstep) {
        double re = 0, im = 0;
        for (int n = 0; n < N; ++n) {
          const double a = sign * 2.0 * M_PI * (double)(((long long)n * k) % N) / N;
          re += in[n].x * std::cos(a) - in[n].y * std::sin(a);
          im += in[n].x * std::sin(a) + in[n].y * std::cos(a);
        }
        num += (buf[k].x - re) * (buf[k].x - re) + (buf[k].y - im) * (buf[k].y - im);
        den += re * re + im * im;
      }
      const double e = std::sqrt(num / den);
      if (e > worst) worst = e;
      printf("N %5d sign %+d rel %.3g\n", N, sign, e);
    }
  }
  printf("worst %.3g\n", worst);
  return worst < 1e-6 ? 0 : 1;
}
