// Host check of crocodile_gb300/csrc/fft32.h: the register-blocked Stockham
// stages (radix 16, one first stage of radix 2, 4 or 8), run thread by
// thread as the kernels run them (all threads' loads of a stage before any
// store, one buffer, twiddles from the per-stage tables), against a direct
// DFT in double precision for N = 32 .. 8192 and both signs; and every
// twiddle of the per-stage tables against the exact value (at most 2^-22
// off: one rounding, or the product of two rounded entries).  Prints the worst
// error relative to the transform's norm; exit status 0 when it is below
// 1e-6 and every twiddle is within that bound.
#include <cmath>
#include <cstdio>
#include <vector>

#include "fft32.h"

using namespace cg::f32;

int main() {
  double worst = 0, tw_worst = 0;
  unsigned seed = 12345;
  auto rnd = [&]() {
    seed = seed * 1664525u + 1013904223u;
    return (float)((seed >> 8) * (1.0 / 16777216.0) - 0.5);
  };
  for (int logn = 5; logn <= 13; ++logn) {
    const int N = 1 << logn, T = N / 16;
    for (int sign = -1; sign <= 1; sign += 2) {
      std::vector<cf> in(N), buf(N), tw(N);
      for (auto &c : in) c = {rnd(), rnd()};
      for (int j = 0; j < N; ++j) {
        const double a = sign * 2.0 * M_PI * j / N;
        tw[j] = {(float)std::cos(a), (float)std::sin(a)};
      }
      // the kernels' per-stage table
      std::vector<cf> tab(tw_table_entries(logn) + 1);
      tw_table_fill(logn, [&](long long j) { return tw[j]; }, tab.data());
      auto tb = [&](int i) { return tab[i]; };
      auto twf = [&](int s, int r, int k) { return tw_lookup(logn, s, r, k, tb); };
      for (int s = 1; s < stage_count(logn); ++s) {
        const int logr = stage_logr(logn, s), logp = stage_logp(logn, s);
        for (int r = 1; r < (1 << logr); ++r)
          for (int k = 1; k < (1 << logp); ++k) {
            const cf w = twf(s, r, k);
            const double a = sign * 2.0 * M_PI * (double)((long long)r * k << (logn - logp - logr)) / N;
            const double e = std::fmax(std::fabs(w.x - std::cos(a)), std::fabs(w.y - std::sin(a)));
            if (e > tw_worst) tw_worst = e;
          }
      }
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
  printf("twiddle worst abs %.3g\n", tw_worst);
  printf("worst %.3g\n", worst);
  return worst < 1e-6 && tw_worst <= 0x1p-22 ? 0 : 1;
}
