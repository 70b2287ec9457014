// Host check of crocodile_gb300/csrc/fft32.h: the in-place radix-4 DIT line
// transform (bit-reversed load, odd and even log2 N, both signs) against a
// direct DFT in double precision, for N = 2 .. 8192.  Prints the worst error
// relative to the transform's norm; exit status 0 when it is below 1e-5.
#include <cmath>
#include <cstdio>
#include <vector>

#include "fft32.h"

using namespace cg::f32;

struct Buf {
  std::vector<cf> v;
  cf get(int i) const { return v[i]; }
  void set(int i, cf a) { v[i] = a; }
};
struct Tw {
  std::vector<cf> v;
  cf get(int k) const { return v[k]; }
};

int main() {
  double worst = 0;
  unsigned s = 12345;
  auto rnd = [&]() {
    s = s * 1664525u + 1013904223u;
    return (float)((s >> 8) * (1.0 / 16777216.0) - 0.5);
  };
  for (int logn = 1; logn <= 13; ++logn) {
    const int N = 1 << logn;
    for (int sign = -1; sign <= 1; sign += 2) {
      std::vector<cf> in(N);
      for (auto &c : in) c = {rnd(), rnd()};
      Tw tw;
      tw.v.resize(N / 2 > 0 ? N / 2 : 1);
      for (int k = 0; k < N / 2; ++k) {
        const double a = sign * 2.0 * M_PI * k / N;
        tw.v[k] = {(float)std::cos(a), (float)std::sin(a)};
      }
      Buf x;
      x.v.resize(N);
      for (int i = 0; i < N; ++i) x.v[bitrev(i, logn)] = in[i];
      line_serial(x, tw, logn, sign);
      double num = 0, den = 0;
      const int kstep = N > 512 ? N / 512 : 1;  // direct DFT on a sample of outputs
      for (int k = 0; k < N; k += kstep) {
        double re = 0, im = 0;
        for (int n = 0; n < N; ++n) {
          const double a = sign * 2.0 * M_PI * (double)(((long long)n * k) % N) / N;
          re += in[n].x * std::cos(a) - in[n].y * std::sin(a);
          im += in[n].x * std::sin(a) + in[n].y * std::cos(a);
        }
        num += (x.v[k].x - re) * (x.v[k].x - re) + (x.v[k].y - im) * (x.v[k].y - im);
        den += re * re + im * im;
      }
      const double e = std::sqrt(num / den);
      if (e > worst) worst = e;
      printf("N %5d sign %+d rel %.3g\n", N, sign, e);
    }
  }
  printf("worst %.3g\n", worst);
  return worst < 1e-5 ? 0 : 1;
}
