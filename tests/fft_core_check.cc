// Host build of the fused transforms' Stockham core (monofonic_gb300/csrc/fused.cuh)
// for tests/test_fft_core.py: runs every stage of a length-L transform of P
// pencils and prints the result, for comparison with numpy's FFT.
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <utility>
#include <vector>

#include "../monofonic_gb300/csrc/fused.cuh"

using namespace mfx::ff;

int main(int argc, char **argv) {
  const int L = std::atoi(argv[1]), P = std::atoi(argv[2]), inv = std::atoi(argv[3]), layout = std::atoi(argv[4]);
  const int es = layout ? P : 1, ps = layout ? 1 : L;
  std::vector<float2> x(L * P), y(L * P), tw(L);
  for (int t = 0; t < L; ++t) tw[t] = make_float2(float(std::cos(-2 * M_PI * t / L)), float(std::sin(-2 * M_PI * t / L)));
  for (int p = 0; p < P; ++p)
    for (int n = 0; n < L; ++n) {
      float a, b;
      if (std::scanf("%f %f", &a, &b) != 2) return 1;
      x[n * es + p * ps] = make_float2(a, b);
    }
  const Stages S = make_stages(L);
  if (S.n <= 0) return 2;
  float2 *X = x.data(), *Y = y.data();
  int Ns = 1;
  for (int s = 0; s < S.n; ++s) {
    const int R = S.r[s], nb = L / R;
    for (int p = 0; p < P; ++p)
      for (int j = 0; j < nb; ++j) {
        if (inv) stage_bfly<true>(X, Y, tw.data(), L, R, Ns, j, p, es, ps);
        else stage_bfly<false>(X, Y, tw.data(), L, R, Ns, j, p, es, ps);
      }
    std::swap(X, Y);
    Ns *= R;
  }
  for (int p = 0; p < P; ++p)
    for (int k = 0; k < L; ++k) std::printf("%.9e %.9e\n", X[k * es + p * ps].x, X[k * es + p * ps].y);
  return 0;
}
