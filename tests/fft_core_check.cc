// Host build of the fused transforms' pencil FFT (monofonic_gb300/csrc/fused.cuh)
// for tests/test_fft_core.py.  Runs the same Step / Tile code the CUDA kernels
// run, one "thread" after another between the barriers, on PP pencils of
// length L, and prints the result for comparison with numpy's FFT.
//   fft_core_check L PP inverse pencil_fast < re im pairs (pencil-major)
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <vector>

#include "../monofonic_gb300/csrc/fused.cuh"

using namespace mfx::ff;

template <int L, int PP, bool PF, bool INV>
static void host_pencil_fft(std::vector<float2> &data, const std::vector<float2> &tw) {
  using F = Fac<L>;
  using T = Tile<L, PP, PF>;
  std::vector<float2> buf(T::elems);
  constexpr int RMAX = 32;
  // step 1: from data (pencil-major) into buf
  {
    using S = Step<L, F::R1, 1, INV>;
    std::vector<float2> regs(static_cast<size_t>(PP) * S::J * RMAX);
    for (int t = 0; t < PP * S::J; ++t) {
      int q, j;
      split<PP, S::J, PF>(t, q, j);
      S::template gather<!PF>(j, [&](int n) { return data[size_t(q) * L + n]; }, tw.data(), &regs[size_t(t) * RMAX]);
    }
    for (int t = 0; t < PP * S::J; ++t) {
      int q, j;
      split<PP, S::J, PF>(t, q, j);
      S::scatter(j, [&](int n, float2 x) { buf[T::at(q, n)] = x; }, &regs[size_t(t) * RMAX]);
    }
  }
  if constexpr (F::steps == 3) {
    using S = Step<L, F::R2, F::R1, INV>;
    std::vector<float2> regs(static_cast<size_t>(PP) * S::J * RMAX);
    for (int t = 0; t < PP * S::J; ++t) {
      int q, j;
      split<PP, S::J, PF>(t, q, j);
      S::template gather<!PF>(j, [&](int n) { return buf[T::at(q, n)]; }, tw.data(), &regs[size_t(t) * RMAX]);
    }
    for (int t = 0; t < PP * S::J; ++t) {
      int q, j;
      split<PP, S::J, PF>(t, q, j);
      S::scatter(j, [&](int n, float2 x) { buf[T::at(q, n)] = x; }, &regs[size_t(t) * RMAX]);
    }
  }
  {
    constexpr int RL = F::steps == 3 ? F::R3 : F::R2;
    using S = Step<L, RL, L / RL, INV>;
    std::vector<float2> regs(static_cast<size_t>(PP) * S::J * RMAX);
    for (int t = 0; t < PP * S::J; ++t) {
      int q, j;
      split<PP, S::J, PF>(t, q, j);
      S::template gather<!PF>(j, [&](int n) { return buf[T::at(q, n)]; }, tw.data(), &regs[size_t(t) * RMAX]);
    }
    for (int t = 0; t < PP * S::J; ++t) {
      int q, j;
      split<PP, S::J, PF>(t, q, j);
      S::scatter(j, [&](int n, float2 x) { data[size_t(q) * L + n] = x; }, &regs[size_t(t) * RMAX]);
    }
  }
}

template <int L> static int run(int pp, int inv, int pf, std::vector<float2> &data) {
  // the flat table and, after it, the per-step tables the non-PF (z) transforms read
  std::vector<float2> tw(TwTab<L>::elems);
  for (int t = 0; t < L; ++t)
    tw[t] = make_float2(float(std::cos(-2.0 * M_PI * t / L)), float(std::sin(-2.0 * M_PI * t / L)));
  for (int e = 0; e < TwTab<L>::n2 + TwTab<L>::n3; ++e) tw[L + e] = tw[TwTab<L>::src(e)];
  if (pp != 3) return 3;
  if (inv && pf) host_pencil_fft<L, 3, true, true>(data, tw);
  if (inv && !pf) host_pencil_fft<L, 3, false, true>(data, tw);
  if (!inv && pf) host_pencil_fft<L, 3, true, false>(data, tw);
  if (!inv && !pf) host_pencil_fft<L, 3, false, false>(data, tw);
  return 0;
}

int main(int argc, char **argv) {
  if (argc < 5) return 1;
  const int L = std::atoi(argv[1]), PP = std::atoi(argv[2]), inv = std::atoi(argv[3]), pf = std::atoi(argv[4]);
  std::vector<float2> data(size_t(L) * PP);
  for (auto &v : data) {
    float a, b;
    if (std::scanf("%f %f", &a, &b) != 2) return 1;
    v = make_float2(a, b);
  }
  int rc = 2;
  switch (L) {
    case 16: rc = run<16>(PP, inv, pf, data); break;
    case 24: rc = run<24>(PP, inv, pf, data); break;
    case 32: rc = run<32>(PP, inv, pf, data); break;
    case 64: rc = run<64>(PP, inv, pf, data); break;
    case 128: rc = run<128>(PP, inv, pf, data); break;
    case 256: rc = run<256>(PP, inv, pf, data); break;
    case 512: rc = run<512>(PP, inv, pf, data); break;
    case 1024: rc = run<1024>(PP, inv, pf, data); break;
    case 48: rc = run<48>(PP, inv, pf, data); break;
    case 96: rc = run<96>(PP, inv, pf, data); break;
    case 144: rc = run<144>(PP, inv, pf, data); break;
    case 192: rc = run<192>(PP, inv, pf, data); break;
    case 288: rc = run<288>(PP, inv, pf, data); break;
    case 384: rc = run<384>(PP, inv, pf, data); break;
    case 576: rc = run<576>(PP, inv, pf, data); break;
    case 768: rc = run<768>(PP, inv, pf, data); break;
    case 1152: rc = run<1152>(PP, inv, pf, data); break;
    case 1536: rc = run<1536>(PP, inv, pf, data); break;
    default: break;
  }
  if (rc) return rc;
  for (const auto &v : data) std::printf("%.9e %.9e\n", v.x, v.y);
  return 0;
}
