// Host build of the fused transforms' pencil FFT (monofonic_gb300/csrc/fused.cuh)
// for tests/test_fft_core.py.  Runs the same Step / Tile code the CUDA kernels
// run, one "thread" after another between the barriers, on PP pencils of
// length L, and prints the result for comparison with numpy's FFT.
//   fft_core_check L PP inverse pencil_fast < re im pairs (pencil-major)
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
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

// One step of the multi-item form (pencil_fft_mi's mi_step): every butterfly
// of PP pencils read (ld), then every one written (st) -- the barrier between.
template <class S, int PP, class Ld, class St>
static void emu_mi_step(const float2 *tw, const Ld &ld, const St &st) {
  constexpr int RMAX = 32;
  std::vector<float2> regs(static_cast<size_t>(PP) * S::J * RMAX);
  for (int t = 0; t < PP * S::J; ++t) {
    int q, j;
    split<PP, S::J, true>(t, q, j);
    S::gather(j, [&](int n) { return ld(q, n); }, tw, &regs[size_t(t) * RMAX]);
  }
  for (int t = 0; t < PP * S::J; ++t) {
    int q, j;
    split<PP, S::J, true>(t, q, j);
    S::scatter(j, [&](int n, float2 x) { st(q, n, x); }, &regs[size_t(t) * RMAX]);
  }
}

// The x/y passes' in-place form (fused.cuh xy_units_inplace + xy_fft_halves_out)
// on 16 pencils of length L: input rows below `side` in the side buffer, the
// others at their stage positions in the tile; the first steps of both halves
// of 8 pencils, then the other steps of one half and of the other, each in
// place in its columns; then the tile's rows out.
template <int L, bool INV> static void host_inplace_fft(std::vector<float2> &data, const float2 *tw, int side) {
  constexpr int P = 16, H = 8;
  using F = Fac<L>;
  std::vector<float2> sidebuf(static_cast<size_t>(side) * P);
  std::vector<float2> tile(static_cast<size_t>(L) * P);
  for (int q = 0; q < P; ++q)
    for (int r = 0; r < L; ++r) (r < side ? sidebuf : tile)[size_t(r) * P + q] = data[size_t(q) * L + r];
  auto stage = [&](int i) { return i < side * P ? sidebuf[i] : tile[i]; };
  for (int h = 0; h < 2; ++h) {
    const int q0 = h * H;
    emu_mi_step<Step<L, F::R1, 1, INV>, H>(
        tw, [&](int q, int n) { return stage(n * P + q + q0); },
        [&](int q, int n, float2 x) { tile[size_t(n) * P + q0 + q] = x; });
  }
  std::fill(sidebuf.begin(), sidebuf.end(), make_float2(NAN, NAN));  // free: the next unit's rows land here
  for (int h = 0; h < 2; ++h) {
    const int q0 = h * H;
    auto lb = [&](int q, int n) { return tile[size_t(n) * P + q0 + q]; };
    auto sb = [&](int q, int n, float2 x) { tile[size_t(n) * P + q0 + q] = x; };
    if constexpr (F::steps == 3) emu_mi_step<Step<L, F::R2, F::R1, INV>, H>(tw, lb, sb);
    constexpr int RL = F::steps == 3 ? F::R3 : F::R2;
    emu_mi_step<Step<L, RL, L / RL, INV>, H>(tw, lb, sb);
  }
  for (int k = 0; k < L; ++k)
    for (int q = 0; q < P; ++q) data[size_t(q) * L + k] = tile[size_t(k) * P + q];
}

template <int L> static int run_inplace(int inv, int side, std::vector<float2> &data) {
  std::vector<float2> tw(L);
  for (int t = 0; t < L; ++t)
    tw[t] = make_float2(float(std::cos(-2.0 * M_PI * t / L)), float(std::sin(-2.0 * M_PI * t / L)));
  if (inv) host_inplace_fft<L, true>(data, tw.data(), side);
  else host_inplace_fft<L, false>(data, tw.data(), side);
  return 0;
}

// the x/y tile forms' sizes (XY) for every tile the launcher admits (the
// kz range divides into tiles, at most 1024 threads, shared memory within a
// CTA's 227 KB for both row counts, as fused_launch.cuh's xy_ok): an in-place
// form has a side buffer of at least one row and no more rows than its input,
// its stage rows lie within the tile, and its halves are P / 2 wide.
// Returns the number of violations; counts the admissible in-place forms.
static int g_inplace = 0;
template <int M, int P> static int check_xy() {
  using A = XY<M, P, M>;
  using B = XY<M, P, 2 * M / 3>;
  const bool ok = (M / 3) % P == 0 && A::threads <= 1024 && A::smem <= kXYSmemMax && B::smem <= kXYSmemMax &&
                  A::threads == B::threads && A::inplace == B::inplace;
  if (!ok) return 0;
  int bad = 0;
  auto one = [&](auto X, int rows) {
    using T = decltype(X);
    std::printf("M=%d P=%d rows=%d lean=%d inplace=%d side=%d threads=%d smem=%zu\n", M, P, rows, int(T::lean),
                int(T::inplace), T::side, T::threads, T::smem);
    if (!T::inplace) return;
    ++g_inplace;
    if (T::side < 1 || T::side > rows || size_t(rows) * P > size_t(T::tile) || T::HP * 2 != P ||
        size_t(M + T::tile + T::side * P) * sizeof(float2) != T::smem)
      ++bad;
  };
  one(A(), M);
  one(B(), 2 * M / 3);
  return bad;
}
template <int M> static int check_xy_m() {
  return check_xy<M, 4>() + check_xy<M, 8>() + check_xy<M, 16>() + check_xy<M, 32>();
}

int main(int argc, char **argv) {
  if (argc >= 2 && std::string(argv[1]) == "xy") {
    const int bad = check_xy_m<96>() + check_xy_m<144>() + check_xy_m<192>() + check_xy_m<288>() +
                    check_xy_m<384>() + check_xy_m<576>() + check_xy_m<768>() + check_xy_m<1152>() +
                    check_xy_m<1536>();
    std::printf("inplace %d bad %d\n", g_inplace, bad);
    return bad ? 4 : 0;
  }
  if (argc >= 5 && std::string(argv[1]) == "ip") {
    // fft_core_check ip L inverse side < 16 pencils (pencil-major)
    const int L = std::atoi(argv[2]), inv = std::atoi(argv[3]), side = std::atoi(argv[4]);
    std::vector<float2> data(size_t(L) * 16);
    for (auto &v : data) {
      float a, b;
      if (std::scanf("%f %f", &a, &b) != 2) return 1;
      v = make_float2(a, b);
    }
    if (side < 0 || side > L) return 1;
    int rc = 2;
    switch (L) {
      case 96: rc = run_inplace<96>(inv, side, data); break;
      case 576: rc = run_inplace<576>(inv, side, data); break;
      case 768: rc = run_inplace<768>(inv, side, data); break;
      case 1152: rc = run_inplace<1152>(inv, side, data); break;
      default: break;
    }
    if (rc) return rc;
    for (const auto &v : data) std::printf("%.9e %.9e\n", v.x, v.y);
    return 0;
  }
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
