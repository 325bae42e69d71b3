// Pruned, fused 3D transforms for the Orszag-padded convolutions (FP32 form).
//
// The padded fields live on the M-grid (M = 3N/2) but their spectra are
// non-zero only on the N-grid modes, and the z Nyquist plane kz = N/2 is zero
// in every padded spectrum (phi and every unpadded result zero each Nyquist
// index).  A 3D transform is done as three passes of 1D transforms whose
// pencils skip what is known to be zero; nothing on the M-grid is ever stored
// in real space.  Fields are kept in two mixed layouts (complex float):
//
//   B-space [N][M][N/2]  kx on the N-grid, y transformed (padded), kz < N/2
//   C-space [M][M][N/2]  x and y transformed (padded), kz < N/2
//
// and the z transforms of all the fields a source needs are done together, per
// (x, y) row, inside one CTA, with the real-space products formed in shared
// memory between the inverse and the forward z transforms:
//
//   Y3    phi (N-grid k-space) -> B0 = Y(phi), B1 = Y(ky phi), B2 = Y(ky^2 phi)
//         (the Hessian factors separate: k_a k_b = (x part)(y part)(z part))
//   X6    B0..B2 -> the six Hessians -k_a k_b phi in C-space (x inverse FFT)
//   ZSRC2 per row: six inverse z transforms (three complex, two real pencils
//         each), the 2LPT source (ic_generator.cc:530-534) and the five
//         products of convolve3's first pairs (ic_generator.cc:581-609), then
//         forward z transforms -> D-space (= C-space layout)
//   XF    D -> E (B-space layout): forward x FFT, keeps the N-grid kx
//   YF    E -> N-grid k-space: forward y FFT, unpad (zero every Nyquist index,
//         convolution.hh:600-636), scale, inverse Laplacian (grid_fft.hh:440-449)
//         or, for the pairs, truncate and transform back along y (B-space)
//   XI    B-space -> C-space (x inverse FFT) for the truncated pair products
//   ZSRC3 per row: 17 inverse z transforms (phi1 and phi2 Hessians, the five
//         truncated pair products), the 3LPT sources phi3a + phi3b and A3
//         (ic_generator.cc:581-628) with compensated sums, four forward z
//         transforms -> D-space
//
// Each 1D transform is a compile-time mixed-radix Stockham FFT: two or three
// steps of radix 4..24 butterflies held in registers, with one shared-memory
// exchange between steps.  The first step reads its inputs straight from
// global memory (or a shared-memory real row) and the last step writes its
// outputs straight to their destination, so the x/y passes move each element
// through shared memory once.
#pragma once
#include <stdint.h>

#include <type_traits>
#include <utility>
#if defined(__CUDACC__)
#include <cuda_runtime.h>
#define MFX_HD __host__ __device__ __forceinline__
#define MFX_CX __host__ __device__ constexpr
#else
// host-only compilation (tests of the transform core on the CPU)
#include <cmath>
struct float2 {
  float x, y;
};
inline float2 make_float2(float a, float b) { return float2{a, b}; }
#define MFX_HD inline
#define MFX_CX constexpr
#endif

namespace mfx {
namespace ff {

// ---------------------------------------------------------------------------
// compile-time helpers
// ---------------------------------------------------------------------------
template <int I> using Ic = std::integral_constant<int, I>;

template <class F, int... I> MFX_HD void static_for_(F &&f, std::integer_sequence<int, I...>) {
  (f(Ic<I>{}), ...);
}
template <int N, class F> MFX_HD void static_for(F &&f) { static_for_(f, std::make_integer_sequence<int, N>{}); }

// cos / sin by their Taylor series, evaluated by the compiler for the
// twiddles inside a butterfly (|x| <= pi: the 30th terms are below 1e-40)
MFX_CX double cx_cos(double x) {
  double t = 1.0, s = 1.0;
  for (int k = 1; k <= 30; ++k) {
    t *= -x * x / double((2 * k - 1) * (2 * k));
    s += t;
  }
  return s;
}
MFX_CX double cx_sin(double x) {
  double t = x, s = x;
  for (int k = 1; k <= 30; ++k) {
    t *= -x * x / double((2 * k) * (2 * k + 1));
    s += t;
  }
  return s;
}

// W^NUM of W = exp(-2 pi i / DEN), with the quarter turns exact
template <int NUM, int DEN> struct Tw {
  static constexpr int n = NUM % DEN;
  static constexpr bool quarter = (4 * n) % DEN == 0;
  static constexpr int q = (4 * n) / DEN;
  static constexpr double ang = -6.283185307179586476925286766559 * double(2 * n > DEN ? n - DEN : n) / double(DEN);
  static constexpr float c = float(cx_cos(ang)), s = float(cx_sin(ang));
};

MFX_HD float2 cmul(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }

// x * W^NUM (forward) or x * conj(W)^NUM (INV)
template <int NUM, int DEN, bool INV> MFX_HD float2 twmul(float2 x) {
  using T = Tw<NUM, DEN>;
  if constexpr (T::quarter) {
    constexpr int q = INV ? (4 - T::q) & 3 : T::q;
    if constexpr (q == 0) return x;
    else if constexpr (q == 1) return make_float2(x.y, -x.x);  // * (-i)
    else if constexpr (q == 2) return make_float2(-x.x, -x.y);
    else return make_float2(-x.y, x.x);  // * (+i)
  } else {
    constexpr float c = T::c, s = INV ? -T::s : T::s;
    return make_float2(x.x * c - x.y * s, x.x * s + x.y * c);
  }
}

// In-register DFT of R points (forward: sum_n v[n] W_R^{nk}; INV: conjugate
// W, unnormalised).  R = A*B is split as n = A b + a, k = k2 + B k1: B-point
// DFTs of the A decimated sequences, twiddles W_R^{a k2}, A-point DFTs.
template <int R, bool INV> MFX_HD void dft(float2 *v) {
  if constexpr (R == 1) {
  } else if constexpr (R == 2) {
    const float2 a = v[0], b = v[1];
    v[0] = make_float2(a.x + b.x, a.y + b.y);
    v[1] = make_float2(a.x - b.x, a.y - b.y);
  } else if constexpr (R == 3) {
    const float h = 0.86602540378443864676f;  // sqrt(3)/2
    const float2 s = make_float2(v[1].x + v[2].x, v[1].y + v[2].y);
    const float2 d = make_float2(v[1].x - v[2].x, v[1].y - v[2].y);
    const float2 t = make_float2(v[0].x - 0.5f * s.x, v[0].y - 0.5f * s.y);
    // forward: y1 = t - i h d, y2 = t + i h d
    const float2 ihd = INV ? make_float2(-h * d.y, h * d.x) : make_float2(h * d.y, -h * d.x);
    v[0] = make_float2(v[0].x + s.x, v[0].y + s.y);
    v[1] = make_float2(t.x + ihd.x, t.y + ihd.y);
    v[2] = make_float2(t.x - ihd.x, t.y - ihd.y);
  } else if constexpr (R == 4) {
    const float2 a = make_float2(v[0].x + v[2].x, v[0].y + v[2].y);
    const float2 b = make_float2(v[0].x - v[2].x, v[0].y - v[2].y);
    const float2 c = make_float2(v[1].x + v[3].x, v[1].y + v[3].y);
    const float2 d = make_float2(v[1].x - v[3].x, v[1].y - v[3].y);
    // forward: y1 = b - i d, y3 = b + i d
    const float2 id = INV ? make_float2(-d.y, d.x) : make_float2(d.y, -d.x);
    v[0] = make_float2(a.x + c.x, a.y + c.y);
    v[2] = make_float2(a.x - c.x, a.y - c.y);
    v[1] = make_float2(b.x + id.x, b.y + id.y);
    v[3] = make_float2(b.x - id.x, b.y - id.y);
  } else {
    constexpr int A = (R % 4 == 0) ? 4 : ((R % 2 == 0) ? 2 : 3);
    constexpr int B = R / A;
    static_assert(A * B == R, "radix must be 2^a 3^b");
    float2 u[R];
    static_for<A>([&](auto ai) {
      constexpr int a = decltype(ai)::value;
      float2 s[B];
      static_for<B>([&](auto bi) { s[decltype(bi)::value] = v[A * decltype(bi)::value + a]; });
      dft<B, INV>(s);
      static_for<B>([&](auto ki) {
        constexpr int k = decltype(ki)::value;
        u[a * B + k] = twmul<a * k, R, INV>(s[k]);
      });
    });
    static_for<B>([&](auto ki) {
      constexpr int k2 = decltype(ki)::value;
      float2 s[A];
      static_for<A>([&](auto ai) { s[decltype(ai)::value] = u[decltype(ai)::value * B + k2]; });
      dft<A, INV>(s);
      static_for<A>([&](auto ji) { v[k2 + B * decltype(ji)::value] = s[decltype(ji)::value]; });
    });
  }
}

// Radices of each supported length (R3 = 1: two steps): every padded length
// M = 3N/2 with N/2 a multiple of 8 and N <= 1024 whose length is 2^a 3^b, and
// the matching N-grid lengths of the assembly passes.
template <int L> struct Fac;
MFX_CX int cmax(int a, int b) { return a > b ? a : b; }
#define MFX_FAC(L, a, b, c)                                                  \
  template <> struct Fac<L> {                                                \
    static constexpr int R1 = a, R2 = b, R3 = c;                             \
    static constexpr int steps = (c > 1) ? 3 : 2;                            \
    static constexpr int maxJ = cmax(cmax(L / a, L / b), c > 1 ? L / c : 0); \
  }
MFX_FAC(16, 4, 4, 1);
MFX_FAC(24, 4, 6, 1);
MFX_FAC(32, 4, 8, 1);
MFX_FAC(64, 8, 8, 1);
MFX_FAC(128, 16, 8, 1);
MFX_FAC(256, 16, 16, 1);
MFX_FAC(512, 8, 8, 8);
MFX_FAC(1024, 16, 8, 8);
MFX_FAC(48, 8, 6, 1);
MFX_FAC(96, 8, 12, 1);
MFX_FAC(144, 12, 12, 1);
MFX_FAC(192, 16, 12, 1);
MFX_FAC(288, 8, 6, 6);
MFX_FAC(384, 8, 8, 6);
MFX_FAC(576, 8, 8, 9);
MFX_FAC(768, 8, 12, 8);
MFX_FAC(1152, 8, 12, 12);
MFX_FAC(1536, 16, 12, 8);
#undef MFX_FAC

// The twiddle table of a length in shared memory: W_L^t for t < L, then one
// table per later Stockham step laid out [r - 1][k] (W_L^(r k S) for the
// step's r < R, k < NS), so that the lanes of a warp, which hold consecutive
// butterflies j and so consecutive k = j mod NS, read consecutive words
// instead of words r k S apart (bank conflicts in the flat table).  The
// values are copies of the flat table's: the transforms are unchanged.
template <int L> struct TwTab {
  using F = Fac<L>;
  static constexpr int n2 = (F::R2 - 1) * F::R1;                                 // step 2: NS = R1
  static constexpr int n3 = F::steps == 3 ? (F::R3 - 1) * F::R1 * F::R2 : 0;  // step 3: NS = R1 R2
  static constexpr int elems = (L + n2 + n3 + 1) & ~1;  // even: what follows stays 16-byte aligned
  static constexpr int off(int NS) { return NS == F::R1 ? L : L + n2; }
  // flat-table index of entry e (< n2 + n3) of the per-step tables
  MFX_HD static int src(int e) {
    const bool s2 = e < n2;
    const int NS = s2 ? F::R1 : F::R1 * F::R2, R = s2 ? F::R2 : F::R3, x = s2 ? e : e - n2;
    const int r = x / NS + 1, k = x - (r - 1) * NS;
    return r * k * (L / (NS * R));
  }
};

// Shared-memory tile of PP pencils of length L.  PF: pencil index fastest
// (x/y passes, whose pencils are adjacent in global memory); otherwise each
// pencil is contiguous, padded by one slot per 16 against bank conflicts.
template <int L, int PP, bool PF> struct Tile {
  static constexpr int padL = L + (L >> 4);
  static constexpr int elems = PF ? L * PP : PP * padL;
  MFX_HD static int at(int q, int n) { return PF ? n * PP + q : q * padL + n + (n >> 4); }
};

template <int PP, int J, bool PF> MFX_HD void split(int t, int &q, int &j) {
  if (PF) {
    q = t % PP;
    j = t / PP;
  } else {
    j = t % J;
    q = t / J;
  }
}

// One Stockham step of radix R after NS points have been combined: task j
// reads x[j + r L/R], applies W_{NS R}^{r (j mod NS)}, does an R-point DFT and
// writes y[(j / NS) NS R + (j mod NS) + r NS].  tw[t] = W_L^t.
template <int L, int R, int NS, bool INV> struct Step {
  static constexpr int J = L / R;
  // TWS: tw holds the per-step tables of TwTab<L> after the flat one
  template <bool TWS = false, class Ld> MFX_HD static void gather(int j, const Ld &ld, const float2 *tw, float2 *v) {
    static_for<R>([&](auto ri) {
      constexpr int r = decltype(ri)::value;
      v[r] = ld(j + r * J);
    });
    if constexpr (NS > 1) {
      const int k = j % NS;
      constexpr int S = L / (NS * R);
      static_for<R - 1>([&](auto ri) {
        constexpr int r = decltype(ri)::value + 1;
        float2 w = TWS ? tw[TwTab<L>::off(NS) + (r - 1) * NS + k] : tw[r * k * S];
        if (INV) w.y = -w.y;
        v[r] = cmul(v[r], w);
      });
    }
    dft<R, INV>(v);
  }
  template <class St> MFX_HD static void scatter(int j, const St &st, const float2 *v) {
    const int k = j % NS, base = (j / NS) * NS * R + k;
    static_for<R>([&](auto ri) {
      constexpr int r = decltype(ri)::value;
      st(base + r * NS, v[r]);
    });
  }
};

#if defined(__CUDACC__)
// PP pencils of length L through one CTA (blockDim.x >= PP * Fac<L>::maxJ;
// every thread must call it).  ld(q, n) returns input n of pencil q;
// st(q, k, v) takes output k.  buf and buf2 each hold Tile<L, PP, PF>::elems
// values; the steps alternate between them, so that a step's reads and the
// next step's writes never share a buffer (one barrier per exchange).  ld may
// read either buffer; st may write obuf() (the buffer the last step does not
// read); the caller synchronises before reading what st wrote to shared
// memory.  LDB = false: ld reads neither buffer and nothing but an earlier
// call of the same shape reads buf, which then needs no barrier before the
// first step's writes when that call's last step read buf2 (three steps).
// B1 = false: no barrier there at all (the caller has one between any earlier
// reader of buf and this call).
template <int L> __device__ __forceinline__ float2 *obuf(float2 *buf, float2 *buf2) {
  return Fac<L>::steps == 3 ? buf : buf2;
}

// SL: a barrier between the last step's gathers and its scatters, so that st
// may write the buffer the last step reads (buf for two steps, buf2 for three)
template <int L, int PP, bool PF, bool INV, bool LDB = true, bool B1 = true, bool SL = false, class Ld, class St>
__device__ __forceinline__ void pencil_fft(float2 *buf, float2 *buf2, const float2 *tw, const Ld &ld, const St &st) {
  using F = Fac<L>;
  using T = Tile<L, PP, PF>;
  const int t = threadIdx.x;
  {
    using S = Step<L, F::R1, 1, INV>;
    float2 v[F::R1];
    int q, j;
    split<PP, S::J, PF>(t, q, j);
    const bool act = t < PP * S::J;
    if (act) S::template gather<!PF>(j, [&](int n) { return ld(q, n); }, tw, v);
    // ld may read buf; an earlier call's last step may still read it
    if constexpr (B1 && (LDB || F::steps != 3)) __syncthreads();
    if (act) S::scatter(j, [&](int n, float2 x) { buf[T::at(q, n)] = x; }, v);
    __syncthreads();
  }
  float2 *src = buf;
  if constexpr (F::steps == 3) {
    using S = Step<L, F::R2, F::R1, INV>;
    float2 v[F::R2];
    int q, j;
    split<PP, S::J, PF>(t, q, j);
    if (t < PP * S::J) {
      S::template gather<!PF>(j, [&](int n) { return buf[T::at(q, n)]; }, tw, v);
      S::scatter(j, [&](int n, float2 x) { buf2[T::at(q, n)] = x; }, v);
    }
    __syncthreads();
    src = buf2;
  }
  {
    constexpr int RL = F::steps == 3 ? F::R3 : F::R2;
    using S = Step<L, RL, L / RL, INV>;
    float2 v[RL];
    int q, j;
    split<PP, S::J, PF>(t, q, j);
    if constexpr (SL) {
      const bool act = t < PP * S::J;
      if (act) S::template gather<!PF>(j, [&](int n) { return src[T::at(q, n)]; }, tw, v);
      __syncthreads();
      if (act) S::scatter(j, [&](int n, float2 x) { st(q, n, x); }, v);
    } else if (t < PP * S::J) {
      S::template gather<!PF>(j, [&](int n) { return src[T::at(q, n)]; }, tw, v);
      S::scatter(j, [&](int n, float2 x) { st(q, n, x); }, v);
    }
  }
}
#endif

#if defined(__CUDACC__)
// a step hook that does nothing
struct NoHook {
  __device__ __forceinline__ void operator()() const {}
};

// One step of the in-place, multi-item form: NT threads each hold up to
// ceil(PP J / NT) butterflies, read all of them (ld), meet at a barrier, call
// hk (every thread: the step's source is no longer read) and write them (st);
// task order as split<PP, J, PF>.
template <int L, int R, int NS, bool INV, int PP, bool PF, int NT, class Ld, class St, class Hk = NoHook>
__device__ __forceinline__ void mi_step(const float2 *tw, const Ld &ld, const St &st, const Hk &hk = Hk()) {
  using S = Step<L, R, NS, INV>;
  constexpr int NI = PP * S::J, I = (NI + NT - 1) / NT;
  float2 v[I][R];
#pragma unroll
  for (int it = 0; it < I; ++it) {
    const int t = int(threadIdx.x) + it * NT;
    if (t < NI) {
      int q, j;
      split<PP, S::J, PF>(t, q, j);
      S::gather(j, [&](int n) { return ld(q, n); }, tw, v[it]);
    }
  }
  __syncthreads();
  hk();
#pragma unroll
  for (int it = 0; it < I; ++it) {
    const int t = int(threadIdx.x) + it * NT;
    if (t < NI) {
      int q, j;
      split<PP, S::J, PF>(t, q, j);
      S::scatter(j, [&](int n, float2 x) { st(q, n, x); }, v[it]);
    }
  }
}

// PP pencils of length L in place in buf (Tile<L, PP, PF>), NT threads (for
// the x/y tiles fewer than PP * maxJ: the tiles too wide for one butterfly
// per thread).  ld(q, n) may read buf and st(q, k, v) may write it; the
// caller synchronises before reading what st wrote.  One barrier per step and
// one between steps.  h1 runs (every thread) once the first step has read its
// input, h2 once the last step has read buf.
// LD (PF only): the row stride of buf, for PP pencils within a wider tile
template <int L, int PP, bool PF, bool INV, int NT, int LD = PP, class Ld, class St, class H1 = NoHook,
          class H2 = NoHook>
__device__ __forceinline__ void pencil_fft_mi(float2 *buf, const float2 *tw, const Ld &ld, const St &st,
                                              const H1 &h1 = H1(), const H2 &h2 = H2()) {
  using F = Fac<L>;
  using T = Tile<L, PP, PF>;
  auto at = [](int q, int n) { return PF ? n * LD + q : T::at(q, n); };
  auto lb = [&](int q, int n) { return buf[at(q, n)]; };
  auto sb = [&](int q, int n, float2 x) { buf[at(q, n)] = x; };
  mi_step<L, F::R1, 1, INV, PP, PF, NT>(tw, ld, sb, h1);
  __syncthreads();
  if constexpr (F::steps == 3) {
    mi_step<L, F::R2, F::R1, INV, PP, PF, NT>(tw, lb, sb);
    __syncthreads();
  }
  constexpr int RL = F::steps == 3 ? F::R3 : F::R2;
  mi_step<L, RL, L / RL, INV, PP, PF, NT>(tw, lb, st, h2);
}
#endif

// ---------------------------------------------------------------------------
// index maps
// ---------------------------------------------------------------------------
// N-grid index of padded index ip (convolution.hh:563-572), -1 in the gap
MFX_HD int unpad_index(int ip, int N) {
  const int nh = N >> 1;
  return ip <= nh ? ip : (ip > N ? ip - nh : -1);
}
MFX_HD int sidx(int i, int n) { return i > (n >> 1) ? i - n : i; }

// slot order of the Hessians: 0 xx 1 yy 2 zz 3 xy 4 xz 5 yz
MFX_HD int hslot(int x, int y) {
  if (x == y) return x;
  const int lo = x < y ? x : y, hi = x < y ? y : x;
  return lo == 0 ? (hi == 1 ? 3 : 4) : 5;
}

// Kahan accumulation (Kahan 1965, "Further remarks on reducing truncation
// errors") of the sources' products, with the running compensation c folded
// into each product by one FMA: y = a*b - c rounded once, t = s + y,
// c = (t - s) - y.  Four operations a term (TwoProduct + TwoSum take about
// ten); the sum's error stays within about 2u of the sum of |terms|.
struct Acc32 {
  float s = 0.f, c = 0.f;
  MFX_HD void step(float y) {
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  MFX_HD void add_prod(float k, float a, float b) { step(fmaf(k * a, b, -c)); }
  // a coefficient C in {1, -1, 2}, whose product with a is exact
  template <int C> MFX_HD void add_prod(float a, float b) {
    static_assert(C == 1 || C == -1 || C == 2, "exact coefficients only");
    step(fmaf(float(C) * a, b, -c));
  }
  MFX_HD float value() const { return s - c; }
};

// 2LPT source (ic_generator.cc:530-534) from the six phi1 Hessians
MFX_HD float src_phi2(const float *h) {
  Acc32 S;
  S.add_prod<1>(h[0], h[1] + h[2]);
  S.add_prod<1>(h[1], h[2]);
  S.add_prod<-1>(h[3], h[3]);
  S.add_prod<-1>(h[4], h[4]);
  S.add_prod<-1>(h[5], h[5]);
  return S.value();
}

// phi3a + phi3b (ic_generator.cc:581-609) and A3 (613-628) from the phi1
// Hessians p, the phi2 Hessians q and the truncated pair products T
MFX_HD void src_phi3(const float *p, const float *q, const float *T, float *s) {
  const float c57 = -5.0f / 7.0f, c107 = 10.0f / 7.0f;
  Acc32 S;
  S.add_prod<1>(T[0], p[2]);
  S.add_prod<2>(T[1], p[5]);
  S.add_prod<-1>(T[2], p[0]);
  S.add_prod<-1>(T[3], p[1]);
  S.add_prod<-1>(T[4], p[2]);
  S.add_prod(c57, p[0], q[1] + q[2]);
  S.add_prod(c57, p[1], q[2] + q[0]);
  S.add_prod(c57, p[2], q[0] + q[1]);
  S.add_prod(c107, p[3], q[3]);
  S.add_prod(c107, p[4], q[4]);
  S.add_prod(c107, p[5], q[5]);
  s[0] = S.value();
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int d1 = (d + 1) % 3, d2 = (d + 2) % 3;
    Acc32 A;
    A.add_prod<1>(q[hslot(d, d1)], p[hslot(d, d2)]);
    A.add_prod<-1>(q[hslot(d, d2)], p[hslot(d, d1)]);
    A.add_prod<1>(p[hslot(d1, d2)], q[hslot(d1, d1)] - q[hslot(d2, d2)]);
    A.add_prod<-1>(q[hslot(d1, d2)], p[hslot(d1, d1)] - p[hslot(d2, d2)]);
    s[1 + d] = A.value();
  }
}

// the five first pairs of convolve3 (ic_generator.cc:581-609):
// xx*yy, xy*xz, yz^2, xz^2, xy^2
MFX_HD void pair_products(const float *h, float *t) {
  t[0] = h[0] * h[1];
  t[1] = h[3] * h[4];
  t[2] = h[5] * h[5];
  t[3] = h[4] * h[4];
  t[4] = h[3] * h[3];
}

// Hermitian spectra of two real z pencils packed as A + iB (A[0], B[0] real)
// and their separation after a forward transform of a + ib
MFX_HD float2 pack_pair(float2 a, float2 b) { return make_float2(a.x - b.y, a.y + b.x); }
MFX_HD float2 pack_pair_conj(float2 a, float2 b) { return make_float2(a.x + b.y, b.x - a.y); }
MFX_HD void unpack_pair(float2 z, float2 zm, float2 &a, float2 &b) {
  a = make_float2(0.5f * (z.x + zm.x), 0.5f * (z.y - zm.y));
  b = make_float2(0.5f * (z.y + zm.y), -0.5f * (z.x - zm.x));
}

// CTAs per SM the register allocation is sized for: as many as leave each
// thread at least 64 registers, at most four
MFX_CX int min_blocks(int threads) {
  return 65536 / (threads * 64) < 1 ? 1 : (65536 / (threads * 64) > 4 ? 4 : 65536 / (threads * 64));
}

// x/y tile of P pencils.  Lean form, for tiles whose P * maxJ butterflies
// exceed 1024 threads: a third as many threads, each holding up to three
// butterflies of a step (registers for them: the register file is shared out
// in whole warps per scheduler), and one tile buffer (in-place transforms)
// beside the staging.
//
// In-place form, for lean tiles whose two stages do not fit beside the tile
// (P = 16 at M = 1152: 128-byte row pieces, where 64-byte ones halve the HBM
// rate of these strided rows): one stage only, the tile itself, which holds
// the unit's input rows from `side` up (at their stage positions r * P + q)
// while rows below `side` sit in a side buffer.  The side buffer of the next
// unit is fetched once the first steps of the transform's two halves have
// read this unit's input, the tile's rows once the result has left the tile;
// a unit makes one output (the transform overwrites its input).
constexpr size_t kXYSmemMax = 227 * 1024;
template <int M, int P, int ROWS> struct XY {
  static constexpr bool lean = P * Fac<M>::maxJ > 1024;
  static constexpr int nbuf = lean ? 1 : 2;
  static constexpr int tile = Tile<M, P, true>::elems;
  static constexpr size_t staged(int rows) { return size_t(M + nbuf * tile + 2 * rows * P) * sizeof(float2); }
  // decided on M rows, so that both row counts of a length take one form
  static constexpr bool inplace = lean && staged(M) > kXYSmemMax;
  // the in-place form transforms the tile in two halves of P / 2 pencils (the
  // registers of a P / 2 tile: all of a step's data is held across its barrier)
  static constexpr int HP = inplace ? P / 2 : P;
  static constexpr bool hlean = HP * Fac<M>::maxJ > 1024;
  static constexpr int threads = hlean ? (HP * Fac<M>::maxJ / 3) / 32 * 32 : HP * Fac<M>::maxJ;
  static constexpr int minb = (lean || inplace) ? 1 : min_blocks(threads);
  static constexpr size_t side_room = kXYSmemMax - size_t(M + tile) * sizeof(float2);
  static constexpr int side = !inplace ? 0
                              : (side_room / (P * sizeof(float2)) < size_t(ROWS) ? int(side_room / (P * sizeof(float2)))
                                                                                   : ROWS);
  static constexpr size_t smem = inplace ? size_t(M + tile + side * P) * sizeof(float2) : staged(ROWS);
};

#if defined(__CUDACC__)
// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
struct FArgs {
  const float2 *src[17];  // inputs per component
  float2 *dst[6];         // outputs per component
  const float2 *tw;       // W_M^t, t < M (global)
  int *status;            // set to nonzero by a kernel whose bounded wait ran out
  int ncomp;              // components in this launch
  int mode;               // X6: 0 Hessians from B0..B2, 1 plain; YF: 0 unpad, 1 truncate; ZSRC2: 1 with pairs
  float kfac, fac;
};

template <int M> struct Dims {
  static constexpr int N = 2 * M / 3, nh = N / 2, Kh = N / 2, nk = N / 2 + 1;
};

__device__ __forceinline__ float2 *ff_smem() {
  extern __shared__ float4 ff_smem4[];
  return reinterpret_cast<float2 *>(ff_smem4);
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

template <int M> __device__ __forceinline__ void load_tw(float2 *tw, const float2 *g) {
  for (int t = threadIdx.x; t < M; t += blockDim.x) tw[t] = g[t];
  __syncthreads();
}
// the flat table and the per-step tables (TwTab<M>) of the non-PF transforms
template <int M> __device__ __forceinline__ void load_tw_steps(float2 *tw, const float2 *g) {
  using TT = TwTab<M>;
  load_tw<M>(tw, g);
  for (int e = threadIdx.x; e < TT::n2 + TT::n3; e += blockDim.x) tw[M + e] = tw[TT::src(e)];
  __syncthreads();
}

// ---------------------------------------------------------------------------
// x/y passes (persistent): each CTA walks units blockIdx.x, + gridDim.x, ...
// A unit is one tile of P adjacent kz pencils (one outer index, one kz block,
// one input field).  The tile's input rows (P complex each, a fixed stride
// apart in global memory) are staged into shared memory with cp.async while
// the previous unit is transformed, and the first FFT step gathers from the
// stage.  Element offsets fit 32 bits for every supported size (N <= 1024).
// ---------------------------------------------------------------------------
template <int CHUNK> __device__ __forceinline__ void cp_async(void *dst, const void *src) {
  if constexpr (CHUNK == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }

// stages ROWS rows of P complex (row r at src + r * stride) as stage[r * P + q]
template <int P, int ROWS, int CHUNK>
__device__ __forceinline__ void stage_rows(float2 *stage, const float2 *src, unsigned stride) {
  constexpr int per_row = P * 8 / CHUNK, E = CHUNK / 8;
  for (int t = threadIdx.x; t < ROWS * per_row; t += blockDim.x) {
    const int r = t / per_row, c = t - r * per_row;
    cp_async<CHUNK>(stage + r * P + c * E, src + r * stride + c * E);
  }
}

// the transform of an x/y tile: pencil_fft, or pencil_fft_mi in the lean form
// (buf2 == buf there).  LDB as for pencil_fft: false where ld reads the stage
// and the tile's earlier transforms are all of this kind
template <int M, int P, bool INV, bool LDB = true, class Ld, class St>
__device__ __forceinline__ void xy_fft(float2 *buf, float2 *buf2, const float2 *tw, const Ld &ld, const St &st) {
  if constexpr (XY<M, P, M>::lean)
    pencil_fft_mi<M, P, true, INV, XY<M, P, M>::threads>(buf, tw, ld, st);
  else
    pencil_fft<M, P, true, INV, LDB>(buf, buf2, tw, ld, st);
}
// The in-place form's transform: the P-pencil tile buf in two halves of P / 2
// pencils, each in place in its columns (ld(q, n) and st(q, k, v) take the
// tile's pencil index q < P).  The first steps of both halves run first (the
// reads of the staged input), then h1 (the side buffer is free: the next
// unit's side rows load during the remaining steps), then the other steps of
// one half and of the other.  One copy of each step's code serves both halves
// (two inlined copies spill); the halves touch disjoint columns.  The caller
// synchronises before reading what st wrote.
template <int M, int P, bool INV, class Ld, class St, class H1 = NoHook>
__device__ __forceinline__ void xy_fft_halves(float2 *buf, const float2 *tw, const Ld &ld, const St &st,
                                              const H1 &h1 = H1()) {
  using F = Fac<M>;
  constexpr int H = P / 2, NT = XY<M, P, M>::threads;
#pragma unroll 1
  for (int h = 0; h < 2; ++h) {
    const int q0 = h * H;
    mi_step<M, F::R1, 1, INV, H, true, NT>(
        tw, [&](int q, int n) { return ld(q + q0, n); }, [&](int q, int n, float2 x) { buf[n * P + q0 + q] = x; });
  }
  h1();
  __syncthreads();
#pragma unroll 1
  for (int h = 0; h < 2; ++h) {
    const int q0 = h * H;
    auto lb = [&](int q, int n) { return buf[n * P + q0 + q]; };
    if constexpr (F::steps == 3) {
      mi_step<M, F::R2, F::R1, INV, H, true, NT>(tw, lb, [&](int q, int n, float2 x) { buf[n * P + q0 + q] = x; });
      __syncthreads();
    }
    constexpr int RL = F::steps == 3 ? F::R3 : F::R2;
    mi_step<M, RL, M / RL, INV, H, true, NT>(tw, lb, [&](int q, int k, float2 v) { st(q + q0, k, v); });
  }
}
// the same into the tile, then out2(q, k, v0, v1) for each pair of pencils
// (q even) of each row k: a row's P pencils leave in one piece (128 bytes for
// 16); h2 runs once the tile has been read
template <int M, int P, class Out2, class H2 = NoHook>
__device__ __forceinline__ void xy_store_rows(const float2 *buf, const Out2 &out2, const H2 &h2 = H2()) {
  __syncthreads();
  constexpr int PR = P / 2;  // pencil pairs per row
  for (int t = threadIdx.x; t < M * PR; t += blockDim.x) {
    const int k = t / PR, q = (t - k * PR) * 2;
    const float4 v = *reinterpret_cast<const float4 *>(buf + k * P + q);
    out2(q, k, make_float2(v.x, v.y), make_float2(v.z, v.w));
  }
  __syncthreads();
  h2();
}
template <int M, int P, bool INV, class Ld, class Out2, class H1 = NoHook, class H2 = NoHook>
__device__ __forceinline__ void xy_fft_halves_out(float2 *buf, const float2 *tw, const Ld &ld, const Out2 &out2,
                                                  const H1 &h1 = H1(), const H2 &h2 = H2()) {
  xy_fft_halves<M, P, INV>(buf, tw, ld, [&](int q, int k, float2 v) { buf[k * P + q] = v; }, h1);
  xy_store_rows<M, P>(buf, out2, h2);
}

// the tile buffers and the staging area of an x/y kernel's shared memory
// (in the in-place form `stage` is the side buffer)
template <int M, int P, int ROWS = M> struct XYMem {
  float2 *tw, *buf, *buf2, *stage;
  __device__ __forceinline__ XYMem(float2 *base) {
    tw = base;
    buf = tw + M;
    buf2 = XY<M, P, M>::lean ? buf : buf + Tile<M, P, true>::elems;
    stage = buf + XY<M, P, M>::nbuf * Tile<M, P, true>::elems;
  }
};

// the in-place form's input rows: stage row r at side[r * P + q] below the
// side buffer's rows, at tile[r * P + q] from there on
struct SplitStage {
  const float2 *side, *tile;
  int lim;  // side rows * P
  __device__ __forceinline__ float2 operator[](int i) const { return i < lim ? side[i] : tile[i]; }
};

// stages rows [r0, r1) of P complex (row r at src + r * stride) as dst[r * P + q]
template <int P, int CHUNK>
__device__ __forceinline__ void stage_row_range(float2 *dst, const float2 *src, unsigned stride, int r0, int r1) {
  constexpr int per_row = P * 8 / CHUNK, E = CHUNK / 8;
  for (int t = threadIdx.x + r0 * per_row; t < r1 * per_row; t += blockDim.x) {
    const int r = t / per_row, c = t - r * per_row;
    cp_async<CHUNK>(dst + r * P + c * E, src + r * stride + c * E);
  }
}

// The persistent unit loop: fetch(u, stage) issues unit u's copies,
// work(u, stage) transforms it.  One barrier per unit: after it every
// thread's copies of unit u have landed and every thread has finished unit
// u - 1, whose stage the copies of the next unit then overwrite while unit u
// is transformed.
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
template <class Fetch, class Work>
__device__ __forceinline__ void xy_units(unsigned units, unsigned stage_elems, float2 *stage0, const Fetch &fetch,
                                         const Work &work) {
  unsigned u = blockIdx.x;
  if (u < units) fetch(u, stage0);
  cp_async_commit();
#pragma unroll 1
  for (unsigned it = 0; u < units; ++it, u += gridDim.x) {
    float2 *cur = stage0 + (it & 1) * stage_elems, *nxt = stage0 + ((it & 1) ^ 1) * stage_elems;
    const unsigned un = u + gridDim.x;
    cp_async_wait_all();
    __syncthreads();
    if (un < units) fetch(un, nxt);
    cp_async_commit();
    work(u, cur);
  }
}

// The in-place form's unit loop: src(u) is unit u's first input row (ROWS
// rows, `stride` apart); work(u, stage, h1, h2) transforms unit u from the
// SplitStage and calls h1 and h2 through its transforms (xy_fft_halves,
// xy_fft_halves_out, xy_store_rows), which fetch the next unit's side rows and
// tile rows.  One barrier per unit: after it every thread's copies of unit u
// have landed.
template <int M, int P, int ROWS, int CHUNK = 16, class Src, class Work>
__device__ __forceinline__ void xy_units_inplace(unsigned units, float2 *side, float2 *tile, unsigned stride,
                                                 const Src &src, const Work &work) {
  constexpr int S = XY<M, P, ROWS>::side;
  const SplitStage st{side, tile, S * P};
  unsigned u = blockIdx.x;
  if (u < units) {
    stage_row_range<P, CHUNK>(side, src(u), stride, 0, S);
    stage_row_range<P, CHUNK>(tile, src(u), stride, S, ROWS);
  }
  cp_async_commit();
#pragma unroll 1
  for (; u < units; u += gridDim.x) {
    const unsigned un = u + gridDim.x;
    cp_async_wait_all();
    __syncthreads();
    work(
        u, st,
        [&] {
          if (un < units) stage_row_range<P, CHUNK>(side, src(un), stride, 0, S);
          cp_async_commit();
        },
        [&] {
          if (un < units) stage_row_range<P, CHUNK>(tile, src(un), stride, S, ROWS);
          cp_async_commit();
        });
  }
}

// Y3: B_o = inverse-y of fac (ky)^o phi, o < 3, padded in y.
// units: (i < N) x (Kh/P kz blocks), times the three outputs in the in-place
// form; input rows j < N of phi (8-byte aligned)
template <int M, int P> __global__ void __launch_bounds__(XY<M, P, 2 * M / 3>::threads, XY<M, P, 2 * M / 3>::minb)
    k_ff_y3(FArgs a) {
  using D = Dims<M>;
  using X = XY<M, P, D::N>;
  constexpr int ROWS = D::N, KB = D::Kh / P;
  const XYMem<M, P> sm(ff_smem());
  float2 *tw = sm.tw, *buf = sm.buf, *buf2 = sm.buf2, *stage = sm.stage;
  load_tw<M>(tw, a.tw);
  // output o of unit (i, kz block) from its staged rows
  auto one = [&](unsigned i, unsigned kz0, int o, const auto &st, const auto &h1, const auto &h2) {
    float2 *out = a.dst[o] + (i * M * D::Kh + kz0);
    auto ld = [&](int q, int n) -> float2 {
      const int j = unpad_index(n, D::N);
      if (j < 0) return make_float2(0.f, 0.f);
      const float2 v = st[j * P + q];
      float f = a.fac;
      if (o > 0) {
        const float gy = (j != D::nh) ? float(sidx(j, D::N)) * a.kfac : 0.f;
        f *= (o == 1) ? gy : gy * gy;
      }
      return make_float2(v.x * f, v.y * f);
    };
    if constexpr (X::inplace)
      xy_fft_halves_out<M, P, true>(
          buf, tw, ld,
          [&](int q, int n, float2 v0, float2 v1) {
            *reinterpret_cast<float4 *>(out + unsigned(n) * D::Kh + q) = make_float4(v0.x, v0.y, v1.x, v1.y);
          },
          h1, h2);
    else
      xy_fft<M, P, true, false>(buf, buf2, tw, ld, [&](int q, int n, float2 v) { out[unsigned(n) * D::Kh + q] = v; });
  };
  if constexpr (X::inplace) {
    xy_units_inplace<M, P, ROWS, 8>(
        unsigned(D::N * KB) * 3u, stage, buf, D::nk,
        [&](unsigned u) {
          const unsigned t = u / 3, i = t / KB, kz0 = (t % KB) * P;
          return a.src[0] + (i * D::N * D::nk + kz0);
        },
        [&](unsigned u, const SplitStage &st, const auto &h1, const auto &h2) {
          const unsigned t = u / 3, i = t / KB, kz0 = (t % KB) * P;
          one(i, kz0, int(u % 3), st, h1, h2);
        });
  } else {
    xy_units(
        unsigned(D::N * KB), ROWS * P, stage,
        [&](unsigned u, float2 *st) {
          const unsigned i = u / KB, kz0 = (u % KB) * P;
          stage_rows<P, ROWS, 8>(st, a.src[0] + (i * D::N * D::nk + kz0), D::nk);
        },
        [&](unsigned u, const float2 *st) {
          const unsigned i = u / KB, kz0 = (u % KB) * P;
#pragma unroll 1
          for (int o = 0; o < 3; ++o) one(i, kz0, o, st, NoHook(), NoHook());
        });
  }
}

// X inverse into C-space.  mode 0: the six Hessians from B0 = Y(phi),
// B1 = Y(ky phi), B2 = Y(ky^2 phi) (slot order xx yy zz xy xz yz; the factor
// -k_a k_b splits into its x and z parts): a unit stages one B tile and makes
// every Hessian that derives from it (B0: xx zz xz, B1: xy yz, B2: yy), or in
// the in-place form one Hessian (units over the six slots).
// mode 1: component c of src[c] (units also run over c < ncomp).
// units: (y < M) x (Kh/P kz blocks) x (3 sources | 6 slots | ncomp); input rows i < N
template <int M, int P> __global__ void __launch_bounds__(XY<M, P, 2 * M / 3>::threads, XY<M, P, 2 * M / 3>::minb)
    k_ff_x_inv(FArgs a) {
  using D = Dims<M>;
  using X = XY<M, P, D::N>;
  constexpr int ROWS = D::N, KB = D::Kh / P;
  const XYMem<M, P> sm(ff_smem());
  float2 *tw = sm.tw, *buf = sm.buf, *buf2 = sm.buf2, *stage = sm.stage;
  load_tw<M>(tw, a.tw);
  // output slot c of the unit at offset off (kz block kz0) from its staged rows
  auto one = [&](unsigned off, unsigned kz0, int c, const auto &st, const auto &h1, const auto &h2) {
    float2 *out = a.dst[c] + off;
    auto ld = [&](int q, int n) -> float2 {
      const int i = unpad_index(n, D::N);
      if (i < 0) return make_float2(0.f, 0.f);
      float2 v = st[i * P + q];
      if (a.mode == 0) {
        const float gx = (i != D::nh) ? float(sidx(i, D::N)) * a.kfac : 0.f;
        const float gz = float(kz0 + q) * a.kfac;
        const float f = c == 0 ? -gx * gx : c == 1 ? -1.f : c == 2 ? -gz * gz : c == 3 ? -gx : c == 4 ? -gx * gz : -gz;
        v.x *= f;
        v.y *= f;
      }
      return v;
    };
    if constexpr (X::inplace)
      xy_fft_halves_out<M, P, true>(
          buf, tw, ld,
          [&](int q, int n, float2 v0, float2 v1) {
            *reinterpret_cast<float4 *>(out + unsigned(n) * M * D::Kh + q) = make_float4(v0.x, v0.y, v1.x, v1.y);
          },
          h1, h2);
    else
      xy_fft<M, P, true, false>(buf, buf2, tw, ld,
                                [&](int q, int n, float2 v) { out[unsigned(n) * M * D::Kh + q] = v; });
  };
  if constexpr (X::inplace) {
    // mode 0: slot c from source B0 (xx zz xz), B1 (xy yz) or B2 (yy)
    const unsigned nout = a.mode ? unsigned(a.ncomp) : 6u;
    auto source = [&](unsigned c) -> unsigned {
      return a.mode ? c : (c == 1 ? 2u : (c == 3 || c == 5) ? 1u : 0u);
    };
    xy_units_inplace<M, P, ROWS>(
        unsigned(M * KB) * nout, stage, buf, unsigned(M * D::Kh),
        [&](unsigned u) {
          const unsigned c = u % nout, t = u / nout, yy = t / KB, kz0 = (t % KB) * P;
          return a.src[source(c)] + (yy * D::Kh + kz0);
        },
        [&](unsigned u, const SplitStage &st, const auto &h1, const auto &h2) {
          const unsigned c = u % nout, t = u / nout, yy = t / KB, kz0 = (t % KB) * P;
          one(yy * D::Kh + kz0, kz0, int(c), st, h1, h2);
        });
  } else {
    const unsigned nsrc = a.mode ? unsigned(a.ncomp) : 3u;
    xy_units(
        unsigned(M * KB) * nsrc, ROWS * P, stage,
        [&](unsigned u, float2 *st) {
          const unsigned s = u % nsrc, t = u / nsrc, yy = t / KB, kz0 = (t % KB) * P;
          stage_rows<P, ROWS, 16>(st, a.src[s] + (yy * D::Kh + kz0), unsigned(M * D::Kh));
        },
        [&](unsigned u, const float2 *st) {
          const unsigned s = u % nsrc, t = u / nsrc, yy = t / KB, kz0 = (t % KB) * P;
          const unsigned off = yy * D::Kh + kz0;
          // components made from source s: mode 0: B0 -> xx zz xz, B1 -> xy yz, B2 -> yy
          const int ncs = a.mode ? 1 : (s == 0 ? 3 : (s == 1 ? 2 : 1));
#pragma unroll 1
          for (int k = 0; k < ncs; ++k) {
            const int c = a.mode ? int(s) : (s == 0 ? 2 * k : (s == 1 ? (k == 0 ? 3 : 5) : 1));
            one(off, kz0, c, st, NoHook(), NoHook());
          }
        });
  }
}

// X forward: C-space layout -> B-space layout, keeping the N-grid kx.
// units: (y < M) x (Kh/P kz blocks) x (c < ncomp); input rows n < M
template <int M, int P> __global__ void __launch_bounds__(XY<M, P, M>::threads, XY<M, P, M>::minb) k_ff_x_fwd(FArgs a) {
  using D = Dims<M>;
  using X = XY<M, P, M>;
  constexpr int ROWS = M, KB = D::Kh / P;
  const XYMem<M, P> sm(ff_smem());
  float2 *tw = sm.tw, *buf = sm.buf, *buf2 = sm.buf2, *stage = sm.stage;
  load_tw<M>(tw, a.tw);
  const unsigned nc = unsigned(a.ncomp);
  auto src = [&](unsigned u) {
    const unsigned c = u % nc, t = u / nc, yy = t / KB, kz0 = (t % KB) * P;
    return a.src[c] + (yy * D::Kh + kz0);
  };
  auto one = [&](unsigned u, const auto &st, const auto &h1, const auto &h2) {
    const unsigned c = u % nc, t = u / nc, yy = t / KB, kz0 = (t % KB) * P;
    float2 *dst = a.dst[c] + (yy * D::Kh + kz0);
    auto ld = [&](int q, int n) { return st[n * P + q]; };
    if constexpr (X::inplace)
      xy_fft_halves_out<M, P, false>(
          buf, tw, ld,
          [&](int q, int k, float2 v0, float2 v1) {
            const int i = unpad_index(k, D::N);
            if (i >= 0)
              *reinterpret_cast<float4 *>(dst + unsigned(i) * M * D::Kh + q) = make_float4(v0.x, v0.y, v1.x, v1.y);
          },
          h1, h2);
    else
      xy_fft<M, P, false, false>(buf, buf2, tw, ld, [&](int q, int k, float2 v) {
        const int i = unpad_index(k, D::N);
        if (i >= 0) dst[unsigned(i) * M * D::Kh + q] = v;
      });
  };
  if constexpr (X::inplace) {
    xy_units_inplace<M, P, ROWS>(unsigned(M * KB) * nc, stage, buf, unsigned(M * D::Kh), src, one);
  } else {
    xy_units(
        unsigned(M * KB) * nc, ROWS * P, stage,
        [&](unsigned u, float2 *st) { stage_rows<P, ROWS, 16>(st, src(u), unsigned(M * D::Kh)); },
        [&](unsigned u, const float2 *st) { one(u, st, NoHook(), NoHook()); });
  }
}

// Y forward.  MODE 0: keep the N-grid ky, zero every Nyquist index and the
// mean, scale by fac / -k^2 -> N-grid k-space (kz = N/2 plane zeroed);
// MODE 1: truncation of a convolve3 pair (zero outside the N-grid modes and on
// Nyquist, scale by fac) and inverse y transform -> B-space (may be in place:
// a unit's tile is staged whole before any of its outputs is written, and no
// other unit touches it).
// units: (i < N) x (Kh/P kz blocks) x (c < ncomp); input rows n < M
template <int M, int P, int MODE>
__global__ void __launch_bounds__(XY<M, P, M>::threads, XY<M, P, M>::minb) k_ff_y_fwd(FArgs a) {
  using D = Dims<M>;
  using T = Tile<M, P, true>;
  using X = XY<M, P, M>;
  constexpr int ROWS = M, KB = D::Kh / P;
  const XYMem<M, P> sm(ff_smem());
  float2 *tw = sm.tw, *buf = sm.buf, *buf2 = sm.buf2, *stage = sm.stage;
  load_tw<M>(tw, a.tw);
  const unsigned nc = unsigned(a.ncomp);
  auto src = [&](unsigned u) {
    const unsigned c = u % nc, t = u / nc, i = t / KB, kz0 = (t % KB) * P;
    return a.src[c] + (i * M * D::Kh + kz0);
  };
  auto one = [&](unsigned u, const auto &st, const auto &h1, const auto &h2) {
    const unsigned c = u % nc, t = u / nc, i = t / KB, kz0 = (t % KB) * P;
    float2 *dst = a.dst[c];
    auto ld = [&](int q, int n) { return st[n * P + q]; };
    if constexpr (MODE == 0) {
      const float kx = float(sidx(int(i), D::N)) * a.kfac;
      float2 *out = dst + i * D::N * D::nk + kz0;
      // the N-grid spectrum's rows (nk apart: 8-byte aligned only)
      auto put = [&](int q, int k, float2 v) {
        const int j = unpad_index(k, D::N);
        if (j < 0) return;
        const int kz = int(kz0) + q;
        float2 r = make_float2(0.f, 0.f);
        if (int(i) != D::nh && j != D::nh && (int(i) | j | kz) != 0) {
          const float ky = float(sidx(j, D::N)) * a.kfac, kk = float(kz) * a.kfac;
          const float f = -a.fac * __frcp_rn(kx * kx + ky * ky + kk * kk);
          r = make_float2(v.x * f, v.y * f);
        }
        out[unsigned(j) * D::nk + q] = r;
      };
      if constexpr (X::inplace)
        xy_fft_halves_out<M, P, false>(
            buf, tw, ld,
            [&](int q, int k, float2 v0, float2 v1) {
              put(q, k, v0);
              put(q + 1, k, v1);
            },
            h1, h2);
      else
        xy_fft<M, P, false, false>(buf, buf2, tw, ld, put);
      if (kz0 == 0)
        for (int j = threadIdx.x; j < D::N; j += blockDim.x)
          dst[(i * D::N + j) * D::nk + D::nh] = make_float2(0.f, 0.f);
    } else {
      float2 *out = dst + (i * M * D::Kh + kz0);
      const bool row_kept = int(i) != D::nh;
      float2 *mid = obuf<M>(buf, buf2);
      auto trunc = [&](int q, int k, float2 v) {
        const int j = unpad_index(k, D::N);
        const bool keep = row_kept && j >= 0 && j != D::nh;
        mid[T::at(q, k)] = keep ? make_float2(v.x * a.fac, v.y * a.fac) : make_float2(0.f, 0.f);
      };
      auto lm = [&](int q, int n) { return mid[T::at(q, n)]; };
      // in-place form: one copy of the transform's code for both transforms,
      // the inverse as the conjugate of the forward transform of the
      // conjugate (negations are exact: the same roundings); two inlined
      // transforms spill there (456 bytes a thread; 40 this way).  The
      // 8-pencil lean form keeps two transforms: its single copy, with the
      // phase tests in the loads and stores, measured slower (768^3 YF-trunc
      // 12.2 -> 17.2 ms)
      if constexpr (X::inplace) {
#pragma unroll 1
        for (int ph = 0; ph < 2; ++ph) {
          xy_fft_halves<M, P, false>(
              buf, tw,
              [&](int q, int n) -> float2 {
                if (ph == 0) return st[n * P + q];
                const float2 v = mid[T::at(q, n)];
                return make_float2(v.x, -v.y);
              },
              [&](int q, int k, float2 v) {
                if (ph == 0)
                  trunc(q, k, v);
                else
                  buf[k * P + q] = make_float2(v.x, -v.y);
              },
              [&] {
                if (ph == 0) h1();
              });
          __syncthreads();
        }
        xy_store_rows<M, P>(
            buf,
            [&](int q, int n, float2 v0, float2 v1) {
              *reinterpret_cast<float4 *>(out + unsigned(n) * D::Kh + q) = make_float4(v0.x, v0.y, v1.x, v1.y);
            },
            h2);
      } else {
        xy_fft<M, P, false, false>(buf, buf2, tw, ld, trunc);
        __syncthreads();
        xy_fft<M, P, true>(buf, buf2, tw, lm, [&](int q, int n, float2 v) { out[unsigned(n) * D::Kh + q] = v; });
      }
    }
  };
  if constexpr (X::inplace) {
    xy_units_inplace<M, P, ROWS>(unsigned(D::N * KB) * nc, stage, buf, unsigned(D::Kh), src, one);
  } else {
    xy_units(
        unsigned(D::N * KB) * nc, ROWS * P, stage,
        [&](unsigned u, float2 *st) { stage_rows<P, ROWS, 16>(st, src(u), unsigned(D::Kh)); },
        [&](unsigned u, const float2 *st) { one(u, st, NoHook(), NoHook()); });
  }
}

// ---------------------------------------------------------------------------
// z row kernels (persistent): each CTA walks rows blockIdx.x, + gridDim.x, ...
// RW rows at a time.  The NIN C-space input spectra of the next row group are
// fetched into shared memory by bulk asynchronous copies (one thread issues
// them, an mbarrier counts the bytes) while the current group's sources and
// forward transforms run, so global latency stays off the FFT critical path
// (one stage only: shared memory is what bounds the CTAs per SM).  Inverse z transforms
// (fields paired into complex pencils, G per round) fill h[w][c][z]; the
// sources are formed in place; NOUT real sources per row go through forward z
// transforms and their kz < Kh spectra to global memory (D-space).
// ---------------------------------------------------------------------------
constexpr int kMbarSpins = 1 << 20;  // bounded mbarrier wait (try_wait suspends between polls)

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n"
      " .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
  for (int it = 0; it < kMbarSpins; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
// global -> shared bulk copy (16-byte aligned, size a multiple of 16)
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// z-pass shape: RW rows per group, G pencils per transform; WIDE: one CTA per
// SM by shared memory and registers (the wide shape of the long lengths)
template <int M, int RW, int G, int NIN, bool WIDE = false> struct ZR {
  using D = Dims<M>;
  static constexpr int nin_pad = NIN + (NIN & 1);
  static constexpr int threads = G * Fac<M>::maxJ;
  static constexpr int srow = NIN * D::Kh;  // float2 per row in the stage
  static constexpr size_t head = 32;        // two mbarriers and a status word
  static constexpr size_t smem = head + size_t(TwTab<M>::elems) * sizeof(float2) + size_t(RW * srow) * sizeof(float2) +
                                 size_t(RW) * nin_pad * M * sizeof(float) +
                                 size_t(2 * Tile<M, G, false>::elems) * sizeof(float2);
  // CTAs per SM: by shared memory (228 KB per SM) and by at least 56
  // registers a thread (no spills for the 2LPT pass at 384 with five CTAs),
  // at most five (small CTAs of the short lengths keep their registers)
  static constexpr int by_smem = int(233472 / (smem + 1024));
  static constexpr int by_regs0 = 65536 / (threads * 56) < 1 ? 1 : 65536 / (threads * 56);
  static constexpr int by_regs = by_regs0 < 5 ? by_regs0 : 5;
  static constexpr int minb = WIDE ? 1 : (by_regs < by_smem ? by_regs : (by_smem < 1 ? 1 : by_smem));
};

// issues the bulk copies of row group g (RW rows x NIN spectra) into stage
template <int M, int RW, int NIN>
__device__ __forceinline__ void z_fetch(const FArgs &a, size_t g, float2 *stage, uint64_t *bar) {
  using D = Dims<M>;
  constexpr uint32_t bytes = uint32_t(D::Kh) * sizeof(float2);
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the stage was last read by the generic proxy
  mbar_expect_tx(bar, bytes * RW * NIN);
  for (int w = 0; w < RW; ++w)
    for (int c = 0; c < NIN; ++c)
      bulk_g2s(stage + (w * NIN + c) * D::Kh, a.src[c] + (g * RW + w) * D::Kh, bytes, bar);
}

// inverse z transforms of the staged spectra into the pair-interleaved
// scratch h2[w * NP/2 + c/2][z] (float2: field c in x for even c, y for odd c)
template <int M, int RW, int G, int NIN>
__device__ __forceinline__ void z_inverse(const float2 *stage, float *h, float2 *buf, float2 *buf2, const float2 *tw) {
  using D = Dims<M>;
  constexpr int NP = ZR<M, RW, G, NIN>::nin_pad;
  constexpr int NPI = RW * (NP / 2);  // complex pencils
#pragma unroll 1
  for (int g0 = 0; g0 < NPI; g0 += G) {
    pencil_fft<M, G, false, true, false>(
        buf, buf2, tw,
        [&](int q, int n) -> float2 {
          const int g = g0 + q;
          if (g >= NPI) return make_float2(0.f, 0.f);
          const int w = g / (NP / 2), c0 = 2 * (g - w * (NP / 2)), c1 = c0 + 1;
          int m;
          bool conj;
          if (n < D::Kh) {
            m = n;
            conj = false;
          } else if (n > M - D::Kh) {
            m = M - n;
            conj = true;
          } else {
            return make_float2(0.f, 0.f);
          }
          const float2 *row = stage + w * NIN * D::Kh;
          float2 va = row[c0 * D::Kh + m];
          float2 vb = c1 < NIN ? row[c1 * D::Kh + m] : make_float2(0.f, 0.f);
          if (m == 0) {
            va.y = 0.f;
            vb.y = 0.f;
          }
          return conj ? pack_pair_conj(va, vb) : pack_pair(va, vb);
        },
        [&](int q, int n, float2 v) {
          const int g = g0 + q;
          if (g >= NPI) return;
          // fields (c0, c0 + 1) of row w are pair g of h2[g][z] = (x: c0, y: c0 + 1)
          reinterpret_cast<float2 *>(h)[g * M + n] = v;
        });
  }
  __syncthreads();
}

// forward z transforms of NOUT real sources per row held in the pair scratch
// (source o of row w in field slot o) and the kz < Kh spectra written to dst[o]
template <int M, int RW, int G0, int NP, int NOUT>
__device__ __forceinline__ void z_forward(const FArgs &a, size_t r0, const float *h, float2 *buf, float2 *buf2,
                                          const float2 *tw) {
  using D = Dims<M>;
  constexpr int NR = RW * NOUT;      // real outputs
  constexpr int NPO = (NR + 1) / 2;  // complex pencils
  constexpr int G = G0 < NPO ? G0 : NPO;
  using T = Tile<M, G, false>;
  float2 *ob = obuf<M>(buf, buf2);
#pragma unroll 1
  for (int g0 = 0; g0 < NPO; g0 += G) {
    pencil_fft<M, G, false, false, false>(
        buf, buf2, tw,
        [&](int q, int n) -> float2 {
          const int g = g0 + q;
          if (g >= NPO) return make_float2(0.f, 0.f);
          if constexpr (NOUT % 2 == 0) {
            // sources (2g', 2g'+1) of one row share a pair slot
            const int w = g / (NOUT / 2), o = 2 * (g - w * (NOUT / 2));
            return reinterpret_cast<const float2 *>(h)[(w * (NP / 2) + o / 2) * M + n];
          } else {
            const int f0 = 2 * g, f1 = f0 + 1;
            auto at = [&](int f) {
              const int w = f / NOUT, o = f % NOUT;
              return h[((w * (NP / 2) + o / 2) * M + n) * 2 + (o & 1)];
            };
            return make_float2(at(f0), f1 < NR ? at(f1) : 0.f);
          }
        },
        [&](int q, int k, float2 v) { ob[T::at(q, k)] = v; });
    __syncthreads();
    for (int t = threadIdx.x; t < G * D::Kh; t += blockDim.x) {
      const int q = t / D::Kh, k = t - q * D::Kh, g = g0 + q;
      if (g >= NPO) continue;
      const float2 z = ob[T::at(q, k)], zm = ob[T::at(q, k == 0 ? 0 : M - k)];
      float2 sa, sb;
      unpack_pair(z, zm, sa, sb);
      const int f0 = 2 * g, f1 = f0 + 1;
      a.dst[f0 % NOUT][(r0 + f0 / NOUT) * D::Kh + k] = sa;
      if (f1 < NR) a.dst[f1 % NOUT][(r0 + f1 / NOUT) * D::Kh + k] = sb;
    }
    // the next round's transform writes ob; after the last round the barrier
    // at the top of the next row group stands before any write to it
    if (g0 + G < NPO) __syncthreads();
  }
}

// the persistent row loop shared by ZSRC2 and ZSRC3; `sources(pairs)` forms
// the sources of one element in place (pairs[p * M]: fields 2p, 2p + 1).  One stage: the next group's copies are
// issued as soon as the inverse transforms have read the current one, and
// land while the sources and the forward transforms run.
template <int M, int RW, int G, int NIN, int NOUT, class Src>
__device__ __forceinline__ void z_rows(const FArgs &a, const Src &sources) {
  using Z = ZR<M, RW, G, NIN>;
  constexpr int NP = Z::nin_pad;
  char *base = reinterpret_cast<char *>(ff_smem());
  uint64_t *bar = reinterpret_cast<uint64_t *>(base);
  volatile int *flag = reinterpret_cast<volatile int *>(base + 16);
  float2 *tw = reinterpret_cast<float2 *>(base + Z::head);
  float2 *stage = tw + TwTab<M>::elems;  // RW * srow
  float *h = reinterpret_cast<float *>(stage + RW * Z::srow);
  float2 *buf = reinterpret_cast<float2 *>(h + RW * NP * M);
  float2 *buf2 = buf + Tile<M, G, false>::elems;
  const size_t ngroups = size_t(M) * M / RW;
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    *flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  load_tw_steps<M>(tw, a.tw);  // includes a barrier
  size_t g = blockIdx.x;
  if (threadIdx.x == 0 && g < ngroups) z_fetch<M, RW, NIN>(a, g, stage, bar);
#pragma unroll 1
  for (uint32_t it = 0; g < ngroups; ++it, g += gridDim.x) {
    const size_t gn = g + gridDim.x;
    if (threadIdx.x == 0 && !mbar_wait_bounded(bar, it & 1)) *flag = 1;
    __syncthreads();
    if (*flag) {
      // the copies did not land: report, let them finish (bounded), leave
      if (threadIdx.x == 0) {
        if (a.status) atomicExch(a.status, 1);
        mbar_wait_bounded(bar, it & 1);
      }
      return;
    }
    z_inverse<M, RW, G, NIN>(stage, h, buf, buf2, tw);  // ends with a barrier: the stage is free
    if (threadIdx.x == 0 && gn < ngroups) z_fetch<M, RW, NIN>(a, gn, stage, bar);
    for (int t = threadIdx.x; t < RW * M; t += blockDim.x) {
      const int w = t / M, n = t - w * M;
      sources(reinterpret_cast<float2 *>(h) + size_t(w) * (NP / 2) * M + n);
    }
    __syncthreads();
    z_forward<M, RW, G, NP, NOUT>(a, g * RW, h, buf, buf2, tw);
  }
}

// the sources of one z element from its pair slots hp[c * stride] (slot c:
// fields 2c, 2c + 1), formed in place
// ZSRC2: phi1 Hessians (src[0..5], C-space) -> 2LPT source (dst[0]) and, with
// mode 1, the five first-pair products of convolve3 (dst[1..5]).
template <int MODE> struct Src2 {
  __device__ __forceinline__ void operator()(float2 *hp, int stride) const {
    float v[6], s[6];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float2 x = hp[c * stride];
      v[2 * c] = x.x;
      v[2 * c + 1] = x.y;
    }
    s[0] = src_phi2(v);
    if (MODE) {
      pair_products(v, s + 1);
#pragma unroll
      for (int c = 0; c < 3; ++c) hp[c * stride] = make_float2(s[2 * c], s[2 * c + 1]);
    } else {
      hp[0].x = s[0];
    }
  }
};
// ZSRC3: phi1 Hessians src[0..5], phi2 Hessians src[6..11] and the truncated
// pair products src[12..16] (C-space) -> phi3 source (dst[0]) and A3 (dst[1..3]).
// The outputs may alias inputs: a row's spectra are staged before any of its
// outputs is written.
struct Src3 {
  __device__ __forceinline__ void operator()(float2 *hp, int stride) const {
    float f[18], s[4];
#pragma unroll
    for (int c = 0; c < 9; ++c) {
      const float2 x = hp[c * stride];
      f[2 * c] = x.x;
      f[2 * c + 1] = x.y;
    }
    src_phi3(f, f + 6, f + 12, s);
    hp[0] = make_float2(s[0], s[1]);
    hp[stride] = make_float2(s[2], s[3]);
  }
};

template <int M, int RW, int G, int MODE, bool WIDE>
__global__ void __launch_bounds__(ZR<M, RW, G, 6, WIDE>::threads, ZR<M, RW, G, 6, WIDE>::minb) k_ff_zsrc2(FArgs a) {
  z_rows<M, RW, G, 6, MODE ? 6 : 1>(a, [&](float2 *hp) { Src2<MODE>()(hp, M); });
}

template <int M, int RW, int G, bool WIDE>
__global__ void __launch_bounds__(ZR<M, RW, G, 17, WIDE>::threads, ZR<M, RW, G, 17, WIDE>::minb) k_ff_zsrc3(FArgs a) {
  z_rows<M, RW, G, 17, 4>(a, [&](float2 *hp) { Src3()(hp, M); });
}

// ---------------------------------------------------------------------------
// Warp z passes (z tile 4): one row per group, three warps per CTA, each
// complex pencil transformed by one warp in place in its own padded slot of
// the row scratch with __syncwarp between the steps: three CTA barriers per
// row (staged inputs in, inverse transforms done, sources formed) instead of
// two per transform.  For lengths whose steps have at most 96 butterflies
// (three per lane).
// ---------------------------------------------------------------------------
template <int L> struct WP {
  static constexpr int padL = L + (L >> 4);
  MFX_HD static int at(int n) { return n + (n >> 4); }
};

template <int L, int R, int NS, bool INV, class Ld, class St>
__device__ __forceinline__ void warp_step(const float2 *tw, int lane, const Ld &ld, const St &st) {
  using S = Step<L, R, NS, INV>;
  constexpr int I = (S::J + 31) / 32;
  float2 v[I][R];
#pragma unroll
  for (int it = 0; it < I; ++it) {
    const int j = lane + 32 * it;
    if (j < S::J) S::template gather<true>(j, ld, tw, v[it]);
  }
  __syncwarp();
#pragma unroll
  for (int it = 0; it < I; ++it) {
    const int j = lane + 32 * it;
    if (j < S::J) S::scatter(j, st, v[it]);
  }
  __syncwarp();
}

// one pencil of length L through one warp, in place in p (WP layout): ld(n)
// gives input n (it may read p); output k lands in p[WP<L>::at(k)]
template <int L, bool INV, class Ld>
__device__ __forceinline__ void warp_fft(float2 *p, const float2 *tw, const Ld &ld) {
  using F = Fac<L>;
  const int lane = int(threadIdx.x) & 31;
  auto lp = [&](int n) { return p[WP<L>::at(n)]; };
  auto sp = [&](int n, float2 x) { p[WP<L>::at(n)] = x; };
  warp_step<L, F::R1, 1, INV>(tw, lane, ld, sp);
  if constexpr (F::steps == 3) warp_step<L, F::R2, F::R1, INV>(tw, lane, lp, sp);
  constexpr int RL = F::steps == 3 ? F::R3 : F::R2;
  warp_step<L, RL, L / RL, INV>(tw, lane, lp, sp);
}

template <int M, int NIN> struct ZW {
  using D = Dims<M>;
  static constexpr int NPI = (NIN + (NIN & 1)) / 2;  // complex pencils of the inverse transforms
  static constexpr int warps = 3;                     // each takes NPI / 3 pencils (3 or 1)
  static_assert(NPI % warps == 0, "whole pencils per warp");
  static constexpr int threads = 32 * warps;
  static constexpr int padL = WP<M>::padL;
  static constexpr size_t head = 32;
  static constexpr size_t smem = head + size_t(TwTab<M>::elems) * sizeof(float2) + size_t(NIN * D::Kh) * sizeof(float2) +
                                 size_t(NPI * padL) * sizeof(float2);
  // CTAs per SM by shared memory and by about 168 registers a thread (a lane
  // holds up to three butterflies of a step; 128 spilled in the 2LPT pass)
  static constexpr int by_smem = int(233472 / (smem + 1024));
  static constexpr int by_regs = 65536 / (threads * 168) < 1 ? 1 : 65536 / (threads * 168);
  static constexpr int minb = by_regs < by_smem ? by_regs : (by_smem < 1 ? 1 : by_smem);
  static constexpr bool ok = Fac<M>::maxJ <= 96;
};

template <int M, int NIN, int NOUT, class Src>
__device__ __forceinline__ void z_rows_w(const FArgs &a, const Src &sources) {
  using Z = ZW<M, NIN>;
  using D = Dims<M>;
  constexpr int NPO = (NOUT + 1) / 2, padL = Z::padL;
  char *base = reinterpret_cast<char *>(ff_smem());
  uint64_t *bar = reinterpret_cast<uint64_t *>(base);
  volatile int *flag = reinterpret_cast<volatile int *>(base + 16);
  float2 *tw = reinterpret_cast<float2 *>(base + Z::head);
  float2 *stage = tw + TwTab<M>::elems;  // [c][Kh]
  float2 *h = stage + NIN * D::Kh;  // pencil p at h + p * padL (WP layout)
  const size_t ngroups = size_t(M) * M;
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    *flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  load_tw_steps<M>(tw, a.tw);  // includes a barrier
  const int warp = int(threadIdx.x) >> 5, lane = int(threadIdx.x) & 31;
  size_t g = blockIdx.x;
  if (threadIdx.x == 0 && g < ngroups) z_fetch<M, 1, NIN>(a, g, stage, bar);
#pragma unroll 1
  for (uint32_t it = 0; g < ngroups; ++it, g += gridDim.x) {
    const size_t gn = g + gridDim.x;
    if (threadIdx.x == 0 && !mbar_wait_bounded(bar, it & 1)) *flag = 1;
    __syncthreads();
    if (*flag) {
      // the copies did not land: report, let them finish (bounded), leave
      if (threadIdx.x == 0) {
        if (a.status) atomicExch(a.status, 1);
        mbar_wait_bounded(bar, it & 1);
      }
      return;
    }
#pragma unroll 1
    for (int pc = warp; pc < Z::NPI; pc += Z::warps) {
      // inverse transform of pencil pc: fields (2 pc, 2 pc + 1) as A + iB
      const int c0 = 2 * pc, c1 = c0 + 1;
      warp_fft<M, true>(h + pc * padL, tw, [&](int n) -> float2 {
        int m;
        bool conj;
        if (n < D::Kh) {
          m = n;
          conj = false;
        } else if (n > M - D::Kh) {
          m = M - n;
          conj = true;
        } else {
          return make_float2(0.f, 0.f);
        }
        float2 va = stage[c0 * D::Kh + m];
        float2 vb = c1 < NIN ? stage[c1 * D::Kh + m] : make_float2(0.f, 0.f);
        if (m == 0) {
          va.y = 0.f;
          vb.y = 0.f;
        }
        return conj ? pack_pair_conj(va, vb) : pack_pair(va, vb);
      });
    }
    __syncthreads();  // the stage is free; every field of the row is in h
    if (threadIdx.x == 0 && gn < ngroups) z_fetch<M, 1, NIN>(a, gn, stage, bar);
    for (int n = threadIdx.x; n < M; n += blockDim.x) sources(h + WP<M>::at(n), padL);
    __syncthreads();
#pragma unroll 1
    for (int pc = warp; pc < NPO; pc += Z::warps) {
      // forward transform of sources (2 pc, 2 pc + 1) and their kz < Kh spectra
      float2 *hp = h + pc * padL;
      const bool odd_last = (NOUT & 1) && pc == NPO - 1;
      warp_fft<M, false>(hp, tw, [&](int n) -> float2 {
        float2 v = hp[WP<M>::at(n)];
        if (odd_last) v.y = 0.f;
        return v;
      });
      const int f0 = 2 * pc, f1 = f0 + 1;
      for (int k = lane; k < D::Kh; k += 32) {
        const float2 z = hp[WP<M>::at(k)], zm = hp[WP<M>::at(k == 0 ? 0 : M - k)];
        float2 sa, sb;
        unpack_pair(z, zm, sa, sb);
        a.dst[f0][g * D::Kh + k] = sa;
        if (f1 < NOUT) a.dst[f1][g * D::Kh + k] = sb;
      }
    }
    // h is rewritten after the barrier at the top of the next row
  }
}

template <int M, int MODE>
__global__ void __launch_bounds__(ZW<M, 6>::threads, ZW<M, 6>::minb) k_ff_zsrc2w(FArgs a) {
  z_rows_w<M, 6, MODE ? 6 : 1>(a, Src2<MODE>());
}

template <int M>
__global__ void __launch_bounds__(ZW<M, 17>::threads, ZW<M, 17>::minb) k_ff_zsrc3w(FArgs a) {
  z_rows_w<M, 17, 4>(a, Src3());
}
#endif

}  // namespace ff
}  // namespace mfx
