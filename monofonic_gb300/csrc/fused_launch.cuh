// Host-side launchers of the fused transforms (fused.cuh), one instantiation
// per padded length M (the ff_m*.cu translation units compile them in
// parallel).  ff_launch_m<M> launches one pass with pencil tile `p`: pencils
// per CTA for the x/y passes (4, 8, 16 or 32); for the z passes 1 or 2 rows per
// CTA, 3: the wide shape (one row, many pencils per transform), 4: the warp
// passes (one row, one warp per pencil).
#pragma once
#include <cuda_runtime.h>

#include "fused.cuh"
#include "fused_asm.cuh"

namespace mfx {
namespace ff {

enum FFOp { FF_Y3 = 0, FF_XINV = 1, FF_XFWD = 2, FF_YFWD = 3, FF_ZSRC2 = 4, FF_ZSRC3 = 5, FF_NOPS = 6 };

// complex pencils per round of the z passes: the largest divisor of the row
// tile's pencil count that keeps the CTA within 256 threads (small CTAs, so
// that the barriers of one leave the SM to the others)
constexpr int zg_pick(int npi, int cap) {
  int g = 1;
  for (int d = 1; d <= npi; ++d)
    if (npi % d == 0 && d <= cap) g = d;
  return g;
}
template <int M, int RW, int NIN> struct ZG {
  static constexpr int npi = RW * ((NIN + (NIN & 1)) / 2);
  static constexpr int cap = 256 / Fac<M>::maxJ > 0 ? 256 / Fac<M>::maxJ : 1;
  static constexpr int G = zg_pick(npi, cap);
};

constexpr size_t kFFSmemMax = 227 * 1024;

// the wide z shape (tile 3): one row per group and as many pencils per
// transform as about 92 registers a thread (704 threads) and the shared
// memory allow (one CTA per SM), the fewest rounds per row and, among those,
// the fewest idle pencils.  For the long padded lengths, whose narrow shapes
// leave only a few warps per SM.
constexpr size_t zw_smem(int M, int NIN, int G, int twe) {
  const size_t kh = size_t(M / 3), np = size_t(NIN + (NIN & 1));
  return 32 + size_t(twe) * 8 + NIN * kh * 8 + np * size_t(M) * 4 + 2 * size_t(G) * size_t(M + (M >> 4)) * 8;
}
constexpr int zw_pick(int M, int NIN, int maxJ, int twe) {
  const int npi = (NIN + (NIN & 1)) / 2;
  int gmax = 0;
  for (int g = 1; g <= npi && g * maxJ <= 704 && zw_smem(M, NIN, g, twe) <= kFFSmemMax; ++g) gmax = g;
  if (gmax == 0) return 0;
  const int rounds = (npi + gmax - 1) / gmax;
  return (npi + rounds - 1) / rounds;
}
template <int M, int NIN> struct ZGW {
  static constexpr int G = zw_pick(M, NIN, Fac<M>::maxJ, TwTab<M>::elems);
};

template <int M, int RW> constexpr bool ff_z_fits() {
  if constexpr (RW == 4) {
    return ZW<M, 17>::ok && ZW<M, 17>::smem <= kFFSmemMax && ZW<M, 6>::smem <= kFFSmemMax;
  } else if constexpr (RW == 3) {
    return ZGW<M, 6>::G > 0 && ZGW<M, 17>::G > 0;
  } else {
    return ZR<M, RW, ZG<M, RW, 6>::G, 6>::smem <= kFFSmemMax && ZR<M, RW, ZG<M, RW, 17>::G, 17>::smem <= kFFSmemMax;
  }
}

// an x/y tile of P pencils fits one CTA (threads, shared memory) and the kz
// range; the in-place form needs a side buffer of at least one row
template <int M, int P> constexpr bool xy_ok() {
  return (M / 3) % P == 0 && XY<M, P, M>::threads <= 1024 && XY<M, P, M>::smem <= kFFSmemMax &&
         XY<M, P, 2 * M / 3>::smem <= kFFSmemMax && (!XY<M, P, M>::inplace || XY<M, P, M>::side > 0) &&
         (!XY<M, P, 2 * M / 3>::inplace || XY<M, P, 2 * M / 3>::side > 0);
}

template <int M> bool ff_valid_m(int op, int p) {
  if (op == FF_ZSRC2 || op == FF_ZSRC3)
    return (p == 1 && ff_z_fits<M, 1>()) || (p == 2 && ff_z_fits<M, 2>()) || (p == 3 && ff_z_fits<M, 3>()) ||
           (p == 4 && ff_z_fits<M, 4>());
  if (op < 0 || op >= FF_NOPS) return false;
  return (p == 4 && xy_ok<M, 4>()) || (p == 8 && xy_ok<M, 8>()) || (p == 16 && xy_ok<M, 16>()) ||
         (p == 32 && xy_ok<M, 32>());
}

// lets a kernel instance use up to 227 KB of dynamic shared memory; the
// static flag is per expansion site, i.e. per kernel instance, and per device
#define MFX_FF_ALLOW_SMEM(kernel)                                                               \
  do {                                                                                          \
    static int done_[64] = {};                                                                  \
    int dev_ = 0;                                                                               \
    cudaGetDevice(&dev_);                                                                       \
    if (dev_ >= 0 && dev_ < 64 && !done_[dev_]) {                                               \
      cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024); \
      done_[dev_] = 1;                                                                          \
    }                                                                                           \
  } while (0)

// persistent grid: as many CTAs as fit on the device at once, at most `units`
template <class K> static unsigned ff_persistent_grid(K kernel, int threads, size_t smem, size_t units) {
  int dev = 0, nsm = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, smem) != cudaSuccess || per < 1) per = 1;
  const size_t g = size_t(nsm > 0 ? nsm : 1) * size_t(per);
  return unsigned(g < units ? g : units);
}

// launches a persistent kernel instance; the grid is computed once per
// instance (the devices of one engine are of one kind)
#define MFX_FF_PERSISTENT(kernel, threads, smem, units, stream, args)                   \
  do {                                                                              \
    MFX_FF_ALLOW_SMEM(kernel);                                                      \
    static unsigned grid_ = 0;                                                      \
    if (!grid_) grid_ = ff_persistent_grid(kernel, threads, smem, size_t(1) << 40); \
    const unsigned g_ = grid_ < (units) ? grid_ : unsigned(units);                   \
    kernel<<<g_, threads, smem, stream>>>(args);                                    \
  } while (0)

template <int M, int P> cudaError_t ff_launch_xy(int op, const FArgs &a, cudaStream_t s) {
  if constexpr (!xy_ok<M, P>()) {
    return cudaErrorInvalidConfiguration;
  } else {
    constexpr int N = 2 * M / 3, KB = (M / 3) / P;
    using XN = XY<M, P, N>;
    using XM = XY<M, P, M>;
    const size_t nc = size_t(a.ncomp > 0 ? a.ncomp : 1);
    switch (op) {
      // the in-place form makes one output a unit: Y3's three, mode 0's six Hessians
      case FF_Y3:
        MFX_FF_PERSISTENT((k_ff_y3<M, P>), XN::threads, XN::smem, size_t(N) * KB * (XN::inplace ? 3 : 1), s, a);
        break;
      case FF_XINV:
        MFX_FF_PERSISTENT((k_ff_x_inv<M, P>), XN::threads, XN::smem,
                          size_t(M) * KB * (a.mode ? nc : (XN::inplace ? 6 : 3)), s, a);
        break;
      case FF_XFWD:
        MFX_FF_PERSISTENT((k_ff_x_fwd<M, P>), XM::threads, XM::smem, size_t(M) * KB * nc, s, a);
        break;
      case FF_YFWD:
        if (a.mode == 0)
          MFX_FF_PERSISTENT((k_ff_y_fwd<M, P, 0>), XM::threads, XM::smem, size_t(N) * KB * nc, s, a);
        else
          MFX_FF_PERSISTENT((k_ff_y_fwd<M, P, 1>), XM::threads, XM::smem, size_t(N) * KB * nc, s, a);
        break;
      default:
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
  }
}

// z tile p: 1 and 2 rows per group (two tile buffers), 3 the wide shape, 4
// the warp passes
template <int M, int P> cudaError_t ff_launch_z(int op, const FArgs &a, cudaStream_t s) {
  if constexpr (!ff_z_fits<M, P>()) {
    return cudaErrorInvalidConfiguration;
  } else if constexpr (P == 4) {
    const size_t groups = size_t(M) * M;
    if (op == FF_ZSRC2) {
      using Z = ZW<M, 6>;
      if (a.mode)
        MFX_FF_PERSISTENT((k_ff_zsrc2w<M, 1>), Z::threads, Z::smem, groups, s, a);
      else
        MFX_FF_PERSISTENT((k_ff_zsrc2w<M, 0>), Z::threads, Z::smem, groups, s, a);
    } else {
      using Z = ZW<M, 17>;
      MFX_FF_PERSISTENT((k_ff_zsrc3w<M>), Z::threads, Z::smem, groups, s, a);
    }
    return cudaGetLastError();
  } else {
    constexpr int RW = P == 3 ? 1 : P;
    constexpr bool W = P == 3;
    const size_t groups = size_t(M) * M / RW;
    if (op == FF_ZSRC2) {
      constexpr int G = W ? ZGW<M, 6>::G : ZG<M, RW, 6>::G;
      using Z = ZR<M, RW, G, 6, W>;
      static_assert(Z::smem <= kFFSmemMax, "z tile exceeds shared memory");
      if (a.mode)
        MFX_FF_PERSISTENT((k_ff_zsrc2<M, RW, G, 1, W>), Z::threads, Z::smem, groups, s, a);
      else
        MFX_FF_PERSISTENT((k_ff_zsrc2<M, RW, G, 0, W>), Z::threads, Z::smem, groups, s, a);
    } else {
      constexpr int G = W ? ZGW<M, 17>::G : ZG<M, RW, 17>::G;
      using Z = ZR<M, RW, G, 17, W>;
      static_assert(Z::smem <= kFFSmemMax, "z tile exceeds shared memory");
      MFX_FF_PERSISTENT((k_ff_zsrc3<M, RW, G, W>), Z::threads, Z::smem, groups, s, a);
    }
    return cudaGetLastError();
  }
}

template <int M> cudaError_t ff_launch_m(int op, int p, const FArgs &a, cudaStream_t s) {
  if (!ff_valid_m<M>(op, p)) return cudaErrorInvalidConfiguration;
  if (op == FF_ZSRC2 || op == FF_ZSRC3) {
    switch (p) {
      case 1: return ff_launch_z<M, 1>(op, a, s);
      case 2: return ff_launch_z<M, 2>(op, a, s);
      case 3: return ff_launch_z<M, 3>(op, a, s);
      default: return ff_launch_z<M, 4>(op, a, s);
    }
  }
  switch (p) {
    case 4: return ff_launch_xy<M, 4>(op, a, s);
    case 8: return ff_launch_xy<M, 8>(op, a, s);
    case 16: return ff_launch_xy<M, 16>(op, a, s);
    default: return ff_launch_xy<M, 32>(op, a, s);
  }
}

// the fused assembly passes on the N-grid (N = 2M/3) of padded length M
enum FAOp { FA_X = 0, FA_Y = 1, FA_Z = 2 };

template <int M> cudaError_t fa_launch_m(int op, bool plt, const FAArgs &a, cudaStream_t s) {
  constexpr int N = 2 * M / 3;
  using F = FA<N>;
  if constexpr (F::s1 > kFFSmemMax || F::s2 > kFFSmemMax || F::s3 > kFFSmemMax || F::t1 > 1024) {
    return cudaErrorInvalidConfiguration;
  } else {
    constexpr size_t units1 = size_t(N) * (F::Kh / F::P);
    switch (op) {
      case FA_X:
        if (a.nsub > 1 && a.halves) {
          if constexpr (F::halves) {
            if (plt) MFX_FF_PERSISTENT((k_fa_x_halves<N, true>), F::t1h, F::s1h + (F::halves_xs ? F::s1h_x : 0), size_t(N) * (F::Kh / F::P8), s, a);
            else MFX_FF_PERSISTENT((k_fa_x_halves<N, false>), F::t1h, F::s1h + (F::halves_xs ? F::s1h_x : 0), size_t(N) * (F::Kh / F::P8), s, a);
          } else {
            return cudaErrorInvalidValue;
          }
        } else if (a.nsub > 1) {
          if constexpr (F::keep) {
            if (plt) MFX_FF_PERSISTENT((k_fa_x<N, true, true>), F::t1k, F::s1k, units1, s, a);
            else MFX_FF_PERSISTENT((k_fa_x<N, false, true>), F::t1k, F::s1k, units1, s, a);
          } else {
            return cudaErrorInvalidValue;
          }
        } else {
          if (plt) MFX_FF_PERSISTENT((k_fa_x<N, true, false>), F::t1, F::s1, units1, s, a);
          else MFX_FF_PERSISTENT((k_fa_x<N, false, false>), F::t1, F::s1, units1, s, a);
        }
        break;
      case FA_Y:
        if (a.yzphase)
          MFX_FF_PERSISTENT((k_fa_y<N, true>), F::t2, F::s2 + size_t(N + F::Kh) * 8, size_t(N) * (F::Kh / F::P2) * 6, s, a);
        else
          MFX_FF_PERSISTENT((k_fa_y<N, false>), F::t2, F::s2, size_t(N) * (F::Kh / F::P2) * 6, s, a);
        break;
      case FA_Z:
        MFX_FF_PERSISTENT((k_fa_z<N>), F::t3, F::s3, size_t(N) * N / F::RW, s, a);
        break;
      default:
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
  }
}

// per-M entry points (defined in the ff_m*.cu units)
#define MFX_FF_LENGTHS(X) X(24) X(48) X(96) X(144) X(192) X(288) X(384) X(576) X(768) X(1152) X(1536)
#define MFX_FF_DECL(M)                                                            \
  cudaError_t ff_launch_##M(int op, int p, const FArgs &a, cudaStream_t s);     \
  cudaError_t fa_launch_##M(int op, bool plt, const FAArgs &a, cudaStream_t s); \
  bool fa_keep_##M();                                                           \
  bool fa_all_##M();                                                            \
  bool fa_halves_##M();                                                         \
  bool ff_valid_##M(int op, int p);
MFX_FF_LENGTHS(MFX_FF_DECL)
#undef MFX_FF_DECL

#define MFX_FF_DEFINE(M)                                                                                     \
  cudaError_t ff_launch_##M(int op, int p, const FArgs &a, cudaStream_t s) { return ff_launch_m<M>(op, p, a, s); } \
  cudaError_t fa_launch_##M(int op, bool plt, const FAArgs &a, cudaStream_t s) {                               \
    return fa_launch_m<M>(op, plt, a, s);                                                                      \
  }                                                                                                            \
  bool fa_keep_##M() { return FA<2 * M / 3>::keep; }                                                          \
  bool fa_all_##M() { return FA<2 * M / 3>::keep || FA<2 * M / 3>::halves; }                                  \
  bool fa_halves_##M() { return FA<2 * M / 3>::halves; }                                                      \
  bool ff_valid_##M(int op, int p) { return ff_valid_m<M>(op, p); }

inline bool ff_length_supported(int M) {
#define MFX_FF_CASE(L) \
  if (M == L) return true;
  MFX_FF_LENGTHS(MFX_FF_CASE)
#undef MFX_FF_CASE
  return false;
}

inline int ff_maxj(int M) {
#define MFX_FF_CASE(L) \
  if (M == L) return Fac<L>::maxJ;
  MFX_FF_LENGTHS(MFX_FF_CASE)
#undef MFX_FF_CASE
  return 0;
}

inline bool ff_valid(int M, int op, int p) {
#define MFX_FF_CASE(L) \
  if (M == L) return ff_valid_##L(op, p);
  MFX_FF_LENGTHS(MFX_FF_CASE)
#undef MFX_FF_CASE
  return false;
}

// whether ASM1 in halves (tiles of 8 pencils) is built for this length
inline bool fa_halves(int M) {
#define MFX_FF_CASE(L) \
  if (M == L) return fa_halves_##L();
  MFX_FF_LENGTHS(MFX_FF_CASE)
#undef MFX_FF_CASE
  return false;
}

// whether ASM1 emits several sub-lattices from one assembly of each mode at
// this length, in either form (4-pencil tiles or halves)
inline bool fa_all(int M) {
#define MFX_FF_CASE(L) \
  if (M == L) return fa_all_##L();
  MFX_FF_LENGTHS(MFX_FF_CASE)
#undef MFX_FF_CASE
  return false;
}

// whether ASM1 with 4-pencil tiles emits several sub-lattices at this length
inline bool fa_keep(int M) {
#define MFX_FF_CASE(L) \
  if (M == L) return fa_keep_##L();
  MFX_FF_LENGTHS(MFX_FF_CASE)
#undef MFX_FF_CASE
  return false;
}

inline cudaError_t fa_launch(int M, int op, bool plt, const FAArgs &a, cudaStream_t s) {
#define MFX_FF_CASE(L) \
  if (M == L) return fa_launch_##L(op, plt, a, s);
  MFX_FF_LENGTHS(MFX_FF_CASE)
#undef MFX_FF_CASE
  return cudaErrorInvalidValue;
}

inline cudaError_t ff_launch(int M, int op, int p, const FArgs &a, cudaStream_t s) {
#define MFX_FF_CASE(L) \
  if (M == L) return ff_launch_##L(op, p, a, s);
  MFX_FF_LENGTHS(MFX_FF_CASE)
#undef MFX_FF_CASE
  return cudaErrorInvalidValue;
}

}  // namespace ff
}  // namespace mfx
