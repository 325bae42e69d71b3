// MUSIC1 white noise on the device (the [random] generator = MUSIC1 plugin,
// one level: the seed given at the grid's own level).
//
//   random_music.cc:92-116            Fill_Grid copies the level's cells into the grid
//   random_music_wnoise_generator.cc  cubes of cubesize^3 cells, cube
//     :588-626                        icube = (ic ncubes + jc) ncubes + kc seeded with
//                                     baseseed + icube, cells ii, jj, kk (kk fastest)
//                                     drawn in order by gsl_ran_ugaussian_ratio_method
//                                     on gsl_rng_mt19937
//   ic_generator.cc:294-383           forward transform (1/sqrt(N^3)), fixing,
//                                     inversion, 1/volfac
//   ic_generator.cc:509-516           phi(1) = -w amplitude(k) / k^2, DC zeroed
//
// The generators are GSL's, restated from their published algorithms:
// MT19937 (Matsumoto and Nishimura 1998, with their 2002 seeding: x0 = s,
// x_i = 1812433253 (x_{i-1} ^ (x_{i-1} >> 30)) + i, seed 0 meaning 4357;
// uniform = output / 2^32) and Leva's ratio-of-uniforms normal (ACM TOMS 18
// (1992) 449) with its published bounding constants.
//
// One warp draws one cube.  The 624-word state lives in shared memory and the
// twist runs in four dependency-ordered phases across the lanes.  Each normal
// of the ratio method consumes a pair of consecutive outputs (u, v) and either
// accepts it or moves on to the next pair, so the pairs of one state block are
// tested in parallel (one pair per lane) and the accepted ones are ranked in
// stream order with a ballot: cell c of the cube gets the c-th accepted pair,
// exactly as the sequential generator hands them out.  624 outputs are 312
// whole pairs, so no pair straddles a twist.
//
// The mean subtraction of the reference (cube means, then the global mean)
// shifts every cell by one constant, which only moves the k = 0 mode; the
// k-space kernel sets that mode to zero, the value the reference's zero-mean
// field has up to rounding.
#pragma once
#include <cstdint>

#include "kernels.cuh"

namespace mfx {
namespace music {

constexpr int kMtN = 624, kMtM = 397;
constexpr uint32_t kMtMatrix = 0x9908b0dfu, kUpper = 0x80000000u, kLower = 0x7fffffffu;

__device__ __forceinline__ uint32_t mt_mix(uint32_t a, uint32_t b, uint32_t c) {
  const uint32_t y = (a & kUpper) | (b & kLower);
  return c ^ (y >> 1) ^ ((y & 1u) ? kMtMatrix : 0u);
}

__device__ __forceinline__ uint32_t mt_temper(uint32_t y) {
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

// Regenerates the 624-word block in place.  Element k of the sequential
// twist reads x[k], x[k+1] and x[(k+397) mod 624]; the last of these is an
// old word for k < 227 and a new one (x[k-227]) after that, and x[0] is new
// for k = 623.  Each phase reads all its inputs before any lane writes.
__device__ __forceinline__ void mt_twist(uint32_t *x, int lane) {
  constexpr int P1 = kMtN - kMtM;  // 227
  uint32_t t[8];
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int k = lane + 32 * r;
    if (k < P1) t[r] = mt_mix(x[k], x[k + 1], x[k + kMtM]);
  }
  __syncwarp();
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int k = lane + 32 * r;
    if (k < P1) x[k] = t[r];
  }
  __syncwarp();
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int k = P1 + lane + 32 * r;
    if (k < 2 * P1) t[r] = mt_mix(x[k], x[k + 1], x[k - P1]);
  }
  __syncwarp();
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int k = P1 + lane + 32 * r;
    if (k < 2 * P1) x[k] = t[r];
  }
  __syncwarp();
#pragma unroll
  for (int r = 0; r < 6; ++r) {
    const int k = 2 * P1 + lane + 32 * r;
    if (k < kMtN - 1) t[r] = mt_mix(x[k], x[k + 1], x[k - P1]);
  }
  __syncwarp();
#pragma unroll
  for (int r = 0; r < 6; ++r) {
    const int k = 2 * P1 + lane + 32 * r;
    if (k < kMtN - 1) x[k] = t[r];
  }
  __syncwarp();
  if (lane == 0) x[kMtN - 1] = mt_mix(x[kMtN - 1], x[0], x[kMtM - 1]);
  __syncwarp();
}

// The ratio method's acceptance of one pair of outputs, in the operation
// order of the sequential C code (no contraction): u = 1 - U1,
// v = 1.7156 (U2 - 1/2), x = u - s, y = |v| - t, Q = x^2 + y (a y - b x);
// accepted when Q < r1, or Q <= r2 and v^2 <= -4 u^2 ln u.  A float estimate
// of Q (error below 1e-6 here), from u and v formed in float straight from
// the integers, settles the pairs far from both bounds; the rest take the
// exact double test.
constexpr double kS = 0.449871, kT = -0.386595, kA = 0.19600, kB = 0.25472, kR1 = 0.27597, kR2 = 0.27846;
constexpr double kTwo32 = 1.0 / 4294967296.0;

// u and v in float: 1 - U1 = (2^32 - w1) 2^-32 and U2 - 1/2 = (w2 - 2^31) 2^-32
// keep their relative precision (a float U1 near 1 would not)
__device__ __forceinline__ void leva_uv_f(uint32_t w1, uint32_t w2, float &uf, float &vf) {
  uf = float(0x100000000ull - uint64_t(w1)) * float(kTwo32);
  vf = float(int32_t(w2 - 0x80000000u)) * float(kTwo32) * 1.7156f;
}
__device__ __forceinline__ void leva_uv_d(uint32_t w1, uint32_t w2, double &u, double &v) {
  u = __dsub_rn(1.0, double(w1) * kTwo32);
  v = __dmul_rn(double(w2) * kTwo32 - 0.5, 1.7156);
}
__device__ __forceinline__ bool leva_accept(uint32_t w1, uint32_t w2, float uf, float vf) {
  {
    const float xf = uf - float(kS), yf = fabsf(vf) - float(kT);
    const float qf = xf * xf + yf * (float(kA) * yf - float(kB) * xf);
    if (qf < float(kR1) - 1e-5f) return true;
    if (qf > float(kR2) + 1e-5f) return false;
  }
  double u, v;
  leva_uv_d(w1, w2, u, v);
  const double x = __dsub_rn(u, kS), y = __dsub_rn(fabs(v), kT);
  const double q = __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, __dsub_rn(__dmul_rn(kA, y), __dmul_rn(kB, x))));
  if (q < kR1) return true;
  if (q > kR2) return false;
  return !(__dmul_rn(v, v) > __dmul_rn(__dmul_rn(__dmul_rn(-4.0, u), u), log(u)));
}

// The accepted pair's normal v / u: the exact double quotient for the FP64
// form; for the FP32 form the float quotient of the float u and v (within
// two units in the last place of the double quotient rounded to float)
template <typename R> __device__ __forceinline__ R leva_value(uint32_t w1, uint32_t w2, float uf, float vf);
template <> __device__ __forceinline__ double leva_value<double>(uint32_t w1, uint32_t w2, float, float) {
  double u, v;
  leva_uv_d(w1, w2, u, v);
  return v / u;
}
template <> __device__ __forceinline__ float leva_value<float>(uint32_t, uint32_t, float uf, float vf) {
  return vf / uf;
}

struct CubeArgs {
  const long long *seed;  // baseseed of the level (device memory)
  int N;             // grid cells per axis
  int cs;            // cube edge (N itself when N < cubesize)
  int nc;            // cubes per axis
  long long row;     // real elements between consecutive k-rows (2 (N/2 + 1))
};

// One warp per cube: blockDim.x == 32, gridDim.x == nc^3.  Writes cube cells
// into the padded real layout of an in-place r2c transform.
template <typename R> __global__ void __launch_bounds__(32) k_music_cubes(CubeArgs a, R *out) {
  __shared__ uint32_t x[kMtN];
  const int lane = threadIdx.x;
  const long long icube = blockIdx.x;
  const int nc = a.nc, cs = a.cs;
  const int ic = int(icube / (nc * nc)), jc = int((icube / nc) % nc), kc = int(icube % nc);
  if (lane == 0) {
    // gsl_rng_set(mt19937, baseseed + icube): the seed as an unsigned long,
    // its low 32 bits used
    const unsigned long long cseed = static_cast<unsigned long long>(*a.seed + icube);
    uint32_t s = cseed == 0 ? 4357u : uint32_t(cseed & 0xffffffffull);
    x[0] = s;
    for (int k = 1; k < kMtN; ++k) {
      s = 1812433253u * (s ^ (s >> 30)) + uint32_t(k);
      x[k] = s;
    }
  }
  __syncwarp();
  const int total = cs * cs * cs, cs2 = cs * cs;
  R *base = out + (size_t(ic) * cs * a.N + size_t(jc) * cs) * size_t(a.row) + size_t(kc) * cs;
  int produced = 0;
  const unsigned lt = (1u << lane) - 1u;
  while (produced < total) {
    mt_twist(x, lane);
    for (int p0 = 0; p0 < kMtN / 2 && produced < total; p0 += 32) {
      const int p = p0 + lane;
      bool acc = false;
      uint32_t w1 = 0, w2 = 0;
      float uf = 1.f, vf = 0.f;
      if (p < kMtN / 2) {
        w1 = mt_temper(x[2 * p]);
        w2 = mt_temper(x[2 * p + 1]);
        leva_uv_f(w1, w2, uf, vf);
        acc = leva_accept(w1, w2, uf, vf);
      }
      const unsigned m = __ballot_sync(0xffffffffu, acc);
      const int c = produced + __popc(m & lt);
      if (acc && c < total) {
        const int ii = c / cs2, jj = (c / cs) % cs, kk = c % cs;
        base[(size_t(ii) * a.N + jj) * size_t(a.row) + kk] = leva_value<R>(w1, w2, uf, vf);
      }
      produced += __popc(m);
    }
    __syncwarp();
  }
}

// The dummy seed of a level no seed[level] key names (random_music.cc:176-183):
// -|(-2 - l) % 123 + (-2 + 7342523521 l) % 123456789|, C's remainder.
inline long long dummy_seed(int level) {
  const long long ltemp = -2;
  const long long v = (ltemp - level) % 123 + (ltemp + 7342523521LL * level) % 123456789;
  return -(v < 0 ? -v : v);
}

// Coarse mode replacement (random_music_wnoise_generator.cc:462-505): every
// coarse k-space mode off the coarse Nyquist indices overwrites the fine
// mode of the same wave vector, times exp(-i pi/2 (kx + ky + kz)/nc) sqrt(8)
// (a half coarse cell).  Both fields are unnormalised r2c outputs.
template <typename R>
__global__ void __launch_bounds__(256) k_music_embed(const typename Cplx<R>::T *coarse, typename Cplx<R>::T *fine,
                                                     int nc, int nf) {
  const int hc = nc >> 1, kc = hc + 1, kf = (nf >> 1) + 1;
  const size_t total = size_t(nc) * nc * kc;
  for (size_t idx = size_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < total;
       idx += size_t(gridDim.x) * blockDim.x) {
    const int k = int(idx % kc);
    const size_t t = idx / kc;
    const int j = int(t % nc), i = int(t / nc);
    if (i == hc || j == hc || k == hc) continue;
    const int ii = i > hc ? i + (nf >> 1) : i, jj = j > hc ? j + (nf >> 1) : j;
    const double kx = i <= hc ? i : i - nc, ky = j <= hc ? j : j - nc;
    const double ph = (kx / nc + ky / nc + double(k) / nc) * -0.5 * 3.141592653589793;
    double sn, cs;
    sincos(ph, &sn, &cs);
    const double s8 = 2.8284271247461903;  // sqrt(8)
    const auto v = coarse[idx];
    const double re = double(v.x), im = double(v.y);
    fine[(size_t(ii) * nf + jj) * kf + k] = mkc<R>(R((re * cs - im * sn) * s8), R((re * sn + im * cs) * s8));
  }
}

// Restriction (random_music_wnoise_generator.cc:288-380), `steps` levels at
// once: every mode of the coarse grid (nc) takes the mode of the same wave
// vector of the fine grid (nf = nc 2^steps) times exp(+i pi/2 (kx + ky + kz)
// / n) / sqrt(8) for each level n = nc, 2 nc, ... passed through.  Both are
// unnormalised r2c outputs.
template <typename R>
__global__ void __launch_bounds__(256) k_music_restrict(const typename Cplx<R>::T *fine, typename Cplx<R>::T *coarse,
                                                        int nc, int steps) {
  const int hc = nc >> 1, kc = hc + 1, nf = nc << steps, kf = (nf >> 1) + 1;
  const size_t total = size_t(nc) * nc * kc;
  double geo = 0.0;  // sum over the levels passed of 1 / n
  for (int s = 0; s < steps; ++s) geo += 1.0 / double(nc << s);
  const double scale = pow(8.0, -0.5 * steps);
  for (size_t idx = size_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < total;
       idx += size_t(gridDim.x) * blockDim.x) {
    const int k = int(idx % kc);
    const size_t t = idx / kc;
    const int j = int(t % nc), i = int(t / nc);
    const int kx = i <= hc ? i : i - nc, ky = j <= hc ? j : j - nc;
    const int ii = kx >= 0 ? kx : kx + nf, jj = ky >= 0 ? ky : ky + nf;
    const double ph = double(kx + ky + k) * geo * 0.5 * 3.141592653589793;
    double sn, cs;
    sincos(ph, &sn, &cs);
    const auto v = fine[(size_t(ii) * nf + jj) * kf + k];
    const double re = double(v.x), im = double(v.y);
    coarse[idx] = mkc<R>(R((re * cs - im * sn) * scale), R((re * sn + im * cs) * scale));
  }
}

// The Hermitian part of the kz = 0 and kz = n/2 planes of an r2c spectrum,
// in place: what a c2r followed by an r2c leaves of them (the reference takes
// that round trip between levels).  One thread per pair (i, j) <-> (-i, -j).
template <typename R>
__global__ void __launch_bounds__(256) k_music_hermitian_planes(typename Cplx<R>::T *f, int n) {
  const int kn = (n >> 1) + 1;
  const size_t total = size_t(n) * n * 2;
  for (size_t idx = size_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < total;
       idx += size_t(gridDim.x) * blockDim.x) {
    const int k = (idx & 1) ? (n >> 1) : 0;
    const size_t t = idx >> 1;
    const int j = int(t % n), i = int(t / n);
    const int pi = i ? n - i : 0, pj = j ? n - j : 0;
    if (size_t(pi) * n + pj < t) continue;  // the partner's thread writes both
    auto &a = f[(size_t(i) * n + j) * kn + k];
    auto &b = f[(size_t(pi) * n + pj) * kn + k];
    const R re = R(0.5) * (a.x + b.x), im = R(0.5) * (a.y - b.y);
    a = mkc<R>(re, im);
    b = mkc<R>(re, -im);
  }
}

// A real-space field (double, [x][y][z]) into the padded real layout of an
// in-place r2c, rounded to R
template <typename R>
__global__ void __launch_bounds__(256) k_field_to_padded(const double *src, R *dst, int n) {
  const size_t total = size_t(n) * n * n;
  const size_t row = 2 * size_t(n / 2 + 1);
  for (size_t idx = size_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < total;
       idx += size_t(gridDim.x) * blockDim.x) {
    const size_t k = idx % n, col = idx / n;
    dst[col * row + k] = R(src[idx]);
  }
}

struct KArgs {
  const double *amp;  // amp[n] = amplitude(kf sqrt n)/(kf^2 n)
  size_t amp_len;
  int N;
  int mode;           // 0: raw noise, 1: normalised noise, 2: phi(1)
  int fixing;
  int keep_dc;        // 1: the k = 0 mode stays (a given field's mean); 0: zero
  double unit;        // 1/sqrt(N^3): the forward transform's norm
  double norm;        // (+-1)/volfac
  double out_scale;   // extra factor on phi(1) (per-field scaling of the FP32 form)
};

// k-space pass over the r2c output of the cube noise, in place: the unitary
// norm, the k = 0 mode set to zero, then (modes 1, 2) fixing, inversion and
// 1/volfac, and (mode 2) -amplitude(k)/k^2.  Unlike NGenIC's noise the
// Nyquist planes carry modes.
template <typename R> __global__ void __launch_bounds__(256) k_music_phi1(KArgs a, typename Cplx<R>::T *f) {
  const int N = a.N, nk = (N >> 1) + 1;
  const size_t total = size_t(N) * N * nk;
  for (size_t idx = size_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < total;
       idx += size_t(gridDim.x) * blockDim.x) {
    const int k = int(idx % nk);
    const size_t col = idx / nk;
    const int j = int(col % N), i = int(col / N);
    if ((i | j | k) == 0 && (a.mode == 2 || !a.keep_dc)) {
      f[idx] = mkc<R>(R(0), R(0));
      continue;
    }
    auto z = f[idx];
    R re = R(double(z.x) * a.unit), im = R(double(z.y) * a.unit);
    if (a.mode >= 1) {
      if (a.fixing) {
        const R m = sqrt(re * re + im * im);
        if (m != R(0)) {
          re /= m;
          im /= m;
        }
      }
      re *= R(a.norm);
      im *= R(a.norm);
      if (a.mode == 2) {
        const int si = signed_idx(i, N), sj = signed_idx(j, N);
        const size_t n = size_t(si * si + sj * sj + k * k);
        const R fa = (n < a.amp_len) ? R(-a.amp[n] * a.out_scale) : R(0);
        re *= fa;
        im *= fa;
      }
    }
    f[idx] = mkc<R>(re, im);
  }
}

}  // namespace music
}  // namespace mfx
