// Device kernels of the LPT hot path.  Every kernel is templated on the real
// type R (double: the reference's plain FP64 algorithm; float: the FP32 form).
//
// Memory layout (identical to the reference's non-distributed Grid_FFT,
// grid_fft.cc:40-112): a real field of size n^3 is stored with rows padded to
// n+2 reals; the same buffer holds the k-space field as n x n x (n/2+1)
// complex values, kelem(i,j,k) = c[(i*n + j)*(n/2+1) + k].  N-grid fields are
// the LPT potentials, M-grid (M = 3N/2) fields the Orszag-padded products.
// FFTs are unnormalised cuFFT transforms; the unitary 1/sqrt(n^3) of the
// reference (grid_fft.cc:69, 199-270) is folded into the kernel before or
// after each transform.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "ranlxd.cuh"

namespace mfx {

template <typename R> struct Cplx;
template <> struct Cplx<double> { using T = double2; };
template <> struct Cplx<float> { using T = float2; };

template <typename R> __device__ __forceinline__ typename Cplx<R>::T mkc(R re, R im) {
  typename Cplx<R>::T c;
  c.x = re;
  c.y = im;
  return c;
}

// signed mode index: get_k's i > n/2 -> i - n (grid_fft.hh:281-296)
__device__ __forceinline__ int signed_idx(int i, int n) { return i > (n >> 1) ? i - n : i; }

// ---------------------------------------------------------------------------
// compensated FP32 arithmetic (Ogita, Rump & Oishi, "Accurate sum and dot
// product", SIAM J. Sci. Comput. 26 (2005)): TwoSum and FMA-based TwoProduct.
// For double the accumulator degenerates to a plain sum (the reference's FP64
// arithmetic).
// ---------------------------------------------------------------------------
template <typename R> struct Acc {
  R hi, lo;
  __device__ __forceinline__ Acc(R h = R(0), R l = R(0)) : hi(h), lo(l) {}
  __device__ __forceinline__ void add(R v);
  __device__ __forceinline__ void add_prod(R a, R b);       // += a*b
  __device__ __forceinline__ void add_prod(R c, R a, R b);  // += c*a*b
  __device__ __forceinline__ R value() const { return hi + lo; }
};

template <> __device__ __forceinline__ void Acc<double>::add(double v) { hi += v; }
template <> __device__ __forceinline__ void Acc<double>::add_prod(double a, double b) { hi += a * b; }
template <> __device__ __forceinline__ void Acc<double>::add_prod(double c, double a, double b) {
  hi += c * (a * b);
}

template <> __device__ __forceinline__ void Acc<float>::add(float v) {
  const float s = hi + v;
  const float bp = s - hi;
  const float err = (hi - (s - bp)) + (v - bp);
  hi = s;
  lo += err;
}
template <> __device__ __forceinline__ void Acc<float>::add_prod(float a, float b) {
  const float p = a * b;
  const float e = fmaf(a, b, -p);
  add(p);
  lo += e;
}
template <> __device__ __forceinline__ void Acc<float>::add_prod(float c, float a, float b) {
  const float p = a * b;
  const float e = fmaf(a, b, -p);
  const float q = c * p;
  const float e2 = fmaf(c, p, -q) + c * e;
  add(q);
  lo += e2;
}

// ---------------------------------------------------------------------------
// RANLUX words (device bit-exactness hook)
// ---------------------------------------------------------------------------
static __global__ void k_ranlux_words(uint32_t seed, size_t count, uint64_t *out) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  Ranlxd1 r;
  r.seed31(seed);
  for (size_t q = 0; q < count; ++q) out[q] = r.next();
}

// ---------------------------------------------------------------------------
// (1) NGenIC white noise -> normalisation -> phi(1)
//     random_ngenic.cc:84-154, ic_generator.cc:378-383, 509-516
// One thread per (i,j) column; the column's RANLUX stream is drawn in the
// reference's order (phase, amplitude with rejection of 0) for every k,
// Nyquist and DC included.
// ---------------------------------------------------------------------------
struct NoiseArgs {
  const uint32_t *seeds;
  const double *amp;  // amp[n] = amplitude(kf sqrt n)/(kf^2 n)
  size_t amp_len;
  int N;
  int mode;           // 0: raw noise, 1: normalised noise, 2: phi(1)
  int fixing;
  double norm;        // (+-1)/volfac
  double out_scale;   // extra factor on phi(1) (per-field scaling of the FP32 form)
};

// Box-Muller of two 48-bit uniforms u_a = a 2^-48, u_b = b 2^-48
// (random_ngenic.cc:117-121): z = sqrt(-ln u_b) exp(2 pi i u_a).
template <typename R> struct NoiseMath;
template <> struct NoiseMath<double> {
  static __device__ __forceinline__ void z(uint64_t a, uint64_t b, double &re, double &im) {
    const double phase = (double(a) * kTwoM48) * 2 * 3.141592653589793;
    const double am = sqrt(-log(double(b) * kTwoM48));
    double s, c;
    sincos(phase, &s, &c);
    re = am * c;
    im = am * s;
  }
};
// The FP32 form keeps the variates' 48 bits where float would drop them:
// ln u_b as log1p(-(1 - u_b)) with 1 - u_b taken exactly from the integer when
// u_b >= 1/2 (a plain float u_b within 2^-25 of 1 rounds to 1 and would zero
// the mode), and the phase pi x, x = 2 u_a, split as x_hi + x_lo with the
// small part applied to the sine and cosine to first order (|pi x_lo| < 4e-7).
template <> struct NoiseMath<float> {
  static __device__ __forceinline__ void z(uint64_t a, uint64_t b, float &re, float &im) {
    const float lnu = (b < (uint64_t(1) << 47)) ? logf(float(b) * 3.5527136788005009e-15f)  // 2^-48
                                                : log1pf(-float((uint64_t(1) << 48) - b) * 3.5527136788005009e-15f);
    const float am = sqrtf(-lnu);
    const uint64_t ahi = a & ~((uint64_t(1) << 24) - 1);
    const float xh = float(ahi) * 7.1054273576010019e-15f;     // 2^-47: x = a 2^-47 in [0, 2)
    const float xl = float(a - ahi) * 7.1054273576010019e-15f;  // < 2^-23
    float s, c;
    sincospif(xh, &s, &c);
    const float pxl = 3.14159265358979f * xl;
    const float s1 = fmaf(pxl, c, s), c1 = fmaf(-pxl, s, c);
    re = am * c1;
    im = am * s1;
  }
};

template <typename R>
__global__ void __launch_bounds__(128) k_noise_phi1(NoiseArgs a, typename Cplx<R>::T *out) {
  using C = typename Cplx<R>::T;
  const int N = a.N, nh = N >> 1, nk = nh + 1;
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= N * N) return;
  const int i = col / N, j = col - (col / N) * N;
  const int ii = i > 0 ? N - i : 0, jj = j > 0 ? N - j : 0;
  const int si = signed_idx(i, N), sj = signed_idx(j, N);
  Ranlxd1 rng;
  rng.seed31(a.seeds[col]);
  C *colp = out + size_t(col) * nk;
  for (int k = 0; k < nk; ++k) {
    const uint64_t ua = rng.next();
    uint64_t ub;
    int tries = 0;
    do {
      ub = rng.next();
    } while (ub == 0 && ++tries < 1024);  // the reference rejects 0 and 1; 1 is not representable
    const bool skip = (i == nh) | (j == nh) | (k == nh) | ((i | j | k) == 0);
    if (skip) {
      colp[k] = mkc<R>(R(0), R(0));
      continue;
    }
    // k = 0 plane: only the half that the reference assigns directly writes;
    // the other half receives the conjugate from its partner column.
    if (k == 0 && (i > nh || (i == 0 && j > nh))) continue;
    R re, im;
    NoiseMath<R>::z(ua, ub, re, im);
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
        const size_t n = size_t(si * si + sj * sj + k * k);
        const R f = (n < a.amp_len) ? R(-a.amp[n] * a.out_scale) : R(0);
        re *= f;
        im *= f;
      }
    }
    colp[k] = mkc<R>(re, im);
    if (k == 0) out[(size_t(ii) * N + jj) * nk] = mkc<R>(re, -im);
  }
}

// ---------------------------------------------------------------------------
// (2) Orszag pad-insert of Hessians: M-grid k-space <- (-g_a g_b) phi * fac
//     convolution.hh:552-575 with the Hessian functor of convolution.hh:136-157
// ---------------------------------------------------------------------------
struct PadArgs {
  const void *phi;  // N-grid k-space
  void *out[6];     // M-grid k-space buffers
  int8_t ca[6], cb[6];
  int ncomp;
  int N, M;
  double kfac, fac;
};

template <typename R> __global__ void __launch_bounds__(256) k_pad_hessian(PadArgs a) {
  using C = typename Cplx<R>::T;
  const int N = a.N, nh = N >> 1, nk = nh + 1, M = a.M, mk = (M >> 1) + 1;
  const size_t total = size_t(M) * M * mk;
  const C *phi = reinterpret_cast<const C *>(a.phi);
  for (size_t idx = size_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < total;
       idx += size_t(gridDim.x) * blockDim.x) {
    const int kp = int(idx % mk);
    const size_t t = idx / mk;
    const int jp = int(t % M), ip = int(t / M);
    const bool in = (kp <= nh) && (ip <= nh || ip > N) && (jp <= nh || jp > N);
    C v = mkc<R>(R(0), R(0));
    R g[3] = {R(0), R(0), R(0)};
    if (in) {
      const int i = ip <= nh ? ip : ip - nh;
      const int j = jp <= nh ? jp : jp - nh;
      v = phi[(size_t(i) * N + j) * nk + kp];
      const R kf = R(a.kfac);
      g[0] = (i != nh) ? R(signed_idx(i, N)) * kf : R(0);
      g[1] = (j != nh) ? R(signed_idx(j, N)) * kf : R(0);
      g[2] = (kp != nh) ? R(kp) * kf : R(0);
      v.x *= R(a.fac);
      v.y *= R(a.fac);
    }
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      if (c < a.ncomp) {
        const R h = -(g[a.ca[c]] * g[a.cb[c]]);
        reinterpret_cast<C *>(a.out[c])[idx] = mkc<R>(v.x * h, v.y * h);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// (3) real-space products on the padded M-grid (convolution.hh:510-514)
// Elementwise over all M*M*(M+2) reals (the row padding is harmless).
// Hessian slot order: 0:xx 1:yy 2:zz 3:xy 4:xz 5:yz
// ---------------------------------------------------------------------------
struct SrcArgs {
  const void *h1[6];  // Hessians of phi(1)
  const void *h2[6];  // Hessians of phi(2)
  const void *t[5];   // pairwise-truncated products of the phi(3a) triples
  void *out[5];
  size_t count;       // number of reals
};

// phi(2) source, ic_generator.cc:530-534:
//   xx (yy + zz) + yy zz - xy^2 - xz^2 - yz^2
template <typename R> __global__ void __launch_bounds__(256) k_src2(SrcArgs a) {
  const R *H[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) H[c] = reinterpret_cast<const R *>(a.h1[c]);
  R *out = reinterpret_cast<R *>(a.out[0]);
  for (size_t q = size_t(blockIdx.x) * blockDim.x + threadIdx.x; q < a.count;
       q += size_t(gridDim.x) * blockDim.x) {
    const R xx = H[0][q], yy = H[1][q], zz = H[2][q], xy = H[3][q], xz = H[4][q], yz = H[5][q];
    Acc<R> s;
    s.add_prod(xx, yy + zz);
    s.add_prod(yy, zz);
    s.add_prod(R(-1), xy, xy);
    s.add_prod(R(-1), xz, xz);
    s.add_prod(R(-1), yz, yz);
    out[q] = s.value();
  }
}

// First pairs of the five phi(3a) triple products (ic_generator.cc:581-585,
// convolve3 = convolve2(convolve2(a, b), c), convolution.hh:525-532):
//   xx*yy, xy*xz, yz*yz, xz*xz, xy*xy   -> out[0..4]
template <typename R> __global__ void __launch_bounds__(256) k_pairs3a(SrcArgs a) {
  const R *H[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) H[c] = reinterpret_cast<const R *>(a.h1[c]);
  for (size_t q = size_t(blockIdx.x) * blockDim.x + threadIdx.x; q < a.count;
       q += size_t(gridDim.x) * blockDim.x) {
    const R xx = H[0][q], yy = H[1][q], xy = H[3][q], xz = H[4][q], yz = H[5][q];
    reinterpret_cast<R *>(a.out[0])[q] = xx * yy;
    reinterpret_cast<R *>(a.out[1])[q] = xy * xz;
    reinterpret_cast<R *>(a.out[2])[q] = yz * yz;
    reinterpret_cast<R *>(a.out[3])[q] = xz * xz;
    reinterpret_cast<R *>(a.out[4])[q] = xy * xy;
  }
}

// Full phi(3) source and the three transverse A(3) sources in one pass over
// the 12 Hessians and the 5 truncated pair products:
//   phi3a (ic_generator.cc:581-585): T0 zz + 2 T1 yz - T2 xx - T3 yy - T4 zz
//   phi3b (ic_generator.cc:592-609): -5/7 sum_i phi_ii (phi2_jj + phi2_kk)
//                                    +10/7 sum_{i<j} phi_ij phi2_ij
//   A3_d  (ic_generator.cc:613-628)
// out[0] = phi3 source, out[1..3] = A3 sources.  Outputs may alias t[] slots
// (each element is read before it is written by the same thread).
template <typename R> __global__ void __launch_bounds__(256) k_src3(SrcArgs a) {
  const R c57 = R(-5.0 / 7.0), c107 = R(10.0 / 7.0);
  for (size_t q = size_t(blockIdx.x) * blockDim.x + threadIdx.x; q < a.count;
       q += size_t(gridDim.x) * blockDim.x) {
    R p[6], s[6], T[5];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      p[c] = reinterpret_cast<const R *>(a.h1[c])[q];
      s[c] = reinterpret_cast<const R *>(a.h2[c])[q];
    }
#pragma unroll
    for (int c = 0; c < 5; ++c) T[c] = reinterpret_cast<const R *>(a.t[c])[q];
    Acc<R> S;
    S.add_prod(T[0], p[2]);
    S.add_prod(R(2), T[1], p[5]);
    S.add_prod(R(-1), T[2], p[0]);
    S.add_prod(R(-1), T[3], p[1]);
    S.add_prod(R(-1), T[4], p[2]);
    S.add_prod(c57, p[0], s[1] + s[2]);
    S.add_prod(c57, p[1], s[2] + s[0]);
    S.add_prod(c57, p[2], s[0] + s[1]);
    S.add_prod(c107, p[3], s[3]);
    S.add_prod(c107, p[4], s[4]);
    S.add_prod(c107, p[5], s[5]);
    reinterpret_cast<R *>(a.out[0])[q] = S.value();
    // A_d with (d, d', d'') cyclic; slot(a,b) of the symmetric Hessian
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int d1 = (d + 1) % 3, d2 = (d + 2) % 3;
      auto slot = [](int x, int y) {
        if (x == y) return x;
        const int lo_ = x < y ? x : y, hi_ = x < y ? y : x;
        return lo_ == 0 ? (hi_ == 1 ? 3 : 4) : 5;
      };
      Acc<R> A;
      A.add_prod(s[slot(d, d1)], p[slot(d, d2)]);
      A.add_prod(R(-1), s[slot(d, d2)], p[slot(d, d1)]);
      A.add_prod(p[slot(d1, d2)], s[slot(d1, d1)] - s[slot(d2, d2)]);
      A.add_prod(R(-1), s[slot(d1, d2)], p[slot(d1, d1)] - p[slot(d2, d2)]);
      reinterpret_cast<R *>(a.out[1 + d])[q] = A.value();
    }
  }
}

// ---------------------------------------------------------------------------
// (4) unpad (convolution.hh:600-636) + inverse Laplacian (grid_fft.hh:440-449)
//     N-grid out(i,j,k) = -fac * F(ip,jp,k) / |k|^2, zero on any Nyquist index
//     and at DC.
// ---------------------------------------------------------------------------
struct UnpadArgs {
  const void *F;  // M-grid k-space
  void *out;      // N-grid k-space
  int N, M;
  double kfac, fac;
};

template <typename R> __global__ void __launch_bounds__(256) k_unpad_invlap(UnpadArgs a) {
  using C = typename Cplx<R>::T;
  const int N = a.N, nh = N >> 1, nk = nh + 1, M = a.M, mk = (M >> 1) + 1;
  const size_t total = size_t(N) * N * nk;
  const C *F = reinterpret_cast<const C *>(a.F);
  C *out = reinterpret_cast<C *>(a.out);
  for (size_t idx = size_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < total;
       idx += size_t(gridDim.x) * blockDim.x) {
    const int k = int(idx % nk);
    const size_t t = idx / nk;
    const int j = int(t % N), i = int(t / N);
    C r = mkc<R>(R(0), R(0));
    if (i != nh && j != nh && k != nh && (i | j | k) != 0) {
      const int ip = i > nh ? i + nh : i, jp = j > nh ? j + nh : j;
      const C v = F[(size_t(ip) * M + jp) * mk + k];
      const R kf = R(a.kfac);
      const R kx = R(signed_idx(i, N)) * kf, ky = R(signed_idx(j, N)) * kf, kz = R(k) * kf;
      const R f = -R(a.fac) / (kx * kx + ky * ky + kz * kz);
      r = mkc<R>(v.x * f, v.y * f);
    }
    out[idx] = r;
  }
}

// In-place on an M-grid k-space field: keep the N-grid modes (minus Nyquist)
// scaled by fac, zero the rest.  Realises unpad -> pad of convolve3's second
// convolve2 (convolution.hh:525-532).
struct TruncArgs {
  void *F;
  int N, M;
  double fac;
};

template <typename R> __global__ void __launch_bounds__(256) k_trunc_repad(TruncArgs a) {
  using C = typename Cplx<R>::T;
  const int N = a.N, nh = N >> 1, M = a.M, mk = (M >> 1) + 1;
  const size_t total = size_t(M) * M * mk;
  C *F = reinterpret_cast<C *>(a.F);
  for (size_t idx = size_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < total;
       idx += size_t(gridDim.x) * blockDim.x) {
    const int kp = int(idx % mk);
    const size_t t = idx / mk;
    const int jp = int(t % M), ip = int(t / M);
    const bool keep = (kp < nh) && (ip < nh || ip > N) && (jp < nh || jp > N);
    C v = mkc<R>(R(0), R(0));
    if (keep) {
      v = F[idx];
      v.x *= R(a.fac);
      v.y *= R(a.fac);
    }
    F[idx] = v;
  }
}

// ---------------------------------------------------------------------------
// (5) displacement / velocity assembly in k-space (ic_generator.cc:929-1053)
//     with the per-sub-lattice phase shift of Grid_FFT::shift_field
//     (grid_fft.hh:832-842, particle_generator.hh:510-522) folded in.
// ---------------------------------------------------------------------------
// Sub-lattice shifts as the reference applies them: one shift_field per
// step (grid_fft.hh:832-842, particle_generator.hh:510-522), each an r2c,
// a phase exp(i s.k dx) and a c2r.  The c2r keeps only the Hermitian part of
// the kz = 0 and kz = N/2 planes, where a Nyquist index stands for both +k
// and -k: there a step multiplies the Nyquist axes' phase by its real part,
// cos(sum of their step angles), so the product over the steps, not the
// phase of the total shift, is what reaches those modes.  Folding the phase
// into the assembly keeps that product (nyq_phase).  Active only for noise
// that fills the Nyquist planes (MUSIC1); NGenIC's potentials vanish there.
struct NyqSteps {
  int active;
  int nsteps[4];         // per sub-lattice
  double ang[4][4][3];   // [sub-lattice][step][axis]: step shift * Nyquist k * dx
};

// The phase a sub-lattice's modes on the projected planes receive; false
// where the plain phase of the total shift applies.  ph: [ns][3][N]
// exp(i s_a k_a dx) of the total shifts.
template <typename R>
__device__ __forceinline__ bool nyq_phase(const NyqSteps &t, const double2 *ph, int s, int i, int j, int k, int N,
                                          R &er, R &ei) {
  const int nh = N >> 1;
  if (!t.active || (k != 0 && k != nh)) return false;
  const bool nx = i == nh, ny = j == nh, nz = k == nh;
  if (!(nx || ny || nz)) return false;
  double c = 1.0;
  for (int st = 0; st < t.nsteps[s]; ++st)
    c *= cos((nx ? t.ang[s][st][0] : 0.0) + (ny ? t.ang[s][st][1] : 0.0) + (nz ? t.ang[s][st][2] : 0.0));
  const double2 *p = ph + size_t(s) * 3 * N;
  double re = c, im = 0.0;
  auto mul = [&](double2 e) {
    const double r = re * e.x - im * e.y;
    im = re * e.y + im * e.x;
    re = r;
  };
  if (!nx) mul(p[i]);
  if (!ny) mul(p[N + j]);
  if (!nz) mul(p[2 * N + k]);
  er = R(re);
  ei = R(im);
  return true;
}

struct AsmArgs {
  const void *phi[3];   // phi1, phi2, phi3 (N-grid k-space, unscaled)
  const void *A3[3];
  const double *plt;    // 4 tables of 64*64*33 (D_r, D_theta, D_phi, alpha^-1) or null
  const float4 *plt4;   // the same tables interleaved per mode in float (FP32 form)
  const double2 *phase; // [ns][3][N] exp(i s_a k_a dx)
  const float2 *phase32; // the same rounded to float (FP32 form)
  void *out[24];        // [shift][pos x,y,z, vel x,y,z]
  int N, order, nshift, shift0;
  double kfac, mapratio, boxlen;
  double g1, g2, g3, g3c, vfac1, vfac2, vfac3;
  double pfac, vfac;    // lunit/L * 1/sqrt(N^3),  vunit/L * 1/sqrt(N^3)
  double in_scale1, in_scale2, in_scale3;  // undo per-field scaling
  // the FP32 form's coefficients, rounded from the FP64 ones once on the host
  // (a float kernel that re-derived them per mode would keep the slow FP64
  // pipe busy): kfac, g_n * in_scale_n (n = 1, 2, 3), g3c * in_scale3,
  // vfac1..3, pfac, vfac
  float fkfac, fs1, fs2, fs3, fsa, fv1, fv2, fv3, fpfac, fvfac;
  // baryon + CDM runs: the linear relative-velocity term of a species
  // (ic_generator.cc:1016-1020) as a factor 1 + qvbc[n] on phi1's velocity
  // weight, n = |k|^2 / kf^2 (null: no term)
  const double *qvbc;
  const float *qvbc32;
  size_t qvbc_len;
  NyqSteps nyq;
};

// the float coefficients of an AsmArgs from its FP64 ones
inline void asm_float_coefficients(AsmArgs &a) {
  a.fkfac = float(a.kfac);
  a.fs1 = float(a.g1 * a.in_scale1);
  a.fs2 = float(a.g2 * a.in_scale2);
  a.fs3 = float(a.g3 * a.in_scale3);
  a.fsa = float(a.g3c * a.in_scale3);
  a.fv1 = float(a.vfac1);
  a.fv2 = float(a.vfac2);
  a.fv3 = float(a.vfac3);
  a.fpfac = float(a.pfac);
  a.fvfac = float(a.vfac);
}

// get_cic_kspace (grid_fft.hh:347-373) on a 64 x 64 x 33 real table
__device__ __forceinline__ double plt_cic(const double *T, double x, double y, double z) {
  const int ix = int(floor(x)), iy = int(floor(y)), iz = int(floor(z));
  const double dx = x - double(ix), tx = 1.0 - dx;
  const double dy = y - double(iy), ty = 1.0 - dy;
  const double dz = z - double(iz), tz = 1.0 - dz;
  const int ix1 = (ix + 1) % 64, iy1 = (iy + 1) % 64, iz1 = min(iz + 1, 32);
  auto e = [T](int a, int b, int c) { return T[(size_t(a) * 64 + b) * 33 + c]; };
  double v = 0.0;
  v += e(ix, iy, iz) * tx * ty * tz;
  v += e(ix, iy, iz1) * tx * ty * dz;
  v += e(ix, iy1, iz) * tx * dy * tz;
  v += e(ix, iy1, iz1) * tx * dy * dz;
  v += e(ix1, iy, iz) * dx * ty * tz;
  v += e(ix1, iy, iz1) * dx * ty * dz;
  v += e(ix1, iy1, iz) * dx * dy * tz;
  v += e(ix1, iy1, iz1) * dx * dy * dz;
  return v;
}

// FP32 form of the PLT gradient: the interpolation point x = i * 64/N is
// split exactly in integers (ix = floor(64 i / N), dx = (64 i mod N)/N), the
// direction of the interpolation point's k equals that of the mode's signed
// index vector, and the four tables are read as one float4 per CIC corner.
// the FP32 form's PLT tables interleaved per mode, (D_r, D_theta, D_phi,
// alpha^-1) rounded to float, from the four FP64 tables of nm entries each
static __global__ void k_plt_to_f4(const double *T, float4 *out, size_t nm) {
  for (size_t q = size_t(blockIdx.x) * blockDim.x + threadIdx.x; q < nm; q += size_t(gridDim.x) * blockDim.x)
    out[q] = make_float4(float(T[q]), float(T[nm + q]), float(T[2 * nm + q]), float(T[3 * nm + q]));
}

// the FP32 form's PLT tables read from global memory (through the read-only path)
struct PltGlobal {
  const float4 *T;
  __device__ __forceinline__ float4 operator()(int p, int q, int r) const { return __ldg(&T[(p * 64 + q) * 33 + r]); }
};

// e(p, q, r): entry (p, q, r) of the 64 x 64 x 33 float4 table
template <class TA>
__device__ __forceinline__ void plt_grad_f32(const TA &e, int i, int j, int k, int N, float kfac, float G[3],
                                             float &vcorr) {
  const int ix = (64 * i) / N, iy = (64 * j) / N, iz = (64 * k) / N;
  const float invN = 1.0f / float(N);
  const float dx = float((64 * i) % N) * invN, dy = float((64 * j) % N) * invN, dz = float((64 * k) % N) * invN;
  const float tx = 1.0f - dx, ty = 1.0f - dy, tz = 1.0f - dz;
  const int ix1 = (ix + 1) & 63, iy1 = (iy + 1) & 63, iz1 = min(iz + 1, 32);
  const float w[8] = {tx * ty * tz, tx * ty * dz, tx * dy * tz, tx * dy * dz,
                      dx * ty * tz, dx * ty * dz, dx * dy * tz, dx * dy * dz};
  const float4 c[8] = {e(ix, iy, iz), e(ix, iy, iz1), e(ix, iy1, iz), e(ix, iy1, iz1),
                       e(ix1, iy, iz), e(ix1, iy, iz1), e(ix1, iy1, iz), e(ix1, iy1, iz1)};
  float Dr = 0.f, Dt = 0.f, Dp = 0.f, al = 0.f;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    Dr = fmaf(c[q].x, w[q], Dr);
    Dt = fmaf(c[q].y, w[q], Dt);
    Dp = fmaf(c[q].z, w[q], Dp);
    al = fmaf(c[q].w, w[q], al);
  }
  // angles of k from reciprocal square roots (no IEEE divisions)
  const float sx = float(signed_idx(i, N)), sy = float(signed_idx(j, N)), sz = float(signed_idx(k, N));
  const float kperp2 = sx * sx + sy * sy, kr2 = kperp2 + sz * sz;
  float st = 0.f, ct = 1.f, sp = 0.f, cp = 1.f, kr = 0.f;
  if (kr2 > 0.f) {
    const float rkr = rsqrtf(kr2);
    kr = kr2 * rkr;
    ct = sz * rkr;
    if (kperp2 > 0.f) {
      const float rkp = rsqrtf(kperp2);
      st = kperp2 * rkp * rkr;
      cp = sx * rkp;
      sp = sy * rkp;
    }
  }
  const float kmod = kfac * kr;
  G[0] = kmod * (Dr * st * cp + Dt * ct * cp - Dp * sp);
  G[1] = kmod * (Dr * st * sp + Dt * ct * sp + Dp * cp);
  G[2] = kmod * (Dr * ct - Dt * st);
  vcorr = al;
}

// particle::lattice_gradient::gradient / vfac_corr (particle_plt.hh:551-585):
// the plain form evaluates the reference's FP64 expressions (interpolation
// point i * 64/N in double, get_cic_kspace on the double tables); the FP32
// form uses plt_grad_f32.
template <typename R>
__device__ __forceinline__ void plt_grad(const AsmArgs &a, int i, int j, int k, int N, R G[3], R &vcorr) {
  if constexpr (sizeof(R) == 4) {
    plt_grad_f32(PltGlobal{a.plt4}, i, j, k, N, a.fkfac, G, vcorr);
  } else {
    const double x = double(i) * a.mapratio, y = double(j) * a.mapratio, z = double(k) * a.mapratio;
    const double twopi = 2.0 * 3.141592653589793;
    const double kx = (x - double(x > 32.0) * 64.0) * twopi;
    const double ky = (y - double(y > 32.0) * 64.0) * twopi;
    const double kz = (z - double(z > 32.0) * 64.0) * twopi;
    const double kr = sqrt(kx * kx + ky * ky + kz * kz);
    const double kmod = kr / a.mapratio / a.boxlen;
    const size_t TS = size_t(64) * 64 * 33;
    const double Dr = plt_cic(a.plt, x, y, z);
    const double Dt = plt_cic(a.plt + TS, x, y, z);
    const double Dp = plt_cic(a.plt + 2 * TS, x, y, z);
    const double al = plt_cic(a.plt + 3 * TS, x, y, z);
    double st = 0.0, ct = 1.0, sp = 0.0, cp = 1.0;
    if (kr > 0.0) {
      const double kperp = sqrt(kx * kx + ky * ky);
      st = kperp / kr;
      ct = kz / kr;
      if (kperp > 0.0) {
        cp = kx / kperp;
        sp = ky / kperp;
      }
    }
    G[0] = R(kmod * (Dr * st * cp + Dt * ct * cp - Dp * sp));
    G[1] = R(kmod * (Dr * st * sp + Dt * ct * sp + Dp * cp));
    G[2] = R(kmod * (Dr * ct - Dt * st));
    vcorr = R(1.0 / (1.0 / al));
  }
}

// One k-space mode of the displacement (P) and velocity (V) components before
// the sub-lattice phase (ic_generator.cc:929-1053): idx = (i N + j)(N/2+1) + k.
// TAB: the FP32 form's PLT table accessor for the mode's own gradient (the
// kz = 0 mirror still reads the tables in global memory); void: global memory.
template <typename R, bool PLT, class TAB = void>
__device__ __forceinline__ void asm_mode(const AsmArgs &a, int i, int j, int k, size_t idx,
                                         typename Cplx<R>::T P[3], typename Cplx<R>::T V[3],
                                         const TAB *tab = nullptr) {
  using C = typename Cplx<R>::T;
  const int N = a.N, nh = N >> 1;
  // Gp: gradient applied to the displacement, Gv: gradient times vfac_corr
  // applied to the velocity
  R Gp[3], Gv[3];
  // the coefficients in R (the FP32 form's were rounded on the host)
  constexpr bool F32 = sizeof(R) == 4;
  const R c_kf = F32 ? R(a.fkfac) : R(a.kfac);
  const R c_s1 = F32 ? R(a.fs1) : R(a.g1 * a.in_scale1), c_s2 = F32 ? R(a.fs2) : R(a.g2 * a.in_scale2);
  const R c_s3 = F32 ? R(a.fs3) : R(a.g3 * a.in_scale3), c_sa = F32 ? R(a.fsa) : R(a.g3c * a.in_scale3);
  const R c_v1 = F32 ? R(a.fv1) : R(a.vfac1), c_v2 = F32 ? R(a.fv2) : R(a.vfac2), c_v3 = F32 ? R(a.fv3) : R(a.vfac3);
  const R c_pf = F32 ? R(a.fpfac) : R(a.pfac), c_vf = F32 ? R(a.fvfac) : R(a.vfac);
  if (!PLT) {
    // op::fourier_gradient (operators.hh:46-56): Nyquist index zeroed, exactly odd in k
    const R kf = c_kf;
    Gp[0] = (i != nh) ? R(signed_idx(i, N)) * kf : R(0);
    Gp[1] = (j != nh) ? R(signed_idx(j, N)) * kf : R(0);
    Gp[2] = (k != nh) ? R(k) * kf : R(0);
#pragma unroll
    for (int d = 0; d < 3; ++d) Gv[d] = Gp[d];
  } else {
    R G[3], vc;
    if constexpr (!std::is_void<TAB>::value && sizeof(R) == 4)
      plt_grad_f32(*tab, i, j, k, N, a.fkfac, G, vc);
    else
      plt_grad<R>(a, i, j, k, N, G, vc);
    if (k == 0 || k == nh) {
      // On the kz = 0 and kz = N/2 planes the c2r sees both k and -k.  The
      // interpolated PLT gradient is not exactly odd where the CIC stencil
      // touches the table's Nyquist node (stored once, with +k), so the plane
      // would not be Hermitian and the real field would depend on the FFT
      // library's pass order.  Taking the odd part makes the input Hermitian;
      // it equals what a c2c-then-c2r transform of the unsymmetrised plane
      // yields.  (The kz = N/2 plane carries modes only with noise that fills
      // the Nyquist planes, MUSIC1's.)
      const int im = i ? N - i : 0, jm = j ? N - j : 0;
      R Gm[3], vcm;
      plt_grad<R>(a, im, jm, k, N, Gm, vcm);
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        Gp[d] = R(0.5) * (G[d] - Gm[d]);
        Gv[d] = R(0.5) * (G[d] * vc - Gm[d] * vcm);
      }
    } else {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        Gp[d] = G[d];
        Gv[d] = G[d] * vc;
      }
    }
  }
  // phi_tot and its velocity weighting (ic_generator.cc:939-958, 994-1010)
  const C *p1 = reinterpret_cast<const C *>(a.phi[0]);
  C f1 = p1[idx];
  R ps_re = c_s1 * f1.x, ps_im = c_s1 * f1.y;
  R vs_re = c_v1 * ps_re, vs_im = c_v1 * ps_im;
  if (a.qvbc) {
    // -vfac1 C A_theta_bc w grad / k^2 with w = -phi1 / A(k): phi1's velocity
    // weight times 1 + C A_theta_bc / (A k^2 g1)
    const int si = signed_idx(i, N), sj = signed_idx(j, N);
    const size_t n = size_t(si * si + sj * sj + k * k);
    const R q = n < a.qvbc_len ? (F32 ? R(a.qvbc32[n]) : R(a.qvbc[n])) : R(0);
    vs_re += q * vs_re;
    vs_im += q * vs_im;
  }
  C Ad[3] = {mkc<R>(0, 0), mkc<R>(0, 0), mkc<R>(0, 0)};
  if (a.order > 1) {
    const C f2 = reinterpret_cast<const C *>(a.phi[1])[idx];
    const R s2 = c_s2;
    ps_re += s2 * f2.x;
    ps_im += s2 * f2.y;
    vs_re += c_v2 * (s2 * f2.x);
    vs_im += c_v2 * (s2 * f2.y);
  }
  if (a.order > 2) {
    const C f3 = reinterpret_cast<const C *>(a.phi[2])[idx];
    const R s3 = c_s3;
    ps_re += s3 * f3.x;
    ps_im += s3 * f3.y;
    vs_re += c_v3 * (s3 * f3.x);
    vs_im += c_v3 * (s3 * f3.y);
    const R sa = c_sa;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const C v = reinterpret_cast<const C *>(a.A3[d])[idx];
      Ad[d] = mkc<R>(sa * v.x, sa * v.y);
    }
  }
  const bool dc = (idx == 0);
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int d1 = (d + 1) % 3, d2 = (d + 2) % 3;
    // i*(G_d phi) + i*(G_d' A_d'' - G_d'' A_d')
    R tre = Gp[d] * ps_re, tim = Gp[d] * ps_im;
    R vre = Gv[d] * vs_re, vim = Gv[d] * vs_im;
    if (a.order > 2) {
      tre += Gp[d1] * Ad[d2].x - Gp[d2] * Ad[d1].x;
      tim += Gp[d1] * Ad[d2].y - Gp[d2] * Ad[d1].y;
      vre += c_v3 * (Gv[d1] * Ad[d2].x - Gv[d2] * Ad[d1].x);
      vim += c_v3 * (Gv[d1] * Ad[d2].y - Gv[d2] * Ad[d1].y);
    }
    const R pf = c_pf, vf = c_vf;
    P[d] = dc ? mkc<R>(0, 0) : mkc<R>(-tim * pf, tre * pf);
    V[d] = dc ? mkc<R>(0, 0) : mkc<R>(-vim * vf, vre * vf);
  }
}

// the phase of sub-lattice s at mode (i, j, k): exp(i s.k dx) (grid_fft.hh:836-839);
// the FP32 form multiplies the float tables (FP64 arithmetic is slow here)
// NYQ = false: the caller's potentials vanish on every Nyquist index (the
// FP32 form's fused assembly, which runs with NGenIC noise only)
template <typename R, bool NYQ = true>
__device__ __forceinline__ void lattice_phase(const AsmArgs &a, int s, int i, int j, int k, R &er, R &ei) {
  const int N = a.N;
  if constexpr (NYQ) {
    if (nyq_phase<R>(a.nyq, a.phase, s, i, j, k, N, er, ei)) return;
  }
  if constexpr (sizeof(R) == 4) {
    if (a.phase32) {
      const float2 *ph = a.phase32 + size_t(s) * 3 * N;
      const float2 ex = ph[i], ey = ph[N + j], ez = ph[2 * N + k];
      const float exy_re = ex.x * ey.x - ex.y * ey.y, exy_im = ex.x * ey.y + ex.y * ey.x;
      er = exy_re * ez.x - exy_im * ez.y;
      ei = exy_re * ez.y + exy_im * ez.x;
      return;
    }
  }
  const double2 *ph = a.phase + size_t(s) * 3 * N;
  const double2 ex = ph[i], ey = ph[N + j], ez = ph[2 * N + k];
  const double exy_re = ex.x * ey.x - ex.y * ey.y, exy_im = ex.x * ey.y + ex.y * ey.x;
  er = R(exy_re * ez.x - exy_im * ez.y);
  ei = R(exy_re * ez.y + exy_im * ez.x);
}

template <typename R, bool PLT>
__global__ void __launch_bounds__(256) k_assemble(AsmArgs a) {
  using C = typename Cplx<R>::T;
  const int N = a.N, nh = N >> 1, nk = nh + 1;
  const size_t total = size_t(N) * N * nk;
  for (size_t idx = size_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < total;
       idx += size_t(gridDim.x) * blockDim.x) {
    const int k = int(idx % nk);
    const size_t t = idx / nk;
    const int j = int(t % N), i = int(t / N);
    C P[3], V[3];
    asm_mode<R, PLT>(a, i, j, k, idx, P, V);
    for (int s = 0; s < a.nshift; ++s) {
      R er, ei;
      lattice_phase<R>(a, a.shift0 + s, i, j, k, er, ei);
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        reinterpret_cast<C *>(a.out[s * 6 + d])[idx] = mkc<R>(P[d].x * er - P[d].y * ei, P[d].x * ei + P[d].y * er);
        reinterpret_cast<C *>(a.out[s * 6 + 3 + d])[idx] =
            mkc<R>(V[d].x * er - V[d].y * ei, V[d].x * ei + V[d].y * er);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// (5a) particle ids [first, first + count) into dst (particle_generator.hh:
//      229-248): particle p = shift * N^3 + cell carries base + ns * cell + shift
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) k_fill_ids(T *dst, uint64_t first, uint64_t count, uint64_t base, uint64_t ns,
                                                  uint64_t n3) {
  for (uint64_t q = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; q < count;
       q += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t p = first + q, s = p / n3;
    dst[q] = T(base + ns * (p - s * n3) + s);
  }
}

// ---------------------------------------------------------------------------
// (5b) particle masses of a baryon + CDM species (ic_generator.cc:749-780,
//      particle_generator.hh:369-427): delta_bc(k) = w A_delta_bc(k) =
//      ratio[n] * phi1 (ratio = -A_delta_bc / A per |k|^2 index n, with the
//      field's scale folded in), times the sub-lattice phase; after the c2r,
//      mass = (1 + C delta_bc(x) / sqrt(N^3)) * mass_factor / (n_s N^3)
// ---------------------------------------------------------------------------
struct MassArgs {
  const void *phi1;      // N-grid k-space
  const double *ratio;   // per |k|^2 index
  size_t ratio_len;
  const double2 *phase;  // [ns][3][N]
  void *field;           // N-grid, in-place c2r layout
  void *mass;            // particle masses (double or float)
  int N, shift, nshift_total;
  double c_species, norm, scale;  // norm = 1/sqrt(N^3), scale = mass_factor / (n_s N^3)
  NyqSteps nyq;
};

template <typename R>
__global__ void __launch_bounds__(256) k_mass_field(MassArgs a) {
  using C = typename Cplx<R>::T;
  const int N = a.N, nk = N / 2 + 1;
  const size_t total = size_t(N) * N * nk;
  const C *p1 = reinterpret_cast<const C *>(a.phi1);
  C *out = reinterpret_cast<C *>(a.field);
  const double2 *ph = a.phase + size_t(a.shift) * 3 * N;
  for (size_t idx = size_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < total;
       idx += size_t(gridDim.x) * blockDim.x) {
    const int k = int(idx % nk);
    const size_t t = idx / nk;
    const int j = int(t % N), i = int(t / N);
    const int si = signed_idx(i, N), sj = signed_idx(j, N);
    const size_t n = size_t(si * si + sj * sj + k * k);
    const double r = (n > 0 && n < a.ratio_len) ? a.ratio[n] : 0.0;
    double er, ei;
    if (!nyq_phase<double>(a.nyq, a.phase, a.shift, i, j, k, N, er, ei)) {
      const double2 ex = ph[i], ey = ph[N + j], ez = ph[2 * N + k];
      const double exy_re = ex.x * ey.x - ex.y * ey.y, exy_im = ex.x * ey.y + ex.y * ey.x;
      er = exy_re * ez.x - exy_im * ez.y;
      ei = exy_re * ez.y + exy_im * ez.x;
    }
    const C f = p1[idx];
    const double vr = r * double(f.x), vi = r * double(f.y);
    out[idx] = mkc<R>(R(vr * er - vi * ei), R(vr * ei + vi * er));
  }
}

template <typename R, typename M>
__global__ void __launch_bounds__(256) k_masses(MassArgs a) {
  const int N = a.N;
  const size_t n3 = size_t(N) * N * N;
  const R *f = reinterpret_cast<const R *>(a.field);
  M *mass = reinterpret_cast<M *>(a.mass) + size_t(a.shift) * n3;
  for (size_t c = size_t(blockIdx.x) * blockDim.x + threadIdx.x; c < n3; c += size_t(gridDim.x) * blockDim.x) {
    const size_t row = c / size_t(N), k = c - row * size_t(N);
    const double rho = double(f[row * size_t(N + 2) + k]) * a.norm;
    mass[c] = M(((1.0 + a.c_species * rho) * a.scale));
  }
}

// ---------------------------------------------------------------------------
// (6) particle read-out for one sub-lattice shift (particle_generator.hh:212-253,
//     499-543, 597-639): pos = (idx + s)/N * lunit + Psi, vel = v, ID.
// ---------------------------------------------------------------------------
struct PartArgs {
  const void *f[6];  // real fields (rows padded to N+2): pos x,y,z, vel x,y,z
  void *pos, *vel, *ids;
  int N, nshift_total, ishift, pos64, vel64, id64;
  double sx, sy, sz, lunit;
  // unperturbed coordinates (m + s_axis)/N * lunit per axis, [3][N], computed on
  // the host with the reference's expression (grid_fft.hh:240-250)
  const double *qtab;
  uint64_t id_offset;
};

// two consecutive reals of a field row (rows padded to N+2 are 8- / 16-byte
// aligned at even k for float / double)
template <typename R> __device__ __forceinline__ void load2(const R *p, R &x, R &y);
template <> __device__ __forceinline__ void load2<float>(const float *p, float &x, float &y) {
  const float2 v = *reinterpret_cast<const float2 *>(p);
  x = v.x;
  y = v.y;
}
template <> __device__ __forceinline__ void load2<double>(const double *p, double &x, double &y) {
  const double2 v = *reinterpret_cast<const double2 *>(p);
  x = v.x;
  y = v.y;
}

// 12 consecutive outputs (4 particles x xyz) with 16-byte vector stores
__device__ __forceinline__ void store12(double *o, const double *v) {
#pragma unroll
  for (int q = 0; q < 6; ++q) reinterpret_cast<double2 *>(o)[q] = make_double2(v[2 * q], v[2 * q + 1]);
}
__device__ __forceinline__ void store12(float *o, const float *v) {
#pragma unroll
  for (int q = 0; q < 3; ++q) reinterpret_cast<float4 *>(o)[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
}
__device__ __forceinline__ void store12(float *o, const double *v) {
#pragma unroll
  for (int q = 0; q < 3; ++q)
    reinterpret_cast<float4 *>(o)[q] =
        make_float4(float(v[4 * q]), float(v[4 * q + 1]), float(v[4 * q + 2]), float(v[4 * q + 3]));
}

// 6 consecutive outputs (2 particles x xyz, the first at an even index): 16-byte
// stores for double, 8-byte ones for float
__device__ __forceinline__ void store6(double *o, const double *v) {
#pragma unroll
  for (int q = 0; q < 3; ++q) reinterpret_cast<double2 *>(o)[q] = make_double2(v[2 * q], v[2 * q + 1]);
}
__device__ __forceinline__ void store6(float *o, const float *v) {
#pragma unroll
  for (int q = 0; q < 3; ++q) reinterpret_cast<float2 *>(o)[q] = make_float2(v[2 * q], v[2 * q + 1]);
}
__device__ __forceinline__ void store6(float *o, const double *v) {
#pragma unroll
  for (int q = 0; q < 3; ++q) reinterpret_cast<float2 *>(o)[q] = make_float2(float(v[2 * q]), float(v[2 * q + 1]));
}

// One thread per 4 consecutive cells along k (N is a multiple of 4): every
// store is a 16-byte vector store and a warp writes one contiguous run.
template <typename R, typename PosT, typename VelT>
__global__ void __launch_bounds__(256) k_particles(PartArgs a) {
  const int N = a.N;
  const size_t n3 = size_t(N) * N * N, nq = n3 / 4;
  const size_t rowp = size_t(N + 2);
  const size_t base = size_t(a.ishift) * n3;
  for (size_t g = size_t(blockIdx.x) * blockDim.x + threadIdx.x; g < nq; g += size_t(gridDim.x) * blockDim.x) {
    const size_t cell = 4 * g;
    const int k = int(cell % N);
    const size_t tt = cell / N;
    const int j = int(tt % N), i = int(tt / N);
    const size_t r = (size_t(i) * N + j) * rowp + k;
    double pv[12];
    VelT vv[12];  // velocities never pass through FP64 when stored as float
    const double qx = __ldg(&a.qtab[i]), qy = __ldg(&a.qtab[N + j]);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const R *fp = reinterpret_cast<const R *>(a.f[d]) + r;
      const R *fv = reinterpret_cast<const R *>(a.f[3 + d]) + r;
      R p0, p1, p2, p3, v0, v1, v2, v3;
      load2<R>(fp, p0, p1);
      load2<R>(fp + 2, p2, p3);
      load2<R>(fv, v0, v1);
      load2<R>(fv + 2, v2, v3);
      const R ps[4] = {p0, p1, p2, p3}, vs[4] = {v0, v1, v2, v3};
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const double q = d == 0 ? qx : (d == 1 ? qy : __ldg(&a.qtab[2 * N + k + c]));
        pv[3 * c + d] = q + double(ps[c]);
        vv[3 * c + d] = VelT(vs[c]);
      }
    }
    store12(reinterpret_cast<PosT *>(a.pos) + 3 * (base + cell), pv);
    store12(reinterpret_cast<VelT *>(a.vel) + 3 * (base + cell), vv);
    if (a.ids) {
      const uint64_t id0 = a.id_offset + uint64_t(a.nshift_total) * cell + uint64_t(a.ishift);
      const uint64_t st = uint64_t(a.nshift_total);
      if (a.id64) {
        ulonglong2 *o = reinterpret_cast<ulonglong2 *>(reinterpret_cast<uint64_t *>(a.ids) + base + cell);
        o[0] = make_ulonglong2(id0, id0 + st);
        o[1] = make_ulonglong2(id0 + 2 * st, id0 + 3 * st);
      } else {
        *reinterpret_cast<uint4 *>(reinterpret_cast<uint32_t *>(a.ids) + base + cell) =
            make_uint4(uint32_t(id0), uint32_t(id0 + st), uint32_t(id0 + 2 * st), uint32_t(id0 + 3 * st));
      }
    }
  }
}

}  // namespace mfx
