// Pruned, fused 3D transforms for the Orszag-padded convolutions (FP32 form).
//
// The padded fields live on the M-grid (M = 3N/2) but their spectra are
// non-zero only on the N-grid modes.  A 3D transform is done here as three
// passes of 1D transforms whose pencils skip what is known to be zero, with
// the pointwise work of the reference's convolver folded into the passes:
//
//   c2r of a padded Hessian (convolution.hh:552-575 then the c2r):
//     Y pass  (i in the N-grid, kz < N/2): reads phi, applies the Hessian
//             factor -g_a g_b and the pad/normalisation factor, zero-pads the
//             y modes, inverse FFT along y                        -> B[i][y][kz]
//     X pass  (y, kz < N/2): zero-pads the x modes, inverse FFT    -> C[x][y][kz]
//     Z pass  (x, y): rebuilds the Hermitian z pencil from kz < N/2,
//             inverse FFT, real part                               -> H[x][y][z]
//   r2c of a real-space product followed by unpad (convolution.hh:600-636):
//     Z pass  forms the product(s) from the input fields on the fly,
//             forward FFT, keeps kz < N/2                          -> D[x][y][kz]
//     X pass  forward FFT along x, keeps the N-grid x modes       -> E[i][y][kz]
//     Y pass  forward FFT along y, keeps the N-grid y modes, zeroes every
//             Nyquist index, applies the unpad factor and -1/k^2  -> out[i][j][kz]
//     (or, for the pairwise truncation of convolve3, truncates and transforms
//      back along y, then X and Z c2r passes follow)
//
// kz = N/2 (the z Nyquist plane) is identically zero in every padded spectrum
// (phi and all unpadded results zero every Nyquist index), so pencils only
// carry kz < N/2.  Each 1D transform is a mixed-radix (4, 2, 3) Stockham FFT in
// shared memory on P pencils per CTA.
#pragma once
#include <stdint.h>
#if defined(__CUDACC__)
#include <cuda_runtime.h>
#else
// host-only compilation (tests of the transform core on the CPU)
#include <cmath>
struct float2 {
  float x, y;
};
inline float2 make_float2(float a, float b) { return float2{a, b}; }
#define __host__
#define __device__
#define __forceinline__ inline
#endif

namespace mfx {
namespace ff {

struct Stages {
  int n;
  int r[24];
};

// radix sequence for L = 2^a 3^b: 4s first, then a 2, then 3s
__host__ __device__ inline Stages make_stages(int L) {
  Stages s;
  s.n = 0;
  int m = L;
  while (m % 4 == 0) {
    s.r[s.n++] = 4;
    m /= 4;
  }
  if (m % 2 == 0) {
    s.r[s.n++] = 2;
    m /= 2;
  }
  while (m % 3 == 0) {
    s.r[s.n++] = 3;
    m /= 3;
  }
  if (m != 1) s.n = -1;  // unsupported length
  return s;
}

__host__ __device__ inline bool supported_length(int L) { return make_stages(L).n > 0; }

__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// One radix-R butterfly (forward: e^{-2 pi i nk/R}; INV: e^{+...})
template <bool INV> __host__ __device__ __forceinline__ void butterfly(int R, float2 *v) {
  if (R == 2) {
    const float2 a = v[0], b = v[1];
    v[0] = make_float2(a.x + b.x, a.y + b.y);
    v[1] = make_float2(a.x - b.x, a.y - b.y);
  } else if (R == 4) {
    const float2 a = make_float2(v[0].x + v[2].x, v[0].y + v[2].y);
    const float2 b = make_float2(v[0].x - v[2].x, v[0].y - v[2].y);
    const float2 c = make_float2(v[1].x + v[3].x, v[1].y + v[3].y);
    const float2 d = make_float2(v[1].x - v[3].x, v[1].y - v[3].y);
    // forward: y1 = b - i d, y3 = b + i d
    const float2 id = INV ? make_float2(-d.y, d.x) : make_float2(d.y, -d.x);  // (+-i) d
    v[0] = make_float2(a.x + c.x, a.y + c.y);
    v[2] = make_float2(a.x - c.x, a.y - c.y);
    v[1] = make_float2(b.x + id.x, b.y + id.y);
    v[3] = make_float2(b.x - id.x, b.y - id.y);
  } else {  // R == 3
    const float h = 0.86602540378443864676f;  // sqrt(3)/2
    const float2 s = make_float2(v[1].x + v[2].x, v[1].y + v[2].y);
    const float2 d = make_float2(v[1].x - v[2].x, v[1].y - v[2].y);
    const float2 t = make_float2(v[0].x - 0.5f * s.x, v[0].y - 0.5f * s.y);
    // forward: y1 = t - i h d, y2 = t + i h d
    const float2 ihd = INV ? make_float2(-h * d.y, h * d.x) : make_float2(h * d.y, -h * d.x);
    v[0] = make_float2(v[0].x + s.x, v[0].y + s.y);
    v[1] = make_float2(t.x + ihd.x, t.y + ihd.y);
    v[2] = make_float2(t.x - ihd.x, t.y - ihd.y);
  }
}

// Stockham stage: x -> y.  Element (n, p) of a tile lives at n*es + p*ps.
// `t` enumerates (butterfly j, pencil p) pairs; pfast selects which index
// varies fastest across consecutive t (for bank-conflict-free access).
template <bool INV>
__host__ __device__ __forceinline__ void stage_bfly(const float2 *x, float2 *y, const float2 *tw, int L, int R,
                                                    int Ns, int j, int p, int es, int ps) {
  const int nb = L / R;
  const int k = j % Ns;
  const int tstep = k * (L / (Ns * R));
  float2 v[4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
    if (r < R) v[r] = x[(j + r * nb) * es + p * ps];
#pragma unroll
  for (int r = 1; r < 4; ++r) {
    if (r < R) {
      float2 w = tw[(r * tstep) % L];
      if (INV) w.y = -w.y;
      v[r] = cmul(v[r], w);
    }
  }
  butterfly<INV>(R, v);
  const int base = (j / Ns) * Ns * R + k;
#pragma unroll
  for (int r = 0; r < 4; ++r)
    if (r < R) y[(base + r * Ns) * es + p * ps] = v[r];
}

#if defined(__CUDACC__)
// P pencils of length L in shared memory (ping-pong x/y); returns the buffer
// holding the result.  tw[t] = exp(-2 pi i t / L).
template <bool INV>
__device__ float2 *fft_tile(float2 *x, float2 *y, const float2 *tw, int L, int P, int es, int ps, bool pfast) {
  // radices in make_stages order (4s, then a 2, then 3s), derived from the
  // remaining length so that no stage table is needed
  for (int Ns = 1; Ns < L;) {
    const int m = L / Ns;
    const int R = (m % 4 == 0) ? 4 : ((m % 2 == 0) ? 2 : 3);
    const int nb = L / R;
    for (int t = threadIdx.x; t < nb * P; t += blockDim.x) {
      int j, p;
      if (pfast) {
        p = t % P;
        j = t / P;
      } else {
        j = t % nb;
        p = t / nb;
      }
      stage_bfly<INV>(x, y, tw, L, R, Ns, j, p, es, ps);
    }
    __syncthreads();
    float2 *tmp = x;
    x = y;
    y = tmp;
    Ns *= R;
  }
  return x;
}

__device__ __forceinline__ void load_twiddles(float2 *tw, int L) {
  for (int t = threadIdx.x; t < L; t += blockDim.x) {
    float s, c;
    sincospif(-2.0f * float(t) / float(L), &s, &c);
    tw[t] = make_float2(c, s);
  }
}

// N-grid index of padded index ip (convolution.hh:563-572), -1 in the gap
__device__ __forceinline__ int unpad_index(int ip, int N) {
  const int nh = N >> 1;
  return ip <= nh ? ip : (ip > N ? ip - nh : -1);
}
__device__ __forceinline__ int sidx(int i, int n) { return i > (n >> 1) ? i - n : i; }

// Buffers (complex float unless noted), Kh = N/2:
//   phi  N-grid k-space [N][N][N/2+1]
//   B/E  [N][M][Kh]     after the y transform (x still in N-grid modes)
//   C/D  [M][M][Kh]     after the x transform
//   H    real [M][M][M+2] (the in-place padded layout)
struct PassArgs {
  const float2 *in;
  float2 *out;
  float2 *out2;           // Y-forward truncation: transformed-back tile
  const float *rin[17];   // Z r2c: input real fields
  float *rout;            // Z c2r: real output
  float2 *dout[4];        // Z r2c: outputs
  int N, M, Kh;
  int ca, cb;             // Hessian component
  int kind, nout;         // Z r2c source kind / output count
  float kfac, fac;
  float coef;
};

__device__ __forceinline__ float *smem_base() {
  extern __shared__ float4 ff_smem[];
  return reinterpret_cast<float *>(ff_smem);
}

// c2r, Y pass: Hessian (ca, cb) of phi, padded along y, inverse FFT along y.
// grid (N, Kh / P).
template <int P> __global__ void __launch_bounds__(256) k_ff_hess_y(PassArgs a) {
  const int N = a.N, M = a.M, Kh = a.Kh, nh = N >> 1, nk = nh + 1;
  float2 *tw = reinterpret_cast<float2 *>(smem_base());
  float2 *x = tw + M, *y = x + M * P;
  const int i = blockIdx.x, kz0 = blockIdx.y * P;
  load_twiddles(tw, M);
  const float gi = (i != nh) ? float(sidx(i, N)) * a.kfac : 0.f;
  for (int t = threadIdx.x; t < M * P; t += blockDim.x) {
    const int n = t / P, p = t - (t / P) * P, kz = kz0 + p;
    const int j = unpad_index(n, N);
    float2 v = make_float2(0.f, 0.f);
    if (j >= 0) {
      v = a.in[(size_t(i) * N + j) * nk + kz];
      const float g[3] = {gi, (j != nh) ? float(sidx(j, N)) * a.kfac : 0.f, float(kz) * a.kfac};
      const float h = -(g[a.ca] * g[a.cb]) * a.fac;
      v.x *= h;
      v.y *= h;
    }
    x[n * P + p] = v;
  }
  __syncthreads();
  const float2 *r = fft_tile<true>(x, y, tw, M, P, P, 1, true);
  for (int t = threadIdx.x; t < M * P; t += blockDim.x) {
    const int n = t / P, p = t - (t / P) * P;
    a.out[(size_t(i) * M + n) * Kh + kz0 + p] = r[n * P + p];
  }
}

// c2r, X pass: zero-pad x, inverse FFT along x.  grid (M, Kh / P).
template <int P> __global__ void __launch_bounds__(256) k_ff_x_inv(PassArgs a) {
  const int N = a.N, M = a.M, Kh = a.Kh;
  float2 *tw = reinterpret_cast<float2 *>(smem_base());
  float2 *x = tw + M, *y = x + M * P;
  const int yy = blockIdx.x, kz0 = blockIdx.y * P;
  load_twiddles(tw, M);
  for (int t = threadIdx.x; t < M * P; t += blockDim.x) {
    const int n = t / P, p = t - (t / P) * P;
    const int i = unpad_index(n, N);
    x[n * P + p] = (i >= 0) ? a.in[(size_t(i) * M + yy) * Kh + kz0 + p] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  const float2 *r = fft_tile<true>(x, y, tw, M, P, P, 1, true);
  for (int t = threadIdx.x; t < M * P; t += blockDim.x) {
    const int n = t / P, p = t - (t / P) * P;
    a.out[(size_t(n) * M + yy) * Kh + kz0 + p] = r[n * P + p];
  }
}

// c2r, Z pass: Hermitian z pencil from kz < Kh, inverse FFT, real part into
// the padded real layout.  grid (M*M / P).
template <int P> __global__ void __launch_bounds__(256) k_ff_z_c2r(PassArgs a) {
  const int M = a.M, Kh = a.Kh;
  float2 *tw = reinterpret_cast<float2 *>(smem_base());
  float2 *x = tw + M, *y = x + M * P;
  const size_t r0 = size_t(blockIdx.x) * P;
  load_twiddles(tw, M);
  for (int t = threadIdx.x; t < M * P; t += blockDim.x) {
    const int p = t / M, n = t - (t / M) * M;
    float2 v = make_float2(0.f, 0.f);
    if (n < Kh) {
      v = a.in[(r0 + p) * Kh + n];
      if (n == 0) v.y = 0.f;
    } else if (n > M - Kh) {
      const float2 c = a.in[(r0 + p) * Kh + (M - n)];
      v = make_float2(c.x, -c.y);
    }
    x[p * M + n] = v;
  }
  __syncthreads();
  const float2 *r = fft_tile<true>(x, y, tw, M, P, 1, M, false);
  for (int t = threadIdx.x; t < M * P; t += blockDim.x) {
    const int p = t / M, n = t - (t / M) * M;
    a.rout[(r0 + p) * size_t(M + 2) + n] = r[p * M + n].x;
  }
}

// sources formed on the fly in the Z r2c pass (slot order of the Hessians:
// 0 xx 1 yy 2 zz 3 xy 4 xz 5 yz; rin[0..5] = phi1 Hessians, rin[6..11] =
// phi2 Hessians, rin[12..16] = truncated phi3a pair products)
enum { SRC_COPY = 0, SRC_PHI2 = 1, SRC_PAIR = 2, SRC_PHI3 = 3 };

__device__ __forceinline__ int hslot(int x, int y) {
  if (x == y) return x;
  const int lo = x < y ? x : y, hi = x < y ? y : x;
  return lo == 0 ? (hi == 1 ? 3 : 4) : 5;
}

// compensated accumulation (Ogita-Rump-Oishi TwoSum / FMA TwoProduct)
struct Acc32 {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float v) {
    const float s = hi + v, bp = s - hi;
    lo += (hi - (s - bp)) + (v - bp);
    hi = s;
  }
  __device__ __forceinline__ void add_prod(float c, float a, float b) {
    const float p = a * b, e = fmaf(a, b, -p), q = c * p, e2 = fmaf(c, p, -q) + c * e;
    add(q);
    lo += e2;
  }
  __device__ __forceinline__ float value() const { return hi + lo; }
};

__device__ __forceinline__ void sources(const PassArgs &a, size_t idx, float *s) {
  if (a.kind == SRC_COPY) {
    s[0] = a.rin[0][idx];
  } else if (a.kind == SRC_PAIR) {
    s[0] = a.rin[0][idx] * a.rin[1][idx];
  } else if (a.kind == SRC_PHI2) {
    // ic_generator.cc:530-534
    float h[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) h[c] = a.rin[c][idx];
    Acc32 S;
    S.add_prod(1.f, h[0], h[1] + h[2]);
    S.add_prod(1.f, h[1], h[2]);
    S.add_prod(-1.f, h[3], h[3]);
    S.add_prod(-1.f, h[4], h[4]);
    S.add_prod(-1.f, h[5], h[5]);
    s[0] = S.value();
  } else {
    // phi3a + phi3b (ic_generator.cc:581-609) and A3 (613-628)
    float p[6], q[6], T[5];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      p[c] = a.rin[c][idx];
      q[c] = a.rin[6 + c][idx];
    }
#pragma unroll
    for (int c = 0; c < 5; ++c) T[c] = a.rin[12 + c][idx];
    const float c57 = -5.0f / 7.0f, c107 = 10.0f / 7.0f;
    Acc32 S;
    S.add_prod(1.f, T[0], p[2]);
    S.add_prod(2.f, T[1], p[5]);
    S.add_prod(-1.f, T[2], p[0]);
    S.add_prod(-1.f, T[3], p[1]);
    S.add_prod(-1.f, T[4], p[2]);
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
      A.add_prod(1.f, q[hslot(d, d1)], p[hslot(d, d2)]);
      A.add_prod(-1.f, q[hslot(d, d2)], p[hslot(d, d1)]);
      A.add_prod(1.f, p[hslot(d1, d2)], q[hslot(d1, d1)] - q[hslot(d2, d2)]);
      A.add_prod(-1.f, q[hslot(d1, d2)], p[hslot(d1, d1)] - p[hslot(d2, d2)]);
      s[1 + d] = A.value();
    }
  }
}

// r2c, Z pass with the real-space product formed on the fly; keeps kz < Kh.
// grid (M*M / P); nout pencils per row.
template <int P> __global__ void __launch_bounds__(256) k_ff_z_r2c(PassArgs a) {
  const int M = a.M, Kh = a.Kh, no = a.nout;
  float2 *tw = reinterpret_cast<float2 *>(smem_base());
  float2 *x = tw + M, *y = x + M * P * no;
  const size_t r0 = size_t(blockIdx.x) * P;
  load_twiddles(tw, M);
  for (int t = threadIdx.x; t < M * P; t += blockDim.x) {
    const int p = t / M, n = t - (t / M) * M;
    float s[4];
    sources(a, (r0 + p) * size_t(M + 2) + n, s);
    for (int o = 0; o < no; ++o) x[(p * no + o) * M + n] = make_float2(s[o], 0.f);
  }
  __syncthreads();
  const float2 *r = fft_tile<false>(x, y, tw, M, P * no, 1, M, false);
  for (int t = threadIdx.x; t < Kh * P * no; t += blockDim.x) {
    const int q = t / Kh, k = t - (t / Kh) * Kh;
    const int p = q / no, o = q - (q / no) * no;
    a.dout[o][(r0 + p) * Kh + k] = r[q * M + k];
  }
}

// r2c, X pass: forward FFT along x, keep the N-grid x modes.  grid (M, Kh / P).
template <int P> __global__ void __launch_bounds__(256) k_ff_x_fwd(PassArgs a) {
  const int N = a.N, M = a.M, Kh = a.Kh;
  float2 *tw = reinterpret_cast<float2 *>(smem_base());
  float2 *x = tw + M, *y = x + M * P;
  const int yy = blockIdx.x, kz0 = blockIdx.y * P;
  load_twiddles(tw, M);
  for (int t = threadIdx.x; t < M * P; t += blockDim.x) {
    const int n = t / P, p = t - (t / P) * P;
    x[n * P + p] = a.in[(size_t(n) * M + yy) * Kh + kz0 + p];
  }
  __syncthreads();
  const float2 *r = fft_tile<false>(x, y, tw, M, P, P, 1, true);
  for (int t = threadIdx.x; t < M * P; t += blockDim.x) {
    const int n = t / P, p = t - (t / P) * P;
    const int i = unpad_index(n, N);
    if (i >= 0) a.out[(size_t(i) * M + yy) * Kh + kz0 + p] = r[n * P + p];
  }
}

// r2c, Y pass: forward FFT along y, keep the N-grid y modes.
//  kind 0: unpad (zero every Nyquist index), scale, inverse Laplacian
//          (grid_fft.hh:440-449) -> N-grid k-space out
//  kind 1: truncation of convolve3's first pair: zero outside the N-grid
//          modes and on Nyquist, scale, inverse FFT along y -> out2 [N][M][Kh]
// grid (N, Kh / P).
template <int P> __global__ void __launch_bounds__(256) k_ff_y_fwd(PassArgs a) {
  const int N = a.N, M = a.M, Kh = a.Kh, nh = N >> 1, nk = nh + 1;
  float2 *tw = reinterpret_cast<float2 *>(smem_base());
  float2 *x = tw + M, *y = x + M * P;
  const int i = blockIdx.x, kz0 = blockIdx.y * P;
  load_twiddles(tw, M);
  for (int t = threadIdx.x; t < M * P; t += blockDim.x) {
    const int n = t / P, p = t - (t / P) * P;
    x[n * P + p] = a.in[(size_t(i) * M + n) * Kh + kz0 + p];
  }
  __syncthreads();
  float2 *r = fft_tile<false>(x, y, tw, M, P, P, 1, true);
  float2 *other = (r == x) ? y : x;
  if (a.kind == 0) {
    for (int t = threadIdx.x; t < M * P; t += blockDim.x) {
      const int n = t / P, p = t - (t / P) * P, kz = kz0 + p;
      const int j = unpad_index(n, N);
      if (j < 0) continue;
      float2 v = make_float2(0.f, 0.f);
      if (i != nh && j != nh && (i | j | kz) != 0) {
        const float kx = float(sidx(i, N)) * a.kfac, ky = float(sidx(j, N)) * a.kfac, kzz = float(kz) * a.kfac;
        const float f = -a.fac / (kx * kx + ky * ky + kzz * kzz);
        v = r[n * P + p];
        v.x *= f;
        v.y *= f;
      }
      a.out[(size_t(i) * N + j) * nk + kz] = v;
    }
    if (blockIdx.y == 0)  // the kz = N/2 plane of this row is zero
      for (int j = threadIdx.x; j < N; j += blockDim.x) a.out[(size_t(i) * N + j) * nk + nh] = make_float2(0.f, 0.f);
  } else {
    for (int t = threadIdx.x; t < M * P; t += blockDim.x) {
      const int n = t / P, p = t - (t / P) * P;
      const int j = unpad_index(n, N);
      float2 v = make_float2(0.f, 0.f);
      if (j >= 0 && j != nh && i != nh) {
        v = r[n * P + p];
        v.x *= a.fac;
        v.y *= a.fac;
      }
      r[n * P + p] = v;
    }
    __syncthreads();
    const float2 *b = fft_tile<true>(r, other, tw, M, P, P, 1, true);
    for (int t = threadIdx.x; t < M * P; t += blockDim.x) {
      const int n = t / P, p = t - (t / P) * P;
      a.out2[(size_t(i) * M + n) * Kh + kz0 + p] = b[n * P + p];
    }
  }
}
#endif

}  // namespace ff
}  // namespace mfx
