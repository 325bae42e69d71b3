// Fused displacement / velocity assembly and particle read-out (FP32 form).
//
// One sub-lattice s at a time, the six real components (Psi_x,y,z, v_x,y,z)
// that the reference assembles in k-space and transforms back one by one
// (ic_generator.cc:929-1053, then particle_generator.hh:499-687) are produced
// by three passes of the pencil FFT of fused.cuh, the N-grid counterpart of
// the padded passes:
//
//   ASM1  units (j, kz block): every mode (i, j, kz) of the tile is assembled
//         (asm_mode: PLT gradient, phi sum, A3 curl, sub-lattice phase) into
//         shared memory and transformed back along x           -> Q[c][x][j][kz]
//   ASM2  units (x, kz block, c): inverse y transform, in place -> Q[c][x][y][kz]
//   ASM3  rows (x, y), persistent, spectra staged by bulk copies: inverse z
//         transforms of the three component pairs, then q + Psi (FP64), v and
//         the IDs of the row's N particles with 16-byte vector stores
//
// kz runs over [0, N/2): the kz = N/2 plane of every component is zero (the
// potentials' Nyquist planes are), and the kz = 0 plane is Hermitian (asm_mode
// takes the odd part of the PLT gradient there), so the z pass is a c2r.
#pragma once
#include "fused.cuh"
#include "kernels.cuh"

namespace mfx {
namespace ff {

struct FAArgs {
  AsmArgs as;             // potentials, PLT tables, phases, coefficients
  float2 *q[6];           // component fields [N][N][N/2] of sub-lattice `shift` (ASM2 in place, ASM3 input)
  float2 *qx[24];         // ASM1 output: component c of sub-lattice shift + s at qx[6 s + c], s < nsub
  int nsub;               // sub-lattices ASM1 emits from one assembly of each mode (1 unless FA::keep)
  // x-only phases: ASM1 applies only the x factor of the sub-lattice phase,
  // that of sub-lattice xsub[s] for output s, and ASM2 the y and z factors
  // (yzphase).  The phase factors per axis commute with the other axes'
  // transforms, so sub-lattices with equal x-shifts share one ASM1 output
  // (FCC: two instead of four).
  int xonly, xsub[4];
  int yzphase;
  const float2 *qin[6];   // ASM2 input when not in place (null: q)
  int halves;             // ASM1 in halves (tiles of 8 pencils; FA::halves), with nsub > 1
  const float2 *tw;       // W_N^t, t < N
  int *status;            // set when a bounded wait ran out
  int shift;              // sub-lattice
  // particle output (particle_generator.hh:212-253, 499-543, 597-639)
  void *pos, *vel, *ids;
  int pos64, vel64, id64, nshift_total;
  // 1: the positions array receives the float displacements Psi (3 floats a
  // particle) instead of q + Psi; the fetch forms q + Psi in FP64 on the host
  // (mfx_job_set_host_positions), the same doubles the device would store
  int pos_disp;
  const double *qtab;     // [3][N] unperturbed coordinates of this sub-lattice
  uint64_t id_offset;
  // The velocity components are carried times vscale and multiplied by
  // vunscale = 1 / vscale at the read-out: the z pass pairs v_x with Psi_z in
  // one complex FFT, whose FP32 rounding follows the larger of the two, so
  // both are brought to the displacements' magnitude.
  float vscale;
  double vunscale;
  float vunscale_f;  // the same in float (velocities stored as float)
};

// The part of the PLT tables (64 x 64 x 33 float4) the CIC gradients of a
// tile (j, kz0 .. kz0 + P - 1; all x) touch: every x, two y rows, at most NZ
// z planes; staged in shared memory once per tile by ASM1 in halves (which
// assembles each mode twice), so that the eight table reads per mode stay off
// L2 (768^3 FCC: 42.3 -> 41.0 ms; the 4-pencil form at 256^3 gained nothing).
template <int N, int P> struct PltSlice {
  static constexpr int NZ = (64 * (P - 1) + N - 1) / N + 2;
  static constexpr int elems = 64 * 2 * NZ;
  const float4 *s;
  int iy0, iz0, nz;
  __device__ __forceinline__ float4 operator()(int p, int q, int r) const {
    return s[(p * 2 + (q == iy0 ? 0 : 1)) * nz + (r - iz0)];
  }
};
// tile shapes per N: pencils P of ASM1 (P2 of ASM2), components CG per
// assembly round (6 / CG rounds re-assemble the tile), rows RW of the z pass
template <int N> struct FA {
  static constexpr int maxJ = Fac<N>::maxJ;
  static constexpr int P = 4;
  // ASM2 pencils: the widest tile (64- or 128-byte row pieces) whose threads
  // and shared memory fit one CTA
  static constexpr size_t s2_of(int p2, int nb) { return size_t(N + nb * N * p2 + 2 * N * p2) * 8; }
  static constexpr int P2 = ((N / 2) % 16 == 0 && 16 * maxJ <= 1024 &&
                             s2_of(16, Fac<N>::steps == 3 ? 2 : 1) <= 227 * 1024)
                                ? 16
                                : ((8 * maxJ <= 768) ? 8 : 4);
  static constexpr int CG = (6 * P * maxJ <= 512) ? 6 : ((3 * P * maxJ <= 1024) ? 3 : 2);
  static constexpr int RW = (256 / (3 * maxJ)) >= 8 ? 8 : ((256 / (3 * maxJ)) >= 4 ? 4 : ((256 / (3 * maxJ)) >= 2 ? 2 : 1));
  static constexpr int Kh = N / 2, nk = N / 2 + 1;
  static constexpr int t1 = CG * P * maxJ;  // ASM1 threads
  static constexpr int t2 = P2 * maxJ;      // ASM2 threads
  static constexpr int t3 = 3 * RW * maxJ;  // ASM3 threads
  static constexpr int nbuf = Fac<N>::steps == 3 ? 2 : 1;
  static constexpr size_t s1 = size_t(N + nbuf * Tile<N, CG * P, true>::elems) * sizeof(float2);
  // ASM1 keeping each mode's six pre-phase components in shared memory, to emit
  // every sub-lattice from one assembly: component group CGK (the largest
  // divisor of 6 up to CG whose tiles fit beside the kept components)
  template <int cg>
  static constexpr size_t s1k_of = size_t(N + nbuf * Tile<N, cg * P, true>::elems + 6 * N * P) * sizeof(float2);
  static constexpr size_t kKeepMax = 220 * 1024;
  static constexpr int CGK = (CG >= 6 && s1k_of<6> <= kKeepMax)   ? 6
                             : (CG >= 3 && s1k_of<3> <= kKeepMax) ? 3
                             : (CG >= 2 && s1k_of<2> <= kKeepMax) ? 2
                                                                  : 1;
  static constexpr bool keep = s1k_of<CGK> <= kKeepMax;
  static constexpr int t1k = CGK * P * maxJ;
  static constexpr size_t s1k = s1k_of<CGK>;
  // ASM1 in halves (x8): tiles of 8 pencils (64-byte row pieces instead of 32),
  // each mode assembled twice — once for the three displacement components,
  // once for the three velocity components, each half kept in shared memory —
  // and every component transformed in place (one tile buffer)
  static constexpr int P8 = 8;
  static constexpr int t1h = 384;
  static constexpr size_t s1h = size_t(N + N * P8 + 3 * N * P8) * sizeof(float2) +
                                size_t(PltSlice<N, P8>::elems) * sizeof(float4);
  static constexpr bool halves = Kh % P8 == 0 && s1h <= 227 * 1024;
  // the x factors of the phases of two shared x pass outputs (x-only), staged
  // after the PLT slice when they fit
  static constexpr size_t s1h_x = 2 * size_t(N) * sizeof(float2);
  static constexpr bool halves_xs = s1h + s1h_x <= 227 * 1024;
  static constexpr size_t s2 = size_t(N + nbuf * Tile<N, P2, true>::elems + 2 * N * P2) * sizeof(float2);
  // CTAs per SM the registers are sized for: no more than shared memory allows
  static constexpr int minb2 = min_blocks(t2) < int(233472 / (s2 + 1024)) ? min_blocks(t2)
                               : (int(233472 / (s2 + 1024)) < 1 ? 1 : int(233472 / (s2 + 1024)));
  static constexpr size_t head = 32;
  // ASM3: the components land in the tile buffer the transform's last step
  // reads (in place) or has finished with, so no buffer of their own
  static constexpr size_t s3 = head + size_t(TwTab<N>::elems) * sizeof(float2) + size_t(RW * 6 * Kh) * sizeof(float2) +
                               size_t(nbuf * Tile<N, 3 * RW, false>::elems) * sizeof(float2);
  // CTAs per SM the ASM3 registers are sized for (about 104 a thread; 72 for
  // the one-row groups of the long lengths, which fit them without spills),
  // no more than shared memory allows
  static constexpr int regs3 = RW == 1 ? 72 : 104;
  static constexpr int minb3_r = 65536 / (t3 * regs3) < 1 ? 1 : 65536 / (t3 * regs3);
  static constexpr int minb3_s = int(233472 / (s3 + 1024)) < 1 ? 1 : int(233472 / (s3 + 1024));
  static constexpr int minb3 = minb3_r < minb3_s ? minb3_r : minb3_s;
};

// stages the slice of tile (j, kz0) with nt threads (the caller synchronises)
template <int N, int P>
__device__ __forceinline__ PltSlice<N, P> stage_plt(const float4 *T, float4 *sm, int j, int kz0, int nt) {
  PltSlice<N, P> sl;
  sl.s = sm;
  sl.iy0 = (64 * j) / N;
  sl.iz0 = (64 * kz0) / N;
  const int izh = min((64 * (kz0 + P - 1)) / N + 1, 32);
  sl.nz = izh - sl.iz0 + 1;
  const int iy1 = (sl.iy0 + 1) & 63;
  for (int t = threadIdx.x; t < 128 * sl.nz; t += nt) {
    const int pq = t / sl.nz, r = sl.iz0 + (t - pq * sl.nz), p = pq >> 1, q = (pq & 1) ? iy1 : sl.iy0;
    sm[t] = __ldg(&T[(p * 64 + q) * 33 + r]);
  }
  return sl;
}

// ASM1: assembly of the tile's modes and the inverse x transform.  KEEP:
// each mode is assembled once (PLT gradient, potentials), its six pre-phase
// components kept in shared memory, and the a.nsub sub-lattices emitted from
// them, each with its own phase; otherwise one sub-lattice (a.shift), the
// assembly repeated for each group of CG components.
template <int N, bool PLT, bool KEEP>
__global__ void __launch_bounds__(KEEP ? FA<N>::t1k : FA<N>::t1, min_blocks(KEEP ? FA<N>::t1k : FA<N>::t1))
    k_fa_x(FAArgs a) {
  using F = FA<N>;
  constexpr int P = F::P, CG = KEEP ? F::CGK : F::CG, PP = CG * P, KB = F::Kh / P;
  float2 *tw = ff_smem(), *buf = tw + N, *buf2 = buf + (F::nbuf == 2 ? Tile<N, PP, true>::elems : 0);
  float2 *pv = buf + F::nbuf * Tile<N, PP, true>::elems;  // [6][mode] (KEEP)
  load_tw<N>(tw, a.tw);
  const int nsub = KEEP ? a.nsub : 1;
#pragma unroll 1
  for (unsigned u = blockIdx.x; u < unsigned(N * KB); u += gridDim.x) {
    const int j = int(u / KB), kz0 = int(u % KB) * P;
    if constexpr (KEEP) {
      // each thread later reads back only the entries it wrote here
      for (int t = threadIdx.x; t < N * P; t += blockDim.x) {
        const int i = t / P, p = t - (t / P) * P, kz = kz0 + p;
        float2 Pm[3], Vm[3];
        asm_mode<float, PLT>(a.as, i, j, kz, (size_t(i) * N + j) * F::nk + kz, Pm, Vm);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          pv[c * (N * P) + t] = Pm[c];
          pv[(3 + c) * (N * P) + t] = make_float2(Vm[c].x * a.vscale, Vm[c].y * a.vscale);
        }
      }
    }
#pragma unroll 1
    for (int s = 0; s < nsub; ++s) {
#pragma unroll 1
      for (int g0 = 0; g0 < 6; g0 += CG) {
        // the tile's modes, components g0 .. g0 + CG - 1, PF layout: buf[i][c][p]
        for (int t = threadIdx.x; t < N * P; t += blockDim.x) {
          const int i = t / P, p = t - (t / P) * P, kz = kz0 + p;
          float2 v6[CG];
          if constexpr (KEEP) {
#pragma unroll
            for (int c = 0; c < CG; ++c) v6[c] = pv[(g0 + c) * (N * P) + t];
          } else {
            float2 Pm[3], Vm[3];
            asm_mode<float, PLT>(a.as, i, j, kz, (size_t(i) * N + j) * F::nk + kz, Pm, Vm);
#pragma unroll
            for (int c = 0; c < CG; ++c) {
              const int cc = g0 + c;
              v6[c] = cc < 3 ? Pm[cc] : make_float2(Vm[cc - 3].x * a.vscale, Vm[cc - 3].y * a.vscale);
            }
          }
          float er, ei;
          if (a.xonly) {
            const float2 e = a.as.phase32[size_t(a.xsub[s]) * 3 * N + i];
            er = e.x;
            ei = e.y;
          } else {
            lattice_phase<float, false>(a.as, a.shift + s, i, j, kz, er, ei);
          }
#pragma unroll
          for (int c = 0; c < CG; ++c) {
            const float2 v = v6[c];
            buf[i * PP + c * P + p] = make_float2(v.x * er - v.y * ei, v.x * ei + v.y * er);
          }
        }
        __syncthreads();
        pencil_fft<N, PP, true, true>(
            buf, buf2, tw, [&](int q, int n) { return buf[n * PP + q]; },
            [&](int q, int x, float2 v) {
              const int c = q / P, p = q - (q / P) * P;
              a.qx[s * 6 + g0 + c][(unsigned(x) * N + j) * F::Kh + kz0 + p] = v;
            });
        __syncthreads();  // the next round assembles into buf
      }
    }
  }
}

// ASM1 in halves: as the KEEP form, with tiles of 8 pencils and the six
// components in two halves of three (the displacement, then the velocity
// components), each half from its own assembly of the tile's modes; every
// (sub-lattice, component) pencil set is transformed in place.
template <int N, bool PLT>
__global__ void __launch_bounds__(FA<N>::t1h, 1) k_fa_x_halves(FAArgs a) {
  using F = FA<N>;
  constexpr int P = F::P8, KB = F::Kh / P, NT = F::t1h;
  using T = Tile<N, P, true>;
  float2 *tw = ff_smem(), *buf = tw + N, *pv = buf + T::elems;  // pv [3][mode]
  float4 *plts = reinterpret_cast<float4 *>(pv + 3 * N * P);    // PLT slice
  // x-only phases from shared memory (two outputs at most), else global
  float2 *phx = reinterpret_cast<float2 *>(plts + PltSlice<N, P>::elems);
  const bool xs = F::halves_xs && a.xonly && a.nsub <= 2;
  if (xs)
    for (int t = threadIdx.x; t < a.nsub * N; t += NT)
      phx[t] = a.as.phase32[size_t(a.xsub[t / N]) * 3 * N + (t - (t / N) * N)];
  load_tw<N>(tw, a.tw);  // includes a barrier
#pragma unroll 1
  for (unsigned u = blockIdx.x; u < unsigned(N * KB); u += gridDim.x) {
    const int j = int(u / KB), kz0 = int(u % KB) * P;
    PltSlice<N, P> sl{};
    if constexpr (PLT) {
      // the previous tile's assemblies ended before its transforms' barriers
      sl = stage_plt<N, P>(a.as.plt4, plts, j, kz0, NT);
      __syncthreads();
    }
#pragma unroll 1
    for (int h = 0; h < 2; ++h) {
      // each thread later reads back only the entries it wrote here
      for (int t = threadIdx.x; t < N * P; t += NT) {
        const int i = t / P, p = t - (t / P) * P, kz = kz0 + p;
        float2 Pm[3], Vm[3];
        if constexpr (PLT)
          asm_mode<float, PLT>(a.as, i, j, kz, (size_t(i) * N + j) * F::nk + kz, Pm, Vm, &sl);
        else
          asm_mode<float, PLT>(a.as, i, j, kz, (size_t(i) * N + j) * F::nk + kz, Pm, Vm);
#pragma unroll
        for (int c = 0; c < 3; ++c)
          pv[c * (N * P) + t] = h == 0 ? Pm[c] : make_float2(Vm[c].x * a.vscale, Vm[c].y * a.vscale);
      }
#pragma unroll 1
      for (int s = 0; s < a.nsub; ++s) {
#pragma unroll 1
        for (int c = 0; c < 3; ++c) {
          // the previous transform's last step has read buf before its barrier
          for (int t = threadIdx.x; t < N * P; t += NT) {
            const int i = t / P, p = t - (t / P) * P;
            float er, ei;
            if (xs) {
              const float2 e = phx[s * N + i];
              er = e.x;
              ei = e.y;
            } else if (a.xonly) {
              const float2 e = a.as.phase32[size_t(a.xsub[s]) * 3 * N + i];
              er = e.x;
              ei = e.y;
            } else {
              lattice_phase<float, false>(a.as, a.shift + s, i, j, kz0 + p, er, ei);
            }
            const float2 v = pv[c * (N * P) + t];
            buf[T::at(p, i)] = make_float2(v.x * er - v.y * ei, v.x * ei + v.y * er);
          }
          __syncthreads();
          float2 *dst = a.qx[s * 6 + 3 * h + c] + (unsigned(j) * F::Kh + kz0);
          pencil_fft_mi<N, P, true, true, NT>(
              buf, tw, [&](int q, int n) { return buf[T::at(q, n)]; },
              [&](int q, int x, float2 v) { dst[unsigned(x) * N * F::Kh + q] = v; });
        }
      }
    }
  }
}

// ASM2: inverse y transforms of the six components, in place (or from qin).
// YZ: the y and z factors of sub-lattice a.shift's phase applied on input
// (x-only ASM1), both staged in shared memory after the tile areas (a global
// load of the z factors at the start of each unit's transform held up its
// first step: 6.1 instead of 4.4 ms a launch at 768^3)
template <int N, bool YZ>
__global__ void __launch_bounds__(FA<N>::t2, FA<N>::minb2) k_fa_y(FAArgs a) {
  using F = FA<N>;
  constexpr int P = F::P2, KB = F::Kh / P;
  float2 *tw = ff_smem(), *buf = tw + N, *buf2 = buf + (F::nbuf == 2 ? Tile<N, P, true>::elems : 0),
         *stage = buf + F::nbuf * Tile<N, P, true>::elems;
  float2 *phy = stage + 2 * N * P;  // YZ: [N] y factors, then [Kh] z factors of the sub-lattice phase
  float2 *phzs = phy + N;
  if constexpr (YZ)
    for (int t = threadIdx.x; t < N + F::Kh; t += blockDim.x) phy[t] = a.as.phase32[size_t(a.shift) * 3 * N + N + t];
  load_tw<N>(tw, a.tw);  // includes a barrier
  xy_units(
      unsigned(N * KB * 6), N * P, stage,
      [&](unsigned u, float2 *st) {
        const unsigned c = u % 6, t = u / 6, x = t / KB, kz0 = (t % KB) * P;
        const float2 *src = a.qin[c] ? a.qin[c] : a.q[c];
        stage_rows<P, N, 16>(st, src + (x * N * F::Kh + kz0), unsigned(F::Kh));
      },
      [&](unsigned u, const float2 *st) {
        const unsigned c = u % 6, t = u / 6, x = t / KB, kz0 = (t % KB) * P;
        float2 *out = a.q[c] + (x * N * F::Kh + kz0);
        const float2 *phz = phzs + kz0;
        pencil_fft<N, P, true, true>(
            buf, buf2, tw,
            [&](int q, int n) {
              const float2 v = st[n * P + q];
              if constexpr (!YZ) {
                return v;
              } else {
                const float2 ey = phy[n], ez = phz[q];
                const float er = ey.x * ez.x - ey.y * ez.y, ei = ey.x * ez.y + ey.y * ez.x;
                return make_float2(v.x * er - v.y * ei, v.x * ei + v.y * er);
              }
            },
            [&](int q, int y, float2 v) { out[unsigned(y) * F::Kh + q] = v; });
      });
}

// float -> double by moving the bit fields (exact, the same value the FP64
// conversion gives): keeps the conversions of the read-out off the FP64 pipe,
// which is narrow on this part and also carries the q + Psi additions
__device__ __forceinline__ double f2d_exact(float f) {
  const uint32_t u = __float_as_uint(f);
  uint32_t e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
  uint32_t ed;
  if (e == 0xffu) {
    ed = 0x7ffu;  // inf / nan (the payload moves along)
  } else if (e != 0u) {
    ed = e + (1023u - 127u);
  } else if (m != 0u) {
    // subnormal float: normalise (a normal double)
    const int lz = __clz(int(m)) - 8;  // shift bringing the leading one to bit 23
    m = (m << lz) & 0x7fffffu;
    ed = uint32_t(1023 - 126 - lz);
  } else {
    ed = 0u;  // +-0
  }
  const uint64_t d = (uint64_t(u & 0x80000000u) << 32) | (uint64_t(ed) << 52) | (uint64_t(m) << 29);
  return __longlong_as_double(static_cast<long long>(d));
}

// ASM3: inverse z transforms (c2r, component pairs (0,1), (2,3), (4,5)) and the
// particles of RW rows at a time
template <int N>
__global__ void __launch_bounds__(FA<N>::t3, FA<N>::minb3) k_fa_z(FAArgs a) {
  using F = FA<N>;
  constexpr int RW = F::RW, Kh = F::Kh, G = 3 * RW;
  char *base = reinterpret_cast<char *>(ff_smem());
  uint64_t *bar = reinterpret_cast<uint64_t *>(base);
  volatile int *flag = reinterpret_cast<volatile int *>(base + 16);
  float2 *tw = reinterpret_cast<float2 *>(base + F::head);
  float2 *stage = tw + TwTab<N>::elems;          // [w][c][Kh]
  float2 *buf = stage + RW * 6 * Kh;
  float2 *buf2 = F::nbuf == 2 ? buf + Tile<N, G, false>::elems : nullptr;
  // [w][pair][z]: written by the transform's last step into buf, which that
  // step reads in place with two steps (a barrier between its reads and
  // writes) and has finished with after the middle step with three
  float2 *h2 = buf;
  const size_t ngroups = size_t(N) * N / RW;
  constexpr uint32_t rowbytes = uint32_t(Kh) * sizeof(float2);
  auto fetch = [&](size_t g) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(bar, rowbytes * 6 * RW);
    for (int w = 0; w < RW; ++w)
      for (int c = 0; c < 6; ++c) bulk_g2s(stage + (w * 6 + c) * Kh, a.q[c] + (g * RW + w) * Kh, rowbytes, bar);
  };
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    *flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  load_tw_steps<N>(tw, a.tw);
  size_t g = blockIdx.x;
  if (threadIdx.x == 0 && g < ngroups) fetch(g);
  const size_t n3 = size_t(N) * N * N, pbase = size_t(a.shift) * n3;
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
    // buf (h2) was last read by the previous group's read-out, before the barrier above
    pencil_fft<N, G, false, true, false, false, Fac<N>::steps == 2>(
        buf, buf2, tw,
        [&](int q, int n) -> float2 {
          const int w = q / 3, c0 = 2 * (q - w * 3);
          int m;
          bool conj;
          if (n < Kh) {
            m = n;
            conj = false;
          } else if (n > N - Kh) {
            m = N - n;
            conj = true;
          } else {
            return make_float2(0.f, 0.f);
          }
          const float2 *row = stage + w * 6 * Kh;
          float2 va = row[c0 * Kh + m], vb = row[(c0 + 1) * Kh + m];
          if (m == 0) {
            va.y = 0.f;
            vb.y = 0.f;
          }
          return conj ? pack_pair_conj(va, vb) : pack_pair(va, vb);
        },
        [&](int q, int z, float2 v) { h2[q * N + z] = v; });
    __syncthreads();  // the stage is free, the components are in h2
    if (threadIdx.x == 0 && gn < ngroups) fetch(gn);
    // two particles per thread (registers for three CTAs per SM); every store
    // a 16- or 8-byte vector store
    for (int t = threadIdx.x; t < RW * (N / 2); t += blockDim.x) {
      const int w = t / (N / 2), z0 = 2 * (t - w * (N / 2));
      const size_t row = g * RW + w, cell = row * N + z0;
      const int x = int(row / N), y = int(row - size_t(x) * N);
      const float2 *hw = h2 + w * 3 * N;
      // q + Psi in FP64; the velocities stay in float unless stored in FP64
      // (FP64 arithmetic and conversions are slow on this part)
      float pf[6], vv[6];
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const float2 a0 = hw[z0 + c], a1 = hw[N + z0 + c], a2 = hw[2 * N + z0 + c];
        pf[3 * c + 0] = a0.x;
        pf[3 * c + 1] = a0.y;
        pf[3 * c + 2] = a1.x;
        vv[3 * c + 0] = a1.y;
        vv[3 * c + 1] = a2.x;
        vv[3 * c + 2] = a2.y;
      }
      if (a.pos_disp) {
        store6(reinterpret_cast<float *>(a.pos) + 3 * (pbase + cell), pf);
      } else {
        double pv[6];
        const double qx = a.qtab[x], qy = a.qtab[N + y];
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          pv[3 * c + 0] = qx + f2d_exact(pf[3 * c + 0]);
          pv[3 * c + 1] = qy + f2d_exact(pf[3 * c + 1]);
          pv[3 * c + 2] = a.qtab[2 * N + z0 + c] + f2d_exact(pf[3 * c + 2]);
        }
        if (a.pos64) store6(reinterpret_cast<double *>(a.pos) + 3 * (pbase + cell), pv);
        else store6(reinterpret_cast<float *>(a.pos) + 3 * (pbase + cell), pv);
      }
      if (a.vel64) {
        double vd[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) vd[c] = double(vv[c]) * a.vunscale;
        store6(reinterpret_cast<double *>(a.vel) + 3 * (pbase + cell), vd);
      } else {
#pragma unroll
        for (int c = 0; c < 6; ++c) vv[c] *= a.vunscale_f;
        store6(reinterpret_cast<float *>(a.vel) + 3 * (pbase + cell), vv);
      }
      if (a.ids) {
        const uint64_t st = uint64_t(a.nshift_total), id0 = a.id_offset + st * cell + uint64_t(a.shift);
        if (a.id64)
          *reinterpret_cast<ulonglong2 *>(reinterpret_cast<uint64_t *>(a.ids) + pbase + cell) =
              make_ulonglong2(id0, id0 + st);
        else
          *reinterpret_cast<uint2 *>(reinterpret_cast<uint32_t *>(a.ids) + pbase + cell) =
              make_uint2(uint32_t(id0), uint32_t(id0 + st));
      }
    }
    // h2 is rewritten by the next group's transform, after the barrier at its top
  }
}

}  // namespace ff
}  // namespace mfx
