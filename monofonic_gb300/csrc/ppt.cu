// Semiclassical (PPT) Eulerian fields of a species (ic_generator.cc:783-901):
// the wave function psi = rho exp(i Phi / (hbar D+)) built from the real-space
// potentials, one free drift step in k-space, and the density contrast and
// velocities read off psi -- the fields the reference writes through
// output_plugin::write_grid_data for output_type::field_eulerian.
//
// Everything runs in FP64 (the phases Phi / hbar reach hundreds of radians,
// beyond what float arguments of exp(i x) keep), through cuFFT: Z2D for the
// potentials, Z2Z for psi.  cuFFT transforms are unnormalised; the 1/sqrt(N^3)
// of the reference's unitary c2r and the 1/N^3 of a forward-backward pair are
// folded into the pointwise kernels.
#include <cuda_runtime.h>
#include <cufft.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <stdexcept>
#include <vector>

#include "../../include/mfx.h"
#include "common.h"
#include "kernels.cuh"

namespace mfx {
namespace {

__device__ __forceinline__ double kcomp(int i, int n, double kfac) { return double(signed_idx(i, n)) * kfac; }

// padded k-space double field <- factor(n) * src (k-space of R), n = |k|^2/kf^2:
// factor = scale for every mode (ratio == null) or ratio[n] (DC zeroed)
template <typename R>
__global__ void k_ppt_load(const typename Cplx<R>::T *src, double2 *dst, int N, double scale, const double *ratio,
                           size_t ratio_len) {
  const int nk = N / 2 + 1;
  const size_t total = size_t(N) * N * nk;
  for (size_t idx = size_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < total;
       idx += size_t(gridDim.x) * blockDim.x) {
    const int k = int(idx % nk);
    const size_t t = idx / nk;
    const int j = int(t % N), i = int(t / N);
    double f = scale;
    if (ratio) {
      const int si = signed_idx(i, N), sj = signed_idx(j, N);
      const size_t n = size_t(si * si + sj * sj + k * k);
      f = (n > 0 && n < ratio_len) ? ratio[n] : 0.0;
    }
    const auto v = src[idx];
    dst[idx] = make_double2(f * double(v.x), f * double(v.y));
  }
}

// max over the nearest-neighbour steps of the real potential, the loop of
// ic_generator.cc:813-829 (x stops one plane short; y and z wrap); values are
// non-negative, so the bit patterns order like the doubles
__global__ void k_ppt_maxdphi(const double *phr, int N, double norm, unsigned long long *out) {
  const size_t total = size_t(N - 1) * N * N;
  const size_t rs = size_t(N + 2);
  double m = 0.0;
  for (size_t c = size_t(blockIdx.x) * blockDim.x + threadIdx.x; c < total; c += size_t(gridDim.x) * blockDim.x) {
    const int k = int(c % N);
    const size_t t = c / N;
    const int j = int(t % N), i = int(t / N);
    const int jr = (j + 1) % N, kr = (k + 1) % N;
    const double p = phr[(size_t(i) * N + j) * rs + k];
    const double dx = fabs(phr[(size_t(i + 1) * N + j) * rs + k] - p);
    const double dy = fabs(phr[(size_t(i) * N + jr) * rs + k] - p);
    const double dz = fabs(phr[(size_t(i) * N + j) * rs + kr] - p);
    m = fmax(m, fmax(dx, fmax(dy, dz)));
  }
  m *= norm;
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, static_cast<unsigned long long>(__double_as_longlong(m)));
}

// psi = rho exp(i (phi + phi2) / (hbar D+)) on the dense N^3 complex grid
__global__ void k_ppt_psi(const double *phr, const double *ph2r, const double *rhor, double2 *psi, int N, double norm,
                          double inv, double c_species) {
  const size_t total = size_t(N) * N * N, rs = size_t(N + 2);
  for (size_t c = size_t(blockIdx.x) * blockDim.x + threadIdx.x; c < total; c += size_t(gridDim.x) * blockDim.x) {
    const size_t row = c / size_t(N), k = c - row * size_t(N), q = row * rs + k;
    double ph = phr[q];
    if (ph2r) ph += ph2r[q];
    const double rho = rhor ? sqrt(1.0 + c_species * rhor[q] * norm) : 1.0;
    double s, co;
    sincos(ph * norm * inv, &s, &co);
    psi[c] = make_double2(rho * co, rho * s);
  }
}

// psi_k *= exp(-i hbar k^2 D+ / 2) / N^3
__global__ void k_ppt_drift(double2 *psi, int N, double kfac, double a, double inv_n3) {
  const size_t total = size_t(N) * N * N;
  for (size_t c = size_t(blockIdx.x) * blockDim.x + threadIdx.x; c < total; c += size_t(gridDim.x) * blockDim.x) {
    const int k = int(c % N);
    const size_t t = c / N;
    const int j = int(t % N), i = int(t / N);
    const double kx = kcomp(i, N, kfac), ky = kcomp(j, N, kfac), kz = kcomp(k, N, kfac);
    double s, co;
    sincos(-a * (kx * kx + ky * ky + kz * kz), &s, &co);
    const double2 v = psi[c];
    psi[c] = make_double2((v.x * co - v.y * s) * inv_n3, (v.x * s + v.y * co) * inv_n3);
  }
}

// psi *= exp(i phi2 / (hbar D+)); delta = |psi|^2 - 1
__global__ void k_ppt_kick_density(double2 *psi, const double *ph2r, double *delta, int N, double norm, double inv) {
  const size_t total = size_t(N) * N * N, rs = size_t(N + 2);
  for (size_t c = size_t(blockIdx.x) * blockDim.x + threadIdx.x; c < total; c += size_t(gridDim.x) * blockDim.x) {
    double2 v = psi[c];
    if (ph2r) {
      const size_t row = c / size_t(N), k = c - row * size_t(N);
      double s, co;
      sincos(ph2r[row * rs + k] * norm * inv, &s, &co);
      v = make_double2(v.x * co - v.y * s, v.x * s + v.y * co);
      psi[c] = v;
    }
    delta[c] = v.x * v.x + v.y * v.y - 1.0;
  }
}

// g_k = psi_k * i k_d / N^3
__global__ void k_ppt_grad(double2 *g, int N, int d, double kfac, double inv_n3) {
  const size_t total = size_t(N) * N * N;
  for (size_t c = size_t(blockIdx.x) * blockDim.x + threadIdx.x; c < total; c += size_t(gridDim.x) * blockDim.x) {
    const int k = int(c % N);
    const size_t t = c / N;
    const int j = int(t % N), i = int(t / N);
    const double kd = kcomp(d == 0 ? i : (d == 1 ? j : k), N, kfac) * inv_n3;
    const double2 v = g[c];
    g[c] = make_double2(-v.y * kd, v.x * kd);
  }
}

// v = vu Re[(conj(psi) g - psi conj(g)) / (2i / hbar)] / (1 + delta)
//   = vu hbar Im(conj(psi) g) / (1 + delta)
__global__ void k_ppt_velocity(const double2 *psi, const double2 *g, const double *delta, double *v, int N, double vu,
                               double hbar) {
  const size_t total = size_t(N) * N * N;
  for (size_t c = size_t(blockIdx.x) * blockDim.x + threadIdx.x; c < total; c += size_t(gridDim.x) * blockDim.x) {
    const double2 p = psi[c], q = g[c];
    const double im = p.x * q.y - p.y * q.x;
    v[c] = vu * (hbar * im) / (1.0 + delta[c]);
  }
}

unsigned blocks_for(size_t n) {
  const size_t b = (n + 255) / 256;
  return unsigned(b < 152 * 16 ? (b ? b : 1) : 152 * 16);
}

// the call's device scratch and plans, released on every return path
struct Scratch {
  cudaStream_t st = nullptr;
  void *p = nullptr;
  cufftHandle z2d = 0, z2z = 0;
  bool has_z2d = false, has_z2z = false;
  ~Scratch() {
    if (p) {
      cudaFreeAsync(p, st);
      cudaStreamSynchronize(st);
    }
    if (has_z2d) cufftDestroy(z2d);
    if (has_z2z) cufftDestroy(z2z);
  }
};

#define PCU(call)                                                                                    \
  do {                                                                                               \
    const cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess)                                                                           \
      return set_error(e_ == cudaErrorMemoryAllocation ? MFX_ENOMEM : MFX_ECUDA, "%s: %s", #call,       \
                       cudaGetErrorString(e_));                                                      \
  } while (0)
#define PCF(call)                                                                                      \
  do {                                                                                                 \
    const cufftResult r_ = (call);                                                                     \
    if (r_ != CUFFT_SUCCESS) return set_error(MFX_ECUDA, "%s failed (cuFFT status %d)", #call, int(r_)); \
  } while (0)

int ppt_fields(mfx_job *job, double c_species, const double *amp_dbc, size_t amp_len, double *delta, double *vx,
               double *vy, double *vz, double *hbar_out) {
  JobFields f{};
  int rc = job_fields(job, &f);
  if (rc != MFX_OK) return rc;
  if (!f.has_potentials) return set_error(MFX_ESTATE, "job has no potentials (run it first)");
  const int N = f.N;
  const size_t alen = 3 * size_t(N / 2) * (N / 2) + 1;
  if (amp_dbc && amp_len < alen) return set_error(MFX_EINVAL, "amp_dbc needs %zu entries (got %zu)", alen, amp_len);
  if (!std::isfinite(c_species)) return set_error(MFX_EINVAL, "c_species must be finite");
  const double dplus = -f.g1;
  if (!(dplus > 0)) return set_error(MFX_EINVAL, "the job's g1 = -D+ must be negative");
  PCU(cudaSetDevice(f.device));
  Scratch sc;
  sc.st = static_cast<cudaStream_t>(f.stream);
  cudaStream_t st = sc.st;
  const size_t n3 = size_t(N) * N * N, rfield = size_t(N) * N * (N + 2) * 8, cfield = n3 * 16;
  const bool two = f.order >= 2 && f.phi2;
  const size_t nr = 1 + (two ? 1 : 0) + (amp_dbc ? 1 : 0);
  const size_t bytes = nr * rfield + 2 * cfield + n3 * 8 + alen * 8 + 256;
  PCU(cudaMallocAsync(&sc.p, bytes, st));
  char *base = static_cast<char *>(sc.p);
  double *phr = reinterpret_cast<double *>(base);
  double *ph2r = two ? reinterpret_cast<double *>(base + rfield) : nullptr;
  double *rhor = amp_dbc ? reinterpret_cast<double *>(base + (two ? 2 : 1) * rfield) : nullptr;
  double2 *psi = reinterpret_cast<double2 *>(base + nr * rfield);
  double2 *grad = psi + n3;
  double *dl = reinterpret_cast<double *>(grad + n3);
  double *ratio = dl + n3;
  unsigned long long *mx = reinterpret_cast<unsigned long long *>(ratio + alen);
  PCF(cufftPlan3d(&sc.z2d, N, N, N, CUFFT_Z2D));
  sc.has_z2d = true;
  PCF(cufftPlan3d(&sc.z2z, N, N, N, CUFFT_Z2Z));
  sc.has_z2z = true;
  PCF(cufftSetStream(sc.z2d, st));
  PCF(cufftSetStream(sc.z2z, st));
  const double norm = 1.0 / std::sqrt(double(n3));  // the unitary c2r of the reference
  const size_t kt = size_t(N) * N * (N / 2 + 1);
  // real-space growth-scaled potentials g1 phi1 (and g2 phi2); the padded
  // complex layout of the k-space fields is the in-place Z2D layout
  auto load = [&](const void *src, double scale, const double *r, size_t rl, double *dst) -> int {
    if (f.fp64)
      k_ppt_load<double><<<blocks_for(kt), 256, 0, st>>>(static_cast<const double2 *>(src),
                                                          reinterpret_cast<double2 *>(dst), N, scale, r, rl);
    else
      k_ppt_load<float><<<blocks_for(kt), 256, 0, st>>>(static_cast<const float2 *>(src),
                                                         reinterpret_cast<double2 *>(dst), N, scale, r, rl);
    PCU(cudaGetLastError());
    PCF(cufftExecZ2D(sc.z2d, reinterpret_cast<cufftDoubleComplex *>(dst), reinterpret_cast<cufftDoubleReal *>(dst)));
    return MFX_OK;
  };
  if ((rc = load(f.phi1, f.g1 / f.scale1, nullptr, 0, phr)) != MFX_OK) return rc;
  if (two && (rc = load(f.phi2, f.g2 / f.scale2, nullptr, 0, ph2r)) != MFX_OK) return rc;
  if (amp_dbc) {
    // delta_bc(k) = w A_delta_bc with w = -phi1 / A (phi1 = -A w)
    std::vector<double> r(alen, 0.0);
    for (size_t n = 1; n < alen; ++n)
      if (n < f.amp_len && f.amp[n] != 0.0) r[n] = -amp_dbc[n] / (f.amp[n] * f.scale1);
    PCU(cudaMemcpyAsync(ratio, r.data(), alen * 8, cudaMemcpyHostToDevice, st));
    if ((rc = load(f.phi1, 0.0, ratio, alen, rhor)) != MFX_OK) return rc;
  }
  // hbar (ic_generator.cc:813-834)
  PCU(cudaMemsetAsync(mx, 0, sizeof(unsigned long long), st));
  k_ppt_maxdphi<<<blocks_for(size_t(N - 1) * N * N), 256, 0, st>>>(phr, N, norm, mx);
  PCU(cudaGetLastError());
  unsigned long long bits = 0;
  PCU(cudaMemcpyAsync(&bits, mx, sizeof bits, cudaMemcpyDeviceToHost, st));
  PCU(cudaStreamSynchronize(st));
  double maxdphi;
  static_assert(sizeof(maxdphi) == sizeof(bits), "64-bit double");
  std::memcpy(&maxdphi, &bits, sizeof bits);
  const double hbar = maxdphi / M_PI / dplus * 1.01;
  if (!(hbar > 0)) return set_error(MFX_EINVAL, "the potential is flat: hbar = %g", hbar);
  const double inv = 1.0 / (hbar * dplus);
  k_ppt_psi<<<blocks_for(n3), 256, 0, st>>>(phr, ph2r, rhor, psi, N, norm, inv, c_species);
  PCU(cudaGetLastError());
  // one drift step (ic_generator.cc:857-863)
  const double kfac = 2.0 * M_PI / f.boxlen, inv_n3 = 1.0 / double(n3);
  auto *zpsi = reinterpret_cast<cufftDoubleComplex *>(psi);
  PCF(cufftExecZ2Z(sc.z2z, zpsi, zpsi, CUFFT_FORWARD));
  k_ppt_drift<<<blocks_for(n3), 256, 0, st>>>(psi, N, kfac, 0.5 * hbar * dplus, inv_n3);
  PCU(cudaGetLastError());
  PCF(cufftExecZ2Z(sc.z2z, zpsi, zpsi, CUFFT_INVERSE));
  // second kick (2LPT and above) and the density (ic_generator.cc:865-878)
  k_ppt_kick_density<<<blocks_for(n3), 256, 0, st>>>(psi, two ? ph2r : nullptr, dl, N, norm, inv);
  PCU(cudaGetLastError());
  if (delta) PCU(cudaMemcpyAsync(delta, dl, n3 * 8, cudaMemcpyDefault, st));
  // velocities (ic_generator.cc:880-900)
  const double vu = dplus * f.vfac1 / f.boxlen * f.vunit;
  double *outs[3] = {vx, vy, vz};
  auto *zg = reinterpret_cast<cufftDoubleComplex *>(grad);
  for (int d = 0; d < 3; ++d) {
    if (!outs[d]) continue;
    PCU(cudaMemcpyAsync(grad, psi, cfield, cudaMemcpyDeviceToDevice, st));
    PCF(cufftExecZ2Z(sc.z2z, zg, zg, CUFFT_FORWARD));
    k_ppt_grad<<<blocks_for(n3), 256, 0, st>>>(grad, N, d, kfac, inv_n3);
    PCU(cudaGetLastError());
    PCF(cufftExecZ2Z(sc.z2z, zg, zg, CUFFT_INVERSE));
    // the real-space phi1 buffer (N^2 (N+2) doubles) is free once psi exists:
    // the velocity lands there, dense, and is copied out
    k_ppt_velocity<<<blocks_for(n3), 256, 0, st>>>(psi, grad, dl, phr, N, vu, hbar);
    PCU(cudaGetLastError());
    PCU(cudaMemcpyAsync(outs[d], phr, n3 * 8, cudaMemcpyDefault, st));
  }
  PCU(cudaStreamSynchronize(st));
  if (hbar_out) *hbar_out = hbar;
  return MFX_OK;
}

}  // namespace
}  // namespace mfx

extern "C" int mfx_job_ppt_fields(mfx_job *job, double c_species, const double *amp_dbc, size_t amp_len,
                                  double *delta, double *vx, double *vy, double *vz, double *hbar) {
  try {
    return mfx::ppt_fields(job, c_species, amp_dbc, amp_len, delta, vx, vy, vz, hbar);
  } catch (const std::bad_alloc &) {
    return mfx::set_error(MFX_ENOMEM, "host allocation failed");
  } catch (const std::exception &ex) {
    return mfx::set_error(MFX_ECUDA, "%s", ex.what());
  }
}
