// PLT (particle linear theory) eigenmode tables for SC / BCC / FCC lattices,
// the GB300 counterpart of particle::lattice_gradient::init_D
// (particle_plt.hh:68-515), after Joyce, Marcos et al. (2005) and Marcos
// (2008), "discreteness effects" in cosmological N-body initial conditions.
//
//   device: Ewald sums of the lattice dynamical matrix at every site of the
//           64^3 mesh (particle_plt.hh:176-273), 6 real-to-complex FFTs of
//           its components (particle_plt.hh:283-288);
//   host:   per-mode 3x3 eigensystem, fold of the candidate k-vectors into the
//           first Brillouin zone with first-insert-wins bookkeeping in the
//           reference's serial loop order (particle_plt.hh:339-395),
//           neighbour averaging for modes not on the reciprocal lattice
//           (particle_plt.hh:405-459) and the spherical projection to the
//           production tables D_r, D_theta, D_phi, alpha^{-1}
//           (particle_plt.hh:461-499).
// The result depends only on the lattice type; callers cache it.
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <map>
#include <new>
#include <stdexcept>
#include <tuple>
#include <vector>

#include "../../include/mfx.h"
#include "common.h"

namespace mfx {

namespace {

constexpr int NG = MFX_PLT_NGRID;  // 64
constexpr int NK = NG / 2 + 1;     // 33
constexpr int NR = NG + 2;         // padded row

struct Lat {
  double bravais[9], recip[9];
  int invrecip[9];
  int charge_fac;
  std::vector<std::array<double, 3>> normals;
};

Lat lattice_props(int ilat) {
  const double pi = M_PI, twopi = 2.0 * M_PI, fourpi = 4.0 * M_PI;
  Lat L;
  if (ilat == 0) {
    L = Lat{{1, 0, 0, 0, 1, 0, 0, 0, 1}, {twopi, 0, 0, 0, twopi, 0, 0, 0, twopi}, {2, 0, 0, 0, 2, 0, 0, 0, 2}, 1, {}};
    L.normals = {{pi, 0, 0}, {-pi, 0, 0}, {0, pi, 0}, {0, -pi, 0}, {0, 0, pi}, {0, 0, -pi}};
  } else if (ilat == 1) {
    L = Lat{{1, 0, 0.5, 0, 1, 0.5, 0, 0, 0.5}, {twopi, 0, 0, 0, twopi, 0, -twopi, -twopi, fourpi},
            {2, 0, 0, 0, 2, 0, 1, 1, 1}, 2, {}};
    L.normals = {{0, pi, pi},  {0, -pi, pi},  {0, pi, -pi}, {0, -pi, -pi}, {pi, 0, pi},  {-pi, 0, pi},
                 {pi, 0, -pi}, {-pi, 0, -pi}, {pi, pi, 0},  {-pi, pi, 0},  {pi, -pi, 0}, {-pi, -pi, 0}};
  } else {
    L = Lat{{0, 0.5, 0, 0.5, 0, 1, 0.5, 0.5, 0}, {-fourpi, fourpi, twopi, 0, 0, twopi, fourpi, 0, -twopi},
            {0, 1, 1, 1, 0, 1, 0, 2, 0}, 4, {}};
    L.normals = {{twopi, 0, 0}, {-twopi, 0, 0}, {0, twopi, 0}, {0, -twopi, 0}, {0, 0, twopi}, {0, 0, -twopi},
                 {pi, pi, pi},  {pi, pi, -pi},  {pi, -pi, pi}, {pi, -pi, -pi}, {-pi, pi, pi}, {-pi, pi, -pi},
                 {-pi, -pi, pi}, {-pi, -pi, -pi}};
  }
  return L;
}

struct EwaldArgs {
  double B[9], Rc[9];
  double alpha, charge, fft_norm;
  double *D[6];  // xx, xy, xz, yy, yz, zz real fields, rows padded to 66
};

__device__ __forceinline__ void matvec(const double *A, const double v[3], double r[3]) {
  for (int mu = 0; mu < 3; ++mu) {
    r[mu] = 0.0;
    for (int nu = 0; nu < 3; ++nu) r[mu] += A[3 * mu + nu] * v[nu];
  }
}

// One thread per lattice site: real-space images |n_i| <= 3 and reciprocal
// terms |m_i| <= 3 (m != 0) of the Ewald-summed tidal tensor
// (particle_plt.hh:176-273).
__global__ void __launch_bounds__(128) k_plt_ewald(EwaldArgs a) {
  const int site = blockIdx.x * blockDim.x + threadIdx.x;
  if (site >= NG * NG * NG) return;
  const int i = site / (NG * NG), j = (site / NG) % NG, k = site % NG;
  const double dx = 1.0 / double(NG);
  const double pi = 3.141592653589793, fourpi = 4.0 * pi;
  const double sqrtpi = sqrt(pi), pi32 = pow(pi, 1.5);
  const double alpha = a.alpha, alpha2 = alpha * alpha, alpha3 = alpha2 * alpha;
  double x[3] = {dx * double(i), dx * double(j), dx * double(k)};
  double ar[3];
  matvec(a.B, x, ar);
  for (int q = 0; q < 3; ++q) ar[q] = fmod(2.0 + ar[q], 1.0);  // wrap_abs
  double D[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int ix = -3; ix <= 3; ix++)
    for (int iy = -3; iy <= 3; iy++)
      for (int iz = -3; iz <= 3; iz++) {
        const double n[3] = {double(ix), double(iy), double(iz)};
        double bn[3];
        matvec(a.B, n, bn);
        const double d[3] = {ar[0] - bn[0], ar[1] - bn[1], ar[2] - bn[2]};
        const double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        if (r < 1e-14) continue;
        const double r2 = r * r, r3 = r2 * r, r5 = r3 * r2;
        const double ex = exp(-alpha2 * r2);
        const double K1 = -alpha3 / pi32 * ex / r2;
        const double K2 = (erfc(alpha * r) + 2.0 * alpha / sqrtpi * ex * r) / fourpi;
        for (int mu = 0; mu < 3; ++mu)
          for (int nu = mu; nu < 3; ++nu) {
            const double dd = d[mu] * d[nu] * K1 + ((mu == nu ? 1.0 : 0.0) / r3 - 3.0 * (d[mu] * d[nu]) / r5) * K2;
            D[mu][nu] += dd;
            if (mu != nu) D[nu][mu] += dd;
          }
      }
  for (int ix = -3; ix <= 3; ix++)
    for (int iy = -3; iy <= 3; iy++)
      for (int iz = -3; iz <= 3; iz++) {
        if (abs(ix) + abs(iy) + abs(iz) == 0) continue;
        const double m[3] = {double(ix) / NG, double(iy) / NG, double(iz) / NG};
        double kk[3];
        matvec(a.Rc, m, kk);
        const double kmod2 = kk[0] * kk[0] + kk[1] * kk[1] + kk[2] * kk[2];
        const double kr = kk[0] * ar[0] + kk[1] * ar[1] + kk[2] * ar[2];
        const double term = exp(-kmod2 / (4 * alpha2)) * cos(kr) / kmod2 * a.fft_norm;
        for (int mu = 0; mu < 3; ++mu)
          for (int nu = mu; nu < 3; ++nu) {
            const double dd = kk[mu] * kk[nu] * term;
            D[mu][nu] += dd;
            if (mu != nu) D[nu][mu] += dd;
          }
      }
  const size_t r = (size_t(i) * NG + j) * NR + k;
  const bool origin = (site == 0);  // r = 0 carries the background, particle_plt.hh:276-281
  a.D[0][r] = origin ? 1.0 / 3.0 : D[0][0] * a.charge;
  a.D[1][r] = origin ? 0.0 : D[0][1] * a.charge;
  a.D[2][r] = origin ? 0.0 : D[0][2] * a.charge;
  a.D[3][r] = origin ? 1.0 / 3.0 : D[1][1] * a.charge;
  a.D[4][r] = origin ? 0.0 : D[1][2] * a.charge;
  a.D[5][r] = origin ? 1.0 / 3.0 : D[2][2] * a.charge;
}

// symmetric 3x3 eigensystem by cyclic Jacobi rotations; eigenvalues ascending,
// eigenvectors as columns of V
void eigen_sym3(const double Ain[3][3], double ev[3], double V[3][3]) {
  double A[3][3];
  for (int p = 0; p < 3; ++p)
    for (int q = 0; q < 3; ++q) {
      A[p][q] = Ain[p][q];
      V[p][q] = (p == q) ? 1.0 : 0.0;
    }
  for (int sweep = 0; sweep < 64; ++sweep) {
    const double off = A[0][1] * A[0][1] + A[0][2] * A[0][2] + A[1][2] * A[1][2];
    const double dia = A[0][0] * A[0][0] + A[1][1] * A[1][1] + A[2][2] * A[2][2];
    if (off == 0.0 || off < 1e-36 * dia) break;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        if (A[p][q] == 0.0) continue;
        const double theta = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int r = 0; r < 3; ++r) {  // A <- A J
          const double arp = A[r][p], arq = A[r][q];
          A[r][p] = c * arp - s * arq;
          A[r][q] = s * arp + c * arq;
        }
        for (int r = 0; r < 3; ++r) {  // A <- J^T A
          const double apr = A[p][r], aqr = A[q][r];
          A[p][r] = c * apr - s * aqr;
          A[q][r] = s * apr + c * aqr;
        }
        for (int r = 0; r < 3; ++r) {
          const double vrp = V[r][p], vrq = V[r][q];
          V[r][p] = c * vrp - s * vrq;
          V[r][q] = s * vrp + c * vrq;
        }
      }
  }
  int idx[3] = {0, 1, 2};
  std::sort(idx, idx + 3, [&](int x, int y) { return A[x][x] < A[y][y]; });
  double Vs[3][3];
  for (int c = 0; c < 3; ++c) {
    ev[c] = A[idx[c]][idx[c]];
    for (int r = 0; r < 3; ++r) Vs[r][c] = V[r][idx[c]];
  }
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) V[r][c] = Vs[r][c];
}

struct V3d {
  double x = 0, y = 0, z = 0;
};

// host half of init_D: the 6 k-space tensor components -> production tables
void plt_postprocess(int ilat, const std::vector<double> &Dk /* 6 * NG*NG*NK complex */, double *out) {
  const Lat L = lattice_props(ilat);
  const double twopi = 2.0 * M_PI;
  const size_t nm = size_t(NG) * NG * NK;
  auto cre = [&](int c, size_t q) { return Dk[(size_t(c) * nm + q) * 2]; };
  auto sgn = [](int i) { return double(i) - double(i > NG / 2) * NG; };  // get_k index map
  // eigen data per mode: (eval2, eval1), (eval0, e3x), (e3y, e3z)
  std::vector<std::array<double, 6>> eig(nm);
  std::vector<char> has(nm, 0);
  std::map<std::tuple<int, int, int>, size_t> iimap;
  for (int i = 0; i < NG; i++)
    for (int j = 0; j < NG; j++)
      for (int k = 0; k < NK; k++) {
        const size_t q = (size_t(i) * NG + j) * NK + k;
        const double kv[3] = {sgn(i) * twopi, sgn(j) * twopi, sgn(k) * twopi};
        double D[3][3];
        D[0][0] = cre(0, q);
        D[0][1] = D[1][0] = cre(1, q);
        D[0][2] = D[2][0] = cre(2, q);
        D[1][1] = cre(3, q);
        D[1][2] = D[2][1] = cre(4, q);
        D[2][2] = cre(5, q);
        double ev[3], V[3][3];
        eigen_sym3(D, ev, V);
        double e3[3] = {V[0][2], V[1][2], V[2][2]};
        for (double &e : e3) e /= (twopi * NG);
        double ar[3], a[3];
        for (int c = 0; c < 3; ++c) ar[c] = kv[c] / (twopi * NG);
        for (int mu = 0; mu < 3; ++mu) {
          a[mu] = 0.0;
          for (int nu = 0; nu < 3; ++nu) a[mu] += L.recip[3 * mu + nu] * ar[nu];
        }
        for (int l1 = -1; l1 <= 1; ++l1)
          for (int l2 = -1; l2 <= 1; ++l2)
            for (int l3 = -1; l3 <= 1; ++l3)
              for (int isign = 0; isign <= 1; ++isign) {
                const double sign = 2.0 * double(isign) - 1.0;
                const double vs[3] = {double(l1), double(l2), double(l3)};
                double vk[3];
                for (int mu = 0; mu < 3; ++mu) {
                  double rv = 0.0;
                  for (int nu = 0; nu < 3; ++nu) rv += L.recip[3 * mu + nu] * vs[nu];
                  vk[mu] = sign * a[mu] + rv;
                }
                bool in_fbz = true;
                for (const auto &n : L.normals) {
                  const double nv = n[0] * vk[0] + n[1] * vk[1] + n[2] * vk[2];
                  const double nn = n[0] * n[0] + n[1] * n[1] + n[2] * n[2];
                  if (nv > 1.0001 * nn) {
                    in_fbz = false;
                    break;
                  }
                }
                if (!in_fbz) continue;
                const int ix = int(std::round(vk[0] * NG / twopi));
                const int iy = int(std::round(vk[1] * NG / twopi));
                const int iz = int(std::round(vk[2] * NG / twopi));
                iimap.insert({std::make_tuple(ix, iy, iz), q});  // first insert wins
                eig[q] = {ev[2], ev[1], ev[0], e3[0], e3[1], e3[2]};
                has[q] = 1;
              }
      }
  // interpolation to modes not covered (particle_plt.hh:405-459)
  std::vector<std::array<double, 6>> lv(nm);
  for (int i = 0; i < NG; i++)
    for (int j = 0; j < NG; j++)
      for (int k = 0; k < NK; k++) {
        const int ii = i > NG / 2 ? i - NG : i, jj = j > NG / 2 ? j - NG : j, kk = k > NG / 2 ? k - NG : k;
        const double kv[3] = {double(ii), double(jj), double(kk)};
        auto align = [&](V3d v) {
          const double dot = v.x * kv[0] + v.y * kv[1] + v.z * kv[2];
          if (dot < 0.0) {
            v.x = -v.x;
            v.y = -v.y;
            v.z = -v.z;
          }
          return v;
        };
        const int vi[3] = {i, j, k};
        bool inlat = true;
        for (int mu = 0; mu < 3; ++mu) {
          int s = 0;
          for (int nu = 0; nu < 3; ++nu) s += L.invrecip[3 * mu + nu] * vi[nu];
          if (s % 2 != 0) inlat = false;
        }
        V3d l, v;
        if (!inlat) {
          int count = 0;
          const int nb[6][3] = {{ii - 1, jj, kk}, {ii + 1, jj, kk}, {ii, jj - 1, kk},
                                {ii, jj + 1, kk}, {ii, jj, kk - 1}, {ii, jj, kk + 1}};
          for (const auto &b : nb) {
            auto it = iimap.find(std::make_tuple(b[0], b[1], b[2]));
            if (it == iimap.end()) continue;
            const auto &e = eig[it->second];
            ++count;
            l.x += e[0];
            l.y += e[1];
            l.z += e[2];
            V3d w = align(V3d{e[3], e[4], e[5]});
            v.x += w.x;
            v.y += w.y;
            v.z += w.z;
          }
          const double c = double(count);
          l.x /= c; l.y /= c; l.z /= c;
          v.x /= c; v.y /= c; v.z /= c;
        } else {
          auto it = iimap.find(std::make_tuple(ii, jj, kk));
          if (it != iimap.end()) {
            const auto &e = eig[it->second];
            l = V3d{e[0], e[1], e[2]};
            v = align(V3d{e[3], e[4], e[5]});
          }
        }
        const size_t q = (size_t(i) * NG + j) * NK + k;
        lv[q] = {l.x, l.y, l.z, v.x, v.y, v.z};
      }
  // production tables (particle_plt.hh:461-499)
  double *Dr = out, *Dt = out + nm, *Dp = out + 2 * nm, *Ai = out + 3 * nm;
  for (int i = 0; i < NG; i++)
    for (int j = 0; j < NG; j++)
      for (int k = 0; k < NK; k++) {
        const size_t q = (size_t(i) * NG + j) * NK + k;
        const double kx = sgn(i) * twopi, ky = sgn(j) * twopi, kz = sgn(k) * twopi;
        const double mu1 = lv[q][0];
        double e1[3] = {lv[q][3], lv[q][4], lv[q][5]};
        const double en = std::sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
        for (double &e : e1) e /= en;
        const double kr = std::sqrt(kx * kx + ky * ky + kz * kz);
        const double kphi = kr > 0.0 ? std::atan2(ky, kx) : 0.0;
        const double kth = kr > 0.0 ? std::acos(kz / kr) : 0.0;
        const double st = std::sin(kth), ct = std::cos(kth), sp = std::sin(kphi), cp = std::cos(kphi);
        const double er[3] = {st * cp, st * sp, ct}, et[3] = {ct * cp, ct * sp, -st}, ep[3] = {-sp, cp, 0.0};
        double renorm = e1[0] * er[0] + e1[1] * er[1] + e1[2] * er[2];
        if (renorm < 0.01) renorm = 1.0;
        Dr[q] = 1.0;
        Dt[q] = (e1[0] * et[0] + e1[1] * et[1] + e1[2] * et[2]) / renorm;
        Dp[q] = (e1[0] * ep[0] + e1[1] * ep[1] + e1[2] * ep[2]) / renorm;
        Ai[q] = 1.0 / (0.25 * (std::sqrt(1. + 24 * mu1) - 1.));
      }
  Ai[0] = 1.0;
  Dr[0] = 1.0;
  Dt[0] = 0.0;
  Dp[0] = 0.0;
}

}  // namespace

}  // namespace mfx

using namespace mfx;

extern "C" int mfx_plt_table_build(mfx_engine *eng, int lattice, double *out) {
  try {
    if (!eng || !out) return set_error(MFX_EINVAL, "null argument");
    if (lattice < 0 || lattice > 2) return set_error(MFX_EINVAL, "PLT tables exist for SC, BCC and FCC only");
    const int dev = engine_device(eng);
    if (cudaSetDevice(dev) != cudaSuccess) return set_error(MFX_ECUDA, "cudaSetDevice failed");
    const Lat L = lattice_props(lattice);
    const size_t field = size_t(NG) * NG * NR;  // reals per padded field
    double *d = nullptr;
    if (cudaMalloc(&d, 6 * field * sizeof(double)) != cudaSuccess)
      return set_error(MFX_ENOMEM, "PLT: device allocation failed");
    EwaldArgs a;
    for (int q = 0; q < 9; ++q) {
      a.B[q] = L.bravais[q];
      a.Rc[q] = L.recip[q];
    }
    const double eta = 4.0;
    a.alpha = 1.0 / std::sqrt(2) / eta;
    a.charge = 1.0 / std::pow(double(NG), 3) / L.charge_fac;
    a.fft_norm = 1.0 / std::pow(double(NG), 3.0);
    for (int c = 0; c < 6; ++c) a.D[c] = d + size_t(c) * field;
    k_plt_ewald<<<(NG * NG * NG + 127) / 128, 128>>>(a);
    cudaError_t e = cudaGetLastError();
    cufftHandle plan = 0;
    bool planned = false;
    std::vector<double> Dk(6 * size_t(NG) * NG * NK * 2);
    if (e == cudaSuccess) {
      int n[3] = {NG, NG, NG}, rem[3] = {NG, NG, NR}, cem[3] = {NG, NG, NK};
      if (cufftPlanMany(&plan, 3, n, rem, 1, int(field), cem, 1, NG * NG * NK, CUFFT_D2Z, 6) != CUFFT_SUCCESS) {
        cudaFree(d);
        return set_error(MFX_ECUDA, "PLT: cuFFT plan failed");
      }
      planned = true;
      if (cufftExecD2Z(plan, d, (cufftDoubleComplex *)d) != CUFFT_SUCCESS) e = cudaErrorUnknown;
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) {
      // unitary normalisation of the reference's forward transform, undone by
      // its division by fft_norm12 (both 1/512 exactly): raw DFT values
      const size_t nc = size_t(NG) * NG * NK;
      for (int c = 0; c < 6 && e == cudaSuccess; ++c)
        e = cudaMemcpy(Dk.data() + c * nc * 2, d + c * field, nc * 2 * sizeof(double), cudaMemcpyDeviceToHost);
    }
    if (planned) cufftDestroy(plan);
    cudaFree(d);
    if (e != cudaSuccess) return set_error(MFX_ECUDA, "PLT Ewald/FFT failed: %s", cudaGetErrorString(e));
    plt_postprocess(lattice, Dk, out);
    return MFX_OK;
  } catch (const std::bad_alloc &) {
    return set_error(MFX_ENOMEM, "host allocation failed");
  } catch (const std::exception &ex) {
    return set_error(MFX_EINVAL, "%s", ex.what());
  }
}
