/*
 * ORACLE -- test infrastructure only.  Nothing in the product links this file;
 * only tests/ (as a checker of it against oracle/lpt.py) and bench.py's CPU
 * baseline leg and reference arm load it.
 *
 * C++/OpenMP restatement of monofonIC's CPU hot path for one dark-matter
 * species, written to keep the reference's loop structure so that its timing
 * stands for the reference's OpenMP path on the same host cores:
 *
 *   Fill_Grid (NGenIC, serial per-column RANLUX, random_ngenic.cc:84-154; the
 *     restatement in oracle/ranlux.c is linked into the same library)
 *   -> noise normalise / fix / invert (ic_generator.cc:378-383)
 *   -> phi1 = -A(k) w (ic_generator.cc:509-516; A from the amplitude table)
 *   -> 2LPT / 3LPT potentials, one Orszag convolve2 / convolve3 per reference
 *      call (ic_generator.cc:525-628; convolution.hh:495-651): pad_insert of
 *      both Hessian functors, two padded c2r, a real-space product, one padded
 *      r2c, unpad into the output operator -- 3 padded FFTs per convolve2,
 *      99 for 3LPT
 *   -> growth scaling (ic_generator.cc:645-658)
 *   -> per component: the k-space assembly loop with the per-mode PLT
 *      gradient / vfac_corr calls (ic_generator.cc:929-1053;
 *      particle_plt.hh:551-585), a c2r, then per sub-lattice shift_field
 *      (r2c, phase, c2r; grid_fft.hh:832-842) and the read-out into the
 *      particle container (particle_generator.hh:499-639)
 *   -> particle ids (particle_generator.hh:212-253).
 *
 * Loops are OpenMP-parallel where the reference's are (`#pragma omp parallel
 * for` in the cited loops) and serial where the reference's are (the NGenIC
 * fill and the particle read-out).  The FFTs are this file's own batched
 * mixed-radix (4, 2, 3) Stockham transforms, multi-threaded over pencils, in
 * the reference's in-place Grid_FFT layout (real rows padded to N+2, k-space
 * [N][N][N/2+1]) with its unitary 1/sqrt(N^3) normalisation both ways; the
 * multi-dimensional c2r runs the complex x and y transforms before the real
 * transform along z, as FFTW's rdft2 plans do.  The reference uses FFTW3
 * (absent here), so this is a CPU restatement, not FFTW.
 */
#include <omp.h>

#include <chrono>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

extern "C" void mfxo_ngenic_fill(size_t nres, const uint32_t *table, double *out, double *uniforms);

namespace {

using cplx = std::complex<double>;
constexpr double kPi = 3.14159265358979323846;

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// ---------------------------------------------------------------------------
// Batched 1D complex FFT: B independent transforms of length n, stored split
// (real block, imaginary block), element t of transform b at t*B + b, so that
// the innermost loops run over b and vectorise.  Stockham autosort, radices
// 4, 2 and 3; stage s with radix R reads x[j + r*n/R] and writes
// y[(j/Ns)*Ns*R + j%Ns + r*Ns] after the twiddle exp(-+2 pi i r (j%Ns)/(Ns R)).
// ---------------------------------------------------------------------------
struct Fft1 {
  int n = 0;
  std::vector<int> radix, span;                 // per stage: R, Ns
  std::vector<std::vector<double>> twr, twi;    // per stage: [(j%Ns)*(R-1) + r-1]

  explicit Fft1(int len) : n(len) {
    int rest = n, ns = 1;
    while (rest > 1) {
      int R = (rest % 4 == 0) ? 4 : (rest % 2 == 0) ? 2 : (rest % 3 == 0) ? 3 : 0;
      if (R == 0) std::abort();  // lengths are 2^a 3^b here
      std::vector<double> wr(size_t(ns) * (R - 1)), wi(size_t(ns) * (R - 1));
      for (int jr = 0; jr < ns; ++jr)
        for (int r = 1; r < R; ++r) {
          const double ang = -2.0 * kPi * double(r) * double(jr) / double(ns * R);
          wr[size_t(jr) * (R - 1) + r - 1] = std::cos(ang);
          wi[size_t(jr) * (R - 1) + r - 1] = std::sin(ang);
        }
      radix.push_back(R);
      span.push_back(ns);
      twr.push_back(std::move(wr));
      twi.push_back(std::move(wi));
      ns *= R;
      rest /= R;
    }
  }

  // Transforms B columns in (xr, xi); y is scratch of the same size.  sign -1:
  // forward (exp(-i...)), +1: backward, unnormalised.  Returns true when the
  // result is in (yr, yi), false when it is in (xr, xi).
  bool run(double *xr, double *xi, double *yr, double *yi, int B, int sign) const {
    double *ar = xr, *ai = xi, *br = yr, *bi = yi;
    const double s = double(sign);
    for (size_t st = 0; st < radix.size(); ++st) {
      const int R = radix[st], ns = span[st], m = n / R;
      // the tables hold the forward twiddles; the backward transform takes their conjugates
      const double *wr = twr[st].data(), *wi = twi[st].data();
      for (int j = 0; j < m; ++j) {
        const int jr = j % ns;
        const size_t o = size_t(j - jr) * R + jr;
        const double *tr = wr + size_t(jr) * (R - 1), *ti = wi + size_t(jr) * (R - 1);
        if (R == 4) {
          const double w1r = tr[0], w1i = -s * ti[0], w2r = tr[1], w2i = -s * ti[1];
          const double w3r = tr[2], w3i = -s * ti[2];
          const double *x0r = ar + size_t(j) * B, *x0i = ai + size_t(j) * B;
          const double *x1r = ar + size_t(j + m) * B, *x1i = ai + size_t(j + m) * B;
          const double *x2r = ar + size_t(j + 2 * m) * B, *x2i = ai + size_t(j + 2 * m) * B;
          const double *x3r = ar + size_t(j + 3 * m) * B, *x3i = ai + size_t(j + 3 * m) * B;
          double *y0r = br + o * B, *y0i = bi + o * B;
          double *y1r = br + (o + ns) * B, *y1i = bi + (o + ns) * B;
          double *y2r = br + (o + 2 * size_t(ns)) * B, *y2i = bi + (o + 2 * size_t(ns)) * B;
          double *y3r = br + (o + 3 * size_t(ns)) * B, *y3i = bi + (o + 3 * size_t(ns)) * B;
#pragma omp simd
          for (int b = 0; b < B; ++b) {
            const double v0r = x0r[b], v0i = x0i[b];
            const double v1r = x1r[b] * w1r - x1i[b] * w1i, v1i = x1r[b] * w1i + x1i[b] * w1r;
            const double v2r = x2r[b] * w2r - x2i[b] * w2i, v2i = x2r[b] * w2i + x2i[b] * w2r;
            const double v3r = x3r[b] * w3r - x3i[b] * w3i, v3i = x3r[b] * w3i + x3i[b] * w3r;
            const double ar_ = v0r + v2r, ai_ = v0i + v2i, br_ = v0r - v2r, bi_ = v0i - v2i;
            const double cr = v1r + v3r, ci = v1i + v3i, dr = v1r - v3r, di = v1i - v3i;
            // X1 = b + sign*i*d, X3 = b - sign*i*d   (i*d = (-di, dr))
            y0r[b] = ar_ + cr;
            y0i[b] = ai_ + ci;
            y2r[b] = ar_ - cr;
            y2i[b] = ai_ - ci;
            y1r[b] = br_ - s * di;
            y1i[b] = bi_ + s * dr;
            y3r[b] = br_ + s * di;
            y3i[b] = bi_ - s * dr;
          }
        } else if (R == 2) {
          const double w1r = tr[0], w1i = -s * ti[0];
          const double *x0r = ar + size_t(j) * B, *x0i = ai + size_t(j) * B;
          const double *x1r = ar + size_t(j + m) * B, *x1i = ai + size_t(j + m) * B;
          double *y0r = br + o * B, *y0i = bi + o * B;
          double *y1r = br + (o + ns) * B, *y1i = bi + (o + ns) * B;
#pragma omp simd
          for (int b = 0; b < B; ++b) {
            const double v1r = x1r[b] * w1r - x1i[b] * w1i, v1i = x1r[b] * w1i + x1i[b] * w1r;
            const double v0r = x0r[b], v0i = x0i[b];
            y0r[b] = v0r + v1r;
            y0i[b] = v0i + v1i;
            y1r[b] = v0r - v1r;
            y1i[b] = v0i - v1i;
          }
        } else {  // R == 3
          const double w1r = tr[0], w1i = -s * ti[0], w2r = tr[1], w2i = -s * ti[1];
          const double h = s * 0.86602540378443864676;  // sign * sin(2 pi / 3)
          const double *x0r = ar + size_t(j) * B, *x0i = ai + size_t(j) * B;
          const double *x1r = ar + size_t(j + m) * B, *x1i = ai + size_t(j + m) * B;
          const double *x2r = ar + size_t(j + 2 * m) * B, *x2i = ai + size_t(j + 2 * m) * B;
          double *y0r = br + o * B, *y0i = bi + o * B;
          double *y1r = br + (o + ns) * B, *y1i = bi + (o + ns) * B;
          double *y2r = br + (o + 2 * size_t(ns)) * B, *y2i = bi + (o + 2 * size_t(ns)) * B;
#pragma omp simd
          for (int b = 0; b < B; ++b) {
            const double v0r = x0r[b], v0i = x0i[b];
            const double v1r = x1r[b] * w1r - x1i[b] * w1i, v1i = x1r[b] * w1i + x1i[b] * w1r;
            const double v2r = x2r[b] * w2r - x2i[b] * w2i, v2i = x2r[b] * w2i + x2i[b] * w2r;
            const double sr = v1r + v2r, si = v1i + v2i, dr = v1r - v2r, di = v1i - v2i;
            const double tr_ = v0r - 0.5 * sr, ti_ = v0i - 0.5 * si;
            // X1 = t + sign*i*h*d, X2 = t - sign*i*h*d  with h = sin(2pi/3), i*d = (-di, dr)
            y0r[b] = v0r + sr;
            y0i[b] = v0i + si;
            y1r[b] = tr_ - h * di;
            y1i[b] = ti_ + h * dr;
            y2r[b] = tr_ + h * di;
            y2i[b] = ti_ - h * dr;
          }
        }
      }
      std::swap(ar, br);
      std::swap(ai, bi);
    }
    return ar == yr;
  }
};

// ---------------------------------------------------------------------------
// 3D real FFT in the Grid_FFT in-place layout: real rows of n+2 doubles,
// k-space kelem(i,j,k) = complex element (i*n + j)*(n/2+1) + k.
// ---------------------------------------------------------------------------
constexpr int kBatch = 16;

struct Fft3 {
  int n, h, nk;
  Fft1 full, half;
  std::vector<double> er, ei;  // exp(-2 pi i k / n), k = 0..h

  explicit Fft3(int len) : n(len), h(len / 2), nk(len / 2 + 1), full(len), half(len / 2) {
    er.resize(h + 1);
    ei.resize(h + 1);
    for (int k = 0; k <= h; ++k) {
      er[k] = std::cos(-2.0 * kPi * k / n);
      ei[k] = std::sin(-2.0 * kPi * k / n);
    }
  }

  // complex transforms along y (axis 1) or x (axis 0) for every (plane, kz) column
  void pass_c2c(double *a, int axis, int sign, double scale) const {
    const size_t nkz = size_t(nk);
    const size_t stride = axis == 1 ? nkz : size_t(n) * nkz;  // in complex elements
    const int nblk = (nk + kBatch - 1) / kBatch;
#pragma omp parallel
    {
      std::vector<double> buf(4 * size_t(n) * kBatch);
      double *xr = buf.data(), *xi = xr + size_t(n) * kBatch, *yr = xi + size_t(n) * kBatch,
             *yi = yr + size_t(n) * kBatch;
#pragma omp for schedule(static)
      for (long long t = 0; t < (long long)n * nblk; ++t) {
        const size_t other = size_t(t / nblk);
        const int k0 = int(t % nblk) * kBatch, B = std::min(kBatch, nk - k0);
        // base of column (other, ., k0): axis 1 -> plane i = other; axis 0 -> row j = other
        const size_t base = axis == 1 ? other * size_t(n) * nkz : other * nkz;
        for (int q = 0; q < n; ++q) {
          const double *src = a + 2 * (base + size_t(q) * stride + k0);
          for (int b = 0; b < B; ++b) {
            xr[size_t(q) * kBatch + b] = src[2 * b];
            xi[size_t(q) * kBatch + b] = src[2 * b + 1];
          }
          for (int b = B; b < kBatch; ++b) xr[size_t(q) * kBatch + b] = xi[size_t(q) * kBatch + b] = 0.0;
        }
        const bool in_y = full.run(xr, xi, yr, yi, kBatch, sign);
        const double *rr = in_y ? yr : xr, *ri = in_y ? yi : xi;
        for (int q = 0; q < n; ++q) {
          double *dst = a + 2 * (base + size_t(q) * stride + k0);
          for (int b = 0; b < B; ++b) {
            dst[2 * b] = rr[size_t(q) * kBatch + b] * scale;
            dst[2 * b + 1] = ri[size_t(q) * kBatch + b] * scale;
          }
        }
      }
    }
  }

  // real <-> half-complex along z for every (x, y) row
  void pass_z(double *a, bool forward, double scale) const {
    const size_t rows = size_t(n) * n, rlen = size_t(n) + 2;
    const long long nblk = (long long)((rows + kBatch - 1) / kBatch);
#pragma omp parallel
    {
      std::vector<double> buf(4 * size_t(h) * kBatch);
      double *xr = buf.data(), *xi = xr + size_t(h) * kBatch, *yr = xi + size_t(h) * kBatch,
             *yi = yr + size_t(h) * kBatch;
#pragma omp for schedule(static)
      for (long long blk = 0; blk < nblk; ++blk) {
        const size_t r0 = size_t(blk) * kBatch;
        const int B = int(std::min<size_t>(kBatch, rows - r0));
        if (forward) {
          for (int b = 0; b < B; ++b) {
            const double *row = a + (r0 + b) * rlen;
            for (int t = 0; t < h; ++t) {
              xr[size_t(t) * kBatch + b] = row[2 * t];
              xi[size_t(t) * kBatch + b] = row[2 * t + 1];
            }
          }
          for (int b = B; b < kBatch; ++b)
            for (int t = 0; t < h; ++t) xr[size_t(t) * kBatch + b] = xi[size_t(t) * kBatch + b] = 0.0;
          const bool in_y = half.run(xr, xi, yr, yi, kBatch, -1);
          const double *zr = in_y ? yr : xr, *zi = in_y ? yi : xi;
          for (int b = 0; b < B; ++b) {
            double *row = a + (r0 + b) * rlen;
            for (int k = 0; k <= h; ++k) {
              const int k1 = k % h, k2 = (h - k) % h;
              const double z1r = zr[size_t(k1) * kBatch + b], z1i = zi[size_t(k1) * kBatch + b];
              const double z2r = zr[size_t(k2) * kBatch + b], z2i = -zi[size_t(k2) * kBatch + b];
              // E = (Z_k + conj Z_{h-k})/2, O = (Z_k - conj Z_{h-k})/(2i), X_k = E + e^{-2 pi i k/n} O
              const double Er = 0.5 * (z1r + z2r), Ei = 0.5 * (z1i + z2i);
              const double Or = 0.5 * (z1i - z2i), Oi = -0.5 * (z1r - z2r);
              row[2 * k] = (Er + er[k] * Or - ei[k] * Oi) * scale;
              row[2 * k + 1] = (Ei + er[k] * Oi + ei[k] * Or) * scale;
            }
          }
        } else {
          for (int b = 0; b < B; ++b) {
            const double *row = a + (r0 + b) * rlen;
            for (int k = 0; k < h; ++k) {
              // the real transform takes only the real parts of the k = 0 and k = h entries
              double x1r = row[2 * k], x1i = (k == 0) ? 0.0 : row[2 * k + 1];
              double x2r = row[2 * (h - k)], x2i = (k == 0) ? 0.0 : -row[2 * (h - k) + 1];
              const double Er = 0.5 * (x1r + x2r), Ei = 0.5 * (x1i + x2i);
              const double Dr = 0.5 * (x1r - x2r), Di = 0.5 * (x1i - x2i);
              // O = D * e^{+2 pi i k/n};  Z = E + i O
              const double Or = Dr * er[k] + Di * ei[k], Oi = Di * er[k] - Dr * ei[k];
              xr[size_t(k) * kBatch + b] = Er - Oi;
              xi[size_t(k) * kBatch + b] = Ei + Or;
            }
          }
          for (int b = B; b < kBatch; ++b)
            for (int t = 0; t < h; ++t) xr[size_t(t) * kBatch + b] = xi[size_t(t) * kBatch + b] = 0.0;
          const bool in_y = half.run(xr, xi, yr, yi, kBatch, +1);
          const double *zr = in_y ? yr : xr, *zi = in_y ? yi : xi;
          for (int b = 0; b < B; ++b) {
            double *row = a + (r0 + b) * rlen;
            for (int t = 0; t < h; ++t) {
              row[2 * t] = 2.0 * zr[size_t(t) * kBatch + b] * scale;
              row[2 * t + 1] = 2.0 * zi[size_t(t) * kBatch + b] * scale;
            }
            row[n] = row[n + 1] = 0.0;
          }
        }
      }
    }
  }

  // Grid_FFT::FourierTransformForward + ApplyNorm (grid_fft.cc:199-238)
  void r2c(double *a) const {
    pass_z(a, true, 1.0);
    pass_c2c(a, 1, -1, 1.0);
    pass_c2c(a, 0, -1, 1.0 / std::sqrt(double(n) * n * n));
  }
  // Grid_FFT::FourierTransformBackward + ApplyNorm (grid_fft.cc:241-270)
  void c2r(double *a) const {
    pass_c2c(a, 0, +1, 1.0 / std::sqrt(double(n) * n * n));
    pass_c2c(a, 1, +1, 1.0);
    pass_z(a, false, 1.0);
  }
};

// ---------------------------------------------------------------------------
// Grids
// ---------------------------------------------------------------------------
struct Grid {
  int n = 0;
  size_t nk = 0;
  double *a = nullptr;
  explicit Grid(int len) : n(len), nk(size_t(len / 2 + 1)) {
    a = static_cast<double *>(std::malloc(sizeof(double) * size_t(n) * n * (n + 2)));
    if (!a) std::abort();
    zero();
  }
  ~Grid() { std::free(a); }
  Grid(const Grid &) = delete;
  Grid &operator=(const Grid &) = delete;
  size_t ncplx() const { return size_t(n) * n * nk; }
  cplx *k() { return reinterpret_cast<cplx *>(a); }
  const cplx *k() const { return reinterpret_cast<const cplx *>(a); }
  size_t idx(size_t i, size_t j, size_t kk) const { return (i * n + j) * nk + kk; }
  void zero() {
    const size_t tot = size_t(n) * n * (n + 2);
#pragma omp parallel for schedule(static)
    for (long long q = 0; q < (long long)tot; ++q) a[q] = 0.0;
  }
};

// Grid_FFT::get_k (grid_fft.hh:281-296) for a grid of length L
inline double kcomp(size_t i, int n, double kfac) { return (double(i) - double(i > size_t(n / 2)) * n) * kfac; }

// ---------------------------------------------------------------------------
// PLT gradient: lattice_gradient::gradient / vfac_corr (particle_plt.hh:551-585)
// with Grid_FFT::get_cic_kspace (grid_fft.hh:347-373) on the 64^3 tables
// ---------------------------------------------------------------------------
constexpr int kTab = 64, kTabK = 33;

struct PltGradient {
  const double *tab;  // 4 x 64 x 64 x 33: D_r, D_theta, D_phi, alpha^{-1}
  double mapratio, boxlen;
  PltGradient(const double *t, int n, double L) : tab(t), mapratio(double(kTab) / n), boxlen(L) {}

  double cic(int which, double x, double y, double z) const {
    const double *T = tab + size_t(which) * kTab * kTab * kTabK;
    const int ix = int(std::floor(x)), iy = int(std::floor(y)), iz = int(std::floor(z));
    const double dx = x - ix, tx = 1.0 - dx, dy = y - iy, ty = 1.0 - dy, dz = z - iz, tz = 1.0 - dz;
    const int ix1 = (ix + 1) % kTab, iy1 = (iy + 1) % kTab, iz1 = std::min(iz + 1, kTabK - 1);
    auto at = [&](int a, int b, int c) { return T[(size_t(a) * kTab + b) * kTabK + c]; };
    double v = 0.0;
    v += at(ix, iy, iz) * tx * ty * tz;
    v += at(ix, iy, iz1) * tx * ty * dz;
    v += at(ix, iy1, iz) * tx * dy * tz;
    v += at(ix, iy1, iz1) * tx * dy * dz;
    v += at(ix1, iy, iz) * dx * ty * tz;
    v += at(ix1, iy, iz1) * dx * ty * dz;
    v += at(ix1, iy1, iz) * dx * dy * tz;
    v += at(ix1, iy1, iz1) * dx * dy * dz;
    return v;
  }

  cplx gradient(int d, size_t i, size_t j, size_t k) const {
    const double x = i * mapratio, y = j * mapratio, z = k * mapratio;
    const double tp = 2.0 * kPi;
    const double kx = (x - double(x > 32.0) * 64.0) * tp, ky = (y - double(y > 32.0) * 64.0) * tp,
                 kz = (z - double(z > 32.0) * 64.0) * tp;
    const double kr = std::sqrt(kx * kx + ky * ky + kz * kz);
    const double kmod = kr / mapratio / boxlen;
    const double Dr = cic(0, x, y, z), Dt = cic(1, x, y, z), Dp = cic(2, x, y, z);
    const double kphi = kr > 0.0 ? std::atan2(ky, kx) : 0.0, kth = kr > 0.0 ? std::acos(kz / kr) : 0.0;
    const double st = std::sin(kth), ct = std::cos(kth), sp = std::sin(kphi), cp = std::cos(kphi);
    if (d == 0) return cplx(0.0, kmod * (Dr * st * cp + Dt * ct * cp - Dp * sp));
    if (d == 1) return cplx(0.0, kmod * (Dr * st * sp + Dt * ct * sp + Dp * cp));
    return cplx(0.0, kmod * (Dr * ct - Dt * st));
  }

  double vfac_corr(size_t i, size_t j, size_t k) const {
    const double alpha = 1.0 / cic(3, i * mapratio, j * mapratio, k * mapratio);
    return 1.0 / alpha;
  }
};

// op::fourier_gradient (operators.hh:38-61) with the Nyquist index zeroed as in
// Grid_FFT::gradient (grid_fft.hh:376-385)
struct FourierGradient {
  int n;
  double kfac;
  cplx gradient(int d, size_t i, size_t j, size_t k) const {
    const size_t q = d == 0 ? i : d == 1 ? j : k;
    if (q == size_t(n / 2)) return cplx(0.0, 0.0);
    return cplx(0.0, kcomp(q, n, kfac));
  }
  double vfac_corr(size_t, size_t, size_t) const { return 1.0; }
};

// ---------------------------------------------------------------------------
// Orszag 3/2 convolver (convolution.hh:412-652), non-distributed branch
// ---------------------------------------------------------------------------
struct Orszag {
  int n, m;
  double kfac;
  const Fft3 &fm;
  Grid f1, f2, fbuf;
  Orszag(int len, double L, const Fft3 &fft_m) : n(len), m(3 * len / 2), kfac(2 * kPi / L), fm(fft_m), f1(m), f2(m), fbuf(len) {}

  // Grid_FFT::gradient of the N-grid (grid_fft.hh:376-385)
  cplx grad(int d, size_t i, size_t j, size_t k) const {
    const size_t q = d == 0 ? i : d == 1 ? j : k;
    return cplx(0.0, q == size_t(n / 2) ? 0.0 : kcomp(q, n, kfac));
  }

  template <class F>
  void pad_insert(F kfunc, Grid &fp) {
    const double rfac = std::pow(1.5, 1.5);
    const size_t nh = size_t(m / 3);
    fp.zero();
    cplx *dst = fp.k();
#pragma omp parallel for schedule(static)
    for (long long ii = 0; ii < 2LL * m / 3; ++ii) {
      const size_t i = size_t(ii), ip = i > nh ? i + nh : i;
      for (size_t j = 0; j < size_t(2 * m / 3); ++j) {
        const size_t jp = j > nh ? j + nh : j;
        for (size_t k = 0; k < nh + 1; ++k) dst[fp.idx(ip, jp, k)] = kfunc(i, j, k) * rfac;
      }
    }
  }

  template <class Op>
  void unpad(Grid &fp, Op output_op) {
    const double rfac = std::sqrt(double(m) * m * m) / std::sqrt(double(n) * n * n);
    const size_t nh = size_t(n / 2);
    const cplx *src = fp.k();
    cplx *dst = fbuf.k();
#pragma omp parallel for schedule(static)
    for (long long ii = 0; ii < n; ++ii) {
      const size_t i = size_t(ii), ip = i > nh ? i + nh : i;
      for (size_t j = 0; j < size_t(n); ++j) {
        const size_t jp = j > nh ? j + nh : j;
        for (size_t k = 0; k < fbuf.nk; ++k) {
          dst[fbuf.idx(i, j, k)] = src[fp.idx(ip, jp, k)] / rfac;
          if (i == nh || j == nh || k == nh) dst[fbuf.idx(i, j, k)] = 0.0;
        }
      }
    }
    const long long tot = (long long)fbuf.ncplx();
#pragma omp parallel for schedule(static)
    for (long long q = 0; q < tot; ++q) output_op(size_t(q), dst[q]);
  }

  template <class F1, class F2, class Op>
  void convolve2(F1 kf1, F2 kf2, Op output_op) {
    pad_insert(kf1, f1);
    pad_insert(kf2, f2);
    fm.c2r(f1.a);
    fm.c2r(f2.a);
    const long long tot = (long long)m * m * (m + 2);
    double *a1 = f1.a, *a2 = f2.a;
#pragma omp parallel for schedule(static)
    for (long long q = 0; q < tot; ++q) a2[q] *= a1[q];
    fm.r2c(f2.a);
    unpad(f2, output_op);
  }

  template <class F1, class F2, class F3, class Op>
  void convolve3(F1 kf1, F2 kf2, F3 kf3, Op output_op) {
    convolve2(kf1, kf2, [](size_t, cplx) {});  // unpad leaves the product in fbuf
    const cplx *fb = fbuf.k();
    const size_t nk = fbuf.nk;
    const int nn = n;
    convolve2([fb, nk, nn](size_t i, size_t j, size_t k) { return fb[(i * nn + j) * nk + k]; }, kf3, output_op);
  }

  // kfunc builders (convolution.hh:74-275)
  auto hessian(const Grid &g, int a, int b) const {
    const cplx *p = g.k();
    const size_t nk = g.nk;
    const int nn = n;
    return [this, p, nk, nn, a, b](size_t i, size_t j, size_t k) {
      return grad(a, i, j, k) * grad(b, i, j, k) * p[(i * nn + j) * nk + k];
    };
  }
  auto sum_of_hessians(const Grid &g, int a1, int b1, int a2, int b2) const {
    const cplx *p = g.k();
    const size_t nk = g.nk;
    const int nn = n;
    return [this, p, nk, nn, a1, b1, a2, b2](size_t i, size_t j, size_t k) {
      return (grad(a1, i, j, k) * grad(b1, i, j, k) + grad(a2, i, j, k) * grad(b2, i, j, k)) *
             p[(i * nn + j) * nk + k];
    };
  }
  auto difference_of_hessians(const Grid &g, int a1, int b1, int a2, int b2) const {
    const cplx *p = g.k();
    const size_t nk = g.nk;
    const int nn = n;
    return [this, p, nk, nn, a1, b1, a2, b2](size_t i, size_t j, size_t k) {
      return (grad(a1, i, j, k) * grad(b1, i, j, k) - grad(a2, i, j, k) * grad(b2, i, j, k)) *
             p[(i * nn + j) * nk + k];
    };
  }
};

// output operators (operators.hh:26-35)
auto assign_to(Grid &g) {
  cplx *p = g.k();
  return [p](size_t i, cplx v) { p[i] = v; };
}
auto add_to(Grid &g) {
  cplx *p = g.k();
  return [p](size_t i, cplx v) { p[i] += v; };
}
auto subtract_from(Grid &g) {
  cplx *p = g.k();
  return [p](size_t i, cplx v) { p[i] -= v; };
}
auto multiply_add_to(Grid &g, double f) {
  cplx *p = g.k();
  return [p, f](size_t i, cplx v) { p[i] += f * v; };
}

// Grid_FFT::apply_InverseLaplacian + zero_DC_mode (grid_fft.hh:440-449, 844-850)
void inverse_laplacian(Grid &g, double kfac) {
  const int n = g.n;
  cplx *p = g.k();
#pragma omp parallel for schedule(static)
  for (long long ii = 0; ii < n; ++ii)
    for (size_t j = 0; j < size_t(n); ++j)
      for (size_t k = 0; k < g.nk; ++k) {
        const double kx = kcomp(size_t(ii), n, kfac), ky = kcomp(j, n, kfac), kz = kcomp(k, n, kfac);
        const double k2 = kx * kx + ky * ky + kz * kz;
        p[g.idx(size_t(ii), j, k)] *= -1.0 / k2;
      }
  p[0] = 0.0;
}

void scale(Grid &g, double f) {
  cplx *p = g.k();
  const long long tot = (long long)g.ncplx();
#pragma omp parallel for schedule(static)
  for (long long q = 0; q < tot; ++q) p[q] *= f;
}

const double kShifts[3][4][3] = {
    {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}},
    {{0, 0, 0}, {0.5, 0.5, 0.5}, {0, 0, 0}, {0, 0, 0}},
    {{0, 0, 0}, {0, 0.5, 0.5}, {0.5, 0, 0.5}, {0.5, 0.5, 0}},
};  // particle_generator.hh:47-54

// Grid_FFT::shift_field (grid_fft.hh:832-842)
void shift_field(Grid &g, const Fft3 &fn, const double s[3], double L) {
  fn.r2c(g.a);
  const int n = g.n;
  const double kfac = 2 * kPi / L, dx = L / n;
  cplx *p = g.k();
#pragma omp parallel for schedule(static)
  for (long long ii = 0; ii < n; ++ii)
    for (size_t j = 0; j < size_t(n); ++j)
      for (size_t k = 0; k < g.nk; ++k) {
        const double sh = s[0] * kcomp(size_t(ii), n, kfac) * dx + s[1] * kcomp(j, n, kfac) * dx +
                          s[2] * kcomp(k, n, kfac) * dx;
        p[g.idx(size_t(ii), j, k)] *= std::exp(cplx(0.0, sh));
      }
  fn.c2r(g.a);
}

struct Job {
  int n, order, lattice;
  double L, lunit, vunit;
  double g1, g2, g3, g3c, vfac1, vfac2, vfac3;
};

template <class Grad>
void assemble_and_read_out(const Job &J, const Grad &lg, Grid &phi, Grid *phi2, Grid *phi3, Grid **A3, Grid &tmp,
                           const Fft3 &fn, double *pos, double *vel) {
  const int n = J.n, ns = 1 << J.lattice;
  const size_t n3 = size_t(n) * n * n;
  for (int pass = 0; pass < 2; ++pass) {  // 0: positions, 1: velocities
    for (int idim = 0; idim < 3; ++idim) {
      const int idimp = (idim + 1) % 3, idimpp = (idim + 2) % 3;
      cplx *t = tmp.k();
      const cplx *p1 = phi.k(), *p2 = phi2 ? phi2->k() : nullptr, *p3 = phi3 ? phi3->k() : nullptr;
      const cplx *ap = J.order > 2 ? A3[idimp]->k() : nullptr, *app = J.order > 2 ? A3[idimpp]->k() : nullptr;
      const double unit = (pass == 0 ? J.lunit : J.vunit) / J.L;
#pragma omp parallel for schedule(static)
      for (long long ii = 0; ii < n; ++ii) {
        const size_t i = size_t(ii);
        for (size_t j = 0; j < size_t(n); ++j)
          for (size_t k = 0; k < tmp.nk; ++k) {
            const size_t q = tmp.idx(i, j, k);
            if (pass == 0) {  // ic_generator.cc:939-965
              cplx phitot = p1[q];
              if (J.order > 1) phitot += p2[q];
              if (J.order > 2) phitot += p3[q];
              cplx v = lg.gradient(idim, i, j, k) * phitot;
              if (J.order > 2) v += lg.gradient(idimp, i, j, k) * app[q] - lg.gradient(idimpp, i, j, k) * ap[q];
              t[q] = v * unit;
            } else {  // ic_generator.cc:994-1053
              cplx pv = J.vfac1 * p1[q];
              if (J.order > 1) pv += J.vfac2 * p2[q];
              if (J.order > 2) pv += J.vfac3 * p3[q];
              cplx v = lg.gradient(idim, i, j, k) * pv;
              if (J.order > 2)
                v += J.vfac3 * (lg.gradient(idimp, i, j, k) * app[q] - lg.gradient(idimpp, i, j, k) * ap[q]);
              v *= lg.vfac_corr(i, j, k);
              t[q] = v * unit;
            }
          }
      }
      t[0] = 0.0;  // zero_DC_mode
      fn.c2r(tmp.a);
      // set_positions / set_velocities (particle_generator.hh:499-543, 597-639): serial read-out
      for (int ish = 0; ish < ns; ++ish) {
        if (ish > 0) {
          const double d[3] = {kShifts[J.lattice][ish][0] - kShifts[J.lattice][ish - 1][0],
                               kShifts[J.lattice][ish][1] - kShifts[J.lattice][ish - 1][1],
                               kShifts[J.lattice][ish][2] - kShifts[J.lattice][ish - 1][2]};
          shift_field(tmp, fn, d, J.L);
        }
        const double sh = kShifts[J.lattice][ish][idim];
        size_t ip = size_t(ish) * n3;
        for (size_t i = 0; i < size_t(n); ++i)
          for (size_t j = 0; j < size_t(n); ++j) {
            const double *row = tmp.a + (i * n + j) * size_t(n + 2);
            for (size_t k = 0; k < size_t(n); ++k, ++ip) {
              if (pass == 0) {
                const size_t c = idim == 0 ? i : idim == 1 ? j : k;
                pos[3 * ip + idim] = ((double(c) + sh) / double(n)) * J.lunit + row[k];
              } else {
                vel[3 * ip + idim] = row[k];
              }
            }
          }
      }
    }
  }
}

}  // namespace

extern "C" {

/* Batched 1D transform check hook: `count` transforms of length `len`
   (interleaved complex, contiguous per transform), in place; sign -1 forward,
   +1 backward (unnormalised). */
int mfxo_omp_fft1(int len, int count, int sign, double *data) {
  Fft1 f(len);
  std::vector<double> buf(4 * size_t(len) * kBatch);
  double *xr = buf.data(), *xi = xr + size_t(len) * kBatch, *yr = xi + size_t(len) * kBatch,
         *yi = yr + size_t(len) * kBatch;
  for (int c0 = 0; c0 < count; c0 += kBatch) {
    const int B = std::min(kBatch, count - c0);
    for (int b = 0; b < kBatch; ++b)
      for (int t = 0; t < len; ++t) {
        xr[size_t(t) * kBatch + b] = b < B ? data[2 * (size_t(c0 + b) * len + t)] : 0.0;
        xi[size_t(t) * kBatch + b] = b < B ? data[2 * (size_t(c0 + b) * len + t) + 1] : 0.0;
      }
    const bool in_y = f.run(xr, xi, yr, yi, kBatch, sign);
    const double *rr = in_y ? yr : xr, *ri = in_y ? yi : xi;
    for (int b = 0; b < B; ++b)
      for (int t = 0; t < len; ++t) {
        data[2 * (size_t(c0 + b) * len + t)] = rr[size_t(t) * kBatch + b];
        data[2 * (size_t(c0 + b) * len + t) + 1] = ri[size_t(t) * kBatch + b];
      }
  }
  return 0;
}

/* 3D unitary transform in the Grid_FFT in-place layout: forward (r2c) when
   forward != 0, else backward (c2r).  `a` holds n*n*(n+2) doubles. */
int mfxo_omp_fft3(int n, int forward, double *a) {
  Fft3 f(n);
  if (forward)
    f.r2c(a);
  else
    f.c2r(a);
  return 0;
}

int mfxo_omp_threads(void) { return omp_get_max_threads(); }

/* The whole hot path for one species.  amp_table[q] = A(|k|^2 = kf^2 q), the
   amplitude / k^2 of ic_generator.cc:509-516; coef = g1, g2, g3, g3c, vfac1,
   vfac2, vfac3 (ic_generator.cc:252-269); plt_table = 4 x 64 x 64 x 33 PLT
   tables or NULL.  pos / vel: 3 * n_s * n^3 doubles (interleaved xyz), ids:
   n_s * n^3.  fields (optional): phi, phi2, phi3, A3x, A3y, A3z after growth
   scaling, n*n*(n/2+1) complex each (only the computed ones are written).
   times (optional, 6 entries): noise, phi1, phi2, phi3 (3a + 3b), A3,
   assembly + particles, in seconds. */
int mfxo_omp_lpt(int n, double L, int order, int lattice, int fixing, int inversion, const uint32_t *seed_table,
                 const double *amp_table, size_t amp_len, const double *plt_table, const double *coef, double lunit,
                 double vunit, double *pos, double *vel, uint64_t *ids, double *fields, double *times) {
  if (n < 8 || n % 4 != 0 || order < 1 || order > 3 || lattice < 0 || lattice > 2) return -1;
  Job J{n, order, lattice, L, lunit, vunit, coef[0], coef[1], coef[2], coef[3], coef[4], coef[5], coef[6]};
  const double kfac = 2 * kPi / L;
  double tm[6] = {0, 0, 0, 0, 0, 0};
  Fft3 fn(n), fm(3 * n / 2);
  Grid phi(n);
  // ---- white noise (RNG_ngenic::Fill_Grid, serial) ----
  double t0 = now_s();
  mfxo_ngenic_fill(size_t(n), seed_table, phi.a, nullptr);
  // normalise / fix / invert (ic_generator.cc:378-383; volfac ic_generator.cc:247)
  {
    const double volfac = std::pow(L / n / 2.0 / kPi, 1.5);
    const double sgn = inversion ? -1.0 : 1.0;
    cplx *w = phi.k();
    const long long tot = (long long)phi.ncplx();
#pragma omp parallel for schedule(static)
    for (long long q = 0; q < tot; ++q) {
      cplx v = w[q];
      if (fixing && std::abs(v) != 0.0) v /= std::abs(v);
      w[q] = sgn * v / volfac;
    }
  }
  tm[0] = now_s() - t0;
  // ---- phi1 = -A(k) w (ic_generator.cc:509-516) ----
  t0 = now_s();
  {
    cplx *w = phi.k();
#pragma omp parallel for schedule(static)
    for (long long ii = 0; ii < n; ++ii)
      for (size_t j = 0; j < size_t(n); ++j)
        for (size_t k = 0; k < phi.nk; ++k) {
          const long long si = ii > n / 2 ? ii - n : ii, sj = (long long)j > n / 2 ? (long long)j - n : (long long)j;
          const size_t nn2 = size_t(si * si + sj * sj) + k * k;
          const double A = nn2 < amp_len ? amp_table[nn2] : 0.0;
          w[phi.idx(size_t(ii), j, k)] *= -A;
        }
    w[0] = 0.0;
  }
  tm[1] = now_s() - t0;
  Orszag C(n, L, fm);
  Grid *phi2 = nullptr, *phi3 = nullptr, *A3[3] = {nullptr, nullptr, nullptr};
  if (order > 1) {  // ic_generator.cc:525-548
    t0 = now_s();
    phi2 = new Grid(n);
    C.convolve2(C.hessian(phi, 0, 0), C.sum_of_hessians(phi, 1, 1, 2, 2), assign_to(*phi2));
    C.convolve2(C.hessian(phi, 1, 1), C.hessian(phi, 2, 2), add_to(*phi2));
    C.convolve2(C.hessian(phi, 0, 1), C.hessian(phi, 0, 1), subtract_from(*phi2));
    C.convolve2(C.hessian(phi, 0, 2), C.hessian(phi, 0, 2), subtract_from(*phi2));
    C.convolve2(C.hessian(phi, 1, 2), C.hessian(phi, 1, 2), subtract_from(*phi2));
    inverse_laplacian(*phi2, kfac);
    tm[2] = now_s() - t0;
  }
  if (order > 2) {  // ic_generator.cc:577-628
    t0 = now_s();
    phi3 = new Grid(n);
    C.convolve3(C.hessian(phi, 0, 0), C.hessian(phi, 1, 1), C.hessian(phi, 2, 2), assign_to(*phi3));
    C.convolve3(C.hessian(phi, 0, 1), C.hessian(phi, 0, 2), C.hessian(phi, 1, 2), multiply_add_to(*phi3, 2.0));
    C.convolve3(C.hessian(phi, 1, 2), C.hessian(phi, 1, 2), C.hessian(phi, 0, 0), subtract_from(*phi3));
    C.convolve3(C.hessian(phi, 0, 2), C.hessian(phi, 0, 2), C.hessian(phi, 1, 1), subtract_from(*phi3));
    C.convolve3(C.hessian(phi, 0, 1), C.hessian(phi, 0, 1), C.hessian(phi, 2, 2), subtract_from(*phi3));
    const double c57 = -5.0 / 7.0, c107 = 10.0 / 7.0;
    C.convolve2(C.hessian(phi, 0, 0), C.sum_of_hessians(*phi2, 1, 1, 2, 2), multiply_add_to(*phi3, c57));
    C.convolve2(C.hessian(phi, 1, 1), C.sum_of_hessians(*phi2, 2, 2, 0, 0), multiply_add_to(*phi3, c57));
    C.convolve2(C.hessian(phi, 2, 2), C.sum_of_hessians(*phi2, 0, 0, 1, 1), multiply_add_to(*phi3, c57));
    C.convolve2(C.hessian(phi, 0, 1), C.hessian(*phi2, 0, 1), multiply_add_to(*phi3, c107));
    C.convolve2(C.hessian(phi, 0, 2), C.hessian(*phi2, 0, 2), multiply_add_to(*phi3, c107));
    C.convolve2(C.hessian(phi, 1, 2), C.hessian(*phi2, 1, 2), multiply_add_to(*phi3, c107));
    inverse_laplacian(*phi3, kfac);
    tm[3] = now_s() - t0;
    t0 = now_s();
    for (int d = 0; d < 3; ++d) {
      const int dp = (d + 1) % 3, dpp = (d + 2) % 3;
      A3[d] = new Grid(n);
      C.convolve2(C.hessian(*phi2, d, dp), C.hessian(phi, d, dpp), assign_to(*A3[d]));
      C.convolve2(C.hessian(*phi2, d, dpp), C.hessian(phi, d, dp), subtract_from(*A3[d]));
      C.convolve2(C.hessian(phi, dp, dpp), C.difference_of_hessians(*phi2, dp, dp, dpp, dpp), add_to(*A3[d]));
      C.convolve2(C.hessian(*phi2, dp, dpp), C.difference_of_hessians(phi, dp, dp, dpp, dpp), subtract_from(*A3[d]));
      inverse_laplacian(*A3[d], kfac);
    }
    tm[4] = now_s() - t0;
  }
  // growth scaling (ic_generator.cc:645-658)
  t0 = now_s();
  scale(phi, J.g1);
  if (phi2) scale(*phi2, J.g2);
  if (phi3) {
    scale(*phi3, J.g3);
    for (int d = 0; d < 3; ++d) scale(*A3[d], J.g3c);
  }
  if (fields) {
    const size_t nc = phi.ncplx();
    Grid *out[6] = {&phi, phi2, phi3, A3[0], A3[1], A3[2]};
    for (int f = 0; f < 6; ++f)
      if (out[f]) std::memcpy(fields + 2 * nc * f, out[f]->a, sizeof(cplx) * nc);
  }
  // displacement / velocity assembly and particles (ic_generator.cc:929-1060)
  Grid &tmp = C.fbuf;  // the reference's tmp is another N-grid; the convolver's buffer is free now
  if (plt_table) {
    PltGradient lg(plt_table, n, L);
    assemble_and_read_out(J, lg, phi, phi2, phi3, A3, tmp, fn, pos, vel);
  } else {
    FourierGradient lg{n, kfac};
    assemble_and_read_out(J, lg, phi, phi2, phi3, A3, tmp, fn, pos, vel);
  }
  // particle ids (particle_generator.hh:212-253)
  {
    const size_t n3 = size_t(n) * n * n, ns = size_t(1) << lattice;
#pragma omp parallel for schedule(static)
    for (long long c = 0; c < (long long)n3; ++c)
      for (size_t il = 0; il < ns; ++il) ids[il * n3 + size_t(c)] = ns * size_t(c) + il;
  }
  tm[5] = now_s() - t0;
  delete phi2;
  delete phi3;
  for (auto *a : A3) delete a;
  if (times)
    for (int q = 0; q < 6; ++q) times[q] = tm[q];
  return 0;
}

}  // extern "C"
