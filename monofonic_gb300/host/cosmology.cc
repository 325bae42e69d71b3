// Host-side cosmology of the IC engine.  See cosmology.h for the reference
// interfaces each piece mirrors.
#include "cosmology.h"

#include <cmath>
#include <queue>
#include <stdexcept>

namespace mfx {

// ---------------------------------------------------------------------------
// parameters (cosmology_parameters.hh:80-241; defaults are the reference's
// "Planck2018EE+BAO+SN" set, cosmology_parameters.cc:110-132)
// ---------------------------------------------------------------------------
static const std::map<std::string, double> &planck18_bao_sn() {
  static const std::map<std::string, double> p = {
      {"h", 0.67742},        {"Omega_m", 0.3099},  {"Omega_b", 0.048891054}, {"Omega_DE", 0.6901},
      {"Omega_k", 0.0},      {"w_0", -1.0},        {"w_a", 0.0},             {"n_s", 0.96822},
      {"A_s", 2.1064e-9},    {"alpha_s", 0.0},     {"beta_s", 0.0},          {"k_p", 0.05},
      {"YHe", 0.245421},     {"N_ur", 2.046},      {"m_nu1", 0.06},          {"m_nu2", 0.0},
      {"m_nu3", 0.0},        {"deg_nu1", 1.0},     {"deg_nu2", 1.0},         {"deg_nu3", 1.0},
      {"Tcmb", 2.7255},      {"O_nu_norm", 93.13861}};
  return p;
}

cosmo_parameters::cosmo_parameters(const config_file &cf) {
  const std::string pset = cf.get_value_safe<std::string>("cosmology", "ParameterSet", "none");
  const auto &dp = planck18_bao_sn();
  auto D = [&](const char *k) { return dp.at(k); };
  if (pset == "none") {
    pmap_["Tcmb"] = cf.get_value_safe<double>("cosmology", "Tcmb", D("Tcmb"));
    pmap_["YHe"] = cf.get_value_safe<double>("cosmology", "YHe", D("YHe"));
    pmap_["h"] = cf.get_value_safe<double>("cosmology", "H0", D("h") * 100.0) / 100.0;
    if (!cf.contains_key("cosmology/n_s"))
      pmap_["n_s"] = cf.get_value_safe<double>("cosmology", "nspec", D("n_s"));
    else
      pmap_["n_s"] = cf.get_value_safe<double>("cosmology", "n_s", D("n_s"));
    pmap_["A_s"] = cf.get_value_safe<double>("cosmology", "A_s",
                                             cf.contains_key("cosmology/sigma_8") ? -1.0 : D("A_s"));
    pmap_["k_p"] = cf.get_value_safe<double>("cosmology", "k_p", D("k_p"));
    pmap_["sigma_8"] = cf.get_value_safe<double>("cosmology", "sigma_8", -1.0);
    pmap_["alpha_s"] = cf.get_value_safe<double>("cosmology", "alpha_s", D("alpha_s"));
    pmap_["beta_s"] = cf.get_value_safe<double>("cosmology", "beta_s", D("beta_s"));
    pmap_["Omega_b"] = cf.get_value_safe<double>("cosmology", "Omega_b", D("Omega_b"));
    pmap_["Omega_m"] = cf.get_value_safe<double>("cosmology", "Omega_m", D("Omega_m"));
    pmap_["m_nu1"] = cf.get_value_safe<double>("cosmology", "m_nu1", D("m_nu1"));
    pmap_["m_nu2"] = cf.get_value_safe<double>("cosmology", "m_nu2", D("m_nu2"));
    pmap_["m_nu3"] = cf.get_value_safe<double>("cosmology", "m_nu3", D("m_nu3"));
    pmap_["deg_nu1"] = cf.get_value_safe<double>("cosmology", "deg_nu1", D("deg_nu1"));
    pmap_["deg_nu2"] = cf.get_value_safe<double>("cosmology", "deg_nu2", D("deg_nu1"));
    pmap_["deg_nu3"] = cf.get_value_safe<double>("cosmology", "deg_nu3", D("deg_nu1"));
    const int n_massive = int(get("m_nu1") > 1e-9) + int(get("m_nu2") > 1e-9) + int(get("m_nu3") > 1e-9);
    pmap_["O_nu_norm"] = cf.get_value_safe<double>("cosmology", "O_nu_norm", D("O_nu_norm"));
    pmap_["N_ur"] = cf.get_value_safe<double>("cosmology", "N_ur", 3.046 - n_massive);
    pmap_["w_0"] = cf.get_value_safe<double>("cosmology", "w_0", D("w_0"));
    pmap_["w_a"] = cf.get_value_safe<double>("cosmology", "w_a", D("w_a"));
    pmap_["Omega_k"] = cf.get_value_safe<double>("cosmology", "Omega_k", D("Omega_k"));
  } else if (pset == "Planck2018EE+BAO+SN") {
    for (const auto &e : dp) pmap_[e.first] = e.second;
  } else {
    throw std::runtime_error("Unsupported cosmology/ParameterSet '" + pset +
                             "' (supported: none, Planck2018EE+BAO+SN)");
  }
  const double h = get("h");
  pmap_["H0"] = 100.0 * h;
  pmap_["N_nu_massive"] = int(get("m_nu1") > 1e-9) + int(get("m_nu2") > 1e-9) + int(get("m_nu3") > 1e-9);
  const double sum_m_nu = get("m_nu1") * get("deg_nu1") + get("m_nu2") * get("deg_nu2") + get("m_nu3") * get("deg_nu3");
  pmap_["Omega_nu_massive"] = sum_m_nu / (pmap_["O_nu_norm"] * h * h);
  pmap_["Omega_gamma"] = 4 * phys_const::sigma_SI / std::pow(phys_const::c_SI, 3) * std::pow(get("Tcmb"), 4.0) /
                         phys_const::rhocrit_h2_SI / (get("h") * get("h"));
  pmap_["Omega_nu_massless"] = get("N_ur") * get("Omega_gamma") * 7. / 8. * std::pow(4. / 11., 4. / 3.);
  pmap_["Omega_r"] = get("Omega_gamma") + get("Omega_nu_massless");
  pmap_["Omega_c"] = get("Omega_m") - get("Omega_b") - get("Omega_nu_massive");
  if (cf.get_value_safe<bool>("cosmology", "ZeroRadiation", false)) pmap_["Omega_r"] = 0.0;
  pmap_["f_b"] = get("Omega_b") / get("Omega_m");
  pmap_["f_c"] = 1.0 - get("f_b");
  pmap_["Omega_DE"] = 1.0 - get("Omega_m") - get("Omega_r") - get("Omega_k");
  for (const char *k : {"dplus", "pnorm", "sqrtpnorm", "vfact", "dplus_start", "dplus_target"}) pmap_[k] = 0.0;
}

double cosmo_parameters::get(const std::string &k) const {
  auto it = pmap_.find(k);
  if (it == pmap_.end()) throw std::runtime_error("unknown cosmological parameter '" + k + "'");
  return it->second;
}

// compute_running_factor, cosmology_parameters.cc:153-168
static double running_factor(const cosmo_parameters &cp, double k) {
  const double alpha_s = cp.get("alpha_s"), beta_s = cp.get("beta_s");
  if (alpha_s == 0.0 && beta_s == 0.0) return 1.0;
  const double k_p = cp.get("k_p");
  const double lnk = std::log(k / k_p);
  const double running = 0.5 * (alpha_s * lnk + beta_s * lnk * lnk / 3.0);
  return std::pow(k / k_p, 0.5 * running);
}

double TransferFunction_plugin::get_vfac_asymptotic() const {
  throw std::runtime_error("Transfer function does not have asymptotic growth factors.");
}

// ---------------------------------------------------------------------------
// Eisenstein & Hu (1998, ApJ 496, 605) baryon+CDM fitting formula, as used by
// transfer_eisenstein.cc:58-243 (units Mpc inside, h/Mpc at the interface)
// ---------------------------------------------------------------------------
namespace {
struct EisensteinHu {
  double h0, omhh, obhh, theta, z_eq, k_eq, z_d, R_d, R_eq, s, k_silk;
  double a_c, b_c, a_b, b_b, b_node, fb, fc;

  void setup(double H0, double Om, double Ob, double Tcmb) {
    h0 = H0 * 0.01;
    omhh = Om * H0 * H0 * (0.01 * 0.01);
    const double f_baryon = Ob / Om;
    if (f_baryon <= 0.0 || omhh <= 0.0) throw std::runtime_error("Eisenstein&Hu: illegal input");
    obhh = omhh * f_baryon;
    if (Tcmb <= 0.0) Tcmb = 2.728;
    theta = Tcmb / 2.7;
    const double t2 = theta * theta, t4 = t2 * t2;
    z_eq = 2.50e4 * omhh / t4;
    k_eq = 0.0746 * omhh / t2;
    const double b1 = 0.313 * std::pow(omhh, -0.419) * (1 + 0.607 * std::pow(omhh, 0.674));
    const double b2 = 0.238 * std::pow(omhh, 0.223);
    z_d = 1291 * std::pow(omhh, 0.251) / (1 + 0.659 * std::pow(omhh, 0.828)) * (1 + b1 * std::pow(obhh, b2));
    R_d = 31.5 * obhh / t4 * (1000 / (1 + z_d));
    R_eq = 31.5 * obhh / t4 * (1000 / z_eq);
    s = 2. / 3. / k_eq * std::sqrt(6. / R_eq) *
        std::log((std::sqrt(1 + R_d) + std::sqrt(R_d + R_eq)) / (1 + std::sqrt(R_eq)));
    k_silk = 1.6 * std::pow(obhh, 0.52) * std::pow(omhh, 0.73) * (1 + std::pow(10.4 * omhh, -0.95));
    const double a1 = std::pow(46.9 * omhh, 0.670) * (1 + std::pow(32.1 * omhh, -0.532));
    const double a2 = std::pow(12.0 * omhh, 0.424) * (1 + std::pow(45.0 * omhh, -0.582));
    a_c = std::pow(a1, -f_baryon) * std::pow(a2, -(f_baryon * f_baryon * f_baryon));
    const double bb1 = 0.944 / (1 + std::pow(458 * omhh, -0.708));
    const double bb2 = std::pow(0.395 * omhh, -0.0266);
    b_c = 1.0 / (1 + bb1 * (std::pow(1 - f_baryon, bb2) - 1));
    const double y = z_eq / (1 + z_d);
    const double G = y * (-6. * std::sqrt(1 + y) + (2. + 3. * y) * std::log((std::sqrt(1 + y) + 1) / (std::sqrt(1 + y) - 1)));
    a_b = 2.07 * k_eq * s * std::pow(1 + R_d, -0.75) * G;
    b_node = 8.41 * std::pow(omhh, 0.435);
    b_b = 0.5 + f_baryon + (3. - 2. * f_baryon) * std::sqrt(std::pow(17.2 * omhh, 2.0) + 1);
    fb = Ob / Om;
    fc = (Om - Ob) / Om;
  }

  // baryon and CDM parts for k in 1/Mpc
  void parts(double k, double &Tb, double &Tc) const {
    k = std::fabs(k);
    if (k == 0.0) {
      Tb = Tc = 1.0;
      return;
    }
    const double q = k / 13.41 / k_eq;
    const double xx = k * s;
    const double ln_beta = std::log(2.718282 + 1.8 * b_c * q);
    const double ln_nobeta = std::log(2.718282 + 1.8 * q);
    const double C_alpha = 14.2 / a_c + 386.0 / (1 + 69.9 * std::pow(q, 1.08));
    const double C_noalpha = 14.2 + 386.0 / (1 + 69.9 * std::pow(q, 1.08));
    const double xr = xx / 5.4;
    const double f = 1.0 / (1.0 + (xr * xr) * (xr * xr));
    Tc = f * ln_beta / (ln_beta + C_noalpha * (q * q)) + (1 - f) * ln_beta / (ln_beta + C_alpha * (q * q));
    const double bn = b_node / xx;
    const double s_tilde = s * std::pow(1. + bn * bn * bn, -1. / 3.);
    const double xt = k * s_tilde;
    const double T0 = ln_nobeta / (ln_nobeta + C_noalpha * (q * q));
    const double x52 = xx / 5.2, bbx = b_b / xx;
    Tb = std::sin(xt) / xt * (T0 / (1. + x52 * x52) + a_b / (1. + bbx * bbx * bbx) * std::exp(-std::pow(k / k_silk, 1.4)));
  }

  double at_k(double k_hmpc) const {
    double tb, tc;
    parts(k_hmpc * h0, tb, tc);
    return fb * tb + fc * tc;
  }
};

class transfer_eisenstein_plugin : public TransferFunction_plugin {
 public:
  transfer_eisenstein_plugin(const config_file &cf, const cosmo_parameters &cp) : TransferFunction_plugin(cf, cp) {
    eh_.setup(cp.get("H0"), cp.get("Omega_m"), cp.get("Omega_b"), cp.get("Tcmb"));
  }
  double compute(double k, tf_type type) const override {
    if (type == theta_bc || type == delta_bc) return 0.0;
    return eh_.at_k(k) * running_factor(cosmo_params_, k);
  }
  double get_kmin() const override { return 1e-4; }
  double get_kmax() const override { return 1.e4; }

 private:
  EisensteinHu eh_;
};

std::unique_ptr<TransferFunction_plugin> make_eisenstein(const config_file &cf, const cosmo_parameters &cp) {
  return std::make_unique<transfer_eisenstein_plugin>(cf, cp);
}

struct register_eisenstein {
  register_eisenstein() { get_TransferFunction_plugin_map()["eisenstein"] = &make_eisenstein; }
} s_register_eisenstein;
}  // namespace

std::map<std::string, tf_creator> &get_TransferFunction_plugin_map() {
  static std::map<std::string, tf_creator> m;
  return m;
}

std::unique_ptr<TransferFunction_plugin> select_TransferFunction_plugin(const config_file &cf,
                                                                        const cosmo_parameters &cp) {
  const std::string name = cf.get_value<std::string>("cosmology", "transfer");
  auto &m = get_TransferFunction_plugin_map();
  auto it = m.find(name);
  if (it == m.end()) throw std::runtime_error("Unknown transfer function plug-in '" + name + "'");
  return it->second(cf, cp);
}

// ---------------------------------------------------------------------------
// natural cubic spline in (log x, log y)
// ---------------------------------------------------------------------------
void loglog_spline::set_data(const std::vector<double> &x, const std::vector<double> &y) {
  const size_t n = x.size();
  if (n < 3 || y.size() != n) throw std::runtime_error("spline needs >= 3 matching points");
  x_.resize(n);
  y_.resize(n);
  for (size_t i = 0; i < n; ++i) {
    x_[i] = std::log(x[i]);
    y_[i] = std::log(y[i]);
  }
  // Natural spline: second derivatives s_i with s_0 = s_{n-1} = 0 solve
  //   h_{i-1} s_{i-1} + 2 (h_{i-1} + h_i) s_i + h_i s_{i+1}
  //     = 6 [(y_{i+1} - y_i)/h_i - (y_i - y_{i-1})/h_{i-1}],  0 < i < n-1,
  // a symmetric tridiagonal system solved by forward elimination.
  std::vector<double> h(n - 1), s2(n, 0.0), dd(n, 0.0), rr(n, 0.0);
  for (size_t i = 0; i + 1 < n; ++i) h[i] = x_[i + 1] - x_[i];
  for (size_t i = 1; i + 1 < n; ++i) {
    dd[i] = 2.0 * (h[i - 1] + h[i]);
    rr[i] = 6.0 * ((y_[i + 1] - y_[i]) / h[i] - (y_[i] - y_[i - 1]) / h[i - 1]);
  }
  for (size_t i = 2; i + 1 < n; ++i) {
    const double m = h[i - 1] / dd[i - 1];
    dd[i] -= m * h[i - 1];
    rr[i] -= m * rr[i - 1];
  }
  for (size_t i = n - 2; i >= 1; --i) {
    s2[i] = (rr[i] - h[i] * s2[i + 1]) / dd[i];
    if (i == 1) break;
  }
  // cubic per interval: y_i + b dx + c dx^2 + d dx^3
  b_.assign(n, 0.0);
  c_.assign(n, 0.0);
  d_.assign(n, 0.0);
  for (size_t i = 0; i + 1 < n; ++i) {
    c_[i] = 0.5 * s2[i];
    d_[i] = (s2[i + 1] - s2[i]) / (6.0 * h[i]);
    b_[i] = (y_[i + 1] - y_[i]) / h[i] - h[i] * (2.0 * s2[i] + s2[i + 1]) / 6.0;
  }
}

double loglog_spline::operator()(double x) const {
  const double lx = std::log(x);
  // interval with x_[i] <= lx < x_[i+1] (binary search)
  size_t lo = 0, hi = x_.size() - 1;
  if (lx <= x_.front()) hi = 1;
  else if (lx >= x_.back()) lo = x_.size() - 2;
  while (hi - lo > 1) {
    const size_t mid = (lo + hi) / 2;
    if (x_[mid] > lx) hi = mid;
    else lo = mid;
  }
  const double dx = lx - x_[lo];
  return std::exp(y_[lo] + dx * (b_[lo] + dx * (c_[lo] + dx * d_[lo])));
}

// ---------------------------------------------------------------------------
// calculator
// ---------------------------------------------------------------------------
namespace {
struct V3 {
  double v[3];
  double &operator[](int i) { return v[i]; }
  double operator[](int i) const { return v[i]; }
};
inline V3 operator+(const V3 &a, const V3 &b) { return {{a[0] + b[0], a[1] + b[1], a[2] + b[2]}}; }
inline V3 operator*(double s, const V3 &a) { return {{s * a[0], s * a[1], s * a[2]}}; }
inline V3 vabs(const V3 &a) { return {{std::fabs(a[0]), std::fabs(a[1]), std::fabs(a[2])}}; }

// Cash-Karp embedded Runge-Kutta step (Press & Teukolsky 1992, Computers in
// Physics 6, 188), the scheme of the reference's math/ode_integrate.hh:39-67
template <typename F> V3 ck_step(double h, double t, V3 &y, F f) {
  constexpr double a2 = 0.20, a3 = 0.30, a4 = 0.60, a5 = 1.0, a6 = 0.8750, b21 = 0.20, b31 = 3.0 / 40.0,
                   b32 = 9.0 / 40.0, b41 = 0.30, b42 = -0.90, b43 = 1.20, b51 = -11.0 / 54.0, b52 = 2.50,
                   b53 = -70.0 / 27.0, b54 = 35.0 / 27.0, b61 = 1631.0 / 55296.0, b62 = 175.0 / 512.0,
                   b63 = 575.0 / 13824.0, b64 = 44275.0 / 110592.0, b65 = 253.0 / 4096.0, c1 = 37.0 / 378.0,
                   c3 = 250.0 / 621.0, c4 = 125.0 / 594.0, c6 = 512.0 / 1771.0, dc1 = c1 - 2825.0 / 27648.0,
                   dc3 = c3 - 18575.0 / 48384.0, dc4 = c4 - 13525.0 / 55296.0, dc5 = -277.0 / 14336.0,
                   dc6 = c6 - 0.250;
  const V3 k1 = h * f(t, y);
  const V3 k2 = h * f(t + a2 * h, y + b21 * k1);
  const V3 k3 = h * f(t + a3 * h, y + b31 * k1 + b32 * k2);
  const V3 k4 = h * f(t + a4 * h, y + b41 * k1 + b42 * k2 + b43 * k3);
  const V3 k5 = h * f(t + a5 * h, y + b51 * k1 + b52 * k2 + b53 * k3 + b54 * k4);
  const V3 k6 = h * f(t + a6 * h, y + b61 * k1 + b62 * k2 + b63 * k3 + b64 * k4 + b65 * k5);
  y = y + (c1 * k1 + c3 * k3 + c4 * k4 + c6 * k6);
  return dc1 * k1 + dc3 * k3 + dc4 * k4 + dc5 * k5 + dc6 * k6;
}

// quality-controlled step (ode_integrate.hh:72-111).  As in the reference, a
// rejected trial continues from the state the rejected trial left behind.
template <typename F>
void rk_step_qs(double htry, double &t, V3 &y, const V3 &yscale, F f, double eps, double &hdid, double &hnext) {
  constexpr double SAFETY = 0.9, PSHRNK = -0.25, PGROW = -0.2, ERRCON = 1.89e-4;
  double h = htry;
  V3 ytemp = y;
  for (;;) {
    const V3 yerr = ck_step(h, t, ytemp, f);
    double errmax = 0.0;
    for (int i = 0; i < 3; ++i) errmax = std::max(errmax, std::fabs(yerr[i] / yscale[i]));
    errmax = errmax / eps;
    if (errmax > 1.0) {
      h *= std::max(0.1, SAFETY * std::pow(errmax, PSHRNK));
      if (t + h == t) throw std::runtime_error("stepsize underflow in rkqs");
      continue;
    }
    hnext = (errmax > ERRCON) ? h * SAFETY * std::pow(errmax, PGROW) : 5 * h;
    hdid = h;
    t += h;
    y = ytemp;
    return;
  }
}

// Gauss-Legendre nodes/weights on [-1,1] by Newton iteration on P_n
void gauss_legendre(int n, std::vector<double> &x, std::vector<double> &w) {
  x.resize(n);
  w.resize(n);
  for (int i = 0; i < (n + 1) / 2; ++i) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), pp = 0;
    for (int it = 0; it < 100; ++it) {
      double p1 = 1.0, p2 = 0.0;
      for (int j = 1; j <= n; ++j) {
        const double p3 = p2;
        p2 = p1;
        p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1.0);
      const double z1 = z;
      z = z1 - p1 / pp;
      if (std::fabs(z - z1) < 1e-16) break;
    }
    x[i] = -z;
    x[n - 1 - i] = z;
    w[i] = w[n - 1 - i] = 2.0 / ((1.0 - z * z) * pp * pp);
  }
}

// globally adaptive Gauss-Legendre quadrature (order 20 vs 40 error estimate,
// bisection of the worst interval) of g over [a, b]
template <typename G> double integrate_adaptive(G g, double a, double b, double rel) {
  static std::vector<double> x20, w20, x40, w40;
  if (x20.empty()) {
    gauss_legendre(20, x20, w20);
    gauss_legendre(40, x40, w40);
  }
  struct Seg {
    double a, b, val, err;
    bool operator<(const Seg &o) const { return err < o.err; }
  };
  auto eval = [&](double lo, double hi) {
    const double c = 0.5 * (hi + lo), r = 0.5 * (hi - lo);
    double s20 = 0, s40 = 0;
    for (int i = 0; i < 20; ++i) s20 += w20[i] * g(c + r * x20[i]);
    for (int i = 0; i < 40; ++i) s40 += w40[i] * g(c + r * x40[i]);
    return Seg{lo, hi, s40 * r, std::fabs(s40 - s20) * r};
  };
  std::priority_queue<Seg> q;
  const int n0 = 64;
  double total = 0, err = 0;
  for (int i = 0; i < n0; ++i) {
    Seg s = eval(a + (b - a) * i / n0, a + (b - a) * (i + 1) / n0);
    total += s.val;
    err += s.err;
    q.push(s);
  }
  for (int it = 0; it < 20000 && err > rel * std::fabs(total); ++it) {
    Seg s = q.top();
    q.pop();
    const double m = 0.5 * (s.a + s.b);
    Seg l = eval(s.a, m), r = eval(m, s.b);
    total += l.val + r.val - s.val;
    err += l.err + r.err - s.err;
    q.push(l);
    q.push(r);
  }
  // re-sum to remove accumulated update rounding
  total = 0;
  while (!q.empty()) {
    total += q.top().val;
    q.pop();
  }
  return total;
}
}  // namespace

double calculator::H_of_a(double a) const {
  double HH2 = 0.0;
  HH2 += cosmo_param_["Omega_r"] / (a * a * a * a);
  HH2 += cosmo_param_["Omega_m"] / (a * a * a);
  HH2 += cosmo_param_["Omega_k"] / (a * a);
  HH2 += cosmo_param_["Omega_DE"] * std::pow(a, -3. * (1. + cosmo_param_["w_0"] + cosmo_param_["w_a"])) *
         std::exp(-3. * (1.0 - a) * cosmo_param_["w_a"]);
  return cosmo_param_["H0"] * std::sqrt(HH2);
}

// linear growth ODE in conformal time (cosmology_calculator.hh:92-152)
void calculator::compute_growth(std::vector<double> &tab_a, std::vector<double> &tab_D, std::vector<double> &tab_f) {
  const double a0 = 1e-10, D0 = a0;
  const double Dprime0 = 2.0 * D0 * H_of_a(a0) / std::pow(phys_const::c_SI, 2);
  const double t0 = 1.0 / (a0 * H_of_a(a0));
  V3 yy{{a0, D0, Dprime0}};
  double dt = 1e-9, dtdid = 0, dtnext = 0, t = t0;
  const double amax = 2.0, eps = 1e-10;
  const double Omega_m = cosmo_param_["Omega_m"], H0 = cosmo_param_["H0"];
  auto rhs = [&](double, const V3 &y) -> V3 {
    const double a = y[0], D = y[1], Dprime = y[2];
    V3 dy;
    dy[0] = a * a * H_of_a(a);
    dy[1] = Dprime;
    dy[2] = -a * H_of_a(a) * Dprime + 3.0 / 2.0 * Omega_m * std::pow(H0, 2) * D / a;
    return dy;
  };
  while (yy[0] < amax) {
    const V3 yyscale = vabs(yy) + dt * vabs(rhs(t, yy));
    rk_step_qs(dt, t, yy, yyscale, rhs, eps, dtdid, dtnext);
    tab_a.push_back(yy[0]);
    tab_D.push_back(yy[1]);
    tab_f.push_back(yy[2]);
    dt = dtnext;
  }
  for (size_t i = 0; i < tab_a.size(); ++i) tab_f[i] = tab_f[i] / (tab_a[i] * H_of_a(tab_a[i]) * tab_D[i]);
}

calculator::calculator(const config_file &cf)
    : cosmo_param_(cf),
      astart_(1.0 / (1.0 + cf.get_value<double>("setup", "zstart"))),
      atarget_(1.0 / (1.0 + cf.get_value_safe<double>("cosmology", "ztarget", 0.0))) {
  std::vector<double> ta, tD, tf;
  compute_growth(ta, tD, tf);
  D_of_a_.set_data(ta, tD);
  f_of_a_.set_data(ta, tf);
  Dnow_ = D_of_a_(1.0);
  Dplus_start_ = D_of_a_(astart_) / Dnow_;
  Dplus_target_ = D_of_a_(atarget_) / Dnow_;
  cosmo_param_.set("dplus_start", Dplus_start_);
  cosmo_param_.set("dplus_target", Dplus_target_);
  transfer_function_ = select_TransferFunction_plugin(cf, cosmo_param_);
  transfer_function_->intialise();
  if (!transfer_function_->tf_isnormalised_) {
    if (cosmo_param_["A_s"] > -1.) {
      const double h = cosmo_param_["h"];
      cosmo_param_.set("pnorm", cosmo_param_["A_s"] * std::pow(cosmo_param_["k_p"] / h, 1.0 - cosmo_param_["n_s"]) *
                                    (h * h * h * h) / (4 * M_PI * Dplus_target_ * Dplus_target_));
    } else {
      const double s8 = compute_sigma8();
      cosmo_param_.set("pnorm", cosmo_param_["sigma_8"] * cosmo_param_["sigma_8"] / (s8 * s8));
    }
  } else {
    cosmo_param_.set("pnorm", 1.0 / Dplus_target_ / Dplus_target_);
  }
  cosmo_param_.set("sqrtpnorm", std::sqrt(cosmo_param_["pnorm"]));
  vfac_start_ = transfer_function_->tf_has_asymptotic_growth_factors() ? transfer_function_->get_vfac_asymptotic()
                                                                       : get_vfact(astart_);
  cosmo_param_.set("vfact_start", vfac_start_);
  m_n_s_ = cosmo_param_["n_s"];
  m_sqrtpnorm_ = cosmo_param_["sqrtpnorm"];
}

double calculator::get_amplitude(double k, tf_type type) const {
  return std::pow(k, 0.5 * m_n_s_) * transfer_function_->compute(k, type) * m_sqrtpnorm_;
}

double calculator::get_amplitude_delta_bc(double k, bool withvbc) const {
  const double dratio = Dplus_target_ / Dplus_start_;
  const double dbc = transfer_function_->compute(k, delta_bc) +
                     (withvbc ? 2.0 * transfer_function_->compute(k, theta_bc) * (std::sqrt(dratio) - 1.0) : 0.0);
  return std::pow(k, 0.5 * m_n_s_) * dbc * (m_sqrtpnorm_ * Dplus_target_);
}

double calculator::get_amplitude_theta_bc(double k, bool withvbc) const {
  const double dratio = Dplus_target_ / Dplus_start_;
  const double tbc = transfer_function_->compute(k, theta_bc) * std::sqrt(dratio);
  return withvbc ? std::pow(k, 0.5 * m_n_s_) * tbc * (m_sqrtpnorm_ * Dplus_target_) : 0.0;
}

// sigma_8 of the unnormalised spectrum (cosmology_calculator.hh:441-455,
// 472-485): 4 pi int k^2 W^2(8k) k^n_s T^2 dk over [kmin, kmax], integrated
// in ln k to a relative accuracy far below the reference's 1e-10 target.
double calculator::compute_sigma8() const {
  const double kmin = transfer_function_->get_kmin(), kmax = transfer_function_->get_kmax();
  const double ns = cosmo_param_["n_s"];
  const tf_type tt = transfer_function_->tf_has_total0() ? delta_matter0 : delta_matter;
  auto dsigma = [&](double u) {
    const double k = std::exp(u);
    const double x = k * 8.0;
    const double w = (x < 0.001) ? 1.0 - 0.1 * x * x : 3.0 * (std::sin(x) - x * std::cos(x)) / (x * x * x);
    const double tf = transfer_function_->compute(k, tt);
    return k * (k * k * w * w * std::pow(k, ns) * tf * tf);
  };
  const double sigma0 = 4.0 * M_PI * integrate_adaptive(dsigma, std::log(kmin), std::log(kmax), 1e-14);
  return std::sqrt(sigma0);
}

}  // namespace mfx
