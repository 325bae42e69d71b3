// Host-side cosmology for the IC engine: parameters, the transfer-function
// plugin interface with the Eisenstein & Hu plugin, and the calculator that
// provides D+(a), vfact and the P(k) amplitude.
//
// Interfaces mirror the reference so its callers read the same:
//   cosmology::parameters        include/cosmology_parameters.hh:29-253
//   TransferFunction_plugin      include/transfer_function_plugin.hh:48-149
//   transfer_eisenstein_plugin   src/plugins/transfer_eisenstein.cc:206-258
//   cosmology::calculator        include/cosmology_calculator.hh:44-523
#pragma once
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "config_file.h"

namespace mfx {

enum tf_type {
  delta_matter, delta_cdm, delta_baryon, theta_matter, theta_cdm, theta_baryon,
  delta_bc, theta_bc, delta_matter0, delta_cdm0, delta_baryon0, theta_matter0,
  theta_cdm0, theta_baryon0, delta_nu, theta_nu
};

// physical_constants.hh:24-73 (PDG 2018 values used by the reference)
namespace phys_const {
constexpr double pi_ = 3.141592653589793115997963468544185161590576171875;
constexpr double Mpc_SI = 3.0857e22;
constexpr double c_SI = 2.99792458e8;
constexpr double G_SI = 6.6740800e-11;
constexpr double kB_SI = 1.38064852e-23;
constexpr double hbar_SI = 1.054571800e-34;
constexpr double sigma_SI = (pi_ * pi_) * (kB_SI * kB_SI * kB_SI * kB_SI) / 60. /
                            (hbar_SI * hbar_SI * hbar_SI) / (c_SI * c_SI);
constexpr double rhocrit_h2_SI = 3 * 1e10 / (8 * pi_ * G_SI) / Mpc_SI / Mpc_SI;
}  // namespace phys_const

class cosmo_parameters {
 public:
  explicit cosmo_parameters(const config_file &cf);
  double operator[](const std::string &k) const { return get(k); }
  double get(const std::string &k) const;
  void set(const std::string &k, double v) { pmap_[k] = v; }

 private:
  std::map<std::string, double> pmap_;
};

class TransferFunction_plugin {
 public:
  TransferFunction_plugin(const config_file &cf, const cosmo_parameters &cp) : pcf_(&cf), cosmo_params_(cp) {}
  virtual ~TransferFunction_plugin() {}
  virtual void intialise() {}
  virtual double compute(double k, tf_type type) const = 0;
  virtual double get_kmin() const = 0;
  virtual double get_kmax() const = 0;
  bool tf_is_distinct() const { return tf_distinct_; }
  bool tf_has_velocities() const { return tf_withvel_; }
  bool tf_has_total0() const { return tf_withtotal0_; }
  bool tf_has_asymptotic_growth_factors() const { return tf_with_asymptotic_growth_factors_; }
  virtual double get_vfac_asymptotic() const;

  bool tf_distinct_ = false, tf_withvel_ = false, tf_withtotal0_ = false;
  bool tf_with_asymptotic_growth_factors_ = false, tf_isnormalised_ = false;

 protected:
  const config_file *pcf_;
  const cosmo_parameters &cosmo_params_;
};

// name -> creator registry (transfer_function_plugin.hh:116-149)
using tf_creator = std::unique_ptr<TransferFunction_plugin> (*)(const config_file &, const cosmo_parameters &);
std::map<std::string, tf_creator> &get_TransferFunction_plugin_map();
std::unique_ptr<TransferFunction_plugin> select_TransferFunction_plugin(const config_file &cf,
                                                                        const cosmo_parameters &cp);

// log-x / log-y natural cubic spline (the reference's
// interpolated_function_1d<true,true,false>, math/interpolate.hh:28-103)
class loglog_spline {
 public:
  void set_data(const std::vector<double> &x, const std::vector<double> &y);
  double operator()(double x) const;

 private:
  std::vector<double> x_, y_, b_, c_, d_;
};

class calculator {
 public:
  explicit calculator(const config_file &cf);
  double H_of_a(double a) const;
  double get_growth_factor(double a) const { return D_of_a_(a) / Dnow_; }
  double get_f(double a) const { return f_of_a_(a); }
  double get_vfact(double a) const { return f_of_a_(a) * a * H_of_a(a) / cosmo_param_["h"]; }
  double get_vfact_start() const { return vfac_start_; }
  double get_amplitude(double k, tf_type type) const;
  // back-scaled delta_bc and relative-velocity theta_bc amplitudes of a baryon
  // + CDM run (cosmology_calculator.hh:434-450); zero for transfer functions
  // without separate baryon and CDM transfers (E&H)
  double get_amplitude_delta_bc(double k, bool withvbc) const;
  double get_amplitude_theta_bc(double k, bool withvbc) const;
  double compute_sigma8() const;

  cosmo_parameters cosmo_param_;
  std::unique_ptr<TransferFunction_plugin> transfer_function_;

 private:
  void compute_growth(std::vector<double> &a, std::vector<double> &D, std::vector<double> &f);
  loglog_spline D_of_a_, f_of_a_;
  double Dnow_ = 1, Dplus_start_ = 1, Dplus_target_ = 1, astart_ = 1, atarget_ = 1;
  double vfac_start_ = 0, m_n_s_ = 1, m_sqrtpnorm_ = 1;
};

}  // namespace mfx
