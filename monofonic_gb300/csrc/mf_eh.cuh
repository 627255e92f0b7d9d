// Eisenstein & Hu (1998) transfer-function fit, host and device.
// Restates TFset_parameters / TFfit_onek / at_k of
// src/plugins/transfer_eisenstein.cc:58-201 (Units: Mpc inside the fit,
// h/Mpc at the at_k boundary).
#pragma once

#include <cmath>

#include "mf_cosmo.h"

namespace mf {

#if defined(__CUDACC__)
#define MF_HD __host__ __device__
#else
#define MF_HD
#endif

// T_full mixture of the fit at k in h/Mpc (at_k, transfer_eisenstein.cc:196-201)
MF_HD inline double eh_eval(const EHParams& P, double k_hmpc) {
  double k = k_hmpc * P.m_h0;
  k = fabs(k);
  if (k == 0.0) return P.fb * 1.0 + P.fc * 1.0;
  const double q = k / 13.41 / P.k_equality;
  const double xx = k * P.sound_horizon;
  const double ln_beta = log(2.718282 + 1.8 * P.beta_c * q);
  const double ln_nobeta = log(2.718282 + 1.8 * q);
  const double q108 = pow(q, 1.08);
  const double C_alpha = 14.2 / P.alpha_c + 386.0 / (1 + 69.9 * q108);
  const double C_noalpha = 14.2 + 386.0 / (1 + 69.9 * q108);
  const double x54 = xx / 5.4;
  const double f = 1.0 / (1.0 + (x54 * x54) * (x54 * x54));
  const double Tc = f * ln_beta / (ln_beta + C_noalpha * q * q) + (1 - f) * ln_beta / (ln_beta + C_alpha * q * q);
  const double bn = P.beta_node / xx;
  const double s_tilde = P.sound_horizon * pow(1. + bn * bn * bn, -1. / 3.);
  const double xt = k * s_tilde;
  const double Tb_T0 = ln_nobeta / (ln_nobeta + C_noalpha * q * q);
  const double x52 = xx / 5.2;
  const double bb = P.beta_b / xx;
  const double Tb = sin(xt) / xt *
                    (Tb_T0 / (1. + x52 * x52) + P.alpha_b / (1. + bb * bb * bb) * exp(-pow(k / P.k_silk, 1.4)));
  return P.fb * Tb + P.fc * Tc;
}

}  // namespace mf
