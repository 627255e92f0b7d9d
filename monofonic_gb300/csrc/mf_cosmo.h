// Host cosmology for the pipeline: derived parameters, linear growth,
// sigma_8 normalisation and the Eisenstein & Hu fit parameters.
#pragma once

#include "../../include/monofonic_gb300_ic.h"

namespace mf {

// TFset_parameters outputs (src/plugins/transfer_eisenstein.cc:58-122) and
// the at_k mixing weights (:186-201); shared by the host and device fits
struct EHParams {
  double m_h0, omhh, obhh, k_equality, sound_horizon, k_silk, alpha_c, beta_c, alpha_b, beta_b, beta_node;
  double fb, fc;
};

void eh_setup(double H0, double Omega_m, double Omega_b, double Tcmb, EHParams* p);
double eh_at_k(const EHParams& p, double k);  // k in h/Mpc

}  // namespace mf
