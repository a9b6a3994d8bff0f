// kf_material.h — surface material effects for a heavy charged particle
// (host and device, FP64): the reference's pointwise material interaction
// after a measurement (Propagator/detail/PointwiseMaterialInteraction.hpp,
// .ipp:14-51, with the formulas of Material/detail/Interactions.ipp).
//
//   Bethe mean energy loss (RPP2018 eq. 33.5 times the thickness, density
//   correction eq. 33.6 above beta gamma 10), Interactions.ipp:150-176;
//   Landau width as a Gaussian sigma on q/p, :298-345;
//   Highland scattering angle theta0 (RPP2018 eq. 33.15), :495-546.
//
// Constants as the reference's double build evaluates them: literals that
// the reference writes as floats (0.038f, 0.9f) keep their float values.
#pragma once

#include <cfloat>
#include <cmath>

#ifdef __CUDACC__
#define KFM_HD __host__ __device__ __forceinline__
#else
#define KFM_HD inline
#endif

namespace kfm {

struct Relativistic {
  double q2OverBeta2, beta2, betaGamma, gamma;
};
// RelativisticQuantities (Interactions.ipp:28-49)
KFM_HD Relativistic relativistic(double m, double qop, double q) {
  Relativistic r;
  r.q2OverBeta2 = q * q + (m * qop) * (m * qop);
  const double mOverP = m * fabs(qop / q);
  const double pOverM = 1.0 / mOverP;
  r.beta2 = 1.0 / (1.0 + mOverP * mOverP);
  r.betaGamma = pOverM;
  r.gamma = sqrt(1.0 + pOverM * pOverM);
  return r;
}

constexpr double kElectronMass = 0.5109989461e-3; // GeV
constexpr double kBetheK = 0.307075e-3 * 100.;    // GeV mm^2 / mol
constexpr double kPlasmaScale = 28.816e-9;        // GeV

// (K/2) (Z rho_molar) x q^2/beta^2
KFM_HD double epsilon(double electronDensity, double thickness, const Relativistic &r) {
  return 0.5 * kBetheK * electronDensity * thickness * r.q2OverBeta2;
}

// mean energy loss (GeV) in `thickness` (mm) of material (Z, molar density)
KFM_HD double betheLoss(double thickness, double Z, double molarRho, double m, double qop,
                        double q) {
  const double I = 16e-9 * pow(Z, (double)0.9f); // mean excitation energy
  const double Ne = Z * molarRho;
  const Relativistic r = relativistic(m, qop, q);
  double dhalf = 0.;
  if (!(r.betaGamma < 10.0))
    dhalf = log(r.betaGamma) + log(kPlasmaScale * sqrt(Ne) / I) - 0.5;
  const double u = 2 * kElectronMass * r.betaGamma * r.betaGamma;
  const double mf = kElectronMass / m;
  const double wmax = u / (1.0 + 2 * r.gamma * mf + mf * mf);
  return epsilon(Ne, thickness, r) * (0.5 * log(u / I) + 0.5 * log(wmax / I) - r.beta2 - dhalf);
}

// sigma of q/p from the Landau width: fwhm = 4 epsilon, sigma_E = fwhm /
// (2 sqrt(2 ln 2)), sigma_qop = |q/beta| / p^2 sigma_E
KFM_HD double landauSigmaQop(double thickness, double Z, double molarRho, double m, double qop,
                             double q) {
  const Relativistic r = relativistic(m, qop, q);
  const double sigmaE = 4 * epsilon(Z * molarRho, thickness, r) / (2 * sqrt(2 * log(2.0)));
  const double pInv = qop / q;
  return sqrt(r.q2OverBeta2) * pInv * pInv * sigmaE;
}

// Highland theta0 for a thickness of xOverX0 radiation lengths
KFM_HD double highlandTheta0(double xOverX0, double m, double qop, double q) {
  const double t = sqrt(xOverX0 * relativistic(m, qop, q).q2OverBeta2);
  return 13.6e-3 * fabs(qop / q) * t * (1.0 + (double)0.038f * 2 * log(t));
}

// Per-plane constants of a homogeneous slab, computed once per geometry so
// that a crossing spends no pow() and one logarithm on the mean excitation
// energy: mat = (thickness, X0, L0, Ar, Z, molar density).
struct Slab {
  double t0;      // thickness (mm)
  double x0frac;  // thickness / X0 (0 for X0 <= 2 eps, as the reference)
  double Ne;      // electron density Z * molar density
  double logI;    // log of the mean excitation energy 16 eV Z^0.9 (GeV)
  double plasma;  // log(28.816 eV sqrt(Ne) / I), the density correction's constant
  int valid;      // Ar > 0 and thickness > 0
};
KFM_HD Slab slab(const double mat[6]) {
  Slab s;
  const double t0 = mat[0], X0 = mat[1], Ar = mat[3], Z = mat[4], rho = mat[5];
  s.valid = (0.0 < Ar) && (0.0 < t0);
  s.t0 = t0;
  s.x0frac = (2 * DBL_EPSILON < X0) ? (t0 / X0) : 0.;
  s.Ne = Z * rho;
  const double I = 16e-9 * pow(Z, (double)0.9f);
  s.logI = log(I);
  s.plasma = log(kPlasmaScale * sqrt(s.Ne) / I);
  return s;
}

constexpr double kFwhmOverSigma = 2.3548200450309493; // 2 sqrt(2 ln 2) of a Gaussian

// The interaction at a plane crossed along unit direction d (normal n):
// slab thickness and x/X0 scaled by 1/|n.d|; returns the new |p| and the
// variances to add to the phi, theta and q/p entries of the bound covariance.
// flags bit 0 scattering, bit 1 energy loss.  Returns false (nothing to do)
// without material.  The expressions are those of betheLoss, landauSigmaQop
// and highlandTheta0 above with the relativistic factors shared and
// 0.5 log(u / I) + 0.5 log(wmax / I) taken as 0.5 log(u wmax) - log I.
struct Effects {
  double p, varPhi, varTheta, varQop, eloss;
};
KFM_HD bool interact(const Slab &sl, int flags, const double n[3], const double d[3], double p,
                     double q, double m, Effects &e) {
  if (!(flags & 3) || !sl.valid) return false;
  const double pc = 1. / fabs(n[0] * d[0] + n[1] * d[1] + n[2] * d[2]);
  const double thickness = sl.t0 * pc;
  const double qop = q / p;
  const Relativistic r = relativistic(m, qop, q);
  const double eps = epsilon(sl.Ne, thickness, r);
  e.eloss = 0.;
  e.varPhi = e.varTheta = e.varQop = 0.;
  if (flags & 2) {
    double dhalf = 0.;
    if (!(r.betaGamma < 10.0)) dhalf = log(r.betaGamma) + sl.plasma - 0.5;
    const double u = 2 * kElectronMass * r.betaGamma * r.betaGamma;
    const double mf = kElectronMass / m;
    const double wmax = u / (1.0 + 2 * r.gamma * mf + mf * mf);
    e.eloss = eps * (0.5 * log(u * wmax) - sl.logI - r.beta2 - dhalf);
    const double pInv = qop / q;
    const double s = sqrt(r.q2OverBeta2) * pInv * pInv * (4 * eps / kFwhmOverSigma);
    e.varQop = s * s;
  }
  if (flags & 1) {
    const double t = sqrt(sl.x0frac * pc * r.q2OverBeta2);
    const double th0 = 13.6e-3 * fabs(qop / q) * t * (1.0 + (double)0.038f * 2 * log(t));
    const double perp = sqrt(d[0] * d[0] + d[1] * d[1]);
    const double sPhi = th0 * (sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) / perp);
    e.varPhi = sPhi * sPhi;
    e.varTheta = th0 * th0;
  }
  const double nextE = sqrt(m * m + p * p) - e.eloss;
  e.p = (m < nextE) ? sqrt(nextE * nextE - m * m) : 0.;
  return true;
}
KFM_HD bool interact(const double mat[6], int flags, const double n[3], const double d[3],
                     double p, double q, double m, Effects &e) {
  return interact(slab(mat), flags, n, d, p, q, m, e);
}

} // namespace kfm
