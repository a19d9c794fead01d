// CMEM coefficient set-up on the host, FP64: CMEM::Init with
// CalcDynamicPressure, CalcMagneticPressure, CalcInitialAlpha and
// DefineLinearCoeffs (src/Cmem.cpp:38-115, 250-325). The reference's float
// parameters and constants enter exactly; its quirks stay: p2 takes p3's
// value when set (:90), 0 means "unset", and B is replaced by the field
// magnitude |b| in tesla (:310).
#include <cmath>

#include "birp_host.h"

namespace birp {

// Lin et al. magnetopause coefficients a0..a21 (the table of
// src/Cmem.cpp:253, which has to be the same numbers).
static const float kLin[22] = {12.544f,   -0.194f,  0.305f,    0.0573f, 2.178f,   0.0571f, -0.999f, 16.473f,
                               0.00152f,  0.382f,   0.0431f,   -0.00763f, -0.210f, 0.0405f, -4.430f, -0.636f,
                               -2.600f,   0.832f,   -5.328f,   1.103f,  -0.907f,  1.450f};

static double mag3(const double* v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }

void cmem_coefficients(const birp_cmem_params& g, CmemDev& m) {
  double v[3] = {400, 0, 0}, b[3] = {0, 0, 5};
  if (g.has_v)
    for (int i = 0; i < 3; ++i) v[i] = g.v[i];
  if (g.has_b)
    for (int i = 0; i < 3; ++i) b[i] = g.b[i];
  const double dipole = g.dipole;
  const double alpha = g.alpha, beta = g.beta;
  const double p0 = g.p0 == 0 ? (double)0.786300004f : (double)g.p0;
  const double p1 = g.p1 == 0 ? 1.0 : (double)g.p1;
  const double p2 = g.p2 == 0 ? 3.0 : (double)g.p3;
  const double p3 = g.p3 == 0 ? 4.0 : (double)g.p3;
  const double bs = g.bs == 0 ? (double)12.64f : (double)g.bs;
  const double A1 = g.A1 == 0 ? (double)7.2e-06f : (double)g.A1;
  const double A2 = g.A2 == 0 ? (double)3.5e-06f : (double)g.A2;
  const double density = g.density == 0 ? 5.0 : (double)g.density;
  const double pdyn = 0.5 * (double)0.00000000000000000000000000167f * (density * 1000000) *
                      ((mag3(v) * 1000) * (mag3(v) * 1000)) * 1e9;
  const double Bt = mag3(b) * 1e-9;
  const double pmag = (Bt * Bt) / (2 * (4 * M_PI * 1e-7)) * 1e9;
  const double alpha0 = ((double)0.58f - 0.010 * b[2]) * (1 + (double)0.010f * pdyn) + (double)0.2f;
  const double ay = g.ay_bs == 0 ? alpha0 : (double)g.ay_bs;
  const double az = g.az_bs == 0 ? alpha0 : (double)g.az_bs;
  double a[22];
  for (int i = 0; i < 22; ++i) a[i] = kLin[i];
  const double bc0 = a[6] + a[7] * ((std::exp(a[8] * b[2]) - 1) / (std::exp(a[9] * b[2]) + 1));
  const double bc1 = a[10], bc3 = a[13];
  const double pt = pdyn + pmag;
  const double charlie = a[14] * std::pow(pt, a[15]);
  const double dn = a[16] + a[17] * dipole + a[18] * (dipole * dipole);
  const double ds = a[16] - a[17] * dipole + a[18] * (dipole * dipole);
  const double tn = a[19] + a[20] * dipole, ts = a[19] - a[20] * dipole;
  const double r0 = a[0] * std::pow(pt, a[1]) * (1 + a[2] * ((std::exp(a[3] * b[2]) - 1) / (std::exp(a[4] * b[2]) + 1)));

  m.p0r0 = (float)(p0 * r0);
  m.p1 = (float)p1;
  m.p2c = (float)(p2 * charlie);
  m.p3dn = (float)(p3 * dn);
  m.p3ds = (float)(p3 * ds);
  m.a5 = (float)a[5];
  m.a21 = (float)a[21];
  m.bs = (float)bs;
  m.ay = (float)ay;
  m.az = (float)az;
  m.A1 = (float)A1;
  m.A2 = (float)A2;
  m.B = (float)Bt;
  m.alpha = (float)alpha;
  m.beta = (float)beta;
  m.bc0 = (float)bc0;
  m.bc1 = (float)bc1;
  m.bc3 = (float)bc3;
  m.cos_tn = (float)std::cos(tn);
  m.sin_tn = (float)std::sin(tn);
  m.cos_ts = (float)std::cos(ts);
  m.sin_ts = (float)std::sin(ts);
  m.d_p0 = p0;
  m.d_p1 = p1;
  m.d_p2 = p2;
  m.d_p3 = p3;
  m.d_dn = dn;
  m.d_ds = ds;
  m.d_tn = tn;
  m.d_ts = ts;
  m.d_r0 = r0;
  m.d_charlie = charlie;
  m.d_a5 = a[5];
  m.d_a21 = a[21];
  m.d_bs = bs;
  m.d_ay = ay;
  m.d_az = az;
  m.d_A1 = A1;
  m.d_A2 = A2;
  m.d_B = Bt;
  m.d_alpha = alpha;
  m.d_beta = beta;
  m.d_bc0 = bc0;
  m.d_bc1 = bc1;
  m.d_bc3 = bc3;
  // FP32 radii of the shell surfaces agree with FP64 to ~1e-6 of (r + 5 Re)
  // (checked by birp_cmem_margin_check); decide in FP64 within 2e-5 of it.
  m.eps_rel = 2e-5f;
}

}  // namespace birp
