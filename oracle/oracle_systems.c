/*
 * oracle_systems.c -- C callbacks F/B/S of the test systems, with the
 * reference's callback signatures (src/api.h:4-10, pypde/cfuncs.py:6-8).
 *
 * TEST INFRASTRUCTURE ONLY (see ader_oracle.h).  They play the part of the
 * user's numba-compiled cfuncs: the reference C++ build (through
 * ref_driver.cpp) and the C port both call these same functions, so the
 * two checkers see bit-identical flux values.  The GPU library carries its
 * own device implementations of the same formulas, written in the same
 * operation order (pypde_gb300/csrc/systems.cuh).
 *
 * Systems:
 *   euler     V = ndim+2   Q = (rho, m_0..m_{ndim-1}, E), gamma = 1.4.  F only.
 *   cattaneo  V = 2ndim+3  Euler + relaxing heat flux q_0..q_{ndim-1} + a
 *             passive s = log10(tau).  T = p/rho.  F_d adds q_d to the
 *             energy flux and kappa_h T to q_d, kappa_h = kappa/tau_ref =
 *             1e-2/1e-2 = 1 (a fixed heat-wave speed); the local tau enters
 *             only the stiff relaxation S_q = -q/tau, 1/tau = 10^-s by
 *             pow10_portable.  F and S.
 *   ncp       V = 3, a non-conservative test system with F, B and S:
 *             F_d = a_d (Q0^2/2, Q0 Q1, Q0 Q2),
 *             B_d = a_d [[0,0,0],[0,Q0,0.2],[0,0.2,Q0]],
 *             S   = (0, 0.1(Q2-Q1), -0.1(Q1+Q2)),  a = (1, 0.5, 0.25).
 *   burgers2  V = 1, viscous Burgers in the second-order form F(Q, DQ, d):
 *             F_d = a_d Q0^2/2 - 0.01 DQ[d].
 */
#include "ader_oracle.h"

#include <math.h>
#include <string.h>

#define GAMMA 1.4
#define KAPPA_H 1.0 /* kappa / tau_ref = 1e-2 / 1e-2 */

static int g_ndim = 1;

/* 10^x = 2^n e^r with n = round(x log2 10), |r| <= ln2/2, and e^r by its
 * Taylor polynomial of degree 16 in Horner form (truncation below 1e-22).
 * Built only from IEEE +, *, floor and ldexp, so the host and the device
 * evaluate it to the same bits (a libm exp/pow may differ between the two in
 * the last place).  INV_FACT[k] is the double nearest to 1/k!. */
static const double INV_FACT[17] = {
    1.0, 1.0, 0.5, 0.16666666666666666,
    0.041666666666666664, 0.008333333333333333, 0.001388888888888889, 0.0001984126984126984,
    2.48015873015873e-05, 2.7557319223985893e-06, 2.755731922398589e-07, 2.505210838544172e-08,
    2.08767569878681e-09, 1.6059043836821613e-10, 1.1470745597729725e-11, 7.647163731819816e-13,
    4.779477332387385e-14};

static double pow10_portable(double x) {
  double y = x * 3.321928094887362;
  double n = floor(y + 0.5);
  double r = (y - n) * 0.6931471805599453;
  double p = INV_FACT[16];
  for (int k = 15; k >= 0; k--)
    p = p * r + INV_FACT[k];
  return ldexp(p, (int)n);
}

static void euler_core(double *out, const double *Q, int ndim, int d,
                       double *p_out) {
  double r = Q[0];
  double ke = 0.0;
  for (int i = 0; i < ndim; i++)
    ke += Q[1 + i] * Q[1 + i];
  double p = (GAMMA - 1.0) * (Q[ndim + 1] - 0.5 * ke / r);
  double ud = Q[1 + d] / r;
  out[0] = Q[1 + d];
  for (int i = 0; i < ndim; i++)
    out[1 + i] = Q[1 + i] * ud;
  out[1 + d] += p;
  out[ndim + 1] = (Q[ndim + 1] + p) * ud;
  *p_out = p;
}

static void euler_F(double *out, double *Q, double *dQ, int d) {
  (void)dQ;
  double p;
  euler_core(out, Q, g_ndim, d, &p);
}

static void cattaneo_F(double *out, double *Q, double *dQ, int d) {
  (void)dQ;
  int nd = g_ndim;
  double p;
  euler_core(out, Q, nd, d, &p);
  double T = p / Q[0];
  out[nd + 1] += Q[nd + 2 + d];
  for (int i = 0; i < nd; i++)
    out[nd + 2 + i] = 0.0;
  out[nd + 2 + d] = KAPPA_H * T;
  out[2 * nd + 2] = 0.0;
}

static void cattaneo_S(double *out, double *Q) {
  int nd = g_ndim;
  double inv_tau = pow10_portable(-Q[2 * nd + 2]);
  for (int i = 0; i < nd + 2; i++)
    out[i] = 0.0;
  for (int i = 0; i < nd; i++)
    out[nd + 2 + i] = -Q[nd + 2 + i] * inv_tau;
  out[2 * nd + 2] = 0.0;
}

static const double NCP_A[3] = {1.0, 0.5, 0.25};

static void ncp_F(double *out, double *Q, double *dQ, int d) {
  (void)dQ;
  double a = NCP_A[d];
  out[0] = a * (0.5 * Q[0] * Q[0]);
  out[1] = a * (Q[0] * Q[1]);
  out[2] = a * (Q[0] * Q[2]);
}

static void ncp_B(double *out, double *Q, int d) {
  double a = NCP_A[d];
  for (int i = 0; i < 9; i++)
    out[i] = 0.0;
  out[4] = a * Q[0];
  out[5] = a * 0.2;
  out[7] = a * 0.2;
  out[8] = a * Q[0];
}

static void ncp_S(double *out, double *Q) {
  out[0] = 0.0;
  out[1] = 0.1 * (Q[2] - Q[1]);
  out[2] = -0.1 * (Q[1] + Q[2]);
}

static void burgers2_F(double *out, double *Q, double *dQ, int d) {
  out[0] = NCP_A[d] * (0.5 * Q[0] * Q[0]) - 0.01 * dQ[d];
}

/* The variables that the flux in direction d transports, for a system
 * that declares them (the device systems' EIG_ACTIVE / eig_active): fills
 * idx (ascending) and returns their count, or 0.  cattaneo: rho, the
 * momenta, E and q_d; the other heat-flux components and log tau are
 * passive. */
int ora_system_eig_active(ora_flux_fn F, int ndim, int d, int *idx) {
  if (F == cattaneo_F) {
    for (int k = 0; k < ndim + 2; k++)
      idx[k] = k;
    idx[ndim + 2] = ndim + 2 + d;
    return ndim + 3;
  }
  return 0;
}

int ora_system_lookup(const char *name, int ndim, int *V, ora_flux_fn *F,
                      ora_ncp_fn *B, ora_src_fn *S, int *secondOrder) {
  if (ndim < 1 || ndim > 3)
    return -1;
  g_ndim = ndim;
  *F = 0;
  *B = 0;
  *S = 0;
  *secondOrder = 0;
  if (!strcmp(name, "euler")) {
    *V = ndim + 2;
    *F = euler_F;
  } else if (!strcmp(name, "cattaneo")) {
    *V = 2 * ndim + 3;
    *F = cattaneo_F;
    *S = cattaneo_S;
  } else if (!strcmp(name, "ncp")) {
    *V = 3;
    *F = ncp_F;
    *B = ncp_B;
    *S = ncp_S;
  } else if (!strcmp(name, "burgers2")) {
    *V = 1;
    *F = burgers2_F;
    *secondOrder = 1;
  } else {
    return -2;
  }
  return 0;
}

/* ---- FP32 twins, for the FP32 Newton sweeps of the mixed-precision
 * stiff predictor: the device systems instantiated with float
 * (pypde_gb300/csrc/systems.cuh, templates on the scalar type), in the same
 * operation order, every constant rounded to float before it is used. */
static float pow10_portable32(float x) {
  float y = x * (float)3.321928094887362;
  float n = floorf(y + 0.5f);
  float r = (y - n) * (float)0.6931471805599453;
  float p = (float)INV_FACT[16];
  for (int k = 15; k >= 0; k--)
    p = p * r + (float)INV_FACT[k];
  return ldexpf(p, (int)n);
}

static float euler_core32(float *out, const float *Q, int ndim, int d) {
  float r = Q[0];
  float ke = 0.0f;
  for (int i = 0; i < ndim; i++)
    ke += Q[1 + i] * Q[1 + i];
  float p = ((float)1.4 - 1.0f) * (Q[ndim + 1] - 0.5f * ke / r);
  float ud = Q[1 + d] / r;
  out[0] = Q[1 + d];
  for (int i = 0; i < ndim; i++)
    out[1 + i] = Q[1 + i] * ud;
  out[1 + d] += p;
  out[ndim + 1] = (Q[ndim + 1] + p) * ud;
  return p;
}

static void euler_F32(float *out, const float *Q, const float *dQ, int d) {
  (void)dQ;
  euler_core32(out, Q, g_ndim, d);
}

static void cattaneo_F32(float *out, const float *Q, const float *dQ, int d) {
  (void)dQ;
  int nd = g_ndim;
  float p = euler_core32(out, Q, nd, d);
  float T = p / Q[0];
  out[nd + 1] += Q[nd + 2 + d];
  for (int i = 0; i < nd; i++)
    out[nd + 2 + i] = 0.0f;
  out[nd + 2 + d] = 1.0f * T;
  out[2 * nd + 2] = 0.0f;
}

static void cattaneo_S32(float *out, const float *Q) {
  int nd = g_ndim;
  float inv_tau = pow10_portable32(-Q[2 * nd + 2]);
  for (int i = 0; i < nd + 2; i++)
    out[i] = 0.0f;
  for (int i = 0; i < nd; i++)
    out[nd + 2 + i] = -Q[nd + 2 + i] * inv_tau;
  out[2 * nd + 2] = 0.0f;
}

static float ncp_a32(int d) { return d == 0 ? 1.0f : (d == 1 ? 0.5f : 0.25f); }

static void ncp_F32(float *out, const float *Q, const float *dQ, int d) {
  (void)dQ;
  float a = ncp_a32(d);
  out[0] = a * (0.5f * Q[0] * Q[0]);
  out[1] = a * (Q[0] * Q[1]);
  out[2] = a * (Q[0] * Q[2]);
}

static void ncp_B32(float *out, const float *Q, int d) {
  float a = ncp_a32(d);
  for (int i = 0; i < 9; i++)
    out[i] = 0.0f;
  out[4] = a * Q[0];
  out[5] = a * (float)0.2;
  out[7] = a * (float)0.2;
  out[8] = a * Q[0];
}

static void ncp_S32(float *out, const float *Q) {
  out[0] = 0.0f;
  out[1] = (float)0.1 * (Q[2] - Q[1]);
  out[2] = (float)-0.1 * (Q[1] + Q[2]);
}

static void burgers2_F32(float *out, const float *Q, const float *dQ, int d) {
  out[0] = ncp_a32(d) * (0.5f * Q[0] * Q[0]) - (float)0.01 * dQ[d];
}

int ora_system_lookup32(const char *name, int ndim, ora_flux32_fn *F,
                        ora_ncp32_fn *B, ora_src32_fn *S) {
  if (ndim < 1 || ndim > 3)
    return -1;
  g_ndim = ndim;
  *F = 0;
  *B = 0;
  *S = 0;
  if (!strcmp(name, "euler")) {
    *F = euler_F32;
  } else if (!strcmp(name, "cattaneo")) {
    *F = cattaneo_F32;
    *S = cattaneo_S32;
  } else if (!strcmp(name, "ncp")) {
    *F = ncp_F32;
    *B = ncp_B32;
    *S = ncp_S32;
  } else if (!strcmp(name, "burgers2")) {
    *F = burgers2_F32;
  } else {
    return -2;
  }
  return 0;
}
