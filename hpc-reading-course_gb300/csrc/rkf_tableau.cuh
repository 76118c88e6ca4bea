// rkf_tableau.cuh -- Fehlberg's 4(5) Runge-Kutta pair (E. Fehlberg, NASA TR
// R-315, 1969), the tableau of PETSc's TSRK5F that the reference's ts_rk45
// (code/src/time_stepping/ts_rk.cpp:41-52) selects. One copy per translation
// unit in constant memory; every kernel that forms stage inputs, the candidate
// solution or the error estimate reads these.
#pragma once

namespace sbp {

// kRkfA[s][j]: weight of k_{j+1} in the input of stage s+1 (row 0 unused).
static __constant__ double kRkfA[6][5] = {
    {0, 0, 0, 0, 0},
    {1.0 / 4, 0, 0, 0, 0},
    {3.0 / 32, 9.0 / 32, 0, 0, 0},
    {1932.0 / 2197, -7200.0 / 2197, 7296.0 / 2197, 0, 0},
    {439.0 / 216, -8.0, 3680.0 / 513, -845.0 / 4104, 0},
    {-8.0 / 27, 2.0, -3544.0 / 2565, 1859.0 / 4104, -11.0 / 40}};
// 5th-order weights (the step) and the embedded 4th-order weights.
static __constant__ double kRkfB5[6] = {16.0 / 135, 0.0, 6656.0 / 12825, 28561.0 / 56430, -9.0 / 50, 2.0 / 55};
static __constant__ double kRkfB4[6] = {25.0 / 216, 0.0, 1408.0 / 2565, 2197.0 / 4104, -1.0 / 5, 0.0};

// Candidate u5 = u + h s5 and embedded u4 = u + h s4 with s5 = sum b5_j k_j,
// s4 = sum b4_j k_j left to right; the weights that are zero (b5_2 = b4_2 =
// b4_6 = 0) are skipped, which leaves every sum bit for bit unchanged.
// k2 is not read.
__device__ __forceinline__ void rkf_candidate(double u, double h, double k1, double k3, double k4, double k5, double k6,
                                              double& u5, double& u4) {
  double s5 = kRkfB5[0] * k1, s4 = kRkfB4[0] * k1;
  s5 = fma(kRkfB5[2], k3, s5);
  s4 = fma(kRkfB4[2], k3, s4);
  s5 = fma(kRkfB5[3], k4, s5);
  s4 = fma(kRkfB4[3], k4, s4);
  s5 = fma(kRkfB5[4], k5, s5);
  s4 = fma(kRkfB4[4], k5, s4);
  s5 = fma(kRkfB5[5], k6, s5);
  u5 = fma(h, s5, u);
  u4 = fma(h, s4, u);
}

// One term ((u5 - u4) / tol)^2 of the weighted error norm, tol = atol + rtol
// max(|u5|, |u4|); a zero tolerance contributes 0. The quotient uses 1/tol from
// the FP32 reciprocal refined by one Newton-Raphson step in FP64
// (r <- r + r (1 - tol r): the seed's relative error of about 2^-23 squares to
// about 2^-46), not an FP64 division, which costs several times as many FP64
// instructions on this part. Outside [1e-30, 1e30] (and for NaN) the plain
// quotient is used.
__device__ __forceinline__ double rkf_err_term(double u5, double u4, double atol, double rtol) {
  const double tol = atol + rtol * fmax(fabs(u5), fabs(u4));
  const double d = u5 - u4;
  if (tol > 1e-30 && tol < 1e30) {
    double r = (double)__frcp_rn((float)tol);
    r = fma(r, fma(-tol, r, 1.0), r);
    const double e = d * r;
    return e * e;
  }
  if (tol == 0.0) return 0.0;
  const double e = d / tol;
  return e * e;
}

}  // namespace sbp
