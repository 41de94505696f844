// tmk_fault.cuh -- FP64 fault-face friction solves, boundary-data updates and
// the Drucker-Prager return, one face (or cell) per thread.
//
// Friction laws follow ibcLinElast/RSIBCF.ChF (RSFAULTBCF, RSNEWTON, RSSETBND)
// and ibcLinElast/SWIBCF.ChF (SWFAULTBCF, SWSETBND) with the reference's
// operation order; plasticity follows srcLinElast/PlasticPhysicsF.ChF.
#pragma once
#include "tmk_device.cuh"

namespace tmk {

TMK_D double gaussian(double w, double r) { double q = r / w; return exp(-(0.5 * (q * q))); }
TMK_D double smoothfn(double w, double r) {
  if (r >= w) return 0.0;
  if (r <= 0) return 1.0;
  return exp(r * r / (r * r - w * w));
}
TMK_D double boxcar(double w, double r) { return (r >= w) ? 0.0 : 1.0; }

constexpr int RS_IMAX = 100;

// Rate-and-state parameters of one fault face: the scenario's a, b, L, or the
// face's own when the level carries per-face friction (an extension: the
// reference varies only a and Vw along x, by the linear ramp that RSSETF sets,
// ibcLinElast/RSIBCF.ChF:8-55).
struct RSFace { double a, b, L; };
TMK_D RSFace rs_face(const DevParams& P, const double* fric, int off, int stride) {
  if (!fric) return RSFace{P.rs_a, P.rs_b, P.rs_L};
  return RSFace{fric[off], fric[off + stride], fric[off + 2 * stride]};
}

// RSNEWTON (ibcLinElast/RSIBCF.ChF:336-401): bracketed Newton on the slip rate
// for  sn a asinh(V exp(psi/a)/(2V0)) + Zs/2 V = phi  on (0, phi/Zs).  The loop
// is bounded by IMAX; returns the iterations used.
TMK_D int rs_newton(const DevParams& P, double phi, double psi, double sn, double c_rs_a, double& V,
                    double& tau) {
  const double atolG = 2.220446049250313e-16 * 1e4;
  double Vmin = 0.0, Vmax = phi / P.Zs;
  if (V < Vmin || V > Vmax) V = (Vmin + Vmax) / 2.0;
  double alpha = sn * c_rs_a;
  double beta = exp(psi / c_rs_a) / (2.0 * P.rs_V0);
  double eta = 0.5 * P.Zs;
  double fval = alpha * asinh(beta * V) + eta * V - phi;
  int it;
  for (it = 1; it <= RS_IMAX; ++it) {
    if (fval < 0) Vmin = V; else Vmax = V;
    double dfval = alpha * beta / sqrt((beta * beta) * (V * V) + 1) + eta;
    double dV = -fval / dfval;
    V = V + dV;
    if (V < Vmin || V > Vmax) V = (Vmin + Vmax) / 2.0;
    fval = alpha * asinh(beta * V) + eta * V - phi;
    if (fabs(fval) <= atolG) break;
    if (fabs(dV) <= 0.0) break;
  }
  tau = alpha * asinh(beta * V);
  return it;
}

// RSFAULTBCF (ibcLinElast/RSIBCF.ChF:158-323) at one fault face; Wi, Wg: 22 comps.
TMK_D int rs_fault(const DevParams& P, const RSFace& fr, const double* Wi, double psi, double x, double* Wg) {
  const double Zs = P.Zs, Zp = P.Zp, lam = P.lam, G = P.G;
  double vx1 = Wi[0], vy1 = Wi[1], vz1 = Wi[2], sxx1 = Wi[3], syy1 = Wi[4], szz1 = Wi[5];
  double sxy1 = Wi[6], sxz1 = Wi[7], syz1 = Wi[8];
  double vx2 = Wi[11], vy2 = Wi[12], vz2 = Wi[13], sxx2 = Wi[14], syy2 = Wi[15], szz2 = Wi[16];
  double sxy2 = Wi[17], sxz2 = Wi[18], syz2 = Wi[19];
  double wpxy1 = -sxy1 - Zs * vx1;
  double wpyy1 = -syy1 - Zp * vy1;
  double wpxy2 = sxy2 - Zs * vx2;
  double wpyy2 = syy2 - Zp * vy2;
  double wpyz1 = 0.0, wpyz2 = 0.0;
  (void)syz1; (void)syz2;
  double tau_xy_0 = P.rs_nsig * gaussian(P.rs_r0, x);
  double tau_yz_0 = 0.0;
  double phi_xy = 0.5 * (wpxy2 - wpxy1) + tau_xy_0;
  double phi_yz = 0.5 * (wpyz2 - wpyz1) + tau_yz_0;
  double phi = sqrt(phi_xy * phi_xy + phi_yz * phi_yz);
  syy1 = -(wpyy1 - wpyy2) / 2.0;
  syy2 = -(wpyy1 - wpyy2) / 2.0;
  vy1 = -(wpyy1 + wpyy2) / 2.0 / Zp;
  vy2 = -(wpyy1 + wpyy2) / 2.0 / Zp;
  double V = sqrt((vx1 - vx2) * (vx1 - vx2) + (vz1 - vz2) * (vz1 - vz2));
  double c_ramp = fmin(1.0, fmax(0.0, (x - P.ramp_x) / P.ramp_w));
  double c_rs_a = fr.a + P.ramp_a * c_ramp;
  double tau;
  int it = rs_newton(P, phi, psi, -syy1, c_rs_a, V, tau);
  sxy1 = (phi_xy / phi) * tau - tau_xy_0;
  syz1 = (phi_yz / phi) * tau - tau_yz_0;
  double Vx = (phi_xy / phi) * V;
  double Vz = (phi_yz / phi) * V;
  vx1 = -(sxy1 + wpxy1) / Zs;
  vz1 = -(syz1 + wpyz1) / Zs;
  double SHF = -(vy1 - syy1) * lam / (lam + 2.0 * G);
  Wg[0] = vx1; Wg[1] = vy1; Wg[2] = vz1;
  Wg[3] = sxx1 + SHF; Wg[4] = syy1; Wg[5] = szz1 + SHF;
  Wg[6] = sxy1; Wg[7] = sxz1; Wg[8] = syz1;
  Wg[9] = 0.0; Wg[10] = 0.0;
  sxy2 = (phi_xy / phi) * tau - tau_xy_0;
  syz2 = (phi_yz / phi) * tau - tau_yz_0;
  vx2 = vx1 - Vx;
  vz2 = vz1 - Vz;
  SHF = -(vy2 - syy2) * lam / (lam + 2.0 * G);
  Wg[11] = vx2; Wg[12] = vy2; Wg[13] = vz2;
  Wg[14] = sxx2 + SHF; Wg[15] = syy2; Wg[16] = szz2 + SHF;
  Wg[17] = sxy2; Wg[18] = sxz2; Wg[19] = syz2;
  Wg[20] = 0.0; Wg[21] = 0.0;
  return it;
}

// RSSETBND (ibcLinElast/RSIBCF.ChF:61-151) for one face, B in/out (11 comps,
// strided).  When `final_` is false only psi is produced (the predictor's
// tmp data, of which the fault solve reads nothing else).  Returns the new
// psi (NaN is reported by the caller; the reference stops there).
TMK_D double rs_setbnd(const DevParams& P, const RSFace& fr, const double* U, double* B, int bstride, double dt,
                       double x, double time, bool final_) {
  double tau_xy_0 = P.rs_nsig * gaussian(P.rs_r0, x);
  double c_ramp = fmin(1.0, fmax(0.0, (x - P.ramp_x) / P.ramp_w));
  double c_rs_a = fr.a + P.ramp_a * c_ramp;
  double c_rs_Vw = P.rs_Vw + P.ramp_Vw * c_ramp;
  double Vx = U[0] - U[11];
  double Vz = U[2] - U[13];
  double V = sqrt(Vx * Vx + Vz * Vz);
  double psi = B[10 * bstride];
  double dPsi;
  if (P.state_law == 1) {
    // aging law (extension), exact at constant V over dt:
    // theta' = theta exp(-x) + dt (1-exp(-x))/x, x = V dt / L
    double xx = V * dt / fr.L;
    double phi1 = (xx > 1e-12) ? -expm1(-xx) / xx : 1.0 - 0.5 * xx;
    double q = (psi - P.rs_f0) / fr.b - xx;
    dPsi = P.rs_f0 + fr.b * log(exp(q) + (P.rs_V0 * dt / fr.L) * phi1);
  } else {
    double f = c_rs_a * asinh(V * exp(psi / c_rs_a) / (2.0 * P.rs_V0));
    double fss = P.rs_f0 - (fr.b - c_rs_a) * log(V / P.rs_V0);
    if (P.rs_fexp > 0.0) {
      double q = V / c_rs_Vw, q2 = q * q, q4 = q2 * q2, q8 = q4 * q4;
      fss = P.rs_fw + (fss - P.rs_fw) / pow(1.0 + q8, 0.125);
    }
    dPsi = psi - dt * (V / fr.L) * (f - fss);
  }
  if (final_) {
    double rt = B[9 * bstride];
    B[0] = Vx;
    B[1 * bstride] = Vz;
    B[2 * bstride] = V;
    B[3 * bstride] = U[6] + tau_xy_0;
    B[4 * bstride] = U[8] + 0.0;
    B[6 * bstride] = B[6 * bstride] + dt * Vx;
    B[7 * bstride] = B[7 * bstride] + dt * Vz;
    B[8 * bstride] = B[8 * bstride] + dt * V;
    if (rt > time && V > P.rs_thr) B[9 * bstride] = time;
    else if (rt > time) B[9 * bstride] = 1e10;
    B[5 * bstride] = U[4];
    B[10 * bstride] = dPsi;
  }
  return dPsi;
}

// ------------------------------------------------ mixed-form rate-and-state
// The same friction law for the mixed form, arranged for latency: on GB300 a
// dependent FP64 operation takes ~70 cycles and an FP64 division or
// transcendental several hundred, so the per-face chain of the two friction
// solves and boundary updates is the fault kernel's run time.  Here the
// quantities that depend only on the face (nucleation shear, ramped a, the
// reciprocals of a, b, L) are computed once per step beside the predictors,
// divisions by constants become products with reciprocals, reciprocals inside
// the Newton loop are Newton-Raphson refinements of an FP32 seed, the Newton
// step uses an FP32 reciprocal of the derivative (the iteration's fixed point
// is unchanged), and the solve starts from the slip rate of the states it is
// given.  Everything stays FP64; the results agree with the reference
// ordering to rounding and are checked by the rupture metrics.

// Reciprocal by two Newton-Raphson refinements r <- r + r (1 - x r) of an FP32
// seed (x within FP32 range and nonzero).
TMK_D double recip_nr(double x) {
  const double r0 = (double)__frcp_rn((float)x);
  const double r1 = fma(r0, fma(-x, r0, 1.0), r0);
  return fma(r1, fma(-x, r1, 1.0), r1);
}

struct RSFaceK {
  double tau0;    // nucleation shear at the face
  double a, inv_a, b, inv_b, inv_L;
  double c_Vw;    // ramped weakening velocity (slip law with fexp > 0)
};

TMK_D RSFaceK rs_face_k(const DevParams& P, const RSFace& fr, double x) {
  RSFaceK k;
  k.tau0 = P.rs_nsig * gaussian(P.rs_r0, x);
  const double c_ramp = fmin(1.0, fmax(0.0, (x - P.ramp_x) / P.ramp_w));
  k.a = fr.a + P.ramp_a * c_ramp;
  k.inv_a = 1.0 / k.a;
  k.b = fr.b;
  k.inv_b = 1.0 / fr.b;
  k.inv_L = 1.0 / fr.L;
  k.c_Vw = P.rs_Vw + P.ramp_Vw * c_ramp;
  return k;
}

// The friction equation of RSNEWTON solved for z = asinh(beta V) instead of V:
//   f(z) = alpha z + c sinh z - phi = 0,  c = eta / beta,  V = sinh(z)/beta,  tau = alpha z.
// f is smooth and monotone in z on the same bracket (0, asinh(beta phi/Zs)], so
// Newton converges in a few steps where the iteration in V creeps up through
// tens of decades; it starts from the guess V0 when that lies inside the
// bracket.  As in the reference, a root beyond the bracket's upper end
// V = phi/Zs yields that end.
//
// GB300 issues one FP64 warp instruction per 64 cycles on an SM sub-partition,
// so the iterations run in FP32 (c e^{+-z} as e^{+-z + ln c}, whose exponent
// stays below log(phi) inside the bracket), and one FP64 Newton step from the
// FP32 root finishes the solve: from a start within ~1e-5 of the root the step
// lands within ~1e-10, far below the FP32 volume arithmetic of the mixed form.
// V is then the FP64 c sinh z of that step's start advanced to its end to
// second order.  A step that is not small (an FP32 iteration that did not
// converge) hands the solve to the FP64 iteration from there.
TMK_D int rs_newton_zk(const DevParams& P, const RSFaceK& fk, double phi, double psi, double sn, double V0,
                       double& V, double& tau) {
  const double atolG = 2.220446049250313e-16 * 1e4;
  const double alpha = sn * fk.a;
  const double lb = psi * fk.inv_a - P.ln_2V0;        // ln beta, beta = e^(psi/a) / (2 V0)
  const double eta = 0.5 * P.Zs;
  const double Vmax = phi * P.inv_Zs;
  if (!(alpha > 0.0) || !(phi > 0.0) || !(lb > -600.0 && lb < 600.0) || !(P.rs_V0 > 0.0))
    return rs_newton(P, phi, psi, sn, fk.a, V, tau);
  const double lc = P.ln_halfZs - lb;                 // ln c
  // bracket end z_max = asinh(beta Vmax) (= ln(2 beta Vmax) to FP64 resolution past e^20)
  const double lbv = lb + log(Vmax);
  const double zmax = lbv > 20.0 ? 0.6931471805599453 + lbv : asinh(exp(lbv));
  if (alpha * zmax + eta * Vmax - phi <= 0.0) {      // root beyond the reference's bracket
    V = Vmax;
    tau = alpha * zmax;
    return RS_IMAX + 1;
  }
  // FP32 Newton from the guess
  const float a32 = (float)alpha, lc32 = (float)lc, phi32 = (float)phi, zmax32 = (float)zmax;
  float z;
  if (V0 > 0.0 && V0 < Vmax) {
    const float lg = (float)lb + logf((float)V0);    // ln(beta V0)
    z = fminf(lg > 9.f ? 0.6931472f + lg : asinhf(expf(lg)), zmax32);
  } else {
    z = fminf(phi32 / a32, zmax32);
  }
  int it;
  for (it = 1; it <= 30; ++it) {
    const float ep = expf(z + lc32), em = expf(lc32 - z);
    const float f = a32 * z + 0.5f * (ep - em) - phi32;
    const float dz = -f / (a32 + 0.5f * (ep + em));
    float zn = z + dz;
    if (zn < 0.f) zn = 0.5f * z;
    if (zn > zmax32) zn = 0.5f * (z + zmax32);
    z = zn;
    if (fabsf(dz) <= 2e-6f * fmaxf(1.f, z)) break;
  }
  // one FP64 Newton step
  const double z0 = (double)z;
  const double ep = exp(z0 + lc), em = exp(lc - z0);  // independent: issued together
  const double sh = 0.5 * (ep - em), ch = 0.5 * (ep + em);
  const double f = alpha * z0 + sh - phi;
  const double dz = -f * recip_nr(alpha + ch);
  if (fabs(dz) <= 1e-4 * fmax(1.0, z0) && z0 + dz >= 0.0 && z0 + dz <= zmax) {
    const double z1 = z0 + dz;
    V = (sh + ch * dz) * (2.0 * P.inv_Zs);            // c sinh(z1) / eta
    tau = alpha * z1;
    return it;
  }
  // the FP64 iteration from the FP32 result
  const double c = exp(lc);
  double zz = fmin(fmax(z0 + dz, 0.0), zmax);
  int jt;
  for (jt = 1; jt <= RS_IMAX; ++jt) {
    const double e = exp(zz), ie = zz > 20.0 ? 0.0 : recip_nr(e);   // e^-2z below FP64 resolution past 20
    const double f2 = alpha * zz + c * 0.5 * (e - ie) - phi;
    const double d2 = -f2 * (double)__frcp_rn((float)(alpha + c * 0.5 * (e + ie)));
    double zn = zz + d2;
    if (zn < 0.0) zn = 0.5 * zz;
    if (zn > zmax) zn = 0.5 * (zz + zmax);
    zz = zn;
    if (fabs(f2) <= atolG || fabs(d2) <= 1e-15 * fmax(1.0, zz)) break;
  }
  const double e = exp(zz + lc), ie = exp(lc - zz);
  V = 0.5 * (e - ie) * (2.0 * P.inv_Zs);
  tau = alpha * zz;
  return it + jt;
}

// RSFAULTBCF for the mixed form (same states in, same face states out).
TMK_D int rs_fault_k(const DevParams& P, const RSFaceK& fk, const double* Wi, double psi, double* Wg) {
  const double Zs = P.Zs, Zp = P.Zp;
  double vx1 = Wi[0], vy1 = Wi[1], vz1 = Wi[2], sxx1 = Wi[3], syy1 = Wi[4], szz1 = Wi[5];
  double sxy1 = Wi[6], sxz1 = Wi[7], syz1 = Wi[8];
  double vx2 = Wi[11], vy2 = Wi[12], vz2 = Wi[13], sxx2 = Wi[14], syy2 = Wi[15], szz2 = Wi[16];
  double sxy2 = Wi[17], sxz2 = Wi[18], syz2 = Wi[19];
  const double wpxy1 = -sxy1 - Zs * vx1, wpyy1 = -syy1 - Zp * vy1;
  const double wpxy2 = sxy2 - Zs * vx2, wpyy2 = syy2 - Zp * vy2;
  const double phi_xy = 0.5 * (wpxy2 - wpxy1) + fk.tau0;
  const double phi = fabs(phi_xy);      // the antiplane traction term is zero in 2-D
  syy1 = -0.5 * (wpyy1 - wpyy2);
  syy2 = syy1;
  vy1 = -0.5 * (wpyy1 + wpyy2) * P.inv_Zp;
  vy2 = vy1;
  const double dvx = vx1 - vx2, dvz = vz1 - vz2;
  double V = sqrt(dvx * dvx + dvz * dvz), tau;
  const int it = rs_newton_zk(P, fk, phi, psi, -syy1, V, V, tau);
  // phi_xy / phi: +-1, NaN when phi is zero or NaN (as the reference's quotient)
  const double sgn = phi > 0.0 ? copysign(1.0, phi_xy) : __longlong_as_double(0x7ff8000000000000ll);
  sxy1 = sgn * tau - fk.tau0;
  syz1 = 0.0 * tau;                     // (phi_yz / phi) tau - tau_yz_0 with phi_yz = tau_yz_0 = 0
  const double Vx = sgn * V, Vz = 0.0 * V;
  vx1 = -(sxy1 + wpxy1) * P.inv_Zs;
  vz1 = -(syz1 + 0.0) * P.inv_Zs;
  double SHF = -(vy1 - syy1) * P.lam_r;
  Wg[0] = vx1; Wg[1] = vy1; Wg[2] = vz1;
  Wg[3] = sxx1 + SHF; Wg[4] = syy1; Wg[5] = szz1 + SHF;
  Wg[6] = sxy1; Wg[7] = sxz1; Wg[8] = syz1;
  Wg[9] = 0.0; Wg[10] = 0.0;
  sxy2 = sxy1;
  syz2 = syz1;
  vx2 = vx1 - Vx;
  vz2 = vz1 - Vz;
  SHF = -(vy2 - syy2) * P.lam_r;
  Wg[11] = vx2; Wg[12] = vy2; Wg[13] = vz2;
  Wg[14] = sxx2 + SHF; Wg[15] = syy2; Wg[16] = szz2 + SHF;
  Wg[17] = sxy2; Wg[18] = sxz2; Wg[19] = syz2;
  Wg[20] = 0.0; Wg[21] = 0.0;
  (void)syz2;
  return it;
}

// RSSETBND for the mixed form (see rs_setbnd).
TMK_D double rs_setbnd_k(const DevParams& P, const RSFaceK& fk, const double* U, double* B, int bstride, double dt,
                         double time, bool final_) {
  const double Vx = U[0] - U[11];
  const double Vz = U[2] - U[13];
  const double V = sqrt(Vx * Vx + Vz * Vz);
  const double psi = B[10 * bstride];
  double dPsi;
  if (P.state_law == 1) {
    const double xx = V * dt * fk.inv_L;
    const double q = (psi - P.rs_f0) * fk.inv_b - xx;
    const double eq = exp(q), em1 = expm1(-xx);          // independent: issued together
    const double phi1 = (xx > 1e-12) ? -em1 / xx : 1.0 - 0.5 * xx;
    dPsi = P.rs_f0 + fk.b * log(eq + (P.rs_V0 * dt * fk.inv_L) * phi1);
  } else {
    const double f = fk.a * asinh(V * exp(psi * fk.inv_a) * P.inv_2V0);
    double fss = P.rs_f0 - (fk.b - fk.a) * log(V / P.rs_V0);
    if (P.rs_fexp > 0.0) {
      const double q = V / fk.c_Vw, q2 = q * q, q4 = q2 * q2, q8 = q4 * q4;
      fss = P.rs_fw + (fss - P.rs_fw) / pow(1.0 + q8, 0.125);
    }
    dPsi = psi - dt * (V * fk.inv_L) * (f - fss);
  }
  if (final_) {
    const double rt = B[9 * bstride];
    B[0] = Vx;
    B[1 * bstride] = Vz;
    B[2 * bstride] = V;
    B[3 * bstride] = U[6] + fk.tau0;
    B[4 * bstride] = U[8] + 0.0;
    B[6 * bstride] = B[6 * bstride] + dt * Vx;
    B[7 * bstride] = B[7 * bstride] + dt * Vz;
    B[8 * bstride] = B[8 * bstride] + dt * V;
    if (rt > time && V > P.rs_thr) B[9 * bstride] = time;
    else if (rt > time) B[9 * bstride] = 1e10;
    B[5 * bstride] = U[4];
    B[10 * bstride] = dPsi;
  }
  return dPsi;
}

// Out-of-line copies of the mixed-form solve and boundary update for a kernel
// that calls each twice (first pass and final): one copy of their code instead
// of one per call site.  The fault kernel runs few warps per SM along long
// chains of dependent FP64 operations, where instruction fetch stalls show.
static __device__ __noinline__ int rs_fault_k_ool(const DevParams& P, const RSFaceK& fk, const double* Wi,
                                                  double psi, double* Wg) {
  return rs_fault_k(P, fk, Wi, psi, Wg);
}
static __device__ __noinline__ double rs_setbnd_k_ool(const DevParams& P, const RSFaceK& fk, const double* U,
                                                      double* B, int bstride, double dt, double time, bool final_) {
  return rs_setbnd_k(P, fk, U, B, bstride, dt, time, final_);
}

// SWFAULTBCF (ibcLinElast/SWIBCF.ChF:79-267) at one fault face.  Side 2 is read
// and written at component offset P.sw_off (9 as in the reference source).
// Components the law does not write keep the values already in Wg.  Z3 (the
// 3-D fault plane): the nucleation patches and the friction box are products
// of x and z profiles, tau_0 += (tau valx) valz and box value valx valz
// (:118-126,175-180).
template <bool Z3 = false>
TMK_D void sw_fault(const DevParams& P, const double* Wi, double slip_total, double xcell, double* Wg,
                    double zcell = 0.0) {
  const int off = P.sw_off;
  const double Zs = P.Zs, Zp = P.Zp, lam = P.lam, G = P.G;
  double x = xcell - P.sw_fbc0;
  const double z = zcell - P.sw_fbc1;
  double vx1 = Wi[0], vy1 = Wi[1], vz1 = Wi[2], sxx1 = Wi[3], syy1 = Wi[4], szz1 = Wi[5];
  double sxy1 = Wi[6], sxz1 = Wi[7], syz1 = Wi[8];
  double vx2 = Wi[off + 0], vy2 = Wi[off + 1], vz2 = Wi[off + 2], sxx2 = Wi[off + 3], syy2 = Wi[off + 4];
  double szz2 = Wi[off + 5], sxy2 = Wi[off + 6], sxz2 = Wi[off + 7], syz2 = Wi[off + 8];
  double wpxy1 = -sxy1 - Zs * vx1;
  double wpyy1 = -syy1 - Zp * vy1;
  double wpyz1 = -syz1 - Zs * vz1;
  double wpxy2 = sxy2 - Zs * vx2;
  double wpyy2 = syy2 - Zp * vy2;
  double wpyz2 = syz2 - Zs * vz2;
  double tau_0 = 0;
  for (int ip = 0; ip < P.sw_np; ++ip) {
    double valx = smoothfn(P.sw_smooth, fabs(x - P.sw_xc[ip]) - P.sw_xw[ip]);
    if constexpr (Z3) {
      double valz = smoothfn(P.sw_smooth, fabs(z - P.sw_zc[ip]) - P.sw_zw[ip]);
      tau_0 = tau_0 + P.sw_tau[ip] * valx * valz;
    } else {
      tau_0 = tau_0 + P.sw_tau[ip] * valx;
    }
  }
  double a1 = 0.5 * (wpxy2 - wpxy1) + tau_0, a2 = 0.5 * (wpyz2 - wpyz1);
  double tau_lock = sqrt(a1 * a1 + a2 * a2);
  syy1 = -(wpyy1 - wpyy2) / 2.0;
  syy2 = -(wpyy1 - wpyy2) / 2.0;
  vy1 = -(wpyy1 + wpyy2) / 2.0 / Zp;
  vy2 = -(wpyy1 + wpyy2) / 2.0 / Zp;
  double valx = boxcar(P.sw_fbw0, fabs(x));
  double fric;
  if constexpr (Z3) {
    double valz = boxcar(P.sw_fbw1, fabs(z));
    fric = P.sw_fs * valx * valz + (1 - valx * valz) * P.sw_outside;
  } else {
    fric = P.sw_fs * valx + (1 - valx) * P.sw_outside;
  }
  fric = fric - (fric - P.sw_fd) * fmin(1.0, slip_total / P.sw_dw);
  double tau = fmin(tau_lock, -syy1 * fric) - tau_0;
  double phi_xy = 0.5 * (wpxy2 - wpxy1);
  double phi_yz = 0.5 * (wpyz2 - wpyz1);
  double phi = sqrt(phi_xy * phi_xy + phi_yz * phi_yz);
  sxy1 = (phi_xy / phi) * tau;
  syz1 = (phi_yz / phi) * tau;
  vx1 = -(sxy1 + wpxy1) / Zs;
  vz1 = -(syz1 + wpyz1) / Zs;
  double SHF = -(vy1 - syy1) * lam / (lam + 2.0 * G);
  Wg[0] = vx1; Wg[1] = vy1; Wg[2] = vz1;
  Wg[3] = sxx1 + SHF; Wg[4] = syy1; Wg[5] = szz1 + SHF;
  Wg[6] = sxy1; Wg[7] = sxz1; Wg[8] = syz1;
  sxy2 = (phi_xy / phi) * tau;
  syz2 = (phi_yz / phi) * tau;
  vx2 = (sxy2 - wpxy2) / Zs;
  vz2 = (syz2 - wpyz2) / Zs;
  SHF = -(vy2 - syy2) * lam / (lam + 2.0 * G);
  Wg[off + 0] = vx2; Wg[off + 1] = vy2; Wg[off + 2] = vz2;
  Wg[off + 3] = sxx2 + SHF; Wg[off + 4] = syy2; Wg[off + 5] = szz2 + SHF;
  Wg[off + 6] = sxy2; Wg[off + 7] = sxz2; Wg[off + 8] = syz2;
}

// SWSETBND (ibcLinElast/SWIBCF.ChF:32-72).  Predictor (final_=false): returns the
// predicted slip_total only.  Final: updates B in place; as in the reference's
// in-place call the rupture test reads the V just written.
TMK_D double sw_setbnd(const DevParams& P, const double* U, double* B, int bstride, double dt, double time,
                       bool final_) {
  const int off = P.sw_off;
  double vx = U[0] - U[off + 0];
  double vz = U[2] - U[off + 2];
  double V = sqrt((vx * vx + vz * vz));
  double st = B[7 * bstride] + dt * V;
  if (final_) {
    double rt = B[8 * bstride];
    B[0] = vx;
    B[1 * bstride] = vz;
    B[2 * bstride] = U[6];
    B[3 * bstride] = U[8];
    B[4 * bstride] = V;
    B[5 * bstride] = B[5 * bstride] + dt * vx;
    B[6 * bstride] = B[6 * bstride] + dt * vz;
    B[7 * bstride] = st;
    if (rt > time && V > P.sw_thr) B[8 * bstride] = time;
  }
  return st;
}

// The plasticity parameters (PLASTICSETF) and moduli in arithmetic T.
template <typename T>
struct PlasticK {
  T mu, beta, eta, pb, ph, G, K;
  TMK_HD void load(const DevParams& P) {
    mu = (T)P.p_mu; beta = (T)P.p_beta; eta = (T)P.p_eta; pb = (T)P.p_b; ph = (T)P.p_h;
    G = (T)P.G; K = (T)P.K;
  }
};

// PLASTICFLOW (srcLinElast/PlasticPhysicsF.ChF:74-181) on one side's stresses;
// returns whether the point yielded (else only p_lam, set to 0, changed).  The
// parameters come in T already: a pass over many cells converts them once (on
// GB300 each FP64-to-FP32 conversion uses the narrow FP64 pipe).
template <typename T>
TMK_D bool plastic_flow_k(const PlasticK<T>& c, T& sxx, T& syy, T& szz, T& sxy, T& sxz, T& syz, T& p_lam,
                          T& p_gam, T dt) {
  const T mu = c.mu, beta = c.beta, eta = c.eta, pb = c.pb, ph = c.ph;
  const T G = c.G, K = c.K;
  T sigma = (sxx + syy + szz) / T(3);
  T J2 = ((sxx - syy) * (sxx - syy) + (syy - szz) * (syy - szz) + (szz - sxx) * (szz - sxx)) / T(6) +
         sxy * sxy + sxz * sxz + syz * syz;
  T tau = sqrt(J2);
  T b = pb + p_gam * ph;
  T Y = tau - fmax(-mu * sigma + b, T(0));
  if (Y <= T(0)) { p_lam = T(0); return false; }
  p_lam = Y / (dt * (ph + G + mu * beta * K) + eta);
  p_gam = p_gam + dt * p_lam;
  T sig_e = sigma;
  tau = tau - dt * p_lam * G;
  sigma = sigma - dt * p_lam * K * beta;
  T factor = tau / (tau + dt * p_lam * G);
  sxx = sigma + factor * (sxx - sig_e);
  syy = sigma + factor * (syy - sig_e);
  szz = sigma + factor * (szz - sig_e);
  sxy = factor * sxy;
  sxz = factor * sxz;
  syz = factor * syz;
  return true;
}

// the same from the scenario's parameters
template <typename T>
TMK_D bool plastic_flow(const DevParams& P, T& sxx, T& syy, T& szz, T& sxy, T& sxz, T& syz, T& p_lam,
                        T& p_gam, T dt) {
  PlasticK<T> c;
  c.load(P);
  return plastic_flow_k<T>(c, sxx, syy, szz, sxy, sxz, syz, p_lam, p_gam, dt);
}

}  // namespace tmk
