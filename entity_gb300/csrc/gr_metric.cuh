// Kerr metric in quasi-spherical Kerr-Schild coordinates (r_g = c = 1), 2D
// (r, theta): the device counterpart of metric::QKerrSchild<Dim::_2D>
// (src/metrics/qkerr_schild.h). A point's derived quantities (r, theta,
// sin, cos, Sigma, Delta, A, z) are formed once and shared by every
// component evaluated there; the component formulas are the reference's.
// Templated on the arithmetic type M so that the pusher can run near the
// horizon in double inside a single-precision build.
#pragma once

#include <cuda_runtime.h>

namespace pic {

__device__ __forceinline__ float  mexp(float x) { return expf(x); }
__device__ __forceinline__ double mexp(double x) { return exp(x); }
__device__ __forceinline__ void   msincos(float x, float* s, float* c) { sincosf(x, s, c); }
__device__ __forceinline__ void   msincos(double x, double* s, double* c) { sincos(x, s, c); }
__device__ __forceinline__ float  mcos(float x) { return cosf(x); }
__device__ __forceinline__ double mcos(double x) { return cos(x); }

// src/global/utils/numeric.h:91-103
constexpr double kPi          = 3.14159265358979323846;
constexpr double kInvPi       = 0.31830988618379067154;
constexpr double kPiSqr       = 9.86960440108935861882;
constexpr double kInvPiSqr    = 0.10132118364233777144;
constexpr double kSmallAngleGR = 1e-5;

template <typename M>
struct QKS {
  M   a, r0, h0, chi_min, eta_min, dchi, deta, dchi_inv, deta_inv;
  M   x2_small, x2_large;  // code x2 of theta = SMALL_ANGLE_GR and pi - SMALL_ANGLE_GR
  int small_angle;

  template <typename N>
  __host__ __device__ QKS<N> as() const {
    QKS<N> o;
    o.a = (N)a, o.r0 = (N)r0, o.h0 = (N)h0, o.chi_min = (N)chi_min, o.eta_min = (N)eta_min;
    o.dchi = (N)dchi, o.deta = (N)deta, o.dchi_inv = (N)dchi_inv, o.deta_inv = (N)deta_inv;
    o.x2_small = (N)x2_small, o.x2_large = (N)x2_large;
    o.small_angle = small_angle;
    return o;
  }

  // qkerr_schild.h:843-881 (h = 0 gives theta = eta)
  __device__ M dtheta_deta(M eta) const {
    if (fabs(h0) <= eps()) return (M)1;
    return (M)1 + (M)2 * h0 + (M)12.0 * h0 * (eta * (M)kInvPi) * ((eta * (M)kInvPi) - (M)1);
  }
  __device__ M eta2theta(M eta) const {
    if (fabs(h0) <= eps()) return eta;
    return eta + (M)2 * h0 * eta * ((M)kPi - (M)2 * eta) * ((M)kPi - eta) * (M)kInvPiSqr;
  }
  __device__ M dx_dt(M eta) const {
    if (fabs(h0) <= eps()) return deta;
    return deta * ((M)1 + (M)2 * h0 * (M)kInvPiSqr *
                            ((M)6 * (eta * eta) - (M)6 * (M)kPi * eta + (M)kPiSqr));
  }
  __device__ static M eps() { return sizeof(M) == 4 ? (M)1.1920929e-07 : (M)2.220446049250313e-16; }
  // theta clamped to [SMALL_ANGLE_GR, pi - SMALL_ANGLE_GR] in code units
  // (gr.hpp:352-364); the bounds' code coordinates come from the host
  __device__ M clamp_x2(M x2) const {
    const M th = eta2theta(x2 * deta + eta_min);
    const M small = (M)kSmallAngleGR, large = (M)kPi - small;
    if (th < small) return x2_small;
    if (th >= large) return x2_large;
    return x2;
  }
};

// a point (x1, x2) in code units with the quantities every component needs
template <typename M>
struct QPt {
  M chi, ex, r, eta, th, s, c, dtde, Sg, Dl, A, z;
};

template <typename M>
__device__ __forceinline__ QPt<M> qpt(const QKS<M>& m, M x1, M x2) {
  QPt<M> p;
  p.chi  = x1 * m.dchi + m.chi_min;
  p.ex   = mexp(p.chi);
  p.r    = m.r0 + p.ex;
  p.eta  = x2 * m.deta + m.eta_min;
  p.th   = m.eta2theta(p.eta);
  msincos(p.th, &p.s, &p.c);
  p.dtde = m.dtheta_deta(p.eta);
  const M a2 = m.a * m.a;
  p.Sg = p.r * p.r + a2 * (p.c * p.c);
  p.Dl = p.r * p.r - (M)2 * p.r + a2;
  const M rr = p.r * p.r + a2;
  p.A  = rr * rr - a2 * p.Dl * (p.s * p.s);
  p.z  = (M)2 * p.r / p.Sg;
  return p;
}

// h_ij (qkerr_schild.h:145-188), h^ij (194-233)
template <typename M> __device__ __forceinline__ M h_11(const QKS<M>& m, const QPt<M>& p) {
  return m.dchi * m.dchi * (p.ex * p.ex) * ((M)1 + p.z);
}
template <typename M> __device__ __forceinline__ M h_22(const QKS<M>& m, const QPt<M>& p) {
  return m.deta * m.deta * (p.dtde * p.dtde) * p.Sg;
}
template <typename M> __device__ __forceinline__ M h_33(const QKS<M>&, const QPt<M>& p) {
  return p.A * (p.s * p.s) / p.Sg;
}
template <typename M> __device__ __forceinline__ M h_13(const QKS<M>& m, const QPt<M>& p) {
  return -m.dchi * p.ex * m.a * ((M)1 + p.z) * (p.s * p.s);
}
template <typename M> __device__ __forceinline__ M h11(const QKS<M>& m, const QPt<M>& p) {
  return ((M)1 / (p.ex * p.ex) / (m.dchi * m.dchi)) * p.A / (p.Sg * (p.Sg + (M)2 * p.r));
}
template <typename M> __device__ __forceinline__ M h22(const QKS<M>& m, const QPt<M>& p) {
  return (M)1 / (p.Sg * (p.dtde * p.dtde) * (m.deta * m.deta));
}
template <typename M> __device__ __forceinline__ M h33(const QKS<M>&, const QPt<M>& p) {
  return (M)1 / (p.Sg * (p.s * p.s));
}
template <typename M> __device__ __forceinline__ M h13(const QKS<M>& m, const QPt<M>& p) {
  return ((M)1 / p.ex * m.dchi_inv) * m.a / p.Sg;
}
// lapse and shift (qkerr_schild.h:322-396)
template <typename M> __device__ __forceinline__ M alpha(const QKS<M>&, const QPt<M>& p) {
  return (M)1 / sqrt((M)1 + p.z);
}
template <typename M> __device__ __forceinline__ M beta1(const QKS<M>& m, const QPt<M>& p) {
  return ((M)1 / p.ex) * m.dchi_inv * p.z / ((M)1 + p.z);
}
template <typename M> __device__ __forceinline__ M dr_alpha(const QKS<M>& m, const QPt<M>& p) {
  const M dx_r = m.dchi * p.ex, dr_S = (M)2 * p.r * dx_r, al = alpha(m, p);
  return -(dx_r * p.Sg - p.r * dr_S) * (al * al * al) / (p.Sg * p.Sg);
}
template <typename M> __device__ __forceinline__ M dt_alpha(const QKS<M>& m, const QPt<M>& p) {
  const M dxdt = m.deta * ((M)1 + (M)2 * m.h0 * (M)kInvPiSqr *
                                    ((M)6 * (p.eta * p.eta) - (M)6 * (M)kPi * p.eta + (M)kPiSqr));
  const M dt_S = -(M)2 * (m.a * m.a) * p.s * p.c * dxdt;
  const M al   = alpha(m, p);
  return p.r * dt_S * (al * al * al) / (p.Sg * p.Sg);
}
template <typename M> __device__ __forceinline__ M dr_beta1(const QKS<M>& m, const QPt<M>& p) {
  const M dx_r = m.dchi * p.ex, dr_S = (M)2 * p.r * dx_r, q = p.Sg + (M)2 * p.r;
  return ((M)1 / p.ex) * m.dchi_inv * (M)2 * (dx_r * p.Sg - p.r * dr_S) / (q * q) -
         m.dchi * ((M)1 / p.ex) * m.dchi_inv * p.z / ((M)1 + p.z);
}
// qkerr_schild.h:471-500 (zero below machine epsilon)
template <typename M> __device__ __forceinline__ M dt_Sigma(const QKS<M>& m, const QPt<M>& p) {
  const M v = -(M)2 * (m.a * m.a) * p.s * p.c * m.dx_dt(p.eta);
  return fabs(v) <= QKS<M>::eps() ? (M)0 : v;
}
template <typename M> __device__ __forceinline__ M dt_A(const QKS<M>& m, const QPt<M>& p) {
  const M v = -(M)2 * (m.a * m.a) * p.s * p.c * p.Dl * m.dx_dt(p.eta);
  return fabs(v) <= QKS<M>::eps() ? (M)0 : v;
}
template <typename M> __device__ __forceinline__ M dt_beta1(const QKS<M>& m, const QPt<M>& p) {
  const M q = p.Sg * ((M)1 + p.z);
  return -((M)1 / p.ex) * m.dchi_inv * (M)2 * p.r * dt_Sigma(m, p) / (q * q);
}
// derivatives of h^ij (qkerr_schild.h:402-545)
template <typename M> __device__ __forceinline__ M dr_h11(const QKS<M>& m, const QPt<M>& p) {
  const M dx_r = m.dchi * p.ex, dr_S = (M)2 * p.r * dx_r, dr_D = (M)2 * dx_r * (p.r - (M)1);
  const M a2 = m.a * m.a;
  const M dr_A = (M)4 * p.r * dx_r * (p.r * p.r + a2) - a2 * (p.s * p.s) * dr_D;
  const M q = p.Sg * (p.Sg + (M)2 * p.r), e2 = (M)1 / (p.ex * p.ex);
  return (e2 / (m.dchi * m.dchi) *
          (q * dr_A - (M)2 * p.A * (p.r * dr_S + p.Sg * (dr_S + dx_r))) / (q * q)) -
         (M)2 * m.dchi * e2 / (m.dchi * m.dchi) * p.A / q;
}
template <typename M> __device__ __forceinline__ M dr_h22(const QKS<M>& m, const QPt<M>& p) {
  const M dr_S = (M)2 * p.r * (m.dchi * p.ex);
  return -dr_S / (p.Sg * p.Sg) / (m.deta * m.deta);
}
template <typename M> __device__ __forceinline__ M dr_h33(const QKS<M>& m, const QPt<M>& p) {
  const M dr_S = (M)2 * p.r * (m.dchi * p.ex);
  return -dr_S / (p.Sg * p.Sg) / (p.s * p.s);
}
template <typename M> __device__ __forceinline__ M dr_h13(const QKS<M>& m, const QPt<M>& p) {
  const M dr_S = (M)2 * p.r * (m.dchi * p.ex), ei = (M)1 / p.ex * m.dchi_inv;
  return -m.a * dr_S / (p.Sg * p.Sg) * ei - m.dchi * ei * m.a / p.Sg;
}
template <typename M> __device__ __forceinline__ M dt_h11(const QKS<M>& m, const QPt<M>& p) {
  const M q = p.Sg * (p.Sg + (M)2 * p.r);
  return (M)1 / (p.ex * p.ex) / (m.dchi * m.dchi) *
         (q * dt_A(m, p) - (M)2 * p.A * dt_Sigma(m, p) * (p.r + p.Sg)) / (q * q);
}
template <typename M> __device__ __forceinline__ M dt_h22(const QKS<M>& m, const QPt<M>& p) {
  return -dt_Sigma(m, p) / (p.Sg * p.Sg) / (m.deta * m.deta);
}
template <typename M> __device__ __forceinline__ M dt_h33(const QKS<M>& m, const QPt<M>& p) {
  const M q = p.Sg * p.s;
  return -(dt_Sigma(m, p) + (M)2 * p.c / p.s * p.Sg * m.dx_dt(p.eta)) / (q * q);
}
template <typename M> __device__ __forceinline__ M dt_h13(const QKS<M>& m, const QPt<M>& p) {
  return -m.a * dt_Sigma(m, p) / (p.Sg * p.Sg) * ((M)1 / p.ex * m.dchi_inv);
}
// qkerr_schild.h:552-582
template <typename M> __device__ __forceinline__ M sqrt_det_h(const QKS<M>& m, const QPt<M>& p) {
  return m.dchi * p.ex * p.dtde * m.deta * p.Sg * p.s * sqrt((M)1 + p.z);
}
template <typename M> __device__ __forceinline__ M sqrt_det_h_tilde(const QKS<M>& m,
                                                                    const QPt<M>& p) {
  return m.dchi * p.ex * p.dtde * m.deta * p.Sg * sqrt((M)1 + p.z);
}
// qkerr_schild.h:590-612
template <typename M> __device__ __forceinline__ M polar_area(const QKS<M>& m, M x1) {
  const M ex = mexp(x1 * m.dchi + m.chi_min), r = m.r0 + ex, rr = r * r + m.a * m.a;
  if (m.small_angle) {
    const M dth = m.eta2theta((M)0.5 * m.deta);
    return m.dchi * ex * rr * sqrt((M)1 + (M)2 * r / rr) * ((M)48 - dth * dth) * (dth * dth) /
           (M)384;
  }
  return m.dchi * ex * rr * sqrt((M)1 + (M)2 * r / rr) * ((M)1 - mcos(m.eta2theta((M)0.5 * m.deta)));
}

// the metric at one point, as the vector transforms and the pusher use it
template <typename M>
struct QMet {
  M h_11, h_22, h_33, h_13, h11, h22, h33, h13, alpha, beta1;
};
template <typename M>
__device__ __forceinline__ QMet<M> qmet(const QKS<M>& m, const QPt<M>& p) {
  QMet<M> g;
  g.h_11 = h_11(m, p), g.h_22 = h_22(m, p), g.h_33 = h_33(m, p), g.h_13 = h_13(m, p);
  g.h11 = h11(m, p), g.h22 = h22(m, p), g.h33 = h33(m, p), g.h13 = h13(m, p);
  g.alpha = alpha(m, p), g.beta1 = beta1(m, p);
  return g;
}

// vector transformations (qkerr_schild.h:662-760, 2D)
template <typename M>
__device__ __forceinline__ void d_to_u(const QMet<M>& g, const M* v, M* o) {
  const M a = v[0] * g.h11 + v[2] * g.h13, b = v[1] * g.h22, c = v[0] * g.h13 + v[2] * g.h33;
  o[0] = a, o[1] = b, o[2] = c;
}
template <typename M>
__device__ __forceinline__ void u_to_t(const QMet<M>& g, const M* v, M* o) {
  const M a = v[0] / sqrt(g.h11), b = v[1] * sqrt(g.h_22);
  const M c = v[2] * sqrt(g.h_33) + v[0] * g.h_13 / sqrt(g.h_33);
  o[0] = a, o[1] = b, o[2] = c;
}
template <typename M>
__device__ __forceinline__ void d_to_t(const QMet<M>& g, const M* v, M* o) {
  const M A0 = sqrt(g.h11);
  const M a = v[0] * A0 - v[2] * A0 * g.h_13 / g.h_33, b = v[1] / sqrt(g.h_22);
  const M c = v[2] / sqrt(g.h_33);
  o[0] = a, o[1] = b, o[2] = c;
}
template <typename M>
__device__ __forceinline__ void t_to_d(const QMet<M>& g, const M* v, M* o) {
  const M a = v[0] / sqrt(g.h11) + v[2] * g.h_13 / sqrt(g.h_33);
  const M b = v[1] * sqrt(g.h_22), c = v[2] * sqrt(g.h_33);
  o[0] = a, o[1] = b, o[2] = c;
}

}  // namespace pic
