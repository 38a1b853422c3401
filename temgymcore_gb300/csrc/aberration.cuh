// aberration.cuh - Krivanek wave aberration of AberratedLensKrivanek
// (components.py:177-215, aberrations.py:42-108) as a polynomial.
//
// The reference evaluates W(alpha, phi) = 1/2 a^2 B2 + 1/3 a^3 B3 + 1/4 a^4 B4
// + 1/5 a^5 B5 + 1/6 a^6 B6 with brackets B_n = sum_m C_{n-1,m} cos(m (phi -
// phi_{n-1,m})) at alpha = |u|, phi = arg u of the ideal (thin-lens) slopes
// u = (ax, ay), and its gradient through the polar chain rule.  Every term
// alpha^n cos(m (phi - phi0)) equals |u|^(n-m) Re(u^m e^(-i m phi0)) with n - m
// even, so W is a real polynomial of degree <= 6 in (ax, ay).  The host expands
// it once per component (float64) into monomial coefficients w[p][q] of
// ax^p ay^q (p + q <= 6); the gradient and Hessian are then exact polynomial
// derivatives, evaluated with Horner's rule and no atan2 / hypot / cos(m phi).
#pragma once

#include <cmath>
#include <cstring>

namespace tg {

// Triangle storage of a bivariate polynomial of degree <= D:
// coefficient of x^p y^q at tri_off(D, p) + q, p + q <= D.
__host__ __device__ constexpr int tri_off(int D, int p) { return p * (D + 1) - p * (p - 1) / 2; }
__host__ __device__ constexpr int tri_size(int D) { return (D + 1) * (D + 2) / 2; }

constexpr int kAberW = tri_size(6);   // 28: W
constexpr int kAberG = tri_size(5);   // 21: dW/dx, dW/dy
constexpr int kAberFloats = kAberW + 2 * kAberG;  // 70 per component (device float32)
constexpr int kMaxAber = 4;           // aberrated lenses per model
constexpr int kKrivanek = 25;         // KrivanekCoeffs fields (aberrations.py:5-31)

// Horner evaluation of a triangle polynomial of degree D.
template <int D, typename T>
__host__ __device__ __forceinline__ T tri_eval(const T* c, T x, T y) {
  T acc = T(0);
#pragma unroll
  for (int p = D; p >= 0; --p) {
    T inner = T(0);
#pragma unroll
    for (int q = D - p; q >= 0; --q) inner = inner * y + c[tri_off(D, p) + q];
    acc = acc * x + inner;
  }
  return acc;
}

// Value and both first partial derivatives of a triangle polynomial of
// degree D (Horner in x over Horner in y, derivatives carried along).
template <int D, typename T>
__host__ __device__ __forceinline__ void tri_eval_d(const T* c, T x, T y, T* v, T* vx, T* vy) {
  T a = T(0), ax = T(0), ay = T(0);
#pragma unroll
  for (int p = D; p >= 0; --p) {
    T q = T(0), qy = T(0);
#pragma unroll
    for (int r = D - p; r >= 0; --r) {
      qy = qy * y + q;
      q = q * y + c[tri_off(D, p) + r];
    }
    ax = ax * x + a;
    a = a * x + q;
    ay = ay * x + qy;
  }
  *v = a;
  *vx = ax;
  *vy = ay;
}

// ---- host: Krivanek coefficients -> monomials of W (float64)
// kc: C10, C12, phi12, C21, phi21, C23, phi23, C30, C32, phi32, C34, phi34,
//     C41, phi41, C43, phi43, C45, phi45, C50, C52, phi52, C54, phi54, C56, phi56
inline void aber_monomials(const double* kc, double w[kAberW]) {
  // dense (x^p y^q) scratch of degree <= 6
  double re[7][7], im[7][7];
  std::memset(w, 0, sizeof(double) * kAberW);
  // term: weight * s^j * Re(u^m e^(-i m phi0)), s = x^2 + y^2, u = x + i y
  auto add_term = [&](double weight, int j, int m, double C, double phi0) {
    if (C == 0.0) return;
    // u^m as a complex polynomial
    std::memset(re, 0, sizeof(re));
    std::memset(im, 0, sizeof(im));
    re[0][0] = 1.0;
    for (int k = 0; k < m; ++k) {  // multiply by (x + i y)
      double nr[7][7] = {}, ni[7][7] = {};
      for (int p = 0; p <= 6; ++p)
        for (int q = 0; p + q <= 6; ++q) {
          if (re[p][q] == 0.0 && im[p][q] == 0.0) continue;
          if (p + 1 + q <= 6) { nr[p + 1][q] += re[p][q]; ni[p + 1][q] += im[p][q]; }
          if (p + q + 1 <= 6) { nr[p][q + 1] -= im[p][q]; ni[p][q + 1] += re[p][q]; }
        }
      std::memcpy(re, nr, sizeof(re));
      std::memcpy(im, ni, sizeof(im));
    }
    // Re(u^m e^(-i m phi0)) = Re(u^m) cos(m phi0) + Im(u^m) sin(m phi0)
    const double cm = std::cos(m * phi0), sm = std::sin(m * phi0);
    double poly[7][7];
    for (int p = 0; p <= 6; ++p)
      for (int q = 0; q <= 6; ++q) poly[p][q] = (p + q <= 6) ? re[p][q] * cm + im[p][q] * sm : 0.0;
    for (int k = 0; k < j; ++k) {  // multiply by s = x^2 + y^2
      double np[7][7] = {};
      for (int p = 0; p <= 6; ++p)
        for (int q = 0; p + q <= 6; ++q) {
          if (poly[p][q] == 0.0) continue;
          if (p + 2 + q <= 6) np[p + 2][q] += poly[p][q];
          if (p + q + 2 <= 6) np[p][q + 2] += poly[p][q];
        }
      std::memcpy(poly, np, sizeof(poly));
    }
    for (int p = 0; p <= 6; ++p)
      for (int q = 0; p + q <= 6; ++q) w[tri_off(6, p) + q] += weight * C * poly[p][q];
  };
  const double h2 = 0.5, h3 = 1.0 / 3.0, h4 = 0.25, h5 = 0.2, h6 = 1.0 / 6.0;
  add_term(h2, 1, 0, kc[0], 0.0);       // C10
  add_term(h2, 0, 2, kc[1], kc[2]);     // C12
  add_term(h3, 1, 1, kc[3], kc[4]);     // C21
  add_term(h3, 0, 3, kc[5], kc[6]);     // C23
  add_term(h4, 2, 0, kc[7], 0.0);       // C30
  add_term(h4, 1, 2, kc[8], kc[9]);     // C32
  add_term(h4, 0, 4, kc[10], kc[11]);   // C34
  add_term(h5, 2, 1, kc[12], kc[13]);   // C41
  add_term(h5, 1, 3, kc[14], kc[15]);   // C43
  add_term(h5, 0, 5, kc[16], kc[17]);   // C45
  add_term(h6, 3, 0, kc[18], 0.0);      // C50
  add_term(h6, 2, 2, kc[19], kc[20]);   // C52
  add_term(h6, 1, 4, kc[21], kc[22]);   // C54
  add_term(h6, 0, 6, kc[23], kc[24]);   // C56
}

// d/dx and d/dy of a degree-6 triangle into degree-5 triangles.
inline void aber_gradient(const double w[kAberW], double gx[kAberG], double gy[kAberG]) {
  std::memset(gx, 0, sizeof(double) * kAberG);
  std::memset(gy, 0, sizeof(double) * kAberG);
  for (int p = 0; p <= 6; ++p)
    for (int q = 0; p + q <= 6; ++q) {
      const double c = w[tri_off(6, p) + q];
      if (p > 0) gx[tri_off(5, p - 1) + q] += p * c;
      if (q > 0) gy[tri_off(5, p) + q - 1] += q * c;
    }
}

// W, its gradient and Hessian at (x, y) from the monomials (float64; host
// ABCD and the per-beam field preparation).
__host__ __device__ inline void aber_eval_f64(const double* w, double x, double y, double* W,
                                              double* Wx, double* Wy, double* Hxx, double* Hxy,
                                              double* Hyy) {
  double xp[7], yp[7];
  xp[0] = yp[0] = 1.0;
  for (int i = 1; i <= 6; ++i) { xp[i] = xp[i - 1] * x; yp[i] = yp[i - 1] * y; }
  double v = 0.0, gx = 0.0, gy = 0.0, hxx = 0.0, hxy = 0.0, hyy = 0.0;
  for (int p = 0; p <= 6; ++p)
    for (int q = 0; p + q <= 6; ++q) {
      const double c = w[tri_off(6, p) + q];
      if (c == 0.0) continue;
      v += c * xp[p] * yp[q];
      if (p > 0) gx += c * p * xp[p - 1] * yp[q];
      if (q > 0) gy += c * q * xp[p] * yp[q - 1];
      if (p > 1) hxx += c * p * (p - 1) * xp[p - 2] * yp[q];
      if (p > 0 && q > 0) hxy += c * p * q * xp[p - 1] * yp[q - 1];
      if (q > 1) hyy += c * q * (q - 1) * xp[p] * yp[q - 2];
    }
  *W = v; *Wx = gx; *Wy = gy; *Hxx = hxx; *Hxy = hxy; *Hyy = hyy;
}

}  // namespace tg
