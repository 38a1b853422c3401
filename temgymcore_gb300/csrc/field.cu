// field.cu - Gaussian-beamlet detector field (gaussian.py:225-369).
//
// Kernels
//   k_field_prep        one thread per beam, float64: traces the central ray
//                       and composes its 5x5 ABCD (the reference's
//                       vmap(jacobian(run_to_end))), forms Q1^-1, Q2^-1, the
//                       amplitude prefactor and the per-pixel polynomial
//                       (field_common.cuh), reduces k*pl exactly mod 2*pi.
//   k_field_direct<L>   fast direct sum (any Q2, the astigmatic case): each
//                       thread owns a strip of L pixels of one row; per beam it
//                       evaluates the exact fixed-point phase and the envelope
//                       at the strip start, then walks the strip with two
//                       complex multiplications per pixel (a geometric
//                       recurrence: the phase/envelope are quadratic in col).
//   k_field_direct_f64  the all-float64 comparator: evaluates the polynomial,
//                       sin/cos and exp in float64 for every (beam, pixel).
//   k_field_operands    separable case: per-beam row and column phasor
//                       factors split into bf16 hi + lo planes for the
//                       tensor-core GEMM (field_gemm.cu).
//   k_field_reduce      deterministic sum of per-chunk partial images.
#include <cuda_bf16.h>
#include <math.h>

#include <cstring>

#include "field_common.cuh"
#include "tg_common.cuh"

TG_DEFINE_ERROR_WORD(field)

namespace tg {

struct cd {
  double re, im;
};
__device__ __forceinline__ cd C(double r, double i = 0.0) { return cd{r, i}; }
__device__ __forceinline__ cd operator+(cd a, cd b) { return cd{a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ cd operator-(cd a, cd b) { return cd{a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ cd operator*(cd a, cd b) {
  return cd{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
__device__ __forceinline__ cd operator*(double s, cd a) { return cd{s * a.re, s * a.im}; }
__device__ __forceinline__ cd cdiv(cd a, cd b) {
  double d = b.re * b.re + b.im * b.im;
  const double inv = 1.0 / d;  // one float64 division (slow on GB300) instead of two
  return cd{(a.re * b.re + a.im * b.im) * inv, (a.im * b.re - a.re * b.im) * inv};
}
// principal square root (branch cut on the negative real axis, sign of imag kept)
__device__ __forceinline__ cd csqrt_(cd z) {
  double r = hypot(z.re, z.im);
  if (z.re >= 0.0) {
    double t = sqrt(0.5 * (r + z.re));
    return cd{t, t > 0.0 ? z.im / (2.0 * t) : z.im};
  }
  double t = sqrt(0.5 * (r - z.re));
  return cd{fabs(z.im) / (2.0 * t), copysign(t, z.im)};
}

struct cm2 {
  cd a, b, c, d;  // [[a, b], [c, d]]
};
__device__ __forceinline__ cm2 mm(cm2 x, cm2 y) {
  return cm2{x.a * y.a + x.b * y.c, x.a * y.b + x.b * y.d, x.c * y.a + x.d * y.c,
             x.c * y.b + x.d * y.d};
}
__device__ __forceinline__ cm2 madd(cm2 x, cm2 y) { return cm2{x.a + y.a, x.b + y.b, x.c + y.c, x.d + y.d}; }
__device__ __forceinline__ cm2 inv2c(cm2 m) {  // explicit inverse: inf/nan when singular
  cd det = m.a * m.d - m.b * m.c;
  cd one = C(1.0);
  cd r = cdiv(one, det);
  return cm2{m.d * r, C(0.0) - m.b * r, C(0.0) - m.c * r, m.a * r};
}
__device__ __forceinline__ double nz(double v) { return isfinite(v) ? v : 0.0; }
__device__ __forceinline__ cm2 nan_to_num(cm2 m) {
  return cm2{C(nz(m.a.re), nz(m.a.im)), C(nz(m.b.re), nz(m.b.im)), C(nz(m.c.re), nz(m.c.im)),
             C(nz(m.d.re), nz(m.d.im))};
}
__device__ __forceinline__ cm2 real2(double a, double b, double c, double d) {
  return cm2{C(a), C(b), C(c), C(d)};
}

// 2*pi as a sum of two doubles; k*pl reduced exactly (FMA TwoProduct).
__device__ __forceinline__ double reduce_phase(double k, double pl) {
  const double C1 = 6.283185307179586, C2 = 2.4492935982947064e-16;
  double p = k * pl;
  double e = fma(k, pl, -p);
  double n = rint(p * 0.15915494309189535);
  double r = fma(-n, C1, p);
  r = fma(-n, C2, r);
  return r + e;
}

// frac(v / 2pi) as a 64-bit fixed-point turn.
__device__ __forceinline__ uint64_t to_turns(double rad) {
  double t = rad * 0.15915494309189535;
  double hi = t - floor(t);  // [0, 1)
  // refine: t has relative error ~1e-16; the fraction keeps 53 bits
  double f = hi * 18446744073709551616.0;
  if (!(f < 18446744073709551615.0)) f = 0.0;  // 1.0 - eps rounding or NaN
  return (uint64_t)f;
}

struct PrepArgs {
  int64_t n;
  const double *x, *y, *dx, *dy;
  double z;
  const double* pl;
  const float* amp;  // complex64 pairs
  const double *waist, *radii;
  const double* wl;
  double wl_scalar;
  const double* theta;
  PixMap pm;
  BeamFast* fast;
  BeamF64* f64;
  int32_t* flags;  // [0]: non-separable beams seen
  int32_t input_plane;  // 1: field of the beams in their own plane (no model)
  int32_t unit_amp;     // 1: every amplitude taken as 1 (the field adjoint's records)
};

__global__ void __launch_bounds__(128)
k_field_prep(const __grid_constant__ DModel M, const __grid_constant__ PrepArgs A) {
  int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= A.n) return;
  // ---- central ray + 5x5 ABCD (rows x, y, dx, dy, 1)
  double m[5][5];
#pragma unroll
  for (int i = 0; i < 5; ++i)
#pragma unroll
    for (int j = 0; j < 5; ++j) m[i][j] = (i == j) ? 1.0 : 0.0;
  double x = A.x[b], y = A.y[b], dx = A.dx[b], dy = A.dy[b];
  const double x0 = x, y0 = y, dx0 = dx, dy0 = dy;
  for (int s = 0; s < M.n; ++s) {
    const DStep& st = M.s[s];
    switch (st.kind) {
      case D_FREE: {
        double d = st.a[0];
#pragma unroll
        for (int j = 0; j < 5; ++j) {
          m[0][j] += d * m[2][j];
          m[1][j] += d * m[3][j];
        }
        x += dx * d;
        y += dy * d;
      } break;
      case D_LENS: {  // a[1] = 1/f from the host: no float64 division per element
        const double k = st.a[1];
#pragma unroll
        for (int j = 0; j < 5; ++j) {
          m[2][j] = fma(-m[0][j], k, m[2][j]);
          m[3][j] = fma(-m[1][j], k, m[3][j]);
        }
        dx = fma(-x, k, dx);
        dy = fma(-y, k, dy);
      } break;
      case D_SHIFT:
        m[0][4] += st.a[0]; m[1][4] += st.a[1]; m[2][4] += st.a[2]; m[3][4] += st.a[3];
        x += st.a[0]; y += st.a[1]; dx += st.a[2]; dy += st.a[3];
        break;
      case D_BIPRISM: {
        double sg = x > 0.0 ? 1.0 : (x < 0.0 ? -1.0 : 0.0);
        m[2][4] += st.a[0] * sg;
        dx += st.a[0] * sg;
      } break;
      case D_ABER: {  // Jacobian (I - H/f) [-I/f, I] at the ideal slopes; no offset column
        const double k1 = 1.0 / st.a[0];
        const double ux = dx - x * k1, uy = dy - y * k1;
        double W, Wx, Wy, Hxx, Hxy, Hyy;
        aber_eval_f64(M.aber[st.pad], ux, uy, &W, &Wx, &Wy, &Hxx, &Hxy, &Hyy);
        const double a20 = -k1 + Hxx * k1 * k1, a21 = Hxy * k1 * k1, a22 = 1.0 - Hxx * k1, a23 = -Hxy * k1;
        const double a30 = Hxy * k1 * k1, a31 = -k1 + Hyy * k1 * k1, a32 = -Hxy * k1, a33 = 1.0 - Hyy * k1;
#pragma unroll
        for (int j = 0; j < 5; ++j) {
          const double r0 = m[0][j], r1 = m[1][j], r2 = m[2][j], r3 = m[3][j];
          m[2][j] = a20 * r0 + a21 * r1 + a22 * r2 + a23 * r3;
          m[3][j] = a30 * r0 + a31 * r1 + a32 * r2 + a33 * r3;
        }
        dx = ux - Wx * k1;
        dy = uy - Wy * k1;
      } break;
      case D_ROTATE: {
        double c = st.a[0], sn = st.a[1];
#pragma unroll
        for (int j = 0; j < 5; ++j) {
          double r0 = m[0][j], r1 = m[1][j], r2 = m[2][j], r3 = m[3][j];
          m[0][j] = c * r0 - sn * r1;
          m[1][j] = sn * r0 + c * r1;
          m[2][j] = c * r2 - sn * r3;
          m[3][j] = sn * r2 + c * r3;
        }
        double nx = x * c - y * sn, ny = x * sn + y * c;
        double ndx = dx * c - dy * sn, ndy = dx * sn + dy * c;
        x = nx; y = ny; dx = ndx; dy = ndy;
      } break;
      default:
        break;
    }
  }
  const cm2 Am = real2(m[0][0], m[0][1], m[1][0], m[1][1]);
  const cm2 Bm = real2(m[0][2], m[0][3], m[1][2], m[1][3]);
  const cm2 Cm = real2(m[2][0], m[2][1], m[3][0], m[3][1]);
  const cm2 Dm = real2(m[2][2], m[2][3], m[3][2], m[3][3]);
  const double e0x = m[0][4], e0y = m[1][4], fx = m[2][4], fy = m[3][4];
  // ---- Q1^-1 = R diag(1/qx, 1/qy) R^T (gaussian.py:138-177)
  const double wl = A.wl ? A.wl[b] : A.wl_scalar;
  const double wx = A.waist[2 * b], wy = A.waist[2 * b + 1];
  const double Rx = A.radii[2 * b], Ry = A.radii[2 * b + 1];
  const double PI = 3.141592653589793;
  cd qx = C(isinf(Rx) ? 0.0 : -1.0 / Rx, wl / (PI * wx * wx));
  cd qy = C(isinf(Ry) ? 0.0 : -1.0 / Ry, wl / (PI * wy * wy));
  const double th = A.theta ? A.theta[b] : 0.0;
  double cth, sth;
  sincos(th, &sth, &cth);
  // R D R^T with R = [[c, -s], [s, c]]
  cm2 Q1i{cth * cth * qx + sth * sth * qy, cth * sth * qx - sth * cth * qy,
          sth * cth * qx - cth * sth * qy, sth * sth * qx + cth * cth * qy};
  const cd amp = A.unit_amp ? C(1.0) : C((double)A.amp[2 * b], (double)A.amp[2 * b + 1]);
  const double k = 2.0 * PI / wl;
  const double hk = 0.5 * k;
  // Phase polynomial (k/2) (s^T S s + L.s + c0) of the pixel position r,
  // s = r - origin, and the prefactor pref:
  cd Sxx, Syy, Sxy, Lx, Ly, c0, pref;
  double ox, oy;
  if (A.input_plane) {
    // the beams in their own plane (gaussian.py:402-409): s = r1 - r1m,
    // S = Q1^-1, L = 2 theta1m, no constant, pref = amplitude
    Sxx = Q1i.a; Syy = Q1i.d; Sxy = 0.5 * (Q1i.b + Q1i.c);
    Lx = C(2.0 * dx0); Ly = C(2.0 * dy0);
    c0 = C(0.0);
    pref = amp;
    ox = x0; oy = y0;
  } else {
    // ---- Q2^-1 = (A + B Q1i)^-1 (C + D Q1i)   (gaussian.py:92-96)
    const cm2 denom = madd(Am, mm(Bm, Q1i));
    const cm2 Q2 = mm(inv2c(denom), madd(Cm, mm(Dm, Q1i)));
    const cm2 Binv = nan_to_num(inv2c(Bm));
    const cm2 Q1 = nan_to_num(inv2c(Q1i));
    // central ray at output: r2m = A r1m + B theta1m
    const double r2mx = m[0][0] * x0 + m[0][1] * y0 + m[0][2] * dx0 + m[0][3] * dy0;
    const double r2my = m[1][0] * x0 + m[1][1] * y0 + m[1][2] * dx0 + m[1][3] * dy0;
    const cd det = denom.a * denom.d - denom.b * denom.c;
    pref = cdiv(amp, csqrt_(det));
    const cm2 ABinv = mm(Am, Binv);
    const cm2 P = mm(Q1, inv2c(mm(Bm, madd(mm(Am, Q1), Bm))));
    // quadratic (symmetric part), linear and constant terms in s = r2 - e
    Sxx = Q2.a; Syy = Q2.d; Sxy = 0.5 * (Q2.b + Q2.c);
    // Binv^T r1m and P^T r2m
    const cd bx = Binv.a * C(x0) + Binv.c * C(y0), by = Binv.b * C(x0) + Binv.d * C(y0);
    const cd px_ = P.a * C(r2mx) + P.c * C(r2my), py_ = P.b * C(r2mx) + P.d * C(r2my);
    Lx = C(2.0 * fx) - 2.0 * bx + 2.0 * px_;
    Ly = C(2.0 * fy) - 2.0 * by + 2.0 * py_;
    const cd q1 = C(x0) * (ABinv.a * C(x0) + ABinv.b * C(y0)) + C(y0) * (ABinv.c * C(x0) + ABinv.d * C(y0));
    const cd q2 = C(r2mx) * (P.a * C(r2mx) + P.b * C(r2my)) + C(r2my) * (P.c * C(r2mx) + P.d * C(r2my));
    c0 = q1 - q2;
    ox = e0x; oy = e0y;
  }
  // pixel map: s = s0 + row*u + col*v
  const double s0x = A.pm.t[5] - ox, s0y = A.pm.t[2] - oy;
  const double ux = A.pm.t[3], uy = A.pm.t[0], vx = A.pm.t[4], vy = A.pm.t[1];
  auto quad = [&](double ax, double ay, double bx2, double by2) -> cd {  // a^T S b
    return C(ax * bx2) * Sxx + C(ay * by2) * Syy + C(ax * by2 + ay * bx2) * Sxy;
  };
  cd k_cc = hk * quad(vx, vy, vx, vy);
  cd k_rr = hk * quad(ux, uy, ux, uy);
  cd k_rc = hk * (2.0 * quad(ux, uy, vx, vy));
  cd k_c = hk * (2.0 * quad(s0x, s0y, vx, vy) + C(vx) * Lx + C(vy) * Ly);
  cd k_r = hk * (2.0 * quad(s0x, s0y, ux, uy) + C(ux) * Lx + C(uy) * Ly);
  cd k_0 = hk * (quad(s0x, s0y, s0x, s0y) + C(s0x) * Lx + C(s0y) * Ly + c0);
  const double ph_off = reduce_phase(k, A.pl[b]);
  const double arg_pref = atan2(pref.im, pref.re);
  const double lnamp = log(hypot(pref.re, pref.im));
  // ---- float64 record
  BeamF64 r64;
  r64.re[0] = k_cc.re; r64.re[1] = k_rr.re; r64.re[2] = k_rc.re;
  r64.re[3] = k_c.re; r64.re[4] = k_r.re; r64.re[5] = k_0.re;
  r64.im[0] = k_cc.im; r64.im[1] = k_rr.im; r64.im[2] = k_rc.im;
  r64.im[3] = k_c.im; r64.im[4] = k_r.im; r64.im[5] = k_0.im;
  r64.ph0 = ph_off + arg_pref;
  r64.lnamp = lnamp;
  r64.pad[0] = r64.pad[1] = 0.0;
  A.f64[b] = r64;
  // ---- fast record: fixed-point phase, centred float32 envelope
  BeamFast f;
  f.p_cc = to_turns(k_cc.re);
  f.p_rr = to_turns(k_rr.re);
  f.p_rc = to_turns(k_rc.re);
  f.p_c = to_turns(k_c.re);
  f.p_r = to_turns(k_r.re);
  f.p_0 = to_turns(k_0.re) + to_turns(ph_off) + to_turns(arg_pref);
  // envelope: log-amp = lnamp - Im Phi(row, col)
  const double bcc = k_cc.im, brr = k_rr.im, brc = k_rc.im, bc = k_c.im, br = k_r.im;
  double rs, cs;
  const double hdet = 4.0 * brr * bcc - brc * brc;  // Hessian [[2brr, brc], [brc, 2bcc]]
  if (brr > 0.0 && hdet > 0.0) {
    rs = (-2.0 * bcc * br + brc * bc) / hdet;
    cs = (-2.0 * brr * bc + brc * br) / hdet;
    if (!(fabs(rs) < 1e7 && fabs(cs) < 1e7)) { rs = 0.5 * (A.pm.h - 1); cs = 0.5 * (A.pm.w - 1); }
  } else {
    rs = 0.5 * (A.pm.h - 1);
    cs = 0.5 * (A.pm.w - 1);
  }
  rs = rint(rs * 16.0) / 16.0;  // exactly representable centre in float32
  cs = rint(cs * 16.0) / 16.0;
  const double imphi_c = bcc * cs * cs + brr * rs * rs + brc * rs * cs + bc * cs + br * rs + k_0.im;
  f.r0 = (float)rs;
  f.c0 = (float)cs;
  f.e0 = (float)(lnamp - imphi_c);
  f.b_cc = (float)bcc;
  f.b_rr = (float)brr;
  f.b_rc = (float)brc;
  f.l_c = (float)(2.0 * bcc * cs + brc * rs + bc);
  f.l_r = (float)(2.0 * brr * rs + brc * cs + br);
  {
    double ang = 2.0 * k_cc.re;  // radians: step of the phase increment
    double mag = exp(-2.0 * bcc);
    double sa, ca;
    sincos(ang, &sa, &ca);
    f.rho_re = (float)(mag * ca);
    f.rho_im = (float)(mag * sa);
  }
  A.fast[b] = f;
  if (k_rc.re != 0.0 || k_rc.im != 0.0) atomicOr(A.flags, 1);
}

// ---------------------------------------------------------------- direct
constexpr int kDirThreads = 256;
constexpr int kBeamBatch = 64;

struct DirArgs {
  const BeamFast* beams;
  int64_t n;
  int64_t chunk;       // beams per blockIdx.y
  int32_t h, w;
  int32_t tile_rows;   // rows per tile
  int32_t strips_x;    // strips per tile row
  float2* out;         // [gridDim.y][h][w] partials (or the image if gridDim.y == 1)
};

// Per (beam, strip) the log-amplitude decides how the strip is summed: skip
// when it stays below kDirSkipLog (e^-60 of a unit amplitude), the geometric
// recurrence while its start and per-step ratios stay inside float32 range
// (|log| < 80), otherwise a per-pixel evaluation.
constexpr float kDirSkipLog = -60.f;
constexpr float kDirRecurMax = 80.f;
// Strips of 32 pixels with the recurrence restarted exactly after 16: the
// per-(beam, strip) set-up (exact phase, envelope range) is paid once per 32
// pixels and the float32 recurrence error stays that of 16 steps.  Measured
// at 16,384 beams, 512^2: 16-pixel strips 2.25 ms (4.5e-6 of the float64
// kernel), 32 without restart 1.81 ms (1.2e-5), 32 with restart 2.01 ms
// (4.0e-6), 24 pixels 2.46 ms.
constexpr int kDirRestart = 16;  // pixels between exact restarts of the recurrence

template <int L>
__global__ void __launch_bounds__(kDirThreads)
k_field_direct(const __grid_constant__ DirArgs A) {
  __shared__ BeamFast sb[kBeamBatch];
  const int tiles_x = (A.w + A.strips_x * L - 1) / (A.strips_x * L);
  const int tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
  const int lr = threadIdx.x / A.strips_x, ls = threadIdx.x % A.strips_x;
  const int row = ty * A.tile_rows + lr;
  const int col0 = (tx * A.strips_x + ls) * L;
  const int64_t b0 = (int64_t)blockIdx.y * A.chunk;
  int64_t b1 = b0 + A.chunk;
  if (b1 > A.n) b1 = A.n;
  float are[L], aim[L];
#pragma unroll
  for (int j = 0; j < L; ++j) { are[j] = 0.f; aim[j] = 0.f; }
  const uint64_t urow = (uint64_t)row, ucol = (uint64_t)col0;
  const uint64_t urow2 = urow * urow, ucol2 = ucol * ucol, urc = urow * ucol;
  const uint64_t ustep = 2 * ucol + 1;
  for (int64_t bb = b0; bb < b1; bb += kBeamBatch) {
    const int nb = (int)((b1 - bb) < kBeamBatch ? (b1 - bb) : kBeamBatch);
    __syncthreads();
    {
      const uint4* src = reinterpret_cast<const uint4*>(A.beams + bb);
      uint4* dst = reinterpret_cast<uint4*>(sb);
      const int words = nb * (int)(sizeof(BeamFast) / 16);
      for (int i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    for (int k = 0; k < nb; ++k) {
      const BeamFast& B = sb[k];
      // exact phase at the strip start and its first column step
      uint64_t th = B.p_cc * ucol2 + B.p_rr * urow2 + B.p_rc * urc + B.p_c * ucol + B.p_r * urow + B.p_0;
      uint64_t dth = B.p_cc * ustep + B.p_rc * urow + B.p_c;
      const float dr = (float)row - B.r0, dc = (float)col0 - B.c0;
      const float la = B.e0 - (B.b_cc * dc * dc + B.b_rr * dr * dr + B.b_rc * dr * dc + B.l_c * dc + B.l_r * dr);
      const float dla = -(B.b_cc * (2.f * dc + 1.f) + B.b_rc * dr + B.l_c);
      // log-amplitude along the strip: la(j) = la + j dla - b_cc j (j - 1)
      const float jl = (float)(L - 1);
      const float la_end = la + jl * dla - B.b_cc * jl * (jl - 1.f);
      const float dla_end = dla - 2.f * B.b_cc * (jl - 1.f);
      float jv = B.b_cc > 0.f ? 0.5f + dla / (2.f * B.b_cc) : (dla > 0.f ? jl : 0.f);
      jv = fminf(fmaxf(jv, 0.f), jl);
      const float la_max = fmaxf(fmaxf(la, la_end), la + jv * dla - B.b_cc * jv * (jv - 1.f));
      if (!(la_max > kDirSkipLog)) continue;  // below e^-60 of unit amplitude everywhere (or NaN)
      // the log-amplitude and its column step at offset d from the centre,
      // evaluated directly (as la itself) where values are formed: summing
      // la + j dla - b_cc j (j - 1) over a 32-pixel strip cancels terms of a
      // few hundred down to the value and costs float32 accuracy
      auto la_at = [&](float d) {
        return B.e0 - (B.b_cc * d * d + B.b_rr * dr * dr + B.b_rc * dr * d + B.l_c * d + B.l_r * dr);
      };
      auto dla_at = [&](float d) { return -(B.b_cc * (2.f * d + 1.f) + B.b_rc * dr + B.l_c); };
      if (la > -kDirRecurMax && fabsf(dla) < kDirRecurMax && fabsf(dla_end) < kDirRecurMax) {
        // the geometric recurrence stays inside float32 range: z_j+1 = z_j w_j, w_j+1 = w_j rho
        float2 z = cexpf_turn(la, th);
        float2 w = cexpf_turn(dla, dth);
        const float rr = B.rho_re, ri = B.rho_im;
#pragma unroll
        for (int j = 0; j < L; ++j) {
          if (j > 0 && j % kDirRestart == 0) {
            // re-anchor every kDirRestart pixels at the exact value (the
            // phase at column j by integer differences), so the float32
            // recurrence error stays that of kDirRestart steps
            const float dj = dc + (float)j;
            const uint64_t uj = (uint64_t)j;
            z = cexpf_turn(la_at(dj), th + uj * dth + uj * (uj - 1) * B.p_cc);
            w = cexpf_turn(dla_at(dj), dth + 2 * uj * B.p_cc);
          }
          are[j] += z.x;
          aim[j] += z.y;
          float zr = z.x * w.x - z.y * w.y;
          float zi = z.x * w.y + z.y * w.x;
          z = make_float2(zr, zi);
          float wr = w.x * rr - w.y * ri;
          float wi = w.x * ri + w.y * rr;
          w = make_float2(wr, wi);
        }
      } else {
        // a beam narrow against the strip: every pixel evaluated directly
        // (exact fixed-point phase stepped by integer differences)
        const uint64_t ddth = 2 * B.p_cc;
#pragma unroll
        for (int j = 0; j < L; ++j) {
          const float2 z = cexpf_turn(la_at(dc + (float)j), th);
          are[j] += z.x;
          aim[j] += z.y;
          th += dth;
          dth += ddth;
        }
      }
    }
  }
  if (row < A.h) {
    float2* o = A.out + (size_t)blockIdx.y * A.h * A.w + (size_t)row * A.w;
#pragma unroll
    for (int j = 0; j < L; ++j)
      if (col0 + j < A.w) o[col0 + j] = make_float2(are[j], aim[j]);
  }
}

// ---------------------------------------------------------------- float64
struct DirF64Args {
  const BeamF64* beams;
  int64_t n, chunk;
  int32_t h, w;
  float2* out;  // [gridDim.y][h][w]
};

__global__ void __launch_bounds__(256)
k_field_direct_f64(const __grid_constant__ DirF64Args A) {
  __shared__ BeamF64 sb[32];
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t npx = (int64_t)A.h * A.w;
  const double row = (double)(p / A.w), col = (double)(p % A.w);
  const int64_t b0 = (int64_t)blockIdx.y * A.chunk;
  int64_t b1 = b0 + A.chunk;
  if (b1 > A.n) b1 = A.n;
  double sr = 0.0, si = 0.0;
  for (int64_t bb = b0; bb < b1; bb += 32) {
    const int nb = (int)((b1 - bb) < 32 ? (b1 - bb) : 32);
    __syncthreads();
    for (int i = threadIdx.x; i < nb * 16; i += blockDim.x)
      reinterpret_cast<double*>(sb)[i] = reinterpret_cast<const double*>(A.beams + bb)[i];
    __syncthreads();
    if (p < npx) {
      for (int k = 0; k < nb; ++k) {
        const BeamF64& B = sb[k];
        double ph = ((B.re[0] * col + B.re[2] * row + B.re[3]) * col + (B.re[1] * row + B.re[4]) * row + B.re[5]) + B.ph0;
        double lg = B.lnamp - ((B.im[0] * col + B.im[2] * row + B.im[3]) * col + (B.im[1] * row + B.im[4]) * row + B.im[5]);
        double s, c;
        sincos(ph, &s, &c);
        double a = exp(lg);
        sr += a * c;
        si += a * s;
      }
    }
  }
  if (p < npx) A.out[(size_t)blockIdx.y * npx + p] = make_float2((float)sr, (float)si);
}

__global__ void k_field_reduce(const float2* __restrict__ part, int nchunk, int64_t npx,
                               float2* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npx) return;
  float sr = 0.f, si = 0.f;
  for (int c = 0; c < nchunk; ++c) {
    float2 v = part[(size_t)c * npx + i];
    sr += v.x;
    si += v.y;
  }
  out[i] = make_float2(sr, si);
}

// ---------------------------------------------------------------- operands
// Separable beams (c_rc == 0): field = sum_b V[row][b] * U[b][col] with
//   U[b][col] = exp(-(b_cc dc^2 + l_c dc) + i 2pi (p_cc col^2 + p_c col))
//   V[row][b] = exp(e0 - (b_rr dr^2 + l_r dr) + i 2pi (p_rr row^2 + p_r row + p_0))
// Each value is split into bf16 hi + lo for re and im: planes
//   [0] re_hi [1] re_lo [2] im_hi [3] im_lo, each [lines][kpad] (k contiguous).
struct OperandArgs {
  const BeamFast* beams;
  int64_t n, kpad;
  int32_t lines_v, lines_u;  // padded rows (V) and cols (U)
  int32_t h, w;
  __nv_bfloat16_raw* v_planes;  // 4 * lines_v * kpad
  __nv_bfloat16_raw* u_planes;  // 4 * lines_u * kpad
};

}  // namespace tg

namespace tg {

// One thread per (beam, block of kOpLines lines): the beam's coefficients are
// loaded once and the phase advances by exact 64-bit increments from line to
// line.  blockIdx.y is the line block ([0, lines_v / kOpLines) V rows, then U
// columns; both paddings are multiples of kOpLines), blockIdx.x * blockDim.x
// + threadIdx.x the beam, so there is no index division and the line loop
// needs no bound.  Consecutive threads take consecutive beams: each plane
// store of a warp is one contiguous 64-byte run.
constexpr int kOpLines = 32;  // measured (16,384 beams, 512^2, whole evaluation): 8 lines 0.108 ms, 16 0.0998, 32 0.0982, 64 0.0977

__global__ void __launch_bounds__(256) k_field_operands(const __grid_constant__ OperandArgs A) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= A.kpad) return;
  const int vblocks = A.lines_v / kOpLines;
  const bool isv = (int)blockIdx.y < vblocks;
  const int line0 = ((int)blockIdx.y - (isv ? 0 : vblocks)) * kOpLines;
  const int live_lines = isv ? A.h : A.w;
  const int64_t kpad = A.kpad;
  const int64_t plane = (isv ? A.lines_v : A.lines_u) * kpad;
  __nv_bfloat16_raw* dst = (isv ? A.v_planes : A.u_planes) + line0 * kpad + b;
  const bool live_b = b < A.n;
  uint64_t p2 = 0, p1 = 0, p0 = 0;
  float cen = 0.f, e0 = 0.f, bq = 0.f, bl = 0.f;
  if (live_b) {
    const BeamFast& B = A.beams[b];
    if (B.p_rc != 0 || B.b_rc != 0.f) atomicOr(&g_tg_err, 0x10u);
    if (isv) { p2 = B.p_rr; p1 = B.p_r; p0 = B.p_0; cen = B.r0; e0 = B.e0; bq = B.b_rr; bl = B.l_r; }
    else { p2 = B.p_cc; p1 = B.p_c; p0 = 0; cen = B.c0; e0 = 0.f; bq = B.b_cc; bl = B.l_c; }
  }
  // exact phase at line0 and its first difference; second difference 2*p2
  const uint64_t u0 = (uint64_t)line0;
  uint64_t th = p2 * (u0 * u0) + p1 * u0 + p0;
  uint64_t dth = p2 * (2 * u0 + 1) + p1;
  const uint64_t ddth = 2 * p2;
#pragma unroll 4
  for (int j = 0; j < kOpLines; ++j) {
    float re = 0.f, im = 0.f;
    if (live_b && line0 + j < live_lines) {
      const float2 z = sep_operand(e0, bq, bl, cen, line0 + j, th);
      re = z.x;
      im = z.y;
    }
    uint32_t h2, l2;  // low half re, high half im
    split_bf16x2(re, im, h2, l2);
    dst[0] = __nv_bfloat16_raw{(unsigned short)(h2 & 0xffffu)};
    dst[plane] = __nv_bfloat16_raw{(unsigned short)(l2 & 0xffffu)};
    dst[2 * plane] = __nv_bfloat16_raw{(unsigned short)(h2 >> 16)};
    dst[3 * plane] = __nv_bfloat16_raw{(unsigned short)(l2 >> 16)};
    dst += kpad;
    th += dth;
    dth += ddth;
  }
}

static int sm_count_field() {
  static int cached = 0;
  if (!cached) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&cached, cudaDevAttrMultiProcessorCount, dev);
    if (cached <= 0) cached = 148;
  }
  return cached;
}

int build_dmodel(const tg_model* model, double z_in, DModel* dm) {
  if (!model || model->n_components < 0 || model->n_components > TG_MAX_COMPONENTS)
    return TG_ERR_INVALID;
  if (model->n_components > 0 && !model->components) return TG_ERR_INVALID;
  if (model->propagator != TG_PROP_PARAXIAL) return TG_ERR_UNSUPPORTED;  // make_gaussian_image is paraxial
  std::memset(dm, 0, sizeof(DModel));
  // reuse the float32 program compiler for distances/z bookkeeping, but keep
  // every coefficient in float64 here.
  double z = z_in;
  int n = 0;
  for (int i = 0; i < model->n_components; ++i) {
    const tg_component& c = model->components[i];
    if (c.flags & TG_FLAG_PER_PROBE) return TG_ERR_UNSUPPORTED;
    double d = c.z - z;
    dm->s[n].kind = D_FREE;
    dm->s[n].a[0] = d;
    ++n;
    z = z + d;
    DStep& s = dm->s[n++];
    const double* p = c.p;
    switch (c.kind) {
      case TG_PLANE:
      case TG_APERTURE:
        s.kind = D_NOP;
        break;
      case TG_LENS:
      case TG_THICKLENS:
        if (!(p[0] != 0.0)) return TG_ERR_INVALID;
        s.kind = D_LENS;
        s.a[0] = p[0];
        s.a[1] = 1.0 / p[0];
        if (c.kind == TG_THICKLENS) z = z - (c.z - p[1]);
        break;
      case TG_SCANNER:
        s.kind = D_SHIFT;
        s.a[0] = p[0]; s.a[1] = p[1]; s.a[2] = p[2]; s.a[3] = p[3];
        break;
      case TG_DESCANNER: {
        s.kind = D_SHIFT;
        const double* M = p + 4;
        const double* off = p + 20;
        double sub[4] = {p[0], p[1], p[2], p[3]};
        for (int r = 0; r < 4; ++r) {
          double v = ((p[0] * M[4 * r] + p[1] * M[4 * r + 1]) + off[r]) - sub[r];
          if (M[4 * r + 2] != 0.0 || M[4 * r + 3] != 0.0) v += p[2] * M[4 * r + 2] + p[3] * M[4 * r + 3];
          s.a[r] = v;
        }
      } break;
      case TG_DEFLECTOR:
        s.kind = D_SHIFT;
        s.a[2] = p[0];
        s.a[3] = p[1];
        break;
      case TG_BIPRISM:
        s.kind = D_BIPRISM;
        s.a[0] = p[0];
        break;
      case TG_ROTATOR: {
        double a = p[0] * (M_PI / 180.0);
        s.kind = D_ROTATE;
        s.a[0] = std::cos(a);
        s.a[1] = std::sin(a);
      } break;
      case TG_ABERLENS:
        if (!(p[0] != 0.0)) return TG_ERR_INVALID;
        if (dm->n_aber >= kMaxAber) return TG_ERR_TOO_LARGE;
        s.kind = D_ABER;
        s.pad = dm->n_aber;
        s.a[0] = p[0];
        aber_monomials(p + 1, dm->aber[dm->n_aber++]);
        break;
      default:
        return TG_ERR_UNSUPPORTED;
    }
  }
  dm->n = n;
  return TG_OK;
}

static inline size_t al256(size_t v) { return (v + 255) & ~(size_t)255; }

struct FieldLayout {
  size_t fast, f64, flags, part, vplanes, uplanes, total;
  int chunks;
  int64_t kpad;
  int lines_v, lines_u;
};

constexpr int kDirL = 32;
constexpr int kDirTileRows = 32;
constexpr int kDirStrips = kDirThreads / kDirTileRows;  // 8 strips of kDirL columns

int field_gemm_splits(int64_t n, int h, int w);  // field_gemm.cu

// Resident k_field_direct blocks per SM (register-limited), from the
// occupancy calculator once per process.
static int dir_blocks_per_sm() {
  static int cached = 0;
  if (!cached) {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_field_direct<kDirL>, kDirThreads, 0) != cudaSuccess || b < 1)
      b = 2;
    cached = b;
  }
  return cached;
}
// Beam chunks (blockIdx.y) for the direct sum: kDirWaves waves of resident
// blocks, more (up to kDirWavesMax) while every chunk keeps kDirChunkBeams
// beams; chunk sizes are not rounded to whole shared-memory batches.  Blocks
// differ in cost (beams far from a tile skip most strips), so finer chunks
// balance better once they are long enough.  Measured on 512^2 (ms, 16,384
// astigmatic / 16,384 / 4,096 / 1,024 beams): one wave 2.31 / 2.12 / 0.59 / 0.16,
// two 1.94 / 1.95 / 0.50 / 0.14, three 1.91 / 1.91 / 0.50 / 0.15, four
// 1.88 / 1.93 / 0.50 / 0.15, six 1.85 / 1.88 / 0.51 / 0.17; the earlier
// 64-beam-rounded chunks for ~4 blocks a SM 1.99 / 2.02 / 0.56 / 0.15.
constexpr int kDirWaves = 3;
constexpr int kDirWavesMax = 6;
constexpr int64_t kDirChunkBeams = 256;

static FieldLayout field_layout(int64_t n, int h, int w, int method) {
  FieldLayout L;
  std::memset(&L, 0, sizeof(L));
  size_t off = 0;
  L.fast = off; off = al256(off + (size_t)n * sizeof(BeamFast));
  L.f64 = off; off = al256(off + (size_t)n * sizeof(BeamF64));
  L.flags = off; off = al256(off + 256);
  const int sms = sm_count_field();
  if (method == TG_FIELD_DIRECT) {
    int tiles = ((h + kDirTileRows - 1) / kDirTileRows) * ((w + kDirStrips * kDirL - 1) / (kDirStrips * kDirL));
    const int64_t res = (int64_t)sms * dir_blocks_per_sm();
    const int64_t lo = (res * kDirWaves + tiles - 1) / tiles, hi = (res * kDirWavesMax + tiles - 1) / tiles;
    const int64_t by_beams = n / kDirChunkBeams;
    int want = (int)(by_beams < lo ? lo : (by_beams > hi ? hi : by_beams));
    int64_t maxc = (n + 15) / 16;  // at least 16 beams a chunk
    L.chunks = (int)(want < maxc ? want : maxc);
    if (L.chunks < 1) L.chunks = 1;
  } else if (method == TG_FIELD_DIRECT_F64) {
    int64_t blocks = ((int64_t)h * w + 255) / 256;
    int want = (int)((sms * 8 + blocks - 1) / blocks);
    int64_t maxc = (n + 31) / 32;
    L.chunks = (int)(want < maxc ? want : maxc);
    if (L.chunks < 1) L.chunks = 1;
  } else {
    L.chunks = field_gemm_splits(n, h, w);
    L.kpad = ((n + 32LL * L.chunks - 1) / (32LL * L.chunks)) * 32LL * L.chunks;
    L.lines_v = ((h + 127) / 128) * 128;
    L.lines_u = ((w + 127) / 128) * 128;
    L.vplanes = off; off = al256(off + (size_t)4 * L.lines_v * L.kpad * 2);
    L.uplanes = off; off = al256(off + (size_t)4 * L.lines_u * L.kpad * 2);
  }
  L.part = off;
  off = al256(off + (size_t)L.chunks * h * w * sizeof(float2));
  L.total = off;
  return L;
}

int launch_field_gemm(const __nv_bfloat16_raw* vplanes, const __nv_bfloat16_raw* uplanes,
                      int lines_v, int lines_u, int64_t kpad, int splits, int h, int w,
                      float2* part, cudaStream_t s);  // field_gemm.cu

static bool field_method_ok(int method) {
  return method == TG_FIELD_DIRECT || method == TG_FIELD_SEPARABLE || method == TG_FIELD_DIRECT_F64;
}

}  // namespace tg

using namespace tg;

extern "C" size_t tg_field_workspace(int64_t n_beams, int32_t h, int32_t w, int32_t method) {
  if (n_beams < 0 || h <= 0 || w <= 0) return 0;
  if (!field_method_ok(method))
    return 0;
  return field_layout(n_beams, h, w, method).total;
}

namespace tg {
static int field_prep_launch(const DModel& dm, const tg_beams* beams, const tg_pixel_map* pm,
                             void* workspace, size_t ws_bytes, int32_t* flags, void* stream,
                             int input_plane, int unit_amp = 0) {
  if (!beams || !pm || pm->h <= 0 || pm->w <= 0 || beams->n < 0) return TG_ERR_INVALID;
  if (beams->n > 0 && (!beams->x || !beams->y || !beams->dx || !beams->dy || !beams->pathlength ||
                       !beams->amplitude || !beams->waist_xy || !beams->radii))
    return TG_ERR_INVALID;
  FieldLayout L = field_layout(beams->n, pm->h, pm->w, TG_FIELD_DIRECT);
  if (!workspace || ws_bytes < L.part) return TG_ERR_WORKSPACE;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  char* ws = reinterpret_cast<char*>(workspace);
  int32_t* fl = flags ? flags : reinterpret_cast<int32_t*>(ws + L.flags);
  if (cudaMemsetAsync(fl, 0, sizeof(int32_t), s) != cudaSuccess) return TG_ERR_CUDA;
  if (beams->n == 0) return TG_OK;
  PrepArgs A;
  std::memset(&A, 0, sizeof(A));
  A.n = beams->n;
  A.x = beams->x; A.y = beams->y; A.dx = beams->dx; A.dy = beams->dy;
  A.z = beams->z;
  A.pl = beams->pathlength;
  A.amp = beams->amplitude;
  A.waist = beams->waist_xy;
  A.radii = beams->radii;
  A.wl = beams->wavelength;
  A.wl_scalar = beams->wavelength_scalar;
  A.theta = beams->theta;
  A.pm.h = pm->h;
  A.pm.w = pm->w;
  for (int i = 0; i < 6; ++i) A.pm.t[i] = pm->t[i];
  A.fast = reinterpret_cast<BeamFast*>(ws + L.fast);
  A.f64 = reinterpret_cast<BeamF64*>(ws + L.f64);
  A.flags = fl;
  A.input_plane = input_plane;
  A.unit_amp = unit_amp;
  // 64-thread blocks: one thread per beam is all the parallelism there is, so
  // spread the (float64-bound) beams over every SM
  int blocks = (int)((beams->n + 63) / 64);
  k_field_prep<<<blocks, 64, 0, s>>>(dm, A);
  return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
}
}  // namespace tg

namespace tg {
// For the field adjoint (field_adjoint.cu): the bytes of the per-beam records
// (BeamFast at offset 0, then BeamF64 and a status word), and the records of
// unit-amplitude beams written there.
size_t field_records_bytes(int64_t n) { return field_layout(n, 1, 1, TG_FIELD_DIRECT).part; }

int field_prep_unit_amp(const DModel& dm, const tg_beams* beams, const tg_pixel_map* pm, void* records,
                        size_t bytes, void* stream, int input_plane) {
  return field_prep_launch(dm, beams, pm, records, bytes, nullptr, stream, input_plane, 1);
}
}  // namespace tg

extern "C" int tg_field_prep(const tg_model* model, const tg_beams* beams,
                             const tg_pixel_map* pm, void* workspace, size_t ws_bytes,
                             int32_t* flags, void* stream) {
  if (!model || !beams) return TG_ERR_INVALID;
  DModel dm;
  int st = build_dmodel(model, beams->z, &dm);
  if (st != TG_OK) return st;
  return field_prep_launch(dm, beams, pm, workspace, ws_bytes, flags, stream, 0);
}

extern "C" int tg_field_prep_input(const tg_beams* beams, const tg_pixel_map* pm, void* workspace,
                                   size_t ws_bytes, int32_t* flags, void* stream) {
  DModel dm;
  std::memset(&dm, 0, sizeof(dm));
  return field_prep_launch(dm, beams, pm, workspace, ws_bytes, flags, stream, 1);
}

extern "C" int tg_field_eval(int32_t method, int64_t n_beams, const tg_pixel_map* pm,
                             float* out, void* workspace, size_t ws_bytes, void* stream) {
  if (!pm || pm->h <= 0 || pm->w <= 0 || n_beams < 0 || !out) return TG_ERR_INVALID;
  if (!field_method_ok(method))
    return TG_ERR_INVALID;
  FieldLayout L = field_layout(n_beams, pm->h, pm->w, method);
  if (!workspace || ws_bytes < L.total) return TG_ERR_WORKSPACE;
  if (((uintptr_t)workspace & 255) != 0) return TG_ERR_ALIGN;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  char* ws = reinterpret_cast<char*>(workspace);
  const int64_t npx = (int64_t)pm->h * pm->w;
  float2* o = reinterpret_cast<float2*>(out);
  if (n_beams == 0) {
    return cudaMemsetAsync(out, 0, (size_t)npx * sizeof(float2), s) == cudaSuccess ? TG_OK : TG_ERR_CUDA;
  }
  float2* part = reinterpret_cast<float2*>(ws + L.part);
  if (method == TG_FIELD_DIRECT) {
    DirArgs A;
    A.beams = reinterpret_cast<const BeamFast*>(ws + L.fast);
    A.n = n_beams;
    A.chunk = (n_beams + L.chunks - 1) / L.chunks;
    A.h = pm->h;
    A.w = pm->w;
    A.tile_rows = kDirTileRows;
    A.strips_x = kDirStrips;
    A.out = part;
    int tiles = ((pm->h + kDirTileRows - 1) / kDirTileRows) *
                ((pm->w + kDirStrips * kDirL - 1) / (kDirStrips * kDirL));
    int chunks = (int)((n_beams + A.chunk - 1) / A.chunk);
    k_field_direct<kDirL><<<dim3(tiles, chunks), kDirThreads, 0, s>>>(A);
    k_field_reduce<<<(int)((npx + 255) / 256), 256, 0, s>>>(part, chunks, npx, o);
  } else if (method == TG_FIELD_DIRECT_F64) {
    DirF64Args A;
    A.beams = reinterpret_cast<const BeamF64*>(ws + L.f64);
    A.n = n_beams;
    A.chunk = ((n_beams + L.chunks - 1) / L.chunks + 31) / 32 * 32;
    A.h = pm->h;
    A.w = pm->w;
    A.out = part;
    int chunks = (int)((n_beams + A.chunk - 1) / A.chunk);
    k_field_direct_f64<<<dim3((unsigned)((npx + 255) / 256), chunks), 256, 0, s>>>(A);
    k_field_reduce<<<(int)((npx + 255) / 256), 256, 0, s>>>(part, chunks, npx, o);
  } else {
    OperandArgs A;
    A.beams = reinterpret_cast<const BeamFast*>(ws + L.fast);
    A.n = n_beams;
    A.kpad = L.kpad;
    A.lines_v = L.lines_v;
    A.lines_u = L.lines_u;
    A.h = pm->h;
    A.w = pm->w;
    A.v_planes = reinterpret_cast<__nv_bfloat16_raw*>(ws + L.vplanes);
    A.u_planes = reinterpret_cast<__nv_bfloat16_raw*>(ws + L.uplanes);
    if (L.lines_v % kOpLines || L.lines_u % kOpLines || L.kpad > INT32_MAX) return TG_ERR_TOO_LARGE;
    k_field_operands<<<dim3((unsigned)((L.kpad + 255) / 256), (unsigned)((L.lines_v + L.lines_u) / kOpLines)), 256,
                       0, s>>>(A);
    int st = launch_field_gemm(A.v_planes, A.u_planes, L.lines_v, L.lines_u, L.kpad, L.chunks,
                               pm->h, pm->w, part, s);
    if (st != TG_OK) return st;
    k_field_reduce<<<(int)((npx + 255) / 256), 256, 0, s>>>(part, L.chunks, npx, o);
  }
  return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
}

// ---------------------------------------------------------------- no-alloc
// tg_field_direct_noalloc: the direct field sum for callers that cannot
// allocate device memory.  Its scratch (beam records and per-chunk partial
// images) lives in one file-scope device array of fixed size, so the call
// itself never allocates.  Every GPU that loads this library holds the array
// until the process exits.
#include <mutex>

namespace tg {

constexpr size_t kNoAllocBytes = (size_t)32 << 20;  // 32 MiB per device
constexpr int64_t kNoAllocMaxBeams = 32768;
static __device__ __align__(256) unsigned char g_field_noalloc[kNoAllocBytes];
static std::mutex g_noalloc_mu;
static void* g_noalloc_addr[256];  // last looked-up device address, per device ordinal
static_assert(sizeof(BeamFast) == 96 && sizeof(BeamF64) == 128, "record sizes stated in the header");

// Device address of the scratch array on the current device.  Host code may
// not use the symbol itself as a pointer (it is a host-side stand-in), so the
// address is looked up with the device current: on every call that is not
// being captured into a CUDA graph (after a device reset or on a new context
// the address can change), and taken from the last such call while the
// stream is being captured.
static int noalloc_scratch(cudaStream_t s, void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) return TG_ERR_CUDA;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) return TG_ERR_CUDA;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (cs == cudaStreamCaptureStatusNone) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_field_noalloc) != cudaSuccess || !p) return TG_ERR_CUDA;
    g_noalloc_addr[dev] = p;
  } else if (!g_noalloc_addr[dev]) {
    return TG_ERR_CUDA;  // no uncaptured call on this device yet
  }
  *out = g_noalloc_addr[dev];
  return TG_OK;
}

}  // namespace tg

extern "C" int tg_field_direct_noalloc(const tg_model* model, const tg_beams* beams,
                                       const tg_pixel_map* pm, float* out, void* stream) {
  if (!model || !beams || !pm) return TG_ERR_INVALID;
  if (beams->n < 0 || pm->h <= 0 || pm->w <= 0) return TG_ERR_INVALID;
  if (beams->n > kNoAllocMaxBeams) return TG_ERR_TOO_LARGE;
  const FieldLayout L = field_layout(beams->n, pm->h, pm->w, TG_FIELD_DIRECT);
  const size_t per_chunk = (size_t)pm->h * pm->w * sizeof(float2);
  if (L.part > kNoAllocBytes || kNoAllocBytes - L.part < per_chunk) return TG_ERR_TOO_LARGE;
  if (!out) return TG_ERR_INVALID;
  void* scratch = nullptr;
  int st = noalloc_scratch(reinterpret_cast<cudaStream_t>(stream), &scratch);
  if (st != TG_OK) return st;
  st = tg_field_prep(model, beams, pm, scratch, L.part, nullptr, stream);
  if (st != TG_OK) return st;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int64_t n = beams->n, npx = (int64_t)pm->h * pm->w;
  float2* o = reinterpret_cast<float2*>(out);
  if (n == 0)
    return cudaMemsetAsync(out, 0, (size_t)npx * sizeof(float2), s) == cudaSuccess ? TG_OK : TG_ERR_CUDA;
  int64_t chunks = L.chunks;
  const int64_t fit = (int64_t)((kNoAllocBytes - L.part) / per_chunk);
  if (chunks > fit) chunks = fit;
  char* ws = reinterpret_cast<char*>(scratch);
  DirArgs A;
  A.beams = reinterpret_cast<const BeamFast*>(ws + L.fast);
  A.n = n;
  A.chunk = (n + chunks - 1) / chunks;
  A.h = pm->h;
  A.w = pm->w;
  A.tile_rows = kDirTileRows;
  A.strips_x = kDirStrips;
  A.out = reinterpret_cast<float2*>(ws + L.part);  // every in-range pixel is overwritten
  const int tiles = ((pm->h + kDirTileRows - 1) / kDirTileRows) *
                    ((pm->w + kDirStrips * kDirL - 1) / (kDirStrips * kDirL));
  const int used = (int)((n + A.chunk - 1) / A.chunk);
  k_field_direct<kDirL><<<dim3(tiles, used), kDirThreads, 0, s>>>(A);
  k_field_reduce<<<(int)((npx + 255) / 256), 256, 0, s>>>(A.out, used, npx, o);
  return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
}

// ------------------------------------------- one-call field entry points
// tg_field_prep followed by tg_field_eval with a fixed method, for callers
// that want the detector field in one call (the caller's workspace holds
// the records and partials: tg_field_workspace(n, h, w, method) bytes).
extern "C" int tg_field_direct(const tg_model* model, const tg_beams* beams, const tg_pixel_map* pm,
                               float* out, void* workspace, size_t ws_bytes, void* stream) {
  int st = tg_field_prep(model, beams, pm, workspace, ws_bytes, nullptr, stream);
  if (st != TG_OK) return st;
  return tg_field_eval(TG_FIELD_DIRECT, beams->n, pm, out, workspace, ws_bytes, stream);
}

extern "C" int tg_field_separable(const tg_model* model, const tg_beams* beams, const tg_pixel_map* pm,
                                  float* out, void* workspace, size_t ws_bytes, void* stream) {
  int st = tg_field_prep(model, beams, pm, workspace, ws_bytes, nullptr, stream);
  if (st != TG_OK) return st;
  return tg_field_eval(TG_FIELD_SEPARABLE, beams->n, pm, out, workspace, ws_bytes, stream);
}
