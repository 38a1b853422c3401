// field_points.cu - the Gaussian-beamlet field from per-beam ABCD blocks at
// arbitrary sample points: propagate_misaligned_gaussian_jax_scan
// (gaussian.py:319-337 with _beam_field, gaussian.py:276-316) and
// evaluate_misaligned_input_gaussian_jax_scan (gaussian.py:410-427 with
// _input_beam_field, gaussian.py:402-409).  Complex128 out, as the reference.
//
//   k_points_prep   one thread per beam, float64: reduces the per-point
//                   formula to a complex quadratic in s = r - origin,
//                     Phi(s) = cxx sx^2 + cyy sy^2 + cxy sx sy + cx sx + cy sy + c0
//                   ((k/2) folded in), plus ln|pref| and the phase constant
//                   (phase_offset reduced mod 2 pi, plus arg(pref)).
//   k_points_eval   one thread per point, one block row per beam chunk:
//                   beam records staged 32 at a time in shared memory, every
//                   (beam, point) term in float64 (polynomial, sincos, exp).
//   k_points_reduce the chunk partials summed in chunk order (deterministic).
#include <math.h>
#include <stdint.h>

#include "tg_common.cuh"

namespace tg {

struct alignas(16) PointBeam {  // 128 bytes
  double re[6];  // cxx, cyy, cxy, cx, cy, c0 real parts (radians)
  double im[6];  // imaginary parts (the envelope exponent)
  double ox, oy; // origin of s: e (detector) or r1m (input plane)
  double ph0;    // phase_offset mod 2 pi + arg(pref)
  double lnamp;  // ln |pref|
};

struct z2 {
  double re, im;
};
__device__ __forceinline__ z2 operator+(z2 a, z2 b) { return z2{a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ z2 operator-(z2 a, z2 b) { return z2{a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ z2 operator*(z2 a, z2 b) {
  return z2{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
__device__ __forceinline__ z2 operator*(double s, z2 a) { return z2{s * a.re, s * a.im}; }
__device__ __forceinline__ z2 R2(double r) { return z2{r, 0.0}; }
__device__ __forceinline__ z2 zrecip(z2 b) {  // Smith's method (Smith 1962)
  if (fabs(b.re) >= fabs(b.im)) {
    const double r = b.im / b.re, d = b.re + b.im * r;
    return z2{1.0 / d, -r / d};
  }
  const double r = b.re / b.im, d = b.re * r + b.im;
  return z2{r / d, -1.0 / d};
}
__device__ __forceinline__ z2 zsqrt(z2 z) {  // principal branch
  const double r = hypot(z.re, z.im);
  if (z.re >= 0.0) {
    const double t = sqrt(0.5 * (r + z.re));
    return z2{t, t > 0.0 ? z.im / (2.0 * t) : z.im};
  }
  const double t = sqrt(0.5 * (r - z.re));
  return z2{fabs(z.im) / (2.0 * t), copysign(t, z.im)};
}

struct m2 {  // [[a, b], [c, d]]
  z2 a, b, c, d;
};
__device__ __forceinline__ m2 mul(m2 x, m2 y) {
  return m2{x.a * y.a + x.b * y.c, x.a * y.b + x.b * y.d, x.c * y.a + x.d * y.c, x.c * y.b + x.d * y.d};
}
__device__ __forceinline__ m2 add(m2 x, m2 y) { return m2{x.a + y.a, x.b + y.b, x.c + y.c, x.d + y.d}; }
__device__ __forceinline__ m2 inv(m2 m) {  // explicit inverse: inf / nan when singular
  const z2 r = zrecip(m.a * m.d - m.b * m.c);
  return m2{m.d * r, R2(0.0) - m.b * r, R2(0.0) - m.c * r, m.a * r};
}
__device__ __forceinline__ double fin(double v) { return isfinite(v) ? v : 0.0; }
__device__ __forceinline__ m2 nan_to_num(m2 m) {  // gaussian.py:283-287
  return m2{z2{fin(m.a.re), fin(m.a.im)}, z2{fin(m.b.re), fin(m.b.im)}, z2{fin(m.c.re), fin(m.c.im)},
            z2{fin(m.d.re), fin(m.d.im)}};
}
__device__ __forceinline__ m2 load_real(const double* p) { return m2{R2(p[0]), R2(p[1]), R2(p[2]), R2(p[3])}; }
__device__ __forceinline__ m2 load_cplx(const double* p) {
  return m2{z2{p[0], p[1]}, z2{p[2], p[3]}, z2{p[4], p[5]}, z2{p[6], p[7]}};
}

struct PtPrepArgs {
  int64_t n;
  int32_t input_plane;  // 1: evaluate_misaligned_input (no A, B, C, D, e, f)
  int32_t pad;
  const double* amp;    // [n] complex128
  const double* po;     // [n] phase offsets (radians)
  const double* q1;     // [n][2][2] complex128 Q1^-1
  const double *a, *b, *c, *d;  // [n][2][2] float64
  const double *e, *f;  // [n][2]
  const double *r1m, *t1m;      // [n][2]
  const double* k;      // [n]
  PointBeam* out;
};

__global__ void __launch_bounds__(128) k_points_prep(const __grid_constant__ PtPrepArgs A) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.n) return;
  const double hk = 0.5 * A.k[i];
  const m2 Q1i = load_cplx(A.q1 + 8 * i);
  const double x0 = A.r1m[2 * i], y0 = A.r1m[2 * i + 1];
  const double tx = A.t1m[2 * i], ty = A.t1m[2 * i + 1];
  z2 S_xx, S_yy, S_xy, Lx, Ly, c0, pref = z2{A.amp[2 * i], A.amp[2 * i + 1]};
  double ox, oy;
  if (A.input_plane) {
    // (k/2) (s^T Q1^-1 s + 2 s . theta1m), s = r1 - r1m (gaussian.py:402-409)
    S_xx = Q1i.a; S_yy = Q1i.d; S_xy = Q1i.b + Q1i.c;
    Lx = R2(2.0 * tx); Ly = R2(2.0 * ty);
    c0 = R2(0.0);
    ox = x0; oy = y0;
  } else {
    const m2 Am = load_real(A.a + 4 * i), Bm = load_real(A.b + 4 * i);
    const m2 Cm = load_real(A.c + 4 * i), Dm = load_real(A.d + 4 * i);
    // Q2^-1 = (A + B Q1^-1)^-1 (C + D Q1^-1)   (gaussian.py:92-96, 323)
    const m2 denom = add(Am, mul(Bm, Q1i));
    const m2 Q2 = mul(inv(denom), add(Cm, mul(Dm, Q1i)));
    const m2 Binv = nan_to_num(inv(Bm));
    const m2 Q1 = nan_to_num(inv(Q1i));
    // central ray at the output: r2m = A r1m + B theta1m
    const double r2x = Am.a.re * x0 + Am.b.re * y0 + Bm.a.re * tx + Bm.b.re * ty;
    const double r2y = Am.c.re * x0 + Am.d.re * y0 + Bm.c.re * tx + Bm.d.re * ty;
    pref = pref * zrecip(zsqrt(denom.a * denom.d - denom.b * denom.c));
    const m2 ABinv = mul(Am, Binv);
    const m2 P = mul(Q1, inv(mul(Bm, add(mul(Am, Q1), Bm))));  // Q1 (B (A Q1 + B))^-1
    // s^T Q2 s + [r1m^T ABinv r1m - 2 r1m^T Binv s] - [r2m^T P r2m - 2 r2m^T P s] + 2 s . f
    S_xx = Q2.a; S_yy = Q2.d; S_xy = Q2.b + Q2.c;
    const z2 bx = Binv.a * R2(x0) + Binv.c * R2(y0), by = Binv.b * R2(x0) + Binv.d * R2(y0);
    const z2 px = P.a * R2(r2x) + P.c * R2(r2y), py = P.b * R2(r2x) + P.d * R2(r2y);
    Lx = R2(2.0 * A.f[2 * i]) - 2.0 * bx + 2.0 * px;
    Ly = R2(2.0 * A.f[2 * i + 1]) - 2.0 * by + 2.0 * py;
    const z2 q1 = R2(x0) * (ABinv.a * R2(x0) + ABinv.b * R2(y0)) + R2(y0) * (ABinv.c * R2(x0) + ABinv.d * R2(y0));
    const z2 q2 = R2(r2x) * (P.a * R2(r2x) + P.b * R2(r2y)) + R2(r2y) * (P.c * R2(r2x) + P.d * R2(r2y));
    c0 = q1 - q2;
    ox = A.e[2 * i]; oy = A.e[2 * i + 1];
  }
  PointBeam B;
  const z2 cf[6] = {hk * S_xx, hk * S_yy, hk * S_xy, hk * Lx, hk * Ly, hk * c0};
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    B.re[j] = cf[j].re;
    B.im[j] = cf[j].im;
  }
  B.ox = ox;
  B.oy = oy;
  // phase_offset mod 2 pi with 2 pi as a sum of two doubles (exact for |po| < 2^52 rad)
  const double C1 = 6.283185307179586, C2 = 2.4492935982947064e-16;
  const double po = A.po[i];
  const double nt = rint(po * 0.15915494309189535);
  const double red = fma(-nt, C2, fma(-nt, C1, po));
  B.ph0 = red + atan2(pref.im, pref.re);
  B.lnamp = log(hypot(pref.re, pref.im));
  A.out[i] = B;
}

struct PtEvalArgs {
  const PointBeam* beams;
  int64_t n, npts, chunk;
  const double* r;   // [npts][2] (x, y)
  double2* part;     // [chunks][npts]
};

__global__ void __launch_bounds__(256) k_points_eval(const __grid_constant__ PtEvalArgs A) {
  __shared__ PointBeam sb[32];
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = p < A.npts;
  const double x = live ? A.r[2 * p] : 0.0, y = live ? A.r[2 * p + 1] : 0.0;
  const int64_t b0 = (int64_t)blockIdx.y * A.chunk;
  const int64_t b1 = (b0 + A.chunk < A.n) ? b0 + A.chunk : A.n;
  double sr = 0.0, si = 0.0;
  for (int64_t bb = b0; bb < b1; bb += 32) {
    const int nb = (int)((b1 - bb) < 32 ? (b1 - bb) : 32);
    __syncthreads();
    for (int j = threadIdx.x; j < nb * 16; j += blockDim.x)
      reinterpret_cast<double*>(sb)[j] = reinterpret_cast<const double*>(A.beams + bb)[j];
    __syncthreads();
    if (live) {
      for (int j = 0; j < nb; ++j) {
        const PointBeam& B = sb[j];
        const double sx = x - B.ox, sy = y - B.oy;
        const double ph = ((B.re[0] * sx + B.re[2] * sy + B.re[3]) * sx + (B.re[1] * sy + B.re[4]) * sy + B.re[5]) + B.ph0;
        const double lg = B.lnamp - ((B.im[0] * sx + B.im[2] * sy + B.im[3]) * sx + (B.im[1] * sy + B.im[4]) * sy + B.im[5]);
        double s, c;
        sincos(ph, &s, &c);
        const double a = exp(lg);
        sr += a * c;
        si += a * s;
      }
    }
  }
  if (live) A.part[(size_t)blockIdx.y * A.npts + p] = make_double2(sr, si);
}

__global__ void __launch_bounds__(256) k_points_reduce(const double2* __restrict__ part, int nchunk,
                                                       int64_t npts, double2* __restrict__ out) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npts) return;
  double sr = 0.0, si = 0.0;
  for (int c = 0; c < nchunk; ++c) {
    const double2 v = part[(size_t)c * npts + p];
    sr += v.x;
    si += v.y;
  }
  out[p] = make_double2(sr, si);
}

static int points_sm_count() {
  static int cached = 0;
  if (!cached) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&cached, cudaDevAttrMultiProcessorCount, dev);
    if (cached <= 0) cached = 148;
  }
  return cached;
}

// Beam chunks: enough (point-block x chunk) blocks to fill the GPU a few
// times over, each chunk a whole number of 32-beam stages.
static void points_layout(int64_t n, int64_t npts, int64_t* chunk, int64_t* chunks) {
  const int64_t pblocks = (npts + 255) / 256;
  const int64_t target = (int64_t)points_sm_count() * 8;
  int64_t c = (target + pblocks - 1) / pblocks;
  const int64_t stages = (n + 31) / 32;
  if (c > stages) c = stages;
  if (c < 1) c = 1;
  int64_t per = ((stages + c - 1) / c) * 32;
  *chunk = per;
  *chunks = (n + per - 1) / per;
  if (*chunks < 1) *chunks = 1;
}

static size_t points_ws(int64_t n, int64_t npts) {
  int64_t chunk, chunks;
  points_layout(n, npts, &chunk, &chunks);
  const size_t rec = ((size_t)n * sizeof(PointBeam) + 255) & ~(size_t)255;
  return rec + (size_t)chunks * (size_t)npts * sizeof(double2);
}

static int points_run(const PtPrepArgs& P, int64_t npts, const double* r, double* out, void* ws,
                      size_t ws_bytes, cudaStream_t s) {
  if (P.n == 0 || npts == 0) {
    if (npts > 0 && cudaMemsetAsync(out, 0, (size_t)npts * 16, s) != cudaSuccess) return TG_ERR_CUDA;
    return TG_OK;
  }
  if (!ws || ws_bytes < points_ws(P.n, npts) || (reinterpret_cast<uintptr_t>(ws) & 15) != 0)
    return TG_ERR_WORKSPACE;
  int64_t chunk, chunks;
  points_layout(P.n, npts, &chunk, &chunks);
  PtPrepArgs Q = P;
  Q.out = reinterpret_cast<PointBeam*>(ws);
  const size_t rec = ((size_t)P.n * sizeof(PointBeam) + 255) & ~(size_t)255;
  double2* part = reinterpret_cast<double2*>(reinterpret_cast<char*>(ws) + rec);
  k_points_prep<<<(int)((P.n + 127) / 128), 128, 0, s>>>(Q);
  PtEvalArgs E{Q.out, P.n, npts, chunk, r, part};
  k_points_eval<<<dim3((unsigned)((npts + 255) / 256), (unsigned)chunks), 256, 0, s>>>(E);
  k_points_reduce<<<(int)((npts + 255) / 256), 256, 0, s>>>(part, (int)chunks, npts,
                                                           reinterpret_cast<double2*>(out));
  return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
}

}  // namespace tg

using namespace tg;

extern "C" size_t tg_misaligned_gaussian_workspace(int64_t n_beams, int64_t n_points) {
  if (n_beams <= 0 || n_points <= 0) return 0;
  return points_ws(n_beams, n_points);
}

extern "C" int tg_propagate_misaligned_gaussian(int64_t n, const double* amp, const double* phase_offset,
                                                const double* q1_inv, const double* a, const double* b,
                                                const double* c, const double* d, const double* e,
                                                const double* f, const double* r1m, const double* theta1m,
                                                const double* k, int64_t n_points, const double* r2,
                                                double* out, void* workspace, size_t ws_bytes, void* stream) {
  if (n < 0 || n_points < 0) return TG_ERR_INVALID;
  if (n_points > 0 && (!r2 || !out)) return TG_ERR_INVALID;
  if (n > 0 && (!amp || !phase_offset || !q1_inv || !a || !b || !c || !d || !e || !f || !r1m || !theta1m || !k))
    return TG_ERR_INVALID;
  if (n > 0x7fffffffLL * 32 || n_points > 0x7fffffffLL * 255) return TG_ERR_TOO_LARGE;
  PtPrepArgs P{n, 0, 0, amp, phase_offset, q1_inv, a, b, c, d, e, f, r1m, theta1m, k, nullptr};
  return points_run(P, n_points, r2, out, workspace, ws_bytes, reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int tg_evaluate_misaligned_input_gaussian(int64_t n, const double* amp, const double* phase_offset,
                                                     const double* q1_inv, const double* r1m,
                                                     const double* theta1m, const double* k, int64_t n_points,
                                                     const double* r1, double* out, void* workspace,
                                                     size_t ws_bytes, void* stream) {
  if (n < 0 || n_points < 0) return TG_ERR_INVALID;
  if (n_points > 0 && (!r1 || !out)) return TG_ERR_INVALID;
  if (n > 0 && (!amp || !phase_offset || !q1_inv || !r1m || !theta1m || !k)) return TG_ERR_INVALID;
  if (n > 0x7fffffffLL * 32 || n_points > 0x7fffffffLL * 255) return TG_ERR_TOO_LARGE;
  PtPrepArgs P{n, 1, 0, amp, phase_offset, q1_inv, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
               r1m, theta1m, k, nullptr};
  return points_run(P, n_points, r1, out, workspace, ws_bytes, reinterpret_cast<cudaStream_t>(stream));
}
