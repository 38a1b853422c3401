// source.cu - device-side ray sources and Gaussian-beam decomposition.
//
//   k_source_rings      PointSource / ParallelBeam deterministic rays
//                       (source.py:82-188 with utils.py:117-175
//                       concentric_rings): one thread per angle partition
//                       runs the reference's float64 running-angle recurrence
//                       (utils.py:47-80 multi_cumsum_inplace), so every ring
//                       layout, radius and angle matches it; sin / cos are
//                       CUDA's float64 functions (within 2 ulp of the host's).
//   k_source_random     random mode: uniform points in the disc from a
//                       counter-based hash of (seed, index) - the same
//                       distribution as utils.py:178-202 random_coords, not
//                       the same draws (those come from NumPy's global
//                       generator), and exactly the requested count.
//   k_decompose_q       gaussian.py:35-89 decompose_Q_inv for a batch of
//                       2x2 complex Q^-1: waists, radii, rotation.
//   k_beam_q_inv        the other direction, GaussianRay.q_inv / Q_inv
//                       (gaussian.py:138-177): per-axis 1/q and
//                       R(theta) diag(1/qx, 1/qy) R(theta)^T.
//   k_qinv_abcd         Qinv_ABCD (gaussian.py:92-96): (A + B Q)^-1 (C + D Q)
//                       by 2x2 LU with partial pivoting, as the reference's
//                       linalg.solve does it.
//   k_beam_profile      the textbook helpers zR, w_z, R, q_inv(z, w0, wl)
//                       (gaussian.py:13-28, 99-109) elementwise.
//   k_gaussian_beam     gaussian_beam (gaussian.py:31-32) elementwise.
#include <cmath>
#include <cstring>

#include "tg_common.cuh"

namespace tg {

// Ring layout of concentric_rings (utils.py:135-175), float64 as NumPy does it.
struct RingLayout {
  int64_t num;      // requested (approximate) count
  int32_t rings;    // number of rings R
  int32_t pad;
  double ppu;       // points per unit circumference: num / sum(round(2 pi k))
  double extent;    // outer radius (metres or radians)
  int64_t total;    // sum of points over the rings
};

__host__ __device__ inline int64_t ring_points(int k, double ppu) {  // ring k = 0..R-1
  const double two_pi = 6.283185307179586;  // 2 * np.pi
  const double nk = rint(two_pi * (double)(k + 1));
  return (int64_t)rint(nk * ppu);
}

__host__ __device__ inline double ring_radius(int k, const RingLayout& L) {
  // np.linspace(0, extent, R + 1)[1:]: k * (extent / R), the last one exactly extent
  return (k == L.rings - 1) ? L.extent : (double)(k + 1) * (L.extent / (double)L.rings);
}

static int ring_layout(int64_t num, double extent, RingLayout* L) {
  if (num < 1) return TG_ERR_INVALID;
  if (num > ((int64_t)1 << 40)) return TG_ERR_TOO_LARGE;
  std::memset(L, 0, sizeof(*L));
  const double pi = 3.141592653589793;
  const double t = std::floor((-1.0 + std::sqrt(1.0 + (double)(4 * num) / pi)) / 2.0);
  const int rings = t < 1.0 ? 1 : (int)t;
  int64_t sum_nk = 0;
  for (int k = 0; k < rings; ++k) sum_nk += (int64_t)std::nearbyint(6.283185307179586 * (double)(k + 1));
  L->num = num;
  L->rings = rings;
  L->ppu = (double)num / (double)sum_nk;
  L->extent = extent;
  int64_t total = 0;
  for (int k = 0; k < rings; ++k) {
    const int64_t p = ring_points(k, L->ppu);
    total += p > 0 ? p : 0;
  }
  L->total = total;
  return TG_OK;
}

struct SourceArgs {
  RingLayout L;
  int32_t kind;  // 0 = point source, 1 = parallel beam
  int32_t pad;
  double off_x, off_y;
  double* out;   // [total][5]: x, y, dx, dy, 1
};

__device__ inline void write_row(const SourceArgs& A, int64_t v, double r, double ang) {
  double s, c;
  sincos(ang, &s, &c);
  const double py = r * s, px = r * c;  // concentric_rings returns (r sin, r cos) = (y, x)
  double* o = A.out + v * 5;
  if (A.kind == 0) {  // PointSource: positions at the offset, slopes on the disc (source.py:117-135)
    o[0] = 0.0 + A.off_x; o[1] = 0.0 + A.off_y; o[2] = px; o[3] = py;
  } else {            // ParallelBeam: positions on the disc, zero slopes (source.py:170-188)
    o[0] = px + A.off_x; o[1] = py + A.off_y; o[2] = 0.0; o[3] = 0.0;
  }
  o[4] = 1.0;
}

// Partition i of multi_cumsum_inplace covers indices s_i .. s_i + p_i with
// s_i = (points of rings < i) + i: the running angle restarts at 0 at s_i and
// adds, at every later index, the angular step of the ring that index lies in.
__global__ void __launch_bounds__(128) k_source_rings(const __grid_constant__ SourceArgs A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.L.rings) return;
  int64_t ring_start = 0;
  for (int j = 0; j < i; ++j) {
    const int64_t p = ring_points(j, A.L.ppu);
    ring_start += p > 0 ? p : 0;
  }
  const int64_t pi_pts = ring_points(i, A.L.ppu) > 0 ? ring_points(i, A.L.ppu) : 0;
  const int64_t s = ring_start + i;
  if (s >= A.L.total) return;
  int64_t e = s + pi_pts;  // inclusive
  if (e > A.L.total - 1) e = A.L.total - 1;
  // ring containing index s
  int k = i;
  int64_t rs = ring_start, rp = pi_pts;
  while (s >= rs + rp && k + 1 < A.L.rings) {
    rs += rp;
    ++k;
    const int64_t p = ring_points(k, A.L.ppu);
    rp = p > 0 ? p : 0;
  }
  double ang = 0.0;
  for (int64_t v = s; v <= e; ++v) {
    while (v >= rs + rp && k + 1 < A.L.rings) {
      rs += rp;
      ++k;
      const int64_t p = ring_points(k, A.L.ppu);
      rp = p > 0 ? p : 0;
    }
    if (v > s) ang = 6.283185307179586 / (double)rp + ang;  // values[v] += values[v - 1]
    write_row(A, v, ring_radius(k, A.L), ang);
  }
}

__device__ __forceinline__ uint64_t mix64(uint64_t z) {  // SplitMix64 finaliser
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

__global__ void __launch_bounds__(256) k_source_random(const __grid_constant__ SourceArgs A, uint64_t seed) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < A.L.total;
       v += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t h1 = mix64(seed ^ mix64(2 * (uint64_t)v));
    const uint64_t h2 = mix64(seed ^ mix64(2 * (uint64_t)v + 1));
    const double u1 = (double)(h1 >> 11) * 0x1.0p-53, u2 = (double)(h2 >> 11) * 0x1.0p-53;
    write_row(A, v, A.L.extent * sqrt(u1), 6.283185307179586 * u2);
  }
}

// ---------------------------------------------------------------- decompose
struct DecompArgs {
  int64_t n;
  const double* q;    // [n][2][2] complex128 (re, im interleaved)
  const double* wl;   // [n] or NULL (wl_scalar)
  double wl_scalar;
  double eps;
  double* waist;      // [n][2]
  double* radii;      // [n][2]
  double* theta;      // [n]
};

__global__ void __launch_bounds__(128) k_decompose_q(const __grid_constant__ DecompArgs A) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= A.n) return;
  const double* q = A.q + b * 8;
  const double qr[2][2] = {{q[0], q[2]}, {q[4], q[6]}};
  const double qi[2][2] = {{q[1], q[3]}, {q[5], q[7]}};
  const double wl = A.wl ? A.wl[b] : A.wl_scalar;
  const double PI = 3.141592653589793;
  // eigh of the symmetrised imaginary part, ascending eigenvalues
  const double a = qi[0][0], d = qi[1][1], c = 0.5 * (qi[0][1] + qi[1][0]);
  double v[2][2];  // columns = eigenvectors
  if (c == 0.0) {
    if (a <= d) { v[0][0] = 1; v[1][0] = 0; v[0][1] = 0; v[1][1] = 1; }
    else        { v[0][0] = 0; v[1][0] = 1; v[0][1] = 1; v[1][1] = 0; }
  } else {
    const double h = 0.5 * (a - d), r = hypot(h, c);
    const double l1 = 0.5 * (a + d) - r;  // smaller eigenvalue
    // eigenvector of l1: (c, l1 - a) or (l1 - d, c); take the better conditioned
    double x = c, y = l1 - a;
    const double x2 = l1 - d, y2 = c;
    if (hypot(x2, y2) > hypot(x, y)) { x = x2; y = y2; }
    const double nn = hypot(x, y);
    v[0][0] = x / nn; v[1][0] = y / nn;
    v[0][1] = -v[1][0]; v[1][1] = v[0][0];  // orthogonal, right-handed
  }
  auto fix_det = [&]() {
    if (v[0][0] * v[1][1] - v[0][1] * v[1][0] < 0.0) { v[0][1] = -v[0][1]; v[1][1] = -v[1][1]; }
  };
  fix_det();
  // diagonal of V^T Q V (complex)
  double dr[2], di[2];
  for (int k = 0; k < 2; ++k) {
    double sr = 0.0, si = 0.0;
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j) {
        sr += v[i][k] * qr[i][j] * v[j][k];
        si += v[i][k] * qi[i][j] * v[j][k];
      }
    dr[k] = sr; di[k] = si;
  }
  auto waist_of = [&](double im) {
    return fabs(im) > A.eps ? sqrt(fabs(wl / (PI * im))) : INFINITY;
  };
  if (waist_of(di[0]) < waist_of(di[1])) {  // larger waist first
    double t = dr[0]; dr[0] = dr[1]; dr[1] = t;
    t = di[0]; di[0] = di[1]; di[1] = t;
    for (int i = 0; i < 2; ++i) { t = v[i][0]; v[i][0] = v[i][1]; v[i][1] = t; }
    fix_det();
  }
  for (int k = 0; k < 2; ++k) {
    A.waist[2 * b + k] = waist_of(di[k]);
    A.radii[2 * b + k] = fabs(dr[k]) > A.eps ? 1.0 / dr[k] : INFINITY;
  }
  A.theta[b] = atan2(v[1][0], v[0][0]);
}

// ---------------------------------------------------------------- Q^-1 of beams
// Complex float64 with the products written out; the reference's einsum adds
// the same terms (R diag R^T has two non-zero terms per entry).
struct BeamQArgs {
  int64_t n;
  const double* waist;  // [n][2]
  const double* radii;  // [n][2]
  const double* wl;     // [n] or NULL (wl_scalar)
  double wl_scalar;
  const double* theta;  // [n] or NULL (theta_scalar)
  double theta_scalar;
  double* qxy;          // [n][2] complex128, or NULL
  double* q;            // [n][2][2] complex128, or NULL
};

__global__ void __launch_bounds__(128) k_beam_q_inv(const __grid_constant__ BeamQArgs A) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= A.n) return;
  const double PI = 3.141592653589793;
  const double wl = A.wl ? A.wl[b] : A.wl_scalar;
  double re[2], im[2];
  for (int k = 0; k < 2; ++k) {
    const double w = A.waist[2 * b + k], r = A.radii[2 * b + k];
    im[k] = wl / (PI * (w * w));
    re[k] = isinf(r) ? 0.0 : -1.0 / r;
  }
  if (A.qxy) {
    A.qxy[4 * b + 0] = re[0]; A.qxy[4 * b + 1] = im[0];
    A.qxy[4 * b + 2] = re[1]; A.qxy[4 * b + 3] = im[1];
  }
  if (A.q) {
    double s, c;
    sincos(A.theta ? A.theta[b] : A.theta_scalar, &s, &c);
    // R = [[c, -s], [s, c]]:  (R D R^T)_ip = R_i0 d0 R_p0 + R_i1 d1 R_p1
    const double R[2][2] = {{c, -s}, {s, c}};
    double* o = A.q + 8 * b;
    for (int i = 0; i < 2; ++i)
      for (int p = 0; p < 2; ++p) {
        const double a0 = R[i][0] * R[p][0], a1 = R[i][1] * R[p][1];
        o[4 * i + 2 * p + 0] = a0 * re[0] + a1 * re[1];
        o[4 * i + 2 * p + 1] = a0 * im[0] + a1 * im[1];
      }
  }
}

// ---------------------------------------------------------------- Qinv_ABCD
struct zc {
  double re, im;
};
__device__ __forceinline__ zc zadd(zc a, zc b) { return zc{a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ zc zsub(zc a, zc b) { return zc{a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ zc zmul(zc a, zc b) { return zc{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
// Smith's complex division (Smith 1962): scales by the larger component of
// the divisor, so no intermediate overflows where the quotient does not.
__device__ __forceinline__ zc zdiv(zc a, zc b) {
  if (fabs(b.re) >= fabs(b.im)) {
    const double r = b.im / b.re, d = b.re + b.im * r;
    return zc{(a.re + a.im * r) / d, (a.im - a.re * r) / d};
  }
  const double r = b.re / b.im, d = b.re * r + b.im;
  return zc{(a.re * r + a.im) / d, (a.im * r - a.re) / d};
}
__device__ __forceinline__ double cabs1(zc a) { return fabs(a.re) + fabs(a.im); }

struct QabcdArgs {
  int64_t n;
  const double* q;                // [n][2][2] complex128
  const double *a, *b, *c, *d;    // [n][2][2] float64
  double* out;                    // [n][2][2] complex128
};

__global__ void __launch_bounds__(128) k_qinv_abcd(const __grid_constant__ QabcdArgs A) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= A.n) return;
  zc Q[2][2];
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) Q[i][j] = zc{A.q[8 * t + 4 * i + 2 * j], A.q[8 * t + 4 * i + 2 * j + 1]};
  const double *a = A.a + 4 * t, *b = A.b + 4 * t, *c = A.c + 4 * t, *d = A.d + 4 * t;
  zc L[2][2], Rh[2][2];  // lhs = A + B Q, rhs = C + D Q
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) {
      zc bq = zadd(zmul(zc{b[2 * i], 0.0}, Q[0][j]), zmul(zc{b[2 * i + 1], 0.0}, Q[1][j]));
      zc dq = zadd(zmul(zc{d[2 * i], 0.0}, Q[0][j]), zmul(zc{d[2 * i + 1], 0.0}, Q[1][j]));
      L[i][j] = zadd(zc{a[2 * i + j], 0.0}, bq);
      Rh[i][j] = zadd(zc{c[2 * i + j], 0.0}, dq);
    }
  // LU with partial pivoting on |re| + |im| (the LAPACK getrf pivot rule)
  if (cabs1(L[1][0]) > cabs1(L[0][0])) {
    for (int j = 0; j < 2; ++j) {
      zc s = L[0][j]; L[0][j] = L[1][j]; L[1][j] = s;
      s = Rh[0][j]; Rh[0][j] = Rh[1][j]; Rh[1][j] = s;
    }
  }
  const zc l10 = zdiv(L[1][0], L[0][0]);
  const zc u11 = zsub(L[1][1], zmul(l10, L[0][1]));
  double* o = A.out + 8 * t;
  for (int j = 0; j < 2; ++j) {
    const zc y1 = zsub(Rh[1][j], zmul(l10, Rh[0][j]));
    const zc x1 = zdiv(y1, u11);
    const zc x0 = zdiv(zsub(Rh[0][j], zmul(L[0][1], x1)), L[0][0]);
    o[2 * j] = x0.re; o[2 * j + 1] = x0.im;
    o[4 + 2 * j] = x1.re; o[4 + 2 * j + 1] = x1.im;
  }
}

// ---------------------------------------------------------------- textbook helpers
struct ProfileArgs {
  int64_t n;
  const double *z, *w0, *wl;  // [n] each (broadcast on the host), NULL where unused
  const double* zr_in;        // [n] Rayleigh ranges given (w_z, R), or NULL: from w0, wl
  double *zr, *wz, *r;        // [n] each, or NULL
  double* qinv;               // [n] complex128, or NULL
};

__global__ void __launch_bounds__(256) k_beam_profile(const __grid_constant__ ProfileArgs A) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.n) return;
  const double PI = 3.141592653589793;
  const double z = A.z ? A.z[i] : 0.0, w0 = A.w0 ? A.w0[i] : 0.0, wl = A.wl ? A.wl[i] : 0.0;
  const double zr = A.zr_in ? A.zr_in[i] : (PI * (w0 * w0)) / wl;  // zR
  const double q = z / zr;
  const double wz = w0 * sqrt(1.0 + q * q);                          // w_z
  const bool focus = fabs(z) < 1e-10;
  const double ratio = focus ? 0.0 : zr / z;
  const double r = focus ? INFINITY : z * (1.0 + ratio * ratio);     // R
  if (A.zr) A.zr[i] = zr;
  if (A.wz) A.wz[i] = wz;
  if (A.r) A.r[i] = r;
  if (A.qinv) {  // q_inv(z, w0, wl): i wl / (pi w0^2) at the focus, else -1/R + i wl / (pi w(z)^2)
    A.qinv[2 * i] = focus ? 0.0 : -1.0 / r;
    A.qinv[2 * i + 1] = focus ? wl / (PI * (w0 * w0)) : wl / (PI * (wz * wz));
  }
}

struct BeamArgs {
  int64_t n;
  const double *x, *y, *ox, *oy;  // [n] each (broadcast on the host)
  const double* qinv;             // [n] complex128
  const double* k;                // [n]
  double* out;                    // [n] complex128
};

// exp(1j * k * ((x + ox)^2 + (y + oy)^2) / 2 * q_inv), left to right as written
__global__ void __launch_bounds__(256) k_gaussian_beam(const __grid_constant__ BeamArgs A) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.n) return;
  const double u = A.x[i] + A.ox[i], v = A.y[i] + A.oy[i];
  const double s = (A.k[i] * (u * u + v * v)) / 2.0;  // real factor of 1j * s * q
  const double qr = A.qinv[2 * i], qi = A.qinv[2 * i + 1];
  // 1j * s * (qr + 1j qi) = -s qi + 1j s qr
  const double mag = exp(-(s * qi));
  double sn, cs;
  sincos(s * qr, &sn, &cs);
  A.out[2 * i] = mag * cs;
  A.out[2 * i + 1] = mag * sn;
}

static int sm_count_source() {
  static int cached = 0;
  if (!cached) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&cached, cudaDevAttrMultiProcessorCount, dev);
    if (cached <= 0) cached = 148;
  }
  return cached;
}

}  // namespace tg

using namespace tg;

extern "C" int tg_source_count(int64_t num_approx, int32_t random, int64_t* n_rays) {
  if (!n_rays) return TG_ERR_INVALID;
  if (random) {
    if (num_approx < 1) return TG_ERR_INVALID;
    *n_rays = num_approx;
    return TG_OK;
  }
  RingLayout L;
  int st = ring_layout(num_approx, 1.0, &L);
  if (st != TG_OK) return st;
  *n_rays = L.total;
  return TG_OK;
}

extern "C" int tg_source_generate(int32_t kind, int32_t random, int64_t num_approx, uint64_t seed,
                                  double extent, double off_x, double off_y, double* out,
                                  int64_t capacity, void* stream) {
  if (kind != 0 && kind != 1) return TG_ERR_INVALID;
  SourceArgs A;
  std::memset(&A, 0, sizeof(A));
  if (random) {
    if (num_approx < 1) return TG_ERR_INVALID;
    A.L.total = num_approx;
    A.L.extent = extent;
  } else {
    int st = ring_layout(num_approx, extent, &A.L);
    if (st != TG_OK) return st;
  }
  if (!out || capacity < A.L.total) return TG_ERR_WORKSPACE;
  A.kind = kind;
  A.off_x = off_x;
  A.off_y = off_y;
  A.out = out;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (random) {
    int64_t blocks = (A.L.total + 255) / 256;
    if (blocks > (int64_t)sm_count_source() * 8) blocks = (int64_t)sm_count_source() * 8;
    k_source_random<<<(int)blocks, 256, 0, s>>>(A, seed);
  } else {
    k_source_rings<<<(A.L.rings + 127) / 128, 128, 0, s>>>(A);
  }
  return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
}

extern "C" int tg_decompose_q_inv(int64_t n, const double* q_inv, const double* wavelength,
                                  double wavelength_scalar, double eps, double* waist, double* radii,
                                  double* theta, void* stream) {
  if (n < 0) return TG_ERR_INVALID;
  if (n > 0 && (!q_inv || !waist || !radii || !theta)) return TG_ERR_INVALID;
  if (n == 0) return TG_OK;
  DecompArgs A;
  A.n = n;
  A.q = q_inv;
  A.wl = wavelength;
  A.wl_scalar = wavelength_scalar;
  A.eps = eps;
  A.waist = waist;
  A.radii = radii;
  A.theta = theta;
  k_decompose_q<<<(int)((n + 127) / 128), 128, 0, reinterpret_cast<cudaStream_t>(stream)>>>(A);
  return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
}

extern "C" int tg_beam_q_inv(int64_t n, const double* waist, const double* radii, const double* wavelength,
                             double wavelength_scalar, const double* theta, double theta_scalar,
                             double* q_xy, double* q_inv, void* stream) {
  if (n < 0) return TG_ERR_INVALID;
  if (n > 0 && (!waist || !radii || (!q_xy && !q_inv))) return TG_ERR_INVALID;
  if (n == 0) return TG_OK;
  BeamQArgs A;
  A.n = n;
  A.waist = waist;
  A.radii = radii;
  A.wl = wavelength;
  A.wl_scalar = wavelength_scalar;
  A.theta = theta;
  A.theta_scalar = theta_scalar;
  A.qxy = q_xy;
  A.q = q_inv;
  k_beam_q_inv<<<(int)((n + 127) / 128), 128, 0, reinterpret_cast<cudaStream_t>(stream)>>>(A);
  return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
}

extern "C" int tg_qinv_abcd(int64_t n, const double* q_inv, const double* a, const double* b,
                            const double* c, const double* d, double* out, void* stream) {
  if (n < 0) return TG_ERR_INVALID;
  if (n > 0 && (!q_inv || !a || !b || !c || !d || !out)) return TG_ERR_INVALID;
  if (n == 0) return TG_OK;
  QabcdArgs A{n, q_inv, a, b, c, d, out};
  k_qinv_abcd<<<(int)((n + 127) / 128), 128, 0, reinterpret_cast<cudaStream_t>(stream)>>>(A);
  return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
}

extern "C" int tg_beam_profile(int64_t n, const double* z, const double* w0, const double* wavelength,
                               const double* z_r_in, double* z_r, double* w_z, double* r, double* q_inv,
                               void* stream) {
  if (n < 0) return TG_ERR_INVALID;
  if (n == 0) return TG_OK;
  // every requested output has its inputs (q_inv takes its own zR from w0, wavelength)
  const bool zr_src = z_r_in || (w0 && wavelength);
  if (!z_r && !w_z && !r && !q_inv) return TG_ERR_INVALID;
  if (z_r && !zr_src) return TG_ERR_INVALID;
  if (w_z && !(w0 && z && zr_src)) return TG_ERR_INVALID;
  if (r && !(z && zr_src)) return TG_ERR_INVALID;
  if (q_inv && (z_r_in || !(z && w0 && wavelength))) return TG_ERR_INVALID;
  ProfileArgs A{n, z, w0, wavelength, z_r_in, z_r, w_z, r, q_inv};
  k_beam_profile<<<(int)((n + 255) / 256), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(A);
  return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
}

extern "C" int tg_gaussian_beam(int64_t n, const double* x, const double* y, const double* q_inv,
                                const double* k, const double* offset_x, const double* offset_y,
                                double* out, void* stream) {
  if (n < 0) return TG_ERR_INVALID;
  if (n > 0 && (!x || !y || !q_inv || !k || !offset_x || !offset_y || !out)) return TG_ERR_INVALID;
  if (n == 0) return TG_OK;
  BeamArgs A{n, x, y, offset_x, offset_y, q_inv, k, out};
  k_gaussian_beam<<<(int)((n + 255) / 256), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(A);
  return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
}
