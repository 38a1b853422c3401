// field_adjoint.cu - adjoint of the Gaussian-beamlet detector field
// (make_gaussian_image, gaussian.py:225-316, and the input-plane field,
// gaussian.py:372-409, under jax.grad / jax.vjp).
//
// Every beam's field is F_b(row, col) = amp_b E_b with
//   E_b = exp(log pref_b + i k pl_b + i Phi_b(row, col)),
//   Phi_b = kap_cc col^2 + kap_rr row^2 + kap_rc row col + kap_c col + kap_r row + kap_0
// (complex coefficients: the real part is the phase, the imaginary part the
// Gaussian envelope; field_common.cuh).  For a real loss L with upstream
// gradient G = dL/dRe F + i dL/dIm F (PyTorch's convention for complex
// tensors) and any real parameter p of beam b,
//   dL/dp = Re( amp_b [ i sum_j (d kap_j / dp) mu_j + (d log pref / dp) mu_1 ] ),
//   mu_j  = sum_pixels conj(G) E_b m_j,   m_j in {col^2, row^2, row col, col, row, 1},
// dL/d pl_b = -k Im(amp_b mu_1) and the amplitude's gradient is conj(mu_1).
// So the adjoint is
//   1. k_field_moments: the six complex moments of every beam, a reduction
//      over (beam, pixel) that evaluates E_b with the direct kernel's exact
//      fixed-point phase and float32 recurrence (unit-amplitude records),
//      about the beam's envelope centre for conditioning; for separable
//      beams (method TG_FIELD_SEPARABLE) instead one split-BF16 GEMM on the
//      tensor cores and a pass over the rows (k_adj_gplanes, k_adj_uplanes,
//      the forward's k_field_gemm, k_adj_sep_moments; see below);
//   2. k_field_moment_sum: the per-block partials summed in a fixed order;
//   3. k_field_beam_grad<4>: per beam, the preparation arithmetic again in
//      float64 forward mode for d kap / dp and d log pref / dp, contracted
//      with the moments.  The directions (the central ray's x, y, dx, dy and
//      the model's step parameters, up to 32 a launch) run in groups on
//      blockIdx.y: the central ray's four together, whose group computes the
//      ABCD algebra in plain float64 (it does not depend on the ray) and the
//      derivatives of the few ray-dependent terms in closed form, and the
//      step parameters two at a time;
//   4. k_field_model_sum: the model parameters' per-block sums in a fixed
//      order, written as per-step sums in the layout of tg_trace_vjp.
// Every reduction runs in a fixed order, so the gradients are deterministic.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "field_common.cuh"
#include "tg_common.cuh"

TG_DEFINE_ERROR_WORD(fadj)

namespace tg {

// ------------------------------------------------------------ moments
constexpr int kML = 16;               // columns per lane (one strip)
constexpr int kMRows = 8;             // rows per staged band
constexpr int kMBeams = 64;           // beams per block
constexpr int kMThreads = 256;
constexpr int kMCols = 32 * kML;      // columns per block (one warp's strips)
constexpr float kMSkipLog = -60.f;    // strip below e^-60 of unit amplitude: no contribution
constexpr float kMRecurMax = 80.f;    // geometric recurrence while |log| stays below

struct MomArgs {
  const BeamFast* beams;  // unit-amplitude records
  const float2* g;        // [h][w] upstream gradient
  int64_t n;
  int32_t h, w, col_chunks, rows_per_split;
  float* part;            // [gridDim.x][n][12]
};

__device__ __forceinline__ float2 exp_turn(float logamp, uint64_t turns) {
  const int32_t hi = (int32_t)(turns >> 32);  // [-1/2, 1/2) turn
  const float ang = (float)hi * 1.4629180792671596e-09f;  // 2 pi / 2^32
  float s, c;
  __sincosf(ang, &s, &c);
  const float a = __expf(logamp);
  return make_float2(a * c, a * s);
}

__global__ void __launch_bounds__(kMThreads, 3) k_field_moments(const __grid_constant__ MomArgs A) {
  // the band of the gradient image, transposed so that lane l's column j of
  // its strip sits at [row][j][l] (conflict-free reads)
  __shared__ float2 sg[kMRows][kML][32];
  __shared__ double acc[kMBeams][12];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int cx = blockIdx.x % A.col_chunks, rs = blockIdx.x / A.col_chunks;
  const int cbase = cx * kMCols;
  const int col0 = cbase + lane * kML;
  const int r_begin = rs * A.rows_per_split;
  const int r_end = min(A.h, r_begin + A.rows_per_split);
  const int64_t b0 = (int64_t)blockIdx.y * kMBeams;
  const int nb = (int)min((int64_t)kMBeams, A.n - b0);
  for (int i = threadIdx.x; i < kMBeams * 12; i += blockDim.x) (&acc[0][0])[i] = 0.0;
  const uint64_t ucol = (uint64_t)col0, ucol2 = ucol * ucol, ustep = 2 * ucol + 1;
  for (int band = r_begin; band < r_end; band += kMRows) {
    __syncthreads();
    for (int i = threadIdx.x; i < kMRows * kMCols; i += blockDim.x) {
      const int rr = i / kMCols, cc = i % kMCols;
      const int row = band + rr, col = cbase + cc;
      sg[rr][cc % kML][cc / kML] =
          (row < r_end && col < A.w) ? A.g[(size_t)row * A.w + col] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    for (int k = warp; k < nb; k += kMThreads / 32) {
      float s[12];
#pragma unroll
      for (int i = 0; i < 12; ++i) s[i] = 0.f;
      if (col0 < A.w) {
        const BeamFast B = A.beams[b0 + k];
        // exact phase at the strip start of the band's first row, its step to
        // the next row (and that step's own step), and the column step
        const uint64_t ub = (uint64_t)band;
        uint64_t th_row = B.p_cc * ucol2 + B.p_rr * (ub * ub) + B.p_rc * (ub * ucol) + B.p_c * ucol +
                          B.p_r * ub + B.p_0;
        uint64_t dth_row = B.p_rr * (2 * ub + 1) + B.p_rc * ucol + B.p_r;
        uint64_t dth_col = B.p_cc * ustep + B.p_rc * ub + B.p_c;
        for (int rr = 0; rr < kMRows; ++rr) {
          const int row = band + rr;
          if (row >= r_end) break;
          uint64_t th = th_row, dth = dth_col;
          th_row += dth_row;
          dth_row += 2 * B.p_rr;
          dth_col += B.p_rc;
          const float dr = (float)row - B.r0, dc = (float)col0 - B.c0;
          const float la = B.e0 - (B.b_cc * dc * dc + B.b_rr * dr * dr + B.b_rc * dr * dc + B.l_c * dc + B.l_r * dr);
          const float dla = -(B.b_cc * (2.f * dc + 1.f) + B.b_rc * dr + B.l_c);
          const float jl = (float)(kML - 1);
          const float la_end = la + jl * dla - B.b_cc * jl * (jl - 1.f);
          const float dla_end = dla - 2.f * B.b_cc * (jl - 1.f);
          float jv = B.b_cc > 0.f ? 0.5f + dla / (2.f * B.b_cc) : (dla > 0.f ? jl : 0.f);
          jv = fminf(fmaxf(jv, 0.f), jl);
          const float la_max = fmaxf(fmaxf(la, la_end), la + jv * dla - B.b_cc * jv * (jv - 1.f));
          if (!(la_max > kMSkipLog)) continue;
          // sums of conj(G) E times 1, j and j^2 over the strip (j the column
          // within it, a compile-time constant), shifted to the moments about
          // the centre, c = dc + j, once per strip
          float s0r = 0.f, s0i = 0.f, t1r = 0.f, t1i = 0.f, t2r = 0.f, t2i = 0.f;
          auto add = [&](int j, float2 z) {  // conj(G) E at column col0 + j
            if (col0 + j < A.w) {
              const float2 g = sg[rr][j][lane];
              const float pr = g.x * z.x + g.y * z.y, pi = g.x * z.y - g.y * z.x;
              s0r += pr; s0i += pi;
              t1r = fmaf((float)j, pr, t1r); t1i = fmaf((float)j, pi, t1i);
              t2r = fmaf((float)(j * j), pr, t2r); t2i = fmaf((float)(j * j), pi, t2i);
            }
          };
          if (la > -kMRecurMax && fabsf(dla) < kMRecurMax && fabsf(dla_end) < kMRecurMax) {
            float2 z = exp_turn(la, th), wv = exp_turn(dla, dth);
            const float rr_ = B.rho_re, ri = B.rho_im;
#pragma unroll
            for (int j = 0; j < kML; ++j) {
              add(j, z);
              z = make_float2(z.x * wv.x - z.y * wv.y, z.x * wv.y + z.y * wv.x);
              wv = make_float2(wv.x * rr_ - wv.y * ri, wv.x * ri + wv.y * rr_);
            }
          } else {
            const uint64_t ddth = 2 * B.p_cc;
#pragma unroll
            for (int j = 0; j < kML; ++j) {
              const float fj = (float)j;
              add(j, exp_turn(la + fj * dla - B.b_cc * fj * (fj - 1.f), th));
              th += dth;
              dth += ddth;
            }
          }
          const float s1r = fmaf(dc, s0r, t1r), s1i = fmaf(dc, s0i, t1i);
          const float s2r = fmaf(dc, fmaf(dc, s0r, 2.f * t1r), t2r), s2i = fmaf(dc, fmaf(dc, s0i, 2.f * t1i), t2i);
          // moments about the centre: 1, dc, dr, dc^2, dr dc, dr^2
          s[0] += s0r; s[1] += s0i;
          s[2] += s1r; s[3] += s1i;
          s[4] = fmaf(dr, s0r, s[4]); s[5] = fmaf(dr, s0i, s[5]);
          s[6] += s2r; s[7] += s2i;
          s[8] = fmaf(dr, s1r, s[8]); s[9] = fmaf(dr, s1i, s[9]);
          s[10] = fmaf(dr * dr, s0r, s[10]); s[11] = fmaf(dr * dr, s0i, s[11]);
        }
      }
#pragma unroll
      for (int i = 0; i < 12; ++i) {
        float v = s[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) acc[k][i] += (double)v;
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nb * 12; i += blockDim.x)
    A.part[((size_t)blockIdx.x * A.n + b0) * 12 + i] = (float)acc[i / 12][i % 12];
}

// moments[b][i] = sum over the blocks' partials in block order (float64)
// The sum is carried as an unevaluated float32 pair (TwoSum per partial,
// exact to ~2^-48 of the terms) and rounded to float64 once with integer
// operations: no float64 instruction, which GB300 issues at ~1/64 of the
// float32 rate.
__global__ void k_field_moment_sum(const float* __restrict__ part, int nparts, int64_t n,
                                   double* __restrict__ mom) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * 12) return;
  float hi = 0.f, lo = 0.f;
  for (int p = 0; p < nparts; ++p) {
    const float v = part[(size_t)p * n * 12 + i];
    const float s = __fadd_rn(hi, v), bb = __fsub_rn(s, hi);
    lo = __fadd_rn(lo, __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(v, bb)));
    hi = s;
  }
  mom[i] = add_f64_f32(f32_to_f64(hi), lo);
}

// ------------------------------------------------------------ dual numbers
// value + derivatives along N directions (forward mode, float64)
template <int N>
struct Du {
  double v, d[N > 0 ? N : 1];  // N = 0: a plain value (d unused)
};
template <int N>
__device__ __forceinline__ Du<N> dc_(double v) {
  Du<N> r;
  r.v = v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = 0.0;
  return r;
}
template <int N>
__device__ __forceinline__ Du<N> operator+(const Du<N>& a, const Du<N>& b) {
  Du<N> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ Du<N> operator-(const Du<N>& a, const Du<N>& b) {
  Du<N> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ Du<N> operator*(const Du<N>& a, const Du<N>& b) {
  Du<N> r;
  r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ Du<N> operator*(double s, const Du<N>& a) {
  Du<N> r;
  r.v = s * a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = s * a.d[i];
  return r;
}
// Division by one float64 reciprocal (GB300's float64 divide is a
// multi-instruction sequence on its slow float64 pipe): 1 divide instead of
// N + 1.
template <int N>
__device__ __forceinline__ Du<N> operator/(const Du<N>& a, const Du<N>& b) {
  const double inv = 1.0 / b.v;
  Du<N> r;
  r.v = a.v * inv;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * inv;
  return r;
}
template <int N>
__device__ __forceinline__ Du<N> recip(const Du<N>& b) {
  Du<N> r;
  r.v = 1.0 / b.v;
  const double r2 = r.v * r.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -b.d[i] * r2;
  return r;
}

// complex dual and 2x2 complex dual matrices
template <int N>
struct Cx {
  Du<N> re, im;
};
template <int N>
__device__ __forceinline__ Cx<N> cx_(const Du<N>& re) { return Cx<N>{re, dc_<N>(0.0)}; }
template <int N>
__device__ __forceinline__ Cx<N> cx_(double re, double im) { return Cx<N>{dc_<N>(re), dc_<N>(im)}; }
template <int N>
__device__ __forceinline__ Cx<N> operator+(const Cx<N>& a, const Cx<N>& b) { return Cx<N>{a.re + b.re, a.im + b.im}; }
template <int N>
__device__ __forceinline__ Cx<N> operator-(const Cx<N>& a, const Cx<N>& b) { return Cx<N>{a.re - b.re, a.im - b.im}; }
template <int N>
__device__ __forceinline__ Cx<N> operator*(const Cx<N>& a, const Cx<N>& b) {
  return Cx<N>{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <int N>
__device__ __forceinline__ Cx<N> operator*(double s, const Cx<N>& a) { return Cx<N>{s * a.re, s * a.im}; }
template <int N>
__device__ __forceinline__ Cx<N> operator*(const Du<N>& s, const Cx<N>& a) { return Cx<N>{s * a.re, s * a.im}; }
template <int N>
__device__ __forceinline__ Cx<N> operator/(const Cx<N>& a, const Cx<N>& b) {
  const Du<N> inv = recip(b.re * b.re + b.im * b.im);  // one divide for both parts
  return Cx<N>{(a.re * b.re + a.im * b.im) * inv, (a.im * b.re - a.re * b.im) * inv};
}

template <int N>
struct M2 {
  Cx<N> a, b, c, d;  // [[a, b], [c, d]]
};
template <int N>
__device__ __forceinline__ M2<N> operator*(const M2<N>& x, const M2<N>& y) {
  return M2<N>{x.a * y.a + x.b * y.c, x.a * y.b + x.b * y.d, x.c * y.a + x.d * y.c, x.c * y.b + x.d * y.d};
}
template <int N>
__device__ __forceinline__ M2<N> operator+(const M2<N>& x, const M2<N>& y) {
  return M2<N>{x.a + y.a, x.b + y.b, x.c + y.c, x.d + y.d};
}
template <int N>
__device__ __forceinline__ M2<N> inv2(const M2<N>& m) {  // explicit inverse (inf / nan when singular)
  const Cx<N> det = m.a * m.d - m.b * m.c;
  const Cx<N> one = cx_<N>(1.0, 0.0);
  const Cx<N> r = one / det;
  const Cx<N> z = cx_<N>(0.0, 0.0);
  return M2<N>{m.d * r, (z - m.b) * r, (z - m.c) * r, m.a * r};
}
// nan_to_num of the reference (gaussian.py:283-287): a non-finite entry
// becomes 0 (and so does its derivative)
template <int N>
__device__ __forceinline__ Du<N> fin0(const Du<N>& a) { return isfinite(a.v) ? a : dc_<N>(0.0); }
template <int N>
__device__ __forceinline__ M2<N> nan0(const M2<N>& m) {
  auto f = [](const Cx<N>& c) { return Cx<N>{fin0(c.re), fin0(c.im)}; };
  return M2<N>{f(m.a), f(m.b), f(m.c), f(m.d)};
}

// Products with a constant (N = 0) factor: a dual times a plain value costs
// N + 1 multiplies instead of 2N + 1 (float64 is the adjoint's bound).
template <int N, typename = std::enable_if_t<(N > 0)>>
__device__ __forceinline__ Du<N> operator*(const Du<N>& a, const Du<0>& b) {
  return b.v * a;
}
template <int N, typename = std::enable_if_t<(N > 0)>>
__device__ __forceinline__ Du<N> operator*(const Du<0>& a, const Du<N>& b) {
  return a.v * b;
}
template <int N, typename = std::enable_if_t<(N > 0)>>
__device__ __forceinline__ Cx<N> operator*(const Cx<N>& a, const Cx<0>& b) {
  return Cx<N>{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <int N, typename = std::enable_if_t<(N > 0)>>
__device__ __forceinline__ Cx<N> operator*(const Cx<0>& a, const Cx<N>& b) {
  return Cx<N>{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <int N, typename = std::enable_if_t<(N > 0)>>
__device__ __forceinline__ M2<N> operator*(const M2<N>& x, const M2<0>& y) {
  return M2<N>{x.a * y.a + x.b * y.c, x.a * y.b + x.b * y.d, x.c * y.a + x.d * y.c, x.c * y.b + x.d * y.d};
}
template <int N, typename = std::enable_if_t<(N > 0)>>
__device__ __forceinline__ M2<N> operator*(const M2<0>& x, const M2<N>& y) {
  return M2<N>{x.a * y.a + x.b * y.c, x.a * y.b + x.b * y.d, x.c * y.a + x.d * y.c, x.c * y.b + x.d * y.d};
}

// ------------------------------------------------------------ beam gradient
// Direction groups, 64 threads a block.  Measured on the separable
// 16,384-beam adjoint (whole call; Lens + Detector: the central ray's four
// directions and three step parameters): one launch per group of 4
// directions 0.93 ms (8 directions a thread, 14 KB of stack: 1.40 ms); all
// groups in one launch (blockIdx.y) 0.90 ms; the central-ray group without
// dual parts in the matrix algebra 0.82 ms; step groups carried at the
// narrowest width that holds them 0.76 ms, and at most 2 step directions a
// group 0.73 ms (1: 0.78; the central ray in groups of 2: 0.76); the
// central ray's group in closed form (beam_grad_ray) 0.69 ms, bit-identical
// across these layouts; the step groups with their constant factors (Q1,
// Q1^-1, the central ray, the pixel map) as plain values 0.65 ms.  The
// kernel takes 254 registers, so an SM holds 8 of its warps, and it keeps
// the float64 pipe ~86 % busy; dual and complex divisions by one float64
// reciprocal (1 divide instead of N + 1, or 2 (N + 1) for a complex
// quotient) 0.65 -> 0.64 ms.
constexpr int kBGThreads = 64;
constexpr int kBGDirs = 4;          // directions a thread carries (at most)
constexpr int kBGRayDirs = 4;       // central-ray directions a thread carries
constexpr int kBGStepDirs = 2;      // model-step directions a thread carries
constexpr int kBGLaunchDirs = 32;   // directions a launch carries (groups on blockIdx.y)
enum DirKind : int32_t { DIR_X = 0, DIR_Y = 1, DIR_DX = 2, DIR_DY = 3, DIR_STEP = 4 };

struct BGArgs {
  int64_t n;
  const double *x, *y, *dx, *dy;
  const double* pl;
  const float* amp;  // complex64 pairs
  const double *waist, *radii;
  const double* wl;
  double wl_scalar;
  const double* theta;
  PixMap pm;
  const BeamFast* rec;  // unit-amplitude records: the envelope centres
  const double* mom;    // [n][12] moments about the centres
  int32_t input_plane;
  int32_t n_dir;  // directions of this launch
  int32_t group_first[kBGLaunchDirs], group_n[kBGLaunchDirs];  // group blockIdx.y: its directions
  int32_t dir_kind[kBGLaunchDirs], dir_step[kBGLaunchDirs], dir_a[kBGLaunchDirs];  // dir_a: a[] entry, -1 = angle
  double dir_seed[kBGLaunchDirs];                                                 // d a[dir_a] / d parameter
  double *gx, *gy, *gdx, *gdy;  // per beam, for DIR_X .. DIR_DY directions (may be NULL)
  double* gpl;                  // per beam d L / d pathlength (may be NULL)
  float* gamp;                  // per beam complex64 gradient of the amplitude (may be NULL)
  double* model_part;           // [direction][gridDim.x] sums over the block's beams (DIR_STEP)
};

// One beam's contributions along the model-step directions [g0, g0 + nd)
// of the launch (nd <= ND): the ABCD matrices, Q2, B^-1, P, the prefactor
// and everything built from them carry ND dual directions; Q1, Q1^-1, the
// central ray and the pixel map are constants, so their products with duals
// cost N + 1 float64 multiplies.  The propagated central ray is needed by
// value only (the biprism's sign).  Step groups exist only for the detector
// field: the input-plane field has no model (the host rejects its step sums).
template <int ND, int NC>
__device__ __forceinline__ void beam_grad_step(const DModel& M, const BGArgs& A, int64_t b, int g0, int nd,
                                               double (&contrib)[NC]) {
  using D = Du<ND>;
  using X = Cx<ND>;
  const double x0 = A.x[b], y0 = A.y[b], dx0 = A.dx[b], dy0 = A.dy[b];
  const double PI = 3.141592653589793;
  const double wl = A.wl ? A.wl[b] : A.wl_scalar;
  const double k = 2.0 * PI / wl, hk = 0.5 * k;
  // Q1^-1 = R diag(1/qx, 1/qy) R^T (gaussian.py:138-177): no directions
  const double wx = A.waist[2 * b], wy = A.waist[2 * b + 1];
  const double Rx = A.radii[2 * b], Ry = A.radii[2 * b + 1];
  const double qxr = isinf(Rx) ? 0.0 : -1.0 / Rx, qxi = wl / (PI * wx * wx);
  const double qyr = isinf(Ry) ? 0.0 : -1.0 / Ry, qyi = wl / (PI * wy * wy);
  const double th = A.theta ? A.theta[b] : 0.0;
  double sth, cth;
  sincos(th, &sth, &cth);
  const M2<0> Q1i{cx_<0>(cth * cth * qxr + sth * sth * qyr, cth * cth * qxi + sth * sth * qyi),
                  cx_<0>(cth * sth * (qxr - qyr), cth * sth * (qxi - qyi)),
                  cx_<0>(cth * sth * (qxr - qyr), cth * sth * (qxi - qyi)),
                  cx_<0>(sth * sth * qxr + cth * cth * qyr, sth * sth * qxi + cth * cth * qyi)};
  X Sxx, Syy, Sxy, Lx, Ly, c0;
  D ox, oy;
  X dlp = cx_<ND>(0.0, 0.0);  // d log pref as a complex dual (its derivative parts are used)
  // central ray and 5x5 ABCD (rows x, y, dx, dy, 1) with the model's
  // step parameters as directions
  double x = x0, y = y0, dx = dx0, dy = dy0;
  D m[5][5];
#pragma unroll
  for (int i = 0; i < 5; ++i)
#pragma unroll
    for (int j = 0; j < 5; ++j) m[i][j] = dc_<ND>(i == j ? 1.0 : 0.0);
  for (int s = 0; s < M.n; ++s) {
    const DStep& st = M.s[s];
    D a[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) a[j] = dc_<ND>(st.a[j]);
#pragma unroll
    for (int d = 0; d < ND; ++d) {
      if (d >= nd || A.dir_kind[g0 + d] != DIR_STEP || A.dir_step[g0 + d] != s) continue;
      if (A.dir_a[g0 + d] >= 0) {
        a[A.dir_a[g0 + d] & 3].d[d] = A.dir_seed[g0 + d];
      } else {  // rotation angle (radians): d(cos, sin) = (-sin, cos)
        a[0].d[d] = -st.a[1];
        a[1].d[d] = st.a[0];
      }
    }
    switch (st.kind) {
      case D_FREE:
        for (int j = 0; j < 5; ++j) {
          m[0][j] = m[0][j] + a[0] * m[2][j];
          m[1][j] = m[1][j] + a[0] * m[3][j];
        }
        x += dx * st.a[0];
        y += dy * st.a[0];
        break;
      case D_LENS:  // a[1] = 1/f
        for (int j = 0; j < 5; ++j) {
          m[2][j] = m[2][j] - m[0][j] * a[1];
          m[3][j] = m[3][j] - m[1][j] * a[1];
        }
        dx -= x * st.a[1];
        dy -= y * st.a[1];
        break;
      case D_SHIFT:
        m[0][4] = m[0][4] + a[0]; m[1][4] = m[1][4] + a[1];
        m[2][4] = m[2][4] + a[2]; m[3][4] = m[3][4] + a[3];
        x += st.a[0]; y += st.a[1]; dx += st.a[2]; dy += st.a[3];
        break;
      case D_BIPRISM: {
        const double sg = x > 0.0 ? 1.0 : (x < 0.0 ? -1.0 : 0.0);
        m[2][4] = m[2][4] + sg * a[0];
        dx += sg * st.a[0];
      } break;
      case D_ROTATE:
        for (int j = 0; j < 5; ++j) {
          const D r0 = m[0][j], r1 = m[1][j], r2 = m[2][j], r3 = m[3][j];
          m[0][j] = a[0] * r0 - a[1] * r1;
          m[1][j] = a[1] * r0 + a[0] * r1;
          m[2][j] = a[0] * r2 - a[1] * r3;
          m[3][j] = a[1] * r2 + a[0] * r3;
        }
        {
          const double c = st.a[0], sn = st.a[1];
          const double nx = c * x - sn * y, ny = sn * x + c * y;
          const double ndx = c * dx - sn * dy, ndy = sn * dx + c * dy;
          x = nx; y = ny; dx = ndx; dy = ndy;
        }
        break;
      default:  // D_NOP (an aberrated lens is rejected on the host)
        break;
    }
  }
  const M2<ND> Am{cx_<ND>(m[0][0]), cx_<ND>(m[0][1]), cx_<ND>(m[1][0]), cx_<ND>(m[1][1])};
  const M2<ND> Bm{cx_<ND>(m[0][2]), cx_<ND>(m[0][3]), cx_<ND>(m[1][2]), cx_<ND>(m[1][3])};
  const M2<ND> Cm{cx_<ND>(m[2][0]), cx_<ND>(m[2][1]), cx_<ND>(m[3][0]), cx_<ND>(m[3][1])};
  const M2<ND> Dm{cx_<ND>(m[2][2]), cx_<ND>(m[2][3]), cx_<ND>(m[3][2]), cx_<ND>(m[3][3])};
  // Q2^-1 = (A + B Q1^-1)^-1 (C + D Q1^-1)   (gaussian.py:92-96)
  const M2<ND> denom = Am + Bm * Q1i;
  const M2<ND> Q2 = inv2(denom) * (Cm + Dm * Q1i);
  const M2<ND> Binv = nan0(inv2(Bm));
  const M2<0> Q1 = nan0(inv2(Q1i));
  const D r2mx = x0 * m[0][0] + y0 * m[0][1] + dx0 * m[0][2] + dy0 * m[0][3];
  const D r2my = x0 * m[1][0] + y0 * m[1][1] + dx0 * m[1][2] + dy0 * m[1][3];
  // pref = amp / sqrt(det): d log pref = -d det / (2 det)
  {
    const Cx<ND> det = denom.a * denom.d - denom.b * denom.c;
    Cx<ND> dd;
    dd.re = det.re;
    dd.im = det.im;
    dd.re.v = 0.0;  // the quotient below uses only the derivative parts
    dd.im.v = 0.0;
    dlp = (-0.5) * (dd / cx_<ND>(det.re.v, det.im.v));
  }
  const M2<ND> ABinv = Am * Binv;
  const M2<ND> P = Q1 * inv2(Bm * (Am * Q1 + Bm));
  Sxx = Q2.a;
  Syy = Q2.d;
  Sxy = 0.5 * (Q2.b + Q2.c);
  const X bx = x0 * Binv.a + y0 * Binv.c;
  const X by = x0 * Binv.b + y0 * Binv.d;
  const X px = P.a * cx_<ND>(r2mx) + P.c * cx_<ND>(r2my);
  const X py = P.b * cx_<ND>(r2mx) + P.d * cx_<ND>(r2my);
  Lx = 2.0 * (cx_<ND>(m[2][4]) - bx + px);
  Ly = 2.0 * (cx_<ND>(m[3][4]) - by + py);
  const X q1 = x0 * (x0 * ABinv.a + y0 * ABinv.b) +
               y0 * (x0 * ABinv.c + y0 * ABinv.d);
  const X q2 = cx_<ND>(r2mx) * (P.a * cx_<ND>(r2mx) + P.b * cx_<ND>(r2my)) +
               cx_<ND>(r2my) * (P.c * cx_<ND>(r2mx) + P.d * cx_<ND>(r2my));
  c0 = q1 - q2;
  ox = m[0][4];
  oy = m[1][4];
  // the polynomial in (row, col): s = s0 + row u + col v
  const D s0x = dc_<ND>(A.pm.t[5]) - ox, s0y = dc_<ND>(A.pm.t[2]) - oy;
  const double ux = A.pm.t[3], uy = A.pm.t[0], vx = A.pm.t[4], vy = A.pm.t[1];
  // a^T S b with constant a and b, with a dual and b constant, with both dual
  auto quad_cc = [&](double ax, double ay, double bx2, double by2) -> X {
    return (ax * bx2) * Sxx + (ay * by2) * Syy + (ax * by2 + ay * bx2) * Sxy;
  };
  auto quad_dc = [&](const D& ax, const D& ay, double bx2, double by2) -> X {
    return (bx2 * ax) * Sxx + (by2 * ay) * Syy + (by2 * ax + bx2 * ay) * Sxy;
  };
  auto quad_dd = [&](const D& ax, const D& ay, const D& bx2, const D& by2) -> X {
    return (ax * bx2) * Sxx + (ay * by2) * Syy + (ax * by2 + ay * bx2) * Sxy;
  };
  X kap[6];  // cc, rr, rc, c, r, 0
  kap[0] = hk * quad_cc(vx, vy, vx, vy);
  kap[1] = hk * quad_cc(ux, uy, ux, uy);
  kap[2] = hk * (2.0 * quad_cc(ux, uy, vx, vy));
  kap[3] = hk * (2.0 * quad_dc(s0x, s0y, vx, vy) + vx * Lx + vy * Ly);
  kap[4] = hk * (2.0 * quad_dc(s0x, s0y, ux, uy) + ux * Lx + uy * Ly);
  kap[5] = hk * (quad_dd(s0x, s0y, s0x, s0y) + s0x * Lx + s0y * Ly + c0);
  // moments about the envelope centre -> moments of the monomials
  const double* mo = A.mom + b * 12;
  const double r0 = (double)A.rec[b].r0, cc0 = (double)A.rec[b].c0;
  double mr[6], mi[6];  // centred: 1, dc, dr, dc^2, dr dc, dr^2
  for (int i = 0; i < 6; ++i) { mr[i] = mo[2 * i]; mi[i] = mo[2 * i + 1]; }
  double ur[6], ui[6];  // by kap order: col^2, row^2, row col, col, row, 1
  ur[5] = mr[0]; ui[5] = mi[0];
  ur[3] = mr[1] + cc0 * mr[0]; ui[3] = mi[1] + cc0 * mi[0];
  ur[4] = mr[2] + r0 * mr[0]; ui[4] = mi[2] + r0 * mi[0];
  ur[0] = mr[3] + 2.0 * cc0 * mr[1] + cc0 * cc0 * mr[0];
  ui[0] = mi[3] + 2.0 * cc0 * mi[1] + cc0 * cc0 * mi[0];
  ur[1] = mr[5] + 2.0 * r0 * mr[2] + r0 * r0 * mr[0];
  ui[1] = mi[5] + 2.0 * r0 * mi[2] + r0 * r0 * mi[0];
  ur[2] = mr[4] + cc0 * mr[2] + r0 * mr[1] + r0 * cc0 * mr[0];
  ui[2] = mi[4] + cc0 * mi[2] + r0 * mi[1] + r0 * cc0 * mi[0];
  // times the amplitude: F = amp E
  const double ar = (double)A.amp[2 * b], ai = (double)A.amp[2 * b + 1];
  double wr[6], wi[6];
  for (int j = 0; j < 6; ++j) {
    wr[j] = ar * ur[j] - ai * ui[j];
    wi[j] = ar * ui[j] + ai * ur[j];
  }
  // dL/dp = Re(i sum_j dkap_j w_j + dlogpref w_1) = -sum_j Im(dkap_j w_j) + Re(dlogpref w_1)
#pragma unroll
  for (int d = 0; d < ND; ++d) {
    if (d >= nd) break;
    double g = 0.0;
    for (int j = 0; j < 6; ++j) g -= kap[j].re.d[d] * wi[j] + kap[j].im.d[d] * wr[j];
    g += dlp.re.d[d] * wr[5] - dlp.im.d[d] * wi[5];
    contrib[d] = g;
    const int kd = A.dir_kind[g0 + d];
    if (kd == DIR_X && A.gx) A.gx[b] = g;
    if (kd == DIR_Y && A.gy) A.gy[b] = g;
    if (kd == DIR_DX && A.gdx) A.gdx[b] = g;
    if (kd == DIR_DY && A.gdy) A.gdy[b] = g;
  }
  if (A.gpl && blockIdx.y == 0) A.gpl[b] = -k * wi[5];
  if (A.gamp && blockIdx.y == 0) {
    A.gamp[2 * b] = (float)ur[5];
    A.gamp[2 * b + 1] = (float)(-ui[5]);
  }
}

// The central ray's group (x, y, dx, dy): the ABCD algebra does not depend
// on the ray, so S (= Q2, or Q1^-1 in the input plane), B^-1, P and the
// prefactor are constants and only L, c0 (and, in the input plane, s0 = r -
// r1m) carry derivatives.  Their partial derivatives with respect to each
// ray coordinate are written out (float64, no dual numbers), which is about
// a third of the float64 work of carrying four dual directions through the
// whole polynomial.
template <int NC>
__device__ __forceinline__ void beam_grad_ray(const DModel& M, const BGArgs& A, int64_t b, int g0, int nd,
                                              double (&contrib)[NC]) {
  using XP = Cx<0>;
  auto cr = [](double v) { return cx_<0>(v, 0.0); };
  const double x0 = A.x[b], y0 = A.y[b], dx0 = A.dx[b], dy0 = A.dy[b];
  const double PI = 3.141592653589793;
  const double wl = A.wl ? A.wl[b] : A.wl_scalar;
  const double k = 2.0 * PI / wl, hk = 0.5 * k;
  const double wx = A.waist[2 * b], wy = A.waist[2 * b + 1];
  const double Rx = A.radii[2 * b], Ry = A.radii[2 * b + 1];
  const double qxr = isinf(Rx) ? 0.0 : -1.0 / Rx, qxi = wl / (PI * wx * wx);
  const double qyr = isinf(Ry) ? 0.0 : -1.0 / Ry, qyi = wl / (PI * wy * wy);
  const double th = A.theta ? A.theta[b] : 0.0;
  double sth, cth;
  sincos(th, &sth, &cth);
  const M2<0> Q1i{cx_<0>(cth * cth * qxr + sth * sth * qyr, cth * cth * qxi + sth * sth * qyi),
                  cx_<0>(cth * sth * (qxr - qyr), cth * sth * (qxi - qyi)),
                  cx_<0>(cth * sth * (qxr - qyr), cth * sth * (qxi - qyi)),
                  cx_<0>(sth * sth * qxr + cth * cth * qyr, sth * sth * qxi + cth * cth * qyi)};
  XP Sxx, Syy, Sxy;
  XP Lx, Ly;              // values (used in the input plane, where s0 moves with the ray)
  XP dLx[4], dLy[4], dc0[4];
  double ds0x[4], ds0y[4];  // d s0 / d (x, y, dx, dy)
  double ox, oy;
  if (A.input_plane) {  // gaussian.py:402-409: s = r1 - r1m, S = Q1^-1, L = 2 theta1m
    Sxx = Q1i.a;
    Syy = Q1i.d;
    Sxy = 0.5 * (Q1i.b + Q1i.c);
    Lx = cr(2.0 * dx0);
    Ly = cr(2.0 * dy0);
    for (int c = 0; c < 4; ++c) {
      dLx[c] = cr(c == 2 ? 2.0 : 0.0);
      dLy[c] = cr(c == 3 ? 2.0 : 0.0);
      dc0[c] = cr(0.0);
      ds0x[c] = c == 0 ? -1.0 : 0.0;
      ds0y[c] = c == 1 ? -1.0 : 0.0;
    }
    ox = x0;
    oy = y0;
  } else {
    double x = x0, y = y0, dx = dx0, dy = dy0;  // the central ray, for the biprism's sign
    double m[5][5];
    for (int i = 0; i < 5; ++i)
      for (int j = 0; j < 5; ++j) m[i][j] = i == j ? 1.0 : 0.0;
    for (int s = 0; s < M.n; ++s) {
      const DStep& st = M.s[s];
      switch (st.kind) {
        case D_FREE:
          for (int j = 0; j < 5; ++j) {
            m[0][j] = m[0][j] + st.a[0] * m[2][j];
            m[1][j] = m[1][j] + st.a[0] * m[3][j];
          }
          x += dx * st.a[0];
          y += dy * st.a[0];
          break;
        case D_LENS:
          for (int j = 0; j < 5; ++j) {
            m[2][j] = m[2][j] - m[0][j] * st.a[1];
            m[3][j] = m[3][j] - m[1][j] * st.a[1];
          }
          dx -= x * st.a[1];
          dy -= y * st.a[1];
          break;
        case D_SHIFT:
          m[0][4] += st.a[0]; m[1][4] += st.a[1]; m[2][4] += st.a[2]; m[3][4] += st.a[3];
          x += st.a[0]; y += st.a[1]; dx += st.a[2]; dy += st.a[3];
          break;
        case D_BIPRISM: {
          const double sg = x > 0.0 ? 1.0 : (x < 0.0 ? -1.0 : 0.0);
          m[2][4] += sg * st.a[0];
          dx += sg * st.a[0];
        } break;
        case D_ROTATE: {
          const double c = st.a[0], sn = st.a[1];
          for (int j = 0; j < 5; ++j) {
            const double r0 = m[0][j], r1 = m[1][j], r2 = m[2][j], r3 = m[3][j];
            m[0][j] = c * r0 - sn * r1;
            m[1][j] = sn * r0 + c * r1;
            m[2][j] = c * r2 - sn * r3;
            m[3][j] = sn * r2 + c * r3;
          }
          const double nx = c * x - sn * y, ny = sn * x + c * y;
          const double ndx = c * dx - sn * dy, ndy = sn * dx + c * dy;
          x = nx; y = ny; dx = ndx; dy = ndy;
        } break;
        default:
          break;
      }
    }
    const M2<0> Am{cr(m[0][0]), cr(m[0][1]), cr(m[1][0]), cr(m[1][1])};
    const M2<0> Bm{cr(m[0][2]), cr(m[0][3]), cr(m[1][2]), cr(m[1][3])};
    const M2<0> Cm{cr(m[2][0]), cr(m[2][1]), cr(m[3][0]), cr(m[3][1])};
    const M2<0> Dm{cr(m[2][2]), cr(m[2][3]), cr(m[3][2]), cr(m[3][3])};
    const M2<0> Q2 = inv2(Am + Bm * Q1i) * (Cm + Dm * Q1i);
    const M2<0> Binv = nan0(inv2(Bm));
    const M2<0> Q1 = nan0(inv2(Q1i));
    const M2<0> AB = Am * Binv;
    const M2<0> P = Q1 * inv2(Bm * (Am * Q1 + Bm));
    Sxx = Q2.a;
    Syy = Q2.d;
    Sxy = 0.5 * (Q2.b + Q2.c);
    const double r2mx = m[0][0] * x0 + m[0][1] * y0 + m[0][2] * dx0 + m[0][3] * dy0;
    const double r2my = m[1][0] * x0 + m[1][1] * y0 + m[1][2] * dx0 + m[1][3] * dy0;
    const XP abx = AB.a * cr(x0) + AB.b * cr(y0), aby = AB.c * cr(x0) + AB.d * cr(y0);
    const XP pmx = P.a * cr(r2mx) + P.b * cr(r2my), pmy = P.c * cr(r2mx) + P.d * cr(r2my);
    for (int c = 0; c < 4; ++c) {
      const double ex = c == 0 ? 1.0 : 0.0, ey = c == 1 ? 1.0 : 0.0;  // d (x0, y0)
      const double erx = m[0][c], ery = m[1][c];                      // d (r2mx, r2my)
      // L = 2 (m[2..3][4] - B^-1^T r1m + P^T r2m): the first part is constant
      const XP dbx = Binv.a * cr(ex) + Binv.c * cr(ey), dby = Binv.b * cr(ex) + Binv.d * cr(ey);
      const XP dpx = P.a * cr(erx) + P.c * cr(ery), dpy = P.b * cr(erx) + P.d * cr(ery);
      dLx[c] = 2.0 * (dpx - dbx);
      dLy[c] = 2.0 * (dpy - dby);
      // c0 = r1m^T (A B^-1) r1m - r2m^T P r2m
      const XP dq1 = cr(ex) * abx + cr(x0) * (AB.a * cr(ex) + AB.b * cr(ey)) + cr(ey) * aby +
                     cr(y0) * (AB.c * cr(ex) + AB.d * cr(ey));
      const XP dq2 = cr(erx) * pmx + cr(r2mx) * (P.a * cr(erx) + P.b * cr(ery)) + cr(ery) * pmy +
                     cr(r2my) * (P.c * cr(erx) + P.d * cr(ery));
      dc0[c] = dq1 - dq2;
      ds0x[c] = 0.0;
      ds0y[c] = 0.0;
    }
    Lx = cr(0.0);  // enters only with d s0, which is zero here
    Ly = cr(0.0);
    ox = m[0][4];
    oy = m[1][4];
  }
  const double s0x = A.pm.t[5] - ox, s0y = A.pm.t[2] - oy;
  const double ux = A.pm.t[3], uy = A.pm.t[0], vx = A.pm.t[4], vy = A.pm.t[1];
  auto quad = [&](double ax, double ay, double bx2, double by2) -> XP {  // a^T S b
    return (ax * bx2) * Sxx + (ay * by2) * Syy + (ax * by2 + ay * bx2) * Sxy;
  };
  // moments about the envelope centre -> moments of the monomials col, row, 1
  const double* mo = A.mom + b * 12;
  const double r0 = (double)A.rec[b].r0, cc0 = (double)A.rec[b].c0;
  const double ur3 = mo[2] + cc0 * mo[0], ui3 = mo[3] + cc0 * mo[1];
  const double ur4 = mo[4] + r0 * mo[0], ui4 = mo[5] + r0 * mo[1];
  const double ur5 = mo[0], ui5 = mo[1];
  const double ar = (double)A.amp[2 * b], ai = (double)A.amp[2 * b + 1];
  const double wr3 = ar * ur3 - ai * ui3, wi3 = ar * ui3 + ai * ur3;
  const double wr4 = ar * ur4 - ai * ui4, wi4 = ar * ui4 + ai * ur4;
  const double wr5 = ar * ur5 - ai * ui5, wi5 = ar * ui5 + ai * ur5;
  // dL/dp = -sum_j Im(dkap_j w_j) over j = col, row, 1 (kap_cc, kap_rr,
  // kap_rc and the prefactor do not move with the central ray)
  for (int d = 0; d < nd && d < NC; ++d) {
    const int kd = A.dir_kind[g0 + d];
    if (kd < DIR_X || kd > DIR_DY) continue;
    const int c = kd;  // DIR_X .. DIR_DY = 0 .. 3
    const XP k3 = hk * (2.0 * quad(ds0x[c], ds0y[c], vx, vy) + vx * dLx[c] + vy * dLy[c]);
    const XP k4 = hk * (2.0 * quad(ds0x[c], ds0y[c], ux, uy) + ux * dLx[c] + uy * dLy[c]);
    const XP k5 = hk * (2.0 * quad(ds0x[c], ds0y[c], s0x, s0y) + ds0x[c] * Lx + ds0y[c] * Ly + s0x * dLx[c] +
                        s0y * dLy[c] + dc0[c]);
    const double g = -(k3.re.v * wi3 + k3.im.v * wr3) - (k4.re.v * wi4 + k4.im.v * wr4) -
                     (k5.re.v * wi5 + k5.im.v * wr5);
    contrib[d] = g;
    if (kd == DIR_X && A.gx) A.gx[b] = g;
    if (kd == DIR_Y && A.gy) A.gy[b] = g;
    if (kd == DIR_DX && A.gdx) A.gdx[b] = g;
    if (kd == DIR_DY && A.gdy) A.gdy[b] = g;
  }
  if (A.gpl && blockIdx.y == 0) A.gpl[b] = -k * wi5;
  if (A.gamp && blockIdx.y == 0) {
    A.gamp[2 * b] = (float)ur5;
    A.gamp[2 * b + 1] = (float)(-ui5);
  }
}

// the step body with the narrowest dual width that holds a group of nd <= CAP
// directions
template <int CAP, int NC>
__device__ __forceinline__ void beam_grad_fit(const DModel& M, const BGArgs& A, int64_t b, int g0, int nd,
                                              double (&contrib)[NC]) {
  if constexpr (CAP <= 1) {
    beam_grad_step<1>(M, A, b, g0, nd, contrib);
  } else if constexpr (CAP == 2) {
    if (nd <= 1) beam_grad_step<1>(M, A, b, g0, nd, contrib);
    else beam_grad_step<2>(M, A, b, g0, nd, contrib);
  } else {
    if (nd <= 1) beam_grad_step<1>(M, A, b, g0, nd, contrib);
    else if (nd == 2) beam_grad_step<2>(M, A, b, g0, nd, contrib);
    else if (nd == 3 || CAP == 3) beam_grad_step<3>(M, A, b, g0, nd, contrib);
    else beam_grad_step<CAP>(M, A, b, g0, nd, contrib);
  }
}

// ND: directions carried by a thread; the launch's direction groups run on
// blockIdx.y (fewer directions a thread keep the dual numbers small enough
// for registers, at the cost of recomputing the values once per group).
template <int ND>
__global__ void __launch_bounds__(kBGThreads)
k_field_beam_grad(const __grid_constant__ DModel M, const __grid_constant__ BGArgs A) {
  __shared__ double red[kBGThreads][ND];
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int g0 = A.group_first[blockIdx.y], nd = A.group_n[blockIdx.y];  // this group's directions
  double contrib[ND];
#pragma unroll
  for (int d = 0; d < ND; ++d) contrib[d] = 0.0;
  bool step = false;  // the same for the whole block
  for (int d = 0; d < nd; ++d)
    if (A.dir_kind[g0 + d] == DIR_STEP) step = true;
  if (b < A.n) {
    // the dual width that fits the group: fewer directions, shorter chains
    if (step)
      beam_grad_fit<kBGStepDirs>(M, A, b, g0, nd, contrib);
    else
      beam_grad_ray(M, A, b, g0, nd, contrib);
  }
  // the block's sums of the model directions, in a fixed order
#pragma unroll
  for (int d = 0; d < ND; ++d)
    red[threadIdx.x][d] = (d < nd && A.dir_kind[g0 + d] == DIR_STEP) ? contrib[d] : 0.0;
  __syncthreads();
  for (int s = kBGThreads / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s)
#pragma unroll
      for (int d = 0; d < ND; ++d) red[threadIdx.x][d] += red[threadIdx.x + s][d];
    __syncthreads();
  }
  if ((int)threadIdx.x < nd && A.model_part)
    A.model_part[(size_t)(g0 + threadIdx.x) * gridDim.x + blockIdx.x] = red[0][threadIdx.x];
}

// raw[target[d]] = sum over blocks (in order) of direction d's per-block sums
struct ModelSumArgs {
  int32_t n_dir, blocks;
  int32_t target[kBGLaunchDirs];  // index into raw (step * 4 + slot), -1 = none
};

// One warp per direction: lane l adds blocks l, l + 32, ... in order, then a
// fixed shuffle tree (deterministic, independent of timing).
__global__ void k_field_model_sum(const double* __restrict__ part, const __grid_constant__ ModelSumArgs A,
                                  double* __restrict__ raw) {
  const int d = blockIdx.x, lane = threadIdx.x;
  if (d >= A.n_dir || A.target[d] < 0) return;  // uniform over the warp
  double a = 0.0;
  for (int bk = lane; bk < A.blocks; bk += 32) a += part[(size_t)d * A.blocks + bk];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  if (lane == 0) raw[A.target[d]] = a;
}

// ------------------------------------------- separable moments (tensor cores)
// For separable beams E_b(r, c) = V_b(r) U_b(c) (the factors of the separable
// forward), so the six moments factor through one complex GEMM:
//   X_a[r][b] = sum_c conj(G[r][c]) U_b(c) dc^a,  a = 0, 1, 2,  dc = c - c0_b,
//   mu_{a,k}[b] = sum_r V_b(r) dr^k X_a[r][b],      dr = r - r0_b,
// with (a, k) over (0,0) (1,0) (0,1) (2,0) (1,1) (0,2).  conj(G) and
// U_b dc^a go into bf16 hi + lo planes (K = the column index, contiguous) for
// the split-BF16 tcgen05 GEMM of the forward (field_gemm.cu): its "V" operand
// is conj(G) ([rows][cols]), its "U" operand the 3 x beams lines U_b dc^a
// (line a * bpad + b), so X = [rows][3 * bpad] complex.  The moments about
// the envelope centre keep dc and dr small where the beam lives (no
// cancellation between large powers).

// conj(G) as four bf16 planes [rows_pad][cols_pad] (zero beyond h x w).
__global__ void k_adj_gplanes(const float2* __restrict__ g, int h, int w, int rows_pad, int cols_pad,
                              __nv_bfloat16_raw* __restrict__ planes) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t total = (int64_t)rows_pad * cols_pad;
  if (i >= total) return;
  const int r = (int)(i / cols_pad), c = (int)(i % cols_pad);
  float re = 0.f, im = 0.f;
  if (r < h && c < w) {
    const float2 v = g[(size_t)r * w + c];
    re = v.x;
    im = -v.y;
  }
  uint32_t h2, l2;
  split_bf16x2(re, im, h2, l2);
  planes[i] = __nv_bfloat16_raw{(unsigned short)(h2 & 0xffffu)};
  planes[total + i] = __nv_bfloat16_raw{(unsigned short)(l2 & 0xffffu)};
  planes[2 * total + i] = __nv_bfloat16_raw{(unsigned short)(h2 >> 16)};
  planes[3 * total + i] = __nv_bfloat16_raw{(unsigned short)(l2 >> 16)};
}

// U_b(c) dc^a as four bf16 planes [3 * bpad][cols_pad]: one thread per (beam,
// block of 16 columns), the column factor of the separable forward (exact
// fixed-point phase stepped by 64-bit differences), three powers of dc, 32
// bytes per plane and power stored as two 16-byte vectors.  Consecutive
// threads take consecutive column blocks of one beam, so a warp's store is one
// contiguous run of a plane row.
constexpr int kAdjCols = 16;

__global__ void __launch_bounds__(128) k_adj_uplanes(const BeamFast* __restrict__ beams, int64_t n,
                                                     int64_t bpad, int w, int cols_pad,
                                                     __nv_bfloat16_raw* __restrict__ planes) {
  const int cblocks = cols_pad / kAdjCols;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= bpad * cblocks) return;
  const int64_t b = t / cblocks;
  const int c0 = (int)(t % cblocks) * kAdjCols;
  const int64_t plane = 3 * bpad * (int64_t)cols_pad;
  const bool live = b < n;
  uint64_t p2 = 0, p1 = 0;
  float cen = 0.f, bq = 0.f, bl = 0.f;
  if (live) {
    const BeamFast& B = beams[b];
    if (B.p_rc != 0 || B.b_rc != 0.f) atomicOr(&g_tg_err, 0x10u);
    p2 = B.p_cc; p1 = B.p_c; cen = B.c0; bq = B.b_cc; bl = B.l_c;
  }
  const uint64_t u0 = (uint64_t)c0;
  uint64_t th = p2 * (u0 * u0) + p1 * u0;
  uint64_t dth = p2 * (2 * u0 + 1) + p1;
  const uint64_t ddth = 2 * p2;
  float ur[kAdjCols], ui[kAdjCols];
#pragma unroll
  for (int j = 0; j < kAdjCols; ++j) {
    ur[j] = 0.f;
    ui[j] = 0.f;
    if (live && c0 + j < w) {
      const float2 z = sep_operand(0.f, bq, bl, cen, c0 + j, th);
      ur[j] = z.x;
      ui[j] = z.y;
    }
    th += dth;
    dth += ddth;
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    uint32_t rh[kAdjCols / 2], rl[kAdjCols / 2], ih[kAdjCols / 2], il[kAdjCols / 2];
#pragma unroll
    for (int j = 0; j < kAdjCols; j += 2) {
      float m0 = 1.f, m1 = 1.f;
      if (a > 0) {
        const float d0 = (float)(c0 + j) - cen, d1 = (float)(c0 + j + 1) - cen;
        m0 = a == 1 ? d0 : d0 * d0;
        m1 = a == 1 ? d1 : d1 * d1;
      }
      uint32_t h2, l2;
      split_bf16x2(ur[j] * m0, ur[j + 1] * m1, h2, l2);
      rh[j / 2] = h2; rl[j / 2] = l2;
      split_bf16x2(ui[j] * m0, ui[j + 1] * m1, h2, l2);
      ih[j / 2] = h2; il[j / 2] = l2;
    }
    const int64_t row = (int64_t)a * bpad + b;
    uint4* dst = reinterpret_cast<uint4*>(planes + row * cols_pad + c0);
    const int64_t pv = plane / 8;  // plane stride in uint4
    dst[0] = make_uint4(rh[0], rh[1], rh[2], rh[3]); dst[1] = make_uint4(rh[4], rh[5], rh[6], rh[7]);
    dst[pv] = make_uint4(rl[0], rl[1], rl[2], rl[3]); dst[pv + 1] = make_uint4(rl[4], rl[5], rl[6], rl[7]);
    dst[2 * pv] = make_uint4(ih[0], ih[1], ih[2], ih[3]); dst[2 * pv + 1] = make_uint4(ih[4], ih[5], ih[6], ih[7]);
    dst[3 * pv] = make_uint4(il[0], il[1], il[2], il[3]); dst[3 * pv + 1] = make_uint4(il[4], il[5], il[6], il[7]);
  }
}

// Moment partials from X: one thread per (beam, group of kAdjRows rows) walks
// its rows with the row factor V_b(r) (exact fixed-point phase from the
// group's first row, as the forward's V operand), float32 sums written as
// the partial of its row group; k_field_moment_sum adds the groups in order.
constexpr int kAdjRows = 32;

__global__ void __launch_bounds__(128) k_adj_sep_moments(const BeamFast* __restrict__ beams, int64_t n,
                                                         const float2* __restrict__ x, int h, int64_t bpad,
                                                         float* __restrict__ part) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n) return;
  const int r0 = (int)blockIdx.y * kAdjRows, r1 = min(h, r0 + kAdjRows);
  const BeamFast& B = beams[b];
  const uint64_t p2 = B.p_rr, p1 = B.p_r, u0 = (uint64_t)r0;
  uint64_t th = p2 * (u0 * u0) + p1 * u0 + B.p_0;
  uint64_t dth = p2 * (2 * u0 + 1) + p1;
  const uint64_t ddth = 2 * p2;
  const int64_t ld = 3 * bpad;
  float s[12];
#pragma unroll
  for (int i = 0; i < 12; ++i) s[i] = 0.f;
  for (int r = r0; r < r1; ++r) {
    const float2 v = sep_operand(B.e0, B.b_rr, B.l_r, B.r0, r, th);
    th += dth;
    dth += ddth;
    const float dr = (float)r - B.r0;
    const float2* xr = x + (size_t)r * ld + b;
    const float2 x0 = xr[0], x1 = xr[bpad], x2 = xr[2 * bpad];
    const float p0r = v.x * x0.x - v.y * x0.y, p0i = v.x * x0.y + v.y * x0.x;
    const float p1r = v.x * x1.x - v.y * x1.y, p1i = v.x * x1.y + v.y * x1.x;
    const float p2r = v.x * x2.x - v.y * x2.y, p2i = v.x * x2.y + v.y * x2.x;
    s[0] += p0r; s[1] += p0i;                                // 1
    s[2] += p1r; s[3] += p1i;                                // dc
    s[4] = fmaf(dr, p0r, s[4]); s[5] = fmaf(dr, p0i, s[5]);  // dr
    s[6] += p2r; s[7] += p2i;                                // dc^2
    s[8] = fmaf(dr, p1r, s[8]); s[9] = fmaf(dr, p1i, s[9]);  // dr dc
    const float dr2 = dr * dr;
    s[10] = fmaf(dr2, p0r, s[10]); s[11] = fmaf(dr2, p0i, s[11]);  // dr^2
  }
  float* dst = part + ((size_t)blockIdx.y * n + b) * 12;
#pragma unroll
  for (int i = 0; i < 12; ++i) dst[i] = s[i];
}

// ------------------------------------------------------------ host
struct AdjLayout {
  size_t rec, part, mom, model, total;
  int col_chunks, row_splits, rows_per_split, beam_chunks, bg_blocks;
  // separable moments on the tensor cores (method TG_FIELD_SEPARABLE)
  size_t gplanes, uplanes, xprod;
  int rows_pad, cols_pad;
  int64_t bpad;
};

static inline size_t al256a(size_t v) { return (v + 255) & ~(size_t)255; }

static AdjLayout adj_layout(int64_t n, int h, int w, int method = TG_FIELD_DIRECT) {
  AdjLayout L;
  std::memset(&L, 0, sizeof(L));
  L.col_chunks = (w + kMCols - 1) / kMCols;
  L.beam_chunks = (int)((n + kMBeams - 1) / kMBeams);
  if (L.beam_chunks < 1) L.beam_chunks = 1;
  // enough blocks to fill the GPU: split the rows when there are few beams
  const int want = 2048;
  int splits = (want + L.col_chunks * L.beam_chunks - 1) / (L.col_chunks * L.beam_chunks);
  const int max_splits = (h + kMRows - 1) / kMRows;
  if (splits > max_splits) splits = max_splits;
  if (splits < 1) splits = 1;
  L.rows_per_split = ((h + splits - 1) / splits + kMRows - 1) / kMRows * kMRows;
  L.row_splits = (h + L.rows_per_split - 1) / L.rows_per_split;
  L.bg_blocks = (int)((n + kBGThreads - 1) / kBGThreads);
  if (L.bg_blocks < 1) L.bg_blocks = 1;
  size_t off = 0;
  L.rec = off; off = al256a(off + field_records_bytes(n));
  size_t nparts = (size_t)L.col_chunks * L.row_splits;
  if (method == TG_FIELD_SEPARABLE) {  // the row groups of k_adj_sep_moments
    const size_t rg = (size_t)(h + kAdjRows - 1) / kAdjRows;
    if (rg > nparts) nparts = rg;
  }
  L.part = off; off = al256a(off + nparts * n * 12 * sizeof(float));
  L.mom = off; off = al256a(off + (size_t)n * 12 * sizeof(double));
  L.model = off; off = al256a(off + (size_t)L.bg_blocks * kBGLaunchDirs * sizeof(double));
  if (method == TG_FIELD_SEPARABLE) {
    L.rows_pad = (h + 127) / 128 * 128;
    L.cols_pad = (w + 31) / 32 * 32;
    L.bpad = (n + 127) / 128 * 128;
    L.gplanes = off; off = al256a(off + (size_t)4 * L.rows_pad * L.cols_pad * 2);
    L.uplanes = off; off = al256a(off + (size_t)4 * 3 * L.bpad * L.cols_pad * 2);
    L.xprod = off; off = al256a(off + (size_t)h * 3 * L.bpad * sizeof(float2));
  }
  L.total = off;
  return L;
}

struct Dir {
  int32_t kind, step, a;
  double seed;
  int32_t target;  // raw index, -1 for a ray direction
};

}  // namespace tg

using namespace tg;

extern "C" size_t tg_field_vjp_workspace(int64_t n_beams, int32_t h, int32_t w) {
  if (n_beams < 0 || h <= 0 || w <= 0) return 0;
  return adj_layout(n_beams, h, w).total;
}

extern "C" size_t tg_field_vjp_workspace_ex(int32_t method, int64_t n_beams, int32_t h, int32_t w) {
  if (n_beams < 0 || h <= 0 || w <= 0) return 0;
  if (method != TG_FIELD_DIRECT && method != TG_FIELD_SEPARABLE) return 0;
  return adj_layout(n_beams, h, w, method).total;
}

namespace tg {
int launch_field_gemm(const __nv_bfloat16_raw* vplanes, const __nv_bfloat16_raw* uplanes, int lines_v,
                      int lines_u, int64_t kpad, int splits, int h, int w, float2* part,
                      cudaStream_t s);  // field_gemm.cu
}

static int field_vjp_impl(const tg_model* model, const tg_beams* beams, const tg_pixel_map* pm,
                          const float* grad, const tg_field_grads* out, void* workspace, size_t ws_bytes,
                          void* stream, int method = TG_FIELD_DIRECT) {
  if (method != TG_FIELD_DIRECT && method != TG_FIELD_SEPARABLE) return TG_ERR_INVALID;
  if (!beams || !pm || !grad || !out || pm->h <= 0 || pm->w <= 0 || beams->n < 0) return TG_ERR_INVALID;
  const bool input_plane = model == nullptr;
  if (input_plane && out->raw) return TG_ERR_INVALID;  // no model, no per-step sums
  const int64_t n = beams->n;
  if (n > 0 && (!beams->x || !beams->y || !beams->dx || !beams->dy || !beams->pathlength ||
                !beams->amplitude || !beams->waist_xy || !beams->radii))
    return TG_ERR_INVALID;
  DModel dm;
  std::memset(&dm, 0, sizeof(dm));
  if (!input_plane) {
    int st = build_dmodel(model, beams->z, &dm);
    if (st != TG_OK) return st;
    if (dm.n_aber) return TG_ERR_UNSUPPORTED;  // the aberrated lens has no field adjoint here
  }
  const AdjLayout L = adj_layout(n, pm->h, pm->w, method);
  if (!workspace || ws_bytes < L.total) return TG_ERR_WORKSPACE;
  if (((uintptr_t)workspace & 255) != 0) return TG_ERR_ALIGN;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  char* ws = reinterpret_cast<char*>(workspace);
  const int nsteps = input_plane ? 0 : dm.n;
  if (out->raw && cudaMemsetAsync(out->raw, 0, sizeof(double) * 4 * (size_t)nsteps, s) != cudaSuccess)
    return TG_ERR_CUDA;
  if (n == 0) return TG_OK;
  // 1. unit-amplitude records
  int st = field_prep_unit_amp(dm, beams, pm, ws + L.rec, field_records_bytes(n), stream, input_plane ? 1 : 0);
  if (st != TG_OK) return st;
  // 2. moments
  MomArgs MA;
  MA.beams = reinterpret_cast<const BeamFast*>(ws + L.rec);
  MA.g = reinterpret_cast<const float2*>(grad);
  MA.n = n;
  MA.h = pm->h;
  MA.w = pm->w;
  MA.col_chunks = L.col_chunks;
  MA.rows_per_split = L.rows_per_split;
  MA.part = reinterpret_cast<float*>(ws + L.part);
  double* mom = reinterpret_cast<double*>(ws + L.mom);
  if (method == TG_FIELD_SEPARABLE) {
    // the GEMM X = conj(G) (U dc^a)^T on the tensor cores, then the rows
    auto* gp = reinterpret_cast<__nv_bfloat16_raw*>(ws + L.gplanes);
    auto* up = reinterpret_cast<__nv_bfloat16_raw*>(ws + L.uplanes);
    float2* xp = reinterpret_cast<float2*>(ws + L.xprod);
    const int64_t gtot = (int64_t)L.rows_pad * L.cols_pad;
    k_adj_gplanes<<<(unsigned)((gtot + 255) / 256), 256, 0, s>>>(MA.g, pm->h, pm->w, L.rows_pad, L.cols_pad, gp);
    const int64_t uthreads = L.bpad * (L.cols_pad / kAdjCols);
    k_adj_uplanes<<<(unsigned)((uthreads + 127) / 128), 128, 0, s>>>(MA.beams, n, L.bpad, pm->w, L.cols_pad, up);
    if (3 * L.bpad > INT32_MAX) return TG_ERR_TOO_LARGE;
    int st2 = launch_field_gemm(gp, up, L.rows_pad, (int)(3 * L.bpad), L.cols_pad, 1, pm->h, (int)(3 * L.bpad),
                                xp, s);
    if (st2 != TG_OK) return st2;
    const int rgroups = (pm->h + kAdjRows - 1) / kAdjRows;
    k_adj_sep_moments<<<dim3((unsigned)((n + 127) / 128), (unsigned)rgroups), 128, 0, s>>>(
        MA.beams, n, xp, pm->h, L.bpad, MA.part);
    k_field_moment_sum<<<(int)((n * 12 + 255) / 256), 256, 0, s>>>(MA.part, rgroups, n, mom);
  } else {
    k_field_moments<<<dim3(L.col_chunks * L.row_splits, L.beam_chunks), kMThreads, 0, s>>>(MA);
    k_field_moment_sum<<<(int)((n * 12 + 255) / 256), 256, 0, s>>>(MA.part, L.col_chunks * L.row_splits, n, mom);
  }
  // 3. directions: the central ray's x, y, dx, dy, then the model's step parameters
  std::vector<Dir> dirs;
  const bool ray = out->x || out->y || out->dx || out->dy;
  if (ray) {
    for (int j = 0; j < 4; ++j) dirs.push_back(Dir{j, 0, 0, 1.0, -1});
  }
  if (out->raw) {
    for (int s2 = 0; s2 < dm.n; ++s2) {
      const DStep& stp = dm.s[s2];
      const int kind = model->components[s2 / 2].kind;
      switch (stp.kind) {
        case D_FREE: dirs.push_back(Dir{DIR_STEP, s2, 0, 1.0, 4 * s2}); break;
        case D_LENS: dirs.push_back(Dir{DIR_STEP, s2, 1, -1.0 / (stp.a[0] * stp.a[0]), 4 * s2}); break;
        case D_BIPRISM: dirs.push_back(Dir{DIR_STEP, s2, 0, 1.0, 4 * s2}); break;
        case D_ROTATE: dirs.push_back(Dir{DIR_STEP, s2, -1, 1.0, 4 * s2}); break;
        case D_SHIFT:
          if (kind == TG_DEFLECTOR) {  // def_x, def_y in slots 0, 1 (as tg_trace_vjp)
            dirs.push_back(Dir{DIR_STEP, s2, 2, 1.0, 4 * s2});
            dirs.push_back(Dir{DIR_STEP, s2, 3, 1.0, 4 * s2 + 1});
          } else {
            for (int j = 0; j < 4; ++j) dirs.push_back(Dir{DIR_STEP, s2, j, 1.0, 4 * s2 + j});
          }
          break;
        default: break;
      }
    }
  }
  double* mpart = reinterpret_cast<double*>(ws + L.model);
  // launches of up to kBGLaunchDirs directions, kBGDirs a thread (groups on blockIdx.y)
  const int launches = dirs.empty() ? 1 : (int)((dirs.size() + kBGLaunchDirs - 1) / kBGLaunchDirs);
  for (int li = 0; li < launches; ++li) {
    BGArgs B;
    std::memset(&B, 0, sizeof(B));
    B.n = n;
    B.x = beams->x; B.y = beams->y; B.dx = beams->dx; B.dy = beams->dy;
    B.pl = beams->pathlength;
    B.amp = beams->amplitude;
    B.waist = beams->waist_xy;
    B.radii = beams->radii;
    B.wl = beams->wavelength;
    B.wl_scalar = beams->wavelength_scalar;
    B.theta = beams->theta;
    B.pm.h = pm->h;
    B.pm.w = pm->w;
    for (int i = 0; i < 6; ++i) B.pm.t[i] = pm->t[i];
    B.rec = MA.beams;
    B.mom = mom;
    B.input_plane = input_plane ? 1 : 0;
    ModelSumArgs S;
    std::memset(&S, 0, sizeof(S));
    bool any_model = false;
    B.n_dir = 0;
    for (int d = 0; d < kBGLaunchDirs; ++d) {
      const size_t i = (size_t)li * kBGLaunchDirs + d;
      S.target[d] = -1;
      if (i >= dirs.size()) continue;
      B.n_dir = d + 1;
      B.dir_kind[d] = dirs[i].kind;
      B.dir_step[d] = dirs[i].step;
      B.dir_a[d] = dirs[i].a;
      B.dir_seed[d] = dirs[i].seed;
      S.target[d] = dirs[i].target;
      if (dirs[i].kind == DIR_STEP) any_model = true;
    }
    // every group writes the ray directions it carries; the pathlength and
    // amplitude gradients need no direction and come from the first group
    B.gx = out->x; B.gy = out->y; B.gdx = out->dx; B.gdy = out->dy;
    if (li == 0) {
      B.gpl = out->pathlength;
      B.gamp = out->amplitude;
    }
    B.model_part = mpart;
    // groups: the central ray's four directions together, the model's steps
    // kBGStepDirs at a time (a group never mixes the two kinds)
    int groups = 0;
    for (int d = 0; d < B.n_dir;) {
      const bool st = B.dir_kind[d] == DIR_STEP;
      const int cap = st ? kBGStepDirs : kBGRayDirs;
      int e = d;
      while (e < B.n_dir && e - d < cap && (B.dir_kind[e] == DIR_STEP) == st) ++e;
      B.group_first[groups] = d;
      B.group_n[groups] = e - d;
      ++groups;
      d = e;
    }
    if (groups == 0) {  // no directions: the pathlength and amplitude gradients only
      B.group_first[0] = 0;
      B.group_n[0] = 0;
      groups = 1;
    }
    k_field_beam_grad<kBGDirs><<<dim3(L.bg_blocks, groups), kBGThreads, 0, s>>>(dm, B);
    if (any_model && out->raw) {
      S.n_dir = B.n_dir;
      S.blocks = L.bg_blocks;
      k_field_model_sum<<<B.n_dir, 32, 0, s>>>(mpart, S, out->raw);
    }
  }
  return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
}

extern "C" int tg_field_vjp(const tg_model* model, const tg_beams* beams, const tg_pixel_map* pm,
                            const float* grad, const tg_field_grads* out, void* workspace, size_t ws_bytes,
                            void* stream) {
  if (!model) return TG_ERR_INVALID;
  return field_vjp_impl(model, beams, pm, grad, out, workspace, ws_bytes, stream);
}

extern "C" int tg_field_vjp_input(const tg_beams* beams, const tg_pixel_map* pm, const float* grad,
                                  const tg_field_grads* out, void* workspace, size_t ws_bytes, void* stream) {
  return field_vjp_impl(nullptr, beams, pm, grad, out, workspace, ws_bytes, stream);
}

extern "C" int tg_field_vjp_ex(int32_t method, const tg_model* model, const tg_beams* beams,
                               const tg_pixel_map* pm, const float* grad, const tg_field_grads* out,
                               void* workspace, size_t ws_bytes, void* stream) {
  if (!model) return TG_ERR_INVALID;
  return field_vjp_impl(model, beams, pm, grad, out, workspace, ws_bytes, stream, method);
}

extern "C" int tg_field_vjp_input_ex(int32_t method, const tg_beams* beams, const tg_pixel_map* pm,
                                     const float* grad, const tg_field_grads* out, void* workspace,
                                     size_t ws_bytes, void* stream) {
  return field_vjp_impl(nullptr, beams, pm, grad, out, workspace, ws_bytes, stream, method);
}
