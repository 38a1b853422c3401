// transfer.cu - ray transfer through stacks of 5x5 matrices
// (transfer.py:6-112): every ray through the cumulative products of a matrix
// sequence, and a point source's fan through one matrix.
//
// The reference's helpers are float64 NumPy / JAX.  25 float64 multiply-adds
// per (ray, plane) against 40 written bytes would make the transfer float64-
// pipe bound on GB300 (float64 issues at ~1/64 of the float32 rate), so the
// stack transfer runs in double-float arithmetic: every matrix entry and ray
// component as an unevaluated float32 pair (hi + lo, 48 significant bits),
// products with their exact rounding error (FMA), sums with TwoSum, and the
// result rounded back to float64 with integer operations.  Errors stay at a
// few 2^-47 of the sum of the term magnitudes; a ray or matrix with a nonzero
// entry outside [2^-39, 2^62] (where a product's error term would leave the
// normal float32 range) takes the float64 path.
#include <cstring>

#include "tg_common.cuh"

namespace tg {

constexpr int kMaxTransfer = 120;  // matrices per call (24 KB of kernel parameters)

struct TransferMats {
  int32_t m;
  int32_t pad;
  double c[kMaxTransfer][25];  // cumulative products, row-major
};

// ---------------------------------------------------------------- double-float
struct DF {
  float h, l;
};

// a float64 value inside the double-float range (zero, or |v| in [2^-39, 2^62])
__host__ __device__ inline bool df_range(double v) {
  const double a = v < 0 ? -v : v;
  return v == 0.0 || (a >= 1.8189894035458565e-12 && a <= 4.611686018427388e18);
}

__device__ __forceinline__ DF df_split(double v) {
  const float h = __double2float_rn(v);
  return DF{h, __double2float_rn(v - (double)h)};  // v - h is exact in float64
}

// a * b: the product of the heads with its exact rounding error, plus the
// cross terms (lo * lo is below the precision kept)
__device__ __forceinline__ DF df_mul(DF a, DF b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return DF{p, e};
}

// a + b: TwoSum of the heads, the tails added to the error; the pair is
// left unrenormalised (a short sum of products stays within a few 2^-47 of
// the term magnitudes) and df_norm is applied once per result
__device__ __forceinline__ DF df_add(DF a, DF b) {
  const float s = __fadd_rn(a.h, b.h);
  const float bb = __fsub_rn(s, a.h);
  const float err = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(b.h, bb));
  return DF{s, __fadd_rn(err, __fadd_rn(a.l, b.l))};
}

// Fast2Sum renormalisation: |lo| <= ulp(hi) / 2 afterwards
__device__ __forceinline__ DF df_norm(DF a) {
  const float h = __fadd_rn(a.h, a.l);
  return DF{h, __fsub_rn(a.l, __fsub_rn(h, a.h))};
}

// hi + lo as a float64, faithfully rounded (within one float64 ulp: far below
// the pair's own 2^-47), with a few integer operations.  For a renormalised
// pair |lo| <= ulp32(hi) / 2, so in units of hi's float64 ulp lo is its
// 24-bit significand shifted by sh = e_lo - e_hi + 29 <= 4, and the sum can
// leave hi's binade only downwards and only when hi is a power of two: then
// the grid below is twice as fine and lo counts double.  Zero, denormal and
// non-finite parts take the general rounding.
__device__ __forceinline__ double df_to_double(DF a) {
  const uint32_t hb = __float_as_uint(a.h), lb = __float_as_uint(a.l);
  const int eh = (int)((hb >> 23) & 0xffu), el = (int)((lb >> 23) & 0xffu);
  if ((lb << 1) == 0u) return f32_to_f64(a.h);
  if (eh == 0 || eh == 0xff || el == 0 || el == 0xff) return add_f64_f32(f32_to_f64(a.h), a.l);
  const long long d = __double_as_longlong(f32_to_f64(a.h));
  const uint32_t ml = (lb & 0x7fffffu) | 0x800000u;
  const bool shrink = (hb >> 31) != (lb >> 31);  // lo reduces hi's magnitude
  int sh = el - eh + 29;
  if (shrink && (d & 0xfffffffffffffLL) == 0) ++sh;  // below a power of two: half-ulp grid
  const long long n = sh >= 0 ? (long long)ml << sh : (sh > -25 ? (long long)(ml >> -sh) : 0LL);
  return __longlong_as_double(d + (shrink ? -n : n));
}

constexpr int kTrRays = 64;  // rays staged per block iteration

// out[n][p][i] = sum_j C[p][i][j] ray[n][j] in double-float.  A block splits
// the matrices into float32 pairs once, then per group of kTrRays rays stages
// their split components in shared memory (the split is shared by all
// planes) and runs one (ray, plane) pair per thread: a warp writes 32
// consecutive 40-byte records.
__global__ void __launch_bounds__(256)
k_transfer_rays_df(const __grid_constant__ TransferMats T, int64_t n, const double* __restrict__ rays,
                   double* __restrict__ out) {
  extern __shared__ DF tsm[];  // [m * 25] matrix pairs, then [kTrRays * 5] ray pairs
  __shared__ int s_ok[kTrRays];
  const int m = T.m;
  DF* mc = tsm;
  DF* rv = tsm + m * 25;
  for (int i = threadIdx.x; i < m * 25; i += blockDim.x) mc[i] = df_split((&T.c[0][0])[i]);
  for (int64_t g = (int64_t)blockIdx.x * kTrRays; g < n; g += (int64_t)gridDim.x * kTrRays) {
    const int nr = (int)((n - g) < kTrRays ? (n - g) : kTrRays);
    __syncthreads();  // the previous group's pairs are done with rv / s_ok
    for (int i = threadIdx.x; i < nr * 5; i += blockDim.x) rv[i] = df_split(rays[g * 5 + i]);
    for (int i = threadIdx.x; i < nr; i += blockDim.x) {
      const double* v = rays + (g + i) * 5;
      s_ok[i] = df_range(v[0]) && df_range(v[1]) && df_range(v[2]) && df_range(v[3]) && df_range(v[4]);
    }
    __syncthreads();
    const int pairs = nr * m;
    for (int q = threadIdx.x; q < pairs; q += blockDim.x) {
      const int r = q / m, p = q - r * m;
      double* o = out + ((g + r) * m + p) * 5;
      if (s_ok[r]) {
        const DF* c = mc + p * 25;
        const DF* v = rv + r * 5;
#pragma unroll
        for (int i = 0; i < 5; ++i) {
          DF acc = df_mul(c[5 * i], v[0]);
#pragma unroll
          for (int j = 1; j < 5; ++j) acc = df_add(acc, df_mul(c[5 * i + j], v[j]));
          o[i] = df_to_double(df_norm(acc));
        }
      } else {  // outside the double-float range: float64
        const double* v = rays + (g + r) * 5;
        const double* c = T.c[p];
#pragma unroll
        for (int i = 0; i < 5; ++i)
          o[i] = c[5 * i + 0] * v[0] + c[5 * i + 1] * v[1] + c[5 * i + 2] * v[2] +
                 c[5 * i + 3] * v[3] + c[5 * i + 4] * v[4];
      }
    }
  }
}

// out[n][p][i] = sum_j C[p][i][j] ray[n][j], one (ray, plane) pair per thread:
// a warp writes 32 consecutive 40-byte records.
__global__ void __launch_bounds__(256)
k_transfer_rays(const __grid_constant__ TransferMats T, int64_t n, const double* __restrict__ rays,
                double* __restrict__ out) {
  __shared__ double sc[kMaxTransfer * 25];
  for (int i = threadIdx.x; i < T.m * 25; i += blockDim.x) sc[i] = T.c[i / 25][i % 25];
  __syncthreads();
  const int64_t total = n * (int64_t)T.m;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t / T.m;
    const int p = (int)(t - r * T.m);
    const double* v = rays + r * 5;
    const double v0 = v[0], v1 = v[1], v2 = v[2], v3 = v[3], v4 = v[4];
    const double* c = sc + p * 25;
    double* o = out + t * 5;
#pragma unroll
    for (int i = 0; i < 5; ++i)
      o[i] = c[5 * i + 0] * v0 + c[5 * i + 1] * v1 + c[5 * i + 2] * v2 + c[5 * i + 3] * v3 +
             c[5 * i + 4] * v4;
  }
}

struct PtSrcArgs {
  double x0, y0;
  double t[25];
  int64_t n;
  const double *sx, *sy;
  double* out;  // [4][n]
};

// rows x, y, dx, dy of T [x0, y0, sx, sy, 1] for every slope pair
__global__ void __launch_bounds__(256) k_transfer_pt_src(const __grid_constant__ PtSrcArgs A) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < A.n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const double v[5] = {A.x0, A.y0, A.sx[k], A.sy[k], 1.0};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      double s = 0.0;
#pragma unroll
      for (int j = 0; j < 5; ++j) s += A.t[5 * i + j] * v[j];
      A.out[(int64_t)i * A.n + k] = s;
    }
  }
}

static int sm_count_transfer() {
  static int cached = 0;
  if (!cached) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&cached, cudaDevAttrMultiProcessorCount, dev);
    if (cached <= 0) cached = 148;
  }
  return cached;
}

static void mat5(const double* a, const double* b, double* out) {
  double t[25];
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 5; ++j) {
      double s = 0.0;
      for (int k = 0; k < 5; ++k) s += a[5 * i + k] * b[5 * k + j];
      t[5 * i + j] = s;
    }
  std::memcpy(out, t, sizeof(t));
}

}  // namespace tg

using namespace tg;

extern "C" int tg_transfer_cumulative(int32_t m, const double* matrices, double* cumulative) {
  if (m <= 0 || !matrices || !cumulative) return TG_ERR_INVALID;
  // transfer.py:150-183: start from the LAST matrix and multiply the earlier
  // ones on the left: cumulative[k] = M[m-1-k] @ ... @ M[m-1]
  double total[25];
  std::memcpy(total, matrices + (int64_t)(m - 1) * 25, sizeof(total));
  std::memcpy(cumulative, total, sizeof(total));
  for (int k = 1; k < m; ++k) {
    mat5(matrices + (int64_t)(m - 1 - k) * 25, total, total);
    std::memcpy(cumulative + (int64_t)k * 25, total, sizeof(total));
  }
  return TG_OK;
}

extern "C" int tg_transfer_rays(int64_t n, const double* rays, int32_t m, const double* matrices,
                                double* out, void* stream) {
  if (n < 0 || m <= 0 || !matrices) return TG_ERR_INVALID;
  if (m > kMaxTransfer) return TG_ERR_TOO_LARGE;
  if (n > 0 && (!rays || !out)) return TG_ERR_INVALID;
  TransferMats T;
  std::memset(&T, 0, sizeof(T));
  T.m = m;
  int st = tg_transfer_cumulative(m, matrices, &T.c[0][0]);
  if (st != TG_OK) return st;
  if (n == 0) return TG_OK;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  bool df = true;
  for (int i = 0; i < m * 25 && df; ++i) df = df_range((&T.c[0][0])[i]);
  if (df) {
    const size_t smem = (size_t)(m * 25 + kTrRays * 5) * sizeof(DF);  // <= 26.6 KB
    int64_t blocks = (n + kTrRays - 1) / kTrRays;
    const int64_t cap = (int64_t)sm_count_transfer() * 8;
    if (blocks > cap) blocks = cap;
    k_transfer_rays_df<<<(int)blocks, 256, smem, s>>>(T, n, rays, out);
    return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
  }
  const int64_t total = n * (int64_t)m;
  int64_t blocks = (total + 255) / 256;
  const int64_t cap = (int64_t)sm_count_transfer() * 8;
  if (blocks > cap) blocks = cap;
  k_transfer_rays<<<(int)blocks, 256, 0, s>>>(T, n, rays, out);
  return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
}

extern "C" int tg_transfer_rays_pt_src(double x0, double y0, int64_t n, const double* slopes_x,
                                       const double* slopes_y, const double* matrix, double* out,
                                       void* stream) {
  if (n < 0 || !matrix) return TG_ERR_INVALID;
  if (n > 0 && (!slopes_x || !slopes_y || !out)) return TG_ERR_INVALID;
  if (n == 0) return TG_OK;
  PtSrcArgs A;
  A.x0 = x0;
  A.y0 = y0;
  std::memcpy(A.t, matrix, sizeof(A.t));
  A.n = n;
  A.sx = slopes_x;
  A.sy = slopes_y;
  A.out = out;
  int64_t blocks = (n + 255) / 256;
  const int64_t cap = (int64_t)sm_count_transfer() * 8;
  if (blocks > cap) blocks = cap;
  k_transfer_pt_src<<<(int)blocks, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(A);
  return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
}
