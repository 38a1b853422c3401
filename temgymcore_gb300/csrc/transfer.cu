// transfer.cu - ray transfer through stacks of 5x5 matrices
// (transfer.py:6-112): every ray through the cumulative products of a matrix
// sequence, and a point source's fan through one matrix.
//
// Both are float64 on purpose (the reference's helpers are float64 NumPy /
// JAX): 25 float64 multiply-adds per (ray, plane) against 40 written bytes
// makes the transfer float64-pipe bound on GB300 (float64 is ~1/64 of the
// float32 rate), not HBM bound.
#include <cstring>

#include "tg_common.cuh"

namespace tg {

constexpr int kMaxTransfer = 120;  // matrices per call (24 KB of kernel parameters)

struct TransferMats {
  int32_t m;
  int32_t pad;
  double c[kMaxTransfer][25];  // cumulative products, row-major
};

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
  const int64_t total = n * (int64_t)m;
  int64_t blocks = (total + 255) / 256;
  const int64_t cap = (int64_t)sm_count_transfer() * 8;
  if (blocks > cap) blocks = cap;
  k_transfer_rays<<<(int)blocks, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(T, n, rays, out);
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
