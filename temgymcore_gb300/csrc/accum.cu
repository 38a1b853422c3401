// accum.cu - inplace_sum (utils.py:83-114): buffer[py, px] += frame[i] for
// every hit i with mask[i] set and (py, px) inside the buffer.
//
//   k_inplace_sum<IdxT, ValT>  grid-stride over hits, one atomic add per hit
//                              into the caller's buffer.  Integer buffers are
//                              exact (adds commute); float buffers round per
//                              add in whatever order the atomics land, so they
//                              match the serial reference to the rounding of
//                              the sum, not bit for bit.
#include <stdint.h>

#include "tg_common.cuh"

namespace tg {

template <typename T>
__device__ __forceinline__ void atomic_add_val(T* p, T v);
template <>
__device__ __forceinline__ void atomic_add_val<int32_t>(int32_t* p, int32_t v) { atomicAdd(p, v); }
template <>
__device__ __forceinline__ void atomic_add_val<int64_t>(int64_t* p, int64_t v) {
  // two's complement: an unsigned add wraps to the signed sum
  atomicAdd(reinterpret_cast<unsigned long long*>(p), (unsigned long long)v);
}
template <>
__device__ __forceinline__ void atomic_add_val<float>(float* p, float v) { atomicAdd(p, v); }
template <>
__device__ __forceinline__ void atomic_add_val<double>(double* p, double v) { atomicAdd(p, v); }

template <typename IdxT, typename ValT>
__global__ void __launch_bounds__(256)
k_inplace_sum(int64_t n, const IdxT* __restrict__ py, const IdxT* __restrict__ px,
              const uint8_t* __restrict__ mask, const ValT* __restrict__ frame, int32_t h, int32_t w,
              ValT* __restrict__ buffer) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (mask && !mask[i]) continue;
    const int64_t y = (int64_t)py[i], x = (int64_t)px[i];
    if (y < 0 || y >= h || x < 0 || x >= w) continue;
    atomic_add_val<ValT>(buffer + y * w + x, frame ? frame[i] : (ValT)1);
  }
}

static int accum_sms() {
  static int cached = 0;
  if (!cached) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&cached, cudaDevAttrMultiProcessorCount, dev);
    if (cached <= 0) cached = 148;
  }
  return cached;
}

template <typename IdxT, typename ValT>
static int launch_sum(int64_t n, const void* py, const void* px, const uint8_t* mask, const void* frame,
                      int32_t h, int32_t w, void* buffer, cudaStream_t s) {
  int64_t blocks = (n + 255) / 256;
  const int64_t cap = (int64_t)accum_sms() * 8;
  if (blocks > cap) blocks = cap;
  k_inplace_sum<IdxT, ValT><<<(int)blocks, 256, 0, s>>>(
      n, reinterpret_cast<const IdxT*>(py), reinterpret_cast<const IdxT*>(px), mask,
      reinterpret_cast<const ValT*>(frame), h, w, reinterpret_cast<ValT*>(buffer));
  return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
}

template <typename IdxT>
static int dispatch_val(int32_t dtype, int64_t n, const void* py, const void* px, const uint8_t* mask,
                        const void* frame, int32_t h, int32_t w, void* buffer, cudaStream_t s) {
  switch (dtype) {
    case 0: return launch_sum<IdxT, int32_t>(n, py, px, mask, frame, h, w, buffer, s);
    case 1: return launch_sum<IdxT, int64_t>(n, py, px, mask, frame, h, w, buffer, s);
    case 2: return launch_sum<IdxT, float>(n, py, px, mask, frame, h, w, buffer, s);
    case 3: return launch_sum<IdxT, double>(n, py, px, mask, frame, h, w, buffer, s);
    default: return TG_ERR_INVALID;
  }
}

}  // namespace tg

using namespace tg;

extern "C" int tg_inplace_sum(int64_t n, const void* pix_y, const void* pix_x, int32_t idx_i64,
                              const uint8_t* mask, const void* frame, int32_t dtype, int32_t h, int32_t w,
                              void* buffer, void* stream) {
  if (n < 0 || h <= 0 || w <= 0 || !buffer || dtype < 0 || dtype > 3) return TG_ERR_INVALID;
  if ((int64_t)h * w > 0x7fffffffLL) return TG_ERR_TOO_LARGE;
  if (n == 0) return TG_OK;
  if (!pix_y || !pix_x) return TG_ERR_INVALID;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  return idx_i64 ? dispatch_val<int64_t>(dtype, n, pix_y, pix_x, mask, frame, h, w, buffer, s)
                 : dispatch_val<int32_t>(dtype, n, pix_y, pix_x, mask, frame, h, w, buffer, s);
}
