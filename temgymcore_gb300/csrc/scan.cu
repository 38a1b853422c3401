// scan.cu - 4D-STEM batch: one ray bundle traced through the model at every
// scan position (probe), binned into one dense detector image per probe.
//
// This replaces the reference's per-scan-position Python loop of
// run_to_end (run.py:85-116) + Detector.into_image (grid.py:231-280).
//
// Kernel layout: a persistent grid walks the probes; one CTA owns one probe
// at a time.  The CTA
//   1. derives the probe's scan position (float64, from the ScanGrid pixel
//      map or an explicit list) and the per-probe Scanner/Descanner shifts,
//   2. traces the bundle (L2-resident, read by every CTA) in registers and
//      keeps each ray's packed pixel in shared memory,
//   3. reduces the hits' bounding box; when it fits the shared-memory window
//      (the normal case: a probe lights a small disc) it histograms there,
//   4. writes the dense image once: the window rows, and a quarter of the
//      image's rows of zeros around them, as 16-byte stores; the other rows
//      are all zeros and leave as TMA bulk copies from a zero buffer in
//      shared memory (asynchronous: the CTA goes on to the next probe while
//      the copy engine streams them).  Both write paths run at once.
// A probe whose hits do not fit the window, or a bundle larger than the
// shared ray buffer, takes the slow path: zero-fill, barrier, global atomics.
// The HBM traffic is therefore the dense histogram write, ~h*w*4 bytes/probe.
#include <cstring>

#include "tg_common.cuh"

TG_DEFINE_ERROR_WORD(scan)

namespace tg {

constexpr int kScanThreads = 256;
constexpr int kMaxSmemRays = 4096;  // packed pixels kept in shared memory
constexpr int kWinBins = 5632;      // shared histogram window (u32 counters)
constexpr int kScanBands = 1;       // row bands per probe image (work items per probe)
constexpr int kZeroBytes = 8192;    // zero source of the bulk row copies;
                                    // static shared memory stays under 48 KB

struct ScanArgs {
  int64_t n;  // rays per probe
  const float *x, *y, *dx, *dy;
  double z_scalar;
  int32_t n_probes, cols;
  double t[6];
  const double* positions;
  int32_t* hist;  // [n_probes][h][w]
  float* probe_xy;  // optional [n_probes][2][n]
  int32_t h, w;
  int32_t vec4;  // rows are 16-byte aligned: dense write with int4 stores
  int32_t bulk;  // images in device memory: zero rows as TMA bulk copies
  int32_t store_rows;  // zero rows next to the window written by stores, not bulk copies
};

__device__ __forceinline__ void probe_shifts(const Program& P, const ScanArgs& A, int p,
                                             float4* pshift) {
  double spx, spy;
  if (A.positions) {
    spx = A.positions[2 * (size_t)p];
    spy = A.positions[2 * (size_t)p + 1];
  } else {
    double r = (double)(p / A.cols), c = (double)(p % A.cols);
    spy = __dadd_rn(__dadd_rn(__dmul_rn(A.t[0], r), __dmul_rn(A.t[1], c)), A.t[2]);
    spx = __dadd_rn(__dadd_rn(__dmul_rn(A.t[3], r), __dmul_rn(A.t[4], c)), A.t[5]);
  }
  for (int k = 0; k < P.n_probe_ops; ++k) {
    const double* q = P.pcoef[k];
    pshift[k] = make_float4((float)(q[0] * spx + q[1] * spy + q[2]),
                            (float)(q[3] * spx + q[4] * spy + q[5]),
                            (float)(q[6] * spx + q[7] * spy + q[8]),
                            (float)(q[9] * spx + q[10] * spy + q[11]));
  }
}

__device__ __forceinline__ void trace_one(const Program& P, const float4* pshift, float x,
                                          float y, float dx, float dy, double z, RayS& r,
                                          bool& alive) {
  r = RayS{x, y, dx, dy, 0.f};
  uint64_t sb = 0;
  alive = true;
  (void)z;  // the bundle starts from one plane: no per-ray first distance
  for (int s = 0; s < P.n_steps; ++s)
    op_forward(P.op[s], pshift, r, 0.f, sb, alive, &P.aber[0][0]);
}

__device__ __forceinline__ int block_min(int v, int* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  int r = red[0];
  for (int i = 1; i < (int)(blockDim.x >> 5); ++i) r = min(r, red[i]);
  return r;
}

__device__ __forceinline__ int block_max(int v, int* red) {
  return -block_min(-v, red);
}

__global__ void __launch_bounds__(kScanThreads)
k_scan_hist(const __grid_constant__ Program P, const __grid_constant__ ScanArgs A,
            const __grid_constant__ BinCoef B) {
  __shared__ float4 pshift[kMaxProbeOps];
  __shared__ uint32_t pix[kMaxSmemRays];  // (py << 16) | px, or 0xffffffff = no hit
  __shared__ uint32_t win[kWinBins];
  __shared__ __align__(128) int4 zbuf[kZeroBytes / 16];
  __shared__ int red[kScanThreads / 32];
  const int64_t n = A.n;
  const bool fits = n <= kMaxSmemRays;
  const int H = A.h, W = A.w;
  for (int i = threadIdx.x; i < kZeroBytes / 16; i += blockDim.x) zbuf[i] = make_int4(0, 0, 0, 0);
  // the bulk copies read zbuf through the async proxy
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();
  const uint32_t zsrc = (uint32_t)__cvta_generic_to_shared(zbuf);
  // work item = (probe, band of kScanBands row bands); each band re-traces
  // the (L2-resident) bundle and keeps only its rows' hits.  Measured on the
  // 64x64-probe workload: one band 0.179 ms, two bands 0.186 ms (the doubled
  // per-item trace and barriers cost more than the finer balance gains)
  for (int it = blockIdx.x; it < kScanBands * A.n_probes; it += gridDim.x) {
    const int p = it / kScanBands, band = it - p * kScanBands;
    const int ra = (int)((int64_t)band * H / kScanBands), rb = (int)((int64_t)(band + 1) * H / kScanBands);
    if (threadIdx.x == 0) probe_shifts(P, A, p, pshift);
    __syncthreads();
    int rmin = 0x7fffffff, rmax = -1, cmin = 0x7fffffff, cmax = -1;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
      RayS r;
      bool alive;
      trace_one(P, pshift, A.x[i], A.y[i], A.dx[i], A.dy[i], A.z_scalar, r, alive);
      if (A.probe_xy && band == 0) {  // written once per probe
        A.probe_xy[(size_t)p * 2 * n + i] = r.x;
        A.probe_xy[(size_t)p * 2 * n + n + i] = r.y;
      }
      int py, px;
      bin_yx(r.x, r.y, B, py, px);
      bool ok = alive && py >= ra && py < rb && px >= 0 && px < W;
      if (!(isfinite(r.x) && isfinite(r.y))) atomicOr(&g_tg_err, TG_EW_NONFINITE);
      if (fits) pix[i] = ok ? ((uint32_t)py << 16) | (uint32_t)px : 0xffffffffu;
      if (ok) {
        rmin = min(rmin, py); rmax = max(rmax, py);
        cmin = min(cmin, px); cmax = max(cmax, px);
      }
    }
    rmin = block_min(rmin, red);
    rmax = block_max(rmax, red);
    cmin = block_min(cmin, red);
    cmax = block_max(cmax, red);
    int32_t* img = A.hist + (size_t)p * H * W;
    const int wr = rmax - rmin + 1, wc = cmax - cmin + 1;
    const bool any = rmax >= 0;
    const bool windowed = fits && (!any || (int64_t)wr * wc <= kWinBins);
    if (windowed) {
      if (any) {
        for (int i = threadIdx.x; i < wr * wc; i += blockDim.x) win[i] = 0u;
        __syncthreads();
        for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
          uint32_t v = pix[i];
          if (v != 0xffffffffu) {
            int py = (int)(v >> 16), px = (int)(v & 0xffffu);
            atomicAdd(&win[(py - rmin) * wc + (px - cmin)], 1u);
          }
        }
        __syncthreads();
      }
      if (A.vec4) {
        // the window rows and store_rows zero rows around them are written
        // by 16-byte stores, [r0, r1); band rows outside are zeros: bulk
        // copies of the zero buffer (row starts are 16-byte aligned: W is a multiple of 4 and
        // the images 16-byte aligned); one thread issues them, the group is
        // committed and left in flight.  Images in host memory (written
        // across the host link) take 16-byte stores for every row instead.
        int r0 = A.bulk ? (any ? rmin : ra) : ra, r1 = A.bulk ? (any ? rmax + 1 : ra) : rb;
        if (A.bulk && A.store_rows > 0) {  // store_rows more zero rows by stores, around the window
          int below = min(A.store_rows >> 1, r0 - ra);
          const int above = min(A.store_rows - below, rb - r1);
          below = min(A.store_rows - above, r0 - ra);
          r0 -= below;
          r1 += above;
        }
        if (A.bulk && threadIdx.x == 0) {
          char* base = reinterpret_cast<char*>(img);
          const int64_t row_bytes = (int64_t)W * 4;
          const int64_t spans[2][2] = {{ra * row_bytes, r0 * row_bytes}, {r1 * row_bytes, rb * row_bytes}};
          for (int sp = 0; sp < 2; ++sp)
            for (int64_t off = spans[sp][0]; off < spans[sp][1]; off += kZeroBytes) {
              const int64_t left = spans[sp][1] - off;
              const uint32_t bytes = (uint32_t)(left < kZeroBytes ? left : kZeroBytes);
              asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;"
                           :: "l"(base + off), "r"(zsrc), "r"(bytes) : "memory");
            }
          asm volatile("cp.async.bulk.commit_group;" ::: "memory");
          // keep at most four items' copies in flight (a hardware wait on
          // the copy engine, no polling)
          asm volatile("cp.async.bulk.wait_group.read 4;" ::: "memory");
        }
        // window rows: counts inside [cmin, cmax], zeros elsewhere
        const int w4 = W >> 2;
        const int total = (r1 - r0) * w4;
        int4* rows = reinterpret_cast<int4*>(img) + (int64_t)r0 * w4;
        for (int i = threadIdx.x; i < total; i += blockDim.x) {
          const int row = r0 + i / w4, c0 = (i % w4) << 2;
          int4 v = make_int4(0, 0, 0, 0);
          if (any && row >= rmin && row <= rmax && c0 + 3 >= cmin && c0 <= cmax) {
            const uint32_t* wrow = win + (row - rmin) * wc;
            int c = c0;
            v.x = (c >= cmin && c <= cmax) ? (int)wrow[c - cmin] : 0; ++c;
            v.y = (c >= cmin && c <= cmax) ? (int)wrow[c - cmin] : 0; ++c;
            v.z = (c >= cmin && c <= cmax) ? (int)wrow[c - cmin] : 0; ++c;
            v.w = (c >= cmin && c <= cmax) ? (int)wrow[c - cmin] : 0;
          }
          __stcs(rows + i, v);
        }
      } else {
        for (int i = ra * W + threadIdx.x; i < rb * W; i += blockDim.x) {
          const int row = i / W, c = i - row * W;
          int v = 0;
          if (any && row >= rmin && row <= rmax && c >= cmin && c <= cmax)
            v = (int)win[(row - rmin) * wc + (c - cmin)];
          __stcs(img + i, v);
        }
      }
    } else {
      // slow path: zero the band's rows, then global atomics (re-trace if needed)
      for (int i = ra * W + threadIdx.x; i < rb * W; i += blockDim.x) img[i] = 0;
      __syncthreads();
      for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        int py, px;
        bool ok;
        if (fits) {
          uint32_t v = pix[i];
          ok = v != 0xffffffffu;
          py = (int)(v >> 16);
          px = (int)(v & 0xffffu);
        } else {
          RayS r;
          bool alive;
          trace_one(P, pshift, A.x[i], A.y[i], A.dx[i], A.dy[i], A.z_scalar, r, alive);
          bin_yx(r.x, r.y, B, py, px);
          ok = alive && py >= ra && py < rb && px >= 0 && px < W;
        }
        if (ok) atomicAdd(img + py * W + px, 1);
      }
    }
    __syncthreads();  // shared buffers are reused by the next item
  }
  // every bulk copy has read zbuf and written its rows before the CTA exits
  if (A.bulk && threadIdx.x == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

static int sm_count_scan() {
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

extern "C" int tg_scan_hist(const tg_model* model, const tg_rays* bundle, const tg_scan* scan,
                            const tg_grid* grid, int32_t* hist, float* probe_xy, void* stream) {
  if (!model || !bundle || !scan || !grid) return TG_ERR_INVALID;
  if (!hist && scan->n_probes > 0) return TG_ERR_INVALID;
  if (bundle->n < 0 || scan->n_probes < 0 || grid->h <= 0 || grid->w <= 0) return TG_ERR_INVALID;
  if (grid->h > 65535 || grid->w > 65535) return TG_ERR_TOO_LARGE;
  if (!scan->positions && scan->cols <= 0) return TG_ERR_INVALID;
  if (bundle->z) return TG_ERR_UNSUPPORTED;  // one source plane for the bundle
  if (bundle->n > 0 && (!bundle->x || !bundle->y || !bundle->dx || !bundle->dy))
    return TG_ERR_INVALID;
  Program P;
  int st = compile_program(model, false, bundle->z_scalar, &P);
  if (st != TG_OK) return st;
  if (scan->n_probes == 0) return TG_OK;
  ScanArgs A;
  std::memset(&A, 0, sizeof(A));
  A.n = bundle->n;
  A.x = bundle->x; A.y = bundle->y; A.dx = bundle->dx; A.dy = bundle->dy;
  A.z_scalar = bundle->z_scalar;
  A.n_probes = scan->n_probes;
  A.cols = scan->cols;
  for (int i = 0; i < 6; ++i) A.t[i] = scan->t[i];
  A.positions = scan->positions;
  A.hist = hist;
  A.probe_xy = probe_xy;
  A.h = grid->h;
  A.w = grid->w;
  A.vec4 = ((grid->w & 3) == 0) && ((reinterpret_cast<uintptr_t>(hist) & 15) == 0);
  // a quarter of the rows go out as stores beside the bulk copies: the two
  // write paths run in parallel (256x256 images, 64x64 probes: 0.1815 ms with
  // bulk copies alone, 0.1777 ms with 64 stored rows; 32 and 80 rows between)
  A.store_rows = grid->h / 4;
  {  // images may live in pinned host memory (written by the kernel across the host link)
    cudaPointerAttributes pa;
    if (cudaPointerGetAttributes(&pa, hist) != cudaSuccess) return TG_ERR_CUDA;
    A.bulk = A.vec4 && pa.type == cudaMemoryTypeDevice;
    if (pa.type != cudaMemoryTypeDevice && pa.type != cudaMemoryTypeHost && pa.type != cudaMemoryTypeManaged)
      return TG_ERR_INVALID;  // unregistered host memory
  }
  BinCoef B = make_bincoef(grid);
  static int per_sm = 0;  // residency, queried once
  if (!per_sm) {
    int q = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&q, k_scan_hist, kScanThreads, 0);
    per_sm = q > 0 ? q : 1;
  }
  int blocks = sm_count_scan() * per_sm;
  if (blocks > kScanBands * scan->n_probes) blocks = kScanBands * scan->n_probes;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  k_scan_hist<<<blocks, kScanThreads, 0, s>>>(P, A, B);
  return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
}
