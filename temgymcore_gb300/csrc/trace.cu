// trace.cu - fused forward ray chain (+ binning + histogram), standalone
// binning, and the recompute-based adjoint.
//
// One kernel pass reads each ray once (x, y, dx, dy as float4 vectors of four
// consecutive rays per thread), runs the whole component chain in registers,
// and writes the outputs once.  No float64 arithmetic runs per ray in the
// usual case: the pathlength's float64 base + float32 part is rounded with
// float32 / integer operations (add_f64_f32), and only the rare coordinates
// near a pixel-rounding tie take an exact float64 binning evaluation (see
// tg_common.cuh).
#include <cstring>

#include "tg_common.cuh"

TG_DEFINE_ERROR_WORD(trace)

namespace tg {

struct FwdArgs {
  int64_t n;
  const float *x, *y, *dx, *dy;
  const double* z;
  double z_scalar;
  const double* pl;
  double pl_scalar;
  const float* amp;
  float *ox, *oy, *odx, *ody;
  double* opl;
  double* oz;
  float* oamp;
  int32_t *pix_y, *pix_x;
  void* hist;
  int32_t h, w;
  int32_t do_bin;
  int32_t opl_vec;  // opl is 16-byte aligned: paired double stores
  int32_t pix_vec;  // pix_y / pix_x (those given) are 16-byte aligned
  uint32_t* rows;   // shared-histogram variant: per-CTA packed uint16 counters [gridDim.x][(h * w + 1) / 2]
};

// Shared-histogram variant of the forward kernel: each CTA (kShThreads
// threads, one per SM) keeps the whole detector in shared memory as uint16
// counters packed in pairs and adds each hit with one shared atomic.  A hit
// that brings its counter to 16384 moves those 16384 counts into the caller's
// histogram (one global atomic, rare: only pixels with more than 16383 hits
// on one SM) and takes them off the counter, so no counter reaches 65536
// (that would take 49152 more hits on the pixel before the subtraction lands;
// a CTA has at most a few thousand in flight) and no periodic flush is
// needed: at the end the CTA writes its packed
// counters once to its own row of the workspace, and k_hist_rows adds the
// rows into the histogram.  Global atomics (even warp-aggregated) then no
// longer bound the fused pass: measured at 16.8 M rays, 256x256 spread 0.193
// -> 0.167 ms, 64x64 (~4k hits per pixel) 0.482 -> 0.143 ms.  Each hit is one
// plain shared atomic: warp aggregation by __match_any_sync measured slower
// here (0.168 / 0.154 ms).
constexpr int kShThreads = 1024;
constexpr int kShMaxBins = 2 * (200 * 1024 / 4);  // 200 KB of packed counters

__host__ __device__ inline int sh_words(int bins) { return (bins + 1) >> 1; }

template <typename CountT>
__device__ __forceinline__ void hist_add_sh(uint32_t* shw, int bin, bool valid, CountT* hist) {
  if (valid) {
    const uint32_t sh = 16u * (uint32_t)(bin & 1);
    const uint32_t old = atomicAdd(shw + (bin >> 1), 1u << sh);
    if (((old >> sh) & 0xffffu) == 0x3fffu) {  // this hit made the count 16384
      atomicSub(shw + (bin >> 1), 0x4000u << sh);
      if constexpr (sizeof(CountT) == 8)
        atomicAdd(reinterpret_cast<unsigned long long*>(hist) + bin, 16384ull);
      else
        atomicAdd(reinterpret_cast<unsigned int*>(hist) + bin, 16384u);
    }
  }
}

// Writes the CTA's packed counters to its workspace row; all threads of the
// CTA call it once, at the end.
__device__ __forceinline__ void sh_store_row(const uint32_t* shw, uint32_t* row, int words) {
  __syncthreads();
  for (int i = threadIdx.x; i < words; i += blockDim.x) row[i] = shw[i];
}

// R consecutive floats from p + i0: 16-byte vector loads when vec (R = 4 or
// 8, p + i0 16-byte aligned and all R in range), else per element with the
// tail past n read as 0.  For R = 8 both vector loads are issued before the
// values are unpacked (this form also spills fewer registers in the
// 128-register adjoint).  kStream: evict-first loads (ld.global.cs), for data
// read once by a kernel that streams many arrays.
template <bool kStream>
__device__ __forceinline__ float4 ld4(const float* p) {
  return kStream ? __ldcs(reinterpret_cast<const float4*>(p)) : __ldg(reinterpret_cast<const float4*>(p));
}

template <int R, bool kStream = false>
__device__ __forceinline__ void load4(const float* __restrict__ p, int64_t i0,
                                      int64_t n, float v[R], bool vec) {
  if constexpr (R == 4) {
    if (vec) {
      const float4 t = ld4<kStream>(p + i0);
      v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
      return;
    }
  } else if constexpr (R == 8) {
    if (vec) {
      const float4 t = ld4<kStream>(p + i0);
      const float4 u = ld4<kStream>(p + i0 + 4);
      v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
      v[4] = u.x; v[5] = u.y; v[6] = u.z; v[7] = u.w;
      return;
    }
  }
#pragma unroll
  for (int k = 0; k < R; ++k) v[k] = (i0 + k < n) ? __ldg(p + i0 + k) : 0.f;
}

// kStream: evict-first vector stores (st.global.cs).
template <int R, bool kStream = false>
__device__ __forceinline__ void store4(float* __restrict__ p, int64_t i0,
                                       int64_t n, const float v[R], bool vec) {
  if (R == 2 && vec) {
    *reinterpret_cast<float2*>(p + i0) = make_float2(v[0], v[R - 1]);
  } else if (R % 4 == 0 && vec) {
#pragma unroll
    for (int q = 0; q + 3 < R; q += 4) {
      const float4 t = make_float4(v[q], v[q + 1], v[q + 2], v[q + 3]);
      if (kStream) __stcs(reinterpret_cast<float4*>(p + i0 + q), t);
      else *reinterpret_cast<float4*>(p + i0 + q) = t;
    }
  } else {
#pragma unroll
    for (int k = 0; k < R; ++k)
      if (i0 + k < n) p[i0 + k] = v[k];
  }
}

struct NoOp {
  __device__ __forceinline__ void operator()() const {}
};

// The chain, the outputs, the pixels and the histogram for rays i0 .. i0+R-1
// whose inputs are in x, y, dx, dy (vec: all R in range and every output
// array aligned for R-wide vector stores).  All 32 lanes of the warp call it
// (the global histogram's warp aggregation).  after_chain runs once the
// coordinates are stored (every input consumed), before the pathlength, the
// binning and the histogram.
template <int R, typename CountT, bool kSh, typename AfterChain = NoOp>
__device__ __forceinline__ void fwd_rays(const Program& P, const FwdArgs& A, const BinCoef& B,
                                         uint32_t* shw, int64_t i0, float (&x)[R],
                                         float (&y)[R], float (&dx)[R], float (&dy)[R],
                                         bool vec, AfterChain after_chain = AfterChain()) {
  const int64_t n = A.n;
  const double pl_uniform = A.pl_scalar + P.pl_const;
  {
    RayS r[R];
    double dvar[R];  // per-ray first distance (per-ray input z only), float64 once per ray
    float dvf[R];
    uint64_t sb[R];
    bool alive[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
      r[k] = RayS{x[k], y[k], dx[k], dy[k], 0.f};
      dvar[k] = 0.0;
      dvf[k] = 0.f;
      sb[k] = 0;
      alive[k] = true;
    }
    if (A.z) {
#pragma unroll
      for (int k = 0; k < R; ++k) {
        dvar[k] = P.zc_first - (i0 + k < n ? A.z[i0 + k] : A.z_scalar);
        dvf[k] = (float)dvar[k];
      }
    }
    for (int s = 0; s < P.n_steps; ++s) {
      const Op op = P.op[s];
#pragma unroll
      for (int k = 0; k < R; ++k)
        op_forward(op, nullptr, r[k], dvf[k], sb[k], alive[k], &P.aber[0][0]);
    }
#pragma unroll
    for (int k = 0; k < R; ++k) {
      x[k] = r[k].x; y[k] = r[k].y; dx[k] = r[k].dx; dy[k] = r[k].dy;
    }
    store4<R>(A.ox, i0, n, x, vec);
    store4<R>(A.oy, i0, n, y, vec);
    store4<R>(A.odx, i0, n, dx, vec);
    store4<R>(A.ody, i0, n, dy, vec);
    // every input value has reached an issued instruction (the output of each
    // coordinate depends on its input), so their registers hold the data
    after_chain();
    if (A.opl) {
      // no float64 arithmetic per ray for a uniform base (one add per
      // per-ray input): GB300 issues float64 at ~1/64 of the float32 rate,
      // so base + plv is rounded with float32 / integer operations
      double o[R];
#pragma unroll
      for (int k = 0; k < R; ++k) {
        double base = pl_uniform;
        if (A.pl && i0 + k < n) base = A.pl[i0 + k] + P.pl_const;
        if (A.z) base += dvar[k];
        o[k] = add_f64_f32(base, r[k].plv);
      }
      if (R == 4 && vec && A.opl_vec) {  // two 16-byte stores (i0 is a multiple of 4)
        reinterpret_cast<double2*>(A.opl + i0)[0] = make_double2(o[0], o[1]);
        reinterpret_cast<double2*>(A.opl + i0)[1] = make_double2(o[2 % R], o[3 % R]);
      } else if (R == 2 && vec && A.opl_vec) {  // one 16-byte store (i0 even)
        *reinterpret_cast<double2*>(A.opl + i0) = make_double2(o[0], o[R - 1]);
      } else {
#pragma unroll
        for (int k = 0; k < R; ++k)
          if (i0 + k < n) A.opl[i0 + k] = o[k];
      }
    }
    if (A.oz) {
#pragma unroll
      for (int k = 0; k < R; ++k)
        if (i0 + k < n) A.oz[i0 + k] = P.z_out;
    }
    if (A.oamp) {
#pragma unroll
      for (int k = 0; k < R; ++k)
        if (i0 + k < n) {
          float a0 = A.amp ? A.amp[i0 + k] : 1.f;
          A.oamp[i0 + k] = alive[k] ? a0 : 0.f;
        }
    }
    if (A.do_bin) {
      int pys[R], pxs[R];
#pragma unroll
      for (int k = 0; k < R; ++k) {
        int py, px;
        bin_yx(x[k], y[k], B, py, px);
        pys[k] = py;
        pxs[k] = px;
        const bool inr = (i0 + k < n);
        if (inr && !(isfinite(x[k]) && isfinite(y[k]))) atomicOr(&g_tg_err, TG_EW_NONFINITE);
        if (A.hist) {
          bool ok = inr && alive[k] && py >= 0 && py < A.h && px >= 0 && px < A.w;
          if (kSh) hist_add_sh<CountT>(shw, ok ? py * A.w + px : 0, ok, reinterpret_cast<CountT*>(A.hist));
          else hist_add_warp<CountT>(reinterpret_cast<CountT*>(A.hist), ok ? py * A.w + px : 0, ok);
        }
      }
      // pixel indices: one vector store per array where aligned
      if ((R == 2 || R == 4) && vec && A.pix_vec) {
        if (R == 2) {
          if (A.pix_y) *reinterpret_cast<int2*>(A.pix_y + i0) = make_int2(pys[0], pys[R - 1]);
          if (A.pix_x) *reinterpret_cast<int2*>(A.pix_x + i0) = make_int2(pxs[0], pxs[R - 1]);
        } else {
          if (A.pix_y) *reinterpret_cast<int4*>(A.pix_y + i0) = make_int4(pys[0], pys[1 % R], pys[2 % R], pys[3 % R]);
          if (A.pix_x) *reinterpret_cast<int4*>(A.pix_x + i0) = make_int4(pxs[0], pxs[1 % R], pxs[2 % R], pxs[3 % R]);
        }
      } else {
#pragma unroll
        for (int k = 0; k < R; ++k)
          if (i0 + k < n) {
            if (A.pix_y) A.pix_y[i0 + k] = pys[k];
            if (A.pix_x) A.pix_x[i0 + k] = pxs[k];
          }
      }
    }
  }
}

// kPf (shared-histogram variant, R = 4): each thread prefetches its next
// four rays (x, y, dx, dy: four 16-byte cp.async) into its own 64-byte slot of
// shared memory as soon as the current ones' coordinates are stored (every
// value read from the slot has then been used), so the loads run under the
// pathlength, the binning and the histogram atomics.  The slots take
// kPfBytes ahead of the histogram words.
constexpr int kPfBytes = 4 * kShThreads * 16;  // 64 KB

template <int R, typename CountT, bool kSh = false, bool kPf = false>
__global__ void __launch_bounds__(kSh ? kShThreads : 256)
k_trace_fwd(const __grid_constant__ Program P, const __grid_constant__ FwdArgs A,
            const __grid_constant__ BinCoef B) {
  static_assert(!kPf || (kSh && R == 4), "prefetch: shared-histogram variant, four rays per thread");
  extern __shared__ __align__(16) uint32_t shm[];
  // kSh: [(h * w + 1) / 2] packed uint16 counters (after the prefetch slots with kPf)
  uint32_t* shw = kPf ? shm + kPfBytes / 4 : shm;
  const int64_t n = A.n;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x * R;
  const int bins = A.h * A.w;
  if (kSh) {
    for (int i = threadIdx.x; i < ((bins + 1) >> 1); i += blockDim.x) shw[i] = 0u;
    __syncthreads();
  }
  // prefetch slot of array a (x, y, dx, dy) for this thread
  const uint32_t slot = smem_u32(shm) + 16u * threadIdx.x;
  auto prefetch = [&](int64_t j0) {
    cp_async16(slot, A.x + j0);
    cp_async16(slot + 16u * kShThreads, A.y + j0);
    cp_async16(slot + 32u * kShThreads, A.dx + j0);
    cp_async16(slot + 48u * kShThreads, A.dy + j0);
  };
  if (kPf) {
    const int64_t j0 = (int64_t)blockIdx.x * blockDim.x * R + (int64_t)threadIdx.x * R;
    if (j0 + 3 < n) prefetch(j0);
    cp_async_commit();
  }
  // block-uniform loop: every lane of every warp takes the same trip count,
  // so warp-collective histogram aggregation below is always legal.
  for (int64_t blk = (int64_t)blockIdx.x * blockDim.x * R; blk < n; blk += stride) {
    const int64_t i0 = blk + (int64_t)threadIdx.x * R;
    const bool vec = (R == 4) && (i0 + 3 < n);
    float x[R], y[R], dx[R], dy[R];
    if (kPf && vec) {  // the copies issued for these rays (same condition)
      cp_async_wait_all();
      const float4* sl = reinterpret_cast<const float4*>(shm) + threadIdx.x;
      const float4 a = sl[0], b = sl[kShThreads], c = sl[2 * kShThreads], d = sl[3 * kShThreads];
      x[0] = a.x; x[1 % R] = a.y; x[2 % R] = a.z; x[3 % R] = a.w;
      y[0] = b.x; y[1 % R] = b.y; y[2 % R] = b.z; y[3 % R] = b.w;
      dx[0] = c.x; dx[1 % R] = c.y; dx[2 % R] = c.z; dx[3 % R] = c.w;
      dy[0] = d.x; dy[1 % R] = d.y; dy[2 % R] = d.z; dy[3 % R] = d.w;
    } else {
      load4<R>(A.x, i0, n, x, vec);
      load4<R>(A.y, i0, n, y, vec);
      load4<R>(A.dx, i0, n, dx, vec);
      load4<R>(A.dy, i0, n, dy, vec);
    }
    const int64_t ni0 = i0 + stride;
    // the slot is free once the values read from it have been used
    auto next = [&]() {
      if (kPf) {
        if (ni0 + 3 < n) prefetch(ni0);
        cp_async_commit();
      }
    };
    fwd_rays<R, CountT, kSh>(P, A, B, shw, i0, x, y, dx, dy, vec, next);
  }
  if (kSh) sh_store_row(shw, A.rows + (size_t)blockIdx.x * sh_words(bins), sh_words(bins));
}

// hist[b] += sum over the CTA rows of their packed uint16 counters.  A block
// takes 32 words (64 bins) and splits the rows over its 8 warps (warp g sums
// rows g, g + 8, ...: each load of a warp is one 128-byte run), so that a
// thread keeps only ~nrows / 8 loads in its chain; the 8 partial sums are
// then added in shared memory.  Integer sums: the order does not matter.
constexpr int kRowsWords = 32, kRowsGroups = 8;

template <typename CountT>
__global__ void __launch_bounds__(kRowsWords * kRowsGroups)
k_hist_rows(const uint32_t* __restrict__ rows, int nrows, int bins, CountT* __restrict__ hist) {
  __shared__ unsigned long long slo[kRowsGroups][kRowsWords], shi[kRowsGroups][kRowsWords];
  const int words = sh_words(bins);
  const int wi = threadIdx.x % kRowsWords, g = threadIdx.x / kRowsWords;
  const int i = blockIdx.x * kRowsWords + wi;
  unsigned long long lo[4] = {0ull, 0ull, 0ull, 0ull}, hi[4] = {0ull, 0ull, 0ull, 0ull};
  if (i < words) {
    int r = g;
    for (; r + 3 * kRowsGroups < nrows; r += 4 * kRowsGroups) {  // four loads in flight
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const uint32_t v = __ldcs(rows + (size_t)(r + u * kRowsGroups) * words + i);
        lo[u] += v & 0xffffu;
        hi[u] += v >> 16;
      }
    }
    for (; r < nrows; r += kRowsGroups) {
      const uint32_t v = __ldcs(rows + (size_t)r * words + i);
      lo[0] += v & 0xffffu;
      hi[0] += v >> 16;
    }
  }
  slo[g][wi] = (lo[0] + lo[1]) + (lo[2] + lo[3]);
  shi[g][wi] = (hi[0] + hi[1]) + (hi[2] + hi[3]);
  __syncthreads();
  if (g == 0 && i < words) {
    unsigned long long a = 0ull, b = 0ull;
#pragma unroll
    for (int k = 0; k < kRowsGroups; ++k) {
      a += slo[k][wi];
      b += shi[k][wi];
    }
    hist[2 * i] += (CountT)a;
    if (2 * i + 1 < bins) hist[2 * i + 1] += (CountT)b;
  }
}

static inline int hist_rows_blocks(int bins) { return (sh_words(bins) + kRowsWords - 1) / kRowsWords; }

struct BinArgs {
  int64_t n;
  const float *x, *y;
  const uint8_t* mask;
  int32_t *pix_y, *pix_x;
  void* hist;
  int32_t h, w;
  uint32_t* rows;  // shared-histogram variant: per-CTA packed uint16 counters
};

// kSh: the shared-memory histogram variant (as for k_trace_fwd).
template <typename CountT, bool kSh = false>
__global__ void __launch_bounds__(kSh ? kShThreads : 256)
k_bin(const __grid_constant__ BinArgs A, const __grid_constant__ BinCoef B) {
  extern __shared__ uint32_t shw[];
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int bins = A.h * A.w;
  if (kSh) {
    for (int i = threadIdx.x; i < ((bins + 1) >> 1); i += blockDim.x) shw[i] = 0u;
    __syncthreads();
  }
  for (int64_t blk = (int64_t)blockIdx.x * blockDim.x; blk < A.n; blk += stride) {
    const int64_t i = blk + threadIdx.x;
    const bool inr = i < A.n;
    float x = inr ? A.x[i] : 0.f, y = inr ? A.y[i] : 0.f;
    int py, px;
    bin_yx(x, y, B, py, px);
    if (inr) {
      if (A.pix_y) A.pix_y[i] = py;
      if (A.pix_x) A.pix_x[i] = px;
      if (!(isfinite(x) && isfinite(y))) atomicOr(&g_tg_err, TG_EW_NONFINITE);
    }
    if (A.hist) {
      bool ok = inr && (!A.mask || A.mask[i]) && py >= 0 && py < A.h && px >= 0 && px < A.w;
      if (kSh) hist_add_sh<CountT>(shw, ok ? py * A.w + px : 0, ok, reinterpret_cast<CountT*>(A.hist));
      else hist_add_warp<CountT>(reinterpret_cast<CountT*>(A.hist), ok ? py * A.w + px : 0, ok);
    }
  }
  if (kSh) sh_store_row(shw, A.rows + (size_t)blockIdx.x * sh_words(bins), sh_words(bins));
}

// Histogram of existing pixel indices (grid.py:231-280 into_image given
// (py, px)): out-of-range indices are dropped.  kSh as for k_trace_fwd.
template <typename IdxT, typename CountT, bool kSh = false>
__global__ void __launch_bounds__(kSh ? kShThreads : 256)
k_hist_pix(int64_t n, const IdxT* __restrict__ pix_y, const IdxT* __restrict__ pix_x, int h, int w,
           CountT* __restrict__ hist, uint32_t* __restrict__ rows) {
  extern __shared__ uint32_t shw[];
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int bins = h * w;
  if (kSh) {
    for (int i = threadIdx.x; i < ((bins + 1) >> 1); i += blockDim.x) shw[i] = 0u;
    __syncthreads();
  }
  for (int64_t blk = (int64_t)blockIdx.x * blockDim.x; blk < n; blk += stride) {  // block-uniform
    const int64_t i = blk + threadIdx.x;
    const bool inr = i < n;
    const long long py = inr ? (long long)pix_y[i] : -1, px = inr ? (long long)pix_x[i] : -1;
    const bool ok = py >= 0 && py < h && px >= 0 && px < w;
    const int bin = ok ? (int)(py * w + px) : 0;
    if (kSh) hist_add_sh<CountT>(shw, bin, ok, hist);
    else hist_add_warp<CountT>(hist, bin, ok);
  }
  if (kSh) sh_store_row(shw, rows + (size_t)blockIdx.x * sh_words(bins), sh_words(bins));
}

static int sm_count() {
  static int cached = 0;
  if (!cached) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&cached, cudaDevAttrMultiProcessorCount, dev);
    if (cached <= 0) cached = 148;
  }
  return cached;
}

static inline bool al16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

}  // namespace tg

using namespace tg;

template <auto Kernel>
static int fwd_per_sm(int threads) {
  static int v = 0;
  if (!v) {
    int q = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&q, Kernel, threads, 0);
    v = q > 0 ? q : 1;
  }
  return v;
}

// The shared-histogram variant applies to histograms of at most kShMaxBins
// bins when there are enough rays per bin for the L2 atomics to dominate.
static bool use_shared_hist(int64_t n, int64_t h, int64_t w) {
  if (h <= 0 || w <= 0) return false;
  const int64_t bins = h * w;
  return bins <= kShMaxBins && n >= 32 * bins;
}

static bool use_shared_hist(int64_t n, const tg_grid* grid) {
  return grid && use_shared_hist(n, grid->h, grid->w);
}

// Opt a shared-histogram kernel into the full shared-memory budget, once per
// instantiation (before any graph capture that replays it).
template <auto Kernel>
static cudaError_t shared_hist_attr() {
  static cudaError_t done = cudaFuncSetAttribute(Kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (kShMaxBins / 2) * (int)sizeof(uint32_t));
  return done;
}

static size_t shared_hist_bytes(int64_t h, int64_t w) {
  return (size_t)sm_count() * (size_t)sh_words((int)(h * w)) * sizeof(uint32_t);
}

static size_t shared_hist_bytes(const tg_grid* grid) { return shared_hist_bytes(grid->h, grid->w); }

static int smem_optin() {
  static int v = 0;
  if (!v) {
    int dev = 0, q = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&q, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    v = q > 0 ? q : 48 * 1024;
  }
  return v;
}

// The prefetching shared-histogram kernel with the whole opt-in budget.
template <auto Kernel>
static cudaError_t prefetch_attr() {
  static cudaError_t done =
      cudaFuncSetAttribute(Kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_optin());
  return done;
}

static int trace_fwd_impl(const tg_model* model, const tg_rays* in, tg_rays* out,
                          double* z_out, const tg_grid* grid, int32_t* pix_y,
                          int32_t* pix_x, void* hist, int32_t hist_i64,
                          void* workspace, size_t ws_bytes, void* stream) {
  if (!model || !in || !out) return TG_ERR_INVALID;
  if (in->n < 0) return TG_ERR_INVALID;
  if (in->n > 0 && (!in->x || !in->y || !in->dx || !in->dy || !out->x || !out->y ||
                    !out->dx || !out->dy))
    return TG_ERR_INVALID;
  if ((pix_y || pix_x || hist) && !grid) return TG_ERR_INVALID;
  if (grid && (grid->h <= 0 || grid->w <= 0)) return TG_ERR_INVALID;
  Program P;
  int st = compile_program(model, in->z != nullptr, in->z_scalar, &P);
  if (st != TG_OK) return st;
  if (P.n_probe_ops) return TG_ERR_UNSUPPORTED;  // per-probe models: tg_scan_*
  if (z_out) *z_out = P.z_out;
  if (in->n == 0) return TG_OK;
  FwdArgs A;
  std::memset(&A, 0, sizeof(A));
  A.n = in->n;
  A.x = in->x; A.y = in->y; A.dx = in->dx; A.dy = in->dy;
  A.z = in->z; A.z_scalar = in->z_scalar;
  A.pl = in->pathlength; A.pl_scalar = in->pl_scalar;
  A.amp = in->amplitude;
  A.ox = out->x; A.oy = out->y; A.odx = out->dx; A.ody = out->dy;
  A.opl = out->pathlength; A.oz = out->z; A.oamp = out->amplitude;
  A.pix_y = pix_y; A.pix_x = pix_x; A.hist = hist;
  A.do_bin = (grid != nullptr) && (pix_y || pix_x || hist);
  BinCoef B;
  std::memset(&B, 0, sizeof(B));
  if (grid) {
    B = make_bincoef(grid);
    A.h = grid->h;
    A.w = grid->w;
  }
  bool vec = al16(A.x) && al16(A.y) && al16(A.dx) && al16(A.dy) && al16(A.ox) &&
             al16(A.oy) && al16(A.odx) && al16(A.ody);
  A.opl_vec = A.opl && al16(A.opl);
  A.pix_vec = (!pix_y || al16(pix_y)) && (!pix_x || al16(pix_x));
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (hist && workspace && use_shared_hist(A.n, grid) && ws_bytes >= shared_hist_bytes(grid) &&
      (reinterpret_cast<uintptr_t>(workspace) & 15) == 0) {
    // one CTA of kShThreads per SM, the detector's packed counters in shared memory
    const int bins = grid->h * grid->w;
    const size_t smem = (size_t)((bins + 1) / 2) * sizeof(uint32_t);
    const int R = vec ? 4 : 1;
    const int64_t need = (A.n + (int64_t)kShThreads * R - 1) / ((int64_t)kShThreads * R);
    const int blocks = (int)(need < sm_count() ? need : sm_count());
    A.rows = reinterpret_cast<uint32_t*>(workspace);
    cudaError_t e = cudaSuccess;
    if (vec && smem + kPfBytes <= (size_t)smem_optin()) {  // prefetch slots fit
      if (hist_i64) {
        e = prefetch_attr<k_trace_fwd<4, long long, true, true>>();
        if (e == cudaSuccess)
          k_trace_fwd<4, long long, true, true><<<blocks, kShThreads, smem + kPfBytes, s>>>(P, A, B);
      } else {
        e = prefetch_attr<k_trace_fwd<4, int, true, true>>();
        if (e == cudaSuccess)
          k_trace_fwd<4, int, true, true><<<blocks, kShThreads, smem + kPfBytes, s>>>(P, A, B);
      }
    } else if (vec) {
      if (hist_i64) {
        e = shared_hist_attr<k_trace_fwd<4, long long, true>>();
        if (e == cudaSuccess) k_trace_fwd<4, long long, true><<<blocks, kShThreads, smem, s>>>(P, A, B);
      } else {
        e = shared_hist_attr<k_trace_fwd<4, int, true>>();
        if (e == cudaSuccess) k_trace_fwd<4, int, true><<<blocks, kShThreads, smem, s>>>(P, A, B);
      }
    } else {
      if (hist_i64) {
        e = shared_hist_attr<k_trace_fwd<1, long long, true>>();
        if (e == cudaSuccess) k_trace_fwd<1, long long, true><<<blocks, kShThreads, smem, s>>>(P, A, B);
      } else {
        e = shared_hist_attr<k_trace_fwd<1, int, true>>();
        if (e == cudaSuccess) k_trace_fwd<1, int, true><<<blocks, kShThreads, smem, s>>>(P, A, B);
      }
    }
    if (e != cudaSuccess || cudaGetLastError() != cudaSuccess) return TG_ERR_CUDA;
    const int rb = hist_rows_blocks(bins);
    if (hist_i64) k_hist_rows<long long><<<rb, kRowsWords * kRowsGroups, 0, s>>>(A.rows, blocks, bins, reinterpret_cast<long long*>(hist));
    else k_hist_rows<int><<<rb, kRowsWords * kRowsGroups, 0, s>>>(A.rows, blocks, bins, reinterpret_cast<int*>(hist));
    return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
  }
  const int threads = 256;
  const int R = vec ? 4 : 1;
  int64_t blocks_needed = (A.n + (int64_t)threads * R - 1) / ((int64_t)threads * R);
  // every block resident at once: with the grid-stride loop each block has
  // the same share, so blocks waiting for a slot would lengthen the tail
  // residency per variant, queried once (a per-call query costs host time)
  const int per_sm = vec ? (hist_i64 ? fwd_per_sm<k_trace_fwd<4, long long>>(threads)
                                     : fwd_per_sm<k_trace_fwd<4, int>>(threads))
                         : (hist_i64 ? fwd_per_sm<k_trace_fwd<1, long long>>(threads)
                                     : fwd_per_sm<k_trace_fwd<1, int>>(threads));
  int64_t cap = (int64_t)sm_count() * per_sm;
  int blocks = (int)(blocks_needed < cap ? blocks_needed : cap);
  if (vec) {
    if (hist_i64) k_trace_fwd<4, long long><<<blocks, threads, 0, s>>>(P, A, B);
    else k_trace_fwd<4, int><<<blocks, threads, 0, s>>>(P, A, B);
  } else {
    if (hist_i64) k_trace_fwd<1, long long><<<blocks, threads, 0, s>>>(P, A, B);
    else k_trace_fwd<1, int><<<blocks, threads, 0, s>>>(P, A, B);
  }
  return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
}

extern "C" int tg_trace_fwd(const tg_model* model, const tg_rays* in, tg_rays* out,
                            double* z_out, const tg_grid* grid, int32_t* pix_y,
                            int32_t* pix_x, void* hist, int32_t hist_i64,
                            void* stream) {
  return trace_fwd_impl(model, in, out, z_out, grid, pix_y, pix_x, hist, hist_i64, nullptr, 0,
                        stream);
}

extern "C" size_t tg_trace_image_workspace(int64_t n, const tg_grid* grid) {
  return use_shared_hist(n, grid) ? shared_hist_bytes(grid) : 0;
}

extern "C" int tg_trace_image(const tg_model* model, const tg_rays* in, tg_rays* out,
                              double* z_out, const tg_grid* grid, int32_t* pix_y,
                              int32_t* pix_x, void* hist, int32_t hist_i64, void* workspace,
                              size_t ws_bytes, void* stream) {
  return trace_fwd_impl(model, in, out, z_out, grid, pix_y, pix_x, hist, hist_i64, workspace,
                        ws_bytes, stream);
}

static int bin_impl(int64_t n, const float* x, const float* y, const uint8_t* mask,
                    const tg_grid* grid, int32_t* pix_y, int32_t* pix_x, void* hist,
                    int32_t hist_i64, void* workspace, size_t ws_bytes, void* stream) {
  if (n < 0 || !grid || grid->h <= 0 || grid->w <= 0) return TG_ERR_INVALID;
  if (n > 0 && (!x || !y)) return TG_ERR_INVALID;
  if (n == 0) return TG_OK;
  BinArgs A;
  std::memset(&A, 0, sizeof(A));
  A.n = n; A.x = x; A.y = y; A.mask = mask; A.pix_y = pix_y; A.pix_x = pix_x;
  A.hist = hist; A.h = grid->h; A.w = grid->w;
  BinCoef B = make_bincoef(grid);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (hist && workspace && use_shared_hist(n, grid) && ws_bytes >= shared_hist_bytes(grid) &&
      (reinterpret_cast<uintptr_t>(workspace) & 15) == 0) {
    const int bins = grid->h * grid->w;
    const size_t smem = (size_t)((bins + 1) / 2) * sizeof(uint32_t);
    const int64_t need = (n + kShThreads - 1) / kShThreads;
    const int blocks = (int)(need < sm_count() ? need : sm_count());
    A.rows = reinterpret_cast<uint32_t*>(workspace);
    cudaError_t e;
    if (hist_i64) {
      e = shared_hist_attr<k_bin<long long, true>>();
      if (e == cudaSuccess) k_bin<long long, true><<<blocks, kShThreads, smem, s>>>(A, B);
    } else {
      e = shared_hist_attr<k_bin<int, true>>();
      if (e == cudaSuccess) k_bin<int, true><<<blocks, kShThreads, smem, s>>>(A, B);
    }
    if (e != cudaSuccess || cudaGetLastError() != cudaSuccess) return TG_ERR_CUDA;
    const int rb = hist_rows_blocks(bins);
    if (hist_i64) k_hist_rows<long long><<<rb, kRowsWords * kRowsGroups, 0, s>>>(A.rows, blocks, bins, reinterpret_cast<long long*>(hist));
    else k_hist_rows<int><<<rb, kRowsWords * kRowsGroups, 0, s>>>(A.rows, blocks, bins, reinterpret_cast<int*>(hist));
    return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
  }
  int64_t need = (n + 255) / 256;
  int per_sm = 1;
  if (hist_i64) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bin<long long>, 256, 0);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bin<int>, 256, 0);
  if (per_sm < 1) per_sm = 1;
  int64_t cap = (int64_t)sm_count() * per_sm;
  int blocks = (int)(need < cap ? need : cap);
  if (hist_i64) k_bin<long long><<<blocks, 256, 0, s>>>(A, B);
  else k_bin<int><<<blocks, 256, 0, s>>>(A, B);
  return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
}

extern "C" int tg_bin(int64_t n, const float* x, const float* y, const uint8_t* mask,
                      const tg_grid* grid, int32_t* pix_y, int32_t* pix_x, void* hist,
                      int32_t hist_i64, void* stream) {
  return bin_impl(n, x, y, mask, grid, pix_y, pix_x, hist, hist_i64, nullptr, 0, stream);
}

extern "C" int tg_bin_image(int64_t n, const float* x, const float* y, const uint8_t* mask,
                            const tg_grid* grid, int32_t* pix_y, int32_t* pix_x, void* hist,
                            int32_t hist_i64, void* workspace, size_t ws_bytes, void* stream) {
  return bin_impl(n, x, y, mask, grid, pix_y, pix_x, hist, hist_i64, workspace, ws_bytes, stream);
}

extern "C" size_t tg_hist_workspace(int64_t n, int32_t h, int32_t w) {
  return use_shared_hist(n, h, w) ? shared_hist_bytes(h, w) : 0;
}

template <typename IdxT, typename CountT>
static int hist_pix_launch(int64_t n, const void* py, const void* px, int h, int w, void* hist,
                           void* workspace, size_t ws_bytes, cudaStream_t s) {
  const IdxT* y = reinterpret_cast<const IdxT*>(py);
  const IdxT* x = reinterpret_cast<const IdxT*>(px);
  CountT* hh = reinterpret_cast<CountT*>(hist);
  const int bins = h * w;
  if (workspace && use_shared_hist(n, h, w) && ws_bytes >= shared_hist_bytes(h, w) &&
      (reinterpret_cast<uintptr_t>(workspace) & 15) == 0) {
    const size_t smem = (size_t)((bins + 1) / 2) * sizeof(uint32_t);
    const int64_t need = (n + kShThreads - 1) / kShThreads;
    const int blocks = (int)(need < sm_count() ? need : sm_count());
    uint32_t* rows = reinterpret_cast<uint32_t*>(workspace);
    const cudaError_t e = shared_hist_attr<k_hist_pix<IdxT, CountT, true>>();
    if (e != cudaSuccess) return TG_ERR_CUDA;
    k_hist_pix<IdxT, CountT, true><<<blocks, kShThreads, smem, s>>>(n, y, x, h, w, hh, rows);
    if (cudaGetLastError() != cudaSuccess) return TG_ERR_CUDA;
    k_hist_rows<CountT><<<hist_rows_blocks(bins), kRowsWords * kRowsGroups, 0, s>>>(rows, blocks, bins, hh);
  } else {
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_hist_pix<IdxT, CountT>, 256, 0);
    if (per_sm < 1) per_sm = 1;
    const int64_t need = (n + 255) / 256, cap = (int64_t)sm_count() * per_sm;
    k_hist_pix<IdxT, CountT><<<(int)(need < cap ? need : cap), 256, 0, s>>>(n, y, x, h, w, hh, nullptr);
  }
  return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
}

extern "C" int tg_hist_pixels(int64_t n, const void* pix_y, const void* pix_x, int32_t idx_i64,
                              int32_t h, int32_t w, void* hist, int32_t hist_i64, void* workspace,
                              size_t ws_bytes, void* stream) {
  if (n < 0 || h <= 0 || w <= 0 || !hist) return TG_ERR_INVALID;
  if ((int64_t)h * w > 0x7fffffff) return TG_ERR_TOO_LARGE;
  if (n > 0 && (!pix_y || !pix_x)) return TG_ERR_INVALID;
  if (n == 0) return TG_OK;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (idx_i64)
    return hist_i64 ? hist_pix_launch<long long, long long>(n, pix_y, pix_x, h, w, hist, workspace, ws_bytes, s)
                    : hist_pix_launch<long long, int>(n, pix_y, pix_x, h, w, hist, workspace, ws_bytes, s);
  return hist_i64 ? hist_pix_launch<int, long long>(n, pix_y, pix_x, h, w, hist, workspace, ws_bytes, s)
                  : hist_pix_launch<int, int>(n, pix_y, pix_x, h, w, hist, workspace, ws_bytes, s);
}

// =====================================================================
// Adjoint (reverse mode) of the forward chain.
//
// Each thread re-runs the forward chain for its rays (keeping only the final
// state and the biprism sign bits), then walks the steps backwards: it
// recovers the state entering each step by applying that step's inverse
// (every step is invertible; biprism signs come from the recorded bits),
// propagates the adjoint (lambda_x, lambda_y, lambda_dx, lambda_dy,
// lambda_pl) through the step's transposed Jacobian, and accumulates the
// step's parameter sensitivities.  Nothing is stored between the passes.
//
// Per-step sums (float32 within a warp, float64 across warps and blocks):
//   propagator : dL/dd
//   lens       : dL/df
//   shift      : dL/d(delta x, delta y, delta dx, delta dy)
//   deflector  : dL/d(def_x, def_y)
//   biprism    : dL/d(def_x)
//   rotator    : dL/d(angle in radians)
// Block partials go to the workspace and are reduced in a fixed order by a
// second kernel, so results are deterministic run to run.
// =====================================================================
namespace tg {

struct VjpArgs {
  int64_t n;
  const float *x, *y, *dx, *dy;
  const double* z;
  double z_scalar;
  const float *gx, *gy, *gdx, *gdy;
  const double* gpl;
  float *ix, *iy, *idx, *idy;
  double *ipl, *iz;
  double* partial;  // [gridDim.x][n_steps][4], NULL: no parameter sums
};

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ int op_nsums(int kind) {
  switch (kind) {
    case OP_FREE: case OP_FREE_VARZ: case OP_LENS: case OP_BIPRISM: case OP_ROTATE: case OP_ABER: return 1;
    case OP_DEFLECT: return 2;
    case OP_SHIFT: case OP_PROBE_SHIFT: return 4;
    default: return 0;
  }
}

constexpr int kVjpThreads = 256;
constexpr int kVjpRays = 8;  // rays per thread on the aligned path

// Eight rays per thread under a two-blocks-per-SM register bound (128
// registers, a few bytes spilled): the per-ray chains are long and
// dependent, so independent rays in flight per thread matter more than
// warps per SM.  Measured at 16.8 M rays: 0.197 ms with 4 rays (79
// registers, 3 blocks), 0.251 ms with 2, 0.375 ms with 1, 0.215 ms with 8
// unbounded (144 registers, 1 block), 0.172 ms with 8 bounded.
// ABER: the model holds aberrated lenses.  Their slope map has no
// closed-form inverse, so at each one the reverse walk recomputes the state
// entering it from the ray's input (forward steps up to the lens) and applies
// the lens's adjoint (aber_reverse); the other steps invert as usual.
template <int R, bool ABER>
__global__ void __launch_bounds__(kVjpThreads, 2)
k_trace_vjp(const __grid_constant__ Program P, const __grid_constant__ VjpArgs A) {
  const float* aw = ABER ? &P.aber[0][0] : nullptr;
  // per-warp float32 step sums (each warp owns a row: no atomics, no float64
  // in the ray loop); combined in float64 in warp order at the end
  __shared__ float wacc[kVjpThreads / 32][kMaxSteps * 4];
  const bool sums = A.partial != nullptr;
  if (sums)
    for (int i = threadIdx.x; i < (kVjpThreads / 32) * kMaxSteps * 4; i += blockDim.x) (&wacc[0][0])[i] = 0.f;
  __syncthreads();
  const int64_t n = A.n;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x * R;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t blk = (int64_t)blockIdx.x * blockDim.x * R; blk < n; blk += stride) {
    const int64_t i0 = blk + (int64_t)threadIdx.x * R;
    const bool vec = (R == 4 || R == 8) && (i0 + R - 1 < n);
    float x[R], y[R], dx[R], dy[R];
    load4<R>(A.x, i0, n, x, vec);
    load4<R>(A.y, i0, n, y, vec);
    load4<R>(A.dx, i0, n, dx, vec);
    load4<R>(A.dy, i0, n, dy, vec);
    RayS r[R];
    Adj ad[R];
    float dvf[R];  // per-ray first distance (per-ray input z only)
    uint64_t sb[R];
    bool alive[R];
    float gz[R];
    float gx[R], gy[R], gdx[R], gdy[R];
    load4<R>(A.gx, i0, n, gx, vec);
    load4<R>(A.gy, i0, n, gy, vec);
    load4<R>(A.gdx, i0, n, gdx, vec);
    load4<R>(A.gdy, i0, n, gdy, vec);
#pragma unroll
    for (int k = 0; k < R; ++k) {
      const bool inr = i0 + k < n;
      r[k] = RayS{x[k], y[k], dx[k], dy[k], 0.f};
      dvf[k] = 0.f;
      sb[k] = 0;
      alive[k] = true;
      gz[k] = 0.f;
      float gp = (A.gpl && inr) ? (float)A.gpl[i0 + k] : 0.f;
      // rays beyond n carry zero adjoints so they add nothing to the sums
      ad[k] = inr ? Adj{gx[k], gy[k], gdx[k], gdy[k], gp} : Adj{0.f, 0.f, 0.f, 0.f, 0.f};
    }
    if (A.z) {
#pragma unroll
      for (int k = 0; k < R; ++k) dvf[k] = (float)(P.zc_first - (i0 + k < n ? A.z[i0 + k] : A.z_scalar));
    }
    for (int s = 0; s < P.n_steps; ++s) {
      const Op op = P.op[s];
#pragma unroll
      for (int k = 0; k < R; ++k)
        op_forward(op, nullptr, r[k], dvf[k], sb[k], alive[k], aw);
    }
    for (int s = P.n_steps - 1; s >= 0; --s) {
      const Op op = P.op[s];
      float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int k = 0; k < R; ++k) {
        float ck[4] = {0.f, 0.f, 0.f, 0.f};
        if (ABER && op.kind == OP_ABER) {
          RayS q{x[k], y[k], dx[k], dy[k], 0.f};  // recompute the state entering the lens
          uint64_t sq = 0;
          bool aq = true;
          for (int t = 0; t < s; ++t) op_forward(P.op[t], nullptr, q, dvf[k], sq, aq, aw);
          aber_reverse(aw + op.aux * kAberFloats, op.c[0], op.c[1], q, ad[k], ck[0]);
          r[k] = q;
        } else {
          op_reverse(op, nullptr, r[k], ad[k], sb[k], dvf[k], ck, gz[k]);
        }
        c[0] += ck[0]; c[1] += ck[1]; c[2] += ck[2]; c[3] += ck[3];
      }
      if (sums) {
        const int ns = op_nsums(op.kind);
        for (int j = 0; j < ns; ++j) {
          float v = warp_sum(c[j]);
          if (lane == 0) wacc[warp][4 * s + j] += v;
        }
      }
    }
#pragma unroll
    for (int k = 0; k < R; ++k) {
      gx[k] = ad[k].lx; gy[k] = ad[k].ly; gdx[k] = ad[k].ldx; gdy[k] = ad[k].ldy;
    }
    if (A.ix) store4<R>(A.ix, i0, n, gx, vec);
    if (A.iy) store4<R>(A.iy, i0, n, gy, vec);
    if (A.idx) store4<R>(A.idx, i0, n, gdx, vec);
    if (A.idy) store4<R>(A.idy, i0, n, gdy, vec);
#pragma unroll
    for (int k = 0; k < R; ++k) {
      if (i0 + k < n) {
        if (A.ipl) A.ipl[i0 + k] = A.gpl ? A.gpl[i0 + k] : 0.0;
        if (A.iz) A.iz[i0 + k] = f32_to_f64(gz[k]);
      }
    }
  }
  if (sums) {
    __syncthreads();
    double* dst = A.partial + (size_t)blockIdx.x * P.n_steps * 4;
    for (int i = threadIdx.x; i < P.n_steps * 4; i += blockDim.x) {
      double t = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += (double)wacc[w][i];
      dst[i] = t;
    }
  }
}

// ---------------------------------------------------- lean adjoint
// k_trace_vjp_lean: the adjoint for the chains most calls trace: free space
// (paraxial or direction cosines, uniform distances), lenses, scanners /
// descanners (shifts), deflectors, rotators and apertures, with no upstream
// pathlength gradient.  The pathlength adjoint is then zero at every step
// (no step feeds it), no biprism sign or per-ray distance has to be kept,
// and an aperture's mask does not enter the adjoint, so each ray carries its
// state (x, y, dx, dy) and its adjoint (lx, ly, ldx, ldy) only: 8 registers
// a ray instead of ~14, which buys more rays in flight per SM.  The step
// arithmetic is op_forward / op_reverse with the pathlength terms taken out
// (they multiply the zero adjoint).
__host__ __device__ inline bool lean_kind(int kind) {
  return kind == OP_NOP || kind == OP_FREE || kind == OP_LENS || kind == OP_SHIFT ||
         kind == OP_DEFLECT || kind == OP_ROTATE || kind == OP_APERTURE;
}

struct Ray4 {
  float x, y, dx, dy;
};

__device__ __forceinline__ void lean_forward(const Op& op, Ray4& r) {
  switch (op.kind) {
    case OP_FREE: {
      const float d = op.c[0];
      if (op.aux) {
        const float t = d / (1.f + fmaf(r.dx, r.dx, r.dy * r.dy));
        r.x = fmaf(r.dx, t, r.x);
        r.y = fmaf(r.dy, t, r.y);
      } else {
        r.x = fmaf(r.dx, d, r.x);
        r.y = fmaf(r.dy, d, r.y);
      }
    } break;
    case OP_LENS:
      r.dx = fmaf(-r.x, op.c[0], r.dx);
      r.dy = fmaf(-r.y, op.c[0], r.dy);
      break;
    case OP_SHIFT:
      r.x += op.c[0]; r.y += op.c[1]; r.dx += op.c[2]; r.dy += op.c[3];
      break;
    case OP_DEFLECT:
      r.dx += op.c[0]; r.dy += op.c[1];
      break;
    case OP_ROTATE: {
      const float c = op.c[0], sn = op.c[1];
      const float x = r.x, y = r.y, dx = r.dx, dy = r.dy;
      r.x = fmaf(x, c, -(y * sn));
      r.y = fmaf(x, sn, y * c);
      r.dx = fmaf(dx, c, -(dy * sn));
      r.dy = fmaf(dx, sn, dy * c);
    } break;
    default:  // OP_NOP, OP_APERTURE (its mask does not enter the adjoint)
      break;
  }
}

__device__ __forceinline__ void lean_reverse(const Op& op, Ray4& r, Ray4& a, float c[4]) {
  switch (op.kind) {
    case OP_FREE: {
      const float d = op.c[0];
      if (op.aux) {
        const float dx = r.dx, dy = r.dy;
        const float n2 = 1.f + fmaf(dx, dx, dy * dy);
        const float inv = 1.f / n2;
        c[0] = (a.x * dx + a.y * dy) * inv;
        const float t = d / n2;
        r.x = fmaf(-dx, t, r.x);
        r.y = fmaf(-dy, t, r.y);
        const float di = d * inv, di2 = 2.f * di * inv;
        const float jxx = di - di2 * dx * dx, jyy = di - di2 * dy * dy, jxy = -di2 * dx * dy;
        a.dx += a.x * jxx + a.y * jxy;
        a.dy += a.x * jxy + a.y * jyy;
      } else {
        c[0] = a.x * r.dx + a.y * r.dy;
        r.x = fmaf(-r.dx, d, r.x);
        r.y = fmaf(-r.dy, d, r.y);
        a.dx = fmaf(a.x, d, a.dx);
        a.dy = fmaf(a.y, d, a.dy);
      }
    } break;
    case OP_LENS: {
      const float k = op.c[0];
      const float x = r.x, y = r.y;
      r.dx = fmaf(x, k, r.dx);
      r.dy = fmaf(y, k, r.dy);
      c[0] = (a.dx * x + a.dy * y) * (k * k);
      a.x = a.x - a.dx * k;
      a.y = a.y - a.dy * k;
    } break;
    case OP_SHIFT:
      r.x -= op.c[0]; r.y -= op.c[1]; r.dx -= op.c[2]; r.dy -= op.c[3];
      c[0] = a.x; c[1] = a.y; c[2] = a.dx; c[3] = a.dy;
      break;
    case OP_DEFLECT:
      c[0] = a.dx; c[1] = a.dy;
      r.dx -= op.c[0]; r.dy -= op.c[1];
      break;
    case OP_ROTATE: {
      const float cs = op.c[0], sn = op.c[1];
      c[0] = -a.x * r.y + a.y * r.x - a.dx * r.dy + a.dy * r.dx;
      const float x = r.x, y = r.y, dx = r.dx, dy = r.dy;
      r.x = x * cs + y * sn;
      r.y = -x * sn + y * cs;
      r.dx = dx * cs + dy * sn;
      r.dy = -dx * sn + dy * cs;
      const float lx = a.x, ly = a.y, ldx = a.dx, ldy = a.dy;
      a.x = lx * cs + ly * sn;
      a.y = -lx * sn + ly * cs;
      a.dx = ldx * cs + ldy * sn;
      a.dy = -ldx * sn + ldy * cs;
    } break;
    default:
      break;
  }
}

// Shape measured at 16.8 M rays (Lens + Detector, CUDA events): 8 rays a
// thread at two blocks per SM (124 registers) 0.160 ms, three blocks (80
// registers) 0.209 ms, 4 rays at four / five blocks 0.214 / 0.261 ms; with
// evict-first loads and stores 0.157 ms (three blocks 0.189 ms).
constexpr int kLeanRays = 8;    // rays per thread
constexpr int kLeanBlocks = 2;  // resident blocks per SM (register bound)

template <int R>
__global__ void __launch_bounds__(kVjpThreads, kLeanBlocks)
k_trace_vjp_lean(const __grid_constant__ Program P, const __grid_constant__ VjpArgs A) {
  __shared__ float wacc[kVjpThreads / 32][kMaxSteps * 4];
  const bool sums = A.partial != nullptr;
  if (sums)
    for (int i = threadIdx.x; i < (kVjpThreads / 32) * kMaxSteps * 4; i += blockDim.x) (&wacc[0][0])[i] = 0.f;
  __syncthreads();
  const int64_t n = A.n;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x * R;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t blk = (int64_t)blockIdx.x * blockDim.x * R; blk < n; blk += stride) {
    const int64_t i0 = blk + (int64_t)threadIdx.x * R;
    const bool vec = i0 + R - 1 < n;
    Ray4 r[R], ad[R];
    {
      float x[R], y[R], dx[R], dy[R], gx[R], gy[R], gdx[R], gdy[R];
      load4<R, true>(A.x, i0, n, x, vec);
      load4<R, true>(A.y, i0, n, y, vec);
      load4<R, true>(A.dx, i0, n, dx, vec);
      load4<R, true>(A.dy, i0, n, dy, vec);
      load4<R, true>(A.gx, i0, n, gx, vec);
      load4<R, true>(A.gy, i0, n, gy, vec);
      load4<R, true>(A.gdx, i0, n, gdx, vec);
      load4<R, true>(A.gdy, i0, n, gdy, vec);
#pragma unroll
      for (int k = 0; k < R; ++k) {
        r[k] = Ray4{x[k], y[k], dx[k], dy[k]};
        // rays beyond n carry zero adjoints (load4 reads them as 0)
        ad[k] = Ray4{gx[k], gy[k], gdx[k], gdy[k]};
      }
    }
    for (int s = 0; s < P.n_steps; ++s) {
      const Op op = P.op[s];
#pragma unroll
      for (int k = 0; k < R; ++k) lean_forward(op, r[k]);
    }
    for (int s = P.n_steps - 1; s >= 0; --s) {
      const Op op = P.op[s];
      float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int k = 0; k < R; ++k) {
        float ck[4] = {0.f, 0.f, 0.f, 0.f};
        lean_reverse(op, r[k], ad[k], ck);
        c[0] += ck[0]; c[1] += ck[1]; c[2] += ck[2]; c[3] += ck[3];
      }
      if (sums) {
        const int ns = op_nsums(op.kind);
        for (int j = 0; j < ns; ++j) {
          float v = warp_sum(c[j]);
          if (lane == 0) wacc[warp][4 * s + j] += v;
        }
      }
    }
    float o[R];
#pragma unroll
    for (int k = 0; k < R; ++k) o[k] = ad[k].x;
    if (A.ix) store4<R, true>(A.ix, i0, n, o, vec);
#pragma unroll
    for (int k = 0; k < R; ++k) o[k] = ad[k].y;
    if (A.iy) store4<R, true>(A.iy, i0, n, o, vec);
#pragma unroll
    for (int k = 0; k < R; ++k) o[k] = ad[k].dx;
    if (A.idx) store4<R, true>(A.idx, i0, n, o, vec);
#pragma unroll
    for (int k = 0; k < R; ++k) o[k] = ad[k].dy;
    if (A.idy) store4<R, true>(A.idy, i0, n, o, vec);
#pragma unroll
    for (int k = 0; k < R; ++k) {
      if (i0 + k < n) {
        if (A.ipl) A.ipl[i0 + k] = 0.0;  // no upstream pathlength gradient
        if (A.iz) A.iz[i0 + k] = 0.0;    // uniform input z
      }
    }
  }
  if (sums) {
    __syncthreads();
    double* dst = A.partial + (size_t)blockIdx.x * P.n_steps * 4;
    for (int i = threadIdx.x; i < P.n_steps * 4; i += blockDim.x) {
      double t = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += (double)wacc[w][i];
      dst[i] = t;
    }
  }
}

// raw[i] += sum over blocks of partial[b][i]: one block per entry i, thread t
// adds the blocks t, t + 256, ... in order, then a fixed shared-memory tree
// combines the 256 sums (the same order on every run).
constexpr int kReduceThreads = 256;

__global__ void __launch_bounds__(kReduceThreads)
k_reduce_partials(const double* __restrict__ partial, int nblocks, int width, double* __restrict__ raw) {
  __shared__ double sh[kReduceThreads];
  const int i = blockIdx.x;
  double a = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += kReduceThreads) a += partial[(size_t)b * width + i];
  sh[threadIdx.x] = a;
  __syncthreads();
#pragma unroll
  for (int h = kReduceThreads / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) sh[threadIdx.x] += sh[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) raw[i] += sh[0];
}

template <auto Kernel>
static int vjp_per_sm() {
  static int per_sm = 0;
  if (!per_sm) {
    int v = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, Kernel, kVjpThreads, 0);
    per_sm = v > 0 ? v : 1;
  }
  return per_sm;
}

static int vjp_grid(int64_t n, bool lean) {
  const int per_sm = lean ? vjp_per_sm<k_trace_vjp_lean<kLeanRays>>() : vjp_per_sm<k_trace_vjp<kVjpRays, false>>();
  const int64_t per_block = (int64_t)kVjpThreads * (lean ? kLeanRays : kVjpRays);
  int64_t need = (n + per_block - 1) / per_block;
  int64_t cap = (int64_t)sm_count() * per_sm;
  int64_t g = need < cap ? need : cap;
  return (int)(g < 1 ? 1 : g);
}

// Blocks whose partial sums a workspace must hold (either kernel).
static int vjp_grid_max(int64_t n) {
  const int a = vjp_grid(n, false), b = vjp_grid(n, true);
  return a > b ? a : b;
}

}  // namespace tg

extern "C" size_t tg_trace_vjp_workspace(int64_t n, const tg_model* model) {
  if (!model || n < 0) return 0;
  return (size_t)vjp_grid_max(n) * (size_t)(2 * model->n_components) * 4 * sizeof(double);
}

extern "C" int tg_trace_vjp(const tg_model* model, const tg_rays* in, const tg_rays* gout,
                            tg_rays* gin, double* raw, void* workspace, size_t ws_bytes,
                            void* stream) {
  if (!model || !in || !gout) return TG_ERR_INVALID;
  if (in->n < 0 || gout->n != in->n) return TG_ERR_INVALID;
  if (in->n > 0 && (!in->x || !in->y || !in->dx || !in->dy || !gout->x || !gout->y ||
                    !gout->dx || !gout->dy))
    return TG_ERR_INVALID;
  Program P;
  int st = compile_program(model, in->z != nullptr, in->z_scalar, &P);
  if (st != TG_OK) return st;
  if (P.n_probe_ops) return TG_ERR_UNSUPPORTED;
  if (in->n == 0) return TG_OK;
  VjpArgs A;
  std::memset(&A, 0, sizeof(A));
  A.n = in->n;
  A.x = in->x; A.y = in->y; A.dx = in->dx; A.dy = in->dy;
  A.z = in->z; A.z_scalar = in->z_scalar;
  A.gx = gout->x; A.gy = gout->y; A.gdx = gout->dx; A.gdy = gout->dy;
  A.gpl = gout->pathlength;
  if (gin) {
    if (gin->n != in->n) return TG_ERR_INVALID;
    A.ix = gin->x; A.iy = gin->y; A.idx = gin->dx; A.idy = gin->dy;
    A.ipl = gin->pathlength; A.iz = gin->z;
  }
  A.partial = (raw && P.n_steps > 0) ? reinterpret_cast<double*>(workspace) : nullptr;
  bool vec = al16(A.x) && al16(A.y) && al16(A.dx) && al16(A.dy) && al16(A.gx) &&
             al16(A.gy) && al16(A.gdx) && al16(A.gdy) && (!A.ix || al16(A.ix)) &&
             (!A.iy || al16(A.iy)) && (!A.idx || al16(A.idx)) && (!A.idy || al16(A.idy));
  bool lean = vec && P.n_aber == 0 && !A.z && !A.gpl;
  for (int i = 0; i < P.n_steps && lean; ++i) lean = lean_kind(P.op[i].kind);
  const int grid = vjp_grid(in->n, lean);
  const size_t need = (size_t)grid * P.n_steps * 4 * sizeof(double);
  if (A.partial && (!workspace || ws_bytes < need)) return TG_ERR_WORKSPACE;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (P.n_aber > 0) {
    if (vec) k_trace_vjp<4, true><<<grid, kVjpThreads, 0, s>>>(P, A);
    else k_trace_vjp<1, true><<<grid, kVjpThreads, 0, s>>>(P, A);
  } else {
    if (lean) k_trace_vjp_lean<kLeanRays><<<grid, kVjpThreads, 0, s>>>(P, A);
    else if (vec) k_trace_vjp<kVjpRays, false><<<grid, kVjpThreads, 0, s>>>(P, A);
    else k_trace_vjp<1, false><<<grid, kVjpThreads, 0, s>>>(P, A);
  }
  if (A.partial) {
    int width = P.n_steps * 4;
    k_reduce_partials<<<width, kReduceThreads, 0, s>>>(A.partial, grid, width, raw);
  }
  return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
}

// ------------------------------------------------------- tg_trace_adj
// Gradient of loss = sum_i |(x, y)_out,i - target_i|^2 for one model in one
// call: forward trace into the workspace, upstream gradient 2 (out - target),
// then the adjoint.  Workspace layout (256-byte aligned pieces): x, y, dx, dy
// outputs (float32 [4][n]), upstream x, y, zero dx, dy (float32 [4][n]), the
// adjoint's partial sums.
namespace tg {

__global__ void k_residual_grad(int64_t n, const float* __restrict__ ox, const float* __restrict__ oy,
                                const float* __restrict__ tx, const float* __restrict__ ty,
                                float* __restrict__ gx, float* __restrict__ gy, float* __restrict__ gdx,
                                float* __restrict__ gdy) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    gx[i] = 2.f * (ox[i] - tx[i]);
    gy[i] = 2.f * (oy[i] - ty[i]);
    gdx[i] = 0.f;
    gdy[i] = 0.f;
  }
}

static inline size_t al256t(size_t v) { return (v + 255) & ~(size_t)255; }

}  // namespace tg

extern "C" size_t tg_trace_adj_workspace(int64_t n, const tg_model* model) {
  if (!model || n < 0) return 0;
  const size_t vec = al256t((size_t)n * sizeof(float));
  return 8 * vec + al256t(tg_trace_vjp_workspace(n, model));
}

extern "C" int tg_trace_adj(const tg_model* model, const tg_rays* in, const float* target_x,
                            const float* target_y, double* dparams, tg_rays* dray, void* workspace,
                            size_t ws_bytes, void* stream) {
  if (!model || !in || !dparams) return TG_ERR_INVALID;
  if (in->n < 0 || (in->n > 0 && (!target_x || !target_y))) return TG_ERR_INVALID;
  const int64_t n = in->n;
  const size_t need = tg_trace_adj_workspace(n, model);
  if (!workspace || ws_bytes < need) return TG_ERR_WORKSPACE;
  if (((uintptr_t)workspace & 255) != 0) return TG_ERR_ALIGN;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const size_t steps = (size_t)(2 * model->n_components);
  if (cudaMemsetAsync(dparams, 0, steps * 4 * sizeof(double), s) != cudaSuccess) return TG_ERR_CUDA;
  if (n == 0) return TG_OK;
  char* ws = reinterpret_cast<char*>(workspace);
  const size_t vec = al256t((size_t)n * sizeof(float));
  float* v[8];
  for (int i = 0; i < 8; ++i) v[i] = reinterpret_cast<float*>(ws + i * vec);
  tg_rays out;
  std::memset(&out, 0, sizeof(out));
  out.n = n;
  out.x = v[0]; out.y = v[1]; out.dx = v[2]; out.dy = v[3];
  int st = tg_trace_fwd(model, in, &out, nullptr, nullptr, nullptr, nullptr, nullptr, 0, stream);
  if (st != TG_OK) return st;
  int blocks = (int)((n + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  k_residual_grad<<<blocks, 256, 0, s>>>(n, v[0], v[1], target_x, target_y, v[4], v[5], v[6], v[7]);
  tg_rays gout;
  std::memset(&gout, 0, sizeof(gout));
  gout.n = n;
  gout.x = v[4]; gout.y = v[5]; gout.dx = v[6]; gout.dy = v[7];
  return tg_trace_vjp(model, in, &gout, dray, dparams, ws + 8 * vec, ws_bytes - 8 * vec, stream);
}

namespace tg {
__global__ void k_selftest_add(const double* __restrict__ b, const float* __restrict__ p,
                               double* __restrict__ fast, double* __restrict__ ref, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    fast[i] = add_f64_f32(b[i], p[i]);
    ref[i] = __dadd_rn(b[i], (double)p[i]);
  }
}
}  // namespace tg

extern "C" int tg_selftest_add_f64_f32(const double* b, const float* p, double* fast, double* ref,
                                       int64_t n, void* stream) {
  if (n < 0 || (n > 0 && (!b || !p || !fast || !ref))) return TG_ERR_INVALID;
  if (n == 0) return TG_OK;
  int blocks = (int)((n + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  k_selftest_add<<<blocks, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(b, p, fast, ref, n);
  return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
}
