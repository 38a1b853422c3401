// field_gemm.cu - separable beamlet field as a split-BF16 complex GEMM on the
// 5th-generation tensor cores (tcgen05 + TMEM + TMA), sm_103a.
//
// For separable beams the detector field is F[row][col] = sum_b V[row][b] U[b][col]
// (field.cu, k_field_operands).  Each complex operand is stored as bf16 planes
// re_hi, re_lo, im_hi, im_lo (value ~= hi + lo to ~2^-17 relative), K-major
// (beam index contiguous).  Per 16-deep K slice the CTA issues 12 MMAs
// (hi*hi + hi*lo + lo*hi) into two float32 accumulators held in tensor
// memory, each 128 x 256 with the U operand stacked as [Ur | Ui]:
//   D0 = Vr [Ur | Ui],  D1 = Vi [Ur | Ui];
//   Fr = D0[:, :128] - D1[:, 128:],  Fi = D0[:, 128:] + D1[:, :128].
// Output tile 128 x 128 complex (UMMA M = 128, N = 256, K = 16: six MMAs per
// K slice), K blocks of 32 bf16 (64-byte rows, 64-byte swizzle), a 3-stage
// TMA -> MMA pipeline on mbarriers, split-K over beams across CTAs (partials
// reduced deterministically in field.cu).
// Roles: warp 0 lane 0 issues TMA loads, warp 1 lane 0 issues MMAs, all four
// warps drain TMEM in the epilogue.  Every wait is bounded: on timeout the
// kernel records TG_EW_MMA, drains its own copies (bounded) and frees TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "tg_common.cuh"

TG_DEFINE_ERROR_WORD(gemm)

namespace tg {

constexpr int kGStages = 3;
constexpr int kTileBytes = 128 * 64;            // 128 lines x 32 bf16
constexpr int kStageBytes = 8 * kTileBytes;     // 4 V planes + [Ur;Ui] hi and lo
constexpr int kGemmSmem = kGStages * kStageBytes + 1024 /*align*/ + 256 /*barriers*/;
// kind::f16 instruction descriptor: f32 accumulate, bf16 A and B, both
// K-major, N = 256, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((256u >> 3) << 17) | ((128u >> 4) << 24);
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int c0, int c1,
                                            uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(mbar)
      : "memory");
}

// K-major, 64-byte swizzle shared-memory matrix descriptor (tcgen05 format).
__device__ __forceinline__ uint64_t sdesc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);   // start address
  d |= (uint64_t)1 << 16;                    // leading byte offset (unused, 1)
  d |= (uint64_t)(512u >> 4) << 32;          // stride byte offset: 8 rows x 64 B
  d |= (uint64_t)1 << 46;                    // descriptor version
  d |= (uint64_t)4 << 61;                    // SWIZZLE_64B
  return d;
}

__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(kIdesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t mbar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
      : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}

struct GemmMaps {
  CUtensorMap v[4];
  CUtensorMap u[4];
};

struct GemmArgs {
  int32_t nkb;     // K blocks (of 32) per split
  int32_t h, w;
  float2* part;    // [splits][h][w]
};

__global__ void __launch_bounds__(128, 1)
k_field_gemm(const __grid_constant__ GemmMaps maps, const __grid_constant__ GemmArgs A) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kGStages * kStageBytes);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * kGStages + 2);
  const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + kGStages);
  const uint32_t done = smem_u32(bars + 2 * kGStages);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int mt = blockIdx.x, nt = blockIdx.y, sp = blockIdx.z;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kGStages; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(
                     smem_u32(tmem_slot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const int kb0 = sp * A.nkb;
  bool ok = true;
  int loads_issued = 0;

  if (warp == 0 && lane == 0) {
    // ---------------- TMA producer
    for (int i = 0; i < A.nkb && ok; ++i) {
      const int s = i % kGStages;
      const uint32_t ph = (uint32_t)(i / kGStages) & 1u;
      if (!mbar_wait(empty0 + 8 * s, ph ^ 1u, &g_tg_err, TG_EW_MMA)) { ok = false; break; }
      const uint32_t base = smem_u32(smem + s * kStageBytes);
      mbar_expect_tx(full0 + 8 * s, kStageBytes);
      const int kc = (kb0 + i) * 32;
      for (int p = 0; p < 4; ++p) tma_load_2d(base + p * kTileBytes, &maps.v[p], kc, mt * 128, full0 + 8 * s);
      // U planes: re_hi, re_lo, im_hi, im_lo -> [re_hi; im_hi] at tile 4-5, [re_lo; im_lo] at 6-7
      tma_load_2d(base + 4 * kTileBytes, &maps.u[0], kc, nt * 128, full0 + 8 * s);
      tma_load_2d(base + 5 * kTileBytes, &maps.u[2], kc, nt * 128, full0 + 8 * s);
      tma_load_2d(base + 6 * kTileBytes, &maps.u[1], kc, nt * 128, full0 + 8 * s);
      tma_load_2d(base + 7 * kTileBytes, &maps.u[3], kc, nt * 128, full0 + 8 * s);
      ++loads_issued;
    }
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer
    const uint32_t d0 = tmem, d1 = tmem + 256;
    bool first = true;
    for (int i = 0; i < A.nkb; ++i) {
      const int s = i % kGStages;
      const uint32_t ph = (uint32_t)(i / kGStages) & 1u;
      if (!mbar_wait(full0 + 8 * s, ph, &g_tg_err, TG_EW_MMA)) { ok = false; break; }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t base = smem_u32(smem + s * kStageBytes);
#pragma unroll
      for (int kk = 0; kk < 2; ++kk) {
        const uint32_t ko = kk * 32;  // bytes: 16 bf16
        const uint64_t vrh = sdesc(base + 0 * kTileBytes + ko), vrl = sdesc(base + 1 * kTileBytes + ko);
        const uint64_t vih = sdesc(base + 2 * kTileBytes + ko), vil = sdesc(base + 3 * kTileBytes + ko);
        const uint64_t bh = sdesc(base + 4 * kTileBytes + ko), bl = sdesc(base + 6 * kTileBytes + ko);
        const uint32_t acc = first ? 0u : 1u;
        umma(d0, vrh, bh, acc); umma(d0, vrh, bl, 1u); umma(d0, vrl, bh, 1u);
        umma(d1, vih, bh, acc); umma(d1, vih, bl, 1u); umma(d1, vil, bh, 1u);
        first = false;
      }
      umma_commit(empty0 + 8 * s);  // smem stage free once these MMAs finish
    }
    umma_commit(done);  // accumulators complete (or, after a timeout, all issued MMAs)
  }
  __syncwarp();

  // ---------------- epilogue: TMEM -> registers -> partial image
  const bool got = mbar_wait(done, 0, &g_tg_err, TG_EW_MMA);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const int row = mt * 128 + warp * 32 + lane;
  float2* out = A.part + (size_t)sp * A.h * A.w + (size_t)row * A.w;
  const uint32_t lane_base = ((uint32_t)(warp * 32)) << 16;
  for (int c = 0; c < 4; ++c) {
    uint32_t a_re[32], a_im[32], b_re[32], b_im[32];
    tmem_ld32(tmem + lane_base + 0 + c * 32, a_re);    // D0: Vr Ur
    tmem_ld32(tmem + lane_base + 128 + c * 32, a_im);  // D0: Vr Ui
    tmem_ld32(tmem + lane_base + 256 + c * 32, b_re);  // D1: Vi Ur
    tmem_ld32(tmem + lane_base + 384 + c * 32, b_im);  // D1: Vi Ui
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    const int col0 = nt * 128 + c * 32;
    if (got && row < A.h) {
      if (col0 + 32 <= A.w && (A.w & 1) == 0) {
#pragma unroll
        for (int j = 0; j < 32; j += 2) {
          float4 v = make_float4(__uint_as_float(a_re[j]) - __uint_as_float(b_im[j]),
                                 __uint_as_float(a_im[j]) + __uint_as_float(b_re[j]),
                                 __uint_as_float(a_re[j + 1]) - __uint_as_float(b_im[j + 1]),
                                 __uint_as_float(a_im[j + 1]) + __uint_as_float(b_re[j + 1]));
          *reinterpret_cast<float4*>(out + col0 + j) = v;
        }
      } else {
        for (int j = 0; j < 32; ++j)
          if (col0 + j < A.w)
            out[col0 + j] = make_float2(__uint_as_float(a_re[j]) - __uint_as_float(b_im[j]),
                                        __uint_as_float(a_im[j]) + __uint_as_float(b_re[j]));
      }
    }
  }
  // drain: a producer that issued loads must see them land before the CTA exits
  if (warp == 0 && lane == 0 && !got) {
    for (int i = (loads_issued > kGStages ? loads_issued - kGStages : 0); i < loads_issued; ++i)
      mbar_wait(full0 + 8 * (i % kGStages), (uint32_t)(i / kGStages) & 1u, &g_tg_err, TG_EW_MMA);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
  }
}

// ---------------------------------------------------------------- host
typedef CUresult (*EncodeFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                             const cuuint64_t*, const cuuint32_t*, const cuuint32_t*,
                             CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                             CUtensorMapFloatOOBfill);

static EncodeFn encode_fn() {
  static EncodeFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeFn>(p);
  }
  return fn;
}

static bool make_map(CUtensorMap* m, const void* base, int64_t kpad, int lines) {
  EncodeFn enc = encode_fn();
  if (!enc) return false;
  cuuint64_t dims[2] = {(cuuint64_t)kpad, (cuuint64_t)lines};
  cuuint64_t strides[1] = {(cuuint64_t)kpad * 2};
  cuuint32_t box[2] = {32, 128};
  cuuint32_t es[2] = {1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, es,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
             CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int field_gemm_splits(int64_t n, int h, int w) {
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int tiles = ((h + 127) / 128) * ((w + 127) / 128);
  int s = sms / (tiles > 0 ? tiles : 1);
  const int64_t kblocks = (n + 31) / 32;
  if (s > kblocks) s = (int)kblocks;
  return s < 1 ? 1 : s;
}

int launch_field_gemm(const __nv_bfloat16_raw* vplanes, const __nv_bfloat16_raw* uplanes, int lines_v,
                      int lines_u, int64_t kpad, int splits, int h, int w, float2* part,
                      cudaStream_t s) {
  // the eight tensor maps of a plane buffer, encoded once per (buffers,
  // shape) and kept in a small round-robin cache (an evaluation cycles through
  // two buffers; a few plans may alternate)
  struct Entry {
    const void *v, *u;
    int64_t kpad;
    int lv, lu;
    GemmMaps maps;
  };
  static std::mutex mu;
  static Entry cache[8];
  static int used = 0, next = 0;
  GemmMaps maps;
  {
    std::lock_guard<std::mutex> lock(mu);
    int hit = -1;
    for (int i = 0; i < used; ++i)
      if (cache[i].v == vplanes && cache[i].u == uplanes && cache[i].kpad == kpad && cache[i].lv == lines_v &&
          cache[i].lu == lines_u)
        hit = i;
    if (hit < 0) {
      Entry e;
      std::memset(&e, 0, sizeof(e));
      e.v = vplanes; e.u = uplanes; e.kpad = kpad; e.lv = lines_v; e.lu = lines_u;
      const size_t pv = (size_t)lines_v * kpad, pu = (size_t)lines_u * kpad;
      for (int p = 0; p < 4; ++p) {
        if (!make_map(&e.maps.v[p], vplanes + p * pv, kpad, lines_v)) return TG_ERR_CUDA;
        if (!make_map(&e.maps.u[p], uplanes + p * pu, kpad, lines_u)) return TG_ERR_CUDA;
      }
      hit = used < 8 ? used++ : next;
      next = (hit + 1) % 8;
      cache[hit] = e;
    }
    maps = cache[hit].maps;
  }
  GemmArgs A;
  A.nkb = (int)(kpad / 32 / splits);
  A.h = h;
  A.w = w;
  A.part = part;
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(k_field_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmem) !=
        cudaSuccess)
      return TG_ERR_CUDA;
    attr = true;
  }
  dim3 grid(lines_v / 128, lines_u / 128, splits);
  k_field_gemm<<<grid, 128, kGemmSmem, s>>>(maps, A);
  return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
}

}  // namespace tg
