// batch.cu - many independent models with uneven component and ray counts in
// ONE persistent launch over a packed model table (forward + adjoint).
//
// The reference runs each model separately (run.py:85-116 per model, jax.grad
// per model); here the host packs every model's compiled steps, a per-model
// header and a tile list into one device buffer (the plan).  A persistent
// grid pulls tiles (a model and a contiguous run of its rays) from an atomic
// work counter, stages that model's steps in shared memory, traces the rays
// forward, writes the outputs, and - when targets are given - walks the chain
// backwards from the loss sum |r - target|^2 to produce per-step parameter
// sums.  Per-tile partials are reduced per model in a fixed order, so the
// results do not depend on which CTA took which tile.
#include <cstring>
#include <vector>

#include "tg_common.cuh"

TG_DEFINE_ERROR_WORD(batch)

namespace tg {

struct BModel {
  int32_t op_off, n_steps, tile_off, n_tiles;
  int64_t ray_off, n_rays;
  double pl_const, z_out;
  int64_t part_off;  // doubles
};

struct BTile {
  int32_t model, count;
  int64_t start;  // absolute ray index
};

struct BHeader {
  int32_t n_models, n_tiles, total_steps, tile_rays;
  int64_t models_off, tiles_off, ops_off, step_model_off;  // byte offsets in the plan
  int64_t partial_doubles;
};

struct BatchIO {
  const float *x, *y, *dx, *dy;
  float *ox, *oy, *odx, *ody;
  double* opl;
  const float *tx, *ty;
  double* raw;
};

__device__ __forceinline__ float bt_warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ int bt_nsums(int kind) {
  switch (kind) {
    case OP_FREE: case OP_LENS: case OP_BIPRISM: case OP_ROTATE: return 1;
    case OP_DEFLECT: return 2;
    case OP_SHIFT: return 4;
    default: return 0;
  }
}

template <int R>
__global__ void __launch_bounds__(512)
k_batch(const uint8_t* __restrict__ plan, const __grid_constant__ BatchIO io,
        int32_t* __restrict__ counter, double* __restrict__ partial) {
  extern __shared__ float wacc[];  // [warps][n_steps * 4] per-warp float32 sums of this tile
  __shared__ Op sops[kMaxSteps];
  __shared__ int s_tile;
  const int nwarps = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5;
  const BHeader H = *reinterpret_cast<const BHeader*>(plan);
  const BModel* models = reinterpret_cast<const BModel*>(plan + H.models_off);
  const BTile* tiles = reinterpret_cast<const BTile*>(plan + H.tiles_off);
  const Op* ops = reinterpret_cast<const Op*>(plan + H.ops_off);
  const bool adj = io.tx != nullptr;
  const int lane = threadIdx.x & 31;
  for (;;) {
    if (threadIdx.x == 0) s_tile = atomicAdd(counter, 1);
    __syncthreads();
    const int t = s_tile;
    if (t >= H.n_tiles) break;
    const BTile T = tiles[t];
    if (T.model < 0 || T.model >= H.n_models) {  // corrupt plan: flag and skip
      if (threadIdx.x == 0) atomicOr(&g_tg_err, TG_EW_TABLE);
      __syncthreads();
      continue;
    }
    const BModel M = models[T.model];
    const int ns = M.n_steps;
    for (int i = threadIdx.x; i < ns; i += blockDim.x) sops[i] = ops[M.op_off + i];
    if (adj)
      for (int i = threadIdx.x; i < nwarps * ns * 4; i += blockDim.x) wacc[i] = 0.f;
    __syncthreads();
    const int64_t end = T.start + T.count;
    for (int64_t blk = T.start; blk < end; blk += (int64_t)blockDim.x * R) {
      RayS r[R];
      Adj ad[R];
      uint64_t sb[R];
      bool alive[R];
      double dv[R];
      int64_t idx[R];
      bool inr[R];
#pragma unroll
      for (int k = 0; k < R; ++k) {
        idx[k] = blk + (int64_t)threadIdx.x + (int64_t)k * blockDim.x;  // coalesced per k
        inr[k] = idx[k] < end;
        const int64_t i = inr[k] ? idx[k] : T.start;
        r[k] = RayS{io.x[i], io.y[i], io.dx[i], io.dy[i], 0.f};
        sb[k] = 0;
        alive[k] = true;
        dv[k] = 0.0;
      }
      for (int s = 0; s < ns; ++s) {
        const Op op = sops[s];
#pragma unroll
        for (int k = 0; k < R; ++k) op_forward(op, nullptr, r[k], 0.0, 0.0, dv[k], sb[k], alive[k]);
      }
#pragma unroll
      for (int k = 0; k < R; ++k) {
        if (inr[k]) {
          const int64_t i = idx[k];
          io.ox[i] = r[k].x;
          io.oy[i] = r[k].y;
          io.odx[i] = r[k].dx;
          io.ody[i] = r[k].dy;
          if (io.opl) io.opl[i] = M.pl_const + (double)r[k].plv;
        }
      }
      if (!adj) continue;
#pragma unroll
      for (int k = 0; k < R; ++k) {
        const float lx = inr[k] ? 2.f * (r[k].x - io.tx[idx[k]]) : 0.f;
        const float ly = inr[k] ? 2.f * (r[k].y - io.ty[idx[k]]) : 0.f;
        ad[k] = Adj{lx, ly, 0.f, 0.f, 0.f};
      }
      for (int s = ns - 1; s >= 0; --s) {
        const Op op = sops[s];
        float c[4] = {0.f, 0.f, 0.f, 0.f};
        float gz = 0.f;
#pragma unroll
        for (int k = 0; k < R; ++k) {
          float ck[4] = {0.f, 0.f, 0.f, 0.f};
          op_reverse(op, nullptr, r[k], ad[k], sb[k], dv[k], ck, gz);
          c[0] += ck[0]; c[1] += ck[1]; c[2] += ck[2]; c[3] += ck[3];
        }
        // warp sums accumulate in float32 in the warp's own shared row (no
        // atomics, no float64: GB300 issues float64 at ~1/60 of float32)
        const int nsum = bt_nsums(op.kind);
        for (int j = 0; j < nsum; ++j) {
          const float v = bt_warp_sum(c[j]);
          if (lane == 0) wacc[warp * ns * 4 + 4 * s + j] += v;
        }
      }
    }
    __syncthreads();
    if (adj) {
      double* dst = partial + M.part_off + (int64_t)(t - M.tile_off) * ns * 4;
      for (int i = threadIdx.x; i < ns * 4; i += blockDim.x) {
        double a = 0.0;
        for (int w = 0; w < nwarps; ++w) a += (double)wacc[w * ns * 4 + i];
        dst[i] = a;
      }
    }
    __syncthreads();
  }
}

// raw[s][j] = sum over the model's tiles, in tile order.
__global__ void k_batch_reduce(const uint8_t* __restrict__ plan, const double* __restrict__ partial,
                               double* __restrict__ raw) {
  const BHeader H = *reinterpret_cast<const BHeader*>(plan);
  const BModel* models = reinterpret_cast<const BModel*>(plan + H.models_off);
  const int32_t* step_model = reinterpret_cast<const int32_t*>(plan + H.step_model_off);
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)H.total_steps * 4) return;
  const int s = (int)(e >> 2), j = (int)(e & 3);
  const BModel M = models[step_model[s]];
  const int ls = s - M.op_off;
  double acc = 0.0;
  for (int tt = 0; tt < M.n_tiles; ++tt) acc += partial[M.part_off + (int64_t)tt * M.n_steps * 4 + ls * 4 + j];
  raw[e] = acc;
}

static int sm_count_batch() {
  static int cached = 0;
  if (!cached) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&cached, cudaDevAttrMultiProcessorCount, dev);
    if (cached <= 0) cached = 148;
  }
  return cached;
}

static inline int64_t al16(int64_t v) { return (v + 15) & ~(int64_t)15; }

}  // namespace tg

using namespace tg;

extern "C" int tg_batch_plan(int32_t n_models, const tg_model* models, const int64_t* n_rays,
                             const double* z_in, int32_t tile_rays, void* plan, size_t plan_bytes,
                             tg_batch_info* info) {
  if (n_models < 0 || (n_models > 0 && (!models || !n_rays)) || tile_rays <= 0 || !info)
    return TG_ERR_INVALID;
  std::vector<BModel> bm(n_models);
  std::vector<BTile> bt;
  std::vector<Op> ops;
  std::vector<int32_t> step_model;
  int64_t ray_off = 0, part_off = 0;
  int32_t max_steps = 0;
  for (int m = 0; m < n_models; ++m) {
    if (n_rays[m] < 0) return TG_ERR_INVALID;
    Program P;
    int st = compile_program(&models[m], false, z_in ? z_in[m] : 0.0, &P);
    if (st != TG_OK) return st;
    if (P.n_probe_ops) return TG_ERR_UNSUPPORTED;
    BModel& M = bm[m];
    M.op_off = (int32_t)ops.size();
    M.n_steps = P.n_steps;
    if (P.n_steps > max_steps) max_steps = P.n_steps;
    M.tile_off = (int32_t)bt.size();
    M.ray_off = ray_off;
    M.n_rays = n_rays[m];
    M.pl_const = P.pl_const;
    M.z_out = P.z_out;
    M.part_off = part_off;
    for (int s = 0; s < P.n_steps; ++s) {
      ops.push_back(P.op[s]);
      step_model.push_back(m);
    }
    int32_t nt = 0;
    for (int64_t r = 0; r < n_rays[m]; r += tile_rays, ++nt) {
      BTile T;
      T.model = m;
      T.start = ray_off + r;
      T.count = (int32_t)((n_rays[m] - r) < tile_rays ? (n_rays[m] - r) : tile_rays);
      bt.push_back(T);
    }
    M.n_tiles = nt;
    part_off += (int64_t)nt * P.n_steps * 4;
    ray_off += n_rays[m];
    if (bt.size() > 0x7fffffff || ops.size() > 0x7fffffff) return TG_ERR_TOO_LARGE;
  }
  BHeader H;
  std::memset(&H, 0, sizeof(H));
  H.n_models = n_models;
  H.n_tiles = (int32_t)bt.size();
  H.total_steps = (int32_t)ops.size();
  H.tile_rays = tile_rays;
  int64_t off = al16(sizeof(BHeader));
  H.models_off = off; off = al16(off + (int64_t)sizeof(BModel) * n_models);
  H.tiles_off = off; off = al16(off + (int64_t)sizeof(BTile) * bt.size());
  H.ops_off = off; off = al16(off + (int64_t)sizeof(Op) * ops.size());
  H.step_model_off = off; off = al16(off + (int64_t)sizeof(int32_t) * step_model.size());
  H.partial_doubles = part_off;
  info->plan_bytes = (size_t)off;
  info->n_tiles = H.n_tiles;
  info->total_steps = H.total_steps;
  info->total_rays = ray_off;
  info->max_steps = max_steps;
  info->workspace_bytes = 256 + (size_t)part_off * sizeof(double);
  if (!plan) return TG_OK;  // size query
  if (plan_bytes < (size_t)off) return TG_ERR_WORKSPACE;
  uint8_t* p = reinterpret_cast<uint8_t*>(plan);
  std::memset(p, 0, (size_t)off);
  std::memcpy(p, &H, sizeof(H));
  if (n_models) std::memcpy(p + H.models_off, bm.data(), sizeof(BModel) * n_models);
  if (!bt.empty()) std::memcpy(p + H.tiles_off, bt.data(), sizeof(BTile) * bt.size());
  if (!ops.empty()) std::memcpy(p + H.ops_off, ops.data(), sizeof(Op) * ops.size());
  if (!step_model.empty())
    std::memcpy(p + H.step_model_off, step_model.data(), sizeof(int32_t) * step_model.size());
  return TG_OK;
}

extern "C" int tg_batch_run(const void* plan_dev, const tg_batch_info* info, const tg_batch_io* io,
                            int32_t block, int32_t rays_per_thread, void* workspace,
                            size_t ws_bytes, void* stream) {
  if (!plan_dev || !info || !io) return TG_ERR_INVALID;
  if (block != 128 && block != 256 && block != 512) return TG_ERR_INVALID;
  if (rays_per_thread != 1 && rays_per_thread != 2 && rays_per_thread != 4) return TG_ERR_INVALID;
  if (info->total_rays > 0 && (!io->x || !io->y || !io->dx || !io->dy || !io->out_x ||
                               !io->out_y || !io->out_dx || !io->out_dy))
    return TG_ERR_INVALID;
  const bool adj = io->target_x != nullptr;
  if (adj && (!io->target_y || !io->raw)) return TG_ERR_INVALID;
  if (!workspace || ws_bytes < info->workspace_bytes) return TG_ERR_WORKSPACE;
  if (((uintptr_t)workspace & 255) != 0) return TG_ERR_ALIGN;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  int32_t* counter = reinterpret_cast<int32_t*>(workspace);
  double* partial = reinterpret_cast<double*>(reinterpret_cast<uint8_t*>(workspace) + 256);
  if (cudaMemsetAsync(counter, 0, sizeof(int32_t), s) != cudaSuccess) return TG_ERR_CUDA;
  if (info->n_tiles == 0) return TG_OK;
  BatchIO A;
  A.x = io->x; A.y = io->y; A.dx = io->dx; A.dy = io->dy;
  A.ox = io->out_x; A.oy = io->out_y; A.odx = io->out_dx; A.ody = io->out_dy;
  A.opl = io->out_pathlength;
  A.tx = io->target_x; A.ty = io->target_y;
  A.raw = io->raw;
  const uint8_t* plan = reinterpret_cast<const uint8_t*>(plan_dev);
  // per-warp float32 step sums: warps x max steps x 4 (max steps <= kMaxSteps)
  const size_t dyn = (size_t)(block / 32) * (info->max_steps > 0 ? info->max_steps : 1) * 4 * sizeof(float);
  if (dyn > 48 * 1024) return TG_ERR_TOO_LARGE;
  int per_sm = 1;
  if (rays_per_thread == 1) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<1>, block, dyn);
  else if (rays_per_thread == 2) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<2>, block, dyn);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<4>, block, dyn);
  if (per_sm < 1) per_sm = 1;
  int grid = sm_count_batch() * per_sm;
  if (grid > info->n_tiles) grid = info->n_tiles;
  if (rays_per_thread == 1) k_batch<1><<<grid, block, dyn, s>>>(plan, A, counter, partial);
  else if (rays_per_thread == 2) k_batch<2><<<grid, block, dyn, s>>>(plan, A, counter, partial);
  else k_batch<4><<<grid, block, dyn, s>>>(plan, A, counter, partial);
  if (adj && info->total_steps > 0) {
    const int64_t nel = (int64_t)info->total_steps * 4;
    k_batch_reduce<<<(int)((nel + 255) / 256), 256, 0, s>>>(plan, partial, io->raw);
  }
  return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
}
