// batch.cu - many independent models with uneven component and ray counts in
// ONE persistent launch over a packed model table (forward + adjoint).
//
// The reference runs each model separately (run.py:85-116 per model, jax.grad
// per model); here the host packs every model's compiled steps, a per-model
// header and a tile list into one device buffer (the plan).  A persistent
// grid pulls tiles (a model and a contiguous run of its rays) from an atomic
// work counter, stages that model's steps in shared memory, traces the rays
// forward and writes the outputs.  Per-tile partials are reduced per model in
// a fixed order, so the results do not depend on which CTA took which tile.
//
// Adjoint of loss = sum |(x, y)_out - target|^2 by moments.  The loss gradient
// w.r.t. the output, l = 2 (x - tx, y - ty), reaches every step through the
// LINEAR part of the chain, which is the same for every ray (a biprism's
// sign(x) only moves the affine offset).  Every per-step sum therefore follows
// exactly from a handful of per-model moments of the rays:
//   W[a][c] = sum_i l_a,i v_c,i     (v = input x, y, dx, dy, 1; a = x, y)
//   S_b[a]  = sum_i sign_b,i l_a,i  (one pair per biprism b)
// k_batch accumulates the moments next to the forward pass (no reverse walk
// per ray) and k_batch_steps turns them into the per-step sums with float64
// 5x5 algebra, one thread per model.
#include <cstring>
#include <vector>

#include "tg_common.cuh"

TG_DEFINE_ERROR_WORD(batch)

namespace tg {

struct BModel {
  int32_t op_off, n_steps, tile_off, n_tiles;
  int64_t ray_off, n_rays;
  double pl_const, z_out;
  int64_t part_off;  // doubles: this model's first tile partial
  int32_t n_bip, n_mom;  // biprisms, moments (10 + 2 * n_bip)
  int64_t mom_off;       // doubles: this model's moments
};

struct BTile {
  int32_t model, count;
  int64_t start;  // absolute ray index
};

struct BHeader {
  int32_t n_models, n_tiles, total_steps, tile_rays;
  int64_t models_off, tiles_off, ops_off, mom_model_off;  // byte offsets in the plan
  int64_t partial_doubles, moment_doubles;
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

template <int R>
__global__ void __launch_bounds__(512)
k_batch(const uint8_t* __restrict__ plan, const __grid_constant__ BatchIO io,
        int32_t* __restrict__ counter, double* __restrict__ partial) {
  extern __shared__ float wacc[];  // [warps][n_mom] per-warp float32 moments of this tile
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
    const int ns = M.n_steps, nm = M.n_mom, nb = M.n_bip;
    for (int i = threadIdx.x; i < ns; i += blockDim.x) sops[i] = ops[M.op_off + i];
    if (adj)
      for (int i = threadIdx.x; i < nwarps * nm; i += blockDim.x) wacc[i] = 0.f;
    __syncthreads();
    float mw[10];
#pragma unroll
    for (int j = 0; j < 10; ++j) mw[j] = 0.f;
    const int64_t end = T.start + T.count;
    for (int64_t blk = T.start; blk < end; blk += (int64_t)blockDim.x * R) {
      RayS r[R];
      float v0[R][4];
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
        v0[k][0] = io.x[i]; v0[k][1] = io.y[i]; v0[k][2] = io.dx[i]; v0[k][3] = io.dy[i];
        r[k] = RayS{v0[k][0], v0[k][1], v0[k][2], v0[k][3], 0.f};
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
      float lx[R], ly[R];
#pragma unroll
      for (int k = 0; k < R; ++k) {
        lx[k] = inr[k] ? 2.f * (r[k].x - io.tx[idx[k]]) : 0.f;
        ly[k] = inr[k] ? 2.f * (r[k].y - io.ty[idx[k]]) : 0.f;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          mw[c] = fmaf(lx[k], v0[k][c], mw[c]);
          mw[5 + c] = fmaf(ly[k], v0[k][c], mw[5 + c]);
        }
        mw[4] += lx[k];
        mw[9] += ly[k];
      }
      // biprism sign moments (few per model): warp sums into the warp's row
      for (int b2 = 0; b2 < nb; ++b2) {
        float sx = 0.f, sy = 0.f;
#pragma unroll
        for (int k = 0; k < R; ++k) {
          const uint32_t bits = (uint32_t)(sb[k] >> (2 * b2)) & 3u;
          const float sg = bits == 1u ? 1.f : (bits == 2u ? -1.f : 0.f);
          sx = fmaf(sg, lx[k], sx);
          sy = fmaf(sg, ly[k], sy);
        }
        sx = bt_warp_sum(sx);
        sy = bt_warp_sum(sy);
        if (lane == 0) {
          wacc[warp * nm + 10 + 2 * b2] += sx;
          wacc[warp * nm + 11 + 2 * b2] += sy;
        }
      }
    }
    if (adj) {
#pragma unroll
      for (int j = 0; j < 10; ++j) {
        const float v = bt_warp_sum(mw[j]);
        if (lane == 0) wacc[warp * nm + j] += v;
      }
    }
    __syncthreads();
    if (adj) {
      double* dst = partial + M.part_off + (int64_t)(t - M.tile_off) * nm;
      for (int i = threadIdx.x; i < nm; i += blockDim.x) {
        double a = 0.0;
        for (int w = 0; w < nwarps; ++w) a += (double)wacc[w * nm + i];
        dst[i] = a;
      }
    }
    __syncthreads();
  }
}

// moments[e] = sum over the model's tiles of the tile partials, in tile order.
__global__ void k_batch_reduce(const uint8_t* __restrict__ plan, const double* __restrict__ partial,
                               double* __restrict__ moments) {
  const BHeader H = *reinterpret_cast<const BHeader*>(plan);
  const BModel* models = reinterpret_cast<const BModel*>(plan + H.models_off);
  const int32_t* mom_model = reinterpret_cast<const int32_t*>(plan + H.mom_model_off);
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= H.moment_doubles) return;
  const BModel M = models[mom_model[e]];
  const int j = (int)(e - M.mom_off);
  // eight independent partial sums keep eight loads in flight; the summation
  // order is fixed, so the result is deterministic
  double a[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  const double* src = partial + M.part_off + j;
  int tt = 0;
  for (; tt + 8 <= M.n_tiles; tt += 8) {
#pragma unroll
    for (int u = 0; u < 8; ++u) a[u] += src[(int64_t)(tt + u) * M.n_mom];
  }
  for (int u = 0; tt < M.n_tiles; ++tt, ++u) a[u] += src[(int64_t)tt * M.n_mom];
  moments[e] = ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]));
}

// 5x5 step matrix (linear part + non-biprism offsets) of one compiled step,
// in the float32 values the forward pass used.
__device__ void step_matrix(const Op& op, float T[5][5]) {
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 5; ++j) T[i][j] = (i == j) ? 1.f : 0.f;
  switch (op.kind) {
    case OP_FREE: T[0][2] = op.c[0]; T[1][3] = op.c[0]; break;
    case OP_LENS: T[2][0] = -op.c[0]; T[3][1] = -op.c[0]; break;
    case OP_SHIFT: T[0][4] = op.c[0]; T[1][4] = op.c[1]; T[2][4] = op.c[2]; T[3][4] = op.c[3]; break;
    case OP_DEFLECT: T[2][4] = op.c[0]; T[3][4] = op.c[1]; break;
    case OP_ROTATE: {
      const float c = op.c[0], sn = op.c[1];
      T[0][0] = c; T[0][1] = -sn; T[1][0] = sn; T[1][1] = c;
      T[2][2] = c; T[2][3] = -sn; T[3][2] = sn; T[3][3] = c;
    } break;
    default: break;  // biprism offset enters through its sign moment; others are identity
  }
}

// One warp per model: per-step sums (the quantities of the generic adjoint)
// from the moments.  Every lane walks the chain once (the 5x5 prefix/suffix
// products are short, independent multiply-adds, run in float32 - the
// precision of the traced rays) and leaves, per step, the adjoint map G_s,
// the first four rows of the prefix C_s and the moment-weighted biprism
// offsets E_s in shared memory; then the lanes split the steps and contract
// them with the moments in float64.
//   E_{s,a} = sum_b S_b[a] (effect at step s of biprism b's offset), so the
//   bilinear sum of a step is sum_a (G_s Q C_s)[a] . W[a] + (G_s Q E_{s,a})[a].
constexpr int kStepFloats = 16 + 20 + 8;  // G_s, C_s rows 0..3, E_s (a = x, y)

__global__ void __launch_bounds__(32)
k_batch_steps(const uint8_t* __restrict__ plan, const double* __restrict__ moments,
              double* __restrict__ raw) {
  extern __shared__ float st[];  // [n_steps][kStepFloats]
  const BHeader H = *reinterpret_cast<const BHeader*>(plan);
  const int m = blockIdx.x;
  if (m >= H.n_models) return;
  const BModel M = reinterpret_cast<const BModel*>(plan + H.models_off)[m];
  const Op* ops = reinterpret_cast<const Op*>(plan + H.ops_off) + M.op_off;
  const double* mo = moments + M.mom_off;
  const int ns = M.n_steps;
  const int lane = threadIdx.x;
  {  // backward: G_s = linear part of (T_{ns-1} ... T_{s+1}); lambda after s = G_s^T l
    float Rm[4][4];
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) Rm[i][j] = (i == j) ? 1.f : 0.f;
    for (int s = ns - 1; s >= 0; --s) {
      if (lane == 0)
        for (int i = 0; i < 16; ++i) st[s * kStepFloats + i] = Rm[i >> 2][i & 3];
      float T[5][5];
      step_matrix(ops[s], T);
      float N2[4][4];
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
          float v = 0.f;
          for (int k = 0; k < 4; ++k) v = fmaf(Rm[i][k], T[k][j], v);
          N2[i][j] = v;
        }
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) Rm[i][j] = N2[i][j];
    }
  }
  {  // forward: C_s and E_s
    float Cm[5][5], E[2][4];
    for (int i = 0; i < 5; ++i)
      for (int j = 0; j < 5; ++j) Cm[i][j] = (i == j) ? 1.f : 0.f;
    for (int a = 0; a < 2; ++a)
      for (int j = 0; j < 4; ++j) E[a][j] = 0.f;
    for (int s = 0; s < ns; ++s) {
      const Op op = ops[s];
      float T[5][5];
      step_matrix(op, T);
      float N5[5][5];
      for (int i = 0; i < 5; ++i)
        for (int j = 0; j < 5; ++j) {
          float v = 0.f;
          for (int k = 0; k < 5; ++k) v = fmaf(T[i][k], Cm[k][j], v);
          N5[i][j] = v;
        }
      for (int i = 0; i < 5; ++i)
        for (int j = 0; j < 5; ++j) Cm[i][j] = N5[i][j];
      for (int a = 0; a < 2; ++a) {
        float ne[4];
        for (int i = 0; i < 4; ++i) {
          float v = 0.f;
          for (int k = 0; k < 4; ++k) v = fmaf(T[i][k], E[a][k], v);
          ne[i] = v;
        }
        for (int i = 0; i < 4; ++i) E[a][i] = ne[i];
      }
      if (op.kind == OP_BIPRISM) {  // this biprism's offset def * sign * e_dx, weighted by S_b
        E[0][2] += (float)(op.c[0] * mo[10 + 2 * op.aux]);
        E[1][2] += (float)(op.c[0] * mo[11 + 2 * op.aux]);
      }
      if (lane == 0) {
        float* o = st + s * kStepFloats + 16;
        for (int i = 0; i < 4; ++i)
          for (int j = 0; j < 5; ++j) o[5 * i + j] = Cm[i][j];
        for (int a = 0; a < 2; ++a)
          for (int j = 0; j < 4; ++j) o[20 + 4 * a + j] = E[a][j];
      }
    }
  }
  __syncwarp();
  for (int s = lane; s < ns; s += 32) {
    const Op op = ops[s];
    const float* Gs = st + s * kStepFloats;       // Gs[4*i+j]
    const float* Cs = Gs + 16;                    // Cs[5*i+j], rows 0..3
    const float* Es = Gs + 36;                    // Es[4*a+j]
    auto lin = [&](int j) { return (double)Gs[0 * 4 + j] * mo[4] + (double)Gs[1 * 4 + j] * mo[9]; };
    auto bil = [&](const float Q[4][4]) {
      double acc = 0.0;
      for (int a = 0; a < 2; ++a) {
        float GQ[4];
        for (int j = 0; j < 4; ++j) {
          float v = 0.f;
          for (int k = 0; k < 4; ++k) v = fmaf(Gs[a * 4 + k], Q[k][j], v);
          GQ[j] = v;
        }
        for (int c = 0; c < 5; ++c) {
          float v = 0.f;
          for (int j = 0; j < 4; ++j) v = fmaf(GQ[j], Cs[5 * j + c], v);
          acc += (double)v * mo[5 * a + c];
        }
        float v = 0.f;
        for (int j = 0; j < 4; ++j) v = fmaf(GQ[j], Es[4 * a + j], v);
        acc += (double)v;
      }
      return acc;
    };
    double r4[4] = {0.0, 0.0, 0.0, 0.0};
    switch (op.kind) {
      case OP_FREE: {
        const float Q[4][4] = {{0, 0, 1, 0}, {0, 0, 0, 1}, {0, 0, 0, 0}, {0, 0, 0, 0}};
        r4[0] = bil(Q);
      } break;
      case OP_LENS: {
        const float k2 = op.c[0] * op.c[0];
        const float Q[4][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}, {k2, 0, 0, 0}, {0, k2, 0, 0}};
        r4[0] = bil(Q);
      } break;
      case OP_ROTATE: {
        const float Q[4][4] = {{0, -1, 0, 0}, {1, 0, 0, 0}, {0, 0, 0, -1}, {0, 0, 1, 0}};
        r4[0] = bil(Q);
      } break;
      case OP_SHIFT:
        r4[0] = lin(0); r4[1] = lin(1); r4[2] = lin(2); r4[3] = lin(3);
        break;
      case OP_DEFLECT:
        r4[0] = lin(2); r4[1] = lin(3);
        break;
      case OP_BIPRISM: {
        const int b = op.aux;
        r4[0] = (double)Gs[0 * 4 + 2] * mo[10 + 2 * b] + (double)Gs[1 * 4 + 2] * mo[11 + 2 * b];
      } break;
      default: break;
    }
    double* out = raw + (int64_t)(M.op_off + s) * 4;
    out[0] = r4[0]; out[1] = r4[1]; out[2] = r4[2]; out[3] = r4[3];
  }
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
  std::vector<int32_t> mom_model;
  int64_t ray_off = 0, part_off = 0, mom_off = 0;
  int32_t max_steps = 0, max_mom = 10;
  for (int m = 0; m < n_models; ++m) {
    if (n_rays[m] < 0) return TG_ERR_INVALID;
    Program P;
    int st = compile_program(&models[m], false, z_in ? z_in[m] : 0.0, &P);
    if (st != TG_OK) return st;
    if (P.n_probe_ops) return TG_ERR_UNSUPPORTED;
    BModel& M = bm[m];
    std::memset(&M, 0, sizeof(M));
    M.op_off = (int32_t)ops.size();
    M.n_steps = P.n_steps;
    if (P.n_steps > max_steps) max_steps = P.n_steps;
    M.tile_off = (int32_t)bt.size();
    M.ray_off = ray_off;
    M.n_rays = n_rays[m];
    M.pl_const = P.pl_const;
    M.z_out = P.z_out;
    M.part_off = part_off;
    M.n_bip = P.n_biprism;
    M.n_mom = 10 + 2 * P.n_biprism;
    M.mom_off = mom_off;
    if (M.n_mom > max_mom) max_mom = M.n_mom;
    for (int s = 0; s < P.n_steps; ++s) ops.push_back(P.op[s]);
    for (int j = 0; j < M.n_mom; ++j) mom_model.push_back(m);
    int32_t nt = 0;
    for (int64_t r = 0; r < n_rays[m]; r += tile_rays, ++nt) {
      BTile T;
      T.model = m;
      T.start = ray_off + r;
      T.count = (int32_t)((n_rays[m] - r) < tile_rays ? (n_rays[m] - r) : tile_rays);
      bt.push_back(T);
    }
    M.n_tiles = nt;
    part_off += (int64_t)nt * M.n_mom;
    mom_off += M.n_mom;
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
  H.mom_model_off = off; off = al16(off + (int64_t)sizeof(int32_t) * mom_model.size());
  H.partial_doubles = part_off;
  H.moment_doubles = mom_off;
  info->plan_bytes = (size_t)off;
  info->n_tiles = H.n_tiles;
  info->total_steps = H.total_steps;
  info->total_rays = ray_off;
  info->max_steps = max_steps;
  info->max_moments = max_mom;
  info->n_models = n_models;
  info->partial_doubles = part_off;
  info->moment_doubles = mom_off;
  // workspace: counter | tile partials | moments
  info->workspace_bytes = 256 + (size_t)(part_off + mom_off) * sizeof(double);
  if (!plan) return TG_OK;  // size query
  if (plan_bytes < (size_t)off) return TG_ERR_WORKSPACE;
  uint8_t* p = reinterpret_cast<uint8_t*>(plan);
  std::memset(p, 0, (size_t)off);
  std::memcpy(p, &H, sizeof(H));
  if (n_models) std::memcpy(p + H.models_off, bm.data(), sizeof(BModel) * n_models);
  if (!bt.empty()) std::memcpy(p + H.tiles_off, bt.data(), sizeof(BTile) * bt.size());
  if (!ops.empty()) std::memcpy(p + H.ops_off, ops.data(), sizeof(Op) * ops.size());
  if (!mom_model.empty())
    std::memcpy(p + H.mom_model_off, mom_model.data(), sizeof(int32_t) * mom_model.size());
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
  // per-warp float32 moments: warps x max moments (10 + 2 per biprism)
  const size_t dyn = (size_t)(block / 32) * (info->max_moments > 0 ? info->max_moments : 10) * sizeof(float);
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
    // moments then per-step sums; sizes come from the plan header on the device
    double* moments = partial + info->partial_doubles;
    const int64_t nmom = info->moment_doubles;
    k_batch_reduce<<<(int)((nmom + 255) / 256), 256, 0, s>>>(plan, partial, moments);
    const size_t sm_steps = (size_t)(info->max_steps > 0 ? info->max_steps : 1) * kStepFloats * sizeof(float);
    k_batch_steps<<<info->n_models, 32, sm_steps, s>>>(plan, moments, io->raw);
  }
  return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
}
